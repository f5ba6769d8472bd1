// Batched and served forms of the plume step: many independent scenes of
// uneven sizes, each stage one launch over all scenes' tiles (mg_batch.h).
//
// Engine.  A set of member scenes, each with its own device block: flags,
// two velocity buffers (3n, ping-pong), two density buffers, 4n forward /
// scratch values, the inflow mask, pressure, the CG vectors rhs / residual /
// search / tmp, 2-byte stencil codes and the per-tile partial sums -- about
// 80 bytes per cell.  Freed blocks are kept in a size-keyed pool.  Members
// can join and leave between steps (the served form); the tile lists are
// rebuilt when they do.
//
// Step: inflow, advection (forward SL of density and velocity in one pass,
// MacCormack correction + clamp in the next, outflow BC), setWallBcs +
// addBuoyancy, then solvePressure: MakeRhs + codes, CG init, CG sweeps until
// every member has converged, correctVelocity.  Sweeps run over the tiles of
// the members still iterating: the host reads the number of finished scenes
// every few sweeps and, when it changed, drops their tiles.  A scene's
// results depend only on its own data, so it computes the same alone and in
// any mix.
//
// Served form.  Jobs (a plume scene run for a number of steps) arrive at
// given times; a job is admitted in arrival order once it has arrived and
// its block fits the device-memory budget; every tick advances all resident
// jobs by one step together (continuous batching); a finished job leaves
// (its final fields copied to the host if requested) and its block returns
// to the pool for the next one.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mantagpu.h"
#include "mg_batch.h"

using namespace mgpu;

namespace {

#define CKB(call)                                                                                  \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return set_error(MG_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

int tiles_of(int nx, int ny, int nz, int rows) { return ((nx + kBTX - 1) / kBTX) * ((ny + rows - 1) / rows) * nz; }

constexpr int kMicTile = 16;  // edge of the MIC dataflow tiles
int mic_tiles(int n) { return (n + kMicTile - 1) / kMicTile; }

// bytes of one scene's device block (3D scenes also hold the MIC diagonal
// and the face words of the dataflow sweeps; dam-break scenes the
// ghost-fluid diagonal and the extrapolation marks)
size_t scene_bytes(int nx, int ny, int nz, int kind = 0) {
  const size_t n = (size_t)nx * ny * nz;
  size_t b = align256(n * sizeof(int)) + 2 * align256(3 * n * sizeof(float)) + 2 * align256(n * sizeof(float)) +
             align256(4 * n * sizeof(float)) + 6 * align256(n * sizeof(float)) + align256(n * sizeof(code_t)) +
             align256(2 * (size_t)tiles_of(nx, ny, nz, kBTY) * sizeof(double));
  if (nz > 1)
    b += align256(n * sizeof(float)) +
         align256(mic_flow_face_words(mic_tiles(nx) * mic_tiles(ny) * mic_tiles(nz)) * sizeof(unsigned long long));
  if (kind == 1) b += align256(n * sizeof(float)) + align256(n * sizeof(int));
  return b;
}

struct SceneRec {
  BScene s;
  void* mem = nullptr;
  void* refMem = nullptr;  // p64 | b64 of the FP64 refinement, allocated when first used
  size_t bytes = 0;
  int step = 0;  // steps taken: the inflow noise index
  int cur = 0;   // which ping-pong buffers are current
};

// the kernel arguments a captured sweep graph depends on
struct GraphKey {
  const void* tiles;
  int active, rowsK;
  const void* scenes;
  const void* flow;
  const void* order;
  int micTiles, micScenes;
  bool operator==(const GraphKey& o) const {
    return tiles == o.tiles && active == o.active && rowsK == o.rowsK && scenes == o.scenes && flow == o.flow &&
           order == o.order && micTiles == o.micTiles && micScenes == o.micScenes;
  }
};

struct Engine {
  cudaStream_t stream = nullptr;
  float dt = 1.f;
  float cgAccuracy = 1e-3f, cgMaxIterFac = 1.5f;
  int lag = 8;
  std::vector<SceneRec*> members;
  std::multimap<size_t, void*> pool;
  size_t liveBytes = 0;
  // device tables
  BScene* dScenes = nullptr;
  size_t scenesCap = 0;
  CgScalars* dSc = nullptr;
  size_t scCap = 0;
  std::vector<CgScalars> hSc;
  std::vector<BScene> hScenes;
  // tiles: 32 x 8 for the stages; 32 x 8R (R = 1 << k) for the CG sweeps
  // MIC(0) for 3D scenes (the reference's PcMIC; 2D scenes run without a
  // preconditioner, as GridCg does in 2D): flow table, dispatch order
  bool micFor3D = true;
  // FP64 residual refinement of every scene's solve (off by default)
  bool refine = false;
  double refineAccuracy = 1e-5, innerAccuracy = 1e-2;
  int maxRefine = 10;
  std::vector<FlowScene> hFlow;
  std::vector<int2> hOrder2;
  std::vector<int> hMicScene;
  FlowScene* dFlow = nullptr;
  size_t flowCap = 0;
  int2* dOrder2 = nullptr;
  size_t orderCap = 0;
  int* dMicScene = nullptr;
  size_t micSceneCap = 0;
  int* dMicCounter = nullptr;  // [0] tile counter, [1] wait error, [2] sweep epoch
  // `lag` CG sweeps captured as a CUDA graph, and what it was captured with
  cudaGraphExec_t sweepGraph = nullptr;
  GraphKey graphKey{};
  unsigned long long graphNodes = 0;
  long long graphLaunches = 0;
  std::vector<BTile> tiles1;
  std::vector<BTile> tilesDam;  // the 32 x 8 tiles of the dam-break scenes
  BTile* dTilesDam = nullptr;
  size_t tilesDamCap = 0;
  std::vector<BTile> tilesR[4];
  std::vector<int> startR[4];
  BTile* dTiles = nullptr;
  size_t tilesCap = 0;
  BTile* dActive = nullptr;
  size_t activeCap = 0;
  bool dirty = true;
  int rowsK = -1;
  float tuneMs[4] = {0.f, 0.f, 0.f, 0.f};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  int* dDone = nullptr;

  ~Engine() {
    if (stream) cudaStreamSynchronize(stream);
    for (auto* m : members) {
      cudaFree(m->mem);
      cudaFree(m->refMem);
      delete m;
    }
    for (auto& kv : pool) cudaFree(kv.second);
    cudaFree(dScenes);
    cudaFree(dSc);
    cudaFree(dTiles);
    cudaFree(dActive);
    cudaFree(dDone);
    cudaFree(dFlow);
    cudaFree(dTilesDam);
    cudaFree(dOrder2);
    cudaFree(dMicScene);
    cudaFree(dMicCounter);
    if (sweepGraph) cudaGraphExecDestroy(sweepGraph);
    if (ev[0]) cudaEventDestroy(ev[0]);
    if (ev[1]) cudaEventDestroy(ev[1]);
    if (stream) cudaStreamDestroy(stream);
  }
};

int engine_init(Engine& e, float dt) {
  e.dt = dt;
  CKB(cudaStreamCreateWithFlags(&e.stream, cudaStreamNonBlocking));
  CKB(cudaEventCreate(&e.ev[0]));
  CKB(cudaEventCreate(&e.ev[1]));
  CKB(cudaMalloc(&e.dDone, sizeof(int)));
  CKB(cudaMalloc(&e.dMicCounter, 3 * sizeof(int)));
  CKB(cudaMemset(e.dMicCounter, 0, 3 * sizeof(int)));
  return MG_OK;
}

void* pool_take(Engine& e, size_t bytes) {
  auto it = e.pool.find(bytes);
  if (it != e.pool.end()) {
    void* p = it->second;
    e.pool.erase(it);
    return p;
  }
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    // return the pooled blocks to the device and retry once
    cudaStreamSynchronize(e.stream);
    for (auto& kv : e.pool) cudaFree(kv.second);
    e.pool.clear();
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
  }
  return p;
}

// a scene joins the engine: device block, flags and source set up.  kind 0
// is the smoke plume, kind 1 the dam break (a liquid box x < 0.4 nx,
// y < 0.6 ny in a closed domain)
int scene_add(Engine& e, int nx, int ny, int nz, const float* gravity, unsigned long long seed, SceneRec** out,
              int kind = 0) {
  if (nx < 3 || ny < 3 || nz < 1 || (nz > 1 && nz < 3)) return set_error(MG_ERR_ARG, "scene is too small");
  if ((long long)nx * ny * nz >= (1LL << 31)) return set_error(MG_ERR_ARG, "scene exceeds 2^31 - 1 cells");
  if (kind != 0 && kind != 1) return set_error(MG_ERR_ARG, "scene kind: 0 plume or 1 dam break");
  auto r = new SceneRec();
  r->bytes = scene_bytes(nx, ny, nz, kind);
  r->mem = pool_take(e, r->bytes);
  if (!r->mem) {
    delete r;
    return set_error(MG_ERR_NOMEM, "plume scene: out of device memory");
  }
  e.liveBytes += r->bytes;
  CKB(cudaMemsetAsync(r->mem, 0, r->bytes, e.stream));
  BScene& s = r->s;
  s.d.nx = nx;
  s.d.ny = ny;
  s.d.nz = nz;
  s.d.is3d = nz > 1;
  s.d.n = (long long)nx * ny * nz;
  s.d.sy = nx;
  s.d.sz = s.d.is3d ? (long long)nx * ny : 0;
  const size_t n = (size_t)s.d.n;
  unsigned char* p = (unsigned char*)r->mem;
  auto take = [&](size_t bytes) {
    unsigned char* q = p;
    p += align256(bytes);
    return q;
  };
  s.flags = (int*)take(n * sizeof(int));
  s.vel[0] = (float*)take(3 * n * sizeof(float));
  s.vel[1] = (float*)take(3 * n * sizeof(float));
  s.dens[0] = (float*)take(n * sizeof(float));
  s.dens[1] = (float*)take(n * sizeof(float));
  s.fwd = (float*)take(4 * n * sizeof(float));
  s.mask = (float*)take(n * sizeof(float));
  s.pres = (float*)take(n * sizeof(float));
  s.rhs = (float*)take(n * sizeof(float));
  s.res = (float*)take(n * sizeof(float));
  s.search = (float*)take(n * sizeof(float));
  s.tmp = (float*)take(n * sizeof(float));
  s.code = (code_t*)take(n * sizeof(code_t));
  s.ntiles = tiles_of(nx, ny, nz, kBTY);
  s.part = (double*)take(2 * (size_t)s.ntiles * sizeof(double));
  s.P = nullptr;
  s.face = nullptr;
  s.tx = mic_tiles(nx);
  s.ty = mic_tiles(ny);
  s.tz = mic_tiles(nz);
  if (nz > 1) {
    s.P = (float*)take(n * sizeof(float));
    s.face = (unsigned long long*)take(mic_flow_face_words(s.tx * s.ty * s.tz) * sizeof(unsigned long long));
  }
  s.mic = (nz > 1 && e.micFor3D) ? 1 : 0;
  s.kind = kind;
  s.A0f = nullptr;
  s.itmp = nullptr;
  s.p64 = nullptr;
  s.b64 = nullptr;
  if (kind == 1) {
    s.A0f = (float*)take(n * sizeof(float));
    s.itmp = (int*)take(n * sizeof(int));
  }
  s.sc = nullptr;
  s.dt = e.dt;
  s.seed = seed;
  s.step = 0;
  const int m = std::max(nx, std::max(ny, nz));
  const float gridScale = (float)(1.0 / (double)m);
  const float dt = e.dt;
  if (kind == 0) {
    // addBuoyancy(gravity, scale=True, coefficient=1): f = -g*dt/dx, 0.5*f
    s.bx = 0.5f * (((-gravity[0]) * dt) / gridScale * 1.f);
    s.by = 0.5f * (((-gravity[1]) * dt) / gridScale * 1.f);
    s.bz = 0.5f * (((-gravity[2]) * dt) / gridScale * 1.f);
  } else {
    // addGravity(gravity, scale=True): f = g*dt/dx (extforces.cpp:61-65)
    s.bx = (gravity[0] * dt) / gridScale;
    s.by = (gravity[1] * dt) / gridScale;
    s.bz = (gravity[2] * dt) / gridScale;
  }
  // initDomain(boundaryWidth=0) walls, fillGrid, setOpenBound(0, 'Y',
  // Outflow|Empty), Cylinder(center = gs*(0.5,0.1,0.5), radius = 0.14*nx,
  // z = gs*(0,0.02,0)).applyToGrid(mask, 1)
  const int wz = s.d.is3d ? kObstacle : 0;  // initDomain sets no z sides in 2D
  const int types[6] = {kObstacle, kObstacle, kObstacle, kObstacle, wz, wz};
  launch_init_domain(s.d, s.flags, 0, types, e.stream);
  if (kind == 1) {
    // the dam-break scene: phi = Box(p0 = 0, p1 = (0.4 nx, 0.6 ny, nz)).computeLevelset();
    // flags.updateFromLevelset(phi)
    const float p0[3] = {0.f, 0.f, 0.f};
    const float p1[3] = {(float)(0.4 * nx), (float)(0.6 * ny), (float)nz};
    launch_box_sdf(s.d, s.dens[0], p0, p1, e.stream);
    launch_update_from_levelset(s.d, s.flags, s.dens[0], e.stream);
    CKB(cudaGetLastError());
    e.members.push_back(r);
    e.dirty = true;
    *out = r;
    return MG_OK;
  }
  launch_fill_grid(s.d, s.flags, kFluid, e.stream);
  const int lo[3] = {0, 0, 0}, up[3] = {0, 1, 0};
  launch_set_open_bound(s.d, s.flags, 0, lo, up, kOutflow | kEmpty, e.stream);
  const float gs[3] = {(float)nx, (float)ny, (float)nz};
  const float center[3] = {gs[0] * 0.5f, gs[1] * 0.1f, gs[2] * 0.5f};
  const float zdir[3] = {gs[0] * 0.f, gs[1] * 0.02f, gs[2] * 0.f};
  float zn[3], mZ;
  cylinder_axis(zdir, zn, &mZ);
  const float one[3] = {1.f, 0.f, 0.f};
  launch_shape_apply(s.d, 1, s.mask, nullptr, nullptr, one, 0, nullptr, center, zn, (float)(nx * 0.14), mZ, e.stream);
  CKB(cudaGetLastError());
  e.members.push_back(r);
  e.dirty = true;
  *out = r;
  return MG_OK;
}

void scene_remove(Engine& e, SceneRec* r) {
  e.members.erase(std::find(e.members.begin(), e.members.end(), r));
  if (r->refMem) {
    cudaStreamSynchronize(e.stream);
    cudaFree(r->refMem);
  }
  e.pool.emplace(r->bytes, r->mem);
  e.liveBytes -= r->bytes;
  delete r;
  e.dirty = true;
}

template <typename T>
int ensure_cap(T** p, size_t* cap, size_t want) {
  if (*cap >= want) return MG_OK;
  const size_t c = std::max(want, *cap * 2);
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  CKB(cudaMalloc(p, sizeof(T) * c));
  *cap = c;
  return MG_OK;
}

// scene table (each scene's current buffers presented as index 0, its step
// index) and, after a membership change, the tile lists
int engine_tables(Engine& e) {
  const size_t nm = e.members.size();
  if (ensure_cap(&e.dScenes, &e.scenesCap, nm) || ensure_cap(&e.dSc, &e.scCap, nm)) return MG_ERR_CUDA;
  e.hScenes.resize(nm);
  e.hSc.resize(nm);
  for (size_t q = 0; q < nm; q++) {
    BScene s = e.members[q]->s;
    s.sc = e.dSc + q;
    s.step = e.members[q]->step;
    if (e.members[q]->cur) {
      std::swap(s.vel[0], s.vel[1]);
      std::swap(s.dens[0], s.dens[1]);
    }
    e.hScenes[q] = s;
  }
  CKB(cudaMemcpyAsync(e.dScenes, e.hScenes.data(), sizeof(BScene) * nm, cudaMemcpyHostToDevice, e.stream));
  if (!e.dirty) return MG_OK;
  e.tiles1.clear();
  e.tilesDam.clear();
  for (int k = 0; k < 4; k++) {
    e.tilesR[k].clear();
    e.startR[k].clear();
  }
  for (size_t q = 0; q < nm; q++) {
    const Dims& d = e.members[q]->s.d;
    const int cnt1 = tiles_of(d.nx, d.ny, d.nz, kBTY);
    int local = 0;
    for (int z = 0; z < d.nz; z++)
      for (int y = 0; y < d.ny; y += kBTY)
        for (int x = 0; x < d.nx; x += kBTX) {
          e.tiles1.push_back(BTile{(int)q, x, y, z, local, cnt1});
          if (e.members[q]->s.kind == 1) e.tilesDam.push_back(BTile{(int)q, x, y, z, local, cnt1});
          local++;
        }
    for (int k = 0; k < 4; k++) {
      const int rows = kBTY << k;
      const int cnt = tiles_of(d.nx, d.ny, d.nz, rows);
      e.startR[k].push_back((int)e.tilesR[k].size());
      int l = 0;
      for (int z = 0; z < d.nz; z++)
        for (int y = 0; y < d.ny; y += rows)
          for (int x = 0; x < d.nx; x += kBTX) e.tilesR[k].push_back(BTile{(int)q, x, y, z, l++, cnt});
    }
  }
  for (int k = 0; k < 4; k++) e.startR[k].push_back((int)e.tilesR[k].size());
  // MIC scenes: one FlowScene each; tiles ordered by wavefront level (a+b+c
  // within the scene) and then scene, so a tile comes after every tile it
  // waits for
  e.hFlow.clear();
  e.hOrder2.clear();
  e.hMicScene.clear();
  int maxLevel = 0;
  for (size_t q = 0; q < nm; q++) {
    const BScene& b = e.hScenes[q];
    if (!b.mic) continue;
    FlowScene f;
    f.d = b.d;
    f.code = b.code;
    f.A0f = b.A0f;  // ghost-fluid diagonal of dam-break scenes
    f.P = b.P;
    f.r = b.res;
    f.z = b.tmp;
    f.part = b.part;
    f.sc = b.sc;
    f.tx = b.tx;
    f.ty = b.ty;
    f.tz = b.tz;
    f.face = b.face;
    e.hFlow.push_back(f);
    e.hMicScene.push_back((int)q);
    maxLevel = std::max(maxLevel, b.tx + b.ty + b.tz - 3);
  }
  for (int L = 0; L <= maxLevel; L++)
    for (size_t m = 0; m < e.hFlow.size(); m++) {
      const FlowScene& f = e.hFlow[m];
      for (int c = 0; c < f.tz; c++)
        for (int b = 0; b < f.ty; b++) {
          const int a = L - b - c;
          if (a >= 0 && a < f.tx) e.hOrder2.push_back(make_int2((int)m, a + f.tx * (b + f.ty * c)));
        }
    }
  if (!e.hFlow.empty()) {
    if (ensure_cap(&e.dFlow, &e.flowCap, e.hFlow.size()) || ensure_cap(&e.dOrder2, &e.orderCap, e.hOrder2.size()) ||
        ensure_cap(&e.dMicScene, &e.micSceneCap, e.hMicScene.size()))
      return MG_ERR_CUDA;
    CKB(cudaMemcpyAsync(e.dFlow, e.hFlow.data(), sizeof(FlowScene) * e.hFlow.size(), cudaMemcpyHostToDevice, e.stream));
    CKB(cudaMemcpyAsync(e.dOrder2, e.hOrder2.data(), sizeof(int2) * e.hOrder2.size(), cudaMemcpyHostToDevice, e.stream));
    CKB(cudaMemcpyAsync(e.dMicScene, e.hMicScene.data(), sizeof(int) * e.hMicScene.size(), cudaMemcpyHostToDevice,
                        e.stream));
  }
  if (ensure_cap(&e.dTiles, &e.tilesCap, e.tiles1.size()) || ensure_cap(&e.dActive, &e.activeCap, e.tiles1.size()))
    return MG_ERR_CUDA;
  CKB(cudaMemcpyAsync(e.dTiles, e.tiles1.data(), sizeof(BTile) * e.tiles1.size(), cudaMemcpyHostToDevice, e.stream));
  if (!e.tilesDam.empty()) {
    if (ensure_cap(&e.dTilesDam, &e.tilesDamCap, e.tilesDam.size())) return MG_ERR_CUDA;
    CKB(cudaMemcpyAsync(e.dTilesDam, e.tilesDam.data(), sizeof(BTile) * e.tilesDam.size(), cudaMemcpyHostToDevice,
                        e.stream));
  }
  e.dirty = false;
  return MG_OK;
}

int engine_tables(Engine& e);

// the double pressure and right-hand side of every member (FP64 refinement),
// allocated on first use; the scene table is uploaded again
int engine_refine_buffers(Engine& e) {
  bool changed = false;
  for (auto* m : e.members) {
    if (m->refMem) continue;
    const size_t n = (size_t)m->s.d.n;
    if (cudaMalloc(&m->refMem, 2 * n * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      m->refMem = nullptr;
      return set_error(MG_ERR_NOMEM, "batched refinement: out of device memory");
    }
    m->s.p64 = (double*)m->refMem;
    m->s.b64 = (double*)m->refMem + n;
    changed = true;
  }
  return changed ? engine_tables(e) : MG_OK;
}

// One batched GridCg solve (pressure.cpp:407-419) of every scene not
// skipped, each to its own accuracy: PcMIC in 3D with (int)(cgMaxIterFac *
// max size) iterations at most; in 2D GridCg drops MIC (conjugategrad.cpp:
// 315-321) and allows 4 times as many.  The right-hand side is in rhs.
int engine_cg(Engine& e, const BatchMic& mic, const std::vector<float>& acc, const std::vector<char>& skip,
              int* sweepsOut) {
  const int nm = (int)e.members.size();
  const int nt = (int)e.tiles1.size();
  cudaStream_t st = e.stream;
  int maxIterAll = 0, nskip = 0;
  for (int q = 0; q < nm; q++) {
    const Dims& d = e.members[q]->s.d;
    CgScalars c{};
    c.accuracy = acc[q];
    c.maxIter = (int)(e.cgMaxIterFac * (float)std::max(d.nx, std::max(d.ny, d.nz))) * (d.is3d ? 1 : 4);
    c.resNorm = 1e20f;
    c.refNorm = e.hSc[q].refNorm;
    if (skip[q]) {
      c.done = 1;
      nskip++;
    }
    e.hSc[q] = c;
    if (!skip[q]) maxIterAll = std::max(maxIterAll, c.maxIter);
  }
  CKB(cudaMemcpyAsync(e.dSc, e.hSc.data(), sizeof(CgScalars) * nm, cudaMemcpyHostToDevice, st));
  CKB(cudaMemcpyAsync(e.dDone, &nskip, sizeof(int), cudaMemcpyHostToDevice, st));
  launch_b_pcg_init(e.dTiles, nt, e.dScenes, st);
  if (mic.nscenes > 0) launch_b_mic_init(e.dTiles, nt, e.dScenes, mic, st);
  // CG sweeps over the tiles of the scenes still iterating.  Autotuner: the
  // first solve runs its first 4 x lag sweeps with tiles 8, 16, 32 and 64
  // rows tall (lag sweeps each, timed with events) and keeps the fastest;
  // results do not depend on the choice.
  int kk = e.rowsK >= 0 ? e.rowsK : 0;
  int active = 0, doneSeen = -1, sweeps = 0;
  (void)nt;
  std::vector<BTile> list;
  auto rebuild = [&](bool all) -> int {
    list.clear();
    for (int q = 0; q < nm; q++)
      if (all || !e.hSc[q].done)
        list.insert(list.end(), e.tilesR[kk].begin() + e.startR[kk][q], e.tilesR[kk].begin() + e.startR[kk][q + 1]);
    active = (int)list.size();
    if (active) CKB(cudaMemcpyAsync(e.dActive, list.data(), sizeof(BTile) * active, cudaMemcpyHostToDevice, st));
    return MG_OK;
  };
  if (rebuild(false)) return MG_ERR_CUDA;
  const bool tuning = e.rowsK < 0;
  if (tuning) CKB(cudaEventRecord(e.ev[0], st));
  while (active > 0 && sweeps < maxIterAll) {
    // once the tile height is tuned, `lag` sweeps run as one CUDA graph,
    // captured for the current sweep list and captured again when it changes
    const bool useGraph = !(tuning && e.rowsK < 0) && sweeps % e.lag == 0 && sweeps + e.lag <= maxIterAll;
    if (useGraph) {
      const GraphKey key{e.dActive, active, kk, e.dScenes, mic.flow, mic.order, mic.ntiles, mic.nscenes};
      if (!e.sweepGraph || !(key == e.graphKey)) {
        if (e.sweepGraph) cudaGraphExecDestroy(e.sweepGraph);
        e.sweepGraph = nullptr;
        const unsigned long long before = t_launches;
        cudaGraph_t g = nullptr;
        CKB(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        for (int q = 0; q < e.lag; q++) launch_b_pcg_iteration(e.dActive, active, e.dScenes, 1 << kk, e.dDone, &mic, st);
        const cudaError_t ce = cudaStreamEndCapture(st, &g);
        e.graphNodes = uncount_captured(before);
        if (ce != cudaSuccess) {
          if (g) cudaGraphDestroy(g);
          return set_error(MG_ERR_CUDA, std::string("capturing the batched CG sweeps failed: ") + cudaGetErrorString(ce));
        }
        const cudaError_t ie = cudaGraphInstantiate(&e.sweepGraph, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
          e.sweepGraph = nullptr;
          return set_error(MG_ERR_CUDA, std::string("instantiating the batched CG sweeps failed: ") + cudaGetErrorString(ie));
        }
        e.graphKey = key;
      }
      CKB(cudaGraphLaunch(e.sweepGraph, st));
      g_launches.fetch_add(e.graphNodes, std::memory_order_relaxed);
      e.graphLaunches++;
      sweeps += e.lag;
    } else {
      launch_b_pcg_iteration(e.dActive, active, e.dScenes, 1 << kk, e.dDone, &mic, st);
      sweeps++;
    }
    if (sweeps % e.lag == 0 || sweeps == maxIterAll) {
      bool relist = false;
      if (tuning && e.rowsK < 0 && sweeps <= 4 * e.lag) {
        CKB(cudaEventRecord(e.ev[1], st));
        CKB(cudaEventSynchronize(e.ev[1]));
        float ms = 0.f;
        CKB(cudaEventElapsedTime(&ms, e.ev[0], e.ev[1]));
        e.tuneMs[kk] = ms;
        if (kk < 3) {
          kk++;
          relist = true;
        } else {
          int best = 0;
          for (int q = 1; q < 4; q++)
            if (e.tuneMs[q] < e.tuneMs[best]) best = q;
          e.rowsK = best;
          relist = kk != best;
          kk = best;
        }
      }
      int nd = 0;
      CKB(cudaMemcpyAsync(&nd, e.dDone, sizeof(int), cudaMemcpyDeviceToHost, st));
      CKB(cudaStreamSynchronize(st));
      if (nd >= nm) break;
      if (nd != doneSeen || relist) {
        doneSeen = nd;
        CKB(cudaMemcpyAsync(e.hSc.data(), e.dSc, sizeof(CgScalars) * nm, cudaMemcpyDeviceToHost, st));
        CKB(cudaStreamSynchronize(st));
        if (rebuild(false)) return MG_ERR_CUDA;
      }
      if (tuning && e.rowsK < 0) CKB(cudaEventRecord(e.ev[0], st));
    }
  }
  *sweepsOut = sweeps;
  CKB(cudaStreamSynchronize(st));
  return MG_OK;
}

// one plume step of every member
int engine_step(Engine& e, mg_batch_stats* stats) {
  if (e.members.empty()) return MG_OK;
  if (engine_tables(e)) return MG_ERR_CUDA;
  const int nm = (int)e.members.size();
  const int nt = (int)e.tiles1.size();
  cudaStream_t st = e.stream;
  const int cur = 0, nxt = 1;  // the table presents every scene's current buffers as 0
  const int ntDam = (int)e.tilesDam.size();
  launch_b_inflow(e.dTiles, nt, e.dScenes, cur, st);
  launch_b_advect_velocity(e.dTiles, nt, e.dScenes, cur, st);
  launch_b_dam_advect(e.dTilesDam, ntDam, e.dScenes, cur, st);
  launch_b_forces(e.dTiles, nt, e.dScenes, nxt, st);
  launch_b_pressure_setup(e.dTiles, nt, e.dScenes, nxt, st, e.dTilesDam, ntDam);
  BatchMic mic;
  mic.flow = e.dFlow;
  mic.order = e.dOrder2;
  mic.ntiles = (int)e.hOrder2.size();
  mic.nscenes = (int)e.hFlow.size();
  mic.ctas = mic_flow_device_ctas();
  mic.sceneOf = e.dMicScene;
  mic.counter = e.dMicCounter;
  mic.error = e.dMicCounter + 1;
  mic.epochDev = (unsigned int*)(e.dMicCounter + 2);
  mic.spinLimit = 200000000LL;
  if (mic.nscenes > 0) CKB(cudaMemsetAsync(mic.error, 0, sizeof(int), st));
  std::vector<char> skip(nm, 0);
  std::vector<float> acc(nm, e.cgAccuracy);
  const long long graphLaunches0 = e.graphLaunches;
  int sweeps = 0, st1 = engine_cg(e, mic, acc, skip, &sweeps);
  if (st1) return st1;
  int refinements = 0;
  if (e.refine) {
    // FP64 residual refinement (the precision form, refine.cu) per scene:
    // p64 accumulates the FP32 solutions, r = b - A p64 in double; scenes
    // whose max|r| is below refineAccuracy stop, the others solve A delta = r
    // in FP32 to innerAccuracy * max|r|
    if (engine_refine_buffers(e)) return MG_ERR_NOMEM;
    launch_b_ref_first(e.dTiles, nt, e.dScenes, st);
    for (refinements = 1; refinements <= e.maxRefine; refinements++) {
      launch_b_ref_residual(e.dTiles, nt, e.dScenes, st);
      CKB(cudaMemcpyAsync(e.hSc.data(), e.dSc, sizeof(CgScalars) * nm, cudaMemcpyDeviceToHost, st));
      CKB(cudaStreamSynchronize(st));
      int open = 0;
      for (int q = 0; q < nm; q++) {
        skip[q] = !(e.hSc[q].refNorm >= e.refineAccuracy);
        acc[q] = (float)(e.innerAccuracy * e.hSc[q].refNorm);
        if (!skip[q] && !(acc[q] > 1e-30f)) skip[q] = 1;
        open += !skip[q];
      }
      if (!open || refinements == e.maxRefine) break;
      int sw = 0;
      st1 = engine_cg(e, mic, acc, skip, &sw);
      if (st1) return st1;
      sweeps += sw;
      launch_b_ref_add(e.dTiles, nt, e.dScenes, st);
    }
    launch_b_ref_finish(e.dTiles, nt, e.dScenes, st);
  }
  launch_b_correct(e.dTiles, nt, e.dScenes, nxt, st);
  launch_b_dam_correct(e.dTilesDam, ntDam, e.dScenes, nxt, st);
  CKB(cudaMemcpyAsync(e.hSc.data(), e.dSc, sizeof(CgScalars) * nm, cudaMemcpyDeviceToHost, st));
  CKB(cudaStreamSynchronize(st));
  CKB(cudaGetLastError());
  for (auto* m : e.members) {
    m->cur = 1 - m->cur;
    m->step++;
  }
  if (stats) {
    stats->sweeps = sweeps;
    stats->graphLaunches = e.graphLaunches - graphLaunches0;
    int mx = 0, diverged = 0;
    long long sum = 0;
    for (auto& c : e.hSc) {
      mx = std::max(mx, c.iterations);
      sum += c.iterations;
      diverged += c.status == 2;
    }
    stats->maxIterations = mx;
    stats->totalIterations = sum;
    stats->diverged = diverged;
  }
  if (mic.nscenes > 0) {
    int err = 0;
    CKB(cudaMemcpy(&err, mic.error, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) return set_error(MG_ERR_TIMEOUT, "MIC wavefront (batched): a tile wait exceeded its spin limit");
  }
  for (auto& c : e.hSc)
    if (c.status == 2)
      return set_error(MG_ERR_SOLVER, "GridCg::iterate: The CG solver diverged, residual norm > 1e30, stopping.");
  return MG_OK;
}

int scene_download(Engine& e, SceneRec* r, int what, void* host, size_t bytes) {
  const BScene& s = r->s;
  const size_t n = (size_t)s.d.n;
  const size_t want = what == MG_BATCH_VELOCITY ? 3 * n * sizeof(float) : n * sizeof(float);
  if (bytes != want) return set_error(MG_ERR_ARG, "download: byte count does not match the scene");
  cudaStream_t st = e.stream;
  switch (what) {
    case MG_BATCH_DENSITY: CKB(cudaMemcpyAsync(host, s.dens[r->cur], want, cudaMemcpyDeviceToHost, st)); break;
    case MG_BATCH_PRESSURE: CKB(cudaMemcpyAsync(host, s.pres, want, cudaMemcpyDeviceToHost, st)); break;
    case MG_BATCH_FLAGS: CKB(cudaMemcpyAsync(host, s.flags, want, cudaMemcpyDeviceToHost, st)); break;
    case MG_BATCH_SOURCE: CKB(cudaMemcpyAsync(host, s.mask, want, cudaMemcpyDeviceToHost, st)); break;
    case MG_BATCH_VELOCITY: {
      // SoA planes -> the reference's AoS Vec3 on the host
      std::vector<float> h(3 * n);
      CKB(cudaMemcpyAsync(h.data(), s.vel[r->cur], want, cudaMemcpyDeviceToHost, st));
      CKB(cudaStreamSynchronize(st));
      float* o = (float*)host;
      for (size_t i = 0; i < n; i++) {
        o[3 * i] = h[i];
        o[3 * i + 1] = h[n + i];
        o[3 * i + 2] = h[2 * n + i];
      }
      return MG_OK;
    }
    default: return set_error(MG_ERR_ARG, "download: unknown field");
  }
  CKB(cudaStreamSynchronize(st));
  return MG_OK;
}

}  // namespace

// ============================================================== batched form
struct mg_batch_s {
  Engine e;
  std::vector<SceneRec*> scenes;  // creation order
};

extern "C" int mg_batch_create(int count, const int* sizes, const float* gravity, const unsigned long long* seeds, float dt,
                               mg_batch* out) {
  if (!library_ready()) return set_error(MG_ERR_STATE, "mg_init has not been called");
  if (count < 1 || !sizes || !gravity || !seeds || !out) return set_error(MG_ERR_ARG, "mg_batch_create: invalid argument");
  auto b = new mg_batch_s();
  int st = engine_init(b->e, dt);
  for (int q = 0; q < count && !st; q++) {
    SceneRec* r = nullptr;
    st = scene_add(b->e, sizes[3 * q], sizes[3 * q + 1], sizes[3 * q + 2], gravity + 3 * q, seeds[q], &r);
    if (!st) b->scenes.push_back(r);
  }
  if (!st && cudaStreamSynchronize(b->e.stream) != cudaSuccess) st = set_error(MG_ERR_CUDA, "mg_batch_create: setup failed");
  if (st) {
    delete b;
    return st;
  }
  *out = b;
  return MG_OK;
}

extern "C" int mg_batch_destroy(mg_batch b) {
  delete b;
  return MG_OK;
}

extern "C" int mg_batch_set_solver(mg_batch b, float cgAccuracy, float cgMaxIterFac) {
  if (!b || !(cgAccuracy > 0.f) || !(cgMaxIterFac > 0.f)) return set_error(MG_ERR_ARG, "mg_batch_set_solver: invalid argument");
  b->e.cgAccuracy = cgAccuracy;
  b->e.cgMaxIterFac = cgMaxIterFac;
  return MG_OK;
}

extern "C" int mg_batch_set_refinement(mg_batch b, double refineAccuracy, double innerAccuracy, int maxRefine) {
  if (!b || refineAccuracy < 0. || !(innerAccuracy > 0.) || maxRefine < 1)
    return set_error(MG_ERR_ARG, "mg_batch_set_refinement: invalid argument");
  b->e.refine = refineAccuracy > 0.;
  b->e.refineAccuracy = refineAccuracy;
  b->e.innerAccuracy = innerAccuracy;
  b->e.maxRefine = maxRefine;
  return MG_OK;
}

extern "C" int mg_batch_set_preconditioner(mg_batch b, int preconditioner) {
  if (!b || (preconditioner != MG_PC_NONE && preconditioner != MG_PC_MIC))
    return set_error(MG_ERR_ARG, "mg_batch_set_preconditioner: PcNone or PcMIC");
  b->e.micFor3D = preconditioner == MG_PC_MIC;
  for (auto* m : b->e.members) m->s.mic = (m->s.d.is3d && b->e.micFor3D) ? 1 : 0;
  b->e.dirty = true;
  return MG_OK;
}

extern "C" int mg_batch_step(mg_batch b, mg_batch_stats* stats) {
  if (!b) return set_error(MG_ERR_ARG, "mg_batch_step: null batch");
  return engine_step(b->e, stats);
}

extern "C" int mg_batch_scene_iterations(mg_batch b, int scene, int* iterations, float* resNorm) {
  if (!b || scene < 0 || scene >= (int)b->scenes.size()) return set_error(MG_ERR_ARG, "mg_batch_scene_iterations: invalid scene");
  const auto& m = b->e.members;
  const size_t q = std::find(m.begin(), m.end(), b->scenes[scene]) - m.begin();
  const bool have = q < b->e.hSc.size();
  if (iterations) *iterations = have ? b->e.hSc[q].iterations : 0;
  if (resNorm) *resNorm = have ? b->e.hSc[q].resNorm : 0.f;
  return MG_OK;
}

extern "C" int mg_batch_download(mg_batch b, int scene, int what, void* host, size_t bytes) {
  if (!b || scene < 0 || scene >= (int)b->scenes.size() || !host) return set_error(MG_ERR_ARG, "mg_batch_download: invalid argument");
  return scene_download(b->e, b->scenes[scene], what, host, bytes);
}

extern "C" int mg_batch_noise(unsigned long long seed, int step, long long cells, float* out) {
  if (!out || cells < 0) return set_error(MG_ERR_ARG, "mg_batch_noise: invalid argument");
  for (long long i = 0; i < cells; i++) out[i] = batch_noise(seed, step, i);
  return MG_OK;
}

extern "C" int mg_batch_tuning(mg_batch b, int* sweepRows, float* ms) {
  if (!b) return set_error(MG_ERR_ARG, "mg_batch_tuning: null batch");
  if (sweepRows) *sweepRows = b->e.rowsK < 0 ? 0 : kBTY << b->e.rowsK;
  if (ms)
    for (int q = 0; q < 4; q++) ms[q] = b->e.tuneMs[q];
  return MG_OK;
}

extern "C" int mg_batch_info(mg_batch b, int* count, long long* cells, long long* tiles, size_t* bytes) {
  if (!b) return set_error(MG_ERR_ARG, "mg_batch_info: null batch");
  long long c = 0, t = 0;
  for (auto* r : b->scenes) {
    c += r->s.d.n;
    t += r->s.ntiles;
  }
  if (count) *count = (int)b->scenes.size();
  if (cells) *cells = c;
  if (tiles) *tiles = t;
  if (bytes) *bytes = b->e.liveBytes;
  return MG_OK;
}

extern "C" int mg_batch_sync(mg_batch b) {
  if (!b) return set_error(MG_ERR_ARG, "mg_batch_sync: null batch");
  CKB(cudaStreamSynchronize(b->e.stream));
  return MG_OK;
}

// =============================================================== served form
namespace {
struct Job {
  int kind = 0;  // 0 plume, 1 dam break
  int nx, ny, nz;
  float gravity[3];
  unsigned long long seed;
  int steps;
  double arrival;  // seconds after the run starts
  int keep;        // copy the final fields to the host
  // outcome
  double admitted = -1., finished = -1.;
  int stepsDone = 0;
  double stepMsSum = 0.;
  std::vector<float> dens, vel, pres;
  SceneRec* rec = nullptr;
};
}  // namespace

struct mg_server_s {
  Engine e;
  size_t budget = 0;
  std::vector<Job> jobs;
  std::vector<float> tickMs;
  std::vector<int> tickJobs;
  double wall = 0.;
  long long cellSteps = 0;
  size_t peakBytes = 0;
};

extern "C" int mg_serve_create(size_t budgetBytes, float dt, mg_server* out) {
  if (!library_ready()) return set_error(MG_ERR_STATE, "mg_init has not been called");
  if (!out || budgetBytes == 0) return set_error(MG_ERR_ARG, "mg_serve_create: invalid argument");
  auto s = new mg_server_s();
  s->budget = budgetBytes;
  const int st = engine_init(s->e, dt);
  if (st) {
    delete s;
    return st;
  }
  *out = s;
  return MG_OK;
}

extern "C" int mg_serve_destroy(mg_server s) {
  delete s;
  return MG_OK;
}

extern "C" int mg_serve_set_solver(mg_server s, float cgAccuracy, float cgMaxIterFac) {
  if (!s || !(cgAccuracy > 0.f) || !(cgMaxIterFac > 0.f)) return set_error(MG_ERR_ARG, "mg_serve_set_solver: invalid argument");
  s->e.cgAccuracy = cgAccuracy;
  s->e.cgMaxIterFac = cgMaxIterFac;
  return MG_OK;
}

extern "C" size_t mg_serve_job_bytes(int nx, int ny, int nz) { return scene_bytes(nx, ny, nz); }
extern "C" size_t mg_serve_job_bytes_kind(int kind, int nx, int ny, int nz) { return scene_bytes(nx, ny, nz, kind); }

extern "C" int mg_serve_submit_kind(mg_server s, int kind, int nx, int ny, int nz, const float* gravity,
                                    unsigned long long seed, int steps, double arrival, int keepResult, int* job) {
  if (!s || !gravity || steps < 1 || arrival < 0.) return set_error(MG_ERR_ARG, "mg_serve_submit: invalid argument");
  if (kind != 0 && kind != 1) return set_error(MG_ERR_ARG, "mg_serve_submit: kind is 0 (plume) or 1 (dam break)");
  if (nx < 3 || ny < 3 || nz < 1 || (nz > 1 && nz < 3)) return set_error(MG_ERR_ARG, "mg_serve_submit: scene is too small");
  if (scene_bytes(nx, ny, nz, kind) > s->budget)
    return set_error(MG_ERR_ARG, "mg_serve_submit: the job alone exceeds the memory budget");
  Job j;
  j.kind = kind;
  j.nx = nx;
  j.ny = ny;
  j.nz = nz;
  std::memcpy(j.gravity, gravity, sizeof j.gravity);
  j.seed = seed;
  j.steps = steps;
  j.arrival = arrival;
  j.keep = keepResult;
  s->jobs.push_back(std::move(j));
  if (job) *job = (int)s->jobs.size() - 1;
  return MG_OK;
}

extern "C" int mg_serve_submit(mg_server s, int nx, int ny, int nz, const float* gravity, unsigned long long seed, int steps,
                               double arrival, int keepResult, int* job) {
  return mg_serve_submit_kind(s, 0, nx, ny, nz, gravity, seed, steps, arrival, keepResult, job);
}

// run until every submitted job has finished.  Arrival times are honoured
// against the wall clock: with nothing resident the loop waits for the next
// arrival.
extern "C" int mg_serve_run(mg_server s, mg_serve_stats* stats) {
  if (!s) return set_error(MG_ERR_ARG, "mg_serve_run: null server");
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  auto now = [&]() { return std::chrono::duration<double>(clk::now() - t0).count(); };
  std::vector<int> order;
  for (size_t q = 0; q < s->jobs.size(); q++)
    if (s->jobs[q].finished < 0.) order.push_back((int)q);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return s->jobs[a].arrival < s->jobs[b].arrival; });
  size_t next = 0, finished = 0;
  std::vector<int> resident;
  while (finished < order.size()) {
    // admission in arrival order while the next job has arrived and fits
    const double tn = now();
    while (next < order.size()) {
      Job& j = s->jobs[order[next]];
      if (j.arrival > tn) break;
      if (s->e.liveBytes + scene_bytes(j.nx, j.ny, j.nz, j.kind) > s->budget) break;
      SceneRec* r = nullptr;
      const int st = scene_add(s->e, j.nx, j.ny, j.nz, j.gravity, j.seed, &r, j.kind);
      if (st) return st;
      j.rec = r;
      j.admitted = now();
      resident.push_back(order[next]);
      next++;
    }
    s->peakBytes = std::max(s->peakBytes, s->e.liveBytes);
    if (resident.empty()) {
      const double wait = s->jobs[order[next]].arrival - now();
      if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.01)));
      continue;
    }
    const double ta = now();
    const int st = engine_step(s->e, nullptr);
    if (st) return st;
    const double dtick = now() - ta;
    s->tickMs.push_back((float)(1e3 * dtick));
    s->tickJobs.push_back((int)resident.size());
    std::vector<int> still;
    for (int id : resident) {
      Job& j = s->jobs[id];
      j.stepsDone++;
      j.stepMsSum += 1e3 * dtick;
      s->cellSteps += (long long)j.nx * j.ny * j.nz;
      if (j.stepsDone < j.steps) {
        still.push_back(id);
        continue;
      }
      if (j.keep) {
        const size_t n = (size_t)j.nx * j.ny * j.nz;
        j.dens.resize(n);
        j.pres.resize(n);
        j.vel.resize(3 * n);
        int e1 = scene_download(s->e, j.rec, MG_BATCH_DENSITY, j.dens.data(), n * sizeof(float));
        if (!e1) e1 = scene_download(s->e, j.rec, MG_BATCH_PRESSURE, j.pres.data(), n * sizeof(float));
        if (!e1) e1 = scene_download(s->e, j.rec, MG_BATCH_VELOCITY, j.vel.data(), 3 * n * sizeof(float));
        if (e1) return e1;
      }
      scene_remove(s->e, j.rec);
      j.rec = nullptr;
      j.finished = now();
      finished++;
    }
    resident.swap(still);
  }
  s->wall = now();
  if (stats) {
    stats->jobs = (int)order.size();
    stats->ticks = (long long)s->tickMs.size();
    stats->wallSeconds = s->wall;
    stats->cellSteps = s->cellSteps;
    stats->peakBytes = s->peakBytes;
  }
  return MG_OK;
}

extern "C" int mg_serve_job_info(mg_server s, int job, mg_serve_job* info) {
  if (!s || job < 0 || job >= (int)s->jobs.size() || !info) return set_error(MG_ERR_ARG, "mg_serve_job_info: invalid job");
  const Job& j = s->jobs[job];
  info->arrival = j.arrival;
  info->admitted = j.admitted;
  info->finished = j.finished;
  info->steps = j.stepsDone;
  info->meanStepMs = j.stepsDone ? j.stepMsSum / j.stepsDone : 0.;
  return MG_OK;
}

extern "C" int mg_serve_job_result(mg_server s, int job, int what, void* host, size_t bytes) {
  if (!s || job < 0 || job >= (int)s->jobs.size() || !host) return set_error(MG_ERR_ARG, "mg_serve_job_result: invalid job");
  const Job& j = s->jobs[job];
  const std::vector<float>* v = what == MG_BATCH_DENSITY    ? &j.dens
                                : what == MG_BATCH_VELOCITY ? &j.vel
                                : what == MG_BATCH_PRESSURE ? &j.pres
                                                            : nullptr;
  if (!v) return set_error(MG_ERR_ARG, "mg_serve_job_result: density, velocity or pressure only");
  if (v->empty()) return set_error(MG_ERR_STATE, "mg_serve_job_result: the job kept no result (or has not finished)");
  if (bytes != v->size() * sizeof(float)) return set_error(MG_ERR_ARG, "mg_serve_job_result: byte count does not match");
  std::memcpy(host, v->data(), bytes);
  return MG_OK;
}

extern "C" int mg_serve_ticks(mg_server s, int* count, float* ms, int* jobs) {
  if (!s || !count) return set_error(MG_ERR_ARG, "mg_serve_ticks: invalid argument");
  const int n = std::min(*count, (int)s->tickMs.size());
  for (int q = 0; q < n; q++) {
    if (ms) ms[q] = s->tickMs[q];
    if (jobs) jobs[q] = s->tickJobs[q];
  }
  *count = (int)s->tickMs.size();
  return MG_OK;
}
