// Batched form of the plume step: many independent scenes of uneven sizes,
// each stage one launch over all scenes' tiles (mg_batch.h).
//
// Memory: one arena per batch.  Per scene (n cells): flags, two velocity
// buffers (3n, ping-pong), two density buffers, 4n forward/scratch values,
// the inflow mask, pressure and the CG vectors rhs / residual / search / tmp,
// plus 2-byte stencil codes: ~80 bytes per cell.  Scenes start on 256-byte
// boundaries.
//
// Step: inflow, advection (forward SL of density and velocity in one pass,
// MacCormack correction + clamp in the next, outflow BC), setWallBcs +
// addBuoyancy, then solvePressure: MakeRhs + codes, CG init, CG iterations
// until every scene has converged, correctVelocity.  CG iterations run over
// the tiles of the scenes still iterating: the host reads the number of
// finished scenes every few iterations and, when it changed, drops their
// tiles from the list.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mantagpu.h"
#include "mg_batch.h"

using namespace mgpu;

struct mg_batch_s {
  int count = 0;
  float dt = 1.f;
  cudaStream_t stream = nullptr;
  unsigned char* arena = nullptr;
  size_t arenaBytes = 0;
  std::vector<BScene> scenes;     // host copy of the table
  BScene* dScenes = nullptr;
  std::vector<BTile> tiles;       // all 32 x 8 tiles, scene-major
  std::vector<int> tileStart;     // first tile of each scene
  BTile* dTiles = nullptr;
  // CG sweep tiles 32 x 8R cells for R = 1, 2, 4, 8 (rowsK[k] = 1 << k)
  std::vector<BTile> tilesR[4];
  std::vector<int> startR[4];
  BTile* dActive = nullptr;       // sweep tiles of the scenes still iterating
  int rowsK = -1;                 // autotuned sweep tile height (index), -1 until chosen
  float tuneMs[4] = {0.f, 0.f, 0.f, 0.f};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  CgScalars* dSc = nullptr;
  std::vector<CgScalars> hSc;
  int* dDone = nullptr;
  int cur = 0;
  int step = 0;
  float cgAccuracy = 1e-3f;
  float cgMaxIterFac = 1.5f;
  int lag = 8;
};

#define CKB(call)                                                                                  \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return set_error(MG_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

extern "C" int mg_batch_create(int count, const int* sizes, const float* gravity, const unsigned long long* seeds, float dt,
                               mg_batch* out) {
  if (!library_ready()) return set_error(MG_ERR_STATE, "mg_init has not been called");
  if (count < 1 || !sizes || !gravity || !seeds || !out) return set_error(MG_ERR_ARG, "mg_batch_create: invalid argument");
  auto b = new mg_batch_s();
  b->count = count;
  b->dt = dt;
  // layout
  std::vector<size_t> off(count);
  size_t total = 0;
  for (int q = 0; q < count; q++) {
    const int nx = sizes[3 * q], ny = sizes[3 * q + 1], nz = sizes[3 * q + 2];
    if (nx < 3 || ny < 3 || nz < 1 || (nz > 1 && nz < 3)) {
      delete b;
      return set_error(MG_ERR_ARG, "mg_batch_create: scene " + std::to_string(q) + " is too small");
    }
    const size_t n = (size_t)nx * ny * nz;
    const int ntiles = ((nx + kBTX - 1) / kBTX) * ((ny + kBTY - 1) / kBTY) * nz;
    off[q] = total;
    total += align256(n * sizeof(int));                  // flags
    total += 2 * align256(3 * n * sizeof(float));        // vel[2]
    total += 2 * align256(n * sizeof(float));            // dens[2]
    total += align256(4 * n * sizeof(float));            // fwd
    total += 6 * align256(n * sizeof(float));            // mask, pres, rhs, res, search, tmp
    total += align256(n * sizeof(code_t));               // code
    total += align256(2 * (size_t)ntiles * sizeof(double));  // part
  }
  b->arenaBytes = total;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&b->arena, total) != cudaSuccess) {
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    cudaGetLastError();
    return set_error(MG_ERR_NOMEM, "mg_batch_create: out of device memory");
  }
  cudaMemsetAsync(b->arena, 0, total, b->stream);
  CKB(cudaMalloc(&b->dSc, sizeof(CgScalars) * count));
  CKB(cudaMemset(b->dSc, 0, sizeof(CgScalars) * count));
  CKB(cudaMalloc(&b->dDone, sizeof(int)));
  b->hSc.assign(count, CgScalars{});
  b->scenes.resize(count);
  for (int q = 0; q < count; q++) {
    const int nx = sizes[3 * q], ny = sizes[3 * q + 1], nz = sizes[3 * q + 2];
    BScene& s = b->scenes[q];
    s.d.nx = nx;
    s.d.ny = ny;
    s.d.nz = nz;
    s.d.is3d = nz > 1;
    s.d.n = (long long)nx * ny * nz;
    s.d.sy = nx;
    s.d.sz = s.d.is3d ? (long long)nx * ny : 0;
    const size_t n = (size_t)s.d.n;
    const int ntiles = ((nx + kBTX - 1) / kBTX) * ((ny + kBTY - 1) / kBTY) * nz;
    unsigned char* p = b->arena + off[q];
    auto take = [&](size_t bytes) {
      unsigned char* r = p;
      p += align256(bytes);
      return r;
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
    s.part = (double*)take(2 * (size_t)ntiles * sizeof(double));
    s.sc = b->dSc + q;
    s.dt = dt;
    s.seed = seeds[q];
    s.ntiles = ntiles;
    // addBuoyancy(gravity, scale=True, coefficient=1): f = -g*dt/dx, 0.5*f
    const int m = std::max(nx, std::max(ny, nz));
    const float gridScale = (float)(1.0 / (double)m);
    s.bx = 0.5f * (((-gravity[3 * q]) * dt) / gridScale * 1.f);
    s.by = 0.5f * (((-gravity[3 * q + 1]) * dt) / gridScale * 1.f);
    s.bz = 0.5f * (((-gravity[3 * q + 2]) * dt) / gridScale * 1.f);
    // scene setup: initDomain(boundaryWidth=0) walls, fillGrid,
    // setOpenBound(0, 'Y', Outflow|Empty), the cylinder source
    const int wz = s.d.is3d ? kObstacle : 0;  // initDomain sets no z sides in 2D
    const int types[6] = {kObstacle, kObstacle, kObstacle, kObstacle, wz, wz};
    launch_init_domain(s.d, s.flags, 0, types, b->stream);
    launch_fill_grid(s.d, s.flags, kFluid, b->stream);
    const int lo[3] = {0, 0, 0}, up[3] = {0, 1, 0};
    launch_set_open_bound(s.d, s.flags, 0, lo, up, kOutflow | kEmpty, b->stream);
    // Cylinder(center = gs*(0.5,0.1,0.5), radius = 0.14*nx, z = gs*(0,0.02,0))
    const float gs[3] = {(float)nx, (float)ny, (float)nz};
    const float center[3] = {gs[0] * 0.5f, gs[1] * 0.1f, gs[2] * 0.5f};
    const float zdir[3] = {gs[0] * 0.f, gs[1] * 0.02f, gs[2] * 0.f};
    float zn[3], mZ;
    cylinder_axis(zdir, zn, &mZ);
    const float one[3] = {1.f, 0.f, 0.f};
    launch_shape_apply(s.d, 1, s.mask, nullptr, nullptr, one, 0, nullptr, center, zn, (float)(nx * 0.14), mZ, b->stream);
    b->tileStart.push_back((int)b->tiles.size());
    int local = 0;
    for (int z = 0; z < nz; z++)
      for (int y = 0; y < ny; y += kBTY)
        for (int x = 0; x < nx; x += kBTX) b->tiles.push_back(BTile{q, x, y, z, local++, ntiles});
    for (int kk = 0; kk < 4; kk++) {
      const int rows = kBTY << kk;
      const int cnt = ((nx + kBTX - 1) / kBTX) * ((ny + rows - 1) / rows) * nz;
      b->startR[kk].push_back((int)b->tilesR[kk].size());
      int l = 0;
      for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y += rows)
          for (int x = 0; x < nx; x += kBTX) b->tilesR[kk].push_back(BTile{q, x, y, z, l++, cnt});
    }
  }
  b->tileStart.push_back((int)b->tiles.size());
  for (int kk = 0; kk < 4; kk++) b->startR[kk].push_back((int)b->tilesR[kk].size());
  CKB(cudaEventCreate(&b->ev[0]));
  CKB(cudaEventCreate(&b->ev[1]));
  CKB(cudaMalloc(&b->dScenes, sizeof(BScene) * count));
  CKB(cudaMemcpyAsync(b->dScenes, b->scenes.data(), sizeof(BScene) * count, cudaMemcpyHostToDevice, b->stream));
  CKB(cudaMalloc(&b->dTiles, sizeof(BTile) * b->tiles.size()));
  CKB(cudaMalloc(&b->dActive, sizeof(BTile) * b->tiles.size()));
  CKB(cudaMemcpyAsync(b->dTiles, b->tiles.data(), sizeof(BTile) * b->tiles.size(), cudaMemcpyHostToDevice, b->stream));
  CKB(cudaStreamSynchronize(b->stream));
  CKB(cudaGetLastError());
  *out = b;
  return MG_OK;
}

extern "C" int mg_batch_destroy(mg_batch b) {
  if (!b) return MG_OK;
  cudaStreamSynchronize(b->stream);
  cudaFree(b->arena);
  cudaFree(b->dScenes);
  cudaFree(b->dTiles);
  cudaFree(b->dActive);
  cudaFree(b->dSc);
  cudaFree(b->dDone);
  if (b->ev[0]) cudaEventDestroy(b->ev[0]);
  if (b->ev[1]) cudaEventDestroy(b->ev[1]);
  cudaStreamDestroy(b->stream);
  delete b;
  return MG_OK;
}

extern "C" int mg_batch_set_solver(mg_batch b, float cgAccuracy, float cgMaxIterFac) {
  if (!b || !(cgAccuracy > 0.f) || !(cgMaxIterFac > 0.f)) return set_error(MG_ERR_ARG, "mg_batch_set_solver: invalid argument");
  b->cgAccuracy = cgAccuracy;
  b->cgMaxIterFac = cgMaxIterFac;
  return MG_OK;
}

extern "C" int mg_batch_step(mg_batch b, mg_batch_stats* stats) {
  if (!b) return set_error(MG_ERR_ARG, "mg_batch_step: null batch");
  const int cur = b->cur, nxt = 1 - cur;
  const int nt = (int)b->tiles.size();
  cudaStream_t st = b->stream;
  launch_b_inflow(b->dTiles, nt, b->dScenes, cur, b->step, st);
  launch_b_advect_velocity(b->dTiles, nt, b->dScenes, cur, st);
  launch_b_forces(b->dTiles, nt, b->dScenes, nxt, st);
  // GridCg setup of every scene: PcNone with the reference's 2D iteration
  // limit, (int)(cgMaxIterFac * max size) * 4 (pressure.cpp:407-409)
  int maxIterAll = 0;
  for (int q = 0; q < b->count; q++) {
    const Dims& d = b->scenes[q].d;
    CgScalars c{};
    c.accuracy = b->cgAccuracy;
    c.maxIter = (int)(b->cgMaxIterFac * (float)std::max(d.nx, std::max(d.ny, d.nz))) * 4;
    c.resNorm = 1e20f;
    b->hSc[q] = c;
    maxIterAll = std::max(maxIterAll, c.maxIter);
  }
  CKB(cudaMemcpyAsync(b->dSc, b->hSc.data(), sizeof(CgScalars) * b->count, cudaMemcpyHostToDevice, st));
  CKB(cudaMemsetAsync(b->dDone, 0, sizeof(int), st));
  launch_b_pressure_setup(b->dTiles, nt, b->dScenes, nxt, st);
  // CG sweeps over the tiles of the scenes still iterating.  Autotuner: the
  // first solve runs its first 4 x lag sweeps with tiles 8, 16, 32 and 64
  // rows tall (lag sweeps each, timed with events) and keeps the fastest;
  // results do not depend on the choice.
  int kk = b->rowsK >= 0 ? b->rowsK : 0;
  int active = 0, doneSeen = -1, sweeps = 0;
  std::vector<BTile> list;
  auto rebuild = [&](bool all) -> int {
    list.clear();
    for (int q = 0; q < b->count; q++)
      if (all || !b->hSc[q].done)
        list.insert(list.end(), b->tilesR[kk].begin() + b->startR[kk][q], b->tilesR[kk].begin() + b->startR[kk][q + 1]);
    active = (int)list.size();
    if (active) CKB(cudaMemcpyAsync(b->dActive, list.data(), sizeof(BTile) * active, cudaMemcpyHostToDevice, st));
    return MG_OK;
  };
  if (rebuild(true)) return MG_ERR_CUDA;
  const bool tuning = b->rowsK < 0;
  if (tuning) CKB(cudaEventRecord(b->ev[0], st));
  while (active > 0 && sweeps < maxIterAll) {
    launch_b_pcg_iteration(b->dActive, active, b->dScenes, 1 << kk, b->dDone, st);
    sweeps++;
    if (sweeps % b->lag == 0 || sweeps == maxIterAll) {
      bool relist = false;
      if (tuning && b->rowsK < 0 && sweeps <= 4 * b->lag) {
        CKB(cudaEventRecord(b->ev[1], st));
        CKB(cudaEventSynchronize(b->ev[1]));
        float ms = 0.f;
        CKB(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
        b->tuneMs[kk] = ms;
        if (kk < 3) {
          kk++;
          relist = true;
        } else {
          int best = 0;
          for (int q = 1; q < 4; q++)
            if (b->tuneMs[q] < b->tuneMs[best]) best = q;
          b->rowsK = best;
          relist = kk != best;
          kk = best;
        }
      }
      int nd = 0;
      CKB(cudaMemcpyAsync(&nd, b->dDone, sizeof(int), cudaMemcpyDeviceToHost, st));
      CKB(cudaStreamSynchronize(st));
      if (nd >= b->count) break;
      if (nd != doneSeen || relist) {
        doneSeen = nd;
        CKB(cudaMemcpyAsync(b->hSc.data(), b->dSc, sizeof(CgScalars) * b->count, cudaMemcpyDeviceToHost, st));
        CKB(cudaStreamSynchronize(st));
        if (rebuild(false)) return MG_ERR_CUDA;
      }
      if (tuning && b->rowsK < 0) CKB(cudaEventRecord(b->ev[0], st));
    }
  }
  launch_b_correct(b->dTiles, nt, b->dScenes, nxt, st);
  CKB(cudaMemcpyAsync(b->hSc.data(), b->dSc, sizeof(CgScalars) * b->count, cudaMemcpyDeviceToHost, st));
  CKB(cudaStreamSynchronize(st));
  CKB(cudaGetLastError());
  b->cur = nxt;
  b->step++;
  if (stats) {
    stats->sweeps = sweeps;
    int mx = 0;
    long long sum = 0;
    int diverged = 0;
    for (auto& c : b->hSc) {
      mx = std::max(mx, c.iterations);
      sum += c.iterations;
      diverged += c.status == 2;
    }
    stats->maxIterations = mx;
    stats->totalIterations = sum;
    stats->diverged = diverged;
  }
  for (auto& c : b->hSc)
    if (c.status == 2)
      return set_error(MG_ERR_SOLVER, "GridCg::iterate: The CG solver diverged, residual norm > 1e30, stopping.");
  return MG_OK;
}

extern "C" int mg_batch_scene_iterations(mg_batch b, int scene, int* iterations, float* resNorm) {
  if (!b || scene < 0 || scene >= b->count) return set_error(MG_ERR_ARG, "mg_batch_scene_iterations: invalid scene");
  if (iterations) *iterations = b->hSc[scene].iterations;
  if (resNorm) *resNorm = b->hSc[scene].resNorm;
  return MG_OK;
}

extern "C" int mg_batch_download(mg_batch b, int scene, int what, void* host, size_t bytes) {
  if (!b || scene < 0 || scene >= b->count || !host) return set_error(MG_ERR_ARG, "mg_batch_download: invalid argument");
  const BScene& s = b->scenes[scene];
  const size_t n = (size_t)s.d.n;
  const size_t want = what == MG_BATCH_VELOCITY ? 3 * n * sizeof(float) : n * sizeof(float);
  if (bytes != want) return set_error(MG_ERR_ARG, "mg_batch_download: byte count does not match the scene");
  cudaStream_t st = b->stream;
  switch (what) {
    case MG_BATCH_DENSITY: CKB(cudaMemcpyAsync(host, s.dens[b->cur], want, cudaMemcpyDeviceToHost, st)); break;
    case MG_BATCH_PRESSURE: CKB(cudaMemcpyAsync(host, s.pres, want, cudaMemcpyDeviceToHost, st)); break;
    case MG_BATCH_FLAGS: CKB(cudaMemcpyAsync(host, s.flags, want, cudaMemcpyDeviceToHost, st)); break;
    case MG_BATCH_SOURCE: CKB(cudaMemcpyAsync(host, s.mask, want, cudaMemcpyDeviceToHost, st)); break;
    case MG_BATCH_VELOCITY: {
      // SoA planes -> the reference's AoS Vec3 on the host
      std::vector<float> h(3 * n);
      CKB(cudaMemcpyAsync(h.data(), s.vel[b->cur], want, cudaMemcpyDeviceToHost, st));
      CKB(cudaStreamSynchronize(st));
      float* o = (float*)host;
      for (size_t i = 0; i < n; i++) {
        o[3 * i] = h[i];
        o[3 * i + 1] = h[n + i];
        o[3 * i + 2] = h[2 * n + i];
      }
      return MG_OK;
    }
    default: return set_error(MG_ERR_ARG, "mg_batch_download: unknown field");
  }
  CKB(cudaStreamSynchronize(st));
  return MG_OK;
}

extern "C" int mg_batch_noise(unsigned long long seed, int step, long long cells, float* out) {
  if (!out || cells < 0) return set_error(MG_ERR_ARG, "mg_batch_noise: invalid argument");
  for (long long i = 0; i < cells; i++) out[i] = batch_noise(seed, step, i);
  return MG_OK;
}

extern "C" int mg_batch_tuning(mg_batch b, int* sweepRows, float* ms) {
  if (!b) return set_error(MG_ERR_ARG, "mg_batch_tuning: null batch");
  if (sweepRows) *sweepRows = b->rowsK < 0 ? 0 : kBTY << b->rowsK;
  if (ms)
    for (int q = 0; q < 4; q++) ms[q] = b->tuneMs[q];
  return MG_OK;
}

extern "C" int mg_batch_info(mg_batch b, int* count, long long* cells, long long* tiles, size_t* bytes) {
  if (!b) return set_error(MG_ERR_ARG, "mg_batch_info: null batch");
  long long c = 0;
  for (auto& s : b->scenes) c += s.d.n;
  if (count) *count = b->count;
  if (cells) *cells = c;
  if (tiles) *tiles = (long long)b->tiles.size();
  if (bytes) *bytes = b->arenaBytes;
  return MG_OK;
}

extern "C" int mg_batch_sync(mg_batch b) {
  if (!b) return set_error(MG_ERR_ARG, "mg_batch_sync: null batch");
  CKB(cudaStreamSynchronize(b->stream));
  return MG_OK;
}
