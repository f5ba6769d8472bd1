// libmantagpu runtime: the C ABI declared in include/mantagpu.h.
//
// Owns the CUDA device state of every FluidSolver-equivalent (stream, grid
// storage pool, CG/MIC state) and translates each mantaflow plugin call into
// kernel launches on the solver's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "../../include/mantagpu.h"
#include "mg_common.cuh"
#include "mg_kernels.h"
#include "mg_multigrid.h"
#include "mg_batch.h"

using namespace mgpu;

std::atomic<unsigned long long> mgpu::g_launches{0};
thread_local unsigned long long mgpu::t_launches = 0;

// upper bound on any single device-side wait in the MIC wavefronts (ns);
// a wait that runs out flags an error instead of spinning on
static const long long kWaitNs = 200000000LL;

// ------------------------------------------------------------------ errors
static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

// for the other translation units of the library (batch.cu, serve.cu)
int mgpu::set_error(int code, const std::string& msg) { return fail(code, msg); }

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return fail(MG_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

// MANTA_GB300_SYNC_CHECK=1 synchronises after every launch site so that a
// failing kernel is reported where it was launched (debugging aid).
static bool sync_check() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("MANTA_GB300_SYNC_CHECK");
    v = (e && e[0] == '1') ? 1 : 0;
  }
  return v == 1;
}

#define CKL()                                                                                         \
  do {                                                                                                \
    cudaError_t e_ = cudaGetLastError();                                                              \
    if (e_ == cudaSuccess && sync_check()) e_ = cudaDeviceSynchronize();                              \
    if (e_ != cudaSuccess)                                                                            \
      return fail(MG_ERR_CUDA, std::string("kernel launch (") + __func__ + ":" + std::to_string(__LINE__) + \
                                   "): " + cudaGetErrorString(e_));                                   \
  } while (0)

// ----------------------------------------------------------------- context
struct Ctx {
  bool init = false;
  int device = -1;
  int sms = 0;
  int micCtasPerSm = 1;
  int waveCtasPerSm4 = 1, waveCtasPerSm8 = 1;
  int flowCtasPerSm = 1;
  std::set<mg_solver> solvers;
  std::mutex mu;
};
static Ctx g_ctx;

struct Prof {
  std::string name;
  cudaEvent_t a, b;
};

struct mg_solver_s {
  Dims d;
  int dim;
  float dt = 1.f;
  cudaStream_t stream = nullptr;
  // asynchronous grid transfers: copy streams, created on first use; a
  // transfer is split into one chunk per stream so several copy engines
  // move it at once
  static constexpr int kMaxCopyStreams = 8;
  int ncopy = 0;
  cudaStream_t copyStream[kMaxCopyStreams] = {};  // device -> host
  cudaStream_t upStream[kMaxCopyStreams] = {};    // host -> device
  std::multimap<size_t, void*> pool;  // free device buffers by size
  std::set<mg_grid> grids;
  size_t poolBytes = 0;  // free buffers in the pool
  size_t tmpBytes = 0;   // pool buffers handed out to temporaries
  // CG state (allocated on first solve)
  code_t* code = nullptr;
  float* A0f = nullptr;
  float* residual = nullptr;
  float* search = nullptr;
  float* tmp = nullptr;
  float* P = nullptr;
  float* Aoff = nullptr;  // fractions: the stored off-diagonals Ai | Aj | Ak (3n floats)
  double* part = nullptr;
  float* partf = nullptr;
  CgScalars* sc = nullptr;
  CgScalars* scHost = nullptr;
  int* intScratch = nullptr;
  int nblocks = 0;
  size_t partCount = 0;
  MicPlan mic{};
  MicColPlan micCol{};
  bool useMicCol = false;
  MicWavePlan micWave{};
  bool useMicWave = false;
  unsigned long long* micFace = nullptr;  // tile-dataflow sweeps: face words
  bool useMicFlow = false;
  unsigned int epoch = 0;
  long long waitNs = kWaitNs;  // limit of each device-side MIC wait
  bool stallNext = false;      // the next MIC solve's waits run out (test of the timeout path)
  bool stall = false;          // ... during this solve
  size_t memLimit = 0;         // cap on the device memory the solver holds (0: none)
  mgpu::MgHierarchy* mg = nullptr;  // static multigrid cache (gMapMG)
  // one MG-PCG iteration captured as a CUDA graph, replayed while the
  // buffers and hierarchy it was captured with are unchanged
  cudaGraphExec_t iterGraph = nullptr;
  PcgBuffers iterKey{};
  unsigned long long iterSig = 0;
  const void* iterMg = nullptr;
  unsigned long long iterNodes = 0;
  // profiling
  bool prof = false;
  std::vector<Prof> profEvents;
  Prof profOpen;
  std::vector<cudaEvent_t> evFree;
  std::map<std::string, std::pair<double, long long>> profAcc;
  cudaEvent_t marks[8] = {};
};

struct mg_grid_s {
  mg_solver s;
  int kind;
  void* data;   // device: n floats / ints, or 3n floats (SoA) for Vec3/MAC
  // asynchronous transfers: a device staging copy of the grid (AoS for
  // Vec3/MAC), ready / free events, allocated on first use
  void* stage = nullptr;
  cudaEvent_t stageReady = nullptr;
  cudaEvent_t stageFree[mg_solver_s::kMaxCopyStreams] = {};  // one per stream the last transfer used
  int nFree = 0;
  int comps() const { return (kind == MG_VEC3 || kind == MG_MAC) ? 3 : 1; }
  size_t bytes() const { return sizeof(float) * (size_t)comps() * (size_t)s->d.n; }
  float* f() const { return (float*)data; }
  int* i() const { return (int*)data; }
  Mac mac() const {
    float* b = (float*)data;
    return Mac{b, b + s->d.n, b + 2 * s->d.n};
  }
  CMac cmac() const {
    const float* b = (const float*)data;
    return CMac{b, b + s->d.n, b + 2 * s->d.n};
  }
};

// ------------------------------------------------------------- profiling
struct ProfScope {
  mg_solver s;
  Prof p;
  bool on;
  ProfScope(mg_solver s_, const char* name) : s(s_), on(s_->prof && name) {
    if (!on) return;
    p.name = name;
    p.a = take();
    p.b = take();
    cudaEventRecord(p.a, s->stream);
  }
  ~ProfScope() {
    if (!on) return;
    cudaEventRecord(p.b, s->stream);
    s->profEvents.push_back(p);
  }
  cudaEvent_t take() {
    if (!s->evFree.empty()) {
      cudaEvent_t e = s->evFree.back();
      s->evFree.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
};

static void prof_collect(mg_solver s) {
  if (s->profEvents.empty()) return;
  cudaStreamSynchronize(s->stream);
  for (auto& p : s->profEvents) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    auto& acc = s->profAcc[p.name];
    acc.first += ms;
    acc.second += 1;
    s->evFree.push_back(p.a);
    s->evFree.push_back(p.b);
  }
  s->profEvents.clear();
}

// ------------------------------------------------------------------ pool
// device bytes held by the solver: grids (and their staging copies), the
// pool, CG state and the multigrid hierarchy
static size_t held_bytes(mg_solver s) {
  size_t b = s->poolBytes + s->tmpBytes;
  for (auto g : s->grids) b += g->bytes() * (g->stage ? 2 : 1);
  const size_t n = (size_t)s->d.n;
  if (s->code) b += n * (sizeof(code_t) + 4 * sizeof(float));
  if (s->A0f) b += n * sizeof(float);
  if (s->Aoff) b += 3 * n * sizeof(float);
  if (s->mg) b += mg_hierarchy_bytes(s->mg);
  return b;
}
// a new allocation of `bytes` would exceed the solver's memory cap
static bool over_limit(mg_solver s, size_t bytes) { return s->memLimit && held_bytes(s) + bytes > s->memLimit; }

static void* pool_get(mg_solver s, size_t bytes) {
  auto it = s->pool.find(bytes);
  if (it != s->pool.end()) {
    void* p = it->second;
    s->pool.erase(it);
    s->poolBytes -= bytes;
    s->tmpBytes += bytes;
    return p;
  }
  if (over_limit(s, bytes)) return nullptr;
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  s->tmpBytes += bytes;
  return p;
}
static void pool_put(mg_solver s, void* p, size_t bytes) {
  if (!p) return;
  s->pool.emplace(bytes, p);
  s->poolBytes += bytes;
  s->tmpBytes -= bytes;
}

// RAII temp grid storage (FluidSolver::GridStorage, fluidsolver.cpp:33-50)
struct Tmp {
  mg_solver s;
  size_t bytes;
  void* p;
  Tmp(mg_solver s_, size_t b) : s(s_), bytes(b), p(pool_get(s_, b)) {}
  ~Tmp() {
    if (p) pool_put(s, p, bytes);
  }
  float* f() const { return (float*)p; }
  int* i() const { return (int*)p; }
  Mac mac() const {
    float* b = (float*)p;
    return Mac{b, b + s->d.n, b + 2 * s->d.n};
  }
  CMac cmac() const {
    float* b = (float*)p;
    return CMac{b, b + s->d.n, b + 2 * s->d.n};
  }
  void release() { p = nullptr; }
};

static bool valid_solver(mg_solver s) { return s && g_ctx.solvers.count(s); }
// a grid handle is valid while one of the live solvers holds it; the test
// never dereferences the handle, so a stale one (after mg_grid_destroy,
// mg_solver_destroy or mg_shutdown) is refused, not read
static bool valid_grid(mg_grid g) {
  if (!g) return false;
  for (mg_solver s : g_ctx.solvers)
    if (s->grids.count(g)) return true;
  return false;
}

bool mgpu::library_ready() { return g_ctx.init; }

#define NEED_INIT() \
  if (!g_ctx.init) return fail(MG_ERR_STATE, "mg_init has not been called")
#define NEED_GRID(g, what) \
  if (!valid_grid(g)) return fail(MG_ERR_ARG, std::string(what) + ": invalid grid handle")

static bool is_real(mg_grid g) { return g->kind == MG_REAL || g->kind == MG_LEVELSET; }
static bool is_vec(mg_grid g) { return g->kind == MG_MAC || g->kind == MG_VEC3; }

// ================================================================ library
extern "C" int mg_init(int device) {
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  if (g_ctx.init) {
    if (device != g_ctx.device) return fail(MG_ERR_STATE, "mg_init: already initialised on another device");
    return MG_OK;
  }
  int n = 0;
  CK(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return fail(MG_ERR_ARG, "mg_init: no such CUDA device");
  CK(cudaSetDevice(device));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, device));
  g_ctx.sms = prop.multiProcessorCount;
  g_ctx.micCtasPerSm = mic_ctas_per_sm();
  if (mic_col_prepare() || mic_wave_prepare(&g_ctx.waveCtasPerSm4, &g_ctx.waveCtasPerSm8) ||
      mic_flow_prepare(&g_ctx.flowCtasPerSm) || pcg_prepare(g_ctx.sms))
    return fail(MG_ERR_CUDA, "mg_init: cannot configure the MIC kernels");
  g_ctx.device = device;
  g_ctx.init = true;
  return MG_OK;
}

extern "C" int mg_solver_destroy(mg_solver s);
static void noalloc_forget();

extern "C" int mg_shutdown(void) {
  if (!g_ctx.init) return MG_OK;
  std::vector<mg_solver> all(g_ctx.solvers.begin(), g_ctx.solvers.end());
  for (auto s : all) mg_solver_destroy(s);
  noalloc_forget();
  noise_release();
  g_ctx.init = false;
  g_ctx.device = -1;
  return MG_OK;
}

extern "C" const char* mg_last_error(void) { return g_err.c_str(); }
extern "C" int mg_version(void) { return 100; }
extern "C" int mg_device_count(int* out) {
  if (!out) return fail(MG_ERR_ARG, "mg_device_count: null out");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  *out = n;
  return MG_OK;
}

// ================================================================= solver
extern "C" int mg_solver_create(int nx, int ny, int nz, int dim, mg_solver* out) {
  NEED_INIT();
  if (!out) return fail(MG_ERR_ARG, "mg_solver_create: null out");
  if (dim != 2 && dim != 3) return fail(MG_ERR_ARG, "mg_solver_create: dim must be 2 or 3");
  if (dim == 2 && nz != 1) return fail(MG_ERR_ARG, "mg_solver_create: 2D solvers need nz == 1");
  if (nx < 3 || ny < 3 || (dim == 3 && nz < 3)) return fail(MG_ERR_ARG, "mg_solver_create: grid must be >= 3 cells per axis");
  if ((long long)nx * ny * nz >= (1LL << 31))
    return fail(MG_ERR_ARG, "mg_solver_create: grids are limited to 2^31 - 1 cells (32-bit cell offsets in the kernels)");
  auto s = new mg_solver_s();
  s->dim = dim;
  s->d.nx = nx;
  s->d.ny = ny;
  s->d.nz = nz;
  s->d.is3d = dim == 3;
  s->d.n = (long long)nx * ny * nz;
  s->d.sy = nx;
  s->d.sz = dim == 3 ? (long long)nx * ny : 0;
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete s;
    return fail(MG_ERR_CUDA, "mg_solver_create: cudaStreamCreate failed");
  }
  for (auto& e : s->marks) cudaEventCreate(&e);
  g_ctx.solvers.insert(s);
  *out = s;
  return MG_OK;
}

static void free_cg_state(mg_solver s) {
  cudaFree(s->code); cudaFree(s->A0f); cudaFree(s->residual); cudaFree(s->search); cudaFree(s->tmp); cudaFree(s->P);
  cudaFree(s->part); cudaFree(s->partf); cudaFree(s->sc); cudaFreeHost(s->scHost); cudaFree(s->intScratch);
  cudaFree(s->mic.order); cudaFree(s->mic.tileDone); cudaFree(s->mic.counter); cudaFree(s->mic.error);
  s->code = nullptr; s->A0f = nullptr; s->residual = s->search = s->tmp = s->P = nullptr;
  s->part = nullptr; s->partf = nullptr; s->sc = nullptr; s->scHost = nullptr; s->intScratch = nullptr;
  s->mic = MicPlan{};
  // micCol.error aliases mic.error (freed above)
  cudaFree(s->micCol.order); cudaFree(s->micCol.prog); cudaFree(s->micCol.counter);
  // micWave.error aliases mic.error as well
  cudaFree(s->micWave.order); cudaFree(s->micWave.counter); cudaFree(s->micWave.exchange);
  cudaFree(s->micFace);
  s->micFace = nullptr;
  cudaFree(s->Aoff);
  s->Aoff = nullptr;
  cudaGetLastError();  // a failed free must not surface as a later launch error
  s->micCol = MicColPlan{};
  s->micWave = MicWavePlan{};
}

static void free_stage(mg_grid g) {
  if (g->stage) cudaFree(g->stage);
  if (g->stageReady) cudaEventDestroy(g->stageReady);
  for (auto& e : g->stageFree)
    if (e) cudaEventDestroy(e);
  g->stage = nullptr;
  g->stageReady = nullptr;
  for (auto& e : g->stageFree) e = nullptr;
  g->nFree = 0;
}
static void sync_copies(mg_solver s) {
  for (int k = 0; k < s->ncopy; k++) {
    cudaStreamSynchronize(s->copyStream[k]);
    cudaStreamSynchronize(s->upStream[k]);
  }
}

extern "C" int mg_solver_destroy(mg_solver s) {
  if (!valid_solver(s)) return fail(MG_ERR_ARG, "mg_solver_destroy: invalid solver");
  sync_copies(s);
  cudaStreamSynchronize(s->stream);
  particles_release(s);
  for (auto g : s->grids) {
    free_stage(g);
    cudaFree(g->data);
    delete g;
  }
  s->grids.clear();
  for (auto& kv : s->pool) cudaFree(kv.second);
  s->pool.clear();
  free_cg_state(s);
  if (s->mg) mg_hierarchy_destroy(s->mg);
  if (s->iterGraph) cudaGraphExecDestroy(s->iterGraph);
  prof_collect(s);
  for (auto e : s->evFree) cudaEventDestroy(e);
  for (auto e : s->marks) cudaEventDestroy(e);
  for (int k = 0; k < s->ncopy; k++) {
    cudaStreamDestroy(s->copyStream[k]);
    cudaStreamDestroy(s->upStream[k]);
  }
  cudaStreamDestroy(s->stream);
  g_ctx.solvers.erase(s);
  delete s;
  return MG_OK;
}

extern "C" int mg_solver_set_dt(mg_solver s, float dt) {
  if (!valid_solver(s)) return fail(MG_ERR_ARG, "mg_solver_set_dt: invalid solver");
  s->dt = dt;
  return MG_OK;
}
extern "C" int mg_solver_get_dt(mg_solver s, float* dt) {
  if (!valid_solver(s) || !dt) return fail(MG_ERR_ARG, "mg_solver_get_dt: invalid argument");
  *dt = s->dt;
  return MG_OK;
}
extern "C" int mg_solver_sync(mg_solver s) {
  if (!valid_solver(s)) return fail(MG_ERR_ARG, "mg_solver_sync: invalid solver");
  CK(cudaStreamSynchronize(s->stream));
  return MG_OK;
}
extern "C" int mg_solver_memory(mg_solver s, size_t* bytes) {
  if (!valid_solver(s) || !bytes) return fail(MG_ERR_ARG, "mg_solver_memory: invalid argument");
  *bytes = held_bytes(s);
  return MG_OK;
}

extern "C" int mg_solver_set_memory_limit(mg_solver s, size_t bytes) {
  if (!valid_solver(s)) return fail(MG_ERR_ARG, "mg_solver_set_memory_limit: invalid solver");
  s->memLimit = bytes;
  return MG_OK;
}

extern "C" int mg_solver_set_wait_limit(mg_solver s, long long limitNs, int stallNextSolve) {
  if (!valid_solver(s) || limitNs < 0) return fail(MG_ERR_ARG, "mg_solver_set_wait_limit: invalid argument");
  s->waitNs = limitNs ? limitNs : kWaitNs;
  s->stallNext = stallNextSolve != 0;
  return MG_OK;
}

// ================================================================== grids
extern "C" int mg_grid_create(mg_solver s, int kind, mg_grid* out) {
  if (!valid_solver(s) || !out) return fail(MG_ERR_ARG, "mg_grid_create: invalid argument");
  if (kind < MG_REAL || kind > MG_LEVELSET) return fail(MG_ERR_ARG, "mg_grid_create: unknown grid kind");
  auto g = new mg_grid_s();
  g->s = s;
  g->kind = kind;
  const size_t bytes = g->bytes();
  if (over_limit(s, bytes)) {
    delete g;
    return fail(MG_ERR_NOMEM, "mg_grid_create: the solver's memory limit is reached");
  }
  if (cudaMalloc(&g->data, bytes) != cudaSuccess) {
    cudaGetLastError();
    delete g;
    return fail(MG_ERR_NOMEM, "mg_grid_create: out of device memory");
  }
  CK(cudaMemsetAsync(g->data, 0, bytes, s->stream));
  s->grids.insert(g);
  *out = g;
  return MG_OK;
}

extern "C" int mg_solver_size(mg_solver s, int* nx, int* ny, int* nz) {
  if (!valid_solver(s)) return fail(MG_ERR_ARG, "mg_solver_size: invalid solver");
  if (nx) *nx = s->d.nx;
  if (ny) *ny = s->d.ny;
  if (nz) *nz = s->d.nz;
  return MG_OK;
}

int mgpu::solver_info(mg_solver s, Dims* d, cudaStream_t* st) {
  if (!valid_solver(s)) return fail(MG_ERR_ARG, "invalid solver");
  *d = s->d;
  *st = s->stream;
  return MG_OK;
}

extern "C" int mg_grid_device(mg_grid g, void** data, void** stream) {
  NEED_GRID(g, "mg_grid_device");
  if (data) *data = g->data;
  if (stream) *stream = (void*)g->s->stream;
  return MG_OK;
}

extern "C" int mg_grid_get_info(mg_grid g, int* nx, int* ny, int* nz, int* kind) {
  NEED_GRID(g, "mg_grid_get_info");
  if (nx) *nx = g->s->d.nx;
  if (ny) *ny = g->s->d.ny;
  if (nz) *nz = g->s->d.nz;
  if (kind) *kind = g->kind;
  return MG_OK;
}

extern "C" int mg_grid_destroy(mg_grid g) {
  NEED_GRID(g, "mg_grid_destroy");
  sync_copies(g->s);
  cudaStreamSynchronize(g->s->stream);
  free_stage(g);
  cudaFree(g->data);
  g->s->grids.erase(g);
  delete g;
  return MG_OK;
}

extern "C" int mg_grid_upload(mg_grid g, const void* host, size_t bytes) {
  NEED_GRID(g, "mg_grid_upload");
  if (!host || bytes != g->bytes()) return fail(MG_ERR_ARG, "mg_grid_upload: host buffer size does not match the grid");
  mg_solver s = g->s;
  ProfScope ps(s, "h2d");
  if (!is_vec(g)) {
    CK(cudaMemcpyAsync(g->data, host, bytes, cudaMemcpyHostToDevice, s->stream));
  } else {
    Tmp st(s, bytes);
    if (!st.p) return fail(MG_ERR_NOMEM, "mg_grid_upload: out of device memory");
    CK(cudaMemcpyAsync(st.p, host, bytes, cudaMemcpyHostToDevice, s->stream));
    launch_aos_to_soa(s->d.n, st.f(), g->mac(), s->stream);
    CKL();
  }
  CK(cudaStreamSynchronize(s->stream));
  return MG_OK;
}

extern "C" int mg_grid_download(mg_grid g, void* host, size_t bytes) {
  NEED_GRID(g, "mg_grid_download");
  if (!host || bytes != g->bytes()) return fail(MG_ERR_ARG, "mg_grid_download: host buffer size does not match the grid");
  mg_solver s = g->s;
  ProfScope ps(s, "d2h");
  if (!is_vec(g)) {
    CK(cudaMemcpyAsync(host, g->data, bytes, cudaMemcpyDeviceToHost, s->stream));
  } else {
    Tmp st(s, bytes);
    if (!st.p) return fail(MG_ERR_NOMEM, "mg_grid_download: out of device memory");
    launch_soa_to_aos(s->d.n, g->cmac(), st.f(), s->stream);
    CKL();
    CK(cudaMemcpyAsync(host, st.p, bytes, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return MG_OK;
  }
  CK(cudaStreamSynchronize(s->stream));
  return MG_OK;
}

// ---- asynchronous transfers.  An upload copies host -> staging on the
// solver's copy stream, then staging -> grid on the compute stream; a
// download snapshots grid -> staging on the compute stream, then staging ->
// host on the copy stream.  Events order the two streams and keep a grid's
// staging buffer from being refilled before its previous transfer is done,
// so a caller can queue step t+1 while step t's results are still leaving.
static int ensure_stage(mg_grid g) {
  mg_solver s = g->s;
  if (!s->ncopy) {
    int n = 4;
    if (const char* e = std::getenv("MANTAGPU_COPY_STREAMS")) n = std::atoi(e);
    n = std::max(1, std::min(n, (int)mg_solver_s::kMaxCopyStreams));
    // downloads and uploads on streams of their own: the next step's upload
    // must not queue behind this step's downloads
    for (int k = 0; k < n; k++) {
      CK(cudaStreamCreateWithFlags(&s->copyStream[k], cudaStreamNonBlocking));
      CK(cudaStreamCreateWithFlags(&s->upStream[k], cudaStreamNonBlocking));
    }
    s->ncopy = n;
  }
  if (!g->stage) {
    if (cudaMalloc(&g->stage, g->bytes()) != cudaSuccess) {
      cudaGetLastError();
      g->stage = nullptr;
      return fail(MG_ERR_NOMEM, "asynchronous transfer: out of device memory");
    }
    CK(cudaEventCreateWithFlags(&g->stageReady, cudaEventDisableTiming));
    for (int k = 0; k < mg_solver_s::kMaxCopyStreams; k++)
      CK(cudaEventCreateWithFlags(&g->stageFree[k], cudaEventDisableTiming));
  }
  return MG_OK;
}
// wait on stream st until the grid's staging copy is free
static int wait_stage_free(mg_grid g, cudaStream_t st) {
  for (int k = 0; k < g->nFree; k++) CK(cudaStreamWaitEvent(st, g->stageFree[k], 0));
  return MG_OK;
}
// the copy split into one 256-byte-aligned chunk per copy stream, each after
// `ready`; records the grid's free events on the streams it used
static int chunked_copy(mg_grid g, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaEvent_t ready,
                        cudaStream_t* streams) {
  mg_solver s = g->s;
  const size_t per = ((bytes + s->ncopy - 1) / s->ncopy + 255) & ~(size_t)255;
  int used = 0;
  for (int k = 0; k < s->ncopy && (size_t)k * per < bytes; k++) {
    const size_t off = (size_t)k * per, len = std::min(per, bytes - off);
    if (ready) CK(cudaStreamWaitEvent(streams[k], ready, 0));
    CK(cudaMemcpyAsync((char*)dst + off, (const char*)src + off, len, kind, streams[k]));
    CK(cudaEventRecord(g->stageFree[k], streams[k]));
    used++;
  }
  g->nFree = used;
  return MG_OK;
}

extern "C" int mg_grid_upload_async(mg_grid g, const void* host, size_t bytes) {
  NEED_GRID(g, "mg_grid_upload_async");
  if (!host || bytes != g->bytes()) return fail(MG_ERR_ARG, "mg_grid_upload_async: host buffer size does not match the grid");
  int st = ensure_stage(g);
  if (st) return st;
  mg_solver s = g->s;
  ProfScope ps(s, "h2d");
  for (int k = 0; k < s->ncopy; k++)
    if ((st = wait_stage_free(g, s->upStream[k]))) return st;
  if ((st = chunked_copy(g, g->stage, host, bytes, cudaMemcpyHostToDevice, nullptr, s->upStream))) return st;
  // the compute stream waits for every chunk, then moves staging -> grid
  for (int k = 0; k < g->nFree; k++) CK(cudaStreamWaitEvent(s->stream, g->stageFree[k], 0));
  if (is_vec(g)) {
    launch_aos_to_soa(s->d.n, (const float*)g->stage, g->mac(), s->stream);
    CKL();
  } else {
    CK(cudaMemcpyAsync(g->data, g->stage, bytes, cudaMemcpyDeviceToDevice, s->stream));
  }
  CK(cudaEventRecord(g->stageFree[0], s->stream));
  g->nFree = 1;
  return MG_OK;
}

extern "C" int mg_grid_download_async(mg_grid g, void* host, size_t bytes) {
  NEED_GRID(g, "mg_grid_download_async");
  if (!host || bytes != g->bytes()) return fail(MG_ERR_ARG, "mg_grid_download_async: host buffer size does not match the grid");
  int st = ensure_stage(g);
  if (st) return st;
  mg_solver s = g->s;
  ProfScope ps(s, "d2h");
  if ((st = wait_stage_free(g, s->stream))) return st;
  if (is_vec(g)) {
    launch_soa_to_aos(s->d.n, g->cmac(), (float*)g->stage, s->stream);
    CKL();
  } else {
    CK(cudaMemcpyAsync(g->stage, g->data, bytes, cudaMemcpyDeviceToDevice, s->stream));
  }
  CK(cudaEventRecord(g->stageReady, s->stream));
  return chunked_copy(g, host, g->stage, bytes, cudaMemcpyDeviceToHost, g->stageReady, s->copyStream);
}

extern "C" int mg_solver_wait_copies(mg_solver s) {
  if (!valid_solver(s)) return fail(MG_ERR_ARG, "mg_solver_wait_copies: invalid solver");
  for (int k = 0; k < s->ncopy; k++) {
    CK(cudaStreamSynchronize(s->copyStream[k]));
    CK(cudaStreamSynchronize(s->upStream[k]));
  }
  CK(cudaStreamSynchronize(s->stream));
  return MG_OK;
}

extern "C" int mg_grid_swap(mg_grid a, mg_grid b) {
  NEED_GRID(a, "mg_grid_swap");
  NEED_GRID(b, "mg_grid_swap");
  if (a->s != b->s || a->bytes() != b->bytes()) return fail(MG_ERR_SOLVER, "Grid::swap(): Grid dimensions mismatch.");
  std::swap(a->data, b->data);
  return MG_OK;
}

extern "C" int mg_grid_copy(mg_grid dst, mg_grid src) {
  NEED_GRID(dst, "mg_grid_copy");
  NEED_GRID(src, "mg_grid_copy");
  if (dst->s != src->s || dst->bytes() != src->bytes()) return fail(MG_ERR_ARG, "mg_grid_copy: grids differ in size");
  CK(cudaMemcpyAsync(dst->data, src->data, dst->bytes(), cudaMemcpyDeviceToDevice, dst->s->stream));
  return MG_OK;
}

extern "C" int mg_grid_set_const(mg_grid g, float x, float y, float z) {
  NEED_GRID(g, "mg_grid_set_const");
  mg_solver s = g->s;
  if (g->kind == MG_INT || g->kind == MG_FLAGS) {
    const int v = (int)x;
    std::vector<int> h((size_t)s->d.n, v);
    CK(cudaMemcpyAsync(g->data, h.data(), g->bytes(), cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
  } else if (is_vec(g)) {
    Mac m = g->mac();
    launch_set_const(s->d.n, m.u, x, s->stream);
    launch_set_const(s->d.n, m.v, y, s->stream);
    launch_set_const(s->d.n, m.w, z, s->stream);
  } else {
    launch_set_const(s->d.n, g->f(), x, s->stream);
  }
  CKL();
  return MG_OK;
}

extern "C" int mg_grid_join(mg_grid a, mg_grid b, int keepMax) {
  NEED_GRID(a, "mg_grid_join");
  NEED_GRID(b, "mg_grid_join");
  if (!is_real(a) || !is_real(b) || a->s != b->s) return fail(MG_ERR_UNSUPPORTED, "mg_grid_join: Real grids of one solver only");
  ProfScope ps(a->s, "join");
  launch_join(a->s->d.n, a->f(), b->f(), keepMax, a->s->stream);
  CKL();
  return MG_OK;
}

extern "C" int mg_grid_get_max_abs(mg_grid g, float* out) {
  NEED_GRID(g, "mg_grid_get_max_abs");
  if (!is_real(g) || !out) return fail(MG_ERR_ARG, "mg_grid_get_max_abs: Real grid and out pointer required");
  mg_solver s = g->s;
  Tmp part(s, sizeof(float) * 2 * 1024);
  const int nb = launch_minmax_partial(s->d.n, g->f(), part.f(), s->stream);
  CKL();
  std::vector<float> h(2 * nb);
  CK(cudaMemcpyAsync(h.data(), part.p, sizeof(float) * 2 * nb, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  float mn = 3.402823466e+38f, mx = -3.402823466e+38f;
  for (int q = 0; q < nb; q++) {
    mn = std::min(mn, h[2 * q]);
    mx = std::max(mx, h[2 * q + 1]);
  }
  const float a = std::fabs(mn), b = std::fabs(mx);
  *out = a < b ? b : a;
  return MG_OK;
}

extern "C" int mg_host_alloc(size_t bytes, void** out) {
  NEED_INIT();
  if (!out) return fail(MG_ERR_ARG, "mg_host_alloc: null out");
  CK(cudaMallocHost(out, bytes));
  return MG_OK;
}
extern "C" int mg_host_free(void* p) {
  CK(cudaFreeHost(p));
  return MG_OK;
}

// ============================================================== advection
extern "C" int mg_advect_semi_lagrange(mg_grid flags, mg_grid vel, mg_grid grid, int order, float strength,
                                       int orderSpace, int openBounds, int boundaryWidth, int clampMode, int orderTrace) {
  NEED_GRID(flags, "advectSemiLagrange");
  NEED_GRID(vel, "advectSemiLagrange");
  NEED_GRID(grid, "advectSemiLagrange");
  (void)openBounds;
  (void)boundaryWidth;  // deprecated in the reference, no effect
  if (!(order == 1 || order == 2))
    return fail(MG_ERR_SOLVER, "AdvectSemiLagrange: Only order 1 (regular SL) and 2 (MacCormack) supported");
  if (flags->kind != MG_FLAGS || vel->kind != MG_MAC) return fail(MG_ERR_ARG, "advectSemiLagrange: flags must be a FlagGrid and vel a MACGrid");
  if (flags->s != vel->s || grid->s != vel->s) return fail(MG_ERR_ARG, "advectSemiLagrange: grids of different solvers");
  if (orderTrace != 1 && orderTrace != 2) return fail(MG_ERR_SOLVER, "Unknown backtracing order " + std::to_string(orderTrace));
  if (orderSpace != 1 && orderSpace != 2) return fail(MG_ERR_SOLVER, "Unknown interpolation order " + std::to_string(orderSpace));
  mg_solver s = flags->s;
  const Dims& d = s->d;
  const float dt = s->dt;
  if (grid->kind == MG_INT || grid->kind == MG_FLAGS)
    return fail(MG_ERR_SOLVER, "AdvectSemiLagrange: Grid Type is not supported (only Real, Vec3, MAC, Levelset)");
  if (grid->kind == MG_MAC) {
    const size_t bytes = grid->bytes();
    Tmp fwd(s, bytes);
    if (!fwd.p) return fail(MG_ERR_NOMEM, "advectSemiLagrange: out of device memory");
    {
      ProfScope ps(s, "advect_mac_fwd");
      launch_advect_sl_mac(d, vel->cmac(), grid->cmac(), fwd.mac(), dt, orderSpace, orderTrace, s->stream);
    }
    CKL();
    const float ts = (float)std::max(1.0, (double)dt * 4);
    if (order == 1) {
      Tmp dst(s, bytes);
      if (!dst.p) return fail(MG_ERR_NOMEM, "advectSemiLagrange: out of device memory");
      {
        ProfScope ps(s, "advect_outflow");
        launch_outflow_bc(d, flags->i(), fwd.cmac(), grid->cmac(), dst.mac(), fwd.mac(), ts, s->stream);
      }
      CKL();
      std::swap(grid->data, fwd.p);  // orig.swap(fwd); old storage returns to the pool
    } else {
      Tmp nw(s, bytes);
      if (!nw.p) return fail(MG_ERR_NOMEM, "advectSemiLagrange: out of device memory");
      {
        ProfScope ps(s, "advect_mac_maccormack");
        launch_advect_maccormack_mac(d, flags->i(), vel->cmac(), grid->cmac(), fwd.cmac(), nw.mac(), dt, strength, clampMode,
                                     orderSpace, orderTrace, s->stream);
      }
      CKL();
      {
        ProfScope ps(s, "advect_outflow");
        launch_outflow_bc(d, flags->i(), nw.cmac(), grid->cmac(), fwd.mac(), nw.mac(), ts, s->stream);
      }
      CKL();
      std::swap(grid->data, nw.p);
    }
    return MG_OK;
  }
  const int ch = grid->kind == MG_VEC3 ? 3 : 1;
  const size_t bytes = grid->bytes();
  Tmp fwd(s, bytes);
  if (!fwd.p) return fail(MG_ERR_NOMEM, "advectSemiLagrange: out of device memory");
  {
    ProfScope ps(s, ch == 1 ? "advect_real_fwd" : "advect_vec3_fwd");
    launch_advect_sl(d, ch, vel->cmac(), grid->f(), fwd.f(), dt, orderSpace, orderTrace, s->stream);
  }
  CKL();
  if (order == 1) {
    std::swap(grid->data, fwd.p);
    return MG_OK;
  }
  Tmp nw(s, bytes);
  if (!nw.p) return fail(MG_ERR_NOMEM, "advectSemiLagrange: out of device memory");
  {
    ProfScope ps(s, ch == 1 ? "advect_real_maccormack" : "advect_vec3_maccormack");
    launch_advect_maccormack(d, ch, flags->i(), vel->cmac(), grid->f(), fwd.f(), nw.f(), dt, strength, clampMode,
                             orderSpace, orderTrace, s->stream);
  }
  CKL();
  std::swap(grid->data, nw.p);
  return MG_OK;
}

// ---------------------------------------------- advection without allocation
// mg_advect_semi_lagrange_noalloc keeps its two temporaries (the forward
// trace and the MacCormack / outflow result) in this fixed device array
// instead of the solver's pool, for callers that must not allocate device
// memory once they run: hosts that have handed the rest of the GPU to their
// own allocator, and latency-bound loops where a cudaMalloc/cudaFree (which
// may synchronise the device) cannot be afforded.  Each temporary holds up to
// kNoAllocSlotFloats floats: a Real or levelset grid of up to 3,145,728 cells,
// a Vec3 or MAC grid of up to 1,048,576 cells.  Every launch of a call writes
// each cell that a later launch of the same call reads, so nothing has to
// start at zero.  All calls share the one array: calls that overlap on the GPU
// (solvers on different streams running at the same time) race on it.
constexpr size_t kNoAllocSlotFloats = (size_t)3 << 20;
static __device__ __align__(256) float g_noallocScratch[2 * kNoAllocSlotFloats];
static float* g_noallocPtr[64] = {};  // per device ordinal, set on first use

// mg_shutdown forgets the resolved addresses: a host may reset the device
// before the next mg_init, after which the module (and the array) reload
static void noalloc_forget() {
  for (auto& p : g_noallocPtr) p = nullptr;
}

// Resolves the array's device address for the current device.  Runs once per
// device, on the first call, which should therefore come before any stream
// capture on that device.
static int noalloc_scratch(float** out) {
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  const int dev = g_ctx.device;
  if (dev < 0 || dev >= 64) return fail(MG_ERR_STATE, "advectSemiLagrange (no-alloc): device ordinal out of range");
  if (!g_noallocPtr[dev]) {
    CK(cudaSetDevice(dev));
    void* p = nullptr;
    CK(cudaGetSymbolAddress(&p, g_noallocScratch));
    g_noallocPtr[dev] = (float*)p;
  }
  *out = g_noallocPtr[dev];
  return MG_OK;
}

extern "C" int mg_advect_semi_lagrange_noalloc(mg_grid flags, mg_grid vel, mg_grid grid, int order, float strength,
                                               int orderSpace, int openBounds, int boundaryWidth, int clampMode,
                                               int orderTrace) {
  NEED_GRID(flags, "advectSemiLagrange");
  NEED_GRID(vel, "advectSemiLagrange");
  NEED_GRID(grid, "advectSemiLagrange");
  (void)openBounds;
  (void)boundaryWidth;
  if (!(order == 1 || order == 2))
    return fail(MG_ERR_SOLVER, "AdvectSemiLagrange: Only order 1 (regular SL) and 2 (MacCormack) supported");
  if (flags->kind != MG_FLAGS || vel->kind != MG_MAC) return fail(MG_ERR_ARG, "advectSemiLagrange: flags must be a FlagGrid and vel a MACGrid");
  if (flags->s != vel->s || grid->s != vel->s) return fail(MG_ERR_ARG, "advectSemiLagrange: grids of different solvers");
  if (orderTrace != 1 && orderTrace != 2) return fail(MG_ERR_SOLVER, "Unknown backtracing order " + std::to_string(orderTrace));
  if (orderSpace != 1 && orderSpace != 2) return fail(MG_ERR_SOLVER, "Unknown interpolation order " + std::to_string(orderSpace));
  if (grid->kind == MG_INT || grid->kind == MG_FLAGS)
    return fail(MG_ERR_SOLVER, "AdvectSemiLagrange: Grid Type is not supported (only Real, Vec3, MAC, Levelset)");
  mg_solver s = flags->s;
  const Dims& d = s->d;
  const float dt = s->dt;
  const size_t floats = (size_t)grid->comps() * (size_t)d.n;
  if (floats > kNoAllocSlotFloats)
    return fail(MG_ERR_ARG, "mg_advect_semi_lagrange_noalloc: the grid holds " + std::to_string(floats) +
                                " floats; the fixed scratch takes at most " + std::to_string(kNoAllocSlotFloats) +
                                " (a Real grid of 3145728 cells, a Vec3/MAC grid of 1048576 cells)");
  float* scratch = nullptr;
  const int st = noalloc_scratch(&scratch);
  if (st) return st;
  float* A = scratch;
  float* B = scratch + kNoAllocSlotFloats;
  const Mac mA{A, A + d.n, A + 2 * d.n}, mB{B, B + d.n, B + 2 * d.n};
  const CMac cA{A, A + d.n, A + 2 * d.n}, cB{B, B + d.n, B + 2 * d.n};
  const float* result;
  if (grid->kind == MG_MAC) {
    launch_advect_sl_mac(d, vel->cmac(), grid->cmac(), mA, dt, orderSpace, orderTrace, s->stream);
    CKL();
    const float ts = (float)std::max(1.0, (double)dt * 4);
    if (order == 1) {
      launch_outflow_bc(d, flags->i(), cA, grid->cmac(), mB, mA, ts, s->stream);
      result = A;
    } else {
      launch_advect_maccormack_mac(d, flags->i(), vel->cmac(), grid->cmac(), cA, mB, dt, strength, clampMode, orderSpace,
                                   orderTrace, s->stream);
      CKL();
      launch_outflow_bc(d, flags->i(), cB, grid->cmac(), mA, mB, ts, s->stream);
      result = B;
    }
    CKL();
  } else {
    const int ch = grid->comps();
    launch_advect_sl(d, ch, vel->cmac(), grid->f(), A, dt, orderSpace, orderTrace, s->stream);
    CKL();
    result = A;
    if (order == 2) {
      launch_advect_maccormack(d, ch, flags->i(), vel->cmac(), grid->f(), A, B, dt, strength, clampMode, orderSpace,
                               orderTrace, s->stream);
      CKL();
      result = B;
    }
  }
  // the result goes back into the grid's own storage (the pooled entry point
  // swaps storage instead)
  CK(cudaMemcpyAsync(grid->data, result, floats * sizeof(float), cudaMemcpyDeviceToDevice, s->stream));
  return MG_OK;
}

extern "C" int mg_reset_phi_in_obs(mg_grid flags, mg_grid sdf) {
  NEED_GRID(flags, "resetPhiInObs");
  NEED_GRID(sdf, "resetPhiInObs");
  launch_reset_phi_in_obs(flags->s->d, flags->i(), sdf->f(), flags->s->stream);
  CKL();
  return MG_OK;
}

// =================================================================== forces
extern "C" int mg_set_wall_bcs(mg_grid flags, mg_grid vel, mg_grid obvel, mg_grid fractions, mg_grid phiObs,
                               int boundaryWidth) {
  NEED_GRID(flags, "setWallBcs");
  NEED_GRID(vel, "setWallBcs");
  (void)boundaryWidth;
  if (fractions && phiObs)
    return fail(MG_ERR_UNSUPPORTED, "setWallBcs: the fractions/phiObs (KnSetWallBcsFrac) mode is not supported");
  if (obvel && !valid_grid(obvel)) return fail(MG_ERR_ARG, "setWallBcs: invalid obvel");
  mg_solver s = flags->s;
  ProfScope ps(s, "set_wall_bcs");
  Mac ob;
  if (obvel) ob = obvel->mac();
  launch_set_wall_bcs(s->d, flags->i(), vel->mac(), obvel ? &ob : nullptr, s->stream);
  CKL();
  return MG_OK;
}

static float grid_dx(const Dims& d) {
  const int m = std::max(d.nx, std::max(d.ny, d.nz));
  return (float)(1.0 / (double)m);  // mDx = 1.0 / mSize.max() (grid.cpp:55)
}

extern "C" int mg_add_buoyancy(mg_grid flags, mg_grid density, mg_grid vel, float gx, float gy, float gz, float coefficient,
                               int scale) {
  NEED_GRID(flags, "addBuoyancy");
  NEED_GRID(density, "addBuoyancy");
  NEED_GRID(vel, "addBuoyancy");
  mg_solver s = flags->s;
  const float gridScale = scale ? grid_dx(s->d) : 1.f;
  const float dt = s->dt;
  // f = -gravity * dt / gridScale * coefficient, then (0.5 * f) per axis
  const float fx = ((-gx) * dt) / gridScale * coefficient;
  const float fy = ((-gy) * dt) / gridScale * coefficient;
  const float fz = ((-gz) * dt) / gridScale * coefficient;
  ProfScope ps(s, "add_buoyancy");
  launch_add_buoyancy(s->d, flags->i(), density->f(), vel->mac(), 0.5f * fx, 0.5f * fy, 0.5f * fz, s->stream);
  CKL();
  return MG_OK;
}

extern "C" int mg_add_gravity(mg_grid flags, mg_grid vel, float gx, float gy, float gz, mg_grid exclude, int scale) {
  NEED_GRID(flags, "addGravity");
  NEED_GRID(vel, "addGravity");
  if (exclude && !valid_grid(exclude)) return fail(MG_ERR_ARG, "addGravity: invalid exclude grid");
  mg_solver s = flags->s;
  const float gridScale = scale ? grid_dx(s->d) : 1.f;
  const float dt = s->dt;
  ProfScope ps(s, "add_gravity");
  launch_add_force(s->d, flags->i(), vel->mac(), (gx * dt) / gridScale, (gy * dt) / gridScale, (gz * dt) / gridScale,
                   exclude ? exclude->f() : nullptr, s->stream);
  CKL();
  return MG_OK;
}

extern "C" int mg_add_gravity_no_scale(mg_grid flags, mg_grid vel, float gx, float gy, float gz, mg_grid exclude) {
  return mg_add_gravity(flags, vel, gx, gy, gz, exclude, 0);
}

static void desc_to_vec(const char* desc, int* lo, int* up, bool* bad) {
  lo[0] = lo[1] = lo[2] = up[0] = up[1] = up[2] = 0;
  *bad = false;
  for (const char* c = desc; c && *c; c++) {
    switch (*c) {
      case 'x': lo[0] = 1; break;
      case 'y': lo[1] = 1; break;
      case 'z': lo[2] = 1; break;
      case 'X': up[0] = 1; break;
      case 'Y': up[1] = 1; break;
      case 'Z': up[2] = 1; break;
      default: *bad = true;
    }
  }
}

extern "C" int mg_set_open_bound(mg_grid flags, int bWidth, const char* openBound, int type) {
  NEED_GRID(flags, "setOpenBound");
  if (!openBound || !openBound[0]) return MG_OK;
  int lo[3], up[3];
  bool bad;
  desc_to_vec(openBound, lo, up, &bad);
  if (bad) return fail(MG_ERR_SOLVER, "invalid character in boundary description string. Only [xyzXYZ] allowed.");
  mg_solver s = flags->s;
  launch_set_open_bound(s->d, flags->i(), bWidth, lo, up, type, s->stream);
  CKL();
  return MG_OK;
}

extern "C" int mg_reset_outflow(mg_grid flags, mg_grid phi, mg_grid real) {
  NEED_GRID(flags, "resetOutflow");
  mg_solver s = flags->s;
  launch_reset_outflow(s->d, flags->i(), phi ? phi->f() : nullptr, real ? real->f() : nullptr, s->stream);
  CKL();
  return MG_OK;
}

extern "C" int mg_extrapolate_mac_simple(mg_grid flags, mg_grid vel, int distance, mg_grid phiObs, int intoObs) {
  NEED_GRID(flags, "extrapolateMACSimple");
  NEED_GRID(vel, "extrapolateMACSimple");
  mg_solver s = flags->s;
  if (phiObs) {
    NEED_GRID(phiObs, "extrapolateMACSimple");
    if (!is_real(phiObs) || phiObs->s != s) return fail(MG_ERR_ARG, "extrapolateMACSimple: phiObs must be a levelset of the same solver");
  }
  Tmp tmp(s, sizeof(int) * (size_t)s->d.n);
  Tmp snap(s, vel->bytes());
  if (!tmp.p || !snap.p) return fail(MG_ERR_NOMEM, "extrapolateMACSimple: out of device memory");
  ProfScope ps(s, "extrapolate_mac_simple");
  launch_extrapolate_mac_simple(s->d, flags->i(), vel->mac(), tmp.i(), snap.mac(), distance, intoObs,
                                phiObs ? phiObs->f() : nullptr, s->stream);
  CKL();
  return MG_OK;
}

extern "C" int mg_extrapolate_ls_simple(mg_grid phi, int distance, int inside) {
  NEED_GRID(phi, "extrapolateLsSimple");
  if (!is_real(phi)) return fail(MG_ERR_ARG, "extrapolateLsSimple: phi must be a Real or Levelset grid");
  mg_solver s = phi->s;
  Tmp tmp(s, sizeof(int) * (size_t)s->d.n), mark(s, sizeof(int) * (size_t)s->d.n);
  if (!tmp.p || !mark.p) return fail(MG_ERR_NOMEM, "extrapolateLsSimple: out of device memory");
  ProfScope ps(s, "extrapolate_ls_simple");
  launch_extrapolate_ls_simple(s->d, phi->f(), tmp.i(), mark.i(), distance, inside, s->stream);
  CKL();
  return MG_OK;
}

// ================================================================ pressure
extern "C" void mg_pressure_params_default(mg_pressure_params* p) {
  if (!p) return;
  p->cgAccuracy = 1e-3f;
  p->gfClamp = 1e-4f;
  p->cgMaxIterFac = 1.5f;
  p->precondition = 1;
  p->preconditioner = MG_PC_MIC;
  p->enforceCompatibility = 0;
  p->useL2Norm = 0;
  p->zeroPressureFixing = 0;
  p->surfTens = 0.f;
}

static int ensure_cg_state(mg_solver s) {
  if (s->code) return MG_OK;
  const size_t n = (size_t)s->d.n;
  CK(cudaMalloc(&s->code, n * sizeof(code_t)));
  CK(cudaMalloc(&s->residual, n * sizeof(float)));
  CK(cudaMalloc(&s->search, n * sizeof(float)));
  CK(cudaMalloc(&s->tmp, n * sizeof(float)));
  s->nblocks = std::max(1, std::min(g_ctx.sms * 4, (int)((n + 255) / 256)));
  const dim3 g = grid3(s->d, dim3(32, 8, 1));
  const size_t nb3 = (size_t)g.x * g.y * g.z;
  int tx = (s->d.nx + 15) / 16, ty = (s->d.ny + 15) / 16, tz = (s->d.nz + 15) / 16;
  const size_t ntiles = (size_t)tx * ty * tz;
  s->partCount = std::max(std::max(2 * nb3, ntiles), (size_t)(2 * s->nblocks));
  CK(cudaMalloc(&s->part, s->partCount * sizeof(double)));
  CK(cudaMalloc(&s->partf, 2 * (size_t)s->nblocks * sizeof(float)));
  CK(cudaMalloc(&s->sc, sizeof(CgScalars)));
  CK(cudaMemset(s->sc, 0, sizeof(CgScalars)));
  CK(cudaMallocHost(&s->scHost, sizeof(CgScalars)));
  CK(cudaMalloc(&s->intScratch, 16 * sizeof(int)));
  if (s->d.is3d) {
    CK(cudaMalloc(&s->P, n * sizeof(float)));
    MicPlan& m = s->mic;
    m.tx = tx; m.ty = ty; m.tz = tz;
    m.ntiles = (int)ntiles;
    std::vector<int> order(ntiles);
    mic_plan_order(tx, ty, tz, order.data());
    CK(cudaMalloc(&m.order, ntiles * sizeof(int)));
    CK(cudaMemcpy(m.order, order.data(), ntiles * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&m.tileDone, ntiles * sizeof(unsigned int)));
    CK(cudaMemset(m.tileDone, 0, ntiles * sizeof(unsigned int)));
    CK(cudaMalloc(&m.counter, sizeof(int)));
    CK(cudaMalloc(&m.error, sizeof(int)));
    CK(cudaMemset(m.error, 0, sizeof(int)));
    m.ctas = g_ctx.sms * g_ctx.micCtasPerSm;
    // tile-dataflow sweeps (micflow.cu) by default; MANTA_GB300_MIC selects
    // the whole-tile sweeps ("tile", pressure.cu), the column-block sweeps
    // ("column", mic.cu) or the warp wavefronts ("wave", micwave.cu)
    const char* ev = getenv("MANTA_GB300_MIC");
    const std::string mk = ev ? std::string(ev) : std::string("flow");
    s->useMicCol = mic_col_supported(s->d) && mk == "column";
    s->useMicWave = mic_wave_supported(s->d) && mk == "wave";
    s->useMicFlow = !s->useMicCol && !s->useMicWave && mk != "tile";
    if (s->useMicFlow) {
      const size_t words = mic_flow_face_words(m.ntiles);
      CK(cudaMalloc(&s->micFace, words * sizeof(unsigned long long)));
      CK(cudaMemset(s->micFace, 0, words * sizeof(unsigned long long)));
    }
    if (s->useMicWave) {
      MicWavePlan& w = s->micWave;
      const char* zv = getenv("MANTA_GB300_MIC_ZW");  // tuning: z-lines per lane
      w.zw = (zv && atoi(zv) == 4) ? 4 : 8;
      mic_wave_geometry(s->d, w.zw, &w.nyb, &w.nzb, &w.rows);
      w.nunits = w.nyb * w.nzb;
      std::vector<int> ord((size_t)w.nunits);
      mic_wave_order(w.nyb, w.nzb, ord.data());
      CK(cudaMalloc(&w.order, ord.size() * sizeof(int)));
      CK(cudaMemcpy(w.order, ord.data(), ord.size() * sizeof(int), cudaMemcpyHostToDevice));
      CK(cudaMalloc(&w.counter, sizeof(int)));
      const size_t words = mic_wave_exchange_words(s->d, w.zw);
      CK(cudaMalloc(&w.exchange, words * sizeof(unsigned long long)));
      CK(cudaMemset(w.exchange, 0, words * sizeof(unsigned long long)));
      w.error = m.error;
      if ((size_t)w.nunits > s->partCount) return fail(MG_ERR_STATE, "MIC: partial buffer too small");
    }
    if (s->useMicCol) {
      MicColPlan& c = s->micCol;
      mic_col_geometry(s->d, &c.nby, &c.nbz);
      c.nblocks = c.nby * c.nbz;
      std::vector<int> ord((size_t)c.nblocks);
      mic_col_order(c.nby, c.nbz, ord.data());
      CK(cudaMalloc(&c.order, ord.size() * sizeof(int)));
      CK(cudaMemcpy(c.order, ord.data(), ord.size() * sizeof(int), cudaMemcpyHostToDevice));
      CK(cudaMalloc(&c.prog, ord.size() * sizeof(unsigned long long)));
      CK(cudaMemset(c.prog, 0, ord.size() * sizeof(unsigned long long)));
      CK(cudaMalloc(&c.counter, sizeof(int)));
      c.error = m.error;
      c.pubMask = 7;  // progress published every 8 steps
      if ((size_t)c.nblocks > s->partCount) return fail(MG_ERR_STATE, "MIC: partial buffer too small");
    }
  }
  return MG_OK;
}

static MicPlan flow_plan(mg_solver s) {
  MicPlan m = s->mic;
  m.ctas = g_ctx.sms * g_ctx.flowCtasPerSm;
  return m;
}

static int wave_ctas(mg_solver s) {
  return g_ctx.sms * (s->micWave.zw == 4 ? g_ctx.waveCtasPerSm4 : g_ctx.waveCtasPerSm8);
}

static PcgBuffers cg_buffers(mg_solver s, mg_grid flags, float* rhs, mg_grid pressure) {
  PcgBuffers b;
  b.d = s->d;
  b.flags = flags->i();
  b.code = s->code;
  b.A0f = nullptr;
  b.Aif = b.Ajf = b.Akf = nullptr;
  b.rhs = rhs;
  b.pressure = pressure ? pressure->f() : nullptr;
  b.residual = s->residual;
  b.search = s->search;
  b.tmp = s->tmp;
  b.P = s->P;
  b.part = s->part;
  b.partf = s->partf;
  b.sc = s->sc;
  b.nblocks = s->nblocks;
  return b;
}

static bool check_params(const mg_pressure_params* p) { return p != nullptr; }

extern "C" int mg_compute_pressure_rhs(mg_grid rhs, mg_grid vel, mg_grid pressure, mg_grid flags,
                                       const mg_pressure_params* p, mg_grid phi, mg_grid perCellCorr, mg_grid fractions,
                                       mg_grid obvel, mg_grid curv) {
  NEED_GRID(rhs, "computePressureRhs");
  NEED_GRID(vel, "computePressureRhs");
  NEED_GRID(flags, "computePressureRhs");
  (void)pressure;
  if (!check_params(p)) return fail(MG_ERR_ARG, "computePressureRhs: null params");
  if (fractions && (!valid_grid(fractions) || fractions->kind != MG_MAC))
    return fail(MG_ERR_ARG, "computePressureRhs: fractions must be a MACGrid");
  if (obvel && (!valid_grid(obvel) || obvel->kind != MG_MAC))
    return fail(MG_ERR_ARG, "computePressureRhs: obvel must be a MACGrid");
  mg_solver s = flags->s;
  int st = ensure_cg_state(s);
  if (st) return st;
  PcgBuffers b = cg_buffers(s, flags, rhs->f(), nullptr);
  Mac v = vel->mac();
  {
    ProfScope ps(s, "make_rhs");
    // obvel enters MakeRhs only together with fractions (pressure.cpp:56-60)
    launch_make_rhs(b, v.u, v.v, v.w, perCellCorr ? perCellCorr->f() : nullptr, phi ? phi->f() : nullptr,
                    curv ? curv->f() : nullptr, p->surfTens, p->gfClamp, p->enforceCompatibility != 0, s->stream,
                    fractions ? fractions->f() : nullptr, (fractions && obvel) ? obvel->f() : nullptr);
  }
  CKL();
  if (p->enforceCompatibility) {
    launch_compat_shift(b, s->stream);
    CKL();
  }
  return MG_OK;
}

// event pairs around the multigrid kernel families while profiling
static void mg_prof_hook(void* ctx, const char* family, int begin) {
  mg_solver s = (mg_solver)ctx;
  if (begin) {
    ProfScope tk(s, nullptr);
    s->profOpen.name = family;
    s->profOpen.a = tk.take();
    s->profOpen.b = tk.take();
    cudaEventRecord(s->profOpen.a, s->stream);
  } else {
    cudaEventRecord(s->profOpen.b, s->stream);
    s->profEvents.push_back(s->profOpen);
  }
}

// doInit's preconditioner application: r -> tmp
static int apply_precond(mg_solver s, const PcgBuffers& b, int pc, bool init) {
  if (pc == kPcMic && b.Aif) {
    // fractions: the stored-coefficient MIC(0), plane by plane
    {
      ProfScope ps(s, "mic_forward");
      launch_mic_planes(b, 1, s->stream);
    }
    {
      ProfScope ps(s, "mic_backward");
      launch_mic_planes(b, init ? 3 : 2, s->stream);
    }
  } else if (pc == kPcMic) {
    {
      ProfScope ps(s, "mic_forward");
      if (s->useMicFlow) launch_mic_flow(b, flow_plan(s), s->micFace, 1, ++s->epoch, s->waitNs, s->stream, s->stall);
      else if (s->useMicWave) launch_mic_wave(b, s->micWave, 1, ++s->epoch, s->waitNs, wave_ctas(s), s->stream);
      else if (s->useMicCol) launch_mic_col(b, s->micCol, 1, ++s->epoch, s->waitNs, g_ctx.sms, s->stream);
      else launch_mic(b, s->mic, 1, ++s->epoch, s->waitNs, s->stream);
    }
    {
      ProfScope ps(s, "mic_backward");
      if (s->useMicFlow) launch_mic_flow(b, flow_plan(s), s->micFace, init ? 3 : 2, ++s->epoch, s->waitNs, s->stream, s->stall);
      else if (s->useMicWave)
        launch_mic_wave(b, s->micWave, init ? 3 : 2, ++s->epoch, s->waitNs, wave_ctas(s), s->stream);
      else if (s->useMicCol) launch_mic_col(b, s->micCol, init ? 3 : 2, ++s->epoch, s->waitNs, g_ctx.sms, s->stream);
      else launch_mic(b, s->mic, init ? 3 : 2, ++s->epoch, s->waitNs, s->stream);
    }
  } else if (pc == kPcMg) {
    mg_set_profiler(s->mg, s->prof ? mg_prof_hook : nullptr, s);
    const int st = mg_apply(s->mg, b, init, s->stream);
    if (st) return fail(MG_ERR_CUDA, "multigrid V-cycle failed");
  } else {
    ProfScope ps(s, "pcg_copy");
    launch_pcg_copy_dot(b, s->stream);
  }
  CKL();
  return MG_OK;
}

static bool same_buffers(const PcgBuffers& a, const PcgBuffers& b) {
  return a.d.nx == b.d.nx && a.d.ny == b.d.ny && a.d.nz == b.d.nz && a.code == b.code &&
         a.A0f == b.A0f && a.pressure == b.pressure && a.residual == b.residual &&
         a.search == b.search && a.tmp == b.tmp && a.P == b.P && a.part == b.part && a.partf == b.partf &&
         a.sc == b.sc && a.nblocks == b.nblocks;
}

// GridCg::iterate with the multigrid preconditioner as one graph launch:
// about a hundred short kernels per iteration, most of them on small coarse
// levels, whose launch gaps would otherwise dominate.  Captured on first use
// and whenever the buffers or the hierarchy's kernel parameters change.
static int mg_iteration_graph(mg_solver s, const PcgBuffers& b) {
  const unsigned long long sig = mg_hierarchy_signature(s->mg);
  if (s->iterGraph && same_buffers(s->iterKey, b) && s->iterSig == sig && s->iterMg == s->mg) return MG_OK;
  if (s->iterGraph) {
    cudaGraphExecDestroy(s->iterGraph);
    s->iterGraph = nullptr;
  }
  const unsigned long long before = t_launches;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  launch_pcg_spmv(b, s->stream);
  launch_pcg_axpy(b, s->stream);
  const int e = mg_apply(s->mg, b, false, s->stream);
  launch_pcg_update(b, s->stream);
  const cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
  s->iterNodes = uncount_captured(before);
  if (e || ce != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(MG_ERR_CUDA, std::string("capturing the multigrid iteration failed: ") + cudaGetErrorString(ce));
  }
  const cudaError_t ie = cudaGraphInstantiate(&s->iterGraph, g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) {
    s->iterGraph = nullptr;
    return fail(MG_ERR_CUDA, std::string("instantiating the multigrid iteration failed: ") + cudaGetErrorString(ie));
  }
  s->iterKey = b;
  s->iterSig = sig;
  s->iterMg = s->mg;
  return MG_OK;
}

extern "C" int mg_solve_pressure_system(mg_grid rhs, mg_grid vel, mg_grid pressure, mg_grid flags,
                                        const mg_pressure_params* p, mg_grid phi, mg_grid perCellCorr, mg_grid fractions,
                                        mg_grid curv, mg_pressure_result* out) {
  NEED_GRID(rhs, "solvePressureSystem");
  NEED_GRID(vel, "solvePressureSystem");
  NEED_GRID(pressure, "solvePressureSystem");
  NEED_GRID(flags, "solvePressureSystem");
  (void)perCellCorr;
  (void)curv;
  if (!check_params(p)) return fail(MG_ERR_ARG, "solvePressureSystem: null params");
  if (fractions && (!valid_grid(fractions) || fractions->kind != MG_MAC))
    return fail(MG_ERR_ARG, "solvePressureSystem: fractions must be a MACGrid");
  mg_solver s = flags->s;
  const Dims& d = s->d;
  int preconditioner = p->precondition ? p->preconditioner : MG_PC_NONE;
  if (preconditioner == MG_PC_NONE)
    return fail(MG_ERR_SOLVER, "GridCg<APPLYMAT>::setICPreconditioner: Invalid method specified.");
  if (preconditioner < 0 || preconditioner > MG_PC_MG_STATIC)
    return fail(MG_ERR_ARG, "solvePressureSystem: unknown preconditioner");
  int st = ensure_cg_state(s);
  if (st) return st;
  PcgBuffers b = cg_buffers(s, flags, rhs->f(), pressure);
  {
    ProfScope ps(s, "make_codes");
    launch_make_codes(b, s->stream);
  }
  CKL();
  if (fractions || phi) {
    if (!s->A0f) CK(cudaMalloc(&s->A0f, sizeof(float) * (size_t)d.n));
    b.A0f = s->A0f;
  }
  if (fractions) {
    // MakeLaplaceMatrix with fractions: the float matrix as the reference stores it
    if (!s->Aoff) CK(cudaMalloc(&s->Aoff, 3 * sizeof(float) * (size_t)d.n));
    b.Aif = s->Aoff;
    b.Ajf = s->Aoff + d.n;
    b.Akf = s->Aoff + 2 * d.n;
    launch_make_frac_matrix(b, fractions->f(), s->stream);
    CKL();
  }
  if (phi) {
    launch_ghost_fluid_diag(b, phi->f(), p->gfClamp, s->stream);
    CKL();
  }
  if (p->zeroPressureFixing || p->cgAccuracy < 1e-07) {
    launch_count_empty(b, s->intScratch, s->stream);
    CKL();
    int numEmpty = 0;
    CK(cudaMemcpyAsync(&numEmpty, s->intScratch, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (numEmpty == 0) {
      std::vector<int> hf((size_t)d.n);
      CK(cudaMemcpy(hf.data(), flags->data, sizeof(int) * hf.size(), cudaMemcpyDeviceToHost));
      long long fix = -1;
      const int tc[3] = {d.nx / 2, d.ny - 1, d.is3d ? d.nz / 2 : 0};
      for (int q = 0; q < 3 && fix < 0; q++) {
        const long long e = ix(d, tc[0], tc[1] - q, tc[2]);
        if (hf[e] & kFluid) fix = e;
      }
      for (int k = d.is3d ? 1 : 0; k < (d.is3d ? d.nz - 1 : 1) && fix < 0; k++)
        for (int j = 1; j < d.ny - 1 && fix < 0; j++)
          for (int i = 1; i < d.nx - 1 && fix < 0; i++)
            if (hf[ix(d, i, j, k)] & kFluid) fix = ix(d, i, j, k);
      if (fix >= 0) {
        launch_fix_pressure(b, fix, s->stream);
        CKL();
      }
    }
  }
  int pc = kPcNone;
  int maxIter;
  if (preconditioner == MG_PC_MIC) {
    maxIter = (int)(p->cgMaxIterFac * (float)std::max(d.nx, std::max(d.ny, d.nz))) * (d.is3d ? 1 : 4);
    pc = d.is3d ? kPcMic : kPcNone;  // mICP only in 3D (conjugategrad.cpp:315-321)
  } else {
    maxIter = 100;
    pc = kPcMg;
    // PcMGDynamic builds the hierarchy for this matrix and forgets it
    // afterwards; PcMGStatic keeps the first one (pressure.cpp:418-451)
    if (s->mg && preconditioner == MG_PC_MG_DYNAMIC) mg_hierarchy_reset(s->mg);
    if (!s->mg) {
      s->mg = mg_hierarchy_create(d);
      if (!s->mg) return fail(MG_ERR_NOMEM, "solvePressureSystem: multigrid allocation failed");
    }
    const int e = mg_setup(s->mg, b, (float)((double)p->cgAccuracy * 1E-4), s->stream);
    if (e) return fail(MG_ERR_CUDA, std::string("multigrid setup failed: ") + cudaGetErrorString(cudaGetLastError()));
  }
  // GridCg::doInit
  CgScalars init{};
  init.accuracy = p->cgAccuracy;
  init.useL2 = p->useL2Norm;
  init.maxIter = maxIter;
  init.resNorm = 1e20f;
  CK(cudaMemcpyAsync(s->sc, &init, sizeof(CgScalars), cudaMemcpyHostToDevice, s->stream));
  {
    ProfScope ps(s, "pcg_init");
    launch_pcg_init(b, s->stream);
  }
  CKL();
  if (pc == kPcMic) {
    ProfScope ps(s, "mic_init");
    s->stall = s->stallNext;
    s->stallNext = false;
    CK(cudaMemsetAsync(s->mic.error, 0, sizeof(int), s->stream));
    if (b.Aif) launch_mic_planes(b, 0, s->stream);
    else if (s->useMicFlow) launch_mic_flow(b, flow_plan(s), s->micFace, 0, ++s->epoch, s->waitNs, s->stream, s->stall);
    else if (s->useMicWave) launch_mic_wave(b, s->micWave, 0, ++s->epoch, s->waitNs, wave_ctas(s), s->stream);
    else if (s->useMicCol) launch_mic_col(b, s->micCol, 0, ++s->epoch, s->waitNs, g_ctx.sms, s->stream);
    else launch_mic(b, s->mic, 0, ++s->epoch, s->waitNs, s->stream);
    CKL();
  }
  if (pc != kPcNone) {
    st = apply_precond(s, b, pc, true);
    if (st) return st;
  } else {
    ProfScope ps(s, "pcg_copy");
    CK(cudaMemcpyAsync(b.tmp, b.residual, sizeof(float) * (size_t)d.n, cudaMemcpyDeviceToDevice, s->stream));
  }
  {
    ProfScope ps(s, "pcg_set_search");
    launch_pcg_set_search(b, s->stream);
  }
  CKL();
  // GridCg::iterate until converged or maxIter; the host polls the device
  // flag a few iterations behind so the GPU never waits for the CPU.  While
  // profiling it polls every iteration, so that every launch it times did
  // work (launches after convergence return at once)
  const int lag = s->prof ? 1 : 4;
  std::vector<cudaEvent_t> ev;
  int it = 0;
  bool done = false;
  int* doneHost = &s->scHost->done;
  *doneHost = 0;
  // the MG iteration runs as a CUDA graph unless per-kernel profiling is on
  const bool graph = pc == kPcMg && !s->prof;
  if (graph) {
    st = mg_iteration_graph(s, b);
    if (st) return st;
  }
  while (it < maxIter && !done) {
    if (graph) {
      CK(cudaGraphLaunch(s->iterGraph, s->stream));
      g_launches.fetch_add(s->iterNodes, std::memory_order_relaxed);
      it++;
      if (it % lag == 0 || it == maxIter) {
        CK(cudaMemcpyAsync(s->scHost, s->sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        done = s->scHost->done != 0;
      }
      continue;
    }
    {
      ProfScope ps(s, "pcg_spmv");
      launch_pcg_spmv(b, s->stream);
    }
    {
      ProfScope ps(s, "pcg_axpy");
      launch_pcg_axpy(b, s->stream);
    }
    if (s->prof) {
      // the axpy's residual norm may have converged the solve, after which
      // the iteration's remaining launches would return at once: leave them
      // out, so the profile times only launches that did work
      CKL();
      CK(cudaMemcpyAsync(s->scHost, s->sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, s->stream));
      CK(cudaStreamSynchronize(s->stream));
      if (s->scHost->done) {
        it++;
        break;
      }
    }
    st = apply_precond(s, b, pc, false);
    if (st) return st;
    {
      ProfScope ps(s, "pcg_update");
      launch_pcg_update(b, s->stream);
    }
    CKL();
    it++;
    if (it % lag == 0 || it == maxIter) {
      CK(cudaMemcpyAsync(s->scHost, s->sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, s->stream));
      CK(cudaStreamSynchronize(s->stream));
      done = s->scHost->done != 0;
    }
  }
  CK(cudaMemcpyAsync(s->scHost, s->sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (pc == kPcMic) {
    s->stall = false;
    int err = 0;
    CK(cudaMemcpy(&err, s->mic.error, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) return fail(MG_ERR_TIMEOUT, "MIC wavefront: a tile wait exceeded its spin limit");
  }
  if (out) {
    out->iterations = s->scHost->iterations;
    out->resNorm = s->scHost->resNorm;
  }
  if (s->scHost->status == 2)
    return fail(MG_ERR_SOLVER, "GridCg::iterate: The CG solver diverged, residual norm > 1e30, stopping.");
  if (s->scHost->status == 4) return fail(MG_ERR_TIMEOUT, "PCG: a plane copy of the streamed SpMV exceeded its wait limit");
  if (s->mg && preconditioner == MG_PC_MG_DYNAMIC) mg_hierarchy_reset(s->mg);
  return MG_OK;
}

extern "C" void mg_refine_params_default(mg_refine_params* r) {
  if (!r) return;
  r->refineAccuracy = 1e-5;
  r->innerAccuracy = 1e-2;
  r->maxRefine = 10;
}

// solvePressure with FP64 residual refinement: MakeRhs, then FP32 PCG solves
// of A delta = (float) r accumulated into a double pressure until the
// double-precision residual max|b - A p| drops below refineAccuracy, then
// correctVelocity with the rounded pressure
extern "C" int mg_solve_pressure_refined(mg_grid vel, mg_grid pressure, mg_grid flags, const mg_pressure_params* p,
                                         mg_grid phi, const mg_refine_params* rp, mg_refine_result* out) {
  NEED_GRID(vel, "solvePressureRefined");
  NEED_GRID(pressure, "solvePressureRefined");
  NEED_GRID(flags, "solvePressureRefined");
  mg_pressure_params def;
  if (!p) {
    mg_pressure_params_default(&def);
    p = &def;
  }
  mg_refine_params rdef;
  if (!rp) {
    mg_refine_params_default(&rdef);
    rp = &rdef;
  }
  if (!(rp->refineAccuracy > 0.) || !(rp->innerAccuracy > 0.) || rp->maxRefine < 1)
    return fail(MG_ERR_ARG, "solvePressureRefined: refineAccuracy and innerAccuracy must be > 0, maxRefine >= 1");
  if (p->enforceCompatibility) return fail(MG_ERR_UNSUPPORTED, "solvePressureRefined: enforceCompatibility is not supported");
  mg_solver s = flags->s;
  const size_t n = (size_t)s->d.n;
  Tmp rhs(s, sizeof(float) * n), delta(s, sizeof(float) * n), b64(s, sizeof(double) * n), p64(s, sizeof(double) * n),
      norm(s, sizeof(double));
  if (!rhs.p || !delta.p || !b64.p || !p64.p || !norm.p) return fail(MG_ERR_NOMEM, "solvePressureRefined: out of device memory");
  mg_grid_s rg, dg;
  rg.s = dg.s = s;
  rg.kind = dg.kind = MG_REAL;
  rg.data = rhs.p;
  dg.data = delta.p;
  s->grids.insert(&rg);
  s->grids.insert(&dg);
  struct Unreg {
    mg_solver s;
    mg_grid a, b;
    ~Unreg() {
      s->grids.erase(a);
      s->grids.erase(b);
    }
  } unreg{s, &rg, &dg};
  int st = mg_compute_pressure_rhs(&rg, vel, pressure, flags, p, phi, nullptr, nullptr, nullptr, nullptr);
  if (st) return st;
  CK(cudaMemsetAsync(p64.p, 0, sizeof(double) * n, s->stream));
  double* const P64 = (double*)p64.p;
  double* const B64 = (double*)b64.p;
  mg_pressure_params pin = *p;
  double rnorm = 0.;
  int total = 0, k = 0;
  for (; k < rp->maxRefine; k++) {
    // inner FP32 solve of A delta = r (the first one is the plain solve; it
    // also applies the pressure pinning to rhs, which the double right-hand
    // side then takes over)
    if (k > 0) pin.cgAccuracy = (float)(rp->innerAccuracy * rnorm);
    if (k > 0 && pin.cgAccuracy < 1e-30f) break;
    mg_pressure_result r{};
    st = mg_solve_pressure_system(&rg, vel, &dg, flags, &pin, phi, nullptr, nullptr, nullptr, &r);
    if (st) return st;
    total += r.iterations;
    if (k == 0) launch_to_double((long long)n, rhs.f(), B64, s->stream);
    launch_add_delta((long long)n, P64, delta.f(), s->stream);
    launch_residual64(s->d, s->code, phi ? s->A0f : nullptr, B64, P64, rhs.f(), s->part, &s->sc->counters[5],
                      (double*)norm.p, s->stream);
    CKL();
    CK(cudaMemcpyAsync(&rnorm, norm.p, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (rnorm < rp->refineAccuracy) {
      k++;
      break;
    }
  }
  launch_to_float((long long)n, P64, pressure->f(), s->stream);
  CKL();
  st = mg_correct_velocity(vel, pressure, flags, p, phi, nullptr, nullptr, nullptr);
  if (st) return st;
  if (out) {
    out->refinements = k;
    out->iterations = total;
    out->resNorm = rnorm;
  }
  return MG_OK;
}

extern "C" int mg_correct_velocity(mg_grid vel, mg_grid pressure, mg_grid flags, const mg_pressure_params* p,
                                   mg_grid phi, mg_grid perCellCorr, mg_grid fractions, mg_grid curv) {
  NEED_GRID(vel, "correctVelocity");
  NEED_GRID(pressure, "correctVelocity");
  NEED_GRID(flags, "correctVelocity");
  (void)perCellCorr;
  (void)fractions;
  if (!check_params(p)) return fail(MG_ERR_ARG, "correctVelocity: null params");
  mg_solver s = flags->s;
  ProfScope ps(s, "correct_velocity");
  launch_correct_velocity(s->d, flags->i(), vel->mac(), pressure->f(), phi ? phi->f() : nullptr,
                          curv ? curv->f() : nullptr, p->gfClamp, p->surfTens, s->stream);
  CKL();
  return MG_OK;
}

extern "C" int mg_solve_pressure(mg_grid vel, mg_grid pressure, mg_grid flags, const mg_pressure_params* p, mg_grid phi,
                                 mg_grid perCellCorr, mg_grid fractions, mg_grid obvel, mg_grid curv, mg_grid retRhs,
                                 mg_pressure_result* out) {
  NEED_GRID(vel, "solvePressure");
  NEED_GRID(pressure, "solvePressure");
  NEED_GRID(flags, "solvePressure");
  mg_pressure_params def;
  if (!p) {
    mg_pressure_params_default(&def);
    p = &def;
  }
  mg_solver s = flags->s;
  Tmp rhs(s, sizeof(float) * (size_t)s->d.n);
  if (!rhs.p) return fail(MG_ERR_NOMEM, "solvePressure: out of device memory");
  mg_grid_s rg;
  rg.s = s;
  rg.kind = MG_REAL;
  rg.data = rhs.p;
  s->grids.insert(&rg);
  struct Unreg {
    mg_solver s;
    mg_grid g;
    ~Unreg() { s->grids.erase(g); }
  } unreg{s, &rg};
  int st = mg_compute_pressure_rhs(&rg, vel, pressure, flags, p, phi, perCellCorr, fractions, obvel, curv);
  if (st) return st;
  st = mg_solve_pressure_system(&rg, vel, pressure, flags, p, phi, perCellCorr, fractions, curv, out);
  if (st) return st;
  st = mg_correct_velocity(vel, pressure, flags, p, phi, perCellCorr, nullptr, curv);
  if (st) return st;
  if (retRhs) {
    NEED_GRID(retRhs, "solvePressure");
    CK(cudaMemcpyAsync(retRhs->data, rhs.p, sizeof(float) * (size_t)s->d.n, cudaMemcpyDeviceToDevice, s->stream));
  }
  return MG_OK;
}

extern "C" int mg_multigrid_vcycle(mg_grid flags, mg_grid phi, mg_grid src, mg_grid dst, float gfClamp,
                                   float coarseAccuracy) {
  NEED_GRID(flags, "mg_multigrid_vcycle");
  NEED_GRID(src, "mg_multigrid_vcycle");
  NEED_GRID(dst, "mg_multigrid_vcycle");
  mg_solver s = flags->s;
  int st = ensure_cg_state(s);
  if (st) return st;
  PcgBuffers b = cg_buffers(s, flags, nullptr, nullptr);
  launch_make_codes(b, s->stream);
  CKL();
  if (phi) {
    if (!s->A0f) CK(cudaMalloc(&s->A0f, sizeof(float) * (size_t)s->d.n));
    b.A0f = s->A0f;
    launch_ghost_fluid_diag(b, phi->f(), gfClamp, s->stream);
    CKL();
  }
  mgpu::MgHierarchy* h = mg_hierarchy_create(s->d);
  if (!h) return fail(MG_ERR_NOMEM, "mg_multigrid_vcycle: multigrid allocation failed");
  CgScalars init{};
  CK(cudaMemcpyAsync(s->sc, &init, sizeof(CgScalars), cudaMemcpyHostToDevice, s->stream));
  CK(cudaMemcpyAsync(b.residual, src->f(), sizeof(float) * (size_t)s->d.n, cudaMemcpyDeviceToDevice, s->stream));
  int e = mg_setup(h, b, coarseAccuracy, s->stream);
  if (!e) e = mg_apply(h, b, true, s->stream);
  if (!e)
    e = cudaMemcpyAsync(dst->f(), b.tmp, sizeof(float) * (size_t)s->d.n, cudaMemcpyDeviceToDevice, s->stream) !=
        cudaSuccess;
  cudaStreamSynchronize(s->stream);
  mg_hierarchy_destroy(h);
  if (e) return fail(MG_ERR_CUDA, "mg_multigrid_vcycle: multigrid failed");
  return MG_OK;
}

extern "C" int mg_multigrid_describe(mg_grid flags, mg_multigrid_layout* out) {
  NEED_GRID(flags, "mg_multigrid_describe");
  if (!out) return fail(MG_ERR_ARG, "mg_multigrid_describe: out is NULL");
  mg_solver s = flags->s;
  int st = ensure_cg_state(s);
  if (st) return st;
  PcgBuffers b = cg_buffers(s, flags, nullptr, nullptr);
  launch_make_codes(b, s->stream);
  CKL();
  mgpu::MgHierarchy* h = mg_hierarchy_create(s->d);
  if (!h) return fail(MG_ERR_NOMEM, "mg_multigrid_describe: multigrid allocation failed");
  const int e = mg_setup(h, b, 1e-8f, s->stream);
  cudaStreamSynchronize(s->stream);
  mgpu::MgLayout L;
  mgpu::mg_hierarchy_describe(h, &L);
  mg_hierarchy_destroy(h);
  if (e) return fail(MG_ERR_CUDA, "mg_multigrid_describe: multigrid setup failed");
  out->levels = L.levels;
  out->tailFirst = L.tailFirst;
  out->tailCtas = L.tailCtas;
  for (int l = 0; l < 32; l++) {
    for (int c = 0; c < 3; c++) out->size[l][c] = L.size[l][c];
    out->dictStencils[l] = L.dictStencils[l];
  }
  return MG_OK;
}

extern "C" int mg_release_mg(mg_solver s) {
  if (!s) {
    for (auto x : g_ctx.solvers)
      if (x->mg) {
        cudaStreamSynchronize(x->stream);
        mg_hierarchy_destroy(x->mg);
        x->mg = nullptr;
      }
    return MG_OK;
  }
  if (!valid_solver(s)) return fail(MG_ERR_ARG, "releaseMG: invalid solver");
  if (s->mg) {
    cudaStreamSynchronize(s->stream);
    mg_hierarchy_destroy(s->mg);
    s->mg = nullptr;
  }
  return MG_OK;
}

// ================================================================== setup
extern "C" int mg_flags_init_domain(mg_grid flags, int boundaryWidth, const char* wallIn, const char* openIn,
                                    const char* inflowIn, const char* outflowIn, mg_grid phiWalls) {
  NEED_GRID(flags, "initDomain");
  if (phiWalls) return fail(MG_ERR_UNSUPPORTED, "initDomain: phiWalls is not supported");
  std::string wall = std::string(wallIn ? wallIn : "xXyYzZ") + "      ";
  std::string open = std::string(openIn ? openIn : "") + "      ";
  std::string inflow = std::string(inflowIn ? inflowIn : "") + "      ";
  std::string outflow = std::string(outflowIn ? outflowIn : "") + "      ";
  mg_solver s = flags->s;
  int types[6] = {0, 0, 0, 0, 0, 0};
  bool set[6] = {false, false, false, false, false, false};
  const char dirs[6] = {'x', 'X', 'y', 'Y', 'z', 'Z'};
  for (int i = 0; i < 6; ++i)
    for (int q = 0; q < 6; q++) {
      if (q >= 4 && !s->d.is3d) continue;
      if (set[q]) continue;
      const char ch = dirs[q];
      if (open[i] == ch) { types[q] = kOpen; set[q] = true; }
      else if (inflow[i] == ch) { types[q] = kInflow; set[q] = true; }
      else if (outflow[i] == ch) { types[q] = kOutflow; set[q] = true; }
      else if (wall[i] == ch) { types[q] = kObstacle; set[q] = true; }
    }
  launch_init_domain(s->d, flags->i(), boundaryWidth, types, s->stream);
  CKL();
  return MG_OK;
}

extern "C" int mg_flags_fill_grid(mg_grid flags, int type) {
  NEED_GRID(flags, "fillGrid");
  launch_fill_grid(flags->s->d, flags->i(), type, flags->s->stream);
  CKL();
  return MG_OK;
}

extern "C" int mg_flags_update_from_levelset(mg_grid flags, mg_grid levelset) {
  NEED_GRID(flags, "updateFromLevelset");
  NEED_GRID(levelset, "updateFromLevelset");
  ProfScope ps(flags->s, "update_from_levelset");
  launch_update_from_levelset(flags->s->d, flags->i(), levelset->f(), flags->s->stream);
  CKL();
  return MG_OK;
}

// Cylinder ctor: mZ = normalize(mZDir) (shapes.cpp:316-322, vectorbase.h:416-432)
void mgpu::cylinder_axis(const float* z, float* zn, float* mZout) {
  float zx = z[0], zy = z[1], zz = z[2], mZ;
  const float l = zx * zx + zy * zy + zz * zz;
  if (std::fabs((double)l - 1.) < (double)(1e-6f * 1e-6f)) {
    mZ = 1.f;
  } else if (l > 1e-6f * 1e-6f) {
    mZ = std::sqrt(l);
    const float inv = (float)(1. / (double)mZ);
    zx = zx * inv;
    zy = zy * inv;
    zz = zz * inv;
  } else {
    zx = zy = zz = 0.f;
    mZ = 0.f;
  }
  zn[0] = zx;
  zn[1] = zy;
  zn[2] = zz;
  *mZout = mZ;
}

static int shape_apply(mg_grid grid, int shape, const float* a, const float* b, float radius, float mZ, const float* value,
                       int ivalue, mg_grid respect) {
  mg_solver s = grid->s;
  const int* rf = respect ? respect->i() : nullptr;
  if (is_vec(grid)) {
    if (grid->kind == MG_VEC3) {
      // ApplyShapeToGrid<Vec3>: every component at the cell centre
      Mac m = grid->mac();
      for (int c = 0; c < 3; c++) {
        const float v[3] = {value[c], 0.f, 0.f};
        launch_shape_apply(s->d, shape, m.c(c), nullptr, nullptr, v, 0, rf, a, b, radius, mZ, s->stream);
      }
    } else {
      Mac m = grid->mac();
      launch_shape_apply(s->d, shape, nullptr, nullptr, &m, value, 0, rf, a, b, radius, mZ, s->stream);
    }
  } else if (grid->kind == MG_INT || grid->kind == MG_FLAGS) {
    const float v[3] = {0.f, 0.f, 0.f};
    launch_shape_apply(s->d, shape, nullptr, grid->i(), nullptr, v, ivalue, rf, a, b, radius, mZ, s->stream);
  } else {
    launch_shape_apply(s->d, shape, grid->f(), nullptr, nullptr, value, 0, rf, a, b, radius, mZ, s->stream);
  }
  CKL();
  return MG_OK;
}

extern "C" int mg_shape_box_apply(mg_grid grid, const float* p0, const float* p1, const float* value, int ivalue,
                                  mg_grid respectFlags) {
  NEED_GRID(grid, "Box.applyToGrid");
  if (!p0 || !p1 || !value) return fail(MG_ERR_ARG, "Box.applyToGrid: null argument");
  return shape_apply(grid, 0, p0, p1, 0.f, 0.f, value, ivalue, respectFlags);
}

extern "C" int mg_shape_cylinder_apply(mg_grid grid, const float* center, float radius, const float* z,
                                       const float* value, int ivalue, mg_grid respectFlags) {
  NEED_GRID(grid, "Cylinder.applyToGrid");
  if (!center || !z || !value) return fail(MG_ERR_ARG, "Cylinder.applyToGrid: null argument");
  float zn[3], mZ;
  cylinder_axis(z, zn, &mZ);
  return shape_apply(grid, 1, center, zn, radius, mZ, value, ivalue, respectFlags);
}

extern "C" int mg_shape_box_levelset(mg_grid phi, const float* p0, const float* p1) {
  NEED_GRID(phi, "Box.computeLevelset");
  if (!is_real(phi) || !p0 || !p1) return fail(MG_ERR_ARG, "Box.computeLevelset: Real grid and corners required");
  launch_box_sdf(phi->s->d, phi->f(), p0, p1, phi->s->stream);
  CKL();
  return MG_OK;
}

// ================================================================= timing
extern "C" int mg_profile_enable(mg_solver s, int on) {
  if (!valid_solver(s)) return fail(MG_ERR_ARG, "mg_profile_enable: invalid solver");
  if (!on) prof_collect(s);
  s->prof = on != 0;
  return MG_OK;
}
extern "C" int mg_profile_reset(mg_solver s) {
  if (!valid_solver(s)) return fail(MG_ERR_ARG, "mg_profile_reset: invalid solver");
  prof_collect(s);
  s->profAcc.clear();
  return MG_OK;
}
extern "C" int mg_profile_read(mg_solver s, int* count, const char** names, double* ms, long long* launches) {
  if (!valid_solver(s) || !count) return fail(MG_ERR_ARG, "mg_profile_read: invalid argument");
  prof_collect(s);
  int i = 0;
  for (auto& kv : s->profAcc) {
    if (i >= *count) break;
    if (names) names[i] = kv.first.c_str();
    if (ms) ms[i] = kv.second.first;
    if (launches) launches[i] = kv.second.second;
    i++;
  }
  *count = i;
  return MG_OK;
}
extern "C" int mg_mark(mg_solver s, int slot) {
  if (!valid_solver(s) || slot < 0 || slot >= 8) return fail(MG_ERR_ARG, "mg_mark: invalid argument");
  CK(cudaEventRecord(s->marks[slot], s->stream));
  return MG_OK;
}
extern "C" int mg_elapsed(mg_solver s, int a, int b, float* ms) {
  if (!valid_solver(s) || a < 0 || a >= 8 || b < 0 || b >= 8 || !ms) return fail(MG_ERR_ARG, "mg_elapsed: invalid argument");
  CK(cudaEventSynchronize(s->marks[b]));
  CK(cudaEventElapsedTime(ms, s->marks[a], s->marks[b]));
  return MG_OK;
}

extern "C" int mg_launch_count(long long* out) {
  if (!out) return fail(MG_ERR_ARG, "mg_launch_count: null out");
  *out = (long long)g_launches.load();
  return MG_OK;
}
