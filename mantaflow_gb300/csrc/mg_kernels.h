// Host-side launcher declarations for the grid-step kernels.
#pragma once
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "mg_common.cuh"

namespace mgpu {

// number of kernels this library has launched (the bench's gpu_launches),
// and the calling thread's share (graph captures subtract what they
// recorded, which runs only when the graph is launched)
extern std::atomic<unsigned long long> g_launches;
extern thread_local unsigned long long t_launches;
inline void count_launch() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  t_launches++;
}
// after a capture on this thread that began when t_launches was `before`:
// the number of kernels captured, no longer counted as launched
inline unsigned long long uncount_captured(unsigned long long before) {
  const unsigned long long n = t_launches - before;
  t_launches = before;
  g_launches.fetch_sub(n, std::memory_order_relaxed);
  return n;
}

// ---- advection (advect.cu)
void launch_advect_sl(const Dims& d, int ch, CMac vel, const float* src, float* dst, float dt, int orderSpace,
                      int orderTrace, cudaStream_t s);
void launch_advect_maccormack(const Dims& d, int ch, const int* flags, CMac vel, const float* orig, const float* fwd,
                              float* dst, float dt, float strength, int clampMode, int orderSpace, int orderTrace,
                              cudaStream_t s);
void launch_advect_sl_mac(const Dims& d, CMac vel, CMac src, Mac dst, float dt, int orderSpace, int orderTrace,
                         cudaStream_t s);
void launch_advect_maccormack_mac(const Dims& d, const int* flags, CMac vel, CMac orig, CMac fwd, Mac dst, float dt,
                                  float strength, int clampMode, int orderSpace, int orderTrace, cudaStream_t s);
void launch_outflow_bc(const Dims& d, const int* flags, CMac vel, CMac velPrev, Mac velDst, Mac velOut, float timeStep,
                       cudaStream_t s);
void launch_reset_phi_in_obs(const Dims& d, const int* flags, float* sdf, cudaStream_t s);

// ---- forces, setup, utilities (forces.cu)
void launch_set_wall_bcs(const Dims& d, const int* flags, Mac vel, const Mac* obvel, cudaStream_t s);
void launch_add_buoyancy(const Dims& d, const int* flags, const float* rho, Mac vel, float hx, float hy, float hz,
                         cudaStream_t s);
void launch_add_force(const Dims& d, const int* flags, Mac vel, float fx, float fy, float fz, const float* exclude,
                      cudaStream_t s);
void launch_extrapolate_mac_simple(const Dims& d, const int* flags, Mac vel, int* tmp, Mac snap, int distance, int intoObs,
                                   const float* phiObs, cudaStream_t s);
// extrapolateLsSimple; tmp, mark: int scratch grids
void launch_extrapolate_ls_simple(const Dims& d, float* phi, int* tmp, int* mark, int distance, int inside,
                                  cudaStream_t s);
void launch_init_domain(const Dims& d, int* flags, int bw, const int* types, cudaStream_t s);
void launch_fill_grid(const Dims& d, int* flags, int type, cudaStream_t s);
void launch_set_open_bound(const Dims& d, int* flags, int bw, const int* lo, const int* up, int type, cudaStream_t s);
void launch_reset_outflow(const Dims& d, int* flags, float* phi, float* real, cudaStream_t s);
void launch_update_from_levelset(const Dims& d, int* flags, const float* phi, cudaStream_t s);
void launch_box_sdf(const Dims& d, float* phi, const float* p0, const float* p1, cudaStream_t s);
void launch_shape_apply(const Dims& d, int shape, float* freal, int* fint, Mac* mac, const float* value, int ivalue,
                        const int* respect, const float* a, const float* b, float radius, float mZ, cudaStream_t s);
void launch_aos_to_soa(long long n, const float* aos, Mac soa, cudaStream_t s);
void launch_soa_to_aos(long long n, CMac soa, float* aos, cudaStream_t s);
void launch_join(long long n, float* a, const float* b, int keepMax, cudaStream_t s);
void launch_set_const(long long n, float* a, float v, cudaStream_t s);
int launch_minmax_partial(long long n, const float* a, float* part, cudaStream_t s);

// ---- pressure projection (pressure.cu)
// Per-cell 7-point stencil code replacing the reference's four stored
// coefficient grids A0/Ai/Aj/Ak (conjugategrad.h:154-187):
//   bits 0-2  A0: number of non-obstacle neighbours (interior fluid cells)
//   bit  3    cell is fluid
//   bits 4-6  Ai(c-x), Aj(c-y), Ak(c-z) == -1   (link to the lower neighbour)
//   bits 7-9  Ai(c),   Aj(c),   Ak(c)   == -1   (link to the upper neighbour)
typedef uint16_t code_t;
enum : int { kCodeFluid = 8, kLowX = 16, kLowY = 32, kLowZ = 64, kHighX = 128, kHighY = 256, kHighZ = 512 };

// device-resident scalars of one CG solve (GridCg members, conjugategrad.h:65-114)
struct CgScalars {
  float sigma, alpha, beta, resNorm, dp, accuracy;
  int iterations, done, status, maxIter;
  int useL2, pad;
  double sum;   // MakeRhs sum (enforceCompatibility)
  double refNorm;  // batched FP64 refinement: max|b - A p64| of the scene
  int cnt, pad2;
  unsigned int counters[8];  // last-block tickets
};

enum { kPcNone = 0, kPcMic = 1, kPcMg = 2 };

struct PcgBuffers {
  Dims d;
  const int* flags;
  code_t* code;
  float* A0f;       // non-null with ghost fluid or fractions: float diagonal
  float* Aif;       // non-null with fractions: float off-diagonals (the
  float* Ajf;       // reference's stored Ai, Aj, Ak; the codes still carry
  float* Akf;       // the fluid bit and the links)
  float* rhs;
  float* pressure;
  float* residual;
  float* search;
  float* tmp;
  float* P;         // MIC diagonal (Aprecond)
  double* part;     // per-block / per-tile partial sums
  float* partf;     // per-block partial max/min
  CgScalars* sc;
  int nblocks;      // blocks of the streaming kernels
};

struct MicPlan {
  int tx, ty, tz;         // tiles per axis
  int ntiles;
  int* order;             // tile dispatch order (wavefront levels)
  unsigned int* tileDone; // epoch stamp per tile
  int* counter;           // dispenser, zeroed before each sweep
  int* error;             // spin-limit diagnostics
  int ctas;               // persistent CTAs
};

// sums: also the per-block sums of rhs and fluid cells (enforceCompatibility)
// frac / obvel: the fractions and obstacle-velocity MAC grids (three planes
// of n floats each) or null
void launch_make_rhs(const PcgBuffers& b, const float* vu, const float* vv, const float* vw, const float* perCellCorr,
                     const float* phi, const float* curv, float surfTens, float gfClamp, bool sums, cudaStream_t s,
                     const float* frac = nullptr, const float* obvel = nullptr);
// MakeLaplaceMatrix with fractions: b.A0f and b.Aif/Ajf/Akf
void launch_make_frac_matrix(const PcgBuffers& b, const float* frac, cudaStream_t s);
// the stored-coefficient MIC(0) (fractions): one launch per i+j+k plane;
// mode 0 factor, 1 forward, 2 backward (+beta), 3 backward for doInit (+sigma)
void launch_mic_planes(const PcgBuffers& b, int mode, cudaStream_t s);
void launch_compat_shift(const PcgBuffers& b, cudaStream_t s);
void launch_make_codes(const PcgBuffers& b, cudaStream_t s);
void launch_ghost_fluid_diag(const PcgBuffers& b, const float* phi, float gfClamp, cudaStream_t s);
void launch_count_empty(const PcgBuffers& b, int* out, cudaStream_t s);
void launch_fix_pressure(const PcgBuffers& b, long long fix, cudaStream_t s);
void launch_pcg_init(const PcgBuffers& b, cudaStream_t s);
void launch_pcg_set_search(const PcgBuffers& b, cudaStream_t s);
void launch_pcg_spmv(const PcgBuffers& b, cudaStream_t s);
void launch_pcg_axpy(const PcgBuffers& b, cudaStream_t s);
void launch_pcg_copy_dot(const PcgBuffers& b, cudaStream_t s);   // PcNone: tmp = residual, sigmaNew
void launch_pcg_update(const PcgBuffers& b, cudaStream_t s);
void launch_mic(const PcgBuffers& b, const MicPlan& m, int mode, unsigned int epoch, long long spinLimit, cudaStream_t s);
// column-block MIC sweeps (mic.cu), for grids with nx % 8 == 0
struct MicColPlan {
  int nby, nbz, nblocks;
  int* order;                 // block dispatch order ((b + c) levels)
  unsigned long long* prog;   // per-block progress, epoch in the high word
  int* counter;
  int* error;
  int pubMask;                // progress published every pubMask+1 steps
};
bool mic_col_supported(const Dims& d);
void mic_col_geometry(const Dims& d, int* nby, int* nbz);
void mic_col_order(int nby, int nbz, int* order);
int mic_col_prepare();
void launch_mic_col(const PcgBuffers& b, const MicColPlan& m, int mode, unsigned int epoch, long long spinLimit,
                    int ctas, cudaStream_t s);
// warp-wavefront MIC sweeps (micwave.cu), for grids with nx % 8 == 0
struct MicWavePlan {
  int zw;                          // z-lines per lane: 4 or 8
  int nyb, nzb, nunits, rows;
  int* order;                      // unit dispatch order ((yb + zb) levels)
  int* counter;
  int* error;
  unsigned long long* exchange;    // face words, epoch-tagged (zeroed once)
};
bool mic_wave_supported(const Dims& d);
void mic_wave_geometry(const Dims& d, int zw, int* nyb, int* nzb, int* rows);
size_t mic_wave_exchange_words(const Dims& d, int zw);
void mic_wave_order(int nyb, int nzb, int* order);
int mic_wave_prepare(int* ctasPerSm4, int* ctasPerSm8);
void launch_mic_wave(const PcgBuffers& b, const MicWavePlan& m, int mode, unsigned int epoch, long long spinLimit,
                     int ctas, cudaStream_t s);
// one scene of a tile-dataflow MIC sweep: its grids, its 16^3 tile grid and
// its face words (mic_flow_face_words(tx*ty*tz) of them)
struct FlowScene {
  Dims d;
  const code_t* code;
  const float* A0f;
  float* P;
  const float* r;
  float* z;
  double* part;
  CgScalars* sc;
  int tx, ty, tz;
  unsigned long long* face;
};
// epochDev: a device word the launch advances before sweeping (so that a
// captured CUDA graph replays with new epochs)
void launch_mic_flow_batch(const FlowScene* scenes, const int2* order2, int ntiles, int ctas, int* counter, int* error,
                           int mode, unsigned int* epochDev, long long spinLimit, cudaStream_t s);
// resident CTAs of one MIC sweep launch on the device (after mic_flow_prepare)
int mic_flow_device_ctas();
// tile-dataflow MIC sweeps (micflow.cu): the tiles of a MicPlan, faces
// published as epoch-tagged words (face: mic_flow_face_words() words).
// stall: the sweep waits for an epoch no tile publishes, so its first wait
// runs out after spinLimit (the timeout path's test)
int mic_flow_prepare(int* ctasPerSm);
size_t mic_flow_face_words(int ntiles);
void launch_mic_flow(const PcgBuffers& b, const MicPlan& m, unsigned long long* face, int mode, unsigned int epoch,
                     long long spinLimit, cudaStream_t s, bool stall = false);
// once per device: the z-marching SpMV's resident CTAs and the streamed
// SpMV's shared-memory size (MANTAGPU_SPMV selects the kernel per launch)
int pcg_prepare(int sms);
// sum of nparts per-block dot partials -> beta/sigma (init: sigma only)
void launch_mic_finish(const PcgBuffers& b, int nparts, bool init, cudaStream_t s);

// precision form (refine.cu): FP64 residual refinement around the FP32 PCG
void launch_to_double(long long n, const float* a, double* b, cudaStream_t s);
void launch_to_float(long long n, const double* a, float* b, cudaStream_t s);
void launch_add_delta(long long n, double* p, const float* d, cudaStream_t s);
// r = b - A p (double), rf = (float) r, *norm = max|r|; counter starts at 0
void launch_residual64(const Dims& d, const code_t* code, const float* A0f, const double* b, const double* p, float* rf,
                       double* part, unsigned int* counter, double* norm, cudaStream_t s);

void launch_correct_velocity(const Dims& d, const int* flags, Mac vel, const float* p, const float* phi, const float* curv,
                             float gfClamp, float surfTens, cudaStream_t s);
void mic_plan_order(int tx, int ty, int tz, int* order);
int mic_ctas_per_sm();

}  // namespace mgpu
