// Batched form: many independent scenes of uneven sizes stepped together.
//
// Every stage is one kernel launch over a flat list of tiles spanning all
// scenes.  A tile is a 32 x 8 block of cells in one z-plane of one scene
// (one CTA); the CTA reads its scene's sizes and buffers from the scene
// table and runs exactly the per-cell code of the single-scene kernel.  The
// pressure solve keeps one CgScalars per scene: each tile leaves its partial
// dot products / norms in a slot of its own, and the last tile of a scene
// to finish (a per-scene ticket) reduces that scene's slots in tile order,
// so per-scene results do not depend on how tiles are scheduled.
#pragma once
#include <string>

#include "../../include/mantagpu.h"
#include "mg_kernels.h"

namespace mgpu {

constexpr int kBTX = 32, kBTY = 8;  // tile = CTA shape

// runtime.cu: the calling thread's error text, and whether mg_init ran
int set_error(int code, const std::string& msg);
bool library_ready();
// Cylinder's axis: the unit direction and the length of the z vector
void cylinder_axis(const float* z, float* zn, float* mZ);
// noise.cu: frees the device noise tile (mg_shutdown)
void noise_release();
// particles.cu: frees the particle systems of a solver (all of them for
// nullptr) and their particle data, whose handles become invalid
void particles_release(mg_solver s);
// runtime.cu: a solver's dimensions and stream (MG_ERR_ARG for a bad handle)
int solver_info(mg_solver s, Dims* d, cudaStream_t* st);

struct BTile {
  int scene;
  int x0, y0, z;
  int local;  // index of the tile within its scene (32 x 8 tiles)
  int count;  // tiles of this scene in the list the tile belongs to
};

// one scene of a batch (device pointers; MAC grids are 3 planes of n floats)
struct BScene {
  Dims d;
  int* flags;
  float* vel[2];   // ping-pong velocity (MAC)
  float* dens[2];  // ping-pong density
  float* fwd;      // 3 planes: forward SL values, then outflow scratch
  float* mask;     // inflow source (Shape::applyToGrid value 1)
  float* pres;
  float* rhs;
  float* res;
  float* search;
  float* tmp;
  code_t* code;
  CgScalars* sc;
  double* part;    // per-tile partials (ntiles doubles, 2 per tile for max-abs)
  // MIC(0) preconditioning (3D scenes, the reference's PcMIC): the
  // diagonal P and the 16^3 tile grid of the dataflow sweeps with its face
  // words; mic 0 runs GridCg without a preconditioner (the reference's 2D
  // path)
  float* P;
  unsigned long long* face;
  int mic, tx, ty, tz;
  // kind 0: smoke plume.  kind 1: dam break (free-surface liquid; dens[]
  // holds the levelset phi, A0f the ghost-fluid diagonal, itmp the marks of
  // the MAC extrapolation)
  int kind;
  float* A0f;
  int* itmp;
  // FP64 refinement (when the batch refines): the pressure accumulated in
  // double and the double right-hand side
  double* p64;
  double* b64;
  float dt;
  float bx, by, bz;  // plume: buoyancy factors -gravity*dt/dx (KnAddBuoyancy), 0.5 applied in-kernel;
                     // dam break: the gravity force gravity*dt/dx (KnApplyForce)
  unsigned long long seed;
  int step;        // steps this scene has taken: the inflow noise index
  int ntiles;
};

__host__ __device__ inline Mac bmac(float* p, long long n) { return Mac{p, p + n, p + 2 * n}; }
__host__ __device__ inline CMac bcmac(const float* p, long long n) { return CMac{p, p + n, p + 2 * n}; }

// stages (cur: index of the current vel/dens buffers; results go to 1-cur)
void launch_b_inflow(const BTile* t, int nt, const BScene* s, int cur, cudaStream_t st);
void launch_b_advect_density(const BTile* t, int nt, const BScene* s, int cur, cudaStream_t st);
void launch_b_advect_velocity(const BTile* t, int nt, const BScene* s, int cur, cudaStream_t st);
void launch_b_forces(const BTile* t, int nt, const BScene* s, int nxt, cudaStream_t st);
// MakeRhs + codes and the dam scenes' ghost-fluid diagonal (their own tile
// list)
void launch_b_pressure_setup(const BTile* t, int nt, const BScene* s, int nxt, cudaStream_t st, const BTile* tDam,
                             int ntDam);
// GridCg::doInit without a preconditioner: x = 0, r = rhs, z = s = r, sigma
// (MIC scenes then apply theirs: launch_b_mic_init)
void launch_b_pcg_init(const BTile* t, int nt, const BScene* s, cudaStream_t st);
// FP64 refinement: b64 = rhs, p64 = pres; r = b64 - A p64 in double into rhs
// (as float) with max|r| into the scene's refNorm; p64 += pres; pres = p64
void launch_b_ref_first(const BTile* t, int nt, const BScene* s, cudaStream_t st);
void launch_b_ref_residual(const BTile* t, int nt, const BScene* s, cudaStream_t st);
void launch_b_ref_add(const BTile* t, int nt, const BScene* s, cudaStream_t st);
void launch_b_ref_finish(const BTile* t, int nt, const BScene* s, cudaStream_t st);
// the MIC(0) sweeps of a batch: the FlowScene table of its MIC scenes, the
// (scene, tile) dispatch order, and the BScene index of each MIC scene
struct BatchMic {
  const FlowScene* flow;
  const int2* order;
  int ntiles, nscenes, ctas;
  const int* sceneOf;  // [nscenes]: index into the BScene table
  int* counter;
  int* error;
  unsigned int* epochDev;  // device word, advanced on the device before each sweep
  long long spinLimit;
};
// doInit's preconditioner application for the MIC scenes: P, z = M^-1 r,
// sigma = dot(z, r), search = z
void launch_b_mic_init(const BTile* t, int nt, const BScene* s, const BatchMic& m, cudaStream_t st);
// one CG sweep over tiles 32 x 8*rows cells tall (rows 1, 2, 4 or 8); with
// mic, the MIC scenes apply their preconditioner between the residual
// update and the search-vector update
void launch_b_pcg_iteration(const BTile* t, int nt, const BScene* s, int rows, int* ndone, const BatchMic* mic,
                            cudaStream_t st);
void launch_b_correct(const BTile* t, int nt, const BScene* s, int nxt, cudaStream_t st);
// dam-break scenes (over their own tiles): extrapolateMACSimple(vel, 4),
// advect phi and velocity (SL order 1), updateFromLevelset; after the
// solve's velocity update, the ghost-fluid corrections and setWallBcs
void launch_b_dam_advect(const BTile* t, int nt, const BScene* s, int cur, cudaStream_t st);
void launch_b_dam_gf_diag(const BTile* t, int nt, const BScene* s, int nxt, cudaStream_t st);
void launch_b_dam_correct(const BTile* t, int nt, const BScene* s, int nxt, cudaStream_t st);
// uniform [0,1) inflow noise of a scene's cell at a step (the batch's
// per-scene seeded source); also used to fill single-scene grids for
// comparisons
__host__ __device__ inline float batch_noise(unsigned long long seed, int step, long long cell) {
  // splitmix64 of (seed, step, cell): a counter-based generator
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * ((unsigned long long)step * 0x100000001B3ull + (unsigned long long)cell + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  return (float)(z >> 40) * (1.0f / 16777216.0f);  // 24 random bits
}

}  // namespace mgpu
