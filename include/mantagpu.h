/*
 * mantagpu.h -- C ABI of libmantagpu, the GB300 implementation of mantaflow's
 * grid-step hot path.
 *
 * Every entry point replaces one mantaflow Python plugin or one member of the
 * classes those plugins take (paths relative to the mantaflow source tree).
 * A plugin translation unit of the reference (source/plugin/*.cpp) calls
 * these with the grids it receives, converting a non-zero status into the
 * reference's errMsg with mg_last_error()'s text.
 *
 * Conventions
 *  - Every function returns MG_OK (0) or an MG_ERR_* code; mg_last_error()
 *    returns the message of the calling thread's last failure.  Messages the
 *    reference raises as Manta::Error (source/general.h:42-58) are reproduced
 *    verbatim.
 *  - Grids live in device memory and are owned by the library.  Host buffers
 *    passed to mg_grid_upload / mg_grid_download use the reference layout
 *    (source/grid.h:70): x fastest, Real = float, Vec3/MAC = 3 floats per
 *    cell, flags = int32.
 *  - Calls on one solver are ordered on that solver's CUDA stream.  Plugin
 *    calls return once the work is queued unless they must report a value
 *    (mg_solve_pressure's iteration count, downloads, reductions).
 */
#ifndef MANTAGPU_H
#define MANTAGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MG_OK 0
#define MG_ERR_ARG 1
#define MG_ERR_CUDA 2
#define MG_ERR_UNSUPPORTED 3
#define MG_ERR_SOLVER 4      /* the reference's errMsg paths (divergence, asserts) */
#define MG_ERR_TIMEOUT 5     /* a bounded device-side wait gave up */
#define MG_ERR_NOMEM 6
#define MG_ERR_STATE 7       /* library not initialised / wrong device */

/* FlagGrid::CellType (source/grid.h:292-304) */
#define MG_FLAG_FLUID 1
#define MG_FLAG_OBSTACLE 2
#define MG_FLAG_EMPTY 4
#define MG_FLAG_INFLOW 8
#define MG_FLAG_OUTFLOW 16
#define MG_FLAG_OPEN 32
#define MG_FLAG_STICK 64

/* preconditioners (plugin/pressure.cpp:27) */
#define MG_PC_NONE 0
#define MG_PC_MIC 1
#define MG_PC_MG_DYNAMIC 2
#define MG_PC_MG_STATIC 3

/* grid kinds: Grid<Real>, Grid<int>, Grid<Vec3>, MACGrid, FlagGrid,
 * LevelsetGrid (source/grid.h:92-365, source/levelset.h:23) */
enum mg_grid_kind { MG_REAL = 0, MG_INT = 1, MG_VEC3 = 2, MG_MAC = 3, MG_FLAGS = 4, MG_LEVELSET = 5 };

typedef struct mg_solver_s* mg_solver; /* FluidSolver (source/fluidsolver.h) */
typedef struct mg_grid_s* mg_grid;     /* a grid bound to one solver */

/* ---- library ------------------------------------------------------------ */
int mg_init(int device);               /* select the CUDA device; idempotent */
int mg_shutdown(void);                 /* free every solver and grid */
const char* mg_last_error(void);
int mg_version(void);
int mg_device_count(int* out);

/* ---- FluidSolver (source/fluidsolver.cpp:107-158) ------------------------ */
/* FluidSolver(name, gridSize, dim): nz must be 1 for dim == 2 */
int mg_solver_create(int nx, int ny, int nz, int dim, mg_solver* out);
int mg_solver_destroy(mg_solver s);
/* FluidSolver::mDt, the `timestep` property; default 1.0 */
int mg_solver_set_dt(mg_solver s, float dt);
int mg_solver_get_dt(mg_solver s, float* dt);
/* wait for all queued work of the solver */
int mg_solver_sync(mg_solver s);
/* bytes of device memory held by the solver (grids, pool, solver state) */
int mg_solver_memory(mg_solver s, size_t* bytes);
/* No counterpart in the reference (its grids come from the host heap).  Caps
 * the device memory the solver may hold: a grid creation or temporary grid
 * that would take mg_solver_memory above `bytes` is refused with
 * MG_ERR_NOMEM and the reference's out-of-memory text, leaving the solver
 * usable.  0 (the default) removes the cap. */
int mg_solver_set_memory_limit(mg_solver s, size_t bytes);
/* No counterpart in the reference (its MIC(0) sweeps are serial loops).  The
 * device-side waits of the MIC(0) wavefront sweeps give up after
 * `limitNs` nanoseconds (default 200 ms; 0 restores it); the solve then
 * returns MG_ERR_TIMEOUT instead of hanging.  With stallNextSolve != 0 the
 * next MIC(0) solve's sweeps wait for tile words that no tile publishes, so
 * its first wait runs out: a failure-path test that leaves the GPU usable. */
int mg_solver_set_wait_limit(mg_solver s, long long limitNs, int stallNextSolve);

/* ---- grids (source/grid.cpp) --------------------------------------------- */
/* Grid<T>(parent): a zero-initialised grid (grid.cpp:48-58) */
int mg_grid_create(mg_solver s, int kind, mg_grid* out);
int mg_grid_destroy(mg_grid g);
/* host <-> device in the reference layout; bytes must equal the grid size */
int mg_grid_upload(mg_grid g, const void* host, size_t bytes);
int mg_grid_download(mg_grid g, void* host, size_t bytes);
/* Asynchronous forms of mg_grid_upload / mg_grid_download for pipelined
 * hosts (no counterpart in the reference, whose copies are synchronous).
 * They return at once; the host buffer (pinned: mg_host_alloc) must stay
 * untouched until mg_solver_wait_copies returns.  The transfer runs on the
 * solver's copy streams (uploads and downloads on separate ones) through a
 * device staging copy of the grid, ordered against the solver's kernels: an
 * upload lands before any kernel queued after it, a download takes the grid
 * as it is after the kernels queued before it, and the next step's upload
 * and kernels may run while it streams out. */
int mg_grid_upload_async(mg_grid g, const void* host, size_t bytes);
int mg_grid_download_async(mg_grid g, void* host, size_t bytes);
/* Block until every asynchronous transfer and kernel of the solver is done. */
int mg_solver_wait_copies(mg_solver s);
/* FluidSolver::getGridSize */
int mg_solver_size(mg_solver s, int* nx, int* ny, int* nz);
/* The grid's device storage (n floats / ints, or three planes of n floats for
 * Vec3/MAC) and its solver's CUDA stream (a cudaStream_t), for callers that
 * launch their own kernels on a grid.  Valid until the grid is destroyed or
 * swapped. */
int mg_grid_device(mg_grid g, void** data, void** stream);
/* Grid<T>::getSizeX/Y/Z and getType: the grid's dimensions and kind */
int mg_grid_get_info(mg_grid g, int* nx, int* ny, int* nz, int* kind);
/* Grid<T>::save (grid.cpp:135-156) for .uni (writeGridUni, fileio/iogrids.cpp:
 * 386-432), .raw (writeGridRaw, :255-271) and .npz (writeGridNumpy,
 * :836-884), written from the device mirror.  The gzip streams of .uni/.raw
 * hold stored (uncompressed) deflate blocks, which every gzip reader
 * accepts; .npz is an uncompressed zip of arr_0.npy, shape (nz, ny, nx, 1|3).
 * Other extensions: MG_ERR_UNSUPPORTED with the reference's message. */
int mg_grid_save(mg_grid g, const char* path);
/* Grid<T>::swap (grid.cpp:99-110): exchanges the storage of two grids */
int mg_grid_swap(mg_grid a, mg_grid b);
/* Grid<T>::copyFrom */
int mg_grid_copy(mg_grid dst, mg_grid src);
/* Grid<T>::setConst (Real/Int/Levelset use x; Vec3/MAC use x,y,z) */
int mg_grid_set_const(mg_grid g, float x, float y, float z);
/* Grid<Real>::join (grid.cpp:303-311), knJoinReal */
int mg_grid_join(mg_grid a, mg_grid b, int keepMax);
/* Grid<Real>::getMaxAbs (grid.cpp:319-323) */
int mg_grid_get_max_abs(mg_grid g, float* out);
/* page-locked host memory for fast uploads/downloads */
int mg_host_alloc(size_t bytes, void** out);
int mg_host_free(void* p);

/* ---- plugins: advection (plugin/advection.cpp) --------------------------- */
/* advectSemiLagrange (:442-460); dt from the solver */
int mg_advect_semi_lagrange(mg_grid flags, mg_grid vel, mg_grid grid, int order, float strength, int orderSpace,
                            int openBounds, int boundaryWidth, int clampMode, int orderTrace);
/* No counterpart in the reference.  Same arguments and results as
 * mg_advect_semi_lagrange, but allocates no device memory: its two
 * temporaries live in a fixed 24 MiB device array inside the library, for
 * callers that cannot allocate once running (a host whose own allocator holds
 * the rest of the GPU, a latency-bound loop that cannot afford a
 * cudaMalloc/cudaFree).  Limit: grids of up to 3,145,728 floats (a Real grid
 * of 3,145,728 cells, a Vec3/MAC grid of 1,048,576 cells); larger grids return
 * MG_ERR_ARG.  The result is written back into the grid's own storage.  The
 * first call on a device looks up the array's address, so make it before any
 * stream capture.  All calls share the array: calls that overlap on the GPU
 * (solvers on different streams) race. */
int mg_advect_semi_lagrange_noalloc(mg_grid flags, mg_grid vel, mg_grid grid, int order, float strength,
                                    int orderSpace, int openBounds, int boundaryWidth, int clampMode, int orderTrace);
/* resetPhiInObs (:401) */
int mg_reset_phi_in_obs(mg_grid flags, mg_grid sdf);

/* ---- plugins: forces and boundaries (plugin/extforces.cpp) --------------- */
/* setWallBcs (:307-315); obvel, fractions, phiObs may be NULL */
int mg_set_wall_bcs(mg_grid flags, mg_grid vel, mg_grid obvel, mg_grid fractions, mg_grid phiObs, int boundaryWidth);
/* addBuoyancy (:83-87) */
int mg_add_buoyancy(mg_grid flags, mg_grid density, mg_grid vel, float gx, float gy, float gz, float coefficient,
                    int scale);
/* addGravity (:61-65); exclude may be NULL */
int mg_add_gravity(mg_grid flags, mg_grid vel, float gx, float gy, float gz, mg_grid exclude, int scale);
/* addGravityNoScale (:67-69) */
int mg_add_gravity_no_scale(mg_grid flags, mg_grid vel, float gx, float gy, float gz, mg_grid exclude);
/* setOpenBound (:105-130); type defaults to Outflow|Empty in the reference */
int mg_set_open_bound(mg_grid flags, int bWidth, const char* openBound, int type);
/* resetOutflow (:133-160) without particles; phi, real may be NULL */
int mg_reset_outflow(mg_grid flags, mg_grid phi, mg_grid real);

/* ---- plugins: simple extrapolation (fastmarch.cpp) ----------------------- */
/* extrapolateMACSimple (:337-375); phiObs (a levelset, may be NULL) adds
 * knUnprojectNormalComp (:316-330) */
int mg_extrapolate_mac_simple(mg_grid flags, mg_grid vel, int distance, mg_grid phiObs, int intoObs);
/* extrapolateLsSimple (fastmarch.cpp:470-507): phi is a Real or Levelset grid */
int mg_extrapolate_ls_simple(mg_grid phi, int distance, int inside);

/* ---- wavelet noise and the density source (noisefield.h, noisefield.cpp,
 * plugin/initplugins.cpp) ---------------------------------------------------- */
typedef struct mg_noise_s* mg_noise; /* WaveletNoiseField, Python name NoiseField */
/* the NoiseField properties posOffset, posScale, valOffset, valScale, clamp,
 * clampNeg, clampPos, timeAnim (noisefield.h:52-63) */
typedef struct {
  float posOffset[3], posScale[3];
  float valOffset, valScale;
  int clamp;
  float clampNeg, clampPos;
  float timeAnim;
} mg_noise_params;
void mg_noise_params_default(mg_noise_params* p);
/* WaveletNoiseField(parent, fixedSeed=-1) (noisefield.cpp:61-78): the shared
 * 3 x 128^3 noise tile is generated on the host (generateTile, :94-190) on
 * first use and kept in device memory until mg_shutdown */
int mg_noise_create(mg_solver s, int fixedSeed, mg_noise* out);
int mg_noise_destroy(mg_noise n);
int mg_noise_set_params(mg_noise n, const mg_noise_params* p);
/* mSeedOffset, the normalized random offset into the tile */
int mg_noise_seed_offset(mg_noise n, float* out3);
/* out(i,j,k) = evaluate(Vec3(i,j,k)) (noisefield.h:332-357) at the solver time
 * solverTime (FluidSolver::getTime, for timeAnim) */
int mg_noise_evaluate_grid(mg_noise n, mg_grid out, float solverTime);
/* densityInflow(flags, density, noise, shape, scale, sigma) (initplugins.cpp:
 * 38-43) with sdf = shape->computeLevelset() computed by the caller */
int mg_density_inflow(mg_grid flags, mg_grid density, mg_noise noise, mg_grid sdf, float scale, float sigma,
                      float solverTime);
/* Cylinder::computeLevelset (CylinderSDF, shapes.cpp:367-388) */
int mg_shape_cylinder_levelset(mg_grid phi, const float* center, float radius, const float* z);

/* ---- particles and the FLIP transfers (source/particle.h,
 * source/plugin/flip.cpp) ----------------------------------------------------- */
/* BasicParticleSystem (particle.h:193-230) of one solver, holding up to
 * `capacity` particles in device memory; ParticleDataImpl<Real|Vec3|int>
 * (particle.h:306) per-particle data of one particle system.  Destroying a
 * particle system destroys its data; destroying the solver destroys both. */
typedef struct mg_particles_s* mg_particles;
typedef struct mg_pdata_s* mg_pdata;
/* ParticleBase::PDELETE (particle.h:41): a deleted particle, skipped */
#define MG_PARTICLE_DELETED 1024
int mg_particles_create(mg_solver s, long long capacity, mg_particles* out);
int mg_particles_destroy(mg_particles p);
/* `count` records in the layout of BasicParticleData (particle.h:182-191):
 * float pos[3], int flag -- 16 bytes each.  Upload sets the particle count
 * (at most the capacity); download takes exactly the particle count. */
int mg_particles_upload(mg_particles p, const void* host, long long count);
int mg_particles_download(mg_particles p, void* host, long long count);
int mg_particles_size(mg_particles p, long long* count);
/* kind MG_REAL (float), MG_VEC3 (3 floats per particle) or MG_INT (int32);
 * transfers take exactly the particle count; created zeroed */
int mg_pdata_create(mg_particles p, int kind, mg_pdata* out);
int mg_pdata_destroy(mg_pdata d);
int mg_pdata_upload(mg_pdata d, const void* host, long long count);
int mg_pdata_download(mg_pdata d, void* host, long long count);
/* mapPartsToMAC (flip.cpp:573-595): vel = the particle velocities splatted
 * with their trilinear MAC weights, divided by the summed weights; velOld =
 * vel; weight (a Vec3 grid, may be NULL) receives the summed weights.
 * ptype (an MG_INT particle data, may be NULL) and exclude skip particles
 * whose type has an excluded bit.  Results equal the reference's
 * particle-order sums bit for bit.  In 2D the particles of the slab
 * 0 <= z < 1 match the reference; others are taken to lie in the slab (the
 * reference indexes outside the grid for them), here and in the transfers
 * below. */
int mg_map_parts_to_mac(mg_grid flags, mg_grid vel, mg_grid velOld, mg_particles parts, mg_pdata partVel,
                        mg_grid weight, mg_pdata ptype, int exclude);
/* mapMACToParts (flip.cpp:651-655): partVel = vel interpolated (PIC) */
int mg_map_mac_to_parts(mg_grid flags, mg_grid vel, mg_particles parts, mg_pdata partVel, mg_pdata ptype,
                        int exclude);
/* flipVelocityUpdate (flip.cpp:669-673): partVel = flipRatio * (partVel +
 * vel(p) - velOld(p)) + (1 - flipRatio) * vel(p) */
int mg_flip_velocity_update(mg_grid flags, mg_grid vel, mg_grid velOld, mg_particles parts, mg_pdata partVel,
                            float flipRatio, mg_pdata ptype, int exclude);
/* mapPartsToGrid / mapPartsToGridVec3 (flip.cpp:599-622): target is a Real
 * grid with MG_REAL data or a Vec3 grid with MG_VEC3 data */
int mg_map_parts_to_grid(mg_grid flags, mg_grid target, mg_particles parts, mg_pdata source);
/* mapGridToParts / mapGridToPartsVec3 (flip.cpp:625-638) */
int mg_map_grid_to_parts(mg_grid source, mg_particles parts, mg_pdata target);

/* ---- plugins: pressure (plugin/pressure.cpp) ----------------------------- */
typedef struct {
  float cgAccuracy;          /* 1e-3 */
  float gfClamp;             /* 1e-4 */
  float cgMaxIterFac;        /* 1.5 */
  int precondition;          /* 1 (deprecated switch: 0 forces PcNone) */
  int preconditioner;        /* MG_PC_MIC */
  int enforceCompatibility;  /* 0 */
  int useL2Norm;             /* 0 */
  int zeroPressureFixing;    /* 0 */
  float surfTens;            /* 0 */
} mg_pressure_params;

typedef struct {
  int iterations;            /* GridCg::getIterations */
  float resNorm;             /* GridCg::getResNorm */
} mg_pressure_result;

void mg_pressure_params_default(mg_pressure_params* p);
/* solvePressure (:480-521).  phi, perCellCorr, fractions, obvel, curv,
 * retRhs may be NULL; out may be NULL.  With fractions (a MACGrid of face
 * fractions, MakeLaplaceMatrix's float form) the matrix is stored as floats,
 * MIC(0) runs plane by plane, the multigrid preconditioners take the stored
 * off-diagonals into their level 0, and pressure fixing zeroes the fixed
 * cell's stored entries like fixPressure (:226-245). */
int mg_solve_pressure(mg_grid vel, mg_grid pressure, mg_grid flags, const mg_pressure_params* p, mg_grid phi,
                      mg_grid perCellCorr, mg_grid fractions, mg_grid obvel, mg_grid curv, mg_grid retRhs,
                      mg_pressure_result* out);
/* computePressureRhs (:277-299) */
int mg_compute_pressure_rhs(mg_grid rhs, mg_grid vel, mg_grid pressure, mg_grid flags, const mg_pressure_params* p,
                            mg_grid phi, mg_grid perCellCorr, mg_grid fractions, mg_grid obvel, mg_grid curv);
/* solvePressureSystem (:312-452); rhs is modified when pressure is pinned */
int mg_solve_pressure_system(mg_grid rhs, mg_grid vel, mg_grid pressure, mg_grid flags, const mg_pressure_params* p,
                             mg_grid phi, mg_grid perCellCorr, mg_grid fractions, mg_grid curv,
                             mg_pressure_result* out);
/* correctVelocity (:455-476) */
int mg_correct_velocity(mg_grid vel, mg_grid pressure, mg_grid flags, const mg_pressure_params* p, mg_grid phi,
                        mg_grid perCellCorr, mg_grid fractions, mg_grid curv);
/* Precision form of solvePressure (no counterpart in the reference; its
 * FP64 build, -DDOUBLEPRECISION=ON, is what it reproduces).  The stencils
 * and the inner PCG run in FP32; the pressure is accumulated in double and
 * after every inner solve the residual max|b - A p| is recomputed in double:
 * FP32 PCG solves of A delta = r repeat until it is below refineAccuracy,
 * each inner solve to cgAccuracy = innerAccuracy * max|r| (the first one at
 * the caller's cgAccuracy).  maxRefine bounds the inner solves. */
typedef struct {
  double refineAccuracy;     /* 1e-5 */
  double innerAccuracy;      /* 1e-2 */
  int maxRefine;             /* 10 */
} mg_refine_params;
typedef struct {
  int refinements;           /* inner solves */
  int iterations;            /* CG iterations over all inner solves */
  double resNorm;            /* final max|b - A p| in double */
} mg_refine_result;
void mg_refine_params_default(mg_refine_params* r);
int mg_solve_pressure_refined(mg_grid vel, mg_grid pressure, mg_grid flags, const mg_pressure_params* p, mg_grid phi,
                              const mg_refine_params* rp, mg_refine_result* out);
/* releaseMG (:252-266); s == NULL releases every solver's hierarchy */
int mg_release_mg(mg_solver s);
/* One multigrid V-cycle dst = M^-1 src for the Poisson matrix of flags (with
 * the ghost-fluid diagonal when phi is given): GridMg::setA, setRhs and
 * doVCycle (source/multigrid.cpp:386-504) on a fresh hierarchy, as
 * InitPreconditionMultigrid / ApplyPreconditionMultigrid do
 * (conjugategrad.cpp:100-106, 162-167).  A diagnostic entry for checking
 * the preconditioner on its own; solvePressure does not need it. */
int mg_multigrid_vcycle(mg_grid flags, mg_grid phi, mg_grid src, mg_grid dst, float gfClamp, float coarseAccuracy);
/* How the multigrid hierarchy for flags is laid out and run: level sizes
 * (GridMg ctor, multigrid.cpp:240-265), the first level of the coarse end
 * that runs as one cluster launch, and per level the number of distinct
 * stencils when the level reads a stencil dictionary (0: stencil planes).
 * Builds a fresh hierarchy like mg_multigrid_vcycle; diagnostic only. */
typedef struct mg_multigrid_layout {
  int levels;
  int tailFirst;
  int tailCtas;
  int size[32][3];
  int dictStencils[32];
} mg_multigrid_layout;
int mg_multigrid_describe(mg_grid flags, mg_multigrid_layout* out);

/* ---- scene setup (source/grid.cpp, source/shapes.cpp) -------------------- */
/* FlagGrid::initDomain (grid.cpp:732-822); phiWalls must be NULL */
int mg_flags_init_domain(mg_grid flags, int boundaryWidth, const char* wall, const char* open, const char* inflow,
                         const char* outflow, mg_grid phiWalls);
/* FlagGrid::fillGrid (grid.cpp:856-861) */
int mg_flags_fill_grid(mg_grid flags, int type);
/* FlagGrid::updateFromLevelset (grid.cpp:844-854) */
int mg_flags_update_from_levelset(mg_grid flags, mg_grid levelset);
/* Shape::applyToGrid for Box (shapes.cpp:38-86, 151-154); value[3] for
 * Vec3/MAC, value[0] for Real, ivalue for Int/Flags; respectFlags may be NULL */
int mg_shape_box_apply(mg_grid grid, const float* p0, const float* p1, const float* value, int ivalue,
                       mg_grid respectFlags);
/* Shape::applyToGrid for Cylinder(center, radius, z) (shapes.cpp:316-329) */
int mg_shape_cylinder_apply(mg_grid grid, const float* center, float radius, const float* z, const float* value,
                            int ivalue, mg_grid respectFlags);
/* Box::computeLevelset (BoxSDF, shapes.cpp:178-232) into a Real/Levelset grid */
int mg_shape_box_levelset(mg_grid phi, const float* p0, const float* p1);

/* ---- batched form (no counterpart in the reference) ---------------------- */
/* Many independent plume scenes (the reference's smoke plume: walls, open
 * top, cylinder source with seeded uniform inflow noise, buoyancy, MacCormack
 * advection, setWallBcs, addBuoyancy, solvePressure) stepped together: every
 * stage is one launch over all scenes' tiles, and the pressure solve iterates
 * until every scene has converged, each with its own CG scalars.  The
 * pressure solve is the reference's GridCg with PcMIC: MIC(0) for 3D scenes
 * with (int)(cgMaxIterFac * max size) iterations at most, no preconditioner
 * for 2D scenes with 4 times as many (conjugategrad.cpp:315-321,
 * pressure.cpp:407-419).  Once the CG tile height is tuned, the sweeps run
 * as CUDA graphs of 8 sweeps between convergence polls. */
typedef struct mg_batch_s* mg_batch;
typedef struct {
  int sweeps;                  /* CG iterations launched (the slowest scene's count) */
  int maxIterations;           /* largest per-scene iteration count */
  long long totalIterations;   /* sum over scenes */
  int diverged;                /* scenes whose residual exceeded 1e35 */
  long long graphLaunches;     /* CUDA graph launches of CG sweeps in this step */
} mg_batch_stats;
#define MG_BATCH_DENSITY 0
#define MG_BATCH_VELOCITY 1    /* AoS Vec3, 3 floats per cell */
#define MG_BATCH_PRESSURE 2
#define MG_BATCH_FLAGS 3
#define MG_BATCH_SOURCE 4      /* the inflow cylinder mask */
/* sizes: count*3 ints (nx, ny, nz; nz = 1 for 2D); gravity: count*3 floats
 * (addBuoyancy's gravity, scaled by dt/dx); seeds: per-scene inflow noise */
int mg_batch_create(int count, const int* sizes, const float* gravity, const unsigned long long* seeds, float dt,
                    mg_batch* out);
int mg_batch_destroy(mg_batch b);
/* solvePressure's cgAccuracy (1e-3) and cgMaxIterFac (1.5) */
int mg_batch_set_solver(mg_batch b, float cgAccuracy, float cgMaxIterFac);
/* MG_PC_MIC (the default): 3D scenes precondition with MIC(0), whose
 * dataflow sweeps run over the tiles of all 3D scenes in one launch; 2D
 * scenes run GridCg without a preconditioner, as the reference does in 2D.
 * MG_PC_NONE: no scene is preconditioned. */
int mg_batch_set_preconditioner(mg_batch b, int preconditioner);
/* The precision form for a batch (mg_solve_pressure_refined per scene):
 * after the FP32 solve each scene's pressure is accumulated in double, its
 * residual max|b - A p| formed in double, and FP32 solves of A delta = r to
 * innerAccuracy * max|r| repeat until it is below refineAccuracy (maxRefine
 * rounds at most).  refineAccuracy 0 switches the refinement off (the
 * default).  Each scene holds 16 more bytes per cell while it refines. */
int mg_batch_set_refinement(mg_batch b, double refineAccuracy, double innerAccuracy, int maxRefine);
/* one plume step of every scene; stats may be NULL */
int mg_batch_step(mg_batch b, mg_batch_stats* stats);
int mg_batch_scene_iterations(mg_batch b, int scene, int* iterations, float* resNorm);
/* a field of one scene in the reference layout; bytes must match */
int mg_batch_download(mg_batch b, int scene, int what, void* host, size_t bytes);
/* the uniform [0,1) inflow noise a scene with this seed uses at a step, per
 * cell (host computation, for feeding the same inflow to a single scene) */
int mg_batch_noise(unsigned long long seed, int step, long long cells, float* out);
int mg_batch_info(mg_batch b, int* count, long long* cells, long long* tiles, size_t* bytes);
/* the CG sweep tile height the batch's autotuner chose on its first solve
 * (0 before) and the four timings (ms per lag sweeps, 8/16/32/64 rows) */
int mg_batch_tuning(mg_batch b, int* sweepRows, float* ms);
int mg_batch_sync(mg_batch b);

/* ---- served form (no counterpart in the reference) ----------------------- */
/* A request loop for plume jobs (the batched form's scene, run for a number
 * of steps): jobs arrive at given times and are admitted in arrival order
 * once arrived and once their device memory (mg_serve_job_bytes) fits the
 * budget; every tick advances all resident jobs by one step in one batched
 * step; a finished job leaves and frees its memory for the next.  A job's
 * results depend only on its own scene: the same alone and in any mix. */
typedef struct mg_server_s* mg_server;
typedef struct {
  int jobs;
  long long ticks;
  double wallSeconds;        /* from the start of mg_serve_run to the last job's end */
  long long cellSteps;       /* sum over jobs of cells x steps */
  size_t peakBytes;          /* largest device memory held by resident jobs */
} mg_serve_stats;
typedef struct {
  double arrival, admitted, finished;  /* seconds after the start of the run */
  int steps;
  double meanStepMs;         /* mean tick duration over the job's steps */
} mg_serve_job;
int mg_serve_create(size_t budgetBytes, float dt, mg_server* out);
int mg_serve_destroy(mg_server s);
int mg_serve_set_solver(mg_server s, float cgAccuracy, float cgMaxIterFac);
size_t mg_serve_job_bytes(int nx, int ny, int nz);
/* a job of `steps` plume steps on an nx x ny x nz grid (nz = 1: 2D) arriving
 * `arrival` seconds after mg_serve_run starts; keepResult copies its final
 * density, velocity and pressure to the host when it finishes */
int mg_serve_submit(mg_server s, int nx, int ny, int nz, const float* gravity, unsigned long long seed, int steps,
                    double arrival, int keepResult, int* job);
/* mg_serve_submit for a job of a given kind: 0 the smoke plume, 1 the dam
 * break of the free-surface liquid scene (initDomain closed box, phi of the
 * box x < 0.4 nx, y < 0.6 ny; per step extrapolateMACSimple(vel, 4), advect
 * phi and vel (SL order 1), updateFromLevelset, addGravity, setWallBcs,
 * ghost-fluid solvePressure(phi), setWallBcs).  A dam-break job's "density"
 * result is its levelset phi; 3D jobs of both kinds precondition with MIC(0). */
int mg_serve_submit_kind(mg_server s, int kind, int nx, int ny, int nz, const float* gravity, unsigned long long seed,
                         int steps, double arrival, int keepResult, int* job);
/* device bytes a job of that kind and size holds while resident */
size_t mg_serve_job_bytes_kind(int kind, int nx, int ny, int nz);
/* run until every submitted job has finished */
int mg_serve_run(mg_server s, mg_serve_stats* stats);
int mg_serve_job_info(mg_server s, int job, mg_serve_job* info);
int mg_serve_job_result(mg_server s, int job, int what, void* host, size_t bytes);
/* tick durations and resident job counts (count: in capacity, out total) */
int mg_serve_ticks(mg_server s, int* count, float* ms, int* jobs);

/* ---- timing (CUDA events on the solver's stream) ------------------------- */
/* per-kernel-family device time accumulated while profiling is on */
int mg_profile_enable(mg_solver s, int on);
/* name[i] / milliseconds[i] / launches[i] for i < *count (in, capacity; out, used) */
int mg_profile_read(mg_solver s, int* count, const char** names, double* ms, long long* launches);
int mg_profile_reset(mg_solver s);
/* device time between two marks on the solver's stream, in ms */
int mg_mark(mg_solver s, int slot);
int mg_elapsed(mg_solver s, int slot0, int slot1, float* ms);
/* kernels launched by this library since load (all solvers) */
int mg_launch_count(long long* out);

#ifdef __cplusplus
}
#endif
#endif
