/*
 * manta_oracle.h -- CPU restatement of mantaflow's grid-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity oracle for the GPU
 * implementation in mantaflow_gb300/.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline / reference legs load it; the product never
 * links or calls it.
 *
 * Parity status: pinned.  tests/golden/ holds outputs of the reference's own
 * float executable (single OpenMP thread, so every reduction is serial) on
 * seeded inputs, and tests/test_oracle_golden.py checks this oracle against
 * them bit for bit (CG/MG paths included).
 *
 * Precision: Real is the og_real typedef, float by default -- the reference's float
 * build, which the goldens pin.  Compiled with -DOG_REAL=double the same
 * source restates the reference's double build (-DDOUBLEPRECISION=ON:
 * Real = double, VECTOR_EPSILON = 1e-10, util/vectorbase.h:40-56); that
 * variant is the FP64 oracle of the precision tests and has no goldens of
 * its own.
 *
 * Layout is the reference's (source/grid.h:70): x fastest, index
 * i + nx*j + strideZ*k with strideZ = 0 in 2D.  Real = og_real.  Vec3 and MAC
 * grids are array-of-structs, 3 floats per cell (util/vectorbase.h:199-205).
 * Flags are int32 bit sets (source/grid.h:292-304).
 *
 * Arithmetic follows the reference expression by expression: where the
 * reference mixes a double literal into a Real expression the restatement
 * computes that sub-expression in double and rounds once, as the C++ does.
 * Build with -ffp-contract=off (no FMA contraction), never -ffast-math.
 */
#ifndef MANTA_ORACLE_H
#define MANTA_ORACLE_H

#ifndef OG_REAL
#define OG_REAL float
#endif
typedef OG_REAL og_real;

#ifdef __cplusplus
extern "C" {
#endif

enum {
  OG_FLUID = 1, OG_OBSTACLE = 2, OG_EMPTY = 4, OG_INFLOW = 8,
  OG_OUTFLOW = 16, OG_OPEN = 32, OG_STICK = 64
};

/* grid kinds for og_advect_semi_lagrange (source/grid.h:55-62 GridType) */
enum { OG_KIND_REAL = 0, OG_KIND_VEC3 = 1, OG_KIND_MAC = 2 };

/* preconditioners (plugin/pressure.cpp:27) */
enum { OG_PC_NONE = 0, OG_PC_MIC = 1, OG_PC_MG_DYNAMIC = 2, OG_PC_MG_STATIC = 3 };

typedef struct {
  int nx, ny, nz;   /* grid size; nz == 1 for 2D */
  int is3d;
} og_dims;

/* advectSemiLagrange (plugin/advection.cpp:442-460).  grid is updated in
 * place.  dt is FluidSolver::getDt(). */
int og_advect_semi_lagrange(og_dims d, const int* flags, const og_real* vel,
                            int kind, og_real* grid, int order, og_real strength,
                            int orderSpace, int clampMode, int orderTrace, og_real dt);

/* setWallBcs without fractions (plugin/extforces.cpp:186-217, 307-315). */
void og_set_wall_bcs(og_dims d, const int* flags, og_real* vel, const og_real* obvel);

/* addBuoyancy (plugin/extforces.cpp:72-87). */
void og_add_buoyancy(og_dims d, const int* flags, const og_real* density, og_real* vel,
                     og_real gx, og_real gy, og_real gz, og_real coefficient, int scale, og_real dt);

/* addGravity (plugin/extforces.cpp:46-65). exclude may be NULL. */
void og_add_gravity(og_dims d, const int* flags, og_real* vel, og_real gx, og_real gy, og_real gz,
                    const og_real* exclude, int scale, og_real dt);

/* extrapolateMACSimple (fastmarch.cpp:337-375); phiObs may be NULL */
void og_extrapolate_mac_simple(og_dims d, const int* flags, og_real* vel, int distance, const og_real* phiObs,
                               int intoObs);
void og_extrapolate_ls_simple(og_dims d, og_real* phi, int distance, int inside);

typedef struct {
  og_real cgAccuracy;        /* 1e-3 */
  og_real gfClamp;           /* 1e-4 */
  og_real cgMaxIterFac;      /* 1.5 */
  int preconditioner;      /* OG_PC_* */
  int enforceCompatibility;
  int useL2Norm;
  int zeroPressureFixing;
  og_real surfTens;          /* used only with phi and curv */
} og_pressure_params;

typedef struct {
  int iterations;
  og_real resNorm;
  int fixPidx;             /* pinned cell or -1 */
} og_pressure_result;

/* opaque multigrid hierarchy (multigrid.h:31-137); one per solver for the
 * static mode, like gMapMG in plugin/pressure.cpp:250 */
typedef struct og_mg og_mg;
og_mg* og_mg_create(og_dims d);
void og_mg_destroy(og_mg* mg);

/* computePressureRhs (plugin/pressure.cpp:277-299). */
void og_compute_pressure_rhs(og_dims d, og_real* rhs, const og_real* vel, const int* flags,
                             const og_real* phi, const og_real* perCellCorr, const og_real* curv,
                             const og_pressure_params* p);

/* solvePressureSystem (plugin/pressure.cpp:312-452).  rhs is modified when
 * pressure is pinned (fixPressure).  mg_cache: pointer to the solver's MG
 * slot (may hold NULL); used only by the MG preconditioners. */
int og_solve_pressure_system(og_dims d, og_real* rhs, og_real* pressure, const int* flags,
                             const og_real* phi, const og_pressure_params* p,
                             og_mg** mg_cache, og_pressure_result* out);

/* correctVelocity (plugin/pressure.cpp:455-476). */
void og_correct_velocity(og_dims d, og_real* vel, const og_real* pressure, const int* flags,
                         const og_real* phi, const og_real* curv, const og_pressure_params* p);

/* solvePressure (plugin/pressure.cpp:480-521): rhs, system, correction.
 * retRhs may be NULL. */
int og_solve_pressure(og_dims d, og_real* vel, og_real* pressure, const int* flags,
                      const og_real* phi, const og_real* perCellCorr, const og_real* curv,
                      const og_pressure_params* p, og_mg** mg_cache,
                      og_pressure_result* out, og_real* retRhs);

/* Building blocks exposed for kernel-level parity tests. */
void og_make_laplace_matrix(og_dims d, const int* flags, og_real* A0, og_real* Ai, og_real* Aj, og_real* Ak);
void og_apply_ghost_fluid_diagonal(og_dims d, og_real* A0, const int* flags, const og_real* phi, og_real gfClamp);
void og_mic_init(og_dims d, const int* flags, og_real* Aprecond, const og_real* A0,
                 const og_real* Ai, const og_real* Aj, const og_real* Ak);
void og_mic_apply(og_dims d, og_real* dst, const og_real* src, const int* flags, const og_real* Aprecond,
                  const og_real* Ai, const og_real* Aj, const og_real* Ak);
void og_apply_matrix(og_dims d, const int* flags, og_real* dst, const og_real* src, const og_real* A0,
                     const og_real* Ai, const og_real* Aj, const og_real* Ak);
/* one MG V-cycle from zero: setA (if not set) + setRhs + doVCycle */
void og_mg_vcycle(og_mg* mg, const og_real* A0, const og_real* Ai, const og_real* Aj, const og_real* Ak,
                  og_real* dst, const og_real* rhs, og_real coarseAccuracy);
/* number of levels / coarse vertex types for hierarchy parity tests */
int og_mg_num_levels(const og_mg* mg);
void og_mg_level_size(const og_mg* mg, int l, int* sz);
const signed char* og_mg_level_types(const og_mg* mg, int l);
const og_real* og_mg_level_matrix(const og_mg* mg, int l);

/* Scene setup (source/grid.cpp:732-861, plugin/extforces.cpp:105-160,
 * shapes.cpp:151-154, 178-228, 324-329). */
void og_init_domain(og_dims d, int* flags, int boundaryWidth, const char* wall,
                    const char* open, const char* inflow, const char* outflow);
void og_fill_grid(og_dims d, int* flags, int type);
void og_set_open_bound(og_dims d, int* flags, int bWidth, const char* openBound, int type);
void og_update_from_levelset(og_dims d, int* flags, const og_real* phi);
void og_box_sdf(og_dims d, og_real* phi, og_real p0x, og_real p0y, og_real p0z, og_real p1x, og_real p1y, og_real p1z);
/* Cylinder::isInside applied to cell centres (shape.applyToGrid), Real grid */
void og_cylinder_apply(og_dims d, og_real* grid, og_real cx, og_real cy, og_real cz, og_real radius,
                       og_real zx, og_real zy, og_real zz, og_real value, const int* respectFlags);
void og_box_apply(og_dims d, og_real* grid, og_real p0x, og_real p0y, og_real p0z,
                  og_real p1x, og_real p1y, og_real p1z, og_real value, const int* respectFlags);
/* Grid<Real>::join keepMax (grid.cpp:303-311) */
void og_join_real(long long n, og_real* a, const og_real* b, int keepMax);
og_real og_get_max_abs(long long n, const og_real* a);

/* thread count used by the parallel sweeps (1 = the reference's serial order) */
void og_set_num_threads(int n);
int og_get_num_threads(void);

/* wavelet noise (noisefield.h/.cpp), float build */
typedef struct {
  float gsInv[3];      /* 1/max(grid size); z: 1 in 2D */
  float seedOffset[3]; /* mSeedOffset */
  float timeOffset;    /* getTime(): solver time * dx * timeAnim */
  float posScale[3], posOffset[3];
  float valOffset, valScale, clampNeg, clampPos;
  int clamp;
} og_noise_params;
void og_noise_tile(float* tile3x128cubed);
void og_noise_seed_offset(int fixedSeed, float* out3);
float og_noise_evaluate(const og_noise_params* q, const float* tile, float x, float y, float z);
void og_cylinder_sdf(og_dims d, float* phi, const float* center, float radius, const float* zaxis, float maxz);
void og_density_inflow(og_dims d, const int* flags, float* density, const float* sdf, const og_noise_params* q,
                       const float* tile, float scale, float sigma);

/* fractions / obstacle velocity (MAC grids) for the next pressure calls */
void og_set_fractions(const og_real* fractions, const og_real* obvel);

/* resetOutflow (extforces.cpp:133-160) without particles; phi / real may be
 * NULL */
void og_reset_outflow(og_dims d, int* flags, og_real* phi, og_real* real);
/* resetPhiInObs (advection.cpp:396-401) */
void og_reset_phi_in_obs(og_dims d, const int* flags, og_real* sdf);

/* FLIP transfers (plugin/flip.cpp:549-673).  Particles are pos[3*i] and
 * flag[i] (BasicParticleData, particle.h:182-191); ptype may be NULL; Vec3
 * data and grids are array-of-structs. */
void og_map_parts_to_mac(og_dims d, og_real* vel, og_real* velOld, og_real* weight, long long np, const og_real* pos,
                         const int* pflag, const og_real* pvel, const int* ptype, int exclude);
void og_map_parts_to_grid(og_dims d, og_real* target, int comps, long long np, const og_real* pos, const int* pflag,
                          const og_real* src);
void og_map_mac_to_parts(og_dims d, const og_real* vel, const og_real* velOld, og_real flipRatio, long long np,
                         const og_real* pos, const int* pflag, og_real* pvel, const int* ptype, int exclude);
void og_map_grid_to_parts(og_dims d, const og_real* grid, int comps, long long np, const og_real* pos,
                          const int* pflag, og_real* target);

#ifdef __cplusplus
}
#endif
#endif
