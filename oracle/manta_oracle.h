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
 * Layout is the reference's (source/grid.h:70): x fastest, index
 * i + nx*j + strideZ*k with strideZ = 0 in 2D.  Real = float.  Vec3 and MAC
 * grids are array-of-structs, 3 floats per cell (util/vectorbase.h:199-205).
 * Flags are int32 bit sets (source/grid.h:292-304).
 *
 * Arithmetic follows the reference expression by expression: where the
 * reference mixes a double literal into a float expression the restatement
 * computes that sub-expression in double and rounds once, as the C++ does.
 * Build with -ffp-contract=off (no FMA contraction), never -ffast-math.
 */
#ifndef MANTA_ORACLE_H
#define MANTA_ORACLE_H

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
int og_advect_semi_lagrange(og_dims d, const int* flags, const float* vel,
                            int kind, float* grid, int order, float strength,
                            int orderSpace, int clampMode, int orderTrace, float dt);

/* setWallBcs without fractions (plugin/extforces.cpp:186-217, 307-315). */
void og_set_wall_bcs(og_dims d, const int* flags, float* vel, const float* obvel);

/* addBuoyancy (plugin/extforces.cpp:72-87). */
void og_add_buoyancy(og_dims d, const int* flags, const float* density, float* vel,
                     float gx, float gy, float gz, float coefficient, int scale, float dt);

/* addGravity (plugin/extforces.cpp:46-65). exclude may be NULL. */
void og_add_gravity(og_dims d, const int* flags, float* vel, float gx, float gy, float gz,
                    const float* exclude, int scale, float dt);

/* extrapolateMACSimple (fastmarch.cpp:337-375), phiObs unsupported (NULL). */
void og_extrapolate_mac_simple(og_dims d, const int* flags, float* vel, int distance, int intoObs);

typedef struct {
  float cgAccuracy;        /* 1e-3 */
  float gfClamp;           /* 1e-4 */
  float cgMaxIterFac;      /* 1.5 */
  int preconditioner;      /* OG_PC_* */
  int enforceCompatibility;
  int useL2Norm;
  int zeroPressureFixing;
  float surfTens;          /* used only with phi and curv */
} og_pressure_params;

typedef struct {
  int iterations;
  float resNorm;
  int fixPidx;             /* pinned cell or -1 */
} og_pressure_result;

/* opaque multigrid hierarchy (multigrid.h:31-137); one per solver for the
 * static mode, like gMapMG in plugin/pressure.cpp:250 */
typedef struct og_mg og_mg;
og_mg* og_mg_create(og_dims d);
void og_mg_destroy(og_mg* mg);

/* computePressureRhs (plugin/pressure.cpp:277-299). */
void og_compute_pressure_rhs(og_dims d, float* rhs, const float* vel, const int* flags,
                             const float* phi, const float* perCellCorr, const float* curv,
                             const og_pressure_params* p);

/* solvePressureSystem (plugin/pressure.cpp:312-452).  rhs is modified when
 * pressure is pinned (fixPressure).  mg_cache: pointer to the solver's MG
 * slot (may hold NULL); used only by the MG preconditioners. */
int og_solve_pressure_system(og_dims d, float* rhs, float* pressure, const int* flags,
                             const float* phi, const og_pressure_params* p,
                             og_mg** mg_cache, og_pressure_result* out);

/* correctVelocity (plugin/pressure.cpp:455-476). */
void og_correct_velocity(og_dims d, float* vel, const float* pressure, const int* flags,
                         const float* phi, const float* curv, const og_pressure_params* p);

/* solvePressure (plugin/pressure.cpp:480-521): rhs, system, correction.
 * retRhs may be NULL. */
int og_solve_pressure(og_dims d, float* vel, float* pressure, const int* flags,
                      const float* phi, const float* perCellCorr, const float* curv,
                      const og_pressure_params* p, og_mg** mg_cache,
                      og_pressure_result* out, float* retRhs);

/* Building blocks exposed for kernel-level parity tests. */
void og_make_laplace_matrix(og_dims d, const int* flags, float* A0, float* Ai, float* Aj, float* Ak);
void og_apply_ghost_fluid_diagonal(og_dims d, float* A0, const int* flags, const float* phi, float gfClamp);
void og_mic_init(og_dims d, const int* flags, float* Aprecond, const float* A0,
                 const float* Ai, const float* Aj, const float* Ak);
void og_mic_apply(og_dims d, float* dst, const float* src, const int* flags, const float* Aprecond,
                  const float* Ai, const float* Aj, const float* Ak);
void og_apply_matrix(og_dims d, const int* flags, float* dst, const float* src, const float* A0,
                     const float* Ai, const float* Aj, const float* Ak);
/* one MG V-cycle from zero: setA (if not set) + setRhs + doVCycle */
void og_mg_vcycle(og_mg* mg, const float* A0, const float* Ai, const float* Aj, const float* Ak,
                  float* dst, const float* rhs, float coarseAccuracy);
/* number of levels / coarse vertex types for hierarchy parity tests */
int og_mg_num_levels(const og_mg* mg);
void og_mg_level_size(const og_mg* mg, int l, int* sz);
const signed char* og_mg_level_types(const og_mg* mg, int l);
const float* og_mg_level_matrix(const og_mg* mg, int l);

/* Scene setup (source/grid.cpp:732-861, plugin/extforces.cpp:105-160,
 * shapes.cpp:151-154, 178-228, 324-329). */
void og_init_domain(og_dims d, int* flags, int boundaryWidth, const char* wall,
                    const char* open, const char* inflow, const char* outflow);
void og_fill_grid(og_dims d, int* flags, int type);
void og_set_open_bound(og_dims d, int* flags, int bWidth, const char* openBound, int type);
void og_update_from_levelset(og_dims d, int* flags, const float* phi);
void og_box_sdf(og_dims d, float* phi, float p0x, float p0y, float p0z, float p1x, float p1y, float p1z);
/* Cylinder::isInside applied to cell centres (shape.applyToGrid), Real grid */
void og_cylinder_apply(og_dims d, float* grid, float cx, float cy, float cz, float radius,
                       float zx, float zy, float zz, float value, const int* respectFlags);
void og_box_apply(og_dims d, float* grid, float p0x, float p0y, float p0z,
                  float p1x, float p1y, float p1z, float value, const int* respectFlags);
/* Grid<Real>::join keepMax (grid.cpp:303-311) */
void og_join_real(long long n, float* a, const float* b, int keepMax);
float og_get_max_abs(long long n, const float* a);

/* thread count used by the parallel sweeps (1 = the reference's serial order) */
void og_set_num_threads(int n);
int og_get_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
