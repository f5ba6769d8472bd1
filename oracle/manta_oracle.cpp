/*
 * manta_oracle.cpp -- CPU restatement of mantaflow's grid-step hot path.
 * C++ only for std::sort, which the reference uses to order the multigrid
 * coarsening paths (multigrid.cpp:312-318); the rest is plain C.
 *
 * TEST INFRASTRUCTURE ONLY (see manta_oracle.h).  Every function names the
 * reference file:line it restates.  Loops mirror the reference's KERNEL
 * ranges (source/kernel.cpp:8-18: bnd=1 skips one cell layer, and in 2D
 * only k=0 is visited) and its OpenMP partition (one k-slab range per
 * thread, preprocessor/codegen_kernel.cpp:213-299).  With one thread every
 * reduction runs in index order, which is the order the reference's golden
 * outputs were generated with.
 */
#include "manta_oracle.h"

#include <algorithm>
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Real-typed helpers: the float build keeps the reference's float calls and
 * literals (OG_R(0.5) is 0.5f), the double build the double ones */
#define OG_R(x) ((og_real)(x))
#if defined(OG_REAL_IS_DOUBLE)
#define og_fabs fabs
#define og_sqrt sqrt
#define OG_REAL_MAX DBL_MAX
#define OG_VEC_EPS 1e-10
#else
#define og_fabs fabsf
#define og_sqrt sqrtf
#define OG_REAL_MAX FLT_MAX
#define OG_VEC_EPS 1e-6f
#endif

static int g_threads = 1;
void og_set_num_threads(int n) { g_threads = n < 1 ? 1 : n; }
int og_get_num_threads(void) { return g_threads; }

typedef long long ll;

#define SX(d) ((ll)1)
#define SY(d) ((ll)(d).nx)
#define SZ(d) ((d).is3d ? (ll)(d).nx * (d).ny : (ll)0)
#define NCELL(d) ((ll)(d).nx * (d).ny * (d).nz)
#define IX(d, i, j, k) ((ll)(i) + SY(d) * (j) + SZ(d) * (k))
#define CELLS(d) ((ll)(d).nx * (d).ny * (d).nz)

/* loop helpers: reference KERNEL ijk range with boundary width b */
#define KLO(d, b) ((d).is3d ? (b) : 0)
#define KHI(d, b) ((d).is3d ? (d).nz - (b) : 1)

static inline int isF(const int* f, ll i) { return (f[i] & OG_FLUID) != 0; }
static inline int isO(const int* f, ll i) { return (f[i] & OG_OBSTACLE) != 0; }
static inline int isE(const int* f, ll i) { return (f[i] & OG_EMPTY) != 0; }
static inline int isOut(const int* f, ll i) { return (f[i] & OG_OUTFLOW) != 0; }
static inline int isStk(const int* f, ll i) { return (f[i] & OG_STICK) != 0; }

static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int iclamp(int v, int lo, int hi) { if (v < lo) return lo; if (v > hi) return hi; return v; }

/* ------------------------------------------------------------------------ */
/* MAC accessors, source/grid.h:424-470.  0.5*(a+b) and 0.25*(...) are exact
 * scalings of a Real sum, so Real arithmetic reproduces them.            */

typedef struct { og_real x, y, z; } v3;

static inline v3 mac_centered(og_dims d, const og_real* u, ll idx) {
  v3 v;
  v.x = OG_R(0.5) * (u[3 * idx + 0] + u[3 * (idx + 1) + 0]);
  v.y = OG_R(0.5) * (u[3 * idx + 1] + u[3 * (idx + SY(d)) + 1]);
  v.z = OG_R(0.);
  if (d.is3d) v.z = OG_R(0.5) * (u[3 * idx + 2] + u[3 * (idx + SZ(d)) + 2]);
  return v;
}
static inline v3 mac_at_x(og_dims d, const og_real* u, ll idx) {
  const ll Y = SY(d), Z = SZ(d);
  v3 v;
  v.x = u[3 * idx];
  v.y = OG_R(0.25) * (u[3 * idx + 1] + u[3 * (idx - 1) + 1] + u[3 * (idx + Y) + 1] + u[3 * (idx + Y - 1) + 1]);
  v.z = OG_R(0.);
  if (d.is3d) v.z = OG_R(0.25) * (u[3 * idx + 2] + u[3 * (idx - 1) + 2] + u[3 * (idx + Z) + 2] + u[3 * (idx + Z - 1) + 2]);
  return v;
}
static inline v3 mac_at_y(og_dims d, const og_real* u, ll idx) {
  const ll Y = SY(d), Z = SZ(d);
  v3 v;
  v.x = OG_R(0.25) * (u[3 * idx] + u[3 * (idx - Y)] + u[3 * (idx + 1)] + u[3 * (idx + 1 - Y)]);
  v.y = u[3 * idx + 1];
  v.z = OG_R(0.);
  if (d.is3d) v.z = OG_R(0.25) * (u[3 * idx + 2] + u[3 * (idx - Y) + 2] + u[3 * (idx + Z) + 2] + u[3 * (idx + Z - Y) + 2]);
  return v;
}
static inline v3 mac_at_z(og_dims d, const og_real* u, ll idx) {
  const ll Y = SY(d), Z = SZ(d);
  v3 v;
  v.x = OG_R(0.25) * (u[3 * idx] + u[3 * (idx - Z)] + u[3 * (idx + 1)] + u[3 * (idx + 1 - Z)]);
  v.y = OG_R(0.25) * (u[3 * idx + 1] + u[3 * (idx - Z) + 1] + u[3 * (idx + Y) + 1] + u[3 * (idx + Y - Z) + 1]);
  v.z = u[3 * idx + 2];
  return v;
}

/* ------------------------------------------------------------------------ */
/* Trilinear interpolation, util/interpol.h:50-90 (BUILD_INDEX) and
 * :116-157 (BUILD_INDEX_SHIFT / interpolMAC).                               */

typedef struct {
  int xi, yi, zi;
  og_real s0, s1, t0, t1, f0, f1;
} wts;

static inline wts build_index(og_dims d, og_real x, og_real y, og_real z) {
  wts w;
  og_real px = x - OG_R(0.5), py = y - OG_R(0.5), pz = z - OG_R(0.5);
  w.xi = (int)px; w.yi = (int)py; w.zi = (int)pz;
  w.s1 = px - (og_real)w.xi; w.s0 = OG_R(1.) - w.s1;
  w.t1 = py - (og_real)w.yi; w.t0 = OG_R(1.) - w.t1;
  w.f1 = pz - (og_real)w.zi; w.f0 = OG_R(1.) - w.f1;
  if (px < OG_R(0.)) { w.xi = 0; w.s0 = OG_R(1.); w.s1 = OG_R(0.); }
  if (py < OG_R(0.)) { w.yi = 0; w.t0 = OG_R(1.); w.t1 = OG_R(0.); }
  if (pz < OG_R(0.)) { w.zi = 0; w.f0 = OG_R(1.); w.f1 = OG_R(0.); }
  if (w.xi >= d.nx - 1) { w.xi = d.nx - 2; w.s0 = OG_R(0.); w.s1 = OG_R(1.); }
  if (w.yi >= d.ny - 1) { w.yi = d.ny - 2; w.t0 = OG_R(0.); w.t1 = OG_R(1.); }
  if (d.nz > 1) { if (w.zi >= d.nz - 1) { w.zi = d.nz - 2; w.f0 = OG_R(0.); w.f1 = OG_R(1.); } }
  return w;
}

static inline wts build_index_shift(og_dims d, og_real x, og_real y, og_real z) {
  wts w;
  w.xi = (int)x; w.yi = (int)y; w.zi = (int)z;
  w.s1 = x - (og_real)w.xi; w.s0 = OG_R(1.) - w.s1;
  w.t1 = y - (og_real)w.yi; w.t0 = OG_R(1.) - w.t1;
  w.f1 = z - (og_real)w.zi; w.f0 = OG_R(1.) - w.f1;
  if (x < 0) { w.xi = 0; w.s0 = OG_R(1.); w.s1 = OG_R(0.); }
  if (y < 0) { w.yi = 0; w.t0 = OG_R(1.); w.t1 = OG_R(0.); }
  if (z < 0) { w.zi = 0; w.f0 = OG_R(1.); w.f1 = OG_R(0.); }
  if (w.xi >= d.nx - 1) { w.xi = d.nx - 2; w.s0 = OG_R(0.); w.s1 = OG_R(1.); }
  if (w.yi >= d.ny - 1) { w.yi = d.ny - 2; w.t0 = OG_R(0.); w.t1 = OG_R(1.); }
  if (d.nz > 1) { if (w.zi >= d.nz - 1) { w.zi = d.nz - 2; w.f0 = OG_R(0.); w.f1 = OG_R(1.); } }
  return w;
}

/* interpol<T> on one Real channel: data[stride*idx + c] */
static inline og_real interp_ch(og_dims d, const og_real* data, int stride, int c, og_real x, og_real y, og_real z) {
  wts w = build_index(d, x, y, z);
  const ll X = 1, Y = SY(d), Z = SZ(d);
  const ll idx = (ll)w.xi + Y * w.yi + Z * w.zi;
#define D(o) data[stride * (idx + (o)) + c]
  return ((D(0) * w.t0 + D(Y) * w.t1) * w.s0 + (D(X) * w.t0 + D(X + Y) * w.t1) * w.s1) * w.f0 +
         ((D(Z) * w.t0 + D(Y + Z) * w.t1) * w.s0 + (D(X + Z) * w.t0 + D(X + Y + Z) * w.t1) * w.s1) * w.f1;
#undef D
}

/* interpolMAC (util/interpol.h:127-157) */
static inline v3 interp_mac(og_dims d, const og_real* u, og_real x, og_real y, og_real z) {
  wts w = build_index(d, x, y, z);
  wts s = build_index_shift(d, x, y, z);
  const ll X = 1, Y = SY(d), Z = SZ(d);
  v3 r;
  {
    const ll b = ((ll)w.zi * d.ny + w.yi) * d.nx + s.xi;
#define R(o) u[3 * (b + (o)) + 0]
    r.x = w.f0 * ((R(0) * w.t0 + R(Y) * w.t1) * s.s0 + (R(X) * w.t0 + R(X + Y) * w.t1) * s.s1) +
          w.f1 * ((R(Z) * w.t0 + R(Z + Y) * w.t1) * s.s0 + (R(X + Z) * w.t0 + R(X + Y + Z) * w.t1) * s.s1);
#undef R
  }
  {
    const ll b = ((ll)w.zi * d.ny + s.yi) * d.nx + w.xi;
#define R(o) u[3 * (b + (o)) + 1]
    r.y = w.f0 * ((R(0) * s.t0 + R(Y) * s.t1) * w.s0 + (R(X) * s.t0 + R(X + Y) * s.t1) * w.s1) +
          w.f1 * ((R(Z) * s.t0 + R(Z + Y) * s.t1) * w.s0 + (R(X + Z) * s.t0 + R(X + Y + Z) * s.t1) * w.s1);
#undef R
  }
  {
    const ll b = ((ll)s.zi * d.ny + w.yi) * d.nx + w.xi;
#define R(o) u[3 * (b + (o)) + 2]
    r.z = s.f0 * ((R(0) * w.t0 + R(Y) * w.t1) * w.s0 + (R(X) * w.t0 + R(X + Y) * w.t1) * w.s1) +
          s.f1 * ((R(Z) * w.t0 + R(Z + Y) * w.t1) * w.s0 + (R(X + Z) * w.t0 + R(X + Y + Z) * w.t1) * w.s1);
#undef R
  }
  return r;
}

/* ------------------------------------------------------------------------ */
/* Catmull-Rom cubic, util/interpolHigh.h:22-40, 42-160.  For Real grids the
 * reference forms a2/a3 in double (double literals) and rounds once.        */

static inline og_real cubic_real(og_real t, const og_real* p) {
  og_real d0 = (og_real)((double)(p[2] - p[0]) * 0.5);
  og_real d1 = (og_real)((double)(p[3] - p[1]) * 0.5);
  og_real dk = p[2] - p[1];
  og_real a0 = p[1], a1 = d0;
  og_real a2 = (og_real)(3.0 * dk - 2.0 * d0 - d1);
  og_real a3 = (og_real)(-2.0 * dk + d0 + d1);
  og_real sq = t * t, cu = sq * t;
  return a3 * cu + a2 * sq + a1 * t + a0;
}
/* Vec3 variant: every Vec3 operator rounds to Real per component */
static inline og_real cubic_vec(og_real t, const og_real* p) {
  og_real d0 = (og_real)((double)(p[2] - p[0]) * 0.5);
  og_real d1 = (og_real)((double)(p[3] - p[1]) * 0.5);
  og_real dk = p[2] - p[1];
  og_real a0 = p[1], a1 = d0;
  og_real a2 = (og_real)(3.0 * dk);
  a2 = a2 - (og_real)(2.0 * d0);
  a2 = a2 - d1;
  og_real a3 = (og_real)(-2.0 * dk);
  a3 = a3 + d0;
  a3 = a3 + d1;
  og_real sq = t * t, cu = sq * t;
  return a3 * cu + a2 * sq + a1 * t + a0;
}

static og_real interp_cubic_ch(og_dims d, const og_real* data, int stride, int c, og_real x, og_real y, og_real z, int vecmode) {
  og_real (*cub)(og_real, const og_real*) = vecmode ? cubic_vec : cubic_real;
  const ll Z = SZ(d);
  if (Z == 0) {
    const og_real px = x - OG_R(0.5), py = y - OG_R(0.5);
    const int x1 = (int)px, x2 = x1 + 1, x3 = x1 + 2, x0 = x1 - 1;
    const int y1 = (int)py, y2 = y1 + 1, y3 = y1 + 2, y0 = y1 - 1;
    if (x0 < 0 || y0 < 0 || x3 >= d.nx || y3 >= d.ny) return interp_ch(d, data, stride, c, x, y, z);
    const og_real xI = px - x1, yI = py - y1;
    const int yy[4] = {y0 * d.nx, y1 * d.nx, y2 * d.nx, y3 * d.nx};
    const int xx[4] = {x0, x1, x2, x3};
    og_real fin[4];
    for (int r = 0; r < 4; r++) {
      og_real pts[4];
      for (int q = 0; q < 4; q++) pts[q] = data[stride * (ll)(xx[q] + yy[r]) + c];
      fin[r] = cub(xI, pts);
    }
    return cub(yI, fin);
  }
  const og_real px = x - OG_R(0.5), py = y - OG_R(0.5), pz = z - OG_R(0.5);
  const int x1 = (int)px, x2 = x1 + 1, x3 = x1 + 2, x0 = x1 - 1;
  const int y1 = (int)py, y2 = y1 + 1, y3 = y1 + 2, y0 = y1 - 1;
  const int z1 = (int)pz, z2 = z1 + 1, z3 = z1 + 2, z0 = z1 - 1;
  if (x0 < 0 || y0 < 0 || z0 < 0 || x3 >= d.nx || y3 >= d.ny || z3 >= d.nz) return interp_ch(d, data, stride, c, x, y, z);
  const og_real xI = px - x1, yI = py - y1, zI = pz - z1;
  const int slab = d.nx * d.ny;
  const int zz[4] = {z0 * slab, z1 * slab, z2 * slab, z3 * slab};
  const int yy[4] = {y0 * d.nx, y1 * d.nx, y2 * d.nx, y3 * d.nx};
  const int xx[4] = {x0, x1, x2, x3};
  og_real zp[4];
  for (int s = 0; s < 4; s++) {
    og_real yp[4];
    for (int r = 0; r < 4; r++) {
      og_real pts[4];
      for (int q = 0; q < 4; q++) pts[q] = data[stride * (ll)(xx[q] + yy[r] + zz[s]) + c];
      yp[r] = cub(xI, pts);
    }
    zp[s] = cub(yI, yp);
  }
  return cub(zI, zp);
}

/* ------------------------------------------------------------------------ */
/* SemiLagrange (advection.cpp:25-41) for Real (ch=1) and Vec3 (ch=3) grids */

static void semi_lagrange(og_dims d, const og_real* vel, og_real* dst, const og_real* src, int ch, og_real dt,
                          int orderSpace, int orderTrace) {
  int k;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        og_real px, py, pz;
        v3 vc = mac_centered(d, vel, idx);
        if (orderTrace == 1) {
          px = (i + OG_R(0.5)) - vc.x * dt;
          py = (j + OG_R(0.5)) - vc.y * dt;
          pz = (k + OG_R(0.5)) - vc.z * dt;
        } else {
          const og_real p0x = i + OG_R(0.5), p0y = j + OG_R(0.5), p0z = k + OG_R(0.5);
          const og_real p1x = p0x - (og_real)((double)(vc.x * dt) * 0.5);
          const og_real p1y = p0y - (og_real)((double)(vc.y * dt) * 0.5);
          const og_real p1z = p0z - (og_real)((double)(vc.z * dt) * 0.5);
          v3 vi = interp_mac(d, vel, p1x, p1y, p1z);
          px = p0x - vi.x * dt;
          py = p0y - vi.y * dt;
          pz = p0z - vi.z * dt;
        }
        for (int c = 0; c < ch; c++) {
          if (orderSpace == 1)
            dst[ch * idx + c] = interp_ch(d, src, ch, c, px, py, pz);
          else
            dst[ch * idx + c] = interp_cubic_ch(d, src, ch, c, px, py, pz, ch == 3);
        }
      }
}

/* cubic MAC sampling, util/interpolHigh.h:171-178 */
static og_real interp_cubic_mac_c(og_dims d, const og_real* u, int c, og_real x, og_real y, og_real z) {
  if (c == 0) return interp_cubic_ch(d, u, 3, 0, x + OG_R(0.5), y, z, 1);
  if (c == 1) return interp_cubic_ch(d, u, 3, 1, x, y + OG_R(0.5), z, 1);
  if (SZ(d) == 0) return OG_R(0.);
  return interp_cubic_ch(d, u, 3, 2, x, y, z + OG_R(0.5), 1);
}

/* SemiLagrangeMAC (advection.cpp:44-77) */
static void semi_lagrange_mac(og_dims d, const og_real* vel, og_real* dst, const og_real* src, og_real dt,
                              int orderSpace, int orderTrace) {
  int k;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        og_real out[3];
        if (orderTrace == 1) {
          v3 a[3];
          a[0] = mac_at_x(d, vel, idx);
          a[1] = mac_at_y(d, vel, idx);
          a[2] = mac_at_z(d, vel, idx);
          for (int c = 0; c < 3; c++) {
            const og_real px = (i + OG_R(0.5)) - a[c].x * dt;
            const og_real py = (j + OG_R(0.5)) - a[c].y * dt;
            const og_real pz = (k + OG_R(0.5)) - a[c].z * dt;
            out[c] = orderSpace == 1 ? interp_ch(d, src, 3, c, px, py, pz) : interp_cubic_mac_c(d, src, c, px, py, pz);
          }
        } else {
          const og_real p0x = (og_real)(i + 0.5), p0y = (og_real)(j + 0.5), p0z = (og_real)(k + 0.5);
          for (int c = 0; c < 3; c++) {
            og_real q0x = (og_real)i + (c == 0 ? OG_R(0.) : OG_R(0.5));
            og_real q0y = (og_real)j + (c == 1 ? OG_R(0.) : OG_R(0.5));
            og_real q0z = (og_real)k + (c == 2 ? OG_R(0.) : OG_R(0.5));
            if (c == 0) { q0x = (og_real)i; q0y = j + OG_R(0.5); q0z = k + OG_R(0.5); }
            if (c == 1) { q0x = i + OG_R(0.5); q0y = (og_real)j; q0z = k + OG_R(0.5); }
            if (c == 2) { q0x = i + OG_R(0.5); q0y = j + OG_R(0.5); q0z = (og_real)k; }
            v3 a = c == 0 ? mac_at_x(d, src, idx) : (c == 1 ? mac_at_y(d, src, idx) : mac_at_z(d, src, idx));
            const og_real q1x = q0x - (og_real)((double)(a.x * dt) * 0.5);
            const og_real q1y = q0y - (og_real)((double)(a.y * dt) * 0.5);
            const og_real q1z = q0z - (og_real)((double)(a.z * dt) * 0.5);
            v3 vi = interp_mac(d, src, q1x, q1y, q1z);
            const og_real px = p0x - vi.x * dt, py = p0y - vi.y * dt, pz = p0z - vi.z * dt;
            out[c] = orderSpace == 1 ? interp_ch(d, src, 3, c, px, py, pz) : interp_cubic_mac_c(d, src, c, px, py, pz);
          }
        }
        dst[3 * idx + 0] = out[0];
        dst[3 * idx + 1] = out[1];
        dst[3 * idx + 2] = out[2];
      }
}

/* MacCormackCorrect (advection.cpp:81-91): dst = fwd (+ correction on fluid
 * cells), the correction formed in double as in the reference.  ch=1/3.   */
static void maccormack_correct(og_dims d, const int* flags, og_real* dst, const og_real* old, const og_real* fwd,
                               const og_real* bwd, og_real strength, int ch) {
  const ll n = NCELL(d);
  ll idx;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (idx = 0; idx < n; idx++) {
    for (int c = 0; c < ch; c++) {
      og_real v = fwd[ch * idx + c];
      if (isF(flags, idx)) {
        if (ch == 1)
          v = (og_real)((double)v + (double)strength * 0.5 * (double)(old[idx] - bwd[idx]));
        else /* Vec3 += : strength*0.5*(Vec3) rounds per component first */
          v = v + (og_real)((double)strength * 0.5 * (double)(old[3 * idx + c] - bwd[3 * idx + c]));
      }
      dst[ch * idx + c] = v;
    }
  }
}

/* MacCormackCorrectMAC (advection.cpp:94-115) */
static void maccormack_correct_mac(og_dims d, const int* flags, og_real* dst, const og_real* old, const og_real* fwd,
                                   const og_real* bwd, og_real strength) {
  int k;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (k = 0; k < d.nz; k++)
    for (int j = 0; j < d.ny; j++)
      for (int i = 0; i < d.nx; i++) {
        const ll idx = IX(d, i, j, k);
        int skip[3] = {0, 0, 0};
        if (!isF(flags, idx)) skip[0] = skip[1] = skip[2] = 1;
        if (i > 0 && !isF(flags, idx - 1)) skip[0] = 1;
        if (j > 0 && !isF(flags, idx - SY(d))) skip[1] = 1;
        if (k > 0 && !isF(flags, idx - SZ(d))) skip[2] = 1;
        for (int c = 0; c < 3; c++) {
          const ll e = 3 * idx + c;
          if (skip[c]) dst[e] = fwd[e];
          else dst[e] = (og_real)((double)fwd[e] + (double)strength * 0.5 * (double)(old[e] - bwd[e]));
        }
      }
}

#define CHECKF(fl) ((fl) & (OG_FLUID | OG_EMPTY))

/* doClampComponent (advection.cpp:144-186) for ch channels; cmpMinMax of a
 * Vec3 reverts the whole vector when any component is out of range.       */
static void clamp_component(og_dims d, const int* flags, og_real* dv, const og_real* orig, const og_real* fwd,
                            int ch, og_real posx, og_real posy, og_real posz, v3 vel, int clampMode) {
  og_real mn[3], mx[3];
  int haveFl = 0;
  for (int c = 0; c < ch; c++) { mn[c] = OG_REAL_MAX; mx[c] = -OG_REAL_MAX; }
  int px[2], py[2], pz[2], np = 1;
  px[0] = (int)(posx - vel.x); py[0] = (int)(posy - vel.y); pz[0] = (int)(posz - vel.z);
  if (clampMode == 1) { np = 2; px[1] = (int)(posx + vel.x); py[1] = (int)(posy + vel.y); pz[1] = (int)(posz + vel.z); }
  const int gx = d.nx - 1, gy = d.ny - 1, gz = d.nz - 1;
  for (int l = 0; l < np; l++) {
    const int i0 = iclamp(px[l], 0, gx - 1);
    const int j0 = iclamp(py[l], 0, gy - 1);
    const int k0 = iclamp(pz[l], 0, d.is3d ? (gz - 1) : 1);
    const int i1 = i0 + 1, j1 = j0 + 1, k1 = d.is3d ? (k0 + 1) : k0;
    const int ci[8] = {i0, i1, i0, i1, i0, i1, i0, i1};
    const int cj[8] = {j0, j0, j1, j1, j0, j0, j1, j1};
    const int ck[8] = {k0, k0, k0, k0, k1, k1, k1, k1};
    const int ncorner = d.is3d ? 8 : 4;
    for (int q = 0; q < ncorner; q++) {
      const ll e = IX(d, ci[q], cj[q], ck[q]);
      if (CHECKF(flags[e])) {
        for (int c = 0; c < ch; c++) {
          const og_real v = orig[ch * e + c];
          if (v < mn[c]) mn[c] = v;
          if (v > mx[c]) mx[c] = v;
        }
        haveFl = 1;
      }
    }
  }
  if (!haveFl) { for (int c = 0; c < ch; c++) dv[c] = fwd[c]; return; }
  if (clampMode == 1) {
    for (int c = 0; c < ch; c++) {
      if (dv[c] < mn[c]) dv[c] = mn[c];
      else if (dv[c] > mx[c]) dv[c] = mx[c];
    }
  } else {
    int out = 0;
    for (int c = 0; c < ch; c++) out |= (dv[c] < mn[c]) || (dv[c] > mx[c]);
    if (out) for (int c = 0; c < ch; c++) dv[c] = fwd[c];
  }
}

/* MacCormackClamp (advection.cpp:241-267) */
static void maccormack_clamp(og_dims d, const int* flags, const og_real* vel, og_real* dst, const og_real* orig,
                             const og_real* fwd, og_real dt, int clampMode, int ch) {
  int k;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        og_real dv[3];
        for (int c = 0; c < ch; c++) dv[c] = dst[ch * idx + c];
        v3 vc = mac_centered(d, vel, idx);
        v3 vd = {vc.x * dt, vc.y * dt, vc.z * dt};
        clamp_component(d, flags, dv, orig, fwd + ch * idx, ch, (og_real)i, (og_real)j, (og_real)k, vd, clampMode);
        if (clampMode == 1) {
          const int fx = (int)(((og_real)i + OG_R(0.5)) - vd.x), fy = (int)(((og_real)j + OG_R(0.5)) - vd.y), fz = (int)(((og_real)k + OG_R(0.5)) - vd.z);
          const int bx = (int)(((og_real)i + OG_R(0.5)) + vd.x), by = (int)(((og_real)j + OG_R(0.5)) + vd.y), bz = (int)(((og_real)k + OG_R(0.5)) + vd.z);
          const int gx = d.nx - 1, gy = d.ny - 1, gz = d.nz - 1;
          int rev = fx < 0 || fy < 0 || fz < 0 || bx < 0 || by < 0 || bz < 0 ||
                    fx > gx || fy > gy || ((fz > gz) && d.is3d) ||
                    bx > gx || by > gy || ((bz > gz) && d.is3d);
          if (!rev) rev = isO(flags, IX(d, fx, fy, fz)) || isO(flags, IX(d, bx, by, bz));
          if (rev) for (int c = 0; c < ch; c++) dv[c] = fwd[ch * idx + c];
        }
        for (int c = 0; c < ch; c++) dst[ch * idx + c] = dv[c];
      }
}

/* doClampComponentMAC (advection.cpp:191-235) */
static og_real clamp_component_mac(og_dims d, const int* flags, og_real dst, const og_real* orig, og_real fwd, int c,
                                 int i, int j, int k, v3 vel, int clampMode) {
  og_real mn = OG_REAL_MAX, mx = -OG_REAL_MAX;
  const og_real posx = (og_real)i, posy = (og_real)j, posz = (og_real)k;
  int px[2], py[2], pz[2], np = 1;
  px[0] = (int)(posx - vel.x); py[0] = (int)(posy - vel.y); pz[0] = (int)(posz - vel.z);
  if (clampMode == 1) { np = 2; px[1] = (int)(posx + vel.x); py[1] = (int)(posy + vel.y); pz[1] = (int)(posz + vel.z); }
  int ni = i, nj = j, nk = k;
  if (c == 0) ni -= 1; else if (c == 1) nj -= 1; else nk -= 1;
  if (clampMode == 2 && !(CHECKF(flags[IX(d, i, j, k)]) && CHECKF(flags[IX(d, ni, nj, nk)]))) return fwd;
  const int gx = d.nx - 1, gy = d.ny - 1, gz = d.nz - 1;
  for (int l = 0; l < np; l++) {
    const int i0 = iclamp(px[l], 0, gx - 1);
    const int j0 = iclamp(py[l], 0, gy - 1);
    const int k0 = iclamp(pz[l], 0, d.is3d ? (gz - 1) : 0);
    const int i1 = i0 + 1, j1 = j0 + 1, k1 = d.is3d ? (k0 + 1) : k0;
    const int ci[8] = {i0, i1, i0, i1, i0, i1, i0, i1};
    const int cj[8] = {j0, j0, j1, j1, j0, j0, j1, j1};
    const int ck[8] = {k0, k0, k0, k0, k1, k1, k1, k1};
    const int ncorner = d.is3d ? 8 : 4;
    for (int q = 0; q < ncorner; q++) {
      const og_real v = orig[3 * IX(d, ci[q], cj[q], ck[q]) + c];
      if (v < mn) mn = v;
      if (v > mx) mx = v;
    }
  }
  if (clampMode == 1) {
    if (dst < mn) dst = mn;
    else if (dst > mx) dst = mx;
  } else {
    if (dst < mn || dst > mx) dst = fwd;
  }
  return dst;
}

/* MacCormackClampMAC (advection.cpp:270-287) */
static void maccormack_clamp_mac(og_dims d, const int* flags, const og_real* vel, og_real* dst, const og_real* orig,
                                 const og_real* fwd, og_real dt, int clampMode) {
  int k;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        v3 a = mac_at_x(d, vel, idx);
        v3 va = {a.x * dt, a.y * dt, a.z * dt};
        dst[3 * idx + 0] = clamp_component_mac(d, flags, dst[3 * idx + 0], orig, fwd[3 * idx + 0], 0, i, j, k, va, clampMode);
        a = mac_at_y(d, vel, idx);
        v3 vb = {a.x * dt, a.y * dt, a.z * dt};
        dst[3 * idx + 1] = clamp_component_mac(d, flags, dst[3 * idx + 1], orig, fwd[3 * idx + 1], 1, i, j, k, vb, clampMode);
        if (d.is3d) {
          a = mac_at_z(d, vel, idx);
          v3 vz = {a.x * dt, a.y * dt, a.z * dt};
          dst[3 * idx + 2] = clamp_component_mac(d, flags, dst[3 * idx + 2], orig, fwd[3 * idx + 2], 2, i, j, k, vz, clampMode);
        }
      }
}

/* getBulkVel + extrapolateVelConvectiveBC + copyChangedVels
 * (advection.cpp:324-391) */
static void apply_outflow_bc(og_dims d, const int* flags, og_real* vel, const og_real* velPrev, double timeStep) {
  const ll n = NCELL(d);
  og_real* velDst = (og_real*)calloc((size_t)(3 * n), sizeof(og_real));
  const og_real ts = (og_real)(timeStep * 4 > 1.0 ? timeStep * 4 : 1.0);
  int k;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (k = 0; k < d.nz; k++)
    for (int j = 0; j < d.ny; j++)
      for (int i = 0; i < d.nx; i++) {
        const ll idx = IX(d, i, j, k);
        if (!isOut(flags, idx)) continue;
        /* bulk velocity: mean over the 3^dim neighbourhood of fluid/outflow cells */
        og_real ax = OG_R(0.), ay = OG_R(0.), az = OG_R(0.);
        int count = 0;
        const int nmax = d.is3d ? 1 : 0;
        for (int nn = -nmax; nn <= nmax; nn++)
          for (int m = -1; m <= 1; m++)
            for (int l = -1; l <= 1; l++) {
              const int x = i + l, y = j + m, z = k + nn;
              if (x >= 0 && y >= 0 && z >= 0 && x < d.nx && y < d.ny && z < d.nz) {
                const ll e = IX(d, x, y, z);
                if (isF(flags, e) || isOut(flags, e)) {
                  ax += vel[3 * e]; ay += vel[3 * e + 1]; az += vel[3 * e + 2];
                  count++;
                }
              }
            }
        og_real bulk[3] = {ax, ay, az};
        if (count > 0) { bulk[0] = ax / (og_real)count; bulk[1] = ay / (og_real)count; bulk[2] = az / (og_real)count; }
        const int dim = d.is3d ? 3 : 2;
        int cnt = 0;
        og_real dx = OG_R(0.), dy = OG_R(0.), dz = OG_R(0.);
        const int cur[3] = {i, j, k};
        for (int c = 0; c < dim; c++) {
          int lo[3] = {i, j, k}, up[3] = {i, j, k}, fl[3] = {i, j, k}, fu[3] = {i, j, k};
          const og_real factor = ts * (bulk[c] > OG_R(1.0) ? bulk[c] : OG_R(1.0));
          lo[c] = fl[c] = cur[c] - 1;
          up[c] = fu[c] = cur[c] + 1;
          for (int dd = 0; dd < 2; dd++) {
            const int inL = fl[0] >= 0 && fl[1] >= 0 && fl[2] >= 0 && fl[0] < d.nx && fl[1] < d.ny && fl[2] < d.nz;
            const int inU = fu[0] >= 0 && fu[1] >= 0 && fu[2] >= 0 && fu[0] < d.nx && fu[1] < d.ny && fu[2] < d.nz;
            const int fromL = inL && isF(flags, IX(d, fl[0], fl[1], fl[2]));
            const int fromU = inU && isF(flags, IX(d, fu[0], fu[1], fu[2]));
            if (fromL || fromU) {
              if (fromL) {
                const ll e = IX(d, lo[0], lo[1], lo[2]);
                dx += ((vel[3 * idx + 0] - velPrev[3 * idx + 0]) / factor) + vel[3 * e + 0];
                dy += ((vel[3 * idx + 1] - velPrev[3 * idx + 1]) / factor) + vel[3 * e + 1];
                dz += ((vel[3 * idx + 2] - velPrev[3 * idx + 2]) / factor) + vel[3 * e + 2];
                cnt++;
              }
              if (fromU) {
                const ll e = IX(d, up[0], up[1], up[2]);
                dx += ((vel[3 * idx + 0] - velPrev[3 * idx + 0]) / factor) + vel[3 * e + 0];
                dy += ((vel[3 * idx + 1] - velPrev[3 * idx + 1]) / factor) + vel[3 * e + 1];
                dz += ((vel[3 * idx + 2] - velPrev[3 * idx + 2]) / factor) + vel[3 * e + 2];
                cnt++;
              }
              break;
            }
            fl[c]--;
            fu[c]++;
          }
        }
        if (cnt > 0) { dx /= (og_real)cnt; dy /= (og_real)cnt; dz /= (og_real)cnt; }
        velDst[3 * idx] = dx; velDst[3 * idx + 1] = dy; velDst[3 * idx + 2] = dz;
      }
  ll idx;
  for (idx = 0; idx < n; idx++)
    if (isOut(flags, idx)) {
      vel[3 * idx] = velDst[3 * idx];
      vel[3 * idx + 1] = velDst[3 * idx + 1];
      vel[3 * idx + 2] = velDst[3 * idx + 2];
    }
  free(velDst);
}

/* fnAdvectSemiLagrange and its MAC specialisation (advection.cpp:292-321,
 * 406-436); advectSemiLagrange dispatch (:442-460).                        */
int og_advect_semi_lagrange(og_dims d, const int* flags, const og_real* vel, int kind, og_real* grid, int order,
                            og_real strength, int orderSpace, int clampMode, int orderTrace, og_real dt) {
  if (order != 1 && order != 2) return -1;
  if (orderTrace != 1 && orderTrace != 2) return -2;
  const ll n = NCELL(d);
  const int ch = kind == OG_KIND_REAL ? 1 : 3;
  og_real* fwd = (og_real*)calloc((size_t)(ch * n), sizeof(og_real));
  if (kind != OG_KIND_MAC) {
    semi_lagrange(d, vel, fwd, grid, ch, dt, orderSpace, orderTrace);
    if (order == 1) {
      memcpy(grid, fwd, sizeof(og_real) * ch * n);
    } else {
      og_real* bwd = (og_real*)calloc((size_t)(ch * n), sizeof(og_real));
      og_real* nw = (og_real*)calloc((size_t)(ch * n), sizeof(og_real));
      semi_lagrange(d, vel, bwd, fwd, ch, -dt, orderSpace, orderTrace);
      maccormack_correct(d, flags, nw, grid, fwd, bwd, strength, ch);
      maccormack_clamp(d, flags, vel, nw, grid, fwd, dt, clampMode, ch);
      memcpy(grid, nw, sizeof(og_real) * ch * n);
      free(bwd);
      free(nw);
    }
  } else {
    semi_lagrange_mac(d, vel, fwd, grid, dt, orderSpace, orderTrace);
    if (order == 1) {
      apply_outflow_bc(d, flags, fwd, grid, (double)dt);
      memcpy(grid, fwd, sizeof(og_real) * 3 * n);
    } else {
      og_real* bwd = (og_real*)calloc((size_t)(3 * n), sizeof(og_real));
      og_real* nw = (og_real*)calloc((size_t)(3 * n), sizeof(og_real));
      semi_lagrange_mac(d, vel, bwd, fwd, -dt, orderSpace, orderTrace);
      maccormack_correct_mac(d, flags, nw, grid, fwd, bwd, strength);
      maccormack_clamp_mac(d, flags, vel, nw, grid, fwd, dt, clampMode);
      apply_outflow_bc(d, flags, nw, grid, (double)dt);
      memcpy(grid, nw, sizeof(og_real) * 3 * n);
      free(bwd);
      free(nw);
    }
  }
  free(fwd);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Forces and wall boundary conditions, plugin/extforces.cpp                */

/* KnSetWallBcs (:186-217), all cells, i>0 checks */
void og_set_wall_bcs(og_dims d, const int* flags, og_real* vel, const og_real* obvel) {
  int k;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (k = 0; k < d.nz; k++)
    for (int j = 0; j < d.ny; j++)
      for (int i = 0; i < d.nx; i++) {
        const ll idx = IX(d, i, j, k);
        const int curFluid = isF(flags, idx), curObs = isO(flags, idx);
        if (!curFluid && !curObs) continue;
        og_real bx = OG_R(0.), by = OG_R(0.), bz = OG_R(0.);
        if (obvel) {
          bx = obvel[3 * idx]; by = obvel[3 * idx + 1];
          if (d.is3d) bz = obvel[3 * idx + 2];
        }
        og_real* v = vel + 3 * idx;
        if (i > 0 && isO(flags, idx - 1)) v[0] = bx;
        if (i > 0 && curObs && isF(flags, idx - 1)) v[0] = bx;
        if (j > 0 && isO(flags, idx - SY(d))) v[1] = by;
        if (j > 0 && curObs && isF(flags, idx - SY(d))) v[1] = by;
        if (!d.is3d) {
          v[2] = OG_R(0.);
        } else {
          if (k > 0 && isO(flags, idx - SZ(d))) v[2] = bz;
          if (k > 0 && curObs && isF(flags, idx - SZ(d))) v[2] = bz;
        }
        if (curFluid) {
          if ((i > 0 && isStk(flags, idx - 1)) || (i < d.nx - 1 && isStk(flags, idx + 1))) v[1] = v[2] = OG_R(0.);
          if ((j > 0 && isStk(flags, idx - SY(d))) || (j < d.ny - 1 && isStk(flags, idx + SY(d)))) v[0] = v[2] = OG_R(0.);
          if (d.is3d && ((k > 0 && isStk(flags, idx - SZ(d))) || (k < d.nz - 1 && isStk(flags, idx + SZ(d))))) v[0] = v[1] = OG_R(0.);
        }
      }
}

/* addBuoyancy (:83-87) -> KnAddBuoyancy (:72-80).  The increment
 * (0.5*s)*(rho+rho') is formed in double and added in double. */
void og_add_buoyancy(og_dims d, const int* flags, const og_real* density, og_real* vel, og_real gx, og_real gy, og_real gz,
                     og_real coefficient, int scale, og_real dt) {
  const og_real dx = (og_real)(1.0 / (double)imax(d.nx, imax(d.ny, d.nz)));
  const og_real gridScale = scale ? dx : OG_R(1.);
  const og_real fx = ((-gx) * dt) / gridScale * coefficient;
  const og_real fy = ((-gy) * dt) / gridScale * coefficient;
  const og_real fz = ((-gz) * dt) / gridScale * coefficient;
  int k;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        if (!isF(flags, idx)) continue;
        og_real* v = vel + 3 * idx;
        if (isF(flags, idx - 1))
          v[0] = (og_real)((double)v[0] + (0.5 * fx) * (double)(density[idx] + density[idx - 1]));
        if (isF(flags, idx - SY(d)))
          v[1] = (og_real)((double)v[1] + (0.5 * fy) * (double)(density[idx] + density[idx - SY(d)]));
        if (d.is3d && isF(flags, idx - SZ(d)))
          v[2] = (og_real)((double)v[2] + (0.5 * fz) * (double)(density[idx] + density[idx - SZ(d)]));
      }
}

/* addGravity (:61-65) -> KnApplyForce (:46-58), additive */
void og_add_gravity(og_dims d, const int* flags, og_real* vel, og_real gx, og_real gy, og_real gz, const og_real* exclude,
                    int scale, og_real dt) {
  const og_real dx = (og_real)(1.0 / (double)imax(d.nx, imax(d.ny, d.nz)));
  const og_real gridScale = scale ? dx : OG_R(1.);
  const og_real fx = (gx * dt) / gridScale, fy = (gy * dt) / gridScale, fz = (gz * dt) / gridScale;
  int k;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        const int curFluid = isF(flags, idx), curEmpty = isE(flags, idx);
        if (!curFluid && !curEmpty) continue;
        if (exclude && (exclude[idx] < 0.)) continue;
        og_real* v = vel + 3 * idx;
        if (isF(flags, idx - 1) || (curFluid && isE(flags, idx - 1))) v[0] = v[0] + fx;
        if (isF(flags, idx - SY(d)) || (curFluid && isE(flags, idx - SY(d)))) v[1] = v[1] + fy;
        if (d.is3d && (isF(flags, idx - SZ(d)) || (curFluid && isE(flags, idx - SZ(d))))) v[2] = v[2] + fz;
      }
}

/* extrapolateMACSimple (fastmarch.cpp:337-375) with knExtrapolateMACSimple
 * (:230-258, in place: a cell reads neighbours of layer d only, so the
 * in-place update is order independent) and knExtrapolateIntoBnd (:260-300) */
/* knUnprojectNormalComp (fastmarch.cpp:316-330) with getNormal (:298-314)
 * and normalize (util/vectorbase.h:416-429) */
static void unproject_normal_comp(og_dims d, og_real* vel, const og_real* phi, og_real maxDist) {
  for (int k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        if (phi[idx] > 0. || phi[idx] < -maxDist) continue;
        int ii = i, jj = j, kk = k, kd = 1;
        if (ii > d.nx - 2) ii = d.nx - 2;
        if (ii < 1) ii = 1;
        if (jj > d.ny - 2) jj = d.ny - 2;
        if (jj < 1) jj = 1;
        if (d.is3d) {
          if (kk > d.nz - 2) kk = d.nz - 2;
          if (kk < 1) kk = 1;
        } else {
          kd = 0;
        }
        og_real n[3] = {phi[IX(d, ii + 1, jj, kk)] - phi[IX(d, ii - 1, jj, kk)],
                        phi[IX(d, ii, jj + 1, kk)] - phi[IX(d, ii, jj - 1, kk)],
                        phi[IX(d, ii, jj, kk + kd)] - phi[IX(d, ii, jj, kk - kd)]};
        og_real* v = vel + 3 * idx;
        if (n[0] * v[0] + n[1] * v[1] + n[2] * v[2] < 0.) {
          const og_real l = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
          const og_real eps2 = OG_R(OG_VEC_EPS) * OG_R(OG_VEC_EPS);
          if (fabs(l - 1.) < eps2) {
          } else if (l > eps2) {
            const og_real norm = og_sqrt(l);
            const og_real sc = (og_real)(1. / (double)norm);
            for (int c = 0; c < 3; c++) n[c] *= sc;
          } else {
            n[0] = n[1] = n[2] = OG_R(0.);
          }
          const og_real dl = n[0] * v[0] + n[1] * v[1] + n[2] * v[2];
          for (int c = 0; c < 3; c++) v[c] -= n[c] * dl;
        }
      }
}

void og_extrapolate_mac_simple(og_dims d, const int* flags, og_real* vel, int distance, const og_real* phiObs,
                               int intoObs) {
  const ll n = NCELL(d);
  int* tmp = (int*)malloc(sizeof(int) * (size_t)n);
  const int dim = d.is3d ? 3 : 2;
  const ll st[3] = {1, SY(d), SZ(d)};
  for (int c = 0; c < dim; c++) {
    memset(tmp, 0, sizeof(int) * (size_t)n);
    for (int k = KLO(d, 1); k < KHI(d, 1); k++)
      for (int j = 1; j < d.ny - 1; j++)
        for (int i = 1; i < d.nx - 1; i++) {
          const ll idx = IX(d, i, j, k), nb = idx - st[c];
          int mark = 0;
          if (!intoObs) {
            if (isF(flags, idx) || isF(flags, nb)) mark = 1;
          } else {
            if ((isF(flags, idx) || isF(flags, nb)) && !isO(flags, idx) && !isO(flags, nb)) mark = 1;
          }
          if (mark) tmp[idx] = 1;
        }
    for (int dd = 1; dd < 1 + distance; dd++) {
      for (int k = KLO(d, 1); k < KHI(d, 1); k++)
        for (int j = 1; j < d.ny - 1; j++)
          for (int i = 1; i < d.nx - 1; i++) {
            const ll idx = IX(d, i, j, k);
            if (tmp[idx] != 0) continue;
            const ll nbo[6] = {1, -1, SY(d), -SY(d), SZ(d), -SZ(d)};
            int nbs = 0;
            og_real avg = OG_R(0.);
            for (int q = 0; q < 2 * dim; q++)
              if (tmp[idx + nbo[q]] == dd) { avg += vel[3 * (idx + nbo[q]) + c]; nbs++; }
            if (nbs > 0) {
              tmp[idx] = dd + 1;
              vel[3 * idx + c] = avg / (og_real)nbs;
            }
          }
    }
  }
  if (phiObs) unproject_normal_comp(d, vel, phiObs, (og_real)distance);
  /* copy tangential values into the domain sides from a snapshot */
  og_real* vt = (og_real*)malloc(sizeof(og_real) * 3 * (size_t)n);
  memcpy(vt, vel, sizeof(og_real) * 3 * (size_t)n);
  for (int k = 0; k < d.nz; k++)
    for (int j = 0; j < d.ny; j++)
      for (int i = 0; i < d.nx; i++) {
        const ll idx = IX(d, i, j, k);
        int cc = 0;
        og_real v[3] = {OG_R(0.), OG_R(0.), OG_R(0.)};
        const int obs = isO(flags, idx);
#define TAKE(e) do { v[0] = vt[3 * (e)]; v[1] = vt[3 * (e) + 1]; v[2] = vt[3 * (e) + 2]; } while (0)
        if (i == 0) { TAKE(idx + 1); if (obs && v[0] < OG_R(0.)) v[0] = OG_R(0.); cc++; }
        else if (i == d.nx - 1) { TAKE(idx - 1); if (obs && v[0] > OG_R(0.)) v[0] = OG_R(0.); cc++; }
        if (j == 0) { TAKE(idx + SY(d)); if (obs && v[1] < OG_R(0.)) v[1] = OG_R(0.); cc++; }
        else if (j == d.ny - 1) { TAKE(idx - SY(d)); if (obs && v[1] > OG_R(0.)) v[1] = OG_R(0.); cc++; }
        if (d.is3d) {
          if (k == 0) { TAKE(idx + SZ(d)); if (obs && v[2] < OG_R(0.)) v[2] = OG_R(0.); cc++; }
          else if (k == d.nz - 1) { TAKE(idx - SZ(d)); if (obs && v[2] > OG_R(0.)) v[2] = OG_R(0.); cc++; }
        }
#undef TAKE
        if (cc > 0) {
          vel[3 * idx] = v[0] / (og_real)cc; vel[3 * idx + 1] = v[1] / (og_real)cc; vel[3 * idx + 2] = v[2] / (og_real)cc;
        }
      }
  free(vt);
  free(tmp);
}

/* extrapolateLsSimple (fastmarch.cpp:470-507): mark the inside (phi < 0, or
 * phi > 0 with inside), the first layer around it (tmp = 2, values kept),
 * then layers d = 2..distance by knExtrapolateLsSimple (:443-461; a cell
 * reads only neighbours of layer d, so the in-place pass is order
 * independent: avg over +x,-x,+y,-y,+z,-z in float, then avg / nbs +
 * direction), and knSetRemaining (:464-468) for cells never reached.  All
 * passes skip the outermost layer (bnd = 1). */
void og_extrapolate_ls_simple(og_dims d, og_real* phi, int distance, int inside) {
  const ll n = NCELL(d);
  int* tmp = (int*)calloc((size_t)n, sizeof(int));
  const int dim = d.is3d ? 3 : 2;
  const og_real direction = inside ? OG_R(-1.) : OG_R(1.);
  const ll nbo[6] = {1, -1, SY(d), -SY(d), SZ(d), -SZ(d)};
  for (int k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        if (inside ? phi[idx] > OG_R(0.) : phi[idx] < OG_R(0.)) tmp[idx] = 1;
      }
  for (int k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        if (tmp[idx]) continue;
        for (int q = 0; q < 2 * dim; q++)
          if (tmp[idx + nbo[q]] == 1) { tmp[idx] = 2; break; }
      }
  for (int dd = 2; dd < 1 + distance; dd++)
    for (int k = KLO(d, 1); k < KHI(d, 1); k++)
      for (int j = 1; j < d.ny - 1; j++)
        for (int i = 1; i < d.nx - 1; i++) {
          const ll idx = IX(d, i, j, k);
          if (tmp[idx] != 0) continue;
          int nbs = 0;
          og_real avg = OG_R(0.);
          for (int q = 0; q < 2 * dim; q++)
            if (tmp[idx + nbo[q]] == dd) { avg += phi[idx + nbo[q]]; nbs++; }
          if (nbs > 0) {
            tmp[idx] = dd + 1;
            phi[idx] = avg / (og_real)nbs + direction;
          }
        }
  const og_real rem = (og_real)(direction * (og_real)(distance + 2));
  for (int k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        if (tmp[idx] == 0) phi[idx] = rem;
      }
  free(tmp);
}

/* ------------------------------------------------------------------------ */
/* Pressure projection, plugin/pressure.cpp + conjugategrad.*               */

/* thetaHelper / ghostFluidHelper (pressure.cpp:115-128) */
static inline og_real theta_helper(og_real inside, og_real outside) {
  const og_real denom = inside - outside;
  if (denom > -1e-04) return OG_R(0.5);
  og_real r = inside / denom;
  if (r > OG_R(1.)) r = OG_R(1.);
  if (r < OG_R(0.)) r = OG_R(0.);
  return r;
}
static inline og_real gf_helper(const og_real* phi, ll idx, ll off, og_real gfClamp) {
  og_real alpha = theta_helper(phi[idx], phi[idx + off]);
  if (alpha < gfClamp) return gfClamp;
  return (og_real)(1. - (1. / (double)alpha));
}
static inline og_real surf_tens_helper(const og_real* phi, const og_real* curv, ll idx, ll off, og_real surfTens, og_real gfClamp) {
  return surfTens * (curv[idx + off] - gf_helper(phi, idx, off, gfClamp) * curv[idx]);
}

/* Face fractions and obstacle velocity of the next MakeRhs /
 * MakeLaplaceMatrix (MAC grids in the reference layout, or NULL): set
 * around a call, test infrastructure only. */
static const og_real* g_fractions = NULL;
static const og_real* g_obvel = NULL;
void og_set_fractions(const og_real* fractions, const og_real* obvel) {
  g_fractions = fractions;
  g_obvel = obvel;
}

/* MakeRhs (pressure.cpp:32-84); returns sum, cnt */
static void make_rhs(og_dims d, const int* flags, og_real* rhs, const og_real* vel, const og_real* perCellCorr,
                     const og_real* phi, const og_real* curv, og_real surfTens, og_real gfClamp, double* sumOut, int* cntOut) {
  double sum = 0;
  int cnt = 0;
  const ll X = 1, Y = SY(d), Z = SZ(d);
  for (int k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        if (!isF(flags, idx)) { rhs[idx] = OG_R(0.); continue; }
        og_real set;
        if (!g_fractions) {
          set = vel[3 * idx] - vel[3 * (idx + X)] + vel[3 * idx + 1] - vel[3 * (idx + Y) + 1];
          if (d.is3d) set += vel[3 * idx + 2] - vel[3 * (idx + Z) + 2];
        } else {
          const og_real* f = g_fractions;
          set = f[3 * idx] * vel[3 * idx] - f[3 * (idx + X)] * vel[3 * (idx + X)] + f[3 * idx + 1] * vel[3 * idx + 1] -
                f[3 * (idx + Y) + 1] * vel[3 * (idx + Y) + 1];
          if (d.is3d) set += f[3 * idx + 2] * vel[3 * idx + 2] - f[3 * (idx + Z) + 2] * vel[3 * (idx + Z) + 2];
          if (g_obvel) {
            const og_real* o = g_obvel;
            set += (1 - f[3 * idx]) * o[3 * idx] - (1 - f[3 * (idx + X)]) * o[3 * (idx + X)] +
                   (1 - f[3 * idx + 1]) * o[3 * idx + 1] - (1 - f[3 * (idx + Y) + 1]) * o[3 * (idx + Y) + 1];
            if (d.is3d) set += (1 - f[3 * idx + 2]) * o[3 * idx + 2] - (1 - f[3 * (idx + Z) + 2]) * o[3 * (idx + Z) + 2];
          }
        }
        if (phi && curv) {
          if (isE(flags, idx - X)) set += surf_tens_helper(phi, curv, idx, -X, surfTens, gfClamp);
          if (isE(flags, idx + X)) set += surf_tens_helper(phi, curv, idx, +X, surfTens, gfClamp);
          if (isE(flags, idx - Y)) set += surf_tens_helper(phi, curv, idx, -Y, surfTens, gfClamp);
          if (isE(flags, idx + Y)) set += surf_tens_helper(phi, curv, idx, +Y, surfTens, gfClamp);
          if (d.is3d) {
            if (isE(flags, idx - Z)) set += surf_tens_helper(phi, curv, idx, -Z, surfTens, gfClamp);
            if (isE(flags, idx + Z)) set += surf_tens_helper(phi, curv, idx, +Z, surfTens, gfClamp);
          }
        }
        if (perCellCorr) set += perCellCorr[idx];
        sum += set;
        cnt++;
        rhs[idx] = set;
      }
  *sumOut = sum;
  *cntOut = cnt;
}

void og_compute_pressure_rhs(og_dims d, og_real* rhs, const og_real* vel, const int* flags, const og_real* phi,
                             const og_real* perCellCorr, const og_real* curv, const og_pressure_params* p) {
  double sum;
  int cnt;
  make_rhs(d, flags, rhs, vel, perCellCorr, phi, curv, p->surfTens, p->gfClamp, &sum, &cnt);
  if (p->enforceCompatibility) {
    const og_real add = (og_real)(-sum / (double)(og_real)cnt);
    const ll n = NCELL(d);
    for (ll idx = 0; idx < n; idx++) rhs[idx] += add;
  }
}

/* MakeLaplaceMatrix (conjugategrad.h:154-187), no fractions; A* zeroed */
void og_make_laplace_matrix(og_dims d, const int* flags, og_real* A0, og_real* Ai, og_real* Aj, og_real* Ak) {
  const ll n = NCELL(d);
  memset(A0, 0, sizeof(og_real) * n); memset(Ai, 0, sizeof(og_real) * n);
  memset(Aj, 0, sizeof(og_real) * n); memset(Ak, 0, sizeof(og_real) * n);
  const ll X = 1, Y = SY(d), Z = SZ(d);
  int k;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        if (!isF(flags, idx)) continue;
        if (g_fractions) {
          /* the fractions form (conjugategrad.h:172-186) */
          const og_real* f = g_fractions;
          A0[idx] += f[3 * idx];
          A0[idx] += f[3 * (idx + X)];
          A0[idx] += f[3 * idx + 1];
          A0[idx] += f[3 * (idx + Y) + 1];
          if (d.is3d) A0[idx] += f[3 * idx + 2];
          if (d.is3d) A0[idx] += f[3 * (idx + Z) + 2];
          if (isF(flags, idx + X)) Ai[idx] = -f[3 * (idx + X)];
          if (isF(flags, idx + Y)) Aj[idx] = -f[3 * (idx + Y) + 1];
          if (d.is3d && isF(flags, idx + Z)) Ak[idx] = -f[3 * (idx + Z) + 2];
          continue;
        }
        if (!isO(flags, idx - X)) A0[idx] += OG_R(1.);
        if (!isO(flags, idx + X)) A0[idx] += OG_R(1.);
        if (!isO(flags, idx - Y)) A0[idx] += OG_R(1.);
        if (!isO(flags, idx + Y)) A0[idx] += OG_R(1.);
        if (d.is3d && !isO(flags, idx - Z)) A0[idx] += OG_R(1.);
        if (d.is3d && !isO(flags, idx + Z)) A0[idx] += OG_R(1.);
        if (isF(flags, idx + X)) Ai[idx] = -OG_R(1.);
        if (isF(flags, idx + Y)) Aj[idx] = -OG_R(1.);
        if (d.is3d && isF(flags, idx + Z)) Ak[idx] = -OG_R(1.);
      }
}

/* ApplyGhostFluidDiagonal (pressure.cpp:136-151) */
void og_apply_ghost_fluid_diagonal(og_dims d, og_real* A0, const int* flags, const og_real* phi, og_real gfClamp) {
  const ll X = 1, Y = SY(d), Z = SZ(d);
  int k;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        if (!isF(flags, idx)) continue;
        if (isE(flags, idx - X)) A0[idx] -= gf_helper(phi, idx, -X, gfClamp);
        if (isE(flags, idx + X)) A0[idx] -= gf_helper(phi, idx, +X, gfClamp);
        if (isE(flags, idx - Y)) A0[idx] -= gf_helper(phi, idx, -Y, gfClamp);
        if (isE(flags, idx + Y)) A0[idx] -= gf_helper(phi, idx, +Y, gfClamp);
        if (d.is3d) {
          if (isE(flags, idx - Z)) A0[idx] -= gf_helper(phi, idx, -Z, gfClamp);
          if (isE(flags, idx + Z)) A0[idx] -= gf_helper(phi, idx, +Z, gfClamp);
        }
      }
}

/* InitPreconditionModifiedIncompCholesky2 (conjugategrad.cpp:66-97).  The
 * recurrence is lexicographic and serial in the reference. */
void og_mic_init(og_dims d, const int* flags, og_real* P, const og_real* A0, const og_real* Ai, const og_real* Aj,
                 const og_real* Ak) {
  const ll n = NCELL(d);
  memset(P, 0, sizeof(og_real) * n);
  const ll X = 1, Y = SY(d), Z = SZ(d);
  for (int k = 0; k < d.nz; k++)
    for (int j = 0; j < d.ny; j++)
      for (int i = 0; i < d.nx; i++) {
        const ll idx = IX(d, i, j, k);
        if (!isF(flags, idx)) continue;
        const og_real tau = OG_R(0.97), sigma = OG_R(0.25);
        /* neighbours outside the grid contribute nothing (the reference
         * reads out of range there; fluid never touches the border) */
        const og_real ai = i > 0 ? Ai[idx - X] : OG_R(0.), pi = i > 0 ? P[idx - X] : OG_R(0.);
        const og_real aj = j > 0 ? Aj[idx - Y] : OG_R(0.), pj = j > 0 ? P[idx - Y] : OG_R(0.);
        const og_real ak = k > 0 ? Ak[idx - Z] : OG_R(0.), pk = k > 0 ? P[idx - Z] : OG_R(0.);
        const og_real aji = i > 0 ? Aj[idx - X] : OG_R(0.), aki = i > 0 ? Ak[idx - X] : OG_R(0.);
        const og_real aij = j > 0 ? Ai[idx - Y] : OG_R(0.), akj = j > 0 ? Ak[idx - Y] : OG_R(0.);
        const og_real aik = k > 0 ? Ai[idx - Z] : OG_R(0.), ajk = k > 0 ? Aj[idx - Z] : OG_R(0.);
        og_real e = OG_R(0.);
        const og_real q1 = ai * pi, q2 = aj * pj, q3 = ak * pk;
        e = A0[idx] - q1 * q1 - q2 * q2 - q3 * q3;
        const og_real t1 = ai * (aji + aki) * (pi * pi);
        const og_real t2 = aj * (aij + akj) * (pj * pj);
        const og_real t3 = ak * (aik + ajk) * (pk * pk);
        const double s = (double)(t1 + t2 + t3) + 0.;
        e = (og_real)((double)e - (double)tau * s);
        if (e < sigma * A0[idx]) e = A0[idx];
        P[idx] = (og_real)(1. / (double)og_sqrt(e));
      }
}

/* ApplyPreconditionModifiedIncompCholesky2 (conjugategrad.cpp:135-160) */
void og_mic_apply(og_dims d, og_real* dst, const og_real* src, const int* flags, const og_real* P, const og_real* Ai,
                  const og_real* Aj, const og_real* Ak) {
  const ll X = 1, Y = SY(d), Z = SZ(d);
  for (int k = 0; k < d.nz; k++)
    for (int j = 0; j < d.ny; j++)
      for (int i = 0; i < d.nx; i++) {
        const ll idx = IX(d, i, j, k);
        if (!isF(flags, idx)) continue;
        const og_real p = P[idx];
        og_real t = src[idx];
        if (i > 0) t = t - dst[idx - X] * Ai[idx - X] * P[idx - X];
        if (j > 0) t = t - dst[idx - Y] * Aj[idx - Y] * P[idx - Y];
        if (k > 0) t = t - dst[idx - Z] * Ak[idx - Z] * P[idx - Z];
        dst[idx] = p * t;
      }
  for (int k = d.nz - 1; k >= 0; k--)
    for (int j = d.ny - 1; j >= 0; j--)
      for (int i = d.nx - 1; i >= 0; i--) {
        const ll idx = IX(d, i, j, k);
        if (!isF(flags, idx)) continue;
        const og_real p = P[idx];
        og_real t = dst[idx];
        if (i < d.nx - 1) t = t - dst[idx + X] * Ai[idx] * p;
        if (j < d.ny - 1) t = t - dst[idx + Y] * Aj[idx] * p;
        if (k < d.nz - 1) t = t - dst[idx + Z] * Ak[idx] * p;
        dst[idx] = p * t;
      }
}

/* ApplyMatrix / ApplyMatrix2D (conjugategrad.h:118-151) */
void og_apply_matrix(og_dims d, const int* flags, og_real* dst, const og_real* src, const og_real* A0, const og_real* Ai,
                     const og_real* Aj, const og_real* Ak) {
  const ll n = NCELL(d);
  const ll X = 1, Y = SY(d), Z = SZ(d);
  ll idx;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (idx = 0; idx < n; idx++) {
    if (!isF(flags, idx)) { dst[idx] = src[idx]; continue; }
    og_real v = src[idx] * A0[idx] + src[idx - X] * Ai[idx - X] + src[idx + X] * Ai[idx] + src[idx - Y] * Aj[idx - Y] +
              src[idx + Y] * Aj[idx];
    if (d.is3d) v = v + src[idx - Z] * Ak[idx - Z] + src[idx + Z] * Ak[idx];
    dst[idx] = v;
  }
}

/* GridDotProduct (conjugategrad.cpp:175-178): Real products, double sum.
 * Partials per thread are combined in thread order. */
static double dot_product(ll n, const og_real* a, const og_real* b) {
  double total = 0.;
  if (g_threads <= 1) {
    for (ll i = 0; i < n; i++) total += (a[i] * b[i]);
    return total;
  }
  double part[256];
  int nt = g_threads > 256 ? 256 : g_threads;
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    int t = omp_get_thread_num(), T = omp_get_num_threads();
#else
    int t = 0, T = 1;
#endif
    ll lo = n * t / T, hi = n * (t + 1) / T;
    double s = 0.;
    for (ll i = lo; i < hi; i++) s += (a[i] * b[i]);
    part[t] = s;
#pragma omp barrier
#pragma omp single
    {
      for (int q = 0; q < T; q++) total += part[q];
    }
  }
  return total;
}

static double sum_sqr(ll n, const og_real* a) {
  double s = 0.;
  for (ll i = 0; i < n; i++) s += (double)a[i] * (double)a[i];
  return s;
}

/* Grid<Real>::getMaxAbs (grid.cpp:319-323) */
og_real og_get_max_abs(ll n, const og_real* a) {
  og_real amin = OG_REAL_MAX, amax = -OG_REAL_MAX;
  for (ll i = 0; i < n; i++) {
    if (a[i] < amin) amin = a[i];
    if (a[i] > amax) amax = a[i];
  }
  const og_real x = og_fabs(amin), y = og_fabs(amax);
  return x > y ? x : y;
}

/* ------------------------------------------------------------------------ */
/* Multigrid preconditioner (multigrid.cpp), restated without topology
 * awareness exactly like the reference.                                     */

enum { VT_INACTIVE = 0, VT_ACTIVE = 1, VT_ACTIVE_TRIVIAL = 2, VT_REMOVED = 3, VT_ZERO = 4, VT_FREE = 5 };

typedef struct { int U[3], W[3], N[3]; int sc, sf; og_real rw, iw; int inU; } og_path;

#define MG_MAXL 32
struct og_mg {
  og_dims d;
  int nlev, is3d, dim, S, S0;
  int smin[3], smax[3];
  int size[MG_MAXL][3];
  int pitch[MG_MAXL][3];
  ll n[MG_MAXL];
  og_real* A[MG_MAXL];
  og_real* x[MG_MAXL];
  og_real* b[MG_MAXL];
  og_real* r[MG_MAXL];
  signed char* type[MG_MAXL];
  double *cg1, *cg2, *cg3, *cg4;
  og_path* paths;
  int npaths;
  int isASet;
  og_real coarseAcc, trivialScale;
};

static inline ll mg_lin(const og_mg* m, int l, const int* V) {
  return (ll)V[0] + (ll)V[1] * m->pitch[l][1] + (ll)V[2] * m->pitch[l][2];
}
static inline void mg_vec(const og_mg* m, int l, ll v, int* V) {
  const ll sx = m->size[l][0], sy = m->size[l][1];
  V[0] = (int)(v % sx);
  V[1] = (int)((v % (sx * sy)) / sx);
  V[2] = (int)(v / (sx * sy));
}
static inline int mg_in(const og_mg* m, int l, const int* V) {
  return V[0] >= 0 && V[1] >= 0 && V[2] >= 0 && V[0] < m->size[l][0] && V[1] < m->size[l][1] && V[2] < m->size[l][2];
}

/* GridMg::GridMg (multigrid.cpp:220-319) */
og_mg* og_mg_create(og_dims d) {
  og_mg* m = (og_mg*)calloc(1, sizeof(og_mg));
  m->d = d;
  m->is3d = d.nz > 1;
  m->dim = m->is3d ? 3 : 2;
  m->S = m->is3d ? 14 : 5;
  m->S0 = m->is3d ? 4 : 3;
  m->smin[0] = -1; m->smin[1] = -1; m->smin[2] = m->is3d ? -1 : 0;
  m->smax[0] = 1; m->smax[1] = 1; m->smax[2] = m->is3d ? 1 : 0;
  m->coarseAcc = OG_R(1e-8);
  m->trivialScale = OG_R(1e-6);
  m->size[0][0] = d.nx; m->size[0][1] = d.ny; m->size[0][2] = d.nz;
  int L = 1;
  ll n = (ll)d.nx * d.ny * d.nz;
  for (int l = 1; l <= 100 && l < MG_MAXL; l++) {
    if (m->size[l - 1][0] <= 5 && m->size[l - 1][1] <= 5 && m->size[l - 1][2] <= 5) break;
    if (n <= 1000) break;
    for (int c = 0; c < 3; c++) m->size[l][c] = (m->size[l - 1][c] + 2) / 2;
    n = (ll)m->size[l][0] * m->size[l][1] * m->size[l][2];
    L = l + 1;
  }
  m->nlev = L;
  for (int l = 0; l < L; l++) {
    m->pitch[l][0] = 1;
    m->pitch[l][1] = m->size[l][0];
    m->pitch[l][2] = m->size[l][0] * m->size[l][1];
    m->n[l] = (ll)m->size[l][0] * m->size[l][1] * m->size[l][2];
    m->A[l] = (og_real*)calloc((size_t)(m->n[l] * (l == 0 ? m->S0 : m->S)), sizeof(og_real));
    m->x[l] = (og_real*)calloc((size_t)m->n[l], sizeof(og_real));
    m->b[l] = (og_real*)calloc((size_t)m->n[l], sizeof(og_real));
    m->r[l] = (og_real*)calloc((size_t)m->n[l], sizeof(og_real));
    m->type[l] = (signed char*)calloc((size_t)m->n[l], 1);
  }
  const ll nc = m->n[L - 1];
  m->cg1 = (double*)calloc((size_t)nc, sizeof(double));
  m->cg2 = (double*)calloc((size_t)nc, sizeof(double));
  m->cg3 = (double*)calloc((size_t)nc, sizeof(double));
  m->cg4 = (double*)calloc((size_t)nc, sizeof(double));
  /* coarsening paths V <- U <- W <- N around reference vertex V=(1,1,1) */
  static const int p7[7][3] = {{0, 0, 0}, {-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
  m->paths = (og_path*)malloc(sizeof(og_path) * 4096);
  m->npaths = 0;
  const int V[3] = {1, 1, 1};
  int U[3];
  for (U[2] = 2 * V[2] + m->smin[2]; U[2] <= 2 * V[2] + m->smax[2]; U[2]++)
    for (U[1] = 2 * V[1] + m->smin[1]; U[1] <= 2 * V[1] + m->smax[1]; U[1]++)
      for (U[0] = 2 * V[0] + m->smin[0]; U[0] <= 2 * V[0] + m->smax[0]; U[0]++)
        for (int i = 0; i < 1 + 2 * m->dim; i++) {
          int W[3] = {U[0] + p7[i][0], U[1] + p7[i][1], U[2] + p7[i][2]};
          int N[3];
          for (N[2] = W[2] / 2; N[2] <= (W[2] + 1) / 2; N[2]++)
            for (N[1] = W[1] / 2; N[1] <= (W[1] + 1) / 2; N[1]++)
              for (N[0] = W[0] / 2; N[0] <= (W[0] + 1) / 2; N[0]++) {
                const int s = N[0] + 3 * N[1] + 9 * N[2];
                if (s >= 13) {
                  og_path* p = &m->paths[m->npaths++];
                  for (int c = 0; c < 3; c++) {
                    p->N[c] = N[c] - 1;
                    p->U[c] = U[c] - 2 * V[c];
                    p->W[c] = W[c] - 2 * V[c];
                  }
                  p->sc = s - 13;
                  p->sf = (i + 1) / 2;
                  p->inU = (i % 2 == 0);
                  p->rw = OG_R(1.) / (og_real)(1 << ((U[0] % 2) + (U[1] % 2) + (U[2] % 2)));
                  p->iw = OG_R(1.) / (og_real)(1 << ((W[0] % 2) + (W[1] % 2) + (W[2] % 2)));
                }
              }
        }
  /* same comparator and algorithm as the reference's std::sort call, so
   * paths with equal keys land in the same order */
  std::sort(m->paths, m->paths + m->npaths, [](const og_path& p1, const og_path& p2) {
    if (p1.sc == p2.sc)
      return (p1.U[0] + 1) + 3 * (p1.U[1] + 1) + 9 * (p1.U[2] + 1) < (p2.U[0] + 1) + 3 * (p2.U[1] + 1) + 9 * (p2.U[2] + 1);
    return p1.sc < p2.sc;
  });
  return m;
}

void og_mg_destroy(og_mg* m) {
  if (!m) return;
  for (int l = 0; l < m->nlev; l++) {
    free(m->A[l]); free(m->x[l]); free(m->b[l]); free(m->r[l]); free(m->type[l]);
  }
  free(m->cg1); free(m->cg2); free(m->cg3); free(m->cg4);
  free(m->paths);
  free(m);
}

int og_mg_num_levels(const og_mg* m) { return m->nlev; }
void og_mg_level_size(const og_mg* m, int l, int* sz) { sz[0] = m->size[l][0]; sz[1] = m->size[l][1]; sz[2] = m->size[l][2]; }
const signed char* og_mg_level_types(const og_mg* m, int l) { return m->type[l]; }
const og_real* og_mg_level_matrix(const og_mg* m, int l) { return m->A[l]; }

/* NKMinHeap (multigrid.cpp:59-203): bucket lists, head insertion */
typedef struct { int key, prev, next; } hentry;
typedef struct { int N, K, size, minKey; hentry* e; } nkheap;

static void heap_init(nkheap* h, int N, int K) {
  h->N = N; h->K = K; h->size = 0; h->minKey = -1;
  h->e = (hentry*)malloc(sizeof(hentry) * (size_t)(N + K));
  for (int i = 0; i < N + K; i++) { h->e[i].key = -1; h->e[i].prev = -1; h->e[i].next = -1; }
}
static void heap_set_key(nkheap* h, int ID, int key) {
  const int kid = h->K + ID;
  if (h->e[kid].key == key) return;
  if (h->e[kid].key != -1) {
    int pred = h->e[kid].prev, succ = h->e[kid].next;
    h->e[pred].next = succ;
    if (succ != -1) h->e[succ].prev = pred;
    int removedKey = h->e[kid].key;
    if (removedKey == h->minKey) {
      if (h->size == 1) h->minKey = -1;
      else for (; h->minKey < h->K; h->minKey++) if (h->e[h->minKey].next != -1) break;
    }
    h->size--;
  }
  h->e[kid].key = key;
  if (key == -1) { h->e[kid].next = h->e[kid].prev = -1; return; }
  h->size++;
  if (h->minKey == -1) h->minKey = key;
  else h->minKey = h->minKey < key ? h->minKey : key;
  int tmp = h->e[key].next;
  h->e[key].next = kid;
  h->e[kid].prev = key;
  h->e[kid].next = tmp;
  if (tmp != -1) h->e[tmp].prev = kid;
}
static int heap_pop_min(nkheap* h) {
  if (h->size == 0) return -1;
  const int kid = h->e[h->minKey].next;
  const int ID = kid - h->K;
  int pred = h->e[kid].prev, succ = h->e[kid].next;
  h->e[pred].next = succ;
  if (succ != -1) h->e[succ].prev = pred;
  h->e[kid].key = -1; h->e[kid].prev = -1; h->e[kid].next = -1;
  h->size--;
  if (h->size == 0) h->minKey = -1;
  else for (; h->minKey < h->K; h->minKey++) if (h->e[h->minKey].next != -1) break;
  return ID;
}

/* GridMg::genCoarseGrid (multigrid.cpp:520-578) */
static void mg_gen_coarse_grid(og_mg* m, int l) {
  for (ll i = 0; i < m->n[l]; i++) m->type[l][i] = VT_FREE;
  nkheap h;
  heap_init(&h, (int)m->n[l - 1], m->is3d ? 9 : 5);
  for (ll v = 0; v < m->n[l - 1]; v++) {
    if (m->type[l - 1][v] != VT_INACTIVE) {
      int V[3];
      mg_vec(m, l - 1, v, V);
      heap_set_key(&h, (int)v, 1 << ((V[0] % 2) + (V[1] % 2) + (V[2] % 2)));
    }
  }
  while (h.size > 0) {
    const int v = heap_pop_min(&h);
    int V[3];
    mg_vec(m, l - 1, v, V);
    int vdone = 0;
    int I[3];
    for (I[2] = V[2] / 2; I[2] <= (V[2] + 1) / 2; I[2]++)
      for (I[1] = V[1] / 2; I[1] <= (V[1] + 1) / 2; I[1]++)
        for (I[0] = V[0] / 2; I[0] <= (V[0] + 1) / 2; I[0]++) {
          const ll i = mg_lin(m, l, I);
          if (m->type[l][i] == VT_FREE) {
            if (vdone) m->type[l][i] = VT_REMOVED;
            else { m->type[l][i] = VT_ZERO; vdone = 1; }
            int lo[3], hi[3], R[3];
            for (int c = 0; c < 3; c++) { lo[c] = imax(0, I[c] * 2 - 1); hi[c] = imin(m->size[l - 1][c] - 1, I[c] * 2 + 1); }
            for (R[2] = lo[2]; R[2] <= hi[2]; R[2]++)
              for (R[1] = lo[1]; R[1] <= hi[1]; R[1]++)
                for (R[0] = lo[0]; R[0] <= hi[0]; R[0]++) {
                  const int r = (int)mg_lin(m, l - 1, R);
                  const int key = h.e[h.K + r].key;
                  if (key > 1) heap_set_key(&h, r, key - 1);
                  else if (key > -1) heap_set_key(&h, r, -1);
                }
          }
        }
  }
  free(h.e);
  for (ll i = 0; i < m->n[l]; i++) {
    if (m->type[l][i] == VT_FREE) m->type[l][i] = VT_REMOVED;
    if (m->type[l][i] == VT_ZERO) m->type[l][i] = VT_ACTIVE;
    if (m->type[l][i] == VT_REMOVED) m->type[l][i] = VT_INACTIVE;
  }
}

/* knGenCoarseGridOperator (multigrid.cpp:580-657) */
static void mg_gen_coarse_op(og_mg* m, int l) {
  const int S = m->S, S0 = m->S0;
  ll idx;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (idx = 0; idx < m->n[l]; idx++) {
    if (m->type[l][idx] == VT_INACTIVE) continue;
    og_real* A = m->A[l] + idx * S;
    for (int i = 0; i < S; i++) A[i] = OG_R(0.);
    int V[3];
    mg_vec(m, l, idx, V);
    if (l == 1) {
      for (int q = 0; q < m->npaths; q++) {
        const og_path* p = &m->paths[q];
        int N[3] = {V[0] + p->N[0], V[1] + p->N[1], V[2] + p->N[2]};
        if (!mg_in(m, l, N)) continue;
        if (m->type[l][mg_lin(m, l, N)] == VT_INACTIVE) continue;
        int U[3] = {2 * V[0] + p->U[0], 2 * V[1] + p->U[1], 2 * V[2] + p->U[2]};
        if (!mg_in(m, l - 1, U)) continue;
        const ll u = mg_lin(m, l - 1, U);
        if (m->type[l - 1][u] == VT_INACTIVE) continue;
        int W[3] = {2 * V[0] + p->W[0], 2 * V[1] + p->W[1], 2 * V[2] + p->W[2]};
        if (!mg_in(m, l - 1, W)) continue;
        const ll w = mg_lin(m, l - 1, W);
        if (m->type[l - 1][w] == VT_INACTIVE) continue;
        if (p->inU) A[p->sc] += p->rw * m->A[l - 1][u * S0 + p->sf] * p->iw;
        else A[p->sc] += p->rw * m->A[l - 1][w * S0 + p->sf] * p->iw;
      }
    } else {
      int ulo[3], uhi[3], U[3];
      for (int c = 0; c < 3; c++) { ulo[c] = imax(0, V[c] * 2 - 1); uhi[c] = imin(m->size[l - 1][c] - 1, V[c] * 2 + 1); }
      for (U[2] = ulo[2]; U[2] <= uhi[2]; U[2]++)
        for (U[1] = ulo[1]; U[1] <= uhi[1]; U[1]++)
          for (U[0] = ulo[0]; U[0] <= uhi[0]; U[0]++) {
            const ll u = mg_lin(m, l - 1, U);
            if (m->type[l - 1][u] == VT_INACTIVE) continue;
            const og_real rw = OG_R(1.) / (og_real)(1 << ((U[0] % 2) + (U[1] % 2) + (U[2] % 2)));
            int nlo[3], nhi[3], N[3];
            for (int c = 0; c < 3; c++) { nlo[c] = (U[c] - 1) / 2; nhi[c] = imin(m->size[l][c] - 1, (U[c] + 2) / 2); }
            for (N[2] = nlo[2]; N[2] <= nhi[2]; N[2]++)
              for (N[1] = nlo[1]; N[1] <= nhi[1]; N[1]++)
                for (N[0] = nlo[0]; N[0] <= nhi[0]; N[0]++) {
                  const ll nn = mg_lin(m, l, N);
                  if (m->type[l][nn] == VT_INACTIVE) continue;
                  const int sc = (N[0] - V[0] + m->smax[0]) + 3 * (N[1] - V[1] + m->smax[1]) + 9 * (N[2] - V[2] + m->smax[2]);
                  if (sc < S - 1) continue;
                  int wlo[3], whi[3], W[3];
                  for (int c = 0; c < 3; c++) {
                    wlo[c] = imax(0, imax(U[c] - 1, N[c] * 2 - 1));
                    whi[c] = imin(m->size[l - 1][c] - 1, imin(U[c] + 1, N[c] * 2 + 1));
                  }
                  for (W[2] = wlo[2]; W[2] <= whi[2]; W[2]++)
                    for (W[1] = wlo[1]; W[1] <= whi[1]; W[1]++)
                      for (W[0] = wlo[0]; W[0] <= whi[0]; W[0]++) {
                        const ll w = mg_lin(m, l - 1, W);
                        if (m->type[l - 1][w] == VT_INACTIVE) continue;
                        const int sf = (W[0] - U[0] + m->smax[0]) + 3 * (W[1] - U[1] + m->smax[1]) + 9 * (W[2] - U[2] + m->smax[2]);
                        const og_real iw = OG_R(1.) / (og_real)(1 << ((W[0] % 2) + (W[1] % 2) + (W[2] % 2)));
                        if (sf < S) A[sc - S + 1] += rw * m->A[l - 1][w * S + S - 1 - sf] * iw;
                        else A[sc - S + 1] += rw * m->A[l - 1][u * S + sf - S + 1] * iw;
                      }
                }
          }
    }
  }
}

/* GridMg::setA (multigrid.cpp:386-415) with knCopyA/knActivateVertices */
static void mg_set_a(og_mg* m, const og_real* A0, const og_real* Ai, const og_real* Aj, const og_real* Ak) {
  const int S0 = m->S0;
  const ll n = m->n[0];
  for (ll v = 0; v < n; v++) {
    m->A[0][v * S0 + 0] = A0[v];
    m->A[0][v * S0 + 1] = Ai[v];
    m->A[0][v * S0 + 2] = Aj[v];
    if (m->is3d) m->A[0][v * S0 + 3] = Ak[v];
  }
  for (ll v = 0; v < n; v++) {
    m->type[0][v] = VT_INACTIVE;
    if (m->A[0][v * S0 + 0] != OG_R(0.)) {
      m->type[0][v] = VT_ACTIVE;
      int V[3];
      mg_vec(m, 0, v, V);
      og_real a[7];
      a[0] = m->A[0][v * S0 + 0];
      a[1] = m->A[0][v * S0 + 1];
      a[2] = m->A[0][v * S0 + 2];
      a[3] = m->is3d ? m->A[0][v * S0 + 3] : OG_R(0.);
      a[4] = V[0] != 0 ? m->A[0][(v - m->pitch[0][0]) * S0 + 1] : OG_R(0.);
      a[5] = V[1] != 0 ? m->A[0][(v - m->pitch[0][1]) * S0 + 2] : OG_R(0.);
      a[6] = (V[2] != 0 && m->is3d) ? m->A[0][(v - m->pitch[0][2]) * S0 + 3] : OG_R(0.);
      const int trivial = a[0] == OG_R(1.) && a[1] == OG_R(0.) && a[2] == OG_R(0.) && a[3] == OG_R(0.) && a[4] == OG_R(0.) && a[5] == OG_R(0.) && a[6] == OG_R(0.);
      if (trivial) {
        m->type[0][v] = VT_ACTIVE_TRIVIAL;
        m->A[0][v * S0 + 0] *= m->trivialScale;
      }
    }
  }
  for (int l = 1; l < m->nlev; l++) {
    mg_gen_coarse_grid(m, l);
    mg_gen_coarse_op(m, l);
  }
  m->isASet = 1;
}

/* knSmoothColor + smoothGS (multigrid.cpp:668-737) */
static void mg_smooth(og_mg* m, int l, int reversed) {
  static const int a[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
  int colors[8][4], ncol[8], nc;
  if (m->is3d) {
    if (l == 0) {
      nc = 2;
      int c0[4] = {0, 3, 5, 6}, c1[4] = {1, 2, 4, 7};
      for (int q = 0; q < 4; q++) { colors[0][q] = c0[q]; colors[1][q] = c1[q]; }
      ncol[0] = ncol[1] = 4;
    } else {
      nc = 8;
      for (int q = 0; q < 8; q++) { colors[q][0] = q; ncol[q] = 1; }
    }
  } else {
    if (l == 0) {
      nc = 2;
      colors[0][0] = 0; colors[0][1] = 3; colors[1][0] = 1; colors[1][1] = 2;
      ncol[0] = ncol[1] = 2;
    } else {
      nc = 4;
      for (int q = 0; q < 4; q++) { colors[q][0] = q; ncol[q] = 1; }
    }
  }
  const int bs[3] = {(m->size[l][0] + 1) / 2, (m->size[l][1] + 1) / 2, (m->size[l][2] + 1) / 2};
  const ll nb = (ll)bs[0] * bs[1] * bs[2];
  const int S = m->S, S0 = m->S0;
  og_real* x = m->x[l];
  for (int cc = 0; cc < nc; cc++) {
    const int color = reversed ? nc - 1 - cc : cc;
    ll bi;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (bi = 0; bi < nb; bi++) {
      const int bo[3] = {(int)(bi % bs[0]), (int)((bi % ((ll)bs[0] * bs[1])) / bs[0]), (int)(bi / ((ll)bs[0] * bs[1]))};
      for (int o = 0; o < ncol[color]; o++) {
        const int* off = a[colors[color][o]];
        int V[3] = {bo[0] * 2 + off[0], bo[1] * 2 + off[1], bo[2] * 2 + off[2]};
        if (!mg_in(m, l, V)) continue;
        const ll v = mg_lin(m, l, V);
        if (m->type[l][v] == VT_INACTIVE) continue;
        og_real sum = m->b[l][v];
        if (l == 0) {
          for (int dd = 0; dd < m->dim; dd++) {
            if (V[dd] > 0) { const ll nn = v - m->pitch[0][dd]; sum -= m->A[0][nn * S0 + dd + 1] * x[nn]; }
            if (V[dd] < m->size[0][dd] - 1) { const ll nn = v + m->pitch[0][dd]; sum -= m->A[0][v * S0 + dd + 1] * x[nn]; }
          }
          x[v] = sum / m->A[0][v * S0 + 0];
        } else {
          int s = 0, Sv[3];
          for (Sv[2] = m->smin[2]; Sv[2] <= m->smax[2]; Sv[2]++)
            for (Sv[1] = m->smin[1]; Sv[1] <= m->smax[1]; Sv[1]++)
              for (Sv[0] = m->smin[0]; Sv[0] <= m->smax[0]; Sv[0]++, s++) {
                if (s == S - 1) continue;
                int N[3] = {V[0] + Sv[0], V[1] + Sv[1], V[2] + Sv[2]};
                if (!mg_in(m, l, N)) continue;
                const ll nn = mg_lin(m, l, N);
                if (m->type[l][nn] == VT_INACTIVE) continue;
                if (s < S) sum -= m->A[l][nn * S + S - 1 - s] * x[nn];
                else sum -= m->A[l][v * S + s - S + 1] * x[nn];
              }
          x[v] = sum / m->A[l][v * S + 0];
        }
      }
    }
  }
}

/* knCalcResidual (multigrid.cpp:739-771) */
static void mg_residual(og_mg* m, int l) {
  const int S = m->S, S0 = m->S0;
  const og_real* x = m->x[l];
  ll idx;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (idx = 0; idx < m->n[l]; idx++) {
    if (m->type[l][idx] == VT_INACTIVE) continue;
    int V[3];
    mg_vec(m, l, idx, V);
    og_real sum = m->b[l][idx];
    if (l == 0) {
      for (int dd = 0; dd < m->dim; dd++) {
        if (V[dd] > 0) { const ll nn = idx - m->pitch[0][dd]; sum -= m->A[0][nn * S0 + dd + 1] * x[nn]; }
        if (V[dd] < m->size[0][dd] - 1) { const ll nn = idx + m->pitch[0][dd]; sum -= m->A[0][idx * S0 + dd + 1] * x[nn]; }
      }
      sum -= m->A[0][idx * S0 + 0] * x[idx];
    } else {
      int s = 0, Sv[3];
      for (Sv[2] = m->smin[2]; Sv[2] <= m->smax[2]; Sv[2]++)
        for (Sv[1] = m->smin[1]; Sv[1] <= m->smax[1]; Sv[1]++)
          for (Sv[0] = m->smin[0]; Sv[0] <= m->smax[0]; Sv[0]++, s++) {
            int N[3] = {V[0] + Sv[0], V[1] + Sv[1], V[2] + Sv[2]};
            if (!mg_in(m, l, N)) continue;
            const ll nn = mg_lin(m, l, N);
            if (m->type[l][nn] == VT_INACTIVE) continue;
            if (s < S) sum -= m->A[l][nn * S + S - 1 - s] * x[nn];
            else sum -= m->A[l][idx * S + s - S + 1] * x[nn];
          }
    }
    m->r[l][idx] = sum;
  }
}

/* knRestrict (multigrid.cpp:904-927) */
static void mg_restrict(og_mg* m, int ld) {
  const int ls = ld - 1;
  ll idx;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (idx = 0; idx < m->n[ld]; idx++) {
    if (m->type[ld][idx] == VT_INACTIVE) continue;
    int V[3], lo[3], hi[3], R[3];
    mg_vec(m, ld, idx, V);
    for (int c = 0; c < 3; c++) { lo[c] = imax(0, V[c] * 2 - 1); hi[c] = imin(m->size[ls][c] - 1, V[c] * 2 + 1); }
    og_real sum = OG_R(0.);
    for (R[2] = lo[2]; R[2] <= hi[2]; R[2]++)
      for (R[1] = lo[1]; R[1] <= hi[1]; R[1]++)
        for (R[0] = lo[0]; R[0] <= hi[0]; R[0]++) {
          const ll r = mg_lin(m, ls, R);
          if (m->type[ls][r] == VT_INACTIVE) continue;
          const og_real rw = OG_R(1.) / (og_real)(1 << ((R[0] % 2) + (R[1] % 2) + (R[2] % 2)));
          sum += rw * m->r[ls][r];
        }
    m->b[ld][idx] = sum;
  }
}

/* knInterpolate (multigrid.cpp:934-954): dst = r[ld] */
static void mg_interpolate(og_mg* m, int ld) {
  const int ls = ld + 1;
  ll idx;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (idx = 0; idx < m->n[ld]; idx++) {
    if (m->type[ld][idx] == VT_INACTIVE) continue;
    int V[3], I[3];
    mg_vec(m, ld, idx, V);
    og_real sum = OG_R(0.);
    for (I[2] = V[2] / 2; I[2] <= (V[2] + 1) / 2; I[2]++)
      for (I[1] = V[1] / 2; I[1] <= (V[1] + 1) / 2; I[1]++)
        for (I[0] = V[0] / 2; I[0] <= (V[0] + 1) / 2; I[0]++) {
          const ll i = mg_lin(m, ls, I);
          if (m->type[ls][i] != VT_INACTIVE) sum += m->x[ls][i];
        }
    const og_real iw = OG_R(1.) / (og_real)(1 << ((V[0] % 2) + (V[1] % 2) + (V[2] % 2)));
    m->r[ld][idx] = iw * sum;
  }
}

/* GridMg::solveCG (multigrid.cpp:793-902): Jacobi-PCG in double, serial */
static double mg_apply_stencil(og_mg* m, ll v, int l, const double* vec) {
  int V[3];
  mg_vec(m, l, v, V);
  double sum = 0;
  const int S = m->S, S0 = m->S0;
  if (l == 0) {
    for (int dd = 0; dd < m->dim; dd++) {
      if (V[dd] > 0) { const ll nn = v - m->pitch[0][dd]; sum += m->A[0][nn * S0 + dd + 1] * vec[nn]; }
      if (V[dd] < m->size[0][dd] - 1) { const ll nn = v + m->pitch[0][dd]; sum += m->A[0][v * S0 + dd + 1] * vec[nn]; }
    }
    sum += m->A[0][v * S0 + 0] * vec[v];
  } else {
    int s = 0, Sv[3];
    for (Sv[2] = m->smin[2]; Sv[2] <= m->smax[2]; Sv[2]++)
      for (Sv[1] = m->smin[1]; Sv[1] <= m->smax[1]; Sv[1]++)
        for (Sv[0] = m->smin[0]; Sv[0] <= m->smax[0]; Sv[0]++, s++) {
          int N[3] = {V[0] + Sv[0], V[1] + Sv[1], V[2] + Sv[2]};
          if (!mg_in(m, l, N)) continue;
          const ll nn = mg_lin(m, l, N);
          if (m->type[l][nn] == VT_INACTIVE) continue;
          if (s < S) sum += m->A[l][nn * S + S - 1 - s] * vec[nn];
          else sum += m->A[l][v * S + s - S + 1] * vec[nn];
        }
  }
  return sum;
}

static void mg_solve_cg(og_mg* m, int l) {
  double *z = m->cg1, *p = m->cg2, *x = m->cg3, *r = m->cg4;
  const ll n = m->n[l];
  const int S = m->S, S0 = m->S0;
  double alphaTop = 0, initialResidual = 0;
  for (ll v = 0; v < n; v++) x[v] = m->x[l][v];
  for (ll v = 0; v < n; v++) {
    if (m->type[l][v] == VT_INACTIVE) continue;
    r[v] = m->b[l][v] - mg_apply_stencil(m, v, l, x);
    if (l == 0) z[v] = r[v] / m->A[0][v * S0 + 0];
    else z[v] = r[v] / m->A[l][v * S + 0];
    initialResidual += r[v] * r[v];
    p[v] = z[v];
    alphaTop += r[v] * z[v];
  }
  initialResidual = sqrt(initialResidual);
  int iter = 0;
  const int maxIter = 10000;
  double residual = -1;
  for (; iter < maxIter && initialResidual > 1E-12; iter++) {
    double alphaBot = 0;
    for (ll v = 0; v < n; v++) {
      if (m->type[l][v] == VT_INACTIVE) continue;
      z[v] = mg_apply_stencil(m, v, l, p);
      alphaBot += p[v] * z[v];
    }
    const double alpha = alphaTop / alphaBot;
    double alphaTopNew = 0;
    residual = 0;
    for (ll v = 0; v < n; v++) {
      if (m->type[l][v] == VT_INACTIVE) continue;
      x[v] += alpha * p[v];
      r[v] -= alpha * z[v];
      residual += r[v] * r[v];
      if (l == 0) z[v] = r[v] / m->A[0][v * S0 + 0];
      else z[v] = r[v] / m->A[l][v * S + 0];
      alphaTopNew += r[v] * z[v];
    }
    residual = sqrt(residual);
    if (residual / initialResidual < m->coarseAcc) break;
    const double beta = alphaTopNew / alphaTop;
    alphaTop = alphaTopNew;
    for (ll v = 0; v < n; v++) p[v] = z[v] + beta * p[v];
  }
  for (ll v = 0; v < n; v++) m->x[l][v] = (og_real)x[v];
}

/* GridMg::doVCycle (multigrid.cpp:448-504) from a zero initial guess.  The
 * trailing residual norm of the reference is not used by the CG and is not
 * computed here. */
static void mg_do_vcycle(og_mg* m, og_real* dst) {
  const int maxL = m->nlev - 1;
  memset(m->x[0], 0, sizeof(og_real) * m->n[0]);
  for (int l = 0; l < maxL; l++) {
    mg_smooth(m, l, 0);
    mg_residual(m, l);
    mg_restrict(m, l + 1);
    memset(m->x[l + 1], 0, sizeof(og_real) * m->n[l + 1]);
  }
  mg_solve_cg(m, maxL);
  for (int l = maxL - 1; l >= 0; l--) {
    mg_interpolate(m, l);
    for (ll i = 0; i < m->n[l]; i++) m->x[l][i] += m->r[l][i];
    mg_smooth(m, l, 1);
  }
  memcpy(dst, m->x[0], sizeof(og_real) * m->n[0]);
}

/* knSetRhs (multigrid.cpp:417-432) */
static void mg_set_rhs(og_mg* m, const og_real* rhs) {
  for (ll i = 0; i < m->n[0]; i++) {
    m->b[0][i] = rhs[i];
    if (m->type[0][i] == VT_ACTIVE_TRIVIAL) m->b[0][i] *= m->trivialScale;
  }
}

void og_mg_vcycle(og_mg* m, const og_real* A0, const og_real* Ai, const og_real* Aj, const og_real* Ak, og_real* dst,
                  const og_real* rhs, og_real coarseAccuracy) {
  if (!m->isASet) mg_set_a(m, A0, Ai, Aj, Ak);
  m->coarseAcc = coarseAccuracy;
  mg_set_rhs(m, rhs);
  mg_do_vcycle(m, dst);
}

/* ------------------------------------------------------------------------ */
/* solvePressureSystem (pressure.cpp:312-452) with GridCg (conjugategrad.cpp
 * :209-299)                                                                 */

static void scaled_add(ll n, og_real* me, const og_real* other, og_real factor) {
  ll i;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (i = 0; i < n; i++) me[i] += factor * other[i];
}

int og_solve_pressure_system(og_dims d, og_real* rhs, og_real* pressure, const int* flags, const og_real* phi,
                             const og_pressure_params* p, og_mg** mg_cache, og_pressure_result* out) {
  const ll n = NCELL(d);
  og_real* residual = (og_real*)calloc((size_t)n, sizeof(og_real));
  og_real* search = (og_real*)calloc((size_t)n, sizeof(og_real));
  og_real* A0 = (og_real*)calloc((size_t)n, sizeof(og_real));
  og_real* Ai = (og_real*)calloc((size_t)n, sizeof(og_real));
  og_real* Aj = (og_real*)calloc((size_t)n, sizeof(og_real));
  og_real* Ak = (og_real*)calloc((size_t)n, sizeof(og_real));
  og_real* tmp = (og_real*)calloc((size_t)n, sizeof(og_real));
  og_real* pca0 = NULL;
  int pc = p->preconditioner;
  int status = 0;
  og_make_laplace_matrix(d, flags, A0, Ai, Aj, Ak);
  if (phi) og_apply_ghost_fluid_diagonal(d, A0, flags, phi, p->gfClamp);

  ll fixPidx = -1;
  if (p->zeroPressureFixing || p->cgAccuracy < 1e-07) {
    int numEmpty = 0;
    for (ll idx = 0; idx < n; idx++) if (isE(flags, idx)) numEmpty++;
    if (numEmpty == 0) {
      const int tc[3] = {d.nx / 2, d.ny - 1, d.is3d ? d.nz / 2 : 0};
      for (int q = 0; q < 3 && fixPidx < 0; q++) {
        const ll e = IX(d, tc[0], tc[1] - q, tc[2]);
        if (isF(flags, e)) fixPidx = e;
      }
      if (fixPidx == -1) {
        for (int k = KLO(d, 1); k < KHI(d, 1) && fixPidx < 0; k++)
          for (int j = 1; j < d.ny - 1 && fixPidx < 0; j++)
            for (int i = 1; i < d.nx - 1 && fixPidx < 0; i++)
              if (isF(flags, IX(d, i, j, k))) fixPidx = IX(d, i, j, k);
      }
    }
    if (fixPidx >= 0) {
      /* fixPressure(fixPidx, 0, ...) (pressure.cpp:226-245) */
      const ll X = 1, Y = SY(d), Z = SZ(d);
      const og_real value = OG_R(0.);
      rhs[fixPidx + X] -= Ai[fixPidx] * value;
      rhs[fixPidx + Y] -= Aj[fixPidx] * value;
      rhs[fixPidx - X] -= Ai[fixPidx - X] * value;
      rhs[fixPidx - Y] -= Aj[fixPidx - Y] * value;
      if (d.is3d) {
        rhs[fixPidx + Z] -= Ak[fixPidx] * value;
        rhs[fixPidx - Z] -= Ak[fixPidx - Z] * value;
      }
      rhs[fixPidx] = value;
      A0[fixPidx] = OG_R(1.);
      Ai[fixPidx] = Aj[fixPidx] = Ak[fixPidx] = OG_R(0.);
      Ai[fixPidx - X] = OG_R(0.);
      Aj[fixPidx - Y] = OG_R(0.);
      if (d.is3d) Ak[fixPidx - Z] = OG_R(0.);
    }
  }

  int maxIter = 0;
  og_mg* mg = NULL;
  if (pc == OG_PC_NONE) {
    /* GridCg::setICPreconditioner asserts on PC_None (conjugategrad.cpp:311) */
    status = -5;
    goto done;
  }
  if (pc == OG_PC_MIC) {
    maxIter = (int)(p->cgMaxIterFac * (og_real)imax(d.nx, imax(d.ny, d.nz))) * (d.is3d ? 1 : 4);
    if (!d.is3d) pc = OG_PC_NONE; /* mICP only in 3D (conjugategrad.cpp:315-321) */
    if (pc == OG_PC_MIC) pca0 = (og_real*)calloc((size_t)n, sizeof(og_real));
  } else if (pc == OG_PC_MG_DYNAMIC || pc == OG_PC_MG_STATIC) {
    maxIter = 100;
    mg = *mg_cache;
    if (mg && pc == OG_PC_MG_DYNAMIC) { og_mg_destroy(mg); *mg_cache = NULL; mg = NULL; }
    if (!mg) { mg = og_mg_create(d); *mg_cache = mg; }
  } else {
    status = -3;
    goto done;
  }

  {
    /* GridCg::doInit (conjugategrad.cpp:209-235) */
    const og_real acc = p->cgAccuracy;
    int iterations = 0;
    og_real sigma, resNorm = OG_R(1e20);
    memset(pressure, 0, sizeof(og_real) * n);
    memcpy(residual, rhs, sizeof(og_real) * n);
    if (pc == OG_PC_MIC) {
      og_mic_init(d, flags, pca0, A0, Ai, Aj, Ak);
      og_mic_apply(d, tmp, residual, flags, pca0, Ai, Aj, Ak);
    } else if (mg) {
      if (!mg->isASet) mg_set_a(mg, A0, Ai, Aj, Ak);
      mg->coarseAcc = (og_real)((double)acc * 1E-4);
      mg_set_rhs(mg, residual);
      mg_do_vcycle(mg, tmp);
    } else {
      memcpy(tmp, residual, sizeof(og_real) * n);
    }
    memcpy(search, tmp, sizeof(og_real) * n);
    sigma = (og_real)dot_product(n, tmp, residual);

    for (int iter = 0; iter < maxIter; iter++) {
      /* GridCg::iterate (conjugategrad.cpp:237-299) */
      iterations++;
      og_apply_matrix(d, flags, tmp, search, A0, Ai, Aj, Ak);
      const og_real dp = (og_real)dot_product(n, tmp, search);
      og_real alpha = OG_R(0.);
      if (og_fabs(dp) > OG_R(0.)) alpha = sigma / dp;
      scaled_add(n, pressure, search, alpha);
      scaled_add(n, residual, tmp, -alpha);
      if (pc == OG_PC_MIC) og_mic_apply(d, tmp, residual, flags, pca0, Ai, Aj, Ak);
      else if (mg) { mg_set_rhs(mg, residual); mg_do_vcycle(mg, tmp); }
      else memcpy(tmp, residual, sizeof(og_real) * n);
      if (p->useL2Norm) resNorm = (og_real)sum_sqr(n, residual);
      else resNorm = og_get_max_abs(n, residual);
      if (resNorm < acc) { sigma = resNorm; break; }
      const og_real sigmaNew = (og_real)dot_product(n, tmp, residual);
      const og_real beta = sigmaNew / sigma;
      ll i;
#pragma omp parallel for schedule(static) num_threads(g_threads)
      for (i = 0; i < n; i++) search[i] = tmp[i] + beta * search[i];
      sigma = sigmaNew;
      if (!(resNorm < 1e35)) { status = -4; break; }
    }
    if (out) { out->iterations = iterations; out->resNorm = resNorm; out->fixPidx = (int)fixPidx; }
  }
  if (mg && pc == OG_PC_MG_DYNAMIC) { og_mg_destroy(mg); *mg_cache = NULL; }

done:
  free(residual); free(search); free(A0); free(Ai); free(Aj); free(Ak); free(tmp); free(pca0);
  return status;
}

/* knCorrectVelocity (pressure.cpp:87-109), knCorrectVelocityGhostFluid
 * (:154-187), knReplaceClampedGhostFluidVels (:198-214) */
void og_correct_velocity(og_dims d, og_real* vel, const og_real* pr, const int* flags, const og_real* phi,
                         const og_real* curv, const og_pressure_params* p) {
  const ll X = 1, Y = SY(d), Z = SZ(d);
  int k;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        og_real* v = vel + 3 * idx;
        if (isF(flags, idx)) {
          if (isF(flags, idx - X)) v[0] -= (pr[idx] - pr[idx - X]);
          if (isF(flags, idx - Y)) v[1] -= (pr[idx] - pr[idx - Y]);
          if (d.is3d && isF(flags, idx - Z)) v[2] -= (pr[idx] - pr[idx - Z]);
          if (isE(flags, idx - X)) v[0] -= pr[idx];
          if (isE(flags, idx - Y)) v[1] -= pr[idx];
          if (d.is3d && isE(flags, idx - Z)) v[2] -= pr[idx];
        } else if (isE(flags, idx) && !isOut(flags, idx)) {
          if (isF(flags, idx - X)) v[0] += pr[idx - X]; else v[0] = OG_R(0.);
          if (isF(flags, idx - Y)) v[1] += pr[idx - Y]; else v[1] = OG_R(0.);
          if (d.is3d) { if (isF(flags, idx - Z)) v[2] += pr[idx - Z]; else v[2] = OG_R(0.); }
        }
      }
  if (!phi) return;
  const og_real gfc = p->gfClamp;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        og_real* v = vel + 3 * idx;
        if (isF(flags, idx)) {
          if (isE(flags, idx - X)) v[0] += pr[idx] * gf_helper(phi, idx, -X, gfc);
          if (isE(flags, idx - Y)) v[1] += pr[idx] * gf_helper(phi, idx, -Y, gfc);
          if (d.is3d && isE(flags, idx - Z)) v[2] += pr[idx] * gf_helper(phi, idx, -Z, gfc);
        } else if (isE(flags, idx) && !isOut(flags, idx)) {
          if (isF(flags, idx - X)) v[0] -= pr[idx - X] * gf_helper(phi, idx - X, +X, gfc); else v[0] = OG_R(0.);
          if (isF(flags, idx - Y)) v[1] -= pr[idx - Y] * gf_helper(phi, idx - Y, +Y, gfc); else v[1] = OG_R(0.);
          if (d.is3d) { if (isF(flags, idx - Z)) v[2] -= pr[idx - Z] * gf_helper(phi, idx - Z, +Z, gfc); else v[2] = OG_R(0.); }
        }
        if (curv) {
          const og_real st = p->surfTens;
          if (isF(flags, idx)) {
            if (isE(flags, idx - X)) v[0] += surf_tens_helper(phi, curv, idx, -X, st, gfc);
            if (isE(flags, idx - Y)) v[1] += surf_tens_helper(phi, curv, idx, -Y, st, gfc);
            if (d.is3d && isE(flags, idx - Z)) v[2] += surf_tens_helper(phi, curv, idx, -Z, st, gfc);
          } else if (isE(flags, idx) && !isOut(flags, idx)) {
            v[0] -= isF(flags, idx - X) ? surf_tens_helper(phi, curv, idx - X, +X, st, gfc) : OG_R(0.);
            v[1] -= isF(flags, idx - Y) ? surf_tens_helper(phi, curv, idx - Y, +Y, st, gfc) : OG_R(0.);
            if (d.is3d) v[2] -= isF(flags, idx - Z) ? surf_tens_helper(phi, curv, idx - Z, +Z, st, gfc) : OG_R(0.);
          }
        }
      }
#define CLAMPED(e, off) (theta_helper(phi[(e)], phi[(e) + (off)]) < gfc)
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (k = KLO(d, 1); k < KHI(d, 1); k++)
    for (int j = 1; j < d.ny - 1; j++)
      for (int i = 1; i < d.nx - 1; i++) {
        const ll idx = IX(d, i, j, k);
        if (!isE(flags, idx)) continue;
        og_real* v = vel + 3 * idx;
        if (isF(flags, idx - X) && CLAMPED(idx - X, +X)) v[0] = vel[3 * (idx - X) + 0];
        if (isF(flags, idx - Y) && CLAMPED(idx - Y, +Y)) v[1] = vel[3 * (idx - Y) + 1];
        if (d.is3d && isF(flags, idx - Z) && CLAMPED(idx - Z, +Z)) v[2] = vel[3 * (idx - Z) + 2];
        if (isF(flags, idx + X) && CLAMPED(idx + X, -X)) v[0] = vel[3 * (idx + X) + 0];
        if (isF(flags, idx + Y) && CLAMPED(idx + Y, -Y)) v[1] = vel[3 * (idx + Y) + 1];
        if (d.is3d && isF(flags, idx + Z) && CLAMPED(idx + Z, -Z)) v[2] = vel[3 * (idx + Z) + 2];
      }
#undef CLAMPED
}

int og_solve_pressure(og_dims d, og_real* vel, og_real* pressure, const int* flags, const og_real* phi,
                      const og_real* perCellCorr, const og_real* curv, const og_pressure_params* p, og_mg** mg_cache,
                      og_pressure_result* out, og_real* retRhs) {
  const ll n = NCELL(d);
  og_real* rhs = (og_real*)calloc((size_t)n, sizeof(og_real));
  og_compute_pressure_rhs(d, rhs, vel, flags, phi, perCellCorr, curv, p);
  int st = og_solve_pressure_system(d, rhs, pressure, flags, phi, p, mg_cache, out);
  if (st == 0) og_correct_velocity(d, vel, pressure, flags, phi, curv, p);
  if (retRhs) memcpy(retRhs, rhs, sizeof(og_real) * n);
  free(rhs);
  return st;
}

/* ------------------------------------------------------------------------ */
/* Scene setup                                                               */

/* FlagGrid::initDomain + initBoundaries (grid.cpp:732-842), no phiWalls */
void og_init_domain(og_dims d, int* flags, int boundaryWidth, const char* wallIn, const char* openIn,
                    const char* inflowIn, const char* outflowIn) {
  char wall[64], open[64], inflow[64], outflow[64];
  snprintf(wall, sizeof wall, "%s      ", wallIn);
  snprintf(open, sizeof open, "%s      ", openIn);
  snprintf(inflow, sizeof inflow, "%s      ", inflowIn);
  snprintf(outflow, sizeof outflow, "%s      ", outflowIn);
  int types[6] = {0, 0, 0, 0, 0, 0}, set[6] = {0, 0, 0, 0, 0, 0};
  const char lo[6] = {'x', 'X', 'y', 'Y', 'z', 'Z'};
  for (int i = 0; i < 6; ++i) {
    for (int s = 0; s < 6; s++) {
      if (s >= 4 && !d.is3d) continue;
      if (set[s]) continue;
      const char ch = lo[s];
      if (open[i] == ch) { types[s] = OG_OPEN; set[s] = 1; }
      else if (inflow[i] == ch) { types[s] = OG_INFLOW; set[s] = 1; }
      else if (outflow[i] == ch) { types[s] = OG_OUTFLOW; set[s] = 1; }
      else if (wall[i] == ch) { types[s] = OG_OBSTACLE; set[s] = 1; }
    }
  }
  const ll n = NCELL(d);
  for (ll idx = 0; idx < n; idx++) flags[idx] = OG_EMPTY;
  const int w = boundaryWidth;
  for (int k = 0; k < d.nz; k++)
    for (int j = 0; j < d.ny; j++)
      for (int i = 0; i < d.nx; i++) {
        const ll idx = IX(d, i, j, k);
        if (i <= w) flags[idx] = types[0];
        if (i >= d.nx - 1 - w) flags[idx] = types[1];
        if (j <= w) flags[idx] = types[2];
        if (j >= d.ny - 1 - w) flags[idx] = types[3];
        if (d.is3d) {
          if (k <= w) flags[idx] = types[4];
          if (k >= d.nz - 1 - w) flags[idx] = types[5];
        }
      }
}

/* FlagGrid::fillGrid (grid.cpp:856-861) */
void og_fill_grid(og_dims d, int* flags, int type) {
  const ll n = NCELL(d);
  for (ll idx = 0; idx < n; idx++) {
    const int f = flags[idx];
    if ((f & OG_OBSTACLE) == 0 && (f & OG_INFLOW) == 0 && (f & OG_OUTFLOW) == 0 && (f & OG_OPEN) == 0)
      flags[idx] = (f & ~(OG_EMPTY | OG_FLUID)) | type;
  }
}

/* setOpenBound (plugin/extforces.cpp:105-130) */
void og_set_open_bound(og_dims d, int* flags, int bWidth, const char* openBound, int type) {
  if (!openBound || !openBound[0]) return;
  int lo[3] = {0, 0, 0}, up[3] = {0, 0, 0};
  for (const char* c = openBound; *c; c++) {
    if (*c == 'x') lo[0] = 1; else if (*c == 'y') lo[1] = 1; else if (*c == 'z') lo[2] = 1;
    else if (*c == 'X') up[0] = 1; else if (*c == 'Y') up[1] = 1; else if (*c == 'Z') up[2] = 1;
  }
  for (int k = 0; k < d.nz; k++)
    for (int j = 0; j < d.ny; j++)
      for (int i = 0; i < d.nx; i++) {
        const ll idx = IX(d, i, j, k);
        const int loX = lo[0] && i <= bWidth, loY = lo[1] && j <= bWidth;
        const int upX = up[0] && i >= d.nx - bWidth - 1, upY = up[1] && j >= d.ny - bWidth - 1;
        const int innerI = i > bWidth && i < d.nx - bWidth - 1, innerJ = j > bWidth && j < d.ny - bWidth - 1;
        if (!d.is3d && (loX || upX || loY || upY)) {
          if ((loX || upX || innerI) && (loY || upY || innerJ) && isO(flags, idx)) flags[idx] = type;
        } else {
          const int loZ = lo[2] && k <= bWidth, upZ = up[2] && k >= d.nz - bWidth - 1;
          const int innerK = k > bWidth && k < d.nz - bWidth - 1;
          if (loX || upX || loY || upY || loZ || upZ) {
            if ((loX || upX || innerI) && (loY || upY || innerJ) && (loZ || upZ || innerK) && isO(flags, idx))
              flags[idx] = type;
          }
        }
      }
}

/* FlagGrid::updateFromLevelset (grid.cpp:844-854); invalidTimeValue is
 * -1000 (levelset.h) */
void og_update_from_levelset(og_dims d, int* flags, const og_real* phi) {
  const ll n = NCELL(d);
  for (ll idx = 0; idx < n; idx++) {
    if (!isO(flags, idx) && !isOut(flags, idx)) {
      const og_real ph = phi[idx];
      if (ph <= -OG_R(1000.)) continue;
      flags[idx] &= ~(OG_EMPTY | OG_FLUID);
      flags[idx] |= (ph <= 0) ? OG_FLUID : OG_EMPTY;
    }
  }
}

static inline og_real fmaxf_(og_real a, og_real b) { return a < b ? b : a; }
static inline og_real fminf_(og_real a, og_real b) { return b < a ? b : a; }

/* norm() of vectorbase.h:379-384 in Real */
static inline og_real vnorm(og_real x, og_real y, og_real z) {
  const og_real l = x * x + y * y + z * z;
  if (l <= OG_VEC_EPS * OG_VEC_EPS) return OG_R(0.);
  return (fabs(l - 1.) < OG_VEC_EPS * OG_VEC_EPS) ? OG_R(1.) : og_sqrt(l);
}

/* BoxSDF (shapes.cpp:178-228) */
void og_box_sdf(og_dims d, og_real* phi, og_real p1x, og_real p1y, og_real p1z, og_real p2x, og_real p2y, og_real p2z) {
  for (int k = 0; k < d.nz; k++)
    for (int j = 0; j < d.ny; j++)
      for (int i = 0; i < d.nx; i++) {
        const ll idx = IX(d, i, j, k);
        const og_real px = (og_real)(i + 0.5), py = (og_real)(j + 0.5), pz = (og_real)(k + 0.5);
        og_real v;
#define SQ(a) ((a) * (a))
        if (px <= p2x && px >= p1x && py <= p2y && py >= p1y && pz <= p2z && pz >= p1z) {
          og_real mx = fmaxf_(px - p2x, p1x - px), my = fmaxf_(py - p2y, p1y - py), mz = fmaxf_(pz - p2z, p1z - pz);
          if (!d.is3d) mz = mx;
          v = fmaxf_(mx, fmaxf_(my, mz));
        } else if (py <= p2y && py >= p1y && pz <= p2z && pz >= p1z) {
          v = fmaxf_(px - p2x, p1x - px);
        } else if (px <= p2x && px >= p1x && pz <= p2z && pz >= p1z) {
          v = fmaxf_(py - p2y, p1y - py);
        } else if (px <= p2x && px >= p1x && py <= p2y && py >= p1y) {
          v = fmaxf_(pz - p2z, p1z - pz);
        } else if (px > p1x && px < p2x) {
          og_real m1 = og_sqrt(SQ(p1y - py) + SQ(p1z - pz)), m2 = og_sqrt(SQ(p2y - py) + SQ(p1z - pz));
          og_real m3 = og_sqrt(SQ(p1y - py) + SQ(p2z - pz)), m4 = og_sqrt(SQ(p2y - py) + SQ(p2z - pz));
          v = fminf_(m1, fminf_(m2, fminf_(m3, m4)));
        } else if (py > p1y && py < p2y) {
          og_real m1 = og_sqrt(SQ(p1x - px) + SQ(p1z - pz)), m2 = og_sqrt(SQ(p2x - px) + SQ(p1z - pz));
          og_real m3 = og_sqrt(SQ(p1x - px) + SQ(p2z - pz)), m4 = og_sqrt(SQ(p2x - px) + SQ(p2z - pz));
          v = fminf_(m1, fminf_(m2, fminf_(m3, m4)));
        } else if (pz > p1x && pz < p2z) {
          og_real m1 = og_sqrt(SQ(p1y - py) + SQ(p1x - px)), m2 = og_sqrt(SQ(p2y - py) + SQ(p1x - px));
          og_real m3 = og_sqrt(SQ(p1y - py) + SQ(p2x - px)), m4 = og_sqrt(SQ(p2y - py) + SQ(p2x - px));
          v = fminf_(m1, fminf_(m2, fminf_(m3, m4)));
        } else {
          og_real m = vnorm(px - p1x, py - p1y, pz - p1z);
          m = fminf_(m, vnorm(px - p1x, py - p1y, pz - p2z));
          m = fminf_(m, vnorm(px - p1x, py - p2y, pz - p1z));
          m = fminf_(m, vnorm(px - p1x, py - p2y, pz - p2z));
          m = fminf_(m, vnorm(px - p2x, py - p1y, pz - p1z));
          m = fminf_(m, vnorm(px - p2x, py - p1y, pz - p2z));
          m = fminf_(m, vnorm(px - p2x, py - p2y, pz - p1z));
          m = fminf_(m, vnorm(px - p2x, py - p2y, pz - p2z));
          v = m;
        }
#undef SQ
        phi[idx] = v;
      }
}

/* Cylinder ctor normalisation (shapes.cpp:316-322) + isInside (:324-329)
 * at cell centres, ApplyShapeToGrid (:38-45) */
void og_cylinder_apply(og_dims d, og_real* grid, og_real cx, og_real cy, og_real cz, og_real radius, og_real zx, og_real zy, og_real zz,
                       og_real value, const int* respectFlags) {
  /* normalize(mZDir): returns the length, scales by 1/len in double */
  og_real nz_ = OG_R(0.);
  {
    const og_real l = zx * zx + zy * zy + zz * zz;
    if (fabs(l - 1.) < OG_VEC_EPS * OG_VEC_EPS) nz_ = OG_R(1.);
    else if (l > OG_VEC_EPS * OG_VEC_EPS) {
      nz_ = og_sqrt(l);
      /* v *= 1./norm: operator*=(S) takes the factor as Real */
      const og_real inv = (og_real)(1. / (double)nz_);
      zx = zx * inv; zy = zy * inv; zz = zz * inv;
    } else { zx = zy = zz = OG_R(0.); nz_ = OG_R(0.); }
  }
  const og_real mZ = nz_;
  for (int k = 0; k < d.nz; k++)
    for (int j = 0; j < d.ny; j++)
      for (int i = 0; i < d.nx; i++) {
        const ll idx = IX(d, i, j, k);
        if (respectFlags && isO(respectFlags, idx)) continue;
        const og_real px = (og_real)(i + 0.5) - cx, py = (og_real)(j + 0.5) - cy, pz = (og_real)(k + 0.5) - cz;
        const og_real z = px * zx + py * zy + pz * zz;
        if (og_fabs(z) > mZ) continue;
        const og_real r2 = (px * px + py * py + pz * pz) - z * z;
        if (r2 < radius * radius) grid[idx] = value;
      }
}

/* Box::isInside (shapes.cpp:151-154) at cell centres */
void og_box_apply(og_dims d, og_real* grid, og_real p0x, og_real p0y, og_real p0z, og_real p1x, og_real p1y, og_real p1z, og_real value,
                  const int* respectFlags) {
  for (int k = 0; k < d.nz; k++)
    for (int j = 0; j < d.ny; j++)
      for (int i = 0; i < d.nx; i++) {
        const ll idx = IX(d, i, j, k);
        if (respectFlags && isO(respectFlags, idx)) continue;
        const og_real px = (og_real)(i + 0.5), py = (og_real)(j + 0.5), pz = (og_real)(k + 0.5);
        if (px >= p0x && py >= p0y && pz >= p0z && px <= p1x && py <= p1y && pz <= p1z) grid[idx] = value;
      }
}

/* knJoinReal (grid.cpp): keep max (or min) per cell */
void og_join_real(ll n, og_real* a, const og_real* b, int keepMax) {
  for (ll i = 0; i < n; i++) a[i] = keepMax ? fmaxf_(a[i], b[i]) : fminf_(a[i], b[i]);
}

/* ------------------------------------------------------------------ noise */
/* MTRand (util/randomstream.h): MT19937 with the reference's seeding,
 * tempering and double conversions; RandomStream's getRandNorm and
 * getVec3Norm on top. */
typedef struct {
  unsigned int st[624];
  int left, next;
} og_mt;

static void og_mt_reload(og_mt* m) {
  unsigned int* s = m->st;
  for (int i = 0; i < 624; i++) {
    const unsigned int y = (s[i] & 0x80000000u) | (s[(i + 1) % 624] & 0x7fffffffu);
    s[i] = s[(i + 397) % 624] ^ (y >> 1) ^ ((s[(i + 1) % 624] & 1u) ? 0x9908b0dfu : 0u);
  }
  m->left = 624;
  m->next = 0;
}
static void og_mt_seed(og_mt* m, unsigned int seed) {
  m->st[0] = seed;
  for (int i = 1; i < 624; i++) m->st[i] = 1812433253u * (m->st[i - 1] ^ (m->st[i - 1] >> 30)) + (unsigned int)i;
  og_mt_reload(m);
}
static unsigned int og_mt_int(og_mt* m) {
  if (m->left == 0) og_mt_reload(m);
  m->left--;
  unsigned int y = m->st[m->next++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  return y ^ (y >> 18);
}
static double og_mt_rand(og_mt* m) { return (double)og_mt_int(m) * (1.0 / 4294967295.0); }
static double og_mt_norm(og_mt* m, double mean, double variance) {
  const double u = ((double)og_mt_int(m) + 0.5) * (1.0 / 4294967296.0);
  const double r = sqrt(-2.0 * log(1.0 - u)) * variance;
  const double phi = 2.0 * 3.14159265358979323846264338328 * ((double)og_mt_int(m) * (1.0 / 4294967296.0));
  return mean + r * cos(phi);
}

/* WaveletNoiseField::generateTile (noisefield.cpp:94-190) for the float build:
 * 3 tiles of 128^3 normal noise, minus their down/up-sampled version along x,
 * y and z (periodic), plus the result read at a (65,65,65) offset. */
static const float og_aco[32] = {
    0.000334f, -0.001528f, 0.000410f, 0.003545f, -0.000938f, -0.008233f, 0.002172f, 0.019120f,
    -0.005040f, -0.044412f, 0.011655f, 0.103311f, -0.025936f, -0.243780f, 0.033979f, 0.655340f,
    0.655340f, 0.033979f, -0.243780f, -0.025936f, 0.103311f, 0.011655f, -0.044412f, -0.005040f,
    0.019120f, 0.002172f, -0.008233f, -0.000938f, 0.003546f, 0.000410f, -0.001528f, 0.000334f};
static const float og_pco[4] = {0.25f, 0.75f, 0.75f, 0.25f};

static void og_noise_down(const float* from, float* to, int n, int stride) {
  for (int i = 0; i < n / 2; i++) {
    float acc = 0.f;
    for (int k = 2 * i - 16; k < 2 * i + 16; k++) acc += og_aco[16 + k - 2 * i] * from[(k & 127) * stride];
    to[i * stride] = acc;
  }
}
static void og_noise_up(const float* from, float* to, int n, int stride) {
  for (int i = 0; i < n; i++) {
    float acc = 0.f;
    for (int k = i / 2 - 1; k < i / 2 + 3; k++) {
      int mm = k % (n / 2);
      if (mm < 0) mm += n / 2;
      acc = (float)((double)acc + 0.5 * (double)og_pco[1 + k - i / 2] * (double)from[mm * stride]);
    }
    to[i * stride] = acc;
  }
}

void og_noise_tile(float* noise) {
  const int n = 128, n3 = n * n * n;
  og_mt mt;
  og_mt_seed(&mt, 13322223u);
  for (int i = 0; i < 3 * n3; i++) noise[i] = (float)og_mt_norm(&mt, 0.0, 1.0);
  float* t1 = (float*)calloc((size_t)3 * n3, sizeof(float));
  float* t2 = (float*)calloc((size_t)3 * n3, sizeof(float));
  for (int tile = 0; tile < 3; tile++) {
    for (int iy = 0; iy < n; iy++)
      for (int iz = 0; iz < n; iz++) {
        const int i = iy * n + iz * n * n + tile * n3;
        og_noise_down(noise + i, t1 + i, n, 1);
        og_noise_up(t1 + i, t2 + i, n, 1);
      }
    for (int ix = 0; ix < n; ix++)
      for (int iz = 0; iz < n; iz++) {
        const int i = ix + iz * n * n + tile * n3;
        og_noise_down(t2 + i, t1 + i, n, n);
        og_noise_up(t1 + i, t2 + i, n, n);
      }
    for (int ix = 0; ix < n; ix++)
      for (int iy = 0; iy < n; iy++) {
        const int i = ix + iy * n + tile * n3;
        og_noise_down(t2 + i, t1 + i, n, n * n);
        og_noise_up(t1 + i, t2 + i, n, n * n);
      }
  }
  for (int i = 0; i < 3 * n3; i++) noise[i] -= t2[i];
  const int off = 65;
  int c = 0;
  for (int tile = 0; tile < 3; tile++)
    for (int ix = 0; ix < n; ix++)
      for (int iy = 0; iy < n; iy++)
        for (int iz = 0; iz < n; iz++)
          t1[c++] = noise[((ix + off) & 127) + ((iy + off) & 127) * n + ((iz + off) & 127) * n * n + tile * n3];
  for (int i = 0; i < 3 * n3; i++) noise[i] += t1[i];
  free(t1);
  free(t2);
}

/* WaveletNoiseField(parent, fixedSeed): mSeedOffset = normalized getVec3 of
 * RandomStream(fixedSeed) (noisefield.cpp:61-78; seed -1 -> 13322223 + 123) */
void og_noise_seed_offset(int fixedSeed, float* out) {
  og_mt mt;
  og_mt_seed(&mt, (unsigned int)(fixedSeed == -1 ? 13322223 + 123 : fixedSeed));
  float v[3];
  for (int c = 0; c < 3; c++) v[c] = (float)og_mt_rand(&mt);
  const float l = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  if (fabs((double)l - 1.) < (double)(1e-6f * 1e-6f)) {
  } else if (l > 1e-6f * 1e-6f) {
    const float norm = sqrtf(l);
    const float s = (float)(1. / (double)norm);
    for (int c = 0; c < 3; c++) v[c] = v[c] * s;
  } else {
    v[0] = v[1] = v[2] = 0.f;
  }
  for (int c = 0; c < 3; c++) out[c] = v[c];
}

/* WaveletNoiseField::evaluate (noisefield.h:332-357) with WNoise (:155-196):
 * quadratic B-spline weights around ceil(p - 0.5), 27 tile samples summed x
 * fastest, then z. */
static float og_wnoise(const float* p, const float* data) {
  float w[3][3];
  int mid[3];
  for (int a = 0; a < 3; a++) {
    mid[a] = (int)ceilf(p[a] - 0.5f);
    const float t = (float)mid[a] - (p[a] - 0.5f);
    w[a][0] = t * t * 0.5f;
    w[a][2] = (1.f - t) * (1.f - t) * 0.5f;
    w[a][1] = 1.f - w[a][0] - w[a][2];
  }
  float result = 0.f;
  for (int z = -1; z <= 1; z++)
    for (int y = -1; y <= 1; y++)
      for (int x = -1; x <= 1; x++) {
        float weight = 1.0f;
        weight *= w[0][x + 1];
        weight *= w[1][y + 1];
        weight *= w[2][z + 1];
        const int xC = (mid[0] + x) & 127, yC = (mid[1] + y) & 127, zC = (mid[2] + z) & 127;
        result += weight * data[(zC * 128 + yC) * 128 + xC];
      }
  return result;
}

float og_noise_evaluate(const og_noise_params* q, const float* tile, float x, float y, float z) {
  float p[3] = {x, y, z};
  p[0] *= q->gsInv[0];
  p[1] *= q->gsInv[1];
  p[2] *= q->gsInv[2];
  for (int c = 0; c < 3; c++) p[c] += q->seedOffset[c];
  for (int c = 0; c < 3; c++) p[c] += q->timeOffset;
  for (int c = 0; c < 3; c++) p[c] *= q->posScale[c];
  for (int c = 0; c < 3; c++) p[c] += q->posOffset[c];
  float v = og_wnoise(p, tile);
  v += q->valOffset;
  v *= q->valScale;
  if (q->clamp) {
    if (v < q->clampNeg) v = q->clampNeg;
    if (v > q->clampPos) v = q->clampPos;
  }
  return v;
}

/* CylinderSDF (shapes.cpp:367-385), the Cylinder's levelset */
void og_cylinder_sdf(og_dims d, float* phi, const float* center, float radius, const float* zaxis, float maxz) {
  for (int k = 0; k < d.nz; k++)
    for (int j = 0; j < d.ny; j++)
      for (int i = 0; i < d.nx; i++) {
        const float px = (float)(i + 0.5) - center[0], py = (float)(j + 0.5) - center[1], pz = (float)(k + 0.5) - center[2];
        const float z = fabsf(px * zaxis[0] + py * zaxis[1] + pz * zaxis[2]);
        const float r = sqrtf((px * px + py * py + pz * pz) - z * z);
        float v;
        if (z < maxz) v = r < radius ? fmaxf_(r - radius, z - maxz) : r - radius;
        else if (r < radius) v = fabsf(z - maxz);
        else v = sqrtf((z - maxz) * (z - maxz) + (r - radius) * (r - radius));
        phi[IX(d, i, j, k)] = v;
      }
}

/* densityInflow (initplugins.cpp:38-43) with KnApplyNoiseInfl (:27-36) */
void og_density_inflow(og_dims d, const int* flags, float* density, const float* sdf, const og_noise_params* q,
                       const float* tile, float scale, float sigma) {
  for (int k = 0; k < d.nz; k++)
    for (int j = 0; j < d.ny; j++)
      for (int i = 0; i < d.nx; i++) {
        const ll idx = IX(d, i, j, k);
        if (!isF(flags, idx) || sdf[idx] > sigma) continue;
        double f = 1.0 - 0.5 / (double)sigma * (double)(sdf[idx] + sigma);
        if (f < 0.0) f = 0.0;
        else if (f > 1.0) f = 1.0;
        const float factor = (float)f;
        const float target = og_noise_evaluate(q, tile, (float)i, (float)j, (float)k) * scale * factor;
        if (density[idx] < target) density[idx] = target;
      }
}

/* ------------------------------------------------------------------------ */
/* FLIP transfers (plugin/flip.cpp:549-673).  Particles: pos[3*i] (Vec3
 * records), flag[i] (BasicParticleData::flag, particle.h:182-191); a particle
 * is active unless flag has ParticleBase::PDELETE (particle.h:41, :122).     */

#define OG_PDELETE (1 << 10)

static inline int part_skipped(const int* pflag, const int* ptype, int exclude, ll p) {
  return (pflag[p] & OG_PDELETE) != 0 || (ptype && (ptype[p] & exclude) != 0);
}

/* setInterpolMAC (util/interpol.h:159-195): every component's 8 faces get the
 * weight into sum and weight * value into data, in the reference's order
 * (in 2D the z stride is 0 and both z layers land on one face) */
static void set_interpol_mac(og_dims d, og_real* data, og_real* sum, og_real x, og_real y, og_real z,
                             const og_real* val) {
  const wts w = build_index(d, x, y, z);
  const wts s = build_index_shift(d, x, y, z);
  const ll X = 1, Y = SY(d), Z = SZ(d);
#define ADD(arr, o, c, v) (arr)[3 * (o) + (c)] += (v)
  { /* X: x shifted */
    const ll b = ((ll)w.zi * d.ny + w.yi) * d.nx + s.xi;
    og_real* ref = data + 3 * b;
    og_real* sm = sum + 3 * b;
    const og_real s0f0 = s.s0 * w.f0, s1f0 = s.s1 * w.f0, s0f1 = s.s0 * w.f1, s1f1 = s.s1 * w.f1;
    const og_real w0 = w.t0 * s0f0, wx = w.t0 * s1f0, wy = w.t1 * s0f0, wxy = w.t1 * s1f0;
    const og_real wz = w.t0 * s0f1, wxz = w.t0 * s1f1, wyz = w.t1 * s0f1, wxyz = w.t1 * s1f1;
    const og_real v = val[0];
    ADD(sm, Z, 0, wz); ADD(sm, X + Z, 0, wxz); ADD(sm, Y + Z, 0, wyz); ADD(sm, X + Y + Z, 0, wxyz);
    ADD(ref, Z, 0, wz * v); ADD(ref, X + Z, 0, wxz * v); ADD(ref, Y + Z, 0, wyz * v); ADD(ref, X + Y + Z, 0, wxyz * v);
    ADD(sm, 0, 0, w0); ADD(sm, X, 0, wx); ADD(sm, Y, 0, wy); ADD(sm, X + Y, 0, wxy);
    ADD(ref, 0, 0, w0 * v); ADD(ref, X, 0, wx * v); ADD(ref, Y, 0, wy * v); ADD(ref, X + Y, 0, wxy * v);
  }
  { /* Y: y shifted */
    const ll b = ((ll)w.zi * d.ny + s.yi) * d.nx + w.xi;
    og_real* ref = data + 3 * b;
    og_real* sm = sum + 3 * b;
    const og_real s0f0 = w.s0 * w.f0, s1f0 = w.s1 * w.f0, s0f1 = w.s0 * w.f1, s1f1 = w.s1 * w.f1;
    const og_real w0 = s.t0 * s0f0, wx = s.t0 * s1f0, wy = s.t1 * s0f0, wxy = s.t1 * s1f0;
    const og_real wz = s.t0 * s0f1, wxz = s.t0 * s1f1, wyz = s.t1 * s0f1, wxyz = s.t1 * s1f1;
    const og_real v = val[1];
    ADD(sm, Z, 1, wz); ADD(sm, X + Z, 1, wxz); ADD(sm, Y + Z, 1, wyz); ADD(sm, X + Y + Z, 1, wxyz);
    ADD(ref, Z, 1, wz * v); ADD(ref, X + Z, 1, wxz * v); ADD(ref, Y + Z, 1, wyz * v); ADD(ref, X + Y + Z, 1, wxyz * v);
    ADD(sm, 0, 1, w0); ADD(sm, X, 1, wx); ADD(sm, Y, 1, wy); ADD(sm, X + Y, 1, wxy);
    ADD(ref, 0, 1, w0 * v); ADD(ref, X, 1, wx * v); ADD(ref, Y, 1, wy * v); ADD(ref, X + Y, 1, wxy * v);
  }
  { /* Z: z shifted; the z = 0 layer first */
    const ll b = ((ll)s.zi * d.ny + w.yi) * d.nx + w.xi;
    og_real* ref = data + 3 * b;
    og_real* sm = sum + 3 * b;
    const og_real s0f0 = w.s0 * s.f0, s1f0 = w.s1 * s.f0, s0f1 = w.s0 * s.f1, s1f1 = w.s1 * s.f1;
    const og_real w0 = w.t0 * s0f0, wx = w.t0 * s1f0, wy = w.t1 * s0f0, wxy = w.t1 * s1f0;
    const og_real wz = w.t0 * s0f1, wxz = w.t0 * s1f1, wyz = w.t1 * s0f1, wxyz = w.t1 * s1f1;
    const og_real v = val[2];
    ADD(sm, 0, 2, w0); ADD(sm, X, 2, wx); ADD(sm, Y, 2, wy); ADD(sm, X + Y, 2, wxy);
    ADD(sm, Z, 2, wz); ADD(sm, X + Z, 2, wxz); ADD(sm, Y + Z, 2, wyz); ADD(sm, X + Y + Z, 2, wxyz);
    ADD(ref, 0, 2, w0 * v); ADD(ref, X, 2, wx * v); ADD(ref, Y, 2, wy * v); ADD(ref, X + Y, 2, wxy * v);
    ADD(ref, Z, 2, wz * v); ADD(ref, X + Z, 2, wxz * v); ADD(ref, Y + Z, 2, wyz * v); ADD(ref, X + Y + Z, 2, wxyz * v);
  }
#undef ADD
}

/* mapPartsToMAC (flip.cpp:573-595) with knMapLinearVec3ToMACGrid (:561-570)
 * run serially in particle order; weight (AoS Vec3) may be NULL */
void og_map_parts_to_mac(og_dims d, og_real* vel, og_real* velOld, og_real* weight, ll np, const og_real* pos,
                         const int* pflag, const og_real* pvel, const int* ptype, int exclude) {
  const ll n3 = 3 * CELLS(d);
  og_real* w = weight ? weight : (og_real*)malloc(sizeof(og_real) * n3);
  for (ll i = 0; i < n3; i++) { w[i] = OG_R(0.); vel[i] = OG_R(0.); }
  for (ll p = 0; p < np; p++) {
    if (part_skipped(pflag, ptype, exclude, p)) continue;
    set_interpol_mac(d, vel, w, pos[3 * p], pos[3 * p + 1], pos[3 * p + 2], pvel + 3 * p);
  }
  /* Grid<Vec3>::stomp (grid.cpp:224-226), then MACGrid::safeDivide
   * (safeDivide, general.h:150) */
  for (ll i = 0; i < n3; i++) {
    if (w[i] < OG_R(OG_VEC_EPS)) w[i] = OG_R(0.);
    if (w[i] != OG_R(0.)) vel[i] = vel[i] / w[i];
    velOld[i] = vel[i];
  }
  if (!weight) free(w);
}

/* mapPartsToGrid / mapPartsToGridVec3 (flip.cpp:599-622): setInterpol
 * (util/interpol.h:93-112) per particle, then knSafeDivReal (:549-557);
 * comps 1 (Real) or 3 (Vec3, AoS) */
void og_map_parts_to_grid(og_dims d, og_real* target, int comps, ll np, const og_real* pos, const int* pflag,
                          const og_real* src) {
  const ll n = CELLS(d);
  og_real* sum = (og_real*)calloc((size_t)n, sizeof(og_real));
  for (ll i = 0; i < n * comps; i++) target[i] = OG_R(0.);
  const ll X = 1, Y = SY(d), Z = SZ(d);
  for (ll p = 0; p < np; p++) {
    if (pflag[p] & OG_PDELETE) continue;
    const wts w = build_index(d, pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]);
    const ll b = (ll)w.xi + Y * w.yi + Z * w.zi;
    const og_real s0f0 = w.s0 * w.f0, s1f0 = w.s1 * w.f0, s0f1 = w.s0 * w.f1, s1f1 = w.s1 * w.f1;
    const og_real w0 = w.t0 * s0f0, wx = w.t0 * s1f0, wy = w.t1 * s0f0, wxy = w.t1 * s1f0;
    const og_real wz = w.t0 * s0f1, wxz = w.t0 * s1f1, wyz = w.t1 * s0f1, wxyz = w.t1 * s1f1;
    const og_real* v = src + (ll)comps * p;
    og_real* sm = sum + b;
    og_real* ref = target + (ll)comps * b;
#define ADDV(o, wt)                                                  \
  for (int c = 0; c < comps; c++) ref[(ll)comps * (o) + c] += (wt) * v[c];
    sm[Z] += wz; sm[X + Z] += wxz; sm[Y + Z] += wyz; sm[X + Y + Z] += wxyz;
    ADDV(Z, wz) ADDV(X + Z, wxz) ADDV(Y + Z, wyz) ADDV(X + Y + Z, wxyz)
    sm[0] += w0; sm[X] += wx; sm[Y] += wy; sm[X + Y] += wxy;
    ADDV(0, w0) ADDV(X, wx) ADDV(Y, wy) ADDV(X + Y, wxy)
#undef ADDV
  }
  for (ll i = 0; i < n; i++) {
    for (int c = 0; c < comps; c++) {
      og_real* t = target + (ll)comps * i + c;
      if (sum[i] < OG_R(OG_VEC_EPS)) *t = OG_R(0.);
      else if (sum[i] != OG_R(0.)) *t = *t / sum[i];
    }
  }
  free(sum);
}

/* mapMACToParts (flip.cpp:643-655); with velOld, flipVelocityUpdate
 * (:659-673): pvel = flipRatio * (pvel + delta) + (1.0 - flipRatio) * v,
 * whose second product the reference forms in double */
void og_map_mac_to_parts(og_dims d, const og_real* vel, const og_real* velOld, og_real flipRatio, ll np,
                         const og_real* pos, const int* pflag, og_real* pvel, const int* ptype, int exclude) {
  for (ll p = 0; p < np; p++) {
    if (part_skipped(pflag, ptype, exclude, p)) continue;
    const og_real x = pos[3 * p], y = pos[3 * p + 1], z = pos[3 * p + 2];
    const v3 v = interp_mac(d, vel, x, y, z);
    og_real* pv = pvel + 3 * p;
    if (!velOld) {
      pv[0] = v.x; pv[1] = v.y; pv[2] = v.z;
      continue;
    }
    const v3 o = interp_mac(d, velOld, x, y, z);
    const og_real dl[3] = {v.x - o.x, v.y - o.y, v.z - o.z};
    const og_real vv[3] = {v.x, v.y, v.z};
    const double keep = 1.0 - (double)flipRatio;
    for (int c = 0; c < 3; c++) pv[c] = flipRatio * (pv[c] + dl[c]) + (og_real)(keep * (double)vv[c]);
  }
}

/* mapGridToParts / mapGridToPartsVec3 (knMapFromGrid, flip.cpp:625-638) */
void og_map_grid_to_parts(og_dims d, const og_real* grid, int comps, ll np, const og_real* pos, const int* pflag,
                          og_real* target) {
  for (ll p = 0; p < np; p++) {
    if (pflag[p] & OG_PDELETE) continue;
    for (int c = 0; c < comps; c++)
      target[(ll)comps * p + c] = interp_ch(d, grid, comps, c, pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]);
  }
}

/* ------------------------------------------------------------------------ */
/* resetOutflow (plugin/extforces.cpp:133-160) without particles: outflow
 * cells lose the fluid flag and gain the empty flag; phi = 0.5, real = 0
 * there.  phi / real may be NULL. */
void og_reset_outflow(og_dims d, int* flags, og_real* phi, og_real* real) {
  const ll n = NCELL(d);
  for (ll idx = 0; idx < n; idx++) {
    if (!(flags[idx] & OG_OUTFLOW)) continue;
    flags[idx] = (flags[idx] | OG_EMPTY) & ~OG_FLUID;
    if (phi) phi[idx] = OG_R(0.5);
    if (real) real[idx] = OG_R(0.);
  }
}

/* resetPhiInObs (plugin/advection.cpp:396-401) */
void og_reset_phi_in_obs(og_dims d, const int* flags, og_real* sdf) {
  const ll n = NCELL(d);
  for (ll idx = 0; idx < n; idx++)
    if ((flags[idx] & OG_OBSTACLE) && sdf[idx] < OG_R(0.)) sdf[idx] = OG_R(0.1);
}
