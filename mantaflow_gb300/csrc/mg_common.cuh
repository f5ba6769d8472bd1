// Device-side building blocks shared by the grid-step kernels.
//
// HBM layout (one GPU, device resident):
//   * Real / Levelset grids: float[n], x fastest, index i + nx*j + sz*k with
//     sz = 0 in 2D -- the reference layout (source/grid.h:70).
//   * MAC / Vec3 grids: structure-of-arrays, three float planes u|v|w of n
//     cells each.  The host API keeps the reference's array-of-structs Vec3
//     (util/vectorbase.h:199-205); uploads/downloads transpose on the GPU.
//   * Flag grids: int32[n], same bits as FlagGrid::CellType (source/grid.h:292).
//
// Arithmetic mirrors the reference expression by expression.  The library is
// built with -fmad=false so a*b+c is never contracted (the reference's x86-64
// -O3 build emits no FMA).  Where the reference forms a float expression in
// double (a double literal in the product) and rounds once, the kernels use
// an explicit fmaf(), which rounds the exact a*b+c once.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mgpu {

enum : int {
  kFluid = 1, kObstacle = 2, kEmpty = 4, kInflow = 8, kOutflow = 16, kOpen = 32, kStick = 64
};

struct Dims {
  int nx, ny, nz;
  int is3d;
  long long n;   // cells
  long long sy;  // nx
  long long sz;  // nx*ny in 3D, 0 in 2D
};

__host__ __device__ inline long long ix(const Dims& d, int i, int j, int k) {
  return (long long)i + d.sy * j + d.sz * k;
}

__device__ __forceinline__ bool isF(const int* f, long long i) { return (__ldg(f + i) & kFluid) != 0; }
__device__ __forceinline__ bool isO(const int* f, long long i) { return (__ldg(f + i) & kObstacle) != 0; }
__device__ __forceinline__ bool isE(const int* f, long long i) { return (__ldg(f + i) & kEmpty) != 0; }
__device__ __forceinline__ bool isOut(const int* f, long long i) { return (__ldg(f + i) & kOutflow) != 0; }

// SoA view of a MAC or Vec3 grid
struct Mac {
  float* u;
  float* v;
  float* w;
  __host__ __device__ __forceinline__ float* c(int comp) const { return comp == 0 ? u : (comp == 1 ? v : w); }
};
struct CMac {
  const float* u;
  const float* v;
  const float* w;
  __host__ __device__ __forceinline__ const float* c(int comp) const { return comp == 0 ? u : (comp == 1 ? v : w); }
};

struct V3 {
  float x, y, z;
};

// MACGrid::getCentered / getAtMACX/Y/Z (source/grid.h:424-470).  0.5*(a+b)
// and 0.25*(((a+b)+c)+d) are exact scalings of float sums.
__device__ __forceinline__ V3 mac_centered(const Dims& d, CMac m, long long i64) {
  const int i = (int)i64;  // grids stay below 2^31 cells (checked at creation)
  V3 r;
  r.x = 0.5f * (__ldg(m.u + i) + __ldg(m.u + i + 1));
  r.y = 0.5f * (__ldg(m.v + i) + __ldg(m.v + i + (int)d.sy));
  r.z = d.is3d ? 0.5f * (__ldg(m.w + i) + __ldg(m.w + i + (int)d.sz)) : 0.f;
  return r;
}
__device__ __forceinline__ V3 mac_at_x(const Dims& d, CMac m, long long i64) {
  const int i = (int)i64;  // grids stay below 2^31 cells (checked at creation)
  const int Y = (int)d.sy, Z = (int)d.sz;
  V3 r;
  r.x = __ldg(m.u + i);
  r.y = 0.25f * (__ldg(m.v + i) + __ldg(m.v + i - 1) + __ldg(m.v + i + Y) + __ldg(m.v + i + Y - 1));
  r.z = d.is3d ? 0.25f * (__ldg(m.w + i) + __ldg(m.w + i - 1) + __ldg(m.w + i + Z) + __ldg(m.w + i + Z - 1)) : 0.f;
  return r;
}
__device__ __forceinline__ V3 mac_at_y(const Dims& d, CMac m, long long i64) {
  const int i = (int)i64;  // grids stay below 2^31 cells (checked at creation)
  const int Y = (int)d.sy, Z = (int)d.sz;
  V3 r;
  r.x = 0.25f * (__ldg(m.u + i) + __ldg(m.u + i - Y) + __ldg(m.u + i + 1) + __ldg(m.u + i + 1 - Y));
  r.y = __ldg(m.v + i);
  r.z = d.is3d ? 0.25f * (__ldg(m.w + i) + __ldg(m.w + i - Y) + __ldg(m.w + i + Z) + __ldg(m.w + i + Z - Y)) : 0.f;
  return r;
}
__device__ __forceinline__ V3 mac_at_z(const Dims& d, CMac m, long long i64) {
  const int i = (int)i64;  // grids stay below 2^31 cells (checked at creation)
  const int Y = (int)d.sy, Z = (int)d.sz;
  V3 r;
  r.x = 0.25f * (__ldg(m.u + i) + __ldg(m.u + i - Z) + __ldg(m.u + i + 1) + __ldg(m.u + i + 1 - Z));
  r.y = 0.25f * (__ldg(m.v + i) + __ldg(m.v + i - Z) + __ldg(m.v + i + Y) + __ldg(m.v + i + Y - Z));
  r.z = __ldg(m.w + i);
  return r;
}

// Trilinear weights with border clamp: BUILD_INDEX (util/interpol.h:50-66)
// and the unshifted variant of BUILD_INDEX_SHIFT (:116-130).
struct Wts {
  int xi, yi, zi;
  float s0, s1, t0, t1, f0, f1;
};

template <bool kShift>
__device__ __forceinline__ Wts build_index(const Dims& d, float x, float y, float z) {
  Wts w;
  const float px = kShift ? x : x - 0.5f;
  const float py = kShift ? y : y - 0.5f;
  const float pz = kShift ? z : z - 0.5f;
  w.xi = (int)px; w.yi = (int)py; w.zi = (int)pz;
  w.s1 = px - (float)w.xi; w.s0 = 1.f - w.s1;
  w.t1 = py - (float)w.yi; w.t0 = 1.f - w.t1;
  w.f1 = pz - (float)w.zi; w.f0 = 1.f - w.f1;
  if (px < 0.f) { w.xi = 0; w.s0 = 1.f; w.s1 = 0.f; }
  if (py < 0.f) { w.yi = 0; w.t0 = 1.f; w.t1 = 0.f; }
  if (pz < 0.f) { w.zi = 0; w.f0 = 1.f; w.f1 = 0.f; }
  if (w.xi >= d.nx - 1) { w.xi = d.nx - 2; w.s0 = 0.f; w.s1 = 1.f; }
  if (w.yi >= d.ny - 1) { w.yi = d.ny - 2; w.t0 = 0.f; w.t1 = 1.f; }
  if (d.nz > 1) {
    if (w.zi >= d.nz - 1) { w.zi = d.nz - 2; w.f0 = 0.f; w.f1 = 1.f; }
  }
  return w;
}

// interpol<T> for one float plane (util/interpol.h:68-78)
__device__ __forceinline__ float interp(const Dims& d, const float* __restrict__ a, float x, float y, float z) {
  const Wts w = build_index<false>(d, x, y, z);
  const int X = 1, Y = (int)d.sy, Z = (int)d.sz;
  const int b = w.xi + Y * w.yi + Z * w.zi;
  const float* p = a + b;
  return ((__ldg(p) * w.t0 + __ldg(p + Y) * w.t1) * w.s0 + (__ldg(p + X) * w.t0 + __ldg(p + X + Y) * w.t1) * w.s1) * w.f0 +
         ((__ldg(p + Z) * w.t0 + __ldg(p + Y + Z) * w.t1) * w.s0 +
          (__ldg(p + X + Z) * w.t0 + __ldg(p + X + Y + Z) * w.t1) * w.s1) * w.f1;
}

// interpolMAC (util/interpol.h:127-157): per component, one axis shifted.
// kSlab: in 2D, read the z = 0 slab whatever z is (for arbitrary particle
// positions; the reference's 2D particles stay in 0 <= z < 1, where this
// changes nothing)
template <bool kSlab = false>
__device__ __forceinline__ V3 interp_mac(const Dims& d, CMac m, float x, float y, float z) {
  Wts w = build_index<false>(d, x, y, z);
  Wts s = build_index<true>(d, x, y, z);
  if (kSlab && !d.is3d) w.zi = s.zi = 0;
  const int X = 1, Y = (int)d.sy, Z = (int)d.sz;
  V3 r;
  {
    const float* p = m.u + ((w.zi * d.ny + w.yi) * d.nx + s.xi);
    r.x = w.f0 * ((__ldg(p) * w.t0 + __ldg(p + Y) * w.t1) * s.s0 + (__ldg(p + X) * w.t0 + __ldg(p + X + Y) * w.t1) * s.s1) +
          w.f1 * ((__ldg(p + Z) * w.t0 + __ldg(p + Z + Y) * w.t1) * s.s0 +
                  (__ldg(p + X + Z) * w.t0 + __ldg(p + X + Y + Z) * w.t1) * s.s1);
  }
  {
    const float* p = m.v + ((w.zi * d.ny + s.yi) * d.nx + w.xi);
    r.y = w.f0 * ((__ldg(p) * s.t0 + __ldg(p + Y) * s.t1) * w.s0 + (__ldg(p + X) * s.t0 + __ldg(p + X + Y) * s.t1) * w.s1) +
          w.f1 * ((__ldg(p + Z) * s.t0 + __ldg(p + Z + Y) * s.t1) * w.s0 +
                  (__ldg(p + X + Z) * s.t0 + __ldg(p + X + Y + Z) * s.t1) * w.s1);
  }
  {
    const float* p = m.w + ((s.zi * d.ny + w.yi) * d.nx + w.xi);
    r.z = s.f0 * ((__ldg(p) * w.t0 + __ldg(p + Y) * w.t1) * w.s0 + (__ldg(p + X) * w.t0 + __ldg(p + X + Y) * w.t1) * w.s1) +
          s.f1 * ((__ldg(p + Z) * w.t0 + __ldg(p + Z + Y) * w.t1) * w.s0 +
                  (__ldg(p + X + Z) * w.t0 + __ldg(p + X + Y + Z) * w.t1) * w.s1);
  }
  return r;
}

// Catmull-Rom helpers (util/interpolHigh.h:22-40).  For Real grids the
// reference forms a2/a3 in double; for Vec3 every operator rounds to float.
__device__ __forceinline__ float cubic_real(float t, const float* p) {
  const float d0 = (float)((double)(p[2] - p[0]) * 0.5);
  const float d1 = (float)((double)(p[3] - p[1]) * 0.5);
  const float dk = p[2] - p[1];
  const float a0 = p[1], a1 = d0;
  const float a2 = (float)(3.0 * (double)dk - 2.0 * (double)d0 - (double)d1);
  const float a3 = (float)(-2.0 * (double)dk + (double)d0 + (double)d1);
  const float sq = t * t, cu = sq * t;
  return a3 * cu + a2 * sq + a1 * t + a0;
}
__device__ __forceinline__ float cubic_vec(float t, const float* p) {
  const float d0 = (float)((double)(p[2] - p[0]) * 0.5);
  const float d1 = (float)((double)(p[3] - p[1]) * 0.5);
  const float dk = p[2] - p[1];
  const float a0 = p[1], a1 = d0;
  float a2 = (float)(3.0 * (double)dk);
  a2 = a2 - (float)(2.0 * (double)d0);
  a2 = a2 - d1;
  float a3 = (float)(-2.0 * (double)dk);
  a3 = a3 + d0;
  a3 = a3 + d1;
  const float sq = t * t, cu = sq * t;
  return a3 * cu + a2 * sq + a1 * t + a0;
}

// interpolCubic / interpolCubic2D (util/interpolHigh.h:42-160)
template <bool kVec>
__device__ inline float interp_cubic(const Dims& d, const float* __restrict__ a, float x, float y, float z) {
  if (d.sz == 0) {
    const float px = x - 0.5f, py = y - 0.5f;
    const int x1 = (int)px, x0 = x1 - 1, x3 = x1 + 2;
    const int y1 = (int)py, y0 = y1 - 1, y3 = y1 + 2;
    if (x0 < 0 || y0 < 0 || x3 >= d.nx || y3 >= d.ny) return interp(d, a, x, y, z);
    const float xI = px - x1, yI = py - y1;
    float fin[4];
    for (int r = 0; r < 4; r++) {
      float pts[4];
      for (int q = 0; q < 4; q++) pts[q] = __ldg(a + (x0 + q) + (long long)(y0 + r) * d.nx);
      fin[r] = kVec ? cubic_vec(xI, pts) : cubic_real(xI, pts);
    }
    return kVec ? cubic_vec(yI, fin) : cubic_real(yI, fin);
  }
  const float px = x - 0.5f, py = y - 0.5f, pz = z - 0.5f;
  const int x1 = (int)px, x0 = x1 - 1, x3 = x1 + 2;
  const int y1 = (int)py, y0 = y1 - 1, y3 = y1 + 2;
  const int z1 = (int)pz, z0 = z1 - 1, z3 = z1 + 2;
  if (x0 < 0 || y0 < 0 || z0 < 0 || x3 >= d.nx || y3 >= d.ny || z3 >= d.nz) return interp(d, a, x, y, z);
  const float xI = px - x1, yI = py - y1, zI = pz - z1;
  float zp[4];
  for (int s = 0; s < 4; s++) {
    float yp[4];
    for (int r = 0; r < 4; r++) {
      float pts[4];
      for (int q = 0; q < 4; q++) pts[q] = __ldg(a + (x0 + q) + (long long)(y0 + r) * d.nx + (long long)(z0 + s) * d.sz);
      yp[r] = kVec ? cubic_vec(xI, pts) : cubic_real(xI, pts);
    }
    zp[s] = kVec ? cubic_vec(yI, yp) : cubic_real(yI, yp);
  }
  return kVec ? cubic_vec(zI, zp) : cubic_real(zI, zp);
}

// launch helper: 2D tiles over (x, y), grid z over k
inline dim3 grid3(const Dims& d, dim3 b) {
  return dim3((unsigned)((d.nx + b.x - 1) / b.x), (unsigned)((d.ny + b.y - 1) / b.y), (unsigned)d.nz);
}

}  // namespace mgpu
