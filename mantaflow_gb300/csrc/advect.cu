// Semi-Lagrangian and MacCormack advection (plugin/advection.cpp).
//
// Scalar / Vec3 MacCormack runs as two sweeps instead of the reference's four
// (SemiLagrange fwd, SemiLagrange bwd, MacCormackCorrect, MacCormackClamp):
//   k_sl_*          fwd = SL(orig, dt) on the interior, 0 on the border
//                   (the reference's fresh zeroed grid, advection.cpp:298-300)
//   k_maccormack_*  bwd = SL(fwd, -dt) evaluated on the fly, then the
//                   correction and the clamp; bwd is never stored.
// Per cell the arithmetic is the reference's, so the result is the same.
#include "mg_common.cuh"
#include "mg_kernels.h"
#include "mg_batch.h"

#include <algorithm>
#include <cfloat>

namespace mgpu {

// ---------------------------------------------------------------- scalar SL
// SemiLagrange (advection.cpp:25-41) for CH float planes (1: Real, 3: Vec3)
template <int CH, int kOrderSpace, int kTrace>
__device__ __forceinline__ void sl_real_cell(const Dims& d, CMac vel, const float* __restrict__ src, float* __restrict__ dst,
                                                 float dt, int i, int j, int k) {
  const long long idx = ix(d, i, j, k);
  const bool inner = i >= 1 && i < d.nx - 1 && j >= 1 && j < d.ny - 1 && (!d.is3d || (k >= 1 && k < d.nz - 1));
  if (!inner) {
#pragma unroll
    for (int c = 0; c < CH; c++) dst[c * d.n + idx] = 0.f;
    return;
  }
  const V3 vc = mac_centered(d, vel, idx);
  float px, py, pz;
  if (kTrace == 1) {
    px = (i + 0.5f) - vc.x * dt;
    py = (j + 0.5f) - vc.y * dt;
    pz = (k + 0.5f) - vc.z * dt;
  } else {
    const float p0x = i + 0.5f, p0y = j + 0.5f, p0z = k + 0.5f;
    const V3 vi = interp_mac(d, vel, p0x - (vc.x * dt) * 0.5f, p0y - (vc.y * dt) * 0.5f, p0z - (vc.z * dt) * 0.5f);
    px = p0x - vi.x * dt;
    py = p0y - vi.y * dt;
    pz = p0z - vi.z * dt;
  }
#pragma unroll
  for (int c = 0; c < CH; c++) {
    const float* s = src + c * d.n;
    dst[c * d.n + idx] = kOrderSpace == 1 ? interp(d, s, px, py, pz) : interp_cubic<CH == 3>(d, s, px, py, pz);
  }
}

template <int CH, int kOrderSpace, int kTrace>
__global__ void __launch_bounds__(256) k_sl_cell(Dims d, CMac vel, const float* __restrict__ src, float* __restrict__ dst,
                                                 float dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  sl_real_cell<CH, kOrderSpace, kTrace>(d, vel, src, dst, dt, i, j, k);
}

// doClampComponent (advection.cpp:144-186) over CH planes.  Returns true
// when a fluid/empty corner was found (haveFl).
template <int CH>
__device__ __forceinline__ void clamp_component(const Dims& d, const int* __restrict__ flags, float* dv,
                                                const float* __restrict__ orig, const float* fwdv, float posx, float posy,
                                                float posz, V3 vel, int clampMode) {
  float mn[CH], mx[CH];
#pragma unroll
  for (int c = 0; c < CH; c++) { mn[c] = FLT_MAX; mx[c] = -FLT_MAX; }
  bool haveFl = false;
  const int np = clampMode == 1 ? 2 : 1;
  for (int l = 0; l < np; l++) {
    const float sg = l == 0 ? -1.f : 1.f;
    const int qx = (int)(l == 0 ? posx - vel.x : posx + vel.x);
    const int qy = (int)(l == 0 ? posy - vel.y : posy + vel.y);
    const int qz = (int)(l == 0 ? posz - vel.z : posz + vel.z);
    (void)sg;
    const int i0 = min(max(qx, 0), d.nx - 2);
    const int j0 = min(max(qy, 0), d.ny - 2);
    const int k0 = min(max(qz, 0), d.is3d ? d.nz - 2 : 1);
    const int k1 = d.is3d ? k0 + 1 : k0;
    const int nq = d.is3d ? 8 : 4;
    // the corners' flags and values are loaded together, then visited in
    // the reference's order (k0 plane first)
    int fl[8];
    float ov[8][CH];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const long long e = ix(d, i0 + (q & 1), j0 + ((q >> 1) & 1), q < 4 ? k0 : k1);
      fl[q] = __ldg(flags + e);
#pragma unroll
      for (int c = 0; c < CH; c++) ov[q][c] = __ldg(orig + c * d.n + e);
    }
#pragma unroll
    for (int q = 0; q < 8; q++) {
      if (q < nq && (fl[q] & (kFluid | kEmpty))) {
#pragma unroll
        for (int c = 0; c < CH; c++) {
          const float v = ov[q][c];
          if (v < mn[c]) mn[c] = v;
          if (v > mx[c]) mx[c] = v;
        }
        haveFl = true;
      }
    }
  }
  if (!haveFl) {
#pragma unroll
    for (int c = 0; c < CH; c++) dv[c] = fwdv[c];
    return;
  }
  if (clampMode == 1) {
#pragma unroll
    for (int c = 0; c < CH; c++) {
      if (dv[c] < mn[c]) dv[c] = mn[c];
      else if (dv[c] > mx[c]) dv[c] = mx[c];
    }
  } else {
    bool out = false;
#pragma unroll
    for (int c = 0; c < CH; c++) out |= (dv[c] < mn[c]) || (dv[c] > mx[c]);
    if (out) {
#pragma unroll
      for (int c = 0; c < CH; c++) dv[c] = fwdv[c];
    }
  }
}

// bwd = SL(fwd, -dt), MacCormackCorrect (advection.cpp:81-91) and
// MacCormackClamp (:241-267) in one sweep.  newGrid -> dst.
template <int CH, int kOrderSpace, int kTrace>
__device__ __forceinline__ void maccormack_real_cell(const Dims& d, const int* __restrict__ flags, CMac vel,
                                                         const float* __restrict__ orig, const float* __restrict__ fwd,
                                                         float* __restrict__ dst, float dt, float strength, int clampMode, int i, int j, int k) {
  const long long idx = ix(d, i, j, k);
  const bool fluid = isF(flags, idx);
  const float hs = strength * 0.5f;  // exact
  const bool inner = i >= 1 && i < d.nx - 1 && j >= 1 && j < d.ny - 1 && (!d.is3d || (k >= 1 && k < d.nz - 1));
  if (!inner) {
    // fwd and bwd are zero on the border; only the correction can be non-zero
#pragma unroll
    for (int c = 0; c < CH; c++) {
      float v = 0.f;
      const float o = __ldg(orig + c * d.n + idx);
      if (fluid) v = CH == 1 ? fmaf(hs, o - 0.f, 0.f) : 0.f + (hs * (o - 0.f));
      dst[c * d.n + idx] = v;
    }
    return;
  }
  const V3 vc = mac_centered(d, vel, idx);
  // backward trace through fwd with -dt: p0 - vc*(-dt) == p0 + vc*dt
  float px, py, pz;
  if (kTrace == 1) {
    px = (i + 0.5f) - vc.x * (-dt);
    py = (j + 0.5f) - vc.y * (-dt);
    pz = (k + 0.5f) - vc.z * (-dt);
  } else {
    const float p0x = i + 0.5f, p0y = j + 0.5f, p0z = k + 0.5f;
    const V3 vi = interp_mac(d, vel, p0x - (vc.x * (-dt)) * 0.5f, p0y - (vc.y * (-dt)) * 0.5f, p0z - (vc.z * (-dt)) * 0.5f);
    px = p0x - vi.x * (-dt);
    py = p0y - vi.y * (-dt);
    pz = p0z - vi.z * (-dt);
  }
  float dv[CH], fw[CH];
#pragma unroll
  for (int c = 0; c < CH; c++) {
    const float* f = fwd + c * d.n;
    const float bwd = kOrderSpace == 1 ? interp(d, f, px, py, pz) : interp_cubic<CH == 3>(d, f, px, py, pz);
    fw[c] = __ldg(f + idx);
    float v = fw[c];
    if (fluid) {
      const float diff = __ldg(orig + c * d.n + idx) - bwd;
      // Real: fwd + strength*0.5*(old-bwd) formed in double, one rounding.
      // Vec3: the double product rounds to float first, then the add.
      v = CH == 1 ? fmaf(hs, diff, v) : v + hs * diff;
    }
    dv[c] = v;
  }
  const V3 vd = {vc.x * dt, vc.y * dt, vc.z * dt};
  clamp_component<CH>(d, flags, dv, orig, fw, (float)i, (float)j, (float)k, vd, clampMode);
  if (clampMode == 1) {
    const int fx = (int)(((float)i + 0.5f) - vd.x), fy = (int)(((float)j + 0.5f) - vd.y), fz = (int)(((float)k + 0.5f) - vd.z);
    const int bx = (int)(((float)i + 0.5f) + vd.x), by = (int)(((float)j + 0.5f) + vd.y), bz = (int)(((float)k + 0.5f) + vd.z);
    const int gx = d.nx - 1, gy = d.ny - 1, gz = d.nz - 1;
    bool rev = fx < 0 || fy < 0 || fz < 0 || bx < 0 || by < 0 || bz < 0 || fx > gx || fy > gy || ((fz > gz) && d.is3d) ||
               bx > gx || by > gy || ((bz > gz) && d.is3d);
    if (!rev) rev = isO(flags, ix(d, fx, fy, fz)) || isO(flags, ix(d, bx, by, bz));
    if (rev) {
#pragma unroll
      for (int c = 0; c < CH; c++) dv[c] = fw[c];
    }
  }
#pragma unroll
  for (int c = 0; c < CH; c++) dst[c * d.n + idx] = dv[c];
}

template <int CH, int kOrderSpace, int kTrace>
__global__ void __launch_bounds__(256, 6) k_maccormack_cell(Dims d, const int* __restrict__ flags, CMac vel,
                                                         const float* __restrict__ orig, const float* __restrict__ fwd,
                                                         float* __restrict__ dst, float dt, float strength, int clampMode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  maccormack_real_cell<CH, kOrderSpace, kTrace>(d, flags, vel, orig, fwd, dst, dt, strength, clampMode, i, j, k);
}

// ------------------------------------------------------------------- MAC SL
// MACGrid::getInterpolatedComponentHi<c> (grid.h:268-274): orderSpace 1 is
// trilinear on the component's plane; orderSpace 2 is interpolCubicMAC's
// component (interpolHigh.h:171-178), the Vec3 Catmull-Rom sample half a
// cell further along the component's axis (0 for z in 2D).
template <int kOS>
__device__ __forceinline__ float sample_mac_comp(const Dims& d, const float* __restrict__ plane, int c, float x, float y,
                                                 float z) {
  if (kOS == 1) return interp(d, plane, x, y, z);
  if (c == 0) return interp_cubic<true>(d, plane, x + 0.5f, y, z);
  if (c == 1) return interp_cubic<true>(d, plane, x, y + 0.5f, z);
  if (!d.is3d) return 0.f;
  return interp_cubic<true>(d, plane, x, y, z + 0.5f);
}

// SemiLagrangeMAC (advection.cpp:44-77), src sampled per component.
template <int kTrace, int kOS>
__device__ __forceinline__ void sl_mac_cell(const Dims& d, CMac vel, CMac src, int i, int j, int k, float dt, float* out) {
  const long long idx = ix(d, i, j, k);
  if (kTrace == 1) {
    const V3 ax = mac_at_x(d, vel, idx);
    out[0] = sample_mac_comp<kOS>(d, src.u, 0, (i + 0.5f) - ax.x * dt, (j + 0.5f) - ax.y * dt, (k + 0.5f) - ax.z * dt);
    const V3 ay = mac_at_y(d, vel, idx);
    out[1] = sample_mac_comp<kOS>(d, src.v, 1, (i + 0.5f) - ay.x * dt, (j + 0.5f) - ay.y * dt, (k + 0.5f) - ay.z * dt);
    const V3 az = mac_at_z(d, vel, idx);
    out[2] = sample_mac_comp<kOS>(d, src.w, 2, (i + 0.5f) - az.x * dt, (j + 0.5f) - az.y * dt, (k + 0.5f) - az.z * dt);
  } else {
    // the midpoint trace samples src, as the reference does
    const float p0x = i + 0.5f, p0y = j + 0.5f, p0z = k + 0.5f;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float qx = c == 0 ? (float)i : i + 0.5f;
      const float qy = c == 1 ? (float)j : j + 0.5f;
      const float qz = c == 2 ? (float)k : k + 0.5f;
      const V3 a = c == 0 ? mac_at_x(d, src, idx) : (c == 1 ? mac_at_y(d, src, idx) : mac_at_z(d, src, idx));
      const V3 vi = interp_mac(d, src, qx - (a.x * dt) * 0.5f, qy - (a.y * dt) * 0.5f, qz - (a.z * dt) * 0.5f);
      out[c] = sample_mac_comp<kOS>(d, src.c(c), c, p0x - vi.x * dt, p0y - vi.y * dt, p0z - vi.z * dt);
    }
  }
}

template <int kTrace, int kOS>
__device__ __forceinline__ void sl_mac_grid_cell(const Dims& d, CMac vel, CMac src, Mac dst, float dt, int i, int j, int k) {
  const long long idx = ix(d, i, j, k);
  const bool inner = i >= 1 && i < d.nx - 1 && j >= 1 && j < d.ny - 1 && (!d.is3d || (k >= 1 && k < d.nz - 1));
  float out[3] = {0.f, 0.f, 0.f};
  if (inner) sl_mac_cell<kTrace, kOS>(d, vel, src, i, j, k, dt, out);
  dst.u[idx] = out[0];
  dst.v[idx] = out[1];
  dst.w[idx] = out[2];
}

template <int kTrace, int kOS>
__global__ void __launch_bounds__(256) k_sl_mac(Dims d, CMac vel, CMac src, Mac dst, float dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  sl_mac_grid_cell<kTrace, kOS>(d, vel, src, dst, dt, i, j, k);
}

// doClampComponentMAC (advection.cpp:191-235)
__device__ __forceinline__ float clamp_component_mac(const Dims& d, int fo, int fnb, float dst, const float* __restrict__ orig,
                                                     float fwd, int i, int j, int k, V3 vel, int clampMode) {
  // fo, fnb: flags of the cell and of its lower neighbour along the component
  float mn = FLT_MAX, mx = -FLT_MAX;
  const float posx = (float)i, posy = (float)j, posz = (float)k;
  if (clampMode == 2 && !((fo & (kFluid | kEmpty)) && (fnb & (kFluid | kEmpty)))) return fwd;
  const int np = clampMode == 1 ? 2 : 1;
  const int Y = (int)d.sy, Z = (int)d.sz;  // grids hold < 2^31 cells
  for (int l = 0; l < np; l++) {
    const int qx = (int)(l == 0 ? posx - vel.x : posx + vel.x);
    const int qy = (int)(l == 0 ? posy - vel.y : posy + vel.y);
    const int qz = (int)(l == 0 ? posz - vel.z : posz + vel.z);
    const int i0 = min(max(qx, 0), d.nx - 2);
    const int j0 = min(max(qy, 0), d.ny - 2);
    const int k0 = min(max(qz, 0), d.is3d ? d.nz - 2 : 0);
    const float* p = orig + (i0 + Y * j0 + Z * k0);
    const int nk = d.is3d ? 2 : 1;
    for (int kk = 0; kk < nk; kk++) {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const float v = __ldg(p + (q & 1) + Y * (q >> 1) + Z * kk);
        if (v < mn) mn = v;
        if (v > mx) mx = v;
      }
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

// bwd = SLMAC(fwd, -dt) on the fly, MacCormackCorrectMAC (advection.cpp:94-115),
// MacCormackClampMAC (:270-287).  orig is the grid being advected.
template <int kTrace, int kOS>
__device__ __forceinline__ void maccormack_mac_cell(const Dims& d, const int* __restrict__ flags, CMac vel, CMac orig,
                                                        CMac fwd, Mac dst, float dt, float strength, int clampMode, int i, int j, int k) {
  const long long idx = ix(d, i, j, k);
  bool skip[3];
  const int f0 = __ldg(flags + idx);
  const int fm[3] = {i > 0 ? __ldg(flags + idx - 1) : 0, j > 0 ? __ldg(flags + idx - d.sy) : 0,
                     k > 0 ? __ldg(flags + idx - d.sz) : 0};
  skip[0] = skip[1] = skip[2] = !(f0 & kFluid);
  if (i > 0 && !(fm[0] & kFluid)) skip[0] = true;
  if (j > 0 && !(fm[1] & kFluid)) skip[1] = true;
  if (k > 0 && !(fm[2] & kFluid)) skip[2] = true;
  const bool inner = i >= 1 && i < d.nx - 1 && j >= 1 && j < d.ny - 1 && (!d.is3d || (k >= 1 && k < d.nz - 1));
  const float hs = strength * 0.5f;
  float bwd[3] = {0.f, 0.f, 0.f};
  // face velocities, shared by the backward trace (order-1 trace) and the
  // clamp, which both sample vel at the cell's faces
  V3 ax{0.f, 0.f, 0.f}, ay{0.f, 0.f, 0.f}, az{0.f, 0.f, 0.f};
  if (inner) {
    ax = mac_at_x(d, vel, idx);
    ay = mac_at_y(d, vel, idx);
    az = mac_at_z(d, vel, idx);
    if (kTrace == 1) {
      // SemiLagrangeMAC(fwd, -dt), as sl_mac_cell<1> forms it
      const float mdt = -dt;
      bwd[0] = sample_mac_comp<kOS>(d, fwd.u, 0, (i + 0.5f) - ax.x * mdt, (j + 0.5f) - ax.y * mdt, (k + 0.5f) - ax.z * mdt);
      bwd[1] = sample_mac_comp<kOS>(d, fwd.v, 1, (i + 0.5f) - ay.x * mdt, (j + 0.5f) - ay.y * mdt, (k + 0.5f) - ay.z * mdt);
      bwd[2] = sample_mac_comp<kOS>(d, fwd.w, 2, (i + 0.5f) - az.x * mdt, (j + 0.5f) - az.y * mdt, (k + 0.5f) - az.z * mdt);
    } else {
      sl_mac_cell<kTrace, kOS>(d, vel, fwd, i, j, k, -dt, bwd);
    }
  }
  float fw[3], val[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    fw[c] = __ldg(fwd.c(c) + idx);
    val[c] = skip[c] ? fw[c] : fmaf(hs, __ldg(orig.c(c) + idx) - bwd[c], fw[c]);
  }
  if (inner) {
    val[0] = clamp_component_mac(d, f0, fm[0], val[0], orig.u, fw[0], i, j, k, V3{ax.x * dt, ax.y * dt, ax.z * dt}, clampMode);
    val[1] = clamp_component_mac(d, f0, fm[1], val[1], orig.v, fw[1], i, j, k, V3{ay.x * dt, ay.y * dt, ay.z * dt}, clampMode);
    if (d.is3d)
      val[2] = clamp_component_mac(d, f0, fm[2], val[2], orig.w, fw[2], i, j, k, V3{az.x * dt, az.y * dt, az.z * dt}, clampMode);
  }
  dst.u[idx] = val[0];
  dst.v[idx] = val[1];
  dst.w[idx] = val[2];
}

template <int kTrace, int kOS>
__global__ void __launch_bounds__(256, 5) k_maccormack_mac(Dims d, const int* __restrict__ flags, CMac vel, CMac orig,
                                                        CMac fwd, Mac dst, float dt, float strength, int clampMode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  maccormack_mac_cell<kTrace, kOS>(d, flags, vel, orig, fwd, dst, dt, strength, clampMode, i, j, k);
}

// extrapolateVelConvectiveBC (advection.cpp:346-381): velDst for outflow
// cells, from vel (the advected field) and velPrev (the field before).
__device__ __forceinline__ void outflow_bc_cell(const Dims& d, const int* __restrict__ flags, CMac vel, CMac velPrev, Mac velDst, float timeStep, int i, int j, int k) {
  const long long idx = ix(d, i, j, k);
  if (!isOut(flags, idx)) return;
  float ax = 0.f, ay = 0.f, az = 0.f;
  int count = 0;
  const int nmax = d.is3d ? 1 : 0;
  for (int nn = -nmax; nn <= nmax; nn++)
    for (int m = -1; m <= 1; m++)
      for (int l = -1; l <= 1; l++) {
        const int x = i + l, y = j + m, z = k + nn;
        if (x >= 0 && y >= 0 && z >= 0 && x < d.nx && y < d.ny && z < d.nz) {
          const long long e = ix(d, x, y, z);
          if (__ldg(flags + e) & (kFluid | kOutflow)) {
            ax += __ldg(vel.u + e);
            ay += __ldg(vel.v + e);
            az += __ldg(vel.w + e);
            count++;
          }
        }
      }
  float bulk[3] = {ax, ay, az};
  if (count > 0) {
    bulk[0] = ax / (float)count;
    bulk[1] = ay / (float)count;
    bulk[2] = az / (float)count;
  }
  const int dim = d.is3d ? 3 : 2;
  int cnt = 0;
  float dx = 0.f, dy = 0.f, dz = 0.f;
  const float cu = __ldg(vel.u + idx), cv = __ldg(vel.v + idx), cw = __ldg(vel.w + idx);
  const float pu = __ldg(velPrev.u + idx), pv = __ldg(velPrev.v + idx), pw = __ldg(velPrev.w + idx);
  const int cur[3] = {i, j, k};
  const int size[3] = {d.nx, d.ny, d.nz};
  const long long st[3] = {1, d.sy, d.sz};
  for (int c = 0; c < dim; c++) {
    const float factor = timeStep * (bulk[c] > 1.0f ? bulk[c] : 1.0f);
    int lo = cur[c] - 1, up = cur[c] + 1;
    for (int dd = 0; dd < 2; dd++) {
      const int fl = cur[c] - 1 - dd, fu = cur[c] + 1 + dd;
      const bool fromL = fl >= 0 && fl < size[c] && isF(flags, idx + (long long)(fl - cur[c]) * st[c]);
      const bool fromU = fu >= 0 && fu < size[c] && isF(flags, idx + (long long)(fu - cur[c]) * st[c]);
      if (fromL || fromU) {
        if (fromL) {
          const long long e = idx + (long long)(lo - cur[c]) * st[c];
          dx += ((cu - pu) / factor) + __ldg(vel.u + e);
          dy += ((cv - pv) / factor) + __ldg(vel.v + e);
          dz += ((cw - pw) / factor) + __ldg(vel.w + e);
          cnt++;
        }
        if (fromU) {
          const long long e = idx + (long long)(up - cur[c]) * st[c];
          dx += ((cu - pu) / factor) + __ldg(vel.u + e);
          dy += ((cv - pv) / factor) + __ldg(vel.v + e);
          dz += ((cw - pw) / factor) + __ldg(vel.w + e);
          cnt++;
        }
        break;
      }
    }
  }
  if (cnt > 0) {
    dx /= (float)cnt;
    dy /= (float)cnt;
    dz /= (float)cnt;
  }
  velDst.u[idx] = dx;
  velDst.v[idx] = dy;
  velDst.w[idx] = dz;
}

__global__ void k_outflow_bc(Dims d, const int* __restrict__ flags, CMac vel, CMac velPrev, Mac velDst, float timeStep) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  outflow_bc_cell(d, flags, vel, velPrev, velDst, timeStep, i, j, k);
}

// The same over four consecutive cells per thread: outflow cells are a
// boundary layer, so nearly every thread only reads its four flags (one
// 16-byte load) and returns.  n is a multiple of 4 (checked by the caller).
template <bool COPY>
__global__ void k_outflow_q(Dims d, const int* __restrict__ flags, CMac vel, CMac velPrev, Mac velDst, float timeStep) {
  const long long nq = d.n >> 2;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (long long)gridDim.x * blockDim.x) {
    const int4 f4 = __ldg(reinterpret_cast<const int4*>(flags) + q);
    if (!((f4.x | f4.y | f4.z | f4.w) & kOutflow)) continue;
    const int fl[4] = {f4.x, f4.y, f4.z, f4.w};
#pragma unroll 1
    for (int e = 0; e < 4; e++) {
      if (!(fl[e] & kOutflow)) continue;
      const long long idx = 4 * q + e;
      // grids hold fewer than 2^31 cells: 32-bit division
      const unsigned u = (unsigned)idx, q = u / (unsigned)d.nx, r = q / (unsigned)d.ny;
      const int i = (int)(u - q * (unsigned)d.nx), j = (int)(q - r * (unsigned)d.ny), k = (int)r;
      if (COPY) {
        velDst.u[idx] = vel.u[idx];
        velDst.v[idx] = vel.v[idx];
        velDst.w[idx] = vel.w[idx];
      } else {
        outflow_bc_cell(d, flags, vel, velPrev, velDst, timeStep, i, j, k);
      }
    }
  }
}

// copyChangedVels (advection.cpp:384)
__device__ __forceinline__ void copy_outflow_cell(const Dims& d, const int* __restrict__ flags, CMac src, Mac dst, int i, int j, int k) {
  const long long idx = ix(d, i, j, k);
  if (!isOut(flags, idx)) return;
  dst.u[idx] = src.u[idx];
  dst.v[idx] = src.v[idx];
  dst.w[idx] = src.w[idx];
}

__global__ void k_copy_outflow(Dims d, const int* __restrict__ flags, CMac src, Mac dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  copy_outflow_cell(d, flags, src, dst, i, j, k);
}

// knResetPhiInObs (advection.cpp:394-399)
__global__ void k_reset_phi_in_obs(Dims d, const int* __restrict__ flags, float* sdf) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= d.n) return;
  if (isO(flags, idx) && sdf[idx] < 0.f) sdf[idx] = 0.1f;
}

// ----------------------------------------------------------------- batched
// The plume's advection for every scene of a batch (advectSemiLagrange
// order 2, clampMode 2, of density and then of velocity, both with the
// velocity at the start of the step): the same cell bodies as above.
#define BATCH_CELL                                                       \
  const BTile tl = tiles[blockIdx.x];                                    \
  const BScene& sc = S[tl.scene];                                        \
  const Dims d = sc.d;                                                   \
  const int i = tl.x0 + threadIdx.x, j = tl.y0 + threadIdx.y, k = tl.z; \
  if (i >= d.nx || j >= d.ny) return;

// forward SL of density (into sc.fwd plane 3) and velocity (sc.fwd planes 0-2)
__global__ void __launch_bounds__(256) k_b_advect_fwd(const BTile* __restrict__ tiles, const BScene* __restrict__ S, int cur) {
  BATCH_CELL
  if (sc.kind != 0) return;  // plume scenes only
  const CMac v = bcmac(sc.vel[cur], d.n);
  sl_real_cell<1, 1, 1>(d, v, sc.dens[cur], sc.fwd + 3 * d.n, sc.dt, i, j, k);
  sl_mac_grid_cell<1, 1>(d, v, v, bmac(sc.fwd, d.n), sc.dt, i, j, k);
}
// MacCormack correction and clamp of both into the next buffers
__global__ void __launch_bounds__(256) k_b_advect_mc(const BTile* __restrict__ tiles, const BScene* __restrict__ S, int cur) {
  BATCH_CELL
  if (sc.kind != 0) return;  // plume scenes only
  const CMac v = bcmac(sc.vel[cur], d.n);
  maccormack_real_cell<1, 1, 1>(d, sc.flags, v, sc.dens[cur], sc.fwd + 3 * d.n, sc.dens[1 - cur], sc.dt, 1.f, 2, i, j, k);
  maccormack_mac_cell<1, 1>(d, sc.flags, v, v, bcmac(sc.fwd, d.n), bmac(sc.vel[1 - cur], d.n), sc.dt, 1.f, 2, i, j, k);
}
// applyOutflowBC (advection.cpp:387-391): convective values into the scratch
__global__ void __launch_bounds__(256) k_b_outflow(const BTile* __restrict__ tiles, const BScene* __restrict__ S, int cur) {
  BATCH_CELL
  if (sc.kind != 0) return;  // plume scenes only
  const float ts = fmaxf(1.f, sc.dt * 4.f);
  outflow_bc_cell(d, sc.flags, bcmac(sc.vel[1 - cur], d.n), bcmac(sc.vel[cur], d.n), bmac(sc.fwd, d.n), ts, i, j, k);
}
__global__ void __launch_bounds__(256) k_b_outflow_copy(const BTile* __restrict__ tiles, const BScene* __restrict__ S, int cur) {
  BATCH_CELL
  if (sc.kind != 0) return;  // plume scenes only
  copy_outflow_cell(d, sc.flags, bcmac(sc.fwd, d.n), bmac(sc.vel[1 - cur], d.n), i, j, k);
}
// dam break: advectSemiLagrange(phi, order 1) into the next buffer
__global__ void __launch_bounds__(256) k_b_dam_advect_phi(const BTile* __restrict__ tiles, const BScene* __restrict__ S,
                                                          int cur) {
  BATCH_CELL
  sl_real_cell<1, 1, 1>(d, bcmac(sc.vel[cur], d.n), sc.dens[cur], sc.dens[1 - cur], sc.dt, i, j, k);
}
// dam break: advectSemiLagrange(vel, order 1) into the next buffer (a closed
// box has no outflow cells, so applyOutflowBC changes nothing)
__global__ void __launch_bounds__(256) k_b_dam_advect_vel(const BTile* __restrict__ tiles, const BScene* __restrict__ S,
                                                          int cur) {
  BATCH_CELL
  const CMac v = bcmac(sc.vel[cur], d.n);
  sl_mac_grid_cell<1, 1>(d, v, v, bmac(sc.vel[1 - cur], d.n), sc.dt, i, j, k);
}
#undef BATCH_CELL

void launch_b_dam_advect_sl(const BTile* t, int nt, const BScene* s, int cur, bool vel, cudaStream_t st) {
  count_launch();
  if (vel) k_b_dam_advect_vel<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s, cur);
  else k_b_dam_advect_phi<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s, cur);
}

void launch_b_advect_density(const BTile* t, int nt, const BScene* s, int cur, cudaStream_t st) {
  (void)t; (void)nt; (void)s; (void)cur; (void)st;  // density and velocity advect together (launch_b_advect_velocity)
}
void launch_b_advect_velocity(const BTile* t, int nt, const BScene* s, int cur, cudaStream_t st) {
  const dim3 b(kBTX, kBTY, 1);
  count_launch();
  k_b_advect_fwd<<<nt, b, 0, st>>>(t, s, cur);
  count_launch();
  k_b_advect_mc<<<nt, b, 0, st>>>(t, s, cur);
  count_launch();
  k_b_outflow<<<nt, b, 0, st>>>(t, s, cur);
  count_launch();
  k_b_outflow_copy<<<nt, b, 0, st>>>(t, s, cur);
}

// ------------------------------------------------------------- launchers
static const dim3 kBlk(32, 8, 1);

template <int CH, int OS, int TR>
static void launch_sl(const Dims& d, CMac vel, const float* src, float* dst, float dt, cudaStream_t s) {
  count_launch();
  k_sl_cell<CH, OS, TR><<<grid3(d, kBlk), kBlk, 0, s>>>(d, vel, src, dst, dt);
}
template <int CH, int OS, int TR>
static void launch_mc(const Dims& d, const int* flags, CMac vel, const float* orig, const float* fwd, float* dst, float dt,
                      float strength, int clampMode, cudaStream_t s) {
  count_launch();
  k_maccormack_cell<CH, OS, TR><<<grid3(d, kBlk), kBlk, 0, s>>>(d, flags, vel, orig, fwd, dst, dt, strength, clampMode);
}

template <int CH>
static void dispatch_sl(const Dims& d, CMac vel, const float* src, float* dst, float dt, int os, int tr, cudaStream_t s) {
  if (os == 1 && tr == 1) launch_sl<CH, 1, 1>(d, vel, src, dst, dt, s);
  else if (os == 1) launch_sl<CH, 1, 2>(d, vel, src, dst, dt, s);
  else if (tr == 1) launch_sl<CH, 2, 1>(d, vel, src, dst, dt, s);
  else launch_sl<CH, 2, 2>(d, vel, src, dst, dt, s);
}
template <int CH>
static void dispatch_mc(const Dims& d, const int* flags, CMac vel, const float* orig, const float* fwd, float* dst, float dt,
                        float strength, int cm, int os, int tr, cudaStream_t s) {
  if (os == 1 && tr == 1) launch_mc<CH, 1, 1>(d, flags, vel, orig, fwd, dst, dt, strength, cm, s);
  else if (os == 1) launch_mc<CH, 1, 2>(d, flags, vel, orig, fwd, dst, dt, strength, cm, s);
  else if (tr == 1) launch_mc<CH, 2, 1>(d, flags, vel, orig, fwd, dst, dt, strength, cm, s);
  else launch_mc<CH, 2, 2>(d, flags, vel, orig, fwd, dst, dt, strength, cm, s);
}

void launch_advect_sl(const Dims& d, int ch, CMac vel, const float* src, float* dst, float dt, int orderSpace,
                      int orderTrace, cudaStream_t s) {
  if (ch == 1) dispatch_sl<1>(d, vel, src, dst, dt, orderSpace, orderTrace, s);
  else dispatch_sl<3>(d, vel, src, dst, dt, orderSpace, orderTrace, s);
}

void launch_advect_maccormack(const Dims& d, int ch, const int* flags, CMac vel, const float* orig, const float* fwd,
                              float* dst, float dt, float strength, int clampMode, int orderSpace, int orderTrace,
                              cudaStream_t s) {
  if (ch == 1) dispatch_mc<1>(d, flags, vel, orig, fwd, dst, dt, strength, clampMode, orderSpace, orderTrace, s);
  else dispatch_mc<3>(d, flags, vel, orig, fwd, dst, dt, strength, clampMode, orderSpace, orderTrace, s);
}

void launch_advect_sl_mac(const Dims& d, CMac vel, CMac src, Mac dst, float dt, int orderSpace, int orderTrace,
                         cudaStream_t s) {
  count_launch();
  const dim3 g = grid3(d, kBlk);
  if (orderSpace == 1) {
    if (orderTrace == 1) k_sl_mac<1, 1><<<g, kBlk, 0, s>>>(d, vel, src, dst, dt);
    else k_sl_mac<2, 1><<<g, kBlk, 0, s>>>(d, vel, src, dst, dt);
  } else {
    if (orderTrace == 1) k_sl_mac<1, 2><<<g, kBlk, 0, s>>>(d, vel, src, dst, dt);
    else k_sl_mac<2, 2><<<g, kBlk, 0, s>>>(d, vel, src, dst, dt);
  }
}

void launch_advect_maccormack_mac(const Dims& d, const int* flags, CMac vel, CMac orig, CMac fwd, Mac dst, float dt,
                                  float strength, int clampMode, int orderSpace, int orderTrace, cudaStream_t s) {
  count_launch();
  const dim3 g = grid3(d, kBlk);
  if (orderSpace == 1) {
    if (orderTrace == 1) k_maccormack_mac<1, 1><<<g, kBlk, 0, s>>>(d, flags, vel, orig, fwd, dst, dt, strength, clampMode);
    else k_maccormack_mac<2, 1><<<g, kBlk, 0, s>>>(d, flags, vel, orig, fwd, dst, dt, strength, clampMode);
  } else {
    if (orderTrace == 1) k_maccormack_mac<1, 2><<<g, kBlk, 0, s>>>(d, flags, vel, orig, fwd, dst, dt, strength, clampMode);
    else k_maccormack_mac<2, 2><<<g, kBlk, 0, s>>>(d, flags, vel, orig, fwd, dst, dt, strength, clampMode);
  }
}

void launch_outflow_bc(const Dims& d, const int* flags, CMac vel, CMac velPrev, Mac velDst, Mac velOut, float timeStep,
                       cudaStream_t s) {
  if ((d.n & 3) == 0) {
    // one quad per thread: a thread of the boundary layer then handles at
    // most four outflow cells
    const unsigned nb = (unsigned)((d.n / 4 + 255) / 256);
    count_launch();
    k_outflow_q<false><<<nb, 256, 0, s>>>(d, flags, vel, velPrev, velDst, timeStep);
    count_launch();
    k_outflow_q<true><<<nb, 256, 0, s>>>(d, flags, CMac{velDst.u, velDst.v, velDst.w}, CMac{nullptr, nullptr, nullptr},
                                         velOut, timeStep);
    return;
  }
  count_launch();
  k_outflow_bc<<<grid3(d, kBlk), kBlk, 0, s>>>(d, flags, vel, velPrev, velDst, timeStep);
  count_launch();
  k_copy_outflow<<<grid3(d, kBlk), kBlk, 0, s>>>(d, flags, CMac{velDst.u, velDst.v, velDst.w}, velOut);
}

void launch_reset_phi_in_obs(const Dims& d, const int* flags, float* sdf, cudaStream_t s) {
  count_launch();
  k_reset_phi_in_obs<<<(unsigned)((d.n + 255) / 256), 256, 0, s>>>(d, flags, sdf);
}

}  // namespace mgpu
