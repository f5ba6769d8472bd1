// Pressure projection on the GPU: plugin/pressure.cpp + conjugategrad.*.
//
//  * The Poisson matrix is not stored as four float grids.  A 16-bit stencil
//    code per cell (see mg_kernels.h) carries the same coefficients: A0 is a
//    small integer and every off-diagonal entry is 0 or -1 without
//    fractions, so the SpMV below performs exactly the reference's float
//    operations (x*A0 + x(c-X)*Ai(c-X) + ...) while reading 2 bytes of
//    matrix per cell instead of 16.  With ghost fluid the diagonal is kept
//    as a float grid.
//  * PCG scalars live on the device.  Reductions are two-level: per-block
//    (or per-tile) partials, then the last block to finish reduces them in
//    index order (deterministic) and updates the scalars.  Dot products
//    accumulate float products in double, as GridDotProduct does.
//  * MIC(0) (conjugategrad.cpp:66-97, 135-160) is a lexicographic recurrence.
//    The sweeps run as tiled wavefronts: 16^3 tiles dispatched in
//    i+j+k tile order to persistent CTAs, each tile waiting (bounded spin)
//    for its three upwind tiles, and inside a tile one thread per (y,z) line
//    stepping through the 46 cell levels.  Each cell sees exactly the values
//    the serial loop would, so the result is the reference's bit for bit.
#include "mg_common.cuh"
#include "mg_kernels.h"
#include "mg_tma.cuh"
#include "mg_reduce.cuh"
#include "mg_batch.h"

#include <algorithm>
#include <cfloat>
#include <cstdlib>
#include <string>

namespace mgpu {

static const dim3 kBlk(32, 8, 1);
static const int kThreads = 256;

#define CELL_IJK                                        \
  const int i = blockIdx.x * blockDim.x + threadIdx.x; \
  const int j = blockIdx.y * blockDim.y + threadIdx.y; \
  const int k = blockIdx.z;                             \
  if (i >= d.nx || j >= d.ny) return;                   \
  const long long idx = ix(d, i, j, k);

#define INNER (i >= 1 && i < d.nx - 1 && j >= 1 && j < d.ny - 1 && (!d.is3d || (k >= 1 && k < d.nz - 1)))

// ------------------------------------------------------------------ MakeRhs
// MakeRhs (pressure.cpp:32-84) without fractions/obvel.
__global__ void __launch_bounds__(256) k_make_rhs(Dims d, const int* __restrict__ flags, float* rhs, const float* __restrict__ vu,
                                                  const float* __restrict__ vv, const float* __restrict__ vw,
                                                  const float* __restrict__ corr, const float* __restrict__ phi,
                                                  const float* __restrict__ curv, float surfTens, float gfClamp,
                                                  double* part, CgScalars* sc, unsigned int nblk,
                                                  const float* __restrict__ frac, const float* __restrict__ obv);

__device__ __forceinline__ float theta_helper(float inside, float outside) {
  const float denom = inside - outside;
  if ((double)denom > -1e-04) return 0.5f;
  float r = inside / denom;
  r = r < 1.f ? r : 1.f;       // std::min(Real(1), .)
  return 0.f < r ? r : 0.f;    // std::max(Real(0), .)
}
// ghostFluidHelper (pressure.cpp:121-126): returns gfClamp when clamped,
// else (float)(1. - 1./alpha) computed in double (surface cells only)
__device__ __forceinline__ float gf_helper(const float* __restrict__ phi, long long idx, long long off, float gfClamp) {
  const float alpha = theta_helper(phi[idx], phi[idx + off]);
  if (alpha < gfClamp) return gfClamp;
  return (float)(1. - (1. / (double)alpha));
}
__device__ __forceinline__ float surf_tens_helper(const float* phi, const float* curv, long long idx, long long off,
                                                  float st, float gfc) {
  return st * (curv[idx + off] - gf_helper(phi, idx, off, gfc) * curv[idx]);
}

// -div(u) of a fluid cell as MakeRhs forms it
__device__ __forceinline__ float mac_neg_div(const Dims& d, const float* __restrict__ vu, const float* __restrict__ vv,
                                             const float* __restrict__ vw, long long idx) {
  float set = vu[idx] - vu[idx + 1] + vv[idx] - vv[idx + d.sy];
  if (d.is3d) set += vw[idx] - vw[idx + d.sz];
  return set;
}

__global__ void __launch_bounds__(256) k_make_rhs(Dims d, const int* __restrict__ flags, float* rhs, const float* __restrict__ vu,
                                                  const float* __restrict__ vv, const float* __restrict__ vw,
                                                  const float* __restrict__ corr, const float* __restrict__ phi,
                                                  const float* __restrict__ curv, float surfTens, float gfClamp,
                                                  double* part, CgScalars* sc, unsigned int nblk,
                                                  const float* __restrict__ frac, const float* __restrict__ obv) {
  double sum = 0.;
  double cnt = 0.;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i < d.nx && j < d.ny) {
    const long long idx = ix(d, i, j, k);
    if (INNER) {
      // the divergence's loads are issued with the flag load
      const float div = frac ? 0.f : mac_neg_div(d, vu, vv, vw, idx);
      if (!isF(flags, idx)) {
        rhs[idx] = 0.f;
      } else {
        float set;
        if (!frac) {
          set = div;
        } else {
          // the fraction-weighted divergence, and the obstacle velocity's
          // share of the faces (pressure.cpp:50-60)
          const float *fu = frac, *fv = frac + d.n, *fw = frac + 2 * d.n;
          const long long X = 1, Y = d.sy, Z = d.sz;
          set = fu[idx] * vu[idx] - fu[idx + X] * vu[idx + X] + fv[idx] * vv[idx] - fv[idx + Y] * vv[idx + Y];
          if (d.is3d) set += fw[idx] * vw[idx] - fw[idx + Z] * vw[idx + Z];
          if (obv) {
            const float *ou = obv, *ov = obv + d.n, *ow = obv + 2 * d.n;
            set += (1.f - fu[idx]) * ou[idx] - (1.f - fu[idx + X]) * ou[idx + X] + (1.f - fv[idx]) * ov[idx] -
                   (1.f - fv[idx + Y]) * ov[idx + Y];
            if (d.is3d) set += (1.f - fw[idx]) * ow[idx] - (1.f - fw[idx + Z]) * ow[idx + Z];
          }
        }
        if (phi && curv) {
          const long long X = 1, Y = d.sy, Z = d.sz;
          if (isE(flags, idx - X)) set += surf_tens_helper(phi, curv, idx, -X, surfTens, gfClamp);
          if (isE(flags, idx + X)) set += surf_tens_helper(phi, curv, idx, +X, surfTens, gfClamp);
          if (isE(flags, idx - Y)) set += surf_tens_helper(phi, curv, idx, -Y, surfTens, gfClamp);
          if (isE(flags, idx + Y)) set += surf_tens_helper(phi, curv, idx, +Y, surfTens, gfClamp);
          if (d.is3d) {
            if (isE(flags, idx - Z)) set += surf_tens_helper(phi, curv, idx, -Z, surfTens, gfClamp);
            if (isE(flags, idx + Z)) set += surf_tens_helper(phi, curv, idx, +Z, surfTens, gfClamp);
          }
        }
        if (corr) set += corr[idx];
        sum = set;
        cnt = 1.;
        rhs[idx] = set;
      }
    } else {
      rhs[idx] = 0.f;  // fresh grid: the border stays zero
    }
  }
  if (!nblk) return;  // the sums serve enforceCompatibility only
  const unsigned int b = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  const double bs = block_sum(sum);
  const double bc = block_sum(cnt);
  if (threadIdx.x + blockDim.x * threadIdx.y == 0) {
    part[2 * b] = bs;
    part[2 * b + 1] = bc;
  }
}

// rhs += (Real)(-sum / (Real)cnt) on every cell (pressure.cpp:296-297)
__global__ void k_compat_reduce(const double* part, int nb, CgScalars* sc) {
  const int nt = blockDim.x;
  double s = 0., c = 0.;
  for (int q = threadIdx.x; q < nb; q += nt) { s += __ldcg(part + 2 * q); c += __ldcg(part + 2 * q + 1); }
  s = block_sum(s);
  c = block_sum(c);
  if (threadIdx.x == 0) {
    sc->sum = s;
    sc->cnt = (int)c;
  }
}
__global__ void k_compat_shift(long long n, float* rhs, const CgScalars* sc) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const float add = (float)(-sc->sum / (double)(float)sc->cnt);
  rhs[idx] += add;
}

// ------------------------------------------------------- stencil codes
// MakeLaplaceMatrix (conjugategrad.h:154-187) as codes.  The batched form
// builds them in two passes (the single-scene path in one sweep,
// make_codes_full_cell below).  Pass 1: A0 count, fluid bit and the upward
// links of interior fluid cells.
__device__ __forceinline__ void make_codes_cell(const Dims& d, const int* __restrict__ flags, code_t* code, int i, int j, int k) {
  const long long idx = ix(d, i, j, k);
  const int f = __ldg(flags + idx);
  int c = (f & kFluid) ? kCodeFluid : 0;
  if (INNER) {
    // the six neighbours' flags are loaded with the cell's own
    const int fxm = __ldg(flags + idx - 1), fxp = __ldg(flags + idx + 1);
    const int fym = __ldg(flags + idx - d.sy), fyp = __ldg(flags + idx + d.sy);
    const int fzm = d.is3d ? __ldg(flags + idx - d.sz) : 0, fzp = d.is3d ? __ldg(flags + idx + d.sz) : 0;
    if (f & kFluid) {
      int a0 = 0;
      a0 += !(fxm & kObstacle);
      a0 += !(fxp & kObstacle);
      a0 += !(fym & kObstacle);
      a0 += !(fyp & kObstacle);
      if (d.is3d) {
        a0 += !(fzm & kObstacle);
        a0 += !(fzp & kObstacle);
      }
      c |= a0;
      if (fxp & kFluid) c |= kHighX;
      if (fyp & kFluid) c |= kHighY;
      if (d.is3d && (fzp & kFluid)) c |= kHighZ;
    }
  }
  code[idx] = (code_t)c;
}
// pass 2: lower links mirror the upper link of the lower neighbour
__device__ __forceinline__ void make_codes_low_cell(const Dims& d, code_t* code, int i, int j, int k) {
  const long long idx = ix(d, i, j, k);
  int c = code[idx];
  if (i > 0 && (code[idx - 1] & kHighX)) c |= kLowX;
  if (j > 0 && (code[idx - d.sy] & kHighY)) c |= kLowY;
  if (k > 0 && (code[idx - d.sz] & kHighZ)) c |= kLowZ;
  code[idx] = (code_t)c;
}

// both passes in one: a cell's lower links are its lower neighbours' upper
// links, which the flags decide directly (the neighbour is an interior
// fluid cell and this cell is fluid), so one sweep forms the whole code
__device__ __forceinline__ void make_codes_full_cell(const Dims& d, const int* __restrict__ flags, code_t* code, int i,
                                                     int j, int k) {
  const long long idx = ix(d, i, j, k);
  const bool xm = i > 0, xp = i < d.nx - 1, ym = j > 0, yp = j < d.ny - 1, zm = k > 0, zp = k < d.nz - 1;
  const int f = __ldg(flags + idx);
  const int fxm = __ldg(flags + (xm ? idx - 1 : idx)), fxp = __ldg(flags + (xp ? idx + 1 : idx));
  const int fym = __ldg(flags + (ym ? idx - d.sy : idx)), fyp = __ldg(flags + (yp ? idx + d.sy : idx));
  int fzm = 0, fzp = 0;
  if (d.is3d) {
    fzm = __ldg(flags + (zm ? idx - d.sz : idx));
    fzp = __ldg(flags + (zp ? idx + d.sz : idx));
  }
  const bool fl = f & kFluid;
  int c = fl ? kCodeFluid : 0;
  const bool iin = i >= 1 && i < d.nx - 1, jin = j >= 1 && j < d.ny - 1, kin = !d.is3d || (k >= 1 && k < d.nz - 1);
  if (fl && iin && jin && kin) {
    int a0 = 0;
    a0 += !(fxm & kObstacle);
    a0 += !(fxp & kObstacle);
    a0 += !(fym & kObstacle);
    a0 += !(fyp & kObstacle);
    if (d.is3d) {
      a0 += !(fzm & kObstacle);
      a0 += !(fzp & kObstacle);
    }
    c |= a0;
    if (fxp & kFluid) c |= kHighX;
    if (fyp & kFluid) c |= kHighY;
    if (d.is3d && (fzp & kFluid)) c |= kHighZ;
  }
  if (fl) {
    // the lower neighbour is interior: its own index inside, the others as here
    if (i >= 2 && i - 1 < d.nx - 1 && jin && kin && (fxm & kFluid)) c |= kLowX;
    if (j >= 2 && j - 1 < d.ny - 1 && iin && kin && (fym & kFluid)) c |= kLowY;
    if (d.is3d && k >= 2 && k - 1 < d.nz - 1 && iin && jin && (fzm & kFluid)) c |= kLowZ;
  }
  code[idx] = (code_t)c;
}

__global__ void k_make_codes_full(Dims d, const int* __restrict__ flags, code_t* code) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  make_codes_full_cell(d, flags, code, i, j, k);
}


// ApplyGhostFluidDiagonal (pressure.cpp:136-151): float diagonal
__device__ __forceinline__ void ghost_fluid_diag_cell(const Dims& d, const int* __restrict__ flags,
                                                      const code_t* __restrict__ code, const float* __restrict__ phi,
                                                      float gfClamp, float* A0f, int i, int j, int k,
                                                      const float* base = nullptr) {
  const long long idx = ix(d, i, j, k);
  float a = base ? base[idx] : (float)(code[idx] & 7);  // base: the fractions' diagonal
  if (INNER && isF(flags, idx)) {
    const long long X = 1, Y = d.sy, Z = d.sz;
    if (isE(flags, idx - X)) a -= gf_helper(phi, idx, -X, gfClamp);
    if (isE(flags, idx + X)) a -= gf_helper(phi, idx, +X, gfClamp);
    if (isE(flags, idx - Y)) a -= gf_helper(phi, idx, -Y, gfClamp);
    if (isE(flags, idx + Y)) a -= gf_helper(phi, idx, +Y, gfClamp);
    if (d.is3d) {
      if (isE(flags, idx - Z)) a -= gf_helper(phi, idx, -Z, gfClamp);
      if (isE(flags, idx + Z)) a -= gf_helper(phi, idx, +Z, gfClamp);
    }
  }
  A0f[idx] = a;
}
__global__ void k_ghost_fluid_diag(Dims d, const int* __restrict__ flags, const code_t* __restrict__ code,
                                   const float* __restrict__ phi, float gfClamp, float* A0f, int inPlace) {
  CELL_IJK
  (void)idx;
  ghost_fluid_diag_cell(d, flags, code, phi, gfClamp, A0f, i, j, k, inPlace ? A0f : nullptr);
}

// CountEmptyCells (pressure.cpp:217-220)
__global__ void k_count_empty(long long n, const int* __restrict__ flags, int* out) {
  int c = 0;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x)
    c += (__ldg(flags + idx) & kEmpty) ? 1 : 0;
  c = warp_sum(c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// fixPressure(fixPidx, 0, ...) (pressure.cpp:226-245): the rhs updates of
// the neighbours subtract A*0 and leave them unchanged.
__global__ void k_fix_pressure(Dims d, long long f, code_t* code, float* A0f, float* Ai, float* Aj, float* Ak,
                               float* rhs) {
  if (threadIdx.x != 0) return;
  rhs[f] = 0.f;
  code[f] = (code_t)((code[f] & kCodeFluid) | 1);
  if (A0f) A0f[f] = 1.f;
  if (Ai) {  // the stored matrix (fractions): the row's and the column's entries
    Ai[f] = Aj[f] = Ak[f] = 0.f;
    Ai[f - 1] = 0.f;
    Aj[f - d.sy] = 0.f;
    if (d.is3d) Ak[f - d.sz] = 0.f;
  }
  code[f - 1] &= (code_t)~kHighX;
  code[f + 1] &= (code_t)~kLowX;
  code[f - d.sy] &= (code_t)~kHighY;
  code[f + d.sy] &= (code_t)~kLowY;
  if (d.is3d) {
    code[f - d.sz] &= (code_t)~kHighZ;
    code[f + d.sz] &= (code_t)~kLowZ;
  }
}

__device__ __forceinline__ float diag(const code_t c, const float* A0f, long long idx) {
  return A0f ? A0f[idx] : (float)(c & 7);
}

// ------------------------------------------------------------------- PCG
// doInit part 1 (conjugategrad.cpp:209-216): dst=0, residual=rhs, tmp=0
__global__ void k_pcg_init(long long n, float* p, const float* __restrict__ rhs, float* r, float* tmp) {
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
    p[idx] = 0.f;
    r[idx] = rhs[idx];
    tmp[idx] = 0.f;
  }
}

// search = tmp; sigma = dot(tmp, residual) (conjugategrad.cpp:232-234)
__global__ void __launch_bounds__(256) k_pcg_set_search(long long n, const float* __restrict__ tmp,
                                                        const float* __restrict__ r, float* search, double* part,
                                                        CgScalars* sc) {
  FSum acc;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
    const float t = tmp[idx];
    search[idx] = t;
    acc.add(t * r[idx]);
  }
  const double b = block_sum(acc.value());
  if (threadIdx.x == 0) part[blockIdx.x] = b;
  if (last_block(&sc->counters[0], gridDim.x)) {
    const double s = sum_partials(part, gridDim.x);
    if (threadIdx.x == 0) sc->sigma = (float)s;
  }
}

// tmp = A*search (ApplyMatrix, conjugategrad.h:118-151) and dp = dot(tmp,
// search); the last block forms alpha = sigma/dp (conjugategrad.cpp:249-253)
__global__ void __launch_bounds__(256) k_pcg_spmv(Dims d, const code_t* __restrict__ code, const float* __restrict__ A0f,
                                                  const float* __restrict__ x, float* y, double* part, CgScalars* sc) {
  if (sc->done) return;
  FSum acc;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < d.n; idx += (long long)gridDim.x * blockDim.x) {
    const int c = code[idx];
    const float xc = x[idx];
    float v;
    if (!(c & kCodeFluid)) {
      v = xc;
    } else {
      v = xc * diag((code_t)c, A0f, idx);
      if (c & kLowX) v = v - x[idx - 1];
      if (c & kHighX) v = v - x[idx + 1];
      if (c & kLowY) v = v - x[idx - d.sy];
      if (c & kHighY) v = v - x[idx + d.sy];
      if (c & kLowZ) v = v - x[idx - d.sz];
      if (c & kHighZ) v = v - x[idx + d.sz];
    }
    y[idx] = v;
    acc.add(v * xc);
  }
  const double b = block_sum(acc.value());
  if (threadIdx.x == 0) part[blockIdx.x] = b;
  if (last_block(&sc->counters[1], gridDim.x)) {
    const double s = sum_partials(part, gridDim.x);
    if (threadIdx.x == 0) {
      const float dp = (float)s;
      sc->dp = dp;
      float alpha = 0.f;
      if (fabsf(dp) > 0.f) alpha = sc->sigma / dp;
      sc->alpha = alpha;
    }
  }
}

// dst += alpha*search, residual += -alpha*tmp, then the residual norm
// (max-abs, or sum of squares with useL2Norm) and the convergence test
// (conjugategrad.cpp:255-276).
__global__ void __launch_bounds__(256) k_pcg_axpy(long long n, float* p, const float* __restrict__ s, float* r,
                                                  const float* __restrict__ t, double* part, float* partf, CgScalars* sc) {
  if (sc->done) return;
  const float alpha = sc->alpha, na = -alpha;
  const int l2 = sc->useL2;
  float mn = FLT_MAX, mx = -FLT_MAX;
  double ss = 0.;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
    p[idx] = p[idx] + alpha * s[idx];
    const float rv = r[idx] + na * t[idx];
    r[idx] = rv;
    mn = fminf(mn, rv);
    mx = fmaxf(mx, rv);
    if (l2) ss += (double)rv * (double)rv;
  }
  block_minmax(mn, mx);
  const double bs = l2 ? block_sum(ss) : 0.;
  if (threadIdx.x == 0) {
    partf[2 * blockIdx.x] = mn;
    partf[2 * blockIdx.x + 1] = mx;
    part[blockIdx.x] = bs;
  }
  if (last_block(&sc->counters[2], gridDim.x)) {
    float res = 0.f;
    if (l2) {
      const double a = sum_partials(part, gridDim.x);
      res = (float)a;
    } else {
      float amin, amax;
      minmax_partials(partf, gridDim.x, amin, amax);
      const float x = fabsf(amin), y = fabsf(amax);
      res = x < y ? y : x;
    }
    if (threadIdx.x != 0) return;
    sc->iterations += 1;
    sc->resNorm = res;
    if (res < sc->accuracy) {
      sc->sigma = res;
      sc->done = 1;
    }
  }
}

// PcNone: tmp = residual and sigmaNew = dot(tmp, residual)
__global__ void __launch_bounds__(256) k_pcg_copy_dot(long long n, const float* __restrict__ r, float* tmp, double* part,
                                                      CgScalars* sc) {
  if (sc->done) return;
  FSum acc;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
    const float v = r[idx];
    tmp[idx] = v;
    acc.add(v * v);
  }
  const double b = block_sum(acc.value());
  if (threadIdx.x == 0) part[blockIdx.x] = b;
  if (last_block(&sc->counters[3], gridDim.x)) {
    const double s = sum_partials(part, gridDim.x);
    if (threadIdx.x != 0) return;
    const float sigmaNew = (float)s;
    sc->beta = sigmaNew / sc->sigma;
    sc->sigma = sigmaNew;
    if (!(sc->resNorm < 1e35f)) { sc->status = 2; sc->done = 1; }
  }
}

// search = tmp + beta*search (UpdateSearchVec, conjugategrad.cpp:193-196)
__global__ void k_pcg_update(long long n, const float* __restrict__ t, float* s, const CgScalars* sc) {
  if (sc->done) return;
  const float beta = sc->beta;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x)
    s[idx] = t[idx] + beta * s[idx];
}

// ---- four cells per thread (x size a multiple of 4, so a float4 never
// leaves its x-row and every row starts 16-byte aligned).  A thread keeps
// 48-64 bytes of loads in flight per iteration instead of 12-16, which is
// what it takes to cover HBM latency at full bandwidth.  Each cell performs
// the same float operations as the scalar kernels above.
__device__ __forceinline__ float fget(const float4& v, int e) { return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w; }

// The inputs of one quad (four x-consecutive cells): its stencil codes, x
// at the quad and its four y/z neighbour quads, and the x neighbours of its
// end cells.  Loaded before any arithmetic so that a thread keeps two quads'
// loads in flight.
struct SpmvQuad {
  uint2 cw;
  float4 xc, ylo, yhi, zlo, zhi, A0;
  float xl, xr;
};

__device__ __forceinline__ void spmv_load(const Dims& d, const code_t* __restrict__ code, const float* __restrict__ A0f,
                                          const float* __restrict__ x, long long q, SpmvQuad& Q) {
  const float4* x4 = reinterpret_cast<const float4*>(x);
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  Q.cw = __ldg(reinterpret_cast<const uint2*>(code) + q);
  const int any = (int)((Q.cw.x | Q.cw.y | (Q.cw.x >> 16) | (Q.cw.y >> 16)) & 0xffffu);
  Q.xc = __ldg(x4 + q);
  Q.ylo = (any & kLowY) ? __ldg(x4 + q - (d.sy >> 2)) : z4;
  Q.yhi = (any & kHighY) ? __ldg(x4 + q + (d.sy >> 2)) : z4;
  Q.zlo = (any & kLowZ) ? __ldg(x4 + q - (d.sz >> 2)) : z4;
  Q.zhi = (any & kHighZ) ? __ldg(x4 + q + (d.sz >> 2)) : z4;
  Q.xl = (Q.cw.x & kLowX) ? __ldg(x + (q << 2) - 1) : 0.f;
  Q.xr = ((Q.cw.y >> 16) & kHighX) ? __ldg(x + (q << 2) + 4) : 0.f;
  if (A0f) Q.A0 = __ldg(reinterpret_cast<const float4*>(A0f) + q);
  else
    Q.A0 = make_float4((float)(Q.cw.x & 7), (float)((Q.cw.x >> 16) & 7), (float)(Q.cw.y & 7),
                       (float)((Q.cw.y >> 16) & 7));
}

// ApplyMatrix (conjugategrad.h:118-151) on one quad, and its part of the
// fused dot(y, x)
__device__ __forceinline__ float4 spmv_apply(const SpmvQuad& Q, FSum& acc) {
  const int c[4] = {(int)(Q.cw.x & 0xffffu), (int)(Q.cw.x >> 16), (int)(Q.cw.y & 0xffffu), (int)(Q.cw.y >> 16)};
  float out[4];
#pragma unroll
  for (int e = 0; e < 4; e++) {
    const int ce = c[e];
    const float xv = fget(Q.xc, e);
    float v;
    if (!(ce & kCodeFluid)) {
      v = xv;
    } else {
      v = xv * fget(Q.A0, e);
      if (ce & kLowX) v = v - (e == 0 ? Q.xl : fget(Q.xc, e - 1));
      if (ce & kHighX) v = v - (e == 3 ? Q.xr : fget(Q.xc, e + 1));
      if (ce & kLowY) v = v - fget(Q.ylo, e);
      if (ce & kHighY) v = v - fget(Q.yhi, e);
      if (ce & kLowZ) v = v - fget(Q.zlo, e);
      if (ce & kHighZ) v = v - fget(Q.zhi, e);
    }
    out[e] = v;
    acc.add(v * xv);
  }
  return make_float4(out[0], out[1], out[2], out[3]);
}

// A thread takes the quads q, q + stride, q + 2 stride, ... two per loop
// trip, in that order (the dot's summation order does not depend on the
// pairing).
__global__ void __launch_bounds__(256, 4) k_pcg_spmv4(Dims d, const code_t* __restrict__ code,
                                                   const float* __restrict__ A0f, const float* __restrict__ x,
                                                   float* y, double* part, CgScalars* sc) {
  if (sc->done) return;
  FSum acc;
  const long long nq = d.n >> 2;
  const long long stride = (long long)gridDim.x * blockDim.x;
  float4* y4 = reinterpret_cast<float4*>(y);
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; q + stride < nq; q += 2 * stride) {
    SpmvQuad Q0, Q1;
    spmv_load(d, code, A0f, x, q, Q0);
    spmv_load(d, code, A0f, x, q + stride, Q1);
    y4[q] = spmv_apply(Q0, acc);
    y4[q + stride] = spmv_apply(Q1, acc);
  }
  if (q < nq) {
    SpmvQuad Q0;
    spmv_load(d, code, A0f, x, q, Q0);
    y4[q] = spmv_apply(Q0, acc);
  }
  const double b = block_sum(acc.value());
  if (threadIdx.x == 0) part[blockIdx.x] = b;
  if (last_block(&sc->counters[1], gridDim.x)) {
    const double s = sum_partials(part, gridDim.x);
    if (threadIdx.x == 0) {
      const float dp = (float)s;
      sc->dp = dp;
      float alpha = 0.f;
      if (fabsf(dp) > 0.f) alpha = sc->sigma / dp;
      sc->alpha = alpha;
    }
  }
}

// ---- the same SpMV marching along z in registers.  A thread owns one quad
// of one row and walks a run of zc planes; x of the planes below, at and
// above the quad rotate through registers, so every plane of x and of the
// codes is read from memory once per run.  While plane z is computed, the
// loads of plane z+1 (codes, the neighbouring rows' quads, the end cells' x
// neighbours) and x of plane z+2 are in flight.  The neighbouring rows are
// the quads of other threads of the CTA (L1) or of the next CTA (L2); their
// addresses are clamped into the grid so the loads need no test, and a
// clamped value is only read when the code has the link, which implies the
// neighbour exists.  Same cell arithmetic as k_pcg_spmv4; 0.63 of the
// measured copy peak in the plume step at 256^3 against 0.54 for the
// plane-streamed kernel below, which keeps two CTAs per SM.
struct ZmGeom {
  int nq, TY, zc;  // quads per row, rows per CTA, planes per CTA
};

// spmv_apply without branches: a non-fluid cell (code 0: no diagonal, no
// links) gives x * 1 = x, the reference's copy; a fluid cell x * A0 minus
// its linked neighbours in the reference's order.
__device__ __forceinline__ float4 spmv_apply_sel(const SpmvQuad& Q, FSum& acc) {
  const unsigned c[4] = {Q.cw.x & 0xffffu, Q.cw.x >> 16, Q.cw.y & 0xffffu, Q.cw.y >> 16};
  float out[4];
#pragma unroll
  for (int e = 0; e < 4; e++) {
    const unsigned ce = c[e];
    const float xv = fget(Q.xc, e);
    float v = xv * ((ce & kCodeFluid) ? fget(Q.A0, e) : 1.f);
    if (ce & kLowX) v = v - (e == 0 ? Q.xl : fget(Q.xc, e - 1));
    if (ce & kHighX) v = v - (e == 3 ? Q.xr : fget(Q.xc, e + 1));
    if (ce & kLowY) v = v - fget(Q.ylo, e);
    if (ce & kHighY) v = v - fget(Q.yhi, e);
    if (ce & kLowZ) v = v - fget(Q.zlo, e);
    if (ce & kHighZ) v = v - fget(Q.zhi, e);
    out[e] = v;
    acc.add(v * xv);
  }
  return make_float4(out[0], out[1], out[2], out[3]);
}

__global__ void __launch_bounds__(256, 4) k_pcg_spmv_zm(Dims d, ZmGeom g, const code_t* __restrict__ code,
                                                      const float* __restrict__ A0f, const float* __restrict__ x,
                                                      float* y, double* part, CgScalars* sc) {
  if (sc->done) return;
  FSum acc;
  const int r = threadIdx.x / g.nq, xq = threadIdx.x - r * g.nq;
  const int row = blockIdx.x * g.TY + r;
  const int zs = blockIdx.y * g.zc, ze = min(zs + g.zc, d.nz);
  if (r < g.TY && row < d.ny) {
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const int pq = (int)(d.sz >> 2);  // quads per plane; grids hold < 2^31 cells
    const int dn = row > 0 ? g.nq : 0, up = row + 1 < d.ny ? g.nq : 0;
    const int nlast = (int)d.n - 1;
    const float4* x4 = reinterpret_cast<const float4*>(x);
    const uint2* c2 = reinterpret_cast<const uint2*>(code);
    const float4* A4 = reinterpret_cast<const float4*>(A0f);
    float4* y4 = reinterpret_cast<float4*>(y);
    int q = zs * pq + row * g.nq + xq;
    // x below, at and above plane z (and x of plane z+2 in flight), the
    // codes and the neighbour rows / end cells of plane z
    float4 cm = zs > 0 ? __ldg(x4 + q - pq) : z4;
    float4 cc = __ldg(x4 + q);
    float4 cp = zs + 1 < d.nz ? __ldg(x4 + q + pq) : z4;
    uint2 cw = __ldg(c2 + q);
    float4 ylo = __ldg(x4 + q - dn), yhi = __ldg(x4 + q + up);
    float xl = __ldg(x + max(4 * q - 1, 0)), xr = __ldg(x + min(4 * q + 4, nlast));
#pragma unroll 2
    for (int z = zs; z < ze; z++) {
      const bool more = z + 1 < ze;
      const int qn = q + pq;
      float4 cn = z4, nylo = ylo, nyhi = yhi;
      uint2 ncw = cw;
      float nxl = xl, nxr = xr;
      if (more) {
        ncw = __ldg(c2 + qn);
        nylo = __ldg(x4 + qn - dn);
        nyhi = __ldg(x4 + qn + up);
        nxl = __ldg(x + (4 * qn - 1));  // qn >= pq > 0
        nxr = __ldg(x + min(4 * qn + 4, nlast));
        if (z + 2 < d.nz) cn = __ldg(x4 + qn + pq);
      }
      SpmvQuad Q;
      Q.cw = cw;
      Q.xc = cc;
      Q.ylo = ylo;
      Q.yhi = yhi;
      Q.zlo = cm;
      Q.zhi = cp;
      Q.xl = xl;
      Q.xr = xr;
      if (A0f) Q.A0 = __ldg(A4 + q);
      else
        Q.A0 = make_float4((float)(cw.x & 7u), (float)((cw.x >> 16) & 7u), (float)(cw.y & 7u), (float)((cw.y >> 16) & 7u));
      y4[q] = spmv_apply_sel(Q, acc);
      cm = cc;
      cc = cp;
      cp = cn;
      cw = ncw;
      ylo = nylo;
      yhi = nyhi;
      xl = nxl;
      xr = nxr;
      q = qn;
    }
  }
  const double b = block_sum(acc.value());
  const unsigned nb = gridDim.x * gridDim.y;
  if (threadIdx.x == 0) part[blockIdx.x + gridDim.x * blockIdx.y] = b;
  if (last_block(&sc->counters[1], nb)) {
    const double s2 = sum_partials(part, (int)nb);
    if (threadIdx.x == 0) {
      const float dp = (float)s2;
      sc->dp = dp;
      float alpha = 0.f;
      if (fabsf(dp) > 0.f) alpha = sc->sigma / dp;
      sc->alpha = alpha;
    }
  }
}

// ---- the same SpMV streamed plane by plane through shared memory.  A CTA
// owns a slab of TY full-width rows and a run of z planes, and keeps a ring
// of kStreamSlots planes in shared memory.  One producer warp fills the ring
// with bulk asynchronous copies (per plane: the slab's rows plus their y
// halo, and the plane's stencil codes), each completing a "full" mbarrier;
// eight consumer warps compute plane z from planes z-1, z and z+1 and hand
// the slot of plane z-1 back through an "empty" mbarrier.  No block-wide
// barrier runs per plane, so warps drift freely and the producer keeps up to
// kStreamSlots - 3 planes in flight.  x is read from DRAM once per plane (the
// y halo rows come from L2) and no neighbour is re-read from L2 by a gather.
// Same cell arithmetic as k_pcg_spmv4.
constexpr int kStreamSlots = 8;
// bytes of one ring slot at most (a multiple of 128): 8 slots of 14 KB keep
// two CTAs on an SM (2 x 112 KB) and give a 256-cell-wide grid slabs of 8
// rows, two quads per consumer thread, as the fastest measured setting
// (40.5 us at 256^3 against 44.6 us with 6-row slabs in 12 KB slots)
constexpr int kStreamSlotBudget = 14336;
constexpr int kStreamQuads = 2;                  // quads per consumer thread and plane at most
constexpr int kStreamConsumers = 256;            // consumer threads (8 warps); + 1 producer warp
constexpr long long kStreamWaitNs = 100000000LL;  // bound of one copy wait

struct StreamGeom {
  int TY, zc;                  // rows per slab, planes per CTA
  unsigned slotBytes, xBytes;  // ring slot size, offset of the code rows in a slot
};

__global__ void __launch_bounds__(kStreamConsumers + 32, 2)
    k_pcg_spmv_stream(Dims d, StreamGeom g, const code_t* __restrict__ code, const float* __restrict__ A0f,
                      const float* __restrict__ x, float* y, double* part, CgScalars* sc) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[kStreamSlots], empty[kStreamSlots];
  __shared__ int s_fail, s_issued;
  if (sc->done) return;
  const int nx = d.nx;
  const int y0 = blockIdx.x * g.TY, ty = min(g.TY, d.ny - y0);
  const int ya = max(y0 - 1, 0), yb = min(y0 + g.TY + 1, d.ny);
  const int zs = blockIdx.y * g.zc, ze = min(zs + g.zc, d.nz);
  const int p0 = zs - 1;        // plane of ring index 0
  const int np = ze + 1 - p0;   // ring indices 0 .. np-1: planes zs-1 .. ze
  const long long sz = d.sz;
  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int k = 0; k < kStreamSlots; k++) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], kStreamConsumers / 32);
    }
    s_fail = 0;
    s_issued = 0;
    mbar_fence_init();
  }
  __syncthreads();
  auto slotBase = [&](int i) { return smem + (size_t)(i % kStreamSlots) * g.slotBytes; };
  FSum acc;
  if (tid >= kStreamConsumers) {
    // ---- producer warp: lane 0 fills ring index i once its slot's previous
    // plane (ring index i - kStreamSlots) has been handed back
    if (tid == kStreamConsumers) {
      for (int i = 0; i < np; i++) {
        if (i >= kStreamSlots &&
            !mbar_wait(&empty[i % kStreamSlots], (unsigned)((i - kStreamSlots) / kStreamSlots) & 1u, kStreamWaitNs)) {
          atomicExch(&s_fail, 1);
          break;
        }
        if (*((volatile int*)&s_fail)) break;
        const int p = p0 + i;
        uint64_t* bar = &full[i % kStreamSlots];
        s_issued = i + 1;
        if (p < 0 || p >= d.nz) {
          mbar_arrive_expect(bar, 0);  // completes the slot's phase
          continue;
        }
        const unsigned xb = (unsigned)((yb - ya) * nx) * 4u;
        const bool withCode = p >= zs && p < ze;
        const unsigned cb = withCode ? (unsigned)(ty * nx) * 2u : 0u;
        mbar_arrive_expect(bar, xb + cb);
        bulk_g2s(slotBase(i), x + p * sz + (long long)ya * nx, xb, bar);
        if (withCode) bulk_g2s(slotBase(i) + g.xBytes, code + p * sz + (long long)y0 * nx, cb, bar);
      }
    }
  } else {
    // ---- consumers: this thread's quads of a plane (fixed for the CTA)
    const int nq4 = nx >> 2, quads = ty * nq4;
    int nmine = 0, ro[kStreamQuads], co[kStreamQuads], go[kStreamQuads];
    for (int e = tid; e < quads && nmine < kStreamQuads; e += kStreamConsumers) {
      const int r = e / nq4, xq = e - r * nq4;
      ro[nmine] = (y0 + r - ya) * nx + 4 * xq;  // the quad in a slot's x rows
      co[nmine] = r * nx + 4 * xq;              // its codes in the slot's code rows
      go[nmine] = (y0 + r) * nq4 + xq;          // its float4 index within a plane
      nmine++;
    }
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4* A4 = reinterpret_cast<const float4*>(A0f);
    float4* y4 = reinterpret_cast<float4*>(y);
    const bool leader = (tid & 31) == 0;
    int waited = 0;  // ring indices below this one have been waited for
    for (int z = zs; z < ze; z++) {
      const int ic = z - p0;
      bool ok = true;
      for (; waited <= ic + 1 && ok; waited++)
        ok = mbar_wait(&full[waited % kStreamSlots], (unsigned)(waited / kStreamSlots) & 1u, kStreamWaitNs);
      if (!__all_sync(0xffffffffu, ok) || *((volatile int*)&s_fail)) {
        if (leader) atomicExch(&s_fail, 1);
        break;
      }
      const float* xm = reinterpret_cast<const float*>(slotBase(ic - 1));
      const float* xcen = reinterpret_cast<const float*>(slotBase(ic));
      const float* xp = reinterpret_cast<const float*>(slotBase(ic + 1));
      const code_t* cs = reinterpret_cast<const code_t*>(slotBase(ic) + g.xBytes);
      const long long planeQ = ((long long)z * sz) >> 2;
#pragma unroll
      for (int u = 0; u < kStreamQuads; u++) {
        if (u < nmine) {
          const int o = ro[u];
          SpmvQuad Q;
          Q.cw = *reinterpret_cast<const uint2*>(cs + co[u]);
          const int any = (int)((Q.cw.x | Q.cw.y | (Q.cw.x >> 16) | (Q.cw.y >> 16)) & 0xffffu);
          Q.xc = *reinterpret_cast<const float4*>(xcen + o);
          Q.ylo = (any & kLowY) ? *reinterpret_cast<const float4*>(xcen + o - nx) : z4;
          Q.yhi = (any & kHighY) ? *reinterpret_cast<const float4*>(xcen + o + nx) : z4;
          Q.zlo = (any & kLowZ) ? *reinterpret_cast<const float4*>(xm + o) : z4;
          Q.zhi = (any & kHighZ) ? *reinterpret_cast<const float4*>(xp + o) : z4;
          Q.xl = (Q.cw.x & kLowX) ? xcen[o - 1] : 0.f;
          Q.xr = ((Q.cw.y >> 16) & kHighX) ? xcen[o + 4] : 0.f;
          const long long q = planeQ + go[u];
          if (A0f) Q.A0 = __ldg(A4 + q);
          else
            Q.A0 = make_float4((float)(Q.cw.x & 7), (float)((Q.cw.x >> 16) & 7), (float)(Q.cw.y & 7),
                               (float)((Q.cw.y >> 16) & 7));
          y4[q] = spmv_apply(Q, acc);
        }
      }
      // the warp is done with plane z-1 (read for the last time)
      __syncwarp();
      if (leader) mbar_arrive(&empty[(ic - 1) % kStreamSlots]);
    }
  }
  __syncthreads();
  if (s_fail) {
    // a copy wait ran out: let every copy in flight land (bounded) before the
    // block's shared memory is given up, and end the solve with an error
    if (tid == 0) {
      const int issued = s_issued;
      for (int i = issued > kStreamSlots ? issued - kStreamSlots : 0; i < issued; i++)
        mbar_wait(&full[i % kStreamSlots], (unsigned)(i / kStreamSlots) & 1u, kStreamWaitNs);
      sc->status = 4;
      sc->done = 1;
    }
    return;
  }
  const double b = block_sum(acc.value());
  const unsigned nb = gridDim.x * gridDim.y;
  if (tid == 0) part[blockIdx.x + gridDim.x * blockIdx.y] = b;
  if (last_block(&sc->counters[1], nb)) {
    const double s2 = sum_partials(part, (int)nb);
    if (tid == 0) {
      const float dp = (float)s2;
      sc->dp = dp;
      float alpha = 0.f;
      if (fabsf(dp) > 0.f) alpha = sc->sigma / dp;
      sc->alpha = alpha;
    }
  }
}

// Slab height and z run for the streamed SpMV, or false where it does not
// apply (2D, rows not a multiple of 8 cells, rows too long for a slab of 2).
static bool stream_geom(const Dims& d, int maxBlocks, int sms, StreamGeom* g, dim3* grid) {
  if (!d.is3d || d.nx % 8 != 0) return false;
  int TY = 16;
  while (TY >= 2 && (size_t)(TY + 2) * d.nx * 4 + (size_t)TY * d.nx * 2 > (size_t)kStreamSlotBudget) TY--;
  if (TY < 2 || (size_t)TY * (d.nx / 4) > (size_t)kStreamQuads * kStreamConsumers) return false;
  g->TY = TY;
  g->xBytes = (unsigned)((TY + 2) * d.nx * 4);
  g->slotBytes = (unsigned)(((size_t)g->xBytes + (size_t)TY * d.nx * 2 + 127) / 128 * 128);
  const int slabs = (d.ny + TY - 1) / TY;
  const int target = std::min(maxBlocks, 2 * sms);
  // at least 6 planes per CTA: the two halo planes of a run cost extra reads
  int chunks = std::max(1, std::min(std::max(1, d.nz / 6), target / std::max(1, slabs)));
  g->zc = (d.nz + chunks - 1) / chunks;
  chunks = (d.nz + g->zc - 1) / g->zc;
  if (slabs * chunks > maxBlocks) return false;
  *grid = dim3((unsigned)slabs, (unsigned)chunks, 1);
  return true;
}

// Quads per row, rows per CTA and the z run for the z-marching SpMV, or
// false where it does not apply (2D, rows not a multiple of 4 cells or
// longer than 1024 cells, more CTAs than the solver keeps partials for).
// The z runs are cut so that one wave of CTAs covers the grid.
static bool zm_geom(const Dims& d, int maxBlocks, int slots, ZmGeom* g, dim3* grid) {
  if (!d.is3d || (d.nx & 3) != 0 || d.nx / 4 > 256) return false;
  g->nq = d.nx / 4;
  g->TY = std::max(1, 256 / g->nq);
  const int rowsB = (d.ny + g->TY - 1) / g->TY;
  const int target = std::max(1, std::min(maxBlocks, slots));
  int chunks = std::max(1, std::min(std::max(1, d.nz / 4), target / rowsB));
  g->zc = (d.nz + chunks - 1) / chunks;
  chunks = (d.nz + g->zc - 1) / g->zc;
  if (rowsB * chunks > maxBlocks || rowsB > 65535) return false;
  *grid = dim3((unsigned)rowsB, (unsigned)chunks, 1);
  return true;
}

static int g_sms = 0;
enum { kSpmvQuad = 0, kSpmvStream = 1, kSpmvZm = 2 };
static int g_zmSlots = 0;  // resident CTAs of k_pcg_spmv_zm on the whole GPU

// the PCG matrix-vector kernel: z-marching in registers by default;
// MANTAGPU_SPMV=stream selects the plane-streamed one (shared-memory ring
// filled by bulk asynchronous copies), =quad the grid-stride quad kernel.
// Read at every launch, so a process can switch between solves.
static int spmv_mode() {
  const char* e = getenv("MANTAGPU_SPMV");
  if (e && std::string(e) == "quad") return kSpmvQuad;
  if (e && std::string(e) == "stream") return kSpmvStream;
  return kSpmvZm;
}

int pcg_prepare(int sms) {
  g_sms = sms;
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pcg_spmv_zm, 256, 0) != cudaSuccess || per < 1) per = 1;
  g_zmSlots = per * sms;
  const size_t smem = (size_t)kStreamSlots * kStreamSlotBudget;
  return cudaFuncSetAttribute(k_pcg_spmv_stream, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess
             ? 0
             : 1;
}

__global__ void __launch_bounds__(256) k_pcg_axpy4(long long n, float* p, const float* __restrict__ s, float* r,
                                                   const float* __restrict__ t, double* part, float* partf,
                                                   CgScalars* sc) {
  if (sc->done) return;
  const float alpha = sc->alpha, na = -alpha;
  const int l2 = sc->useL2;
  float mn = FLT_MAX, mx = -FLT_MAX;
  double ss = 0.;
  const long long nq = n >> 2;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (long long)gridDim.x * blockDim.x) {
    float4 pv = reinterpret_cast<const float4*>(p)[q];
    const float4 sv = __ldg(reinterpret_cast<const float4*>(s) + q);
    float4 rv = reinterpret_cast<const float4*>(r)[q];
    const float4 tv = __ldg(reinterpret_cast<const float4*>(t) + q);
    pv.x = pv.x + alpha * sv.x; pv.y = pv.y + alpha * sv.y; pv.z = pv.z + alpha * sv.z; pv.w = pv.w + alpha * sv.w;
    rv.x = rv.x + na * tv.x; rv.y = rv.y + na * tv.y; rv.z = rv.z + na * tv.z; rv.w = rv.w + na * tv.w;
    reinterpret_cast<float4*>(p)[q] = pv;
    reinterpret_cast<float4*>(r)[q] = rv;
    mn = fminf(fminf(mn, fminf(rv.x, rv.y)), fminf(rv.z, rv.w));
    mx = fmaxf(fmaxf(mx, fmaxf(rv.x, rv.y)), fmaxf(rv.z, rv.w));
    if (l2) {
      ss += (double)rv.x * (double)rv.x;
      ss += (double)rv.y * (double)rv.y;
      ss += (double)rv.z * (double)rv.z;
      ss += (double)rv.w * (double)rv.w;
    }
  }
  block_minmax(mn, mx);
  const double bs = l2 ? block_sum(ss) : 0.;
  if (threadIdx.x == 0) {
    partf[2 * blockIdx.x] = mn;
    partf[2 * blockIdx.x + 1] = mx;
    part[blockIdx.x] = bs;
  }
  if (last_block(&sc->counters[2], gridDim.x)) {
    float res = 0.f;
    if (l2) {
      const double a = sum_partials(part, gridDim.x);
      res = (float)a;
    } else {
      float amin, amax;
      minmax_partials(partf, gridDim.x, amin, amax);
      const float x = fabsf(amin), y = fabsf(amax);
      res = x < y ? y : x;
    }
    if (threadIdx.x != 0) return;
    sc->iterations += 1;
    sc->resNorm = res;
    if (res < sc->accuracy) {
      sc->sigma = res;
      sc->done = 1;
    }
  }
}

__global__ void __launch_bounds__(256) k_pcg_update4(long long n, const float* __restrict__ t, float* s,
                                                     const CgScalars* sc) {
  if (sc->done) return;
  const float beta = sc->beta;
  const long long nq = n >> 2;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (long long)gridDim.x * blockDim.x) {
    const float4 tv = __ldg(reinterpret_cast<const float4*>(t) + q);
    float4 sv = reinterpret_cast<const float4*>(s)[q];
    sv.x = tv.x + beta * sv.x; sv.y = tv.y + beta * sv.y; sv.z = tv.z + beta * sv.z; sv.w = tv.w + beta * sv.w;
    reinterpret_cast<float4*>(s)[q] = sv;
  }
}

// ---------------------------------------------------------------- MIC(0)
constexpr int T = 16;           // tile edge
constexpr int TC = T * T * T;   // cells per tile
constexpr int NL = 3 * T - 2;   // cell levels per tile

struct MicArgs {
  Dims d;
  const code_t* code;
  const float* A0f;
  float* P;
  const float* r;     // residual (forward input) / residual for the dot (backward)
  float* z;           // tmp
  double* part;       // per-tile dot partials (backward)
  CgScalars* sc;
  int tx, ty, tz, ntiles;
  const int* order;
  unsigned int* tileDone;
  int* counter;
  int* error;
  unsigned int epoch;
  long long spinLimit;
};

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned int* p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Wait (thread 0) until tile `t` carries this sweep's epoch; gives up after
// spinLimit nanoseconds, records the failure and lets the sweep finish.
__device__ __forceinline__ unsigned long long gtimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void wait_tile(const MicArgs& a, int t) {
  if (t < 0) return;
  const unsigned long long t0 = gtimer_ns();
  while (ld_acquire(a.tileDone + t) != a.epoch) {
    // once any wait has given up the sweep is already wrong: stop waiting
    if (gtimer_ns() - t0 > (unsigned long long)a.spinLimit || *((volatile int*)a.error) != 0) {
      atomicExch(a.error, 1);
      return;
    }
    __nanosleep(32);
  }
}

// MODE 0: InitPreconditionModifiedIncompCholesky2 -> P
// MODE 1: forward substitution r -> z
// MODE 2: backward substitution z -> z, plus dot(z, r) per tile
template <int MODE>
__global__ void __launch_bounds__(256) k_mic(MicArgs a) {
  __shared__ float s_val[TC];     // z (fwd/bwd) or P (init)
  __shared__ float s_P[TC];       // P (fwd/bwd) / A0 (init)
  __shared__ code_t s_code[TC];
  __shared__ float h_val[3][T * T];   // halo faces: value (z or P)
  __shared__ float h_P[3][T * T];     // halo faces: P (fwd/bwd)
  __shared__ code_t h_code[3][T * T]; // halo faces: code (init)
  __shared__ int s_tile;
  const Dims& d = a.d;
  const int tid = threadIdx.x;
  const int ly = tid & (T - 1), lz = tid >> 4;
  if (MODE != 0 && a.sc->done) return;  // converged before this application
  for (;;) {
    if (tid == 0) {
      const int q = atomicAdd(a.counter, 1);
      s_tile = q < a.ntiles ? (MODE == 2 ? a.order[a.ntiles - 1 - q] : a.order[q]) : -1;
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile < 0) return;
    const int ta = tile % a.tx, tb = (tile / a.tx) % a.ty, tcz = tile / (a.tx * a.ty);
    const int x0 = ta * T, y0 = tb * T, z0 = tcz * T;
    // stage this tile's inputs (independent of the neighbours)
    for (int e = tid; e < TC; e += kThreads) {
      const int x = x0 + (e & (T - 1)), y = y0 + ((e >> 4) & (T - 1)), zc = z0 + (e >> 8);
      code_t c = 0;
      float v = 0.f, p = 0.f;
      if (x < d.nx && y < d.ny && zc < d.nz) {
        const long long g = ix(d, x, y, zc);
        c = a.code[g];
        if (MODE == 0) {
          p = a.A0f ? a.A0f[g] : (float)(c & 7);
        } else {
          p = a.P[g];
          v = MODE == 1 ? a.r[g] : a.z[g];
        }
      }
      s_code[e] = c;
      s_P[e] = p;
      s_val[e] = v;
    }
    // wait for the upwind tiles (downwind for the backward sweep)
    if (tid == 0) {
      if (MODE == 2) {
        wait_tile(a, ta + 1 < a.tx ? tile + 1 : -1);
        wait_tile(a, tb + 1 < a.ty ? tile + a.tx : -1);
        wait_tile(a, tcz + 1 < a.tz ? tile + a.tx * a.ty : -1);
      } else {
        wait_tile(a, ta > 0 ? tile - 1 : -1);
        wait_tile(a, tb > 0 ? tile - a.tx : -1);
        wait_tile(a, tcz > 0 ? tile - a.tx * a.ty : -1);
      }
    }
    __syncthreads();
    // halo faces from the neighbours (written by other CTAs: bypass L1)
    for (int f = 0; f < 3; f++) {
      const int u = tid & (T - 1), w = tid >> 4;  // face coordinates
      int x, y, zc;
      if (f == 0) { x = MODE == 2 ? x0 + T : x0 - 1; y = y0 + u; zc = z0 + w; }
      else if (f == 1) { x = x0 + u; y = MODE == 2 ? y0 + T : y0 - 1; zc = z0 + w; }
      else { x = x0 + u; y = y0 + w; zc = MODE == 2 ? z0 + T : z0 - 1; }
      float hv = 0.f, hp = 0.f;
      code_t hc = 0;
      if (x >= 0 && y >= 0 && zc >= 0 && x < d.nx && y < d.ny && zc < d.nz) {
        const long long g = ix(d, x, y, zc);
        hc = a.code[g];
        if (MODE == 0) {
          hv = __ldcg(a.P + g);
        } else {
          hv = __ldcg(a.z + g);
          hp = a.P[g];
        }
      }
      h_val[f][tid] = hv;
      h_P[f][tid] = hp;
      h_code[f][tid] = hc;
    }
    __syncthreads();
    double acc = 0.;
    // the wavefront: thread (ly, lz) owns the x-line of the tile
    for (int s = 0; s < NL; s++) {
      const int L = MODE == 2 ? NL - 1 - s : s;
      const int x = L - ly - lz;
      if (x >= 0 && x < T) {
        const int e = x + T * ly + T * T * lz;
        const int c = s_code[e];
        if (MODE == 0) {
          float pv = 0.f;
          if (c & kCodeFluid) {
            // neighbour P values and the codes of the lower neighbours
            const float px = x > 0 ? s_val[e - 1] : h_val[0][ly + T * lz];
            const float py = ly > 0 ? s_val[e - T] : h_val[1][x + T * lz];
            const float pz = lz > 0 ? s_val[e - T * T] : h_val[2][x + T * ly];
            const int cx = x > 0 ? s_code[e - 1] : h_code[0][ly + T * lz];
            const int cy = ly > 0 ? s_code[e - T] : h_code[1][x + T * lz];
            const int cz = lz > 0 ? s_code[e - T * T] : h_code[2][x + T * ly];
            const float A0 = s_P[e];
            float ev = A0;
            if (c & kLowX) ev = ev - px * px;
            if (c & kLowY) ev = ev - py * py;
            if (c & kLowZ) ev = ev - pz * pz;
            // Ai(c-x)*(Aj(c-x)+Ak(c-x)) etc. are 0, 1 or 2
            const float k1 = (c & kLowX) ? (float)(((cx & kHighY) ? 1 : 0) + ((cx & kHighZ) ? 1 : 0)) : 0.f;
            const float k2 = (c & kLowY) ? (float)(((cy & kHighX) ? 1 : 0) + ((cy & kHighZ) ? 1 : 0)) : 0.f;
            const float k3 = (c & kLowZ) ? (float)(((cz & kHighX) ? 1 : 0) + ((cz & kHighY) ? 1 : 0)) : 0.f;
            const float t1 = k1 * (px * px), t2 = k2 * (py * py), t3 = k3 * (pz * pz);
            const float S = (t1 + t2) + t3;
            ev = fmaf(-0.97f, S, ev);       // e -= tau*(...) in double, one rounding
            if (ev < 0.25f * A0) ev = A0;   // stability cutoff sigma = 0.25
            pv = 1.f / sqrtf(ev);
          }
          s_val[e] = pv;
        } else if (MODE == 1) {
          float zv = 0.f;
          if (c & kCodeFluid) {
            float t = s_val[e];
            if (c & kLowX) t = t + (x > 0 ? s_val[e - 1] * s_P[e - 1] : h_val[0][ly + T * lz] * h_P[0][ly + T * lz]);
            if (c & kLowY) t = t + (ly > 0 ? s_val[e - T] * s_P[e - T] : h_val[1][x + T * lz] * h_P[1][x + T * lz]);
            if (c & kLowZ) t = t + (lz > 0 ? s_val[e - T * T] * s_P[e - T * T] : h_val[2][x + T * ly] * h_P[2][x + T * ly]);
            zv = s_P[e] * t;
          }
          s_val[e] = zv;
        } else {
          float zv = 0.f;
          if (c & kCodeFluid) {
            const float p = s_P[e];
            float t = s_val[e];
            if (c & kHighX) t = t + (x < T - 1 ? s_val[e + 1] : h_val[0][ly + T * lz]) * p;
            if (c & kHighY) t = t + (ly < T - 1 ? s_val[e + T] : h_val[1][x + T * lz]) * p;
            if (c & kHighZ) t = t + (lz < T - 1 ? s_val[e + T * T] : h_val[2][x + T * ly]) * p;
            zv = p * t;
          }
          s_val[e] = zv;
        }
      }
      __syncthreads();
    }
    // write back, and the fused dot(z, residual) for the backward sweep
    for (int e = tid; e < TC; e += kThreads) {
      const int x = x0 + (e & (T - 1)), y = y0 + ((e >> 4) & (T - 1)), zc = z0 + (e >> 8);
      if (x < d.nx && y < d.ny && zc < d.nz) {
        const long long g = ix(d, x, y, zc);
        if (MODE == 0) {
          a.P[g] = s_val[e];
        } else {
          a.z[g] = s_val[e];
          if (MODE == 2) acc += (double)(s_val[e] * a.r[g]);
        }
      }
    }
    if (MODE == 2) {
      const double b = block_sum(acc);
      if (tid == 0) a.part[tile] = b;
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      st_release(a.tileDone + tile, a.epoch);
    }
  }
}

// sigmaNew = sum of per-tile partials in tile order; beta; divergence check
__global__ void k_mic_finish_dot(const double* part, int ntiles, CgScalars* sc) {
  if (sc->done) return;
  const double s = sum_partials(part, ntiles);
  if (threadIdx.x != 0) return;
  const float sigmaNew = (float)s;
  sc->beta = sigmaNew / sc->sigma;
  sc->sigma = sigmaNew;
  if (!(sc->resNorm < 1e35f)) { sc->status = 2; sc->done = 1; }
}

// sigma for doInit after the first MIC application
__global__ void k_mic_init_sigma(const double* part, int ntiles, CgScalars* sc) {
  const double s = sum_partials(part, ntiles);
  if (threadIdx.x == 0) sc->sigma = (float)s;
}

// ------------------------------------------------------- correctVelocity
// knCorrectVelocity (pressure.cpp:87-109); every load is issued before the
// flag tests
__device__ __forceinline__ void correct_velocity_cell(const Dims& d, const int* __restrict__ flags, Mac vel, const float* __restrict__ p, int i, int j, int k) {
  const long long idx = ix(d, i, j, k);
  if (!INNER) return;
  const long long X = 1, Y = d.sy, Z = d.sz;
  const int f = __ldg(flags + idx), fxm = __ldg(flags + idx - X), fym = __ldg(flags + idx - Y);
  const int fzm = d.is3d ? __ldg(flags + idx - Z) : 0;
  const float pc = p[idx], pxm = p[idx - X], pym = p[idx - Y];
  const float pzm = d.is3d ? p[idx - Z] : 0.f;
  float u = vel.u[idx], v = vel.v[idx], w = vel.w[idx];
  if (f & kFluid) {
    if (fxm & kFluid) u -= (pc - pxm);
    if (fym & kFluid) v -= (pc - pym);
    if (d.is3d && (fzm & kFluid)) w -= (pc - pzm);
    if (fxm & kEmpty) u -= pc;
    if (fym & kEmpty) v -= pc;
    if (d.is3d && (fzm & kEmpty)) w -= pc;
    vel.u[idx] = u; vel.v[idx] = v; vel.w[idx] = w;
  } else if ((f & kEmpty) && !(f & kOutflow)) {
    if (fxm & kFluid) u += pxm; else u = 0.f;
    if (fym & kFluid) v += pym; else v = 0.f;
    if (d.is3d) { if (fzm & kFluid) w += pzm; else w = 0.f; }
    vel.u[idx] = u; vel.v[idx] = v; vel.w[idx] = w;
  }
}

__global__ void k_correct_velocity(Dims d, const int* __restrict__ flags, Mac vel, const float* __restrict__ p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  correct_velocity_cell(d, flags, vel, p, i, j, k);
}

// knCorrectVelocityGhostFluid (pressure.cpp:154-187)
__device__ __forceinline__ void correct_velocity_gf_cell(const Dims& d, const int* __restrict__ flags, Mac vel,
                                                         const float* __restrict__ p, const float* __restrict__ phi,
                                                         float gfc, const float* __restrict__ curv, float st, int i,
                                                         int j, int k) {
  const long long idx = ix(d, i, j, k);
  if (!INNER) return;
  const long long X = 1, Y = d.sy, Z = d.sz;
  float u = vel.u[idx], v = vel.v[idx], w = vel.w[idx];
  if (isF(flags, idx)) {
    if (isE(flags, idx - X)) u += p[idx] * gf_helper(phi, idx, -X, gfc);
    if (isE(flags, idx - Y)) v += p[idx] * gf_helper(phi, idx, -Y, gfc);
    if (d.is3d && isE(flags, idx - Z)) w += p[idx] * gf_helper(phi, idx, -Z, gfc);
  } else if (isE(flags, idx) && !isOut(flags, idx)) {
    if (isF(flags, idx - X)) u -= p[idx - X] * gf_helper(phi, idx - X, +X, gfc); else u = 0.f;
    if (isF(flags, idx - Y)) v -= p[idx - Y] * gf_helper(phi, idx - Y, +Y, gfc); else v = 0.f;
    if (d.is3d) { if (isF(flags, idx - Z)) w -= p[idx - Z] * gf_helper(phi, idx - Z, +Z, gfc); else w = 0.f; }
  }
  if (curv) {
    if (isF(flags, idx)) {
      if (isE(flags, idx - X)) u += surf_tens_helper(phi, curv, idx, -X, st, gfc);
      if (isE(flags, idx - Y)) v += surf_tens_helper(phi, curv, idx, -Y, st, gfc);
      if (d.is3d && isE(flags, idx - Z)) w += surf_tens_helper(phi, curv, idx, -Z, st, gfc);
    } else if (isE(flags, idx) && !isOut(flags, idx)) {
      u -= isF(flags, idx - X) ? surf_tens_helper(phi, curv, idx - X, +X, st, gfc) : 0.f;
      v -= isF(flags, idx - Y) ? surf_tens_helper(phi, curv, idx - Y, +Y, st, gfc) : 0.f;
      if (d.is3d) w -= isF(flags, idx - Z) ? surf_tens_helper(phi, curv, idx - Z, +Z, st, gfc) : 0.f;
    }
  }
  vel.u[idx] = u; vel.v[idx] = v; vel.w[idx] = w;
}

// knReplaceClampedGhostFluidVels (pressure.cpp:198-214): writes only empty
// cells and reads only fluid ones, so it is race free in place.
__global__ void k_correct_velocity_gf(Dims d, const int* __restrict__ flags, Mac vel, const float* __restrict__ p,
                                      const float* __restrict__ phi, float gfc, const float* __restrict__ curv, float st) {
  CELL_IJK
  (void)idx;
  correct_velocity_gf_cell(d, flags, vel, p, phi, gfc, curv, st, i, j, k);
}

__device__ __forceinline__ void replace_clamped_gf_cell(const Dims& d, const int* __restrict__ flags, Mac vel,
                                                        const float* __restrict__ phi, float gfc, int i, int j, int k) {
  const long long idx = ix(d, i, j, k);
  if (!INNER) return;
  if (!isE(flags, idx)) return;
  const long long X = 1, Y = d.sy, Z = d.sz;
#define CLAMPED(e, off) (theta_helper(phi[(e)], phi[(e) + (off)]) < gfc)
  if (isF(flags, idx - X) && CLAMPED(idx - X, +X)) vel.u[idx] = vel.u[idx - X];
  if (isF(flags, idx - Y) && CLAMPED(idx - Y, +Y)) vel.v[idx] = vel.v[idx - Y];
  if (d.is3d && isF(flags, idx - Z) && CLAMPED(idx - Z, +Z)) vel.w[idx] = vel.w[idx - Z];
  if (isF(flags, idx + X) && CLAMPED(idx + X, -X)) vel.u[idx] = vel.u[idx + X];
  if (isF(flags, idx + Y) && CLAMPED(idx + Y, -Y)) vel.v[idx] = vel.v[idx + Y];
  if (d.is3d && isF(flags, idx + Z) && CLAMPED(idx + Z, -Z)) vel.w[idx] = vel.w[idx + Z];
#undef CLAMPED
}
__global__ void k_replace_clamped_gf(Dims d, const int* __restrict__ flags, Mac vel, const float* __restrict__ phi, float gfc) {
  CELL_IJK
  (void)idx;
  replace_clamped_gf_cell(d, flags, vel, phi, gfc, i, j, k);
}

// ---------------------------------------------------- stored coefficients
// With fractions the Poisson matrix has float off-diagonals: it is stored as
// the reference stores it (A0, Ai, Aj, Ak), and the SpMV and MIC(0) read the
// floats.  The stencil codes still carry the fluid bit and the links.

// MakeLaplaceMatrix with fractions (conjugategrad.h:172-186)
__global__ void k_make_frac_matrix(Dims d, const int* __restrict__ flags, const float* __restrict__ frac, float* A0,
                                   float* Ai, float* Aj, float* Ak) {
  CELL_IJK
  float a0 = 0.f, ai = 0.f, aj = 0.f, ak = 0.f;
  if (INNER && isF(flags, idx)) {
    const float *fu = frac, *fv = frac + d.n, *fw = frac + 2 * d.n;
    const long long X = 1, Y = d.sy, Z = d.sz;
    a0 += fu[idx];
    a0 += fu[idx + X];
    a0 += fv[idx];
    a0 += fv[idx + Y];
    if (d.is3d) {
      a0 += fw[idx];
      a0 += fw[idx + Z];
    }
    if (isF(flags, idx + X)) ai = -fu[idx + X];
    if (isF(flags, idx + Y)) aj = -fv[idx + Y];
    if (d.is3d && isF(flags, idx + Z)) ak = -fw[idx + Z];
  }
  A0[idx] = a0;
  Ai[idx] = ai;
  Aj[idx] = aj;
  Ak[idx] = ak;
}

// ApplyMatrix (conjugategrad.h:118-132) with the stored floats: the terms of
// absent links (zero coefficients) are left out, which adds nothing; fused
// dot(tmp, search) -> alpha as in k_pcg_spmv4
__global__ void __launch_bounds__(256) k_pcg_spmv_stored(Dims d, const code_t* __restrict__ code,
                                                         const float* __restrict__ A0, const float* __restrict__ Ai,
                                                         const float* __restrict__ Aj, const float* __restrict__ Ak,
                                                         const float* __restrict__ x, float* y, double* part,
                                                         CgScalars* sc) {
  if (sc->done) return;
  FSum acc;
  const long long Y = d.sy, Z = d.sz;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < d.n;
       idx += (long long)gridDim.x * blockDim.x) {
    const int c = code[idx];
    const float xv = x[idx];
    float v = xv;
    if (c & kCodeFluid) {
      v = xv * A0[idx];
      if (c & kLowX) v = v + x[idx - 1] * Ai[idx - 1];
      if (c & kHighX) v = v + x[idx + 1] * Ai[idx];
      if (c & kLowY) v = v + x[idx - Y] * Aj[idx - Y];
      if (c & kHighY) v = v + x[idx + Y] * Aj[idx];
      if (c & kLowZ) v = v + x[idx - Z] * Ak[idx - Z];
      if (c & kHighZ) v = v + x[idx + Z] * Ak[idx];
    }
    y[idx] = v;
    acc.add(v * xv);
  }
  const double b = block_sum(acc.value());
  if (threadIdx.x == 0) part[blockIdx.x] = b;
  if (last_block(&sc->counters[1], gridDim.x)) {
    const double s2 = sum_partials(part, gridDim.x);
    if (threadIdx.x == 0) {
      const float dp = (float)s2;
      sc->dp = dp;
      sc->alpha = fabsf(dp) > 0.f ? sc->sigma / dp : 0.f;
    }
  }
}

// InitPreconditionModifiedIncompCholesky2 / ApplyPreconditionModifiedIncomp-
// Cholesky2 (conjugategrad.cpp:66-97, 135-160) on the cells of one plane
// i + j + k = L, with the stored floats.  The cells of a plane depend only
// on the plane before (forward) or after (backward), so plane by plane is the
// reference's lexicographic result.  MODE 0 factor, 1 forward, 2 backward.
template <int MODE>
__global__ void k_mic_plane(Dims d, int L, const code_t* __restrict__ code, const float* __restrict__ A0,
                            const float* __restrict__ Ai, const float* __restrict__ Aj, const float* __restrict__ Ak,
                            float* P, const float* __restrict__ r, float* z, const CgScalars* sc) {
  if (MODE != 0 && sc->done) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  const int i = L - j - k;
  if (j >= d.ny || i < 0 || i >= d.nx) return;
  const long long idx = ix(d, i, j, k), Y = d.sy, Z = d.sz;
  const bool fl = (code[idx] & kCodeFluid) != 0;
  if (MODE == 0) {
    float pv = 0.f;
    if (fl) {
      float e = A0[idx];
      float S = 0.f;
      if (i > 0) {
        const long long q = idx - 1;
        const float t = Ai[q] * P[q];
        e = e - t * t;
        S = S + Ai[q] * (Aj[q] + Ak[q]) * (P[q] * P[q]);
      }
      if (j > 0) {
        const long long q = idx - Y;
        const float t = Aj[q] * P[q];
        e = e - t * t;
        S = S + Aj[q] * (Ai[q] + Ak[q]) * (P[q] * P[q]);
      }
      if (k > 0) {
        const long long q = idx - Z;
        const float t = Ak[q] * P[q];
        e = e - t * t;
        S = S + Ak[q] * (Ai[q] + Aj[q]) * (P[q] * P[q]);
      }
      // e -= tau * (...): the sum is widened to double by its "+ 0."
      e = (float)((double)e - (double)0.97f * (double)S);
      if (e < 0.25f * A0[idx]) e = A0[idx];
      pv = 1.f / sqrtf(e);
    }
    P[idx] = pv;
  } else if (MODE == 1) {
    float zv = 0.f;
    if (fl) {
      float t = r[idx];
      if (i > 0) t = t - z[idx - 1] * Ai[idx - 1] * P[idx - 1];
      if (j > 0) t = t - z[idx - Y] * Aj[idx - Y] * P[idx - Y];
      if (k > 0) t = t - z[idx - Z] * Ak[idx - Z] * P[idx - Z];
      zv = P[idx] * t;
    }
    z[idx] = zv;
  } else {
    if (fl) {
      const float p = P[idx];
      float t = z[idx];
      if (i < d.nx - 1) t = t - z[idx + 1] * Ai[idx] * p;
      if (j < d.ny - 1) t = t - z[idx + Y] * Aj[idx] * p;
      if (k < d.nz - 1) t = t - z[idx + Z] * Ak[idx] * p;
      z[idx] = p * t;
    }
  }
}

// dot(z, r) per block after the backward sweep
__global__ void __launch_bounds__(256) k_dot_partials(long long n, const float* __restrict__ a,
                                                      const float* __restrict__ b, double* part, const CgScalars* sc,
                                                      int init) {
  if (!init && sc->done) return;
  FSum acc;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x)
    acc.add(a[idx] * b[idx]);
  const double s2 = block_sum(acc.value());
  if (threadIdx.x == 0) part[blockIdx.x] = s2;
}

void launch_make_frac_matrix(const PcgBuffers& b, const float* frac, cudaStream_t s) {
  count_launch();
  k_make_frac_matrix<<<grid3(b.d, kBlk), kBlk, 0, s>>>(b.d, b.flags, frac, b.A0f, b.Aif, b.Ajf, b.Akf);
}

void launch_mic_planes(const PcgBuffers& b, int mode, cudaStream_t s) {
  const int last = b.d.nx + b.d.ny + b.d.nz - 3;
  const dim3 g((unsigned)((b.d.ny + 127) / 128), (unsigned)b.d.nz);
  for (int q = 0; q <= last; q++) {
    count_launch();
    if (mode == 0)
      k_mic_plane<0><<<g, 128, 0, s>>>(b.d, q, b.code, b.A0f, b.Aif, b.Ajf, b.Akf, b.P, b.residual, b.tmp, b.sc);
    else if (mode == 1)
      k_mic_plane<1><<<g, 128, 0, s>>>(b.d, q, b.code, b.A0f, b.Aif, b.Ajf, b.Akf, b.P, b.residual, b.tmp, b.sc);
    else
      k_mic_plane<2><<<g, 128, 0, s>>>(b.d, last - q, b.code, b.A0f, b.Aif, b.Ajf, b.Akf, b.P, b.residual, b.tmp,
                                       b.sc);
  }
  if (mode >= 2) {
    count_launch();
    k_dot_partials<<<b.nblocks, kThreads, 0, s>>>(b.d.n, b.tmp, b.residual, b.part, b.sc, mode == 3);
    launch_mic_finish(b, b.nblocks, mode == 3, s);
  }
}

// ------------------------------------------------------------- launchers
void launch_make_rhs(const PcgBuffers& b, const float* vu, const float* vv, const float* vw, const float* perCellCorr,
                     const float* phi, const float* curv, float surfTens, float gfClamp, bool sums, cudaStream_t s,
                     const float* frac, const float* obvel) {
  const dim3 g = grid3(b.d, kBlk);
  count_launch();
  k_make_rhs<<<g, kBlk, 0, s>>>(b.d, b.flags, b.rhs, vu, vv, vw, perCellCorr, phi, curv, surfTens, gfClamp, b.part, b.sc,
                                sums ? g.x * g.y * g.z : 0u, frac, obvel);
}
void launch_compat_shift(const PcgBuffers& b, cudaStream_t s) {
  const dim3 g = grid3(b.d, kBlk);
  count_launch();
  k_compat_reduce<<<1, 256, 0, s>>>(b.part, (int)(g.x * g.y * g.z), b.sc);
  count_launch();
  k_compat_shift<<<(unsigned)((b.d.n + 255) / 256), 256, 0, s>>>(b.d.n, b.rhs, b.sc);
}
void launch_make_codes(const PcgBuffers& b, cudaStream_t s) {
  count_launch();
  k_make_codes_full<<<grid3(b.d, kBlk), kBlk, 0, s>>>(b.d, b.flags, b.code);
}
void launch_ghost_fluid_diag(const PcgBuffers& b, const float* phi, float gfClamp, cudaStream_t s) {
  count_launch();
  // with fractions the diagonal already holds their sum: adjust it in place
  k_ghost_fluid_diag<<<grid3(b.d, kBlk), kBlk, 0, s>>>(b.d, b.flags, b.code, phi, gfClamp, b.A0f, b.Aif ? 1 : 0);
}
void launch_count_empty(const PcgBuffers& b, int* out, cudaStream_t s) {
  cudaMemsetAsync(out, 0, sizeof(int), s);
  count_launch();
  k_count_empty<<<304, 256, 0, s>>>(b.d.n, b.flags, out);
}
void launch_fix_pressure(const PcgBuffers& b, long long fix, cudaStream_t s) {
  count_launch();
  k_fix_pressure<<<1, 32, 0, s>>>(b.d, fix, b.code, b.A0f, b.Aif, b.Ajf, b.Akf, b.rhs);
}
void launch_pcg_init(const PcgBuffers& b, cudaStream_t s) {
  count_launch();
  k_pcg_init<<<b.nblocks, kThreads, 0, s>>>(b.d.n, b.pressure, b.rhs, b.residual, b.tmp);
}
void launch_pcg_set_search(const PcgBuffers& b, cudaStream_t s) {
  count_launch();
  k_pcg_set_search<<<b.nblocks, kThreads, 0, s>>>(b.d.n, b.tmp, b.residual, b.search, b.part, b.sc);
}
// four-cell kernels need rows of a multiple of 4 cells
static bool vec4_ok(const Dims& d) { return (d.nx & 3) == 0; }
static int vec4_blocks(const PcgBuffers& b) {
  const long long need = (b.d.n / 4 + kThreads - 1) / kThreads;
  return (int)std::max(1LL, std::min((long long)b.nblocks, need));
}
void launch_pcg_spmv(const PcgBuffers& b, cudaStream_t s) {
  count_launch();
  if (b.Aif) {
    k_pcg_spmv_stored<<<b.nblocks, kThreads, 0, s>>>(b.d, b.code, b.A0f, b.Aif, b.Ajf, b.Akf, b.search, b.tmp, b.part,
                                                    b.sc);
    return;
  }
  StreamGeom g;
  ZmGeom zg;
  dim3 grid;
  const int mode = spmv_mode();
  if (mode == kSpmvZm && zm_geom(b.d, 2 * b.nblocks, g_zmSlots, &zg, &grid)) {
    k_pcg_spmv_zm<<<grid, 256, 0, s>>>(b.d, zg, b.code, b.A0f, b.search, b.tmp, b.part, b.sc);
    return;
  }
  if (mode != kSpmvQuad && stream_geom(b.d, 2 * b.nblocks, g_sms, &g, &grid)) {
    k_pcg_spmv_stream<<<grid, kStreamConsumers + 32, (size_t)kStreamSlots * g.slotBytes, s>>>(
        b.d, g, b.code, b.A0f, b.search, b.tmp, b.part, b.sc);
    return;
  }
  if (vec4_ok(b.d))
    k_pcg_spmv4<<<vec4_blocks(b), kThreads, 0, s>>>(b.d, b.code, b.A0f, b.search, b.tmp, b.part, b.sc);
  else
    k_pcg_spmv<<<b.nblocks, kThreads, 0, s>>>(b.d, b.code, b.A0f, b.search, b.tmp, b.part, b.sc);
}
void launch_pcg_axpy(const PcgBuffers& b, cudaStream_t s) {
  count_launch();
  if (vec4_ok(b.d))
    k_pcg_axpy4<<<vec4_blocks(b), kThreads, 0, s>>>(b.d.n, b.pressure, b.search, b.residual, b.tmp, b.part, b.partf,
                                                    b.sc);
  else
    k_pcg_axpy<<<b.nblocks, kThreads, 0, s>>>(b.d.n, b.pressure, b.search, b.residual, b.tmp, b.part, b.partf, b.sc);
}
void launch_pcg_copy_dot(const PcgBuffers& b, cudaStream_t s) {
  count_launch();
  k_pcg_copy_dot<<<b.nblocks, kThreads, 0, s>>>(b.d.n, b.residual, b.tmp, b.part, b.sc);
}
void launch_pcg_update(const PcgBuffers& b, cudaStream_t s) {
  count_launch();
  if (vec4_ok(b.d))
    k_pcg_update4<<<vec4_blocks(b), kThreads, 0, s>>>(b.d.n, b.tmp, b.search, b.sc);
  else
    k_pcg_update<<<b.nblocks, kThreads, 0, s>>>(b.d.n, b.tmp, b.search, b.sc);
}

// mode: 0 init P, 1 forward, 2 backward (+dot, beta), 3 backward for doInit (+sigma)
void launch_mic(const PcgBuffers& b, const MicPlan& m, int mode, unsigned int epoch, long long spinLimit, cudaStream_t s) {
  MicArgs a;
  a.d = b.d;
  a.code = b.code;
  a.A0f = b.A0f;
  a.P = b.P;
  a.r = b.residual;
  a.z = b.tmp;
  a.part = b.part;
  a.sc = b.sc;
  a.tx = m.tx; a.ty = m.ty; a.tz = m.tz; a.ntiles = m.ntiles;
  a.order = m.order;
  a.tileDone = m.tileDone;
  a.counter = m.counter;
  a.error = m.error;
  a.epoch = epoch;
  a.spinLimit = spinLimit;
  cudaMemsetAsync(m.counter, 0, sizeof(int), s);
  const int ctas = m.ctas < m.ntiles ? m.ctas : m.ntiles;
  if (mode == 0) { count_launch(); k_mic<0><<<ctas, kThreads, 0, s>>>(a); }
  else if (mode == 1) { count_launch(); k_mic<1><<<ctas, kThreads, 0, s>>>(a); }
  else {
    count_launch();
    k_mic<2><<<ctas, kThreads, 0, s>>>(a);
    launch_mic_finish(b, m.ntiles, mode == 3, s);
  }
}

void launch_mic_finish(const PcgBuffers& b, int nparts, bool init, cudaStream_t s) {
  count_launch();
  if (init) k_mic_init_sigma<<<1, 256, 0, s>>>(b.part, nparts, b.sc);
  else k_mic_finish_dot<<<1, 256, 0, s>>>(b.part, nparts, b.sc);
}

// forward dispatch order: tiles sorted by wavefront level a+b+c
void mic_plan_order(int tx, int ty, int tz, int* order) {
  int n = 0;
  for (int L = 0; L <= tx + ty + tz - 3; L++)
    for (int c = 0; c < tz; c++)
      for (int b = 0; b < ty; b++) {
        const int a = L - b - c;
        if (a >= 0 && a < tx) order[n++] = a + tx * (b + ty * c);
      }
}

int mic_ctas_per_sm() {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_mic<1>, kThreads, 0);
  return nb > 0 ? nb : 1;
}

void launch_correct_velocity(const Dims& d, const int* flags, Mac vel, const float* p, const float* phi, const float* curv,
                             float gfClamp, float surfTens, cudaStream_t s) {
  count_launch();
  k_correct_velocity<<<grid3(d, kBlk), kBlk, 0, s>>>(d, flags, vel, p);
  if (phi) {
    count_launch();
    k_correct_velocity_gf<<<grid3(d, kBlk), kBlk, 0, s>>>(d, flags, vel, p, phi, gfClamp, curv, surfTens);
    count_launch();
    k_replace_clamped_gf<<<grid3(d, kBlk), kBlk, 0, s>>>(d, flags, vel, phi, gfClamp);
  }
}

// ----------------------------------------------------------------- batched
// The plume's solvePressure for every scene of a batch: MakeRhs,
// MakeLaplaceMatrix (as codes), GridCg with PcNone -- the reference's 2D
// path, run for every scene here -- and knCorrectVelocity.  Per-scene CG
// scalars; per-tile partials reduced by the scene's last tile in tile order.
#define BATCH_TILE                                                       \
  const BTile tl = tiles[blockIdx.x];                                    \
  const BScene& sc = S[tl.scene];                                        \
  const Dims d = sc.d;                                                   \
  const int i = tl.x0 + threadIdx.x, j = tl.y0 + threadIdx.y, k = tl.z; \
  const bool in = i < d.nx && j < d.ny;                                  \
  const long long idx = in ? ix(d, i, j, k) : 0;

// MakeRhs and MakeLaplaceMatrix pass 1
__global__ void __launch_bounds__(256) k_b_rhs_codes(const BTile* __restrict__ tiles, const BScene* __restrict__ S, int nxt) {
  BATCH_TILE
  if (!in) return;
  float r = 0.f;
  if (INNER && isF(sc.flags, idx)) {
    const float* v = sc.vel[nxt];
    r = mac_neg_div(d, v, v + d.n, v + 2 * d.n, idx);
  }
  sc.rhs[idx] = r;
  make_codes_cell(d, sc.flags, sc.code, i, j, k);
}

// MakeLaplaceMatrix pass 2 and GridCg::doInit with PcNone: x = 0, r = rhs,
// z = r, s = z, sigma = dot(z, r)
__global__ void __launch_bounds__(256) k_b_pcg_init(const BTile* __restrict__ tiles, const BScene* __restrict__ S) {
  BATCH_TILE
  FSum acc;
  if (in) {
    make_codes_low_cell(d, sc.code, i, j, k);
    const float r = sc.rhs[idx];
    sc.pres[idx] = 0.f;
    sc.res[idx] = r;
    sc.tmp[idx] = r;
    sc.search[idx] = r;
    acc.add(r * r);
  }
  const double b = block_sum(acc.value());
  if (lin_tid() == 0) sc.part[tl.local] = b;
  if (last_block(&sc.sc->counters[0], tl.count)) {
    const double s2 = sum_partials(sc.part, sc.ntiles);
    if (lin_tid() == 0) sc.sc->sigma = (float)s2;
  }
}

// The CG sweep kernels take tiles R row-groups tall (32 x 8R cells per CTA,
// R chosen by the batch's autotuner).  Reductions stay on the 32 x 8
// sub-tile grid of R = 1: sub-tile r of a tile writes the slot the R = 1
// tile at that place would, summed over the same thread order, so results
// do not depend on R.
#define BATCH_ROWS                                                        \
  const BTile tl = tiles[blockIdx.x];                                     \
  const BScene& sc = S[tl.scene];                                         \
  const Dims d = sc.d;                                                    \
  const int txc = (d.nx + kBTX - 1) / kBTX, tyc = (d.ny + kBTY - 1) / kBTY; \
  const int i = tl.x0 + threadIdx.x, k = tl.z;                            \
  const int yt0 = tl.y0 / kBTY;

__device__ __forceinline__ int sub_slot(int txc, int tyc, int x0, int yt, int z) { return x0 / kBTX + txc * (yt + tyc * z); }

// per 32 x 8 sub-tile sums of one float per thread: warp sums in
// double-float, the 8 warp sums added in warp order by thread r, written
// to slot[r] as a double.  Sub-tiles past the grid (valid[r] false) write
// nothing.
template <int R>
__device__ __forceinline__ void subtile_sums(const float* v, double* part, const int* slot, const bool* valid) {
  __shared__ ff wsum[R][8];
  const int lane = lin_tid() & 31, wid = lin_tid() >> 5;
#pragma unroll
  for (int r = 0; r < R; r++) {
    const ff a = warp_sum_ff(ff{v[r], 0.f});
    if (lane == 0) wsum[r][wid] = a;
  }
  __syncthreads();
  if (lin_tid() < R) {
    const int r = lin_tid();
    if (valid[r]) {
      ff t{0.f, 0.f};
      for (int w = 0; w < 8; w++) t = ff_add(t, wsum[r][w]);
      part[slot[r]] = ff_d(t);
    }
  }
}

// tmp = A s (ApplyMatrix) and dot(tmp, s) -> alpha
template <int R>
__global__ void __launch_bounds__(256) k_b_pcg_spmv(const BTile* __restrict__ tiles, const BScene* __restrict__ S) {
  BATCH_ROWS
  CgScalars* g = sc.sc;
  if (g->done) return;
  float pv[R];
  int slot[R];
  bool valid[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    valid[r] = yt0 + r < tyc;
    slot[r] = sub_slot(txc, tyc, tl.x0, yt0 + r, k);
    const int j = tl.y0 + kBTY * r + threadIdx.y;
    pv[r] = 0.f;
    if (valid[r] && i < d.nx && j < d.ny) {
      const long long idx = ix(d, i, j, k);
      const int c = sc.code[idx];
      const float* x = sc.search;
      const float xc = x[idx];
      float v;
      if (!(c & kCodeFluid)) {
        v = xc;
      } else {
        v = xc * (sc.A0f ? sc.A0f[idx] : (float)(c & 7));
        if (c & kLowX) v = v - x[idx - 1];
        if (c & kHighX) v = v - x[idx + 1];
        if (c & kLowY) v = v - x[idx - d.sy];
        if (c & kHighY) v = v - x[idx + d.sy];
        if (c & kLowZ) v = v - x[idx - d.sz];
        if (c & kHighZ) v = v - x[idx + d.sz];
      }
      sc.tmp[idx] = v;
      pv[r] = v * xc;
    }
  }
  subtile_sums<R>(pv, sc.part, slot, valid);
  if (last_block(&g->counters[1], tl.count)) {
    const double s2 = sum_partials(sc.part, sc.ntiles);
    if (lin_tid() == 0) {
      const float dp = (float)s2;
      g->dp = dp;
      g->alpha = fabsf(dp) > 0.f ? g->sigma / dp : 0.f;
    }
  }
}

// x += alpha s, r -= alpha tmp, z = r (PcNone), resNorm = max|r| and the
// convergence test; then sigmaNew = dot(z, r) and beta (GridCg::iterate)
template <int R>
__global__ void __launch_bounds__(256) k_b_pcg_axpy(const BTile* __restrict__ tiles, const BScene* __restrict__ S,
                                                    int* ndone) {
  BATCH_ROWS
  CgScalars* g = sc.sc;
  if (g->done) return;
  const float alpha = g->alpha, na = -alpha;
  float sq[R], mx[R];
  int slot[R];
  bool valid[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    valid[r] = yt0 + r < tyc;
    slot[r] = sub_slot(txc, tyc, tl.x0, yt0 + r, k);
    const int j = tl.y0 + kBTY * r + threadIdx.y;
    sq[r] = 0.f;
    mx[r] = 0.f;
    if (valid[r] && i < d.nx && j < d.ny) {
      const long long idx = ix(d, i, j, k);
      sc.pres[idx] = sc.pres[idx] + alpha * sc.search[idx];
      const float rv = sc.res[idx] + na * sc.tmp[idx];
      sc.res[idx] = rv;
      if (!sc.mic) sc.tmp[idx] = rv;  // z = r without a preconditioner
      mx[r] = fabsf(rv);
      sq[r] = rv * rv;
    }
  }
  // max |r| per sub-tile, then the dot sums
  __shared__ float smx[R][8];
  const int lane = lin_tid() & 31, wid = lin_tid() >> 5;
#pragma unroll
  for (int r = 0; r < R; r++) {
    float m = mx[r];
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) smx[r][wid] = m;
  }
  subtile_sums<R>(sq, sc.part, slot, valid);  // its barrier also publishes smx
  if (lin_tid() < R && valid[lin_tid()]) {
    const int r = lin_tid();
    float m = 0.f;
    for (int w = 0; w < 8; w++) m = fmaxf(m, smx[r][w]);
    sc.part[sc.ntiles + slot[r]] = (double)m;
  }
  if (last_block(&g->counters[2], tl.count)) {
    const double s2 = sum_partials(sc.part, sc.ntiles);
    const double mxp = max_partials(sc.part + sc.ntiles, sc.ntiles);
    if (lin_tid() != 0) return;
    const float res = (float)mxp;
    g->iterations += 1;
    g->resNorm = res;
    if (res < g->accuracy) {
      g->sigma = res;
      g->done = 1;
      atomicAdd(ndone, 1);
      return;
    }
    if (sc.mic) {
      // beta and the divergence test follow the MIC sweeps (k_b_mic_finish)
      if (g->iterations >= g->maxIter) {
        g->done = 1;
        atomicAdd(ndone, 1);
      }
      return;
    }
    const float sigmaNew = (float)s2;
    g->beta = sigmaNew / g->sigma;
    g->sigma = sigmaNew;
    if (!(res < 1e35f)) {
      g->status = 2;
      g->done = 1;
      atomicAdd(ndone, 1);
    } else if (g->iterations >= g->maxIter) {
      g->done = 1;
      atomicAdd(ndone, 1);
    }
  }
}

// s = z + beta s (UpdateSearchVec)
template <int R>
__global__ void __launch_bounds__(256) k_b_pcg_update(const BTile* __restrict__ tiles, const BScene* __restrict__ S) {
  BATCH_ROWS
  (void)txc;
  if (sc.sc->done) return;
  const float beta = sc.sc->beta;
#pragma unroll
  for (int r = 0; r < R; r++) {
    if (yt0 + r >= tyc) break;
    const int j = tl.y0 + kBTY * r + threadIdx.y;
    if (i < d.nx && j < d.ny) {
      const long long idx = ix(d, i, j, k);
      sc.search[idx] = sc.tmp[idx] + beta * sc.search[idx];
    }
  }
}
#undef BATCH_ROWS

__global__ void __launch_bounds__(256) k_b_correct(const BTile* __restrict__ tiles, const BScene* __restrict__ S, int nxt) {
  BATCH_TILE
  if (!in) return;
  correct_velocity_cell(d, sc.flags, bmac(sc.vel[nxt], d.n), sc.pres, i, j, k);
}
// search = z for the MIC scenes after doInit's preconditioner application
__global__ void __launch_bounds__(256) k_b_mic_search(const BTile* __restrict__ tiles, const BScene* __restrict__ S) {
  BATCH_TILE
  if (!in || !sc.mic) return;
  sc.search[idx] = sc.tmp[idx];
}

// dam break: ApplyGhostFluidDiagonal from the advected phi (pass-1 codes)
__global__ void __launch_bounds__(256) k_b_dam_gf_diag(const BTile* __restrict__ tiles, const BScene* __restrict__ S,
                                                       int nxt) {
  BATCH_TILE
  if (!in) return;
  (void)idx;
  ghost_fluid_diag_cell(d, sc.flags, sc.code, sc.dens[nxt], 1e-4f, sc.A0f, i, j, k);
}
// dam break: knCorrectVelocityGhostFluid, then knReplaceClampedGhostFluidVels
// (pressure.cpp:154-214), each a pass of its own (the second reads
// neighbours' corrected velocities)
__global__ void __launch_bounds__(256) k_b_dam_correct_gf(const BTile* __restrict__ tiles, const BScene* __restrict__ S,
                                                          int nxt) {
  BATCH_TILE
  if (!in) return;
  (void)idx;
  correct_velocity_gf_cell(d, sc.flags, bmac(sc.vel[nxt], d.n), sc.pres, sc.dens[nxt], 1e-4f, nullptr, 0.f, i, j, k);
}
__global__ void __launch_bounds__(256) k_b_dam_replace_clamped(const BTile* __restrict__ tiles,
                                                               const BScene* __restrict__ S, int nxt) {
  BATCH_TILE
  if (!in) return;
  (void)idx;
  replace_clamped_gf_cell(d, sc.flags, bmac(sc.vel[nxt], d.n), sc.dens[nxt], 1e-4f, i, j, k);
}

// ---- batched FP64 refinement (the precision form of refine.cu per scene)
__global__ void __launch_bounds__(256) k_b_ref_first(const BTile* __restrict__ tiles, const BScene* __restrict__ S) {
  BATCH_TILE
  if (!in) return;
  sc.b64[idx] = (double)sc.rhs[idx];
  sc.p64[idx] = (double)sc.pres[idx];
}
// r = b - A p64 in double (identity rows off the fluid), rhs = (float) r,
// max|r| per 32 x 8 tile, reduced by the scene's last tile into refNorm
__global__ void __launch_bounds__(256) k_b_ref_residual(const BTile* __restrict__ tiles, const BScene* __restrict__ S) {
  BATCH_TILE
  double m = 0.;
  if (in) {
    const int c = sc.code[idx];
    const double* p = sc.p64;
    const double pc = p[idx];
    double ap = pc;
    if (c & kCodeFluid) {
      ap = (double)(sc.A0f ? sc.A0f[idx] : (float)(c & 7)) * pc;
      if (c & kLowX) ap -= p[idx - 1];
      if (c & kHighX) ap -= p[idx + 1];
      if (c & kLowY) ap -= p[idx - d.sy];
      if (c & kHighY) ap -= p[idx + d.sy];
      if (c & kLowZ) ap -= p[idx - d.sz];
      if (c & kHighZ) ap -= p[idx + d.sz];
    }
    const double r = sc.b64[idx] - ap;
    sc.rhs[idx] = (float)r;
    m = fabs(r);
  }
  __shared__ double sh[8];
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((lin_tid() & 31) == 0) sh[lin_tid() >> 5] = m;
  __syncthreads();
  if (lin_tid() == 0) {
    double t = 0.;
    for (int w = 0; w < 8; w++) t = fmax(t, sh[w]);
    sc.part[tl.local] = t;
  }
  if (last_block(&sc.sc->counters[4], tl.count)) {
    const double mx = max_partials(sc.part, sc.ntiles);
    if (lin_tid() == 0) sc.sc->refNorm = mx;
  }
}
__global__ void __launch_bounds__(256) k_b_ref_add(const BTile* __restrict__ tiles, const BScene* __restrict__ S) {
  BATCH_TILE
  if (!in) return;
  sc.p64[idx] += (double)sc.pres[idx];
}
__global__ void __launch_bounds__(256) k_b_ref_finish(const BTile* __restrict__ tiles, const BScene* __restrict__ S) {
  BATCH_TILE
  if (!in) return;
  sc.pres[idx] = (float)sc.p64[idx];
}

#undef BATCH_TILE

// sigma (doInit) or beta (iterate) of each MIC scene from the per-tile
// dot(z, r) partials its backward sweep left, summed in tile order; the
// divergence test of GridCg::iterate (conjugategrad.cpp:288-295)
template <bool kInit>
__global__ void k_b_mic_finish(const BScene* __restrict__ S, const int* __restrict__ sceneOf, const FlowScene* F,
                               int* ndone) {
  const BScene& sc = S[sceneOf[blockIdx.x]];
  CgScalars* g = sc.sc;
  if (!kInit && g->done) return;
  const double s2 = sum_partials(sc.part, F[blockIdx.x].tx * F[blockIdx.x].ty * F[blockIdx.x].tz);
  if (threadIdx.x != 0) return;
  const float sigmaNew = (float)s2;
  if (kInit) {
    g->sigma = sigmaNew;
    return;
  }
  g->beta = sigmaNew / g->sigma;
  g->sigma = sigmaNew;
  if (!(g->resNorm < 1e35f)) {
    g->status = 2;
    g->done = 1;
    atomicAdd(ndone, 1);
  }
}

void launch_b_mic_init(const BTile* t, int nt, const BScene* s, const BatchMic& m, cudaStream_t st) {
  if (m.nscenes == 0) return;
  for (int mode = 0; mode <= 2; mode++)
    launch_mic_flow_batch(m.flow, m.order, m.ntiles, m.ctas, m.counter, m.error, mode == 2 ? 3 : mode, m.epochDev,
                          m.spinLimit, st);
  count_launch();
  k_b_mic_finish<true><<<m.nscenes, 256, 0, st>>>(s, m.sceneOf, m.flow, nullptr);
  count_launch();
  k_b_mic_search<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s);
}

void launch_b_dam_gf_diag(const BTile* t, int nt, const BScene* s, int nxt, cudaStream_t st);
void launch_b_pressure_setup(const BTile* t, int nt, const BScene* s, int nxt, cudaStream_t st, const BTile* tDam,
                             int ntDam) {
  const dim3 b(kBTX, kBTY, 1);
  count_launch();
  k_b_rhs_codes<<<nt, b, 0, st>>>(t, s, nxt);
  launch_b_dam_gf_diag(tDam, ntDam, s, nxt, st);
}
void launch_b_ref_first(const BTile* t, int nt, const BScene* s, cudaStream_t st) {
  count_launch();
  k_b_ref_first<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s);
}
void launch_b_ref_residual(const BTile* t, int nt, const BScene* s, cudaStream_t st) {
  count_launch();
  k_b_ref_residual<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s);
}
void launch_b_ref_add(const BTile* t, int nt, const BScene* s, cudaStream_t st) {
  count_launch();
  k_b_ref_add<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s);
}
void launch_b_ref_finish(const BTile* t, int nt, const BScene* s, cudaStream_t st) {
  count_launch();
  k_b_ref_finish<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s);
}
void launch_b_pcg_init(const BTile* t, int nt, const BScene* s, cudaStream_t st) {
  count_launch();
  k_b_pcg_init<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s);
}
template <int R>
static void pcg_iteration(const BTile* t, int nt, const BScene* s, int* ndone, const BatchMic* mic, cudaStream_t st) {
  const dim3 b(kBTX, kBTY, 1);
  count_launch();
  k_b_pcg_spmv<R><<<nt, b, 0, st>>>(t, s);
  count_launch();
  k_b_pcg_axpy<R><<<nt, b, 0, st>>>(t, s, ndone);
  if (mic && mic->nscenes > 0) {
    launch_mic_flow_batch(mic->flow, mic->order, mic->ntiles, mic->ctas, mic->counter, mic->error, 1, mic->epochDev,
                          mic->spinLimit, st);
    launch_mic_flow_batch(mic->flow, mic->order, mic->ntiles, mic->ctas, mic->counter, mic->error, 2, mic->epochDev,
                          mic->spinLimit, st);
    count_launch();
    k_b_mic_finish<false><<<mic->nscenes, 256, 0, st>>>(s, mic->sceneOf, mic->flow, ndone);
  }
  count_launch();
  k_b_pcg_update<R><<<nt, b, 0, st>>>(t, s);
}
void launch_b_pcg_iteration(const BTile* t, int nt, const BScene* s, int rows, int* ndone, const BatchMic* mic,
                            cudaStream_t st) {
  switch (rows) {
    case 1: pcg_iteration<1>(t, nt, s, ndone, mic, st); break;
    case 2: pcg_iteration<2>(t, nt, s, ndone, mic, st); break;
    case 4: pcg_iteration<4>(t, nt, s, ndone, mic, st); break;
    default: pcg_iteration<8>(t, nt, s, ndone, mic, st); break;
  }
}
void launch_b_correct(const BTile* t, int nt, const BScene* s, int nxt, cudaStream_t st) {
  count_launch();
  k_b_correct<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s, nxt);
}
void launch_b_dam_gf_diag(const BTile* t, int nt, const BScene* s, int nxt, cudaStream_t st) {
  if (nt == 0) return;
  count_launch();
  k_b_dam_gf_diag<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s, nxt);
}
void launch_b_dam_walls(const BTile* t, int nt, const BScene* s, int nxt, cudaStream_t st);
void launch_b_dam_correct(const BTile* t, int nt, const BScene* s, int nxt, cudaStream_t st) {
  if (nt == 0) return;
  count_launch();
  k_b_dam_correct_gf<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s, nxt);
  count_launch();
  k_b_dam_replace_clamped<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s, nxt);
  launch_b_dam_walls(t, nt, s, nxt, st);
}

}  // namespace mgpu
