// Deterministic block and grid reductions shared by the PCG and multigrid
// kernels: warp shuffles, per-warp partials summed in warp order, and a
// "last block" ticket so the block that finishes last reduces the per-block
// partials in index order.  Results do not depend on block scheduling.
#pragma once
#include <cfloat>
#include <cuda_runtime.h>

namespace mgpu {

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ int lin_tid() { return threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z); }
__device__ __forceinline__ int nwarps() { return (blockDim.x * blockDim.y * blockDim.z) >> 5; }

// block sum in a fixed order; result valid in thread 0
template <typename T>
__device__ __forceinline__ T block_sum(T v) {
  __shared__ T sh[32];
  const int t = lin_tid();
  const int lane = t & 31, wid = t >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  T r = 0;
  if (t == 0)
    for (int q = 0; q < nwarps(); q++) r += sh[q];
  return r;
}

__device__ __forceinline__ void block_minmax(float& mn, float& mx) {
  __shared__ float s0[32], s1[32];
  const int t = lin_tid();
  const int lane = t & 31, wid = t >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  __syncthreads();
  if (lane == 0) { s0[wid] = mn; s1[wid] = mx; }
  __syncthreads();
  if (t == 0)
    for (int q = 1; q < nwarps(); q++) { mn = fminf(mn, s0[q]); mx = fmaxf(mx, s1[q]); }
}

// all threads of a block: sum of part[0..n) in a fixed order (strided
// per-thread sums, then a fixed tree); the result is valid in thread 0.
// The partials come from other blocks, so they are read from L2.
__device__ __forceinline__ double sum_partials(const double* part, int n) {
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  double v = 0.;
  for (int q = lin_tid(); q < n; q += nt) v += __ldcg(part + q);
  return block_sum(v);
}
__device__ __forceinline__ void minmax_partials(const float* part, int n, float& mn, float& mx) {
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  mn = FLT_MAX;
  mx = -FLT_MAX;
  for (int q = lin_tid(); q < n; q += nt) {
    mn = fminf(mn, __ldcg(part + 2 * q));
    mx = fmaxf(mx, __ldcg(part + 2 * q + 1));
  }
  block_minmax(mn, mx);
}

// all threads of a block: max of part[0..n), result valid in thread 0
__device__ __forceinline__ double max_partials(const double* part, int n) {
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  double v = 0.;
  for (int q = lin_tid(); q < n; q += nt) v = fmax(v, __ldcg(part + q));
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((lin_tid() & 31) == 0) sh[lin_tid() >> 5] = v;
  __syncthreads();
  if (lin_tid() == 0)
    for (int q = 0; q < nwarps(); q++) v = fmax(v, sh[q]);
  return v;
}

// "last block" ticket: true in every thread of the block that finishes last
__device__ __forceinline__ bool last_block(unsigned int* counter, unsigned int total) {
  __shared__ bool last;
  __syncthreads();
  if (lin_tid() == 0) {
    __threadfence();
    const unsigned int t = atomicAdd(counter, 1u);
    last = (t == total - 1);
    if (last) *counter = 0;  // reset for the next launch
  }
  __syncthreads();
  return last;
}

// Double-float ("ff") arithmetic: a value is the unevaluated sum h + l of
// two floats (48-bit significand), built from Knuth's exact two-sum and the
// FMA-exact product.  GB300 runs FP64 at a small fraction of its FP32 rate,
// so sums and scalars that need more than float precision use these.
struct ff {
  float h, l;
};
__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return ff{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ ff quick_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return ff{s, b - (s - a)};
}
__device__ __forceinline__ ff two_prod(float a, float b) {
  const float p = a * b;
  return ff{p, fmaf(a, b, -p)};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  ff s = two_sum(a.h, b.h);
  const ff t = two_sum(a.l, b.l);
  s.l = s.l + t.h;
  s = quick_two_sum(s.h, s.l);
  s.l = s.l + t.l;
  return quick_two_sum(s.h, s.l);
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.h, -a.l}; }
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  ff p = two_prod(a.h, b.h);
  p.l = p.l + (a.h * b.l + a.l * b.h);
  return quick_two_sum(p.h, p.l);
}
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
  ff p = two_prod(a.h, b);
  p.l = p.l + a.l * b;
  return quick_two_sum(p.h, p.l);
}
__device__ __forceinline__ ff ff_div_f(ff a, float b) {
  const float q1 = a.h / b;
  const ff p = two_prod(q1, b);
  ff r = two_sum(a.h, -p.h);
  r.l = (r.l - p.l) + a.l;
  const float q2 = (r.h + r.l) / b;
  return quick_two_sum(q1, q2);
}
__device__ __forceinline__ double ff_d(ff a) { return (double)a.h + (double)a.l; }
__device__ __forceinline__ ff d_ff(double d) {
  const float h = (float)d;
  return ff{h, (float)(d - (double)h)};
}
__device__ __forceinline__ ff warp_sum_ff(ff v) {
  for (int o = 16; o > 0; o >>= 1) {
    const ff w{__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
    v = ff_add(v, w);
  }
  return v;
}

// Per-thread sum of float products as an unevaluated pair h + l: each
// addition is Knuth's exact two-sum, its rounding error kept in l.  This
// carries ~48 bits, far beyond the float terms, and costs a few FP32
// instructions instead of a convert and an add on the FP64 pipe, which
// GB300 runs at a small fraction of its FP32 rate.  Threads convert to
// double once, before the block and grid sums.
struct FSum {
  float h = 0.f, l = 0.f;
  __device__ __forceinline__ void add(float p) {
    const float s = h + p;
    const float bb = s - h;
    l += (h - (s - bb)) + (p - bb);
    h = s;
  }
  __device__ __forceinline__ double value() const { return (double)h + (double)l; }
};

}  // namespace mgpu
