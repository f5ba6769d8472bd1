// Precision form of the pressure solve: FP64 residual refinement around the
// FP32 PCG (mixed-precision iterative refinement).
//
// The Poisson system A p = b is the reference's (stencil codes of
// pressure.cu, float ghost-fluid diagonal when present).  The pressure is
// accumulated in double, p64 += delta, and after every FP32 inner solve the
// residual r = b - A p64 is formed in double on the GPU; its max-abs norm is
// the refinement's stopping test.  These kernels and the PCG's dot-product
// reductions are the only FP64 steps: stencils, advection and the inner PCG
// stay FP32.  Non-fluid rows are identity rows (ApplyMatrix,
// conjugategrad.h:118-151).
#include "mg_common.cuh"
#include "mg_kernels.h"
#include "mg_reduce.cuh"

namespace mgpu {

namespace {

#define GRID_STRIDE(v, n) \
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < (n); v += (long long)gridDim.x * blockDim.x)

__global__ void k_to_double(long long n, const float* __restrict__ a, double* b) {
  GRID_STRIDE(i, n) b[i] = (double)a[i];
}
__global__ void k_to_float(long long n, const double* __restrict__ a, float* b) {
  GRID_STRIDE(i, n) b[i] = (float)a[i];
}
__global__ void k_add_delta(long long n, double* p, const float* __restrict__ d) {
  GRID_STRIDE(i, n) p[i] += (double)d[i];
}

// r = b - A p in double, rf = (float) r, and max|r| into *norm (last block)
__global__ void __launch_bounds__(256) k_residual64(Dims d, const code_t* __restrict__ code,
                                                   const float* __restrict__ A0f, const double* __restrict__ b,
                                                   const double* __restrict__ p, float* rf, double* part,
                                                   unsigned int* counter, double* norm) {
  double mx = 0.;
  GRID_STRIDE(i, d.n) {
    const int c = code[i];
    const double pc = p[i];
    double ap;
    if (!(c & kCodeFluid)) {
      ap = pc;
    } else {
      ap = (double)(A0f ? A0f[i] : (float)(c & 7)) * pc;
      if (c & kLowX) ap -= p[i - 1];
      if (c & kHighX) ap -= p[i + 1];
      if (c & kLowY) ap -= p[i - d.sy];
      if (c & kHighY) ap -= p[i + d.sy];
      if (c & kLowZ) ap -= p[i - d.sz];
      if (c & kHighZ) ap -= p[i + d.sz];
    }
    const double r = b[i] - ap;
    rf[i] = (float)r;
    mx = fmax(mx, fabs(r));
  }
  // block max in a fixed order, then the last block over the partials
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) m = fmax(m, sh[q]);
    part[blockIdx.x] = m;
  }
  if (last_block(counter, gridDim.x)) {
    const double m = max_partials(part, gridDim.x);
    if (threadIdx.x == 0) *norm = m;
  }
}

int blocks(long long n) {
  const long long b = (n + 255) / 256;
  return (int)(b < 4096 ? (b < 1 ? 1 : b) : 4096);
}

}  // namespace

void launch_to_double(long long n, const float* a, double* b, cudaStream_t s) {
  count_launch();
  k_to_double<<<blocks(n), 256, 0, s>>>(n, a, b);
}
void launch_to_float(long long n, const double* a, float* b, cudaStream_t s) {
  count_launch();
  k_to_float<<<blocks(n), 256, 0, s>>>(n, a, b);
}
void launch_add_delta(long long n, double* p, const float* d, cudaStream_t s) {
  count_launch();
  k_add_delta<<<blocks(n), 256, 0, s>>>(n, p, d);
}
void launch_residual64(const Dims& d, const code_t* code, const float* A0f, const double* b, const double* p, float* rf,
                       double* part, unsigned int* counter, double* norm, cudaStream_t s) {
  count_launch();
  k_residual64<<<blocks(d.n), 256, 0, s>>>(d, code, A0f, b, p, rf, part, counter, norm);
}

}  // namespace mgpu
