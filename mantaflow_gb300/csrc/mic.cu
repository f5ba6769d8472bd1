// MIC(0) preconditioner sweeps as pipelined column blocks.
//
// The reference computes the modified incomplete Cholesky factor and applies
// it with lexicographic loops (conjugategrad.cpp:66-97, 135-160): cell
// (i,j,k) needs the finished values of (i-1,j,k), (i,j-1,k), (i,j,k-1).
// Any order that respects those three dependencies reproduces the serial
// result exactly, so the GPU runs a skewed wavefront:
//
//  * A CTA owns a column block of 32 y-lines x BZW z-lines over the whole
//    x range.  Thread (lane j, warp w) owns one x-line and at step s works on
//    x = s - j - w, so its y- and z-neighbours finished that x one step
//    earlier; their results come through a double-buffered shared-memory
//    exchange, the x-neighbour is the thread's own previous cell.  One
//    barrier per step.
//  * Neighbouring column blocks form a pipeline: a block needs the block
//    below it in y and in z to be a fixed number of steps ahead.  Producers
//    publish their step count (release) every few steps; consumers acquire it
//    with a bounded spin.  Blocks are handed out in (b + c) order, so a block
//    only ever waits for blocks that were handed out earlier and are running:
//    the scheme cannot deadlock whatever the residency.
//  * Each thread streams its own line through a private shared-memory ring of
//    8-cell chunks filled with cp.async three chunks ahead, and writes its
//    outputs back as whole 32-byte chunks.
//
// The backward sweep mirrors x, y and z.  Grids whose x size is not a
// multiple of 8 use the tiled kernel in pressure.cu instead.
#include "mg_common.cuh"
#include "mg_kernels.h"

namespace mgpu {

constexpr int kCW = 8;     // cells per staged chunk
constexpr int kNR = 4;     // chunks per ring (3 in flight)
constexpr int kRing = kCW * kNR;
constexpr int kLag = 39;   // steps a y-neighbour block must be ahead (31 + chunk flush)

struct MicColArgs {
  Dims d;
  const code_t* code;
  const float* A0f;
  float* P;
  const float* r;
  float* z;
  double* part;
  CgScalars* sc;
  int nby, nbz, nblocks;
  const int* order;
  unsigned long long* prog;
  int* counter;
  int* error;
  unsigned int epoch;
  long long spinLimit;
};

__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// thread 0: wait until block `blk` has published at least `need` (bounded)
__device__ __forceinline__ void wait_progress(const MicColArgs& a, int blk, unsigned long long need,
                                              unsigned long long& cache) {
  if (blk < 0 || cache >= need) return;
  long long n = 0;
  for (;;) {
    cache = ld_acquire64(a.prog + blk);
    if (cache >= need) return;
    if (++n > a.spinLimit || *((volatile int*)a.error) != 0) {
      atomicExch(a.error, 2);
      cache = ~0ull;  // stop waiting for this block
      return;
    }
    __nanosleep(20);
  }
}

// MODE 0: factor (P), MODE 1: forward substitution, MODE 2: backward
// substitution with the fused dot(z, residual)
template <int MODE, int BZW>
__global__ void __launch_bounds__(32 * BZW, 1) k_mic_col(MicColArgs a) {
  constexpr int NT = 32 * BZW;
  constexpr int NF = MODE == 2 ? 3 : (MODE == 1 ? 2 : 1);  // staged float arrays per thread
  extern __shared__ __align__(16) unsigned char smem[];
  float* ringF = reinterpret_cast<float*>(smem);                    // [NF][NT][kRing]
  code_t* ringC = reinterpret_cast<code_t*>(ringF + NF * NT * kRing);  // [NT][kRing]
  float2* xb = reinterpret_cast<float2*>(ringC + NT * kRing);        // [2][BZW][32]
  __shared__ int s_blk;
  const Dims& d = a.d;
  const int tid = threadIdx.x, j = tid & 31, w = tid >> 5;
  const int jm = MODE == 2 ? 31 - j : j;        // position in sweep order
  const int wm = MODE == 2 ? BZW - 1 - w : w;
  const int jn = MODE == 2 ? j + 1 : j - 1;     // upwind lane / warp
  const int wn = MODE == 2 ? w + 1 : w - 1;
  if (MODE != 0 && a.sc->done) return;
  const int S = d.nx + 31 + BZW - 1;
  const int nch = d.nx / kCW;
  const unsigned long long E = (unsigned long long)a.epoch << 32;
  float* myF = ringF + tid * kRing;
  code_t* myC = ringC + tid * kRing;

  for (;;) {
    if (tid == 0) {
      const int q = atomicAdd(a.counter, 1);
      s_blk = q < a.nblocks ? (MODE == 2 ? a.order[a.nblocks - 1 - q] : a.order[q]) : -1;
    }
    __syncthreads();
    const int blk = s_blk;
    if (blk < 0) return;
    const int b = blk % a.nby, c = blk / a.nby;
    const int y = 32 * b + j, zc = BZW * c + w;
    const bool line = y < d.ny && zc < d.nz;
    const long long base = line ? ix(d, 0, y, zc) : 0;
    int depY, depZ;
    if (MODE == 2) {
      depY = b + 1 < a.nby ? blk + 1 : -1;
      depZ = c + 1 < a.nbz ? blk + a.nby : -1;
    } else {
      depY = b > 0 ? blk - 1 : -1;
      depZ = c > 0 ? blk - a.nby : -1;
    }
    // global neighbour (outside this block) of threads on the upwind faces
    const bool gy = jm == 0 && (MODE == 2 ? y + 1 < d.ny : y > 0);
    const bool gz = wm == 0 && (MODE == 2 ? zc + 1 < d.nz : zc > 0);
    const long long nbY = MODE == 2 ? base + d.sy : base - d.sy;
    const long long nbZ = MODE == 2 ? base + d.sz : base - d.sz;

    auto chunk_lo = [&](int cm) { return MODE == 2 ? d.nx - kCW * (cm + 1) : kCW * cm; };
    auto prefetch = [&](int cm) {
      if (line && cm < nch) {
        const int slot = (cm % kNR) * kCW;
        const long long g = base + chunk_lo(cm);
        if (MODE == 1) {
          cp_async16(myF + slot, a.r + g);
          cp_async16(myF + slot + 4, a.r + g + 4);
          cp_async16(myF + NT * kRing + slot, a.P + g);
          cp_async16(myF + NT * kRing + slot + 4, a.P + g + 4);
        } else if (MODE == 2) {
          cp_async16(myF + slot, a.z + g);
          cp_async16(myF + slot + 4, a.z + g + 4);
          cp_async16(myF + NT * kRing + slot, a.r + g);
          cp_async16(myF + NT * kRing + slot + 4, a.r + g + 4);
          cp_async16(myF + 2 * NT * kRing + slot, a.P + g);
          cp_async16(myF + 2 * NT * kRing + slot + 4, a.P + g + 4);
        } else if (a.A0f) {
          cp_async16(myF + slot, a.A0f + g);
          cp_async16(myF + slot + 4, a.A0f + g + 4);
        }
        cp_async16(myC + slot, a.code + g);
      }
      cp_async_commit();
    };
    for (int q = 0; q < kNR - 1; q++) prefetch(q);

    float vprev = 0.f, pprev = 0.f;
    int cprev = 0;
    double acc = 0.;
    unsigned long long cacheY = 0, cacheZ = 0;
    for (int s = 0; s < S; s++) {
      if (tid == 0) {
        wait_progress(a, depY, E | (unsigned long long)min(S, s + kLag), cacheY);
        wait_progress(a, depZ, E | (unsigned long long)min(S, s + BZW + kCW - 1), cacheZ);
      }
      __syncthreads();
      if (tid == 0 && (s & 3) == 0 && s > 0) {
        __threadfence();
        st_release64(a.prog + blk, E | (unsigned long long)s);  // steps < s are complete
      }
      const int xm = s - jm - wm;
      float outv = 0.f, outp = 0.f;
      if (line && xm >= 0 && xm < d.nx) {
        const int cm = xm >> 3;
        if ((xm & 7) == 0) {
          prefetch(cm + kNR - 1);
          cp_async_wait<kNR - 1>();
        }
        const int off = MODE == 2 ? 7 - (xm & 7) : (xm & 7);
        const int slot = (cm % kNR) * kCW + off;
        const int x = MODE == 2 ? d.nx - 1 - xm : xm;
        const int cd = myC[slot];
        const float2 ny = jm > 0 ? xb[((s - 1) & 1) * BZW * 32 + w * 32 + jn] : make_float2(0.f, 0.f);
        const float2 nz = wm > 0 ? xb[((s - 1) & 1) * BZW * 32 + wn * 32 + j] : make_float2(0.f, 0.f);
        if (MODE == 0) {
          // InitPreconditionModifiedIncompCholesky2 (conjugategrad.cpp:66-97)
          float pv = 0.f;
          if (cd & kCodeFluid) {
            float py, pz;
            int cy, cz;
            if (jm > 0) { py = ny.x; cy = __float_as_int(ny.y); }
            else if (gy) { py = __ldcg(a.P + nbY + x); cy = a.code[nbY + x]; }
            else { py = 0.f; cy = 0; }
            if (wm > 0) { pz = nz.x; cz = __float_as_int(nz.y); }
            else if (gz) { pz = __ldcg(a.P + nbZ + x); cz = a.code[nbZ + x]; }
            else { pz = 0.f; cz = 0; }
            const float px = pprev;
            const int cx = cprev;
            const float A0 = a.A0f ? myF[slot] : (float)(cd & 7);
            float ev = A0;
            if (cd & kLowX) ev = ev - px * px;
            if (cd & kLowY) ev = ev - py * py;
            if (cd & kLowZ) ev = ev - pz * pz;
            const float k1 = (cd & kLowX) ? (float)(((cx & kHighY) ? 1 : 0) + ((cx & kHighZ) ? 1 : 0)) : 0.f;
            const float k2 = (cd & kLowY) ? (float)(((cy & kHighX) ? 1 : 0) + ((cy & kHighZ) ? 1 : 0)) : 0.f;
            const float k3 = (cd & kLowZ) ? (float)(((cz & kHighX) ? 1 : 0) + ((cz & kHighY) ? 1 : 0)) : 0.f;
            const float S3 = (k1 * (px * px) + k2 * (py * py)) + k3 * (pz * pz);
            ev = fmaf(-0.97f, S3, ev);       // e -= tau*(...): double in the reference, one rounding
            if (ev < 0.25f * A0) ev = A0;
            pv = 1.f / sqrtf(ev);
          }
          outv = pv;
          outp = __int_as_float(cd);
          myF[slot] = pv;
        } else if (MODE == 1) {
          // forward substitution (conjugategrad.cpp:141-148)
          float zv = 0.f;
          if (cd & kCodeFluid) {
            float t = myF[slot];
            if (cd & kLowX) t = t + vprev * pprev;
            if (cd & kLowY) {
              if (jm > 0) t = t + ny.x * ny.y;
              else t = t + __ldcg(a.z + nbY + x) * __ldg(a.P + nbY + x);
            }
            if (cd & kLowZ) {
              if (wm > 0) t = t + nz.x * nz.y;
              else t = t + __ldcg(a.z + nbZ + x) * __ldg(a.P + nbZ + x);
            }
            zv = myF[NT * kRing + slot] * t;
          }
          outv = zv;
          outp = myF[NT * kRing + slot];
          myF[slot] = zv;
        } else {
          // backward substitution (conjugategrad.cpp:150-159)
          float zv = 0.f;
          const float p = myF[2 * NT * kRing + slot];
          if (cd & kCodeFluid) {
            float t = myF[slot];
            if (cd & kHighX) t = t + vprev * p;
            if (cd & kHighY) t = t + (jm > 0 ? ny.x : __ldcg(a.z + nbY + x)) * p;
            if (cd & kHighZ) t = t + (wm > 0 ? nz.x : __ldcg(a.z + nbZ + x)) * p;
            zv = p * t;
          }
          acc += (double)(zv * myF[NT * kRing + slot]);
          outv = zv;
          myF[slot] = zv;
        }
        vprev = outv;
        pprev = MODE == 1 ? outp : (MODE == 0 ? outv : 0.f);
        cprev = cd;
        if ((xm & 7) == 7) {  // chunk complete: write it back in one piece
          const float4* src = reinterpret_cast<const float4*>(myF + (cm % kNR) * kCW);
          float* dst = (MODE == 0 ? a.P : a.z) + base + chunk_lo(cm);
          reinterpret_cast<float4*>(dst)[0] = src[0];
          reinterpret_cast<float4*>(dst)[1] = src[1];
        }
      }
      xb[(s & 1) * BZW * 32 + w * 32 + j] = make_float2(outv, outp);
    }
    cp_async_wait_all();
    __syncthreads();
    if (MODE == 2) {
      // fixed-order block reduction of the per-thread partial dots
      __shared__ double red[32];
      double v = acc;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (j == 0) red[w] = v;
      __syncthreads();
      if (tid == 0) {
        double t = 0.;
        for (int q = 0; q < BZW; q++) t += red[q];
        a.part[blk] = t;
      }
    }
    if (tid == 0) {
      __threadfence();
      st_release64(a.prog + blk, E | (unsigned long long)S);
    }
    __syncthreads();
  }
}

constexpr int kBZW = 8;

template <int MODE>
static size_t mic_col_smem() {
  constexpr int NT = 32 * kBZW;
  constexpr int NF = MODE == 2 ? 3 : (MODE == 1 ? 2 : 1);
  return (size_t)NF * NT * kRing * sizeof(float) + (size_t)NT * kRing * sizeof(code_t) + 2 * kBZW * 32 * sizeof(float2);
}

bool mic_col_supported(const Dims& d) { return d.is3d && d.nx % kCW == 0 && d.nx >= 2 * kCW; }

void mic_col_geometry(const Dims& d, int* nby, int* nbz) {
  *nby = (d.ny + 31) / 32;
  *nbz = (d.nz + kBZW - 1) / kBZW;
}

void mic_col_order(int nby, int nbz, int* order) {
  int n = 0;
  for (int L = 0; L <= nby + nbz - 2; L++)
    for (int c = 0; c < nbz; c++) {
      const int b = L - c;
      if (b >= 0 && b < nby) order[n++] = b + nby * c;
    }
}

int mic_col_prepare() {
  cudaError_t e = cudaSuccess;
  e = cudaFuncSetAttribute(k_mic_col<0, kBZW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mic_col_smem<0>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mic_col<1, kBZW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mic_col_smem<1>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mic_col<2, kBZW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mic_col_smem<2>());
  return e == cudaSuccess ? 0 : 1;
}

// mode: 0 factor, 1 forward, 2 backward (+beta), 3 backward for doInit (+sigma)
void launch_mic_col(const PcgBuffers& b, const MicColPlan& m, int mode, unsigned int epoch, long long spinLimit,
                    int ctas, cudaStream_t s) {
  MicColArgs a;
  a.d = b.d;
  a.code = b.code;
  a.A0f = b.A0f;
  a.P = b.P;
  a.r = b.residual;
  a.z = b.tmp;
  a.part = b.part;
  a.sc = b.sc;
  a.nby = m.nby;
  a.nbz = m.nbz;
  a.nblocks = m.nblocks;
  a.order = m.order;
  a.prog = m.prog;
  a.counter = m.counter;
  a.error = m.error;
  a.epoch = epoch;
  a.spinLimit = spinLimit;
  cudaMemsetAsync(m.counter, 0, sizeof(int), s);
  const int n = ctas < m.nblocks ? ctas : m.nblocks;
  count_launch();
  if (mode == 0) k_mic_col<0, kBZW><<<n, 32 * kBZW, mic_col_smem<0>(), s>>>(a);
  else if (mode == 1) k_mic_col<1, kBZW><<<n, 32 * kBZW, mic_col_smem<1>(), s>>>(a);
  else k_mic_col<2, kBZW><<<n, 32 * kBZW, mic_col_smem<2>(), s>>>(a);
  if (mode >= 2) launch_mic_finish(b, m.nblocks, mode == 3, s);
}

}  // namespace mgpu
