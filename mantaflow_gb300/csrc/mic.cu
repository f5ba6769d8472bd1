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
// The backward sweep mirrors x, y and z.  These sweeps are selected with
// MANTA_GB300_MIC=column on grids whose x size is a multiple of 8; the tiled
// kernel in pressure.cu is the default (at 256^3 on a GB300 it is about 15%
// faster: each column-block step costs ~0.6 us of barrier and shared-memory
// latency, which the skewed schedule's ~nx+ny+nz steps cannot hide).
#include "mg_common.cuh"
#include "mg_kernels.h"

namespace mgpu {

constexpr int kCW = 8;     // cells per staged chunk
constexpr int kNR = 4;     // chunks per ring (3 in flight)
constexpr int kRing = kCW * kNR;
constexpr int kLag = 39;   // steps a y-neighbour block must be ahead (31 + chunk flush)
constexpr int kAhead = 8;  // steps between reading an upwind value and using it

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
  long long spinLimit;  // nanoseconds any single wait may last
  int pubMask;    // publish progress when (step & pubMask) == 0
};

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
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

__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ unsigned long long lds_acquire64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.cta.shared.u64 %0, [%1];" : "=l"(v) : "r"((unsigned)__cvta_generic_to_shared(p)) : "memory");
  return v;
}
__device__ __forceinline__ void sts_release64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.cta.shared.u64 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared(p)), "l"(v) : "memory");
}
// barrier over the compute warps only (the sync warp runs free)
template <int BZW>
__device__ __forceinline__ void compute_bar() {
  asm volatile("bar.sync 1, %0;" ::"n"(32 * BZW) : "memory");
}

// MODE 0: factor (P), MODE 1: forward substitution, MODE 2: backward
// substitution with the fused dot(z, residual).
//
// Warps 0..BZW-1 compute.  Warp BZW is the block's sync warp: it publishes
// the compute warps' completed step count to global memory (fence.acq_rel +
// relaxed store, a release) and keeps acquiring the progress of the blocks
// this one depends on (relaxed polls, then fence.acq_rel), handing both over
// through shared memory with CTA-scope release/acquire.  The compute warps
// therefore never wait on an L2 round trip inside a step.
template <int MODE, int BZW>
__global__ void __launch_bounds__(32 * (BZW + 1), 1) k_mic_col(MicColArgs a) {
  constexpr int NT = 32 * BZW;
  constexpr int NF = MODE == 2 ? 3 : (MODE == 1 ? 2 : 1);  // staged float arrays per thread
  extern __shared__ __align__(16) unsigned char smem[];
  float* ringF = reinterpret_cast<float*>(smem);                       // [NF][NT][kRing]
  code_t* ringC = reinterpret_cast<code_t*>(ringF + NF * NT * kRing);  // [NT][kRing]
  float2* xb = reinterpret_cast<float2*>(ringC + NT * kRing);          // [2][BZW][32]
  __shared__ int s_blk;
  __shared__ unsigned long long s_availY, s_availZ, s_done;
  __shared__ double red[32];
  const Dims& d = a.d;
  const int tid = threadIdx.x, j = tid & 31, w = tid >> 5;
  const bool syncWarp = w == BZW;
  const int jm = MODE == 2 ? 31 - j : j;  // position in sweep order
  const int wm = MODE == 2 ? BZW - 1 - w : w;
  const int jn = MODE == 2 ? j + 1 : j - 1;  // upwind lane / warp
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
      s_availY = s_availZ = 0;
      s_done = E;
    }
    __syncthreads();
    const int blk = s_blk;
    if (blk < 0) return;
    const int b = blk % a.nby, c = blk / a.nby;
    int depY, depZ;
    if (MODE == 2) {
      depY = b + 1 < a.nby ? blk + 1 : -1;
      depZ = c + 1 < a.nbz ? blk + a.nby : -1;
    } else {
      depY = b > 0 ? blk - 1 : -1;
      depZ = c > 0 ? blk - a.nby : -1;
    }

    if (syncWarp) {
      // ---------------------------------------------------------- sync warp
      if (j == 0) {
        unsigned long long published = E, haveY = 0, haveZ = 0;
        const unsigned long long fin = E | (unsigned long long)S;
        if (depY < 0) { haveY = ~0ull; sts_release64(&s_availY, haveY); }
        if (depZ < 0) { haveZ = ~0ull; sts_release64(&s_availZ, haveZ); }
        long long spins = 0;
        unsigned long long idleSince = 0;
        for (;;) {
          bool idle = true;
          const unsigned long long done = lds_acquire64(&s_done);
          if (done > published && ((done - published) > (unsigned long long)a.pubMask || done == fin)) {
            fence_acq_rel_gpu();
            st_relaxed64(a.prog + blk, done);
            published = done;
            idle = false;
          }
          if (haveY < fin) {
            const unsigned long long v = ld_relaxed64(a.prog + depY);
            if (v > haveY && v >= E) {
              fence_acq_rel_gpu();
              haveY = v;
              sts_release64(&s_availY, v);
              idle = false;
            }
          }
          if (haveZ < fin) {
            const unsigned long long v = ld_relaxed64(a.prog + depZ);
            if (v > haveZ && v >= E) {
              fence_acq_rel_gpu();
              haveZ = v;
              sts_release64(&s_availZ, v);
              idle = false;
            }
          }
          if (published == fin) break;
          if (idle) {
            if (spins == 0) idleSince = gtimer();
            ++spins;
            if (gtimer() - idleSince > (unsigned long long)a.spinLimit || *((volatile int*)a.error) != 0) {
              atomicExch(a.error, 3);
              // let the compute warps run to the end (results are flagged)
              sts_release64(&s_availY, ~0ull);
              sts_release64(&s_availZ, ~0ull);
              while (lds_acquire64(&s_done) != fin) __nanosleep(64);
              published = fin;
              st_relaxed64(a.prog + blk, fin);
              break;
            }
            __nanosleep(32);
          } else {
            spins = 0;
          }
        }
      }
      __syncwarp();
    } else {
      // ------------------------------------------------------ compute warps
      const int y = 32 * b + j, zc = BZW * c + w;
      const bool line = y < d.ny && zc < d.nz;
      const long long base = line ? ix(d, 0, y, zc) : 0;
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
      unsigned long long haveY = 0, haveZ = 0;
      // Upwind values from the neighbouring blocks are read kAhead steps
      // before they are needed, into register queues indexed by step % 8
      // (static after unrolling), so no step waits on an L2 round trip.
      float qya[kAhead], qyb[kAhead], qza[kAhead], qzb[kAhead];
#pragma unroll
      for (int u = 0; u < kAhead; u++) qya[u] = qyb[u] = qza[u] = qzb[u] = 0.f;
      for (int g = -kAhead; g < S; g += kAhead) {
#pragma unroll
        for (int u = 0; u < kAhead; u++) {
          const int s = g + u;
          if (s >= S) break;
          if (tid == 0) {
            // The sync warp has acquired the neighbours' progress.  A shared
            // memory acquire costs about as much as five barrier steps, so
            // it is repeated only when the cached value no longer covers
            // this step (bounded in time; the sync warp flags errors first).
            const unsigned long long nY = E | (unsigned long long)min(S, s + kLag + kAhead);
            const unsigned long long nZ = E | (unsigned long long)min(S, s + BZW + kCW - 1 + kAhead);
            long long n = 0;
            unsigned long long tq = 0;
            while (haveY < nY || haveZ < nZ) {
              haveY = lds_acquire64(&s_availY);
              haveZ = lds_acquire64(&s_availZ);
              if (haveY >= nY && haveZ >= nZ) break;
              if (n++ == 0) tq = gtimer();
              if ((n & 255) == 0 && (gtimer() - tq > 2ull * (unsigned long long)a.spinLimit ||
                                     *((volatile int*)a.error) != 0)) {
                atomicExch(a.error, 4);
                haveY = haveZ = ~0ull;
                break;
              }
            }
          }
          compute_bar<BZW>();
          // steps < s are complete; hand that over at the publish granularity
          if (tid == 0 && s > 0 && (s & a.pubMask) == 0) sts_release64(&s_done, E | (unsigned long long)s);
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
            const int cd = myC[slot];
            const float2 ny = jm > 0 ? xb[((s - 1) & 1) * BZW * 32 + w * 32 + jn] : make_float2(qya[u], qyb[u]);
            const float2 nz = wm > 0 ? xb[((s - 1) & 1) * BZW * 32 + wn * 32 + j] : make_float2(qza[u], qzb[u]);
            if (MODE == 0) {
              // InitPreconditionModifiedIncompCholesky2 (conjugategrad.cpp:66-97)
              float pv = 0.f;
              if (cd & kCodeFluid) {
                const float py = ny.x, pz = nz.x;
                const int cy = __float_as_int(ny.y), cz = __float_as_int(nz.y);
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
                ev = fmaf(-0.97f, S3, ev);  // e -= tau*(...): double in the reference, one rounding
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
                if (cd & kLowY) t = t + ny.x * ny.y;
                if (cd & kLowZ) t = t + nz.x * nz.y;
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
                if (cd & kHighY) t = t + ny.x * p;
                if (cd & kHighZ) t = t + nz.x * p;
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
          // refill this step's queue slot with the upwind values for xm + kAhead
          const int xn = xm + kAhead;
          if (line && xn >= 0 && xn < d.nx) {
            const int xg = MODE == 2 ? d.nx - 1 - xn : xn;
            if (gy) {
              if (MODE == 0) { qya[u] = __ldcg(a.P + nbY + xg); qyb[u] = __int_as_float((int)a.code[nbY + xg]); }
              else if (MODE == 1) { qya[u] = __ldcg(a.z + nbY + xg); qyb[u] = __ldg(a.P + nbY + xg); }
              else qya[u] = __ldcg(a.z + nbY + xg);
            }
            if (gz) {
              if (MODE == 0) { qza[u] = __ldcg(a.P + nbZ + xg); qzb[u] = __int_as_float((int)a.code[nbZ + xg]); }
              else if (MODE == 1) { qza[u] = __ldcg(a.z + nbZ + xg); qzb[u] = __ldg(a.P + nbZ + xg); }
              else qza[u] = __ldcg(a.z + nbZ + xg);
            }
          }
          xb[(s & 1) * BZW * 32 + w * 32 + j] = make_float2(outv, outp);
        }
      }
      cp_async_wait_all();
      if (MODE == 2) {
        // fixed-order reduction of the per-thread partial dots
        double v = acc;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (j == 0) red[w] = v;
      }
      compute_bar<BZW>();
      if (tid == 0) {
        if (MODE == 2) {
          double t = 0.;
          for (int q = 0; q < BZW; q++) t += red[q];
          a.part[blk] = t;
        }
        sts_release64(&s_done, E | (unsigned long long)S);  // the sync warp publishes it
      }
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
  a.pubMask = m.pubMask;
  cudaMemsetAsync(m.counter, 0, sizeof(int), s);
  const int n = ctas < m.nblocks ? ctas : m.nblocks;
  count_launch();
  const int nt = 32 * (kBZW + 1);  // compute warps + the sync warp
  if (mode == 0) k_mic_col<0, kBZW><<<n, nt, mic_col_smem<0>(), s>>>(a);
  else if (mode == 1) k_mic_col<1, kBZW><<<n, nt, mic_col_smem<1>(), s>>>(a);
  else k_mic_col<2, kBZW><<<n, nt, mic_col_smem<2>(), s>>>(a);
  if (mode >= 2) launch_mic_finish(b, m.nblocks, mode == 3, s);
}

}  // namespace mgpu
