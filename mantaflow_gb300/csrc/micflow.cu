// MIC(0) preconditioner sweeps as a tile dataflow.
//
// The reference factors and applies the modified incomplete Cholesky
// preconditioner with lexicographic loops (conjugategrad.cpp:66-97,
// 135-160): cell (x,y,z) needs the finished values of (x-1,y,z), (x,y-1,z)
// and (x,y,z-1).  Any order that respects those dependencies reproduces the
// serial result bit for bit.
//
//  * The grid is cut into 16^3 tiles, handed out to persistent CTAs in
//    (a+b+c) tile order.  A CTA stages its tile in shared memory and sweeps
//    the tile's 46 diagonal cell levels with one thread per x-line and one
//    barrier per level.  The neighbour values live in a tile padded by one
//    cell on its three upwind sides, so the level body is the same for every
//    cell: three shared-memory reads, the cell's arithmetic, two writes.
//  * Two more warps (the halo warps) move data across tile faces: during
//    level L they fill the padding cells that level L+1 reads and publish
//    the face cells that level L-1 computed.  Every such task is a fixed
//    cell sequence linear in L, set up once per tile, so a halo lane spends
//    a handful of instructions per level and never holds the barrier up.
//  * A tile does not wait for its upstream tiles to finish.  Each cell on a
//    tile's three downstream faces is published the moment it is computed,
//    as a 64-bit word holding the value, the cell's stencil code and the
//    sweep's epoch.  One store carries data and tag together, so a reader
//    that sees the current epoch sees the value: no flag and no fence.  The
//    downstream tile reads the words it needs level by level (prefetched
//    four levels ahead, polled with a time bound when not there yet), so
//    neighbouring tiles overlap like the stages of a pipeline.
//  * Tiles are handed out in an order in which a tile only waits for tiles
//    handed out before it, which are running or done: no deadlock whatever
//    the residency.
//
// The backward sweep runs the same schedule in mirrored coordinates.
#include <cstring>

#include "mg_common.cuh"
#include "mg_kernels.h"

namespace mgpu {

namespace {

constexpr int kT = 16;               // tile edge
constexpr int kTC = kT * kT * kT;    // cells per tile
constexpr int kNL = 3 * kT - 2;      // cell levels per tile
constexpr int kQ = 4;                // halo prefetch distance (levels)

struct FlowArgs {
  FlowScene one;              // the scene of a single-scene launch
  const FlowScene* scenes;    // batched launch: the scene table
  int ntiles;
  const int* order;           // single scene: tile indices in dispatch order
  const int2* order2;         // batched: (scene, tile) pairs in dispatch order
  int* counter;
  int* error;
  unsigned int epoch;
  const unsigned int* epochDev;  // batched launches: the epoch in device memory (set by k_flow_prep)
  unsigned int waitXor;  // 0; non-zero only to make every wait run out (failure-path tests)
  long long spinLimit;
};

__device__ __forceinline__ unsigned long long ftimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned long long ld_word(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_word(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long make_word(float v, int code, unsigned ep16) {
  return ((unsigned long long)((ep16 << 16) | (unsigned)(code & 0xffff)) << 32) | (unsigned long long)__float_as_uint(v);
}
__device__ __forceinline__ bool current(unsigned long long w, unsigned ep16) { return (unsigned)(w >> 48) == ep16; }

// the word at p once it carries this sweep's epoch; gives up after `limit`
// nanoseconds or once another wait has given up.  Giving up flags the error
// and ends the CG (done), so the solve's later launches return at once and
// the host reports the timeout.
__device__ __noinline__ unsigned long long poll_word(const unsigned long long* p, unsigned ep16, long long limit,
                                                    int* error, CgScalars* sc) {
  unsigned long long v = ld_word(p);
  if (current(v, ep16)) return v;
  const unsigned long long t0 = ftimer();
  for (unsigned n = 1;; n++) {
    v = ld_word(p);
    if (current(v, ep16)) return v;
    if ((n & 31) == 0 && (ftimer() - t0 > (unsigned long long)limit || *((volatile int*)error) != 0)) {
      if (atomicExch(error, 6) == 0) {
        sc->status = 3;
        sc->done = 1;
      }
      return v;
    }
  }
}

}  // namespace

// padded index of tile cell (x,y,z), x,y,z in [-1,16).  Row stride 19 and
// plane stride 324 (not 17 and 289): a warp's cells of one level, (L-y-z,
// y, z) for y = 0..15 and two z, then fall on 32 distinct banks.
constexpr int kSY = 19, kSZ = 324;
__host__ __device__ constexpr int pad(int x, int y, int z) { return (x + 1) + kSY * (y + 1) + kSZ * (z + 1); }
constexpr int kPad = kSZ * (kT + 1);

template <int MODE>
__host__ __device__ constexpr size_t flow_smem() {
  // s_n (padded neighbour values), s_cp (padded codes), then s_P and s_v
  // (unpadded; forward: r -> z, backward: r for the dot)
  return (size_t)kPad * 4 + (size_t)((kPad * 2 + 15) / 16 * 16) + (MODE != 0 ? 2 * (size_t)kTC * 4 : 0);
}

// MODE 0: factor (P).  MODE 1: forward substitution r -> z.  MODE 2:
// backward substitution z -> z with the fused dot(z, r) per tile.
template <int MODE, bool kBatch>
__global__ void __launch_bounds__(320) k_mic_flow(FlowArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  float* s_n = reinterpret_cast<float*>(smem);                                  // [kPad] value neighbours use
  code_t* s_cp = reinterpret_cast<code_t*>(smem + (size_t)kPad * 4);             // [kPad] stencil codes
  float* s_P = reinterpret_cast<float*>(smem + (size_t)kPad * 4 + (size_t)((kPad * 2 + 15) / 16 * 16));  // [kTC]
  float* s_v = s_P + kTC;                                   // [kTC] forward: r -> z; backward: r
  __shared__ int s_tile, s_scene;
  __shared__ double s_red[8];
  const int tid = threadIdx.x;
  const bool haloWarp = tid >= 256;
  const int ly = tid & (kT - 1), lz = (tid >> 4) & (kT - 1);
  const int hw = (tid - 256) >> 5, hl = tid & 31;  // halo warp 0/1 and its lane
  if (!kBatch && MODE != 0 && a.one.sc->done) return;
  const unsigned ep16 = (kBatch ? *((volatile const unsigned int*)a.epochDev) : a.epoch) & 0xffffu;
  const unsigned wep16 = ep16 ^ a.waitXor;  // the epoch the fill words must carry
  auto gx = [&](int c, int n) { return MODE == 2 ? n - 1 - c : c; };  // global coordinate of a sweep coordinate

  for (;;) {
    if (tid == 0) {
      const int q = atomicAdd(a.counter, 1);
      if (kBatch) {
        const int2 e = q < a.ntiles ? a.order2[q] : make_int2(-1, -1);
        s_scene = e.x;
        s_tile = e.y;
      } else {
        s_scene = 0;
        s_tile = q < a.ntiles ? a.order[q] : -1;
      }
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile < 0) return;
    const FlowScene& S = kBatch ? a.scenes[s_scene] : a.one;
    // a converged scene's tiles are skipped whole (its downstream tiles too)
    if (kBatch && MODE != 0 && S.sc->done) {
      __syncthreads();
      continue;
    }
    const Dims& d = S.d;
    const int ta = tile % S.tx, tb = (tile / S.tx) % S.ty, tc = tile / (S.tx * S.ty);
    const int x0 = ta * kT, y0 = tb * kT, z0 = tc * kT;
    const int nxT = min(kT, d.nx - x0), nyT = min(kT, d.ny - y0), nzT = min(kT, d.nz - z0);  // tile extents

    // ---- stage the tile (inputs only; independent of the neighbours)
    if (!haloWarp) {
#pragma unroll
      for (int q = 0; q < kTC / 256; q++) {
        const int e = tid + 256 * q;
        const int x = e & (kT - 1), y = (e >> 4) & (kT - 1), zc = e >> 8;
        code_t c = 0;
        float v = 0.f, p = 0.f, rv = 0.f;
        if (x < nxT && y < nyT && zc < nzT) {
          const long long g = ix(d, gx(x0 + x, d.nx), gx(y0 + y, d.ny), gx(z0 + zc, d.nz));
          c = S.code[g];
          if (MODE == 0) {
            v = S.A0f ? S.A0f[g] : 0.f;
          } else {
            p = S.P[g];
            rv = S.r[g];
            if (MODE == 2) v = S.z[g];
          }
        }
        const int pe = pad(x, y, zc);
        s_cp[pe] = c;
        if (MODE != 1) s_n[pe] = v;  // backward: z in, z out; factor: A0 (ghost fluid) in, P out
        if (MODE != 0) {
          s_P[e] = p;
          s_v[e] = rv;
        }
      }
    }
    __syncthreads();

    const bool lineOk = ly < nyT && lz < nzT;

    // Halo tasks of this lane.  A fill task copies the face word of an
    // upstream tile into the padding cell that level Lh reads, for Lh in
    // [fLo, fHi): word fSrc + fSS*Lh -> s_n/s_cp[fDst + fDS*Lh].  A publish
    // task stores the face cell that level Lp computed, for Lp in [pLo, pHi):
    // s_n/s_cp[pSrc + pSS*Lp] -> word pDst + pDS*Lp.
    //   warp 0, lanes 0-15:  x-face fill and publish (hi = lane = y)
    //   warp 0, lanes 16-31: z-face fill and publish (hi = y)
    //   warp 1, lanes 0-15:  y-face fill and publish (hi = z)
    bool fOK = false, pOK = false;
    int fLo = 0, fHi = 0, fSS = 0, fDst = 0, fDS = 0, pLo = 0, pHi = 0, pSrc = 0, pSS = 0, pDS = 0;
    const unsigned long long* fSrc = S.face;
    unsigned long long* pDst = S.face;
    if (haloWarp) {
      const int hi = hl & 15;
      if (hw == 0 && hl < 16) {           // x: thread (hi, zz) reads (-1, hi, zz) at level hi + zz
        fOK = ta > 0 && hi < nyT;
        fLo = hi; fHi = hi + nzT;
        fSrc = S.face + ((long long)(tile - 1) * 3 + 0) * (kT * kT) + hi - kT * hi; fSS = kT;
        fDst = pad(-1, hi, -hi); fDS = kSZ;
        pOK = ta + 1 < S.tx && hi < nyT && nxT == kT;  // cell (15, hi, zz) at level 15 + hi + zz
        pLo = kT - 1 + hi; pHi = pLo + nzT;
        pDst = S.face + (long long)tile * 3 * (kT * kT) + hi - kT * (kT - 1 + hi); pDS = kT;
        pSrc = pad(kT - 1, hi, -(kT - 1) - hi); pSS = kSZ;
      } else if (hw == 0) {               // z: thread (hi, 0) reads (x, hi, -1) at level x + hi
        fOK = tc > 0 && hi < nyT;
        fLo = hi; fHi = hi + nxT;
        fSrc = S.face + ((long long)(tile - S.tx * S.ty) * 3 + 2) * (kT * kT) + (kT - 1) * hi; fSS = 1;
        fDst = pad(-hi, hi, -1); fDS = 1;
        pOK = tc + 1 < S.tz && hi < nyT && nzT == kT;  // cell (x, hi, 15) at level x + hi + 15
        pLo = kT - 1 + hi; pHi = pLo + nxT;
        pDst = S.face + (long long)tile * 3 * (kT * kT) + 2 * kT * kT + (kT - 1) * hi - (kT - 1); pDS = 1;
        pSrc = pad(-(kT - 1) - hi, hi, kT - 1); pSS = 1;
      } else if (hl < 16) {               // y: thread (0, hi) reads (x, -1, hi) at level x + hi
        fOK = tb > 0 && hi < nzT;
        fLo = hi; fHi = hi + nxT;
        fSrc = S.face + ((long long)(tile - S.tx) * 3 + 1) * (kT * kT) + (kT - 1) * hi; fSS = 1;
        fDst = pad(-hi, -1, hi); fDS = 1;
        pOK = tb + 1 < S.ty && hi < nzT && nyT == kT;  // cell (x, 15, hi) at level x + 15 + hi
        pLo = kT - 1 + hi; pHi = pLo + nxT;
        pDst = S.face + (long long)tile * 3 * (kT * kT) + kT * kT + (kT - 1) * hi - (kT - 1); pDS = 1;
        pSrc = pad(-(kT - 1) - hi, kT - 1, hi); pSS = 1;
      }
    }
    unsigned long long q[kQ];  // fill words, loaded kQ levels ahead
#pragma unroll
    for (int u = 0; u < kQ; u++) q[u] = 0;

    for (int L0 = -kQ - 1; L0 <= kNL; L0 += kQ) {
#pragma unroll
      for (int u = 0; u < kQ; u++) {
        const int L = L0 + u;
        if (L > kNL) break;
        if (haloWarp) {
          const int Lp = L - 1;  // publish what level L-1 computed
          if (pOK && Lp >= pLo && Lp < pHi) {
            const int pe = pSrc + pSS * Lp;
            st_word(pDst + pDS * Lp, make_word(s_n[pe], s_cp[pe], ep16));
          }
          const int Lh = L + 1;  // fill what level L+1 reads
          if (fOK && Lh >= fLo && Lh < fHi) {
            unsigned long long w = q[u];
            if (!current(w, wep16)) w = poll_word(fSrc + fSS * Lh, wep16, a.spinLimit, a.error, S.sc);
            const int pe = fDst + fDS * Lh;
            s_n[pe] = __uint_as_float((unsigned)w);
            s_cp[pe] = (code_t)((w >> 32) & 0xffffu);
          }
          const int Ln = Lh + kQ;  // and load the word of level L+1+kQ into the slot just used
          if (fOK && Ln >= fLo && Ln < fHi) q[u] = ld_word(fSrc + fSS * Ln);
        } else if (L >= 0 && L < kNL) {
          const int x = L - ly - lz;
          if (lineOk && x >= 0 && x < nxT) {
            const int pe = pad(x, ly, lz);
            const int e = x + kT * ly + kT * kT * lz;
            const int cd = s_cp[pe];
            if (MODE == 0) {
              // InitPreconditionModifiedIncompCholesky2 (conjugategrad.cpp:66-97)
              float pv = 0.f;
              if (cd & kCodeFluid) {
                const float px = s_n[pe - 1], py = s_n[pe - kSY], pz = s_n[pe - kSZ];
                const int cx = s_cp[pe - 1], cy = s_cp[pe - kSY], cz = s_cp[pe - kSZ];
                const float A0 = S.A0f ? s_n[pe] : (float)(cd & 7);
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
              s_n[pe] = pv;
            } else if (MODE == 1) {
              // forward substitution (conjugategrad.cpp:141-148); the
              // neighbours hold z*P, the product the reference forms
              const float p = s_P[e];
              float zv = 0.f;
              if (cd & kCodeFluid) {
                float t = s_v[e];
                if (cd & kLowX) t = t + s_n[pe - 1];
                if (cd & kLowY) t = t + s_n[pe - kSY];
                if (cd & kLowZ) t = t + s_n[pe - kSZ];
                zv = p * t;
              }
              s_v[e] = zv;
              s_n[pe] = zv * p;
            } else {
              // backward substitution (conjugategrad.cpp:150-159) in sweep
              // coordinates: the reference's upper neighbours are upwind
              const float p = s_P[e];
              float zv = 0.f;
              if (cd & kCodeFluid) {
                float t = s_n[pe];
                if (cd & kHighX) t = t + s_n[pe - 1] * p;
                if (cd & kHighY) t = t + s_n[pe - kSY] * p;
                if (cd & kHighZ) t = t + s_n[pe - kSZ] * p;
                zv = p * t;
              }
              s_n[pe] = zv;
            }
          }
        }
        __syncthreads();
      }
    }

    // ---- write back, and the backward sweep's dot(z, residual)
    double acc = 0.;
    if (!haloWarp) {
#pragma unroll
      for (int q = 0; q < kTC / 256; q++) {
        const int e = tid + 256 * q;
        const int x = e & (kT - 1), y = (e >> 4) & (kT - 1), zc = e >> 8;
        if (x < nxT && y < nyT && zc < nzT) {
          const long long g = ix(d, gx(x0 + x, d.nx), gx(y0 + y, d.ny), gx(z0 + zc, d.nz));
          const float v = MODE == 1 ? s_v[e] : s_n[pad(x, y, zc)];
          if (MODE == 0) S.P[g] = v;
          else S.z[g] = v;
          if (MODE == 2) acc += (double)(v * s_v[e]);
        }
      }
    }
    if (MODE == 2) {
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (!haloWarp && (tid & 31) == 0) s_red[tid >> 5] = acc;
      __syncthreads();
      if (tid == 0) {
        double t = 0.;
        for (int w = 0; w < 8; w++) t += s_red[w];
        S.part[tile] = t;
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- host side
template <bool kB>
static cudaError_t flow_attrs() {
  cudaError_t e = cudaFuncSetAttribute(k_mic_flow<0, kB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)flow_smem<0>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mic_flow<1, kB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)flow_smem<1>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mic_flow<2, kB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)flow_smem<2>());
  return e;
}

static int g_flowCtas = 0;  // resident CTAs of a sweep on the whole device

int mic_flow_prepare(int* ctasPerSm) {
  cudaError_t e = flow_attrs<false>();
  if (e == cudaSuccess) e = flow_attrs<true>();
  int n = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mic_flow<1, false>, 320, flow_smem<1>());
  *ctasPerSm = n > 0 ? n : 1;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  g_flowCtas = *ctasPerSm * (sms > 0 ? sms : 1);
  return e == cudaSuccess ? 0 : 1;
}

int mic_flow_device_ctas() { return g_flowCtas > 0 ? g_flowCtas : 1; }

size_t mic_flow_face_words(int ntiles) { return (size_t)ntiles * 3 * kT * kT; }

template <bool kB>
static void flow_launch(const FlowArgs& a, int mode, int ctas, cudaStream_t s) {
  count_launch();
  if (mode == 0) k_mic_flow<0, kB><<<ctas, 320, flow_smem<0>(), s>>>(a);
  else if (mode == 1) k_mic_flow<1, kB><<<ctas, 320, flow_smem<1>(), s>>>(a);
  else k_mic_flow<2, kB><<<ctas, 320, flow_smem<2>(), s>>>(a);
}

// mode: 0 factor, 1 forward, 2 backward (+beta), 3 backward for doInit (+sigma)
void launch_mic_flow(const PcgBuffers& b, const MicPlan& m, unsigned long long* face, int mode, unsigned int epoch,
                     long long spinLimit, cudaStream_t s, bool stall) {
  FlowArgs a;
  a.one.d = b.d;
  a.one.code = b.code;
  a.one.A0f = b.A0f;
  a.one.P = b.P;
  a.one.r = b.residual;
  a.one.z = b.tmp;
  a.one.part = b.part;
  a.one.sc = b.sc;
  a.one.tx = m.tx;
  a.one.ty = m.ty;
  a.one.tz = m.tz;
  a.one.face = face;
  a.scenes = nullptr;
  a.ntiles = m.ntiles;
  a.order = m.order;
  a.order2 = nullptr;
  a.counter = m.counter;
  a.error = m.error;
  a.epoch = epoch;
  a.epochDev = nullptr;
  a.waitXor = stall ? 0x8000u : 0u;
  a.spinLimit = spinLimit;
  cudaMemsetAsync(m.counter, 0, sizeof(int), s);
  flow_launch<false>(a, mode, m.ctas < m.ntiles ? m.ctas : m.ntiles, s);
  if (mode >= 2) launch_mic_finish(b, m.ntiles, mode == 3, s);
}

// before each batched sweep: the tile counter back to zero and the next
// epoch (never 0 in its low 16 bits, the value of freshly cleared face
// words).  On the device, so that a captured graph replays new epochs.
__global__ void k_flow_prep(int* counter, unsigned int* epoch) {
  *counter = 0;
  unsigned int e = *epoch + 1u;
  if ((e & 0xffffu) == 0u) e++;
  *epoch = e;
}

// the sweep over the tiles of several scenes in one launch: order2 lists
// (scene, tile) pairs so that each tile comes after the tiles it waits for
// (wavefront level first); the backward modes leave each scene's per-tile
// dot partials in its part[] for the caller's per-scene reduction
void launch_mic_flow_batch(const FlowScene* scenes, const int2* order2, int ntiles, int ctas, int* counter, int* error,
                           int mode, unsigned int* epochDev, long long spinLimit, cudaStream_t s) {
  FlowArgs a;
  memset(&a.one, 0, sizeof(a.one));
  a.scenes = scenes;
  a.ntiles = ntiles;
  a.order = nullptr;
  a.order2 = order2;
  a.counter = counter;
  a.error = error;
  a.epoch = 0u;
  a.epochDev = epochDev;
  a.waitXor = 0u;
  a.spinLimit = spinLimit;
  count_launch();
  k_flow_prep<<<1, 1, 0, s>>>(counter, epochDev);
  flow_launch<true>(a, mode == 3 ? 2 : mode, ctas < ntiles ? ctas : ntiles, s);
}

}  // namespace mgpu
