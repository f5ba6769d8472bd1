// MIC(0) preconditioner sweeps as warp wavefronts.
//
// The reference factors and applies the modified incomplete Cholesky
// preconditioner with lexicographic loops (conjugategrad.cpp:66-97,
// 135-160): cell (x,y,z) needs the finished values of (x-1,y,z), (x,y-1,z)
// and (x,y,z-1).  Any schedule that respects those three dependencies
// reproduces the serial result bit for bit.  This one needs no block
// barrier and no memory fence:
//
//  * A warp owns a unit of 32 y-lines x ZW z-lines (ZW = 4 or 8) over the
//    whole x range.
//    Lane j holds the ZW lines (y0+j, z0+k), k = 0..ZW-1 ("layers"), and at
//    step s works on x = s - j - k in every layer at once.  So at step s the
//    x- and z-neighbours of a cell are the lane's own results of step s-1
//    (registers) and the y-neighbour is lane j-1's result of step s-1
//    (one shuffle).  The ZW layers of a step are independent, and the step
//    body has no branches, so they interleave: ZW-way instruction-level
//    parallelism per lane.
//  * Neighbouring units hand values across their faces through words of 64
//    bits in global memory: the value in the low half, the sweep's epoch
//    (16 bits) and the cell's stencil code in the high half.  A word is
//    written once per sweep with one store, so a reader that sees the
//    current epoch sees the value written with it; no flag, no fence.  The
//    words are laid out by step, so one step of a unit writes and reads
//    contiguous runs.  Readers prefetch them eight steps ahead with
//    cp.async.cg (L2, never a stale L1 line) and fall back to a bounded poll
//    when a word is not there yet.
//  * Units are handed out in (yb + zb) order, so a unit only waits for
//    units handed out before it, which are running or done: the scheme
//    cannot deadlock whatever the residency.
//  * Each lane streams its ZW lines through private shared-memory rings of
//    two 8-cell chunks, filled by cp.async one chunk ahead, and writes its
//    results back chunk by chunk.  Every step commits one cp.async group and
//    waits for the group of eight steps earlier.
//
// The backward sweep runs the same schedule on mirrored coordinates.
#include "mg_common.cuh"
#include "mg_kernels.h"

namespace mgpu {

namespace {

constexpr int kRC = 16;     // ring cells per line: two chunks of 8
constexpr int kPD = 8;      // prefetch distance in steps (exchange rows, chunks)

struct WaveArgs {
  Dims d;
  const code_t* code;
  const float* A0f;
  float* P;
  const float* r;
  float* z;
  double* part;
  CgScalars* sc;
  int nyb, nzb, nunits;
  const int* order;
  int* counter;
  int* error;
  unsigned long long* exY;  // [nyb][nzb][rows][ZW]
  unsigned long long* exZ;  // [nzb][nyb][rows][32]
  int rows;                 // nx + 32
  unsigned int epoch;
  long long spinLimit;      // nanoseconds a single wait may last
};

__device__ __forceinline__ unsigned long long wtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed_v2u64(unsigned long long* p, unsigned long long v0, unsigned long long v1) {
  asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(v0), "l"(v1) : "memory");
}
__device__ __forceinline__ void cpa16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpa_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cpa_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ unsigned long long pack_word(float v, int code, unsigned ep16) {
  return ((unsigned long long)((ep16 << 16) | (unsigned)(code & 0xffff)) << 32) | (unsigned long long)__float_as_uint(v);
}
__device__ __forceinline__ float word_value(unsigned long long w) { return __uint_as_float((unsigned)w); }
__device__ __forceinline__ int word_code(unsigned long long w) { return (int)((w >> 32) & 0xffffu); }
__device__ __forceinline__ bool word_current(unsigned long long w, unsigned ep16) { return (unsigned)(w >> 48) == ep16; }

// the word at g once it carries this sweep's epoch; gives up (and flags the
// error) after `limit` nanoseconds or when another wait has given up
__device__ __noinline__ unsigned long long wait_word(const unsigned long long* g, unsigned ep16, long long limit,
                                                    int* error) {
  unsigned long long v = ld_relaxed_u64(g);
  if (word_current(v, ep16)) return v;
  const unsigned long long t0 = wtimer();
  for (unsigned n = 1;; n++) {
    v = ld_relaxed_u64(g);
    if (word_current(v, ep16)) return v;
    if ((n & 63) == 0 && (wtimer() - t0 > (unsigned long long)limit || *((volatile int*)error) != 0)) {
      atomicExch(error, 5);
      return v;
    }
  }
}

}  // namespace

// Lane activity of a step: layers k with a valid line and 0 <= x - k < nx,
// where x = s - j is the position of layer 0.
template <int ZW>
__device__ __forceinline__ unsigned step_mask(int sj, int nx, unsigned lineMask) {
  constexpr unsigned full = (1u << ZW) - 1u;
  if (sj < 0 || sj - (ZW - 1) >= nx) return 0u;
  unsigned m = sj >= ZW - 1 ? full : ((1u << (sj + 1)) - 1u);   // k <= sj
  const int lo = sj - nx + 1;                                     // k >= sj - nx + 1
  if (lo > 0) m &= ~((1u << lo) - 1u);
  return m & lineMask;
}

// MODE 0: factor (P).  MODE 1: forward substitution r -> z.  MODE 2:
// backward substitution z -> z with the fused dot(z, r) per unit.
template <int MODE, int ZW>
__global__ void __launch_bounds__(32) k_mic_wave(WaveArgs a) {
  constexpr int NF = MODE == 2 ? 3 : (MODE == 1 ? 2 : 1);  // staged float arrays
  constexpr int AS = 32 * ZW * kRC;                         // floats per staged array
  extern __shared__ __align__(16) unsigned char smem[];
  float* ringF = reinterpret_cast<float*>(smem);                          // [NF][32][ZW][kRC]
  code_t* ringC = reinterpret_cast<code_t*>(ringF + NF * AS);            // [32][ZW][kRC]
  unsigned long long* bufZ = reinterpret_cast<unsigned long long*>(ringC + 32 * ZW * kRC);  // [kPD][32]
  unsigned long long* bufY = bufZ + kPD * 32;                             // [kPD][ZW]
  const Dims& d = a.d;
  const int j = threadIdx.x;
  if (MODE != 0 && a.sc->done) return;
  const unsigned ep16 = a.epoch & 0xffffu;
  const int S = d.nx + 31 + ZW - 1;  // steps of a unit
  const int nch = d.nx >> 3;
  float* const myF = ringF + j * ZW * kRC;    // layer k of array A: myF + A*AS + k*kRC
  code_t* const myC = ringC + j * ZW * kRC;   // layer k: myC + k*kRC

  for (;;) {
    int q = 0;
    if (j == 0) q = atomicAdd(a.counter, 1);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= a.nunits) return;
    const int unit = a.order[q];
    const int yb = unit % a.nyb, zb = unit / a.nyb;
    // sweep coordinates: the backward sweep mirrors x, y and z
    const int ys = 32 * yb + j;
    const bool yok = ys < d.ny;
    const int yg = MODE == 2 ? d.ny - 1 - ys : ys;
    const bool hasYup = yb > 0, hasZup = zb > 0;
    const bool hasYdn = yb + 1 < a.nyb, hasZdn = zb + 1 < a.nzb;
    unsigned lineMask = 0;
#pragma unroll
    for (int k = 0; k < ZW; k++)
      if (yok && ZW * zb + k < d.nz) lineMask |= 1u << k;
    const unsigned rowMask = __shfl_sync(0xffffffffu, lineMask, 0);  // lane 0's layers
    auto line_base = [&](int k) -> long long {
      const int zs = ZW * zb + k;
      const int zg = MODE == 2 ? d.nz - 1 - zs : zs;
      return (long long)yg * d.sy + (long long)zg * d.sz;
    };
    auto chunk_lo = [&](int c) { return MODE == 2 ? d.nx - 8 * (c + 1) : 8 * c; };
    auto load_chunk = [&](int k, int c) {
      const long long g = line_base(k) + chunk_lo(c);
      float* f = myF + k * kRC + (c & 1) * 8;
      if (MODE == 1) {
        cpa16(f, a.r + g);
        cpa16(f + 4, a.r + g + 4);
        cpa16(f + AS, a.P + g);
        cpa16(f + AS + 4, a.P + g + 4);
      } else if (MODE == 2) {
        cpa16(f, a.z + g);
        cpa16(f + 4, a.z + g + 4);
        cpa16(f + AS, a.r + g);
        cpa16(f + AS + 4, a.r + g + 4);
        cpa16(f + 2 * AS, a.P + g);
        cpa16(f + 2 * AS + 4, a.P + g + 4);
      } else if (a.A0f) {
        cpa16(f, a.A0f + g);
        cpa16(f + 4, a.A0f + g + 4);
      }
      cpa16(myC + k * kRC + (c & 1) * 8, a.code + g);
    };
    const unsigned long long* srcZ = a.exZ + ((long long)((zb - 1) * a.nyb + yb) * a.rows) * 32;  // [row][32]
    const unsigned long long* srcY = a.exY + ((long long)((yb - 1) * a.nzb + zb) * a.rows) * ZW;  // [row][ZW]
    unsigned long long* dstZ = a.exZ + ((long long)(zb * a.nyb + yb) * a.rows) * 32;
    unsigned long long* dstY = a.exY + ((long long)(yb * a.nzb + zb) * a.rows) * ZW;

    float wv[ZW];  // each layer's result of the previous step (what its neighbours use)
    int cv[ZW];    // and that cell's stencil code
#pragma unroll
    for (int k = 0; k < ZW; k++) { wv[k] = 0.f; cv[k] = 0; }
    double acc = 0.;

    for (int g = -kPD; g < S; g += kPD) {
#pragma unroll
      for (int u = 0; u < kPD; u++) {
        const int s = g + u;
        if (s >= S) break;
        const int sj = s - j;  // x of layer 0
        // (a) everything issued eight steps ago has landed (lanes 0-15
        // fetched the z-face words of all 32 lanes)
        cpa_wait<kPD - 1>();
        __syncwarp();
        const unsigned act = step_mask<ZW>(sj, d.nx, lineMask);
        // (b) face values from the neighbouring units: lane j's layer 0 reads
        // a z-face word, lane 0 reads the y-face words of all its layers.  If
        // a prefetched copy is stale the warp polls every missing word at
        // once (lane k < ZW taking y-face word k) and lane 0 collects them.
        unsigned long long ez = 0;
        unsigned long long ey[ZW];
#pragma unroll
        for (int k = 0; k < ZW; k++) ey[k] = 0;
        {
          const bool needZ = hasZup && (act & 1u);
          bool stale = false;
          if (needZ) {
            ez = bufZ[u * 32 + j];
            stale = !word_current(ez, ep16);
          }
          if (j == 0 && hasYup && act) {
#pragma unroll
            for (int k = 0; k < ZW; k++) {
              ey[k] = bufY[u * ZW + k];
              if (act >> k & 1u) stale |= !word_current(ey[k], ep16);
            }
          }
          if (__any_sync(0xffffffffu, stale)) {
            if (needZ && !word_current(ez, ep16)) ez = wait_word(srcZ + (long long)s * 32 + j, ep16, a.spinLimit, a.error);
            unsigned long long w0 = 0;
            const unsigned act0 = __shfl_sync(0xffffffffu, act, 0);
            if (hasYup && j < ZW && (act0 >> j & 1u))
              w0 = wait_word(srcY + (long long)s * ZW + j, ep16, a.spinLimit, a.error);
#pragma unroll
            for (int k = 0; k < ZW; k++) {
              const unsigned long long w = __shfl_sync(0xffffffffu, w0, k);
              if (j == 0 && (act0 >> k & 1u)) ey[k] = w;
            }
          }
        }
        // (c) the cells of this step.  Inactive layers compute on whatever
        // the ring holds; only their stores are masked.  Layers run last to
        // first so that wv[k-1] is still the previous step's value.
        float wy[ZW];
        int cy[ZW];
#pragma unroll
        for (int k = 0; k < ZW; k++) {
          wy[k] = __shfl_up_sync(0xffffffffu, wv[k], 1);
          if (MODE == 0) cy[k] = __shfl_up_sync(0xffffffffu, cv[k], 1);
        }
        float dsum = 0.f;
#pragma unroll
        for (int k = ZW - 1; k >= 0; k--) {
          const bool on = act >> k & 1u;
          const int x = sj - k;
          const int off = MODE == 2 ? ((x & (kRC - 1)) ^ 7) : (x & (kRC - 1));
          float* f = myF + k * kRC + off;
          const int cd = myC[k * kRC + off];
          const float vy = j > 0 ? wy[k] : word_value(ey[k]);
          const float vz = k > 0 ? wv[k - 1] : word_value(ez);
          float out;
          if (MODE == 0) {
            // InitPreconditionModifiedIncompCholesky2 (conjugategrad.cpp:66-97)
            const float px = wv[k], py = vy, pz = vz;
            const int cx = cv[k];
            const int ccy = j > 0 ? cy[k] : word_code(ey[k]);
            const int ccz = k > 0 ? cv[k - 1] : word_code(ez);
            const float A0 = a.A0f ? f[0] : (float)(cd & 7);
            float ev = A0;
            if (cd & kLowX) ev = ev - px * px;
            if (cd & kLowY) ev = ev - py * py;
            if (cd & kLowZ) ev = ev - pz * pz;
            const float k1 = (cd & kLowX) ? (float)(((cx & kHighY) ? 1 : 0) + ((cx & kHighZ) ? 1 : 0)) : 0.f;
            const float k2 = (cd & kLowY) ? (float)(((ccy & kHighX) ? 1 : 0) + ((ccy & kHighZ) ? 1 : 0)) : 0.f;
            const float k3 = (cd & kLowZ) ? (float)(((ccz & kHighX) ? 1 : 0) + ((ccz & kHighY) ? 1 : 0)) : 0.f;
            const float S3 = (k1 * (px * px) + k2 * (py * py)) + k3 * (pz * pz);
            ev = fmaf(-0.97f, S3, ev);  // e -= tau*(...): double in the reference, one rounding
            if (ev < 0.25f * A0) ev = A0;
            out = (cd & kCodeFluid) ? 1.f / sqrtf(ev) : 0.f;
            if (on) f[0] = out;
          } else if (MODE == 1) {
            // forward substitution (conjugategrad.cpp:141-148); neighbours
            // pass z*P, the product the reference forms for them
            const float p = f[AS];
            float t = f[0];
            if (cd & kLowX) t = t + wv[k];
            if (cd & kLowY) t = t + vy;
            if (cd & kLowZ) t = t + vz;
            const float zv = (cd & kCodeFluid) ? p * t : 0.f;
            if (on) f[0] = zv;
            out = zv * p;
          } else {
            // backward substitution (conjugategrad.cpp:150-159) in sweep
            // coordinates: the reference's upper neighbours are upwind
            const float p = f[2 * AS];
            float t = f[0];
            if (cd & kHighX) t = t + wv[k] * p;
            if (cd & kHighY) t = t + vy * p;
            if (cd & kHighZ) t = t + vz * p;
            const float zv = (cd & kCodeFluid) ? p * t : 0.f;
            if (on) {
              f[0] = zv;
              dsum += zv * f[AS];
            }
            out = zv;
          }
          wv[k] = out;
          cv[k] = cd;
        }
        if (MODE == 2) acc += (double)dsum;
        // (d) hand this step's face values to the downstream units: the last
        // layer of every lane (one row, contiguous over lanes) and lane 31's
        // layers (one row, contiguous over layers).  Words of inactive cells
        // are never read.
        if (hasZdn) {
          const int row = s - ZW + 1;
          if (row >= 0 && row < a.rows) st_relaxed_u64(dstZ + (long long)row * 32 + j, pack_word(wv[ZW - 1], cv[ZW - 1], ep16));
        }
        if (hasYdn && j == 31) {
          const int row = s - 31;
          if (row >= 0 && row < a.rows) {
#pragma unroll
            for (int k = 0; k < ZW; k += 2)
              st_relaxed_v2u64(dstY + (long long)row * ZW + k, pack_word(wv[k], cv[k], ep16),
                               pack_word(wv[k + 1], cv[k + 1], ep16));
          }
        }
        // (e) the layer whose chunk this step completed writes it back
        {
          const int k = (sj + 1) & 7;
          if (k < ZW && (act >> k & 1u)) {
            const int c = (sj - k) >> 3;
            const float4* src = reinterpret_cast<const float4*>(myF + k * kRC + (c & 1) * 8);
            float* dst = (MODE == 0 ? a.P : a.z) + line_base(k) + chunk_lo(c);
            reinterpret_cast<float4*>(dst)[0] = src[0];
            reinterpret_cast<float4*>(dst)[1] = src[1];
          }
        }
        // (f) loads for eight steps ahead: the face words of step s+8 and the
        // next chunk of the layer that starts a chunk at this step
        {
          const int sn = s + kPD;
          if (sn >= 0 && sn < a.rows) {
            if (hasZup && j < 16) cpa16(bufZ + u * 32 + 2 * j, srcZ + (long long)sn * 32 + 2 * j);
            if (j == 0 && hasYup) {
#pragma unroll
              for (int h = 0; h < ZW; h += 2) cpa16(bufY + u * ZW + h, srcY + (long long)sn * ZW + h);
            }
          }
          if (s == -kPD) {
#pragma unroll
            for (int k = 0; k < ZW; k++)
              if (lineMask >> k & 1u) load_chunk(k, 0);
          } else if (s >= 0) {
            const int k = sj & 7;
            const int x = sj - k;  // x % 8 == 0
            if (k < ZW && (lineMask >> k & 1u) && x >= 0 && (x >> 3) + 1 < nch) load_chunk(k, (x >> 3) + 1);
          }
          cpa_commit();
        }
      }
    }
    cpa_wait_all();
    if (MODE == 2) {
      double v = acc;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (j == 0) a.part[unit] = v;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- host side
template <int MODE, int ZW>
static size_t wave_smem() {
  constexpr int NF = MODE == 2 ? 3 : (MODE == 1 ? 2 : 1);
  return (size_t)NF * 32 * ZW * kRC * sizeof(float) + (size_t)32 * ZW * kRC * sizeof(code_t) +
         (size_t)kPD * (32 + ZW) * sizeof(unsigned long long);
}

bool mic_wave_supported(const Dims& d) { return d.is3d && d.nx % 8 == 0 && d.nx >= 16; }

void mic_wave_geometry(const Dims& d, int zw, int* nyb, int* nzb, int* rows) {
  *nyb = (d.ny + 31) / 32;
  *nzb = (d.nz + zw - 1) / zw;
  *rows = d.nx + 32;
}

size_t mic_wave_exchange_words(const Dims& d, int zw) {
  int nyb, nzb, rows;
  mic_wave_geometry(d, zw, &nyb, &nzb, &rows);
  return (size_t)nyb * nzb * rows * (32 + zw);
}

void mic_wave_order(int nyb, int nzb, int* order) {
  int n = 0;
  for (int L = 0; L <= nyb + nzb - 2; L++)
    for (int c = 0; c < nzb; c++) {
      const int b = L - c;
      if (b >= 0 && b < nyb) order[n++] = b + nyb * c;
    }
}

template <int ZW>
static cudaError_t wave_prepare_zw(int* ctasPerSm) {
  cudaError_t e = cudaFuncSetAttribute(k_mic_wave<0, ZW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wave_smem<0, ZW>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mic_wave<1, ZW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wave_smem<1, ZW>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mic_wave<2, ZW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wave_smem<2, ZW>());
  int n = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mic_wave<2, ZW>, 32, wave_smem<2, ZW>());
  *ctasPerSm = n > 0 ? n : 1;
  return e;
}

int mic_wave_prepare(int* ctasPerSm4, int* ctasPerSm8) {
  cudaError_t e = wave_prepare_zw<4>(ctasPerSm4);
  if (e == cudaSuccess) e = wave_prepare_zw<8>(ctasPerSm8);
  return e == cudaSuccess ? 0 : 1;
}

// mode: 0 factor, 1 forward, 2 backward (+beta), 3 backward for doInit (+sigma)
void launch_mic_wave(const PcgBuffers& b, const MicWavePlan& m, int mode, unsigned int epoch, long long spinLimit,
                     int ctas, cudaStream_t s) {
  WaveArgs a;
  a.d = b.d;
  a.code = b.code;
  a.A0f = b.A0f;
  a.P = b.P;
  a.r = b.residual;
  a.z = b.tmp;
  a.part = b.part;
  a.sc = b.sc;
  a.nyb = m.nyb;
  a.nzb = m.nzb;
  a.nunits = m.nunits;
  a.order = m.order;
  a.counter = m.counter;
  a.error = m.error;
  a.exY = m.exchange;
  a.exZ = m.exchange + (size_t)m.nyb * m.nzb * m.rows * m.zw;
  a.rows = m.rows;
  a.epoch = epoch;
  a.spinLimit = spinLimit;
  cudaMemsetAsync(m.counter, 0, sizeof(int), s);
  const int n = ctas < m.nunits ? ctas : m.nunits;
  count_launch();
  if (m.zw == 4) {
    if (mode == 0) k_mic_wave<0, 4><<<n, 32, wave_smem<0, 4>(), s>>>(a);
    else if (mode == 1) k_mic_wave<1, 4><<<n, 32, wave_smem<1, 4>(), s>>>(a);
    else k_mic_wave<2, 4><<<n, 32, wave_smem<2, 4>(), s>>>(a);
  } else {
    if (mode == 0) k_mic_wave<0, 8><<<n, 32, wave_smem<0, 8>(), s>>>(a);
    else if (mode == 1) k_mic_wave<1, 8><<<n, 32, wave_smem<1, 8>(), s>>>(a);
    else k_mic_wave<2, 8><<<n, 32, wave_smem<2, 8>(), s>>>(a);
  }
  if (mode >= 2) launch_mic_finish(b, m.nunits, mode == 3, s);
}

}  // namespace mgpu
