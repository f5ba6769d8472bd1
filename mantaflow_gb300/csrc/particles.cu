// Particle systems and the FLIP grid transfers (plugin/flip.cpp:549-673):
// mapPartsToMAC, mapMACToParts, flipVelocityUpdate, mapPartsToGrid(Vec3),
// mapGridToParts(Vec3).
//
// Layout: a BasicParticleSystem (particle.h:182-193) is kept as four device
// arrays -- x, y, z, flag -- and a ParticleDataImpl<Real|Vec3|int>
// (particle.h:306) as one or three; the host side keeps the reference's
// records (16-byte {Vec3 pos; int flag;}, 12-byte Vec3) and uploads and
// downloads transpose them on the GPU.
//
// Grid-to-particle transfers are one thread per particle.  Particle-to-grid
// transfers (the reference's single-threaded setInterpolated loops,
// knMapLinearVec3ToMACGrid and knMapLinear) add every particle's weighted
// value into the 8 faces or cells around it, in particle order, so a face's
// float sums depend on that order.  Here each face gathers instead of each
// particle scattering: the particles are sorted, stably, by the cell their
// interpolation stencil starts at (one LSD radix sort per MAC component),
// and a face merges the up to 8 sorted buckets that reach it by particle
// index, adding the same float products in the same order as the reference.
// The result is the reference's bit for bit, with no atomics.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <set>
#include <string>

#include "../../include/mantagpu.h"
#include "mg_batch.h"
#include "mg_common.cuh"
#include "mg_kernels.h"

using namespace mgpu;

namespace {

constexpr int kPDelete = 1 << 10;  // ParticleBase::PDELETE (particle.h:41)
constexpr float kVecEps = 1e-6f;   // VECTOR_EPSILON of the float build (util/vectorbase.h:52)
constexpr int kRsThreads = 256, kRsItems = 8, kRsTile = kRsThreads * kRsItems;

// ---------------------------------------------------------------- records
__global__ void k_parts_unpack(long long n, const float4* __restrict__ rec, float* x, float* y, float* z, int* flag) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float4 r = rec[i];
    x[i] = r.x;
    y[i] = r.y;
    z[i] = r.z;
    flag[i] = __float_as_int(r.w);
  }
}
__global__ void k_parts_pack(long long n, float4* rec, const float* __restrict__ x, const float* __restrict__ y,
                             const float* __restrict__ z, const int* __restrict__ flag) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    rec[i] = make_float4(x[i], y[i], z[i], __int_as_float(flag[i]));
}
// Vec3 records <-> three planes (dir 0: unpack, 1: pack)
__global__ void k_vec_transpose(long long n, float* rec, float* a, float* b, float* c, int dir) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (dir == 0) {
      a[i] = rec[3 * i];
      b[i] = rec[3 * i + 1];
      c[i] = rec[3 * i + 2];
    } else {
      rec[3 * i] = a[i];
      rec[3 * i + 1] = b[i];
      rec[3 * i + 2] = c[i];
    }
  }
}

// -------------------------------------------------------- stencil buckets
// The first cell of a particle's interpolation stencil: BUILD_INDEX
// (util/interpol.h:50-66) for cell-centred grids (comp -1), BUILD_INDEX_SHIFT
// (:116-130) with component comp shifted for MAC faces.  In 2D the z index
// is 0 for every particle of the slab z in [0,1) (the reference's 2D
// particles sit at z = 0.5); it is taken as 0 for any other z as well.
// Particles that are deleted, or whose type matches exclude, get the key
// ncells, past every bucket.
struct PartView {
  const float* x;
  const float* y;
  const float* z;
  const int* flag;
  const int* ptype;  // may be null
  int exclude;
};

__device__ __forceinline__ bool part_skip(const PartView& p, long long i) {
  return (p.flag[i] & kPDelete) != 0 || (p.ptype && (p.ptype[i] & p.exclude) != 0);
}

__global__ void k_stencil_keys(Dims d, PartView p, long long n, int comp, unsigned* keys, unsigned* vals) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned key = (unsigned)d.n;
  if (!part_skip(p, i)) {
    const float px = p.x[i], py = p.y[i], pz = p.z[i];
    const Wts w = build_index<false>(d, px, py, pz);
    int xi = w.xi, yi = w.yi, zi = w.zi;
    if (comp >= 0) {
      const Wts s = build_index<true>(d, px, py, pz);
      if (comp == 0) xi = s.xi;
      if (comp == 1) yi = s.yi;
      if (comp == 2) zi = s.zi;
    }
    if (!d.is3d) zi = 0;
    key = (unsigned)(xi + d.nx * (yi + d.ny * zi));
  }
  keys[i] = key;
  vals[i] = (unsigned)i;
}

// -------------------------------------------------------------- radix sort
// One stable pass of an LSD radix sort on 8-bit digits.  A CTA owns a tile
// of 2048 consecutive elements; counts are stored digit-major (digit x
// tiles), so their exclusive scan gives every (digit, tile) its first output
// slot in digit order, then tile order.
__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const unsigned* __restrict__ keys, long long n, int shift,
                                                        unsigned* hist, int tiles) {
  __shared__ unsigned h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kRsTile;
  for (int r = 0; r < kRsItems; r++) {
    const long long i = base + r * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// Within a tile, elements are placed in index order: rounds of 256 in turn,
// warps in turn within a round, lanes in turn within a warp (a lane's rank
// among the lanes holding its digit comes from __match_any_sync).
__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const unsigned* __restrict__ kin,
                                                           const unsigned* __restrict__ vin, unsigned* kout,
                                                           unsigned* vout, long long n, int shift,
                                                           const unsigned* __restrict__ offs, int tiles) {
  __shared__ unsigned run[256];
  __shared__ unsigned wc[kRsThreads / 32][256];
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  run[t] = offs[(size_t)t * tiles + blockIdx.x];
  const long long base = (long long)blockIdx.x * kRsTile;
  for (int r = 0; r < kRsItems; r++) {
#pragma unroll
    for (int q = 0; q < kRsThreads / 32; q++) wc[q][t] = 0;
    __syncthreads();
    const long long i = base + r * kRsThreads + t;
    const bool ok = i < n;
    unsigned key = 0, val = 0, dig = 0, rank = 0;
    const unsigned act = __ballot_sync(0xffffffffu, ok);
    if (ok) {
      key = kin[i];
      val = vin[i];
      dig = (key >> shift) & 255u;
      const unsigned peers = __match_any_sync(act, dig);
      rank = __popc(peers & ((1u << lane) - 1u));
      if (rank == 0) wc[w][dig] = __popc(peers);
    }
    __syncthreads();
    // thread t owns digit t: exclusive prefix over the warps, after the
    // slots taken by earlier rounds
    unsigned acc = run[t];
#pragma unroll
    for (int q = 0; q < kRsThreads / 32; q++) {
      const unsigned c = wc[q][t];
      wc[q][t] = acc;
      acc += c;
    }
    run[t] = acc;
    __syncthreads();
    if (ok) {
      const unsigned dst = wc[w][dig] + rank;
      kout[dst] = key;
      vout[dst] = val;
    }
    __syncthreads();
  }
}

// exclusive scan of n unsigned values in place: per-block scans of 2048,
// one CTA scanning the block totals, then the block offsets added
__device__ __forceinline__ unsigned block_excl_scan(unsigned v, unsigned* sh, unsigned* total) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    unsigned s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < (int)(blockDim.x >> 5)) sh[lane] = s;
  }
  __syncthreads();
  const unsigned before = (w > 0 ? sh[w - 1] : 0u) + x - v;
  *total = sh[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(kRsThreads) k_scan_tiles(unsigned* a, long long n, unsigned* sums) {
  __shared__ unsigned sh[32];
  const long long base = (long long)blockIdx.x * kRsTile + (long long)threadIdx.x * kRsItems;
  unsigned v[kRsItems], tot = 0;
#pragma unroll
  for (int q = 0; q < kRsItems; q++) {
    v[q] = base + q < n ? a[base + q] : 0u;
    tot += v[q];
  }
  unsigned blockTotal;
  unsigned run = block_excl_scan(tot, sh, &blockTotal);
#pragma unroll
  for (int q = 0; q < kRsItems; q++) {
    if (base + q < n) a[base + q] = run;
    run += v[q];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = blockTotal;
}

__global__ void __launch_bounds__(kRsThreads) k_scan_sums(unsigned* sums, int m) {
  __shared__ unsigned sh[32];
  unsigned carry = 0;
  for (int b0 = 0; b0 < m; b0 += kRsThreads) {
    const int i = b0 + threadIdx.x;
    const unsigned v = i < m ? sums[i] : 0u;
    unsigned tot;
    const unsigned ex = block_excl_scan(v, sh, &tot);
    if (i < m) sums[i] = carry + ex;
    carry += tot;
  }
}

__global__ void k_scan_add(unsigned* a, long long n, const unsigned* __restrict__ sums) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) a[i] += sums[i / kRsTile];
}

// starts[b] = first position of key >= b in the sorted keys (b = 0..ncells)
__global__ void k_bucket_starts(const unsigned* __restrict__ keys, long long n, long long ncells, unsigned* starts) {
  const long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (b > ncells) return;
  long long lo = 0, hi = n;
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if ((long long)keys[mid] < b)
      lo = mid + 1;
    else
      hi = mid;
  }
  starts[b] = (unsigned)lo;
}

}  // namespace

namespace {

// ----------------------------------------------------- particle -> grid
// Positions and values copied into bucket order after a sort, so that the
// faces' merges read them in sequence instead of gathering each particle
// from its own index (every particle is read by up to 8 faces per sort).
struct SortedParts {
  const float* x;
  const float* y;
  const float* z;
  const float* v[3];
};
__global__ void k_sorted_copy(long long n, const unsigned* __restrict__ sorted, PartView p, const float* __restrict__ v0,
                              const float* __restrict__ v1, const float* __restrict__ v2, float* sx, float* sy,
                              float* sz, float* s0, float* s1, float* s2) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned k = sorted[i];
  sx[i] = p.x[k];
  sy[i] = p.y[k];
  sz[i] = p.z[k];
  s0[i] = __ldg(v0 + k);
  if (v1) {
    s1[i] = __ldg(v1 + k);
    s2[i] = __ldg(v2 + k);
  }
}

// The weights setInterpol / setInterpolMAC give the stencil corner (dx, dy,
// dz) of a particle: T[dy] * (S[dx] * F[dz]) (util/interpol.h:93-112,
// 159-195), with the axis of MAC component comp shifted.
struct CornerW {
  float S[2], T[2], F[2];
};
// One axis of BUILD_INDEX / BUILD_INDEX_SHIFT: the weights of the lower and
// upper sample for the coordinate q (already shifted by -0.5 or not), with
// the border clamps (the upper one only where the axis has more than one
// cell).  The same operations as build_index, one axis at a time, so a
// component's weights take three axes instead of both full variants.
__device__ __forceinline__ void axis_weights(float q, int n, bool clampHigh, float* w) {
  const int i = (int)q;
  float w1 = q - (float)i, w0 = 1.f - w1;
  if (q < 0.f) {
    w0 = 1.f;
    w1 = 0.f;
  }
  if (clampHigh && i >= n - 1) {
    w0 = 0.f;
    w1 = 1.f;
  }
  w[0] = w0;
  w[1] = w1;
}
__device__ __forceinline__ CornerW corner_weights(const Dims& d, float px, float py, float pz, int comp) {
  CornerW c;
  axis_weights(comp == 0 ? px : px - 0.5f, d.nx, true, c.S);
  axis_weights(comp == 1 ? py : py - 0.5f, d.ny, true, c.T);
  axis_weights(comp == 2 ? pz : pz - 0.5f, d.nz, d.nz > 1, c.F);
  return c;
}

// One thread per face (comp >= 0, MAC component comp) or cell (comp -1):
// merge the sorted buckets of the up to 8 stencil origins that reach it by
// particle index and add each particle's weight and weighted value in that
// order.  In 2D the z stride is 0, so the reference adds both z layers of a
// particle's stencil to the same face: the z = 1 layer first, except for the
// MAC z component, which adds its z = 0 layer first.
// Then, for MAC faces (mapPartsToMAC, flip.cpp:585-594): weights below
// VECTOR_EPSILON are stomped to 0 and the sum divided by a non-zero weight
// (safeDivide, general.h:150); vel, velOld and the optional weight grid are
// written.  For cells (mapPartsToGrid, knSafeDivReal, flip.cpp:549-557):
// weights below VECTOR_EPSILON give 0, others divide.
template <int kComps>
__global__ void __launch_bounds__(256) k_p2g_gather(Dims d, int comp, SortedParts sp,
                                                    const unsigned* __restrict__ sorted,
                                                    const unsigned* __restrict__ starts, float* o0, float* o1,
                                                    float* o2, float* old, float* wout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  constexpr unsigned kNone = 0xffffffffu;
  unsigned cur[8], end[8], head[8];
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int bi = i - (q & 1), bj = j - ((q >> 1) & 1), bk = k - (q >> 2);
    const bool ok = bi >= 0 && bi <= d.nx - 2 && bj >= 0 && bj <= d.ny - 2 &&
                    (d.is3d ? (bk >= 0 && bk <= d.nz - 2) : (q >> 2) == 0);
    cur[q] = end[q] = 0;
    if (ok) {
      const long long key = bi + (long long)d.nx * (bj + (long long)d.ny * (d.is3d ? bk : 0));
      cur[q] = starts[key];
      end[q] = starts[key + 1];
    }
    head[q] = cur[q] < end[q] ? sorted[cur[q]] : kNone;
  }
  const bool zFirst0 = comp == 2;  // 2D: which z layer the reference adds first
  float sum = 0.f, r0 = 0.f, r1 = 0.f, r2 = 0.f;
  for (;;) {
    unsigned best = head[0];
    int bq = 0;
#pragma unroll
    for (int q = 1; q < 8; q++)
      if (head[q] < best) {
        best = head[q];
        bq = q;
      }
    if (best == kNone) break;
    unsigned at = cur[0];  // the particle's slot in bucket order
#pragma unroll
    for (int q = 1; q < 8; q++)
      if (q == bq) at = cur[q];
    const CornerW c = corner_weights(d, __ldg(sp.x + at), __ldg(sp.y + at), __ldg(sp.z + at), comp);
    const int dx = bq & 1, dy = (bq >> 1) & 1, dz = bq >> 2;
    const float a0 = __ldg(sp.v[0] + at);
    const float a1 = kComps == 3 ? __ldg(sp.v[1] + at) : 0.f;
    const float a2 = kComps == 3 ? __ldg(sp.v[2] + at) : 0.f;
    if (d.is3d) {
      const float w = c.T[dy] * (c.S[dx] * c.F[dz]);
      sum += w;
      r0 += w * a0;
      if (kComps == 3) {
        r1 += w * a1;
        r2 += w * a2;
      }
    } else {
#pragma unroll
      for (int layer = 0; layer < 2; layer++) {
        const int lz = zFirst0 ? layer : 1 - layer;
        const float w = c.T[dy] * (c.S[dx] * c.F[lz]);
        sum += w;
        r0 += w * a0;
        if (kComps == 3) {
          r1 += w * a1;
          r2 += w * a2;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 8; q++)
      if (q == bq) {
        cur[q]++;
        head[q] = cur[q] < end[q] ? sorted[cur[q]] : kNone;
      }
  }
  const long long o = ix(d, i, j, k);
  if (comp >= 0) {
    const float ws = sum < kVecEps ? 0.f : sum;
    const float v = ws != 0.f ? r0 / ws : r0;
    o0[o] = v;
    old[o] = v;
    if (wout) wout[o] = ws;
  } else if (sum < kVecEps) {
    o0[o] = 0.f;
    if (kComps == 3) {
      o1[o] = 0.f;
      o2[o] = 0.f;
    }
  } else {
    o0[o] = r0 / sum;
    if (kComps == 3) {
      o1[o] = r1 / sum;
      o2[o] = r2 / sum;
    }
  }
}

// ----------------------------------------------------- grid -> particle
// mapMACToParts (knMapLinearMACGridToVec3_PIC, flip.cpp:643-650) and, with
// old, flipVelocityUpdate (knMapLinearMACGridToVec3_FLIP, :659-668):
//   pvel = flipRatio * (pvel + (v - vOld)) + (1.0 - flipRatio) * v
// where the second product is formed in double and rounded to float.
__global__ void k_mac_to_parts(Dims d, PartView p, long long n, CMac vel, CMac old, float flipRatio, float* pu,
                               float* pv, float* pw) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n || part_skip(p, i)) return;
  const float x = p.x[i], y = p.y[i], z = p.z[i];
  const V3 v = interp_mac<true>(d, vel, x, y, z);
  if (!old.u) {
    pu[i] = v.x;
    pv[i] = v.y;
    pw[i] = v.z;
    return;
  }
  const V3 o = interp_mac<true>(d, old, x, y, z);
  const float dlx = v.x - o.x, dly = v.y - o.y, dlz = v.z - o.z;
  const double keep = 1.0 - (double)flipRatio;
  pu[i] = flipRatio * (pu[i] + dlx) + (float)(keep * (double)v.x);
  pv[i] = flipRatio * (pv[i] + dly) + (float)(keep * (double)v.y);
  pw[i] = flipRatio * (pw[i] + dlz) + (float)(keep * (double)v.z);
}

// mapGridToParts(Vec3) (knMapFromGrid, flip.cpp:625-631): every active
// particle, interpol<T> per component
__global__ void k_grid_to_parts(Dims d, PartView p, long long n, const float* __restrict__ g0,
                                const float* __restrict__ g1, const float* __restrict__ g2, float* t0, float* t1,
                                float* t2) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n || (p.flag[i] & kPDelete) != 0) return;
  const float x = p.x[i], y = p.y[i], z = p.z[i];
  t0[i] = interp(d, g0, x, y, z);
  if (g1) {
    t1[i] = interp(d, g1, x, y, z);
    t2[i] = interp(d, g2, x, y, z);
  }
}

}  // namespace

// ================================================================ host side
struct mg_particles_s {
  mg_solver s;
  Dims d;
  cudaStream_t st;
  long long cap = 0, n = 0;
  float *x = nullptr, *y = nullptr, *z = nullptr;
  int* flag = nullptr;
  // sorting scratch: keys and particle indices (ping-pong), per-tile digit
  // counts and their scan's block totals, bucket starts (ncells + 1)
  unsigned *keys[2] = {nullptr, nullptr}, *vals[2] = {nullptr, nullptr};
  unsigned *hist = nullptr, *sums = nullptr, *starts = nullptr;
  float* sorted[6] = {};  // positions and up to 3 values in bucket order
  void* stage = nullptr;  // 16 bytes per particle for record transfers
};

struct mg_pdata_s {
  mg_particles p;
  int kind;  // MG_REAL, MG_VEC3, MG_INT
  float* c[3] = {nullptr, nullptr, nullptr};
};

namespace {

std::mutex g_partMu;
std::set<mg_particles> g_parts;
std::set<mg_pdata> g_pdata;

bool valid_parts(mg_particles p) {
  std::lock_guard<std::mutex> lk(g_partMu);
  return p && g_parts.count(p);
}
bool valid_pdata(mg_pdata d) {
  std::lock_guard<std::mutex> lk(g_partMu);
  return d && g_pdata.count(d) && g_parts.count(d->p);
}

void free_parts(mg_particles p) {
  cudaStreamSynchronize(p->st);
  void* bufs[] = {p->x, p->y, p->z, p->flag, p->keys[0], p->keys[1], p->vals[0], p->vals[1], p->hist, p->sums,
                  p->starts, p->stage};
  for (void* b : bufs)
    if (b) cudaFree(b);
  for (float* b : p->sorted)
    if (b) cudaFree(b);
}

int tiles_of(long long n) { return (int)((n + kRsTile - 1) / kRsTile); }

int blocks_of(long long n, int b = 256) { return (int)std::max<long long>(1, (n + b - 1) / b); }

int launch_status(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(MG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return MG_OK;
}

// exclusive scan of m counts in place
void scan_counts(mg_particles p, unsigned* a, long long m) {
  const int blocks = (int)((m + kRsTile - 1) / kRsTile);
  count_launch();
  k_scan_tiles<<<blocks, kRsThreads, 0, p->st>>>(a, m, p->sums);
  count_launch();
  k_scan_sums<<<1, kRsThreads, 0, p->st>>>(p->sums, blocks);
  count_launch();
  k_scan_add<<<blocks_of(m), 256, 0, p->st>>>(a, m, p->sums);
}

// sort the live particles by the first cell of their stencil (comp -1: cell
// centred, 0..2: MAC component); returns the particle indices in bucket order
// and fills p->starts
const unsigned* sort_stencil(mg_particles p, int comp, const PartView& v) {
  const long long n = p->n, ncells = p->d.n;
  if (n == 0) {
    cudaMemsetAsync(p->starts, 0, (size_t)(ncells + 1) * sizeof(unsigned), p->st);
    return p->vals[0];
  }
  count_launch();
  k_stencil_keys<<<blocks_of(n), 256, 0, p->st>>>(p->d, v, n, comp, p->keys[0], p->vals[0]);
  int bits = 0;
  while (bits < 32 && (ncells >> bits) != 0) bits++;
  const int passes = (bits + 7) / 8;
  const int tiles = tiles_of(n);
  int a = 0;
  for (int pass = 0; pass < passes; pass++) {
    const int shift = 8 * pass;
    count_launch();
    k_rs_hist<<<tiles, kRsThreads, 0, p->st>>>(p->keys[a], n, shift, p->hist, tiles);
    scan_counts(p, p->hist, 256LL * tiles);
    count_launch();
    k_rs_scatter<<<tiles, kRsThreads, 0, p->st>>>(p->keys[a], p->vals[a], p->keys[1 - a], p->vals[1 - a], n, shift,
                                                   p->hist, tiles);
    a = 1 - a;
  }
  count_launch();
  k_bucket_starts<<<blocks_of(ncells + 1), 256, 0, p->st>>>(p->keys[a], n, ncells, p->starts);
  return p->vals[a];
}

// the live particles' positions and values (1 or 3 planes) in bucket order
SortedParts sorted_copy(mg_particles p, const unsigned* sorted, const PartView& v, const float* v0, const float* v1,
                        const float* v2) {
  const long long n = p->n;
  if (n > 0) {
    count_launch();
    k_sorted_copy<<<blocks_of(n), 256, 0, p->st>>>(n, sorted, v, v0, v1, v2, p->sorted[0], p->sorted[1],
                                                    p->sorted[2], p->sorted[3], p->sorted[4], p->sorted[5]);
  }
  SortedParts sp{p->sorted[0], p->sorted[1], p->sorted[2], {p->sorted[3], p->sorted[4], p->sorted[5]}};
  return sp;
}

PartView view_of(mg_particles p, mg_pdata ptype, int exclude) {
  PartView v{p->x, p->y, p->z, p->flag, ptype ? (const int*)ptype->c[0] : nullptr, exclude};
  return v;
}

// a grid of the particle system's solver, of one of the given kinds
int grid_of(mg_particles p, mg_grid g, unsigned kindMask, const char* what, float** data, int* kind) {
  int nx, ny, nz, k;
  if (mg_grid_get_info(g, &nx, &ny, &nz, &k)) return set_error(MG_ERR_ARG, std::string(what) + ": invalid grid");
  if (!((kindMask >> k) & 1u)) return set_error(MG_ERR_ARG, std::string(what) + ": wrong grid type");
  void* dp = nullptr;
  void* sp = nullptr;
  mg_grid_device(g, &dp, &sp);
  if ((cudaStream_t)sp != p->st || nx != p->d.nx || ny != p->d.ny || nz != p->d.nz)
    return set_error(MG_ERR_ARG, std::string(what) + ": grid and particles belong to different solvers");
  *data = (float*)dp;
  if (kind) *kind = k;
  return MG_OK;
}

int pdata_of(mg_particles p, mg_pdata d, int kind, const char* what) {
  if (!valid_pdata(d)) return set_error(MG_ERR_ARG, std::string(what) + ": invalid particle data");
  if (d->p != p) return set_error(MG_ERR_ARG, std::string(what) + ": particle data of another particle system");
  if (d->kind != kind) return set_error(MG_ERR_ARG, std::string(what) + ": wrong particle data type");
  return MG_OK;
}

}  // namespace

extern "C" int mg_grid_get_info(mg_grid g, int* nx, int* ny, int* nz, int* kind);
extern "C" int mg_grid_device(mg_grid g, void** data, void** stream);

extern "C" int mg_particles_create(mg_solver s, long long capacity, mg_particles* out) {
  if (!out) return set_error(MG_ERR_ARG, "mg_particles_create: null out");
  if (capacity < 0 || capacity > (1LL << 30))
    return set_error(MG_ERR_ARG, "mg_particles_create: capacity must be in [0, 2^30]");
  auto p = new mg_particles_s();
  if (solver_info(s, &p->d, &p->st)) {
    delete p;
    return MG_ERR_ARG;
  }
  p->s = s;
  p->cap = capacity;
  const long long c = std::max<long long>(capacity, 1);
  const long long tiles = tiles_of(c);
  const long long histN = 256 * tiles;
  bool ok = cudaMalloc(&p->x, c * 4) == cudaSuccess && cudaMalloc(&p->y, c * 4) == cudaSuccess &&
            cudaMalloc(&p->z, c * 4) == cudaSuccess && cudaMalloc(&p->flag, c * 4) == cudaSuccess &&
            cudaMalloc(&p->keys[0], c * 4) == cudaSuccess && cudaMalloc(&p->keys[1], c * 4) == cudaSuccess &&
            cudaMalloc(&p->vals[0], c * 4) == cudaSuccess && cudaMalloc(&p->vals[1], c * 4) == cudaSuccess &&
            cudaMalloc(&p->hist, histN * 4) == cudaSuccess &&
            cudaMalloc(&p->sums, ((histN + kRsTile - 1) / kRsTile) * 4) == cudaSuccess &&
            cudaMalloc(&p->starts, (p->d.n + 1) * 4) == cudaSuccess && cudaMalloc(&p->stage, c * 16) == cudaSuccess;
  for (int q = 0; q < 6 && ok; q++) ok = cudaMalloc(&p->sorted[q], c * 4) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    free_parts(p);
    delete p;
    return set_error(MG_ERR_NOMEM, "BasicParticleSystem: out of device memory");
  }
  {
    std::lock_guard<std::mutex> lk(g_partMu);
    g_parts.insert(p);
  }
  *out = p;
  return MG_OK;
}

extern "C" int mg_particles_destroy(mg_particles p) {
  if (!p) return MG_OK;
  {
    std::lock_guard<std::mutex> lk(g_partMu);
    if (!g_parts.count(p)) return set_error(MG_ERR_ARG, "mg_particles_destroy: invalid particle system");
    g_parts.erase(p);
    cudaStreamSynchronize(p->st);
    // its particle data goes with it
    for (auto it = g_pdata.begin(); it != g_pdata.end();) {
      if ((*it)->p != p) {
        ++it;
        continue;
      }
      for (float* b : (*it)->c)
        if (b) cudaFree(b);
      delete *it;
      it = g_pdata.erase(it);
    }
  }
  free_parts(p);
  delete p;
  return MG_OK;
}

extern "C" int mg_particles_upload(mg_particles p, const void* host, long long count) {
  if (!valid_parts(p)) return set_error(MG_ERR_ARG, "mg_particles_upload: invalid particle system");
  if (count < 0 || count > p->cap) return set_error(MG_ERR_ARG, "mg_particles_upload: count exceeds the capacity");
  if (count > 0 && !host) return set_error(MG_ERR_ARG, "mg_particles_upload: null host buffer");
  if (count > 0) {
    if (cudaMemcpyAsync(p->stage, host, (size_t)count * 16, cudaMemcpyHostToDevice, p->st) != cudaSuccess)
      return launch_status("mg_particles_upload");
    count_launch();
    k_parts_unpack<<<blocks_of(count), 256, 0, p->st>>>(count, (const float4*)p->stage, p->x, p->y, p->z, p->flag);
  }
  p->n = count;
  return launch_status("mg_particles_upload");
}

extern "C" int mg_particles_download(mg_particles p, void* host, long long count) {
  if (!valid_parts(p)) return set_error(MG_ERR_ARG, "mg_particles_download: invalid particle system");
  if (count != p->n) return set_error(MG_ERR_ARG, "mg_particles_download: count must equal the particle count");
  if (count == 0) return MG_OK;
  if (!host) return set_error(MG_ERR_ARG, "mg_particles_download: null host buffer");
  count_launch();
  k_parts_pack<<<blocks_of(count), 256, 0, p->st>>>(count, (float4*)p->stage, p->x, p->y, p->z, p->flag);
  if (cudaMemcpyAsync(host, p->stage, (size_t)count * 16, cudaMemcpyDeviceToHost, p->st) != cudaSuccess ||
      cudaStreamSynchronize(p->st) != cudaSuccess)
    return launch_status("mg_particles_download");
  return launch_status("mg_particles_download");
}

extern "C" int mg_particles_size(mg_particles p, long long* count) {
  if (!valid_parts(p) || !count) return set_error(MG_ERR_ARG, "mg_particles_size: invalid argument");
  *count = p->n;
  return MG_OK;
}

extern "C" int mg_pdata_create(mg_particles p, int kind, mg_pdata* out) {
  if (!out) return set_error(MG_ERR_ARG, "mg_pdata_create: null out");
  if (!valid_parts(p)) return set_error(MG_ERR_ARG, "mg_pdata_create: invalid particle system");
  if (kind != MG_REAL && kind != MG_VEC3 && kind != MG_INT)
    return set_error(MG_ERR_ARG, "mg_pdata_create: kind must be MG_REAL, MG_VEC3 or MG_INT");
  auto d = new mg_pdata_s();
  d->p = p;
  d->kind = kind;
  const long long c = std::max<long long>(p->cap, 1);
  const int comps = kind == MG_VEC3 ? 3 : 1;
  bool ok = true;
  for (int q = 0; q < comps && ok; q++) ok = cudaMalloc(&d->c[q], c * 4) == cudaSuccess;
  for (int q = 0; q < comps && ok; q++) ok = cudaMemsetAsync(d->c[q], 0, c * 4, p->st) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    for (float* b : d->c)
      if (b) cudaFree(b);
    delete d;
    return set_error(MG_ERR_NOMEM, "ParticleDataImpl: out of device memory");
  }
  {
    std::lock_guard<std::mutex> lk(g_partMu);
    g_pdata.insert(d);
  }
  *out = d;
  return MG_OK;
}

extern "C" int mg_pdata_destroy(mg_pdata d) {
  if (!d) return MG_OK;
  mg_particles p;
  {
    std::lock_guard<std::mutex> lk(g_partMu);
    if (!g_pdata.count(d)) return set_error(MG_ERR_ARG, "mg_pdata_destroy: invalid particle data");
    g_pdata.erase(d);
    p = g_parts.count(d->p) ? d->p : nullptr;
  }
  if (p) cudaStreamSynchronize(p->st);
  for (float* b : d->c)
    if (b) cudaFree(b);
  delete d;
  return MG_OK;
}

static int pdata_transfer(mg_pdata d, void* host, long long count, bool up) {
  const char* what = up ? "mg_pdata_upload" : "mg_pdata_download";
  if (!valid_pdata(d)) return set_error(MG_ERR_ARG, std::string(what) + ": invalid particle data");
  mg_particles p = d->p;
  if (count != p->n) return set_error(MG_ERR_ARG, std::string(what) + ": count must equal the particle count");
  if (count == 0) return MG_OK;
  if (!host) return set_error(MG_ERR_ARG, std::string(what) + ": null host buffer");
  if (d->kind != MG_VEC3) {
    const cudaError_t e = up ? cudaMemcpyAsync(d->c[0], host, (size_t)count * 4, cudaMemcpyHostToDevice, p->st)
                             : cudaMemcpyAsync(host, d->c[0], (size_t)count * 4, cudaMemcpyDeviceToHost, p->st);
    if (e != cudaSuccess) return launch_status(what);
  } else if (up) {
    if (cudaMemcpyAsync(p->stage, host, (size_t)count * 12, cudaMemcpyHostToDevice, p->st) != cudaSuccess)
      return launch_status(what);
    count_launch();
    k_vec_transpose<<<blocks_of(count), 256, 0, p->st>>>(count, (float*)p->stage, d->c[0], d->c[1], d->c[2], 0);
  } else {
    count_launch();
    k_vec_transpose<<<blocks_of(count), 256, 0, p->st>>>(count, (float*)p->stage, d->c[0], d->c[1], d->c[2], 1);
    if (cudaMemcpyAsync(host, p->stage, (size_t)count * 12, cudaMemcpyDeviceToHost, p->st) != cudaSuccess)
      return launch_status(what);
  }
  if (!up && cudaStreamSynchronize(p->st) != cudaSuccess) return launch_status(what);
  return launch_status(what);
}

extern "C" int mg_pdata_upload(mg_pdata d, const void* host, long long count) {
  return pdata_transfer(d, const_cast<void*>(host), count, true);
}
extern "C" int mg_pdata_download(mg_pdata d, void* host, long long count) {
  return pdata_transfer(d, host, count, false);
}

// ----------------------------------------------------------- the transfers
extern "C" int mg_map_parts_to_mac(mg_grid flags, mg_grid vel, mg_grid velOld, mg_particles parts, mg_pdata partVel,
                                   mg_grid weight, mg_pdata ptype, int exclude) {
  const char* what = "mapPartsToMAC";
  if (!valid_parts(parts)) return set_error(MG_ERR_ARG, "mapPartsToMAC: invalid particle system");
  float *f, *v, *vo, *w = nullptr;
  if (grid_of(parts, flags, 1u << MG_FLAGS, what, &f, nullptr) || grid_of(parts, vel, 1u << MG_MAC, what, &v, nullptr) ||
      grid_of(parts, velOld, 1u << MG_MAC, what, &vo, nullptr))
    return MG_ERR_ARG;
  if (weight && grid_of(parts, weight, (1u << MG_VEC3) | (1u << MG_MAC), what, &w, nullptr)) return MG_ERR_ARG;
  if (pdata_of(parts, partVel, MG_VEC3, what)) return MG_ERR_ARG;
  if (ptype && pdata_of(parts, ptype, MG_INT, what)) return MG_ERR_ARG;
  const Dims& d = parts->d;
  const PartView pv = view_of(parts, ptype, exclude);
  const dim3 b(32, 8, 1);
  for (int c = 0; c < 3; c++) {
    const unsigned* sorted = sort_stencil(parts, c, pv);
    const SortedParts sp = sorted_copy(parts, sorted, pv, partVel->c[c], nullptr, nullptr);
    count_launch();
    k_p2g_gather<1><<<grid3(d, b), b, 0, parts->st>>>(d, c, sp, sorted, parts->starts, v + c * d.n, nullptr, nullptr,
                                                      vo + c * d.n, w ? w + c * d.n : nullptr);
  }
  return launch_status(what);
}

extern "C" int mg_map_parts_to_grid(mg_grid flags, mg_grid target, mg_particles parts, mg_pdata source) {
  const char* what = "mapPartsToGrid";
  if (!valid_parts(parts)) return set_error(MG_ERR_ARG, "mapPartsToGrid: invalid particle system");
  float *f, *t;
  int kind = 0;
  if (grid_of(parts, flags, 1u << MG_FLAGS, what, &f, nullptr) ||
      grid_of(parts, target, (1u << MG_REAL) | (1u << MG_LEVELSET) | (1u << MG_VEC3) | (1u << MG_MAC), what, &t,
              &kind))
    return MG_ERR_ARG;
  const bool vec = kind == MG_VEC3 || kind == MG_MAC;
  if (pdata_of(parts, source, vec ? MG_VEC3 : MG_REAL, what)) return MG_ERR_ARG;
  const Dims& d = parts->d;
  const PartView pv = view_of(parts, nullptr, 0);
  const unsigned* sorted = sort_stencil(parts, -1, pv);
  const SortedParts sp = sorted_copy(parts, sorted, pv, source->c[0], vec ? source->c[1] : nullptr,
                                     vec ? source->c[2] : nullptr);
  const dim3 b(32, 8, 1);
  count_launch();
  if (vec)
    k_p2g_gather<3><<<grid3(d, b), b, 0, parts->st>>>(d, -1, sp, sorted, parts->starts, t, t + d.n, t + 2 * d.n,
                                                      nullptr, nullptr);
  else
    k_p2g_gather<1><<<grid3(d, b), b, 0, parts->st>>>(d, -1, sp, sorted, parts->starts, t, nullptr, nullptr, nullptr,
                                                      nullptr);
  return launch_status(what);
}

static int mac_to_parts(const char* what, mg_grid flags, mg_grid vel, mg_grid velOld, mg_particles parts,
                        mg_pdata partVel, float flipRatio, mg_pdata ptype, int exclude) {
  if (!valid_parts(parts)) return set_error(MG_ERR_ARG, std::string(what) + ": invalid particle system");
  float *f, *v, *vo = nullptr;
  if (grid_of(parts, flags, 1u << MG_FLAGS, what, &f, nullptr) || grid_of(parts, vel, 1u << MG_MAC, what, &v, nullptr))
    return MG_ERR_ARG;
  if (velOld && grid_of(parts, velOld, 1u << MG_MAC, what, &vo, nullptr)) return MG_ERR_ARG;
  if (pdata_of(parts, partVel, MG_VEC3, what)) return MG_ERR_ARG;
  if (ptype && pdata_of(parts, ptype, MG_INT, what)) return MG_ERR_ARG;
  const Dims& d = parts->d;
  if (parts->n == 0) return MG_OK;
  const CMac cv{v, v + d.n, v + 2 * d.n};
  const CMac co = vo ? CMac{vo, vo + d.n, vo + 2 * d.n} : CMac{nullptr, nullptr, nullptr};
  count_launch();
  k_mac_to_parts<<<blocks_of(parts->n), 256, 0, parts->st>>>(d, view_of(parts, ptype, exclude), parts->n, cv, co,
                                                              flipRatio, partVel->c[0], partVel->c[1], partVel->c[2]);
  return launch_status(what);
}

extern "C" int mg_map_mac_to_parts(mg_grid flags, mg_grid vel, mg_particles parts, mg_pdata partVel, mg_pdata ptype,
                                   int exclude) {
  return mac_to_parts("mapMACToParts", flags, vel, nullptr, parts, partVel, 0.f, ptype, exclude);
}

extern "C" int mg_flip_velocity_update(mg_grid flags, mg_grid vel, mg_grid velOld, mg_particles parts,
                                       mg_pdata partVel, float flipRatio, mg_pdata ptype, int exclude) {
  if (!velOld) return set_error(MG_ERR_ARG, "flipVelocityUpdate: null velOld");
  return mac_to_parts("flipVelocityUpdate", flags, vel, velOld, parts, partVel, flipRatio, ptype, exclude);
}

extern "C" int mg_map_grid_to_parts(mg_grid source, mg_particles parts, mg_pdata target) {
  const char* what = "mapGridToParts";
  if (!valid_parts(parts)) return set_error(MG_ERR_ARG, "mapGridToParts: invalid particle system");
  float* g;
  int kind = 0;
  if (grid_of(parts, source, (1u << MG_REAL) | (1u << MG_LEVELSET) | (1u << MG_VEC3) | (1u << MG_MAC), what, &g,
              &kind))
    return MG_ERR_ARG;
  const bool vec = kind == MG_VEC3 || kind == MG_MAC;
  if (pdata_of(parts, target, vec ? MG_VEC3 : MG_REAL, what)) return MG_ERR_ARG;
  if (parts->n == 0) return MG_OK;
  const Dims& d = parts->d;
  count_launch();
  k_grid_to_parts<<<blocks_of(parts->n), 256, 0, parts->st>>>(
      d, view_of(parts, nullptr, 0), parts->n, g, vec ? g + d.n : nullptr, vec ? g + 2 * d.n : nullptr, target->c[0],
      target->c[1], target->c[2]);
  return launch_status(what);
}

// mg_solver_destroy: the solver's particle systems and their data go with it
void mgpu::particles_release(mg_solver s) {
  std::lock_guard<std::mutex> lk(g_partMu);
  for (auto it = g_pdata.begin(); it != g_pdata.end();) {
    mg_pdata d = *it;
    if (s && d->p->s != s) {
      ++it;
      continue;
    }
    for (float* b : d->c)
      if (b) cudaFree(b);
    delete d;
    it = g_pdata.erase(it);
  }
  for (auto it = g_parts.begin(); it != g_parts.end();) {
    mg_particles p = *it;
    if (s && p->s != s) {
      ++it;
      continue;
    }
    free_parts(p);
    delete p;
    it = g_parts.erase(it);
  }
}
