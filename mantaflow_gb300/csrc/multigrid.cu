// Multigrid preconditioner on the GPU: GridMg (multigrid.cpp:220-954), the
// Galerkin multigrid of Dick, Rogowsky and Westermann (2015) without topology
// awareness, as the reference ships it.
//
// Hierarchy.  Level sizes (n+2)/2 per axis until every side is <= 5 or a
// level has <= 1000 vertices (multigrid.cpp:240-265).  Level 0 is the
// pressure matrix itself, held as the 16-bit Poisson code of pressure.cu
// (A0 count, fluid bit, -1 links) plus two bits: vertex active (A0 != 0) and
// "trivial" (A0 == 1 without links, whose row and right-hand side are scaled
// by 1e-6, multigrid.cpp:345-347, 377-382).  With ghost fluid the float
// diagonal is kept beside it, and with face fractions also the stored float
// off-diagonals Ai, Aj, Ak (the links then say which entries to use; the
// level-0 passes subtract A * x instead of adding x).  Coarse levels store their symmetric 27-point
// (3D) / 9-point (2D) Galerkin stencils as 14 / 5 planes of n floats
// (structure of arrays, so neighbouring threads read neighbouring words),
// plus a byte of vertex type and x, b, r vectors.
//
// Setup (GridMg::setA, multigrid.cpp:386-415).  The coarse-vertex selection
// (genCoarseGrid, :520-578) is a sequential bucket-queue algorithm whose
// order decides which coarse vertices survive, so it runs on the host on the
// vertex-type bytes of the finer level, keeping the reference's queue order.
// It depends only on the level-0 types: a selection is reused while they are
// unchanged (a PcMGDynamic solve on unchanged flags rebuilds only the
// operators).  The Galerkin operators R*A*I (knGenCoarseGridOperator,
// :580-657) are computed on the GPU, one thread per coarse vertex, adding
// the same terms in the same order as the reference (level 1 walks the
// reference's sorted table of fine-grid paths).
//
// V-cycle (doVCycle, :448-504; V(1,1), zero initial guess).  Gauss-Seidel
// uses red/black colours on level 0 (7-point stencil) and eight (four in 2D)
// 2x2x2 block colours on coarse levels; within a colour every vertex reads
// only other colours, so each pass reproduces the reference's float
// arithmetic exactly, and restriction and interpolation sum their terms in
// the reference's loop order.  Level 0 runs as two fused kernels streamed
// along z (entry: both pre-smoothing colours and the residual; exit:
// interpolation, both post-smoothing colours and the outer CG's dot).
// Coarse levels with many slots run one launch per colour, reading a stencil
// dictionary where the level's stencils repeat.  The remaining levels and
// the coarsest solve run as one thread-block-cluster launch; the coarsest
// level is solved by Jacobi-preconditioned CG (solveCG, :793-902) in
// double-float arithmetic with tree-summed dot products, which differs from
// the serial double reference only far below float resolution (a one-CTA
// kernel solves it when the hierarchy has a single level or the GPU cannot
// co-schedule the cluster).
#include "mg_multigrid.h"
#include "mg_reduce.cuh"

#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace mgpu {

namespace {

enum : int8_t { kVtInactive = 0, kVtActive = 1, kVtTrivial = 2 };
// level-0 bits above the Poisson code (bits 0-9)
enum : int { kMgActive = 1 << 10, kMgTrivial = 1 << 11 };
constexpr float kTrivialScale = 1e-6f;  // GridMg::mTrivialEquationScale
constexpr int kMaxLevels = 32;
constexpr int kCgThreads = 1024;        // coarsest level: <= 1000 vertices
constexpr int kThreads1 = 256;

// a coarse level (l >= 1).  Smoothed levels are stored colour-blocked: the
// vertices of each of the 8 (2D: 4) Gauss-Seidel colours (x&1, y&1, z&1)
// form their own sub-grid of 2x2x2 blocks, so a colour pass and the
// neighbours it reads are contiguous in memory.  The coarsest level keeps the
// plain x-fastest order.
struct Lev {
  int sx, sy, sz;
  long long n, py, pz;  // n: storage slots (colour-blocked: ncol * nb)
  int colored, bx, by;  // colour-blocked: blocks per row / column
  long long nb;         // blocks per colour
  int8_t* type;
  float* A;  // stencil entry s of vertex v at A[s * n + v]
  float* x;
  float* b;
  float* r;
  // stencil dictionary (null: none): the full 27 (2D: 9) coefficients of
  // vertex v, in applyAStencil's order, are T[sid[v] * kDictStride + s]
  const uint16_t* sid;
  const float* T;
};

// level 0: snapshot of the Poisson matrix taken by setA
struct Lev0 {
  Dims d;
  uint16_t* code;  // Poisson code | kMgActive | kMgTrivial
  float* a0f;      // trivial-scaled float diagonal (ghost fluid, fractions) or null
  float* ai;       // with fractions: the stored off-diagonals Ai, Aj, Ak
  float* aj;       // (entries of linked pairs; the code's links still say
  float* ak;       // which pairs are linked); null: the Poisson -1 links
  float* r;        // residual
  float* xd;       // x after pre-smoothing: read (with halo) by the up pass
};

// One term of the level-1 Galerkin product (knGenCoarseGridOperator, level
// 1 branch): coarse neighbour N = V + n, fine vertices U = 2V + u and W = 2V
// + w, fine stencil entry sf taken at U (inU) or W, weights rw / iw, added
// into coarse entry sc.  Built once per dimension like the reference's
// precomputed path list, sorted by (sc, U).
struct Path {
  signed char n[3], u[3], w[3];
  signed char sc, sf, inU;
  float rw, iw;
};
constexpr int kMaxPaths = 512;
__constant__ Path c_paths[2][kMaxPaths];  // [0] 2D, [1] 3D
int g_npaths[2] = {0, 0};
bool g_pathsReady = false;
int g_tailCta = 0;  // CTAs of the cluster V-cycle tail (0: per-level launches)

__host__ __device__ __forceinline__ int parity3(int a, int b, int c) { return (a & 1) + (b & 1) + (c & 1); }
// 2^-e (0 <= e <= 3), the reference's 1/(1<<e): exact, so the device forms
// it from its exponent bits instead of a division
__host__ __device__ __forceinline__ float inv_pow2(int e) {
#ifdef __CUDA_ARCH__
  return __int_as_float((127 - e) << 23);
#else
  return 1.f / (float)(1 << e);
#endif
}

__device__ __forceinline__ float l0_diag(int c, const float* __restrict__ a0f, long long v) {
  if (a0f) return a0f[v];
  return (c & kMgTrivial) ? kTrivialScale : (float)(c & 7);
}
__device__ __forceinline__ float l0_rhs(int c, const float* __restrict__ res, long long v) {
  const float b = res[v];
  return (c & kMgTrivial) ? b * kTrivialScale : b;
}
// fine-level stencil entry sf of level-0 vertex u: A0, Ai, Aj, Ak
__device__ __forceinline__ float l0_entry(const Lev0& F, long long u, int sf) {
  const int c = F.code[u];
  if (sf == 0) return l0_diag(c, F.a0f, u);
  if (F.ai) return (sf == 1 ? F.ai : (sf == 2 ? F.aj : F.ak))[u];
  const int bit = sf == 1 ? kHighX : (sf == 2 ? kHighY : kHighZ);
  return (c & bit) ? -1.f : 0.f;
}

__host__ __device__ __forceinline__ long long lin(const Lev& L, int x, int y, int z) {
  if (L.colored)
    return (long long)((x & 1) | ((y & 1) << 1) | ((z & 1) << 2)) * L.nb + (x >> 1) +
           (long long)L.bx * ((y >> 1) + (long long)L.by * (z >> 1));
  return x + L.py * y + L.pz * z;
}
__device__ __forceinline__ bool inside(const Lev& L, int x, int y, int z) {
  return x >= 0 && y >= 0 && z >= 0 && x < L.sx && y < L.sy && z < L.sz;
}
// slot -> vertex; padding slots of a colour-blocked level map outside the
// grid and have type inactive
// a block index's block coordinates; 32-bit: a level holds fewer than 2^31
// slots (the finest grid has fewer than 2^31 cells)
__device__ __forceinline__ void block_xyz(long long bi64, int bx, int by, int& x, int& y, int& z) {
  const unsigned bi = (unsigned)bi64, q = bi / (unsigned)bx, r = q / (unsigned)by;
  x = (int)(bi - q * (unsigned)bx);
  y = (int)(q - r * (unsigned)by);
  z = (int)r;
}
__device__ __forceinline__ void coords(const Lev& L, long long v, int& x, int& y, int& z) {
  if (L.colored) {
    const unsigned u = (unsigned)v, c = u / (unsigned)L.nb, bi = u - c * (unsigned)L.nb;
    int bxi, byi, bzi;
    block_xyz(bi, L.bx, L.by, bxi, byi, bzi);
    x = 2 * bxi + (int)(c & 1);
    y = 2 * byi + (int)((c >> 1) & 1);
    z = 2 * bzi + (int)(c >> 2);
    return;
  }
  const unsigned u = (unsigned)v, q = u / (unsigned)L.sx, r = q / (unsigned)L.sy;
  x = (int)(u - q * (unsigned)L.sx);
  y = (int)(q - r * (unsigned)L.sy);
  z = (int)r;
}

// The 27 neighbours of a vertex of a colour-blocked level: slot offsets and
// in-level flags separate per axis.  A step d along x moves to colour bit
// (x+d)&1 and block column (x+d)>>1 (likewise y, z), so the neighbour's
// slot is v + ox[dx+1] + oy[dy+1] + oz[dz+1]: nine offsets and nine flags
// per vertex instead of an index computation per neighbour.
struct Nb3 {
  int ox[3], oy[3], oz[3];
  bool ix[3], iy[3], iz[3];
};
__device__ __forceinline__ Nb3 nb3(const Lev& L, int vx, int vy, int vz) {
  Nb3 r;
  const int cx = vx & 1, cy = vy & 1, cz = vz & 1;
  const int nb = (int)L.nb, bx = L.bx, bxy = L.bx * L.by;
#pragma unroll
  for (int d = -1; d <= 1; d++) {
    r.ox[d + 1] = (((cx + d) & 1) - cx) * nb + ((cx + d) >> 1);
    r.oy[d + 1] = 2 * (((cy + d) & 1) - cy) * nb + bx * ((cy + d) >> 1);
    r.oz[d + 1] = 4 * (((cz + d) & 1) - cz) * nb + bxy * ((cz + d) >> 1);
    r.ix[d + 1] = (unsigned)(vx + d) < (unsigned)L.sx;
    r.iy[d + 1] = (unsigned)(vy + d) < (unsigned)L.sy;
    r.iz[d + 1] = (unsigned)(vz + d) < (unsigned)L.sz;
  }
  return r;
}

#define GRID_STRIDE(v, n) \
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < (n); v += (long long)gridDim.x * blockDim.x)

// ---------------------------------------------------------------- setup
// knCopyA + knActivateVertices (multigrid.cpp:333-384).  With stored
// off-diagonals (fractions) they are copied too, and an equation is trivial
// when A0 == 1 and its six entries compare equal to zero (analyzeStencil,
// :320-347): a linked pair whose face fraction is 0 has an entry of -0.
__global__ void k_mg_snapshot0(Dims d, const code_t* __restrict__ code, const float* __restrict__ A0f,
                               const float* __restrict__ Ai, const float* __restrict__ Aj,
                               const float* __restrict__ Ak, uint16_t* code0, float* a0f0, float* ai0, float* aj0,
                               float* ak0, int8_t* type0) {
  GRID_STRIDE(v, d.n) {
    int c = code[v] & 0x3ff;
    float a0 = A0f ? A0f[v] : (float)(c & 7);
    if (Ai) {
      ai0[v] = Ai[v];
      aj0[v] = Aj[v];
      ak0[v] = Ak[v];
    }
    int8_t t = kVtInactive;
    if (a0 != 0.f) {
      t = kVtActive;
      c |= kMgActive;
      bool links = (c & (kLowX | kLowY | kLowZ | kHighX | kHighY | kHighZ)) != 0;
      if (Ai) {
        const unsigned u = (unsigned)v, q = u / (unsigned)d.nx, r = q / (unsigned)d.ny;  // < 2^31 cells
        const int i = (int)(u - q * (unsigned)d.nx), j = (int)(q - r * (unsigned)d.ny), k = d.is3d ? (int)r : 0;
        links = Ai[v] != 0.f || Aj[v] != 0.f || (d.is3d && Ak[v] != 0.f) || (i > 0 && Ai[v - 1] != 0.f) ||
                (j > 0 && Aj[v - d.sy] != 0.f) || (d.is3d && k > 0 && Ak[v - d.sz] != 0.f);
      }
      if (a0 == 1.f && !links) {
        t = kVtTrivial;
        c |= kMgTrivial;
        a0 = a0 * kTrivialScale;
      }
    }
    code0[v] = (uint16_t)c;
    if (a0f0) a0f0[v] = a0;
    type0[v] = t;
  }
}

// knGenCoarseGridOperator, level 1 from the 7-point level 0 (paths)
template <bool IS3D>
__global__ void k_mg_coarse_op1(Lev C, Lev0 F, int S, int npaths) {
  const Path* P = c_paths[IS3D ? 1 : 0];
  const int fx = F.d.nx, fy = F.d.ny, fz = F.d.nz;
  GRID_STRIDE(v, C.n) {
    if (C.type[v] == kVtInactive) continue;
    int vx, vy, vz;
    coords(C, v, vx, vy, vz);
    int cur = 0;
    float acc = 0.f;
    for (int q = 0; q < npaths; q++) {
      const Path& p = P[q];
      if (p.sc != cur) {
        C.A[(long long)cur * C.n + v] = acc;
        for (int e = cur + 1; e < p.sc; e++) C.A[(long long)e * C.n + v] = 0.f;
        cur = p.sc;
        acc = 0.f;
      }
      const int nx = vx + p.n[0], ny = vy + p.n[1], nz = vz + p.n[2];
      if (!inside(C, nx, ny, nz) || C.type[lin(C, nx, ny, nz)] == kVtInactive) continue;
      const int ux = 2 * vx + p.u[0], uy = 2 * vy + p.u[1], uz = 2 * vz + p.u[2];
      if (ux < 0 || uy < 0 || uz < 0 || ux >= fx || uy >= fy || uz >= fz) continue;
      const long long u = ix(F.d, ux, uy, uz);
      if (!(F.code[u] & kMgActive)) continue;
      const int wx = 2 * vx + p.w[0], wy = 2 * vy + p.w[1], wz = 2 * vz + p.w[2];
      if (wx < 0 || wy < 0 || wz < 0 || wx >= fx || wy >= fy || wz >= fz) continue;
      const long long w = ix(F.d, wx, wy, wz);
      if (!(F.code[w] & kMgActive)) continue;
      const float a = l0_entry(F, p.inU ? u : w, p.sf);
      acc = acc + (p.rw * a) * p.iw;
    }
    C.A[(long long)cur * C.n + v] = acc;
    for (int e = cur + 1; e < S; e++) C.A[(long long)e * C.n + v] = 0.f;
  }
}

// knGenCoarseGridOperator, levels >= 2 from a 27-point (9-point) level
template <bool IS3D>
__global__ void k_mg_coarse_op(Lev C, Lev F, int S) {
  constexpr int SZ = IS3D ? 1 : 0;  // stencil half-extent in z
  GRID_STRIDE(v, C.n) {
    if (C.type[v] == kVtInactive) continue;
    float A[14];
#pragma unroll
    for (int e = 0; e < 14; e++) A[e] = 0.f;
    int vx, vy, vz;
    coords(C, v, vx, vy, vz);
    const int ulo[3] = {max(0, 2 * vx - 1), max(0, 2 * vy - 1), max(0, 2 * vz - 1)};
    const int uhi[3] = {min(F.sx - 1, 2 * vx + 1), min(F.sy - 1, 2 * vy + 1), min(F.sz - 1, 2 * vz + 1)};
    for (int uz = ulo[2]; uz <= uhi[2]; uz++)
      for (int uy = ulo[1]; uy <= uhi[1]; uy++)
        for (int ux = ulo[0]; ux <= uhi[0]; ux++) {
          const long long u = lin(F, ux, uy, uz);
          if (F.type[u] == kVtInactive) continue;
          const float rw = inv_pow2(parity3(ux, uy, uz));
          const int nlo[3] = {(ux - 1) / 2, (uy - 1) / 2, (uz - 1) / 2};
          const int nhi[3] = {min(C.sx - 1, (ux + 2) / 2), min(C.sy - 1, (uy + 2) / 2), min(C.sz - 1, (uz + 2) / 2)};
          for (int nz = nlo[2]; nz <= nhi[2]; nz++)
            for (int ny = nlo[1]; ny <= nhi[1]; ny++)
              for (int nx = nlo[0]; nx <= nhi[0]; nx++) {
                const long long nn = lin(C, nx, ny, nz);
                if (C.type[nn] == kVtInactive) continue;
                const int sc = (nx - vx + 1) + 3 * (ny - vy + 1) + 9 * (nz - vz + SZ);
                if (sc < S - 1) continue;
                const int wlo[3] = {max(0, max(ux - 1, 2 * nx - 1)), max(0, max(uy - 1, 2 * ny - 1)),
                                    max(0, max(uz - 1, 2 * nz - 1))};
                const int whi[3] = {min(F.sx - 1, min(ux + 1, 2 * nx + 1)), min(F.sy - 1, min(uy + 1, 2 * ny + 1)),
                                    min(F.sz - 1, min(uz + 1, 2 * nz + 1))};
                for (int wz = wlo[2]; wz <= whi[2]; wz++)
                  for (int wy = wlo[1]; wy <= whi[1]; wy++)
                    for (int wx = wlo[0]; wx <= whi[0]; wx++) {
                      const long long w = lin(F, wx, wy, wz);
                      if (F.type[w] == kVtInactive) continue;
                      const int sf = (wx - ux + 1) + 3 * (wy - uy + 1) + 9 * (wz - uz + SZ);
                      const float iw = inv_pow2(parity3(wx, wy, wz));
                      const float a = sf < S ? F.A[(long long)(S - 1 - sf) * F.n + w] : F.A[(long long)(sf - S + 1) * F.n + u];
                      A[sc - S + 1] = A[sc - S + 1] + (rw * a) * iw;
                    }
              }
        }
    for (int e = 0; e < S; e++) C.A[(long long)e * C.n + v] = A[e];
  }
}

// ------------------------------------------------------------ V-cycle
// Sum over the 27 (9) stencil neighbours of a coarse vertex, in the
// reference's FOR_VECLIN_MINMAX order (x fastest): sum -= A * x[N].
// Inactive and padding vertices hold x = 0 (and zero matrix entries), so
// their terms subtract zero and need no type test.  The loads of one z-plane
// of the stencil (9 matrix entries, 9 values) are issued together before
// its subtractions; the chain of float operations is the reference's.
// vectors that other CTAs of the same launch write (the cluster V-cycle
// below) are read at L2, past the SM's non-coherent L1
template <bool CG>
__device__ __forceinline__ float ldv(const float* p) {
  if (CG) return __ldcg(p);
  return *p;
}

template <bool IS3D, bool SKIP_CENTER, bool CG = false>
__device__ __forceinline__ float stencil_sub(const Lev& L, int vx, int vy, int vz, long long v, float sum) {
  constexpr int ZL = IS3D ? -1 : 0, ZH = IS3D ? 1 : 0;
  constexpr int S = IS3D ? 14 : 5;
  const Nb3 o = nb3(L, vx, vy, vz);  // L is colour-blocked
  const int vi = (int)v;
#pragma unroll
  for (int dz = ZL; dz <= ZH; dz++) {
    float a[9], xv[9];
    bool in[9];
#pragma unroll
    for (int dy = -1; dy <= 1; dy++)
#pragma unroll
      for (int dx = -1; dx <= 1; dx++) {
        const int q = (dy + 1) * 3 + (dx + 1);
        const int s = (dz - ZL) * 9 + q;
        in[q] = o.ix[dx + 1] && o.iy[dy + 1] && o.iz[dz + 1] && !(SKIP_CENTER && s == S - 1);
        const int nn = in[q] ? vi + o.ox[dx + 1] + o.oy[dy + 1] + o.oz[dz + 1] : vi;
        a[q] = s < S ? L.A[(long long)(S - 1 - s) * L.n + nn] : L.A[(long long)(s - S + 1) * L.n + vi];
        xv[q] = ldv<CG>(&L.x[nn]);
      }
#pragma unroll
    for (int q = 0; q < 9; q++)
      if (in[q]) sum = sum - a[q] * xv[q];
  }
  return sum;
}

// The same sum with every load of the stencil (and of the centre's type,
// right-hand side and diagonal) issued before any arithmetic: one memory
// round trip per vertex, for the cluster tail, whose passes have about one
// vertex per thread and nothing else to overlap the latency with.
// Levels in the tail have few slots (kTailSlots): offsets are 32-bit.
template <bool IS3D, bool SKIP_CENTER>
__device__ __forceinline__ float stencil_sub_flat(const Lev& L, int vx, int vy, int vz, int v, float sum) {
  constexpr int NZ = IS3D ? 3 : 1, ZL = IS3D ? -1 : 0;
  constexpr int S = IS3D ? 14 : 5;
  const int n = (int)L.n;
  const Nb3 o = nb3(L, vx, vy, vz);  // L is colour-blocked
  float a[NZ * 9], xv[NZ * 9];
  unsigned inm = 0;
#pragma unroll
  for (int s = 0; s < NZ * 9; s++) {
    const int dx = s % 3, dy = (s / 3) % 3, dz = s / 9 + ZL + 1;
    const bool in = o.ix[dx] && o.iy[dy] && o.iz[dz] && !(SKIP_CENTER && s == S - 1);
    inm |= in ? 1u << s : 0u;
    const int nn = in ? v + o.ox[dx] + o.oy[dy] + o.oz[dz] : v;
    a[s] = s < S ? L.A[(S - 1 - s) * n + nn] : L.A[(s - S + 1) * n + v];
    xv[s] = __ldcg(&L.x[nn]);
  }
#pragma unroll
  for (int s = 0; s < NZ * 9; s++)
    if (inm & (1u << s)) sum = sum - a[s] * xv[s];
  return sum;
}

// ---- stencil dictionary.  A coarse level's Galerkin stencils repeat:
// away from walls, obstacles and free surfaces every vertex of a level has
// the same 27 coefficients.  The dictionary holds each distinct tuple once;
// a vertex keeps a 16-bit id, so a colour pass reads 2 bytes of matrix per
// vertex instead of 108.  The tuples are compared bit for bit when the
// dictionary is built (a level with a hash collision or more than
// kDictCap distinct stencils keeps reading its planes), so smoothing and
// residual do exactly the same float operations on the same values.
constexpr int kDictCap = 65535;  // ids 1..kDictCap; id 0: inactive vertices
constexpr int kDictStride = 28;
constexpr int kDictTableBits = 17;
constexpr int kDictTable = 1 << kDictTableBits;
constexpr int kDictProbes = 256;

// the coefficient tuple of slot v (zero outside the level)
template <bool IS3D>
__device__ __forceinline__ void dict_tuple(const Lev& L, long long v, float* a) {
  constexpr int NZ = IS3D ? 3 : 1, ZL = IS3D ? -1 : 0;
  constexpr int S = IS3D ? 14 : 5;
  int vx, vy, vz;
  coords(L, v, vx, vy, vz);
  const Nb3 o = nb3(L, vx, vy, vz);  // L is colour-blocked
  const int vi = (int)v;
#pragma unroll
  for (int s = 0; s < NZ * 9; s++) {
    const int dx = s % 3, dy = (s / 3) % 3, dz = s / 9 + ZL + 1;
    const bool in = o.ix[dx] && o.iy[dy] && o.iz[dz];
    const int nn = in ? vi + o.ox[dx] + o.oy[dy] + o.oz[dz] : vi;
    const float c = s < S ? L.A[(long long)(S - 1 - s) * L.n + nn] : L.A[(long long)(s - S + 1) * L.n + vi];
    a[s] = in ? c : 0.f;
  }
}
template <int NS>
__device__ __forceinline__ unsigned long long dict_hash(const float* a) {
  unsigned long long h = 0x9E3779B97F4A7C15ull;
#pragma unroll
  for (int s = 0; s < NS; s++) {
    h ^= (unsigned long long)__float_as_uint(a[s]) + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h *= 0xBF58476D1CE4E5B9ull;
  }
  return (h ^ (h >> 31)) | 1ull;  // 0 marks an empty table slot
}
// the table slot of hash hv (inserting it when ins); -1 after kDictProbes
__device__ __forceinline__ int dict_slot(unsigned long long* keys, unsigned long long hv, bool ins) {
  int slot = (int)(hv & (kDictTable - 1));
  for (int k = 0; k < kDictProbes; k++) {
    const unsigned long long cur = ins ? atomicCAS(&keys[slot], 0ull, hv) : keys[slot];
    if (cur == hv || (ins && cur == 0ull)) return slot;
    if (!ins && cur == 0ull) return -1;
    slot = (slot + 1) & (kDictTable - 1);
  }
  return -1;
}
// flags: [0] table overflow, [1] tuple mismatch, [2] distinct tuples
template <bool IS3D>
__global__ void __launch_bounds__(256) k_dict_insert(Lev L, unsigned long long* keys, int* rep, int* flags) {
  constexpr int NS = IS3D ? 27 : 9;
  GRID_STRIDE(v, L.n) {
    if (L.type[v] == kVtInactive) continue;
    float a[NS];
    dict_tuple<IS3D>(L, v, a);
    const int slot = dict_slot(keys, dict_hash<NS>(a), true);
    if (slot < 0) flags[0] = 1;
    else atomicMin(&rep[slot], (int)v);  // the lowest slot index represents the tuple
  }
}
// ids in table order: one CTA of 1024 threads, 128 table slots per thread
__global__ void __launch_bounds__(1024) k_dict_ids(const unsigned long long* keys, int* slotId, int* flags) {
  constexpr int PER = kDictTable / 1024;
  __shared__ int scan[1024];
  const int t = threadIdx.x;
  int cnt = 0;
  for (int k = 0; k < PER; k++) cnt += keys[t * PER + k] != 0ull;
  scan[t] = cnt;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {  // inclusive Hillis-Steele scan
    const int add = t >= o ? scan[t - o] : 0;
    __syncthreads();
    scan[t] += add;
    __syncthreads();
  }
  int id = scan[t] - cnt + 1;
  for (int k = 0; k < PER; k++) {
    const int q = t * PER + k;
    slotId[q] = keys[q] != 0ull ? id++ : 0;
  }
  if (t == 1023) flags[2] = scan[1023];
}
template <bool IS3D>
__global__ void __launch_bounds__(256) k_dict_fill(Lev L, unsigned long long* keys, const int* rep, const int* slotId,
                                                   uint16_t* sid, float* T, int* flags) {
  constexpr int NS = IS3D ? 27 : 9;
  GRID_STRIDE(v, L.n) {
    if (L.type[v] == kVtInactive) {
      sid[v] = 0;
      continue;
    }
    float a[NS];
    dict_tuple<IS3D>(L, v, a);
    const int slot = dict_slot(keys, dict_hash<NS>(a), false);
    const int id = slot < 0 ? 0 : slotId[slot];
    if (slot < 0 || id > kDictCap) {
      flags[0] = 1;
      sid[v] = 0;
      continue;
    }
    sid[v] = (uint16_t)id;
    if (rep[slot] == (int)v)
#pragma unroll
      for (int s = 0; s < NS; s++) T[(long long)id * kDictStride + s] = a[s];
  }
}
template <bool IS3D>
__global__ void __launch_bounds__(256) k_dict_verify(Lev L, const uint16_t* sid, const float* T, int* flags) {
  constexpr int NS = IS3D ? 27 : 9;
  GRID_STRIDE(v, L.n) {
    if (L.type[v] == kVtInactive) continue;
    float a[NS];
    dict_tuple<IS3D>(L, v, a);
    const float* t = T + (long long)sid[v] * kDictStride;
    bool same = sid[v] != 0;
#pragma unroll
    for (int s = 0; s < NS; s++) same = same && __float_as_uint(a[s]) == __float_as_uint(t[s]);
    if (!same) flags[1] = 1;
  }
}

// stencil_sub with the coefficients from the dictionary tuple t (CG: x is
// written by other CTAs of the same launch and read at L2)
template <bool IS3D, bool SKIP_CENTER, bool CG = false>
__device__ __forceinline__ float stencil_sub_dict(const Lev& L, const float* __restrict__ t, int vx, int vy, int vz,
                                                  float sum) {
  constexpr int ZL = IS3D ? -1 : 0, ZH = IS3D ? 1 : 0;
  constexpr int S = IS3D ? 14 : 5;
  const Nb3 o = nb3(L, vx, vy, vz);  // L is colour-blocked
  const int vi = (int)lin(L, vx, vy, vz);
#pragma unroll
  for (int dz = ZL; dz <= ZH; dz++) {
    float a[9], xv[9];
    bool in[9];
#pragma unroll
    for (int dy = -1; dy <= 1; dy++)
#pragma unroll
      for (int dx = -1; dx <= 1; dx++) {
        const int q = (dy + 1) * 3 + (dx + 1);
        const int s = (dz - ZL) * 9 + q;
        in[q] = o.ix[dx + 1] && o.iy[dy + 1] && o.iz[dz + 1] && !(SKIP_CENTER && s == S - 1);
        a[q] = t[s];
        xv[q] = in[q] ? ldv<CG>(&L.x[vi + o.ox[dx + 1] + o.oy[dy + 1] + o.oz[dz + 1]]) : 0.f;
      }
#pragma unroll
    for (int q = 0; q < 9; q++)
      if (in[q]) sum = sum - a[q] * xv[q];
  }
  return sum;
}

// knSmoothColor on a coarse level, one vertex: block bi of colour offset
// (ox, oy, oz) in 2x2x2 blocks, bx x by blocks per z-plane
template <bool IS3D, bool CG>
__device__ __forceinline__ void smooth_vertex(const Lev& L, long long bi, int ox, int oy, int oz, int bx, int by) {
  int vx, vy, vz;
  block_xyz(bi, bx, by, vx, vy, vz);
  vx = 2 * vx + ox;
  vy = 2 * vy + oy;
  vz = 2 * vz + oz;
  if (!inside(L, vx, vy, vz)) return;
  const long long v = L.colored ? (long long)(ox | (oy << 1) | (oz << 2)) * L.nb + bi : lin(L, vx, vy, vz);
  if (L.type[v] == kVtInactive) return;
  const float sum = stencil_sub<IS3D, true, CG>(L, vx, vy, vz, v, ldv<CG>(&L.b[v]));
  L.x[v] = sum / L.A[v];
}

// smooth_vertex for the cluster tail: the vertex type is tested after all
// loads were issued (inactive vertices only cost loads)
template <bool IS3D>
__device__ __forceinline__ void smooth_vertex_flat(const Lev& L, long long bi, int ox, int oy, int oz, int bx, int by) {
  int vx, vy, vz;
  block_xyz(bi, bx, by, vx, vy, vz);
  vx = 2 * vx + ox;
  vy = 2 * vy + oy;
  vz = 2 * vz + oz;
  if (!inside(L, vx, vy, vz)) return;
  const long long v = L.colored ? (long long)(ox | (oy << 1) | (oz << 2)) * L.nb + bi : lin(L, vx, vy, vz);
  const int8_t ty = L.type[v];
  const float diag = L.A[v];
  const float sum = stencil_sub_flat<IS3D, true>(L, vx, vy, vz, (int)v, __ldcg(&L.b[v]));
  if (ty != kVtInactive) L.x[v] = sum / diag;
}

template <bool IS3D>
__device__ __forceinline__ void residual_vertex_flat(const Lev& L, long long v) {
  int vx, vy, vz;
  coords(L, v, vx, vy, vz);
  const int8_t ty = L.type[v];
  const float r = stencil_sub_flat<IS3D, false>(L, vx, vy, vz, (int)v, __ldcg(&L.b[v]));
  if (ty != kVtInactive) L.r[v] = r;
}

// the same two passes for the cluster tail on a level with a stencil
// dictionary: the vertex's id, then its tuple and every x at once
template <bool IS3D>
__device__ __forceinline__ void smooth_vertex_dict_flat(const Lev& L, long long bi, int ox, int oy, int oz, int bx, int by) {
  constexpr int S = IS3D ? 14 : 5;
  int vx, vy, vz;
  block_xyz(bi, bx, by, vx, vy, vz);
  vx = 2 * vx + ox;
  vy = 2 * vy + oy;
  vz = 2 * vz + oz;
  if (!inside(L, vx, vy, vz)) return;
  const long long v = (long long)(ox | (oy << 1) | (oz << 2)) * L.nb + bi;
  const int8_t ty = L.type[v];
  const float* t = L.T + (int)L.sid[v] * kDictStride;
  const float sum = stencil_sub_dict<IS3D, true, true>(L, t, vx, vy, vz, __ldcg(&L.b[v]));
  if (ty != kVtInactive) L.x[v] = sum / t[S - 1];
}
template <bool IS3D>
__device__ __forceinline__ void residual_vertex_dict_flat(const Lev& L, long long v) {
  int vx, vy, vz;
  coords(L, v, vx, vy, vz);
  if (!inside(L, vx, vy, vz)) return;  // padding slot
  const int8_t ty = L.type[v];
  const float* t = L.T + (int)L.sid[v] * kDictStride;
  const float r = stencil_sub_dict<IS3D, false, true>(L, t, vx, vy, vz, __ldcg(&L.b[v]));
  if (ty != kVtInactive) L.r[v] = r;
}

// knCalcResidual on a coarse level, one storage slot
template <bool IS3D, bool CG>
__device__ __forceinline__ void residual_vertex(const Lev& L, long long v) {
  if (L.type[v] == kVtInactive) return;
  int vx, vy, vz;
  coords(L, v, vx, vy, vz);
  L.r[v] = stencil_sub<IS3D, false, CG>(L, vx, vy, vz, v, ldv<CG>(&L.b[v]));
}

// knRestrict into slot v of level D from the level below (level 0 when
// FROM0), plus knSet(x[D], 0) of the next smoothing's initial guess
template <bool FROM0, bool CG>
__device__ __forceinline__ void restrict_vertex_at(const Lev& D, const Lev& S, const Lev0& F, long long v, int vx, int vy,
                                                   int vz) {
  const int sx = FROM0 ? F.d.nx : S.sx, sy = FROM0 ? F.d.ny : S.sy, sz = FROM0 ? F.d.nz : S.sz;
  const long long py = F.d.sy, pz = F.d.sz;
  D.x[v] = 0.f;
  const int8_t ty = D.type[v];
  // the fine vertices 2V-1 .. 2V+1 inside the level, in the reference's
  // loop order; all loads first (the type is tested after them)
  float rv[27];
  bool in[27];
#pragma unroll
  for (int q = 0; q < 27; q++) {
    const int rx = 2 * vx - 1 + q % 3, ry = 2 * vy - 1 + (q / 3) % 3, rz = 2 * vz - 1 + q / 9;
    in[q] = rx >= 0 && ry >= 0 && rz >= 0 && rx < sx && ry < sy && rz < sz;
    // inactive fine vertices hold r = 0: adding their term adds zero
    rv[q] = in[q] ? (FROM0 ? F.r[rx + py * ry + pz * rz] : ldv<CG>(&S.r[lin(S, rx, ry, rz)])) : 0.f;
  }
  float sum = 0.f;
#pragma unroll
  for (int q = 0; q < 27; q++) {
    const int rx = 2 * vx - 1 + q % 3, ry = 2 * vy - 1 + (q / 3) % 3, rz = 2 * vz - 1 + q / 9;
    if (in[q]) sum = sum + inv_pow2(parity3(rx, ry, rz)) * rv[q];
  }
  if (ty != kVtInactive) D.b[v] = sum;
}
template <bool FROM0, bool CG>
__device__ __forceinline__ void restrict_vertex(const Lev& D, const Lev& S, const Lev0& F, long long v) {
  int vx, vy, vz;
  coords(D, v, vx, vy, vz);
  restrict_vertex_at<FROM0, CG>(D, S, F, v, vx, vy, vz);
}

// knInterpolate from level S = D+1 and knAddAssign: x[D] += I * x[S]
template <bool IS3D, bool CG>
__device__ __forceinline__ void interp_vertex(const Lev& D, const Lev& S, long long v) {
  const int8_t ty = D.type[v];
  int vx, vy, vz;
  coords(D, v, vx, vy, vz);
  if (!inside(D, vx, vy, vz)) return;  // padding slot
  // coarse parents V/2 .. (V+1)/2 per axis (one or two), in the
  // reference's loop order; inactive coarse vertices hold x = 0
  const int hx = (vx + 1) / 2 - vx / 2, hy = (vy + 1) / 2 - vy / 2, hz = (vz + 1) / 2 - vz / 2;
  float cv[8];
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int ox = q & 1, oy = (q >> 1) & 1, oz = q >> 2;
    const bool use = (ox <= hx) && (oy <= hy) && (oz <= hz);
    cv[q] = use ? ldv<CG>(&S.x[lin(S, vx / 2 + ox, vy / 2 + oy, vz / 2 + oz)]) : 0.f;
  }
  float sum = 0.f;
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int ox = q & 1, oy = (q >> 1) & 1, oz = q >> 2;
    if ((ox <= hx) && (oy <= hy) && (oz <= hz)) sum = sum + cv[q];
  }
  const float xv = ldv<CG>(&D.x[v]) + inv_pow2(parity3(vx, vy, vz)) * sum;
  if (ty != kVtInactive) D.x[v] = xv;
}

template <bool IS3D>
__global__ void __launch_bounds__(256, 3) k_mg_smooth(Lev L, int S, int ox, int oy, int oz, const CgScalars* sc) {
  if (sc->done) return;
  const int bx = (L.sx + 1) / 2, by = (L.sy + 1) / 2, bz = (L.sz + 1) / 2;
  const long long nb = (long long)bx * by * bz;
  GRID_STRIDE(bi, nb) smooth_vertex<IS3D, false>(L, bi, ox, oy, oz, bx, by);
}

template <bool IS3D>
__global__ void __launch_bounds__(256, 3) k_mg_residual(Lev L, int S, const CgScalars* sc) {
  if (sc->done) return;
  GRID_STRIDE(v, L.n) residual_vertex<IS3D, false>(L, v);
}

// the same passes on a level with a stencil dictionary
template <bool IS3D>
__global__ void __launch_bounds__(256, 4) k_mg_smooth_dict(Lev L, int ox, int oy, int oz, const CgScalars* sc) {
  if (sc->done) return;
  const int bx = (L.sx + 1) / 2, by = (L.sy + 1) / 2, bz = (L.sz + 1) / 2;
  const long long nb = (long long)bx * by * bz;
  constexpr int S = IS3D ? 14 : 5;
  GRID_STRIDE(bi, nb) {
    int vx, vy, vz;
    block_xyz(bi, bx, by, vx, vy, vz);
    vx = 2 * vx + ox;
    vy = 2 * vy + oy;
    vz = 2 * vz + oz;
    if (!inside(L, vx, vy, vz)) continue;
    const long long v = (long long)(ox | (oy << 1) | (oz << 2)) * L.nb + bi;
    // the vertex type is tested after every load was issued (an inactive
    // vertex has id 0, whose table entry exists)
    const int8_t ty = L.type[v];
    const float* t = L.T + (int)L.sid[v] * kDictStride;
    const float sum = stencil_sub_dict<IS3D, true>(L, t, vx, vy, vz, L.b[v]);
    if (ty != kVtInactive) L.x[v] = sum / t[S - 1];
  }
}

template <bool IS3D>
__global__ void __launch_bounds__(256, 4) k_mg_residual_dict(Lev L, const CgScalars* sc) {
  if (sc->done) return;
  GRID_STRIDE(v, L.n) {
    const int8_t ty = L.type[v];
    int vx, vy, vz;
    coords(L, v, vx, vy, vz);
    if (!inside(L, vx, vy, vz)) continue;  // padding slot
    const float* t = L.T + (int)L.sid[v] * kDictStride;
    const float r = stencil_sub_dict<IS3D, false>(L, t, vx, vy, vz, L.b[v]);
    if (ty != kVtInactive) L.r[v] = r;
  }
}

template <bool FROM0>
__global__ void __launch_bounds__(256) k_mg_restrict(Lev D, Lev S, Lev0 F, const CgScalars* sc) {
  if (sc->done) return;
  GRID_STRIDE(v, D.n) restrict_vertex<FROM0, false>(D, S, F, v);
}

// restriction from level 0 with threads in x-fastest coarse order over a
// coarse plane (a warp's 27 gathers then cover 64 neighbouring fine cells
// per row instead of 128; no idle lanes at the end of a row)
__global__ void __launch_bounds__(256) k_mg_restrict0(Lev D, Lev0 F, const CgScalars* sc) {
  if (sc->done) return;
  const unsigned e = blockIdx.x * 256u + threadIdx.x;  // a coarse plane holds < 2^31 vertices
  if (e >= (unsigned)D.sx * (unsigned)D.sy) return;
  const int vy = (int)(e / (unsigned)D.sx), vx = (int)(e - (unsigned)vy * (unsigned)D.sx), vz = blockIdx.y;
  restrict_vertex_at<true, false>(D, D, F, lin(D, vx, vy, vz), vx, vy, vz);
}

template <bool IS3D>
__global__ void __launch_bounds__(256) k_mg_interp_add(Lev D, Lev S, const CgScalars* sc) {
  if (sc->done) return;
  GRID_STRIDE(v, D.n) interp_vertex<IS3D, false>(D, S, v);
}

// ---- fused level-0 passes, streamed along z.  A CTA of 512 threads owns
// a column of fine cells over zc planes (in 2D, one plane) and walks the
// column's region -- 32 x 32 cells per plane starting at (28 tx, 28 ty) --
// plane by plane.  It owns the region minus a 2-cell halo on each side
// where the grid goes on (28 x 28 cells inside the grid, up to 30 where a
// region edge is the grid's edge: at 256 cells, 9 tiles per row instead of
// the 10 a fixed 28-cell tile takes), keeping the last five planes of code,
// right-hand side, diagonal and x in shared memory.  In each step plane p
// is staged (stage A, two cells per thread), plane p-1 gets its colour-1
// pass (B, one colour-1 cell per thread) and plane p-2 its last pass (C), so
// every cell goes through exactly the float operations of the per-colour
// Gauss-Seidel passes, in the same order; halo cells are recomputed by each
// CTA that needs them.  With five planes in the ring, stage A of the next
// step writes a plane no thread still reads, so a step needs two barriers.
constexpr int kTX = 28, kTY = 28, kZC = 32;  // kZC: default planes per CTA (even)
constexpr int kRX = 32, kRY = 32, kRing = 5;
// tiles of the level-0 passes along an axis of n cells (tile t's region
// starts at 28 t; the last one reaches the grid's edge)
__host__ __device__ constexpr int level0_tiles(int n) { return n <= kRX ? 1 : (n - 4 + kTX - 1) / kTX; }
// the owned cells of a region along one axis: [lo, hi) in region coordinates
__device__ __forceinline__ int owned_lo(int o) { return o == 0 ? 0 : 2; }
__device__ __forceinline__ int owned_hi(int o, int n, int r) { return o + r >= n ? r : r - 2; }
constexpr int kT0 = 512;  // threads of a level-0 CTA: rows w and w + 16 of warp w

struct Ring0 {  // five planes of the region (dynamic shared memory)
  float res[kRing][kRY][kRX];
  float x[kRing][kRY][kRX];
  float diag[kRing][kRY][kRX];
  uint16_t code[kRing][kRY][kRX];
};
__device__ __forceinline__ int ring0(int p) { return (p + 10) % kRing; }  // p >= -2

// one plane of this thread's two region cells (rows w and w + 16)
struct Plane0 {
  int c[2];
  float r[2], a[2], xd[2];
};
template <bool UP>
__device__ __forceinline__ void load_plane0(const Lev0& F, const float* __restrict__ res, int ox, int oy, int p, Plane0& P) {
  const Dims& d = F.d;
  const int gx = ox + (int)(threadIdx.x & 31);
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int gy = oy + (int)(threadIdx.x >> 5) + 16 * k;
    const bool in = p >= 0 && p < d.nz && gx >= 0 && gy >= 0 && gx < d.nx && gy < d.ny;
    const long long g = in ? ix(d, gx, gy, p) : 0;
    P.c[k] = in ? F.code[g] : 0;
    P.r[k] = in ? res[g] : 0.f;
    P.a[k] = (in && F.a0f) ? F.a0f[g] : 0.f;
    if (UP) P.xd[k] = in ? F.xd[g] : 0.f;
  }
}

__device__ __forceinline__ float scaled_b(int c, float r) { return (c & kMgTrivial) ? r * kTrivialScale : r; }

// stage A: the plane into the ring; x is the colour-0 value from the zero
// guess (down) or x + I * x[1] (up, from the two coarse planes in cx)
template <bool IS3D, bool UP>
__device__ __forceinline__ void stage0_a(Ring0& R, const Plane0& P, bool hasA0f, int ox, int oy, int p, int cx0, int cy0,
                                         const float (*cx)[kRY / 2 + 1][kRX / 2 + 1]) {
  const int sl = ring0(p);
  const int lx = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int row = (threadIdx.x >> 5) + 16 * k;
    const int c = P.c[k];
    const bool act = (c & kMgActive) != 0;
    const float diag = hasA0f ? P.a[k] : ((c & kMgTrivial) ? kTrivialScale : (float)(c & 7));
    const float r = act ? P.r[k] : 0.f;
    float x = 0.f;
    if (!UP) {
      if (((ox + lx + oy + row + p) & 1) == 0 && act) x = scaled_b(c, r) / diag;
    } else {
      x = P.xd[k];
      if (act) {
        const int vx = ox + lx, vy = oy + row, vz = p;
        const int hx = vx & 1, hy = vy & 1, hz = vz & 1;  // two parents along odd axes
        const int bx = vx / 2 - cx0, by = vy / 2 - cy0;
        float sum = 0.f;
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int ax = j & 1, ay = (j >> 1) & 1, az = j >> 2;
          if (ax <= hx && ay <= hy && az <= hz) sum = sum + cx[(vz / 2 + az) & 1][by + ay][bx + ax];
        }
        x = x + inv_pow2(hx + hy + hz) * sum;
      }
    }
    R.code[sl][row][lx] = (uint16_t)c;
    R.res[sl][row][lx] = r;
    R.diag[sl][row][lx] = diag;
    R.x[sl][row][lx] = x;
  }
}

// the linked neighbours' terms in the kLow/kHigh order of the reference's
// sums (knSmoothColor, knCalcResidual: sum -= A * x[N]).  Poisson links
// have A = -1, so the term is an exact addition; with fractions (FRAC) the
// stored entries of cell g's pairs are read at L2 and the product
// subtracted.  Unlinked pairs have zero entries and are left out.
template <bool IS3D, bool FRAC>
__device__ __forceinline__ float add_links0(const Ring0& R, const Lev0& F, long long g, int c, int q, int row, int lx,
                                            float sum) {
  const int sl = ring0(q);
  if (FRAC) {
    if (c & kLowX) sum = sum - F.ai[g - 1] * R.x[sl][row][lx - 1];
    if (c & kHighX) sum = sum - F.ai[g] * R.x[sl][row][lx + 1];
    if (c & kLowY) sum = sum - F.aj[g - F.d.sy] * R.x[sl][row - 1][lx];
    if (c & kHighY) sum = sum - F.aj[g] * R.x[sl][row + 1][lx];
    if (IS3D) {
      if (c & kLowZ) sum = sum - F.ak[g - F.d.sz] * R.x[ring0(q - 1)][row][lx];
      if (c & kHighZ) sum = sum - F.ak[g] * R.x[ring0(q + 1)][row][lx];
    }
    return sum;
  }
  if (c & kLowX) sum = sum + R.x[sl][row][lx - 1];
  if (c & kHighX) sum = sum + R.x[sl][row][lx + 1];
  if (c & kLowY) sum = sum + R.x[sl][row - 1][lx];
  if (c & kHighY) sum = sum + R.x[sl][row + 1][lx];
  if (IS3D) {
    if (c & kLowZ) sum = sum + R.x[ring0(q - 1)][row][lx];
    if (c & kHighZ) sum = sum + R.x[ring0(q + 1)][row][lx];
  }
  return sum;
}

// stage B: colour 1 on plane q (reads colour-0 values only).  A region row
// holds 16 colour-1 cells: thread t takes cell t & 15 of row t >> 4, so no
// lane idles on colour 0.  A cell on the region's outer ring is left out
// where the grid goes on beyond the ring (its neighbour there is not in the
// region); where the grid ends at the ring, the cell has no link across it
// and is computed.
template <bool IS3D, bool FRAC>
__device__ __forceinline__ void stage0_b(Ring0& R, const Lev0& F, int ox, int oy, int q) {
  const int t = threadIdx.x;
  const int row = t >> 4;
  const int lx = ((1 + ox + oy + row + q) & 1) + 2 * (t & 15);
  if ((lx == 0 && ox > 0) || (lx == kRX - 1 && ox + kRX < F.d.nx) || (row == 0 && oy > 0) ||
      (row == kRY - 1 && oy + kRY < F.d.ny))
    return;
  const int sl = ring0(q);
  const int c = R.code[sl][row][lx];
  if (!(c & kMgActive)) return;
  // an active cell lies inside the grid
  const long long g = FRAC ? ix(F.d, ox + lx, oy + row, q) : 0;
  R.x[sl][row][lx] = add_links0<IS3D, FRAC>(R, F, g, c, q, row, lx, scaled_b(c, R.res[sl][row][lx])) / R.diag[sl][row][lx];
}

// V-cycle entry on level 0: colour 0 from x = 0, colour 1, then the
// residual (knSmoothColor x2 + knCalcResidual); writes x (to F.xd) and r of
// the owned cells
template <bool IS3D, bool FRAC>
__global__ void __launch_bounds__(kT0, 2) k_mg0_down(Lev0 F, const float* __restrict__ res, int zc, const CgScalars* sc) {
  if (sc->done) return;
  extern __shared__ __align__(16) unsigned char t0_smem[];
  Ring0& R = *reinterpret_cast<Ring0*>(t0_smem);
  const Dims& d = F.d;
  constexpr int ZH = IS3D ? 1 : 0;
  const int ox = blockIdx.x * kTX, oy = blockIdx.y * kTY;
  const int xlo = owned_lo(ox), xhi = owned_hi(ox, d.nx, kRX), ylo = owned_lo(oy), yhi = owned_hi(oy, d.ny, kRY);
  const int zb = IS3D ? blockIdx.z * zc : 0, ze = IS3D ? min(zb + zc, d.nz) : 1;
  const int pbeg = zb - 2 * ZH, pend = ze - 1 + 2 * ZH;
  const bool hasA0f = F.a0f != nullptr;
  const int lx = threadIdx.x & 31;
  Plane0 P;
  load_plane0<false>(F, res, ox, oy, pbeg, P);
  for (int p = pbeg; p <= pend; p++) {
    stage0_a<IS3D, false>(R, P, hasA0f, ox, oy, p, 0, 0, nullptr);
    if (p < pend) load_plane0<false>(F, res, ox, oy, p + 1, P);
    __syncthreads();
    const int q = p - ZH;
    if (q >= zb - ZH && q <= ze - 1 + ZH) stage0_b<IS3D, FRAC>(R, F, ox, oy, q);
    __syncthreads();
    // stage C: residual and x of the owned cells of plane s
    const int s = p - 2 * ZH;
    if (s >= zb && s < ze) {
      const int sl = ring0(s);
      const int gx = ox + lx;
#pragma unroll
      for (int k = 0; k < 2; k++) {
        const int row = (threadIdx.x >> 5) + 16 * k;
        const int gy = oy + row;
        if (lx < xlo || lx >= xhi || row < ylo || row >= yhi || gx >= d.nx || gy >= d.ny) continue;
        const long long g = ix(d, gx, gy, s);
        const int c = R.code[sl][row][lx];
        const float xv = R.x[sl][row][lx];
        F.xd[g] = xv;
        if (!(c & kMgActive)) continue;
        float sum = add_links0<IS3D, FRAC>(R, F, g, c, s, row, lx, scaled_b(c, R.res[sl][row][lx]));
        sum = sum - R.diag[sl][row][lx] * xv;
        F.r[g] = sum;
      }
    }
  }
}

// V-cycle exit on level 0: interpolation from level 1 added to x
// (knInterpolate + knAddAssign), colour 1, colour 0, then (unless init)
// sigmaNew = dot(x, residual) and beta like GridCg::iterate.  It reads x
// from F.xd, halo included, and writes the result to x0: reading and writing
// one array would race with the neighbouring CTAs' writes.
template <bool IS3D, bool DOT, bool FRAC>
__global__ void __launch_bounds__(kT0, 2) k_mg0_up(Lev0 F, const float* __restrict__ res, int zc, float* x0, Lev C,
                                                   double* part, CgScalars* sc) {
  if (sc->done) return;
  constexpr int CX = kRX / 2 + 1, CY = kRY / 2 + 1;
  extern __shared__ __align__(16) unsigned char t0_smem[];
  Ring0& R = *reinterpret_cast<Ring0*>(t0_smem);
  __shared__ float scx[2][CY][CX];  // level-1 parents of the region, two coarse planes
  const Dims& d = F.d;
  constexpr int ZH = IS3D ? 1 : 0;
  const int ox = blockIdx.x * kTX, oy = blockIdx.y * kTY;
  const int xlo = owned_lo(ox), xhi = owned_hi(ox, d.nx, kRX), ylo = owned_lo(oy), yhi = owned_hi(oy, d.ny, kRY);
  const int zb = IS3D ? blockIdx.z * zc : 0, ze = IS3D ? min(zb + zc, d.nz) : 1;
  const int pbeg = zb - 2 * ZH, pend = ze - 1 + 2 * ZH;  // pbeg is even
  const bool hasA0f = F.a0f != nullptr;
  const int lx = threadIdx.x & 31;
  // coarse parents of the region: level-1 vertices (cx0 .. cx0 + CX - 1) x
  // (cy0 .. cy0 + CY - 1) of coarse plane cz, one per thread
  const int cx0 = ox >> 1, cy0 = oy >> 1;
  const int cq = threadIdx.x;
  const int cax = cx0 + cq % CX, cay = cy0 + cq / CX;
  auto coarse = [&](int cz) -> float {
    const bool in = cq < CX * CY && cz >= 0 && cz < C.sz && cax >= 0 && cay >= 0 && cax < C.sx && cay < C.sy;
    return in ? C.x[lin(C, cax, cay, cz)] : 0.f;
  };
  if (cq < CX * CY) scx[(pbeg / 2 + 8) & 1][cq / CX][cq % CX] = coarse(pbeg / 2);
  Plane0 P;
  load_plane0<true>(F, res, ox, oy, pbeg, P);
  FSum acc;
  __syncthreads();
  for (int p = pbeg; p <= pend; p++) {
    // coarse plane p/2 + 1 is first read at fine plane p + 1; its slot held
    // coarse plane p/2 - 1, last read at fine plane p - 1.  It is loaded
    // here and stored after stage B.
    const bool even = ((p + 8) & 1) == 0;
    const float cnext = even ? coarse(p / 2 + 1) : 0.f;
    stage0_a<IS3D, true>(R, P, hasA0f, ox, oy, p, cx0, cy0, scx);
    if (p < pend) load_plane0<true>(F, res, ox, oy, p + 1, P);
    __syncthreads();
    const int q = p - ZH;
    if (q >= zb - ZH && q <= ze - 1 + ZH) stage0_b<IS3D, FRAC>(R, F, ox, oy, q);
    if (even && cq < CX * CY) scx[(p / 2 + 1 + 8) & 1][cq / CX][cq % CX] = cnext;
    __syncthreads();
    // stage C: colour 0 of the owned cells of plane s (reads colour-1
    // values only), store, dot
    const int s = p - 2 * ZH;
    if (s >= zb && s < ze) {
      const int sl = ring0(s);
      const int gx = ox + lx;
#pragma unroll
      for (int k = 0; k < 2; k++) {
        const int row = (threadIdx.x >> 5) + 16 * k;
        const int gy = oy + row;
        if (lx < xlo || lx >= xhi || row < ylo || row >= yhi || gx >= d.nx || gy >= d.ny) continue;
        const long long g = ix(d, gx, gy, s);
        const int c = R.code[sl][row][lx];
        float v = R.x[sl][row][lx];
        if (((gx + gy + s) & 1) == 0 && (c & kMgActive))
          v = add_links0<IS3D, FRAC>(R, F, g, c, s, row, lx, scaled_b(c, R.res[sl][row][lx])) / R.diag[sl][row][lx];
        x0[g] = v;
        if (DOT) acc.add(v * R.res[sl][row][lx]);  // inactive cells: x = 0
      }
    }
  }
  if (!DOT) return;
  const double bsum = block_sum(acc.value());
  const unsigned int nblk = gridDim.x * gridDim.y * gridDim.z;
  const unsigned int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  if (threadIdx.x == 0) part[bid] = bsum;
  if (last_block(&sc->counters[4], nblk)) {
    const double s = sum_partials(part, nblk);
    if (threadIdx.x != 0) return;
    const float sigmaNew = (float)s;
    sc->beta = sigmaNew / sc->sigma;
    sc->sigma = sigmaNew;
    if (!(sc->resNorm < 1e35f)) {
      sc->status = 2;
      sc->done = 1;
    }
  }
}

// ---- coarsest level: GridMg::solveCG in double-float arithmetic
// GB300 executes FP64 at a small fraction of its FP32 rate, and a CG on
// <= 1000 unknowns is latency bound, so the vectors and dot products use
// unevaluated float pairs (h + l, 48-bit significand: Dekker's exact
// product via FMA and Knuth's exact two-sum) and only the per-iteration
// scalars (alpha, beta, the residual ratio) are formed in double, once per
// CTA.  The iterates agree with an IEEE-double CG to ~1e-14 relative, far
// below the float resolution of the result; the stopping rule, iteration
// limit and order of operations are the reference's.
// CTA sum of NV pairs per thread in a fixed order; the sums are valid in
// thread 0 after the call (the caller publishes derived scalars)
template <int NV>
__device__ __forceinline__ void cta_sum_ff(ff* v, ff (*red)[32]) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; q++) v[q] = warp_sum_ff(v[q]);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; q++) red[q][wid] = v[q];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) {
      ff t = lane < nw ? red[q][lane] : ff{0.f, 0.f};
      v[q] = warp_sum_ff(t);
    }
  }
}

constexpr int kCgNb = 27;  // stencil entries per vertex (level 0: 7)

// GridMg::solveCG on the coarsest level, one CTA, one vertex per thread.
// The stencil of each vertex (coefficients in applyAStencil's order and the
// neighbours' indices) is gathered once into shared memory.
template <bool IS3D, bool L0>
__global__ void __launch_bounds__(kCgThreads) k_mg_coarse_cg(Lev L, Lev0 F, const float* __restrict__ res, float* x0, int S,
                                                             float accuracy, const CgScalars* sc) {
  if (sc->done) return;
  extern __shared__ __align__(16) unsigned char cg_smem[];
  float* coef = (float*)cg_smem;                                  // [kCgNb][kCgThreads]
  short* nbr = (short*)(cg_smem + kCgNb * kCgThreads * sizeof(float));  // [kCgNb][kCgThreads]
  __shared__ float sph[kCgThreads], spl[kCgThreads];
  __shared__ ff red[2][32];
  __shared__ double bc[4];
  __shared__ int stop;
  const int n = L0 ? (int)F.d.n : (int)L.n;
  const int v = threadIdx.x;
  bool act = false;
  float diag = 1.f, bv = 0.f;
  int nn = 0;
  if (v < n) {
    if (L0) {
      const int c = F.code[v];
      act = (c & kMgActive) != 0;
      if (act) {
        diag = l0_diag(c, F.a0f, v);
        bv = l0_rhs(c, res, v);
        const Dims& d = F.d;
        const int lo[3] = {kLowX, kLowY, kLowZ}, hi[3] = {kHighX, kHighY, kHighZ};
        const long long st[3] = {1, d.sy, d.sz};
        const float* st3[3] = {F.ai, F.aj, F.ak};  // stored entries (fractions) or null
        for (int q = 0; q < (IS3D ? 3 : 2); q++) {
          if (c & lo[q]) {
            coef[nn * kCgThreads + v] = F.ai ? st3[q][v - st[q]] : -1.f;
            nbr[nn * kCgThreads + v] = (short)(v - st[q]);
            nn++;
          }
          if (c & hi[q]) {
            coef[nn * kCgThreads + v] = F.ai ? st3[q][v] : -1.f;
            nbr[nn * kCgThreads + v] = (short)(v + st[q]);
            nn++;
          }
        }
        coef[nn * kCgThreads + v] = diag;
        nbr[nn * kCgThreads + v] = (short)v;
        nn++;
      }
    } else {
      act = L.type[v] != kVtInactive;
      if (act) {
        diag = L.A[v];
        bv = L.b[v];
        constexpr int ZL = IS3D ? -1 : 0, ZH = IS3D ? 1 : 0;
        int vx, vy, vz;
        coords(L, v, vx, vy, vz);
        int s = 0;
        for (int dz = ZL; dz <= ZH; dz++)
          for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++, s++) {
              const int nx = vx + dx, ny = vy + dy, nz = vz + dz;
              if (!inside(L, nx, ny, nz)) continue;
              const int q = (int)lin(L, nx, ny, nz);
              if (L.type[q] == kVtInactive) continue;
              coef[nn * kCgThreads + v] =
                  s < S ? L.A[(long long)(S - 1 - s) * L.n + q] : L.A[(long long)(s - S + 1) * L.n + v];
              nbr[nn * kCgThreads + v] = (short)q;
              nn++;
            }
      }
    }
  }
  // x = mx[l] = 0, so r = b - A*0 = b
  ff x{0.f, 0.f}, r{0.f, 0.f}, z{0.f, 0.f}, p{0.f, 0.f};
  if (act) {
    r = ff{bv, 0.f};
    z = ff_div_f(r, diag);
    p = z;
  }
  sph[v] = p.h;
  spl[v] = p.l;
  {
    ff t[2] = {ff_mul(r, r), ff_mul(r, z)};
    cta_sum_ff<2>(t, red);
    if (v == 0) {
      bc[0] = sqrt(ff_d(t[0]));  // initialResidual
      bc[1] = ff_d(t[1]);        // alphaTop
    }
    __syncthreads();
  }
  const double initialResidual = bc[0];
  double alphaTop = bc[1];  // meaningful in thread 0
  for (int iter = 0; iter < 10000 && initialResidual > 1E-12; iter++) {
    ff q{0.f, 0.f};
    for (int e = 0; e < nn; e++) {
      const int k = nbr[e * kCgThreads + v];
      q = ff_add(q, ff_mul_f(ff{sph[k], spl[k]}, coef[e * kCgThreads + v]));
    }
    {
      ff t[1] = {act ? ff_mul(p, q) : ff{0.f, 0.f}};
      cta_sum_ff<1>(t, red);
      if (v == 0) bc[2] = alphaTop / ff_d(t[0]);  // alpha
      __syncthreads();
    }
    const ff alpha = d_ff(bc[2]);
    ff t[2] = {ff{0.f, 0.f}, ff{0.f, 0.f}};
    if (act) {
      x = ff_add(x, ff_mul(alpha, p));
      r = ff_add(r, ff_neg(ff_mul(alpha, q)));
      z = ff_div_f(r, diag);
      t[0] = ff_mul(r, r);
      t[1] = ff_mul(r, z);
    }
    cta_sum_ff<2>(t, red);
    if (v == 0) {
      const double residual = sqrt(ff_d(t[0]));
      const double atn = ff_d(t[1]);
      stop = residual / initialResidual < (double)accuracy;
      bc[3] = atn / alphaTop;  // beta
      alphaTop = atn;
    }
    __syncthreads();
    if (stop) break;
    p = ff_add(z, ff_mul(d_ff(bc[3]), p));
    sph[v] = p.h;
    spl[v] = p.l;
    __syncthreads();
  }
  if (v < n) {
    const float xf = (float)ff_d(x);
    if (L0) x0[v] = xf;
    else L.x[v] = xf;
  }
}
constexpr size_t kCgDynSmem = (size_t)kCgNb * kCgThreads * (sizeof(float) + sizeof(short));

// ---- the coarse end of the V-cycle in one launch: one thread-block
// cluster (16 CTAs, 8 where 16 cannot be co-scheduled) runs the levels from
// `first` down, the coarsest-level CG and the levels back up.  The colour
// passes of these levels have a few thousand to a few hundred thousand
// vertices; as separate launches each costs a launch and a cold pipeline,
// here a hardware cluster barrier.  Every pass does the per-vertex float
// operations of the separate kernels above (the same device functions), so
// the levels' results are bit-identical to them; vectors written inside
// the launch are read at L2 (ldv<true>).
constexpr int kTailThreads = 384;
constexpr int kTailMaxCta = 16;
constexpr int kTailVpc = 128;  // coarsest-level vertices per CTA (<= 1024 over >= 8 CTAs)
constexpr long long kTailSlots = 100000;  // largest level run inside the cluster (33^3 and below)

struct TailSmem {
  float coef[kCgNb][kTailVpc];  // own vertices' stencils (applyAStencil order)
  short nbr[kCgNb][kTailVpc];
  unsigned char nn[kTailVpc];
  float ph[kCgThreads], pl[kCgThreads];  // the whole search vector p
  float zh[kCgThreads], zl[kCgThreads];  // the whole z: every CTA stores its share into every CTA
  ff wpart[kTailThreads / 32][2];        // per-warp partial dot products
  ff cpart[kTailMaxCta][3];              // per-CTA partials (rr, rz | pq), stored by each CTA into every CTA
};

// f1 < f2 for normalised pairs
__device__ __forceinline__ bool ff_lt(ff a, ff b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
// a / b for pairs (long division: a float quotient and a correction)
__device__ __forceinline__ ff ff_div(ff a, ff b) {
  const float q1 = a.h / b.h;
  const ff r = ff_add(a, ff_neg(ff_mul(b, ff{q1, 0.f})));
  const float q2 = r.h / b.h;
  return quick_two_sum(q1, q2);
}

// The CTA's sums of NV pairs held by the lanes with sub == 0 (zero
// elsewhere), stored into cpart[rank][slot..] of every CTA of the cluster;
// the caller's cluster barrier publishes them.  The pq slot is apart from
// the rr / rz slots: a CTA may store the next phase's sums while another
// still reads this phase's.
template <int NV>
__device__ __forceinline__ void tail_push_sums(cooperative_groups::cluster_group& cl, TailSmem& sm, ff* v, int tpv,
                                               int slot) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o >= tpv; o >>= 1)
#pragma unroll
    for (int q = 0; q < NV; q++) {
      const ff w{__shfl_xor_sync(0xffffffffu, v[q].h, o), __shfl_xor_sync(0xffffffffu, v[q].l, o)};
      v[q] = ff_add(v[q], w);
    }
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; q++) sm.wpart[wid][q] = v[q];
  __syncthreads();
  if (wid == 0) {
    const int ncta = (int)cl.num_blocks(), rank = (int)cl.block_rank();
#pragma unroll
    for (int q = 0; q < NV; q++) {
      ff t = lane < nw ? sm.wpart[lane][q] : ff{0.f, 0.f};
      for (int o = 16; o > 0; o >>= 1) {
        const ff w{__shfl_xor_sync(0xffffffffu, t.h, o), __shfl_xor_sync(0xffffffffu, t.l, o)};
        t = ff_add(t, w);
      }
      if (lane < ncta) *cl.map_shared_rank(&sm.cpart[rank][slot + q], lane) = t;
    }
  }
}

// after the cluster barrier: the cluster's sum of cpart[.][q], summed in
// the same order in every warp of every CTA (identical bits everywhere)
__device__ __forceinline__ ff tail_total(const TailSmem& sm, int q, int ncta) {
  const int lane = threadIdx.x & 31;
  ff t = lane < ncta ? sm.cpart[lane][q] : ff{0.f, 0.f};
  for (int o = 16; o > 0; o >>= 1) {
    const ff w{__shfl_xor_sync(0xffffffffu, t.h, o), __shfl_xor_sync(0xffffffffu, t.l, o)};
    t = ff_add(t, w);
  }
  return t;
}

// this CTA's z values into zh/zl of every CTA (the tpv lanes of a vertex
// hold the same z and share its stores)
__device__ __forceinline__ void tail_push_z(cooperative_groups::cluster_group& cl, TailSmem& sm, bool own, int v, int sub,
                                            int tpv, ff z) {
  if (!own) return;
  const int ncta = (int)cl.num_blocks();
  for (int rk = sub; rk < ncta; rk += tpv) {
    *cl.map_shared_rank(&sm.zh[v], rk) = z.h;
    *cl.map_shared_rank(&sm.zl[v], rk) = z.l;
  }
}

// GridMg::solveCG (multigrid.cpp:793-902) on the coarsest level across the
// cluster: CTA c owns vertices [c*vpc, (c+1)*vpc), tpv threads per vertex
// split its stencil.  Each CTA stores its partial dot products and its z
// values into the shared memory of every CTA before a cluster barrier, so
// every CTA then holds the whole z (and rebuilds the whole p) and all
// partials; an iteration has two barriers and no remote loads.  Vectors,
// dot products and scalars are double-float pairs on the FP32 pipe (the
// stencil product is a compensated sum of exact float products); the
// iterates follow an IEEE-double CG to ~1e-14 relative.  Every warp forms
// the scalars from the same rank-ordered sums, so all CTAs take the same
// branches.
template <bool IS3D>
__device__ void tail_coarse_cg(cooperative_groups::cluster_group& cl, const Lev& L, int S, float accuracy, TailSmem& sm) {
  const int ncta = (int)cl.num_blocks(), rank = (int)cl.block_rank();
  const int n = (int)L.n;
  const int vpc = (n + ncta - 1) / ncta;
  int tpv = 8;
  while (tpv > 1 && tpv * vpc > (int)blockDim.x) tpv >>= 1;
  const int lv = threadIdx.x / tpv, sub = threadIdx.x % tpv;
  const int v = rank * vpc + lv;
  const bool own = lv < vpc && v < n;
  bool act = false;
  float diag = 1.f, bv = 0.f;
  if (own) {
    act = L.type[v] != kVtInactive;
    if (act) {
      diag = L.A[v];
      bv = __ldcg(&L.b[v]);
    }
    if (sub == 0) {
      int nn = 0;
      if (act) {
        constexpr int ZL = IS3D ? -1 : 0, ZH = IS3D ? 1 : 0;
        int vx, vy, vz;
        coords(L, v, vx, vy, vz);
        int s = 0;
        for (int dz = ZL; dz <= ZH; dz++)
          for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++, s++) {
              const int nx = vx + dx, ny = vy + dy, nz = vz + dz;
              if (!inside(L, nx, ny, nz)) continue;
              const int q = (int)lin(L, nx, ny, nz);
              if (L.type[q] == kVtInactive) continue;
              sm.coef[nn][lv] = s < S ? L.A[(long long)(S - 1 - s) * L.n + q] : L.A[(long long)(s - S + 1) * L.n + v];
              sm.nbr[nn][lv] = (short)q;
              nn++;
            }
      }
      sm.nn[lv] = (unsigned char)nn;
    }
  }
  const bool lead = act && sub == 0;
  // x = 0, so r = b - A*0 = b
  ff x{0.f, 0.f}, r{0.f, 0.f}, z{0.f, 0.f};
  if (act) {
    r = ff{bv, 0.f};
    z = ff_div_f(r, diag);
  }
  tail_push_z(cl, sm, own, v, sub, tpv, z);
  {
    ff t[2] = {lead ? ff_mul(r, r) : ff{0.f, 0.f}, lead ? ff_mul(r, z) : ff{0.f, 0.f}};
    tail_push_sums<2>(cl, sm, t, tpv, 0);
  }
  cl.sync();
  const ff rr0 = tail_total(sm, 0, ncta);
  ff alphaTop = tail_total(sm, 1, ncta);
  // residual / initialResidual < accuracy  <=>  rr < rr0 * accuracy^2
  const ff stopAt = ff_mul(rr0, two_prod(accuracy, accuracy));
  for (int u = threadIdx.x; u < n; u += blockDim.x) {  // p = z
    sm.ph[u] = sm.zh[u];
    sm.pl[u] = sm.zl[u];
  }
  __syncthreads();
  const int nn = own ? sm.nn[lv] : 0;
  // initialResidual > 1e-12
  for (int iter = 0; iter < 10000 && rr0.h > 1e-24f; iter++) {
    // q = A p: this lane's share of the stencil as a compensated sum, then
    // the vertex's lanes
    float qs = 0.f, qe = 0.f;
    for (int e = sub; e < nn; e += tpv) {
      const int k = sm.nbr[e][lv];
      const float c = sm.coef[e][lv];
      const ff pr = two_prod(c, sm.ph[k]);
      const ff t = two_sum(qs, pr.h);
      qs = t.h;
      qe = qe + (t.l + (pr.l + c * sm.pl[k]));
    }
    ff q = two_sum(qs, qe);
    for (int o = tpv >> 1; o > 0; o >>= 1) {
      const ff w{__shfl_xor_sync(0xffffffffu, q.h, o), __shfl_xor_sync(0xffffffffu, q.l, o)};
      q = ff_add(q, w);
    }
    const ff p = own ? ff{sm.ph[v], sm.pl[v]} : ff{0.f, 0.f};
    {
      ff t[1] = {lead ? ff_mul(p, q) : ff{0.f, 0.f}};
      tail_push_sums<1>(cl, sm, t, tpv, 2);
    }
    cl.sync();
    const ff alpha = ff_div(alphaTop, tail_total(sm, 2, ncta));
    ff t[2] = {ff{0.f, 0.f}, ff{0.f, 0.f}};
    if (act) {
      x = ff_add(x, ff_mul(alpha, p));
      r = ff_add(r, ff_neg(ff_mul(alpha, q)));
      z = ff_div_f(r, diag);
      if (sub == 0) {
        t[0] = ff_mul(r, r);
        t[1] = ff_mul(r, z);
      }
    }
    tail_push_z(cl, sm, own, v, sub, tpv, z);
    tail_push_sums<2>(cl, sm, t, tpv, 0);
    cl.sync();
    const ff rr = tail_total(sm, 0, ncta);
    const ff atn = tail_total(sm, 1, ncta);
    if (ff_lt(rr, stopAt)) break;
    const ff beta = ff_div(atn, alphaTop);
    alphaTop = atn;
    for (int u = threadIdx.x; u < n; u += blockDim.x) {
      const ff pu = ff_add(ff{sm.zh[u], sm.zl[u]}, ff_mul(beta, ff{sm.ph[u], sm.pl[u]}));
      sm.ph[u] = pu.h;
      sm.pl[u] = pu.l;
    }
    __syncthreads();
  }
  if (own && sub == 0) L.x[v] = x.h + x.l;
}

template <bool IS3D>
__global__ void __launch_bounds__(kTailThreads, 1) k_mg_tail(const Lev* __restrict__ levs, int first, int last, int S,
                                                             float accuracy, const CgScalars* sc) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  if (sc->done) return;  // the same for every CTA of the cluster
  __shared__ TailSmem sm;
  const long long T = (long long)cl.num_blocks() * blockDim.x;
  const long long t0 = (long long)cl.block_rank() * blockDim.x + threadIdx.x;
  constexpr int ncol = IS3D ? 8 : 4;
  for (int l = first; l < last; l++) {
    const Lev L = levs[l];
    const int bx = (L.sx + 1) / 2, by = (L.sy + 1) / 2;
    const long long nb = (long long)bx * by * ((L.sz + 1) / 2);
    for (int c = 0; c < ncol; c++) {
      if (L.sid)
        for (long long bi = t0; bi < nb; bi += T) smooth_vertex_dict_flat<IS3D>(L, bi, c & 1, (c >> 1) & 1, c >> 2, bx, by);
      else
        for (long long bi = t0; bi < nb; bi += T) smooth_vertex_flat<IS3D>(L, bi, c & 1, (c >> 1) & 1, c >> 2, bx, by);
      cl.sync();
    }
    if (L.sid)
      for (long long v = t0; v < L.n; v += T) residual_vertex_dict_flat<IS3D>(L, v);
    else
      for (long long v = t0; v < L.n; v += T) residual_vertex_flat<IS3D>(L, v);
    cl.sync();
    const Lev D = levs[l + 1];
    for (long long v = t0; v < D.n; v += T) restrict_vertex<false, true>(D, L, Lev0{}, v);
    cl.sync();
  }
  tail_coarse_cg<IS3D>(cl, levs[last], S, accuracy, sm);
  cl.sync();  // x of the coarsest level written; no CTA reads another's shared memory any more
  for (int l = last - 1; l >= first; l--) {
    const Lev D = levs[l], Sv = levs[l + 1];
    for (long long v = t0; v < D.n; v += T) interp_vertex<IS3D, true>(D, Sv, v);
    cl.sync();
    const int bx = (D.sx + 1) / 2, by = (D.sy + 1) / 2;
    const long long nb = (long long)bx * by * ((D.sz + 1) / 2);
    for (int c = ncol - 1; c >= 0; c--) {
      if (D.sid)
        for (long long bi = t0; bi < nb; bi += T) smooth_vertex_dict_flat<IS3D>(D, bi, c & 1, (c >> 1) & 1, c >> 2, bx, by);
      else
        for (long long bi = t0; bi < nb; bi += T) smooth_vertex_flat<IS3D>(D, bi, c & 1, (c >> 1) & 1, c >> 2, bx, by);
      cl.sync();
    }
  }
}

// sigmaNew = dot(tmp, residual) and beta (GridCg::iterate after the
// preconditioner, conjugategrad.cpp:277-299)
__global__ void __launch_bounds__(256) k_mg_dot_beta(long long n, const float* __restrict__ t, const float* __restrict__ r,
                                                     double* part, CgScalars* sc) {
  if (sc->done) return;
  FSum acc;
  GRID_STRIDE(idx, n) acc.add(t[idx] * r[idx]);
  const double b = block_sum(acc.value());
  if (threadIdx.x == 0) part[blockIdx.x] = b;
  if (last_block(&sc->counters[4], gridDim.x)) {
    const double s = sum_partials(part, gridDim.x);
    if (threadIdx.x != 0) return;
    const float sigmaNew = (float)s;
    sc->beta = sigmaNew / sc->sigma;
    sc->sigma = sigmaNew;
    if (!(sc->resNorm < 1e35f)) {
      sc->status = 2;
      sc->done = 1;
    }
  }
}

// ------------------------------------------------------------- host side
// The reference's precomputed coarsening paths (GridMg ctor,
// multigrid.cpp:285-318) around the coarse vertex V = (1,1,1), sorted by
// coarse entry and fine vertex.
void build_paths(int dim, std::vector<Path>& out) {
  static const int p7[7][3] = {{0, 0, 0}, {-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
  const int smin[3] = {-1, -1, dim == 3 ? -1 : 0}, smax[3] = {1, 1, dim == 3 ? 1 : 0};
  const int V[3] = {1, 1, 1};
  struct Tmp {
    Path p;
    int key;
  };
  std::vector<Tmp> t;
  int U[3];
  for (U[2] = 2 * V[2] + smin[2]; U[2] <= 2 * V[2] + smax[2]; U[2]++)
    for (U[1] = 2 * V[1] + smin[1]; U[1] <= 2 * V[1] + smax[1]; U[1]++)
      for (U[0] = 2 * V[0] + smin[0]; U[0] <= 2 * V[0] + smax[0]; U[0]++)
        for (int i = 0; i < 1 + 2 * dim; i++) {
          const int W[3] = {U[0] + p7[i][0], U[1] + p7[i][1], U[2] + p7[i][2]};
          int N[3];
          for (N[2] = W[2] / 2; N[2] <= (W[2] + 1) / 2; N[2]++)
            for (N[1] = W[1] / 2; N[1] <= (W[1] + 1) / 2; N[1]++)
              for (N[0] = W[0] / 2; N[0] <= (W[0] + 1) / 2; N[0]++) {
                const int s = N[0] + 3 * N[1] + 9 * N[2];
                if (s < 13) continue;
                Tmp e;
                for (int c = 0; c < 3; c++) {
                  e.p.n[c] = (signed char)(N[c] - V[c]);
                  e.p.u[c] = (signed char)(U[c] - 2 * V[c]);
                  e.p.w[c] = (signed char)(W[c] - 2 * V[c]);
                }
                e.p.sc = (signed char)(s - 13);
                e.p.sf = (signed char)((i + 1) / 2);
                e.p.inU = (signed char)(i % 2 == 0);
                e.p.rw = inv_pow2(parity3(U[0], U[1], U[2]));
                e.p.iw = inv_pow2(parity3(W[0], W[1], W[2]));
                e.key = (U[0] - 2 * V[0] + 1) + 3 * (U[1] - 2 * V[1] + 1) + 9 * (U[2] - 2 * V[2] + 1);
                t.push_back(e);
              }
        }
  // std::sort with the reference's comparator (coarse entry, then fine
  // vertex): elements with equal keys keep the order std::sort gives them
  std::sort(t.begin(), t.end(), [](const Tmp& a, const Tmp& b) {
    if (a.p.sc == b.p.sc) return a.key < b.key;
    return a.p.sc < b.p.sc;
  });
  out.clear();
  for (auto& e : t) out.push_back(e.p);
}

int ensure_paths() {
  if (g_pathsReady) return 0;
  for (int dim = 2; dim <= 3; dim++) {
    std::vector<Path> p;
    build_paths(dim, p);
    if ((int)p.size() > kMaxPaths) return 1;
    g_npaths[dim - 2] = (int)p.size();
    if (cudaMemcpyToSymbol(c_paths, p.data(), p.size() * sizeof(Path), (size_t)(dim - 2) * kMaxPaths * sizeof(Path)) !=
        cudaSuccess)
      return 1;
  }
  const int dyn = (int)kCgDynSmem;
  if (cudaFuncSetAttribute(k_mg_coarse_cg<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg_coarse_cg<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg_coarse_cg<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg_coarse_cg<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess)
    return 1;
  const int r0 = (int)sizeof(Ring0);
  const auto ring = cudaFuncAttributeMaxDynamicSharedMemorySize;
  if (cudaFuncSetAttribute(k_mg0_down<true, false>, ring, r0) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg0_down<false, false>, ring, r0) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg0_down<true, true>, ring, r0) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg0_down<false, true>, ring, r0) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg0_up<true, true, false>, ring, r0) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg0_up<true, false, false>, ring, r0) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg0_up<false, true, false>, ring, r0) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg0_up<false, false, false>, ring, r0) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg0_up<true, true, true>, ring, r0) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg0_up<true, false, true>, ring, r0) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg0_up<false, true, true>, ring, r0) != cudaSuccess ||
      cudaFuncSetAttribute(k_mg0_up<false, false, true>, ring, r0) != cudaSuccess)
    return 1;
  // the cluster V-cycle tail: 16 CTAs where the GPU can co-schedule them
  g_tailCta = 0;
  if (cudaFuncSetAttribute(k_mg_tail<true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
      cudaFuncSetAttribute(k_mg_tail<false>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
    for (int c = 16; c >= 8 && !g_tailCta; c /= 2) {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = c;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3(c);
      cfg.blockDim = dim3(kTailThreads);
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int nc = 0;
      if (cudaOccupancyMaxActiveClusters(&nc, k_mg_tail<true>, &cfg) == cudaSuccess && nc >= 1) g_tailCta = c;
    }
  }
  cudaGetLastError();  // a GPU without clusters keeps the per-level launches
  g_pathsReady = true;
  return 0;
}

// genCoarseGrid (multigrid.cpp:520-578): every active fine vertex starts
// with the number of coarse vertices it can interpolate from (2^#odd
// coordinates) as key; repeatedly the vertex with the fewest free coarse
// parents is taken, its first free parent becomes a coarse vertex and the
// others are removed, and every fine vertex near a decided parent loses one
// from its key.  Keys are 1..8, held as buckets of doubly linked lists with
// insertion at the head; the next vertex is the head of the lowest non-empty
// bucket -- the order the reference's NKMinHeap yields.
void gen_coarse_grid(const int fs[3], const std::vector<int8_t>& tf, const int cs[3], std::vector<int8_t>& tc) {
  enum : int8_t { kFree = 5, kZero = 4, kRemoved = 3 };
  const long long nf = (long long)fs[0] * fs[1] * fs[2];
  const long long nc = (long long)cs[0] * cs[1] * cs[2];
  const long long fpy = fs[0], fpz = (long long)fs[0] * fs[1];
  const long long cpy = cs[0], cpz = (long long)cs[0] * cs[1];
  tc.assign((size_t)nc, kFree);
  constexpr int kBuckets = 9;
  std::vector<int> key((size_t)nf, -1), prv((size_t)nf), nxt((size_t)nf);
  int head[kBuckets];
  for (int b = 0; b < kBuckets; b++) head[b] = -1;
  int count = 0;
  // node ids: >= 0 vertices; prv == -(b+1) marks the head of bucket b
  auto unlink = [&](int id) {
    const int p = prv[id], q = nxt[id];
    if (p < 0) head[-p - 1] = q;
    else nxt[p] = q;
    if (q >= 0) prv[q] = p;
    count--;
  };
  auto set_key = [&](int id, int k) {
    if (key[id] == k) return;
    if (key[id] != -1) unlink(id);
    key[id] = k;
    if (k == -1) return;
    const int h = head[k];
    prv[id] = -(k + 1);
    nxt[id] = h;
    if (h >= 0) prv[h] = id;
    head[k] = id;
    count++;
  };
  for (long long v = 0; v < nf; v++) {
    if (tf[(size_t)v] == kVtInactive) continue;
    const int x = (int)(v % fs[0]), y = (int)((v / fpy) % fs[1]), z = (int)(v / fpz);
    set_key((int)v, 1 << parity3(x, y, z));
  }
  while (count > 0) {
    int b = 1;
    while (head[b] < 0) b++;
    const int v = head[b];
    unlink(v);
    key[v] = -1;
    const int X = (int)(v % fs[0]), Y = (int)((v / fpy) % fs[1]), Z = (int)(v / fpz);
    bool vdone = false;
    for (int iz = Z / 2; iz <= (Z + 1) / 2; iz++)
      for (int iy = Y / 2; iy <= (Y + 1) / 2; iy++)
        for (int ixx = X / 2; ixx <= (X + 1) / 2; ixx++) {
          const long long i = ixx + cpy * iy + cpz * iz;
          if (tc[(size_t)i] != kFree) continue;
          if (vdone) tc[(size_t)i] = kRemoved;
          else {
            tc[(size_t)i] = kZero;
            vdone = true;
          }
          const int lx = std::max(0, ixx * 2 - 1), hx = std::min(fs[0] - 1, ixx * 2 + 1);
          const int ly = std::max(0, iy * 2 - 1), hy = std::min(fs[1] - 1, iy * 2 + 1);
          const int lz = std::max(0, iz * 2 - 1), hz = std::min(fs[2] - 1, iz * 2 + 1);
          for (int rz = lz; rz <= hz; rz++)
            for (int ry = ly; ry <= hy; ry++)
              for (int rx = lx; rx <= hx; rx++) {
                const int r = (int)(rx + fpy * ry + fpz * rz);
                const int k = key[r];
                if (k > 1) set_key(r, k - 1);
                else if (k > -1) set_key(r, -1);
              }
        }
  }
  for (long long i = 0; i < nc; i++) {
    int8_t& t = tc[(size_t)i];
    t = (t == kZero) ? kVtActive : kVtInactive;
  }
}

int blocks_for(long long n) {
  // one vertex per thread: each thread's loads are then independent of the
  // others' (a grid-stride loop would serialise their memory latency)
  const long long b = (n + kThreads1 - 1) / kThreads1;
  return (int)std::max(1LL, std::min(b, 1LL << 30));
}

}  // namespace

struct MgHierarchy {
  Dims d;
  int nlev = 0, is3d = 0, S = 0;
  int size[kMaxLevels][3];
  Lev lev[kMaxLevels];
  Lev0 l0;
  int8_t* type0 = nullptr;
  std::vector<int8_t> htype[kMaxLevels];   // vertex types, x-fastest
  std::vector<int8_t> upload[kMaxLevels];  // the same in storage order
  std::vector<int8_t> selType0;  // level-0 types the current selection was made for
  bool selValid = false;
  bool isASet = false;
  unsigned long long gen = 0;  // bumped by every rebuild
  bool useA0f = false;  // the snapshot has a float diagonal (ghost fluid, fractions)
  bool useFrac = false;  // the snapshot has stored off-diagonals (fractions)
  MgProfHook hook = nullptr;
  void* hookCtx = nullptr;
  float coarseAcc = 1e-8f;
  Lev* dlev = nullptr;  // lev[] on the device, for the cluster tail
  int tailFirst = 0;    // first level of the cluster tail (0: none)
  int zc = kZC;         // planes per CTA of the level-0 passes
  // stencil dictionaries of the levels run by per-level launches
  uint16_t* dsid[kMaxLevels] = {};
  float* dT[kMaxLevels] = {};
  unsigned long long* dkeys = nullptr;
  int* drep = nullptr;
  int* dslot = nullptr;
  int* dflags = nullptr;  // 3 ints per level
  int ndict[kMaxLevels] = {};  // distinct stencils of the level (0: planes)
  size_t bytes = 0;
  std::vector<void*> allocs;
  bool ok = true;

  template <typename T>
  T* alloc(long long count) {
    void* p = nullptr;
    const size_t nb = sizeof(T) * (size_t)std::max(1LL, count);
    if (cudaMalloc(&p, nb) != cudaSuccess) {
      ok = false;
      return nullptr;
    }
    cudaMemset(p, 0, nb);
    allocs.push_back(p);
    bytes += nb;
    return (T*)p;
  }
};

// planes per CTA of the level-0 passes: the even run length in [16, 64]
// that minimises waves x planes a CTA walks (its run plus the 4-plane halo),
// with two CTAs resident per SM; ties go to the longer run (less halo work).
// At 256^3 (9 x 9 tiles per plane) that is 38 planes: 567 CTAs, 1.9 waves.
static int level0_planes(const Dims& d) {
  if (!d.is3d) return kZC;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      sms <= 0) {
    cudaGetLastError();
    return kZC;
  }
  const long long cols = (long long)level0_tiles(d.nx) * level0_tiles(d.ny);
  const long long slots = 2LL * sms;
  int best = kZC;
  long long bestCost = -1;
  for (int zc = 16; zc <= 64; zc += 2) {
    const long long ctas = cols * ((d.nz + zc - 1) / zc);
    const long long cost = ((ctas + slots - 1) / slots) * (zc + 4);
    if (bestCost < 0 || cost <= bestCost) {
      bestCost = cost;
      best = zc;
    }
  }
  return best;
}

MgHierarchy* mg_hierarchy_create(const Dims& d) {
  if (ensure_paths()) return nullptr;
  MgHierarchy* h = new MgHierarchy();
  h->d = d;
  h->is3d = d.is3d;
  h->S = d.is3d ? 14 : 5;
  // level sizes (GridMg ctor, multigrid.cpp:240-265)
  h->size[0][0] = d.nx;
  h->size[0][1] = d.ny;
  h->size[0][2] = d.nz;
  int L = 1;
  long long n = d.n;
  for (int l = 1; l <= 100 && l < kMaxLevels; l++) {
    if (h->size[l - 1][0] <= 5 && h->size[l - 1][1] <= 5 && h->size[l - 1][2] <= 5) break;
    if (n <= 1000) break;
    for (int c = 0; c < 3; c++) h->size[l][c] = (h->size[l - 1][c] + 2) / 2;
    n = (long long)h->size[l][0] * h->size[l][1] * h->size[l][2];
    L = l + 1;
  }
  h->nlev = L;
  const long long n0 = d.n;
  h->l0.d = d;
  h->l0.code = h->alloc<uint16_t>(n0);
  h->l0.a0f = nullptr;
  h->l0.ai = h->l0.aj = h->l0.ak = nullptr;
  h->l0.r = L > 1 ? h->alloc<float>(n0) : nullptr;
  h->l0.xd = L > 1 ? h->alloc<float>(n0) : nullptr;
  h->type0 = h->alloc<int8_t>(n0);
  for (int l = 1; l < L; l++) {
    Lev& v = h->lev[l];
    v.sx = h->size[l][0];
    v.sy = h->size[l][1];
    v.sz = h->size[l][2];
    v.py = v.sx;
    v.pz = (long long)v.sx * v.sy;
    v.colored = l < L - 1;
    v.bx = (v.sx + 1) / 2;
    v.by = (v.sy + 1) / 2;
    v.nb = (long long)v.bx * v.by * ((v.sz + 1) / 2);
    v.n = v.colored ? v.nb * (d.is3d ? 8 : 4) : (long long)v.sx * v.sy * v.sz;
    v.type = h->alloc<int8_t>(v.n);
    v.A = h->alloc<float>(v.n * h->S);
    v.x = h->alloc<float>(v.n);
    v.b = h->alloc<float>(v.n);
    v.r = h->alloc<float>(v.n);
  }
  const long long nc = L > 1 ? h->lev[L - 1].n : n0;
  if (nc > kCgThreads) h->ok = false;  // the level loop guarantees <= 1000
  h->zc = level0_planes(d);
  if (const char* e = std::getenv("MANTAGPU_MG0_PLANES")) h->zc = std::max(2, std::atoi(e) & ~1);
  // the levels of at most kTailSlots storage slots (and the coarsest) run in
  // one cluster launch
  if (h->ok && L > 1 && g_tailCta && nc <= (long long)g_tailCta * kTailVpc) {
    long long lim = kTailSlots;
    if (const char* e = std::getenv("MANTAGPU_MG_TAIL_SLOTS")) lim = std::atoll(e);
    int f = L - 1;
    while (f > 1 && h->lev[f - 1].n <= lim) f--;
    h->tailFirst = f;
    h->dlev = h->alloc<Lev>(L);
    if (h->ok && cudaMemcpy(h->dlev, h->lev, sizeof(Lev) * (size_t)L, cudaMemcpyHostToDevice) != cudaSuccess) h->ok = false;
  }
  // dictionary buffers for the colour-blocked levels (the cluster tail's too
  // unless MANTAGPU_MG_NO_TAIL_DICT is set)
  if (h->ok && !std::getenv("MANTAGPU_MG_NO_DICT")) {
    bool any = false;
    const bool tailDict = !std::getenv("MANTAGPU_MG_NO_TAIL_DICT");
    for (int l = 1; l < L - 1 && (tailDict || !h->tailFirst || l < h->tailFirst); l++) {
      h->dsid[l] = h->alloc<uint16_t>(h->lev[l].n);
      h->dT[l] = h->alloc<float>((long long)(kDictCap + 1) * kDictStride);
      any = true;
    }
    if (any) {
      h->dkeys = h->alloc<unsigned long long>(kDictTable);
      h->drep = h->alloc<int>(kDictTable);
      h->dslot = h->alloc<int>(kDictTable);
      h->dflags = h->alloc<int>(3 * kMaxLevels);
    }
  }
  if (!h->ok) {
    mg_hierarchy_destroy(h);
    return nullptr;
  }
  return h;
}

void mg_hierarchy_destroy(MgHierarchy* h) {
  if (!h) return;
  for (void* p : h->allocs) cudaFree(p);
  delete h;
}

void mg_hierarchy_reset(MgHierarchy* h) {
  if (h) h->isASet = false;
}

size_t mg_hierarchy_bytes(const MgHierarchy* h) { return h ? h->bytes : 0; }
unsigned long long mg_hierarchy_signature(const MgHierarchy* h) {
  if (!h) return 0;
  unsigned int acc;
  std::memcpy(&acc, &h->coarseAcc, sizeof acc);
  return (h->gen << 35) ^ ((unsigned long long)h->useFrac << 34) ^ ((unsigned long long)h->useA0f << 33) ^
         (unsigned long long)acc;
}
int mg_hierarchy_levels(const MgHierarchy* h) { return h ? h->nlev : 0; }
void mg_hierarchy_describe(const MgHierarchy* h, MgLayout* out) {
  *out = MgLayout{};
  if (!h) return;
  out->levels = h->nlev;
  out->tailFirst = h->tailFirst;
  out->tailCtas = h->tailFirst ? g_tailCta : 0;
  for (int l = 0; l < h->nlev && l < 32; l++) {
    for (int c = 0; c < 3; c++) out->size[l][c] = h->size[l][c];
    out->dictStencils[l] = h->ndict[l];
  }
}

int mg_setup(MgHierarchy* h, const PcgBuffers& b, float coarseAccuracy, cudaStream_t s) {
  h->coarseAcc = coarseAccuracy;
  if (h->isASet) return 0;
  h->gen++;
  const Dims& d = h->d;
  if (b.A0f && !h->l0.a0f) {
    h->l0.a0f = h->alloc<float>(d.n);
    if (!h->ok) return 1;
  }
  if (b.Aif && !h->l0.ai) {
    h->l0.ai = h->alloc<float>(d.n);
    h->l0.aj = h->alloc<float>(d.n);
    h->l0.ak = h->alloc<float>(d.n);
    if (!h->ok) return 1;
  }
  // inactive vertices keep zero x, b, r and matrix rows: the V-cycle
  // kernels rely on it instead of testing vertex types
  if (h->l0.r && cudaMemsetAsync(h->l0.r, 0, sizeof(float) * (size_t)d.n, s) != cudaSuccess) return 1;
  for (int l = 1; l < h->nlev; l++) {
    const Lev& v = h->lev[l];
    if (cudaMemsetAsync(v.A, 0, sizeof(float) * (size_t)(v.n * h->S), s) != cudaSuccess ||
        cudaMemsetAsync(v.x, 0, sizeof(float) * (size_t)v.n, s) != cudaSuccess ||
        cudaMemsetAsync(v.b, 0, sizeof(float) * (size_t)v.n, s) != cudaSuccess ||
        cudaMemsetAsync(v.r, 0, sizeof(float) * (size_t)v.n, s) != cudaSuccess)
      return 1;
  }
  float* a0f = b.A0f ? h->l0.a0f : nullptr;
  const bool frac = b.Aif != nullptr;
  Lev0 l0 = h->l0;
  l0.a0f = a0f;
  if (!frac) l0.ai = l0.aj = l0.ak = nullptr;
  count_launch();
  k_mg_snapshot0<<<blocks_for(d.n), kThreads1, 0, s>>>(d, b.code, b.A0f, b.Aif, b.Ajf, b.Akf, h->l0.code, a0f, l0.ai,
                                                        l0.aj, l0.ak, h->type0);
  if (cudaGetLastError() != cudaSuccess) return 1;
  h->useA0f = a0f != nullptr;
  h->useFrac = frac;
  if (h->nlev > 1) {
    // vertex selection on the host, reused while the level-0 types repeat
    h->htype[0].resize((size_t)d.n);
    if (cudaMemcpyAsync(h->htype[0].data(), h->type0, (size_t)d.n, cudaMemcpyDeviceToHost, s) != cudaSuccess) return 1;
    if (cudaStreamSynchronize(s) != cudaSuccess) return 1;
    for (auto& t : h->htype[0])
      if (t == kVtTrivial) t = kVtActive;  // genCoarseGrid tests only for inactive
    const bool reuse = h->selValid && h->selType0 == h->htype[0];
    if (!reuse) {
      for (int l = 1; l < h->nlev; l++) {
        gen_coarse_grid(h->size[l - 1], h->htype[l - 1], h->size[l], h->htype[l]);
        const Lev& v = h->lev[l];
        std::vector<int8_t>& st = h->upload[l];
        st.assign((size_t)v.n, kVtInactive);
        long long q = 0;
        for (int z = 0; z < v.sz; z++)
          for (int y = 0; y < v.sy; y++)
            for (int x = 0; x < v.sx; x++) st[(size_t)lin(v, x, y, z)] = h->htype[l][(size_t)q++];
        if (cudaMemcpyAsync(v.type, st.data(), st.size(), cudaMemcpyHostToDevice, s) != cudaSuccess) return 1;
      }
      h->selType0 = h->htype[0];
      h->selValid = true;
      if (cudaStreamSynchronize(s) != cudaSuccess) return 1;
    }
    // Galerkin operators
    for (int l = 1; l < h->nlev; l++) {
      const long long n = h->lev[l].n;
      count_launch();
      if (l == 1) {
        if (h->is3d) k_mg_coarse_op1<true><<<blocks_for(n), kThreads1, 0, s>>>(h->lev[1], l0, h->S, g_npaths[1]);
        else k_mg_coarse_op1<false><<<blocks_for(n), kThreads1, 0, s>>>(h->lev[1], l0, h->S, g_npaths[0]);
      } else {
        if (h->is3d) k_mg_coarse_op<true><<<blocks_for(n), kThreads1, 0, s>>>(h->lev[l], h->lev[l - 1], h->S);
        else k_mg_coarse_op<false><<<blocks_for(n), kThreads1, 0, s>>>(h->lev[l], h->lev[l - 1], h->S);
      }
      if (cudaGetLastError() != cudaSuccess) return 1;
    }
    // stencil dictionaries (a level keeps its planes unless every tuple was
    // found and verified bit for bit)
    bool anyDict = false;
    for (int l = 1; l < h->nlev; l++) {
      h->lev[l].sid = nullptr;
      h->lev[l].T = nullptr;
      h->ndict[l] = 0;
      if (!h->dsid[l]) continue;
      anyDict = true;
      const Lev& v = h->lev[l];
      int* fl = h->dflags + 3 * l;
      if (cudaMemsetAsync(h->dkeys, 0, sizeof(unsigned long long) * kDictTable, s) != cudaSuccess ||
          cudaMemsetAsync(h->drep, 0x7f, sizeof(int) * kDictTable, s) != cudaSuccess ||
          cudaMemsetAsync(fl, 0, sizeof(int) * 3, s) != cudaSuccess ||
          cudaMemsetAsync(h->dT[l], 0, sizeof(float) * kDictStride, s) != cudaSuccess)
        return 1;
      count_launch();
      if (h->is3d) k_dict_insert<true><<<blocks_for(v.n), kThreads1, 0, s>>>(v, h->dkeys, h->drep, fl);
      else k_dict_insert<false><<<blocks_for(v.n), kThreads1, 0, s>>>(v, h->dkeys, h->drep, fl);
      count_launch();
      k_dict_ids<<<1, 1024, 0, s>>>(h->dkeys, h->dslot, fl);
      count_launch();
      if (h->is3d) k_dict_fill<true><<<blocks_for(v.n), kThreads1, 0, s>>>(v, h->dkeys, h->drep, h->dslot, h->dsid[l], h->dT[l], fl);
      else k_dict_fill<false><<<blocks_for(v.n), kThreads1, 0, s>>>(v, h->dkeys, h->drep, h->dslot, h->dsid[l], h->dT[l], fl);
      count_launch();
      if (h->is3d) k_dict_verify<true><<<blocks_for(v.n), kThreads1, 0, s>>>(v, h->dsid[l], h->dT[l], fl);
      else k_dict_verify<false><<<blocks_for(v.n), kThreads1, 0, s>>>(v, h->dsid[l], h->dT[l], fl);
      if (cudaGetLastError() != cudaSuccess) return 1;
    }
    if (anyDict) {
      int hf[3 * kMaxLevels];
      if (cudaMemcpyAsync(hf, h->dflags, sizeof hf, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess)
        return 1;
      for (int l = 1; l < h->nlev; l++) {
        if (!h->dsid[l]) continue;
        const int* f = hf + 3 * l;
        if (f[0] || f[1] || f[2] > kDictCap) continue;
        h->lev[l].sid = h->dsid[l];
        h->lev[l].T = h->dT[l];
        h->ndict[l] = f[2];
      }
    }
    // the cluster tail reads the levels from the device copy
    if (h->dlev && cudaMemcpyAsync(h->dlev, h->lev, sizeof(Lev) * (size_t)h->nlev, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return 1;
  }
  h->isASet = true;
  return 0;
}

void mg_set_profiler(MgHierarchy* h, MgProfHook hook, void* ctx) {
  h->hook = hook;
  h->hookCtx = ctx;
}

namespace {
struct Fam {
  const MgHierarchy* h;
  const char* name;
  Fam(const MgHierarchy* h_, const char* n) : h(h_), name(n) {
    if (h->hook) h->hook(h->hookCtx, name, 1);
  }
  ~Fam() {
    if (h->hook) h->hook(h->hookCtx, name, 0);
  }
};
}  // namespace

int mg_apply(MgHierarchy* h, const PcgBuffers& b, bool init, cudaStream_t s) {
  const Dims& d = h->d;
  const int L = h->nlev - 1;
  const int S = h->S;
  Lev0 l0 = h->l0;
  if (!h->useA0f) l0.a0f = nullptr;
  if (!h->useFrac) l0.ai = l0.aj = l0.ak = nullptr;
  const bool frac = h->useFrac;
  const CgScalars* sc = b.sc;
  float* x0 = b.tmp;
  const float* res = b.residual;
  const Lev none{};
  const int zc = h->zc;
  const dim3 gt(level0_tiles(d.nx), level0_tiles(d.ny), d.is3d ? (d.nz + zc - 1) / zc : 1);
  if (gt.y > 65535u || gt.z > 65535u) return 1;  // beyond the launch limits (> 1.8 M cells along y or z)
  static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
  const int ncol = h->is3d ? 8 : 4;
  auto smooth = [&](int l, bool reversed) {
    Fam f(h, "mg_smooth_coarse");
    const Lev& v = h->lev[l];
    const int nb = blocks_for((long long)((v.sx + 1) / 2) * ((v.sy + 1) / 2) * ((v.sz + 1) / 2));
    for (int q = 0; q < ncol; q++) {
      const int c = reversed ? ncol - 1 - q : q;
      count_launch();
      if (v.sid) {
        if (h->is3d) k_mg_smooth_dict<true><<<nb, kThreads1, 0, s>>>(v, off[c][0], off[c][1], off[c][2], sc);
        else k_mg_smooth_dict<false><<<nb, kThreads1, 0, s>>>(v, off[c][0], off[c][1], off[c][2], sc);
      } else {
        if (h->is3d) k_mg_smooth<true><<<nb, kThreads1, 0, s>>>(v, S, off[c][0], off[c][1], off[c][2], sc);
        else k_mg_smooth<false><<<nb, kThreads1, 0, s>>>(v, S, off[c][0], off[c][1], off[c][2], sc);
      }
    }
  };
  if (L == 0) {
    // a single level: the whole V-cycle is the coarsest-level CG
    Fam f(h, "mg_coarse_cg");
    count_launch();
    if (h->is3d) k_mg_coarse_cg<true, true><<<1, kCgThreads, kCgDynSmem, s>>>(none, l0, res, x0, S, h->coarseAcc, sc);
    else k_mg_coarse_cg<false, true><<<1, kCgThreads, kCgDynSmem, s>>>(none, l0, res, x0, S, h->coarseAcc, sc);
  } else {
    // level 0 pre-smoothing (colour 0 from x = 0, then colour 1)
    {
      Fam f(h, "mg_down_l0");
      count_launch();
      if (frac) {
        if (h->is3d) k_mg0_down<true, true><<<gt, kT0, sizeof(Ring0), s>>>(l0, res, zc, sc);
        else k_mg0_down<false, true><<<gt, kT0, sizeof(Ring0), s>>>(l0, res, zc, sc);
      } else {
        if (h->is3d) k_mg0_down<true, false><<<gt, kT0, sizeof(Ring0), s>>>(l0, res, zc, sc);
        else k_mg0_down<false, false><<<gt, kT0, sizeof(Ring0), s>>>(l0, res, zc, sc);
      }
    }
    {
      Fam f(h, "mg_restrict_l0");
      count_launch();
      const Lev& v1 = h->lev[1];
      if (v1.sz <= 65535)
        k_mg_restrict0<<<dim3((unsigned)(((long long)v1.sx * v1.sy + 255) / 256), v1.sz), kThreads1, 0, s>>>(v1, l0, sc);
      else  // grid dimensions beyond the y / z launch limits: slot order
        k_mg_restrict<true><<<blocks_for(v1.n), kThreads1, 0, s>>>(v1, none, l0, sc);
    }
    // levels below the cluster tail (all of them without one)
    const int first = h->tailFirst ? h->tailFirst : L;
    for (int l = 1; l < first; l++) {
      smooth(l, false);
      Fam f(h, "mg_transfer_coarse");
      count_launch();
      const Lev& v = h->lev[l];
      if (v.sid) {
        if (h->is3d) k_mg_residual_dict<true><<<blocks_for(v.n), kThreads1, 0, s>>>(v, sc);
        else k_mg_residual_dict<false><<<blocks_for(v.n), kThreads1, 0, s>>>(v, sc);
      } else {
        if (h->is3d) k_mg_residual<true><<<blocks_for(v.n), kThreads1, 0, s>>>(v, S, sc);
        else k_mg_residual<false><<<blocks_for(v.n), kThreads1, 0, s>>>(v, S, sc);
      }
      count_launch();
      k_mg_restrict<false><<<blocks_for(h->lev[l + 1].n), kThreads1, 0, s>>>(h->lev[l + 1], h->lev[l], l0, sc);
    }
    if (h->tailFirst) {
      Fam f(h, "mg_tail");
      count_launch();
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = g_tailCta;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3(g_tailCta);
      cfg.blockDim = dim3(kTailThreads);
      cfg.stream = s;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      const Lev* dl = h->dlev;
      const float acc = h->coarseAcc;
      if (h->is3d) cudaLaunchKernelEx(&cfg, k_mg_tail<true>, dl, first, L, S, acc, sc);
      else cudaLaunchKernelEx(&cfg, k_mg_tail<false>, dl, first, L, S, acc, sc);
    } else {
      Fam f(h, "mg_coarse_cg");
      count_launch();
      if (h->is3d) k_mg_coarse_cg<true, false><<<1, kCgThreads, kCgDynSmem, s>>>(h->lev[L], l0, res, x0, S, h->coarseAcc, sc);
      else k_mg_coarse_cg<false, false><<<1, kCgThreads, kCgDynSmem, s>>>(h->lev[L], l0, res, x0, S, h->coarseAcc, sc);
    }
    for (int l = first - 1; l >= 1; l--) {
      {
      Fam f(h, "mg_transfer_coarse");
      count_launch();
      if (h->is3d) k_mg_interp_add<true><<<blocks_for(h->lev[l].n), kThreads1, 0, s>>>(h->lev[l], h->lev[l + 1], sc);
      else k_mg_interp_add<false><<<blocks_for(h->lev[l].n), kThreads1, 0, s>>>(h->lev[l], h->lev[l + 1], sc);
      }
      smooth(l, true);
    }
    {
      Fam f(h, "mg_up_l0");
      count_launch();
      const Lev& v1 = h->lev[1];
      if (frac) {
        if (h->is3d) {
          if (init) k_mg0_up<true, false, true><<<gt, kT0, sizeof(Ring0), s>>>(l0, res, zc, x0, v1, b.part, b.sc);
          else k_mg0_up<true, true, true><<<gt, kT0, sizeof(Ring0), s>>>(l0, res, zc, x0, v1, b.part, b.sc);
        } else {
          if (init) k_mg0_up<false, false, true><<<gt, kT0, sizeof(Ring0), s>>>(l0, res, zc, x0, v1, b.part, b.sc);
          else k_mg0_up<false, true, true><<<gt, kT0, sizeof(Ring0), s>>>(l0, res, zc, x0, v1, b.part, b.sc);
        }
      } else {
        if (h->is3d) {
          if (init) k_mg0_up<true, false, false><<<gt, kT0, sizeof(Ring0), s>>>(l0, res, zc, x0, v1, b.part, b.sc);
          else k_mg0_up<true, true, false><<<gt, kT0, sizeof(Ring0), s>>>(l0, res, zc, x0, v1, b.part, b.sc);
        } else {
          if (init) k_mg0_up<false, false, false><<<gt, kT0, sizeof(Ring0), s>>>(l0, res, zc, x0, v1, b.part, b.sc);
          else k_mg0_up<false, true, false><<<gt, kT0, sizeof(Ring0), s>>>(l0, res, zc, x0, v1, b.part, b.sc);
        }
      }
    }
  }
  if (!init && L == 0) {
    Fam f(h, "mg_dot");
    count_launch();
    k_mg_dot_beta<<<b.nblocks, kThreads1, 0, s>>>(d.n, b.tmp, b.residual, b.part, b.sc);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace mgpu
