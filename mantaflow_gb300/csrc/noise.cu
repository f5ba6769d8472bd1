// Wavelet noise (noisefield.h / noisefield.cpp) and the noise-modulated
// density source of the smoke scenes (densityInflow, plugin/initplugins.cpp).
//
// The 3 x 128^3 noise tile is set up once per process on the host, as the
// reference builds it (WaveletNoiseField::generateTile, noisefield.cpp:
// 94-190): normally distributed values from a Mersenne twister seeded with
// 13322223 (util/randomstream.h), minus their periodic down/up-sampled copy
// along each axis, plus the result read at an offset of 65 cells.  It then
// stays in device memory; evaluation (WNoise, a quadratic B-spline over 27
// tile samples) and the inflow run on the GPU with the reference's float
// arithmetic.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mantagpu.h"
#include "mg_batch.h"
#include "mg_common.cuh"
#include "mg_kernels.h"

using namespace mgpu;

namespace {

constexpr int kTile = 128;
constexpr size_t kTileCells = (size_t)kTile * kTile * kTile;

// MT19937 as util/randomstream.h's MTRand: Knuth's seeding, the twist of the
// whole state at once, the standard tempering; rand() on [0,1], randExc()
// on [0,1), randDblExc() on (0,1), and randNorm by Box-Muller.
class Twister {
 public:
  explicit Twister(uint32_t seed) {
    s_[0] = seed;
    for (int i = 1; i < 624; i++) s_[i] = 1812433253u * (s_[i - 1] ^ (s_[i - 1] >> 30)) + (uint32_t)i;
    twist();
  }
  uint32_t next() {
    if (pos_ == 624) twist();
    uint32_t y = s_[pos_++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    return y ^ (y >> 18);
  }
  double closed() { return (double)next() * (1.0 / 4294967295.0); }
  double half_open() { return (double)next() * (1.0 / 4294967296.0); }
  double open() { return ((double)next() + 0.5) * (1.0 / 4294967296.0); }
  double normal(double mean, double variance) {
    const double r = std::sqrt(-2.0 * std::log(1.0 - open())) * variance;
    const double phi = 2.0 * 3.14159265358979323846264338328 * half_open();
    return mean + r * std::cos(phi);
  }

 private:
  void twist() {
    for (int i = 0; i < 624; i++) {
      const uint32_t nxt = s_[i + 1 < 624 ? i + 1 : 0];
      const uint32_t y = (s_[i] & 0x80000000u) | (nxt & 0x7fffffffu);
      s_[i] = s_[i + 397 < 624 ? i + 397 : i + 397 - 624] ^ (y >> 1) ^ ((nxt & 1u) ? 0x9908b0dfu : 0u);
    }
    pos_ = 0;
  }
  uint32_t s_[624];
  int pos_ = 0;
};

// the analysis (32 taps) and refinement (4 taps) filters of the tile setup
const float kDown[32] = {0.000334f, -0.001528f, 0.000410f, 0.003545f, -0.000938f, -0.008233f, 0.002172f, 0.019120f,
                         -0.005040f, -0.044412f, 0.011655f, 0.103311f, -0.025936f, -0.243780f, 0.033979f, 0.655340f,
                         0.655340f, 0.033979f, -0.243780f, -0.025936f, 0.103311f, 0.011655f, -0.044412f, -0.005040f,
                         0.019120f, 0.002172f, -0.008233f, -0.000938f, 0.003546f, 0.000410f, -0.001528f, 0.000334f};
const float kUp[4] = {0.25f, 0.75f, 0.75f, 0.25f};

// one periodic line of 128 values (stride apart): down-sample to 64, then
// up-sample back to 128 into `out`; `half` is scratch for the 64 values.
// The down-sampling sums float products; the up-sampling adds each
// 0.5 * coefficient * value product in double and rounds the sum to float,
// as the reference's mixed-precision expressions do.
void smooth_line(const float* in, float* half, float* out, int stride) {
  for (int i = 0; i < kTile / 2; i++) {
    float acc = 0.f;
    for (int t = 0; t < 32; t++) acc += kDown[t] * in[((2 * i - 16 + t) & (kTile - 1)) * stride];
    half[i * stride] = acc;
  }
  for (int i = 0; i < kTile; i++) {
    float acc = 0.f;
    for (int t = 0; t < 4; t++) {
      const int k = i / 2 - 1 + t;
      const int m = ((k % (kTile / 2)) + kTile / 2) % (kTile / 2);
      acc = (float)((double)acc + 0.5 * (double)kUp[t] * (double)half[m * stride]);
    }
    out[i * stride] = acc;
  }
}

std::vector<float> make_tile() {
  std::vector<float> noise(3 * kTileCells), a(3 * kTileCells, 0.f), b(3 * kTileCells, 0.f);
  Twister rng(13322223u);
  for (auto& v : noise) v = (float)rng.normal(0.0, 1.0);
  const int n = kTile, n2 = n * n;
  for (int t = 0; t < 3; t++) {
    const size_t base = (size_t)t * kTileCells;
    // along x, then y, then z; each pass reads the previous pass's result
    for (int z = 0; z < n; z++)
      for (int y = 0; y < n; y++) {
        const size_t o = base + (size_t)y * n + (size_t)z * n2;
        smooth_line(&noise[o], &a[o], &b[o], 1);
      }
    for (int z = 0; z < n; z++)
      for (int x = 0; x < n; x++) {
        const size_t o = base + x + (size_t)z * n2;
        smooth_line(&b[o], &a[o], &b[o], n);
      }
    for (int y = 0; y < n; y++)
      for (int x = 0; x < n; x++) {
        const size_t o = base + x + (size_t)y * n;
        smooth_line(&b[o], &a[o], &b[o], n2);
      }
  }
  for (size_t i = 0; i < noise.size(); i++) noise[i] -= b[i];
  // plus the tile read 65 cells further along every axis, stored z fastest
  // and added as it lies (the reference's transposed sum)
  size_t c = 0;
  for (int t = 0; t < 3; t++)
    for (int x = 0; x < n; x++)
      for (int y = 0; y < n; y++)
        for (int z = 0; z < n; z++)
          a[c++] = noise[(size_t)t * kTileCells + ((x + 65) & (n - 1)) + (size_t)((y + 65) & (n - 1)) * n +
                         (size_t)((z + 65) & (n - 1)) * n2];
  for (size_t i = 0; i < noise.size(); i++) noise[i] += a[i];
  return noise;
}

std::mutex g_tileMu;
float* g_tileDev = nullptr;  // device copy of the tile, kept until mg_shutdown
int g_tileUsers = 0;

}  // namespace

struct mg_noise_s {
  int nx, ny, nz, is3d;
  float seedOffset[3];
  mg_noise_params p;
};

// evaluate() arguments of one launch
struct NoiseEval {
  float gsInv[3], seed[3], timeOffset, posScale[3], posOffset[3];
  float valOffset, valScale, clampNeg, clampPos;
  int clamp;
};

namespace mgpu {

// WNoise (noisefield.h:155-196)
__device__ __forceinline__ float wnoise(float px, float py, float pz, const float* __restrict__ data) {
  const float p[3] = {px, py, pz};
  float w[3][3];
  int mid[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    mid[a] = (int)ceilf(p[a] - 0.5f);
    const float t = (float)mid[a] - (p[a] - 0.5f);
    w[a][0] = t * t * 0.5f;
    w[a][2] = (1.f - t) * (1.f - t) * 0.5f;
    w[a][1] = 1.f - w[a][0] - w[a][2];
  }
  float r = 0.f;
#pragma unroll
  for (int z = 0; z < 3; z++)
#pragma unroll
    for (int y = 0; y < 3; y++)
#pragma unroll
      for (int x = 0; x < 3; x++) {
        const float weight = (w[0][x] * w[1][y]) * w[2][z];
        const int xc = (mid[0] + x - 1) & (kTile - 1), yc = (mid[1] + y - 1) & (kTile - 1),
                  zc = (mid[2] + z - 1) & (kTile - 1);
        r += weight * __ldg(data + (zc * kTile + yc) * kTile + xc);
      }
  return r;
}

// WaveletNoiseField::evaluate (noisefield.h:332-357) at Vec3(i, j, k)
__device__ __forceinline__ float noise_at(const NoiseEval& q, const float* __restrict__ tile, int i, int j, int k) {
  float px = (float)i * q.gsInv[0], py = (float)j * q.gsInv[1], pz = (float)k * q.gsInv[2];
  px += q.seed[0];
  py += q.seed[1];
  pz += q.seed[2];
  px += q.timeOffset;
  py += q.timeOffset;
  pz += q.timeOffset;
  px *= q.posScale[0];
  py *= q.posScale[1];
  pz *= q.posScale[2];
  px += q.posOffset[0];
  py += q.posOffset[1];
  pz += q.posOffset[2];
  float v = wnoise(px, py, pz, tile);
  v += q.valOffset;
  v *= q.valScale;
  if (q.clamp) {
    if (v < q.clampNeg) v = q.clampNeg;
    if (v > q.clampPos) v = q.clampPos;
  }
  return v;
}

__global__ void k_noise_eval(Dims d, NoiseEval q, const float* __restrict__ tile, float* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  out[ix(d, i, j, k)] = noise_at(q, tile, i, j, k);
}

// KnApplyNoiseInfl (plugin/initplugins.cpp:27-36): the sdf-based fade factor
// is formed in double and clamped to [0,1] (clamp keeps a NaN), then rounded
__global__ void k_density_inflow(Dims d, const int* __restrict__ flags, float* density, const float* __restrict__ sdf,
                                 NoiseEval q, const float* __restrict__ tile, float scale, float sigma) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  const long long idx = ix(d, i, j, k);
  const float s = sdf[idx];
  if (!(__ldg(flags + idx) & kFluid) || s > sigma) return;
  double f = 1.0 - 0.5 / (double)sigma * (double)(s + sigma);
  if (f < 0.0) f = 0.0;
  else if (f > 1.0) f = 1.0;
  const float factor = (float)f;
  const float target = noise_at(q, tile, i, j, k) * scale * factor;
  if (density[idx] < target) density[idx] = target;
}

// CylinderSDF (shapes.cpp:367-385)
__global__ void k_cylinder_sdf(Dims d, float* phi, float cx, float cy, float cz, float radius, float zx, float zy,
                               float zz, float maxz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  const float px = (float)(i + 0.5) - cx, py = (float)(j + 0.5) - cy, pz = (float)(k + 0.5) - cz;
  const float z = fabsf(px * zx + py * zy + pz * zz);
  const float r = sqrtf((px * px + py * py + pz * pz) - z * z);
  float v;
  if (z < maxz) {
    const float a = r - radius, b = z - maxz;
    v = r < radius ? (a < b ? b : a) : a;
  } else if (r < radius) {
    v = fabsf(z - maxz);
  } else {
    v = sqrtf((z - maxz) * (z - maxz) + (r - radius) * (r - radius));
  }
  phi[ix(d, i, j, k)] = v;
}

}  // namespace mgpu

namespace {

int tile_acquire(float** out) {
  std::lock_guard<std::mutex> lk(g_tileMu);
  if (!g_tileDev) {
    const std::vector<float> t = make_tile();
    float* p = nullptr;
    if (cudaMalloc(&p, t.size() * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      return set_error(MG_ERR_NOMEM, "WaveletNoiseField: out of device memory for the noise tile");
    }
    if (cudaMemcpy(p, t.data(), t.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaFree(p);
      return set_error(MG_ERR_CUDA, "WaveletNoiseField: uploading the noise tile failed");
    }
    g_tileDev = p;
  }
  g_tileUsers++;
  *out = g_tileDev;
  return MG_OK;
}

NoiseEval eval_args(const mg_noise_s* n, float solverTime) {
  NoiseEval q;
  const int m = std::max(n->nx, std::max(n->ny, n->nz));
  const float scale = (float)(1.0 / (double)m);
  q.gsInv[0] = scale;
  q.gsInv[1] = scale;
  q.gsInv[2] = n->is3d ? scale : 1.f;
  for (int c = 0; c < 3; c++) q.seed[c] = n->seedOffset[c];
  const float dx = (float)(1.0 / (double)m);  // FluidSolver::getDx
  q.timeOffset = (solverTime * dx) * n->p.timeAnim;
  for (int c = 0; c < 3; c++) {
    q.posScale[c] = n->p.posScale[c];
    q.posOffset[c] = n->p.posOffset[c];
  }
  q.valOffset = n->p.valOffset;
  q.valScale = n->p.valScale;
  q.clamp = n->p.clamp;
  q.clampNeg = n->p.clampNeg;
  q.clampPos = n->p.clampPos;
  return q;
}

}  // namespace

extern "C" int mg_grid_get_info(mg_grid g, int* nx, int* ny, int* nz, int* kind);
extern "C" int mg_grid_device(mg_grid g, void** data, void** stream);

extern "C" void mg_noise_params_default(mg_noise_params* p) {
  if (!p) return;
  for (int c = 0; c < 3; c++) {
    p->posOffset[c] = 0.f;
    p->posScale[c] = 1.f;
  }
  p->valOffset = 0.f;
  p->valScale = 1.f;
  p->clamp = 0;
  p->clampNeg = 0.f;
  p->clampPos = 1.f;
  p->timeAnim = 0.f;
}

extern "C" int mg_noise_create(mg_solver s, int fixedSeed, mg_noise* out) {
  if (!out) return set_error(MG_ERR_ARG, "mg_noise_create: null out");
  int nx = 0, ny = 0, nz = 0;
  if (mg_solver_size(s, &nx, &ny, &nz)) return MG_ERR_ARG;
  float* tile = nullptr;
  const int st = tile_acquire(&tile);
  if (st) return st;
  auto n = new mg_noise_s();
  n->nx = nx;
  n->ny = ny;
  n->nz = nz;
  n->is3d = nz > 1;
  mg_noise_params_default(&n->p);
  // mSeedOffset: RandomStream(fixedSeed).getVec3Norm() (noisefield.cpp:72-76;
  // -1 selects randomSeed + 123), normalized as util/vectorbase.h's normalize
  Twister rng((uint32_t)(fixedSeed == -1 ? 13322223 + 123 : fixedSeed));
  float v[3];
  for (auto& c : v) c = (float)rng.closed();
  const float l = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  if (std::fabs((double)l - 1.) < (double)(1e-6f * 1e-6f)) {
  } else if (l > 1e-6f * 1e-6f) {
    const float inv = (float)(1. / (double)std::sqrt(l));
    for (auto& c : v) c = c * inv;
  } else {
    v[0] = v[1] = v[2] = 0.f;
  }
  for (int c = 0; c < 3; c++) n->seedOffset[c] = v[c];
  *out = n;
  return MG_OK;
}

extern "C" int mg_noise_destroy(mg_noise n) {
  if (!n) return MG_OK;
  std::lock_guard<std::mutex> lk(g_tileMu);
  g_tileUsers--;
  delete n;
  return MG_OK;
}

extern "C" int mg_noise_set_params(mg_noise n, const mg_noise_params* p) {
  if (!n || !p) return set_error(MG_ERR_ARG, "mg_noise_set_params: invalid argument");
  n->p = *p;
  return MG_OK;
}

extern "C" int mg_noise_seed_offset(mg_noise n, float* out3) {
  if (!n || !out3) return set_error(MG_ERR_ARG, "mg_noise_seed_offset: invalid argument");
  for (int c = 0; c < 3; c++) out3[c] = n->seedOffset[c];
  return MG_OK;
}

// the grid's device storage and its solver's stream, for this translation unit
static int grid_dev(mg_grid g, int wantKind, const char* what, float** data, cudaStream_t* st, Dims* d) {
  int nx, ny, nz, kind;
  if (mg_grid_get_info(g, &nx, &ny, &nz, &kind)) return MG_ERR_ARG;
  if (wantKind >= 0 && kind != wantKind && !(wantKind == MG_REAL && kind == MG_LEVELSET))
    return set_error(MG_ERR_ARG, std::string(what) + ": wrong grid type");
  void* p = nullptr;
  void* s = nullptr;
  mg_grid_device(g, &p, &s);
  *data = (float*)p;
  *st = (cudaStream_t)s;
  d->nx = nx;
  d->ny = ny;
  d->nz = nz;
  d->is3d = nz > 1;
  d->n = (long long)nx * ny * nz;
  d->sy = nx;
  d->sz = nz > 1 ? (long long)nx * ny : 0;
  return MG_OK;
}

extern "C" int mg_noise_evaluate_grid(mg_noise n, mg_grid out, float solverTime) {
  if (!n) return set_error(MG_ERR_ARG, "mg_noise_evaluate_grid: null noise");
  float* o;
  cudaStream_t st;
  Dims d;
  if (grid_dev(out, MG_REAL, "mg_noise_evaluate_grid", &o, &st, &d)) return MG_ERR_ARG;
  const dim3 b(32, 8, 1);
  count_launch();
  k_noise_eval<<<grid3(d, b), b, 0, st>>>(d, eval_args(n, solverTime), g_tileDev, o);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(MG_ERR_CUDA, std::string("noise evaluation: ") + cudaGetErrorString(e));
  return MG_OK;
}

extern "C" int mg_density_inflow(mg_grid flags, mg_grid density, mg_noise noise, mg_grid sdf, float scale, float sigma,
                                 float solverTime) {
  if (!noise) return set_error(MG_ERR_ARG, "densityInflow: null noise");
  float *f, *dn, *sd;
  cudaStream_t st, st2, st3;
  Dims d, d2, d3;
  if (grid_dev(flags, MG_FLAGS, "densityInflow", &f, &st, &d) || grid_dev(density, MG_REAL, "densityInflow", &dn, &st2, &d2) ||
      grid_dev(sdf, MG_REAL, "densityInflow", &sd, &st3, &d3))
    return MG_ERR_ARG;
  if (st2 != st || st3 != st) return set_error(MG_ERR_ARG, "densityInflow: grids of different solvers");
  const dim3 b(32, 8, 1);
  count_launch();
  k_density_inflow<<<grid3(d, b), b, 0, st>>>(d, (const int*)f, dn, sd, eval_args(noise, solverTime), g_tileDev, scale,
                                              sigma);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(MG_ERR_CUDA, std::string("densityInflow: ") + cudaGetErrorString(e));
  return MG_OK;
}

extern "C" int mg_shape_cylinder_levelset(mg_grid phi, const float* center, float radius, const float* z) {
  if (!center || !z) return set_error(MG_ERR_ARG, "Cylinder::computeLevelset: null argument");
  float* p;
  cudaStream_t st;
  Dims d;
  if (grid_dev(phi, MG_REAL, "Cylinder::computeLevelset", &p, &st, &d)) return MG_ERR_ARG;
  // Cylinder(center, radius, z): mZDir = z normalized, mZ = its length
  // (shapes.cpp:316-322)
  float zd[3], mz;
  cylinder_axis(z, zd, &mz);
  const dim3 b(32, 8, 1);
  count_launch();
  k_cylinder_sdf<<<grid3(d, b), b, 0, st>>>(d, p, center[0], center[1], center[2], radius, zd[0], zd[1], zd[2], mz);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(MG_ERR_CUDA, std::string("Cylinder::computeLevelset: ") + cudaGetErrorString(e));
  return MG_OK;
}

// mg_shutdown: the tile goes with the device state
void mgpu::noise_release() {
  std::lock_guard<std::mutex> lk(g_tileMu);
  if (g_tileDev) cudaFree(g_tileDev);
  g_tileDev = nullptr;
  g_tileUsers = 0;
}
