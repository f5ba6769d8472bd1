// Forces, wall boundary conditions, simple extrapolation, scene setup and
// grid utilities (plugin/extforces.cpp, fastmarch.cpp, grid.cpp, shapes.cpp).
#include "mg_common.cuh"
#include "mg_kernels.h"
#include "mg_batch.h"

#include <algorithm>
#include <cfloat>

namespace mgpu {

static const dim3 kBlk(32, 8, 1);

#define CELL_IJK                                        \
  const int i = blockIdx.x * blockDim.x + threadIdx.x; \
  const int j = blockIdx.y * blockDim.y + threadIdx.y; \
  const int k = blockIdx.z;                             \
  if (i >= d.nx || j >= d.ny) return;                   \
  const long long idx = ix(d, i, j, k);

#define INNER (i >= 1 && i < d.nx - 1 && j >= 1 && j < d.ny - 1 && (!d.is3d || (k >= 1 && k < d.nz - 1)))

// KnSetWallBcs (extforces.cpp:186-217): every cell, i>0 style checks.
// Every load is issued first (neighbour addresses clamped into the grid; a
// clamped value is never used), then the reference's tests in its order.
__device__ __forceinline__ void set_wall_bcs_cell(const Dims& d, const int* __restrict__ flags, Mac vel, CMac obvel, int hasObvel, int i, int j, int k) {
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
  float u = vel.u[idx], v = vel.v[idx], w = vel.w[idx];
  float bx = 0.f, by = 0.f, bz = 0.f;
  if (hasObvel) {
    bx = obvel.u[idx];
    by = obvel.v[idx];
    if (d.is3d) bz = obvel.w[idx];
  }
  const bool curFluid = f & kFluid, curObs = f & kObstacle;
  if (!curFluid && !curObs) return;
  if (xm && (fxm & kObstacle)) u = bx;
  if (xm && curObs && (fxm & kFluid)) u = bx;
  if (ym && (fym & kObstacle)) v = by;
  if (ym && curObs && (fym & kFluid)) v = by;
  if (!d.is3d) {
    w = 0.f;
  } else {
    if (zm && (fzm & kObstacle)) w = bz;
    if (zm && curObs && (fzm & kFluid)) w = bz;
  }
  if (curFluid) {
    if ((xm && (fxm & kStick)) || (xp && (fxp & kStick))) v = w = 0.f;
    if ((ym && (fym & kStick)) || (yp && (fyp & kStick))) u = w = 0.f;
    if (d.is3d && ((zm && (fzm & kStick)) || (zp && (fzp & kStick)))) u = v = 0.f;
  }
  vel.u[idx] = u;
  vel.v[idx] = v;
  vel.w[idx] = w;
}

__global__ void k_set_wall_bcs(Dims d, const int* __restrict__ flags, Mac vel, CMac obvel, int hasObvel) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  set_wall_bcs_cell(d, flags, vel, obvel, hasObvel, i, j, k);
}

// KnAddBuoyancy (extforces.cpp:72-80).  (0.5*s)*(rho+rho') is formed in
// double and added in double in the reference: one fmaf rounding here.
// Every load is issued before the flag tests.
__device__ __forceinline__ void add_buoyancy_cell(const Dims& d, const int* __restrict__ flags, const float* __restrict__ rho, Mac vel, float hx,
                               float hy, float hz, int i, int j, int k) {
  const long long idx = ix(d, i, j, k);
  if (!INNER) return;
  const int f = __ldg(flags + idx), fxm = __ldg(flags + idx - 1), fym = __ldg(flags + idx - d.sy);
  const int fzm = d.is3d ? __ldg(flags + idx - d.sz) : 0;
  const float r = __ldg(rho + idx), rxm = __ldg(rho + idx - 1), rym = __ldg(rho + idx - d.sy);
  const float rzm = d.is3d ? __ldg(rho + idx - d.sz) : 0.f;
  const float u = vel.u[idx], v = vel.v[idx], w = d.is3d ? vel.w[idx] : 0.f;
  if (!(f & kFluid)) return;
  if (fxm & kFluid) vel.u[idx] = fmaf(hx, r + rxm, u);
  if (fym & kFluid) vel.v[idx] = fmaf(hy, r + rym, v);
  if (d.is3d && (fzm & kFluid)) vel.w[idx] = fmaf(hz, r + rzm, w);
}

__global__ void k_add_buoyancy(Dims d, const int* __restrict__ flags, const float* __restrict__ rho, Mac vel, float hx,
                               float hy, float hz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny) return;
  add_buoyancy_cell(d, flags, rho, vel, hx, hy, hz, i, j, k);
}

// KnApplyForce additive (extforces.cpp:46-58)
__device__ __forceinline__ void add_force_cell(const Dims& d, const int* __restrict__ flags, Mac vel, float fx, float fy,
                                               float fz, const float* __restrict__ exclude, int i, int j, int k) {
  const long long idx = ix(d, i, j, k);
  if (!INNER) return;
  const int f = __ldg(flags + idx);
  const bool curFluid = f & kFluid, curEmpty = f & kEmpty;
  if (!curFluid && !curEmpty) return;
  if (exclude && exclude[idx] < 0.f) return;
  if (isF(flags, idx - 1) || (curFluid && isE(flags, idx - 1))) vel.u[idx] = vel.u[idx] + fx;
  if (isF(flags, idx - d.sy) || (curFluid && isE(flags, idx - d.sy))) vel.v[idx] = vel.v[idx] + fy;
  if (d.is3d && (isF(flags, idx - d.sz) || (curFluid && isE(flags, idx - d.sz)))) vel.w[idx] = vel.w[idx] + fz;
}
__global__ void k_add_force(Dims d, const int* __restrict__ flags, Mac vel, float fx, float fy, float fz,
                            const float* __restrict__ exclude) {
  CELL_IJK
  (void)idx;
  add_force_cell(d, flags, vel, fx, fy, fz, exclude, i, j, k);
}

// extrapolateMACSimple marking (fastmarch.cpp:350-362): tmp = 1 on faces of
// component c next to fluid, 0 elsewhere (also clears the border)
__device__ __forceinline__ void extrap_mark_cell(const Dims& d, const int* __restrict__ flags, int* tmp, int c, int intoObs,
                                                 int i, int j, int k) {
  const long long idx = ix(d, i, j, k);
  int mark = 0;
  if (INNER) {
    const long long nb = idx - (c == 0 ? 1 : (c == 1 ? d.sy : d.sz));
    if (!intoObs) mark = isF(flags, idx) || isF(flags, nb);
    else mark = (isF(flags, idx) || isF(flags, nb)) && !isO(flags, idx) && !isO(flags, nb);
  }
  tmp[idx] = mark;
}
__global__ void k_extrap_mark(Dims d, const int* __restrict__ flags, int* tmp, int c, int intoObs) {
  CELL_IJK
  (void)idx;
  extrap_mark_cell(d, flags, tmp, c, intoObs, i, j, k);
}

// knExtrapolateMACSimple (fastmarch.cpp:230-258).  The reference updates in
// place; a cell only reads neighbours marked with layer d and writes d+1,
// so the result does not depend on the visiting order.
__device__ __forceinline__ void extrap_layer_cell(const Dims& d, float* comp, int* tmp, int layer, int i, int j, int k) {
  const long long idx = ix(d, i, j, k);
  if (!INNER) return;
  if (tmp[idx] != 0) return;
  const long long nb[6] = {1, -1, d.sy, -d.sy, d.sz, -d.sz};
  const int dim = d.is3d ? 3 : 2;
  int nbs = 0;
  float avg = 0.f;
  for (int q = 0; q < 2 * dim; q++)
    if (tmp[idx + nb[q]] == layer) {
      avg += comp[idx + nb[q]];
      nbs++;
    }
  if (nbs > 0) {
    tmp[idx] = layer + 1;
    comp[idx] = avg / (float)nbs;
  }
}
__global__ void k_extrap_layer(Dims d, float* comp, int* tmp, int layer) {
  CELL_IJK
  (void)idx;
  extrap_layer_cell(d, comp, tmp, layer, i, j, k);
}

// knExtrapolateIntoBnd (fastmarch.cpp:260-300) reading a snapshot
__device__ __forceinline__ void extrap_into_bnd_cell(const Dims& d, const int* __restrict__ flags, Mac vel, CMac vt, int i,
                                                     int j, int k) {
  const long long idx = ix(d, i, j, k);
  int cc = 0;
  float v0 = 0.f, v1 = 0.f, v2 = 0.f;
  const bool obs = isO(flags, idx);
#define TAKE(e) do { v0 = vt.u[(e)]; v1 = vt.v[(e)]; v2 = vt.w[(e)]; } while (0)
  if (i == 0) { TAKE(idx + 1); if (obs && v0 < 0.f) v0 = 0.f; cc++; }
  else if (i == d.nx - 1) { TAKE(idx - 1); if (obs && v0 > 0.f) v0 = 0.f; cc++; }
  if (j == 0) { TAKE(idx + d.sy); if (obs && v1 < 0.f) v1 = 0.f; cc++; }
  else if (j == d.ny - 1) { TAKE(idx - d.sy); if (obs && v1 > 0.f) v1 = 0.f; cc++; }
  if (d.is3d) {
    if (k == 0) { TAKE(idx + d.sz); if (obs && v2 < 0.f) v2 = 0.f; cc++; }
    else if (k == d.nz - 1) { TAKE(idx - d.sz); if (obs && v2 > 0.f) v2 = 0.f; cc++; }
  }
#undef TAKE
  if (cc > 0) {
    vel.u[idx] = v0 / (float)cc;
    vel.v[idx] = v1 / (float)cc;
    vel.w[idx] = v2 / (float)cc;
  }
}
// knUnprojectNormalComp (fastmarch.cpp:316-330) with getNormal
// (:298-314): in the band -maxDist <= phiObs <= 0, a velocity pointing
// against the levelset's central-difference normal loses that component
// (normalize as util/vectorbase.h:416-429).  Reads and writes only its own
// cell's velocity; getNormal's clamps are no-ops on the inner cells.
__global__ void k_unproject_normal(Dims d, const float* __restrict__ phi, Mac vel, float maxDist) {
  CELL_IJK
  if (!INNER) return;
  const float p = phi[idx];
  if (p > 0.f || p < -maxDist) return;
  float nx = phi[idx + 1] - phi[idx - 1];
  float ny = phi[idx + d.sy] - phi[idx - d.sy];
  float nz = d.is3d ? phi[idx + d.sz] - phi[idx - d.sz] : p - p;
  const float vx = vel.u[idx], vy = vel.v[idx], vz = vel.w[idx];
  if (!(nx * vx + ny * vy + nz * vz < 0.f)) return;
  const float l = nx * nx + ny * ny + nz * nz;
  const float eps2 = 1e-6f * 1e-6f;
  if (fabs((double)l - 1.) < (double)eps2) {
  } else if (l > eps2) {
    const float sc = (float)(1. / (double)sqrtf(l));
    nx = nx * sc;
    ny = ny * sc;
    nz = nz * sc;
  } else {
    nx = ny = nz = 0.f;
  }
  const float dl = nx * vx + ny * vy + nz * vz;
  vel.u[idx] = vx - nx * dl;
  vel.v[idx] = vy - ny * dl;
  vel.w[idx] = vz - nz * dl;
}

__global__ void k_extrap_into_bnd(Dims d, const int* __restrict__ flags, Mac vel, CMac vt) {
  CELL_IJK
  (void)idx;
  extrap_into_bnd_cell(d, flags, vel, vt, i, j, k);
}

// ------------------------------------------------------- levelset extrapolation
// extrapolateLsSimple (fastmarch.cpp:470-507).  Pass 1 marks the inside
// (phi < 0; phi > 0 for inside marching) with 1, pass 2 the first layer
// around it with 2 (tmp 1 -> 2 never feeds pass 2 itself, so the reference's
// serial loop is order independent).  Both skip the outermost layer.
__global__ void k_els_mark(Dims d, const float* __restrict__ phi, int* tmp, int inside) {
  CELL_IJK
  int t = 0;
  if (INNER) t = inside ? (phi[idx] > 0.f) : (phi[idx] < 0.f);
  tmp[idx] = t;
}
__global__ void k_els_first(Dims d, const int* __restrict__ mark, int* tmp) {
  CELL_IJK
  if (!INNER || mark[idx]) return;
  const long long nb[6] = {1, -1, d.sy, -d.sy, d.sz, -d.sz};
  const int dim = d.is3d ? 3 : 2;
  for (int q = 0; q < 2 * dim; q++)
    if (mark[idx + nb[q]] == 1) {
      tmp[idx] = 2;
      return;
    }
}
// knExtrapolateLsSimple (fastmarch.cpp:443-461): the float average of the
// layer-d neighbours (+x,-x,+y,-y,+z,-z order) divided by their count, plus
// the marching direction; in place like the MAC layers above.
__global__ void k_els_layer(Dims d, float* phi, int* tmp, int layer, float direction) {
  CELL_IJK
  if (!INNER || tmp[idx] != 0) return;
  const long long nb[6] = {1, -1, d.sy, -d.sy, d.sz, -d.sz};
  const int dim = d.is3d ? 3 : 2;
  int nbs = 0;
  float avg = 0.f;
  for (int q = 0; q < 2 * dim; q++)
    if (tmp[idx + nb[q]] == layer) {
      avg += phi[idx + nb[q]];
      nbs++;
    }
  if (nbs > 0) {
    tmp[idx] = layer + 1;
    phi[idx] = avg / (float)nbs + direction;
  }
}
// knSetRemaining (fastmarch.cpp:464-468)
__global__ void k_els_remaining(Dims d, float* phi, const int* __restrict__ tmp, float value) {
  CELL_IJK
  if (INNER && tmp[idx] == 0) phi[idx] = value;
}

// ------------------------------------------------------------------ setup
// FlagGrid::initDomain -> setConst(TypeEmpty) + initBoundaries (grid.cpp:824-842)
__global__ void k_init_domain(Dims d, int* flags, int w, int t0, int t1, int t2, int t3, int t4, int t5) {
  CELL_IJK
  int f = kEmpty;
  if (i <= w) f = t0;
  if (i >= d.nx - 1 - w) f = t1;
  if (j <= w) f = t2;
  if (j >= d.ny - 1 - w) f = t3;
  if (d.is3d) {
    if (k <= w) f = t4;
    if (k >= d.nz - 1 - w) f = t5;
  }
  flags[idx] = f;
}

// FlagGrid::fillGrid (grid.cpp:856-861)
__global__ void k_fill_grid(Dims d, int* flags, int type) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= d.n) return;
  const int f = flags[idx];
  if ((f & kObstacle) == 0 && (f & kInflow) == 0 && (f & kOutflow) == 0 && (f & kOpen) == 0)
    flags[idx] = (f & ~(kEmpty | kFluid)) | type;
}

// setOpenBound (extforces.cpp:105-130)
__global__ void k_set_open_bound(Dims d, int* flags, int bw, int lox, int loy, int loz, int upx, int upy, int upz, int type) {
  CELL_IJK
  const bool loX = lox && i <= bw, loY = loy && j <= bw;
  const bool upX = upx && i >= d.nx - bw - 1, upY = upy && j >= d.ny - bw - 1;
  const bool innerI = i > bw && i < d.nx - bw - 1, innerJ = j > bw && j < d.ny - bw - 1;
  const bool obs = (flags[idx] & kObstacle) != 0;
  if (!d.is3d && (loX || upX || loY || upY)) {
    if ((loX || upX || innerI) && (loY || upY || innerJ) && obs) flags[idx] = type;
  } else {
    const bool loZ = loz && k <= bw, upZ = upz && k >= d.nz - bw - 1;
    const bool innerK = k > bw && k < d.nz - bw - 1;
    if (loX || upX || loY || upY || loZ || upZ) {
      if ((loX || upX || innerI) && (loY || upY || innerJ) && (loZ || upZ || innerK) && obs) flags[idx] = type;
    }
  }
}

// resetOutflow without particles (extforces.cpp:133-160)
__global__ void k_reset_outflow(Dims d, int* flags, float* phi, float* real) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= d.n) return;
  const int f = flags[idx];
  if (!(f & kOutflow)) return;
  flags[idx] = (f | kEmpty) & ~kFluid;
  if (phi) phi[idx] = 0.5f;
  if (real) real[idx] = 0.f;
}

// FlagGrid::updateFromLevelset (grid.cpp:844-854), invalid time -1000
__device__ __forceinline__ void update_from_levelset_cell(int* flags, const float* __restrict__ phi, long long idx) {
  const int f = flags[idx];
  if ((f & kObstacle) || (f & kOutflow)) return;
  const float p = phi[idx];
  if (p <= -1000.f) return;
  flags[idx] = (f & ~(kEmpty | kFluid)) | (p <= 0.f ? kFluid : kEmpty);
}
__global__ void k_update_from_levelset(Dims d, int* flags, const float* __restrict__ phi) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= d.n) return;
  update_from_levelset_cell(flags, phi, idx);
}

__device__ __forceinline__ float smax(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ float smin(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float vnorm(float x, float y, float z) {
  const float l = x * x + y * y + z * z;
  if (l <= 1e-6f * 1e-6f) return 0.f;
  return (fabs((double)l - 1.) < (double)(1e-6f * 1e-6f)) ? 1.f : sqrtf(l);
}

// BoxSDF (shapes.cpp:178-228), including its `p.z > p1.x` lines-Z test
__global__ void k_box_sdf(Dims d, float* phi, float p1x, float p1y, float p1z, float p2x, float p2y, float p2z) {
  CELL_IJK
  const float px = i + 0.5f, py = j + 0.5f, pz = k + 0.5f;
  float v;
#define SQ(a) ((a) * (a))
  if (px <= p2x && px >= p1x && py <= p2y && py >= p1y && pz <= p2z && pz >= p1z) {
    const float mx = smax(px - p2x, p1x - px), my = smax(py - p2y, p1y - py);
    float mz = smax(pz - p2z, p1z - pz);
    if (!d.is3d) mz = mx;
    v = smax(mx, smax(my, mz));
  } else if (py <= p2y && py >= p1y && pz <= p2z && pz >= p1z) {
    v = smax(px - p2x, p1x - px);
  } else if (px <= p2x && px >= p1x && pz <= p2z && pz >= p1z) {
    v = smax(py - p2y, p1y - py);
  } else if (px <= p2x && px >= p1x && py <= p2y && py >= p1y) {
    v = smax(pz - p2z, p1z - pz);
  } else if (px > p1x && px < p2x) {
    const float m1 = sqrtf(SQ(p1y - py) + SQ(p1z - pz)), m2 = sqrtf(SQ(p2y - py) + SQ(p1z - pz));
    const float m3 = sqrtf(SQ(p1y - py) + SQ(p2z - pz)), m4 = sqrtf(SQ(p2y - py) + SQ(p2z - pz));
    v = smin(m1, smin(m2, smin(m3, m4)));
  } else if (py > p1y && py < p2y) {
    const float m1 = sqrtf(SQ(p1x - px) + SQ(p1z - pz)), m2 = sqrtf(SQ(p2x - px) + SQ(p1z - pz));
    const float m3 = sqrtf(SQ(p1x - px) + SQ(p2z - pz)), m4 = sqrtf(SQ(p2x - px) + SQ(p2z - pz));
    v = smin(m1, smin(m2, smin(m3, m4)));
  } else if (pz > p1x && pz < p2z) {
    const float m1 = sqrtf(SQ(p1y - py) + SQ(p1x - px)), m2 = sqrtf(SQ(p2y - py) + SQ(p1x - px));
    const float m3 = sqrtf(SQ(p1y - py) + SQ(p2x - px)), m4 = sqrtf(SQ(p2y - py) + SQ(p2x - px));
    v = smin(m1, smin(m2, smin(m3, m4)));
  } else {
    float m = vnorm(px - p1x, py - p1y, pz - p1z);
    m = smin(m, vnorm(px - p1x, py - p1y, pz - p2z));
    m = smin(m, vnorm(px - p1x, py - p2y, pz - p1z));
    m = smin(m, vnorm(px - p1x, py - p2y, pz - p2z));
    m = smin(m, vnorm(px - p2x, py - p1y, pz - p1z));
    m = smin(m, vnorm(px - p2x, py - p1y, pz - p2z));
    m = smin(m, vnorm(px - p2x, py - p2y, pz - p1z));
    m = smin(m, vnorm(px - p2x, py - p2y, pz - p2z));
    v = m;
  }
#undef SQ
  phi[idx] = v;
}

// Shape::applyToGrid for Box / Cylinder on Real or int grids
// (shapes.cpp:38-45, 151-154, 324-329).  shape: 0 box, 1 cylinder.
__global__ void k_shape_apply(Dims d, int shape, float* freal, int* fint, float value, int ivalue,
                              const int* __restrict__ respect, float a0, float a1, float a2, float b0, float b1, float b2,
                              float radius, float mZ) {
  CELL_IJK
  if (respect && isO(respect, idx)) return;
  const float px = i + 0.5f, py = j + 0.5f, pz = k + 0.5f;
  bool inside;
  if (shape == 0) {
    inside = px >= a0 && py >= a1 && pz >= a2 && px <= b0 && py <= b1 && pz <= b2;
  } else {
    const float qx = px - a0, qy = py - a1, qz = pz - a2;
    const float z = qx * b0 + qy * b1 + qz * b2;
    if (fabsf(z) > mZ) inside = false;
    else inside = ((qx * qx + qy * qy + qz * qz) - z * z) < radius * radius;
  }
  if (!inside) return;
  if (freal) freal[idx] = value;
  else fint[idx] = ivalue;
}

// Shape::applyToGrid for MAC grids (ApplyShapeToMACGrid, shapes.cpp:58-65)
__global__ void k_shape_apply_mac(Dims d, int shape, Mac g, float vx, float vy, float vz, const int* __restrict__ respect,
                                  float a0, float a1, float a2, float b0, float b1, float b2, float radius, float mZ) {
  CELL_IJK
  if (respect && isO(respect, idx)) return;
  for (int c = 0; c < 3; c++) {
    const float px = c == 0 ? (float)i : i + 0.5f;
    const float py = c == 1 ? (float)j : j + 0.5f;
    const float pz = c == 2 ? (float)k : k + 0.5f;
    bool inside;
    if (shape == 0) {
      inside = px >= a0 && py >= a1 && pz >= a2 && px <= b0 && py <= b1 && pz <= b2;
    } else {
      const float qx = px - a0, qy = py - a1, qz = pz - a2;
      const float z = qx * b0 + qy * b1 + qz * b2;
      if (fabsf(z) > mZ) inside = false;
      else inside = ((qx * qx + qy * qy + qz * qz) - z * z) < radius * radius;
    }
    if (inside) g.c(c)[idx] = c == 0 ? vx : (c == 1 ? vy : vz);
  }
}

// ------------------------------------------------------------------ utils
__global__ void k_aos_to_soa(long long n, const float* __restrict__ aos, Mac soa) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  soa.u[idx] = aos[3 * idx];
  soa.v[idx] = aos[3 * idx + 1];
  soa.w[idx] = aos[3 * idx + 2];
}
__global__ void k_soa_to_aos(long long n, CMac soa, float* __restrict__ aos) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  aos[3 * idx] = soa.u[idx];
  aos[3 * idx + 1] = soa.v[idx];
  aos[3 * idx + 2] = soa.w[idx];
}

// Grid<Real>::join (grid.cpp knJoinReal): keep max / min
// four cells per thread (n a multiple of 4; grids start 256-byte aligned)
__global__ void k_join4(long long nq, float4* a, const float4* __restrict__ b, int keepMax) {
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (long long)gridDim.x * blockDim.x) {
    const float4 x = a[q], y = __ldg(b + q);
    float4 o;
    o.x = keepMax ? (x.x < y.x ? y.x : x.x) : (y.x < x.x ? y.x : x.x);
    o.y = keepMax ? (x.y < y.y ? y.y : x.y) : (y.y < x.y ? y.y : x.y);
    o.z = keepMax ? (x.z < y.z ? y.z : x.z) : (y.z < x.z ? y.z : x.z);
    o.w = keepMax ? (x.w < y.w ? y.w : x.w) : (y.w < x.w ? y.w : x.w);
    a[q] = o;
  }
}
__global__ void k_join(long long n, float* a, const float* __restrict__ b, int keepMax) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const float x = a[idx], y = b[idx];
  a[idx] = keepMax ? (x < y ? y : x) : (y < x ? y : x);
}

__global__ void k_set_const(long long n, float* a, float v) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < n) a[idx] = v;
}

// min / max over a float array: two-stage, deterministic
__global__ void k_minmax_partial(long long n, const float* __restrict__ a, float* part) {
  float mn = FLT_MAX, mx = -FLT_MAX;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (long long)gridDim.x * blockDim.x) {
    const float v = a[idx];
    if (v < mn) mn = v;
    if (v > mx) mx = v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  __shared__ float smn[32], smx[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { smn[wid] = mn; smx[wid] = mx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < (int)(blockDim.x >> 5); q++) { mn = fminf(mn, smn[q]); mx = fmaxf(mx, smx[q]); }
    part[2 * blockIdx.x] = mn;
    part[2 * blockIdx.x + 1] = mx;
  }
}

// ------------------------------------------------------------- launchers
static inline unsigned nblk(long long n, int b) { return (unsigned)((n + b - 1) / b); }

void launch_set_wall_bcs(const Dims& d, const int* flags, Mac vel, const Mac* obvel, cudaStream_t s) {
  CMac ob = obvel ? CMac{obvel->u, obvel->v, obvel->w} : CMac{nullptr, nullptr, nullptr};
  count_launch();
  k_set_wall_bcs<<<grid3(d, kBlk), kBlk, 0, s>>>(d, flags, vel, ob, obvel ? 1 : 0);
}
void launch_add_buoyancy(const Dims& d, const int* flags, const float* rho, Mac vel, float hx, float hy, float hz,
                         cudaStream_t s) {
  count_launch();
  k_add_buoyancy<<<grid3(d, kBlk), kBlk, 0, s>>>(d, flags, rho, vel, hx, hy, hz);
}
void launch_add_force(const Dims& d, const int* flags, Mac vel, float fx, float fy, float fz, const float* exclude,
                      cudaStream_t s) {
  count_launch();
  k_add_force<<<grid3(d, kBlk), kBlk, 0, s>>>(d, flags, vel, fx, fy, fz, exclude);
}
void launch_extrapolate_mac_simple(const Dims& d, const int* flags, Mac vel, int* tmp, Mac snap, int distance, int intoObs,
                                   const float* phiObs, cudaStream_t s) {
  const int dim = d.is3d ? 3 : 2;
  for (int c = 0; c < dim; c++) {
    count_launch();
    k_extrap_mark<<<grid3(d, kBlk), kBlk, 0, s>>>(d, flags, tmp, c, intoObs);
    for (int l = 1; l < 1 + distance; l++) {
      count_launch();
      k_extrap_layer<<<grid3(d, kBlk), kBlk, 0, s>>>(d, vel.c(c), tmp, l);
    }
  }
  if (phiObs) {
    count_launch();
    k_unproject_normal<<<grid3(d, kBlk), kBlk, 0, s>>>(d, phiObs, vel, (float)distance);
  }
  cudaMemcpyAsync(snap.u, vel.u, sizeof(float) * d.n, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(snap.v, vel.v, sizeof(float) * d.n, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(snap.w, vel.w, sizeof(float) * d.n, cudaMemcpyDeviceToDevice, s);
  count_launch();
  k_extrap_into_bnd<<<grid3(d, kBlk), kBlk, 0, s>>>(d, flags, vel, CMac{snap.u, snap.v, snap.w});
}
void launch_extrapolate_ls_simple(const Dims& d, float* phi, int* tmp, int* mark, int distance, int inside,
                                  cudaStream_t s) {
  const float direction = inside ? -1.f : 1.f;
  count_launch();
  k_els_mark<<<grid3(d, kBlk), kBlk, 0, s>>>(d, phi, mark, inside);
  cudaMemcpyAsync(tmp, mark, sizeof(int) * d.n, cudaMemcpyDeviceToDevice, s);
  count_launch();
  k_els_first<<<grid3(d, kBlk), kBlk, 0, s>>>(d, mark, tmp);
  for (int l = 2; l < 1 + distance; l++) {
    count_launch();
    k_els_layer<<<grid3(d, kBlk), kBlk, 0, s>>>(d, phi, tmp, l, direction);
  }
  count_launch();
  k_els_remaining<<<grid3(d, kBlk), kBlk, 0, s>>>(d, phi, tmp, direction * (float)(distance + 2));
}
void launch_init_domain(const Dims& d, int* flags, int bw, const int* types, cudaStream_t s) {
  count_launch();
  k_init_domain<<<grid3(d, kBlk), kBlk, 0, s>>>(d, flags, bw, types[0], types[1], types[2], types[3], types[4], types[5]);
}
void launch_fill_grid(const Dims& d, int* flags, int type, cudaStream_t s) {
  count_launch();
  k_fill_grid<<<nblk(d.n, 256), 256, 0, s>>>(d, flags, type);
}
void launch_set_open_bound(const Dims& d, int* flags, int bw, const int* lo, const int* up, int type, cudaStream_t s) {
  count_launch();
  k_set_open_bound<<<grid3(d, kBlk), kBlk, 0, s>>>(d, flags, bw, lo[0], lo[1], lo[2], up[0], up[1], up[2], type);
}
void launch_reset_outflow(const Dims& d, int* flags, float* phi, float* real, cudaStream_t s) {
  count_launch();
  k_reset_outflow<<<nblk(d.n, 256), 256, 0, s>>>(d, flags, phi, real);
}
void launch_update_from_levelset(const Dims& d, int* flags, const float* phi, cudaStream_t s) {
  count_launch();
  k_update_from_levelset<<<nblk(d.n, 256), 256, 0, s>>>(d, flags, phi);
}
void launch_box_sdf(const Dims& d, float* phi, const float* p0, const float* p1, cudaStream_t s) {
  count_launch();
  k_box_sdf<<<grid3(d, kBlk), kBlk, 0, s>>>(d, phi, p0[0], p0[1], p0[2], p1[0], p1[1], p1[2]);
}
void launch_shape_apply(const Dims& d, int shape, float* freal, int* fint, Mac* mac, const float* value, int ivalue,
                        const int* respect, const float* a, const float* b, float radius, float mZ, cudaStream_t s) {
  count_launch();
  if (mac)
    k_shape_apply_mac<<<grid3(d, kBlk), kBlk, 0, s>>>(d, shape, *mac, value[0], value[1], value[2], respect, a[0], a[1],
                                                       a[2], b[0], b[1], b[2], radius, mZ);
  else
    k_shape_apply<<<grid3(d, kBlk), kBlk, 0, s>>>(d, shape, freal, fint, value[0], ivalue, respect, a[0], a[1], a[2], b[0],
                                                   b[1], b[2], radius, mZ);
}
void launch_aos_to_soa(long long n, const float* aos, Mac soa, cudaStream_t s) {
  count_launch();
  k_aos_to_soa<<<nblk(n, 256), 256, 0, s>>>(n, aos, soa);
}
void launch_soa_to_aos(long long n, CMac soa, float* aos, cudaStream_t s) {
  count_launch();
  k_soa_to_aos<<<nblk(n, 256), 256, 0, s>>>(n, soa, aos);
}
void launch_join(long long n, float* a, const float* b, int keepMax, cudaStream_t s) {
  count_launch();
  if ((n & 3) == 0 && ((uintptr_t)a & 15) == 0 && ((uintptr_t)b & 15) == 0) {
    const long long nq = n / 4;
    k_join4<<<(unsigned)std::min<long long>(nblk(nq, 256), 1 << 16), 256, 0, s>>>(nq, reinterpret_cast<float4*>(a),
                                                                                reinterpret_cast<const float4*>(b), keepMax);
  } else {
    k_join<<<nblk(n, 256), 256, 0, s>>>(n, a, b, keepMax);
  }
}
void launch_set_const(long long n, float* a, float v, cudaStream_t s) {
  count_launch();
  k_set_const<<<nblk(n, 256), 256, 0, s>>>(n, a, v);
}
int launch_minmax_partial(long long n, const float* a, float* part, cudaStream_t s) {
  const int blocks = 304;
  count_launch();
  k_minmax_partial<<<blocks, 256, 0, s>>>(n, a, part);
  return blocks;
}

// ----------------------------------------------------------------- batched
#define BATCH_CELL                                                       \
  const BTile tl = tiles[blockIdx.x];                                    \
  const BScene& sc = S[tl.scene];                                        \
  const Dims d = sc.d;                                                   \
  const int i = tl.x0 + threadIdx.x, j = tl.y0 + threadIdx.y, k = tl.z; \
  if (i >= d.nx || j >= d.ny) return;

// inflow: density = max(density, U[0,1) * source) (Grid::join, grid.cpp:303-311)
__global__ void __launch_bounds__(256) k_b_inflow(const BTile* __restrict__ tiles, const BScene* __restrict__ S, int cur) {
  BATCH_CELL
  if (sc.kind != 0) return;  // plume scenes only
  const long long idx = ix(d, i, j, k);
  const float b = batch_noise(sc.seed, sc.step, idx) * sc.mask[idx];
  float* a = sc.dens[cur];
  const float x = a[idx];
  a[idx] = x < b ? b : x;
}
// setWallBcs then addBuoyancy: both read and write only their own cell's
// velocity, so one pass applies them in the reference's order
// (dam break: addGravity, then setWallBcs; also one pass)
__global__ void __launch_bounds__(256) k_b_forces(const BTile* __restrict__ tiles, const BScene* __restrict__ S, int nxt) {
  BATCH_CELL
  const Mac v = bmac(sc.vel[nxt], d.n);
  if (sc.kind == 0) {
    set_wall_bcs_cell(d, sc.flags, v, CMac{nullptr, nullptr, nullptr}, 0, i, j, k);
    add_buoyancy_cell(d, sc.flags, sc.dens[nxt], v, sc.bx, sc.by, sc.bz, i, j, k);
  } else {
    add_force_cell(d, sc.flags, v, sc.bx, sc.by, sc.bz, nullptr, i, j, k);
    set_wall_bcs_cell(d, sc.flags, v, CMac{nullptr, nullptr, nullptr}, 0, i, j, k);
  }
}

// ---- dam-break passes over the dam scenes' tiles
// extrapolateMACSimple(flags, vel, distance=4) (fastmarch.cpp:337-375) on
// the current velocity: marks and layers per component, then the domain
// sides from a snapshot (in the scene's forward scratch)
__global__ void __launch_bounds__(256) k_b_dam_extrap_mark(const BTile* __restrict__ tiles, const BScene* __restrict__ S,
                                                           int c) {
  BATCH_CELL
  if (c >= (d.is3d ? 3 : 2)) return;  // 2D: x and y only
  extrap_mark_cell(d, sc.flags, sc.itmp, c, 0, i, j, k);
}
__global__ void __launch_bounds__(256) k_b_dam_extrap_layer(const BTile* __restrict__ tiles, const BScene* __restrict__ S,
                                                            int cur, int c, int layer) {
  BATCH_CELL
  if (c >= (d.is3d ? 3 : 2)) return;
  extrap_layer_cell(d, sc.vel[cur] + (long long)c * d.n, sc.itmp, layer, i, j, k);
}
__global__ void __launch_bounds__(256) k_b_dam_snapshot(const BTile* __restrict__ tiles, const BScene* __restrict__ S,
                                                        int cur) {
  BATCH_CELL
  const long long idx = ix(d, i, j, k);
  for (int c = 0; c < 3; c++) sc.fwd[c * d.n + idx] = sc.vel[cur][c * d.n + idx];
}
__global__ void __launch_bounds__(256) k_b_dam_extrap_bnd(const BTile* __restrict__ tiles, const BScene* __restrict__ S,
                                                          int cur) {
  BATCH_CELL
  extrap_into_bnd_cell(d, sc.flags, bmac(sc.vel[cur], d.n), bcmac(sc.fwd, d.n), i, j, k);
}
// FlagGrid::updateFromLevelset (grid.cpp:844-854) from the advected phi
__global__ void __launch_bounds__(256) k_b_dam_flags(const BTile* __restrict__ tiles, const BScene* __restrict__ S,
                                                     int nxt) {
  BATCH_CELL
  update_from_levelset_cell(sc.flags, sc.dens[nxt], ix(d, i, j, k));
}
// the final setWallBcs of the dam-break step
__global__ void __launch_bounds__(256) k_b_dam_walls(const BTile* __restrict__ tiles, const BScene* __restrict__ S,
                                                     int nxt) {
  BATCH_CELL
  set_wall_bcs_cell(d, sc.flags, bmac(sc.vel[nxt], d.n), CMac{nullptr, nullptr, nullptr}, 0, i, j, k);
}
#undef BATCH_CELL

void launch_b_dam_advect_sl(const BTile* t, int nt, const BScene* s, int cur, bool vel, cudaStream_t st);

void launch_b_dam_advect(const BTile* t, int nt, const BScene* s, int cur, cudaStream_t st) {
  if (nt == 0) return;
  const dim3 b(kBTX, kBTY, 1);
  for (int c = 0; c < 3; c++) {  // 2D scenes skip c = 2 in the kernels
    count_launch();
    k_b_dam_extrap_mark<<<nt, b, 0, st>>>(t, s, c);
    for (int l = 1; l <= 4; l++) {
      count_launch();
      k_b_dam_extrap_layer<<<nt, b, 0, st>>>(t, s, cur, c, l);
    }
  }
  count_launch();
  k_b_dam_snapshot<<<nt, b, 0, st>>>(t, s, cur);
  count_launch();
  k_b_dam_extrap_bnd<<<nt, b, 0, st>>>(t, s, cur);
  launch_b_dam_advect_sl(t, nt, s, cur, false, st);
  count_launch();
  k_b_dam_flags<<<nt, b, 0, st>>>(t, s, 1 - cur);
  launch_b_dam_advect_sl(t, nt, s, cur, true, st);
}

void launch_b_dam_walls(const BTile* t, int nt, const BScene* s, int nxt, cudaStream_t st) {
  count_launch();
  k_b_dam_walls<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s, nxt);
}

void launch_b_inflow(const BTile* t, int nt, const BScene* s, int cur, cudaStream_t st) {
  count_launch();
  k_b_inflow<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s, cur);
}
void launch_b_forces(const BTile* t, int nt, const BScene* s, int nxt, cudaStream_t st) {
  count_launch();
  k_b_forces<<<nt, dim3(kBTX, kBTY, 1), 0, st>>>(t, s, nxt);
}

}  // namespace mgpu
