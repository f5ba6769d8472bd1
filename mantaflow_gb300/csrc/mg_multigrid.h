// Multigrid preconditioner on the GPU (GridMg, multigrid.cpp; Dick,
// Rogowsky and Westermann 2015, without topology awareness).
#pragma once
#include <cuda_runtime.h>

#include "mg_kernels.h"

namespace mgpu {

struct MgHierarchy;

MgHierarchy* mg_hierarchy_create(const Dims& d);
void mg_hierarchy_destroy(MgHierarchy* h);
// forget the matrix: the next mg_setup builds the hierarchy again (the
// reference deletes the GridMg of a PcMGDynamic solve, pressure.cpp:418-451).
// Device buffers and the coarse-vertex selection cache are kept.
void mg_hierarchy_reset(MgHierarchy* h);
size_t mg_hierarchy_bytes(const MgHierarchy* h);
int mg_hierarchy_levels(const MgHierarchy* h);
// level sizes and how each level is run (after mg_setup)
struct MgLayout {
  int levels;
  int tailFirst;  // first level of the single-launch cluster tail (0: none)
  int tailCtas;   // CTAs of that cluster
  int size[32][3];
  int dictStencils[32];  // distinct stencils of a dictionary level (0: planes)
};
void mg_hierarchy_describe(const MgHierarchy* h, MgLayout* out);
// changes whenever the kernel parameters of mg_apply change (rebuild,
// coarsest-level accuracy, ghost-fluid diagonal): a captured graph of
// mg_apply stays valid while the signature and the PcgBuffers are the same
unsigned long long mg_hierarchy_signature(const MgHierarchy* h);
// GridMg::setA when the hierarchy has no matrix yet (InitPreconditionMultigrid,
// conjugategrad.cpp:100-106), then setCoarsestLevelAccuracy; 0 on success.
// The matrix is read from b.code / b.A0f on the GPU.
int mg_setup(MgHierarchy* h, const PcgBuffers& b, float coarseAccuracy, cudaStream_t s);
// ApplyPreconditionMultigrid (conjugategrad.cpp:162-167): setRhs(residual)
// and doVCycle(tmp) from a zero guess.  Unless init, the last kernel also
// forms sigmaNew = dot(tmp, residual) and beta like GridCg::iterate.
int mg_apply(MgHierarchy* h, const PcgBuffers& b, bool init, cudaStream_t s);
// per-kernel-family timing: mg_apply calls hook(ctx, family, 1) before and
// hook(ctx, family, 0) after each family of launches while a hook is set
typedef void (*MgProfHook)(void* ctx, const char* family, int begin);
void mg_set_profiler(MgHierarchy* h, MgProfHook hook, void* ctx);

}  // namespace mgpu
