// Multigrid preconditioner on the GPU (multigrid.cpp, Dick et al. 2015).
#pragma once
#include <cuda_runtime.h>

#include "mg_kernels.h"

namespace mgpu {

struct MgHierarchy;

MgHierarchy* mg_hierarchy_create(const Dims& d);
void mg_hierarchy_destroy(MgHierarchy* h);
size_t mg_hierarchy_bytes(const MgHierarchy* h);
// GridMg::setA when the hierarchy has no matrix yet, then
// setCoarsestLevelAccuracy; returns 0 on success
int mg_setup(MgHierarchy* h, const PcgBuffers& b, float coarseAccuracy, cudaStream_t s);
// setRhs(residual) + doVCycle(tmp); init selects the doInit bookkeeping
int mg_apply(MgHierarchy* h, const PcgBuffers& b, bool init, cudaStream_t s);

}  // namespace mgpu
