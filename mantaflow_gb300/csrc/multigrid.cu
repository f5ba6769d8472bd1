// Multigrid preconditioner (placeholder until the GPU hierarchy lands).
#include "mg_multigrid.h"

namespace mgpu {

struct MgHierarchy {
  Dims d;
};

MgHierarchy* mg_hierarchy_create(const Dims& d) { return new MgHierarchy{d}; }
void mg_hierarchy_destroy(MgHierarchy* h) { delete h; }
size_t mg_hierarchy_bytes(const MgHierarchy*) { return 0; }
int mg_setup(MgHierarchy*, const PcgBuffers&, float, cudaStream_t) { return 1; }
int mg_apply(MgHierarchy*, const PcgBuffers&, bool, cudaStream_t) { return 1; }

}  // namespace mgpu
