// Barnes-Hut octree on the GPU (placeholder until the tree kernels land).
#include "engine.h"
#include "gh_common.cuh"

namespace gh {

int tree_force(const double*, const double*, int64_t, const double*, int64_t, double, double,
               double*, cudaStream_t) {
  return set_error(GH_ERR_ARG, "tree force not available in this build");
}

int tree_run(double*, double*, const double*, int64_t, int64_t, double, double, double, double*,
             double*, int64_t, cudaStream_t) {
  return set_error(GH_ERR_ARG, "tree force not available in this build");
}

}  // namespace gh
