// Gather-scatter kernel instances with 256-thread CTAs: plans with scaled
// or cast tiles (element arithmetic).
#include "g2g_scatter_impl.cuh"

namespace g2g {

cudaError_t launch_scatter_256_elem(const PlanList &list, const ScatterConfig &cfg,
                                    cudaStream_t stream) {
    return launch_elem_paths<256>(list, cfg, stream);
}

} // namespace g2g
