// Gather-scatter kernel instances with 512-thread CTAs: plans with scaled
// or cast tiles (element arithmetic).
#include "g2g_scatter_impl.cuh"

namespace g2g {

cudaError_t launch_scatter_512_elem(const PlanList &list, const ScatterConfig &cfg,
                                    cudaStream_t stream) {
    return launch_elem_paths<512>(list, cfg, stream);
}

} // namespace g2g
