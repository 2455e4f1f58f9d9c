// Gather-scatter kernel instances with 256-thread CTAs: plain copies and
// transposes.
#include "g2g_scatter_impl.cuh"

namespace g2g {

cudaError_t launch_scatter_256(const PlanList &list, const ScatterConfig &cfg,
                               cudaStream_t stream) {
    return launch_plain_paths<256>(list, cfg, stream);
}

} // namespace g2g
