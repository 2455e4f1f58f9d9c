// Host-side helpers shared by the C-ABI translation units.
#pragma once

#include "../../include/grid2grid_gb300.h"
#include "g2g_internal.hpp"
#include "g2g_launch.hpp"

#include <cstdint>
#include <vector>

namespace g2g {

// Records a printf-style message as the calling thread's last error and
// returns `st`.
g2g_status fail(g2g_status st, const char *fmt, ...);

// m*n*sizeof(T) summed over the plan's pairs (no synchronisation).
int64_t plan_bytes_moved(const g2g_plan *plan);

// Everything the device planner needs for one transform, built and validated
// on the host: the arrays to upload, their sizes, the work-list bound and the
// launch configuration. No CUDA allocation is made to build it.
struct HostPlanImage {
    int device = 0;
    std::vector<PairInfo> pairs;
    std::vector<int32_t> splits;
    std::vector<SrcEntry> src_tables;
    std::vector<DstEntry> dst_tables;
    int64_t n_parts = 0;
    int64_t n_cells = 0;
    int64_t max_cells_per_pair = 0;
    int64_t tile_capacity = 0;
    int64_t bytes_moved = 0;
    ScatterConfig cfg;
};

// Validates one transform's descriptors exactly as g2g_plan_create does and
// fills `out`; makes the device holding the blocks current.
g2g_status build_host_image(const g2g_layout_desc *initial, const g2g_layout_desc *final_,
                            g2g_dtype dtype, const g2g_op *op, HostPlanImage *out);

} // namespace g2g
