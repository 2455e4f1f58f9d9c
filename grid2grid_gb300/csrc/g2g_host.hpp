// Host-side helpers shared by the C-ABI translation units.
#pragma once

#include "../../include/grid2grid_gb300.h"

#include <cstdint>

namespace g2g {

// Records a printf-style message as the calling thread's last error and
// returns `st`.
g2g_status fail(g2g_status st, const char *fmt, ...);

// m*n*sizeof(T) summed over the plan's pairs (no synchronisation).
int64_t plan_bytes_moved(const g2g_plan *plan);

} // namespace g2g
