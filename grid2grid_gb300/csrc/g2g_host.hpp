// Host-side helpers shared by the C-ABI translation units.
#pragma once

#include "../../include/grid2grid_gb300.h"
#include "g2g_internal.hpp"
#include "g2g_launch.hpp"

#include <cstdint>
#include <cstring>
#include <functional>
#include <cstddef>
#include <vector>

namespace g2g {

// Records a printf-style message as the calling thread's last error and
// returns `st`.
g2g_status fail(g2g_status st, const char *fmt, ...);

// Returns the status of `expr` from the calling function unless it succeeded.
#define G2G_TRY(expr)                                                                   \
    do {                                                                                \
        g2g_status s_ = (expr);                                                         \
        if (s_ != G2G_SUCCESS)                                                          \
            return s_;                                                                  \
    } while (0)

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

// A plan over part of a transform: the blocks one shard of a sharded
// transform holds, or a packed exchange buffer. `init_held` / `final_held`
// (one entry per virtual rank) name the ranks whose blocks the descriptor
// lists -- all of them, and no other; `*_absent_ok` lets a descriptor list
// any subset of blocks. Cells whose source or destination block is not
// listed take no part. `elems` is the number of elements the plan moves
// (for its byte counts), -1 for m*n.
struct PartialSpec {
    const std::vector<char> *init_held = nullptr;
    const std::vector<char> *final_held = nullptr;
    bool init_absent_ok = false;
    bool final_absent_ok = false;
    int64_t elems = -1;
};
g2g_status create_plan_partial(const g2g_layout_desc *initial, const g2g_layout_desc *final_,
                               g2g_dtype dtype, const g2g_op *op, const PartialSpec &part,
                               g2g_plan **plan);
// Runs the validation of create_plan_partial without planning.
g2g_status validate_partial(const g2g_layout_desc *initial, const g2g_layout_desc *final_,
                            g2g_dtype dtype, const g2g_op *op, const PartialSpec &part);

// Validates one transform's descriptors exactly as g2g_plan_create does and
// fills `out`; makes the device holding the blocks current.
g2g_status build_host_image(const g2g_layout_desc *initial, const g2g_layout_desc *final_,
                            g2g_dtype dtype, const g2g_op *op, HostPlanImage *out);

// 128-bit signature of a request: two 64-bit multiply-rotate streams over
// the bytes taken eight at a time (a descriptor of 16 K blocks is about
// 400 KB, hashed on every blocking call and server submission), each field's
// length mixed in after it.
struct Sig {
    uint64_t a = 0x243f6a8885a308d3ull, b = 0x13198a2e03707344ull;
    static uint64_t rotl(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }
    void word(uint64_t w) {
        a = rotl(a ^ (w * 0x87c37b91114253d5ull), 31) * 0x4cf5ad432745937full;
        b = rotl(b ^ (w * 0x9e3779b97f4a7c15ull), 29) * 0xff51afd7ed558ccdull + a;
    }
    void add(const void *p, size_t n) {
        const unsigned char *c = (const unsigned char *)p;
        size_t i = 0;
        for (; i + 8 <= n; i += 8) {
            uint64_t w;
            std::memcpy(&w, c + i, 8);
            word(w);
        }
        if (i < n) {
            uint64_t w = 0;
            std::memcpy(&w, c + i, n - i);
            word(w);
        }
        word((uint64_t)n);
    }
    template <typename T> void add(const T &v) { add(&v, sizeof(T)); }
    bool operator==(const Sig &o) const { return a == o.a && b == o.b; }
};
struct SigHash {
    size_t operator()(const Sig &s) const { return (size_t)(s.a ^ (s.b * 31)); }
};

inline void add_layout(Sig &s, const g2g_layout_desc *d) {
    s.add(d->n_block_rows);
    s.add(d->n_block_cols);
    s.add(d->n_ranks);
    s.add(d->n_reordering);
    s.add(d->n_blocks);
    if (d->rows_split && d->n_block_rows >= 0)
        s.add(d->rows_split, sizeof(int32_t) * ((size_t)d->n_block_rows + 1));
    if (d->cols_split && d->n_block_cols >= 0)
        s.add(d->cols_split, sizeof(int32_t) * ((size_t)d->n_block_cols + 1));
    if (d->owners && d->n_block_rows > 0 && d->n_block_cols > 0)
        s.add(d->owners, sizeof(int32_t) * (size_t)d->n_block_rows * d->n_block_cols);
    if (d->reordering && d->n_reordering > 0)
        s.add(d->reordering, sizeof(int32_t) * (size_t)d->n_reordering);
    if (d->blocks && d->n_blocks > 0)
        s.add(d->blocks, sizeof(g2g_block_desc) * (size_t)d->n_blocks);
}

// Plans (through `make` on a miss) or finds in the one-shot plan cache the
// plan stored under `key` (null: no caching), executes it on `stream` and
// waits: the blocking calls' common path.
g2g_status cached_one_shot(const Sig *key, const std::function<g2g_status(g2g_plan **)> &make,
                           void *stream);

} // namespace g2g
