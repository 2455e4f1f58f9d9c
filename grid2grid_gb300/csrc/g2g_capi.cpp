// Host side of the C ABI (include/grid2grid_gb300.h): descriptor validation,
// the dense block tables, plan lifetime, execution, graph capture, tuning.
//
// Validation turns every condition under which the reference throws
// (interval.cpp:5-17, grid2D.cpp:29-43, block.cpp:167-174,
// grid_cover.hpp:57-62) or asserts (communication_data.cpp:227-239,
// grid_cover.cpp:70, grid2D.cpp:117) -- or silently hangs in MPI because a
// block is not held by its owner -- into G2G_ERROR_INVALID_ARGUMENT with a
// message, before any device work is queued.
#include "../../include/grid2grid_gb300.h"
#include "g2g_host.hpp"
#include "g2g_internal.hpp"
#include "g2g_launch.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <list>
#include <map>
#include <functional>
#include <mutex>
#include <unordered_map>
#include <string>
#include <vector>

namespace {
thread_local std::string t_last_error;
}

namespace g2g {
g2g_status fail(g2g_status st, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_last_error = buf;
    return st;
}
} // namespace g2g

namespace {
using g2g::fail;

#define G2G_CUDA(call)                                                                  \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return fail(e_ == cudaErrorMemoryAllocation ? G2G_ERROR_OUT_OF_MEMORY       \
                                                        : G2G_ERROR_CUDA,               \
                        "CUDA error %s (%s) at %s:%d", cudaGetErrorName(e_),            \
                        cudaGetErrorString(e_), __FILE__, __LINE__);                    \
    } while (0)

int dtype_esz(int dt) {
    switch (dt) {
    case G2G_FLOAT32: return 4;
    case G2G_FLOAT64: return 8;
    case G2G_COMPLEX64: return 8;
    case G2G_COMPLEX128: return 16;
    default: return 0;
    }
}
uint32_t esz_code(int esz) { return esz == 4 ? 0u : esz == 8 ? 1u : 2u; }
bool dtype_complex(int dt) { return dt == G2G_COMPLEX64 || dt == G2G_COMPLEX128; }

// --------------------------------------------------------------- per device
struct DeviceState {
    int sm_count = 0;
    cudaStream_t plan_stream = nullptr;
    // Pinned staging for plan uploads; planning holds `mu` from the upload
    // to the synchronisation that ends it, so one buffer serves all plans.
    std::mutex mu;
    void *pinned = nullptr;
    size_t pinned_bytes = 0;
};
std::mutex g_dev_mu;
std::map<int, DeviceState> g_devices;

g2g_status device_state(DeviceState **out, int *dev_out) {
    int dev = 0;
    G2G_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_dev_mu);
    DeviceState &ds = g_devices[dev];
    if (!ds.plan_stream) {
        G2G_CUDA(cudaDeviceGetAttribute(&ds.sm_count, cudaDevAttrMultiProcessorCount, dev));
        G2G_CUDA(cudaStreamCreateWithFlags(&ds.plan_stream, cudaStreamNonBlocking));
    }
    *out = &ds;
    if (dev_out)
        *dev_out = dev;
    return G2G_SUCCESS;
}

// ------------------------------------------------------------ host layouts
struct HBlock {
    int rank, row, col;
    bool trans, conj;
    int64_t stride;
    uint64_t data;
};

struct HLayout {
    std::vector<int32_t> rs, cs, owners;
    std::vector<int32_t> reo;
    int n_ranks = 0;
    std::vector<HBlock> blocks;
    int nbr() const { return (int)rs.size() - 1; }
    int nbc() const { return (int)cs.size() - 1; }
    int owner(int i, int j) const {
        int r = owners[(size_t)i * nbc() + j];
        return reo.empty() ? r : reo[r];
    }
};

g2g_status check_splits(const int32_t *s, int n, const char *what, const char *which) {
    if (n < 0)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: negative number of %s blocks",
                    which, what);
    if (!s)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: %s_split is NULL", which, what);
    for (int i = 0; i <= n; ++i) {
        if (s[i] < 0)
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "%s layout: %s_split[%d] = %d is negative (interval bounds must be "
                        ">= 0)",
                        which, what, i, s[i]);
        if (i && s[i] < s[i - 1])
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "%s layout: %s_split is decreasing at index %d (%d > %d); "
                        "intervals need start <= end",
                        which, what, i, s[i - 1], s[i]);
    }
    return G2G_SUCCESS;
}

// Reads and validates one layout descriptor. `P` is the number of virtual
// ranks of the transform (the communicator size). A partial layout (one
// shard's part of a layout spread over several processes, or a packed
// exchange buffer) lists only some blocks: with `held` set, exactly the
// blocks owned by the ranks r with held[r] != 0; with `absent_ok`, any
// subset. Blocks not listed take no part in the plan.
g2g_status load_layout(const g2g_layout_desc *d, const char *which, int P, bool is_final,
                       int align, HLayout &L, const std::vector<char> *held = nullptr,
                       bool absent_ok = false) {
    if (!d)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout descriptor is NULL", which);
    G2G_TRY(check_splits(d->rows_split, d->n_block_rows, "rows", which));
    G2G_TRY(check_splits(d->cols_split, d->n_block_cols, "cols", which));
    const int nbr = d->n_block_rows, nbc = d->n_block_cols;
    L.rs.assign(d->rows_split, d->rows_split + nbr + 1);
    L.cs.assign(d->cols_split, d->cols_split + nbc + 1);
    L.n_ranks = d->n_ranks;
    if (d->n_ranks < 0)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: negative n_ranks", which);
    const size_t nblk = (size_t)nbr * (size_t)nbc;
    if (nblk && !d->owners)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: owners is NULL", which);
    L.owners.assign(d->owners, d->owners + nblk);
    if (d->n_reordering < 0 || (d->n_reordering > 0 && !d->reordering))
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: bad rank reordering", which);
    if (d->n_reordering > 0) {
        L.reo.assign(d->reordering, d->reordering + d->n_reordering);
        for (int r : L.reo)
            if (r < 0 || r >= P)
                return fail(G2G_ERROR_INVALID_ARGUMENT,
                            "%s layout: reordering maps to rank %d outside [0, %d)", which,
                            r, P);
    }
    const int owner_limit =
        L.reo.empty() ? d->n_ranks : std::max((int)L.reo.size(), d->n_ranks);
    for (size_t k = 0; k < nblk; ++k) {
        int o = L.owners[k];
        if (o < 0 || o >= owner_limit || (!L.reo.empty() && o >= (int)L.reo.size()))
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "%s layout: block (%d, %d) has owner %d outside [0, %d)", which,
                        (int)(k / (size_t)std::max(nbc, 1)), (int)(k % (size_t)std::max(nbc, 1)),
                        o, owner_limit);
        if (L.reo.empty() && o >= P)
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "%s layout: owner %d is not a rank of the transform (%d ranks)",
                        which, o, P);
    }
    if (d->n_blocks < 0 || (d->n_blocks > 0 && !d->blocks))
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: bad local block list", which);
    std::vector<char> seen(nblk, 0);
    L.blocks.resize(d->n_blocks);
    for (int b = 0; b < d->n_blocks; ++b) {
        const g2g_block_desc &bd = d->blocks[b];
        if (bd.rank < 0 || bd.rank >= P)
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "%s layout: local block %d belongs to rank %d outside [0, %d)", which,
                        b, bd.rank, P);
        if (bd.row < 0 || bd.row >= nbr || bd.col < 0 || bd.col >= nbc)
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "%s layout: local block %d has coordinates (%d, %d) outside the "
                        "%d x %d grid",
                        which, b, bd.row, bd.col, nbr, nbc);
        size_t idx = (size_t)bd.row * nbc + bd.col;
        if (seen[idx])
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "%s layout: block (%d, %d) is listed more than once", which, bd.row,
                        bd.col);
        seen[idx] = 1;
        int own = L.owner(bd.row, bd.col);
        if (own != bd.rank)
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "%s layout: block (%d, %d) is held by rank %d but owned by rank %d",
                        which, bd.row, bd.col, bd.rank, own);
        if (held && !(*held)[bd.rank])
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "%s layout: block (%d, %d) of rank %d is listed, but rank %d belongs "
                        "to another shard",
                        which, bd.row, bd.col, bd.rank, bd.rank);
        if (is_final && bd.transpose_on_copy)
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "final layout: block (%d, %d) is marked transpose_on_copy; a "
                        "destination block cannot be transposed",
                        bd.row, bd.col);
        const int64_t nr = L.rs[bd.row + 1] - L.rs[bd.row];
        const int64_t nc = L.cs[bd.col + 1] - L.cs[bd.col];
        const int64_t srows = bd.transpose_on_copy ? nc : nr; // storage rows
        const int64_t scols = bd.transpose_on_copy ? nr : nc;
        if (nr > 0 && nc > 0) {
            if (!bd.data)
                return fail(G2G_ERROR_INVALID_ARGUMENT,
                            "%s layout: block (%d, %d) has a NULL data pointer", which,
                            bd.row, bd.col);
            if (((uintptr_t)bd.data) % (uintptr_t)align != 0)
                return fail(G2G_ERROR_INVALID_ARGUMENT,
                            "%s layout: block (%d, %d) data pointer is not aligned to its "
                            "element type (%d bytes)",
                            which, bd.row, bd.col, align);
            if (bd.stride < 1 || (scols > 1 && bd.stride < srows))
                return fail(G2G_ERROR_INVALID_ARGUMENT,
                            "%s layout: block (%d, %d) has stride %lld < %lld stored rows",
                            which, bd.row, bd.col, (long long)bd.stride, (long long)srows);
        }
        HBlock hb;
        hb.rank = bd.rank;
        hb.row = bd.row;
        hb.col = bd.col;
        hb.trans = bd.transpose_on_copy != 0;
        hb.conj = hb.trans && bd.conjugate_on_copy != 0; // conj acts only with transpose
        hb.stride = bd.stride;
        hb.data = (uint64_t)(uintptr_t)bd.data;
        L.blocks[b] = hb;
    }
    for (size_t k = 0; k < nblk && !absent_ok; ++k)
        if (!seen[k]) {
            int i = (int)(k / (size_t)nbc), j = (int)(k % (size_t)nbc);
            if (held && !(*held)[L.owner(i, j)])
                continue;
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "%s layout: block (%d, %d) owned by rank %d is missing from that "
                        "rank's local blocks",
                        which, i, j, L.owner(i, j));
        }
    return G2G_SUCCESS;
}

// grid_layout::transpose_or_conjugate (grid_layout.hpp:18-25): transposes the
// grid and the owners and marks every block (block.cpp:249-288).
void transpose_layout(HLayout &L, char flag) {
    if (flag != 'T' && flag != 'C')
        return;
    const int nbr = L.nbr(), nbc = L.nbc();
    std::vector<int32_t> t((size_t)nbr * nbc);
    for (int i = 0; i < nbr; ++i)
        for (int j = 0; j < nbc; ++j)
            t[(size_t)j * nbr + i] = L.owners[(size_t)i * nbc + j];
    L.owners.swap(t);
    std::swap(L.rs, L.cs);
    for (HBlock &b : L.blocks) {
        std::swap(b.row, b.col);
        b.trans = true;
        if (flag == 'C')
            b.conj = true;
    }
}

// ------------------------------------------------------------------- plans
struct PairHost {
    HLayout a, b; // a: initial after op, b: final
    int dtype = 0;     // the final layout's element type
    int esz = 0;
    int src_dtype = 0; // the initial layout's (another one: a fused cast)
    int src_esz = 0;
    bool cast = false;
    bool scaled = false;
    bool any_trans = false;
    double alpha[2] = {1, 0}, beta[2] = {0, 0};
    int64_t m = 0, n = 0;
    int64_t elems = 0; // elements the pair moves: m*n, fewer for a partial plan
};

g2g_tuning default_tuning() {
    g2g_tuning t;
    std::memset(&t, 0, sizeof(t));
    t.tile_bytes = 16 * 1024;
    t.tile_dim = 32;
    t.ctas_per_sm = 8;
    t.threads = 256;
    t.unroll = 4;
    t.stages = -1; // TMA staging is opt-in (no faster on measured workloads)
    t.ring = 1;
    t.tile_run = 1;
    t.l2_prefetch = -1;
    t.tensor_boxes = -1;
    return t;
}

g2g_tuning merge_tuning(const g2g_tuning &base, const g2g_tuning *over) {
    g2g_tuning t = base;
    if (!over)
        return t;
    if (over->tile_bytes) t.tile_bytes = over->tile_bytes;
    if (over->tile_dim) t.tile_dim = over->tile_dim;
    if (over->ctas_per_sm) t.ctas_per_sm = over->ctas_per_sm;
    if (over->threads) t.threads = over->threads;
    if (over->unroll) t.unroll = over->unroll;
    if (over->stages) t.stages = over->stages;
    if (over->ring) t.ring = over->ring;
    if (over->tile_run) t.tile_run = over->tile_run;
    if (over->l2_prefetch) t.l2_prefetch = over->l2_prefetch;
    if (over->tensor_boxes) t.tensor_boxes = over->tensor_boxes;
    return t;
}

g2g_status check_tuning(const g2g_tuning &t) {
    if (t.tile_bytes < 512 || t.tile_bytes > (1 << 24))
        return fail(G2G_ERROR_INVALID_ARGUMENT, "tuning: tile_bytes %d outside [512, 16M]",
                    t.tile_bytes);
    if (t.tile_dim != 16 && t.tile_dim != 32)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "tuning: tile_dim must be 16 or 32");
    if (t.threads != 256 && t.threads != 512)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "tuning: threads must be 256 or 512");
    if (t.unroll != 1 && t.unroll != 2 && t.unroll != 4)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "tuning: unroll must be 1, 2 or 4");
    if (t.stages != -1 && (t.stages < 2 || t.stages > 4))
        return fail(G2G_ERROR_INVALID_ARGUMENT, "tuning: stages must be -1 or 2..4");
    if (t.ring != -1 && t.ring != 1)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "tuning: ring must be -1 or 1");
    if (t.tile_run < 1 || t.tile_run > 64 || (t.tile_run & (t.tile_run - 1)))
        return fail(G2G_ERROR_INVALID_ARGUMENT, "tuning: tile_run must be a power of two in [1, 64]");
    if (t.l2_prefetch != -1 && t.l2_prefetch != 1)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "tuning: l2_prefetch must be -1 or 1");
    if (t.tensor_boxes != -1 && t.tensor_boxes != 1)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "tuning: tensor_boxes must be -1 or 1");
    if (t.ctas_per_sm < 1 || t.ctas_per_sm > 32)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "tuning: ctas_per_sm outside [1, 32]");
    return G2G_SUCCESS;
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

} // namespace

struct g2g_plan {
    int device = 0;
    int sm_count = 0;
    int n_pairs = 0;
    int n_ranks = 0;
    std::vector<PairHost> host;
    std::vector<g2g::PairInfo> pinfo;
    std::vector<int32_t> splits;
    std::vector<g2g::SrcEntry> src_tables;
    std::vector<g2g::DstEntry> dst_tables;
    int64_t n_parts = 0, n_cells = 0, max_cells_per_pair = 0;
    int64_t bytes_moved = 0, bytes_min_traffic = 0;
    bool any_trans = false;
    int max_trans_esz = 0;
    int paths = 0; // tile paths the work list needs (1 copy, 2 transpose,
                   // 4 scaled real, 8 scaled complex, 16 cast, 32 transposes
                   // of 4- or 8-byte elements)
    bool host_memory = false; // some block lives in pinned host memory
    g2g_tuning tuning;
    // device
    void *dmem = nullptr;
    size_t dmem_bytes = 0;
    g2g::PlanDevice dev;
    long long n_tiles = 0; // copy tiles + CTA-level tiles
    long long n_copy = 0;
    long long n_pieces = 0;
    cudaStream_t last_stream = nullptr;
    cudaEvent_t done = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaStream_t graph_stream = nullptr;
    // plain copies as tensor-map boxes (built when the tuning first asks)
    bool tma_ok = false;
    int tma_esz = 0, tma_box_rows = 0, tma_box_cols = 0;
    void *tma_mem = nullptr;
    g2g::TmaPlan tma;
};

namespace g2g {
int64_t plan_bytes_moved(const g2g_plan *plan) { return plan ? plan->bytes_moved : 0; }
} // namespace g2g

namespace {

int64_t tile_capacity_bound(const PairHost &p, const g2g_tuning &t) {
    const int64_t pr = p.a.nbr() + p.b.nbr() + 1, pc = p.a.nbc() + p.b.nbc() + 1;
    int64_t bound = 0;
    bool has_plain = false, has_trans = false;
    for (const HBlock &b : p.a.blocks) {
        if (b.trans) has_trans = true; else has_plain = true;
    }
    if (has_trans) {
        const int64_t td = t.tile_dim;
        bound += (p.m / td + pr) * (p.n / td + pc);
    }
    if (has_plain) {
        const int64_t tile_rows = std::max<int64_t>(1, 4096 / p.esz);
        const int64_t tcmin = std::max<int64_t>(1, t.tile_bytes / (tile_rows * p.esz));
        bound += (p.m / tile_rows + pr) * (p.n / tcmin + pc);
    }
    return bound;
}

// A fused cast converts float <-> double, complex<float> <-> complex<double>
// (each part) and real -> complex (imaginary part +0).
bool cast_supported(int from, int to) {
    const bool fc = dtype_complex(from), tc = dtype_complex(to);
    return from != to && !(fc && !tc);
}

g2g_status build_pair(const g2g_layout_desc *di, const g2g_layout_desc *df, int dtype,
                      const g2g_op *op, int pair_index, PairHost &p, int src_dtype = -1,
                      const g2g::PartialSpec *part = nullptr) {
    (void)pair_index;
    p.dtype = dtype;
    p.esz = dtype_esz(dtype);
    if (!p.esz)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "unknown dtype %d", dtype);
    p.src_dtype = src_dtype < 0 ? dtype : src_dtype;
    p.src_esz = dtype_esz(p.src_dtype);
    if (!p.src_esz)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "unknown source dtype %d", p.src_dtype);
    p.cast = p.src_dtype != dtype;
    if (p.cast && !cast_supported(p.src_dtype, dtype))
        return fail(G2G_ERROR_UNSUPPORTED,
                    "cast from dtype %d to dtype %d is not supported (complex to real)",
                    p.src_dtype, dtype);
    if (!di || !df)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "layout descriptor is NULL");
    const int P = std::max(1, std::max(di->n_ranks, df->n_ranks));
    // element alignment: that of the real component (float or double)
    auto comp_align = [](int dt) { return (dt == G2G_FLOAT32 || dt == G2G_COMPLEX64) ? 4 : 8; };
    if (part && ((part->init_held && (int)part->init_held->size() < P) ||
                 (part->final_held && (int)part->final_held->size() < P)))
        return fail(G2G_ERROR_INVALID_ARGUMENT, "shard rank sets must cover all %d ranks", P);
    G2G_TRY(load_layout(di, "initial", P, false, comp_align(p.src_dtype), p.a,
                        part ? part->init_held : nullptr, part && part->init_absent_ok));
    G2G_TRY(load_layout(df, "final", P, true, comp_align(dtype), p.b,
                        part ? part->final_held : nullptr, part && part->final_absent_ok));
    char trans = 'N';
    if (op) {
        trans = (char)std::toupper((unsigned char)op->trans);
        if (trans != 'N' && trans != 'T' && trans != 'C')
            return fail(G2G_ERROR_INVALID_ARGUMENT, "trans must be 'N', 'T' or 'C', got '%c'",
                        op->trans);
        p.alpha[0] = op->alpha[0];
        p.alpha[1] = op->alpha[1];
        p.beta[0] = op->beta[0];
        p.beta[1] = op->beta[1];
        if (!dtype_complex(dtype) && (p.alpha[1] != 0.0 || p.beta[1] != 0.0))
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "alpha/beta have an imaginary part but the dtype is real");
    }
    transpose_layout(p.a, trans);
    if (p.a.rs.front() != p.b.rs.front() || p.a.rs.back() != p.b.rs.back() ||
        p.a.cs.front() != p.b.cs.front() || p.a.cs.back() != p.b.cs.back())
        return fail(G2G_ERROR_INVALID_ARGUMENT,
                    "initial (after op '%c') and final layouts cover different matrices: "
                    "rows [%d, %d) vs [%d, %d), cols [%d, %d) vs [%d, %d)",
                    trans, p.a.rs.front(), p.a.rs.back(), p.b.rs.front(), p.b.rs.back(),
                    p.a.cs.front(), p.a.cs.back(), p.b.cs.front(), p.b.cs.back());
    // (alpha, beta) == (1, 0) in the element type is a plain copy
    // (memory_utils.hpp:92-95, communication_data.cpp:165)
    if (dtype == G2G_FLOAT32 || dtype == G2G_COMPLEX64) {
        float ar = (float)p.alpha[0], ai = (float)p.alpha[1];
        float br = (float)p.beta[0], bi = (float)p.beta[1];
        p.scaled = !(ar == 1.0f && ai == 0.0f && br == 0.0f && bi == 0.0f);
    } else {
        p.scaled = !(p.alpha[0] == 1.0 && p.alpha[1] == 0.0 && p.beta[0] == 0.0 &&
                     p.beta[1] == 0.0);
    }
    if (p.cast && p.scaled)
        return fail(G2G_ERROR_UNSUPPORTED, "a cast transform takes alpha = 1, beta = 0");
    for (const HBlock &b : p.a.blocks)
        if (b.trans)
            p.any_trans = true;
    p.m = p.b.rs.back() - p.b.rs.front();
    p.n = p.b.cs.back() - p.b.cs.front();
    p.elems = (part && part->elems >= 0) ? part->elems : p.m * p.n;
    return G2G_SUCCESS;
}

// Lays out the plan's host arrays and PairInfo offsets.
void assemble(g2g_plan &pl) {
    pl.pinfo.resize(pl.n_pairs);
    pl.splits.clear();
    pl.src_tables.clear();
    pl.dst_tables.clear();
    pl.n_parts = 0;
    pl.n_cells = 0;
    pl.max_cells_per_pair = 0;
    pl.bytes_moved = 0;
    pl.bytes_min_traffic = 0;
    pl.any_trans = false;
    pl.max_trans_esz = 0;
    pl.paths = 0;
    // every CTA-level tile a plain transpose of 4-byte (8-byte) elements;
    // every tile a scaled transpose of 4-byte (8-byte) elements
    bool only_w4 = true, only_w8 = true, only_w16 = true, only_w4s = true, only_w8s = true;
    for (int k = 0; k < pl.n_pairs; ++k) {
        PairHost &p = pl.host[k];
        g2g::PairInfo &pi = pl.pinfo[k];
        std::memset(&pi, 0, sizeof(pi));
        pi.a_nr = p.a.nbr();
        pi.a_nc = p.a.nbc();
        pi.b_nr = p.b.nbr();
        pi.b_nc = p.b.nbc();
        pi.a_rs = (int32_t)pl.splits.size();
        pl.splits.insert(pl.splits.end(), p.a.rs.begin(), p.a.rs.end());
        pi.a_cs = (int32_t)pl.splits.size();
        pl.splits.insert(pl.splits.end(), p.a.cs.begin(), p.a.cs.end());
        pi.b_rs = (int32_t)pl.splits.size();
        pl.splits.insert(pl.splits.end(), p.b.rs.begin(), p.b.rs.end());
        pi.b_cs = (int32_t)pl.splits.size();
        pl.splits.insert(pl.splits.end(), p.b.cs.begin(), p.b.cs.end());
        pi.src_table = (int64_t)pl.src_tables.size();
        pl.src_tables.resize(pl.src_tables.size() + (size_t)pi.a_nr * pi.a_nc);
        for (const HBlock &b : p.a.blocks) {
            g2g::SrcEntry &e = pl.src_tables[pi.src_table + (int64_t)b.row * pi.a_nc + b.col];
            e.data = b.data;
            e.ld = b.stride;
            e.flags = (b.trans ? 1u : 0u) | (b.conj && dtype_complex(p.dtype) ? 2u : 0u);
            e.pad = 0;
        }
        pi.dst_table = (int64_t)pl.dst_tables.size();
        pl.dst_tables.resize(pl.dst_tables.size() + (size_t)pi.b_nr * pi.b_nc);
        for (const HBlock &b : p.b.blocks) {
            g2g::DstEntry &e = pl.dst_tables[pi.dst_table + (int64_t)b.row * pi.b_nc + b.col];
            e.data = b.data;
            e.ld = b.stride;
        }
        pi.row_parts = pl.n_parts;
        pl.n_parts += pi.a_nr + pi.b_nr + 2;
        pi.col_parts = pl.n_parts;
        pl.n_parts += pi.a_nc + pi.b_nc + 2;
        const int64_t cells = (int64_t)(pi.a_nr + pi.b_nr + 1) * (pi.a_nc + pi.b_nc + 1);
        pi.cells = pl.n_cells;
        pl.n_cells += cells;
        pl.max_cells_per_pair = std::max(pl.max_cells_per_pair, cells);
        // scaled and cast tiles are warp-level when no destination element
        // straddles a 16-byte chunk: every final block starts on a multiple
        // of min(sizeof(T), 16) bytes (column and row offsets keep that)
        bool dst_chunked = true;
        for (const HBlock &b : p.b.blocks)
            dst_chunked = dst_chunked && b.data % (uint64_t)std::min(p.esz, 16) == 0;
        const bool warp_elem = (p.scaled || p.cast) && dst_chunked;
        pi.kind = esz_code(p.esz) | ((uint32_t)p.dtype << g2g::KIND_DTYPE_SHIFT) |
                  (p.scaled ? g2g::KIND_SCALED : 0u) |
                  (warp_elem ? g2g::KIND_WARP_ELEM : 0u) |
                  (p.cast ? (g2g::KIND_CAST |
                             ((uint32_t)p.src_dtype << g2g::KIND_SRC_DTYPE_SHIFT))
                          : 0u);
        pi.tile_rows = (int32_t)std::max(1, 4096 / p.esz);
        pi.tile_bytes = pl.tuning.tile_bytes;
        pi.tile_dim = pl.tuning.tile_dim;
        {
            bool all_trans = !p.a.blocks.empty();
            for (const HBlock &b : p.a.blocks)
                all_trans = all_trans && b.trans;
            pi.row_major_cells = all_trans ? 1 : 0;
        }
        pi.alpha[0] = p.alpha[0];
        pi.alpha[1] = p.alpha[1];
        pi.beta[0] = p.beta[0];
        pi.beta[1] = p.beta[1];
        const int64_t bytes = p.elems * p.esz;
        pl.bytes_moved += bytes;
        pl.bytes_min_traffic += p.cast ? p.elems * (p.src_esz + p.esz)
                                       : (p.scaled ? 3 : 2) * bytes;
        if (p.any_trans) {
            pl.any_trans = true;
            pl.max_trans_esz = std::max(pl.max_trans_esz, p.esz);
        }
        bool any_plain = false;
        for (const HBlock &b : p.a.blocks)
            if (!b.trans)
                any_plain = true;
        if (p.cast)
            pl.paths |= 16 | (warp_elem && any_plain ? 1 : 0);
        else if (p.scaled) // real and complex arithmetic are separate kernel paths
            pl.paths |= ((p.dtype == G2G_COMPLEX64 || p.dtype == G2G_COMPLEX128) ? 8 : 4) |
                        (warp_elem && any_plain ? 1 : 0);
        else // 32: plain transposes of 4- or 8-byte elements (wide / tall tiles)
            pl.paths |= (any_plain ? 1 : 0) | (p.any_trans ? 2 : 0) |
                        (p.any_trans && p.esz <= 8 ? 32 : 0);
        if (p.cast || p.scaled || (p.any_trans && p.esz != 4))
            only_w4 = false;
        if (p.cast || p.scaled || (p.any_trans && p.esz != 8))
            only_w8 = false;
        if (p.cast || p.scaled || (p.any_trans && p.esz != 16))
            only_w16 = false;
        if (!p.scaled || p.cast || any_plain || p.esz != 4)
            only_w4s = false;
        if (!p.scaled || p.cast || any_plain || p.esz != 8)
            only_w8s = false;
    }
    if (only_w4 && (pl.paths & 2))
        pl.paths |= 64;
    if (only_w8 && (pl.paths & 2))
        pl.paths |= 128;
    if (only_w16 && (pl.paths & 2))
        pl.paths |= 256;
    if (only_w4s && pl.n_pairs > 0)
        pl.paths |= 1024;
    if (only_w8s && pl.n_pairs > 0)
        pl.paths |= 2048;
}

// Makes the device that holds the plan's blocks current for this library's
// runtime (callers such as torch keep their own current-device state).
// Picks the device of the plan's device-memory blocks and notes blocks in
// pinned host memory (reachable from the GPU at the same address: the kernel
// then reads or writes them over the host link). Pageable memory is refused.
// Attributes are looked up once per 2 MB of address space.
g2g_status bind_device(g2g_plan &pl) {
    std::unordered_map<uintptr_t, int> seen; // 2 MB region -> cudaMemoryType
    int device = -1;
    for (const PairHost &p : pl.host)
        for (const HLayout *L : {&p.a, &p.b})
            for (const HBlock &b : L->blocks) {
                if (!b.data)
                    continue;
                const uintptr_t region = (uintptr_t)b.data >> 21;
                auto it = seen.find(region);
                int type;
                if (it != seen.end()) {
                    type = it->second;
                } else {
                    cudaPointerAttributes attr;
                    G2G_CUDA(cudaPointerGetAttributes(&attr, (const void *)(uintptr_t)b.data));
                    type = (int)attr.type;
                    if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) {
                        if (device < 0)
                            device = attr.device;
                    } else if (attr.type != cudaMemoryTypeHost) {
                        return fail(G2G_ERROR_INVALID_ARGUMENT,
                                    "block data at %p is neither device memory nor pinned host "
                                    "memory (pin it with cudaHostRegister / cudaHostAlloc)",
                                    (void *)(uintptr_t)b.data);
                    }
                    seen.emplace(region, type);
                }
                if (type == (int)cudaMemoryTypeHost)
                    pl.host_memory = true;
            }
    if (device >= 0)
        G2G_CUDA(cudaSetDevice(device));
    return G2G_SUCCESS;
}

// Allocates device memory, uploads, runs the device planner, waits for it.
g2g_status plan_on_device(g2g_plan &pl) {
    DeviceState *ds = nullptr;
    G2G_TRY(device_state(&ds, &pl.device));
    pl.sm_count = ds->sm_count;
    int64_t capacity = 0;
    for (const PairHost &p : pl.host)
        capacity += tile_capacity_bound(p, pl.tuning);
    capacity = std::max<int64_t>(capacity, 1);

    // sub-buffer layout of the single allocation
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = align_up(off + std::max<size_t>(bytes, 1), 256);
        return o;
    };
    const size_t o_pairs = take(sizeof(g2g::PairInfo) * pl.pinfo.size());
    const size_t o_splits = take(sizeof(int32_t) * pl.splits.size());
    const size_t o_src = take(sizeof(g2g::SrcEntry) * pl.src_tables.size());
    const size_t o_dst = take(sizeof(g2g::DstEntry) * pl.dst_tables.size());
    const size_t upload_end = off;
    const size_t o_parts = take(sizeof(g2g::Part) * (size_t)pl.n_parts);
    const size_t o_cells = take(sizeof(long long) * (size_t)pl.n_cells);
    const size_t o_cells_cta = take(sizeof(long long) * (size_t)pl.n_cells);
    const size_t o_sums = take(sizeof(long long) * (size_t)g2g::scan_sums_capacity(pl.n_cells));
    const size_t o_counters = take(64);
    const size_t o_tiles = take(sizeof(g2g::Tile) * (size_t)capacity);
    const size_t total = off;

    if (pl.dmem && pl.dmem_bytes < total) {
        G2G_CUDA(cudaStreamSynchronize(ds->plan_stream));
        G2G_CUDA(cudaFreeAsync(pl.dmem, ds->plan_stream));
        pl.dmem = nullptr;
    }
    if (!pl.dmem) {
        G2G_CUDA(cudaMallocAsync(&pl.dmem, total, ds->plan_stream));
        pl.dmem_bytes = total;
    }
    char *base = (char *)pl.dmem;
    g2g::PlanDevice &d = pl.dev;
    d.pairs = (g2g::PairInfo *)(base + o_pairs);
    d.splits = (int32_t *)(base + o_splits);
    d.src_tables = (g2g::SrcEntry *)(base + o_src);
    d.dst_tables = (g2g::DstEntry *)(base + o_dst);
    d.parts = (g2g::Part *)(base + o_parts);
    d.cell_tiles = (long long *)(base + o_cells);
    d.cell_tiles_cta = (long long *)(base + o_cells_cta);
    d.scan_sums = (long long *)(base + o_sums);
    d.n_copy = (long long *)(base + o_counters);
    d.n_pieces = (unsigned long long *)(base + o_counters + 8);
    d.overflow = (int *)(base + o_counters + 16);
    d.status = (int *)(base + o_counters + 24);
    d.n_cta = (long long *)(base + o_counters + 32);
    d.tiles = (g2g::Tile *)(base + o_tiles);
    d.tile_capacity = capacity;
    d.max_cells_per_pair = pl.max_cells_per_pair;

    // one pinned staging copy of everything the host built
    std::vector<char> staging(upload_end, 0);
    std::memcpy(staging.data() + o_pairs, pl.pinfo.data(),
                sizeof(g2g::PairInfo) * pl.pinfo.size());
    if (!pl.splits.empty())
        std::memcpy(staging.data() + o_splits, pl.splits.data(),
                    sizeof(int32_t) * pl.splits.size());
    if (!pl.src_tables.empty())
        std::memcpy(staging.data() + o_src, pl.src_tables.data(),
                    sizeof(g2g::SrcEntry) * pl.src_tables.size());
    if (!pl.dst_tables.empty())
        std::memcpy(staging.data() + o_dst, pl.dst_tables.data(),
                    sizeof(g2g::DstEntry) * pl.dst_tables.size());
    std::lock_guard<std::mutex> lk(ds->mu);
    if (ds->pinned_bytes < upload_end) {
        if (ds->pinned)
            cudaFreeHost(ds->pinned);
        ds->pinned = nullptr;
        ds->pinned_bytes = 0;
        size_t want = std::max<size_t>(upload_end, (size_t)1 << 20);
        G2G_CUDA(cudaMallocHost(&ds->pinned, want));
        ds->pinned_bytes = want;
    }
    void *pinned = ds->pinned;
    std::memcpy(pinned, staging.data(), upload_end);
    cudaError_t e = cudaMemcpyAsync(base, pinned, upload_end, cudaMemcpyHostToDevice,
                                    ds->plan_stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(base + o_counters, 0, 64, ds->plan_stream);
    if (e == cudaSuccess)
        e = g2g::launch_plan(d, pl.n_pairs, pl.n_cells, ds->plan_stream);
    long long counters[5] = {0, 0, 0, 0, 0};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(pinned, base + o_counters, 40, cudaMemcpyDeviceToHost,
                            ds->plan_stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(ds->plan_stream);
    if (e == cudaSuccess)
        std::memcpy(counters, pinned, 40);
    G2G_CUDA(e);
    if (((int *)counters)[4] != 0)
        return fail(G2G_ERROR_CUDA,
                    "internal error: tile work list exceeded its bound (%lld > %lld)",
                    counters[0] + counters[4], (long long)capacity);
    pl.n_copy = counters[0];
    pl.n_tiles = counters[0] + counters[4];
    pl.n_pieces = counters[1];
    return G2G_SUCCESS;
}

// Largest dynamic shared memory a CTA can opt into on sm_100-class GPUs.
constexpr size_t kMaxSmemPerCta = 227 * 1024;

// A launch runs the staged ring of 4- or 8-byte transposes when those, of
// one element size, are its only tiles (bit 64 or 128 set, no copy tiles).
bool uses_staged_ring(int paths) {
    return ((paths & ~(64 | 32)) == 2 && (paths & 64)) ||
           ((paths & ~(128 | 32)) == 2 && (paths & 128)) || paths == (2 | 256);
}
// ... and the staged ring of scaled transposes when every tile is a scaled
// transpose of one element size (bit 1024 or 2048 set).
bool uses_staged_scaled_ring(int paths) {
    return paths == (4 | 1024) || ((paths & 2048) && !(paths & ~(4 | 8 | 2048)));
}

g2g::ScatterConfig scatter_config(const g2g_plan &pl) {
    g2g::ScatterConfig c;
    c.threads = pl.tuning.threads;
    c.unroll = pl.tuning.unroll;
    c.ctas_per_sm = pl.tuning.ctas_per_sm;
    c.sm_count = pl.sm_count;
    c.tile_dim = pl.tuning.tile_dim;
    long long g = (long long)pl.sm_count * pl.tuning.ctas_per_sm;
    if (g > pl.n_tiles)
        g = pl.n_tiles;
    c.grid = (int)std::max<long long>(g, 1);
    c.smem_bytes = pl.max_trans_esz ? g2g::transpose_smem_bytes(c.tile_dim, pl.max_trans_esz)
                                    : 0;
    c.trans_bytes = c.smem_bytes;
    c.paths = pl.paths ? pl.paths : 1;
    // narrow transposes only: their staged ring, unless the tuning asks for
    // the register path or blocks live in host memory
    if (pl.tuning.ring == -1 || pl.host_memory)
        c.paths &= ~(64 | 128 | 256 | 1024 | 2048);
    if (uses_staged_ring(c.paths))
        c.smem_bytes = g2g::staged_transpose_smem_bytes(c.tile_dim);
    if (uses_staged_scaled_ring(c.paths))
        c.smem_bytes = g2g::staged_scaled_transpose_smem_bytes(c.tile_dim);
    // blocks in host memory take the register path: plain loads and stores
    c.ring = (pl.tuning.ring == 1 && !pl.host_memory) ? 1 : 0;
    c.run_shift = 0;
    while ((1 << c.run_shift) < pl.tuning.tile_run && c.run_shift < 6)
        ++c.run_shift;
    c.l2_prefetch = pl.tuning.l2_prefetch == 1 ? 1 : 0;
    c.stages = 0;
    if ((c.paths & 1) && pl.tuning.stages >= 2 && !pl.host_memory) {
        c.stage_bytes = g2g::stage_bytes_for(pl.tuning.tile_bytes);
        int st = pl.tuning.stages;
        while (st >= 2 && 128 + (size_t)st * c.stage_bytes + c.trans_bytes > kMaxSmemPerCta)
            --st;
        c.stages = st >= 2 ? st : 0;
    }
    if (c.ring && g2g::ring_smem_bytes(c) > kMaxSmemPerCta)
        c.ring = 0; // ring too large for one CTA: loads through registers
    return c;
}

void add_to_list(g2g::PlanList &l, const g2g_plan &pl) {
    g2g::PlanRef &r = l.p[l.n++];
    r.tiles = pl.dev.tiles;
    r.pairs = pl.dev.pairs;
    r.first_copy = l.total_copy;
    r.first_cta = l.total_cta;
    r.n_copy = pl.n_copy;
    l.total_copy += pl.n_copy;
    l.total_cta += pl.n_tiles - pl.n_copy;
}

g2g::PlanList single_list(const g2g_plan &pl) {
    g2g::PlanList l;
    l.status = pl.dev.status;
    add_to_list(l, pl);
    return l;
}

// Launches the gather-scatter over `l`. The TMA-staged kernel is the one that
// can raise the device status (a bounded wait that expired): its launches
// clear the status first, so the status always describes the last execution.
cudaError_t launch_list(const g2g::PlanList &l, const g2g::ScatterConfig &cfg, cudaStream_t s) {
    if (cfg.stages >= 2 && l.status) {
        cudaError_t e = cudaMemsetAsync(l.status, 0, sizeof(int), s);
        if (e != cudaSuccess)
            return e;
    }
    return g2g::launch_scatter(l, cfg, s);
}

// Configuration that covers every plan of a multi-plan launch: the union of
// their tile paths, the largest shared-memory need, the first plan's knobs.
g2g::ScatterConfig merged_config(g2g_plan *const *plans, int n) {
    g2g::ScatterConfig c = scatter_config(*plans[0]);
    long long tiles = 0;
    // bit 64 (128) holds for the launch when every plan with CTA-level tiles
    // has it, bit 1024 (2048) when every plan has it
    bool w4 = true, w8 = true, w16 = true, w4s = true, w8s = true;
    for (int k = 0; k < n; ++k) {
        const g2g::ScatterConfig ck = scatter_config(*plans[k]);
        if (plans[k]->host_memory) {
            c.ring = 0;
            c.stages = 0;
        }
        if ((ck.paths & (2 | 4 | 8 | 16)) && !(ck.paths & 64))
            w4 = false;
        if ((ck.paths & (2 | 4 | 8 | 16)) && !(ck.paths & 128))
            w8 = false;
        if ((ck.paths & (2 | 4 | 8 | 16)) && !(ck.paths & 256))
            w16 = false;
        if (!(ck.paths & 1024))
            w4s = false;
        if (!(ck.paths & 2048))
            w8s = false;
        c.paths |= ck.paths;
        c.trans_bytes = std::max(c.trans_bytes, ck.trans_bytes);
        tiles += plans[k]->n_tiles;
    }
    c.paths = (c.paths & ~(64 | 128 | 256 | 1024 | 2048)) | (w4 && (c.paths & 2) ? 64 : 0) |
              (w8 && (c.paths & 2) ? 128 : 0) | (w16 && (c.paths & 2) ? 256 : 0) |
              (w4s ? 1024 : 0) | (w8s ? 2048 : 0);
    c.smem_bytes = uses_staged_ring(c.paths) ? g2g::staged_transpose_smem_bytes(c.tile_dim)
                   : uses_staged_scaled_ring(c.paths)
                       ? g2g::staged_scaled_transpose_smem_bytes(c.tile_dim)
                       : c.trans_bytes;
    if (c.stages >= 2) {
        while (c.stages >= 2 &&
               128 + (size_t)c.stages * c.stage_bytes + c.trans_bytes > kMaxSmemPerCta)
            --c.stages;
        if (c.stages < 2)
            c.stages = 0;
    } else if (c.paths & 1) {
        c.stages = 0;
    }
    if (c.ring && g2g::ring_smem_bytes(c) > kMaxSmemPerCta)
        c.ring = 0;
    long long g = (long long)c.sm_count * plans[0]->tuning.ctas_per_sm;
    c.grid = (int)std::max<long long>(1, std::min(g, std::max<long long>(tiles, 1)));
    return c;
}

long long gcd_ll(long long a, long long b) {
    while (b) {
        const long long t = a % b;
        a = b;
        b = t;
    }
    return a < 0 ? -a : a;
}

// Whether the plan's pieces can move as 2-D tensor-map boxes, and the box:
// plain copies (no op arithmetic, no transposes, no casts) of one element
// size between device blocks at 16-byte aligned addresses with strides that
// are multiples of 16 bytes, every split point of both grids (from the
// first) a multiple of the box's rows and columns, so that every piece and
// its offsets in both blocks are whole boxes. A box is 2-16 KB.
void tma_eligibility(g2g_plan &pl) {
    pl.tma_ok = false;
    if (pl.host_memory || pl.n_pairs < 1)
        return;
    int esz = 0;
    long long gr = 0, gc = 0;
    for (const PairHost &p : pl.host) {
        if (p.scaled || p.cast || p.any_trans)
            return;
        if (esz && p.esz != esz)
            return;
        esz = p.esz;
        for (const HLayout *L : {&p.a, &p.b}) {
            for (int32_t x : L->rs)
                gr = gcd_ll(gr, x - L->rs.front());
            for (int32_t x : L->cs)
                gc = gcd_ll(gc, x - L->cs.front());
            for (const HBlock &b : L->blocks)
                if ((b.data & 15u) != 0 || ((uint64_t)b.stride * (uint64_t)esz) % 16u != 0)
                    return;
        }
    }
    if (gr <= 0 || gc <= 0)
        return;
    // rows: the largest divisor of gr whose bytes are a multiple of 16, at
    // most 256 map words; columns: the largest divisor of gc up to 256 that
    // keeps the box within 16 KB
    const int words_per_elem = esz <= 4 ? 1 : esz / 8;
    int br = 0;
    for (long long d = std::min<long long>(gr, 256 / words_per_elem); d >= 1; --d)
        if (gr % d == 0 && (d * esz) % 16 == 0 && d * esz <= 1024) {
            br = (int)d;
            break;
        }
    if (!br)
        return;
    int bc = 0;
    for (long long d = std::min<long long>(gc, 256); d >= 1; --d)
        if (gc % d == 0 && (long long)br * d * esz <= 16384) {
            bc = (int)d;
            break;
        }
    if (!bc || (long long)br * bc * esz < 2048)
        return;
    pl.tma_ok = true;
    pl.tma_esz = esz;
    pl.tma_box_rows = br;
    pl.tma_box_cols = bc;
}

// The merged partition of two split vectors: (start, length, interval of a,
// interval of b) of every non-empty part.
struct HPart {
    int32_t start, len, ia, ib;
};
std::vector<HPart> merge_parts(const std::vector<int32_t> &a, const std::vector<int32_t> &b) {
    std::vector<HPart> out;
    size_t i = 0, j = 0;
    int32_t pos = a.front();
    while (i + 1 < a.size() && j + 1 < b.size()) {
        const int32_t end = std::min(a[i + 1], b[j + 1]);
        if (end > pos)
            out.push_back({pos, end - pos, (int32_t)i, (int32_t)j});
        pos = std::max(pos, end);
        if (a[i + 1] <= pos)
            ++i;
        if (j + 1 < b.size() && b[j + 1] <= pos)
            ++j;
    }
    return out;
}

// Builds the tensor maps and the box list, and uploads them. Blocks of one
// rank with one stride whose origins lie in the columns of a common array
// (a ScaLAPACK local array: origin = row offset + column offset x stride)
// share one map over that array, addressed by the block's row and column
// offsets in it, so that a launch touches a few descriptors; any other
// block gets a map of its own.
g2g_status build_tma(g2g_plan &pl) {
    if (pl.tma_mem)
        return G2G_SUCCESS;
    const int esz = pl.tma_esz, br = pl.tma_box_rows, bc = pl.tma_box_cols;
    const int word = esz == 4 ? 4 : 8, wpe = esz / word;
    std::vector<unsigned char> maps;
    std::vector<g2g::TmaBox> boxes;
    struct Origin {
        int32_t map = -1;
        int64_t x = 0, y = 0; // element row and column of the block in its map
    };
    for (const PairHost &p : pl.host) {
        std::vector<Origin> aorg((size_t)p.a.nbr() * p.a.nbc()),
            borg((size_t)p.b.nbr() * p.b.nbc());
        for (int side = 0; side < 2; ++side) {
            const HLayout &L = side ? p.b : p.a;
            std::vector<Origin> &org = side ? borg : aorg;
            // groups of blocks by (rank, stride): the lowest origin is the base
            std::map<std::pair<int, int64_t>, std::vector<const HBlock *>> groups;
            for (const HBlock &b : L.blocks) {
                if (L.rs[b.row + 1] > L.rs[b.row] && L.cs[b.col + 1] > L.cs[b.col])
                    groups[{b.rank, b.stride}].push_back(&b);
            }
            for (auto &g : groups) {
                const int64_t ld = g.first.second, ldb = ld * esz;
                uint64_t base = UINT64_MAX;
                for (const HBlock *b : g.second)
                    base = std::min<uint64_t>(base, b->data);
                int64_t max_col = 0;
                std::vector<const HBlock *> own;
                std::vector<std::pair<const HBlock *, Origin>> shared;
                for (const HBlock *b : g.second) {
                    const uint64_t off = b->data - base;
                    const int64_t rows = L.rs[b->row + 1] - L.rs[b->row];
                    const int64_t cols = L.cs[b->col + 1] - L.cs[b->col];
                    Origin o;
                    o.y = (int64_t)(off / (uint64_t)ldb);
                    o.x = (int64_t)((off % (uint64_t)ldb) / (uint64_t)esz);
                    // (coordinates are 32-bit: far-apart blocks get maps of their own)
                    if (off % (uint64_t)esz != 0 || o.x + rows > ld ||
                        o.y + cols > (int64_t)INT32_MAX || (o.x + rows) * wpe > (int64_t)INT32_MAX) {
                        own.push_back(b);
                        continue;
                    }
                    max_col = std::max(max_col, o.y + cols);
                    shared.push_back({b, o});
                }
                if (!shared.empty()) {
                    const int32_t idx = (int32_t)(maps.size() / 128);
                    maps.resize(maps.size() + 128);
                    cudaError_t e = g2g::encode_box_map(
                        maps.data() + (size_t)idx * 128, (const void *)(uintptr_t)base, word,
                        (uint64_t)(ld * wpe), (uint64_t)max_col, (uint64_t)ldb,
                        (uint32_t)(br * wpe), (uint32_t)bc);
                    if (e != cudaSuccess)
                        return fail(G2G_ERROR_CUDA, "tensor map of a local array: %s",
                                    cudaGetErrorString(e));
                    for (auto &so : shared) {
                        so.second.map = idx;
                        org[(size_t)so.first->row * L.nbc() + so.first->col] = so.second;
                    }
                }
                for (const HBlock *b : own) {
                    const int64_t rows = L.rs[b->row + 1] - L.rs[b->row];
                    const int64_t cols = L.cs[b->col + 1] - L.cs[b->col];
                    const int32_t idx = (int32_t)(maps.size() / 128);
                    maps.resize(maps.size() + 128);
                    cudaError_t e = g2g::encode_box_map(
                        maps.data() + (size_t)idx * 128, (const void *)(uintptr_t)b->data, word,
                        (uint64_t)(rows * wpe), (uint64_t)cols, (uint64_t)ldb,
                        (uint32_t)(br * wpe), (uint32_t)bc);
                    if (e != cudaSuccess)
                        return fail(G2G_ERROR_CUDA, "tensor map of a block: %s",
                                    cudaGetErrorString(e));
                    Origin o;
                    o.map = idx;
                    org[(size_t)b->row * L.nbc() + b->col] = o;
                }
            }
        }
        const std::vector<HPart> rp = merge_parts(p.a.rs, p.b.rs);
        const std::vector<HPart> cp = merge_parts(p.a.cs, p.b.cs);
        for (const HPart &c : cp)
            for (const HPart &r : rp) {
                const Origin &so = aorg[(size_t)r.ia * p.a.nbc() + c.ia];
                const Origin &dn = borg[(size_t)r.ib * p.b.nbc() + c.ib];
                if (so.map < 0 || dn.map < 0)
                    continue;
                const int64_t sr = so.x + r.start - p.a.rs[r.ia], sc = so.y + c.start - p.a.cs[c.ia];
                const int64_t dr = dn.x + r.start - p.b.rs[r.ib], dc = dn.y + c.start - p.b.cs[c.ib];
                for (int32_t j = 0; j < c.len; j += bc)
                    for (int32_t i = 0; i < r.len; i += br)
                        boxes.push_back({so.map, dn.map, (int32_t)((sr + i) * wpe),
                                         (int32_t)(sc + j), (int32_t)((dr + i) * wpe),
                                         (int32_t)(dc + j)});
            }
    }
    const size_t maps_bytes = (maps.size() + 255) / 256 * 256;
    const size_t total = maps_bytes + boxes.size() * sizeof(g2g::TmaBox);
    G2G_CUDA(cudaMalloc(&pl.tma_mem, std::max<size_t>(total, 256)));
    cudaError_t e = cudaMemcpy(pl.tma_mem, maps.data(), maps.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !boxes.empty())
        e = cudaMemcpy((char *)pl.tma_mem + maps_bytes, boxes.data(),
                       boxes.size() * sizeof(g2g::TmaBox), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(pl.tma_mem);
        pl.tma_mem = nullptr;
        G2G_CUDA(e);
    }
    pl.tma.maps = (const unsigned char *)pl.tma_mem;
    pl.tma.boxes = (const g2g::TmaBox *)((char *)pl.tma_mem + maps_bytes);
    pl.tma.n_boxes = (long long)boxes.size();
    pl.tma.box_bytes = br * bc * esz;
    return G2G_SUCCESS;
}

bool use_tma(const g2g_plan &pl) { return pl.tma_ok && pl.tuning.tensor_boxes == 1; }

g2g_status create_plan(int n_pairs, const g2g_layout_desc *inits, const g2g_layout_desc *finals,
                       const g2g_dtype *dtypes, g2g_dtype single_dtype, const g2g_op *ops,
                       g2g_plan **out, int src_dtype = -1,
                       const g2g::PartialSpec *part = nullptr) {
    if (!out)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "plan output pointer is NULL");
    *out = nullptr;
    if (n_pairs < 1)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "n_pairs must be >= 1");
    if (!inits || !finals)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "layout arrays are NULL");
    g2g_plan *pl = new g2g_plan();
    pl->n_pairs = n_pairs;
    pl->tuning = default_tuning();
    pl->host.resize(n_pairs);
    for (int k = 0; k < n_pairs; ++k) {
        int dt = dtypes ? (int)dtypes[k] : (int)single_dtype;
        g2g_status st = build_pair(&inits[k], &finals[k], dt, ops ? &ops[k] : nullptr, k,
                                   pl->host[k], src_dtype, part);
        if (st != G2G_SUCCESS) {
            if (n_pairs > 1)
                t_last_error = "pair " + std::to_string(k) + ": " + t_last_error;
            delete pl;
            return st;
        }
        pl->n_ranks = std::max(pl->n_ranks, std::max(inits[k].n_ranks, finals[k].n_ranks));
    }
    assemble(*pl);
    g2g_status st = bind_device(*pl);
    if (st == G2G_SUCCESS)
        st = plan_on_device(*pl);
    if (st != G2G_SUCCESS) {
        g2g_plan_destroy(pl);
        return st;
    }
    // Launch shape by the tiles the plan holds. Plain copies run best as 16
    // warps per SM, each with its cp.async ring (a 2 KB stage in flight while
    // the previous one is stored): more concurrent column streams lose DRAM
    // locality. With CTA-level tiles as well, 256-thread CTAs keep more of
    // those in flight.
    if (pl->host_memory) {
        // the register path at full occupancy: more in flight over the host link
        pl->tuning.threads = 256;
        pl->tuning.ctas_per_sm = 8;
    } else if (pl->n_copy > 0) {
        const bool cta_tiles = pl->n_tiles > pl->n_copy;
        pl->tuning.threads = cta_tiles ? 256 : 512;
        pl->tuning.ctas_per_sm = cta_tiles ? 3 : 2;
    }
    tma_eligibility(*pl);
    G2G_CUDA(cudaEventCreateWithFlags(&pl->done, cudaEventDisableTiming));

    *out = pl;
    return G2G_SUCCESS;
}

} // namespace

namespace {

// Plans of the one-shot calls, keyed by a 128-bit signature of the
// descriptors, dtypes and ops: repeated transforms between the same buffers
// (the usual pattern of iterative callers) skip validation, upload and the
// planner. Plans hold only metadata; the caller's buffers are never retained.
// G2G_PLAN_CACHE_ENTRIES sets the capacity (0 turns the cache off).
struct OneShotCache {
    struct Entry {
        g2g_plan *plan = nullptr;
        int refs = 0;
        std::list<g2g::Sig>::iterator lru;
    };
    std::mutex mu;
    std::unordered_map<g2g::Sig, Entry, g2g::SigHash> map;
    std::list<g2g::Sig> lru; // most recent first
    int capacity = -1;
    int cap() {
        if (capacity < 0) {
            const char *e = std::getenv("G2G_PLAN_CACHE_ENTRIES");
            capacity = e ? std::max(0, std::atoi(e)) : 64;
        }
        return capacity;
    }
};
OneShotCache g_cache;

g2g::Sig one_shot_sig(int n, const g2g_layout_desc *init, const g2g_layout_desc *fin,
                      const g2g_dtype *dtypes, g2g_dtype dtype, const g2g_op *ops) {
    g2g::Sig sig;
    sig.add(n);
    for (int k = 0; k < n; ++k) {
        g2g::add_layout(sig, &init[k]);
        g2g::add_layout(sig, &fin[k]);
        const g2g_dtype dt = dtypes ? dtypes[k] : dtype;
        sig.add(dt);
        g2g_op o;
        std::memset(&o, 0, sizeof(o));
        o.trans = 'N';
        o.alpha[0] = 1.0;
        if (ops) {
            o.trans = ops[k].trans;
            std::memcpy(o.alpha, ops[k].alpha, sizeof(o.alpha));
            std::memcpy(o.beta, ops[k].beta, sizeof(o.beta));
        }
        sig.add(o.trans);
        sig.add(o.alpha);
        sig.add(o.beta);
    }
    return sig;
}

} // namespace

namespace g2g {

// plan (cached under `key`, planned by `make` on a miss; no caching when key
// is null or the cache is off) + execute + wait
g2g_status cached_one_shot(const Sig *key, const std::function<g2g_status(g2g_plan **)> &make,
                           void *stream) {
    const bool cached = key && g_cache.cap() > 0;
    g2g_plan *plan = nullptr;
    Sig sig;
    if (cached) {
        sig = *key;
        std::lock_guard<std::mutex> lk(g_cache.mu);
        auto it = g_cache.map.find(sig);
        if (it != g_cache.map.end()) {
            it->second.refs++;
            g_cache.lru.erase(it->second.lru);
            g_cache.lru.push_front(sig);
            it->second.lru = g_cache.lru.begin();
            plan = it->second.plan;
        }
    }
    if (!plan) {
        g2g_status st = make(&plan);
        if (st != G2G_SUCCESS)
            return st;
        if (cached) {
            std::vector<g2g_plan *> victims;
            {
                std::lock_guard<std::mutex> lk(g_cache.mu);
                auto it = g_cache.map.find(sig);
                if (it != g_cache.map.end()) { // planned concurrently by another thread
                    victims.push_back(plan);
                    plan = it->second.plan;
                    it->second.refs++;
                } else {
                    g_cache.lru.push_front(sig);
                    OneShotCache::Entry e;
                    e.plan = plan;
                    e.refs = 1;
                    e.lru = g_cache.lru.begin();
                    g_cache.map.emplace(sig, e);
                    auto li = g_cache.lru.end();
                    while ((int)g_cache.map.size() > g_cache.cap() && li != g_cache.lru.begin()) {
                        --li;
                        auto ci = g_cache.map.find(*li);
                        if (ci != g_cache.map.end() && ci->second.refs == 0) {
                            victims.push_back(ci->second.plan);
                            g_cache.map.erase(ci);
                            li = g_cache.lru.erase(li);
                        }
                    }
                }
            }
            for (g2g_plan *v : victims)
                g2g_plan_destroy(v);
        }
    }
    g2g_status st = g2g_plan_execute(plan, stream);
    if (st == G2G_SUCCESS) {
        cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
        if (e != cudaSuccess)
            st = fail(G2G_ERROR_CUDA, "transform failed: %s", cudaGetErrorString(e));
    }
    if (st == G2G_SUCCESS && plan->n_tiles > 0 &&
        (scatter_config(*plan).stages >= 2 || use_tma(*plan))) {
        // the staged and tensor-box kernels record an expired bounded wait
        // in the status
        int dst = 0;
        cudaError_t e = cudaMemcpy(&dst, plan->dev.status, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess)
            st = fail(G2G_ERROR_CUDA, "transform status: %s", cudaGetErrorString(e));
        else if (dst != 0)
            st = fail(G2G_ERROR_TIMEOUT, "transform: a bounded wait of the staged kernel expired");
    }
    if (cached) {
        std::lock_guard<std::mutex> lk(g_cache.mu);
        auto it = g_cache.map.find(sig);
        if (it != g_cache.map.end() && it->second.plan == plan)
            it->second.refs--;
        return st;
    }
    g2g_status st2 = g2g_plan_destroy(plan);
    return st != G2G_SUCCESS ? st : st2;
}

} // namespace g2g

namespace {

// the reference's blocking transform call: plan cached under the layouts'
// signature
g2g_status one_shot(int n, const g2g_layout_desc *init, const g2g_layout_desc *fin,
                    const g2g_dtype *dtypes, g2g_dtype dtype, const g2g_op *ops,
                    void *stream) {
    g2g::Sig sig;
    const bool keyed = n >= 1 && init && fin && g_cache.cap() > 0;
    if (keyed)
        sig = one_shot_sig(n, init, fin, dtypes, dtype, ops);
    return g2g::cached_one_shot(
        keyed ? &sig : nullptr,
        [&](g2g_plan **p) { return create_plan(n, init, fin, dtypes, dtype, ops, p); }, stream);
}

} // namespace

extern "C" {

const char *g2g_last_error_string(void) { return t_last_error.c_str(); }

const char *g2g_version_string(void) { return "grid2grid_gb300 0.1 (sm_103a)"; }

g2g_status g2g_plan_create(const g2g_layout_desc *initial, const g2g_layout_desc *final_,
                           g2g_dtype dtype, const g2g_op *op, void *stream,
                           g2g_plan **plan) {
    (void)stream;
    return create_plan(1, initial, final_, nullptr, dtype, op, plan);
}

g2g_status g2g_plan_create_cast(const g2g_layout_desc *initial, g2g_dtype src_dtype,
                                const g2g_layout_desc *final_, g2g_dtype dst_dtype,
                                const g2g_op *op, void *stream, g2g_plan **plan) {
    (void)stream;
    return create_plan(1, initial, final_, nullptr, dst_dtype, op, plan, (int)src_dtype);
}

g2g_status g2g_transform_cast(const g2g_layout_desc *initial, g2g_dtype src_dtype,
                              const g2g_layout_desc *final_, g2g_dtype dst_dtype,
                              const g2g_op *op, void *stream) {
    g2g_plan *plan = nullptr;
    G2G_TRY(g2g_plan_create_cast(initial, src_dtype, final_, dst_dtype, op, stream, &plan));
    g2g_status st = g2g_plan_execute(plan, stream);
    if (st == G2G_SUCCESS) {
        cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
        if (e != cudaSuccess)
            st = fail(G2G_ERROR_CUDA, "cast transform failed: %s", cudaGetErrorString(e));
    }
    g2g_status st2 = g2g_plan_destroy(plan);
    return st != G2G_SUCCESS ? st : st2;
}

g2g_status g2g_plan_create_batch(int32_t n_pairs, const g2g_layout_desc *initials,
                                 const g2g_layout_desc *finals, const g2g_dtype *dtypes,
                                 const g2g_op *ops, void *stream, g2g_plan **plan) {
    (void)stream;
    if (!dtypes)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "dtypes is NULL");
    return create_plan(n_pairs, initials, finals, dtypes, G2G_FLOAT32, ops, plan);
}

g2g_status g2g_plan_execute(g2g_plan *plan, void *stream) {
    if (!plan)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "plan is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    G2G_CUDA(cudaSetDevice(plan->device));
    if (plan->n_tiles > 0) {
        if (plan->graph && plan->graph_stream == s) {
            G2G_CUDA(cudaGraphLaunch(plan->graph, s));
        } else if (use_tma(*plan)) {
            G2G_TRY(build_tma(*plan));
            G2G_CUDA(cudaMemsetAsync(plan->dev.status, 0, sizeof(int), s));
            G2G_CUDA(g2g::launch_tma_boxes(plan->tma, plan->sm_count, plan->dev.status, s));
        } else {
            G2G_CUDA(launch_list(single_list(*plan), scatter_config(*plan), s));
        }
    }
    G2G_CUDA(cudaEventRecord(plan->done, s));
    plan->last_stream = s;
    return G2G_SUCCESS;
}

g2g_status g2g_plans_execute(int32_t n_plans, g2g_plan *const *plans, void *stream) {
    if (n_plans < 1 || !plans)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "no plans to execute");
    for (int k = 0; k < n_plans; ++k) {
        if (!plans[k])
            return fail(G2G_ERROR_INVALID_ARGUMENT, "plan %d is NULL", k);
        if (plans[k]->device != plans[0]->device)
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "plans of one launch must live on one device (plan %d)", k);
    }
    cudaStream_t s = (cudaStream_t)stream;
    G2G_CUDA(cudaSetDevice(plans[0]->device));
    // no kernel instance carries both the cast conversions and the alpha/beta
    // arithmetic: cast plans launch apart from the others, in order
    std::vector<g2g_plan *> groups[2];
    for (int k = 0; k < n_plans; ++k)
        groups[(plans[k]->paths & 16) ? 1 : 0].push_back(plans[k]);
    for (const std::vector<g2g_plan *> &grp : groups) {
        const int m = (int)grp.size();
        for (int base = 0; base < m; base += g2g::kMaxPlansPerLaunch) {
            const int n = std::min(m - base, g2g::kMaxPlansPerLaunch);
            g2g::PlanList l;
            l.n = 0;
            l.status = grp[base]->dev.status;
            for (int k = 0; k < n; ++k) {
                const g2g_plan *p = grp[base + k];
                if (p->n_tiles > 0)
                    add_to_list(l, *p);
            }
            if (l.n > 0)
                G2G_CUDA(launch_list(l, merged_config(grp.data() + base, n), s));
        }
    }
    for (int k = 0; k < n_plans; ++k) {
        G2G_CUDA(cudaEventRecord(plans[k]->done, s));
        plans[k]->last_stream = s;
    }
    return G2G_SUCCESS;
}

g2g_status g2g_plan_capture_graph(g2g_plan *plan, void *stream) {
    if (!plan)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "plan is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    if (!s)
        return fail(G2G_ERROR_INVALID_ARGUMENT,
                    "graph capture needs a non-default stream");
    G2G_CUDA(cudaSetDevice(plan->device));
    if (plan->graph) {
        cudaGraphExecDestroy(plan->graph);
        plan->graph = nullptr;
    }
    if (plan->n_tiles == 0)
        return G2G_SUCCESS;
    cudaGraph_t g = nullptr;
    if (use_tma(*plan))
        G2G_TRY(build_tma(*plan)); // uploads happen before the capture
    G2G_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaSuccess;
    if (use_tma(*plan)) {
        le = cudaMemsetAsync(plan->dev.status, 0, sizeof(int), s);
        if (le == cudaSuccess)
            le = g2g::launch_tma_boxes(plan->tma, plan->sm_count, plan->dev.status, s);
    } else {
        le = launch_list(single_list(*plan), scatter_config(*plan), s);
    }
    cudaError_t ee = cudaStreamEndCapture(s, &g);
    G2G_CUDA(le);
    G2G_CUDA(ee);
    cudaError_t ie = cudaGraphInstantiate(&plan->graph, g, 0);
    cudaGraphDestroy(g);
    G2G_CUDA(ie);
    plan->graph_stream = s;
    return G2G_SUCCESS;
}

g2g_status g2g_plan_set_tuning(g2g_plan *plan, const g2g_tuning *tuning) {
    if (!plan || !tuning)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "plan or tuning is NULL");
    g2g_tuning t = merge_tuning(plan->tuning, tuning);
    G2G_TRY(check_tuning(t));
    const bool replan = t.tile_bytes != plan->tuning.tile_bytes ||
                        t.tile_dim != plan->tuning.tile_dim;
    plan->tuning = t;
    if (plan->graph) {
        cudaGraphExecDestroy(plan->graph);
        plan->graph = nullptr;
    }
    if (replan) {
        // the work list may be in use by queued executions
        if (plan->last_stream || plan->done)
            G2G_CUDA(cudaEventSynchronize(plan->done));
        assemble(*plan);
        G2G_TRY(plan_on_device(*plan));
    }
    return G2G_SUCCESS;
}

g2g_status g2g_plan_autotune(g2g_plan *plan, void *stream, int32_t iters, g2g_tuning *best) {
    if (!plan)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "plan is NULL");
    if (iters < 1)
        iters = 3;
    cudaStream_t s = (cudaStream_t)stream;
    const g2g_tuning start = plan->tuning;
    std::vector<g2g_tuning> cands;
    const int tile_bytes_opts[] = {4 * 1024, 8 * 1024, 16 * 1024, 32 * 1024, 64 * 1024};
    const int tile_dim_opts[] = {16, 32};
    const int threads_opts[] = {256, 512};
    const int unroll_opts[] = {2, 4};
    const int ctas_opts[] = {2, 4, 8};
    const int stage_opts[] = {-1, 2, 3, 4};
    const int ring_opts[] = {1, -1};
    const int run_opts[] = {1, 2};
    const int prefetch_opts[] = {-1, 1};
    for (int tb : tile_bytes_opts)
        for (int td : tile_dim_opts) {
            if (!plan->any_trans && td != start.tile_dim)
                continue;
            for (int th : threads_opts)
                for (int u : unroll_opts)
                    for (int c : ctas_opts)
                        for (int sg : stage_opts)
                            for (int rg : ring_opts)
                                for (int run : run_opts)
                                    for (int pf : prefetch_opts) {
                                        if (th * c > 2048)
                                            continue;
                                        // without copy tiles the stages are moot and
                                        // the ring knob only picks the staged ring of
                                        // narrow transposes or their register path
                                        if (!(plan->paths & 1) &&
                                            (sg != -1 ||
                                             (rg != 1 &&
                                              !(plan->paths & (64 | 128 | 256 | 1024 | 2048)))))
                                            continue;
                                        if (sg != -1 && rg != 1)
                                            continue;
                                        // runs and prefetch only matter to the ring
                                        if ((run != 1 || pf != -1) && (sg != -1 || rg != 1))
                                            continue;
                                        if (run != 1 && pf != -1)
                                            continue;
                                        g2g_tuning t = start;
                                        t.tile_bytes = tb;
                                        t.tile_dim = td;
                                        t.threads = th;
                                        t.unroll = u;
                                        t.ctas_per_sm = c;
                                        t.stages = sg;
                                        t.ring = rg;
                                        t.tile_run = run;
                                        t.l2_prefetch = pf;
                                        t.tensor_boxes = -1;
                                        cands.push_back(t);
                                    }
        }
    if (plan->tma_ok) { // the tensor-box kernel takes none of the other knobs
        g2g_tuning t = start;
        t.tensor_boxes = 1;
        cands.push_back(t);
    }
    cudaEvent_t e0, e1;
    G2G_CUDA(cudaEventCreate(&e0));
    G2G_CUDA(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    g2g_tuning best_t = start;
    for (const g2g_tuning &t : cands) {
        g2g_status st = g2g_plan_set_tuning(plan, &t);
        if (st != G2G_SUCCESS)
            continue;
        if (g2g_plan_execute(plan, s) != G2G_SUCCESS) // warm-up
            continue;
        cudaEventRecord(e0, s);
        for (int i = 0; i < iters; ++i)
            g2g_plan_execute(plan, s);
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess)
            break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_ms) {
            best_ms = ms;
            best_t = plan->tuning;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    G2G_TRY(g2g_plan_set_tuning(plan, &best_t));
    if (best)
        *best = plan->tuning;
    return G2G_SUCCESS;
}

g2g_status g2g_plan_get_info(const g2g_plan *plan, g2g_plan_info *info) {
    if (!plan || !info)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "plan or info is NULL");
    std::memset(info, 0, sizeof(*info));
    info->n_pairs = plan->n_pairs;
    info->n_ranks = plan->n_ranks;
    info->n_pieces = plan->n_pieces;
    info->n_tiles = plan->n_tiles;
    info->bytes_moved = plan->bytes_moved;
    info->bytes_min_traffic = plan->bytes_min_traffic;
    info->metadata_bytes = (int64_t)plan->dmem_bytes;
    info->graph_captured = plan->graph ? 1 : 0;
    info->tensor_boxes_ok = plan->tma_ok ? 1 : 0;
    info->tile_paths = plan->paths;
    info->tuning = plan->tuning;
    if (plan->dev.status) {
        G2G_CUDA(cudaSetDevice(plan->device));
        G2G_CUDA(cudaEventSynchronize(plan->done));
        int st = 0;
        G2G_CUDA(cudaMemcpy(&st, plan->dev.status, sizeof(int), cudaMemcpyDeviceToHost));
        info->device_status = st;
    }
    return G2G_SUCCESS;
}

g2g_status g2g_plan_destroy(g2g_plan *plan) {
    if (!plan)
        return G2G_SUCCESS;
    g2g_status st = G2G_SUCCESS;
    if (plan->graph)
        cudaGraphExecDestroy(plan->graph);
    if (plan->dmem) {
        DeviceState *ds = nullptr;
        cudaSetDevice(plan->device);
        if (device_state(&ds, nullptr) == G2G_SUCCESS) {
            // free after the last execution that used the plan
            if (plan->done && plan->last_stream != nullptr)
                cudaStreamWaitEvent(ds->plan_stream, plan->done, 0);
            else if (plan->done)
                cudaEventSynchronize(plan->done);
            cudaError_t e = cudaFreeAsync(plan->dmem, ds->plan_stream);
            if (e != cudaSuccess)
                st = fail(G2G_ERROR_CUDA, "cudaFreeAsync failed: %s", cudaGetErrorString(e));
        }
    }
    if (plan->tma_mem) {
        cudaSetDevice(plan->device);
        if (plan->done)
            cudaEventSynchronize(plan->done);
        cudaFree(plan->tma_mem);
    }
    if (plan->done)
        cudaEventDestroy(plan->done);
    delete plan;
    return st;
}

g2g_status g2g_transform(const g2g_layout_desc *initial, const g2g_layout_desc *final_,
                         g2g_dtype dtype, const g2g_op *op, void *stream) {
    return one_shot(1, initial, final_, nullptr, dtype, op, stream);
}

g2g_status g2g_transform_batch(int32_t n_pairs, const g2g_layout_desc *initials,
                               const g2g_layout_desc *finals, const g2g_dtype *dtypes,
                               const g2g_op *ops, void *stream) {
    if (!dtypes)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "dtypes is NULL");
    return one_shot(n_pairs, initials, finals, dtypes, G2G_FLOAT32, ops, stream);
}

g2g_status g2g_plan_cache_clear(void) {
    std::vector<g2g_plan *> victims;
    {
        std::lock_guard<std::mutex> lk(g_cache.mu);
        for (auto it = g_cache.map.begin(); it != g_cache.map.end();) {
            if (it->second.refs == 0) {
                victims.push_back(it->second.plan);
                g_cache.lru.erase(it->second.lru);
                it = g_cache.map.erase(it);
            } else {
                ++it;
            }
        }
    }
    g2g_status st = G2G_SUCCESS;
    for (g2g_plan *p : victims) {
        g2g_status s2 = g2g_plan_destroy(p);
        if (s2 != G2G_SUCCESS)
            st = s2;
    }
    return st;
}

g2g_status g2g_grid_cover(const int32_t *splits_a, int32_t n_a, const int32_t *splits_b,
                          int32_t n_b, int32_t *start_index, int32_t *end_index,
                          void *stream) {
    if (!splits_a || !splits_b || n_a < 1 || n_b < 1 || (n_a > 1 && (!start_index || !end_index)))
        return fail(G2G_ERROR_INVALID_ARGUMENT, "grid cover: bad arguments");
    G2G_TRY(check_splits(splits_a, n_a - 1, "first", "cover"));
    G2G_TRY(check_splits(splits_b, n_b - 1, "second", "cover"));
    if (splits_a[0] != splits_b[0] || splits_a[n_a - 1] != splits_b[n_b - 1])
        return fail(G2G_ERROR_INVALID_ARGUMENT,
                    "grid cover: split vectors must share their first and last entries");
    if (n_a == 1)
        return G2G_SUCCESS;
    cudaStream_t s = (cudaStream_t)stream;
    int32_t *d = nullptr;
    const size_t bytes = sizeof(int32_t) * ((size_t)n_a + n_b + 2 * (size_t)(n_a - 1));
    G2G_CUDA(cudaMallocAsync((void **)&d, bytes, s));
    int32_t *da = d, *db = d + n_a, *ds = db + n_b, *de = ds + (n_a - 1);
    cudaError_t e = cudaMemcpyAsync(da, splits_a, sizeof(int32_t) * n_a,
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(db, splits_b, sizeof(int32_t) * n_b, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = g2g::launch_cover(da, n_a, db, n_b, ds, de, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(start_index, ds, sizeof(int32_t) * (n_a - 1),
                            cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(end_index, de, sizeof(int32_t) * (n_a - 1),
                            cudaMemcpyDeviceToHost, s);
    cudaError_t fe = cudaFreeAsync(d, s);
    if (e == cudaSuccess)
        e = fe;
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    G2G_CUDA(e);
    return G2G_SUCCESS;
}

} // extern "C"

namespace g2g {

g2g_status build_host_image(const g2g_layout_desc *initial, const g2g_layout_desc *final_,
                            g2g_dtype dtype, const g2g_op *op, HostPlanImage *out) {
    if (!out)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "plan image output is NULL");
    g2g_plan pl;
    pl.n_pairs = 1;
    pl.tuning = default_tuning();
    pl.host.resize(1);
    G2G_TRY(build_pair(initial, final_, (int)dtype, op, 0, pl.host[0]));
    assemble(pl);
    G2G_TRY(bind_device(pl));
    G2G_CUDA(cudaGetDevice(&pl.device));
    G2G_CUDA(cudaDeviceGetAttribute(&pl.sm_count, cudaDevAttrMultiProcessorCount, pl.device));
    int64_t capacity = 0;
    for (const PairHost &p : pl.host)
        capacity += tile_capacity_bound(p, pl.tuning);
    out->device = pl.device;
    out->pairs = pl.pinfo;
    out->splits = pl.splits;
    out->src_tables = pl.src_tables;
    out->dst_tables = pl.dst_tables;
    out->n_parts = pl.n_parts;
    out->n_cells = pl.n_cells;
    out->max_cells_per_pair = pl.max_cells_per_pair;
    out->tile_capacity = std::max<int64_t>(capacity, 1);
    out->bytes_moved = pl.bytes_moved;
    pl.n_tiles = out->tile_capacity; // grid bound only; the launch uses exact counts
    out->cfg = scatter_config(pl);
    return G2G_SUCCESS;
}

g2g_status create_plan_partial(const g2g_layout_desc *initial, const g2g_layout_desc *final_,
                               g2g_dtype dtype, const g2g_op *op, const PartialSpec &part,
                               g2g_plan **plan) {
    return create_plan(1, initial, final_, nullptr, dtype, op, plan, -1, &part);
}

g2g_status validate_partial(const g2g_layout_desc *initial, const g2g_layout_desc *final_,
                            g2g_dtype dtype, const g2g_op *op, const PartialSpec &part) {
    PairHost p;
    return build_pair(initial, final_, (int)dtype, op, 0, p, -1, &part);
}

} // namespace g2g
