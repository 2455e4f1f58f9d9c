// Sharded transform: the virtual ranks of a transform spread over several
// GPUs (one process each), the reference's exchange step between them.
//
// The reference redistributes between MPI ranks by packing every piece bound
// for another rank into a send buffer, exchanging the buffers and unpacking
// them, local pieces copied directly (exchange_async, transform.cpp:41-124;
// communication_data, communication_data.cpp:51-99). Here a rank of the
// transform is a virtual rank and a GPU (a shard) holds the blocks of a set
// of virtual ranks. One shard's part of the transform is three plans of the
// ordinary gather-scatter, built from descriptors that list only the blocks
// its ranks hold:
//
//   local   pieces whose source and destination ranks are both on this
//           shard: source block -> destination block, op and alpha/beta
//           applied (copy_local_blocks, communication_data.cpp:224-252);
//   pack    pieces bound for another shard: source block -> this shard's
//           send buffer, op applied (copy_to_buffer,
//           communication_data.cpp:132-142), one launch with `local`;
//   unpack  pieces received from another shard: receive buffer ->
//           destination block, alpha/beta applied (copy_from_buffer,
//           communication_data.cpp:157-173).
//
// Between pack and unpack the caller exchanges the buffers (an all-to-all
// with per-shard byte counts, e.g. NCCL through torch.distributed). The
// packed buffers are described as layouts on the grid cover (the union of
// both grids' split points, so each cover cell is exactly one piece), whose
// blocks sit at the pieces' buffer offsets with the piece rows as stride.
//
// Buffer order. A piece is packed column-major with leading dimension = its
// rows, in final orientation. The section of shard g's send buffer for shard
// h holds, for each source rank s of g and then each destination rank d of
// h (ascending), the pieces s sends to d ordered by (column interval, row
// interval) -- the order of the reference's message sort
// (communication_data.cpp:26-30, block.cpp:207-225) -- so the (s, d) segment
// equals rank s's send-buffer segment for d in the reference, and its length
// is the reference's counts[d] on rank s. Sections follow in shard order.
#include "../../include/grid2grid_gb300.h"
#include "g2g_host.hpp"

#include <algorithm>
#include <cctype>
#include <cstring>
#include <memory>
#include <vector>

namespace {

using g2g::fail;

int esz_of(int dt) {
    switch (dt) {
    case G2G_FLOAT32: return 4;
    case G2G_FLOAT64: return 8;
    case G2G_COMPLEX64: return 8;
    case G2G_COMPLEX128: return 16;
    default: return 0;
    }
}

// An owned copy of a layout descriptor (the caller's arrays may go away
// between creation and binding).
struct DescCopy {
    std::vector<int32_t> rs, cs, owners, reo;
    std::vector<g2g_block_desc> blocks;
    g2g_layout_desc d;
    void take(const g2g_layout_desc &src) {
        rs.assign(src.rows_split, src.rows_split + src.n_block_rows + 1);
        cs.assign(src.cols_split, src.cols_split + src.n_block_cols + 1);
        owners.assign(src.owners,
                      src.owners + (size_t)src.n_block_rows * (size_t)src.n_block_cols);
        if (src.n_reordering > 0)
            reo.assign(src.reordering, src.reordering + src.n_reordering);
        if (src.n_blocks > 0)
            blocks.assign(src.blocks, src.blocks + src.n_blocks);
        d = src;
        fix();
    }
    void fix() {
        d.rows_split = rs.data();
        d.cols_split = cs.data();
        d.owners = owners.data();
        d.reordering = reo.empty() ? nullptr : reo.data();
        d.n_reordering = (int32_t)reo.size();
        d.blocks = blocks.empty() ? nullptr : blocks.data();
        d.n_blocks = (int32_t)blocks.size();
    }
};

// The grid and owners of a layout as the transform sees it: the initial one
// after op ('T' / 'C' transpose the grid and the owner matrix,
// grid_layout.hpp:18-25), owners through the layout's reordering
// (grid2D.cpp:116-122).
struct GridView {
    const int32_t *rs, *cs;
    int nbr, nbc;
    const g2g_layout_desc *d;
    bool transposed;
    int owner(int i, int j) const {
        const int r = transposed ? d->owners[(size_t)j * d->n_block_cols + i]
                                 : d->owners[(size_t)i * d->n_block_cols + j];
        return d->n_reordering > 0 ? d->reordering[r] : r;
    }
};

GridView view_of(const g2g_layout_desc &d, bool transposed) {
    GridView v;
    v.d = &d;
    v.transposed = transposed;
    v.rs = transposed ? d.cols_split : d.rows_split;
    v.cs = transposed ? d.rows_split : d.cols_split;
    v.nbr = transposed ? d.n_block_cols : d.n_block_rows;
    v.nbc = transposed ? d.n_block_rows : d.n_block_cols;
    return v;
}

// Index of the interval of split vector s[0..n] that holds the non-empty
// cover interval starting at x (the last k with s[k] <= x).
int interval_of(const int32_t *s, int n, int32_t x) {
    return (int)(std::upper_bound(s, s + n + 1, x) - s) - 1;
}

struct Cell {
    int32_t u, v;   // cover row / column interval
    int32_t s, d;   // source and destination ranks
    int32_t peer;   // the other shard
};

} // namespace

struct g2g_exchange {
    int n_shards = 0, shard = 0, P = 0;
    g2g_dtype dtype = G2G_FLOAT32;
    int esz = 0;
    g2g_op op;
    DescCopy init, fin;
    std::vector<char> held; // ranks of this shard
    std::vector<int32_t> cover_rs, cover_cs;
    std::vector<int64_t> rank_counts;           // P x P elements
    std::vector<int64_t> send_bytes, recv_bytes; // per shard
    std::vector<g2g_exchange_piece> local, send, recv;
    int64_t local_elems = 0, send_elems = 0, recv_elems = 0;
    g2g_plan *local_plan = nullptr, *pack_plan = nullptr, *unpack_plan = nullptr;
    DescCopy send_cover, recv_cover;

    void free_plans() {
        g2g_plan_destroy(local_plan);
        g2g_plan_destroy(pack_plan);
        g2g_plan_destroy(unpack_plan);
        local_plan = pack_plan = unpack_plan = nullptr;
    }
};

namespace {

// A layout on the cover grid holding `pieces` at `base` + offset: the packed
// send or receive buffer of the shard.
void cover_layout(const g2g_exchange &ex, const std::vector<g2g_exchange_piece> &pieces,
                  const std::vector<int32_t> &owner_of_cell, uint64_t base, DescCopy &out) {
    out.rs = ex.cover_rs;
    out.cs = ex.cover_cs;
    out.owners = owner_of_cell;
    out.reo.clear();
    const int nc = (int)ex.cover_cs.size() - 1;
    out.blocks.resize(pieces.size());
    for (size_t k = 0; k < pieces.size(); ++k) {
        const g2g_exchange_piece &p = pieces[k];
        g2g_block_desc &b = out.blocks[k];
        std::memset(&b, 0, sizeof(b));
        b.row = (int32_t)(std::lower_bound(ex.cover_rs.begin(), ex.cover_rs.end(), p.row_start) -
                          ex.cover_rs.begin());
        b.col = (int32_t)(std::lower_bound(ex.cover_cs.begin(), ex.cover_cs.end(), p.col_start) -
                          ex.cover_cs.begin());
        b.rank = owner_of_cell[(size_t)b.row * nc + b.col];
        b.stride = std::max<int64_t>(1, p.row_end - p.row_start);
        b.data = (void *)(uintptr_t)(base + (uint64_t)p.offset * (uint64_t)ex.esz);
    }
    std::memset(&out.d, 0, sizeof(out.d));
    out.d.n_block_rows = (int32_t)ex.cover_rs.size() - 1;
    out.d.n_block_cols = nc;
    out.d.n_ranks = ex.P;
    out.fix();
}

} // namespace

extern "C" {

g2g_status g2g_exchange_create(const g2g_layout_desc *initial, const g2g_layout_desc *final_,
                               g2g_dtype dtype, const g2g_op *op, int32_t n_shards,
                               const int32_t *shard_of_rank, int32_t shard,
                               g2g_exchange **out) {
    if (!out)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "exchange output pointer is NULL");
    *out = nullptr;
    if (!initial || !final_)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "layout descriptor is NULL");
    if (n_shards < 1 || shard < 0 || shard >= n_shards || !shard_of_rank)
        return fail(G2G_ERROR_INVALID_ARGUMENT,
                    "exchange: shard %d of %d shards, shard_of_rank %s", shard, n_shards,
                    shard_of_rank ? "given" : "NULL");
    const int esz = esz_of((int)dtype);
    if (!esz)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "unknown dtype %d", (int)dtype);
    const int P = std::max(1, std::max(initial->n_ranks, final_->n_ranks));
    std::unique_ptr<g2g_exchange> ex(new g2g_exchange());
    ex->n_shards = n_shards;
    ex->shard = shard;
    ex->P = P;
    ex->dtype = dtype;
    ex->esz = esz;
    std::memset(&ex->op, 0, sizeof(ex->op));
    ex->op.trans = 'N';
    ex->op.alpha[0] = 1.0;
    if (op)
        ex->op = *op;
    ex->held.assign(P, 0);
    for (int r = 0; r < P; ++r) {
        if (shard_of_rank[r] < 0 || shard_of_rank[r] >= n_shards)
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "exchange: rank %d is mapped to shard %d outside [0, %d)", r,
                        shard_of_rank[r], n_shards);
        ex->held[r] = shard_of_rank[r] == shard;
    }
    // full validation of both descriptors, as the plans will see them
    g2g::PartialSpec part;
    part.init_held = &ex->held;
    part.final_held = &ex->held;
    G2G_TRY(g2g::validate_partial(initial, final_, dtype, op, part));
    ex->init.take(*initial);
    ex->fin.take(*final_);
    const char trans = (char)std::toupper((unsigned char)ex->op.trans);
    const GridView A = view_of(ex->init.d, trans == 'T' || trans == 'C');
    const GridView B = view_of(ex->fin.d, false);

    // the grid cover: the union of both grids' split points
    for (int pass = 0; pass < 2; ++pass) {
        const int32_t *a = pass ? A.cs : A.rs, *b = pass ? B.cs : B.rs;
        const int na = pass ? A.nbc : A.nbr, nb = pass ? B.nbc : B.nbr;
        std::vector<int32_t> &c = pass ? ex->cover_cs : ex->cover_rs;
        c.assign(a, a + na + 1);
        c.insert(c.end(), b, b + nb + 1);
        std::sort(c.begin(), c.end());
        c.erase(std::unique(c.begin(), c.end()), c.end());
    }
    const int nr = (int)ex->cover_rs.size() - 1, nc = (int)ex->cover_cs.size() - 1;
    std::vector<int32_t> ia_r(nr), ib_r(nr), ia_c(nc), ib_c(nc);
    for (int u = 0; u < nr; ++u) {
        ia_r[u] = interval_of(A.rs, A.nbr, ex->cover_rs[u]);
        ib_r[u] = interval_of(B.rs, B.nbr, ex->cover_rs[u]);
    }
    for (int v = 0; v < nc; ++v) {
        ia_c[v] = interval_of(A.cs, A.nbc, ex->cover_cs[v]);
        ib_c[v] = interval_of(B.cs, B.nbc, ex->cover_cs[v]);
    }

    // every cell is one piece: rank counts for all pairs, this shard's cells
    ex->rank_counts.assign((size_t)P * P, 0);
    ex->send_bytes.assign(n_shards, 0);
    ex->recv_bytes.assign(n_shards, 0);
    std::vector<Cell> sends, recvs;
    for (int v = 0; v < nc; ++v) {
        const int64_t w = ex->cover_cs[v + 1] - ex->cover_cs[v];
        for (int u = 0; u < nr; ++u) {
            const int64_t h = ex->cover_rs[u + 1] - ex->cover_rs[u];
            const int s = A.owner(ia_r[u], ia_c[v]);
            const int d = B.owner(ib_r[u], ib_c[v]);
            ex->rank_counts[(size_t)s * P + d] += h * w;
            const int gs = shard_of_rank[s], gd = shard_of_rank[d];
            if (gs == shard && gd == shard) {
                g2g_exchange_piece p;
                p.row_start = ex->cover_rs[u];
                p.row_end = ex->cover_rs[u + 1];
                p.col_start = ex->cover_cs[v];
                p.col_end = ex->cover_cs[v + 1];
                p.src_rank = s;
                p.dst_rank = d;
                p.offset = -1;
                ex->local.push_back(p);
                ex->local_elems += h * w;
            } else if (gs == shard) {
                sends.push_back({u, v, s, d, gd});
            } else if (gd == shard) {
                recvs.push_back({u, v, s, d, gs});
            }
        }
    }
    // buffer order: (peer shard, source rank, destination rank, column, row)
    auto order = [](const Cell &x, const Cell &y) {
        if (x.peer != y.peer) return x.peer < y.peer;
        if (x.s != y.s) return x.s < y.s;
        if (x.d != y.d) return x.d < y.d;
        if (x.v != y.v) return x.v < y.v;
        return x.u < y.u;
    };
    std::stable_sort(sends.begin(), sends.end(), order);
    std::stable_sort(recvs.begin(), recvs.end(), order);
    for (int pass = 0; pass < 2; ++pass) {
        const std::vector<Cell> &cells = pass ? recvs : sends;
        std::vector<g2g_exchange_piece> &pieces = pass ? ex->recv : ex->send;
        std::vector<int64_t> &bytes = pass ? ex->recv_bytes : ex->send_bytes;
        int64_t off = 0;
        pieces.reserve(cells.size());
        for (const Cell &c : cells) {
            g2g_exchange_piece p;
            p.row_start = ex->cover_rs[c.u];
            p.row_end = ex->cover_rs[c.u + 1];
            p.col_start = ex->cover_cs[c.v];
            p.col_end = ex->cover_cs[c.v + 1];
            p.src_rank = c.s;
            p.dst_rank = c.d;
            p.offset = off;
            const int64_t n = (int64_t)(p.row_end - p.row_start) * (p.col_end - p.col_start);
            off += n;
            bytes[c.peer] += n * esz;
            pieces.push_back(p);
        }
        (pass ? ex->recv_elems : ex->send_elems) = off;
    }
    *out = ex.release();
    return G2G_SUCCESS;
}

g2g_status g2g_exchange_get_counts(const g2g_exchange *ex, int64_t *send_bytes,
                                   int64_t *recv_bytes) {
    if (!ex)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "exchange is NULL");
    if (send_bytes)
        std::copy(ex->send_bytes.begin(), ex->send_bytes.end(), send_bytes);
    if (recv_bytes)
        std::copy(ex->recv_bytes.begin(), ex->recv_bytes.end(), recv_bytes);
    return G2G_SUCCESS;
}

g2g_status g2g_exchange_get_rank_counts(const g2g_exchange *ex, int32_t n_ranks,
                                        int64_t *counts) {
    if (!ex || !counts)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "exchange or counts is NULL");
    if (n_ranks != ex->P)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "exchange: n_ranks %d, the transform has %d",
                    n_ranks, ex->P);
    std::copy(ex->rank_counts.begin(), ex->rank_counts.end(), counts);
    return G2G_SUCCESS;
}

g2g_status g2g_exchange_get_pieces(const g2g_exchange *ex, int32_t which, int64_t capacity,
                                   g2g_exchange_piece *pieces, int64_t *n_pieces) {
    if (!ex || !n_pieces)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "exchange or n_pieces is NULL");
    const std::vector<g2g_exchange_piece> *v =
        which == G2G_EXCHANGE_LOCAL ? &ex->local
                                    : (which == G2G_EXCHANGE_SEND
                                           ? &ex->send
                                           : (which == G2G_EXCHANGE_RECV ? &ex->recv : nullptr));
    if (!v)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "exchange: piece list %d is not 0, 1 or 2",
                    which);
    *n_pieces = (int64_t)v->size();
    if (pieces) {
        if (capacity < (int64_t)v->size())
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "exchange: %lld pieces do not fit a capacity of %lld",
                        (long long)v->size(), (long long)capacity);
        std::copy(v->begin(), v->end(), pieces);
    }
    return G2G_SUCCESS;
}

g2g_status g2g_exchange_bind(g2g_exchange *ex, void *send_buffer, void *recv_buffer,
                             void *stream) {
    (void)stream;
    if (!ex)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "exchange is NULL");
    if ((ex->send_elems > 0 && !send_buffer) || (ex->recv_elems > 0 && !recv_buffer))
        return fail(G2G_ERROR_INVALID_ARGUMENT,
                    "exchange: a send or receive buffer is NULL but holds pieces");
    ex->free_plans();
    const int nc = (int)ex->cover_cs.size() - 1, nr = (int)ex->cover_rs.size() - 1;
    g2g_op pack_op;
    std::memset(&pack_op, 0, sizeof(pack_op));
    pack_op.trans = ex->op.trans;
    pack_op.alpha[0] = 1.0;
    g2g_op unpack_op = ex->op;
    unpack_op.trans = 'N';
    if (!ex->local.empty()) {
        g2g::PartialSpec part;
        part.init_held = &ex->held;
        part.final_held = &ex->held;
        part.elems = ex->local_elems;
        G2G_TRY(g2g::create_plan_partial(&ex->init.d, &ex->fin.d, ex->dtype, &ex->op, part,
                                         &ex->local_plan));
    }
    if (!ex->send.empty()) {
        std::vector<int32_t> owner((size_t)nr * nc, 0);
        for (const g2g_exchange_piece &p : ex->send) {
            const int u = (int)(std::lower_bound(ex->cover_rs.begin(), ex->cover_rs.end(),
                                                 p.row_start) - ex->cover_rs.begin());
            const int v = (int)(std::lower_bound(ex->cover_cs.begin(), ex->cover_cs.end(),
                                                 p.col_start) - ex->cover_cs.begin());
            owner[(size_t)u * nc + v] = p.dst_rank;
        }
        cover_layout(*ex, ex->send, owner, (uint64_t)(uintptr_t)send_buffer, ex->send_cover);
        g2g::PartialSpec part;
        part.init_held = &ex->held;
        part.final_absent_ok = true;
        part.elems = ex->send_elems;
        g2g_status st = g2g::create_plan_partial(&ex->init.d, &ex->send_cover.d, ex->dtype,
                                                 &pack_op, part, &ex->pack_plan);
        if (st != G2G_SUCCESS) {
            ex->free_plans();
            return st;
        }
    }
    if (!ex->recv.empty()) {
        std::vector<int32_t> owner((size_t)nr * nc, 0);
        for (const g2g_exchange_piece &p : ex->recv) {
            const int u = (int)(std::lower_bound(ex->cover_rs.begin(), ex->cover_rs.end(),
                                                 p.row_start) - ex->cover_rs.begin());
            const int v = (int)(std::lower_bound(ex->cover_cs.begin(), ex->cover_cs.end(),
                                                 p.col_start) - ex->cover_cs.begin());
            owner[(size_t)u * nc + v] = p.src_rank;
        }
        cover_layout(*ex, ex->recv, owner, (uint64_t)(uintptr_t)recv_buffer, ex->recv_cover);
        g2g::PartialSpec part;
        part.init_absent_ok = true;
        part.final_held = &ex->held;
        part.elems = ex->recv_elems;
        g2g_status st = g2g::create_plan_partial(&ex->recv_cover.d, &ex->fin.d, ex->dtype,
                                                 &unpack_op, part, &ex->unpack_plan);
        if (st != G2G_SUCCESS) {
            ex->free_plans();
            return st;
        }
    }
    return G2G_SUCCESS;
}

g2g_status g2g_exchange_pack(g2g_exchange *ex, void *stream) {
    if (!ex)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "exchange is NULL");
    if ((!ex->local.empty() && !ex->local_plan) || (!ex->send.empty() && !ex->pack_plan))
        return fail(G2G_ERROR_INVALID_ARGUMENT, "exchange: pack before g2g_exchange_bind");
    g2g_plan *plans[2];
    int n = 0;
    if (ex->local_plan)
        plans[n++] = ex->local_plan;
    if (ex->pack_plan)
        plans[n++] = ex->pack_plan;
    if (n == 0)
        return G2G_SUCCESS;
    return g2g_plans_execute(n, plans, stream);
}

g2g_status g2g_exchange_unpack(g2g_exchange *ex, void *stream) {
    if (!ex)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "exchange is NULL");
    if (!ex->recv.empty() && !ex->unpack_plan)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "exchange: unpack before g2g_exchange_bind");
    if (!ex->unpack_plan)
        return G2G_SUCCESS;
    return g2g_plan_execute(ex->unpack_plan, stream);
}

g2g_status g2g_exchange_get_plan_info(const g2g_exchange *ex, int32_t which,
                                      g2g_plan_info *info) {
    if (!ex || !info)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "exchange or info is NULL");
    const g2g_plan *p = which == G2G_EXCHANGE_LOCAL
                            ? ex->local_plan
                            : (which == G2G_EXCHANGE_SEND ? ex->pack_plan : ex->unpack_plan);
    if (!p) {
        std::memset(info, 0, sizeof(*info));
        return G2G_SUCCESS;
    }
    return g2g_plan_get_info(p, info);
}

g2g_status g2g_exchange_destroy(g2g_exchange *ex) {
    if (!ex)
        return G2G_SUCCESS;
    ex->free_plans();
    delete ex;
    return G2G_SUCCESS;
}

} // extern "C"
