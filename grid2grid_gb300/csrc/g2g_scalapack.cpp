// ScaLAPACK-descriptor front end: block-cyclic layouts over all virtual ranks
// (the reference's get_scalapack_grid, src/grid2grid/scalapack_layout.cpp
// :152-278, for every rank at once) and p?gemr2d on one GPU.
#include "g2g_host.hpp"

#include <grid2grid_gb300.h>

#include <cstring>
#include <new>
#include <utility>
#include <vector>

struct g2g_layout {
    std::vector<int32_t> rows_split, cols_split, owners;
    std::vector<g2g_block_desc> blocks;
    g2g_layout_desc desc;
};

namespace {

using g2g::fail;

int dtype_bytes(g2g_dtype dt) {
    switch (dt) {
    case G2G_FLOAT32: return 4;
    case G2G_FLOAT64: return 8;
    case G2G_COMPLEX64: return 8;
    case G2G_COMPLEX128: return 16;
    default: return 0;
    }
}

// Split points of [begin, end) at multiples of blk, relative to begin
// (scalapack_layout.cpp:152-177).
std::vector<int32_t> line_split(int64_t begin, int64_t end, int64_t blk) {
    const int64_t len = end - begin;
    const int64_t rem = blk - begin % blk;
    std::vector<int32_t> s{0};
    if (rem >= len) {
        s.push_back((int32_t)len);
        return s;
    }
    s.push_back((int32_t)rem);
    for (int64_t k = 0; k < (len - rem) / blk; ++k)
        s.push_back((int32_t)(s.back() + blk));
    if (s.back() != len)
        s.push_back((int32_t)len);
    return s;
}

int rank_from_grid(int pr, int pc, const g2g_scalapack_desc &d) {
    return d.row_major ? pr * d.npcol + pc : pc * d.nprow + pr;
}

// Block rows (or columns) of an extent owned by process coordinate p when
// the first block sits on process src.
int64_t owned_blocks(int64_t extent, int64_t blk, int p, int src, int np) {
    const int64_t nb = (extent + blk - 1) / blk;
    const int rel = ((p - src) % np + np) % np;
    return nb / np + (rel < nb % np ? 1 : 0);
}

g2g_status check_desc(const g2g_scalapack_desc *d, const char *what) {
    if (!d)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s: descriptor is NULL", what);
    if (d->m < 0 || d->n < 0 || d->mb < 1 || d->nb < 1 || d->nprow < 1 || d->npcol < 1)
        return fail(G2G_ERROR_INVALID_ARGUMENT,
                    "%s: need m, n >= 0, mb, nb >= 1 and a process grid of at least 1x1", what);
    if (d->rsrc < 0 || d->rsrc >= d->nprow || d->csrc < 0 || d->csrc >= d->npcol)
        return fail(G2G_ERROR_INVALID_ARGUMENT,
                    "%s: source process (%d, %d) outside the %dx%d grid", what, d->rsrc,
                    d->csrc, d->nprow, d->npcol);
    if ((int64_t)d->nprow * d->npcol > (1 << 24))
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s: process grid too large", what);
    return G2G_SUCCESS;
}

g2g_status build(const g2g_scalapack_desc *d, int32_t ia, int32_t ja, int32_t m, int32_t n,
                 void *const *rank_data, const int32_t *lld, g2g_dtype dtype, g2g_layout &L,
                 const char *what) {
    G2G_TRY(check_desc(d, what));
    const int esz = dtype_bytes(dtype);
    if (!esz)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s: unknown dtype %d", what, (int)dtype);
    if (m < 0 || n < 0)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s: negative submatrix size", what);
    if (ia < 1 || ja < 1)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s: ia, ja are 1-based", what);
    if ((int64_t)ia - 1 + m > d->m || (int64_t)ja - 1 + n > d->n)
        return fail(G2G_ERROR_INVALID_ARGUMENT,
                    "%s: submatrix (%d:%d, %d:%d) outside the %dx%d matrix", what, ia,
                    ia + m - 1, ja, ja + n - 1, d->m, d->n);
    const int P = d->nprow * d->npcol;
    if (!rank_data)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s: rank data pointers are NULL", what);
    // leading dimensions: given, or the rank's local block rows x mb
    std::vector<int64_t> llds(P);
    for (int r = 0; r < P; ++r) {
        const int pr = d->row_major ? r / d->npcol : r % d->nprow;
        const int64_t local_rows = owned_blocks(d->m, d->mb, pr, d->rsrc, d->nprow) * d->mb;
        llds[r] = lld ? (int64_t)lld[r] : (local_rows > 0 ? local_rows : 1);
        if (llds[r] < 1)
            return fail(G2G_ERROR_INVALID_ARGUMENT, "%s: lld[%d] = %lld < 1", what, r,
                        (long long)llds[r]);
    }
    const int64_t i0 = ia - 1, j0 = ja - 1;
    L.rows_split = line_split(i0, i0 + m, d->mb);
    L.cols_split = line_split(j0, j0 + n, d->nb);
    const int nbr = (int)L.rows_split.size() - 1, nbc = (int)L.cols_split.size() - 1;
    const int64_t br0 = i0 / d->mb, bc0 = j0 / d->nb;
    const int src_r = (int)((br0 % d->nprow + d->rsrc) % d->nprow);
    const int src_c = (int)((bc0 % d->npcol + d->csrc) % d->npcol);
    L.owners.assign((size_t)nbr * nbc, 0);
    L.blocks.clear();
    L.blocks.reserve((size_t)nbr * nbc);
    // column by column, as get_scalapack_grid emits a rank's blocks
    for (int j = 0; j < nbc; ++j)
        for (int i = 0; i < nbr; ++i) {
            const int pr = (i % d->nprow + src_r) % d->nprow;
            const int pc = (j % d->npcol + src_c) % d->npcol;
            const int o = rank_from_grid(pr, pc, *d);
            L.owners[(size_t)i * nbc + j] = o;
            if (!rank_data[o])
                return fail(G2G_ERROR_INVALID_ARGUMENT,
                            "%s: rank %d owns blocks but its data pointer is NULL", what, o);
            const int64_t loc_r = (br0 + i) / d->nprow, loc_c = (bc0 + j) / d->npcol;
            const int64_t sub_r = i0 + L.rows_split[i] - (br0 + i) * d->mb;
            const int64_t sub_c = j0 + L.cols_split[j] - (bc0 + j) * d->nb;
            const int64_t rows = L.rows_split[i + 1] - L.rows_split[i];
            const int64_t off = loc_r * d->mb + sub_r + llds[o] * (loc_c * d->nb + sub_c);
            if (rows > 0 && llds[o] < loc_r * d->mb + sub_r + rows)
                return fail(G2G_ERROR_INVALID_ARGUMENT,
                            "%s: lld[%d] = %lld is below the rank's local rows (%lld)", what, o,
                            (long long)llds[o], (long long)(loc_r * d->mb + sub_r + rows));
            g2g_block_desc b;
            std::memset(&b, 0, sizeof(b));
            b.rank = o;
            b.row = i;
            b.col = j;
            b.stride = llds[o];
            b.data = (void *)((uintptr_t)rank_data[o] + (uintptr_t)(off * esz));
            L.blocks.push_back(b);
        }
    std::memset(&L.desc, 0, sizeof(L.desc));
    L.desc.n_block_rows = nbr;
    L.desc.n_block_cols = nbc;
    L.desc.rows_split = L.rows_split.data();
    L.desc.cols_split = L.cols_split.data();
    L.desc.owners = L.owners.data();
    L.desc.n_ranks = P;
    L.desc.n_blocks = (int32_t)L.blocks.size();
    L.desc.blocks = L.blocks.data();
    return G2G_SUCCESS;
}

// Every argument of a gemr2d call that its plan depends on.
g2g::Sig gemr2d_key(int32_t m, int32_t n, void *const *a_data, int32_t ia, int32_t ja,
                    const g2g_scalapack_desc *da, const int32_t *lld_a, void *const *b_data,
                    int32_t ib, int32_t jb, const g2g_scalapack_desc *db, const int32_t *lld_b,
                    g2g_dtype dtype, const g2g_op *op) {
    g2g::Sig k;
    k.add((uint32_t)0x67656d72u); // a tag apart from the layout signatures
    const int32_t v[] = {m, n, ia, ja, ib, jb, (int32_t)dtype};
    k.add(v);
    for (const auto &side : {std::make_pair(da, std::make_pair(a_data, lld_a)),
                             std::make_pair(db, std::make_pair(b_data, lld_b))}) {
        const g2g_scalapack_desc *d = side.first;
        const int32_t f[] = {d->m, d->n, d->mb, d->nb, d->rsrc, d->csrc,
                             d->nprow, d->npcol, d->row_major};
        k.add(f);
        const size_t P = (size_t)d->nprow * (size_t)d->npcol;
        k.add(side.second.first, P * sizeof(void *));
        if (side.second.second)
            k.add(side.second.second, P * sizeof(int32_t));
        else
            k.add((int32_t)-1);
    }
    g2g_op o;
    std::memset(&o, 0, sizeof(o));
    o.trans = 'N';
    o.alpha[0] = 1.0;
    if (op) {
        o.trans = op->trans;
        std::memcpy(o.alpha, op->alpha, sizeof(o.alpha));
        std::memcpy(o.beta, op->beta, sizeof(o.beta));
    }
    k.add(o.trans);
    k.add(o.alpha);
    k.add(o.beta);
    return k;
}

} // namespace

extern "C" {

g2g_status g2g_layout_create_scalapack(const g2g_scalapack_desc *desc, int32_t ia, int32_t ja,
                                       int32_t m, int32_t n, void *const *rank_data,
                                       const int32_t *lld, g2g_dtype dtype,
                                       g2g_layout **layout) {
    if (!layout)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "layout output pointer is NULL");
    *layout = nullptr;
    g2g_layout *L = new (std::nothrow) g2g_layout();
    if (!L)
        return fail(G2G_ERROR_OUT_OF_MEMORY, "host allocation failed");
    const g2g_status st = build(desc, ia, ja, m, n, rank_data, lld, dtype, *L, "scalapack layout");
    if (st != G2G_SUCCESS) {
        delete L;
        return st;
    }
    *layout = L;
    return G2G_SUCCESS;
}

g2g_status g2g_layout_get_desc(const g2g_layout *layout, g2g_layout_desc *out) {
    if (!layout || !out)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "layout or output is NULL");
    *out = layout->desc;
    return G2G_SUCCESS;
}

g2g_status g2g_layout_destroy(g2g_layout *layout) {
    delete layout;
    return G2G_SUCCESS;
}

g2g_status g2g_gemr2d(int32_t m, int32_t n, void *const *a_data, int32_t ia, int32_t ja,
                      const g2g_scalapack_desc *desc_a, const int32_t *lld_a,
                      void *const *b_data, int32_t ib, int32_t jb,
                      const g2g_scalapack_desc *desc_b, const int32_t *lld_b, g2g_dtype dtype,
                      const g2g_op *op, void *stream) {
    if (m < 0 || n < 0)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "gemr2d: negative size %d x %d", m, n);
    const char t = op ? (char)(op->trans >= 'a' ? op->trans - 32 : op->trans) : 'N';
    const bool trans = t == 'T' || t == 'C';
    G2G_TRY(check_desc(desc_a, "gemr2d A"));
    G2G_TRY(check_desc(desc_b, "gemr2d B"));
    if (m == 0 || n == 0)
        return G2G_SUCCESS;
    if (!a_data || !b_data)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "gemr2d: rank data array is NULL");
    // The call's own arguments key the plan cache, so a repeated call (an
    // iterative caller's usual pattern) skips building both block lists
    // (p x q blocks each) and hashing them.
    const g2g::Sig key = gemr2d_key(m, n, a_data, ia, ja, desc_a, lld_a, b_data, ib, jb, desc_b,
                                    lld_b, dtype, op);
    return g2g::cached_one_shot(
        &key,
        [&](g2g_plan **plan) {
            g2g_layout A, B;
            G2G_TRY(build(desc_a, ia, ja, trans ? n : m, trans ? m : n, a_data, lld_a, dtype, A,
                          "gemr2d A"));
            G2G_TRY(build(desc_b, ib, jb, m, n, b_data, lld_b, dtype, B, "gemr2d B"));
            if (A.desc.n_ranks != B.desc.n_ranks) {
                // one set of virtual ranks: the smaller grid's ranks are a prefix
                const int32_t P =
                    A.desc.n_ranks > B.desc.n_ranks ? A.desc.n_ranks : B.desc.n_ranks;
                A.desc.n_ranks = P;
                B.desc.n_ranks = P;
            }
            return g2g_plan_create(&A.desc, &B.desc, dtype, op, nullptr, plan);
        },
        stream);
}

} // extern "C"
