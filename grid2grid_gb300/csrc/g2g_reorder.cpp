// Communication volume between virtual ranks and the rank reordering that
// keeps most of it local (the reference's communication_volume,
// src/grid2grid/transform.cpp:9-39, and optimal_reordering,
// src/grid2grid/ranks_reordering.cpp:4-61). Host-side: they read the grids
// and owners only, as the reference does before a transform.
#include "g2g_host.hpp"

#include <grid2grid_gb300.h>

#include <algorithm>
#include <cstring>
#include <vector>

namespace {

using g2g::fail;

g2g_status check_grid(const g2g_layout_desc *d, int32_t n_ranks, const char *which) {
    if (!d)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout is NULL", which);
    if (d->n_block_rows < 1 || d->n_block_cols < 1 || !d->rows_split || !d->cols_split ||
        !d->owners)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: empty grid", which);
    for (int i = 0; i < d->n_block_rows; ++i)
        if (d->rows_split[i + 1] < d->rows_split[i])
            return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: rows_split decreases", which);
    for (int j = 0; j < d->n_block_cols; ++j)
        if (d->cols_split[j + 1] < d->cols_split[j])
            return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: cols_split decreases", which);
    if (d->n_reordering > 0 && !d->reordering)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: reordering is NULL", which);
    const int64_t cells = (int64_t)d->n_block_rows * d->n_block_cols;
    for (int64_t k = 0; k < cells; ++k) {
        int o = d->owners[k];
        if (o < 0 || (d->n_reordering > 0 && o >= d->n_reordering))
            return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: owner %d out of range", which,
                        o);
        if (d->n_reordering > 0)
            o = d->reordering[o];
        if (o < 0 || o >= n_ranks)
            return fail(G2G_ERROR_INVALID_ARGUMENT,
                        "%s layout: owner %d outside the %d ranks", which, o, n_ranks);
    }
    return G2G_SUCCESS;
}

int owner(const g2g_layout_desc *d, int i, int j) {
    const int o = d->owners[(size_t)i * d->n_block_cols + j];
    return d->n_reordering > 0 ? d->reordering[o] : o;
}

// The merged partition of two split vectors: for each part, its length and
// the block of either vector it lies in (grid_cover.cpp:54-121 on both).
struct MergedPart {
    int64_t len;
    int a, b;
};
std::vector<MergedPart> merge(const int32_t *a, int na, const int32_t *b, int nb) {
    std::vector<MergedPart> out;
    int i = 0, j = 0;
    int64_t pos = a[0];
    while (i < na && j < nb) {
        const int64_t end = std::min<int64_t>(a[i + 1], b[j + 1]);
        if (end > pos)
            out.push_back({end - pos, i, j});
        pos = std::max<int64_t>(pos, end);
        if (a[i + 1] <= pos)
            ++i;
        if (j < nb && b[j + 1] <= pos)
            ++j;
    }
    return out;
}

struct Edge {
    int64_t w;
    int r, s;
};

} // namespace

extern "C" {

g2g_status g2g_communication_volume(const g2g_layout_desc *initial,
                                    const g2g_layout_desc *final_, int32_t n_ranks,
                                    int64_t *volume) {
    if (n_ranks < 1 || !volume)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "communication volume: bad output arguments");
    G2G_TRY(check_grid(initial, n_ranks, "initial"));
    G2G_TRY(check_grid(final_, n_ranks, "final"));
    const g2g_layout_desc &I = *initial, &F = *final_;
    if (I.rows_split[0] != F.rows_split[0] || I.cols_split[0] != F.cols_split[0] ||
        I.rows_split[I.n_block_rows] != F.rows_split[F.n_block_rows] ||
        I.cols_split[I.n_block_cols] != F.cols_split[F.n_block_cols])
        return fail(G2G_ERROR_INVALID_ARGUMENT,
                    "communication volume: the layouts cover different matrices");
    std::memset(volume, 0, sizeof(int64_t) * (size_t)n_ranks * (size_t)n_ranks);
    const std::vector<MergedPart> rows =
        merge(I.rows_split, I.n_block_rows, F.rows_split, F.n_block_rows);
    const std::vector<MergedPart> cols =
        merge(I.cols_split, I.n_block_cols, F.cols_split, F.n_block_cols);
    for (const MergedPart &c : cols)
        for (const MergedPart &r : rows) {
            const int src = owner(&I, r.a, c.a), dst = owner(&F, r.b, c.b);
            const int lo = std::min(src, dst), hi = std::max(src, dst);
            volume[(size_t)lo * n_ranks + hi] += r.len * c.len;
        }
    return G2G_SUCCESS;
}

g2g_status g2g_optimal_reordering(const int64_t *volume, int32_t n_ranks,
                                  int32_t *permutation, int32_t *reordered) {
    if (!volume || n_ranks < 1 || !permutation)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "optimal reordering: bad arguments");
    const size_t P = (size_t)n_ranks;
    auto vol = [&](int r, int s) { return volume[(size_t)r * P + s]; };
    // the edges that carry volume, and every rank on one of them kept where
    // it is (weight 1)
    std::vector<char> on_edge(P, 0);
    std::vector<Edge> edges;
    for (int r = 0; r < n_ranks; ++r)
        for (int s = r + 1; s < n_ranks; ++s)
            if (vol(r, s) > 0) {
                on_edge[r] = on_edge[s] = 1;
                const int64_t w = vol(r, s) - vol(r, r) - vol(s, s);
                if (w != 0)
                    edges.push_back({w, r, s});
            }
    for (int r = 0; r < n_ranks; ++r)
        if (on_edge[r] || vol(r, r) > 0)
            edges.push_back({1, r, r});
    std::stable_sort(edges.begin(), edges.end(), [](const Edge &x, const Edge &y) {
        if (x.w != y.w)
            return x.w > y.w;
        return x.r != y.r ? x.r < y.r : x.s < y.s;
    });
    std::vector<char> visited(P, 0);
    for (int r = 0; r < n_ranks; ++r)
        permutation[r] = r;
    bool moved = false;
    for (const Edge &e : edges) {
        if (visited[e.r] || visited[e.s])
            continue;
        permutation[e.r] = e.s;
        permutation[e.s] = e.r;
        if (e.r != e.s)
            moved = true;
        visited[e.r] = visited[e.s] = 1;
    }
    if (reordered)
        *reordered = moved ? 1 : 0;
    return G2G_SUCCESS;
}

} // extern "C"
