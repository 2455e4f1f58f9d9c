// grid2grid C++ interface on GB300: communication volume and rank reordering.
//
// comm_volume, communication_volume and optimal_reordering of kabicm/grid2grid
// (src/grid2grid/comm_volume.hpp, transform.cpp:9-39,
// ranks_reordering.cpp:4-61) with the same names and meaning, over
// g2g_communication_volume / g2g_optimal_reordering. Volumes are 64-bit here
// (the reference sums element counts in int). The greedy matching takes
// tied weights in (rank, rank) order; the reference's order for ties is its
// hash map's.
#pragma once

#include "transform.hpp"

#include <unordered_map>
#include <utility>
#include <vector>

namespace grid2grid {

struct edge_t {
    int src = 0;
    int dest = 0;
    edge_t() = default;
    edge_t(int s, int d) : src(s), dest(d) {}
    edge_t sorted() const { return src <= dest ? edge_t{src, dest} : edge_t{dest, src}; }
    bool operator==(const edge_t &o) const { return src == o.src && dest == o.dest; }
};

struct edge_hash {
    size_t operator()(const edge_t &e) const {
        return std::hash<long long>()(((long long)e.src << 32) ^ (unsigned)e.dest);
    }
};

struct comm_volume {
    using volume_t = std::unordered_map<edge_t, long long, edge_hash>;
    volume_t volume; // edge {min rank, max rank} -> elements exchanged
    comm_volume() = default;
    explicit comm_volume(volume_t &&v) : volume(std::move(v)) {}
    comm_volume &operator+=(const comm_volume &o) {
        for (const auto &kv : o.volume)
            volume[kv.first.sorted()] += kv.second;
        return *this;
    }
    comm_volume operator+(const comm_volume &o) const {
        comm_volume r = *this;
        r += o;
        return r;
    }
    size_t total_volume() const {
        size_t s = 0;
        for (const auto &kv : volume)
            if (kv.first.src != kv.first.dest)
                s += (size_t)kv.second;
        return s;
    }
};

namespace detail {
// A descriptor of a grid and its owners only (no blocks).
struct grid_desc {
    std::vector<int32_t> rs, cs, owners, reordering;
    g2g_layout_desc d;
    explicit grid_desc(const assigned_grid2D &g) {
        rs.assign(g.grid().rows_split.begin(), g.grid().rows_split.end());
        cs.assign(g.grid().cols_split.begin(), g.grid().cols_split.end());
        for (const std::vector<int> &row : g.ranks())
            owners.insert(owners.end(), row.begin(), row.end());
        reordering.assign(g.reordering().begin(), g.reordering().end());
        std::memset(&d, 0, sizeof(d));
        d.n_block_rows = g.grid().n_rows;
        d.n_block_cols = g.grid().n_cols;
        d.rows_split = rs.data();
        d.cols_split = cs.data();
        d.owners = owners.data();
        d.n_ranks = g.num_ranks();
        d.n_reordering = (int32_t)reordering.size();
        d.reordering = reordering.empty() ? nullptr : reordering.data();
    }
};
inline int ranks_of(const assigned_grid2D &a, const assigned_grid2D &b) {
    int P = a.num_ranks() > b.num_ranks() ? a.num_ranks() : b.num_ranks();
    for (int r : a.reordering())
        P = r + 1 > P ? r + 1 : P;
    for (int r : b.reordering())
        P = r + 1 > P ? r + 1 : P;
    return P;
}
} // namespace detail

// Elements each pair of ranks exchanges in transform(g_init -> g_final)
// (transform.cpp:9-39).
inline comm_volume communication_volume(assigned_grid2D &g_init, assigned_grid2D &g_final) {
    detail::grid_desc a(g_init), b(g_final);
    const int P = detail::ranks_of(g_init, g_final);
    std::vector<int64_t> v((size_t)P * P);
    detail::check(g2g_communication_volume(&a.d, &b.d, P, v.data()));
    comm_volume::volume_t w;
    for (int r = 0; r < P; ++r)
        for (int s = r; s < P; ++s)
            if (v[(size_t)r * P + s])
                w[edge_t{r, s}] = v[(size_t)r * P + s];
    return comm_volume(std::move(w));
}

// The rank relabeling that keeps the most data local (ranks_reordering.cpp:4-61).
inline std::vector<int> optimal_reordering(comm_volume &volume, int n_ranks, bool &reordered) {
    std::vector<int64_t> v((size_t)n_ranks * n_ranks, 0);
    for (const auto &kv : volume.volume) {
        const edge_t e = kv.first.sorted();
        if (e.src < 0 || e.dest >= n_ranks)
            throw std::runtime_error("grid2grid (GB300): edge outside the ranks");
        v[(size_t)e.src * n_ranks + e.dest] += kv.second;
    }
    std::vector<int32_t> p(n_ranks);
    int32_t re = 0;
    detail::check(g2g_optimal_reordering(v.data(), n_ranks, p.data(), &re));
    reordered = re != 0;
    return std::vector<int>(p.begin(), p.end());
}

} // namespace grid2grid
