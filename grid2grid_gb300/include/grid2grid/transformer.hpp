// grid2grid C++ interface on GB300: batched transforms.
//
// transformer<T> of kabicm/grid2grid (src/grid2grid/transformer.hpp:8-62):
// queue (from, to[, trans, alpha, beta]) pairs, then run them all in one
// collective transform -- here one launch of the device gather-scatter.
// Pairs scheduled without scalars are plain copies ('N', 1, 0); the
// reference would read past its scalar vectors when both kinds are mixed.
#pragma once

#include "transform.hpp"

namespace grid2grid {

template <typename T> struct transformer {
    std::vector<layout_ref<T>> from;
    std::vector<layout_ref<T>> to;
    std::vector<T> alpha;
    std::vector<T> beta;
    std::vector<char> transpose;

    gpu_comm comm;
    int P = 0;
    int rank = 0;

    transformer() = default;
    explicit transformer(gpu_comm c) : comm(c), P(comm_size(c)), rank(comm_rank(c)) {}

    void schedule(grid_layout<T> &from_layout, grid_layout<T> &to_layout) {
        from.push_back(from_layout);
        to.push_back(to_layout);
        alpha.push_back(T{1});
        beta.push_back(T{0});
        transpose.push_back('N');
    }

    void schedule(grid_layout<T> &from_layout, grid_layout<T> &to_layout, const char trans,
                  const T a, const T b) {
        from.push_back(from_layout);
        to.push_back(to_layout);
        alpha.push_back(a);
        beta.push_back(b);
        transpose.push_back(trans);
    }

    void transform() {
        grid2grid::transform<T>(from, to, transpose.data(), alpha.data(), beta.data(), comm);
        clear();
    }

    void clear() {
        from.clear();
        to.clear();
        alpha.clear();
        beta.clear();
        transpose.clear();
    }
};

} // namespace grid2grid
