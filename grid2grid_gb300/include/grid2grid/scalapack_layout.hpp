// grid2grid C++ interface on GB300: block-cyclic (ScaLAPACK) layouts.
//
// The layout builders of kabicm/grid2grid (src/grid2grid/scalapack_layout.hpp
// :11-429, scalapack_layout.cpp:10-346) with the same names and meaning
// (this project's own implementation): get_scalapack_grid (all four
// overloads) builds one rank's grid_layout of a block-cyclic matrix, with
// submatrix offset, rank-grid ordering and source process; the buffer
// pointer is that rank's DEVICE buffer. initialize_locally / validate work on
// a rank's HOST copy of its buffer, as in the reference's tests.
#pragma once

#include "grid_layout.hpp"

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdlib>
#include <iostream>
#include <vector>

namespace grid2grid {
namespace scalapack {

enum ordering { row_major, column_major };

struct int_pair {
    int row = 0;
    int col = 0;
    int_pair() = default;
    int_pair(int r, int c) : row(r), col(c) {}
    void transpose() { std::swap(row, col); }
};
struct rank_grid_coord : int_pair {
    using int_pair::int_pair;
    rank_grid_coord() = default;
};
struct rank_decomposition : int_pair {
    using int_pair::int_pair;
    rank_decomposition() = default;
    int n_total() const { return row * col; }
};
struct elem_grid_coord : int_pair {
    using int_pair::int_pair;
    elem_grid_coord() = default;
};
struct block_dim : int_pair {
    using int_pair::int_pair;
    block_dim() = default;
    int size() const { return row * col; }
};
struct matrix_dim : int_pair {
    using int_pair::int_pair;
    matrix_dim() = default;
    int size() const { return row * col; }
};

struct data_layout {
    matrix_dim matrix_dimension;
    block_dim block_dimension;
    rank_decomposition rank_grid;
    ordering rank_grid_ordering = ordering::column_major;
    data_layout() = default;
    data_layout(matrix_dim m, block_dim b, rank_decomposition r, ordering o)
        : matrix_dimension(m), block_dimension(b), rank_grid(r), rank_grid_ordering(o) {}
};

// scalapack_layout.cpp:10-24
inline rank_grid_coord rank_to_grid(int rank, rank_decomposition g, ordering o) {
    if (rank < 0 || rank >= g.n_total())
        throw std::runtime_error("Error in rank_to_grid: rank does not belong to the grid.");
    return o == ordering::column_major ? rank_grid_coord(rank % g.row, rank / g.row)
                                       : rank_grid_coord(rank / g.col, rank % g.col);
}

// scalapack_layout.cpp:40-57
inline int rank_from_grid(rank_grid_coord c, rank_decomposition g, ordering o) {
    if (c.row < 0 || c.row >= g.row || c.col < 0 || c.col >= g.col)
        throw std::runtime_error(
            "Error in rank_from_grid: rank coordinates do not belong to the rank grid.");
    return o == ordering::column_major ? c.col * g.row + c.row : c.row * g.col + c.col;
}

namespace detail {
// blocks of a dimension owned by process coordinate p (scalapack_layout.cpp:122-139)
inline int owned_blocks(int extent, int blk, int p, int np) {
    const int nb = (extent + blk - 1) / blk;
    return nb / np + (p < nb % np ? 1 : 0);
}
// global element of local index li held by process coordinate p
inline int global_index(int li, int blk, int p, int np) {
    return ((li / blk) * np + p) * blk + li % blk;
}
} // namespace detail

// Elements of rank's local buffer, padding of partial blocks included
// (scalapack_layout.cpp:141-149).
inline size_t local_size(int rank, const data_layout &l) {
    const rank_grid_coord c = rank_to_grid(rank, l.rank_grid, l.rank_grid_ordering);
    const size_t r = (size_t)detail::owned_blocks(l.matrix_dimension.row, l.block_dimension.row,
                                                  c.row, l.rank_grid.row);
    const size_t k = (size_t)detail::owned_blocks(l.matrix_dimension.col, l.block_dimension.col,
                                                  c.col, l.rank_grid.col);
    return r * k * (size_t)l.block_dimension.row * (size_t)l.block_dimension.col;
}

// Fills a rank's local (host) buffer with f(global row, global col), padding
// with T() (scalapack_layout.hpp:299-331).
template <typename T, typename Function>
void initialize_locally(T *buffer, Function f, int rank, const data_layout &l) {
    const rank_grid_coord c = rank_to_grid(rank, l.rank_grid, l.rank_grid_ordering);
    const int lr = detail::owned_blocks(l.matrix_dimension.row, l.block_dimension.row, c.row,
                                        l.rank_grid.row) *
                   l.block_dimension.row;
    const size_t n = local_size(rank, l);
    for (size_t i = 0; i < n; ++i) {
        const int li = (int)(i % (size_t)(lr ? lr : 1)), lj = (int)(i / (size_t)(lr ? lr : 1));
        const int gi = detail::global_index(li, l.block_dimension.row, c.row, l.rank_grid.row);
        const int gj = detail::global_index(lj, l.block_dimension.col, c.col, l.rank_grid.col);
        buffer[i] = (gi < l.matrix_dimension.row && gj < l.matrix_dimension.col)
                        ? (T)f(gi, gj)
                        : T();
    }
}

// Checks a rank's local (host) buffer against f (scalapack_layout.hpp:333-383).
template <typename Function, typename T>
bool validate(Function f, const std::vector<T> &buffer, int rank, const data_layout &l,
              double eps = 1e-6) {
    if (buffer.size() != local_size(rank, l))
        return false;
    const rank_grid_coord c = rank_to_grid(rank, l.rank_grid, l.rank_grid_ordering);
    const int lr = detail::owned_blocks(l.matrix_dimension.row, l.block_dimension.row, c.row,
                                        l.rank_grid.row) *
                   l.block_dimension.row;
    bool ok = true;
    for (size_t i = 0; i < buffer.size(); ++i) {
        const int li = (int)(i % (size_t)(lr ? lr : 1)), lj = (int)(i / (size_t)(lr ? lr : 1));
        const int gi = detail::global_index(li, l.block_dimension.row, c.row, l.rank_grid.row);
        const int gj = detail::global_index(lj, l.block_dimension.col, c.col, l.rank_grid.col);
        if (gi >= l.matrix_dimension.row || gj >= l.matrix_dimension.col)
            continue;
        if (std::abs(buffer[i] - (T)f(gi, gj)) > eps) {
            std::cout << "(" << gi << ", " << gj << ") = " << buffer[i] << " instead of "
                      << (T)f(gi, gj) << std::endl;
            ok = false;
        }
    }
    return ok;
}

} // namespace scalapack

namespace detail {
// split points of [begin, end) at multiples of blk, relative to begin
// (scalapack_layout.cpp:152-177)
inline std::vector<int> line_split(int begin, int end, int blk) {
    const int len = end - begin;
    const int rem = blk - begin % blk;
    std::vector<int> s{0};
    if (rem >= len) {
        s.push_back(len);
        return s;
    }
    s.push_back(rem);
    for (int k = 0; k < (len - rem) / blk; ++k)
        s.push_back(s.back() + blk);
    if (s.back() != len)
        s.push_back(len);
    return s;
}
} // namespace detail

// One rank's grid_layout of a block-cyclic matrix (scalapack_layout.cpp:178-278):
// lld = local leading dimension, ij = 1-based start of the submatrix,
// subm_dim its size, rank_src the process holding the first block.
template <typename T>
grid_layout<T> get_scalapack_grid(int lld, scalapack::matrix_dim m_dim,
                                  scalapack::elem_grid_coord ij, scalapack::matrix_dim subm_dim,
                                  scalapack::block_dim b_dim,
                                  scalapack::rank_decomposition r_grid,
                                  scalapack::ordering rank_grid_ordering,
                                  scalapack::rank_grid_coord rank_src, T *ptr, const int rank) {
    (void)m_dim;
    if (ij.row < 1 || ij.col < 1)
        throw std::runtime_error("get_scalapack_grid: ij is 1-based");
    const int i0 = ij.row - 1, j0 = ij.col - 1;
    std::vector<int> rs = detail::line_split(i0, i0 + subm_dim.row, b_dim.row);
    std::vector<int> cs = detail::line_split(j0, j0 + subm_dim.col, b_dim.col);
    const int nbr = (int)rs.size() - 1, nbc = (int)cs.size() - 1;
    const int br0 = i0 / b_dim.row, bc0 = j0 / b_dim.col;
    const int src_r = (br0 % r_grid.row + rank_src.row) % r_grid.row;
    const int src_c = (bc0 % r_grid.col + rank_src.col) % r_grid.col;
    std::vector<std::vector<int>> owners(nbr, std::vector<int>(nbc));
    std::vector<block<T>> blocks;
    for (int j = 0; j < nbc; ++j) {
        const int pc = (j % r_grid.col + src_c) % r_grid.col;
        for (int i = 0; i < nbr; ++i) {
            const int pr = (i % r_grid.row + src_r) % r_grid.row;
            owners[i][j] = scalapack::rank_from_grid(scalapack::rank_grid_coord(pr, pc), r_grid,
                                                     rank_grid_ordering);
            if (owners[i][j] != rank)
                continue;
            const int loc_r = (br0 + i) / r_grid.row, loc_c = (bc0 + j) / r_grid.col;
            const int sub_r = i0 + rs[i] - (br0 + i) * b_dim.row;
            const int sub_c = j0 + cs[j] - (bc0 + j) * b_dim.col;
            const size_t off = (size_t)(loc_r * b_dim.row + sub_r) +
                               (size_t)lld * (size_t)(loc_c * b_dim.col + sub_c);
            T *p = reinterpret_cast<T *>(reinterpret_cast<uintptr_t>(ptr) + off * sizeof(T));
            blocks.push_back(block<T>(interval(rs[i], rs[i + 1]), interval(cs[j], cs[j + 1]),
                                      block_coordinates(i, j), p, lld));
        }
    }
    grid2D g(std::move(rs), std::move(cs));
    assigned_grid2D ag(std::move(g), std::move(owners), r_grid.n_total());
    return grid_layout<T>(std::move(ag), local_blocks<T>(std::move(blocks)));
}

template <typename T>
grid_layout<T> get_scalapack_grid(int lld, scalapack::matrix_dim m_dim,
                                  scalapack::elem_grid_coord ij, scalapack::matrix_dim subm_dim,
                                  scalapack::block_dim b_dim,
                                  scalapack::rank_decomposition r_grid,
                                  scalapack::ordering rank_grid_ordering,
                                  scalapack::rank_grid_coord rank_src, const T *ptr,
                                  const int rank) {
    return get_scalapack_grid<T>(lld, m_dim, ij, subm_dim, b_dim, r_grid, rank_grid_ordering,
                                 rank_src, const_cast<T *>(ptr), rank);
}

// Whole matrix, leading dimension = the rank's local rows
// (scalapack_layout.cpp:305-335).
template <typename T>
grid_layout<T> get_scalapack_grid(scalapack::matrix_dim m_dim, scalapack::block_dim b_dim,
                                  scalapack::rank_decomposition r_grid,
                                  scalapack::ordering rank_grid_ordering, T *ptr, int rank) {
    const scalapack::rank_grid_coord c =
        scalapack::rank_to_grid(rank, r_grid, rank_grid_ordering);
    const int lld =
        scalapack::detail::owned_blocks(m_dim.row, b_dim.row, c.row, r_grid.row) * b_dim.row;
    return get_scalapack_grid<T>(lld, m_dim, scalapack::elem_grid_coord(1, 1), m_dim, b_dim,
                                 r_grid, rank_grid_ordering, scalapack::rank_grid_coord(0, 0),
                                 ptr, rank);
}

template <typename T>
grid_layout<T> get_scalapack_grid(scalapack::data_layout &layout, T *ptr, int rank) {
    return get_scalapack_grid<T>(layout.matrix_dimension, layout.block_dimension,
                                 layout.rank_grid, layout.rank_grid_ordering, ptr, rank);
}

} // namespace grid2grid
