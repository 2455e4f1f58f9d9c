// grid2grid C++ interface on GB300: intervals and grids.
//
// Same names, members and error behaviour as kabicm/grid2grid's
// src/grid2grid/interval.hpp:9-41 and grid2D.hpp:17-125 (this project's own
// implementation): a matrix split into a grid of blocks, each block owned by
// one rank, optionally through a rank reordering.
#pragma once

#include <algorithm>
#include <ostream>
#include <stdexcept>
#include <utility>
#include <vector>

namespace grid2grid {

// Half-open interval [start, end); negative or reversed bounds throw
// (interval.cpp:5-17).
struct interval {
    int start = 0;
    int end = 0;

    interval() = default;
    interval(int s, int e) : start(s), end(e) {
        if (s < 0 || e < 0)
            throw std::runtime_error(
                "ERROR: in class interval (grid2grid): start, end > 0 must be satisfied.");
        if (s > e)
            throw std::runtime_error(
                "ERROR: in class interval (grid2grid): start<=end must be satisfied.");
    }
    int length() const { return end - start; }
    bool contains(interval o) const { return start <= o.start && end >= o.end; }
    bool non_empty() const { return end > start; }
    bool empty() const { return end == start; }
    interval intersection(const interval &o) const {
        if (!non_empty() || !o.non_empty() || start >= o.end || end <= o.start)
            return {};
        return {std::max(start, o.start), std::min(end, o.end)};
    }
    bool operator==(const interval &o) const {
        return empty() ? o.empty() : (start == o.start && end == o.end);
    }
    bool operator!=(const interval &o) const { return !(*this == o); }
    bool operator<(const interval &o) const {
        return start < o.start || (start == o.start && end < o.end);
    }
};

inline std::ostream &operator<<(std::ostream &os, const interval &i) {
    return os << "interval[" << i.start << ", " << i.end << ")" << std::endl;
}

// Split points of a matrix into a grid of blocks: block (i, j) covers rows
// [rows_split[i], rows_split[i+1]) x cols [cols_split[j], cols_split[j+1]).
struct grid2D {
    int n_rows = 0; // blocks in a column of the grid
    int n_cols = 0; // blocks in a row of the grid
    std::vector<int> rows_split;
    std::vector<int> cols_split;

    grid2D() = default;
    grid2D(std::vector<int> &&r_split, std::vector<int> &&c_split)
        : n_rows(r_split.size() ? (int)r_split.size() - 1 : 0),
          n_cols(c_split.size() ? (int)c_split.size() - 1 : 0), rows_split(std::move(r_split)),
          cols_split(std::move(c_split)) {}

    interval row_interval(int index) const {
        if (index < 0 || (size_t)index + 1 >= rows_split.size())
            throw std::runtime_error("ERROR: in class grid2D, row index out of range.");
        return {rows_split[index], rows_split[index + 1]};
    }
    interval col_interval(int index) const {
        if (index < 0 || (size_t)index + 1 >= cols_split.size())
            throw std::runtime_error("ERROR: in class grid2D, col index out of range.");
        return {cols_split[index], cols_split[index + 1]};
    }
    void transpose() {
        std::swap(rows_split, cols_split);
        std::swap(n_rows, n_cols);
    }
};

// A grid whose block (i, j) belongs to rank ranks[i][j] (or to
// reordering[ranks[i][j]] once reorder_ranks was called).
class assigned_grid2D {
  public:
    assigned_grid2D() = default;
    assigned_grid2D(grid2D &&g, std::vector<std::vector<int>> &&proc, int n_ranks)
        : g_(std::move(g)), ranks_(std::move(proc)), n_ranks_(n_ranks) {}

    int owner(int i, int j) const { return reordered_rank(ranks_[i][j]); }
    const grid2D &grid() const { return g_; }
    int num_ranks() const { return n_ranks_; }
    interval rows_interval(int index) const { return g_.row_interval(index); }
    interval cols_interval(int index) const { return g_.col_interval(index); }
    int block_size(int row_index, int col_index) const {
        return rows_interval(row_index).length() * cols_interval(col_index).length();
    }
    void transpose() {
        g_.transpose();
        const int m = (int)ranks_.size(), n = m ? (int)ranks_[0].size() : 0;
        std::vector<std::vector<int>> t(n, std::vector<int>(m));
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < n; ++j)
                t[j][i] = ranks_[i][j];
        ranks_.swap(t);
    }
    void reorder_ranks(std::vector<int> &reordering) { reordering_ = reordering; }
    int reordered_rank(int rank) const {
        return ranks_reordered() ? reordering_[rank] : rank;
    }
    bool ranks_reordered() const { return !reordering_.empty(); }
    const std::vector<int> &reordering() const { return reordering_; }
    const std::vector<std::vector<int>> &ranks() const { return ranks_; }
    int num_blocks_row() const noexcept { return g_.n_rows; }
    int num_blocks_col() const noexcept { return g_.n_cols; }
    int num_rows() const noexcept { return g_.rows_split.empty() ? 0 : g_.rows_split.back(); }
    int num_cols() const noexcept { return g_.cols_split.empty() ? 0 : g_.cols_split.back(); }

    friend bool operator==(const assigned_grid2D &a, const assigned_grid2D &b) noexcept {
        return a.g_.rows_split == b.g_.rows_split && a.g_.cols_split == b.g_.cols_split &&
               a.ranks_ == b.ranks_;
    }

  private:
    grid2D g_;
    std::vector<std::vector<int>> ranks_;
    int n_ranks_ = 0;
    std::vector<int> reordering_;
};

} // namespace grid2grid
