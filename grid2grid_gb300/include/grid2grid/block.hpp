// grid2grid C++ interface on GB300: locally stored blocks.
//
// Same names and meaning as kabicm/grid2grid's src/grid2grid/block.hpp:60-190
// (this project's own implementation). The data pointer of a block is a
// DEVICE address here: the block is a column-major view of caller-owned GPU
// memory with an arbitrary stride.
#pragma once

#include "grid2D.hpp"

#include <algorithm>
#include <vector>

namespace grid2grid {

struct block_coordinates {
    int row = 0;
    int col = 0;
    block_coordinates() = default;
    block_coordinates(int r, int c) : row(r), col(c) {}
    void transpose() { std::swap(row, col); }
};

struct block_range {
    interval rows_interval;
    interval cols_interval;
    block_range() = default;
    block_range(interval r, interval c) : rows_interval(r), cols_interval(c) {}
    block_range intersection(const block_range &o) const {
        return {rows_interval.intersection(o.rows_interval),
                cols_interval.intersection(o.cols_interval)};
    }
    bool non_empty() const { return rows_interval.non_empty() && cols_interval.non_empty(); }
    bool empty() const { return rows_interval.empty() || cols_interval.empty(); }
};

// A column-major block of rows_interval x cols_interval at `data` with
// leading dimension `stride`. After transpose_or_conjugate('T'/'C') the
// intervals and coordinates are those of the transposed layout and the
// memory still holds the untransposed block (block.cpp:249-288).
template <typename T> struct block {
    int tag = 0;
    interval rows_interval;
    interval cols_interval;
    bool transpose_on_copy = false;
    bool conjugate_on_copy = false;
    block_coordinates coordinates;
    T *data = nullptr;
    int stride = 0;

    block() = default;
    block(const assigned_grid2D &grid, block_coordinates coord, T *ptr, int stride_)
        : rows_interval(grid.rows_interval(coord.row)),
          cols_interval(grid.cols_interval(coord.col)), coordinates(coord), data(ptr),
          stride(stride_) {}
    block(const assigned_grid2D &grid, block_coordinates coord, T *ptr)
        : block(grid, coord, ptr, grid.rows_interval(coord.row).length()) {}
    block(interval r, interval c, block_coordinates coord, T *ptr, int stride_)
        : rows_interval(r), cols_interval(c), coordinates(coord), data(ptr), stride(stride_) {}
    block(interval r, interval c, block_coordinates coord, T *ptr)
        : block(r, c, coord, ptr, r.length()) {}
    block(block_range &range, block_coordinates coord, T *ptr, int stride_)
        : block(range.rows_interval, range.cols_interval, coord, ptr, stride_) {}
    block(block_range &range, block_coordinates coord, T *ptr)
        : block(range.rows_interval, range.cols_interval, coord, ptr) {}
    // coordinates found from the grid (the interval's start among the splits)
    block(const assigned_grid2D &grid, interval r, interval c, T *ptr, int stride_)
        : rows_interval(r), cols_interval(c), data(ptr), stride(stride_) {
        coordinates = block_coordinates(index_of(grid.grid().rows_split, r.start),
                                        index_of(grid.grid().cols_split, c.start));
    }
    block(const assigned_grid2D &grid, interval r, interval c, T *ptr)
        : block(grid, r, c, ptr, r.length()) {}
    block(const assigned_grid2D &grid, block_range &range, T *ptr, int stride_)
        : block(grid, range.rows_interval, range.cols_interval, ptr, stride_) {}
    block(const assigned_grid2D &grid, block_range &range, T *ptr)
        : block(grid, range.rows_interval, range.cols_interval, ptr) {}

    int n_rows() const { return rows_interval.length(); }
    int n_cols() const { return cols_interval.length(); }
    std::pair<int, int> size() const { return {n_rows(), n_cols()}; }
    size_t total_size() const { return (size_t)n_rows() * (size_t)n_cols(); }
    bool non_empty() const { return rows_interval.non_empty() && cols_interval.non_empty(); }

    // the sub-rectangle [r_range x c_range] (current coordinates) as a block
    // view of the same memory (block.cpp:165-196)
    block<T> subblock(interval r_range, interval c_range) const {
        if (!rows_interval.contains(r_range) || !cols_interval.contains(c_range))
            throw std::runtime_error(
                "ERROR: current block does not contain requested subblock.");
        interval rr = r_range, cr = c_range, rb = rows_interval, cb = cols_interval;
        if (transpose_on_copy) {
            std::swap(rr, cr);
            std::swap(rb, cb);
        }
        block<T> b = *this;
        b.rows_interval = r_range;
        b.cols_interval = c_range;
        b.data = data + (size_t)(cr.start - cb.start) * stride + (rr.start - rb.start);
        return b;
    }

    void transpose_or_conjugate(char flag) {
        if (flag != 'T' && flag != 'C')
            return;
        std::swap(rows_interval, cols_interval);
        coordinates.transpose();
        transpose_on_copy = true; // set, never cleared, as in block.cpp:283-287
        if (flag == 'C')
            conjugate_on_copy = true;
    }

    bool operator<(const block &o) const {
        if (cols_interval != o.cols_interval)
            return cols_interval < o.cols_interval;
        if (rows_interval != o.rows_interval)
            return rows_interval < o.rows_interval;
        return tag < o.tag;
    }

  private:
    static int index_of(const std::vector<int> &splits, int start) {
        return (int)(std::lower_bound(splits.begin(), splits.end(), start) - splits.begin());
    }
};

template <typename T> bool operator==(const block<T> &a, const block<T> &b) noexcept {
    return a.rows_interval.start == b.rows_interval.start &&
           a.rows_interval.end == b.rows_interval.end &&
           a.cols_interval.start == b.cols_interval.start &&
           a.cols_interval.end == b.cols_interval.end &&
           a.coordinates.row == b.coordinates.row && a.coordinates.col == b.coordinates.col &&
           a.stride == b.stride && a.data == b.data &&
           a.transpose_on_copy == b.transpose_on_copy &&
           a.conjugate_on_copy == b.conjugate_on_copy;
}

// The blocks one rank holds (block.hpp:167-190).
template <typename T> class local_blocks {
  public:
    local_blocks() = default;
    explicit local_blocks(std::vector<block<T>> &&blocks) : blocks_(std::move(blocks)) {
        for (const block<T> &b : blocks_)
            total_size_ += b.total_size();
    }
    block<T> &get_block(int i) { return blocks_[i]; }
    const block<T> &get_block(int i) const { return blocks_[i]; }
    int num_blocks() const { return (int)blocks_.size(); }
    size_t size() const { return total_size_; }
    void transpose_or_conjugate(char flag) {
        for (block<T> &b : blocks_)
            b.transpose_or_conjugate(flag);
    }
    friend bool operator==(const local_blocks &a, const local_blocks &b) noexcept {
        return a.blocks_ == b.blocks_;
    }

  private:
    std::vector<block<T>> blocks_;
    size_t total_size_ = 0;
};

} // namespace grid2grid
