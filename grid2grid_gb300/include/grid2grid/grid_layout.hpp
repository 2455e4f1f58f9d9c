// grid2grid C++ interface on GB300: one rank's view of a layout.
//
// Same names and meaning as kabicm/grid2grid's src/grid2grid/grid_layout.hpp:7-66
// (this project's own implementation).
#pragma once

#include "block.hpp"

#include <cctype>
#include <functional>

namespace grid2grid {

template <typename T> class grid_layout {
  public:
    grid_layout() = default;
    grid_layout(assigned_grid2D &&g, local_blocks<T> &&b)
        : grid(std::move(g)), blocks(std::move(b)) {}

    int num_ranks() const { return grid.num_ranks(); }

    // 'T' / 'C' transpose the grid and the owners and mark every local block
    // (grid_layout.hpp:18-25); 'N' does nothing; any other flag throws.
    void transpose_or_conjugate(char flag) {
        flag = (char)std::toupper((unsigned char)flag);
        if (flag != 'N' && flag != 'T' && flag != 'C')
            throw std::runtime_error("ERROR: transpose flag must be N, T or C.");
        if (flag == 'T' || flag == 'C') {
            grid.transpose();
            blocks.transpose_or_conjugate(flag);
        }
    }
    void reorder_ranks(std::vector<int> &reordering) { grid.reorder_ranks(reordering); }
    int reordered_rank(int rank) const { return grid.reordered_rank(rank); }
    bool ranks_reordered() const { return grid.ranks_reordered(); }
    int num_cols() const noexcept { return grid.num_cols(); }
    int num_rows() const noexcept { return grid.num_rows(); }
    int num_blocks_col() const noexcept { return grid.num_blocks_col(); }
    int num_blocks_row() const noexcept { return grid.num_blocks_row(); }

    assigned_grid2D grid;
    local_blocks<T> blocks;
};

template <typename T> using layout_ref = std::reference_wrapper<grid_layout<T>>;

} // namespace grid2grid
