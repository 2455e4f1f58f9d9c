// Internal device-side structures shared by the host planner (g2g_capi.cpp),
// the device planner (g2g_planner.cu) and the gather-scatter kernels
// (g2g_scatter.cu). Not part of the public ABI.
//
// Data layout in HBM for one plan (all arrays device-resident, written once
// at plan time, read by every execution):
//   PairInfo[n_pairs]           per-pair geometry offsets and scalars
//   int32 splits[]              initial (possibly transposed) and final splits
//   SrcEntry  src_table[]       dense initial block table, per pair
//   DstEntry  dst_table[]       dense final block table, per pair
//   Part      parts[]           merged row/col parts per pair and dimension
//   int64     cell_tiles[]      tile count per (row part, col part) cell, scanned
//   Tile      tiles[]           the gather-scatter work list (48 B each)
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace g2g {

// Tile kind bits.
enum : uint32_t {
    KIND_ESZ_MASK = 0x3u,   // element size: 0 -> 4 B, 1 -> 8 B, 2 -> 16 B
    KIND_TRANS = 0x4u,      // source is read transposed
    KIND_CONJ = 0x8u,       // flip the sign of the imaginary part
    KIND_SCALED = 0x10u,    // dst = beta*dst + alpha*src instead of a copy
    KIND_CAST = 0x20u,      // source elements of another type, converted
    KIND_WARP_ELEM = 0x40u, // with KIND_SCALED or KIND_CAST: every destination
                            // element lies inside one 16-byte chunk, so
                            // non-transposed tiles are warp-level work items
    KIND_DTYPE_SHIFT = 8u,  // g2g_dtype in bits 8-9 (the destination's)
    KIND_SRC_DTYPE_SHIFT = 10u, // with KIND_CAST: the source's g2g_dtype, bits 10-11
};

__host__ __device__ inline int kind_esz(uint32_t kind) { return 4 << (kind & KIND_ESZ_MASK); }
// Bytes of a source element: the destination's unless the tile converts.
__host__ __device__ inline int kind_src_esz(uint32_t kind) {
    if (!(kind & KIND_CAST))
        return kind_esz(kind);
    const uint32_t dt = (kind >> KIND_SRC_DTYPE_SHIFT) & 3u; // 0 f32, 1 f64, 2 c64, 3 c128
    return dt == 0 ? 4 : (dt == 3 ? 16 : 8);
}

// One entry of the dense initial block table: where block (i, j) of the
// (transposed) initial grid lives. The table has one entry per grid block.
struct SrcEntry {
    uint64_t data;   // byte address of the block's element (0, 0)
    int64_t ld;      // stride in elements
    uint32_t flags;  // bit 0 transpose_on_copy, bit 1 conjugate_on_copy
    uint32_t pad;
};

struct DstEntry {
    uint64_t data;
    int64_t ld;
};

// Per-pair geometry. Offsets index the plan's concatenated arrays.
struct PairInfo {
    int32_t a_nr, a_nc;        // initial grid: block rows / cols
    int32_t b_nr, b_nc;        // final grid
    int32_t a_rs, a_cs;        // offsets of initial rows/cols splits in splits[]
    int32_t b_rs, b_cs;        // offsets of final rows/cols splits
    int64_t src_table;         // offset of the pair's SrcEntry table
    int64_t dst_table;         // offset of the pair's DstEntry table
    int64_t row_parts;         // offset in parts[] of the a_nr + b_nr + 1 row parts
    int64_t col_parts;         // offset in parts[] of the a_nc + b_nc + 1 col parts
    int64_t cells;             // offset of the pair's cells in cell_tiles[]
    uint32_t kind;             // esz / dtype / scaled bits shared by all pieces
    int32_t tile_rows;         // non-transposed tile: max rows per tile
    int32_t tile_bytes;        // non-transposed tile: target bytes per tile
    int32_t tile_dim;          // transposed tile edge (elements)
    int32_t row_major_cells;   // 1: cells numbered row part by row part (pairs
                               // whose source is read transposed), 0: column
                               // strips (row parts fastest)
    double alpha[2];
    double beta[2];
};

// One part of the merged partition of a dimension: the half-open range
// [start, start + len) lies inside interval ia of the initial grid and
// interval ib of the final grid. len == 0 for a boundary both grids share.
struct Part {
    int32_t start;
    int32_t len;
    int32_t ia;
    int32_t ib;
};

// One work item of the gather-scatter: a rows x cols sub-rectangle in final
// coordinates. Column c of the destination starts at dst + c*dst_ld; the
// source element (r, c) is at src + c*src_ld + r*esz, or at
// src + r*src_ld + c*esz when the tile is transposed.
struct __align__(16) Tile {
    uint64_t src;
    uint64_t dst;
    int64_t src_ld;   // bytes
    int64_t dst_ld;   // bytes
    int32_t rows;
    int32_t cols;
    uint32_t kind;
    int32_t pair;
};
static_assert(sizeof(Tile) == 48, "Tile is 48 bytes");

} // namespace g2g
