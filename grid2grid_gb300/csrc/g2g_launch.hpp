// Host-callable launchers for the device code (planner and gather-scatter).
#pragma once

#include "g2g_internal.hpp"

#include <cuda_runtime.h>

namespace g2g {

// Device pointers of one plan's metadata (all inside one allocation).
struct PlanDevice {
    PairInfo *pairs = nullptr;
    int32_t *splits = nullptr;
    SrcEntry *src_tables = nullptr;
    DstEntry *dst_tables = nullptr;
    Part *parts = nullptr;
    long long *cell_tiles = nullptr;     // copy-tile counts, then exclusive offsets
    long long *cell_tiles_cta = nullptr; // transposed/scaled tile counts, then offsets
    long long *scan_sums = nullptr;
    Tile *tiles = nullptr;               // [copy tiles | CTA-level tiles]
    long long *n_copy = nullptr;         // device scalar: copy tiles
    long long *n_cta = nullptr;          // device scalar: CTA-level tiles
    unsigned long long *n_pieces = nullptr;
    int *overflow = nullptr;           // device flag: tile capacity exceeded
    int *status = nullptr;             // device flag: kernel error (bounded wait expired)
    long long tile_capacity = 0;
    long long max_cells_per_pair = 0;
};

// Runs the device planner (merge, tile counts, scan, emission) on `stream`.
cudaError_t launch_plan(const PlanDevice &d, int n_pairs, long long n_cells,
                        cudaStream_t stream);
long long scan_sums_capacity(long long n_cells);

// Grid cover (interval_cover form) of split vector a by b, device arrays.
cudaError_t launch_cover(const int32_t *a, int na, const int32_t *b, int nb,
                         int32_t *start, int32_t *end, cudaStream_t stream);

// Plans executed by one launch of the gather-scatter: a persistent kernel
// walks the concatenation of their work lists. Passed by value as a
// __grid_constant__ kernel parameter (8 KB), so a launch uploads nothing.
constexpr int kMaxPlansPerLaunch = 256;
struct PlanRef {
    const Tile *tiles;       // the plan's work list: n_copy copy tiles, then n_cta
    const PairInfo *pairs;
    long long first_copy;    // index of the plan's first copy tile in the launch
    long long first_cta;     // index of the plan's first CTA-level tile
    long long n_copy;
};
struct PlanList {
    int n = 0;
    int pad = 0;
    long long total_copy = 0; // copy tiles over all plans (warp-level items)
    long long total_cta = 0;  // transposed / scaled tiles (CTA-level items)
    int *status = nullptr;
    PlanRef p[kMaxPlansPerLaunch];
};

struct ScatterConfig {
    int threads = 256;       // 128, 256 or 512
    int unroll = 4;          // 1, 2, 4 or 8
    int grid = 0;            // CTAs (persistent); 0 = SM count x ctas_per_sm
    int ctas_per_sm = 4;
    int sm_count = 0;        // for the residency clamp of the persistent grid
    int tile_dim = 32;       // transposed tile edge (16 or 32)
    size_t smem_bytes = 0;   // dynamic shared memory (transposed tiles)
    int paths = 7;           // tile paths present: 1 copy, 2 transpose, 4 scaled real,
                             // 8 scaled complex, 16 cast, 32 transposes of 4- or
                             // 8-byte elements, 64 / 128 transposes of 4- / 8-byte
                             // elements as the only CTA-level tiles, 1024 / 2048
                             // scaled transposes of 4- / 8-byte elements only
    int stages = 0;          // TMA staging ring depth for plain copies (0 = none)
    int ring = 0;            // plain copies through the per-warp cp.async ring
    int run_shift = 0;       // ring: runs of 2^run_shift consecutive tiles per warp
    int l2_prefetch = 0;     // ring: bulk L2 prefetch of each tile's source columns
    int stage_bytes = 0;     // bytes per stage
    size_t trans_bytes = 0;  // shared memory for direct transposed / scaled tiles
    bool dry_run = false;    // prepare the kernel instance (load it, query its
                             // occupancy, raise its shared-memory limit), no launch
};

// Stage size that holds any plain tile of `tile_bytes` whose columns are at
// least 256 bytes: columns are staged as their 16-byte aligned cover.
int stage_bytes_for(int tile_bytes);
// Dynamic shared memory of the staged kernel.
size_t staged_smem_bytes(const ScatterConfig &cfg);
// Dynamic shared memory of the ring kernel.
size_t ring_smem_bytes(const ScatterConfig &cfg);
// Resident CTAs per SM of kernel `fn` at `threads` threads and `smem` bytes
// of dynamic shared memory on the current device; sets the kernel's shared
// memory limit first when it is above the default. Computed once per
// (device, kernel, threads, smem) and cached: launches pay a table lookup.
cudaError_t kernel_occupancy(const void *fn, int threads, size_t smem, int *occ);
// The kernel instances by CTA size, plain and element-arithmetic plans
// apart (one translation unit each, compiled in parallel).
cudaError_t launch_scatter_256(const PlanList &list, const ScatterConfig &cfg,
                               cudaStream_t stream);
cudaError_t launch_scatter_512(const PlanList &list, const ScatterConfig &cfg,
                               cudaStream_t stream);
cudaError_t launch_scatter_256_elem(const PlanList &list, const ScatterConfig &cfg,
                                    cudaStream_t stream);
cudaError_t launch_scatter_512_elem(const PlanList &list, const ScatterConfig &cfg,
                                    cudaStream_t stream);


// Shared memory a transposed tile of edge `tile_dim` with elements of `esz`
// bytes needs (at least that of a plain transposed tile of 4-byte elements,
// whose edge is twice `tile_dim`).
size_t transpose_smem_bytes(int tile_dim, int esz);

// Shared memory of the staged ring of plain transposed tiles of 4- or 8-byte
// elements (tile paths with bit 64 or 128: those tiles, of one element size,
// are a launch's only tiles).
size_t staged_transpose_smem_bytes(int tile_dim);
// ... and of the staged ring of scaled transposed tiles (bits 1024 / 2048),
// whose stages hold the destination columns too.
size_t staged_scaled_transpose_smem_bytes(int tile_dim);

// Launches the gather-scatter over the plans of `list`.
cudaError_t launch_scatter(const PlanList &list, const ScatterConfig &cfg,
                           cudaStream_t stream);

// Plain copies as 2-D tensor-map boxes (g2g_tma.cu). One box moves a
// box_rows x box_cols sub-block from the source block's tensor map at
// (sx, sy) to the destination block's at (dx, dy); coordinates are in map
// words (4 or 8 bytes) along the rows and in columns.
struct TmaBox {
    int32_t src_map, dst_map; // indices into the plan's tensor maps (128 B each)
    int32_t sx, sy, dx, dy;
};
struct TmaPlan {
    const unsigned char *maps = nullptr; // device, 128-byte tensor maps
    const TmaBox *boxes = nullptr;       // device work list
    long long n_boxes = 0;
    int box_bytes = 0;
};
// Encodes a 2-D tensor map over a column-major block: rows_words words of
// word_bytes (4 or 8) per column, `cols` columns ld_bytes apart, boxes of
// box_rows_words x box_cols. Host only (driver entry point).
cudaError_t encode_box_map(void *map, const void *base, int word_bytes, uint64_t rows_words,
                           uint64_t cols, uint64_t ld_bytes, uint32_t box_rows_words,
                           uint32_t box_cols);
size_t tma_smem_bytes(int box_bytes);
cudaError_t launch_tma_boxes(const TmaPlan &p, int sm_count, int *status, cudaStream_t s);

// Prepares every kernel instance a plan or a merged launch can select on the
// current device (dry runs of launch_scatter), so that no later launch pays
// for loading its module lazily.
cudaError_t preload_scatter_kernels();

} // namespace g2g
