// Device planner: turns the validated block tables of a plan into the
// gather-scatter work list, with no host round trip.
//
//  1. merge_parts_kernel   one CTA per (pair, dimension): a parallel merge of
//     the initial and final split vectors. Every split finds its slot in the
//     merged sequence by a binary search in the other vector (lower bound for
//     initial splits, upper bound for final splits, so equal values get two
//     slots and the part between them is empty). Each slot records the
//     initial interval ia and final interval ib the part starting there lies
//     in. This is the grid cover of the reference (grid_cover.cpp:54-121) in
//     partition form: interval k of the initial grid is covered by the final
//     intervals ib of the parts whose ia == k.
//  2. cell_tiles_kernel    one thread per (row part, col part) cell, i.e. per
//     piece of the reference's utils::decompose_block (utils.hpp:10-65):
//     the number of tiles the piece is cut into. Cells are numbered column
//     part by column part (row parts fastest), which fixes the order of the
//     work list.
//  3. scan_*               exclusive scans of the tile counts over all cells of
//     all pairs (three-phase: per-CTA sums, scan of sums, apply), one for
//     plain-copy cells and one for transposed / scaled cells: the work list
//     holds every copy tile (warp-level work) before the CTA-level tiles.
//  4. emit_tiles_kernel    one warp per cell writes the cell's tiles, with the
//     source address computed as block<T>::subblock does (block.cpp:165-196)
//     and the destination address in the final owner's block.
//  5. cover_kernel         start/end indices per initial interval, the
//     reference's interval_cover form (for the g2g_grid_cover entry point).
#include "g2g_internal.hpp"
#include "g2g_launch.hpp"

#include <cuda_runtime.h>

namespace g2g {

namespace {

// number of entries of v[0, n) that are < x
__device__ inline int lower_bound_dev(const int32_t *v, int n, int32_t x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (v[mid] < x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// number of entries of v[0, n) that are <= x
__device__ inline int upper_bound_dev(const int32_t *v, int n, int32_t x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (v[mid] <= x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__global__ void merge_parts_kernel(const PairInfo *__restrict__ pairs,
                                   const int32_t *__restrict__ splits,
                                   Part *__restrict__ parts) {
    const PairInfo p = pairs[blockIdx.x];
    const bool rows = blockIdx.y == 0;
    const int na = (rows ? p.a_nr : p.a_nc) + 1; // split entries
    const int nb = (rows ? p.b_nr : p.b_nc) + 1;
    const int32_t *A = splits + (rows ? p.a_rs : p.a_cs);
    const int32_t *B = splits + (rows ? p.b_rs : p.b_cs);
    Part *out = parts + (rows ? p.row_parts : p.col_parts);
    // slots 0 .. na+nb-1 hold the merged splits; part u spans slot u..u+1
    for (int k = threadIdx.x; k < na; k += blockDim.x) {
        int lb = lower_bound_dev(B, nb, A[k]);
        int pos = k + lb;
        out[pos].start = A[k];
        out[pos].ia = k;
        out[pos].ib = lb - 1;
    }
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        int ub = upper_bound_dev(A, na, B[i]);
        int pos = i + ub;
        out[pos].start = B[i];
        out[pos].ib = i;
        out[pos].ia = ub - 1;
    }
    __syncthreads();
    const int n_slots = na + nb;
    for (int u = threadIdx.x; u < n_slots; u += blockDim.x) {
        int len = (u + 1 < n_slots) ? out[u + 1].start - out[u].start : 0;
        // a part outside either grid (possible only for malformed input,
        // which the host rejects) is made empty
        if (out[u].ia < 0 || out[u].ia >= na - 1 || out[u].ib < 0 || out[u].ib >= nb - 1)
            len = 0;
        out[u].len = len;
    }
}

__device__ inline void cell_coords(const PairInfo &p, long long cidx, int nrp, int ncp, int &u,
                                   int &v) {
    if (p.row_major_cells) {
        u = (int)(cidx / ncp);
        v = (int)(cidx - (long long)u * ncp);
    } else {
        v = (int)(cidx / nrp);
        u = (int)(cidx - (long long)v * nrp);
    }
}

__device__ inline void tile_shape(const PairInfo &p, uint32_t kind, int len_r,
                                  int len_c, int &tr, int &tc) {
    if (kind & KIND_TRANS) {
        // transposes (plain or scaled) of 4-byte elements take twice the
        // edge, those of 8-byte elements twice the rows: a tile then holds as
        // many bytes as one of 16-byte elements
        // (4-byte ones are 4 columns short of that: a source line of at
        // most 2 td - 4 elements at any 4-byte phase lies in the 2 td / 4
        // aligned 16-byte blocks the line's lanes load, one each)
        const bool shaped = !(kind & KIND_CAST);
        const int esz = kind_esz(kind);
        tr = shaped && esz <= 8 ? 2 * p.tile_dim : p.tile_dim;
        tc = shaped && esz == 4 ? 2 * p.tile_dim - 4 : p.tile_dim;
    } else {
        int esz = kind_esz(kind);
        tr = len_r < p.tile_rows ? len_r : p.tile_rows;
        long long c = (long long)p.tile_bytes / ((long long)tr * esz);
        tc = c < 1 ? 1 : (c > (1 << 30) ? (1 << 30) : (int)c);
    }
}

// Plain copies, and non-transposed scaled or converting tiles whose
// destination elements never straddle a 16-byte chunk, are warp-level work
// items; the other (transposed, scaled, converting) tiles CTA-level ones.
// The work list holds all warp-level tiles first.
__device__ inline bool is_copy_kind(uint32_t kind) {
    if (kind & KIND_TRANS)
        return false;
    return !(kind & (KIND_SCALED | KIND_CAST)) || (kind & KIND_WARP_ELEM);
}

// A block a partial plan does not hold (one shard's part of a sharded
// transform, a packed exchange buffer) has a null address in its table; its
// cells take no part. Every listed block that is not empty has an address.
__global__ void cell_tiles_kernel(const PairInfo *__restrict__ pairs, int n_pairs,
                                  const Part *__restrict__ parts,
                                  const SrcEntry *__restrict__ src_tables,
                                  const DstEntry *__restrict__ dst_tables,
                                  long long *__restrict__ cell_tiles,
                                  long long *__restrict__ cell_tiles_cta,
                                  unsigned long long *__restrict__ n_pieces) {
    const int pi = blockIdx.y;
    const PairInfo p = pairs[pi];
    const int nrp = p.a_nr + p.b_nr + 1; // row parts (the last slot is a boundary)
    const int ncp = p.a_nc + p.b_nc + 1;
    const long long n_cells = (long long)nrp * ncp;
    unsigned long long local_pieces = 0;
    for (long long cidx = (long long)blockIdx.x * blockDim.x + threadIdx.x; cidx < n_cells;
         cidx += (long long)gridDim.x * blockDim.x) {
        // column-strip order: the row parts of one column part are
        // consecutive, so pieces that share destination (and source) columns
        // are in flight together and their boundary sectors meet in L2. A
        // transposed source is stored the other way round, so its pairs walk
        // row parts instead, keeping consecutive reads in one source column.
        int u, v;
        cell_coords(p, cidx, nrp, ncp, u, v);
        Part pr = parts[p.row_parts + u];
        Part pc = parts[p.col_parts + v];
        long long cnt = 0;
        bool copy = true;
        if (pr.len > 0 && pc.len > 0 &&
            src_tables[p.src_table + (long long)pr.ia * p.a_nc + pc.ia].data != 0 &&
            dst_tables[p.dst_table + (long long)pr.ib * p.b_nc + pc.ib].data != 0) {
            const SrcEntry e = src_tables[p.src_table + (long long)pr.ia * p.a_nc + pc.ia];
            uint32_t kind = p.kind | ((e.flags & 1u) ? KIND_TRANS : 0u) |
                            ((e.flags & 2u) ? KIND_CONJ : 0u);
            int tr, tc;
            tile_shape(p, kind, pr.len, pc.len, tr, tc);
            cnt = (long long)((pr.len + tr - 1) / tr) * ((pc.len + tc - 1) / tc);
            copy = is_copy_kind(kind);
            ++local_pieces;
        }
        cell_tiles[p.cells + cidx] = copy ? cnt : 0;
        cell_tiles_cta[p.cells + cidx] = copy ? 0 : cnt;
    }
    // one atomic per warp
    for (int off = 16; off > 0; off >>= 1)
        local_pieces += __shfl_down_sync(0xffffffffu, local_pieces, off);
    if ((threadIdx.x & 31) == 0 && local_pieces)
        atomicAdd(n_pieces, local_pieces);
}

constexpr int SCAN_THREADS = 1024;

__device__ inline long long block_exclusive_scan(long long x, long long *smem_warp,
                                                 long long &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long v = x;
    for (int off = 1; off < 32; off <<= 1) {
        long long y = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off)
            v += y;
    }
    if (lane == 31)
        smem_warp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        long long w = lane < (int)(blockDim.x >> 5) ? smem_warp[lane] : 0;
        for (int off = 1; off < 32; off <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off)
                w += y;
        }
        smem_warp[lane] = w; // inclusive scan of warp sums
    }
    __syncthreads();
    long long warp_prefix = warp ? smem_warp[warp - 1] : 0;
    total = smem_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_prefix + v - x;
}

__global__ void scan_partial_kernel(const long long *__restrict__ in, long long n,
                                    long long chunk, long long *__restrict__ sums) {
    long long begin = (long long)blockIdx.x * chunk;
    long long end = begin + chunk < n ? begin + chunk : n;
    long long s = 0;
    for (long long i = begin + threadIdx.x; i < end; i += blockDim.x)
        s += in[i];
    for (int off = 16; off > 0; off >>= 1)
        s += __shfl_down_sync(0xffffffffu, s, off);
    __shared__ long long ws[32];
    if ((threadIdx.x & 31) == 0)
        ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
            t += ws[w];
        sums[blockIdx.x] = t;
    }
}

__global__ void scan_sums_kernel(long long *__restrict__ sums, int n_sums,
                                 long long *__restrict__ total_out) {
    __shared__ long long ws[32];
    long long carry = 0;
    for (int base = 0; base < n_sums; base += blockDim.x) {
        int i = base + threadIdx.x;
        long long x = i < n_sums ? sums[i] : 0;
        long long tot;
        long long ex = block_exclusive_scan(x, ws, tot);
        if (i < n_sums)
            sums[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0)
        *total_out = carry;
}

__global__ void scan_apply_kernel(long long *__restrict__ data, long long n, long long chunk,
                                  const long long *__restrict__ sums) {
    __shared__ long long ws[32];
    long long begin = (long long)blockIdx.x * chunk;
    long long end = begin + chunk < n ? begin + chunk : n;
    long long carry = sums[blockIdx.x];
    for (long long base = begin; base < end; base += blockDim.x) {
        long long i = base + threadIdx.x;
        long long x = i < end ? data[i] : 0;
        long long tot;
        long long ex = block_exclusive_scan(x, ws, tot);
        if (i < end)
            data[i] = carry + ex;
        carry += tot;
    }
}

__global__ void emit_tiles_kernel(const PairInfo *__restrict__ pairs,
                                  const int32_t *__restrict__ splits,
                                  const Part *__restrict__ parts,
                                  const SrcEntry *__restrict__ src_tables,
                                  const DstEntry *__restrict__ dst_tables,
                                  const long long *__restrict__ cell_offsets,
                                  const long long *__restrict__ cell_offsets_cta,
                                  const long long *__restrict__ n_copy,
                                  Tile *__restrict__ tiles, long long capacity,
                                  int *__restrict__ overflow) {
    const int pi = blockIdx.y;
    const PairInfo p = pairs[pi];
    const int nrp = p.a_nr + p.b_nr + 1;
    const int ncp = p.a_nc + p.b_nc + 1;
    const long long n_cells = (long long)nrp * ncp;
    const int lane = threadIdx.x & 31;
    const long long warps_total = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long cidx = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
         cidx < n_cells; cidx += warps_total) {
        int u, v; // cell order as in cell_tiles_kernel
        cell_coords(p, cidx, nrp, ncp, u, v);
        Part pr = parts[p.row_parts + u];
        Part pc = parts[p.col_parts + v];
        if (pr.len <= 0 || pc.len <= 0)
            continue;
        const SrcEntry se = src_tables[p.src_table + (long long)pr.ia * p.a_nc + pc.ia];
        const DstEntry de = dst_tables[p.dst_table + (long long)pr.ib * p.b_nc + pc.ib];
        if (se.data == 0 || de.data == 0) // a block the plan does not hold
            continue;
        const bool trans = (se.flags & 1u) != 0;
        uint32_t kind = p.kind | (trans ? KIND_TRANS : 0u) | ((se.flags & 2u) ? KIND_CONJ : 0u);
        const int esz = kind_esz(kind), sesz = kind_src_esz(kind);
        int tr, tc;
        tile_shape(p, kind, pr.len, pc.len, tr, tc);
        const int ntr = (pr.len + tr - 1) / tr;
        const int ntc = (pc.len + tc - 1) / tc;
        const long long ntiles = (long long)ntr * ntc;
        const long long base = is_copy_kind(kind)
                                   ? cell_offsets[p.cells + cidx]
                                   : *n_copy + cell_offsets_cta[p.cells + cidx];
        if (base + ntiles > capacity) {
            if (lane == 0)
                atomicExch(overflow, 1);
            continue;
        }
        // cell origin relative to the source block (current coordinates)
        const int32_t *ars = splits + p.a_rs, *acs = splits + p.a_cs;
        const int32_t *brs = splits + p.b_rs, *bcs = splits + p.b_cs;
        const long long sr = pr.start - ars[pr.ia];
        const long long sc = pc.start - acs[pc.ia];
        const long long dr = pr.start - brs[pr.ib];
        const long long dc = pc.start - bcs[pc.ib];
        for (long long t = lane; t < ntiles; t += 32) {
            int ti = (int)(t % ntr); // row tiles fastest: consecutive tiles walk down a column
            int tj = (int)(t / ntr);
            long long r0 = (long long)ti * tr, c0 = (long long)tj * tc;
            Tile T;
            long long rr = sr + r0, cc = sc + c0;
            long long src_off = trans ? (rr * se.ld + cc) : (rr + cc * se.ld);
            T.src = se.data + (uint64_t)(src_off * sesz);
            T.dst = de.data + (uint64_t)(((dr + r0) + (dc + c0) * de.ld) * esz);
            T.src_ld = se.ld * sesz;
            T.dst_ld = de.ld * esz;
            T.rows = (int)((pr.len - r0) < tr ? (pr.len - r0) : tr);
            T.cols = (int)((pc.len - c0) < tc ? (pc.len - c0) : tc);
            T.kind = kind;
            T.pair = pi;
            tiles[base + t] = T;
        }
    }
}

__global__ void cover_kernel(const int32_t *__restrict__ a, int na,
                             const int32_t *__restrict__ b, int nb,
                             int32_t *__restrict__ start, int32_t *__restrict__ end) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < na - 1;
         k += gridDim.x * blockDim.x) {
        // max i with b[i] <= a[k]; min i with b[i] >= a[k+1]
        int s = upper_bound_dev(b, nb, a[k]) - 1;
        int e = lower_bound_dev(b, nb, a[k + 1]);
        start[k] = s < 0 ? 0 : s;
        end[k] = e > nb - 1 ? nb - 1 : e;
    }
}

} // namespace

cudaError_t launch_plan(const PlanDevice &d, int n_pairs, long long n_cells,
                        cudaStream_t stream) {
    merge_parts_kernel<<<dim3(n_pairs, 2), 256, 0, stream>>>(d.pairs, d.splits, d.parts);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess)
        return err;
    // cells: grid.y = pair, grid.x strides over the pair's cells
    int gx = (int)((d.max_cells_per_pair + 255) / 256);
    if (gx > 1024)
        gx = 1024;
    if (gx < 1)
        gx = 1;
    cell_tiles_kernel<<<dim3(gx, n_pairs), 256, 0, stream>>>(d.pairs, n_pairs, d.parts,
                                                             d.src_tables, d.dst_tables,
                                                             d.cell_tiles,
                                                             d.cell_tiles_cta, d.n_pieces);
    if ((err = cudaGetLastError()) != cudaSuccess)
        return err;
    // exclusive scans of both count arrays -> tile offsets; totals -> n_copy, n_cta
    long long chunk = 4096;
    long long nblk = (n_cells + chunk - 1) / chunk;
    if (nblk > SCAN_THREADS * 64) {
        chunk = (n_cells + SCAN_THREADS * 64 - 1) / (SCAN_THREADS * 64);
        nblk = (n_cells + chunk - 1) / chunk;
    }
    if (nblk < 1)
        nblk = 1;
    long long *arrays[2] = {d.cell_tiles, d.cell_tiles_cta};
    long long *totals[2] = {d.n_copy, d.n_cta};
    for (int k = 0; k < 2; ++k) {
        scan_partial_kernel<<<(unsigned)nblk, 256, 0, stream>>>(arrays[k], n_cells, chunk,
                                                               d.scan_sums);
        scan_sums_kernel<<<1, SCAN_THREADS, 0, stream>>>(d.scan_sums, (int)nblk, totals[k]);
        scan_apply_kernel<<<(unsigned)nblk, 256, 0, stream>>>(arrays[k], n_cells, chunk,
                                                             d.scan_sums);
    }
    if ((err = cudaGetLastError()) != cudaSuccess)
        return err;
    int ex = (int)((d.max_cells_per_pair + 7) / 8);
    if (ex > 2048)
        ex = 2048;
    if (ex < 1)
        ex = 1;
    emit_tiles_kernel<<<dim3(ex, n_pairs), 256, 0, stream>>>(
        d.pairs, d.splits, d.parts, d.src_tables, d.dst_tables, d.cell_tiles,
        d.cell_tiles_cta, d.n_copy, d.tiles, d.tile_capacity, d.overflow);
    return cudaGetLastError();
}

long long scan_sums_capacity(long long n_cells) {
    long long chunk = 4096;
    long long nblk = (n_cells + chunk - 1) / chunk;
    if (nblk > SCAN_THREADS * 64)
        nblk = SCAN_THREADS * 64;
    return nblk < 1 ? 1 : nblk;
}

cudaError_t launch_cover(const int32_t *a, int na, const int32_t *b, int nb,
                         int32_t *start, int32_t *end, cudaStream_t stream) {
    int n = na - 1;
    if (n <= 0)
        return cudaSuccess;
    int blocks = (n + 255) / 256;
    cover_kernel<<<blocks, 256, 0, stream>>>(a, na, b, nb, start, end);
    return cudaGetLastError();
}

} // namespace g2g
