// Communication volume and rank reordering on the device: the reference's
// communication_volume (src/grid2grid/transform.cpp:9-39) and
// optimal_reordering (src/grid2grid/ranks_reordering.cpp:4-61), computed
// where a sharded transform keeps its layouts, to pick the rank-to-GPU map.
//
//  volume_parts_kernel  one CTA per dimension: the merged partition of the
//                       initial and final split vectors (each split finds its
//                       slot by a binary search in the other vector).
//  volume_cells_kernel  one thread per (row part, column part) cell: the
//                       cell's elements are added to vol[min(s,d), max(s,d)],
//                       s / d the cell's initial / final owner. With few
//                       ranks the CTA sums into a shared-memory copy of the
//                       matrix first (one global atomic per entry per CTA).
//  matching_kernel      one CTA: the greedy matching by decreasing edge
//                       weight, as the locally dominant matching (every free
//                       rank points at its best edge to a free rank or at
//                       its own "stay" edge; mutual choices are matched;
//                       repeat). Under a strict order of the edges -- weight,
//                       then (r, s) -- this matching is the one the greedy
//                       pass over the sorted edge list makes.
#include "../../include/grid2grid_gb300.h"
#include "g2g_host.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

namespace {

using g2g::fail;

struct VPart {
    int32_t start, len, ia, ib;
};

// Device copy of one grid: splits and owners through its reordering.
struct VGrid {
    const int32_t *rs, *cs, *owner; // owner: row-major, reordering applied
    int nbr, nbc;
};

__device__ int vlower(const int32_t *v, int n, int32_t x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (v[mid] < x) lo = mid + 1; else hi = mid;
    }
    return lo;
}
__device__ int vupper(const int32_t *v, int n, int32_t x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (v[mid] <= x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__global__ void volume_parts_kernel(VGrid a, VGrid b, VPart *rows, VPart *cols) {
    const bool r = blockIdx.x == 0;
    const int na = (r ? a.nbr : a.nbc) + 1, nb = (r ? b.nbr : b.nbc) + 1;
    const int32_t *A = r ? a.rs : a.cs, *B = r ? b.rs : b.cs;
    VPart *out = r ? rows : cols;
    for (int k = threadIdx.x; k < na; k += blockDim.x) {
        const int lb = vlower(B, nb, A[k]);
        out[k + lb] = {A[k], 0, k, lb - 1};
    }
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        const int ub = vupper(A, na, B[i]);
        out[i + ub] = {B[i], 0, ub - 1, i};
    }
    __syncthreads();
    const int n = na + nb;
    for (int u = threadIdx.x; u < n; u += blockDim.x) {
        int len = u + 1 < n ? out[u + 1].start - out[u].start : 0;
        if (out[u].ia < 0 || out[u].ia >= na - 1 || out[u].ib < 0 || out[u].ib >= nb - 1)
            len = 0;
        out[u].len = len;
    }
}

constexpr int kSharedRanks = 64; // P x P int64 sums in shared memory up to 64 ranks

__global__ void volume_cells_kernel(VGrid a, VGrid b, const VPart *rows, int nrp,
                                    const VPart *cols, int ncp, int P,
                                    unsigned long long *vol) {
    extern __shared__ unsigned long long svol[];
    const bool local = P <= kSharedRanks;
    if (local) {
        for (int k = threadIdx.x; k < P * P; k += blockDim.x)
            svol[k] = 0;
        __syncthreads();
    }
    const long long n = (long long)nrp * ncp;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const int v = (int)(c / nrp), u = (int)(c - (long long)v * nrp);
        const VPart pr = rows[u], pc = cols[v];
        if (pr.len <= 0 || pc.len <= 0)
            continue;
        const int s = a.owner[(long long)pr.ia * a.nbc + pc.ia];
        const int d = b.owner[(long long)pr.ib * b.nbc + pc.ib];
        const int lo = s < d ? s : d, hi = s < d ? d : s;
        const unsigned long long e = (unsigned long long)pr.len * (unsigned long long)pc.len;
        if (local)
            atomicAdd(&svol[lo * P + hi], e);
        else
            atomicAdd(&vol[(long long)lo * P + hi], e);
    }
    if (local) {
        __syncthreads();
        for (int k = threadIdx.x; k < P * P; k += blockDim.x)
            if (svol[k])
                atomicAdd(&vol[k], svol[k]);
    }
}

// Edge r-s (r < s) is better than edge x-y when its weight is larger, or
// equal with (r, s) before (x, y); a rank's own edge is r-r with weight 1.
__device__ __forceinline__ bool better(long long w, int r, int s, long long w2, int r2,
                                       int s2) {
    if (w != w2)
        return w > w2;
    return r != r2 ? r < r2 : s < s2;
}

__device__ __forceinline__ long long vget(const long long *vol, int P, int r, int s) {
    return r <= s ? vol[(long long)r * P + s] : vol[(long long)s * P + r];
}

constexpr int kMatchThreads = 1024;

// partner[r]: -1 while free, else the matched rank (r itself: stays)
__global__ void __launch_bounds__(kMatchThreads)
    matching_kernel(const long long *vol, int P, int *partner, int *choice, int *on_edge,
                    int *reordered) {
    __shared__ int changed;
    for (int r = threadIdx.x; r < P; r += blockDim.x) {
        partner[r] = -1;
        int e = vol[(long long)r * P + r] > 0;
        for (int s = 0; s < P && !e; ++s)
            e = s != r && vget(vol, P, r, s) > 0;
        on_edge[r] = e;
    }
    __syncthreads();
    for (int round = 0; round <= P; ++round) {
        // every free rank picks its best edge to a free rank
        for (int r = threadIdx.x; r < P; r += blockDim.x) {
            choice[r] = -1;
            if (partner[r] >= 0)
                continue;
            long long bw = 0;
            int br = -1, bs = -1, best = -1;
            if (on_edge[r]) { // staying put weighs 1
                bw = 1;
                br = bs = best = r;
            }
            for (int s = 0; s < P; ++s) {
                if (s == r || partner[s] >= 0)
                    continue;
                const long long v = vget(vol, P, r, s);
                if (v <= 0)
                    continue;
                const long long w = v - vget(vol, P, r, r) - vget(vol, P, s, s);
                if (w == 0)
                    continue;
                const int lo = r < s ? r : s, hi = r < s ? s : r;
                if (best < 0 || better(w, lo, hi, bw, br, bs)) {
                    bw = w;
                    br = lo;
                    bs = hi;
                    best = s;
                }
            }
            choice[r] = best;
        }
        if (threadIdx.x == 0)
            changed = 0;
        __syncthreads();
        // mutual choices (and own edges) are matched
        for (int r = threadIdx.x; r < P; r += blockDim.x) {
            const int c = choice[r];
            if (c >= 0 && (c == r || choice[c] == r)) {
                partner[r] = c;
                changed = 1;
            }
        }
        __syncthreads();
        if (!changed)
            break;
        __syncthreads();
    }
    __syncthreads();
    // permutation: matched ranks swap, the others stay
    for (int r = threadIdx.x; r < P; r += blockDim.x) {
        const int c = partner[r];
        partner[r] = c < 0 ? r : c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int moved = 0;
        for (int r = 0; r < P; ++r)
            moved |= partner[r] != r;
        *reordered = moved;
    }
}

g2g_status check_volume_grid(const g2g_layout_desc *d, int P, const char *which) {
    if (!d || d->n_block_rows < 1 || d->n_block_cols < 1 || !d->rows_split || !d->cols_split ||
        !d->owners)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: empty or NULL grid", which);
    for (int i = 0; i < d->n_block_rows; ++i)
        if (d->rows_split[i + 1] < d->rows_split[i])
            return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: rows_split decreases", which);
    for (int j = 0; j < d->n_block_cols; ++j)
        if (d->cols_split[j + 1] < d->cols_split[j])
            return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: cols_split decreases", which);
    if (d->n_reordering > 0 && !d->reordering)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: reordering is NULL", which);
    const long long cells = (long long)d->n_block_rows * d->n_block_cols;
    for (long long k = 0; k < cells; ++k) {
        int o = d->owners[k];
        if (o < 0 || (d->n_reordering > 0 && o >= d->n_reordering))
            return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: owner %d out of range", which, o);
        if (d->n_reordering > 0)
            o = d->reordering[o];
        if (o < 0 || o >= P)
            return fail(G2G_ERROR_INVALID_ARGUMENT, "%s layout: owner %d outside the %d ranks",
                        which, o, P);
    }
    return G2G_SUCCESS;
}

#define VCUDA(call)                                                                     \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return fail(G2G_ERROR_CUDA, "CUDA error %s at %s:%d", cudaGetErrorString(e_), \
                        __FILE__, __LINE__);                                            \
    } while (0)

} // namespace

extern "C" {

g2g_status g2g_communication_volume_device(const g2g_layout_desc *initial,
                                           const g2g_layout_desc *final_, int32_t n_ranks,
                                           int64_t *volume, void *stream) {
    if (n_ranks < 1 || !volume)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "communication volume: bad output arguments");
    G2G_TRY(check_volume_grid(initial, n_ranks, "initial"));
    G2G_TRY(check_volume_grid(final_, n_ranks, "final"));
    const g2g_layout_desc &I = *initial, &F = *final_;
    if (I.rows_split[0] != F.rows_split[0] || I.cols_split[0] != F.cols_split[0] ||
        I.rows_split[I.n_block_rows] != F.rows_split[F.n_block_rows] ||
        I.cols_split[I.n_block_cols] != F.cols_split[F.n_block_cols])
        return fail(G2G_ERROR_INVALID_ARGUMENT,
                    "communication volume: the layouts cover different matrices");
    // one host image: both grids' splits and owners (reordering applied)
    std::vector<int32_t> img;
    size_t off[6];
    for (int k = 0; k < 2; ++k) {
        const g2g_layout_desc &d = k ? F : I;
        off[3 * k] = img.size();
        img.insert(img.end(), d.rows_split, d.rows_split + d.n_block_rows + 1);
        off[3 * k + 1] = img.size();
        img.insert(img.end(), d.cols_split, d.cols_split + d.n_block_cols + 1);
        off[3 * k + 2] = img.size();
        const size_t cells = (size_t)d.n_block_rows * d.n_block_cols;
        for (size_t c = 0; c < cells; ++c)
            img.push_back(d.n_reordering > 0 ? d.reordering[d.owners[c]] : d.owners[c]);
    }
    const int nrp = I.n_block_rows + F.n_block_rows + 2;
    const int ncp = I.n_block_cols + F.n_block_cols + 2;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t bytes = img.size() * 4 + (size_t)(nrp + ncp) * sizeof(VPart) + 64;
    char *dmem = nullptr;
    VCUDA(cudaMallocAsync((void **)&dmem, bytes, s));
    int32_t *dimg = (int32_t *)dmem;
    VPart *rows = (VPart *)(dmem + ((img.size() * 4 + 15) & ~(size_t)15));
    VPart *cols = rows + nrp;
    cudaError_t e = cudaMemcpyAsync(dimg, img.data(), img.size() * 4, cudaMemcpyHostToDevice, s);
    VGrid a{dimg + off[0], dimg + off[1], dimg + off[2], I.n_block_rows, I.n_block_cols};
    VGrid b{dimg + off[3], dimg + off[4], dimg + off[5], F.n_block_rows, F.n_block_cols};
    if (e == cudaSuccess)
        e = cudaMemsetAsync(volume, 0, sizeof(int64_t) * (size_t)n_ranks * n_ranks, s);
    if (e == cudaSuccess) {
        volume_parts_kernel<<<2, 256, 0, s>>>(a, b, rows, cols);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        const long long cells = (long long)nrp * ncp;
        int grid = (int)std::min<long long>((cells + 255) / 256, 2048);
        const size_t smem = n_ranks <= kSharedRanks ? sizeof(long long) * n_ranks * n_ranks : 0;
        volume_cells_kernel<<<std::max(grid, 1), 256, smem, s>>>(
            a, b, rows, nrp, cols, ncp, n_ranks, (unsigned long long *)volume);
        e = cudaGetLastError();
    }
    cudaError_t fe = cudaFreeAsync(dmem, s);
    if (e == cudaSuccess)
        e = fe;
    VCUDA(e);
    return G2G_SUCCESS;
}

g2g_status g2g_optimal_reordering_device(const int64_t *volume, int32_t n_ranks,
                                         int32_t *permutation, int32_t *reordered,
                                         void *stream) {
    if (!volume || n_ranks < 1 || !permutation || !reordered)
        return fail(G2G_ERROR_INVALID_ARGUMENT, "optimal reordering: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    int *scratch = nullptr;
    VCUDA(cudaMallocAsync((void **)&scratch, sizeof(int) * 2 * (size_t)n_ranks, s));
    matching_kernel<<<1, kMatchThreads, 0, s>>>((const long long *)volume, n_ranks,
                                                permutation, scratch, scratch + n_ranks,
                                                reordered);
    cudaError_t e = cudaGetLastError();
    cudaError_t fe = cudaFreeAsync(scratch, s);
    VCUDA(e);
    VCUDA(fe);
    return G2G_SUCCESS;
}

} // extern "C"
