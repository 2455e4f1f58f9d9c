// g2g_transform_noalloc: the one-shot transform for callers that cannot
// allocate device memory -- applications that hand all of HBM to their own
// pool allocator and forbid any other allocation, processes held to a strict
// per-process memory quota, and latency-critical loops that cannot afford the
// implicit device synchronisation of cudaFree. It allocates nothing: the
// planner's metadata and the gather-scatter work list live in the
// file-scope device array below, and the host side calls no cudaMalloc*,
// cudaFree*, cudaMallocHost / cudaHostAlloc, stream or event creation, nor
// any allocating library routine. (Validation copies the caller's
// descriptors into ordinary host containers, as g2g_plan_create does.)
//
// Limits and sharing:
//  * the array holds kNoAllocScratchBytes (32 MiB) on every GPU on which
//    this code is loaded, until the process exits; a transform whose metadata
//    needs more (roughly: more than ~600 000 work tiles) is rejected with
//    G2G_ERROR_OUT_OF_MEMORY before any device work is queued;
//  * every call uses the same array and leaves the last call's metadata in
//    it; the counters a call needs zeroed are cleared by that call. Calls
//    that overlap on the GPU race on the array: issue them one at a time per
//    device (each call returns only after its transform has completed);
//  * the first call on a device resolves the array's device address with
//    cudaGetSymbolAddress while that device is current.
#include "g2g_host.hpp"

#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

namespace {

constexpr size_t kNoAllocScratchBytes = 32u << 20;
constexpr int kMaxDevices = 64;

// File-scope scratch: plan metadata of the most recent no-allocation call.
static __device__ __align__(256) unsigned char g2g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_scratch_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on `device` (which must be current).
// In host code the array's name is only a host-side stand-in, never a device
// address, so the address is resolved here, once per device.
g2g_status scratch_for(int device, unsigned char **out) {
    if (device < 0 || device >= kMaxDevices)
        return g2g::fail(G2G_ERROR_UNSUPPORTED, "no-allocation transform: device %d", device);
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g2g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return g2g::fail(G2G_ERROR_CUDA,
                             "no-allocation transform: cudaGetSymbolAddress failed: %s",
                             cudaGetErrorString(e));
        g_scratch_addr[device] = p;
    }
    *out = (unsigned char *)g_scratch_addr[device];
    return G2G_SUCCESS;
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

#define NOALLOC_CUDA(call)                                                              \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return g2g::fail(G2G_ERROR_CUDA, "no-allocation transform: %s at %s:%d",    \
                             cudaGetErrorString(e_), __FILE__, __LINE__);               \
    } while (0)

} // namespace

extern "C" g2g_status g2g_transform_noalloc(const g2g_layout_desc *initial,
                                            const g2g_layout_desc *final_, g2g_dtype dtype,
                                            const g2g_op *op, void *stream) {
    g2g::HostPlanImage img;
    g2g_status st = g2g::build_host_image(initial, final_, dtype, op, &img);
    if (st != G2G_SUCCESS)
        return st;
    unsigned char *base = nullptr;
    st = scratch_for(img.device, &base);
    if (st != G2G_SUCCESS)
        return st;

    // carve the metadata out of the scratch array
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = align_up(off + (bytes ? bytes : 1), 256);
        return o;
    };
    const size_t o_pairs = take(sizeof(g2g::PairInfo) * img.pairs.size());
    const size_t o_splits = take(sizeof(int32_t) * img.splits.size());
    const size_t o_src = take(sizeof(g2g::SrcEntry) * img.src_tables.size());
    const size_t o_dst = take(sizeof(g2g::DstEntry) * img.dst_tables.size());
    const size_t o_parts = take(sizeof(g2g::Part) * (size_t)img.n_parts);
    const size_t o_cells = take(sizeof(long long) * (size_t)img.n_cells);
    const size_t o_cells_cta = take(sizeof(long long) * (size_t)img.n_cells);
    const size_t o_sums =
        take(sizeof(long long) * (size_t)g2g::scan_sums_capacity(img.n_cells));
    const size_t o_counters = take(64);
    const size_t o_tiles = take(sizeof(g2g::Tile) * (size_t)img.tile_capacity);
    if (off > kNoAllocScratchBytes)
        return g2g::fail(G2G_ERROR_OUT_OF_MEMORY,
                         "no-allocation transform: the plan needs %zu bytes of metadata but "
                         "the fixed scratch holds %zu; use g2g_transform",
                         off, kNoAllocScratchBytes);

    g2g::PlanDevice d;
    d.pairs = (g2g::PairInfo *)(base + o_pairs);
    d.splits = (int32_t *)(base + o_splits);
    d.src_tables = (g2g::SrcEntry *)(base + o_src);
    d.dst_tables = (g2g::DstEntry *)(base + o_dst);
    d.parts = (g2g::Part *)(base + o_parts);
    d.cell_tiles = (long long *)(base + o_cells);
    d.cell_tiles_cta = (long long *)(base + o_cells_cta);
    d.scan_sums = (long long *)(base + o_sums);
    d.n_copy = (long long *)(base + o_counters);
    d.n_pieces = (unsigned long long *)(base + o_counters + 8);
    d.overflow = (int *)(base + o_counters + 16);
    d.status = (int *)(base + o_counters + 24);
    d.n_cta = (long long *)(base + o_counters + 32);
    d.tiles = (g2g::Tile *)(base + o_tiles);
    d.tile_capacity = img.tile_capacity;
    d.max_cells_per_pair = img.max_cells_per_pair;

    cudaStream_t s = (cudaStream_t)stream;
    NOALLOC_CUDA(cudaMemcpyAsync(d.pairs, img.pairs.data(),
                                 sizeof(g2g::PairInfo) * img.pairs.size(),
                                 cudaMemcpyHostToDevice, s));
    NOALLOC_CUDA(cudaMemcpyAsync(d.splits, img.splits.data(),
                                 sizeof(int32_t) * img.splits.size(), cudaMemcpyHostToDevice,
                                 s));
    if (!img.src_tables.empty())
        NOALLOC_CUDA(cudaMemcpyAsync(d.src_tables, img.src_tables.data(),
                                     sizeof(g2g::SrcEntry) * img.src_tables.size(),
                                     cudaMemcpyHostToDevice, s));
    if (!img.dst_tables.empty())
        NOALLOC_CUDA(cudaMemcpyAsync(d.dst_tables, img.dst_tables.data(),
                                     sizeof(g2g::DstEntry) * img.dst_tables.size(),
                                     cudaMemcpyHostToDevice, s));
    // the previous call's counters are still in the array: clear them
    NOALLOC_CUDA(cudaMemsetAsync(base + o_counters, 0, 64, s));
    NOALLOC_CUDA(g2g::launch_plan(d, (int)img.pairs.size(), img.n_cells, s));
    long long counters[5] = {0, 0, 0, 0, 0};
    NOALLOC_CUDA(cudaMemcpyAsync(counters, base + o_counters, sizeof(counters),
                                 cudaMemcpyDeviceToHost, s));
    NOALLOC_CUDA(cudaStreamSynchronize(s));
    if (((int *)counters)[4] != 0)
        return g2g::fail(G2G_ERROR_CUDA,
                         "no-allocation transform: work list exceeded its bound");
    const long long n_copy = counters[0], n_cta = counters[4];
    if (n_copy + n_cta > 0) {
        g2g::PlanList l;
        l.n = 1;
        l.status = d.status;
        l.total_copy = n_copy;
        l.total_cta = n_cta;
        l.p[0].tiles = d.tiles;
        l.p[0].pairs = d.pairs;
        l.p[0].first_copy = 0;
        l.p[0].first_cta = 0;
        l.p[0].n_copy = n_copy;
        g2g::ScatterConfig cfg = img.cfg;
        long long g = (long long)cfg.sm_count * cfg.ctas_per_sm;
        cfg.grid = (int)(g < 1 ? 1 : g);
        NOALLOC_CUDA(g2g::launch_scatter(l, cfg, s));
    }
    // finish before returning: the next call reuses the array
    int status = 0;
    NOALLOC_CUDA(cudaMemcpyAsync(&status, d.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    NOALLOC_CUDA(cudaStreamSynchronize(s));
    if (status != 0)
        return g2g::fail(G2G_ERROR_TIMEOUT, "no-allocation transform: a bounded wait expired");
    return G2G_SUCCESS;
}
