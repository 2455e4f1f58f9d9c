// Host side of the gather-scatter: shared-memory sizes of the kernel variants
// and the launch entry, which dispatches to the translation units of the
// kernel instances (g2g_scatter_256.cu, g2g_scatter_512.cu and their
// element-arithmetic counterparts g2g_scatter_256e.cu, g2g_scatter_512e.cu),
// compiled in parallel.
#include "g2g_scatter_impl.cuh"

#include <map>
#include <mutex>
#include <tuple>

namespace g2g {

cudaError_t kernel_occupancy(const void *fn, int threads, size_t smem, int *occ) {
    static std::mutex mu;
    static std::map<std::tuple<int, const void *, int, size_t>, int> cache;
    static std::map<std::pair<int, const void *>, size_t> smem_limit; // as set so far
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess)
        return e;
    const auto key = std::make_tuple(device, fn, threads, smem);
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
        *occ = it->second;
        return cudaSuccess;
    }
    // the limit only ever grows, so every size cached for this kernel stays
    // launchable
    size_t &limit = smem_limit[std::make_pair(device, fn)];
    if (smem > 48 * 1024 && smem > limit) {
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
        limit = smem;
    }
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, smem);
    if (e != cudaSuccess)
        return e;
    cache[key] = n;
    *occ = n;
    return cudaSuccess;
}

size_t transpose_smem_bytes(int tile_dim, int esz) {
    // room for the plain transposed tiles of 4-byte elements (twice the
    // edge) and of 8-byte ones (twice the rows) too
    const size_t wide = ((size_t)(2 * tile_dim) * (size_t)(2 * tile_dim + 1) + 4u) * 4u;
    const size_t tall = (size_t)(2 * tile_dim) * (size_t)(tile_dim + 1) * 8u;
    const size_t own = (size_t)tile_dim * (size_t)(tile_dim + 1) * (size_t)esz;
    const size_t m = wide > tall ? wide : tall;
    return own > m ? own : m;
}

size_t staged_transpose_smem_bytes(int tile_dim) {
    return staged_smem_bytes(tile_dim);
}

size_t staged_scaled_transpose_smem_bytes(int tile_dim) {
    return staged_scaled_smem_bytes(tile_dim);
}

int stage_bytes_for(int tile_bytes) {
    const long long b = (long long)tile_bytes * 9 / 8 + 512;
    return (int)((b + 127) / 128 * 128);
}

size_t ring_smem_bytes(const ScatterConfig &cfg) {
    const int u = cfg.unroll == 1 ? 1 : (cfg.unroll == 2 ? 2 : 4);
    // kernels with scaled tiles stage destination chunks as well, kernels
    // with cast tiles up to three source blocks per chunk
    size_t per_warp = 0;
    switch (ring_extra_rows(cfg.paths)) {
    case 1:
        per_warp = u == 1 ? ring_warp_bytes<1, 1>()
                          : (u == 2 ? ring_warp_bytes<2, 1>() : ring_warp_bytes<4, 1>());
        break;
    case 2:
        per_warp = u == 1 ? ring_warp_bytes<1, 2>()
                          : (u == 2 ? ring_warp_bytes<2, 2>() : ring_warp_bytes<4, 2>());
        break;
    default:
        per_warp = u == 1 ? ring_warp_bytes<1, 0>()
                          : (u == 2 ? ring_warp_bytes<2, 0>() : ring_warp_bytes<4, 0>());
    }
    const size_t ring = (size_t)(cfg.threads / 32) * per_warp;
    return ring > cfg.trans_bytes ? ring : cfg.trans_bytes;
}

size_t staged_smem_bytes(const ScatterConfig &cfg) {
    return 128 + (size_t)cfg.stages * (size_t)cfg.stage_bytes + cfg.trans_bytes;
}

cudaError_t launch_scatter(const PlanList &list, const ScatterConfig &cfg,
                           cudaStream_t stream) {
    if (cfg.grid <= 0 || list.n < 1 || list.n > kMaxPlansPerLaunch)
        return cudaErrorInvalidConfiguration;
    if (list.total_copy + list.total_cta <= 0)
        return cudaSuccess;
    const bool elem = (cfg.paths & (PATH_SCALED | PATH_CAST)) != 0;
    switch (cfg.threads) {
    case 512:
        return elem ? launch_scatter_512_elem(list, cfg, stream)
                    : launch_scatter_512(list, cfg, stream);
    default:
        return elem ? launch_scatter_256_elem(list, cfg, stream)
                    : launch_scatter_256(list, cfg, stream);
    }
}

cudaError_t preload_scatter_kernels() {
    PlanList list;
    list.n = 1;
    list.total_copy = 1;
    const int path_sets[] = {PATH_COPY, PATH_TRANSPOSE, PATH_COPY | PATH_TRANSPOSE,
                             PATH_TRANSPOSE | PATH_NARROW_TRANSPOSE,
                             PATH_COPY | PATH_TRANSPOSE | PATH_NARROW_TRANSPOSE,
                             PATH_TRANSPOSE | PATH_NARROW_TRANSPOSE | PATH_W4_STAGED,
                             PATH_TRANSPOSE | PATH_NARROW_TRANSPOSE | PATH_W8_STAGED,
                             PATH_TRANSPOSE | PATH_W16_STAGED,
                             PATH_COPY | PATH_SCALED_REAL, PATH_COPY | PATH_SCALED_COMPLEX,
                             PATH_COPY | PATH_CAST, PATH_SCALED_REAL | PATH_W4S_STAGED,
                             PATH_SCALED | PATH_W8S_STAGED};
    for (int threads : {256, 512})
        for (int unroll : {1, 2, 4})
            for (int paths : path_sets)
                for (int mode = 0; mode <= 4; ++mode) { // direct, ring, 2..4 stages
                    if (mode >= 1 && !(paths & PATH_COPY))
                        continue;
                    ScatterConfig c;
                    c.threads = threads;
                    c.unroll = unroll;
                    c.grid = 1;
                    c.paths = paths;
                    c.tile_dim = 32;
                    c.trans_bytes = c.smem_bytes = transpose_smem_bytes(32, 16);
                    if (paths & (PATH_W4_STAGED | PATH_W8_STAGED | PATH_W16_STAGED))
                        c.smem_bytes = staged_smem_bytes(32);
                    if (paths & (PATH_W4S_STAGED | PATH_W8S_STAGED))
                        c.smem_bytes = staged_scaled_smem_bytes(32);
                    c.ring = mode == 1;
                    c.stages = mode >= 2 ? mode : 0;
                    c.stage_bytes = stage_bytes_for(16 * 1024);
                    c.dry_run = true;
                    const cudaError_t e = launch_scatter(list, c, nullptr);
                    if (e != cudaSuccess)
                        return e;
                }
    return cudaSuccess;
}

} // namespace g2g
