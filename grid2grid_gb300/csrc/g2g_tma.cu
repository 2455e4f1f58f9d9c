// Plain copies as 2-D tensor-map boxes: the Blackwell TMA path of the
// gather-scatter.
//
// When every block of a plan lies at a 16-byte aligned address with a
// leading dimension that is a multiple of 16 bytes, and every piece of the
// transform is a whole number of boxes of one shape (the split points of
// both grids are multiples of the box's rows and columns, as in block-cyclic
// to block-cyclic redistributions), each piece moves as boxes: a
// cp.async.bulk.tensor load of the box from the source block's tensor map
// into a shared-memory stage, completing on an mbarrier, then a
// cp.async.bulk.tensor store of the stage into the destination block's
// tensor map. No thread touches the data; one elected thread per CTA keeps
// a ring of stages in flight (loads of the next boxes while the stores of
// the previous ones drain).
//
// Every wait is bounded: if a load never completes, the CTA records the
// error in the plan's status word, waits (bounded) for its other stages and
// its stores, and returns. Tensor maps cover this GPU's memory only; no
// cluster multicast is used.
#include "g2g_launch.hpp"

#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

namespace g2g {

namespace {

__device__ __forceinline__ uint32_t tma_smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void tma_mbar_init(uint32_t bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tma_mbar_expect(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool tma_mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t tma_now_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr uint64_t kBoxWaitLimitNs = 2000000000ull; // 2 s

__device__ __forceinline__ bool tma_mbar_wait(uint32_t bar, uint32_t parity, uint64_t limit) {
    if (tma_mbar_try(bar, parity))
        return true;
    const uint64_t t0 = tma_now_ns();
    for (;;) {
        if (tma_mbar_try(bar, parity))
            return true;
        if (tma_now_ns() - t0 > limit)
            return false;
    }
}

__device__ __forceinline__ void tma_load_box(uint32_t dst, const void *map, int x, int y,
                                             uint32_t bar) {
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
                 "l"(map), "r"(x), "r"(y), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tma_store_box(const void *map, int x, int y, uint32_t src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];"
                 ::"l"(map), "r"(x), "r"(y), "r"(src)
                 : "memory");
}

__device__ __forceinline__ void tma_commit() {
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// At most N store groups may still be reading shared memory.
template <int N> __device__ __forceinline__ void tma_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void tma_wait_all() {
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// S stages of box_bytes each. Box j of this CTA is work item
// blockIdx.x + j * gridDim.x. The elected thread issues the loads of boxes
// 0 .. S-1, then for each box j: wait for its load, store it, and once the
// store of box j - D has read its stage (at most D stores still reading),
// load box j - D + S into that stage. Loads thus run S - D boxes ahead and
// a store has D boxes' time to drain before its stage is needed again.
template <int S, int D>
__global__ void __launch_bounds__(32, 1)
    tma_box_kernel(const TmaBox *__restrict__ boxes, long long n,
                   const unsigned char *__restrict__ maps, int box_bytes, int *status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    // the stages, then the S mbarriers
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + (size_t)S * (size_t)box_bytes);
    if (threadIdx.x != 0)
        return;
    const long long G = gridDim.x;
    const long long first = blockIdx.x;
    if (first >= n)
        return;
    const long long mine = (n - first + G - 1) / G; // boxes of this CTA
    for (int k = 0; k < S; ++k)
        tma_mbar_init(tma_smem_addr(&bars[k]));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    const uint32_t stage0 = tma_smem_addr(smem);
    auto issue = [&](long long j) {
        const TmaBox b = boxes[first + j * G];
        const int k = (int)(j % S);
        const uint32_t bar = tma_smem_addr(&bars[k]);
        tma_mbar_expect(bar, (uint32_t)box_bytes);
        tma_load_box(stage0 + (uint32_t)(k * box_bytes), maps + (size_t)b.src_map * 128, b.sx, b.sy,
                     bar);
    };
    const long long pro = mine < S ? mine : S;
    for (long long j = 0; j < pro; ++j)
        issue(j);
    uint32_t phase = 0; // bit k: parity of stage k's next completion
    for (long long j = 0; j < mine; ++j) {
        const int k = (int)(j % S);
        const uint32_t bar = tma_smem_addr(&bars[k]);
        if (!tma_mbar_wait(bar, (phase >> k) & 1u, kBoxWaitLimitNs)) {
            atomicExch(status, 1);
            // the other stages' loads (bounded), then the stores issued
            for (long long i = j + 1; i < j + S && i < mine; ++i) {
                const int q = (int)(i % S);
                tma_mbar_wait(tma_smem_addr(&bars[q]), (phase >> q) & 1u, kBoxWaitLimitNs / 4);
            }
            tma_wait_all();
            return;
        }
        phase ^= 1u << k;
        const TmaBox b = boxes[first + j * G];
        tma_store_box(maps + (size_t)b.dst_map * 128, b.dx, b.dy,
                      stage0 + (uint32_t)(k * box_bytes));
        tma_commit();
        // the store of box j - D has read its stage: reload it with box j - D + S
        if (j >= D && j - D + S < mine) {
            tma_wait_read<D>();
            issue(j - D + S);
        }
    }
    tma_wait_all();
}

// Measured on block-cyclic redistributions (double 4096^2 and 16384^2,
// complex<double> 8192^2, float 16384^2; stages x slack 8x1, 8x2, 12x2,
// 6x1, 4x1, 2x1): 8 x 2 was best or within 2 % of the best on each.
constexpr int kBoxStages = 8;
constexpr int kBoxSlack = 2;

} // namespace

size_t tma_smem_bytes(int box_bytes) {
    return (size_t)kBoxStages * (size_t)box_bytes + 8u * (size_t)kBoxStages;
}

cudaError_t launch_tma_boxes(const TmaPlan &p, int sm_count, int *status, cudaStream_t s) {
    if (p.n_boxes <= 0)
        return cudaSuccess;
    auto k = tma_box_kernel<kBoxStages, kBoxSlack>;
    const size_t smem = tma_smem_bytes(p.box_bytes);
    int occ = 0;
    cudaError_t e = kernel_occupancy((const void *)k, 32, smem, &occ);
    if (e != cudaSuccess)
        return e;
    if (occ < 1)
        return cudaErrorInvalidConfiguration;
    long long grid = (long long)sm_count * occ;
    if (grid > p.n_boxes)
        grid = p.n_boxes;
    k<<<(unsigned)(grid < 1 ? 1 : grid), 32, smem, s>>>(p.boxes, p.n_boxes, p.maps, p.box_bytes,
                                                       status);
    return cudaGetLastError();
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library links the static CUDA runtime, not the driver library).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
cudaError_t encode_box_map(void *map, const void *base, int word_bytes, uint64_t rows_words,
                           uint64_t cols, uint64_t ld_bytes, uint32_t box_rows_words,
                           uint32_t box_cols) {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    static cudaError_t fn_err = cudaSuccess;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        fn_err = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                                  cudaEnableDefault, &q);
        if (fn_err == cudaSuccess && q != cudaDriverEntryPointSuccess)
            fn_err = cudaErrorNotSupported;
        fn = (EncodeTiledFn)p;
    });
    if (fn_err != cudaSuccess || !fn)
        return fn_err != cudaSuccess ? fn_err : cudaErrorNotSupported;
    const cuuint64_t dims[2] = {rows_words, cols};
    const cuuint64_t strides[1] = {ld_bytes};
    const cuuint32_t box[2] = {box_rows_words, box_cols};
    const cuuint32_t elem_strides[2] = {1, 1};
    const CUresult r = fn((CUtensorMap *)map,
                          word_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT32
                                          : CU_TENSOR_MAP_DATA_TYPE_UINT64,
                          2, const_cast<void *>(base), dims, strides, box, elem_strides,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

} // namespace g2g
