// The gather-scatter: one persistent kernel that replaces the reference's
// pack (communication_data.cpp:132-142), MPI exchange (transform.cpp:41-124),
// local copy (communication_data.cpp:224-252) and unpack
// (communication_data.cpp:157-173). Every tile of the work list is a
// sub-rectangle of one piece (initial block x final block); its source is read
// once and its destination written once, straight from the initial owner's
// strided block into the final owner's strided block.
//
// Four tile paths (uniform per tile, so no divergence):
//  * plain copies    non-transposed: byte movement in 16-byte chunks aligned
//                    to the DESTINATION, the chunks of a tile's columns walked
//                    as one flat sequence by the lanes of a warp. When source
//                    and destination are misaligned differently (arbitrary
//                    strides), a chunk is assembled from two aligned source
//                    blocks, funnel-shifted by whole words. Loads and stores
//                    are 128-bit; only the head and tail chunk of a column
//                    store single words (memory_utils.hpp:41-77). Two forms:
//                    the source blocks staged by cp.async in a per-warp ring
//                    in shared memory (ring kernel, default), or held in
//                    registers (copy_tile).
//  * transposed      plain, transposed (+ conjugated): a tile staged through
//                    shared memory with a padded pitch, loaded coalesced along
//                    the source's storage columns and stored coalesced along
//                    the destination's columns, the next tile's loads issued
//                    before the current one is stored (memory_utils.hpp:124-184);
//                    td x td for 16-byte elements, 2td x 2td for 4-byte,
//                    2td x td for 8-byte ones (the same bytes per tile).
//  * scaled tiles    dst = beta*dst + alpha*op(src) in the element type with
//                    the rounding of the reference's host arithmetic: every
//                    product and sum rounded separately, complex products in
//                    the C99 Annex G form that GCC's std::complex multiply uses
//                    (memory_utils.hpp:25-39,79-122,186-256). Non-transposed
//                    ones ride the copy ring with their destination chunks.
//  * cast tiles      dst = convert(op(src)) between float / double / complex
//                    types (no counterpart in the reference); non-transposed
//                    ones ride the copy ring, up to three source blocks per
//                    destination chunk.
#pragma once

#include "g2g_internal.hpp"
#include "g2g_launch.hpp"

#include <cuda_runtime.h>
#include <math.h>

#include <type_traits>

namespace g2g {

namespace {

// Tile paths a kernel instance contains; a plan launches the smallest
// instance that covers its tiles, so the plain copy does not carry the
// register cost of the scaled complex arithmetic.
enum : int {
    PATH_COPY = 1,
    PATH_TRANSPOSE = 2,
    PATH_SCALED_REAL = 4,    // scaled float / double tiles
    PATH_SCALED_COMPLEX = 8, // scaled complex tiles (more registers)
    PATH_SCALED = PATH_SCALED_REAL | PATH_SCALED_COMPLEX,
    PATH_CAST = 16,          // tiles converting the element type
    PATH_NARROW_TRANSPOSE = 32, // plain transposed tiles of 4- or 8-byte elements
                                // (the wide and tall tile shapes)
    PATH_W4_STAGED = 64, // every CTA-level tile a plain transpose of 4-byte
                         // elements, staged raw through a cp.async ring
    PATH_W8_STAGED = 128, // the same for 8-byte elements
    PATH_W16_STAGED = 256, // and for 16-byte ones (td x td tiles)
    PATH_W4S_STAGED = 1024, // every tile a scaled transposed tile of 4-byte
                            // elements: the ring stages their destination too
    PATH_W8S_STAGED = 2048  // the same for 8-byte elements
};

// ---------------------------------------------------------------- memory ops
__device__ __forceinline__ uint4 ldg_v4(uint64_t addr) {
    uint4 v;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
        : "l"(addr));
    return v;
}

__device__ __forceinline__ void cp_async16(uint32_t saddr, uint64_t gaddr) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr), "l"(gaddr)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N> __device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void st_v4(uint64_t addr, uint4 v) {
    asm volatile("st.global.v4.u32 [%0], {%1,%2,%3,%4};" ::"l"(addr), "r"(v.x), "r"(v.y),
                 "r"(v.z), "r"(v.w)
                 : "memory");
}

__device__ __forceinline__ void st_u32(uint64_t addr, uint32_t v) {
    asm volatile("st.global.u32 [%0], %1;" ::"l"(addr), "r"(v) : "memory");
}

template <typename W> __device__ __forceinline__ W ldg_w(uint64_t addr);
template <> __device__ __forceinline__ uint32_t ldg_w<uint32_t>(uint64_t a) {
    uint32_t v;
    asm("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(v) : "l"(a));
    return v;
}
template <> __device__ __forceinline__ unsigned long long ldg_w<unsigned long long>(uint64_t a) {
    unsigned long long v;
    asm("ld.global.nc.L1::no_allocate.u64 %0, [%1];" : "=l"(v) : "l"(a));
    return v;
}
template <> __device__ __forceinline__ uint4 ldg_w<uint4>(uint64_t a) { return ldg_v4(a); }
// A read-only load that allocates in L1 (a sector that the CTA's other
// warps read too is then fetched once per SM).
__device__ __forceinline__ uint32_t ldg_l1_u32(uint64_t a) {
    uint32_t v;
    asm("ld.global.nc.u32 %0, [%1];" : "=r"(v) : "l"(a));
    return v;
}


template <typename W> __device__ __forceinline__ void st_w(uint64_t addr, W v);
template <> __device__ __forceinline__ void st_w<uint32_t>(uint64_t a, uint32_t v) {
    st_u32(a, v);
}
template <> __device__ __forceinline__ void st_w<unsigned long long>(uint64_t a,
                                                                     unsigned long long v) {
    asm volatile("st.global.u64 [%0], %1;" ::"l"(a), "l"(v) : "memory");
}
template <> __device__ __forceinline__ void st_w<uint4>(uint64_t a, uint4 v) { st_v4(a, v); }

// Flip the sign bit of the highest 32-bit word of an element: the sign of the
// imaginary part of a little-endian std::complex<float|double>, i.e.
// std::conj (block.cpp:15-21), NaN payloads included.
__device__ __forceinline__ void flip_top_sign(uint32_t &w) { w ^= 0x80000000u; }
__device__ __forceinline__ void flip_top_sign(unsigned long long &w) {
    w ^= 0x8000000000000000ull;
}
__device__ __forceinline__ void flip_top_sign(uint4 &w) { w.w ^= 0x80000000u; }

// word-granular funnel: 4 words starting at word q of the 8-word window lo:hi
__device__ __forceinline__ uint4 funnel_words(uint4 lo, uint4 hi, uint32_t q) {
    uint32_t a0, a1, a2, a3, a4;
    if (q & 2u) {
        a0 = lo.z; a1 = lo.w; a2 = hi.x; a3 = hi.y; a4 = hi.z;
    } else {
        a0 = lo.x; a1 = lo.y; a2 = lo.z; a3 = lo.w; a4 = hi.x;
    }
    uint4 o;
    if (q & 1u) {
        o.x = a1; o.y = a2; o.z = a3; o.w = a4;
    } else {
        o.x = a0; o.y = a1; o.z = a2; o.w = a3;
    }
    return o;
}

// ------------------------------------------------------------ plain copy tile
// The tile's columns are cut into 16-byte chunks aligned to the DESTINATION;
// the chunks of all columns form one flat sequence (column by column) that the
// lanes walk 32 at a time, so a warp instruction covers 32 chunks whatever
// the column length (no lane idles on short columns).
//  * aligned tiles (source and destination at the same 16-byte phase in every
//    column): chunk k of a column is one 128-bit load and one 128-bit store;
//  * otherwise destination chunk k is assembled from aligned source blocks k
//    and k + 1 (funnel shift by whole words). Lane i loads block k; block
//    k + 1 is the next chunk of the sequence, loaded by the next lane (warp
//    shuffle) -- or, past lane 31, by lane 0 of the next unrolled step. Only
//    the last lane of the last step loads its next block itself. A column is
//    given as many chunks as aligned source blocks it touches, so its last
//    chunk never needs the next column's block.
// A column of a tile is at most 4 KB (tiles are cut at 4096 / sizeof(T)
// rows), so per-chunk arithmetic is 32-bit, relative to the column's first
// aligned destination chunk. Only 16-byte blocks overlapping the column are
// read, so no access leaves the pages the column lives in; stores cover
// exactly the column (word-masked head and tail chunks).
// NWARP warps share a tile in runs of 32 * U consecutive chunks.
template <int NWARP, int U>
__device__ __forceinline__ void copy_tile(const Tile &t, const int warp) {
    const int lane = threadIdx.x & 31;
    const int esz = kind_esz(t.kind);
    const int L = t.rows * esz; // bytes per column, <= 4096
    if (L <= 0 || t.cols <= 0)
        return;
    const bool aligned = (((t.src - t.dst) | (uint64_t)(t.src_ld - t.dst_ld)) & 15u) == 0;
    // chunks per column: the aligned source blocks a column touches from the
    // block under its first destination chunk (exact when every column has
    // the same 16-byte phases, else the bound over all phases: element
    // addresses are 4-byte aligned, so the source lead is at most 24 bytes)
    int cpc;
    if (((t.dst_ld | t.src_ld) & 15) == 0) {
        const int d0 = (int)(t.dst & 15u);
        const int sh = (int)((t.src - (uint64_t)d0) & 15u);
        cpc = (sh + d0 + L + 15) >> 4;
    } else {
        cpc = aligned ? ((L + 27) >> 4) : ((L + 39) >> 4);
    }
    const int total = t.cols * cpc;
    // flat chunk index of this lane: run r = i * NWARP + warp, idx = r * 32U + u * 32 + lane
    int col, k;
    {
        const int idx = warp * 32 * U + lane;
        col = idx / cpc;
        k = idx - col * cpc;
    }
    const int dq = 32 / cpc, dr = 32 - dq * cpc;                 // +32 chunks
    const int skip = (NWARP - 1) * 32 * U;                       // to this warp's next run
    const int sq = skip / cpc, sr = skip - sq * cpc;
    for (int base = warp * 32 * U; base < total; base += NWARP * 32 * U) { // warp-uniform
        uint4 lo[U];
        uint4 ex;
        uint64_t chunk[U];
        uint32_t qm[U]; // bits 0-3 store mask, bits 4-5 word shift
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const bool colok = col < t.cols;
            const uint64_t d = t.dst + (uint64_t)((long long)col * t.dst_ld);
            const uint64_t s = t.src + (uint64_t)((long long)col * t.src_ld);
            const int d0 = (int)(d & 15u);        // destination phase
            const uint64_t sa = s - (uint64_t)d0; // source byte of chunk 0's first byte
            const int sh = (int)(sa & 15u);       // source phase vs. destination
            const int rel = k << 4;
            const int lo_lim = sh + d0, hi_lim = sh + d0 + L;
            const bool need = colok && rel < hi_lim && rel + 16 > lo_lim;
            lo[u] = need ? ldg_v4(sa - (uint64_t)sh + (uint64_t)rel)
                         : make_uint4(0u, 0u, 0u, 0u);
            if (u == U - 1 && !aligned) { // the last lane's next block, from no lane
                const bool nx = colok && lane == 31 && sh != 0 && rel + 16 < hi_lim;
                ex = nx ? ldg_v4(sa - (uint64_t)sh + (uint64_t)(rel + 16))
                        : make_uint4(0u, 0u, 0u, 0u);
            }
            // words of this chunk inside the destination column [d0, d0 + L)
            int wlo = (d0 - rel) >> 2, whi = (d0 + L - rel) >> 2;
            wlo = wlo < 0 ? 0 : (wlo > 4 ? 4 : wlo);
            whi = whi < 0 ? 0 : (whi > 4 ? 4 : whi);
            uint32_t m = ((1u << whi) - 1u) & ~((1u << wlo) - 1u);
            m = colok ? m : 0u;
            chunk[u] = d - (uint64_t)d0 + (uint64_t)rel;
            qm[u] = m | ((uint32_t)(sh >> 2) << 4);
            col += dq;
            k += dr;
            if (k >= cpc) {
                k -= cpc;
                ++col;
            }
        }
        if (NWARP > 1) {
            col += sq;
            k += sr;
            if (k >= cpc) {
                k -= cpc;
                ++col;
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            uint4 o = lo[u];
            if (!aligned) { // tile-uniform
                // lane i takes the block of chunk idx + 1: lane i + 1's, or for
                // lane 31 lane 0's of the next step (its own extra load last)
                uint4 v = lo[u];
                if (u + 1 < U && lane == 0)
                    v = lo[u + 1];
                const int srcl = (lane + 1) & 31;
                uint4 nb;
                nb.x = __shfl_sync(0xffffffffu, v.x, srcl);
                nb.y = __shfl_sync(0xffffffffu, v.y, srcl);
                nb.z = __shfl_sync(0xffffffffu, v.z, srcl);
                nb.w = __shfl_sync(0xffffffffu, v.w, srcl);
                if (u == U - 1 && lane == 31)
                    nb = ex;
                const uint32_t q = (qm[u] >> 4) & 3u;
                if (q)
                    o = funnel_words(lo[u], nb, q);
            }
            const uint32_t m = qm[u] & 15u;
            if (m == 0xFu) {
                st_v4(chunk[u], o);
            } else if (m) {
                if (m & 1u) st_u32(chunk[u], o.x);
                if (m & 2u) st_u32(chunk[u] + 4, o.y);
                if (m & 4u) st_u32(chunk[u] + 8, o.z);
                if (m & 8u) st_u32(chunk[u] + 12, o.w);
            }
        }
    }
}

// Copy tile `ti` (warp-level items) / CTA-level tile `ti` of the plans of a
// launch, and the pair table of its plan.
__device__ __forceinline__ int plan_of(const PlanList &L, long long ti, bool copy) {
    int lo = 0, hi = L.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((copy ? L.p[mid].first_copy : L.p[mid].first_cta) <= ti)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ const Tile *locate_copy(const PlanList &L, long long ti,
                                                   const PairInfo *&pairs) {
    const int k = plan_of(L, ti, true);
    pairs = L.p[k].pairs;
    return L.p[k].tiles + (ti - L.p[k].first_copy);
}
__device__ __forceinline__ const Tile *locate_cta(const PlanList &L, long long ti,
                                                  const PairInfo *&pairs) {
    const int k = plan_of(L, ti, false);
    pairs = L.p[k].pairs;
    return L.p[k].tiles + L.p[k].n_copy + (ti - L.p[k].first_cta);
}

// ------------------------------------------------------------ TMA staging
// The staged kernel keeps several tiles in flight per CTA without holding
// their data in registers: one lane per column issues a 1-D TMA bulk copy
// (cp.async.bulk) of the column's 16-byte aligned cover into a ring of
// shared-memory stages; an mbarrier per stage counts the bytes landed. The
// CTA then shifts each destination chunk out of shared memory and stores it
// with 128-bit stores.
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t global_timer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Waits for a stage, giving up after `limit_ns` (returns false then).
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity,
                                                  uint64_t limit_ns) {
    if (mbar_try_wait(bar, parity))
        return true;
    const uint64_t t0 = global_timer_ns();
    for (uint32_t i = 0; i < (1u << 30); ++i) {
        if (mbar_try_wait(bar, parity))
            return true;
        if (global_timer_ns() - t0 > limit_ns)
            return false;
    }
    return false;
}
__device__ __forceinline__ void bulk_load(uint32_t dst, uint64_t src, uint32_t bytes,
                                          uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
                 "[%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ uint4 lds_v4(uint32_t a) {
    uint4 v;
    asm volatile("ld.shared.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "r"(a));
    return v;
}
__device__ __forceinline__ uint2 lds_v2(uint32_t a) {
    uint2 v;
    asm volatile("ld.shared.v2.u32 {%0,%1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(a));
    return v;
}
__device__ __forceinline__ uint32_t lds_u32(uint32_t a) {
    uint32_t v;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(a));
    return v;
}

// Bytes one staged column takes: its 16-byte aligned cover, at most
// round_up(L, 16) + 16.
__device__ __forceinline__ int staged_pitch(int L) { return ((L + 15) & ~15) + 16; }

// Plain tiles whose columns are long enough for bulk copies to pay off and
// whose columns fit one stage.
__device__ __forceinline__ bool tma_eligible(const Tile &t, int stage_bytes) {
    if (t.kind & (KIND_TRANS | KIND_SCALED | KIND_CAST))
        return false;
    const int L = t.rows * kind_esz(t.kind);
    return L >= 256 && (long long)t.cols * staged_pitch(L) <= (long long)stage_bytes;
}

// Warp 0: start the bulk copies of tile `ti` into `stage` (nothing when the
// tile is past the end or not eligible).
__device__ __forceinline__ void issue_stage(const PlanList &list, long long ti, long long n,
                                            unsigned char *stage, uint32_t bar,
                                            int stage_bytes) {
    if (ti >= n)
        return;
    const int lane = threadIdx.x & 31;
    const PairInfo *unused;
    const Tile t = *locate_copy(list, ti, unused);
    if (!tma_eligible(t, stage_bytes))
        return;
    const int L = t.rows * kind_esz(t.kind);
    const int pitch = staged_pitch(L);
    uint32_t total = 0;
    for (int c = lane; c < t.cols; c += 32) {
        const uint64_t s = t.src + (uint64_t)((long long)c * t.src_ld);
        total += (uint32_t)(((s + (uint64_t)L + 15u) & ~15ull) - (s & ~15ull));
    }
    for (int off = 16; off > 0; off >>= 1)
        total += __shfl_xor_sync(0xffffffffu, total, off);
    if (lane == 0) {
        // order earlier generic-proxy reads of this stage before the async writes
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(bar, total);
    }
    __syncwarp();
    const uint32_t sbase = smem_addr(stage);
    for (int c = lane; c < t.cols; c += 32) {
        const uint64_t s = t.src + (uint64_t)((long long)c * t.src_ld);
        const uint64_t a0 = s & ~15ull;
        const uint32_t len = (uint32_t)(((s + (uint64_t)L + 15u) & ~15ull) - a0);
        bulk_load(sbase + (uint32_t)(c * pitch), a0, len, bar);
    }
}

// All threads: write tile t from its staged columns. Column c's cover starts
// at stage + c * pitch and holds source byte x at offset x - (s & ~15); the
// destination chunk at d - d0 + rel reads its words at
// c * pitch + (s & 15) - d0 + rel. Only words of the destination column are
// read and written.
template <int THREADS, int U>
__device__ __forceinline__ void consume_stage(const Tile &t, const unsigned char *stage) {
    constexpr int NWARP = THREADS / 32;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int L = t.rows * kind_esz(t.kind);
    const int pitch = staged_pitch(L);
    const int cpc = ((t.dst_ld & 15) == 0) ? (((int)(t.dst & 15u) + L + 15) >> 4)
                                           : ((L + 27) >> 4);
    int lpc_shift = 0;
    while (lpc_shift < 5 && (1 << lpc_shift) < cpc)
        ++lpc_shift;
    const int lpc = 1 << lpc_shift;
    const int cpw = 32 >> lpc_shift;
    const int sub = lane >> lpc_shift;
    const int kl = lane & (lpc - 1);
    const int col_step = NWARP * cpw;
    const int warp_col0 = warp * cpw;
    const int ncolit =
        t.cols > warp_col0 ? (t.cols - warp_col0 + col_step - 1) / col_step : 0;
    const int nkit = (cpc + lpc - 1) >> lpc_shift;
    const int my_col0 = warp_col0 + sub;
    const uint32_t sbase = smem_addr(stage);

    int colit = 0, kit = 0;
    while (colit < ncolit) {
        uint4 v[U];
        uint64_t chunk[U];
        uint32_t wm[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int c = my_col0 + colit * col_step;
            const bool colok = (colit < ncolit) && (c < t.cols);
            const uint64_t d = t.dst + (uint64_t)((long long)c * t.dst_ld);
            const uint64_t s = t.src + (uint64_t)((long long)c * t.src_ld);
            const int d0 = (int)(d & 15u);
            const int off0 = (int)(s & 15u) - d0;
            const int rel = (kl + (kit << lpc_shift)) << 4;
            int wlo = (d0 - rel) >> 2, whi = (d0 + L - rel) >> 2;
            wlo = wlo < 0 ? 0 : (wlo > 4 ? 4 : wlo);
            whi = whi < 0 ? 0 : (whi > 4 ? 4 : whi);
            uint32_t m = ((1u << whi) - 1u) & ~((1u << wlo) - 1u);
            m = colok ? m : 0u;
            const uint32_t sp = sbase + (uint32_t)(c * pitch + off0 + rel);
            uint4 x = make_uint4(0u, 0u, 0u, 0u);
            if (m == 0xFu) {
                if ((off0 & 15) == 0) {
                    x = lds_v4(sp);
                } else if ((off0 & 7) == 0) {
                    const uint2 a = lds_v2(sp), b = lds_v2(sp + 8);
                    x = make_uint4(a.x, a.y, b.x, b.y);
                } else {
                    x = make_uint4(lds_u32(sp), lds_u32(sp + 4), lds_u32(sp + 8),
                                   lds_u32(sp + 12));
                }
            } else if (m) {
                if (m & 1u) x.x = lds_u32(sp);
                if (m & 2u) x.y = lds_u32(sp + 4);
                if (m & 4u) x.z = lds_u32(sp + 8);
                if (m & 8u) x.w = lds_u32(sp + 12);
            }
            v[u] = x;
            chunk[u] = d - (uint64_t)d0 + (uint64_t)rel;
            wm[u] = m;
            if (++kit == nkit) {
                kit = 0;
                ++colit;
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t m = wm[u];
            const uint4 o = v[u];
            if (m == 0xFu) {
                st_v4(chunk[u], o);
            } else if (m) {
                if (m & 1u) st_u32(chunk[u], o.x);
                if (m & 2u) st_u32(chunk[u] + 4, o.y);
                if (m & 4u) st_u32(chunk[u] + 8, o.z);
                if (m & 8u) st_u32(chunk[u] + 12, o.w);
            }
        }
    }
}

// --------------------------------------------------------------- scaled tiles
struct cplxf {
    float x, y;
};
struct cplxd {
    double x, y;
};

template <typename T> __device__ __forceinline__ T ld_elem(uint64_t a);
template <> __device__ __forceinline__ float ld_elem<float>(uint64_t a) {
    return *reinterpret_cast<const float *>(a);
}
template <> __device__ __forceinline__ double ld_elem<double>(uint64_t a) {
    return *reinterpret_cast<const double *>(a);
}
template <> __device__ __forceinline__ cplxf ld_elem<cplxf>(uint64_t a) {
    const float *p = reinterpret_cast<const float *>(a);
    return cplxf{p[0], p[1]};
}
template <> __device__ __forceinline__ cplxd ld_elem<cplxd>(uint64_t a) {
    const double *p = reinterpret_cast<const double *>(a);
    return cplxd{p[0], p[1]};
}
template <typename T> __device__ __forceinline__ void st_elem(uint64_t a, T v);
template <> __device__ __forceinline__ void st_elem<float>(uint64_t a, float v) {
    *reinterpret_cast<float *>(a) = v;
}
template <> __device__ __forceinline__ void st_elem<double>(uint64_t a, double v) {
    *reinterpret_cast<double *>(a) = v;
}
template <> __device__ __forceinline__ void st_elem<cplxf>(uint64_t a, cplxf v) {
    float *p = reinterpret_cast<float *>(a);
    p[0] = v.x;
    p[1] = v.y;
}
template <> __device__ __forceinline__ void st_elem<cplxd>(uint64_t a, cplxd v) {
    double *p = reinterpret_cast<double *>(a);
    p[0] = v.x;
    p[1] = v.y;
}

__device__ __forceinline__ float conj_elem(float v) { return v; }
__device__ __forceinline__ double conj_elem(double v) { return v; }
__device__ __forceinline__ cplxf conj_elem(cplxf v) {
    v.y = __int_as_float(__float_as_int(v.y) ^ 0x80000000);
    return v;
}
__device__ __forceinline__ cplxd conj_elem(cplxd v) {
    v.y = __longlong_as_double(__double_as_longlong(v.y) ^ (long long)0x8000000000000000ull);
    return v;
}

// Rounded-separately arithmetic (no contraction into FMA).
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }

// Complex product as GCC computes std::complex<R> * std::complex<R>: the
// textbook formula with each operation rounded, and when both parts come out
// NaN the recovery of C99 Annex G (G.5.1, multiplicative operators): boxed
// infinities, NaN operands set to signed zeros, recomputation scaled by inf.
template <typename R>
__device__ __noinline__ void cmul_nan(R a, R b, R c, R d, R ac, R bd, R ad, R bc, R *xo,
                                      R *yo) {
    bool recalc = false;
    const R one = R(1), zero = R(0);
    if (isinf(a) || isinf(b)) {
        a = copysign(isinf(a) ? one : zero, a);
        b = copysign(isinf(b) ? one : zero, b);
        if (isnan(c)) c = copysign(zero, c);
        if (isnan(d)) d = copysign(zero, d);
        recalc = true;
    }
    if (isinf(c) || isinf(d)) {
        c = copysign(isinf(c) ? one : zero, c);
        d = copysign(isinf(d) ? one : zero, d);
        if (isnan(a)) a = copysign(zero, a);
        if (isnan(b)) b = copysign(zero, b);
        recalc = true;
    }
    if (!recalc && (isinf(ac) || isinf(bd) || isinf(ad) || isinf(bc))) {
        if (isnan(a)) a = copysign(zero, a);
        if (isnan(b)) b = copysign(zero, b);
        if (isnan(c)) c = copysign(zero, c);
        if (isnan(d)) d = copysign(zero, d);
        recalc = true;
    }
    if (recalc) {
        const R inf = R(INFINITY);
        *xo = rmul(inf, rsub(rmul(a, c), rmul(b, d)));
        *yo = rmul(inf, radd(rmul(a, d), rmul(b, c)));
    }
}

// NaN tests on the bit patterns (integer pipe: the FP64 pipe of this GPU is
// narrow and the complex<double> products already load it).
__device__ __forceinline__ bool nan_bits(float v) {
    return (__float_as_uint(v) & 0x7fffffffu) > 0x7f800000u;
}
__device__ __forceinline__ bool nan_bits(double v) {
    return ((unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull) >
           0x7ff0000000000000ull;
}

// (the recovery, rare, is a separate function so that the common path keeps
// few registers)
template <typename R>
__device__ __forceinline__ void cmul(R a, R b, R c, R d, R &x, R &y) {
    const R ac = rmul(a, c), bd = rmul(b, d), ad = rmul(a, d), bc = rmul(b, c);
    x = rsub(ac, bd);
    y = radd(ad, bc);
    if (nan_bits(x) && nan_bits(y))
        cmul_nan(a, b, c, d, ac, bd, ad, bc, &x, &y);
}

// Arithmetic with an operand known to be a zero, on the integer pipe. Every
// result that is not a NaN is the IEEE-754 result bit for bit (signed zeros
// included); NaN results are NaNs (their payload is left to the
// implementation, as for the FP pipe's own operations). Selects, no
// branches: the operands differ from lane to lane.
template <typename R> struct FBits;
template <> struct FBits<double> {
    using U = unsigned long long;
    static constexpr U SIGN = 0x8000000000000000ull, ABS = 0x7fffffffffffffffull,
                       INF = 0x7ff0000000000000ull;
    static __device__ __forceinline__ U get(double v) {
        return (unsigned long long)__double_as_longlong(v);
    }
    static __device__ __forceinline__ double put(U b) { return __longlong_as_double((long long)b); }
};
// z * d for a zero z whose sign bit is zs: a NaN when d is infinite or a NaN,
// else a zero with the sign zs ^ sign(d)
template <typename R>
__device__ __forceinline__ R zmul(typename FBits<R>::U zs, R d) {
    using F = FBits<R>;
    const typename F::U b = F::get(d);
    return F::put((b & F::ABS) >= F::INF ? F::ABS /* a quiet NaN */ : ((b & F::SIGN) ^ zs));
}
// x + z for z a zero or a NaN: a NaN z gives a NaN, a non-zero x itself, and
// two zeros -0 only when both are -0 (round to nearest)
template <typename R> __device__ __forceinline__ R addz(R x, R z) {
    using F = FBits<R>;
    const typename F::U bx = F::get(x), bz = F::get(z);
    const typename F::U r = (bx & F::ABS) != 0 ? bx : (bx & bz & F::SIGN);
    return F::put((bz & F::ABS) > F::INF ? bz : r);
}
template <typename R> __device__ __forceinline__ R subz(R x, R z) {
    using F = FBits<R>;
    return addz(x, F::put(F::get(z) ^ F::SIGN));
}

// (a + b i) * (c + d i) for b a zero (sign bit bs): the two products with b
// are formed by zmul, the sums with them by addz / subz -- two rounded
// multiplications instead of four multiplications and two additions, the
// same result as cmul (the Annex G recovery sees the same values).
template <typename R>
__device__ __forceinline__ void cmul_rz(R a, typename FBits<R>::U bs, R c, R d, R &x, R &y) {
    const R ac = rmul(a, c), ad = rmul(a, d);
    const R bd = zmul<R>(bs, d), bc = zmul<R>(bs, c);
    x = subz(ac, bd);
    y = addz(ad, bc);
    if (nan_bits(x) && nan_bits(y))
        cmul_nan(a, FBits<R>::put(bs), c, d, ac, bd, ad, bc, &x, &y);
}
// (a + b i) * (c + d i) for a and b both zeros (sign bits as, bs): no
// rounded operation; the parts are zeros or NaNs (the recovery, reached
// only for an infinite c or d, multiplies an infinity by a zero)
template <typename R>
__device__ __forceinline__ void cmul_zz(typename FBits<R>::U as, typename FBits<R>::U bs, R c,
                                        R d, R &x, R &y) {
    const R ac = zmul<R>(as, c), ad = zmul<R>(as, d);
    const R bd = zmul<R>(bs, d), bc = zmul<R>(bs, c);
    x = subz(ac, bd);
    y = addz(ad, bc);
    if (nan_bits(x) && nan_bits(y))
        cmul_nan(FBits<R>::put(as), FBits<R>::put(bs), c, d, ac, bd, ad, bc, &x, &y);
}

// The pair's alpha and beta in the element type, and what is known about
// them: a real alpha or beta (imaginary part a zero) and a zero beta let
// complex<double> skip rounded operations whose results are fixed by a zero
// operand. GB300's FP64 pipe is narrow, and the scaled complex<double> tiles
// are bound by it.
enum : uint32_t { COEF_ALPHA_REAL = 1u, COEF_BETA_REAL = 2u, COEF_BETA_ZERO = 4u };
template <typename T> struct Coef {
    T alpha, beta;
    uint32_t zf;
};

// beta*d + alpha*v, as memory_utils.hpp:36 / :111 / :236 evaluate it.
__device__ __forceinline__ float axpby(float alpha, float v, float beta, float d) {
    return radd(rmul(beta, d), rmul(alpha, v));
}
__device__ __forceinline__ double axpby(double alpha, double v, double beta, double d) {
    return radd(rmul(beta, d), rmul(alpha, v));
}
__device__ __forceinline__ cplxf axpby(cplxf alpha, cplxf v, cplxf beta, cplxf d) {
    float bx, by, ax, ay;
    cmul(beta.x, beta.y, d.x, d.y, bx, by);
    cmul(alpha.x, alpha.y, v.x, v.y, ax, ay);
    return cplxf{radd(bx, ax), radd(by, ay)};
}
__device__ __forceinline__ cplxd axpby(cplxd alpha, cplxd v, cplxd beta, cplxd d) {
    double bx, by, ax, ay;
    cmul(beta.x, beta.y, d.x, d.y, bx, by);
    cmul(alpha.x, alpha.y, v.x, v.y, ax, ay);
    return cplxd{radd(bx, ax), radd(by, ay)};
}

template <typename T> __device__ __forceinline__ T scalar_from(const double *v);
template <> __device__ __forceinline__ float scalar_from<float>(const double *v) {
    return (float)v[0];
}
template <> __device__ __forceinline__ double scalar_from<double>(const double *v) {
    return v[0];
}
template <> __device__ __forceinline__ cplxf scalar_from<cplxf>(const double *v) {
    return cplxf{(float)v[0], (float)v[1]};
}
template <> __device__ __forceinline__ cplxd scalar_from<cplxd>(const double *v) {
    return cplxd{v[0], v[1]};
}

__device__ __forceinline__ bool is_zero_bits(double v) {
    return (FBits<double>::get(v) & FBits<double>::ABS) == 0;
}
template <typename T> __device__ __forceinline__ Coef<T> coef_from(const PairInfo &p) {
    Coef<T> k;
    k.alpha = scalar_from<T>(p.alpha);
    k.beta = scalar_from<T>(p.beta);
    k.zf = 0;
    return k;
}
template <> __device__ __forceinline__ Coef<cplxd> coef_from<cplxd>(const PairInfo &p) {
    Coef<cplxd> k;
    k.alpha = cplxd{p.alpha[0], p.alpha[1]};
    k.beta = cplxd{p.beta[0], p.beta[1]};
    k.zf = (is_zero_bits(k.alpha.y) ? COEF_ALPHA_REAL : 0u) |
           (is_zero_bits(k.beta.y) ? COEF_BETA_REAL : 0u) |
           (is_zero_bits(k.beta.x) && is_zero_bits(k.beta.y) ? COEF_BETA_ZERO : 0u);
    return k;
}

// Which form of beta*d + alpha*v a tile runs (uniform per tile, a template
// argument of the tile loops so that they stay free of branches): 0 the
// general one, 1 complex<double> with real alpha and beta, 2 complex<double>
// with a real alpha and a zero beta. Only complex<double> takes the special
// forms: the scaled double tiles share their kernel instances with the float
// ones, whose register allocation an extra form raises (measured: float 'T'
// with alpha/beta 12 % slower) for a saving of two operations that only
// pays with a zero beta.
template <typename T> __device__ __forceinline__ int coef_mode(const Coef<T> &) { return 0; }
template <> __device__ __forceinline__ int coef_mode<cplxd>(const Coef<cplxd> &k) {
    const uint32_t real2 = COEF_ALPHA_REAL | COEF_BETA_REAL;
    if ((k.zf & real2) != real2)
        return 0;
    return (k.zf & COEF_BETA_ZERO) ? 2 : 1;
}
template <typename T> struct CoefModes { static constexpr bool special = false; };
template <> struct CoefModes<cplxd> { static constexpr bool special = true; };
// Calls f(std::integral_constant<int, CM>) with the tile's form.
template <typename T, typename F>
__device__ __forceinline__ void coef_dispatch(const Coef<T> &k, F &&f) {
    if constexpr (CoefModes<T>::special) {
        const int m = coef_mode<T>(k);
        if (m == 2) {
            f(std::integral_constant<int, 2>());
            return;
        }
        if (m == 1) {
            f(std::integral_constant<int, 1>());
            return;
        }
    }
    f(std::integral_constant<int, 0>());
}

template <typename T, int CM> struct AxpbyM {
    static __device__ __forceinline__ T run(const Coef<T> &k, T v, T d) {
        return axpby(k.alpha, v, k.beta, d);
    }
};
// complex<double>, real alpha and beta: 6 rounded operations instead of 14
template <> struct AxpbyM<cplxd, 1> {
    static __device__ __forceinline__ cplxd run(const Coef<cplxd> &k, cplxd v, cplxd d) {
        using F = FBits<double>;
        double bx, by, ax, ay;
        cmul_rz<double>(k.beta.x, F::get(k.beta.y), d.x, d.y, bx, by);
        cmul_rz<double>(k.alpha.x, F::get(k.alpha.y), v.x, v.y, ax, ay);
        return cplxd{radd(bx, ax), radd(by, ay)};
    }
};
// complex<double>, real alpha and zero beta: 2 rounded operations
template <> struct AxpbyM<cplxd, 2> {
    static __device__ __forceinline__ cplxd run(const Coef<cplxd> &k, cplxd v, cplxd d) {
        using F = FBits<double>;
        double bx, by, ax, ay;
        cmul_zz<double>(F::get(k.beta.x), F::get(k.beta.y), d.x, d.y, bx, by);
        cmul_rz<double>(k.alpha.x, F::get(k.alpha.y), v.x, v.y, ax, ay);
        return cplxd{addz(ax, bx), addz(ay, by)};
    }
};
template <int CM, typename T>
__device__ __forceinline__ T axpby_m(const Coef<T> &k, T v, T d) {
    return AxpbyM<T, CM>::run(k, v, d);
}

// beta*d + alpha*v on the whole elements of a 16-byte chunk.
template <int CM>
__device__ __forceinline__ uint4 axpby_chunk_t(const Coef<float> &k, uint4 v, uint4 d, float *) {
    const float alpha = k.alpha, beta = k.beta;
    return make_uint4(
        __float_as_uint(axpby(alpha, __uint_as_float(v.x), beta, __uint_as_float(d.x))),
        __float_as_uint(axpby(alpha, __uint_as_float(v.y), beta, __uint_as_float(d.y))),
        __float_as_uint(axpby(alpha, __uint_as_float(v.z), beta, __uint_as_float(d.z))),
        __float_as_uint(axpby(alpha, __uint_as_float(v.w), beta, __uint_as_float(d.w))));
}
__device__ __forceinline__ double dbl(uint32_t lo, uint32_t hi) {
    return __hiloint2double((int)hi, (int)lo);
}
__device__ __forceinline__ void dbl_words(double x, uint32_t &lo, uint32_t &hi) {
    lo = (uint32_t)__double2loint(x);
    hi = (uint32_t)__double2hiint(x);
}
template <int CM>
__device__ __forceinline__ uint4 axpby_chunk_t(const Coef<double> &k, uint4 v, uint4 d, double *) {
    const double alpha = k.alpha, beta = k.beta;
    uint4 o;
    dbl_words(axpby(alpha, dbl(v.x, v.y), beta, dbl(d.x, d.y)), o.x, o.y);
    dbl_words(axpby(alpha, dbl(v.z, v.w), beta, dbl(d.z, d.w)), o.z, o.w);
    return o;
}
template <int CM>
__device__ __forceinline__ uint4 axpby_chunk_t(const Coef<cplxf> &k, uint4 v, uint4 d, cplxf *) {
    const cplxf alpha = k.alpha, beta = k.beta;
    const cplxf a = axpby(alpha, cplxf{__uint_as_float(v.x), __uint_as_float(v.y)}, beta,
                          cplxf{__uint_as_float(d.x), __uint_as_float(d.y)});
    const cplxf b = axpby(alpha, cplxf{__uint_as_float(v.z), __uint_as_float(v.w)}, beta,
                          cplxf{__uint_as_float(d.z), __uint_as_float(d.w)});
    return make_uint4(__float_as_uint(a.x), __float_as_uint(a.y), __float_as_uint(b.x),
                      __float_as_uint(b.y));
}
template <int CM>
__device__ __forceinline__ uint4 axpby_chunk_t(const Coef<cplxd> &k, uint4 v, uint4 d, cplxd *) {
    const cplxd a = axpby_m<CM>(k, cplxd{dbl(v.x, v.y), dbl(v.z, v.w)},
                                cplxd{dbl(d.x, d.y), dbl(d.z, d.w)});
    uint4 o;
    dbl_words(a.x, o.x, o.y);
    dbl_words(a.y, o.z, o.w);
    return o;
}
template <int CM, typename T>
__device__ __forceinline__ uint4 axpby_chunk(const Coef<T> &k, uint4 v, uint4 d) {
    return axpby_chunk_t<CM>(k, v, d, (T *)nullptr);
}

// A destination read that stays coherent with this kernel's own writes.
__device__ __forceinline__ uint4 ld_dst_v4(uint64_t addr) {
    uint4 v;
    asm volatile("ld.global.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(addr));
    return v;
}

// Scaled non-transposed tile, CTA-wide: copy_tile's chunk walk (NWARP warps
// in runs of 32 x U chunks) with the destination chunk read as well and
// beta*d + alpha*s computed on its elements. Needs every element of the
// destination to sit inside one 16-byte chunk (its address a multiple of
// min(sizeof(T), 16)), which scaled_tile checks.
template <int NWARP, int U, typename T, int CM>
__device__ __forceinline__ void scaled_copy_tile_m(const Tile &t, const int warp,
                                                   const Coef<T> &cf) {
    const int lane = threadIdx.x & 31;
    const int L = t.rows * (int)sizeof(T);
    if (L <= 0 || t.cols <= 0)
        return;
    const bool aligned = (((t.src - t.dst) | (uint64_t)(t.src_ld - t.dst_ld)) & 15u) == 0;
    int cpc;
    if (((t.dst_ld | t.src_ld) & 15) == 0) {
        const int d0 = (int)(t.dst & 15u);
        const int sh = (int)((t.src - (uint64_t)d0) & 15u);
        cpc = (sh + d0 + L + 15) >> 4;
    } else {
        cpc = aligned ? ((L + 27) >> 4) : ((L + 39) >> 4);
    }
    const int total = t.cols * cpc;
    int col, k;
    {
        const int idx = warp * 32 * U + lane;
        col = idx / cpc;
        k = idx - col * cpc;
    }
    const int dq = 32 / cpc, dr = 32 - dq * cpc;
    const int skip = (NWARP - 1) * 32 * U;
    const int sq = skip / cpc, sr = skip - sq * cpc;
    for (int base = warp * 32 * U; base < total; base += NWARP * 32 * U) { // warp-uniform
        uint4 lo[U], dd[U];
        uint4 ex;
        uint64_t chunk[U];
        uint32_t qm[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const bool colok = col < t.cols;
            const uint64_t d = t.dst + (uint64_t)((long long)col * t.dst_ld);
            const uint64_t s = t.src + (uint64_t)((long long)col * t.src_ld);
            const int d0 = (int)(d & 15u);
            const uint64_t sa = s - (uint64_t)d0;
            const int sh = (int)(sa & 15u);
            const int rel = k << 4;
            const int lo_lim = sh + d0, hi_lim = sh + d0 + L;
            const bool need = colok && rel < hi_lim && rel + 16 > lo_lim;
            lo[u] = need ? ldg_v4(sa - (uint64_t)sh + (uint64_t)rel)
                         : make_uint4(0u, 0u, 0u, 0u);
            if (u == U - 1 && !aligned) {
                const bool nx = colok && lane == 31 && sh != 0 && rel + 16 < hi_lim;
                ex = nx ? ldg_v4(sa - (uint64_t)sh + (uint64_t)(rel + 16))
                        : make_uint4(0u, 0u, 0u, 0u);
            }
            int wlo = (d0 - rel) >> 2, whi = (d0 + L - rel) >> 2;
            wlo = wlo < 0 ? 0 : (wlo > 4 ? 4 : wlo);
            whi = whi < 0 ? 0 : (whi > 4 ? 4 : whi);
            uint32_t m = ((1u << whi) - 1u) & ~((1u << wlo) - 1u);
            m = colok ? m : 0u;
            chunk[u] = d - (uint64_t)d0 + (uint64_t)rel;
            dd[u] = m ? ld_dst_v4(chunk[u]) : make_uint4(0u, 0u, 0u, 0u);
            qm[u] = m | ((uint32_t)(sh >> 2) << 4);
            col += dq;
            k += dr;
            if (k >= cpc) {
                k -= cpc;
                ++col;
            }
        }
        if (NWARP > 1) {
            col += sq;
            k += sr;
            if (k >= cpc) {
                k -= cpc;
                ++col;
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            uint4 o = lo[u];
            if (!aligned) { // tile-uniform
                uint4 v = lo[u];
                if (u + 1 < U && lane == 0)
                    v = lo[u + 1];
                const int srcl = (lane + 1) & 31;
                uint4 nb;
                nb.x = __shfl_sync(0xffffffffu, v.x, srcl);
                nb.y = __shfl_sync(0xffffffffu, v.y, srcl);
                nb.z = __shfl_sync(0xffffffffu, v.z, srcl);
                nb.w = __shfl_sync(0xffffffffu, v.w, srcl);
                if (u == U - 1 && lane == 31)
                    nb = ex;
                const uint32_t q = (qm[u] >> 4) & 3u;
                if (q)
                    o = funnel_words(lo[u], nb, q);
            }
            const uint32_t m = qm[u] & 15u;
            if (m) {
                o = axpby_chunk<CM>(cf, o, dd[u]);
                if (m == 0xFu) {
                    st_v4(chunk[u], o);
                } else {
                    if (m & 1u) st_u32(chunk[u], o.x);
                    if (m & 2u) st_u32(chunk[u] + 4, o.y);
                    if (m & 4u) st_u32(chunk[u] + 8, o.z);
                    if (m & 8u) st_u32(chunk[u] + 12, o.w);
                }
            }
        }
    }
}

template <int NWARP, int U, typename T>
__device__ __forceinline__ void scaled_copy_tile(const Tile &t, const int warp, const Coef<T> &cf) {
    coef_dispatch(cf, [&](auto cm) {
        scaled_copy_tile_m<NWARP, U, T, decltype(cm)::value>(t, warp, cf);
    });
}

template <int THREADS, typename T>
__device__ __forceinline__ void scaled_tile(const Tile &t, const PairInfo *pairs,
                                            unsigned char *smem_raw, int td) {
    constexpr int NWARP = THREADS / 32;
    constexpr int E = (int)sizeof(T);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const Coef<T> k = coef_from<T>(pairs[t.pair]);
    const T alpha = k.alpha, beta = k.beta;
    const int R = t.rows, C = t.cols;
    if ((t.dst & (uint64_t)((E < 16 ? E : 16) - 1)) == 0) { // whole elements per chunk
        scaled_copy_tile<NWARP, 2, T>(t, warp, k);
        return;
    }
    for (int c = warp; c < C; c += NWARP) {
        const uint64_t sc = t.src + (uint64_t)((long long)c * t.src_ld);
        const uint64_t dc = t.dst + (uint64_t)((long long)c * t.dst_ld);
        for (int r = lane; r < R; r += 32) {
            const T v = ld_elem<T>(sc + (uint64_t)r * E);
            const T d = ld_elem<T>(dc + (uint64_t)r * E);
            st_elem<T>(dc + (uint64_t)r * E, axpby(alpha, v, beta, d));
        }
    }
    (void)smem_raw;
    (void)td;
    (void)R;
}

// ------------------------------------------- pipelined transposed tiles
// One code path for every element size: each thread holds up to NE elements
// of a tile as raw 16-byte register slots; the element size and alignment
// (uniform per tile) pick 4/8/16-byte or split accesses. The CTA-level loop
// issues the NEXT tile's loads into the slots before it stores the current
// tile from shared memory, so loads stay in flight across the barriers.
enum : int { EM_4 = 0, EM_8 = 1, EM_8_SPLIT = 2, EM_16 = 3, EM_16_SPLIT8 = 4, EM_16_SPLIT4 = 5 };

__device__ __forceinline__ int elem_mode(const Tile &t) {
    const int esz = kind_esz(t.kind);
    const uint64_t a = t.src | t.dst | (uint64_t)t.src_ld | (uint64_t)t.dst_ld;
    if (esz == 4)
        return EM_4;
    if (esz == 8)
        return (a & 7u) == 0 ? EM_8 : EM_8_SPLIT;
    return (a & 15u) == 0 ? EM_16 : ((a & 7u) == 0 ? EM_16_SPLIT8 : EM_16_SPLIT4);
}

__device__ __forceinline__ uint4 ld_elem_raw(uint64_t a, int mode) {
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    switch (mode) {
    case EM_4: v.x = ldg_w<uint32_t>(a); break;
    case EM_8: {
        const unsigned long long w = ldg_w<unsigned long long>(a);
        v.x = (uint32_t)w;
        v.y = (uint32_t)(w >> 32);
        break;
    }
    case EM_8_SPLIT:
        v.x = ldg_w<uint32_t>(a);
        v.y = ldg_w<uint32_t>(a + 4);
        break;
    case EM_16: v = ldg_v4(a); break;
    case EM_16_SPLIT8: {
        const unsigned long long w0 = ldg_w<unsigned long long>(a);
        const unsigned long long w1 = ldg_w<unsigned long long>(a + 8);
        v = make_uint4((uint32_t)w0, (uint32_t)(w0 >> 32), (uint32_t)w1, (uint32_t)(w1 >> 32));
        break;
    }
    default:
        v = make_uint4(ldg_w<uint32_t>(a), ldg_w<uint32_t>(a + 4), ldg_w<uint32_t>(a + 8),
                       ldg_w<uint32_t>(a + 12));
        break;
    }
    return v;
}

__device__ __forceinline__ void st_elem_raw(uint64_t a, uint4 v, int mode) {
    switch (mode) {
    case EM_4: st_u32(a, v.x); break;
    case EM_8:
        st_w<unsigned long long>(a, (unsigned long long)v.x | ((unsigned long long)v.y << 32));
        break;
    case EM_8_SPLIT:
        st_u32(a, v.x);
        st_u32(a + 4, v.y);
        break;
    case EM_16: st_v4(a, v); break;
    case EM_16_SPLIT8:
        st_w<unsigned long long>(a, (unsigned long long)v.x | ((unsigned long long)v.y << 32));
        st_w<unsigned long long>(a + 8, (unsigned long long)v.z | ((unsigned long long)v.w << 32));
        break;
    default:
        st_u32(a, v.x);
        st_u32(a + 4, v.y);
        st_u32(a + 8, v.z);
        st_u32(a + 12, v.w);
        break;
    }
}

__device__ __forceinline__ void sts_elem(unsigned char *p, uint4 v, int esz) {
    if (esz == 4)
        *reinterpret_cast<uint32_t *>(p) = v.x;
    else if (esz == 8)
        *reinterpret_cast<uint2 *>(p) = make_uint2(v.x, v.y);
    else
        *reinterpret_cast<uint4 *>(p) = v;
}

__device__ __forceinline__ uint4 lds_elem(const unsigned char *p, int esz) {
    if (esz == 4)
        return make_uint4(*reinterpret_cast<const uint32_t *>(p), 0u, 0u, 0u);
    if (esz == 8) {
        const uint2 w = *reinterpret_cast<const uint2 *>(p);
        return make_uint4(w.x, w.y, 0u, 0u);
    }
    return *reinterpret_cast<const uint4 *>(p);
}

__device__ __forceinline__ bool is_plain_transpose(const Tile &t) {
    return (t.kind & KIND_TRANS) && !(t.kind & KIND_SCALED);
}

// A td x td tile (td a power of two) over a CTA: thread x owns one lane of
// the tile's contiguous direction and every (THREADS / td)-th line of the
// other, so its addresses advance by a constant step. The element mode is
// uniform per tile and a template argument here, so no access branches on it.
template <int MODE> struct ModeEsz {
    static constexpr int value = MODE == EM_4 ? 4 : (MODE <= EM_8_SPLIT ? 8 : 16);
};

// Load view: line r = storage column of the source (= final row), lane c
// along it (= final column).
template <int THREADS, int NE, int MODE>
__device__ __forceinline__ void load_slots_m(const Tile &t, int td_shift, uint4 (&v)[NE]) {
    constexpr int ESZ = ModeEsz<MODE>::value;
    const int c = threadIdx.x & ((1 << td_shift) - 1);
    const int r0 = threadIdx.x >> td_shift;
    const int rstep = THREADS >> td_shift;
    if (c >= t.cols)
        return;
    uint64_t a = t.src + (uint64_t)((long long)r0 * t.src_ld + (long long)c * ESZ);
    const uint64_t step = (uint64_t)((long long)rstep * t.src_ld);
#pragma unroll
    for (int i = 0; i < NE; ++i) {
        if (r0 + i * rstep < t.rows)
            v[i] = ld_elem_raw(a, MODE);
        a += step;
    }
}

template <int THREADS, int NE, int MODE>
__device__ __forceinline__ void slots_to_smem_m(const Tile &t, int td_shift,
                                                const uint4 (&v)[NE], unsigned char *smem) {
    constexpr int ESZ = ModeEsz<MODE>::value;
    const int td = 1 << td_shift;
    const int c = threadIdx.x & (td - 1);
    const int r0 = threadIdx.x >> td_shift;
    const int rstep = THREADS >> td_shift;
    if (c >= t.cols)
        return;
    unsigned char *p = smem + (size_t)(r0 * (td + 1) + c) * ESZ;
    const int step = rstep * (td + 1) * ESZ;
#pragma unroll
    for (int i = 0; i < NE; ++i) {
        if (r0 + i * rstep < t.rows)
            sts_elem(p, v[i], ESZ);
        p += step;
    }
}

// Store view: line c = destination storage column (= final column), lane r
// along it (= final row).
template <int THREADS, int NE, int MODE>
__device__ __forceinline__ void smem_to_global_m(const Tile &t, int td_shift,
                                                 const unsigned char *smem) {
    constexpr int ESZ = ModeEsz<MODE>::value;
    const int td = 1 << td_shift;
    const int r = threadIdx.x & (td - 1);
    const int c0 = threadIdx.x >> td_shift;
    const int cstep = THREADS >> td_shift;
    if (r >= t.rows)
        return;
    const bool conj = (t.kind & KIND_CONJ) != 0;
    const unsigned char *p = smem + (size_t)(r * (td + 1) + c0) * ESZ;
    uint64_t a = t.dst + (uint64_t)((long long)c0 * t.dst_ld + (long long)r * ESZ);
    const uint64_t step = (uint64_t)((long long)cstep * t.dst_ld);
#pragma unroll
    for (int i = 0; i < NE; ++i) {
        if (c0 + i * cstep < t.cols) {
            uint4 e = lds_elem(p, ESZ);
            if (conj) { // sign of the imaginary part: top word of the element
                if (ESZ == 8)
                    e.y ^= 0x80000000u;
                else if (ESZ == 16)
                    e.w ^= 0x80000000u;
            }
            st_elem_raw(a, e, MODE);
        }
        p += cstep * ESZ;
        a += step;
    }
}

#define G2G_MODE_DISPATCH(FN, ...)                                                  \
    switch (elem_mode(t)) {                                                         \
    case EM_4: FN<THREADS, NE, EM_4>(__VA_ARGS__); break;                           \
    case EM_8: FN<THREADS, NE, EM_8>(__VA_ARGS__); break;                           \
    case EM_8_SPLIT: FN<THREADS, NE, EM_8_SPLIT>(__VA_ARGS__); break;               \
    case EM_16: FN<THREADS, NE, EM_16>(__VA_ARGS__); break;                         \
    case EM_16_SPLIT8: FN<THREADS, NE, EM_16_SPLIT8>(__VA_ARGS__); break;           \
    default: FN<THREADS, NE, EM_16_SPLIT4>(__VA_ARGS__); break;                     \
    }

template <int THREADS, int NE>
__device__ __forceinline__ void load_tile_slots(const Tile &t, int td_shift, uint4 (&v)[NE]) {
    G2G_MODE_DISPATCH(load_slots_m, t, td_shift, v)
}
template <int THREADS, int NE>
__device__ __forceinline__ void slots_to_smem(const Tile &t, int td_shift, const uint4 (&v)[NE],
                                              unsigned char *smem) {
    G2G_MODE_DISPATCH(slots_to_smem_m, t, td_shift, v, smem)
}
template <int THREADS, int NE>
__device__ __forceinline__ void smem_to_global(const Tile &t, int td_shift,
                                               const unsigned char *smem) {
    G2G_MODE_DISPATCH(smem_to_global_m, t, td_shift, smem)
}
#undef G2G_MODE_DISPATCH

// Plain transposed tiles of 4-byte elements are twice as tall and nearly
// twice as wide (2 td final rows, 2 td - 4 final columns; shift tsh =
// td_shift + 1 for the 2 td x 2 td shared-memory tile): four elements per
// 16-byte register slot, so a thread holds 4 NE of them and a CTA keeps as
// many bytes in flight as with 16-byte elements. A tile line -- one source
// storage column of up to 2 td - 4 elements -- lies, at any 4-byte phase,
// in the 2 td / 4 aligned 16-byte blocks starting at its aligned base; the
// line's 2 td / 4 lanes load one block each, whole, and each block's words
// go to the elements they hold when the slots are written to shared memory
// (so the loads stay in flight until then, across the previous tile's
// stores). The line's bytes are read once, as the sectors that hold them:
// 4-byte loads at a random phase split every warp request over one more
// sector than the data holds, and L2 fetched the shared ones twice (reads
// 1.44x the data on random grids). Stores run along destination columns.
template <int W> __device__ __forceinline__ void slot_set(uint4 &v, uint32_t x) {
    if (W == 0) v.x = x; else if (W == 1) v.y = x; else if (W == 2) v.z = x; else v.w = x;
}
template <int W> __device__ __forceinline__ uint32_t slot_get(const uint4 &v) {
    return W == 0 ? v.x : (W == 1 ? v.y : (W == 2 ? v.z : v.w));
}
__device__ __forceinline__ uint32_t slot_word(const uint4 &v, int w) {
    return w == 0 ? v.x : (w == 1 ? v.y : (w == 2 ? v.z : v.w));
}
// Slot i of a thread holds block g of line r0 + i * rstep.
template <int THREADS, int NE>
__device__ __forceinline__ void load_slots_w4(const Tile &t, int tsh, uint4 (&v)[NE]) {
    const int gsh = tsh - 2; // log2 of the lanes per line
    const int g = threadIdx.x & ((1 << gsh) - 1);
    const int r0 = threadIdx.x >> gsh;
    const int rstep = THREADS >> gsh;
    const int run = t.cols * 4; // bytes of a line
    const int rel = g << 4;     // this lane's block, from the line's aligned base
#pragma unroll
    for (int i = 0; i < NE; ++i) {
        const int r = r0 + i * rstep;
        const uint64_t s = t.src + (uint64_t)((long long)r * t.src_ld);
        const int ph = (int)(s & 15u);
        // only blocks holding bytes of the line are read
        if (r < t.rows && rel < ph + run)
            v[i] = ldg_v4(s - (uint64_t)ph + (uint64_t)rel);
    }
}
// Shared memory [line][element] with a pitch of 2 td + 1 words, after a
// guard of 4 words: word w of block g holds element 4 g + w - q (q the
// line's phase in words). Lanes g >= 8 write their words in the order
// 2, 3, 0, 1, so that the lanes of a warp spread over the banks. Every word
// of every slot is written, unchecked: elements -3..-1 of a line fall on
// words 2 td - 2 .. 2 td of the line before (or the guard), elements from
// t.cols up on words of the line past its last element, and lines past
// t.rows inside the tile; a line holds at most 2 td - 4 elements, so none of
// those words is read back (slots not loaded hold unspecified words).
constexpr int kW4Guard = 4; // words ahead of line 0
template <int THREADS, int NE>
__device__ __forceinline__ void slots_to_smem_w4(const Tile &t, int tsh, const uint4 (&v)[NE],
                                                 unsigned char *smem) {
    const int T = 1 << tsh;
    const int gsh = tsh - 2;
    const int g = threadIdx.x & ((1 << gsh) - 1);
    const int r0 = threadIdx.x >> gsh;
    const int rstep = THREADS >> gsh;
    const bool rot = (g & 8) != 0; // the words in the order 2, 3, 0, 1
    uint32_t *p = reinterpret_cast<uint32_t *>(smem) + kW4Guard + r0 * (T + 1) + 4 * g +
                  (rot ? 2 : 0);
    const int step = rstep * (T + 1);
    uint64_t s = t.src + (uint64_t)((long long)r0 * t.src_ld);
    const uint64_t sstep = (uint64_t)((long long)rstep * t.src_ld);
#pragma unroll
    for (int i = 0; i < NE; ++i) {
        if (r0 + i * rstep >= T) // lines past the tile's 2 td (td = 16)
            break;
        // first word written, then the others
        uint32_t *w = p - (int)((s & 15u) >> 2);
        const uint4 q = rot ? make_uint4(v[i].z, v[i].w, v[i].x, v[i].y) : v[i];
        uint32_t *w2 = rot ? w - 2 : w + 2;
        w[0] = q.x;
        w[1] = q.y;
        w2[0] = q.z;
        w2[1] = q.w;
        p += step;
        s += sstep;
    }
}
// Stores of the tall tiles: one warp per destination column, lanes along
// its rows, every 32-lane pass starting on a 32-byte sector of the
// destination, so that a pass writes whole sectors except at the column's
// two ends (a store covering part of a sector that is absent from L2 makes
// L2 fetch the rest from DRAM): double and complex<float> 'T' on random
// grids 0.70 -> 0.75 of the copy peak.
template <int THREADS, int MODE>
__device__ __forceinline__ void smem_to_global_sect(const Tile &t, int pitch,
                                                    const unsigned char *smem) {
    constexpr int ESZ = ModeEsz<MODE>::value;
    constexpr int NWARP = THREADS / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool conj = (t.kind & KIND_CONJ) != 0;
    for (int c = warp; c < t.cols; c += NWARP) {
        const uint64_t dcol = t.dst + (uint64_t)((long long)c * t.dst_ld);
        const int lead = (int)(dcol & 31u) / ESZ; // elements of the first sector before row 0
        for (int r = lane - lead; r < t.rows; r += 32) {
            if (r < 0)
                continue;
            uint4 e = lds_elem(smem + (size_t)(r * pitch + c) * ESZ, ESZ);
            if (ESZ == 8 && conj) // complex<float>: the imaginary sign is the top word's
                e.y ^= 0x80000000u;
            st_elem_raw(dcol + (uint64_t)r * ESZ, e, MODE);
        }
    }
}
// (4-byte elements keep the thread-per-row view: for them the passes'
// extra index arithmetic costs more issue slots than the fills save.)
template <int THREADS, int NE>
__device__ __forceinline__ void smem_to_global_w4(const Tile &t, int tsh,
                                                  const unsigned char *smem) {
    const int T = 1 << tsh;
    const int r = threadIdx.x & (T - 1);
    const int c0 = threadIdx.x >> tsh;
    const int cstep = THREADS >> tsh;
    if (r >= t.rows)
        return;
    const uint32_t *p = reinterpret_cast<const uint32_t *>(smem) + kW4Guard + r * (T + 1) + c0;
    uint64_t a = t.dst + (uint64_t)((long long)c0 * t.dst_ld + (long long)r * 4);
    const uint64_t step = (uint64_t)((long long)cstep * t.dst_ld);
#pragma unroll
    for (int i = 0; i < 4 * NE; ++i) {
        if (c0 + i * cstep < t.cols)
            st_u32(a, p[i * cstep]);
        a += step;
    }
}
// Plain transposed tiles of 8-byte elements are twice as tall: 2 td final
// rows (the destination's contiguous direction: 512-byte runs at td = 32) by
// td final columns, two elements per register slot. Loads: lanes along the
// final columns (the source's contiguous direction), lines over the final
// rows; stores: lanes along the final rows, lines over the final columns.
// Shared memory [row][col] with a pitch of td + 1 elements keeps both views
// free of bank conflicts.
template <int THREADS, int NE, int MODE>
__device__ __forceinline__ void load_slots_t8(const Tile &t, int csh, uint4 (&v)[NE]) {
    const int c = threadIdx.x & ((1 << csh) - 1);
    const int r0 = threadIdx.x >> csh;
    const int rstep = THREADS >> csh;
    if (c >= t.cols)
        return;
    uint64_t a = t.src + (uint64_t)((long long)r0 * t.src_ld + (long long)c * 8);
    const uint64_t step = (uint64_t)((long long)rstep * t.src_ld);
#pragma unroll
    for (int i = 0; i < NE; ++i) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (r0 + (2 * i + h) * rstep < t.rows) {
                const uint4 e = ld_elem_raw(a, MODE);
                if (h == 0) {
                    v[i].x = e.x;
                    v[i].y = e.y;
                } else {
                    v[i].z = e.x;
                    v[i].w = e.y;
                }
            }
            a += step;
        }
    }
}
template <int THREADS, int NE>
__device__ __forceinline__ void slots_to_smem_t8(const Tile &t, int csh, const uint4 (&v)[NE],
                                                 unsigned char *smem) {
    const int TC = 1 << csh;
    const int c = threadIdx.x & (TC - 1);
    const int r0 = threadIdx.x >> csh;
    const int rstep = THREADS >> csh;
    if (c >= t.cols)
        return;
    uint2 *p = reinterpret_cast<uint2 *>(smem) + r0 * (TC + 1) + c;
    const int step = rstep * (TC + 1);
#pragma unroll
    for (int i = 0; i < NE; ++i) {
        if (r0 + (2 * i) * rstep < t.rows)
            p[0] = make_uint2(v[i].x, v[i].y);
        if (r0 + (2 * i + 1) * rstep < t.rows)
            p[step] = make_uint2(v[i].z, v[i].w);
        p += 2 * step;
    }
}
template <int THREADS, int NE, int MODE>
__device__ __forceinline__ void smem_to_global_t8(const Tile &t, int csh,
                                                  const unsigned char *smem) {
    smem_to_global_sect<THREADS, MODE>(t, (1 << csh) + 1, smem);
}

// Plain transposed tiles: the wide form for 4-byte elements, the tall form
// for 8-byte ones, the td x td form for 16-byte ones. Kernel instances whose
// plans hold no narrow transposes (NARROW false) carry the td x td form only,
// so its register allocation is not shared with the other two.
template <int THREADS, int NE, bool NARROW>
__device__ __forceinline__ void plain_load_slots(const Tile &t, int td_shift, uint4 (&v)[NE]) {
    if constexpr (!NARROW) {
        load_tile_slots<THREADS, NE>(t, td_shift, v);
        return;
    }
    switch (elem_mode(t)) {
    case EM_4: load_slots_w4<THREADS, NE>(t, td_shift + 1, v); break;
    case EM_8: load_slots_t8<THREADS, NE, EM_8>(t, td_shift, v); break;
    case EM_8_SPLIT: load_slots_t8<THREADS, NE, EM_8_SPLIT>(t, td_shift, v); break;
    default: load_tile_slots<THREADS, NE>(t, td_shift, v); break;
    }
}
template <int THREADS, int NE, bool NARROW>
__device__ __forceinline__ void plain_slots_to_smem(const Tile &t, int td_shift,
                                                    const uint4 (&v)[NE], unsigned char *smem) {
    if constexpr (!NARROW) {
        slots_to_smem<THREADS, NE>(t, td_shift, v, smem);
        return;
    }
    switch (kind_esz(t.kind)) {
    case 4: slots_to_smem_w4<THREADS, NE>(t, td_shift + 1, v, smem); break;
    case 8: slots_to_smem_t8<THREADS, NE>(t, td_shift, v, smem); break;
    default: slots_to_smem<THREADS, NE>(t, td_shift, v, smem); break;
    }
}
template <int THREADS, int NE, bool NARROW>
__device__ __forceinline__ void plain_smem_to_global(const Tile &t, int td_shift,
                                                     const unsigned char *smem) {
    if constexpr (!NARROW) {
        smem_to_global<THREADS, NE>(t, td_shift, smem);
        return;
    }
    switch (elem_mode(t)) {
    case EM_4: smem_to_global_w4<THREADS, NE>(t, td_shift + 1, smem); break;
    case EM_8: smem_to_global_t8<THREADS, NE, EM_8>(t, td_shift, smem); break;
    case EM_8_SPLIT: smem_to_global_t8<THREADS, NE, EM_8_SPLIT>(t, td_shift, smem); break;
    default: smem_to_global<THREADS, NE>(t, td_shift, smem); break;
    }
}

// ------------------------------------------------- scaled transposed tiles
// Element words <-> element type.
template <typename T> __device__ __forceinline__ T from_words(uint4 v);
template <> __device__ __forceinline__ float from_words<float>(uint4 v) {
    return __uint_as_float(v.x);
}
template <> __device__ __forceinline__ double from_words<double>(uint4 v) {
    return dbl(v.x, v.y);
}
template <> __device__ __forceinline__ cplxf from_words<cplxf>(uint4 v) {
    return cplxf{__uint_as_float(v.x), __uint_as_float(v.y)};
}
template <> __device__ __forceinline__ cplxd from_words<cplxd>(uint4 v) {
    return cplxd{dbl(v.x, v.y), dbl(v.z, v.w)};
}
__device__ __forceinline__ uint4 to_words(float x) {
    return make_uint4(__float_as_uint(x), 0u, 0u, 0u);
}
__device__ __forceinline__ uint4 to_words(double x) {
    uint4 o = make_uint4(0u, 0u, 0u, 0u);
    dbl_words(x, o.x, o.y);
    return o;
}
__device__ __forceinline__ uint4 to_words(cplxf x) {
    return make_uint4(__float_as_uint(x.x), __float_as_uint(x.y), 0u, 0u);
}
__device__ __forceinline__ uint4 to_words(cplxd x) {
    uint4 o;
    dbl_words(x.x, o.x, o.y);
    dbl_words(x.y, o.z, o.w);
    return o;
}

// A destination element read (coherent with this kernel's writes), by mode.
__device__ __forceinline__ uint32_t ld_dst_u32(uint64_t a) {
    uint32_t v;
    asm volatile("ld.global.u32 %0, [%1];" : "=r"(v) : "l"(a));
    return v;
}
__device__ __forceinline__ unsigned long long ld_dst_u64(uint64_t a) {
    unsigned long long v;
    asm volatile("ld.global.u64 %0, [%1];" : "=l"(v) : "l"(a));
    return v;
}
template <int MODE> __device__ __forceinline__ uint4 ld_dst_elem(uint64_t a) {
    if (MODE == EM_4)
        return make_uint4(ld_dst_u32(a), 0u, 0u, 0u);
    if (MODE == EM_8) {
        const unsigned long long w = ld_dst_u64(a);
        return make_uint4((uint32_t)w, (uint32_t)(w >> 32), 0u, 0u);
    }
    if (MODE == EM_8_SPLIT)
        return make_uint4(ld_dst_u32(a), ld_dst_u32(a + 4), 0u, 0u);
    if (MODE == EM_16)
        return ld_dst_v4(a);
    if (MODE == EM_16_SPLIT8) {
        const unsigned long long w0 = ld_dst_u64(a), w1 = ld_dst_u64(a + 8);
        return make_uint4((uint32_t)w0, (uint32_t)(w0 >> 32), (uint32_t)w1,
                          (uint32_t)(w1 >> 32));
    }
    return make_uint4(ld_dst_u32(a), ld_dst_u32(a + 4), ld_dst_u32(a + 8), ld_dst_u32(a + 12));
}

// smem_to_global_m with beta*d + alpha*e on every element, for a tile of
// 2^rsh rows by 2^csh columns staged [row][column] with a pitch of
// 2^csh + 1 elements.
template <int THREADS, int MODE, typename T, int CM>
__device__ __forceinline__ void smem_to_global_scaled_cm(const Tile &t, int rsh, int csh,
                                                         const unsigned char *smem,
                                                         const Coef<T> &k) {
    constexpr int ESZ = ModeEsz<MODE>::value;
    static_assert(ESZ == (int)sizeof(T), "element mode matches the element type");
    const int pitch = (1 << csh) + 1;
    const int r = threadIdx.x & ((1 << rsh) - 1);
    const int c0 = threadIdx.x >> rsh;
    const int cstep = THREADS >> rsh;
    const int n = ((1 << (rsh + csh)) + THREADS - 1) / THREADS; // elements per thread
    if (r >= t.rows)
        return;
    const bool conj = (t.kind & KIND_CONJ) != 0;
    // (4-byte tiles come in the wide layout, after its guard words)
    const unsigned char *p =
        smem + (ESZ == 4 ? kW4Guard * 4 : 0) + (size_t)(r * pitch + c0) * ESZ;
    uint64_t a = t.dst + (uint64_t)((long long)c0 * t.dst_ld + (long long)r * ESZ);
    const uint64_t step = (uint64_t)((long long)cstep * t.dst_ld);
    // the destination elements are pulled into L1 together (prefetches hold
    // no registers), then combined one at a time: the complex arithmetic of
    // several elements would not fit the register budget
#pragma unroll 1
    for (int i = 0; i < n; ++i)
        if (c0 + i * cstep < t.cols)
            asm volatile("prefetch.global.L1 [%0];" ::"l"(a + (uint64_t)i * step));
#pragma unroll 1
    for (int i = 0; i < n; ++i) {
        if (c0 + i * cstep < t.cols) {
            uint4 e = lds_elem(p, ESZ);
            if (conj) {
                if (ESZ == 8)
                    e.y ^= 0x80000000u;
                else if (ESZ == 16)
                    e.w ^= 0x80000000u;
            }
            const T d = from_words<T>(ld_dst_elem<MODE>(a));
            st_elem_raw(a, to_words(axpby_m<CM>(k, from_words<T>(e), d)), MODE);
        }
        p += cstep * ESZ;
        a += step;
    }
}
template <int THREADS, int MODE, typename T>
__device__ __forceinline__ void smem_to_global_scaled_m(const Tile &t, int rsh, int csh,
                                                        const unsigned char *smem,
                                                        const Coef<T> &k) {
    coef_dispatch(k, [&](auto cm) {
        smem_to_global_scaled_cm<THREADS, MODE, T, decltype(cm)::value>(t, rsh, csh, smem, k);
    });
}

// Stores a scaled transposed (+ conjugated) tile already staged in shared
// memory (by the transposed path's loads, in the tile shape of its element
// size: 4-byte 2td x 2td, 8-byte 2td rows x td columns, 16-byte td x td):
// beta*d + alpha*op(s).
template <int THREADS, typename T>
__device__ __forceinline__ void scaled_transpose_store(const Tile &t, const PairInfo *pairs,
                                                       const unsigned char *smem, int td) {
    const int td_shift = td >= 32 ? 5 : 4;
    const Coef<T> k = coef_from<T>(pairs[t.pair]);
    const int mode = elem_mode(t);
    if constexpr (sizeof(T) == 4) {
        smem_to_global_scaled_m<THREADS, EM_4, T>(t, td_shift + 1, td_shift + 1, smem, k);
    } else if constexpr (sizeof(T) == 8) {
        if (mode == EM_8)
            smem_to_global_scaled_m<THREADS, EM_8, T>(t, td_shift + 1, td_shift, smem, k);
        else
            smem_to_global_scaled_m<THREADS, EM_8_SPLIT, T>(t, td_shift + 1, td_shift, smem, k);
    } else {
        if (mode == EM_16)
            smem_to_global_scaled_m<THREADS, EM_16, T>(t, td_shift, td_shift, smem, k);
        else if (mode == EM_16_SPLIT8)
            smem_to_global_scaled_m<THREADS, EM_16_SPLIT8, T>(t, td_shift, td_shift, smem, k);
        else
            smem_to_global_scaled_m<THREADS, EM_16_SPLIT4, T>(t, td_shift, td_shift, smem, k);
    }
}

// -------------------------------------------------------------- cast tiles
// A fused cast: final = convert(op(initial)). float <-> double and
// complex<float> <-> complex<double> round each part to nearest (the CUDA
// conversion intrinsics, IEEE round-to-nearest-even); real -> complex sets
// the imaginary part to +0; 'C' flips the imaginary sign after the
// conversion. Non-transposed tiles whose destination elements sit whole in
// 16-byte chunks run on the copy ring (ring_store_cast); the others are
// CTA-wide: non-transposed ones walk columns (warps) and rows (lanes, four
// elements in flight each), transposed ones go through a padded
// shared-memory tile of destination elements.
__device__ __forceinline__ float cvt(float v, float *) { return v; }
__device__ __forceinline__ double cvt(float v, double *) { return (double)v; }
__device__ __forceinline__ float cvt(double v, float *) { return __double2float_rn(v); }
__device__ __forceinline__ double cvt(double v, double *) { return v; }
__device__ __forceinline__ cplxf cvt(float v, cplxf *) { return cplxf{v, 0.0f}; }
__device__ __forceinline__ cplxd cvt(float v, cplxd *) { return cplxd{(double)v, 0.0}; }
__device__ __forceinline__ cplxf cvt(double v, cplxf *) {
    return cplxf{__double2float_rn(v), 0.0f};
}
__device__ __forceinline__ cplxd cvt(double v, cplxd *) { return cplxd{v, 0.0}; }
__device__ __forceinline__ cplxf cvt(cplxf v, cplxf *) { return v; }
__device__ __forceinline__ cplxd cvt(cplxf v, cplxd *) { return cplxd{(double)v.x, (double)v.y}; }
__device__ __forceinline__ cplxf cvt(cplxd v, cplxf *) {
    return cplxf{__double2float_rn(v.x), __double2float_rn(v.y)};
}
__device__ __forceinline__ cplxd cvt(cplxd v, cplxd *) { return v; }
template <typename D, typename S> __device__ __forceinline__ D convert(S v) {
    return cvt(v, (D *)nullptr);
}

// A non-transposed cast tile element by element, columns over NWARP warps
// (warp `warp` of them), four elements in flight per lane.
// (one function per conversion, called per tile: the kernel does not carry
// the registers of all twelve)
template <int NWARP, typename S, typename D>
__device__ __noinline__ void cast_cols(const Tile &t, int warp) {
    constexpr int ES = (int)sizeof(S), ED = (int)sizeof(D);
    const int lane = threadIdx.x & 31;
    const int R = t.rows, Cn = t.cols;
    for (int c = warp; c < Cn; c += NWARP) {
        const uint64_t sc = t.src + (uint64_t)((long long)c * t.src_ld);
        const uint64_t dc = t.dst + (uint64_t)((long long)c * t.dst_ld);
        for (int r0 = lane; r0 < R; r0 += 32 * 4) {
            S v[4];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (r0 + 32 * k < R)
                    v[k] = ld_elem<S>(sc + (uint64_t)(r0 + 32 * k) * ES);
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (r0 + 32 * k < R)
                    st_elem<D>(dc + (uint64_t)(r0 + 32 * k) * ED, convert<D>(v[k]));
        }
    }
}

template <int THREADS, typename S, typename D>
__device__ __noinline__ void cast_tile(const Tile &t, unsigned char *smem_raw, int td) {
    constexpr int NWARP = THREADS / 32;
    constexpr int ED = (int)sizeof(D);
    constexpr int ES = (int)sizeof(S);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool conj = (t.kind & KIND_CONJ) != 0;
    const int R = t.rows, Cn = t.cols;
    if (!(t.kind & KIND_TRANS)) {
        cast_cols<NWARP, S, D>(t, warp);
        return;
    }
    D *smem = reinterpret_cast<D *>(smem_raw);
    const int pitch = td + 1;
    __syncthreads(); // earlier tiles are out of shared memory
    for (int r = warp; r < R; r += NWARP)
        for (int c = lane; c < Cn; c += 32)
            smem[r * pitch + c] = convert<D>(
                ld_elem<S>(t.src + (uint64_t)((long long)r * t.src_ld + (long long)c * ES)));
    __syncthreads();
    for (int c = warp; c < Cn; c += NWARP) {
        const uint64_t dc = t.dst + (uint64_t)((long long)c * t.dst_ld);
        for (int r = lane; r < R; r += 32) {
            D v = smem[r * pitch + c];
            if (conj)
                v = conj_elem(v);
            st_elem<D>(dc + (uint64_t)r * ED, v);
        }
    }
}

template <typename T> struct is_cplx { static constexpr bool value = false; };
template <> struct is_cplx<cplxf> { static constexpr bool value = true; };
template <> struct is_cplx<cplxd> { static constexpr bool value = true; };

template <int THREADS, typename S>
__device__ __forceinline__ void cast_to(const Tile &t, unsigned char *smem, int td) {
    switch ((t.kind >> KIND_DTYPE_SHIFT) & 3u) {
    case 0: // complex -> real is refused on the host
        if constexpr (!is_cplx<S>::value)
            cast_tile<THREADS, S, float>(t, smem, td);
        break;
    case 1:
        if constexpr (!is_cplx<S>::value)
            cast_tile<THREADS, S, double>(t, smem, td);
        break;
    case 2: cast_tile<THREADS, S, cplxf>(t, smem, td); break;
    default: cast_tile<THREADS, S, cplxd>(t, smem, td); break;
    }
}
template <int THREADS>
__device__ __forceinline__ void cast_dispatch(const Tile &t, unsigned char *smem, int td) {
    switch ((t.kind >> KIND_SRC_DTYPE_SHIFT) & 3u) {
    case 0: cast_to<THREADS, float>(t, smem, td); break;
    case 1: cast_to<THREADS, double>(t, smem, td); break;
    case 2: cast_to<THREADS, cplxf>(t, smem, td); break;
    default: cast_to<THREADS, cplxd>(t, smem, td); break;
    }
}

// ------------------------------------------------------------------ kernel
// (a kernel carries the arithmetic of the element types its plan scales:
// real, complex or both)
template <int THREADS, int PATHS>
__device__ __forceinline__ void scaled_dispatch(const Tile &t, const PairInfo *pairs,
                                                unsigned char *smem, int td) {
    switch ((t.kind >> KIND_DTYPE_SHIFT) & 3u) {
    case 0:
        if constexpr ((PATHS & PATH_SCALED_REAL) != 0)
            scaled_tile<THREADS, float>(t, pairs, smem, td);
        break;
    case 1:
        if constexpr ((PATHS & PATH_SCALED_REAL) != 0)
            scaled_tile<THREADS, double>(t, pairs, smem, td);
        break;
    case 2:
        if constexpr ((PATHS & PATH_SCALED_COMPLEX) != 0)
            scaled_tile<THREADS, cplxf>(t, pairs, smem, td);
        break;
    default:
        if constexpr ((PATHS & PATH_SCALED_COMPLEX) != 0)
            scaled_tile<THREADS, cplxd>(t, pairs, smem, td);
        break;
    }
}
template <int THREADS, int PATHS>
__device__ __forceinline__ void scaled_transpose_dispatch(const Tile &t, const PairInfo *pairs,
                                                          const unsigned char *smem, int td) {
    switch ((t.kind >> KIND_DTYPE_SHIFT) & 3u) {
    case 0:
        if constexpr ((PATHS & PATH_SCALED_REAL) != 0)
            scaled_transpose_store<THREADS, float>(t, pairs, smem, td);
        break;
    case 1:
        if constexpr ((PATHS & PATH_SCALED_REAL) != 0)
            scaled_transpose_store<THREADS, double>(t, pairs, smem, td);
        break;
    case 2:
        if constexpr ((PATHS & PATH_SCALED_COMPLEX) != 0)
            scaled_transpose_store<THREADS, cplxf>(t, pairs, smem, td);
        break;
    default:
        if constexpr ((PATHS & PATH_SCALED_COMPLEX) != 0)
            scaled_transpose_store<THREADS, cplxd>(t, pairs, smem, td);
        break;
    }
}



// Register budget: 64 per thread (1024 resident threads per SM), enough for
// U = 4 chunks per lane in flight on the register path without spilling.
template <int U, int THREADS> struct MinBlocks {
    static constexpr int value = (1024 / THREADS) > 0 ? (1024 / THREADS) : 1;
};

// Kernels with scaled tiles: 128 registers (512 resident threads per SM)
// for the complex arithmetic (and the element conversions of cast tiles),
// 80 (768 threads) for the real one, so that neither spills.
template <int PATHS, int U, int THREADS> struct MinBlocksP {
    static constexpr int value =
        (PATHS & (PATH_SCALED_COMPLEX | PATH_CAST)) ? ((512 / THREADS) > 0 ? (512 / THREADS) : 1)
        : (PATHS & PATH_SCALED_REAL)  ? ((768 / THREADS) > 0 ? (768 / THREADS) : 1)
                                      : MinBlocks<U, THREADS>::value;
};

// Plain transposed tiles of one narrow element size when they are the
// launch's only tiles (PATH_W4_STAGED: 4-byte elements, tiles of 2 td final
// rows by 2 td - 4 columns; PATH_W8_STAGED: 8-byte elements, 2 td rows by td
// columns): the tile's source lines are copied raw into a ring of kStages
// shared-memory stages with cp.async (the line's aligned 16-byte blocks, one
// per lane), so that a CTA keeps the next kStages - 1 tiles in flight while
// it stores the current one, without holding them in registers; the stores
// read each element at its line's phase. A stage is 2 td lines of 2 td + 4
// words (16-byte aligned lines). A line of 4-byte elements (at most 2 td - 4
// of them, 8 td - 16 bytes) lies at any phase in 2 td / 4 blocks, one of
// 8-byte elements (at most td, 8 td bytes) in 2 td / 4 + 1; either way its
// elements sit at words q .. q + cols * ES / 4 - 1 < 2 td + 4, q its phase
// in words.
// Two stages: more CTAs per SM (shared memory is what limits them) beat a
// deeper ring (float 'T' on random grids 16384² 0.410 -> 0.395 ms with two
// stages instead of three, block-cyclic 64x64 -> 96x200 0.637 -> 0.542 ms).
constexpr int kStages = 2;
template <int T> struct StagedTile {
    static constexpr int pitch = T + 4; // words per line
    static constexpr int bytes = T * pitch * 4;
};
__host__ __device__ constexpr size_t staged_smem_bytes(int td) {
    return (size_t)kStages * (size_t)(2 * td) * (size_t)(2 * td + 4) * 4u;
}
// Issues the copies of tile t's source lines into the stage at shared
// address st (one 16-byte block per lane and pass; blocks past the line's
// last element and lines past t.rows are not copied).
template <int THREADS, int T, int ES>
__device__ __forceinline__ void staged_issue(const Tile &t, uint32_t st) {
    constexpr int G = ES == 4 ? T / 4 : T / 4 + 1;    // lanes (blocks) per line
    constexpr int RSTEP = THREADS / G;                // lines per pass
    constexpr int NP = (T + RSTEP - 1) / RSTEP;       // passes
    constexpr int P = StagedTile<T>::pitch;
    const int g = threadIdx.x % G;
    const int r0 = threadIdx.x / G;
    if (r0 >= RSTEP) // threads past the last whole line group
        return;
    const int run = t.cols * ES;
    const int rel = g * 16;
    uint64_t s = t.src + (uint64_t)((long long)r0 * t.src_ld);
    const uint64_t sstep = (uint64_t)((long long)RSTEP * t.src_ld);
    uint32_t d = st + (uint32_t)((r0 * P + 4 * g) * 4);
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        const int ph = (int)(s & 15u);
        if (r0 + i * RSTEP < t.rows && rel < ph + run)
            cp_async16(d, s - (uint64_t)ph + (uint64_t)rel);
        s += sstep;
        d += (uint32_t)(RSTEP * P * 4);
    }
}
// Stores tile t from its stage: a thread per final row (source line) r,
// columns c0, c0 + CSTEP, ...; element c of line r starts at word
// q_r + c * ES / 4. AL8: 8-byte elements whose source and destination
// addresses and strides are all multiples of 8 (one 8-byte shared-memory
// read and one 8-byte store per element; else two of 4 bytes).
template <int THREADS, int T, int ES, bool AL8>
__device__ __forceinline__ void staged_store(const Tile &t, const uint32_t *st) {
    constexpr int CSTEP = THREADS / T;
    constexpr int CMAX = ES == 4 ? T - 4 : T / 2;
    constexpr int NC = (CMAX + CSTEP - 1) / CSTEP;
    constexpr int P = StagedTile<T>::pitch;
    constexpr int EW = ES / 4; // words per element
    const int r = threadIdx.x % T;
    const int c0 = threadIdx.x / T;
    if (r >= t.rows)
        return;
    const uint64_t s = t.src + (uint64_t)((long long)r * t.src_ld);
    const uint32_t *p = st + r * P + (int)((s & 15u) >> 2) + c0 * EW;
    uint64_t a = t.dst + (uint64_t)((long long)c0 * t.dst_ld + (long long)r * ES);
    const uint64_t step = (uint64_t)((long long)CSTEP * t.dst_ld);
    // complex<float> 'C': the imaginary part's sign is the top word's
    const uint32_t flip = (ES == 8 && (t.kind & KIND_CONJ)) ? 0x80000000u : 0u;
#pragma unroll
    for (int i = 0; i < NC; ++i) {
        if (c0 + i * CSTEP < t.cols) {
            const uint32_t *e = p + i * CSTEP * EW;
            if constexpr (ES == 4) {
                st_u32(a, e[0]);
            } else if constexpr (AL8) {
                const uint2 v = *reinterpret_cast<const uint2 *>(e);
                asm volatile("st.global.v2.u32 [%0], {%1, %2};" ::"l"(a), "r"(v.x),
                             "r"(v.y ^ flip)
                             : "memory");
            } else {
                st_u32(a, e[0]);
                st_u32(a + 4, e[1] ^ flip);
            }
        }
        a += step;
    }
}
// The CTA's tiles ti = blockIdx.x + k G in order: tile k sits in stage
// k % S; at step k the CTA waits for its own copies of tile k, meets at a
// barrier (tile k's lines are then visible to all its threads, and every
// thread has stored tile k - 1), refills stage (k - 1) % S with tile
// k + S - 1 and stores tile k. Every step commits one copy group (empty
// when no tile is left), so the wait always counts S - 2 younger groups.
template <int THREADS, int TDS, int ES>
__device__ __forceinline__ void cta_phase_staged(const PlanList &list, unsigned char *smem) {
    constexpr int T = 2 << TDS; // 2 td lines per tile
    constexpr int S = kStages;
    constexpr int SB = StagedTile<T>::bytes;
    const long long n = list.total_cta;
    const long long G = gridDim.x;
    const uint32_t base = smem_addr(smem);
    const PairInfo *unused;
#pragma unroll
    for (int k = 0; k < S - 1; ++k) {
        const long long ti = (long long)blockIdx.x + (long long)k * G;
        if (ti < n)
            staged_issue<THREADS, T, ES>(*locate_cta(list, ti, unused),
                                         base + (uint32_t)(k * SB));
        cp_async_commit();
    }
    int st = 0;
    for (long long ti = blockIdx.x; ti < n; ti += G) {
        cp_async_wait<S - 2>();
        __syncthreads();
        const long long nx = ti + (long long)(S - 1) * G;
        const int sn = st == 0 ? S - 1 : st - 1;
        if (nx < n)
            staged_issue<THREADS, T, ES>(*locate_cta(list, nx, unused),
                                         base + (uint32_t)(sn * SB));
        cp_async_commit();
        const Tile t = *locate_cta(list, ti, unused);
        const uint32_t *stage = reinterpret_cast<const uint32_t *>(smem + st * SB);
        if (ES == 8 && elem_mode(t) == EM_8)
            staged_store<THREADS, T, ES, true>(t, stage);
        else
            staged_store<THREADS, T, ES, false>(t, stage);
        st = st + 1 == S ? 0 : st + 1;
    }
    cp_async_wait<0>();
}

// Plain transposed tiles of 16-byte elements (td x td) on the same ring
// (PATH_W16_STAGED): a source line of td elements, 16 td bytes at a phase of
// at most 12, lies in td + 1 aligned blocks (td + 1 lanes a line, a pitch of
// 4 (td + 1) words); a stage is smaller than the narrow ring's.
template <int TD> struct StagedTile16 {
    static constexpr int blocks = TD + 1;
    static constexpr int pitch = 4 * blocks;
    static constexpr int bytes = TD * pitch * 4;
};
template <int THREADS, int TD>
__device__ __forceinline__ void staged_issue16(const Tile &t, uint32_t st) {
    constexpr int G = StagedTile16<TD>::blocks;
    constexpr int RSTEP = THREADS / G;
    constexpr int NP = (TD + RSTEP - 1) / RSTEP;
    constexpr int P = StagedTile16<TD>::pitch;
    const int g = threadIdx.x % G;
    const int r0 = threadIdx.x / G;
    if (r0 >= RSTEP)
        return;
    const int run = t.cols * 16;
    const int rel = g * 16;
    uint64_t s = t.src + (uint64_t)((long long)r0 * t.src_ld);
    const uint64_t sstep = (uint64_t)((long long)RSTEP * t.src_ld);
    uint32_t d = st + (uint32_t)((r0 * P + 4 * g) * 4);
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        const int ph = (int)(s & 15u);
        if (r0 + i * RSTEP < t.rows && rel < ph + run)
            cp_async16(d, s - (uint64_t)ph + (uint64_t)rel);
        s += sstep;
        d += (uint32_t)(RSTEP * P * 4);
    }
}
// A thread per final row r, columns c0, c0 + CSTEP, ...; element c of line r
// at words q_r + 4 c .. + 3. AL: every address and stride a multiple of 16
// (one 16-byte read and store), else 4-byte words.
template <int THREADS, int TD, bool AL>
__device__ __forceinline__ void staged_store16(const Tile &t, const uint32_t *st) {
    constexpr int CSTEP = THREADS / TD;
    constexpr int NC = (TD + CSTEP - 1) / CSTEP;
    constexpr int P = StagedTile16<TD>::pitch;
    const int r = threadIdx.x % TD;
    const int c0 = threadIdx.x / TD;
    if (r >= t.rows)
        return;
    const uint64_t s = t.src + (uint64_t)((long long)r * t.src_ld);
    const uint32_t *p = st + r * P + (int)((s & 15u) >> 2) + c0 * 4;
    uint64_t a = t.dst + (uint64_t)((long long)c0 * t.dst_ld + (long long)r * 16);
    const uint64_t step = (uint64_t)((long long)CSTEP * t.dst_ld);
    // complex<double> 'C': the imaginary part's sign is its top word's
    const uint32_t flip = (t.kind & KIND_CONJ) ? 0x80000000u : 0u;
#pragma unroll
    for (int i = 0; i < NC; ++i) {
        if (c0 + i * CSTEP < t.cols) {
            const uint32_t *e = p + i * CSTEP * 4;
            if constexpr (AL) {
                const uint4 v = *reinterpret_cast<const uint4 *>(e);
                st_v4(a, make_uint4(v.x, v.y, v.z, v.w ^ flip));
            } else {
                st_u32(a, e[0]);
                st_u32(a + 4, e[1]);
                st_u32(a + 8, e[2]);
                st_u32(a + 12, e[3] ^ flip);
            }
        }
        a += step;
    }
}
template <int THREADS, int TDS>
__device__ __forceinline__ void cta_phase_staged16(const PlanList &list, unsigned char *smem) {
    constexpr int TD = 1 << TDS;
    constexpr int S = kStages;
    constexpr int SB = StagedTile16<TD>::bytes;
    const long long n = list.total_cta;
    const long long G = gridDim.x;
    const uint32_t base = smem_addr(smem);
    const PairInfo *unused;
#pragma unroll
    for (int k = 0; k < S - 1; ++k) {
        const long long ti = (long long)blockIdx.x + (long long)k * G;
        if (ti < n)
            staged_issue16<THREADS, TD>(*locate_cta(list, ti, unused), base + (uint32_t)(k * SB));
        cp_async_commit();
    }
    int st = 0;
    for (long long ti = blockIdx.x; ti < n; ti += G) {
        cp_async_wait<S - 2>();
        __syncthreads();
        const long long nx = ti + (long long)(S - 1) * G;
        const int sn = st == 0 ? S - 1 : st - 1;
        if (nx < n)
            staged_issue16<THREADS, TD>(*locate_cta(list, nx, unused), base + (uint32_t)(sn * SB));
        cp_async_commit();
        const Tile t = *locate_cta(list, ti, unused);
        const uint32_t *stage = reinterpret_cast<const uint32_t *>(smem + st * SB);
        if (elem_mode(t) == EM_16)
            staged_store16<THREADS, TD, true>(t, stage);
        else
            staged_store16<THREADS, TD, false>(t, stage);
        st = st + 1 == S ? 0 : st + 1;
    }
    cp_async_wait<0>();
}

// Scaled transposed tiles of one element size (4 or 8 bytes) when they are
// the launch's only tiles (PATH_W4S_STAGED, PATH_W8S_STAGED): the ring stages
// the source lines as above and, behind them in the same stage, the tile's
// destination columns (final rows are their contiguous direction): column c
// at c * 4 GD words, GD = (2 td * ES + 27) / 16 blocks for a run of at most
// 2 td elements at a phase of at most 12 bytes. The stores combine
// beta * d + alpha * op(s) with both operands read from the stage, so no
// destination load waits in the store loop.
template <int TD, int ES> struct StagedDst {
    static constexpr int lines = 2 * TD;                // final rows of a tile
    static constexpr int cmax = ES == 4 ? 2 * TD - 4 : TD; // its columns at most
    static constexpr int blocks = (lines * ES + 27) / 16;
    static constexpr int pitch = 4 * blocks; // words per column
    static constexpr int bytes = cmax * pitch * 4;
};
// Two stages as well (a stage is twice the plain ring's): three CTAs of two
// stages per SM outran two CTAs of three (float 'T' with α/β on random grids
// 16384² 0.748 -> 0.606 ms).
constexpr int kScaledStages = 2;
__host__ __device__ constexpr size_t staged_scaled_smem_bytes(int td) {
    const size_t src = (size_t)(2 * td) * (size_t)(2 * td + 4) * 4u;
    const size_t d4 = (size_t)(2 * td - 4) * 4u * (size_t)((2 * td * 4 + 27) / 16) * 4u;
    const size_t d8 = (size_t)td * 4u * (size_t)((2 * td * 8 + 27) / 16) * 4u;
    return (size_t)kScaledStages * (src + (d4 > d8 ? d4 : d8));
}
template <int THREADS, int TD, int ES>
__device__ __forceinline__ void staged_issue_dst(const Tile &t, uint32_t st) {
    constexpr int GD = StagedDst<TD, ES>::blocks;
    const int total = t.cols * GD;
    const int run = t.rows * ES;
    for (int f = threadIdx.x; f < total; f += THREADS) {
        const int c = f / GD;
        const int g = f - c * GD;
        const uint64_t dc = t.dst + (uint64_t)((long long)c * t.dst_ld);
        const int ph = (int)(dc & 15u);
        if (g * 16 < ph + run)
            cp_async16(st + (uint32_t)((c * GD + g) * 16), dc - (uint64_t)ph + (uint64_t)(g * 16));
    }
}
template <int THREADS, int TD, int ES, typename T, int MODE, int CM>
__device__ __forceinline__ void staged_store_scaled(const Tile &t, const uint32_t *ss,
                                                    const uint32_t *sd, const Coef<T> &k) {
    using SD = StagedDst<TD, ES>;
    constexpr int TL = SD::lines;
    constexpr int P = StagedTile<TL>::pitch;
    constexpr int CSTEP = THREADS / TL;
    constexpr int NC = (SD::cmax + CSTEP - 1) / CSTEP;
    constexpr int EW = ES / 4;
    const int r = threadIdx.x % TL;
    const int c0 = threadIdx.x / TL;
    if (r >= t.rows)
        return;
    const uint64_t s = t.src + (uint64_t)((long long)r * t.src_ld);
    const uint32_t *ps = ss + r * P + (int)((s & 15u) >> 2) + c0 * EW;
    const uint32_t *pd = sd + c0 * SD::pitch + r * EW;
    uint64_t a = t.dst + (uint64_t)((long long)c0 * t.dst_ld + (long long)r * ES);
    const uint64_t step = (uint64_t)((long long)CSTEP * t.dst_ld);
    const uint32_t flip = (ES == 8 && (t.kind & KIND_CONJ)) ? 0x80000000u : 0u;
#pragma unroll
    for (int i = 0; i < NC; ++i) {
        if (c0 + i * CSTEP < t.cols) {
            const uint32_t *e = ps + i * CSTEP * EW;
            // the column's phase: that of the element's address less its row
            const int qd = (int)(((a - (uint64_t)(r * ES)) & 15u) >> 2);
            const uint32_t *dw = pd + i * CSTEP * SD::pitch + qd;
            uint4 sv = make_uint4(e[0], 0u, 0u, 0u), dv = make_uint4(dw[0], 0u, 0u, 0u);
            if constexpr (EW == 2) {
                sv.y = e[1] ^ flip;
                dv.y = dw[1];
            }
            st_elem_raw(a, to_words(axpby_m<CM>(k, from_words<T>(sv), from_words<T>(dv))),
                        MODE);
        }
        a += step;
    }
}
template <int THREADS, int TD, int ES, typename T>
__device__ __forceinline__ void staged_store_scaled_t(const Tile &t, const uint32_t *ss,
                                                      const uint32_t *sd, const PairInfo *pairs) {
    const Coef<T> k = coef_from<T>(pairs[t.pair]);
    const bool al = ES == 4 || elem_mode(t) == EM_8;
    coef_dispatch(k, [&](auto cm) {
        constexpr int CM = decltype(cm)::value;
        if (ES == 4)
            staged_store_scaled<THREADS, TD, ES, T, EM_4, CM>(t, ss, sd, k);
        else if (al)
            staged_store_scaled<THREADS, TD, ES, T, EM_8, CM>(t, ss, sd, k);
        else
            staged_store_scaled<THREADS, TD, ES, T, EM_8_SPLIT, CM>(t, ss, sd, k);
    });
}
// The ring of cta_phase_staged, of kScaledStages stages, each holding the
// source lines and then the destination columns of its tile (with two
// stages the wait is for all copies: the next tile's are issued after it).
template <int THREADS, int TDS, int ES, int PATHS>
__device__ __forceinline__ void cta_phase_staged_scaled(const PlanList &list,
                                                        unsigned char *smem) {
    constexpr int TD = 1 << TDS;
    constexpr int S = kScaledStages;
    constexpr int SBS = StagedTile<2 * TD>::bytes;
    constexpr int SB = SBS + StagedDst<TD, ES>::bytes;
    const long long n = list.total_cta;
    const long long G = gridDim.x;
    const uint32_t base = smem_addr(smem);
    const PairInfo *unused;
#pragma unroll
    for (int k = 0; k < S - 1; ++k) {
        const long long ti = (long long)blockIdx.x + (long long)k * G;
        if (ti < n) {
            const Tile t = *locate_cta(list, ti, unused);
            staged_issue<THREADS, 2 * TD, ES>(t, base + (uint32_t)(k * SB));
            staged_issue_dst<THREADS, TD, ES>(t, base + (uint32_t)(k * SB + SBS));
        }
        cp_async_commit();
    }
    int st = 0;
    for (long long ti = blockIdx.x; ti < n; ti += G) {
        cp_async_wait<S - 2>();
        __syncthreads();
        const long long nx = ti + (long long)(S - 1) * G;
        const int sn = st == 0 ? S - 1 : st - 1;
        if (nx < n) {
            const Tile t = *locate_cta(list, nx, unused);
            staged_issue<THREADS, 2 * TD, ES>(t, base + (uint32_t)(sn * SB));
            staged_issue_dst<THREADS, TD, ES>(t, base + (uint32_t)(sn * SB + SBS));
        }
        cp_async_commit();
        const PairInfo *pairs;
        const Tile t = *locate_cta(list, ti, pairs);
        const uint32_t *ss = reinterpret_cast<const uint32_t *>(smem + st * SB);
        const uint32_t *sd = reinterpret_cast<const uint32_t *>(smem + st * SB + SBS);
        if constexpr (ES == 4) {
            staged_store_scaled_t<THREADS, TD, 4, float>(t, ss, sd, pairs);
        } else {
            const uint32_t dt = (t.kind >> KIND_DTYPE_SHIFT) & 3u;
            if constexpr ((PATHS & PATH_SCALED_COMPLEX) != 0) {
                if (dt == 2u) {
                    staged_store_scaled_t<THREADS, TD, 8, cplxf>(t, ss, sd, pairs);
                    st = st + 1 == S ? 0 : st + 1;
                    continue;
                }
            }
            staged_store_scaled_t<THREADS, TD, 8, double>(t, ss, sd, pairs);
        }
        st = st + 1 == S ? 0 : st + 1;
    }
    cp_async_wait<0>();
}

// CTA-level tiles (transposed, and scaled or cast ones that are not
// warp-level) of a launch, static striding, with the next plain transposed
// tile's loads issued before the current tile is stored.
// The tile edge is a template argument (TDS = log2 td): every lane mapping,
// pitch and loop bound of the tile helpers is then a constant.
template <int THREADS, int PATHS, int TDS>
__device__ __forceinline__ void cta_phase_t(const PlanList &list, unsigned char *smem) {
    if constexpr ((PATHS & PATH_W4_STAGED) != 0) {
        cta_phase_staged<THREADS, TDS, 4>(list, smem);
        return;
    }
    if constexpr ((PATHS & PATH_W8_STAGED) != 0) {
        cta_phase_staged<THREADS, TDS, 8>(list, smem);
        return;
    }
    if constexpr ((PATHS & PATH_W16_STAGED) != 0) {
        cta_phase_staged16<THREADS, TDS>(list, smem);
        return;
    }
    if constexpr ((PATHS & PATH_W4S_STAGED) != 0) {
        cta_phase_staged_scaled<THREADS, TDS, 4, PATHS>(list, smem);
        return;
    }
    if constexpr ((PATHS & PATH_W8S_STAGED) != 0) {
        cta_phase_staged_scaled<THREADS, TDS, 8, PATHS>(list, smem);
        return;
    }
    constexpr int td = 1 << TDS;
    constexpr int NE = 1024 / THREADS; // slots for a 32 x 32 tile
    // Kernels with scaled or cast tiles move plain transposed tiles one at a
    // time: the next tile's loads held across their element code would cost
    // more registers than the overlap gains.
    constexpr bool PIPE = (PATHS & PATH_TRANSPOSE) && !(PATHS & (PATH_SCALED | PATH_CAST));
    // kernels with element arithmetic take every plain transposed shape
    constexpr bool NARROW = (PATHS & (PATH_NARROW_TRANSPOSE | PATH_SCALED | PATH_CAST)) != 0;
    constexpr int td_shift = TDS;
    const long long n = list.total_cta;
    const long long G = gridDim.x;
    uint4 v[NE];
    long long ti = blockIdx.x;
    Tile cur;
    const PairInfo *cur_pairs = nullptr;
    if (ti < n) {
        cur = *locate_cta(list, ti, cur_pairs);
        if (PIPE && is_plain_transpose(cur))
            plain_load_slots<THREADS, NE, NARROW>(cur, td_shift, v);
    }
    while (ti < n) {
        const long long next = ti + G;
        // the next descriptor is read now and the one after is pulled into
        // L2, so neither miss sits between the barriers
        Tile nxt;
        const PairInfo *nxt_pairs = nullptr;
        if (next < n) {
            nxt = *locate_cta(list, next, nxt_pairs);
            if (threadIdx.x == 0 && next + G < n) {
                const PairInfo *unused;
                asm volatile("prefetch.global.L2 [%0];" ::"l"(locate_cta(list, next + G, unused)));
            }
        }
        const bool staged = !(cur.kind & KIND_CAST) &&
                            ((PATHS & PATH_SCALED) ? (cur.kind & KIND_TRANS) != 0
                                                   : is_plain_transpose(cur));
        if ((PATHS & (PATH_TRANSPOSE | PATH_SCALED)) && staged) {
            __syncthreads(); // earlier tiles are out of shared memory
            // transposed tiles, plain or scaled, staged through shared memory
            // (transposed tiles of 4- and 8-byte elements, plain or scaled,
            // come in the wide and tall shapes)
            if (!PIPE)
                plain_load_slots<THREADS, NE, NARROW>(cur, td_shift, v);
            plain_slots_to_smem<THREADS, NE, NARROW>(cur, td_shift, v, smem);
            __syncthreads();
            if (PIPE && next < n && is_plain_transpose(nxt))
                plain_load_slots<THREADS, NE, NARROW>(nxt, td_shift, v); // in flight during the stores
            if ((PATHS & PATH_SCALED) && (cur.kind & KIND_SCALED))
                scaled_transpose_dispatch<THREADS, PATHS>(cur, cur_pairs, smem, td);
            else
                plain_smem_to_global<THREADS, NE, NARROW>(cur, td_shift, smem);
        } else {
            if ((PATHS & PATH_CAST) && (cur.kind & KIND_CAST))
                cast_dispatch<THREADS>(cur, smem, td);
            else if (PATHS & PATH_SCALED)
                scaled_dispatch<THREADS, PATHS>(cur, cur_pairs, smem, td);
            if (PIPE && next < n && is_plain_transpose(nxt))
                plain_load_slots<THREADS, NE, NARROW>(nxt, td_shift, v);
        }
        if (next < n) {
            cur = nxt;
            cur_pairs = nxt_pairs;
        }
        ti = next;
    }
}

template <int THREADS, int PATHS>
__device__ __forceinline__ void cta_phase(const PlanList &list, unsigned char *smem, int td) {
    if (td >= 32)
        cta_phase_t<THREADS, PATHS, 5>(list, smem);
    else
        cta_phase_t<THREADS, PATHS, 4>(list, smem);
}

// A non-transposed cast tile from source type S on the register path.
template <int NWARP, typename S>
__device__ __forceinline__ void cast_cols_to(const Tile &t, int warp) {
    switch ((t.kind >> KIND_DTYPE_SHIFT) & 3u) {
    case 0:
        if constexpr (!is_cplx<S>::value)
            cast_cols<NWARP, S, float>(t, warp);
        break;
    case 1:
        if constexpr (!is_cplx<S>::value)
            cast_cols<NWARP, S, double>(t, warp);
        break;
    case 2: cast_cols<NWARP, S, cplxf>(t, warp); break;
    default: cast_cols<NWARP, S, cplxd>(t, warp); break;
    }
}

// A warp-level work item on the register path: a plain copy, or (kernels
// with scaled or cast tiles) a non-transposed scaled or cast tile, by NWARP
// warps.
template <int NWARP, int U, int PATHS>
__device__ __forceinline__ void warp_tile(const Tile &t, int warp, const PairInfo *pairs) {
    if constexpr ((PATHS & PATH_CAST) != 0) {
        if (t.kind & KIND_CAST) {
            switch ((t.kind >> KIND_SRC_DTYPE_SHIFT) & 3u) {
            case 0: cast_cols_to<NWARP, float>(t, warp); break;
            case 1: cast_cols_to<NWARP, double>(t, warp); break;
            case 2: cast_cols_to<NWARP, cplxf>(t, warp); break;
            default: cast_cols_to<NWARP, cplxd>(t, warp); break;
            }
            return;
        }
    }
    if constexpr ((PATHS & PATH_SCALED) != 0) {
        if (t.kind & KIND_SCALED) {
            switch ((t.kind >> KIND_DTYPE_SHIFT) & 3u) {
            case 0:
                if constexpr ((PATHS & PATH_SCALED_REAL) != 0)
                    scaled_copy_tile<NWARP, 2, float>(t, warp, coef_from<float>(pairs[t.pair]));
                break;
            case 1:
                if constexpr ((PATHS & PATH_SCALED_REAL) != 0)
                    scaled_copy_tile<NWARP, 2, double>(t, warp, coef_from<double>(pairs[t.pair]));
                break;
            case 2:
                if constexpr ((PATHS & PATH_SCALED_COMPLEX) != 0)
                    scaled_copy_tile<NWARP, 2, cplxf>(t, warp, coef_from<cplxf>(pairs[t.pair]));
                break;
            default:
                if constexpr ((PATHS & PATH_SCALED_COMPLEX) != 0)
                    scaled_copy_tile<NWARP, 2, cplxd>(t, warp, coef_from<cplxd>(pairs[t.pair]));
                break;
            }
            return;
        }
    }
    copy_tile<NWARP, U>(t, warp);
}

template <int THREADS, int U, int PATHS>
__global__ void __launch_bounds__(THREADS, (MinBlocksP<PATHS, U, THREADS>::value))
    scatter_kernel(const __grid_constant__ PlanList list, int td) {
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr int NWARP = THREADS / 32;
    const int warp = threadIdx.x >> 5;
    // phase 1: plain copies, one warp per tile, so a CTA keeps NWARP tiles in
    // flight however small the pieces are
    if (PATHS & PATH_COPY) {
        const long long GW = (long long)gridDim.x * NWARP;
        for (long long ti = (long long)blockIdx.x * NWARP + warp; ti < list.total_copy;
             ti += GW) {
            const PairInfo *pairs;
            if ((threadIdx.x & 31) == 0 && ti + GW < list.total_copy) {
                const PairInfo *unused;
                asm volatile("prefetch.global.L2 [%0];" ::"l"(locate_copy(list, ti + GW, unused)));
            }
            const Tile t = *locate_copy(list, ti, pairs);
            warp_tile<1, U, PATHS>(t, 0, pairs);
        }
    }
    // phase 2: transposed and scaled tiles, one CTA per tile
    if (PATHS & (PATH_TRANSPOSE | PATH_SCALED | PATH_CAST))
        cta_phase<THREADS, PATHS>(list, smem, td);
}

// ------------------------------------------------------ cp.async copy ring
// Phase 1 of the ring kernel: the plain copy tiles of a warp form one stream
// of stages of 32 x U chunks (the chunk sequence of copy_tile, cut into
// stages; a stage belongs to one tile). The warp keeps RING_D - 1 stages in
// flight as cp.async 16-byte copies into a per-warp ring in shared memory
// while it stores the oldest landed stage, so its reads continue across tile
// boundaries and overlap its own stores. Two stages (one in flight while one
// is stored) at 16 warps per SM measured best on the layouts tried: deeper
// rings or more warps put more concurrent column streams on the DRAM and
// lose row locality. A stage is then stored from shared memory:
// chunk i of a stage reads its source blocks at ring slots i and i + 1 (slot
// 32U holds the block after the stage's last chunk, loaded by lane 31).
// The issuing and the storing side each walk the chunk sequence with their
// own cursor (column, chunk, column addresses), advanced by additions only.
// Every wait is cp.async.wait_group, which completes with the copies.
#ifndef G2G_RING_D
#define G2G_RING_D 2
#endif
constexpr int RING_D = G2G_RING_D; // stages per warp ring (RING_D - 1 in flight)

// Tile descriptors reach the warp through a queue in shared memory: the
// descriptor of the warp's tile j + RING_LA is copied (cp.async, in the same
// commit group as the stage being issued) when the issuing side enters tile
// j. A stage enters at most one tile and the groups of all but the last
// RING_D - 1 stages have landed when a stage is issued, so it has landed by
// the time that tile is entered, however short the tiles in between are. The
// storing side, at most RING_D - 1 stages behind, reads the same entries.
constexpr int RING_LA = RING_D;
constexpr int RING_Q = (2 * RING_D + 1 <= 8) ? 8 : 16; // entries; > RING_LA + RING_D
constexpr int RING_QE = 64;                            // bytes per entry (a 48-byte Tile)
// The ring kernel's option word: log2 of the run length, prefetch switch.
constexpr int RING_OPT_RUN_MASK = 0xff;
constexpr int RING_OPT_L2_PREFETCH = 0x100;
static_assert(sizeof(Tile) <= RING_QE, "a Tile fits a queue entry");

// Per-warp shared memory: RING_D stages of 32U + 1 source blocks plus XR
// extra rows of 32U blocks (kernels with scaled tiles: one row, the
// destination chunks they update; with cast tiles: two rows, a chunk's second
// and third source blocks), the descriptor queue, one valid flag per stage
// (0: no stage, the warp's work is done).
template <int U, int XR> __host__ __device__ constexpr int ring_stage_bytes() {
    return (U * 32 + 1) * 16 + XR * U * 32 * 16;
}
template <int U, int XR> __host__ __device__ constexpr int ring_warp_bytes() {
    return RING_D * ring_stage_bytes<U, XR>() + RING_Q * RING_QE +
           ((RING_D * 4 + 15) / 16) * 16;
}
__host__ __device__ constexpr int ring_extra_rows(int paths) {
    return (paths & PATH_SCALED) ? 1 : ((paths & PATH_CAST) ? 2 : 0);
}

// ring reads, ordered after the wait and warp barrier that make them valid
__device__ __forceinline__ uint32_t lds_ring_u32(uint32_t a) {
    uint32_t v;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ uint4 lds_ring(uint32_t a) {
    uint4 v;
    asm volatile("ld.shared.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "r"(a)
                 : "memory");
    return v;
}

// Per-tile constants of a chunk walk (chunks per column as in copy_tile).
struct RingTile {
    uint64_t dst, src;
    long long dld, sld;     // column strides, bytes
    long long stepd, steps; // dq columns, bytes
    int cols, L, cpc, dq, dr, total;
    float rcp; // 1 / cpc, for the quotients of small numbers by cpc
    bool aligned;
    uint32_t kind; // KIND_SCALED: beta*dst + alpha*src (dtype in the kind);
                   // KIND_CAST: converted elements (both dtypes in the kind)
    int pair;
    int edsh, essh; // cast tiles: log2 of the destination / source element sizes
};
__device__ __forceinline__ void ring_tile_init(RingTile &c, const Tile &t) {
    c.kind = t.kind;
    c.pair = t.pair;
    c.dst = t.dst;
    c.src = t.src;
    c.dld = t.dst_ld;
    c.sld = t.src_ld;
    c.cols = t.cols;
    c.L = t.rows * kind_esz(t.kind);
    c.aligned = (((t.src - t.dst) | (uint64_t)(t.src_ld - t.dst_ld)) & 15u) == 0;
    if (t.kind & KIND_CAST) {
        const uint32_t sdt = (t.kind >> KIND_SRC_DTYPE_SHIFT) & 3u; // f32, f64, c64, c128
        c.edsh = 2 + (int)(t.kind & KIND_ESZ_MASK);
        c.essh = 2 + (sdt != 0u ? 1 : 0) + (sdt == 3u ? 1 : 0);
        // a cast chunk fetches its own source blocks: the walk counts the
        // destination chunks a column touches (the lead d0 is at most 12)
        c.cpc = (t.dst_ld & 15) == 0 ? (int)(((t.dst & 15u) + (uint64_t)c.L + 15u) >> 4)
                                     : ((c.L + 27) >> 4);
    } else if (((t.dst_ld | t.src_ld) & 15) == 0) {
        const int d0 = (int)(t.dst & 15u);
        const int sh = (int)((t.src - (uint64_t)d0) & 15u);
        c.cpc = (sh + d0 + c.L + 15) >> 4;
    } else {
        c.cpc = c.aligned ? ((c.L + 27) >> 4) : ((c.L + 39) >> 4);
    }
    // floor(32 / cpc) from a correctly rounded reciprocal: (32 + 1/2) / cpc
    // lies at least 1/(2 cpc) from an integer, far above the rounding error
    c.rcp = __frcp_rn((float)c.cpc);
    c.dq = __float2int_rz(32.5f * c.rcp);
    c.dr = 32 - c.dq * c.cpc;
    c.stepd = (long long)c.dq * c.dld;
    c.steps = (long long)c.dq * c.sld;
    c.total = c.cols * c.cpc;
}

// A lane's position: chunk k of column col, whose addresses are d / s.
struct RingWalk {
    uint64_t d, s;
    int col, k;
};
__device__ __forceinline__ void ring_walk_init(RingWalk &w, const RingTile &c, int lane) {
    w.col = __float2int_rz(((float)lane + 0.5f) * c.rcp); // lane / cpc, lane < 32
    w.k = lane - w.col * c.cpc;
    w.d = c.dst + (uint64_t)((long long)w.col * c.dld);
    w.s = c.src + (uint64_t)((long long)w.col * c.sld);
}
__device__ __forceinline__ void ring_walk_step(RingWalk &w, const RingTile &c) { // +32 chunks
    w.col += c.dq;
    w.k += c.dr;
    w.d += (uint64_t)c.stepd;
    w.s += (uint64_t)c.steps;
    if (w.k >= c.cpc) {
        w.k -= c.cpc;
        ++w.col;
        w.d += (uint64_t)c.dld;
        w.s += (uint64_t)c.sld;
    }
}

// Cast tiles on the ring (destination elements whole within each 16-byte
// chunk): the walk runs over destination chunks; the chunk of lane i in step
// u needs source elements [jlo, jhi) of its column, at most 32 bytes, which
// lie in at most three aligned source blocks, staged in rows 0, 1 and 2 of
// slot u * 32 + i. The storing side converts them into the chunk.
struct CastSpan {
    int jlo, jhi, j0; // elements in the chunk, j0 the first element slot (may be < 0)
    int first;        // byte of element jlo from the column's aligned source base
    int nblk;         // source blocks (0: the chunk holds no destination bytes)
};
// edsh / essh: log2 of the destination / source element sizes
__device__ __forceinline__ CastSpan cast_span(const RingTile &c, const RingWalk &w, int edsh,
                                              int essh) {
    CastSpan p;
    const int d0 = (int)(w.d & 15u);
    const int relb = (w.k << 4) - d0; // chunk start from the column start, bytes
    p.nblk = 0;
    p.j0 = relb >> edsh; // exact: d0 is a multiple of the element size
    p.jlo = relb < 0 ? 0 : p.j0;
    p.jhi = (relb + 16 < c.L ? relb + 16 : c.L) >> edsh;
    p.first = 0;
    if (w.col < c.cols && relb < c.L && relb + 16 > 0) {
        const int s0 = (int)(w.s & 15u);
        p.first = s0 + (p.jlo << essh);
        p.nblk = ((s0 + (p.jhi << essh) - 1) >> 4) - (p.first >> 4) + 1;
    }
    return p;
}
template <int U>
__device__ __forceinline__ void ring_issue_cast(const RingTile &c, RingWalk &w, uint32_t slots,
                                                int lane) {
    constexpr uint32_t ROW1 = (U * 32 + 1) * 16, ROW = U * 32 * 16;
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const CastSpan p = cast_span(c, w, c.edsh, c.essh);
        const uint32_t slot = slots + (uint32_t)((u * 32 + lane) << 4);
        const uint64_t a0 = (w.s & ~15ull) + (uint64_t)(p.first & ~15);
        if (p.nblk > 0)
            cp_async16(slot, a0);
        if (p.nblk > 1)
            cp_async16(slot + ROW1, a0 + 16);
        if (p.nblk > 2)
            cp_async16(slot + ROW1 + ROW, a0 + 32);
        ring_walk_step(w, c);
    }
}
// Word of the staged source window at byte `o` from its first block.
template <int U>
__device__ __forceinline__ uint32_t cast_word(uint32_t slot, int o) {
    constexpr uint32_t ROW1 = (U * 32 + 1) * 16, ROW = U * 32 * 16;
    const int q = o >> 4;
    return lds_ring_u32(slot + (q == 0 ? 0u : (q == 1 ? ROW1 : ROW1 + ROW)) + (uint32_t)(o & 15));
}
// A source element of the staged window at byte `o` (its words may lie in
// two consecutive blocks).
template <int U, typename S> struct CastSrc;
template <int U> struct CastSrc<U, float> {
    static __device__ __forceinline__ float get(uint32_t slot, int o) {
        return __uint_as_float(cast_word<U>(slot, o));
    }
};
template <int U> struct CastSrc<U, double> {
    static __device__ __forceinline__ double get(uint32_t slot, int o) {
        return dbl(cast_word<U>(slot, o), cast_word<U>(slot, o + 4));
    }
};
template <int U> struct CastSrc<U, cplxf> {
    static __device__ __forceinline__ cplxf get(uint32_t slot, int o) {
        return cplxf{__uint_as_float(cast_word<U>(slot, o)),
                     __uint_as_float(cast_word<U>(slot, o + 4))};
    }
};
template <int U> struct CastSrc<U, cplxd> {
    static __device__ __forceinline__ cplxd get(uint32_t slot, int o) {
        return cplxd{dbl(cast_word<U>(slot, o), cast_word<U>(slot, o + 4)),
                     dbl(cast_word<U>(slot, o + 8), cast_word<U>(slot, o + 12))};
    }
};
// A source element from its words.
template <typename S> __device__ __forceinline__ S src_words(const uint32_t *w);
template <> __device__ __forceinline__ float src_words<float>(const uint32_t *w) {
    return __uint_as_float(w[0]);
}
template <> __device__ __forceinline__ double src_words<double>(const uint32_t *w) {
    return dbl(w[0], w[1]);
}
template <> __device__ __forceinline__ cplxf src_words<cplxf>(const uint32_t *w) {
    return cplxf{__uint_as_float(w[0]), __uint_as_float(w[1])};
}
template <> __device__ __forceinline__ cplxd src_words<cplxd>(const uint32_t *w) {
    return cplxd{dbl(w[0], w[1]), dbl(w[2], w[3])};
}
// A converted element as destination words.
template <typename D> __device__ __forceinline__ void put_words(uint32_t *w, D v);
template <> __device__ __forceinline__ void put_words<float>(uint32_t *w, float v) {
    w[0] = __float_as_uint(v);
}
template <> __device__ __forceinline__ void put_words<double>(uint32_t *w, double v) {
    dbl_words(v, w[0], w[1]);
}
template <> __device__ __forceinline__ void put_words<cplxf>(uint32_t *w, cplxf v) {
    w[0] = __float_as_uint(v.x);
    w[1] = __float_as_uint(v.y);
}
template <> __device__ __forceinline__ void put_words<cplxd>(uint32_t *w, cplxd v) {
    dbl_words(v.x, w[0], w[1]);
    dbl_words(v.y, w[2], w[3]);
}
// Stores one landed stage of a cast tile: each chunk's elements converted,
// whole chunks with one 16-byte store, head and tail chunks by element.
template <int U, typename S, typename D>
__device__ __forceinline__ void ring_store_cast(const RingTile &c, RingWalk &w, uint32_t slots,
                                                int lane) {
    constexpr int ES = (int)sizeof(S), ED = (int)sizeof(D), EPC = 16 / ED;
#pragma unroll
    for (int u = 0; u < U; ++u) {
        constexpr int EDSH = ED == 4 ? 2 : (ED == 8 ? 3 : 4);
        constexpr int ESSH = ES == 4 ? 2 : (ES == 8 ? 3 : 4);
        const CastSpan p = cast_span(c, w, EDSH, ESSH);
        if (p.nblk > 0) {
            const uint32_t slot = slots + (uint32_t)((u * 32 + lane) << 4);
            // byte of element 0 in the staged window (may be < 0)
            const int o0 = (int)(w.s & 15u) - (p.first & ~15);
            const uint64_t chunk = w.d - (w.d & 15u) + (uint64_t)(w.k << 4);
            if (p.jlo == p.j0 && p.jhi == p.j0 + EPC) {
                // the chunk's source bytes from word q of the first block on,
                // gathered from the rows with 16-byte reads
                constexpr uint32_t ROW1 = (U * 32 + 1) * 16, ROW = U * 32 * 16;
                const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
                const uint32_t q = (uint32_t)((p.first & 15) >> 2);
                const uint4 r0 = lds_ring(slot);
                const uint4 r1 = p.nblk > 1 ? lds_ring(slot + ROW1) : zero;
                const uint4 w0 = funnel_words(r0, r1, q);
                uint32_t sw[8] = {w0.x, w0.y, w0.z, w0.w, 0u, 0u, 0u, 0u};
                if constexpr (EPC * ES > 16) {
                    const uint4 r2 = p.nblk > 2 ? lds_ring(slot + ROW1 + ROW) : zero;
                    const uint4 w1 = funnel_words(r1, r2, q);
                    sw[4] = w1.x;
                    sw[5] = w1.y;
                    sw[6] = w1.z;
                    sw[7] = w1.w;
                }
                uint32_t x[4];
#pragma unroll
                for (int e = 0; e < EPC; ++e)
                    put_words<D>(x + e * (ED / 4), convert<D>(src_words<S>(sw + e * (ES / 4))));
                st_v4(chunk, make_uint4(x[0], x[1], x[2], x[3]));
            } else {
#pragma unroll
                for (int e = 0; e < EPC; ++e) {
                    const int j = p.j0 + e;
                    if (j >= p.jlo && j < p.jhi)
                        st_elem<D>(chunk + (uint64_t)(e * ED),
                                   convert<D>(CastSrc<U, S>::get(slot, o0 + j * ES)));
                }
            }
        }
        ring_walk_step(w, c);
    }
}
template <int U, typename S>
__device__ __forceinline__ void ring_store_cast_to(const RingTile &c, RingWalk &w,
                                                   uint32_t slots, int lane) {
    switch ((c.kind >> KIND_DTYPE_SHIFT) & 3u) {
    case 0:
        if constexpr (!is_cplx<S>::value)
            ring_store_cast<U, S, float>(c, w, slots, lane);
        break;
    case 1:
        if constexpr (!is_cplx<S>::value)
            ring_store_cast<U, S, double>(c, w, slots, lane);
        break;
    case 2: ring_store_cast<U, S, cplxf>(c, w, slots, lane); break;
    default: ring_store_cast<U, S, cplxd>(c, w, slots, lane); break;
    }
}
template <int U>
__device__ __forceinline__ void ring_store_cast_dispatch(const RingTile &c, RingWalk &w,
                                                         uint32_t slots, int lane) {
    switch ((c.kind >> KIND_SRC_DTYPE_SHIFT) & 3u) {
    case 0: ring_store_cast_to<U, float>(c, w, slots, lane); break;
    case 1: ring_store_cast_to<U, double>(c, w, slots, lane); break;
    case 2: ring_store_cast_to<U, cplxf>(c, w, slots, lane); break;
    default: ring_store_cast_to<U, cplxd>(c, w, slots, lane); break;
    }
}
// Issues the cp.async copies of one stage into ring slots `slots`; for a
// scaled tile (SC kernels) also the destination chunks, after the source
// blocks. Only this lane's own destination words of a chunk are ever stored,
// and no other work item writes them, so the chunk's other words may be stale.
template <int U, int PATHS>
__device__ __forceinline__ void ring_issue(const RingTile &c, RingWalk &w, uint32_t slots,
                                           int lane) {
    if constexpr ((PATHS & PATH_CAST) != 0) {
        if (c.kind & KIND_CAST) {
            ring_issue_cast<U>(c, w, slots, lane);
            return;
        }
    }
    const bool scaled = (PATHS & PATH_SCALED) && (c.kind & KIND_SCALED);
#pragma unroll
    for (int u = 0; u < U; ++u) {
        if (w.col < c.cols) {
            const int d0 = (int)(w.d & 15u);
            const uint64_t sa = w.s - (uint64_t)d0; // source byte under chunk 0's first byte
            const int sh = (int)(sa & 15u);
            const uint64_t base = sa - (uint64_t)sh;
            const int rel = w.k << 4;
            const int lo = sh + d0, hi = sh + d0 + c.L;
            const uint32_t slot = slots + (uint32_t)((u * 32 + lane) << 4);
            if (rel < hi && rel + 16 > lo)
                cp_async16(slot, base + (uint64_t)rel);
            if (u == U - 1 && lane == 31 && sh != 0 && rel + 16 < hi)
                cp_async16(slot + 16, base + (uint64_t)(rel + 16));
            if (scaled && rel + 16 > d0 && rel < d0 + c.L)
                cp_async16(slot + (uint32_t)((U * 32 + 1) * 16),
                           w.d - (uint64_t)d0 + (uint64_t)rel);
        }
        ring_walk_step(w, c);
    }
}

// Stores one landed stage from its ring slots.
template <int U>
__device__ __forceinline__ void ring_store(const RingTile &c, RingWalk &w, uint32_t slots,
                                           int lane) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
        if (w.col < c.cols) {
            const int d0 = (int)(w.d & 15u);
            const int rel = w.k << 4;
            const int end = d0 + c.L;
            if (rel + 16 > d0 && rel < end) { // the chunk holds destination words
                const uint32_t slot = slots + (uint32_t)((u * 32 + lane) << 4);
                uint4 o = lds_ring(slot);
                if (!c.aligned) {
                    const int sh = (int)((w.s - (uint64_t)d0) & 15u);
                    if (sh)
                        o = funnel_words(o, lds_ring(slot + 16), (uint32_t)(sh >> 2));
                }
                const uint64_t chunk = w.d - (uint64_t)d0 + (uint64_t)rel;
                if (rel >= d0 && rel + 16 <= end) {
                    st_v4(chunk, o);
                } else { // head or tail chunk of the column: whole words
                    const int wlo = rel >= d0 ? 0 : (d0 - rel) >> 2;
                    const int whi = rel + 16 <= end ? 4 : (end - rel) >> 2;
                    if (wlo <= 0 && whi > 0) st_u32(chunk, o.x);
                    if (wlo <= 1 && whi > 1) st_u32(chunk + 4, o.y);
                    if (wlo <= 2 && whi > 2) st_u32(chunk + 8, o.z);
                    if (wlo <= 3 && whi > 3) st_u32(chunk + 12, o.w);
                }
            }
        }
        ring_walk_step(w, c);
    }
}

// Stores one landed stage of a scaled tile: each destination chunk becomes
// beta*d + alpha*s on its whole elements (the pair's alpha and beta, rounded
// as scaled_copy_tile rounds them), then the chunk walk's word-masked store.
template <int U, typename T, int CM>
__device__ __forceinline__ void ring_store_scaled_m(const RingTile &c, RingWalk &w,
                                                    uint32_t slots, int lane,
                                                    const Coef<T> &k) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
        if (w.col < c.cols) {
            const int d0 = (int)(w.d & 15u);
            const int rel = w.k << 4;
            const int end = d0 + c.L;
            if (rel + 16 > d0 && rel < end) {
                const uint32_t slot = slots + (uint32_t)((u * 32 + lane) << 4);
                uint4 o = lds_ring(slot);
                if (!c.aligned) {
                    const int sh = (int)((w.s - (uint64_t)d0) & 15u);
                    if (sh)
                        o = funnel_words(o, lds_ring(slot + 16), (uint32_t)(sh >> 2));
                }
                o = axpby_chunk<CM>(k, o, lds_ring(slot + (uint32_t)((U * 32 + 1) * 16)));
                const uint64_t chunk = w.d - (uint64_t)d0 + (uint64_t)rel;
                if (rel >= d0 && rel + 16 <= end) {
                    st_v4(chunk, o);
                } else {
                    const int wlo = rel >= d0 ? 0 : (d0 - rel) >> 2;
                    const int whi = rel + 16 <= end ? 4 : (end - rel) >> 2;
                    if (wlo <= 0 && whi > 0) st_u32(chunk, o.x);
                    if (wlo <= 1 && whi > 1) st_u32(chunk + 4, o.y);
                    if (wlo <= 2 && whi > 2) st_u32(chunk + 8, o.z);
                    if (wlo <= 3 && whi > 3) st_u32(chunk + 12, o.w);
                }
            }
        }
        ring_walk_step(w, c);
    }
}
template <int U, typename T>
__device__ __forceinline__ void ring_store_scaled(const RingTile &c, RingWalk &w,
                                                  uint32_t slots, int lane,
                                                  const PairInfo *pp) {
    const Coef<T> k = coef_from<T>(*pp);
    coef_dispatch(k, [&](auto cm) {
        ring_store_scaled_m<U, T, decltype(cm)::value>(c, w, slots, lane, k);
    });
}
template <int U, int PATHS>
__device__ __forceinline__ void ring_store_scaled_dispatch(const RingTile &c, RingWalk &w,
                                                           uint32_t slots, int lane,
                                                           const PairInfo *pp) {
    switch ((c.kind >> KIND_DTYPE_SHIFT) & 3u) {
    case 0:
        if constexpr ((PATHS & PATH_SCALED_REAL) != 0)
            ring_store_scaled<U, float>(c, w, slots, lane, pp);
        break;
    case 1:
        if constexpr ((PATHS & PATH_SCALED_REAL) != 0)
            ring_store_scaled<U, double>(c, w, slots, lane, pp);
        break;
    case 2:
        if constexpr ((PATHS & PATH_SCALED_COMPLEX) != 0)
            ring_store_scaled<U, cplxf>(c, w, slots, lane, pp);
        break;
    default:
        if constexpr ((PATHS & PATH_SCALED_COMPLEX) != 0)
            ring_store_scaled<U, cplxd>(c, w, slots, lane, pp);
        break;
    }
}

// Lanes 0-2 copy the descriptor of copy tile `ti` (if any) into queue entry
// `entry` (a shared-memory address); tiles are 16-byte aligned in HBM.
__device__ __forceinline__ void ring_queue_fetch(const PlanList &list, long long ti,
                                                 uint32_t entry, int lane) {
    if (lane < 3 && ti < list.total_copy) {
        const PairInfo *unused;
        const uint64_t g = (uint64_t)locate_copy(list, ti, unused);
        cp_async16(entry + (uint32_t)(lane * 16), g + (uint64_t)(lane * 16));
    }
}

// Which copy tiles a warp takes: runs of 2^run_shift consecutive tiles, the
// runs dealt round-robin over the grid's warps (one tile per run: plain
// static striding). Consecutive tiles are neighbouring cells of a column
// strip, so a run keeps one warp streaming along the same block columns.
struct RingOrder {
    long long base;   // first tile of the warp's first run
    long long stride; // tiles between the starts of its runs
    int shift;        // log2 of the run length
    int l2_prefetch;  // bulk L2 prefetch of each multi-stage tile's columns
};
__device__ __forceinline__ long long tile_of(const RingOrder &o, int j) {
    return o.base + (long long)(j >> o.shift) * o.stride + (j & ((1 << o.shift) - 1));
}

// When a warp enters a tile of several stages and the plan asks for it,
// each lane asks L2 for one source column of the tile in a single bulk
// prefetch (a hint: nothing waits on it), so the tile's later stages find
// their blocks in L2. Only the aligned 16-byte cover of each column is named,
// which lies in the column's own blocks. It pays on plans of small tiles and
// costs a little on 16 KB tiles of long columns, so it is a tuning switch.
template <int U>
__device__ __forceinline__ void ring_prefetch_tile(const RingTile &c, const RingOrder &o,
                                                   int lane) {
    if (!o.l2_prefetch || c.total <= 32 * U || c.L < 256 || lane >= c.cols)
        return;
    const int Ls = (c.kind & KIND_CAST) ? c.L / kind_esz(c.kind) * kind_src_esz(c.kind) : c.L;
    const uint64_t s = c.src + (uint64_t)((long long)lane * c.sld);
    const uint64_t start = s & ~15ull, end = (s + (uint64_t)Ls + 15u) & ~15ull;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(start),
                 "r"((uint32_t)(end - start))
                 : "memory");
}

// The issuing side: its tile (index ti, ordinal j among the warp's tiles),
// the tile's walk constants and this lane's position, the next chunk.
struct RingIssue {
    long long ti;
    int j;
    RingTile c;
    RingWalk w;
    int idx0;
};

// Fills ring stage `st` from the issuing cursor (or marks it empty) and commits it.
template <int U, int PATHS>
__device__ __forceinline__ void ring_fill(const PlanList &list, RingIssue &q,
                                          const RingOrder &ord, uint32_t slots,
                                          const unsigned char *queue, uint32_t queue_s,
                                          int *valid, int lane) {
    if (q.ti < list.total_copy) {
        if (lane == 0)
            *valid = 1;
        ring_issue<U, PATHS>(q.c, q.w, slots, lane);
        q.idx0 += 32 * U;
        if (q.idx0 >= q.c.total) { // on to the warp's next tile
            ++q.j;
            q.ti = tile_of(ord, q.j);
            q.idx0 = 0;
            if (q.ti < list.total_copy) {
                ring_tile_init(q.c, *reinterpret_cast<const Tile *>(
                                        queue + (q.j & (RING_Q - 1)) * RING_QE));
                ring_walk_init(q.w, q.c, lane);
                ring_prefetch_tile<U>(q.c, ord, lane);
                ring_queue_fetch(list, tile_of(ord, q.j + RING_LA),
                                 queue_s + (uint32_t)(((q.j + RING_LA) & (RING_Q - 1)) * RING_QE),
                                 lane);
                const long long pf = tile_of(ord, q.j + RING_LA + 2);
                if (lane == 0 && pf < list.total_copy) {
                    const PairInfo *unused;
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(locate_copy(list, pf, unused)));
                }
            }
        }
    } else if (lane == 0) {
        *valid = 0;
    }
    cp_async_commit();
}

template <int U, int PATHS>
__device__ __forceinline__ void ring_copy_phase(const PlanList &list, unsigned char *smem,
                                                int warp, int nwarp, int ring_opts) {
    constexpr bool SC = (PATHS & PATH_SCALED) != 0;
    constexpr bool CC = (PATHS & PATH_CAST) != 0;
    constexpr int XR = ring_extra_rows(PATHS);
    constexpr int SLOT_BYTES = ring_stage_bytes<U, XR>();
    const int lane = threadIdx.x & 31;
    unsigned char *wbase = smem + (size_t)warp * ring_warp_bytes<U, XR>();
    unsigned char *queue = wbase + RING_D * SLOT_BYTES;
    int *valid = reinterpret_cast<int *>(queue + RING_Q * RING_QE);
    const uint32_t slots0 = smem_addr(wbase);
    const uint32_t queue_s = smem_addr(queue);
    const long long GW = (long long)gridDim.x * nwarp;
    RingOrder ord;
    const int run_shift = ring_opts & RING_OPT_RUN_MASK;
    ord.shift = run_shift;
    ord.l2_prefetch = ring_opts & RING_OPT_L2_PREFETCH;
    ord.base = ((long long)blockIdx.x * nwarp + warp) << run_shift;
    ord.stride = GW << run_shift;
    RingIssue q;
    q.j = 0;
    q.ti = tile_of(ord, 0);
    q.idx0 = 0;
    // descriptors of the first RING_LA + 1 tiles, landed before the first fill
#pragma unroll
    for (int k = 0; k <= RING_LA; ++k)
        ring_queue_fetch(list, tile_of(ord, k), queue_s + (uint32_t)(k * RING_QE), lane);
    cp_async_commit();
    if (lane < 2) {
        const long long pf = tile_of(ord, RING_LA + 1 + lane);
        if (pf < list.total_copy) {
            const PairInfo *unused;
            asm volatile("prefetch.global.L2 [%0];" ::"l"(locate_copy(list, pf, unused)));
        }
    }
    cp_async_wait<0>();
    __syncwarp();
    if (q.ti < list.total_copy) {
        ring_tile_init(q.c, *reinterpret_cast<const Tile *>(queue));
        ring_walk_init(q.w, q.c, lane);
        ring_prefetch_tile<U>(q.c, ord, lane);
    }
#pragma unroll
    for (int st = 0; st < RING_D - 1; ++st)
        ring_fill<U, PATHS>(list, q, ord, slots0 + (uint32_t)(st * SLOT_BYTES), queue,
                            queue_s, valid + st, lane);
    // the storing side: its tile ordinal, walk constants and position
    int js = -1;
    RingTile c;
    RingWalk w;
    int idx0 = 0;
    c.total = 0;
    const PairInfo *pp = nullptr; // the scaled tile's pair (SC kernels)
    int sp = 0; // stage to store; the stage before it is filled next
    for (;;) {
        const int sf = sp == 0 ? RING_D - 1 : sp - 1;
        ring_fill<U, PATHS>(list, q, ord, slots0 + (uint32_t)(sf * SLOT_BYTES), queue,
                            queue_s, valid + sf, lane);
        cp_async_wait<RING_D - 1>();
        __syncwarp();
        if (!valid[sp]) // stages are filled in order: nothing after this
            break;
        if (idx0 >= c.total) { // the stage starts the next tile
            ++js;
            ring_tile_init(c, *reinterpret_cast<const Tile *>(
                                  queue + (js & (RING_Q - 1)) * RING_QE));
            ring_walk_init(w, c, lane);
            idx0 = 0;
            if (SC && (c.kind & KIND_SCALED)) {
                const PairInfo *pairs;
                locate_copy(list, tile_of(ord, js), pairs);
                pp = pairs + c.pair;
            }
        }
        if (SC && (c.kind & KIND_SCALED))
            ring_store_scaled_dispatch<U, PATHS>(c, w, slots0 + (uint32_t)(sp * SLOT_BYTES),
                                                 lane, pp);
        else if (CC && (c.kind & KIND_CAST))
            ring_store_cast_dispatch<U>(c, w, slots0 + (uint32_t)(sp * SLOT_BYTES), lane);
        else
            ring_store<U>(c, w, slots0 + (uint32_t)(sp * SLOT_BYTES), lane);
        idx0 += 32 * U;
        __syncwarp();
        sp = sp + 1 == RING_D ? 0 : sp + 1;
    }
    cp_async_wait<0>();
}

// Registers: the ring kernel runs 16 warps per SM on copy-only plans (one
// 512-thread CTA, or two of 256), 24 with CTA-level tiles (three of 256).
template <int THREADS, int PATHS> struct RingMinBlocks {
    static constexpr int value = (PATHS & (PATH_SCALED_COMPLEX | PATH_CAST))
                                     ? ((512 / THREADS) > 0 ? (512 / THREADS) : 1)
                                     : ((768 / THREADS) > 0 ? (768 / THREADS) : 1);
};

template <int THREADS, int U, int PATHS>
__global__ void __launch_bounds__(THREADS, (RingMinBlocks<THREADS, PATHS>::value))
    scatter_ring_kernel(const __grid_constant__ PlanList list, int td, int ring_opts) {
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr int NWARP = THREADS / 32;
    ring_copy_phase<U, PATHS>(list, smem, threadIdx.x >> 5, NWARP, ring_opts);
    if (PATHS & (PATH_TRANSPOSE | PATH_SCALED | PATH_CAST)) {
        __syncthreads(); // the ring's shared memory becomes the CTA tiles'
        cta_phase<THREADS, PATHS>(list, smem, td);
    }
}

// The staged variant: a ring of S shared-memory stages filled by TMA bulk
// copies (see issue_stage / consume_stage); tiles that are not eligible for
// staging (short columns, scaled, cast) run on the register path in the same
// loop, CTA-level tiles after it. Every wait is bounded: on expiry the CTA records the error in
// *status, waits (bounded) for its other stages and returns.
constexpr uint64_t STAGE_WAIT_LIMIT_NS = 2000000000ull; // 2 s

template <int THREADS, int U, int PATHS, int S>
__global__ void __launch_bounds__(THREADS, 1)
    scatter_staged_kernel(const __grid_constant__ PlanList list, int td, int stage_bytes) {
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    unsigned char *stages = smem + 128;
    unsigned char *direct = stages + (size_t)S * (size_t)stage_bytes;
    const long long n = list.total_copy;
    int *status = list.status;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        for (int k = 0; k < S; ++k)
            mbar_init(smem_addr(&bars[k]), 1);
        mbar_fence_init();
    }
    __syncthreads();
    const long long G = gridDim.x;
    if (warp == 0)
        for (int k = 0; k < S; ++k)
            issue_stage(list, blockIdx.x + k * G, n, stages + (size_t)k * stage_bytes,
                        smem_addr(&bars[k]), stage_bytes);
    uint32_t phase = 0;
    int st = 0;
    for (long long ti = blockIdx.x; ti < n; ti += G) {
        const PairInfo *pairs;
        const Tile t = *locate_copy(list, ti, pairs);
        unsigned char *stage = stages + (size_t)st * stage_bytes;
        const uint32_t bar = smem_addr(&bars[st]);
        if ((PATHS & PATH_COPY) && tma_eligible(t, stage_bytes)) {
            const bool ok = mbar_wait_bounded(bar, (phase >> st) & 1u, STAGE_WAIT_LIMIT_NS);
            if (!__syncthreads_and(ok)) {
                if (threadIdx.x == 0) {
                    atomicExch(status, 1);
                    for (int k = 0; k < S; ++k)
                        mbar_wait_bounded(smem_addr(&bars[k]), (phase >> k) & 1u,
                                          STAGE_WAIT_LIMIT_NS / 4);
                }
                __syncthreads();
                return;
            }
            phase ^= 1u << st;
            consume_stage<THREADS, U>(t, stage);
        } else {
            warp_tile<THREADS / 32, U, PATHS>(t, warp, pairs);
        }
        __syncthreads(); // the stage is free again
        if (warp == 0)
            issue_stage(list, ti + (long long)S * G, n, stage, bar, stage_bytes);
        st = (st + 1 == S) ? 0 : st + 1;
    }
    if (PATHS & (PATH_TRANSPOSE | PATH_SCALED | PATH_CAST))
        cta_phase<THREADS, PATHS>(list, direct, td);
}

template <typename K>
cudaError_t prepare(K k, const ScatterConfig &cfg, size_t smem, long long total,
                    unsigned &grid_out) {
    int occ = 0;
    cudaError_t e = kernel_occupancy((const void *)k, cfg.threads, smem, &occ);
    if (e != cudaSuccess)
        return e;
    if (occ < 1)
        return cudaErrorInvalidConfiguration;
    // a persistent grid must be resident at once (static striding)
    long long grid = cfg.grid;
    const long long resident = (long long)cfg.sm_count * occ;
    if (cfg.sm_count > 0 && grid > resident)
        grid = resident;
    if (grid > total)
        grid = total;
    grid_out = (unsigned)(grid < 1 ? 1 : grid);
    return cudaSuccess;
}

template <int THREADS, int U, int PATHS, int S>
cudaError_t launch_staged(const PlanList &list, const ScatterConfig &cfg, cudaStream_t s) {
    auto k = scatter_staged_kernel<THREADS, U, PATHS, S>;
    const size_t smem = staged_smem_bytes(cfg);
    unsigned grid = 0;
    cudaError_t e = prepare(k, cfg, smem, list.total_copy + list.total_cta, grid);
    if (e != cudaSuccess || cfg.dry_run)
        return e;
    k<<<grid, THREADS, smem, s>>>(list, cfg.tile_dim, cfg.stage_bytes);
    return cudaGetLastError();
}

template <int THREADS, int U, int PATHS>
cudaError_t launch_ring(const PlanList &list, const ScatterConfig &cfg, cudaStream_t s) {
    auto k = scatter_ring_kernel<THREADS, U, PATHS>;
    const size_t smem = ring_smem_bytes(cfg);
    unsigned grid = 0;
    cudaError_t e = prepare(k, cfg, smem, list.total_copy + list.total_cta, grid);
    if (e != cudaSuccess || cfg.dry_run)
        return e;
    k<<<grid, THREADS, smem, s>>>(list, cfg.tile_dim,
                                  cfg.run_shift | (cfg.l2_prefetch ? RING_OPT_L2_PREFETCH : 0));
    return cudaGetLastError();
}

template <int THREADS, int U, int PATHS>
cudaError_t launch_t(const PlanList &list, const ScatterConfig &cfg, cudaStream_t s) {
    if constexpr ((PATHS & PATH_COPY) != 0) {
        if (cfg.ring && cfg.stages < 2)
            return launch_ring<THREADS, U, PATHS>(list, cfg, s);
        if (cfg.stages >= 2) {
            switch (cfg.stages) {
            case 2: return launch_staged<THREADS, U, PATHS, 2>(list, cfg, s);
            case 3: return launch_staged<THREADS, U, PATHS, 3>(list, cfg, s);
            default: return launch_staged<THREADS, U, PATHS, 4>(list, cfg, s);
            }
        }
    }
    auto k = scatter_kernel<THREADS, U, PATHS>;
    unsigned grid = 0;
    cudaError_t e = prepare(k, cfg, cfg.smem_bytes, list.total_copy + list.total_cta, grid);
    if (e != cudaSuccess || cfg.dry_run)
        return e;
    k<<<grid, THREADS, cfg.smem_bytes, s>>>(list, cfg.tile_dim);
    return cudaGetLastError();
}

template <int THREADS, int PATHS>
cudaError_t launch_u(const PlanList &l, const ScatterConfig &cfg, cudaStream_t s) {
    switch (cfg.unroll) {
    case 1: return launch_t<THREADS, 1, PATHS>(l, cfg, s);
    case 2: return launch_t<THREADS, 2, PATHS>(l, cfg, s);
    default: return launch_t<THREADS, 4, PATHS>(l, cfg, s);
    }
}

// Plans with plain copies and transposes only.
template <int THREADS>
cudaError_t launch_plain_paths(const PlanList &l, const ScatterConfig &cfg, cudaStream_t s) {
    if (cfg.paths == PATH_COPY)
        return launch_u<THREADS, PATH_COPY>(l, cfg, s);
    // transposes of 4- or 8-byte elements only: the staged ring (no copy
    // tiles, so the unroll knob has nothing to act on)
    if ((cfg.paths & ~(PATH_W4_STAGED | PATH_NARROW_TRANSPOSE)) == PATH_TRANSPOSE &&
        (cfg.paths & PATH_W4_STAGED))
        return launch_t<THREADS, 1, PATH_TRANSPOSE | PATH_NARROW_TRANSPOSE | PATH_W4_STAGED>(
            l, cfg, s);
    if ((cfg.paths & ~(PATH_W8_STAGED | PATH_NARROW_TRANSPOSE)) == PATH_TRANSPOSE &&
        (cfg.paths & PATH_W8_STAGED))
        return launch_t<THREADS, 1, PATH_TRANSPOSE | PATH_NARROW_TRANSPOSE | PATH_W8_STAGED>(
            l, cfg, s);
    if (cfg.paths == (PATH_TRANSPOSE | PATH_W16_STAGED))
        return launch_t<THREADS, 1, PATH_TRANSPOSE | PATH_W16_STAGED>(l, cfg, s);
    const bool narrow = (cfg.paths & PATH_NARROW_TRANSPOSE) != 0;
    // (without copy tiles the unroll knob acts on nothing: one instance)
    if ((cfg.paths & ~PATH_NARROW_TRANSPOSE) == PATH_TRANSPOSE)
        return narrow ? launch_t<THREADS, 1, PATH_TRANSPOSE | PATH_NARROW_TRANSPOSE>(l, cfg, s)
                      : launch_t<THREADS, 1, PATH_TRANSPOSE>(l, cfg, s);
    return narrow ? launch_u<THREADS, PATH_COPY | PATH_TRANSPOSE | PATH_NARROW_TRANSPOSE>(l, cfg, s)
                  : launch_u<THREADS, PATH_COPY | PATH_TRANSPOSE>(l, cfg, s);
}

// Plans with element arithmetic: scaled or cast tiles (and any others).
template <int THREADS>
cudaError_t launch_elem_paths(const PlanList &l, const ScatterConfig &cfg, cudaStream_t s) {
    // scaled transposes of one element size only: the staged ring (no copy
    // tiles, so the unroll knob has nothing to act on)
    if (cfg.paths == (PATH_SCALED_REAL | PATH_W4S_STAGED))
        return launch_t<THREADS, 1, PATH_SCALED_REAL | PATH_W4S_STAGED>(l, cfg, s);
    if ((cfg.paths & PATH_W8S_STAGED) && !(cfg.paths & ~(PATH_SCALED | PATH_W8S_STAGED)))
        return launch_t<THREADS, 1, PATH_SCALED | PATH_W8S_STAGED>(l, cfg, s);
    if (cfg.paths & PATH_CAST) {
        if (cfg.paths & PATH_SCALED) // not generated: cast and scaled plans launch apart
            return cudaErrorNotSupported;
        return launch_u<THREADS, PATH_COPY | PATH_TRANSPOSE | PATH_CAST>(l, cfg, s);
    }
    if (cfg.paths & PATH_SCALED_COMPLEX)
        return launch_u<THREADS, PATH_COPY | PATH_TRANSPOSE | PATH_SCALED>(l, cfg, s);
    return launch_u<THREADS, PATH_COPY | PATH_TRANSPOSE | PATH_SCALED_REAL>(l, cfg, s);
}

} // namespace

} // namespace g2g
