// The C++ interface driven the way kabicm/grid2grid's own test driver
// (examples/scalapack2scalapack.cpp) drives the reference: every rank builds
// its block-cyclic layouts with get_scalapack_grid, fills its buffer with
// initialize_locally, calls grid2grid::transform collectively and checks its
// result with validate -- here with P virtual ranks as threads, device
// buffers, and a gpu_communicator in place of MPI_COMM_WORLD. Also covers
// the 'T' / 'C' overload with alpha/beta, the vector overload through
// transformer<T>, transform_all_ranks, error behaviour, and
// communication_volume / optimal_reordering (what a caller runs before
// relabeling its ranks).
#include <grid2grid/ranks_reordering.hpp>
#include <grid2grid/scalapack_layout.hpp>
#include <grid2grid/transform.hpp>
#include <grid2grid/transformer.hpp>

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <complex>
#include <cstdio>
#include <thread>
#include <vector>

using namespace grid2grid;

static int cantor(int i, int j) {
    const int s = i + j;
    return (s * (s + 1)) / 2 + j;
}

#define CK(x)                                                                           \
    do {                                                                                \
        cudaError_t e = (x);                                                            \
        if (e != cudaSuccess) {                                                         \
            std::printf("CUDA error %s at line %d\n", cudaGetErrorString(e), __LINE__); \
            std::exit(2);                                                               \
        }                                                                               \
    } while (0)

template <typename T> struct device_buffer {
    T *p = nullptr;
    size_t n = 0;
    explicit device_buffer(const std::vector<T> &h) : n(h.size()) {
        CK(cudaMalloc(&p, sizeof(T) * (n ? n : 1)));
        CK(cudaMemcpy(p, h.data(), sizeof(T) * n, cudaMemcpyHostToDevice));
    }
    std::vector<T> host() const {
        std::vector<T> h(n);
        CK(cudaMemcpy(h.data(), p, sizeof(T) * n, cudaMemcpyDeviceToHost));
        return h;
    }
    ~device_buffer() { cudaFree(p); }
};

// scalapack2scalapack: cantor values from a (bm1 x bn1) into a (bm2 x bn2)
// block-cyclic layout on a pm x pn grid; the destination starts as -1.
static bool scalapack2scalapack(int m, int n, int bm1, int bn1, int bm2, int bn2, int pm,
                                int pn) {
    const int P = pm * pn;
    gpu_communicator world(P);
    std::atomic<bool> ok{true};
    auto values = [](int i, int j) { return 1.0 * cantor(i, j); };
    auto rank_main = [&](int rank) {
        scalapack::data_layout l1({m, n}, {bm1, bn1}, {pm, pn}, scalapack::column_major);
        scalapack::data_layout l2({m, n}, {bm2, bn2}, {pm, pn}, scalapack::column_major);
        std::vector<double> b1(scalapack::local_size(rank, l1));
        scalapack::initialize_locally(b1.data(), values, rank, l1);
        std::vector<double> b2(scalapack::local_size(rank, l2), -1.0);
        device_buffer<double> d1(b1), d2(b2);
        grid_layout<double> g1 = get_scalapack_grid(l1, d1.p, rank);
        grid_layout<double> g2 = get_scalapack_grid(l2, d2.p, rank);
        transform(g1, g2, world.comm(rank));
        if (!scalapack::validate(values, d2.host(), rank, l2))
            ok = false;
    };
    std::vector<std::thread> th;
    for (int r = 0; r < P; ++r)
        th.emplace_back(rank_main, r);
    for (auto &t : th)
        t.join();
    std::printf("scalapack2scalapack %dx%d %dx%d->%dx%d on %dx%d: %s\n", m, n, bm1, bn1, bm2,
                bn2, pm, pn, ok ? "ok" : "FAILED");
    return ok;
}

using cd = std::complex<double>;

// final = 0.5 * final + 2 * conj(initial^T) with complex values, and the same
// pair again through transformer<T> next to a plain pair.
static bool conjugate_scaled(int m, int n) {
    const int pm = 2, pn = 3, P = pm * pn;
    gpu_communicator world(P);
    std::atomic<bool> ok{true};
    auto v = [](int i, int j) { return cd(cantor(i, j), i - j); };   // initial (n x m)
    auto w = [](int i, int j) { return cd(i, j); };                  // final before
    auto want = [&](int i, int j) { return 0.5 * w(i, j) + 2.0 * std::conj(v(j, i)); };
    auto rank_main = [&](int rank) {
        scalapack::data_layout li({n, m}, {7, 5}, {pm, pn}, scalapack::row_major);
        scalapack::data_layout lf({m, n}, {4, 9}, {pm, pn}, scalapack::column_major);
        std::vector<cd> bi(scalapack::local_size(rank, li)), bf(scalapack::local_size(rank, lf));
        scalapack::initialize_locally(bi.data(), v, rank, li);
        scalapack::initialize_locally(bf.data(), w, rank, lf);
        device_buffer<cd> di(bi), df(bf), df2(bf), di2(bi), dp(bf);
        grid_layout<cd> gi = get_scalapack_grid(li, di.p, rank);
        grid_layout<cd> gf = get_scalapack_grid(lf, df.p, rank);
        transform(gi, gf, 'C', cd(2.0, 0.0), cd(0.5, 0.0), world.comm(rank));
        // the initial layout is left transposed, as in the reference
        if (!(gi.num_rows() == m && gi.num_cols() == n && gi.blocks.num_blocks() > 0
                  ? gi.blocks.get_block(0).transpose_on_copy
                  : true))
            ok = false;
        if (!scalapack::validate(want, df.host(), rank, lf))
            ok = false;
        // transformer: the same scaled pair plus a plain copy pair
        grid_layout<cd> gi2 = get_scalapack_grid(li, di2.p, rank);
        grid_layout<cd> gf2 = get_scalapack_grid(lf, df2.p, rank);
        scalapack::data_layout lp({n, m}, {3, 8}, {pm, pn}, scalapack::column_major);
        std::vector<cd> bp(scalapack::local_size(rank, lp), cd(-1, -1));
        device_buffer<cd> dpp(bp);
        grid_layout<cd> gsrc = get_scalapack_grid(li, di.p, rank); // untransposed view again
        grid_layout<cd> gp = get_scalapack_grid(lp, dpp.p, rank);
        transformer<cd> tr(world.comm(rank));
        tr.schedule(gi2, gf2, 'C', cd(2.0, 0.0), cd(0.5, 0.0));
        tr.schedule(gsrc, gp);
        tr.transform();
        if (!scalapack::validate(want, df2.host(), rank, lf))
            ok = false;
        if (!scalapack::validate(v, dpp.host(), rank, lp))
            ok = false;
    };
    std::vector<std::thread> th;
    for (int r = 0; r < P; ++r)
        th.emplace_back(rank_main, r);
    for (auto &t : th)
        t.join();
    std::printf("conjugate_scaled %dx%d: %s\n", m, n, ok ? "ok" : "FAILED");
    return ok;
}

// all ranks from one thread, float, and the error behaviour
static bool all_ranks_and_errors() {
    const int m = 97, n = 61, pm = 3, pn = 2, P = 6;
    scalapack::data_layout l1({m, n}, {8, 16}, {pm, pn}, scalapack::column_major);
    scalapack::data_layout l2({m, n}, {32, 5}, {pm, pn}, scalapack::row_major);
    auto values = [](int i, int j) { return (float)cantor(i, j); };
    std::vector<std::unique_ptr<device_buffer<float>>> d1, d2;
    std::vector<grid_layout<float>> g1, g2;
    for (int r = 0; r < P; ++r) {
        std::vector<float> b1(scalapack::local_size(r, l1)), b2(scalapack::local_size(r, l2), -1);
        scalapack::initialize_locally(b1.data(), values, r, l1);
        d1.emplace_back(new device_buffer<float>(b1));
        d2.emplace_back(new device_buffer<float>(b2));
        g1.push_back(get_scalapack_grid(l1, d1.back()->p, r));
        g2.push_back(get_scalapack_grid(l2, d2.back()->p, r));
    }
    transform_all_ranks(g1, g2);
    bool ok = true;
    for (int r = 0; r < P; ++r)
        ok = ok && scalapack::validate(values, d2[r]->host(), r, l2);
    // a final layout of another shape must throw on every rank, not hang
    scalapack::data_layout bad({m + 1, n}, {32, 5}, {pm, pn}, scalapack::row_major);
    gpu_communicator world(P);
    std::atomic<int> thrown{0};
    std::vector<std::thread> th;
    for (int r = 0; r < P; ++r)
        th.emplace_back([&, r] {
            std::vector<float> hb(scalapack::local_size(r, bad));
            device_buffer<float> db(hb);
            grid_layout<float> gb = get_scalapack_grid(bad, db.p, r);
            try {
                transform(g1[r], gb, world.comm(r));
            } catch (const std::runtime_error &e) {
                if (std::string(e.what()).find("different matrices") != std::string::npos)
                    ++thrown;
            }
        });
    for (auto &t : th)
        t.join();
    ok = ok && thrown == P;
    std::printf("all_ranks_and_errors: %s (%d ranks threw)\n", ok ? "ok" : "FAILED",
                thrown.load());
    return ok;
}

// communication_volume covers every element once; the relabeling from
// optimal_reordering keeps at least as much local as the identity.
static bool reordering_volume(int m, int n) {
    const int P = 6;
    scalapack::data_layout l1({m, n}, {40, 30}, {2, 3}, scalapack::column_major);
    scalapack::data_layout l2({m, n}, {25, 70}, {3, 2}, scalapack::row_major);
    std::vector<double> dummy(1);
    grid_layout<double> a = get_scalapack_grid(l1, dummy.data(), 0);
    grid_layout<double> b = get_scalapack_grid(l2, dummy.data(), 0);
    comm_volume v = communication_volume(a.grid, b.grid);
    long long all = 0, local = 0;
    for (const auto &kv : v.volume) {
        all += kv.second;
        if (kv.first.src == kv.first.dest)
            local += kv.second;
    }
    bool re = false;
    std::vector<int> perm = optimal_reordering(v, P, re);
    b.reorder_ranks(perm);
    comm_volume v2 = communication_volume(a.grid, b.grid);
    long long local2 = 0;
    for (const auto &kv : v2.volume)
        if (kv.first.src == kv.first.dest)
            local2 += kv.second;
    std::vector<int> sorted = perm;
    std::sort(sorted.begin(), sorted.end());
    bool ok = all == (long long)m * n && local2 >= local;
    for (int r = 0; r < P; ++r)
        ok = ok && sorted[r] == r;
    std::printf("reordering_volume %dx%d: %s (local %lld -> %lld of %lld, reordered %d)\n", m, n,
                ok ? "ok" : "FAILED", local, local2, all, (int)re);
    return ok;
}

int main() {
    bool ok = true;
    // the reference's four ctest cases (examples/CMakeLists.txt:20-30)
    ok &= scalapack2scalapack(10, 10, 2, 2, 5, 5, 2, 2);
    ok &= scalapack2scalapack(10, 10, 2, 3, 3, 5, 2, 2);
    ok &= scalapack2scalapack(10, 12, 2, 3, 2, 6, 2, 2);
    ok &= scalapack2scalapack(10, 12, 2, 3, 3, 5, 2, 2);
    // larger, uneven process grids
    ok &= scalapack2scalapack(1000, 777, 32, 17, 100, 61, 3, 4);
    ok &= conjugate_scaled(150, 83);
    ok &= all_ranks_and_errors();
    ok &= reordering_volume(600, 500);
    std::printf(ok ? "ALL OK\n" : "SOME FAILED\n");
    return ok ? 0 : 1;
}
