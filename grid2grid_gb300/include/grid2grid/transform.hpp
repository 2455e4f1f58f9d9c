// grid2grid C++ interface on GB300: the transform.
//
// The four grid2grid::transform overloads of kabicm/grid2grid
// (src/grid2grid/transform.hpp:13-43) with the same argument meaning and
// error behaviour (std::runtime_error), on top of the C ABI of
// include/grid2grid_gb300.h. The MPI communicator becomes a
// gpu_communicator: P virtual ranks whose blocks all live in one GPU's
// memory. Each virtual rank calls transform with its own grid_layout and its
// gpu_comm handle, exactly where the reference calls it with MPI_Comm; the
// calls are collective: the last rank to arrive launches one device
// gather-scatter over every rank's blocks, and all calls return after it
// has completed. A single-threaded caller holding every rank's layout uses
// transform_all_ranks instead.
#pragma once

#include "grid_layout.hpp"

#include <grid2grid_gb300.h>

#include <complex>
#include <condition_variable>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

namespace grid2grid {

namespace detail {

template <typename T> struct dtype_of;
template <> struct dtype_of<float> { static constexpr g2g_dtype value = G2G_FLOAT32; };
template <> struct dtype_of<double> { static constexpr g2g_dtype value = G2G_FLOAT64; };
template <> struct dtype_of<std::complex<float>> {
    static constexpr g2g_dtype value = G2G_COMPLEX64;
};
template <> struct dtype_of<std::complex<double>> {
    static constexpr g2g_dtype value = G2G_COMPLEX128;
};

inline void scalar_parts(float v, double *o) { o[0] = v; o[1] = 0.0; }
inline void scalar_parts(double v, double *o) { o[0] = v; o[1] = 0.0; }
inline void scalar_parts(std::complex<float> v, double *o) { o[0] = v.real(); o[1] = v.imag(); }
inline void scalar_parts(std::complex<double> v, double *o) { o[0] = v.real(); o[1] = v.imag(); }

template <typename T> g2g_op make_op(char trans, T alpha, T beta) {
    g2g_op op;
    std::memset(&op, 0, sizeof(op));
    op.trans = trans;
    scalar_parts(alpha, op.alpha);
    scalar_parts(beta, op.beta);
    return op;
}

// The C descriptor of one layout over all virtual ranks: the grid and owners
// of rank 0's view, every rank's local blocks tagged with the rank.
struct layout_desc {
    std::vector<int32_t> rs, cs, owners, reordering;
    std::vector<g2g_block_desc> blocks;
    g2g_layout_desc d;

    template <typename T> void build(const std::vector<const grid_layout<T> *> &per_rank) {
        const grid_layout<T> &L0 = *per_rank[0];
        const grid2D &g = L0.grid.grid();
        rs.assign(g.rows_split.begin(), g.rows_split.end());
        cs.assign(g.cols_split.begin(), g.cols_split.end());
        owners.clear();
        for (const std::vector<int> &row : L0.grid.ranks())
            owners.insert(owners.end(), row.begin(), row.end());
        reordering.assign(L0.grid.reordering().begin(), L0.grid.reordering().end());
        blocks.clear();
        for (size_t r = 0; r < per_rank.size(); ++r) {
            const local_blocks<T> &lb = per_rank[r]->blocks;
            for (int k = 0; k < lb.num_blocks(); ++k) {
                const block<T> &b = lb.get_block(k);
                g2g_block_desc bd;
                std::memset(&bd, 0, sizeof(bd));
                bd.rank = (int32_t)r;
                bd.row = b.coordinates.row;
                bd.col = b.coordinates.col;
                bd.transpose_on_copy = b.transpose_on_copy;
                bd.conjugate_on_copy = b.conjugate_on_copy;
                bd.stride = b.stride;
                bd.data = (void *)b.data;
                blocks.push_back(bd);
            }
        }
        std::memset(&d, 0, sizeof(d));
        d.n_block_rows = g.n_rows;
        d.n_block_cols = g.n_cols;
        d.rows_split = rs.data();
        d.cols_split = cs.data();
        d.owners = owners.data();
        d.n_ranks = L0.num_ranks();
        d.n_reordering = (int32_t)reordering.size();
        d.reordering = reordering.empty() ? nullptr : reordering.data();
        d.n_blocks = (int32_t)blocks.size();
        d.blocks = blocks.data();
    }
};

inline void check(g2g_status st) {
    if (st != G2G_SUCCESS)
        throw std::runtime_error(std::string("grid2grid (GB300): ") + g2g_last_error_string());
}

// One rank's arguments to a collective transform.
template <typename T> struct call_args {
    std::vector<grid_layout<T> *> from, to;
    std::vector<g2g_op> ops; // empty: plain copies
};

// Runs the transform of every pair over all ranks' contributions.
template <typename T>
void run_collective(const std::vector<const void *> &slots, void *stream) {
    const call_args<T> &a0 = *static_cast<const call_args<T> *>(slots[0]);
    const size_t n_pairs = a0.from.size();
    for (const void *s : slots)
        if (static_cast<const call_args<T> *>(s)->from.size() != n_pairs)
            throw std::runtime_error(
                "grid2grid (GB300): ranks passed different numbers of layouts");
    std::vector<layout_desc> init(n_pairs), fin(n_pairs);
    std::vector<g2g_layout_desc> di(n_pairs), df(n_pairs);
    for (size_t k = 0; k < n_pairs; ++k) {
        std::vector<const grid_layout<T> *> f, t;
        for (const void *s : slots) {
            const call_args<T> &a = *static_cast<const call_args<T> *>(s);
            f.push_back(a.from[k]);
            t.push_back(a.to[k]);
        }
        init[k].build(f);
        fin[k].build(t);
        di[k] = init[k].d;
        df[k] = fin[k].d;
    }
    std::vector<g2g_dtype> dts(n_pairs, dtype_of<T>::value);
    const g2g_op *ops = a0.ops.empty() ? nullptr : a0.ops.data();
    if (n_pairs == 1)
        check(g2g_transform(&di[0], &df[0], dts[0], ops, stream));
    else if (n_pairs > 1)
        check(g2g_transform_batch((int32_t)n_pairs, di.data(), df.data(), dts.data(), ops,
                                  stream));
}

} // namespace detail

class gpu_communicator;

// A virtual rank's handle: what an MPI_Comm is to one MPI rank.
struct gpu_comm {
    gpu_communicator *world = nullptr;
    int rank = 0;
};

// P virtual ranks on the current GPU; transforms run on `stream`
// (a cudaStream_t, NULL = legacy default stream).
class gpu_communicator {
  public:
    explicit gpu_communicator(int n_ranks, void *stream = nullptr)
        : n_(n_ranks), stream_(stream), slots_((size_t)(n_ranks > 0 ? n_ranks : 1), nullptr) {
        if (n_ranks < 1)
            throw std::runtime_error("grid2grid (GB300): a communicator needs >= 1 rank");
    }
    gpu_comm comm(int rank) {
        if (rank < 0 || rank >= n_)
            throw std::runtime_error("grid2grid (GB300): rank outside the communicator");
        return gpu_comm{this, rank};
    }
    int size() const { return n_; }
    void *stream() const { return stream_; }

    // Collective: every rank contributes; the last to arrive runs `run` over
    // all contributions; every rank returns (or throws) with its outcome.
    template <typename Run> void collective(int rank, const void *contribution, Run run) {
        std::unique_lock<std::mutex> lk(mu_);
        const unsigned long gen = generation_;
        slots_[rank] = contribution;
        if (++arrived_ == n_) {
            std::vector<const void *> slots = slots_;
            lk.unlock();
            std::string err;
            try {
                run(slots, stream_);
            } catch (const std::exception &e) {
                err = e.what();
            }
            lk.lock();
            error_ = err;
            arrived_ = 0;
            ++generation_;
            cv_.notify_all();
        } else {
            cv_.wait(lk, [&] { return generation_ != gen; });
        }
        if (!error_.empty())
            throw std::runtime_error(error_);
    }

  private:
    int n_;
    void *stream_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::vector<const void *> slots_;
    int arrived_ = 0;
    unsigned long generation_ = 0;
    std::string error_;
};

inline int comm_rank(gpu_comm c) { return c.rank; }
inline int comm_size(gpu_comm c) { return c.world->size(); }

// final_layout = initial_layout (transform.hpp:13-16).
template <typename T>
void transform(grid_layout<T> &initial_layout, grid_layout<T> &final_layout, gpu_comm comm) {
    detail::call_args<T> a;
    a.from.push_back(&initial_layout);
    a.to.push_back(&final_layout);
    comm.world->collective(comm.rank, &a, detail::run_collective<T>);
}

// final_layout = beta * final_layout + alpha * op(initial_layout), op from
// trans in {N, T, C}; like the reference, the initial layout is left
// transposed (transform.hpp:20-25, transform.cpp:144-164).
template <typename T>
void transform(grid_layout<T> &initial_layout, grid_layout<T> &final_layout, const char trans,
               const T alpha, const T beta, gpu_comm comm) {
    detail::call_args<T> a;
    a.from.push_back(&initial_layout);
    a.to.push_back(&final_layout);
    a.ops.push_back(detail::make_op(trans, alpha, beta));
    comm.world->collective(comm.rank, &a, detail::run_collective<T>);
    initial_layout.transpose_or_conjugate(trans);
}

// final_layouts[i] = initial_layouts[i] for all i, one launch
// (transform.hpp:30-33).
template <typename T>
void transform(std::vector<layout_ref<T>> &initial_layouts,
               std::vector<layout_ref<T>> &final_layouts, gpu_comm comm) {
    if (initial_layouts.size() != final_layouts.size())
        throw std::runtime_error("grid2grid (GB300): layout vectors differ in length");
    detail::call_args<T> a;
    for (size_t k = 0; k < initial_layouts.size(); ++k) {
        a.from.push_back(&initial_layouts[k].get());
        a.to.push_back(&final_layouts[k].get());
    }
    comm.world->collective(comm.rank, &a, detail::run_collective<T>);
}

// final_layouts[i] = beta[i] * final_layouts[i] + alpha[i] * op_i(initial_layouts[i])
// (transform.hpp:38-43).
template <typename T>
void transform(std::vector<layout_ref<T>> &initial_layouts,
               std::vector<layout_ref<T>> &final_layouts, const char *trans, const T *alpha,
               const T *beta, gpu_comm comm) {
    if (initial_layouts.size() != final_layouts.size())
        throw std::runtime_error("grid2grid (GB300): layout vectors differ in length");
    detail::call_args<T> a;
    for (size_t k = 0; k < initial_layouts.size(); ++k) {
        a.from.push_back(&initial_layouts[k].get());
        a.to.push_back(&final_layouts[k].get());
        a.ops.push_back(detail::make_op(trans[k], alpha[k], beta[k]));
    }
    comm.world->collective(comm.rank, &a, detail::run_collective<T>);
    for (size_t k = 0; k < initial_layouts.size(); ++k)
        initial_layouts[k].get().transpose_or_conjugate(trans[k]);
}

// Every rank's layouts from one thread: initial[r] / final[r] is rank r's view.
template <typename T>
void transform_all_ranks(std::vector<grid_layout<T>> &initial, std::vector<grid_layout<T>> &final_,
                         void *stream = nullptr, char trans = 'N', T alpha = T{1},
                         T beta = T{0}) {
    if (initial.size() != final_.size() || initial.empty())
        throw std::runtime_error("grid2grid (GB300): one initial and one final layout per rank");
    std::vector<detail::call_args<T>> args(initial.size());
    std::vector<const void *> slots;
    for (size_t r = 0; r < initial.size(); ++r) {
        args[r].from.push_back(&initial[r]);
        args[r].to.push_back(&final_[r]);
        args[r].ops.push_back(detail::make_op(trans, alpha, beta));
        slots.push_back(&args[r]);
    }
    detail::run_collective<T>(slots, stream);
    for (grid_layout<T> &L : initial)
        L.transpose_or_conjugate(trans);
}

} // namespace grid2grid
