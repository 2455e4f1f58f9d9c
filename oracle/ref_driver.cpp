// Reference driver -- TEST INFRASTRUCTURE ONLY (part of the oracle).
//
// Runs the UNMODIFIED reference library (kabicm/grid2grid, compiled from its
// own src/grid2grid/*.cpp by oracle/Makefile into oracle/_ref/) with its P MPI
// ranks played by P threads over the thread-MPI shim (oracle/mpishim). The
// layouts come in as the product's C descriptors (include/grid2grid_gb300.h)
// whose block pointers are HOST addresses; every thread-rank builds its own
// grid_layout<T> from the blocks tagged with its rank and calls the
// reference's public grid2grid::transform / transformer<T>.
//
// Exposed with C linkage for ctypes (oracle/oracle.py). Only tests and the
// fixture generator in tests/golden/ load the resulting library.
#include <grid2grid/grid_cover.hpp>
#include <grid2grid/scalapack_layout.hpp>
#include <grid2grid/transform.hpp>
#include <grid2grid/ranks_reordering.hpp>
#include <grid2grid/transformer.hpp>

#include "../include/grid2grid_gb300.h"
#include "mpishim/mpi.h"

#include <complex>
#include <cstring>
#include <exception>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace {

std::string g_error;
std::mutex g_error_mu;

void set_error(const std::string &s) {
    std::lock_guard<std::mutex> lk(g_error_mu);
    if (g_error.empty())
        g_error = s;
}

template <typename T> T make_scalar(const double *v);
template <> float make_scalar<float>(const double *v) { return (float)v[0]; }
template <> double make_scalar<double>(const double *v) { return v[0]; }
template <> std::complex<float> make_scalar<std::complex<float>>(const double *v) {
    return std::complex<float>((float)v[0], (float)v[1]);
}
template <> std::complex<double> make_scalar<std::complex<double>>(const double *v) {
    return std::complex<double>(v[0], v[1]);
}

// Builds rank `rank`'s grid_layout<T> from a descriptor holding all ranks.
template <typename T>
grid2grid::grid_layout<T> build_layout(const g2g_layout_desc &d, int rank) {
    std::vector<int> rs(d.rows_split, d.rows_split + d.n_block_rows + 1);
    std::vector<int> cs(d.cols_split, d.cols_split + d.n_block_cols + 1);
    std::vector<std::vector<int>> owners(d.n_block_rows,
                                         std::vector<int>(d.n_block_cols));
    for (int i = 0; i < d.n_block_rows; ++i)
        for (int j = 0; j < d.n_block_cols; ++j)
            owners[i][j] = d.owners[(size_t)i * d.n_block_cols + j];
    grid2grid::grid2D g(std::move(rs), std::move(cs));
    grid2grid::assigned_grid2D ag(std::move(g), std::move(owners), d.n_ranks);

    std::vector<grid2grid::block<T>> blocks;
    for (int b = 0; b < d.n_blocks; ++b) {
        const g2g_block_desc &bd = d.blocks[b];
        if (bd.rank != rank)
            continue;
        // Intervals in the layout's current coordinates are the grid's
        // intervals at (row, col); storage follows block.hpp:60-146.
        grid2grid::interval ri(d.rows_split[bd.row], d.rows_split[bd.row + 1]);
        grid2grid::interval ci(d.cols_split[bd.col], d.cols_split[bd.col + 1]);
        grid2grid::block<T> blk(ri, ci, grid2grid::block_coordinates(bd.row, bd.col),
                                (T *)bd.data, (int)bd.stride);
        blk.transpose_on_copy = bd.transpose_on_copy != 0;
        blk.conjugate_on_copy = bd.conjugate_on_copy != 0;
        blocks.push_back(blk);
    }
    grid2grid::local_blocks<T> lb(std::move(blocks));
    grid2grid::grid_layout<T> layout(std::move(ag), std::move(lb));
    if (d.n_reordering > 0) {
        std::vector<int> reo(d.reordering, d.reordering + d.n_reordering);
        layout.reorder_ranks(reo);
    }
    return layout;
}

// mode: 0 plain single overload per pair; 1 scaled single overload per pair;
//       2 plain vector overload; 3 scaled vector overload; 4 transformer<T>.
template <typename T>
int run_transform(int n_pairs, const g2g_layout_desc *inits,
                  const g2g_layout_desc *finals, const g2g_op *ops, int mode) {
    int P = 1;
    for (int k = 0; k < n_pairs; ++k) {
        P = std::max(P, inits[k].n_ranks);
        P = std::max(P, finals[k].n_ranks);
    }
    tmpi_world *world = tmpi_world_create(P);
    int rc = 0;
    auto body = [&](int rank) {
        try {
            MPI_Comm comm = tmpi_comm(world, rank);
            std::vector<grid2grid::grid_layout<T>> from, to;
            from.reserve(n_pairs);
            to.reserve(n_pairs);
            for (int k = 0; k < n_pairs; ++k) {
                from.push_back(build_layout<T>(inits[k], rank));
                to.push_back(build_layout<T>(finals[k], rank));
            }
            std::vector<char> trans(n_pairs, 'N');
            std::vector<T> alpha(n_pairs, T{1}), beta(n_pairs, T{0});
            if (ops) {
                for (int k = 0; k < n_pairs; ++k) {
                    trans[k] = ops[k].trans;
                    alpha[k] = make_scalar<T>(ops[k].alpha);
                    beta[k] = make_scalar<T>(ops[k].beta);
                }
            }
            if (mode == 0) {
                for (int k = 0; k < n_pairs; ++k)
                    grid2grid::transform<T>(from[k], to[k], comm);
            } else if (mode == 1) {
                for (int k = 0; k < n_pairs; ++k)
                    grid2grid::transform<T>(from[k], to[k], trans[k], alpha[k],
                                            beta[k], comm);
            } else if (mode == 2 || mode == 3) {
                std::vector<grid2grid::layout_ref<T>> f, t;
                for (int k = 0; k < n_pairs; ++k) {
                    f.push_back(from[k]);
                    t.push_back(to[k]);
                }
                if (mode == 2)
                    grid2grid::transform<T>(f, t, comm);
                else
                    grid2grid::transform<T>(f, t, trans.data(), alpha.data(),
                                            beta.data(), comm);
            } else {
                grid2grid::transformer<T> tr(comm);
                for (int k = 0; k < n_pairs; ++k)
                    tr.schedule(from[k], to[k], trans[k], alpha[k], beta[k]);
                tr.transform();
            }
        } catch (const std::exception &e) {
            set_error(std::string("rank ") + std::to_string(rank) + ": " + e.what());
        }
    };
    std::vector<std::thread> threads;
    for (int r = 0; r < P; ++r)
        threads.emplace_back(body, r);
    for (auto &t : threads)
        t.join();
    if (tmpi_world_pending_bytes(world) != 0) {
        set_error("unreceived messages left in the thread-MPI mailboxes");
        rc = 2;
    }
    tmpi_world_destroy(world);
    if (!g_error.empty())
        rc = rc ? rc : 1;
    return rc;
}

} // namespace

extern "C" {

const char *g2g_ref_last_error(void) { return g_error.c_str(); }

// Runs the reference transform over thread-ranks; returns 0 on success.
int g2g_ref_transform(int dtype, int n_pairs, const g2g_layout_desc *inits,
                      const g2g_layout_desc *finals, const g2g_op *ops, int mode) {
    g_error.clear();
    switch (dtype) {
    case G2G_FLOAT32:
        return run_transform<float>(n_pairs, inits, finals, ops, mode);
    case G2G_FLOAT64:
        return run_transform<double>(n_pairs, inits, finals, ops, mode);
    case G2G_COMPLEX64:
        return run_transform<std::complex<float>>(n_pairs, inits, finals, ops, mode);
    case G2G_COMPLEX128:
        return run_transform<std::complex<double>>(n_pairs, inits, finals, ops, mode);
    default:
        set_error("bad dtype");
        return 1;
    }
}

// grid2grid::get_decomp_cover (grid_cover.cpp:54-121) on host arrays.
int g2g_ref_decomp_cover(const int *a, int na, const int *b, int nb, int *start,
                         int *end) {
    std::vector<int> va(a, a + na), vb(b, b + nb);
    std::vector<grid2grid::interval_cover> c = grid2grid::get_decomp_cover(va, vb);
    for (size_t k = 0; k < c.size(); ++k) {
        start[k] = c[k].start_index;
        end[k] = c[k].end_index;
    }
    return (int)c.size();
}

// Full get_scalapack_grid (scalapack_layout.cpp:178-278) for one rank with a
// null base pointer; block pointers come back as element offsets.
// ij is 1-based like the reference. Returns the number of local blocks, or -1
// if a capacity is too small.
int g2g_ref_scalapack_grid(int lld, int m, int n, int i1, int j1, int sub_m,
                           int sub_n, int mb, int nb, int pr, int pc,
                           int row_major, int src_r, int src_c, int rank,
                           int cap, int *rows_split, int *n_rs, int *cols_split,
                           int *n_cs, int *owners, int *n_ranks, int *blk_row,
                           int *blk_col, long long *blk_offset, int *blk_stride) {
    using namespace grid2grid;
    double *base = nullptr;
    grid_layout<double> L = get_scalapack_grid<double>(
        lld, scalapack::matrix_dim{m, n}, scalapack::elem_grid_coord{i1, j1},
        scalapack::matrix_dim{sub_m, sub_n}, scalapack::block_dim{mb, nb},
        scalapack::rank_decomposition{pr, pc},
        row_major ? scalapack::ordering::row_major : scalapack::ordering::column_major,
        scalapack::rank_grid_coord{src_r, src_c}, base, rank);
    const grid2D &g = L.grid.grid();
    if ((int)g.rows_split.size() > cap || (int)g.cols_split.size() > cap ||
        L.blocks.num_blocks() > cap ||
        (long long)g.n_rows * g.n_cols > (long long)cap)
        return -1;
    *n_rs = (int)g.rows_split.size();
    *n_cs = (int)g.cols_split.size();
    for (size_t i = 0; i < g.rows_split.size(); ++i)
        rows_split[i] = g.rows_split[i];
    for (size_t j = 0; j < g.cols_split.size(); ++j)
        cols_split[j] = g.cols_split[j];
    for (int i = 0; i < g.n_rows; ++i)
        for (int j = 0; j < g.n_cols; ++j)
            owners[i * g.n_cols + j] = L.grid.owner(i, j);
    *n_ranks = L.num_ranks();
    for (int b = 0; b < L.blocks.num_blocks(); ++b) {
        const block<double> &blk = L.blocks.get_block(b);
        blk_row[b] = blk.coordinates.row;
        blk_col[b] = blk.coordinates.col;
        blk_offset[b] = (long long)(blk.data - base);
        blk_stride[b] = blk.stride;
    }
    return L.blocks.num_blocks();
}

// Simple get_scalapack_grid overload (scalapack_layout.cpp:305-335) and
// scalapack::local_size (:141-149); same outputs as above.
int g2g_ref_scalapack_grid_simple(int m, int n, int mb, int nb, int pr, int pc,
                                  int row_major, int rank, int cap,
                                  int *rows_split, int *n_rs, int *cols_split,
                                  int *n_cs, int *owners, int *n_ranks,
                                  int *blk_row, int *blk_col,
                                  long long *blk_offset, int *blk_stride,
                                  long long *local_size) {
    using namespace grid2grid;
    scalapack::data_layout dl(scalapack::matrix_dim{m, n}, scalapack::block_dim{mb, nb},
                              scalapack::rank_decomposition{pr, pc},
                              row_major ? scalapack::ordering::row_major
                                        : scalapack::ordering::column_major);
    *local_size = (long long)scalapack::local_size(rank, dl);
    double *base = nullptr;
    grid_layout<double> L = get_scalapack_grid<double>(dl, base, rank);
    const grid2D &g = L.grid.grid();
    if ((int)g.rows_split.size() > cap || (int)g.cols_split.size() > cap ||
        L.blocks.num_blocks() > cap ||
        (long long)g.n_rows * g.n_cols > (long long)cap)
        return -1;
    *n_rs = (int)g.rows_split.size();
    *n_cs = (int)g.cols_split.size();
    for (size_t i = 0; i < g.rows_split.size(); ++i)
        rows_split[i] = g.rows_split[i];
    for (size_t j = 0; j < g.cols_split.size(); ++j)
        cols_split[j] = g.cols_split[j];
    for (int i = 0; i < g.n_rows; ++i)
        for (int j = 0; j < g.n_cols; ++j)
            owners[i * g.n_cols + j] = L.grid.owner(i, j);
    *n_ranks = L.num_ranks();
    for (int b = 0; b < L.blocks.num_blocks(); ++b) {
        const block<double> &blk = L.blocks.get_block(b);
        blk_row[b] = blk.coordinates.row;
        blk_col[b] = blk.coordinates.col;
        blk_offset[b] = (long long)(blk.data - base);
        blk_stride[b] = blk.stride;
    }
    return L.blocks.num_blocks();
}

// scalapack::initialize_locally (scalapack_layout.hpp:299-331) with the
// value function  v(i, j) = i + j * m  (as double) into `buffer` of
// local_size elements; returns the buffer size written.
long long g2g_ref_initialize_locally(double *buffer, int m, int n, int mb, int nb,
                                     int pr, int pc, int row_major, int rank,
                                     int value_kind) {
    using namespace grid2grid;
    scalapack::data_layout dl(scalapack::matrix_dim{m, n}, scalapack::block_dim{mb, nb},
                              scalapack::rank_decomposition{pr, pc},
                              row_major ? scalapack::ordering::row_major
                                        : scalapack::ordering::column_major);
    size_t sz = scalapack::local_size(rank, dl);
    if (value_kind == 0) {
        auto f = [m](int i, int j) { return (double)i + (double)j * (double)m; };
        scalapack::initialize_locally(buffer, f, rank, dl);
    } else {
        // the example's cantor pairing values (cantor_mapping.hpp:14-17),
        // written out here to keep that header's non-inline definitions out
        auto f = [](int i, int j) {
            int s = i + j;
            return 1.0 * ((s * (s + 1)) / 2 + j);
        };
        scalapack::initialize_locally(buffer, f, rank, dl);
    }
    return (long long)sz;
}

// communication_volume and optimal_reordering of the reference on the grids
// of two layouts. volume: P x P row-major, entry [r*P + s] for the edge
// {r, s} (r <= s); perm: P entries. Returns 0, or -1 with the error set.
// presize: 1 = every self entry {r, r} inserted (volume 0) before
// optimal_reordering runs. The reference's loop inserts them itself while it
// iterates the same unordered_map (ranks_reordering.cpp:28-29), so without
// them its result depends on when the map rehashes.
int g2g_ref_comm_volume(const g2g_layout_desc *init, const g2g_layout_desc *fin, int P,
                        long long *volume, int *perm, int *reordered, int presize) {
    g_error.clear();
    try {
        grid2grid::grid_layout<double> li = build_layout<double>(*init, -1);
        grid2grid::grid_layout<double> lf = build_layout<double>(*fin, -1);
        grid2grid::comm_volume cv = grid2grid::communication_volume(li.grid, lf.grid);
        if (presize)
            for (int r = 0; r < P; ++r)
                cv.volume[grid2grid::edge_t{r, r}] += 0;
        for (int k = 0; k < P * P; ++k)
            volume[k] = 0;
        for (const auto &e : cv.volume) {
            if (e.first.src < 0 || e.first.dest >= P || e.first.src >= P)
                throw std::runtime_error("rank outside P");
            volume[(size_t)e.first.src * P + e.first.dest] = e.second;
        }
        bool re = false;
        std::vector<int> p = grid2grid::optimal_reordering(cv, P, re);
        for (int r = 0; r < P; ++r)
            perm[r] = p[r];
        *reordered = re ? 1 : 0;
    } catch (const std::exception &e) {
        set_error(e.what());
        return -1;
    }
    return 0;
}

} // extern "C"
