// CPU restatement of grid2grid's transform path -- TEST INFRASTRUCTURE ONLY.
//
// This is the oracle: the checker the GPU path is compared against, and the
// CPU baseline that bench.py times on the host cores. It is never linked into
// the product. It restates, in this project's own code, the reference's
// algorithm (kabicm/grid2grid) step by step over P virtual ranks:
//   grid cover             grid_cover.cpp:54-121
//   block decomposition    utils.hpp:10-89, block.cpp:165-196
//   message ordering       utils.hpp:141-144, communication_data.cpp:26-30,
//                          block.cpp:207-225
//   counts / displacements communication_data.cpp:51-99
//   pack                   communication_data.cpp:101-142,
//                          memory_utils.hpp:41-77,124-184
//   exchange               transform.cpp:41-124 (one copy per peer segment)
//   local copy             communication_data.cpp:197-252
//   unpack (+ scaling)     communication_data.cpp:157-190,
//                          memory_utils.hpp:79-122,186-256
//   transpose_or_conjugate grid_layout.hpp:18-25, grid2D.cpp:107-110,
//                          block.cpp:249-288
// Ranks are processed by a pool of worker threads, phase by phase, the way
// MPI ranks would run on that many cores. Arithmetic for alpha/beta uses the
// element type's own operators (std::complex for complex types), compiled
// with -ffp-contract=off.
#include "../../include/grid2grid_gb300.h"

#include <algorithm>
#include <atomic>
#include <cctype>
#include <complex>
#include <cstring>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

namespace {

std::string g_err;

struct Interval {
    int start = 0, end = 0;
    int length() const { return end - start; }
};

bool operator<(const Interval &a, const Interval &b) {
    return a.start < b.start || (a.start == b.start && a.end < b.end);
}
bool operator==(const Interval &a, const Interval &b) {
    if (a.length() == 0)
        return b.length() == 0;
    return a.start == b.start && a.end == b.end;
}

// One block or piece: current-coordinate intervals; memory holds the
// untransposed block when `trans` is set (block.hpp:60-146).
struct Blk {
    Interval rows, cols;
    unsigned char *data = nullptr;
    int64_t stride = 0;
    bool trans = false, conj = false;
    int tag = 0;
    int row_coord = 0, col_coord = 0;
    int64_t size() const { return (int64_t)rows.length() * cols.length(); }
};

struct Layout {
    std::vector<int> rs, cs;          // splits
    std::vector<int> owners;          // row-major
    std::vector<int> reordering;
    int n_ranks = 0;
    std::vector<std::vector<Blk>> local; // per rank
    int nbr() const { return (int)rs.size() - 1; }
    int nbc() const { return (int)cs.size() - 1; }
    int owner(int i, int j) const {
        int r = owners[(size_t)i * nbc() + j];
        return reordering.empty() ? r : reordering[r];
    }
};

// The cover of one split vector by another: for every interval k of `a`,
// [start, end) indexes the intervals of `b` it overlaps, with
// start = max i: b[i] <= a[k] and end = min i: b[i] >= a[k+1]
// (grid_cover.cpp:54-121 computes the same in one merge pass).
void decomp_cover(const std::vector<int> &a, const std::vector<int> &b,
                  std::vector<std::pair<int, int>> &out) {
    out.clear();
    int nb = (int)b.size();
    int lo = 0, hi = 0;
    for (size_t k = 0; k + 1 < a.size(); ++k) {
        while (lo + 1 < nb && b[lo + 1] <= a[k])
            ++lo;
        if (hi < lo)
            hi = lo;
        while (hi < nb - 1 && b[hi] < a[k + 1])
            ++hi;
        out.push_back({lo, hi});
    }
}

// block<T>::subblock (block.cpp:165-196): a sub-rectangle given in current
// coordinates; the pointer is computed in storage coordinates.
Blk subblock(const Blk &b, Interval r, Interval c, int esz) {
    Interval rr = r, cr = c, rb = b.rows, cb = b.cols;
    if (b.trans) {
        std::swap(rr, cr);
        std::swap(rb, cb);
    }
    Blk s = b;
    s.rows = r;
    s.cols = c;
    s.data = b.data + ((int64_t)(cr.start - cb.start) * b.stride +
                       (rr.start - rb.start)) * esz;
    return s;
}

struct Msg {
    Blk b;
    int peer;
};

bool msg_less(const Msg &x, const Msg &y) {
    // (peer, cols, rows, tag): communication_data.cpp:26-30, block.cpp:207-225
    if (x.peer != y.peer)
        return x.peer < y.peer;
    if (!(x.b.cols == y.b.cols))
        return x.b.cols < y.b.cols;
    if (!(x.b.rows == y.b.rows))
        return x.b.rows < y.b.rows;
    return x.b.tag < y.b.tag;
}

// Decompose every local block of `from` over the grid of `over`, tagging each
// piece with the owner (in `over`) of the covering block (utils.hpp:10-89).
void decompose(const std::vector<Blk> &blocks, const Layout &from,
               const Layout &over, int esz, std::vector<Msg> &out) {
    std::vector<std::pair<int, int>> rc, cc;
    decomp_cover(from.rs, over.rs, rc);
    decomp_cover(from.cs, over.cs, cc);
    for (const Blk &b : blocks) {
        int rf = rc[b.row_coord].first, rl = rc[b.row_coord].second;
        int cf = cc[b.col_coord].first, cl = cc[b.col_coord].second;
        int row_start = b.rows.start;
        for (int i = rf; i < rl; ++i) {
            int row_end = std::min(over.rs[i + 1], b.rows.end);
            int col_start = b.cols.start;
            for (int j = cf; j < cl; ++j) {
                int col_end = std::min(over.cs[j + 1], b.cols.end);
                Blk s = subblock(b, {row_start, row_end}, {col_start, col_end}, esz);
                if (s.rows.length() > 0 && s.cols.length() > 0)
                    out.push_back({s, over.owner(i, j)});
                col_start = col_end;
            }
            row_start = row_end;
        }
    }
}

template <typename T> T scalar_of(const double *v);
template <> float scalar_of<float>(const double *v) { return (float)v[0]; }
template <> double scalar_of<double>(const double *v) { return v[0]; }
template <> std::complex<float> scalar_of<std::complex<float>>(const double *v) {
    return {(float)v[0], (float)v[1]};
}
template <> std::complex<double> scalar_of<std::complex<double>>(const double *v) {
    return {v[0], v[1]};
}

template <typename T> T conj_of(T x) { return x; }
template <> std::complex<float> conj_of(std::complex<float> x) { return std::conj(x); }
template <> std::complex<double> conj_of(std::complex<double> x) { return std::conj(x); }

// Copy piece `s` (current coords R x C, source possibly transposed and
// conjugated) into column-major memory `dst` with leading dimension `ld`.
// Plain copies move bytes (memory_utils.hpp:17-77); scaled copies compute
// dst = beta*dst + alpha*src in T (memory_utils.hpp:25-39,79-122,186-256).
template <typename T>
void copy_piece(const Blk &s, T *dst, int64_t ld, bool scaled, T alpha, T beta) {
    const int R = s.rows.length(), C = s.cols.length();
    const T *src = (const T *)s.data;
    if (!s.trans) {
        for (int c = 0; c < C; ++c) {
            const T *sc = src + (int64_t)c * s.stride;
            T *dc = dst + (int64_t)c * ld;
            if (!scaled) {
                std::memcpy((void *)dc, (const void *)sc, sizeof(T) * R);
            } else {
                for (int r = 0; r < R; ++r)
                    dc[r] = beta * dc[r] + alpha * sc[r];
            }
        }
    } else {
        // storage is C rows x R cols: element (r, c) sits at src[r*stride + c]
        for (int c = 0; c < C; ++c) {
            T *dc = dst + (int64_t)c * ld;
            for (int r = 0; r < R; ++r) {
                T v = src[(int64_t)r * s.stride + c];
                if (s.conj)
                    v = conj_of(v);
                if (!scaled)
                    std::memcpy((void *)&dc[r], (const void *)&v, sizeof(T));
                else
                    dc[r] = beta * dc[r] + alpha * v;
            }
        }
    }
}

// Apply grid_layout::transpose_or_conjugate (grid_layout.hpp:18-25).
void transpose_layout(Layout &L, char flag) {
    if (flag != 'T' && flag != 'C')
        return;
    int nbr = L.nbr(), nbc = L.nbc();
    std::vector<int> t((size_t)nbr * nbc);
    for (int i = 0; i < nbr; ++i)
        for (int j = 0; j < nbc; ++j)
            t[(size_t)j * nbr + i] = L.owners[(size_t)i * nbc + j];
    L.owners.swap(t);
    std::swap(L.rs, L.cs);
    for (auto &blocks : L.local)
        for (Blk &b : blocks) {
            std::swap(b.rows, b.cols);
            std::swap(b.row_coord, b.col_coord);
            b.trans = true; // block.cpp:283-287: flags are set, never cleared
            if (flag == 'C')
                b.conj = true;
        }
}

bool load_layout(const g2g_layout_desc &d, int P, Layout &L) {
    if (d.n_block_rows < 0 || d.n_block_cols < 0 || !d.rows_split || !d.cols_split)
        return false;
    L.rs.assign(d.rows_split, d.rows_split + d.n_block_rows + 1);
    L.cs.assign(d.cols_split, d.cols_split + d.n_block_cols + 1);
    L.owners.assign(d.owners, d.owners + (size_t)d.n_block_rows * d.n_block_cols);
    if (d.n_reordering > 0)
        L.reordering.assign(d.reordering, d.reordering + d.n_reordering);
    L.n_ranks = d.n_ranks;
    L.local.assign(P, {});
    for (int k = 0; k < d.n_blocks; ++k) {
        const g2g_block_desc &bd = d.blocks[k];
        if (bd.rank < 0 || bd.rank >= P || bd.row < 0 || bd.row >= d.n_block_rows ||
            bd.col < 0 || bd.col >= d.n_block_cols)
            return false;
        Blk b;
        b.rows = {L.rs[bd.row], L.rs[bd.row + 1]};
        b.cols = {L.cs[bd.col], L.cs[bd.col + 1]};
        b.row_coord = bd.row;
        b.col_coord = bd.col;
        b.data = (unsigned char *)bd.data;
        b.stride = bd.stride;
        b.trans = bd.transpose_on_copy != 0;
        b.conj = bd.conjugate_on_copy != 0;
        L.local[bd.rank].push_back(b);
    }
    return true;
}

template <typename F> void parallel_for(int n, int threads, F f) {
    threads = std::max(1, std::min(threads, n));
    if (threads == 1) {
        for (int i = 0; i < n; ++i)
            f(i);
        return;
    }
    std::atomic<int> next(0);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&]() {
            for (int i = next++; i < n; i = next++)
                f(i);
        });
    for (auto &th : pool)
        th.join();
}

struct RankData {
    std::vector<Msg> send_remote, send_local, recv_remote, recv_local;
    std::vector<int64_t> send_off, recv_off;  // per remote message, elements
    std::vector<int64_t> send_counts, send_dspls, recv_counts, recv_dspls;
    std::vector<unsigned char> send_buf, recv_buf;
};

template <typename T>
int transform_pair(const g2g_layout_desc &di, const g2g_layout_desc &df,
                   const g2g_op *op, int threads) {
    const int esz = (int)sizeof(T);
    int P = std::max(1, std::max(di.n_ranks, df.n_ranks));
    Layout A, B;
    if (!load_layout(di, P, A) || !load_layout(df, P, B)) {
        g_err = "bad layout descriptor";
        return 1;
    }
    char trans = op ? (char)std::toupper((unsigned char)op->trans) : 'N';
    if (trans != 'N' && trans != 'T' && trans != 'C') {
        g_err = "trans must be N, T or C";
        return 1;
    }
    transpose_layout(A, trans);
    if (A.rs.back() != B.rs.back() || A.cs.back() != B.cs.back() ||
        A.rs.front() != B.rs.front() || A.cs.front() != B.cs.front()) {
        g_err = "initial and final grids cover different matrices";
        return 1;
    }
    const double one[2] = {1.0, 0.0}, zero[2] = {0.0, 0.0};
    T alpha = scalar_of<T>(op ? op->alpha : one);
    T beta = scalar_of<T>(op ? op->beta : zero);
    const bool scaled = !(alpha == T{1} && beta == T{0});

    std::vector<RankData> rd(P);
    // plan + pack (prepare_to_send / prepare_to_recv, copy_to_buffer)
    parallel_for(P, threads, [&](int r) {
        RankData &d = rd[r];
        std::vector<Msg> send, recv;
        decompose(A.local[r], A, B, esz, send);
        decompose(B.local[r], B, A, esz, recv);
        std::sort(send.begin(), send.end(), msg_less);
        std::sort(recv.begin(), recv.end(), msg_less);
        d.send_counts.assign(P, 0);
        d.recv_counts.assign(P, 0);
        int64_t off = 0;
        for (const Msg &m : send) {
            if (m.peer != r) {
                d.send_remote.push_back(m);
                d.send_off.push_back(off);
                off += m.b.size();
                d.send_counts[m.peer] += m.b.size();
            } else {
                d.send_local.push_back(m);
            }
        }
        d.send_buf.resize((size_t)off * esz);
        off = 0;
        for (const Msg &m : recv) {
            if (m.peer != r) {
                d.recv_remote.push_back(m);
                d.recv_off.push_back(off);
                off += m.b.size();
                d.recv_counts[m.peer] += m.b.size();
            } else {
                d.recv_local.push_back(m);
            }
        }
        d.recv_buf.resize((size_t)off * esz);
        d.send_dspls.assign(P, 0);
        d.recv_dspls.assign(P, 0);
        for (int p = 1; p < P; ++p) {
            d.send_dspls[p] = d.send_dspls[p - 1] + d.send_counts[p - 1];
            d.recv_dspls[p] = d.recv_dspls[p - 1] + d.recv_counts[p - 1];
        }
        for (size_t k = 0; k < d.send_remote.size(); ++k) {
            const Blk &b = d.send_remote[k].b;
            copy_piece<T>(b, (T *)(d.send_buf.data() + d.send_off[k] * esz),
                          b.rows.length(), false, T{1}, T{0});
        }
    });
    // consistency of the two sides (the reference would hang or misplace data)
    for (int s = 0; s < P; ++s)
        for (int r = 0; r < P; ++r)
            if (rd[s].send_counts[r] != rd[r].recv_counts[s]) {
                g_err = "send/recv volume mismatch between ranks " +
                        std::to_string(s) + " and " + std::to_string(r) +
                        " (blocks not held by their owners?)";
                return 1;
            }
    for (int r = 0; r < P; ++r)
        if (rd[r].send_local.size() != rd[r].recv_local.size()) {
            g_err = "local piece lists differ on rank " + std::to_string(r);
            return 1;
        }
    // exchange: receiver r pulls sender s's segment for r (MPI_Isend/Irecv)
    parallel_for(P, threads, [&](int r) {
        RankData &d = rd[r];
        for (int s = 0; s < P; ++s) {
            int64_t n = d.recv_counts[s];
            if (n)
                std::memcpy(d.recv_buf.data() + d.recv_dspls[s] * esz,
                            rd[s].send_buf.data() + rd[s].send_dspls[r] * esz,
                            (size_t)n * esz);
        }
    });
    // local copies and unpack (copy_local_blocks, copy_from_buffer)
    parallel_for(P, threads, [&](int r) {
        RankData &d = rd[r];
        for (size_t k = 0; k < d.send_local.size(); ++k) {
            const Blk &src = d.send_local[k].b;
            const Blk &dst = d.recv_local[k].b;
            copy_piece<T>(src, (T *)dst.data, dst.stride, scaled, alpha, beta);
        }
        for (size_t k = 0; k < d.recv_remote.size(); ++k) {
            const Blk &dst = d.recv_remote[k].b;
            Blk src;
            src.rows = dst.rows;
            src.cols = dst.cols;
            src.data = d.recv_buf.data() + d.recv_off[k] * esz;
            src.stride = dst.rows.length();
            copy_piece<T>(src, (T *)dst.data, dst.stride, scaled, alpha, beta);
        }
    });
    return 0;
}

// One rank's communication_data (communication_data.cpp:51-99) and packed
// send buffer (copy_to_buffer, communication_data.cpp:132-142): the piece
// lists of prepare_to_send / prepare_to_recv (utils.hpp:146-212) sorted by
// (peer, cols, rows, tag), counts per peer, displacements as exclusive sums.
template <typename T>
int rank_exchange(const g2g_layout_desc &di, const g2g_layout_desc &df, const g2g_op *op,
                  int rank, int64_t *send_counts, int64_t *send_dspls, int64_t *recv_counts,
                  int64_t *recv_dspls, unsigned char *send_out, int64_t send_capacity) {
    const int esz = (int)sizeof(T);
    int P = std::max(1, std::max(di.n_ranks, df.n_ranks));
    Layout A, B;
    if (!load_layout(di, P, A) || !load_layout(df, P, B) || rank < 0 || rank >= P) {
        g_err = "bad layout descriptor or rank";
        return 1;
    }
    char trans = op ? (char)std::toupper((unsigned char)op->trans) : 'N';
    transpose_layout(A, trans);
    std::vector<Msg> send, recv;
    decompose(A.local[rank], A, B, esz, send);
    decompose(B.local[rank], B, A, esz, recv);
    std::sort(send.begin(), send.end(), msg_less);
    std::sort(recv.begin(), recv.end(), msg_less);
    for (int p = 0; p < P; ++p)
        send_counts[p] = recv_counts[p] = 0;
    int64_t total = 0;
    for (const Msg &m : send)
        if (m.peer != rank) {
            if (send_out) {
                if ((total + m.b.size()) * esz > send_capacity) {
                    g_err = "send buffer too small";
                    return 1;
                }
                copy_piece<T>(m.b, (T *)(send_out + total * esz), m.b.rows.length(), false,
                              T{1}, T{0});
            }
            total += m.b.size();
            send_counts[m.peer] += m.b.size();
        }
    for (const Msg &m : recv)
        if (m.peer != rank)
            recv_counts[m.peer] += m.b.size();
    send_dspls[0] = recv_dspls[0] = 0;
    for (int p = 1; p < P; ++p) {
        send_dspls[p] = send_dspls[p - 1] + send_counts[p - 1];
        recv_dspls[p] = recv_dspls[p - 1] + recv_counts[p - 1];
    }
    return 0;
}

int transform_dispatch(int dtype, const g2g_layout_desc &di,
                       const g2g_layout_desc &df, const g2g_op *op, int threads) {
    switch (dtype) {
    case G2G_FLOAT32:
        return transform_pair<float>(di, df, op, threads);
    case G2G_FLOAT64:
        return transform_pair<double>(di, df, op, threads);
    case G2G_COMPLEX64:
        return transform_pair<std::complex<float>>(di, df, op, threads);
    case G2G_COMPLEX128:
        return transform_pair<std::complex<double>>(di, df, op, threads);
    default:
        g_err = "bad dtype";
        return 1;
    }
}

} // namespace

extern "C" {

const char *g2g_oracle_last_error(void) { return g_err.c_str(); }

// Transforms n_pairs layout pairs one after another; ops may be NULL.
int g2g_oracle_transform(int n_pairs, const g2g_layout_desc *inits,
                         const g2g_layout_desc *finals, const int *dtypes,
                         const g2g_op *ops, int threads) {
    g_err.clear();
    for (int k = 0; k < n_pairs; ++k) {
        int rc = transform_dispatch(dtypes[k], inits[k], finals[k],
                                    ops ? &ops[k] : nullptr, threads);
        if (rc)
            return rc;
    }
    return 0;
}

// Rank `rank`'s send / receive counts and displacements (P entries each,
// elements) and, when send_buffer is not NULL, its packed send buffer.
int g2g_oracle_rank_exchange(const g2g_layout_desc *di, const g2g_layout_desc *df, int dtype,
                             const g2g_op *op, int rank, int64_t *send_counts,
                             int64_t *send_dspls, int64_t *recv_counts, int64_t *recv_dspls,
                             void *send_buffer, int64_t send_capacity_bytes) {
    g_err.clear();
    unsigned char *out = (unsigned char *)send_buffer;
    switch (dtype) {
    case G2G_FLOAT32:
        return rank_exchange<float>(*di, *df, op, rank, send_counts, send_dspls, recv_counts,
                                    recv_dspls, out, send_capacity_bytes);
    case G2G_FLOAT64:
        return rank_exchange<double>(*di, *df, op, rank, send_counts, send_dspls, recv_counts,
                                     recv_dspls, out, send_capacity_bytes);
    case G2G_COMPLEX64:
        return rank_exchange<std::complex<float>>(*di, *df, op, rank, send_counts, send_dspls,
                                                  recv_counts, recv_dspls, out,
                                                  send_capacity_bytes);
    case G2G_COMPLEX128:
        return rank_exchange<std::complex<double>>(*di, *df, op, rank, send_counts, send_dspls,
                                                   recv_counts, recv_dspls, out,
                                                   send_capacity_bytes);
    default:
        g_err = "bad dtype";
        return 1;
    }
}

// The cover of split vector a by split vector b; returns n_a - 1.
int g2g_oracle_decomp_cover(const int *a, int na, const int *b, int nb,
                            int *start, int *end) {
    std::vector<int> va(a, a + na), vb(b, b + nb);
    std::vector<std::pair<int, int>> c;
    decomp_cover(va, vb, c);
    for (size_t k = 0; k < c.size(); ++k) {
        start[k] = c[k].first;
        end[k] = c[k].second;
    }
    return (int)c.size();
}

} // extern "C"
