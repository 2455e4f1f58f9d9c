"""p?gemr2d on one GPU (g2g_gemr2d): block-cyclic submatrix redistributions
given as ScaLAPACK descriptors, against the oracle run on the same layouts
built by get_scalapack_grid's rules (scalapack_layout.cpp:178-278)."""
import ctypes as C

import numpy as np
import pytest

from grid2grid_gb300 import capi
from grid2grid_gb300 import layouts as Ls

import g2g_testlib as T

pytestmark = pytest.mark.gpu


def _desc(M, N, mb, nb, pr, pc, rm, src):
    d = capi.ScalapackDesc()
    d.m, d.n, d.mb, d.nb = M, N, mb, nb
    d.rsrc, d.csrc = src
    d.nprow, d.npcol, d.row_major = pr, pc, int(rm)
    return d


def _side(rng, M, N, ia, ja, m, n, dt):
    pr, pc = int(rng.integers(1, 4)), int(rng.integers(1, 4))
    mb, nb = int(rng.integers(1, 48)), int(rng.integers(1, 48))
    src = (int(rng.integers(0, pr)), int(rng.integers(0, pc)))
    rm = bool(rng.integers(0, 2))
    lld = [int(x) for x in rng.integers(M, M + 6, size=pr * pc)]
    L = Ls.scalapack_layout(M, N, mb, nb, pr, pc, dt, rm, lld=lld, ij=(ia, ja),
                            sub=(m, n), src=src)
    return L, _desc(M, N, mb, nb, pr, pc, rm, src), lld


def _gemr2d(La, da, llda, aa, ia, ja, Lb, db, lldb, ab, ib, jb, m, n, dt, op):
    import torch
    lib = capi.load()
    ta, tb = T.to_device([aa, ab])
    pa = (C.c_void_p * len(llda))(*[ta.data_ptr() + int(o) for o in La.rank_base])
    pb = (C.c_void_p * len(lldb))(*[tb.data_ptr() + int(o) for o in Lb.rank_base])
    la = (C.c_int32 * len(llda))(*llda)
    lb = (C.c_int32 * len(lldb))(*lldb)
    opa = None if op is None else C.byref(capi.make_op(*op))
    capi.check(lib.g2g_gemr2d(m, n, pa, ia, ja, C.byref(da), la, pb, ib, jb, C.byref(db), lb,
                              dt, opa, C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    return tb.cpu().numpy()


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("dt", [capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64, capi.COMPLEX128])
def test_gemr2d_matches_oracle(seed, dt):
    rng = np.random.default_rng(50 * seed + dt)
    m, n = int(rng.integers(1, 180)), int(rng.integers(1, 180))
    Ma, Na = m + int(rng.integers(0, 40)), n + int(rng.integers(0, 40))
    Mb, Nb = m + int(rng.integers(0, 40)), n + int(rng.integers(0, 40))
    ia, ja = int(rng.integers(1, Ma - m + 2)), int(rng.integers(1, Na - n + 2))
    ib, jb = int(rng.integers(1, Mb - m + 2)), int(rng.integers(1, Nb - n + 2))
    La, da, llda = _side(rng, Ma, Na, ia, ja, m, n, dt)
    Lb, db, lldb = _side(rng, Mb, Nb, ib, jb, m, n, dt)
    P = max(La.n_ranks, Lb.n_ranks)
    La.n_ranks = Lb.n_ranks = P
    aa = Ls.fill_random(np.zeros(La.arena_bytes, np.uint8), rng)
    ab = Ls.fill_random(np.zeros(Lb.arena_bytes, np.uint8), rng)
    want = T.port_run([La], [Lb], [aa], [ab])[0]
    got = _gemr2d(La, da, llda, aa, ia, ja, Lb, db, lldb, ab, ib, jb, m, n, dt, None)
    T.assert_arenas_equal(got, want, Lb, what=f"gemr2d seed {seed} dtype {dt}")


@pytest.mark.parametrize("trans", ["T", "C"])
def test_gemr2d_transposed_matches_oracle(trans):
    """With op 'T' / 'C' sub(A) is n x m (the transform's trans overload)."""
    rng = np.random.default_rng(77 if trans == "T" else 78)
    dt = capi.COMPLEX64
    m, n = 150, 97
    ia, ja, ib, jb = 5, 9, 3, 2
    La, da, llda = _side(rng, n + 20, m + 15, ia, ja, n, m, dt)
    Lb, db, lldb = _side(rng, m + 4, n + 8, ib, jb, m, n, dt)
    P = max(La.n_ranks, Lb.n_ranks)
    La.n_ranks = Lb.n_ranks = P
    aa = Ls.fill_random(np.zeros(La.arena_bytes, np.uint8), rng)
    ab = Ls.fill_random(np.zeros(Lb.arena_bytes, np.uint8), rng)
    op = (trans, 1.0, 0.0)
    want = T.port_run([La], [Lb], [aa], [ab], [op])[0]
    got = _gemr2d(La, da, llda, aa, ia, ja, Lb, db, lldb, ab, ib, jb, m, n, dt, op)
    T.assert_arenas_equal(got, want, Lb, what=f"gemr2d op {trans}")


def test_gemr2d_known_answer_values():
    """sub(B) = sub(A) for A(i, j) = i + j*M (global, 0-based): every element
    of B's submatrix holds A's value at the matching global position."""
    rng = np.random.default_rng(5)
    dt = capi.FLOAT64
    M, N, m, n, ia, ja, ib, jb = 300, 260, 211, 173, 40, 61, 7, 11
    La, da, llda = _side(rng, M, N, ia, ja, m, n, dt)
    Lb, db, lldb = _side(rng, m + 30, n + 20, ib, jb, m, n, dt)
    P = max(La.n_ranks, Lb.n_ranks)
    La.n_ranks = Lb.n_ranks = P

    def values(L, k):
        i, j = int(L.blocks["row"][k]), int(L.blocks["col"][k])
        r = np.arange(L.rows_split[i], L.rows_split[i + 1])[:, None]
        c = np.arange(L.cols_split[j], L.cols_split[j + 1])[None, :]
        return ((r + ia - 1) + (c + ja - 1) * M).astype(np.float64)

    aa = np.zeros(La.arena_bytes, np.uint8)
    for k in range(La.n_blocks):
        La.block_view(aa, k)[...] = values(La, k).view(np.uint64)
    ab = np.zeros(Lb.arena_bytes, np.uint8)
    got = _gemr2d(La, da, llda, aa, ia, ja, Lb, db, lldb, ab, ib, jb, m, n, dt, None)
    for k in range(Lb.n_blocks):
        np.testing.assert_array_equal(Lb.block_view(got, k), values(Lb, k).view(np.uint64))
