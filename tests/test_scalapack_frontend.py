"""ScaLAPACK-descriptor front end on the CPU: the C builder
g2g_layout_create_scalapack against the reference's get_scalapack_grid
(golden layouts, scalapack_layout.cpp:178-278), against the Python builder
on random descriptors, and its argument checks. No device work."""
import ctypes as C

import numpy as np
import pytest

from grid2grid_gb300 import capi
from grid2grid_gb300 import layouts as Ls

pytestmark = pytest.mark.skipif(not __import__("os").path.exists(capi.LIB_PATH),
                                reason="library not built")

ESZ = 8  # float64
FAKE_BASE = 1 << 40


def _desc(m, n, mb, nb, pr, pc, row_major, rsrc=0, csrc=0):
    d = capi.ScalapackDesc()
    d.m, d.n, d.mb, d.nb = m, n, mb, nb
    d.rsrc, d.csrc, d.nprow, d.npcol = rsrc, csrc, pr, pc
    d.row_major = int(row_major)
    return d


def _bases(P):
    return [FAKE_BASE + (r << 32) for r in range(P)]


def _build(d, ia, ja, m, n, lld, dtype=capi.FLOAT64):
    lib = capi.load()
    P = d.nprow * d.npcol
    data = (C.c_void_p * P)(*_bases(P))
    lp = None if lld is None else (C.c_int32 * P)(*lld)
    h = C.c_void_p()
    st = lib.g2g_layout_create_scalapack(C.byref(d), ia, ja, m, n, data, lp, dtype,
                                         C.byref(h))
    return st, h


def _blocks_of(h):
    lib = capi.load()
    ld = capi.LayoutDesc()
    capi.check(lib.g2g_layout_get_desc(h, C.byref(ld)))
    rs = [ld.rows_split[i] for i in range(ld.n_block_rows + 1)]
    cs = [ld.cols_split[i] for i in range(ld.n_block_cols + 1)]
    owners = [[ld.owners[i * ld.n_block_cols + j] for j in range(ld.n_block_cols)]
              for i in range(ld.n_block_rows)]
    blocks = [ld.blocks[k] for k in range(ld.n_blocks)]
    return ld, rs, cs, owners, blocks


def test_builder_matches_reference_golden(golden):
    """Every golden get_scalapack_grid layout (the reference run per rank),
    including the expectations of examples/scalapack_submatrix.cpp and
    examples/parallel_scalapack_submatrix.cpp."""
    lib = capi.load()
    recs = golden.scalapack["examples"] + golden.scalapack["random"]
    for rec in recs:
        (lld, m, n, i1, j1, sm, sn, mb, nb, pr, pc, rm, sr, sc) = rec["args"]
        d = _desc(m, n, mb, nb, pr, pc, rm, sr, sc)
        st, h = _build(d, i1, j1, sm, sn, [lld] * (pr * pc))
        assert st == capi.SUCCESS, lib.g2g_last_error_string()
        try:
            ld, rs, cs, owners, blocks = _blocks_of(h)
            assert ld.n_ranks == pr * pc
            for rank_s, ref in rec["reference"].items():
                r = int(rank_s)
                assert rs == ref["rows_split"] and cs == ref["cols_split"]
                assert owners == ref["owners"]
                mine = [b for b in blocks if b.rank == r]
                assert len(mine) == len(ref["blocks"])
                for b, rb in zip(mine, ref["blocks"]):
                    assert [b.row, b.col] == rb["coord"]
                    assert b.stride == rb["stride"]
                    assert (b.data - _bases(pr * pc)[r]) // ESZ == rb["offset"]
        finally:
            lib.g2g_layout_destroy(h)


@pytest.mark.parametrize("seed", range(8))
def test_builder_matches_python_builder(seed):
    rng = np.random.default_rng(300 + seed)
    lib = capi.load()
    for _ in range(20):
        pr, pc = int(rng.integers(1, 5)), int(rng.integers(1, 5))
        M, N = int(rng.integers(1, 300)), int(rng.integers(1, 300))
        mb, nb = int(rng.integers(1, 40)), int(rng.integers(1, 40))
        rsrc, csrc = int(rng.integers(0, pr)), int(rng.integers(0, pc))
        ia, ja = int(rng.integers(1, M + 1)), int(rng.integers(1, N + 1))
        m, n = int(rng.integers(1, M - ia + 2)), int(rng.integers(1, N - ja + 2))
        rm = bool(rng.integers(0, 2))
        lld = [int(x) for x in rng.integers(M, M + 9, size=pr * pc)]
        L = Ls.scalapack_layout(M, N, mb, nb, pr, pc, capi.FLOAT64, rm, lld=lld,
                                ij=(ia, ja), sub=(m, n), src=(rsrc, csrc))
        st, h = _build(_desc(M, N, mb, nb, pr, pc, rm, rsrc, csrc), ia, ja, m, n, lld)
        assert st == capi.SUCCESS, lib.g2g_last_error_string()
        try:
            ld, rs, cs, owners, blocks = _blocks_of(h)
            assert rs == L.rows_split.tolist() and cs == L.cols_split.tolist()
            assert owners == L.owners.tolist()
            assert len(blocks) == L.n_blocks
            got = sorted((b.rank, b.row, b.col, b.stride,
                          (b.data - _bases(pr * pc)[b.rank]) // ESZ) for b in blocks)
            want = sorted((int(L.blocks["rank"][k]), int(L.blocks["row"][k]),
                           int(L.blocks["col"][k]), int(L.blocks["stride"][k]),
                           (int(L.offsets[k]) - int(L.rank_base[L.blocks["rank"][k]])) // ESZ)
                          for k in range(L.n_blocks))
            assert got == want
        finally:
            lib.g2g_layout_destroy(h)


def test_default_lld_is_local_block_rows():
    """lld == NULL: a rank's local block rows x mb (the simple overload,
    scalapack_layout.cpp:318-324), counted from the source process row."""
    lib = capi.load()
    d = _desc(100, 50, 16, 8, 3, 2, False, rsrc=1)
    st, h = _build(d, 1, 1, 100, 50, None)
    assert st == capi.SUCCESS
    try:
        _, _, _, _, blocks = _blocks_of(h)
        # 7 block rows from process row 1: rows 1, 2, 0 own 3, 2, 2 blocks
        want = {0: 2 * 16, 1: 3 * 16, 2: 2 * 16}
        for b in blocks:
            assert b.stride == want[b.rank % 3]
    finally:
        lib.g2g_layout_destroy(h)


@pytest.mark.parametrize("bad", [
    dict(ia=0), dict(ja=0), dict(m=101), dict(n=-1), dict(rsrc=2), dict(csrc=-1),
    dict(mb=0), dict(nprow=0), dict(lld=[5] * 4), dict(null_rank=1), dict(dtype=9)])
def test_builder_rejects_bad_arguments(bad):
    lib = capi.load()
    p = dict(M=100, N=80, mb=10, nb=10, nprow=2, npcol=2, rsrc=0, csrc=0, ia=1, ja=1,
             m=100, n=80, lld=[60] * 4, dtype=capi.FLOAT64)
    p.update({k: v for k, v in bad.items() if k != "null_rank"})
    d = _desc(p["M"], p["N"], p["mb"], p["nb"], p["nprow"], p["npcol"], False,
              p["rsrc"], p["csrc"])
    P = max(1, p["nprow"] * p["npcol"])
    bases = _bases(P)
    if "null_rank" in bad:
        bases[bad["null_rank"]] = 0
    data = (C.c_void_p * P)(*bases)
    lld = (C.c_int32 * P)(*(p["lld"] + [60] * P)[:P])
    h = C.c_void_p()
    st = lib.g2g_layout_create_scalapack(C.byref(d), p["ia"], p["ja"], p["m"], p["n"],
                                         data, lld, p["dtype"], C.byref(h))
    assert st == capi.ERROR_INVALID_ARGUMENT
    assert not h.value
    assert lib.g2g_last_error_string()


def test_gemr2d_argument_checks_need_no_device():
    """Empty and invalid requests are answered on the host."""
    lib = capi.load()
    d = _desc(10, 10, 4, 4, 1, 1, False)
    data = (C.c_void_p * 1)(FAKE_BASE)
    assert lib.g2g_gemr2d(0, 5, data, 1, 1, C.byref(d), None, data, 1, 1, C.byref(d), None,
                          capi.FLOAT64, None, None) == capi.SUCCESS
    assert lib.g2g_gemr2d(-1, 5, data, 1, 1, C.byref(d), None, data, 1, 1, C.byref(d),
                          None, capi.FLOAT64, None, None) == capi.ERROR_INVALID_ARGUMENT
    assert lib.g2g_gemr2d(5, 5, data, 7, 1, C.byref(d), None, data, 1, 1, C.byref(d), None,
                          capi.FLOAT64, None, None) == capi.ERROR_INVALID_ARGUMENT
    # a missing rank array is refused before the plan cache is consulted
    assert lib.g2g_gemr2d(5, 5, None, 1, 1, C.byref(d), None, data, 1, 1, C.byref(d), None,
                          capi.FLOAT64, None, None) == capi.ERROR_INVALID_ARGUMENT
    assert b"NULL" in lib.g2g_last_error_string()
    # a request that fails validation is not cached: the same call fails again
    for _ in range(2):
        assert lib.g2g_gemr2d(5, 5, data, 7, 1, C.byref(d), None, data, 1, 1, C.byref(d),
                              None, capi.FLOAT64, None, None) == capi.ERROR_INVALID_ARGUMENT
