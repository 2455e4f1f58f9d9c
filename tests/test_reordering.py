"""communication_volume / optimal_reordering on the CPU (no device work):
the library against the reference's results on seeded grid pairs (golden
fixtures, and the live reference oracle where it is built)."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from grid2grid_gb300 import capi
from grid2grid_gb300 import layouts as Ls

import oracle

pytestmark = pytest.mark.skipif(not os.path.exists(capi.LIB_PATH), reason="library not built")

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reordering.json")


def _desc(g, P):
    rs = np.ascontiguousarray(g["rows_split"], dtype=np.int32)
    cs = np.ascontiguousarray(g["cols_split"], dtype=np.int32)
    ow = np.ascontiguousarray(g["owners"], dtype=np.int32).ravel()
    d = capi.LayoutDesc()
    d.n_block_rows, d.n_block_cols = len(rs) - 1, len(cs) - 1
    d.rows_split = rs.ctypes.data_as(C.POINTER(C.c_int32))
    d.cols_split = cs.ctypes.data_as(C.POINTER(C.c_int32))
    d.owners = ow.ctypes.data_as(C.POINTER(C.c_int32))
    d.n_ranks = P
    keep = [rs, cs, ow]
    if g.get("reordering") is not None:
        reo = np.ascontiguousarray(g["reordering"], dtype=np.int32)
        d.n_reordering = len(reo)
        d.reordering = reo.ctypes.data_as(C.POINTER(C.c_int32))
        keep.append(reo)
    return d, keep


def ours(di, df, P):
    lib = capi.load()
    vol = np.zeros(P * P, np.int64)
    capi.check(lib.g2g_communication_volume(C.byref(di), C.byref(df), P,
                                            vol.ctypes.data_as(C.POINTER(C.c_int64))))
    perm = np.zeros(P, np.int32)
    re = C.c_int32(0)
    capi.check(lib.g2g_optimal_reordering(vol.ctypes.data_as(C.POINTER(C.c_int64)), P,
                                          perm.ctypes.data_as(C.POINTER(C.c_int32)),
                                          C.byref(re)))
    return vol.reshape(P, P), perm, bool(re.value)


def weights_tie(vol):
    """True when two edges the greedy matching sees share a weight (their
    order is then the implementation's: ours is (r, s), the reference's its
    hash map's)."""
    P = vol.shape[0]
    ws = []
    on = np.zeros(P, bool)
    for r in range(P):
        for s in range(r + 1, P):
            if vol[r, s] > 0:
                on[r] = on[s] = True
                w = vol[r, s] - vol[r, r] - vol[s, s]
                if w:
                    ws.append(w)
    ws += [1] * int(np.count_nonzero(on | (np.diag(vol) > 0)))
    pos = [w for w in ws if w > 1] + ([1] if 1 in ws else [])
    return len(pos) != len(set(pos))


def test_volume_and_reordering_match_reference_golden():
    with open(GOLDEN) as f:
        cases = json.load(f)["cases"]
    assert len(cases) >= 40
    exact = 0
    for c in cases:
        P = c["n_ranks"]
        di, k1 = _desc(c["initial"], P)
        df, k2 = _desc(c["final"], P)
        vol, perm, re = ours(di, df, P)
        np.testing.assert_array_equal(vol, np.array(c["volume"]))
        if not weights_tie(vol):
            np.testing.assert_array_equal(perm, c["permutation"])
            assert re == c["reordered"]
            exact += 1
    assert exact >= len(cases) * 3 // 4


def test_reordering_is_a_product_of_swaps_that_keeps_more_local():
    with open(GOLDEN) as f:
        cases = json.load(f)["cases"]
    for c in cases:
        P = c["n_ranks"]
        di, k1 = _desc(c["initial"], P)
        df, k2 = _desc(c["final"], P)
        vol, perm, _ = ours(di, df, P)
        assert sorted(perm.tolist()) == list(range(P))
        assert all(perm[perm[r]] == r for r in range(P))  # disjoint swaps
        # every swap taken had a positive weight: it keeps more data local
        for r in range(P):
            s = int(perm[r])
            if r < s:
                assert vol[r, s] - vol[r, r] - vol[s, s] > 0


@pytest.mark.skipif(not oracle.ref_available(), reason="reference oracle not built here")
@pytest.mark.parametrize("seed", range(4))
def test_matches_live_reference(seed):
    rng = np.random.default_rng(900 + seed)
    for _ in range(30):
        P = int(rng.integers(2, 12))
        m, n = int(rng.integers(20, 400)), int(rng.integers(20, 400))
        Li = Ls.random_grid_layout(m, n, P, capi.FLOAT64, rng, ext_lo=1, ext_hi=max(1, m // 3))
        Lf = Ls.scalapack_layout(m, n, int(rng.integers(4, 60)), int(rng.integers(4, 60)),
                                 1, P, capi.FLOAT64)
        if rng.random() < 0.3:
            Lf.reorder_ranks(list(rng.permutation(P)))
        di, k1 = Li.desc(0)
        df, k2 = Lf.desc(0)
        vol, perm, re = ours(di, df, P)
        rvol, rperm, rre = oracle.ref_comm_volume(Li, Lf, P)
        np.testing.assert_array_equal(vol, rvol)
        if not weights_tie(vol):
            np.testing.assert_array_equal(perm, rperm)
            assert re == rre


def test_rejects_bad_arguments():
    lib = capi.load()
    g = {"rows_split": [0, 5, 10], "cols_split": [0, 10], "owners": [[0], [3]]}
    di, k1 = _desc(g, 4)
    g2 = {"rows_split": [0, 10], "cols_split": [0, 4, 9], "owners": [[1, 2]]}
    df, k2 = _desc(g2, 4)
    vol = np.zeros(16, np.int64)
    vp = vol.ctypes.data_as(C.POINTER(C.c_int64))
    # different matrices (10 vs 9 columns)
    assert lib.g2g_communication_volume(C.byref(di), C.byref(df), 4, vp) == \
        capi.ERROR_INVALID_ARGUMENT
    # an owner beyond n_ranks
    g3 = {"rows_split": [0, 10], "cols_split": [0, 4, 10], "owners": [[1, 5]]}
    df3, k3 = _desc(g3, 4)
    assert lib.g2g_communication_volume(C.byref(di), C.byref(df3), 4, vp) == \
        capi.ERROR_INVALID_ARGUMENT
    perm = np.zeros(4, np.int32)
    assert lib.g2g_optimal_reordering(None, 4, perm.ctypes.data_as(C.POINTER(C.c_int32)),
                                      None) == capi.ERROR_INVALID_ARGUMENT
