"""communication_volume and optimal_reordering computed on the device: the
same volumes as the host functions and the reference's golden fixtures, and
the same permutations as the host's greedy matching (every case, ties
included, since both use the same strict edge order)."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from grid2grid_gb300 import capi
from grid2grid_gb300 import layouts as Ls

import test_reordering as R

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reordering.json")


@pytest.fixture(scope="module", autouse=True)
def _setup():
    import torch
    assert torch.cuda.is_available()
    from grid2grid_gb300 import build
    build.build()
    capi.load()


def device(di, df, P):
    import torch
    lib = capi.load()
    s = torch.cuda.current_stream()
    sp = C.c_void_p(s.cuda_stream)
    vol = torch.full((P * P,), -7, dtype=torch.int64, device="cuda")
    capi.check(lib.g2g_communication_volume_device(C.byref(di), C.byref(df), P,
                                                   C.c_void_p(vol.data_ptr()), sp))
    perm = torch.full((P,), -1, dtype=torch.int32, device="cuda")
    re = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    capi.check(lib.g2g_optimal_reordering_device(C.c_void_p(vol.data_ptr()), P,
                                                 C.c_void_p(perm.data_ptr()),
                                                 C.c_void_p(re.data_ptr()), sp))
    torch.cuda.synchronize()
    return vol.cpu().numpy().reshape(P, P), perm.cpu().numpy(), bool(re.item())


def test_device_volume_and_matching_match_golden_and_host():
    with open(GOLDEN) as f:
        cases = json.load(f)["cases"]
    for c in cases:
        P = c["n_ranks"]
        di, k1 = R._desc(c["initial"], P)
        df, k2 = R._desc(c["final"], P)
        vol, perm, re = device(di, df, P)
        np.testing.assert_array_equal(vol, np.array(c["volume"]))
        hvol, hperm, hre = R.ours(di, df, P)
        np.testing.assert_array_equal(perm, hperm)
        assert re == hre


@pytest.mark.parametrize("seed", range(3))
def test_device_matches_host_on_random_grids(seed):
    """Random grids with up to 200 ranks (global atomics beyond 64), many
    tied weights on block-cyclic pairs."""
    rng = np.random.default_rng(700 + seed)
    for k in range(12):
        P = int(rng.choice([2, 5, 16, 63, 64, 65, 130, 200]))
        m, n = int(rng.integers(50, 3000)), int(rng.integers(50, 3000))
        if k % 2:
            Li = Ls.random_grid_layout(m, n, P, capi.FLOAT32, rng, ext_hi=max(1, m // 5))
        else:
            Li = Ls.scalapack_layout(m, n, int(rng.integers(8, 200)), int(rng.integers(8, 200)),
                                     1, P, capi.FLOAT32)
        Lf = Ls.scalapack_layout(m, n, int(rng.integers(8, 200)), int(rng.integers(8, 200)),
                                 P, 1, capi.FLOAT32, row_major=bool(k % 3))
        if rng.random() < 0.3:
            Lf.reorder_ranks([int(x) for x in rng.permutation(P)])
        di, k1 = Li.desc(0)
        df, k2 = Lf.desc(0)
        vol, perm, re = device(di, df, P)
        hvol, hperm, hre = R.ours(di, df, P)
        np.testing.assert_array_equal(vol, hvol)
        np.testing.assert_array_equal(perm, hperm)
        assert re == hre
