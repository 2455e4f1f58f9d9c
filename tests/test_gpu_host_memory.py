"""Layouts whose blocks live in pinned host memory: the gather-scatter reads
and writes them in place over the host link (no staging copies), with the
same results as for device memory."""
import ctypes as C

import numpy as np
import pytest

from grid2grid_gb300 import capi
from grid2grid_gb300 import layouts as Ls

import g2g_testlib as T

pytestmark = pytest.mark.gpu


def _pinned(a):
    import torch
    t = torch.empty(len(a), dtype=torch.uint8, pin_memory=True)
    t.numpy()[:] = a
    return t


def _run(Li, Lf, ai, af, where, op=None):
    """where = (initial, final) in {"host", "device"}; returns the final arena."""
    import torch
    lib = capi.load()
    ti = _pinned(ai) if where[0] == "host" else torch.from_numpy(ai.copy()).cuda()
    tf = _pinned(af) if where[1] == "host" else torch.from_numpy(af.copy()).cuda()
    dI, k1 = Li.desc(ti.data_ptr())
    dF, k2 = Lf.desc(tf.data_ptr())
    opa = None if op is None else C.byref(capi.make_op(*op))
    capi.check(lib.g2g_transform(C.byref(dI), C.byref(dF), Li.dtype, opa, None))
    torch.cuda.synchronize()
    return tf.numpy().copy() if where[1] == "host" else tf.cpu().numpy()


@pytest.mark.parametrize("where", [("host", "host"), ("host", "device"), ("device", "host")])
@pytest.mark.parametrize("dt", [capi.FLOAT32, capi.COMPLEX128])
@pytest.mark.parametrize("op", [None, ("T", 1.0, 0.0), ("N", 2.0, 0.5)])
def test_host_memory_matches_oracle(where, dt, op):
    rng = np.random.default_rng(11 + dt + (0 if op is None else 3 * len(op[0])))
    m, n, P = 333, 250, 6
    t = "N" if op is None else op[0]
    Li = Ls.random_grid_layout(m if t == "N" else n, n if t == "N" else m, P, dt, rng,
                               ext_hi=90)
    Lf = Ls.random_grid_layout(m, n, P, dt, rng, ext_hi=90)
    ai = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
    af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    ops = None if op is None else [op]
    want = T.port_run([Li], [Lf], [ai], [af], ops)[0]
    got = _run(Li, Lf, ai, af, where, op)
    T.assert_arenas_equal(got, want, Lf, nan_equivalent=op is not None and op[1] != 1.0,
                          what=f"{where} dt{dt} {op}")


def test_pageable_host_memory_is_refused():
    """Only pinned host memory is reachable from the GPU; a pageable buffer
    is refused on the host before any device work."""
    lib = capi.load()
    rng = np.random.default_rng(3)
    Li = Ls.random_grid_layout(64, 64, 2, capi.FLOAT32, rng, ext_hi=40)
    Lf = Ls.random_grid_layout(64, 64, 2, capi.FLOAT32, rng, ext_hi=40)
    ai = np.zeros(Li.arena_bytes, np.uint8)
    af = np.zeros(Lf.arena_bytes, np.uint8)
    dI, k1 = Li.desc(ai.ctypes.data)
    dF, k2 = Lf.desc(af.ctypes.data)
    st = lib.g2g_transform(C.byref(dI), C.byref(dF), capi.FLOAT32, None, None)
    assert st == capi.ERROR_INVALID_ARGUMENT
    assert b"pinned" in lib.g2g_last_error_string()
