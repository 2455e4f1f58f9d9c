"""g2g_transform_noalloc: the transform for callers that cannot allocate
device memory (their application owns all of HBM through its own pool, or
runs under a strict memory quota, or cannot take cudaFree's implicit device
synchronisation). Its plan metadata lives in a fixed array inside the
library instead of a per-call allocation. Its results must equal those of
g2g_transform and of the oracle port (bit-exact, the tolerance every parity
test here uses) on two calls in a row, which also checks that a call does not
depend on what the previous call left in the shared array.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

import g2g_testlib as T
import oracle
from grid2grid_gb300 import capi
from grid2grid_gb300 import layouts as Ls

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _setup():
    import torch
    assert torch.cuda.is_available()
    from grid2grid_gb300 import build
    build.build()
    capi.load()
    oracle.build_port()


def _run(entry, Li, Lf, ai, af, op):
    import torch
    lib = capi.load()
    di = torch.from_numpy(ai).cuda()
    df = torch.from_numpy(af).cuda()
    dI, k1 = Li.desc(di.data_ptr())
    dF, k2 = Lf.desc(df.data_ptr())
    s = torch.cuda.current_stream()
    fn = getattr(lib, entry)
    capi.check(fn(C.byref(dI), C.byref(dF), Li.dtype, C.byref(capi.make_op(*op)),
                  C.c_void_p(s.cuda_stream)))
    torch.cuda.synchronize()
    return df.cpu().numpy()


def _case(seed, dt, t, m, n):
    rng = np.random.default_rng(seed)
    Li = Ls.random_grid_layout(m if t == "N" else n, n if t == "N" else m, 7, dt, rng,
                               ext_hi=180)
    Lf = Ls.random_grid_layout(m, n, 7, dt, rng, ext_hi=130)
    ai = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
    af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    return Li, Lf, ai, af


def test_noalloc_matches_transform_on_two_calls_in_a_row():
    # two different transforms back to back: the second must not see the
    # first one's metadata
    first = _case(1, capi.FLOAT32, "N", 900, 700)
    second = _case(2, capi.COMPLEX128, "C", 500, 800)
    for (Li, Lf, ai, af), op in ((first, ("N", 1.0, 0.0)), (second, ("C", 1.0, 0.0))):
        want = _run("g2g_transform", Li, Lf, ai, af, op)
        got = _run("g2g_transform_noalloc", Li, Lf, ai, af, op)
        T.assert_arenas_equal(got, want, Lf, what=f"noalloc {op}")
        port = T.port_run([Li], [Lf], [ai], [af], [op])[0]
        T.assert_arenas_equal(got, port, Lf, what=f"noalloc vs port {op}")
    # the same transform twice in a row
    Li, Lf, ai, af = first
    want = _run("g2g_transform", Li, Lf, ai, af, ("N", 1.0, 0.0))
    for _ in range(2):
        got = _run("g2g_transform_noalloc", Li, Lf, ai, af, ("N", 1.0, 0.0))
        T.assert_arenas_equal(got, want, Lf, what="noalloc repeat")


def _finite(L, rng):
    comp = np.float32 if L.dtype in (capi.FLOAT32, capi.COMPLEX64) else np.float64
    w = np.dtype(comp).itemsize
    return np.frombuffer(rng.standard_normal(L.arena_bytes // w).astype(comp).tobytes(),
                         np.uint8).copy()


@pytest.mark.parametrize("dt,op", [(capi.FLOAT64, ("T", 1.0, 0.0)),
                                   (capi.FLOAT32, ("N", 2.0, 0.5)),
                                   (capi.COMPLEX64, ("C", complex(0.5, -1.0), complex(2.0, 0.25))),
                                   (capi.COMPLEX128, ("T", -1.5, 0.0))])
def test_noalloc_scaled_and_transposed_match_port(dt, op):
    """'T', 'C' and alpha/beta != (1, 0) through the no-allocation call, on
    finite values: bit-exact against the oracle port and g2g_transform."""
    rng = np.random.default_rng(90 + dt)
    Li, Lf, _, _ = _case(30 + dt, dt, op[0], 413, 291)
    ai, af = _finite(Li, rng), _finite(Lf, rng)
    port = T.port_run([Li], [Lf], [ai], [af], [op])[0]
    for _ in range(2):
        got = _run("g2g_transform_noalloc", Li, Lf, ai, af, op)
        T.assert_arenas_equal(got, port, Lf, what=f"noalloc vs port dt{dt} {op}")
    want = _run("g2g_transform", Li, Lf, ai, af, op)
    T.assert_arenas_equal(got, want, Lf, what=f"noalloc vs transform dt{dt} {op}")


def test_noalloc_layouts_in_pinned_host_memory():
    """Both layouts in pinned host memory: the kernel reads and writes them in
    place over the host link; the result equals the oracle port's."""
    import torch
    lib = capi.load()
    Li, Lf, ai, af = _case(44, capi.COMPLEX64, "T", 377, 255)
    op = ("T", 1.0, 0.0)
    port = T.port_run([Li], [Lf], [ai], [af], [op])[0]
    hi = torch.from_numpy(ai.copy()).pin_memory()
    hf = torch.from_numpy(af.copy()).pin_memory()
    dI, k1 = Li.desc(hi.data_ptr())
    dF, k2 = Lf.desc(hf.data_ptr())
    s = torch.cuda.current_stream()
    for _ in range(2):
        hf.copy_(torch.from_numpy(af))
        capi.check(lib.g2g_transform_noalloc(C.byref(dI), C.byref(dF), capi.COMPLEX64,
                                             C.byref(capi.make_op(*op)),
                                             C.c_void_p(s.cuda_stream)))
        T.assert_arenas_equal(hf.numpy(), port, Lf, what="noalloc pinned host")


def test_noalloc_rejects_a_plan_larger_than_its_scratch():
    # a 4096 x 1 grid of 1 x 1 blocks into a 1 x 4096 grid: the cover has
    # (4096 + 1 + 1) x (1 + 4096 + 1) cells, ~16.8 M, and the planner keeps
    # two 8-byte counts per cell (~268 MB), far more than the fixed 32 MiB
    # array holds; descriptors point at a dummy device buffer and the call
    # must fail before any device work
    import torch
    lib = capi.load()
    buf = torch.zeros(16, dtype=torch.uint8, device="cuda")
    m = 4096
    rs = np.arange(m + 1, dtype=np.int32)
    own = np.zeros((m, 1), dtype=np.int32)
    Li = Ls.Layout(rs, [0, m], own, 1, capi.FLOAT32, np.zeros(m, np.int32),
                   np.arange(m, dtype=np.int32), np.zeros(m, np.int32),
                   np.zeros(m, np.int64), np.ones(m, np.int64), 16)
    Lf = Ls.Layout([0, m], rs, own.T.copy(), 1, capi.FLOAT32, np.zeros(m, np.int32),
                   np.zeros(m, np.int32), np.arange(m, dtype=np.int32),
                   np.zeros(m, np.int64), np.ones(m, np.int64), 16)
    dI, k1 = Li.desc(buf.data_ptr())
    dF, k2 = Lf.desc(buf.data_ptr())
    st = lib.g2g_transform_noalloc(C.byref(dI), C.byref(dF), capi.FLOAT32, None, None)
    assert st == capi.ERROR_OUT_OF_MEMORY
    assert b"scratch" in lib.g2g_last_error_string()
