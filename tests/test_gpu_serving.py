"""Batched and served execution on the GPU: several cached plans in one
launch (g2g_plans_execute) and the continuous-batching server
(g2g_server_*). Every result must equal the oracle's, and each request's
result must be the same when it runs alone and when it runs in a mix of
concurrent requests."""
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


def _pool(n, seed, max_dim=600):
    """n independent layout pairs of mixed dtype and op, with host arenas."""
    rng = np.random.default_rng(seed)
    inits, finals, ias, fas, ops = [], [], [], [], []
    for k in range(n):
        dt = int(rng.choice([0, 1, 2, 3]))
        t = "NTC"[int(rng.integers(0, 3))]
        m, nn = int(rng.integers(1, max_dim)), int(rng.integers(1, max_dim))
        P = int(rng.integers(1, 24))
        Li = Ls.random_grid_layout(m if t == "N" else nn, nn if t == "N" else m, P, dt, rng,
                                   ext_hi=int(rng.integers(1, 250)))
        Lf = Ls.random_grid_layout(m, nn, P, dt, rng, ext_hi=int(rng.integers(1, 250)))
        inits.append(Li)
        finals.append(Lf)
        ias.append(Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng))
        fas.append(Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng))
        ops.append((t, 1.0, 0.0))
    return inits, finals, ias, fas, ops


class Device:
    """Device copies of a pool and descriptor arrays pointing at them."""

    def __init__(self, inits, finals, ias, fas, ops):
        import torch
        self.di = [torch.from_numpy(a).cuda() for a in ias]
        self.df = [torch.from_numpy(a).cuda() for a in fas]
        self.fas = fas
        self.dI, self.k1 = T.descs(inits, [t.data_ptr() for t in self.di])
        self.dF, self.k2 = T.descs(finals, [t.data_ptr() for t in self.df])
        n = len(inits)
        self.dts = (C.c_int * n)(*[L.dtype for L in inits])
        self.ops = T.make_ops(ops, n)
        self.n = n

    def reset_finals(self):
        import torch
        for t, a in zip(self.df, self.fas):
            t.copy_(torch.from_numpy(a))
        torch.cuda.synchronize()

    def finals_host(self):
        import torch
        torch.cuda.synchronize()
        return [t.cpu().numpy() for t in self.df]


def test_plans_execute_matches_port():
    inits, finals, ias, fas, ops = _pool(40, 3)
    want = T.port_run(inits, finals, ias, fas, ops)
    d = Device(inits, finals, ias, fas, ops)
    lib = capi.load()
    plans = (C.c_void_p * d.n)()
    for k in range(d.n):
        p = C.c_void_p()
        capi.check(lib.g2g_plan_create(C.byref(d.dI[k]), C.byref(d.dF[k]), d.dts[k],
                                       C.byref(d.ops[k]), None, C.byref(p)))
        plans[k] = p.value
    import torch
    s = torch.cuda.Stream()
    capi.check(lib.g2g_plans_execute(d.n, plans, C.c_void_p(s.cuda_stream)))
    s.synchronize()
    got = d.finals_host()
    for k in range(d.n):
        T.assert_arenas_equal(got[k], want[k], finals[k], what=f"plans_execute pair {k}")
        capi.check(lib.g2g_plan_destroy(plans[k]))


def _server(lib, **kw):
    cfg = capi.ServerConfig()
    for k, v in kw.items():
        setattr(cfg, k, v)
    srv = C.c_void_p()
    capi.check(lib.g2g_server_create(C.byref(cfg), C.byref(srv)))
    return srv


@pytest.mark.parametrize("batch", [256, 1])
def test_server_same_alone_and_in_mix(batch):
    """Each request's result alone equals its result among concurrent ones,
    and both equal the oracle's."""
    inits, finals, ias, fas, ops = _pool(24, 11)
    want = T.port_run(inits, finals, ias, fas, ops)
    d = Device(inits, finals, ias, fas, ops)
    lib = capi.load()
    srv = _server(lib, max_batch_requests=batch, max_launches_in_flight=3)
    try:
        # alone: one request at a time
        alone = []
        for k in range(d.n):
            d.reset_finals()
            tk = C.c_uint64()
            capi.check(lib.g2g_server_submit(srv, C.byref(d.dI[k]), C.byref(d.dF[k]),
                                             d.dts[k], C.byref(d.ops[k]), C.byref(tk)))
            capi.check(lib.g2g_server_wait(srv, tk.value, -1, None))
            alone.append(d.finals_host()[k])
        # in the mix: all requests arrive within ~100 us
        d.reset_finals()
        n = d.n
        idx = (C.c_int32 * n)(*range(n))
        arr = (C.c_double * n)(*[k * 4e-6 for k in range(n)])
        times = (capi.RequestTimes * n)()
        capi.check(lib.g2g_server_replay(srv, n, d.dI, d.dF, d.dts, d.ops, n, idx, arr, times))
        mix = d.finals_host()
        stats = capi.ServerStats()
        capi.check(lib.g2g_server_get_stats(srv, C.byref(stats)))
    finally:
        capi.check(lib.g2g_server_destroy(srv))
    for k in range(d.n):
        T.assert_arenas_equal(alone[k], want[k], finals[k], what=f"alone {k}")
        T.assert_arenas_equal(mix[k], alone[k], finals[k], what=f"mix vs alone {k}")
        assert times[k].status == 0
        assert times[k].submit_ns <= times[k].launch_ns <= times[k].complete_ns
    assert stats.completed == 2 * d.n
    assert stats.plan_cache_hits >= d.n  # the mix reused the plans made alone
    if batch == 1:
        assert stats.launches == 2 * d.n
    else:
        assert max(times[k].batch_size for k in range(d.n)) >= 1


def test_server_budget_admission():
    inits, finals, ias, fas, ops = _pool(12, 5, max_dim=300)
    want = T.port_run(inits, finals, ias, fas, ops)
    d = Device(inits, finals, ias, fas, ops)
    lib = capi.load()
    biggest = max(L.m * L.n * L.esz for L in finals)
    # room for one request at a time: admission serialises them
    srv = _server(lib, hbm_budget_bytes=2 * biggest + 1)
    try:
        n = d.n
        idx = (C.c_int32 * n)(*range(n))
        arr = (C.c_double * n)(*([0.0] * n))
        times = (capi.RequestTimes * n)()
        capi.check(lib.g2g_server_replay(srv, n, d.dI, d.dF, d.dts, d.ops, n, idx, arr, times))
        stats = capi.ServerStats()
        capi.check(lib.g2g_server_get_stats(srv, C.byref(stats)))
        assert stats.inflight_bytes_peak <= 2 * biggest + 1
        got = d.finals_host()
        for k in range(n):
            T.assert_arenas_equal(got[k], want[k], finals[k], what=f"budget {k}")
    finally:
        capi.check(lib.g2g_server_destroy(srv))
    # a request larger than the whole budget is refused
    srv = _server(lib, hbm_budget_bytes=16)
    try:
        tk = C.c_uint64()
        st = lib.g2g_server_submit(srv, C.byref(d.dI[0]), C.byref(d.dF[0]), d.dts[0],
                                   C.byref(d.ops[0]), C.byref(tk))
        assert st == capi.ERROR_BUDGET
        assert b"budget" in lib.g2g_last_error_string()
    finally:
        capi.check(lib.g2g_server_destroy(srv))


def test_server_rejects_invalid_request():
    rng = np.random.default_rng(9)
    Li = Ls.random_grid_layout(40, 30, 3, capi.FLOAT32, rng, ext_hi=9)
    Lf = Ls.random_grid_layout(41, 30, 3, capi.FLOAT32, rng, ext_hi=9)  # other shape
    d = Device([Li], [Lf], [np.zeros(Li.arena_bytes, np.uint8)],
               [np.zeros(Lf.arena_bytes, np.uint8)], [("N", 1.0, 0.0)])
    lib = capi.load()
    srv = _server(lib)
    try:
        tk = C.c_uint64()
        st = lib.g2g_server_submit(srv, C.byref(d.dI[0]), C.byref(d.dF[0]), d.dts[0],
                                   C.byref(d.ops[0]), C.byref(tk))
        assert st == capi.ERROR_INVALID_ARGUMENT
        assert lib.g2g_server_wait(srv, 12345, 0, None) == capi.ERROR_INVALID_ARGUMENT
        stats = capi.ServerStats()
        capi.check(lib.g2g_server_get_stats(srv, C.byref(stats)))
        assert stats.submitted == 0
    finally:
        capi.check(lib.g2g_server_destroy(srv))
