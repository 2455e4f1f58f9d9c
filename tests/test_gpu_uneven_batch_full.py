"""Parity of the batched and served paths at their benchmark size.

The uneven batch is the 256-redistribution workload the benchmark times
(m, n log-uniform in [64, 8192], float / double / complex<float>, 4-64 virtual
ranks, block-cyclic or random-split layouts; about 311 000 pieces). It runs
through every path a caller of the batched API takes, each launch over the
whole work list:

  * one batch plan (the vector transform, transform.cpp:184-204 /
    transformer.hpp:44-53), autotuned, captured as a CUDA graph and replayed;
  * the 256 cached per-transform plans as one multi-plan launch;
  * an open-loop Poisson stream of requests drawn from the same 256 pairs
    through the continuous-batching server.

Every destination arena -- padding bytes included -- must equal the oracle
port's result, bit for bit. The port runs pair by pair in groups so that the
host holds a few GB at a time."""
import ctypes as C

import numpy as np
import pytest

import g2g_testlib as T
import oracle
from grid2grid_gb300 import capi
from grid2grid_gb300 import workloads as W

pytestmark = pytest.mark.gpu

GROUP = 32  # pairs the port checks at a time


@pytest.fixture(scope="module")
def batch():
    import torch
    assert torch.cuda.is_available()
    from grid2grid_gb300 import build
    build.build()
    capi.load()
    oracle.build_port()
    w = W.uneven_batch(256)
    g = torch.Generator(device="cuda")
    g.manual_seed(77)
    di = [torch.randint(0, 256, (L.arena_bytes,), dtype=torch.uint8, device="cuda",
                        generator=g) for L in w.inits]
    df0 = [torch.randint(0, 256, (L.arena_bytes,), dtype=torch.uint8, device="cuda",
                         generator=g) for L in w.finals]
    df = [t.clone() for t in df0]
    dI, k1 = T.descs(w.inits, [t.data_ptr() for t in di])
    dF, k2 = T.descs(w.finals, [t.data_ptr() for t in df])
    n = len(w.inits)
    dts = (C.c_int * n)(*w.dtypes())
    yield dict(w=w, di=di, df0=df0, df=df, dI=dI, dF=dF, dts=dts, n=n, keep=(k1, k2))
    del di, df0, df
    torch.cuda.empty_cache()


def _reset(b):
    import torch
    for t, t0 in zip(b["df"], b["df0"]):
        t.copy_(t0)
    torch.cuda.synchronize()


def _check_against_port(b, what, pairs=None):
    """Every pair in `pairs` (all by default) equals the port's result; the
    others still hold their original bytes."""
    import torch
    torch.cuda.synchronize()
    w = b["w"]
    n = b["n"]
    chosen = set(range(n) if pairs is None else pairs)
    for g0 in range(0, n, GROUP):
        ks = [k for k in range(g0, min(n, g0 + GROUP)) if k in chosen]
        if ks:
            ia = [b["di"][k].cpu().numpy() for k in ks]
            want = [b["df0"][k].cpu().numpy() for k in ks]
            oracle.port_transform([w.inits[k] for k in ks], [w.finals[k] for k in ks], ia,
                                  want, None, threads=16)
            for k, wk in zip(ks, want):
                T.assert_arenas_equal(b["df"][k].cpu().numpy(), wk, w.finals[k],
                                      what=f"{what} pair {k}")
            del ia, want
        for k in range(g0, min(n, g0 + GROUP)):
            if k not in chosen:
                assert torch.equal(b["df"][k], b["df0"][k]), f"{what}: pair {k} was written"


def test_batch_plan_autotuned_graph_matches_port(batch):
    """g2g_plan_create_batch -> g2g_plan_autotune -> g2g_plan_capture_graph ->
    g2g_plan_execute: one launch over the 256 pairs, the benchmark's path."""
    import torch
    b = batch
    lib = capi.load()
    s = torch.cuda.Stream()
    sp = C.c_void_p(s.cuda_stream)
    plan = C.c_void_p()
    capi.check(lib.g2g_plan_create_batch(b["n"], b["dI"], b["dF"], b["dts"], None, sp,
                                         C.byref(plan)))
    try:
        info = capi.PlanInfo()
        capi.check(lib.g2g_plan_get_info(plan, C.byref(info)))
        assert info.n_pairs == 256 and info.n_pieces > 250_000
        assert info.bytes_moved == b["w"].bytes_moved
        tuned = capi.Tuning()
        capi.check(lib.g2g_plan_autotune(plan, sp, 1, C.byref(tuned)))
        _reset(b)
        capi.check(lib.g2g_plan_capture_graph(plan, sp))
        for _ in range(2):  # graph replays; the copy is idempotent
            capi.check(lib.g2g_plan_execute(plan, sp))
        s.synchronize()
        capi.check(lib.g2g_plan_get_info(plan, C.byref(info)))
        assert info.graph_captured == 1 and info.device_status == 0
        _check_against_port(b, f"batch plan (tuning {tuned.tile_bytes}B tiles, "
                               f"{tuned.threads} threads, ring {tuned.ring})")
    finally:
        capi.check(lib.g2g_plan_destroy(plan))


def test_multi_plan_launch_matches_port(batch):
    """The 256 cached per-transform plans executed as one launch
    (g2g_plans_execute), and one launch per plan back to back."""
    import torch
    b = batch
    lib = capi.load()
    s = torch.cuda.Stream()
    sp = C.c_void_p(s.cuda_stream)
    n = b["n"]
    plans = (C.c_void_p * n)()
    try:
        for k in range(n):
            p = C.c_void_p()
            capi.check(lib.g2g_plan_create(C.byref(b["dI"][k]), C.byref(b["dF"][k]),
                                           b["dts"][k], None, sp, C.byref(p)))
            plans[k] = p.value
        _reset(b)
        capi.check(lib.g2g_plans_execute(n, plans, sp))
        s.synchronize()
        _check_against_port(b, "multi-plan launch")
        _reset(b)
        for k in range(n):
            capi.check(lib.g2g_plan_execute(plans[k], sp))
        s.synchronize()
        _check_against_port(b, "plain launches")
    finally:
        for k in range(n):
            if plans[k]:
                capi.check(lib.g2g_plan_destroy(plans[k]))


def test_served_poisson_stream_matches_port(batch):
    """An open-loop Poisson stream (20k requests/s) drawn from the 256 pairs
    through the continuous-batching server: requests that arrive while others
    are on the GPU are merged into shared launches. Every requested pair ends
    equal to its result alone (the port's), every other pair is untouched."""
    b = batch
    lib = capi.load()
    n = b["n"]
    cfg = capi.ServerConfig()
    cfg.hbm_budget_bytes = 120 * 10**9
    cfg.max_batch_requests = 256
    cfg.max_launches_in_flight = 3
    srv = C.c_void_p()
    capi.check(lib.g2g_server_create(C.byref(cfg), C.byref(srv)))
    try:
        rng = np.random.default_rng(2027)
        N = 600
        arrivals = np.cumsum(rng.exponential(1.0 / 20000, size=N)).astype(np.float64)
        # a third of the pairs are never requested: they must stay untouched
        pool = rng.permutation(n)[: 2 * n // 3]
        pick = rng.choice(pool, size=N).astype(np.int32)
        _reset(b)
        times = (capi.RequestTimes * N)()
        capi.check(lib.g2g_server_replay(srv, n, b["dI"], b["dF"], b["dts"], None, N,
                                         pick.ctypes.data_as(C.POINTER(C.c_int32)),
                                         arrivals.ctypes.data_as(C.POINTER(C.c_double)),
                                         times))
        t = np.ctypeslib.as_array(times)
        assert np.all(t["status"] == 0)
        assert t["batch_size"].max() > 1, "no two requests shared a launch"
        stats = capi.ServerStats()
        capi.check(lib.g2g_server_get_stats(srv, C.byref(stats)))
        assert stats.completed >= N
        _check_against_port(b, "served stream", pairs=sorted(set(pick.tolist())))
    finally:
        capi.check(lib.g2g_server_destroy(srv))
