"""Plain copies as 2-D tensor-map boxes (tuning tensor_boxes = 1): block
layouts at 16-byte aligned addresses with 16-byte multiple strides whose
pieces are whole boxes of one shape move through cp.async.bulk.tensor loads
and stores. Results must equal the oracle port's bit for bit, padding
included; plans that do not qualify run the ordinary kernels under the same
tuning."""
import ctypes as C

import numpy as np
import pytest

import g2g_testlib as T
import oracle
from grid2grid_gb300 import capi
from grid2grid_gb300 import layouts as Ls
from grid2grid_gb300 import workloads as W

pytestmark = pytest.mark.gpu

BOXES = dict(tensor_boxes=1)


@pytest.fixture(scope="module", autouse=True)
def _setup():
    import torch
    assert torch.cuda.is_available()
    from grid2grid_gb300 import build
    build.build()
    capi.load()
    oracle.build_port()


def _plan_ok(Li, Lf):
    import torch
    lib = capi.load()
    di = torch.zeros(Li.arena_bytes, dtype=torch.uint8, device="cuda")
    df = torch.zeros(Lf.arena_bytes, dtype=torch.uint8, device="cuda")
    dI, k1 = Li.desc(di.data_ptr())
    dF, k2 = Lf.desc(df.data_ptr())
    plan = C.c_void_p()
    capi.check(lib.g2g_plan_create(C.byref(dI), C.byref(dF), Li.dtype, None, None,
                                   C.byref(plan)))
    info = capi.PlanInfo()
    capi.check(lib.g2g_plan_get_info(plan, C.byref(info)))
    capi.check(lib.g2g_plan_destroy(plan))
    return info.tensor_boxes_ok


def test_block_cyclic_f64_4096_known_answer_as_boxes():
    """entry(i, j) = i + j * 4096 lands at (i, j) of the 128 x 64 layout."""
    import torch
    w = W.block_cyclic_f64_4096()
    assert _plan_ok(w.inits[0], w.finals[0]) == 1
    ia, fa = W.fill_arenas(w)
    for how in ("plan", "graph"):
        got = T.gpu_run(w.inits, w.finals, ia, fa, how=how, tuning=BOXES, executes=2)[0]
        v = w.finals[0].gather(got).view(np.float64)
        m = 4096
        want = (np.arange(m, dtype=np.float64)[:, None]
                + np.arange(m, dtype=np.float64)[None, :] * m)
        assert np.array_equal(v, want), how
    torch.cuda.synchronize()


@pytest.mark.parametrize("dt", [capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64, capi.COMPLEX128])
def test_block_cyclic_pairs_as_boxes_match_port(dt):
    """Block-cyclic pairs whose block sizes share a factor, several grids and
    rank orders, local arrays padded (lld above the local rows)."""
    rng = np.random.default_rng(60 + dt)
    esz = capi.DTYPE_SIZE[dt]
    q = max(1, 16 // esz)  # rows of 16 bytes
    for _ in range(3):
        f = int(rng.choice([4, 8])) * q * 4  # boxes of at least 4 KB
        m, n = f * int(rng.integers(3, 20)), f * int(rng.integers(3, 20))
        pr, pc = int(rng.integers(1, 4)), int(rng.integers(1, 4))
        mb1, nb1 = f * int(rng.integers(1, 4)), f * int(rng.integers(1, 4))
        mb2, nb2 = f * int(rng.integers(1, 5)), f * int(rng.integers(1, 5))
        lld1 = Ls.scalapack_lld(m, mb1, pr, pc, 0) + q * int(rng.integers(0, 3))
        Li = Ls.scalapack_layout(m, n, mb1, nb1, pr, pc, dt, row_major=bool(rng.random() < 0.5),
                                 lld=[lld1 + 0 * r for r in range(pr * pc)])
        Lf = Ls.scalapack_layout(m, n, mb2, nb2, pc, pr, dt)
        assert _plan_ok(Li, Lf) == 1, (m, n, mb1, nb1, mb2, nb2, lld1)
        ai = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
        af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
        want = T.port_run([Li], [Lf], [ai], [af])[0]
        got = T.gpu_run([Li], [Lf], [ai], [af], how="plan", tuning=BOXES, executes=2)[0]
        T.assert_arenas_equal(got, want, Lf, what=f"boxes dt{dt} {m}x{n}")


def test_plans_that_do_not_qualify_run_as_before():
    """Random grids (odd strides), a transpose, alpha/beta: tensor_boxes is
    ignored and the results stay the port's."""
    rng = np.random.default_rng(77)
    Li = Ls.random_grid_layout(300, 200, 5, capi.FLOAT32, rng, ext_hi=90)
    Lf = Ls.random_grid_layout(300, 200, 5, capi.FLOAT32, rng, ext_hi=90)
    assert _plan_ok(Li, Lf) == 0
    ai = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
    af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    want = T.port_run([Li], [Lf], [ai], [af])[0]
    got = T.gpu_run([Li], [Lf], [ai], [af], how="plan", tuning=BOXES)[0]
    T.assert_arenas_equal(got, want, Lf, what="random grids")
    Li = Ls.scalapack_layout(256, 192, 32, 32, 2, 2, capi.FLOAT64)
    Lf = Ls.scalapack_layout(192, 256, 64, 32, 2, 2, capi.FLOAT64)
    ai = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
    af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    for op in (("T", 1.0, 0.0), ("N", 2.0, 0.5)):
        Lfo = Lf if op[0] == "T" else Ls.scalapack_layout(256, 192, 64, 32, 2, 2, capi.FLOAT64)
        afo = af if op[0] == "T" else Ls.fill_random(np.zeros(Lfo.arena_bytes, np.uint8), rng)
        if op[0] == "N":
            ai2 = np.frombuffer(rng.standard_normal(Li.arena_bytes // 8).tobytes(), np.uint8).copy()
            afo = np.frombuffer(rng.standard_normal(Lfo.arena_bytes // 8).tobytes(), np.uint8).copy()
        else:
            ai2 = ai
        want = T.port_run([Li], [Lfo], [ai2], [afo], [op])[0]
        got = T.gpu_run([Li], [Lfo], [ai2], [afo], [op], how="plan", tuning=BOXES)[0]
        T.assert_arenas_equal(got, want, Lfo, what=f"boxes ignored {op}")


def test_autotune_may_pick_boxes_and_stays_exact():
    import torch
    lib = capi.load()
    w = W.block_cyclic_f64_4096(1024)
    ia, fa = W.fill_arenas(w)
    di = torch.from_numpy(ia[0]).cuda()
    df = torch.from_numpy(fa[0]).cuda()
    dI, k1 = w.inits[0].desc(di.data_ptr())
    dF, k2 = w.finals[0].desc(df.data_ptr())
    s = torch.cuda.Stream()
    sp = C.c_void_p(s.cuda_stream)
    plan = C.c_void_p()
    capi.check(lib.g2g_plan_create(C.byref(dI), C.byref(dF), capi.FLOAT64, None, sp,
                                   C.byref(plan)))
    t = capi.Tuning()
    capi.check(lib.g2g_plan_autotune(plan, sp, 1, C.byref(t)))
    assert t.tensor_boxes in (-1, 1)
    capi.check(lib.g2g_plan_execute(plan, sp))
    s.synchronize()
    info = capi.PlanInfo()
    capi.check(lib.g2g_plan_get_info(plan, C.byref(info)))
    assert info.device_status == 0
    capi.check(lib.g2g_plan_destroy(plan))
    got = w.finals[0].gather(df.cpu().numpy()).view(np.float64)
    m = 1024
    want = np.arange(m, dtype=np.float64)[:, None] + np.arange(m, dtype=np.float64)[None, :] * m
    assert np.array_equal(got, want)
