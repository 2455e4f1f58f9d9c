"""Plain transposes of one narrow element size as a launch's only tiles (tile
path 64: float; 128: double and complex<float>), and scaled ones (1024,
2048): their source lines (and for scaled tiles the destination columns)
are staged raw through a ring of shared-memory stages with cp.async and
stored at each line's phase. Results must equal the oracle port's bit for bit,
padding included, under every tile edge and CTA size (and on the register
path that the tuning's ring = -1 selects instead), for plans, graphs,
one-shot calls, batches and multi-plan launches, at 8- and 4-byte aligned
addresses; plans that mix them with other tiles keep the other kernels and
stay exact too."""
import ctypes as C

import numpy as np
import pytest

import g2g_testlib as T
import oracle
from grid2grid_gb300 import capi
from grid2grid_gb300 import layouts as Ls

pytestmark = pytest.mark.gpu

STAGED = 64
STAGED8 = 128


def _staged(paths, bit=STAGED):
    """The launch runs the staged ring: its bit and no tiles but transposes."""
    return bool(paths & bit) and (paths & ~(bit | 32)) == 2


@pytest.fixture(scope="module", autouse=True)
def _setup():
    import torch
    assert torch.cuda.is_available()
    from grid2grid_gb300 import build
    build.build()
    capi.load()
    oracle.build_port()


def _tile_paths(inits, finals, ops):
    import torch
    lib = capi.load()
    di = [torch.zeros(L.arena_bytes, dtype=torch.uint8, device="cuda") for L in inits]
    df = [torch.zeros(L.arena_bytes, dtype=torch.uint8, device="cuda") for L in finals]
    dI, k1 = T.descs(inits, [t.data_ptr() for t in di])
    dF, k2 = T.descs(finals, [t.data_ptr() for t in df])
    n = len(inits)
    dts = (C.c_int * n)(*[L.dtype for L in inits])
    plan = C.c_void_p()
    capi.check(lib.g2g_plan_create_batch(n, dI, dF, dts, T.make_ops(ops, n), None,
                                         C.byref(plan)))
    info = capi.PlanInfo()
    capi.check(lib.g2g_plan_get_info(plan, C.byref(info)))
    capi.check(lib.g2g_plan_destroy(plan))
    return info.tile_paths


def _float_pair(rng, m, n, t, ext_hi=90, P=5, mis=(0, 0), dt=capi.FLOAT32, byte_mis=(0, 0)):
    Li = Ls.random_grid_layout(n, m, P, dt, rng, ext_hi=ext_hi, base_misalign=mis[0],
                               byte_misalign=byte_mis[0])
    Lf = Ls.random_grid_layout(m, n, P, dt, rng, ext_hi=ext_hi, base_misalign=mis[1],
                               byte_misalign=byte_mis[1])
    ai = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
    af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    return Li, Lf, ai, af, (t, 1.0, 0.0)


TUNINGS = [None, dict(tile_dim=16), dict(threads=512), dict(tile_dim=16, threads=512),
           dict(ctas_per_sm=1), dict(ctas_per_sm=2, threads=512), dict(ring=-1)]


@pytest.mark.parametrize("tuning", TUNINGS)
def test_float_transposes_staged_match_port(tuning):
    """Random grids with padded strides, edge tiles in both directions
    (sizes not multiples of the 2 td x (2 td - 4) tile), 'T' and 'C'."""
    rng = np.random.default_rng(900 + TUNINGS.index(tuning))
    for t, (m, n) in (("T", (611, 437)), ("C", (389, 700))):
        Li, Lf, ai, af, op = _float_pair(rng, m, n, t)
        assert _staged(_tile_paths([Li], [Lf], [op]))
        want = T.port_run([Li], [Lf], [ai], [af], [op])[0]
        for how in ("plan", "graph"):
            got = T.gpu_run([Li], [Lf], [ai], [af], [op], how=how, tuning=tuning,
                            executes=2)[0]
            T.assert_arenas_equal(got, want, Lf, what=f"{t} {how} {tuning}")


@pytest.mark.parametrize("mis", [(1, 2), (3, 0), (2, 3)])
def test_misaligned_bases_and_tiny_tiles_staged(mis):
    """Blocks at any 4-byte phase, grids with many 1-wide splits (tiles of
    one row or one column)."""
    rng = np.random.default_rng(930 + mis[0] * 4 + mis[1])
    Li, Lf, ai, af, op = _float_pair(rng, 300, 200, "T", ext_hi=70, P=7, mis=mis)
    assert _staged(_tile_paths([Li], [Lf], [op]))
    want = T.port_run([Li], [Lf], [ai], [af], [op])[0]
    got = T.gpu_run([Li], [Lf], [ai], [af], [op], how="transform")[0]
    T.assert_arenas_equal(got, want, Lf, what=f"misaligned {mis}")
    Li = Ls.random_grid_layout(130, 97, 9, capi.FLOAT32, rng, ext_hi=3, base_misalign=mis[0])
    Lf = Ls.random_grid_layout(97, 130, 9, capi.FLOAT32, rng, ext_hi=5, base_misalign=mis[1])
    ai = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
    af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    op = ("T", 1.0, 0.0)
    want = T.port_run([Li], [Lf], [ai], [af], [op])[0]
    got = T.gpu_run([Li], [Lf], [ai], [af], [op], how="plan", tuning=dict(tile_dim=16))[0]
    T.assert_arenas_equal(got, want, Lf, what=f"thin splits {mis}")


def test_batches_staged_and_mixed():
    """A batch of float transposes runs staged; adding a double transpose or
    a plain float copy to it takes the batch off the staged ring, and every
    result stays the port's."""
    rng = np.random.default_rng(950)
    pairs = [_float_pair(rng, int(rng.integers(40, 500)), int(rng.integers(40, 500)),
                         "TC"[k % 2]) for k in range(5)]
    Lis, Lfs, ais, afs, ops = map(list, zip(*pairs))
    assert _staged(_tile_paths(Lis, Lfs, ops))
    want = T.port_run(Lis, Lfs, ais, afs, ops)
    for how in ("batch", "plan"):
        got = T.gpu_run(Lis, Lfs, ais, afs, ops, how=how)
        for k in range(len(Lis)):
            T.assert_arenas_equal(got[k], want[k], Lfs[k], what=f"{how} pair {k}")
    # + a double transpose, + a float copy
    Ld_i = Ls.random_grid_layout(150, 210, 4, capi.FLOAT64, rng, ext_hi=40)
    Ld_f = Ls.random_grid_layout(210, 150, 4, capi.FLOAT64, rng, ext_hi=40)
    Lc_i = Ls.random_grid_layout(180, 120, 4, capi.FLOAT32, rng, ext_hi=40)
    Lc_f = Ls.random_grid_layout(180, 120, 4, capi.FLOAT32, rng, ext_hi=40)
    for extra_i, extra_f, extra_op in ((Ld_i, Ld_f, ("T", 1.0, 0.0)),
                                      (Lc_i, Lc_f, ("N", 1.0, 0.0))):
        Li2, Lf2 = Lis + [extra_i], Lfs + [extra_f]
        ops2 = ops + [extra_op]
        ai2 = ais + [Ls.fill_random(np.zeros(extra_i.arena_bytes, np.uint8), rng)]
        af2 = afs + [Ls.fill_random(np.zeros(extra_f.arena_bytes, np.uint8), rng)]
        assert not _staged(_tile_paths(Li2, Lf2, ops2))
        want2 = T.port_run(Li2, Lf2, ai2, af2, ops2)
        got2 = T.gpu_run(Li2, Lf2, ai2, af2, ops2, how="plan")
        for k in range(len(Li2)):
            T.assert_arenas_equal(got2[k], want2[k], Lf2[k], what=f"mixed pair {k}")


def test_multi_plan_launch_staged_and_mixed():
    """g2g_plans_execute over cached plans: float transposes only (staged),
    then with a plan of plain copies among them (not staged)."""
    import torch
    lib = capi.load()
    rng = np.random.default_rng(970)
    pairs = [_float_pair(rng, int(rng.integers(60, 400)), int(rng.integers(60, 400)), "T")
             for _ in range(3)]
    Lc_i = Ls.random_grid_layout(220, 160, 4, capi.FLOAT32, rng, ext_hi=40)
    Lc_f = Ls.random_grid_layout(220, 160, 4, capi.FLOAT32, rng, ext_hi=40)
    copy_pair = (Lc_i, Lc_f, Ls.fill_random(np.zeros(Lc_i.arena_bytes, np.uint8), rng),
                 Ls.fill_random(np.zeros(Lc_f.arena_bytes, np.uint8), rng), ("N", 1.0, 0.0))
    s = torch.cuda.Stream()
    sp = C.c_void_p(s.cuda_stream)
    for group in (pairs, pairs + [copy_pair]):
        keep, plans, outs = [], [], []
        for Li, Lf, ai, af, op in group:
            di = torch.from_numpy(ai).cuda()
            df = torch.from_numpy(af).cuda()
            dI, k1 = T.descs([Li], [di.data_ptr()])
            dF, k2 = T.descs([Lf], [df.data_ptr()])
            keep += [di, df, k1, k2]
            plan = C.c_void_p()
            capi.check(lib.g2g_plan_create(dI, dF, Li.dtype, T.make_ops([op], 1), sp,
                                           C.byref(plan)))
            plans.append(plan)
            outs.append(df)
        arr = (C.c_void_p * len(plans))(*[p.value for p in plans])
        for _ in range(2):
            capi.check(lib.g2g_plans_execute(len(plans), arr, sp))
        s.synchronize()
        for p in plans:
            capi.check(lib.g2g_plan_destroy(p))
        for (Li, Lf, ai, af, op), df in zip(group, outs):
            want = T.port_run([Li], [Lf], [ai], [af], [op])[0]
            T.assert_arenas_equal(df.cpu().numpy(), want, Lf, what=f"multi {len(group)}")


@pytest.mark.parametrize("dt", [capi.FLOAT64, capi.COMPLEX64])
@pytest.mark.parametrize("tuning", [None, dict(tile_dim=16), dict(threads=512), dict(ring=-1)])
def test_eight_byte_transposes_staged_match_port(dt, tuning):
    """Double and complex<float> 'T' / 'C' on random grids (8-byte aligned:
    one 8-byte read and store per element), then complex<float> blocks at
    4-byte aligned addresses (two 4-byte halves per element)."""
    rng = np.random.default_rng(990 + dt * 7 + (0 if tuning is None else len(str(tuning))))
    cases = [("T", (433, 611), (0, 0)), ("C", (700, 389), (0, 0))]
    if dt == capi.COMPLEX64:
        cases += [("C", (301, 257), (4, 0)), ("T", (257, 301), (0, 4)), ("T", (199, 211), (4, 4))]
    for t, (m, n), bm in cases:
        Li, Lf, ai, af, op = _float_pair(rng, m, n, t, dt=dt, byte_mis=bm)
        assert _staged(_tile_paths([Li], [Lf], [op]), STAGED8)
        want = T.port_run([Li], [Lf], [ai], [af], [op])[0]
        for how in ("plan", "graph"):
            got = T.gpu_run([Li], [Lf], [ai], [af], [op], how=how, tuning=tuning,
                            executes=2)[0]
            T.assert_arenas_equal(got, want, Lf, what=f"dt{dt} {t} {bm} {how} {tuning}")


def test_eight_byte_batches_and_mixed():
    """A batch of double and complex<float> transposes runs staged; a float
    transpose among them takes it off the ring; results stay the port's."""
    rng = np.random.default_rng(1010)
    pairs = [_float_pair(rng, int(rng.integers(40, 400)), int(rng.integers(40, 400)),
                         "TC"[k % 2], dt=(capi.FLOAT64, capi.COMPLEX64)[k % 2]) for k in range(4)]
    Lis, Lfs, ais, afs, ops = map(list, zip(*pairs))
    assert _staged(_tile_paths(Lis, Lfs, ops), STAGED8)
    want = T.port_run(Lis, Lfs, ais, afs, ops)
    got = T.gpu_run(Lis, Lfs, ais, afs, ops, how="plan")
    for k in range(len(Lis)):
        T.assert_arenas_equal(got[k], want[k], Lfs[k], what=f"pair {k}")
    Li, Lf, ai, af, op = _float_pair(rng, 120, 90, "T")
    Li2, Lf2, ai2, af2, ops2 = Lis + [Li], Lfs + [Lf], ais + [ai], afs + [af], ops + [op]
    paths = _tile_paths(Li2, Lf2, ops2)
    assert not _staged(paths, STAGED8) and not _staged(paths, STAGED)
    want2 = T.port_run(Li2, Lf2, ai2, af2, ops2)
    got2 = T.gpu_run(Li2, Lf2, ai2, af2, ops2, how="plan")
    for k in range(len(Li2)):
        T.assert_arenas_equal(got2[k], want2[k], Lf2[k], what=f"mixed pair {k}")


STAGED_SC4, STAGED_SC8 = 1024, 2048


def _scaled_staged(paths, bit):
    return bool(paths & bit) and not (paths & ~(4 | 8 | bit))


def _normal_arena(rng, L, dt):
    comp = np.float32 if dt in (capi.FLOAT32, capi.COMPLEX64) else np.float64
    return np.frombuffer(rng.standard_normal(L.arena_bytes // np.dtype(comp).itemsize)
                         .astype(comp).tobytes(), np.uint8).copy()


@pytest.mark.parametrize("dt", [capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64])
@pytest.mark.parametrize("tuning", [None, dict(tile_dim=16), dict(threads=512), dict(ring=-1)])
def test_scaled_transposes_staged_match_port(dt, tuning):
    """final = beta * final + alpha * op(initial) with every tile a scaled
    transpose of one element size (tile paths 1024 / 2048): source lines and
    destination columns staged; 'T' and 'C', several coefficient forms,
    4-byte aligned complex<float> blocks; finite values, bit for bit."""
    rng = np.random.default_rng(1200 + dt * 5 + (0 if tuning is None else len(str(tuning))))
    bit = STAGED_SC4 if dt == capi.FLOAT32 else STAGED_SC8
    coefs = [(2.0, 0.5), (1.0, 1.0), (-0.75, 0.0), (0.5, -1.5)]
    cases = [("T", (433, 301), (0, 0)), ("C", (280, 377), (0, 0))]
    if dt == capi.COMPLEX64:
        cases.append(("C", (211, 173), (4, 4)))
    for k, (t, (m, n), bm) in enumerate(cases):
        Li, Lf, _, _, _ = _float_pair(rng, m, n, t, dt=dt, byte_mis=bm, ext_hi=120)
        ai, af = _normal_arena(rng, Li, dt), _normal_arena(rng, Lf, dt)
        a, b = coefs[k % len(coefs)]
        op = (t, a, b)
        assert _scaled_staged(_tile_paths([Li], [Lf], [op]), bit)
        want = T.port_run([Li], [Lf], [ai], [af], [op])[0]
        for how in ("plan", "graph"):
            got = T.gpu_run([Li], [Lf], [ai], [af], [op], how=how, tuning=tuning, executes=1)[0]
            T.assert_arenas_equal(got, want, Lf, what=f"scaled dt{dt} {op} {bm} {how} {tuning}")


def test_scaled_transposes_batch_and_mixed():
    """A batch of scaled double and complex<float> transposes runs staged;
    with a plain transpose or a scaled copy among them it does not; results
    stay the port's."""
    rng = np.random.default_rng(1300)
    pairs, ops = [], []
    for k in range(4):
        dt = (capi.FLOAT64, capi.COMPLEX64)[k % 2]
        Li, Lf, _, _, _ = _float_pair(rng, int(rng.integers(50, 300)), int(rng.integers(50, 300)),
                                      "TC"[k % 2], dt=dt, ext_hi=100)
        pairs.append((Li, Lf, _normal_arena(rng, Li, dt), _normal_arena(rng, Lf, dt)))
        ops.append(("TC"[k % 2], 1.5, -0.25))
    Lis, Lfs, ais, afs = map(list, zip(*pairs))
    assert _scaled_staged(_tile_paths(Lis, Lfs, ops), STAGED_SC8)
    want = T.port_run(Lis, Lfs, ais, afs, ops)
    got = T.gpu_run(Lis, Lfs, ais, afs, ops, how="plan")
    for k in range(len(Lis)):
        T.assert_arenas_equal(got[k], want[k], Lfs[k], what=f"scaled batch pair {k}")
    Lx, Ly, _, _, _ = _float_pair(rng, 120, 90, "T", dt=capi.FLOAT64)
    Lc_i = Ls.random_grid_layout(110, 95, 4, capi.FLOAT64, rng, ext_hi=40)
    Lc_f = Ls.random_grid_layout(110, 95, 4, capi.FLOAT64, rng, ext_hi=40)
    for Li, Lf, op in ((Lx, Ly, ("T", 1.0, 0.0)), (Lc_i, Lc_f, ("N", 2.0, 0.5))):
        Li2, Lf2, ops2 = Lis + [Li], Lfs + [Lf], ops + [op]
        ai2 = ais + [_normal_arena(rng, Li, capi.FLOAT64)]
        af2 = afs + [_normal_arena(rng, Lf, capi.FLOAT64)]
        assert not _scaled_staged(_tile_paths(Li2, Lf2, ops2), STAGED_SC8)
        want2 = T.port_run(Li2, Lf2, ai2, af2, ops2)
        got2 = T.gpu_run(Li2, Lf2, ai2, af2, ops2, how="plan")
        for k in range(len(Li2)):
            T.assert_arenas_equal(got2[k], want2[k], Lf2[k], what=f"scaled mixed pair {k}")


STAGED16 = 256


@pytest.mark.parametrize("tuning", [None, dict(tile_dim=16), dict(threads=512), dict(ring=-1)])
def test_complex_double_transposes_staged_match_port(tuning):
    """complex<double> 'T' / 'C' (tile path 256) at 16-byte aligned addresses
    (one 16-byte read and store per element), with blocks at 8-byte aligned
    ones (4-byte words), and a block-cyclic pair."""
    rng = np.random.default_rng(1030 + (0 if tuning is None else len(str(tuning))))
    for t, (m, n), bm in (("T", (233, 301), (0, 0)), ("C", (300, 180), (0, 0)),
                          ("T", (150, 211), (8, 0)), ("C", (211, 150), (0, 8)),
                          ("T", (97, 131), (8, 8))):
        Li, Lf, ai, af, op = _float_pair(rng, m, n, t, dt=capi.COMPLEX128, byte_mis=bm, ext_hi=70)
        assert _staged(_tile_paths([Li], [Lf], [op]), STAGED16)
        want = T.port_run([Li], [Lf], [ai], [af], [op])[0]
        for how in ("plan", "graph"):
            got = T.gpu_run([Li], [Lf], [ai], [af], [op], how=how, tuning=tuning,
                            executes=2)[0]
            T.assert_arenas_equal(got, want, Lf, what=f"c128 {t} {bm} {how} {tuning}")
    Li = Ls.scalapack_layout(512, 384, 64, 64, 2, 2, capi.COMPLEX128)
    Lf = Ls.scalapack_layout(384, 512, 96, 40, 2, 2, capi.COMPLEX128)
    ai = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
    af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    op = ("T", 1.0, 0.0)
    assert _staged(_tile_paths([Li], [Lf], [op]), STAGED16)
    want = T.port_run([Li], [Lf], [ai], [af], [op])[0]
    got = T.gpu_run([Li], [Lf], [ai], [af], [op], how="plan", tuning=tuning)[0]
    T.assert_arenas_equal(got, want, Lf, what=f"c128 block-cyclic {tuning}")
