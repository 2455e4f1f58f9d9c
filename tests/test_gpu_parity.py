"""GPU parity through the C ABI: the device gather-scatter must reproduce the
reference bit for bit -- every golden vector the reference produced, and the
oracle port on fresh seeded cases of every dtype and op -- including every
padding byte of the destination, which must stay untouched. Full-size
workloads are checked against the port and through size-independent
properties (round trips, conservation of the element multiset)."""
import ctypes as C

import numpy as np
import pytest

import g2g_testlib as T
import oracle
from grid2grid_gb300 import capi
from grid2grid_gb300 import layouts as Ls
from grid2grid_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _setup():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    from grid2grid_gb300 import build
    build.build()
    capi.load()
    oracle.build_port()


def _how_for(mode):
    return "transform" if mode in (oracle.MODE_SINGLE, oracle.MODE_SINGLE_SCALED) else "batch"


def test_golden_transforms_on_gpu(golden):
    n = 0
    for c in golden.cases():
        how = _how_for(c["mode"])
        if how == "transform" and len(c["inits"]) == 1:
            got = T.gpu_run(c["inits"], c["finals"], c["init_arenas"], c["final_before"],
                            c["ops"], how="transform")
        else:
            got = T.gpu_run(c["inits"], c["finals"], c["init_arenas"], c["final_before"],
                            c["ops"], how="batch")
        for k, (g, w) in enumerate(zip(got, c["final_after"])):
            T.assert_arenas_equal(g, w, c["finals"][k], what=f"{c['name']} pair {k}")
        n += 1
    assert n >= 60


def test_golden_covers_on_gpu(golden):
    lib = capi.load()
    for rec in golden.covers:
        a = np.array(rec["a"], np.int32)
        b = np.array(rec["b"], np.int32)
        s = np.zeros(max(len(a) - 1, 1), np.int32)
        e = np.zeros(max(len(a) - 1, 1), np.int32)
        IP = C.POINTER(C.c_int32)
        capi.check(lib.g2g_grid_cover(a.ctypes.data_as(IP), len(a), b.ctypes.data_as(IP),
                                      len(b), s.ctypes.data_as(IP), e.ctypes.data_as(IP),
                                      None))
        assert s[:len(a) - 1].tolist() == rec["start"]
        assert e[:len(a) - 1].tolist() == rec["end"]


def _random_case(rng, dt, t, m, n, P, **kw):
    Li = Ls.random_grid_layout(m if t == "N" else n, n if t == "N" else m, P, dt, rng, **kw)
    Lf = Ls.random_grid_layout(m, n, P, dt, rng, **kw)
    ai = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
    af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    return Li, Lf, ai, af


@pytest.mark.parametrize("dt", [capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64, capi.COMPLEX128])
@pytest.mark.parametrize("t", ["N", "T", "C"])
@pytest.mark.parametrize("seed", [0, 1])
def test_random_grids_match_port(dt, t, seed):
    rng = np.random.default_rng(100 * seed + 10 * dt + "NTC".index(t))
    m, n = int(rng.integers(1, 700)), int(rng.integers(1, 700))
    P = int(rng.integers(1, 20))
    Li, Lf, ai, af = _random_case(rng, dt, t, m, n, P, ext_hi=int(rng.integers(1, 300)),
                                  align=int(rng.choice([16, 256])))
    ops = [(t, 1.0, 0.0)]
    want = T.port_run([Li], [Lf], [ai], [af], ops)[0]
    got = T.gpu_run([Li], [Lf], [ai], [af], ops)[0]
    T.assert_arenas_equal(got, want, Lf, what=f"dt{dt} {t} m{m} n{n} P{P}")


@pytest.mark.parametrize("dt", [capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64, capi.COMPLEX128])
@pytest.mark.parametrize("misalign", [1, 2, 3])
def test_misaligned_bases_match_port(dt, misalign):
    """Blocks starting at any element-aligned address (not 16-byte aligned)."""
    rng = np.random.default_rng(7 + misalign + 10 * dt)
    esz = capi.DTYPE_SIZE[dt]
    mis = misalign if esz == 4 else (misalign % 2 if esz == 8 else 0)
    for t in "NT":
        Li = Ls.random_grid_layout(300 if t == "N" else 200, 200 if t == "N" else 300, 5, dt,
                                   rng, ext_hi=90, base_misalign=mis)
        Lf = Ls.random_grid_layout(300, 200, 5, dt, rng, ext_hi=70,
                                   base_misalign=(mis + 1) % 4 if esz == 4 else 0)
        ai = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
        af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
        ops = [(t, 1.0, 0.0)]
        want = T.port_run([Li], [Lf], [ai], [af], ops)[0]
        got = T.gpu_run([Li], [Lf], [ai], [af], ops)[0]
        T.assert_arenas_equal(got, want, Lf, what=f"misaligned dt{dt} {t}")


@pytest.mark.parametrize("dt", [capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64, capi.COMPLEX128])
@pytest.mark.parametrize("t", ["N", "T", "C"])
def test_scaled_match_port(dt, t):
    """final = beta*final + alpha*op(initial) on finite values: bit-exact."""
    rng = np.random.default_rng(55 + dt * 3 + "NTC".index(t))
    cplx = dt in (capi.COMPLEX64, capi.COMPLEX128)
    m, n = 257, 190
    Li = Ls.random_grid_layout(m if t == "N" else n, n if t == "N" else m, 6, dt, rng,
                               ext_hi=80)
    Lf = Ls.random_grid_layout(m, n, 6, dt, rng, ext_hi=80)
    comp = np.float32 if dt in (capi.FLOAT32, capi.COMPLEX64) else np.float64
    ai = np.frombuffer(rng.standard_normal(Li.arena_bytes // np.dtype(comp).itemsize)
                       .astype(comp).tobytes(), np.uint8).copy()
    af = np.frombuffer(rng.standard_normal(Lf.arena_bytes // np.dtype(comp).itemsize)
                       .astype(comp).tobytes(), np.uint8).copy()
    for alpha, beta in [((0.75 - 1.25j) if cplx else 0.75, (-0.5 + 0.375j) if cplx else -0.5),
                        (3.0, 0.0), (1.0, 1.0), (1.0, -0.0)]:
        ops = [(t, alpha, beta)]
        want = T.port_run([Li], [Lf], [ai], [af], ops)[0]
        got = T.gpu_run([Li], [Lf], [ai], [af], ops)[0]
        T.assert_arenas_equal(got, want, Lf, what=f"scaled dt{dt} {t} {alpha} {beta}")


def _normal_arena(rng, L, dt):
    comp = np.float32 if dt in (capi.FLOAT32, capi.COMPLEX64) else np.float64
    n = L.arena_bytes // np.dtype(comp).itemsize
    a = np.zeros(L.arena_bytes, np.uint8)
    a[:n * np.dtype(comp).itemsize] = np.frombuffer(
        rng.standard_normal(n).astype(comp).tobytes(), np.uint8)
    return a


@pytest.mark.parametrize("tuning", [
    None, dict(ring=-1), dict(stages=2), dict(threads=512, unroll=2),
    dict(tile_bytes=2048, unroll=1, l2_prefetch=1), dict(ring=1, tile_run=4)])
def test_scaled_tiles_mixed_with_copies_match_port(tuning):
    """Scaled pairs in one plan with plain and transposed ones. Non-transposed
    scaled tiles are warp-level work items (on the copy ring, the register
    path or beside the TMA-staged copies) when every destination element
    lies in one 16-byte chunk; complex<float> blocks at 4 mod 8 and
    complex<double> blocks at 8 mod 16 keep them CTA-level."""
    rng = np.random.default_rng(303)
    cases = [  # dtype, op, alpha, beta, destination byte misalignment
        (capi.FLOAT32, "N", 2.0, 0.5, 4), (capi.FLOAT64, "N", -1.5, 0.25, 8),
        (capi.COMPLEX64, "N", 0.5 + 1j, 0.25 - 0.5j, 0),
        (capi.COMPLEX64, "N", 0.5 + 1j, 1.0 - 0.5j, 4),
        (capi.COMPLEX128, "N", 2.0 - 1j, 0.5 + 0.5j, 0),
        (capi.COMPLEX128, "N", 2.0 - 1j, 0.5 + 0.5j, 8),
        (capi.FLOAT32, "T", 2.0, 0.5, 0), (capi.COMPLEX128, "C", 0.5, 2.0, 0),
        (capi.FLOAT32, "N", 1.0, 0.0, 0), (capi.FLOAT64, "T", 1.0, 0.0, 0)]
    inits, finals, ias, fas, ops = [], [], [], [], []
    for dt, t, alpha, beta, mis in cases:
        m, n = int(rng.integers(100, 400)), int(rng.integers(100, 400))
        Li = Ls.random_grid_layout(m if t == "N" else n, n if t == "N" else m, 5, dt, rng,
                                   ext_hi=150)
        Lf = Ls.random_grid_layout(m, n, 5, dt, rng, ext_hi=150, byte_misalign=mis)
        inits.append(Li); finals.append(Lf)
        ias.append(_normal_arena(rng, Li, dt)); fas.append(_normal_arena(rng, Lf, dt))
        ops.append((t, alpha, beta))
    want = T.port_run(inits, finals, ias, fas, ops)
    got = T.gpu_run(inits, finals, ias, fas, ops, how="plan", tuning=tuning)
    for k in range(len(inits)):
        T.assert_arenas_equal(got[k], want[k], finals[k], what=f"{tuning} case {cases[k]}")


def _special_arena(rng, L, dt):
    """Arena of special operands: signed zeros, infinities, NaNs, subnormals,
    ones, the largest finite values and normals, each part drawn
    independently."""
    comp = np.float32 if dt in (capi.FLOAT32, capi.COMPLEX64) else np.float64
    fi = np.finfo(comp)
    pool = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, -np.nan, fi.smallest_subnormal,
                     -fi.smallest_subnormal, 1.0, -1.0, fi.max, -fi.max, 0.5, -3.25],
                    dtype=comp)
    n = L.arena_bytes // np.dtype(comp).itemsize
    vals = pool[rng.integers(0, len(pool), size=n)]
    normal = rng.random(n) < 0.3
    vals[normal] = rng.standard_normal(int(normal.sum())).astype(comp)
    a = np.zeros(L.arena_bytes, np.uint8)
    a[:n * np.dtype(comp).itemsize] = np.frombuffer(vals.tobytes(), np.uint8)
    return a


@pytest.mark.parametrize("dt", [capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64, capi.COMPLEX128])
@pytest.mark.parametrize("t", ["N", "T"])
def test_real_and_zero_coefficients_on_special_operands(dt, t):
    """Real alpha / beta (imaginary parts +0 or -0) and zero betas, for which
    the complex<double> kernels form the products with a zero operand on the
    integer pipe: signed zeros, infinities, NaNs and subnormals in both
    operands, bit-exact against the port except NaN payloads."""
    rng = np.random.default_rng(1200 + 10 * dt + (t == "T"))
    m, n = 211, 157
    Li = Ls.random_grid_layout(m if t == "N" else n, n if t == "N" else m, 4, dt, rng,
                               ext_hi=70)
    Lf = Ls.random_grid_layout(m, n, 4, dt, rng, ext_hi=70)
    ai, af = _special_arena(rng, Li, dt), _special_arena(rng, Lf, dt)
    cplx = dt in (capi.COMPLEX64, capi.COMPLEX128)
    coefs = [(2.0, 0.5), (-3.0, 0.0), (0.5, -0.0), (1.0, 0.25), (-0.0, 2.0), (0.0, 0.0)]
    if cplx:
        coefs += [(complex(2.0, -0.0), complex(0.5, -0.0)),
                  (complex(-1.5, 0.0), complex(-0.0, -0.0)),
                  (complex(0.0, -0.0), complex(0.25, 0.0)), (complex(2.0, 1.0), 0.5),
                  (3.0, complex(0.5, -2.0))]
    for alpha, beta in coefs:
        ops = [(t, alpha, beta)]
        want = T.port_run([Li], [Lf], [ai], [af], ops)[0]
        got = T.gpu_run([Li], [Lf], [ai], [af], ops)[0]
        T.assert_arenas_equal(got, want, Lf, nan_equivalent=True,
                              what=f"dt{dt} {t} alpha={alpha} beta={beta}")


def test_scaled_special_values_nan_equivalent():
    """Inf/NaN through alpha/beta (Annex G complex products): equal up to NaN
    payloads, which IEEE leaves to the implementation."""
    for dt in (capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64, capi.COMPLEX128):
        rng = np.random.default_rng(99 + dt)
        Li, Lf, ai, af = _random_case(rng, dt, "N", 120, 90, 3, ext_hi=40)
        cplx = dt in (capi.COMPLEX64, capi.COMPLEX128)
        for alpha, beta in [(float("inf"), 0.5), (0.5, float("nan")),
                            ((complex(float("inf"), 1.0) if cplx else float("inf")), 0.0)]:
            ops = [("N", alpha, beta)]
            want = T.port_run([Li], [Lf], [ai], [af], ops)[0]
            got = T.gpu_run([Li], [Lf], [ai], [af], ops)[0]
            T.assert_arenas_equal(got, want, Lf, nan_equivalent=True,
                                  what=f"special dt{dt} {alpha} {beta}")


def test_mixed_dtype_batch_matches_port():
    rng = np.random.default_rng(31)
    inits, finals, ias, fas, ops = [], [], [], [], []
    for k in range(24):
        dt = int(rng.choice([0, 1, 2, 3]))
        t = "NTC"[k % 3]
        m, n = int(rng.integers(1, 400)), int(rng.integers(1, 400))
        Li, Lf, ai, af = _random_case(rng, dt, t, m, n, int(rng.integers(1, 40)),
                                      ext_hi=int(rng.integers(1, 200)))
        inits.append(Li); finals.append(Lf); ias.append(ai); fas.append(af)
        ops.append((t, 1.0, 0.0))
    want = T.port_run(inits, finals, ias, fas, ops)
    for how in ("batch", "plan", "graph"):
        got = T.gpu_run(inits, finals, ias, fas, ops, how=how)
        for k in range(len(inits)):
            T.assert_arenas_equal(got[k], want[k], finals[k], what=f"{how} pair {k}")


@pytest.mark.parametrize("tuning", [
    dict(threads=256, unroll=1, stages=-1), dict(threads=256, unroll=2, stages=2), dict(threads=512, unroll=4, stages=4),
    dict(threads=512, unroll=4, stages=-1), dict(tile_bytes=4096, tile_dim=16, stages=3),
    dict(tile_bytes=65536, tile_dim=32, ctas_per_sm=1, threads=512),
    dict(threads=256, unroll=1, ring=-1), dict(threads=512, unroll=4, ring=-1),
    dict(threads=256, unroll=2, ring=1), dict(threads=512, unroll=1, ring=1),
    dict(tile_bytes=512, unroll=4, ring=1, ctas_per_sm=1),
    dict(tile_bytes=2048, ring=1, tile_run=8), dict(threads=256, ring=1, tile_run=64),
    dict(tile_bytes=4096, ring=1, l2_prefetch=1), dict(threads=256, unroll=1, ring=1, l2_prefetch=1)])
def test_tunings_give_identical_results(tuning):
    rng = np.random.default_rng(77)
    inits, finals, ias, fas, ops = [], [], [], [], []
    for k, (dt, t) in enumerate([(0, "N"), (1, "T"), (2, "C"), (3, "N"), (3, "C")]):
        Li, Lf, ai, af = _random_case(rng, dt, t, 333, 277, 7, ext_hi=150)
        inits.append(Li); finals.append(Lf); ias.append(ai); fas.append(af)
        ops.append((t, 1.0, 0.0))
    want = T.port_run(inits, finals, ias, fas, ops)
    got = T.gpu_run(inits, finals, ias, fas, ops, how="plan", tuning=tuning, executes=2)
    for k in range(len(inits)):
        T.assert_arenas_equal(got[k], want[k], finals[k], what=f"{tuning} pair {k}")


def test_repeated_execution_is_idempotent():
    rng = np.random.default_rng(5)
    Li, Lf, ai, af = _random_case(rng, capi.COMPLEX64, "C", 500, 300, 9, ext_hi=120)
    ops = [("C", 1.0, 0.0)]
    want = T.port_run([Li], [Lf], [ai], [af], ops)[0]
    got = T.gpu_run([Li], [Lf], [ai], [af], ops, how="graph", executes=3)[0]
    T.assert_arenas_equal(got, want, Lf, what="graph x3")


def test_reordered_and_idle_ranks():
    rng = np.random.default_rng(8)
    Li = Ls.scalapack_layout(301, 257, 17, 9, 3, 4, capi.FLOAT64)
    Lf = Ls.scalapack_layout(301, 257, 23, 31, 4, 3, capi.FLOAT64, row_major=True)
    perm = list(rng.permutation(12))
    Lf.reorder_ranks(perm)
    Lf.blocks["rank"] = [perm[r] for r in Lf.blocks["rank"]]
    Li.n_ranks = 20  # ranks 12..19 hold nothing
    ai = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
    af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    want = T.port_run([Li], [Lf], [ai], [af])[0]
    got = T.gpu_run([Li], [Lf], [ai], [af])[0]
    T.assert_arenas_equal(got, want, Lf, what="reordered")


def test_submatrix_layouts():
    """ScaLAPACK submatrix layouts (ij offset, source process) both sides."""
    rng = np.random.default_rng(12)
    Li = Ls.scalapack_layout(300, 280, 27, 13, 2, 3, capi.COMPLEX128, row_major=True,
                             lld=310, ij=(21, 8), sub=(176, 137), src=(1, 2))
    Lf = Ls.scalapack_layout(200, 200, 32, 32, 3, 2, capi.COMPLEX128, lld=205,
                             ij=(5, 40), sub=(176, 137), src=(2, 0))
    ai = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
    af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    want = T.port_run([Li], [Lf], [ai], [af])[0]
    got = T.gpu_run([Li], [Lf], [ai], [af])[0]
    T.assert_arenas_equal(got, want, Lf, what="submatrix")


def test_plan_info_counts():
    lib = capi.load()
    w = W.block_cyclic_f64_4096(512)
    import torch
    di = torch.zeros(w.inits[0].arena_bytes, dtype=torch.uint8, device="cuda")
    df = torch.zeros(w.finals[0].arena_bytes, dtype=torch.uint8, device="cuda")
    dI, k1 = T.descs(w.inits, [di.data_ptr()])
    dF, k2 = T.descs(w.finals, [df.data_ptr()])
    plan = C.c_void_p()
    capi.check(lib.g2g_plan_create(dI, dF, capi.FLOAT64, None, None, C.byref(plan)))
    info = capi.PlanInfo()
    capi.check(lib.g2g_plan_get_info(plan, C.byref(info)))
    assert info.n_pieces == (512 // 32) * (512 // 32)  # every 32x32 block is one piece
    assert info.bytes_moved == 512 * 512 * 8
    assert info.bytes_min_traffic == 2 * info.bytes_moved
    assert info.n_tiles >= info.n_pieces
    capi.check(lib.g2g_plan_destroy(plan))


# ------------------------------------------------------------ full sizes
def _device_random(nbytes, seed):
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    return torch.randint(0, 256, (nbytes,), dtype=torch.uint8, device="cuda", generator=g)


def _run_device(w, dev_i, dev_f):
    lib = capi.load()
    dI, k1 = T.descs(w.inits, [t.data_ptr() for t in dev_i])
    dF, k2 = T.descs(w.finals, [t.data_ptr() for t in dev_f])
    n = len(w.inits)
    dts = (C.c_int * n)(*w.dtypes())
    opa = T.make_ops(w.ops, n)
    import torch
    capi.check(lib.g2g_transform_batch(n, dI, dF, dts, opa,
                                       C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()


def test_full_block_cyclic_f64_4096_known_answer():
    """entry(i, j) = i + j*4096 must arrive at (i, j) of the 128x64 layout."""
    import torch
    w = W.block_cyclic_f64_4096()
    ia, fa = W.fill_arenas(w)
    dev_i = [torch.from_numpy(ia[0]).cuda()]
    dev_f = [torch.from_numpy(fa[0]).cuda()]
    _run_device(w, dev_i, dev_f)
    out = dev_f[0].cpu().numpy()
    got = w.finals[0].gather(out).view(np.float64)
    m = 4096
    want = (np.arange(m, dtype=np.float64)[:, None] + np.arange(m, dtype=np.float64)[None, :] * m)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("name", ["random_grid_f32_16384", "transposed_c128_8192"])
def test_full_size_matches_port(name):
    import torch
    w = W.BY_NAME[name]()
    dev_i = [_device_random(L.arena_bytes, 1 + k) for k, L in enumerate(w.inits)]
    dev_f = [_device_random(L.arena_bytes, 100 + k) for k, L in enumerate(w.finals)]
    ia = [t.cpu().numpy() for t in dev_i]
    fa = [t.cpu().numpy() for t in dev_f]
    _run_device(w, dev_i, dev_f)
    want = T.port_run(w.inits, w.finals, ia, fa, w.ops, threads=16)
    for k in range(len(w.finals)):
        got = dev_f[k].cpu().numpy()
        T.assert_arenas_equal(got, want[k], w.finals[k], what=name)


def test_full_size_round_trip_and_conservation():
    """random_grid_f32_16384 forward then backward restores every element of
    the initial layout; the multiset of elements is conserved."""
    import torch
    w = W.random_grid_f32_16384()
    Li, Lf = w.inits[0], w.finals[0]
    dev_i = _device_random(Li.arena_bytes, 11)
    dev_f = _device_random(Lf.arena_bytes, 12)
    dev_back = _device_random(Li.arena_bytes, 13)
    back = W.Workload("back", [Lf], [Li], None)
    _run_device(w, [dev_i], [dev_f])
    _run_device(back, [dev_f], [dev_back])
    a = Li.gather(dev_i.cpu().numpy())
    b = Li.gather(dev_back.cpu().numpy())
    assert np.array_equal(a, b)
    f = Lf.gather(dev_f.cpu().numpy())
    assert int(a.astype(np.uint64).sum()) == int(f.astype(np.uint64).sum())
    assert np.array_equal(np.sort(a, axis=None), np.sort(f, axis=None))


def test_one_shot_plan_cache_reuse():
    """Repeated one-shot transforms between the same buffers reuse the cached
    plan; new source data must still come through, bit-exact."""
    import torch
    lib = capi.load()
    rng = np.random.default_rng(321)
    Li, Lf, ai, af = _random_case(rng, capi.COMPLEX64, "T", 333, 222, 5, ext_hi=100)
    di = torch.from_numpy(ai).cuda()
    df = torch.from_numpy(af).cuda()
    dI, k1 = Li.desc(di.data_ptr())
    dF, k2 = Lf.desc(df.data_ptr())
    op = capi.make_op("T", 1.0, 0.0)
    for trial in range(3):
        src = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
        di.copy_(torch.from_numpy(src))
        df.copy_(torch.from_numpy(af))
        capi.check(lib.g2g_transform(C.byref(dI), C.byref(dF), capi.COMPLEX64, C.byref(op),
                                     None))
        want = T.port_run([Li], [Lf], [src], [af], [("T", 1.0, 0.0)])[0]
        T.assert_arenas_equal(df.cpu().numpy(), want, Lf, what=f"cached one-shot {trial}")
    capi.check(lib.g2g_plan_cache_clear())


@pytest.mark.parametrize("tuning", [
    dict(threads=512, unroll=4, ring=1), dict(threads=256, unroll=1, ring=1),
    dict(threads=512, unroll=2, ring=1, tile_bytes=512), dict(threads=256, unroll=4, ring=-1)])
def test_tiny_pieces_and_short_tiles(tuning):
    """Grids with extents of 1-3 elements: hundreds of thousands of pieces a
    few chunks long, so a warp's stages cross many tile boundaries and its
    descriptor queue turns over constantly; mixed element sizes in one batch;
    a tiny pair whose tiles are fewer than the warps of the grid."""
    rng = np.random.default_rng(4242)
    inits, finals, ias, fas = [], [], [], []
    for dt, m, n, hi in [(capi.FLOAT32, 300, 260, 3), (capi.COMPLEX128, 97, 120, 2),
                         (capi.FLOAT64, 200, 333, 5), (capi.COMPLEX64, 3, 2, 1)]:
        Li, Lf, ai, af = _random_case(rng, dt, "N", m, n, 7, ext_lo=1, ext_hi=hi)
        inits.append(Li); finals.append(Lf); ias.append(ai); fas.append(af)
    want = T.port_run(inits, finals, ias, fas)
    got = T.gpu_run(inits, finals, ias, fas, how="plan", tuning=tuning, executes=2)
    for k in range(len(inits)):
        T.assert_arenas_equal(got[k], want[k], finals[k], what=f"{tuning} pair {k}")


@pytest.mark.gpu
@pytest.mark.parametrize("dt", [capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64, capi.COMPLEX128])
@pytest.mark.parametrize("t", ["T", "C"])
@pytest.mark.parametrize("tile_dim,threads", [(16, 256), (32, 256), (32, 512)])
def test_transposed_tile_shapes_match_port(dt, t, tile_dim, threads):
    """Plain transposes on every tile shape: 4-byte elements on tiles of twice
    the edge, 8-byte ones on tiles of twice the rows (8-byte aligned and
    4-byte aligned complex<float>), 16-byte ones on td x td tiles; blocks at
    4 / 8 bytes past a 16-byte boundary, pieces of every size up to 300."""
    rng = np.random.default_rng(500 + 10 * dt + tile_dim + threads + (t == "C"))
    comp = 8 if dt in (capi.FLOAT64, capi.COMPLEX128) else 4
    inits, finals, ias, fas = [], [], [], []
    for mis in (0, 4, 8, 12):
        m, n = int(rng.integers(50, 420)), int(rng.integers(50, 420))
        mi = (mis - mis % comp)
        Li = Ls.random_grid_layout(n, m, 5, dt, rng, ext_hi=300, byte_misalign=mi)
        Lf = Ls.random_grid_layout(m, n, 5, dt, rng, ext_hi=300,
                                   byte_misalign=(mi + comp) % 16 - ((mi + comp) % 16) % comp)
        inits.append(Li); finals.append(Lf)
        ias.append(Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng))
        fas.append(Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng))
    ops = [(t, 1.0, 0.0)] * len(inits)
    want = T.port_run(inits, finals, ias, fas, ops)
    got = T.gpu_run(inits, finals, ias, fas, ops, how="plan",
                    tuning=dict(tile_dim=tile_dim, threads=threads))
    for k in range(len(inits)):
        T.assert_arenas_equal(got[k], want[k], finals[k], what=f"dt{dt} {t} td{tile_dim} pair {k}")
