"""Fused dtype cast (g2g_transform_cast): final = convert(op(initial)) on
the GPU against numpy's conversions of the same matrices (the reference has
no such operation). Bit-exact except NaN payloads, which IEEE leaves to the
implementation (compared as NaN)."""
import ctypes as C

import numpy as np
import pytest

from grid2grid_gb300 import capi
from grid2grid_gb300 import layouts as Ls

import g2g_testlib as T

NP = {capi.FLOAT32: np.float32, capi.FLOAT64: np.float64,
      capi.COMPLEX64: np.complex64, capi.COMPLEX128: np.complex128}
CASTS = [(capi.FLOAT64, capi.FLOAT32), (capi.FLOAT32, capi.FLOAT64),
         (capi.COMPLEX128, capi.COMPLEX64), (capi.COMPLEX64, capi.COMPLEX128),
         (capi.FLOAT32, capi.COMPLEX64), (capi.FLOAT64, capi.COMPLEX128),
         (capi.FLOAT64, capi.COMPLEX64), (capi.FLOAT32, capi.COMPLEX128)]


def _values(rng, L, dt):
    """A source arena of finite values spanning many exponents plus special
    values (inf, nan, subnormals, values that overflow or underflow a float)."""
    a = np.zeros(L.arena_bytes, np.uint8)
    base = np.float64 if dt in (capi.FLOAT64, capi.COMPLEX128) else np.float32
    for b in range(L.n_blocks):
        v = L.block_view(a, b)
        n = v.size * (2 if dt in (capi.COMPLEX64, capi.COMPLEX128) else 1)
        x = rng.standard_normal(n) * np.exp2(rng.integers(-140, 140, size=n))
        special = np.array([np.inf, -np.inf, np.nan, 0.0, -0.0, 1e-45, 3.5e38, 1e300, -1e-310])
        k = rng.integers(0, n, size=max(1, n // 50))
        x[k] = rng.choice(special, size=len(k))
        with np.errstate(over="ignore"):
            xs = x.astype(base)
        v[...] = xs.view(v.dtype).reshape(v.shape) if v.size else v
    return a


def _expected(Li, Lf, ai, af, src, dst, trans):
    g = Li.gather(ai).view(NP[src])          # op(initial) in the final coordinates
    with np.errstate(over="ignore", invalid="ignore"):
        x = g.astype(NP[dst])
    if trans == "C" and np.iscomplexobj(x):
        x = np.conj(x)
    out = af.copy()
    for b in range(Lf.n_blocks):
        i, j = int(Lf.blocks["row"][b]), int(Lf.blocks["col"][b])
        blk = x[Lf.rows_split[i]:Lf.rows_split[i + 1], Lf.cols_split[j]:Lf.cols_split[j + 1]]
        v = Lf.block_view(out, b)
        v[...] = np.ascontiguousarray(blk).view(v.dtype).reshape(v.shape) if v.size else v
    return out


def _comp(dt):
    """Bytes of the real component: the alignment an element address needs."""
    return 8 if dt in (capi.FLOAT64, capi.COMPLEX128) else 4


def _layouts(rng, src, dst, trans, m=257, n=190, P=5, ext_hi=70, mis=(0, 0)):
    """mis: byte offsets of every initial / final block past an aligned
    address (rounded down to the component alignment of each side)."""
    Li = Ls.random_grid_layout(m if trans == "N" else n, n if trans == "N" else m, P, src, rng,
                               ext_hi=ext_hi, byte_misalign=mis[0] - mis[0] % _comp(src))
    Lf = Ls.random_grid_layout(m, n, P, dst, rng, ext_hi=ext_hi,
                               byte_misalign=mis[1] - mis[1] % _comp(dst))
    return Li, Lf


def _check_cast(rng, Li, Lf, src, dst, trans, where=("device", "device"), ai=None):
    import torch
    if ai is None:
        ai = _values(rng, Li, src)
    af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    Lt = Li.copy().transpose_or_conjugate(trans) if trans != "N" else Li
    want = _expected(Lt, Lf, ai, af, src, dst, trans)
    lib = capi.load()

    def place(a, w):
        if w == "device":
            return T.to_device([a])[0]
        t = torch.empty(len(a), dtype=torch.uint8, pin_memory=True)
        t.numpy()[:] = a
        return t
    di, df = place(ai, where[0]), place(af, where[1])
    dI, k1 = Li.desc(di.data_ptr())
    dF, k2 = Lf.desc(df.data_ptr())
    op = capi.make_op(trans, 1.0, 0.0)
    capi.check(lib.g2g_transform_cast(C.byref(dI), src, C.byref(dF), dst, C.byref(op), None))
    torch.cuda.synchronize()
    got = df.cpu().numpy().copy()
    Lcmp = Ls.Layout(Lf.rows_split, Lf.cols_split, Lf.owners, Lf.n_ranks,
                     capi.FLOAT64 if _comp(dst) == 8 else capi.FLOAT32, [], [], [], [], [], 0)
    T.assert_arenas_equal(got, want, Lcmp, nan_equivalent=True,
                          what=f"cast {src}->{dst} op {trans} {where}")


@pytest.mark.gpu
@pytest.mark.parametrize("src,dst", CASTS)
@pytest.mark.parametrize("trans", ["N", "T", "C"])
def test_cast_matches_numpy(src, dst, trans):
    rng = np.random.default_rng(100 * src + 10 * dst + "NTC".index(trans))
    Li, Lf = _layouts(rng, src, dst, trans)
    _check_cast(rng, Li, Lf, src, dst, trans)


@pytest.mark.gpu
@pytest.mark.parametrize("src,dst", CASTS)
@pytest.mark.parametrize("mis", [(0, 4), (4, 8), (8, 12)])
def test_cast_long_columns_and_misaligned_blocks(src, dst, mis):
    """Columns of up to 700 rows (tiles of several 16-byte chunks per column,
    staged through shared memory), pieces of many short columns (tiles too
    wide to stage), blocks at 4, 8 or 12 bytes past a 16-byte boundary
    (destination elements that straddle 16-byte chunks)."""
    rng = np.random.default_rng(1000 * src + 100 * dst + mis[0] + mis[1])
    Li, Lf = _layouts(rng, src, dst, "N", m=1500, n=1200, P=7, ext_hi=700, mis=mis)
    _check_cast(rng, Li, Lf, src, dst, "N")
    Li, Lf = _layouts(rng, src, dst, "N", m=40, n=2600, P=3, ext_hi=2000, mis=mis)
    _check_cast(rng, Li, Lf, src, dst, "N")


@pytest.mark.gpu
@pytest.mark.parametrize("where", [("host", "device"), ("device", "host")])
def test_cast_host_memory(where):
    """Layouts in pinned host memory: the cast reads / writes them in place."""
    rng = np.random.default_rng(41)
    for src, dst in [(capi.FLOAT32, capi.FLOAT64), (capi.COMPLEX128, capi.COMPLEX64)]:
        Li, Lf = _layouts(rng, src, dst, "N", m=600, n=300, ext_hi=400)
        _check_cast(rng, Li, Lf, src, dst, "N", where)


def test_cast_argument_checks():
    """Complex -> real and scaled casts are refused on the host."""
    lib = capi.load()
    rng = np.random.default_rng(1)
    Li, Lf = _layouts(rng, capi.COMPLEX64, capi.FLOAT32, "N", m=20, n=20)
    dI, k1 = Li.desc(1 << 20)
    dF, k2 = Lf.desc(1 << 30)
    plan = C.c_void_p()
    st = lib.g2g_plan_create_cast(C.byref(dI), capi.COMPLEX64, C.byref(dF), capi.FLOAT32,
                                  None, None, C.byref(plan))
    assert st == capi.ERROR_UNSUPPORTED
    Li, Lf = _layouts(rng, capi.FLOAT64, capi.FLOAT32, "N", m=20, n=20)
    dI, k1 = Li.desc(1 << 20)
    dF, k2 = Lf.desc(1 << 30)
    op = capi.make_op("N", 2.0, 0.0)
    st = lib.g2g_plan_create_cast(C.byref(dI), capi.FLOAT64, C.byref(dF), capi.FLOAT32,
                                  C.byref(op), None, C.byref(plan))
    assert st == capi.ERROR_UNSUPPORTED


def _f64_boundaries(rng, n):
    """Bit patterns of binary64 values at the binary32 rounding boundaries:
    exponents around the subnormal, normal and overflow limits, dropped bits
    at, just below and just above one half ulp (ties to even and odd)."""
    sign = rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63)
    E = rng.choice(np.r_[0, 1, np.arange(860, 905), np.arange(1140, 1155), 2046, 2047],
                   n).astype(np.uint64)
    frac = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    # the bits a binary32 result drops: 29 in the normal range, 926 - E below it
    sh = np.where((E >= 897) & (E <= 1150), 29, np.clip(926 - E.astype(np.int64), 1, 52))
    sh = sh.astype(np.uint64)
    half = np.uint64(1) << (sh - np.uint64(1))
    low = np.stack([np.zeros(n, np.uint64), half, half - np.uint64(1), half + np.uint64(1),
                    (np.uint64(1) << sh) - np.uint64(1), frac & ((np.uint64(1) << sh) - np.uint64(1))])
    pick = low[rng.integers(0, low.shape[0], n), np.arange(n)]
    frac = (frac & ~((np.uint64(1) << sh) - np.uint64(1))) | pick
    frac = np.where(rng.random(n) < 0.5, frac ^ (np.uint64(1) << sh), frac)  # odd and even
    frac &= np.uint64((1 << 52) - 1)
    return sign | (E << np.uint64(52)) | frac


@pytest.mark.gpu
@pytest.mark.parametrize("src,dst", [(capi.FLOAT64, capi.FLOAT32), (capi.COMPLEX128, capi.COMPLEX64),
                                     (capi.FLOAT64, capi.COMPLEX64)])
def test_cast_rounding_boundaries(src, dst):
    """Narrowing at every rounding boundary (ties to even, subnormal results,
    overflow to infinity) against numpy's IEEE conversion, bit for bit."""
    rng = np.random.default_rng(7 + src + dst)
    Li, Lf = _layouts(rng, src, dst, "N", m=600, n=300, ext_hi=400)
    ai = _f64_boundaries(rng, Li.arena_bytes // 8).view(np.uint8).copy()
    _check_cast(rng, Li, Lf, src, dst, "N", ai=ai)


@pytest.mark.gpu
@pytest.mark.parametrize("src,dst", [(capi.FLOAT32, capi.FLOAT64), (capi.COMPLEX64, capi.COMPLEX128),
                                     (capi.FLOAT32, capi.COMPLEX128)])
def test_cast_widening_every_class(src, dst):
    """Widening of random binary32 bit patterns of every class (zeros,
    subnormals, normals of every exponent, infinities, NaNs)."""
    rng = np.random.default_rng(17 + src + dst)
    Li, Lf = _layouts(rng, src, dst, "N", m=600, n=300, ext_hi=400)
    u = rng.integers(0, 1 << 32, Li.arena_bytes // 4, dtype=np.uint64).astype(np.uint32)
    sub = rng.random(len(u)) < 0.2  # a fifth subnormal or zero
    u[sub] &= np.uint32(0x807FFFFF)
    _check_cast(rng, Li, Lf, src, dst, "N", ai=u.view(np.uint8).copy())


@pytest.mark.gpu
def test_cast_scaled_and_plain_plans_in_one_multi_plan_launch():
    """g2g_plans_execute over a cast plan, a scaled plan and a plain plan:
    the cast plan launches apart (no kernel instance carries both kinds of
    element arithmetic); every result as when run alone."""
    import torch
    rng = np.random.default_rng(77)
    lib = capi.load()
    # cast float64 -> float32
    Lci, Lcf = _layouts(rng, capi.FLOAT64, capi.FLOAT32, "N", m=300, n=200)
    aci = _values(rng, Lci, capi.FLOAT64)
    acf = Ls.fill_random(np.zeros(Lcf.arena_bytes, np.uint8), rng)
    want_c = _expected(Lci, Lcf, aci, acf, capi.FLOAT64, capi.FLOAT32, "N")
    # scaled float32 and plain complex<double> pairs, checked against the oracle
    pairs = []
    for dt, op in [(capi.FLOAT32, ("N", 2.0, 0.5)), (capi.COMPLEX128, ("T", 1.0, 0.0))]:
        m, n = 250, 180
        Li = Ls.random_grid_layout(m if op[0] == "N" else n, n if op[0] == "N" else m, 4, dt,
                                   rng, ext_hi=90)
        Lf = Ls.random_grid_layout(m, n, 4, dt, rng, ext_hi=90)
        comp = np.float32 if dt == capi.FLOAT32 else np.float64
        ai = np.frombuffer(rng.standard_normal(Li.arena_bytes // np.dtype(comp).itemsize)
                           .astype(comp).tobytes(), np.uint8).copy()
        af = np.frombuffer(rng.standard_normal(Lf.arena_bytes // np.dtype(comp).itemsize)
                           .astype(comp).tobytes(), np.uint8).copy()
        want = T.port_run([Li], [Lf], [ai], [af], [op])[0]
        pairs.append((Li, Lf, ai, af, op, want))
    keep, plans, outs = [], [], []
    dci, dcf = T.to_device([aci, acf])
    dI, k1 = Lci.desc(dci.data_ptr())
    dF, k2 = Lcf.desc(dcf.data_ptr())
    keep += [k1, k2, dI, dF]
    p = C.c_void_p()
    capi.check(lib.g2g_plan_create_cast(C.byref(dI), capi.FLOAT64, C.byref(dF), capi.FLOAT32,
                                        None, None, C.byref(p)))
    plans.append(p.value)
    outs.append(dcf)
    for Li, Lf, ai, af, op, _ in pairs:
        di, df = T.to_device([ai, af])
        dI, k1 = Li.desc(di.data_ptr())
        dF, k2 = Lf.desc(df.data_ptr())
        o = capi.make_op(*op)
        keep += [k1, k2, dI, dF, o, di]
        p = C.c_void_p()
        capi.check(lib.g2g_plan_create(C.byref(dI), C.byref(dF), Li.dtype, C.byref(o), None,
                                       C.byref(p)))
        plans.append(p.value)
        outs.append(df)
    s = torch.cuda.Stream()
    arr = (C.c_void_p * len(plans))(*plans)
    capi.check(lib.g2g_plans_execute(len(plans), arr, C.c_void_p(s.cuda_stream)))
    s.synchronize()
    Lcmp = Ls.Layout(Lcf.rows_split, Lcf.cols_split, Lcf.owners, Lcf.n_ranks, capi.FLOAT32,
                     [], [], [], [], [], 0)
    T.assert_arenas_equal(outs[0].cpu().numpy(), want_c, Lcmp, nan_equivalent=True,
                          what="cast plan in a multi-plan launch")
    for (Li, Lf, ai, af, op, want), out in zip(pairs, outs[1:]):
        T.assert_arenas_equal(out.cpu().numpy(), want, Lf, what=f"{op} plan in a multi-plan launch")
    for p in plans:
        capi.check(lib.g2g_plan_destroy(C.c_void_p(p)))


@pytest.mark.gpu
@pytest.mark.parametrize("tuning", [dict(unroll=1), dict(unroll=2), dict(ring=-1),
                                    dict(stages=2, threads=256), dict(threads=512, unroll=2),
                                    dict(tile_bytes=2048, l2_prefetch=1)])
def test_cast_tunings_give_identical_results(tuning):
    """The cast on every kernel form a tuning selects: the copy ring at each
    unroll, the register path, the TMA-staged kernel (cast tiles beside it on
    the register path)."""
    import torch
    rng = np.random.default_rng(808)
    lib = capi.load()
    for src, dst in [(capi.FLOAT32, capi.FLOAT64), (capi.COMPLEX128, capi.COMPLEX64),
                     (capi.FLOAT64, capi.COMPLEX128)]:
        Li, Lf = _layouts(rng, src, dst, "N", m=700, n=400, ext_hi=500, mis=(4, 8))
        ai = _values(rng, Li, src)
        af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
        want = _expected(Li, Lf, ai, af, src, dst, "N")
        di, df = T.to_device([ai, af])
        dI, k1 = Li.desc(di.data_ptr())
        dF, k2 = Lf.desc(df.data_ptr())
        plan = C.c_void_p()
        capi.check(lib.g2g_plan_create_cast(C.byref(dI), src, C.byref(dF), dst, None, None,
                                            C.byref(plan)))
        t = capi.Tuning()
        for k, v in tuning.items():
            setattr(t, k, v)
        capi.check(lib.g2g_plan_set_tuning(plan, C.byref(t)))
        capi.check(lib.g2g_plan_execute(plan, None))
        torch.cuda.synchronize()
        capi.check(lib.g2g_plan_destroy(plan))
        Lcmp = Ls.Layout(Lf.rows_split, Lf.cols_split, Lf.owners, Lf.n_ranks,
                         capi.FLOAT64 if _comp(dst) == 8 else capi.FLOAT32, [], [], [], [], [], 0)
        T.assert_arenas_equal(df.cpu().numpy(), want, Lcmp, nan_equivalent=True,
                              what=f"cast {src}->{dst} {tuning}")
