"""The C-ABI library on the CPU: it loads, exports every function the public
header declares, and rejects invalid descriptors on the host with
G2G_ERROR_INVALID_ARGUMENT before any CUDA call (no GPU needed). These are the
conditions under which the reference throws std::runtime_error, asserts, or
hangs in MPI."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

import g2g_testlib as T
from grid2grid_gb300 import capi
from grid2grid_gb300 import layouts as Ls

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from grid2grid_gb300 import build
    build.build()
    return capi.load()


def test_exports_every_header_symbol(lib):
    raw = C.CDLL(capi.LIB_PATH)
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        names += capi.header_symbols(h)
    assert len(names) >= 13
    missing = [n for n in names if not hasattr(raw, n)]
    assert not missing, missing
    # the ctypes binding declares exactly what the headers declare
    bound = {s[0] for s in capi.SIGNATURES}
    assert set(names) == bound, set(names) ^ bound


@pytest.mark.parametrize("lang,std", [("c", "c99"), ("c", "c11"), ("c++", "c++11")])
def test_header_is_plain_c(tmp_path, lang, std):
    """The boundary header compiles on its own as strict C and as C++: plain
    structs, pointers and sizes, no CUDA or C++ types in the signatures."""
    import shutil
    import subprocess
    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    src = tmp_path / ("h.c" if lang == "c" else "h.cpp")
    src.write_text('#include "grid2grid_gb300.h"\nint main(void) { return 0; }\n')
    r = subprocess.run([cc, f"-std={std}", "-pedantic", "-Wall", "-Werror", "-fsyntax-only",
                        "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_version_and_error_string(lib):
    assert b"sm_103a" in lib.g2g_version_string()
    assert isinstance(lib.g2g_last_error_string(), bytes)


def _pair(m=20, n=16, P=3, dt=capi.FLOAT64, seed=0):
    rng = np.random.default_rng(seed)
    Li = Ls.random_grid_layout(m, n, P, dt, rng, ext_hi=7)
    Lf = Ls.random_grid_layout(m, n, P, dt, rng, ext_hi=7)
    return Li, Lf


def _create(lib, Li, Lf, op=None, dt=None):
    dI, k1 = T.descs([Li], [0x10000])
    dF, k2 = T.descs([Lf], [0x20000000])
    plan = C.c_void_p()
    opp = None if op is None else C.byref(capi.make_op(*op))
    st = lib.g2g_plan_create(dI, dF, Li.dtype if dt is None else dt, opp, None,
                             C.byref(plan))
    msg = lib.g2g_last_error_string().decode()
    return st, msg


def _expect_invalid(lib, Li, Lf, needle, **kw):
    st, msg = _create(lib, Li, Lf, **kw)
    assert st == capi.ERROR_INVALID_ARGUMENT, (st, msg)
    assert needle in msg, msg


def test_rejects_different_matrices(lib):
    Li, _ = _pair(20, 16)
    _, Lf = _pair(21, 16)
    _expect_invalid(lib, Li, Lf, "different matrices")


def test_rejects_transposed_shape_mismatch(lib):
    Li, Lf = _pair(20, 16)
    _expect_invalid(lib, Li, Lf, "different matrices", op=("T", 1.0, 0.0))


def test_rejects_decreasing_split(lib):
    Li, Lf = _pair()
    Li.rows_split = Li.rows_split.copy()
    if len(Li.rows_split) > 2:
        Li.rows_split[1], Li.rows_split[2] = Li.rows_split[2], Li.rows_split[1]
        _expect_invalid(lib, Li, Lf, "decreasing")


def test_rejects_negative_split(lib):
    Li, Lf = _pair()
    Li.rows_split = Li.rows_split.copy()
    Li.rows_split[0] = -1
    _expect_invalid(lib, Li, Lf, "negative")


def test_rejects_block_not_held_by_owner(lib):
    Li, Lf = _pair(P=3)
    Li.blocks["rank"][0] = (Li.blocks["rank"][0] + 1) % 3
    _expect_invalid(lib, Li, Lf, "owned by rank")


def test_rejects_missing_block(lib):
    Li, Lf = _pair()
    Lf.blocks = Lf.blocks[1:]
    Lf.offsets = Lf.offsets[1:]
    _expect_invalid(lib, Li, Lf, "missing")


def test_rejects_duplicate_block(lib):
    Li, Lf = _pair()
    Li.blocks = np.concatenate([Li.blocks, Li.blocks[:1]])
    Li.offsets = np.concatenate([Li.offsets, Li.offsets[:1]])
    _expect_invalid(lib, Li, Lf, "more than once")


def test_rejects_short_stride(lib):
    Li, Lf = _pair()
    k = int(np.argmax([Li.storage_shape(b)[0] * (Li.storage_shape(b)[1] > 1)
                       for b in range(Li.n_blocks)]))
    Li.blocks["stride"][k] = Li.storage_shape(k)[0] - 1
    _expect_invalid(lib, Li, Lf, "stride")


def test_rejects_owner_outside_ranks(lib):
    Li, Lf = _pair(P=2)
    Li.owners = Li.owners.copy()
    Li.owners[0, 0] = 7
    _expect_invalid(lib, Li, Lf, "owner")


def test_rejects_transposed_destination(lib):
    Li, Lf = _pair()
    Lf.blocks["trans"][0] = 1
    _expect_invalid(lib, Li, Lf, "transpose_on_copy")


def test_rejects_bad_trans_and_dtype_and_imaginary_scalars(lib):
    Li, Lf = _pair()
    _expect_invalid(lib, Li, Lf, "trans", op=("X", 1.0, 0.0))
    _expect_invalid(lib, Li, Lf, "imaginary", op=("N", 1j, 0.0))
    st, msg = _create(lib, Li, Lf, dt=9)
    assert st == capi.ERROR_INVALID_ARGUMENT and "dtype" in msg


def test_rejects_null_pointer_block(lib):
    Li, Lf = _pair()
    dI, k1 = T.descs([Li], [0])
    # block at offset 0 of a NULL base -> NULL data pointer
    k = int(np.argmin(Li.offsets))
    if Li.offsets[k] == 0:
        dF, k2 = T.descs([Lf], [0x20000000])
        plan = C.c_void_p()
        st = lib.g2g_plan_create(dI, dF, Li.dtype, None, None, C.byref(plan))
        assert st == capi.ERROR_INVALID_ARGUMENT
        assert b"NULL" in lib.g2g_last_error_string()


def test_batch_reports_failing_pair(lib):
    Li, Lf = _pair()
    Lj, Lg = _pair(seed=3)
    Lg.blocks = Lg.blocks[1:]
    Lg.offsets = Lg.offsets[1:]
    dI, k1 = T.descs([Li, Lj], [0x10000, 0x30000])
    dF, k2 = T.descs([Lf, Lg], [0x50000, 0x70000])
    dts = (C.c_int * 2)(Li.dtype, Lj.dtype)
    plan = C.c_void_p()
    st = lib.g2g_plan_create_batch(2, dI, dF, dts, None, None, C.byref(plan))
    assert st == capi.ERROR_INVALID_ARGUMENT
    assert lib.g2g_last_error_string().startswith(b"pair 1:")


def test_null_arguments(lib):
    plan = C.c_void_p()
    assert lib.g2g_plan_create(None, None, 0, None, None, C.byref(plan)) == \
        capi.ERROR_INVALID_ARGUMENT
    assert lib.g2g_plan_execute(None, None) == capi.ERROR_INVALID_ARGUMENT
    assert lib.g2g_plan_destroy(None) == capi.SUCCESS
    info = capi.PlanInfo()
    assert lib.g2g_plan_get_info(None, C.byref(info)) == capi.ERROR_INVALID_ARGUMENT
    a = (C.c_int32 * 3)(0, 5, 10)
    b = (C.c_int32 * 2)(0, 11)
    s = (C.c_int32 * 2)()
    e = (C.c_int32 * 2)()
    assert lib.g2g_grid_cover(a, 3, b, 2, s, e, None) == capi.ERROR_INVALID_ARGUMENT
