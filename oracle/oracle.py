"""Oracle loaders -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, as the checker. Two CPU implementations of the transform path:

  * the PORT   (_build/libg2g_oracle.so, from port/g2g_oracle.cpp): this
    project's restatement of the reference algorithm; builds anywhere g++ is.
  * the REFERENCE (_ref/libg2g_ref.so): kabicm/grid2grid's own sources,
    unmodified, over the thread-MPI shim; builds only where the reference
    checkout is present (see Makefile).

Both take the product's layout descriptors with HOST block pointers.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libg2g_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libg2g_ref.so")
# the reference checkout: $G2G_REFERENCE_ROOT, else a sibling of this repository
REF_ROOT = os.environ.get("G2G_REFERENCE_ROOT",
                          os.path.normpath(os.path.join(HERE, "..", "..", "reference")))

_port = None
_ref = None


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_LIB


def build_ref() -> str | None:
    """Builds the reference oracle when its sources are present."""
    if not os.path.isdir(os.path.join(REF_ROOT, "src", "grid2grid")):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={REF_ROOT}"], check=True)
    return REF_LIB


def _capi():
    import grid2grid_gb300.capi as capi
    return capi


def port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_LIB):
            build_port()
        capi = _capi()
        lib = C.CDLL(PORT_LIB)
        lib.g2g_oracle_transform.restype = C.c_int
        lib.g2g_oracle_transform.argtypes = [
            C.c_int, C.POINTER(capi.LayoutDesc), C.POINTER(capi.LayoutDesc),
            C.POINTER(C.c_int), C.POINTER(capi.Op), C.c_int]
        lib.g2g_oracle_last_error.restype = C.c_char_p
        I64P = C.POINTER(C.c_int64)
        lib.g2g_oracle_rank_exchange.restype = C.c_int
        lib.g2g_oracle_rank_exchange.argtypes = [
            C.POINTER(capi.LayoutDesc), C.POINTER(capi.LayoutDesc), C.c_int,
            C.POINTER(capi.Op), C.c_int, I64P, I64P, I64P, I64P, C.c_void_p, C.c_int64]
        lib.g2g_oracle_decomp_cover.restype = C.c_int
        lib.g2g_oracle_decomp_cover.argtypes = [
            C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int), C.c_int,
            C.POINTER(C.c_int), C.POINTER(C.c_int)]
        _port = lib
    return _port


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB):
            raise OSError("reference oracle not built (needs the reference checkout)")
        capi = _capi()
        lib = C.CDLL(REF_LIB)
        lib.g2g_ref_transform.restype = C.c_int
        lib.g2g_ref_transform.argtypes = [
            C.c_int, C.c_int, C.POINTER(capi.LayoutDesc), C.POINTER(capi.LayoutDesc),
            C.POINTER(capi.Op), C.c_int]
        lib.g2g_ref_last_error.restype = C.c_char_p
        lib.g2g_ref_decomp_cover.restype = C.c_int
        lib.g2g_ref_decomp_cover.argtypes = [
            C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int), C.c_int,
            C.POINTER(C.c_int), C.POINTER(C.c_int)]
        I = C.POINTER(C.c_int)
        lib.g2g_ref_scalapack_grid.restype = C.c_int
        lib.g2g_ref_scalapack_grid.argtypes = [C.c_int] * 16 + [I, I, I, I, I, I, I, I,
                                                                 C.POINTER(C.c_longlong), I]
        lib.g2g_ref_scalapack_grid_simple.restype = C.c_int
        lib.g2g_ref_scalapack_grid_simple.argtypes = [C.c_int] * 9 + [
            I, I, I, I, I, I, I, I, C.POINTER(C.c_longlong), I, C.POINTER(C.c_longlong)]
        lib.g2g_ref_comm_volume.restype = C.c_int
        lib.g2g_ref_comm_volume.argtypes = [
            C.POINTER(capi.LayoutDesc), C.POINTER(capi.LayoutDesc), C.c_int,
            C.POINTER(C.c_longlong), I, I, C.c_int]
        lib.g2g_ref_initialize_locally.restype = C.c_longlong
        lib.g2g_ref_initialize_locally.argtypes = [C.POINTER(C.c_double)] + [C.c_int] * 9
        _ref = lib
    return _ref


def _descs(layouts, arenas):
    capi = _capi()
    arr = (capi.LayoutDesc * len(layouts))()
    keep = []
    for k, (L, a) in enumerate(zip(layouts, arenas)):
        d, kk = L.desc(a.ctypes.data)
        arr[k] = d
        keep.append(kk)
    return arr, keep


def _ops(ops):
    capi = _capi()
    if ops is None:
        return None
    arr = (capi.Op * len(ops))()
    for k, o in enumerate(ops):
        arr[k] = o if isinstance(o, capi.Op) else capi.make_op(*o)
    return arr


def port_transform(inits, finals, init_arenas, final_arenas, ops=None, threads=1):
    """Runs the port on host arenas (final arenas are updated in place)."""
    lib = port()
    di, k1 = _descs(inits, init_arenas)
    df, k2 = _descs(finals, final_arenas)
    dts = (C.c_int * len(inits))(*[L.dtype for L in inits])
    opa = _ops(ops)
    rc = lib.g2g_oracle_transform(len(inits), di, df, dts, opa, int(threads))
    if rc:
        raise RuntimeError("oracle port: " + lib.g2g_oracle_last_error().decode())


def port_rank_exchange(Li, Lf, init_arena, final_arena, rank, op=None, pack=True):
    """The port's communication_data of one rank: send / receive counts and
    displacements per peer (elements) and its packed send buffer (bytes)."""
    lib = port()
    capi = _capi()
    P = max(1, Li.n_ranks, Lf.n_ranks)
    di, k1 = _descs([Li], [init_arena])
    df, k2 = _descs([Lf], [final_arena])
    arrs = [np.zeros(P, np.int64) for _ in range(4)]
    I64P = C.POINTER(C.c_int64)
    o = None if op is None else (op if isinstance(op, capi.Op) else capi.make_op(*op))
    rc = lib.g2g_oracle_rank_exchange(di, df, Li.dtype, None if o is None else C.byref(o),
                                      rank, *[a.ctypes.data_as(I64P) for a in arrs], None, 0)
    if rc:
        raise RuntimeError("oracle port: " + lib.g2g_oracle_last_error().decode())
    buf = None
    if pack:
        buf = np.zeros(max(1, int(arrs[0].sum())) * Li.esz, np.uint8)
        rc = lib.g2g_oracle_rank_exchange(di, df, Li.dtype, None if o is None else C.byref(o),
                                          rank, *[a.ctypes.data_as(I64P) for a in arrs],
                                          buf.ctypes.data, buf.size)
        if rc:
            raise RuntimeError("oracle port: " + lib.g2g_oracle_last_error().decode())
        buf = buf[: int(arrs[0].sum()) * Li.esz]
    return {"send_counts": arrs[0], "send_dspls": arrs[1], "recv_counts": arrs[2],
            "recv_dspls": arrs[3], "send_buffer": buf}


# reference call modes (oracle/ref_driver.cpp)
MODE_SINGLE, MODE_SINGLE_SCALED, MODE_VECTOR, MODE_VECTOR_SCALED, MODE_TRANSFORMER = range(5)


def ref_transform(inits, finals, init_arenas, final_arenas, ops=None, mode=None):
    """Runs the reference library (thread-MPI) on host arenas; every pair
    must have the same dtype."""
    lib = ref()
    dts = {L.dtype for L in inits}
    assert len(dts) == 1, "the reference transforms one element type per call"
    if mode is None:
        mode = MODE_SINGLE_SCALED if ops is not None else MODE_SINGLE
    di, k1 = _descs(inits, init_arenas)
    df, k2 = _descs(finals, final_arenas)
    opa = _ops(ops)
    rc = lib.g2g_ref_transform(dts.pop(), len(inits), di, df, opa, int(mode))
    if rc:
        raise RuntimeError("reference: " + lib.g2g_ref_last_error().decode())


def decomp_cover(a, b, which="port"):
    lib = port() if which == "port" else ref()
    a = np.ascontiguousarray(a, dtype=np.int32)
    b = np.ascontiguousarray(b, dtype=np.int32)
    n = max(len(a) - 1, 0)
    s = np.zeros(max(n, 1), dtype=np.int32)
    e = np.zeros(max(n, 1), dtype=np.int32)
    fn = lib.g2g_oracle_decomp_cover if which == "port" else lib.g2g_ref_decomp_cover
    IP = C.POINTER(C.c_int)
    k = fn(a.ctypes.data_as(IP), len(a), b.ctypes.data_as(IP), len(b),
           s.ctypes.data_as(IP), e.ctypes.data_as(IP))
    return s[:k].copy(), e[:k].copy()


def ref_comm_volume(Li, Lf, P, presize=True):
    """The reference's communication_volume and optimal_reordering on two
    layouts' grids: (P x P volume matrix, permutation, reordered). presize
    inserts every rank's self entry into the volume map first (see
    ref_driver.cpp: the reference's own loop inserts them while iterating)."""
    lib = ref()
    di, k1 = Li.desc(0)
    df, k2 = Lf.desc(0)
    vol = np.zeros(P * P, dtype=np.int64)
    perm = np.zeros(P, dtype=np.int32)
    re = C.c_int(0)
    rc = lib.g2g_ref_comm_volume(C.byref(di), C.byref(df), P,
                                 vol.ctypes.data_as(C.POINTER(C.c_longlong)),
                                 perm.ctypes.data_as(C.POINTER(C.c_int)), C.byref(re),
                                 1 if presize else 0)
    if rc != 0:
        raise RuntimeError(lib.g2g_ref_last_error().decode())
    return vol.reshape(P, P), perm, bool(re.value)
