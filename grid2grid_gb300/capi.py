"""ctypes binding of the C ABI declared in include/grid2grid_gb300.h.

This is the binding a Python caller of the library adds: plain ctypes
structures mirroring the header and a loader for the in-tree shared library
``grid2grid_gb300/_lib/libgrid2grid_gb300.so``. Loading fails loudly when the
library has not been built; there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(_HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libgrid2grid_gb300.so")

# g2g_status
SUCCESS = 0
ERROR_INVALID_ARGUMENT = 1
ERROR_CUDA = 2
ERROR_OUT_OF_MEMORY = 3
ERROR_BUDGET = 4
ERROR_TIMEOUT = 5
ERROR_NOT_READY = 6
ERROR_UNSUPPORTED = 7

# g2g_dtype
FLOAT32, FLOAT64, COMPLEX64, COMPLEX128 = 0, 1, 2, 3
DTYPE_SIZE = {FLOAT32: 4, FLOAT64: 8, COMPLEX64: 8, COMPLEX128: 16}
DTYPE_NAME = {FLOAT32: "float32", FLOAT64: "float64", COMPLEX64: "complex64",
              COMPLEX128: "complex128"}
DTYPE_BY_NAME = {v: k for k, v in DTYPE_NAME.items()}


class BlockDesc(C.Structure):
    _fields_ = [
        ("rank", C.c_int32),
        ("row", C.c_int32),
        ("col", C.c_int32),
        ("transpose_on_copy", C.c_int32),
        ("conjugate_on_copy", C.c_int32),
        ("reserved", C.c_int32),
        ("stride", C.c_int64),
        ("data", C.c_void_p),
    ]


class LayoutDesc(C.Structure):
    _fields_ = [
        ("n_block_rows", C.c_int32),
        ("n_block_cols", C.c_int32),
        ("rows_split", C.POINTER(C.c_int32)),
        ("cols_split", C.POINTER(C.c_int32)),
        ("owners", C.POINTER(C.c_int32)),
        ("n_ranks", C.c_int32),
        ("n_reordering", C.c_int32),
        ("reordering", C.POINTER(C.c_int32)),
        ("n_blocks", C.c_int32),
        ("reserved", C.c_int32),
        ("blocks", C.POINTER(BlockDesc)),
    ]


class Op(C.Structure):
    _fields_ = [
        ("trans", C.c_char),
        ("reserved", C.c_char * 7),
        ("alpha", C.c_double * 2),
        ("beta", C.c_double * 2),
    ]


class Tuning(C.Structure):
    _fields_ = [
        ("tile_bytes", C.c_int32),
        ("tile_dim", C.c_int32),
        ("ctas_per_sm", C.c_int32),
        ("threads", C.c_int32),
        ("unroll", C.c_int32),
        ("stages", C.c_int32),
        ("ring", C.c_int32),
        ("tile_run", C.c_int32),
        ("l2_prefetch", C.c_int32),
        ("tensor_boxes", C.c_int32),
    ]


class ServerConfig(C.Structure):
    _fields_ = [
        ("hbm_budget_bytes", C.c_int64),
        ("max_launches_in_flight", C.c_int32),
        ("max_batch_requests", C.c_int32),
        ("plan_cache_entries", C.c_int32),
        ("reserved", C.c_int32 * 3),
    ]


class RequestTimes(C.Structure):
    _fields_ = [
        ("submit_ns", C.c_int64),
        ("launch_ns", C.c_int64),
        ("complete_ns", C.c_int64),
        ("bytes", C.c_int64),
        ("status", C.c_int32),
        ("batch_size", C.c_int32),
    ]


class ServerStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_int64),
        ("completed", C.c_int64),
        ("launches", C.c_int64),
        ("plan_cache_hits", C.c_int64),
        ("plan_cache_misses", C.c_int64),
        ("bytes_completed", C.c_int64),
        ("inflight_bytes_peak", C.c_int64),
    ]


class PlanInfo(C.Structure):
    _fields_ = [
        ("n_pairs", C.c_int32),
        ("n_ranks", C.c_int32),
        ("n_pieces", C.c_int64),
        ("n_tiles", C.c_int64),
        ("bytes_moved", C.c_int64),
        ("bytes_min_traffic", C.c_int64),
        ("metadata_bytes", C.c_int64),
        ("graph_captured", C.c_int32),
        ("device_status", C.c_int32),
        ("tensor_boxes_ok", C.c_int32),
        ("tile_paths", C.c_int32),
        ("tuning", Tuning),
    ]


def make_op(trans="N", alpha=1.0, beta=0.0) -> Op:
    op = Op()
    op.trans = trans.encode() if isinstance(trans, str) else bytes([trans])
    a = complex(alpha)
    b = complex(beta)
    op.alpha[0], op.alpha[1] = a.real, a.imag
    op.beta[0], op.beta[1] = b.real, b.imag
    return op


# (name, restype, argtypes) of every exported function in the header.
_VP = C.c_void_p
_I32P = C.POINTER(C.c_int32)
class ScalapackDesc(C.Structure):
    _fields_ = [
        ("m", C.c_int32), ("n", C.c_int32),
        ("mb", C.c_int32), ("nb", C.c_int32),
        ("rsrc", C.c_int32), ("csrc", C.c_int32),
        ("nprow", C.c_int32), ("npcol", C.c_int32),
        ("row_major", C.c_int32),
        ("reserved", C.c_int32),
    ]


class ExchangePiece(C.Structure):
    _fields_ = [
        ("row_start", C.c_int32), ("row_end", C.c_int32),
        ("col_start", C.c_int32), ("col_end", C.c_int32),
        ("src_rank", C.c_int32), ("dst_rank", C.c_int32),
        ("offset", C.c_int64),
    ]


EXCHANGE_LOCAL, EXCHANGE_SEND, EXCHANGE_RECV = 0, 1, 2

SIGNATURES = [
    ("g2g_last_error_string", C.c_char_p, []),
    ("g2g_version_string", C.c_char_p, []),
    ("g2g_plan_create", C.c_int,
     [C.POINTER(LayoutDesc), C.POINTER(LayoutDesc), C.c_int, C.POINTER(Op), _VP,
      C.POINTER(_VP)]),
    ("g2g_plan_create_batch", C.c_int,
     [C.c_int32, C.POINTER(LayoutDesc), C.POINTER(LayoutDesc), C.POINTER(C.c_int),
      C.POINTER(Op), _VP, C.POINTER(_VP)]),
    ("g2g_plan_create_cast", C.c_int,
     [C.POINTER(LayoutDesc), C.c_int, C.POINTER(LayoutDesc), C.c_int, C.POINTER(Op), _VP,
      C.POINTER(_VP)]),
    ("g2g_transform_cast", C.c_int,
     [C.POINTER(LayoutDesc), C.c_int, C.POINTER(LayoutDesc), C.c_int, C.POINTER(Op), _VP]),
    ("g2g_plan_execute", C.c_int, [_VP, _VP]),
    ("g2g_plans_execute", C.c_int, [C.c_int32, C.POINTER(_VP), _VP]),
    ("g2g_plan_capture_graph", C.c_int, [_VP, _VP]),
    ("g2g_plan_set_tuning", C.c_int, [_VP, C.POINTER(Tuning)]),
    ("g2g_plan_autotune", C.c_int, [_VP, _VP, C.c_int32, C.POINTER(Tuning)]),
    ("g2g_plan_get_info", C.c_int, [_VP, C.POINTER(PlanInfo)]),
    ("g2g_plan_destroy", C.c_int, [_VP]),
    ("g2g_transform", C.c_int,
     [C.POINTER(LayoutDesc), C.POINTER(LayoutDesc), C.c_int, C.POINTER(Op), _VP]),
    ("g2g_transform_noalloc", C.c_int,
     [C.POINTER(LayoutDesc), C.POINTER(LayoutDesc), C.c_int, C.POINTER(Op), _VP]),
    ("g2g_transform_batch", C.c_int,
     [C.c_int32, C.POINTER(LayoutDesc), C.POINTER(LayoutDesc), C.POINTER(C.c_int),
      C.POINTER(Op), _VP]),
    ("g2g_plan_cache_clear", C.c_int, []),
    ("g2g_grid_cover", C.c_int,
     [_I32P, C.c_int32, _I32P, C.c_int32, _I32P, _I32P, _VP]),
    ("g2g_communication_volume", C.c_int,
     [C.POINTER(LayoutDesc), C.POINTER(LayoutDesc), C.c_int32, C.POINTER(C.c_int64)]),
    ("g2g_optimal_reordering", C.c_int,
     [C.POINTER(C.c_int64), C.c_int32, _I32P, _I32P]),
    ("g2g_communication_volume_device", C.c_int,
     [C.POINTER(LayoutDesc), C.POINTER(LayoutDesc), C.c_int32, _VP, _VP]),
    ("g2g_optimal_reordering_device", C.c_int, [_VP, C.c_int32, _VP, _VP, _VP]),
    ("g2g_layout_create_scalapack", C.c_int,
     [C.POINTER(ScalapackDesc), C.c_int32, C.c_int32, C.c_int32, C.c_int32,
      C.POINTER(_VP), _I32P, C.c_int, C.POINTER(_VP)]),
    ("g2g_layout_get_desc", C.c_int, [_VP, C.POINTER(LayoutDesc)]),
    ("g2g_layout_destroy", C.c_int, [_VP]),
    ("g2g_gemr2d", C.c_int,
     [C.c_int32, C.c_int32,
      C.POINTER(_VP), C.c_int32, C.c_int32, C.POINTER(ScalapackDesc), _I32P,
      C.POINTER(_VP), C.c_int32, C.c_int32, C.POINTER(ScalapackDesc), _I32P,
      C.c_int, C.POINTER(Op), _VP]),
    ("g2g_exchange_create", C.c_int,
     [C.POINTER(LayoutDesc), C.POINTER(LayoutDesc), C.c_int, C.POINTER(Op), C.c_int32,
      _I32P, C.c_int32, C.POINTER(_VP)]),
    ("g2g_exchange_get_counts", C.c_int,
     [_VP, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("g2g_exchange_get_rank_counts", C.c_int, [_VP, C.c_int32, C.POINTER(C.c_int64)]),
    ("g2g_exchange_get_pieces", C.c_int,
     [_VP, C.c_int32, C.c_int64, C.POINTER(ExchangePiece), C.POINTER(C.c_int64)]),
    ("g2g_exchange_bind", C.c_int, [_VP, _VP, _VP, _VP]),
    ("g2g_exchange_pack", C.c_int, [_VP, _VP]),
    ("g2g_exchange_unpack", C.c_int, [_VP, _VP]),
    ("g2g_exchange_get_plan_info", C.c_int, [_VP, C.c_int32, C.POINTER(PlanInfo)]),
    ("g2g_exchange_destroy", C.c_int, [_VP]),
    ("g2g_server_create", C.c_int, [C.POINTER(ServerConfig), C.POINTER(_VP)]),
    ("g2g_server_submit", C.c_int,
     [_VP, C.POINTER(LayoutDesc), C.POINTER(LayoutDesc), C.c_int, C.POINTER(Op),
      C.POINTER(C.c_uint64)]),
    ("g2g_server_wait", C.c_int, [_VP, C.c_uint64, C.c_int64, C.POINTER(RequestTimes)]),
    ("g2g_server_replay", C.c_int,
     [_VP, C.c_int32, C.POINTER(LayoutDesc), C.POINTER(LayoutDesc), C.POINTER(C.c_int),
      C.POINTER(Op), C.c_int64, _I32P, C.POINTER(C.c_double), C.POINTER(RequestTimes)]),
    ("g2g_server_get_stats", C.c_int, [_VP, C.POINTER(ServerStats)]),
    ("g2g_server_destroy", C.c_int, [_VP]),
]

_lib = None


class G2GError(RuntimeError):
    """A non-success g2g_status, with the library's error string."""

    def __init__(self, status: int, message: str):
        super().__init__(f"g2g status {status}: {message}")
        self.status = status


def load(path: str | None = None):
    """Loads the in-tree library (once) and declares every signature."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(
            f"{p} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(p)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int):
    if status != SUCCESS:
        msg = load().g2g_last_error_string().decode(errors="replace")
        raise G2GError(status, msg)
    return status


def header_symbols(header_path: str) -> list[str]:
    """Names of the functions a header declares (for the export test)."""
    import re
    text = open(header_path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(g2g_[a-z0-9_]+)\s*\(", text)))
