"""Test helpers for sharded transforms: host-side restatements of pack,
exchange and unpack over the piece lists the library returns, used to check
the library's exchange plans on the CPU (no GPU needed): the result must be
the oracle port's. Pure copies only (alpha = 1, beta = 0): scaled unpacks run
through the GPU kernels in the GPU tests."""
from __future__ import annotations

import ctypes as C

import numpy as np

from grid2grid_gb300 import capi
from grid2grid_gb300 import exchange as X


def op_matrix(Li, arena, op):
    """op(A) as a matrix of element records, in final coordinates."""
    A = Li.gather(arena)
    t = op[0].upper() if op else "N"
    if t in "TC":
        A = np.ascontiguousarray(A.T)
    if t == "C" and Li.dtype in (capi.COMPLEX64, capi.COMPLEX128):
        w = np.uint32 if Li.dtype == capi.COMPLEX64 else np.uint64
        words = A.view(w).reshape(A.shape + (2,)).copy()
        words[..., 1] ^= w(1) << w(8 * np.dtype(w).itemsize - 1)
        A = words.view(A.dtype).reshape(A.shape)
    return A


def pack(opA, pieces, nbytes, esz):
    """A shard's send buffer: every piece of op(A), column-major, ld = rows."""
    buf = np.zeros(nbytes, np.uint8)
    for p in pieces:
        v = opA[p["row_start"]:p["row_end"], p["col_start"]:p["col_end"]]
        raw = np.ascontiguousarray(v.T).view(np.uint8).ravel()
        o = int(p["offset"]) * esz
        buf[o:o + raw.size] = raw
    return buf


class FinalWriter:
    """Writes pieces (final coordinates) into the blocks of a final layout."""

    def __init__(self, Lf, arena):
        self.L = Lf
        self.arena = arena
        self.index = {(int(r), int(c)): b for b, (r, c) in
                      enumerate(zip(Lf.blocks["row"], Lf.blocks["col"]))}

    def put(self, r0, r1, c0, c1, values):
        L = self.L
        i = int(np.searchsorted(L.rows_split, r0, "right")) - 1
        j = int(np.searchsorted(L.cols_split, c0, "right")) - 1
        b = self.index[(i, j)]
        v = L.block_view(self.arena, b)
        a, c = int(L.rows_split[i]), int(L.cols_split[j])
        v[r0 - a:r1 - a, c0 - c:c1 - c] = values


def unpack(writer, pieces, buf, esz, rec_dtype):
    for p in pieces:
        h, w = p["row_end"] - p["row_start"], p["col_end"] - p["col_start"]
        o = int(p["offset"]) * esz
        vals = buf[o:o + h * w * esz].view(rec_dtype).reshape(w, h).T
        writer.put(p["row_start"], p["row_end"], p["col_start"], p["col_end"], vals)


def local_copy(writer, opA, pieces):
    for p in pieces:
        writer.put(p["row_start"], p["row_end"], p["col_start"], p["col_end"],
                   opA[p["row_start"]:p["row_end"], p["col_start"]:p["col_end"]])


def create(Li_shard, Lf_shard, ia, fa, dtype, op, shard_of_rank, shard, n_shards):
    """Host-only exchange of one shard (descriptors point at host arenas)."""
    lib = capi.load()
    dI, k1 = Li_shard.desc(ia.ctypes.data)
    dF, k2 = Lf_shard.desc(fa.ctypes.data)
    m = (C.c_int32 * len(shard_of_rank))(*shard_of_rank)
    o = capi.make_op(*op) if op else None
    ex = C.c_void_p()
    capi.check(lib.g2g_exchange_create(C.byref(dI), C.byref(dF), dtype,
                                       None if o is None else C.byref(o), n_shards, m, shard,
                                       C.byref(ex)))
    sb = (C.c_int64 * n_shards)()
    rb = (C.c_int64 * n_shards)()
    capi.check(lib.g2g_exchange_get_counts(ex, sb, rb))
    P = max(1, Li_shard.n_ranks, Lf_shard.n_ranks)
    rc = np.zeros(P * P, np.int64)
    capi.check(lib.g2g_exchange_get_rank_counts(ex, P, rc.ctypes.data_as(C.POINTER(C.c_int64))))
    out = {"send_bytes": np.array(sb[:], np.int64), "recv_bytes": np.array(rb[:], np.int64),
           "rank_counts": rc.reshape(P, P),
           "local": X.exchange_pieces(lib, ex, capi.EXCHANGE_LOCAL),
           "send": X.exchange_pieces(lib, ex, capi.EXCHANGE_SEND),
           "recv": X.exchange_pieces(lib, ex, capi.EXCHANGE_RECV)}
    capi.check(lib.g2g_exchange_destroy(ex))
    return out


def rank_segments(pieces, esz):
    """(src, dst) -> (first byte, end byte) of each segment in a buffer."""
    seg = {}
    for p in pieces:
        key = (int(p["src_rank"]), int(p["dst_rank"]))
        o = int(p["offset"]) * esz
        n = int(p["row_end"] - p["row_start"]) * int(p["col_end"] - p["col_start"]) * esz
        a, b = seg.get(key, (o, o))
        assert b == o, f"segment {key} is not contiguous"
        seg[key] = (a, o + n)
    return seg
