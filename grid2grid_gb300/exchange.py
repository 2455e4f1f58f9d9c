"""Sharded transforms: the virtual ranks of a transform spread over several
GPUs, one process per GPU.

The reference exchanges packed buffers between MPI ranks (exchange_async,
src/grid2grid/transform.cpp:41-124). Here a process (a *shard*) holds the
blocks of a set of virtual ranks on its GPU; its part of the transform is

    pack      local pieces into their destination blocks, pieces bound for
              other shards into the send buffer (g2g_exchange_pack, one launch)
    exchange  all-to-all of the packed buffers with per-shard byte counts
              (torch.distributed: NCCL between GPUs, gloo on host tensors)
    unpack    received pieces into their destination blocks
              (g2g_exchange_unpack)

Every shard calls it with the same grids, owners, op and rank-to-shard map,
and with layouts that list only its own ranks' blocks (``shard_layout``).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi


def contiguous_shards(n_ranks: int, n_shards: int) -> list[int]:
    """Rank r -> shard: contiguous, nearly equal ranges of virtual ranks (a
    caller that may relabel ranks first applies optimal_reordering)."""
    if n_shards < 1:
        raise ValueError("n_shards must be >= 1")
    base, extra = divmod(n_ranks, n_shards)
    out = []
    for g in range(n_shards):
        out += [g] * (base + (1 if g < extra else 0))
    return out


def shard_layout(L, shard_of_rank, shard: int):
    """The part of layout L one shard holds: the same grid and owners, only
    the blocks of the shard's ranks."""
    keep = np.array([shard_of_rank[int(r)] == shard for r in L.blocks["rank"]], dtype=bool)
    S = L.copy()
    S.blocks = L.blocks[keep].copy()
    S.offsets = L.offsets[keep].copy()
    return S


def exchange_buffers(send, recv, send_bytes, recv_bytes, group=None):
    """The exchange step: shard g's section for shard h lands in shard h's
    section from g (an all-to-all with per-peer sizes, the reference's
    Isend / Irecv pairs). `send` / `recv` are uint8 tensors on the device the
    process group serves (CUDA for NCCL, host for gloo)."""
    import torch.distributed as dist
    dist.all_to_all_single(recv, send, [int(x) for x in recv_bytes],
                           [int(x) for x in send_bytes], group=group)


class ShardedTransform:
    """One shard's part of a transform from `initial` to `final_` (layout
    descriptors listing this shard's blocks), with device send / receive
    buffers owned by this object."""

    def __init__(self, initial, final_, dtype: int, op, shard_of_rank, shard: int,
                 n_shards: int, device=None, stream=None):
        import torch
        self.lib = capi.load()
        self.n_shards = int(n_shards)
        self.shard = int(shard)
        self._map = (C.c_int32 * len(shard_of_rank))(*[int(x) for x in shard_of_rank])
        self._op = op if (op is None or isinstance(op, capi.Op)) else capi.make_op(*op)
        ex = C.c_void_p()
        capi.check(self.lib.g2g_exchange_create(
            C.byref(initial), C.byref(final_), int(dtype),
            None if self._op is None else C.byref(self._op), self.n_shards, self._map,
            self.shard, C.byref(ex)))
        self.ex = ex
        sb = (C.c_int64 * self.n_shards)()
        rb = (C.c_int64 * self.n_shards)()
        capi.check(self.lib.g2g_exchange_get_counts(ex, sb, rb))
        self.send_bytes = [int(x) for x in sb]
        self.recv_bytes = [int(x) for x in rb]
        dev = torch.device("cuda") if device is None else torch.device(device)
        self.send = torch.empty(max(1, sum(self.send_bytes)), dtype=torch.uint8, device=dev)
        self.recv = torch.empty(max(1, sum(self.recv_bytes)), dtype=torch.uint8, device=dev)
        sp = None if stream is None else C.c_void_p(stream.cuda_stream)
        capi.check(self.lib.g2g_exchange_bind(ex, C.c_void_p(self.send.data_ptr()),
                                              C.c_void_p(self.recv.data_ptr()), sp))

    def pieces(self, which: int):
        return exchange_pieces(self.lib, self.ex, which)

    def pack(self, stream):
        capi.check(self.lib.g2g_exchange_pack(self.ex, C.c_void_p(stream.cuda_stream)))

    def unpack(self, stream):
        capi.check(self.lib.g2g_exchange_unpack(self.ex, C.c_void_p(stream.cuda_stream)))

    def __call__(self, group=None):
        """pack -> all-to-all -> unpack on torch's current stream (the one
        NCCL collectives are ordered with)."""
        import torch
        s = torch.cuda.current_stream(self.send.device)
        self.pack(s)
        exchange_buffers(self.send[:sum(self.send_bytes)], self.recv[:sum(self.recv_bytes)],
                         self.send_bytes, self.recv_bytes, group)
        self.unpack(s)

    def close(self):
        if self.ex:
            capi.check(self.lib.g2g_exchange_destroy(self.ex))
            self.ex = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def exchange_pieces(lib, ex, which: int) -> np.ndarray:
    """A shard's local / send / receive pieces as a structured array."""
    n = C.c_int64()
    capi.check(lib.g2g_exchange_get_pieces(ex, which, 0, None, C.byref(n)))
    arr = (capi.ExchangePiece * max(1, n.value))()
    capi.check(lib.g2g_exchange_get_pieces(ex, which, n.value, arr, C.byref(n)))
    return np.ctypeslib.as_array(arr)[: n.value].copy()
