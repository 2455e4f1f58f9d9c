"""Sharded transforms on one GPU: several shards' parts run through the real
pack and unpack kernels, with the buffer exchange between them done as
device-to-device copies (what NCCL's all-to-all would deliver). Every shard's
send buffer must hold, segment by segment, the reference's packed send
buffers of its ranks (the oracle port's), and the final arenas -- padding
included -- must equal the port's transform, bit for bit (alpha/beta on
finite values)."""
import numpy as np
import pytest

import g2g_testlib as T
import oracle
from grid2grid_gb300 import capi
from grid2grid_gb300 import exchange as X
from grid2grid_gb300 import layouts as Ls
import exchange_testlib as XT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _setup():
    import torch
    assert torch.cuda.is_available()
    from grid2grid_gb300 import build
    build.build()
    capi.load()
    oracle.build_port()


def _finite(L, rng):
    comp = np.float32 if L.dtype in (capi.FLOAT32, capi.COMPLEX64) else np.float64
    w = np.dtype(comp).itemsize
    return np.frombuffer(rng.standard_normal(L.arena_bytes // w).astype(comp).tobytes(),
                         np.uint8).copy()


def _run_shards(Li, Lf, ia, fa, op, smap, G):
    """All shards of a sharded transform on this GPU; returns the final
    arena and every shard's send buffer (host) and piece lists."""
    import torch
    di = torch.from_numpy(ia).cuda()
    df = torch.from_numpy(fa).cuda()
    keep, shards = [], []
    for g in range(G):
        dI, k1 = X.shard_layout(Li, smap, g).desc(di.data_ptr())
        dF, k2 = X.shard_layout(Lf, smap, g).desc(df.data_ptr())
        keep += [k1, k2, dI, dF]
        shards.append(X.ShardedTransform(dI, dF, Li.dtype, op, smap, g, G))
    s = torch.cuda.current_stream()
    for sh in shards:
        sh.pack(s)
    # the exchange: shard g's section for h -> shard h's section from g
    for h, dst in enumerate(shards):
        pos = 0
        for g, src in enumerate(shards):
            n = src.send_bytes[h]
            assert n == dst.recv_bytes[g]
            if n:
                so = sum(src.send_bytes[:h])
                dst.recv[pos:pos + n].copy_(src.send[so:so + n])
            pos += n
    for sh in shards:
        sh.unpack(s)
    torch.cuda.synchronize()
    out = df.cpu().numpy()
    sends = [sh.send[:sum(sh.send_bytes)].cpu().numpy() for sh in shards]
    pieces = [sh.pieces(capi.EXCHANGE_SEND) for sh in shards]
    for sh in shards:
        sh.close()
    return out, sends, pieces


def _check(Li, Lf, ia, fa, op, maps, nan_ok=False):
    P = max(Li.n_ranks, Lf.n_ranks)
    want = T.port_run([Li], [Lf], [ia], [fa], [op])[0]
    port = [oracle.port_rank_exchange(Li, Lf, ia, fa, r, op, pack=True) for r in range(P)]
    for G, smap in maps:
        out, sends, pieces = _run_shards(Li, Lf, ia, fa, op, smap, G)
        T.assert_arenas_equal(out, want, Lf, nan_equivalent=nan_ok,
                              what=f"{G} shards {smap} {op}")
        for g in range(G):
            for (s, d), (a, b) in XT.rank_segments(pieces[g], Li.esz).items():
                o = int(port[s]["send_dspls"][d]) * Li.esz
                assert b - a == int(port[s]["send_counts"][d]) * Li.esz
                assert np.array_equal(sends[g][a:b], port[s]["send_buffer"][o:o + b - a]), \
                    f"send segment {s}->{d} of shard {g}"


@pytest.mark.parametrize("dt", [capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64, capi.COMPLEX128])
@pytest.mark.parametrize("t", ["N", "T", "C"])
def test_sharded_copy_matches_port(dt, t):
    rng = np.random.default_rng(400 + 10 * dt + "NTC".index(t))
    m, n, P = 333, 271, 9
    Li = Ls.random_grid_layout(m if t == "N" else n, n if t == "N" else m, P, dt, rng,
                               ext_hi=110)
    Lf = Ls.random_grid_layout(m, n, P, dt, rng, ext_hi=90)
    ia = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
    fa = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    maps = [(2, X.contiguous_shards(P, 2)), (3, [int(x) for x in rng.integers(0, 3, P)]),
            (1, [0] * P), (P, list(range(P)))]
    _check(Li, Lf, ia, fa, (t, 1.0, 0.0), maps)


@pytest.mark.parametrize("dt,op", [(capi.FLOAT32, ("N", 2.0, 0.5)),
                                   (capi.FLOAT64, ("T", -0.5, 3.0)),
                                   (capi.COMPLEX64, ("C", complex(1.5, -0.5), complex(0.25, 2.0))),
                                   (capi.COMPLEX128, ("N", complex(0.0, 1.0), 0.0))])
def test_sharded_scaled_matches_port(dt, op):
    """alpha/beta at the unpack and in the local copies, finite values."""
    rng = np.random.default_rng(480 + dt)
    t = op[0]
    m, n, P = 257, 190, 6
    Li = Ls.random_grid_layout(m if t == "N" else n, n if t == "N" else m, P, dt, rng,
                               ext_hi=80)
    Lf = Ls.random_grid_layout(m, n, P, dt, rng, ext_hi=80)
    ia, fa = _finite(Li, rng), _finite(Lf, rng)
    _check(Li, Lf, ia, fa, op, [(2, X.contiguous_shards(P, 2)), (3, [0, 1, 2, 2, 1, 0])])


def test_sharded_block_cyclic_reordered():
    """ScaLAPACK layouts, a reordered final grid and idle ranks, two shards."""
    rng = np.random.default_rng(9)
    Li = Ls.scalapack_layout(600, 520, 32, 32, 2, 4, capi.FLOAT64)
    Lf = Ls.scalapack_layout(600, 520, 96, 40, 4, 2, capi.FLOAT64, row_major=True)
    perm = [int(x) for x in rng.permutation(8)]
    Lf.reorder_ranks(perm)
    Lf.blocks["rank"] = [perm[r] for r in Lf.blocks["rank"]]
    Li.n_ranks = 10
    ia = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
    fa = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    _check(Li, Lf, ia, fa, ("N", 1.0, 0.0), [(2, X.contiguous_shards(10, 2))])


def test_sharded_plan_byte_counts():
    """The pack and unpack plans move exactly the bytes the counts name."""
    import ctypes as C
    import torch
    rng = np.random.default_rng(5)
    Li = Ls.random_grid_layout(300, 200, 4, capi.COMPLEX64, rng, ext_hi=70)
    Lf = Ls.random_grid_layout(300, 200, 4, capi.COMPLEX64, rng, ext_hi=70)
    di = torch.zeros(Li.arena_bytes, dtype=torch.uint8, device="cuda")
    df = torch.zeros(Lf.arena_bytes, dtype=torch.uint8, device="cuda")
    smap = [0, 1, 0, 1]
    dI, k1 = X.shard_layout(Li, smap, 0).desc(di.data_ptr())
    dF, k2 = X.shard_layout(Lf, smap, 0).desc(df.data_ptr())
    sh = X.ShardedTransform(dI, dF, capi.COMPLEX64, None, smap, 0, 2)
    lib = capi.load()
    info = capi.PlanInfo()
    capi.check(lib.g2g_exchange_get_plan_info(sh.ex, capi.EXCHANGE_SEND, C.byref(info)))
    assert info.bytes_moved == sum(sh.send_bytes)
    capi.check(lib.g2g_exchange_get_plan_info(sh.ex, capi.EXCHANGE_RECV, C.byref(info)))
    assert info.bytes_moved == sum(sh.recv_bytes)
    capi.check(lib.g2g_exchange_get_plan_info(sh.ex, capi.EXCHANGE_LOCAL, C.byref(info)))
    local = sh.pieces(capi.EXCHANGE_LOCAL)
    n_local = int(((local["row_end"] - local["row_start"]) *
                   (local["col_end"] - local["col_start"])).sum())
    assert info.bytes_moved == n_local * 8
    sh.close()
