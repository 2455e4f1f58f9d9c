"""Sharded transforms on the CPU: the exchange plans the library builds for
every shard (grid cover, per-rank counts, buffer layout, piece lists) checked
against the oracle port, and the whole transform restated on the host from
those piece lists -- pack, exchange, unpack -- against the port's result.
The world-size-2 gloo test runs the same with one process per shard and the
buffers exchanged by torch.distributed (all_to_all_single), as GPUs would
exchange them over NCCL."""
import os

import numpy as np
import pytest

import exchange_testlib as XT
import g2g_testlib as T
import oracle
from grid2grid_gb300 import capi
from grid2grid_gb300 import exchange as X
from grid2grid_gb300 import layouts as Ls


@pytest.fixture(scope="module", autouse=True)
def _setup():
    from grid2grid_gb300 import build
    build.build()
    capi.load()
    oracle.build_port()


def _case(seed, dt, t, m, n, P, reorder=False):
    rng = np.random.default_rng(seed)
    Li = Ls.random_grid_layout(m if t == "N" else n, n if t == "N" else m, P, dt, rng,
                               ext_hi=int(rng.integers(8, 120)))
    Lf = Ls.random_grid_layout(m, n, P, dt, rng, ext_hi=int(rng.integers(8, 120)))
    if reorder:
        perm = [int(x) for x in rng.permutation(P)]
        Lf.reorder_ranks(perm)
        Lf.blocks["rank"] = [perm[r] for r in Lf.blocks["rank"]]
    ia = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
    fa = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    return Li, Lf, ia, fa


def _maps(P, rng):
    yield 2, X.contiguous_shards(P, 2)
    yield 3, [int(x) for x in rng.integers(0, 3, size=P)]
    yield 1, [0] * P


def _check_case(Li, Lf, ia, fa, op):
    """Every shard's exchange, for several rank-to-shard maps, against the
    port: counts per rank pair, buffer segments, final arenas."""
    P = max(Li.n_ranks, Lf.n_ranks)
    esz = Li.esz
    rng = np.random.default_rng(P)
    want = T.port_run([Li], [Lf], [ia], [fa], [op])[0]
    port = [oracle.port_rank_exchange(Li, Lf, ia, fa, r, op, pack=True) for r in range(P)]
    opA = XT.op_matrix(Li, ia, op)
    rec = opA.dtype
    for G, smap in _maps(P, rng):
        parts = []
        for g in range(G):
            Lis, Lfs = X.shard_layout(Li, smap, g), X.shard_layout(Lf, smap, g)
            parts.append(XT.create(Lis, Lfs, ia, fa, Li.dtype, op, smap, g, G))
        # the reference's counts: row s of the rank counts, self excluded
        for e in parts:
            rc = e["rank_counts"]
            for r in range(P):
                sc = rc[r].copy()
                sc[r] = 0
                assert np.array_equal(sc, port[r]["send_counts"]), f"send counts rank {r}"
                cc = rc[:, r].copy()
                cc[r] = 0
                assert np.array_equal(cc, port[r]["recv_counts"]), f"recv counts rank {r}"
        for g in range(G):
            for h in range(G):
                assert parts[g]["send_bytes"][h] == parts[h]["recv_bytes"][g]
                want_b = sum(int(parts[g]["rank_counts"][s, d]) for s in range(P)
                             for d in range(P) if smap[s] == g and smap[d] == h and g != h)
                assert parts[g]["send_bytes"][h] == want_b * esz
        # each (s, d) segment of a shard's send buffer is rank s's segment for
        # d in the reference's own send buffer
        sbufs = [XT.pack(opA, parts[g]["send"], int(parts[g]["send_bytes"].sum()), esz)
                 for g in range(G)]
        for g in range(G):
            for (s, d), (a, b) in XT.rank_segments(parts[g]["send"], esz).items():
                ps = port[s]
                o = int(ps["send_dspls"][d]) * esz
                n = int(ps["send_counts"][d]) * esz
                assert b - a == n
                assert np.array_equal(sbufs[g][a:b], ps["send_buffer"][o:o + n]), (s, d)
        # exchange: the section of g for h lands in h's section from g
        rbufs = []
        for h in range(G):
            secs = []
            for g in range(G):
                so = int(parts[g]["send_bytes"][:h].sum())
                secs.append(sbufs[g][so:so + int(parts[g]["send_bytes"][h])])
            rbufs.append(np.concatenate(secs) if secs else np.zeros(0, np.uint8))
        out = fa.copy()
        wr = XT.FinalWriter(Lf, out)
        for h in range(G):
            XT.unpack(wr, parts[h]["recv"], rbufs[h], esz, rec)
            XT.local_copy(wr, opA, parts[h]["local"])
        T.assert_arenas_equal(out, want, Lf, what=f"{G} shards {smap}")


@pytest.mark.parametrize("dt", [capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64, capi.COMPLEX128])
@pytest.mark.parametrize("t", ["N", "T", "C"])
def test_exchange_plans_match_port(dt, t):
    Li, Lf, ia, fa = _case(10 * dt + "NTC".index(t), dt, t, 237, 181, 7)
    _check_case(Li, Lf, ia, fa, (t, 1.0, 0.0))


def test_exchange_reordered_and_idle_ranks():
    Li = Ls.scalapack_layout(301, 257, 17, 9, 3, 4, capi.FLOAT64)
    Lf = Ls.scalapack_layout(301, 257, 23, 31, 4, 3, capi.FLOAT64, row_major=True)
    rng = np.random.default_rng(8)
    perm = [int(x) for x in rng.permutation(12)]
    Lf.reorder_ranks(perm)
    Lf.blocks["rank"] = [perm[r] for r in Lf.blocks["rank"]]
    Li.n_ranks = 16  # ranks 12..15 hold nothing
    ia = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
    fa = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
    _check_case(Li, Lf, ia, fa, ("N", 1.0, 0.0))


def test_exchange_refuses_blocks_of_other_shards():
    Li, Lf, ia, fa = _case(3, capi.FLOAT32, "N", 100, 90, 4)
    smap = [0, 0, 1, 1]
    with pytest.raises(capi.G2GError, match="another shard"):
        XT.create(Li, X.shard_layout(Lf, smap, 0), ia, fa, Li.dtype, None, smap, 0, 2)
    short = X.shard_layout(Li, smap, 0)  # one block of shard 0 left out
    short.blocks = short.blocks[1:].copy()
    short.offsets = short.offsets[1:].copy()
    with pytest.raises(capi.G2GError, match="missing"):
        XT.create(short, X.shard_layout(Lf, smap, 0), ia, fa, Li.dtype, None, smap, 0, 2)
    with pytest.raises(capi.G2GError, match="shard"):
        XT.create(Li, Lf, ia, fa, Li.dtype, None, [0, 0, 5, 1], 0, 2)


# ------------------------------------------------------------ gloo ranks
def _gloo_worker(rank, world, port, result):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        for dt, t in ((capi.FLOAT32, "N"), (capi.COMPLEX128, "C"), (capi.FLOAT64, "T")):
            Li, Lf, ia, fa = _case(70 + dt, dt, t, 211, 173, 6)
            op = (t, 1.0, 0.0)
            P = 6
            smap = X.contiguous_shards(P, world)
            e = XT.create(X.shard_layout(Li, smap, rank), X.shard_layout(Lf, smap, rank), ia,
                          fa, dt, op, smap, rank, world)
            # counts against the port, for this shard's ranks
            for r in range(P):
                if smap[r] != rank:
                    continue
                pr = oracle.port_rank_exchange(Li, Lf, ia, fa, r, op, pack=False)
                sc = e["rank_counts"][r].copy()
                sc[r] = 0
                assert np.array_equal(sc, pr["send_counts"])
                assert np.array_equal(np.concatenate([[0], np.cumsum(sc)[:-1]]),
                                      pr["send_dspls"])
            opA = XT.op_matrix(Li, ia, op)
            send = torch.from_numpy(XT.pack(opA, e["send"], int(e["send_bytes"].sum()),
                                            Li.esz))
            recv = torch.zeros(int(e["recv_bytes"].sum()), dtype=torch.uint8)
            X.exchange_buffers(send, recv, e["send_bytes"], e["recv_bytes"])
            out = fa.copy()
            wr = XT.FinalWriter(X.shard_layout(Lf, smap, rank), out)
            XT.unpack(wr, e["recv"], recv.numpy(), Li.esz, opA.dtype)
            XT.local_copy(wr, opA, e["local"])
            want = T.port_run([Li], [Lf], [ia], [fa], [op])[0]
            # this shard's blocks, padding included, equal the port's
            for b in range(Lf.n_blocks):
                if smap[int(Lf.blocks["rank"][b])] != rank:
                    continue
                rows, cols = Lf.storage_shape(b)
                o = int(Lf.offsets[b])
                nb = int(Lf.blocks["stride"][b]) * cols * Lf.esz
                assert np.array_equal(out[o:o + nb], want[o:o + nb]), f"block {b}"
        result[rank] = "ok"
    except Exception as ex:  # reported to the parent
        result[rank] = repr(ex)
    finally:
        dist.destroy_process_group()


def test_gloo_two_shards_exchange():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    result = mgr.dict()
    procs = [ctx.Process(target=_gloo_worker, args=(r, 2, port, result)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    for p in procs:
        if p.is_alive():
            p.kill()
    assert dict(result) == {0: "ok", 1: "ok"}, dict(result)
