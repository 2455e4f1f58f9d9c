"""The oracle pinned to the reference: the port (this project's CPU
restatement) must reproduce every golden vector the reference produced, the
reference's own known-answer tests, and its layout-builder fixtures. Where the
reference library itself is built (its checkout present), the port is also
compared with it live on fresh seeded cases."""
import numpy as np
import pytest

import g2g_testlib as T
import oracle
from grid2grid_gb300 import capi
from grid2grid_gb300 import layouts as Ls


@pytest.fixture(scope="module", autouse=True)
def _build():
    oracle.build_port()


def test_port_reproduces_every_golden_transform(golden):
    n = 0
    for c in golden.cases():
        got = T.port_run(c["inits"], c["finals"], c["init_arenas"], c["final_before"],
                         c["ops"])
        for k, (g, w) in enumerate(zip(got, c["final_after"])):
            T.assert_arenas_equal(g, w, c["finals"][k], what=f"{c['name']} pair {k}")
        n += 1
    assert n == len(golden.meta["cases"]) >= 60


def test_port_cover_matches_reference_get_decomp_cover(golden):
    for rec in golden.covers:
        s, e = oracle.decomp_cover(rec["a"], rec["b"], "port")
        assert s.tolist() == rec["start"]
        assert e.tolist() == rec["end"]


@pytest.mark.parametrize("m,n,ibm,ibn,fbm,fbn", [
    (10, 10, 2, 2, 5, 5), (10, 10, 2, 3, 3, 5), (10, 12, 2, 3, 2, 6), (10, 12, 2, 3, 3, 5)])
def test_known_answer_scalapack2scalapack(m, n, ibm, ibn, fbm, fbn):
    """The reference's ctest cases (examples/CMakeLists.txt:20-30): values
    cantor(i, j) in a 2x2 block-cyclic layout must land at the same global
    coordinates of the second layout (scalapack_layout.hpp:333-383)."""
    Li = Ls.scalapack_layout(m, n, ibm, ibn, 2, 2, capi.FLOAT64)
    Lf = Ls.scalapack_layout(m, n, fbm, fbn, 2, 2, capi.FLOAT64)
    ai = np.zeros(Li.arena_bytes, np.uint8)
    af = np.zeros(Lf.arena_bytes, np.uint8)
    for b in range(Li.n_blocks):
        i, j = int(Li.blocks["row"][b]), int(Li.blocks["col"][b])
        r = np.arange(Li.rows_split[i], Li.rows_split[i + 1])
        cc = np.arange(Li.cols_split[j], Li.cols_split[j + 1])
        vals = T.cantor(r[:, None], cc[None, :]).astype(np.float64)
        Li.block_view(ai, b)[...] = vals.view(np.uint64)
    out = T.port_run([Li], [Lf], [ai], [af])[0]
    got = Lf.gather(out).view(np.float64)
    want = T.cantor(np.arange(m)[:, None], np.arange(n)[None, :]).astype(np.float64)
    assert np.array_equal(got, want)


def _check_layout(L, ref, rank):
    assert L.rows_split.tolist() == ref["rows_split"]
    assert L.cols_split.tolist() == ref["cols_split"]
    assert L.owners.tolist() == ref["owners"]
    mine = [b for b in range(L.n_blocks) if L.blocks["rank"][b] == rank]
    assert len(mine) == len(ref["blocks"])
    esz = L.esz
    for b, rb in zip(mine, ref["blocks"]):
        assert [int(L.blocks["row"][b]), int(L.blocks["col"][b])] == rb["coord"]
        assert int(L.blocks["stride"][b]) == rb["stride"]
        assert (int(L.offsets[b]) - int(L.rank_base[rank])) // esz == rb["offset"]


def test_scalapack_layout_builder_matches_reference(golden):
    """get_scalapack_grid with submatrix, ordering and source process
    (scalapack_layout.cpp:178-278), including the expectations written in the
    reference's examples/scalapack_submatrix.cpp and
    examples/parallel_scalapack_submatrix.cpp."""
    recs = golden.scalapack["examples"] + golden.scalapack["random"]
    assert len(golden.scalapack["examples"]) == 2
    for rec in recs:
        (lld, m, n, i1, j1, sm, sn, mb, nb, pr, pc, rm, sr, sc) = rec["args"]
        L = Ls.scalapack_layout(m, n, mb, nb, pr, pc, capi.FLOAT64, bool(rm), lld=lld,
                                ij=(i1, j1), sub=(sm, sn), src=(sr, sc))
        for rank_s, ref in rec["reference"].items():
            _check_layout(L, ref, int(rank_s))


def test_line_split_and_rank_grid():
    assert Ls.line_split(20, 96, 27) == [0, 7, 34, 61, 76]
    assert Ls.line_split(100, 200, 32) == [0, 28, 60, 92, 100]
    assert Ls.line_split(0, 5, 32) == [0, 5]
    assert Ls.rank_from_grid(1, 0, 2, 2, row_major=True) == 2
    assert Ls.rank_from_grid(1, 0, 2, 2, row_major=False) == 1
    assert Ls.rank_to_grid(3, 2, 2, row_major=False) == (1, 1)
    with pytest.raises(ValueError):
        Ls.rank_to_grid(4, 2, 2, row_major=False)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference oracle not built here")
@pytest.mark.parametrize("seed", range(6))
def test_port_matches_reference_live(seed):
    rng = np.random.default_rng(1000 + seed)
    for dt in (capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64, capi.COMPLEX128):
        m, n = int(rng.integers(1, 200)), int(rng.integers(1, 200))
        P = int(rng.integers(1, 9))
        t = "NTC"[seed % 3]
        Li = Ls.random_grid_layout(m if t == "N" else n, n if t == "N" else m, P, dt, rng,
                                   ext_hi=48)
        Lf = Ls.random_grid_layout(m, n, P, dt, rng, ext_hi=48)
        ai = Ls.fill_random(np.zeros(Li.arena_bytes, np.uint8), rng)
        af = Ls.fill_random(np.zeros(Lf.arena_bytes, np.uint8), rng)
        ops = [(t, 1.0, 0.0)]
        got = T.port_run([Li], [Lf], [ai], [af], ops)[0]
        ref_f = af.copy()
        oracle.ref_transform([Li], [Lf], [ai.copy()], [ref_f],
                             [capi.make_op(*ops[0])], oracle.MODE_SINGLE_SCALED)
        T.assert_arenas_equal(got, ref_f, Lf, what=f"dt{dt} {t}")


@pytest.mark.skipif(not oracle.ref_available(), reason="reference oracle not built here")
@pytest.mark.parametrize("seed", range(4))
def test_port_scaled_matches_reference_live(seed):
    """final = beta*final + alpha*op(initial) on finite values: the port and
    the live reference agree bit for bit on fresh layouts, every dtype and op."""
    rng = np.random.default_rng(2000 + seed)
    for dt in (capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64, capi.COMPLEX128):
        cplx = dt in (capi.COMPLEX64, capi.COMPLEX128)
        comp = np.float32 if dt in (capi.FLOAT32, capi.COMPLEX64) else np.float64
        m, n = int(rng.integers(1, 150)), int(rng.integers(1, 150))
        P = int(rng.integers(1, 7))
        t = "NTC"[(seed + dt) % 3]
        Li = Ls.random_grid_layout(m if t == "N" else n, n if t == "N" else m, P, dt, rng,
                                   ext_hi=40)
        Lf = Ls.random_grid_layout(m, n, P, dt, rng, ext_hi=40)
        w = np.dtype(comp).itemsize
        ai = np.frombuffer(rng.standard_normal(Li.arena_bytes // w).astype(comp).tobytes(),
                           np.uint8).copy()
        af = np.frombuffer(rng.standard_normal(Lf.arena_bytes // w).astype(comp).tobytes(),
                           np.uint8).copy()
        a = complex(rng.standard_normal(), rng.standard_normal()) if cplx else float(rng.standard_normal())
        b = complex(rng.standard_normal(), rng.standard_normal()) if cplx else float(rng.standard_normal())
        ops = [(t, a, b)]
        got = T.port_run([Li], [Lf], [ai], [af], ops)[0]
        ref_f = af.copy()
        oracle.ref_transform([Li], [Lf], [ai.copy()], [ref_f],
                             [capi.make_op(*ops[0])], oracle.MODE_SINGLE_SCALED)
        T.assert_arenas_equal(got, ref_f, Lf, what=f"scaled dt{dt} {t} {a} {b}")
