"""Generates the golden fixtures in this folder from the REFERENCE itself.

Runs kabicm/grid2grid's own transform (compiled unmodified from its sources
over the thread-MPI shim, oracle/_ref/libg2g_ref.so) on small seeded cases and
stores inputs and outputs, so the tests can pin the oracle port and the GPU
path on machines where the reference is absent. Needs the reference checkout
($G2G_REFERENCE_ROOT, else a `reference` folder beside this repository):

    python tests/golden/make_golden.py

Outputs (committed):
  transforms.npz / transforms.json  layouts, input arenas, reference outputs
  covers.json                       get_decomp_cover on seeded split pairs
  scalapack_layouts.json            get_scalapack_grid results, including the
                                    expectations hard-coded in the reference's
                                    examples/scalapack_submatrix.cpp and
                                    examples/parallel_scalapack_submatrix.cpp
                                    (parsed from those files as text)
"""
from __future__ import annotations

import ctypes as C
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
import functools  # noqa: E402
from grid2grid_gb300 import capi  # noqa: E402
from grid2grid_gb300 import layouts as Ls  # noqa: E402

# fixtures pack blocks at 16-byte boundaries to stay small
random_grid = functools.partial(Ls.random_grid_layout, align=16, row_align=4, pad_max=3)

LAYOUT_KEYS = ("rows_split", "cols_split", "owners", "offsets")


def layout_record(L, prefix, arrays):
    for k in LAYOUT_KEYS:
        arrays[f"{prefix}.{k}"] = np.asarray(getattr(L, k))
    arrays[f"{prefix}.blocks"] = L.blocks.copy()
    if L.reordering is not None:
        arrays[f"{prefix}.reordering"] = L.reordering
    return {"n_ranks": L.n_ranks, "dtype": L.dtype, "arena_bytes": L.arena_bytes,
            "reordered": L.reordering is not None}


def finite_fill(L, arena, rng):
    """Seeded finite values (for alpha/beta cases, where NaN payloads are
    not reproducible across builds)."""
    vals = rng.standard_normal(arena.size // 4).astype(np.float32)
    if L.esz in (8, 16) and L.dtype in (capi.FLOAT64, capi.COMPLEX128):
        vals = rng.standard_normal(arena.size // 8)
    arena[:] = np.frombuffer(vals.tobytes(), dtype=np.uint8)[:arena.size]
    return arena


def add_case(cases, arrays, name, inits, finals, ops, mode, rng, finite=False):
    idx = len(cases)
    ia = [np.zeros(L.arena_bytes, np.uint8) for L in inits]
    fa = [np.zeros(L.arena_bytes, np.uint8) for L in finals]
    for L, a in zip(inits, ia):
        finite_fill(L, a, rng) if finite else Ls.fill_random(a, rng)
    for L, a in zip(finals, fa):
        finite_fill(L, a, rng) if finite else Ls.fill_random(a, rng)
    rec = {"name": name, "mode": mode, "pairs": [], "finite": finite}
    before = [a.copy() for a in fa]
    oracle.ref_transform(inits, finals, ia, fa,
                         None if ops is None else [capi.make_op(*o) for o in ops], mode)
    for k, (Li, Lf) in enumerate(zip(inits, finals)):
        p = {"init": layout_record(Li, f"c{idx}.p{k}.i", arrays),
             "final": layout_record(Lf, f"c{idx}.p{k}.f", arrays),
             "op": None if ops is None else [ops[k][0], complex(ops[k][1]).real,
                                              complex(ops[k][1]).imag,
                                              complex(ops[k][2]).real,
                                              complex(ops[k][2]).imag]}
        arrays[f"c{idx}.p{k}.init_arena"] = ia[k]
        arrays[f"c{idx}.p{k}.final_before"] = before[k]
        arrays[f"c{idx}.p{k}.final_after"] = fa[k]
        rec["pairs"].append(p)
    cases.append(rec)


def transforms():
    rng = np.random.default_rng(20240601)
    cases, arrays = [], {}
    # the reference's four ctest cases (examples/CMakeLists.txt:20-30)
    for (m, n, ibm, ibn, fbm, fbn) in [(10, 10, 2, 2, 5, 5), (10, 10, 2, 3, 3, 5),
                                       (10, 12, 2, 3, 2, 6), (10, 12, 2, 3, 3, 5)]:
        Li = Ls.scalapack_layout(m, n, ibm, ibn, 2, 2, capi.FLOAT64)
        Lf = Ls.scalapack_layout(m, n, fbm, fbn, 2, 2, capi.FLOAT64)
        add_case(cases, arrays, f"scalapack2scalapack {m}x{n} {ibm}x{ibn}->{fbm}x{fbn} 2x2",
                 [Li], [Lf], None, oracle.MODE_SINGLE, rng)
    # arbitrary grids, every dtype, N / T / C, plain copies of random bits
    for dt in (capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64, capi.COMPLEX128):
        for trial in range(3):
            m, n = int(rng.integers(1, 64)), int(rng.integers(1, 64))
            P = int(rng.integers(1, 7))
            Lf = random_grid(m, n, P, dt, rng, ext_lo=1, ext_hi=24)
            Li = random_grid(m, n, P, dt, rng, ext_lo=1, ext_hi=24)
            add_case(cases, arrays, f"grid N dt{dt} #{trial}", [Li], [Lf], None,
                     oracle.MODE_SINGLE, rng)
            for t in "TC":
                Li = random_grid(n, m, P, dt, rng, ext_lo=1, ext_hi=24)
                add_case(cases, arrays, f"grid {t} dt{dt} #{trial}", [Li], [Lf],
                         [(t, 1.0, 0.0)], oracle.MODE_SINGLE_SCALED, rng)
    # alpha/beta on finite values
    for dt in (capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64, capi.COMPLEX128):
        cplx = dt in (capi.COMPLEX64, capi.COMPLEX128)
        for t in "NTC":
            m, n = int(rng.integers(1, 70)), int(rng.integers(1, 70))
            P = int(rng.integers(1, 5))
            Lf = random_grid(m, n, P, dt, rng, ext_hi=20)
            Li = random_grid(m if t == "N" else n, n if t == "N" else m, P, dt,
                                       rng, ext_hi=20)
            a = complex(0.75, -1.25) if cplx else 0.75
            b = complex(-0.5, 0.375) if cplx else -0.5
            add_case(cases, arrays, f"scaled {t} dt{dt}", [Li], [Lf], [(t, a, b)],
                     oracle.MODE_SINGLE_SCALED, rng, finite=True)
            add_case(cases, arrays, f"beta0 {t} dt{dt}", [Li], [Lf],
                     [(t, 2.0, 0.0)], oracle.MODE_SINGLE_SCALED, rng, finite=True)
    # vector overload and transformer (one dtype, several pairs)
    for mode, name in ((oracle.MODE_VECTOR, "vector"),
                       (oracle.MODE_TRANSFORMER, "transformer")):
        inits, finals, ops = [], [], []
        for k in range(4):
            m, n = int(rng.integers(1, 60)), int(rng.integers(1, 60))
            P = int(rng.integers(2, 6))
            t = "NTC"[k % 3] if mode == oracle.MODE_TRANSFORMER else "N"
            Lf = random_grid(m, n, P, capi.COMPLEX128, rng, ext_hi=16)
            Li = random_grid(m if t == "N" else n, n if t == "N" else m, P,
                                       capi.COMPLEX128, rng, ext_hi=16)
            inits.append(Li); finals.append(Lf)
            ops.append((t, 1.0, 0.0) if mode == oracle.MODE_VECTOR else
                       (t, complex(1.5, 0.5), complex(0.25, -0.75)))
        add_case(cases, arrays, name, inits, finals,
                 None if mode == oracle.MODE_VECTOR else ops, mode, rng,
                 finite=mode == oracle.MODE_TRANSFORMER)
    # rank reordering, ranks that own nothing, 1x1 matrix, identical grids
    Li = Ls.scalapack_layout(37, 29, 4, 3, 2, 3, capi.FLOAT64)
    Lf = Ls.scalapack_layout(37, 29, 5, 7, 3, 2, capi.FLOAT64)
    perm = [3, 5, 0, 1, 4, 2]
    Lf.reorder_ranks(perm)
    # blocks now belong to reordering[owner]
    Lf.blocks["rank"] = [perm[r] for r in Lf.blocks["rank"]]
    add_case(cases, arrays, "reordered final ranks", [Li], [Lf], None,
             oracle.MODE_SINGLE, rng)
    Li = random_grid(33, 21, 2, capi.FLOAT32, rng, ext_hi=9)
    Lf = random_grid(33, 21, 2, capi.FLOAT32, rng, ext_hi=9)
    Li.n_ranks = 5  # ranks 2..4 own nothing
    Lf.n_ranks = 5
    add_case(cases, arrays, "idle ranks", [Li], [Lf], None, oracle.MODE_SINGLE, rng)
    Li = random_grid(1, 1, 1, capi.COMPLEX64, rng)
    Lf = random_grid(1, 1, 1, capi.COMPLEX64, rng)
    add_case(cases, arrays, "1x1", [Li], [Lf], None, oracle.MODE_SINGLE, rng)
    Li = random_grid(50, 40, 3, capi.FLOAT64, rng, ext_hi=12)
    Lf = random_grid(50, 40, 3, capi.FLOAT64, rng, ext_hi=12)
    Lf.rows_split, Lf.cols_split = Li.rows_split.copy(), Li.cols_split.copy()
    Lf.owners = Li.owners[:, ::-1].copy() if Li.owners.shape == Lf.owners.shape else Lf.owners
    Lf = Ls.Layout(Li.rows_split, Li.cols_split, (Li.owners + 1) % 3, 3, capi.FLOAT64,
                   (Li.blocks["rank"] + 1) % 3, Li.blocks["row"], Li.blocks["col"],
                   Li.offsets, Li.blocks["stride"], Li.arena_bytes)
    add_case(cases, arrays, "identical grids", [Li], [Lf], None, oracle.MODE_SINGLE, rng)
    np.savez_compressed(os.path.join(HERE, "transforms.npz"), **arrays)
    with open(os.path.join(HERE, "transforms.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py",
                   "source": "kabicm/grid2grid transform over thread-MPI", "cases": cases},
                  f, indent=1)
    return len(cases)


def covers():
    rng = np.random.default_rng(7)
    out = []
    for trial in range(60):
        total = int(rng.integers(1, 400))
        a = Ls.random_splits(total, rng, 1, int(rng.integers(1, 60)))
        b = Ls.random_splits(total, rng, 1, int(rng.integers(1, 60)))
        if trial % 10 == 0:
            b = list(a)  # identical grids
        s, e = oracle.decomp_cover(a, b, "ref")
        out.append({"a": a, "b": b, "start": s.tolist(), "end": e.tolist()})
    with open(os.path.join(HERE, "covers.json"), "w") as f:
        json.dump(out, f)
    return len(out)


def _parse_example(path):
    """Expected grid of a reference layout example, read from its source."""
    text = open(path).read()
    rs = [int(x) for x in re.search(r"rows_split\{([^}]*)\}", text).group(1).split(",")]
    cs = [int(x) for x in re.search(r"cols_split\{([^}]*)\}", text).group(1).split(",")]
    own_txt = re.search(r"owners = \{(.*?)\};", text, re.S).group(1)
    owners = [[int(x) for x in row.split(",")]
              for row in re.findall(r"\{([^{}]*)\}", own_txt)]
    lld = re.search(r"int lld_m_dim = (\d+)", text)
    lld = int(lld.group(1)) if lld else None
    blocks = {}
    rank_sections = re.split(r"rank ==\s*(\d)\)", text)
    entry = re.compile(r"\{\{\s*(\d+),\s*(\d+)\s*\},\s*\{\s*(\d+),\s*(\d+)\s*\},\s*"
                       r"\{(\d+), (\d+)\},\s*ptr \+\s*(\d+)\s*\+\s*(\d+)\s*\*\s*"
                       r"(lld_m_dim|\d+),\s*(lld_m_dim|\d+)\}")

    def parse(chunk):
        res = []
        for g in entry.findall(chunk):
            mult = lld if g[8] == "lld_m_dim" else int(g[8])
            stride = lld if g[9] == "lld_m_dim" else int(g[9])
            res.append({"rows": [int(g[0]), int(g[1])], "cols": [int(g[2]), int(g[3])],
                        "coord": [int(g[4]), int(g[5])],
                        "offset": int(g[6]) + int(g[7]) * mult, "stride": stride})
        return res
    if len(rank_sections) > 1:
        for k in range(1, len(rank_sections), 2):
            blocks[int(rank_sections[k])] = parse(rank_sections[k + 1].split("}\n    }")[0]
                                                  if False else rank_sections[k + 1])
    else:
        blocks[0] = parse(text)
    return {"rows_split": rs, "cols_split": cs, "owners": owners, "blocks": blocks}


def scalapack_layouts():
    ref = oracle.ref()
    cap = 4096
    I = C.c_int
    out = {"examples": [], "random": []}

    def run_full(args, rank):
        rs = (I * cap)(); nrs = I(); cs = (I * cap)(); ncs = I(); ow = (I * cap)(); nr = I()
        br = (I * cap)(); bc = (I * cap)(); bo = (C.c_longlong * cap)(); bs = (I * cap)()
        k = ref.g2g_ref_scalapack_grid(*args, rank, cap, rs, C.byref(nrs), cs, C.byref(ncs),
                                       ow, C.byref(nr), br, bc, bo, bs)
        assert k >= 0
        nb_r, nb_c = nrs.value - 1, ncs.value - 1
        return {"rows_split": list(rs[:nrs.value]), "cols_split": list(cs[:ncs.value]),
                "owners": [list(ow[i * nb_c:(i + 1) * nb_c]) for i in range(nb_r)],
                "n_ranks": nr.value,
                "blocks": [{"coord": [br[b], bc[b]], "offset": bo[b], "stride": bs[b]}
                           for b in range(k)]}

    ex_root = os.path.join(oracle.REF_ROOT, "examples")
    # (lld, m, n, i1, j1, sub_m, sub_n, mb, nb, pr, pc, row_major, src_r, src_c)
    examples = [("scalapack_submatrix.cpp", (200, 200, 200, 1, 101, 100, 100, 32, 32, 1, 1,
                                             1, 0, 0), 1),
                ("parallel_scalapack_submatrix.cpp", (60, 113, 56, 21, 8, 76, 37, 27, 13, 2,
                                                      2, 1, 0, 0), 4)]
    for fname, args, P in examples:
        expected = _parse_example(os.path.join(ex_root, fname))
        got = {r: run_full(args, r) for r in range(P)}
        for r in range(P):
            g = got[r]
            assert g["rows_split"] == expected["rows_split"], fname
            assert g["cols_split"] == expected["cols_split"], fname
            assert g["owners"] == expected["owners"], fname
            exp_blocks = expected["blocks"][r if r in expected["blocks"] else 0]
            assert [(b["coord"], b["offset"], b["stride"]) for b in g["blocks"]] == \
                   [(b["coord"], b["offset"], b["stride"]) for b in exp_blocks], (fname, r)
        out["examples"].append({"file": fname, "args": list(args), "ranks": P,
                                "expected": expected, "reference": got})
    rng = np.random.default_rng(11)
    for trial in range(25):
        m, n = int(rng.integers(1, 300)), int(rng.integers(1, 300))
        mb, nb = int(rng.integers(1, 40)), int(rng.integers(1, 40))
        pr, pc = int(rng.integers(1, 4)), int(rng.integers(1, 4))
        i1, j1 = int(rng.integers(1, m + 1)), int(rng.integers(1, n + 1))
        sm, sn = int(rng.integers(1, m - i1 + 2)), int(rng.integers(1, n - j1 + 2))
        rm = int(rng.integers(0, 2))
        sr, sc = int(rng.integers(0, pr)), int(rng.integers(0, pc))
        lld = m + int(rng.integers(0, 5))
        args = (lld, m, n, i1, j1, sm, sn, mb, nb, pr, pc, rm, sr, sc)
        out["random"].append({"args": list(args),
                              "reference": {r: run_full(args, r) for r in range(pr * pc)}})
    with open(os.path.join(HERE, "scalapack_layouts.json"), "w") as f:
        json.dump(out, f)
    return len(out["examples"]) + len(out["random"])


if __name__ == "__main__":
    if oracle.build_ref() is None:
        sys.exit("reference checkout not found")
    oracle.build_port()
    print("transform cases:", transforms())
    print("covers:", covers())
    print("scalapack layouts:", scalapack_layouts())
