"""Seeded synthetic redistribution workloads at the benchmark shapes.

No dataset is involved in grid2grid's benchmarks; these generators produce
layouts with the stated sizes, layouts and value distributions:

  block_cyclic_f64_4096      double 4096 x 4096; block-cyclic 32x32 -> 128x64 on a
                             2x2 column-major process grid (4 virtual ranks),
                             lld = local rows; entry(i, j) = double(i + j*4096)
  random_grid_f32_16384      float 16384 x 16384, 16 virtual ranks; initial and
                             final split points with extents U[1, 2048], owners
                             U[0, 16) per block, every block its own allocation
                             with stride = rows rounded up to 16 + U[0, 7];
                             values are random bit patterns
  transposed_c128_8192       complex<double> 8192 x 8192; block-cyclic 64x64 on
                             4x4 into block-cyclic 96x200 on 8x2, op 'T';
                             random bit patterns
  uneven_batch               n independent redistributions: m, n log-uniform in
                             [64, 8192], dtype uniform over float / double /
                             complex<float>, 4-64 virtual ranks, each side a
                             random block-cyclic or random-split layout
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import capi
from . import layouts as Ls


@dataclass
class Workload:
    name: str
    inits: list
    finals: list
    ops: list | None
    values: str = "random"          # "random" bits or "index" (i + j*m)
    meta: dict = field(default_factory=dict)

    @property
    def bytes_moved(self) -> int:
        return sum(L.m * L.n * L.esz for L in self.finals)

    def dtypes(self):
        return [L.dtype for L in self.inits]


def block_cyclic_f64_4096(m: int = 4096) -> Workload:
    Li = Ls.scalapack_layout(m, m, 32, 32, 2, 2, capi.FLOAT64)
    Lf = Ls.scalapack_layout(m, m, 128, 64, 2, 2, capi.FLOAT64)
    return Workload(f"block_cyclic_f64_{m}", [Li], [Lf], None, values="index",
                    meta={"m": m, "n": m, "dtype": "float64",
                          "initial": "block-cyclic 32x32 on 2x2",
                          "final": "block-cyclic 128x64 on 2x2", "ranks": 4})


def random_grid_f32_16384(m: int = 16384, seed: int = 2024, P: int = 16) -> Workload:
    rng = np.random.default_rng(seed)
    Li = Ls.random_grid_layout(m, m, P, capi.FLOAT32, rng)
    Lf = Ls.random_grid_layout(m, m, P, capi.FLOAT32, rng)
    return Workload(f"random_grid_f32_{m}", [Li], [Lf], None,
                    meta={"m": m, "n": m, "dtype": "float32", "ranks": P, "seed": seed,
                          "initial": "random splits U[1,2048], random owners, padded strides",
                          "final": "random splits U[1,2048], random owners, padded strides"})


def transposed_c128_8192(m: int = 8192) -> Workload:
    Li = Ls.scalapack_layout(m, m, 64, 64, 4, 4, capi.COMPLEX128)
    Lf = Ls.scalapack_layout(m, m, 96, 200, 8, 2, capi.COMPLEX128)
    return Workload(f"transposed_c128_{m}", [Li], [Lf], [("T", 1.0, 0.0)],
                    meta={"m": m, "n": m, "dtype": "complex128", "op": "T",
                          "initial": "block-cyclic 64x64 on 4x4",
                          "final": "block-cyclic 96x200 on 8x2", "ranks": 16})


def transposed_random_grid_f32_16384(m: int = 16384, seed: int = 2024, P: int = 16) -> Workload:
    """The random grids of the arbitrary-grid configuration with op 'T' (the
    wide transposed tiles of 4-byte elements)."""
    rng = np.random.default_rng(seed)
    Li = Ls.random_grid_layout(m, m, P, capi.FLOAT32, rng)
    Lf = Ls.random_grid_layout(m, m, P, capi.FLOAT32, rng)
    return Workload(f"transposed_random_grid_f32_{m}", [Li], [Lf], [("T", 1.0, 0.0)],
                    meta={"m": m, "n": m, "dtype": "float32", "ranks": P, "seed": seed,
                          "op": "T",
                          "initial": "random splits U[1,2048], random owners, padded strides",
                          "final": "random splits U[1,2048], random owners, padded strides"})


def transposed_random_grid_f64_16384(m: int = 16384, seed: int = 2024, P: int = 16) -> Workload:
    """The same random grids in double with op 'T' (the tall transposed tiles
    of 8-byte elements)."""
    rng = np.random.default_rng(seed)
    Li = Ls.random_grid_layout(m, m, P, capi.FLOAT64, rng)
    Lf = Ls.random_grid_layout(m, m, P, capi.FLOAT64, rng)
    return Workload(f"transposed_random_grid_f64_{m}", [Li], [Lf], [("T", 1.0, 0.0)],
                    meta={"m": m, "n": m, "dtype": "float64", "ranks": P, "seed": seed,
                          "op": "T",
                          "initial": "random splits U[1,2048], random owners, padded strides",
                          "final": "random splits U[1,2048], random owners, padded strides"})


def _factor_grid(P: int, rng) -> tuple[int, int]:
    divs = [d for d in range(1, P + 1) if P % d == 0]
    pr = int(rng.choice(divs))
    return pr, P // pr


def _random_side(m, n, P, dt, rng):
    if rng.random() < 0.5:
        mb = int(round(math.exp(rng.uniform(math.log(16), math.log(512)))))
        nb = int(round(math.exp(rng.uniform(math.log(16), math.log(512)))))
        pr, pc = _factor_grid(P, rng)
        return Ls.scalapack_layout(m, n, mb, nb, pr, pc, dt, row_major=bool(rng.random() < 0.5))
    hi_r = max(1, min(2048, m // 2))
    return Ls.random_grid_layout(m, n, P, dt, rng, ext_lo=1, ext_hi=hi_r,
                                 pad_max=7)


def uneven_batch(n: int = 256, seed: int = 4, lo: int = 64, hi: int = 8192,
                 dtypes=(capi.FLOAT32, capi.FLOAT64, capi.COMPLEX64)) -> Workload:
    rng = np.random.default_rng(seed)
    inits, finals = [], []
    for _ in range(n):
        m = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        k = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        dt = int(rng.choice(dtypes))
        P = int(rng.integers(4, 65))
        inits.append(_random_side(m, k, P, dt, rng))
        finals.append(_random_side(m, k, P, dt, rng))
    return Workload(f"uneven_batch_{n}", inits, finals, None,
                    meta={"transforms": n, "m_n": f"log-uniform [{lo}, {hi}]",
                          "dtypes": "float32/float64/complex64", "ranks": "U[4, 64]",
                          "seed": seed})


def fill_arenas(w: Workload, seed: int = 7):
    """Host arenas (numpy uint8) for every initial and final layout."""
    rng = np.random.default_rng(seed)
    ia, fa = [], []
    for L in w.inits:
        a = np.zeros(L.arena_bytes, np.uint8)
        if w.values == "index":
            Ls.fill_index_values(L, a)
        else:
            Ls.fill_random(a, rng)
        ia.append(a)
    for L in w.finals:
        a = np.zeros(L.arena_bytes, np.uint8)
        if w.values != "index":
            Ls.fill_random(a, rng)
        fa.append(a)
    return ia, fa


def _column_sectors(L, fills: bool):
    """32-byte sectors spanned by every stored column of every block of L;
    with `fills`, also the sectors a column covers only in part where the
    rest is not the neighbouring column of the same block (padding, another
    block): writing such a sector makes L2 fetch the rest from DRAM."""
    esz = L.esz
    spanned = partial = 0
    rs, cs = L.rows_split, L.cols_split
    for b in range(L.n_blocks):
        i, j = int(L.blocks["row"][b]), int(L.blocks["col"][b])
        h, w = int(rs[i + 1] - rs[i]), int(cs[j + 1] - cs[j])
        if L.blocks["trans"][b]:
            h, w = w, h
        if h == 0 or w == 0:
            continue
        st = int(L.blocks["stride"][b])
        starts = int(L.offsets[b]) + np.arange(w, dtype=np.int64) * st * esz
        ends = starts + h * esz
        first, last = starts // 32, (ends - 1) // 32
        spanned += int((last - first + 1).sum())
        if fills:
            ps, pe = starts % 32 != 0, ends % 32 != 0
            if st == h:  # columns back to back: inner boundaries meet
                ps[1:] = False
                pe[:-1] = False
            n = ps.astype(np.int64) + pe.astype(np.int64) - ((first == last) & ps & pe)
            partial += int(n.sum())
    return spanned * 32, partial * 32


def sector_traffic(w: Workload) -> dict:
    """DRAM bytes any gather-scatter of the workload moves at least: the
    sectors of every source column read once, of every destination column
    written once, and one sector read per partial destination sector whose
    other bytes are not written by the transform (padding, a neighbouring
    block); with the algorithmic 2 x bytes moved for comparison. Offsets
    are arena offsets from 256-byte aligned arena bases."""
    rd = wr = fill = 0
    for Li, Lf in zip(w.inits, w.finals):
        rd += _column_sectors(Li, False)[0]
        a, f = _column_sectors(Lf, True)
        wr += a
        fill += f
    return {"read": rd, "write": wr, "fill": fill, "total": rd + wr + fill,
            "algorithmic": 2 * w.bytes_moved}


BY_NAME = {
    "block_cyclic_f64_4096": block_cyclic_f64_4096,
    "random_grid_f32_16384": random_grid_f32_16384,
    "transposed_c128_8192": transposed_c128_8192,
    "transposed_random_grid_f32_16384": transposed_random_grid_f32_16384,
    "transposed_random_grid_f64_16384": transposed_random_grid_f64_16384,
    "uneven_batch_256": uneven_batch,
    "uneven_batch_64": lambda: uneven_batch(64),
}
