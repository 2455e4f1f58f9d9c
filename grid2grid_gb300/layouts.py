"""Host-side layout descriptions over P virtual ranks.

A ``Layout`` is the Python mirror of the reference's ``grid_layout<T>``
(src/grid2grid/grid_layout.hpp:7-63) for ALL virtual ranks at once: the grid
(``grid2D``: rows_split / cols_split, grid2D.hpp:17-39), the owner matrix with
optional rank reordering (``assigned_grid2D``, grid2D.hpp:46-125) and every
rank's local blocks (``block<T>``: coordinates, pointer, stride, transpose /
conjugate flags, block.hpp:60-146). Block storage is addressed as byte offsets
into one arena per layout, so the same layout can point at device memory (the
GPU path) or at a host copy (the oracle) by changing the arena base.

Builders:
  * ``scalapack_layout``  -- get_scalapack_grid, all four overloads
    (scalapack_layout.cpp:178-346): block-cyclic with optional submatrix,
    rank-grid ordering and source process; one local buffer per rank with
    leading dimension ``lld``.
  * ``random_grid_layout`` -- arbitrary grid-like layout: seeded split points,
    seeded owners, every block its own allocation with a padded stride.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import capi

BLOCK_DTYPE = np.dtype([
    ("rank", np.int32), ("row", np.int32), ("col", np.int32),
    ("trans", np.int32), ("conj", np.int32), ("reserved", np.int32),
    ("stride", np.int64), ("data", np.uint64)])
assert BLOCK_DTYPE.itemsize == C.sizeof(capi.BlockDesc)

ALIGN = 256  # arena placement alignment (that of cudaMalloc)


def _align(x: int, a: int = ALIGN) -> int:
    return (x + a - 1) // a * a


class Layout:
    """A grid layout over ``n_ranks`` virtual ranks with byte-offset blocks."""

    def __init__(self, rows_split, cols_split, owners, n_ranks, dtype,
                 block_rank, block_row, block_col, block_offset, block_stride,
                 arena_bytes, block_trans=None, block_conj=None, reordering=None):
        self.rows_split = np.ascontiguousarray(rows_split, dtype=np.int32)
        self.cols_split = np.ascontiguousarray(cols_split, dtype=np.int32)
        self.owners = np.ascontiguousarray(owners, dtype=np.int32).reshape(
            len(self.rows_split) - 1, len(self.cols_split) - 1)
        self.n_ranks = int(n_ranks)
        self.dtype = int(dtype)
        self.esz = capi.DTYPE_SIZE[self.dtype]
        nb = len(block_rank)
        self.blocks = np.zeros(nb, dtype=BLOCK_DTYPE)
        self.blocks["rank"] = block_rank
        self.blocks["row"] = block_row
        self.blocks["col"] = block_col
        self.blocks["stride"] = block_stride
        self.offsets = np.ascontiguousarray(block_offset, dtype=np.int64)
        if block_trans is not None:
            self.blocks["trans"] = block_trans
        if block_conj is not None:
            self.blocks["conj"] = block_conj
        self.reordering = (None if reordering is None
                           else np.ascontiguousarray(reordering, dtype=np.int32))
        self.arena_bytes = int(arena_bytes)

    # -- geometry ---------------------------------------------------------
    @property
    def m(self) -> int:
        return int(self.rows_split[-1] - self.rows_split[0])

    @property
    def n(self) -> int:
        return int(self.cols_split[-1] - self.cols_split[0])

    @property
    def n_blocks(self) -> int:
        return len(self.blocks)

    def owner(self, i: int, j: int) -> int:
        r = int(self.owners[i, j])
        return r if self.reordering is None else int(self.reordering[r])

    def copy(self) -> "Layout":
        L = Layout.__new__(Layout)
        L.__dict__.update({k: (v.copy() if isinstance(v, np.ndarray) else v)
                           for k, v in self.__dict__.items()})
        return L

    def transpose_or_conjugate(self, flag: str) -> "Layout":
        """grid_layout::transpose_or_conjugate (grid_layout.hpp:18-25), in
        place: 'T'/'C' transpose the grid and the owners and mark every
        block (block.cpp:249-288); 'N' does nothing."""
        flag = flag.upper()
        if flag not in "NTC":
            raise ValueError("flag must be N, T or C")
        if flag == "N":
            return self
        self.rows_split, self.cols_split = self.cols_split, self.rows_split
        self.owners = np.ascontiguousarray(self.owners.T)
        r = self.blocks["row"].copy()
        self.blocks["row"] = self.blocks["col"]
        self.blocks["col"] = r
        self.blocks["trans"] = 1
        if flag == "C":
            self.blocks["conj"] = 1
        return self

    def reorder_ranks(self, reordering) -> "Layout":
        """assigned_grid2D::reorder_ranks (grid2D.cpp:112-114)."""
        self.reordering = np.ascontiguousarray(reordering, dtype=np.int32)
        return self

    def storage_shape(self, b: int):
        """(rows, cols) of block b as stored in memory."""
        i, j = int(self.blocks["row"][b]), int(self.blocks["col"][b])
        nr = int(self.rows_split[i + 1] - self.rows_split[i])
        nc = int(self.cols_split[j + 1] - self.cols_split[j])
        return (nc, nr) if self.blocks["trans"][b] else (nr, nc)

    # -- descriptors --------------------------------------------------------
    def desc(self, base: int):
        """A g2g_layout_desc whose block pointers are ``base + offset``.
        Returns (desc, keepalive); keep both alive while the library runs."""
        blocks = self.blocks.copy()
        blocks["data"] = np.uint64(base) + self.offsets.astype(np.uint64)
        d = capi.LayoutDesc()
        d.n_block_rows = len(self.rows_split) - 1
        d.n_block_cols = len(self.cols_split) - 1
        I32 = C.POINTER(C.c_int32)
        d.rows_split = self.rows_split.ctypes.data_as(I32)
        d.cols_split = self.cols_split.ctypes.data_as(I32)
        own = np.ascontiguousarray(self.owners, dtype=np.int32)
        d.owners = own.ctypes.data_as(I32)
        d.n_ranks = self.n_ranks
        if self.reordering is not None:
            d.n_reordering = len(self.reordering)
            d.reordering = self.reordering.ctypes.data_as(I32)
        d.n_blocks = len(blocks)
        d.blocks = blocks.ctypes.data_as(C.POINTER(capi.BlockDesc))
        return d, (blocks, own, self.rows_split, self.cols_split, self.reordering)

    # -- element access on a host arena (tests) ----------------------------
    def block_view(self, arena: np.ndarray, b: int) -> np.ndarray:
        """Column-major (storage rows x cols) view of block b in a host byte
        arena, as an array of element-sized unsigned integers (or 16-byte
        records)."""
        rows, cols = self.storage_shape(b)
        stride = int(self.blocks["stride"][b])
        off = int(self.offsets[b])
        es = self.esz
        if rows == 0 or cols == 0:
            return np.zeros((rows, cols), dtype=_elem_view_dtype(es))
        nbytes = ((cols - 1) * stride + rows) * es
        raw = arena[off:off + nbytes].view(_elem_view_dtype(es))
        return np.lib.stride_tricks.as_strided(
            raw, shape=(rows, cols), strides=(es, stride * es))

    def gather(self, arena: np.ndarray) -> np.ndarray:
        """The global m x n matrix (element records) held by the layout, in the
        layout's current coordinates."""
        out = np.zeros((self.m, self.n), dtype=_elem_view_dtype(self.esz))
        r0, c0 = int(self.rows_split[0]), int(self.cols_split[0])
        for b in range(self.n_blocks):
            i, j = int(self.blocks["row"][b]), int(self.blocks["col"][b])
            v = self.block_view(arena, b)
            if self.blocks["trans"][b]:
                v = v.T
            out[self.rows_split[i] - r0:self.rows_split[i + 1] - r0,
                self.cols_split[j] - c0:self.cols_split[j + 1] - c0] = v
        return out


def _elem_view_dtype(esz: int):
    return {4: np.uint32, 8: np.uint64, 16: np.dtype((np.void, 16))}[esz]


# ---------------------------------------------------------------- builders
def line_split(begin: int, end: int, blk: int) -> list[int]:
    """Split points of [begin, end) at multiples of blk, relative to begin
    (scalapack_layout.cpp:152-177)."""
    length = end - begin
    rem = blk - begin % blk
    splits = [0]
    if rem >= length:
        splits.append(length)
        return splits
    if rem != 0:
        splits.append(rem)
    for _ in range((length - rem) // blk):
        splits.append(splits[-1] + blk)
    if splits[-1] != length:
        splits.append(length)
    return splits


def rank_from_grid(r: int, c: int, pr: int, pc: int, row_major: bool) -> int:
    """scalapack_layout.cpp:40-57."""
    if not (0 <= r < pr and 0 <= c < pc):
        raise ValueError("rank coordinates do not belong to the rank grid")
    return r * pc + c if row_major else c * pr + r


def rank_to_grid(rank: int, pr: int, pc: int, row_major: bool):
    """scalapack_layout.cpp:10-24."""
    if not 0 <= rank < pr * pc:
        raise ValueError("rank does not belong to the grid")
    return (rank // pc, rank % pc) if row_major else (rank % pr, rank // pr)


def scalapack_local_size(m, n, mb, nb, pr, pc, rank, row_major=False) -> int:
    """scalapack::local_size (scalapack_layout.cpp:141-149): the padded
    local buffer of `rank` in elements."""
    rr, rc = rank_to_grid(rank, pr, pc, row_major)
    nbr = math.ceil(m / mb)
    nbc = math.ceil(n / nb)
    own_r = nbr // pr + (1 if rr < nbr % pr else 0)
    own_c = nbc // pc + (1 if rc < nbc % pc else 0)
    return own_r * own_c * mb * nb


def scalapack_lld(m, mb, pr, pc, rank, row_major=False) -> int:
    """The leading dimension the simple get_scalapack_grid overload uses
    (scalapack_layout.cpp:318-324): local block rows x mb."""
    rr, _ = rank_to_grid(rank, pr, pc, row_major)
    nbr = math.ceil(m / mb)
    return (nbr // pr + (1 if rr < nbr % pr else 0)) * mb


def scalapack_layout(m, n, mb, nb, pr, pc, dtype, row_major=False, *,
                     lld=None, ij=(1, 1), sub=None, src=(0, 0),
                     local_elems=None) -> Layout:
    """get_scalapack_grid for every rank (scalapack_layout.cpp:178-278).

    Rank r's local buffer is placed in the arena at a 256-byte aligned
    offset; ``lld`` (int or per-rank list) defaults to the simple overload's
    local rows. ``ij`` is 1-based as in the reference; ``sub`` is the
    submatrix shape (default: the whole matrix). ``local_elems`` overrides the
    per-rank buffer sizes (default: scalapack::local_size, or what the
    submatrix layout reaches)."""
    P = pr * pc
    esz = capi.DTYPE_SIZE[dtype]
    sm, sn = (m, n) if sub is None else sub
    i0, j0 = ij[0] - 1, ij[1] - 1
    if i0 < 0 or j0 < 0:
        raise ValueError("ij is 1-based")
    rs = line_split(i0, i0 + sm, mb)
    cs = line_split(j0, j0 + sn, nb)
    nbr, nbc = len(rs) - 1, len(cs) - 1
    br0, bc0 = i0 // mb, j0 // nb
    src_r = (br0 % pr + src[0]) % pr
    src_c = (bc0 % pc + src[1]) % pc
    if lld is None:
        llds = [scalapack_lld(m, mb, pr, pc, r, row_major) for r in range(P)]
    elif np.isscalar(lld):
        llds = [int(lld)] * P
    else:
        llds = [int(x) for x in lld]
    owners = np.zeros((nbr, nbc), dtype=np.int32)
    ranks, rows, cols, eoffs = [], [], [], []
    for j in range(nbc):
        rank_col = (j % pc + src_c) % pc
        for i in range(nbr):
            rank_row = (i % pr + src_r) % pr
            o = rank_from_grid(rank_row, rank_col, pr, pc, row_major)
            owners[i, j] = o
            loc_r = (br0 + i) // pr
            loc_c = (bc0 + j) // pc
            sub_r = i0 + rs[i] - (br0 + i) * mb
            sub_c = j0 + cs[j] - (bc0 + j) * nb
            off = loc_r * mb + sub_r + llds[o] * (loc_c * nb + sub_c)
            ranks.append(o); rows.append(i); cols.append(j); eoffs.append(off)
    ranks = np.array(ranks, dtype=np.int32)
    eoffs = np.array(eoffs, dtype=np.int64)
    # per-rank buffer sizes
    if local_elems is None:
        local_elems = []
        for r in range(P):
            sz = scalapack_local_size(m, n, mb, nb, pr, pc, r, row_major) if (
                sub is None and ij == (1, 1) and lld is None) else 0
            mask = ranks == r
            if mask.any():
                # furthest element a local block reaches
                reach = 0
                for k in np.nonzero(mask)[0]:
                    i, j = rows[k], cols[k]
                    h = rs[i + 1] - rs[i]
                    w = cs[j + 1] - cs[j]
                    reach = max(reach, int(eoffs[k]) + (w - 1) * llds[r] + h)
                sz = max(sz, reach)
            local_elems.append(sz)
    rank_base = []
    off = 0
    for r in range(P):
        rank_base.append(off)
        off = _align(off + int(local_elems[r]) * esz)
    arena = max(off, ALIGN)
    byte_offs = np.array([rank_base[r] for r in ranks], dtype=np.int64) + eoffs * esz
    strides = np.array([llds[r] for r in ranks], dtype=np.int64)
    L = Layout(rs, cs, owners, P, dtype, ranks, rows, cols, byte_offs, strides, arena)
    L.rank_base = np.array(rank_base, dtype=np.int64)
    L.local_elems = np.array(local_elems, dtype=np.int64)
    L.lld = np.array(llds, dtype=np.int64)
    return L


def random_splits(total: int, rng: np.random.Generator, lo: int = 1, hi: int = 2048):
    """Split points 0 = s0 < s1 < ... = total with extents drawn U[lo, hi]."""
    s = [0]
    while s[-1] < total:
        s.append(min(total, s[-1] + int(rng.integers(lo, hi + 1))))
    return s


def random_grid_layout(m, n, P, dtype, rng: np.random.Generator, *,
                       ext_lo=1, ext_hi=2048, pad_max=7, row_align=16,
                       base_misalign=0, byte_misalign=0, align=ALIGN) -> Layout:
    """An arbitrary grid-like layout: seeded splits (extents U[ext_lo,
    ext_hi]), owners U[0, P) per block, each block its own allocation with
    stride = rows rounded up to ``row_align`` plus U[0, pad_max], placed at an
    ``align``-byte aligned arena offset (+ ``base_misalign`` elements
    + ``byte_misalign`` bytes)."""
    esz = capi.DTYPE_SIZE[dtype]
    rs = random_splits(m, rng, ext_lo, ext_hi)
    cs = random_splits(n, rng, ext_lo, ext_hi)
    nbr, nbc = len(rs) - 1, len(cs) - 1
    owners = rng.integers(0, P, size=(nbr, nbc)).astype(np.int32)
    ranks, rows, cols, offs, strides = [], [], [], [], []
    off = 0
    for i in range(nbr):
        h = rs[i + 1] - rs[i]
        for j in range(nbc):
            w = cs[j + 1] - cs[j]
            stride = (h + row_align - 1) // row_align * row_align + int(
                rng.integers(0, pad_max + 1))
            ranks.append(int(owners[i, j])); rows.append(i); cols.append(j)
            lead = base_misalign * esz + byte_misalign
            offs.append(off + lead)
            strides.append(stride)
            off = _align(off + lead + stride * w * esz, align)
    return Layout(rs, cs, owners, P, dtype, ranks, rows, cols, offs, strides,
                  max(off, align))


def fill_random(arena: np.ndarray, rng: np.random.Generator) -> np.ndarray:
    """Seeded uniform random bytes (all bit patterns, NaNs included)."""
    arena[:] = rng.integers(0, 256, size=arena.shape, dtype=np.uint8)
    return arena


def fill_index_values(L: Layout, arena: np.ndarray, ld_global: int | None = None):
    """Writes value(i, j) = i + j * m (as the element type) into every block
    of L at its global coordinates; padding is left as it is."""
    m = L.m if ld_global is None else ld_global
    np_t = {capi.FLOAT32: np.float32, capi.FLOAT64: np.float64,
            capi.COMPLEX64: np.complex64, capi.COMPLEX128: np.complex128}[L.dtype]
    for b in range(L.n_blocks):
        i, j = int(L.blocks["row"][b]), int(L.blocks["col"][b])
        r = np.arange(L.rows_split[i], L.rows_split[i + 1], dtype=np.float64)
        c = np.arange(L.cols_split[j], L.cols_split[j + 1], dtype=np.float64)
        vals = (r[:, None] + c[None, :] * m).astype(np_t)
        if L.blocks["trans"][b]:
            vals = vals.T
        v = L.block_view(arena, b)
        v[...] = vals.view(v.dtype).reshape(v.shape) if vals.size else v
