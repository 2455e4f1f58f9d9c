"""Shared helpers for the tests: golden fixtures, running the GPU path through
the C ABI on device arenas, running the oracle, comparing arenas."""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

from grid2grid_gb300 import capi
from grid2grid_gb300 import layouts as Ls

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def layout_from_arrays(arrays, prefix, meta) -> Ls.Layout:
    blocks = arrays[f"{prefix}.blocks"]
    L = Ls.Layout(arrays[f"{prefix}.rows_split"], arrays[f"{prefix}.cols_split"],
                  arrays[f"{prefix}.owners"], meta["n_ranks"], meta["dtype"],
                  blocks["rank"], blocks["row"], blocks["col"],
                  arrays[f"{prefix}.offsets"], blocks["stride"], meta["arena_bytes"],
                  block_trans=blocks["trans"], block_conj=blocks["conj"],
                  reordering=arrays.get(f"{prefix}.reordering") if meta["reordered"] else None)
    return L


class Golden:
    """The reference's own outputs, generated by tests/golden/make_golden.py."""

    def __init__(self):
        with open(os.path.join(GOLDEN, "transforms.json")) as f:
            self.meta = json.load(f)
        npz = np.load(os.path.join(GOLDEN, "transforms.npz"))
        self.arrays = {k: npz[k] for k in npz.files}
        with open(os.path.join(GOLDEN, "covers.json")) as f:
            self.covers = json.load(f)
        with open(os.path.join(GOLDEN, "scalapack_layouts.json")) as f:
            self.scalapack = json.load(f)

    def cases(self):
        for idx, c in enumerate(self.meta["cases"]):
            inits, finals, ia, fb, fa, ops = [], [], [], [], [], []
            for k, p in enumerate(c["pairs"]):
                inits.append(layout_from_arrays(self.arrays, f"c{idx}.p{k}.i", p["init"]))
                finals.append(layout_from_arrays(self.arrays, f"c{idx}.p{k}.f", p["final"]))
                ia.append(self.arrays[f"c{idx}.p{k}.init_arena"])
                fb.append(self.arrays[f"c{idx}.p{k}.final_before"])
                fa.append(self.arrays[f"c{idx}.p{k}.final_after"])
                if p["op"] is not None:
                    t, ar, ai, br, bi = p["op"]
                    ops.append((t, complex(ar, ai), complex(br, bi)))
            yield {"name": c["name"], "mode": c["mode"], "inits": inits, "finals": finals,
                   "init_arenas": ia, "final_before": fb, "final_after": fa,
                   "ops": ops if ops else None}


def make_ops(ops, n):
    if ops is None:
        return None
    arr = (capi.Op * n)()
    for k, o in enumerate(ops):
        arr[k] = o if isinstance(o, capi.Op) else capi.make_op(*o)
    return arr


def descs(layouts, bases):
    arr = (capi.LayoutDesc * len(layouts))()
    keep = []
    for k, (L, b) in enumerate(zip(layouts, bases)):
        d, kk = L.desc(int(b))
        arr[k] = d
        keep.append(kk)
    return arr, keep


def to_device(arenas):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arenas]


def gpu_run(inits, finals, init_arenas, final_arenas, ops=None, how="transform",
            tuning=None, executes=1, stream=None):
    """Runs the GPU path through the C ABI on device copies of the arenas and
    returns the final arenas (host numpy). how: transform | batch | plan |
    graph."""
    import torch
    lib = capi.load()
    di = to_device(init_arenas)
    df = to_device(final_arenas)
    dI, k1 = descs(inits, [t.data_ptr() for t in di])
    dF, k2 = descs(finals, [t.data_ptr() for t in df])
    n = len(inits)
    dts = (C.c_int * n)(*[L.dtype for L in inits])
    opa = make_ops(ops, n)
    if stream is None:
        # graph capture needs a real (non-legacy-default) stream
        stream = torch.cuda.Stream() if how == "graph" else torch.cuda.current_stream()
    s = stream
    sp = C.c_void_p(s.cuda_stream)
    if how == "transform":
        assert n == 1
        capi.check(lib.g2g_transform(dI, dF, inits[0].dtype, opa, sp))
    elif how == "batch":
        capi.check(lib.g2g_transform_batch(n, dI, dF, dts, opa, sp))
    else:
        plan = C.c_void_p()
        capi.check(lib.g2g_plan_create_batch(n, dI, dF, dts, opa, sp, C.byref(plan)))
        try:
            if tuning is not None:
                t = capi.Tuning()
                for k, v in tuning.items():
                    setattr(t, k, v)
                capi.check(lib.g2g_plan_set_tuning(plan, C.byref(t)))
            if how == "graph":
                capi.check(lib.g2g_plan_capture_graph(plan, sp))
            for _ in range(executes):
                capi.check(lib.g2g_plan_execute(plan, sp))
            s.synchronize()
        finally:
            capi.check(lib.g2g_plan_destroy(plan))
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in df]


def port_run(inits, finals, init_arenas, final_arenas, ops=None, threads=4):
    import oracle
    fa = [np.array(a, copy=True) for a in final_arenas]
    ia = [np.array(a, copy=True) for a in init_arenas]
    oracle.port_transform(inits, finals, ia, fa, ops, threads=threads)
    return fa


def assert_arenas_equal(got, want, L=None, nan_equivalent=False, what=""):
    """Bit-exact comparison of two byte arenas (padding included). With
    nan_equivalent, elements that are NaN in both are accepted whatever
    their payload (only for alpha/beta arithmetic)."""
    got = np.asarray(got)
    want = np.asarray(want)
    assert got.shape == want.shape, what
    diff = np.nonzero(got != want)[0]
    if len(diff) == 0:
        return
    if nan_equivalent and L is not None:
        comp = 8 if L.dtype in (capi.FLOAT64, capi.COMPLEX128) else 4
        ft = np.float64 if comp == 8 else np.float32
        words = np.unique(diff // comp)
        g = got[: got.size // comp * comp].view(ft)[words]
        w = want[: want.size // comp * comp].view(ft)[words]
        if np.all(np.isnan(g) & np.isnan(w)):
            return
    raise AssertionError(
        f"{what}: {len(diff)} bytes differ, first at byte {diff[0]} "
        f"(got {got[diff[0]]}, want {want[diff[0]]})")


def cantor(i, j):
    """The reference example's test values (cantor_mapping.hpp:14-17)."""
    s = i + j
    return (s * (s + 1)) // 2 + j
