"""Generates tests/golden/reordering.json: the reference's
communication_volume and optimal_reordering (transform.cpp:9-39,
ranks_reordering.cpp:4-61) on seeded grid pairs, run through the reference
oracle (oracle/_ref, built from the reference checkout). The reference's
volume map gets every rank's self entry before optimal_reordering runs (its
own loop inserts them into the map it iterates; see oracle/ref_driver.cpp).

    python tests/golden/make_reordering_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from grid2grid_gb300 import capi  # noqa: E402
from grid2grid_gb300 import layouts as Ls  # noqa: E402
import oracle  # noqa: E402


def grid_of(L):
    return {"rows_split": L.rows_split.tolist(), "cols_split": L.cols_split.tolist(),
            "owners": L.owners.tolist(),
            "reordering": None if L.reordering is None else L.reordering.tolist()}


def main():
    rng = np.random.default_rng(2026)
    cases = []
    for _ in range(48):
        P = int(rng.integers(2, 13))
        m, n = int(rng.integers(16, 500)), int(rng.integers(16, 500))
        sides = []
        for _side in range(2):
            if rng.random() < 0.5:
                L = Ls.random_grid_layout(m, n, P, capi.FLOAT64, rng, ext_lo=1,
                                          ext_hi=max(1, m // 3))
            else:
                pr = int(rng.integers(1, P + 1))
                pc = max(1, P // pr)
                L = Ls.scalapack_layout(m, n, int(rng.integers(4, 80)),
                                        int(rng.integers(4, 80)), pr, pc, capi.FLOAT64,
                                        bool(rng.integers(0, 2)))
                L.n_ranks = P
            if rng.random() < 0.25:
                L.reorder_ranks(list(rng.permutation(L.n_ranks)))
            sides.append(L)
        vol, perm, re = oracle.ref_comm_volume(sides[0], sides[1], P)
        cases.append({"n_ranks": P, "initial": grid_of(sides[0]), "final": grid_of(sides[1]),
                      "volume": vol.tolist(), "permutation": perm.tolist(),
                      "reordered": re})
    with open(os.path.join(HERE, "reordering.json"), "w") as f:
        json.dump({"cases": cases}, f)
    print(f"wrote {len(cases)} cases")


if __name__ == "__main__":
    main()
