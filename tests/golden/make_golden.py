"""Regenerate oracle_glvl2.npz: the CPU oracle's state after start-up and two
steps on the level-2 grid (nvl 38, ntra 5, dt 400 s, seed 1000).

This fixture pins the oracle against unintended changes (a regression check);
it is not a reference pin -- the reference ships no vectors for this path.
A deterministic sample (every 5th element) of each field is stored.
Run from the repository root: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]

from helpers import make_case, oracle_for  # noqa: E402

FIELDS = ["us3d", "vs3d", "dp3d", "pr3d", "ex3d", "ph3d", "mp3d", "tr3d", "trdp", "ws3d", "relvor", "sdot"]


def compute():
    grid, cfg, fields = make_case(glvl=2, nvl=38, ntra=5, dt=400.0, seed=1000, noise=1.0)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    budgets = []
    for its in (1, 2):
        q, b = o.step(s, its)
        budgets.append([b["qmass"]] + list(q))
    out = {k: s[k][::5].copy() for k in FIELDS}
    out["budgets"] = np.array(budgets)
    return out


if __name__ == "__main__":
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_glvl2.npz"), **compute())
