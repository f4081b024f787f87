"""Writes the oracle's digests of whole piece pipelines too slow to rerun on
every GPU test: one SHA-256 per array of every node of the piece tree
(leaves with their discs, inner nodes without), plus the digest of the input
field, into tests/golden/<name>.json.

The oracle is the CPU restatement of the reference's GridDataManager
(dmsc/src/grid_datamanager.cpp:596-662); the inputs come from integer-only
generators (numpy PCG64 floats), so they are the same bytes on every
platform.  Run from the repository root:

    python tests/golden/make_digests.py            # every case
    python tests/golden/make_digests.py noise4096  # one case
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

GRAPH_KEYS = ("rect_ext", "cellid", "fn", "pair_idx", "flags", "asc_off", "asc", "des_off", "des")
LEAF_KEYS = GRAPH_KEYS + ("adisc_off", "adisc", "ddisc_off", "ddisc")

# name -> (field generator, levels, tresh, split2d)
CASES = {
    "noise4096": (lambda: __import__("mscomplex_gb300.synth", fromlist=["noise"]).noise(4096, seed=2), 4, 0.0, True),
}


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def node_digests(node: dict, leaf: bool) -> dict:
    return {k: digest(node[k]) for k in (LEAF_KEYS if leaf else GRAPH_KEYS)}


def make(name: str) -> dict:
    from oracle import oracle as O
    gen, levels, tresh, split2d = CASES[name]
    f = gen()
    t0 = time.time()
    p = O.Pipeline(f, levels=levels, tresh=tresh, split2d=split2d)
    n = p.nleaves
    nodes = [node_digests(p.piece(i), i < n) for i in range(2 * n - 1)]
    return dict(field=digest(f), shape=list(f.shape), levels=levels, tresh=tresh, split2d=split2d, leaves=n,
                nodes=nodes, oracle_seconds=round(time.time() - t0, 1))


if __name__ == "__main__":
    for name in sys.argv[1:] or list(CASES):
        out = make(name)
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), name + ".json")
        with open(path, "w") as fh:
            json.dump(out, fh, indent=0)
        print(f"{name}: {out['leaves']} leaves, {len(out['nodes'])} nodes, oracle {out['oracle_seconds']} s -> {path}")
