"""Full-size parity against the oracle for the headline workloads.

* The 4096² quantised step (gradient, critical cells, owners, connectivity and
  discs of the whole grid; GridDataset::work, writeout_connectivity and
  postMergeFillDiscs, dmsc/src/grid_dataset.cpp:1044-1231, 1734-1907): every
  cell's flag, pair and owner, the critical list in order, the complex with
  its values (float bits) and arcs with multiplicity, and every disc, against
  the oracle run on the same field.
* The 16384² white-noise piece pipeline (1024² blocks): eight of its 256
  leaves -- the four corners, two edges, two interior -- each against the
  oracle's GridDataset on the same rect / ext window: the leaf's cells and
  critical list as the pipeline computed them, and the leaf's complex.
* The 4096² quantised field's persistence cancellation at 1% of the range
  (GridMSComplex::simplify_un_simplify, dmsc/src/grid_mscomplex.cpp:384-535)
  run to completion on its 1024² corner window: about 2*10^7 exact heap
  operations and 3*10^4 cancellations, the simplified complex and its discs
  against the oracle's.
* The 4096² white-noise pipeline in 16 blocks of 1024² (2D splits, threshold
  0), node by node, against digests of the oracle's pipeline committed under
  tests/golden/ (the oracle needs several minutes for it; the script that
  wrote them is tests/golden/make_digests.py).
"""
import hashlib
import json
import os

import numpy as np
import pytest

from helpers import assert_same_complex, full_rect

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GRAPH_KEYS = ("rect_ext", "cellid", "fn", "pair_idx", "flags", "asc_off", "asc", "des_off", "des")


def same_cells(got, want, what):
    for name, a, b in zip(("flags", "pairs", "own"), got, want):
        assert a.shape == b.shape, f"{what}: {name} shape {a.shape} != {b.shape}"
        if not np.array_equal(a, b):
            bad = np.argwhere(a != b)[:5]
            raise AssertionError(f"{what}: {name} differs at {bad.tolist()}")


def test_simplify_4096_quantised_window_to_completion(gpu_lib, oracle):
    from mscomplex_gb300 import synth
    f = np.ascontiguousarray(synth.bumps4096q()[:1024, :1024])
    r = full_rect(f)
    ds = gpu_lib.GridDataset(r, r).init(f).work()
    m = ds.writeout_connectivity()
    m.simplify_un_simplify(0.01)
    st = m.simplify_stats()
    assert st["pops"] + st["pushes"] > 10_000_000, st
    ds.post_merge_fill_discs(m)
    got = m.export()
    del m, ds
    want = oracle.Dataset(f, r, r, 0.01, True).msc()
    assert_same_complex(got, want, "4096q 1024^2 window at 1%")


def test_step_4096_quantised_vs_oracle(gpu_lib, oracle):
    from mscomplex_gb300 import synth
    f = synth.bumps4096q()
    r = full_rect(f)
    ds = gpu_lib.GridDataset(r, r).init(f).work()
    m = ds.writeout_connectivity()
    ds.post_merge_fill_discs(m)
    got = m.export()
    got_cells = ds.cells()
    got_crit = ds.critical_cells()
    del m, ds
    want_ds = oracle.Dataset(f, r, r, 0.0, True)
    same_cells(got_cells, want_ds.cells(), "4096q step")
    del got_cells
    want = want_ds.msc()
    del want_ds
    assert np.array_equal(got_crit, want["cellid"]), "4096q step: critical list or its order differs"
    assert_same_complex(got, want, "4096q step")


# leaf index bits from the top: y split, x split, ... (bottom / left half first)
C3_LEAVES = {0: "corner (0,0)", 85: "corner (15,0)", 170: "corner (0,15)", 255: "corner (15,15)",
             21: "edge (7,0)", 128: "edge (0,8)", 149: "interior (7,8)", 106: "interior (8,7)"}


def test_pipeline_16384_noise_leaves_vs_oracle(gpu_lib, oracle):
    import torch
    from mscomplex_gb300 import synth
    f = synth.noise(16384, seed=2)
    t = torch.from_numpy(f).cuda()
    p = gpu_lib.GridDataManager(t, levels=8, tresh=0.0, split2d=True)
    assert p.num_pieces == 256
    for i, where in C3_LEAVES.items():
        ds = p.leaf_dataset(i)
        rect, ext = ds.rect.astype(int), ds.ext.astype(int)
        what = f"16384 noise leaf {i} ({where}, rect {rect.tolist()})"
        window = f[ext[1] // 2:ext[3] // 2 + 1, ext[0] // 2:ext[2] // 2 + 1]
        want_ds = oracle.Dataset(window, rect, ext, 0.0, False)
        same_cells(ds.cells(), want_ds.cells(), what)
        want = want_ds.msc()
        del want_ds
        assert np.array_equal(ds.critical_cells(), want["cellid"]), f"{what}: critical list differs"
        # the leaf's own complex (before any merge), recomputed on the same window
        fresh = gpu_lib.GridDataset(rect, ext).init(window).work()
        assert_same_complex(fresh.writeout_connectivity().export(), want, what, keys=GRAPH_KEYS)
        del fresh, want
    del p, t


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_pipeline_4096_noise_vs_oracle_digests(gpu_lib):
    from mscomplex_gb300 import synth
    with open(os.path.join(GOLDEN, "noise4096.json")) as fh:
        gold = json.load(fh)
    f = synth.noise(4096, seed=2)
    assert _digest(f) == gold["field"], "the generated field is not the one the digests were made from"
    p = gpu_lib.GridDataManager(f, levels=gold["levels"], tresh=gold["tresh"], split2d=gold["split2d"])
    n = p.num_pieces
    assert n == gold["leaves"] == 16
    for i, want in enumerate(gold["nodes"]):
        got = p.piece(i).export()
        for k, h in want.items():
            assert _digest(got[k]) == h, f"noise4096 node {i} ({'leaf' if i < n else 'merge'}): {k} differs"
