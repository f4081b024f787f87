"""CPU tests of the oracle: hand-derived known-answer cases and structural
properties.  The reference ships no golden vectors, so these cases were
traced by hand through dmsc/src/grid_dataset.cpp (assignGradients :1743,
collateCriticalPoints :1822, track_gradient_tree_bfs :1376,
writeout_connectivity :1858)."""
import numpy as np
import pytest

from helpers import check_gradient_properties, dims_of, full_rect, smooth_field, tie_field


def test_kat_2x2(oracle):
    # field[y][x]; vertex (x,y) is cell (2x,2y)
    f = np.array([[0, 1], [2, 3]], np.float32)
    ds = oracle.Dataset(f, full_rect(f), full_rect(f))
    flags, pairs, own = ds.cells()
    # flags[x][y]: (0,0) min, (1,1) max, (1,2) saddle; all others paired
    want_flags = np.array([[2, 1, 1], [1, 2, 2], [1, 1, 1]], np.int8)
    assert np.array_equal(flags, want_flags)
    assert tuple(pairs[2, 0]) == (1, 0) and tuple(pairs[1, 0]) == (2, 0)
    assert tuple(pairs[0, 2]) == (0, 1) and tuple(pairs[2, 2]) == (2, 1)
    for c in [(0, 0), (1, 0), (2, 0), (0, 1), (2, 1), (0, 2), (2, 2)]:
        assert tuple(own[c]) == (0, 0)
    assert tuple(own[1, 1]) == (1, 1) and tuple(own[1, 2]) == (1, 2)
    m = ds.msc()
    assert m["cellid"].tolist() == [[0, 0], [1, 1], [1, 2]]
    assert m["fn"].tolist() == [0.0, 1.5, 2.5]
    # saddle (1,2) reaches the minimum twice (a strangulation) and the max once
    assert m["des_off"].tolist() == [0, 0, 1, 3] and m["des"].tolist() == [2, 0, 0]
    assert m["asc_off"].tolist() == [0, 2, 2, 3] and m["asc"].tolist() == [2, 2, 1]
    assert ds.overwrites() == 0


def test_kat_ascending_face_order(oracle):
    # Interior edge (1,2) between vertices (0,1)=10 and (1,1)=11 is the max
    # facet of both of its faces; compareCells sorts vertices ASCENDING
    # (grid_dataset.cpp:1530), so the face above ({1,9,10,11}) is lower than
    # the face below ({2,3,10,11}) and the edge pairs upward.  A descending
    # sort would pick the face below.
    f = np.array([[2, 3, 13], [10, 11, 12], [1, 9, 14]], np.float32)
    ds = oracle.Dataset(f, full_rect(f), full_rect(f))
    flags, pairs, own = ds.cells()
    assert tuple(pairs[1, 2]) == (1, 3)
    assert tuple(pairs[1, 3]) == (1, 2)
    assert flags[1, 1] & 2  # face below stays unpaired by this edge


@pytest.mark.parametrize("seed", range(6))
def test_single_piece_properties(oracle, seed):
    rng = np.random.default_rng(seed)
    ny, nx = rng.integers(2, 40, size=2)
    f = tie_field(ny, nx, 3, seed) if seed % 2 else smooth_field(ny, nx, seed)
    r = full_rect(f)
    ds = oracle.Dataset(f, r, r)
    flags, pairs, own = ds.cells()
    check_gradient_properties(flags, pairs, own, r)
    m = ds.msc()
    d = dims_of(m["cellid"])
    assert (d == 0).sum() - (d == 1).sum() + (d == 2).sum() == 1, "Euler characteristic of a disc"
    assert ds.overwrites() == 0


@pytest.mark.parametrize("levels", [1, 2, 3])
def test_pipeline_levels_run(oracle, levels):
    f = tie_field(33, 29, 4, levels)
    P = oracle.Pipeline(f, levels=levels, tresh=0.0)
    assert P.nleaves == 2 ** levels
    assert P.overwrites == 0
    files = P.disc_files()
    assert files, "discs were written"


def test_pipeline_simplify_runs(oracle):
    f = smooth_field(48, 40, 7)
    P = oracle.Pipeline(f, levels=0, tresh=0.05)
    assert P.ncancel > 0
    root = P.root_simplified()
    # every cancelled pair is recorded as boundary-cancelable with mutual pair_idx
    canc = (root["flags"] & 4) != 0
    idx = np.nonzero(canc)[0]
    assert np.all(root["pair_idx"][root["pair_idx"][idx]] == idx)


def test_pipeline_2d_blocks(oracle):
    f = smooth_field(40, 40, 3)
    P = oracle.Pipeline(f, levels=2, tresh=0.0, split2d=True)
    assert P.nleaves == 4
    rects = [P.piece(i)["rect_ext"][:4].tolist() for i in range(4)]
    assert rects[0] != rects[1]
