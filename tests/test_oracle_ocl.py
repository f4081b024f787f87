"""The oracle's OpenCL-path modes (CPU only).

The reference's OpenCL backend (GridDataset::work_ocl,
dmsc/src/grid_dataset.cpp:353-1022, with dmsc/resources/assigngradient.cl,
collate_critpts.cl and bfs_watershed.cl) differs from its CPU path in
compareCells, which sorts a cell's vertices descending (assigngradient.cl:
40-87).  The oracle restates work_ocl kernel by kernel (MODE_OCL) and also
offers the CPU path with only the comparator changed (MODE_CPU_DESC).  These
tests pin the descending comparator on a hand-traced case and check that the
literal restatement and the one-switch variant agree on every output.
"""
import numpy as np
import pytest

from helpers import check_gradient_properties, tie_field


def test_descending_comparator_known_answer(oracle):
    """3x3 grid, rows y = 0..2:  [1 3 6] / [0 7 4] / [5 8 2].  The vertical
    edge (2,3) joins values 7 (vertex (1,1)) and 8 (vertex (1,2)); it is the
    largest edge of both its faces in either order.  Ascending sort: left face
    (1,3) = [0 5 7 8] < right face (3,3) = [2 4 7 8] (0 < 2), so the edge
    pairs left and (3,3) stays critical.  Descending sort: [8 7 4 2] < [8 7 5 0]
    (4 < 5), so it pairs right and (1,3) stays critical."""
    f = np.array([[1, 3, 6], [0, 7, 4], [5, 8, 2]], np.float32)
    r = (0, 0, 4, 4)
    for mode, face, crit in ((oracle.MODE_CPU, (1, 3), (3, 3)), (oracle.MODE_CPU_DESC, (3, 3), (1, 3)),
                             (oracle.MODE_OCL, (3, 3), (1, 3))):
        flags, pairs, _ = oracle.Dataset(f, r, r, mode=mode).cells()
        assert pairs[2, 3].tolist() == list(face), (mode, pairs[2, 3])
        assert pairs[face].tolist() == [2, 3]
        assert flags[crit] == 2 and flags[face] == 1 and flags[2, 3] == 1


def _cases(n, seed):
    rng = np.random.default_rng(seed)
    for t in range(n):
        ny, nx = int(rng.integers(2, 16)), int(rng.integers(2, 16))
        if t % 2:
            f = tie_field(ny, nx, int(rng.integers(2, 6)), t)
        else:
            f = rng.random((ny, nx)).astype(np.float32)
        r = (0, 0, 2 * (nx - 1), 2 * (ny - 1))
        yield f, r, r
        if ny > 4:  # a piece below a split: one halo row above its rect
            yield f[:ny - 1], (0, 0, 2 * (nx - 1), 2 * (ny - 3)), (0, 0, 2 * (nx - 1), 2 * (ny - 2))
        if nx > 4:  # a piece right of a split: one halo column on its left
            yield f[:, 1:], (2, 0, 2 * (nx - 2), 2 * (ny - 1)), (0, 0, 2 * (nx - 2), 2 * (ny - 1))


def test_literal_work_ocl_equals_cpu_path_with_descending_sort(oracle):
    """work_ocl's kernels (assign_gradient, complete_pairings, the two
    boundary-pair kernels, pointer-jumping owners, saddle incidences) give the
    CPU path's cells, critical list, owners and complex once compareCells
    sorts descending; and that order does change the gradient."""
    differ = 0
    for i, (f, r, e) in enumerate(_cases(150, 7)):
        lit = oracle.Dataset(f, r, e, mode=oracle.MODE_OCL)
        one = oracle.Dataset(f, r, e, mode=oracle.MODE_CPU_DESC)
        for name, a, b in zip(("flags", "pairs", "own"), lit.cells(), one.cells()):
            assert np.array_equal(a, b), f"case {i}: {name} differs"
        ma, mb = lit.msc(), one.msc()
        for k in ma:
            assert np.array_equal(ma[k], mb[k]), f"case {i}: complex {k} differs"
        cpu = oracle.Dataset(f, r, e)
        differ += not np.array_equal(cpu.cells()[1], one.cells()[1])
    assert differ > 20


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_descending_gradient_properties(oracle, seed):
    rng = np.random.default_rng(seed)
    f = tie_field(23, 31, 4, seed) if seed else rng.random((40, 37)).astype(np.float32)
    ny, nx = f.shape
    r = (0, 0, 2 * (nx - 1), 2 * (ny - 1))
    d = oracle.Dataset(f, r, r, mode=oracle.MODE_OCL)
    assert d.overwrites() == 0
    flags, pairs, own = d.cells()
    check_gradient_properties(flags, pairs, own, r)
    m = d.msc()
    dim = (m["cellid"][:, 0] & 1) + (m["cellid"][:, 1] & 1)
    assert int((dim == 0).sum()) - int((dim == 1).sum()) + int((dim == 2).sum()) == 1


def test_ocl_pipeline_runs_and_differs(oracle):
    """On white noise (faces whose vertex orders the two sorts rank apart are
    common; on smooth fields they are rare) the -ocl pipeline differs."""
    from mscomplex_gb300 import synth
    f = synth.noise(64, seed=3)
    a = oracle.Pipeline(f, levels=2, tresh=0.02, split2d=True, ocl=True)
    b = oracle.Pipeline(f, levels=2, tresh=0.02, split2d=True)
    root_a, root_b = a.piece(2 * a.nleaves - 2), b.piece(2 * b.nleaves - 2)
    assert not all(np.array_equal(root_a[k], root_b[k]) for k in ("cellid", "asc", "des"))
