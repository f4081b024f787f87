"""GPU parity of the OpenCL-semantics path (GridDataset::work_ocl +
writeout_connectivity_ocl, dmsc/src/grid_dataset.cpp:353-1022, 1250-1283;
compareCells with the cell's vertices sorted descending,
dmsc/resources/assigngradient.cl:40-87) against the oracle's kernel-by-kernel
restatement of that path, through the C ABI: cells, critical list, owners and
complex of single pieces (with and without a halo), and the -ocl piece
pipeline node by node."""
import numpy as np
import pytest

from helpers import assert_same_complex, full_rect, smooth_field, tie_field

pytestmark = pytest.mark.gpu


def run_ocl(M, oracle, field, rect, ext, what):
    e = np.asarray(ext)
    win = np.ascontiguousarray(field[e[1] // 2:e[3] // 2 + 1, e[0] // 2:e[2] // 2 + 1])
    ods = oracle.Dataset(win, rect, ext, mode=oracle.MODE_OCL)
    gds = M.GridDataset(rect, ext).init(win).work_ocl()
    for name, a, b in zip(("flags", "pairs", "own"), gds.cells(), ods.cells()):
        if not np.array_equal(a, b):
            bad = np.argwhere(a != b)[:5]
            raise AssertionError(f"{what}: {name} differs at {bad.tolist()}")
    om = ods.msc()
    assert np.array_equal(gds.critical_cells(), om["cellid"]), f"{what}: critical list differs"
    assert_same_complex(gds.writeout_connectivity_ocl().export(), om, what)
    assert_same_complex(gds.writeout_connectivity().export(), om, what + " (writeout_connectivity)")
    return gds


@pytest.mark.parametrize("shape", [(2, 2), (3, 3), (2, 9), (7, 2), (5, 17), (64, 64), (65, 66), (130, 63), (200, 150)])
@pytest.mark.parametrize("kind", ["noise", "ties", "smooth"])
def test_work_ocl_single_piece(gpu_lib, oracle, shape, kind):
    ny, nx = shape
    seed = 7 * ny + nx
    if kind == "noise":
        f = np.random.default_rng(seed).random((ny, nx)).astype(np.float32)
    elif kind == "ties":
        f = tie_field(ny, nx, 4, seed)
    else:
        f = smooth_field(ny, nx, seed)
    r = full_rect(f)
    run_ocl(gpu_lib, oracle, f, r, r, f"ocl {kind} {shape}")


def test_work_ocl_known_answer(gpu_lib, oracle):
    """The hand-traced case of the oracle's tests: edge (2,3) pairs with the
    right face (3,3) under the descending sort and the left face (1,3) under
    the ascending one."""
    f = np.array([[1, 3, 6], [0, 7, 4], [5, 8, 2]], np.float32)
    r = full_rect(f)
    g = run_ocl(gpu_lib, oracle, f, r, r, "ocl KAT")
    assert g.cells()[1][2, 3].tolist() == [3, 3]
    cpu = gpu_lib.GridDataset(r, r).init(f).work()
    assert cpu.cells()[1][2, 3].tolist() == [1, 3]


def test_work_ocl_many_tiny(gpu_lib, oracle):
    rng = np.random.default_rng(99)
    for t in range(120):
        ny, nx = (int(v) for v in rng.integers(2, 8, size=2))
        f = rng.permutation(nx * ny).astype(np.float32).reshape(ny, nx) if t % 2 else \
            rng.integers(0, 3, size=(ny, nx)).astype(np.float32)
        r = full_rect(f)
        run_ocl(gpu_lib, oracle, f, r, r, f"ocl tiny #{t}")


@pytest.mark.parametrize("split", ["below", "above", "left", "right"])
def test_work_ocl_piece_with_halo(gpu_lib, oracle, split):
    """Pieces of a split grid: rect plus a one-vertex halo on the split side
    (the boundary-pair kernels mark cells paired across it)."""
    f = np.random.default_rng(5).random((70, 90)).astype(np.float32)
    X, Y = 2 * 89, 2 * 69
    if split == "below":
        r, e = (0, 0, X, 68), (0, 0, X, 70)
    elif split == "above":
        r, e = (0, 68, X, Y), (0, 66, X, Y)
    elif split == "left":
        r, e = (0, 0, 88, Y), (0, 0, 90, Y)
    else:
        r, e = (88, 0, X, Y), (86, 0, X, Y)
    run_ocl(gpu_lib, oracle, f, r, e, f"ocl halo {split}")


@pytest.mark.parametrize("levels,split2d,tresh", [(1, False, 0.0), (2, True, 0.02), (3, True, 0.05)])
def test_ocl_pipeline(gpu_lib, oracle, levels, split2d, tresh):
    from mscomplex_gb300 import synth
    f = synth.noise(96, seed=11)
    want = oracle.Pipeline(f, levels=levels, tresh=tresh, split2d=split2d, ocl=True)
    ctx = gpu_lib.Context()
    ctx.set_use_ocl(True)
    got = gpu_lib.GridDataManager(f, levels=levels, tresh=tresh, split2d=split2d, ctx=ctx)
    N = got.num_pieces
    assert N == want.nleaves
    for i in range(2 * N - 1):
        keys = None if i < N else ("rect_ext", "cellid", "fn", "pair_idx", "flags", "asc_off", "asc", "des_off", "des")
        assert_same_complex(got.piece(i).export(), want.piece(i), f"ocl pipeline L{levels} node {i}", keys=keys)
    del got
    ctx.close()
