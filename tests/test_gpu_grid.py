"""GPU parity of the grid hot path (gradient, collation, owners, complex)
against the oracle, through the C ABI.  Integer / index outputs are compared
bit-exactly, critical-point values as float32 bit patterns."""
import numpy as np
import pytest

from helpers import assert_same_complex, check_gradient_properties, full_rect, smooth_field, tie_field

pytestmark = pytest.mark.gpu


def run_both(M, oracle, field, rect, ext):
    e = np.asarray(ext)
    win = field[e[1] // 2:e[3] // 2 + 1, e[0] // 2:e[2] // 2 + 1]
    ods = oracle.Dataset(win, rect, ext)
    gds = M.GridDataset(rect, ext).init(win).work()
    return ods, gds


def compare_dataset(ods, gds, what):
    of, op, oo = ods.cells()
    gf, gp, go = gds.cells()
    assert np.array_equal(gf, of), f"{what}: flags differ at {np.argwhere(gf != of)[:5].tolist()}"
    assert np.array_equal(gp, op), f"{what}: pairs differ at {np.argwhere(np.any(gp != op, -1))[:5].tolist()}"
    assert np.array_equal(go, oo), f"{what}: owners differ at {np.argwhere(np.any(go != oo, -1))[:5].tolist()}"
    om = ods.msc()
    assert np.array_equal(gds.critical_cells(), om["cellid"]), f"{what}: critical list differs"
    gm = gds.writeout_connectivity().export()
    assert_same_complex(gm, om, what)


@pytest.mark.parametrize("shape", [(2, 2), (3, 3), (2, 7), (9, 2), (5, 17), (64, 64), (65, 65), (63, 130), (129, 67),
                                   (200, 150)])
@pytest.mark.parametrize("kind", ["ties", "smooth"])
def test_single_piece_parity(gpu_lib, oracle, shape, kind):
    ny, nx = shape
    seed = ny * 1000 + nx
    f = tie_field(ny, nx, 3, seed) if kind == "ties" else smooth_field(ny, nx, seed)
    r = full_rect(f)
    ods, gds = run_both(gpu_lib, oracle, f, r, r)
    compare_dataset(ods, gds, f"{kind} {shape}")


def test_many_tiny_grids(gpu_lib, oracle):
    rng = np.random.default_rng(1234)
    for t in range(150):
        ny, nx = rng.integers(2, 7, size=2)
        f = rng.integers(0, 3, size=(ny, nx)).astype(np.float32)
        r = full_rect(f)
        ods, gds = run_both(gpu_lib, oracle, f, r, r)
        compare_dataset(ods, gds, f"tiny #{t} {f.tolist()}")


def test_signed_zero_and_constant(gpu_lib, oracle):
    f = np.zeros((20, 23), np.float32)
    f[::3, ::2] = -0.0
    r = full_rect(f)
    compare_dataset(*run_both(gpu_lib, oracle, f, r, r), "signed zeros")
    g = np.full((70, 66), 5.0, np.float32)
    compare_dataset(*run_both(gpu_lib, oracle, g, full_rect(g), full_rect(g)), "constant")


@pytest.mark.parametrize("seed", range(4))
def test_piece_rect_inside_ext(gpu_lib, oracle, seed):
    """Pieces with a halo ring (rect != ext), as produced by the strip
    decomposition (grid_datamanager.cpp:53-89) and by arbitrary windows."""
    rng = np.random.default_rng(seed)
    ny, nx = 80 + 13 * seed, 70 + 29 * seed
    f = tie_field(ny, nx, 4, seed) if seed % 2 else smooth_field(ny, nx, seed)
    E = full_rect(f)
    for _ in range(3):
        x0, x1 = sorted(rng.integers(0, nx, 2) * 2)
        y0, y1 = sorted(rng.integers(0, ny, 2) * 2)
        if x1 - x0 < 2 or y1 - y0 < 2:
            continue
        ext = (max(0, x0 - 2), max(0, y0 - 2), min(E[2], x1 + 2), min(E[3], y1 + 2))
        rect = (x0, y0, x1, y1)
        compare_dataset(*run_both(gpu_lib, oracle, f, rect, ext), f"piece {rect} in {ext}")


def test_bumps256_parity(gpu_lib, oracle):
    from mscomplex_gb300 import synth
    f = synth.bumps256()
    r = full_rect(f)
    ods, gds = run_both(gpu_lib, oracle, f, r, r)
    compare_dataset(ods, gds, "bumps256")
    flags, pairs, own = gds.cells()
    check_gradient_properties(flags, pairs, own, r)


def test_bumps_quantized_parity(gpu_lib, oracle):
    from mscomplex_gb300 import synth
    f = synth.bumps4096q(n=512)
    r = full_rect(f)
    compare_dataset(*run_both(gpu_lib, oracle, f, r, r), "bumps512q")


def test_device_input_matches_host_input(gpu_lib):
    import torch
    f = smooth_field(100, 90, 5)
    r = full_rect(f)
    a = gpu_lib.GridDataset(r, r).init(f).work()
    t = torch.from_numpy(f).cuda()
    b = gpu_lib.GridDataset(r, r).init(t).work()
    for x, y in zip(a.cells(), b.cells()):
        assert np.array_equal(x, y)


def test_nan_rejected(gpu_lib):
    f = smooth_field(20, 20, 1)
    f[3, 4] = np.nan
    r = full_rect(f)
    with pytest.raises(gpu_lib.DmscError, match="INPUT"):
        gpu_lib.GridDataset(r, r).init(f).work()
