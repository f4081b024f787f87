"""Shared helpers of the test suite: seeded inputs, structural properties and
exact comparisons between the CUDA path and the oracle."""
from __future__ import annotations

import numpy as np

COMPLEX_KEYS = ("rect_ext", "cellid", "fn", "pair_idx", "flags", "asc_off", "asc", "des_off", "des",
                "adisc_off", "adisc", "ddisc_off", "ddisc")


def full_rect(field: np.ndarray):
    ny, nx = field.shape
    return (0, 0, 2 * (nx - 1), 2 * (ny - 1))


def tie_field(ny: int, nx: int, levels: int, seed: int) -> np.ndarray:
    """Heights drawn from a few integer levels: exact ties everywhere."""
    rng = np.random.default_rng(seed)
    return rng.integers(0, levels, size=(ny, nx)).astype(np.float32)


def smooth_field(ny: int, nx: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:ny, 0:nx].astype(np.float64)
    f = np.zeros((ny, nx))
    for _ in range(max(2, nx * ny // 200)):
        cx, cy, s, a = rng.uniform(0, nx), rng.uniform(0, ny), rng.uniform(2, 8), rng.uniform(-1, 1)
        f += a * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * s * s))
    return f.astype(np.float32)


def assert_same_complex(got: dict, want: dict, what: str = "complex", keys=None):
    for k in keys or COMPLEX_KEYS:
        a, b = np.asarray(got[k]), np.asarray(want[k])
        if k == "fn":
            a, b = a.view(np.uint32), b.view(np.uint32)  # bit-exact float compare
        assert a.shape == b.shape, f"{what}: {k} shape {a.shape} != {b.shape}"
        if not np.array_equal(a, b):
            bad = np.argwhere(a != b)[:5]
            raise AssertionError(f"{what}: {k} differs at {bad.tolist()} (got {a[tuple(bad[0])]}, want {b[tuple(bad[0])]})")


def dims_of(cellid: np.ndarray) -> np.ndarray:
    return (cellid[:, 0] & 1) + (cellid[:, 1] & 1)


def check_gradient_properties(flags, pairs, own, ext):
    """Structural properties of a single-piece gradient (rect == ext):
    pairs are mutual neighbours, every non-critical cell is paired, owners of
    vertices/faces are critical cells of the same dimension."""
    cnx, cny = flags.shape
    x0, y0 = int(ext[0]), int(ext[1])
    paired = (flags & 1) != 0
    crit = (flags & 2) != 0
    assert np.all(paired | crit), "every cell is paired or critical"
    assert not np.any(paired & crit), "no paired critical cell when rect == ext"
    xs, ys = np.nonzero(paired)
    px = pairs[xs, ys, 0].astype(int) - x0
    py = pairs[xs, ys, 1].astype(int) - y0
    d = np.abs(px - xs) + np.abs(py - ys)
    assert np.all(d == 1), "pairs are facet/cofacet neighbours"
    assert np.all(pairs[px, py, 0] == xs + x0) and np.all(pairs[px, py, 1] == ys + y0), "pairing is mutual"
    # owners
    ox = own[..., 0].astype(int) - x0
    oy = own[..., 1].astype(int) - y0
    for dim in (0, 2):
        sel = np.zeros_like(paired)
        xx, yy = np.meshgrid(np.arange(cnx), np.arange(cny), indexing="ij")
        sel = ((xx & 1) + (yy & 1)) == dim
        assert np.all(own[sel][:, 0] >= 0), "every vertex/face has an owner"
        tx, ty = ox[sel], oy[sel]
        assert np.all(crit[tx, ty]), "owners are critical"
        assert np.all(((tx & 1) + (ty & 1)) == dim), "owner has the same dimension"
