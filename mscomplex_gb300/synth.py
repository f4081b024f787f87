"""Seeded synthetic height fields for the grid Morse-Smale workloads.

The reference reads a raw float32 file, x fastest (``-gf <file> -d X Y``,
dmsc/src/grid_datamanager.cpp:530-577); these generators produce arrays of
shape (Y, X) in the same element order.  No public dataset is involved: every
workload is synthetic, defined by its shape, seed and value distribution.

Workloads (by what they are):
  * ``bumps256``      256x256, 16 Gaussian bumps + U(0,1e-3) noise, seed 0
  * ``bumps4096q``    4096x4096, 512 bumps, quantised to 1/256 of the range, seed 1
  * ``noise16384``    16384x16384 i.i.d. U[0,1), seed 2
  * ``mixed_batch``   1000 grids, side log-uniform in [64, 2048], seed 3
"""
from __future__ import annotations

import math

import numpy as np


def gaussian_bumps(nx: int, ny: int, nbumps: int, sigma_lo: float, sigma_hi: float, rng: np.random.Generator,
                   noise: float = 0.0, quantize: int = 0) -> np.ndarray:
    """Sum of isotropic Gaussian bumps, float64 accumulation, returned float32 (ny, nx).

    Bump centres are uniform in the grid, sigma uniform in [sigma_lo, sigma_hi]
    pixels, amplitude uniform in [-1, 1].  Each bump is evaluated only within
    4 sigma of its centre (exp(-8) ~ 3e-4 of the amplitude beyond), which keeps
    4096^2 generation fast.  ``quantize=k`` snaps values to k steps of the range.
    """
    cx = rng.uniform(0, nx - 1, nbumps)
    cy = rng.uniform(0, ny - 1, nbumps)
    sg = rng.uniform(sigma_lo, sigma_hi, nbumps)
    amp = rng.uniform(-1.0, 1.0, nbumps)
    f = np.zeros((ny, nx), np.float64)
    for x0, y0, s, a in zip(cx, cy, sg, amp):
        r = 4.0 * s
        xa, xb = max(0, int(math.floor(x0 - r))), min(nx, int(math.ceil(x0 + r)) + 1)
        ya, yb = max(0, int(math.floor(y0 - r))), min(ny, int(math.ceil(y0 + r)) + 1)
        gx = np.exp(-0.5 * ((np.arange(xa, xb) - x0) / s) ** 2)
        gy = np.exp(-0.5 * ((np.arange(ya, yb) - y0) / s) ** 2)
        f[ya:yb, xa:xb] += a * np.outer(gy, gx)
    if noise > 0:
        f += rng.uniform(0.0, noise, f.shape)
    if quantize:
        lo, hi = float(f.min()), float(f.max())
        step = (hi - lo) / quantize if hi > lo else 1.0
        f = lo + np.round((f - lo) / step) * step
    return f.astype(np.float32)


def bumps256(seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return gaussian_bumps(256, 256, 16, 8.0, 32.0, rng, noise=1e-3)


def bumps4096q(seed: int = 1, n: int = 4096) -> np.ndarray:
    """The 4096^2 quantised workload; ``n`` scales it down for tests (bump count
    and sigma range scale with the side so the field looks alike)."""
    rng = np.random.default_rng(seed)
    k = n / 4096.0
    nb = max(4, int(round(512 * k * k)))
    return gaussian_bumps(n, n, nb, max(1.0, 4.0 * k), max(2.0, 64.0 * k), rng, quantize=256)


def noise(n: int, seed: int = 2) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.random((n, n), dtype=np.float32)


def mixed_batch_sides(count: int = 1000, seed: int = 3, lo: int = 64, hi: int = 2048) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(math.log(lo), math.log(hi), count)).astype(np.int64)


def gaussian_sum(nx: int, ny: int, nbumps: int, sigma_lo: float, sigma_hi: float, rng: np.random.Generator,
                 quantize: int = 0) -> np.ndarray:
    """Sum of isotropic Gaussian bumps evaluated everywhere (no window), float64,
    returned float32 (ny, nx).  A Gaussian is separable, so the sum is the
    matrix product Gy diag(a) Gx^T.  Without a window the field has no exact
    zero plateaus between bumps (a windowed sum is exactly 0 wherever no
    window reaches, which makes large flat ties).  ``quantize=k`` snaps values
    to k steps of the range."""
    cx = rng.uniform(0, nx - 1, nbumps)
    cy = rng.uniform(0, ny - 1, nbumps)
    sg = rng.uniform(sigma_lo, sigma_hi, nbumps)
    amp = rng.uniform(-1.0, 1.0, nbumps)
    gx = np.exp(-0.5 * ((np.arange(nx)[None, :] - cx[:, None]) / sg[:, None]) ** 2)  # (nb, nx)
    gy = np.exp(-0.5 * ((np.arange(ny)[:, None] - cy[None, :]) / sg[None, :]) ** 2)  # (ny, nb)
    f = (gy * amp[None, :]) @ gx
    if quantize:
        lo, hi = float(f.min()), float(f.max())
        step = (hi - lo) / quantize if hi > lo else 1.0
        f = lo + np.round((f - lo) / step) * step
    return f.astype(np.float32)


def mixed_grid(side: int, seed: int, quantize: int = 0) -> np.ndarray:
    """One grid of the mixed-size workloads: side x side, a sum of
    area / 8192 Gaussians with sigma U(4, 32) pixels."""
    rng = np.random.default_rng(seed)
    nb = max(1, int(round(side * side / 8192)))
    return gaussian_sum(side, side, nb, 4.0, 32.0, rng, quantize=quantize)


def batch_fields(count: int = 1000, seed: int = 3, lo: int = 64, hi: int = 2048) -> list:
    """The mixed-size batch: sides log-uniform in [lo, hi], each grid a sum of
    Gaussians (count proportional to area / 8192, sigma U(4, 32)) with its own
    seed."""
    sides = mixed_batch_sides(count, seed, lo, hi)
    return [mixed_grid(int(s), seed * 1000003 + i) for i, s in enumerate(sides)]
