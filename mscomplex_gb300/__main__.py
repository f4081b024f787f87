"""Command line of the grid pipeline, with the reference's flags
(dmsc/src/main.cpp:14-29, parse_grid :140-232):

    python -m mscomplex_gb300 -gf <file> -d <x_dim> <y_dim> [-l <levels>]
        [--simp-tresh <tresh>] [--split2d] [--outdir <dir>] [-st] [-ocl] [--num-parallel <n>]

<file> holds x_dim * y_dim float32 heights, x fastest (the reference's raw
grid file, read by GridDataManager::readDataAndInit, grid_datamanager.cpp:
530-577).  The pipeline of GridDataManager runs on the GPU: pieces (2^levels
strips along y, as -l; --split2d alternates y and x), merges, simplification
at the root when tresh > 0, discs.  The disc files are written as the
reference's collectSubdomainManifolds does (prefix "dp__disc_", :414-416) into
--outdir (default: the working directory).  -ocl computes the pieces with the
gradient of the reference's OpenCL backend (GridDataset::work_ocl: cell
vertices sorted descending in compareCells).  --out-of-core keeps the pieces'
complexes in archive files (in --outdir) between the pipeline's stages, as the
reference's compute_out_of_core does.  -st and --num-parallel select CPU
threading in the reference and are accepted without effect.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np


def parse(argv):
    ap = argparse.ArgumentParser(prog="python -m mscomplex_gb300", add_help=True)
    ap.add_argument("-gf", dest="file", required=True, help="raw float32 grid file, x fastest")
    ap.add_argument("-d", dest="dims", nargs=2, type=int, required=True, metavar=("X", "Y"))
    ap.add_argument("-l", dest="levels", type=int, default=1, help="piece levels (2^levels pieces)")
    ap.add_argument("--simp-tresh", dest="tresh", type=float, default=0.0)
    ap.add_argument("--split2d", action="store_true", help="alternate y and x splits (square blocks)")
    ap.add_argument("--outdir", default=".")
    ap.add_argument("-st", action="store_true")
    ap.add_argument("-ocl", action="store_true")
    ap.add_argument("--num-parallel", type=int, default=1)
    ap.add_argument("--out-of-core", action="store_true")
    ap.add_argument("--buffer-zone-width", type=int, default=1)
    a = ap.parse_args(argv)
    if a.dims[0] < 2 or a.dims[1] < 2:
        ap.error("-d needs at least 2 x 2 vertices")
    if a.levels < 0:
        ap.error("-l must be >= 0")
    return a


def load_raw(path: str, x: int, y: int) -> np.ndarray:
    n = x * y
    data = np.fromfile(path, dtype=np.float32, count=n)
    if data.size != n:
        raise ValueError(f"{path}: {data.size} float32 values, expected {x} x {y} = {n}")
    return data.reshape(y, x)


def main(argv=None) -> int:
    a = parse(sys.argv[1:] if argv is None else argv)
    from . import Context, GridDataManager
    field = load_raw(a.file, a.dims[0], a.dims[1])
    os.makedirs(a.outdir, exist_ok=True)
    ctx = Context()
    ctx.set_use_ocl(a.ocl)
    if a.out_of_core:
        ctx.set_out_of_core(a.outdir)
    t0 = time.perf_counter()
    p = GridDataManager(field, levels=a.levels, tresh=a.tresh, split2d=a.split2d, ctx=ctx)
    t1 = time.perf_counter()
    p.write_discs(os.path.join(a.outdir, "dp__disc_"))
    t2 = time.perf_counter()
    for k, v in p.stage_times().items():
        print(f"{k}: timer_time = {v:.3f}")
    print(f"pipeline: timer_time = {1e3 * (t1 - t0):.3f}")
    print(f"write_discs: timer_time = {1e3 * (t2 - t1):.3f}")
    print(f"pieces = {p.num_pieces}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
