"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, as the checker of the CUDA path in ``mscomplex_gb300``; the product
never imports it.  The oracle restates the reference's CPU path
(dmsc/src/grid_dataset.cpp, dmsc/src/grid_mscomplex.cpp,
dmsc/include/discreteMorseAlgorithm.h, dmsc/src/grid_datamanager.cpp).

PARITY UNPINNED: the reference has no tests or golden vectors and cannot be
built here, so the oracle is checked by hand-derived known-answer cases and
structural properties only.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liboracle.so")
_SRC = os.path.join(_HERE, "dmsc_oracle.cpp")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle shared library (g++ -O2) if it is missing or stale."""
    with _lock:
        if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(_SRC):
            subprocess.check_call(["make", "-s", "-C", _HERE])
    return _SO


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_SO)
        vp, i64, f64, i32 = C.c_void_p, C.c_int64, C.c_double, C.c_int
        L.orc_last_error.restype = C.c_char_p
        L.orc_ds_run.restype = vp
        L.orc_ds_run.argtypes = [vp, vp, vp, f64, i32]
        L.orc_ds_run_mode.restype = vp
        L.orc_ds_run_mode.argtypes = [vp, vp, vp, f64, i32, i32]
        L.orc_ds_free.argtypes = [vp]
        L.orc_ds_ncells.restype = i64
        L.orc_ds_ncells.argtypes = [vp]
        L.orc_ds_cells.argtypes = [vp, vp, vp, vp]
        L.orc_ds_overwrites.restype = i64
        L.orc_ds_overwrites.argtypes = [vp]
        L.orc_ds_msc_dump.restype = vp
        L.orc_ds_msc_dump.argtypes = [vp]
        L.orc_dump_sizes.argtypes = [vp, vp]
        L.orc_dump_fill.argtypes = [vp] * 14
        L.orc_dump_free.argtypes = [vp]
        L.orc_pipeline_run.restype = vp
        L.orc_pipeline_run.argtypes = [vp, i32, i32, i32, f64, i32]
        L.orc_pipeline_run_ocl.restype = vp
        L.orc_pipeline_run_ocl.argtypes = [vp, i32, i32, i32, f64, i32, i32]
        L.orc_pipeline_free.argtypes = [vp]
        for f in ("orc_pipeline_nleaves", "orc_pipeline_npieces", "orc_pipeline_ncancel",
                  "orc_pipeline_overwrites", "orc_pipeline_ndisc_files", "orc_pipeline_disc_cells"):
            getattr(L, f).restype = i64
            getattr(L, f).argtypes = [vp]
        L.orc_pipeline_piece_dump.restype = vp
        L.orc_pipeline_piece_dump.argtypes = [vp, i64]
        L.orc_pipeline_root_simplified_dump.restype = vp
        L.orc_pipeline_root_simplified_dump.argtypes = [vp]
        L.orc_pipeline_times.argtypes = [vp, vp]
        L.orc_pipeline_discs.argtypes = [vp, vp, vp]
        L.orc_simplify_stats.argtypes = [vp]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _take_dump(h) -> dict:
    """Convert an oracle complex dump into numpy arrays (and free it)."""
    L = lib()
    sz = np.zeros(5, np.int64)
    L.orc_dump_sizes(h, _ptr(sz))
    n, na, nd, nad, ndd = (int(v) for v in sz)
    d = dict(
        rect_ext=np.zeros(8, np.int16),
        cellid=np.zeros((n, 2), np.int16), fn=np.zeros(n, np.float32),
        pair_idx=np.zeros(n, np.uint32), flags=np.zeros(n, np.uint8),
        asc_off=np.zeros(n + 1, np.uint32), asc=np.zeros(na, np.uint32),
        des_off=np.zeros(n + 1, np.uint32), des=np.zeros(nd, np.uint32),
        adisc_off=np.zeros(n + 1, np.uint32), adisc=np.zeros((nad, 2), np.int16),
        ddisc_off=np.zeros(n + 1, np.uint32), ddisc=np.zeros((ndd, 2), np.int16),
    )
    L.orc_dump_fill(h, *(_ptr(d[k]) for k in ("rect_ext", "cellid", "fn", "pair_idx", "flags", "asc_off", "asc",
                                               "des_off", "des", "adisc_off", "adisc", "ddisc_off", "ddisc")))
    L.orc_dump_free(h)
    return d


def _check(h):
    if not h:
        raise RuntimeError("oracle: " + lib().orc_last_error().decode())
    return h


# Dataset modes: the CPU path; the CPU path with the OpenCL kernels'
# compareCells (vertices sorted descending, dmsc/resources/assigngradient.cl:
# 40-87); the OpenCL path itself restated (GridDataset::work_ocl +
# writeout_connectivity_ocl, dmsc/src/grid_dataset.cpp:353-1022, 1250-1283).
MODE_CPU, MODE_CPU_DESC, MODE_OCL = 0, 1, 2


class Dataset:
    """One GridDataset run: init + work + writeout_connectivity
    (dmsc/src/grid_dataset.cpp:1461, 1734, 1858), optionally followed by
    simplify_un_simplify and postMergeFillDiscs on its own complex.  With
    mode=MODE_OCL: work_ocl + writeout_connectivity_ocl instead."""

    def __init__(self, window: np.ndarray, rect, ext, tresh: float = 0.0, fill_discs: bool = False,
                 mode: int = MODE_CPU):
        window = np.ascontiguousarray(window, dtype=np.float32)
        r = np.asarray(rect, np.int16)
        e = np.asarray(ext, np.int16)
        ny, nx = (e[3] - e[1]) // 2 + 1, (e[2] - e[0]) // 2 + 1
        assert window.shape == (ny, nx), (window.shape, (ny, nx))
        self._h = _check(lib().orc_ds_run_mode(_ptr(window), _ptr(r), _ptr(e), float(tresh), int(fill_discs),
                                               int(mode)))
        self.rect, self.ext = r, e
        self.cnx, self.cny = int(e[2] - e[0]) + 1, int(e[3] - e[1]) + 1

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_ds_free(self._h)
            self._h = None

    def cells(self):
        """flags int8, pairs int16x2, own int16x2 -- reference layout [x][y] (y fastest)."""
        n = int(lib().orc_ds_ncells(self._h))
        flags = np.zeros(n, np.int8)
        pairs = np.zeros((n, 2), np.int16)
        own = np.zeros((n, 2), np.int16)
        lib().orc_ds_cells(self._h, _ptr(flags), _ptr(pairs), _ptr(own))
        sh = (self.cnx, self.cny)
        return flags.reshape(sh), pairs.reshape(sh + (2,)), own.reshape(sh + (2,))

    def overwrites(self) -> int:
        return int(lib().orc_ds_overwrites(self._h))

    def msc(self) -> dict:
        return _take_dump(lib().orc_ds_msc_dump(self._h))


class Pipeline:
    """GridDataManager (dmsc/src/grid_datamanager.cpp:596-662), single-threaded order."""

    def __init__(self, field: np.ndarray, levels: int = 0, tresh: float = 0.0, split2d: bool = False,
                 ocl: bool = False):
        field = np.ascontiguousarray(field, dtype=np.float32)
        Y, X = field.shape
        self._h = _check(lib().orc_pipeline_run_ocl(_ptr(field), X, Y, int(levels), float(tresh), int(split2d),
                                                    int(bool(ocl))))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_pipeline_free(self._h)
            self._h = None

    @property
    def nleaves(self) -> int:
        return int(lib().orc_pipeline_nleaves(self._h))

    @property
    def npieces(self) -> int:
        return int(lib().orc_pipeline_npieces(self._h))

    def piece(self, i: int) -> dict:
        return _take_dump(lib().orc_pipeline_piece_dump(self._h, i))

    def root_simplified(self):
        h = lib().orc_pipeline_root_simplified_dump(self._h)
        return _take_dump(h) if h else None

    @property
    def ncancel(self) -> int:
        return int(lib().orc_pipeline_ncancel(self._h))

    @property
    def overwrites(self) -> int:
        return int(lib().orc_pipeline_overwrites(self._h))

    def times_ms(self):
        t = np.zeros(5, np.float64)
        lib().orc_pipeline_times(self._h, _ptr(t))
        return dict(build=t[0], merge_up=t[1], simplify=t[2], merge_down=t[3], discs=t[4])

    def disc_files(self) -> dict:
        """{(kind, x, y): int16[n,2]} with kind 0 = 'asc_', 1 = 'des_' (write_discs)."""
        L = lib()
        nf = int(L.orc_pipeline_ndisc_files(self._h))
        nc = int(L.orc_pipeline_disc_cells(self._h))
        hdr = np.zeros((nf, 4), np.int32)
        cells = np.zeros((nc, 2), np.int16)
        L.orc_pipeline_discs(self._h, _ptr(hdr), _ptr(cells))
        out, c = {}, 0
        for k, x, y, n in hdr:
            out[(int(k), int(x), int(y))] = cells[c:c + n]
            c += n
        return out


def simplify_stats() -> dict:
    """Counters of the simplifications run by this thread since the last call."""
    a = np.zeros(7, np.uint64)
    lib().orc_simplify_stats(_ptr(a))
    return dict(zip(("pushes", "pops", "cancels", "new_edges", "resubmits", "max_heap", "erase_work"), (int(v) for v in a)))
