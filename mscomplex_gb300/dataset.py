"""Host-side mirror of the reference's grid interfaces over libdmsc.so.

``GridDataset`` mirrors dmsc/include/grid_dataset.h (constructor from
rect/ext, ``init``, ``work``, ``writeout_connectivity``, and access to the
cell flags / pairs / owners and the critical-cell list); ``GridMSComplex``
mirrors dmsc/include/grid_mscomplex.h.  Names and argument meaning follow the
reference; errors raise ``DmscError`` (the reference throws std::logic_error /
std::runtime_error).
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from ._native import DMSC_ERR_PARTIAL, check, load

_ctx_lock = threading.Lock()
_ctx = {}


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Context:
    """GridDataset::init_opencl / stop_opencl equivalent: one per device."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.dmsc_init(device, C.byref(h)))
        self.h = h
        self.device = device

    def set_timing(self, enable: bool = True):
        check(self.lib.dmsc_set_timing(self.h, int(enable)))

    def pool_stats(self) -> dict:
        """Bytes of the device's stream-ordered pool (the library's buffers)."""
        a = np.zeros(4, np.int64)
        check(self.lib.dmsc_pool_stats(self.h, _ptr(a)))
        return dict(zip(("reserved", "reserved_high", "used", "used_high"), (int(v) for v in a)))

    def set_merge_parallel_min(self, min_cps: int):
        """Pipeline tree levels whose largest merge involves at least min_cps
        critical points take the parallel merges (default 2048)."""
        check(self.lib.dmsc_set_merge_parallel_min(self.h, int(min_cps)))

    def set_use_ocl(self, use_ocl: bool = True):
        """GridDataManager's ocl flag (-ocl): pipelines of this context compute
        their pieces with work_ocl."""
        check(self.lib.dmsc_set_use_ocl(self.h, int(bool(use_ocl))))

    def set_out_of_core(self, directory: str | None):
        """GridDataManager's compute_out_of_core (--out-of-core): pipelines of
        this context keep their pieces' complexes in archive files under
        `directory` (None: in device memory)."""
        check(self.lib.dmsc_set_out_of_core(self.h, directory.encode() if directory else None))

    def set_merge_rounds(self, window: int = 0, min_commits: int = 4):
        """merge_up's boundary cancellations on the parallel merges: 0 (the
        default) runs them on one thread per merge; window > 0 in rounds over
        the first `window` pending boundary cells, one thread finishing in
        order after 8 rounds in a row below `min_commits` commits.  Every
        setting gives the same complexes."""
        check(self.lib.dmsc_set_merge_rounds(self.h, int(window), int(min_commits)))

    def close(self):
        if self.h:
            check(self.lib.dmsc_shutdown(self.h))
            self.h = None


def default_context(device: int = 0) -> Context:
    with _ctx_lock:
        if device not in _ctx:
            _ctx[device] = Context(device)
        return _ctx[device]


def _rect(r) -> np.ndarray:
    a = np.asarray(r, dtype=np.int16).reshape(4)
    return np.ascontiguousarray(a)


class GridDataset:
    """One piece of the grid: rect (owned cells) inside ext (rect plus halo),
    both as (left, bottom, right, top) in cell coordinates."""

    def __init__(self, rect, ext=None, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.lib = self.ctx.lib
        self.rect = _rect(rect)
        self.ext = _rect(ext if ext is not None else rect)
        h = C.c_void_p()
        check(self.lib.dmsc_dataset_create(self.ctx.h, _ptr(self.rect), _ptr(self.ext), C.byref(h)))
        self.h = h
        self.cnx = int(self.ext[2] - self.ext[0]) + 1
        self.cny = int(self.ext[3] - self.ext[1]) + 1
        self.vnx = self.cnx // 2 + 1
        self.vny = self.cny // 2 + 1
        self._keep = None

    @classmethod
    def _borrowed(cls, handle, ctx: Context, rect, ext, owner):
        """A view of a dataset that another object owns (a pipeline's leaf)."""
        self = cls.__new__(cls)
        self.ctx, self.lib, self.h = ctx, ctx.lib, handle
        self.rect, self.ext = _rect(rect), _rect(ext)
        self.cnx = int(self.ext[2] - self.ext[0]) + 1
        self.cny = int(self.ext[3] - self.ext[1]) + 1
        self.vnx, self.vny = self.cnx // 2 + 1, self.cny // 2 + 1
        self._keep, self._owner = None, owner
        return self

    def __del__(self):
        if getattr(self, "h", None) and getattr(self, "_owner", None) is None:
            self.lib.dmsc_dataset_destroy(self.h)
        self.h = None

    def init(self, heights, stream=None):
        """GridDataset::init: heights of the ext window, shape (vny, vnx), x fastest.
        A numpy array is copied to the device; a CUDA tensor is borrowed."""
        if hasattr(heights, "is_cuda") and heights.is_cuda:
            t = heights
            if t.dtype.__repr__() != "torch.float32" or t.dim() != 2 or t.stride(1) != 1:
                raise ValueError("device heights must be a 2D float32 tensor with unit x stride")
            if tuple(t.shape) != (self.vny, self.vnx):
                raise ValueError(f"heights shape {tuple(t.shape)} != ext window {(self.vny, self.vnx)}")
            self._keep = t
            if stream is None:
                # the library's own stream does not order with torch's streams
                import torch
                torch.cuda.current_stream(t.device).synchronize()
            check(self.lib.dmsc_dataset_init(self.h, C.c_void_p(t.data_ptr()), t.stride(0), 1, stream))
        else:
            a = np.ascontiguousarray(heights, dtype=np.float32)
            if a.shape != (self.vny, self.vnx):
                raise ValueError(f"heights shape {a.shape} != ext window {(self.vny, self.vnx)}")
            self._keep = a
            check(self.lib.dmsc_dataset_init(self.h, _ptr(a), a.shape[1], 0, stream))
        return self

    def work(self, stream=None):
        """Gradient, critical-cell collation and owner extrema (GridDataset::work)."""
        check(self.lib.dmsc_dataset_work(self.h, stream))
        return self

    def work_ocl(self, stream=None):
        """GridDataset::work_ocl: the gradient of the reference's OpenCL
        kernels (compareCells with vertices sorted descending), collation and
        owner extrema."""
        check(self.lib.dmsc_dataset_work_ocl(self.h, stream))
        return self

    @property
    def num_critical(self) -> int:
        n = C.c_int64()
        check(self.lib.dmsc_dataset_num_critical(self.h, C.byref(n)))
        return n.value

    def cells(self):
        """(flags int8, pairs int16[...,2], own int16[...,2]) in the reference
        layout [x][y] over ext (shape (cnx, cny))."""
        n = self.cnx * self.cny
        flags = np.zeros(n, np.int8)
        pairs = np.zeros((n, 2), np.int16)
        own = np.zeros((n, 2), np.int16)
        check(self.lib.dmsc_dataset_export_cells(self.h, _ptr(flags), _ptr(pairs), _ptr(own), None))
        sh = (self.cnx, self.cny)
        return flags.reshape(sh), pairs.reshape(sh + (2,)), own.reshape(sh + (2,))

    def critical_cells(self) -> np.ndarray:
        n = self.num_critical
        out = np.zeros((n, 2), np.int16)
        if n:
            check(self.lib.dmsc_dataset_export_critical(self.h, _ptr(out), None))
        return out

    STAGES = ("gradient", "collate_scan", "border_resolve", "labels_arcs", "connectivity", "disc_hops", "discs",
              "seg_place_asc", "seg_place_des")

    def stage_times(self, with_discs: bool = False) -> dict:
        """Device times (ms) of the last work / writeout_connectivity (and, with
        with_discs, post_merge_fill_discs: its hop kernel, the whole pass and
        the placement kernel of each disc kind)."""
        n = 9 if with_discs else 5
        ms = np.zeros(n, np.float32)
        check(self.lib.dmsc_dataset_stage_times(self.h, _ptr(ms), n))
        return dict(zip(self.STAGES, (float(v) for v in ms)))

    def post_merge_fill_discs(self, msc: "GridMSComplex", stream=None) -> "GridMSComplex":
        """GridDataset::postMergeFillDiscs: the manifold discs of `msc`."""
        check(self.lib.dmsc_dataset_fill_discs(self.h, msc.h, stream))
        return msc

    def writeout_connectivity(self, msc: "GridMSComplex | None" = None, stream=None) -> "GridMSComplex":
        """GridDataset::writeout_connectivity: the complex of this piece.  With
        `msc`, that complex is overwritten in place (its buffers are reused)."""
        if msc is not None:
            h = C.c_void_p(msc.h.value if isinstance(msc.h, C.c_void_p) else msc.h)
            check(self.lib.dmsc_dataset_writeout_connectivity(self.h, C.byref(h), stream))
            return msc
        h = C.c_void_p()
        check(self.lib.dmsc_dataset_writeout_connectivity(self.h, C.byref(h), stream))
        return GridMSComplex(h, self.ctx)

    def writeout_connectivity_ocl(self, stream=None) -> "GridMSComplex":
        """GridDataset::writeout_connectivity_ocl: the complex from the saddle
        incidences of the last work_ocl (the same complex as
        writeout_connectivity gives)."""
        h = C.c_void_p()
        check(self.lib.dmsc_dataset_writeout_connectivity_ocl(self.h, C.byref(h), stream))
        return GridMSComplex(h, self.ctx)


class GridMSComplex:
    """A Morse-Smale complex held on the device (handle to dmsc_msc)."""

    def __init__(self, handle, ctx: Context, owner=None):
        self.h = handle
        self.ctx = ctx
        self.lib = ctx.lib
        self._owner = owner  # a Pipeline owns its pieces' complexes

    def __del__(self):
        if getattr(self, "h", None) and self._owner is None:
            self.lib.dmsc_msc_destroy(self.h)
        self.h = None

    def simplify_un_simplify(self, tresh: float, max_ops: int = 0, stream=None) -> dict:
        """GridMSComplex::simplify_un_simplify: persistence cancellation at
        `tresh` (fraction of the value range) in the reference's exact order."""
        rc = self.lib.dmsc_msc_simplify_un_simplify(self.h, float(tresh), int(max_ops), stream)
        st = self.simplify_stats()
        check(rc)
        return st

    def simplify_stats(self) -> dict:
        a = np.zeros(5, np.uint64)
        check(self.lib.dmsc_msc_simplify_stats(self.h, _ptr(a)))
        return dict(zip(("pushes", "pops", "cancels", "ops", "status"), (int(v) for v in a)))

    def write_discs(self, prefix: str):
        """GridMSComplex::write_discs: one binary file per disc, appended."""
        check(self.lib.dmsc_msc_write_discs(self.h, prefix.encode()))

    def save(self, path: str):
        """The whole complex to an archive file (this library's layout)."""
        check(self.lib.dmsc_msc_save(self.h, path.encode()))

    @classmethod
    def load(cls, path: str, ctx: Context | None = None) -> "GridMSComplex":
        ctx = ctx or default_context()
        h = C.c_void_p()
        check(ctx.lib.dmsc_msc_load(ctx.h, path.encode(), C.byref(h)))
        return cls(h, ctx)

    def sizes(self):
        s = np.zeros(5, np.int64)
        check(self.lib.dmsc_msc_sizes(self.h, _ptr(s)))
        return [int(v) for v in s]

    EXPORT_KEYS = ("rect_ext", "cellid", "fn", "pair_idx", "flags", "asc_off", "asc", "des_off", "des",
                   "adisc_off", "adisc", "ddisc_off", "ddisc")

    def export_shapes(self) -> dict:
        n, na, nd, nad, ndd = self.sizes()
        return dict(rect_ext=((8,), np.int16), cellid=((n, 2), np.int16), fn=((n,), np.float32),
                    pair_idx=((n,), np.uint32), flags=((n,), np.uint8), asc_off=((n + 1,), np.uint32),
                    asc=((na,), np.uint32), des_off=((n + 1,), np.uint32), des=((nd,), np.uint32),
                    adisc_off=((n + 1,), np.uint32), adisc=((nad, 2), np.int16),
                    ddisc_off=((n + 1,), np.uint32), ddisc=((ndd, 2), np.int16))

    def export(self, out: dict | None = None, stream=None, wait: bool = True) -> dict:
        """Flat arrays with the same keys as the oracle's complex dump.  `out`
        may hold preallocated flat host buffers (e.g. pinned) per key, large
        enough: the result is then views into them.  With wait=False the
        copies are only queued on `stream` (dmsc_msc_export_async): the views
        hold the complex once that stream has reached them, and neither the
        complex nor the buffers may change before; `out` must then be pinned."""
        shapes = self.export_shapes()
        if not wait and out is None:
            raise ValueError("export(wait=False) needs preallocated pinned buffers in `out`")
        if out is None:
            d = {k: np.zeros(sh, dt) for k, (sh, dt) in shapes.items()}
        else:
            d = {}
            for k, (sh, dt) in shapes.items():
                n = int(np.prod(sh))
                buf = out[k].view(dt).reshape(-1)
                if buf.size < n:
                    raise ValueError(f"export buffer {k} holds {buf.size} < {n} elements")
                d[k] = buf[:n].reshape(sh)
        fn = self.lib.dmsc_msc_export if wait else self.lib.dmsc_msc_export_async
        check(fn(self.h, *(_ptr(d[k]) for k in self.EXPORT_KEYS), stream))
        return d


class GridDataManager:
    """The piece pipeline of GridDataManager (dmsc/src/grid_datamanager.cpp):
    the grid split `levels` times into pieces, one complex per piece, merge up
    to the root, simplify_un_simplify(tresh) there, merge down, and the
    manifold discs of every piece.  heights: (size_y, size_x) float32 numpy
    array (copied to the device) or CUDA tensor (read in place)."""

    STAGES = ("pieces", "merge_up", "simplify", "merge_down", "discs")

    def __init__(self, heights, levels: int = 0, tresh: float = 0.0, split2d: bool = False,
                 ctx: Context | None = None, stream=None):
        self.ctx = ctx or default_context()
        self.lib = self.ctx.lib
        h = C.c_void_p()
        if hasattr(heights, "is_cuda") and heights.is_cuda:
            t = heights
            if t.dtype.__repr__() != "torch.float32" or t.dim() != 2 or t.stride(1) != 1:
                raise ValueError("device heights must be a 2D float32 tensor with unit x stride")
            ny, nx = int(t.shape[0]), int(t.shape[1])
            self._keep = t
            if stream is None:
                import torch
                torch.cuda.current_stream(t.device).synchronize()
            rc = self.lib.dmsc_pipeline_run(self.ctx.h, C.c_void_p(t.data_ptr()), t.stride(0), 1, nx, ny,
                                            int(levels), float(tresh), int(bool(split2d)), C.byref(h), stream)
        else:
            a = np.ascontiguousarray(heights, dtype=np.float32)
            if a.ndim != 2:
                raise ValueError("heights must be 2D (size_y, size_x)")
            ny, nx = a.shape
            self._keep = a
            rc = self.lib.dmsc_pipeline_run(self.ctx.h, _ptr(a), nx, 0, nx, ny, int(levels), float(tresh),
                                            int(bool(split2d)), C.byref(h), stream)
        check(rc)
        self.h = h
        n = C.c_int64()
        check(self.lib.dmsc_pipeline_num_pieces(self.h, C.byref(n)))
        self.num_pieces = n.value

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.dmsc_pipeline_destroy(self.h)
            self.h = None

    def piece(self, i: int) -> GridMSComplex:
        """Node i of the piece tree after merge_down: leaves first (with
        discs), then the merges, the root last (2 * num_pieces - 2)."""
        m = C.c_void_p()
        check(self.lib.dmsc_pipeline_piece(self.h, int(i), C.byref(m), None))
        return GridMSComplex(m, self.ctx, owner=self)

    def leaf_dataset(self, i: int) -> GridDataset:
        """Leaf i's dataset (gradient, owners, critical cells of its window),
        owned by the pipeline."""
        if not 0 <= i < self.num_pieces:
            raise IndexError(f"leaf {i} out of range")
        m, d = C.c_void_p(), C.c_void_p()
        check(self.lib.dmsc_pipeline_piece(self.h, int(i), C.byref(m), C.byref(d)))
        re = self.piece(i).export()["rect_ext"]
        return GridDataset._borrowed(d, self.ctx, re[:4], re[4:], owner=self)

    def write_discs(self, prefix: str):
        """collectSubdomainManifolds: write_discs of every piece in leaf order."""
        check(self.lib.dmsc_pipeline_write_discs(self.h, prefix.encode()))

    def stage_times(self) -> dict:
        ms = np.zeros(5, np.float64)
        check(self.lib.dmsc_pipeline_stage_times(self.h, _ptr(ms)))
        return dict(zip(self.STAGES, (float(v) for v in ms)))

    def merge_seq_times(self) -> dict:
        """Of merge up / down, the ms spent in the boundary steps (merge up's
        cancellations in ordered-parallel rounds, merge down's uncancellations
        on one thread per merge)."""
        ms = np.zeros(2, np.float64)
        check(self.lib.dmsc_pipeline_merge_times(self.h, _ptr(ms)))
        return {"merge_up": float(ms[0]), "merge_down": float(ms[1])}


class GridBatch:
    """Many whole grids through work + writeout_connectivity +
    simplify_un_simplify in shared launches (no reference counterpart: the
    reference builds one GridDataset at a time).  fields: 2D float32 arrays
    (size_y, size_x), or one packed 1D array/tensor with `shapes`; tresh: one
    threshold per grid (0 skips simplification)."""

    GRAPH_KEYS = ("rect_ext", "cellid", "fn", "pair_idx", "flags", "asc_off", "asc", "des_off", "des")

    def __init__(self, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.lib = self.ctx.lib
        self.h = C.c_void_p()
        self.n = 0

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.dmsc_batch_destroy(self.h)
            self.h = None

    CLASSES = ("<128", "<256", "<512", "<1024", "<2048", ">=2048")

    @staticmethod
    def autotune(fields, repeats: int = 3, ctx: Context | None = None) -> dict:
        """The batch launch autotuner (dmsc_batch_autotune): per size class of
        the sample's grids (larger side <128, <256, <512, <1024, <2048,
        >=2048), the fastest launch configuration of the two tile kernels
        (threads per block, resident blocks per SM) becomes the context's.
        Returns {class: (threads, blocks_per_sm, us, default_us)}."""
        ctx = ctx or default_context()
        packed, sizes = GridBatch.pack(fields)
        t = np.zeros(24, np.int32)
        check(ctx.lib.dmsc_batch_autotune(ctx.h, len(fields), _ptr(sizes), _ptr(packed), 0, int(repeats), _ptr(t)))
        return {GridBatch.CLASSES[c]: tuple(int(v) for v in t[4 * c:4 * c + 4]) for c in range(6) if t[4 * c]}

    @staticmethod
    def set_launch(size_class: int, threads: int, blocks_per_sm: int, ctx: Context | None = None):
        """Pins one size class's launch configuration (as the autotuner would)."""
        ctx = ctx or default_context()
        check(ctx.lib.dmsc_batch_set_launch(ctx.h, int(size_class), int(threads), int(blocks_per_sm)))

    @staticmethod
    def autotune_reset(ctx: Context | None = None):
        ctx = ctx or default_context()
        check(ctx.lib.dmsc_batch_autotune_reset(ctx.h))

    def tile_times(self):
        """Device ms of the last run's gradient and owner-label tile kernels."""
        ms = np.zeros(2, np.float32)
        check(self.lib.dmsc_batch_tile_times(self.h, _ptr(ms)))
        return float(ms[0]), float(ms[1])

    @staticmethod
    def pack(fields):
        """(packed float32 heights, sizes int32[2n]) of a list of 2D fields."""
        sizes = np.array([[f.shape[1], f.shape[0]] for f in fields], np.int32).reshape(-1)
        packed = np.concatenate([np.ascontiguousarray(f, np.float32).reshape(-1) for f in fields])
        return packed, sizes

    def run(self, fields=None, tresh=0.0, *, packed=None, sizes=None, max_ops: int = 0, stream=None,
            partial_ok: bool = False):
        """Runs the batch.  A grid whose simplification fails (its operation
        budget, an invariant) fails alone; with partial_ok the batch is kept
        and grid_status(i) names the failed grids, otherwise DmscError."""
        if fields is not None:
            packed, sizes = self.pack(fields)
        sizes = np.ascontiguousarray(sizes, np.int32).reshape(-1)
        n = sizes.size // 2
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(tresh, np.float64), (n,)))
        if hasattr(packed, "is_cuda") and packed.is_cuda:
            if packed.dtype.__repr__() != "torch.float32" or not packed.is_contiguous():
                raise ValueError("device heights must be a contiguous float32 tensor")
            if stream is None:
                import torch
                torch.cuda.current_stream(packed.device).synchronize()
            self._keep = packed
            ptr, on_dev = C.c_void_p(packed.data_ptr()), 1
        else:
            packed = np.ascontiguousarray(packed, np.float32)
            self._keep = packed
            ptr, on_dev = _ptr(packed), 0
        rc = self.lib.dmsc_batch_run(self.ctx.h, n, _ptr(sizes), ptr, on_dev, _ptr(t), int(max_ops),
                                     C.byref(self.h), stream)
        if not (partial_ok and rc == DMSC_ERR_PARTIAL):
            check(rc)
        self.n = n
        self._sizes = sizes
        return self

    def sizes(self, i: int):
        s = np.zeros(3, np.int64)
        check(self.lib.dmsc_batch_sizes(self.h, int(i), _ptr(s)))
        return [int(v) for v in s]

    def grid_status(self, i: int):
        """(status code, message) of grid i: DMSC_OK (0) or its own error."""
        code = C.c_int(0)
        msg = C.create_string_buffer(512)
        check(self.lib.dmsc_batch_grid_status(self.h, int(i), C.byref(code), msg, 512))
        return int(code.value), msg.value.decode()

    def simplify_stats(self, i: int) -> dict:
        a = np.zeros(5, np.uint64)
        check(self.lib.dmsc_batch_simplify_stats(self.h, int(i), _ptr(a)))
        return dict(zip(("pushes", "pops", "cancels", "ops", "status"), (int(v) for v in a)))

    def export(self, i: int) -> dict:
        n, na, nd = self.sizes(i)
        d = dict(rect_ext=np.zeros(8, np.int16), cellid=np.zeros((n, 2), np.int16), fn=np.zeros(n, np.float32),
                 pair_idx=np.zeros(n, np.uint32), flags=np.zeros(n, np.uint8), asc_off=np.zeros(n + 1, np.uint32),
                 asc=np.zeros(na, np.uint32), des_off=np.zeros(n + 1, np.uint32), des=np.zeros(nd, np.uint32))
        check(self.lib.dmsc_batch_export(self.h, int(i), *(_ptr(d[k]) for k in self.GRAPH_KEYS), None))
        return d

    def totals(self):
        t = np.zeros(3, np.int64)
        check(self.lib.dmsc_batch_totals(self.h, _ptr(t)))
        return [int(v) for v in t]

    def export_all(self, out: dict | None = None) -> dict:
        """All grids at once (shared arrays plus per-grid bases); `out` may
        hold preallocated flat host buffers per key."""
        ncp, na, nd = self.totals()
        g1 = self.n + 1
        shapes = dict(cp_base=(g1, np.uint32), asc_base=(g1, np.uint32), des_base=(g1, np.uint32),
                      cellid=(ncp, np.uint32), fn=(ncp, np.float32), pair_idx=(ncp, np.uint32), flags=(ncp, np.uint8),
                      asc_off=(ncp + 1, np.uint32), asc=(na, np.uint32), des_off=(ncp + 1, np.uint32),
                      des=(nd, np.uint32))
        d = {}
        for k, (m, dt) in shapes.items():
            if out is None:
                d[k] = np.zeros(m, dt)
            else:
                buf = out[k].view(dt).reshape(-1)
                if buf.size < m:
                    raise ValueError(f"export buffer {k} holds {buf.size} < {m} elements")
                d[k] = buf[:m]
        check(self.lib.dmsc_batch_export_all(self.h, *(_ptr(d[k]) for k in shapes), None))
        return d


class GridServer:
    """Request server with continuous batching over GridBatch (no reference
    counterpart).  submit() copies the heights and returns a request id;
    result() waits and returns the grid's complex (the GridBatch.export keys)
    with its submit / start / done times in ms."""

    def __init__(self, arena_bytes: int = 150 << 30, lanes: int = 2, max_batch: int = 256, max_ops: int = 0,
                 ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.lib = self.ctx.lib
        h = C.c_void_p()
        check(self.lib.dmsc_server_create(self.ctx.h, int(arena_bytes), int(lanes), int(max_batch), int(max_ops),
                                          C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.dmsc_server_destroy(self.h)
            self.h = None

    __del__ = close

    def submit(self, heights: np.ndarray, tresh: float = 0.0) -> int:
        a = np.ascontiguousarray(heights, np.float32)
        if a.ndim != 2:
            raise ValueError("heights must be 2D (size_y, size_x)")
        rid = C.c_int64()
        check(self.lib.dmsc_server_submit(self.h, _ptr(a), a.shape[1], a.shape[0], float(tresh), C.byref(rid)))
        return rid.value

    def wait(self, rid: int, timeout_ms: int = -1) -> bool:
        done, status = C.c_int(), C.c_int()
        check(self.lib.dmsc_server_wait(self.h, int(rid), int(timeout_ms), C.byref(done), C.byref(status)))
        return bool(done.value)

    def result(self, rid: int, release: bool = True) -> dict:
        self.wait(rid)
        sizes = np.zeros(3, np.int64)
        times = np.zeros(3, np.float64)
        err = C.create_string_buffer(512)
        check(self.lib.dmsc_server_result(self.h, int(rid), _ptr(sizes), _ptr(times), err, 512))
        n, na, nd = (int(v) for v in sizes)
        d = dict(cellid=np.zeros((n, 2), np.int16), fn=np.zeros(n, np.float32), pair_idx=np.zeros(n, np.uint32),
                 flags=np.zeros(n, np.uint8), asc_off=np.zeros(n + 1, np.uint32), asc=np.zeros(na, np.uint32),
                 des_off=np.zeros(n + 1, np.uint32), des=np.zeros(nd, np.uint32))
        check(self.lib.dmsc_server_export(self.h, int(rid), *(_ptr(d[k]) for k in
                                                             ("cellid", "fn", "pair_idx", "flags", "asc_off", "asc",
                                                              "des_off", "des"))))
        d["times_ms"] = times
        if release:
            check(self.lib.dmsc_server_release(self.h, int(rid)))
        return d

    def stats(self) -> dict:
        s = np.zeros(4, np.int64)
        check(self.lib.dmsc_server_stats(self.h, _ptr(s)))
        return dict(zip(("batches", "grids_done", "queued", "arena_in_use"), (int(v) for v in s)))
