"""Device primitives of libdmsc.so on CUDA tensors: the reference's
PrefixScan::PreScanBuffer (dmsc/include/prefix_scan.h:105-109) and
BitonicSortProgram::bitonicSort (dmsc/include/bitonic_sort.h:30-39) slots."""
from __future__ import annotations

import ctypes as C

from ._native import check
from .dataset import default_context


def _dev(t, name):
    if not (hasattr(t, "is_cuda") and t.is_cuda) or str(t.dtype) not in ("torch.int32", "torch.uint32"):
        raise ValueError(f"{name} must be a CUDA int32/uint32 tensor")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    return C.c_void_p(t.data_ptr())


def _stream(stream):
    if stream is None:
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return C.c_void_p(stream)


def prefix_scan(x, out=None, total=None, stream=None, ctx=None):
    """Exclusive prefix sum (uint32, wrapping) of a 1-D CUDA tensor."""
    import torch
    ctx = ctx or default_context(x.device.index or 0)
    out = torch.empty_like(x) if out is None else out
    tp = _dev(total, "total") if total is not None else None
    check(ctx.lib.dmsc_prefix_scan(ctx.h, _dev(out, "out"), _dev(x, "x"), x.numel(), tp, _stream(stream)))
    return out


def sort_pairs(keys, vals, batch: int = 1, ascending: bool = True, stream=None, ctx=None):
    """Stable sort of `batch` equal-length (key, value) uint32 arrays."""
    import torch
    ctx = ctx or default_context(keys.device.index or 0)
    n = keys.numel()
    if n % batch:
        raise ValueError("numel must be a multiple of batch")
    ok, ov = torch.empty_like(keys), torch.empty_like(vals)
    check(ctx.lib.dmsc_sort_pairs(ctx.h, _dev(ok, "keys_out"), _dev(ov, "vals_out"), _dev(keys, "keys"), _dev(vals, "vals"),
                                  batch, n // batch, 1 if ascending else 0, _stream(stream)))
    return ok, ov
