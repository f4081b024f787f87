"""GPU test of dmsc_prefix_scan_noalloc, the scan for callers that cannot let a
library allocate device memory (a host runtime that owns the GPU's memory
through its own pool, or a serving loop where cudaMalloc's device-wide
synchronisation is not allowed).

It is compared, through the C ABI, with dmsc_prefix_scan (which takes its
scratch from the allocator) on two calls in a row, so that whatever the first
call leaves in the shared fixed scratch cannot leak into the second result.
The file sorts last so that a run stopping at the first failure has already
run every other test; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _u32_tensor(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint32).view(np.int32)).cuda()


def _host_u32(t):
    return t.cpu().numpy().view(np.uint32)


def test_noalloc_scan_matches_allocating_scan(gpu_lib):
    import torch
    ctx = gpu_lib.default_context(0)
    lib = ctx.lib
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(20261203)
    # calls in a row over different data: two-level scans, then the largest
    # size the fixed scratch serves and a 4096^2 + 1 scan (three levels of
    # partial sums in the fixed array)
    for n in (3_000_017, 4096 * 37 + 5, 1 << 26, 4096 * 4096 + 1):
        x = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
        d_in = _u32_tensor(x)
        want, got = torch.empty_like(d_in), torch.full_like(d_in, -1)
        want_tot, got_tot = torch.zeros(1, dtype=torch.int32, device="cuda"), torch.full((1,), -1, dtype=torch.int32, device="cuda")
        rc = lib.dmsc_prefix_scan(ctx.h, C.c_void_p(want.data_ptr()), C.c_void_p(d_in.data_ptr()), n,
                                  C.c_void_p(want_tot.data_ptr()), stream)
        assert rc == 0, lib.dmsc_last_error()
        rc = lib.dmsc_prefix_scan_noalloc(ctx.h, C.c_void_p(got.data_ptr()), C.c_void_p(d_in.data_ptr()), n,
                                          C.c_void_p(got_tot.data_ptr()), stream)
        assert rc == 0, lib.dmsc_last_error()
        torch.cuda.synchronize()
        assert np.array_equal(_host_u32(got), _host_u32(want)), f"scan differs at n={n}"
        assert _host_u32(got_tot)[0] == _host_u32(want_tot)[0], f"total differs at n={n}"
        assert _host_u32(got)[-1] == (int(np.sum(x[:-1].astype(np.uint64))) % (1 << 32))


def test_noalloc_scan_rejects_sizes_beyond_its_scratch(gpu_lib):
    import torch
    ctx = gpu_lib.default_context(0)
    lib = ctx.lib
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    rc = lib.dmsc_prefix_scan_noalloc(ctx.h, p, p, (1 << 26) + 1, None, None)
    assert rc != 0
    assert b"67108864" in lib.dmsc_last_error()
