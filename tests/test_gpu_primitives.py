"""GPU tests of the scan and sort primitives (PrefixScan / BitonicSortProgram slots)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [0, 1, 7, 4095, 4096, 4097, 100003, 5_000_011])
def test_prefix_scan(gpu_lib, n):
    import torch
    from mscomplex_gb300.primitives import prefix_scan
    rng = np.random.default_rng(n)
    x = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
    t = torch.from_numpy(x.view(np.int32)).cuda()
    tot = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = prefix_scan(t, total=tot).cpu().numpy().view(np.uint32)
    want = (np.cumsum(x.astype(np.uint64)) - x.astype(np.uint64)) % (1 << 32)
    assert np.array_equal(out, want.astype(np.uint32))
    if n:
        assert int(tot.cpu().numpy().view(np.uint32)[0]) == int(np.sum(x.astype(np.uint64)) % (1 << 32))


@pytest.mark.parametrize("batch,length,asc", [(1, 1, True), (1, 1000, True), (1, 70001, False), (7, 513, True),
                                              (64, 4096, False), (3, 1, True)])
def test_sort_pairs(gpu_lib, batch, length, asc):
    import torch
    from mscomplex_gb300.primitives import sort_pairs
    rng = np.random.default_rng(batch * 7 + length)
    k = rng.integers(0, 50, size=batch * length).astype(np.uint32)  # many ties: checks stability
    v = np.arange(batch * length, dtype=np.uint32)
    ok, ov = sort_pairs(torch.from_numpy(k.view(np.int32)).cuda(), torch.from_numpy(v.view(np.int32)).cuda(),
                        batch=batch, ascending=asc)
    ok = ok.cpu().numpy().view(np.uint32).reshape(batch, length)
    ov = ov.cpu().numpy().view(np.uint32).reshape(batch, length)
    kk, vv = k.reshape(batch, length), v.reshape(batch, length)
    for b in range(batch):
        order = np.argsort(kk[b] if asc else -kk[b].astype(np.int64), kind="stable")
        assert np.array_equal(ok[b], kk[b][order])
        assert np.array_equal(ov[b], vv[b][order])
