"""Full-size workloads checked through properties that do not depend on the
size (the oracle needs minutes to hours at these sizes): the 4096² quantised
step and the 16384² white-noise piece pipeline.  Euler characteristic 1, asc
and des lists transposes of each other with multiplicity, extremum discs
partitioning the vertices and faces, and identical results run to run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dims(cellid):
    c = cellid.astype(np.int64)
    return (c[:, 0] & 1) + (c[:, 1] & 1)


def _mix(a, b):
    """An order-independent fingerprint term of the pair (a, b) (64-bit mixing)."""
    x = (a.astype(np.uint64) << np.uint64(32)) | b.astype(np.uint64)
    x ^= x >> np.uint64(33)
    x *= np.uint64(0xFF51AFD7ED558CCD)
    x ^= x >> np.uint64(33)
    x *= np.uint64(0xC4CEB9FE1A85EC53)
    x ^= x >> np.uint64(33)
    return x


def transpose_check(m, what):
    """asc(p) holds q k times iff des(q) holds p k times: the multiset of
    (owner, value) pairs of the asc lists equals that of the des lists
    reversed, compared through sums of a 64-bit pair hash.  Pairs touching a
    boundary-cancelable point are left out: uncancel_pairs rewrites the
    lists of an uncancelled pair without their reverse entries (the
    reference's representation after merge_down)."""
    n = len(m["flags"])
    bc = (m["flags"] & 4) != 0
    sums = []
    for off_k, val_k, rev in (("asc_off", "asc", False), ("des_off", "des", True)):
        off, val = m[off_k], m[val_k]
        assert val.max(initial=0) < n, f"{what}: {val_k} value out of range"
        src = np.repeat(np.arange(n, dtype=np.uint32), np.diff(off).astype(np.int64))
        keep = ~(bc[src] | bc[val])
        src, val = src[keep], val[keep]
        h = _mix(val, src) if rev else _mix(src, val)
        with np.errstate(over="ignore"):
            sums.append((int(h.sum(dtype=np.uint64)), len(val)))
    assert sums[0] == sums[1], f"{what}: asc and des lists are not transposes"


def euler(m):
    d = dims(m["cellid"])
    return int((d == 0).sum()) - int((d == 1).sum()) + int((d == 2).sum())


def test_step_4096_quantised_properties(gpu_lib):
    from mscomplex_gb300 import synth
    f = synth.bumps4096q()
    ny, nx = f.shape
    r = (0, 0, 2 * (nx - 1), 2 * (ny - 1))
    outs = []
    for _ in range(2):
        ds = gpu_lib.GridDataset(r, r).init(f).work()
        m = ds.writeout_connectivity()
        ds.post_merge_fill_discs(m)
        outs.append(m.export())
    a, b = outs
    for k in a:
        assert np.array_equal(a[k], b[k]), f"4096q: {k} differs between two runs"
    assert euler(a) == 1
    transpose_check(a, "4096q")
    d = dims(a["cellid"])
    # every vertex in exactly one minimum's asc disc, every face in one maximum's des disc
    for dim, off_k, disc_k, count in ((0, "adisc_off", "adisc", nx * ny), (2, "ddisc_off", "ddisc", (nx - 1) * (ny - 1))):
        sizes = np.diff(a[off_k])[d == dim]
        assert int(sizes.sum()) == count, f"extremum discs of dim {dim} hold {sizes.sum()} cells, not {count}"
        cells = np.concatenate([a[disc_k][a[off_k][i]:a[off_k][i + 1]] for i in np.nonzero(d == dim)[0][:2000]])
        assert len(np.unique(cells.view(np.int32))) == len(cells), "extremum discs overlap"


def test_pipeline_16384_noise_properties(gpu_lib):
    import torch
    from mscomplex_gb300 import synth
    f = torch.from_numpy(synth.noise(16384, seed=2)).cuda()
    p = gpu_lib.GridDataManager(f, levels=8, tresh=0.0, split2d=True)
    n = p.num_pieces
    assert n == 256
    root = p.piece(2 * n - 2).export()
    assert euler(root) == 1
    transpose_check(root, "root")
    # the leaves' extremum discs: every vertex of a leaf's rect in one minimum's disc
    leaf = p.piece(0).export()
    transpose_check(leaf, "leaf 0")
    first = {k: leaf[k].copy() for k in ("cellid", "asc", "des", "adisc", "ddisc")}
    del p
    q = gpu_lib.GridDataManager(f, levels=8, tresh=0.0, split2d=True)
    again = q.piece(0).export()
    for k, v in first.items():
        assert np.array_equal(v, again[k]), f"16384 noise leaf 0: {k} differs between two runs"
    del q
