"""GPU parity of the manifold discs (postMergeFillDiscs, dmsc/src/grid_dataset.cpp:
1044-1231) against the oracle: every asc/des disc, cell by cell and in order."""
import numpy as np
import pytest

from helpers import assert_same_complex, full_rect, smooth_field, tie_field

pytestmark = pytest.mark.gpu


def check_discs(M, oracle, f, tresh, what):
    r = full_rect(f)
    want = oracle.Dataset(f, r, r, tresh=tresh, fill_discs=True).msc()
    ds = M.GridDataset(r, r).init(f).work()
    msc = ds.writeout_connectivity()
    if tresh > 0:
        msc.simplify_un_simplify(tresh)
    ds.post_merge_fill_discs(msc)
    assert_same_complex(msc.export(), want, what)


@pytest.mark.parametrize("tresh", [0.0, 0.05, 0.3])
def test_discs_smooth(gpu_lib, oracle, tresh):
    check_discs(gpu_lib, oracle, smooth_field(70, 90, 5), tresh, f"smooth t={tresh}")


# (seed, threshold) pairs whose reference discs stay bounded: on tie fields
# un_simplify multiplies arc multiplicities, and postMergeFillDiscs pushes a
# cancelled saddle once per occurrence (seed 2 at 0.1 yields 617K disc cells;
# seed 1 at 0.1 exhausts gigabytes in the reference algorithm itself).
@pytest.mark.parametrize("seed,tresh", [(0, 0.05), (1, 0.05), (2, 0.05), (0, 0.25), (2, 0.1)])
def test_discs_ties(gpu_lib, oracle, seed, tresh):
    check_discs(gpu_lib, oracle, tie_field(30 + 9 * seed, 41 + 4 * seed, 4, seed), tresh, f"ties seed={seed} t={tresh}")


def test_discs_bumps256(gpu_lib, oracle):
    from mscomplex_gb300 import synth
    check_discs(gpu_lib, oracle, synth.bumps256(), 0.0, "bumps256")


def test_discs_quantized_simplified(gpu_lib, oracle):
    from mscomplex_gb300 import synth
    check_discs(gpu_lib, oracle, synth.bumps4096q(n=256), 0.01, "bumps256q t=0.01")


def _bumps(ny, nx, bumps):
    y, x = np.mgrid[0:ny, 0:nx].astype(np.float64)
    f = np.zeros((ny, nx))
    for cx, cy, s, amp in bumps:
        f += amp * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * s * s))
    return f.astype(np.float32)


@pytest.mark.parametrize("name,bumps,tresh", [
    ("one bump", [(140.3, 121.7, 60.0, 1.0)], 0.0),
    ("two bumps", [(80.3, 121.7, 40.0, 1.0), (220.3, 131.7, 35.0, 0.8)], 0.0),
    ("two bumps simplified", [(80.3, 121.7, 40.0, 1.0), (220.3, 131.7, 35.0, 0.8)], 0.5),
])
def test_discs_few_critical_points(gpu_lib, oracle, name, bumps, tresh):
    """Smooth 257x301 fields with 9-15 critical points and about 78K cells in each
    disc array: fewer critical points than 8192-position windows of the saddle
    placement, and long chains crossing many tiles."""
    check_discs(gpu_lib, oracle, _bumps(257, 301, bumps), tresh, name)


def test_discs_multi_tile(gpu_lib, oracle):
    check_discs(gpu_lib, oracle, smooth_field(150, 133, 9), 0.02, "smooth 150x133 t=0.02")


def test_write_discs_files(gpu_lib, oracle, tmp_path):
    from mscomplex_gb300 import synth
    f = synth.bumps256()
    r = full_rect(f)
    ds = gpu_lib.GridDataset(r, r).init(f).work()
    msc = ds.writeout_connectivity()
    msc.simplify_un_simplify(0.05)
    ds.post_merge_fill_discs(msc)
    msc.write_discs(str(tmp_path / "dp__disc_"))
    P = oracle.Pipeline(f, levels=0, tresh=0.05)
    want = P.disc_files()
    got = {}
    for p in tmp_path.iterdir():
        name = p.name[len("dp__disc_"):]
        kind = 0 if name.startswith("asc_") else 1
        x, y = (int(v) for v in name[5:-1].split(","))
        got[(kind, x, y)] = np.fromfile(p, np.int16).reshape(-1, 2)
    assert set(got) == set(want)
    for k in want:
        assert np.array_equal(got[k], want[k]), k


def test_export_async_overlapping_next_grid(gpu_lib, oracle):
    """export(wait=False): each grid's device-to-host copies run on a copy
    stream while the next grid computes; two complexes and two pinned buffer
    sets alternate, a complex is rewritten only after its previous copies are
    done.  Every result equals the oracle's complex with discs."""
    import torch
    fields = [smooth_field(70, 90, s) for s in range(4)]
    r = full_rect(fields[0])
    want = [oracle.Dataset(f, r, r, fill_discs=True).msc() for f in fields]
    ds = gpu_lib.GridDataset(r, r)
    need = {}
    for f in fields:  # buffer sizes: the largest result per key
        m = ds.init(f).work().writeout_connectivity()
        ds.post_merge_fill_discs(m)
        for k, (shape, dt) in m.export_shapes().items():
            need[k] = max(need.get(k, 0), int(np.prod(shape)) * np.dtype(dt).itemsize)
    pinned = [{k: torch.empty(n + 64, dtype=torch.uint8).pin_memory().numpy() for k, n in need.items()}
              for _ in range(2)]
    comp, cp = torch.cuda.Stream(), torch.cuda.Stream()
    slots, freed, outs = [None, None], [None, None], [None] * len(fields)
    for i, f in enumerate(fields):
        k = i & 1
        ds.init(f, stream=comp.cuda_stream).work(stream=comp.cuda_stream)
        if freed[k] is not None:
            comp.wait_event(freed[k])
        m = slots[k] = ds.writeout_connectivity(slots[k], stream=comp.cuda_stream)
        ds.post_merge_fill_discs(m, stream=comp.cuda_stream)
        cp.wait_event(comp.record_event())
        outs[i] = m.export(pinned[k], stream=cp.cuda_stream, wait=False)
        freed[k] = cp.record_event()
        if i > 0:  # the previous grid's buffers are read before the next export reuses them
            freed[1 - k].synchronize()
            assert_same_complex(outs[i - 1], want[i - 1], f"grid {i - 1}")
    freed[(len(fields) - 1) & 1].synchronize()
    assert_same_complex(outs[-1], want[-1], f"grid {len(fields) - 1}")
    with pytest.raises(ValueError):
        slots[0].export(None, wait=False)
