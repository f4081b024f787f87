"""GPU parity of the persistence simplification (simplify + un_simplify,
dmsc/src/grid_mscomplex.cpp:384-535) against the oracle, bit-exact: flags,
pair_idx and the rebuilt asc/des multisets."""
import numpy as np
import pytest

from helpers import assert_same_complex, full_rect, smooth_field, tie_field

pytestmark = pytest.mark.gpu


def check_simplify(M, oracle, f, tresh, what):
    r = full_rect(f)
    want = oracle.Dataset(f, r, r, tresh=tresh).msc()
    msc = M.GridDataset(r, r).init(f).work().writeout_connectivity()
    stats = msc.simplify_un_simplify(tresh)
    got = msc.export()
    assert_same_complex(got, want, what)
    return stats


@pytest.mark.parametrize("tresh", [0.01, 0.05, 0.2])
def test_simplify_smooth(gpu_lib, oracle, tresh):
    check_simplify(gpu_lib, oracle, smooth_field(90, 110, 11), tresh, f"smooth t={tresh}")


@pytest.mark.parametrize("seed", range(4))
def test_simplify_ties(gpu_lib, oracle, seed):
    f = tie_field(40 + 7 * seed, 50 + 5 * seed, 5, seed)
    check_simplify(gpu_lib, oracle, f, 0.3, f"ties seed={seed}")


@pytest.mark.parametrize("seed", range(2))
@pytest.mark.parametrize("tresh", [0.25, 0.2499])
def test_simplify_threshold_on_a_persistence(gpu_lib, oracle, seed, tresh):
    """Heights on 5 integer levels: persistences are whole numbers and the range
    is 4, so at tresh 0.25 a pair of persistence 1 sits exactly on the stop test
    (persistence / range > tresh, strictly) and is still cancelled, while at
    0.2499 it stops the loop (the oracle cancels 649 / 560 pairs for seed 0)."""
    f = tie_field(40 + 7 * seed, 50 + 5 * seed, 5, seed)
    check_simplify(gpu_lib, oracle, f, tresh, f"ties seed={seed} t={tresh}")


def test_simplify_bumps256(gpu_lib, oracle):
    from mscomplex_gb300 import synth
    check_simplify(gpu_lib, oracle, synth.bumps256(), 0.05, "bumps256 t=0.05")


@pytest.mark.parametrize("n", [256, 384])
def test_simplify_quantized_bumps(gpu_lib, oracle, n):
    """Scaled 4096^2 quantised workload at 1%: strangulation resubmission churn."""
    from mscomplex_gb300 import synth
    st = check_simplify(gpu_lib, oracle, synth.bumps4096q(n=n), 0.01, f"bumps{n}q t=0.01")
    assert st["cancels"] > 0 and st["pushes"] > st["pops"] // 2


@pytest.mark.parametrize("side", [200, 512])
def test_simplify_mixed_grid(gpu_lib, oracle, side):
    from mscomplex_gb300 import synth
    check_simplify(gpu_lib, oracle, synth.mixed_grid(side, seed=side), 0.02, f"mixed{side} t=0.02")


def test_simplify_budget_leaves_complex_unchanged(gpu_lib):
    from mscomplex_gb300 import synth
    f = synth.bumps4096q(n=256)
    r = full_rect(f)
    msc = gpu_lib.GridDataset(r, r).init(f).work().writeout_connectivity()
    before = msc.export()
    with pytest.raises(gpu_lib.DmscError, match="DEVICE_TIMEOUT"):
        msc.simplify_un_simplify(0.01, max_ops=1000)
    assert_same_complex(msc.export(), before, "after a stopped simplification")
