"""CPU check of the exactness argument behind the replay's stop test: the
reference stops at the first pair with (double)d / (double)max_persistence >
tresh (dmsc/src/grid_mscomplex.cpp:446-447).  A correctly rounded division by
a fixed positive divisor is monotone in d, and non-negative finite floats
order like their bit patterns, so the test holds exactly from one bit pattern
on; the replay finds that pattern once by bisection and compares bits per pop.
Restated here with numpy's IEEE double division (correctly rounded, as the
device's) and checked against the direct test on many persistences, including
the patterns next to the boundary."""
import numpy as np
import pytest


def over(u, mp, tresh):
    d = np.array([u], np.uint32).view(np.float32)[0]
    with np.errstate(divide="ignore", invalid="ignore"):  # a zero range: d / 0 is inf or NaN, as in IEEE
        return np.float64(d) / np.float64(mp) > tresh


def stop_bits(mp, tresh):
    lo, hi = 0, 0x7F800001
    while lo < hi:
        mid = lo + (hi - lo) // 2
        if over(mid, mp, tresh):
            hi = mid
        else:
            lo = mid + 1
    return lo


@pytest.mark.parametrize("mp,tresh", [(np.float32(1.3505763), 0.01), (np.float32(4.0), 0.25), (np.float32(3.0), 1 / 3),
                                      (np.float32(0.0), 0.05), (np.float32(7.5e-39), 0.5), (np.float32(3.4e38), 1e-30),
                                      (np.float32(2.0), -1.0), (np.float32(1.0), float("nan"))])
def test_stop_bits_match_the_double_division(mp, tresh):
    rng = np.random.default_rng(5)
    stop = stop_bits(mp, tresh)
    cand = [0, 1, 0x7F7FFFFF, 0x7F800000, stop - 2, stop - 1, stop, stop + 1, stop + 2]
    cand += list(rng.integers(0, 0x7F800000, size=3000))
    # persistences a few steps of the quantisation apart, as on quantised fields
    cand += list(np.arange(1, 9, dtype=np.float32).__mul__(np.float32(mp) / np.float32(256)).view(np.uint32))
    for u in cand:
        u = int(u)
        if not 0 <= u <= 0x7F800000:
            continue
        assert (u >= stop) == bool(over(u, mp, tresh)), (hex(u), float(mp), tresh, hex(stop))
