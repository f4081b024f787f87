"""CPU check, on the oracle's gradients, of the step encoding behind the disc
walks (successor words of the hop kernel): a chain step of postMergeFillDiscs
(dmsc/src/grid_dataset.cpp:1190-1228) goes from an edge paired with a face
(asc) or a vertex (des) to the edge paired with the cofacet or facet it
crosses, which is one of six neighbours: the four diagonal ones, or the two
2 cells away along y for an asc horizontal edge or a des vertical edge and
along x otherwise.  The successor has the same kind as the edge."""
import numpy as np
import pytest

from helpers import full_rect, smooth_field, tie_field

PAIRED, CRITICAL = 1, 2


def chain_steps(oracle, f):
    """(kind, rx, ry, dx, dy, successor kind) of every chain step of a grid."""
    r = full_rect(f)
    flags, pairs, _ = oracle.Dataset(f, r, r).cells()
    nx, ny = flags.shape
    out = []
    for x in range(nx):
        for y in range(ny):
            if ((x & 1) + (y & 1)) != 1:
                continue  # edges only
            fl = flags[x, y]
            if (fl & CRITICAL) or not (fl & PAIRED):
                continue
            px, py = pairs[x, y]
            kind = 0 if ((px & 1) + (py & 1)) == 2 else 1  # paired with a face: asc
            d0, d1 = x & 1, y & 1
            cands = [(x + d1, y + d0), (x - d1, y - d0)] if kind == 0 else [(x + d0, y + d1), (x - d0, y - d1)]
            for qx, qy in cands:
                if not (0 <= qx < nx and 0 <= qy < ny):
                    continue
                qf = flags[qx, qy]
                if (qf & CRITICAL) or not (qf & PAIRED):
                    continue
                sx, sy = pairs[qx, qy]
                if (sx, sy) == (x, y):
                    continue
                sf = flags[sx, sy]
                spx, spy = pairs[sx, sy]
                skind = None
                if not (sf & CRITICAL) and (sf & PAIRED):
                    skind = 0 if ((spx & 1) + (spy & 1)) == 2 else 1
                out.append((kind, x, y, int(sx) - x, int(sy) - y, skind))
    return out


@pytest.mark.parametrize("what", ["ties", "smooth", "bumps"])
def test_chain_steps_fit_the_three_bit_codes(oracle, what):
    from mscomplex_gb300 import synth
    f = {"ties": tie_field(61, 53, 4, 3), "smooth": smooth_field(70, 64, 2),
         "bumps": np.ascontiguousarray(synth.bumps4096q(n=96))}[what]
    steps = chain_steps(oracle, f)
    assert len(steps) > 1000
    for kind, x, y, dx, dy, skind in steps:
        axis_y = (x & 1) == (1 if kind == 0 else 0)  # an H edge has an odd x
        diagonal = abs(dx) == 1 and abs(dy) == 1
        axis = (dx == 0 and abs(dy) == 2 and axis_y) or (dy == 0 and abs(dx) == 2 and not axis_y)
        assert diagonal or axis, (what, kind, x, y, dx, dy)
        if skind is not None:
            assert skind == kind, (what, kind, x, y, dx, dy)
