"""CPU check of the rule behind the device's ordered-parallel boundary rounds
(k_merge_up_rounds): on the oracle's complexes of two noise pieces, the rounds
schedule -- and the same schedule cut short by a work budget and finished in
order -- leaves the graph merge_up's row-major loop leaves."""
import copy

import pytest

from rounds_model import Rect, run, run_rounds, same, tasks, union


def two_pieces(oracle, field):
    P = oracle.Pipeline(field, levels=1)
    re = [P.piece(i)["rect_ext"] for i in range(3)]
    ds = []
    for i in range(2):
        r, e = re[i][:4], re[i][4:]
        ds.append(oracle.Dataset(field[e[1] // 2:e[3] // 2 + 1, e[0] // 2:e[2] // 2 + 1], r, e).msc())
    rr = [Rect(*re[i][:4]) for i in range(2)]
    ixn = Rect(max(rr[0].l, rr[1].l), max(rr[0].b, rr[1].b), min(rr[0].r, rr[1].r), min(rr[0].t, rr[1].t))
    return union(ds[0], ds[1], ixn), Rect(*re[2][:4]), Rect(*re[2][4:]), ixn


@pytest.mark.parametrize("n,seed", [(96, 2), (128, 5), (160, 7)])
def test_rounds_leave_the_loop_result(oracle, n, seed):
    from mscomplex_gb300 import synth
    G0, rect, ext, ixn = two_pieces(oracle, synth.noise(n, seed=seed))
    T = tasks(G0, rect, ext, ixn)
    assert sum(1 for t in T if t[1] is not None) > 50
    seq = copy.deepcopy(G0)
    for t in T:
        run(seq, t)
    par = copy.deepcopy(G0)
    rounds = run_rounds(par, T)
    assert same(par, seq)
    assert rounds < len(T)
    cut = copy.deepcopy(G0)  # stopped after a few rounds' work, then in order
    run_rounds(cut, T, budget=3 * len(T))
    assert same(cut, seq)


def test_rounds_on_a_smooth_field(oracle):
    from helpers import smooth_field
    G0, rect, ext, ixn = two_pieces(oracle, smooth_field(90, 120, 4))
    T = tasks(G0, rect, ext, ixn)
    seq = copy.deepcopy(G0)
    for t in T:
        run(seq, t)
    par = copy.deepcopy(G0)
    run_rounds(par, T)
    assert same(par, seq)


@pytest.mark.parametrize("n,seed", [(96, 2), (128, 5)])
def test_down_rounds_leave_the_loop_result(oracle, n, seed):
    """merge_down's uncancellation in the same rounds (footprint: the pair, its
    neighbours and their partners) on the parent that merge_up's loop leaves."""
    from mscomplex_gb300 import synth
    from rounds_model import down_tasks, run_down, run_down_rounds
    G, rect, ext, ixn = two_pieces(oracle, synth.noise(n, seed=seed))
    for t in tasks(G, rect, ext, ixn):
        run(G, t)
    T = down_tasks(G, rect, ext, ixn)
    seq = copy.deepcopy(G)
    for t in T:
        run_down(seq, t)
    par = copy.deepcopy(G)
    run_down_rounds(par, T)
    assert same(par, seq)
