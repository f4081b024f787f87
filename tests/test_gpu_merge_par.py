"""GPU parity of the parallel piece merges (merge_up / merge_down of
dmsc/src/grid_mscomplex.cpp:24-322 with the union, the connectivity and the
child rewrite spread over the GPU): every tree level forced onto them,
against the oracle's pipeline, node by node, and against the one-thread
merges on larger fields."""
import numpy as np
import pytest

from helpers import assert_same_complex, smooth_field, tie_field

pytestmark = pytest.mark.gpu

GRAPH_KEYS = ("rect_ext", "cellid", "fn", "pair_idx", "flags", "asc_off", "asc", "des_off", "des")


@pytest.fixture(scope="module")
def par_ctx(gpu_lib):
    ctx = gpu_lib.Context()
    ctx.set_merge_parallel_min(0)
    yield ctx
    ctx.close()


@pytest.fixture(scope="module")
def seq_ctx(gpu_lib):
    ctx = gpu_lib.Context()
    ctx.set_merge_parallel_min(1 << 62)
    yield ctx
    ctx.close()


def compare(got, want, what, leaves_full=True):
    N = got.num_pieces
    for i in range(2 * N - 1):
        g = got.piece(i).export()
        w = want.piece(i) if not hasattr(want, "num_pieces") else want.piece(i).export()
        if i < N and leaves_full:
            assert_same_complex(g, w, f"{what} leaf {i}")
        else:
            assert_same_complex(g, w, f"{what} node {i}", keys=GRAPH_KEYS)


def check(M, oracle, ctx, f, levels, tresh, split2d, what):
    want = oracle.Pipeline(f, levels=levels, tresh=tresh, split2d=split2d)
    got = M.GridDataManager(f, levels=levels, tresh=tresh, split2d=split2d, ctx=ctx)
    assert got.num_pieces == want.nleaves
    compare(got, want, what)


@pytest.mark.parametrize("levels", [1, 2, 3])
@pytest.mark.parametrize("split2d", [False, True])
@pytest.mark.parametrize("tresh", [0.0, 0.05])
def test_par_smooth(gpu_lib, oracle, par_ctx, levels, split2d, tresh):
    check(gpu_lib, oracle, par_ctx, smooth_field(70, 90, 5), levels, tresh, split2d,
          f"par smooth L{levels} 2d={split2d} t={tresh}")


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_par_ties(gpu_lib, oracle, par_ctx, seed):
    f = tie_field(40 + 7 * seed, 50 + 5 * seed, 5, seed)
    check(gpu_lib, oracle, par_ctx, f, 2 + seed % 2, 0.05, seed % 2 == 1, f"par ties seed={seed}")


def test_par_bumps256(gpu_lib, oracle, par_ctx):
    from mscomplex_gb300 import synth
    check(gpu_lib, oracle, par_ctx, synth.bumps256(), 3, 0.05, True, "par bumps256 L3")


def test_par_quantized(gpu_lib, oracle, par_ctx):
    from mscomplex_gb300 import synth
    check(gpu_lib, oracle, par_ctx, synth.bumps4096q(n=256), 2, 0.01, False, "par bumps256q L2")


@pytest.mark.parametrize("n,levels", [(64, 2), (128, 4), (256, 4)])
def test_par_noise(gpu_lib, oracle, par_ctx, n, levels):
    from mscomplex_gb300 import synth
    check(gpu_lib, oracle, par_ctx, synth.noise(n, seed=2), levels, 0.0, True, f"par noise{n} L{levels}")


def test_par_noise_simplified(gpu_lib, oracle, par_ctx):
    from mscomplex_gb300 import synth
    check(gpu_lib, oracle, par_ctx, synth.noise(96, seed=5), 3, 0.02, False, "par noise96 L3 t=0.02")


@pytest.mark.parametrize("n,levels,split2d", [(512, 3, True), (384, 2, False)])
def test_par_equals_sequential(gpu_lib, par_ctx, seq_ctx, n, levels, split2d):
    """Larger noise fields: the parallel merges against the one-thread merges."""
    from mscomplex_gb300 import synth
    f = synth.noise(n, seed=9)
    a = gpu_lib.GridDataManager(f, levels=levels, tresh=0.0, split2d=split2d, ctx=par_ctx)
    b = gpu_lib.GridDataManager(f, levels=levels, tresh=0.0, split2d=split2d, ctx=seq_ctx)
    compare(a, b, f"noise{n} par vs seq")


@pytest.mark.parametrize("shape,levels,split2d", [((9, 7), 2, True), ((12, 40), 2, False), ((33, 5), 2, True),
                                                   ((17, 17), 3, True), ((40, 9), 3, False)])
def test_par_thin_and_tiny(gpu_lib, oracle, par_ctx, shape, levels, split2d):
    """Pieces only a few vertices wide (shared boundaries next to the outer one)."""
    f = smooth_field(shape[0], shape[1], 11)
    check(gpu_lib, oracle, par_ctx, f, levels, 0.05, split2d, f"par tiny {shape} L{levels}")


@pytest.mark.parametrize("kind", ["constant", "ramp", "checker"])
def test_par_degenerate_fields(gpu_lib, oracle, par_ctx, kind):
    ny, nx = 40, 56
    y, x = np.mgrid[0:ny, 0:nx]
    if kind == "constant":
        f = np.zeros((ny, nx), np.float32)
    elif kind == "ramp":
        f = (x + 0.5 * y).astype(np.float32)
    else:
        f = ((x + y) % 2).astype(np.float32)
    check(gpu_lib, oracle, par_ctx, f, 2, 0.1, True, f"par {kind}")


def test_par_too_thin_pieces_fail_like_the_reference(gpu_lib, oracle, par_ctx):
    """Strips one or two rows high break a reference invariant (its logic_error); both report it."""
    f = smooth_field(6, 40, 11)
    with pytest.raises(RuntimeError):
        oracle.Pipeline(f, levels=3, tresh=0.05, split2d=False)
    with pytest.raises(gpu_lib.DmscError):
        gpu_lib.GridDataManager(f, levels=3, tresh=0.05, split2d=False, ctx=par_ctx)


# merge_up's boundary cancellations in ordered-parallel rounds: every setting
# of the rounds (window, hand-off rate) against the oracle, node by node.
# window 0 runs the loop on one thread per merge; min_commits far above any
# round's commits makes the rounds hand the rest to the in-order thread after
# 8 rounds, so the finishing path runs on every merge with a boundary longer
# than 8 windows; window 1 takes one task per round.
ROUND_SETTINGS = [(2048, 4), (0, 0), (16, 1 << 30), (64, 1 << 30), (1, 0), (3, 2)]


@pytest.fixture(scope="module", params=ROUND_SETTINGS, ids=lambda s: f"win{s[0]}-min{s[1]}")
def rounds_ctx(gpu_lib, request):
    ctx = gpu_lib.Context()
    ctx.set_merge_parallel_min(0)
    ctx.set_merge_rounds(*request.param)
    yield ctx
    ctx.close()


def test_rounds_bumps256(gpu_lib, oracle, rounds_ctx):
    """A smooth field: large extrema sit in most footprints, so groups stay large."""
    from mscomplex_gb300 import synth
    check(gpu_lib, oracle, rounds_ctx, synth.bumps256(), 3, 0.05, True, "rounds bumps256 L3")


def test_rounds_noise(gpu_lib, oracle, rounds_ctx):
    from mscomplex_gb300 import synth
    check(gpu_lib, oracle, rounds_ctx, synth.noise(256, seed=3), 4, 0.0, True, "rounds noise256 L4")


def test_rounds_quantized(gpu_lib, oracle, rounds_ctx):
    from mscomplex_gb300 import synth
    check(gpu_lib, oracle, rounds_ctx, synth.bumps4096q(n=256), 2, 0.01, False, "rounds bumps256q L2")


def test_rounds_settings_rejected(gpu_lib):
    ctx = gpu_lib.Context()
    with pytest.raises(gpu_lib.DmscError):
        ctx.set_merge_rounds(-1, 4)
    with pytest.raises(gpu_lib.DmscError):
        ctx.set_merge_rounds(16, -2)
    ctx.close()
