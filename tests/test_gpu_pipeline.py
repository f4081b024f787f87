"""GPU parity of the whole piece pipeline (GridDataManager,
dmsc/src/grid_datamanager.cpp:596-662) against the oracle: every node of the
piece tree after merge_up, root simplification and merge_down (the merges of
dmsc/src/grid_mscomplex.cpp:24-322), the discs of every leaf, and the disc
files written by all leaves in order."""
import numpy as np
import pytest

from helpers import assert_same_complex, smooth_field, tie_field

pytestmark = pytest.mark.gpu

GRAPH_KEYS = ("rect_ext", "cellid", "fn", "pair_idx", "flags", "asc_off", "asc", "des_off", "des")


def check_pipeline(M, oracle, f, levels, tresh, split2d, what):
    want = oracle.Pipeline(f, levels=levels, tresh=tresh, split2d=split2d)
    got = M.GridDataManager(f, levels=levels, tresh=tresh, split2d=split2d)
    N = got.num_pieces
    assert N == want.nleaves == 2 ** levels
    for i in range(2 * N - 1):
        g, w = got.piece(i).export(), want.piece(i)
        if i < N:
            assert_same_complex(g, w, f"{what} leaf {i}")
        else:
            assert_same_complex(g, w, f"{what} node {i}", keys=GRAPH_KEYS)
            assert len(g["adisc"]) == 0 and len(g["ddisc"]) == 0
    return got, want


@pytest.mark.parametrize("levels", [1, 2, 3])
@pytest.mark.parametrize("split2d", [False, True])
@pytest.mark.parametrize("tresh", [0.0, 0.05])
def test_pipeline_smooth(gpu_lib, oracle, levels, split2d, tresh):
    check_pipeline(gpu_lib, oracle, smooth_field(70, 90, 5), levels, tresh, split2d,
                   f"smooth L{levels} 2d={split2d} t={tresh}")


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_pipeline_ties(gpu_lib, oracle, seed):
    f = tie_field(40 + 7 * seed, 50 + 5 * seed, 5, seed)
    check_pipeline(gpu_lib, oracle, f, 2, 0.05, seed % 2 == 1, f"ties seed={seed}")


def test_pipeline_bumps256(gpu_lib, oracle):
    from mscomplex_gb300 import synth
    check_pipeline(gpu_lib, oracle, synth.bumps256(), 3, 0.05, True, "bumps256 L3")


def test_pipeline_quantized(gpu_lib, oracle):
    from mscomplex_gb300 import synth
    check_pipeline(gpu_lib, oracle, synth.bumps4096q(n=256), 2, 0.01, False, "bumps256q L2")


def test_pipeline_level0_matches_single_piece(gpu_lib, oracle):
    f = smooth_field(60, 50, 3)
    check_pipeline(gpu_lib, oracle, f, 0, 0.05, False, "L0")


def test_pipeline_device_input(gpu_lib, oracle):
    import torch
    f = smooth_field(80, 64, 7)
    want = oracle.Pipeline(f, levels=2, tresh=0.02, split2d=True)
    t = torch.from_numpy(f).cuda()
    got = gpu_lib.GridDataManager(t, levels=2, tresh=0.02, split2d=True)
    for i in range(got.num_pieces):
        assert_same_complex(got.piece(i).export(), want.piece(i), f"device input leaf {i}")


def test_pipeline_write_discs(gpu_lib, oracle, tmp_path):
    from mscomplex_gb300 import synth
    f = synth.bumps256()
    got = gpu_lib.GridDataManager(f, levels=2, tresh=0.05, split2d=True)
    got.write_discs(str(tmp_path / "p__disc_"))
    want = oracle.Pipeline(f, levels=2, tresh=0.05, split2d=True).disc_files()
    files = {}
    for p in tmp_path.iterdir():
        name = p.name[len("p__disc_"):]
        kind = 0 if name.startswith("asc_") else 1
        x, y = (int(v) for v in name[5:-1].split(","))
        files[(kind, x, y)] = np.fromfile(p, np.int16).reshape(-1, 2)
    assert set(files) == set(want)
    for k in want:
        assert np.array_equal(files[k], want[k]), k


def test_pipeline_bad_args(gpu_lib):
    f = smooth_field(20, 20, 1)
    with pytest.raises(gpu_lib.DmscError):
        gpu_lib.GridDataManager(f, levels=-1)
    with pytest.raises(gpu_lib.DmscError):
        gpu_lib.GridDataManager(f[:1], levels=0)


def test_cli_matches_oracle_discs(gpu_lib, oracle, tmp_path):
    from mscomplex_gb300.__main__ import main
    from mscomplex_gb300 import synth
    f = synth.bumps256()
    raw = tmp_path / "f.raw"
    f.tofile(raw)
    out = tmp_path / "out"
    assert main(["-gf", str(raw), "-d", "256", "256", "-l", "2", "--simp-tresh", "0.05", "--outdir", str(out)]) == 0
    want = oracle.Pipeline(f, levels=2, tresh=0.05, split2d=False).disc_files()
    files = {}
    for p in out.iterdir():
        name = p.name[len("dp__disc_"):]
        kind = 0 if name.startswith("asc_") else 1
        x, y = (int(v) for v in name[5:-1].split(","))
        files[(kind, x, y)] = np.fromfile(p, np.int16).reshape(-1, 2)
    assert set(files) == set(want)
    for k in want:
        assert np.array_equal(files[k], want[k]), k
