"""Out of core: complexes to archive files and back (dmsc_msc_save / load,
standing in for write_msgraph_to_archive / read_msgraph_from_archive,
dmsc/src/grid_datamanager.cpp:91-119), and the piece pipeline with its
pieces' complexes kept in archives between stages (GridDataManager's
compute_out_of_core), which must give the in-memory pipeline's results --
themselves checked against the oracle -- node by node."""
import os

import numpy as np
import pytest

from helpers import COMPLEX_KEYS, assert_same_complex, full_rect, smooth_field

pytestmark = pytest.mark.gpu


def test_save_load_round_trip(gpu_lib, tmp_path):
    from mscomplex_gb300 import synth
    f = synth.bumps256()
    r = full_rect(f)
    ds = gpu_lib.GridDataset(r, r).init(f).work()
    m = ds.writeout_connectivity()
    ds.post_merge_fill_discs(m)
    m.simplify_un_simplify(0.05)
    p = str(tmp_path / "a.msc")
    m.save(p)
    back = gpu_lib.GridMSComplex.load(p)
    assert_same_complex(back.export(), m.export(), "round trip")
    # a complex without discs
    m2 = ds.writeout_connectivity()
    m2.save(p)
    assert_same_complex(gpu_lib.GridMSComplex.load(p).export(), m2.export(), "round trip, no discs")


def test_load_rejects_other_files(gpu_lib, tmp_path):
    p = tmp_path / "junk"
    p.write_bytes(b"not an archive at all" * 4)
    with pytest.raises(gpu_lib.DmscError):
        gpu_lib.GridMSComplex.load(str(p))
    with pytest.raises(gpu_lib.DmscError):
        gpu_lib.GridMSComplex.load(str(tmp_path / "missing"))


@pytest.mark.parametrize("levels,split2d,tresh", [(1, False, 0.0), (2, True, 0.05), (3, True, 0.02)])
def test_out_of_core_pipeline_equals_in_memory(gpu_lib, oracle, tmp_path, levels, split2d, tresh):
    from mscomplex_gb300 import synth
    f = synth.bumps4096q(n=192) if levels == 3 else smooth_field(90, 110, levels)
    ctx = gpu_lib.Context()
    ctx.set_merge_parallel_min(0)
    ctx.set_out_of_core(str(tmp_path))
    got = gpu_lib.GridDataManager(f, levels=levels, tresh=tresh, split2d=split2d, ctx=ctx)
    assert len(os.listdir(tmp_path)) == 2 * got.num_pieces - 1  # every node archived after the run
    want = gpu_lib.GridDataManager(f, levels=levels, tresh=tresh, split2d=split2d)
    orc = oracle.Pipeline(f, levels=levels, tresh=tresh, split2d=split2d)
    N = got.num_pieces
    for i in range(2 * N - 1):
        g = got.piece(i).export()
        keys = COMPLEX_KEYS if i < N else COMPLEX_KEYS[:9]
        assert_same_complex(g, want.piece(i).export(), f"ooc L{levels} node {i} vs in memory", keys=keys)
        assert_same_complex(g, orc.piece(i), f"ooc L{levels} node {i} vs oracle", keys=keys)
    d1, d2 = tmp_path / "discs_ooc", tmp_path / "discs_mem"
    d1.mkdir()
    d2.mkdir()
    got.write_discs(str(d1) + "/dp__disc_")
    want.write_discs(str(d2) + "/dp__disc_")
    names = sorted(os.listdir(d1))
    assert names == sorted(os.listdir(d2)) and names
    for n in names:
        assert (d1 / n).read_bytes() == (d2 / n).read_bytes(), n
    del got
    assert not [n for n in os.listdir(tmp_path) if n.startswith("dp_msgraph_")], "archives left behind"
    ctx.close()


def test_out_of_core_without_levels_stays_in_memory(gpu_lib, tmp_path):
    f = smooth_field(40, 50, 3)
    ctx = gpu_lib.Context()
    ctx.set_out_of_core(str(tmp_path))
    p = gpu_lib.GridDataManager(f, levels=0, tresh=0.05, ctx=ctx)
    assert os.listdir(tmp_path) == []
    want = gpu_lib.GridDataManager(f, levels=0, tresh=0.05)
    assert_same_complex(p.piece(0).export(), want.piece(0).export(), "levels 0")
    del p
    ctx.close()
