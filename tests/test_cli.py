"""The command line mirrors the reference's flags (dmsc/src/main.cpp:14-29,
140-232); parsing and the raw loader need no GPU."""
import numpy as np
import pytest

from mscomplex_gb300.__main__ import load_raw, parse


def test_parse_reference_flags():
    a = parse(["-gf", "data.raw", "-d", "64", "32", "-l", "3", "--simp-tresh", "0.05", "-st", "--num-parallel", "4"])
    assert a.file == "data.raw" and a.dims == [64, 32] and a.levels == 3 and a.tresh == 0.05
    assert a.st and a.num_parallel == 4 and not a.split2d


def test_parse_rejects(capsys):
    with pytest.raises(SystemExit):
        parse(["-d", "4", "4"])  # no file
    with pytest.raises(SystemExit):
        parse(["-gf", "f", "-d", "1", "4"])
    with pytest.raises(SystemExit):
        parse(["-gf", "f", "-d", "4", "4", "-l", "-1"])


def test_parse_backend_and_out_of_core_flags():
    a = parse(["-gf", "f", "-d", "8", "8", "-ocl", "--out-of-core", "--outdir", "/tmp/x"])
    assert a.ocl and a.out_of_core and a.outdir == "/tmp/x"


def test_load_raw(tmp_path):
    f = np.arange(6 * 4, dtype=np.float32).reshape(4, 6)
    p = tmp_path / "g.raw"
    f.tofile(p)
    g = load_raw(str(p), 6, 4)
    assert np.array_equal(f, g)
    with pytest.raises(ValueError):
        load_raw(str(p), 7, 4)
