"""GPU check of the C++ wrapper include/dmsc.hpp: a program built against it
runs GridDataset (work, writeout_connectivity twice -- new, then in place --
postMergeFillDiscs, cell and critical-cell exports) and GridDataManager
(2 levels) on a small field, and every array it exports equals the one the
Python binding exports for the same field (the binding's parity with the
oracle is covered by the other gpu tests)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from helpers import full_rect, smooth_field

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = ("cellid", "fn", "pair_idx", "flags", "asc_off", "asc", "des_off", "des", "adisc_off", "adisc", "ddisc_off",
        "ddisc")

PROGRAM = r"""
#include "dmsc.hpp"
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

template <class T> static void dump(const std::string &path, const std::vector<T> &v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}
static void dump_all(const std::string &p, const dmsc_cxx::MSComplexData &d) {
  dump(p + "cellid.bin", d.cellid); dump(p + "fn.bin", d.fn); dump(p + "pair_idx.bin", d.pair_idx);
  dump(p + "flags.bin", d.flags); dump(p + "asc_off.bin", d.asc_off); dump(p + "asc.bin", d.asc);
  dump(p + "des_off.bin", d.des_off); dump(p + "des.bin", d.des); dump(p + "adisc_off.bin", d.adisc_off);
  dump(p + "adisc.bin", d.adisc); dump(p + "ddisc_off.bin", d.ddisc_off); dump(p + "ddisc.bin", d.ddisc);
}

int main(int argc, char **argv) {
  if (argc != 5) return 2;
  const std::string in = argv[1], out = argv[4];
  const int nx = std::stoi(argv[2]), ny = std::stoi(argv[3]);
  std::vector<float> h((size_t)nx * ny);
  std::ifstream f(in, std::ios::binary);
  f.read(reinterpret_cast<char *>(h.data()), (std::streamsize)(h.size() * sizeof(float)));
  if (!f) return 3;
  try {
    dmsc_cxx::Context ctx(0);
    const dmsc_cxx::rect_t r{0, 0, (int16_t)(2 * (nx - 1)), (int16_t)(2 * (ny - 1))};
    dmsc_cxx::GridDataset ds(ctx, r, r);
    ds.init(h.data());
    ds.work();
    dmsc_cxx::GridMSComplex m = ds.writeout_connectivity();
    ds.writeout_connectivity(m);  // in place, reusing its buffers
    ds.postMergeFillDiscs(m);
    dump_all(out + "/ds_", m.data());
    dump(out + "/ds_critical.bin", ds.critical_cells());
    std::vector<int8_t> flags;
    std::vector<int16_t> pairs, own;
    ds.export_cells(&flags, &pairs, &own);
    dump(out + "/ds_cellflags.bin", flags);
    dump(out + "/ds_cellpairs.bin", pairs);
    dump(out + "/ds_cellown.bin", own);
    dmsc_cxx::GridDataManager p(ctx, h.data(), nx, ny, 2, 0.0);
    const int64_t np = p.num_pieces();
    dump_all(out + "/root_", p.piece(2 * np - 2));
    dump_all(out + "/leaf0_", p.piece(0));
    std::printf("OK %lld\n", (long long)np);
  } catch (const std::exception &e) {
    std::printf("EXC %s\n", e.what());
    return 1;
  }
  return 0;
}
"""


def compare(tmp_path, prefix, want, what):
    for k in KEYS:
        got = np.fromfile(tmp_path / f"{prefix}{k}.bin", dtype=want[k].dtype)
        assert np.array_equal(got, want[k].reshape(-1)), f"{what}: {k} differs"


def test_cpp_wrapper_matches_python_binding(gpu_lib, tmp_path):
    M = gpu_lib
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    from mscomplex_gb300 import build
    libdir = os.path.dirname(build.build())
    src = tmp_path / "wrapper_gpu.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "wrapper_gpu"
    r = subprocess.run([gxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"), str(src),
                        "-o", str(exe), "-L" + libdir, "-ldmsc", "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    f = smooth_field(48, 64, 7)
    ny, nx = f.shape
    f.tofile(tmp_path / "h.bin")
    r = subprocess.run([str(exe), str(tmp_path / "h.bin"), str(nx), str(ny), str(tmp_path)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr

    rect = full_rect(f)
    ds = M.GridDataset(rect, rect).init(f).work()
    m = ds.writeout_connectivity()
    ds.post_merge_fill_discs(m)
    compare(tmp_path, "ds_", m.export(), "dataset complex")
    assert np.array_equal(np.fromfile(tmp_path / "ds_critical.bin", np.int16), ds.critical_cells().reshape(-1))
    fl, pa, ow = ds.cells()
    assert np.array_equal(np.fromfile(tmp_path / "ds_cellflags.bin", np.int8), fl.reshape(-1))
    assert np.array_equal(np.fromfile(tmp_path / "ds_cellpairs.bin", np.int16), pa.reshape(-1))
    assert np.array_equal(np.fromfile(tmp_path / "ds_cellown.bin", np.int16), ow.reshape(-1))

    p = M.GridDataManager(f, levels=2, tresh=0.0)
    assert r.stdout.split()[1] == str(p.num_pieces)
    compare(tmp_path, "root_", p.piece(2 * p.num_pieces - 2).export(), "pipeline root")
    compare(tmp_path, "leaf0_", p.piece(0).export(), "pipeline leaf 0")
