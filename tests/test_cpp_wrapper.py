"""CPU checks of the header-only C++ wrapper include/dmsc.hpp: it compiles
against dmsc.h and links with libdmsc.so, a status code becomes the
reference's exception type (std::logic_error for an invariant, else
std::runtime_error) with the library's message, and handles move without
being destroyed twice.  No GPU work: the calls fail on empty handles, and the
context either opens (GPU present) or fails with the library's message."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include "dmsc.hpp"
#include <cstdio>
#include <string>
#include <utility>

static int fails = 0;
static void expect(bool ok, const char *what) {
  if (!ok) { std::printf("FAIL %s\n", what); ++fails; }
}

int main() {
  using namespace dmsc_cxx;
  check(DMSC_OK);
  try { check(DMSC_ERR_INVARIANT); expect(false, "an invariant status throws"); }
  catch (const std::logic_error &e) { expect(dynamic_cast<const logic_error *>(&e) != nullptr, "logic_error type"); }
  catch (...) { expect(false, "an invariant is a std::logic_error"); }
  for (int rc : {DMSC_ERR_BAD_ARG, DMSC_ERR_OOM, DMSC_ERR_CUDA, DMSC_ERR_INT16_OVERFLOW, DMSC_ERR_DEVICE_TIMEOUT,
                 DMSC_ERR_INPUT, DMSC_ERR_STATE, DMSC_ERR_PARTIAL}) {
    try { check(rc); expect(false, "an error status throws"); }
    catch (const runtime_error &e) { expect(e.code() == rc, "runtime_error carries the code"); }
    catch (...) { expect(false, "other errors are std::runtime_error"); }
  }

  // real failures through the C ABI, with the library's own message
  GridMSComplex m;
  expect(m.empty(), "a new complex is empty");
  try { m.sizes(); expect(false, "sizes of an empty complex throw"); }
  catch (const runtime_error &e) {
    expect(e.code() == DMSC_ERR_BAD_ARG, "empty complex: bad argument");
    expect(std::string(e.what()).find("null") != std::string::npos, "empty complex: message from the library");
  }
  try { m.simplify_un_simplify(0.1); expect(false, "simplify of an empty complex throws"); }
  catch (const runtime_error &e) { expect(e.code() == DMSC_ERR_BAD_ARG, "simplify: bad argument"); }
  try { m.write_discs("unused_prefix_"); expect(false, "write_discs of an empty complex throws"); }
  catch (const runtime_error &e) { expect(e.code() == DMSC_ERR_BAD_ARG, "write_discs: bad argument"); }
  try { (void)m.data(); expect(false, "export of an empty complex throws"); }
  catch (const std::runtime_error &) {}

  // move-only handles: an empty one moves without a destroy call
  GridMSComplex a;
  GridMSComplex b(std::move(a));
  a = std::move(b);
  expect(a.empty() && b.empty(), "moves of an empty complex");

  // the context: opens with a GPU, otherwise a runtime_error with the library's message
  try { Context ctx(0); Context moved(std::move(ctx)); expect(ctx.get() == nullptr, "a moved context is empty"); }
  catch (const runtime_error &e) {
    expect(std::string(e.what()).size() > 0, "context failure has a message");
    expect(e.code() == DMSC_ERR_CUDA || e.code() == DMSC_ERR_BAD_ARG, "context failure code");
  }
  try { Context ctx(1 << 20); expect(false, "a device index beyond the devices throws"); }
  catch (const runtime_error &) {}

  std::printf(fails ? "FAILED\n" : "OK\n");
  return fails != 0;
}
"""


def test_cpp_wrapper(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    from mscomplex_gb300 import build
    lib = build.build()
    libdir = os.path.dirname(lib)
    src = tmp_path / "wrapper_check.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "wrapper_check"
    cmd = [gxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe),
           "-L" + libdir, "-ldmsc", "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr
