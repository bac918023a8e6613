"""The library's netCDF classic writer and reader (umwm_gb300/csrc/ncfile.cpp)
on the CPU: a small driver compiled here with g++ writes fixed-size, integer
and record variables (several records), scipy's independent netCDF-3 reader
reads them back, and the library's reader reads a file scipy wrote."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "umwm_gb300", "csrc")

DRIVER = r"""
#include "ncfile.hpp"
#include <cstdio>
#include <cstring>
using namespace umwm;
int main(int argc, char** argv) {
  std::string err;
  if (argc > 2 && std::strcmp(argv[1], "read") == 0) {
    std::vector<size_t> shape;
    std::vector<float> v;
    if (!nc::read_float(argv[2], "F", shape, v, err)) { std::printf("ERR %s\n", err.c_str()); return 1; }
    std::printf("%zu", shape.size());
    for (size_t s : shape) std::printf(" %zu", s);
    for (float x : v) std::printf(" %.9g", x);
    std::printf("\n");
    return 0;
  }
  std::vector<std::pair<std::string, size_t>> dims = {{"x", 3}, {"y", 2}, {"f", 5}, {"time", 0}};
  std::vector<nc::Var> vars;
  auto mk = [&](const char* name, std::vector<int> d, bool is_int, float base) {
    nc::Var v;
    v.name = name;
    v.dims = d;
    v.is_int = is_int;
    v.atts = {{"description", std::string("the ") + name}, {"units", "m"}};
    v.fill = [base](size_t first, size_t n, float* out) {
      for (size_t i = 0; i < n; ++i) out[i] = base + (float)(first + i);
      return true;
    };
    vars.push_back(v);
  };
  mk("frequency", {2}, false, 0.5f);
  mk("seamask", {3, 1, 0}, true, 0.f);
  mk("swh", {3, 1, 0}, false, 100.f);
  mk("wspd", {3}, false, 7.f);
  if (!nc::write(argv[1], dims, vars, err, 4)) { std::printf("ERR %s\n", err.c_str()); return 1; }
  return 0;
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    d = tmp_path_factory.mktemp("nc")
    src = d / "driver.cpp"
    src.write_text(DRIVER)
    exe = d / "driver"
    subprocess.run([gxx, "-O1", "-std=c++17", "-I", SRC, str(src), os.path.join(SRC, "ncfile.cpp"), "-o", str(exe)],
                   check=True)
    return str(exe)


def test_writer_read_by_scipy(driver, tmp_path):
    scipy_io = pytest.importorskip("scipy.io")
    path = str(tmp_path / "out.nc")
    subprocess.run([driver, path], check=True)
    with scipy_io.netcdf_file(path, "r", mmap=False) as f:
        assert f.dimensions == {"x": 3, "y": 2, "f": 5, "time": None}
        assert list(f.variables) == ["frequency", "seamask", "swh", "wspd"]
        np.testing.assert_array_equal(f.variables["frequency"][:], 0.5 + np.arange(5))
        sm = f.variables["seamask"]
        assert sm.typecode() == "i" and sm.shape == (4, 2, 3)
        np.testing.assert_array_equal(sm[:], np.arange(24).reshape(4, 2, 3))
        np.testing.assert_array_equal(f.variables["swh"][:], 100 + np.arange(24, dtype=np.float32).reshape(4, 2, 3))
        np.testing.assert_array_equal(f.variables["wspd"][:], 7 + np.arange(4, dtype=np.float32))  # (time,)
        assert f.variables["swh"].description == b"the swh" and f.variables["swh"].units == b"m"


def test_reader_reads_scipy_file(driver, tmp_path):
    scipy_io = pytest.importorskip("scipy.io")
    path = str(tmp_path / "in.nc")
    F = np.random.default_rng(3).random((4, 6, 5)).astype(np.float32)
    with scipy_io.netcdf_file(path, "w", version=2) as f:  # 64-bit offset, as the reference writes
        f.createDimension("x", 4)
        f.createDimension("th", 6)
        f.createDimension("f", 5)
        v = f.createVariable("F", "f4", ("x", "th", "f"))
        v[:] = F
    out = subprocess.run([driver, "read", path], check=True, capture_output=True, text=True).stdout.split()
    nd = int(out[0])
    shape = [int(s) for s in out[1:1 + nd]]
    vals = np.array([float(s) for s in out[1 + nd:]], dtype=np.float32)
    assert shape == [4, 6, 5]
    np.testing.assert_array_equal(vals.reshape(shape), F)
