"""LineCLFilter (src/common/lineclfilter.cpp:40-77): host code of the
library, so these tests run without a GPU.

The kept points must be the reference's, point for point, against the
reference's own LineCLFilter (built from its sources, in this container
only) on zig-zag paths with noise, drop-cutter output of the oracle, and the
degenerate cases (0-3 points, repeated points, exactly collinear runs)."""
import os
import subprocess

import numpy as np
import pytest

from oracle import checker
from opencamlib_gb300 import _build, _native, cutters as cu, workloads as w

TOLS = [0.0, 1e-6, 1e-3, 0.01, 0.1, 1.0]


def zigzag(n_lines, per_line, noise, seed):
    u = w.uniform(seed, n_lines * per_line * 3).reshape(-1, 3)
    pts = []
    for k in range(n_lines):
        xs = np.linspace(0.0, 50.0, per_line)
        if k % 2:
            xs = xs[::-1]
        for i, x in enumerate(xs):
            r = u[k * per_line + i]
            pts.append((x + noise * (r[0] - 0.5), 0.5 * k + noise * (r[1] - 0.5),
                        2.0 * np.sin(0.2 * x) + noise * (r[2] - 0.5)))
    return np.array(pts)


def check_against_reference(xyz, tol):
    keep = _native.line_filter(xyz, tol)
    assert len(xyz) == 0 or keep[0] == 0
    assert np.all(np.diff(keep) > 0)
    if not checker.available("ref"):
        pytest.skip("the reference build (oracle/_ref) needs the reference sources, absent on this machine")
    np.testing.assert_array_equal(xyz[keep], checker.ref_line_filter(xyz, tol))
    return keep


@pytest.mark.parametrize("tol", TOLS)
def test_zigzag_paths(tol):
    for noise, seed in ((0.0, 1), (1e-4, 2), (0.05, 3)):
        xyz = zigzag(6, 120, noise, seed)
        keep = check_against_reference(xyz, tol)
        assert keep[-1] == len(xyz) - 1


def test_dropcutter_output():
    # CL points of a path drop over a bumpy heightfield (the oracle's CPU
    # drop), filtered as a CAM post-pass would
    tris = w.heightfield_c1()
    x = np.linspace(5.0, 95.0, 900)
    cl = np.stack([x, np.full_like(x, 50.0), np.full_like(x, -50.0)], axis=1)
    z = checker.drop(tris, cu.BallCutter(6.0, 20.0), cl, "port")[0]
    xyz = np.stack([x, cl[:, 1], z], axis=1)
    for tol in TOLS:
        check_against_reference(xyz, tol)


def test_degenerate_lists():
    for n in range(4):
        xyz = zigzag(1, 4, 0.0, 4)[:n]
        keep = check_against_reference(xyz, 0.01)
        if n < 2:
            np.testing.assert_array_equal(keep, np.arange(n))
    same = np.ones((7, 3))
    check_against_reference(same, 0.01)  # v = 0: the reference divides 0 by 0
    rep = np.repeat(zigzag(1, 20, 0.0, 5), 2, axis=0)
    for tol in TOLS:
        check_against_reference(rep, tol)
    line = np.stack([np.arange(50.0), 2.0 * np.arange(50.0), np.zeros(50)], axis=1)
    np.testing.assert_array_equal(check_against_reference(line, 1e-9), [0, 49])


def test_python_mirror():
    import opencamlib_gb300 as ocl
    xyz = zigzag(3, 50, 1e-3, 6)
    f = ocl.LineCLFilter()
    for p in xyz:
        f.addCLPoint(ocl.CLPoint(*p))
    f.setTolerance(0.01)
    f.run()
    got = np.array([[p.x, p.y, p.z] for p in f.getCLPoints()])
    np.testing.assert_array_equal(got, xyz[_native.line_filter(xyz, 0.01)])


def test_cpp_facade(tmp_path):
    # the header-only facade's LineCLFilter against the library, host code only
    xyz = zigzag(4, 60, 1e-3, 7)
    inp = tmp_path / "pts.txt"
    inp.write_text("\n".join("%.17g %.17g %.17g" % tuple(p) for p in xyz) + "\n")
    src = tmp_path / "f.cpp"
    src.write_text(
        '#include "ocl/ocl.hpp"\n#include <cstdio>\n#include <fstream>\n'
        "int main(int argc, char** argv) {\n"
        "  std::ifstream in(argv[1]); double x, y, z; ocl::LineCLFilter f;\n"
        "  while (in >> x >> y >> z) f.addCLPoint(ocl::CLPoint(x, y, z));\n"
        "  f.setTolerance(0.01); f.run();\n"
        "  std::printf(\"%zu\\n\", f.clpoints.size());\n"
        "  for (const ocl::CLPoint& p : f.clpoints) std::printf(\"%.17g %.17g %.17g\\n\", p.x, p.y, p.z);\n"
        "  return 0;\n}\n")
    exe = str(tmp_path / "f")
    _build.build_library()
    out = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(_build.PKG, "include"),
                          "-I", os.path.join(_build.ROOT, "include"), str(src), "-o", exe,
                          "-L", _build.OUT, "-locl_gb300", "-Wl,-rpath," + _build.OUT],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    r = subprocess.run([exe, str(inp)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    n = int(lines[0])
    got = np.array([[float(v) for v in ln.split()] for ln in lines[1:1 + n]])
    np.testing.assert_array_equal(got, xyz[_native.line_filter(xyz, 0.01)])
