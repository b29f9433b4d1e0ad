"""STL reading (STLReader, src/geo/stlreader.cpp:57-150): host code of the
library, so these tests run without a GPU.

Files are generated here (ASCII and binary, seeded coordinates); the reader
must return the float32 coordinates widened to double in file order, follow
the reference's line rules (first five non-blank characters, vertex index
capped at the third, a triangle at "endfacet" after two or more vertices,
vertex lines that do not parse keep the old values), and agree with the
reference's own STLReader (built from its sources, in this container only) on
every file the reference reads in finite time with defined values."""
import os
import struct
import subprocess

import numpy as np
import pytest

from oracle import checker
from opencamlib_gb300 import _build, _native, workloads as w


def tris_f32(n, seed):
    u = w.uniform(seed, 9 * n).reshape(n, 9)
    return (200.0 * u - 100.0).astype(np.float32).astype(np.float64)


def write_ascii(path, tris, newline="\n", title="gen"):
    lines = [f"solid {title}"]
    for t in tris:
        lines.append("  facet normal 0 0 1")
        lines.append("    outer loop")
        for k in range(3):
            lines.append("      vertex %.9g %.9g %.9g" % (t[3 * k], t[3 * k + 1], t[3 * k + 2]))
        lines.append("    endloop")
        lines.append("  endfacet")
    lines.append(f"endsolid {title}")
    with open(path, "w", newline="") as f:
        f.write(newline.join(lines) + newline)


def write_binary(path, tris, header=b"binary stl"):
    with open(path, "wb") as f:
        f.write(header.ljust(80, b" ")[:80])
        f.write(struct.pack("<I", len(tris)))
        for t in tris:
            f.write(struct.pack("<3f", 0.0, 0.0, 1.0))
            f.write(struct.pack("<9f", *t))
            f.write(b"\0\0")


def write_text(path, text):
    with open(path, "w", newline="") as f:
        f.write(text)


def ref_available():
    return checker.available("ref")


def same_as_reference(path):
    if not ref_available():
        pytest.skip("the reference build (oracle/_ref) needs the reference sources, absent on this machine")
    np.testing.assert_array_equal(_native.stl_read(path, strict=False), checker.ref_stl_read(path))


@pytest.mark.parametrize("fmt", ["ascii", "ascii_crlf", "binary"])
def test_round_trip(tmp_path, fmt):
    tris = tris_f32(257, 11)
    p = str(tmp_path / f"m_{fmt}.stl")
    if fmt == "binary":
        write_binary(p, tris)
    else:
        write_ascii(p, tris, "\r\n" if fmt == "ascii_crlf" else "\n")
    got = _native.stl_read(p)
    np.testing.assert_array_equal(got, tris)
    same_as_reference(p)


VALID = "  facet normal 0 0 1\n  outer loop\n  vertex 1 2 3\n  vertex 4 5 6\n  vertex 7 8 9\n  endloop\n  endfacet\n"

QUIRKS = {
    # blanks between the keyword's first five letters still select it; the
    # sscanf of " vertex %f %f %f" then fails and the vertex keeps its value
    "spaced_keyword": VALID + "facet normal 0 0 1\nvertex 10 11 12\nv e r t e x 20 21 22\nvertex 13 14 15\nendfacet\n",
    # a fourth vertex overwrites the third
    "four_vertices": VALID + "facet normal 0 0 1\nvertex 1 1 1\nvertex 2 2 2\nvertex 3 3 3\nvertex 4 4 4\nendfacet\n",
    # two vertex lines are enough for a triangle; the third keeps its value
    "two_vertices": VALID + "facet normal 0 0 1\nvertex 5 5 5\nvertex 6 6 6\nendfacet\n",
    # one vertex line is not
    "one_vertex": VALID + "facet normal 0 0 1\nvertex 5 5 5\nendfacet\n",
    # a partial vertex line sets the values it has
    "partial_vertex": VALID + "facet normal 0 0 1\nvertex 1 2\nvertex 3 4 5\nvertex 6 7 8\nendfacet\n",
    # tabs, a missing final newline, and a triangle without "facet"
    "tabs_no_newline": VALID + "\tfacet normal 0 0 1\n\tvertex\t1.5\t2.5\t3.5\n vertex 4 5 6\nvertex 7 8 9\nendfacet",
    "no_facet_line": VALID + "vertex 9 9 9\nendfacet\n",
    "exponents": VALID + "facet normal 0 0 1\nvertex 1e-3 -2.5E+2 .5\nvertex 0x1p-2 3 4\nvertex 5 6 7\nendfacet\n",
}


@pytest.mark.parametrize("name", sorted(QUIRKS))
def test_ascii_rules(tmp_path, name):
    p = str(tmp_path / f"{name}.stl")
    write_text(p, "solid quirks\n" + QUIRKS[name] + ("" if name == "tabs_no_newline" else "endsolid quirks\n"))
    got = _native.stl_read(p)
    assert got.shape[1] == 9
    # the valid first facet is always read
    np.testing.assert_array_equal(got[0], [1, 2, 3, 4, 5, 6, 7, 8, 9])
    same_as_reference(p)


def test_ascii_rules_expected(tmp_path):
    p = str(tmp_path / "q.stl")
    write_text(p, "solid q\n" + QUIRKS["four_vertices"] + "endsolid q\n")
    np.testing.assert_array_equal(_native.stl_read(p)[1], [1, 1, 1, 2, 2, 2, 4, 4, 4])
    write_text(p, "solid q\n" + QUIRKS["two_vertices"] + "endsolid q\n")
    np.testing.assert_array_equal(_native.stl_read(p)[1], [5, 5, 5, 6, 6, 6, 7, 8, 9])
    write_text(p, "solid q\n" + QUIRKS["one_vertex"] + "endsolid q\n")
    assert _native.stl_read(p).shape == (1, 9)
    write_text(p, "solid q\n" + QUIRKS["spaced_keyword"] + "endsolid q\n")
    np.testing.assert_array_equal(_native.stl_read(p)[1], [10, 11, 12, 4, 5, 6, 13, 14, 15])


def test_binary_with_solid_header(tmp_path):
    # the reference would parse this as ASCII (and can loop forever); the
    # file size identifies it as binary
    tris = tris_f32(40, 12)
    p = str(tmp_path / "solid_bin.stl")
    write_binary(p, tris, header=b"solid binary header")
    np.testing.assert_array_equal(_native.stl_read(p), tris)


def test_long_ascii_line_is_cut(tmp_path):
    p = str(tmp_path / "long.stl")
    write_text(p, "solid l\n" + VALID + "vertex 1 1 1" + " " * 3000 + "\nendsolid l\n")
    np.testing.assert_array_equal(_native.stl_read(p), [[1, 2, 3, 4, 5, 6, 7, 8, 9]])


def test_errors(tmp_path):
    missing = str(tmp_path / "none.stl")
    with pytest.raises(_native.OclError):
        _native.stl_read(missing)
    assert _native.stl_read(missing, strict=False).shape == (0, 9)
    tris = tris_f32(10, 13)
    p = str(tmp_path / "trunc.stl")
    write_binary(p, tris)
    with open(p, "rb") as f:
        data = f.read()
    with open(p, "wb") as f:
        f.write(data[:-30])  # the last facet is cut
    with pytest.raises(_native.OclError):
        _native.stl_read(p)
    np.testing.assert_array_equal(_native.stl_read(p, strict=False), tris[:9])
    for content in (b"", b"sol", b"solid"):
        with open(p, "wb") as f:
            f.write(content)
        assert _native.stl_read(p).shape == (0, 9)


def test_python_reader_fills_a_surface(tmp_path):
    import opencamlib_gb300 as ocl
    tris = tris_f32(20, 14)
    p = str(tmp_path / "s.stl")
    write_binary(p, tris)
    s = ocl.STLSurf()
    s.addTriangle(ocl.Triangle(ocl.Point(0, 0, 0), ocl.Point(1, 0, 0), ocl.Point(0, 1, 0)))
    ocl.STLReader(p, s)
    assert s.size() == 21
    np.testing.assert_array_equal(s.array()[1:], tris)
    ocl.STLReader(str(tmp_path / "missing.stl"), s)  # adds nothing, as the reference
    assert s.size() == 21


def test_cpp_facade_reader(tmp_path):
    # the header-only facade's STLReader against the library, host code only
    tris = tris_f32(33, 15)
    p = str(tmp_path / "f.stl")
    write_ascii(p, tris)
    src = tmp_path / "r.cpp"
    src.write_text(
        '#include "ocl/ocl.hpp"\n#include <cstdio>\n'
        "int main(int argc, char** argv) {\n"
        "  std::string a(argv[1]); std::wstring wp(a.begin(), a.end());\n"
        "  ocl::STLSurf s; ocl::STLReader r(wp, s);\n"
        "  std::printf(\"%u\\n\", s.size());\n"
        "  for (const ocl::Triangle& t : s.tris) for (int k = 0; k < 3; ++k)\n"
        "    std::printf(\"%.17g %.17g %.17g\\n\", t.p[k].x, t.p[k].y, t.p[k].z);\n"
        "  return 0;\n}\n")
    exe = str(tmp_path / "r")
    _build.build_library()
    out = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(_build.PKG, "include"),
                          "-I", os.path.join(_build.ROOT, "include"), str(src), "-o", exe,
                          "-L", _build.OUT, "-locl_gb300", "-Wl,-rpath," + _build.OUT],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    r = subprocess.run([exe, p], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    assert int(lines[0]) == 33
    got = np.array([[float(v) for v in ln.split()] for ln in lines[1:1 + 99]]).reshape(33, 9)
    np.testing.assert_array_equal(got, tris)
