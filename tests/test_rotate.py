"""STLSurf::rotate (src/geo/stlsurf.cpp:44-55, Triangle::rotate
src/geo/triangle.cpp:130-138, Point::xRotate/yRotate/zRotate
src/geo/point.cpp:105-134) in the Python mirror and the C++ facade, bit for
bit against the reference's own STLSurf built from its sources (host code,
no GPU)."""
import math
import os
import subprocess

import numpy as np
import pytest

import opencamlib_gb300 as ocl
from opencamlib_gb300 import workloads as w

ANGLES = [(0.1, 0.2, 0.3), (math.pi / 2, 0.0, 0.0), (0.0, 0.0, math.pi / 2), (-1.3, 2.2, 0.7), (0.0, 0.0, 0.0)]


@pytest.fixture(scope="module")
def ref(oracle_lib):
    if not oracle_lib.available("ref"):
        pytest.skip("the reference build (oracle/_ref) needs the reference sources, absent on this machine")
    return oracle_lib


@pytest.fixture(scope="module")
def tris():
    return w.heightfield(12, 9, seed=3, jitter=0.1, jitter_seed=4)


@pytest.mark.parametrize("angles", ANGLES)
def test_python_stlsurf_rotate(ref, tris, angles):
    want, bb = ref.ref_rotate(tris, *angles)
    s = ocl.STLSurf(tris)
    s.rotate(*angles)
    np.testing.assert_array_equal(s.array(), want)
    np.testing.assert_array_equal(np.array(s.getBounds()), bb)


def test_python_triangle_rotate(ref, tris):
    want, _ = ref.ref_rotate(tris[:1], 0.4, -0.7, 1.9)
    t = ocl.Triangle(ocl.Point(*tris[0, 0:3]), ocl.Point(*tris[0, 3:6]), ocl.Point(*tris[0, 6:9]))
    t.rotate(0.4, -0.7, 1.9)
    np.testing.assert_array_equal(np.array(t.array()), want[0])


def test_rotate_invalidates_the_device_copy(tris):
    s = ocl.STLSurf(tris)
    s._dev = {1: "stale"}  # a cached device copy of the unrotated surface
    s.rotate(0.0, 0.0, 0.5)
    assert s._dev == {}


@pytest.mark.parametrize("angles", ANGLES[:4])
def test_facade_stlsurf_rotate(ref, tris, angles, tmp_path):
    from opencamlib_gb300 import _build
    _build.build_library()
    exe = _build.build_facade_test()
    t, a, o = tmp_path / "t.bin", tmp_path / "a.bin", tmp_path / "o.bin"
    np.ascontiguousarray(tris).tofile(t)
    np.array(angles, dtype=np.float64).tofile(a)
    r = subprocess.run([exe, "rotate", str(t), str(a), str(o)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(o, dtype=np.float64)
    want, bb = ref.ref_rotate(tris, *angles)
    np.testing.assert_array_equal(got[:-6].reshape(-1, 9), want)
    np.testing.assert_array_equal(got[-6:], bb)
    assert os.path.exists(exe)
