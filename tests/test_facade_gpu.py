"""The C++ facade (opencamlib_gb300/include/ocl/ocl.hpp), compiled into
tests/facade/facade_test.cpp the way client code of the reference library
uses it, reproduces the reference's golden results on the GPU."""
import math
import os
import subprocess

import numpy as np
import pytest

from tests.helpers import golden

pytestmark = pytest.mark.gpu

ARGS = {"ball": ["ball", "6", "20"], "bull": ["bull", "6", "1", "20"], "cyl": ["cyl", "6", "20"],
        "cone": ["cone", "6", repr(math.pi / 4), "20"], "ballcone": ["ballcone", "2", "6", repr(math.pi / 4)]}


@pytest.fixture(scope="module")
def exe():
    from opencamlib_gb300 import _build
    _build.build_library()
    p = _build.build_facade_test()
    assert p and os.path.exists(p)
    return p


def _run(exe, tmp_path, mode, tris, data, extra):
    t = tmp_path / "t.bin"
    d = tmp_path / "d.bin"
    o = tmp_path / "o.bin"
    np.ascontiguousarray(tris, dtype=np.float64).tofile(t)
    np.ascontiguousarray(data, dtype=np.float64).tofile(d)
    r = subprocess.run([exe, mode, str(t), str(d), str(o)] + extra, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return np.fromfile(o, dtype=np.float64)


@pytest.mark.parametrize("cname", sorted(ARGS))
def test_facade_batch_drop(exe, tmp_path, cname):
    g = golden("drop_heightfield")
    out = _run(exe, tmp_path, "drop", g["tris"], g["cl"], ARGS[cname]).reshape(-1, 7)
    assert np.max(np.abs(out[:, 2] - g[f"{cname}_z"])) <= 1e-5
    np.testing.assert_array_equal(out[:, 6].astype(np.int32), g[f"{cname}_type"])


@pytest.mark.parametrize("cname", ["ball", "bull"])
def test_facade_push(exe, tmp_path, cname):
    g = golden("push_heightfield")
    out = _run(exe, tmp_path, "push", g["tris"], g["fib_x"], ["0"] + ARGS[cname])
    counts = g[f"{cname}_0_counts"]
    k = 0
    ival, cc, ty = g[f"{cname}_0_ival"], g[f"{cname}_0_cc"], g[f"{cname}_0_type"]
    j = 0
    for n in counts:
        assert int(out[k]) == n
        k += 1
        for _ in range(int(n)):
            # lower upper lcc(3) ucc(3) ltype utype, as the reference's Interval
            assert out[k] == ival[j, 0] and out[k + 1] == ival[j, 1]
            np.testing.assert_array_equal(out[k + 2:k + 8], cc[j])
            assert (int(out[k + 8]), int(out[k + 9])) == tuple(ty[j])
            k += 10
            j += 1
    assert k == len(out)


def test_facade_path(exe, tmp_path):
    g = golden("path_heightfield")
    out = _run(exe, tmp_path, "path", g["tris"], g["spans"], ["0.37", "-5.0"] + ARGS["ball"]).reshape(-1, 7)
    assert np.max(np.abs(out[:, :3] - g["ball_pdc_xyz"])) <= 1e-7


@pytest.mark.parametrize("cname", ["ball", "cone", "ballcone"])
def test_facade_adaptive_path(exe, tmp_path, cname):
    g = golden("path_heightfield")
    out = _run(exe, tmp_path, "apdc", g["tris"], g["spans"], ["0.8", "0.05", "0.999"] + ARGS[cname]).reshape(-1, 7)
    assert out.shape[0] == len(g[f"{cname}_apdc_xyz"])  # the reference's points, in its order
    assert np.max(np.abs(out[:, :3] - g[f"{cname}_apdc_xyz"])) <= 1e-7
    np.testing.assert_array_equal(out[:, 6].astype(np.int32), g[f"{cname}_apdc_type"])


def test_facade_stlreader_surface_cache(exe, oracle_lib, tmp_path):
    # STLReader -> STLSurf -> BatchDropCutter, then addTriangle, then rotate:
    # each run must see the surface as it is (the device copy is rebuilt)
    g = golden("drop_heightfield")
    t32 = g["tris"].astype(np.float32)
    stl = tmp_path / "hf.stl"
    with open(stl, "w") as f:
        f.write("solid hf\n")
        for t in t32:
            f.write("facet normal 0 0 1\nouter loop\n")
            for k in range(3):
                f.write("vertex %.9g %.9g %.9g\n" % (t[3 * k], t[3 * k + 1], t[3 * k + 2]))
            f.write("endloop\nendfacet\n")
        f.write("endsolid hf\n")
    cl = g["cl"][::4]
    c = ARGS["ball"]
    cl_path = tmp_path / "cl.bin"
    np.ascontiguousarray(cl).tofile(cl_path)
    o = tmp_path / "o.bin"
    import subprocess
    r = subprocess.run([exe, "stldrop", str(stl), str(cl_path), str(o)] + c, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = np.fromfile(o, dtype=np.float64).reshape(3, len(cl), 7)
    tris = t32.astype(np.float64)
    from tests.golden.cases import CUTTERS
    ball = CUTTERS["ball"]()
    # run 1: the surface as read
    assert np.abs(out[0, :, 2] - oracle_lib.drop(tris, ball, cl, "port")[0]).max() <= 1e-5
    # run 2: plus a horizontal triangle over everything at maxz + 1
    lo, hi = tris.reshape(-1, 3).min(axis=0), tris.reshape(-1, 3).max(axis=0)
    z = hi[2] + 1.0
    extra = np.array([[lo[0] - 10, lo[1] - 10, z, hi[0] + 30, lo[1] - 10, z, lo[0] - 10, hi[1] + 30, z]])
    t2 = np.concatenate([tris, extra])
    assert np.abs(out[1, :, 2] - oracle_lib.drop(t2, ball, cl, "port")[0]).max() <= 1e-5
    # run 3: rotated a quarter turn about z (STLSurf::rotate)
    if oracle_lib.available("ref"):
        t3, _ = oracle_lib.ref_rotate(t2, 0.0, 0.0, 1.5707963267948966)
    else:
        from opencamlib_gb300 import api
        s3 = api.STLSurf(t2)
        s3.rotate(0.0, 0.0, 1.5707963267948966)
        t3 = s3.array()
    assert np.abs(out[2, :, 2] - oracle_lib.drop(t3, ball, cl, "port")[0]).max() <= 1e-5


def _facade_loops(out):
    n = int(out[0])
    k, loops = 1, []
    for _ in range(n):
        m = int(out[k])
        loops.append(out[k + 1:k + 1 + 3 * m].reshape(-1, 3))
        k += 1 + 3 * m
    return loops, int(out[k]), int(out[k + 1])


@pytest.mark.parametrize("adaptive", [False, True])
@pytest.mark.parametrize("cname", ["ball", "bull", "cone"])
def test_facade_waterline(exe, tmp_path, cname, adaptive):
    """ocl::Waterline / ocl::AdaptiveWaterline (setSTL, setCutter, setZ,
    setSampling, [setMinSampling, setCosLimit], run, getLoops, getXFibers,
    getYFibers) against the reference's loops."""
    from oracle import checker
    g = golden("waterline_heightfield")
    for k, z in enumerate(g["zs"]):
        params = [float(z), float(g["sampling"]), 1.0 if adaptive else 0.0, float(g["min_sampling"]), 0.999]
        out = _run(exe, tmp_path, "waterline", g["tris"], params, ARGS[cname])
        loops, nx, ny = _facade_loops(out)
        key = f"{cname}_{'awl' if adaptive else 'wl'}_{k}"
        pts, off = g[key + "_pts"], g[key + "_off"]
        ref = [pts[off[j]:off[j + 1]] for j in range(len(off) - 1)]
        assert checker.loops_close(loops, ref, 1e-7), key
        assert nx == len(g[key + "_f0"]) and ny == len(g[key + "_f1"])
