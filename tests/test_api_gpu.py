"""The Python mirror of the reference's module (opencamlib_gb300.api: STLSurf,
STLReader, the cutters, BatchDropCutter, PathDropCutter,
AdaptivePathDropCutter, BatchPushCutter, Fiber, Path/Line/Arc), driven the way
the reference's Python examples drive `ocl` (setSTL, setCutter, appendPoint /
appendFiber, run, getCLPoints / getFibers), against the golden fixtures made
by the reference itself."""
import math
import os

import numpy as np
import pytest

from tests.golden.cases import CUTTERS
from tests.helpers import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ocl():
    import opencamlib_gb300 as ocl
    if not ocl.device_available():
        pytest.fail("no CUDA device")
    return ocl


def _surface(ocl, tris):
    s = ocl.STLSurf()
    for t in tris:
        s.addTriangle(ocl.Triangle(ocl.Point(*t[0:3]), ocl.Point(*t[3:6]), ocl.Point(*t[6:9])))
    return s


@pytest.mark.parametrize("cname", ["cyl", "ball", "bull", "cone", "ballcone"])
def test_batch_drop_cutter(ocl, cname):
    g = golden("drop_heightfield")
    s = _surface(ocl, g["tris"])
    bdc = ocl.BatchDropCutter()
    bdc.setSTL(s)
    bdc.setCutter(CUTTERS[cname]())
    for p in g["cl"]:
        bdc.appendPoint(ocl.CLPoint(p[0], p[1], p[2]))
    bdc.run()
    pts = bdc.getCLPoints()
    z = np.array([p.z for p in pts])
    ty = np.array([p.getCC().type for p in pts])
    cc = np.array([[p.cc().x, p.cc().y, p.cc().z] for p in pts])
    assert np.abs(z - g[f"{cname}_z"]).max() <= 1e-5
    np.testing.assert_array_equal(ty, g[f"{cname}_type"])
    lifted = ty != 0
    assert np.abs(cc[lifted] - g[f"{cname}_cc"][lifted]).max() <= 1e-5
    assert bdc.getCalls() > 0


def _path(ocl, spans):
    path = ocl.Path()
    for r in spans:
        p1, p2, c = ocl.Point(*r[1:4]), ocl.Point(*r[4:7]), ocl.Point(*r[7:10])
        path.append(ocl.Line(p1, p2) if r[0] == 0 else ocl.Arc(p1, p2, c, bool(r[10])))
    return path


@pytest.mark.parametrize("cname", ["ball", "bull", "ballcone"])
def test_path_drop_cutter(ocl, cname):
    g = golden("path_heightfield")
    pdc = ocl.PathDropCutter()
    pdc.setSTL(_surface(ocl, g["tris"]))
    pdc.setCutter(CUTTERS[cname]())
    pdc.setPath(_path(ocl, g["spans"]))
    pdc.setSampling(0.37)
    pdc.setZ(-5.0)
    pdc.run()
    pts = pdc.getCLPoints()
    xyz = np.array([[p.x, p.y, p.z] for p in pts])
    assert xyz.shape == g[f"{cname}_pdc_xyz"].shape
    assert np.abs(xyz - g[f"{cname}_pdc_xyz"]).max() <= 1e-7
    np.testing.assert_array_equal([p.getCC().type for p in pts], g[f"{cname}_pdc_type"])


@pytest.mark.parametrize("cname", ["ball", "cone", "ballcone"])
def test_adaptive_path_drop_cutter(ocl, cname):
    g = golden("path_heightfield")
    apdc = ocl.AdaptivePathDropCutter()
    apdc.setSTL(_surface(ocl, g["tris"]))
    apdc.setCutter(CUTTERS[cname]())
    apdc.setPath(_path(ocl, g["spans"]))
    apdc.setSampling(0.8)
    apdc.setMinSampling(0.05)
    apdc.setCosLimit(0.999)
    apdc.run()
    pts = apdc.getCLPoints()
    xyz = np.array([[p.x, p.y, p.z] for p in pts])
    assert xyz.shape == g[f"{cname}_apdc_xyz"].shape  # same points in the reference's order
    assert np.abs(xyz - g[f"{cname}_apdc_xyz"]).max() <= 1e-7
    np.testing.assert_array_equal([p.getCC().type for p in pts], g[f"{cname}_apdc_type"])


@pytest.mark.parametrize("cname", ["ball", "bull", "cyl"])
def test_batch_push_cutter(ocl, cname):
    g = golden("push_heightfield")
    s = _surface(ocl, g["tris"])
    for d, key in ((0, "fib_x"), (1, "fib_y")):
        bpc = ocl.BatchPushCutter()
        bpc.setXDirection() if d == 0 else bpc.setYDirection()
        bpc.setSTL(s)
        bpc.setCutter(CUTTERS[cname]())
        for f in g[key]:
            bpc.appendFiber(ocl.Fiber(ocl.Point(*f[0:3]), ocl.Point(*f[3:6])))
        bpc.run()
        fibers = bpc.getFibers()
        counts = g[f"{cname}_{d}_counts"]
        ival, cc, ty = g[f"{cname}_{d}_ival"], g[f"{cname}_{d}_cc"], g[f"{cname}_{d}_type"]
        k = 0
        for f, n in zip(fibers, counts):
            ints = f.getInts()
            assert len(ints) == n
            for i in ints:
                assert i.lower == ival[k, 0] and i.upper == ival[k, 1]
                assert (i.lower_cc.type, i.upper_cc.type) == tuple(ty[k])
                np.testing.assert_array_equal([i.lower_cc.x, i.lower_cc.y, i.lower_cc.z], cc[k, :3])
                k += 1
        # getCLPoints: both ends of every interval, in fiber order
        assert len(bpc.getCLPoints()) == 2 * int(counts.sum())


def test_stlreader_into_stlsurf_and_drop(ocl, oracle_lib, tmp_path):
    # STLReader -> STLSurf -> BatchDropCutter; the device copy follows
    # addTriangle and rotate
    g = golden("drop_heightfield")
    t32 = g["tris"].astype(np.float32)
    p = os.path.join(tmp_path, "hf.stl")
    rows = np.zeros(len(t32), dtype=[("n", "<f4", 3), ("v", "<f4", 9), ("a", "<u2")])
    rows["v"] = t32
    with open(p, "wb") as f:
        f.write(b"binary".ljust(80, b" "))
        f.write(np.uint32(len(t32)).tobytes())
        f.write(rows.tobytes())
    s = ocl.STLSurf()
    ocl.STLReader(p, s)
    assert s.size() == len(t32)
    np.testing.assert_array_equal(s.array(), t32.astype(np.float64))
    c = CUTTERS["ball"]()

    def run():
        bdc = ocl.BatchDropCutter()
        bdc.setSTL(s)
        bdc.setCutter(c)
        for q in g["cl"][:200]:
            bdc.appendPoint(ocl.CLPoint(*q))
        bdc.run()
        return np.array([q.z for q in bdc.getCLPoints()])

    z0 = run()
    dev0 = s.device()
    top = float(s.array()[:, 2::3].max()) + 1.0
    s.addTriangle(ocl.Triangle(ocl.Point(-50, -50, top), ocl.Point(300, -50, top), ocl.Point(-50, 300, top)))
    z1 = run()
    assert s.device() is not dev0
    np.testing.assert_array_equal(z1, np.full_like(z1, top))
    assert np.all(z0 < top)
    s.rotate(0.3, -0.2, math.pi / 3)
    z2 = run()  # the rotated surface is a new device mesh
    zr = oracle_lib.drop(s.array(), c, g["cl"][:200], "port")[0]
    assert np.abs(z2 - zr).max() <= 1e-5


@pytest.mark.parametrize("adaptive", [False, True])
def test_waterline_mirror(ocl, adaptive):
    """ocl.Waterline / ocl.AdaptiveWaterline as the reference's Python
    binding is used (setSTL, setCutter, setZ, setSampling, run, getLoops)."""
    from oracle import checker
    g = golden("waterline_heightfield")
    s = _surface(ocl, g["tris"])
    for k, z in enumerate(g["zs"]):
        wl = ocl.AdaptiveWaterline() if adaptive else ocl.Waterline()
        wl.setSTL(s)
        wl.setCutter(CUTTERS["bull"]())
        wl.setZ(float(z))
        wl.setSampling(float(g["sampling"]))
        if adaptive:
            wl.setMinSampling(float(g["min_sampling"]))
        wl.run()
        loops = [np.array([[p.x, p.y, p.z] for p in lp]) for lp in wl.getLoops()]
        key = f"bull_{'awl' if adaptive else 'wl'}_{k}"
        pts, off = g[key + "_pts"], g[key + "_off"]
        ref = [pts[off[j]:off[j + 1]] for j in range(len(off) - 1)]
        assert checker.loops_close(loops, ref, 1e-7)
        assert len(wl.getXFibers()) == len(g[key + "_f0"])
        xf = wl.getXFibers()
        n = sum(len(f.ints) for f in xf)
        assert n == len(g[key + "_i0"])
