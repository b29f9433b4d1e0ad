"""Waterline and AdaptiveWaterline on the GPU (ocl_gb300_waterline,
_levels, _adaptive_waterline): fibers pushed on the device, woven on the
host.  Checked against the reference's own Waterline::run and
AdaptiveWaterline::run stored in the golden fixtures (made on another
machine, whose libm's atan and sin may round a bull edge's slope
differently in the last bit: interval ends within 1e-7 mm, loops the same
cyclic point sequences within 1e-7 mm), and bit for bit against the oracle
port run here (same fibers pushed on the host, woven by the same weave)."""
import numpy as np
import pytest

from opencamlib_gb300 import _abi, _native
from opencamlib_gb300 import cutters as cu
from opencamlib_gb300 import workloads as w
from oracle import checker
from tests.golden.cases import CUTTERS
from tests.helpers import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ocl():
    import opencamlib_gb300 as o
    if not o.device_available():
        pytest.fail("no CUDA device")
    return o


def same_loops(a, b):
    ca, cb = checker.canonical_loops(a), checker.canonical_loops(b)
    return len(ca) == len(cb) and all(np.array_equal(x, y) for x, y in zip(ca, cb))


def golden_loops(g, key):
    pts, off = g[key + "_pts"], g[key + "_off"]
    return [pts[off[k]:off[k + 1]] for k in range(len(off) - 1)]


def check_against(g, key, res, tris, cutter):
    fibers = []
    for d in (0, 1):
        fib, off, iv, _, _ = res.fibers(d)
        np.testing.assert_array_equal(fib, g[f"{key}_f{d}"], err_msg=key)
        np.testing.assert_array_equal(off.astype(np.int64), g[f"{key}_o{d}"], err_msg=key)
        ext = np.abs(fib[:, 3:5] - fib[:, 0:2]).max()  # fiber length: t to mm
        assert np.abs(iv - g[f"{key}_i{d}"]).max(initial=0.0) * ext <= 1e-7, key
        # bit for bit against the oracle port on this machine
        port, _ = checker.push(tris, cutter, d, fib, "port")
        np.testing.assert_array_equal(off.astype(np.int64), np.cumsum([0] + [len(r) for r in port]), err_msg=key)
        np.testing.assert_array_equal(iv, np.array([[r[0], r[1]] for rr in port for r in rr]).reshape(-1, 2),
                                      err_msg=key)
        fibers.append((fib, off, iv))
    assert checker.loops_close(res.loops, golden_loops(g, key), 1e-7), key
    assert same_loops(res.loops, _native.weave(*fibers).loops), key


@pytest.mark.parametrize("name", ["heightfield", "sphere_on_plate"])
def test_waterline_matches_reference(ocl, name):
    g = golden("waterline_" + name)
    mesh = ocl.DeviceMesh(g["tris"])
    cnames = sorted({k.split("_")[0] for k in g if k.endswith("_pts")})
    for cname in cnames:
        c = CUTTERS[cname]()
        for k, z in enumerate(g["zs"]):
            res, st = mesh.waterline(c, float(z), float(g["sampling"]))
            check_against(g, f"{cname}_wl_{k}", res, g["tris"], c)
            assert st.iter_limit_hits == 0


@pytest.mark.parametrize("name", ["heightfield", "sphere_on_plate"])
def test_adaptive_waterline_matches_reference(ocl, name):
    g = golden("waterline_" + name)
    mesh = ocl.DeviceMesh(g["tris"])
    cnames = sorted({k.split("_")[0] for k in g if k.endswith("_pts")})
    for cname in cnames:
        c = CUTTERS[cname]()
        for k, z in enumerate(g["zs"]):
            res, _ = mesh.adaptive_waterline(c, float(z), float(g["sampling"]), float(g["min_sampling"]))
            check_against(g, f"{cname}_awl_{k}", res, g["tris"], c)


def test_levels_equal_single_heights(ocl):
    g = golden("waterline_heightfield")
    mesh = ocl.DeviceMesh(g["tris"])
    c = cu.BullCutter(6.0, 1.0, 20.0)
    zs = [10.5, 11.0, 12.25, 14.0, 17.0, 20.0, 31.0]
    many, st = mesh.waterline_levels(c, zs, 0.9)
    assert len(many) == len(zs)
    for z, res in zip(zs, many):
        one, _ = mesh.waterline(c, z, 0.9)
        assert len(one.loops) == len(res.loops)
        for a, b in zip(one.loops, res.loops):
            np.testing.assert_array_equal(a, b)
        for d in (0, 1):
            for x, y in zip(one.fibers(d), res.fibers(d)):
                np.testing.assert_array_equal(x, y)
    assert st.kernel_ms > 0.0


def test_waterline_larger_mesh_against_oracle_fibers(ocl):
    """sphere-on-plate + torus (about 98k triangles), ball and bull cutters
    at three heights: the device fibers equal the oracle port's push, and
    the loops equal the weave of the port's fibers."""
    tris = w.sphere_torus(8)
    mesh = ocl.DeviceMesh(tris)
    for c in (cu.BallCutter(6.0, 20.0), cu.BullCutter(6.0, 1.0, 20.0)):
        for z in (3.0, 17.5, 28.0):
            res, _ = mesh.waterline(c, z, 2.0)
            fibers = []
            for d in (0, 1):
                fib, off, iv, cc, ty = res.fibers(d)
                port, _ = checker.push(tris, c, d, fib, "port")
                po = np.cumsum([0] + [len(r) for r in port])
                np.testing.assert_array_equal(off.astype(np.int64), po)
                pi = np.array([[r[0], r[1]] for rr in port for r in rr]).reshape(-1, 2)
                np.testing.assert_array_equal(iv, pi)
                fibers.append((fib, off, iv))
            assert same_loops(res.loops, _native.weave(*fibers).loops)
            assert len(res.loops) >= 1


def test_waterline_bad_arguments(ocl):
    g = golden("waterline_heightfield")
    mesh = ocl.DeviceMesh(g["tris"])
    c = cu.BallCutter(6.0, 20.0)
    for bad in (0.0, -1.0, float("nan")):
        with pytest.raises(_native.OclError) as e:
            mesh.waterline(c, 12.0, bad)
        assert e.value.status == _abi.BAD_ARG
    with pytest.raises(_native.OclError) as e:
        mesh.adaptive_waterline(c, 12.0, 1.0, 0.0)
    assert e.value.status == _abi.BAD_ARG
