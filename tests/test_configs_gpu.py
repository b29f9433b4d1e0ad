"""Parity at the workload configurations, against the oracle (the C
restatement pinned bit for bit to the reference build; tests/test_oracle.py,
tests/test_realmesh.py):

* the 32,258-triangle bump field with its whole 40,000-point 0.5 mm raster,
  BallCutter d6 (the plain FP64 BatchDropCutter workload);
* the 1,048,576-triangle mesh with a seeded 10,000-point sample of its
  1,000,000-point 0.1 mm raster, all five cutters, mixed and plain FP64;
* the 499,202-triangle sphere-on-plate + torus with a 2% fiber sample (every
  50th fiber) at all 50 waterline z levels, X and Y fibers, Bull d6 r1 and
  Ball d6 (BatchPushCutter).

Drop: max |dz| <= 1e-5 mm, CC types identical, CC points within 1e-5 mm.
Push: the interval list of every fiber in the reference's order, endpoints
within 1e-7 mm along the fiber, CC types identical."""
import numpy as np
import pytest

from opencamlib_gb300 import cutters as cu
from opencamlib_gb300 import workloads as w
from tests.helpers import push_records_equal

pytestmark = pytest.mark.gpu

ZTOL = 1e-5


@pytest.fixture(scope="module")
def ocl():
    import opencamlib_gb300 as ocl
    if not ocl.device_available():
        pytest.fail("no CUDA device")
    return ocl


def _cmp(got, ref, what):
    z, cc, ty = got[:3]
    zr, ccr, tyr = ref[:3]
    dz = np.abs(z - zr)
    assert dz.max() <= ZTOL, f"{what}: max|dz|={dz.max()} at {np.argmax(dz)}"
    np.testing.assert_array_equal(ty, tyr, err_msg=what)
    lifted = tyr != 0
    assert np.abs(cc[lifted] - ccr[lifted]).max(initial=0.0) <= ZTOL, what
    return float(dz.max()), float(np.sqrt(np.mean(dz * dz)))


def test_bump_field_whole_raster_ball(ocl, oracle_lib):
    tris, cl = w.heightfield_c1(), w.raster_c1()
    c = cu.BallCutter(6.0, 20.0)
    mesh = ocl.DeviceMesh(tris)
    ref = oracle_lib.drop(tris, c, cl, "port")
    for prec in ("mixed", "fp64"):
        got = mesh.drop(c, cl, precision=prec)
        assert got[3].violations == 0 and got[3].iter_limit_hits == 0
        _cmp(got, ref, prec)


@pytest.fixture(scope="module")
def c2():
    tris = w.mesh_c2()
    cl = w.raster_c2()[w.subsample(1000 * 1000, 10000, 41)]
    return tris, cl


@pytest.mark.parametrize("cname", ["cyl", "ball", "bull", "cone", "ballcone"])
def test_million_triangle_mesh_sample(ocl, oracle_lib, c2, cname):
    tris, cl = c2
    c = cu.standard_cutters()[cname]
    ref = oracle_lib.drop(tris, c, cl, "port")
    mesh = ocl.DeviceMesh(tris)
    got_m = mesh.drop(c, cl, precision="mixed")
    got_f = mesh.drop(c, cl, precision="fp64")
    assert got_m[3].violations == 0 and got_m[3].iter_limit_hits == 0
    _cmp(got_m, ref, "mixed")
    _cmp(got_f, ref, "fp64")
    # the FP64 path evaluates the reference's exact-overlap pairs
    if cname == "ball":
        assert got_f[3].pairs == oracle_lib.overlap_pairs(tris, c.radius, cl)


@pytest.fixture(scope="module")
def c4():
    tris = w.sphere_torus(1)
    return tris


def _waterline_fibers(direction, r):
    # 50 z levels 1 + 48 k / 49, 2,000 fibers across [0, 100] per level and
    # direction, extent the mesh bbox +- 2 radii; every 50th fiber kept
    f = [w.fibers(direction, 1.0 + 48.0 * k / 49.0, 0.0, 100.0, 2000, -2 * r, 100.0 + 2 * r)[::50] for k in range(50)]
    return np.concatenate(f)


@pytest.mark.parametrize("cname", ["ball", "bull"])
def test_waterline_fiber_sample(ocl, oracle_lib, c4, cname):
    tris = c4
    c = cu.standard_cutters()[cname]
    mesh = ocl.DeviceMesh(tris)
    for d in (0, 1):
        fib = _waterline_fibers(d, c.radius)
        assert len(fib) == 2000
        res, st = mesh.push(c, d, fib)
        assert st.iter_limit_hits == 0
        ref, _ = oracle_lib.push(tris, c, d, fib, "port")
        counts = np.array([len(r) for r in ref], dtype=np.int32)
        flat = [iv for r in ref for iv in r]
        g = {"p_counts": counts,
             "p_ival": np.array([[iv[0], iv[1]] for iv in flat]).reshape(-1, 2),
             "p_cc": np.array([np.concatenate([iv[2], iv[3]]) for iv in flat]).reshape(-1, 6),
             "p_type": np.array([[iv[4], iv[5]] for iv in flat], dtype=np.int32).reshape(-1, 2)}
        length = 100.0 + 4 * c.radius
        push_records_equal(res, g, "p", exact=False, tol=1e-7 / length)
        assert counts.sum() > 100  # the sample cuts the mesh
