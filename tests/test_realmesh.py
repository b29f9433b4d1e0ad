"""The reference's own meshes (its stl/ folder: sphere_on_plate, 30sphere,
mount_rush, wheel_in_box), with drop-cutter results for the five cutters of
the precision workload and push-cutter intervals on sphere_on_plate, made by
the reference build itself (tests/golden/make_golden.py).

CPU: the oracle (C restatement) reproduces them bit for bit.
GPU: the CUDA path, mixed and plain FP64, within 1e-5 mm with identical CC
types; push intervals in the reference's order within 1e-7 mm."""
import numpy as np
import pytest

from tests.golden.cases import CUTTERS
from tests.helpers import golden, push_records_equal

MESHES = ("sphere_on_plate", "30sphere", "mount_rush", "wheel_in_box")
DROP_CUTTERS = ("cyl", "ball", "bull", "cone", "ballcone")
ZTOL = 1e-5


def _mesh(name):
    g = golden("real_" + name)
    return g, g["tris"].astype(np.float64)


@pytest.mark.parametrize("name", MESHES)
def test_oracle_reproduces_reference_on_real_meshes(oracle_lib, name):
    g, tris = _mesh(name)
    for cname in DROP_CUTTERS:
        z, cc, ty, _ = oracle_lib.drop(tris, CUTTERS[cname](), g["cl"], "port")
        np.testing.assert_array_equal(z, g[f"{cname}_z"])
        np.testing.assert_array_equal(cc, g[f"{cname}_cc"])
        np.testing.assert_array_equal(ty, g[f"{cname}_type"])


def test_oracle_push_on_sphere_on_plate(oracle_lib):
    g, tris = _mesh("sphere_on_plate")
    for cname in ("ball", "bull"):
        for d, key in ((0, "fib_x"), (1, "fib_y")):
            res, _ = oracle_lib.push(tris, CUTTERS[cname](), d, g[key], "port")
            push_records_equal(res, g, f"{cname}_{d}", exact=True)


@pytest.fixture(scope="module")
def ocl():
    import opencamlib_gb300 as ocl
    if not ocl.device_available():
        pytest.fail("no CUDA device")
    return ocl


@pytest.mark.gpu
@pytest.mark.parametrize("name", MESHES)
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_gpu_drop_on_real_meshes(ocl, name, prec):
    g, tris = _mesh(name)
    mesh = ocl.DeviceMesh(tris)
    for cname in DROP_CUTTERS:
        z, cc, ty, st = mesh.drop(CUTTERS[cname](), g["cl"], precision=prec)
        assert st.violations == 0 and st.iter_limit_hits == 0
        dz = np.abs(z - g[f"{cname}_z"])
        assert dz.max() <= ZTOL, (cname, dz.max())
        np.testing.assert_array_equal(ty, g[f"{cname}_type"])
        lifted = ty != 0
        assert np.abs(cc[lifted] - g[f"{cname}_cc"][lifted]).max(initial=0.0) <= ZTOL


@pytest.mark.gpu
def test_gpu_mixed_equals_fp64_on_real_meshes(ocl):
    for name in MESHES:
        g, tris = _mesh(name)
        mesh = ocl.DeviceMesh(tris)
        for cname in DROP_CUTTERS:
            a = mesh.drop(CUTTERS[cname](), g["cl"], precision="mixed")
            b = mesh.drop(CUTTERS[cname](), g["cl"], precision="fp64")
            for x, y in zip(a[:3], b[:3]):
                np.testing.assert_array_equal(x, y)


@pytest.mark.gpu
@pytest.mark.parametrize("cname", ["ball", "bull"])
def test_gpu_push_on_sphere_on_plate(ocl, cname):
    g, tris = _mesh("sphere_on_plate")
    mesh = ocl.DeviceMesh(tris)
    for d, key in ((0, "fib_x"), (1, "fib_y")):
        res, st = mesh.push(CUTTERS[cname](), d, g[key])
        assert st.iter_limit_hits == 0
        fib = g[key]
        length = np.linalg.norm(fib[0, 3:] - fib[0, :3])
        push_records_equal(res, g, f"{cname}_{d}", exact=False, tol=1e-7 / length)
