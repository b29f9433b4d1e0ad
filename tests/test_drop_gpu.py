"""Drop-cutter parity on the GPU: the CUDA path against the reference's
golden fixtures and against the CPU oracle.

Tolerances: z within 1e-5 mm of the reference (the workload's stated bound);
CC points within 1e-5 mm; CC types identical.  The mixed-precision path must
return exactly the plain FP64 path's doubles (the FP32 screen only decides
which triangles are evaluated in FP64)."""
import math

import numpy as np
import pytest

from opencamlib_gb300 import workloads as w
from tests.golden.cases import CUTTERS
from tests.helpers import golden

pytestmark = pytest.mark.gpu

ZTOL = 1e-5


@pytest.fixture(scope="module")
def ocl():
    import opencamlib_gb300 as ocl
    if not ocl.device_available():
        pytest.fail("no CUDA device")
    return ocl


def _cmp(z, cc, ty, zr, ccr, tyr, exact_types=True):
    dz = np.abs(z - zr)
    assert np.max(dz) <= ZTOL, f"max|dz|={np.max(dz)} at {np.argmax(dz)}"
    lifted = tyr != 0
    if lifted.any():
        assert np.max(np.abs(cc[lifted] - ccr[lifted])) <= 1e-5
    match = np.mean(ty == tyr)
    if exact_types:
        assert match == 1.0, f"CC type match {match}"
    return match


@pytest.mark.parametrize("case", ["drop_heightfield", "drop_degenerate"])
@pytest.mark.parametrize("cname", sorted(CUTTERS))
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_drop_matches_golden(ocl, case, cname, prec):
    g = golden(case)
    mesh = ocl.DeviceMesh(g["tris"])
    z, cc, ty, st = mesh.drop(CUTTERS[cname](), g["cl"], precision=prec)
    assert st.violations == 0 and st.iter_limit_hits == 0
    _cmp(z, cc, ty, g[f"{cname}_z"], g[f"{cname}_cc"], g[f"{cname}_type"])


@pytest.mark.parametrize("cname", sorted(CUTTERS))
@pytest.mark.parametrize("seed", [11, 12])
def test_mixed_equals_fp64_and_oracle(ocl, oracle_lib, cname, seed):
    tris = w.heightfield(40, 33, seed=seed, jitter=0.03, jitter_seed=seed + 7)
    u = w.uniform(seed + 99, 4000).reshape(-1, 2)
    cl = np.stack([-5 + 110 * u[:, 0], -5 + 110 * u[:, 1], np.full(2000, -50.0)], axis=1)
    mesh = ocl.DeviceMesh(tris)
    c = CUTTERS[cname]()
    z64, cc64, ty64, s64 = mesh.drop(c, cl, precision="fp64")
    zm, ccm, tym, sm = mesh.drop(c, cl, precision="mixed")
    np.testing.assert_array_equal(zm, z64)
    np.testing.assert_array_equal(ccm, cc64)
    np.testing.assert_array_equal(tym, ty64)
    assert sm.violations == 0
    zr, ccr, tyr, _ = oracle_lib.drop(tris, c, cl, "port")
    _cmp(z64, cc64, ty64, zr, ccr, tyr)
    # the FP64 path evaluates exactly the reference's overlap pairs
    assert s64.pairs == oracle_lib.overlap_pairs(tris, c.radius, cl)


def test_bull_near_a_sphere_pole(ocl, oracle_lib):
    """Near the pole of a UV sphere hundreds of thin triangles share one
    vertex, and a bull's point plans more edges than the per-point count
    holds (it saturates at 255): the fold must keep testing the edges past
    the count itself.  Three points whose highest contact lies on such an
    edge; mixed must equal plain FP64 bit for bit, and the oracle."""
    from opencamlib_gb300 import cutters as cu
    tris = w.mesh_of_size("sphere", 213172, 3034)
    d = 8.047591839070233
    c = cu.BullCutter(d, d / 6.0, 20.0)
    pts = np.array([[48.36041448314995, 47.790720164255156, -50.0],
                    [48.196455931464946, 47.95437052245848, -50.0],
                    [47.86853882809494, 48.28167123886512, -50.0]])
    mesh = ocl.DeviceMesh(tris)
    z, cc, ty, st = mesh.drop(c, pts, precision="mixed")
    assert st.violations == 0
    z64, cc64, ty64, _ = mesh.drop(c, pts, precision="fp64")
    np.testing.assert_array_equal(z, z64)
    np.testing.assert_array_equal(cc, cc64)
    np.testing.assert_array_equal(ty, ty64)
    # the bull's device trigonometry may differ from the host's by an ulp
    zr, ccr, tyr = oracle_lib.drop(tris, c, pts, "port")[:3]
    np.testing.assert_allclose(z, zr, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(ty, tyr)
