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
