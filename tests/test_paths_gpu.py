"""PathDropCutter / AdaptivePathDropCutter parity on the GPU against the
reference's golden fixtures (points within 1e-7 mm, CC types identical;
the adaptive sampler must produce the same number of points in the same
order)."""
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


@pytest.mark.parametrize("cname", sorted(CUTTERS))
def test_path_drop_matches_golden(ocl, cname):
    g = golden("path_heightfield")
    mesh = ocl.DeviceMesh(g["tris"])
    xyz, cc, ty, st = mesh.path_drop(CUTTERS[cname](), g["spans"], 0.37, -5.0)
    assert xyz.shape == g[f"{cname}_pdc_xyz"].shape
    assert np.max(np.abs(xyz - g[f"{cname}_pdc_xyz"])) <= 1e-7
    np.testing.assert_array_equal(ty, g[f"{cname}_pdc_type"])


@pytest.mark.parametrize("cname", sorted(CUTTERS))
def test_adaptive_path_drop_matches_golden(ocl, cname):
    g = golden("path_heightfield")
    mesh = ocl.DeviceMesh(g["tris"])
    xyz, cc, ty, st = mesh.adaptive_path_drop(CUTTERS[cname](), g["spans"], 0.8, 0.05, 0.999)
    ref = g[f"{cname}_apdc_xyz"]
    assert xyz.shape == ref.shape
    assert np.max(np.abs(xyz - ref)) <= 1e-7
    np.testing.assert_array_equal(ty, g[f"{cname}_apdc_type"])
