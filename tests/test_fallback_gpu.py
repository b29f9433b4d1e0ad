"""Handed-back CL points on the GPU.

Points whose FP32 candidate list overflows are finished by the exact
per-point kernel (every triangle that may lift the point, sorted by the
reference's KD visit order, folded with the running-height skip), or, with
more candidates than that kernel holds, by the plain FP64 kernel.  A flat,
finely triangulated plate under a flat-bottomed cutter puts hundreds of
triangles at exactly the cutter's height, so every list overflows and the CC
point chosen among equal contacts must follow the reference's KD visit order
(CLPoint::liftZ lifts only on a strictly higher contact).  Results must equal
the oracle's bit for bit."""
import math

import numpy as np
import pytest

from opencamlib_gb300 import cutters as cu
from opencamlib_gb300 import workloads as w

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ocl():
    import opencamlib_gb300 as ocl
    if not ocl.device_available():
        pytest.fail("no CUDA device")
    return ocl


def flat_plate(n: int, size: float = 12.0) -> np.ndarray:
    xs = np.linspace(0.0, size, n)
    X, Y = np.meshgrid(xs, xs)
    return w.grid_triangles(X, Y, np.zeros_like(X))


def points(count: int, seed: int, lo: float = 1.0, hi: float = 11.0) -> np.ndarray:
    u = w.uniform(seed, 2 * count).reshape(-1, 2)
    return np.stack([lo + (hi - lo) * u[:, 0], lo + (hi - lo) * u[:, 1], np.full(count, -5.0)], axis=1)


def _same(got, ref):
    z, cc, ty = got[:3]
    zr, ccr, tyr = ref[:3]
    np.testing.assert_array_equal(z, zr)
    np.testing.assert_array_equal(ty, tyr)
    np.testing.assert_array_equal(cc, ccr)


CASES = {
    # 85 x 85 cells over 12 mm: ~2,800 triangles under a 6 mm cutter, ~300
    # of them at the height of a 2 mm flat centre
    "cyl": (86, lambda: cu.CylCutter(6.0, 20.0)),
    "cylcone": (86, lambda: cu.CylConeCutter(2.0, 6.0, math.pi / 4)),
    "bull": (86, lambda: cu.BullCutter(6.0, 1.0, 20.0)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_exact_kernel_matches_oracle(ocl, oracle_lib, name):
    n, make = CASES[name]
    tris = flat_plate(n)
    cl = points(240, 5)
    c = make()
    mesh = ocl.DeviceMesh(tris)
    z, cc, ty, st = mesh.drop(c, cl, precision="mixed")
    assert st.fallback > 0, "the plate should overflow the candidate lists"
    assert st.plain_points == 0
    assert st.violations == 0 and st.iter_limit_hits == 0
    _same((z, cc, ty), oracle_lib.drop(tris, c, cl, "port"))
    z64, cc64, ty64, _ = mesh.drop(c, cl, precision="fp64")
    _same((z, cc, ty), (z64, cc64, ty64))


LARGE = {
    # the composite folds in KD order: gathered into the exact kernel's
    # global scratch and folded one rank window at a time
    "compcyl": lambda: cu.CompCylCutter(6.0, 20.0),
    "cylcone": lambda: cu.CylConeCutter(2.0, 6.0, math.pi / 4),
    # the flat-bottomed basic cutters the same way
    "cyl": lambda: cu.CylCutter(6.0, 20.0),
    "bull": lambda: cu.BullCutter(6.0, 1.0, 20.0),
}


@pytest.mark.parametrize("name", sorted(LARGE))
def test_exact_kernel_windows_over_large_lists(ocl, oracle_lib, name):
    # 160 x 160 cells over 12 mm: ~10,000 triangles under a 6 mm cutter, more
    # than the exact kernel's shared memory holds
    tris = flat_plate(161)
    cl = points(64, 6)
    c = LARGE[name]()
    mesh = ocl.DeviceMesh(tris)
    z, cc, ty, st = mesh.drop(c, cl, precision="mixed")
    assert st.fallback > 0 and st.plain_points == 0
    assert st.violations == 0
    _same((z, cc, ty), oracle_lib.drop(tris, c, cl, "port"))
    _same((z, cc, ty), mesh.drop(c, cl, precision="fp64")[:3])


def test_plain_kernel_takes_the_largest_lists(ocl, oracle_lib):
    # 1024 x 1024 cells over 12 mm: ~400,000 tied triangles under a 6 mm
    # flat bottom, more than the exact kernel's global scratch holds
    tris = flat_plate(1025)
    cl = points(16, 6)
    mesh = ocl.DeviceMesh(tris)
    for c in (cu.CompCylCutter(6.0, 20.0), cu.CylCutter(6.0, 20.0)):
        z, cc, ty, st = mesh.drop(c, cl, precision="mixed")
        assert st.plain_points > 0
        assert st.violations == 0
        _same((z, cc, ty), oracle_lib.drop(tris, c, cl, "port"))


def test_fallback_on_a_tilted_plate(ocl, oracle_lib):
    # a gently tilted fine plate under a cone: ties broken by tiny height
    # differences, candidate lists still overflow for the flat cutters
    tris = flat_plate(86)
    tris[:, 2::3] = 1e-7 * tris[:, 0::3] + 2e-7 * tris[:, 1::3]
    cl = points(200, 7)
    for c in (cu.CylCutter(6.0, 20.0), cu.ConeCutter(6.0, math.pi / 4, 20.0),
              cu.BallConeCutter(2.0, 6.0, math.pi / 4)):
        mesh = ocl.DeviceMesh(tris)
        z, cc, ty, st = mesh.drop(c, cl, precision="mixed")
        assert st.violations == 0
        _same((z, cc, ty), oracle_lib.drop(tris, c, cl, "port"))


def test_handed_back_points_on_the_bump_field(ocl):
    # the 1,048,576-triangle bump field: cone and composite points whose
    # branch checks fail are redone by the exact kernel, which folds only the
    # triangles above a branch-safe threshold; mixed must equal plain FP64
    tris = w.mesh_c2()
    grid = w.raster_c2().reshape(1000, 1000, 3)
    cl = np.concatenate([grid[i:i + 100, j:j + 100].reshape(-1, 3)
                         for i, j in ((100, 100), (450, 600), (700, 250), (850, 850))])
    mesh = ocl.DeviceMesh(tris)
    handed_back = 0
    for c in (cu.ConeCutter(6.0, math.pi / 4, 20.0), cu.BallConeCutter(2.0, 6.0, math.pi / 4)):
        z, cc, ty, st = mesh.drop(c, cl, precision="mixed")
        assert st.violations == 0
        handed_back += st.fallback
        _same((z, cc, ty), mesh.drop(c, cl, precision="fp64")[:3])
    assert handed_back > 0


@pytest.mark.parametrize("name,cutter", [("cyl20", lambda: cu.CylCutter(20.0, 40.0)),
                                         ("bull12", lambda: cu.BullCutter(12.0, 2.0, 24.0)),
                                         ("ball10", lambda: cu.BallCutter(10.0, 20.0))])
def test_exact_kernel_with_tiny_lists(ocl, name, cutter):
    """Lists of 16 candidates hand almost every point of a box with fillets
    back to the exact kernel; its gather-sort-fold must equal the plain FP64
    kernel, which folds every candidate in KD order."""
    import torch
    tris = w.mesh_of_size("box", 30000, 7)
    c = cutter()
    pts = w.batch_points(tris, 15000, c.radius)
    mesh = ocl.DeviceMesh(tris)
    d_cl = torch.from_numpy(pts).cuda()
    M = len(pts)
    d_z = torch.empty(M, dtype=torch.float64, device="cuda")
    d_cc = torch.empty((M, 3), dtype=torch.float64, device="cuda")
    d_ty = torch.empty(M, dtype=torch.int32, device="cuda")
    b = ocl.DropBatch([(mesh, c, d_cl.data_ptr(), M, d_z.data_ptr(), d_cc.data_ptr(), d_ty.data_ptr())],
                      list_capacity=16)
    st = b.run(stats=True)
    torch.cuda.synchronize()
    assert st.violations == 0
    assert st.fallback > 0 or name == "ball10"  # a ball's lists rarely reach 16
    z64, cc64, ty64, _ = mesh.drop(c, pts, precision="fp64")
    _same((d_z.cpu().numpy(), d_cc.cpu().numpy(), d_ty.cpu().numpy()), (z64, cc64, ty64))


@pytest.mark.parametrize("name,cutter", [("cyl17", lambda: cu.CylCutter(17.0, 40.0)),
                                         ("bull18", lambda: cu.BullCutter(18.0, 3.0, 40.0)),
                                         ("ballcone", lambda: cu.BallConeCutter(2.0, 12.0, math.pi / 4))])
def test_large_cutters_on_a_heightfield_with_short_lists(ocl, name, cutter):
    """Large cutters over a heightfield with lists of 16 candidates (the
    batch autotuner's shortest): thousands of triangles under each cutter,
    points refined or handed back as their lists allow; the batch must equal
    the plain FP64 kernel bit for bit."""
    import torch
    tris = w.mesh_of_size("heightfield", 60000, 5)
    c = cutter()
    pts = w.batch_points(tris, 6000, c.radius)
    mesh = ocl.DeviceMesh(tris)
    d_cl = torch.from_numpy(pts).cuda()
    M = len(pts)
    d_z = torch.empty(M, dtype=torch.float64, device="cuda")
    d_cc = torch.empty((M, 3), dtype=torch.float64, device="cuda")
    d_ty = torch.empty(M, dtype=torch.int32, device="cuda")
    b = ocl.DropBatch([(mesh, c, d_cl.data_ptr(), M, d_z.data_ptr(), d_cc.data_ptr(), d_ty.data_ptr())],
                      list_capacity=16)
    st = b.run(stats=True)
    torch.cuda.synchronize()
    assert st.violations == 0
    z64, cc64, ty64, _ = mesh.drop(c, pts, precision="fp64")
    _same((d_z.cpu().numpy(), d_cc.cpu().numpy(), d_ty.cpu().numpy()), (z64, cc64, ty64))
