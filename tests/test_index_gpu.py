"""The integer part of the path, bit for bit.

* KD visit order: the device's trees (drop XY, push YZ/XZ) and the KD rank in
  every triangle record must equal the reference's KDTree order
  (src/common/kdtree.hpp:141-210 build, :273-304 search, hi before lo) --
  against golden orders made by the reference itself and against the oracle.
* Candidate sets: for every CL point, the triangles the device grid finds
  under the cutter and MillingCutter::overlaps accepts
  (src/cutters/millingcutter.cpp:422-433) must be exactly the set the
  reference forms in BatchDropCutter::dropCutter5 (KD search, then overlaps;
  src/dropcutter/batchdropcutter.cpp:208-222) -- the oracle's
  KD-search restatement gives the sets, compared per point, as sets."""
import numpy as np
import pytest

from opencamlib_gb300 import workloads as w
from tests.golden.cases import degenerate_mesh, degenerate_points
from tests.helpers import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ocl():
    import opencamlib_gb300 as ocl
    if not ocl.device_available():
        pytest.fail("no CUDA device")
    return ocl


@pytest.mark.parametrize("bucket", [1, 3])
@pytest.mark.parametrize("dims", [0, 1, 2])
def test_kd_order_matches_reference_golden(ocl, dims, bucket):
    g = golden("kd_order")
    mesh = ocl.DeviceMesh(g["tris"], bucket_size=bucket)
    np.testing.assert_array_equal(mesh.kd_order(dims), g[f"dims{dims}_b{bucket}"])
    if dims == 0:
        rank = np.empty(len(mesh), dtype=np.int64)
        rank[g[f"dims0_b{bucket}"]] = np.arange(len(mesh))
        np.testing.assert_array_equal(mesh.kd_rank(), rank)


@pytest.mark.parametrize("dims", [0, 1, 2])
def test_kd_order_matches_oracle_on_larger_meshes(ocl, oracle_lib, dims):
    for tris in (w.heightfield_c1(), w.sphere_torus(2), golden("real_mount_rush")["tris"].astype(np.float64)):
        mesh = ocl.DeviceMesh(tris)
        want = oracle_lib.kd_order(tris, "port", 1, dims)
        np.testing.assert_array_equal(mesh.kd_order(dims), want)
        if dims == 0:
            rank = np.empty(len(tris), dtype=np.int64)
            rank[want] = np.arange(len(tris))
            np.testing.assert_array_equal(mesh.kd_rank(), rank)


def _same_sets(got, want):
    go, gi = got
    wo, wi = want
    assert len(go) == len(wo)
    bad = np.nonzero(np.diff(go) != np.diff(wo))[0]
    assert len(bad) == 0, f"set sizes differ at {bad[:10]} (e.g. {np.diff(go)[bad[:3]]} vs {np.diff(wo)[bad[:3]]})"
    np.testing.assert_array_equal(gi, wi)


def test_overlap_sets_degenerate(ocl, oracle_lib):
    tris, cl = degenerate_mesh(), degenerate_points()
    mesh = ocl.DeviceMesh(tris)
    for r in (0.5, 3.0, 10.0):
        _same_sets(mesh.overlap_sets(r, cl), oracle_lib.overlap_sets(tris, r, cl))


def test_overlap_sets_c1_all_points(ocl, oracle_lib):
    # the whole 40,000-point raster of the 32,258-triangle bump field, Ball d6
    tris, cl = w.heightfield_c1(), w.raster_c1()
    mesh = ocl.DeviceMesh(tris)
    got = mesh.overlap_sets(3.0, cl)
    _same_sets(got, oracle_lib.overlap_sets(tris, 3.0, cl))
    assert got[0][-1] > 40000 * 100  # about 143 exact candidates per CL point


def test_overlap_sets_c2_subsample(ocl, oracle_lib):
    # 2,000 seeded points of the 1,000,000-point raster over the
    # 1,048,576-triangle mesh (about 4,000 exact candidates each)
    tris = w.mesh_c2()
    cl = w.raster_c2()[w.subsample(1000 * 1000, 2000, 23)]
    mesh = ocl.DeviceMesh(tris)
    for r in (3.0, 0.5):
        _same_sets(mesh.overlap_sets(r, cl), oracle_lib.overlap_sets(tris, r, cl))


def test_overlap_sets_edges_of_the_grid(ocl, oracle_lib):
    # points outside the mesh bbox, on cell boundaries and far away; radii
    # from below the cell size to larger than the mesh
    tris = w.heightfield(30, 25, seed=9, jitter=0.05, jitter_seed=10)
    mesh = ocl.DeviceMesh(tris)
    u = w.uniform(31, 3000).reshape(-1, 3)
    cl = np.stack([-40 + 180 * u[:, 0], -40 + 180 * u[:, 1], np.full(1000, -50.0)], axis=1)
    step = 100.0 / 29.0
    edge = np.array([[i * step, j * step, 0.0] for i in range(0, 30, 7) for j in range(0, 25, 6)])
    cl = np.concatenate([cl, edge, [[1e4, 1e4, 0.0], [-1e4, 50.0, 0.0]]])
    for r in (0.05, 1.0, 7.5, 150.0):
        _same_sets(mesh.overlap_sets(r, cl), oracle_lib.overlap_sets(tris, r, cl))


@pytest.mark.parametrize("name", ["sphere_on_plate", "wheel_in_box"])
def test_overlap_sets_real_meshes(ocl, oracle_lib, name):
    g = golden("real_" + name)
    tris = g["tris"].astype(np.float64)
    mesh = ocl.DeviceMesh(tris)
    for r in (1.0, 3.0):
        _same_sets(mesh.overlap_sets(r, g["cl"]), oracle_lib.overlap_sets(tris, r, g["cl"]))
