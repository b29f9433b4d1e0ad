"""ocl_gb300_drop_device_noalloc: the drop-cutter entry point for callers
that cannot allocate device memory while they run (a machine-control loop
with a fixed device-memory budget, or a process whose own pool allocator owns
the device).  It must return what the allocating entry point returns, call
after call, although every call reuses one fixed scratch array inside the
library.  Collected last so a failure here never hides another test."""
import ctypes as C
import math

import numpy as np
import pytest

from opencamlib_gb300 import _abi
from opencamlib_gb300 import workloads as w

pytestmark = pytest.mark.gpu



@pytest.fixture(scope="module")
def env():
    import torch

    import opencamlib_gb300 as ocl
    if not ocl.device_available() or not torch.cuda.is_available():
        pytest.fail("no CUDA device")
    return ocl, torch


def _noalloc(ocl, torch, mesh, cutter, cl):
    L = ocl.lib()
    M = cl.shape[0]
    d_cl = torch.from_numpy(np.ascontiguousarray(cl)).to("cuda")
    d_z = torch.full((M,), float("nan"), dtype=torch.float64, device="cuda")
    d_cc = torch.full((M, 3), float("nan"), dtype=torch.float64, device="cuda")
    d_ty = torch.full((M,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    desc = cutter.desc()
    st = L.ocl_gb300_drop_device_noalloc(mesh.handle, C.byref(desc), C.c_void_p(d_cl.data_ptr()), M,
                                         C.c_void_p(d_z.data_ptr()), C.c_void_p(d_cc.data_ptr()),
                                         C.c_void_p(d_ty.data_ptr()), None)
    assert st == 0, L.ocl_gb300_last_error().decode()
    torch.cuda.synchronize()
    return d_z.cpu().numpy(), d_cc.cpu().numpy(), d_ty.cpu().numpy()


def _check(got, ref):
    # the same kernels on the same inputs: the results are the allocating
    # entry point's doubles and CC types exactly
    for a, b in zip(got, ref):
        np.testing.assert_array_equal(a, b)


def test_noalloc_matches_drop_two_calls_in_a_row(env):
    ocl, torch = env
    tris = w.heightfield(64, 64, seed=4, jitter=0.02, jitter_seed=5)
    mesh = ocl.DeviceMesh(tris)
    # first call: many points, bull cutter; second: fewer points, ball cutter,
    # so stale scratch contents from the first call would show
    cl1 = w.raster(90, 90, 100.0 / 89.0, z0=-50.0)
    cl2 = w.raster(50, 40, 2.0, z0=-20.0, x0=1.3, y0=2.1)
    for cutter, cl in ((ocl.BullCutter(6.0, 1.0, 20.0), cl1), (ocl.BallCutter(6.0, 20.0), cl2)):
        ref = mesh.drop(cutter, cl, precision="mixed")[:3]
        _check(_noalloc(ocl, torch, mesh, cutter, cl), ref)


def test_noalloc_cone_and_composite(env):
    ocl, torch = env
    tris = w.heightfield(48, 40, seed=6)
    mesh = ocl.DeviceMesh(tris)
    cl = w.raster(90, 80, 1.2, z0=-50.0)
    for cutter in (ocl.ConeCutter(6.0, math.pi / 4, 20.0), ocl.BallConeCutter(2.0, 6.0, math.pi / 4)):
        ref = mesh.drop(cutter, cl, precision="mixed")[:3]
        _check(_noalloc(ocl, torch, mesh, cutter, cl), ref)


def test_noalloc_hands_back_overflowing_points(env):
    # a fine flat plate under flat-bottomed cutters: hundreds of triangles at
    # the cutter's height, so every 64-entry list overflows and the points
    # go to the handed-back kernels (exact per-point fold, plain FP64) that
    # work in the same fixed array; two calls in a row
    ocl, torch = env
    xs = np.linspace(0.0, 12.0, 86)
    X, Y = np.meshgrid(xs, xs)
    tris = w.grid_triangles(X, Y, np.zeros_like(X))
    mesh = ocl.DeviceMesh(tris)
    u = w.uniform(5, 480).reshape(-1, 2)
    cl = np.stack([1.0 + 10.0 * u[:, 0], 1.0 + 10.0 * u[:, 1], np.full(240, -5.0)], axis=1)
    for cutter in (ocl.CylCutter(6.0, 20.0), ocl.CylConeCutter(2.0, 6.0, math.pi / 4)):
        ref = mesh.drop(cutter, cl, precision="mixed")
        assert ref[3].fallback > 0  # the allocating path hands these points back too
        _check(_noalloc(ocl, torch, mesh, cutter, cl), ref[:3])


def test_noalloc_rejects_too_many_points(env):
    ocl, torch = env
    mesh = ocl.DeviceMesh(w.heightfield(8, 8, seed=1))
    L = ocl.lib()
    M = 8192 + 1
    desc = ocl.BallCutter(6.0, 20.0).desc()
    st = L.ocl_gb300_drop_device_noalloc(mesh.handle, C.byref(desc), C.c_void_p(1), M, C.c_void_p(1),
                                         C.c_void_p(1), C.c_void_p(1), None)
    assert st == _abi.BAD_ARG
    assert "exceed" in L.ocl_gb300_last_error().decode()
