"""ocl_gb300_batch_*: many drop-cutter jobs in persistent work-stealing
launches captured in a CUDA graph.  Every job's results must equal, bit for
bit, what ocl_gb300_drop_device returns for that job alone -- with jobs cut
into several chunks, chunks spread over several waves, graph replays with
new inputs in the same buffers, and the autotuner choosing list capacities."""
import math

import numpy as np
import pytest

from opencamlib_gb300 import _abi
from opencamlib_gb300 import cutters as cu
from opencamlib_gb300 import workloads as w

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    import opencamlib_gb300 as ocl
    if not ocl.device_available() or not torch.cuda.is_available():
        pytest.fail("no CUDA device")
    return ocl, torch


def _mix(ocl):
    """A scaled-down mix: four meshes, the five families and the other
    composite presets, diameters 1-20 mm, 100 to 60,000 points."""
    meshes = {"hf": w.mesh_of_size("heightfield", 20000, 5), "sph": w.mesh_of_size("sphere", 8000, 6),
              "box": w.mesh_of_size("box", 30000, 7), "plate": w.grid_triangles(*np.meshgrid(
                  np.linspace(0, 12, 40), np.linspace(0, 12, 40)), np.zeros((40, 40)))}
    dev = {k: ocl.DeviceMesh(t) for k, t in meshes.items()}
    spec = [("hf", cu.BallCutter(6.0, 20.0), 60000), ("hf", cu.BullCutter(12.0, 2.0, 24.0), 20000),
            ("sph", cu.ConeCutter(4.0, math.pi / 4, 20.0), 9000), ("box", cu.CylCutter(20.0, 40.0), 15000),
            ("box", cu.BallConeCutter(2.0, 6.0, math.pi / 4), 30000), ("hf", cu.CylCutter(1.0, 20.0), 100),
            ("sph", cu.BullConeCutter(4.0, 1.0, 8.0, math.pi / 4), 5000), ("plate", cu.CylCutter(6.0, 20.0), 2000),
            ("box", cu.ConeConeCutter(2.0, math.pi / 3, 6.0, math.pi / 5), 7000),
            ("sph", cu.BallCutter(1.0, 20.0), 12000), ("hf", cu.CylConeCutter(2.0, 6.0, math.pi / 4), 25000)]
    jobs = []
    for k, (m, c, M) in enumerate(spec):
        pts = w.batch_points(meshes[m], M, c.radius)
        jobs.append((m, c, pts))
    return meshes, dev, jobs


def _alone(torch, dev, jobs):
    out = []
    for m, c, pts in jobs:
        z, cc, ty, st = dev[m].drop(c, pts, precision="mixed")
        assert st.violations == 0
        out.append((z, cc, ty))
    return out


def _device_buffers(torch, jobs):
    bufs = []
    for m, c, pts in jobs:
        M = len(pts)
        bufs.append((torch.from_numpy(pts).cuda(), torch.full((M,), np.nan, dtype=torch.float64, device="cuda"),
                     torch.full((M, 3), np.nan, dtype=torch.float64, device="cuda"),
                     torch.full((M,), -1, dtype=torch.int32, device="cuda")))
    return bufs


def _batch(ocl, dev, jobs, bufs, **kw):
    spec = [(dev[m], c, b[0].data_ptr(), len(pts), b[1].data_ptr(), b[2].data_ptr(), b[3].data_ptr())
            for (m, c, pts), b in zip(jobs, bufs)]
    return ocl.DropBatch(spec, **kw)


def _check(torch, bufs, ref):
    torch.cuda.synchronize()
    for k, (b, r) in enumerate(zip(bufs, ref)):
        np.testing.assert_array_equal(b[1].cpu().numpy(), r[0], err_msg=f"job {k} z")
        np.testing.assert_array_equal(b[2].cpu().numpy(), r[1], err_msg=f"job {k} cc")
        np.testing.assert_array_equal(b[3].cpu().numpy(), r[2], err_msg=f"job {k} type")


def test_batch_equals_single_calls(env):
    ocl, torch = env
    meshes, dev, jobs = _mix(ocl)
    ref = _alone(torch, dev, jobs)
    bufs = _device_buffers(torch, jobs)
    # chunks of 8,192 points and a workspace budget that forces several waves
    b = _batch(ocl, dev, jobs, bufs, chunk_points=8192, workspace_bytes=96 << 20, graph=True)
    info = b.info()
    assert info["jobs"] == len(jobs) and info["waves"] > 1 and info["chunks"] > len(jobs)
    st = b.run(stats=True)
    assert st.violations == 0 and st.iter_limit_hits == 0
    _check(torch, bufs, ref)
    # graph replay: the same buffers with new points (moved 0.37 mm in x)
    moved = [(m, c, pts + np.array([0.37, 0.0, 0.0])) for m, c, pts in jobs]
    for (m, c, pts), bb in zip(moved, bufs):
        bb[0].copy_(torch.from_numpy(pts))
        bb[1].fill_(np.nan)
    b.run()
    _check(torch, bufs, _alone(torch, dev, moved))
    b.release()


def test_batch_without_graph_and_one_wave(env):
    ocl, torch = env
    meshes, dev, jobs = _mix(ocl)
    ref = _alone(torch, dev, jobs)
    bufs = _device_buffers(torch, jobs)
    b = _batch(ocl, dev, jobs, bufs, graph=False)
    assert b.info()["waves"] == 1
    b.run()
    _check(torch, bufs, ref)


def test_batch_autotuned(env):
    ocl, torch = env
    meshes, dev, jobs = _mix(ocl)
    ref = _alone(torch, dev, jobs)
    bufs = _device_buffers(torch, jobs)
    b = _batch(ocl, dev, jobs, bufs, autotune=True, list_capacity=64)
    caps = [v["list_capacity"] for v in b.info()["variants"]]
    assert all(c in (64, 128, 256) for c in caps)
    for bb in bufs:  # the probe wrote into the outputs
        bb[1].fill_(np.nan)
    b.run()
    _check(torch, bufs, ref)


def test_batch_errors(env):
    ocl, torch = env
    meshes, dev, jobs = _mix(ocl)
    bufs = _device_buffers(torch, jobs[:2])
    with pytest.raises(ocl.OclError) as e:
        _batch(ocl, dev, jobs[:2], bufs, chunk_points=1 << 20, workspace_bytes=1 << 20)
    assert e.value.status == _abi.BAD_ARG
    with pytest.raises(ocl.OclError):
        _batch(ocl, dev, jobs[:2], bufs, list_capacity=4)


def test_batching_workload_sample_against_fp64(env):
    """Jobs of the 64-job batching workload (seeded heightfield, sphere and
    box meshes; the five cutter families at diameters up to 20 mm): each
    job's mixed results on a seeded sample of its points (scattered, so the
    sparse screen runs too) must equal the plain FP64 kernel's bit for bit.
    Every job whose mesh has at most 250,000 triangles (47 of the 64; job 34
    among them: a sphere whose pole fans out hundreds of thin triangles)."""
    ocl, torch = env
    specs = w.batch_jobs(seed=3, njobs=64)
    chosen = [k for k in range(len(specs)) if specs[k]["N"] <= 250000]
    rng = np.random.default_rng(5)
    for k in chosen:
        sp = specs[k]
        tris = w.mesh_of_size(sp["mesh"], sp["N"], sp["seed"])
        c = w.batch_cutter(sp["cutter"], sp["d"])
        pts = w.batch_points(tris, sp["M"], c.radius)
        sel = pts[np.sort(rng.choice(len(pts), size=min(len(pts), 1500), replace=False))]
        mesh = ocl.DeviceMesh(tris)
        z, cc, ty, st = mesh.drop(c, sel, precision="mixed")
        assert st.violations == 0, f"job {k}"
        z64, cc64, ty64, _ = mesh.drop(c, sel, precision="fp64")
        np.testing.assert_array_equal(z, z64, err_msg=f"job {k} z")
        np.testing.assert_array_equal(cc, cc64, err_msg=f"job {k} cc")
        np.testing.assert_array_equal(ty, ty64, err_msg=f"job {k} type")
        mesh.release()
