"""The request loop (ocl_gb300_server_*): BatchDropCutter and
AdaptivePathDropCutter requests submitted from several threads against
device-resident meshes are admitted into shared batches (continuous
batching; adaptive requests send each bisection level through the next
batch).  Each result must equal, bit for bit, the same request run alone
(ocl_gb300_drop / ocl_gb300_adaptive_path_drop).  Failures are injected on
the host: an unknown mesh, a request larger than the budget allows, a
cancelled request."""
import math
import threading

import numpy as np
import pytest

from opencamlib_gb300 import _abi
from opencamlib_gb300 import cutters as cu
from opencamlib_gb300 import workloads as w

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import opencamlib_gb300 as ocl
    if not ocl.device_available():
        pytest.fail("no CUDA device")
    meshes = [ocl.DeviceMesh(w.mesh_of_size("heightfield", 30000, 3)),
              ocl.DeviceMesh(w.mesh_of_size("sphere", 12000, 4)), ocl.DeviceMesh(w.mesh_of_size("box", 20000, 5))]
    return ocl, meshes


CUTTERS = [cu.CylCutter(6.0, 20.0), cu.BallCutter(3.0, 20.0), cu.BullCutter(8.0, 1.5, 20.0),
           cu.ConeCutter(6.0, math.pi / 4, 20.0), cu.BallConeCutter(2.0, 6.0, math.pi / 4)]


def _requests(n, seed):
    """Seeded mix: half drops (100 .. 20,000 raster points), half adaptive
    paths (zig-zags of 2-6 lines across the mesh, sampling 0.5-2 mm)."""
    u = w.uniform(seed, 6 * n).reshape(n, 6)
    out = []
    for k in range(n):
        mesh = int(u[k, 0] * 3)
        c = CUTTERS[int(u[k, 1] * len(CUTTERS))]
        if k % 2 == 0:
            M = int(100 * 200 ** u[k, 2])
            side = max(1, int(math.sqrt(M)))
            cl = w.raster(side, max(1, M // side), 90.0 / side, z0=-60.0, x0=5.0 + u[k, 3], y0=5.0 + u[k, 4])
            out.append(("drop", mesh, c, cl))
        else:
            nl = 2 + int(u[k, 2] * 5)
            spans = []
            for j in range(nl):
                y = 10.0 + 80.0 * j / max(nl - 1, 1) + u[k, 3]
                a, b = (5.0, 95.0) if j % 2 == 0 else (95.0, 5.0)
                spans.append([0, a, y, -60.0, b, y + 3 * u[k, 4], -60.0, 0, 0, 0, 0])
            out.append(("adaptive", mesh, c, (np.array(spans), 0.5 + 1.5 * u[k, 5], 0.02)))
    return out


def _alone(meshes, req):
    kind, m, c, data = req
    if kind == "drop":
        z, cc, ty, _ = meshes[m].drop(c, data, precision="mixed")
        return z, cc, ty
    spans, samp, minsamp = data
    xyz, cc, ty, _ = meshes[m].adaptive_path_drop(c, spans, samp, minsamp)
    return xyz, cc, ty


def _submit(srv, ids, req):
    kind, m, c, data = req
    if kind == "drop":
        return srv.submit_drop(ids[m], c, data)
    spans, samp, minsamp = data
    return srv.submit_adaptive(ids[m], c, spans, samp, minsamp)


def test_mix_equals_alone(env):
    ocl, meshes = env
    reqs = _requests(24, 51)
    ref = [_alone(meshes, r) for r in reqs]
    srv = ocl.Server(hbm_budget_bytes=4 << 30, slots=2, max_batch_requests=8)
    ids = [srv.add_mesh(m) for m in meshes]
    handles = [None] * len(reqs)

    def client(part):
        for k in range(part, len(reqs), 4):
            handles[k] = _submit(srv, ids, reqs[k])

    th = [threading.Thread(target=client, args=(p,)) for p in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    batches = []
    for k, h in enumerate(handles):
        st, res, info = srv.wait(h)
        assert st == _abi.OK, (k, info)
        for a, b in zip(res, ref[k]):
            np.testing.assert_array_equal(a, b, err_msg=f"request {k}")
        batches.append(info["batches"])
        assert info["latency_ms"] >= info["queue_ms"] >= 0.0
    s = srv.stats()
    assert s["completed"] == len(reqs) and s["failed"] == 0
    assert 0.0 < s["p50_ms"] <= s["p99_ms"] <= s["max_ms"]
    assert s["batches"] < sum(batches)  # requests shared batches
    assert max(batches) > 1  # adaptive requests took one batch per level
    srv.close()


def test_injected_failures(env):
    ocl, meshes = env
    srv = ocl.Server(hbm_budget_bytes=64 << 20, slots=1)
    mid = srv.add_mesh(meshes[0])
    c = cu.BallCutter(6.0, 20.0)
    # an unknown mesh
    with pytest.raises(ocl.OclError) as e:
        srv.submit_drop(mid + 7, c, w.raster(10, 10, 1.0))
    assert e.value.status == _abi.BAD_ARG
    # an adaptive request whose first level holds more points than one
    # batch's buffers may under a 64 MiB budget (drops are split instead)
    many = np.array([[0, 5.0 + 1e-4 * k, 5.0, -60.0, 5.0 + 1e-4 * k, 95.0, -60.0, 0, 0, 0, 0] for k in range(200000)])
    with pytest.raises(ocl.OclError) as e:
        srv.submit_adaptive(mid, c, many, 1.0, 0.1)
    assert e.value.status == _abi.OOM
    # a cancelled request (admission paused so it is still queued)
    srv.pause(True)
    keep = srv.submit_drop(mid, c, w.raster(20, 20, 4.0, z0=-60.0))
    drop = srv.submit_drop(mid, c, w.raster(20, 20, 4.0, z0=-60.0))
    srv.cancel(drop)
    st, _, info = srv.wait(drop)
    assert st == _abi.CANCELLED
    srv.pause(False)
    st, res, _ = srv.wait(keep)
    assert st == _abi.OK
    np.testing.assert_array_equal(res[0], meshes[0].drop(c, w.raster(20, 20, 4.0, z0=-60.0))[0])
    # a timed-out wait leaves the request in place
    srv.pause(True)
    late = srv.submit_drop(mid, c, w.raster(5, 5, 4.0, z0=-60.0))
    assert srv.wait(late, timeout=0.05)[0] == _abi.PENDING
    srv.pause(False)
    assert srv.wait(late)[0] == _abi.OK
    s = srv.stats()
    assert s["rejected"] == 2 and s["cancelled"] == 1 and s["completed"] == 2
    srv.close()


def test_large_drop_split_over_batches(env):
    """A drop request larger than a batch goes through in pieces; each
    piece's points equal the request run alone, and a small request that
    arrives meanwhile finishes before the large one."""
    ocl, meshes = env
    c = cu.BullCutter(8.0, 1.5, 20.0)
    big = w.raster(200, 150, 0.5, z0=-60.0, x0=2.0, y0=3.0)
    small = w.raster(10, 10, 5.0, z0=-60.0, x0=7.0, y0=9.0)
    srv = ocl.Server(hbm_budget_bytes=2 << 30, slots=1, max_batch_points=4096)
    mid = srv.add_mesh(meshes[2])
    hb = srv.submit_drop(mid, c, big)
    hs = srv.submit_drop(mid, c, small)
    st, res_b, info_b = srv.wait(hb)
    assert st == _abi.OK
    st, res_s, info_s = srv.wait(hs)
    assert st == _abi.OK
    assert info_b["batches"] >= len(big) // 4096
    assert info_s["latency_ms"] < info_b["latency_ms"]  # the small one did not wait for all of the large one
    for a, b in zip(res_b, meshes[2].drop(c, big, precision="mixed")[:3]):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(res_s, meshes[2].drop(c, small, precision="mixed")[:3]):
        np.testing.assert_array_equal(a, b)
    srv.close()
