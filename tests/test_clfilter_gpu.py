"""LineCLFilter as a device pass (ocl_gb300_line_filter_device, one warp
per point list): the kept indices of every list equal the host filter's
(ocl_gb300_line_filter, pinned against the reference's LineCLFilter,
src/common/lineclfilter.cpp:40-77), bit for bit, on random lists of every
length class and on PathDropCutter output."""
import numpy as np
import pytest

from opencamlib_gb300 import _native
from opencamlib_gb300 import cutters as cu
from tests.helpers import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    if not t.cuda.is_available():
        pytest.fail("no CUDA device")
    return t


def device_filter(torch, lists, tol):
    sizes = [len(x) for x in lists]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    xyz = np.concatenate([np.asarray(x, dtype=np.float64).reshape(-1, 3) for x in lists]) if lists else np.zeros((0, 3))
    d_xyz = torch.from_numpy(np.ascontiguousarray(xyz)).cuda()
    d_off = torch.from_numpy(off.view(np.int64)).cuda()
    d_keep = torch.full((max(int(off[-1]), 1),), -1, dtype=torch.int64, device="cuda")
    d_n = torch.zeros(max(len(lists), 1), dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    _native.line_filter_device(d_xyz.data_ptr(), d_off.data_ptr(), len(lists), tol, d_keep.data_ptr(), d_n.data_ptr(), s)
    torch.cuda.synchronize()
    keep, n = d_keep.cpu().numpy(), d_n.cpu().numpy()
    return [keep[int(off[p]):int(off[p]) + int(n[p])].tolist() for p in range(len(lists))]


def test_random_lists_match_host(torch):
    rng = np.random.default_rng(7)
    lists = []
    for k in range(3000):
        n = int(rng.integers(0, 400)) if k % 10 else int(rng.integers(0, 4))
        t = np.cumsum(rng.uniform(0.01, 0.2, n))
        x = np.stack([t, np.sin(t * rng.uniform(0.1, 3)) * rng.uniform(0, 2), rng.normal(0, 0.01, n) * (k % 3)], axis=1)
        if k % 7 == 0:
            x[:, 1] = np.round(x[:, 1], 1)  # straight runs
        lists.append(x)
    for tol in (1e-4, 0.003, 0.05):
        got = device_filter(torch, lists, tol)
        for x, g in zip(lists, got):
            assert g == _native.line_filter(x, tol).tolist()


def test_path_drop_output(torch):
    """PathDropCutter points of many zig-zag lines, filtered on the device."""
    import opencamlib_gb300 as ocl
    g = golden("drop_heightfield")
    mesh = ocl.DeviceMesh(g["tris"])
    lists = []
    for k in range(40):
        y = 2.0 + 2.4 * k
        spans = np.array([[0, -2.0, y, 0, 102.0, y + 0.3 * (k % 3), 0, 0, 0, 0, 0]])
        xyz, _, _, _ = mesh.path_drop(cu.BallCutter(6.0, 20.0), spans, 0.05, -20.0)
        lists.append(xyz)
    got = device_filter(torch, lists, 0.01)
    for x, k in zip(lists, got):
        assert k == _native.line_filter(x, 0.01).tolist()
        assert k[0] == 0 and k[-1] == len(x) - 1
    assert sum(len(k) for k in got) < sum(len(x) for x in lists)
