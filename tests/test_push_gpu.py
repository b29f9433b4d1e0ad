"""Push-cutter parity on the GPU against the reference's golden fixtures and
the CPU oracle.  Interval endpoints within 1e-7 mm (|dt| * fiber length), CC
points within 1e-7 mm, CC types identical, intervals in the reference's
order (Fiber::ints after the reference's merges)."""
import numpy as np
import pytest

from opencamlib_gb300 import workloads as w
from tests.golden.cases import CUTTERS
from tests.helpers import golden

pytestmark = pytest.mark.gpu

MMTOL = 1e-7


@pytest.fixture(scope="module")
def ocl():
    import opencamlib_gb300 as ocl
    if not ocl.device_available():
        pytest.fail("no CUDA device")
    return ocl


def _cmp_fibers(res, ref, fibers):
    assert len(res) == len(ref)
    for f, (a, b) in enumerate(zip(res, ref)):
        L = float(np.linalg.norm(fibers[f, 3:6] - fibers[f, 0:3]))
        assert len(a) == len(b), (f, a, b)
        for x, y in zip(a, b):
            assert abs(x[0] - y[0]) * L <= MMTOL and abs(x[1] - y[1]) * L <= MMTOL, (f, x[:2], y[:2])
            assert np.max(np.abs(np.asarray(x[2]) - np.asarray(y[2]))) <= MMTOL
            assert np.max(np.abs(np.asarray(x[3]) - np.asarray(y[3]))) <= MMTOL
            assert x[4] == y[4] and x[5] == y[5], (f, x, y)


def _golden_records(g, prefix):
    counts = g[prefix + "_counts"]
    iv, cc, ty = g[prefix + "_ival"], g[prefix + "_cc"], g[prefix + "_type"]
    out, k = [], 0
    for n in counts:
        out.append([(iv[k + j, 0], iv[k + j, 1], cc[k + j, :3], cc[k + j, 3:], int(ty[k + j, 0]), int(ty[k + j, 1]))
                    for j in range(int(n))])
        k += int(n)
    return out


@pytest.mark.parametrize("cname", sorted(CUTTERS))
def test_push_matches_golden(ocl, cname):
    g = golden("push_heightfield")
    mesh = ocl.DeviceMesh(g["tris"])
    for d, key in ((0, "fib_x"), (1, "fib_y")):
        res, st = mesh.push(CUTTERS[cname](), d, g[key])
        assert st.iter_limit_hits == 0
        _cmp_fibers(res, _golden_records(g, f"{cname}_{d}"), g[key])


@pytest.mark.parametrize("cname", ["ball", "bull", "cyl", "cone", "ballcone"])
def test_push_matches_oracle_sphere_torus(ocl, oracle_lib, cname):
    tris = w.sphere_torus(scale=2)
    mesh = ocl.DeviceMesh(tris)
    for d in (0, 1):
        fib = np.concatenate([w.fibers(d, z, -8.0, 108.0, 40, -10.0, 110.0) for z in (1.0, 9.5, 22.0)])
        res, _ = mesh.push(CUTTERS[cname](), d, fib)
        ref, _ = oracle_lib.push(tris, CUTTERS[cname](), d, fib, "port")
        _cmp_fibers(res, ref, fib)
