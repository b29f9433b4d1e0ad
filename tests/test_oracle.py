"""The CPU oracle (oracle/ocl_oracle.c) pinned against the reference: bit-exact
against the golden fixtures made by the reference itself, and, where the
reference tree is present, against the reference library on fresh seeds."""
import math

import numpy as np
import pytest

from opencamlib_gb300 import workloads as w
from tests.golden.cases import CUTTERS, degenerate_mesh, path_spans
from tests.helpers import golden, push_records_equal


@pytest.mark.parametrize("case", ["drop_heightfield", "drop_degenerate"])
@pytest.mark.parametrize("cname", sorted(CUTTERS))
def test_oracle_drop_matches_golden(oracle_lib, case, cname):
    g = golden(case)
    z, cc, ty, _ = oracle_lib.drop(g["tris"], CUTTERS[cname](), g["cl"], "port", nthreads=2)
    np.testing.assert_array_equal(z, g[f"{cname}_z"])
    np.testing.assert_array_equal(cc, g[f"{cname}_cc"])
    np.testing.assert_array_equal(ty, g[f"{cname}_type"])


@pytest.mark.parametrize("cname", sorted(CUTTERS))
def test_oracle_push_matches_golden(oracle_lib, cname):
    g = golden("push_heightfield")
    for d, key in ((0, "fib_x"), (1, "fib_y")):
        res, _ = oracle_lib.push(g["tris"], CUTTERS[cname](), d, g[key], "port", nthreads=2)
        push_records_equal(res, g, f"{cname}_{d}", exact=True, sort=False)


@pytest.mark.parametrize("cname", sorted(CUTTERS))
def test_oracle_paths_match_golden(oracle_lib, cname):
    g = golden("path_heightfield")
    xyz, cc, ty = oracle_lib.pdc(g["tris"], CUTTERS[cname](), g["spans"], 0.37, -5.0, "port")
    np.testing.assert_array_equal(xyz, g[f"{cname}_pdc_xyz"])
    np.testing.assert_array_equal(ty, g[f"{cname}_pdc_type"])
    xyz, cc, ty = oracle_lib.apdc(g["tris"], CUTTERS[cname](), g["spans"], 0.8, 0.05, 0.999, "port")
    np.testing.assert_array_equal(xyz, g[f"{cname}_apdc_xyz"])
    np.testing.assert_array_equal(cc, g[f"{cname}_apdc_cc"])
    np.testing.assert_array_equal(ty, g[f"{cname}_apdc_type"])


def test_oracle_kd_order_matches_golden(oracle_lib):
    g = golden("kd_order")
    for d in (0, 1, 2):
        for b in (1, 3):
            np.testing.assert_array_equal(oracle_lib.kd_order(g["tris"], "port", b, d), g[f"dims{d}_b{b}"])


def test_oracle_empty_and_outside(oracle_lib):
    tris = degenerate_mesh()
    cl = np.array([[500.0, 500.0, -7.0], [5.0, 5.0, 99.0]])
    for cname, make in CUTTERS.items():
        z, cc, ty, _ = oracle_lib.drop(tris, make(), cl, "port")
        assert z[0] == -7.0 and ty[0] == 0, cname
        assert z[1] == 99.0 and ty[1] == 0, cname
    z, cc, ty, _ = oracle_lib.drop(np.zeros((0, 9)), CUTTERS["ball"](), cl, "port")
    np.testing.assert_array_equal(z, cl[:, 2])


needs_ref = pytest.mark.skipif("not __import__('oracle.checker', fromlist=['x']).available('ref')",
                               reason="reference library not built (reference tree absent)")


@needs_ref
@pytest.mark.parametrize("seed", [3, 7])
@pytest.mark.parametrize("cname", sorted(CUTTERS))
def test_oracle_drop_matches_reference_fresh_seed(oracle_lib, seed, cname):
    tris = w.heightfield(20, 17, seed=seed, jitter=0.05, jitter_seed=seed + 100)
    u = w.uniform(seed + 1000, 600).reshape(-1, 2)
    cl = np.stack([-8 + 116 * u[:, 0], -8 + 116 * u[:, 1], np.full(300, -50.0)], axis=1)
    a = oracle_lib.drop(tris, CUTTERS[cname](), cl, "ref", nthreads=1)
    b = oracle_lib.drop(tris, CUTTERS[cname](), cl, "port", nthreads=1)
    for x, y in zip(a[:3], b[:3]):
        np.testing.assert_array_equal(x, y)
    assert a[3] == b[3]  # single-threaded call counts agree too


@needs_ref
@pytest.mark.parametrize("cname", ["ball", "bull", "cone", "cyl", "ballcone"])
def test_oracle_push_matches_reference_fresh_seed(oracle_lib, cname):
    tris = w.heightfield(18, 15, seed=5, jitter=0.05, jitter_seed=9)
    for d in (0, 1):
        fib = np.concatenate([w.fibers(d, z, -4.0, 104.0, 23, -10.0, 110.0) for z in (10.5, 14.0)])
        a, _ = oracle_lib.push(tris, CUTTERS[cname](), d, fib, "ref", nthreads=1)
        b, _ = oracle_lib.push(tris, CUTTERS[cname](), d, fib, "port", nthreads=1)
        assert len(a) == len(b)
        for ra, rb in zip(a, b):
            assert len(ra) == len(rb)
            for x, y in zip(ra, rb):
                assert x[0] == y[0] and x[1] == y[1] and x[4] == y[4] and x[5] == y[5]
                np.testing.assert_array_equal(x[2], y[2])
                np.testing.assert_array_equal(x[3], y[3])


@needs_ref
def test_presets_match_reference_constructors(oracle_lib):
    from opencamlib_gb300 import cutters as cu
    cases = [(1, (6, 20), cu.CompCylCutter(6, 20)), (2, (6, 20), cu.CompBallCutter(6, 20)),
             (3, (2, 6, math.pi / 4), cu.CylConeCutter(2, 6, math.pi / 4)),
             (4, (2, 6, math.pi / 4), cu.BallConeCutter(2, 6, math.pi / 4)),
             (5, (4, 1, 8, math.pi / 4), cu.BullConeCutter(4, 1, 8, math.pi / 4)),
             (6, (2, math.pi / 3, 6, math.pi / 5), cu.ConeConeCutter(2, math.pi / 3, 6, math.pi / 5))]
    for preset, args, c in cases:
        np.testing.assert_array_equal(oracle_lib.ref_preset_fields(preset, args), oracle_lib.cutter_fields(c))
