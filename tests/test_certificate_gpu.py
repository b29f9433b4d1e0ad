"""The FP32 screen's certificate where it is tightest.

The mixed path leaves a triangle (or one facet, vertex or edge of it) out of
the FP64 fold only when an FP32 bound certifies it cannot change the result.
On adversarial meshes -- near-vertical facets (nz down to 1e-4), 0.005 mm
triangles and slivers, meshes 2,000 mm from the origin or spread over
4,000 mm -- and for cutter diameters 1, 6 and 20 mm of all five families:

* ocl_gb300_certificate_check evaluates every exact-overlap pair's FP64
  contacts on their own and counts any that exceed the bound the path relies
  on (the screen's [lo, hi], the refinement's part skips, the grid-entry
  cull, the bull's planned-edge bound): all counts must be 0;
* mixed equals plain FP64 bit for bit (z, CC point, CC type) with no
  violation of the certified lower bound;
* both equal the oracle within 1e-5 mm with identical CC types."""
import math

import numpy as np
import pytest

from opencamlib_gb300 import cutters as cu
from opencamlib_gb300 import workloads as w

pytestmark = pytest.mark.gpu

ZTOL = 1e-5


def family(d):
    """The five cutter families at diameter d (bull corner d/6, cones 45 deg,
    ball-cone d/3 inside d)."""
    L = max(20.0, 2 * d)
    return {
        "cyl": cu.CylCutter(d, L),
        "ball": cu.BallCutter(d, L),
        "bull": cu.BullCutter(d, d / 6.0, L),
        "cone": cu.ConeCutter(d, math.pi / 4, L),
        "ballcone": cu.BallConeCutter(d / 3.0, d, math.pi / 4),
    }


def cliffs():
    """Steps of 10 mm whose walls span 0.001, 0.01 and 0.1 mm in x: facets
    with nz about 1e-4, 1e-3 and 1e-2, on a gently waved floor."""
    xs = np.linspace(0.0, 40.0, 41)
    walls = [(10.0, 1e-3), (20.0, 1e-2), (30.0, 1e-1)]
    xs = np.unique(np.concatenate([xs] + [[c - h / 2, c + h / 2] for c, h in walls]))
    ys = np.linspace(0.0, 30.0, 31)
    X, Y = np.meshgrid(xs, ys)
    step = ((X > 10.0).astype(float) - (X > 20.0) + (X > 30.0)) * 10.0
    Z = step + 0.3 * np.sin(Y / 3.0) + 0.05 * X
    return w.grid_triangles(X, Y, Z)


def tiny_and_slivers():
    """A 0.495 mm patch of 0.005 mm triangles (a fine ripple), a fan of
    slivers (long thin triangles, widths 1e-6 .. 1e-3 mm) and a coarse base."""
    xs = 5.0 + 0.005 * np.arange(100)
    X, Y = np.meshgrid(xs, xs)
    Z = 3.0 + 0.02 * np.sin(40.0 * X) * np.cos(40.0 * Y)
    patch = w.grid_triangles(X, Y, Z)
    u = w.uniform(77, 5 * 300).reshape(300, 5)
    sl = []
    for k in range(300):
        cx, cy = 10.0 + 10.0 * u[k, 0], 10.0 + 10.0 * u[k, 1]
        a = 2 * math.pi * u[k, 2]
        L = 0.01 * 10 ** (3.3 * u[k, 3])
        eps = 10 ** (-6 + 3 * u[k, 4])
        z0 = 2.0 + u[k, 4]
        bx, by = cx + L * math.cos(a), cy + L * math.sin(a)
        sl.append([cx, cy, z0, bx, by, z0 + 0.5, bx - eps * math.sin(a), by + eps * math.cos(a), z0 + 0.5 + eps])
    base = w.heightfield(9, 9, seed=5, size=30.0)
    base[:, 2::3] -= 30.0  # below the patch and the slivers
    return np.concatenate([patch, np.array(sl), base])


def far_translated():
    """The bump field moved to (+2000, -2000, +500) mm."""
    t = w.heightfield(40, 40, seed=3, jitter=0.02, jitter_seed=4)
    t[:, 0::3] += 2000.0
    t[:, 1::3] -= 2000.0
    t[:, 2::3] += 500.0
    return t


def far_split():
    """Two 30 mm bump patches 4,000 mm apart: the FP32 local frame sits in
    between, so every coordinate is about 2,000 mm from its origin."""
    a = w.heightfield(20, 20, seed=6, size=30.0)
    b = w.heightfield(20, 20, seed=7, size=30.0)
    a[:, 0::3] -= 2000.0
    a[:, 1::3] -= 2000.0
    b[:, 0::3] += 2000.0
    b[:, 1::3] += 2000.0
    return np.concatenate([a, b])


def bumps():
    return w.heightfield(48, 48, seed=2, jitter=0.01, jitter_seed=3)


MESHES = {"cliffs": cliffs, "tiny_slivers": tiny_and_slivers, "far_translated": far_translated,
          "far_split": far_split, "bumps": bumps}


def points(tris, n, seed, r):
    """Uniform over the bbox widened by the radius, plus points near vertices."""
    p = tris.reshape(-1, 3)
    lo, hi = p.min(axis=0), p.max(axis=0)
    u = w.uniform(seed, 2 * n).reshape(n, 2)
    a = np.stack([lo[0] - r + (hi[0] - lo[0] + 2 * r) * u[:, 0], lo[1] - r + (hi[1] - lo[1] + 2 * r) * u[:, 1]], axis=1)
    k = (w.uniform(seed + 1, n // 4) * len(p)).astype(int)
    v = w.uniform(seed + 2, n // 2).reshape(-1, 2) - 0.5
    b = p[k, :2] + 1e-3 * v
    xy = np.concatenate([a, b])
    return np.concatenate([xy, np.full((len(xy), 1), lo[2] - 10.0)], axis=1)


@pytest.fixture(scope="module")
def ocl():
    import opencamlib_gb300 as ocl
    if not ocl.device_available():
        pytest.fail("no CUDA device")
    return ocl


@pytest.fixture(scope="module")
def meshes(ocl):
    out = {}
    for name, make in MESHES.items():
        t = make()
        out[name] = (t, ocl.DeviceMesh(t))
    return out


STRICT = ("tri_hi_exceeded", "tri_lo_exceeded", "part_hi_exceeded", "entry_ub_exceeded", "alt_hi_exceeded")


@pytest.mark.parametrize("d", [1.0, 6.0, 20.0])
@pytest.mark.parametrize("name", sorted(MESHES))
def test_certificate_holds(ocl, oracle_lib, meshes, name, d):
    tris, mesh = meshes[name]
    n = 800 if name != "tiny_slivers" else 400
    for cname, c in family(d).items():
        cl = points(tris, n, 100 + int(d), c.radius)
        cert = mesh.certificate(c, cl)
        assert cert["pairs"] > 0
        bad = {k: cert[k] for k in STRICT if cert[k]}
        assert not bad, f"{name} {cname} d={d}: {bad} {cert}"
        zm, ccm, tym, sm = mesh.drop(c, cl, precision="mixed")
        z64, cc64, ty64, _ = mesh.drop(c, cl, precision="fp64")
        assert sm.violations == 0 and sm.iter_limit_hits == 0, (name, cname)
        np.testing.assert_array_equal(zm, z64, err_msg=f"{name} {cname}")
        np.testing.assert_array_equal(tym, ty64, err_msg=f"{name} {cname}")
        np.testing.assert_array_equal(ccm, cc64, err_msg=f"{name} {cname}")
        sub = slice(0, None, 4)
        zr, ccr, tyr, _ = oracle_lib.drop(tris, c, cl[sub], "port")
        assert np.abs(zm[sub] - zr).max() <= ZTOL, (name, cname)
        np.testing.assert_array_equal(tym[sub], tyr, err_msg=f"{name} {cname}")


def test_certificate_check_sees_the_pairs(ocl, oracle_lib, meshes):
    # the check covers the exact-overlap pairs (the reference's count) and a
    # cutter starting below the mesh lifts on most of them
    tris, mesh = meshes["bumps"]
    c = family(6.0)["ball"]
    cl = points(tris, 200, 5, c.radius)
    cert = mesh.certificate(c, cl)
    assert cert["pairs"] == oracle_lib.overlap_pairs(tris, c.radius, cl)
    assert cert["pairs"] >= cert["lifted"] > cert["pairs"] // 4
    assert cert["error_budget"] > 0 and cert["guard"] > cert["error_budget"]
