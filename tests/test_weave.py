"""The host weave (ocl_gb300_weave: Weave::build + face_traverse,
src/algo/simple_weave.cpp:55-161, src/algo/weave.cpp:49-73) against the
reference's own SimpleWeave: on the fibers of the reference's Waterline and
AdaptiveWaterline runs stored in the golden fixtures (every machine), and,
where the reference is built, on fresh meshes and on random fiber sets.
Loops are compared as cyclic point sequences (the reference's starting
vertex and loop order follow its allocator's addresses)."""
import math

import numpy as np
import pytest

from opencamlib_gb300 import _abi, _native
from opencamlib_gb300 import cutters as cu
from opencamlib_gb300 import workloads as w
from oracle import checker
from tests.helpers import golden

needs_ref = pytest.mark.skipif(not checker.available("ref"),
                               reason="reference library not built (reference tree absent)")


def same_loops(a, b):
    ca, cb = checker.canonical_loops(a), checker.canonical_loops(b)
    return len(ca) == len(cb) and all(np.array_equal(x, y) for x, y in zip(ca, cb))


def golden_loops(g, key):
    pts, off = g[key + "_pts"], g[key + "_off"]
    return [pts[off[k]:off[k + 1]] for k in range(len(off) - 1)]


def golden_cases():
    out = []
    for name in ("heightfield", "sphere_on_plate"):
        g = golden("waterline_" + name)
        for key in sorted(k[:-4] for k in g if k.endswith("_pts")):
            out.append((name, key))
    return out


@pytest.mark.parametrize("name,key", golden_cases())
def test_weave_matches_reference_on_golden_fibers(name, key):
    g = golden("waterline_" + name)
    fibers = [(g[f"{key}_f{d}"], g[f"{key}_o{d}"], g[f"{key}_i{d}"]) for d in (0, 1)]
    got = _native.weave(*fibers)
    assert same_loops(got.loops, golden_loops(g, key)), key
    # the fibers come back as woven
    for d in (0, 1):
        fib, off, iv, _, _ = got.fibers(d)
        np.testing.assert_array_equal(fib, fibers[d][0])
        np.testing.assert_array_equal(off, fibers[d][1])
        np.testing.assert_array_equal(iv, fibers[d][2])


def test_weave_loops_are_closed_walks_over_interval_ends():
    g = golden("waterline_heightfield")
    key = "ball_wl_1"
    fibers = [(g[f"{key}_f{d}"], g[f"{key}_o{d}"], g[f"{key}_i{d}"]) for d in (0, 1)]
    loops = _native.weave(*fibers).loops
    ends = set()
    for fib, off, iv in fibers:
        for f in range(len(fib)):
            for k in range(int(off[f]), int(off[f + 1])):
                for t in iv[k]:
                    p = fib[f, :3] + t * (fib[f, 3:] - fib[f, :3])
                    ends.add(tuple(p))
    seen = set()
    for lp in loops:
        assert len(lp) >= 2
        for p in lp:
            assert tuple(p) in ends
            assert tuple(p) not in seen  # every interval end on one loop once
            seen.add(tuple(p))
        # consecutive CL points differ in x or y only along a fiber or across a cell
        assert np.all(np.isfinite(lp))


def test_weave_rejects_tilted_fibers():
    xf = (np.array([[0.0, 0.0, 1.0, 10.0, 0.5, 1.0]]), np.array([0, 1], dtype=np.uint64), np.array([[0.2, 0.8]]))
    yf = (np.array([[5.0, -1.0, 1.0, 5.0, 1.0, 1.0]]), np.array([0, 1], dtype=np.uint64), np.array([[0.2, 0.8]]))
    with pytest.raises(_native.OclError) as e:
        _native.weave(xf, yf)
    assert e.value.status == _abi.BAD_ARG


def test_weave_empty_and_crossing_free():
    empty = (np.zeros((0, 6)), np.zeros(1, dtype=np.uint64), np.zeros((0, 2)))
    assert _native.weave(empty, empty).loops == []
    # an X interval that no Y interval crosses gives no loop
    xf = (np.array([[0.0, 5.0, 1.0, 10.0, 5.0, 1.0]]), np.array([0, 1], dtype=np.uint64), np.array([[0.2, 0.8]]))
    yf = (np.array([[1.0, 0.0, 1.0, 1.0, 10.0, 1.0]]), np.array([0, 1], dtype=np.uint64), np.array([[0.2, 0.8]]))
    assert _native.weave(xf, yf).loops == []
    # one crossing: a single loop through all four ends
    yf2 = (np.array([[5.0, 0.0, 1.0, 5.0, 10.0, 1.0]]), np.array([0, 1], dtype=np.uint64), np.array([[0.2, 0.8]]))
    loops = _native.weave(xf, yf2).loops
    assert len(loops) == 1 and len(loops[0]) == 4


def _random_fibers(rng, n, d, lo, hi, z, maxk, grid):
    fib, off, iv = [], [0], []
    coords = np.linspace(lo, hi, n) if grid else np.sort(rng.uniform(lo, hi, n))
    for c in coords:
        fib.append([lo - 1, c, z, hi + 1, c, z] if d == 0 else [c, lo - 1, z, c, hi + 1, z])
        k = int(rng.integers(0, maxk + 1))
        cuts = np.sort(rng.uniform(0, 1, 2 * k))
        iv.extend([cuts[2 * j], cuts[2 * j + 1]] for j in range(k))
        off.append(len(iv))
    return np.array(fib).reshape(-1, 6), np.array(off, dtype=np.uint64), np.array(iv).reshape(-1, 2)


@needs_ref
@pytest.mark.parametrize("seed", range(40))
def test_weave_random_fibers_match_reference(seed):
    rng = np.random.default_rng(1000 + seed)
    n, m = int(rng.integers(2, 40)), int(rng.integers(2, 40))
    xf = _random_fibers(rng, n, 0, 0.0, 10.0, 1.0, 3, seed % 2 == 0)
    yf = _random_fibers(rng, m, 1, 0.0, 10.0, 1.0, 3, seed % 3 == 0)
    assert same_loops(_native.weave(xf, yf).loops, checker.ref_weave(xf, yf))


@needs_ref
@pytest.mark.parametrize("adaptive", [False, True])
@pytest.mark.parametrize("cname", ["cyl", "ball", "bull", "cone", "ballcone"])
def test_weave_matches_reference_fresh_mesh(cname, adaptive):
    from tests.golden.cases import CUTTERS
    tris = w.heightfield(18, 21, seed=5, jitter=0.05, jitter_seed=9)
    for z in (10.5, 13.0, 17.5, 26.0):
        loops, xf, yf = checker.ref_waterline(tris, CUTTERS[cname](), z, 1.3, adaptive=adaptive, min_sampling=0.2)
        assert same_loops(_native.weave(xf, yf).loops, loops), (cname, z)


def test_canonical_loops_is_rotation_invariant():
    a = np.arange(12.0).reshape(4, 3)
    assert same_loops([a], [np.roll(a, 2, axis=0)])
    assert not same_loops([a], [a[::-1]])
    assert math.isfinite(float(a.sum()))
