"""Generate the golden fixtures in this folder from the reference itself.

Runs the reference's own drop-cutter / push-cutter / path code (compiled
unmodified into oracle/_ref/liboclref.so by oracle/Makefile) on small seeded
cases and stores inputs and outputs as .npz files.  Needs the reference
source tree (oracle/Makefile REF_SRC); the fixtures are committed so that
the GPU tests run without it.

    python tests/golden/make_golden.py [--real]

The real-mesh fixtures (real_*.npz) are made from the reference's stl/
folder next to its sources (REF_SRC, as for oracle/Makefile) when missing or
with --real; the waterline fixtures (waterline_*.npz) when missing or with
--waterline.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import checker as ck  # noqa: E402
from opencamlib_gb300 import workloads as w  # noqa: E402
from tests.golden.cases import CUTTERS, degenerate_mesh, degenerate_points, path_spans  # noqa: E402


def drop_case(name, tris, cl):
    out = {"tris": tris, "cl": cl}
    for cname, make in CUTTERS.items():
        z, cc, ty, _ = ck.drop(tris, make(), cl, "ref", nthreads=1)
        out[f"{cname}_z"] = z
        out[f"{cname}_cc"] = cc
        out[f"{cname}_type"] = ty
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def push_case(name, tris, fib_x, fib_y):
    out = {"tris": tris, "fib_x": fib_x, "fib_y": fib_y}
    for cname, make in CUTTERS.items():
        for d, fib in ((0, fib_x), (1, fib_y)):
            res, _ = ck.push(tris, make(), d, fib, "ref", nthreads=1)
            counts = np.array([len(r) for r in res], dtype=np.int32)
            flat = [iv for r in res for iv in r]
            out[f"{cname}_{d}_counts"] = counts
            out[f"{cname}_{d}_ival"] = np.array([[iv[0], iv[1]] for iv in flat]).reshape(-1, 2)
            out[f"{cname}_{d}_cc"] = np.array([np.concatenate([iv[2], iv[3]]) for iv in flat]).reshape(-1, 6)
            out[f"{cname}_{d}_type"] = np.array([[iv[4], iv[5]] for iv in flat], dtype=np.int32).reshape(-1, 2)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def path_case(name, tris, spans):
    out = {"tris": tris, "spans": spans}
    for cname, make in CUTTERS.items():
        xyz, cc, ty = ck.pdc(tris, make(), spans, 0.37, -5.0, "ref", nthreads=1)
        out[f"{cname}_pdc_xyz"], out[f"{cname}_pdc_cc"], out[f"{cname}_pdc_type"] = xyz, cc, ty
        xyz, cc, ty = ck.apdc(tris, make(), spans, 0.8, 0.05, 0.999, "ref")
        out[f"{cname}_apdc_xyz"], out[f"{cname}_apdc_cc"], out[f"{cname}_apdc_type"] = xyz, cc, ty
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


# Real meshes shipped with the reference (its stl/ folder), read by the
# reference's own STLReader; the CL raster covers each mesh's bbox widened by
# 4 mm, starting 10 mm below it.
REAL_MESHES = ("sphere_on_plate", "30sphere", "mount_rush", "wheel_in_box")
REAL_CUTTERS = ("cyl", "ball", "bull", "cone", "ballcone")


def real_mesh_case(name, stl_dir):
    tris = ck.ref_stl_read(os.path.join(stl_dir, name + ".stl"))
    t32 = tris.astype(np.float32)
    assert np.array_equal(t32.astype(np.float64), tris)  # STL coordinates are float32
    lo, hi = tris.reshape(-1, 3).min(axis=0), tris.reshape(-1, 3).max(axis=0)
    n = 32
    xs = np.linspace(lo[0] - 4.0, hi[0] + 4.0, n) + 0.0123
    ys = np.linspace(lo[1] - 4.0, hi[1] + 4.0, n) + 0.0071
    X, Y = np.meshgrid(xs, ys)
    cl = np.stack([X.ravel(), Y.ravel(), np.full(X.size, lo[2] - 10.0)], axis=1)
    out = {"tris": t32, "cl": cl}
    for cname in REAL_CUTTERS:
        z, cc, ty, _ = ck.drop(tris, CUTTERS[cname](), cl, "ref")
        out[f"{cname}_z"], out[f"{cname}_cc"], out[f"{cname}_type"] = z, cc, ty
    if name == "sphere_on_plate":
        zs = lo[2] + (hi[2] - lo[2]) * np.array([0.15, 0.5, 0.85])
        fx = np.concatenate([w.fibers(0, z, lo[1] - 2, hi[1] + 2, 25, lo[0] - 8, hi[0] + 8) for z in zs])
        fy = np.concatenate([w.fibers(1, z, lo[0] - 2, hi[0] + 2, 25, lo[1] - 8, hi[1] + 8) for z in zs])
        out["fib_x"], out["fib_y"] = fx, fy
        for cname in ("ball", "bull"):
            for d, fib in ((0, fx), (1, fy)):
                res, _ = ck.push(tris, CUTTERS[cname](), d, fib, "ref")
                flat = [iv for r in res for iv in r]
                out[f"{cname}_{d}_counts"] = np.array([len(r) for r in res], dtype=np.int32)
                out[f"{cname}_{d}_ival"] = np.array([[iv[0], iv[1]] for iv in flat]).reshape(-1, 2)
                out[f"{cname}_{d}_cc"] = np.array([np.concatenate([iv[2], iv[3]]) for iv in flat]).reshape(-1, 6)
                out[f"{cname}_{d}_type"] = np.array([[iv[4], iv[5]] for iv in flat], dtype=np.int32).reshape(-1, 2)
    np.savez_compressed(os.path.join(HERE, "real_" + name + ".npz"), **out)


# Waterline / AdaptiveWaterline cases: (fixture, mesh, cutters, heights,
# sampling, min_sampling); the reference's Waterline::run and
# AdaptiveWaterline::run (cos limit 0.999) at each height.
WATERLINE_CUTTERS = ("cyl", "ball", "bull", "cone", "ballcone")


def waterline_case(name, tris, cutters, zs, sampling, min_sampling):
    out = {"tris": tris, "zs": np.asarray(zs, dtype=np.float64), "sampling": sampling, "min_sampling": min_sampling}
    for cname in cutters:
        for k, z in enumerate(zs):
            for mode in ("wl", "awl"):
                loops, xf, yf = ck.ref_waterline(tris, CUTTERS[cname](), z, sampling, adaptive=mode == "awl",
                                                 min_sampling=min_sampling)
                key = f"{cname}_{mode}_{k}"
                out[key + "_pts"] = np.concatenate(loops).reshape(-1, 3) if loops else np.zeros((0, 3))
                out[key + "_off"] = np.cumsum([0] + [len(lp) for lp in loops]).astype(np.int64)
                for d, (fib, off, iv) in enumerate((xf, yf)):
                    out[f"{key}_f{d}"], out[f"{key}_o{d}"], out[f"{key}_i{d}"] = fib, off.astype(np.int64), iv
    np.savez_compressed(os.path.join(HERE, "waterline_" + name + ".npz"), **out)


def waterline_fixtures(stl_dir):
    hf = w.heightfield(24, 24, seed=1)
    waterline_case("heightfield", hf, WATERLINE_CUTTERS, (11.0, 14.0, 20.0), 1.0, 0.1)
    sop = ck.ref_stl_read(os.path.join(stl_dir, "sphere_on_plate.stl"))
    lo, hi = sop.reshape(-1, 3).min(axis=0), sop.reshape(-1, 3).max(axis=0)
    zs = tuple(float(z) for z in lo[2] + (hi[2] - lo[2]) * np.array([0.1, 0.45, 0.8]))
    waterline_case("sphere_on_plate", sop, ("ball", "bull"), zs, float(hi[0] - lo[0]) / 60.0,
                   float(hi[0] - lo[0]) / 600.0)


def main():
    ck.build(ref=True)
    if not ck.available("ref"):
        raise SystemExit("reference library not built (reference sources missing)")
    hf = w.heightfield(24, 24, seed=1)
    cl = w.raster(40, 40, 100.0 / 39.0, z0=-50.0)
    cl[:, 0] += 0.013
    cl[:, 1] += 0.007
    drop_case("drop_heightfield", hf, cl)
    drop_case("drop_degenerate", degenerate_mesh(), degenerate_points())
    fx = np.concatenate([w.fibers(0, z, -5.0, 105.0, 29, -10.0, 110.0) for z in (11.0, 13.3, 17.1)])
    fy = np.concatenate([w.fibers(1, z, -5.0, 105.0, 29, -10.0, 110.0) for z in (11.0, 13.3, 17.1)])
    push_case("push_heightfield", hf, fx, fy)
    path_case("path_heightfield", hf, path_spans())
    orders = {f"dims{d}_b{b}": ck.kd_order(hf, "ref", b, d) for d in (0, 1, 2) for b in (1, 3)}
    np.savez_compressed(os.path.join(HERE, "kd_order.npz"), tris=hf, **orders)
    stl_dir = os.path.join(os.path.dirname(os.environ.get("REF_SRC", "/root/reference/src").rstrip("/")), "stl")
    if "--real" in sys.argv or not all(os.path.exists(os.path.join(HERE, f"real_{m}.npz")) for m in REAL_MESHES):
        for m in REAL_MESHES:
            real_mesh_case(m, stl_dir)
    if "--waterline" in sys.argv or not all(os.path.exists(os.path.join(HERE, f"waterline_{m}.npz"))
                                            for m in ("heightfield", "sphere_on_plate")):
        waterline_fixtures(stl_dir)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
