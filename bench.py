#!/usr/bin/env python3
"""Drop-cutter benchmark: CL points per second against a 1,048,576-triangle
mesh, FP32-screened + FP64-refined, for the five cutters of the precision
workload.

Workload (seeded synthetic, opencamlib_gb300.workloads.mesh_c2): a 512x1024
jittered bump heightfield + hemisphere r=30 mm + 2-triangle plate over
100x100 mm (exactly 1,048,576 triangles), 1,000,000 CL points on a 0.1 mm
raster starting at z=-50, cutters Cyl d6, Ball d6, Bull d6 r1, Cone d6 45deg,
BallCone 2/6/45deg.  One step = the five BatchDropCutter runs over all points.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  `value` times the device-resident call
(ocl_gb300_drop_device) with CUDA events on the launching stream; `e2e`
times the host-buffer C-ABI call (ocl_gb300_drop: pinned host CL points in,
z/CC/type out).  The reference arm (--impl reference) times the CPU oracle
(a C restatement of the reference's BatchDropCutter, OpenMP on all host
cores) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "CL-points/s at 1M tris, FP32-refined vs plain FP64, max |dz|<=1e-5 mm; p99 ms"
WORKLOAD = ("1,048,576-triangle seeded mesh (512x1024 jittered bump field + hemisphere r=30 mm on a plate), "
            "1,000,000 CL points on a 0.1 mm raster, cutters Cyl d6 / Ball d6 / Bull d6 r1 / Cone d6 45deg / "
            "BallCone 2-6 45deg; one step = one BatchDropCutter run per cutter")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=1024, help="CL points per cutter in the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-aux", action="store_true", help="skip the push and path measurements")
    ap.add_argument("--cutters", default="", help="comma list of cutters (default: all five); for profiling")
    ap.add_argument("--block", type=int, default=0,
                    help="only an N x N block of the raster (a small case for profiling)")
    ap.add_argument("--block-origin", default="400,300", help="raster column,row of the block's corner")
    ap.add_argument("--stride", type=int, default=0,
                    help="only every S-th raster point along x and y (a small case spanning the whole mesh)")
    ap.add_argument("--oracle-sample", type=int, default=4000,
                    help="CL points per cutter compared with the CPU oracle (precision_vs_oracle)")
    ap.add_argument("--no-fp64-full", action="store_true",
                    help="skip the plain FP64 run over the whole raster (mixed == FP64 check and speed-up)")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-job batching measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the request-loop measurement")
    ap.add_argument("--serve-only", action="store_true",
                    help="run only the request-loop measurement and print it")
    ap.add_argument("--batch-only", action="store_true",
                    help="run only the 64-job batching measurement and print it (for profiling)")
    ap.add_argument("--waterline-only", action="store_true",
                    help="run only the waterline measurement and print it (with --wl-levels / --wl-cutters a "
                         "small case for profiling)")
    ap.add_argument("--wl-levels", type=int, default=50, help="waterline heights (evenly from 1 to 49 mm)")
    ap.add_argument("--wl-cutters", default="ball,bull", help="waterline cutters (ball, bull)")
    ap.add_argument("--profile-step", action="store_true",
                    help="run one device step with statistics, print its counters and exit (for ncu)")
    ap.add_argument("--serve-request", type=int, default=-1,
                    help="drop the middle --serve-points points of this drop request of the serving workload "
                         "once, print its counters and exit (a small case for profiling)")
    ap.add_argument("--serve-points", type=int, default=8192)
    return ap.parse_args()


def serve_request_case(k: int, npts: int) -> dict:
    """One drop request of the serving workload (workloads.serving_requests(5,
    200)[k] on its resident mesh), cut to its middle npts points, dropped once
    in mixed precision; returns the call's counters."""
    from opencamlib_gb300 import _native, workloads as w
    meshes = w.serving_meshes(5, 8)
    r = w.serving_requests(5, 200)[k]
    if r["kind"] != "drop":
        raise SystemExit(f"request {k} is not a drop request")
    tris = meshes[r["mesh"]]
    c = w.batch_cutter(r["cutter"], r["d"])
    pts = w.serving_payload(r, tris)
    mid = len(pts) // 2
    pts = pts[max(0, mid - npts // 2): mid + npts // 2]
    z, cc, ty, st = _native.DeviceMesh(tris).drop(c, pts, "mixed")
    return {"request": k, "triangles": int(len(tris)), "cutter": r["cutter"], "d": r["d"], "points": int(len(pts)),
            "handed_back": int(st.fallback), "plain_points": int(st.plain_points), "refined": int(st.refined),
            "kernel_ms": st.kernel_ms, "screen_ms": st.screen_ms, "refine_ms": st.refine_ms,
            "fallback_ms": st.fallback_ms}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[0]) for r in self.rows if len(r) >= 7 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 7 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) < 7:
                continue
            for k, nm in enumerate(names):
                if r[3 + k].lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n):
    """One process per GPU (replicas; opencamlib_gb300.replicas)."""
    from opencamlib_gb300 import replicas
    return replicas.setup("nccl")


def cutters(names=""):
    from opencamlib_gb300 import cutters as cu
    allc = list(cu.standard_cutters().items())
    if not names:
        return allc
    keep = names.split(",")
    return [(n, c) for n, c in allc if n in keep]


def cpu_baseline(tris, cl, sample, nthreads=0):
    """Oracle port (C restatement of BatchDropCutter::dropCutter5, OpenMP) on a
    seeded sample of the raster; KD build excluded from the timing."""
    from oracle import checker
    checker.build(ref=False)
    idx = sample_indices(sample)
    pts = cl[idx]
    total = 0.0
    for _, c in cutters():
        checker.drop(tris, c, pts, "port", nthreads=nthreads)
        total += checker.last_loop_seconds()
    cores = nthreads or os.cpu_count()
    n = len(cutters()) * len(pts)
    return {"value": n / total, "unit": "CL-points/s", "cores": cores, "kind": "port",
            "sample": f"{len(pts)} CL points per cutter x {len(cutters())} cutters "
                      f"(seeded uniform sample of the 0.1 mm raster), {total:.2f} s of CPU loop time"}


def aux_measurements(cl_mesh, cuts, with_cpu, wl_levels=50, wl_cutters=("ball", "bull")):
    """The other operations on the path, measured beside the headline:
    Waterline at the waterline workload's full size (sphere-on-plate + torus,
    499,202 triangles; 50 heights z = 1..49 mm; X and Y fibers over the mesh
    bbox +- 2 cutter radii at 0.056 mm, 2,001 per direction per height, so
    200,100 fibers per cutter; one ocl_gb300_waterline_levels call: both
    fiber directions pushed on the device, the 50 levels woven on host
    threads) and PathDropCutter / AdaptivePathDropCutter on a zig-zag of 100
    line spans across the 1,048,576-triangle mesh.  Device time from the
    library's CUDA events; the CPU figures are the oracle port's push on
    every 50th fiber of every 5th level / every 10th span (OpenMP on all
    host cores)."""
    from opencamlib_gb300 import _native, cutters as cu, workloads as w
    out = {}
    tris = w.sphere_torus(1)
    mesh = _native.DeviceMesh(tris)
    zs = np.linspace(1.0, 49.0, wl_levels)
    wl = {}
    for name, c in (("ball", cu.BallCutter(6.0, 20.0)), ("bull", cu.BullCutter(6.0, 1.0, 20.0))):
        if name not in wl_cutters:
            continue
        bb = tris.reshape(-1, 3)
        extent = float(bb[:, 0].max() - bb[:, 0].min()) + 4 * c.radius
        sampling = extent / 2000.0
        mesh.waterline_levels(c, zs[:1], sampling)  # builds the push indexes
        t0 = time.perf_counter()
        levels, st = mesh.waterline_levels(c, zs, sampling)
        wall = time.perf_counter() - t0
        nfib = sum(len(lv.fibers(d)[0]) for lv in levels for d in (0, 1))
        nint = sum(len(lv.fibers(d)[2]) for lv in levels for d in (0, 1))
        rec = {"levels": len(zs), "sampling_mm": sampling, "fibers": nfib, "intervals": nint,
               "loops": sum(len(lv.loops) for lv in levels),
               "loop_points": int(sum(len(lp) for lv in levels for lp in lv.loops)),
               "wall_ms": wall * 1e3, "push_device_ms": st.kernel_ms, "weave_and_host_ms": wall * 1e3 - st.kernel_ms,
               "fibers_per_s": nfib / wall, "push_fibers_per_s": nfib / (st.kernel_ms / 1e3),
               "candidates": int(st.pairs), "fp64_pushes": int(st.refined)}
        if with_cpu:
            from oracle import checker
            sub = [lv.fibers(d)[0][::50] for lv in levels[::5] for d in (0, 1)]
            t0 = time.perf_counter()
            nsub = 0
            for k, fb in enumerate(sub):
                checker.push(tris, c, k % 2, fb, "port")
                nsub += len(fb)
            cpu_s = time.perf_counter() - t0
            rec["cpu_push_fibers_per_s"] = nsub / cpu_s
            rec["cpu_sample"] = f"{nsub} fibers (every 50th of every 5th level), oracle port push, KD build included"
        wl[name] = rec
    out["waterline"] = wl
    mesh.release()
    if cl_mesh is None:
        return out
    # paths: zig-zag of 100 lines across the bump mesh
    m2 = _native.DeviceMesh(cl_mesh)
    spans = []
    for k in range(100):
        y = 0.5 + k
        a, b = (0.0, 100.0) if k % 2 == 0 else (100.0, 0.0)
        spans.append([0, a, y, 0, b, y, 0, 0, 0, 0, 0])
    spans = np.array(spans, dtype=np.float64)
    paths = {}
    for name, c in cuts:
        if name not in ("ball", "ballcone"):
            continue
        m2.path_drop(c, spans, 0.1, -50.0)
        t0 = time.perf_counter()
        xyz, _, _, st = m2.path_drop(c, spans, 0.1, -50.0)
        pdc_s = time.perf_counter() - t0
        m2.adaptive_path_drop(c, spans, 1.0, 0.01)
        t0 = time.perf_counter()
        axyz, _, _, ast = m2.adaptive_path_drop(c, spans, 1.0, 0.01)
        apdc_s = time.perf_counter() - t0
        rec = {"pdc_points": int(len(xyz)), "pdc_wall_ms": pdc_s * 1e3, "pdc_points_per_s": len(xyz) / pdc_s,
               "apdc_points": int(len(axyz)), "apdc_wall_ms": apdc_s * 1e3, "apdc_points_per_s": len(axyz) / apdc_s}
        if with_cpu:
            from oracle import checker
            t0 = time.perf_counter()
            cx = checker.pdc(cl_mesh, c, spans[::10], 0.1, -50.0, "port")[0]
            rec["cpu_pdc_points_per_s"] = len(cx) / (time.perf_counter() - t0)
            t0 = time.perf_counter()
            ca = checker.apdc(cl_mesh, c, spans[::10], 1.0, 0.01, 0.999, "port")[0]
            rec["cpu_apdc_points_per_s"] = len(ca) / (time.perf_counter() - t0)
            rec["cpu_sample"] = "every 10th span, KD build included; APDC restatement is single-threaded as the reference's"
        paths[name] = rec
    out["paths"] = paths
    m2.release()
    try:
        out["stl_read"] = stl_ingest(cl_mesh)
    except Exception as e:  # reported, never required
        out["stl_read"] = {"error": str(e)}
    return out


def stl_ingest(tris):
    """STLReader on the 1,048,576-triangle mesh written as a binary STL, and
    on its first 100,000 triangles as an ASCII STL (files in a temporary
    directory), then the device upload of what was read."""
    import struct
    import tempfile
    from opencamlib_gb300 import _native
    rec = {}
    with tempfile.TemporaryDirectory() as d:
        t32 = np.ascontiguousarray(tris, dtype=np.float32)
        pb = os.path.join(d, "mesh_bin.stl")
        rows = np.zeros(len(t32), dtype=[("n", "<f4", 3), ("v", "<f4", 9), ("a", "<u2")])
        rows["v"] = t32
        with open(pb, "wb") as f:
            f.write(b"binary".ljust(80, b" "))
            f.write(struct.pack("<I", len(t32)))
            f.write(rows.tobytes())
        pa = os.path.join(d, "mesh_ascii.stl")
        sub = t32[:100000]
        with open(pa, "w") as f:
            f.write("solid bench\n")
            for t in sub:
                f.write("facet normal 0 0 1\nouter loop\n")
                for k in range(3):
                    f.write("vertex %.9g %.9g %.9g\n" % (t[3 * k], t[3 * k + 1], t[3 * k + 2]))
                f.write("endloop\nendfacet\n")
            f.write("endsolid bench\n")
        for name, path, n in (("binary", pb, len(t32)), ("ascii", pa, len(sub))):
            _native.stl_read(path)  # file cache warm
            t0 = time.perf_counter()
            got = _native.stl_read(path)
            dt = time.perf_counter() - t0
            ok = got.shape == (n, 9) and bool(np.array_equal(got, t32[:n].astype(np.float64)))
            rec[name] = {"triangles": n, "bytes": os.path.getsize(path), "read_s": dt,
                         "MB_per_s": os.path.getsize(path) / dt / 1e6, "triangles_per_s": n / dt, "exact": ok}
        try:
            got = _native.stl_read(pb)
            import torch
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            m = _native.DeviceMesh(got)
            torch.cuda.synchronize()
            rec["device_upload_s"] = time.perf_counter() - t0
            m.release()
        except Exception as e:  # reported, never required
            rec["device_upload_error"] = str(e)
    return rec


def sample_indices(sample, seed=17):
    """A seeded uniform sample of the 1000x1000 raster (representative of the
    whole workload: bump field, hemisphere and plate regions)."""
    from opencamlib_gb300 import workloads as w
    return w.subsample(1000 * 1000, sample, seed)


def block_indices(side, i0=400, j0=300):
    """A contiguous side x side block of the raster (coherent warps)."""
    ii, jj = np.meshgrid(np.arange(i0, i0 + side), np.arange(j0, j0 + side))
    return (jj * 1000 + ii).ravel()


def batch_measurements(steps=2, warmup=1, njobs=64, autotune=True):
    """The batching workload: 64 seeded jobs (heightfield / sphere /
    box-with-fillet meshes of 1k-2M triangles, 1k-4M raster points, the five
    cutter families with diameters 1-20 mm; workloads.batch_jobs(seed=3)),
    timed as one ocl_gb300_drop_device call per job (a stream of launches per
    job) and as one batch (persistent work-stealing launches, CUDA graph
    replay); device outputs compared bit for bit."""
    import torch
    from opencamlib_gb300 import _native, workloads as w
    specs = w.batch_jobs(seed=3, njobs=njobs)
    t0 = time.time()
    jobs = []
    for sp in specs:
        tris = w.mesh_of_size(sp["mesh"], sp["N"], sp["seed"])
        c = w.batch_cutter(sp["cutter"], sp["d"])
        pts = w.batch_points(tris, sp["M"], c.radius)
        mesh = _native.DeviceMesh(tris)
        M = len(pts)
        d_cl = torch.from_numpy(pts).cuda()
        bufs = [torch.empty(M, dtype=torch.float64, device="cuda"), torch.empty((M, 3), dtype=torch.float64, device="cuda"),
                torch.empty(M, dtype=torch.int32, device="cuda")]
        ref = [torch.empty_like(b) for b in bufs]
        jobs.append({"spec": sp, "tris": int(len(tris)), "mesh": mesh, "cutter": c, "M": M, "cl": d_cl, "out": bufs,
                     "ref": ref})
    torch.cuda.synchronize()
    setup_s = time.time() - t0
    total = sum(j["M"] for j in jobs)
    stream = torch.cuda.Stream()

    def per_job(target):
        for j in jobs:
            j["mesh"].drop_device(j["cutter"], j["cl"].data_ptr(), j["M"], j[target][0].data_ptr(),
                                  j[target][1].data_ptr(), j[target][2].data_ptr(), stream=stream.cuda_stream,
                                  stats=False)

    def timed(fn):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(steps):
            with torch.cuda.stream(stream):
                ev[0].record(stream)
                fn()
                ev[1].record(stream)
            torch.cuda.synchronize()
            ts.append(ev[0].elapsed_time(ev[1]))
        return ts

    t_single = timed(lambda: per_job("ref"))
    t1 = time.time()
    batch = _native.DropBatch([(j["mesh"], j["cutter"], j["cl"].data_ptr(), j["M"], j["out"][0].data_ptr(),
                                j["out"][1].data_ptr(), j["out"][2].data_ptr()) for j in jobs], autotune=autotune)
    create_s = time.time() - t1
    t_batch = timed(lambda: batch.run(stream.cuda_stream))
    st = batch.run(stream.cuda_stream, stats=True)
    torch.cuda.synchronize()
    same = all(torch.equal(j["out"][k], j["ref"][k]) for j in jobs for k in range(3))
    # every job's mixed results against the plain FP64 kernel on a seeded
    # sample of its points (the batch equals the single calls, so this pins
    # both to the reference's arithmetic)
    rng = np.random.default_rng(11)
    sample_points = sample_bad = 0
    for j in jobs:
        idx = np.sort(rng.choice(j["M"], size=min(j["M"], 2000), replace=False))
        pts = j["cl"].cpu().numpy()[idx]
        z64, cc64, ty64, _ = j["mesh"].drop(j["cutter"], pts, precision="fp64")
        zb, ccb, tyb = (j["out"][0].cpu().numpy()[idx], j["out"][1].cpu().numpy()[idx],
                        j["out"][2].cpu().numpy()[idx])
        sample_points += len(idx)
        sample_bad += int(np.sum((zb != z64) | (tyb != ty64) | np.any(ccb != cc64, axis=1)))
    info = batch.info()
    out = {"jobs": len(jobs), "points": int(total), "triangles": int(sum(j["tris"] for j in jobs)),
           "setup_s": setup_s, "batch_create_s": create_s,
           "one_call_per_job_ms": float(np.median(t_single)), "batch_ms": float(np.median(t_batch)),
           "one_call_per_job_points_per_s": total / (np.median(t_single) / 1e3),
           "batch_points_per_s": total / (np.median(t_batch) / 1e3),
           "speedup": float(np.median(t_single) / np.median(t_batch)), "bit_identical": bool(same),
           "fp64_sample": {"points": sample_points, "mismatched": sample_bad,
                           "sample": "2,000 seeded points per job (all of a smaller job), plain FP64 kernel"},
           "violations": int(st.violations), "handed_back_points": int(st.fallback), "plain_points": int(st.plain_points),
           "launches_per_run": info["launches_per_run"], "waves": info["waves"], "chunks": info["chunks"],
           "workspace_bytes": info["workspace_bytes"], "tuned": info["variants"],
           "launches_one_call_per_job": "about 15 per job (Morton sort, 9 stage kernels) x 64 jobs",
           "workload": "workloads.batch_jobs(seed=3): 64 jobs, N ~ logU[1e3, 2e6] triangles (heightfield / sphere / "
                       "box-with-fillet), M ~ logU[1e3, 4e6] raster points, cutter uniform over 5 families, d ~ U[1, 20] mm"}
    batch.release()
    for j in jobs:
        j["mesh"].release()
    return out


def serving_measurements(nreq=200, serial_sample=20):
    """The serving workload (workloads.serving_requests(seed=5)): 8 resident
    meshes, 200 requests with Poisson arrivals at 200/s, drops and adaptive
    paths 1:1, through ocl_gb300_server (admission under a 32 GiB budget,
    2 batches in flight).  Reports p50/p99 latency from submission to
    completion and CL points per second over the run, and beside it the same
    requests run alone one after another on a sample (mixed precision) and
    the drops of that sample alone in plain FP64."""
    import threading
    from opencamlib_gb300 import _abi, _native, workloads as w
    t0 = time.time()
    mesh_tris = w.serving_meshes(5, 8)
    meshes = [_native.DeviceMesh(t) for t in mesh_tris]
    reqs = w.serving_requests(5, nreq)
    payload = [w.serving_payload(r, mesh_tris[r["mesh"]]) for r in reqs]
    cutter = [w.batch_cutter(r["cutter"], r["d"]) for r in reqs]
    setup_s = time.time() - t0
    srv = _native.Server(hbm_budget_bytes=32 << 30, slots=2, max_batch_requests=64)
    ids = [srv.add_mesh(m) for m in meshes]
    handles = [None] * nreq

    def client():
        start = time.perf_counter()
        for k, r in enumerate(reqs):
            delay = r["t"] - (time.perf_counter() - start)
            if delay > 0:
                time.sleep(delay)
            if r["kind"] == "drop":
                handles[k] = srv.submit_drop(ids[r["mesh"]], cutter[k], payload[k])
            else:
                handles[k] = srv.submit_adaptive(ids[r["mesh"]], cutter[k], payload[k], r["sampling"],
                                                 r["min_sampling"])

    th = threading.Thread(target=client)
    th.start()
    th.join()
    lat = {"drop": [], "adaptive": []}
    bad = 0
    for k, h in enumerate(handles):
        st, res, info = srv.wait(h)
        if st != _abi.OK:
            bad += 1
            continue
        lat[reqs[k]["kind"]].append(info["latency_ms"])
    stats = srv.stats()
    srv.close()
    # the same requests alone, one after another (a sample)
    sample = list(range(0, nreq, max(1, nreq // serial_sample)))[:serial_sample]
    pts_serial, t_serial, pts_fp64, t_fp64 = 0, 0.0, 0, 0.0
    for k in sample:
        r = reqs[k]
        m = meshes[r["mesh"]]
        t1 = time.perf_counter()
        if r["kind"] == "drop":
            m.drop(cutter[k], payload[k], "mixed")
            pts_serial += len(payload[k])
        else:
            xyz, _, _, st = m.adaptive_path_drop(cutter[k], payload[k], r["sampling"], r["min_sampling"])
            pts_serial += len(xyz)
        t_serial += time.perf_counter() - t1
        if r["kind"] == "drop" and len(payload[k]) <= 200000:
            t1 = time.perf_counter()
            m.drop(cutter[k], payload[k], "fp64")
            t_fp64 += time.perf_counter() - t1
            pts_fp64 += len(payload[k])
    for m in meshes:
        m.release()
    pct = lambda v, q: float(np.percentile(v, q)) if v else None
    return {"requests": nreq, "failed": bad, "setup_s": setup_s,
            "p50_ms": stats["p50_ms"], "p99_ms": stats["p99_ms"], "mean_ms": stats["mean_ms"], "max_ms": stats["max_ms"],
            "drop_p50_ms": pct(lat["drop"], 50), "drop_p99_ms": pct(lat["drop"], 99),
            "adaptive_p50_ms": pct(lat["adaptive"], 50), "adaptive_p99_ms": pct(lat["adaptive"], 99),
            "cl_points": stats["points"], "elapsed_s": stats["elapsed_s"],
            "cl_points_per_s": stats["points"] / max(stats["elapsed_s"], 1e-9), "batches": stats["batches"],
            "serial_sample_requests": len(sample),
            "serial_mixed_points_per_s": pts_serial / max(t_serial, 1e-9),
            "serial_fp64_drop_points_per_s": (pts_fp64 / t_fp64) if t_fp64 else None,
            "arrivals": "Poisson 200/s (seeded), 1:1 drops (100-1e6 points) and adaptive paths (10-500 mm, "
                        "sampling 0.1-1, min 0.01), 8 meshes 1e4-2e6 triangles, 5 cutter families d 2-12 mm"}


def mixed_vs_fp64(mesh, cl, cuts):
    """Per cutter, the mixed path and the plain FP64 kernel (the reference's
    KD-tree algorithm on the device) over the same points: results compared
    bit for bit, device times from the library's CUDA events."""
    out = {}
    for name, c in cuts:
        z64, cc64, ty64, s64 = mesh.drop(c, cl, "fp64")
        zm, ccm, tym, sm = mesh.drop(c, cl, "mixed")
        dz = np.abs(zm - z64)
        out[name] = {"points": int(len(cl)), "max_dz_mm": float(dz.max()), "rms_dz_mm": float(np.sqrt(np.mean(dz * dz))),
                     "cctype_match": float(np.mean(tym == ty64)), "cc_max_diff_mm": float(np.abs(ccm - cc64).max()),
                     "bit_identical": bool(np.array_equal(zm, z64) and np.array_equal(ccm, cc64)
                                           and np.array_equal(tym, ty64)),
                     "fp64_kernel_ms": s64.kernel_ms, "mixed_kernel_ms": sm.kernel_ms,
                     "speedup": s64.kernel_ms / max(sm.kernel_ms, 1e-9), "exact_pairs": int(s64.pairs),
                     "violations": int(sm.violations)}
    return out


def precision_vs_oracle(mesh, tris, cl_full, cuts, sample):
    """Per cutter, the mixed path against the CPU oracle (the C restatement
    pinned bit for bit to the reference build) on a seeded sample of the
    raster: max / RMS |dz|, CC type agreement, CC point difference."""
    from oracle import checker
    checker.build(ref=False)
    pts = cl_full[sample_indices(sample, seed=29)]
    out = {}
    for name, c in cuts:
        zm, ccm, tym, _ = mesh.drop(c, pts, "mixed")
        zr, ccr, tyr, _ = checker.drop(tris, c, pts, "port")
        dz = np.abs(zm - zr)
        lifted = tyr != 0
        out[name] = {"points": int(len(pts)), "max_dz_mm": float(dz.max()), "rms_dz_mm": float(np.sqrt(np.mean(dz * dz))),
                     "cctype_match": float(np.mean(tym == tyr)),
                     "cc_max_diff_mm": float(np.abs(ccm[lifted] - ccr[lifted]).max(initial=0.0)),
                     "oracle": "oracle/ocl_oracle.c (C restatement of BatchDropCutter::dropCutter5, "
                               "pinned to the reference build), seeded uniform sample of the raster"}
    return out


def roofline_block(tris, M, cuts, breakdown, stage, args, compute):
    """Compute roofline of the timed step (FP32 screen + FP64 refinement
    against the device's measured FMA peaks; frozen per-pair operation
    counts from opencamlib_gb300.roofline), with the HBM view beside it."""
    from opencamlib_gb300 import roofline as rf
    names = [n for n, _ in cuts]
    step_s = float(stage[:, 3].sum()) / args.steps / 1e3
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    alg_bytes = tris.shape[0] * 72 + M * (24 + 36)
    screen_ms = float(stage[:, 0].mean())
    traffic = None
    if not (args.block or args.stride) and all(rf.SCREEN_DRAM_BYTES.get(n) for n in names):
        traffic = sum(rf.SCREEN_DRAM_BYTES[n] for n in names) / len(names)
    hbm_view = {"bound": "hbm", "kernel": "k_drop_screen (per call)", "achieved": alg_bytes / (screen_ms / 1e3) / 1e9,
                "peak": hbm, "unit": "GB/s", "frac": alg_bytes / (screen_ms / 1e3) / 1e9 / hbm, "traffic": traffic,
                "algorithmic_bytes_per_launch": alg_bytes, "per_launch_ms": screen_ms,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback 6800 GB/s"}
    if not rf.measured(names) or not compute or "fp32_tflops" not in compute:
        hbm_view["note"] = "per-pair operation counts not measured yet: HBM view only (the path is not HBM-bound)"
        return hbm_view
    counts = {n: (int(st.screened), int(st.refined)) for n, st in breakdown}
    p32, p64 = compute["fp32_tflops"] * 1e12, compute["fp64_tflops"] * 1e12
    r = rf.step_roofline(counts, step_s, p32, p64)
    screen_f32 = sum(counts[n][0] * rf.FP32_PER_SCREEN[n] for n in names)
    return {"bound": "fp32+fp64 issue", "kernel": "drop step: k_drop_screen (FP32) + k_drop_refine / k_bull_eval / "
                                                  "k_drop_exact / k_drop_kd (FP64)",
            "achieved": r["achieved_flops_fp32_equiv"] / 1e12, "peak": compute["fp32_tflops"],
            "unit": "TFLOP/s (FP32-equivalent: FP64 operations x P32/P64)", "frac": r["frac"],
            "traffic": traffic,
            "fp32_ops_per_step": r["fp32_ops"], "fp64_ops_per_step": r["fp64_ops"],
            "t_roof_ms": r["t_roof_s"] * 1e3, "t_step_ms": step_s * 1e3,
            "screen_fp32_tflops": screen_f32 / (float(stage[:, 0].sum()) / args.steps / 1e3) / 1e12,
            "peak_source": "ocl_gb300_fma_peaks on this GPU (MEASURED_PEAKS.json has no FP32/FP64 figure)",
            "ops_source": "opencamlib_gb300/roofline.py (ncu instruction counters per screened pair / refined "
                          "triangle; the capture is summarised under profiles/)",
            "hbm": hbm_view}


def run_reference(args):
    rank, world, local, dist = dist_setup(args.gpus)
    if rank != 0:
        return
    from oracle import checker
    from opencamlib_gb300 import workloads as w
    checker.build(ref=False)
    tris = w.mesh_c2()
    cl = w.raster_c2()
    idx = sample_indices(args.cpu_sample)
    pts = cl[idx]
    times = []
    for s in range(args.warmup + args.steps):
        t = 0.0
        for _, c in cutters():
            checker.drop(tris, c, pts, "port")
            t += checker.last_loop_seconds()
        if s >= args.warmup:
            times.append(t)
    n = len(cutters()) * len(pts)
    value = n * len(times) / sum(times)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "CL-points/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": f"{len(pts)} CL points per cutter per step"},
            "cpu_baseline": {"value": value, "unit": "CL-points/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"{len(pts)} CL points per cutter (seeded uniform sample of the raster), "
                                       "5 cutters"},
            "e2e": {"value": value, "unit": "CL-points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    rank, world, local, dist = dist_setup(args.gpus)
    import torch
    torch.cuda.set_device(local)
    if args.waterline_only:
        wl = aux_measurements(None, None, not args.no_cpu_baseline, args.wl_levels, args.wl_cutters.split(","))
        print(json.dumps({"waterline": wl["waterline"]}), flush=True)
        return
    if args.serve_request >= 0:
        print(json.dumps({"serve_request": serve_request_case(args.serve_request, args.serve_points)}), flush=True)
        return
    import opencamlib_gb300 as ocl
    from opencamlib_gb300 import _abi
    from opencamlib_gb300 import workloads as w

    tris = w.mesh_c2()
    cl_full = w.raster_c2()
    bi0, bj0 = (int(v) for v in args.block_origin.split(","))
    cl = cl_full[block_indices(args.block, bi0, bj0)] if args.block else cl_full
    if args.stride:
        cl = cl.reshape(1000, 1000, 3)[::args.stride, ::args.stride].reshape(-1, 3) if not args.block else cl[::args.stride]
    M = cl.shape[0]
    cuts = cutters(args.cutters)
    t0 = time.time()
    mesh = ocl.DeviceMesh(tris)
    torch.cuda.synchronize()
    mesh_s = time.time() - t0

    stream = torch.cuda.Stream()
    d_cl = torch.from_numpy(cl).to("cuda")
    d_z = torch.empty(M, dtype=torch.float64, device="cuda")
    d_cc = torch.empty((M, 3), dtype=torch.float64, device="cuda")
    d_ty = torch.empty(M, dtype=torch.int32, device="cuda")

    def step_device(stats_out=None):
        for name, c in cuts:
            st = mesh.drop_device(c, d_cl.data_ptr(), M, d_z.data_ptr(), d_cc.data_ptr(), d_ty.data_ptr(),
                                  stream=stream.cuda_stream, precision="mixed", stats=stats_out is not None)
            if stats_out is not None:
                stats_out.append((name, st))

    if args.serve_only:
        print(json.dumps({"serving": serving_measurements()}), flush=True)
        return

    if args.batch_only:
        print(json.dumps({"batch": batch_measurements()}), flush=True)
        return

    if args.profile_step:
        # one step with statistics: the launches an ncu capture of this
        # command sees, with the library's own counters for them
        rec = []
        step_device(rec)
        torch.cuda.synchronize()
        print(json.dumps({"profile_step": {n: {"screened": int(st.screened), "refined": int(st.refined),
                                               "fallback_points": int(st.fallback), "launches": int(st.launches),
                                               "kernel_ms": st.kernel_ms, "screen_ms": st.screen_ms,
                                               "refine_ms": st.refine_ms, "fallback_ms": st.fallback_ms}
                                           for n, st in rec},
                          "cl_points": int(M), "triangles": int(tris.shape[0])}), flush=True)
        return

    # warm-up + per-kernel breakdown (stats path syncs; not timed)
    breakdown = []
    for _ in range(max(1, args.warmup)):
        breakdown = []
        step_device(breakdown)
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for k in range(args.steps):
            step_device()
            ev[k + 1].record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    total_ms = ev[0].elapsed_time(ev[-1])
    # per-stage device times of the timed calls (CUDA events the library
    # records on the launching stream; read after the timed region)
    from opencamlib_gb300 import _native
    stage = _native.stage_times(len(cuts) * args.steps)
    from opencamlib_gb300 import replicas
    total_ms = replicas.max_over_ranks(total_ms, dist, "cuda")
    value = replicas.whole_job_rate(len(cuts) * M * args.steps, world, total_ms / 1e3)

    # e2e: host-buffer C-ABI call, pinned host memory, copies inside the timed region
    h_cl = torch.from_numpy(cl).pin_memory().numpy()
    h_z = torch.empty(M, dtype=torch.float64).pin_memory().numpy()
    h_cc = torch.empty((M, 3), dtype=torch.float64).pin_memory().numpy()
    h_ty = torch.empty(M, dtype=torch.int32).pin_memory().numpy()
    L = ocl.lib()
    import ctypes as C
    descs = [c.desc() for _, c in cuts]

    def step_host():
        for d in descs:
            st = L.ocl_gb300_drop(mesh.handle, C.byref(d), h_cl.ctypes.data_as(C.POINTER(C.c_double)), M,
                                  _abi.PREC_MIXED, h_z.ctypes.data_as(C.POINTER(C.c_double)),
                                  h_cc.ctypes.data_as(C.POINTER(C.c_double)),
                                  h_ty.ctypes.data_as(C.POINTER(C.c_int32)), None)
            if st != 0:
                raise RuntimeError(L.ocl_gb300_last_error().decode())

    step_host()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    e_t0 = time.perf_counter()
    for _ in range(args.steps):
        step_host()
    torch.cuda.synchronize()
    e_el = time.perf_counter() - e_t0
    e_el = replicas.max_over_ranks(e_el, dist, "cuda")
    clocks = sampler.stop()
    e2e = replicas.whole_job_rate(len(cuts) * M * args.steps, world, e_el)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    # mixed vs plain FP64 on the GPU over the whole timed point set (the
    # results must be bit-identical), and the plain FP64 kernel's time
    fp64_full = None
    if not args.no_fp64_full:
        fp64_full = mixed_vs_fp64(mesh, cl, cuts)
    # mixed against the CPU oracle (pinned to the reference) on a seeded sample
    prec_oracle = None
    if args.oracle_sample > 0:
        try:
            prec_oracle = precision_vs_oracle(mesh, tris, cl_full, cuts, args.oracle_sample)
        except Exception as e:  # reported, never required
            prec_oracle = {"error": str(e)}

    # stage times of the timed region (CUDA events of the library on the launching stream)
    agg = {"screen": float(stage[:, 0].sum()) / args.steps, "refine": float(stage[:, 1].sum()) / args.steps,
           "fallback": float(stage[:, 2].sum()) / args.steps}
    launches = 0
    for name, st in breakdown:
        launches += int(st.launches)

    aux = None
    if not args.no_aux and not (args.block or args.cutters or args.stride):
        try:
            aux = aux_measurements(tris, cuts, not args.no_cpu_baseline)
        except Exception as e:  # reported, never required
            aux = {"error": str(e)}
    compute = None
    try:  # FP32 / FP64 FMA ceilings of this GPU (the compute bounds of the path)
        from opencamlib_gb300 import _native
        f32, f64 = _native.fma_peaks()
        compute = {"fp32_tflops": f32, "fp64_tflops": f64,
                   "source": "ocl_gb300_fma_peaks: 8 FMA chains per thread on a full-occupancy grid, this GPU"}
    except Exception as e:  # reported, never required
        compute = {"error": str(e)}
    roof = roofline_block(tris, M, cuts, breakdown, stage, args, compute)
    if aux is not None and not args.no_serve and "error" not in aux:
        try:
            aux["serving"] = serving_measurements()
        except Exception as e:  # reported, never required
            aux["serving"] = {"error": str(e)}
    if aux is not None and not args.no_batch and "error" not in aux:
        try:
            aux["batch"] = batch_measurements()
        except Exception as e:  # reported, never required
            aux["batch"] = {"error": str(e)}

    cpu = None
    if not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(tris, cl_full, args.cpu_sample)
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "error": str(e)}

    line = {
        "metric": METRIC, "value": value, "unit": "CL-points/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": WORKLOAD if not (args.block or args.cutters or args.stride) else
                   f"subset of: {WORKLOAD} (block {args.block or 1000} at {args.block_origin}, stride {args.stride or 1}, "
                   f"cutters {[n for n, _ in cuts]})",
                   "triangles": int(tris.shape[0]), "cl_points": int(M),
                   "cutters": [n for n, _ in cuts], "precision": "mixed (FP32 screen, FP64 refine)",
                   "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2: mesh device data ~330 MB (FP64+FP32 records, grid) > 129 MB L2",
                   "mesh_build_s": mesh_s},
        "latency": {"p50_step_ms": float(np.percentile(step_ms, 50)), "p99_step_ms": float(np.percentile(step_ms, 99)),
                    "per_cutter_ms": {n: st.kernel_ms for n, st in breakdown}},
        "per_cutter": {n: {"kernel_ms": st.kernel_ms, "screen_ms": st.screen_ms, "refine_ms": st.refine_ms,
                           "fallback_ms": st.fallback_ms, "fallback_points": int(st.fallback),
                           "overflow_points": int(st.overflow_points), "chain_points": int(st.chain_points),
                           "open_branch_points": int(st.open_branch_points),
                           "untracked_branch_points": int(st.untracked_branch_points),
                           "plain_points": int(st.plain_points),
                           "verify_failed_points": int(st.verify_failed_points),
                           "refined_per_point": st.refined / M, "screened_per_point": st.screened / M}
                       for n, st in breakdown},
        "clocks": clocks,
        "e2e": {"value": e2e, "unit": "CL-points/s", "h2d_bytes_per_step": len(cuts) * M * 24,
                "d2h_bytes_per_step": len(cuts) * M * (8 + 24 + 4)},
        "gpu_launches": launches * args.steps,
        "roofline": roof,
        "kernel_ms_per_step": agg,
        "compute_peaks": compute,
        "precision_vs_oracle": prec_oracle,
        "mixed_vs_fp64": fp64_full,
        "cpu_baseline": cpu,
        "other_operations": aux,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
