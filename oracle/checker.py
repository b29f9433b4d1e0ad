"""TEST INFRASTRUCTURE ONLY: ctypes access to the CPU checkers.

`port` is _build/liboclport.so (the C restatement in ocl_oracle.c, built on
every machine); `ref` is _ref/liboclref.so (the reference's own sources,
built only where the reference tree is present); `binding` is
_ref/libgb300binding.so (opencamlib_gb300/integration's reference-side
binding compiled against the reference's headers, same condition).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from opencamlib_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboclport.so")
REF_SO = os.path.join(HERE, "_ref", "liboclref.so")
BINDING_SO = os.path.join(HERE, "_ref", "libgb300binding.so")

_libs = {}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_long)
_i64p = C.POINTER(C.c_int64)


def build(ref: bool = True, quiet: bool = True) -> None:
    """make port (and ref, plus the binding once the GB300 library is built,
    when the reference tree exists)."""
    targets = ["port"] + (["ref"] if ref else [])
    if ref and os.path.exists(os.path.join(HERE, "..", "opencamlib_gb300", "_build", "libocl_gb300.so")):
        targets.append("binding")
    out = subprocess.run(["make", "-s", "-j8", *targets], cwd=HERE, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


def available(which: str) -> bool:
    return os.path.exists({"port": PORT_SO, "ref": REF_SO, "binding": BINDING_SO}[which])


def binding_cutter(kind: int, args):
    """A reference cutter object (kind 1-4: Cyl, Ball, Bull, Cone; 11-16: the
    composite presets) through the reference-side binding: (status, the
    binding's descriptor, the object's own fields in cutter_fields' layout)."""
    L = _libs.get("binding")
    if L is None:
        L = C.CDLL(BINDING_SO)
        L.binding_cutter.argtypes = [C.c_int, _dp, C.POINTER(_abi.CutterDesc), _dp]
        L.binding_cutter.restype = C.c_int
        L.binding_drop.argtypes = [_dp]
        L.binding_drop.restype = C.c_int
        _libs["binding"] = L
    a = _d(list(args) + [0.0] * (4 - len(args)))
    desc = _abi.CutterDesc()
    out = np.zeros(4 + 9 * _abi.MAX_SUB)
    st = L.binding_cutter(kind, _ptr(a), C.byref(desc), _ptr(out))
    return st, desc, out


def binding_drop():
    """The binding's mesh_create + batch_drop on a two-triangle STLSurf:
    (status, lifted z of one CL point)."""
    binding_cutter(1, (1.0, 1.0))  # loads the library
    z = C.c_double(0.0)
    st = _libs["binding"].binding_drop(C.byref(z))
    return st, z.value


def _lib(which: str):
    if which in _libs:
        return _libs[which]
    path = PORT_SO if which == "port" else REF_SO
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    L = C.CDLL(path)
    p = "oracle_" if which == "port" else "ref_"
    cd = C.POINTER(_abi.CutterDesc)
    f = getattr(L, p + "drop")
    f.argtypes = [_dp, C.c_long, cd, _dp, C.c_long, C.c_int, C.c_uint, _dp, _dp, _ip, _lp]
    f.restype = C.c_int
    f = getattr(L, p + "push")
    f.argtypes = [_dp, C.c_long, cd, C.c_int, _dp, C.c_long, C.c_int, C.c_uint, _ip, _dp, _dp, _ip,
                  C.c_long, _lp]
    f.restype = C.c_long
    f = getattr(L, p + "pdc")
    f.argtypes = [_dp, C.c_long, cd, _dp, C.c_long, C.c_double, C.c_double, C.c_int, C.c_uint, _dp, _dp,
                  _ip, C.c_long]
    f.restype = C.c_long
    f = getattr(L, p + "apdc")
    f.argtypes = [_dp, C.c_long, cd, _dp, C.c_long, C.c_double, C.c_double, C.c_double, C.c_uint, _dp,
                  _dp, _ip, C.c_long]
    f.restype = C.c_long
    f = getattr(L, p + "kd_order")
    f.argtypes = [_dp, C.c_long, C.c_uint, C.c_int, _i64p]
    f.restype = C.c_int
    if which == "port":
        L.oracle_overlap_pairs.argtypes = [_dp, C.c_long, C.c_double, _dp, C.c_long, C.c_int]
        L.oracle_overlap_pairs.restype = C.c_long
        L.oracle_overlap_sets.argtypes = [_dp, C.c_long, C.c_double, _dp, C.c_long, C.c_int, _i64p, _ip, C.c_long]
        L.oracle_overlap_sets.restype = C.c_long
        L.oracle_cutter_fields.argtypes = [cd, _dp]
        L.oracle_cutter_fields.restype = C.c_int
        L.oracle_last_loop_seconds.restype = C.c_double
        L.oracle_edge_contact.argtypes = [cd, C.c_double, C.c_double, _dp, _dp, _dp, _dp]
        L.oracle_edge_contact.restype = C.c_int
    else:
        L.ref_preset_fields.argtypes = [C.c_int, _dp, _dp]
        L.ref_preset_fields.restype = C.c_int
        L.ref_stl_read.argtypes = [C.c_char_p, _dp, C.c_long]
        L.ref_stl_read.restype = C.c_long
        L.ref_line_filter.argtypes = [_dp, C.c_long, C.c_double, _dp, C.c_long]
        L.ref_line_filter.restype = C.c_long
        L.ref_rotate.argtypes = [_dp, C.c_long, C.c_double, C.c_double, C.c_double, _dp, _dp]
        L.ref_rotate.restype = C.c_int
    _libs[which] = L
    return L


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


def drop(tris, cutter, cl, which="port", nthreads=0, bucket=1):
    """BatchDropCutter::run(); returns (z, cc[M,3], type[M], ncalls)."""
    L = _lib(which)
    tris = _d(tris).reshape(-1, 9)
    cl = _d(cl).reshape(-1, 3)
    M = cl.shape[0]
    z = np.empty(M)
    cc = np.empty((M, 3))
    ty = np.empty(M, dtype=np.int32)
    nc = C.c_long(0)
    desc = cutter.desc() if hasattr(cutter, "desc") else cutter
    fn = getattr(L, ("oracle_" if which == "port" else "ref_") + "drop")
    st = fn(_ptr(tris), tris.shape[0], C.byref(desc), _ptr(cl), M, nthreads, bucket, _ptr(z), _ptr(cc),
            _ptr(ty, _ip), C.byref(nc))
    if st != 0:
        raise RuntimeError(f"{which} drop failed: {st}")
    return z, cc, ty, nc.value


def push(tris, cutter, direction, fibers, which="port", nthreads=0, bucket=1):
    """BatchPushCutter::run(); returns a list (per fiber) of interval records
    (lower, upper, lower_cc[3], upper_cc[3], lower_type, upper_type) in the
    reference's vector order, and ncalls."""
    L = _lib(which)
    tris = _d(tris).reshape(-1, 9)
    fib = _d(fibers).reshape(-1, 6)
    F = fib.shape[0]
    counts = np.zeros(F, dtype=np.int32)
    desc = cutter.desc() if hasattr(cutter, "desc") else cutter
    fn = getattr(L, ("oracle_" if which == "port" else "ref_") + "push")
    cap = max(16, 8 * F)
    nc = C.c_long(0)
    while True:
        iv = np.empty(2 * cap)
        cc = np.empty(6 * cap)
        ty = np.empty(2 * cap, dtype=np.int32)
        total = fn(_ptr(tris), tris.shape[0], C.byref(desc), direction, _ptr(fib), F, nthreads, bucket,
                   _ptr(counts, _ip), _ptr(iv), _ptr(cc), _ptr(ty, _ip), cap, C.byref(nc))
        if total < 0:
            raise RuntimeError(f"{which} push failed: {total}")
        if total <= cap:
            break
        cap = total
    out = []
    k = 0
    for f in range(F):
        rec = []
        for _ in range(counts[f]):
            rec.append((iv[2 * k], iv[2 * k + 1], cc[6 * k:6 * k + 3].copy(), cc[6 * k + 3:6 * k + 6].copy(),
                        int(ty[2 * k]), int(ty[2 * k + 1])))
            k += 1
        out.append(rec)
    return out, nc.value


def pdc(tris, cutter, spans, sampling, minz, which="port", nthreads=0, bucket=1):
    L = _lib(which)
    tris = _d(tris).reshape(-1, 9)
    spans = _d(spans).reshape(-1, _abi.SPAN_DOUBLES)
    desc = cutter.desc() if hasattr(cutter, "desc") else cutter
    fn = getattr(L, ("oracle_" if which == "port" else "ref_") + "pdc")
    cap = 1024
    while True:
        xyz = np.empty((cap, 3))
        cc = np.empty((cap, 3))
        ty = np.empty(cap, dtype=np.int32)
        n = fn(_ptr(tris), tris.shape[0], C.byref(desc), _ptr(spans), spans.shape[0], sampling, minz, nthreads,
               bucket, _ptr(xyz), _ptr(cc), _ptr(ty, _ip), cap)
        if n < 0:
            raise RuntimeError(f"{which} pdc failed: {n}")
        if n <= cap:
            return xyz[:n], cc[:n], ty[:n]
        cap = n


def apdc(tris, cutter, spans, sampling, min_sampling, cos_limit=0.999, which="port", bucket=1):
    L = _lib(which)
    tris = _d(tris).reshape(-1, 9)
    spans = _d(spans).reshape(-1, _abi.SPAN_DOUBLES)
    desc = cutter.desc() if hasattr(cutter, "desc") else cutter
    fn = getattr(L, ("oracle_" if which == "port" else "ref_") + "apdc")
    cap = 4096
    while True:
        xyz = np.empty((cap, 3))
        cc = np.empty((cap, 3))
        ty = np.empty(cap, dtype=np.int32)
        n = fn(_ptr(tris), tris.shape[0], C.byref(desc), _ptr(spans), spans.shape[0], sampling, min_sampling,
               cos_limit, bucket, _ptr(xyz), _ptr(cc), _ptr(ty, _ip), cap)
        if n < 0:
            raise RuntimeError(f"{which} apdc failed: {n}")
        if n <= cap:
            return xyz[:n], cc[:n], ty[:n]
        cap = n


def kd_order(tris, which="port", bucket=1, dims=0):
    L = _lib(which)
    tris = _d(tris).reshape(-1, 9)
    order = np.empty(tris.shape[0], dtype=np.int64)
    fn = getattr(L, ("oracle_" if which == "port" else "ref_") + "kd_order")
    st = fn(_ptr(tris), tris.shape[0], bucket, dims, _ptr(order, _i64p))
    if st != 0:
        raise RuntimeError(f"{which} kd_order failed: {st}")
    return order


def overlap_pairs(tris, radius, cl, nthreads=0):
    L = _lib("port")
    tris = _d(tris).reshape(-1, 9)
    cl = _d(cl).reshape(-1, 3)
    return L.oracle_overlap_pairs(_ptr(tris), tris.shape[0], radius, _ptr(cl), cl.shape[0], nthreads)


def overlap_sets(tris, radius, cl, nthreads=0):
    """Exact overlap sets S(cl) as the reference forms them (KD search, then
    MillingCutter::overlaps): (offsets[M+1], ids) with ascending insertion
    indices of point i in ids[offsets[i]:offsets[i+1]]."""
    L = _lib("port")
    tris = _d(tris).reshape(-1, 9)
    cl = _d(cl).reshape(-1, 3)
    M = cl.shape[0]
    counts = np.zeros(M, dtype=np.int64)
    total = L.oracle_overlap_sets(_ptr(tris), tris.shape[0], radius, _ptr(cl), M, nthreads, _ptr(counts, _i64p),
                                  None, 0)
    if total < 0:
        raise RuntimeError("overlap_sets failed")
    ids = np.zeros(max(total, 1), dtype=np.int32)
    L.oracle_overlap_sets(_ptr(tris), tris.shape[0], radius, _ptr(cl), M, nthreads, _ptr(counts, _i64p),
                          _ptr(ids, _ip), total)
    offsets = np.zeros(M + 1, dtype=np.int64)
    np.cumsum(counts, out=offsets[1:])
    return offsets, ids[:total]


def edge_contact(cutter, x, y, p1, p2):
    """singleEdgeDrop of one edge on its own: (status, clz, cc) with status 1
    when the CC lies on the segment, 0 when not, -1 beyond the radius."""
    L = _lib("port")
    a, b = _d(p1).reshape(3), _d(p2).reshape(3)
    clz = C.c_double(0.0)
    cc = np.zeros(3)
    desc = cutter.desc()
    st = L.oracle_edge_contact(C.byref(desc), float(x), float(y), _ptr(a), _ptr(b), C.byref(clz), _ptr(cc))
    return st, clz.value, cc


def cutter_fields(cutter):
    """The oracle's derived cutter fields for a cutter object or a raw
    descriptor (radius, length, diameter, nsub; then per sub-cutter, or for
    a basic cutter once: diameter, radius, length, center_height,
    xy_normal_length, normal_length, radiusvec, heightvec, zoffset)."""
    L = _lib("port")
    out = np.zeros(4 + 9 * _abi.MAX_SUB)
    desc = cutter if isinstance(cutter, _abi.CutterDesc) else cutter.desc()
    if L.oracle_cutter_fields(C.byref(desc), _ptr(out)) != 0:
        raise RuntimeError("bad cutter")
    return out


def _waterline_lib():
    L = _lib("ref")
    if not hasattr(L, "_wl_ready"):
        cd = C.POINTER(_abi.CutterDesc)
        u64p = C.POINTER(C.c_uint64)
        L.ref_waterline.argtypes = [_dp, C.c_long, cd, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, _lp]
        L.ref_waterline.restype = C.c_long
        L.ref_weave.argtypes = [_dp, C.c_long, u64p, _dp, _dp, C.c_long, u64p, _dp, _lp]
        L.ref_weave.restype = C.c_long
        L.ref_loops_get.argtypes = [_dp, _lp]
        L.ref_loops_get.restype = None
        L.ref_fibers_get.argtypes = [C.c_int, _dp, u64p, _dp]
        L.ref_fibers_get.restype = C.c_long
        L._wl_ready = True
    return L


def _ref_loops(L, nloops, npts):
    pts = np.zeros((npts.value, 3))
    off = np.zeros(nloops + 1, dtype=np.int64)
    L.ref_loops_get(_ptr(pts), off.ctypes.data_as(_lp))
    return [pts[off[k]:off[k + 1]].copy() for k in range(nloops)]


def _ref_fibers(L, d):
    u64p = C.POINTER(C.c_uint64)
    tot = np.zeros(1, dtype=np.uint64)
    F = L.ref_fibers_get(d, None, tot.ctypes.data_as(u64p), None)
    fib = np.zeros((F, 6))
    off = np.zeros(F + 1, dtype=np.uint64)
    iv = np.zeros((int(tot[0]), 2))
    L.ref_fibers_get(d, _ptr(fib), off.ctypes.data_as(u64p), _ptr(iv))
    return fib, off, iv


def ref_waterline(tris, cutter, z, sampling, adaptive=False, min_sampling=None, cos_limit=0.999):
    """The reference's Waterline::run or AdaptiveWaterline::run at height z:
    (loops as (n, 3) arrays, X fibers, Y fibers), fibers as (endpoints
    (F, 6), interval offsets (F+1), [lower, upper] t-values (K, 2)).  (The
    run2 variants, SmartWeave, are not offered: the reference's
    SmartWeave::build dereferences an end iterator when the fibers crossing
    an interval are not adjacent, smart_weave.cpp:78-81.)"""
    L = _waterline_lib()
    tris = np.ascontiguousarray(tris, dtype=np.float64)
    desc = cutter.desc()
    npts = C.c_long(0)
    mode = 2 if adaptive else 0
    ms = sampling / 10.0 if min_sampling is None else min_sampling
    n = L.ref_waterline(_ptr(tris), len(tris), C.byref(desc), z, sampling, ms, cos_limit, mode, C.byref(npts))
    if n < 0:
        raise RuntimeError("ref_waterline failed")
    return _ref_loops(L, n, npts), _ref_fibers(L, 0), _ref_fibers(L, 1)


def ref_weave(xfibers, yfibers):
    """The reference's SimpleWeave on the given fibers (as ref_waterline
    returns them): the loops."""
    L = _waterline_lib()
    u64p = C.POINTER(C.c_uint64)
    args = []
    for fib, off, iv in (xfibers, yfibers):
        fib = np.ascontiguousarray(fib, dtype=np.float64)
        off = np.ascontiguousarray(off, dtype=np.uint64)
        iv = np.ascontiguousarray(iv, dtype=np.float64).reshape(-1, 2)
        args.append((fib, off, iv))
    npts = C.c_long(0)
    (xf, xo, xi), (yf, yo, yi) = args
    n = L.ref_weave(_ptr(xf), len(xf), xo.ctypes.data_as(u64p), _ptr(xi), _ptr(yf), len(yf),
                    yo.ctypes.data_as(u64p), _ptr(yi), C.byref(npts))
    return _ref_loops(L, n, npts)


def canonical_loops(loops):
    """Loops in a form that does not depend on where each loop starts or on
    the order of the loops (the reference starts each loop at the CL vertex
    with the lowest address): every loop rotated to its lexicographically
    smallest rotation, then the loops sorted."""
    out = []
    for lp in loops:
        a = np.asarray(lp, dtype=np.float64).reshape(-1, 3)
        n = len(a)
        best = None
        for r in range(n):
            cand = np.roll(a, -r, axis=0)
            key = tuple(cand.ravel())
            if best is None or key < best[0]:
                best = (key, cand)
        out.append(best[1] if best else a)
    out.sort(key=lambda a: (len(a), tuple(a.ravel())))
    return out


def loops_close(a, b, tol):
    """True when the loop lists a and b are the same cyclic point sequences
    up to tol per coordinate (any start, any loop order)."""
    if len(a) != len(b):
        return False
    A = sorted((np.asarray(x, dtype=np.float64).reshape(-1, 3) for x in a), key=lambda x: (len(x), x.min(axis=0).round(6).tolist()))
    B = sorted((np.asarray(x, dtype=np.float64).reshape(-1, 3) for x in b), key=lambda x: (len(x), x.min(axis=0).round(6).tolist()))
    used = [False] * len(B)
    for x in A:
        found = False
        for j, y in enumerate(B):
            if used[j] or len(y) != len(x):
                continue
            if len(x) == 0:
                found = True
            for r in np.nonzero(np.all(np.abs(x - y[0]) <= tol, axis=1))[0]:
                if np.all(np.abs(np.roll(x, -int(r), axis=0) - y) <= tol):
                    found = True
                    break
            if found:
                used[j] = True
                break
        if not found:
            return False
    return True


def ref_preset_fields(preset: int, args):
    L = _lib("ref")
    a = _d(list(args) + [0.0] * (4 - len(args)))
    out = np.zeros(4 + 9 * _abi.MAX_SUB)
    if L.ref_preset_fields(preset, _ptr(a), _ptr(out)) != 0:
        raise RuntimeError("bad preset")
    return out


def ref_stl_read(path) -> np.ndarray:
    """The reference's STLReader on a file: (n, 9) triangles in order."""
    L = _lib("ref")
    p = os.fsencode(path)
    n = L.ref_stl_read(p, None, 0)
    out = np.zeros((n, 9), dtype=np.float64)
    if n:
        L.ref_stl_read(p, _ptr(out), n)
    return out


def ref_line_filter(xyz, tol) -> np.ndarray:
    """The reference's LineCLFilter: the kept points, (k, 3), in order."""
    L = _lib("ref")
    a = _d(xyz).reshape(-1, 3)
    out = np.zeros((max(len(a), 1), 3), dtype=np.float64)
    k = L.ref_line_filter(_ptr(a), len(a), float(tol), _ptr(out), len(out))
    return out[:k]


def ref_rotate(tris, xr, yr, zr):
    """The reference's STLSurf::rotate: (rotated (n, 9) triangles, bbox[6])."""
    L = _lib("ref")
    t = _d(tris).reshape(-1, 9)
    out = np.zeros_like(t)
    bb = np.zeros(6)
    L.ref_rotate(_ptr(t), t.shape[0], float(xr), float(yr), float(zr), _ptr(out), _ptr(bb))
    return out, bb


def last_loop_seconds() -> float:
    """Wall time of the last port drop's CL loop (KD build excluded)."""
    return float(_lib("port").oracle_last_loop_seconds())
