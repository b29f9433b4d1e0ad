"""ctypes binding of libocl_gb300.so (the C ABI in include/ocl_gb300.h).

The library is the only compute path: there is no CPU fallback.  Loading
fails loudly when the library has not been built, and every call that
needs a GPU fails with NO_DEVICE when none is present.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libocl_gb300.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_u64p = C.POINTER(C.c_uint64)

# every entry point declared in include/ocl_gb300.h
EXPORTS = [
    "ocl_gb300_mesh_create", "ocl_gb300_mesh_release", "ocl_gb300_mesh_size", "ocl_gb300_mesh_bbox",
    "ocl_gb300_stl_read", "ocl_gb300_line_filter", "ocl_gb300_line_filter_device",
    "ocl_gb300_drop", "ocl_gb300_drop_device", "ocl_gb300_drop_device_noalloc", "ocl_gb300_push", "ocl_gb300_path_drop",
    "ocl_gb300_adaptive_path_drop", "ocl_gb300_stage_times", "ocl_gb300_fma_peaks", "ocl_gb300_last_error", "ocl_gb300_version",
    "ocl_gb300_device_available", "ocl_gb300_mesh_kd_order", "ocl_gb300_mesh_kd_rank", "ocl_gb300_overlap_sets",
    "ocl_gb300_certificate_check", "ocl_gb300_batch_create", "ocl_gb300_batch_run", "ocl_gb300_batch_info_get",
    "ocl_gb300_batch_release", "ocl_gb300_server_create", "ocl_gb300_server_add_mesh",
    "ocl_gb300_server_submit_drop", "ocl_gb300_server_submit_adaptive", "ocl_gb300_server_wait",
    "ocl_gb300_server_cancel", "ocl_gb300_server_stats_get", "ocl_gb300_server_pause", "ocl_gb300_server_destroy",
    "ocl_gb300_waterline", "ocl_gb300_waterline_levels", "ocl_gb300_adaptive_waterline", "ocl_gb300_weave",
    "ocl_gb300_loops_count", "ocl_gb300_loops_get", "ocl_gb300_loops_fibers", "ocl_gb300_loops_release",
]

_lib = None


class OclError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{_abi.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OclError(_abi.NO_DEVICE, f"CUDA library not built: {LIB_PATH} (run __graft_entry__.build())")
    L = C.CDLL(LIB_PATH)
    cd = C.POINTER(_abi.CutterDesc)
    st = C.POINTER(_abi.Stats)
    L.ocl_gb300_mesh_create.argtypes = [_dp, C.c_uint64, C.c_uint32, C.POINTER(C.c_void_p)]
    L.ocl_gb300_mesh_release.argtypes = [C.c_void_p]
    L.ocl_gb300_mesh_size.argtypes = [C.c_void_p]
    L.ocl_gb300_mesh_size.restype = C.c_uint64
    L.ocl_gb300_mesh_bbox.argtypes = [C.c_void_p, _dp]
    L.ocl_gb300_drop.argtypes = [C.c_void_p, cd, _dp, C.c_uint64, C.c_int, _dp, _dp, _ip, st]
    L.ocl_gb300_drop_device.argtypes = [C.c_void_p, cd, C.c_void_p, C.c_uint64, C.c_int, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, st]
    L.ocl_gb300_drop_device_noalloc.argtypes = [C.c_void_p, cd, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p]
    L.ocl_gb300_push.argtypes = [C.c_void_p, cd, C.c_int, _dp, C.c_uint64, _u64p, _dp, _dp, _ip, C.c_uint64, st]
    L.ocl_gb300_path_drop.argtypes = [C.c_void_p, cd, _dp, C.c_uint64, C.c_double, C.c_double, _dp, _dp, _ip,
                                      C.c_uint64, _u64p, st]
    L.ocl_gb300_adaptive_path_drop.argtypes = [C.c_void_p, cd, _dp, C.c_uint64, C.c_double, C.c_double, C.c_double,
                                               _dp, _dp, _ip, C.c_uint64, _u64p, st]
    L.ocl_gb300_stage_times.argtypes = [C.c_uint64, _dp]
    L.ocl_gb300_fma_peaks.argtypes = [_dp, _dp]
    L.ocl_gb300_stl_read.argtypes = [C.c_char_p, _dp, C.c_uint64, _u64p]
    L.ocl_gb300_line_filter.argtypes = [_dp, C.c_uint64, C.c_double, _u64p, _u64p]
    L.ocl_gb300_line_filter_device.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_double, C.c_void_p,
                                               C.c_void_p, C.c_void_p]
    _i64p = C.POINTER(C.c_int64)
    L.ocl_gb300_mesh_kd_order.argtypes = [C.c_void_p, C.c_int, _i64p]
    L.ocl_gb300_mesh_kd_rank.argtypes = [C.c_void_p, _i64p]
    L.ocl_gb300_overlap_sets.argtypes = [C.c_void_p, C.c_double, _dp, C.c_uint64, _u64p, _ip, C.c_uint64]
    L.ocl_gb300_certificate_check.argtypes = [C.c_void_p, cd, _dp, C.c_uint64, C.POINTER(_abi.Cert)]
    L.ocl_gb300_batch_create.argtypes = [C.POINTER(_abi.DropJob), C.c_uint64, C.POINTER(_abi.BatchOpts),
                                         C.POINTER(C.c_void_p)]
    L.ocl_gb300_batch_run.argtypes = [C.c_void_p, C.c_void_p, st]
    L.ocl_gb300_batch_info_get.argtypes = [C.c_void_p, C.POINTER(_abi.BatchInfo)]
    L.ocl_gb300_batch_release.argtypes = [C.c_void_p]
    L.ocl_gb300_server_create.argtypes = [C.POINTER(_abi.ServerOpts), C.POINTER(C.c_void_p)]
    L.ocl_gb300_server_add_mesh.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_int32)]
    L.ocl_gb300_server_submit_drop.argtypes = [C.c_void_p, C.c_int32, cd, _dp, C.c_uint64, _dp, _dp, _ip, _u64p]
    L.ocl_gb300_server_submit_adaptive.argtypes = [C.c_void_p, C.c_int32, cd, _dp, C.c_uint64, C.c_double,
                                                   C.c_double, C.c_double, _dp, _dp, _ip, C.c_uint64, _u64p, _u64p]
    L.ocl_gb300_server_wait.argtypes = [C.c_void_p, C.c_uint64, C.c_double, C.POINTER(_abi.RequestInfo)]
    L.ocl_gb300_server_cancel.argtypes = [C.c_void_p, C.c_uint64]
    L.ocl_gb300_server_stats_get.argtypes = [C.c_void_p, C.POINTER(_abi.ServerStats)]
    L.ocl_gb300_server_pause.argtypes = [C.c_void_p, C.c_int32]
    L.ocl_gb300_server_destroy.argtypes = [C.c_void_p]
    vpp = C.POINTER(C.c_void_p)
    L.ocl_gb300_waterline.argtypes = [C.c_void_p, cd, C.c_double, C.c_double, vpp, st]
    L.ocl_gb300_waterline_levels.argtypes = [C.c_void_p, cd, _dp, C.c_uint64, C.c_double, vpp, st]
    L.ocl_gb300_adaptive_waterline.argtypes = [C.c_void_p, cd, C.c_double, C.c_double, C.c_double, C.c_double, vpp,
                                               st]
    L.ocl_gb300_weave.argtypes = [_dp, C.c_uint64, _u64p, _dp, _dp, C.c_uint64, _u64p, _dp, vpp]
    L.ocl_gb300_loops_count.argtypes = [C.c_void_p, _u64p, _u64p]
    L.ocl_gb300_loops_get.argtypes = [C.c_void_p, _dp, _u64p]
    L.ocl_gb300_loops_fibers.argtypes = [C.c_void_p, C.c_int, _u64p, _u64p, _dp, _u64p, _dp, _dp, _ip]
    L.ocl_gb300_loops_release.argtypes = [C.c_void_p]
    L.ocl_gb300_last_error.restype = C.c_char_p
    L.ocl_gb300_version.restype = C.c_char_p
    _lib = L
    return L


def check(status):
    if status != 0:
        raise OclError(status, lib().ocl_gb300_last_error().decode())


def stl_read(path, strict: bool = True) -> np.ndarray:
    """(n, 9) float64 triangles of an STL file, as STLReader adds them
    (src/geo/stlreader.cpp:57-150); host code, no device needed.  strict:
    raise on an unreadable or truncated file; else return what was read
    (nothing for a file that cannot be opened, as the reference)."""
    p = os.fsencode(path)
    # one parse into a buffer sized from the file (a binary facet takes 50
    # bytes; an ASCII facet is rarely under 100); only when that guess is
    # short is the file parsed a second time, with the count the first parse
    # reported (a file rewritten in between may then read differently)
    try:
        size = os.path.getsize(path)
    except OSError:
        size = 0
    cap = max(size // 100, (size - 84) // 50, 0) + 16
    n = C.c_uint64(0)
    for _ in range(2):
        out = np.zeros((cap, 9), dtype=np.float64)
        st = lib().ocl_gb300_stl_read(p, _p(out), cap, C.byref(n))
        if st != _abi.OK and n.value > cap:
            cap = n.value
            continue
        break
    if strict:
        check(st)
    return out[:min(n.value, cap)].copy()


def line_filter(xyz, tol: float) -> np.ndarray:
    """Indices of the points LineCLFilter keeps (src/common/lineclfilter.cpp:40-77);
    host code, no device needed."""
    a = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    keep = np.zeros(max(len(a), 1), dtype=np.uint64)
    nk = C.c_uint64(0)
    check(lib().ocl_gb300_line_filter(_p(a), len(a), float(tol), _p(keep, _u64p), C.byref(nk)))
    return keep[:nk.value].astype(np.int64)


class Loops:
    """Waterline loops at one height (an ocl_gb300_loops handle): `loops` is a
    list of (n, 3) arrays of CL points, each a closed loop; `fibers(dir)` the
    X (0) or Y (1) fibers woven: (endpoints (F, 6), interval offsets (F+1),
    [lower, upper] t-values (K, 2), CC points (K, 2, 3), CC types (K, 2))."""

    def __init__(self, handle):
        self._h = handle
        try:
            n, npts = C.c_uint64(0), C.c_uint64(0)
            check(lib().ocl_gb300_loops_count(handle, C.byref(n), C.byref(npts)))
            pts = np.zeros((npts.value, 3))
            off = np.zeros(n.value + 1, dtype=np.uint64)
            check(lib().ocl_gb300_loops_get(handle, _p(pts), _p(off, _u64p)))
            self.loops = [pts[int(off[k]):int(off[k + 1])].copy() for k in range(n.value)]
            self._fibers = [_loops_fibers(handle, d) for d in (0, 1)]
        finally:
            lib().ocl_gb300_loops_release(handle)
            self._h = None

    def fibers(self, direction: int):
        return self._fibers[direction]


def _loops_fibers(handle, d):
    nf, nk = C.c_uint64(0), C.c_uint64(0)
    check(lib().ocl_gb300_loops_fibers(handle, d, C.byref(nf), C.byref(nk), None, None, None, None, None))
    fib = np.zeros((nf.value, 6))
    off = np.zeros(nf.value + 1, dtype=np.uint64)
    iv = np.zeros((nk.value, 2))
    cc = np.zeros((nk.value, 2, 3))
    ty = np.zeros((nk.value, 2), dtype=np.int32)
    check(lib().ocl_gb300_loops_fibers(handle, d, C.byref(nf), C.byref(nk), _p(fib), _p(off, _u64p), _p(iv), _p(cc),
                                       _p(ty, _ip)))
    return fib, off, iv, cc, ty


def weave(xfibers, yfibers) -> "Loops":
    """Weave::build + face_traverse (host code, no device) on X and Y fibers,
    each given as (endpoints (F, 6), interval offsets (F+1), t-values (K, 2))."""
    args = []
    for fib, off, iv in (xfibers[:3], yfibers[:3]):
        fib = _d(fib, 6)
        off = np.ascontiguousarray(off, dtype=np.uint64)
        iv = np.ascontiguousarray(iv, dtype=np.float64).reshape(-1)
        args.append((fib, off, iv))
    (xf, xo, xi), (yf, yo, yi) = args
    h = C.c_void_p()
    check(lib().ocl_gb300_weave(_p(xf), len(xf), _p(xo, _u64p), _p(xi) if xi.size else None, _p(yf), len(yf),
                                _p(yo, _u64p), _p(yi) if yi.size else None, C.byref(h)))
    return Loops(h)


def line_filter_device(d_xyz: int, d_offsets: int, npaths: int, tol: float, d_keep: int, d_nkeep: int,
                       stream: int = 0) -> None:
    """LineCLFilter over many point lists on the device (pointers as ints;
    see ocl_gb300_line_filter_device); enqueued on `stream`."""
    check(lib().ocl_gb300_line_filter_device(C.c_void_p(d_xyz), C.c_void_p(d_offsets), int(npaths), float(tol),
                                             C.c_void_p(d_keep), C.c_void_p(d_nkeep), C.c_void_p(stream)))


def fma_peaks() -> tuple:
    """(FP32, FP64) fused multiply-add throughput of the device, TFLOP/s."""
    a, b = C.c_double(0.0), C.c_double(0.0)
    check(lib().ocl_gb300_fma_peaks(C.byref(a), C.byref(b)))
    return a.value, b.value


def stage_times(count: int) -> np.ndarray:
    """(count, 4) ms of screen / refine / handed-back / whole call for this
    thread's last `count` drop calls (CUDA events on each call's stream)."""
    out = np.zeros(4 * max(count, 1))
    check(lib().ocl_gb300_stage_times(count, _p(out)))
    return out[:4 * count].reshape(count, 4)


def device_available() -> bool:
    return bool(lib().ocl_gb300_device_available())


def _d(a, cols):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a.reshape(-1, cols)


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


PRECISION = {"fp64": _abi.PREC_FP64, "mixed": _abi.PREC_MIXED}


class DeviceMesh:
    """A triangle surface resident in device memory (STLSurf + the setSTL
    indexes of the reference), built once and shared by all operations."""

    def __init__(self, tris, bucket_size: int = 1):
        t = _d(tris, 9)
        self._tris = t
        h = C.c_void_p()
        check(lib().ocl_gb300_mesh_create(_p(t), t.shape[0], bucket_size, C.byref(h)))
        self._h = h
        self.bucket_size = bucket_size

    def __len__(self):
        return int(lib().ocl_gb300_mesh_size(self._h))

    def bbox(self):
        b = np.zeros(6)
        check(lib().ocl_gb300_mesh_bbox(self._h, _p(b)))
        return b

    def release(self):
        if getattr(self, "_h", None):
            lib().ocl_gb300_mesh_release(self._h)
            self._h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def drop(self, cutter, cl, precision: str = "mixed"):
        """BatchDropCutter::run over CL points (M x 3); returns z, cc (M x 3),
        cc type (M) and the call's Stats."""
        cl = _d(cl, 3)
        M = cl.shape[0]
        z = np.empty(M)
        cc = np.empty((M, 3))
        ty = np.empty(M, dtype=np.int32)
        st = _abi.Stats()
        desc = cutter.desc()
        check(lib().ocl_gb300_drop(self._h, C.byref(desc), _p(cl), M, PRECISION[precision], _p(z), _p(cc),
                                   _p(ty, _ip), C.byref(st)))
        return z, cc, ty, st

    def drop_device(self, cutter, d_cl, M, d_z, d_cc, d_type, stream=0, precision: str = "mixed", stats=True):
        """Device-pointer variant (pointers as ints)."""
        st = _abi.Stats() if stats else None
        desc = cutter.desc()
        check(lib().ocl_gb300_drop_device(self._h, C.byref(desc), C.c_void_p(d_cl), M, PRECISION[precision],
                                          C.c_void_p(d_z), C.c_void_p(d_cc), C.c_void_p(d_type), C.c_void_p(stream),
                                          C.byref(st) if st is not None else None))
        return st

    def push(self, cutter, direction: int, fibers):
        """BatchPushCutter::run over fibers (F x 6).  Returns per-fiber lists of
        (lower, upper, lower_cc, upper_cc, lower_type, upper_type) sorted by
        lower, and the Stats."""
        fib = _d(fibers, 6)
        F = fib.shape[0]
        offsets = np.zeros(F + 1, dtype=np.uint64)
        cap = max(64, 4 * F)
        desc = cutter.desc()
        while True:
            iv = np.empty(2 * cap)
            cc = np.empty(6 * cap)
            ty = np.empty(2 * cap, dtype=np.int32)
            st = _abi.Stats()
            status = lib().ocl_gb300_push(self._h, C.byref(desc), direction, _p(fib), F, _p(offsets, _u64p), _p(iv),
                                          _p(cc), _p(ty, _ip), cap, C.byref(st))
            if status == _abi.CAPACITY:
                cap = int(offsets[-1]) + 16
                continue
            check(status)
            break
        out = []
        for f in range(F):
            rec = []
            for k in range(int(offsets[f]), int(offsets[f + 1])):
                rec.append((iv[2 * k], iv[2 * k + 1], cc[6 * k:6 * k + 3].copy(), cc[6 * k + 3:6 * k + 6].copy(),
                            int(ty[2 * k]), int(ty[2 * k + 1])))
            out.append(rec)
        return out, st

    def waterline(self, cutter, z: float, sampling: float):
        """Waterline::run at height z: a Loops (loops and the fibers woven)
        and the Stats."""
        st = _abi.Stats()
        h = C.c_void_p()
        check(lib().ocl_gb300_waterline(self._h, C.byref(cutter.desc()), float(z), float(sampling), C.byref(h),
                                        C.byref(st)))
        return Loops(h), st

    def waterline_levels(self, cutter, zs, sampling: float):
        """Waterline::run at every height in zs in one device pass per fiber
        direction: a list of Loops and the Stats."""
        z = np.ascontiguousarray(zs, dtype=np.float64).reshape(-1)
        hs = (C.c_void_p * max(len(z), 1))()
        st = _abi.Stats()
        check(lib().ocl_gb300_waterline_levels(self._h, C.byref(cutter.desc()), _p(z), len(z), float(sampling),
                                               C.cast(hs, C.POINTER(C.c_void_p)), C.byref(st)))
        return [Loops(C.c_void_p(hs[k])) for k in range(len(z))], st

    def adaptive_waterline(self, cutter, z: float, sampling: float, min_sampling: float = None,
                           cos_limit: float = 0.999):
        """AdaptiveWaterline::run at height z (min_sampling defaults to
        sampling / 10, as setSampling sets it): a Loops and the Stats."""
        ms = sampling / 10.0 if min_sampling is None else min_sampling
        st = _abi.Stats()
        h = C.c_void_p()
        check(lib().ocl_gb300_adaptive_waterline(self._h, C.byref(cutter.desc()), float(z), float(sampling),
                                                 float(ms), float(cos_limit), C.byref(h), C.byref(st)))
        return Loops(h), st

    def path_drop(self, cutter, spans, sampling, min_z):
        spans = _d(spans, _abi.SPAN_DOUBLES)
        cap = max(4096, getattr(self, "_path_cap", 0))
        desc = cutter.desc()
        while True:
            xyz = np.empty((cap, 3))
            cc = np.empty((cap, 3))
            ty = np.empty(cap, dtype=np.int32)
            n = C.c_uint64(0)
            st = _abi.Stats()
            status = lib().ocl_gb300_path_drop(self._h, C.byref(desc), _p(spans), spans.shape[0], sampling, min_z,
                                               _p(xyz), _p(cc), _p(ty, _ip), cap, C.byref(n), C.byref(st))
            if status == _abi.CAPACITY:
                cap = int(n.value)
                self._path_cap = cap
                continue
            check(status)
            k = int(n.value)
            return xyz[:k], cc[:k], ty[:k], st

    def adaptive_path_drop(self, cutter, spans, sampling, min_sampling, cos_limit=0.999):
        spans = _d(spans, _abi.SPAN_DOUBLES)
        cap = max(4096, getattr(self, "_path_cap", 0))
        desc = cutter.desc()
        while True:
            xyz = np.empty((cap, 3))
            cc = np.empty((cap, 3))
            ty = np.empty(cap, dtype=np.int32)
            n = C.c_uint64(0)
            st = _abi.Stats()
            status = lib().ocl_gb300_adaptive_path_drop(self._h, C.byref(desc), _p(spans), spans.shape[0], sampling,
                                                        min_sampling, cos_limit, _p(xyz), _p(cc), _p(ty, _ip), cap,
                                                        C.byref(n), C.byref(st))
            if status == _abi.CAPACITY:
                cap = int(n.value)
                self._path_cap = cap
                continue
            check(status)
            k = int(n.value)
            return xyz[:k], cc[:k], ty[:k], st

    # ---- introspection (parity checks) -------------------------------------
    def kd_order(self, dims: int = 0) -> np.ndarray:
        """Insertion indices in the device's KD leaf visit order (dims 0 XY,
        1 YZ, 2 XZ), as KDTree::search visits them."""
        out = np.zeros(len(self), dtype=np.int64)
        check(lib().ocl_gb300_mesh_kd_order(self._h, dims, _p(out, C.POINTER(C.c_int64))))
        return out

    def kd_rank(self) -> np.ndarray:
        """The KD visit rank of every triangle (insertion order) as stored on the device."""
        out = np.zeros(len(self), dtype=np.int64)
        check(lib().ocl_gb300_mesh_kd_rank(self._h, _p(out, C.POINTER(C.c_int64))))
        return out

    def overlap_sets(self, radius: float, cl):
        """Exact overlap sets the grid yields: (offsets[M+1], ids) with the
        insertion indices of CL point i's set, ascending, in
        ids[offsets[i]:offsets[i+1]]."""
        cl = _d(cl, 3)
        M = cl.shape[0]
        offsets = np.zeros(M + 1, dtype=np.uint64)
        cap = 0
        ids = np.zeros(1, dtype=np.int32)
        while True:
            status = lib().ocl_gb300_overlap_sets(self._h, float(radius), _p(cl), M, _p(offsets, _u64p),
                                                  _p(ids, _ip), cap)
            if status == _abi.CAPACITY:
                cap = int(offsets[-1])
                ids = np.zeros(max(cap, 1), dtype=np.int32)
                continue
            check(status)
            return offsets.astype(np.int64), ids[:int(offsets[-1])]

    def certificate(self, cutter, cl) -> dict:
        """FP64 contacts of every exact-overlap pair against the FP32 bounds
        the mixed path uses to leave work out (ocl_gb300_certificate_check)."""
        cl = _d(cl, 3)
        out = _abi.Cert()
        desc = cutter.desc()
        check(lib().ocl_gb300_certificate_check(self._h, C.byref(desc), _p(cl), cl.shape[0], C.byref(out)))
        return out.as_dict()


class DropBatch:
    """Many BatchDropCutter runs executed together (ocl_gb300_batch_*).

    jobs: sequence of (DeviceMesh, cutter, d_cl, M, d_z, d_cc, d_type) with
    device pointers as ints.  The meshes and buffers must outlive the batch.
    """

    def __init__(self, jobs, workspace_bytes=0, chunk_points=0, autotune=False, graph=True, list_capacity=0):
        self._jobs = list(jobs)
        arr = (_abi.DropJob * max(len(self._jobs), 1))()
        for k, (mesh, cutter, d_cl, M, d_z, d_cc, d_ty) in enumerate(self._jobs):
            arr[k].mesh = mesh.handle
            arr[k].cutter = cutter.desc()
            arr[k].d_cl_xyz = d_cl
            arr[k].M = M
            arr[k].d_z_out = d_z
            arr[k].d_cc_out = d_cc
            arr[k].d_type_out = d_ty
        opts = _abi.BatchOpts(workspace_bytes, chunk_points, 1 if autotune else 0, 1 if graph else 0, list_capacity, 0)
        h = C.c_void_p()
        check(lib().ocl_gb300_batch_create(arr, len(self._jobs), C.byref(opts), C.byref(h)))
        self._h = h

    def run(self, stream=0, stats=False):
        st = _abi.Stats() if stats else None
        check(lib().ocl_gb300_batch_run(self._h, C.c_void_p(stream), C.byref(st) if st is not None else None))
        return st

    def info(self) -> dict:
        out = _abi.BatchInfo()
        check(lib().ocl_gb300_batch_info_get(self._h, C.byref(out)))
        return out.as_dict()

    def release(self):
        if getattr(self, "_h", None):
            lib().ocl_gb300_batch_release(self._h)
            self._h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class ServerRequest:
    """A submitted request: its id and the arrays the results go to (kept
    alive until the request is waited for)."""

    def __init__(self, rid, kind, arrays):
        self.id = rid
        self.kind = kind
        self.arrays = arrays
        self.info = None


class Server:
    """Request loop over device-resident meshes (ocl_gb300_server_*):
    submit_drop / submit_adaptive from any thread, wait() for results."""

    def __init__(self, hbm_budget_bytes=0, slots=0, max_batch_requests=0, list_capacity=0, max_batch_points=0):
        opts = _abi.ServerOpts(hbm_budget_bytes, slots, max_batch_requests, list_capacity, max_batch_points)
        h = C.c_void_p()
        check(lib().ocl_gb300_server_create(C.byref(opts), C.byref(h)))
        self._h = h
        self._meshes = []

    def add_mesh(self, mesh) -> int:
        mid = C.c_int32(0)
        check(lib().ocl_gb300_server_add_mesh(self._h, mesh.handle, C.byref(mid)))
        self._meshes.append(mesh)
        return mid.value

    def submit_drop(self, mesh_id, cutter, cl) -> ServerRequest:
        cl = _d(cl, 3)
        M = cl.shape[0]
        z = np.empty(M)
        cc = np.empty((M, 3))
        ty = np.empty(M, dtype=np.int32)
        rid = C.c_uint64(0)
        desc = cutter.desc()
        check(lib().ocl_gb300_server_submit_drop(self._h, mesh_id, C.byref(desc), _p(cl), M, _p(z), _p(cc),
                                                 _p(ty, _ip), C.byref(rid)))
        return ServerRequest(rid.value, "drop", (cl, z, cc, ty))

    def submit_adaptive(self, mesh_id, cutter, spans, sampling, min_sampling, cos_limit=0.999, cap=None):
        spans = _d(spans, _abi.SPAN_DOUBLES)
        if cap is None:  # bisection ends at min_sampling: about two points per min_sampling of length
            length = float(np.sum(np.hypot(spans[:, 4] - spans[:, 1], spans[:, 5] - spans[:, 2]))) + 1.0
            cap = int(2 * length / min_sampling + 2 * len(spans) + 64)
            if (spans[:, 0] != 0).any():
                cap *= 8  # arcs are longer than their chords
        xyz = np.empty((cap, 3))
        cc = np.empty((cap, 3))
        ty = np.empty(cap, dtype=np.int32)
        n = C.c_uint64(0)
        rid = C.c_uint64(0)
        desc = cutter.desc()
        check(lib().ocl_gb300_server_submit_adaptive(self._h, mesh_id, C.byref(desc), _p(spans), spans.shape[0],
                                                     sampling, min_sampling, cos_limit, _p(xyz), _p(cc),
                                                     _p(ty, _ip), cap, C.byref(n), C.byref(rid)))
        return ServerRequest(rid.value, "adaptive", (spans, xyz, cc, ty, n))

    def wait(self, req: ServerRequest, timeout=-1.0):
        """Waits for the request; returns (status, results, info) with results
        (z, cc, type) for a drop and (xyz, cc, type) for an adaptive path."""
        info = _abi.RequestInfo()
        st = lib().ocl_gb300_server_wait(self._h, req.id, float(timeout), C.byref(info))
        if st == _abi.PENDING:
            return _abi.PENDING, None, None
        check(st)
        d = {"status": info.status, "batches": info.batches, "points": info.points, "queue_ms": info.queue_ms,
             "latency_ms": info.latency_ms, "message": info.message.decode(errors="replace")}
        req.info = d
        if req.kind == "drop":
            _, z, cc, ty = req.arrays
            return info.status, (z, cc, ty), d
        _, xyz, cc, ty, n = req.arrays
        k = min(int(n.value), len(ty))
        return info.status, (xyz[:k], cc[:k], ty[:k]), d

    def cancel(self, req: ServerRequest):
        check(lib().ocl_gb300_server_cancel(self._h, req.id))

    def pause(self, paused=True):
        check(lib().ocl_gb300_server_pause(self._h, 1 if paused else 0))

    def stats(self) -> dict:
        out = _abi.ServerStats()
        check(lib().ocl_gb300_server_stats_get(self._h, C.byref(out)))
        return out.as_dict()

    def close(self):
        if getattr(self, "_h", None):
            lib().ocl_gb300_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
