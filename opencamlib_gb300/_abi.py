"""ctypes mirror of the C ABI structures and constants in include/ocl_gb300.h."""
from __future__ import annotations

import ctypes as C

OK = 0
BAD_ARG = 1
UNSUPPORTED_CUTTER = 2
OOM = 3
DEVICE_ERROR = 4
ITER_LIMIT = 5
NO_DEVICE = 6
CAPACITY = 7

PENDING = 8
CANCELLED = 9

STATUS_NAMES = {OK: "OK", BAD_ARG: "BAD_ARG", UNSUPPORTED_CUTTER: "UNSUPPORTED_CUTTER", OOM: "OOM",
                DEVICE_ERROR: "DEVICE_ERROR", ITER_LIMIT: "ITER_LIMIT", NO_DEVICE: "NO_DEVICE",
                CAPACITY: "CAPACITY", PENDING: "PENDING", CANCELLED: "CANCELLED"}

CUTTER_CYL = 1
CUTTER_BALL = 2
CUTTER_BULL = 3
CUTTER_CONE = 4
CUTTER_COMPOSITE = 5
MAX_SUB = 4

PREC_FP64 = 0
PREC_MIXED = 1

XFIBER = 0
YFIBER = 1

SPAN_DOUBLES = 11

# ocl::CCType numeric values (src/geo/ccpoint.hpp:33-39)
CCTYPE_NAMES = ["NONE", "VERTEX", "VERTEX_CYL", "EDGE", "EDGE_HORIZ", "EDGE_SHAFT", "EDGE_HORIZ_CYL",
                "EDGE_HORIZ_TOR", "EDGE_BALL", "EDGE_POS", "EDGE_NEG", "EDGE_CYL", "EDGE_CONE",
                "EDGE_CONE_BASE", "FACET", "FACET_TIP", "FACET_CYL", "ERROR"]


class SubCutter(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("diameter", C.c_double),
                ("corner_radius", C.c_double), ("angle", C.c_double), ("length", C.c_double),
                ("radius", C.c_double), ("height", C.c_double), ("zoffset", C.c_double)]


class CutterDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("nsub", C.c_int32), ("base", SubCutter),
                ("sub", SubCutter * MAX_SUB), ("composite_length", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("pairs", C.c_uint64), ("refined", C.c_uint64), ("iter_limit_hits", C.c_uint64),
                ("fallback", C.c_uint64), ("violations", C.c_uint64), ("screened", C.c_uint64),
                ("overflow_points", C.c_uint64), ("chain_points", C.c_uint64), ("open_branch_points", C.c_uint64),
                ("untracked_branch_points", C.c_uint64), ("plain_points", C.c_uint64),
                ("verify_failed_points", C.c_uint64), ("launches", C.c_uint64), ("kernel_ms", C.c_double), ("screen_ms", C.c_double),
                ("refine_ms", C.c_double), ("fallback_ms", C.c_double), ("total_ms", C.c_double)]


class Cert(C.Structure):
    """ocl_gb300_cert: FP64 contacts against the FP32 bounds they are certified by."""
    _fields_ = [("pairs", C.c_uint64), ("lifted", C.c_uint64), ("tri_hi_exceeded", C.c_uint64),
                ("tri_hi_unsafe", C.c_uint64), ("tri_lo_exceeded", C.c_uint64), ("part_hi_exceeded", C.c_uint64),
                ("part_hi_unsafe", C.c_uint64), ("entry_ub_exceeded", C.c_uint64), ("entry_ub_unsafe", C.c_uint64),
                ("alt_hi_exceeded", C.c_uint64), ("max_tri_excess", C.c_double), ("max_part_excess", C.c_double),
                ("max_entry_excess", C.c_double), ("max_lo_excess", C.c_double), ("error_budget", C.c_double),
                ("guard", C.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class DropJob(C.Structure):
    """ocl_gb300_drop_job: one BatchDropCutter run of a batch (device buffers)."""
    _fields_ = [("mesh", C.c_void_p), ("cutter", CutterDesc), ("d_cl_xyz", C.c_void_p), ("M", C.c_uint64),
                ("d_z_out", C.c_void_p), ("d_cc_out", C.c_void_p), ("d_type_out", C.c_void_p)]


class BatchOpts(C.Structure):
    _fields_ = [("workspace_bytes", C.c_uint64), ("chunk_points", C.c_uint64), ("autotune", C.c_int32),
                ("graph", C.c_int32), ("list_capacity", C.c_int32), ("reserved", C.c_int32)]


BATCH_MAX_VARIANTS = 16


class BatchInfo(C.Structure):
    _fields_ = [("jobs", C.c_uint64), ("chunks", C.c_uint64), ("waves", C.c_uint64), ("points", C.c_uint64),
                ("launches_per_run", C.c_uint64), ("workspace_bytes", C.c_uint64), ("variants", C.c_int32),
                ("variant_kind", C.c_int32 * BATCH_MAX_VARIANTS), ("variant_sig", C.c_int32 * BATCH_MAX_VARIANTS),
                ("list_capacity", C.c_int32 * BATCH_MAX_VARIANTS), ("grid_mult", C.c_int32 * BATCH_MAX_VARIANTS)]

    def as_dict(self):
        n = self.variants
        return {"jobs": self.jobs, "chunks": self.chunks, "waves": self.waves, "points": self.points,
                "launches_per_run": self.launches_per_run, "workspace_bytes": self.workspace_bytes,
                "variants": [{"kind": self.variant_kind[k], "sig": self.variant_sig[k],
                              "list_capacity": self.list_capacity[k], "grid_mult": self.grid_mult[k]}
                             for k in range(n)]}


class ServerOpts(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("slots", C.c_int32), ("max_batch_requests", C.c_int32),
                ("list_capacity", C.c_int32), ("max_batch_points", C.c_int32)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("batches", C.c_int32), ("points", C.c_uint64), ("queue_ms", C.c_double),
                ("latency_ms", C.c_double), ("message", C.c_char * 160)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("cancelled", C.c_uint64), ("rejected", C.c_uint64), ("batches", C.c_uint64), ("points", C.c_uint64),
                ("pending", C.c_uint64), ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("mean_ms", C.c_double),
                ("max_ms", C.c_double), ("elapsed_s", C.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}
