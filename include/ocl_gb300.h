/*
 * ocl_gb300.h -- C ABI of the GB300 drop-cutter / push-cutter library.
 *
 * Plain C: pointers, sizes and status codes; no C++ or torch types cross it.
 * The C++ facade (opencamlib_gb300/include/ocl/) and the Python binding
 * (opencamlib_gb300/__init__.py) are thin callers of these entry points.
 *
 * Each entry point replaces one step of the reference library's hot path
 * (paths relative to the opencamlib source tree):
 *
 *   ocl_gb300_mesh_create   STLSurf + BatchDropCutter::setSTL / BatchPushCutter::setSTL
 *                           (src/geo/stlsurf.cpp:32-42, src/dropcutter/batchdropcutter.cpp:54-61,
 *                            src/algo/batchpushcutter.cpp:55-70): triangles are uploaded once,
 *                           normals/bboxes precomputed, the KD order (src/common/kdtree.hpp:141-210)
 *                           recorded for tie-breaking, and the XY cell index built on the device.
 *   ocl_gb300_drop          BatchDropCutter::run() -> dropCutter5
 *                           (src/dropcutter/batchdropcutter.cpp:187-231).
 *   ocl_gb300_push          BatchPushCutter::run() -> pushCutter3
 *                           (src/algo/batchpushcutter.cpp:136-188) incl. Fiber::addInterval
 *                           (src/algo/fiber.cpp:58-93).
 *   ocl_gb300_path_drop     PathDropCutter::run() (src/dropcutter/pathdropcutter.cpp:54-80).
 *   ocl_gb300_adaptive_path_drop
 *                           AdaptivePathDropCutter::run()
 *                           (src/dropcutter/adaptivepathdropcutter.cpp:53-94).
 *
 * Errors: the reference reports nothing (asserts compiled out, std::cout);
 * here every entry returns an int status and ocl_gb300_last_error() gives the
 * message of the last failure on the calling thread.
 */
#ifndef OCL_GB300_H
#define OCL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define OCL_GB300_OK                 0
#define OCL_GB300_BAD_ARG            1
#define OCL_GB300_UNSUPPORTED_CUTTER 2
#define OCL_GB300_OOM                3
#define OCL_GB300_DEVICE_ERROR       4
#define OCL_GB300_ITER_LIMIT         5  /* a capped device loop ran out (Brent, candidate lists) */
#define OCL_GB300_NO_DEVICE          6
#define OCL_GB300_CAPACITY           7  /* caller buffer too small; needed size reported */
#define OCL_GB300_PENDING            8  /* server request not finished yet (wait timed out) */
#define OCL_GB300_CANCELLED          9  /* server request cancelled before it finished */

/* ---- CC types: numeric values of ocl::CCType (src/geo/ccpoint.hpp:33-39) */
enum ocl_gb300_cctype {
    OCL_CC_NONE = 0, OCL_CC_VERTEX, OCL_CC_VERTEX_CYL,
    OCL_CC_EDGE, OCL_CC_EDGE_HORIZ, OCL_CC_EDGE_SHAFT,
    OCL_CC_EDGE_HORIZ_CYL, OCL_CC_EDGE_HORIZ_TOR, OCL_CC_EDGE_BALL,
    OCL_CC_EDGE_POS, OCL_CC_EDGE_NEG, OCL_CC_EDGE_CYL, OCL_CC_EDGE_CONE, OCL_CC_EDGE_CONE_BASE,
    OCL_CC_FACET, OCL_CC_FACET_TIP, OCL_CC_FACET_CYL,
    OCL_CC_ERROR
};

/* ---- cutter description ---------------------------------------------- */
enum ocl_gb300_cutter_kind {
    OCL_CUTTER_CYL = 1,       /* CylCutter(d, l)            src/cutters/cylcutter.cpp:39-46  */
    OCL_CUTTER_BALL = 2,      /* BallCutter(d, l)           src/cutters/ballcutter.cpp:38-45 */
    OCL_CUTTER_BULL = 3,      /* BullCutter(d, r, l)        src/cutters/bullcutter.cpp:38-47 */
    OCL_CUTTER_CONE = 4,      /* ConeCutter(d, angle, l=10) src/cutters/conecutter.cpp:39-49 */
    OCL_CUTTER_COMPOSITE = 5  /* CompositeCutter::addCutter src/cutters/compositecutter.cpp:43-51 */
};

/* One basic (non-composite) cutter, by its constructor arguments. */
typedef struct ocl_gb300_subcutter {
    int32_t kind;            /* OCL_CUTTER_CYL .. OCL_CUTTER_CONE */
    int32_t reserved;
    double diameter;
    double corner_radius;    /* BullCutter corner radius r */
    double angle;            /* ConeCutter half-angle, radians */
    double length;           /* constructor length argument */
    /* composite only: addCutter(c, radius, height, zoffset) */
    double radius;
    double height;
    double zoffset;
} ocl_gb300_subcutter;

#define OCL_GB300_MAX_SUB 4

typedef struct ocl_gb300_cutter {
    int32_t kind;            /* OCL_CUTTER_* */
    int32_t nsub;            /* composite: number of sub-cutters (1..4) */
    ocl_gb300_subcutter base;                  /* kind != COMPOSITE */
    ocl_gb300_subcutter sub[OCL_GB300_MAX_SUB]; /* kind == COMPOSITE, in addCutter order */
    double composite_length; /* CompositeCutter::length (set by the preset constructors) */
} ocl_gb300_cutter;

/* ---- meshes ------------------------------------------------------------ */
typedef struct ocl_gb300_mesh_s* ocl_gb300_mesh;

/* tris: ntri x 9 doubles (p0.xyz, p1.xyz, p2.xyz), in STLSurf insertion order.
 * bucket_size: the KD-tree bucket size the reference would use (default 1);
 * it fixes the candidate visit order used to break exact ties. */
int ocl_gb300_mesh_create(const double* tris, uint64_t ntri, uint32_t bucket_size,
                          ocl_gb300_mesh* out);
int ocl_gb300_mesh_release(ocl_gb300_mesh mesh);
uint64_t ocl_gb300_mesh_size(ocl_gb300_mesh mesh);
/* Mesh bbox [minx maxx miny maxy minz maxz] (Bbox::operator[] order, src/geo/bbox.cpp:113-139). */
int ocl_gb300_mesh_bbox(ocl_gb300_mesh mesh, double bb[6]);
/* The triangles STLReader(path, surface) adds to an STLSurf
 * (src/geo/stlreader.cpp:57-150), in file order, as tris[9 n] = p1 p2 p3
 * (float32 coordinates widened to double).  *count receives the number of
 * triangles; call with tris = NULL, cap = 0 to size the output.  Host code
 * only (no device needed).  Errors: a file that cannot be opened, a binary
 * file shorter than its facet count (the complete facets are returned), cap
 * too small.  Where the reference loops forever (a binary file whose header
 * starts with "solid"; ASCII lines over 1,023 characters) this reader reads
 * the binary facets / cuts the line. */
int ocl_gb300_stl_read(const char* path, double* tris, uint64_t cap, uint64_t* count);

/* ---- drop-cutter ------------------------------------------------------- */
/* Precision modes. */
#define OCL_GB300_PREC_FP64   0   /* every candidate pair evaluated in FP64 */
#define OCL_GB300_PREC_MIXED  1   /* FP32 screen on local coordinates + FP64 refine (default) */

typedef struct ocl_gb300_stats {
    uint64_t pairs;          /* FP64 path: exact-overlap (CL, triangle) pairs, sum_cl |S(cl)| */
    uint64_t refined;        /* triangles evaluated in FP64 by the refinement stage */
    uint64_t iter_limit_hits;/* capped loops that ran out (0 on success) */
    uint64_t fallback;       /* CL points redone in plain FP64 (candidate list overflow) */
    uint64_t violations;     /* FP64 results below a certified FP32 bound (always 0) */
    uint64_t screened;       /* FP32 whole-triangle screens */
    uint64_t overflow_points;/* of the fallback points: candidate list overflow */
    uint64_t chain_points;   /* of the fallback points: branch thresholds kept chaining */
    uint64_t open_branch_points; /* points where a triangle's branch (cone tip/rim,
                                    composite facet short-circuit) stayed undecided
                                    by the FP32 screen */
    uint64_t untracked_branch_points; /* of those: collected again below their lower
                                    bound (the branch could not be checked in FP64) */
    uint64_t plain_points;   /* of the fallback points: more candidates than the exact
                                per-point kernel holds, done by the plain FP64 kernel */
    uint64_t verify_failed_points; /* of the fallback points: an undecided branch,
                                checked in FP64, lay below the collection threshold */
    uint64_t launches;       /* kernels of this library launched by the call */
    double   kernel_ms;      /* device time of the call's kernels (CUDA events) */
    double   screen_ms;      /* of which the FP32 screen kernel */
    double   refine_ms;      /* of which the FP64 refinement kernel */
    double   fallback_ms;    /* of which the plain FP64 kernel */
    double   total_ms;       /* wall time of the call incl. copies */
} ocl_gb300_stats;

/* Host buffers: cl_xyz (M x 3) in; z_out (M), cc_out (M x 3), type_out (M) out.
 * z_out starts from cl z (the reference lifts it: liftZ, src/geo/clpoint.cpp:79-99).
 * stats may be NULL. */
int ocl_gb300_drop(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter,
                   const double* cl_xyz, uint64_t M, int precision,
                   double* z_out, double* cc_out, int32_t* type_out,
                   ocl_gb300_stats* stats);

/* Same with device buffers (cudaStream_t passed as void*); no host sync unless stats != NULL. */
int ocl_gb300_drop_device(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter,
                          const double* d_cl_xyz, uint64_t M, int precision,
                          double* d_z_out, double* d_cc_out, int32_t* d_type_out,
                          void* stream, ocl_gb300_stats* stats);

/* Drop-cutter that allocates no device memory.  No counterpart in the
 * reference library.  For callers that cannot allocate while they run -- a
 * machine controller or real-time loop whose device memory is budgeted up
 * front (an allocation can synchronise the device and stall the loop), or a
 * host process whose own pool allocator owns the device's memory.  Device
 * buffers in and out as in ocl_gb300_drop_device (mixed precision, same
 * results); at most OCL_GB300_NOALLOC_MAX_POINTS points per call, larger
 * calls return OCL_GB300_BAD_ARG.  Scratch is one fixed array inside the
 * library (about 6.5 MB), held by every device that loads the library until
 * the process exits; the first call on a device looks its address up, so make
 * that first call before capturing any stream.  All calls share the array:
 * calls that overlap on the GPU (other streams, other host threads) race and
 * must be serialised by the caller.  Points are processed in the order given
 * (spatially ordered inputs run fastest). */
#define OCL_GB300_NOALLOC_MAX_POINTS 8192
int ocl_gb300_drop_device_noalloc(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter,
                                  const double* d_cl_xyz, uint64_t M,
                                  double* d_z_out, double* d_cc_out, int32_t* d_type_out,
                                  void* stream);

/* ---- batches of drop-cutter jobs ----------------------------------------- */
/* Many BatchDropCutter runs (each its own mesh, cutter and device point set,
 * of any size) executed together.  No counterpart in the reference, whose
 * parallelism is one OpenMP loop over the CL points of one run
 * (src/dropcutter/batchdropcutter.cpp:207); each job's results equal
 * ocl_gb300_drop_device's for that job bit for bit.  Jobs are cut into chunks,
 * chunks packed into waves under a workspace budget; each stage of a wave is
 * one persistent launch per kernel variant whose blocks take 128-point tiles
 * of any job through an atomic counter (work stealing); the run is captured
 * once into a CUDA graph and replayed by every later run.
 * The batch keeps the job array's pointers: meshes and device buffers must
 * stay valid (and meshes unchanged) until the batch is released. */
typedef struct ocl_gb300_drop_job {
    ocl_gb300_mesh mesh;
    ocl_gb300_cutter cutter;
    const double* d_cl_xyz;   /* device, M x 3 */
    uint64_t M;
    double* d_z_out;          /* device, M */
    double* d_cc_out;         /* device, M x 3 */
    int32_t* d_type_out;      /* device, M */
} ocl_gb300_drop_job;

typedef struct ocl_gb300_batch_opts {
    uint64_t workspace_bytes; /* budget of the batch's device workspace (0: 8 GiB) */
    uint64_t chunk_points;    /* jobs are cut into chunks of at most this many points (0: 1 Mi) */
    int32_t autotune;         /* 1: pick candidate-list capacity and screen grid size per kernel
                                 variant by timing a probe of the jobs (writes into the jobs'
                                 outputs while it runs) */
    int32_t graph;            /* 1: capture the run into a CUDA graph on the first run, replay after */
    int32_t list_capacity;    /* candidates kept per CL point when not autotuned (16..256; 0: 256) */
    int32_t reserved;
} ocl_gb300_batch_opts;

#define OCL_GB300_BATCH_MAX_VARIANTS 16
typedef struct ocl_gb300_batch_info {
    uint64_t jobs, chunks, waves, points;
    uint64_t launches_per_run;  /* kernel launches of one run (all waves) */
    uint64_t workspace_bytes;
    int32_t variants;           /* screen kernel variants in the batch */
    int32_t variant_kind[OCL_GB300_BATCH_MAX_VARIANTS];  /* OCL_CUTTER_* */
    int32_t variant_sig[OCL_GB300_BATCH_MAX_VARIANTS];   /* composite make-up, -1 generic */
    int32_t list_capacity[OCL_GB300_BATCH_MAX_VARIANTS]; /* chosen per variant */
    int32_t grid_mult[OCL_GB300_BATCH_MAX_VARIANTS];
} ocl_gb300_batch_info;

typedef struct ocl_gb300_batch_s* ocl_gb300_batch;
/* opts may be NULL (defaults: 8 GiB, 1 Mi-point chunks, no autotuning, graph on). */
int ocl_gb300_batch_create(const ocl_gb300_drop_job* jobs, uint64_t njobs, const ocl_gb300_batch_opts* opts,
                           ocl_gb300_batch* out);
/* Runs every job on `stream` (cudaStream_t as void*); no host sync unless
 * stats != NULL (then stats holds the counters summed over all jobs and the
 * run's device time). */
int ocl_gb300_batch_run(ocl_gb300_batch batch, void* stream, ocl_gb300_stats* stats);
int ocl_gb300_batch_info_get(ocl_gb300_batch batch, ocl_gb300_batch_info* out);
int ocl_gb300_batch_release(ocl_gb300_batch batch);

/* ---- serving: a request loop over device-resident meshes ---------------- */
/* No counterpart in the reference (which runs one operation per run() call).
 * Clients on any thread submit BatchDropCutter and AdaptivePathDropCutter
 * requests with host buffers; a scheduler thread keeps up to `slots` batches
 * on the GPU at once (batches as in ocl_gb300_batch_*), admits queued
 * requests into the next batch while its CL points fit the slot's share of
 * the device-memory budget and max_batch_points (a drop request that does
 * not fit whole is split, its pieces going through successive batches), and
 * sends an adaptive request's bisection levels through successive batches
 * (each level rejoins the head of the queue).
 * Results are those of ocl_gb300_drop / ocl_gb300_adaptive_path_drop for the
 * same request, whatever else is in the mix.  Meshes added to a server must
 * outlive it; request buffers must stay valid until ocl_gb300_server_wait
 * returns for the request (call it exactly once per request). */
typedef struct ocl_gb300_server_opts {
    uint64_t hbm_budget_bytes;  /* device memory for in-flight batches (0: 16 GiB; at least 64 MiB) */
    int32_t slots;              /* batches on the GPU at once (0: 2; at most 16) */
    int32_t max_batch_requests; /* requests per batch (0: 64) */
    int32_t list_capacity;      /* candidates kept per CL point (16..256; 0: 256) */
    int32_t max_batch_points;   /* CL points per batch (0: 262,144); a larger drop request is split into
                                   pieces over successive batches, an adaptive level is not split */
} ocl_gb300_server_opts;

typedef struct ocl_gb300_request_info {
    int32_t status;             /* OCL_GB300_OK, _CANCELLED, _CAPACITY (adaptive output too small), ... */
    int32_t batches;            /* batches the request took part in */
    uint64_t points;            /* CL points dropped for it */
    double queue_ms;            /* submission to its first batch */
    double latency_ms;          /* submission to the end of its last batch */
    char message[160];          /* why it failed */
} ocl_gb300_request_info;

typedef struct ocl_gb300_server_stats {
    uint64_t submitted, completed, failed, cancelled, rejected, batches, points, pending;
    double p50_ms, p99_ms, mean_ms, max_ms;  /* latency of completed requests */
    double elapsed_s;           /* first submission to the latest completion */
} ocl_gb300_server_stats;

typedef struct ocl_gb300_server_s* ocl_gb300_server;
int ocl_gb300_server_create(const ocl_gb300_server_opts* opts, ocl_gb300_server* out);
/* Makes `mesh` available to requests as *mesh_id. */
int ocl_gb300_server_add_mesh(ocl_gb300_server server, ocl_gb300_mesh mesh, int32_t* mesh_id);
/* BatchDropCutter request: host cl_xyz (M x 3) in; z_out (M), cc_out (M x 3),
 * type_out (M) written when the request completes.  Rejected at once
 * (BAD_ARG: unknown mesh or bad cutter). */
int ocl_gb300_server_submit_drop(ocl_gb300_server server, int32_t mesh_id, const ocl_gb300_cutter* cutter,
                                 const double* cl_xyz, uint64_t M, double* z_out, double* cc_out,
                                 int32_t* type_out, uint64_t* request_id);
/* AdaptivePathDropCutter request over S spans (as ocl_gb300_adaptive_path_drop);
 * *count receives the number of points; status CAPACITY if cap is too small.
 * Rejected at once with OOM when its first level holds more points than one
 * batch's buffers may under the budget. */
int ocl_gb300_server_submit_adaptive(ocl_gb300_server server, int32_t mesh_id, const ocl_gb300_cutter* cutter,
                                     const double* spans, uint64_t S, double sampling, double min_sampling,
                                     double cos_limit, double* xyz_out, double* cc_out, int32_t* type_out,
                                     uint64_t cap, uint64_t* count, uint64_t* request_id);
/* Waits (timeout_s < 0: without limit) for a request; OCL_GB300_PENDING on
 * timeout (the request stays), else OCL_GB300_OK with info filled and the
 * request forgotten. */
int ocl_gb300_server_wait(ocl_gb300_server server, uint64_t request_id, double timeout_s,
                          ocl_gb300_request_info* info);
/* A queued request ends as CANCELLED; one on the GPU finishes its batch
 * (an adaptive request ends as CANCELLED after it). */
int ocl_gb300_server_cancel(ocl_gb300_server server, uint64_t request_id);
int ocl_gb300_server_stats_get(ocl_gb300_server server, ocl_gb300_server_stats* out);
/* paused != 0: no new batch starts (those on the GPU finish); 0: admission resumes. */
int ocl_gb300_server_pause(ocl_gb300_server server, int32_t paused);
/* Finishes the batches on the GPU; queued requests end as CANCELLED. */
int ocl_gb300_server_destroy(ocl_gb300_server server);

/* ---- push-cutter ------------------------------------------------------- */
#define OCL_GB300_XFIBER 0
#define OCL_GB300_YFIBER 1

/* fibers: F x 6 doubles (p1.xyz, p2.xyz), all X- or all Y-fibers (dir).
 * Output: offsets (F+1): intervals of fiber f are [offsets[f], offsets[f+1]),
 * in the order Fiber::ints holds them after the reference's merges.
 * Per interval i: ival[2i]=lower, ival[2i+1]=upper,
 * cc[6i..6i+2]=lower_cc, cc[6i+3..6i+5]=upper_cc, cctype[2i]/[2i+1].
 * If cap is too small OCL_GB300_CAPACITY is returned, offsets is complete. */
int ocl_gb300_push(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, int dir,
                   const double* fibers, uint64_t F,
                   uint64_t* offsets, double* ival, double* cc, int32_t* cctype,
                   uint64_t cap, ocl_gb300_stats* stats);

/* ---- paths -------------------------------------------------------------- */
/* A path is S spans x 11 doubles: [type, p1.xyz, p2.xyz, c.xyz, dir]
 * type 0 = Line(p1,p2), 1 = Arc(p1,p2,c,dir) (src/geo/path.hpp:43-114). */
#define OCL_GB300_SPAN_DOUBLES 11

/* PathDropCutter: uniform sampling, z starts at min_z.  Output points are
 * written to xyz (cap x 3), cc, type; *count is the number produced. */
int ocl_gb300_path_drop(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter,
                        const double* spans, uint64_t S, double sampling, double min_z,
                        double* xyz, double* cc, int32_t* type, uint64_t cap,
                        uint64_t* count, ocl_gb300_stats* stats);

/* AdaptivePathDropCutter: bisection while step > sampling or (not flat and
 * step > min_sampling).  z starts from the path points (the reference does
 * not apply setZ).  Output in the reference's depth-first order. */
int ocl_gb300_adaptive_path_drop(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter,
                                 const double* spans, uint64_t S, double sampling,
                                 double min_sampling, double cos_limit,
                                 double* xyz, double* cc, int32_t* type, uint64_t cap,
                                 uint64_t* count, ocl_gb300_stats* stats);

/* ---- waterline ------------------------------------------------------------ */
/* Waterline loops at one height, kept in a handle until released: the loop
 * points and the X and Y fibers woven (Waterline::getLoops / getXFibers /
 * getYFibers, src/algo/waterline.hpp:59-63, src/pythonlib/ocl_algo.cpp:105-119).
 * Each loop is a cyclic sequence of CL points, as the reference's
 * Weave::face_traverse walks it (src/algo/weave.cpp:49-73); loops are listed
 * by their first interval end (X intervals first, in fiber and interval
 * order, lower end first; then Y intervals), and each starts there. */
typedef struct ocl_gb300_loops_s* ocl_gb300_loops;

/* Waterline::run (src/algo/waterline.cpp:78-87): X and Y fibers at height z
 * over the mesh bbox grown by two cutter radii, sampling apart
 * (init_fibers, :143-178), pushed on the device (BatchPushCutter), woven on
 * the host (SimpleWeave::build + face_traverse; run2's SmartWeave gives the
 * same loops). */
int ocl_gb300_waterline(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, double z, double sampling,
                        ocl_gb300_loops* out, ocl_gb300_stats* stats);

/* Waterline::run at nz heights in one device pass per fiber direction (the
 * levels' fibers pushed together, the levels woven in parallel on host
 * threads); out[k] receives the loops at zs[k]. */
int ocl_gb300_waterline_levels(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, const double* zs, uint64_t nz,
                               double sampling, ocl_gb300_loops* out, ocl_gb300_stats* stats);

/* AdaptiveWaterline::run (src/algo/adaptivewaterline.cpp:62-220): fibers
 * bisected along the bbox diagonal while the step exceeds sampling, or the
 * fibers are not flat (cos_limit) and the step exceeds min_sampling; each
 * bisection level's fibers are pushed in one device call per direction.
 * The reference's defaults: min_sampling = sampling / 10, cos_limit 0.999. */
int ocl_gb300_adaptive_waterline(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, double z, double sampling,
                                 double min_sampling, double cos_limit, ocl_gb300_loops* out,
                                 ocl_gb300_stats* stats);

/* Weave::build + face_traverse on caller fibers (host code only): X fibers
 * xfib (nx x 6, p1.y == p2.y, p1.z == p2.z), their intervals [xoff[f],
 * xoff[f+1]) as t-values xival (2 per interval); Y fibers likewise.  The
 * intervals of one fiber must not overlap (Fiber::addInterval merges
 * overlapping ones). */
int ocl_gb300_weave(const double* xfib, uint64_t nx, const uint64_t* xoff, const double* xival,
                    const double* yfib, uint64_t ny, const uint64_t* yoff, const double* yival,
                    ocl_gb300_loops* out);

int ocl_gb300_loops_count(ocl_gb300_loops loops, uint64_t* nloops, uint64_t* npoints);
/* points: npoints x 3; offsets: nloops + 1 (loop k is [offsets[k], offsets[k+1])) */
int ocl_gb300_loops_get(ocl_gb300_loops loops, double* points, uint64_t* offsets);
/* The fibers of one direction that were woven.  With fib == NULL only
 * *nfibers and *nintervals are set; otherwise fib (nfibers x 6), offsets
 * (nfibers + 1), ival (2 per interval), and, when not NULL, cc (6 per
 * interval) and cctype (2 per interval) as ocl_gb300_push gives them (zero
 * for fibers passed to ocl_gb300_weave). */
int ocl_gb300_loops_fibers(ocl_gb300_loops loops, int dir, uint64_t* nfibers, uint64_t* nintervals, double* fib,
                           uint64_t* offsets, double* ival, double* cc, int32_t* cctype);
int ocl_gb300_loops_release(ocl_gb300_loops loops);

/* ---- CL point filter ----------------------------------------------------- */
/* LineCLFilter::run (src/common/lineclfilter.cpp:40-77) on n points xyz[3 n]:
 * keep[0 .. *nkeep) receives the indices of the points kept, in order (the
 * first and the last always; lists of 0 or 1 points unchanged); keep must
 * hold n entries.  Host code only (no device needed). */
int ocl_gb300_line_filter(const double* xyz, uint64_t n, double tol, uint64_t* keep, uint64_t* nkeep);

/* The same filter as a device pass over many point lists at once (the CL
 * points of many PathDropCutter / AdaptivePathDropCutter paths), one warp per
 * list.  Device pointers: d_xyz (3 doubles per point), list p is points
 * [d_offsets[p], d_offsets[p+1]); d_keep receives at the same offsets the
 * indices (within the list) of the points kept, d_nkeep[p] their count.
 * Enqueued on `stream` (a cudaStream_t; NULL: the default stream); the
 * decisions are ocl_gb300_line_filter's, bit for bit. */
int ocl_gb300_line_filter_device(const double* d_xyz, const uint64_t* d_offsets, uint64_t npaths, double tol,
                                 uint64_t* d_keep, uint64_t* d_nkeep, void* stream);

/* ---- introspection (parity checks of the index and the FP32 screen) ------ */
/* The KD-tree leaf visit order the device holds: order[k] = insertion index
 * of the k-th triangle in KDTree::search order (src/common/kdtree.hpp:141-210
 * build_node, :273-304 search_node, hi child first).  dims 0 = XY (the
 * drop-cutter tree, BatchDropCutter::setSTL src/dropcutter/batchdropcutter.cpp:54-61),
 * 1 = YZ (X-fibers), 2 = XZ (Y-fibers) (BatchPushCutter::setSTL
 * src/algo/batchpushcutter.cpp:55-70).  order holds mesh_size entries.
 * No counterpart in the reference (its tree is not exposed). */
int ocl_gb300_mesh_kd_order(ocl_gb300_mesh mesh, int dims, int64_t* order);
/* The KD visit rank stored in every triangle's device record (the tie-break
 * of every fold), read back by insertion index.  No counterpart in the reference. */
int ocl_gb300_mesh_kd_rank(ocl_gb300_mesh mesh, int64_t* rank);
/* Exact overlap sets through the device grid: for CL point i (host xyz),
 * the insertion indices of every triangle the grid query finds under a
 * cutter of this radius and MillingCutter::overlaps accepts
 * (src/cutters/millingcutter.cpp:422-433), ascending, in
 * ids[offsets[i] .. offsets[i+1]).  offsets holds M + 1 entries.  If cap is
 * too small OCL_GB300_CAPACITY is returned and offsets is complete.  The set
 * the reference forms per CL point in BatchDropCutter::dropCutter5
 * (src/dropcutter/batchdropcutter.cpp:208-222: KD candidates, then overlaps). */
int ocl_gb300_overlap_sets(ocl_gb300_mesh mesh, double radius, const double* cl_xyz, uint64_t M,
                           uint64_t* offsets, int32_t* ids, uint64_t cap);

/* FP32 certificate check: for every exact-overlap (CL point, triangle) pair,
 * the FP64 contact code on its own (the whole triangle from the CL point's
 * start height, and each facet, vertex and edge contact) against the FP32
 * bounds the mixed-precision path relies on to leave work out (the screen's
 * [lo, hi], the refinement's per-part skips, the grid-entry cull).  Counts
 * of bounds exceeded; "unsafe" ones exceed it by more than the guard margin
 * and could change a result.  No counterpart in the reference. */
typedef struct ocl_gb300_cert {
    uint64_t pairs;             /* exact-overlap pairs checked */
    uint64_t lifted;            /* of those: the FP64 drop lifts the start height */
    uint64_t tri_hi_exceeded;   /* FP64 result above the screen's upper bound */
    uint64_t tri_hi_unsafe;
    uint64_t tri_lo_exceeded;   /* FP64 result below the screen's certified lower bound */
    uint64_t part_hi_exceeded;  /* a facet / vertex / edge contact above its skip bound */
    uint64_t part_hi_unsafe;
    uint64_t entry_ub_exceeded; /* a contact above the grid-entry cull's bound */
    uint64_t entry_ub_unsafe;
    uint64_t alt_hi_exceeded;   /* bull: above the per-lane screen's bound (handed-back points) */
    double max_tri_excess;      /* largest excess of each kind (mm; 0 when none) */
    double max_part_excess;
    double max_entry_excess;
    double max_lo_excess;
    double error_budget;        /* E: FP32 position error budget of the call (mm) */
    double guard;               /* margin of the bound tests (mm) */
} ocl_gb300_cert;
int ocl_gb300_certificate_check(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, const double* cl_xyz,
                                uint64_t M, ocl_gb300_cert* out);

/* ---- misc ----------------------------------------------------------------- */
/* Device time of the stages of the calling thread's last `count` (<= 256)
 * ocl_gb300_drop / _drop_device calls, oldest first: out[4k..4k+3] = FP32
 * screen, FP64 refinement, handed-back points, whole call (ms, CUDA events
 * recorded on the call's stream).  Waits for those calls to finish; it does
 * not synchronise the calls themselves, so a timed loop can read it after.
 * No counterpart in the reference (instrumentation). */
int ocl_gb300_stage_times(uint64_t count, double* out);
/* Measured fused multiply-add throughput of the current device, TFLOP/s
 * (2 flops per FMA): FP32, the ceiling of the FP32 screen, and FP64, the
 * ceiling of the FP64 contact code.  Runs for a few tens of ms.  No
 * counterpart in the reference (instrumentation). */
int ocl_gb300_fma_peaks(double* fp32_tflops, double* fp64_tflops);
const char* ocl_gb300_last_error(void);
const char* ocl_gb300_version(void);
/* 1 if a CUDA device is usable, else 0 (no compute). */
int ocl_gb300_device_available(void);

#ifdef __cplusplus
}
#endif
#endif /* OCL_GB300_H */
