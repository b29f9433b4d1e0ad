/*
 * ocl_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * Entry points of the two CPU checkers for the drop-/push-cutter path:
 *   oracle_*  : liboclport.so, a plain-C restatement of the reference
 *               algorithm (ocl_oracle.c), portable to the Arm GPU host;
 *   ref_*     : _ref/liboclref.so, the reference's own C++ sources compiled
 *               unmodified against a small Boost stand-in (ref_driver.cpp).
 * Both take the same arguments so tests can run either.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load them.
 */
#ifndef OCL_ORACLE_H
#define OCL_ORACLE_H

#include <stdint.h>
#include "../include/ocl_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define OCL_ORACLE_API(name) oracle_##name
#define OCL_REF_API(name) ref_##name

#define OCL_CHECKER_DECLS(P)                                                        \
/* BatchDropCutter::run() over M CL points; returns 0 on success. */               \
int P##drop(const double* tris, long ntri, const ocl_gb300_cutter* c,              \
            const double* cl, long M, int nthreads, unsigned bucket,               \
            double* z, double* cc, int32_t* type, long* ncalls);                   \
/* BatchPushCutter::run(); returns the number of intervals (may exceed cap,      \
 * then only counts are filled).  Intervals are in the reference's vector order. */\
long P##push(const double* tris, long ntri, const ocl_gb300_cutter* c, int dir,    \
             const double* fib, long F, int nthreads, unsigned bucket,             \
             int32_t* counts, double* ival, double* cc, int32_t* cctype, long cap, \
             long* ncalls);                                                        \
/* PathDropCutter::run(); returns the number of points (may exceed cap). */        \
long P##pdc(const double* tris, long ntri, const ocl_gb300_cutter* c,              \
            const double* spans, long S, double sampling, double minz,             \
            int nthreads, unsigned bucket, double* xyz, double* cc,                \
            int32_t* type, long cap);                                              \
/* AdaptivePathDropCutter::run(); returns the number of points. */                 \
long P##apdc(const double* tris, long ntri, const ocl_gb300_cutter* c,             \
             const double* spans, long S, double sampling, double min_sampling,    \
             double cos_limit, unsigned bucket, double* xyz, double* cc,           \
             int32_t* type, long cap);                                             \
/* KD-tree leaf visit order (hi before lo) of all triangles; dims 0=XY,1=YZ,2=XZ. */\
int P##kd_order(const double* tris, long ntri, unsigned bucket, int dims,          \
                int64_t* order);

OCL_CHECKER_DECLS(oracle_)
OCL_CHECKER_DECLS(ref_)

/* Oracle-only helpers used by the GPU tests. */
/* Exact-overlap candidate count sum_cl |S(cl)| (MillingCutter::overlaps). */
long oracle_overlap_pairs(const double* tris, long ntri, double radius,
                          const double* cl, long M, int nthreads);
/* Exact overlap sets S(cl) (KD search + overlaps, as dropCutter5), ascending
 * insertion indices per point; returns the total (ids filled if it fits cap). */
long oracle_overlap_sets(const double* tris, long ntri, double radius, const double* cl, long M,
                         int nthreads, int64_t* counts, int32_t* ids, long cap);

int oracle_cutter_fields(const ocl_gb300_cutter* c, double* out);
/* One edge's contact for a CL point (singleEdgeDrop): 1 with clz and cc[3]
 * when the CC lies on the segment, 0 when not, -1 beyond the radius. */
int oracle_edge_contact(const ocl_gb300_cutter* c, double x, double y, const double* p1, const double* p2,
                        double* clz, double* cc);
double oracle_last_loop_seconds(void);
int ref_preset_fields(int preset, const double* args, double* out);
/* STLSurf::rotate on a triangle list: rotated triangles and the surface bbox. */
int ref_rotate(const double* tris, long ntri, double xr, double yr, double zr, double* out, double* bb);

#ifdef __cplusplus
}
#endif
#endif
