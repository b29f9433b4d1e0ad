/*
 * ocl_oracle.c -- TEST INFRASTRUCTURE ONLY: the CPU oracle for the
 * drop-cutter / push-cutter path.
 *
 * A plain-C restatement of the reference algorithm (aewallin/opencamlib,
 * paths relative to its src/ tree).  Every function cites the reference
 * function it follows and keeps its floating-point operation order, so that
 * compiled with -ffp-contract=off it reproduces the reference bit for bit
 * (pinned against oracle/_ref/liboclref.so and tests/golden/).  It is never
 * linked into the product; only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load it.
 *
 * Two deliberate differences, both in non-terminating corner cases:
 * brent_zero has an iteration cap (the reference loops forever,
 * common/brent_zero.hpp:56), and nothing is printed where the reference
 * writes to std::cout before an assert that release builds compile out.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ocl_oracle.h"

#define TOL 0.0000001            /* common/numeric.cpp:34 */
#define OE_TOL 1e-10             /* cutters/ellipse.cpp:113 */
#define PI_REF 3.1415926535897932 /* common/numeric.hpp:38 */
#define BRENT_CAP 1000

/* ------------------------------------------------------------------ */
/* Point arithmetic (geo/point.cpp)                                    */
/* ------------------------------------------------------------------ */
typedef struct { double x, y, z; } P3;

static inline P3 pt(double x, double y, double z) { P3 p = {x, y, z}; return p; }
static inline P3 padd(P3 a, P3 b) { return pt(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline P3 psub(P3 a, P3 b) { return pt(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline P3 pmul(double s, P3 a) { return pt(a.x * s, a.y * s, a.z * s); }
static inline double sq(double x) { return x * x; }
/* Point::dot point.cpp:61-63 */
static inline double pdot(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* Point::norm point.cpp:50-52 */
static inline double pnorm(P3 a) { return sqrt(sq(a.x) + sq(a.y) + sq(a.z)); }
/* Point::cross point.cpp:54-59 */
static inline P3 pcross(P3 a, P3 p) {
    return pt(a.y * p.z - a.z * p.y, a.z * p.x - a.x * p.z, a.x * p.y - a.y * p.x);
}
/* Point::normalize point.cpp:65-69 */
static inline P3 pnormalize(P3 a) {
    double n = pnorm(a);
    if (n != 0.0) a = pmul(1 / n, a);
    return a;
}
/* Point::xyNorm point.cpp:71-73 */
static inline double pxynorm(P3 a) { return sqrt(sq(a.x) + sq(a.y)); }
/* Point::xyNormalize point.cpp:75-78 (scales all three components) */
static inline P3 pxynormalize(P3 a) {
    if (pxynorm(a) != 0.0) a = pmul(1 / pxynorm(a), a);
    return a;
}
/* Point::xyPerp point.cpp:80-83 */
static inline P3 pxyperp(P3 a) { return pt(-a.y, a.x, a.z); }
/* Point::xyDistance point.cpp:130-134 */
static inline double pxydist(P3 a, P3 b) { return pxynorm(psub(a, b)); }
/* common/numeric.cpp:75-80 */
static inline int iszero_tol(double x) { return fabs(x) < TOL; }
static inline double sgn(double x) { return x < 0.0 ? -1 : 1; }

/* Point::xyDistanceToLine point.cpp:139-156 */
static double xy_distance_to_line(P3 me, P3 p1, P3 p2) {
    if (p1.x == p2.x && p1.y == p2.y) return -1;
    P3 v = pnormalize(pt(p2.y - p1.y, -(p2.x - p1.x), 0));
    P3 r = pt(p1.x - me.x, p1.y - me.y, 0);
    return fabs(pdot(v, r));
}
/* Point::closestPoint point.cpp:159-165 */
static P3 closest_point(P3 me, P3 p1, P3 p2) {
    P3 v = psub(p2, p1);
    double u = pdot(psub(me, p1), v) / pdot(v, v);
    return padd(p1, pmul(u, v));
}
/* Point::xyClosestPoint point.cpp:168-193 */
static P3 xy_closest_point(P3 me, P3 p1, P3 p2) {
    P3 v = psub(p2, p1);
    double u = (me.x - p1.x) * (v.x) + (me.y - p1.y) * (v.y);
    u = u / (v.x * v.x + v.y * v.y);
    return pt(p1.x + u * v.x, p1.y + u * v.y, 0);
}
/* Point::isInside(Triangle) point.cpp:224-239 */
static int inside_tri(P3 p, const P3* t) {
    P3 a = t[0], b = t[1], c = t[2];
    double u = (a.y * c.x - a.x * c.y + (c.y - a.y) * p.x + (a.x - c.x) * p.y) /
               (a.y * c.x - a.x * c.y + (c.y - a.y) * b.x + (a.x - c.x) * b.y);
    double v = (a.x * b.y - a.y * b.x + (a.y - b.y) * p.x + (b.x - a.x) * p.y) /
               (a.x * b.y - a.y * b.x + (a.y - b.y) * c.x + (b.x - a.x) * c.y);
    return u > 0.0 && v > 0.0 && (u + v) < 1.0;
}
/* Point::isInside(p1,p2) point.cpp:241-253 */
static int inside_seg(P3 me, P3 p1, P3 p2) {
    P3 d = psub(p2, p1);
    double t = pdot(psub(me, p1), d) / pdot(d, d);
    if (t > 1.0 || t < 0.0) return 0;
    return 1;
}
/* Point::z_projectOntoEdge point.cpp:337-347 */
static double z_project(P3 me, P3 p1, P3 p2) {
    double t;
    if (fabs(p2.x - p1.x) > fabs(p2.y - p1.y))
        t = (me.x - p1.x) / (p2.x - p1.x);
    else
        t = (me.y - p1.y) / (p2.y - p1.y);
    return p1.z + t * (p2.z - p1.z);
}
/* two_by_two_solver numeric.cpp:118-140 */
static int two_by_two(double a, double b, double c, double d, double e, double f, double* u,
                      double* v) {
    double det = a * d - c * b;
    if (iszero_tol(det)) return 0;
    *u = (1.0 / det) * (d * e - b * f);
    *v = (1.0 / det) * (-c * e + a * f);
    return 1;
}
/* xy_line_line_intersection numeric.cpp:147-154 */
static int xy_line_line(P3 p1, P3 p2, double* v, P3 p3, P3 p4, double* t) {
    return two_by_two(p2.x - p1.x, -(p4.x - p3.x), p2.y - p1.y, -(p4.y - p3.y), (p3.x - p1.x),
                      p3.y - p1.y, v, t);
}
/* xyVectorToDiangle numeric.cpp:36-51 */
static double xy_to_diangle(double x, double y) {
    if (y >= 0)
        return (x >= 0 ? y / (x + y) : 1 - x / (-x + y));
    return (x < 0 ? 2 - y / (-x - y) : 3 + x / (x - y));
}

/* ------------------------------------------------------------------ */
/* Triangle (geo/triangle.cpp), stored flat                            */
/* ------------------------------------------------------------------ */
typedef struct {
    P3 p[3];
    P3 n;          /* Triangle::calcNormal triangle.cpp:65-71 */
    double bb[6];  /* Bbox [minx maxx miny maxy minz maxz] bbox.cpp:113-139 */
} Tri;

static void tri_init(Tri* t, const double* v) {
    for (int k = 0; k < 3; ++k) t->p[k] = pt(v[3 * k], v[3 * k + 1], v[3 * k + 2]);
    P3 v1 = psub(t->p[0], t->p[1]);
    P3 v2 = psub(t->p[0], t->p[2]);
    t->n = pnormalize(pcross(v1, v2));
    /* Bbox::addPoint bbox.cpp:67-89 */
    double mnx = t->p[0].x, mxx = mnx, mny = t->p[0].y, mxy = mny, mnz = t->p[0].z, mxz = mnz;
    for (int k = 1; k < 3; ++k) {
        P3 q = t->p[k];
        if (q.x > mxx) mxx = q.x;
        if (q.x < mnx) mnx = q.x;
        if (q.y > mxy) mxy = q.y;
        if (q.y < mny) mny = q.y;
        if (q.z > mxz) mxz = q.z;
        if (q.z < mnz) mnz = q.z;
    }
    t->bb[0] = mnx; t->bb[1] = mxx; t->bb[2] = mny; t->bb[3] = mxy; t->bb[4] = mnz; t->bb[5] = mxz;
}
/* Triangle::upNormal triangle.cpp:73-75 */
static inline P3 up_normal(const Tri* t) { return (t->n.z < 0) ? pmul(-1.0, t->n) : t->n; }

/* ------------------------------------------------------------------ */
/* KD-tree (common/kdtree.hpp, common/kdnode.hpp)                      */
/* ------------------------------------------------------------------ */
typedef struct {
    int dim;
    double cut;
    int hi, lo;        /* child node index or -1 */
    long leaf_begin;   /* leaf: range in the order array */
    long leaf_end;
} KDNode;

typedef struct {
    KDNode* nodes;
    long nnodes, cap;
    long* order;       /* leaf triangles in DFS (hi before lo) order */
    long norder;
    int dims[4];
    unsigned bucket;
    const Tri* tris;
} KDTree;

static int kd_new_node(KDTree* kd) {
    if (kd->nnodes == kd->cap) {
        kd->cap = kd->cap ? 2 * kd->cap : 1024;
        kd->nodes = (KDNode*)realloc(kd->nodes, sizeof(KDNode) * kd->cap);
    }
    return (int)kd->nnodes++;
}

/* KDTree::build_node kdtree.hpp:141-210 with calc_spread kdtree.hpp:213-268. */
static int kd_build(KDTree* kd, long* idx, long n, long* scratch) {
    const Tri* T = kd->tris;
    double maxval[6], minval[6];
    int first = 1;
    for (long i = 0; i < n; ++i) {
        const double* bb = T[idx[i]].bb;
        for (int m = 0; m < 4; ++m) {
            int d = kd->dims[m];
            double v = bb[d];
            if (first) {
                maxval[d] = v;
                minval[d] = v;
                if (m == 3) first = 0;
            } else {
                if (maxval[d] < v) maxval[d] = v;
                if (minval[d] > v) minval[d] = v;
            }
        }
    }
    double mx = 0;
    int maxM = 0;
    for (int m = 0; m < 4; ++m) {
        double val = maxval[kd->dims[m]] - minval[kd->dims[m]];
        if (val > mx) { mx = val; maxM = m; }
    }
    int sd = kd->dims[maxM];
    double sval = maxval[sd] - minval[sd];
    double cut = minval[sd] + sval / 2;
    int node = kd_new_node(kd);
    kd->nodes[node].dim = sd;
    kd->nodes[node].cut = cut;
    kd->nodes[node].hi = kd->nodes[node].lo = -1;
    kd->nodes[node].leaf_begin = kd->nodes[node].leaf_end = -1;
    if ((unsigned long)n <= kd->bucket || iszero_tol(sval)) {
        kd->nodes[node].leaf_begin = kd->norder;
        for (long i = 0; i < n; ++i) kd->order[kd->norder++] = idx[i];
        kd->nodes[node].leaf_end = kd->norder;
        return node;
    }
    /* stable partition: hi = bb[d] > cut */
    long nhi = 0, nlo = 0;
    for (long i = 0; i < n; ++i)
        if (T[idx[i]].bb[sd] > cut) scratch[nhi++] = idx[i];
    long* lo = scratch + nhi;
    for (long i = 0; i < n; ++i)
        if (!(T[idx[i]].bb[sd] > cut)) lo[nlo++] = idx[i];
    memcpy(idx, scratch, sizeof(long) * n);
    if (nhi > 0) {
        int h = kd_build(kd, idx, nhi, scratch);
        kd->nodes[node].hi = h;
    }
    if (nlo > 0) {
        int l = kd_build(kd, idx + nhi, nlo, scratch);
        kd->nodes[node].lo = l;
    }
    return node;
}

static void kd_init(KDTree* kd, const Tri* tris, long ntri, unsigned bucket, int dims) {
    memset(kd, 0, sizeof(*kd));
    kd->tris = tris;
    kd->bucket = bucket ? bucket : 1;
    /* setXYDimensions / setYZDimensions / setXZDimensions kdtree.hpp:90-115 */
    static const int D[3][4] = {{0, 1, 2, 3}, {2, 3, 4, 5}, {0, 1, 4, 5}};
    for (int m = 0; m < 4; ++m) kd->dims[m] = D[dims][m];
    kd->order = (long*)malloc(sizeof(long) * (ntri > 0 ? ntri : 1));
    if (ntri == 0) return;
    long* idx = (long*)malloc(sizeof(long) * ntri);
    long* scratch = (long*)malloc(sizeof(long) * ntri);
    for (long i = 0; i < ntri; ++i) idx[i] = i;
    kd_build(kd, idx, ntri, scratch);
    free(idx);
    free(scratch);
}
static void kd_free(KDTree* kd) {
    free(kd->nodes);
    free(kd->order);
}

typedef struct { long* v; long n, cap; } LVec;
static void lv_push(LVec* a, long x) {
    if (a->n == a->cap) {
        a->cap = a->cap ? 2 * a->cap : 256;
        a->v = (long*)realloc(a->v, sizeof(long) * a->cap);
    }
    a->v[a->n++] = x;
}

/* KDTree::search_node kdtree.hpp:273-304 */
static void kd_search(const KDTree* kd, int node, const double* bb, LVec* out) {
    const KDNode* nd = &kd->nodes[node];
    if (nd->leaf_begin >= 0) {
        for (long i = nd->leaf_begin; i < nd->leaf_end; ++i) lv_push(out, kd->order[i]);
        return;
    }
    if ((nd->dim % 2) == 0) {
        int maxdim = nd->dim + 1;
        if (nd->cut > bb[maxdim]) {
            if (nd->lo >= 0) kd_search(kd, nd->lo, bb, out);
        } else {
            if (nd->hi >= 0) kd_search(kd, nd->hi, bb, out);
            if (nd->lo >= 0) kd_search(kd, nd->lo, bb, out);
        }
    } else {
        int mindim = nd->dim - 1;
        if (nd->cut < bb[mindim]) {
            if (nd->hi >= 0) kd_search(kd, nd->hi, bb, out);
        } else {
            if (nd->hi >= 0) kd_search(kd, nd->hi, bb, out);
            if (nd->lo >= 0) kd_search(kd, nd->lo, bb, out);
        }
    }
}

/* ------------------------------------------------------------------ */
/* Cutters (cutters/*.cpp)                                             */
/* ------------------------------------------------------------------ */
typedef struct Cutter {
    int kind;
    double diameter, radius, length;
    double xy_normal_length, normal_length, center_height;
    double radius1, radius2;   /* bull */
    double angle;              /* cone */
    /* composite */
    int nsub;
    struct Cutter* sub;
    double radiusvec[OCL_GB300_MAX_SUB], heightvec[OCL_GB300_MAX_SUB], zoffset[OCL_GB300_MAX_SUB];
} Cutter;

/* Constructors: CylCutter cylcutter.cpp:39-46, BallCutter ballcutter.cpp:38-45,
 * BullCutter bullcutter.cpp:38-47, ConeCutter conecutter.cpp:39-49. */
static int cutter_basic(Cutter* c, const ocl_gb300_subcutter* s) {
    memset(c, 0, sizeof(*c));
    c->kind = s->kind;
    double d = s->diameter, l = s->length;
    switch (s->kind) {
    case OCL_CUTTER_CYL:
        c->diameter = d; c->radius = d / 2.0; c->length = l;
        c->xy_normal_length = c->radius; c->normal_length = 0.0; c->center_height = 0.0;
        return 0;
    case OCL_CUTTER_BALL:
        c->diameter = d; c->radius = d / 2.0; c->length = l;
        c->normal_length = c->radius; c->xy_normal_length = 0.0; c->center_height = c->radius;
        return 0;
    case OCL_CUTTER_BULL:
        c->diameter = d; c->radius = d / 2.0; c->radius1 = d / 2.0 - s->corner_radius;
        c->radius2 = s->corner_radius; c->length = l;
        c->xy_normal_length = c->radius1; c->normal_length = c->radius2;
        c->center_height = c->radius2;
        return 0;
    case OCL_CUTTER_CONE:
        c->diameter = d; c->radius = d / 2.0; c->angle = s->angle;
        c->length = c->radius / tan(c->angle) + l;
        c->center_height = c->radius / tan(c->angle);
        c->xy_normal_length = c->radius; c->normal_length = 0.0;
        return 0;
    }
    return -1;
}

static int cutter_make(Cutter* c, const ocl_gb300_cutter* d) {
    if (d->kind != OCL_CUTTER_COMPOSITE) return cutter_basic(c, &d->base);
    /* CompositeCutter::CompositeCutter / addCutter compositecutter.cpp:35-51 */
    memset(c, 0, sizeof(*c));
    c->kind = OCL_CUTTER_COMPOSITE;
    if (d->nsub < 1 || d->nsub > OCL_GB300_MAX_SUB) return -1;
    c->nsub = d->nsub;
    c->sub = (Cutter*)calloc(d->nsub, sizeof(Cutter));
    c->radius = 0;
    c->diameter = 0;
    for (int n = 0; n < d->nsub; ++n) {
        if (cutter_basic(&c->sub[n], &d->sub[n]) != 0) return -1;
        c->radiusvec[n] = d->sub[n].radius;
        c->heightvec[n] = d->sub[n].height;
        c->zoffset[n] = d->sub[n].zoffset;
        if (d->sub[n].radius > c->radius) {
            c->radius = d->sub[n].radius;
            c->diameter = 2 * d->sub[n].radius;
        }
    }
    c->length = d->composite_length;
    return 0;
}
static void cutter_free(Cutter* c) { free(c->sub); }

/* CompositeCutter::validRadius / validHeight compositecutter.cpp:117-143 */
static int comp_valid(const double* vec, int n, double r) {
    double lo = (n == 0) ? -1E-6 : vec[n - 1] - 1E-6;
    double hi = vec[n] + 1e-6;
    return (lo <= r) && (r <= hi);
}
static int radius_to_index(const Cutter* c, double r) {
    for (int n = 0; n < c->nsub; ++n)
        if (comp_valid(c->radiusvec, n, r)) return n;
    return 0;
}
static int height_to_index(const Cutter* c, double h) {
    for (int n = 0; n < c->nsub; ++n)
        if (comp_valid(c->heightvec, n, h)) return n;
    return c->nsub - 1;
}

/* height(r): cylcutter.hpp:52, ballcutter.hpp:51, bullcutter.cpp:54-63,
 * conecutter.cpp:51-54, compositecutter.cpp:58-61 */
static double c_height(const Cutter* c, double r) {
    switch (c->kind) {
    case OCL_CUTTER_CYL: return (r <= c->radius) ? 0.0 : -1.0;
    case OCL_CUTTER_BALL: return c->radius - sqrt(sq(c->radius) - sq(r));
    case OCL_CUTTER_BULL:
        if (r <= c->radius1) return 0.0;
        else if (r <= c->radius) return c->radius2 - sqrt(sq(c->radius2) - sq(r - c->radius1));
        return -1;
    case OCL_CUTTER_CONE: return r / tan(c->angle);
    case OCL_CUTTER_COMPOSITE: {
        int idx = radius_to_index(c, r);
        return c_height(&c->sub[idx], r) + c->zoffset[idx];
    }
    }
    return -1;
}
/* width(h): cylcutter.hpp:53, ballcutter.hpp:52, bullcutter.cpp:66-68,
 * conecutter.cpp:56-61, compositecutter.cpp:64-70 */
static double c_width(const Cutter* c, double h) {
    switch (c->kind) {
    case OCL_CUTTER_CYL: return c->radius;
    case OCL_CUTTER_BALL: return (h >= c->radius) ? c->radius : sqrt(sq(c->radius) - sq(c->radius - h));
    case OCL_CUTTER_BULL:
        return (h >= c->radius2) ? c->radius : c->radius1 + sqrt(sq(c->radius2) - sq(c->radius2 - h));
    case OCL_CUTTER_CONE: return (h < c->center_height) ? h * tan(c->angle) : c->radius;
    case OCL_CUTTER_COMPOSITE: {
        int idx = height_to_index(c, h);
        return c_width(&c->sub[idx], h - c->zoffset[idx]);
    }
    }
    return -1;
}

/* ------------------------------------------------------------------ */
/* CLPoint (geo/clpoint.cpp)                                           */
/* ------------------------------------------------------------------ */
typedef struct { P3 p; int type; } CC;
typedef struct { double x, y, z; CC cc; } CL;

/* CLPoint::liftZ clpoint.cpp:79-99 */
static inline int liftz(CL* cl, double zin, CC cc) {
    if (zin > cl->z) {
        cl->z = zin;
        cl->cc = cc;
        return 1;
    }
    return 0;
}
static inline int below(const CL* cl, const Tri* t) { return cl->z < t->bb[5]; }
static inline P3 clp(const CL* cl) { return pt(cl->x, cl->y, cl->z); }

/* ------------------------------------------------------------------ */
/* Brent / ellipse (common/brent_zero.hpp, cutters/ellipse*.cpp)       */
/* ------------------------------------------------------------------ */
typedef struct { double s, t, diangle; } EPos;

/* EllipsePosition::setDiangle / setD ellipseposition.cpp:41-71 */
static EPos epos_dia(double dia) {
    EPos e;
    e.diangle = dia;
    double d = dia;
    while (d > 4.0) d -= 4.0;
    while (d < 0.0) d += 4.0;
    P3 p = pt((d < 2 ? 1 - d : d - 3), (d < 3 ? ((d > 1) ? 2 - d : d) : d - 4), 0.0);
    p = pnormalize(p);
    e.s = p.x;
    e.t = p.y;
    return e;
}

typedef struct {
    int aligned;
    P3 center;
    double a, b, offset;
    P3 major_dir, minor_dir, error_dir, target;
    EPos e1, e2, ehi;
} Ell;

/* Ellipse::ePoint ellipse.cpp:71-80, AlignedEllipse::ePoint :82-85 */
static P3 ell_epoint(const Ell* E, EPos pos) {
    if (E->aligned)
        return padd(padd(E->center, pmul(E->a * pos.s, E->major_dir)), pmul(E->b * pos.t, E->minor_dir));
    P3 p = E->center;
    p.x += E->a * pos.s;
    p.y += E->b * pos.t;
    return p;
}
/* Ellipse::normal ellipse.cpp:96-101, AlignedEllipse::normal :103-108 */
static P3 ell_normal(const Ell* E, EPos pos) {
    if (E->aligned)
        return pnormalize(padd(pmul(pos.s * E->b, E->major_dir), pmul(pos.t * E->a, E->minor_dir)));
    return pnormalize(pt(E->b * pos.s, E->a * pos.t, 0));
}
/* oePoint ellipse.cpp:88-94 */
static P3 ell_oepoint(const Ell* E, EPos pos) {
    return padd(ell_epoint(E, pos), pmul(E->offset, ell_normal(E, pos)));
}
/* Ellipse::error ellipse.cpp:319-328, AlignedEllipse::error :311-317 */
static double ell_error_pos(const Ell* E, EPos pos) {
    if (E->aligned) {
        P3 p = ell_oepoint(E, pos);
        return pdot(psub(E->target, p), E->error_dir);
    }
    return ell_oepoint(E, pos).y;
}
static double ell_error(const Ell* E, double dia) { return ell_error_pos(E, epos_dia(dia)); }

/* brent_zero brent_zero.hpp:37-123 (iteration cap added) */
static double brent_zero(double a, double b, double eps, double t, const Ell* E, int* capped) {
    double c, d, e, fa, fb, fc, m, p, q, r, s, tol;
    fa = ell_error(E, a);
    fb = ell_error(E, b);
    c = a;
    fc = fa;
    e = b - a;
    d = e;
    for (int it = 0;; ++it) {
        if (it >= BRENT_CAP) { if (capped) ++*capped; break; }
        if (fabs(fc) < fabs(fb)) {
            a = b; b = c; c = a;
            fa = fb; fb = fc; fc = fa;
        }
        tol = 2.0 * eps * fabs(b) + t;
        m = 0.5 * (c - b);
        if ((fabs(m) <= tol) || (fb == 0.0)) break;
        if ((fabs(e) < tol) || (fabs(fa) <= fabs(fb))) {
            e = m;
            d = e;
        } else {
            s = fb / fa;
            if (a == c) {
                p = 2.0 * m * s;
                q = 1.0 - s;
            } else {
                q = fa / fc;
                r = fb / fc;
                p = s * (2.0 * m * a * (q - r) - (b - a) * (r - 1.0));
                q = (q - 1.0) * (r - 1.0) * (s - 1.0);
            }
            if (p > 0.0) q = -q;
            else p = -p;
            s = e;
            e = d;
            if ((2.0 * p < (3.0 * m * q - fabs(tol * q))) && (p < fabs(0.5 * s * q))) {
                d = p / q;
            } else {
                e = m;
                d = e;
            }
        }
        a = b;
        fa = fb;
        if (fabs(d) > tol) b = b + d;
        else if (m > 0.0) b = b + tol;
        else b = b - tol;
        fb = ell_error(E, b);
        if (signbit(fb) == signbit(fc)) {
            c = a;
            fc = fa;
            e = b - a;
            d = e;
        }
    }
    return b;
}

/* Ellipse::find_EllipsePosition2 ellipse.cpp:118-178 */
static void ell_find2(Ell* E) {
    double err1 = fabs(ell_error_pos(E, E->e1));
    /* candidates in the reference's order: (s,-t), (-s,t), (-s,-t), then (s,t) */
    const double sg[4][2] = {{1, -1}, {-1, 1}, {-1, -1}, {1, 1}};
    for (int k = 0; k < 4; ++k) {
        E->e2.s = sg[k][0] > 0 ? E->e1.s : -E->e1.s;
        E->e2.t = sg[k][1] > 0 ? E->e1.t : -E->e1.t;
        if (fabs(ell_error_pos(E, E->e2)) < err1 + OE_TOL) {
            if (k == 3) return;
            if ((fabs(E->e2.s - E->e1.s) > 1E-8) || (fabs(E->e2.t - E->e1.t) > 1E-8)) return;
        }
    }
}

/* Ellipse::solver_brent ellipse.cpp:186-208 */
static void ell_solver_brent(Ell* E, int* capped) {
    EPos apos = epos_dia(0.0), bpos = epos_dia(3.0);
    if (fabs(ell_error_pos(E, apos)) < OE_TOL) {
        E->e1 = apos;
        ell_find2(E);
        return;
    } else if (fabs(ell_error_pos(E, bpos)) < OE_TOL) {
        E->e1 = bpos;
        ell_find2(E);
        return;
    }
    double dia = brent_zero(apos.diangle, bpos.diangle, 3E-16, OE_TOL, E, capped);
    E->e1 = epos_dia(dia);
    ell_find2(E);
}

/* Ellipse::calcEcenter ellipse.cpp:332-338 */
static P3 ell_calc_ecenter(const Ell* E, P3 up1, P3 up2, int sln) {
    P3 cle = ell_oepoint(E, sln == 1 ? E->e1 : E->e2);
    double xoffset = -cle.x;
    double t = (E->center.x + xoffset - up1.x) / (up2.x - up1.x);
    return padd(up1, pmul(t, psub(up2, up1)));
}
/* Ellipse::setEllipsePositionHi ellipse.cpp:344-354 */
static void ell_set_hi(Ell* E, P3 u1, P3 u2) {
    P3 c1 = ell_calc_ecenter(E, u1, u2, 1);
    P3 c2 = ell_calc_ecenter(E, u1, u2, 2);
    if (c1.z >= c2.z) { E->ehi = E->e1; E->center = c1; }
    else { E->ehi = E->e2; E->center = c2; }
}

/* ------------------------------------------------------------------ */
/* Drop-cutter                                                         */
/* ------------------------------------------------------------------ */
typedef struct { int capped; } Ctx;

/* singleEdgeDropCanonical: Cyl cylcutter.cpp:52-70, Ball ballcutter.cpp:50-63,
 * Bull bullcutter.cpp:82-105, Cone conecutter.cpp:109-135 */
static void edge_canonical(const Cutter* c, P3 u1, P3 u2, double* ccu, double* clz, Ctx* ctx) {
    switch (c->kind) {
    case OCL_CUTTER_CYL: {
        double s = sqrt(sq(c->radius) - sq(u1.y));
        P3 cc1 = pt(s, u1.y, 0), cc2 = pt(-s, u1.y, 0);
        cc1.z = z_project(cc1, u1, u2);
        cc2.z = z_project(cc2, u1, u2);
        if (cc1.z > cc2.z) { *ccu = cc1.x; *clz = cc1.z; }
        else { *ccu = cc2.x; *clz = cc2.z; }
        return;
    }
    case OCL_CUTTER_BALL: {
        double s = sqrt(sq(c->radius) - sq(u1.y));
        P3 nrm = pxynormalize(pt(u2.z - u1.z, -(u2.x - u1.x), 0));
        if (nrm.y < 0) nrm = pmul(-1, nrm);
        P3 cc = pt(-s * nrm.x, u1.y, 0);
        cc.z = z_project(cc, u1, u2);
        *ccu = cc.x;
        *clz = cc.z + s * nrm.y - c->radius;
        return;
    }
    case OCL_CUTTER_BULL: {
        if (iszero_tol(u1.z - u2.z)) {
            *ccu = 0;
            *clz = u1.z - c_height(c, u1.y);
            return;
        }
        double b_axis = c->radius2;
        double theta = atan((u2.z - u1.z) / (u2.x - u1.x));
        double a_axis = fabs(c->radius2 / sin(theta));
        Ell E;
        memset(&E, 0, sizeof(E));
        E.center = pt(0, u1.y, 0);
        E.a = a_axis;
        E.b = b_axis;
        E.offset = c->radius1;
        E.e1 = epos_dia(0.0); E.e2 = E.e1; E.ehi = E.e1;
        E.e2.diangle = 0.0;
        ell_solver_brent(&E, &ctx->capped);
        ell_set_hi(&E, u1, u2);
        P3 ell_ccp = ell_epoint(&E, E.ehi);
        P3 cc_u = closest_point(ell_ccp, u1, u2);
        *ccu = cc_u.x;
        *clz = E.center.z - c->radius2;
        return;
    }
    case OCL_CUTTER_CONE: {
        double d = u1.y;
        double m = (u2.z - u1.z) / (u2.x - u1.x);
        double xu = sqrt(sq(c->radius) - sq(u1.y));
        double mu = (c->center_height / c->radius) * xu / sqrt(sq(xu) + sq(d));
        int hyp = (fabs(m) <= fabs(mu));
        double cu;
        if (hyp)
            cu = sgn(m) * sqrt(sq(c->radius) * sq(m) * sq(d) / (sq(c->length) - sq(c->radius) * sq(m)));
        else
            cu = sgn(m) * xu;
        P3 cc = pt(cu, d, 0.0);
        cc.z = z_project(cc, u1, u2);
        if (hyp)
            *clz = cc.z - c->center_height + (c->radius - sqrt(sq(cu) + sq(d))) / tan(c->angle);
        else
            *clz = cc.z - c->center_height;
        *ccu = cu;
        return;
    }
    }
}

/* MillingCutter::singleEdgeDrop millingcutter.cpp:121-136 */
static int single_edge_drop(const Cutter* c, CL* cl, P3 p1, P3 p2, double d, Ctx* ctx) {
    P3 v = psub(p2, p1);
    P3 vxy = pxynormalize(pt(v.x, v.y, 0.0));
    P3 sc = xy_closest_point(clp(cl), p1, p2);
    P3 u1 = pt(pdot(psub(p1, sc), vxy), d, p1.z);
    P3 u2 = pt(pdot(psub(p2, sc), vxy), d, p2.z);
    double ccu, clz;
    edge_canonical(c, u1, u2, &ccu, &clz, ctx);
    CC cc;
    cc.p = padd(sc, pmul(ccu, vxy));
    cc.type = OCL_CC_EDGE;
    cc.p.z = z_project(cc.p, p1, p2);
    if (inside_seg(cc.p, p1, p2)) return liftz(cl, clz, cc);
    return 0;
}

/* One edge's contact (MillingCutter::singleEdgeDrop millingcutter.cpp:100-136)
 * for a CL point at (x, y) on its own: 1 and clz, cc[3] when the CC lies on
 * the segment, 0 when it does not, -1 when the line is beyond the radius. */
int oracle_edge_contact(const ocl_gb300_cutter* cd, double x, double y, const double* a, const double* b,
                        double* clz, double* cc) {
    Cutter c;
    if (cutter_make(&c, cd) != 0) return -2;
    CL cl;
    memset(&cl, 0, sizeof(cl));
    cl.x = x;
    cl.y = y;
    cl.z = -1e300;
    P3 p1 = pt(a[0], a[1], a[2]), p2 = pt(b[0], b[1], b[2]);
    double d = xy_distance_to_line(clp(&cl), p1, p2);
    int r = -1;
    if (d <= c.radius) {
        Ctx ctx = {0};
        r = single_edge_drop(&c, &cl, p1, p2, d, &ctx);
        *clz = cl.z;
        cc[0] = cl.cc.p.x;
        cc[1] = cl.cc.p.y;
        cc[2] = cl.cc.p.z;
    }
    cutter_free(&c);
    return r;
}

/* MillingCutter::edgeDrop millingcutter.cpp:79-94 */
static int edge_drop_basic(const Cutter* c, CL* cl, const Tri* t, Ctx* ctx) {
    int result = 0;
    for (int n = 0; n < 3; ++n) {
        P3 p1 = t->p[n], p2 = t->p[(n + 1) % 3];
        if (!iszero_tol(p1.x - p2.x) || !iszero_tol(p1.y - p2.y)) {
            double d = xy_distance_to_line(clp(cl), p1, p2);
            if (d <= c->radius)
                if (single_edge_drop(c, cl, p1, p2, d, ctx)) result = 1;
        }
    }
    return result;
}

/* MillingCutter::facetDrop millingcutter.cpp:51-75 */
static int facet_drop_base(const Cutter* c, CL* cl, const Tri* t) {
    P3 normal = up_normal(t);
    if (iszero_tol(normal.z)) return 0;
    if (iszero_tol(normal.x) && iszero_tol(normal.y)) {
        CC cc;
        cc.p = pt(cl->x, cl->y, t->p[0].z);
        cc.type = OCL_CC_FACET;
        if (inside_tri(cc.p, t->p)) return liftz(cl, cc.p.z, cc);
        return 0;
    }
    double d = -pdot(normal, t->p[0]);
    normal = pnormalize(normal);
    P3 xyn = pxynormalize(pt(normal.x, normal.y, 0.0));
    P3 rv = padd(pmul(c->xy_normal_length, xyn), pmul(c->normal_length, normal));
    CC cc;
    cc.p = psub(clp(cl), rv);
    cc.p.z = (1.0 / normal.z) * (-d - normal.x * cc.p.x - normal.y * cc.p.y);
    cc.type = OCL_CC_FACET;
    double tip_z = cc.p.z + rv.z - c->center_height;
    if (inside_tri(cc.p, t->p)) return liftz(cl, tip_z, cc);
    return 0;
}

/* ConeCutter::facetDrop conecutter.cpp:70-105 */
static int facet_drop_cone(const Cutter* c, CL* cl, const Tri* t) {
    P3 normal = up_normal(t);
    if (iszero_tol(normal.z)) return 0;
    if (iszero_tol(normal.x) && iszero_tol(normal.y)) {
        CC cc;
        cc.p = pt(cl->x, cl->y, t->p[0].z);
        cc.type = OCL_CC_FACET_TIP;
        if (inside_tri(cc.p, t->p)) return liftz(cl, cc.p.z, cc);
        return 0;
    }
    double a = normal.x, b = normal.y, cc_ = normal.z;
    double d = -pdot(normal, t->p[0]);
    normal = pxynormalize(normal);
    CC cyl;
    cyl.p = psub(clp(cl), pmul(c->radius, normal));
    cyl.p.z = (1.0 / cc_) * (-d - a * cyl.p.x - b * cyl.p.y);
    double cyl_cl_z = cyl.p.z - c->length;
    cyl.type = OCL_CC_FACET_CYL;
    CC tip;
    tip.p = pt(cl->x, cl->y, 0.0);
    tip.p.z = (1.0 / cc_) * (-d - a * tip.p.x - b * tip.p.y);
    double tip_cl_z = tip.p.z;
    tip.type = OCL_CC_FACET_TIP;
    int result = 0;
    result = result || (inside_tri(tip.p, t->p) && liftz(cl, tip_cl_z, tip));
    result = result || (inside_tri(cyl.p, t->p) && liftz(cl, cyl_cl_z, cyl));
    return result;
}

static int facet_drop(const Cutter* c, CL* cl, const Tri* t, Ctx* ctx);
static int edge_drop(const Cutter* c, CL* cl, const Tri* t, Ctx* ctx);

/* CompositeCutter::ccValidRadius compositecutter.cpp:86-102 */
static int cc_valid_radius(const Cutter* c, int n, const CL* cl) {
    if (cl->cc.type == OCL_CC_NONE) return 0;
    double d = pxydist(clp(cl), cl->cc.p);
    double lo = (n == 0) ? -1E-6 : c->radiusvec[n - 1] - 1E-6;
    double hi = c->radiusvec[n] + 1e-6;
    if (d < lo) return 0;
    if (d > hi) return 0;
    return 1;
}

/* CompositeCutter::facetDrop / edgeDrop compositecutter.cpp:152-193 */
static int comp_drop(const Cutter* c, CL* cl, const Tri* t, int facet, Ctx* ctx) {
    int result = 0;
    for (int n = 0; n < c->nsub; ++n) {
        CL tmp;
        tmp.x = cl->x;
        tmp.y = cl->y;
        tmp.z = cl->z + c->zoffset[n];
        tmp.cc.p = pt(0, 0, 0);
        tmp.cc.type = OCL_CC_NONE;
        int hit = facet ? facet_drop(&c->sub[n], &tmp, t, ctx) : edge_drop(&c->sub[n], &tmp, t, ctx);
        if (hit && cc_valid_radius(c, n, &tmp)) {
            CC cc = tmp.cc;
            cc.type = facet ? OCL_CC_FACET : OCL_CC_EDGE;
            if (liftz(cl, tmp.z - c->zoffset[n], cc)) result = 1;
        }
    }
    return result;
}

static int facet_drop(const Cutter* c, CL* cl, const Tri* t, Ctx* ctx) {
    if (c->kind == OCL_CUTTER_CONE) return facet_drop_cone(c, cl, t);
    if (c->kind == OCL_CUTTER_COMPOSITE) return comp_drop(c, cl, t, 1, ctx);
    return facet_drop_base(c, cl, t);
}
static int edge_drop(const Cutter* c, CL* cl, const Tri* t, Ctx* ctx) {
    if (c->kind == OCL_CUTTER_COMPOSITE) return comp_drop(c, cl, t, 0, ctx);
    return edge_drop_basic(c, cl, t, ctx);
}

/* MillingCutter::vertexDrop millingcutter.cpp:36-47 */
static int vertex_drop(const Cutter* c, CL* cl, const Tri* t) {
    int result = 0;
    for (int k = 0; k < 3; ++k) {
        P3 p = t->p[k];
        double q = pxydist(clp(cl), p);
        if (q <= c->radius) {
            CC cc;
            cc.p = p;
            cc.type = OCL_CC_VERTEX;
            if (liftz(cl, p.z - c_height(c, q), cc)) result = 1;
        }
    }
    return result;
}

/* MillingCutter::dropCutter millingcutter.cpp:386-409 */
static void drop_cutter(const Cutter* c, CL* cl, const Tri* t, Ctx* ctx) {
    if (below(cl, t)) {
        int facet = facet_drop(c, cl, t, ctx);
        if (!facet) {
            vertex_drop(c, cl, t);
            if (below(cl, t)) edge_drop(c, cl, t, ctx);
        }
    }
}

/* MillingCutter::overlaps millingcutter.cpp:422-433 */
static inline int overlaps(const Cutter* c, const CL* cl, const Tri* t) {
    if (t->bb[1] < cl->x - c->radius) return 0;
    else if (t->bb[0] > cl->x + c->radius) return 0;
    else if (t->bb[3] < cl->y - c->radius) return 0;
    else if (t->bb[2] > cl->y + c->radius) return 0;
    return 1;
}

typedef struct {
    Tri* tris;
    long ntri;
    KDTree kd;
    Cutter cutter;
} Scene;

static int scene_init(Scene* S, const double* tris, long ntri, const ocl_gb300_cutter* cd,
                      unsigned bucket, int dims) {
    memset(S, 0, sizeof(*S));
    if (cutter_make(&S->cutter, cd) != 0) return OCL_GB300_UNSUPPORTED_CUTTER;
    S->ntri = ntri;
    S->tris = (Tri*)malloc(sizeof(Tri) * (ntri > 0 ? ntri : 1));
    for (long i = 0; i < ntri; ++i) tri_init(&S->tris[i], tris + 9 * i);
    kd_init(&S->kd, S->tris, ntri, bucket, dims);
    return 0;
}
static void scene_free(Scene* S) {
    kd_free(&S->kd);
    free(S->tris);
    cutter_free(&S->cutter);
}

/* PointDropCutter::pointDropCutter1 pointdropcutter.cpp:63-81 (the per-point
 * body of BatchDropCutter::dropCutter5 batchdropcutter.cpp:187-231) */
static long point_drop(const Scene* S, CL* cl, LVec* buf, Ctx* ctx) {
    const Cutter* c = &S->cutter;
    double r = c->radius;
    double bb[6] = {cl->x - r, cl->x + r, cl->y - r, cl->y + r, cl->z, cl->z + c->length};
    buf->n = 0;
    if (S->ntri > 0) kd_search(&S->kd, 0, bb, buf);
    long calls = 0;
    for (long k = 0; k < buf->n; ++k) {
        const Tri* t = &S->tris[buf->v[k]];
        if (overlaps(c, cl, t)) {
            if (below(cl, t)) {
                drop_cutter(c, cl, t, ctx);
                ++calls;
            }
        }
    }
    return calls;
}

static double g_last_loop_seconds = 0.0;

/* Wall time of the last oracle_drop's CL loop (KD build excluded). */
double oracle_last_loop_seconds(void) { return g_last_loop_seconds; }

int oracle_drop(const double* tris, long ntri, const ocl_gb300_cutter* cd, const double* clin,
                long M, int nthreads, unsigned bucket, double* z, double* cc, int32_t* type,
                long* ncalls) {
    Scene S;
    int st = scene_init(&S, tris, ntri, cd, bucket, 0);
    if (st) return st;
    long calls = 0;
#ifdef _OPENMP
    double t0 = omp_get_wtime();
#endif
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel reduction(+ : calls)
    {
        LVec buf = {0, 0, 0};
        Ctx ctx = {0};
#pragma omp for schedule(dynamic, 16)
        for (long i = 0; i < M; ++i) {
            CL cl;
            cl.x = clin[3 * i];
            cl.y = clin[3 * i + 1];
            cl.z = clin[3 * i + 2];
            cl.cc.p = pt(0, 0, 0);
            cl.cc.type = OCL_CC_NONE;
            calls += point_drop(&S, &cl, &buf, &ctx);
            z[i] = cl.z;
            cc[3 * i] = cl.cc.p.x;
            cc[3 * i + 1] = cl.cc.p.y;
            cc[3 * i + 2] = cl.cc.p.z;
            type[i] = cl.cc.type;
        }
        free(buf.v);
    }
#ifdef _OPENMP
    g_last_loop_seconds = omp_get_wtime() - t0;
#endif
    if (ncalls) *ncalls = calls;
    scene_free(&S);
    return 0;
}

long oracle_overlap_pairs(const double* tris, long ntri, double radius, const double* cl, long M,
                          int nthreads) {
    Tri* T = (Tri*)malloc(sizeof(Tri) * (ntri > 0 ? ntri : 1));
    for (long i = 0; i < ntri; ++i) tri_init(&T[i], tris + 9 * i);
    Cutter c;
    memset(&c, 0, sizeof(c));
    c.radius = radius;
    long total = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for reduction(+ : total) schedule(dynamic, 64)
    for (long i = 0; i < M; ++i) {
        CL p;
        p.x = cl[3 * i];
        p.y = cl[3 * i + 1];
        p.z = cl[3 * i + 2];
        for (long k = 0; k < ntri; ++k) total += overlaps(&c, &p, &T[k]);
    }
    free(T);
    return total;
}

/* The exact overlap set S(cl) of BatchDropCutter::dropCutter5
 * (batchdropcutter.cpp:208-222): KD candidates of the cutter's bbox
 * (KDTree::search_cutter_overlap kdtree.hpp:130-135) filtered by
 * MillingCutter::overlaps, as ascending insertion indices.  counts[i] gets
 * |S(cl_i)|; ids (may be NULL) receives the sets back to back while they fit
 * in cap.  Returns the total. */
static int cmp_long(const void* a, const void* b) {
    long x = *(const long*)a, y = *(const long*)b;
    return (x > y) - (x < y);
}

long oracle_overlap_sets(const double* tris, long ntri, double radius, const double* cl, long M,
                         int nthreads, int64_t* counts, int32_t* ids, long cap) {
    ocl_gb300_cutter cd;
    memset(&cd, 0, sizeof(cd));
    cd.kind = OCL_CUTTER_CYL;
    cd.base.kind = OCL_CUTTER_CYL;
    cd.base.diameter = 2.0 * radius;
    cd.base.length = 1.0;
    Scene S;
    if (scene_init(&S, tris, ntri, &cd, 1, 0) != 0) return -1;
    S.cutter.radius = radius;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        LVec buf = {0, 0, 0};
#pragma omp for schedule(dynamic, 16)
        for (long i = 0; i < M; ++i) {
            CL p;
            memset(&p, 0, sizeof(p));
            p.x = cl[3 * i];
            p.y = cl[3 * i + 1];
            p.z = cl[3 * i + 2];
            double bb[6] = {p.x - radius, p.x + radius, p.y - radius, p.y + radius, p.z, p.z + 1.0};
            buf.n = 0;
            if (ntri > 0) kd_search(&S.kd, 0, bb, &buf);
            long n = 0;
            for (long k = 0; k < buf.n; ++k)
                if (overlaps(&S.cutter, &p, &S.tris[buf.v[k]])) ++n;
            counts[i] = n;
        }
        free(buf.v);
    }
    long total = 0;
    for (long i = 0; i < M; ++i) total += counts[i];
    if (ids && total <= cap) {
        long* start = (long*)malloc(sizeof(long) * (M > 0 ? M : 1));
        long acc = 0;
        for (long i = 0; i < M; ++i) {
            start[i] = acc;
            acc += counts[i];
        }
#pragma omp parallel
        {
            LVec buf = {0, 0, 0};
#pragma omp for schedule(dynamic, 16)
            for (long i = 0; i < M; ++i) {
                CL p;
                memset(&p, 0, sizeof(p));
                p.x = cl[3 * i];
                p.y = cl[3 * i + 1];
                p.z = cl[3 * i + 2];
                double bb[6] = {p.x - radius, p.x + radius, p.y - radius, p.y + radius, p.z, p.z + 1.0};
                buf.n = 0;
                if (ntri > 0) kd_search(&S.kd, 0, bb, &buf);
                long n = 0;
                for (long k = 0; k < buf.n; ++k)
                    if (overlaps(&S.cutter, &p, &S.tris[buf.v[k]])) buf.v[n++] = buf.v[k];
                qsort(buf.v, (size_t)n, sizeof(long), cmp_long);
                for (long k = 0; k < n; ++k) ids[start[i] + k] = (int32_t)buf.v[k];
            }
            free(buf.v);
        }
        free(start);
    }
    scene_free(&S);
    return total;
}

int oracle_kd_order(const double* tris, long ntri, unsigned bucket, int dims, int64_t* order) {
    Tri* T = (Tri*)malloc(sizeof(Tri) * (ntri > 0 ? ntri : 1));
    for (long i = 0; i < ntri; ++i) tri_init(&T[i], tris + 9 * i);
    KDTree kd;
    kd_init(&kd, T, ntri, bucket, dims);
    for (long i = 0; i < kd.norder; ++i) order[i] = kd.order[i];
    int ok = (kd.norder == ntri) ? 0 : -1;
    kd_free(&kd);
    free(T);
    return ok;
}

/* ------------------------------------------------------------------ */
/* Push-cutter                                                         */
/* ------------------------------------------------------------------ */
typedef struct { P3 p1, p2, dir; } Fib;

/* Fiber::tval fiber.cpp:95-101, Fiber::point :103-106 */
static inline double f_tval(const Fib* f, P3 p) {
    P3 d = psub(f->p2, f->p1);
    return pdot(psub(p, f->p1), d) / pdot(d, d);
}
static inline P3 f_point(const Fib* f, double t) { return padd(f->p1, pmul(t, psub(f->p2, f->p1))); }

typedef struct { double lower, upper; CC lcc, ucc; } Ival;

/* Interval::Interval interval.cpp:29-35 */
static inline void iv_init(Ival* i) {
    i->lower = 0.0;
    i->upper = 0.0;
    i->lcc.p = pt(0, 0, 0);
    i->lcc.type = OCL_CC_NONE;
    i->ucc = i->lcc;
}
/* Interval::updateUpper / updateLower interval.cpp:62-93 */
static inline void iv_upper(Ival* i, double t, CC p) {
    if (i->ucc.type == OCL_CC_NONE) {
        i->upper = t; i->lower = t; i->ucc = p; i->lcc = p;
    }
    if (t > i->upper) { i->upper = t; i->ucc = p; }
}
static inline void iv_lower(Ival* i, double t, CC p) {
    if (i->lcc.type == OCL_CC_NONE) {
        i->lower = t; i->upper = t; i->lcc = p; i->ucc = p;
    }
    if (t < i->lower) { i->lower = t; i->lcc = p; }
}
/* Interval::update interval.cpp:44-47 */
static inline void iv_update(Ival* i, double t, CC p) {
    iv_upper(i, t, p);
    iv_lower(i, t, p);
}
/* Interval::update_ifCCinEdgeAndTrue interval.cpp:49-58 */
static inline int iv_update_if(Ival* i, double t, CC cc, P3 p1, P3 p2, int cond) {
    if (inside_seg(cc.p, p1, p2) && cond) {
        iv_update(i, t, cc);
        return 1;
    }
    return 0;
}

/* MillingCutter::singleVertexPush millingcutter.cpp:148-167 */
static int single_vertex_push(const Cutter* c, const Fib* f, Ival* i, P3 p, int type) {
    if ((p.z >= f->p1.z) && (p.z <= (f->p1.z + c->length))) {
        P3 pq = xy_closest_point(p, f->p1, f->p2);
        double q = pxynorm(psub(p, pq));
        double h = p.z - f->p1.z;
        double cw = c_width(c, h);
        if (q <= cw) {
            double ofs = sqrt(sq(cw) - sq(q));
            P3 start = psub(pq, pmul(ofs, f->dir));
            P3 stop = padd(pq, pmul(ofs, f->dir));
            CC cc;
            cc.p = p;
            cc.type = type;
            iv_upper(i, f_tval(f, stop), cc);
            iv_lower(i, f_tval(f, start), cc);
            return 1;
        }
    }
    return 0;
}

/* Triangle::zslice_verts triangle.cpp:77-128 */
static int zslice_verts(const Tri* t, P3* p1, P3* p2, double zcut) {
    if ((zcut <= t->bb[4]) || (zcut >= t->bb[5])) return 0;
    P3 below_[3], above_[3];
    int nb = 0, na = 0;
    for (int m = 0; m < 3; ++m) {
        if (t->p[m].z <= zcut) below_[nb++] = t->p[m];
        else above_[na++] = t->p[m];
    }
    if (nb == 2) {
        double t1 = (zcut - above_[0].z) / (below_[0].z - above_[0].z);
        double t2 = (zcut - above_[0].z) / (below_[1].z - above_[0].z);
        *p1 = padd(above_[0], pmul(t1, psub(below_[0], above_[0])));
        *p2 = padd(above_[0], pmul(t2, psub(below_[1], above_[0])));
        return 1;
    } else if (nb == 1) {
        double t1 = (zcut - above_[0].z) / (below_[0].z - above_[0].z);
        double t2 = (zcut - above_[1].z) / (below_[0].z - above_[1].z);
        *p1 = padd(above_[0], pmul(t1, psub(below_[0], above_[0])));
        *p2 = padd(above_[1], pmul(t2, psub(below_[0], above_[1])));
        return 1;
    }
    return 0;
}

/* MillingCutter::vertexPush millingcutter.cpp:139-146, CylCutter::vertexPush cylcutter.cpp:73-91 */
static int vertex_push_basic(const Cutter* c, const Fib* f, Ival* i, const Tri* t) {
    int result = 0;
    for (int k = 0; k < 3; ++k)
        if (single_vertex_push(c, f, i, t->p[k], OCL_CC_VERTEX)) result = 1;
    if (c->kind == OCL_CUTTER_CYL) {
        P3 p1, p2;
        if (zslice_verts(t, &p1, &p2, f->p1.z)) {
            p1.z = f->p1.z;
            p2.z = f->p1.z;
            if (single_vertex_push(c, f, i, p1, OCL_CC_VERTEX_CYL)) result = 1;
            if (single_vertex_push(c, f, i, p2, OCL_CC_VERTEX_CYL)) result = 1;
        }
    }
    return result;
}

/* MillingCutter::generalFacetPush millingcutter.cpp:177-275 */
static int general_facet_push(double normal_length, double center_height, double xy_normal_length,
                              const Fib* fib, Ival* i, const Tri* t) {
    P3 normal = up_normal(t);
    if (normal.x == 0.0 && normal.y == 0.0) return 0; /* Point::zParallel point.cpp:315-322 */
    normal = pnormalize(normal);
    P3 xy_normal = normal;
    xy_normal.z = 0;
    xy_normal = pxynormalize(xy_normal);
    double a, b, e, u, v;
    double c = t->p[1].z - t->p[0].z;
    double d = t->p[2].z - t->p[0].z;
    double f = -t->p[0].z - normal_length * normal.z + fib->p1.z + center_height;
    if (fib->p1.y == fib->p2.y) {
        a = t->p[1].y - t->p[0].y;
        b = t->p[2].y - t->p[0].y;
        e = -t->p[0].y - normal_length * normal.y - xy_normal_length * xy_normal.y + fib->p1.y;
        if (!two_by_two(a, b, c, d, e, f, &u, &v)) return 0;
        CC cc;
        cc.p = padd(padd(t->p[0], pmul(u, psub(t->p[1], t->p[0]))), pmul(v, psub(t->p[2], t->p[0])));
        cc.type = OCL_CC_FACET;
        if (!inside_tri(cc.p, t->p)) return 0;
        double tval = (1.0 / (fib->p2.x - fib->p1.x)) *
                      (t->p[0].x + normal_length * normal.x + xy_normal_length * xy_normal.x -
                       fib->p1.x + u * (t->p[1].x - t->p[0].x) + v * (t->p[2].x - t->p[0].x));
        iv_update(i, tval, cc);
        return 1;
    } else if (fib->p1.x == fib->p2.x) {
        a = t->p[1].x - t->p[0].x;
        b = t->p[2].x - t->p[0].x;
        e = -t->p[0].x - normal_length * normal.x - xy_normal_length * xy_normal.x + fib->p1.x;
        if (!two_by_two(a, b, c, d, e, f, &u, &v)) return 0;
        CC cc;
        cc.p = padd(padd(t->p[0], pmul(u, psub(t->p[1], t->p[0]))), pmul(v, psub(t->p[2], t->p[0])));
        cc.type = OCL_CC_FACET;
        if (!inside_tri(cc.p, t->p)) return 0;
        double tval = (1.0 / (fib->p2.y - fib->p1.y)) *
                      (t->p[0].y + normal_length * normal.y + xy_normal_length * xy_normal.y -
                       fib->p1.y + u * (t->p[1].y - t->p[0].y) + v * (t->p[2].y - t->p[0].y));
        iv_update(i, tval, cc);
        return 1;
    }
    return 0;
}

/* facetPush: MillingCutter::facetPush millingcutter.cpp:169-174, ConeCutter::facetPush conecutter.cpp:137-147 */
static int facet_push_basic(const Cutter* c, const Fib* f, Ival* i, const Tri* t) {
    if (c->kind == OCL_CUTTER_CONE) {
        int result = 0;
        if (general_facet_push(0, 0, 0, f, i, t)) result = 1;
        if (general_facet_push(0, c->center_height, c->xy_normal_length, f, i, t)) result = 1;
        return result;
    }
    return general_facet_push(c->normal_length, c->center_height, c->xy_normal_length, f, i, t);
}

/* MillingCutter::calcCCandUpdateInterval millingcutter.cpp:370-375 */
static int calc_cc_update(double t, double u, P3 q, P3 p1, P3 p2, const Fib* f, Ival* i,
                          double height, int type) {
    CC cc;
    cc.p = padd(q, pmul(u, psub(p2, p1)));
    cc.type = type;
    (void)f;
    return iv_update_if(i, t, cc, p1, p2, (cc.p.z >= height));
}

/* MillingCutter::horizEdgePush millingcutter.cpp:335-368 */
static int horiz_edge_push(const Cutter* c, const Fib* f, Ival* i, P3 p1, P3 p2) {
    int result = 0;
    double h = p1.z - f->p1.z;
    if (h > 0.0) {
        if (iszero_tol(p2.z - p1.z)) {
            double eff = c_width(c, h);
            double qt, qv;
            if (xy_line_line(p1, p2, &qv, f->p1, f->p2, &qt)) {
                P3 q = padd(p1, pmul(qv, psub(p2, p1)));
                double ccv, clt;
                P3 tang = psub(p2, p1);
                tang.z = 0;
                tang = pxynormalize(tang);
                P3 xyn = pxyperp(tang);
                P3 q1 = padd(q, pmul(eff, xyn));
                P3 q2 = padd(q1, psub(p2, p1));
                if (xy_line_line(q1, q2, &ccv, f->p1, f->p2, &clt)) {
                    double t1 = clt;
                    double t2 = qt + (qt - clt);
                    if (calc_cc_update(t1, ccv, q, p1, p2, f, i, f->p1.z, OCL_CC_EDGE_HORIZ)) result = 1;
                    if (calc_cc_update(t2, -ccv, q, p1, p2, f, i, f->p1.z, OCL_CC_EDGE_HORIZ)) result = 1;
                }
            }
        }
    }
    return result;
}

/* MillingCutter::shaftEdgePush millingcutter.cpp:304-332 */
static int shaft_edge_push(const Cutter* c, const Fib* f, Ival* i, P3 p1, P3 p2) {
    double u, v;
    int result = 0;
    if (xy_line_line(p1, p2, &u, f->p1, f->p2, &v)) {
        P3 q = padd(p1, pmul(u, psub(p2, p1)));
        P3 tang = psub(p2, p1);
        tang.z = 0;
        tang = pxynormalize(tang);
        P3 xyn = pxyperp(tang);
        P3 q1 = padd(q, pmul(c->radius, xyn));
        P3 q2 = padd(q1, psub(p2, p1));
        double u_cc, t_cl;
        if (xy_line_line(q1, q2, &u_cc, f->p1, f->p2, &t_cl)) {
            double t1 = t_cl;
            double t2 = v + (v - t_cl);
            if (calc_cc_update(t1, u_cc, q, p1, p2, f, i, f->p1.z + c->center_height, OCL_CC_EDGE_SHAFT)) result = 1;
            if (calc_cc_update(t2, -u_cc, q, p1, p2, f, i, f->p1.z + c->center_height, OCL_CC_EDGE_SHAFT)) result = 1;
        }
    }
    return result;
}

/* BallCutter::calcCCandUpdateInterval ballcutter.cpp:109-116 */
static int ball_cc_update(const Cutter* c, double t, P3 p1, P3 p2, const Fib* f, Ival* i) {
    P3 center = padd(f_point(f, t), pt(0, 0, c->radius));
    CC cc;
    cc.p = closest_point(center, p1, p2);
    cc.type = OCL_CC_EDGE_BALL;
    return iv_update_if(i, t, cc, p1, p2, (center.z - cc.p.z >= 0));
}

/* BallCutter::generalEdgePush ballcutter.cpp:66-106 */
static int ball_edge_push(const Cutter* c, const Fib* f, Ival* i, P3 p1, P3 p2) {
    int result = 0;
    if (iszero_tol(pxynorm(psub(p2, p1)))) return 0;
    P3 ufp1 = padd(f->p1, pt(0, 0, c->radius));
    P3 ufp2 = padd(f->p2, pt(0, 0, c->radius));
    P3 ab = psub(p2, p1);
    P3 ao = psub(ufp1, p1);
    P3 ao_x_ab = pcross(ao, ab);
    P3 v_x_ab = pcross(psub(ufp2, ufp1), ab);
    double ab2 = pdot(ab, ab);
    double a = pdot(v_x_ab, v_x_ab);
    double b = 2 * (pdot(v_x_ab, ao_x_ab));
    double cc = pdot(ao_x_ab, ao_x_ab) - (c->radius * c->radius * ab2);
    double discr = b * b - 4 * a * cc;
    if (iszero_tol(discr)) {
        double t1 = -b / (2 * a);
        if (ball_cc_update(c, t1, p1, p2, f, i)) result = 1;
    } else if (discr > 0.0) {
        double t1 = (-b + sqrt(discr)) / (2 * a);
        double t2 = (-b - sqrt(discr)) / (2 * a);
        if (ball_cc_update(c, t1, p1, p2, f, i)) result = 1;
        if (ball_cc_update(c, t2, p1, p2, f, i)) result = 1;
    }
    return result;
}

/* AlignedEllipse::aligned_solver ellipse.cpp:212-309 */
static int aligned_solver(Ell* E, const Fib* f, int* capped) {
    E->error_dir = pxyperp(f->dir);
    E->target = f->p1;
    double t1 = 0.0;
    if (f->p1.y == f->p2.y)
        t1 = sqrt(sq(E->b * E->minor_dir.y) / (sq(E->a * E->major_dir.y) + sq(E->b * E->minor_dir.y)));
    else if (f->p1.x == f->p2.x)
        t1 = sqrt(sq(E->b * E->minor_dir.x) / (sq(E->a * E->major_dir.x) + sq(E->b * E->minor_dir.x)));
    EPos tmp, apos, bpos;
    apos = epos_dia(0.0);
    bpos = epos_dia(0.0);
    double s1 = sqrt(1.0 - sq(t1));
    int fpos = 0, fneg = 0;
    /* probe order of the reference: (s1,t1), (s1,-t1), (-s1,t1), (-s1,-t1) */
    const double sg[4][2] = {{1, 1}, {1, -1}, {-1, 1}, {-1, -1}};
    for (int k = 0; k < 4; ++k) {
        double xs = sg[k][0] > 0 ? s1 : -s1;
        double ys = sg[k][1] > 0 ? t1 : -t1;
        tmp = epos_dia(xy_to_diangle(xs, ys));
        double err = ell_error(E, tmp.diangle);
        if (err > 0) { fpos = 1; apos = tmp; }
        else if (err < 0) { fneg = 1; bpos = tmp; }
    }
    if (fpos && fneg) {
        double lolim = 0.0, hilim = 0.0;
        if (apos.diangle > bpos.diangle) { lolim = bpos.diangle; hilim = apos.diangle; }
        else if (bpos.diangle > apos.diangle) { hilim = bpos.diangle; lolim = apos.diangle; }
        double s1_ = brent_zero(lolim, hilim, 3E-16, OE_TOL, E, capped);
        double s2_ = brent_zero(hilim - 4.0, lolim, 3E-16, OE_TOL, E, capped);
        E->e1 = epos_dia(s1_);
        E->e2 = epos_dia(s2_);
        return 1;
    }
    return 0;
}

/* BullCutter::generalEdgePush bullcutter.cpp:109-155 */
static int bull_edge_push(const Cutter* c, const Fib* f, Ival* i, P3 p1, P3 p2, Ctx* ctx) {
    int result = 0;
    if (iszero_tol(pxynorm(psub(p2, p1)))) return 0;
    if (iszero_tol(p2.z - p1.z)) return 0;
    double tplane = (f->p1.z + c->radius2 - p1.z) / (p2.z - p1.z);
    P3 ell_center = padd(p1, pmul(tplane, psub(p2, p1)));
    P3 major_dir = psub(p2, p1);
    major_dir.z = 0;
    major_dir = pxynormalize(major_dir);
    P3 minor_dir = pxyperp(major_dir);
    double theta = atan((p2.z - p1.z) / pxynorm(psub(p2, p1)));
    double major_length = fabs(c->radius2 / sin(theta));
    double minor_length = c->radius2;
    Ell E;
    memset(&E, 0, sizeof(E));
    E.aligned = 1;
    E.center = ell_center;
    E.a = major_length;
    E.b = minor_length;
    E.offset = c->radius1;
    E.major_dir = major_dir;
    E.minor_dir = minor_dir;
    if (aligned_solver(&E, f, &ctx->capped)) {
        P3 pcc = ell_epoint(&E, E.e1);
        P3 pcc2 = ell_epoint(&E, E.e2);
        CC cc, cc2;
        cc.p = closest_point(pcc, p1, p2);
        cc2.p = closest_point(pcc2, p1, p2);
        cc.type = OCL_CC_EDGE_POS;
        cc2.type = OCL_CC_EDGE_POS;
        P3 cl = psub(ell_oepoint(&E, E.e1), pt(0, 0, c->center_height));
        P3 cl2 = psub(ell_oepoint(&E, E.e2), pt(0, 0, c->center_height));
        double cl_t = f_tval(f, cl);
        double cl_t2 = f_tval(f, cl2);
        if (iv_update_if(i, cl_t, cc, p1, p2, 1)) result = 1;
        if (iv_update_if(i, cl_t2, cc2, p1, p2, 1)) result = 1;
    }
    return result;
}

/* ConeCutter::circle_CC conecutter.cpp:293-300 */
static int cone_circle_cc(const Cutter* c, double t, P3 p1, P3 p2, const Fib* f, Ival* i) {
    double t_cc = (f->p1.z + c->center_height - p1.z) / (p2.z - p1.z);
    CC cc;
    cc.p = padd(p1, pmul(t_cc, psub(p2, p1)));
    cc.type = OCL_CC_EDGE_CONE_BASE;
    return iv_update_if(i, t, cc, p1, p2, 1);
}
/* ConeCutter::cone_CC conecutter.cpp:270-288 */
static int cone_cone_cc(P3 tang, P3 tip, P3 base, P3 p1, P3 p2, const Fib* f, Ival* i) {
    double u, t;
    if (xy_line_line(f->p1, f->p2, &u, tang, tip, &t)) {
        if ((t >= 0.0) && (t <= 1.0)) {
            CC cc;
            cc.p = padd(base, pmul(t, psub(tip, base)));
            cc.p.z = z_project(cc.p, p1, p2);
            cc.type = OCL_CC_EDGE_CONE;
            return iv_update_if(i, u, cc, p1, p2, 1);
        }
    }
    return 0;
}

/* ConeCutter::generalEdgePush conecutter.cpp:150-268 */
static int cone_edge_push(const Cutter* c, const Fib* f, Ival* i, P3 p1, P3 p2) {
    int result = 0;
    if (iszero_tol(p2.z - p1.z)) return 0;
    double t_tip = (f->p1.z - p1.z) / (p2.z - p1.z);
    P3 p_tip = padd(p1, pmul(t_tip, psub(p2, p1)));
    double t_base = (f->p1.z + c->center_height - p1.z) / (p2.z - p1.z);
    P3 p_base = padd(p1, pmul(t_base, psub(p2, p1)));
    p_base.z = f->p1.z;
    double L = pxynorm(psub(p_base, p_tip));
    double d = xy_distance_to_line(p_base, f->p1, f->p2);
    if (d <= c->radius) {
        double dx = f->p2.x - f->p1.x;
        double dy = f->p2.y - f->p1.y;
        double dr = sqrt(sq(dx) + sq(dy));
        double det = (f->p1.x - p_base.x) * (f->p2.y - p_base.y) - (f->p2.x - p_base.x) * (f->p1.y - p_base.y);
        double discr = sq(c->radius) * sq(dr) - sq(det);
        if (discr >= 0.0) {
            if (discr == 0.0) {
                double x_tang = (det * dy) / sq(dr);
                double y_tang = -(det * dx) / sq(dr);
                P3 p_tang = pt(x_tang + p_base.x, y_tang + p_base.y, 0);
                double t_tang = f_tval(f, p_tang);
                if (cone_circle_cc(c, t_tang, p1, p2, f, i)) result = 1;
            } else {
                double x_pos = (det * dy + sgn(dy) * dx * sqrt(discr)) / sq(dr);
                double y_pos = (-det * dx + fabs(dy) * sqrt(discr)) / sq(dr);
                P3 cl_pos = pt(x_pos + p_base.x, y_pos + p_base.y, 0);
                double t_pos = f_tval(f, cl_pos);
                double x_neg = (det * dy - sgn(dy) * dx * sqrt(discr)) / sq(dr);
                double y_neg = (-det * dx - fabs(dy) * sqrt(discr)) / sq(dr);
                P3 cl_neg = pt(x_neg + p_base.x, y_neg + p_base.y, 0);
                double t_neg = f_tval(f, cl_neg);
                if (cone_circle_cc(c, t_pos, p1, p2, f, i)) result = 1;
                if (cone_circle_cc(c, t_neg, p1, p2, f, i)) result = 1;
            }
        }
    }
    if (L > c->radius) {
        P3 p_mid = pmul(0.5, padd(p_base, p_tip));
        p_mid.z = f->p1.z;
        double r_tang = L / 2;
        P3 pd = psub(p_mid, p_base);
        pd.z = 0;
        double dist = pxynorm(pd);
        int case1 = (iszero_tol(dist) && iszero_tol(fabs(c->radius - r_tang)));
        int case2 = (dist > (c->radius + r_tang));
        int case3 = (dist < fabs(c->radius - r_tang));
        int case4 = (iszero_tol(dist - (c->radius + r_tang)));
        if (!(case1 || case2 || case3 || case4)) {
            double a = (-sq(r_tang) + sq(c->radius) + sq(dist)) / (2.0 * dist);
            P3 v2 = padd(p_base, pmul(a / dist, pd));
            double h = sqrt(sq(c->radius) - sq(a));
            P3 ofs = pt(-pd.y * (h / dist), pd.x * (h / dist), 0);
            P3 tang1 = padd(v2, ofs);
            P3 tang2 = psub(v2, ofs);
            if (cone_cone_cc(tang1, p_tip, p_base, p1, p2, f, i)) result = 1;
            if (cone_cone_cc(tang2, p_tip, p_base, p1, p2, f, i)) result = 1;
        }
    }
    return result;
}

/* MillingCutter::edgePush / singleEdgePush millingcutter.cpp:277-301 */
static int edge_push_basic(const Cutter* c, const Fib* f, Ival* i, const Tri* t, Ctx* ctx) {
    int result = 0;
    for (int n = 0; n < 3; ++n) {
        P3 p1 = t->p[n], p2 = t->p[(n + 1) % 3];
        int r = 0;
        if (horiz_edge_push(c, f, i, p1, p2)) r = 1;
        else {
            if (shaft_edge_push(c, f, i, p1, p2)) r = 1;
            int g = 0;
            if (c->kind == OCL_CUTTER_BALL) g = ball_edge_push(c, f, i, p1, p2);
            else if (c->kind == OCL_CUTTER_BULL) g = bull_edge_push(c, f, i, p1, p2, ctx);
            else if (c->kind == OCL_CUTTER_CONE) g = cone_edge_push(c, f, i, p1, p2);
            if (g) r = 1;
        }
        if (r) result = 1;
    }
    return result;
}

/* CompositeCutter::vertexPush / facetPush / edgePush compositecutter.cpp:196-270 */
static int comp_push(const Cutter* c, const Fib* f, Ival* i, const Tri* t, int which, Ctx* ctx) {
    struct { double t; CC cc; } contacts[2 * OCL_GB300_MAX_SUB];
    int nc = 0;
    for (int n = 0; n < c->nsub; ++n) {
        Ival ci;
        iv_init(&ci);
        Fib cf = *f;
        cf.p1.z = f->p1.z + c->zoffset[n];
        cf.p2.z = f->p2.z + c->zoffset[n];
        const Cutter* s = &c->sub[n];
        int hit;
        if (which == 0) hit = vertex_push_basic(s, &cf, &ci, t);
        else if (which == 1) hit = facet_push_basic(s, &cf, &ci, t);
        else hit = edge_push_basic(s, &cf, &ci, t, ctx);
        if (hit) {
            /* ccValidHeight compositecutter.cpp:104-110 */
            if (n == height_to_index(c, ci.ucc.p.z - f->p1.z)) {
                contacts[nc].t = ci.upper; contacts[nc].cc = ci.ucc; ++nc;
            }
            if (n == height_to_index(c, ci.lcc.p.z - f->p1.z)) {
                contacts[nc].t = ci.lower; contacts[nc].cc = ci.lcc; ++nc;
            }
        }
    }
    for (int k = 0; k < nc; ++k) iv_update(i, contacts[k].t, contacts[k].cc);
    return nc > 0;
}

/* MillingCutter::pushCutter millingcutter.cpp:377-382 */
static void push_cutter(const Cutter* c, const Fib* f, Ival* i, const Tri* t, Ctx* ctx) {
    if (c->kind == OCL_CUTTER_COMPOSITE) {
        comp_push(c, f, i, t, 0, ctx);
        comp_push(c, f, i, t, 1, ctx);
        comp_push(c, f, i, t, 2, ctx);
        return;
    }
    vertex_push_basic(c, f, i, t);
    facet_push_basic(c, f, i, t);
    edge_push_basic(c, f, i, t, ctx);
}

typedef struct { Ival* v; long n, cap; } IVec;
static void ivv_push(IVec* a, Ival x) {
    if (a->n == a->cap) {
        a->cap = a->cap ? 2 * a->cap : 8;
        a->v = (Ival*)realloc(a->v, sizeof(Ival) * a->cap);
    }
    a->v[a->n++] = x;
}
/* Interval::outside / inside / empty interval.cpp:96-118 */
static inline int iv_outside(const Ival* me, const Ival* i) {
    if (me->lower > i->upper) return 1;
    else if (me->upper < i->lower) return 1;
    return 0;
}
static inline int iv_inside(const Ival* me, const Ival* i) {
    return (me->lower > i->lower) && (me->upper < i->upper);
}
static inline int iv_empty(const Ival* i) { return i->lower == 0.0 && i->upper == 0.0; }

/* Fiber::addInterval fiber.cpp:58-93 */
static void fiber_add(IVec* ints, Ival* i, IVec* scratch) {
    if (iv_empty(i)) return;
    if (ints->n == 0) { ivv_push(ints, *i); return; }
    for (long k = 0; k < ints->n; ++k)
        if (iv_inside(i, &ints->v[k])) return;
    int missing = 1;
    for (long k = 0; k < ints->n; ++k)
        if (!iv_outside(i, &ints->v[k])) missing = 0;
    if (missing) { ivv_push(ints, *i); return; }
    scratch->n = 0;
    long w = 0;
    for (long k = 0; k < ints->n; ++k) {
        if (!iv_outside(&ints->v[k], i)) ivv_push(scratch, ints->v[k]);
        else ints->v[w++] = ints->v[k];
    }
    ints->n = w;
    ivv_push(scratch, *i);
    Ival sum;
    iv_init(&sum);
    for (long k = 0; k < scratch->n; ++k) {
        iv_lower(&sum, scratch->v[k].lower, scratch->v[k].lcc);
        iv_upper(&sum, scratch->v[k].upper, scratch->v[k].ucc);
    }
    ivv_push(ints, sum);
}

long oracle_push(const double* tris, long ntri, const ocl_gb300_cutter* cd, int dir,
                 const double* fib, long F, int nthreads, unsigned bucket, int32_t* counts,
                 double* ival, double* cc, int32_t* cctype, long cap, long* ncalls) {
    Scene S;
    int st = scene_init(&S, tris, ntri, cd, bucket, dir == OCL_GB300_XFIBER ? 1 : 2);
    if (st) return -st;
    IVec* res = (IVec*)calloc(F > 0 ? F : 1, sizeof(IVec));
    long calls = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel reduction(+ : calls)
    {
        LVec buf = {0, 0, 0};
        IVec scratch = {0, 0, 0};
        Ctx ctx = {0};
#pragma omp for schedule(dynamic, 4)
        for (long n = 0; n < F; ++n) {
            Fib f;
            f.p1 = pt(fib[6 * n], fib[6 * n + 1], fib[6 * n + 2]);
            f.p2 = pt(fib[6 * n + 3], fib[6 * n + 4], fib[6 * n + 5]);
            f.dir = pnormalize(psub(f.p2, f.p1)); /* Fiber::calcDir fiber.cpp:35-39 */
            /* BatchPushCutter::pushCutter3 batchpushcutter.cpp:136-188 */
            CL cl;
            if (dir == OCL_GB300_XFIBER) { cl.x = 0; cl.y = f.p1.y; cl.z = f.p1.z; }
            else { cl.x = f.p1.x; cl.y = 0; cl.z = f.p1.z; }
            double r = S.cutter.radius;
            double bb[6] = {cl.x - r, cl.x + r, cl.y - r, cl.y + r, cl.z, cl.z + S.cutter.length};
            buf.n = 0;
            if (S.ntri > 0) kd_search(&S.kd, 0, bb, &buf);
            for (long k = 0; k < buf.n; ++k) {
                Ival i;
                iv_init(&i);
                push_cutter(&S.cutter, &f, &i, &S.tris[buf.v[k]], &ctx);
                fiber_add(&res[n], &i, &scratch);
                ++calls;
            }
        }
        free(buf.v);
        free(scratch.v);
    }
    long total = 0;
    for (long n = 0; n < F; ++n) {
        counts[n] = (int32_t)res[n].n;
        for (long k = 0; k < res[n].n; ++k) {
            if (total < cap) {
                const Ival* iv = &res[n].v[k];
                ival[2 * total] = iv->lower;
                ival[2 * total + 1] = iv->upper;
                double* o = cc + 6 * total;
                o[0] = iv->lcc.p.x; o[1] = iv->lcc.p.y; o[2] = iv->lcc.p.z;
                o[3] = iv->ucc.p.x; o[4] = iv->ucc.p.y; o[5] = iv->ucc.p.z;
                cctype[2 * total] = iv->lcc.type;
                cctype[2 * total + 1] = iv->ucc.type;
            }
            ++total;
        }
        free(res[n].v);
    }
    free(res);
    if (ncalls) *ncalls = calls;
    scene_free(&S);
    return total;
}

/* ------------------------------------------------------------------ */
/* Paths (geo/line.cpp, geo/arc.cpp, dropcutter/pathdropcutter.cpp,    */
/* dropcutter/adaptivepathdropcutter.cpp)                              */
/* ------------------------------------------------------------------ */
typedef struct {
    int type;
    P3 p1, p2, c;
    int dir;
    double radius, length;
} Span;

/* Arc::xyIncludedAngle arc.cpp:73-94 */
static double xy_included_angle(P3 v1, P3 v2, int dir) {
    int d = dir ? 1 : (-1);
    double inc = pdot(v1, v2);
    if (inc > 1. - 1.0e-10) return 0;
    if (inc < -1. + 1.0e-10)
        inc = PI_REF;
    else {
        if (inc > 1.0) inc = 1.0;
        inc = acos(inc);
        double x = v1.x * v2.y - v1.y * v2.x;
        if (d * x < 0) inc = 2 * PI_REF - inc;
    }
    return d * inc;
}

static void span_init(Span* s, const double* v) {
    s->type = (int)v[0];
    s->p1 = pt(v[1], v[2], v[3]);
    s->p2 = pt(v[4], v[5], v[6]);
    s->c = pt(v[7], v[8], v[9]);
    s->dir = v[10] != 0.0;
    if (s->type == 1) {
        /* Arc::setProperties arc.cpp:43-51 */
        P3 vs = pxyperp(psub(s->p1, s->c));
        P3 ve = pxyperp(psub(s->p2, s->c));
        s->radius = pxynorm(vs);
        vs = pnormalize(vs);
        ve = pnormalize(ve);
        s->length = fabs(xy_included_angle(vs, ve, s->dir)) * s->radius;
    } else {
        s->length = pxynorm(psub(s->p2, s->p1)); /* Line::length2d line.cpp:40-42 */
    }
}

/* Line::getPoint line.cpp:44-46, Arc::getPoint arc.cpp:53-71 */
static P3 span_point(const Span* s, double t) {
    if (s->type == 0) return padd(pmul(t, psub(s->p2, s->p1)), s->p1);
    if (fabs(t) < 0.00000000000001) return s->p1;
    if (fabs(t - 1.0) < 0.00000000000001) return s->p2;
    double d = t * s->length;
    if (!s->dir) d = -d;
    P3 v = psub(s->p1, s->c);
    double a = d / s->radius;
    double cosa = cos(a), sina = sin(a);
    double temp = -v.y * sina + v.x * cosa; /* Point::xyRotate point.cpp:85-89 */
    v.y = v.x * sina + cosa * v.y;
    v.x = temp;
    return padd(v, s->c);
}

long oracle_pdc(const double* tris, long ntri, const ocl_gb300_cutter* cd, const double* spans,
                long S_, double sampling, double minz, int nthreads, unsigned bucket, double* xyz,
                double* cc, int32_t* type, long cap) {
    /* PathDropCutter::sample_span pathdropcutter.cpp:69-80 */
    long n = 0;
    for (long k = 0; k < S_; ++k) {
        Span s;
        span_init(&s, spans + OCL_GB300_SPAN_DOUBLES * k);
        unsigned int num_steps = (unsigned int)(s.length / sampling + 1);
        n += (long)num_steps + 1;
    }
    double* cl = (double*)malloc(sizeof(double) * 3 * (n > 0 ? n : 1));
    long w = 0;
    for (long k = 0; k < S_; ++k) {
        Span s;
        span_init(&s, spans + OCL_GB300_SPAN_DOUBLES * k);
        unsigned int num_steps = (unsigned int)(s.length / sampling + 1);
        for (unsigned int i = 0; i <= num_steps; i++) {
            double fraction = (double)i / num_steps;
            P3 p = span_point(&s, fraction);
            cl[3 * w] = p.x;
            cl[3 * w + 1] = p.y;
            cl[3 * w + 2] = minz;
            ++w;
        }
    }
    if (n <= cap) {
        double* z = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
        int st = oracle_drop(tris, ntri, cd, cl, n, nthreads, bucket, z, cc, type, NULL);
        if (st) { free(z); free(cl); return -st; }
        for (long i = 0; i < n; ++i) {
            xyz[3 * i] = cl[3 * i];
            xyz[3 * i + 1] = cl[3 * i + 1];
            xyz[3 * i + 2] = z[i];
        }
        free(z);
    }
    free(cl);
    return n;
}

typedef struct {
    const Scene* S;
    const Span* span;
    double sampling, min_sampling, cos_limit;
    double* xyz; double* cc; int32_t* type;
    long n, cap;
    LVec buf;
    Ctx ctx;
} APDC;

static void apdc_emit(APDC* A, const CL* cl) {
    if (A->n < A->cap) {
        A->xyz[3 * A->n] = cl->x; A->xyz[3 * A->n + 1] = cl->y; A->xyz[3 * A->n + 2] = cl->z;
        A->cc[3 * A->n] = cl->cc.p.x; A->cc[3 * A->n + 1] = cl->cc.p.y; A->cc[3 * A->n + 2] = cl->cc.p.z;
        A->type[A->n] = cl->cc.type;
    }
    A->n++;
}

static CL cl_from(P3 p) {
    CL c;
    c.x = p.x; c.y = p.y; c.z = p.z;
    c.cc.p = pt(0, 0, 0);
    c.cc.type = OCL_CC_NONE;
    return c;
}

/* AdaptivePathDropCutter::flat adaptivepathdropcutter.cpp:88-94 */
static int apdc_flat(const APDC* A, const CL* s, const CL* m, const CL* e) {
    P3 v1 = pnormalize(psub(clp(m), clp(s)));
    P3 v2 = pnormalize(psub(clp(e), clp(m)));
    return pdot(v1, v2) > A->cos_limit;
}

/* AdaptivePathDropCutter::adaptive_sample adaptivepathdropcutter.cpp:72-86 */
static void apdc_sample(APDC* A, double start_t, double stop_t, CL start_cl, CL stop_cl, int depth) {
    double mid_t = start_t + (stop_t - start_t) / 2.0;
    CL mid = cl_from(span_point(A->span, mid_t));
    point_drop(A->S, &mid, &A->buf, &A->ctx);
    double fw_step = pxynorm(psub(clp(&stop_cl), clp(&start_cl)));
    if (depth < 60 && ((fw_step > A->sampling) ||
                       ((!apdc_flat(A, &start_cl, &mid, &stop_cl)) && (fw_step > A->min_sampling)))) {
        apdc_sample(A, start_t, mid_t, start_cl, mid, depth + 1);
        apdc_sample(A, mid_t, stop_t, mid, stop_cl, depth + 1);
    } else {
        apdc_emit(A, &stop_cl);
    }
}

long oracle_apdc(const double* tris, long ntri, const ocl_gb300_cutter* cd, const double* spans,
                 long S_, double sampling, double min_sampling, double cos_limit, unsigned bucket,
                 double* xyz, double* cc, int32_t* type, long cap) {
    Scene S;
    int st = scene_init(&S, tris, ntri, cd, bucket, 0);
    if (st) return -st;
    APDC A;
    memset(&A, 0, sizeof(A));
    A.S = &S;
    A.sampling = sampling;
    A.min_sampling = min_sampling;
    A.cos_limit = cos_limit;
    A.xyz = xyz; A.cc = cc; A.type = type; A.cap = cap;
    /* AdaptivePathDropCutter::adaptive_sampling_run adaptivepathdropcutter.cpp:57-70 */
    for (long k = 0; k < S_; ++k) {
        Span s;
        span_init(&s, spans + OCL_GB300_SPAN_DOUBLES * k);
        A.span = &s;
        CL start = cl_from(span_point(&s, 0.0));
        CL stop = cl_from(span_point(&s, 1.0));
        point_drop(&S, &start, &A.buf, &A.ctx);
        point_drop(&S, &stop, &A.buf, &A.ctx);
        apdc_emit(&A, &start);
        apdc_sample(&A, 0.0, 1.0, start, stop, 0);
    }
    free(A.buf.v);
    scene_free(&S);
    return A.n;
}

/* Derived cutter fields, laid out like ref_preset_fields: [radius, length,
 * diameter, nsub, per sub: diameter, radius, length, center_height,
 * xy_normal_length, normal_length, radiusvec, heightvec, zoffset]. */
int oracle_cutter_fields(const ocl_gb300_cutter* cd, double* out) {
    Cutter c;
    if (cutter_make(&c, cd) != 0) return -1;
    out[0] = c.radius; out[1] = c.length; out[2] = c.diameter; out[3] = c.nsub;
    if (c.nsub == 0) {  /* a basic cutter: its own derived fields */
        out[4] = c.diameter; out[5] = c.radius; out[6] = c.length; out[7] = c.center_height;
        out[8] = c.xy_normal_length; out[9] = c.normal_length;
    }
    for (int n = 0; n < c.nsub; ++n) {
        double* o = out + 4 + 9 * n;
        const Cutter* s = &c.sub[n];
        o[0] = s->diameter; o[1] = s->radius; o[2] = s->length; o[3] = s->center_height;
        o[4] = s->xy_normal_length; o[5] = s->normal_length;
        o[6] = c.radiusvec[n]; o[7] = c.heightvec[n]; o[8] = c.zoffset[n];
    }
    cutter_free(&c);
    return 0;
}
