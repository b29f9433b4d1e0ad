// geom64.cuh -- FP64 cutter/triangle contact, device side.
//
// This is the exact evaluation used by the plain FP64 drop kernel and by the
// refinement stage of the mixed-precision kernel.  It follows the reference's
// per-triangle drop semantics (paths relative to opencamlib's src/):
//   MillingCutter::dropCutter  cutters/millingcutter.cpp:386-409
//   facetDrop  millingcutter.cpp:51-75, ConeCutter conecutter.cpp:70-105,
//              CompositeCutter compositecutter.cpp:152-172
//   vertexDrop millingcutter.cpp:36-47
//   edgeDrop   millingcutter.cpp:79-136 + singleEdgeDropCanonical of each
//              cutter (cyl :52-70, ball :50-63, bull :82-105 with the
//              offset-ellipse Brent solve ellipse.cpp:118-208, cone :109-135)
// keeping the operation order, so that a translation unit compiled with
// --fmad=false produces the same doubles as the CPU reference.
//
// Each triangle is evaluated on its own, starting from the CL point's input
// z (the reference evaluates triangles one after another against a running
// z; the maxima agree, and exact ties are broken by the KD visit order).
#pragma once
#include "common.cuh"

namespace oclg {

#define OCLG_TOL 0.0000001
#define OCLG_OE_TOL 1e-10
#define OCLG_BRENT_CAP 200

struct D3 {
    double x, y, z;
};
__device__ __forceinline__ D3 d3(double x, double y, double z) { return D3{x, y, z}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ D3 operator*(double s, D3 a) { return d3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ double sq(double x) { return x * x; }
__device__ __forceinline__ double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double norm3(D3 a) { return sqrt(sq(a.x) + sq(a.y) + sq(a.z)); }
__device__ __forceinline__ double xynorm(D3 a) { return sqrt(sq(a.x) + sq(a.y)); }
__device__ __forceinline__ D3 normalize3(D3 a) {
    double n = norm3(a);
    if (n != 0.0) a = (1 / n) * a;
    return a;
}
__device__ __forceinline__ D3 xynormalize(D3 a) {
    if (xynorm(a) != 0.0) a = (1 / xynorm(a)) * a;
    return a;
}
__device__ __forceinline__ bool zero_tol(double x) { return fabs(x) < OCLG_TOL; }
__device__ __forceinline__ double sgn(double x) { return x < 0.0 ? -1.0 : 1.0; }

// Point::xyDistanceToLine (geo/point.cpp:139-156)
__device__ __forceinline__ double xy_dist_line(D3 me, D3 p1, D3 p2) {
    if (p1.x == p2.x && p1.y == p2.y) return -1;
    D3 v = normalize3(d3(p2.y - p1.y, -(p2.x - p1.x), 0));
    D3 r = d3(p1.x - me.x, p1.y - me.y, 0);
    return fabs(dot(v, r));
}
// Point::closestPoint (point.cpp:159-165)
__device__ __forceinline__ D3 closest_point(D3 me, D3 p1, D3 p2) {
    D3 v = p2 - p1;
    double u = dot(me - p1, v) / dot(v, v);
    return p1 + u * v;
}
// Point::xyClosestPoint (point.cpp:168-193)
__device__ __forceinline__ D3 xy_closest(D3 me, D3 p1, D3 p2) {
    D3 v = p2 - p1;
    double u = (me.x - p1.x) * (v.x) + (me.y - p1.y) * (v.y);
    u = u / (v.x * v.x + v.y * v.y);
    return d3(p1.x + u * v.x, p1.y + u * v.y, 0);
}
// Point::isInside(Triangle) (point.cpp:224-239)
__device__ __forceinline__ bool in_tri(D3 p, const double* t) {
    double ax = t[0], ay = t[1], bx = t[3], by = t[4], cx = t[6], cy = t[7];
    double u = (ay * cx - ax * cy + (cy - ay) * p.x + (ax - cx) * p.y) /
               (ay * cx - ax * cy + (cy - ay) * bx + (ax - cx) * by);
    double v = (ax * by - ay * bx + (ay - by) * p.x + (bx - ax) * p.y) /
               (ax * by - ay * bx + (ay - by) * cx + (bx - ax) * cy);
    return u > 0.0 && v > 0.0 && (u + v) < 1.0;
}
// Point::isInside(p1,p2) (point.cpp:241-253)
__device__ __forceinline__ bool in_seg(D3 me, D3 p1, D3 p2) {
    D3 d = p2 - p1;
    double t = dot(me - p1, d) / dot(d, d);
    return !(t > 1.0 || t < 0.0);
}
// Point::z_projectOntoEdge (point.cpp:337-347)
__device__ __forceinline__ double z_proj(D3 me, D3 p1, D3 p2) {
    double t;
    if (fabs(p2.x - p1.x) > fabs(p2.y - p1.y))
        t = (me.x - p1.x) / (p2.x - p1.x);
    else
        t = (me.y - p1.y) / (p2.y - p1.y);
    return p1.z + t * (p2.z - p1.z);
}

// Running CL state of one triangle evaluation (CLPoint z + CC).
struct CL64 {
    double x, y, z;
    D3 cc;
    int type;
};
__device__ __forceinline__ bool liftz(CL64& cl, double zin, D3 cc, int type) {
    if (zin > cl.z) {
        cl.z = zin;
        cl.cc = cc;
        cl.type = type;
        return true;
    }
    return false;
}

// cutter height(r)
__device__ __forceinline__ double height_basic(const BasicP& c, double r) {
    switch (c.kind) {
    case OCL_CUTTER_CYL: return (r <= c.radius) ? 0.0 : -1.0;
    case OCL_CUTTER_BALL: return c.radius - sqrt(sq(c.radius) - sq(r));
    case OCL_CUTTER_BULL:
        if (r <= c.radius1) return 0.0;
        if (r <= c.radius) return c.radius2 - sqrt(sq(c.radius2) - sq(r - c.radius1));
        return -1;
    case OCL_CUTTER_CONE: return r / c.tan_angle;
    }
    return -1;
}
__device__ __forceinline__ bool comp_valid(const double* vec, int n, double r) {
    double lo = (n == 0) ? -1E-6 : vec[n - 1] - 1E-6;
    double hi = vec[n] + 1e-6;
    return (lo <= r) && (r <= hi);
}
__device__ __forceinline__ double height_any(const CutterP& c, double r) {
    if (c.kind != OCL_CUTTER_COMPOSITE) return height_basic(c.b, r);
    int idx = 0;
    for (int n = 0; n < c.nsub; ++n)
        if (comp_valid(c.radiusvec, n, r)) { idx = n; break; }
    return height_basic(c.sub[idx], r) + c.zoffset[idx];
}

// ---------------------------------------------------------------------------
// Offset ellipse (BullCutter edge drop), ellipse.cpp / ellipseposition.cpp.
// ---------------------------------------------------------------------------
struct EPos {
    double s, t;
};
__device__ __forceinline__ EPos epos(double dia) {
    double d = dia;
    for (int k = 0; k < 64 && d > 4.0; ++k) d -= 4.0;
    for (int k = 0; k < 64 && d < 0.0; ++k) d += 4.0;
    D3 p = d3((d < 2 ? 1 - d : d - 3), (d < 3 ? ((d > 1) ? 2 - d : d) : d - 4), 0.0);
    p = normalize3(p);
    return EPos{p.x, p.y};
}
struct Ell {
    D3 center;
    double a, b, offset;
};
__device__ __forceinline__ D3 ell_epoint(const Ell& E, EPos p) {
    D3 r = E.center;
    r.x += E.a * p.s;
    r.y += E.b * p.t;
    return r;
}
__device__ __forceinline__ D3 ell_oepoint(const Ell& E, EPos p) {
    D3 n = normalize3(d3(E.b * p.s, E.a * p.t, 0));
    return ell_epoint(E, p) + E.offset * n;
}
__device__ __forceinline__ double ell_err(const Ell& E, EPos p) { return ell_oepoint(E, p).y; }

// brent_zero (common/brent_zero.hpp:37-123) with an iteration cap.
__device__ inline double brent_ell(double a, double b, const Ell& E, int* capped) {
    const double eps = 3E-16, t = OCLG_OE_TOL;
    double c, d, e, fa, fb, fc, m, p, q, r, s, tol;
    fa = ell_err(E, epos(a));
    fb = ell_err(E, epos(b));
    c = a;
    fc = fa;
    e = b - a;
    d = e;
    for (int it = 0;; ++it) {
        if (it >= OCLG_BRENT_CAP) {
            *capped += 1;
            break;
        }
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
        fb = ell_err(E, epos(b));
        if (signbit(fb) == signbit(fc)) {
            c = a;
            fc = fa;
            e = b - a;
            d = e;
        }
    }
    return b;
}

// Ellipse::solver_brent + find_EllipsePosition2 + setEllipsePositionHi
// (ellipse.cpp:118-208, 332-354); returns the hi ellipse point and centre z.
__device__ inline void bull_ellipse(const BasicP& c, D3 u1, D3 u2, double a_axis, D3& ell_ccp, double& center_z,
                             int* capped) {
    Ell E;
    E.center = d3(0, u1.y, 0);
    E.a = a_axis;
    E.b = c.radius2;
    E.offset = c.radius1;
    EPos e1, e2;
    EPos apos = epos(0.0), bpos = epos(3.0);
    if (fabs(ell_err(E, apos)) < OCLG_OE_TOL) {
        e1 = apos;
    } else if (fabs(ell_err(E, bpos)) < OCLG_OE_TOL) {
        e1 = bpos;
    } else {
        e1 = epos(brent_ell(0.0, 3.0, E, capped));
    }
    // find_EllipsePosition2: (s,-t), (-s,t), (-s,-t), then (s,t)
    double err1 = fabs(ell_err(E, e1));
    e2 = e1;
    for (int k = 0; k < 4; ++k) {
        e2.s = (k == 1 || k == 2) ? -e1.s : e1.s;
        e2.t = (k == 0 || k == 2) ? -e1.t : e1.t;
        if (fabs(ell_err(E, e2)) < err1 + OCLG_OE_TOL) {
            if (k == 3) break;
            if ((fabs(e2.s - e1.s) > 1E-8) || (fabs(e2.t - e1.t) > 1E-8)) break;
        }
    }
    // calcEcenter for both solutions, keep the higher centre
    D3 c1, c2;
    {
        D3 cle = ell_oepoint(E, e1);
        double t = (E.center.x + (-cle.x) - u1.x) / (u2.x - u1.x);
        c1 = u1 + t * (u2 - u1);
    }
    {
        D3 cle = ell_oepoint(E, e2);
        double t = (E.center.x + (-cle.x) - u1.x) / (u2.x - u1.x);
        c2 = u1 + t * (u2 - u1);
    }
    EPos hi;
    if (c1.z >= c2.z) {
        hi = e1;
        E.center = c1;
    } else {
        hi = e2;
        E.center = c2;
    }
    ell_ccp = ell_epoint(E, hi);
    center_z = E.center.z;
}

// singleEdgeDropCanonical of each basic cutter.
__device__ inline void edge_canonical(const BasicP& c, D3 u1, D3 u2, double& ccu, double& clz, int* capped) {
    switch (c.kind) {
    case OCL_CUTTER_CYL: {
        double s = sqrt(sq(c.radius) - sq(u1.y));
        D3 a = d3(s, u1.y, 0), b = d3(-s, u1.y, 0);
        a.z = z_proj(a, u1, u2);
        b.z = z_proj(b, u1, u2);
        if (a.z > b.z) { ccu = a.x; clz = a.z; }
        else { ccu = b.x; clz = b.z; }
        return;
    }
    case OCL_CUTTER_BALL: {
        double s = sqrt(sq(c.radius) - sq(u1.y));
        D3 nrm = xynormalize(d3(u2.z - u1.z, -(u2.x - u1.x), 0));
        if (nrm.y < 0) nrm = (-1.0) * nrm;
        D3 cc = d3(-s * nrm.x, u1.y, 0);
        cc.z = z_proj(cc, u1, u2);
        ccu = cc.x;
        clz = cc.z + s * nrm.y - c.radius;
        return;
    }
    case OCL_CUTTER_BULL: {
        if (zero_tol(u1.z - u2.z)) {
            ccu = 0;
            clz = u1.z - height_basic(c, u1.y);
            return;
        }
        double theta = atan((u2.z - u1.z) / (u2.x - u1.x));
        double a_axis = fabs(c.radius2 / sin(theta));
        D3 ell_ccp;
        double center_z;
        bull_ellipse(c, u1, u2, a_axis, ell_ccp, center_z, capped);
        D3 cc_u = closest_point(ell_ccp, u1, u2);
        ccu = cc_u.x;
        clz = center_z - c.radius2;
        return;
    }
    case OCL_CUTTER_CONE: {
        double d = u1.y;
        double m = (u2.z - u1.z) / (u2.x - u1.x);
        double xu = sqrt(sq(c.radius) - sq(u1.y));
        double mu = (c.center_height / c.radius) * xu / sqrt(sq(xu) + sq(d));
        bool hyp = (fabs(m) <= fabs(mu));
        double cu;
        if (hyp)
            cu = sgn(m) * sqrt(sq(c.radius) * sq(m) * sq(d) / (sq(c.length) - sq(c.radius) * sq(m)));
        else
            cu = sgn(m) * xu;
        D3 cc = d3(cu, d, 0.0);
        cc.z = z_proj(cc, u1, u2);
        if (hyp)
            clz = cc.z - c.center_height + (c.radius - sqrt(sq(cu) + sq(d))) / c.tan_angle;
        else
            clz = cc.z - c.center_height;
        ccu = cu;
        return;
    }
    }
    ccu = 0;
    clz = -1e300;
}

__device__ __forceinline__ D3 tri_p(const Tri64& t, int k) { return d3(t.p[3 * k], t.p[3 * k + 1], t.p[3 * k + 2]); }

// MillingCutter::edgeDrop + singleEdgeDrop for one basic cutter.
// MillingCutter::singleEdgeDrop (millingcutter.cpp:100-136) for one edge of a
// CL point at (x, y): the contact height and CC point, true when the CC lies
// on the segment.  Independent of the CL point's running height.
__device__ inline bool edge_contact64(const BasicP& c, double x, double y, D3 p1, D3 p2, double& clz, D3& cc,
                                      int* capped) {
    double d = xy_dist_line(d3(x, y, 0.0), p1, p2);
    if (!(d <= c.radius)) return false;
    D3 v = p2 - p1;
    D3 vxy = xynormalize(d3(v.x, v.y, 0.0));
    D3 sc = xy_closest(d3(x, y, 0.0), p1, p2);
    D3 u1 = d3(dot(p1 - sc, vxy), d, p1.z);
    D3 u2 = d3(dot(p2 - sc, vxy), d, p2.z);
    double ccu;
    edge_canonical(c, u1, u2, ccu, clz, capped);
    cc = sc + ccu * vxy;
    cc.z = z_proj(cc, p1, p2);
    return in_seg(cc, p1, p2);
}

__device__ inline bool edge_drop_basic(const BasicP& c, CL64& cl, const Tri64& t, uint32_t flags, int* capped) {
    bool result = false;
    for (int n = 0; n < 3; ++n) {
        if (flags & (TF_EDGE0_SKIP << n)) continue;  // isZero_tol(dx) && isZero_tol(dy)
        double clz;
        D3 cc;
        if (edge_contact64(c, cl.x, cl.y, tri_p(t, n), tri_p(t, (n + 1) % 3), clz, cc, capped))
            if (liftz(cl, clz, cc, OCL_CC_EDGE)) result = true;
    }
    return result;
}

// MillingCutter::facetDrop for a basic (non-cone) cutter.
__device__ inline bool facet_drop_base(const BasicP& c, CL64& cl, const Tri64& t, uint32_t flags) {
    uint32_t mode = flags & TF_FACET_MASK;
    if (mode == TF_FACET_NONE) return false;
    if (mode == TF_FACET_HORIZ) {
        D3 cc = d3(cl.x, cl.y, t.p[2]);
        if (in_tri(cc, t.p)) return liftz(cl, cc.z, cc, OCL_CC_FACET);
        return false;
    }
    D3 nn = d3(t.nn[0], t.nn[1], t.nn[2]);
    D3 xyn = d3(t.xyn[0], t.xyn[1], 0.0);
    D3 rv = c.xy_normal_length * xyn + c.normal_length * nn;
    D3 cc = d3(cl.x, cl.y, cl.z) - rv;
    cc.z = (1.0 / nn.z) * (-t.d - nn.x * cc.x - nn.y * cc.y);
    double tip_z = cc.z + rv.z - c.center_height;
    if (in_tri(cc, t.p)) return liftz(cl, tip_z, cc, OCL_CC_FACET);
    return false;
}

// ConeCutter::facetDrop (conecutter.cpp:70-105)
__device__ inline bool facet_drop_cone(const BasicP& c, CL64& cl, const Tri64& t, uint32_t flags) {
    uint32_t mode = flags & TF_FACET_MASK;
    if (mode == TF_FACET_NONE) return false;
    if (mode == TF_FACET_HORIZ) {
        D3 cc = d3(cl.x, cl.y, t.p[2]);
        if (in_tri(cc, t.p)) return liftz(cl, cc.z, cc, OCL_CC_FACET_TIP);
        return false;
    }
    D3 n = d3(t.n[0], t.n[1], t.n[2]);
    double a = n.x, b = n.y, cz = n.z;
    n = xynormalize(n);
    D3 cyl = d3(cl.x, cl.y, cl.z) - c.radius * n;
    cyl.z = (1.0 / cz) * (-t.d - a * cyl.x - b * cyl.y);
    double cyl_cl_z = cyl.z - c.length;
    D3 tip = d3(cl.x, cl.y, 0.0);
    tip.z = (1.0 / cz) * (-t.d - a * tip.x - b * tip.y);
    if (in_tri(tip, t.p) && liftz(cl, tip.z, tip, OCL_CC_FACET_TIP)) return true;
    if (in_tri(cyl, t.p) && liftz(cl, cyl_cl_z, cyl, OCL_CC_FACET_CYL)) return true;
    return false;
}

__device__ __forceinline__ bool facet_drop_sub(const BasicP& c, CL64& cl, const Tri64& t, uint32_t flags) {
    return c.kind == OCL_CUTTER_CONE ? facet_drop_cone(c, cl, t, flags) : facet_drop_base(c, cl, t, flags);
}

// CompositeCutter::facetDrop / edgeDrop (compositecutter.cpp:152-193).
// sub_skip bit 3n+e: edge e of sub-cutter n cannot lift it (left out);
// facet_skip bit n: no facet contact of sub-cutter n can lift the composite.
__device__ inline bool comp_drop(const CutterP& c, CL64& cl, const Tri64& t, uint32_t flags, bool facet, int* capped,
                                 uint32_t sub_skip = 0, uint32_t facet_skip = 0) {
    bool result = false;
    for (int n = 0; n < c.nsub; ++n) {
        if (facet ? ((facet_skip >> n) & 1u) : ((sub_skip >> (3 * n)) & 7u) == 7u) continue;
        CL64 tmp;
        tmp.x = cl.x;
        tmp.y = cl.y;
        tmp.z = cl.z + c.zoffset[n];
        tmp.cc = d3(0, 0, 0);
        tmp.type = OCL_CC_NONE;
        bool hit = facet ? facet_drop_sub(c.sub[n], tmp, t, flags)
                         : edge_drop_basic(c.sub[n], tmp, t, flags | (((sub_skip >> (3 * n)) & 7u) << 2), capped);
        if (hit && tmp.type != OCL_CC_NONE) {
            double dd = xynorm(d3(tmp.x, tmp.y, tmp.z) - tmp.cc);
            double lo = (n == 0) ? -1E-6 : c.radiusvec[n - 1] - 1E-6;
            double hi = c.radiusvec[n] + 1e-6;
            if (!(dd < lo) && !(dd > hi)) {
                if (liftz(cl, tmp.z - c.zoffset[n], tmp.cc, facet ? OCL_CC_FACET : OCL_CC_EDGE)) result = true;
            }
        }
    }
    return result;
}

// Lowest running height at which the effect of triangle t on a CL point at
// (x, y) changes form, for the cone and the composites (+inf: the effect is
// max(Z, c) for every running height Z, or there is no facet contact).
// Below the returned height every fold gets the same value and CC point from
// the triangle's facet, whatever the running height is.
//   ConeCutter::facetDrop (conecutter.cpp:70-105): the first of tip, rim that
//   lies inside the triangle ends the drop when it lifts;
//   CompositeCutter::facetDrop (compositecutter.cpp:152-172): the facet ends
//   the triangle at the highest valid contact; a cone sub-cutter's rim is only
//   tried from at or above its tip.
__device__ inline double branch_low64(const CutterP& c, double x, double y, const Tri64& t, uint32_t flags) {
    const double INF = 1.0e300;
    if ((flags & TF_FACET_MASK) == TF_FACET_NONE) return INF;
    if (c.kind == OCL_CUTTER_CONE) {
        CL64 tmp{x, y, -INF, d3(0, 0, 0), OCL_CC_NONE};
        return facet_drop_cone(c.b, tmp, t, flags) ? tmp.z : INF;
    }
    if (c.kind != OCL_CUTTER_COMPOSITE) return INF;
    double mh = -INF;  // highest valid contact no tip can hide
    double tipv[OCL_GB300_MAX_SUB], rimv[OCL_GB300_MAX_SUB];
    for (int n = 0; n < c.nsub; ++n) {
        tipv[n] = INF;
        rimv[n] = -INF;
        const BasicP& s = c.sub[n];
        const double zo = c.zoffset[n];
        const double lo = (n == 0) ? -1E-6 : c.radiusvec[n - 1] - 1E-6;
        const double hi = c.radiusvec[n] + 1e-6;
        CL64 tmp{x, y, -INF, d3(0, 0, 0), OCL_CC_NONE};
        if (s.kind == OCL_CUTTER_CONE) {
            const bool hit = facet_drop_cone(s, tmp, t, flags);
            if (!hit) continue;
            const double dd = xynorm(d3(tmp.x, tmp.y, tmp.z) - tmp.cc);
            const bool valid = !(dd < lo) && !(dd > hi);
            if (valid) mh = fmax(mh, tmp.z - zo);
            if (tmp.type == OCL_CC_FACET_TIP) {
                // the rim, tried only from at or above the tip
                CL64 t2{x, y, tmp.z, d3(0, 0, 0), OCL_CC_NONE};
                if (facet_drop_cone(s, t2, t, flags) && t2.type == OCL_CC_FACET_CYL) {
                    const double d2 = xynorm(d3(t2.x, t2.y, t2.z) - t2.cc);
                    if (!(d2 < lo) && !(d2 > hi)) {
                        tipv[n] = tmp.z - zo;
                        rimv[n] = t2.z - zo;
                    }
                }
            }
        } else if (facet_drop_base(s, tmp, t, flags)) {
            const double dd = xynorm(d3(tmp.x, tmp.y, tmp.z) - tmp.cc);
            if (!(dd < lo) && !(dd > hi)) mh = fmax(mh, tmp.z - zo);
        }
    }
    double b = (mh > -INF) ? mh : INF;
    for (int n = 0; n < c.nsub; ++n)
        if (rimv[n] >= mh) b = fmin(b, tipv[n]);
    return b;
}

// MillingCutter::dropCutter for one triangle, from cl.z; cl is updated.
// part_skip bit k (k < 3): vertex k cannot lift cl; bit 8 + n: no facet
// contact of composite sub-cutter n can; PART_SKIP_FACET: the facet contact
// of a basic cutter cannot (all left out).
constexpr uint32_t PART_SKIP_FACET = 1u << 16;
__device__ inline void drop_triangle64(const CutterP& c, CL64& cl, const Tri64& t, uint32_t flags, int* capped,
                                       uint32_t sub_skip = 0, uint32_t part_skip = 0) {
    if (!(cl.z < t.bb[5])) return;
    bool facet;
    if (c.kind == OCL_CUTTER_COMPOSITE) facet = comp_drop(c, cl, t, flags, true, capped, 0, part_skip >> 8);
    else facet = (part_skip & PART_SKIP_FACET) ? false : facet_drop_sub(c.b, cl, t, flags);
    if (facet) return;
    // vertexDrop (millingcutter.cpp:36-47) with the cutter's height(r)
    for (int k = 0; k < 3; ++k) {
        if ((part_skip >> k) & 1u) continue;
        D3 p = tri_p(t, k);
        double q = xynorm(d3(cl.x, cl.y, cl.z) - p);
        if (q <= c.radius) liftz(cl, p.z - height_any(c, q), p, OCL_CC_VERTEX);
    }
    if (!(cl.z < t.bb[5])) return;
    if (c.kind == OCL_CUTTER_COMPOSITE) comp_drop(c, cl, t, flags, false, capped, sub_skip);
    else edge_drop_basic(c.b, cl, t, flags, capped);
}

// MillingCutter::overlaps (millingcutter.cpp:422-433)
__device__ __forceinline__ bool overlaps64(double r, double x, double y, const Tri64& t) {
    if (t.bb[1] < x - r) return false;
    if (t.bb[0] > x + r) return false;
    if (t.bb[3] < y - r) return false;
    if (t.bb[2] > y + r) return false;
    return true;
}

}  // namespace oclg
