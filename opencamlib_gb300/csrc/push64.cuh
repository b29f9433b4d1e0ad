// push64.cuh -- FP64 push-cutter contacts and fiber intervals, device side.
//
// Follows the reference's push semantics (paths relative to opencamlib src/):
//   MillingCutter::pushCutter  cutters/millingcutter.cpp:377-382
//   vertexPush  millingcutter.cpp:139-167 (+ CylCutter::vertexPush
//               cylcutter.cpp:73-91 with Triangle::zslice_verts triangle.cpp:77-128)
//   facetPush   millingcutter.cpp:169-275 (+ ConeCutter::facetPush conecutter.cpp:137-147)
//   edgePush    millingcutter.cpp:277-375 + generalEdgePush of Ball
//               (ballcutter.cpp:66-116), Bull (bullcutter.cpp:109-155 with
//               AlignedEllipse::aligned_solver ellipse.cpp:212-317) and Cone
//               (conecutter.cpp:150-300)
//   Composite   compositecutter.cpp:196-270
//   Interval    algo/interval.cpp:29-118, Fiber::addInterval algo/fiber.cpp:58-93
#pragma once
#include "geom64.cuh"

namespace oclg {

struct Fib64 {
    D3 p1, p2, dir;
};
__device__ __forceinline__ double f_tval(const Fib64& f, D3 p) {
    D3 d = f.p2 - f.p1;
    return dot(p - f.p1, d) / dot(d, d);
}
__device__ __forceinline__ D3 f_point(const Fib64& f, double t) { return f.p1 + t * (f.p2 - f.p1); }
__device__ __forceinline__ D3 xyperp(D3 a) { return d3(-a.y, a.x, a.z); }

struct CCp {
    D3 p;
    int type;
};
struct Ival64 {
    double lower, upper;
    CCp lcc, ucc;
};
__device__ __forceinline__ void iv_init(Ival64& i) {
    i.lower = 0.0;
    i.upper = 0.0;
    i.lcc.p = d3(0, 0, 0);
    i.lcc.type = OCL_CC_NONE;
    i.ucc = i.lcc;
}
__device__ __forceinline__ void iv_upper(Ival64& i, double t, const CCp& p) {
    if (i.ucc.type == OCL_CC_NONE) {
        i.upper = t; i.lower = t; i.ucc = p; i.lcc = p;
    }
    if (t > i.upper) { i.upper = t; i.ucc = p; }
}
__device__ __forceinline__ void iv_lower(Ival64& i, double t, const CCp& p) {
    if (i.lcc.type == OCL_CC_NONE) {
        i.lower = t; i.upper = t; i.lcc = p; i.ucc = p;
    }
    if (t < i.lower) { i.lower = t; i.lcc = p; }
}
__device__ __forceinline__ void iv_update(Ival64& i, double t, const CCp& p) {
    iv_upper(i, t, p);
    iv_lower(i, t, p);
}
__device__ __forceinline__ bool iv_update_if(Ival64& i, double t, const CCp& cc, D3 p1, D3 p2, bool cond) {
    if (in_seg(cc.p, p1, p2) && cond) {
        iv_update(i, t, cc);
        return true;
    }
    return false;
}

// two_by_two_solver / xy_line_line_intersection (common/numeric.cpp:118-154)
__device__ __forceinline__ bool two_by_two(double a, double b, double c, double d, double e, double f, double& u,
                                           double& v) {
    double det = a * d - c * b;
    if (zero_tol(det)) return false;
    u = (1.0 / det) * (d * e - b * f);
    v = (1.0 / det) * (-c * e + a * f);
    return true;
}
__device__ __forceinline__ bool xy_line_line(D3 p1, D3 p2, double& v, D3 p3, D3 p4, double& t) {
    return two_by_two(p2.x - p1.x, -(p4.x - p3.x), p2.y - p1.y, -(p4.y - p3.y), (p3.x - p1.x), p3.y - p1.y, v, t);
}
// xyVectorToDiangle (numeric.cpp:36-51)
__device__ __forceinline__ double xy_to_diangle(double x, double y) {
    if (y >= 0) return (x >= 0 ? y / (x + y) : 1 - x / (-x + y));
    return (x < 0 ? 2 - y / (-x - y) : 3 + x / (x - y));
}

__device__ __forceinline__ double width_basic(const BasicP& c, double h) {
    switch (c.kind) {
    case OCL_CUTTER_CYL: return c.radius;
    case OCL_CUTTER_BALL: return (h >= c.radius) ? c.radius : sqrt(sq(c.radius) - sq(c.radius - h));
    case OCL_CUTTER_BULL: return (h >= c.radius2) ? c.radius : c.radius1 + sqrt(sq(c.radius2) - sq(c.radius2 - h));
    case OCL_CUTTER_CONE: return (h < c.center_height) ? h * c.tan_angle : c.radius;
    }
    return -1;
}

// MillingCutter::singleVertexPush
__device__ inline bool single_vertex_push(const BasicP& c, const Fib64& f, Ival64& i, D3 p, int type) {
    if ((p.z >= f.p1.z) && (p.z <= (f.p1.z + c.length))) {
        D3 pq = xy_closest(p, f.p1, f.p2);
        double q = xynorm(p - pq);
        double h = p.z - f.p1.z;
        double cw = width_basic(c, h);
        if (q <= cw) {
            double ofs = sqrt(sq(cw) - sq(q));
            D3 start = pq - ofs * f.dir;
            D3 stop = pq + ofs * f.dir;
            CCp cc{p, type};
            iv_upper(i, f_tval(f, stop), cc);
            iv_lower(i, f_tval(f, start), cc);
            return true;
        }
    }
    return false;
}

__device__ inline bool vertex_push_basic(const BasicP& c, const Fib64& f, Ival64& i, const Tri64& t) {
    bool result = false;
    for (int k = 0; k < 3; ++k)
        if (single_vertex_push(c, f, i, tri_p(t, k), OCL_CC_VERTEX)) result = true;
    if (c.kind == OCL_CUTTER_CYL) {
        // Triangle::zslice_verts at the fiber height
        double zcut = f.p1.z;
        if (!((zcut <= t.bb[4]) || (zcut >= t.bb[5]))) {
            D3 below[3], above[3];
            int nb = 0, na = 0;
            for (int m = 0; m < 3; ++m) {
                D3 p = tri_p(t, m);
                if (p.z <= zcut) below[nb++] = p;
                else above[na++] = p;
            }
            D3 p1, p2;
            bool ok = true;
            if (nb == 2) {
                double t1 = (zcut - above[0].z) / (below[0].z - above[0].z);
                double t2 = (zcut - above[0].z) / (below[1].z - above[0].z);
                p1 = above[0] + t1 * (below[0] - above[0]);
                p2 = above[0] + t2 * (below[1] - above[0]);
            } else if (nb == 1) {
                double t1 = (zcut - above[0].z) / (below[0].z - above[0].z);
                double t2 = (zcut - above[1].z) / (below[0].z - above[1].z);
                p1 = above[0] + t1 * (below[0] - above[0]);
                p2 = above[1] + t2 * (below[0] - above[1]);
            } else {
                ok = false;
            }
            if (ok) {
                p1.z = f.p1.z;
                p2.z = f.p1.z;
                if (single_vertex_push(c, f, i, p1, OCL_CC_VERTEX_CYL)) result = true;
                if (single_vertex_push(c, f, i, p2, OCL_CC_VERTEX_CYL)) result = true;
            }
        }
    }
    return result;
}

// MillingCutter::generalFacetPush
__device__ inline bool general_facet_push(double normal_length, double center_height, double xy_normal_length,
                                          const Fib64& fib, Ival64& i, const Tri64& t) {
    D3 normal = d3(t.n[0], t.n[1], t.n[2]);
    if (normal.x == 0.0 && normal.y == 0.0) return false;
    normal = normalize3(normal);
    D3 xyn = normal;
    xyn.z = 0;
    xyn = xynormalize(xyn);
    double a, b, e, u, v;
    double c = t.p[5] - t.p[2];
    double d = t.p[8] - t.p[2];
    double f = -t.p[2] - normal_length * normal.z + fib.p1.z + center_height;
    D3 p0 = tri_p(t, 0), p1 = tri_p(t, 1), p2 = tri_p(t, 2);
    if (fib.p1.y == fib.p2.y) {
        a = p1.y - p0.y;
        b = p2.y - p0.y;
        e = -p0.y - normal_length * normal.y - xy_normal_length * xyn.y + fib.p1.y;
        if (!two_by_two(a, b, c, d, e, f, u, v)) return false;
        CCp cc{(p0 + u * (p1 - p0)) + v * (p2 - p0), OCL_CC_FACET};
        if (!in_tri(cc.p, t.p)) return false;
        double tval = (1.0 / (fib.p2.x - fib.p1.x)) * (p0.x + normal_length * normal.x + xy_normal_length * xyn.x -
                                                       fib.p1.x + u * (p1.x - p0.x) + v * (p2.x - p0.x));
        iv_update(i, tval, cc);
        return true;
    } else if (fib.p1.x == fib.p2.x) {
        a = p1.x - p0.x;
        b = p2.x - p0.x;
        e = -p0.x - normal_length * normal.x - xy_normal_length * xyn.x + fib.p1.x;
        if (!two_by_two(a, b, c, d, e, f, u, v)) return false;
        CCp cc{(p0 + u * (p1 - p0)) + v * (p2 - p0), OCL_CC_FACET};
        if (!in_tri(cc.p, t.p)) return false;
        double tval = (1.0 / (fib.p2.y - fib.p1.y)) * (p0.y + normal_length * normal.y + xy_normal_length * xyn.y -
                                                       fib.p1.y + u * (p1.y - p0.y) + v * (p2.y - p0.y));
        iv_update(i, tval, cc);
        return true;
    }
    return false;
}

__device__ inline bool facet_push_basic(const BasicP& c, const Fib64& f, Ival64& i, const Tri64& t) {
    if (c.kind == OCL_CUTTER_CONE) {
        bool r = false;
        if (general_facet_push(0, 0, 0, f, i, t)) r = true;
        if (general_facet_push(0, c.center_height, c.xy_normal_length, f, i, t)) r = true;
        return r;
    }
    return general_facet_push(c.normal_length, c.center_height, c.xy_normal_length, f, i, t);
}

__device__ __forceinline__ bool calc_cc_update(double tt, double u, D3 q, D3 p1, D3 p2, Ival64& i, double height,
                                               int type) {
    CCp cc{q + u * (p2 - p1), type};
    return iv_update_if(i, tt, cc, p1, p2, (cc.p.z >= height));
}

__device__ inline bool horiz_edge_push(const BasicP& c, const Fib64& f, Ival64& i, D3 p1, D3 p2) {
    bool result = false;
    double h = p1.z - f.p1.z;
    if (h > 0.0 && zero_tol(p2.z - p1.z)) {
        double eff = width_basic(c, h);
        double qt, qv;
        if (xy_line_line(p1, p2, qv, f.p1, f.p2, qt)) {
            D3 q = p1 + qv * (p2 - p1);
            double ccv, clt;
            D3 tang = p2 - p1;
            tang.z = 0;
            tang = xynormalize(tang);
            D3 xyn = xyperp(tang);
            D3 q1 = q + eff * xyn;
            D3 q2 = q1 + (p2 - p1);
            if (xy_line_line(q1, q2, ccv, f.p1, f.p2, clt)) {
                double t1 = clt;
                double t2 = qt + (qt - clt);
                if (calc_cc_update(t1, ccv, q, p1, p2, i, f.p1.z, OCL_CC_EDGE_HORIZ)) result = true;
                if (calc_cc_update(t2, -ccv, q, p1, p2, i, f.p1.z, OCL_CC_EDGE_HORIZ)) result = true;
            }
        }
    }
    return result;
}

__device__ inline bool shaft_edge_push(const BasicP& c, const Fib64& f, Ival64& i, D3 p1, D3 p2) {
    double u, v;
    bool result = false;
    if (xy_line_line(p1, p2, u, f.p1, f.p2, v)) {
        D3 q = p1 + u * (p2 - p1);
        D3 tang = p2 - p1;
        tang.z = 0;
        tang = xynormalize(tang);
        D3 xyn = xyperp(tang);
        D3 q1 = q + c.radius * xyn;
        D3 q2 = q1 + (p2 - p1);
        double u_cc, t_cl;
        if (xy_line_line(q1, q2, u_cc, f.p1, f.p2, t_cl)) {
            double t1 = t_cl;
            double t2 = v + (v - t_cl);
            if (calc_cc_update(t1, u_cc, q, p1, p2, i, f.p1.z + c.center_height, OCL_CC_EDGE_SHAFT)) result = true;
            if (calc_cc_update(t2, -u_cc, q, p1, p2, i, f.p1.z + c.center_height, OCL_CC_EDGE_SHAFT)) result = true;
        }
    }
    return result;
}

__device__ __forceinline__ bool ball_cc_update(const BasicP& c, double tt, D3 p1, D3 p2, const Fib64& f, Ival64& i) {
    D3 center = f_point(f, tt) + d3(0, 0, c.radius);
    CCp cc{closest_point(center, p1, p2), OCL_CC_EDGE_BALL};
    return iv_update_if(i, tt, cc, p1, p2, (center.z - cc.p.z >= 0));
}

__device__ inline bool ball_edge_push(const BasicP& c, const Fib64& f, Ival64& i, D3 p1, D3 p2) {
    bool result = false;
    if (zero_tol(xynorm(p2 - p1))) return false;
    D3 ufp1 = f.p1 + d3(0, 0, c.radius);
    D3 ufp2 = f.p2 + d3(0, 0, c.radius);
    D3 ab = p2 - p1;
    D3 ao = ufp1 - p1;
    D3 vv = ufp2 - ufp1;
    D3 ao_x_ab = d3(ao.y * ab.z - ao.z * ab.y, ao.z * ab.x - ao.x * ab.z, ao.x * ab.y - ao.y * ab.x);
    D3 v_x_ab = d3(vv.y * ab.z - vv.z * ab.y, vv.z * ab.x - vv.x * ab.z, vv.x * ab.y - vv.y * ab.x);
    double ab2 = dot(ab, ab);
    double a = dot(v_x_ab, v_x_ab);
    double b = 2 * (dot(v_x_ab, ao_x_ab));
    double cc = dot(ao_x_ab, ao_x_ab) - (c.radius * c.radius * ab2);
    double discr = b * b - 4 * a * cc;
    if (zero_tol(discr)) {
        double t1 = -b / (2 * a);
        if (ball_cc_update(c, t1, p1, p2, f, i)) result = true;
    } else if (discr > 0.0) {
        double t1 = (-b + sqrt(discr)) / (2 * a);
        double t2 = (-b - sqrt(discr)) / (2 * a);
        if (ball_cc_update(c, t1, p1, p2, f, i)) result = true;
        if (ball_cc_update(c, t2, p1, p2, f, i)) result = true;
    }
    return result;
}

// AlignedEllipse (ellipse.cpp:82-108, 212-317)
struct AEll {
    D3 center, major, minor, error_dir, target;
    double a, b, offset;
};
__device__ __forceinline__ D3 aell_epoint(const AEll& E, EPos p) {
    return (E.center + (E.a * p.s) * E.major) + (E.b * p.t) * E.minor;
}
__device__ __forceinline__ D3 aell_oepoint(const AEll& E, EPos p) {
    D3 n = normalize3((p.s * E.b) * E.major + (p.t * E.a) * E.minor);
    return aell_epoint(E, p) + E.offset * n;
}
__device__ __forceinline__ double aell_err(const AEll& E, double dia) {
    D3 p = aell_oepoint(E, epos(dia));
    return dot(E.target - p, E.error_dir);
}

__device__ inline double brent_aell(double a, double b, const AEll& E, int* capped) {
    const double eps = 3E-16, tt = OCLG_OE_TOL;
    double c, d, e, fa, fb, fc, m, p, q, r, s, tol;
    fa = aell_err(E, a);
    fb = aell_err(E, b);
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
        tol = 2.0 * eps * fabs(b) + tt;
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
        fb = aell_err(E, b);
        if (signbit(fb) == signbit(fc)) {
            c = a;
            fc = fa;
            e = b - a;
            d = e;
        }
    }
    return b;
}

// sin_theta: sin(atan(dz / xy length)) of the edge, computed on the host
// (Mesh::d_edge_sin).
__device__ inline bool bull_edge_push(const BasicP& c, const Fib64& f, Ival64& i, D3 p1, D3 p2, double sin_theta,
                                      int* capped) {
    bool result = false;
    if (zero_tol(xynorm(p2 - p1))) return false;
    if (zero_tol(p2.z - p1.z)) return false;
    double tplane = (f.p1.z + c.radius2 - p1.z) / (p2.z - p1.z);
    AEll E;
    E.center = p1 + tplane * (p2 - p1);
    D3 major = p2 - p1;
    major.z = 0;
    E.major = xynormalize(major);
    E.minor = xyperp(E.major);
    E.a = fabs(c.radius2 / sin_theta);
    E.b = c.radius2;
    E.offset = c.radius1;
    // aligned_solver
    E.error_dir = xyperp(f.dir);
    E.target = f.p1;
    double t1 = 0.0;
    if (f.p1.y == f.p2.y)
        t1 = sqrt(sq(E.b * E.minor.y) / (sq(E.a * E.major.y) + sq(E.b * E.minor.y)));
    else if (f.p1.x == f.p2.x)
        t1 = sqrt(sq(E.b * E.minor.x) / (sq(E.a * E.major.x) + sq(E.b * E.minor.x)));
    double s1 = sqrt(1.0 - sq(t1));
    bool fpos = false, fneg = false;
    double apos = 0.0, bpos = 0.0;  // diangles
    for (int k = 0; k < 4; ++k) {
        double xs = (k < 2) ? s1 : -s1;
        double ys = (k & 1) ? -t1 : t1;
        double dia = xy_to_diangle(xs, ys);
        double err = aell_err(E, dia);
        if (err > 0) { fpos = true; apos = dia; }
        else if (err < 0) { fneg = true; bpos = dia; }
    }
    if (fpos && fneg) {
        double lolim = 0.0, hilim = 0.0;
        if (apos > bpos) { lolim = bpos; hilim = apos; }
        else if (bpos > apos) { hilim = bpos; lolim = apos; }
        double d1 = brent_aell(lolim, hilim, E, capped);
        double d2 = brent_aell(hilim - 4.0, lolim, E, capped);
        EPos e1 = epos(d1), e2 = epos(d2);
        CCp cc{closest_point(aell_epoint(E, e1), p1, p2), OCL_CC_EDGE_POS};
        CCp cc2{closest_point(aell_epoint(E, e2), p1, p2), OCL_CC_EDGE_POS};
        D3 cl = aell_oepoint(E, e1) - d3(0, 0, c.center_height);
        D3 cl2 = aell_oepoint(E, e2) - d3(0, 0, c.center_height);
        double cl_t = f_tval(f, cl);
        double cl_t2 = f_tval(f, cl2);
        if (iv_update_if(i, cl_t, cc, p1, p2, true)) result = true;
        if (iv_update_if(i, cl_t2, cc2, p1, p2, true)) result = true;
    }
    return result;
}

__device__ __forceinline__ bool cone_circle_cc(const BasicP& c, double tt, D3 p1, D3 p2, const Fib64& f, Ival64& i) {
    double t_cc = (f.p1.z + c.center_height - p1.z) / (p2.z - p1.z);
    CCp cc{p1 + t_cc * (p2 - p1), OCL_CC_EDGE_CONE_BASE};
    return iv_update_if(i, tt, cc, p1, p2, true);
}
__device__ __forceinline__ bool cone_cone_cc(D3 tang, D3 tip, D3 base, D3 p1, D3 p2, const Fib64& f, Ival64& i) {
    double u, tt;
    if (xy_line_line(f.p1, f.p2, u, tang, tip, tt)) {
        if ((tt >= 0.0) && (tt <= 1.0)) {
            CCp cc{base + tt * (tip - base), OCL_CC_EDGE_CONE};
            cc.p.z = z_proj(cc.p, p1, p2);
            return iv_update_if(i, u, cc, p1, p2, true);
        }
    }
    return false;
}

__device__ inline bool cone_edge_push(const BasicP& c, const Fib64& f, Ival64& i, D3 p1, D3 p2) {
    bool result = false;
    if (zero_tol(p2.z - p1.z)) return false;
    double t_tip = (f.p1.z - p1.z) / (p2.z - p1.z);
    D3 p_tip = p1 + t_tip * (p2 - p1);
    double t_base = (f.p1.z + c.center_height - p1.z) / (p2.z - p1.z);
    D3 p_base = p1 + t_base * (p2 - p1);
    p_base.z = f.p1.z;
    double L = xynorm(p_base - p_tip);
    double d = xy_dist_line(p_base, f.p1, f.p2);
    if (d <= c.radius) {
        double dx = f.p2.x - f.p1.x;
        double dy = f.p2.y - f.p1.y;
        double dr = sqrt(sq(dx) + sq(dy));
        double det = (f.p1.x - p_base.x) * (f.p2.y - p_base.y) - (f.p2.x - p_base.x) * (f.p1.y - p_base.y);
        double discr = sq(c.radius) * sq(dr) - sq(det);
        if (discr >= 0.0) {
            if (discr == 0.0) {
                double x_tang = (det * dy) / sq(dr);
                double y_tang = -(det * dx) / sq(dr);
                D3 p_tang = d3(x_tang + p_base.x, y_tang + p_base.y, 0);
                if (cone_circle_cc(c, f_tval(f, p_tang), p1, p2, f, i)) result = true;
            } else {
                double x_pos = (det * dy + sgn(dy) * dx * sqrt(discr)) / sq(dr);
                double y_pos = (-det * dx + fabs(dy) * sqrt(discr)) / sq(dr);
                D3 cl_pos = d3(x_pos + p_base.x, y_pos + p_base.y, 0);
                double t_pos = f_tval(f, cl_pos);
                double x_neg = (det * dy - sgn(dy) * dx * sqrt(discr)) / sq(dr);
                double y_neg = (-det * dx - fabs(dy) * sqrt(discr)) / sq(dr);
                D3 cl_neg = d3(x_neg + p_base.x, y_neg + p_base.y, 0);
                double t_neg = f_tval(f, cl_neg);
                if (cone_circle_cc(c, t_pos, p1, p2, f, i)) result = true;
                if (cone_circle_cc(c, t_neg, p1, p2, f, i)) result = true;
            }
        }
    }
    if (L > c.radius) {
        D3 p_mid = 0.5 * (p_base + p_tip);
        p_mid.z = f.p1.z;
        double r_tang = L / 2;
        D3 pd = p_mid - p_base;
        pd.z = 0;
        double dist = xynorm(pd);
        bool case1 = (zero_tol(dist) && zero_tol(fabs(c.radius - r_tang)));
        bool case2 = (dist > (c.radius + r_tang));
        bool case3 = (dist < fabs(c.radius - r_tang));
        bool case4 = (zero_tol(dist - (c.radius + r_tang)));
        if (!(case1 || case2 || case3 || case4)) {
            double a = (-sq(r_tang) + sq(c.radius) + sq(dist)) / (2.0 * dist);
            D3 v2 = p_base + (a / dist) * pd;
            double h = sqrt(sq(c.radius) - sq(a));
            D3 ofs = d3(-pd.y * (h / dist), pd.x * (h / dist), 0);
            if (cone_cone_cc(v2 + ofs, p_tip, p_base, p1, p2, f, i)) result = true;
            if (cone_cone_cc(v2 - ofs, p_tip, p_base, p1, p2, f, i)) result = true;
        }
    }
    return result;
}

__device__ inline bool edge_push_basic(const BasicP& c, const Fib64& f, Ival64& i, const Tri64& t, const double* esin,
                                       int* capped) {
    bool result = false;
    for (int n = 0; n < 3; ++n) {
        D3 p1 = tri_p(t, n), p2 = tri_p(t, (n + 1) % 3);
        bool r = false;
        if (horiz_edge_push(c, f, i, p1, p2)) r = true;
        else {
            if (shaft_edge_push(c, f, i, p1, p2)) r = true;
            bool g = false;
            if (c.kind == OCL_CUTTER_BALL) g = ball_edge_push(c, f, i, p1, p2);
            else if (c.kind == OCL_CUTTER_BULL) g = bull_edge_push(c, f, i, p1, p2, esin[n], capped);
            else if (c.kind == OCL_CUTTER_CONE) g = cone_edge_push(c, f, i, p1, p2);
            if (g) r = true;
        }
        if (r) result = true;
    }
    return result;
}

__device__ __forceinline__ int height_index(const CutterP& c, double h) {
    for (int n = 0; n < c.nsub; ++n)
        if (comp_valid(c.heightvec, n, h)) return n;
    return c.nsub - 1;
}

// CompositeCutter vertex/facet/edge push: per sub-cutter on a shifted fiber,
// keep endpoints whose CC height belongs to that sub-cutter.
__device__ inline void comp_push(const CutterP& c, const Fib64& f, Ival64& i, const Tri64& t, const double* esin,
                                 int which, int* capped) {
    double ct[2 * OCL_GB300_MAX_SUB];
    CCp cc[2 * OCL_GB300_MAX_SUB];
    int nc = 0;
    for (int n = 0; n < c.nsub; ++n) {
        Ival64 ci;
        iv_init(ci);
        Fib64 cf = f;
        cf.p1.z = f.p1.z + c.zoffset[n];
        cf.p2.z = f.p2.z + c.zoffset[n];
        const BasicP& s = c.sub[n];
        bool hit;
        if (which == 0) hit = vertex_push_basic(s, cf, ci, t);
        else if (which == 1) hit = facet_push_basic(s, cf, ci, t);
        else hit = edge_push_basic(s, cf, ci, t, esin, capped);
        if (hit) {
            if (n == height_index(c, ci.ucc.p.z - f.p1.z)) { ct[nc] = ci.upper; cc[nc] = ci.ucc; ++nc; }
            if (n == height_index(c, ci.lcc.p.z - f.p1.z)) { ct[nc] = ci.lower; cc[nc] = ci.lcc; ++nc; }
        }
    }
    for (int k = 0; k < nc; ++k) iv_update(i, ct[k], cc[k]);
}

// esin: the triangle's three edge slopes (Mesh::d_edge_sin)
__device__ inline void push_triangle64(const CutterP& c, const Fib64& f, Ival64& i, const Tri64& t, const double* esin,
                                       int* capped) {
    if (c.kind == OCL_CUTTER_COMPOSITE) {
        comp_push(c, f, i, t, esin, 0, capped);
        comp_push(c, f, i, t, esin, 1, capped);
        comp_push(c, f, i, t, esin, 2, capped);
        return;
    }
    vertex_push_basic(c.b, f, i, t);
    facet_push_basic(c.b, f, i, t);
    edge_push_basic(c.b, f, i, t, esin, capped);
}

}  // namespace oclg
