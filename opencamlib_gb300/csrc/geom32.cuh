// geom32.cuh -- FP32 screening of (CL point, triangle) pairs.
//
// For one triangle the screen returns an interval [lo, hi] that contains the
// triangle's FP64 drop contribution as the reference defines it
// (MillingCutter::dropCutter, cutters/millingcutter.cpp:386-409: the facet
// contact when it lifts, else the best vertex/edge contact):
//   lo = -inf unless some contact is certain; hi = -inf when none is possible.
// Coordinates are local to the triangle's first vertex, so FP32 only carries
// differences of nearby points.  Every predicate that decides validity
// (point in triangle, CC inside an edge, distance <= radius) is evaluated
// with a margin: a clear decision is kept, a marginal one widens [lo, hi] to
// cover both outcomes.  Monotone functions (the cutter profile height(r)) are
// evaluated at the ends of the input's error interval instead of through a
// derivative.  The error budget E0 bounds the absolute position error of the
// local coordinates; it is set per mesh from its extent.
#pragma once
#include "common.cuh"

namespace oclg {

#define NEG_INF32 (-3.0e38f)

struct Iv {
    float lo, hi;
};
__device__ __forceinline__ Iv iv_none() { return Iv{NEG_INF32, NEG_INF32}; }
__device__ __forceinline__ void iv_max(Iv& a, Iv b) {
    a.lo = fmaxf(a.lo, b.lo);
    a.hi = fmaxf(a.hi, b.hi);
}

// FP32 copy of the cutter profile.
struct Prof32 {
    int kind;
    float R, r1, r2, inv_tan, center_height, length;
    float xynl, nl;  // xy_normal_length, normal_length
};

// height(r) in FP32 for r in [0, R] (monotone non-decreasing in r).
__device__ __forceinline__ float h32(const Prof32& c, float r) {
    r = fmaxf(r, 0.0f);
    switch (c.kind) {
    case OCL_CUTTER_CYL: return 0.0f;
    case OCL_CUTTER_BALL: {
        float a = fmaxf(c.R * c.R - r * r, 0.0f);
        return c.R - sqrtf(a);
    }
    case OCL_CUTTER_BULL: {
        if (r <= c.r1) return 0.0f;
        float q = fminf(r - c.r1, c.r2);
        return c.r2 - sqrtf(fmaxf(c.r2 * c.r2 - q * q, 0.0f));
    }
    case OCL_CUTTER_CONE: return r * c.inv_tan;
    }
    return 0.0f;
}
// derivative h'(r) (>= 0), used for the edge maximisation.
__device__ __forceinline__ float dh32(const Prof32& c, float r) {
    switch (c.kind) {
    case OCL_CUTTER_BALL: {
        float a = fmaxf(c.R * c.R - r * r, 1e-30f);
        return r * rsqrtf(a);
    }
    case OCL_CUTTER_BULL: {
        if (r <= c.r1) return 0.0f;
        float q = r - c.r1;
        float a = fmaxf(c.r2 * c.r2 - q * q, 1e-30f);
        return q * rsqrtf(a);
    }
    case OCL_CUTTER_CONE: return c.inv_tan;
    }
    return 0.0f;
}

// Vertex drop of one vertex at local (dx, dy) from the CL point, height pz.
__device__ __forceinline__ Iv vertex32(const Prof32& c, float dx, float dy, float pz, float E) {
    float q = sqrtf(dx * dx + dy * dy);
    float qlo = q - E, qhi = q + E;
    if (qlo > c.R) return iv_none();
    Iv r;
    r.hi = pz - h32(c, fmaxf(qlo, 0.0f)) + E;
    if (c.kind == OCL_CUTTER_CYL) {
        r.lo = (qhi < c.R) ? pz - E : NEG_INF32;
    } else {
        r.lo = (qhi <= c.R) ? pz - h32(c, qhi) - E : NEG_INF32;
    }
    return r;
}

// Barycentric position of local point (x, y) in the triangle (0, e1, e2):
// returns 1 = clearly inside, -1 = clearly outside, 0 = marginal.
__device__ __forceinline__ int inside32(const Tri32& t, float x, float y, float eps_b) {
    float det = t.e1[0] * t.e2[1] - t.e1[1] * t.e2[0];
    float inv = 1.0f / det;
    float u = (x * t.e2[1] - y * t.e2[0]) * inv;
    float v = (t.e1[0] * y - t.e1[1] * x) * inv;
    float w = 1.0f - u - v;
    float m = fminf(u, fminf(v, w));
    if (m > eps_b) return 1;
    if (m < -eps_b) return -1;
    return 0;
}

// Combine a candidate contact of value [vlo, vhi] with its validity state.
__device__ __forceinline__ Iv gate(int state, float vlo, float vhi) {
    if (state > 0) return Iv{vlo, vhi};
    if (state < 0) return iv_none();
    return Iv{NEG_INF32, vhi};
}

// Facet contact for cylindrical/spherical/toroidal cutters
// (MillingCutter::facetDrop, millingcutter.cpp:51-75), local frame.
__device__ __forceinline__ Iv facet32(const Prof32& c, const Tri32& t, float wx, float wy, float E, float eps_b) {
    uint32_t mode = t.flags & TF_FACET_MASK;
    if (mode == TF_FACET_NONE) return iv_none();
    if (mode == TF_FACET_HORIZ) {
        int s = inside32(t, wx, wy, eps_b);
        return gate(s, -E, E);
    }
    float nx = t.nn[0], ny = t.nn[1], nz = t.nn[2];
    float xyl = sqrtf(nx * nx + ny * ny);
    float xnx = nx / xyl, xny = ny / xyl;
    float rvx = c.xynl * xnx + c.nl * nx;
    float rvy = c.xynl * xny + c.nl * ny;
    float rvz = c.nl * nz;
    float ccx = wx - rvx, ccy = wy - rvy;
    float zc = -(nx * ccx + ny * ccy) / nz;
    float tip = zc + rvz - c.center_height;
    float err = E * (2.0f + (fabsf(nx) + fabsf(ny)) / nz);
    int s = inside32(t, ccx, ccy, eps_b);
    return gate(s, tip - err, tip + err);
}

// Edge contact in the canonical frame for one edge a->b (local coords).
// Cyl/ball/cone use the reference's closed forms (cylcutter.cpp:52-70,
// ballcutter.cpp:50-63, conecutter.cpp:109-135); for the bull the contact is
// the maximum of the concave function f(u) = z(u) - height(rho(u)) along the
// edge line, which is what the offset-ellipse solve of bullcutter.cpp:82-105
// finds; it is bracketed by bisection on f'.
// State of a CC point at xy distance ~r (error er) against a radius window
// [wlo, whi] (CompositeCutter::ccValidRadius): 1 inside, -1 outside, 0 unsure.
__device__ __forceinline__ int window_state(float r, float er, float wlo, float whi) {
    if (r - er >= wlo && r + er <= whi) return 1;
    if (r + er < wlo || r - er > whi) return -1;
    return 0;
}

// Edge contact of one cutter profile; with a window [wlo, whi] only a CC
// point whose xy distance from the CL may lie in it counts (a composite's
// sub-cutter: compositecutter.cpp:174-193).
__device__ inline Iv edge32(const Prof32& c, float ax, float ay, float az, float bx, float by, float bz, float wx, float wy,
                     float E, bool horiz, float wlo = -1.0f, float whi = 3.0e38f) {
    float dx = bx - ax, dy = by - ay;
    float L = sqrtf(dx * dx + dy * dy);
    float ux = dx / L, uy = dy / L;
    // CL relative to a
    float px = wx - ax, py = wy - ay;
    float d = fabsf(ux * py - uy * px);  // distance CL -> line
    if (d - E > c.R) return iv_none();
    float along = ux * px + uy * py;  // projection of CL on the line, from a
    float u1 = -along;                // a in canonical coordinates
    float u2 = L - along;             // b
    float m = (bz - az) / L;          // dz/du
    float dm = fminf(d, c.R);
    float s2 = c.R * c.R - dm * dm;
    float s = sqrtf(fmaxf(s2, 0.0f));
    float ccu, clz, err;
    int kind = c.kind;
    // E_u: uncertainty of the contact's position along the edge
    float Eu;
    if (kind == OCL_CUTTER_CYL) {
        // cc at +-s, pick the higher
        float z1 = az + (s - u1) * m, z2 = az + (-s - u1) * m;
        if (z1 > z2) { ccu = s; clz = z1; } else { ccu = -s; clz = z2; }
        // ds/dd = d/s: position error grows near tangency
        float dsdd = (s > 1e-6f * c.R) ? dm / s : 1e6f;
        Eu = E * (2.0f + dsdd);
        err = E * (2.0f + fabsf(m) * (1.0f + dsdd));
    } else if (kind == OCL_CUTTER_BALL) {
        float n0 = bz - az, n1 = -(u2 - u1);
        float nl = sqrtf(n0 * n0 + n1 * n1);
        n0 /= nl;
        n1 /= nl;
        if (n1 < 0) { n0 = -n0; n1 = -n1; }
        ccu = -s * n0;
        clz = az + (ccu - u1) * m + s * n1 - c.R;
        float dsdd = (s > 1e-6f * c.R) ? dm / s : 1e6f;
        Eu = E * (2.0f + dsdd);
        err = E * (3.0f + fabsf(m) + dsdd);
    } else if (kind == OCL_CUTTER_CONE) {
        float xu = s;
        float mu = (c.center_height / c.R) * xu / sqrtf(fmaxf(xu * xu + dm * dm, 1e-30f));
        float am = fabsf(m), amu = fabsf(mu);
        float sg = m < 0 ? -1.0f : 1.0f;
        // reference formula: hyperbola case uses length^2 (conecutter.cpp:122)
        float den = c.length * c.length - c.R * c.R * m * m;
        float cu_h = sg * sqrtf(fmaxf(c.R * c.R * m * m * dm * dm / den, 0.0f));
        float z_h = az + (cu_h - u1) * m - c.center_height + (c.R - sqrtf(cu_h * cu_h + dm * dm)) * c.inv_tan;
        float cu_r = sg * xu;
        float z_r = az + (cu_r - u1) * m - c.center_height;
        float dsdd = (s > 1e-6f * c.R) ? dm / s : 1e6f;
        float e0 = E * (3.0f + (am + c.inv_tan) * (2.0f + dsdd));
        float band = 1e-4f * (1.0f + amu);
        Iv r;
        if (am < amu - band) { ccu = cu_h; clz = z_h; }
        else if (am > amu + band) { ccu = cu_r; clz = z_r; }
        else {
            // marginal case split: cover both outcomes, CC test on both
            float lo = fminf(z_h, z_r) - e0, hi = fmaxf(z_h, z_r) + e0;
            float t1 = (cu_h - u1) / (u2 - u1), t2 = (cu_r - u1) / (u2 - u1);
            float et = (E * (2.0f + dsdd) + 1e-6f) / L;
            bool in1 = t1 > et && t1 < 1 - et, in2 = t2 > et && t2 < 1 - et;
            bool out1 = t1 < -et || t1 > 1 + et, out2 = t2 < -et || t2 > 1 + et;
            {
                const float ew = E * (3.0f + dsdd) + 1e-5f * c.R + 1e-6f;
                const int w1 = window_state(sqrtf(cu_h * cu_h + dm * dm), ew, wlo, whi);
                const int w2 = window_state(sqrtf(cu_r * cu_r + dm * dm), ew, wlo, whi);
                in1 = in1 && w1 > 0;
                in2 = in2 && w2 > 0;
                out1 = out1 || w1 < 0;
                out2 = out2 || w2 < 0;
            }
            r.lo = (in1 && in2) ? lo : NEG_INF32;
            r.hi = (out1 && out2) ? NEG_INF32 : hi;
            if (d + E > c.R && r.lo > NEG_INF32) r.lo = NEG_INF32;
            return r;
        }
        Eu = E * (2.0f + dsdd) + 1e-5f * c.R;
        err = e0;
    } else {  // bull
        if (horiz) {
            ccu = 0.0f;
            clz = az - h32(c, dm);
            Eu = E;
            err = E * 2.0f;
            // height is monotone: bracket by d +- E
            float hlo = h32(c, fminf(dm + E, c.R)), hhi = h32(c, fmaxf(dm - E, 0.0f));
            float tcc = (ccu - u1) / (u2 - u1);
            float et = (Eu + 1e-6f) / L;
            int st = (tcc > et && tcc < 1 - et) ? 1 : ((tcc < -et || tcc > 1 + et) ? -1 : 0);
            if (d + E > c.R && st > 0) st = 0;
            st = min(st, window_state(dm, 2.0f * E + 1e-6f, wlo, whi));
            return gate(st, az - hlo - 2.0f * E, az - hhi + 2.0f * E);
        }
        // maximise f(u) = az + (u - u1) m - h(sqrt(u^2 + d^2)) on |u| < s
        float lo_u = -s, hi_u = s;
        for (int it = 0; it < 20; ++it) {
            float mid = 0.5f * (lo_u + hi_u);
            float rho = sqrtf(mid * mid + dm * dm);
            float fp = m - dh32(c, rho) * (rho > 0 ? mid / rho : 0.0f);
            if (fp > 0) lo_u = mid; else hi_u = mid;
        }
        ccu = 0.5f * (lo_u + hi_u);
        float rho = sqrtf(ccu * ccu + dm * dm);
        clz = az + (ccu - u1) * m - h32(c, rho);
        // concave: f(max) <= f(lo_u) + f'(lo_u) (hi_u - lo_u)
        float rl = sqrtf(lo_u * lo_u + dm * dm);
        float fpl = fabsf(m - dh32(c, rl) * (rl > 0 ? lo_u / rl : 0.0f));
        float slack = fminf(fpl * (hi_u - lo_u), 1.0f);
        // sensitivity of the maximum to the line offset d
        float rd = rho > 1e-20f ? dm / rho : 0.0f;
        err = E * (3.0f + fabsf(m) + dh32(c, fminf(rho + E, c.R)) * (1.0f + rd)) + slack;
        float curv = 1.0f + dh32(c, fminf(rho + 4.0f * E, c.R));
        Eu = E * (2.0f + curv) + 1e-4f * c.r2;
    }
    // CC inside the segment (Point::isInside(p1,p2), param in [0,1])
    float tcc = (ccu - u1) / (u2 - u1);
    float et = (Eu + 1e-6f) / L;
    int st = (tcc > et && tcc < 1 - et) ? 1 : ((tcc < -et || tcc > 1 + et) ? -1 : 0);
    if (d + E > c.R && st > 0) st = 0;  // d <= radius is marginal
    st = min(st, window_state(sqrtf(ccu * ccu + dm * dm), Eu + E + 1e-6f, wlo, whi));
    return gate(st, clz - err, clz + err);
}

// The bull's three edge contacts of one triangle at once (same bounds as
// edge32): the three maximisations along the edge lines run interleaved,
// 10 bisection steps each, then one Newton step inside the bracket; the
// concave maximum is bounded by the tangent at the final point over the
// bracket, and the contact position's uncertainty includes the bracket.
// Horizontal and skipped edges take edge32's paths.
__device__ inline void bull_edges32(const Prof32& c, const float* px, const float* py, const float* pz, uint32_t flags,
                                    float wx, float wy, float E, Iv* out) {
    float u1[3], u2[3], m[3], dm[3], lo_u[3], hi_u[3], L[3];
    bool run[3];
#pragma unroll
    for (int n = 0; n < 3; ++n) {
        out[n] = iv_none();
        run[n] = false;
        u1[n] = u2[n] = m[n] = dm[n] = lo_u[n] = hi_u[n] = 0.0f;
        L[n] = 1.0f;
        if (flags & (TF_EDGE0_SKIP << n)) continue;
        const int k = (n + 1) % 3;
        if (flags & (TF_EDGE0_HORIZ << n)) {
            out[n] = edge32(c, px[n], py[n], pz[n], px[k], py[k], pz[k], wx, wy, E, true);
            continue;
        }
        const float dx = px[k] - px[n], dy = py[k] - py[n];
        L[n] = sqrtf(dx * dx + dy * dy);
        const float ux = dx / L[n], uy = dy / L[n];
        const float qx = wx - px[n], qy = wy - py[n];
        const float d = fabsf(ux * qy - uy * qx);
        if (d - E > c.R) continue;
        const float along = ux * qx + uy * qy;
        u1[n] = -along;
        u2[n] = L[n] - along;
        m[n] = (pz[k] - pz[n]) / L[n];
        dm[n] = fminf(d, c.R);
        const float s = sqrtf(fmaxf(c.R * c.R - dm[n] * dm[n], 0.0f));
        lo_u[n] = -s;
        hi_u[n] = s;
        run[n] = true;
    }
    // maximise f(u) = az + (u - u1) m - h(sqrt(u^2 + d^2)) on |u| < s
    for (int it = 0; it < 10; ++it) {
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            const float mid = 0.5f * (lo_u[n] + hi_u[n]);
            const float rho = sqrtf(mid * mid + dm[n] * dm[n]);
            const float fp = m[n] - dh32(c, rho) * (rho > 0 ? mid / rho : 0.0f);
            if (fp > 0) lo_u[n] = mid; else hi_u[n] = mid;
        }
    }
#pragma unroll
    for (int n = 0; n < 3; ++n) {
        if (!run[n]) continue;
        // one Newton step on f' from the bracket's middle, kept inside it
        float ccu = 0.5f * (lo_u[n] + hi_u[n]);
        {
            const float rho = sqrtf(ccu * ccu + dm[n] * dm[n]);
            const float q = rho - c.r1;
            if (q > 0.0f && rho > 0.0f) {
                const float a = fmaxf(c.r2 * c.r2 - q * q, 1e-30f);
                const float ra = rsqrtf(a);
                const float hp = q * ra, hpp = c.r2 * c.r2 * ra * ra * ra;
                const float w = ccu / rho;
                const float fp = m[n] - hp * w;
                const float fpp = -(hpp * w * w + hp * dm[n] * dm[n] / (rho * rho * rho));
                if (fpp < 0.0f) ccu = fminf(fmaxf(ccu - fp / fpp, lo_u[n]), hi_u[n]);
            }
        }
        const float rho = sqrtf(ccu * ccu + dm[n] * dm[n]);
        const float clz = pz[n] + (ccu - u1[n]) * m[n] - h32(c, rho);
        const float fpx = fabsf(m[n] - dh32(c, rho) * (rho > 0 ? ccu / rho : 0.0f));
        const float width = hi_u[n] - lo_u[n];
        const float slack = fminf(fpx * width, 1.0f);
        const float rd = rho > 1e-20f ? dm[n] / rho : 0.0f;
        const float err = E * (3.0f + fabsf(m[n]) + dh32(c, fminf(rho + E, c.R)) * (1.0f + rd)) + slack;
        const float curv = 1.0f + dh32(c, fminf(rho + 4.0f * E, c.R));
        const float Eu = E * (2.0f + curv) + 1e-4f * c.r2 + width;
        // CC inside the segment (Point::isInside(p1,p2), param in [0,1])
        const float tcc = (ccu - u1[n]) / (u2[n] - u1[n]);
        const float et = (Eu + 1e-6f) / L[n];
        int st = (tcc > et && tcc < 1 - et) ? 1 : ((tcc < -et || tcc > 1 + et) ? -1 : 0);
        if (dm[n] + E > c.R && st > 0) st = 0;
        out[n] = gate(st, clz - err, clz + err);
    }
}

// One bull edge in the canonical frame of edge32: f(u) = az + (u - u1) m -
// h(sqrt(u^2 + dm^2)) is concave on |u| < s, and the reference's contact is
// its maximiser u* when that lies on the segment [u1, u2].  The FP64 CC lies
// within Eu0 = E (3 + h'(rho)) + 1e-4 r2 of u*, so only u* in
// [u1 - M, u2 + M] with M >= Eu0 can give a contact: the search bracket
// [A, B] is that range (within the chord), and the whole chord where h' is
// too steep near the segment for a short margin.
struct BullEdge32 {
    float u1, u2, m, dm, L, A, B, az;
};

// f'(u) times rho (same sign as f'; no division).  At rho = 0 -- the CL
// point on the edge line (dm = 0) and u = 0 -- the product vanishes, but there
// f' = m (the flat bottom has h' = 0), so m itself is returned: a zero would
// stop the bisection at u = 0, short of the maximiser on the torus.
__device__ __forceinline__ float bull_fp32(const Prof32& c, const BullEdge32& b, float u) {
    const float rho = sqrtf(u * u + b.dm * b.dm);
    return rho > 0.0f ? b.m * rho - dh32(c, rho) * u : b.m;
}

// Edge n of the triangle (local vertices px/py/pz); false: no contact.
__device__ __forceinline__ bool bull_edge_setup32(const Prof32& c, float ax, float ay, float az, float bx, float by,
                                                  float bz, float wx, float wy, float E, BullEdge32& b) {
    const float dx = bx - ax, dy = by - ay;
    b.L = sqrtf(dx * dx + dy * dy);
    const float ux = dx / b.L, uy = dy / b.L;
    const float qx = wx - ax, qy = wy - ay;
    const float d = fabsf(ux * qy - uy * qx);
    if (d - E > c.R) return false;
    const float along = ux * qx + uy * qy;
    b.u1 = -along;
    b.u2 = b.L - along;
    b.m = (bz - az) / b.L;
    b.dm = fminf(d, c.R);
    b.az = az;
    // half chord of the disc at the largest line distance d may stand for
    const float dl = fmaxf(d - E, 0.0f);
    const float s = sqrtf(fmaxf(c.R * c.R - dl * dl, 0.0f));
    const float r1 = sqrtf(b.u1 * b.u1 + b.dm * b.dm), r2 = sqrtf(b.u2 * b.u2 + b.dm * b.dm);
    // rho on [u1 - M, u2 + M] stays below max(r1, r2) + M
    const float M = E * (3.0f + dh32(c, fminf(fmaxf(r1, r2) + 4.0f * E + 0.01f, c.R))) + 1e-4f * c.r2 + 1e-3f;
    if (M <= 0.01f) {
        b.A = fmaxf(b.u1 - M, -s);
        b.B = fminf(b.u2 + M, s);
    } else {
        b.A = -s;
        b.B = s;
    }
    return b.A < b.B;
}

// true when the maximiser may lie in [A, B] (f' does not change sign outside)
__device__ __forceinline__ bool bull_edge_open32(const Prof32& c, const BullEdge32& b) {
    return !(bull_fp32(c, b, b.A) < 0.0f) && !(bull_fp32(c, b, b.B) > 0.0f);
}

// Bound of the edge contact with the maximiser bracketed in [A, B]: 8
// bisection steps, one Newton step inside the bracket, the concave maximum
// bounded by the tangent over the bracket (as bull_edges32).
__device__ inline Iv bull_edge_solve32(const Prof32& c, const BullEdge32& b, float E) {
    float lo_u = b.A, hi_u = b.B;
    for (int it = 0; it < 8; ++it) {
        const float mid = 0.5f * (lo_u + hi_u);
        if (bull_fp32(c, b, mid) > 0) lo_u = mid; else hi_u = mid;
    }
    float ccu = 0.5f * (lo_u + hi_u);
    {
        const float rho = sqrtf(ccu * ccu + b.dm * b.dm);
        const float q = rho - c.r1;
        if (q > 0.0f && rho > 0.0f) {
            const float a = fmaxf(c.r2 * c.r2 - q * q, 1e-30f);
            const float ra = rsqrtf(a);
            const float hp = q * ra, hpp = c.r2 * c.r2 * ra * ra * ra;
            const float w = ccu / rho;
            const float fp = b.m - hp * w;
            const float fpp = -(hpp * w * w + hp * b.dm * b.dm / (rho * rho * rho));
            if (fpp < 0.0f) ccu = fminf(fmaxf(ccu - fp / fpp, lo_u), hi_u);
        }
    }
    const float rho = sqrtf(ccu * ccu + b.dm * b.dm);
    const float clz = b.az + (ccu - b.u1) * b.m - h32(c, rho);
    const float fpx = fabsf(b.m - dh32(c, rho) * (rho > 0 ? ccu / rho : 0.0f));
    const float width = hi_u - lo_u;
    const float slack = fminf(fpx * width, 1.0f);
    const float rd = rho > 1e-20f ? b.dm / rho : 0.0f;
    const float err = E * (3.0f + fabsf(b.m) + dh32(c, fminf(rho + E, c.R)) * (1.0f + rd)) + slack;
    const float curv = 1.0f + dh32(c, fminf(rho + 4.0f * E, c.R));
    const float Eu = E * (2.0f + curv) + 1e-4f * c.r2 + width;
    const float tcc = (ccu - b.u1) / (b.u2 - b.u1);
    const float et = (Eu + 1e-6f) / b.L;
    int st = (tcc > et && tcc < 1 - et) ? 1 : ((tcc < -et || tcc > 1 + et) ? -1 : 0);
    if (b.dm + E > c.R && st > 0) st = 0;
    return gate(st, clz - err, clz + err);
}

// End points of edge n (0: v0-v1, 1: v1-v2, 2: v2-v0) of t, local frame,
// selected rather than indexed.
__device__ __forceinline__ void tri_edge32(const Tri32& t, int n, float& ax, float& ay, float& az, float& bx,
                                           float& by, float& bz) {
    ax = n == 0 ? 0.0f : (n == 1 ? t.e1[0] : t.e2[0]);
    ay = n == 0 ? 0.0f : (n == 1 ? t.e1[1] : t.e2[1]);
    az = n == 0 ? 0.0f : (n == 1 ? t.e1[2] : t.e2[2]);
    bx = n == 0 ? t.e1[0] : (n == 1 ? t.e2[0] : 0.0f);
    by = n == 0 ? t.e1[1] : (n == 1 ? t.e2[1] : 0.0f);
    bz = n == 0 ? t.e1[2] : (n == 1 ? t.e2[2] : 0.0f);
}

// Warp-collective bull screen, one (point, triangle) pair per lane (have:
// the lane holds one; every lane of the warp calls it).  Same effect interval
// as screen_triangle; the edges whose maximiser may lie on the segment are
// gathered from all lanes and searched one per lane, so the warp runs the
// bisection only for those (most edges' maximisers lie off the segment).
__device__ inline Iv screen_bull_warp(const Prof32& c, const Tri32* __restrict__ t32, uint32_t tri, const Tri32& t,
                                      float wx, float wy, float E, bool have) {
    const int lane = threadIdx.x & 31;
    Iv best = iv_none();
    unsigned need = 0;  // bit n: edge n's maximiser may lie on the segment
    if (have) {
        const float eps_b = E * 4.0f * t.bary_scale + 1e-6f;
        best = vertex32(c, -wx, -wy, 0.0f, E);
        iv_max(best, vertex32(c, t.e1[0] - wx, t.e1[1] - wy, t.e1[2], E));
        iv_max(best, vertex32(c, t.e2[0] - wx, t.e2[1] - wy, t.e2[2], E));
        // one copy of the edge test (instruction cache): the edges' end
        // points are selected, not indexed
#pragma unroll 1
        for (int n = 0; n < 3; ++n) {
            if (t.flags & (TF_EDGE0_SKIP << n)) continue;
            float ax, ay, az, bx, by, bz;
            tri_edge32(t, n, ax, ay, az, bx, by, bz);
            if (t.flags & (TF_EDGE0_HORIZ << n)) {
                iv_max(best, edge32(c, ax, ay, az, bx, by, bz, wx, wy, E, true));
                continue;
            }
            BullEdge32 b;
            if (bull_edge_setup32(c, ax, ay, az, bx, by, bz, wx, wy, E, b) && bull_edge_open32(c, b)) need |= 1u << n;
        }
        iv_max(best, facet32(c, t, wx, wy, E, eps_b));
    }
    const unsigned m0 = __ballot_sync(0xffffffffu, need & 1u);
    const unsigned m1 = __ballot_sync(0xffffffffu, need & 2u);
    const unsigned m2 = __ballot_sync(0xffffffffu, need & 4u);
    const int c0 = __popc(m0), c01 = c0 + __popc(m1), total = c01 + __popc(m2);
    const unsigned below = (1u << lane) - 1u;
    // this lane's edges in the gathered order (n-major)
    const int q0 = __popc(m0 & below), q1 = c0 + __popc(m1 & below), q2 = c01 + __popc(m2 & below);
    for (int r0 = 0; r0 < total; r0 += 32) {
        const int q = r0 + lane;
        int n = 0, owner = lane;
        if (q < total) {
            if (q < c0) owner = __fns(m0, 0, q + 1);
            else if (q < c01) { n = 1; owner = __fns(m1, 0, q - c0 + 1); }
            else { n = 2; owner = __fns(m2, 0, q - c01 + 1); }
        }
        const uint32_t otri = __shfl_sync(0xffffffffu, tri, owner);
        const float owx = __shfl_sync(0xffffffffu, wx, owner), owy = __shfl_sync(0xffffffffu, wy, owner);
        Iv r = iv_none();
        if (q < total) {
            const Tri32 to = t32[otri];
            float ax, ay, az, bx, by, bz;
            tri_edge32(to, n, ax, ay, az, bx, by, bz);
            BullEdge32 b;
            bull_edge_setup32(c, ax, ay, az, bx, by, bz, owx, owy, E, b);
            r = bull_edge_solve32(c, b, E);
        }
        // each owner takes its edges' results back
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int qk = k == 0 ? q0 : (k == 1 ? q1 : q2);
            const bool mine = ((need >> k) & 1u) && qk >= r0 && qk < r0 + 32;
            const int src = mine ? qk - r0 : lane;
            const float lo = __shfl_sync(0xffffffffu, r.lo, src), hi = __shfl_sync(0xffffffffu, r.hi, src);
            if (mine) iv_max(best, Iv{lo, hi});
        }
    }
    return best;
}

// Whole-triangle screen for the basic cutters, local frame (relative to v0).
// Returns the interval of the triangle's effect on the running z
// (dropCutter applied to a CL point already at some height Z >= z0).
// qthr receives the lowest running height at which the reference's branch
// choice for this triangle could change (cone tip/rim short-circuits), or
// +inf when the triangle's effect is a plain max (order-independent); qthr_hi
// the highest one.  Below qthr the effect does not depend on the running
// height Z beyond max(Z, c); above qthr_hi it is max(Z, vertex/edge contacts).
__device__ inline Iv screen_triangle(const Prof32& c, const Tri32& t, float wx, float wy, float E, float z0_rel,
                                     float& qthr, float& qthr_hi) {
    const float eps_b = E * 4.0f * t.bary_scale + 1e-6f;
    qthr = 3.0e38f;
    qthr_hi = NEG_INF32;
    // vertices
    Iv best = vertex32(c, -wx, -wy, 0.0f, E);
    iv_max(best, vertex32(c, t.e1[0] - wx, t.e1[1] - wy, t.e1[2], E));
    iv_max(best, vertex32(c, t.e2[0] - wx, t.e2[1] - wy, t.e2[2], E));
    // edges
    const float px[3] = {0.0f, t.e1[0], t.e2[0]};
    const float py[3] = {0.0f, t.e1[1], t.e2[1]};
    const float pz[3] = {0.0f, t.e1[2], t.e2[2]};
    if (c.kind == OCL_CUTTER_BULL) {
        Iv ev[3];
        bull_edges32(c, px, py, pz, t.flags, wx, wy, E, ev);
        iv_max(best, ev[0]);
        iv_max(best, ev[1]);
        iv_max(best, ev[2]);
    } else {
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            if (t.flags & (TF_EDGE0_SKIP << n)) continue;
            const int k = (n + 1) % 3;
            const bool horiz = (t.flags & (TF_EDGE0_HORIZ << n)) != 0;
            iv_max(best, edge32(c, px[n], py[n], pz[n], px[k], py[k], pz[k], wx, wy, E, horiz));
        }
    }
    if (c.kind == OCL_CUTTER_CONE) {
        // ConeCutter::facetDrop (conecutter.cpp:70-105): the tip contact, when
        // it lifts, ends the triangle; otherwise the rim, otherwise vertices
        // and edges.  With a running height Z: tip if Z < tip, rim if
        // tip <= Z < rim, else max(Z, vertex/edge).
        uint32_t mode = t.flags & TF_FACET_MASK;
        if (mode == TF_FACET_NONE) return best;
        Iv tip, rim;
        int st_tip, st_rim;
        if (mode == TF_FACET_HORIZ) {
            st_tip = inside32(t, wx, wy, eps_b);
            tip = Iv{-E, E};
            st_rim = -1;
            rim = iv_none();
        } else {
            float nx = t.nn[0], ny = t.nn[1], nz = t.nn[2];
            float slope = (fabsf(nx) + fabsf(ny)) / nz;
            float xyl = sqrtf(nx * nx + ny * ny);
            float zt = -(nx * wx + ny * wy) / nz;
            float et = E * (2.0f + slope);
            tip = Iv{zt - et, zt + et};
            st_tip = inside32(t, wx, wy, eps_b);
            float rx = wx - c.R * nx / xyl, ry = wy - c.R * ny / xyl;
            float zr = -(nx * rx + ny * ry) / nz - c.length;
            float er = E * (2.0f + slope * 2.0f);
            rim = Iv{zr - er, zr + er};
            st_rim = inside32(t, rx, ry, eps_b);
        }
        // a contact at or below the start height never lifts
        if (st_tip >= 0 && tip.hi <= z0_rel) st_tip = -1;
        if (st_tip > 0 && !(tip.lo > z0_rel)) st_tip = 0;
        if (st_rim >= 0 && rim.hi <= z0_rel) st_rim = -1;
        if (st_rim > 0 && !(rim.lo > z0_rel)) st_rim = 0;
        float lo_after_tip =
            st_rim > 0 ? rim.lo : (st_rim < 0 ? best.lo : fminf(rim.lo, best.lo));
        Iv r;
        r.lo = st_tip > 0 ? tip.lo : (st_tip < 0 ? lo_after_tip : fminf(tip.lo, lo_after_tip));
        r.hi = best.hi;
        if (st_tip >= 0) r.hi = fmaxf(r.hi, tip.hi);
        if (st_rim >= 0) r.hi = fmaxf(r.hi, rim.hi);
        if (st_tip >= 0 && fmaxf(best.hi, st_rim >= 0 ? rim.hi : NEG_INF32) > tip.lo) {
            qthr = fminf(qthr, tip.lo);
            qthr_hi = fmaxf(qthr_hi, tip.hi);
        }
        if (st_rim >= 0 && best.hi > rim.lo) {
            qthr = fminf(qthr, rim.lo);
            qthr_hi = fmaxf(qthr_hi, rim.hi);
        }
        return r;
    }
    // cyl/ball/bull: a lifting facet contact is the highest contact of the
    // plane, so the effect is the maximum of all certain contacts.
    iv_max(best, facet32(c, t, wx, wy, E, eps_b));
    return best;
}


// Composite cutters (CompositeCutter, compositecutter.cpp:58-193).
struct Comp32 {
    int nsub;
    Prof32 sub[OCL_GB300_MAX_SUB];
    float zoff[OCL_GB300_MAX_SUB];
    float rlim[OCL_GB300_MAX_SUB];  // radiusvec
    float R;
    // radius window of sub-cutter n, [radiusvec[n-1] - 1e-6, radiusvec[n] + 1e-6]
    // (the reference's doubles), rounded inward (in) and outward (out) to float
    float wlo_in[OCL_GB300_MAX_SUB], whi_in[OCL_GB300_MAX_SUB];
    float wlo_out[OCL_GB300_MAX_SUB], whi_out[OCL_GB300_MAX_SUB];
};

// Window state of a CC at xy distance dist (error ed) for sub-cutter n:
// 1 certainly inside, -1 certainly outside, 0 unsure.
__device__ __forceinline__ int comp_window(const Comp32& c, int n, float dist, float ed) {
    const float e = ed + dist * 1.2e-7f;  // rounding of dist +- ed
    if (dist - e >= c.wlo_in[n] && dist + e <= c.whi_in[n]) return 1;
    if (dist + e < c.wlo_out[n] || dist - e > c.whi_out[n]) return -1;
    return 0;
}

// composite height(r): the first sub-cutter whose radius window holds r
__device__ __forceinline__ float hcomp32(const Comp32& c, float r) {
    r = fmaxf(r, 0.0f);
    int idx = 0;
    for (int n = 0; n < c.nsub; ++n)
        if (r <= c.rlim[n] + 1e-6f) { idx = n; break; }
    return h32(c.sub[idx], fminf(r, c.sub[idx].R)) + c.zoff[idx];
}

// Screen of one triangle for a composite cutter.
// The composite facet drop (compositecutter.cpp:152-172) ends the triangle
// as soon as a sub-cutter's facet contact lies in that sub-cutter's radius
// window and lifts; that contact need not be the cutter's highest contact with
// the plane (e.g. the shaft on a facet steeper than the cone), so:
//   lo: the facet outcome if one facet contact certainly lifts, else the
//       lower of (vertex contacts with the composite profile) and every facet
//       contact that may end the triangle;
//   hi: every contact of the composite profile with a vertex, and every facet
//       or edge contact of a sub-cutter whose CC may lie in that sub-cutter's
//       radius window (contacts outside it never lift the composite);
//   qthr: the lowest facet contact that may end the triangle while another
//       contact could be higher (its branch depends on the running height),
//       and the tip of a cone sub-cutter outside the centre window (while the
//       running height is below it the tip lifts, fails the window and hides
//       that sub-cutter's rim);
//   qthr_hi: the highest of those contacts (above it no facet contact lifts
//       and the effect is max(Z, vertex/edge contacts)).
__device__ inline Iv screen_composite(const Comp32& c, const Tri32& t, float wx, float wy, float E, float z0_rel,
                                      float& qthr, float& qthr_hi) {
    const float eps_b = E * 4.0f * t.bary_scale + 1e-6f;
    qthr = 3.0e38f;
    qthr_hi = NEG_INF32;
    const float px[3] = {0.0f, t.e1[0], t.e2[0]};
    const float py[3] = {0.0f, t.e1[1], t.e2[1]};
    const float pz[3] = {0.0f, t.e1[2], t.e2[2]};
    float vlo = NEG_INF32, ohi = NEG_INF32;  // vertex-path lower bound; highest non-facet contact
    // vertices, composite profile (monotone in r)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float dx = px[k] - wx, dy = py[k] - wy;
        float q = sqrtf(dx * dx + dy * dy);
        float qlo = q - E, qhi = q + E;
        if (qlo > c.R) continue;
        ohi = fmaxf(ohi, pz[k] - hcomp32(c, fmaxf(qlo, 0.0f)) + E);
        if (qhi <= c.R) vlo = fmaxf(vlo, pz[k] - hcomp32(c, qhi) - E);
    }
    // edges: a sub-cutter's edge contact counts only when its CC lies in the
    // sub-cutter's radius window (its highest edge contact's CC is tested, so
    // the in-window contacts bound what it can add)
    for (int n = 0; n < c.nsub; ++n) {
        const Prof32& s = c.sub[n];
        const float zo = c.zoff[n];
        const float wlo = (n == 0 ? 0.0f : c.rlim[n - 1]) - 1e-6f, whi = c.rlim[n] + 1e-6f;
        // one copy of the contact model per sub-cutter (instruction cache):
        // the edges' end points are selected, not indexed
#pragma unroll 1
        for (int e = 0; e < 3; ++e) {
            if (t.flags & (TF_EDGE0_SKIP << e)) continue;
            const float ax = e == 0 ? 0.0f : (e == 1 ? t.e1[0] : t.e2[0]);
            const float ay = e == 0 ? 0.0f : (e == 1 ? t.e1[1] : t.e2[1]);
            const float az = e == 0 ? 0.0f : (e == 1 ? t.e1[2] : t.e2[2]);
            const float bx = e == 0 ? t.e1[0] : (e == 1 ? t.e2[0] : 0.0f);
            const float by = e == 0 ? t.e1[1] : (e == 1 ? t.e2[1] : 0.0f);
            const float bz = e == 0 ? t.e1[2] : (e == 1 ? t.e2[2] : 0.0f);
            const bool horiz = (t.flags & (TF_EDGE0_HORIZ << e)) != 0;
            Iv v = edge32(s, ax, ay, az, bx, by, bz, wx, wy, E, horiz, wlo, whi);
            if (v.hi > NEG_INF32) ohi = fmaxf(ohi, v.hi - zo + E);
        }
    }
    // facet contacts of the sub-cutters, with their window/inside states
    const uint32_t mode = t.flags & TF_FACET_MASK;
    // Facet contacts of the sub-cutters (CompositeCutter::facetDrop,
    // compositecutter.cpp:152-172), one slot per (sub-cutter, tip/rim):
    //   pv    value of a contact that may lift the composite (else +inf);
    //   f_certain: the best contact that lifts whenever it is above Z.
    // For Z below f_certain the facet ends the triangle with the highest
    // valid contact, whatever Z is: contacts below f_certain branch nothing.
    constexpr int NS = 2 * OCL_GB300_MAX_SUB;
    float pv[NS];
    float rimv[OCL_GB300_MAX_SUB], tlo[OCL_GB300_MAX_SUB], thi[OCL_GB300_MAX_SUB];
#pragma unroll
    for (int k = 0; k < NS; ++k) pv[k] = 3.0e38f;
#pragma unroll
    for (int k = 0; k < OCL_GB300_MAX_SUB; ++k) {
        rimv[k] = NEG_INF32;
        tlo[k] = 3.0e38f;
        thi[k] = NEG_INF32;
    }
    float f_certain = NEG_INF32;
    float f_hi = NEG_INF32;
    float ev = E * 3.0f;
    if (mode != TF_FACET_NONE) {
        const float nx = t.nn[0], ny = t.nn[1], nz = t.nn[2];
        const float xyl = sqrtf(nx * nx + ny * ny);
        const float slope = (mode == TF_FACET_HORIZ) ? 0.0f : (fabsf(nx) + fabsf(ny)) / nz;
        ev = E * (3.0f + 2.0f * slope);
#pragma unroll
        for (int n = 0; n < OCL_GB300_MAX_SUB; ++n) {
            if (n >= c.nsub) break;
            const Prof32& s = c.sub[n];
            const float zo = c.zoff[n];
            // up to two candidate contacts per sub-cutter: value, window state,
            // inside state, and whether it certainly lifts whenever it is above Z
            float val[2] = {0.0f, 0.0f};
            int win[2] = {-1, -1}, ins[2] = {-1, -1};
            bool sure[2] = {true, true};
            if (s.kind == OCL_CUTTER_CONE) {
                // ConeCutter::facetDrop (conecutter.cpp:70-105): the tip, when it
                // lifts, ends the sub-cutter's drop and hides its rim
                const float zt = (mode == TF_FACET_HORIZ) ? 0.0f : -(nx * wx + ny * wy) / nz;
                const int st_tip = inside32(t, wx, wy, eps_b);
                const float vt = zt - zo;
                const bool tip_may_lift = st_tip >= 0 && vt + ev > z0_rel;
                if (st_tip >= 0) {
                    val[0] = vt; win[0] = comp_window(c, n, 0.0f, 0.0f); ins[0] = st_tip;
                }
                if (mode == TF_FACET_GENERAL) {
                    const float rx = wx - s.R * nx / xyl, ry = wy - s.R * ny / xyl;
                    const int st_rim = inside32(t, rx, ry, eps_b);
                    if (st_rim >= 0) {
                        // the rim CC lies at xy distance R (the reference's
                        // FP64 arithmetic, exact to ~1e-14)
                        val[1] = -(nx * rx + ny * ry) / nz - s.length - zo;
                        win[1] = comp_window(c, n, s.R, 1e-9f + s.R * 1e-9f);
                        ins[1] = st_rim;
                        sure[1] = !tip_may_lift;  // hidden while Z is below the tip
                        // below the tip the rim is not tried: a branch at the tip
                        if (tip_may_lift && win[1] >= 0 && val[1] + ev > z0_rel) {
                            rimv[n] = val[1];
                            tlo[n] = vt - ev;
                            thi[n] = vt + ev;
                        }
                    }
                }
            } else {
                // MillingCutter::facetDrop (millingcutter.cpp:51-75): CC at
                // cl - (xy_normal_length * xyn + normal_length * n), whose xy
                // distance from the CL is xy_normal_length + normal_length |n_xy|
                float ccx, ccy, tip, dist, ed;
                if (mode == TF_FACET_HORIZ) {
                    ccx = wx; ccy = wy; tip = 0.0f;
                    dist = 0.0f;
                    ed = 0.0f;
                } else {
                    float xnx = nx / xyl, xny = ny / xyl;
                    float rvx = s.xynl * xnx + s.nl * nx, rvy = s.xynl * xny + s.nl * ny, rvz = s.nl * nz;
                    ccx = wx - rvx; ccy = wy - rvy;
                    tip = -(nx * ccx + ny * ccy) / nz + rvz - s.center_height;
                    dist = s.xynl + s.nl * xyl;
                    ed = s.nl * xyl * 3e-7f + 1e-9f;
                }
                int st = inside32(t, ccx, ccy, eps_b);
                if (st >= 0) {
                    val[0] = tip - zo; win[0] = comp_window(c, n, dist, ed); ins[0] = st;
                }
            }
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                // radius window (CompositeCutter::ccValidRadius, compositecutter.cpp:86-102)
                if (ins[k] < 0 || win[k] < 0) continue;  // never lifts the composite
                f_hi = fmaxf(f_hi, val[k] + ev);
                if (val[k] + ev <= z0_rel) continue;  // never above the start height
                pv[2 * n + k] = val[k];
                if (win[k] > 0 && ins[k] > 0 && sure[k] && val[k] - ev > z0_rel)
                    f_certain = fmaxf(f_certain, val[k] - ev);
            }
        }
    }
    // branch points: the contacts that may lie above f_certain, and the tips
    // that hide a rim which may lie above it
    bool f_possible = false;
    float f_minlo = 3.0e38f, f_maxhi = NEG_INF32;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        if (pv[k] < 3.0e38f && pv[k] + ev > f_certain) {
            f_possible = true;
            f_minlo = fminf(f_minlo, pv[k] - ev);
            f_maxhi = fmaxf(f_maxhi, pv[k] + ev);
        }
    }
    float tip_thr = 3.0e38f, tip_thr_hi = NEG_INF32;
#pragma unroll
    for (int k = 0; k < OCL_GB300_MAX_SUB; ++k) {
        if (rimv[k] + ev > f_certain && tlo[k] < 3.0e38f) {
            tip_thr = fminf(tip_thr, tlo[k]);
            tip_thr_hi = fmaxf(tip_thr_hi, thi[k]);
        }
    }
    Iv r;
    r.hi = fmaxf(ohi, f_hi);
    if (f_certain > NEG_INF32) r.lo = f_certain;
    else if (f_possible) r.lo = fminf(vlo, f_minlo);
    else r.lo = vlo;
    if (f_possible && ohi > f_minlo) {
        qthr = f_minlo;
        qthr_hi = f_maxhi;
    }
    if (tip_thr < 3.0e38f) {
        qthr = fminf(qthr, tip_thr);
        qthr_hi = fmaxf(qthr_hi, tip_thr_hi);
    }
    return r;
}

// Upper bound (composite frame, local to the triangle's first vertex) of the
// facet contacts of sub-cutter n that may lift the composite: contacts that
// may lie inside the triangle and in the sub-cutter's radius window, with the
// error bounds of screen_composite.  Whatever contact the sub-cutter's facet
// drop ends on, it lifts the composite only if it is one of these.
__device__ inline float comp_facet_hi32(const Comp32& c, const Tri32& t, int n, float wx, float wy, float E) {
    const uint32_t mode = t.flags & TF_FACET_MASK;
    if (mode == TF_FACET_NONE) return NEG_INF32;
    const float eps_b = E * 4.0f * t.bary_scale + 1e-6f;
    const float nx = t.nn[0], ny = t.nn[1], nz = t.nn[2];
    const float xyl = sqrtf(nx * nx + ny * ny);
    const float slope = (mode == TF_FACET_HORIZ) ? 0.0f : (fabsf(nx) + fabsf(ny)) / nz;
    const float ev = E * (3.0f + 2.0f * slope);
    const Prof32& s = c.sub[n];
    const float zo = c.zoff[n];
    float hi = NEG_INF32;
    if (s.kind == OCL_CUTTER_CONE) {
        const float zt = (mode == TF_FACET_HORIZ) ? 0.0f : -(nx * wx + ny * wy) / nz;
        if (inside32(t, wx, wy, eps_b) >= 0 && comp_window(c, n, 0.0f, 0.0f) >= 0) hi = zt - zo + ev;
        if (mode == TF_FACET_GENERAL) {
            const float rx = wx - s.R * nx / xyl, ry = wy - s.R * ny / xyl;
            if (inside32(t, rx, ry, eps_b) >= 0 && comp_window(c, n, s.R, 1e-9f + s.R * 1e-9f) >= 0)
                hi = fmaxf(hi, -(nx * rx + ny * ry) / nz - s.length - zo + ev);
        }
        return hi;
    }
    float ccx, ccy, tip, dist, ed;
    if (mode == TF_FACET_HORIZ) {
        ccx = wx; ccy = wy; tip = 0.0f;
        dist = 0.0f;
        ed = 0.0f;
    } else {
        const float xnx = nx / xyl, xny = ny / xyl;
        const float rvx = s.xynl * xnx + s.nl * nx, rvy = s.xynl * xny + s.nl * ny, rvz = s.nl * nz;
        ccx = wx - rvx; ccy = wy - rvy;
        tip = -(nx * ccx + ny * ccy) / nz + rvz - s.center_height;
        dist = s.xynl + s.nl * xyl;
        ed = s.nl * xyl * 3e-7f + 1e-9f;
    }
    if (inside32(t, ccx, ccy, eps_b) >= 0 && comp_window(c, n, dist, ed) >= 0) hi = tip - zo + ev;
    return hi;
}

}  // namespace oclg
