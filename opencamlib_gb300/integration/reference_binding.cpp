// reference_binding.cpp -- see reference_binding.hpp.  Built against
// OpenCAMLib's headers; the protected cutter fields it needs are read
// through derived "peek" classes (no change to OpenCAMLib's sources).
#include "reference_binding.hpp"

#include <cmath>
#include <cstring>

#include "ballcutter.hpp"
#include "bullcutter.hpp"
#include "clpoint.hpp"
#include "compositecutter.hpp"
#include "conecutter.hpp"
#include "cylcutter.hpp"
#include "stlsurf.hpp"

namespace ocl_gb300_binding {

namespace {

struct PeekMilling : public ocl::MillingCutter {
    static double length_of(const ocl::MillingCutter& c) { return static_cast<const PeekMilling&>(c).length; }
};
struct PeekBull : public ocl::BullCutter {
    static double corner(const ocl::BullCutter& c) { return static_cast<const PeekBull&>(c).radius2; }
};
struct PeekCone : public ocl::ConeCutter {
    static double angle_of(const ocl::ConeCutter& c) { return static_cast<const PeekCone&>(c).angle; }
};
struct PeekComposite : public ocl::CompositeCutter {
    static const PeekComposite& of(const ocl::CompositeCutter& c) { return static_cast<const PeekComposite&>(c); }
    using ocl::CompositeCutter::cutter;
    using ocl::CompositeCutter::heightvec;
    using ocl::CompositeCutter::radiusvec;
    using ocl::CompositeCutter::zoffset;
};

// The l for which radius / tan(angle) + l, in doubles, is `length`.
double cone_argument(double radius, double angle, double length) {
    const double ch = radius / std::tan(angle);
    double l = length - ch;
    for (int k = 0; k < 64 && ch + l != length; ++k) l = std::nextafter(l, ch + l < length ? 1e300 : -1e300);
    return l;
}

int basic_desc(const ocl::MillingCutter& c, ocl_gb300_subcutter* s) {
    std::memset(s, 0, sizeof(*s));
    s->diameter = c.getDiameter();
    s->length = PeekMilling::length_of(c);
    if (dynamic_cast<const ocl::CylCutter*>(&c)) {
        s->kind = OCL_CUTTER_CYL;
    } else if (dynamic_cast<const ocl::BallCutter*>(&c)) {
        s->kind = OCL_CUTTER_BALL;
    } else if (const ocl::BullCutter* b = dynamic_cast<const ocl::BullCutter*>(&c)) {
        s->kind = OCL_CUTTER_BULL;
        s->corner_radius = PeekBull::corner(*b);
    } else if (const ocl::ConeCutter* k = dynamic_cast<const ocl::ConeCutter*>(&c)) {
        s->kind = OCL_CUTTER_CONE;
        s->angle = PeekCone::angle_of(*k);
        s->length = cone_argument(k->getRadius(), s->angle, PeekMilling::length_of(c));
    } else {
        return OCL_GB300_UNSUPPORTED_CUTTER;
    }
    return OCL_GB300_OK;
}

}  // namespace

int cutter_desc(const ocl::MillingCutter& c, ocl_gb300_cutter* out) {
    std::memset(out, 0, sizeof(*out));
    if (const ocl::CompositeCutter* cc = dynamic_cast<const ocl::CompositeCutter*>(&c)) {
        const PeekComposite& p = PeekComposite::of(*cc);
        if (p.cutter.empty() || p.cutter.size() > OCL_GB300_MAX_SUB) return OCL_GB300_UNSUPPORTED_CUTTER;
        out->kind = OCL_CUTTER_COMPOSITE;
        out->nsub = (int32_t)p.cutter.size();
        for (size_t n = 0; n < p.cutter.size(); ++n) {
            const int st = basic_desc(*p.cutter[n], &out->sub[n]);
            if (st) return st;
            out->sub[n].radius = p.radiusvec[n];
            out->sub[n].height = p.heightvec[n];
            out->sub[n].zoffset = p.zoffset[n];
        }
        out->composite_length = PeekMilling::length_of(c);
        return OCL_GB300_OK;
    }
    out->kind = 0;
    const int st = basic_desc(c, &out->base);
    out->kind = out->base.kind;
    return st;
}

int mesh_create(const ocl::STLSurf& s, unsigned bucket_size, ocl_gb300_mesh* out) {
    std::vector<double> tris;
    tris.reserve(9 * s.tris.size());
    for (const ocl::Triangle& t : s.tris)
        for (int k = 0; k < 3; ++k) {
            tris.push_back(t.p[k].x);
            tris.push_back(t.p[k].y);
            tris.push_back(t.p[k].z);
        }
    return ocl_gb300_mesh_create(tris.data(), s.tris.size(), bucket_size, out);
}

int batch_drop(ocl_gb300_mesh mesh, const ocl::MillingCutter& c, std::vector<ocl::CLPoint>& clpoints,
               ocl_gb300_stats* stats) {
    ocl_gb300_cutter d;
    int st = cutter_desc(c, &d);
    if (st) return st;
    const size_t M = clpoints.size();
    std::vector<double> cl(3 * M), z(M), cc(3 * M);
    std::vector<int32_t> ty(M);
    for (size_t i = 0; i < M; ++i) {
        cl[3 * i] = clpoints[i].x;
        cl[3 * i + 1] = clpoints[i].y;
        cl[3 * i + 2] = clpoints[i].z;
    }
    st = ocl_gb300_drop(mesh, &d, cl.data(), M, OCL_GB300_PREC_MIXED, z.data(), cc.data(), ty.data(), stats);
    if (st) return st;
    for (size_t i = 0; i < M; ++i) {
        ocl::CLPoint& p = clpoints[i];
        p.z = z[i];
        delete p.cc.load();
        p.cc = new ocl::CCPoint(cc[3 * i], cc[3 * i + 1], cc[3 * i + 2], (ocl::CCType)ty[i]);
    }
    return OCL_GB300_OK;
}

}  // namespace ocl_gb300_binding
