// binding_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Drives opencamlib_gb300/integration/reference_binding.cpp with cutter and
// surface objects of the reference library (built from its own sources by
// the `binding` target of oracle/Makefile), so tests can check the binding's
// cutter descriptors against the reference objects' own fields.
#include <cstring>
#include <memory>

#include "ballcutter.hpp"
#include "bullcutter.hpp"
#include "compositecutter.hpp"
#include "conecutter.hpp"
#include "cylcutter.hpp"
#include "reference_binding.hpp"
#include "stlsurf.hpp"

namespace {

struct Peek : public ocl::MillingCutter {
    static void basic(const ocl::MillingCutter* m, double* o) {
        const Peek* p = static_cast<const Peek*>(m);
        o[0] = p->diameter; o[1] = p->radius; o[2] = p->length; o[3] = p->center_height;
        o[4] = p->xy_normal_length; o[5] = p->normal_length;
    }
    static void top(const ocl::MillingCutter* m, double* o) {
        const Peek* p = static_cast<const Peek*>(m);
        o[0] = p->radius; o[1] = p->length; o[2] = p->diameter;
    }
};
struct PeekComp : public ocl::CompositeCutter {
    static void dump(const ocl::CompositeCutter* c, double* out) {
        const PeekComp* p = static_cast<const PeekComp*>(c);
        out[3] = (double)p->cutter.size();
        for (size_t n = 0; n < p->cutter.size(); ++n) {
            double* o = out + 4 + 9 * n;
            Peek::basic(p->cutter[n], o);
            o[6] = p->radiusvec[n]; o[7] = p->heightvec[n]; o[8] = p->zoffset[n];
        }
    }
};

ocl::MillingCutter* make(int kind, const double* a) {
    switch (kind) {
    case 1: return new ocl::CylCutter(a[0], a[1]);
    case 2: return new ocl::BallCutter(a[0], a[1]);
    case 3: return new ocl::BullCutter(a[0], a[1], a[2]);
    case 4: return new ocl::ConeCutter(a[0], a[1], a[2]);
    case 11: return new ocl::CompCylCutter(a[0], a[1]);
    case 12: return new ocl::CompBallCutter(a[0], a[1]);
    case 13: return new ocl::CylConeCutter(a[0], a[1], a[2]);
    case 14: return new ocl::BallConeCutter(a[0], a[1], a[2]);
    case 15: return new ocl::BullConeCutter(a[0], a[1], a[2], a[3]);
    case 16: return new ocl::ConeConeCutter(a[0], a[1], a[2], a[3]);
    }
    return nullptr;
}

}  // namespace

extern "C" {

// kind 1..4: Cyl(d,l), Ball(d,l), Bull(d,r,l), Cone(d,angle,l); 11..16 the
// composite presets.  desc: the binding's descriptor; fields: the reference
// object's own fields in oracle_cutter_fields' layout.  Returns the binding's status.
int binding_cutter(int kind, const double* args, ocl_gb300_cutter* desc, double* fields) {
    std::unique_ptr<ocl::MillingCutter> c(make(kind, args));
    if (!c) return -1;
    std::memset(fields, 0, sizeof(double) * (4 + 9 * OCL_GB300_MAX_SUB));
    Peek::top(c.get(), fields);
    if (kind >= 11) PeekComp::dump(static_cast<ocl::CompositeCutter*>(c.get()), fields);
    else Peek::basic(c.get(), fields + 4);
    return ocl_gb300_binding::cutter_desc(*c, desc);
}

// A two-triangle STLSurf through the binding's mesh_create and batch_drop;
// returns the status of the first call that fails (OCL_GB300_NO_DEVICE
// without a GPU), else the lifted z of a CL point above the surface.
int binding_drop(double* z_out) {
    ocl::STLSurf s;
    s.addTriangle(ocl::Triangle(ocl::Point(0, 0, 1), ocl::Point(10, 0, 1), ocl::Point(0, 10, 1)));
    s.addTriangle(ocl::Triangle(ocl::Point(10, 0, 1), ocl::Point(10, 10, 2), ocl::Point(0, 10, 1)));
    ocl_gb300_mesh m = nullptr;
    int st = ocl_gb300_binding::mesh_create(s, 1, &m);
    if (st) return st;
    ocl::BallCutter ball(2.0, 10.0);
    std::vector<ocl::CLPoint> pts;
    pts.push_back(ocl::CLPoint(2.0, 2.0, -5.0));
    st = ocl_gb300_binding::batch_drop(m, ball, pts, nullptr);
    ocl_gb300_mesh_release(m);
    if (st) return st;
    *z_out = pts[0].z;
    return 0;
}

}  // extern "C"
