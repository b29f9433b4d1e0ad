// ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// C entry points (ref_*) over the reference library's own classes, compiled
// together with the unmodified opencamlib sources into oracle/_ref/liboclref.so
// (recipe: oracle/Makefile).  Used to pin the C restatement (ocl_oracle.c) and
// to generate the golden fixtures under tests/golden/.  Project-written glue:
// it only builds reference objects and copies their results out.
#include <cstring>
#include <map>
#include <array>
#include <vector>
#include <memory>

#include <string>

#include "stlsurf.hpp"
#include "stlreader.hpp"
#include "lineclfilter.hpp"
#include "triangle.hpp"
#include "clpoint.hpp"
#include "millingcutter.hpp"
#include "cylcutter.hpp"
#include "ballcutter.hpp"
#include "bullcutter.hpp"
#include "conecutter.hpp"
#include "compositecutter.hpp"
#include "batchdropcutter.hpp"
#include "pathdropcutter.hpp"
#include "adaptivepathdropcutter.hpp"
#include "batchpushcutter.hpp"
#include "path.hpp"
#include "line.hpp"
#include "arc.hpp"
#include "kdtree.hpp"
#include "fiber.hpp"
#include "waterline.hpp"
#include "adaptivewaterline.hpp"
#include "simple_weave.hpp"

#include "ocl_oracle.h"

namespace {

// CompositeCutter keeps `length` protected and only the preset constructors
// set it; this subclass lets a generic composite carry the preset's value.
struct RefComposite : public ocl::CompositeCutter {
    void setLength(double l) { length = l; }
};

struct CutterHolder {
    std::vector<std::unique_ptr<ocl::MillingCutter>> parts;
    ocl::MillingCutter* top = nullptr;
};

ocl::MillingCutter* make_basic(const ocl_gb300_subcutter& s) {
    switch (s.kind) {
    case OCL_CUTTER_CYL: return new ocl::CylCutter(s.diameter, s.length);
    case OCL_CUTTER_BALL: return new ocl::BallCutter(s.diameter, s.length);
    case OCL_CUTTER_BULL: return new ocl::BullCutter(s.diameter, s.corner_radius, s.length);
    case OCL_CUTTER_CONE: return new ocl::ConeCutter(s.diameter, s.angle, s.length);
    default: return nullptr;
    }
}

bool make_cutter(const ocl_gb300_cutter* c, CutterHolder& h) {
    if (c->kind != OCL_CUTTER_COMPOSITE) {
        ocl::MillingCutter* m = make_basic(c->base);
        if (!m) return false;
        h.parts.emplace_back(m);
        h.top = m;
        return true;
    }
    auto* comp = new RefComposite();
    for (int n = 0; n < c->nsub; ++n) {
        ocl::MillingCutter* m = make_basic(c->sub[n]);
        if (!m) { delete comp; return false; }
        h.parts.emplace_back(m);
        comp->addCutter(*m, c->sub[n].radius, c->sub[n].height, c->sub[n].zoffset);
    }
    comp->setLength(c->composite_length);
    h.parts.emplace_back(comp);
    h.top = comp;
    return true;
}

void make_surf(const double* tris, long ntri, ocl::STLSurf& s) {
    for (long i = 0; i < ntri; ++i) {
        const double* t = tris + 9 * i;
        s.addTriangle(ocl::Triangle(ocl::Point(t[0], t[1], t[2]), ocl::Point(t[3], t[4], t[5]),
                                    ocl::Point(t[6], t[7], t[8])));
    }
}

void make_path(const double* spans, long S, ocl::Path& p) {
    for (long i = 0; i < S; ++i) {
        const double* s = spans + OCL_GB300_SPAN_DOUBLES * i;
        ocl::Point p1(s[1], s[2], s[3]), p2(s[4], s[5], s[6]), c(s[7], s[8], s[9]);
        if (s[0] == 0.0)
            p.append(ocl::Line(p1, p2));
        else
            p.append(ocl::Arc(p1, p2, c, s[10] != 0.0));
    }
}

void put_cl(const ocl::CLPoint& cl, long i, double* xyz, double* cc, int32_t* type) {
    ocl::CCPoint ccp = *cl.cc.load();
    if (xyz) { xyz[3 * i] = cl.x; xyz[3 * i + 1] = cl.y; xyz[3 * i + 2] = cl.z; }
    cc[3 * i] = ccp.x; cc[3 * i + 1] = ccp.y; cc[3 * i + 2] = ccp.z;
    type[i] = (int32_t)ccp.type;
}

// Gives access to the protected KD-tree root for the visit-order export.
struct KDAccess : public ocl::KDTree<ocl::Triangle> {
    ocl::KDNode<ocl::Triangle>* getRoot() { return root; }
};

void walk(ocl::KDNode<ocl::Triangle>* n, std::vector<const ocl::Triangle*>& out) {
    if (!n) return;
    if (n->isLeaf) {
        for (const ocl::Triangle& t : *n->tris) out.push_back(&t);
        return;
    }
    walk(n->hi, out);
    walk(n->lo, out);
}


// Reads the protected fields of a reference cutter so tests can compare the
// composite presets (compositecutter.cpp:296-383) with the project's expansion.
struct PeekComposite : public ocl::CompositeCutter {
    static void dump(const ocl::CompositeCutter* c, double* out);
};
struct PeekCutter : public ocl::MillingCutter {
    static void dump(const ocl::MillingCutter* m, double* o) {
        const PeekCutter* p = static_cast<const PeekCutter*>(m);
        o[0] = p->diameter; o[1] = p->radius; o[2] = p->length; o[3] = p->center_height;
        o[4] = p->xy_normal_length; o[5] = p->normal_length;
    }
};
void PeekComposite::dump(const ocl::CompositeCutter* c, double* out) {
    const PeekComposite* p = static_cast<const PeekComposite*>(c);
    out[0] = p->radius; out[1] = p->length; out[2] = p->diameter;
    out[3] = (double)p->cutter.size();
    for (size_t n = 0; n < p->cutter.size(); ++n) {
        double* o = out + 4 + 9 * n;
        PeekCutter::dump(p->cutter[n], o);
        o[6] = p->radiusvec[n]; o[7] = p->heightvec[n]; o[8] = p->zoffset[n];
    }
}

// Waterline and AdaptiveWaterline with their fibers readable (protected in
// the reference classes).
struct RefWaterline : public ocl::Waterline {
    const std::vector<ocl::Fiber>& fibers(int dir) const { return dir == 0 ? xfibers : yfibers; }
};
struct RefAdaptiveWaterline : public ocl::AdaptiveWaterline {
    const std::vector<ocl::Fiber>& fibers(int dir) const { return dir == 0 ? xfibers : yfibers; }
};

// The last ref_waterline / ref_weave result, read back by ref_loops_get and
// ref_fibers_get.
struct WaterlineResult {
    std::vector<std::vector<ocl::Point>> loops;
    std::vector<ocl::Fiber> fibers[2];
};
WaterlineResult g_wl;

void keep_loops(const std::vector<std::vector<ocl::Point>>& loops, long* npts) {
    g_wl.loops = loops;
    long n = 0;
    for (const auto& l : loops) n += (long)l.size();
    *npts = n;
}

// Fibers from endpoint rows (x1 y1 z1 x2 y2 z2), per-fiber interval offsets
// and [lower, upper] t-values, as the weave receives them.
std::vector<ocl::Fiber> make_fibers(const double* fib, long F, const uint64_t* off, const double* iv) {
    std::vector<ocl::Fiber> out;
    for (long k = 0; k < F; ++k) {
        const double* f = fib + 6 * k;
        ocl::Fiber fb(ocl::Point(f[0], f[1], f[2]), ocl::Point(f[3], f[4], f[5]));
        for (uint64_t j = off[k]; j < off[k + 1]; ++j) fb.ints.push_back(ocl::Interval(iv[2 * j], iv[2 * j + 1]));
        out.push_back(fb);
    }
    return out;
}

}  // namespace

extern "C" {

int ref_drop(const double* tris, long ntri, const ocl_gb300_cutter* c, const double* cl, long M,
             int nthreads, unsigned bucket, double* z, double* cc, int32_t* type, long* ncalls) {
    CutterHolder h;
    if (!make_cutter(c, h)) return OCL_GB300_UNSUPPORTED_CUTTER;
    ocl::STLSurf s;
    make_surf(tris, ntri, s);
    ocl::BatchDropCutter bdc;
    if (nthreads > 0) bdc.setThreads(nthreads);
    bdc.setBucketSize(bucket ? bucket : 1);
    bdc.setSTL(s);
    bdc.setCutter(h.top);
    for (long i = 0; i < M; ++i) {
        ocl::CLPoint p(cl[3 * i], cl[3 * i + 1], cl[3 * i + 2]);
        bdc.appendPoint(p);
    }
    bdc.run();
    std::vector<ocl::CLPoint> res = bdc.getCLPoints();
    for (long i = 0; i < M; ++i) {
        z[i] = res[i].z;
        put_cl(res[i], i, nullptr, cc, type);
    }
    if (ncalls) *ncalls = bdc.getCalls();
    return 0;
}

long ref_push(const double* tris, long ntri, const ocl_gb300_cutter* c, int dir, const double* fib,
              long F, int nthreads, unsigned bucket, int32_t* counts, double* ival, double* cc,
              int32_t* cctype, long cap, long* ncalls) {
    CutterHolder h;
    if (!make_cutter(c, h)) return -OCL_GB300_UNSUPPORTED_CUTTER;
    ocl::STLSurf s;
    make_surf(tris, ntri, s);
    ocl::BatchPushCutter bpc;
    if (nthreads > 0) bpc.setThreads(nthreads);
    bpc.setBucketSize(bucket ? bucket : 1);
    if (dir == OCL_GB300_XFIBER) bpc.setXDirection(); else bpc.setYDirection();
    bpc.setSTL(s);
    bpc.setCutter(h.top);
    for (long i = 0; i < F; ++i) {
        const double* f = fib + 6 * i;
        ocl::Fiber fb(ocl::Point(f[0], f[1], f[2]), ocl::Point(f[3], f[4], f[5]));
        bpc.appendFiber(fb);
    }
    bpc.run();
    std::vector<ocl::Fiber>* fibers = bpc.getFibers();
    long total = 0;
    for (long i = 0; i < F; ++i) {
        const ocl::Fiber& f = (*fibers)[i];
        counts[i] = (int32_t)f.ints.size();
        for (const ocl::Interval& in : f.ints) {
            if (total < cap) {
                ival[2 * total] = in.lower;
                ival[2 * total + 1] = in.upper;
                const ocl::CCPoint& lo = in.lower_cc;
                const ocl::CCPoint& up = in.upper_cc;
                double* o = cc + 6 * total;
                o[0] = lo.x; o[1] = lo.y; o[2] = lo.z; o[3] = up.x; o[4] = up.y; o[5] = up.z;
                cctype[2 * total] = (int32_t)lo.type;
                cctype[2 * total + 1] = (int32_t)up.type;
            }
            ++total;
        }
    }
    if (ncalls) *ncalls = bpc.getCalls();
    return total;
}

long ref_pdc(const double* tris, long ntri, const ocl_gb300_cutter* c, const double* spans, long S,
             double sampling, double minz, int nthreads, unsigned bucket, double* xyz, double* cc,
             int32_t* type, long cap) {
    CutterHolder h;
    if (!make_cutter(c, h)) return -OCL_GB300_UNSUPPORTED_CUTTER;
    ocl::STLSurf s;
    make_surf(tris, ntri, s);
    ocl::Path path;
    make_path(spans, S, path);
    ocl::PathDropCutter pdc;
    if (nthreads > 0) pdc.setThreads(nthreads);
    pdc.setBucketSize(bucket ? bucket : 1);
    pdc.setSTL(s);
    pdc.setCutter(h.top);
    pdc.setPath(&path);
    pdc.setSampling(sampling);
    pdc.setZ(minz);
    pdc.run();
    std::vector<ocl::CLPoint> pts = pdc.getPoints();
    long n = (long)pts.size();
    for (long i = 0; i < n && i < cap; ++i) put_cl(pts[i], i, xyz, cc, type);
    for (ocl::Span* sp : path.span_list) delete sp;
    return n;
}

long ref_apdc(const double* tris, long ntri, const ocl_gb300_cutter* c, const double* spans, long S,
              double sampling, double min_sampling, double cos_limit, unsigned bucket, double* xyz,
              double* cc, int32_t* type, long cap) {
    CutterHolder h;
    if (!make_cutter(c, h)) return -OCL_GB300_UNSUPPORTED_CUTTER;
    ocl::STLSurf s;
    make_surf(tris, ntri, s);
    ocl::Path path;
    make_path(spans, S, path);
    ocl::AdaptivePathDropCutter apdc;
    apdc.setBucketSize(bucket ? bucket : 1);
    apdc.setSTL(s);
    apdc.setCutter(h.top);
    apdc.setPath(&path);
    apdc.setSampling(sampling);
    apdc.setMinSampling(min_sampling);
    apdc.setCosLimit(cos_limit);
    apdc.run();
    std::vector<ocl::CLPoint> pts = apdc.getPoints();
    long n = (long)pts.size();
    for (long i = 0; i < n && i < cap; ++i) put_cl(pts[i], i, xyz, cc, type);
    for (ocl::Span* sp : path.span_list) delete sp;
    return n;
}

int ref_kd_order(const double* tris, long ntri, unsigned bucket, int dims, int64_t* order) {
    ocl::STLSurf s;
    make_surf(tris, ntri, s);
    KDAccess kd;
    kd.setBucketSize(bucket ? bucket : 1);
    if (dims == 0) kd.setXYDimensions();
    else if (dims == 1) kd.setYZDimensions();
    else kd.setXZDimensions();
    kd.build(s.tris);
    std::vector<const ocl::Triangle*> visit;
    walk(kd.getRoot(), visit);
    // map leaf copies back to insertion indices by exact vertex coordinates
    std::map<std::array<double, 9>, long> index;
    for (long i = 0; i < ntri; ++i) {
        std::array<double, 9> k;
        std::memcpy(k.data(), tris + 9 * i, sizeof(k));
        index[k] = i;
    }
    if ((long)visit.size() != ntri) return -1;
    for (long i = 0; i < ntri; ++i) {
        const ocl::Triangle* t = visit[i];
        std::array<double, 9> k = {t->p[0].x, t->p[0].y, t->p[0].z, t->p[1].x, t->p[1].y,
                                   t->p[1].z, t->p[2].x, t->p[2].y, t->p[2].z};
        auto it = index.find(k);
        if (it == index.end()) return -2;
        order[i] = it->second;
    }
    return 0;
}

// STLReader(path, surface): the surface's triangles in order (p1 p2 p3),
// up to cap; returns their count.
long ref_stl_read(const char* path, double* out, long cap) {
    std::wstring wp;
    for (const char* c = path; *c; ++c) wp.push_back((wchar_t)(unsigned char)*c);
    ocl::STLSurf surf;
    ocl::STLReader reader(wp, surf);
    long n = 0;
    for (const ocl::Triangle& t : surf.tris) {
        if (n < cap)
            for (int k = 0; k < 3; ++k) {
                out[9 * n + 3 * k] = t.p[k].x;
                out[9 * n + 3 * k + 1] = t.p[k].y;
                out[9 * n + 3 * k + 2] = t.p[k].z;
            }
        ++n;
    }
    return n;
}

// LineCLFilter over n points: the kept points' coordinates in order, up to
// cap; returns their count.
long ref_line_filter(const double* xyz, long n, double tol, double* out, long cap) {
    ocl::LineCLFilter f;
    for (long i = 0; i < n; ++i) f.addCLPoint(ocl::CLPoint(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]));
    f.setTolerance(tol);
    f.run();
    long k = 0;
    for (const ocl::CLPoint& p : f.clpoints) {
        if (k < cap) {
            out[3 * k] = p.x;
            out[3 * k + 1] = p.y;
            out[3 * k + 2] = p.z;
        }
        ++k;
    }
    return k;
}

// STLSurf::rotate(xr, yr, zr) on ntri triangles: the rotated triangles in
// order (p1 p2 p3) into out (9 ntri) and the surface bbox into bb[6]
// (Bbox::operator[] order).
int ref_rotate(const double* tris, long ntri, double xr, double yr, double zr, double* out, double* bb) {
    ocl::STLSurf surf;
    for (long i = 0; i < ntri; ++i) {
        const double* v = tris + 9 * i;
        surf.addTriangle(ocl::Triangle(ocl::Point(v[0], v[1], v[2]), ocl::Point(v[3], v[4], v[5]),
                                       ocl::Point(v[6], v[7], v[8])));
    }
    surf.rotate(xr, yr, zr);
    long n = 0;
    for (const ocl::Triangle& t : surf.tris) {
        for (int k = 0; k < 3; ++k) {
            out[9 * n + 3 * k] = t.p[k].x;
            out[9 * n + 3 * k + 1] = t.p[k].y;
            out[9 * n + 3 * k + 2] = t.p[k].z;
        }
        ++n;
    }
    for (unsigned k = 0; k < 6; ++k) bb[k] = surf.bb[k];
    return 0;
}

// preset: 1 CompCyl(d,l) 2 CompBall(d,l) 3 CylCone(d1,d2,a) 4 BallCone(d1,d2,a)
//         5 BullCone(d1,r1,d2,a) 6 ConeCone(d1,a1,d2,a2)
int ref_preset_fields(int preset, const double* a, double* out) {
    std::unique_ptr<ocl::CompositeCutter> c;
    switch (preset) {
    case 1: c.reset(new ocl::CompCylCutter(a[0], a[1])); break;
    case 2: c.reset(new ocl::CompBallCutter(a[0], a[1])); break;
    case 3: c.reset(new ocl::CylConeCutter(a[0], a[1], a[2])); break;
    case 4: c.reset(new ocl::BallConeCutter(a[0], a[1], a[2])); break;
    case 5: c.reset(new ocl::BullConeCutter(a[0], a[1], a[2], a[3])); break;
    case 6: c.reset(new ocl::ConeConeCutter(a[0], a[1], a[2], a[3])); break;
    default: return -1;
    }
    PeekComposite::dump(c.get(), out);
    return 0;
}

// Waterline::run / run2 (mode 0 / 1) and AdaptiveWaterline::run / run2
// (mode 2 / 3) at height z; the loops and both fiber sets are kept for
// ref_loops_get / ref_fibers_get.  Returns the number of loops, *npts the
// number of loop points.
long ref_waterline(const double* tris, long ntri, const ocl_gb300_cutter* c, double z, double sampling,
                   double min_sampling, double cos_limit, int mode, long* npts) {
    CutterHolder h;
    if (!make_cutter(c, h)) return -1;
    ocl::STLSurf s;
    make_surf(tris, ntri, s);
    if (mode < 2) {
        RefWaterline wl;
        wl.setSTL(s);
        wl.setCutter(h.top);
        wl.setZ(z);
        wl.setSampling(sampling);
        if (mode == 0) wl.run(); else wl.run2();
        keep_loops(wl.getLoops(), npts);
        g_wl.fibers[0] = wl.fibers(0);
        g_wl.fibers[1] = wl.fibers(1);
    } else {
        RefAdaptiveWaterline wl;
        wl.setSTL(s);
        wl.setCutter(h.top);
        wl.setZ(z);
        wl.setSampling(sampling);
        wl.setMinSampling(min_sampling);
        wl.setCosLimit(cos_limit);
        if (mode == 2) wl.run(); else wl.run2();
        keep_loops(wl.getLoops(), npts);
        g_wl.fibers[0] = wl.fibers(0);
        g_wl.fibers[1] = wl.fibers(1);
    }
    return (long)g_wl.loops.size();
}

// SimpleWeave (build + face_traverse) on the given X and Y fibers.
long ref_weave(const double* xfib, long nx, const uint64_t* xoff, const double* xiv, const double* yfib, long ny,
               const uint64_t* yoff, const double* yiv, long* npts) {
    g_wl.fibers[0] = make_fibers(xfib, nx, xoff, xiv);
    g_wl.fibers[1] = make_fibers(yfib, ny, yoff, yiv);
    ocl::weave::SimpleWeave w;
    for (ocl::Fiber& f : g_wl.fibers[0]) w.addFiber(f);
    for (ocl::Fiber& f : g_wl.fibers[1]) w.addFiber(f);
    w.build();
    w.face_traverse();
    keep_loops(w.getLoops(), npts);
    return (long)g_wl.loops.size();
}

// The kept loops: points (3 doubles each) and offsets (nloops + 1).
void ref_loops_get(double* pts, long* off) {
    long n = 0;
    off[0] = 0;
    for (size_t k = 0; k < g_wl.loops.size(); ++k) {
        for (const ocl::Point& p : g_wl.loops[k]) {
            pts[3 * n] = p.x; pts[3 * n + 1] = p.y; pts[3 * n + 2] = p.z;
            ++n;
        }
        off[k + 1] = n;
    }
}

// The kept fibers of one direction: count (fib == nullptr), or endpoints,
// interval offsets and [lower, upper] t-values.
long ref_fibers_get(int dir, double* fib, uint64_t* off, double* iv) {
    const std::vector<ocl::Fiber>& fs = g_wl.fibers[dir];
    if (!fib) {
        long k = 0;
        for (const ocl::Fiber& f : fs) k += (long)f.ints.size();
        off[0] = (uint64_t)k;
        return (long)fs.size();
    }
    uint64_t n = 0;
    for (size_t k = 0; k < fs.size(); ++k) {
        const ocl::Fiber& f = fs[k];
        const double e[6] = {f.p1.x, f.p1.y, f.p1.z, f.p2.x, f.p2.y, f.p2.z};
        std::memcpy(fib + 6 * k, e, sizeof(e));
        off[k] = n;
        for (const ocl::Interval& i : f.ints) {
            iv[2 * n] = i.lower;
            iv[2 * n + 1] = i.upper;
            ++n;
        }
    }
    off[fs.size()] = n;
    return (long)fs.size();
}

}  // extern "C"
