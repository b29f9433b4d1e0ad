// ocl/ocl.hpp -- header-only C++ facade with the reference library's class
// API for the drop-cutter / push-cutter path (namespace ocl):
//
//   geometry   Point, CCPoint/CCType, CLPoint, Bbox, Triangle, STLSurf,
//              STLReader (src/geo/*.hpp), Line, Arc, Path (src/geo/path.hpp)
//   cutters    MillingCutter, CylCutter, BallCutter, BullCutter, ConeCutter,
//              CompositeCutter and its presets (src/cutters/*.hpp)
//   fibers     Interval, Fiber (src/algo/interval.hpp, fiber.hpp)
//   filters    CLFilter, LineCLFilter (src/common/*clfilter.hpp)
//   operations BatchDropCutter, PathDropCutter, AdaptivePathDropCutter,
//              BatchPushCutter (src/dropcutter/*.hpp, src/algo/batchpushcutter.hpp)
//
// Client code written against the reference's headers for these classes
// compiles unchanged; run() executes on the GPU through libocl_gb300.so
// (include/ocl_gb300.h).  Like the reference, setSTL/setCutter/setPath keep
// non-owning pointers and appendPoint/appendFiber copy.  Errors: the reference
// only asserts; here a failing run() leaves the outputs untouched, writes the
// library's message to std::cerr and keeps it in lastError().
#pragma once

#include <atomic>
#include <cmath>
#include <cstring>
#include <iostream>
#include <list>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "ocl_gb300.h"

namespace ocl {

// ---------------------------------------------------------------- geometry
class Point {
   public:
    Point() : x(0), y(0), z(0) {}
    Point(double xin, double yin, double zin) : x(xin), y(yin), z(zin) {}
    Point(double xin, double yin) : x(xin), y(yin), z(0.0) {}
    Point(const Point& p) = default;
    Point& operator=(const Point& p) = default;
    virtual ~Point() {}
    double x, y, z;
    double dot(const Point& p) const { return x * p.x + y * p.y + z * p.z; }
    Point cross(const Point& p) const { return Point(y * p.z - z * p.y, z * p.x - x * p.z, x * p.y - y * p.x); }
    double norm() const { return std::sqrt(x * x + y * y + z * z); }
    double xyNorm() const { return std::sqrt(x * x + y * y); }
    void normalize() {
        double n = norm();
        if (n != 0.0) *this *= (1 / n);
    }
    void xyNormalize() {
        if (xyNorm() != 0.0) *this *= (1 / xyNorm());
    }
    double xyDistance(const Point& p) const { return (*this - p).xyNorm(); }
    Point& operator*=(const double& a) {
        x *= a; y *= a; z *= a;
        return *this;
    }
    Point& operator+=(const Point& p) {
        x += p.x; y += p.y; z += p.z;
        return *this;
    }
    Point& operator-=(const Point& p) {
        x -= p.x; y -= p.y; z -= p.z;
        return *this;
    }
    const Point operator+(const Point& p) const { return Point(*this) += p; }
    const Point operator-(const Point& p) const { return Point(*this) -= p; }
    const Point operator*(const double& a) const { return Point(*this) *= a; }
    bool operator==(const Point& p) const { return x == p.x && y == p.y && z == p.z; }
    bool operator!=(const Point& p) const { return !(*this == p); }
    // rotations about the x, y, z axes (src/geo/point.cpp:105-134): the
    // point times a rotation matrix, each row summed left to right
    void xRotate(double theta) {
        matrixRotate(1, 0, 0, 0, std::cos(theta), -std::sin(theta), 0, std::sin(theta), std::cos(theta));
    }
    void yRotate(double theta) {
        matrixRotate(std::cos(theta), 0, std::sin(theta), 0, 1, 0, -std::sin(theta), 0, std::cos(theta));
    }
    void zRotate(double theta) {
        matrixRotate(std::cos(theta), -std::sin(theta), 0, std::sin(theta), std::cos(theta), 0, 0, 0, 1);
    }
    void matrixRotate(double a, double b, double c, double d, double e, double f, double g, double h, double i) {
        const double xr = a * x + b * y + c * z;
        const double yr = d * x + e * y + f * z;
        const double zr = g * x + h * y + i * z;
        x = xr; y = yr; z = zr;
    }
    std::string str() const {
        std::ostringstream o;
        o << "(" << x << ", " << y << ", " << z << ")";
        return o.str();
    }
};
inline const Point operator*(const double& a, const Point& p) { return Point(p) *= a; }

enum CCType {
    NONE, VERTEX, VERTEX_CYL, EDGE, EDGE_HORIZ, EDGE_SHAFT, EDGE_HORIZ_CYL, EDGE_HORIZ_TOR, EDGE_BALL,
    EDGE_POS, EDGE_NEG, EDGE_CYL, EDGE_CONE, EDGE_CONE_BASE, FACET, FACET_TIP, FACET_CYL, ERROR
};

class CCPoint : public Point {
   public:
    CCPoint() : Point(), type(NONE) {}
    CCPoint(double x, double y, double z) : Point(x, y, z), type(NONE) {}
    CCPoint(double x, double y, double z, CCType t) : Point(x, y, z), type(t) {}
    CCPoint(const Point& p, CCType t) : Point(p), type(t) {}
    explicit CCPoint(const Point& p) : Point(p), type(NONE) {}
    CCType type;
};

class CLPoint : public Point {
   public:
    CLPoint() : Point(), cc(new CCPoint()) {}
    CLPoint(double x, double y, double z) : Point(x, y, z), cc(new CCPoint()) {}
    CLPoint(double x, double y, double z, CCPoint& ccp) : Point(x, y, z), cc(new CCPoint(ccp)) {}
    CLPoint(const CLPoint& c) : Point(c.x, c.y, c.z), cc(new CCPoint(*c.cc.load())) {}
    CLPoint(const Point& p) : Point(p.x, p.y, p.z), cc(new CCPoint()) {}
    ~CLPoint() override { delete cc.load(); }
    CLPoint& operator=(const CLPoint& c) {
        if (this == &c) return *this;
        x = c.x; y = c.y; z = c.z;
        delete cc.load();
        cc = new CCPoint(*c.cc.load());
        return *this;
    }
    std::atomic<CCPoint*> cc;
    CCPoint getCC() { return *cc.load(); }
    bool below(const class Triangle& t) const;
    std::string str() const {
        std::ostringstream o;
        const CCPoint* c = cc.load();
        o << "CL(" << x << ", " << y << ", " << z << ") cc=CC(" << c->x << ", " << c->y << ", " << c->z
          << ", t=" << c->type << ")";
        return o.str();
    }
};

class Bbox {
   public:
    Bbox() : initialized(false) {}
    Bbox(double b1, double b2, double b3, double b4, double b5, double b6)
        : minpt(b1, b3, b5), maxpt(b2, b4, b6), initialized(true) {}
    Point minpt, maxpt;
    void clear() { initialized = false; }
    void addPoint(const Point& p) {
        if (!initialized) {
            minpt = p; maxpt = p; initialized = true;
            return;
        }
        if (p.x > maxpt.x) maxpt.x = p.x;
        if (p.x < minpt.x) minpt.x = p.x;
        if (p.y > maxpt.y) maxpt.y = p.y;
        if (p.y < minpt.y) minpt.y = p.y;
        if (p.z > maxpt.z) maxpt.z = p.z;
        if (p.z < minpt.z) minpt.z = p.z;
    }
    double operator[](const unsigned int idx) const {
        const double v[6] = {minpt.x, maxpt.x, minpt.y, maxpt.y, minpt.z, maxpt.z};
        return idx < 6 ? v[idx] : -1;
    }
    bool initialized;
};

class Triangle {
   public:
    Triangle() : Triangle(Point(1, 0, 0), Point(0, 1, 0), Point(0, 0, 1)) {}
    Triangle(Point p1, Point p2, Point p3) {
        p[0] = p1; p[1] = p2; p[2] = p3;
        calc();
    }
    Triangle(const Triangle& t) {
        p[0] = t.p[0]; p[1] = t.p[1]; p[2] = t.p[2];
        calc();
    }
    Triangle& operator=(const Triangle& t) = default;
    virtual ~Triangle() {}
    Point p[3];
    Point n;
    Bbox bb;
    Point upNormal() const { return (n.z < 0) ? -1.0 * n : n; }
    // Triangle::rotate (src/geo/triangle.cpp:130-138)
    void rotate(double xr, double yr, double zr) {
        for (int k = 0; k < 3; ++k) {
            p[k].xRotate(xr);
            p[k].yRotate(yr);
            p[k].zRotate(zr);
        }
        calc();
    }

   private:
    void calc() {
        Point v1 = p[0] - p[1], v2 = p[0] - p[2];
        n = v1.cross(v2);
        n.normalize();
        bb.clear();
        for (int k = 0; k < 3; ++k) bb.addPoint(p[k]);
    }
};

inline bool CLPoint::below(const Triangle& t) const { return z < t.bb.maxpt.z; }

class STLSurf {
   public:
    STLSurf() {}
    virtual ~STLSurf() {}
    void addTriangle(const Triangle& t) {
        tris.push_back(t);
        bb.addPoint(t.p[0]);
        bb.addPoint(t.p[1]);
        bb.addPoint(t.p[2]);
        ++version_;
    }
    // STLSurf::rotate (src/geo/stlsurf.cpp:44-55): every triangle rotated,
    // the bounding box rebuilt; the device copy is made again on next use
    void rotate(double xr, double yr, double zr) {
        bb.clear();
        for (Triangle& t : tris) {
            t.rotate(xr, yr, zr);
            bb.addPoint(t.p[0]);
            bb.addPoint(t.p[1]);
            bb.addPoint(t.p[2]);
        }
        ++version_;
    }
    unsigned int size() const { return static_cast<unsigned int>(tris.size()); }
    std::list<Triangle> tris;
    Bbox bb;
    // device copy, built on first use by an operation and reused
    ocl_gb300_mesh device(uint32_t bucket) const {
        auto it = dev_.find(bucket);
        if (it != dev_.end() && it->second.version == version_ && it->second.mesh) return it->second.mesh.get();
        std::vector<double> a;
        a.reserve(9 * tris.size());
        for (const Triangle& t : tris)
            for (int k = 0; k < 3; ++k) {
                a.push_back(t.p[k].x); a.push_back(t.p[k].y); a.push_back(t.p[k].z);
            }
        ocl_gb300_mesh m = nullptr;
        int st = ocl_gb300_mesh_create(a.data(), tris.size(), bucket, &m);
        if (st != OCL_GB300_OK) return nullptr;
        Dev d;
        d.version = version_;
        d.mesh = std::shared_ptr<ocl_gb300_mesh_s>(m, [](ocl_gb300_mesh p) { ocl_gb300_mesh_release(p); });
        dev_[bucket] = d;
        return m;
    }

   private:
    struct Dev {
        unsigned long version = 0;
        std::shared_ptr<ocl_gb300_mesh_s> mesh;
    };
    mutable std::map<uint32_t, Dev> dev_;
    unsigned long version_ = 0;
};

// STLReader(filepath, surface) adds the file's triangles to the surface
// (src/geo/stlreader.hpp); a file that cannot be read adds nothing, as in
// the reference.  The path's wide characters are narrowed one by one, as the
// reference does.
class STLReader {
   public:
    STLReader() {}
    STLReader(const std::wstring& filepath, STLSurf& surface) { read_from_file(filepath, surface); }
    virtual ~STLReader() {}

   private:
    void read_from_file(const std::wstring& filepath, STLSurf& surface) {
        std::string path;
        for (wchar_t c : filepath) path.push_back(static_cast<char>(c));
        uint64_t n = 0;
        ocl_gb300_stl_read(path.c_str(), nullptr, 0, &n);
        if (n == 0) return;
        std::vector<double> a(9 * n);
        ocl_gb300_stl_read(path.c_str(), a.data(), n, &n);
        for (uint64_t i = 0; i < n; ++i) {
            const double* t = &a[9 * i];
            surface.addTriangle(Triangle(Point(t[0], t[1], t[2]), Point(t[3], t[4], t[5]), Point(t[6], t[7], t[8])));
        }
    }
};

// ---------------------------------------------------------------- CL filters
// CLFilter / LineCLFilter (src/common/clfilter.hpp, lineclfilter.hpp):
// addCLPoint copies, run() replaces clpoints by the points the filter keeps
// (the selection runs in the library, ocl_gb300_line_filter; the kept points
// are the caller's copies, CC points included).
class CLFilter {
   public:
    CLFilter() {}
    virtual ~CLFilter() {}
    virtual void addCLPoint(const CLPoint& p) = 0;
    virtual void setTolerance(const double tol) = 0;
    virtual void run() = 0;
    std::list<CLPoint> clpoints;
    double tol = 0.0;
};

class LineCLFilter : public CLFilter {
   public:
    LineCLFilter() { clpoints.clear(); }
    virtual ~LineCLFilter() {}
    void addCLPoint(const CLPoint& p) override { clpoints.push_back(p); }
    void setTolerance(const double tolerance) override { tol = tolerance; }
    void run() override {
        const size_t n = clpoints.size();
        if (n < 2) return;
        std::vector<double> xyz;
        xyz.reserve(3 * n);
        std::vector<const CLPoint*> ptr;
        ptr.reserve(n);
        for (const CLPoint& p : clpoints) {
            xyz.push_back(p.x); xyz.push_back(p.y); xyz.push_back(p.z);
            ptr.push_back(&p);
        }
        std::vector<uint64_t> keep(n);
        uint64_t nk = 0;
        if (ocl_gb300_line_filter(xyz.data(), n, tol, keep.data(), &nk) != OCL_GB300_OK) {
            std::cerr << "ocl::LineCLFilter: " << ocl_gb300_last_error() << "\n";
            return;
        }
        std::list<CLPoint> kept;
        for (uint64_t k = 0; k < nk; ++k) kept.push_back(*ptr[keep[k]]);
        clpoints.swap(kept);
    }
};

// ---------------------------------------------------------------- paths
class Line {
   public:
    Line(const Point& a, const Point& b) : p1(a), p2(b) {}
    Point p1, p2;
    double length2d() const { return (p2 - p1).xyNorm(); }
    Point getPoint(double t) const { return (p2 - p1) * t + p1; }
};
class Arc {
   public:
    Arc(const Point& a, const Point& b, const Point& cen, bool d) : p1(a), p2(b), c(cen), dir(d) {}
    Point p1, p2, c;
    bool dir;
};
enum SpanType { LineSpanType, ArcSpanType };
class Span {
   public:
    virtual ~Span() {}
    virtual SpanType type() const = 0;
    virtual void row(double* r) const = 0;
};
class LineSpan : public Span {
   public:
    explicit LineSpan(const Line& l) : line(l) {}
    Line line;
    SpanType type() const override { return LineSpanType; }
    void row(double* r) const override {
        const double v[11] = {0, line.p1.x, line.p1.y, line.p1.z, line.p2.x, line.p2.y, line.p2.z, 0, 0, 0, 0};
        std::memcpy(r, v, sizeof(v));
    }
};
class ArcSpan : public Span {
   public:
    explicit ArcSpan(const Arc& a) : arc(a) {}
    Arc arc;
    SpanType type() const override { return ArcSpanType; }
    void row(double* r) const override {
        const double v[11] = {1, arc.p1.x, arc.p1.y, arc.p1.z, arc.p2.x, arc.p2.y, arc.p2.z,
                              arc.c.x, arc.c.y, arc.c.z, arc.dir ? 1.0 : 0.0};
        std::memcpy(r, v, sizeof(v));
    }
};
class Path {
   public:
    Path() {}
    virtual ~Path() {
        for (Span* s : span_list) delete s;
    }
    std::list<Span*> span_list;
    void append(const Line& l) { span_list.push_back(new LineSpan(l)); }
    void append(const Arc& a) { span_list.push_back(new ArcSpan(a)); }
    std::vector<double> rows() const {
        std::vector<double> r(OCL_GB300_SPAN_DOUBLES * span_list.size());
        size_t k = 0;
        for (const Span* s : span_list) s->row(&r[OCL_GB300_SPAN_DOUBLES * k++]);
        return r;
    }
};

// ---------------------------------------------------------------- cutters
class MillingCutter {
   public:
    virtual ~MillingCutter() {}
    double getDiameter() const { return diameter; }
    double getRadius() const { return radius; }
    double getLength() const { return length; }
    virtual ocl_gb300_cutter desc() const = 0;
    virtual std::string str() const { return "MillingCutter"; }
    virtual ocl_gb300_subcutter sub() const { return ocl_gb300_subcutter(); }

   protected:
    double diameter = 0, radius = 0, length = 0;
    static ocl_gb300_cutter basic(const ocl_gb300_subcutter& s) {
        ocl_gb300_cutter c;
        std::memset(&c, 0, sizeof(c));
        c.kind = s.kind;
        c.base = s;
        return c;
    }
    static ocl_gb300_subcutter mk(int kind, double d, double r, double a, double l) {
        ocl_gb300_subcutter s;
        std::memset(&s, 0, sizeof(s));
        s.kind = kind; s.diameter = d; s.corner_radius = r; s.angle = a; s.length = l;
        return s;
    }
};

class CylCutter : public MillingCutter {
   public:
    CylCutter(double d, double l) : larg(l) { diameter = d; radius = d / 2.0; length = l; }
    ocl_gb300_subcutter sub() const override { return mk(OCL_CUTTER_CYL, diameter, 0, 0, larg); }
    ocl_gb300_cutter desc() const override { return basic(sub()); }
    std::string str() const override { return "CylCutter"; }

   private:
    double larg;
};
class BallCutter : public MillingCutter {
   public:
    BallCutter(double d, double l) : larg(l) { diameter = d; radius = d / 2.0; length = l; }
    ocl_gb300_subcutter sub() const override { return mk(OCL_CUTTER_BALL, diameter, 0, 0, larg); }
    ocl_gb300_cutter desc() const override { return basic(sub()); }
    std::string str() const override { return "BallCutter"; }

   private:
    double larg;
};
class BullCutter : public MillingCutter {
   public:
    BullCutter(double d, double r, double l) : r2(r), larg(l) { diameter = d; radius = d / 2.0; length = l; }
    ocl_gb300_subcutter sub() const override { return mk(OCL_CUTTER_BULL, diameter, r2, 0, larg); }
    ocl_gb300_cutter desc() const override { return basic(sub()); }
    std::string str() const override { return "BullCutter"; }

   private:
    double r2, larg;
};
class ConeCutter : public MillingCutter {
   public:
    ConeCutter(double d, double a, double l = 10) : angle(a), larg(l) {
        diameter = d;
        radius = d / 2.0;
        length = radius / std::tan(angle) + l;
    }
    ocl_gb300_subcutter sub() const override { return mk(OCL_CUTTER_CONE, diameter, 0, angle, larg); }
    ocl_gb300_cutter desc() const override { return basic(sub()); }
    std::string str() const override { return "ConeCutter"; }

   private:
    double angle, larg;
};

class CompositeCutter : public MillingCutter {
   public:
    CompositeCutter() {}
    // cutter c is valid out to radius r and height h, shifted by zoff
    void addCutter(MillingCutter& c, double r, double h, double zoff) {
        ocl_gb300_subcutter s = c.sub();
        s.radius = r;
        s.height = h;
        s.zoffset = zoff;
        parts.push_back(s);
        if (r > radius) {
            radius = r;
            diameter = 2 * r;
        }
    }
    ocl_gb300_cutter desc() const override {
        ocl_gb300_cutter c;
        std::memset(&c, 0, sizeof(c));
        c.kind = OCL_CUTTER_COMPOSITE;
        c.nsub = (int32_t)parts.size();
        for (size_t n = 0; n < parts.size() && n < OCL_GB300_MAX_SUB; ++n) c.sub[n] = parts[n];
        c.composite_length = length;
        return c;
    }
    std::string str() const override { return "CompositeCutter"; }

   protected:
    std::vector<ocl_gb300_subcutter> parts;
};

// Preset composites (src/cutters/compositecutter.cpp:296-383): same sub-cutters,
// radius windows and z offsets as the reference constructors.
class CompCylCutter : public CompositeCutter {
   public:
    CompCylCutter(double diam2, double clength) {
        CylCutter c(diam2, clength);
        addCutter(c, diam2 / 2.0, clength, 0.0);
        length = clength;
    }
};
class CompBallCutter : public CompositeCutter {
   public:
    CompBallCutter(double diam2, double clength) {
        BallCutter c(diam2, clength);
        addCutter(c, diam2 / 2.0, clength, 0.0);
        length = clength;
    }
};
class CylConeCutter : public CompositeCutter {
   public:
    CylConeCutter(double diam1, double diam2, double angle) {
        CylCutter cyl(diam1, 1);
        ConeCutter cone(diam2, angle);
        CylCutter shaft(diam2, 20);
        double cone_offset = -(diam1 / 2) / std::tan(angle);
        double cyl_height = 0.0;
        double cone_height = (diam2 / 2.0) / std::tan(angle) + cone_offset;
        addCutter(cyl, diam1 / 2.0, cyl_height, 0.0);
        addCutter(cone, diam2 / 2.0, cone_height, cone_offset);
        addCutter(shaft, diam2 / 2.0, (diam2 / 2.0) / std::tan(angle) + 20, cone_height);
        length = cyl_height + cone_height + 10;
    }
};
class BallConeCutter : public CompositeCutter {
   public:
    BallConeCutter(double diam1, double diam2, double angle) {
        BallCutter c1(diam1, 1);
        ConeCutter c2(diam2, angle);
        CylCutter shaft(diam2, 20);
        double radius1 = diam1 / 2.0, radius2 = diam2 / 2.0;
        double rcontact = radius1 * std::cos(angle);
        double height1 = radius1 - std::sqrt(radius1 * radius1 - rcontact * rcontact);
        double cone_offset = -((rcontact) / std::tan(angle) - height1);
        double height2 = radius2 / std::tan(angle) + cone_offset;
        addCutter(c1, rcontact, height1, 0.0);
        addCutter(c2, diam2 / 2.0, height2, cone_offset);
        addCutter(shaft, diam2 / 2.0, height2 + 20, height2);
        length = 30;
    }
};
class BullConeCutter : public CompositeCutter {
   public:
    BullConeCutter(double diam1, double radius1, double diam2, double angle) {
        BullCutter c1(diam1, radius1, 1.0);
        ConeCutter c2(diam2, angle);
        CylCutter shaft(diam2, 20);
        double h1 = radius1 * std::sin(angle);
        double rad = std::sqrt(radius1 * radius1 - h1 * h1);
        double rcontact = (diam1 / 2.0) - radius1 + rad;
        double cone_offset = -(rcontact / std::tan(angle) - (radius1 - h1));
        double height1 = radius1 - h1;
        double height2 = (diam2 / 2.0) / std::tan(angle) + cone_offset;
        addCutter(c1, rcontact, height1, 0.0);
        addCutter(c2, diam2 / 2.0, height2, cone_offset);
        addCutter(shaft, diam2 / 2.0, height2 + 20, height2);
        length = 30;
    }
};
class ConeConeCutter : public CompositeCutter {
   public:
    ConeConeCutter(double diam1, double angle1, double diam2, double angle2) {
        ConeCutter c1(diam1, angle1);
        ConeCutter c2(diam2, angle2);
        CylCutter shaft(diam2, 20);
        double height1 = (diam1 / 2.0) / std::tan(angle1);
        double tmp = (diam1 / 2.0) / std::tan(angle2);
        double cone_offset = -(tmp - height1);
        double height2 = (diam2 / 2.0) / std::tan(angle2) + cone_offset;
        addCutter(c1, diam1 / 2.0, height1, 0.0);
        addCutter(c2, diam2 / 2.0, height2, cone_offset);
        addCutter(shaft, diam2 / 2.0, height2 + 20, height2);
        length = 30;
    }
};

// ---------------------------------------------------------------- fibers
class Interval {
   public:
    Interval() : upper(0.0), lower(0.0), in_weave(false) {}
    Interval(const double l, const double u) : upper(u), lower(l), in_weave(false) {}
    virtual ~Interval() {}
    CCPoint upper_cc, lower_cc;
    double upper, lower;
    bool in_weave;
    bool empty() const { return lower == 0.0 && upper == 0.0; }
    bool outside(const Interval& i) const { return lower > i.upper || upper < i.lower; }
    bool inside(const Interval& i) const { return lower > i.lower && upper < i.upper; }
};

class Fiber {
   public:
    Fiber() {}
    Fiber(const Point& a, const Point& b) : p1(a), p2(b) {
        dir = p2 - p1;
        dir.normalize();
    }
    virtual ~Fiber() {}
    Point p1, p2, dir;
    std::vector<Interval> ints;
    bool empty() const { return ints.empty(); }
    unsigned int size() const { return static_cast<unsigned int>(ints.size()); }
    Point point(double t) const { return p1 + t * (p2 - p1); }
    double tval(Point& p) const {
        Point d = p2 - p1;
        return (p - p1).dot(d) / d.dot(d);
    }
    Point upperCLPoint(unsigned int n) const { return point(ints[n].upper); }
    Point lowerCLPoint(unsigned int n) const { return point(ints[n].lower); }
    bool operator==(const Fiber& o) const { return p1 == o.p1 && p2 == o.p2; }
};

// ---------------------------------------------------------------- operations
class Operation {
   public:
    Operation() {}
    virtual ~Operation() {}
    virtual void setSTL(const STLSurf& s) { surf = &s; }
    virtual void setCutter(const MillingCutter* c) { cutter = c; }
    void setThreads(unsigned int n) { nthreads = n; }  // accepted; the GPU path ignores it
    int getThreads() const { return (int)nthreads; }
    int getBucketSize() const { return (int)bucketSize; }
    void setBucketSize(unsigned int s) { bucketSize = s; }
    int getCalls() const { return nCalls; }
    virtual void setSampling(double s) { sampling = s; }
    virtual double getSampling() { return sampling; }
    virtual void run() = 0;
    virtual void reset() {}
    virtual void appendPoint(CLPoint&) {}
    virtual void setXDirection() {}
    virtual void setYDirection() {}
    virtual void appendFiber(Fiber&) {}
    // precision of the drop kernels: OCL_GB300_PREC_MIXED (default) or _FP64
    void setPrecision(int p) { precision = p; }
    const std::string& lastError() const { return error; }
    const ocl_gb300_stats& lastStats() const { return stats; }

   protected:
    double sampling = 0.1;
    int nCalls = 0;
    unsigned int bucketSize = 1;
    const MillingCutter* cutter = nullptr;
    const STLSurf* surf = nullptr;
    unsigned int nthreads = 0;
    int precision = OCL_GB300_PREC_MIXED;
    std::string error;
    ocl_gb300_stats stats{};
    ocl_gb300_mesh mesh() {
        if (!surf || !cutter) {
            fail("setSTL() and setCutter() must be called before run()");
            return nullptr;
        }
        ocl_gb300_mesh m = surf->device(bucketSize);
        if (!m) fail(ocl_gb300_last_error());
        return m;
    }
    bool check(int st) {
        if (st == OCL_GB300_OK) return true;
        fail(ocl_gb300_last_error());
        return false;
    }
    void fail(const std::string& msg) {
        error = msg;
        std::cerr << "ocl_gb300: " << msg << "\n";
    }
};

class BatchDropCutter : public Operation {
   public:
    BatchDropCutter() : clpoints(new std::vector<CLPoint>()) {}
    ~BatchDropCutter() override { delete clpoints; }
    void appendPoint(CLPoint& p) override { clpoints->push_back(p); }
    void run() override {
        ocl_gb300_mesh m = mesh();
        if (!m) return;
        const size_t M = clpoints->size();
        std::vector<double> cl(3 * M), z(M), cc(3 * M);
        std::vector<int32_t> ty(M);
        for (size_t i = 0; i < M; ++i) {
            cl[3 * i] = (*clpoints)[i].x;
            cl[3 * i + 1] = (*clpoints)[i].y;
            cl[3 * i + 2] = (*clpoints)[i].z;
        }
        ocl_gb300_cutter d = cutter->desc();
        if (!check(ocl_gb300_drop(m, &d, cl.data(), M, precision, z.data(), cc.data(), ty.data(), &stats))) return;
        for (size_t i = 0; i < M; ++i) {
            CLPoint& p = (*clpoints)[i];
            p.z = z[i];
            delete p.cc.load();
            p.cc = new CCPoint(cc[3 * i], cc[3 * i + 1], cc[3 * i + 2], (CCType)ty[i]);
        }
        nCalls = (int)(stats.pairs ? stats.pairs : stats.refined);
    }
    std::vector<CLPoint> getCLPoints() { return *clpoints; }
    void clearCLPoints() { clpoints->clear(); }

   protected:
    std::vector<CLPoint>* clpoints;
};

class PathDropCutter : public Operation {
   public:
    PathDropCutter() {}
    void setPath(const Path* p) { path = p; }
    void setZ(const double z) { minimumZ = z; }
    double getZ() const { return minimumZ; }
    std::vector<CLPoint> getPoints() const { return clpoints; }
    void run() override {
        ocl_gb300_mesh m = mesh();
        if (!m || !path) return;
        std::vector<double> spans = path->rows();
        ocl_gb300_cutter d = cutter->desc();
        uint64_t n = 0;
        std::vector<double> xyz, cc;
        std::vector<int32_t> ty;
        int st = call(m, d, spans, xyz, cc, ty, 0, n);
        if (st == OCL_GB300_CAPACITY) st = call(m, d, spans, xyz, cc, ty, n, n);
        if (!check(st)) return;
        clpoints.clear();
        for (uint64_t i = 0; i < n; ++i) {
            CCPoint c(cc[3 * i], cc[3 * i + 1], cc[3 * i + 2], (CCType)ty[i]);
            clpoints.push_back(CLPoint(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], c));
        }
    }

   protected:
    virtual int call(ocl_gb300_mesh m, const ocl_gb300_cutter& d, const std::vector<double>& spans,
                     std::vector<double>& xyz, std::vector<double>& cc, std::vector<int32_t>& ty, uint64_t cap,
                     uint64_t& n) {
        xyz.resize(3 * cap + 3);
        cc.resize(3 * cap + 3);
        ty.resize(cap + 1);
        return ocl_gb300_path_drop(m, &d, spans.data(), spans.size() / OCL_GB300_SPAN_DOUBLES, sampling, minimumZ,
                                   xyz.data(), cc.data(), ty.data(), cap, &n, &stats);
    }
    const Path* path = nullptr;
    double minimumZ = 0.0;
    std::vector<CLPoint> clpoints;
};

class AdaptivePathDropCutter : public PathDropCutter {
   public:
    AdaptivePathDropCutter() {}
    void setMinSampling(double s) { min_sampling = s; }
    void setCosLimit(double lim) { cosLimit = lim; }

   protected:
    int call(ocl_gb300_mesh m, const ocl_gb300_cutter& d, const std::vector<double>& spans, std::vector<double>& xyz,
             std::vector<double>& cc, std::vector<int32_t>& ty, uint64_t cap, uint64_t& n) override {
        xyz.resize(3 * cap + 3);
        cc.resize(3 * cap + 3);
        ty.resize(cap + 1);
        return ocl_gb300_adaptive_path_drop(m, &d, spans.data(), spans.size() / OCL_GB300_SPAN_DOUBLES, sampling,
                                            min_sampling, cosLimit, xyz.data(), cc.data(), ty.data(), cap, &n,
                                            &stats);
    }
    double min_sampling = 0.01;
    double cosLimit = 0.999;
};

class BatchPushCutter : public Operation {
   public:
    BatchPushCutter() : fibers(new std::vector<Fiber>()) {}
    ~BatchPushCutter() override { delete fibers; }
    void setXDirection() override { x_direction = true; y_direction = false; }
    void setYDirection() override { x_direction = false; y_direction = true; }
    void appendFiber(Fiber& f) override { fibers->push_back(f); }
    void reset() override { fibers->clear(); }
    std::vector<Fiber>* getFibers() const { return fibers; }
    void run() override {
        if (!x_direction && !y_direction) {
            fail("setXDirection() or setYDirection() must be called before run()");
            return;
        }
        ocl_gb300_mesh m = mesh();
        if (!m) return;
        const size_t F = fibers->size();
        std::vector<double> fb(6 * F);
        for (size_t k = 0; k < F; ++k) {
            const Fiber& f = (*fibers)[k];
            const double v[6] = {f.p1.x, f.p1.y, f.p1.z, f.p2.x, f.p2.y, f.p2.z};
            std::memcpy(&fb[6 * k], v, sizeof(v));
        }
        ocl_gb300_cutter d = cutter->desc();
        const int dir = x_direction ? OCL_GB300_XFIBER : OCL_GB300_YFIBER;
        std::vector<uint64_t> offs(F + 1);
        uint64_t cap = 4 * F + 16;
        std::vector<double> iv, cc;
        std::vector<int32_t> ty;
        int st;
        for (;;) {
            iv.resize(2 * cap);
            cc.resize(6 * cap);
            ty.resize(2 * cap);
            st = ocl_gb300_push(m, &d, dir, fb.data(), F, offs.data(), iv.data(), cc.data(), ty.data(), cap, &stats);
            if (st != OCL_GB300_CAPACITY) break;
            cap = offs[F] + 16;
        }
        if (!check(st)) return;
        for (size_t k = 0; k < F; ++k) {
            Fiber& f = (*fibers)[k];
            f.ints.clear();
            for (uint64_t j = offs[k]; j < offs[k + 1]; ++j) {
                Interval i(iv[2 * j], iv[2 * j + 1]);
                i.lower_cc = CCPoint(cc[6 * j], cc[6 * j + 1], cc[6 * j + 2], (CCType)ty[2 * j]);
                i.upper_cc = CCPoint(cc[6 * j + 3], cc[6 * j + 4], cc[6 * j + 5], (CCType)ty[2 * j + 1]);
                f.ints.push_back(i);
            }
        }
        nCalls = (int)stats.pairs;
    }

   protected:
    std::vector<Fiber>* fibers;
    bool x_direction = false;
    bool y_direction = false;
};

// Waterline (src/algo/waterline.hpp:41-88): X and Y fibers at height z pushed
// on the GPU, woven on the host into loops.  run2() (the reference's
// SmartWeave) gives the same loops as run().
class Waterline : public Operation {
   public:
    Waterline() {}
    ~Waterline() override {}
    void setZ(const double z) { zh = z; }
    void run() override {
        ocl_gb300_mesh m = mesh();
        if (!m) return;
        ocl_gb300_cutter d = cutter->desc();
        ocl_gb300_loops h = nullptr;
        if (!check(weave(m, d, &h))) return;
        take(h);
    }
    virtual void run2() { run(); }
    std::vector<std::vector<Point>> getLoops() const { return loops; }
    std::vector<Fiber> getXFibers() const { return xfibers; }
    std::vector<Fiber> getYFibers() const { return yfibers; }
    void reset() override {
        xfibers.clear();
        yfibers.clear();
        loops.clear();
    }

   protected:
    virtual int weave(ocl_gb300_mesh m, const ocl_gb300_cutter& d, ocl_gb300_loops* h) {
        return ocl_gb300_waterline(m, &d, zh, sampling, h, &stats);
    }
    // copies the loops and fibers out of the handle and releases it
    void take(ocl_gb300_loops h) {
        uint64_t nl = 0, np = 0;
        ocl_gb300_loops_count(h, &nl, &np);
        std::vector<double> pts(3 * np);
        std::vector<uint64_t> off(nl + 1);
        ocl_gb300_loops_get(h, pts.data(), off.data());
        loops.assign(nl, std::vector<Point>());
        for (uint64_t k = 0; k < nl; ++k)
            for (uint64_t j = off[k]; j < off[k + 1]; ++j) loops[k].push_back(Point(pts[3 * j], pts[3 * j + 1], pts[3 * j + 2]));
        for (int dir = 0; dir < 2; ++dir) {
            std::vector<Fiber>& out = dir == 0 ? xfibers : yfibers;
            uint64_t nf = 0, nk = 0;
            ocl_gb300_loops_fibers(h, dir, &nf, &nk, nullptr, nullptr, nullptr, nullptr, nullptr);
            std::vector<double> fb(6 * nf), iv(2 * nk), cc(6 * nk);
            std::vector<uint64_t> fo(nf + 1);
            std::vector<int32_t> ty(2 * nk);
            ocl_gb300_loops_fibers(h, dir, &nf, &nk, fb.data(), fo.data(), iv.data(), cc.data(), ty.data());
            out.clear();
            for (uint64_t f = 0; f < nf; ++f) {
                Fiber fib(Point(fb[6 * f], fb[6 * f + 1], fb[6 * f + 2]), Point(fb[6 * f + 3], fb[6 * f + 4], fb[6 * f + 5]));
                for (uint64_t j = fo[f]; j < fo[f + 1]; ++j) {
                    Interval i(iv[2 * j], iv[2 * j + 1]);
                    i.lower_cc = CCPoint(cc[6 * j], cc[6 * j + 1], cc[6 * j + 2], (CCType)ty[2 * j]);
                    i.upper_cc = CCPoint(cc[6 * j + 3], cc[6 * j + 4], cc[6 * j + 5], (CCType)ty[2 * j + 1]);
                    fib.ints.push_back(i);
                }
                out.push_back(fib);
            }
        }
        ocl_gb300_loops_release(h);
        nCalls = (int)stats.pairs;
    }
    double zh = 0.0;
    std::vector<std::vector<Point>> loops;
    std::vector<Fiber> xfibers, yfibers;
};

// AdaptiveWaterline (src/algo/adaptivewaterline.hpp:38-92): fibers bisected
// where the loops bend; each bisection level pushed in one GPU call per
// direction.
class AdaptiveWaterline : public Waterline {
   public:
    AdaptiveWaterline() { sampling = 1.0; }
    ~AdaptiveWaterline() override {}
    void setMinSampling(double s) { min_sampling = s; }
    void setCosLimit(double lim) { cosLimit = lim; }
    void setSampling(double s) override {
        sampling = s;
        min_sampling = sampling / 10.0;
    }

   protected:
    int weave(ocl_gb300_mesh m, const ocl_gb300_cutter& d, ocl_gb300_loops* h) override {
        return ocl_gb300_adaptive_waterline(m, &d, zh, sampling, min_sampling, cosLimit, h, &stats);
    }
    double min_sampling = 0.1;
    double cosLimit = 0.999;
};

}  // namespace ocl
