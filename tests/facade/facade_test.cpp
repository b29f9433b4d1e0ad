// facade_test.cpp -- drives the C++ facade (ocl/ocl.hpp) the way client code
// written for the reference library does, for the GPU facade tests.
//
//   facade_test drop <tris.bin> <cl.bin> <out.bin> <cutter> <args...>
//   facade_test push <tris.bin> <fibers.bin> <out.bin> <dir 0|1> <cutter> <args...>
//   facade_test path <tris.bin> <spans.bin> <out.bin> <sampling> <minz> <cutter> <args...>
//   facade_test apdc <tris.bin> <spans.bin> <out.bin> <sampling> <min_sampling> <cos_limit> <cutter> <args...>
//   facade_test rotate <tris.bin> <angles.bin> <out.bin>
//   facade_test stldrop <file.stl> <cl.bin> <out.bin> <cutter> <args...>
//   facade_test waterline <tris.bin> <params.bin> <out.bin> <cutter> <args...>
//
// rotate: STLSurf::rotate(xr, yr, zr); output the triangles, then the bbox (6).
// stldrop: STLReader -> STLSurf -> BatchDropCutter, three runs on one
// surface: as read; after addTriangle of a horizontal triangle over the
// surface's bbox at maxz + 1; after rotate(0, 0, pi/2).  Output: the three
// runs' points one after the other (the device copy must follow each change).
//
// waterline: params = z, sampling, adaptive (0/1), min_sampling, cos_limit;
// Waterline (or AdaptiveWaterline) run(); output: loop count, then per loop
// its point count and points (3 doubles each), then the X and Y fiber counts.
//
// tris.bin: N x 9 doubles; cl.bin: M x 3; fibers.bin: F x 6; spans.bin: S x 11.
// cutter: cyl d l | ball d l | bull d r l | cone d angle l | ballcone d1 d2 angle
// drop/path output: per point x y z ccx ccy ccz type (7 doubles);
// push output: per fiber count, then per interval lower upper lcc(3) ucc(3) ltype utype.
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>

#include "ocl/ocl.hpp"

static std::vector<double> load(const char* path) {
    std::vector<double> v;
    FILE* f = std::fopen(path, "rb");
    if (!f) return v;
    double x;
    while (std::fread(&x, sizeof(double), 1, f) == 1) v.push_back(x);
    std::fclose(f);
    return v;
}

static std::unique_ptr<ocl::MillingCutter> make_cutter(int argc, char** argv, int k) {
    std::string kind = argv[k];
    auto a = [&](int i) { return std::atof(argv[k + 1 + i]); };
    if (kind == "cyl") return std::unique_ptr<ocl::MillingCutter>(new ocl::CylCutter(a(0), a(1)));
    if (kind == "ball") return std::unique_ptr<ocl::MillingCutter>(new ocl::BallCutter(a(0), a(1)));
    if (kind == "bull") return std::unique_ptr<ocl::MillingCutter>(new ocl::BullCutter(a(0), a(1), a(2)));
    if (kind == "cone") return std::unique_ptr<ocl::MillingCutter>(new ocl::ConeCutter(a(0), a(1), a(2)));
    if (kind == "ballcone") return std::unique_ptr<ocl::MillingCutter>(new ocl::BallConeCutter(a(0), a(1), a(2)));
    (void)argc;
    return nullptr;
}

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: facade_test drop|push|path|apdc|rotate|stldrop|waterline ...\n");
        return 2;
    }
    std::string mode = argv[1];
    std::vector<double> T = mode == "stldrop" ? std::vector<double>() : load(argv[2]), P = load(argv[3]);
    ocl::STLSurf surf;
    for (size_t i = 0; i + 9 <= T.size(); i += 9)
        surf.addTriangle(ocl::Triangle(ocl::Point(T[i], T[i + 1], T[i + 2]), ocl::Point(T[i + 3], T[i + 4], T[i + 5]),
                                       ocl::Point(T[i + 6], T[i + 7], T[i + 8])));
    std::vector<double> out;
    auto put_points = [&out](std::vector<ocl::CLPoint> pts) {
        for (ocl::CLPoint& p : pts) {
            ocl::CCPoint cc = p.getCC();
            double r[7] = {p.x, p.y, p.z, cc.x, cc.y, cc.z, (double)cc.type};
            out.insert(out.end(), r, r + 7);
        }
    };
    if (mode == "rotate") {
        if (P.size() < 3) return 2;
        surf.rotate(P[0], P[1], P[2]);
        for (const ocl::Triangle& t : surf.tris)
            for (int k = 0; k < 3; ++k) {
                out.push_back(t.p[k].x);
                out.push_back(t.p[k].y);
                out.push_back(t.p[k].z);
            }
        for (unsigned k = 0; k < 6; ++k) out.push_back(surf.bb[k]);
    } else if (mode == "stldrop") {
        std::string path = argv[2];
        std::wstring wp(path.begin(), path.end());
        ocl::STLReader reader(wp, surf);
        auto cutter = make_cutter(argc, argv, 5);
        ocl::BatchDropCutter bdc;
        bdc.setSTL(surf);
        bdc.setCutter(cutter.get());
        for (int run = 0; run < 3; ++run) {
            if (run == 1) {
                const double z = surf.bb[5] + 1.0;
                surf.addTriangle(ocl::Triangle(ocl::Point(surf.bb[0] - 10, surf.bb[2] - 10, z),
                                               ocl::Point(surf.bb[1] + 30, surf.bb[2] - 10, z),
                                               ocl::Point(surf.bb[0] - 10, surf.bb[3] + 30, z)));
            } else if (run == 2) {
                surf.rotate(0.0, 0.0, 1.5707963267948966);
            }
            bdc.clearCLPoints();
            for (size_t i = 0; i + 3 <= P.size(); i += 3) {
                ocl::CLPoint p(P[i], P[i + 1], P[i + 2]);
                bdc.appendPoint(p);
            }
            bdc.run();
            if (!bdc.lastError().empty()) return 1;
            put_points(bdc.getCLPoints());
        }
    } else if (mode == "apdc") {
        double sampling = std::atof(argv[5]), minsamp = std::atof(argv[6]), coslim = std::atof(argv[7]);
        auto cutter = make_cutter(argc, argv, 8);
        ocl::Path path;
        for (size_t i = 0; i + 11 <= P.size(); i += 11) {
            ocl::Point p1(P[i + 1], P[i + 2], P[i + 3]), p2(P[i + 4], P[i + 5], P[i + 6]), c(P[i + 7], P[i + 8], P[i + 9]);
            if (P[i] == 0.0) path.append(ocl::Line(p1, p2));
            else path.append(ocl::Arc(p1, p2, c, P[i + 10] != 0.0));
        }
        ocl::AdaptivePathDropCutter apdc;
        apdc.setSTL(surf);
        apdc.setCutter(cutter.get());
        apdc.setPath(&path);
        apdc.setSampling(sampling);
        apdc.setMinSampling(minsamp);
        apdc.setCosLimit(coslim);
        apdc.run();
        if (!apdc.lastError().empty()) return 1;
        put_points(apdc.getPoints());
    } else if (mode == "waterline") {
        auto cutter = make_cutter(argc, argv, 5);
        if (P.size() < 5) return 2;
        std::unique_ptr<ocl::Waterline> wl;
        if (P[2] != 0.0) {
            auto* a = new ocl::AdaptiveWaterline();
            a->setSampling(P[1]);
            a->setMinSampling(P[3]);
            a->setCosLimit(P[4]);
            wl.reset(a);
        } else {
            wl.reset(new ocl::Waterline());
            wl->setSampling(P[1]);
        }
        wl->setSTL(surf);
        wl->setCutter(cutter.get());
        wl->setZ(P[0]);
        wl->run();
        if (!wl->lastError().empty()) return 1;
        const std::vector<std::vector<ocl::Point>> loops = wl->getLoops();
        out.push_back((double)loops.size());
        for (const auto& lp : loops) {
            out.push_back((double)lp.size());
            for (const ocl::Point& q : lp) {
                out.push_back(q.x);
                out.push_back(q.y);
                out.push_back(q.z);
            }
        }
        out.push_back((double)wl->getXFibers().size());
        out.push_back((double)wl->getYFibers().size());
    } else if (mode == "drop") {
        auto cutter = make_cutter(argc, argv, 5);
        ocl::BatchDropCutter bdc;
        bdc.setSTL(surf);
        bdc.setCutter(cutter.get());
        for (size_t i = 0; i + 3 <= P.size(); i += 3) {
            ocl::CLPoint p(P[i], P[i + 1], P[i + 2]);
            bdc.appendPoint(p);
        }
        bdc.run();
        if (!bdc.lastError().empty()) return 1;
        for (ocl::CLPoint& p : bdc.getCLPoints()) {
            ocl::CCPoint cc = p.getCC();
            double r[7] = {p.x, p.y, p.z, cc.x, cc.y, cc.z, (double)cc.type};
            out.insert(out.end(), r, r + 7);
        }
    } else if (mode == "push") {
        int dir = std::atoi(argv[5]);
        auto cutter = make_cutter(argc, argv, 6);
        ocl::BatchPushCutter bpc;
        if (dir == 0) bpc.setXDirection(); else bpc.setYDirection();
        bpc.setSTL(surf);
        bpc.setCutter(cutter.get());
        for (size_t i = 0; i + 6 <= P.size(); i += 6) {
            ocl::Fiber f(ocl::Point(P[i], P[i + 1], P[i + 2]), ocl::Point(P[i + 3], P[i + 4], P[i + 5]));
            bpc.appendFiber(f);
        }
        bpc.run();
        if (!bpc.lastError().empty()) return 1;
        for (const ocl::Fiber& f : *bpc.getFibers()) {
            out.push_back((double)f.ints.size());
            for (const ocl::Interval& i : f.ints) {
                double r[10] = {i.lower, i.upper, i.lower_cc.x, i.lower_cc.y, i.lower_cc.z,
                                i.upper_cc.x, i.upper_cc.y, i.upper_cc.z, (double)i.lower_cc.type,
                                (double)i.upper_cc.type};
                out.insert(out.end(), r, r + 10);
            }
        }
    } else if (mode == "path") {
        double sampling = std::atof(argv[5]), minz = std::atof(argv[6]);
        auto cutter = make_cutter(argc, argv, 7);
        ocl::Path path;
        for (size_t i = 0; i + 11 <= P.size(); i += 11) {
            ocl::Point p1(P[i + 1], P[i + 2], P[i + 3]), p2(P[i + 4], P[i + 5], P[i + 6]), c(P[i + 7], P[i + 8], P[i + 9]);
            if (P[i] == 0.0) path.append(ocl::Line(p1, p2));
            else path.append(ocl::Arc(p1, p2, c, P[i + 10] != 0.0));
        }
        ocl::PathDropCutter pdc;
        pdc.setSTL(surf);
        pdc.setCutter(cutter.get());
        pdc.setPath(&path);
        pdc.setSampling(sampling);
        pdc.setZ(minz);
        pdc.run();
        if (!pdc.lastError().empty()) return 1;
        for (ocl::CLPoint& p : pdc.getPoints()) {
            ocl::CCPoint cc = p.getCC();
            double r[7] = {p.x, p.y, p.z, cc.x, cc.y, cc.z, (double)cc.type};
            out.insert(out.end(), r, r + 7);
        }
    } else {
        return 2;
    }
    FILE* f = std::fopen(argv[4], "wb");
    if (!f) return 3;
    std::fwrite(out.data(), sizeof(double), out.size(), f);
    std::fclose(f);
    return 0;
}
