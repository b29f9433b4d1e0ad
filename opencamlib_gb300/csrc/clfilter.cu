// clfilter.cu -- LineCLFilter (src/common/lineclfilter.cpp:40-77), host code:
// drops CL points that lie within a tolerance of the line through their
// neighbours in a run, keeping the first and the last point.
//
// The filter walks the points once with three cursors: a run's start p0, a
// probe p2 and a middle p1 that advances every second accepted probe; p2 is
// accepted while the middle point's distance to the line (p0, p2) is below
// the tolerance (Point::closestPoint, src/geo/point.cpp:166-172, with the
// reference's operation order: no fused multiply-add, so the decisions are
// the reference's).  On the first rejected probe the last accepted point is
// kept and starts the next run.  Output: the indices of the kept points, in
// order.  A filter over one point list is sequential; separate paths are
// independent and can be filtered concurrently by the caller.
#include <cmath>
#include <cstdint>

#include "util.cuh"

namespace {

struct P3 {
    double x, y, z;
};

inline P3 at(const double* xyz, uint64_t i) { return P3{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]}; }

// |closestPoint(p0, p2) - p1| for the middle point p1
inline double line_distance(const P3& p1, const P3& p0, const P3& p2) {
    const double vx = p2.x - p0.x, vy = p2.y - p0.y, vz = p2.z - p0.z;
    const double wx = p1.x - p0.x, wy = p1.y - p0.y, wz = p1.z - p0.z;
    const double u = (wx * vx + wy * vy + wz * vz) / (vx * vx + vy * vy + vz * vz);
    const double cx = p0.x + vx * u, cy = p0.y + vy * u, cz = p0.z + vz * u;
    const double dx = cx - p1.x, dy = cy - p1.y, dz = cz - p1.z;
    return std::sqrt(dx * dx + dy * dy + dz * dz);
}

}  // namespace

using namespace oclg;

extern "C" int ocl_gb300_line_filter(const double* xyz, uint64_t n, double tol, uint64_t* keep, uint64_t* nkeep) {
    if (!nkeep || (n && (!xyz || !keep))) {
        set_error("line_filter: null argument");
        return OCL_GB300_BAD_ARG;
    }
    *nkeep = 0;
    if (n < 2) {  // the reference leaves lists of 0 or 1 points as they are
        for (uint64_t i = 0; i < n; ++i) keep[(*nkeep)++] = i;
        return OCL_GB300_OK;
    }
    uint64_t p0 = 0, p1 = 1, p2 = 2, last_good = 1;
    keep[(*nkeep)++] = 0;
    bool even = true;
    while (p2 < n) {
        if (line_distance(at(xyz, p1), at(xyz, p0), at(xyz, p2)) < tol) {
            last_good = p2;
            ++p2;
            if (even) ++p1;
            even = !even;
        } else {
            keep[(*nkeep)++] = last_good;
            p0 = last_good;
            p1 = p2;
            last_good = p1;
            ++p2;
        }
    }
    keep[(*nkeep)++] = n - 1;
    return OCL_GB300_OK;
}
