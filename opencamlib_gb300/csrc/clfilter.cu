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
// order.
//
// The device pass filters many paths at once, one warp per path.  While
// probes are accepted the state moves on without looking at anything but
// the run start: after k accepted probes the middle cursor has advanced
// ceil(k/2) or floor(k/2) times (it moves on every second accept, starting
// with the first when the parity flag is set).  So lane k tests probe
// p2 + k against its middle point as if the k probes before it were
// accepted, and the first lane that rejects (a ballot) says how far the run
// really goes: up to 32 probes per step, each decided with the host code's
// arithmetic.
#include <cmath>
#include <cstdint>
#include <string>

#include "util.cuh"

namespace {

struct P3 {
    double x, y, z;
};

__host__ __device__ inline P3 at(const double* xyz, uint64_t i) {
    return P3{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
}

// |closestPoint(p0, p2) - p1| for the middle point p1
__host__ __device__ inline double line_distance(const P3& p1, const P3& p0, const P3& p2) {
    const double vx = p2.x - p0.x, vy = p2.y - p0.y, vz = p2.z - p0.z;
    const double wx = p1.x - p0.x, wy = p1.y - p0.y, wz = p1.z - p0.z;
    const double u = (wx * vx + wy * vy + wz * vz) / (vx * vx + vy * vy + vz * vz);
    const double cx = p0.x + vx * u, cy = p0.y + vy * u, cz = p0.z + vz * u;
    const double dx = cx - p1.x, dy = cy - p1.y, dz = cz - p1.z;
    return sqrt(dx * dx + dy * dy + dz * dz);
}

// One warp per path: path p is points [off[p], off[p+1]) of xyz; the kept
// indices (within the path) go to keep[off[p] ...], their count to nkeep[p].
__global__ void __launch_bounds__(256) k_line_filter(const double* __restrict__ xyz, const uint64_t* __restrict__ off,
                                                     uint64_t npaths, double tol, uint64_t* __restrict__ keep,
                                                     uint64_t* __restrict__ nkeep) {
    const uint64_t p = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    if (p >= npaths) return;  // whole warps leave together
    const uint64_t b = off[p], n = off[p + 1] - b;
    const double* X = xyz + 3 * b;
    uint64_t* K = keep + b;
    if (n < 2) {
        if (lane == 0) {
            for (uint64_t i = 0; i < n; ++i) K[i] = i;
            nkeep[p] = n;
        }
        return;
    }
    uint64_t p0 = 0, p1 = 1, p2 = 2, last = 1, cnt = 1;
    bool even = true;
    if (lane == 0) K[0] = 0;
    while (p2 < n) {
        const uint64_t q = p2 + lane;
        const bool valid = q < n;
        bool acc = false;
        if (valid) {
            const uint64_t m = p1 + (even ? (lane + 1) / 2 : lane / 2);
            acc = line_distance(at(X, m), at(X, p0), at(X, q)) < tol;
        }
        const unsigned rej = __ballot_sync(0xffffffffu, valid && !acc);
        const unsigned vm = __ballot_sync(0xffffffffu, valid);
        const unsigned f = rej ? (unsigned)(__ffs(rej) - 1) : (unsigned)__popc(vm);  // probes accepted
        if (f > 0) {
            last = p2 + f - 1;
            p1 += even ? (f + 1) / 2 : f / 2;
            if (f & 1u) even = !even;
        }
        if (rej) {
            if (lane == 0) K[cnt] = last;
            ++cnt;
            p0 = last;
            p1 = p2 + f;
            last = p1;
            p2 = p2 + f + 1;
        } else {
            p2 += f;
        }
    }
    if (lane == 0) {
        K[cnt] = n - 1;
        nkeep[p] = cnt + 1;
    }
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

extern "C" int ocl_gb300_line_filter_device(const double* d_xyz, const uint64_t* d_offsets, uint64_t npaths,
                                            double tol, uint64_t* d_keep, uint64_t* d_nkeep, void* stream) {
    if (npaths == 0) return OCL_GB300_OK;
    if (!d_xyz || !d_offsets || !d_keep || !d_nkeep) {
        set_error("line_filter_device: null argument");
        return OCL_GB300_BAD_ARG;
    }
    const uint64_t blocks = (npaths + 7) / 8;  // 8 warps (paths) per block
    if (blocks > 0x7fffffffull) {
        set_error("line_filter_device: too many paths");
        return OCL_GB300_BAD_ARG;
    }
    k_line_filter<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(d_xyz, d_offsets, npaths, tol, d_keep, d_nkeep);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("line_filter_device: ") + cudaGetErrorString(e));
        return e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? OCL_GB300_NO_DEVICE : OCL_GB300_DEVICE_ERROR;
    }
    return OCL_GB300_OK;
}
