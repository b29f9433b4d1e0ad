// waterline.cu -- Waterline and AdaptiveWaterline (src/algo/waterline.cpp,
// src/algo/adaptivewaterline.cpp): X and Y fibers at a height pushed on the
// device (push_run), woven on the host into waterline loops.
//
// The weave.  The reference (src/algo/simple_weave.cpp:55-161,
// src/algo/weave.cpp:49-73) inserts every crossing of an X interval and a Y
// interval into a half-edge graph, splicing next pointers so that at a
// crossing an arriving edge continues with a right turn and at an interval
// end it turns back, drops X intervals without crossings, and then walks the
// faces that hold interval ends.  That graph is fixed by the fibers alone:
// its vertices are the crossings (strictly inside both intervals) and the
// ends of every interval with at least one crossing, its edges join
// neighbouring vertices along each interval.  So the walk is taken here on
// that arrangement directly, without building it: from an interval end,
// move along the interval to the nearest crossing (found by scanning the
// perpendicular fibers in coordinate order from the current position), turn
// right onto the crossing interval, and so on, turning back at ends.  The
// work is proportional to the lengths of the loops walked, not to the number
// of crossings (the reference builds all of them: about N x N vertices for N
// fibers per direction).
//
// Loop order: the reference starts each loop at the interval end whose
// graph vertex has the lowest address (std::set of vertex descriptors), which
// depends on its allocator.  Here the interval ends are numbered X intervals
// first (fiber order, then interval order; lower end before upper end), then
// Y intervals likewise; every loop starts at its lowest-numbered end and the
// loops are listed in that order.  The loops as cyclic sequences of points
// are the reference's.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "util.cuh"
#include "waterline.cuh"

namespace oclg {

int make_cutter_params(const ocl_gb300_cutter& in, CutterP& cp);
int push_run(Mesh& m, const CutterP& cp, int dir, const double* fibers, uint64_t F, uint64_t* offsets, double* ival,
             double* cc, int32_t* cctype, uint64_t cap, ocl_gb300_stats* stats);

namespace {

// Fiber::point (src/algo/fiber.cpp:102-105): p1 + t * (p2 - p1).
inline void fiber_point(const double* f, double t, double* p) {
    for (int k = 0; k < 3; ++k) p[k] = f[k] + t * (f[3 + k] - f[k]);
}

// One direction's fibers as the weave reads them.
struct Axis {
    int along;                      // 0: X fibers (coordinate x along, fixed y); 1: Y fibers
    const FiberSet* fs;
    std::vector<double> fixed;      // per fiber: p1.y (X fibers) or p1.x (Y fibers)
    std::vector<uint32_t> order;    // fibers by fixed coordinate (stable)
    std::vector<double> sorted;     // fixed coordinates in that order
    std::vector<double> a, b;       // per interval: coordinate along the fiber of point(lower), point(upper)
    std::vector<uint32_t> fiber_of; // per interval
    std::vector<uint8_t> has;       // per interval: at least one crossing
};

void make_axis(const FiberSet& fs, int along, Axis& A) {
    A.along = along;
    A.fs = &fs;
    const uint64_t F = fs.count();
    A.fixed.resize(F);
    for (uint64_t k = 0; k < F; ++k) A.fixed[k] = fs.fib[6 * k + (along == 0 ? 1 : 0)];
    A.order.resize(F);
    for (uint64_t k = 0; k < F; ++k) A.order[k] = (uint32_t)k;
    std::stable_sort(A.order.begin(), A.order.end(), [&](uint32_t p, uint32_t q) { return A.fixed[p] < A.fixed[q]; });
    A.sorted.resize(F);
    for (uint64_t k = 0; k < F; ++k) A.sorted[k] = A.fixed[A.order[k]];
    const uint64_t K = F ? fs.off[F] : 0;
    A.a.resize(K);
    A.b.resize(K);
    A.fiber_of.resize(K);
    A.has.assign(K, 0);
    for (uint64_t k = 0; k < F; ++k)
        for (uint64_t j = fs.off[k]; j < fs.off[k + 1]; ++j) {
            double p[3], q[3];
            fiber_point(&fs.fib[6 * k], fs.ival[2 * j], p);
            fiber_point(&fs.fib[6 * k], fs.ival[2 * j + 1], q);
            A.a[j] = p[along];
            A.b[j] = q[along];
            A.fiber_of[j] = (uint32_t)k;
        }
}

// The first interval of fiber g (of axis P) holding coordinate c strictly
// inside, or -1 (SimpleWeave::build's crossing test, simple_weave.cpp:85-90).
inline int64_t holding(const Axis& P, uint32_t g, double c) {
    const FiberSet& fs = *P.fs;
    for (uint64_t j = fs.off[g]; j < fs.off[g + 1]; ++j)
        if (P.a[j] < c && c < P.b[j]) return (int64_t)j;
    return -1;
}

// From coordinate c on interval k of axis A, heading s (+1 / -1): the first
// crossing strictly between c and the interval's end in that direction (the
// perpendicular interval, its coordinate in *at), or -1 (the end comes first).
int64_t next_crossing(const Axis& A, const Axis& P, uint64_t k, double c, int s, double* at) {
    const double F = A.fixed[A.fiber_of[k]];
    const size_t n = P.sorted.size();
    if (s > 0) {
        const double end = A.b[k];
        for (size_t i = std::upper_bound(P.sorted.begin(), P.sorted.end(), c) - P.sorted.begin();
             i < n && P.sorted[i] < end; ++i) {
            const int64_t j = holding(P, P.order[i], F);
            if (j >= 0) {
                *at = P.sorted[i];
                return j;
            }
        }
    } else {
        const double end = A.a[k];
        for (size_t i = std::lower_bound(P.sorted.begin(), P.sorted.end(), c) - P.sorted.begin(); i > 0 &&
                                                                                                P.sorted[i - 1] > end;
             --i) {
            const int64_t j = holding(P, P.order[i - 1], F);
            if (j >= 0) {
                *at = P.sorted[i - 1];
                return j;
            }
        }
    }
    return -1;
}

}  // namespace

// Weave::build + face_traverse + getLoops on the fibers in `out.fibers`.
int weave_loops(LoopSet& out) {
    Axis ax[2];
    make_axis(out.fibers[0], 0, ax[0]);
    make_axis(out.fibers[1], 1, ax[1]);
    for (int d = 0; d < 2; ++d)
        for (uint64_t k = 0; k < ax[d].a.size(); ++k) {
            double at;
            ax[d].has[k] = ax[d].a[k] < ax[d].b[k] && next_crossing(ax[d], ax[1 - d], k, ax[d].a[k], 1, &at) >= 0;
        }
    const uint64_t KX = ax[0].a.size(), KY = ax[1].a.size();
    // interval end id: 2 * (X interval, or KX + Y interval) + (0 lower, 1 upper)
    std::vector<uint8_t> seen(2 * (KX + KY), 0);
    const uint64_t limit = 64ull * (KX * ax[1].sorted.size() + KY * ax[0].sorted.size()) + 1024;
    uint64_t steps = 0;
    out.pts.clear();
    out.off.assign(1, 0);
    for (uint64_t id0 = 0; id0 < seen.size(); ++id0) {
        int d = id0 / 2 < KX ? 0 : 1;
        uint64_t k = d == 0 ? id0 / 2 : id0 / 2 - KX;
        if (seen[id0] || !ax[d].has[k]) continue;
        uint64_t id = id0;
        do {
            seen[id] = 1;
            const int end = (int)(id & 1);
            {
                double p[3];
                const FiberSet& fs = *ax[d].fs;
                fiber_point(&fs.fib[6 * ax[d].fiber_of[k]], fs.ival[2 * k + end], p);
                out.pts.insert(out.pts.end(), p, p + 3);
            }
            // leave the end along its interval, then turn right at every
            // crossing until an interval end is reached
            double c = end ? ax[d].b[k] : ax[d].a[k];
            int s = end ? -1 : 1;
            for (;;) {
                if (++steps > limit) {
                    set_error("weave: loop walk did not close (inconsistent fibers)");
                    return OCL_GB300_ITER_LIMIT;
                }
                double at;
                const int64_t j = next_crossing(ax[d], ax[1 - d], k, c, s, &at);
                if (j < 0) break;
                c = ax[d].fixed[ax[d].fiber_of[k]];
                if (d == 0) s = -s;  // east -> south, west -> north; north -> east, south -> west
                d = 1 - d;
                k = (uint64_t)j;
            }
            id = 2 * (d == 0 ? k : KX + k) + (s > 0 ? 1 : 0);
        } while (id != id0);
        out.off.push_back(out.pts.size() / 3);
    }
    return OCL_GB300_OK;
}

namespace {

// Pushes the fibers in fs.fib (direction dir) on the device and fills the
// intervals (retrying once with the exact capacity when the first guess is
// too small).
int push_fibers(Mesh& m, const CutterP& cp, int dir, FiberSet& fs, ocl_gb300_stats* acc) {
    const uint64_t F = fs.fib.size() / 6;
    fs.off.assign(F + 1, 0);
    if (F == 0) return OCL_GB300_OK;
    uint64_t cap = std::max<uint64_t>(4 * F, 1024);
    for (int attempt = 0; attempt < 2; ++attempt) {
        fs.ival.resize(2 * cap);
        fs.cc.resize(6 * cap);
        fs.type.resize(2 * cap);
        ocl_gb300_stats st;
        std::memset(&st, 0, sizeof(st));
        const int r = push_run(m, cp, dir, fs.fib.data(), F, fs.off.data(), fs.ival.data(), fs.cc.data(),
                               fs.type.data(), cap, &st);
        if (acc) {
            acc->pairs += st.pairs;
            acc->screened += st.screened;
            acc->refined += st.refined;
            acc->iter_limit_hits += st.iter_limit_hits;
            acc->kernel_ms += st.kernel_ms;
            acc->launches += 2;
        }
        if (r == OCL_GB300_CAPACITY && attempt == 0) {
            cap = fs.off[F];
            continue;
        }
        if (r) return r;
        const uint64_t K = fs.off[F];
        fs.ival.resize(2 * K);
        fs.cc.resize(6 * K);
        fs.type.resize(2 * K);
        return OCL_GB300_OK;
    }
    return OCL_GB300_CAPACITY;
}

// Waterline::generate_range (waterline.cpp:169-178): N + 1 values from start
// in steps of (end - start) / N, accumulated.
std::vector<double> generate_range(double start, double end, int N) {
    std::vector<double> out;
    const double d = (end - start) / (double)N;
    double v = start;
    for (int n = 0; n < N + 1; ++n) {
        out.push_back(v);
        v = v + d;
    }
    return out;
}

struct Extent {
    double minx, maxx, miny, maxy;
};

// The fiber extent of Waterline::init_fibers / adaptive_sampling_run: the
// mesh bbox grown by two cutter radii (waterline.cpp:143-147).
Extent extent_of(const Mesh& m, const CutterP& cp) {
    const double r = cp.radius;
    return {m.bb[0] - 2 * r, m.bb[1] + 2 * r, m.bb[2] - 2 * r, m.bb[3] + 2 * r};
}

void add_fiber(FiberSet& fs, double x1, double y1, double x2, double y2, double z) {
    const double f[6] = {x1, y1, z, x2, y2, z};
    fs.fib.insert(fs.fib.end(), f, f + 6);
}

int check_args(const Mesh& m, double sampling) {
    if (!(sampling > 0.0) || !std::isfinite(sampling)) {
        set_error("waterline: sampling must be positive");
        return OCL_GB300_BAD_ARG;
    }
    if (m.n == 0) {
        set_error("waterline: empty mesh");
        return OCL_GB300_BAD_ARG;
    }
    return OCL_GB300_OK;
}

// Waterline::init_fibers (waterline.cpp:143-165) at each height, appended.
void init_fibers(const Extent& e, double sampling, const double* zs, uint64_t nz, FiberSet& xs, FiberSet& ys) {
    const int Nx = (int)((e.maxx - e.minx) / sampling);
    const int Ny = (int)((e.maxy - e.miny) / sampling);
    const std::vector<double> xv = generate_range(e.minx, e.maxx, Nx);
    const std::vector<double> yv = generate_range(e.miny, e.maxy, Ny);
    for (uint64_t l = 0; l < nz; ++l) {
        for (double y : yv) add_fiber(xs, e.minx, y, e.maxx, y, zs[l]);
        for (double x : xv) add_fiber(ys, x, e.miny, x, e.maxy, zs[l]);
    }
}

// The fibers [f0, f1) of a set as a set of their own.
void slice(const FiberSet& in, uint64_t f0, uint64_t f1, FiberSet& out) {
    out.fib.assign(in.fib.begin() + 6 * f0, in.fib.begin() + 6 * f1);
    const uint64_t k0 = in.off[f0], k1 = in.off[f1];
    out.off.resize(f1 - f0 + 1);
    for (uint64_t f = f0; f <= f1; ++f) out.off[f - f0] = in.off[f] - k0;
    out.ival.assign(in.ival.begin() + 2 * k0, in.ival.begin() + 2 * k1);
    out.cc.assign(in.cc.begin() + 6 * k0, in.cc.begin() + 6 * k1);
    out.type.assign(in.type.begin() + 2 * k0, in.type.begin() + 2 * k1);
}

// Weaves every level on its own host thread pool (the levels are independent).
int weave_all(std::vector<LoopSet>& sets) {
    std::atomic<size_t> next{0};
    std::atomic<int> status{OCL_GB300_OK};
    const unsigned nt = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)sets.size()));
    auto work = [&]() {
        for (size_t l; (l = next.fetch_add(1)) < sets.size();) {
            const int st = weave_loops(sets[l]);
            if (st) status = st;
        }
    };
    if (nt == 1) {
        work();
    } else {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; ++t) th.emplace_back(work);
        for (auto& t : th) t.join();
    }
    return status;
}

// Point::normalize and dot (src/geo/point.cpp:60-79): x * (1 / norm).
inline void normalize3(double* v) {
    const double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (n != 0.0) {
        const double r = 1 / n;
        v[0] *= r;
        v[1] *= r;
        v[2] *= r;
    }
}

// AdaptiveWaterline::flat on three CL points (adaptivewaterline.cpp:213-220).
bool flat_points(const double* a, const double* b, const double* c, double cos_limit) {
    double v1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    double v2[3] = {c[0] - b[0], c[1] - b[1], c[2] - b[2]};
    normalize3(v1);
    normalize3(v2);
    const double dot = v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2];
    return dot > cos_limit;
}

// A growing set of single fibers of one direction, pushed level by level.
struct AdaptiveDir {
    int dir;                      // OCL_GB300_XFIBER / YFIBER
    std::vector<double> fib;      // 6 per fiber
    std::vector<uint64_t> off{0}; // intervals per fiber, CSR
    std::vector<double> ival, cc;
    std::vector<int32_t> type;
    uint64_t count() const { return fib.size() / 6; }
    double coord(uint64_t f) const { return fib[6 * f + (dir == OCL_GB300_XFIBER ? 1 : 0)]; }
    uint64_t size(uint64_t f) const { return off[f + 1] - off[f]; }
    void cl(uint64_t f, uint64_t n, int upper, double* p) const {
        fiber_point(&fib[6 * f], ival[2 * (off[f] + n) + upper], p);
    }
};

// AdaptiveWaterline::flat on three fibers (adaptivewaterline.cpp:189-211).
bool flat_fibers(const AdaptiveDir& A, uint64_t s, uint64_t m, uint64_t e, double cos_limit) {
    if (A.size(s) != A.size(e) || A.size(s) != A.size(m) || A.size(m) != A.size(e)) return false;
    for (uint64_t n = 0; n < A.size(s); ++n) {
        double p[3], q[3], r[3];
        A.cl(s, n, 1, p);
        A.cl(m, n, 1, q);
        A.cl(e, n, 1, r);
        if (!flat_points(p, q, r, cos_limit)) return false;
        A.cl(s, n, 0, p);
        A.cl(m, n, 0, q);
        A.cl(e, n, 0, r);
        if (!flat_points(p, q, r, cos_limit)) return false;
    }
    return true;
}

// Pushes the fibers [from, count) of A and appends their intervals.
int push_new(Mesh& m, const CutterP& cp, AdaptiveDir& A, uint64_t from, ocl_gb300_stats* acc) {
    FiberSet fs;
    fs.fib.assign(A.fib.begin() + 6 * from, A.fib.end());
    int st = push_fibers(m, cp, A.dir, fs, acc);
    if (st) return st;
    const uint64_t base = A.off.back();
    for (uint64_t f = 1; f < fs.off.size(); ++f) A.off.push_back(base + fs.off[f]);
    A.ival.insert(A.ival.end(), fs.ival.begin(), fs.ival.end());
    A.cc.insert(A.cc.end(), fs.cc.begin(), fs.cc.end());
    A.type.insert(A.type.end(), fs.type.begin(), fs.type.end());
    return OCL_GB300_OK;
}

struct Seg {
    double t0, t1;
    uint64_t f0, f1, fm = 0;
    int64_t left = -1, right = -1;
    bool emit = false;
};

// AdaptiveWaterline::xfiber_adaptive_sample / yfiber_adaptive_sample
// (adaptivewaterline.cpp:141-187) for both directions, one bisection level
// at a time: every open segment's mid fiber of a level is pushed in one
// device call per direction, then each segment splits, keeps its stop fiber
// or ends; the kept fibers are listed in the recursion's depth-first order.
int adaptive_fibers(Mesh& m, const CutterP& cp, double zh, double sampling, double min_sampling, double cos_limit,
                    FiberSet out[2], ocl_gb300_stats* acc) {
    const Extent e = extent_of(m, cp);
    // the LineSpan from (minx, miny, zh) to (maxx, maxy, zh); Line::getPoint
    // (src/geo/line.cpp:45-47) is (p2 - p1) * t + p1
    const double p1[3] = {e.minx, e.miny, zh}, p2[3] = {e.maxx, e.maxy, zh};
    auto span = [&](double t, int k) { return (p2[k] - p1[k]) * t + p1[k]; };
    for (int d = 0; d < 2; ++d) {
        AdaptiveDir A;
        A.dir = d == 0 ? OCL_GB300_XFIBER : OCL_GB300_YFIBER;
        auto mk = [&](double t) {
            const double c = span(t, d == 0 ? 1 : 0);
            const double f[6] = {d == 0 ? e.minx : c, d == 0 ? c : e.miny, zh, d == 0 ? e.maxx : c, d == 0 ? c : e.maxy, zh};
            A.fib.insert(A.fib.end(), f, f + 6);
            return A.count() - 1;
        };
        const uint64_t fs0 = mk(0.0), fs1 = mk(1.0);
        int st = push_new(m, cp, A, 0, acc);
        if (st) return st;
        std::vector<Seg> segs;
        segs.push_back({0.0, 1.0, fs0, fs1});
        std::vector<int64_t> open{0};
        for (int level = 0; !open.empty(); ++level) {
            if (level > 64) {
                set_error("adaptive waterline: sampling did not converge (min_sampling too small)");
                return OCL_GB300_ITER_LIMIT;
            }
            const uint64_t from = A.count();
            for (int64_t s : open) {
                Seg& g = segs[s];
                const double mid_t = g.t0 + (g.t1 - g.t0) / 2.0;
                g.fm = mk(mid_t);
            }
            st = push_new(m, cp, A, from, acc);
            if (st) return st;
            std::vector<int64_t> next;
            for (int64_t s : open) {
                const Seg g = segs[s];
                const double fw_step = std::fabs(A.coord(g.f0) - A.coord(g.f1));
                bool split = false;
                if (fw_step > sampling) split = true;
                else if (!flat_fibers(A, g.f0, g.fm, g.f1, cos_limit)) split = fw_step > min_sampling;
                else segs[s].emit = true;
                if (split) {
                    const double mid_t = g.t0 + (g.t1 - g.t0) / 2.0;
                    segs[s].left = (int64_t)segs.size();
                    segs.push_back({g.t0, mid_t, g.f0, g.fm});
                    segs[s].right = (int64_t)segs.size();
                    segs.push_back({mid_t, g.t1, g.fm, g.f1});
                    next.push_back(segs[s].left);
                    next.push_back(segs[s].right);
                }
            }
            open.swap(next);
        }
        // the kept fibers in the recursion's order: the start fiber, then
        // each flat segment's stop fiber, depth first
        std::vector<uint64_t> keep{fs0};
        std::vector<int64_t> stack{0};
        while (!stack.empty()) {
            const Seg& g = segs[stack.back()];
            stack.pop_back();
            if (g.left >= 0) {
                stack.push_back(g.right);
                stack.push_back(g.left);
            } else if (g.emit) {
                keep.push_back(g.f1);
            }
        }
        FiberSet& o = out[d];
        o = FiberSet();
        o.off.push_back(0);
        for (uint64_t f : keep) {
            o.fib.insert(o.fib.end(), A.fib.begin() + 6 * f, A.fib.begin() + 6 * f + 6);
            const uint64_t k0 = A.off[f], k1 = A.off[f + 1];
            o.ival.insert(o.ival.end(), A.ival.begin() + 2 * k0, A.ival.begin() + 2 * k1);
            o.cc.insert(o.cc.end(), A.cc.begin() + 6 * k0, A.cc.begin() + 6 * k1);
            o.type.insert(o.type.end(), A.type.begin() + 2 * k0, A.type.begin() + 2 * k1);
            o.off.push_back(o.off.back() + (k1 - k0));
        }
    }
    return OCL_GB300_OK;
}

}  // namespace

// Waterline::run at each of nz heights: one device push per direction for
// all heights' fibers, then the levels woven in parallel on the host.
int waterline_run(Mesh& m, const CutterP& cp, const double* zs, uint64_t nz, double sampling,
                  std::vector<LoopSet>& out, ocl_gb300_stats* stats) {
    int st = check_args(m, sampling);
    if (st) return st;
    const Extent e = extent_of(m, cp);
    FiberSet xs, ys;
    init_fibers(e, sampling, zs, nz, xs, ys);
    st = push_fibers(m, cp, OCL_GB300_XFIBER, xs, stats);
    if (st) return st;
    st = push_fibers(m, cp, OCL_GB300_YFIBER, ys, stats);
    if (st) return st;
    out.assign(nz, LoopSet());
    const uint64_t nxf = nz ? xs.count() / nz : 0, nyf = nz ? ys.count() / nz : 0;
    for (uint64_t l = 0; l < nz; ++l) {
        slice(xs, l * nxf, (l + 1) * nxf, out[l].fibers[0]);
        slice(ys, l * nyf, (l + 1) * nyf, out[l].fibers[1]);
    }
    return weave_all(out);
}

// AdaptiveWaterline::run (adaptivewaterline.cpp:62-139) at height zh.
int adaptive_waterline_run(Mesh& m, const CutterP& cp, double zh, double sampling, double min_sampling,
                           double cos_limit, LoopSet& out, ocl_gb300_stats* stats) {
    int st = check_args(m, sampling);
    if (st) return st;
    if (!(min_sampling > 0.0) || !std::isfinite(min_sampling)) {
        set_error("adaptive waterline: min_sampling must be positive");
        return OCL_GB300_BAD_ARG;
    }
    st = adaptive_fibers(m, cp, zh, sampling, min_sampling, cos_limit, out.fibers, stats);
    if (st) return st;
    return weave_loops(out);
}

}  // namespace oclg
