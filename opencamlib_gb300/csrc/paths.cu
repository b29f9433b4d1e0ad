// paths.cu -- PathDropCutter and AdaptivePathDropCutter on the GPU.
//
// Span sampling (Line/Arc getPoint) is host work; every drop goes through the
// batched device drop (drop_run).  The adaptive sampler is restated as a
// level-synchronous bisection: all midpoints of one level are dropped in one
// batch, and the emitted points are put back into the reference's
// depth-first order (which is ascending parameter order within a span).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "drop.cuh"
#include "paths.cuh"
#include "util.cuh"

namespace oclg {

static const double PI_REF = 3.1415926535897932;  // common/numeric.hpp:38

// Arc::xyIncludedAngle (geo/arc.cpp:73-94)
static double xy_included_angle(const double* v1, const double* v2, bool dir) {
    int d = dir ? 1 : (-1);
    double inc = v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2];
    if (inc > 1. - 1.0e-10) return 0;
    if (inc < -1. + 1.0e-10)
        inc = PI_REF;
    else {
        if (inc > 1.0) inc = 1.0;
        inc = std::acos(inc);
        double x = v1[0] * v2[1] - v1[1] * v2[0];
        if (d * x < 0) inc = 2 * PI_REF - inc;
    }
    return d * inc;
}

static bool span_init(SpanH& s, const double* v) {
    s.type = (int)v[0];
    for (int a = 0; a < 3; ++a) {
        s.p1[a] = v[1 + a];
        s.p2[a] = v[4 + a];
        s.c[a] = v[7 + a];
    }
    s.dir = v[10] != 0.0;
    for (int k = 0; k < 11; ++k)
        if (!std::isfinite(v[k])) return false;
    if (s.type == 1) {
        // Arc::setProperties (geo/arc.cpp:43-51)
        double vs[3] = {-(s.p1[1] - s.c[1]), s.p1[0] - s.c[0], s.p1[2] - s.c[2]};
        double ve[3] = {-(s.p2[1] - s.c[1]), s.p2[0] - s.c[0], s.p2[2] - s.c[2]};
        s.radius = std::sqrt(vs[0] * vs[0] + vs[1] * vs[1]);
        double n1 = std::sqrt(vs[0] * vs[0] + vs[1] * vs[1] + vs[2] * vs[2]);
        double n2 = std::sqrt(ve[0] * ve[0] + ve[1] * ve[1] + ve[2] * ve[2]);
        if (n1 != 0.0) for (int a = 0; a < 3; ++a) vs[a] = vs[a] * (1 / n1);
        if (n2 != 0.0) for (int a = 0; a < 3; ++a) ve[a] = ve[a] * (1 / n2);
        s.length = std::fabs(xy_included_angle(vs, ve, s.dir)) * s.radius;
        return s.radius > 0.0;
    }
    if (s.type != 0) return false;
    double dx = s.p2[0] - s.p1[0], dy = s.p2[1] - s.p1[1];
    s.length = std::sqrt(dx * dx + dy * dy);  // Line::length2d (geo/line.cpp:40-42)
    return true;
}

// Line::getPoint (geo/line.cpp:44-46), Arc::getPoint (geo/arc.cpp:53-71)
static void span_point(const SpanH& s, double t, double* out) {
    if (s.type == 0) {
        for (int a = 0; a < 3; ++a) out[a] = (s.p2[a] - s.p1[a]) * t + s.p1[a];
        return;
    }
    if (std::fabs(t) < 0.00000000000001) {
        std::memcpy(out, s.p1, 3 * sizeof(double));
        return;
    }
    if (std::fabs(t - 1.0) < 0.00000000000001) {
        std::memcpy(out, s.p2, 3 * sizeof(double));
        return;
    }
    double d = t * s.length;
    if (!s.dir) d = -d;
    double vx = s.p1[0] - s.c[0], vy = s.p1[1] - s.c[1], vz = s.p1[2] - s.c[2];
    double ang = d / s.radius;
    double ca = std::cos(ang), sa = std::sin(ang);
    double tmp = -vy * sa + vx * ca;  // Point::xyRotate (geo/point.cpp:85-89)
    vy = vx * sa + ca * vy;
    vx = tmp;
    out[0] = vx + s.c[0];
    out[1] = vy + s.c[1];
    out[2] = vz + s.c[2];
}

// Batch drop of host points through the device path.
// Device and pinned host buffers of the path drivers, kept by the calling
// thread across batches (the adaptive driver drops one batch per level).
struct PathIO {
    DevBuf<double> dcl, dz, dcc;
    DevBuf<int32_t> dty;
    double* hcl = nullptr;
    double* hz = nullptr;
    double* hcc = nullptr;
    int32_t* hty = nullptr;
    uint64_t cap = 0;
    bool ensure(uint64_t M) {
        if (M <= cap) return true;
        const uint64_t c = std::max<uint64_t>(M, 4096);
        if (!dcl.alloc(3 * c) || !dz.alloc(c) || !dcc.alloc(3 * c) || !dty.alloc(c)) return false;
        cudaFreeHost(hcl);
        cudaFreeHost(hz);
        cudaFreeHost(hcc);
        cudaFreeHost(hty);
        hcl = hz = hcc = nullptr;
        hty = nullptr;
        if (cudaMallocHost(&hcl, 3 * c * sizeof(double)) != cudaSuccess ||
            cudaMallocHost(&hz, c * sizeof(double)) != cudaSuccess ||
            cudaMallocHost(&hcc, 3 * c * sizeof(double)) != cudaSuccess ||
            cudaMallocHost(&hty, c * sizeof(int32_t)) != cudaSuccess) {
            cap = 0;
            return false;
        }
        cap = c;
        return true;
    }
};
static thread_local PathIO tl_path_io;

static int drop_host(Mesh& m, const CutterP& cp, const std::vector<double>& cl, std::vector<double>& z,
                     std::vector<double>& cc, std::vector<int32_t>& ty, ocl_gb300_stats* acc) {
    const uint64_t M = cl.size() / 3;
    z.resize(M);
    cc.resize(3 * M);
    ty.resize(M);
    if (M == 0) return OCL_GB300_OK;
    PathIO& io = tl_path_io;
    if (!io.ensure(M)) return OCL_GB300_OOM;
    std::memcpy(io.hcl, cl.data(), 3 * M * sizeof(double));
    CK(cudaMemcpyAsync(io.dcl.p, io.hcl, 3 * M * sizeof(double), cudaMemcpyHostToDevice, 0));
    ocl_gb300_stats st;
    std::memset(&st, 0, sizeof(st));
    int r = drop_run(m, cp, io.dcl.p, M, OCL_GB300_PREC_MIXED, io.dz.p, io.dcc.p, io.dty.p, 0, acc ? &st : nullptr);
    if (r) return r;
    CK(cudaMemcpyAsync(io.hz, io.dz.p, M * sizeof(double), cudaMemcpyDeviceToHost, 0));
    CK(cudaMemcpyAsync(io.hcc, io.dcc.p, 3 * M * sizeof(double), cudaMemcpyDeviceToHost, 0));
    CK(cudaMemcpyAsync(io.hty, io.dty.p, M * sizeof(int32_t), cudaMemcpyDeviceToHost, 0));
    CK(cudaStreamSynchronize(0));
    std::memcpy(z.data(), io.hz, M * sizeof(double));
    std::memcpy(cc.data(), io.hcc, 3 * M * sizeof(double));
    std::memcpy(ty.data(), io.hty, M * sizeof(int32_t));
    if (acc) {
        acc->pairs += st.pairs;
        acc->refined += st.refined;
        acc->iter_limit_hits += st.iter_limit_hits;
        acc->fallback += st.fallback;
        acc->violations += st.violations;
        acc->screened += st.screened;
        acc->overflow_points += st.overflow_points;
        acc->chain_points += st.chain_points;
        acc->open_branch_points += st.open_branch_points;
        acc->untracked_branch_points += st.untracked_branch_points;
        acc->plain_points += st.plain_points;
        acc->verify_failed_points += st.verify_failed_points;
        acc->kernel_ms += st.kernel_ms;
    }
    return OCL_GB300_OK;
}

int path_drop_run(Mesh& m, const CutterP& cp, const double* spans, uint64_t S, double sampling, double min_z,
                  double* xyz, double* cc, int32_t* type, uint64_t cap, uint64_t* count, ocl_gb300_stats* stats) {
    if (!(sampling > 0.0)) {
        set_error("sampling must be > 0");
        return OCL_GB300_BAD_ARG;
    }
    // PathDropCutter::sample_span (dropcutter/pathdropcutter.cpp:69-80)
    std::vector<double> cl;
    for (uint64_t k = 0; k < S; ++k) {
        SpanH s;
        if (!span_init(s, spans + OCL_GB300_SPAN_DOUBLES * k)) {
            set_error("invalid span " + std::to_string(k));
            return OCL_GB300_BAD_ARG;
        }
        double steps_d = s.length / sampling + 1;
        if (!(steps_d < 4.0e9)) {
            set_error("too many samples on a span");
            return OCL_GB300_BAD_ARG;
        }
        unsigned int num_steps = (unsigned int)(steps_d);
        for (unsigned int i = 0; i <= num_steps; i++) {
            double fraction = (double)i / num_steps;
            double p[3];
            span_point(s, fraction, p);
            cl.push_back(p[0]);
            cl.push_back(p[1]);
            cl.push_back(min_z);
        }
    }
    const uint64_t n = cl.size() / 3;
    *count = n;
    if (n > cap) {
        set_error("output buffer too small");
        return OCL_GB300_CAPACITY;
    }
    std::vector<double> z, ccv;
    std::vector<int32_t> ty;
    if (stats) std::memset(stats, 0, sizeof(*stats));
    int st = drop_host(m, cp, cl, z, ccv, ty, stats);
    if (st) return st;
    for (uint64_t i = 0; i < n; ++i) {
        xyz[3 * i] = cl[3 * i];
        xyz[3 * i + 1] = cl[3 * i + 1];
        xyz[3 * i + 2] = z[i];
    }
    std::memcpy(cc, ccv.data(), 3 * n * sizeof(double));
    std::memcpy(type, ty.data(), n * sizeof(int32_t));
    return OCL_GB300_OK;
}

// AdaptivePathDropCutter::flat (adaptivepathdropcutter.cpp:88-94)
static bool flat_h(const APoint& s, const APoint& m, const APoint& e, double cos_limit) {
    double v1[3], v2[3];
    for (int a = 0; a < 3; ++a) {
        v1[a] = m.p[a] - s.p[a];
        v2[a] = e.p[a] - m.p[a];
    }
    double n1 = std::sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
    double n2 = std::sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
    if (n1 != 0.0) for (int a = 0; a < 3; ++a) v1[a] = v1[a] * (1 / n1);
    if (n2 != 0.0) for (int a = 0; a < 3; ++a) v2[a] = v2[a] * (1 / n2);
    return (v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2]) > cos_limit;
}

int ApdcRun::init(const double* spans, uint64_t S, double sampling, double min_sampling, double cos_limit) {
    if (!(sampling > 0.0) || !(min_sampling > 0.0)) {
        set_error("sampling and min_sampling must be > 0");
        return OCL_GB300_BAD_ARG;
    }
    S_ = S;
    sampling_ = sampling;
    min_sampling_ = min_sampling;
    cos_limit_ = cos_limit;
    sp_.assign(S, SpanH());
    for (uint64_t k = 0; k < S; ++k)
        if (!span_init(sp_[k], spans + OCL_GB300_SPAN_DOUBLES * k)) {
            set_error("invalid span " + std::to_string(k));
            return OCL_GB300_BAD_ARG;
        }
    // span end points first (AdaptivePathDropCutter::adaptive_sampling_run, :57-70)
    cl_.clear();
    for (uint64_t k = 0; k < S; ++k) {
        double a[3], b[3];
        span_point(sp_[k], 0.0, a);
        span_point(sp_[k], 1.0, b);
        cl_.insert(cl_.end(), a, a + 3);
        cl_.insert(cl_.end(), b, b + 3);
    }
    ends_ = true;
    depth_ = 0;
    done_ = S == 0;
    starts_.clear();
    level_.clear();
    leaves_.clear();
    return OCL_GB300_OK;
}

// adaptive_sample (:72-86): every midpoint of the current level
void ApdcRun::next_level() {
    cl_.clear();
    mt_.assign(level_.size(), 0.0);
    for (size_t j = 0; j < level_.size(); ++j) {
        const Iv& iv = level_[j];
        mt_[j] = iv.t0 + (iv.t1 - iv.t0) / 2.0;
        double p[3];
        span_point(sp_[iv.span], mt_[j], p);
        cl_.insert(cl_.end(), p, p + 3);
    }
}

void ApdcRun::consume(const double* z, const double* ccv, const int32_t* ty) {
    auto mk = [&](size_t i) {
        APoint p;
        p.p[0] = cl_[3 * i];
        p.p[1] = cl_[3 * i + 1];
        p.p[2] = z[i];
        std::memcpy(p.cc, ccv + 3 * i, 3 * sizeof(double));
        p.type = ty[i];
        return p;
    };
    if (ends_) {
        ends_ = false;
        starts_.resize(S_);
        for (uint64_t k = 0; k < S_; ++k) {
            starts_[k] = mk(2 * k);
            level_.push_back({k, 0.0, 1.0, mk(2 * k), mk(2 * k + 1)});
        }
        next_level();
        return;
    }
    std::vector<Iv> next;
    for (size_t j = 0; j < level_.size(); ++j) {
        const Iv& iv = level_[j];
        APoint mid = mk(j);
        double dx = iv.b.p[0] - iv.a.p[0], dy = iv.b.p[1] - iv.a.p[1];
        double fw_step = std::sqrt(dx * dx + dy * dy);
        bool split = (fw_step > sampling_) || ((!flat_h(iv.a, mid, iv.b, cos_limit_)) && (fw_step > min_sampling_));
        if (split && depth_ < 60) {
            next.push_back({iv.span, iv.t0, mt_[j], iv.a, mid});
            next.push_back({iv.span, mt_[j], iv.t1, mid, iv.b});
        } else {
            leaves_.push_back({iv.span, iv.t1, iv.b});
        }
    }
    level_.swap(next);
    ++depth_;
    if (level_.empty()) {
        std::stable_sort(leaves_.begin(), leaves_.end(), [](const Leaf& a, const Leaf& b) {
            return a.span != b.span ? a.span < b.span : a.t1 < b.t1;
        });
        cl_.clear();
        done_ = true;
    } else {
        next_level();
    }
}

int ApdcRun::write(double* xyz, double* cc, int32_t* type, uint64_t cap, uint64_t* count) const {
    const uint64_t n = S_ + leaves_.size();
    *count = n;
    if (n > cap) {
        set_error("output buffer too small");
        return OCL_GB300_CAPACITY;
    }
    uint64_t w = 0;
    size_t li = 0;
    for (uint64_t k = 0; k < S_; ++k) {
        auto put = [&](const APoint& p) {
            std::memcpy(xyz + 3 * w, p.p, 3 * sizeof(double));
            std::memcpy(cc + 3 * w, p.cc, 3 * sizeof(double));
            type[w] = p.type;
            ++w;
        };
        put(starts_[k]);
        while (li < leaves_.size() && leaves_[li].span == k) put(leaves_[li++].p);
    }
    return OCL_GB300_OK;
}

int adaptive_path_drop_run(Mesh& m, const CutterP& cp, const double* spans, uint64_t S, double sampling,
                           double min_sampling, double cos_limit, double* xyz, double* cc, int32_t* type,
                           uint64_t cap, uint64_t* count, ocl_gb300_stats* stats) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    ApdcRun run;
    int st = run.init(spans, S, sampling, min_sampling, cos_limit);
    if (st) return st;
    std::vector<double> z, ccv;
    std::vector<int32_t> ty;
    while (!run.done()) {
        st = drop_host(m, cp, run.points(), z, ccv, ty, stats);
        if (st) return st;
        run.consume(z.data(), ccv.data(), ty.data());
    }
    return run.write(xyz, cc, type, cap, count);
}

}  // namespace oclg
