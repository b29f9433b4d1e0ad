// paths.cuh -- host side of the path drivers: spans and the adaptive
// sampler as resumable steps (each step is one batch of CL points to drop).
#pragma once
#include <cstdint>
#include <vector>

namespace oclg {

struct SpanH {
    int type;
    double p1[3], p2[3], c[3];
    bool dir;
    double radius, length;
};

struct APoint {
    double p[3];
    double cc[3];
    int32_t type;
};

// AdaptivePathDropCutter::adaptive_sampling_run
// (src/dropcutter/adaptivepathdropcutter.cpp:53-94) as a level-synchronous
// bisection: points() holds the CL points of the next drop (the span end
// points first, then every midpoint of one bisection level); consume() takes
// their results and prepares the next level.  The emitted points are put in
// the reference's depth-first order (ascending parameter within a span).
class ApdcRun {
   public:
    // OCL_GB300_OK, or OCL_GB300_BAD_ARG for a bad span or sampling
    int init(const double* spans, uint64_t S, double sampling, double min_sampling, double cos_limit);
    const std::vector<double>& points() const { return cl_; }
    bool done() const { return done_; }
    void consume(const double* z, const double* cc, const int32_t* type);
    uint64_t count() const { return S_ + leaves_.size(); }
    // OCL_GB300_CAPACITY (with *count set) when cap is too small
    int write(double* xyz, double* cc, int32_t* type, uint64_t cap, uint64_t* count) const;

   private:
    struct Iv {
        uint64_t span;
        double t0, t1;
        APoint a, b;
    };
    struct Leaf {
        uint64_t span;
        double t1;
        APoint p;
    };
    void next_level();
    std::vector<SpanH> sp_;
    uint64_t S_ = 0;
    double sampling_ = 0, min_sampling_ = 0, cos_limit_ = 0;
    std::vector<double> cl_, mt_;
    bool ends_ = true;  // the next consume() takes the span end points
    int depth_ = 0;
    bool done_ = false;
    std::vector<APoint> starts_;
    std::vector<Iv> level_;
    std::vector<Leaf> leaves_;
};

}  // namespace oclg
