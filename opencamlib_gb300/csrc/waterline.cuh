// waterline.cuh -- fiber sets and waterline loops (waterline.cu) shared with
// the C ABI.
#pragma once
#include <cstdint>
#include <vector>

#include "drop.cuh"

namespace oclg {

// Fibers of one direction with their intervals (t-values on the fiber).
struct FiberSet {
    std::vector<double> fib;     // 6 per fiber: p1, p2
    std::vector<uint64_t> off;   // F + 1
    std::vector<double> ival;    // 2 per interval: lower, upper
    std::vector<double> cc;      // 6 per interval: lower CC point, upper CC point (pushed fibers)
    std::vector<int32_t> type;   // 2 per interval
    uint64_t count() const { return off.empty() ? 0 : off.size() - 1; }
};

// The loops woven from one X and one Y fiber set.
struct LoopSet {
    std::vector<double> pts;     // 3 per loop point
    std::vector<uint64_t> off;   // loops + 1
    FiberSet fibers[2];          // the X and Y fibers woven
};

int weave_loops(LoopSet& out);
int waterline_run(Mesh& m, const CutterP& cp, const double* zs, uint64_t nz, double sampling,
                  std::vector<LoopSet>& out, ocl_gb300_stats* stats);
int adaptive_waterline_run(Mesh& m, const CutterP& cp, double zh, double sampling, double min_sampling,
                           double cos_limit, LoopSet& out, ocl_gb300_stats* stats);

}  // namespace oclg
