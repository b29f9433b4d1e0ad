// mesh.cuh -- device-resident mesh (one STLSurf) and its indexes.
#pragma once
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace oclg {

struct Cell {
    float minx, maxx, miny, maxy;  // union of the entries' bboxes
    float maxz;                    // max triangle z in the cell
    uint32_t start, count;
    float pad;
};
static_assert(sizeof(Cell) == 32, "Cell layout");

// KD-tree node for the push-cutter candidate search (the reference's tree,
// rebuilt on the host with the same splits; src/common/kdtree.hpp:141-304).
struct KDNodeD {
    int32_t dim;     // Bbox index 0..5 of the cut
    int32_t hi, lo;  // child node ids or -1
    int32_t leaf_begin, leaf_end;  // leaf: range in the order array; -1 for inner nodes
    int32_t pad;
    double cut;
};
static_assert(sizeof(KDNodeD) == 32, "KDNodeD layout");

constexpr int KD_STACK = 256;  // device traversal stack (entries per warp)

struct KDTreeD {
    std::vector<KDNodeD> nodes;
    std::vector<int32_t> order;  // insertion indices in leaf visit order
    int max_depth = 0;
};

// dims: 0 = XY (drop), 1 = YZ (X fibers), 2 = XZ (Y fibers)
void kd_build_host(const std::vector<double>& bb6, uint64_t n, unsigned bucket, int dims, KDTreeD& out);

struct PushIndex {
    bool built = false;
    KDNodeD* d_nodes = nullptr;
    float2* d_cut32 = nullptr;   // per node: the cut rounded down and up to float
    int32_t* d_order = nullptr;  // device-order triangle ids in leaf visit order
    int nnodes = 0;
    int max_depth = 0;
};

struct Mesh {
    uint64_t n = 0;
    unsigned bucket = 1;
    double bb[6] = {0, 0, 0, 0, 0, 0};
    std::vector<double> host_bb;     // per triangle, insertion order
    std::vector<int32_t> dev_to_ins; // device order -> insertion index
    std::vector<int32_t> ins_to_dev;
    GridP grid{};
    float E0 = 0.0f;                 // FP32 position error budget of the local frame
    Tri64* d_t64 = nullptr;
    Tri32* d_t32 = nullptr;
    Cell* d_cells = nullptr;
    Entry* d_entries = nullptr;
    uint64_t nentries = 0;
    PushIndex push[2];
    PushIndex drop_kd;               // XY tree of the drop-cutter search (device ids)
    // per triangle (device order) and edge n (vertex n to vertex n+1):
    // sin(atan(dz / xy length)), the bull push's edge slope, computed on the
    // host with the host's libm as the reference does; built on first use
    double* d_edge_sin = nullptr;
    std::mutex mu;
};

int upload_kd(Mesh& M, const KDTreeD& kd, PushIndex& out);
// The edge slopes of d_edge_sin, built on first use.
int ensure_edge_sin(Mesh& m);
// The YZ (X-fibers) or XZ (Y-fibers) tree of the push-cutter, built on first use.
int ensure_push_index(Mesh& m, int dir);
std::string& last_error_ref();
void set_error(const std::string& msg);

}  // namespace oclg
