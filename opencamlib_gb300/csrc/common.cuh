// common.cuh -- device-side data layout shared by the mesh, drop and push code.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/ocl_gb300.h"

namespace oclg {

// ---------------------------------------------------------------------------
// Cutter parameters as the device sees them.  All derived values are computed
// on the host from the constructor arguments with the reference constructors'
// arithmetic (cylcutter.cpp:39-46, ballcutter.cpp:38-45, bullcutter.cpp:38-47,
// conecutter.cpp:39-49, compositecutter.cpp:43-51), so the device never
// re-derives them (and never calls tan() on the device).
// ---------------------------------------------------------------------------
struct BasicP {
    int kind;
    double diameter, radius, length;
    double xy_normal_length, normal_length, center_height;
    double radius1, radius2;  // bull
    double angle, tan_angle;  // cone
};

struct CutterP {
    int kind;      // OCL_CUTTER_*
    int nsub;      // composite
    double radius; // getRadius()
    double length; // getLength()
    BasicP b;      // kind != COMPOSITE
    BasicP sub[OCL_GB300_MAX_SUB];
    double radiusvec[OCL_GB300_MAX_SUB], heightvec[OCL_GB300_MAX_SUB], zoffset[OCL_GB300_MAX_SUB];
};

// ---------------------------------------------------------------------------
// Triangle record in FP64 (refinement / plain path), 24 doubles = 192 B.
// p: vertices in insertion order; n: Triangle::upNormal of the unit normal
// (triangle.cpp:65-75); bb: [minx maxx miny maxy minz maxz]; d = -n.p0;
// nn = normalize(n); xyn = xyNormalize(nn.x, nn.y, 0) -- the values
// MillingCutter::facetDrop (millingcutter.cpp:51-75) derives per call.
// ---------------------------------------------------------------------------
struct Tri64 {
    double p[9];
    double n[3];
    double bb[6];
    double d;
    double nn[3];
    double xyn[2];
};
static_assert(sizeof(Tri64) == 192, "Tri64 layout");

// Per-triangle flags (exact FP64 decisions made once on the host).
enum : uint32_t {
    TF_FACET_NONE = 0,    // isZero_tol(n.z): vertical facet, no facet drop
    TF_FACET_HORIZ = 1,   // isZero_tol(n.x) && isZero_tol(n.y): horizontal special case
    TF_FACET_GENERAL = 2,
    TF_FACET_MASK = 3,
    TF_EDGE0_SKIP = 4,    // edge (p0,p1) has isZero_tol(dx) && isZero_tol(dy)
    TF_EDGE1_SKIP = 8,
    TF_EDGE2_SKIP = 16,
    TF_EDGE0_HORIZ = 32,  // edge (p0,p1) has isZero_tol(dz) (BullCutter horizontal-edge case)
    TF_EDGE1_HORIZ = 64,
    TF_EDGE2_HORIZ = 128,
};

// FP32 screening geometry of one triangle, local to the mesh origin, 64 B.
struct Tri32 {
    float v0[3];   // p0 - origin
    float e1[3];   // p1 - p0 (difference taken in FP64, then rounded)
    float e2[3];   // p2 - p0
    float nn[3];   // unit up-normal
    uint32_t flags;
    uint32_t kd_rank;   // position in the reference KD-tree leaf visit order
    float bary_scale;   // 1 / smallest xy altitude (barycentric error per unit position error)
    float pad;
};
static_assert(sizeof(Tri32) == 64, "Tri32 layout");

// Grid entry: one triangle in its home cell, with its FP32 bbox rounded
// outward, 32 B.  Entries are sorted by (level, home cell), cells row-major.
struct Entry {
    float minx, maxx, miny, maxy;  // local to origin, rounded outward
    float maxz;                    // rounded up
    int32_t tri;                   // triangle index in device order
    float pad[2];
};
static_assert(sizeof(Entry) == 32, "Entry layout");

// Multi-level uniform grid: level L has square cells of cs[L] = cs[0] * 4^L;
// a triangle lives in the finest level whose cell size covers its xy extent,
// in the cell holding its bbox min corner, so a query rectangle widened by
// one cell to the left and below finds every triangle that overlaps it.
constexpr int GRID_MAX_LEVELS = 8;
struct GridP {
    double x0, y0;  // grid origin (FP64)
    int nlev;
    double cs[GRID_MAX_LEVELS], inv_cs[GRID_MAX_LEVELS];
    int ncol[GRID_MAX_LEVELS], nrow[GRID_MAX_LEVELS];
    uint32_t cell_off[GRID_MAX_LEVELS + 1];  // first cell index of each level
    double ox, oy, oz;  // origin of the FP32 local frame
};

__host__ __device__ inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

}  // namespace oclg
