// drop.cu -- BatchDropCutter on the GPU.
//
// Pipeline for M CL points against a device-resident mesh:
//   1. CL points are ordered along a Morton curve, so a warp's 32 lanes hold
//      32 neighbouring points (lanes = CL points).
//   2. Mixed precision:
//      k_drop_screen  one warp per 32 points streams the grid cells under the
//                     warp's footprint, the rows most likely to lift it
//                     first.  Cells and then
//                     triangles are rejected with an FP32 upper bound
//                     (bbox max z minus a lower bound of the cutter profile at
//                     the bbox distance); survivors get the FP32
//                     whole-triangle screen [lo, hi].  A lane keeps a running
//                     certified lower bound and a short list of triangles whose
//                     hi reaches it.
//      k_drop_refine  one thread per point evaluates its listed triangles in
//                     FP64 with the reference semantics and keeps the highest
//                     contact (ties: the reference's KD visit order).
//      k_drop_kd      points whose list overflowed are redone in plain FP64.
//   3. Plain FP64 (OCL_GB300_PREC_FP64): k_drop_kd for every point; it runs
//      the reference's KD search and evaluates every exact-overlap pair in FP64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <string>

#include <cub/cub.cuh>

#include "drop.cuh"
#include "drop_util.cuh"
#include "geom64.cuh"
#include "screen.cuh"
#include "util.cuh"

namespace oclg {

// ---------------------------------------------------------------------------
// Morton ordering of the CL points
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t spread16(uint32_t x) {
    x &= 0xFFFF;
    x = (x | (x << 8)) & 0x00FF00FF;
    x = (x | (x << 4)) & 0x0F0F0F0F;
    x = (x | (x << 2)) & 0x33333333;
    x = (x | (x << 1)) & 0x55555555;
    return x;
}

__global__ void k_morton(const double* cl, uint64_t M, double x0, double y0, double sx, double sy, uint32_t* keys,
                         uint32_t* idx) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    double fx = (cl[3 * i] - x0) * sx, fy = (cl[3 * i + 1] - y0) * sy;
    uint32_t qx = (uint32_t)fmin(fmax(fx, 0.0), 65535.0);
    uint32_t qy = (uint32_t)fmin(fmax(fy, 0.0), 65535.0);
    keys[i] = spread16(qx) | (spread16(qy) << 1);
    idx[i] = (uint32_t)i;
}

__global__ void k_gather_cl(const double* cl, const uint32_t* perm, uint64_t M, double* out) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    uint32_t j = perm[i];
    out[3 * i] = cl[3 * j];
    out[3 * i + 1] = cl[3 * j + 1];
    out[3 * i + 2] = cl[3 * j + 2];
}

struct Best64 {
    double z;
    double cx, cy, cz;
    int type;
    uint32_t rank;
};
__device__ __forceinline__ void merge_best(Best64& b, const CL64& c, uint32_t rank) {
    if (c.z > b.z || (c.z == b.z && rank < b.rank)) {
        b.z = c.z;
        b.cx = c.cc.x;
        b.cy = c.cc.y;
        b.cz = c.cc.z;
        b.type = c.type;
        b.rank = rank;
    }
}

// ---------------------------------------------------------------------------
// Plain FP64 kernel: the reference's own algorithm on the device.  A warp of
// 32 CL points walks the KD tree of the mesh (KDTree::search_node,
// common/kdtree.hpp:273-304) with one visit mask per node, so each lane sees
// exactly its own candidates in the reference's visit order; every candidate
// that overlaps (MillingCutter::overlaps) and is not below the running z is
// dropped in FP64 against that running z (BatchDropCutter::dropCutter5,
// dropcutter/batchdropcutter.cpp:187-231).  Used for OCL_GB300_PREC_FP64 and
// for the points the mixed path hands back.
// ---------------------------------------------------------------------------
// One warp's 32 points (slot `warp` of the list).  FAST (the fallback of the
// mixed path): candidates that cannot overlap or cannot lift the running
// height are skipped after an FP32 test on the outward-rounded bbox, which
// leaves the fold unchanged; the plain FP64 path (FAST = false) evaluates
// every overlap pair in FP64 like the reference.
template <bool FAST>
__device__ __forceinline__ void drop_kd_warp(const DropCtx& ctx, const float* hlb, const uint32_t* __restrict__ list,
                                             int nlist, int warp, uint2* st, int lane) {
    const int base = warp * 32;
    const bool active = base + lane < nlist;
    const uint32_t i = list ? list[active ? base + lane : base] : (uint32_t)(active ? base + lane : base);
    const double x = ctx.cl[3 * i], y = ctx.cl[3 * i + 1], z0 = ctx.cl[3 * i + 2];
    const double R = ctx.cp.radius;
    // KDTree::search_cutter_overlap box (kdtree.hpp:130-135), XY dimensions
    const double bb[4] = {x - R, x + R, y - R, y + R};
    CL64 cl{x, y, z0, d3(0, 0, 0), OCL_CC_NONE};
    unsigned long long pairs = 0;
    int capped = 0;
    const unsigned amask = __ballot_sync(0xffffffffu, active);
    int sp = 0;
    if (ctx.kd_nodes && amask) {
        if (lane == 0) st[0] = make_uint2(0u, amask);
        sp = 1;
    }
    __syncwarp();
    while (sp > 0) {
        --sp;
        const uint2 e = st[sp];
        __syncwarp();
        const KDNodeD nd = ctx.kd_nodes[e.x];
        const bool in = (e.y >> lane) & 1u;
        if (nd.leaf_begin >= 0) {
            for (int k = nd.leaf_begin; k < nd.leaf_end; ++k) {
                if (!in) continue;
                const int32_t tri = ctx.kd_order[k];
                if (FAST) {
                    const Entry e = ctx.entries[tri];
                    const float cxl = (float)(x - ctx.g.ox), cyl = (float)(y - ctx.g.oy);
                    const float gd = ctx.guard;
                    const float dx = fmaxf(0.0f, fmaxf(e.minx - cxl, cxl - e.maxx));
                    const float dy = fmaxf(0.0f, fmaxf(e.miny - cyl, cyl - e.maxy));
                    if (dx > ctx.prof.R + gd || dy > ctx.prof.R + gd) continue;  // cannot overlap
                    const float d = sqrtf(dx * dx + dy * dy);
                    if (d > ctx.prof.R + gd) continue;  // outside the cutter's reach
                    const float ub = e.maxz - hlb_at(hlb, d - gd, (float)HLB_N / ctx.prof.R);
                    if (ub + gd < __double2float_rd(cl.z - ctx.g.oz)) continue;  // cannot lift
                }
                const Tri64& t = ctx.t64[tri];
                if (overlaps64(R, x, y, t)) {
                    ++pairs;
                    if (cl.z < t.bb[5]) drop_triangle64(ctx.cp, cl, t, ctx.t32[tri].flags, &capped);
                }
            }
            continue;
        }
        bool vh, vl;
        if ((nd.dim & 1) == 0) {
            const bool only_lo = nd.cut > bb[nd.dim + 1];
            vh = in && !only_lo && nd.hi >= 0;
            vl = in && nd.lo >= 0;
        } else {
            const bool only_hi = nd.cut < bb[nd.dim - 1];
            vh = in && nd.hi >= 0;
            vl = in && !only_hi && nd.lo >= 0;
        }
        const unsigned mh = __ballot_sync(0xffffffffu, vh), ml = __ballot_sync(0xffffffffu, vl);
        if (lane == 0) {
            if (ml) st[sp] = make_uint2((unsigned)nd.lo, ml);
            if (mh) st[sp + (ml ? 1 : 0)] = make_uint2((unsigned)nd.hi, mh);
        }
        sp += (ml ? 1 : 0) + (mh ? 1 : 0);
        __syncwarp();
    }
    if (active) {
        uint32_t o = ctx.perm[i];
        ctx.out_z[o] = cl.z;
        ctx.out_cc[3 * o] = cl.cc.x;
        ctx.out_cc[3 * o + 1] = cl.cc.y;
        ctx.out_cc[3 * o + 2] = cl.cc.z;
        ctx.out_type[o] = cl.type;
    }
    for (int o = 16; o > 0; o >>= 1) pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
    for (int o = 16; o > 0; o >>= 1) capped += __shfl_xor_sync(0xffffffffu, capped, o);
    if (lane == 0) {
        atomicAdd(&ctx.counters[C_PAIRS], pairs);
        if (capped) atomicAdd(&ctx.counters[C_CAPPED], (unsigned long long)capped);
    }
}

// list == nullptr: points 0..M-1; else the *nlist_dev listed points.  The
// grid strides over warps, so the fallback launch needs no host-side count.
template <bool FAST>
__global__ void __launch_bounds__(128) k_drop_kd(const __grid_constant__ DropCtx ctx, const uint32_t* __restrict__ list,
                                                 const unsigned long long* __restrict__ nlist_dev) {
    __shared__ uint2 s_stack[4][KD_STACK];
    __shared__ float s_hlb[HLB_N];
    for (int k = threadIdx.x; k < HLB_N; k += blockDim.x) s_hlb[k] = ctx.hlb[k];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int wl = threadIdx.x >> 5;
    const int nlist = list ? (int)*nlist_dev : ctx.M;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; warp * 32 < nlist; warp += nwarps)
        drop_kd_warp<FAST>(ctx, s_hlb, list, nlist, warp, s_stack[wl], lane);
}

// Batch: every warp of the persistent grid strides over the points each job
// handed to the plain kernel (counts on the device), job after job.
__global__ void __launch_bounds__(128) k_drop_kd_b(const __grid_constant__ BatchView bv) {
    __shared__ uint2 s_stack[4][KD_STACK];
    __shared__ float s_hlb[HLB_N];
    const int lane = threadIdx.x & 31;
    const int wl = threadIdx.x >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned k = 0; k < bv.njobs; ++k) {
        const DropCtx& ctx = bv.ctxs[bv.jobs[k]];
        const int n = (int)ctx.counters[C_PLAIN];
        if (n == 0) continue;
        __syncthreads();
        for (int q = threadIdx.x; q < HLB_N; q += blockDim.x) s_hlb[q] = ctx.hlb[q];
        __syncthreads();
        for (int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; warp * 32 < n; warp += nwarps)
            drop_kd_warp<true>(ctx, s_hlb, ctx.list2, n, warp, s_stack[wl], lane);
    }
}

// One step of dropCutter5's fold (batchdropcutter.cpp:187-231): the overlap
// and below tests, then MillingCutter::dropCutter on the triangle.
// zfloor (local frame): for the cutters whose fold is a plain maximum
// (cyl/ball/bull: a lifting facet contact is the plane's highest contact), a
// height the final result is certified to reach; an edge that cannot reach
// it cannot give the result, and its FP64 evaluation is skipped.
__device__ __forceinline__ void fold_one(const DropCtx& ctx, CL64& cl, uint32_t tri, float cxl, float cyl,
                                         int& capped, float zfloor = -3.0e38f) {
    const Tri64& t = ctx.t64[tri];
    if (!(overlaps64(ctx.cp.radius, cl.x, cl.y, t) && cl.z < t.bb[5])) return;
    uint32_t fl = ctx.t32[tri].flags;
    uint32_t sub_skip = 0, part_skip = 0;
    if (ctx.composite_screen) {
        // Parts whose FP32 upper bound lies below the running height cannot
        // lift it and are left out of the FP64 evaluation:
        //   a vertex (composite profile);
        //   a sub-cutter's facet drop, when none of its facet contacts that
        //   may lie in its radius window can (only such a contact lifts);
        //   a sub-cutter's edge (the edge drop keeps the highest of its
        //   edges, and the window is tested on that one: an edge below the
        //   running height never becomes it);
        //   a sub-cutter's whole edge drop, when none of its edges' contacts
        //   that may lie in its window can lift.
        const Tri32 t3 = ctx.t32[tri];
        const float wx = cxl - t3.v0[0], wy = cyl - t3.v0[1];
        const float zr = __double2float_rd(cl.z - ctx.g.oz) - t3.v0[2];
        const float lim = zr - ctx.guard - 2.0f * ctx.E;
        const float px[3] = {0.0f, t3.e1[0], t3.e2[0]};
        const float py[3] = {0.0f, t3.e1[1], t3.e2[1]};
        const float pz[3] = {0.0f, t3.e1[2], t3.e2[2]};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float dx = px[k] - wx, dy = py[k] - wy;
            const float qlo = sqrtf(dx * dx + dy * dy) - ctx.E;
            if (qlo > ctx.comp.R || pz[k] - hcomp32(ctx.comp, fmaxf(qlo, 0.0f)) + ctx.E < lim) part_skip |= 1u << k;
        }
        for (int n = 0; n < ctx.comp.nsub; ++n) {
            if (comp_facet_hi32(ctx.comp, t3, n, wx, wy, ctx.E) < lim) part_skip |= 1u << (8 + n);
            const float zo = ctx.comp.zoff[n];
            const float wlo = (n == 0 ? 0.0f : ctx.comp.rlim[n - 1]) - 1e-6f, whi = ctx.comp.rlim[n] + 1e-6f;
            bool any_in_window = false;
            for (int e = 0; e < 3; ++e) {
                if (fl & (TF_EDGE0_SKIP << e)) continue;
                const int k = (e + 1) % 3;
                const bool horiz = (fl & (TF_EDGE0_HORIZ << e)) != 0;
                Iv v = edge32(ctx.comp.sub[n], px[e], py[e], pz[e], px[k], py[k], pz[k], wx, wy, ctx.E, horiz);
                if (v.hi - zo < lim) {
                    sub_skip |= 1u << (3 * n + e);
                    continue;
                }
                if (!any_in_window) {
                    v = edge32(ctx.comp.sub[n], px[e], py[e], pz[e], px[k], py[k], pz[k], wx, wy, ctx.E, horiz, wlo, whi);
                    any_in_window = !(v.hi - zo < lim);
                }
            }
            if (!any_in_window) sub_skip |= 7u << (3 * n);
        }
    } else {
        // an edge whose FP32 upper bound is below the running height cannot
        // lift it; skipping its FP64 evaluation (for the bull: two Brent
        // solves) leaves the fold unchanged
        const Tri32 t3 = ctx.t32[tri];
        const float wx = cxl - t3.v0[0], wy = cyl - t3.v0[1];
        const float zr = fmaxf(__double2float_rd(cl.z - ctx.g.oz), zfloor) - t3.v0[2];
        const float px[3] = {0.0f, t3.e1[0], t3.e2[0]};
        const float py[3] = {0.0f, t3.e1[1], t3.e2[1]};
        const float pz[3] = {0.0f, t3.e1[2], t3.e2[2]};
        for (int e = 0; e < 3; ++e) {
            if (fl & (TF_EDGE0_SKIP << e)) continue;
            const int k = (e + 1) % 3;
            Iv v = edge32(ctx.prof, px[e], py[e], pz[e], px[k], py[k], pz[k], wx, wy, ctx.E,
                          (fl & (TF_EDGE0_HORIZ << e)) != 0);
            if (v.hi + ctx.E < zr - ctx.guard) fl |= (TF_EDGE0_SKIP << e);
        }
        // a vertex whose FP32 upper bound is below the running height cannot
        // lift it (the running height, not the floor: vertices come before
        // the edges and after a facet drop that did not lift)
        const float lim = __double2float_rd(cl.z - ctx.g.oz) - t3.v0[2] - ctx.guard - ctx.E;
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (vertex32(ctx.prof, px[k] - wx, py[k] - wy, pz[k], ctx.E).hi < lim) part_skip |= 1u << k;
        // the same for the facet contact of cyl/ball/bull (one contact that
        // lifts or not; the cone's tip/rim choice is left to the FP64 code)
        if (ctx.prof.kind != OCL_CUTTER_CONE &&
            facet32(ctx.prof, t3, wx, wy, ctx.E, ctx.E * 4.0f * t3.bary_scale + 1e-6f).hi < lim)
            part_skip |= PART_SKIP_FACET;
    }
    drop_triangle64(ctx.cp, cl, t, fl, &capped, sub_skip, part_skip);
}

// ---------------------------------------------------------------------------
// Bull edges ahead of the fold.  The bull's FP64 edge contact (offset-ellipse
// Brent search) does not depend on the running height, so the edges a fold
// may need are listed per CL point (k_bull_plan: every edge of a listed
// triangle whose FP32 bound reaches the point's certified floor), evaluated
// one edge per thread (k_bull_eval: whole warps run the same search), and the
// fold reads the results in its own order.
// ---------------------------------------------------------------------------
// FP32 upper bound of a bull edge's contact (the screen's bound: an edge
// whose maximiser cannot lie on the segment gives none, else the bracketed
// search); the plan and the fold compute it alike.
__device__ __forceinline__ float bull_edge_hi(const DropCtx& ctx, const Tri32& t3, int e, float wx, float wy) {
    Prof32 c = ctx.prof;
    c.kind = OCL_CUTTER_BULL;
    float ax, ay, az, bx, by, bz;
    tri_edge32(t3, e, ax, ay, az, bx, by, bz);
    BullEdge32 b;
    if (!bull_edge_setup32(c, ax, ay, az, bx, by, bz, wx, wy, ctx.E, b) || !bull_edge_open32(c, b)) return NEG_INF32;
    return bull_edge_solve32(c, b, ctx.E).hi;
}

// One point's plan; every lane of the warp calls it (one queue reservation
// per warp).
__device__ __forceinline__ void bull_plan_point(const DropCtx& ctx, const uint32_t i, uint2* __restrict__ queue,
                                                unsigned long long* __restrict__ qcount) {
    const int lane = threadIdx.x & 31;
    int cnt = 0;
    if (i < (uint32_t)ctx.M) {
        const int n = ctx.ncand[i];
        if (n != 0xFFFF) {
            const double x = ctx.cl[3 * i], y = ctx.cl[3 * i + 1];
            const float cxl = (float)(x - ctx.g.ox), cyl = (float)(y - ctx.g.oy);
            const float zfloor = ctx.blo[i];
            const uint32_t* tri = ctx.cand + (size_t)i * ctx.cand_cap;
            for (int q = 0; q < n; ++q) {
                const uint32_t tq = tri[q] & ~CAND_VERIFY;
                if (!overlaps64(ctx.cp.radius, x, y, ctx.t64[tq])) continue;
                const Tri32 t3 = ctx.t32[tq];
                const float wx = cxl - t3.v0[0], wy = cyl - t3.v0[1], zf = zfloor - t3.v0[2];
                for (int e = 0; e < 3; ++e) {
                    if (t3.flags & ((TF_EDGE0_SKIP | TF_EDGE0_HORIZ) << e)) continue;
                    if (bull_edge_hi(ctx, t3, e, wx, wy) + ctx.E < zf - ctx.guard) continue;
                    if (cnt < EDGE_SLOTS) ctx.edge_slots[(size_t)i * EDGE_SLOTS + cnt] = (tq << 2) | (uint32_t)e;
                    ++cnt;
                }
            }
        }
        ctx.edge_n[i] = (uint8_t)min(cnt, EDGE_N_SATURATED);
    }
    // one queue reservation per warp
    const int mine = min(cnt, EDGE_SLOTS);
    int incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    unsigned long long base = 0;
    if (lane == 31 && total) base = atomicAdd(qcount, (unsigned long long)total);
    base = __shfl_sync(0xffffffffu, base, 31);
    for (int k = 0; k < mine; ++k) queue[base + incl - mine + k] = make_uint2(i, (uint32_t)k);
}

__global__ void __launch_bounds__(128) k_bull_plan(const __grid_constant__ DropCtx ctx, uint2* __restrict__ queue,
                                                  unsigned long long* __restrict__ qcount) {
    bull_plan_point(ctx, blockIdx.x * blockDim.x + threadIdx.x, queue, qcount);
}

__global__ void __launch_bounds__(128) k_bull_plan_b(const __grid_constant__ BatchView bv) {
    __shared__ DropCtx s_ctx;
    __shared__ TileState ts;
    if (threadIdx.x == 0) ts.job = 0xFFFFFFFFu;
    uint2 tile;
    while (batch_next_tile(bv, ts, s_ctx, tile))
        bull_plan_point(s_ctx, tile.y * TILE_POINTS + threadIdx.x, s_ctx.edge_queue, s_ctx.counters + C_EDGEQ);
}

// Queue entries [w0, nq) with stride `step` of one call's edge queue.
__device__ __forceinline__ void bull_eval_range(const DropCtx& ctx, const uint2* __restrict__ queue,
                                                unsigned long long nq, unsigned long long w0, unsigned long long step,
                                                int& capped) {
    for (unsigned long long w = w0; w < nq; w += step) {
        const uint2 it = queue[w];
        const uint32_t s = ctx.edge_slots[(size_t)it.x * EDGE_SLOTS + it.y];
        const Tri64& t = ctx.t64[s >> 2];
        const int e = (int)(s & 3u);
        double clz = 0.0;
        D3 cc = d3(0, 0, 0);
        const bool ok = edge_contact64(ctx.cp.b, ctx.cl[3 * it.x], ctx.cl[3 * it.x + 1], tri_p(t, e),
                                       tri_p(t, (e + 1) % 3), clz, cc, &capped);
        EdgeRes r;
        r.clz = clz;
        r.ccx = cc.x;
        r.ccy = cc.y;
        r.ccz = cc.z;
        r.valid = ok ? 1 : 0;
        r.pad = 0;
        ctx.edge_res[(size_t)it.x * EDGE_SLOTS + it.y] = r;
    }
}

__global__ void __launch_bounds__(128) k_bull_eval(const __grid_constant__ DropCtx ctx, const uint2* __restrict__ queue,
                                                  const unsigned long long* __restrict__ qcount) {
    int capped = 0;
    bull_eval_range(ctx, queue, *qcount, blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x,
                    (unsigned long long)gridDim.x * blockDim.x, capped);
    if (capped) atomicAdd(&ctx.counters[C_CAPPED], (unsigned long long)capped);
}

__global__ void __launch_bounds__(128) k_bull_eval_b(const __grid_constant__ BatchView bv) {
    for (unsigned k = 0; k < bv.njobs; ++k) {
        const DropCtx& ctx = bv.ctxs[bv.jobs[k]];
        int capped = 0;
        bull_eval_range(ctx, ctx.edge_queue, ctx.counters[C_EDGEQ],
                        blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x,
                        (unsigned long long)gridDim.x * blockDim.x, capped);
        if (capped) atomicAdd(&ctx.counters[C_CAPPED], (unsigned long long)capped);
    }
}

// MillingCutter::dropCutter for a bull, edges from k_bull_eval where planned
// (the fold walks the point's plan slots in step: an edge is planned when it
// is the next stored slot; past the stored slots the plan's test is
// repeated and the edge is evaluated here).
__device__ __forceinline__ void fold_bull(const DropCtx& ctx, CL64& cl, uint32_t i, uint32_t tq, float cxl, float cyl,
                                          float zfloor, int& slot, int nplan, int& capped) {
    const Tri64& t = ctx.t64[tq];
    if (!overlaps64(ctx.cp.radius, cl.x, cl.y, t)) return;
    const Tri32 t3 = ctx.t32[tq];
    const uint32_t fl = t3.flags;
    const float wx = cxl - t3.v0[0], wy = cyl - t3.v0[1];
    const float zf = zfloor - t3.v0[2];
    // the plan's slots in fold order: an edge is planned when it is the next
    // stored slot; past the stored slots the plan's test is repeated
    float hi[3] = {3.0e38f, 3.0e38f, 3.0e38f};
    int k_of[3] = {-1, -1, -1};
    const uint32_t* slots = ctx.edge_slots + (size_t)i * EDGE_SLOTS;
    for (int e = 0; e < 3; ++e) {
        if (fl & ((TF_EDGE0_SKIP | TF_EDGE0_HORIZ) << e)) continue;
        if (slot >= nplan) break;  // nothing planned from here on
        if (slot < EDGE_SLOTS) {
            if (slots[slot] == ((tq << 2) | (uint32_t)e)) k_of[e] = slot++;
        } else {
            hi[e] = bull_edge_hi(ctx, t3, e, wx, wy);
            if (!(hi[e] + ctx.E < zf - ctx.guard)) k_of[e] = slot++;
        }
    }
    BasicP b = ctx.cp.b;
    b.kind = OCL_CUTTER_BULL;  // one contact model in the kernel
    if (!(cl.z < t.bb[5])) return;
    // facet and vertices whose FP32 upper bound lies below the running height
    // cannot lift it
    const float vlim = __double2float_rd(cl.z - ctx.g.oz) - t3.v0[2] - ctx.guard - ctx.E;
    Prof32 pb = ctx.prof;
    pb.kind = OCL_CUTTER_BULL;
    if (!(facet32(pb, t3, wx, wy, ctx.E, ctx.E * 4.0f * t3.bary_scale + 1e-6f).hi < vlim) &&
        facet_drop_base(b, cl, t, fl))
        return;
    const float vx[3] = {0.0f, t3.e1[0], t3.e2[0]};
    const float vy[3] = {0.0f, t3.e1[1], t3.e2[1]};
    const float vz[3] = {0.0f, t3.e1[2], t3.e2[2]};
    for (int k = 0; k < 3; ++k) {
        if (vertex32(ctx.prof, vx[k] - wx, vy[k] - wy, vz[k], ctx.E).hi < vlim) continue;
        const D3 p = tri_p(t, k);
        const double q = xynorm(d3(cl.x, cl.y, cl.z) - p);
        if (q <= b.radius) liftz(cl, p.z - height_basic(b, q), p, OCL_CC_VERTEX);
    }
    if (!(cl.z < t.bb[5])) return;
    const float zr = fmaxf(__double2float_rd(cl.z - ctx.g.oz), zfloor) - t3.v0[2];
    for (int e = 0; e < 3; ++e) {
        if (fl & (TF_EDGE0_SKIP << e)) continue;
        const bool horiz = (fl & (TF_EDGE0_HORIZ << e)) != 0;
        // an edge the plan left out cannot reach the floor: it cannot lift
        // (a planned result at or below the running height lifts nothing)
        if (!horiz && k_of[e] < 0) continue;
        if (!horiz && k_of[e] < EDGE_SLOTS) {
            const EdgeRes r = ctx.edge_res[(size_t)i * EDGE_SLOTS + k_of[e]];
            if (r.valid) liftz(cl, r.clz, d3(r.ccx, r.ccy, r.ccz), OCL_CC_EDGE);
            continue;
        }
        if (!horiz && hi[e] + ctx.E < zr - ctx.guard) continue;  // cannot lift
        double clz;
        D3 cc;
        if (edge_contact64(b, cl.x, cl.y, tri_p(t, e), tri_p(t, (e + 1) % 3), clz, cc, &capped))
            liftz(cl, clz, cc, OCL_CC_EDGE);
    }
}

// ---------------------------------------------------------------------------
// FP64 refinement: one thread per CL point folds its candidates in the
// reference's visit order (ascending KD rank) against a running height, as
// dropCutter5 does over its KD candidates.  Triangles left out can neither
// reach the final height nor change a branch choice of a collected triangle.
// ---------------------------------------------------------------------------
// BULL_PLAN: the bull with its edges evaluated ahead (fold_bull only); else
// every other case (fold_one only), so each kernel carries one fold.
template <bool BULL_PLAN>
__device__ __forceinline__ void refine_point(const DropCtx& ctx, const uint32_t i) {
    const int n = ctx.ncand[i];
    if (n == 0xFFFF) return;  // handed to the plain path
    const double x = ctx.cl[3 * i], y = ctx.cl[3 * i + 1], z0 = ctx.cl[3 * i + 2];
    const uint32_t* tri = ctx.cand + (size_t)i * ctx.cand_cap;  // already in KD order
    CL64 cl{x, y, z0, d3(0, 0, 0), OCL_CC_NONE};
    int capped = 0;
    const float cxl = (float)(x - ctx.g.ox), cyl = (float)(y - ctx.g.oy);
    // collection threshold less the guard: triangles left out lie below it
    const double tcut = (double)ctx.blo[i] + ctx.g.oz - (double)ctx.guard;
    const float zfloor = ctx.composite_screen || ctx.cp.kind == OCL_CUTTER_CONE ? -3.0e38f : ctx.blo[i];
    int slot = 0;
    // planned edges of the point; 255 is a saturated count (more were
    // planned): past the stored slots the fold repeats the plan's test for
    // every edge, so it stops only at a count it knows
    int nplan = ctx.edge_res ? ctx.edge_n[i] : 0;
    if (nplan == EDGE_N_SATURATED) nplan = 0x7FFFFFFF;
    for (int q = 0; q < n; ++q) {
        const uint32_t tq = tri[q] & ~CAND_VERIFY;
        if (BULL_PLAN) {
            fold_bull(ctx, cl, i, tq, cxl, cyl, zfloor, slot, nplan, capped);
            continue;
        }
        if ((tri[q] & CAND_VERIFY) && cl.z < tcut) {
            // a branch the screen could not decide.  From a running height at
            // or above the cut every fold agrees; below it, the folds agree
            // only if the triangle's lowest branch point is not below the cut
            const Tri64& t = ctx.t64[tq];
            if (overlaps64(ctx.cp.radius, x, y, t) && branch_low64(ctx.cp, x, y, t, ctx.t32[tq].flags) < tcut) {
                ctx.ncand[i] = 0xFFFF;  // the exact kernel redoes this point
                atomicAdd(&ctx.counters[C_VFAIL], 1ull);
                return;
            }
        }
        fold_one(ctx, cl, tq, cxl, cyl, capped, zfloor);
    }
    const uint32_t o = ctx.perm[i];
    ctx.out_z[o] = cl.z;
    ctx.out_cc[3 * o] = cl.cc.x;
    ctx.out_cc[3 * o + 1] = cl.cc.y;
    ctx.out_cc[3 * o + 2] = cl.cc.z;
    ctx.out_type[o] = cl.type;
    // self-check: the FP64 result may not fall below the certified FP32 bound
    const double lb = (double)ctx.blo[i] + ctx.g.oz;
    if (cl.z < lb - 1e-9 * (1.0 + fabs(lb))) atomicAdd(&ctx.counters[C_VIOLATION], 1ull);
    if (n) atomicAdd(&ctx.counters[C_REFINED], (unsigned long long)n);
    if (capped) atomicAdd(&ctx.counters[C_CAPPED], (unsigned long long)capped);
}

template <bool BULL_PLAN>
__global__ void __launch_bounds__(128) k_drop_refine(const __grid_constant__ DropCtx ctx) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint32_t)ctx.M) return;
    refine_point<BULL_PLAN>(ctx, i);
}

template <bool BULL_PLAN>
__global__ void __launch_bounds__(128) k_drop_refine_b(const __grid_constant__ BatchView bv) {
    __shared__ DropCtx s_ctx;
    __shared__ TileState ts;
    if (threadIdx.x == 0) ts.job = 0xFFFFFFFFu;
    uint2 tile;
    while (batch_next_tile(bv, ts, s_ctx, tile)) {
        const uint32_t i = tile.y * TILE_POINTS + threadIdx.x;
        if (i < (uint32_t)s_ctx.M) refine_point<BULL_PLAN>(s_ctx, i);
    }
}

// ---------------------------------------------------------------------------
// Exact fold of one handed-back CL point per block.
// The block gathers every triangle whose certified FP32 upper bound lies above
// the start height (no branch threshold needed), sorts them by KD rank and
// folds them in that order; a triangle whose upper bound is below the running
// height cannot lift it and is passed over, so only a few reach FP64.  Points
// with more than EXACT_CAP such triangles go on to the plain FP64 kernel.
// ---------------------------------------------------------------------------
constexpr int EXACT_CAP = 4096;
constexpr int EXACT_THREADS = 256;
constexpr size_t EXACT_SMEM = (size_t)EXACT_CAP * (8 + 4 + 4 + 4);

// Shared memory of the exact kernel: EXACT_CAP keys (KD rank << 32 | slot),
// triangles, upper bounds and lowest branch thresholds (+inf: none) in the
// dynamic part; the profile table and two reduction words beside it.
struct ExactShared {
    unsigned long long* key;
    uint32_t* tri;
    float* hi;
    float* qt;
    float* hlb;
    int* n;
    int* red;
    unsigned long long* pre;  // two words: the pre-fold's lowest key, its running height
};

// Per-block global scratch of the exact kernel for points with more than
// EXACT_CAP candidates (key == nullptr: none; such points go to the plain
// kernel).  Block b uses entries [b * cap, (b + 1) * cap).
struct ExactGlobal {
    unsigned long long* key;
    uint32_t* tri;
    float* hi;
    float* qt;
    int cap;
};
constexpr int EXACT_GCAP = 1 << 18;       // candidates per point the global scratch holds
constexpr int EXACT_GBLOCKS = 152 * 2;    // exact-kernel blocks (two resident per SM)
constexpr size_t EXACT_GBYTES = (size_t)EXACT_GBLOCKS * EXACT_GCAP * (8 + 4 + 4 + 4);
constexpr int EXACT_BINS = 1024;          // rank histogram of the large path's windows

// (Out of line: one copy serves the shared-memory and the global path.)
// Gather every triangle whose certified FP32 upper bound lies above the start
// height and reaches tcut into (key, tri, hi, qt)[slot] for slot < cap, and
// into the global scratch (gkey, ...)[slot] for cap <= slot < gcap (gkey may
// be null); one thread per grid cell under the cutter, all levels.  Returns
// the number found (may exceed both).
template <bool COMP>
__device__ __noinline__ int exact_gather(const DropCtx& ctx, double x, double y, float cx, float cy, float z0l,
                                            float tcut, const float* s_hlb, int& s_n, unsigned long long* key,
                                            uint32_t* tri, float* hiv, float* qtv, int cap,
                                            unsigned long long* gkey, uint32_t* gtri, float* ghi, float* gqt,
                                            int gcap) {
    const int tid = threadIdx.x;
    const GridP& g = ctx.g;
    const float R = ctx.prof.R, gd = ctx.guard, Rg = R + gd, inv_step = (float)HLB_N / R;
    const double reach = ctx.cp.radius + 1e-9 * (1.0 + ctx.cp.radius);
    if (tid == 0) s_n = 0;
    __syncthreads();
    for (int L = g.nlev - 1; L >= 0; --L) {
        int c0, c1, r0, r1;
        if (!warp_rect(g, L, x, x, y, y, reach, c0, c1, r0, r1)) continue;
        const int ncl = c1 - c0 + 1, ncells = ncl * (r1 - r0 + 1);
        const Cell* cells = ctx.cells + g.cell_off[L];
        for (int k = tid; k < ncells; k += blockDim.x) {
            const Cell cell = cells[(r0 + k / ncl) * g.ncol[L] + c0 + k % ncl];
            if (cell.count == 0) continue;
            float dx = fmaxf(0.0f, fmaxf(cell.minx - cx, cx - cell.maxx));
            float dy = fmaxf(0.0f, fmaxf(cell.miny - cy, cy - cell.maxy));
            float d = sqrtf(dx * dx + dy * dy);
            const float cub = cell.maxz - hlb_at(s_hlb, d - gd, inv_step);
            if (!(d <= Rg && cub > z0l - gd && cub >= tcut - gd)) continue;
            for (uint32_t j = 0; j < cell.count; ++j) {
                const Entry e = ctx.entries[cell.start + j];
                float ex = fmaxf(0.0f, fmaxf(e.minx - cx, cx - e.maxx));
                float ey = fmaxf(0.0f, fmaxf(e.miny - cy, cy - e.maxy));
                float de = sqrtf(ex * ex + ey * ey);
                float ub = e.maxz - hlb_at(s_hlb, de - gd, inv_step);
                if (!(de <= Rg && ub > z0l - gd && ub >= tcut - gd)) continue;
                const Tri32 t = ctx.t32[e.tri];
                float qt, qth;
                Iv v = COMP ? screen_composite(ctx.comp, t, cx - t.v0[0], cy - t.v0[1], ctx.E, z0l - t.v0[2], qt, qth)
                            : screen_triangle(ctx.prof, t, cx - t.v0[0], cy - t.v0[1], ctx.E, z0l - t.v0[2], qt, qth);
                if (!(v.hi > NEG_INF32)) continue;
                const float hi = fminf(v.hi + t.v0[2] + ctx.E, ub + gd);
                if (!(hi > z0l - gd && hi >= tcut)) continue;
                const int slot = atomicAdd(&s_n, 1);
                const unsigned long long kk = ((unsigned long long)t.kd_rank << 32) | (unsigned)slot;
                const float qv = qt < 3.0e38f ? qt + t.v0[2] - ctx.E : 3.0e38f;
                if (slot < cap) {
                    key[slot] = kk;
                    tri[slot] = (uint32_t)e.tri;
                    hiv[slot] = hi;
                    qtv[slot] = qv;
                } else if (gkey && slot < gcap) {
                    gkey[slot] = kk;
                    gtri[slot] = (uint32_t)e.tri;
                    ghi[slot] = hi;
                    gqt[slot] = qv;
                }
            }
        }
    }
    __syncthreads();
    return s_n;
}

// Only triangles whose upper bound reaches T are folded, T at most
// blo - guard (the final height lies above it) and at most every branch
// threshold of the triangles kept.  A triangle left out lifts the running
// height to below T at most; below its branch points a kept triangle's effect
// is max(Z, c) with a fixed c and CC; so max(Z, T) is the same in both folds
// after every triangle, and the final height, above T, is the same with its
// CC and type.
__device__ __forceinline__ float exact_threshold(const DropCtx& ctx, uint32_t i, const float* hiv, const float* qtv,
                                                 int n, int& s_red) {
    const int tid = threadIdx.x;
    const float gd = ctx.guard;
    float T = NEG_INF32;
    if (ctx.blo[i] > NEG_INF32) T = ctx.blo[i] - gd;
    for (int it = 0; T > NEG_INF32; ++it) {
        if (it == 64) {  // not settled: fold everything
            T = NEG_INF32;
            break;
        }
        if (tid == 0) s_red = f2o(3.0e38f);
        __syncthreads();
        float m = 3.0e38f;
        for (int k = tid; k < n; k += blockDim.x)
            if (hiv[k] >= T && qtv[k] - gd < T) m = fminf(m, qtv[k] - gd);
        if (m < 3.0e38f) atomicMin(&s_red, f2o(m));
        __syncthreads();
        const float mt = o2f(s_red);
        __syncthreads();
        if (!(mt < T)) break;
        T = mt;
    }
    return T;
}

// Bitonic sort of keys[0, n) in shared memory (padded to a power of two).
__device__ __forceinline__ void exact_sort(unsigned long long* s_key, int n) {
    const int tid = threadIdx.x;
    int np = 1;
    while (np < n) np <<= 1;
    for (int k = n + tid; k < np; k += blockDim.x) s_key[k] = ~0ull;
    __syncthreads();
    for (int k = 2; k <= np; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int a = tid; a < np; a += blockDim.x) {
                const int b = a ^ j;
                if (b > a) {
                    const unsigned long long ka = s_key[a], kb = s_key[b];
                    if ((ka > kb) == ((a & k) == 0)) {
                        s_key[a] = kb;
                        s_key[b] = ka;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Fold, in warp 0, the nk triangles whose keys are sorted in s_key (the low
// word indexes hiv / tri) in KD order, 32 at a time: every lane folds its own
// triangle from the running height; the first lane that lifts gives the next
// running height (the triangles before it did not lift from there, so the
// sequential fold passes them by).  A triangle that does not lift from a
// height does not lift from any higher one, so for the plain cutters only
// the later lanes that lifted fold again; a composite sub-cutter's facet can
// turn from a hidden contact to a lifting one as the height rises, so there
// every later lane does.
template <bool COMP>
__device__ __noinline__ void exact_fold(const DropCtx& ctx, CL64& cl, const unsigned long long* s_key, int nk,
                                           const float* hiv, const uint32_t* tri, float cxl, float cyl, int& capped,
                                           unsigned& evals) {
    const int lane = threadIdx.x & 31;
    const float gd = ctx.guard;
    for (int q0 = 0; q0 < nk; q0 += 32) {
        const int q = q0 + lane;
        const uint32_t slot = q < nk ? (uint32_t)s_key[q] : 0u;
        const float h = q < nk ? hiv[slot] : NEG_INF32;
        const uint32_t tr = q < nk ? tri[slot] : 0u;
        bool pend = q < nk;
        while (true) {
            const bool go = pend && h + gd >= __double2float_rd(cl.z - ctx.g.oz);
            if (!__any_sync(0xffffffffu, go)) break;
            CL64 mine = cl;
            if (go) {
                fold_one(ctx, mine, tr, cxl, cyl, capped);
                ++evals;
            }
            const bool lifted = go && mine.z > cl.z;
            const unsigned L = __ballot_sync(0xffffffffu, lifted);
            if (!L) break;
            const int b = __ffs(L) - 1;
            cl.z = __shfl_sync(0xffffffffu, mine.z, b);
            cl.cc.x = __shfl_sync(0xffffffffu, mine.cc.x, b);
            cl.cc.y = __shfl_sync(0xffffffffu, mine.cc.y, b);
            cl.cc.z = __shfl_sync(0xffffffffu, mine.cc.z, b);
            cl.type = __shfl_sync(0xffffffffu, mine.type, b);
            pend = go && lane > b && (COMP || lifted);
        }
    }
}

// Entries of the exact kernel's key arrays that are out of the fold: the
// rank word all ones (they sort after every kept key), the slot kept.
constexpr unsigned long long EXACT_DROPPED = 0xFFFFFFFF00000000ull;
constexpr int EXACT_PREFOLD = 4;   // pre-fold rounds at most
constexpr int EXACT_FEW = 64;      // kept triangles the sorted fold takes on cheaply

// Pre-fold of a handed-back point, by the whole block, before its kept
// triangles are sorted: warp 0 folds the lowest-ranked kept triangle (the
// first step of the in-order fold), then every kept triangle that can no
// longer lift is dropped -- its bbox top at or below the running height (the
// reference's below test skips it at this and every higher height) or its
// FP32 upper bound below the running height less the guard (the sorted
// fold's own skip) -- and the lowest-ranked of the rest is next, while many
// remain.  On a flat face under a flat-bottomed cutter, hundreds of
// triangles tie at the face's height; the first fold reaches it and drops
// them all, so they are neither sorted nor folded.  cl (warp 0's running
// point) carries on into the sorted fold.  Returns the kept count.
template <bool COMP>
__device__ __noinline__ int exact_prefold(const DropCtx& ctx, CL64& cl, unsigned long long* key, const float* hiv,
                                          const uint32_t* tri, int n, float cx, float cy, int& capped,
                                          unsigned& evals, unsigned long long* s_min, int& s_cnt) {
    const int tid = threadIdx.x, lane = tid & 31;
    const float gd = ctx.guard;
    int nk = n;
    double* s_z = reinterpret_cast<double*>(s_min + 1);
    for (int it = 0; it < EXACT_PREFOLD; ++it) {
        if (tid == 0) *s_min = ~0ull;
        __syncthreads();
        unsigned long long m = ~0ull;
        for (int k = tid; k < n; k += blockDim.x) {
            const unsigned long long kk = key[k];
            if ((kk >> 32) != 0xFFFFFFFFull && kk < m) m = kk;
        }
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long v = __shfl_xor_sync(0xffffffffu, m, o);
            if (v < m) m = v;
        }
        if (lane == 0 && m != ~0ull) atomicMin(s_min, m);
        __syncthreads();
        const unsigned long long best = *s_min;
        if (best == ~0ull) {
            nk = 0;
            break;
        }
        if (tid < 32) {
            // every lane of warp 0 folds it (cl stays the same across the warp)
            int c1 = 0;
            fold_one(ctx, cl, tri[(uint32_t)best], cx, cy, c1);
            if (lane == 0) {
                ++evals;
                capped += c1;
            }
        }
        if (tid == 0) {
            *s_z = cl.z;
            s_cnt = 0;
        }
        __syncthreads();
        const double Z = *s_z;
        const float zl = __double2float_rd(Z - ctx.g.oz);
        int kept = 0;
        for (int k = tid; k < n; k += blockDim.x) {
            const unsigned long long kk = key[k];
            if ((kk >> 32) == 0xFFFFFFFFull) continue;
            const uint32_t slot = (uint32_t)kk;
            if (kk == best || !(hiv[slot] + gd >= zl) || !(Z < ctx.t64[tri[slot]].bb[5])) key[k] = EXACT_DROPPED | slot;
            else ++kept;
        }
        for (int o = 16; o > 0; o >>= 1) kept += __shfl_xor_sync(0xffffffffu, kept, o);
        if (lane == 0 && kept) atomicAdd(&s_cnt, kept);
        __syncthreads();
        nk = s_cnt;
        __syncthreads();
        if (nk <= EXACT_FEW) break;
    }
    return nk;
}

// One handed-back point, by the whole block.
template <bool COMP>
__device__ __forceinline__ void exact_point(const DropCtx& ctx, const uint32_t i, const ExactShared& S,
                                            const ExactGlobal& G, uint32_t* __restrict__ list2,
                                            unsigned long long* __restrict__ nlist2) {
    unsigned long long* s_key = S.key;
    int& s_red = *S.red;
    const int tid = threadIdx.x, lane = tid & 31;
    const GridP& g = ctx.g;
    const double x = ctx.cl[3 * i], y = ctx.cl[3 * i + 1], z0 = ctx.cl[3 * i + 2];
    const float cx = (float)(x - g.ox), cy = (float)(y - g.oy);
    const float z0l = __double2float_rd(z0 - g.oz);
    const size_t base = (size_t)blockIdx.x * (size_t)G.cap;
    unsigned long long* gk = G.key + base;
    uint32_t* gt = G.tri + base;
    float* gh = G.hi + base;
    float* gq = G.qt + base;
    // Only triangles whose upper bound reaches the fold threshold T matter,
    // and T starts at the screen's certified lower bound less the guard: gather
    // those first; should a branch threshold take T lower, gather again from
    // there (the third time from the start height, which takes in every
    // triangle the threshold can reach).
    float tcut = ctx.blo[i] > NEG_INF32 ? ctx.blo[i] - ctx.guard : NEG_INF32;
    int n = 0;
    float T = NEG_INF32;
    bool in_shared = true;
    for (int pass = 0;; ++pass) {
        // the global scratch takes what shared memory cannot hold
        n = exact_gather<COMP>(ctx, x, y, cx, cy, z0l, tcut, S.hlb, *S.n, s_key, S.tri, S.hi, S.qt, EXACT_CAP,
                               G.key ? gk : nullptr, gt, gh, gq, G.cap);
        in_shared = n <= EXACT_CAP;
        if (!in_shared) {
            if (!(G.key && n <= G.cap)) {
                if (tid == 0) list2[atomicAdd(nlist2, 1ull)] = i;
                __syncthreads();
                return;
            }
            // the first EXACT_CAP entries are in shared memory: all into the
            // global scratch (the slot in a key's low word is its index there)
            for (int k = tid; k < EXACT_CAP; k += blockDim.x) {
                gk[k] = s_key[k];
                gt[k] = S.tri[k];
                gh[k] = S.hi[k];
                gq[k] = S.qt[k];
            }
            __syncthreads();
        }
        T = in_shared ? exact_threshold(ctx, i, S.hi, S.qt, n, s_red) : exact_threshold(ctx, i, gh, gq, n, s_red);
        if (!(T < tcut)) break;
        tcut = pass == 0 ? T : NEG_INF32;
    }
    CL64 cl{x, y, z0, d3(0, 0, 0), OCL_CC_NONE};
    int capped = 0;
    unsigned evals = 0;
    if (in_shared) {
        if (tid == 0) s_red = 0;
        __syncthreads();
        int kept = 0;
        for (int k = tid; k < n; k += blockDim.x) {
            if (S.hi[k] >= T) ++kept;
            else s_key[k] = EXACT_DROPPED | (unsigned)k;  // sorts after the kept keys
        }
        if (kept) atomicAdd(&s_red, kept);
        __syncthreads();
        int nk = s_red;
        __syncthreads();
        if (nk > EXACT_FEW)
            nk = exact_prefold<COMP>(ctx, cl, s_key, S.hi, S.tri, n, cx, cy, capped, evals, S.pre, s_red);
        exact_sort(s_key, n);
        if (tid < 32) exact_fold<COMP>(ctx, cl, s_key, nk, S.hi, S.tri, cx, cy, capped, evals);
    } else {
        // More candidates than shared memory holds: gathered into this
        // block's global scratch and folded in KD order one rank window at a
        // time (each window's ranks chosen so it fits shared memory), the
        // running height carried from window to window.
        for (int k = tid; k < n; k += blockDim.x)
            if (!(gh[k] >= T)) gk[k] = EXACT_DROPPED | (unsigned)k;
        __syncthreads();
        exact_prefold<COMP>(ctx, cl, gk, gh, gt, n, cx, cy, capped, evals, S.pre, s_red);
        int* hist = reinterpret_cast<int*>(S.qt);  // the shared thresholds are not used on this path
        uint64_t cur = 0;
        for (;;) {
            // kept entries with rank >= cur: how many, and the largest rank
            if (tid == 0) {
                s_red = 0;
                hist[0] = -1;
            }
            __syncthreads();
            int cnt = 0, rmax = -1;
            for (int k = tid; k < n; k += blockDim.x) {
                const uint32_t r = (uint32_t)(gk[k] >> 32);
                if (r != 0xFFFFFFFFu && r >= cur) {
                    ++cnt;
                    rmax = max(rmax, (int)r);
                }
            }
            if (cnt) {
                atomicAdd(&s_red, cnt);
                atomicMax(&hist[0], rmax);
            }
            __syncthreads();
            const int total = s_red;
            uint64_t hi = (uint64_t)hist[0] + 1;
            __syncthreads();
            if (total == 0) break;
            if (total > EXACT_CAP) {
                // the longest run of histogram bins from `cur` holding at most EXACT_CAP
                for (;;) {
                    const uint64_t w = (hi - cur + EXACT_BINS - 1) / EXACT_BINS;
                    for (int b = tid; b < EXACT_BINS; b += blockDim.x) hist[b] = 0;
                    __syncthreads();
                    for (int k = tid; k < n; k += blockDim.x) {
                        const uint64_t r = gk[k] >> 32;
                        if (r != 0xFFFFFFFFull && r >= cur && r < hi) atomicAdd(&hist[(r - cur) / w], 1);
                    }
                    __syncthreads();
                    if (tid == 0) {
                        int acc = 0, j = -1;
                        for (int b = 0; b < EXACT_BINS; ++b) {
                            if (acc + hist[b] > EXACT_CAP) break;
                            acc += hist[b];
                            j = b;
                        }
                        s_red = j;
                    }
                    __syncthreads();
                    const int j = s_red;
                    __syncthreads();
                    if (j >= 0) {
                        hi = min(hi, cur + (uint64_t)(j + 1) * w);
                        break;
                    }
                    hi = cur + w;  // the first bin alone is too full (w > 1: ranks are distinct)
                }
            }
            // the window's keys into shared memory, sorted, folded
            if (tid == 0) s_red = 0;
            __syncthreads();
            for (int k = tid; k < n; k += blockDim.x) {
                const uint64_t r = gk[k] >> 32;
                if (r != 0xFFFFFFFFull && r >= cur && r < hi) {
                    const int slot = atomicAdd(&s_red, 1);
                    s_key[slot] = (r << 32) | (unsigned)k;
                }
            }
            __syncthreads();
            const int nw = s_red;
            exact_sort(s_key, nw);
            if (tid < 32) exact_fold<COMP>(ctx, cl, s_key, nw, gh, gt, cx, cy, capped, evals);
            __syncthreads();
            cur = hi;
        }
    }
    if (tid < 32) {
        for (int o = 16; o > 0; o >>= 1) {
            evals += __shfl_xor_sync(0xffffffffu, evals, o);
            capped += __shfl_xor_sync(0xffffffffu, capped, o);
        }
        if (lane == 0) {
            const uint32_t o = ctx.perm[i];
            ctx.out_z[o] = cl.z;
            ctx.out_cc[3 * o] = cl.cc.x;
            ctx.out_cc[3 * o + 1] = cl.cc.y;
            ctx.out_cc[3 * o + 2] = cl.cc.z;
            ctx.out_type[o] = cl.type;
            if (evals) atomicAdd(&ctx.counters[C_REFINED], (unsigned long long)evals);
            if (capped) atomicAdd(&ctx.counters[C_CAPPED], (unsigned long long)capped);
        }
    }
    __syncthreads();
}

#define OCLG_EXACT_SHARED                                                                    \
    extern __shared__ unsigned long long s_key[];                                            \
    __shared__ float s_hlb[HLB_N];                                                           \
    __shared__ int s_n, s_red;                                                               \
    __shared__ unsigned long long s_pre[2];                                                  \
    ExactShared S;                                                                           \
    S.key = s_key;                                                                           \
    S.tri = reinterpret_cast<uint32_t*>(s_key + EXACT_CAP);                                  \
    S.hi = reinterpret_cast<float*>(S.tri + EXACT_CAP);                                      \
    S.qt = S.hi + EXACT_CAP;                                                                 \
    S.hlb = s_hlb;                                                                           \
    S.n = &s_n;                                                                              \
    S.red = &s_red;                                                                          \
    S.pre = s_pre;

template <bool COMP>
__global__ void __launch_bounds__(EXACT_THREADS) k_drop_exact(const __grid_constant__ DropCtx ctx,
                                                              const uint32_t* __restrict__ list,
                                                              const unsigned long long* __restrict__ nlist_dev,
                                                              uint32_t* __restrict__ list2,
                                                              unsigned long long* __restrict__ nlist2,
                                                              const ExactGlobal G) {
    OCLG_EXACT_SHARED
    for (int k = threadIdx.x; k < HLB_N; k += blockDim.x) s_hlb[k] = ctx.hlb[k];
    const int nlist = (int)*nlist_dev;
    for (int p = blockIdx.x; p < nlist; p += gridDim.x) exact_point<COMP>(ctx, list[p], S, G, list2, nlist2);
}

// Batch: every block strides over the handed-back points of each job in turn.
template <bool COMP>
__global__ void __launch_bounds__(EXACT_THREADS) k_drop_exact_b(const __grid_constant__ BatchView bv,
                                                                const ExactGlobal G) {
    OCLG_EXACT_SHARED
    for (unsigned k = 0; k < bv.njobs; ++k) {
        const DropCtx& ctx = bv.ctxs[bv.jobs[k]];
        const int nlist = (int)ctx.counters[C_FALLBACK];
        if (nlist == 0) continue;
        __syncthreads();
        for (int q = threadIdx.x; q < HLB_N; q += blockDim.x) s_hlb[q] = ctx.hlb[q];
        for (int p = blockIdx.x; p < nlist; p += gridDim.x)
            exact_point<COMP>(ctx, ctx.list[p], S, G, ctx.list2, ctx.counters + C_PLAIN);
    }
}
#undef OCLG_EXACT_SHARED

__global__ void k_collect_overflow(const uint16_t* ncand, int M, uint32_t* list, unsigned long long* counter) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    if (ncand[i] == 0xFFFF) {
        unsigned long long slot = atomicAdd(counter, 1ull);
        list[slot] = (uint32_t)i;
    }
}

__global__ void __launch_bounds__(128) k_collect_overflow_b(const __grid_constant__ BatchView bv) {
    __shared__ DropCtx s_ctx;
    __shared__ TileState ts;
    if (threadIdx.x == 0) ts.job = 0xFFFFFFFFu;
    uint2 tile;
    while (batch_next_tile(bv, ts, s_ctx, tile)) {
        const uint32_t i = tile.y * TILE_POINTS + threadIdx.x;
        if (i < (uint32_t)s_ctx.M && s_ctx.ncand[i] == 0xFFFF)
            s_ctx.list[atomicAdd(&s_ctx.counters[C_FALLBACK], 1ull)] = i;
    }
}

// ---------------------------------------------------------------------------
// Batch ordering: Morton keys of every job's points in the job's own frame,
// prefixed by the job index, so one radix sort orders the whole wave job by
// job (each job's points stay a contiguous segment) and along the curve
// within a job.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t batch_job_of(const BatchIn* __restrict__ in, uint32_t njobs, uint64_t g) {
    uint32_t lo = 0, hi = njobs - 1;  // last job with off <= g
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (in[mid].off <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void k_batch_morton(const BatchIn* __restrict__ in, uint32_t njobs, uint64_t Mtot,
                               unsigned long long* __restrict__ keys, uint32_t* __restrict__ idx) {
    const uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (g >= Mtot) return;
    const uint32_t j = batch_job_of(in, njobs, g);
    const BatchIn b = in[j];
    const uint64_t i = g - b.off;
    const double fx = (b.cl[3 * i] - b.x0) * b.sx, fy = (b.cl[3 * i + 1] - b.y0) * b.sy;
    const uint32_t qx = (uint32_t)fmin(fmax(fx, 0.0), 65535.0);
    const uint32_t qy = (uint32_t)fmin(fmax(fy, 0.0), 65535.0);
    keys[g] = ((unsigned long long)j << 32) | (spread16(qx) | (spread16(qy) << 1));
    idx[g] = (uint32_t)g;
}

__global__ void k_batch_gather(const BatchIn* __restrict__ in, const unsigned long long* __restrict__ keys,
                               const uint32_t* __restrict__ idx, uint64_t Mtot, double* __restrict__ cls,
                               uint32_t* __restrict__ perm) {
    const uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (p >= Mtot) return;
    const uint32_t j = (uint32_t)(keys[p] >> 32);
    const BatchIn& b = in[j];
    const uint64_t i = idx[p] - b.off;
    cls[3 * p] = b.cl[3 * i];
    cls[3 * p + 1] = b.cl[3 * i + 1];
    cls[3 * p + 2] = b.cl[3 * i + 2];
    perm[p] = (uint32_t)i;  // the job-local caller index
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct DropWork {
    DevBuf<uint32_t> keys, keys2, perm0, perm;
    DevBuf<double> cls;
    DevBuf<uint32_t> cand;
    DevBuf<float> cand_hi, cand_lo;
    DevBuf<uint16_t> ncand;
    DevBuf<float> blo;
    DevBuf<uint32_t> list, list2, sparse;
    DevBuf<unsigned long long> counters;
    // bull edges ahead of the fold (allocated on first use)
    DevBuf<uint32_t> edge_slots;
    DevBuf<uint8_t> edge_n;
    DevBuf<EdgeRes> edge_res;
    DevBuf<uint2> edge_queue;
    size_t edge_cap = 0;
    bool ensure_edges(size_t M) {
        if (M <= edge_cap) return true;
        const size_t c = std::max<size_t>(M, 1024);
        if (!edge_slots.alloc(c * EDGE_SLOTS) || !edge_n.alloc(c) || !edge_res.alloc(c * EDGE_SLOTS) ||
            !edge_queue.alloc(c * EDGE_SLOTS))
            return false;
        edge_cap = c;
        return true;
    }
    DevBuf<uint8_t> sort_tmp;
    DevBuf<unsigned char> exact_scratch;  // handed-back points with many candidates
    DropCtx* host_ctx = nullptr;  // launch context (kernel parameter)
    // per-call stage events, a ring over the last STAGE_RING calls (read
    // afterwards by ocl_gb300_stage_times without syncing the calls)
    static constexpr int STAGE_RING = 256;
    cudaEvent_t ring[STAGE_RING][5] = {};
    int ring_pos = 0;
    uint64_t ring_count = 0;
    size_t cap = 0;
    bool ensure(size_t M, size_t sort_bytes) {
        if (M > cap || !counters.p) {
            size_t c = std::max<size_t>(M, 1024);
            if (!keys.alloc(c) || !keys2.alloc(c) || !perm0.alloc(c) || !perm.alloc(c) || !cls.alloc(3 * c) ||
                !cand.alloc(c * CAND_K) || !cand_hi.alloc(c * CAND_K) || !cand_lo.alloc(c * CAND_K) || !ncand.alloc(c) || !blo.alloc(c) || !list.alloc(c) || !list2.alloc(c) || !sparse.alloc(c / 32 + 1) ||
                !counters.alloc(C_NCOUNTERS + 1))
                return false;
            cap = c;
        }
        if (sort_bytes > sort_tmp.n && !sort_tmp.alloc(sort_bytes)) return false;
        return true;
    }
};

// One workspace per (host thread, CUDA context): its buffers, events and
// launch context belong to the device that was current when they were made.
// tl_work is the calling thread's workspace for its current context.
static thread_local std::map<uint64_t, DropWork*> tl_works;
static thread_local DropWork* tl_work = nullptr;

static DropWork* work_for_current_context() {
    const uint64_t key = context_key();
    if (!key) return nullptr;
    DropWork*& w = tl_works[key];
    if (!w) w = new DropWork();
    tl_work = w;
    return w;
}

// The dense screen kernel over all warps, then the sparse one over the warps
// whose points it found spread out (a fixed grid striding over the list).
// Seeding kernel (bounds of spread-out warps), the dense screen kernel over
// all warps, then the sparse one over the warps it found scattered (a fixed
// grid striding over the list).  `h` must have `seeded` set.
static void launch_screen(const DropCtx& h, const CutterP& cp, unsigned blocks, cudaStream_t stream) {
    const unsigned sblocks = std::min<unsigned>(blocks, 152u * 4u);
    if (cp.kind == OCL_CUTTER_COMPOSITE) {
        // the presets' make-ups (compositecutter.cpp:298-383) get their own kernels
        const int sig = cp.nsub == 3 ? comp_sig(cp.sub[0].kind, cp.sub[1].kind, cp.sub[2].kind) : -1;
        if (!screen_launch_comp_a_sparse(h, sig, blocks, stream, 0) &&
            !screen_launch_comp_b_sparse(h, sig, blocks, stream, 0))
            screen_launch_comp_any_sparse(h, blocks, stream, 0);
        if (!screen_launch_comp_a(h, sig, blocks, stream) && !screen_launch_comp_b(h, sig, blocks, stream))
            screen_launch_comp_any(h, blocks, stream);
        if (!screen_launch_comp_a_sparse(h, sig, sblocks, stream, 1) &&
            !screen_launch_comp_b_sparse(h, sig, sblocks, stream, 1))
            screen_launch_comp_any_sparse(h, sblocks, stream, 1);
    } else {
        const int kind = cp.kind == OCL_CUTTER_CONE ? OCL_CUTTER_CONE : cp.b.kind;
        screen_launch_basic_sparse(h, kind, blocks, stream, 0);
        screen_launch_basic(h, kind, blocks, stream);
        screen_launch_basic_sparse(h, kind, sblocks, stream, 1);
    }
}

// The exact kernels' dynamic shared memory (above the 48 KB default) is a
// property of each kernel in one context: opted in once per context
// (device), not once per process.
int ensure_exact_smem() {
    static std::mutex mu;
    static std::set<uint64_t> done;
    const uint64_t key = context_key();
    if (!key) return OCL_GB300_DEVICE_ERROR;
    std::lock_guard<std::mutex> lk(mu);
    if (done.count(key)) return OCL_GB300_OK;
    const void* kernels[4] = {(const void*)k_drop_exact<false>, (const void*)k_drop_exact<true>,
                              (const void*)k_drop_exact_b<false>, (const void*)k_drop_exact_b<true>};
    for (const void* k : kernels) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)EXACT_SMEM);
        if (e != cudaSuccess) {
            set_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
            return OCL_GB300_DEVICE_ERROR;
        }
    }
    done.insert(key);
    return OCL_GB300_OK;
}

// k_drop_exact over the handed-back points (count on the device).
// G.key == nullptr: no global scratch (points beyond EXACT_CAP candidates go
// to the plain kernel).  With scratch the grid is at most EXACT_GBLOCKS (one
// scratch region per block).
static int launch_exact(const DropCtx& h, bool composite, const uint32_t* list, const unsigned long long* nlist,
                        uint32_t* list2, unsigned long long* nlist2, unsigned blocks, cudaStream_t stream,
                        const ExactGlobal& G) {
    int st = ensure_exact_smem();
    if (st) return st;
    if (blocks == 0) blocks = 1;
    if (G.key) blocks = std::min<unsigned>(blocks, (unsigned)EXACT_GBLOCKS);
    if (composite)
        k_drop_exact<true><<<blocks, EXACT_THREADS, EXACT_SMEM, stream>>>(h, list, nlist, list2, nlist2, G);
    else
        k_drop_exact<false><<<blocks, EXACT_THREADS, EXACT_SMEM, stream>>>(h, list, nlist, list2, nlist2, G);
    return OCL_GB300_OK;
}

// The exact kernel's global scratch carved from one byte buffer of EXACT_GBYTES.
static ExactGlobal exact_global_in(unsigned char* p) {
    ExactGlobal G;
    const size_t n = (size_t)EXACT_GBLOCKS * EXACT_GCAP;
    G.key = reinterpret_cast<unsigned long long*>(p);
    G.tri = reinterpret_cast<uint32_t*>(p + n * 8);
    G.hi = reinterpret_cast<float*>(p + n * 12);
    G.qt = reinterpret_cast<float*>(p + n * 16);
    G.cap = EXACT_GCAP;
    return G;
}

void init_drop_ctx(const Mesh& m, const CutterP& cp, DropCtx& h) {
    std::memset(&h, 0, sizeof(DropCtx));
    h.cp = cp;
    h.g = m.grid;
    h.cells = m.d_cells;
    h.entries = m.d_entries;
    h.t64 = m.d_t64;
    h.t32 = m.d_t32;
    h.kd_nodes = m.drop_kd.d_nodes;
    h.kd_order = m.drop_kd.d_order;
    h.seeded = true;
    bool composite = false;
    fill_prof(cp, h.prof, h.hlb, composite);
    h.composite_screen = composite;
    fill_comp(cp, h.comp);
    // FP32 position error budget of the local frame (coordinates up to half
    // the mesh extent plus the cutter radius from the origin) and the margin
    // of every bound test
    const double half = 0.5 * std::max(m.bb[1] - m.bb[0], std::max(m.bb[3] - m.bb[2], m.bb[5] - m.bb[4]));
    const double maxabs = half + cp.radius + 1.0;
    h.E = (float)(8.0 * maxabs * std::ldexp(1.0, -24) + 4e-6 * std::max(1.0, cp.radius));
    h.guard = 4.0f * h.E + 1e-5f * (float)cp.radius;
}

// The mixed-precision pipeline over the sorted points of `h` (M of them):
// screens, bull edges, refinement, hand-back; cnt are the pass's counters.
// ev_screen / ev_refine (may be null) mark the end of the screen and
// refinement stages.
static int enqueue_mixed(DropWork& w, const Mesh& m, const CutterP& cp, DropCtx& h, uint64_t M,
                         unsigned long long* cnt, cudaStream_t stream, cudaEvent_t ev_screen, cudaEvent_t ev_refine,
                         uint64_t& launches) {
    h.counters = cnt;
    h.sparse_n = cnt + C_SPARSE;
    const bool composite = h.composite_screen;
    const int TB = 256;
    const unsigned nb = (unsigned)((M + TB - 1) / TB);
    const unsigned warps = (unsigned)((M + 31) / 32);
    const unsigned sblocks = (warps + SCREEN_WARPS - 1) / SCREEN_WARPS;
    launch_screen(h, cp, sblocks, stream);
    if (ev_screen) CK(cudaEventRecord(ev_screen, stream));
    h.edge_slots = nullptr;
    h.edge_n = nullptr;
    h.edge_res = nullptr;
    if (cp.kind == OCL_CUTTER_BULL && m.n < (1ull << 30)) {
        if (!w.ensure_edges(M)) return OCL_GB300_OOM;
        h.edge_slots = w.edge_slots.p;
        h.edge_n = w.edge_n.p;
        h.edge_res = w.edge_res.p;
        k_bull_plan<<<(unsigned)((M + 127) / 128), 128, 0, stream>>>(h, w.edge_queue.p, cnt + C_EDGEQ);
        const unsigned eb = (unsigned)std::min<uint64_t>((M * EDGE_SLOTS + 127) / 128, 152u * 16u);
        k_bull_eval<<<eb, 128, 0, stream>>>(h, w.edge_queue.p, cnt + C_EDGEQ);
        launches += 2;
    }
    if (h.edge_res) k_drop_refine<true><<<(unsigned)((M + 127) / 128), 128, 0, stream>>>(h);
    else k_drop_refine<false><<<(unsigned)((M + 127) / 128), 128, 0, stream>>>(h);
    if (ev_refine) CK(cudaEventRecord(ev_refine, stream));
    k_collect_overflow<<<nb, TB, 0, stream>>>(w.ncand.p, (int)M, w.list.p, cnt + C_FALLBACK);
    // the fallback grids stride over however many points were handed back
    if (!w.exact_scratch.reserve(EXACT_GBYTES)) return OCL_GB300_OOM;
    int st = launch_exact(h, composite, w.list.p, cnt + C_FALLBACK, w.list2.p, cnt + C_PLAIN,
                          (unsigned)std::min<uint64_t>(M, (uint64_t)EXACT_GBLOCKS), stream,
                          exact_global_in(w.exact_scratch.p));
    if (st) return st;
    const unsigned fb_blocks = std::min<unsigned>((warps + 3) / 4, 152u * 16u);
    k_drop_kd<true><<<fb_blocks, 128, 0, stream>>>(h, w.list2.p, cnt + C_PLAIN);
    launches += 7;  // seed, dense and sparse screen, refine, collect, exact, plain
    return OCL_GB300_OK;
}

int drop_run(Mesh& m, const CutterP& cp, const double* d_cl, uint64_t M, int precision, double* d_z, double* d_cc,
             int32_t* d_type, cudaStream_t stream, ocl_gb300_stats* stats) {
    if (M == 0) return OCL_GB300_OK;
    if (M >= (1ull << 31)) {
        set_error("too many CL points");
        return OCL_GB300_BAD_ARG;
    }
    DropWork* wp = work_for_current_context();
    if (!wp) return OCL_GB300_DEVICE_ERROR;
    DropWork& w = *wp;
    size_t sort_bytes = 0;
    CK(cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, w.keys.p, w.keys2.p, w.perm0.p, w.perm.p, (int64_t)M, 0,
                                       32, stream));
    if (!w.ensure(M, sort_bytes)) return OCL_GB300_OOM;
    int st = OCL_GB300_OK;

    if (!w.host_ctx) w.host_ctx = new DropCtx();
    DropCtx* h = w.host_ctx;  // passed by value as the kernels' __grid_constant__ parameter
    init_drop_ctx(m, cp, *h);
    h->cl = w.cls.p;
    h->perm = w.perm.p;
    h->M = (int)M;
    h->out_z = d_z;
    h->out_cc = d_cc;
    h->out_type = d_type;
    h->cand = w.cand.p;
    h->cand_hi = w.cand_hi.p;
    h->cand_lo = w.cand_lo.p;
    h->cand_cap = CAND_K;
    h->ncand = w.ncand.p;
    h->blo = w.blo.p;
    h->sparse_list = w.sparse.p;
    h->sparse_n = w.counters.p + C_SPARSE;
    h->counters = w.counters.p;

    cudaEvent_t* ev = w.ring[w.ring_pos];
    if (!ev[0]) {
        for (int k = 0; k < 5; ++k) CK(cudaEventCreate(&ev[k]));
    }
    w.ring_pos = (w.ring_pos + 1) % DropWork::STAGE_RING;
    ++w.ring_count;
    uint64_t launches = 0;
    CK(cudaEventRecord(ev[0], stream));
    CK(cudaMemsetAsync(w.counters.p, 0, (C_NCOUNTERS + 1) * sizeof(unsigned long long), stream));
    const int TB = 256;
    const unsigned nb = (unsigned)((M + TB - 1) / TB);
    double ex = std::max(m.bb[1] - m.bb[0], 1e-9), ey = std::max(m.bb[3] - m.bb[2], 1e-9);
    double sx = 65535.0 / (ex + 2 * cp.radius), sy = 65535.0 / (ey + 2 * cp.radius);
    k_morton<<<nb, TB, 0, stream>>>(d_cl, M, m.bb[0] - cp.radius, m.bb[2] - cp.radius, sx, sy, w.keys.p, w.perm0.p);
    CK(cub::DeviceRadixSort::SortPairs(w.sort_tmp.p, sort_bytes, w.keys.p, w.keys2.p, w.perm0.p, w.perm.p,
                                       (int64_t)M, 0, 32, stream));
    k_gather_cl<<<nb, TB, 0, stream>>>(d_cl, w.perm.p, M, w.cls.p);
    launches += 2;
    const unsigned warps = (unsigned)((M + 31) / 32);
    CK(cudaEventRecord(ev[1], stream));
    if (m.n == 0) {
        // empty surface: every point keeps its z, CC stays NONE
        CK(cudaMemsetAsync(w.ncand.p, 0, M * sizeof(uint16_t), stream));
        CK(cudaMemsetAsync(w.blo.p, 0xFF, M * sizeof(float), stream));
        CK(cudaEventRecord(ev[2], stream));
        k_drop_refine<false><<<(unsigned)((M + 127) / 128), 128, 0, stream>>>(*h);
        CK(cudaEventRecord(ev[3], stream));
        launches += 1;
    } else if (precision == OCL_GB300_PREC_FP64) {
        CK(cudaEventRecord(ev[2], stream));
        CK(cudaEventRecord(ev[3], stream));
        k_drop_kd<false><<<(warps + 3) / 4, 128, 0, stream>>>(*h, nullptr, nullptr);
        launches += 1;
    } else {
        st = enqueue_mixed(w, m, cp, *h, M, w.counters.p, stream, ev[2], ev[3], launches);
        if (st) return st;
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(ev[4], stream));
    if (stats) {
        unsigned long long c[C_NCOUNTERS];
        CK(cudaMemcpyAsync(c, w.counters.p, sizeof(c), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        float t_all = 0, t_scr = 0, t_ref = 0, t_fb = 0;
        cudaEventElapsedTime(&t_all, ev[0], ev[4]);
        cudaEventElapsedTime(&t_scr, ev[1], ev[2]);
        cudaEventElapsedTime(&t_ref, ev[2], ev[3]);
        cudaEventElapsedTime(&t_fb, ev[3], ev[4]);
        stats->pairs = c[C_PAIRS];
        stats->refined = c[C_REFINED];
        stats->iter_limit_hits = c[C_CAPPED];
        stats->fallback = c[C_FALLBACK];
        stats->violations = c[C_VIOLATION];
        stats->screened = c[C_SCREENED];
        stats->overflow_points = c[C_OVERFLOW];
        stats->chain_points = c[C_CHAIN];
        stats->open_branch_points = c[C_OPEN];
        stats->untracked_branch_points = c[C_UNTRACKED];
        stats->plain_points = c[C_PLAIN];
        stats->verify_failed_points = c[C_VFAIL];
        stats->launches = launches;
        stats->kernel_ms = t_all;
        stats->screen_ms = t_scr;
        stats->refine_ms = t_ref;
        stats->fallback_ms = t_fb;
    }
    return OCL_GB300_OK;
}


// ---------------------------------------------------------------------------
// Batch launchers (ocl_gb300_drop_batch, batch.cu)
// ---------------------------------------------------------------------------
size_t batch_sort_bytes(uint64_t Mtot, int end_bit) {
    size_t b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, b, (unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                    (uint32_t*)nullptr, (uint32_t*)nullptr, (int64_t)Mtot, 0, end_bit);
    return b;
}

void batch_launch_order(const BatchIn* d_in, uint32_t njobs, uint64_t Mtot, unsigned long long* keys, uint32_t* idx,
                        unsigned long long* keys2, uint32_t* idx2, void* sort_tmp, size_t sort_bytes, int end_bit,
                        double* cls, uint32_t* perm, cudaStream_t stream, int* status) {
    const unsigned nb = (unsigned)((Mtot + 255) / 256);
    k_batch_morton<<<nb, 256, 0, stream>>>(d_in, njobs, Mtot, keys, idx);
    const cudaError_t e = cub::DeviceRadixSort::SortPairs(sort_tmp, sort_bytes, keys, keys2, idx, idx2, (int64_t)Mtot,
                                                          0, end_bit, stream);
    if (e != cudaSuccess) {
        set_error(std::string("batch sort: ") + cudaGetErrorString(e));
        *status = OCL_GB300_DEVICE_ERROR;
        return;
    }
    k_batch_gather<<<nb, 256, 0, stream>>>(d_in, keys2, idx2, Mtot, cls, perm);
}

void batch_launch_bull(const BatchView& plan, const BatchView& eval, unsigned blocks, cudaStream_t stream) {
    k_bull_plan_b<<<blocks, TILE_POINTS, 0, stream>>>(plan);
    k_bull_eval_b<<<blocks, 128, 0, stream>>>(eval);
}

void batch_launch_refine(const BatchView& bv, bool bull_plan, unsigned blocks, cudaStream_t stream) {
    if (bull_plan) k_drop_refine_b<true><<<blocks, TILE_POINTS, 0, stream>>>(bv);
    else k_drop_refine_b<false><<<blocks, TILE_POINTS, 0, stream>>>(bv);
}

void batch_launch_collect(const BatchView& bv, unsigned blocks, cudaStream_t stream) {
    k_collect_overflow_b<<<blocks, TILE_POINTS, 0, stream>>>(bv);
}

int batch_launch_exact(const BatchView& bv, bool composite, unsigned blocks, cudaStream_t stream,
                       unsigned char* scratch) {
    int st = ensure_exact_smem();
    if (st) return st;
    const ExactGlobal G = scratch ? exact_global_in(scratch) : ExactGlobal{};
    if (G.key) blocks = std::min<unsigned>(blocks, (unsigned)EXACT_GBLOCKS);
    if (composite) k_drop_exact_b<true><<<blocks, EXACT_THREADS, EXACT_SMEM, stream>>>(bv, G);
    else k_drop_exact_b<false><<<blocks, EXACT_THREADS, EXACT_SMEM, stream>>>(bv, G);
    return OCL_GB300_OK;
}

size_t batch_exact_scratch_bytes() { return EXACT_GBYTES; }

void batch_launch_plain(const BatchView& bv, unsigned blocks, cudaStream_t stream) {
    k_drop_kd_b<<<blocks, 128, 0, stream>>>(bv);
}

int drop_stage_times(uint64_t count, double* out) {
    if (!tl_work) return count == 0 ? OCL_GB300_OK : OCL_GB300_BAD_ARG;
    DropWork& w = *tl_work;
    if (count > w.ring_count || count > (uint64_t)DropWork::STAGE_RING) {
        set_error("stage times: fewer recorded calls than requested");
        return OCL_GB300_BAD_ARG;
    }
    for (uint64_t k = 0; k < count; ++k) {
        const int slot = (int)((w.ring_pos - (int64_t)count + (int64_t)k + 4 * DropWork::STAGE_RING) %
                               DropWork::STAGE_RING);
        cudaEvent_t* ev = w.ring[slot];
        CK(cudaEventSynchronize(ev[4]));
        float t_all = 0, t_scr = 0, t_ref = 0, t_fb = 0;
        CK(cudaEventElapsedTime(&t_all, ev[0], ev[4]));
        CK(cudaEventElapsedTime(&t_scr, ev[1], ev[2]));
        CK(cudaEventElapsedTime(&t_ref, ev[2], ev[3]));
        CK(cudaEventElapsedTime(&t_fb, ev[3], ev[4]));
        out[4 * k] = t_scr;
        out[4 * k + 1] = t_ref;
        out[4 * k + 2] = t_fb;
        out[4 * k + 3] = t_all;
    }
    return OCL_GB300_OK;
}

// ---------------------------------------------------------------------------
// Drop without any device allocation (ocl_gb300_drop_device_noalloc).
//
// For callers that cannot allocate device memory while they run: a machine
// controller or real-time loop whose device memory is budgeted up front (a
// cudaMalloc can synchronise the device and stall the loop), or a host process
// whose own pool allocator owns the device's memory and forbids other
// allocations.  All scratch lives in one file-scope __device__ array sized for
// OCL_GB300_NOALLOC_MAX_POINTS points, loaded with the library and held by
// every device that loads it until the process exits.  Points are processed
// in the caller's order (no sort), so spatially ordered inputs (rasters,
// paths) run best; results equal ocl_gb300_drop's.
// ---------------------------------------------------------------------------
struct NoAllocScratch {
    uint32_t perm[OCL_GB300_NOALLOC_MAX_POINTS];
    uint32_t cand[OCL_GB300_NOALLOC_MAX_POINTS * CAND_K_NOALLOC];
    float cand_hi[OCL_GB300_NOALLOC_MAX_POINTS * CAND_K_NOALLOC];
    float cand_lo[OCL_GB300_NOALLOC_MAX_POINTS * CAND_K_NOALLOC];
    uint32_t list[OCL_GB300_NOALLOC_MAX_POINTS];
    uint32_t list2[OCL_GB300_NOALLOC_MAX_POINTS];
    uint32_t sparse[OCL_GB300_NOALLOC_MAX_POINTS / 32 + 1];
    float blo[OCL_GB300_NOALLOC_MAX_POINTS];
    uint16_t ncand[OCL_GB300_NOALLOC_MAX_POINTS];
    unsigned long long counters[C_NCOUNTERS + 1];
};
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

__global__ void k_noalloc_identity(uint32_t* perm, int M) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < M) perm[i] = (uint32_t)i;
}

// Device address of the scratch array, looked up once per device with that
// device current (the host-side name is only a stand-in for the symbol).
// The cache is keyed by the CUDA context, so a context made after a device
// reset (which reloads the module) gets its own lookup.
static int noalloc_scratch(NoAllocScratch** out) {
    static std::mutex mu;
    static std::map<uint64_t, NoAllocScratch*> addr;
    const uint64_t key = context_key();
    if (!key) return OCL_GB300_DEVICE_ERROR;
    std::lock_guard<std::mutex> lk(mu);
    NoAllocScratch*& a = addr[key];
    if (!a) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error(std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e));
            return OCL_GB300_DEVICE_ERROR;
        }
        a = static_cast<NoAllocScratch*>(p);
    }
    *out = a;
    return OCL_GB300_OK;
}

int drop_run_noalloc(Mesh& m, const CutterP& cp, const double* d_cl, uint64_t M, double* d_z, double* d_cc,
                     int32_t* d_type, cudaStream_t stream) {
    if (M > (uint64_t)OCL_GB300_NOALLOC_MAX_POINTS) {
        set_error("ocl_gb300_drop_device_noalloc: " + std::to_string(M) + " points exceed the maximum of " +
                  std::to_string(OCL_GB300_NOALLOC_MAX_POINTS));
        return OCL_GB300_BAD_ARG;
    }
    if (M == 0) return OCL_GB300_OK;
    NoAllocScratch* sc = nullptr;
    int st = noalloc_scratch(&sc);
    if (st) return st;
    DropCtx h;
    init_drop_ctx(m, cp, h);
    const bool composite = h.composite_screen;
    h.cl = d_cl;  // caller's order
    h.perm = sc->perm;
    h.M = (int)M;
    h.out_z = d_z;
    h.out_cc = d_cc;
    h.out_type = d_type;
    h.cand = sc->cand;
    h.cand_hi = sc->cand_hi;
    h.cand_lo = sc->cand_lo;
    h.cand_cap = CAND_K_NOALLOC;
    h.ncand = sc->ncand;
    h.blo = sc->blo;
    h.sparse_list = sc->sparse;
    h.sparse_n = sc->counters + C_SPARSE;
    h.counters = sc->counters;
    // the array keeps the previous call's contents: clear what must start at zero
    CK(cudaMemsetAsync(sc->counters, 0, sizeof(sc->counters), stream));
    const int TB = 256;
    const unsigned nb = (unsigned)((M + TB - 1) / TB);
    k_noalloc_identity<<<nb, TB, 0, stream>>>(sc->perm, (int)M);
    const unsigned warps = (unsigned)((M + 31) / 32);
    if (m.n == 0) {
        CK(cudaMemsetAsync(sc->ncand, 0, M * sizeof(uint16_t), stream));
        CK(cudaMemsetAsync(sc->blo, 0xFF, M * sizeof(float), stream));
        k_drop_refine<false><<<(unsigned)((M + 127) / 128), 128, 0, stream>>>(h);
    } else {
        const unsigned sblocks = (warps + SCREEN_WARPS - 1) / SCREEN_WARPS;
        launch_screen(h, cp, sblocks, stream);
        k_drop_refine<false><<<(unsigned)((M + 127) / 128), 128, 0, stream>>>(h);
        k_collect_overflow<<<nb, TB, 0, stream>>>(sc->ncand, (int)M, sc->list, sc->counters + C_FALLBACK);
        st = launch_exact(h, composite, sc->list, sc->counters + C_FALLBACK, sc->list2, sc->counters + C_PLAIN,
                          (unsigned)std::min<uint64_t>(M, 152u * 3u), stream, ExactGlobal{});
        if (st) return st;
        const unsigned fb_blocks = std::min<unsigned>((warps + 3) / 4, 152u * 16u);
        k_drop_kd<true><<<fb_blocks, 128, 0, stream>>>(h, sc->list2, sc->counters + C_PLAIN);
    }
    CK(cudaGetLastError());
    return OCL_GB300_OK;
}

}  // namespace oclg
