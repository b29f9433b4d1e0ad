// diag.cu -- introspection entry points used by the parity tests.
//
//   ocl_gb300_mesh_kd_order / _kd_rank   the KD visit orders and ranks the
//       device holds (the tie-break of every fold), read back for comparison
//       with the reference's KDTree (src/common/kdtree.hpp:141-210, 273-304);
//   ocl_gb300_overlap_sets               the exact overlap set S(cl) the grid
//       index yields per CL point: every triangle of the cells under the
//       cutter's reach rectangle (all levels, the screen's rectangle
//       arithmetic) that MillingCutter::overlaps accepts
//       (src/cutters/millingcutter.cpp:422-433);
//   ocl_gb300_certificate_check          every exact-overlap pair's FP64
//       contacts (whole triangle from the start height, and each facet,
//       vertex and edge on its own) against the FP32 bounds the screen, the
//       refinement's part skips and the entry culls certify for it.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "drop.cuh"
#include "drop_util.cuh"
#include "geom64.cuh"
#include "mesh.cuh"
#include "util.cuh"

namespace oclg {

// ---------------------------------------------------------------------------
// KD orders and ranks
// ---------------------------------------------------------------------------
int mesh_kd_order(Mesh& m, int dims, int64_t* order) {
    if (dims < 0 || dims > 2) {
        set_error("dims must be 0 (XY), 1 (YZ) or 2 (XZ)");
        return OCL_GB300_BAD_ARG;
    }
    if (m.n == 0) return OCL_GB300_OK;
    const PushIndex* pi = &m.drop_kd;
    if (dims > 0) {
        const int dir = dims == 1 ? OCL_GB300_XFIBER : OCL_GB300_YFIBER;
        int st = ensure_push_index(m, dir);
        if (st) return st;
        pi = &m.push[dir];
    }
    std::vector<int32_t> dev(m.n);
    CK(cudaMemcpy(dev.data(), pi->d_order, m.n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    for (uint64_t k = 0; k < m.n; ++k) order[k] = m.dev_to_ins[dev[k]];
    return OCL_GB300_OK;
}

int mesh_kd_rank(Mesh& m, int64_t* rank) {
    if (m.n == 0) return OCL_GB300_OK;
    std::vector<Tri32> t(m.n);
    CK(cudaMemcpy(t.data(), m.d_t32, m.n * sizeof(Tri32), cudaMemcpyDeviceToHost));
    for (uint64_t d = 0; d < m.n; ++d) rank[m.dev_to_ins[d]] = t[d].kd_rank;
    return OCL_GB300_OK;
}

// ---------------------------------------------------------------------------
// Exact overlap sets through the grid: one warp per CL point walks the cells
// of its reach rectangle on every level (warp_rect, as the screen and the
// exact kernel do) and tests every entry with the FP64 overlap predicate.
// FILL = false counts, FILL = true writes device ids at offsets.
// ---------------------------------------------------------------------------
template <bool FILL>
__global__ void __launch_bounds__(128) k_overlap_sets(const __grid_constant__ DropCtx ctx, double radius,
                                                      const double* __restrict__ cl, int M,
                                                      unsigned long long* __restrict__ counts,
                                                      const unsigned long long* __restrict__ offsets,
                                                      int32_t* __restrict__ ids) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= M) return;
    const double x = cl[3 * warp], y = cl[3 * warp + 1];
    const GridP& g = ctx.g;
    const double reach = radius + 1e-9 * (1.0 + radius);
    unsigned long long n = 0, pos = FILL ? offsets[warp] : 0;
    for (int L = g.nlev - 1; L >= 0; --L) {
        int c0, c1, r0, r1;
        if (!warp_rect(g, L, x, x, y, y, reach, c0, c1, r0, r1)) continue;
        const Cell* cells = ctx.cells + g.cell_off[L];
        for (int r = r0; r <= r1; ++r)
            for (int c = c0; c <= c1; ++c) {
                const Cell cell = cells[r * g.ncol[L] + c];
                for (uint32_t j0 = 0; j0 < cell.count; j0 += 32) {
                    const uint32_t j = j0 + lane;
                    bool hit = false;
                    int32_t tri = 0;
                    if (j < cell.count) {
                        tri = ctx.entries[cell.start + j].tri;
                        hit = overlaps64(radius, x, y, ctx.t64[tri]);
                    }
                    const unsigned m = __ballot_sync(0xffffffffu, hit);
                    if (FILL && hit) ids[pos + n + __popc(m & ((1u << lane) - 1u))] = tri;
                    n += __popc(m);
                }
            }
    }
    if (!FILL && lane == 0) counts[warp] = n;
}

int overlap_sets(Mesh& m, double radius, const double* cl, uint64_t M, uint64_t* offsets, int32_t* ids,
                 uint64_t cap) {
    if (!(radius >= 0.0) || !std::isfinite(radius)) {
        set_error("radius must be finite and >= 0");
        return OCL_GB300_BAD_ARG;
    }
    offsets[0] = 0;
    if (M == 0) return OCL_GB300_OK;
    if (M >= (1ull << 31)) {
        set_error("too many CL points");
        return OCL_GB300_BAD_ARG;
    }
    if (m.n == 0) {
        for (uint64_t i = 0; i <= M; ++i) offsets[i] = 0;
        return OCL_GB300_OK;
    }
    CutterP cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.kind = OCL_CUTTER_CYL;
    cp.radius = radius;
    cp.b.kind = OCL_CUTTER_CYL;
    cp.b.radius = radius;
    DropCtx h;
    init_drop_ctx(m, cp, h);
    DevBuf<double> dcl(3 * M);
    DevBuf<unsigned long long> dcnt(M), doff(M);
    if (!dcl.ok() || !dcnt.ok() || !doff.ok()) return OCL_GB300_OOM;
    CK(cudaMemcpy(dcl.p, cl, 3 * M * sizeof(double), cudaMemcpyHostToDevice));
    const unsigned blocks = (unsigned)((M * 32 + 127) / 128);
    k_overlap_sets<false><<<blocks, 128>>>(h, radius, dcl.p, (int)M, dcnt.p, nullptr, nullptr);
    CK(cudaGetLastError());
    std::vector<unsigned long long> cnt(M), off(M);
    CK(cudaMemcpy(cnt.data(), dcnt.p, M * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    unsigned long long total = 0;
    for (uint64_t i = 0; i < M; ++i) {
        off[i] = total;
        offsets[i] = total;
        total += cnt[i];
    }
    offsets[M] = total;
    if (total > cap) {
        set_error("overlap sets: " + std::to_string(total) + " ids, output holds " + std::to_string(cap));
        return OCL_GB300_CAPACITY;
    }
    DevBuf<int32_t> dids(std::max<unsigned long long>(total, 1));
    if (!dids.ok()) return OCL_GB300_OOM;
    CK(cudaMemcpy(doff.p, off.data(), M * sizeof(unsigned long long), cudaMemcpyHostToDevice));
    k_overlap_sets<true><<<blocks, 128>>>(h, radius, dcl.p, (int)M, nullptr, doff.p, dids.p);
    CK(cudaGetLastError());
    if (total) CK(cudaMemcpy(ids, dids.p, total * sizeof(int32_t), cudaMemcpyDeviceToHost));
    // device ids -> insertion indices, ascending per point
    for (uint64_t i = 0; i < M; ++i) {
        int32_t* b = ids + offsets[i];
        int32_t* e = ids + offsets[i + 1];
        for (int32_t* p = b; p != e; ++p) *p = m.dev_to_ins[*p];
        std::sort(b, e);
    }
    return OCL_GB300_OK;
}

// ---------------------------------------------------------------------------
// Certificate check
// ---------------------------------------------------------------------------
enum CertCounter {
    K_PAIRS = 0,
    K_LIFTED,
    K_TRI_HI,         // FP64 fold from the start height above the screen's hi
    K_TRI_HI_UNSAFE,  // ... by more than the guard
    K_TRI_LO,         // FP64 fold below the screen's certified lo
    K_PART_HI,        // a part's FP64 contact above the bound its skip uses
    K_PART_HI_UNSAFE,
    K_ENTRY_UB,       // FP64 contact above an entry cull's bound
    K_ENTRY_UB_UNSAFE,
    K_ALT_HI,         // bull: the same checks with screen_triangle's interval
    K_NCOUNT,
    K_MAX_TRI = K_NCOUNT,  // largest positive excess (double bits), per kind
    K_MAX_PART,
    K_MAX_ENTRY,
    K_MAX_LO,
    K_TOTAL
};

__device__ __forceinline__ void excess(unsigned long long* c, int k, int kmax, double ex, double gd, int k_unsafe) {
    if (!(ex > 0.0)) return;
    atomicAdd(&c[k], 1ull);
    if (k_unsafe >= 0 && ex > gd) atomicAdd(&c[k_unsafe], 1ull);
    atomicMax(&c[kmax], (unsigned long long)__double_as_longlong(ex));
}

// One warp per CL point, lanes over the exact-overlap triangles of its cells.
__global__ void __launch_bounds__(128) k_certificate(const __grid_constant__ DropCtx ctx, const double* __restrict__ cl,
                                                     int M, unsigned long long* __restrict__ cnt) {
    __shared__ float s_hlb[HLB_N];
    for (int k = threadIdx.x; k < HLB_N; k += blockDim.x) s_hlb[k] = ctx.hlb[k];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= M) return;
    const GridP& g = ctx.g;
    const CutterP& cp = ctx.cp;
    const double x = cl[3 * warp], y = cl[3 * warp + 1], z0 = cl[3 * warp + 2];
    const float cx = (float)(x - g.ox), cy = (float)(y - g.oy);
    const float z0l = __double2float_rd(z0 - g.oz);
    const float E = ctx.E, gd = ctx.guard, R = ctx.prof.R, inv_step = (float)HLB_N / R;
    const double reach = cp.radius + 1e-9 * (1.0 + cp.radius);
    const bool comp = ctx.composite_screen;
    const int kind = comp ? OCL_CUTTER_COMPOSITE : (cp.kind == OCL_CUTTER_CONE ? OCL_CUTTER_CONE : cp.b.kind);
    int capped = 0;
    for (int L = g.nlev - 1; L >= 0; --L) {
        int c0, c1, r0, r1;
        if (!warp_rect(g, L, x, x, y, y, reach, c0, c1, r0, r1)) continue;
        const Cell* cells = ctx.cells + g.cell_off[L];
        for (int r = r0; r <= r1; ++r)
            for (int c = c0; c <= c1; ++c) {
                const Cell cell = cells[r * g.ncol[L] + c];
                for (uint32_t j0 = 0; j0 < cell.count; j0 += 32) {
                    const uint32_t j = j0 + lane;
                    bool have = false;
                    Entry e{};
                    if (j < cell.count) {
                        e = ctx.entries[cell.start + j];
                        have = overlaps64(cp.radius, x, y, ctx.t64[e.tri]);
                    }
                    if (!__any_sync(0xffffffffu, have)) continue;
                    const uint32_t tri = have ? (uint32_t)e.tri : 0u;
                    const Tri32 t3 = ctx.t32[tri];
                    const float wx = cx - t3.v0[0], wy = cy - t3.v0[1];
                    Prof32 prof = ctx.prof;
                    prof.kind = kind;
                    float qt = 3.0e38f, qth = NEG_INF32;
                    Iv v, valt = iv_none();
                    if (kind == OCL_CUTTER_BULL) {
                        v = screen_bull_warp(prof, ctx.t32, tri, t3, wx, wy, E, have);  // warp-collective
                        if (have) valt = screen_triangle(prof, t3, wx, wy, E, z0l - t3.v0[2], qt, qth);
                    } else if (!have) {
                        continue;
                    } else if (comp) {
                        v = screen_composite(ctx.comp, t3, wx, wy, E, z0l - t3.v0[2], qt, qth);
                    } else {
                        v = screen_triangle(prof, t3, wx, wy, E, z0l - t3.v0[2], qt, qth);
                    }
                    if (!have) continue;
                    const Tri64& t = ctx.t64[tri];
                    atomicAdd(&cnt[K_PAIRS], 1ull);
                    // whole triangle from the start height (MillingCutter::dropCutter)
                    CL64 f{x, y, z0, d3(0, 0, 0), OCL_CC_NONE};
                    drop_triangle64(cp, f, t, t3.flags, &capped);
                    const double rl = f.z - g.oz;  // local frame
                    const bool lifted = f.z > z0;
                    // the screen's interval in the local frame (as scan_cells forms it)
                    const float lo = v.lo > NEG_INF32 ? v.lo + t3.v0[2] - E : NEG_INF32;
                    const float hi = v.hi > NEG_INF32 ? fminf(v.hi + t3.v0[2] + E, e.maxz + gd) : NEG_INF32;
                    if (lifted) {
                        atomicAdd(&cnt[K_LIFTED], 1ull);
                        excess(cnt, K_TRI_HI, K_MAX_TRI, rl - (double)hi, gd, K_TRI_HI_UNSAFE);
                        if (kind == OCL_CUTTER_BULL) {
                            const float ha = valt.hi > NEG_INF32 ? valt.hi + t3.v0[2] + E : NEG_INF32;
                            if (rl > (double)ha) atomicAdd(&cnt[K_ALT_HI], 1ull);
                        }
                        // entry cull: bbox max z less the profile's lower bound at the bbox distance
                        const float ex = fmaxf(0.0f, fmaxf(e.minx - cx, cx - e.maxx));
                        const float ey = fmaxf(0.0f, fmaxf(e.miny - cy, cy - e.maxy));
                        const float de = sqrtf(ex * ex + ey * ey);
                        const float ub = de <= R + gd ? e.maxz - hlb_at(s_hlb, de - gd, inv_step) : NEG_INF32;
                        excess(cnt, K_ENTRY_UB, K_MAX_ENTRY, rl - (double)ub, gd, K_ENTRY_UB_UNSAFE);
                    }
                    if (lo > NEG_INF32) excess(cnt, K_TRI_LO, K_MAX_LO, (double)lo - rl, 0.0, -1);
                    // parts on their own, against the bounds the refinement's skips use
                    const double vz = (double)t3.v0[2] + g.oz;  // part contacts relative to v0
                    const float px[3] = {0.0f, t3.e1[0], t3.e2[0]};
                    const float py[3] = {0.0f, t3.e1[1], t3.e2[1]};
                    const float pz[3] = {0.0f, t3.e1[2], t3.e2[2]};
                    if (!comp) {
                        const BasicP& b = cp.b;
                        for (int k = 0; k < 3; ++k) {
                            const D3 p = tri_p(t, k);
                            const double q = xynorm(d3(x, y, 0.0) - p);
                            if (!(q <= b.radius)) continue;
                            const double cz = p.z - height_basic(b, q) - vz;
                            const float U = vertex32(ctx.prof, px[k] - wx, py[k] - wy, pz[k], E).hi + E;
                            excess(cnt, K_PART_HI, K_MAX_PART, cz - (double)U, gd, K_PART_HI_UNSAFE);
                        }
                        if (kind != OCL_CUTTER_CONE) {
                            CL64 fc{x, y, -1.0e300, d3(0, 0, 0), OCL_CC_NONE};
                            if (facet_drop_base(b, fc, t, t3.flags)) {
                                Prof32 pb = ctx.prof;
                                pb.kind = kind;
                                const float U = facet32(pb, t3, wx, wy, E, E * 4.0f * t3.bary_scale + 1e-6f).hi + E;
                                excess(cnt, K_PART_HI, K_MAX_PART, fc.z - vz - (double)U, gd, K_PART_HI_UNSAFE);
                            }
                        }
                        for (int ed = 0; ed < 3; ++ed) {
                            if (t3.flags & (TF_EDGE0_SKIP << ed)) continue;
                            const int k = (ed + 1) % 3;
                            double clz;
                            D3 cc;
                            if (!edge_contact64(b, x, y, tri_p(t, ed), tri_p(t, k), clz, cc, &capped)) continue;
                            const bool horiz = (t3.flags & (TF_EDGE0_HORIZ << ed)) != 0;
                            float U = edge32(ctx.prof, px[ed], py[ed], pz[ed], px[k], py[k], pz[k], wx, wy, E, horiz).hi + E;
                            excess(cnt, K_PART_HI, K_MAX_PART, clz - vz - (double)U, gd, K_PART_HI_UNSAFE);
                            if (kind == OCL_CUTTER_BULL && !horiz) {
                                // the bull plan's bound (k_bull_plan, fold_bull)
                                Prof32 pb = ctx.prof;
                                pb.kind = OCL_CUTTER_BULL;
                                float ax, ay, az, bx, by, bz;
                                tri_edge32(t3, ed, ax, ay, az, bx, by, bz);
                                BullEdge32 be;
                                float hb = NEG_INF32;
                                if (bull_edge_setup32(pb, ax, ay, az, bx, by, bz, wx, wy, E, be) && bull_edge_open32(pb, be))
                                    hb = bull_edge_solve32(pb, be, E).hi;
                                U = hb + E;
                                excess(cnt, K_PART_HI, K_MAX_PART, clz - vz - (double)U, gd, K_PART_HI_UNSAFE);
                            }
                        }
                    } else {
                        const Comp32& cm = ctx.comp;
                        for (int k = 0; k < 3; ++k) {
                            const D3 p = tri_p(t, k);
                            const double q = xynorm(d3(x, y, 0.0) - p);
                            if (!(q <= cp.radius)) continue;
                            const double cz = p.z - height_any(cp, q) - vz;
                            const float dx = px[k] - wx, dy = py[k] - wy;
                            const float qlo = sqrtf(dx * dx + dy * dy) - E;
                            // fold_one leaves the vertex out when qlo > R or its bound + 2E lies below
                            const float U = qlo > cm.R ? NEG_INF32 : pz[k] - hcomp32(cm, fmaxf(qlo, 0.0f)) + E + 2.0f * E;
                            excess(cnt, K_PART_HI, K_MAX_PART, cz - (double)U, gd, K_PART_HI_UNSAFE);
                        }
                        for (int n = 0; n < cp.nsub; ++n) {
                            const double lo_w = (n == 0) ? -1E-6 : cp.radiusvec[n - 1] - 1E-6;
                            const double hi_w = cp.radiusvec[n] + 1e-6;
                            // facet of sub-cutter n with its CC in the window
                            CL64 fs{x, y, -1.0e300, d3(0, 0, 0), OCL_CC_NONE};
                            if (facet_drop_sub(cp.sub[n], fs, t, t3.flags) && fs.type != OCL_CC_NONE) {
                                const double dd = xynorm(d3(fs.x, fs.y, 0.0) - d3(fs.cc.x, fs.cc.y, 0.0));
                                if (!(dd < lo_w) && !(dd > hi_w)) {
                                    const float U = comp_facet_hi32(cm, t3, n, wx, wy, E) + 2.0f * E;
                                    excess(cnt, K_PART_HI, K_MAX_PART, fs.z - cp.zoffset[n] - vz - (double)U, gd,
                                           K_PART_HI_UNSAFE);
                                }
                            }
                            const float zo = cm.zoff[n];
                            const float wlo = (n == 0 ? 0.0f : cm.rlim[n - 1]) - 1e-6f, whi = cm.rlim[n] + 1e-6f;
                            for (int ed = 0; ed < 3; ++ed) {
                                if (t3.flags & (TF_EDGE0_SKIP << ed)) continue;
                                const int k = (ed + 1) % 3;
                                double clz;
                                D3 cc;
                                if (!edge_contact64(cp.sub[n], x, y, tri_p(t, ed), tri_p(t, k), clz, cc, &capped))
                                    continue;
                                const bool horiz = (t3.flags & (TF_EDGE0_HORIZ << ed)) != 0;
                                const double cz = clz - cp.zoffset[n] - vz;
                                Iv ve = edge32(cm.sub[n], px[ed], py[ed], pz[ed], px[k], py[k], pz[k], wx, wy, E, horiz);
                                excess(cnt, K_PART_HI, K_MAX_PART, cz - (double)(ve.hi - zo + 2.0f * E), gd,
                                       K_PART_HI_UNSAFE);
                                const double dd = xynorm(d3(x, y, 0.0) - d3(cc.x, cc.y, 0.0));
                                if (!(dd < lo_w) && !(dd > hi_w)) {
                                    ve = edge32(cm.sub[n], px[ed], py[ed], pz[ed], px[k], py[k], pz[k], wx, wy, E, horiz,
                                                wlo, whi);
                                    excess(cnt, K_PART_HI, K_MAX_PART, cz - (double)(ve.hi - zo + 2.0f * E), gd,
                                           K_PART_HI_UNSAFE);
                                }
                            }
                        }
                    }
                }
            }
    }
    (void)capped;
}

int certificate_check(Mesh& m, const CutterP& cp, const double* cl, uint64_t M, ocl_gb300_cert* out) {
    std::memset(out, 0, sizeof(*out));
    if (M == 0 || m.n == 0) return OCL_GB300_OK;
    if (M >= (1ull << 31)) {
        set_error("too many CL points");
        return OCL_GB300_BAD_ARG;
    }
    DropCtx h;
    init_drop_ctx(m, cp, h);
    DevBuf<double> dcl(3 * M);
    DevBuf<unsigned long long> dc(K_TOTAL);
    if (!dcl.ok() || !dc.ok()) return OCL_GB300_OOM;
    CK(cudaMemcpy(dcl.p, cl, 3 * M * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemset(dc.p, 0, K_TOTAL * sizeof(unsigned long long)));
    k_certificate<<<(unsigned)((M * 32 + 127) / 128), 128>>>(h, dcl.p, (int)M, dc.p);
    CK(cudaGetLastError());
    unsigned long long c[K_TOTAL];
    CK(cudaMemcpy(c, dc.p, sizeof(c), cudaMemcpyDeviceToHost));
    auto dbl = [](unsigned long long b) {
        double d;
        std::memcpy(&d, &b, sizeof(d));
        return d;
    };
    out->pairs = c[K_PAIRS];
    out->lifted = c[K_LIFTED];
    out->tri_hi_exceeded = c[K_TRI_HI];
    out->tri_hi_unsafe = c[K_TRI_HI_UNSAFE];
    out->tri_lo_exceeded = c[K_TRI_LO];
    out->part_hi_exceeded = c[K_PART_HI];
    out->part_hi_unsafe = c[K_PART_HI_UNSAFE];
    out->entry_ub_exceeded = c[K_ENTRY_UB];
    out->entry_ub_unsafe = c[K_ENTRY_UB_UNSAFE];
    out->alt_hi_exceeded = c[K_ALT_HI];
    out->max_tri_excess = dbl(c[K_MAX_TRI]);
    out->max_part_excess = dbl(c[K_MAX_PART]);
    out->max_entry_excess = dbl(c[K_MAX_ENTRY]);
    out->max_lo_excess = dbl(c[K_MAX_LO]);
    out->error_budget = h.E;
    out->guard = h.guard;
    return OCL_GB300_OK;
}

}  // namespace oclg
