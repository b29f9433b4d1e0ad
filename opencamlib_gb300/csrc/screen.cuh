// screen.cuh -- the FP32 screen kernels (templates; each cutter kind is
// instantiated in its own translation unit, screen_*.cu).
#pragma once
#include "drop.cuh"
#include "drop_util.cuh"
#include "geom32.cuh"

namespace oclg {

// ---------------------------------------------------------------------------
// FP32 screen
// ---------------------------------------------------------------------------
constexpr int SCREEN_WARPS = 4;
constexpr int NBRANCH = 4;  // branching triangles tracked per CL point
// resident screen blocks per SM the register allocation aims at (measured:
// more warps hide the FP32 dependency chains until spills start to cost;
// the cone and composite kernels, with their out-of-line cell scan, run
// best with the registers of four)
constexpr int screen_min_blocks(int kind, int ck) {
    (void)ck;
    return kind != 0 ? 4 : 6;
}

enum ScanPhase { PH_SINGLE = 0, PH_RESOLVE = 1, PH_COLLECT = 2 };

// packed make-up of a three-part composite (sub-cutter kinds), used as the
// kernel's CK for KIND 2
constexpr int comp_sig(int a, int b, int c) { return a | (b << 4) | (c << 8) | (3 << 16); }
constexpr int SIG_BALLCONE = comp_sig(OCL_CUTTER_BALL, OCL_CUTTER_CONE, OCL_CUTTER_CYL);
constexpr int SIG_BULLCONE = comp_sig(OCL_CUTTER_BULL, OCL_CUTTER_CONE, OCL_CUTTER_CYL);
constexpr int SIG_CYLCONE = comp_sig(OCL_CUTTER_CYL, OCL_CUTTER_CONE, OCL_CUTTER_CYL);
constexpr int SIG_CONECONE = comp_sig(OCL_CUTTER_CONE, OCL_CUTTER_CONE, OCL_CUTTER_CYL);

// Launchers, one translation unit each (screen_basic.cu, screen_comp_*.cu).
// The composite ones return false when the make-up is not theirs.
// The *_sparse launchers run the kernels for the warps the dense kernels
// handed over (their grid of `blocks` strides over them); own units too.
void screen_launch_basic(const DropCtx& h, int kind, unsigned blocks, cudaStream_t stream);
bool screen_launch_comp_a(const DropCtx& h, int sig, unsigned blocks, cudaStream_t stream);
bool screen_launch_comp_b(const DropCtx& h, int sig, unsigned blocks, cudaStream_t stream);
void screen_launch_comp_any(const DropCtx& h, unsigned blocks, cudaStream_t stream);
// stage 0: the seeding kernel (before the dense one; `blocks` covers the
// points), stage 1: the sparse kernel (after it)
void screen_launch_basic_sparse(const DropCtx& h, int kind, unsigned blocks, cudaStream_t stream, int stage);
bool screen_launch_comp_a_sparse(const DropCtx& h, int sig, unsigned blocks, cudaStream_t stream, int stage);
bool screen_launch_comp_b_sparse(const DropCtx& h, int sig, unsigned blocks, cudaStream_t stream, int stage);
void screen_launch_comp_any_sparse(const DropCtx& h, unsigned blocks, cudaStream_t stream, int stage);

// Batch launchers: *_dense_b in the dense units, *_b (stage 0 seeding,
// stage 2 sparse screen) in the sparse units; `blocks` is the persistent
// grid.  The composite ones return false when the make-up is not theirs.
void screen_launch_basic_dense_b(const BatchView& bv, int kind, unsigned blocks, cudaStream_t stream);
void screen_launch_basic_b(const BatchView& bv, int kind, unsigned blocks, cudaStream_t stream, int stage);
bool screen_launch_comp_a_dense_b(const BatchView& bv, int sig, unsigned blocks, cudaStream_t stream);
bool screen_launch_comp_a_b(const BatchView& bv, int sig, unsigned blocks, cudaStream_t stream, int stage);
bool screen_launch_comp_b_dense_b(const BatchView& bv, int sig, unsigned blocks, cudaStream_t stream);
bool screen_launch_comp_b_b(const BatchView& bv, int sig, unsigned blocks, cudaStream_t stream, int stage);
void screen_launch_comp_any_dense_b(const BatchView& bv, unsigned blocks, cudaStream_t stream);
void screen_launch_comp_any_b(const BatchView& bv, unsigned blocks, cudaStream_t stream, int stage);

// Float <-> int keys whose integer order is the float order (for atomicMax /
// atomicMin on floats held in shared memory).
__device__ __forceinline__ int f2o(float f) {
    const int b = __float_as_int(f);
    return b >= 0 ? b : b ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float o2f(int o) { return __int_as_float(o >= 0 ? o : o ^ 0x7FFFFFFF); }
__device__ __forceinline__ unsigned f2u(float f) {
    const unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float u2f(unsigned u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u); }

// Branching triangles of one warp's points ([slot][point]): triangles whose
// effect on the running height Z has a branch point in [qlo, qhi] (cone tip
// and rim, composite facet short-circuits).  Wp: the highest certified lower
// bound among triangles visited before it (lower KD rank), packed with that
// triangle's id; H: the highest upper bound among them (or the start height).
//   W > qhi: every fold reaches the triangle with Z above all branch points;
//   H < qlo: every fold reaches it with Z below all branch points;
// either way its branch is decided without the triangles below the bound.
struct BranchTab {
    uint32_t tri[NBRANCH][32];
    uint32_t rank[NBRANCH][32];
    float qlo[NBRANCH][32];
    float qhi[NBRANCH][32];
    float hi[NBRANCH][32];
    unsigned long long Wp[NBRANCH][32];
    int H[NBRANCH][32];  // ordered key of a float
};

// Per-warp state of the 32 points, shared by the lanes that screen
// (point, triangle) pairs on their behalf.
struct WarpPoints {
    float cx[32], cy[32], z0l[32], thr[32];
    int blo[32];       // ordered key of the certified lower bound
    int qx[32];        // ordered key: lowest threshold of untracked branching triangles
    int chain_thr[32]; // ordered key: lowest branch threshold among chained triangles
    int nc[32];        // candidates in the point's list
    int nb[32];        // tracked branching triangles (may run past NBRANCH)
    unsigned pending[32];
    unsigned resolved[32];
    int flags[32];     // PF_*
    unsigned msk[32];  // entries of the current chunk the point wants screened
    int pre[32];       // exclusive prefix of the masks' popcounts
};
constexpr int PF_OVERFLOW = 1, PF_CHAIN = 2;

constexpr int ROWS_SORTED = 64;  // rows of a level the single pass visits best first

struct ScanShared {
    float hlb[HLB_N];
    int rkey[SCREEN_WARPS][ROWS_SORTED];       // ordered key: a row's highest upper bound for the warp
    uint8_t rord[SCREEN_WARPS][ROWS_SORTED];   // rows (from r0) in descending key order
    Cell cel[SCREEN_WARPS][32];  // a row's cells, 32 at a time
    Entry ent[SCREEN_WARPS][32];
    BranchTab br[SCREEN_WARPS];
    WarpPoints pt[SCREEN_WARPS];
};

struct LaneState {
    float blo;          // certified lower bound of the final height
    float qx;           // lowest branch threshold of relevant triangles not tracked
    float thr;          // PH_RESOLVE: cut; PH_COLLECT: collection threshold
    float zu;           // start height rounded up (local frame)
    int nc;
    int nb;             // tracked branching triangles
    unsigned resolved;  // bit j: branch of tracked triangle j is decided
    unsigned pending;   // bit j: PH_RESOLVE still looks for a witness of j
    bool overflow;
    bool chain;         // a collected triangle's branch depends on uncollected ones
    float chain_thr;    // lowest branch threshold among chained triangles
    unsigned long long screened;
};

__device__ __forceinline__ bool is_resolved(const BranchTab& b, int nb, unsigned resolved, int p, uint32_t tri) {
    for (int j = 0; j < nb; ++j)
        if (((resolved >> j) & 1u) && b.tri[j][p] == tri) return true;
    return false;
}

// Lazy prune of point p's list against keep (its owner lane, between chunks).
__device__ __forceinline__ int prune_list(const DropCtx& ctx, uint32_t self, int nc, float keep) {
    const int cap = ctx.cand_cap;
    uint32_t* lt = ctx.cand + (size_t)self * cap;
    float* lh = ctx.cand_hi + (size_t)self * cap;
    float* ll = ctx.cand_lo + (size_t)self * cap;
    int w = 0;
    for (int q = 0; q < min(nc, cap); ++q) {
        const float hq = lh[q];
        if (hq >= keep) {
            lt[w] = lt[q];
            lh[w] = hq;
            ll[w] = ll[q];
            ++w;
        }
    }
    return w;
}

// One pass over the cells under the warp's footprint (coarse levels first;
// rows best first or centre-out, below).  Per chunk of 32 grid entries every lane marks the
// entries its own point wants screened; the marked (point, triangle) pairs are
// then spread over all 32 lanes, and each lane applies its results to the
// pair's point through shared memory.
//   PH_SINGLE   raise blo; collect triangles whose upper bound reaches the
//               running blo; KIND 1/2: track branching ones;
//   PH_RESOLVE  for the pending tracked triangles, the best witness and the
//               highest upper bound among earlier-ranked triangles; a point
//               stops once every pending triangle has a witness;
//   PH_COLLECT  collect everything reaching thr, noting branch thresholds
//               below it that are not decided (chains).
// KIND: 0 cyl/ball/bull, 1 cone, 2 composite; CK: the cutter kind for KIND
// 0/1 (a compile-time constant, so each kernel carries one contact model);
// SPARSE: the kernel for warps whose points are spread out.
template <int KIND, int CK, bool SPARSE>
__device__ __forceinline__ void scan_cells(const DropCtx& ctx, ScanShared& sh, int phase, LaneState& ls, bool active,
                                           uint32_t base, double xmin, double xmax, double ymin, double ymax) {
    const int lane = threadIdx.x & 31;
    const int wl = threadIdx.x >> 5;
    BranchTab& br = sh.br[wl];
    WarpPoints& P = sh.pt[wl];
    const GridP& g = ctx.g;
    const float R = ctx.prof.R;
    const float gd = ctx.guard;
    const float Rg = R + gd;
    const float inv_step = (float)HLB_N / R;
    const double reach = ctx.cp.radius + 1e-9 * (1.0 + ctx.cp.radius);
    const int cap = ctx.cand_cap;
    Prof32 prof = ctx.prof;
    prof.kind = CK;
    // composites with a known make-up (CK = packed sub-cutter kinds): the
    // sub-cutter loop unrolls into one contact model per sub-cutter
    Comp32 comp = ctx.comp;
    if (KIND == 2 && CK >= 0) {
        comp.nsub = CK >> 16;
#pragma unroll
        for (int k = 0; k < OCL_GB300_MAX_SUB; ++k) comp.sub[k].kind = (CK >> (4 * k)) & 15;
    }
    // publish this lane's point state
    P.blo[lane] = f2o(ls.blo);
    P.qx[lane] = f2o(ls.qx);
    P.chain_thr[lane] = f2o(ls.chain_thr);
    P.thr[lane] = ls.thr;
    P.nc[lane] = ls.nc;
    P.nb[lane] = ls.nb;
    P.pending[lane] = ls.pending;
    P.resolved[lane] = ls.resolved;
    P.flags[lane] = (ls.overflow ? PF_OVERFLOW : 0) | (ls.chain ? PF_CHAIN : 0);
    const float cx = P.cx[lane], cy = P.cy[lane], z0l = P.z0l[lane];
    const float lthr = ls.thr;  // kept in a register across the scan
    // the active points' rectangle and lowest start height: an entry that
    // fails the cull against these fails it for every active point
    const float rx0 = warp_min(active ? cx : 3.0e38f), rx1 = warp_max(active ? cx : -3.0e38f);
    const float ry0 = warp_min(active ? cy : 3.0e38f), ry1 = warp_max(active ? cy : -3.0e38f);
    const float zmin = warp_min(active ? z0l : 3.0e38f);
    unsigned long long screened = 0;
    // a single point in this pass (the per-point scans of a scattered warp)
    int solo = -1;
    if (SPARSE) {
        const unsigned am = __ballot_sync(0xffffffffu, active);
        if (__popc(am) == 1) solo = __ffs(am) - 1;
    }
    __syncwarp();
    for (int L = g.nlev - 1; L >= 0; --L) {
        int c0, c1, r0, r1;
        if (!warp_rect(g, L, xmin, xmax, ymin, ymax, reach, c0, c1, r0, r1)) continue;
        const int rc = clampi((int)floor((0.5 * (ymin + ymax) - g.y0) * g.inv_cs[L]), r0, r1);
        const int cc = clampi((int)floor((0.5 * (xmin + xmax) - g.x0) * g.inv_cs[L]), c0, c1);
        const int nr = r1 - r0 + 1, ncl = c1 - c0 + 1;
        const Cell* cells = ctx.cells + g.cell_off[L];
        const int ncol = g.ncol[L];
        // the cylinder's, ball's and bull's single pass visits the rows in
        // descending order of their highest upper bound for the warp (a
        // cell's maxz less the profile's lower bound at its distance from the
        // points' rectangle), so the bounds rise early; once a row's bound
        // lies below every lane's threshold, so do the later rows' and the
        // level is done.  (The cone's bound falls off steeply with the
        // distance, so the rectangle's nearest distance misleads the order:
        // measured, it screened more pairs; it keeps the centre-out order.)
        const bool best_first = KIND == 0 && phase == PH_SINGLE && nr <= ROWS_SORTED;
        if (best_first) {
            for (int k = 0; k < nr; ++k) {
                float best = NEG_INF32;
                for (int c = c0 + lane; c <= c1; c += 32) {
                    const Cell cl = cells[(r0 + k) * ncol + c];
                    const float ex = fmaxf(0.0f, fmaxf(cl.minx - rx1, rx0 - cl.maxx));
                    const float ey = fmaxf(0.0f, fmaxf(cl.miny - ry1, ry0 - cl.maxy));
                    const float de = sqrtf(ex * ex + ey * ey);
                    if (cl.count > 0 && de <= Rg) best = fmaxf(best, cl.maxz - hlb_at(sh.hlb, de - gd, inv_step));
                }
                best = warp_max(best);
                if (lane == 0) sh.rkey[wl][k] = f2o(best);
            }
            __syncwarp();
            for (int k = lane; k < nr; k += 32) {
                const int key = sh.rkey[wl][k];
                int rank = 0;
                for (int j = 0; j < nr; ++j) {
                    const int kj = sh.rkey[wl][j];
                    rank += (kj > key || (kj == key && j < k)) ? 1 : 0;
                }
                sh.rord[wl][rank] = (uint8_t)k;
            }
            __syncwarp();
        }
    for (int kr = 0; kr < nr; ++kr) {
        const int r = best_first ? r0 + sh.rord[wl][kr] : centre_out(kr, rc, r0, r1);
        if (best_first) {
            const float wc = warp_min(active ? o2f(P.blo[lane]) : 3.0e38f);
            if (o2f(sh.rkey[wl][r - r0]) < wc - gd) break;
        }
        if (phase == PH_RESOLVE) {
            if (P.pending[lane] == 0) active = false;
            if (!__any_sync(0xffffffffu, active)) goto done;
        }
        for (int kc0 = 0; kc0 < ncl; kc0 += 32) {
            const int nck = min(32, ncl - kc0);
            __syncwarp();
            if (lane < nck) sh.cel[wl][lane] = cells[r * ncol + centre_out(kc0 + lane, cc, c0, c1)];
            __syncwarp();
            unsigned cmask = nck == 32 ? 0xffffffffu : ((1u << nck) - 1u);
            if (solo >= 0) {
                // one point: each lane culls one of the staged cells for it
                const float scut = __shfl_sync(0xffffffffu, (phase == PH_SINGLE) ? o2f(P.blo[lane]) : lthr, solo);
                const float sx = __shfl_sync(0xffffffffu, cx, solo), sy = __shfl_sync(0xffffffffu, cy, solo);
                bool keep = false;
                if (lane < nck) {
                    const Cell& cl = sh.cel[wl][lane];
                    const float ex = fmaxf(0.0f, fmaxf(cl.minx - sx, sx - cl.maxx));
                    const float ey = fmaxf(0.0f, fmaxf(cl.miny - sy, sy - cl.maxy));
                    const float de = sqrtf(ex * ex + ey * ey);
                    keep = cl.count > 0 && de <= Rg && cl.maxz - hlb_at(sh.hlb, de - gd, inv_step) >= scut - gd;
                }
                cmask = __ballot_sync(0xffffffffu, keep);
            } else {
                // one cull per staged cell against the whole warp (the points'
                // rectangle, the lowest threshold; hlb rises with the
                // distance): a cell it drops fails every lane's own test
                const float wc =
                    warp_min(active ? ((phase == PH_SINGLE) ? o2f(P.blo[lane]) : lthr) : 3.0e38f);
                bool keep = false;
                if (lane < nck) {
                    const Cell& cl = sh.cel[wl][lane];
                    const float ex = fmaxf(0.0f, fmaxf(cl.minx - rx1, rx0 - cl.maxx));
                    const float ey = fmaxf(0.0f, fmaxf(cl.miny - ry1, ry0 - cl.maxy));
                    const float de = sqrtf(ex * ex + ey * ey);
                    keep = cl.count > 0 && de <= Rg && cl.maxz - hlb_at(sh.hlb, de - gd, inv_step) >= wc - gd;
                }
                cmask = __ballot_sync(0xffffffffu, keep);
            }
        for (; cmask; cmask &= cmask - 1) {
            const int kk = __ffs(cmask) - 1;
            const Cell cell = sh.cel[wl][kk];
            if (cell.count == 0) continue;
            // the threshold below which a triangle is of no interest in this phase
            const float cut = (phase == PH_SINGLE) ? o2f(P.blo[lane]) : lthr;
            float dx = fmaxf(0.0f, fmaxf(cell.minx - cx, cx - cell.maxx));
            float dy = fmaxf(0.0f, fmaxf(cell.miny - cy, cy - cell.maxy));
            float d = sqrtf(dx * dx + dy * dy);
            bool pass = active && d <= Rg && cell.maxz - hlb_at(sh.hlb, d - gd, inv_step) >= cut - gd;
            if (!__any_sync(0xffffffffu, pass)) continue;
            for (uint32_t j0 = 0; j0 < cell.count; j0 += 32) {
                const int nj = min(32, (int)(cell.count - j0));
                __syncwarp();
                if (lane < nj) sh.ent[wl][lane] = ctx.entries[cell.start + j0 + lane];
                __syncwarp();
                // 1. the entries this lane's point wants screened: one cull
                // per entry against the whole warp (the points' rectangle,
                // the lowest threshold), then each lane's own cull of the
                // entries that pass it
                const float cut2 = (phase == PH_SINGLE) ? o2f(P.blo[lane]) : lthr;
                const float wcut = warp_min(pass ? cut2 : 3.0e38f);
                bool want = false;
                if (lane < nj) {
                    const Entry& e = sh.ent[wl][lane];
                    const float ex = fmaxf(0.0f, fmaxf(e.minx - rx1, rx0 - e.maxx));
                    const float ey = fmaxf(0.0f, fmaxf(e.miny - ry1, ry0 - e.maxy));
                    const float de = sqrtf(ex * ex + ey * ey);
                    const float ub = e.maxz - hlb_at(sh.hlb, de - gd, inv_step);
                    want = de <= Rg && ub >= wcut - gd && ub > zmin - gd;
                }
                const unsigned wmask = __ballot_sync(0xffffffffu, want);
                unsigned m = 0;
                if (pass) {
                    for (unsigned rest = wmask; rest; rest &= rest - 1) {
                        const int jj = __ffs(rest) - 1;
                        const Entry& e = sh.ent[wl][jj];
                        float ex = fmaxf(0.0f, fmaxf(e.minx - cx, cx - e.maxx));
                        float ey = fmaxf(0.0f, fmaxf(e.miny - cy, cy - e.maxy));
                        float de = sqrtf(ex * ex + ey * ey);
                        float ub = e.maxz - hlb_at(sh.hlb, de - gd, inv_step);
                        if (de <= Rg && ub >= cut2 - gd && ub > z0l - gd) m |= 1u << jj;
                    }
                }
                const int cnt = __popc(m);
                // 2. room in the point's list for what this chunk may add
                if (phase != PH_RESOLVE && cnt && P.nc[lane] + cnt > cap && !(P.flags[lane] & PF_OVERFLOW)) {
                    const float keep = (phase == PH_COLLECT) ? lthr : o2f(P.blo[lane]);
                    P.nc[lane] = prune_list(ctx, base + lane, P.nc[lane], keep - gd);
                }
                if (KIND != 0 && phase == PH_SINGLE && P.nb[lane] >= NBRANCH) {
                    // drop tracked triangles that can no longer reach blo
                    const float keep = o2f(P.blo[lane]) - gd;
                    int w = 0;
                    for (int j = 0; j < NBRANCH; ++j) {
                        if (br.hi[j][lane] < keep) continue;
                        br.tri[w][lane] = br.tri[j][lane];
                        br.rank[w][lane] = br.rank[j][lane];
                        br.qlo[w][lane] = br.qlo[j][lane];
                        br.qhi[w][lane] = br.qhi[j][lane];
                        br.hi[w][lane] = br.hi[j][lane];
                        ++w;
                    }
                    P.nb[lane] = w;
                }
                int incl = cnt;
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += v;
                }
                const int total = __shfl_sync(0xffffffffu, incl, 31);
                if (total == 0) continue;
                P.msk[lane] = m;
                P.pre[lane] = incl - cnt;
                __syncwarp();
                // 3. screen the marked pairs, 32 at a time (the bull's
                // screen is warp-collective: every lane takes part in every
                // round, holding a pair or not)
                constexpr bool WARP_SCREEN = KIND == 0 && CK == OCL_CUTTER_BULL;
                for (int k0 = WARP_SCREEN ? 0 : lane; k0 < total; k0 += 32) {
                    const int k = WARP_SCREEN ? k0 + lane : k0;
                    const bool have = k < total;
                    int p = 0;
#pragma unroll
                    for (int s = 16; s > 0; s >>= 1)
                        if (p + s < 32 && P.pre[p + s] <= k) p += s;
                    const int jj = have ? __fns(P.msk[p], 0, k - P.pre[p] + 1) : 0;
                    const Entry& e = sh.ent[wl][jj];
                    const float px = P.cx[p], py = P.cy[p], pz0 = P.z0l[p];
                    const float ub = e.maxz;  // refined below by the screen
                    float lo, hi, qt = 3.0e38f, qth = NEG_INF32;
                    uint32_t rank;
                    {
                        const Tri32 t = ctx.t32[e.tri];
                        Iv v;
                        if (WARP_SCREEN)
                            v = screen_bull_warp(prof, ctx.t32, e.tri, t, px - t.v0[0], py - t.v0[1], ctx.E, have);
                        else if (KIND == 2)
                            v = screen_composite(comp, t, px - t.v0[0], py - t.v0[1], ctx.E, pz0 - t.v0[2], qt, qth);
                        else
                            v = screen_triangle(prof, t, px - t.v0[0], py - t.v0[1], ctx.E, pz0 - t.v0[2], qt, qth);
                        if (!have) continue;
                        ++screened;
                        lo = v.lo > NEG_INF32 ? v.lo + t.v0[2] - ctx.E : NEG_INF32;
                        hi = v.hi > NEG_INF32 ? fminf(v.hi + t.v0[2] + ctx.E, ub + gd) : NEG_INF32;
                        if (qt < 3.0e38f) {
                            qt = qt + t.v0[2] - ctx.E;
                            qth = qth + t.v0[2] + ctx.E;
                        }
                        rank = t.kd_rank;
                    }
                    if (phase == PH_RESOLVE) {
                        const int nbp = min(P.nb[p], NBRANCH);
                        for (int j = 0; j < nbp; ++j) {
                            if (((P.pending[p] >> j) & 1u) && rank < br.rank[j][p]) {
                                atomicMax(&br.Wp[j][p], ((unsigned long long)f2u(lo) << 32) | (unsigned)e.tri);
                                atomicMax(&br.H[j][p], f2o(hi));
                                if (lo > br.qhi[j][p] + gd) atomicAnd(&P.pending[p], ~(1u << j));
                            }
                        }
                        continue;
                    }
                    if (phase == PH_SINGLE) {
                        if (lo > o2f(P.blo[p])) atomicMax(&P.blo[p], f2o(lo));
                        // track triangles that branch and may still matter
                        if (KIND != 0 && qt < 3.0e38f && hi >= o2f(P.blo[p]) - gd) {
                            const int slot = atomicAdd(&P.nb[p], 1);
                            if (slot < NBRANCH) {
                                br.tri[slot][p] = e.tri;
                                br.rank[slot][p] = rank;
                                br.qlo[slot][p] = qt;
                                br.qhi[slot][p] = qth;
                                br.hi[slot][p] = hi;
                            } else {
                                atomicMin(&P.qx[p], f2o(qt));
                            }
                        }
                    }
                    // collect (PH_SINGLE: lazily pruned against the rising bound)
                    const float keep = (phase == PH_COLLECT) ? P.thr[p] : o2f(P.blo[p]);
                    if (!(hi >= keep - gd && hi > pz0 - gd) || (P.flags[p] & PF_OVERFLOW)) continue;
                    if (phase == PH_COLLECT && qt < P.thr[p] - gd &&
                        !is_resolved(br, min(P.nb[p], NBRANCH), P.resolved[p], p, e.tri)) {
                        atomicOr(&P.flags[p], PF_CHAIN);
                        atomicMin(&P.chain_thr[p], f2o(qt));
                    }
                    const int slot = atomicAdd(&P.nc[p], 1);
                    if (slot < cap) {
                        const size_t o = (size_t)(base + p) * cap + slot;
                        ctx.cand[o] = (uint32_t)e.tri;
                        ctx.cand_hi[o] = hi;
                        ctx.cand_lo[o] = lo;
                    } else {
                        atomicOr(&P.flags[p], PF_OVERFLOW);
                    }
                }
                __syncwarp();
                if (P.nc[lane] > cap) P.nc[lane] = cap;
                __syncwarp();
            }
        }
        }
    }
    }
done:
    __syncwarp();
    ls.blo = o2f(P.blo[lane]);
    ls.qx = o2f(P.qx[lane]);
    ls.chain_thr = o2f(P.chain_thr[lane]);
    ls.nc = min(P.nc[lane], cap);
    ls.nb = min(P.nb[lane], NBRANCH);
    ls.pending = P.pending[lane];
    ls.overflow = (P.flags[lane] & PF_OVERFLOW) != 0;
    ls.chain = (P.flags[lane] & PF_CHAIN) != 0;
    ls.screened += screened;
    __syncwarp();
}

// The cone and composite kernels run three phases of scan_cells; one
// out-of-line copy serves them all (instruction cache).
template <int KIND, int CK, bool SPARSE>
__device__ __noinline__ void scan_cells_shared(const DropCtx& ctx, ScanShared& sh, int phase, LaneState& ls,
                                               bool active, uint32_t base, double xmin, double xmax, double ymin,
                                               double ymax) {
    scan_cells<KIND, CK, SPARSE>(ctx, sh, phase, ls, active, base, xmin, xmax, ymin, ymax);
}

// One pass for the warp: over the common rectangle of its points, or, for
// scattered points, over each point's own rectangle in turn (for that point).
template <int KIND, int CK, bool SPARSE>
__device__ __forceinline__ void scan_warp(const DropCtx& ctx, ScanShared& sh, int phase, LaneState& ls, bool act,
                                          uint32_t base, double x, double y, bool scattered, double xmin, double xmax,
                                          double ymin, double ymax) {
    const int lane = threadIdx.x & 31;
    if (!SPARSE) {
        if (KIND == 0) scan_cells<KIND, CK, SPARSE>(ctx, sh, phase, ls, act, base, xmin, xmax, ymin, ymax);
        else scan_cells_shared<KIND, CK, SPARSE>(ctx, sh, phase, ls, act, base, xmin, xmax, ymin, ymax);
        return;
    }
    const unsigned want = __ballot_sync(0xffffffffu, act);
    for (int o = 0; o < (scattered ? 32 : 1); ++o) {
        if (scattered && !((want >> o) & 1u)) continue;
        double x0 = xmin, x1 = xmax, y0 = ymin, y1 = ymax;
        if (scattered) {
            x0 = x1 = __shfl_sync(0xffffffffu, x, o);
            y0 = y1 = __shfl_sync(0xffffffffu, y, o);
        }
        if (KIND == 0) scan_cells<KIND, CK, SPARSE>(ctx, sh, phase, ls, act && (!scattered || lane == o), base, x0, x1, y0, y1);
        else scan_cells_shared<KIND, CK, SPARSE>(ctx, sh, phase, ls, act && (!scattered || lane == o), base, x0, x1, y0, y1);
    }
}

// Screen kernel.  KIND 0: one pass.  KIND 1/2 (cone, composite): the effect
// of a triangle on the running height can depend on the height reached before
// it (tip/rim short-circuits), so
//   pass 1  blo, the list at blo, and the branching triangles that matter;
//           a branch point below blo is decided by a witness in the list (an
//           earlier-ranked triangle certainly above it);
//   pass 2  (only points with an undecided branch) witnesses among all
//           triangles, or every earlier-ranked triangle below the branch;
//   then    a branch still undecided is checked exactly by the refinement
//           (the triangle is flagged in the list), or, for untracked ones, the
//           list is collected again at the lowest open branch threshold.
// A certified lower bound of a point's result from the triangles of its own
// finest-level cells (the 2 x 2 cells whose triangles may contain it).  Used
// for warps whose points are spread out: the common scan order reaches most
// of them late, so their bounds would rise late and cull little.
template <int KIND, int CK>
__device__ __forceinline__ float seed_blo(const DropCtx& ctx, double x, double y, bool active, float z0l) {
    const GridP& g = ctx.g;
    const float cx = (float)(x - g.ox), cy = (float)(y - g.oy);
    Prof32 prof = ctx.prof;
    prof.kind = CK;
    Comp32 comp = ctx.comp;
    if (KIND == 2 && CK >= 0) {
        comp.nsub = CK >> 16;
#pragma unroll
        for (int k = 0; k < OCL_GB300_MAX_SUB; ++k) comp.sub[k].kind = (CK >> (4 * k)) & 15;
    }
    float blo = z0l;
    const int c = clampi((int)floor((x - g.x0) * g.inv_cs[0]), 0, g.ncol[0] - 1);
    const int r = clampi((int)floor((y - g.y0) * g.inv_cs[0]), 0, g.nrow[0] - 1);
    for (int q = 0; q < 4; ++q) {
        const int cq = c - (q & 1), rq = r - (q >> 1);
        uint32_t start = 0, cnt = 0;
        if (active && cq >= 0 && rq >= 0) {
            const Cell cell = ctx.cells[g.cell_off[0] + rq * g.ncol[0] + cq];
            start = cell.start;
            cnt = min(cell.count, 8u);
        }
        uint32_t most = cnt;
        for (int o = 16; o > 0; o >>= 1) most = max(most, __shfl_xor_sync(0xffffffffu, most, o));
        for (uint32_t k = 0; k < most; ++k) {
            if (k >= cnt) continue;
            const Tri32 t = ctx.t32[start + k];
            float qt, qth;
            Iv v = (KIND == 2) ? screen_composite(comp, t, cx - t.v0[0], cy - t.v0[1], ctx.E, z0l - t.v0[2], qt, qth)
                               : screen_triangle(prof, t, cx - t.v0[0], cy - t.v0[1], ctx.E, z0l - t.v0[2], qt, qth);
            if (v.lo > NEG_INF32) blo = fmaxf(blo, v.lo + t.v0[2] - ctx.E);
        }
    }
    return blo;
}

// One warp per 32 sorted points: seeds the bounds of spread-out warps into
// ctx.blo (the screen starts from them); other warps get the start height.
template <int KIND, int CK>
__device__ __forceinline__ void seed_warp(const DropCtx& ctx, const int base) {
    if (base >= ctx.M) return;
    const int lane = threadIdx.x & 31;
    const bool active = base + lane < ctx.M;
    const uint32_t i = (uint32_t)(active ? base + lane : base);
    const double x = ctx.cl[3 * i], y = ctx.cl[3 * i + 1];
    const float z0l = __double2float_rd(ctx.cl[3 * i + 2] - ctx.g.oz);
    const double xmin = warp_mind(active ? x : 1e300), xmax = warp_maxd(active ? x : -1e300);
    const double ymin = warp_mind(active ? y : 1e300), ymax = warp_maxd(active ? y : -1e300);
    float blo = z0l;
    if ((xmax - xmin) + (ymax - ymin) > ctx.cp.radius) blo = seed_blo<KIND, CK>(ctx, x, y, active, z0l);
    if (active) ctx.blo[i] = blo;
}

template <int KIND, int CK>
__global__ void __launch_bounds__(128) k_drop_seed(const __grid_constant__ DropCtx ctx) {
    seed_warp<KIND, CK>(ctx, ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32);
}

// The same over the tiles of a batch (persistent blocks, work stealing).
template <int KIND, int CK>
__global__ void __launch_bounds__(128) k_drop_seed_b(const __grid_constant__ BatchView bv) {
    __shared__ DropCtx s_ctx;
    __shared__ TileState ts;
    if (threadIdx.x == 0) ts.job = 0xFFFFFFFFu;
    uint2 tile;
    while (batch_next_tile(bv, ts, s_ctx, tile))
        seed_warp<KIND, CK>(s_ctx, (int)(tile.y * TILE_POINTS) + (int)(threadIdx.x >> 5) * 32);
}

template <int KIND, int CK, bool SPARSE>
__device__ __forceinline__ void screen_warp(const DropCtx& ctx, ScanShared& sh, const int base) {
    const int lane = threadIdx.x & 31;
    const int wl = threadIdx.x >> 5;
    const bool active = base + lane < ctx.M;
    const uint32_t i = (uint32_t)(active ? base + lane : base);
    const GridP& g = ctx.g;
    const double x = ctx.cl[3 * i], y = ctx.cl[3 * i + 1], z0 = ctx.cl[3 * i + 2];
    const float gd = ctx.guard;
    BranchTab& br = sh.br[wl];
    WarpPoints& P = sh.pt[wl];
    P.cx[lane] = (float)(x - g.ox);
    P.cy[lane] = (float)(y - g.oy);
    P.z0l[lane] = __double2float_rd(z0 - g.oz);
    LaneState ls;
    ls.blo = P.z0l[lane];
    ls.qx = 3.0e38f;
    ls.thr = 0.0f;
    ls.zu = __double2float_ru(z0 - g.oz);
    ls.nc = 0;
    ls.nb = 0;
    ls.resolved = 0;
    ls.pending = 0;
    ls.overflow = false;
    ls.chain = false;
    ls.chain_thr = 3.0e38f;
    ls.screened = 0;
    double xmin = warp_mind(active ? x : 1e300), xmax = warp_maxd(active ? x : -1e300);
    double ymin = warp_mind(active ? y : 1e300), ymax = warp_maxd(active ? y : -1e300);
    // scattered points (their common rectangle is larger than their own
    // rectangles together, e.g. sparse path samples): each point's rectangle
    // is scanned in turn instead
    bool scattered;
    {
        const double reach = 2.0 * ctx.cp.radius + 2.0 * ctx.g.cs[0];
        const double own = active ? reach * reach : 0.0;
        double sum_own = own;
        for (int o = 16; o > 0; o >>= 1) sum_own += __shfl_xor_sync(0xffffffffu, sum_own, o);
        scattered = (xmax - xmin + reach) * (ymax - ymin + reach) > sum_own;
    }
    if (!SPARSE && scattered) {
        // scattered points go to the sparse kernel
        if (lane == 0) ctx.sparse_list[atomicAdd(ctx.sparse_n, 1ull)] = (uint32_t)(base >> 5);
        return;
    }
    // the seeding kernel's bound (spread-out warps), else the start height
    if (ctx.seeded && active) ls.blo = fmaxf(ls.blo, ctx.blo[i]);
    scan_warp<KIND, CK, SPARSE>(ctx, sh, PH_SINGLE, ls, active, (uint32_t)base, x, y, scattered, xmin, xmax, ymin, ymax);
    ls.thr = ls.blo;
    if (KIND != 0) {
        uint32_t* lt = ctx.cand + (size_t)i * ctx.cand_cap;
        const float* lh = ctx.cand_hi + (size_t)i * ctx.cand_cap;
        const float* ll = ctx.cand_lo + (size_t)i * ctx.cand_cap;
        // keep the branching triangles that can still reach blo; those whose
        // branch points lie at or above blo need no decision
        {
            int w = 0;
            for (int j = 0; j < ls.nb; ++j) {
                if (br.hi[j][lane] < ls.blo - gd) continue;
                br.tri[w][lane] = br.tri[j][lane];
                br.rank[w][lane] = br.rank[j][lane];
                br.qlo[w][lane] = br.qlo[j][lane];
                br.qhi[w][lane] = br.qhi[j][lane];
                br.hi[w][lane] = br.hi[j][lane];
                br.Wp[w][lane] = 0ull;  // no witness yet
                br.H[w][lane] = f2o(ls.zu);
                if (br.qlo[w][lane] < ls.blo) ls.pending |= 1u << w;
                else ls.resolved |= 1u << w;
                ++w;
            }
            ls.nb = w;
        }
        // witnesses in the list (they are folded anyway)
        if (active && ls.pending && !ls.overflow) {
            for (int q = 0; q < ls.nc; ++q) {
                if (!(lh[q] >= ls.blo - gd)) continue;
                const float lq = ll[q];
                const uint32_t rq = ctx.t32[lt[q]].kd_rank;
                for (int j = 0; j < ls.nb; ++j)
                    if (((ls.pending >> j) & 1u) && rq < br.rank[j][lane] && lq > br.qhi[j][lane] + gd) {
                        ls.pending &= ~(1u << j);
                        ls.resolved |= 1u << j;
                    }
                if (!ls.pending) break;
            }
        }
        if (!active || ls.overflow || ls.qx < ls.blo) ls.pending = 0;
        if (__any_sync(0xffffffffu, ls.pending != 0)) {
            float cut = 3.0e38f;
            for (int j = 0; j < ls.nb; ++j)
                if ((ls.pending >> j) & 1u) cut = fminf(cut, br.qlo[j][lane]);
            ls.thr = cut;
            const unsigned was = ls.pending;
            scan_warp<KIND, CK, SPARSE>(ctx, sh, PH_RESOLVE, ls, ls.pending != 0, (uint32_t)base, x, y, scattered, xmin, xmax,
                                ymin, ymax);
            for (int j = 0; j < ls.nb; ++j) {
                if (!((was >> j) & 1u)) continue;
                const unsigned long long wp = br.Wp[j][lane];
                const bool above = wp != 0ull && u2f((unsigned)(wp >> 32)) > br.qhi[j][lane] + gd;
                const bool below = o2f(br.H[j][lane]) < br.qlo[j][lane] - gd;
                if (above || below) ls.resolved |= 1u << j;
            }
            ls.pending = 0;
        }
        // a branch still undecided: the refinement decides it exactly (FP64)
        // for a tracked triangle, which is in the list (flagged); untracked
        // ones lower the collection threshold instead
        float open = 3.0e38f;
        bool verify = false;
        if (active && !ls.overflow) {
            int pos[NBRANCH];
            bool all_found = ls.qx >= ls.blo;
            for (int j = 0; j < ls.nb; ++j) {
                pos[j] = -1;
                if ((ls.resolved >> j) & 1u) continue;
                open = fminf(open, br.qlo[j][lane]);
                for (int q = 0; q < ls.nc && pos[j] < 0; ++q)
                    if (lt[q] == br.tri[j][lane] && lh[q] >= ls.blo - gd) pos[j] = q;
                if (pos[j] < 0) all_found = false;
            }
            if (all_found && open < ls.blo) {
                for (int j = 0; j < ls.nb; ++j)
                    if (pos[j] >= 0) lt[pos[j]] |= CAND_VERIFY;
                verify = true;
                open = 3.0e38f;
            }
            open = fminf(open, ls.qx);
        }
        ls.thr = ls.blo;
        const bool need = active && open < ls.blo && !ls.overflow;
        if (need || (active && verify)) atomicAdd(&ctx.counters[C_OPEN], 1ull);
        if (need) atomicAdd(&ctx.counters[C_UNTRACKED], 1ull);
        if (__any_sync(0xffffffffu, need)) {
            // collect at the lowest open threshold; if a collected triangle's
            // branch threshold lies below it, lower it and collect again
            ls.thr = need ? open : 3.0e38f;
            bool done = !need;
            for (int round = 0; round < 4; ++round) {
                const float keep_thr = ls.thr;
                if (!done) {
                    ls.nc = 0;
                    ls.chain = false;
                    ls.chain_thr = 3.0e38f;
                }
                scan_warp<KIND, CK, SPARSE>(ctx, sh, PH_COLLECT, ls, active && !done, (uint32_t)base, x, y, scattered, xmin,
                                    xmax, ymin, ymax);
                ls.thr = keep_thr;
                const bool again = !done && ls.chain && !ls.overflow && round < 3;
                if (again) ls.thr = fminf(ls.thr, ls.chain_thr);
                else done = true;
                if (!__any_sync(0xffffffffu, again)) break;
            }
            if (!need) ls.thr = ls.blo;
        }
        // witnesses found outside the list must be folded before their
        // triangles: add them (pinned against pruning)
        if (active && !ls.overflow && !ls.chain) {
            float* lhw = ctx.cand_hi + (size_t)i * ctx.cand_cap;
            for (int j = 0; j < ls.nb; ++j) {
                if (!((ls.resolved >> j) & 1u)) continue;
                const unsigned long long wp = br.Wp[j][lane];
                if (wp == 0ull || !(u2f((unsigned)(wp >> 32)) > br.qhi[j][lane] + gd)) continue;
                const uint32_t wt = (uint32_t)(wp & 0xFFFFFFFFull);
                bool have = false;
                for (int q = 0; q < ls.nc && !have; ++q)
                    have = ((lt[q] & ~CAND_VERIFY) == wt && lhw[q] >= ls.thr - gd);
                if (have) continue;
                if (ls.nc == ctx.cand_cap) {
                    ls.overflow = true;
                    break;
                }
                lt[ls.nc] = wt;
                lhw[ls.nc] = 3.0e38f;
                ++ls.nc;
            }
        }
    }
    __syncwarp();
    if (active) {
        if (ls.overflow || ls.chain) {
            ctx.ncand[i] = 0xFFFF;
            atomicAdd(&ctx.counters[ls.overflow ? C_OVERFLOW : C_CHAIN], 1ull);
        } else {
            uint32_t* lt = ctx.cand + (size_t)i * ctx.cand_cap;
            const float* lh = ctx.cand_hi + (size_t)i * ctx.cand_cap;
            int w = 0;
            for (int q = 0; q < ls.nc; ++q)
                if (lh[q] >= ls.thr - gd) lt[w++] = lt[q];
            // order the list by the reference's visit order (ascending KD rank)
            for (int a = 1; a < w; ++a) {
                const uint32_t t = lt[a];
                const uint32_t rk = ctx.t32[t & ~CAND_VERIFY].kd_rank;
                int b = a - 1;
                while (b >= 0 && ctx.t32[lt[b] & ~CAND_VERIFY].kd_rank > rk) {
                    lt[b + 1] = lt[b];
                    --b;
                }
                lt[b + 1] = t;
            }
            ctx.ncand[i] = (uint16_t)w;
        }
        ctx.blo[i] = ls.blo;
    }
    unsigned long long scr = ls.screened;
    for (int o = 16; o > 0; o >>= 1) scr += __shfl_xor_sync(0xffffffffu, scr, o);
    if (lane == 0 && scr) atomicAdd(&ctx.counters[C_SCREENED], scr);
}

template <int KIND, int CK, bool SPARSE>
__global__ void __launch_bounds__(SCREEN_WARPS * 32, screen_min_blocks(KIND, CK))
    k_drop_screen(const __grid_constant__ DropCtx ctx) {
    __shared__ ScanShared sh;
    for (int k = threadIdx.x; k < HLB_N; k += blockDim.x) sh.hlb[k] = ctx.hlb[k];
    __syncthreads();
    const int wl = threadIdx.x >> 5;
    if (!SPARSE) {
        const int base = (blockIdx.x * SCREEN_WARPS + wl) * 32;
        if (base < ctx.M) screen_warp<KIND, CK, SPARSE>(ctx, sh, base);
        return;
    }
    // the warps the dense kernel handed over (count on the device)
    const unsigned long long n = *ctx.sparse_n;
    for (unsigned long long w = blockIdx.x * SCREEN_WARPS + wl; w < n; w += (unsigned long long)gridDim.x * SCREEN_WARPS)
        screen_warp<KIND, CK, SPARSE>(ctx, sh, (int)(ctx.sparse_list[w] << 5));
}

// Batch versions.  Dense: persistent blocks over the launch's tiles (one
// tile = the 4 warps of one block of a job), the job's context and profile
// table in shared memory.  Sparse: every block strides over the scattered
// warps of each job of the launch in turn (counts on the device).
template <int KIND, int CK>
__global__ void __launch_bounds__(SCREEN_WARPS * 32, screen_min_blocks(KIND, CK))
    k_drop_screen_b(const __grid_constant__ BatchView bv) {
    __shared__ ScanShared sh;
    __shared__ DropCtx s_ctx;
    __shared__ TileState ts;
    if (threadIdx.x == 0) ts.job = 0xFFFFFFFFu;
    uint2 tile;
    int r;
    while ((r = batch_next_tile(bv, ts, s_ctx, tile)) != 0) {
        if (r == 2) {
            for (int k = threadIdx.x; k < HLB_N; k += blockDim.x) sh.hlb[k] = s_ctx.hlb[k];
            __syncthreads();
        }
        const int base = (int)(tile.y * SCREEN_WARPS + (threadIdx.x >> 5)) * 32;
        if (base < s_ctx.M) screen_warp<KIND, CK, false>(s_ctx, sh, base);
    }
}

template <int KIND, int CK>
__global__ void __launch_bounds__(SCREEN_WARPS * 32, screen_min_blocks(KIND, CK))
    k_drop_screen_sparse_b(const __grid_constant__ BatchView bv) {
    __shared__ ScanShared sh;
    const int wl = threadIdx.x >> 5;
    for (unsigned k = 0; k < bv.njobs; ++k) {
        const DropCtx& ctx = bv.ctxs[bv.jobs[k]];
        const unsigned long long n = *ctx.sparse_n;
        if (n == 0) continue;
        __syncthreads();
        for (int q = threadIdx.x; q < HLB_N; q += blockDim.x) sh.hlb[q] = ctx.hlb[q];
        __syncthreads();
        for (unsigned long long w = blockIdx.x * SCREEN_WARPS + wl; w < n;
             w += (unsigned long long)gridDim.x * SCREEN_WARPS)
            screen_warp<KIND, CK, true>(ctx, sh, (int)(ctx.sparse_list[w] << 5));
    }
}


}  // namespace oclg
