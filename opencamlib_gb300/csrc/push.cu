// push.cu -- BatchPushCutter on the GPU (BatchPushCutter::pushCutter3,
// algo/batchpushcutter.cpp:136-188).
//
// Lanes are fibers: a warp takes 32 consecutive fibers (a Waterline level's
// fibers are adjacent), walks the KD tree of the fiber direction (YZ for
// X-fibers, XZ for Y-fibers) with one visit mask per node, so every lane gets
// exactly the reference's candidate triangles in the reference's order; each
// candidate is pushed in FP64 (MillingCutter::pushCutter) and its interval is
// merged into the lane's fiber with Fiber::addInterval's rules (fiber.cpp:58-93),
// keeping the reference's interval order and CC points.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "drop.cuh"
#include "drop_util.cuh"
#include "geom32.cuh"
#include "push64.cuh"
#include "util.cuh"

namespace oclg {

constexpr int PUSH_CAP = 48;        // intervals a fiber may hold while merging (first pass, local memory)
constexpr int PUSH_CAP_BIG = 4096;  // second pass for the fibers that overflowed (global scratch)

struct PushRec {
    double lower, upper;
    double lcc[3], ucc[3];
    int32_t ltype, utype;
};
static_assert(sizeof(PushRec) == 72, "PushRec layout");

constexpr int WUB_N = 256;  // entries of the cutter width upper-bound table

struct PushCtx {
    CutterP cp;
    int dir;
    // FP32 prefilter: grid entries (bbox local to the origin, rounded
    // outward, max z rounded up), the origin, the error budget of local FP32
    // coordinates, a lower bound of the cutter's height at each radius and an
    // upper bound of its width at each height
    const Entry* ent;
    double ox, oy, oz;
    float E;
    float R, inv_rstep;     // hlb: height lower bound at radius >= k R / HLB_N
    float inv_hstep;        // wub: width upper bound at heights <= (k + 1) H / WUB_N
    bool use_wub;           // basic cutters (the composite's width bound is R)
    float hlb[HLB_N];
    float wub[WUB_N];
    const Tri64* t64;
    const double* esin;  // edge slopes, 3 per triangle
    const KDNodeD* nodes;
    const float2* cut32;  // the nodes' cuts rounded down / up to float
    const int32_t* order;
    const double* fib;
    int F;
    PushRec* recs;
    uint64_t cap;
    unsigned long long* cursor;
    uint32_t* counts;
    uint64_t* offs;
    unsigned long long* counters;  // [0] calls, [1] capped, [2] merge overflow, [3] cursor, [4] FP64 pushes
};

__device__ __forceinline__ bool iv_outside(const Ival64& a, const Ival64& b) {
    if (a.lower > b.upper) return true;
    if (a.upper < b.lower) return true;
    return false;
}

// FP32 bounds of an interval for the prefilter: the lower end rounded up,
// the upper end rounded down (a bound strictly inside them is strictly
// inside the interval).
__device__ __forceinline__ float2 iv_inner32(const Ival64& i) {
    return make_float2(__double2float_ru(i.lower), __double2float_rd(i.upper));
}

// Fiber::addInterval on a per-lane array (with the FP32 inner bounds of
// every interval kept beside it); returns false on capacity overflow.
__device__ inline bool fiber_add(Ival64* ints, float2* in32, int& n, const Ival64& i, int cap) {
    if (i.lower == 0.0 && i.upper == 0.0) return true;  // Interval::empty (interval.cpp:113-118)
    if (n == 0) {
        in32[n] = iv_inner32(i);
        ints[n++] = i;
        return true;
    }
    for (int k = 0; k < n; ++k)
        if ((i.lower > ints[k].lower) && (i.upper < ints[k].upper)) return true;  // contains
    bool missing = true;
    for (int k = 0; k < n; ++k)
        if (!iv_outside(i, ints[k])) missing = false;
    if (missing) {
        if (n == cap) return false;
        in32[n] = iv_inner32(i);
        ints[n++] = i;
        return true;
    }
    // merge all overlapping intervals (in vector order) with i into one sum
    Ival64 sum;
    iv_init(sum);
    int w = 0;
    for (int k = 0; k < n; ++k) {
        if (!iv_outside(ints[k], i)) {
            iv_lower(sum, ints[k].lower, ints[k].lcc);
            iv_upper(sum, ints[k].upper, ints[k].ucc);
        } else {
            in32[w] = in32[k];
            ints[w++] = ints[k];
        }
    }
    iv_lower(sum, i.lower, i.lcc);
    iv_upper(sum, i.upper, i.ucc);
    n = w;
    in32[n] = iv_inner32(sum);
    ints[n++] = sum;
    return true;
}

// The fiber in the FP32 frame of the prefilter.
struct FiberGeom32 {
    float cr;     // across coordinate, local to the origin
    float z;      // height, local
    float f0;     // along coordinate of p1, local
    float finv;   // 1 / length along (0: degenerate)
    float tmarg;  // error of an along coordinate in t units
};

// The prefilter of one (fiber, candidate) pair: false when the candidate's
// push interval is provably empty or strictly inside an interval the fiber
// holds (Fiber::addInterval ignores such an interval), so leaving it out
// changes nothing.  Every push contact lies on the cutter's surface: within
// the radius of the axis and no lower than the profile height at its
// distance; so a triangle farther than the radius from the fiber's line, or
// entirely below the profile at its nearest distance, has an empty interval,
// and an interval lies within the triangle's along-extent grown by the
// cutter's half-width at the triangle's distance and height.  Evaluated in
// FP32 on the grid entries, every bound taken outward by the error budget E
// of the local frame (entry bboxes rounded outward, fiber coordinates rounded
// to nearest, each FP32 operation's rounding), the cutter's height and width
// from the conservative tables of PushCtx.
__device__ __forceinline__ bool push_needed32(const PushCtx& ctx, const FiberGeom32& g, bool xf, const Entry& e,
                                              const float2* in32, int n, bool overflow) {
    const float E = ctx.E;
    const float lo = xf ? e.miny : e.minx, hi = xf ? e.maxy : e.maxx;
    const float gap = fmaxf(lo - g.cr, g.cr - hi);
    if (gap > ctx.R + E) return false;
    const float dlb = gap - E;  // the true distance is at least this
    if (e.maxz < g.z + fmaxf(hlb_at(ctx.hlb, dlb, ctx.inv_rstep), 0.0f) - E) return false;
    if (n == 0 || overflow || g.finv == 0.0f) return true;
    const float gl = fmaxf(dlb, 0.0f);
    float halfw = __fsqrt_ru(fmaxf(__fmaf_ru(-gl, gl, __fmul_ru(ctx.R, ctx.R)), 0.0f));
    if (ctx.use_wub) {
        const float hub = __fadd_ru(__fsub_ru(e.maxz, g.z), E);
        int k = (int)(fmaxf(hub, 0.0f) * ctx.inv_hstep);
        k = min(k, WUB_N - 1);
        halfw = fminf(halfw, ctx.wub[k]);
    }
    halfw = __fadd_ru(halfw, E);
    const float alo = xf ? e.minx : e.miny, ahi = xf ? e.maxx : e.maxy;
    float a = (alo - halfw - g.f0) * g.finv;
    float b = (ahi + halfw - g.f0) * g.finv;
    if (a > b) {
        const float t = a;
        a = b;
        b = t;
    }
    a = __fsub_rd(a, g.tmarg + 2.4e-7f * fabsf(a));
    b = __fadd_ru(b, g.tmarg + 2.4e-7f * fabsf(b));
    for (int q = 0; q < n; ++q)
        if (a > in32[q].x && b < in32[q].y) return false;
    return true;
}

// The fiber in FP64 (the reference's search box and the FP32 frame's inputs).
struct FiberGeom {
    bool xf;         // X fiber
    double r;        // cutter radius
    double cr;       // the fiber's fixed coordinate across (y of an X fiber)
    double z;        // its height
    double f0, finv; // along-coordinate of p1, 1 / length (0: degenerate)
};

// Per-warp shared state of k_push.
constexpr int PUSH_CHUNK = 32;  // candidates buffered per warp before they are screened and pushed
struct PushWarp {
    uint2 stack[KD_STACK];
    uint32_t tri[PUSH_CHUNK];   // buffered candidates (device triangle ids), in the KD visit order
    uint32_t msk[PUSH_CHUNK];   // lanes whose search reached each candidate
    unsigned pm[PUSH_CHUNK];    // lanes that must push each candidate
    int po[PUSH_CHUNK + 1];     // pairs before each candidate
    Fib64 fib[32];              // the lanes' fibers
    Ival64 res[32];             // one round of pushed intervals
    int owner[32];              // their lanes
};

// list == nullptr: fibers 0..F-1 with the intervals in local memory;
// otherwise the listed fibers with PUSH_CAP_BIG intervals each in scratch.
//
// A warp walks the KD tree for its 32 fibers (lanes) together and buffers
// the candidates it reaches, with the lanes that reached each, 32 at a time.
// Each lane then screens its own fiber against the buffered candidates
// (push_needed32, against the intervals it held when the chunk began: they
// only grow, so what is inside them stays inside).  The (lane, candidate)
// pairs that must be pushed are spread over all lanes, one FP64 push per lane
// per round, in candidate-major order; after each round every lane merges its
// own pushed intervals into its fiber in candidate order with
// Fiber::addInterval's rules.  So every fiber sees every candidate's interval
// in the reference's order, and intervals strictly inside one it holds are
// ignored exactly as the reference ignores them.
__global__ void __launch_bounds__(128) k_push(const PushCtx* __restrict__ ctxp, const uint32_t* __restrict__ list,
                                              int nlist, Ival64* __restrict__ scratch, float2* __restrict__ scratch32) {
    const PushCtx& ctx = *ctxp;
    __shared__ PushWarp s_warp[4];
    const int lane = threadIdx.x & 31;
    const int wl = threadIdx.x >> 5;
    PushWarp& W = s_warp[wl];
    const int base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32;
    const int count = list ? nlist : ctx.F;
    if (base >= count) return;
    const bool active = base + lane < count;
    const int slot = active ? base + lane : base;
    const int f = list ? (int)list[slot] : slot;
    Fib64 fb;
    fb.p1 = d3(ctx.fib[6 * f], ctx.fib[6 * f + 1], ctx.fib[6 * f + 2]);
    fb.p2 = d3(ctx.fib[6 * f + 3], ctx.fib[6 * f + 4], ctx.fib[6 * f + 5]);
    fb.dir = normalize3(fb.p2 - fb.p1);  // Fiber::calcDir (fiber.cpp:35-39)
    W.fib[lane] = fb;
    const double r = ctx.cp.radius;
    // pushCutter3's search point and KDTree::search_cutter_overlap box
    double clx, cly;
    if (ctx.dir == OCL_GB300_XFIBER) { clx = 0; cly = fb.p1.y; }
    else { clx = fb.p1.x; cly = 0; }
    const double bb[6] = {clx - r, clx + r, cly - r, cly + r, fb.p1.z, fb.p1.z + ctx.cp.length};
    // the box in FP32, minima rounded down, maxima up (the walk prunes a
    // subtree only where the FP32 test is certain: it visits every leaf the
    // FP64 test visits, and the triangles of any other leaf lie outside the
    // box, so their push intervals are empty and change nothing)
    float bb32[6];
    for (int k = 0; k < 6; ++k) bb32[k] = (k & 1) ? __double2float_ru(bb[k]) : __double2float_rd(bb[k]);
    FiberGeom geo;
    geo.xf = ctx.dir == OCL_GB300_XFIBER;
    geo.r = r;
    geo.cr = geo.xf ? fb.p1.y : fb.p1.x;
    geo.z = fb.p1.z;
    geo.f0 = geo.xf ? fb.p1.x : fb.p1.y;
    {
        const double fl = geo.xf ? fb.p2.x - fb.p1.x : fb.p2.y - fb.p1.y;
        geo.finv = fl != 0.0 ? 1.0 / fl : 0.0;
    }
    FiberGeom32 g32;
    g32.cr = (float)(geo.cr - (geo.xf ? ctx.oy : ctx.ox));
    g32.z = (float)(geo.z - ctx.oz);
    g32.f0 = (float)(geo.f0 - (geo.xf ? ctx.ox : ctx.oy));
    g32.finv = (float)geo.finv;
    g32.tmarg = 2.0f * ctx.E * fabsf(g32.finv);
    Ival64 local_ints[PUSH_CAP];
    float2 local_in32[PUSH_CAP];
    Ival64* ints = list ? scratch + (size_t)slot * PUSH_CAP_BIG : local_ints;
    float2* in32 = list ? scratch32 + (size_t)slot * PUSH_CAP_BIG : local_in32;
    const int cap = list ? PUSH_CAP_BIG : PUSH_CAP;
    int n = 0;
    bool overflow = false;
    unsigned long long calls = 0;
    unsigned pushed = 0;
    int capped = 0;
    uint2* st = W.stack;
    const unsigned amask = __ballot_sync(0xffffffffu, active);
    int sp = 0;
    int nc = 0;  // buffered candidates (warp-uniform)
    if (ctx.nodes && amask) {
        if (lane == 0) st[0] = make_uint2(0u, amask);
        sp = 1;
    }
    __syncwarp();
    // screens, pushes and merges the buffered candidates (warp-collective)
    auto flush = [&]() {
        unsigned need = 0;
        for (int c = 0; c < nc; ++c) {
            if (!((W.msk[c] >> lane) & 1u)) continue;
            ++calls;
            if (push_needed32(ctx, g32, geo.xf, ctx.ent[W.tri[c]], in32, n, overflow)) need |= 1u << c;
        }
        int tot = 0;
        for (int c = 0; c < nc; ++c) {
            const unsigned m = __ballot_sync(0xffffffffu, (need >> c) & 1u);
            if (lane == 0) {
                W.pm[c] = m;
                W.po[c] = tot;
            }
            tot += __popc(m);
        }
        if (lane == 0) W.po[nc] = tot;
        __syncwarp();
        for (int b0 = 0; b0 < tot; b0 += 32) {
            const int q = b0 + lane;
            int own = -1;
            if (q < tot) {
                int c = 0;  // the last candidate with po[c] <= q (it has pairs)
                for (int s = 16; s > 0; s >>= 1)
                    if (c + s < nc && W.po[c + s] <= q) c += s;
                own = (int)__fns(W.pm[c], 0, q - W.po[c] + 1);
                const uint32_t ti = W.tri[c];
                Ival64 iv;
                iv_init(iv);
                push_triangle64(ctx.cp, W.fib[own], iv, ctx.t64[ti], ctx.esin ? ctx.esin + 3 * (size_t)ti : nullptr,
                                &capped);
                W.res[lane] = iv;
                ++pushed;
            }
            W.owner[lane] = own;
            __syncwarp();
            const int nr = min(32, tot - b0);
            for (int j = 0; j < nr; ++j)
                if (W.owner[j] == lane && !overflow && !fiber_add(ints, in32, n, W.res[j], cap)) overflow = true;
            __syncwarp();
        }
        nc = 0;
    };
    while (sp > 0) {
        --sp;
        const uint2 e = st[sp];
        __syncwarp();
        const KDNodeD nd = ctx.nodes[e.x];
        const bool in = (e.y >> lane) & 1u;
        if (nd.leaf_begin >= 0) {
            for (int k = nd.leaf_begin; k < nd.leaf_end; ++k) {
                if (lane == 0) {
                    W.tri[nc] = (uint32_t)ctx.order[k];
                    W.msk[nc] = e.y;
                }
                ++nc;
                if (nc == PUSH_CHUNK) {
                    __syncwarp();
                    flush();
                }
            }
            __syncwarp();
            continue;
        }
        bool vh, vl;
        const float2 c32 = ctx.cut32[e.x];
        if ((nd.dim & 1) == 0) {
            const bool only_lo = c32.x > bb32[nd.dim + 1];  // cut > box max, certainly
            vh = in && !only_lo && nd.hi >= 0;
            vl = in && nd.lo >= 0;
        } else {
            const bool only_hi = c32.y < bb32[nd.dim - 1];  // cut < box min, certainly
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
    if (nc > 0) {
        __syncwarp();
        flush();
    }
    // reserve output slots for the warp
    int cnt = active ? n : 0;
    int incl = cnt;
    for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    unsigned long long wbase = 0;
    if (lane == 31) wbase = atomicAdd(ctx.cursor, (unsigned long long)incl);
    wbase = __shfl_sync(0xffffffffu, wbase, 31);
    const unsigned long long mine = wbase + (unsigned long long)(incl - cnt);
    if (active) {
        ctx.counts[f] = overflow ? 0xFFFFFFFFu : (uint32_t)n;
        ctx.offs[f] = mine;
        for (int k = 0; k < n; ++k) {
            if (mine + k < ctx.cap) {
                PushRec rec;
                rec.lower = ints[k].lower;
                rec.upper = ints[k].upper;
                rec.lcc[0] = ints[k].lcc.p.x; rec.lcc[1] = ints[k].lcc.p.y; rec.lcc[2] = ints[k].lcc.p.z;
                rec.ucc[0] = ints[k].ucc.p.x; rec.ucc[1] = ints[k].ucc.p.y; rec.ucc[2] = ints[k].ucc.p.z;
                rec.ltype = ints[k].lcc.type;
                rec.utype = ints[k].ucc.type;
                ctx.recs[mine + k] = rec;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) calls += __shfl_xor_sync(0xffffffffu, calls, o);
    for (int o = 16; o > 0; o >>= 1) pushed += __shfl_xor_sync(0xffffffffu, pushed, o);
    for (int o = 16; o > 0; o >>= 1) capped += __shfl_xor_sync(0xffffffffu, capped, o);
    int ov = overflow ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) ov += __shfl_xor_sync(0xffffffffu, ov, o);
    if (lane == 0) {
        atomicAdd(&ctx.counters[0], calls);
        if (pushed) atomicAdd(&ctx.counters[4], (unsigned long long)pushed);
        if (capped) atomicAdd(&ctx.counters[1], (unsigned long long)capped);
        if (ov) atomicAdd(&ctx.counters[2], (unsigned long long)ov);
    }
}

void fill_prof(const CutterP& cp, Prof32& prof, float* hlb, bool& composite);

// The FP32 prefilter's tables and error budget for one call.
static void fill_push_screen(const Mesh& m, const CutterP& cp, const double* fibers, uint64_t F, PushCtx& h) {
    h.ent = m.d_entries;
    h.ox = m.grid.ox;
    h.oy = m.grid.oy;
    h.oz = m.grid.oz;
    Prof32 prof;
    bool composite = false;
    fill_prof(cp, prof, h.hlb, composite);
    const double R = cp.radius;
    h.R = (float)R;
    h.inv_rstep = (float)(HLB_N / R);
    // largest local coordinate of the mesh and of the fibers
    double maxabs = 0.5 * std::max(m.bb[1] - m.bb[0], std::max(m.bb[3] - m.bb[2], m.bb[5] - m.bb[4])) + R + 1.0;
    for (uint64_t k = 0; k < F; ++k) {
        const double* f = fibers + 6 * k;
        for (int j = 0; j < 2; ++j) {
            maxabs = std::max(maxabs, std::fabs(f[3 * j] - h.ox) + 1.0);
            maxabs = std::max(maxabs, std::fabs(f[3 * j + 1] - h.oy) + 1.0);
            maxabs = std::max(maxabs, std::fabs(f[3 * j + 2] - h.oz) + 1.0);
        }
    }
    h.E = (float)(8.0 * maxabs * std::ldexp(1.0, -24) + 4e-6 * std::max(1.0, R));
    // width(h) of a basic cutter is non-decreasing in h: the bin's upper end
    // bounds it from above (the composite's bound is the radius)
    h.use_wub = !composite;
    const double H = std::max(cp.length, R);
    h.inv_hstep = (float)(WUB_N / H);
    for (int k = 0; k < WUB_N; ++k) {
        double w = R;
        if (!composite) {
            const BasicP& b = cp.b;
            const double hh = H * (k + 1) / WUB_N;
            switch (b.kind) {
            case OCL_CUTTER_CYL: w = b.radius; break;
            case OCL_CUTTER_BALL: w = hh >= b.radius ? b.radius : std::sqrt(b.radius * b.radius - (b.radius - hh) * (b.radius - hh)); break;
            case OCL_CUTTER_BULL:
                w = hh >= b.radius2 ? b.radius
                                    : b.radius1 + std::sqrt(b.radius2 * b.radius2 - (b.radius2 - hh) * (b.radius2 - hh));
                break;
            case OCL_CUTTER_CONE: w = hh < b.center_height ? hh * b.tan_angle : b.radius; break;
            }
            w = std::min(w + 1e-6 * (1.0 + R), R + 1e-6 * (1.0 + R));
        }
        const float f = (float)w;
        h.wub[k] = ((double)f >= w) ? f : std::nextafter(f, 3.0e38f);
    }
}

int ensure_push_index(Mesh& m, int dir) {
    PushIndex& pi = m.push[dir];
    if (pi.built) return OCL_GB300_OK;
    KDTreeD kd;
    kd_build_host(m.host_bb, m.n, m.bucket, dir == OCL_GB300_XFIBER ? 1 : 2, kd);
    return upload_kd(m, kd, pi);
}

int push_run(Mesh& m, const CutterP& cp, int dir, const double* fibers, uint64_t F, uint64_t* offsets, double* ival,
             double* cc, int32_t* cctype, uint64_t cap, ocl_gb300_stats* stats) {
    for (uint64_t k = 0; k < F; ++k) {
        const double* f = fibers + 6 * k;
        bool ok = std::isfinite(f[0]) && std::isfinite(f[1]) && std::isfinite(f[2]) && std::isfinite(f[3]) &&
                  std::isfinite(f[4]) && std::isfinite(f[5]) && f[2] == f[5];
        ok = ok && (dir == OCL_GB300_XFIBER ? (f[1] == f[4] && f[0] != f[3]) : (f[0] == f[3] && f[1] != f[4]));
        if (!ok) {
            set_error("fiber " + std::to_string(k) + " is not a horizontal fiber of the requested direction");
            return OCL_GB300_BAD_ARG;
        }
    }
    offsets[0] = 0;
    if (F == 0) return OCL_GB300_OK;
    if (m.n > 0) {
        int st = ensure_push_index(m, dir);
        bool bull = cp.kind == OCL_CUTTER_BULL;
        for (int k = 0; k < cp.nsub && cp.kind == OCL_CUTTER_COMPOSITE; ++k) bull = bull || cp.sub[k].kind == OCL_CUTTER_BULL;
        if (!st && bull) st = ensure_edge_sin(m);
        if (st) return st;
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    DevBuf<double> dfib(6 * F);
    DevBuf<uint32_t> dcounts(F);
    DevBuf<uint64_t> doffs(F);
    DevBuf<unsigned long long> dcnt(5);
    DevBuf<PushCtx> dctx(1);
    if (!dfib.ok() || !dcounts.ok() || !doffs.ok() || !dcnt.ok() || !dctx.ok()) return OCL_GB300_OOM;
    CK(cudaMemcpy(dfib.p, fibers, 6 * F * sizeof(double), cudaMemcpyHostToDevice));
    uint64_t rcap = std::max<uint64_t>(4 * F, 1024);
    std::vector<PushRec> hrec;
    std::vector<uint32_t> hcounts(F);
    std::vector<uint64_t> hoffs(F);
    unsigned long long hc[5] = {0, 0, 0, 0, 0};
    float ms = 0;
    unsigned long long second_overflow = 0;
    for (int attempt = 0; attempt < 3; ++attempt) {
        DevBuf<PushRec> drec(rcap);
        if (!drec.ok()) return OCL_GB300_OOM;
        PushCtx h;
        std::memset(&h, 0, sizeof(h));
        h.cp = cp;
        h.dir = dir;
        h.t64 = m.d_t64;
        h.esin = m.d_edge_sin;
        fill_push_screen(m, cp, fibers, F, h);
        h.nodes = m.n > 0 ? m.push[dir].d_nodes : nullptr;
        h.cut32 = m.n > 0 ? m.push[dir].d_cut32 : nullptr;
        h.order = m.n > 0 ? m.push[dir].d_order : nullptr;
        h.fib = dfib.p;
        h.F = (int)F;
        h.recs = drec.p;
        h.cap = rcap;
        h.cursor = dcnt.p + 3;
        h.counts = dcounts.p;
        h.offs = doffs.p;
        h.counters = dcnt.p;
        CK(cudaMemcpy(dctx.p, &h, sizeof(h), cudaMemcpyHostToDevice));
        CK(cudaMemset(dcnt.p, 0, 5 * sizeof(unsigned long long)));
        const unsigned warps = (unsigned)((F + 31) / 32);
        CK(cudaEventRecord(e0));
        k_push<<<(warps + 3) / 4, 128>>>(dctx.p, nullptr, 0, nullptr, nullptr);
        CK(cudaGetLastError());
        CK(cudaMemcpy(hc, dcnt.p, sizeof(hc), cudaMemcpyDeviceToHost));
        second_overflow = 0;
        if (hc[2] > 0) {
            // fibers that held more intervals than the local buffer: redo them
            // with a large buffer each in global scratch
            CK(cudaMemcpy(hcounts.data(), dcounts.p, F * sizeof(uint32_t), cudaMemcpyDeviceToHost));
            std::vector<uint32_t> lst;
            for (uint64_t k = 0; k < F; ++k)
                if (hcounts[k] == 0xFFFFFFFFu) lst.push_back((uint32_t)k);
            DevBuf<uint32_t> dl(lst.size());
            DevBuf<Ival64> scratch(lst.size() * (size_t)PUSH_CAP_BIG);
            DevBuf<float2> scratch32(lst.size() * (size_t)PUSH_CAP_BIG);
            if (!dl.ok() || !scratch.ok() || !scratch32.ok()) return OCL_GB300_OOM;
            CK(cudaMemcpy(dl.p, lst.data(), lst.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
            CK(cudaMemset(dcnt.p + 2, 0, sizeof(unsigned long long)));
            const unsigned w2 = (unsigned)((lst.size() + 31) / 32);
            k_push<<<(w2 + 3) / 4, 128>>>(dctx.p, dl.p, (int)lst.size(), scratch.p, scratch32.p);
            CK(cudaGetLastError());
            CK(cudaMemcpy(hc, dcnt.p, sizeof(hc), cudaMemcpyDeviceToHost));
            second_overflow = hc[2];
        }
        CK(cudaEventRecord(e1));
        CK(cudaEventSynchronize(e1));
        cudaEventElapsedTime(&ms, e0, e1);
        if (hc[3] > rcap) {
            rcap = hc[3];
            continue;
        }
        hrec.resize(hc[3]);
        if (hc[3]) CK(cudaMemcpy(hrec.data(), drec.p, hc[3] * sizeof(PushRec), cudaMemcpyDeviceToHost));
        break;
    }
    hc[2] = second_overflow;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CK(cudaMemcpy(hcounts.data(), dcounts.p, F * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(hoffs.data(), doffs.p, F * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->pairs = hc[0];
        stats->screened = hc[0];
        stats->refined = hc[4];
        stats->iter_limit_hits = hc[1];
        stats->kernel_ms = ms;
    }
    if (hc[2]) {
        set_error("a fiber collected more than " + std::to_string(PUSH_CAP_BIG) + " disjoint intervals while merging");
        return OCL_GB300_ITER_LIMIT;
    }
    uint64_t total = 0;
    for (uint64_t k = 0; k < F; ++k) {
        offsets[k] = total;
        total += hcounts[k];
    }
    offsets[F] = total;
    if (total > cap) {
        set_error("interval buffer too small");
        return OCL_GB300_CAPACITY;
    }
    for (uint64_t k = 0; k < F; ++k) {
        for (uint32_t j = 0; j < hcounts[k]; ++j) {
            const PushRec& r = hrec[hoffs[k] + j];
            uint64_t o = offsets[k] + j;
            ival[2 * o] = r.lower;
            ival[2 * o + 1] = r.upper;
            std::memcpy(cc + 6 * o, r.lcc, 3 * sizeof(double));
            std::memcpy(cc + 6 * o + 3, r.ucc, 3 * sizeof(double));
            cctype[2 * o] = r.ltype;
            cctype[2 * o + 1] = r.utype;
        }
    }
    return OCL_GB300_OK;
}

}  // namespace oclg
