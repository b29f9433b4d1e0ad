// batch.cu -- ocl_gb300_batch_*: many drop-cutter jobs (each its own mesh,
// cutter and point set, of any size) run together.
//
// Jobs are cut into chunks of at most `chunk_points` points; chunks are
// packed into waves whose workspace (sorted points, candidate lists, bull
// edge plans) fits the budget.  A wave runs the drop pipeline once for all
// its chunks: one radix sort orders every chunk's points (job index above
// the Morton key), then each stage is one persistent launch per kernel
// variant in which blocks take 128-point tiles of any job in turn through an
// atomic counter (work stealing), so a 1,000-point job and a 4,000,000-point
// job share the GPU instead of queueing launch after launch.  The screen
// variants of different cutters are independent and run as parallel
// branches.  The whole run (all waves) is captured once into a CUDA graph
// and replayed.  An autotuner picks, per screen variant, the candidate-list
// capacity and the persistent grid size by timing a probe wave.
//
// Every job's result is the same, bit for bit, as ocl_gb300_drop_device's
// for that job (the same kernels' code on the same inputs; the order of the
// points and the list capacity only decide how work is divided).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "drop.cuh"
#include "screen.cuh"
#include "util.cuh"

namespace oclg {

int make_cutter_params(const ocl_gb300_cutter& in, CutterP& cp);

namespace {

constexpr int SMS = 152;  // persistent grids are sized for the GB300's SM count

// Screen kernel family of a cutter: the basic kinds, or a composite make-up.
struct Variant {
    int kind;  // OCL_CUTTER_CYL .. OCL_CUTTER_CONE, or OCL_CUTTER_COMPOSITE
    int sig;   // composite: comp_sig of a three-part preset, -1 any other
    bool operator<(const Variant& o) const { return kind != o.kind ? kind < o.kind : sig < o.sig; }
    bool operator==(const Variant& o) const { return kind == o.kind && sig == o.sig; }
};

Variant variant_of(const CutterP& cp) {
    if (cp.kind == OCL_CUTTER_COMPOSITE)
        return {OCL_CUTTER_COMPOSITE, cp.nsub == 3 ? comp_sig(cp.sub[0].kind, cp.sub[1].kind, cp.sub[2].kind) : -1};
    return {cp.kind == OCL_CUTTER_CONE ? OCL_CUTTER_CONE : cp.b.kind, 0};
}

struct VariantConf {
    int cap = CAND_K;  // candidates per point
    int grid_mult = 1; // persistent screen grid = blocks per SM x SMs x grid_mult
};

struct SubJob {  // one chunk of a caller job
    int job;
    Mesh* mesh;
    CutterP cp;
    Variant v;
    const double* d_cl;
    uint64_t M;
    double* d_z;
    double* d_cc;
    int32_t* d_type;
    bool bull() const { return cp.kind == OCL_CUTTER_BULL && mesh->n < (1ull << 30); }
    bool composite() const { return cp.kind == OCL_CUTTER_COMPOSITE; }
};

// One stage launch over tiles or over jobs.
struct Launch {
    int kind;     // LaunchKind
    Variant v;    // screen launches
    size_t tile0 = 0, ntiles = 0;  // range in the wave's tile array
    size_t job0 = 0, njobs = 0;    // range in the wave's job-list array
    int counter = -1;              // tile counter index
    unsigned blocks = 1;
    bool flag = false;             // refine: bull plan; exact: composite
};
enum LaunchKind { L_SEED, L_DENSE, L_SPARSE, L_BULL, L_REFINE, L_COLLECT, L_EXACT, L_PLAIN };

struct Wave {
    std::vector<int> sub;  // sub-jobs in this wave
    uint64_t points = 0;
    int end_bit = 32;
    size_t sort_bytes = 0;
    // byte offsets of the wave's tables in the batch's arena: job contexts,
    // inputs, tiles and job lists of the launches
    size_t off_ctx = 0, off_in = 0, off_tiles = 0, off_jobs = 0;
    std::vector<Launch> launches;
    std::vector<std::vector<size_t>> chains;  // screen variant chains (indices into launches)
    int ncounters = 0;
    size_t cand_entries = 0, bull_points = 0;
};

unsigned bits_for(uint64_t n) {
    unsigned b = 0;
    while ((1ull << b) < n) ++b;
    return b;
}

}  // namespace

struct Batch {
    std::vector<SubJob> subs;
    std::map<Variant, VariantConf> conf;
    uint64_t budget = 8ull << 30;
    uint64_t chunk = 1ull << 20;
    bool use_graph = true;
    std::vector<Wave> waves;
    // workspace shared by the waves (sized for the largest)
    DevBuf<unsigned long long> keys, keys2, counters;
    DevBuf<uint32_t> idx, idx2, perm, cand, list, list2, sparse, edge_slots;
    DevBuf<double> cls;
    DevBuf<float> cand_hi, cand_lo, blo;
    DevBuf<uint16_t> ncand;
    DevBuf<uint8_t> edge_n, sort_tmp;
    DevBuf<EdgeRes> edge_res;
    DevBuf<uint2> edge_queue;
    DevBuf<unsigned> tile_counters;
    DevBuf<unsigned char> arena;       // every wave's tables (grow-only)
    DevBuf<unsigned char> exact_scratch;  // handed-back points with many candidates
    std::vector<unsigned char> blob;   // host image of the arena
    size_t max_counters = 0;
    std::vector<cudaStream_t> side;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> joins;
    cudaGraphExec_t exec = nullptr;
    uint64_t launches_per_run = 0;
    uint64_t workspace_bytes = 0;
    uint64_t context = 0;
    ~Batch();
};

Batch::~Batch() {
    if (exec) cudaGraphExecDestroy(exec);
    for (cudaStream_t s : side) cudaStreamDestroy(s);
    if (fork) cudaEventDestroy(fork);
    for (cudaEvent_t e : joins) cudaEventDestroy(e);
}

namespace {

// Workspace bytes of a set of sub-jobs (the largest wave sizes the buffers).
uint64_t wave_bytes(const Batch& b, uint64_t points, uint64_t cand_entries, uint64_t bull_points, size_t njobs) {
    const uint64_t per_point = 2 * 8 + 2 * 4 + 24 + 4 + 2 + 4 + 2 * 4;  // keys, idx, cls, perm, ncand, blo, lists
    const uint64_t bull = bull_points * EDGE_SLOTS * (4 + sizeof(EdgeRes) + sizeof(uint2)) + bull_points;
    (void)b;
    return points * per_point + cand_entries * 12 + bull + (points / 32 + njobs) * 4 +
           njobs * (C_NCOUNTERS + 1) * 8;
}

// Cut jobs into waves in job order under the budget.
int plan_waves(Batch& b) {
    b.waves.clear();
    Wave cur;
    uint64_t cand = 0, bullp = 0;
    auto flush = [&]() {
        if (!cur.sub.empty()) {
            cur.cand_entries = cand;
            cur.bull_points = bullp;
            b.waves.push_back(std::move(cur));
        }
        cur = Wave();
        cand = bullp = 0;
    };
    for (size_t k = 0; k < b.subs.size(); ++k) {
        const SubJob& s = b.subs[k];
        const uint64_t c = s.M * (uint64_t)b.conf[s.v].cap;
        const uint64_t bp = s.bull() ? s.M : 0;
        if (!cur.sub.empty() &&
            wave_bytes(b, cur.points + s.M, cand + c, bullp + bp, cur.sub.size() + 1) > b.budget)
            flush();
        if (wave_bytes(b, s.M, c, bp, 1) > b.budget) {
            set_error("batch: one chunk of " + std::to_string(s.M) + " points needs more workspace than the budget");
            return OCL_GB300_BAD_ARG;
        }
        cur.sub.push_back((int)k);
        cur.points += s.M;
        cand += c;
        bullp += bp;
    }
    flush();
    return OCL_GB300_OK;
}

unsigned blocks_for(size_t work, unsigned per_sm) {
    const size_t cap = (size_t)SMS * per_sm;
    return (unsigned)std::max<size_t>(1, std::min(work, cap));
}

// Device arrays of one wave: contexts (each job's slice of the workspace),
// inputs, tiles and job lists of every launch.
int build_wave(Batch& b, Wave& w) {
    const size_t J = w.sub.size();
    std::vector<DropCtx> ctx(J);
    std::vector<BatchIn> in(J);
    uint64_t off = 0, cand_off = 0, bull_off = 0, sparse_off = 0;
    for (size_t j = 0; j < J; ++j) {
        const SubJob& s = b.subs[w.sub[j]];
        DropCtx& h = ctx[j];
        init_drop_ctx(*s.mesh, s.cp, h);
        h.cl = b.cls.p + 3 * off;
        h.perm = b.perm.p + off;
        h.M = (int)s.M;
        h.out_z = s.d_z;
        h.out_cc = s.d_cc;
        h.out_type = s.d_type;
        h.cand_cap = b.conf[s.v].cap;
        h.cand = b.cand.p + cand_off;
        h.cand_hi = b.cand_hi.p + cand_off;
        h.cand_lo = b.cand_lo.p + cand_off;
        h.ncand = b.ncand.p + off;
        h.blo = b.blo.p + off;
        h.sparse_list = b.sparse.p + sparse_off;
        h.counters = b.counters.p + (size_t)w.sub[j] * (C_NCOUNTERS + 1);
        h.sparse_n = h.counters + C_SPARSE;
        h.list = b.list.p + off;
        h.list2 = b.list2.p + off;
        if (s.bull()) {
            h.edge_slots = b.edge_slots.p + bull_off * EDGE_SLOTS;
            h.edge_n = b.edge_n.p + bull_off;
            h.edge_res = b.edge_res.p + bull_off * EDGE_SLOTS;
            h.edge_queue = b.edge_queue.p + bull_off * EDGE_SLOTS;
            bull_off += s.M;
        }
        const Mesh& m = *s.mesh;
        const double ex = std::max(m.bb[1] - m.bb[0], 1e-9), ey = std::max(m.bb[3] - m.bb[2], 1e-9);
        in[j].cl = s.d_cl;
        in[j].off = off;
        in[j].M = s.M;
        in[j].x0 = m.bb[0] - s.cp.radius;
        in[j].y0 = m.bb[2] - s.cp.radius;
        in[j].sx = 65535.0 / (ex + 2 * s.cp.radius);
        in[j].sy = 65535.0 / (ey + 2 * s.cp.radius);
        off += s.M;
        cand_off += s.M * (uint64_t)h.cand_cap;
        sparse_off += s.M / 32 + 1;
    }
    // tiles and job lists per launch
    std::vector<uint2> tiles;
    std::vector<uint32_t> jl;
    auto tiles_of = [&](auto pred) {
        const size_t t0 = tiles.size();
        for (size_t j = 0; j < J; ++j)
            if (pred(b.subs[w.sub[j]]))
                for (uint32_t t = 0; t < (uint32_t)((b.subs[w.sub[j]].M + TILE_POINTS - 1) / TILE_POINTS); ++t)
                    tiles.push_back(make_uint2((uint32_t)j, t));
        return std::make_pair(t0, tiles.size() - t0);
    };
    auto jobs_of = [&](auto pred) {
        const size_t j0 = jl.size();
        for (size_t j = 0; j < J; ++j)
            if (pred(b.subs[w.sub[j]])) jl.push_back((uint32_t)j);
        return std::make_pair(j0, jl.size() - j0);
    };
    w.launches.clear();
    w.chains.clear();
    int counter = 0;
    std::vector<Variant> vs;
    for (int k : w.sub)
        if (std::find(vs.begin(), vs.end(), b.subs[k].v) == vs.end()) vs.push_back(b.subs[k].v);
    for (const Variant& v : vs) {
        const VariantConf& c = b.conf[v];
        auto same = [&](const SubJob& s) { return s.v == v; };
        auto tr = tiles_of(same);
        auto jr = jobs_of(same);
        const unsigned per_sm = (unsigned)screen_min_blocks(v.kind == OCL_CUTTER_CONE ? 1 : (v.kind == OCL_CUTTER_COMPOSITE ? 2 : 0), 0);
        std::vector<size_t> chain;
        Launch L;
        L.v = v;
        L.kind = L_SEED;
        L.tile0 = tr.first;
        L.ntiles = tr.second;
        L.counter = counter++;
        L.blocks = blocks_for(tr.second, 8);
        chain.push_back(w.launches.size());
        w.launches.push_back(L);
        L.kind = L_DENSE;
        L.counter = counter++;
        L.blocks = blocks_for(tr.second, per_sm * c.grid_mult);
        chain.push_back(w.launches.size());
        w.launches.push_back(L);
        L.kind = L_SPARSE;
        L.counter = -1;
        L.job0 = jr.first;
        L.njobs = jr.second;
        L.blocks = (unsigned)SMS * 4;
        chain.push_back(w.launches.size());
        w.launches.push_back(L);
        w.chains.push_back(chain);
    }
    {
        auto isbull = [](const SubJob& s) { return s.bull(); };
        auto tr = tiles_of(isbull);
        auto jr = jobs_of(isbull);
        if (tr.second) {
            Launch L;
            L.kind = L_BULL;
            L.tile0 = tr.first;
            L.ntiles = tr.second;
            L.job0 = jr.first;
            L.njobs = jr.second;
            L.counter = counter++;
            L.blocks = blocks_for(tr.second, 16);
            w.launches.push_back(L);
            Launch R = L;
            R.kind = L_REFINE;
            R.flag = true;
            R.counter = counter++;
            w.launches.push_back(R);
        }
        auto notbull = [](const SubJob& s) { return !s.bull(); };
        auto tn = tiles_of(notbull);
        if (tn.second) {
            Launch R;
            R.kind = L_REFINE;
            R.flag = false;
            R.tile0 = tn.first;
            R.ntiles = tn.second;
            R.counter = counter++;
            R.blocks = blocks_for(tn.second, 16);
            w.launches.push_back(R);
        }
    }
    {
        auto all = [](const SubJob&) { return true; };
        auto ta = tiles_of(all);
        auto ja = jobs_of(all);
        Launch C;
        C.kind = L_COLLECT;
        C.tile0 = ta.first;
        C.ntiles = ta.second;
        C.counter = counter++;
        C.blocks = blocks_for(ta.second, 16);
        w.launches.push_back(C);
        for (int comp = 0; comp < 2; ++comp) {
            auto pick = [comp](const SubJob& s) { return s.composite() == (comp == 1); };
            auto jr = jobs_of(pick);
            if (!jr.second) continue;
            Launch E;
            E.kind = L_EXACT;
            E.flag = comp == 1;
            E.job0 = jr.first;
            E.njobs = jr.second;
            E.blocks = (unsigned)SMS * 3;
            w.launches.push_back(E);
        }
        Launch P;
        P.kind = L_PLAIN;
        P.job0 = ja.first;
        P.njobs = ja.second;
        P.blocks = (unsigned)SMS * 16;
        w.launches.push_back(P);
    }
    w.ncounters = counter;
    w.end_bit = 32 + (int)bits_for(J);
    w.sort_bytes = batch_sort_bytes(w.points, w.end_bit);
    // the tables go into the host image of the arena (256-byte aligned parts)
    auto put = [&](const void* src, size_t bytes) {
        const size_t off = (b.blob.size() + 255) & ~(size_t)255;
        b.blob.resize(off + std::max<size_t>(bytes, 1));
        if (bytes) std::memcpy(b.blob.data() + off, src, bytes);
        return off;
    };
    w.off_ctx = put(ctx.data(), J * sizeof(DropCtx));
    w.off_in = put(in.data(), J * sizeof(BatchIn));
    w.off_tiles = put(tiles.data(), tiles.size() * sizeof(uint2));
    w.off_jobs = put(jl.data(), jl.size() * sizeof(uint32_t));
    return OCL_GB300_OK;
}

int alloc_workspace(Batch& b) {
    uint64_t P = 0, C = 0, Bp = 0, S = 0, Jm = 0, sortb = 0;
    int ncnt = 0;
    (void)Jm;
    for (const Wave& w : b.waves) {
        P = std::max(P, w.points);
        C = std::max<uint64_t>(C, w.cand_entries);
        Bp = std::max<uint64_t>(Bp, w.bull_points);
        Jm = std::max<uint64_t>(Jm, w.sub.size());
        uint64_t sp = 0;
        for (int k : w.sub) sp += b.subs[k].M / 32 + 1;
        S = std::max(S, sp);
        const int end_bit = 32 + (int)bits_for(w.sub.size());
        sortb = std::max<uint64_t>(sortb, batch_sort_bytes(w.points, end_bit));
    }
    ncnt = 2 * 16 + 8;
    if (!b.keys.reserve(P) || !b.keys2.reserve(P) || !b.idx.reserve(P) || !b.idx2.reserve(P) ||
        !b.cls.reserve(3 * P) || !b.perm.reserve(P) || !b.cand.reserve(C) || !b.cand_hi.reserve(C) ||
        !b.cand_lo.reserve(C) || !b.ncand.reserve(P) || !b.blo.reserve(P) || !b.list.reserve(P) ||
        !b.list2.reserve(P) || !b.sparse.reserve(std::max<uint64_t>(S, 1)) ||
        !b.counters.reserve(b.subs.size() * (C_NCOUNTERS + 1)) || !b.sort_tmp.reserve(std::max<uint64_t>(sortb, 1)) ||
        !b.tile_counters.reserve(ncnt))
        return OCL_GB300_OOM;
    // the exact kernel's scratch only when it is a small part of the budget
    // (without it, points with very many candidates take the plain kernel)
    if (b.budget >= 4 * batch_exact_scratch_bytes() && !b.exact_scratch.reserve(batch_exact_scratch_bytes()))
        return OCL_GB300_OOM;
    if (Bp && (!b.edge_slots.reserve(Bp * EDGE_SLOTS) || !b.edge_n.reserve(Bp) ||
               !b.edge_res.reserve(Bp * EDGE_SLOTS) || !b.edge_queue.reserve(Bp * EDGE_SLOTS)))
        return OCL_GB300_OOM;
    b.max_counters = (size_t)ncnt;
    b.workspace_bytes = P * (2 * 8 + 2 * 4 + 24 + 4 + 2 + 4 + 2 * 4) + C * 12 + S * 4 + sortb + b.exact_scratch.n +
                        Bp * EDGE_SLOTS * (4 + sizeof(EdgeRes) + sizeof(uint2)) + Bp;
    return OCL_GB300_OK;
}

BatchView view_of(const Batch& b, const Wave& w, const Launch& L) {
    BatchView v;
    v.ctxs = reinterpret_cast<const DropCtx*>(b.arena.p + w.off_ctx);
    v.tiles = reinterpret_cast<const uint2*>(b.arena.p + w.off_tiles) + L.tile0;
    v.ntiles = (unsigned)L.ntiles;
    v.next = L.counter >= 0 ? b.tile_counters.p + L.counter : nullptr;
    v.jobs = reinterpret_cast<const uint32_t*>(b.arena.p + w.off_jobs) + L.job0;
    v.njobs = (unsigned)L.njobs;
    return v;
}

void launch_screen_stage(const BatchView& v, const Variant& var, unsigned blocks, cudaStream_t s, int stage) {
    if (var.kind != OCL_CUTTER_COMPOSITE) {
        if (stage == 1) screen_launch_basic_dense_b(v, var.kind, blocks, s);
        else screen_launch_basic_b(v, var.kind, blocks, s, stage);
        return;
    }
    if (stage == 1) {
        if (!screen_launch_comp_a_dense_b(v, var.sig, blocks, s) && !screen_launch_comp_b_dense_b(v, var.sig, blocks, s))
            screen_launch_comp_any_dense_b(v, blocks, s);
    } else {
        if (!screen_launch_comp_a_b(v, var.sig, blocks, s, stage) && !screen_launch_comp_b_b(v, var.sig, blocks, s, stage))
            screen_launch_comp_any_b(v, blocks, s, stage);
    }
}

// All waves on `stream` (screen chains of different variants on side
// streams, joined before the FP64 stages).
int enqueue(Batch& b, cudaStream_t stream, uint64_t* launches) {
    uint64_t n = 0;
    for (Wave& w : b.waves) {
        // this wave's chunks are consecutive: their counter slices are one range
        CK(cudaMemsetAsync(b.counters.p + (size_t)w.sub.front() * (C_NCOUNTERS + 1), 0,
                           w.sub.size() * (C_NCOUNTERS + 1) * sizeof(unsigned long long), stream));
        CK(cudaMemsetAsync(b.tile_counters.p, 0, (size_t)w.ncounters * sizeof(unsigned), stream));
        int st = OCL_GB300_OK;
        batch_launch_order(reinterpret_cast<const BatchIn*>(b.arena.p + w.off_in), (uint32_t)w.sub.size(), w.points, b.keys.p, b.idx.p, b.keys2.p, b.idx2.p,
                           b.sort_tmp.p, b.sort_tmp.n, w.end_bit, b.cls.p, b.perm.p, stream, &st);
        if (st) return st;
        n += 2 + 4;  // Morton, gather, the sort's passes
        // screen chains: parallel branches when more than one variant
        const bool fan = w.chains.size() > 1 && !b.side.empty();
        if (fan) CK(cudaEventRecord(b.fork, stream));
        for (size_t c = 0; c < w.chains.size(); ++c) {
            cudaStream_t s = fan ? b.side[c % b.side.size()] : stream;
            if (fan) CK(cudaStreamWaitEvent(s, b.fork, 0));
            for (size_t li : w.chains[c]) {
                const Launch& L = w.launches[li];
                if (L.kind == L_SPARSE && L.njobs == 0) continue;
                if ((L.kind == L_SEED || L.kind == L_DENSE) && L.ntiles == 0) continue;
                launch_screen_stage(view_of(b, w, L), L.v, L.blocks, s, L.kind == L_SEED ? 0 : (L.kind == L_DENSE ? 1 : 2));
                ++n;
            }
            if (fan) {
                CK(cudaEventRecord(b.joins[c % b.joins.size()], s));
                CK(cudaStreamWaitEvent(stream, b.joins[c % b.joins.size()], 0));
            }
        }
        for (const Launch& L : w.launches) {
            const BatchView v = view_of(b, w, L);
            switch (L.kind) {
            case L_BULL: {
                BatchView ev = v;
                batch_launch_bull(v, ev, L.blocks, stream);
                n += 2;
                break;
            }
            case L_REFINE:
                if (L.ntiles) {
                    batch_launch_refine(v, L.flag, L.blocks, stream);
                    ++n;
                }
                break;
            case L_COLLECT:
                batch_launch_collect(v, L.blocks, stream);
                ++n;
                break;
            case L_EXACT: {
                int st2 = batch_launch_exact(v, L.flag, L.blocks, stream, b.exact_scratch.p);
                if (st2) return st2;
                ++n;
                break;
            }
            case L_PLAIN:
                batch_launch_plain(v, L.blocks, stream);
                ++n;
                break;
            default:
                break;
            }
        }
        CK(cudaGetLastError());
    }
    if (launches) *launches = n;
    return OCL_GB300_OK;
}

int make_subjobs(Batch& b, const ocl_gb300_drop_job* jobs, Mesh* const* meshes, uint64_t njobs) {
    b.subs.clear();
    for (uint64_t k = 0; k < njobs; ++k) {
        const ocl_gb300_drop_job& j = jobs[k];
        if (!meshes[k]) {
            set_error("batch: job " + std::to_string(k) + " has no mesh");
            return OCL_GB300_BAD_ARG;
        }
        if (j.M > 0 && (!j.d_cl_xyz || !j.d_z_out || !j.d_cc_out || !j.d_type_out)) {
            set_error("batch: job " + std::to_string(k) + " has a null buffer");
            return OCL_GB300_BAD_ARG;
        }
        CutterP cp;
        const int st = make_cutter_params(j.cutter, cp);
        if (st) {
            set_error("batch: job " + std::to_string(k) + ": invalid cutter");
            return st;
        }
        Mesh* m = meshes[k];
        if (m->n == 0 && j.M > 0) {
            set_error("batch: job " + std::to_string(k) + ": empty mesh (use ocl_gb300_drop_device)");
            return OCL_GB300_BAD_ARG;
        }
        for (uint64_t o = 0; o < j.M; o += b.chunk) {
            SubJob s;
            s.job = (int)k;
            s.mesh = m;
            s.cp = cp;
            s.v = variant_of(cp);
            s.M = std::min<uint64_t>(b.chunk, j.M - o);
            s.d_cl = j.d_cl_xyz + 3 * o;
            s.d_z = j.d_z_out + o;
            s.d_cc = j.d_cc_out + 3 * o;
            s.d_type = j.d_type_out + o;
            b.subs.push_back(s);
            b.conf[s.v];
        }
    }
    return OCL_GB300_OK;
}

// Waves, workspace (grown only) and the arena's tables, copied on `stream`
// (ordered before the run that uses them; no device-wide synchronisation).
int prepare(Batch& b, cudaStream_t stream) {
    int st = plan_waves(b);
    if (st) return st;
    st = alloc_workspace(b);
    if (st) return st;
    b.blob.clear();
    for (Wave& w : b.waves) {
        st = build_wave(b, w);
        if (st) return st;
    }
    if (!b.arena.reserve(b.blob.size())) return OCL_GB300_OOM;
    CK(cudaMemcpyAsync(b.arena.p, b.blob.data(), b.blob.size(), cudaMemcpyHostToDevice, stream));
    return OCL_GB300_OK;
}

// Candidate-list capacity and screen grid size per variant, timed on a
// probe: the middle 4,096 points of up to 32 chunks of the variant, each
// configuration run twice (the second run timed).  Lists of 64 are not
// tried: the probe's contiguous middles miss the regions whose lists
// overflow (flat faces, fans of thin triangles), and on the 64-job workload
// 64-entry lists handed back 1.36M points instead of 0.30M.
int autotune(Batch& b, const std::vector<SubJob>& all, cudaStream_t stream) {
    const int caps[2] = {128, 256};
    const int mults[2] = {1, 2};
    std::vector<Variant> vs;
    for (const SubJob& s : all)
        if (std::find(vs.begin(), vs.end(), s.v) == vs.end()) vs.push_back(s.v);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int status = OCL_GB300_OK;
    for (const Variant& v : vs) {
        Batch probe;
        probe.budget = b.budget;
        probe.chunk = b.chunk;
        // the middle 4,096 points of at most 32 chunks of the variant
        for (const SubJob& s : all)
            if (s.v == v && probe.subs.size() < 32) {
                SubJob q = s;
                q.M = std::min<uint64_t>(q.M, 4096);
                const uint64_t off = (s.M - q.M) / 2;
                q.d_cl += 3 * off;
                q.d_z += off;
                q.d_cc += 3 * off;
                q.d_type += off;
                probe.subs.push_back(q);
            }
        float best = 1e30f;
        VariantConf pick;
        for (int cap : caps)
            for (int mult : mults) {
                probe.conf[v] = VariantConf{cap, mult};
                status = prepare(probe, stream);
                if (status) break;
                float t = 0.0f;
                for (int rep = 0; rep < 2 && !status; ++rep) {
                    if (cudaEventRecord(e0, stream) != cudaSuccess) status = OCL_GB300_DEVICE_ERROR;
                    if (!status) status = enqueue(probe, stream, nullptr);
                    if (!status && cudaEventRecord(e1, stream) != cudaSuccess) status = OCL_GB300_DEVICE_ERROR;
                    if (!status && cudaEventSynchronize(e1) != cudaSuccess) status = OCL_GB300_DEVICE_ERROR;
                    float ms = 0.0f;
                    if (!status) cudaEventElapsedTime(&ms, e0, e1);
                    if (rep > 0) t += ms;  // rep 0 warms up
                }
                if (status) break;
                if (t < best) {
                    best = t;
                    pick = VariantConf{cap, mult};
                }
            }
        if (status) break;
        b.conf[v] = pick;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return status;
}

}  // namespace

int batch_create(const ocl_gb300_drop_job* jobs, Mesh* const* meshes, uint64_t njobs, const ocl_gb300_batch_opts* opts,
                 Batch** out) {
    *out = nullptr;
    Batch* b = new Batch();
    int list_cap = CAND_K;
    bool tune = false;
    if (opts) {
        if (opts->workspace_bytes) b->budget = opts->workspace_bytes;
        if (opts->chunk_points) b->chunk = opts->chunk_points;
        b->use_graph = opts->graph != 0;
        tune = opts->autotune != 0;
        if (opts->list_capacity) list_cap = opts->list_capacity;
    }
    if (list_cap < 16 || list_cap > CAND_K || b->chunk >= (1ull << 31) || b->chunk == 0) {
        delete b;
        set_error("batch: list capacity must be in [16, 256] and chunks below 2^31 points");
        return OCL_GB300_BAD_ARG;
    }
    b->context = context_key();
    int st = make_subjobs(*b, jobs, meshes, njobs);
    if (!st) st = ensure_exact_smem();  // before any capture
    for (auto& kv : b->conf) kv.second.cap = list_cap;
    if (!st && tune && !b->subs.empty()) {
        cudaStream_t s;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
            st = OCL_GB300_DEVICE_ERROR;
        } else {
            const std::vector<SubJob> all = b->subs;
            st = autotune(*b, all, s);
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }
    if (!st) {
        st = prepare(*b, 0);
        if (!st && cudaStreamSynchronize(0) != cudaSuccess) st = OCL_GB300_DEVICE_ERROR;
    }
    if (!st) {
        for (int k = 0; k < 4; ++k) {
            cudaStream_t s;
            if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
                st = OCL_GB300_DEVICE_ERROR;
                break;
            }
            b->side.push_back(s);
            cudaEvent_t e;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
                st = OCL_GB300_DEVICE_ERROR;
                break;
            }
            b->joins.push_back(e);
        }
        if (!st && cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) st = OCL_GB300_DEVICE_ERROR;
    }
    if (st) {
        delete b;
        return st;
    }
    *out = b;
    return OCL_GB300_OK;
}

int batch_run(Batch& b, cudaStream_t stream, ocl_gb300_stats* stats) {
    if (b.subs.empty()) {
        if (stats) std::memset(stats, 0, sizeof(*stats));
        return OCL_GB300_OK;
    }
    if (context_key() != b.context) {
        set_error("batch: run on another device or context than it was made on");
        return OCL_GB300_BAD_ARG;
    }
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        CK(cudaEventCreate(&t0));
        CK(cudaEventCreate(&t1));
        CK(cudaEventRecord(t0, stream));
    }
    int st = OCL_GB300_OK;
    if (b.use_graph) {
        // captured once (on the first run's stream), replayed after
        if (!b.exec) {
            cudaStream_t cap;
            CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
            st = enqueue(b, cap, &b.launches_per_run);
            cudaGraph_t g = nullptr;
            const cudaError_t e = cudaStreamEndCapture(cap, &g);
            cudaStreamDestroy(cap);
            if (!st && e != cudaSuccess) {
                set_error(std::string("batch graph capture: ") + cudaGetErrorString(e));
                st = OCL_GB300_DEVICE_ERROR;
            }
            if (!st && cudaGraphInstantiate(&b.exec, g, 0) != cudaSuccess) {
                set_error("batch graph instantiation failed");
                st = OCL_GB300_DEVICE_ERROR;
                b.exec = nullptr;
            }
            if (g) cudaGraphDestroy(g);
        }
        if (!st) CK(cudaGraphLaunch(b.exec, stream));
    } else {
        st = enqueue(b, stream, &b.launches_per_run);
    }
    if (st) return st;
    if (stats) {
        CK(cudaEventRecord(t1, stream));
        CK(cudaEventSynchronize(t1));
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, t0, t1);
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        stats->kernel_ms = ms;
        stats->launches = b.launches_per_run;
        // every chunk has its own counter slice
        std::vector<unsigned long long> c(b.subs.size() * (C_NCOUNTERS + 1));
        CK(cudaMemcpy(c.data(), b.counters.p, c.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        for (size_t j = 0; j < b.subs.size(); ++j) {
            const unsigned long long* q = c.data() + j * (C_NCOUNTERS + 1);
            stats->refined += q[C_REFINED];
            stats->iter_limit_hits += q[C_CAPPED];
            stats->fallback += q[C_FALLBACK];
            stats->violations += q[C_VIOLATION];
            stats->screened += q[C_SCREENED];
            stats->overflow_points += q[C_OVERFLOW];
            stats->chain_points += q[C_CHAIN];
            stats->open_branch_points += q[C_OPEN];
            stats->untracked_branch_points += q[C_UNTRACKED];
            stats->plain_points += q[C_PLAIN];
            stats->verify_failed_points += q[C_VFAIL];
        }
    }
    return OCL_GB300_OK;
}

void batch_info(const Batch& b, ocl_gb300_batch_info* out) {
    std::memset(out, 0, sizeof(*out));
    out->jobs = 0;
    for (const SubJob& s : b.subs) out->jobs = std::max<uint64_t>(out->jobs, (uint64_t)s.job + 1);
    out->chunks = b.subs.size();
    out->waves = b.waves.size();
    out->launches_per_run = b.launches_per_run;
    out->workspace_bytes = b.workspace_bytes;
    int k = 0;
    for (const auto& kv : b.conf) {
        if (k >= OCL_GB300_BATCH_MAX_VARIANTS) break;
        out->variant_kind[k] = kv.first.kind;
        out->variant_sig[k] = kv.first.sig;
        out->list_capacity[k] = kv.second.cap;
        out->grid_mult[k] = kv.second.grid_mult;
        ++k;
    }
    out->variants = k;
    for (const Wave& w : b.waves) out->points += w.points;
}

void batch_destroy(Batch* b) { delete b; }

Batch* batch_new(uint64_t workspace_bytes, uint64_t chunk_points, int list_capacity) {
    Batch* b = new Batch();
    if (workspace_bytes) b->budget = workspace_bytes;
    if (chunk_points) b->chunk = chunk_points;
    b->use_graph = false;
    b->context = context_key();
    (void)list_capacity;
    return b;
}

// New jobs on an existing batch: planned on the host, the workspace grown
// only where it is too small, the tables copied on `stream`.  The batch must
// not be running (its previous run on `stream` is ordered before).
int batch_reset(Batch& b, const ocl_gb300_drop_job* jobs, Mesh* const* meshes, uint64_t njobs, int list_capacity,
                cudaStream_t stream) {
    if (b.exec) {
        cudaGraphExecDestroy(b.exec);
        b.exec = nullptr;
    }
    b.use_graph = false;
    int st = make_subjobs(b, jobs, meshes, njobs);
    if (st) return st;
    for (auto& kv : b.conf) kv.second.cap = list_capacity > 0 ? list_capacity : CAND_K;
    st = ensure_exact_smem();
    if (st) return st;
    return prepare(b, stream);
}

}  // namespace oclg
