// mesh.cu -- ocl_gb300_mesh_create: triangle records, KD visit order and the
// device-built uniform XY grid that the drop kernels stream from.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include <cub/cub.cuh>

#include "mesh.cuh"
#include "util.cuh"

namespace oclg {

// ---------------------------------------------------------------------------
// Host: per-triangle FP64 records with the reference's arithmetic
// (Triangle::calcNormal / upNormal triangle.cpp:65-75, Bbox::addPoint
// bbox.cpp:67-89, MillingCutter::facetDrop's derived normal values).
// This file is compiled with -ffp-contract=off so the doubles match.
// ---------------------------------------------------------------------------
static inline bool zero_tol_h(double x) { return std::fabs(x) < 0.0000001; }

static void make_tri64(const double* v, Tri64& t, uint32_t& flags) {
    std::memcpy(t.p, v, 9 * sizeof(double));
    double v1x = v[0] - v[3], v1y = v[1] - v[4], v1z = v[2] - v[5];
    double v2x = v[0] - v[6], v2y = v[1] - v[7], v2z = v[2] - v[8];
    double nx = v1y * v2z - v1z * v2y;
    double ny = v1z * v2x - v1x * v2z;
    double nz = v1x * v2y - v1y * v2x;
    double nrm = std::sqrt(nx * nx + ny * ny + nz * nz);
    if (nrm != 0.0) {
        double s = 1 / nrm;
        nx = nx * s; ny = ny * s; nz = nz * s;
    }
    if (nz < 0) { nx = nx * -1.0; ny = ny * -1.0; nz = nz * -1.0; }
    t.n[0] = nx; t.n[1] = ny; t.n[2] = nz;
    double mn[3] = {v[0], v[1], v[2]}, mx[3] = {v[0], v[1], v[2]};
    for (int k = 1; k < 3; ++k)
        for (int a = 0; a < 3; ++a) {
            double q = v[3 * k + a];
            if (q > mx[a]) mx[a] = q;
            if (q < mn[a]) mn[a] = q;
        }
    t.bb[0] = mn[0]; t.bb[1] = mx[0]; t.bb[2] = mn[1]; t.bb[3] = mx[1]; t.bb[4] = mn[2]; t.bb[5] = mx[2];
    t.d = -(nx * v[0] + ny * v[1] + nz * v[2]);
    double n2 = std::sqrt(nx * nx + ny * ny + nz * nz);
    double ax = nx, ay = ny, az = nz;
    if (n2 != 0.0) {
        double s = 1 / n2;
        ax = ax * s; ay = ay * s; az = az * s;
    }
    t.nn[0] = ax; t.nn[1] = ay; t.nn[2] = az;
    double xl = std::sqrt(ax * ax + ay * ay);
    double bx = ax, by = ay;
    if (xl != 0.0) {
        double s = 1 / std::sqrt(ax * ax + ay * ay);
        bx = bx * s; by = by * s;
    }
    t.xyn[0] = bx; t.xyn[1] = by;
    flags = 0;
    if (zero_tol_h(nz)) flags |= TF_FACET_NONE;
    else if (zero_tol_h(nx) && zero_tol_h(ny)) flags |= TF_FACET_HORIZ;
    else flags |= TF_FACET_GENERAL;
    for (int e = 0; e < 3; ++e) {
        const double* p1 = v + 3 * e;
        const double* p2 = v + 3 * ((e + 1) % 3);
        if (zero_tol_h(p1[0] - p2[0]) && zero_tol_h(p1[1] - p2[1])) flags |= (TF_EDGE0_SKIP << e);
        if (zero_tol_h(p1[2] - p2[2])) flags |= (TF_EDGE0_HORIZ << e);
    }
}

// ---------------------------------------------------------------------------
// KD-tree with the reference's splits (KDTree::build_node kdtree.hpp:141-210,
// calc_spread :213-268): spread over four bbox dimensions, cut at the middle
// of the largest spread, bbox[d] > cut goes to the hi child, a bucket when
// size <= bucketSize or the spread is below 1e-7.  Built iteratively (hi child
// first) so the leaf sequence is the reference's visit order.
// ---------------------------------------------------------------------------
void kd_build_host(const std::vector<double>& bb6, uint64_t n, unsigned bucket, int dims, KDTreeD& out) {
    static const int D[3][4] = {{0, 1, 2, 3}, {2, 3, 4, 5}, {0, 1, 4, 5}};
    const int* dm = D[dims];
    out.nodes.clear();
    out.order.clear();
    out.max_depth = 0;
    if (n == 0) return;
    if (bucket == 0) bucket = 1;
    std::vector<int32_t> idx(n), tmp(n);
    std::iota(idx.begin(), idx.end(), 0);
    struct Task {
        int64_t b, e;
        int32_t parent;
        bool is_hi;
        int depth;
    };
    std::vector<Task> stack;
    stack.push_back({0, (int64_t)n, -1, false, 0});
    out.order.reserve(n);
    while (!stack.empty()) {
        Task tk = stack.back();
        stack.pop_back();
        double maxv[6], minv[6];
        bool first = true;
        for (int64_t i = tk.b; i < tk.e; ++i) {
            const double* bb = &bb6[6 * (size_t)idx[i]];
            for (int m = 0; m < 4; ++m) {
                int d = dm[m];
                double v = bb[d];
                if (first) {
                    maxv[d] = v;
                    minv[d] = v;
                    if (m == 3) first = false;
                } else {
                    if (maxv[d] < v) maxv[d] = v;
                    if (minv[d] > v) minv[d] = v;
                }
            }
        }
        double mxs = 0;
        int maxM = 0;
        for (int m = 0; m < 4; ++m) {
            double val = maxv[dm[m]] - minv[dm[m]];
            if (val > mxs) { mxs = val; maxM = m; }
        }
        int sd = dm[maxM];
        double sval = maxv[sd] - minv[sd];
        double cut = minv[sd] + sval / 2;
        int32_t id = (int32_t)out.nodes.size();
        KDNodeD nd;
        nd.dim = sd;
        nd.cut = cut;
        nd.hi = nd.lo = -1;
        nd.leaf_begin = nd.leaf_end = -1;
        nd.pad = 0;
        out.nodes.push_back(nd);
        if (tk.parent >= 0) {
            if (tk.is_hi) out.nodes[tk.parent].hi = id;
            else out.nodes[tk.parent].lo = id;
        }
        out.max_depth = std::max(out.max_depth, tk.depth);
        int64_t cnt = tk.e - tk.b;
        if ((uint64_t)cnt <= bucket || zero_tol_h(sval)) {
            out.nodes[id].leaf_begin = (int32_t)out.order.size();
            for (int64_t i = tk.b; i < tk.e; ++i) out.order.push_back(idx[i]);
            out.nodes[id].leaf_end = (int32_t)out.order.size();
            continue;
        }
        int64_t nhi = 0;
        for (int64_t i = tk.b; i < tk.e; ++i)
            if (bb6[6 * (size_t)idx[i] + sd] > cut) tmp[tk.b + nhi++] = idx[i];
        int64_t w = tk.b + nhi;
        for (int64_t i = tk.b; i < tk.e; ++i)
            if (!(bb6[6 * (size_t)idx[i] + sd] > cut)) tmp[w++] = idx[i];
        std::copy(tmp.begin() + tk.b, tmp.begin() + tk.e, idx.begin() + tk.b);
        // lo pushed first so the hi subtree is visited first
        if (tk.e - (tk.b + nhi) > 0) stack.push_back({tk.b + nhi, tk.e, id, false, tk.depth + 1});
        if (nhi > 0) stack.push_back({tk.b, tk.b + nhi, id, true, tk.depth + 1});
    }
}

// ---------------------------------------------------------------------------
// Multi-level grid.  Host: level and home cell of every triangle (this fixes
// the device order of the triangles: sorted by (level, home cell)).  Device:
// entries (FP32 bboxes rounded outward) and per-cell bounds over the cell's
// own triangles (union bbox, max z), from the sorted cell keys.
// ---------------------------------------------------------------------------
static void grid_params(Mesh& M, const std::vector<Tri64>& t64, GridP& g) {
    const uint64_t n = M.n;
    double ex = std::max(M.bb[1] - M.bb[0], 1e-9), ey = std::max(M.bb[3] - M.bb[2], 1e-9);
    // finest cell: 1.25 x the 90th percentile of the triangles' xy extent,
    // at least half the mean spacing, at most 4096 cells per axis
    std::vector<double> ext(n);
    for (uint64_t i = 0; i < n; ++i) ext[i] = std::max(t64[i].bb[1] - t64[i].bb[0], t64[i].bb[3] - t64[i].bb[2]);
    double p90 = 0.0;
    if (n > 0) {
        size_t k = (size_t)(0.9 * (double)(n - 1));
        std::nth_element(ext.begin(), ext.begin() + k, ext.end());
        p90 = ext[k];
    }
    double cs = std::max(1.25 * p90, 0.5 * std::sqrt(ex * ey / (double)std::max<uint64_t>(n, 1)));
    cs = std::max(cs, std::max(ex, ey) / 4096.0);
    cs = std::max(cs, 1e-9);
    g.x0 = M.bb[0];
    g.y0 = M.bb[2];
    g.ox = 0.5 * (M.bb[0] + M.bb[1]);
    g.oy = 0.5 * (M.bb[2] + M.bb[3]);
    g.oz = 0.5 * (M.bb[4] + M.bb[5]);
    g.nlev = 0;
    uint32_t off = 0;
    for (int L = 0; L < GRID_MAX_LEVELS; ++L) {
        g.cs[L] = cs;
        g.inv_cs[L] = 1.0 / cs;
        g.ncol[L] = (int)std::floor(ex / cs) + 1;
        g.nrow[L] = (int)std::floor(ey / cs) + 1;
        g.cell_off[L] = off;
        off += (uint32_t)g.ncol[L] * (uint32_t)g.nrow[L];
        g.nlev = L + 1;
        if (g.ncol[L] == 1 && g.nrow[L] == 1) break;
        cs *= 4.0;
    }
    g.cell_off[g.nlev] = off;
}

// level and global home-cell index of one triangle
static uint32_t grid_key(const GridP& g, const double* bb) {
    const double dx = bb[1] - bb[0], dy = bb[3] - bb[2];
    int L = 0;
    while (L < g.nlev - 1 && (dx > g.cs[L] || dy > g.cs[L])) ++L;
    int c = std::min(std::max((int)std::floor((bb[0] - g.x0) * g.inv_cs[L]), 0), g.ncol[L] - 1);
    int r = std::min(std::max((int)std::floor((bb[2] - g.y0) * g.inv_cs[L]), 0), g.nrow[L] - 1);
    return g.cell_off[L] + (uint32_t)r * (uint32_t)g.ncol[L] + (uint32_t)c;
}

__device__ __forceinline__ float f_rd(double x) { return __double2float_rd(x); }
__device__ __forceinline__ float f_ru(double x) { return __double2float_ru(x); }

__global__ void k_grid_entries(const Tri64* t, GridP g, const uint32_t* keys, uint64_t n, Entry* ent,
                               uint32_t* cstart, uint32_t* cend) {
    uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double* bb = t[k].bb;
    Entry e;
    e.minx = f_rd(bb[0] - g.ox);
    e.maxx = f_ru(bb[1] - g.ox);
    e.miny = f_rd(bb[2] - g.oy);
    e.maxy = f_ru(bb[3] - g.oy);
    e.maxz = f_ru(bb[5] - g.oz);
    e.tri = (int32_t)k;
    e.pad[0] = e.pad[1] = 0.0f;
    ent[k] = e;
    const uint32_t key = keys[k];
    if (k == 0 || keys[k - 1] != key) cstart[key] = (uint32_t)k;
    if (k == n - 1 || keys[k + 1] != key) cend[key] = (uint32_t)(k + 1);
}

__global__ void k_grid_cells(const Entry* ent, const uint32_t* cstart, const uint32_t* cend, uint32_t ncells,
                             Cell* cells) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    Cell cl;
    cl.start = cstart[c];
    cl.count = cend[c] > cstart[c] ? cend[c] - cstart[c] : 0;
    cl.minx = cl.miny = 3.0e38f;
    cl.maxx = cl.maxy = cl.maxz = -3.0e38f;
    cl.pad = 0;
    for (uint32_t k = 0; k < cl.count; ++k) {
        Entry e = ent[cl.start + k];
        cl.minx = fminf(cl.minx, e.minx);
        cl.maxx = fmaxf(cl.maxx, e.maxx);
        cl.miny = fminf(cl.miny, e.miny);
        cl.maxy = fmaxf(cl.maxy, e.maxy);
        cl.maxz = fmaxf(cl.maxz, e.maxz);
    }
    cells[c] = cl;
}

static int build_grid(Mesh& m, const std::vector<uint32_t>& keys_dev) {
    const uint64_t n = m.n;
    const GridP& g = m.grid;
    const uint32_t ncells = g.cell_off[g.nlev];
    DevBuf<uint32_t> keys(n), cstart(ncells), cend(ncells);
    if (!keys.ok() || !cstart.ok() || !cend.ok()) return OCL_GB300_OOM;
    CK(cudaMemcpy(keys.p, keys_dev.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CK(cudaMemset(cstart.p, 0, ncells * sizeof(uint32_t)));
    CK(cudaMemset(cend.p, 0, ncells * sizeof(uint32_t)));
    if (m.d_entries) cudaFree(m.d_entries);
    if (m.d_cells) cudaFree(m.d_cells);
    m.d_entries = nullptr;
    m.d_cells = nullptr;
    CK(cudaMalloc(&m.d_entries, std::max<uint64_t>(n, 1) * sizeof(Entry)));
    CK(cudaMalloc(&m.d_cells, (size_t)ncells * sizeof(Cell)));
    const int TB = 256;
    k_grid_entries<<<(unsigned)((n + TB - 1) / TB), TB>>>(m.d_t64, g, keys.p, n, m.d_entries, cstart.p, cend.p);
    k_grid_cells<<<(ncells + TB - 1) / TB, TB>>>(m.d_entries, cstart.p, cend.p, ncells, m.d_cells);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    m.nentries = n;
    return OCL_GB300_OK;
}

// Upload a KD tree with its leaf order translated to device triangle ids.
int upload_kd(Mesh& M, const KDTreeD& kd, PushIndex& out) {
    std::vector<int32_t> ord(kd.order.size());
    for (size_t k = 0; k < ord.size(); ++k) ord[k] = M.ins_to_dev[kd.order[k]];
    out.nnodes = (int)kd.nodes.size();
    out.max_depth = kd.max_depth;
    if (out.max_depth > KD_STACK - 2) {
        set_error("KD tree deeper than the device traversal stack");
        return OCL_GB300_ITER_LIMIT;
    }
    CK(cudaMalloc(&out.d_nodes, std::max<size_t>(kd.nodes.size(), 1) * sizeof(KDNodeD)));
    CK(cudaMalloc(&out.d_order, std::max<size_t>(ord.size(), 1) * sizeof(int32_t)));
    if (!kd.nodes.empty())
        CK(cudaMemcpy(out.d_nodes, kd.nodes.data(), kd.nodes.size() * sizeof(KDNodeD), cudaMemcpyHostToDevice));
    {
        // FP32 copies of the cuts, rounded both ways (a walk in FP32 that
        // prunes only where both roundings agree visits every leaf the FP64
        // walk visits)
        std::vector<float2> c32(std::max<size_t>(kd.nodes.size(), 1));
        for (size_t k = 0; k < kd.nodes.size(); ++k) {
            const double c = kd.nodes[k].cut;
            float lo = (float)c, hi = (float)c;
            if ((double)lo > c) lo = std::nextafter(lo, -3.0e38f);
            if ((double)hi < c) hi = std::nextafter(hi, 3.0e38f);
            c32[k] = make_float2(lo, hi);
        }
        CK(cudaMalloc(&out.d_cut32, c32.size() * sizeof(float2)));
        CK(cudaMemcpy(out.d_cut32, c32.data(), c32.size() * sizeof(float2), cudaMemcpyHostToDevice));
    }
    if (!ord.empty())
        CK(cudaMemcpy(out.d_order, ord.data(), ord.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    out.built = true;
    return OCL_GB300_OK;
}

int mesh_create(const double* tris, uint64_t n, unsigned bucket, Mesh** out) {
    *out = nullptr;
    if (n > 0 && !tris) {
        set_error("null triangle array");
        return OCL_GB300_BAD_ARG;
    }
    if (n >= (1ull << 31)) {
        set_error("too many triangles");
        return OCL_GB300_BAD_ARG;
    }
    for (uint64_t i = 0; i < 9 * n; ++i)
        if (!std::isfinite(tris[i])) {
            set_error("non-finite triangle coordinate");
            return OCL_GB300_BAD_ARG;
        }
    Mesh* m = new Mesh();
    m->n = n;
    m->bucket = bucket ? bucket : 1;
    std::vector<Tri64> t64(n);
    std::vector<uint32_t> flags(n);
    m->host_bb.resize(6 * n);
    for (uint64_t i = 0; i < n; ++i) {
        make_tri64(tris + 9 * i, t64[i], flags[i]);
        std::memcpy(&m->host_bb[6 * i], t64[i].bb, 6 * sizeof(double));
        if (i == 0) {
            std::memcpy(m->bb, t64[i].bb, sizeof(m->bb));
        } else {
            for (int a = 0; a < 3; ++a) {
                m->bb[2 * a] = std::min(m->bb[2 * a], t64[i].bb[2 * a]);
                m->bb[2 * a + 1] = std::max(m->bb[2 * a + 1], t64[i].bb[2 * a + 1]);
            }
        }
    }
    // KD visit order of the drop-cutter tree (XY dimensions)
    KDTreeD kd;
    kd_build_host(m->host_bb, n, m->bucket, 0, kd);
    std::vector<uint32_t> kd_rank(n);
    for (uint64_t r = 0; r < kd.order.size(); ++r) kd_rank[kd.order[r]] = (uint32_t)r;

    // grid parameters decide the device order: sorted by (level, home cell)
    Mesh& M = *m;
    grid_params(M, t64, M.grid);
    std::vector<uint32_t> key(n);
    for (uint64_t i = 0; i < n; ++i) key[i] = grid_key(M.grid, t64[i].bb);
    M.dev_to_ins.resize(n);
    std::iota(M.dev_to_ins.begin(), M.dev_to_ins.end(), 0);
    std::stable_sort(M.dev_to_ins.begin(), M.dev_to_ins.end(),
                     [&](int32_t a, int32_t b) { return key[a] < key[b]; });
    M.ins_to_dev.resize(n);
    for (uint64_t d = 0; d < n; ++d) M.ins_to_dev[M.dev_to_ins[d]] = (int32_t)d;
    std::vector<uint32_t> key_dev(n);
    for (uint64_t d = 0; d < n; ++d) key_dev[d] = key[M.dev_to_ins[d]];

    double ox = 0.5 * (M.bb[0] + M.bb[1]), oy = 0.5 * (M.bb[2] + M.bb[3]), oz = 0.5 * (M.bb[4] + M.bb[5]);
    std::vector<Tri64> t64d(n);
    std::vector<Tri32> t32d(n);
    for (uint64_t d = 0; d < n; ++d) {
        uint64_t i = (uint64_t)M.dev_to_ins[d];
        const Tri64& t = t64[i];
        t64d[d] = t;
        Tri32& s = t32d[d];
        s.v0[0] = (float)(t.p[0] - ox);
        s.v0[1] = (float)(t.p[1] - oy);
        s.v0[2] = (float)(t.p[2] - oz);
        for (int a = 0; a < 3; ++a) {
            s.e1[a] = (float)(t.p[3 + a] - t.p[a]);
            s.e2[a] = (float)(t.p[6 + a] - t.p[a]);
            s.nn[a] = (float)t.nn[a];
        }
        s.flags = flags[i];
        s.kd_rank = kd_rank[i];
        double e1x = t.p[3] - t.p[0], e1y = t.p[4] - t.p[1], e2x = t.p[6] - t.p[0], e2y = t.p[7] - t.p[1];
        double det = std::fabs(e1x * e2y - e1y * e2x);
        double l0 = std::hypot(e1x, e1y), l1 = std::hypot(e2x, e2y), l2 = std::hypot(e2x - e1x, e2y - e1y);
        double lmax = std::max(l0, std::max(l1, l2));
        double bs = det > 0 ? lmax / det : 3.0e38;
        s.bary_scale = (float)std::min(bs, 3.0e38);
        s.pad = 0.0f;
    }
    int st = OCL_GB300_OK;
    if (n > 0) {
        if (cudaMalloc(&M.d_t64, n * sizeof(Tri64)) != cudaSuccess || cudaMalloc(&M.d_t32, n * sizeof(Tri32)) != cudaSuccess) {
            set_error("cudaMalloc failed for the mesh");
            delete m;
            return OCL_GB300_OOM;
        }
        if (cudaMemcpy(M.d_t64, t64d.data(), n * sizeof(Tri64), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(M.d_t32, t32d.data(), n * sizeof(Tri32), cudaMemcpyHostToDevice) != cudaSuccess) {
            set_error("mesh upload failed");
            delete m;
            return OCL_GB300_DEVICE_ERROR;
        }
        st = build_grid(M, key_dev);
        if (st != OCL_GB300_OK) {
            delete m;
            return st;
        }
        st = upload_kd(M, kd, M.drop_kd);
        if (st != OCL_GB300_OK) {
            delete m;
            return st;
        }
    }
    *out = m;
    return OCL_GB300_OK;
}

void mesh_destroy(Mesh* m) {
    if (!m) return;
    cudaFree(m->d_t64);
    cudaFree(m->d_t32);
    cudaFree(m->d_cells);
    cudaFree(m->d_entries);
    for (int k = 0; k < 2; ++k) {
        cudaFree(m->push[k].d_nodes);
        cudaFree(m->push[k].d_order);
        cudaFree(m->push[k].d_cut32);
    }
    cudaFree(m->drop_kd.d_nodes);
    cudaFree(m->drop_kd.d_order);
    cudaFree(m->drop_kd.d_cut32);
    cudaFree(m->d_edge_sin);
    delete m;
}

// BullCutter's push through an edge (src/cutters/bullcutter.cpp:131-132)
// takes theta = atan(dz / xyNorm(p2 - p1)) and sin(theta): a value of the
// edge alone, computed here with the host's atan and sin so that it is the
// reference's double (the device's atan and sin can differ in the last bit).
int ensure_edge_sin(Mesh& m) {
    if (m.d_edge_sin || m.n == 0) return OCL_GB300_OK;
    std::vector<Tri64> t(m.n);
    CK(cudaMemcpy(t.data(), m.d_t64, m.n * sizeof(Tri64), cudaMemcpyDeviceToHost));
    std::vector<double> s(3 * m.n);
    for (uint64_t i = 0; i < m.n; ++i)
        for (int k = 0; k < 3; ++k) {
            const double* p1 = &t[i].p[3 * k];
            const double* p2 = &t[i].p[3 * ((k + 1) % 3)];
            const double dx = p2[0] - p1[0], dy = p2[1] - p1[1], dz = p2[2] - p1[2];
            const double xy = std::sqrt(dx * dx + dy * dy);
            s[3 * i + k] = std::sin(std::atan(dz / xy));
        }
    double* d = nullptr;
    if (cudaMalloc(&d, s.size() * sizeof(double)) != cudaSuccess) {
        set_error("edge slopes: device allocation failed");
        return OCL_GB300_OOM;
    }
    if (cudaMemcpy(d, s.data(), s.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        set_error("edge slopes: copy failed");
        return OCL_GB300_DEVICE_ERROR;
    }
    m.d_edge_sin = d;
    return OCL_GB300_OK;
}

}  // namespace oclg
