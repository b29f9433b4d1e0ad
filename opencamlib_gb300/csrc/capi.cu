// capi.cu -- the extern "C" entry points declared in include/ocl_gb300.h,
// cutter parameter derivation and error reporting.
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "drop.cuh"
#include "geom64.cuh"
#include "mesh.cuh"
#include "util.cuh"
#include "waterline.cuh"

namespace oclg {

static thread_local std::string tl_error;
std::string& last_error_ref() { return tl_error; }
void set_error(const std::string& msg) { tl_error = msg; }

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points
// (no link against the driver library).
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

uint64_t context_key() {
    static std::once_flag once;
    static CtxGetCurrentFn get_cur = nullptr;
    static CtxGetIdFn get_id = nullptr;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
    });
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
        return 0;
    }
    if (get_cur && get_id) {
        void* ctx = nullptr;
        unsigned long long id = 0;
        // the runtime makes the device's primary context current lazily;
        // cudaSetDevice does it now
        if (get_cur(&ctx) == 0 && !ctx && cudaSetDevice(dev) == cudaSuccess) get_cur(&ctx);
        if (ctx && get_id(ctx, &id) == 0) return (uint64_t)id | (1ull << 63);
    }
    return (uint64_t)dev + 1;
}

int mesh_create(const double* tris, uint64_t n, unsigned bucket, Mesh** out);
void mesh_destroy(Mesh* m);
int push_run(Mesh& m, const CutterP& cp, int dir, const double* fibers, uint64_t F, uint64_t* offsets, double* ival,
             double* cc, int32_t* cctype, uint64_t cap, ocl_gb300_stats* stats);
int path_drop_run(Mesh& m, const CutterP& cp, const double* spans, uint64_t S, double sampling, double min_z,
                  double* xyz, double* cc, int32_t* type, uint64_t cap, uint64_t* count, ocl_gb300_stats* stats);
int adaptive_path_drop_run(Mesh& m, const CutterP& cp, const double* spans, uint64_t S, double sampling,
                           double min_sampling, double cos_limit, double* xyz, double* cc, int32_t* type,
                           uint64_t cap, uint64_t* count, ocl_gb300_stats* stats);
int mesh_kd_order(Mesh& m, int dims, int64_t* order);
int mesh_kd_rank(Mesh& m, int64_t* rank);
int overlap_sets(Mesh& m, double radius, const double* cl, uint64_t M, uint64_t* offsets, int32_t* ids,
                 uint64_t cap);
int certificate_check(Mesh& m, const CutterP& cp, const double* cl, uint64_t M, ocl_gb300_cert* out);

// Constructors of the basic cutters (cylcutter.cpp:39-46, ballcutter.cpp:38-45,
// bullcutter.cpp:38-47, conecutter.cpp:39-49); compiled with
// -ffp-contract=off, so derived lengths equal the reference's doubles.
static int make_basic(const ocl_gb300_subcutter& s, BasicP& b) {
    std::memset(&b, 0, sizeof(b));
    b.kind = s.kind;
    const double d = s.diameter, l = s.length;
    if (!(d > 0.0) || !std::isfinite(d) || !std::isfinite(l)) return OCL_GB300_BAD_ARG;
    switch (s.kind) {
    case OCL_CUTTER_CYL:
        if (!(l > 0.0)) return OCL_GB300_BAD_ARG;
        b.diameter = d; b.radius = d / 2.0; b.length = l;
        b.xy_normal_length = b.radius; b.normal_length = 0.0; b.center_height = 0.0;
        return OCL_GB300_OK;
    case OCL_CUTTER_BALL:
        if (!(l > 0.0)) return OCL_GB300_BAD_ARG;
        b.diameter = d; b.radius = d / 2.0; b.length = l;
        b.normal_length = b.radius; b.xy_normal_length = 0.0; b.center_height = b.radius;
        return OCL_GB300_OK;
    case OCL_CUTTER_BULL:
        if (!(l > 0.0) || !(s.corner_radius > 0.0) || !(d / 2.0 - s.corner_radius > 0.0)) return OCL_GB300_BAD_ARG;
        b.diameter = d; b.radius = d / 2.0; b.radius1 = d / 2.0 - s.corner_radius; b.radius2 = s.corner_radius;
        b.length = l; b.xy_normal_length = b.radius1; b.normal_length = b.radius2; b.center_height = b.radius2;
        return OCL_GB300_OK;
    case OCL_CUTTER_CONE:
        if (!(s.angle > 0.0) || !(s.angle < 1.5707963267948966)) return OCL_GB300_BAD_ARG;
        b.diameter = d; b.radius = d / 2.0; b.angle = s.angle; b.tan_angle = std::tan(s.angle);
        b.length = b.radius / std::tan(b.angle) + l;
        b.center_height = b.radius / std::tan(b.angle);
        b.xy_normal_length = b.radius; b.normal_length = 0.0;
        return OCL_GB300_OK;
    }
    return OCL_GB300_UNSUPPORTED_CUTTER;
}

int make_cutter_params(const ocl_gb300_cutter& in, CutterP& cp) {
    std::memset(&cp, 0, sizeof(cp));
    cp.kind = in.kind;
    if (in.kind != OCL_CUTTER_COMPOSITE) {
        int st = make_basic(in.base, cp.b);
        if (st) return st;
        cp.radius = cp.b.radius;
        cp.length = cp.b.length;
        return OCL_GB300_OK;
    }
    // CompositeCutter::addCutter (compositecutter.cpp:43-51)
    if (in.nsub < 1 || in.nsub > OCL_GB300_MAX_SUB) return OCL_GB300_BAD_ARG;
    cp.nsub = in.nsub;
    cp.radius = 0;
    for (int n = 0; n < in.nsub; ++n) {
        int st = make_basic(in.sub[n], cp.sub[n]);
        if (st) return st;
        cp.radiusvec[n] = in.sub[n].radius;
        cp.heightvec[n] = in.sub[n].height;
        cp.zoffset[n] = in.sub[n].zoffset;
        if (in.sub[n].radius > cp.radius) cp.radius = in.sub[n].radius;
    }
    if (!(cp.radius > 0.0)) return OCL_GB300_BAD_ARG;
    cp.length = in.composite_length;
    return OCL_GB300_OK;
}

static double height_basic_host(const BasicP& c, double r) {
    switch (c.kind) {
    case OCL_CUTTER_CYL: return (r <= c.radius) ? 0.0 : -1.0;
    case OCL_CUTTER_BALL: return c.radius - std::sqrt(c.radius * c.radius - r * r);
    case OCL_CUTTER_BULL:
        if (r <= c.radius1) return 0.0;
        if (r <= c.radius) return c.radius2 - std::sqrt(c.radius2 * c.radius2 - (r - c.radius1) * (r - c.radius1));
        return -1;
    case OCL_CUTTER_CONE: return r / c.tan_angle;
    }
    return -1;
}

double height_host(const CutterP& c, double r) {
    if (c.kind != OCL_CUTTER_COMPOSITE) return height_basic_host(c.b, r);
    int idx = 0;
    for (int n = 0; n < c.nsub; ++n) {
        double lo = (n == 0) ? -1E-6 : c.radiusvec[n - 1] - 1E-6;
        double hi = c.radiusvec[n] + 1e-6;
        if (lo <= r && r <= hi) { idx = n; break; }
    }
    return height_basic_host(c.sub[idx], r) + c.zoffset[idx];
}

static void basic_prof(const BasicP& b, Prof32& prof) {
    std::memset(&prof, 0, sizeof(prof));
    prof.kind = b.kind;
    prof.R = (float)b.radius;
    prof.r1 = (float)b.radius1;
    prof.r2 = (float)b.radius2;
    prof.inv_tan = b.kind == OCL_CUTTER_CONE ? (float)(1.0 / b.tan_angle) : 0.0f;
    prof.center_height = (float)b.center_height;
    prof.length = (float)b.length;
    prof.xynl = (float)b.xy_normal_length;
    prof.nl = (float)b.normal_length;
}

void fill_comp(const CutterP& cp, Comp32& comp) {
    std::memset(&comp, 0, sizeof(comp));
    if (cp.kind != OCL_CUTTER_COMPOSITE) return;
    comp.nsub = cp.nsub;
    comp.R = (float)cp.radius;
    for (int n = 0; n < cp.nsub; ++n) {
        basic_prof(cp.sub[n], comp.sub[n]);
        comp.zoff[n] = (float)cp.zoffset[n];
        comp.rlim[n] = (float)cp.radiusvec[n];
        // CompositeCutter::ccValidRadius (compositecutter.cpp:86-102) bounds
        const double lo = (n == 0) ? -1E-6 : cp.radiusvec[n - 1] - 1E-6;
        const double hi = cp.radiusvec[n] + 1e-6;
        float f = (float)lo;
        comp.wlo_in[n] = ((double)f >= lo) ? f : std::nextafter(f, 3.0e38f);
        comp.wlo_out[n] = ((double)f <= lo) ? f : std::nextafter(f, -3.0e38f);
        f = (float)hi;
        comp.whi_in[n] = ((double)f <= hi) ? f : std::nextafter(f, -3.0e38f);
        comp.whi_out[n] = ((double)f >= hi) ? f : std::nextafter(f, 3.0e38f);
    }
}

void fill_prof(const CutterP& cp, Prof32& prof, float* hlb, bool& composite) {
    std::memset(&prof, 0, sizeof(prof));
    composite = cp.kind == OCL_CUTTER_COMPOSITE;
    const BasicP& b = cp.b;
    if (!composite) basic_prof(b, prof);
    prof.R = (float)cp.radius;
    // hlb[k] <= min over r in [k R / N, R] of height(r), built from the top
    // down with dense samples per bin, minus a small margin.
    const double R = cp.radius;
    double run = 1e300;
    for (int k = HLB_N - 1; k >= 0; --k) {
        double r0 = R * k / HLB_N, r1 = R * (k + 1) / HLB_N;
        for (int s = 0; s <= 16; ++s) {
            double r = r0 + (r1 - r0) * s / 16.0;
            if (r > R) r = R;
            double h = height_host(cp, r);
            if (cp.kind == OCL_CUTTER_CYL || (cp.kind != OCL_CUTTER_COMPOSITE && b.kind == OCL_CUTTER_CYL)) h = 0.0;
            if (std::isfinite(h)) run = std::min(run, h);
        }
        double v = run - 1e-6 * (1.0 + R);
        hlb[k] = (float)std::nextafter((float)v, -3.0e38f);
    }
}

}  // namespace oclg

using namespace oclg;

struct ocl_gb300_mesh_s {
    Mesh* m;
};

extern "C" {

int ocl_gb300_stage_times(uint64_t count, double* out) {
    if (count && !out) {
        set_error("stage times: null output");
        return OCL_GB300_BAD_ARG;
    }
    return drop_stage_times(count, out);
}

const char* ocl_gb300_last_error(void) { return tl_error.c_str(); }
const char* ocl_gb300_version(void) { return "opencamlib_gb300 0.1 (sm_103a)"; }

int ocl_gb300_device_available(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n > 0 ? 1 : 0;
}

static int need_device() {
    if (!ocl_gb300_device_available()) {
        set_error("no CUDA device available");
        return OCL_GB300_NO_DEVICE;
    }
    return OCL_GB300_OK;
}

int ocl_gb300_mesh_create(const double* tris, uint64_t ntri, uint32_t bucket_size, ocl_gb300_mesh* out) {
    if (!out) {
        set_error("null output handle");
        return OCL_GB300_BAD_ARG;
    }
    *out = nullptr;
    int st = need_device();
    if (st) return st;
    Mesh* m = nullptr;
    st = mesh_create(tris, ntri, bucket_size, &m);
    if (st) return st;
    *out = new ocl_gb300_mesh_s{m};
    return OCL_GB300_OK;
}

int ocl_gb300_mesh_release(ocl_gb300_mesh mesh) {
    if (!mesh) return OCL_GB300_BAD_ARG;
    mesh_destroy(mesh->m);
    delete mesh;
    return OCL_GB300_OK;
}

uint64_t ocl_gb300_mesh_size(ocl_gb300_mesh mesh) { return mesh ? mesh->m->n : 0; }

int ocl_gb300_mesh_bbox(ocl_gb300_mesh mesh, double bb[6]) {
    if (!mesh || !bb) return OCL_GB300_BAD_ARG;
    std::memcpy(bb, mesh->m->bb, 6 * sizeof(double));
    return OCL_GB300_OK;
}

int ocl_gb300_drop_device(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, const double* d_cl_xyz, uint64_t M,
                          int precision, double* d_z_out, double* d_cc_out, int32_t* d_type_out, void* stream,
                          ocl_gb300_stats* stats) {
    if (!mesh || !cutter) {
        set_error("null mesh or cutter");
        return OCL_GB300_BAD_ARG;
    }
    if (M > 0 && (!d_cl_xyz || !d_z_out || !d_cc_out || !d_type_out)) {
        set_error("null buffer");
        return OCL_GB300_BAD_ARG;
    }
    if (precision != OCL_GB300_PREC_FP64 && precision != OCL_GB300_PREC_MIXED) {
        set_error("unknown precision mode");
        return OCL_GB300_BAD_ARG;
    }
    CutterP cp;
    int st = make_cutter_params(*cutter, cp);
    if (st) {
        set_error(st == OCL_GB300_UNSUPPORTED_CUTTER ? "unsupported cutter kind" : "invalid cutter parameters");
        return st;
    }
    std::lock_guard<std::mutex> lk(mesh->m->mu);
    if (stats) std::memset(stats, 0, sizeof(*stats));
    return drop_run(*mesh->m, cp, d_cl_xyz, M, precision, d_z_out, d_cc_out, d_type_out, (cudaStream_t)stream, stats);
}

int ocl_gb300_drop_device_noalloc(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, const double* d_cl_xyz,
                                  uint64_t M, double* d_z_out, double* d_cc_out, int32_t* d_type_out, void* stream) {
    if (!mesh || !cutter) {
        set_error("null mesh or cutter");
        return OCL_GB300_BAD_ARG;
    }
    if (M > 0 && (!d_cl_xyz || !d_z_out || !d_cc_out || !d_type_out)) {
        set_error("null buffer");
        return OCL_GB300_BAD_ARG;
    }
    CutterP cp;
    int st = make_cutter_params(*cutter, cp);
    if (st) {
        set_error(st == OCL_GB300_UNSUPPORTED_CUTTER ? "unsupported cutter kind" : "invalid cutter parameters");
        return st;
    }
    std::lock_guard<std::mutex> lk(mesh->m->mu);
    return drop_run_noalloc(*mesh->m, cp, d_cl_xyz, M, d_z_out, d_cc_out, d_type_out, (cudaStream_t)stream);
}

int ocl_gb300_drop(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, const double* cl_xyz, uint64_t M,
                   int precision, double* z_out, double* cc_out, int32_t* type_out, ocl_gb300_stats* stats) {
    auto t0 = std::chrono::steady_clock::now();
    if (M == 0) {
        if (stats) std::memset(stats, 0, sizeof(*stats));
        return mesh && cutter ? OCL_GB300_OK : OCL_GB300_BAD_ARG;
    }
    if (!cl_xyz || !z_out || !cc_out || !type_out) {
        set_error("null buffer");
        return OCL_GB300_BAD_ARG;
    }
    // device staging buffers, grown on demand and kept per host thread
    struct HostIO {
        DevBuf<double> cl, z, cc;
        DevBuf<int32_t> ty;
        size_t cap = 0;
    };
    static thread_local HostIO io;
    if (M > io.cap) {
        if (!io.cl.alloc(3 * M) || !io.z.alloc(M) || !io.cc.alloc(3 * M) || !io.ty.alloc(M)) {
            io.cap = 0;
            return OCL_GB300_OOM;
        }
        io.cap = M;
    }
    DevBuf<double>& dcl = io.cl;
    DevBuf<double>& dz = io.z;
    DevBuf<double>& dcc = io.cc;
    DevBuf<int32_t>& dty = io.ty;
    cudaStream_t s = 0;
    CK(cudaMemcpyAsync(dcl.p, cl_xyz, 3 * M * sizeof(double), cudaMemcpyHostToDevice, s));
    int st = ocl_gb300_drop_device(mesh, cutter, dcl.p, M, precision, dz.p, dcc.p, dty.p, s, stats);
    if (st) return st;
    CK(cudaMemcpyAsync(z_out, dz.p, M * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(cc_out, dcc.p, 3 * M * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(type_out, dty.p, M * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (stats)
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return OCL_GB300_OK;
}

static int cutter_or_error(const ocl_gb300_cutter* cutter, CutterP& cp) {
    if (!cutter) {
        set_error("null cutter");
        return OCL_GB300_BAD_ARG;
    }
    int st = make_cutter_params(*cutter, cp);
    if (st) set_error(st == OCL_GB300_UNSUPPORTED_CUTTER ? "unsupported cutter kind" : "invalid cutter parameters");
    return st;
}

int ocl_gb300_push(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, int dir, const double* fibers, uint64_t F,
                   uint64_t* offsets, double* ival, double* cc, int32_t* cctype, uint64_t cap,
                   ocl_gb300_stats* stats) {
    auto t0 = std::chrono::steady_clock::now();
    if (!mesh || !offsets || (F > 0 && !fibers) || (cap > 0 && (!ival || !cc || !cctype))) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    if (dir != OCL_GB300_XFIBER && dir != OCL_GB300_YFIBER) {
        set_error("dir must be OCL_GB300_XFIBER or OCL_GB300_YFIBER");
        return OCL_GB300_BAD_ARG;
    }
    CutterP cp;
    int st = cutter_or_error(cutter, cp);
    if (st) return st;
    std::lock_guard<std::mutex> lk(mesh->m->mu);
    st = push_run(*mesh->m, cp, dir, fibers, F, offsets, ival, cc, cctype, cap, stats);
    if (stats)
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return st;
}

int ocl_gb300_path_drop(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, const double* spans, uint64_t S,
                        double sampling, double min_z, double* xyz, double* cc, int32_t* type, uint64_t cap,
                        uint64_t* count, ocl_gb300_stats* stats) {
    auto t0 = std::chrono::steady_clock::now();
    if (!mesh || !count || (S > 0 && !spans) || (cap > 0 && (!xyz || !cc || !type))) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    CutterP cp;
    int st = cutter_or_error(cutter, cp);
    if (st) return st;
    std::lock_guard<std::mutex> lk(mesh->m->mu);
    st = path_drop_run(*mesh->m, cp, spans, S, sampling, min_z, xyz, cc, type, cap, count, stats);
    if (stats)
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return st;
}

int ocl_gb300_adaptive_path_drop(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, const double* spans,
                                 uint64_t S, double sampling, double min_sampling, double cos_limit, double* xyz,
                                 double* cc, int32_t* type, uint64_t cap, uint64_t* count, ocl_gb300_stats* stats) {
    auto t0 = std::chrono::steady_clock::now();
    if (!mesh || !count || (S > 0 && !spans) || (cap > 0 && (!xyz || !cc || !type))) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    CutterP cp;
    int st = cutter_or_error(cutter, cp);
    if (st) return st;
    std::lock_guard<std::mutex> lk(mesh->m->mu);
    st = adaptive_path_drop_run(*mesh->m, cp, spans, S, sampling, min_sampling, cos_limit, xyz, cc, type, cap, count,
                                stats);
    if (stats)
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return st;
}

int ocl_gb300_mesh_kd_order(ocl_gb300_mesh mesh, int dims, int64_t* order) {
    if (!mesh || (!order && mesh->m->n)) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(mesh->m->mu);
    return mesh_kd_order(*mesh->m, dims, order);
}

int ocl_gb300_mesh_kd_rank(ocl_gb300_mesh mesh, int64_t* rank) {
    if (!mesh || (!rank && mesh->m->n)) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(mesh->m->mu);
    return mesh_kd_rank(*mesh->m, rank);
}

int ocl_gb300_overlap_sets(ocl_gb300_mesh mesh, double radius, const double* cl_xyz, uint64_t M, uint64_t* offsets,
                           int32_t* ids, uint64_t cap) {
    if (!mesh || !offsets || (M > 0 && !cl_xyz) || (cap > 0 && !ids)) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(mesh->m->mu);
    return overlap_sets(*mesh->m, radius, cl_xyz, M, offsets, ids, cap);
}

int ocl_gb300_certificate_check(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, const double* cl_xyz,
                                uint64_t M, ocl_gb300_cert* out) {
    if (!mesh || !out || (M > 0 && !cl_xyz)) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    CutterP cp;
    int st = cutter_or_error(cutter, cp);
    if (st) return st;
    std::lock_guard<std::mutex> lk(mesh->m->mu);
    return certificate_check(*mesh->m, cp, cl_xyz, M, out);
}

struct ocl_gb300_batch_s {
    Batch* b;
};

int ocl_gb300_batch_create(const ocl_gb300_drop_job* jobs, uint64_t njobs, const ocl_gb300_batch_opts* opts,
                           ocl_gb300_batch* out) {
    if (!out || (njobs > 0 && !jobs)) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    *out = nullptr;
    int st = need_device();
    if (st) return st;
    std::vector<Mesh*> meshes(njobs);
    for (uint64_t k = 0; k < njobs; ++k) meshes[k] = jobs[k].mesh ? jobs[k].mesh->m : nullptr;
    Batch* b = nullptr;
    st = batch_create(jobs, meshes.data(), njobs, opts, &b);
    if (st) return st;
    *out = new ocl_gb300_batch_s{b};
    return OCL_GB300_OK;
}

int ocl_gb300_batch_run(ocl_gb300_batch batch, void* stream, ocl_gb300_stats* stats) {
    if (!batch) {
        set_error("null batch");
        return OCL_GB300_BAD_ARG;
    }
    return batch_run(*batch->b, (cudaStream_t)stream, stats);
}

int ocl_gb300_batch_info_get(ocl_gb300_batch batch, ocl_gb300_batch_info* out) {
    if (!batch || !out) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    batch_info(*batch->b, out);
    return OCL_GB300_OK;
}

int ocl_gb300_batch_release(ocl_gb300_batch batch) {
    if (!batch) return OCL_GB300_BAD_ARG;
    batch_destroy(batch->b);
    delete batch;
    return OCL_GB300_OK;
}

struct ocl_gb300_server_s {
    Server* s;
};

int ocl_gb300_server_create(const ocl_gb300_server_opts* opts, ocl_gb300_server* out) {
    if (!out) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    *out = nullptr;
    int st = need_device();
    if (st) return st;
    Server* s = nullptr;
    st = server_create(opts, &s);
    if (st) return st;
    *out = new ocl_gb300_server_s{s};
    return OCL_GB300_OK;
}

int ocl_gb300_server_add_mesh(ocl_gb300_server server, ocl_gb300_mesh mesh, int32_t* mesh_id) {
    if (!server || !mesh || !mesh_id) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    return server_add_mesh(*server->s, mesh->m, mesh_id);
}

int ocl_gb300_server_submit_drop(ocl_gb300_server server, int32_t mesh_id, const ocl_gb300_cutter* cutter,
                                 const double* cl_xyz, uint64_t M, double* z_out, double* cc_out, int32_t* type_out,
                                 uint64_t* request_id) {
    if (!server || !cutter || !request_id || (M > 0 && (!cl_xyz || !z_out || !cc_out || !type_out))) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    return server_submit_drop(*server->s, mesh_id, *cutter, cl_xyz, M, z_out, cc_out, type_out, request_id);
}

int ocl_gb300_server_submit_adaptive(ocl_gb300_server server, int32_t mesh_id, const ocl_gb300_cutter* cutter,
                                     const double* spans, uint64_t S, double sampling, double min_sampling,
                                     double cos_limit, double* xyz_out, double* cc_out, int32_t* type_out,
                                     uint64_t cap, uint64_t* count, uint64_t* request_id) {
    if (!server || !cutter || !request_id || !count || (S > 0 && !spans) ||
        (cap > 0 && (!xyz_out || !cc_out || !type_out))) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    return server_submit_adaptive(*server->s, mesh_id, *cutter, spans, S, sampling, min_sampling, cos_limit, xyz_out,
                                  cc_out, type_out, cap, count, request_id);
}

int ocl_gb300_server_wait(ocl_gb300_server server, uint64_t request_id, double timeout_s,
                          ocl_gb300_request_info* info) {
    if (!server) {
        set_error("null server");
        return OCL_GB300_BAD_ARG;
    }
    return server_wait(*server->s, request_id, timeout_s, info);
}

int ocl_gb300_server_cancel(ocl_gb300_server server, uint64_t request_id) {
    if (!server) {
        set_error("null server");
        return OCL_GB300_BAD_ARG;
    }
    return server_cancel(*server->s, request_id);
}

int ocl_gb300_server_stats_get(ocl_gb300_server server, ocl_gb300_server_stats* out) {
    if (!server || !out) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    return server_stats(*server->s, out);
}

int ocl_gb300_server_pause(ocl_gb300_server server, int32_t paused) {
    if (!server) {
        set_error("null server");
        return OCL_GB300_BAD_ARG;
    }
    return server_pause(*server->s, paused != 0);
}

int ocl_gb300_server_destroy(ocl_gb300_server server) {
    if (!server) return OCL_GB300_BAD_ARG;
    server_destroy(server->s);
    delete server;
    return OCL_GB300_OK;
}

// ---- waterline -------------------------------------------------------------

struct ocl_gb300_loops_s {
    oclg::LoopSet s;
};

static int waterline_common(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, CutterP& cp) {
    if (!mesh) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    return cutter_or_error(cutter, cp);
}

static void total_ms(ocl_gb300_stats* stats, std::chrono::steady_clock::time_point t0) {
    if (stats)
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

int ocl_gb300_waterline_levels(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, const double* zs, uint64_t nz,
                               double sampling, ocl_gb300_loops* out, ocl_gb300_stats* stats) {
    const auto t0 = std::chrono::steady_clock::now();
    if (!out || (nz > 0 && !zs)) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    for (uint64_t k = 0; k < nz; ++k) out[k] = nullptr;
    if (stats) std::memset(stats, 0, sizeof(*stats));
    CutterP cp;
    int st = waterline_common(mesh, cutter, cp);
    if (st) return st;
    std::vector<oclg::LoopSet> sets;
    {
        std::lock_guard<std::mutex> lk(mesh->m->mu);
        st = oclg::waterline_run(*mesh->m, cp, zs, nz, sampling, sets, stats);
    }
    if (st) return st;
    for (uint64_t k = 0; k < nz; ++k) {
        out[k] = new ocl_gb300_loops_s();
        out[k]->s = std::move(sets[k]);
    }
    total_ms(stats, t0);
    return OCL_GB300_OK;
}

int ocl_gb300_waterline(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, double z, double sampling,
                        ocl_gb300_loops* out, ocl_gb300_stats* stats) {
    return ocl_gb300_waterline_levels(mesh, cutter, &z, 1, sampling, out, stats);
}

int ocl_gb300_adaptive_waterline(ocl_gb300_mesh mesh, const ocl_gb300_cutter* cutter, double z, double sampling,
                                 double min_sampling, double cos_limit, ocl_gb300_loops* out,
                                 ocl_gb300_stats* stats) {
    const auto t0 = std::chrono::steady_clock::now();
    if (!out) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    *out = nullptr;
    if (stats) std::memset(stats, 0, sizeof(*stats));
    CutterP cp;
    int st = waterline_common(mesh, cutter, cp);
    if (st) return st;
    auto* h = new ocl_gb300_loops_s();
    {
        std::lock_guard<std::mutex> lk(mesh->m->mu);
        st = oclg::adaptive_waterline_run(*mesh->m, cp, z, sampling, min_sampling, cos_limit, h->s, stats);
    }
    if (st) {
        delete h;
        return st;
    }
    *out = h;
    total_ms(stats, t0);
    return OCL_GB300_OK;
}

static int fibers_in(const double* fib, uint64_t F, const uint64_t* off, const double* iv, int dir,
                     oclg::FiberSet& fs) {
    if (F > 0 && (!fib || !off || (off[F] > 0 && !iv))) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    fs.fib.assign(fib, fib + 6 * F);
    fs.off.assign(1, 0);
    for (uint64_t f = 0; f < F; ++f) {
        const double* p = fib + 6 * f;
        const bool ok = dir == OCL_GB300_XFIBER ? (p[1] == p[4] && p[2] == p[5]) : (p[0] == p[3] && p[2] == p[5]);
        if (!ok || off[f + 1] < off[f]) {
            set_error("weave: fiber " + std::to_string(f) + " is not an axis-parallel fiber of its direction");
            return OCL_GB300_BAD_ARG;
        }
        fs.off.push_back(off[f + 1] - off[0]);
    }
    const uint64_t K = F ? off[F] - off[0] : 0;
    fs.ival.assign(iv ? iv + 2 * off[0] : iv, iv ? iv + 2 * (off[0] + K) : iv);
    fs.cc.assign(6 * K, 0.0);
    fs.type.assign(2 * K, 0);
    return OCL_GB300_OK;
}

int ocl_gb300_weave(const double* xfib, uint64_t nx, const uint64_t* xoff, const double* xival, const double* yfib,
                    uint64_t ny, const uint64_t* yoff, const double* yival, ocl_gb300_loops* out) {
    if (!out) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    *out = nullptr;
    auto* h = new ocl_gb300_loops_s();
    int st = fibers_in(xfib, nx, xoff, xival, OCL_GB300_XFIBER, h->s.fibers[0]);
    if (!st) st = fibers_in(yfib, ny, yoff, yival, OCL_GB300_YFIBER, h->s.fibers[1]);
    if (!st) st = oclg::weave_loops(h->s);
    if (st) {
        delete h;
        return st;
    }
    *out = h;
    return OCL_GB300_OK;
}

int ocl_gb300_loops_count(ocl_gb300_loops loops, uint64_t* nloops, uint64_t* npoints) {
    if (!loops || !nloops || !npoints) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    *nloops = loops->s.off.empty() ? 0 : loops->s.off.size() - 1;
    *npoints = loops->s.pts.size() / 3;
    return OCL_GB300_OK;
}

int ocl_gb300_loops_get(ocl_gb300_loops loops, double* points, uint64_t* offsets) {
    if (!loops || !offsets || (!points && !loops->s.pts.empty())) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    if (!loops->s.pts.empty()) std::memcpy(points, loops->s.pts.data(), loops->s.pts.size() * sizeof(double));
    if (loops->s.off.empty()) offsets[0] = 0;
    else std::memcpy(offsets, loops->s.off.data(), loops->s.off.size() * sizeof(uint64_t));
    return OCL_GB300_OK;
}

int ocl_gb300_loops_fibers(ocl_gb300_loops loops, int dir, uint64_t* nfibers, uint64_t* nintervals, double* fib,
                           uint64_t* offsets, double* ival, double* cc, int32_t* cctype) {
    if (!loops || !nfibers || !nintervals || (dir != OCL_GB300_XFIBER && dir != OCL_GB300_YFIBER)) {
        set_error("bad argument");
        return OCL_GB300_BAD_ARG;
    }
    const oclg::FiberSet& fs = loops->s.fibers[dir];
    *nfibers = fs.count();
    *nintervals = fs.ival.size() / 2;
    if (!fib) return OCL_GB300_OK;
    if (!offsets || (!ival && *nintervals)) {
        set_error("null argument");
        return OCL_GB300_BAD_ARG;
    }
    if (!fs.fib.empty()) std::memcpy(fib, fs.fib.data(), fs.fib.size() * sizeof(double));
    if (fs.off.empty()) offsets[0] = 0;
    else std::memcpy(offsets, fs.off.data(), fs.off.size() * sizeof(uint64_t));
    if (!fs.ival.empty()) std::memcpy(ival, fs.ival.data(), fs.ival.size() * sizeof(double));
    if (cc && !fs.cc.empty()) std::memcpy(cc, fs.cc.data(), fs.cc.size() * sizeof(double));
    if (cctype && !fs.type.empty()) std::memcpy(cctype, fs.type.data(), fs.type.size() * sizeof(int32_t));
    return OCL_GB300_OK;
}

int ocl_gb300_loops_release(ocl_gb300_loops loops) {
    delete loops;
    return OCL_GB300_OK;
}

}  // extern "C"
