// drop.cuh -- drop-cutter launch interface.
#pragma once
#include "geom32.cuh"
#include "mesh.cuh"

namespace oclg {

constexpr int HLB_N = 256;   // entries of the height lower-bound table
constexpr int CAND_K = 256;  // refinement candidates kept per CL point (drop_run)
constexpr int CAND_K_NOALLOC = 64;  // the same for the no-allocation entry point
constexpr uint32_t CAND_VERIFY = 0x80000000u;  // list flag: decide this triangle's branch in FP64
constexpr int EDGE_SLOTS = 8;  // bull edge contacts evaluated ahead of the fold, per CL point
constexpr int EDGE_N_SATURATED = 255;  // per-point planned-edge count: this many or more

struct EdgeRes {  // one edge contact (MillingCutter::singleEdgeDrop), running-height independent
    double clz, ccx, ccy, ccz;
    int valid;
    int pad;
};

enum Counter {
    C_PAIRS = 0,      // exact-overlap pairs evaluated (plain FP64 path)
    C_REFINED = 1,    // FP64 triangle evaluations in the refinement stage
    C_FALLBACK = 2,   // CL points whose candidate list overflowed
    C_VIOLATION = 3,  // FP64 result below a certified FP32 lower bound (must stay 0)
    C_CAPPED = 4,     // Brent solves that hit the iteration cap
    C_SCREENED = 5,   // FP32 whole-triangle screens
    C_OVERFLOW = 6,   // points handed back because their candidate list overflowed
    C_CHAIN = 7,      // points handed back because branch thresholds kept chaining
    C_OPEN = 8,       // points collected below blo: a branch stayed undecided
    C_UNTRACKED = 9,  // of those: more branching triangles than tracked
    C_PLAIN = 10,     // handed-back points whose candidates exceed the exact kernel's buffer
    C_VFAIL = 11,     // points whose undecided branch lay below the collection threshold
    C_EDGEQ = 12,     // bull edges queued for evaluation ahead of the fold
    C_SPARSE = 13,    // warps handed to the sparse screen kernel
    C_NCOUNTERS = 14
};

struct DropCtx {
    CutterP cp;
    Prof32 prof;
    GridP g;
    const Cell* cells;
    const Entry* entries;
    const Tri64* t64;
    const Tri32* t32;
    const KDNodeD* kd_nodes;  // XY KD tree of the plain path
    const int32_t* kd_order;
    const double* cl;       // sorted CL points (M x 3)
    const uint32_t* perm;   // sorted -> caller index
    int M;
    double* out_z;
    double* out_cc;
    int32_t* out_type;
    uint32_t* cand;         // M x cand_cap candidate triangles (sorted by KD rank when final)
    float* cand_hi;         // M x cand_cap their FP32 upper bounds (screen only)
    float* cand_lo;         // M x cand_cap their certified FP32 lower bounds (screen only)
    uint16_t* ncand;        // per CL: count, or 0xFFFF = handed to the plain path
    int cand_cap;           // list capacity per CL point
    float* blo;             // per CL: certified lower bound (local frame)
    bool seeded;            // blo holds the seeding kernel's bounds on entry to the screen
    uint32_t* sparse_list;  // warps handed from the dense to the sparse screen kernel
    unsigned long long* sparse_n;
    // bull: edge contacts evaluated ahead of the fold (null: evaluated inline)
    uint32_t* edge_slots;   // M x EDGE_SLOTS: (triangle << 2 | edge) in fold order
    uint8_t* edge_n;        // per CL: planned edges (may exceed EDGE_SLOTS; EDGE_N_SATURATED: that many or more)
    struct EdgeRes* edge_res;  // M x EDGE_SLOTS results
    unsigned long long* counters;
    // hand-back lists and the bull edge queue of this call (read from here by
    // the batch kernels; the single-call kernels take them as arguments)
    uint32_t* list;
    uint32_t* list2;
    uint2* edge_queue;
    float E;                // FP32 position error budget
    float guard;            // margin for the bound tests
    bool composite_screen;  // composite cutter: screen_composite with comp
    Comp32 comp;
    float hlb[HLB_N];       // lower bound of height(r) on [k R / HLB_N, R]
};

// A launch over many jobs (ocl_gb300_drop_batch).  Each job has its own
// context (mesh, cutter, its slice of the batch's arrays).  Work tiles are
// (job, 128-point block of the job); persistent blocks take them in turn
// through an atomic counter (work stealing), so jobs of very different sizes
// share the GPU without a launch per job.  Stages whose work is counted on
// the device (scattered warps, handed-back points, bull edge queues) stride
// over the device-side lists of the jobs named in `jobs`.
constexpr int TILE_POINTS = 128;  // points per work tile (4 screen warps = one refinement block)
struct BatchView {
    const DropCtx* ctxs;
    const uint2* tiles;   // (job, block of the job)
    unsigned ntiles;
    unsigned* next;       // tile counter of this launch (zeroed before it)
    const uint32_t* jobs; // jobs of this launch
    unsigned njobs;
};

// Per job of a batch wave: the caller's points and the Morton frame of the
// job's mesh (x0, y0 origin; sx, sy scale to 16-bit cells).
struct BatchIn {
    const double* cl;
    uint64_t off;  // first point of the job in the wave
    uint64_t M;
    double x0, y0, sx, sy;
};

// Launchers of the batch kernels (drop.cu); `blocks` is the persistent grid.
void batch_launch_order(const BatchIn* d_in, uint32_t njobs, uint64_t Mtot, unsigned long long* keys,
                        uint32_t* idx, unsigned long long* keys2, uint32_t* idx2, void* sort_tmp, size_t sort_bytes,
                        int end_bit, double* cls, uint32_t* perm, cudaStream_t stream, int* status);
size_t batch_sort_bytes(uint64_t Mtot, int end_bit);
void batch_launch_bull(const BatchView& plan, const BatchView& eval, unsigned blocks, cudaStream_t stream);
void batch_launch_refine(const BatchView& bv, bool bull_plan, unsigned blocks, cudaStream_t stream);
void batch_launch_collect(const BatchView& bv, unsigned blocks, cudaStream_t stream);
// scratch: the exact kernel's global scratch (batch_exact_scratch_bytes(); null: none)
int batch_launch_exact(const BatchView& bv, bool composite, unsigned blocks, cudaStream_t stream,
                       unsigned char* scratch);
size_t batch_exact_scratch_bytes();
void batch_launch_plain(const BatchView& bv, unsigned blocks, cudaStream_t stream);
// Opt the exact kernels into their dynamic shared memory in the current context.
int ensure_exact_smem();

struct Batch;
int batch_create(const ocl_gb300_drop_job* jobs, Mesh* const* meshes, uint64_t njobs, const ocl_gb300_batch_opts* opts,
                 Batch** out);
int batch_run(Batch& b, cudaStream_t stream, ocl_gb300_stats* stats);
void batch_info(const Batch& b, ocl_gb300_batch_info* out);
void batch_destroy(Batch* b);
// A batch without jobs (for repeated use), and new jobs on an existing one.
Batch* batch_new(uint64_t workspace_bytes, uint64_t chunk_points, int list_capacity);
int batch_reset(Batch& b, const ocl_gb300_drop_job* jobs, Mesh* const* meshes, uint64_t njobs, int list_capacity,
                cudaStream_t stream);

struct Server;
int server_create(const ocl_gb300_server_opts* opts, Server** out);
void server_destroy(Server* s);
int server_add_mesh(Server& s, Mesh* m, int32_t* id);
int server_submit_drop(Server& s, int32_t mesh_id, const ocl_gb300_cutter& c, const double* cl, uint64_t M,
                       double* z, double* cc, int32_t* ty, uint64_t* id);
int server_submit_adaptive(Server& s, int32_t mesh_id, const ocl_gb300_cutter& c, const double* spans, uint64_t S,
                           double sampling, double min_sampling, double cos_limit, double* xyz, double* cc,
                           int32_t* ty, uint64_t cap, uint64_t* count, uint64_t* id);
int server_wait(Server& s, uint64_t id, double timeout_s, ocl_gb300_request_info* info);
int server_cancel(Server& s, uint64_t id);
int server_stats(Server& s, ocl_gb300_server_stats* out);
int server_pause(Server& s, bool paused);

struct DropWork;
// The per-call context fields that depend only on the mesh and the cutter:
// mesh arrays, grid, KD tree, FP32 profiles, the error budget E and guard.
void init_drop_ctx(const Mesh& m, const CutterP& cp, DropCtx& h);
int drop_run(Mesh& m, const CutterP& cp, const double* d_cl, uint64_t M, int precision, double* d_z, double* d_cc,
             int32_t* d_type, cudaStream_t stream, ocl_gb300_stats* stats);

// Stage times (screen, refine, fallback, total; ms) of this thread's last
// count drop calls, oldest first.
int drop_stage_times(uint64_t count, double* out);

int drop_run_noalloc(Mesh& m, const CutterP& cp, const double* d_cl, uint64_t M, double* d_z, double* d_cc,
                     int32_t* d_type, cudaStream_t stream);

// Cutter parameters from the ABI description (the reference constructors'
// arithmetic); returns an OCL_GB300_* status.
int make_cutter_params(const ocl_gb300_cutter& in, CutterP& cp);
// FP32 profile and the height lower-bound table for the screen.
void fill_prof(const CutterP& cp, Prof32& prof, float* hlb, bool& composite);
void fill_comp(const CutterP& cp, Comp32& comp);
// Host FP64 cutter height(r) (same arithmetic as the device).
double height_host(const CutterP& cp, double r);

}  // namespace oclg
