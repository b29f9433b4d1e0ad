// serve.cu -- ocl_gb300_server_*: a request loop over device-resident meshes.
//
// Clients (any thread) submit BatchDropCutter requests (host CL points in,
// z / CC / type out) and AdaptivePathDropCutter requests (host spans in,
// sampled points out).  A scheduler thread keeps up to `slots` batches on the
// GPU at once, each on its own stream with its own reusable batch workspace
// (persistent work-stealing launches, batch.cu):
//   * admission: when a slot is free, pending requests join its batch in
//     arrival order while the batch's points fit the slot's share of the
//     device-memory budget (inputs, outputs and batch workspace); a request
//     that could never fit is rejected when it is submitted;
//   * continuous batching: a request that arrives while others run joins the
//     next batch to form; a batch holds at most `max_batch_points` CL points,
//     so batches stay short and a request never waits long for the next
//     one; a drop request larger than what is left in a batch contributes a
//     piece of its points and goes to the back of the queue for the rest
//     (large requests share the GPU round robin with the ones behind them);
//     an adaptive path request contributes one bisection level per
//     batch and goes back to the head of the queue for its next level, so
//     its levels overlap with other requests' work;
//   * with two or more slots the first is a fast lane on a high-priority
//     stream: it takes only adaptive levels and drops (or pieces left) of at
//     most 16,384 points, so an adaptive request's next level does not wait
//     behind large drops, whose batches run on the other slots;
//   * each request's latency is the time from submission to the completion
//     of its last batch; the server keeps p50 / p99 over completed requests.
// The device work of a request is the same as that of the single-request
// entry points (ocl_gb300_drop / ocl_gb300_adaptive_path_drop), so its
// results are identical alone and in any mix.  Failures are reported per
// request (bad arguments, budget, cancellation, device errors); nothing in
// the loop throws.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "drop.cuh"
#include "paths.cuh"
#include "util.cuh"

namespace oclg {

namespace {

using Clock = std::chrono::steady_clock;

constexpr int KIND_DROP = 0;
constexpr int KIND_ADAPTIVE = 1;
// device bytes per CL point of a batch: inputs (24) and outputs (36), the
// sort and list bookkeeping (about 70) and the candidate lists (12 per entry)
constexpr uint64_t POINT_IO_BYTES = 24 + 8 + 24 + 4;

struct Request {
    uint64_t id = 0;
    int kind = KIND_DROP;
    Mesh* mesh = nullptr;
    ocl_gb300_cutter desc{};
    // drop
    const double* cl = nullptr;
    uint64_t M = 0;
    double* z_out = nullptr;
    double* cc_out = nullptr;
    int32_t* type_out = nullptr;
    // adaptive path drop
    ApdcRun run;
    double* xyz_out = nullptr;
    double* acc_out = nullptr;
    int32_t* atype_out = nullptr;
    uint64_t cap = 0;
    uint64_t* count_out = nullptr;
    // state
    int status = OCL_GB300_PENDING;
    std::string message;  // why it failed
    bool admitted = false;
    bool in_flight = false;
    bool cancel = false;
    int batches = 0;
    uint64_t points = 0;
    uint64_t done = 0;  // drop: points already dispatched to finished batches
    Clock::time_point submitted, started, finished;
    // points of the request's next step: a drop's remaining points, an
    // adaptive request's next bisection level
    uint64_t step_points() const { return kind == KIND_DROP ? M - done : run.points().size() / 3; }
    const double* step_cl() const { return kind == KIND_DROP ? cl + 3 * done : run.points().data(); }
};

struct Item {
    Request* r;
    uint64_t off, n;  // the item's points in the slot's buffers
    uint64_t src;     // drop: first point of the piece in the request
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    Batch* batch = nullptr;
    DevBuf<double> dcl, dz, dcc;
    DevBuf<int32_t> dty;
    double* hcl = nullptr;
    double* hz = nullptr;
    double* hcc = nullptr;
    int32_t* hty = nullptr;
    uint64_t hcap = 0;
    std::vector<Item> items;
    uint64_t points = 0;
    bool busy = false;
    bool fast = false;  // takes adaptive levels and small drops only, on a high-priority stream
};

// drop requests (or their remaining pieces) of at most this many points may
// go through the fast slot
constexpr uint64_t FAST_POINTS = 16384;

}  // namespace

struct Server {
    ocl_gb300_server_opts opts{};
    int device = 0;
    uint64_t slot_points = 0;  // most CL points one batch takes (the budget's share and max_batch_points)
    uint64_t io_points = 0;    // most CL points the budget's share holds (an adaptive level must fit)
    std::vector<Mesh*> meshes;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> pending;
    std::map<uint64_t, std::unique_ptr<Request>> reqs;
    std::vector<Slot> slots;
    std::thread th;
    bool stop = false;
    bool paused = false;  // no new batches while set
    uint64_t next_id = 1;
    // statistics
    uint64_t submitted = 0, completed = 0, failed = 0, cancelled = 0, rejected = 0, batches = 0, points = 0;
    std::vector<double> latencies_ms;
    Clock::time_point t_first, t_last;
    bool any = false;
    void loop();
    bool launch(Slot& s);
    void finish(Slot& s, bool ok, const std::string& err);
    void complete(Request* r, int status);
};

namespace {

bool slot_reserve(Slot& s, uint64_t n) {
    if (!s.dcl.reserve(3 * n) || !s.dz.reserve(n) || !s.dcc.reserve(3 * n) || !s.dty.reserve(n)) return false;
    if (n > s.hcap) {
        cudaFreeHost(s.hcl);
        cudaFreeHost(s.hz);
        cudaFreeHost(s.hcc);
        cudaFreeHost(s.hty);
        s.hcl = s.hz = s.hcc = nullptr;
        s.hty = nullptr;
        s.hcap = 0;
        const uint64_t c = std::max<uint64_t>(n, 1u << 16);
        if (cudaMallocHost(&s.hcl, 3 * c * sizeof(double)) != cudaSuccess ||
            cudaMallocHost(&s.hz, c * sizeof(double)) != cudaSuccess ||
            cudaMallocHost(&s.hcc, 3 * c * sizeof(double)) != cudaSuccess ||
            cudaMallocHost(&s.hty, c * sizeof(int32_t)) != cudaSuccess)
            return false;
        s.hcap = c;
    }
    return true;
}

}  // namespace

void Server::complete(Request* r, int status) {
    r->status = status;
    r->finished = Clock::now();
    r->in_flight = false;
    if (status == OCL_GB300_OK) {
        ++completed;
        latencies_ms.push_back(std::chrono::duration<double, std::milli>(r->finished - r->submitted).count());
        t_last = r->finished;
    } else if (status == OCL_GB300_CANCELLED) {
        ++cancelled;
    } else {
        ++failed;
    }
    cv_done.notify_all();
}

// Fill a free slot from the head of the queue and put its batch on the GPU
// (with the lock held).  Returns false when nothing was pending.
bool Server::launch(Slot& s) {
    s.items.clear();
    s.points = 0;
    for (auto it = pending.begin();
         it != pending.end() && (int)s.items.size() < opts.max_batch_requests && s.points < slot_points;) {
        Request* r = *it;
        if (r->cancel) {
            it = pending.erase(it);
            complete(r, OCL_GB300_CANCELLED);
            continue;
        }
        uint64_t n = r->step_points();
        // the fast slot takes adaptive levels and small drops only
        if (s.fast && r->kind == KIND_DROP && n > FAST_POINTS) {
            ++it;
            continue;
        }
        if (r->kind == KIND_DROP) {
            n = std::min(n, slot_points - s.points);  // a piece; the rest in later batches
        } else if (!s.items.empty() && s.points + n > slot_points) {
            break;  // an adaptive level is not split
        }
        it = pending.erase(it);
        if (!r->admitted) {
            r->admitted = true;
            r->started = Clock::now();
        }
        r->in_flight = true;
        s.items.push_back({r, s.points, n, r->kind == KIND_DROP ? r->done : 0});
        s.points += n;
    }
    if (s.items.empty()) return false;
    std::string err;
    int st = OCL_GB300_OK;
    if (cudaSetDevice(device) != cudaSuccess || !slot_reserve(s, s.points)) {
        st = OCL_GB300_OOM;
        err = "server: device buffers for a batch";
    }
    std::vector<ocl_gb300_drop_job> jobs(s.items.size());
    std::vector<Mesh*> ms(s.items.size());
    if (!st) {
        for (size_t k = 0; k < s.items.size(); ++k) {
            const Item& it = s.items[k];
            std::memcpy(s.hcl + 3 * it.off, it.r->step_cl(), 3 * it.n * sizeof(double));
            jobs[k].mesh = nullptr;
            jobs[k].cutter = it.r->desc;
            jobs[k].d_cl_xyz = s.dcl.p + 3 * it.off;
            jobs[k].M = it.n;
            jobs[k].d_z_out = s.dz.p + it.off;
            jobs[k].d_cc_out = s.dcc.p + 3 * it.off;
            jobs[k].d_type_out = s.dty.p + it.off;
            ms[k] = it.r->mesh;
        }
        if (cudaMemcpyAsync(s.dcl.p, s.hcl, 3 * s.points * sizeof(double), cudaMemcpyHostToDevice, s.stream) !=
            cudaSuccess)
            st = OCL_GB300_DEVICE_ERROR;
    }
    if (!st) st = batch_reset(*s.batch, jobs.data(), ms.data(), jobs.size(), opts.list_capacity, s.stream);
    if (!st) st = batch_run(*s.batch, s.stream, nullptr);
    if (!st && (cudaMemcpyAsync(s.hz, s.dz.p, s.points * sizeof(double), cudaMemcpyDeviceToHost, s.stream) ||
                cudaMemcpyAsync(s.hcc, s.dcc.p, 3 * s.points * sizeof(double), cudaMemcpyDeviceToHost, s.stream) ||
                cudaMemcpyAsync(s.hty, s.dty.p, s.points * sizeof(int32_t), cudaMemcpyDeviceToHost, s.stream) ||
                cudaEventRecord(s.done, s.stream)))
        st = OCL_GB300_DEVICE_ERROR;
    if (st) {
        if (err.empty()) err = last_error_ref();
        finish(s, false, err);
        return true;
    }
    s.busy = true;
    ++batches;
    return true;
}

// A slot's batch has finished (or failed): results to the requests, the
// adaptive ones that need another level back to the head of the queue.
void Server::finish(Slot& s, bool ok, const std::string& err) {
    s.busy = false;
    for (auto it = s.items.rbegin(); it != s.items.rend(); ++it) {
        Request* r = it->r;
        ++r->batches;
        r->points += it->n;
        points += it->n;
        if (!ok) {
            r->message = err;
            complete(r, OCL_GB300_DEVICE_ERROR);
            continue;
        }
        if (r->kind == KIND_DROP) {
            for (uint64_t i = 0; i < it->n; ++i) {
                r->z_out[it->src + i] = s.hz[it->off + i];
                r->type_out[it->src + i] = s.hty[it->off + i];
            }
            std::memcpy(r->cc_out + 3 * it->src, s.hcc + 3 * it->off, 3 * it->n * sizeof(double));
            r->done = it->src + it->n;
            if (r->done == r->M) {
                complete(r, OCL_GB300_OK);
            } else if (r->cancel) {
                complete(r, OCL_GB300_CANCELLED);
            } else {
                r->in_flight = false;
                pending.push_back(r);  // its next piece after what is queued (round robin)
            }
            continue;
        }
        r->run.consume(s.hz + it->off, s.hcc + 3 * it->off, s.hty + it->off);
        if (r->run.done()) {
            const int st = r->run.write(r->xyz_out, r->acc_out, r->atype_out, r->cap, r->count_out);
            if (st) r->message = "output buffer too small: " + std::to_string(*r->count_out) + " points";
            complete(r, st);
        } else if (r->cancel) {
            complete(r, OCL_GB300_CANCELLED);
        } else {
            r->in_flight = false;
            pending.push_front(r);  // its next level goes first
        }
    }
    s.items.clear();
}

void Server::loop() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        bool busy = false;
        for (Slot& s : slots) {
            if (!s.busy) continue;
            const cudaError_t e = cudaEventQuery(s.done);
            if (e == cudaSuccess) {
                finish(s, true, "");
            } else if (e != cudaErrorNotReady) {
                finish(s, false, std::string("server batch: ") + cudaGetErrorString(e));
            } else {
                busy = true;
            }
        }
        for (Slot& s : slots)
            if (!s.busy && !pending.empty() && !paused) {
                launch(s);
                busy = busy || s.busy;
            }
        for (const Slot& s : slots) busy = busy || s.busy;
        if (stop && !busy) break;
        if (busy) cv_work.wait_for(lk, std::chrono::microseconds(50));
        else cv_work.wait(lk, [&] { return stop || (!pending.empty() && !paused); });
    }
    // shutting down: what is still queued is cancelled
    while (!pending.empty()) {
        Request* r = pending.front();
        pending.pop_front();
        complete(r, OCL_GB300_CANCELLED);
    }
}

int server_create(const ocl_gb300_server_opts* o, Server** out) {
    *out = nullptr;
    std::unique_ptr<Server> s(new Server());
    if (o) s->opts = *o;
    if (!s->opts.hbm_budget_bytes) s->opts.hbm_budget_bytes = 16ull << 30;
    if (s->opts.slots <= 0) s->opts.slots = 2;
    if (s->opts.max_batch_requests <= 0) s->opts.max_batch_requests = 64;
    if (s->opts.list_capacity == 0) s->opts.list_capacity = CAND_K;
    if (s->opts.max_batch_points == 0) s->opts.max_batch_points = 1 << 18;
    if (s->opts.slots > 16 || s->opts.list_capacity < 16 || s->opts.list_capacity > CAND_K ||
        s->opts.hbm_budget_bytes < (64ull << 20) || s->opts.max_batch_points < 0) {
        set_error("server: slots 1..16, list capacity 16..256, budget at least 64 MiB, max_batch_points >= 0");
        return OCL_GB300_BAD_ARG;
    }
    CK(cudaGetDevice(&s->device));
    // each slot: a quarter of its share for the batch's inputs and outputs,
    // the rest for the batch workspace (chunked into waves by the batch)
    const uint64_t share = s->opts.hbm_budget_bytes / (uint64_t)s->opts.slots;
    s->slot_points = std::max<uint64_t>(std::min<uint64_t>(share / 4 / POINT_IO_BYTES, s->opts.max_batch_points), 1);
    const uint64_t io_points = std::max<uint64_t>(share / 4 / POINT_IO_BYTES, 1);
    s->slots.resize(s->opts.slots);
    int prio_low = 0, prio_high = 0;
    CK(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
    for (size_t k = 0; k < s->slots.size(); ++k) {
        Slot& sl = s->slots[k];
        // with two or more slots the first is the fast one: its batches (the
        // next bisection level of every adaptive request in flight, small
        // drops) are short and its stream's blocks go first on the SMs
        sl.fast = s->slots.size() >= 2 && k == 0;
        CK(cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking, sl.fast ? prio_high : prio_low));
        CK(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
        // chunks small enough that a wave of two fits the workspace (about
        // 70 bytes per point plus 12 per list entry plus a bull edge plan)
        const uint64_t ws = share - share / 4;
        const uint64_t per_point = 70 + 12 * (uint64_t)s->opts.list_capacity + 420;
        const uint64_t chunk = std::max<uint64_t>(1024, std::min<uint64_t>(1ull << 20, ws / (2 * per_point)));
        sl.batch = batch_new(ws, chunk, s->opts.list_capacity);
    }
    s->io_points = io_points;
    Server* raw = s.release();
    raw->th = std::thread([raw] { raw->loop(); });
    *out = raw;
    return OCL_GB300_OK;
}

void server_destroy(Server* s) {
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->th.joinable()) s->th.join();
    for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        batch_destroy(sl.batch);
        cudaFreeHost(sl.hcl);
        cudaFreeHost(sl.hz);
        cudaFreeHost(sl.hcc);
        cudaFreeHost(sl.hty);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    delete s;
}

int server_add_mesh(Server& s, Mesh* m, int32_t* id) {
    std::lock_guard<std::mutex> lk(s.mu);
    s.meshes.push_back(m);
    *id = (int32_t)s.meshes.size() - 1;
    return OCL_GB300_OK;
}

static int enqueue_request(Server& s, std::unique_ptr<Request> r, int32_t mesh_id, uint64_t* id) {
    std::lock_guard<std::mutex> lk(s.mu);
    if (mesh_id < 0 || mesh_id >= (int32_t)s.meshes.size()) {
        ++s.rejected;
        set_error("server: unknown mesh id " + std::to_string(mesh_id));
        return OCL_GB300_BAD_ARG;
    }
    r->mesh = s.meshes[mesh_id];
    if (r->mesh->n == 0) {
        ++s.rejected;
        set_error("server: the mesh has no triangles");
        return OCL_GB300_BAD_ARG;
    }
    if (r->kind == KIND_ADAPTIVE && r->step_points() > s.io_points) {
        ++s.rejected;
        set_error("server: a request of " + std::to_string(r->step_points()) +
                  " CL points per level exceeds what one batch may hold under the budget (" +
                  std::to_string(s.io_points) + ")");
        return OCL_GB300_OOM;
    }
    r->id = s.next_id++;
    r->submitted = Clock::now();
    if (!s.any) {
        s.t_first = r->submitted;
        s.any = true;
    }
    *id = r->id;
    ++s.submitted;
    s.pending.push_back(r.get());
    s.reqs[r->id] = std::move(r);
    s.cv_work.notify_all();
    return OCL_GB300_OK;
}

int make_cutter_params(const ocl_gb300_cutter& in, CutterP& cp);

int server_submit_drop(Server& s, int32_t mesh_id, const ocl_gb300_cutter& c, const double* cl, uint64_t M,
                       double* z, double* cc, int32_t* ty, uint64_t* id) {
    CutterP cp;
    if (make_cutter_params(c, cp)) {
        set_error("server: invalid cutter");
        return OCL_GB300_BAD_ARG;
    }
    std::unique_ptr<Request> r(new Request());
    r->kind = KIND_DROP;
    r->desc = c;
    r->cl = cl;
    r->M = M;
    r->z_out = z;
    r->cc_out = cc;
    r->type_out = ty;
    if (M == 0) {
        std::lock_guard<std::mutex> lk(s.mu);
        r->id = s.next_id++;
        r->submitted = r->finished = Clock::now();
        *id = r->id;
        ++s.submitted;
        Request* raw = r.get();
        s.reqs[r->id] = std::move(r);
        s.complete(raw, OCL_GB300_OK);
        return OCL_GB300_OK;
    }
    return enqueue_request(s, std::move(r), mesh_id, id);
}

int server_submit_adaptive(Server& s, int32_t mesh_id, const ocl_gb300_cutter& c, const double* spans, uint64_t S,
                           double sampling, double min_sampling, double cos_limit, double* xyz, double* cc,
                           int32_t* ty, uint64_t cap, uint64_t* count, uint64_t* id) {
    CutterP cp;
    if (make_cutter_params(c, cp)) {
        set_error("server: invalid cutter");
        return OCL_GB300_BAD_ARG;
    }
    std::unique_ptr<Request> r(new Request());
    r->kind = KIND_ADAPTIVE;
    r->desc = c;
    int st = r->run.init(spans, S, sampling, min_sampling, cos_limit);
    if (st) return st;
    r->xyz_out = xyz;
    r->acc_out = cc;
    r->atype_out = ty;
    r->cap = cap;
    r->count_out = count;
    if (r->run.done()) {  // no spans: nothing to drop
        std::lock_guard<std::mutex> lk(s.mu);
        r->id = s.next_id++;
        r->submitted = r->finished = Clock::now();
        *id = r->id;
        ++s.submitted;
        Request* raw = r.get();
        s.reqs[r->id] = std::move(r);
        s.complete(raw, raw->run.write(xyz, cc, ty, cap, count));
        return OCL_GB300_OK;
    }
    return enqueue_request(s, std::move(r), mesh_id, id);
}

int server_wait(Server& s, uint64_t id, double timeout_s, ocl_gb300_request_info* info) {
    std::unique_lock<std::mutex> lk(s.mu);
    auto it = s.reqs.find(id);
    if (it == s.reqs.end()) {
        set_error("server: unknown request id " + std::to_string(id));
        return OCL_GB300_BAD_ARG;
    }
    Request* r = it->second.get();
    auto ready = [&] { return r->status != OCL_GB300_PENDING; };
    if (timeout_s < 0) s.cv_done.wait(lk, ready);
    else if (!s.cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) return OCL_GB300_PENDING;
    if (info) {
        std::memset(info, 0, sizeof(*info));
        info->status = r->status;
        info->batches = r->batches;
        info->points = r->points;
        info->latency_ms = std::chrono::duration<double, std::milli>(r->finished - r->submitted).count();
        info->queue_ms = r->admitted ? std::chrono::duration<double, std::milli>(r->started - r->submitted).count()
                                     : info->latency_ms;
        std::strncpy(info->message, r->message.c_str(), sizeof(info->message) - 1);
    }
    s.reqs.erase(it);
    return OCL_GB300_OK;
}

int server_cancel(Server& s, uint64_t id) {
    std::lock_guard<std::mutex> lk(s.mu);
    auto it = s.reqs.find(id);
    if (it == s.reqs.end()) {
        set_error("server: unknown request id " + std::to_string(id));
        return OCL_GB300_BAD_ARG;
    }
    Request* r = it->second.get();
    if (r->status != OCL_GB300_PENDING) return OCL_GB300_OK;  // already finished
    r->cancel = true;
    if (!r->in_flight) {
        auto p = std::find(s.pending.begin(), s.pending.end(), r);
        if (p != s.pending.end()) s.pending.erase(p);
        s.complete(r, OCL_GB300_CANCELLED);
    }
    return OCL_GB300_OK;
}

int server_pause(Server& s, bool paused) {
    {
        std::lock_guard<std::mutex> lk(s.mu);
        s.paused = paused;
    }
    s.cv_work.notify_all();
    return OCL_GB300_OK;
}

int server_stats(Server& s, ocl_gb300_server_stats* out) {
    std::lock_guard<std::mutex> lk(s.mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s.submitted;
    out->completed = s.completed;
    out->failed = s.failed;
    out->cancelled = s.cancelled;
    out->rejected = s.rejected;
    out->batches = s.batches;
    out->points = s.points;
    out->pending = s.pending.size();
    if (!s.latencies_ms.empty()) {
        std::vector<double> v = s.latencies_ms;
        std::sort(v.begin(), v.end());
        auto q = [&](double f) {
            const double pos = f * (double)(v.size() - 1);
            const size_t lo = (size_t)pos;
            const size_t hi = std::min(lo + 1, v.size() - 1);
            return v[lo] + (v[hi] - v[lo]) * (pos - (double)lo);
        };
        out->p50_ms = q(0.50);
        out->p99_ms = q(0.99);
        out->max_ms = v.back();
        double sum = 0.0;
        for (double x : v) sum += x;
        out->mean_ms = sum / (double)v.size();
    }
    if (s.any) out->elapsed_s = std::chrono::duration<double>(s.t_last - s.t_first).count();
    return OCL_GB300_OK;
}

}  // namespace oclg
