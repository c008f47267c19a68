// ce_server.cpp -- the serving front end: requests of any size, continuous
// batching onto a few concurrent evaluations, HBM-footprint admission.
//
// The reference serves one caller at a time: RunControllerEngine reads a
// fixed-size round from files, runs it synchronously and returns
// (ref: src/main.cu:467-582, 592-602).  A server here keeps `lanes` sessions of
// the same configuration (each with its own device scratch and streams) and a
// scheduler thread.  Requests (gains and INFO rows in host memory) queue in
// arrival order; when a lane is free the scheduler packs the oldest request
// with the requests behind it of the same model, whatever their plants (a
// batch on several plants carries a plant index per row), up to the lane's
// capacity (a request larger than that is served in pieces), copies their
// rows into the lane's pinned staging buffers, and enqueues H2D, the
// evaluation and D2H on the lane's stream.  While one lane's batch is on the
// GPU the next is staged, and batches of different lanes run concurrently.
// Each candidate's row is computed independently of the batch it lands in, so
// a request's result does not depend on what it was batched with.
//
// Admission: the lane capacity (candidates per batch) is the largest that
// fits `lanes` x (session scratch + batch buffers) into the HBM budget; the
// per-candidate footprint is derived from the configuration.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "ce_host.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    int64_t id = 0;
    int model = 0;
    int plant = 0;        // the plant of every row, or with `plants` the plant of row 0
    bool plants = false;  // one plant per row: row k on plant `plant + k` (a Monte Carlo request)
    int64_t n = 0;
    const float* gains = nullptr;
    const float* info_in = nullptr;
    float* info_out = nullptr;
    int64_t next = 0;      // first row not yet dispatched
    int64_t finished = 0;  // rows completed
    int64_t failed = 0;    // rows that failed, or were dropped from the queue after a failure
    bool done = false;
    std::string error;
    Clock::time_point t_submit, t_done;
    Clock::time_point t_dispatch;  // its first piece handed to a lane
    bool dispatched = false;
    int busy_at_dispatch = 0;      // lanes busy then (this one included)
};

struct Piece {
    std::shared_ptr<Request> req;
    int64_t row0, rows, off;  // request rows [row0, row0+rows) at batch offset `off`
};

struct Lane {
    std::vector<ce_session*> sess;  // one per model
    cudaStream_t stream = nullptr;
    cudaEvent_t start = nullptr;  // the batch's first stream work (timing)
    cudaEvent_t done = nullptr;
    float* d_gains = nullptr;
    float* d_info = nullptr;
    float* h_gains = nullptr;  // pinned
    float* h_info = nullptr;   // pinned
    int* h_idx = nullptr;      // pinned: the plant of each row of a Monte Carlo batch
    bool busy = false;
    std::vector<Piece> pieces;
};

}  // namespace

struct ce_server {
    std::vector<ce_config> cfg;  // per model
    std::vector<int> n_plants;   // per model
    int64_t capacity = 0;        // candidates per batch (per lane)
    int64_t max_work = 0;        // candidate-steps per batch (0: no cap)
    int max_wait_us = 0;
    int precision = CE_PRECISION_MIXED;
    std::vector<Lane> lanes;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;
    std::unordered_map<int64_t, std::shared_ptr<Request>> live;
    int64_t next_id = 1;
    bool stop = false;
    std::thread worker;
    // statistics
    int64_t batches = 0, batched_rows = 0, completed = 0;
    // completed requests, in completion order: latency, queue and service time, busy lanes
    std::vector<double> latency_ms, queue_ms, service_ms, busy_lanes;
    std::vector<double> batch_ms;  // per retired batch: its stream work
};

namespace ce {

namespace {

// Device bytes one evaluation needs per candidate (session scratch + the
// lane's batch buffers), from the sizes the session allocates.
int64_t bytes_per_candidate(const ce_config& c, int precision) {
    const int64_t nt = c.total_dim, pitch = ((c.fit_steps + 7) / 8) * 8;
    const int64_t groups = (c.freq + SWEEP_FG - 1) / SWEEP_FG;
    // 4-byte words per real of each buffer: the simulation's (fit window, summary)
    // and the rest's (LIN_A, eigenvalues, normal equations, sweep scratch)
    const int64_t sim = precision == CE_PRECISION_FP64 || precision == CE_PRECISION_COMPENSATED_DF ? 2 : 1;
    const int64_t real = precision == CE_PRECISION_MIXED ? 1 : 2;
    int64_t f = 0;
    f += 2 * (int64_t)c.cuda_mx_width + 2 * (int64_t)c.info_mx_width;  // gains + INFO, session and lane
    f += real * (nt * nt + 2 * nt);                                    // LIN_A, eigenvalues
    f += sim * (pitch + 4);                                            // fit window, summary
    f += real * (4 * nt * nt + 2 * nt);                                // AtA, Atb
    f += 1 + (MAXT + 1) + 1 + 1;                                       // nominal, fit order, lists
    f += real * (2 * (int64_t)c.freq + groups) + groups;               // sweep scratch
    if (c.observer == CE_OBSERVER_KALMAN) f += (int64_t)KAL_SCHED_STEPS * MAXS + 4;  // gain schedules
    return 4 * f;
}

// A request is done once every row is accounted for: dispatched and retired,
// successfully or not.  Until then a piece of it may still be on the GPU or in
// a lane's staging buffer, and the caller's buffers must stay untouched by the
// caller, so ce_server_wait keeps waiting.  Caller holds the lock.
void settle(ce_server* s, Request& r, Clock::time_point now) {
    if (r.done || r.next != r.n || r.finished + r.failed != r.n) return;
    r.done = true;
    r.t_done = now;
    if (r.error.empty()) {
        using ms = std::chrono::duration<double, std::milli>;
        s->completed++;
        s->latency_ms.push_back(ms(now - r.t_submit).count());
        s->queue_ms.push_back(ms(r.t_dispatch - r.t_submit).count());
        s->service_ms.push_back(ms(now - r.t_dispatch).count());
        s->busy_lanes.push_back((double)r.busy_at_dispatch);
    }
}

void complete_lane(ce_server* s, Lane& L) {
    // each piece's rows go to a disjoint slice of its request's output; the
    // request is not done before this piece retires, so the buffer is still valid
    for (const Piece& p : L.pieces) {
        const int64_t iw = s->cfg[p.req->model].info_mx_width;
        std::memcpy(p.req->info_out + p.row0 * iw, L.h_info + p.off * iw, (size_t)p.rows * iw * sizeof(float));
    }
    const auto now = Clock::now();
    float gpu_ms = 0.0f;
    const bool timed = cudaEventElapsedTime(&gpu_ms, L.start, L.done) == cudaSuccess;
    std::lock_guard<std::mutex> g(s->mu);
    if (timed) s->batch_ms.push_back((double)gpu_ms);
    for (const Piece& p : L.pieces) {
        p.req->finished += p.rows;
        settle(s, *p.req, now);
    }
    L.pieces.clear();
    L.busy = false;
    s->cv_done.notify_all();
}

// The batch on lane L failed (nothing of it is in flight any more).  Each of
// its requests records the first error, its rows still queued are withdrawn
// (they would read the caller's buffers after ce_server_wait returned), and it
// is done once its pieces on other lanes have retired as well.
void fail_pieces(ce_server* s, Lane& L, const std::string& msg) {
    const auto now = Clock::now();
    std::lock_guard<std::mutex> g(s->mu);
    for (const Piece& p : L.pieces) {
        Request& r = *p.req;
        if (r.error.empty()) r.error = msg;
        r.failed += p.rows;
        if (r.next < r.n) {
            r.failed += r.n - r.next;
            r.next = r.n;
            for (auto it = s->queue.begin(); it != s->queue.end(); ++it)
                if (it->get() == &r) {
                    s->queue.erase(it);
                    break;
                }
        }
        settle(s, r, now);
    }
    L.pieces.clear();
    L.busy = false;
    s->cv_done.notify_all();
}

// Take rows for one batch from the queue (caller holds the lock): the oldest
// request's model, then the queued requests of the same model in arrival
// order, whatever their plants.  A batch whose rows all use one plant (tuning
// requests on that plant) runs as an evaluation of that plant; any other batch
// -- tuning requests on several plants, Monte Carlo requests (a plant per row)
// -- runs with a plant index per row (plant = -1).
std::vector<Piece> form_batch(ce_server* s, int& model, int& plant) {
    std::vector<Piece> out;
    if (s->queue.empty()) return out;
    model = s->queue.front()->model;
    plant = s->queue.front()->plants ? -1 : s->queue.front()->plant;
    int64_t room = s->capacity, off = 0;
    if (s->max_work > 0)  // every row of the batch runs the model's horizon
        room = std::min(room, std::max<int64_t>(1, s->max_work / std::max(1, s->cfg[model].time)));
    for (auto it = s->queue.begin(); it != s->queue.end() && room > 0;) {
        Request& r = **it;
        if (r.model != model) {
            ++it;
            continue;
        }
        if (r.plants || r.plant != plant) plant = -1;
        const int64_t take = std::min(room, r.n - r.next);
        out.push_back(Piece{*it, r.next, take, off});
        r.next += take;
        off += take;
        room -= take;
        if (r.next == r.n) it = s->queue.erase(it);
        else ++it;
    }
    return out;
}

void dispatch(ce_server* s, Lane& L, int model, int plant) {
    const int64_t cw = s->cfg[model].cuda_mx_width, iw = s->cfg[model].info_mx_width;
    int64_t n = 0;
    for (const Piece& p : L.pieces) {
        std::memcpy(L.h_gains + p.off * cw, p.req->gains + p.row0 * cw, (size_t)p.rows * cw * sizeof(float));
        std::memcpy(L.h_info + p.off * iw, p.req->info_in + p.row0 * iw, (size_t)p.rows * iw * sizeof(float));
        n = std::max(n, p.off + p.rows);
    }
    CE_CUDA(cudaEventRecord(L.start, L.stream));
    CE_CUDA(cudaMemcpyAsync(L.d_gains, L.h_gains, (size_t)n * cw * sizeof(float), cudaMemcpyHostToDevice, L.stream));
    CE_CUDA(cudaMemcpyAsync(L.d_info, L.h_info, (size_t)n * iw * sizeof(float), cudaMemcpyHostToDevice, L.stream));
    if (plant < 0) {
        for (const Piece& p : L.pieces)
            for (int64_t k = 0; k < p.rows; ++k)
                L.h_idx[p.off + k] = p.req->plants ? p.req->plant + (int)(p.row0 + k) : p.req->plant;
        session_evaluate_plants_indexed(L.sess[model], L.h_idx, n, L.d_gains, L.d_info, L.d_info, L.stream);
    } else if (ce_evaluate_device(L.sess[model], plant, n, L.d_gains, L.d_info, L.d_info, L.stream) != 0) {
        throw std::runtime_error(ce_last_error());
    }
    CE_CUDA(cudaMemcpyAsync(L.h_info, L.d_info, (size_t)n * iw * sizeof(float), cudaMemcpyDeviceToHost, L.stream));
    CE_CUDA(cudaEventRecord(L.done, L.stream));
    std::lock_guard<std::mutex> g(s->mu);
    s->batches++;
    s->batched_rows += n;
}

void worker_loop(ce_server* s, int device) {
    cudaSetDevice(device);
    for (;;) {
        // retire finished batches
        for (Lane& L : s->lanes) {
            if (!L.busy) continue;
            const cudaError_t q = cudaEventQuery(L.done);
            if (q == cudaSuccess) complete_lane(s, L);
            else if (q != cudaErrorNotReady) fail_pieces(s, L, std::string("CUDA error: ") + cudaGetErrorString(q));
        }
        Lane* freeL = nullptr;
        for (Lane& L : s->lanes)
            if (!L.busy) {
                freeL = &L;
                break;
            }
        bool any_busy = false;
        for (Lane& L : s->lanes) any_busy = any_busy || L.busy;
        int model = 0, plant = 0;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->stop && s->queue.empty() && !any_busy) return;
            if (!freeL || s->queue.empty()) {
                // nothing to dispatch: wait for a request, or poll the busy lanes
                s->cv_work.wait_for(lk, std::chrono::microseconds(any_busy ? 50 : 2000));
                continue;
            }
            // continuous batching: a partial batch may wait briefly for more rows
            if (s->max_wait_us > 0) {
                int64_t rows = 0;
                for (auto& r : s->queue) rows += r->n - r->next;
                const auto age = Clock::now() - s->queue.front()->t_submit;
                if (rows < s->capacity && age < std::chrono::microseconds(s->max_wait_us) && !s->stop) {
                    s->cv_work.wait_for(lk, std::chrono::microseconds(50));
                    continue;
                }
            }
            freeL->pieces = form_batch(s, model, plant);
            freeL->busy = !freeL->pieces.empty();
            if (freeL->busy) {
                int busy = 0;
                for (Lane& L : s->lanes) busy += L.busy ? 1 : 0;
                const auto now = Clock::now();
                for (const Piece& p : freeL->pieces)
                    if (!p.req->dispatched) {
                        p.req->dispatched = true;
                        p.req->t_dispatch = now;
                        p.req->busy_at_dispatch = busy;
                    }
            }
        }
        if (freeL->busy) {
            try {
                dispatch(s, *freeL, model, plant);
            } catch (const std::exception& e) {
                cudaStreamSynchronize(freeL->stream);  // nothing of the batch may still be in flight
                fail_pieces(s, *freeL, e.what());
            }
        }
    }
}

void destroy_server(ce_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (Lane& L : s->lanes) {
        if (L.stream) cudaStreamSynchronize(L.stream);
        for (ce_session* x : L.sess)
            if (x) ce_session_destroy(x);
        if (L.done) cudaEventDestroy(L.done);
        if (L.start) cudaEventDestroy(L.start);
        if (L.stream) cudaStreamDestroy(L.stream);
        if (L.d_gains) cudaFree(L.d_gains);
        if (L.d_info) cudaFree(L.d_info);
        if (L.h_gains) cudaFreeHost(L.h_gains);
        if (L.h_info) cudaFreeHost(L.h_info);
        if (L.h_idx) cudaFreeHost(L.h_idx);
    }
    delete s;
}

void create_server(const ce_config* cfg, const ce_plant* plant, const int32_t* n_plants, int n_models,
                   const ce_server_options* opt, ce_server** out) {
    if (!cfg || !plant || !n_plants || !out) fail("ce_server_create: null argument");
    if (n_models < 1) fail("ce_server_create: n_models must be >= 1, got {}", n_models);
    ce_server_options o{};
    if (opt) o = *opt;
    const int lanes = o.lanes > 0 ? o.lanes : 2;
    if (lanes > 8) fail("ce_server_create: at most 8 lanes, got {}", lanes);
    if (o.precision != CE_PRECISION_MIXED && o.precision != CE_PRECISION_FP64 && o.precision != CE_PRECISION_COMPENSATED &&
        o.precision != CE_PRECISION_COMPENSATED_DF)
        fail("ce_server_create: unknown precision {}", o.precision);
    int64_t cap = o.max_batch > 0 ? o.max_batch : 65536;
    // every lane may hold a full batch's scratch for every model
    int64_t per = 0, cw = 0, iw = 0;
    for (int m = 0; m < n_models; ++m) {
        per += bytes_per_candidate(cfg[m], o.precision);
        cw = std::max<int64_t>(cw, cfg[m].cuda_mx_width);
        iw = std::max<int64_t>(iw, cfg[m].info_mx_width);
    }
    if (o.hbm_budget_bytes > 0) {
        const int64_t fit = o.hbm_budget_bytes / ((int64_t)lanes * per);
        if (fit < 1)
            fail("ce_server_create: an HBM budget of {} bytes does not hold one candidate per lane ({} bytes each, {} lanes)",
                 o.hbm_budget_bytes, per, lanes);
        cap = std::min(cap, fit);
    }
    auto s = std::unique_ptr<ce_server, void (*)(ce_server*)>(new ce_server, destroy_server);
    s->cfg.assign(cfg, cfg + n_models);
    s->n_plants.assign(n_plants, n_plants + n_models);
    s->capacity = cap;
    s->max_wait_us = std::max(0, o.max_wait_us);
    s->max_work = std::max<int64_t>(0, o.max_batch_work);
    s->precision = o.precision;
    s->lanes.resize(lanes);
    int device = 0;
    CE_CUDA(cudaGetDevice(&device));
    // every lane's full-batch scratch is allocated now when it fits in 80% of the
    // free device memory (otherwise it grows with the batches, as in a session)
    size_t free_b = 0, total_b = 0;
    CE_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const bool eager = (double)lanes * (double)per * (double)cap <= 0.8 * (double)free_b;
    for (Lane& L : s->lanes) {
        L.sess.assign(n_models, nullptr);
        for (int m = 0; m < n_models; ++m) {
            if (ce_session_create(&cfg[m], &plant[m], n_plants[m], &L.sess[m]) != 0 ||
                ce_session_set_precision(L.sess[m], o.precision) != 0)
                throw std::runtime_error(ce_last_error());
            // a full batch's scratch and, with several plants, the plant table that
            // batches on several plants read
            session_prepare(L.sess[m], eager ? cap : 0, n_plants[m] > 1);
            // the lanes' batches share the GPU: the throughput forms (the latency forms of
            // small batches measured ~5% lower saturation in the serving mix)
            session_set_small_batch_forms(L.sess[m], false);
        }
        CE_CUDA(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking));
        CE_CUDA(cudaEventCreate(&L.start));
        CE_CUDA(cudaEventCreate(&L.done));
        CE_CUDA(cudaMalloc((void**)&L.d_gains, (size_t)cap * cw * sizeof(float)));
        CE_CUDA(cudaMalloc((void**)&L.d_info, (size_t)cap * iw * sizeof(float)));
        CE_CUDA(cudaHostAlloc((void**)&L.h_gains, (size_t)cap * cw * sizeof(float), cudaHostAllocDefault));
        CE_CUDA(cudaHostAlloc((void**)&L.h_info, (size_t)cap * iw * sizeof(float), cudaHostAllocDefault));
        CE_CUDA(cudaHostAlloc((void**)&L.h_idx, (size_t)cap * sizeof(int), cudaHostAllocDefault));
    }
    s->worker = std::thread(worker_loop, s.get(), device);
    *out = s.release();
}

}  // namespace
}  // namespace ce

using namespace ce;

extern "C" {

CE_EXPORT int ce_server_create(const ce_config* cfg, const ce_plant* plant, int32_t n_plants,
                               const ce_server_options* opt, ce_server** out) {
    try {
        create_server(cfg, plant, &n_plants, 1, opt, out);
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

CE_EXPORT int ce_server_create_models(const ce_config* cfgs, const ce_plant* plants, const int32_t* n_plants,
                                      int32_t n_models, const ce_server_options* opt, ce_server** out) {
    try {
        create_server(cfgs, plants, n_plants, n_models, opt, out);
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

CE_EXPORT void ce_server_destroy(ce_server* s) { destroy_server(s); }

}  // extern "C"

namespace {

void submit(ce_server* s, int32_t model, int32_t plant_index, bool plants, int64_t n, const float* cuda_mx,
            const float* info_in, float* info_out, int64_t* request_id) {
    if (!s || !request_id) fail("ce_server_submit: null argument");
    if (model < 0 || model >= (int)s->cfg.size()) fail("model {} out of range [0, {})", model, s->cfg.size());
    if (plant_index < 0 || plant_index >= s->n_plants[model])
        fail("plant index {} out of range [0, {})", plant_index, s->n_plants[model]);
    if (n < 0) fail("candidate count {} is negative", n);
    if (plants && plant_index + n > s->n_plants[model])
        fail("plants [{}, {}) exceed the model's {} plants (one plant per candidate)", plant_index, plant_index + n,
             s->n_plants[model]);
    if (n > 0 && (!cuda_mx || !info_in || !info_out)) fail("ce_server_submit: null buffer");
    // a plant that cannot be evaluated fails its request here, before the
    // request can share a batch with others
    const ce_session* s0 = s->lanes[0].sess[model];
    for (int64_t p = plant_index, last = plants ? plant_index + n : plant_index + 1; p < last; ++p)
        if (const std::string& e = session_plant_error(s0, (int)p); !e.empty()) fail("plant {}: {}", p, e);
    auto r = std::make_shared<Request>();
    r->model = model;
    r->plant = plant_index;
    r->plants = plants;
    r->n = n;
    r->gains = cuda_mx;
    r->info_in = info_in;
    r->info_out = info_out;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (s->stop) fail("ce_server_submit: server is shutting down");
        r->id = s->next_id++;
        s->live.emplace(r->id, r);
        if (n == 0) {
            r->done = true;
            r->t_done = r->t_submit;
        } else {
            s->queue.push_back(r);
        }
        *request_id = r->id;
    }
    s->cv_work.notify_one();
}

}  // namespace

extern "C" {

CE_EXPORT int ce_server_submit_model(ce_server* s, int32_t model, int32_t plant_index, int64_t n, const float* cuda_mx,
                                     const float* info_in, float* info_out, int64_t* request_id) {
    try {
        submit(s, model, plant_index, false, n, cuda_mx, info_in, info_out, request_id);
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

CE_EXPORT int ce_server_submit_plants(ce_server* s, int32_t model, int32_t first_plant, int64_t n,
                                      const float* cuda_mx, const float* info_in, float* info_out,
                                      int64_t* request_id) {
    try {
        submit(s, model, first_plant, true, n, cuda_mx, info_in, info_out, request_id);
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

CE_EXPORT int ce_server_submit(ce_server* s, int32_t plant_index, int64_t n, const float* cuda_mx, const float* info_in,
                               float* info_out, int64_t* request_id) {
    return ce_server_submit_model(s, 0, plant_index, n, cuda_mx, info_in, info_out, request_id);
}

CE_EXPORT int ce_server_wait(ce_server* s, int64_t request_id, int32_t timeout_ms) {
    try {
        if (!s) fail("null server");
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->live.find(request_id);
        if (it == s->live.end()) fail("unknown request id {}", request_id);
        std::shared_ptr<Request> r = it->second;
        auto ready = [&] { return r->done; };
        if (timeout_ms < 0) s->cv_done.wait(lk, ready);
        else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) return CE_PENDING;
        s->live.erase(request_id);
        if (!r->error.empty()) fail("request {} failed: {}", request_id, r->error);
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

CE_EXPORT int ce_server_get_stats(ce_server* s, ce_server_stats* out) {
    try {
        if (!s || !out) fail("null argument");
        std::lock_guard<std::mutex> g(s->mu);
        ce_server_stats st{};
        st.capacity = s->capacity;
        st.lanes = (int32_t)s->lanes.size();
        st.completed = s->completed;
        st.batches = s->batches;
        st.batched_candidates = s->batched_rows;
        st.queued = (int64_t)s->queue.size();
        auto pct = [](std::vector<double> v, double p) {
            if (v.empty()) return 0.0;
            std::sort(v.begin(), v.end());
            const size_t k = std::min(v.size() - 1, (size_t)std::ceil(p * (double)v.size()) - 1);
            return v[k];
        };
        const std::vector<double>& lat = s->latency_ms;
        if (!lat.empty()) {
            st.latency_p50_ms = pct(lat, 0.50);
            st.latency_p99_ms = pct(lat, 0.99);
            st.latency_max_ms = *std::max_element(lat.begin(), lat.end());
            st.queue_p50_ms = pct(s->queue_ms, 0.50);
            st.queue_p99_ms = pct(s->queue_ms, 0.99);
            st.service_p50_ms = pct(s->service_ms, 0.50);
            st.service_p99_ms = pct(s->service_ms, 0.99);
            double q = 0.0, sv = 0.0, b = 0.0;
            int64_t k = 0;
            for (size_t i = 0; i < lat.size(); ++i)
                if (lat[i] >= st.latency_p99_ms) {
                    q += s->queue_ms[i];
                    sv += s->service_ms[i];
                    b += s->busy_lanes[i];
                    ++k;
                }
            st.tail_requests = k;
            if (k) {
                st.tail_queue_ms = q / (double)k;
                st.tail_service_ms = sv / (double)k;
                st.tail_busy_lanes = b / (double)k;
            }
        }
        if (!s->batch_ms.empty()) {
            st.batch_p50_ms = pct(s->batch_ms, 0.50);
            st.batch_p99_ms = pct(s->batch_ms, 0.99);
            st.batch_max_ms = *std::max_element(s->batch_ms.begin(), s->batch_ms.end());
        }
        *out = st;
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

CE_EXPORT int ce_server_reset_stats(ce_server* s) {
    if (!s) return 1;
    std::lock_guard<std::mutex> g(s->mu);
    s->latency_ms.clear();
    s->queue_ms.clear();
    s->service_ms.clear();
    s->busy_lanes.clear();
    s->batch_ms.clear();
    s->completed = s->batches = s->batched_rows = 0;
    return 0;
}

}  // extern "C"
