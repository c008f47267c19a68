// ce_engine.cpp -- sessions, the stage pipeline, the C ABI and RunControllerEngine.
//
// The reference's orchestrator (ref: src/main.cu:385-582) runs every stage
// synchronously, bouncing LIN_A, eigenvalues and AtA/Atb through host memory
// for the Eigen stages.  Here a session keeps the decoded plant tables on the
// host (they travel to the kernels in the launch parameters), the margin
// plants' sweep grids on the device and a grow-only set of device scratch
// buffers.  One evaluation forks the caller's stream onto two session streams:
//
//   high priority:  k_lina_eig (FP64, persistent) ── k_nominal (FP64, persistent)
//   low priority:   k_sim ─ [eig ready] k_fit_classify ─ k_fit ─ k_modal ─ [nominal ready] k_sweep_*
//
// and joins back; batches of >= 32,768 candidates run the per-candidate stages
// in two chunks so the fit of the first starts while the second's eigensolve
// runs.  Only gains in and cost rows out cross the host boundary.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <iomanip>
#include <memory>
#include <sstream>
#include <vector>

#include "ce_host.h"

namespace ce {

thread_local std::string g_last_error;

namespace {

constexpr float PI = 0x1.921fb6p+1f;

}  // namespace

struct Buffers {
    int64_t cap = 0;
    int nt = 0, time = 0, pitch = 0, precision = -1;
    float* gains = nullptr;
    float* info = nullptr;
    void* lina = nullptr;  // float, or double in the FP64 form
    void* eig = nullptr;
    void* ywin = nullptr;
    void* summ = nullptr;
    void* ata = nullptr;
    void* atb = nullptr;
    int* nominal = nullptr;
    int* fit_counts = nullptr;
    int* fit_order = nullptr;
    int* nominal_list = nullptr;
    int* nominal_count = nullptr;
    int* sweep_list = nullptr;
    int* sweep_count = nullptr;
    int* plant_idx = nullptr;  // per candidate: its plant (indexed per-candidate-plant evaluations)
    SweepScratch sweep{};
    KalGroups kal{};  // Kalman observer: candidate grouping by noise weights
    float* traj = nullptr;
    int64_t traj_cap = 0;
    void release() {
        for (void* p : {(void*)gains, (void*)info, (void*)lina, eig, ywin, summ, ata, atb, (void*)nominal,
                        (void*)fit_counts, (void*)fit_order, (void*)nominal_list, (void*)nominal_count,
                        (void*)sweep_list, (void*)sweep_count, sweep.mag, sweep.arg, sweep.bpc, (void*)sweep.fail,
                        (void*)traj, (void*)kal.bucket, (void*)kal.cnt, (void*)kal.order, (void*)kal.sched,
                        (void*)kal.meta, (void*)kal.lists, (void*)plant_idx})
            if (p) cudaFree(p);
        gains = info = traj = nullptr;
        lina = eig = ywin = summ = ata = atb = nullptr;
        nominal = fit_counts = fit_order = nominal_list = nominal_count = sweep_list = sweep_count = nullptr;
        plant_idx = nullptr;
        sweep = SweepScratch{};
        kal = KalGroups{};
        cap = traj_cap = 0;
    }
};

}  // namespace ce

struct ce_session {
    ce_config cfg{};
    int n_plants = 0;
    int precision = CE_PRECISION_MIXED;
    std::vector<ce::Plant> plants;
    std::vector<std::string> plant_err;
    // simulation kernel of each plant in mixed precision: compiled for its
    // instruction program (ce_jit.cpp), or null for the table-driven kernel
    int sim_kind = CE_SIM_SPECIALISED;
    std::vector<ce::SimKernels> sim_kernel;
    std::string sim_log;
    // margin plants and their sweep grids: one per plant in serial mode, the
    // observer model shared by all plants in batch mode (ref: src/allmargin.cu:11-15)
    int grid_np = 1;
    int grid_of(int plant) const { return cfg.serial ? plant : 0; }
    std::vector<float> alpha32;   // per margin plant
    std::vector<double> alpha64;
    float* d_mplant = nullptr;    // grid_np x margin_plant_stride() floats
    void* d_alpha32 = nullptr;    // per margin plant, on the device (per-candidate plants)
    void* d_alpha64 = nullptr;
    // per-candidate plants: the plant table (MC_FIELDS x n_plants) and the
    // simulation kernel compiled for it, built on first use
    float* d_mc_tab = nullptr;
    ce::SimKernels sim_kernel_mc;
    ce_tuning tuning{};  // 0 fields: the library defaults
    float* d_fgrid32 = nullptr;   // grid_np x freq x 8
    double* d_fgrid64 = nullptr;  // built on the first FP64 evaluation
    ce::Buffers buf;
    // stream: host-buffer evaluations; fast: the FP32 stages (lowest
    // priority); side: the FP64 eigensolves (highest priority)
    cudaStream_t stream = nullptr, fast = nullptr, side = nullptr;
    cudaStream_t side2 = nullptr;  // the nominal eigensolve of a small batch, beside LIN_A's
    cudaStream_t side3 = nullptr;  // Kalman: the quad form's stragglers, beside the scheduled form
    // the latency forms of a small batch (wide simulation, more lanes per matrix in the FP64
    // eigensolves, the nominal eigensolve beside LIN_A's); a server's sessions run without them
    bool small_forms = true;
    int eig_arith = CE_EIG_ARITH_FUSED;  // arithmetic of the FP64 eigensolves
    cudaEvent_t ev_fork = nullptr, ev_done = nullptr;
    cudaEvent_t ev_kal = nullptr, ev_kal_quad = nullptr;  // Kalman: schedules ready; quad form done
    cudaEvent_t ev_eig[ce::MAX_CHUNKS] = {}, ev_nom[ce::MAX_CHUNKS] = {};
    int64_t launches = 0;
    int device = 0;
    // stage timing (ce_session_set_profiling)
    bool profiling = false;
    struct Pending {
        int stage;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> event_pool;
    double stage_ms[CE_NUM_STAGES] = {};
    int64_t stage_n[CE_NUM_STAGES] = {};
    cudaEvent_t take_event() {
        if (!event_pool.empty()) {
            cudaEvent_t e = event_pool.back();
            event_pool.pop_back();
            return e;
        }
        cudaEvent_t e;
        CE_CUDA(cudaEventCreate(&e));
        return e;
    }
};

// A ragged batch (ce_ragged_*): instances of different configurations and
// plants evaluated together, one launch per stage over all their candidates.
struct ce_ragged {
    std::vector<ce_config> cfg;             // per instance
    ce_config layout{};                     // the maxima: row widths, dimensions, fit window, sweep size
    ce_session* s = nullptr;                // streams, scratch and the pipeline, sized by `layout`
    ce::Plant* d_plants = nullptr;          // per instance
    ce::Run* d_runs = nullptr;              // per instance, with the strides and slots of `layout`
    int* d_inst = nullptr;                  // instance of each candidate of the current evaluation
    float* d_tab = nullptr;                 // their simulation table (RT_FIELDS x inst_cap)
    int64_t inst_cap = 0;
    // the host path's staging of the caller's packed rows: pinned, and on the device
    float *h_gains = nullptr, *h_info = nullptr;
    int64_t host_g_cap = 0, host_i_cap = 0;
    float *d_g_in = nullptr, *d_i_in = nullptr, *d_i_out = nullptr;
    int64_t dev_g_cap = 0, dev_i_cap = 0;
    std::vector<int> h_inst;        // device position -> instance
    std::vector<int64_t> dev_k;     // device position -> candidate within its instance
    // the prepared evaluation (ce_ragged_prepare): its candidate counts, the device
    // order's settings, and per device position the caller's row offsets and widths
    std::vector<int64_t> prep_counts;
    int prep_lanes = 0, prep_inst_order = -1;
    bool prepared = false;
    int64_t prep_n = 0, g_total = 0, i_total = 0;
    int64_t* d_goff = nullptr;
    int64_t* d_ioff = nullptr;
    int2* d_wid = nullptr;
    int64_t map_cap = 0;
    ce_ragged_tuning tuning{};
    // per instance: the operation of every interpreted slot (NL chains, then DC and U; 0 = empty)
    std::vector<std::array<uint8_t, ce::MAXW * ce::MAX_NL + ce::MAX_DC + ce::MAX_U>> sig;
};

namespace ce {

namespace {

void set_error(const char* msg) { g_last_error = msg ? msg : ""; }

template <typename F>
int guarded(F&& f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        set_error(e.what());
        return 1;
    } catch (...) {
        set_error("unknown error");
        return 1;
    }
}

int fit_pitch(int steps) { return ((steps + 7) / 8) * 8; }

template <typename T>
void dev_alloc(T*& p, size_t count) {
    if (count == 0) count = 1;
    CE_CUDA(cudaMalloc((void**)&p, count * sizeof(T)));
}

// Element size in bytes of each per-candidate buffer of a precision: the fit
// window and the trajectory summaries (FP32 simulation: float), LIN_A and the
// eigenvalues, AtA / Atb, and the sweep scratch.
struct BufElems {
    size_t ywin, summ, lina, eig, ata, sweep;
};
BufElems buf_elems(int precision) {
    if (precision == CE_PRECISION_FP64) return {8, 8, 8, 8, 8, 8};
    if (precision == CE_PRECISION_COMPENSATED) return {4, 4, 8, 8, 8, 8};
    if (precision == CE_PRECISION_COMPENSATED_TRAJ64 || precision == CE_PRECISION_COMPENSATED_DF)
        return {8, 8, 8, 8, 8, 8};
    return {4, 4, 4, 4, 4, 4};
}
// The arithmetic each stage runs in under a session precision: the compensated
// form simulates in FP32 (the mixed kernels), compensated_df in double-float,
// and both run LIN_A, the eigensolves and the sweep in FP64 (the FP64 form's
// kernels).
bool compensated(int prec) {
    return prec == CE_PRECISION_COMPENSATED || prec == CE_PRECISION_COMPENSATED_TRAJ64 ||
           prec == CE_PRECISION_COMPENSATED_DF;
}
int sim_precision(int prec) {
    return prec == CE_PRECISION_COMPENSATED ? CE_PRECISION_MIXED
           : prec == CE_PRECISION_COMPENSATED_TRAJ64 ? CE_PRECISION_FP64 : prec;
}
// the simulation writes a double trajectory (the FP64 and double-float recurrences)
bool sim_double(int prec) { return sim_precision(prec) != CE_PRECISION_MIXED; }
int eig_precision(int prec) { return compensated(prec) ? CE_PRECISION_FP64 : prec; }
bool grids64(int prec) { return prec != CE_PRECISION_MIXED; }

void ensure_buffers(ce_session* s, int64_t n, bool traj) {
    Buffers& b = s->buf;
    const ce_config& c = s->cfg;
    const int nt = c.total_dim, pitch = fit_pitch(c.fit_steps);
    const BufElems e = buf_elems(s->precision);
    if (n > b.cap || b.precision != s->precision || b.nt != nt || b.pitch != pitch) {
        b.release();
        const int64_t cap = n;
        dev_alloc(b.gains, (size_t)cap * c.cuda_mx_width);
        dev_alloc(b.info, (size_t)cap * c.info_mx_width);
        CE_CUDA(cudaMalloc(&b.lina, (size_t)cap * nt * nt * e.lina + 16));
        CE_CUDA(cudaMalloc(&b.eig, (size_t)cap * 2 * nt * e.eig + 16));
        CE_CUDA(cudaMalloc(&b.ywin, (size_t)cap * pitch * e.ywin + 64));
        CE_CUDA(cudaMalloc(&b.summ, (size_t)cap * 4 * e.summ + 64));
        CE_CUDA(cudaMalloc(&b.ata, (size_t)cap * 4 * nt * nt * e.ata + 16));
        CE_CUDA(cudaMalloc(&b.atb, (size_t)cap * 2 * nt * e.ata + 16));
        dev_alloc(b.nominal, (size_t)cap);
        dev_alloc(b.fit_counts, (size_t)(MAXT + 1) * MAX_CHUNKS);
        dev_alloc(b.fit_order, (size_t)(MAXT + 1) * cap);
        dev_alloc(b.nominal_list, (size_t)cap);
        // per chunk: listed count, then the work counters of the two FP64 kernels
        dev_alloc(b.nominal_count, (size_t)3 * MAX_CHUNKS);
        dev_alloc(b.sweep_list, (size_t)cap);
        dev_alloc(b.sweep_count, (size_t)MAX_CHUNKS);
        dev_alloc(b.plant_idx, (size_t)cap);
        // shared by the chunks, which the sweep processes one after the other
        const size_t groups = (size_t)(c.freq + SWEEP_FG - 1) / SWEEP_FG;
        CE_CUDA(cudaMalloc(&b.sweep.mag, (size_t)cap * c.freq * e.sweep + 16));
        CE_CUDA(cudaMalloc(&b.sweep.arg, (size_t)cap * c.freq * e.sweep + 16));
        CE_CUDA(cudaMalloc(&b.sweep.bpc, (size_t)cap * groups * e.sweep + 16));
        dev_alloc(b.sweep.fail, (size_t)cap * groups);
        if (c.observer == CE_OBSERVER_KALMAN) {
            // one block: cnt | fill | totals (cleared together) | hoff | poff
            dev_alloc(b.kal.bucket, (size_t)cap);
            dev_alloc(b.kal.cnt, (size_t)4 * KAL_BUCKETS + KAL_TOTALS);
            b.kal.fill = b.kal.cnt + KAL_BUCKETS;
            b.kal.totals = b.kal.fill + KAL_BUCKETS;
            b.kal.hoff = b.kal.totals + KAL_TOTALS;
            b.kal.poff = b.kal.hoff + KAL_BUCKETS;
            dev_alloc(b.kal.order, (size_t)kal_order_size(cap));
            dev_alloc(b.kal.sched, (size_t)KAL_SCHED_STEPS * MAXS * cap);
            dev_alloc(b.kal.meta, (size_t)cap);
            dev_alloc(b.kal.lists, (size_t)2 * cap);
        }
        b.cap = cap;
        b.nt = nt;
        b.pitch = pitch;
        b.precision = s->precision;
    }
    if (traj && n > b.traj_cap) {
        if (b.traj) cudaFree(b.traj);
        b.traj = nullptr;
        dev_alloc(b.traj, (size_t)n * c.time);
        b.traj_cap = n;
    }
}

// The sizes and scalars of configuration c; the row strides and per-candidate
// slots are those of configuration `layout` (c itself for a uniform
// evaluation, the maxima of a ragged batch).
Run run_from_config(const ce_config& c, const ce_config& layout, int64_t n, float alpha, double alpha64) {
    Run r{};
    r.n = n;
    r.ns = c.statespace_dim;
    r.nd = c.discrete_dim;
    r.nt = c.total_dim;
    r.nw = c.nonlin_dim;
    r.time = c.time;
    r.fit_start_id = c.fit_start_id;
    r.fit_steps = c.fit_steps;
    r.fit_pitch = fit_pitch(layout.fit_steps);
    r.steady_start_id = c.steady_start_id;
    r.ref_step_id = c.ref_step_id;
    r.cuda_w = layout.cuda_mx_width;
    r.info_w = layout.info_mx_width;
    r.info_scoring = c.info_scoring;
    r.info_freqresp = c.info_freqresp;
    r.info_allmargin = c.info_allmargin;
    r.info_modal = c.info_modal;
    r.freq = c.freq;
    r.ts = c.ts;
    r.ref_amp = c.ref_amplitude;
    r.fit_t0 = c.fit_t0;
    r.fit_t1 = c.fit_t1;
    r.unstable_err = c.unstable_err;
    r.eig_fail_err = c.eig_fail_err;
    r.bandwidth = c.bandwidth;
    r.damping = c.damping;
    r.overshoot = c.overshoot;
    r.sse = c.steady_state_error;
    r.target_gm = c.target_gm;
    r.target_pm = c.target_pm;
    r.target_b = c.target_b;
    r.alpha = alpha;
    r.alpha64 = alpha64;
    r.store_traj = 0;
    r.kalman = c.observer == CE_OBSERVER_KALMAN ? 1 : 0;
    const int lt = layout.total_dim;
    r.lina_slot = lt * lt;
    r.eig_slot = 2 * lt;
    r.ata_slot = 4 * lt * lt;
    r.atb_slot = 2 * lt;
    r.grid_off = 0;
    return r;
}

Run make_run(const ce_session* s, int plant, int64_t n) {
    return run_from_config(s->cfg, s->cfg, n, s->alpha32[s->grid_of(plant)],
                           s->alpha64.empty() ? 0.0 : s->alpha64[s->grid_of(plant)]);
}

void build_grids(ce_session* s, int precision);

// The per-candidate plant table (MC_FIELDS x n_plants, field-major) and, for
// the mixed-precision form, the simulation kernel compiled for it, built on
// first use.
void ensure_plant_table(ce_session* s, int precision) {
    if (precision == CE_PRECISION_MIXED && !s->sim_kernel_mc) {
        std::string log;
        s->sim_kernel_mc = specialise_sim(s->plants[0], s->cfg.statespace_dim <= 4 ? 4 : 8,
                                          s->cfg.discrete_dim <= 4 ? 4 : 8, log, true,
                                          s->cfg.observer == CE_OBSERVER_KALMAN);
        if (!s->sim_kernel_mc) fail("per-candidate plants need the specialised simulation kernel: {}", log);
    }
    if (s->d_mc_tab) return;
    const int64_t np = s->n_plants;
    std::vector<float> t((size_t)MC_FIELDS * np, 0.0f);
    auto put = [&](int field, int64_t p, float v) { t[(size_t)field * np + p] = v; };
    for (int64_t p = 0; p < np; ++p) {
        const Plant& P = s->plants[p];
        for (int e = 0; e < MAXD * MAXD; ++e) {
            put(MC_AI + e, p, P.d_ai[e]);
            put(MC_A + e, p, P.d_a[e]);
        }
        for (int i = 0; i < MAXD; ++i) {
            put(MC_BU + i, p, P.d_bu[i]);
            put(MC_C + i, p, P.d_c[i]);
        }
        for (int e = 0; e < MAXD * MAXW; ++e) put(MC_BW + e, p, P.d_bw[e]);
        auto consts = [&](const Instr* ins, int cnt, int slot0) {
            for (int k = 0; k < cnt; ++k) {
                put(MC_CST + 2 * (slot0 + k), p, ins[k].aval);
                put(MC_CST + 2 * (slot0 + k) + 1, p, ins[k].bval);
            }
        };
        consts(P.dc, P.n_dc, 0);
        consts(P.u, P.n_u, MAX_DC);
        for (int w = 0; w < MAXW; ++w) consts(P.nl[w], P.n_nl[w], MAX_DC + MAX_U + w * MAX_NL);
    }
    CE_CUDA(cudaMalloc((void**)&s->d_mc_tab, t.size() * sizeof(float)));
    CE_CUDA(cudaMemcpy(s->d_mc_tab, t.data(), t.size() * sizeof(float), cudaMemcpyHostToDevice));
}

// Chunks of one evaluation: 1 below 16,384 candidates per chunk, else
// CE_CHUNKS (default 2: of 1, 2 and 4 chunks, 2 measured fastest on the
// eight-state workload of 65,536 candidates).
// Whether a single-chunk evaluation of n candidates runs the nominal eigensolve
// over all candidates beside LIN_A's (n <= 4,096; CE_NOMINAL_ALL=0 never).
bool concurrent_nominal(int64_t n) {
    static const bool off = [] {
        const char* e = std::getenv("CE_NOMINAL_ALL");
        return e && e[0] == '0';
    }();
    return !off && n <= 4096;
}

int n_chunks(const ce_session* s, int64_t n) {
    static const int dflt = [] {
        const char* e = std::getenv("CE_CHUNKS");
        const int k = e ? std::atoi(e) : 0;
        return (k >= 1 && k <= MAX_CHUNKS) ? k : 2;
    }();
    int k = (s->tuning.chunks >= 1 && s->tuning.chunks <= MAX_CHUNKS) ? s->tuning.chunks : dflt;
    while (k > 1 && n / k < 16384) --k;
    return k;
}

// One evaluation: gains and info rows already on the device in d_gains / d_info.
// With per_candidate, candidate c uses plant `plant + c` (its values from the
// plant table; the instruction structure and the observer model are shared).
// With plant_idx (device, per_candidate only), candidate c uses plant plant_idx[c]
// instead of plant + c; the caller has checked those plants.
void run_pipeline(ce_session* s, int plant, int64_t n, const float* d_gains, float* d_info, cudaStream_t st,
                  bool traj, bool per_candidate = false, const Ragged* ragged = nullptr,
                  const int* plant_idx = nullptr) {
    const int64_t np_used = plant_idx ? 0 : per_candidate ? n : 1;
    for (int64_t q = 0; q < np_used; ++q)
        if (!s->plant_err[plant + q].empty()) throw std::runtime_error(s->plant_err[plant + q]);
    const int prec = s->precision;
    if (grids64(prec) && !s->d_fgrid64) build_grids(s, CE_PRECISION_FP64);
    if (per_candidate) ensure_plant_table(s, sim_precision(prec));
    ensure_buffers(s, n, traj);
    Buffers& b = s->buf;
    Run r = make_run(s, plant, n);
    if (ragged) r.rg = *ragged;
    r.store_traj = traj ? 1 : 0;
    // without the small-batch forms the eigensolves keep two lanes per matrix
    r.eig_lanes = s->tuning.eig_lanes != 0 || s->small_forms ? s->tuning.eig_lanes : 2;
    r.eig_blocks = s->tuning.eig_blocks_per_sm;
    r.eig_fused = s->eig_arith == CE_EIG_ARITH_FUSED ? 1 : 0;
    if (per_candidate) {
        r.mc.tab = s->d_mc_tab;
        r.mc.np = s->n_plants;
        r.mc.first = plant;
        r.mc.grid_stride = s->cfg.serial ? (int64_t)s->cfg.freq * 8 : 0;
        r.mc.alpha = grids64(prec) ? (const void*)s->d_alpha64 : (const void*)s->d_alpha32;
        r.mc.margin = s->cfg.serial ? 1 : 0;
        r.mc.idx = plant_idx;
    }
    const Plant& P = s->plants[plant];
    const size_t goff = (size_t)s->grid_of(plant) * s->cfg.freq * 8;
    const void* fgrid = grids64(prec) ? (const void*)(s->d_fgrid64 + goff) : (const void*)(s->d_fgrid32 + goff);
    // a chunk's grid argument is the grid of its first plant (mc.first); with
    // plant indices every chunk keeps plant 0's
    const size_t gstep = (size_t)(per_candidate && !plant_idx ? r.mc.grid_stride : 0) * (grids64(prec) ? 8 : 4);
    // each launch optionally bracketed by events on the stream it runs on
    auto timed = [&](int stage, cudaStream_t on, auto&& launch) {
        if (!s->profiling) {
            launch();
            return;
        }
        ce_session::Pending pd{stage, s->take_event(), s->take_event()};
        CE_CUDA(cudaEventRecord(pd.a, on));
        launch();
        CE_CUDA(cudaEventRecord(pd.b, on));
        s->pending.push_back(pd);
    };
    // Fork from the caller's stream onto the session's two streams and join
    // back.  The FP64 eigensolves are persistent kernels with a fixed number
    // of blocks per SM, launched first on a high-priority stream so that every
    // SM takes its share of them; the FP32 stages on the other stream fill the
    // rest of each SM and run alongside.  Large batches are cut into chunks so
    // that the fit of a chunk starts as soon as its eigenvalues are known, while
    // the eigensolves of the next chunks continue.
    const int sprec = sim_precision(prec), eprec = eig_precision(prec);
    const SimKernels sk = sprec != CE_PRECISION_MIXED ? SimKernels{} : per_candidate ? s->sim_kernel_mc : s->sim_kernel[plant];
    cudaStream_t fs = s->fast, ss = s->side;
    const int nch = n_chunks(s, n);
    const int64_t per = (n + nch - 1) / nch;
    const BufElems be = buf_elems(prec);
    const int nt = r.nt, cw = r.cuda_w, iw = r.info_w;
    auto chunk = [&](int k, Run& rc, int64_t& off) {
        off = k * per;
        rc = r;
        rc.n = std::min<int64_t>(per, n - off);
        if (r.mc.idx) rc.mc.idx = r.mc.idx + off;
        else rc.mc.first = r.mc.first + off;
        if (r.rg.inst) rc.rg.inst = r.rg.inst + off;
    };
    auto at = [](const void* p, int64_t off, size_t bytes) {
        return (void*)((const char*)p + (size_t)off * bytes);
    };
    // A small single-chunk batch in mixed precision runs the nominal eigensolve
    // over all its candidates on a third stream, concurrently with LIN_A's,
    // instead of over LIN_A's list after it: the two are independent, and a
    // batch that small leaves the GPU room for both.  Their work counters are
    // cleared here, before either stream starts.
    const bool nom_all = s->small_forms && nch == 1 && prec == CE_PRECISION_MIXED && !ragged && concurrent_nominal(n);
    cudaStream_t ns2 = s->side2;
    if (nom_all) CE_CUDA(cudaMemsetAsync(b.nominal_count, 0, 3 * sizeof(int), st));
    CE_CUDA(cudaEventRecord(s->ev_fork, st));
    CE_CUDA(cudaStreamWaitEvent(fs, s->ev_fork, 0));
    CE_CUDA(cudaStreamWaitEvent(ss, s->ev_fork, 0));
    if (nom_all) CE_CUDA(cudaStreamWaitEvent(ns2, s->ev_fork, 0));
    for (int k = 0; k < nch; ++k) {
        Run rc;
        int64_t off;
        chunk(k, rc, off);
        timed(0, ss, [&] {
            launch_lina_eig(rc, P, eprec, d_gains + off * cw, at(b.lina, off, nt * nt * be.lina), at(b.eig, off, 2 * nt * be.eig),
                            b.nominal + off, nom_all ? nullptr : b.nominal_list + off, b.nominal_count + 3 * k, ss,
                            !nom_all);
        });
        CE_CUDA(cudaEventRecord(s->ev_eig[k], ss));
    }
    for (int k = 0; k < nch; ++k) {
        Run rc;
        int64_t off;
        chunk(k, rc, off);
        cudaStream_t on = nom_all ? ns2 : ss;
        timed(4, on, [&] {
            launch_nominal(rc, P, eprec, d_gains + off * cw, at(b.lina, off, nt * nt * be.lina),
                           nom_all ? nullptr : b.nominal_list + off, b.nominal_count + 3 * k, b.nominal + off, on);
        });
        CE_CUDA(cudaEventRecord(s->ev_nom[k], on));
    }
    timed(1, fs, [&] {
        float* tr = traj ? b.traj : nullptr;
        if (r.kalman) {
            // Kalman observer: group the candidates by noise weights, then the
            // shared-noise form over whole warps of a group and the
            // per-candidate form over the rest
            launch_kalman_groups(r, d_gains, b.kal, fs);
            Run rh = r;
            rh.kal_order = b.kal.order;
            rh.kal_totals = b.kal.totals;
            rh.kal_defer = kal_shared_slots(n) + n;
            rh.kal_sched = b.kal.sched;
            rh.kal_meta = b.kal.meta;
            rh.kal_lists = b.kal.lists;
            rh.kal_sched_n = b.cap;
            rh.kal_list = 1;
            // the per-candidate list: gain schedules, then the scheduled form over the
            // positions whose schedule turned periodic and, on a third stream beside
            // it, the quad form over the rest (the two lists are disjoint)
            Run rp = rh, ra = rh, rb = rh;
            rp.kal_list = 2;
            ra.kal_list = 3;
            rb.kal_list = 4;
            cudaStream_t qs = s->side3;
            if (sk) launch_sim_specialised(sk.shared, rh, P, d_gains, (float*)b.ywin, (SimSummary*)b.summ, tr, fs);
            else launch_sim(rh, P, sprec, d_gains, b.ywin, b.summ, tr, fs);
            // the schedules and the quad form on the high-priority stream: with
            // per-candidate noise they are the step's critical path
            CE_CUDA(cudaEventRecord(s->ev_kal, fs));
            CE_CUDA(cudaStreamWaitEvent(qs, s->ev_kal, 0));
            launch_kalman_schedule(rp, P, d_gains, b.kal, qs);
            CE_CUDA(cudaEventRecord(s->ev_kal, qs));
            CE_CUDA(cudaStreamWaitEvent(fs, s->ev_kal, 0));
            if (sk) {
                launch_sim_specialised(sk.quad, rb, P, d_gains, (float*)b.ywin, (SimSummary*)b.summ, tr, qs);
                launch_sim_specialised(sk.sched, ra, P, d_gains, (float*)b.ywin, (SimSummary*)b.summ, tr, fs);
            } else {
                launch_sim(rb, P, sprec, d_gains, b.ywin, b.summ, tr, qs);
                launch_sim(ra, P, sprec, d_gains, b.ywin, b.summ, tr, fs);
            }
            CE_CUDA(cudaEventRecord(s->ev_kal_quad, qs));
            CE_CUDA(cudaStreamWaitEvent(fs, s->ev_kal_quad, 0));
        } else if (sk) {
            // a batch too small to fill the GPU runs four lanes per candidate
            const bool wide = s->small_forms && sk.wide &&
                              use_wide_sim(n, s->cfg.statespace_dim <= 4 ? 4 : 8, s->cfg.discrete_dim <= 4 ? 4 : 8);
            launch_sim_specialised(wide ? sk.wide : sk.main, r, P, d_gains, (float*)b.ywin, (SimSummary*)b.summ, tr,
                                   fs, wide);
        } else {
            launch_sim(r, P, sprec, d_gains, b.ywin, b.summ, tr, fs);
        }
    });
    for (int k = 0; k < nch; ++k) {
        Run rc;
        int64_t off;
        chunk(k, rc, off);
        CE_CUDA(cudaStreamWaitEvent(fs, s->ev_eig[k], 0));
        const void* eig = at(b.eig, off, 2 * nt * be.eig);
        void* ata = at(b.ata, off, 4 * nt * nt * be.ata);
        void* atb = at(b.atb, off, 2 * nt * be.ata);
        const void* ywin = at(b.ywin, off, (size_t)r.fit_pitch * be.ywin);
        const void* summ = at(b.summ, off, 4 * be.summ);
        timed(2, fs, [&] {
            if (compensated(prec))
                launch_fit_comp(rc, sim_double(prec), eig, ywin, summ, ata, atb,
                                d_info + off * iw, b.fit_counts + (MAXT + 1) * k, b.fit_order + (MAXT + 1) * off,
                                fs);
            else
                launch_fit(rc, prec, eig, ywin, summ, ata, atb, d_info + off * iw, b.fit_counts + (MAXT + 1) * k,
                           b.fit_order + (MAXT + 1) * off, fs);
        });
        timed(3, fs, [&] { launch_modal(rc, prec, eig, ata, atb, d_info + off * iw, fs); });
    }
    for (int k = 0; k < nch; ++k) {
        Run rc;
        int64_t off;
        chunk(k, rc, off);
        CE_CUDA(cudaStreamWaitEvent(fs, s->ev_nom[k], 0));
        timed(5, fs, [&] {
            launch_sweep(rc, eprec, d_gains + off * cw, at(b.lina, off, nt * nt * be.lina), b.nominal + off, at(fgrid, off, gstep),
                         d_info + off * iw, b.sweep_list + off, b.sweep_count + k, b.sweep, fs);
        });
    }
    CE_CUDA(cudaEventRecord(s->ev_done, fs));
    CE_CUDA(cudaStreamWaitEvent(st, s->ev_done, 0));
    // Kalman: three grouping kernels, the gain schedules and two more simulation forms
    s->launches += 1 + 8 * nch + (r.kalman ? 6 : 0);
}

std::vector<Instr> compact(const std::vector<ce_instruction>& rows) {
    std::vector<Instr> out;
    for (const auto& r : rows)
        if (r.op != 0) out.push_back(Instr{r.op, r.col, r.akind, r.bkind, r.aval, r.bval});
    return out;
}

// Build the padded plant of round `p` (ref: src/main.cu:341-383, 390-397).
void build_plant(const ce_config& c, const ce_plant& in, int p, Plant& P) {
    std::memset(&P, 0, sizeof(P));
    const int ns = c.statespace_dim, nd = c.discrete_dim, nw = c.nonlin_dim;
    for (int i = 0; i < ns; ++i) {
        for (int j = 0; j < ns; ++j) {
            P.ss_a[i * MAXS + j] = in.statespace_a[i * ns + j];
            P.ss_ai[i * MAXS + j] = in.statespace_a_i[i * ns + j];
        }
        P.ss_b[i] = in.statespace_b[i];
        P.ss_c[i] = in.statespace_c[i];
    }
    P.ss_d = in.statespace_d[0];
    const size_t oa = (size_t)p * nd * nd, ov = (size_t)p * nd, ow = (size_t)p * nd * nw;
    for (int i = 0; i < nd; ++i) {
        for (int j = 0; j < nd; ++j) {
            P.d_a[i * MAXD + j] = in.discrete_a[oa + i * nd + j];
            P.d_ai[i * MAXD + j] = in.discrete_a_i[oa + i * nd + j];
        }
        P.d_bu[i] = in.discrete_bu[ov + i];
        for (int k = 0; k < nw; ++k) P.d_bw[i * MAXW + k] = in.discrete_bw[ow + i * nw + k];
        P.d_c[i] = in.discrete_c[ov + i];
    }
    // margin plant: observer model (batch) or the true linear plant (serial)
    if (c.serial) {
        for (int i = 0; i < nd; ++i) {
            for (int j = 0; j < nd; ++j) P.m_a[i * MAXS + j] = P.d_a[i * MAXD + j];
            P.m_b[i] = P.d_bu[i];
            P.m_c[i] = P.d_c[i];
        }
        P.m_d = 0.0f;
    } else {
        for (int i = 0; i < ns; ++i) {
            for (int j = 0; j < ns; ++j) P.m_a[i * MAXS + j] = P.ss_a[i * MAXS + j];
            P.m_b[i] = P.ss_b[i];
            P.m_c[i] = P.ss_c[i];
        }
        P.m_d = P.ss_d;
    }
    // instruction tables, decoded with this round's BASE_PARAMS
    const float* bp = in.base_params + (size_t)p * c.n_params;
    std::vector<ce_instruction> rows;
    rows.resize(std::max(c.dc_instructions, 1));
    decode_instructions(in.dc_info, c.dc_dim, c.dc_instructions, bp, c.n_params, rows.data());
    rows.resize(c.dc_instructions);
    auto dc = compact(rows);
    rows.assign(std::max(c.u_instructions, 1), ce_instruction{});
    decode_instructions(in.u_info, c.u_dim, c.u_instructions, bp, c.n_params, rows.data());
    rows.resize(c.u_instructions);
    auto u = compact(rows);
    P.n_dc = (int)dc.size();
    P.n_u = (int)u.size();
    for (int i = 0; i < P.n_dc; ++i) P.dc[i] = dc[i];
    for (int i = 0; i < P.n_u; ++i) P.u[i] = u[i];
    int row = 0;
    for (int i = 0; i < c.nonlin_dim; ++i) {
        const int cnt = c.nl_instructions[i];
        rows.assign(std::max(cnt, 1), ce_instruction{});
        decode_instructions(in.nl_info + (size_t)row * c.nl_dim, c.nl_dim, cnt, bp, c.n_params, rows.data());
        rows.resize(cnt);
        for (auto& r : rows)
            if (r.col == c.discrete_dim) r.col = MAXD;  // plant output slot (ref: src/main.cu:377)
        auto nl = compact(rows);
        P.n_nl[i] = (int)nl.size();
        for (int k = 0; k < P.n_nl[i]; ++k) P.nl[i][k] = nl[k];
        row += cnt;
    }
}

// The sweep grid and the margin plants' response on it, with the plant scaling
// at the crossover (ref: src/main.cu:421-428, src/allmargin.cu:20-41).  The z
// grid is formed here with host float libm, as in the reference; P(z_w) and
// alpha run on the device for all margin plants at once (k_plant_grid).  A
// margin plant without a finite nonzero gain at the crossover makes its
// evaluations fail with the reference's message.
// The z grid of a configuration in float (ref: src/main.cu:424-428, host float
// libm): per frequency z = (cos, sin) of theta_w = exp(log fmin + w*inc)*ts and
// arg z; row F is the crossover e^{j w_c ts} (ref: src/allmargin.cu:36-38).
std::vector<float> zgrid32(const ce_config& c) {
    const int F = c.freq;
    std::vector<float> z32((size_t)(F + 1) * 4, 0.0f);
    const float inc = (logf(c.freq_max) - logf(c.freq_min)) / (float)(F - 1);
    for (int w = 0; w < F; ++w) {
        const float th = expf(logf(c.freq_min) + inc * (float)w) * c.ts;
        z32[4 * w] = cosf(th);
        z32[4 * w + 1] = sinf(th);
        z32[4 * w + 2] = std::atan2(z32[4 * w + 1], z32[4 * w]);
    }
    const float th = c.crossover * c.ts;
    z32[4 * F] = 1.0f * cosf(th);
    z32[4 * F + 1] = 1.0f * sinf(th);
    return z32;
}

void build_grids(ce_session* s, int precision) {
    const ce_config& c = s->cfg;
    const int F = c.freq, n = c.serial ? c.discrete_dim : c.statespace_dim, np = s->grid_np;
    const bool f64 = precision == CE_PRECISION_FP64;
    const size_t rsz = f64 ? sizeof(double) : sizeof(float);
    std::vector<double> z64((size_t)(F + 1) * 4, 0.0);
    const std::vector<float> z32 = zgrid32(c);
    const double inc64 = (std::log((double)c.freq_max) - std::log((double)c.freq_min)) / (double)(F - 1);
    for (int w = 0; w < F; ++w) {
        const double th64 = std::exp(std::log((double)c.freq_min) + inc64 * (double)w) * (double)c.ts;
        z64[4 * w] = std::cos(th64);
        z64[4 * w + 1] = std::sin(th64);
        z64[4 * w + 2] = std::atan2(z64[4 * w + 1], z64[4 * w]);
    }
    {
        const double th64 = (double)c.crossover * (double)c.ts;
        z64[4 * F] = std::cos(th64);
        z64[4 * F + 1] = std::sin(th64);
    }
    const int ms = margin_plant_stride();
    if (!s->d_mplant) {
        std::vector<float> mp((size_t)np * ms, 0.0f);
        for (int p = 0; p < np; ++p) {
            const Plant& P = s->plants[p];
            float* m = mp.data() + (size_t)p * ms;
            std::memcpy(m, P.m_a, sizeof(P.m_a));
            std::memcpy(m + MAXS * MAXS, P.m_b, sizeof(P.m_b));
            std::memcpy(m + MAXS * MAXS + MAXS, P.m_c, sizeof(P.m_c));
            m[MAXS * MAXS + 2 * MAXS] = P.m_d;
        }
        CE_CUDA(cudaMalloc((void**)&s->d_mplant, mp.size() * sizeof(float)));
        CE_CUDA(cudaMemcpy(s->d_mplant, mp.data(), mp.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    void* zg = nullptr;
    void* alpha = nullptr;
    int* bad = nullptr;
    void* grid = nullptr;
    CE_CUDA(cudaMalloc(&zg, (size_t)(F + 1) * 4 * rsz));
    CE_CUDA(cudaMalloc(&alpha, (size_t)np * rsz));
    CE_CUDA(cudaMalloc((void**)&bad, (size_t)np * sizeof(int)));
    CE_CUDA(cudaMalloc(&grid, (size_t)np * F * 8 * rsz));
    std::unique_ptr<void, cudaError_t (*)(void*)> g1(zg, cudaFree), g3(bad, cudaFree);
    (f64 ? s->d_alpha64 : s->d_alpha32) = alpha;
    if (f64) CE_CUDA(cudaMemcpy(zg, z64.data(), z64.size() * sizeof(double), cudaMemcpyHostToDevice));
    else CE_CUDA(cudaMemcpy(zg, z32.data(), z32.size() * sizeof(float), cudaMemcpyHostToDevice));
    launch_plant_grid(precision, np, n, F, s->d_mplant, zg, grid, alpha, bad, s->stream);
    std::vector<int> hbad(np);
    CE_CUDA(cudaMemcpyAsync(hbad.data(), bad, (size_t)np * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    if (f64) {
        s->alpha64.resize(np);
        CE_CUDA(cudaMemcpyAsync(s->alpha64.data(), alpha, (size_t)np * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        s->d_fgrid64 = (double*)grid;
    } else {
        s->alpha32.resize(np);
        CE_CUDA(cudaMemcpyAsync(s->alpha32.data(), alpha, (size_t)np * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
        s->d_fgrid32 = (float*)grid;
    }
    CE_CUDA(cudaStreamSynchronize(s->stream));
    if (!f64)
        for (int p = 0; p < s->n_plants; ++p)
            if (hbad[s->grid_of(p)])
                s->plant_err[p] = std::format("allmargin: plant has no finite nonzero gain at crossover = {} rad/s", c.crossover);
}

// Select the simulation kernel of every plant.  CE_SIM_SPECIALISED compiles
// each distinct instruction program once per process (NVRTC); a failure throws
// with the compiler's log and leaves the session's kernels unchanged.
void select_sim_kernel(ce_session* s, int kind) {
    std::vector<SimKernels> ks(s->n_plants);
    if (kind == CE_SIM_SPECIALISED) {
        // the plants of a session share the DC/U/NL tables, so the programs'
        // structure is the same for all of them: one compiled kernel serves all
        std::string log;
        const SimKernels k = specialise_sim(s->plants[0], s->cfg.statespace_dim <= 4 ? 4 : 8,
                                       s->cfg.discrete_dim <= 4 ? 4 : 8, log, false,
                                       s->cfg.observer == CE_OBSERVER_KALMAN);
        if (!k) fail("specialising the simulation kernel failed: {}", log);
        ks.assign(s->n_plants, k);
    }
    s->sim_kernel = ks;
    s->sim_kind = kind;
}

void check_config(const ce_config& c, const char* who) {
    if (c.statespace_dim < 1 || c.statespace_dim > MAXS || c.discrete_dim < 1 || c.discrete_dim > MAXD ||
        c.nonlin_dim < 0 || c.nonlin_dim > MAXW || c.total_dim != c.statespace_dim + c.discrete_dim)
        fail("{}: config dimensions are out of range or not derived", who);
    if (c.dc_dim != c.discrete_dim || c.u_dim != c.statespace_dim || c.nl_dim != c.discrete_dim + 1)
        fail("{}: instruction table widths are not derived from the dimensions", who);
    if (c.observer != CE_OBSERVER_LUENBERGER && c.observer != CE_OBSERVER_KALMAN)
        fail("{}: unknown observer {}", who, c.observer);
    if (c.cuda_mx_width != (c.observer == CE_OBSERVER_KALMAN ? 3 : 2) * c.statespace_dim +
                               (c.observer == CE_OBSERVER_KALMAN ? 2 : 1))
        fail("{}: cuda_mx_width is not derived from the dimensions and the observer", who);
}

// The session's streams and events: `stream` for host-buffer evaluations, `fast`
// (lowest priority) for the FP32 stages, `side` (highest) for the FP64 eigensolves.
void init_streams(ce_session* s) {
    CE_CUDA(cudaGetDevice(&s->device));
    CE_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    int prio_least = 0, prio_greatest = 0;
    CE_CUDA(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
    CE_CUDA(cudaStreamCreateWithPriority(&s->fast, cudaStreamNonBlocking, prio_least));
    CE_CUDA(cudaStreamCreateWithPriority(&s->side, cudaStreamNonBlocking, prio_greatest));
    CE_CUDA(cudaStreamCreateWithPriority(&s->side2, cudaStreamNonBlocking, prio_greatest));
    CE_CUDA(cudaStreamCreateWithPriority(&s->side3, cudaStreamNonBlocking, prio_greatest));
    CE_CUDA(cudaEventCreateWithFlags(&s->ev_done, cudaEventDisableTiming));
    CE_CUDA(cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming));
    CE_CUDA(cudaEventCreateWithFlags(&s->ev_kal, cudaEventDisableTiming));
    CE_CUDA(cudaEventCreateWithFlags(&s->ev_kal_quad, cudaEventDisableTiming));
    for (int k = 0; k < MAX_CHUNKS; ++k) {
        CE_CUDA(cudaEventCreateWithFlags(&s->ev_eig[k], cudaEventDisableTiming));
        CE_CUDA(cudaEventCreateWithFlags(&s->ev_nom[k], cudaEventDisableTiming));
    }
}

void create_session(const ce_config* cfg_in, const ce_plant* plant, int n_plants, ce_session** out) {
    if (!cfg_in || !plant || !out) fail("ce_session_create: null argument");
    if (n_plants < 1) fail("ce_session_create: n_plants must be >= 1, got {}", n_plants);
    auto s = std::make_unique<ce_session>();
    s->cfg = *cfg_in;
    const ce_config& c = s->cfg;
    check_config(c, "ce_session_create");
    s->n_plants = n_plants;
    s->plants.resize(n_plants);
    s->plant_err.assign(n_plants, std::string());
    s->grid_np = c.serial ? n_plants : 1;
    for (int p = 0; p < n_plants; ++p) build_plant(c, *plant, p, s->plants[p]);
    init_streams(s.get());
    build_grids(s.get(), CE_PRECISION_MIXED);
    // Default: the specialised kernel.  CE_SIM_KERNEL=table in the environment
    // selects the table-driven one; if compiling fails the session keeps the
    // table-driven kernel and ce_session_sim_kernel reports which one runs.
    s->sim_kernel.assign(n_plants, SimKernels{});
    s->sim_kind = CE_SIM_TABLE;
    const char* env = std::getenv("CE_SIM_KERNEL");
    if (!(env && std::string(env) == "table")) {
        try {
            select_sim_kernel(s.get(), CE_SIM_SPECIALISED);
        } catch (const std::exception& e) {
            s->sim_log = e.what();
        }
    }
    *out = s.release();
}

void collect_stage_times(ce_session* s) {
    for (auto& pd : s->pending) {
        CE_CUDA(cudaEventSynchronize(pd.b));
        float ms = 0.0f;
        CE_CUDA(cudaEventElapsedTime(&ms, pd.a, pd.b));
        s->stage_ms[pd.stage] += ms;
        s->stage_n[pd.stage] += 1;
        s->event_pool.push_back(pd.a);
        s->event_pool.push_back(pd.b);
    }
    s->pending.clear();
}

void destroy_session(ce_session* s) {
    if (!s) return;
    for (auto& pd : s->pending) {
        cudaEventDestroy(pd.a);
        cudaEventDestroy(pd.b);
    }
    for (cudaEvent_t e : s->event_pool) cudaEventDestroy(e);
    s->buf.release();
    if (s->d_fgrid32) cudaFree(s->d_fgrid32);
    if (s->d_fgrid64) cudaFree(s->d_fgrid64);
    if (s->d_mplant) cudaFree(s->d_mplant);
    if (s->d_alpha32) cudaFree(s->d_alpha32);
    if (s->d_alpha64) cudaFree(s->d_alpha64);
    if (s->d_mc_tab) cudaFree(s->d_mc_tab);
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_kal) cudaEventDestroy(s->ev_kal);
    if (s->ev_kal_quad) cudaEventDestroy(s->ev_kal_quad);
    for (int k = 0; k < MAX_CHUNKS; ++k) {
        if (s->ev_eig[k]) cudaEventDestroy(s->ev_eig[k]);
        if (s->ev_nom[k]) cudaEventDestroy(s->ev_nom[k]);
    }
    if (s->stream) cudaStreamDestroy(s->stream);
    if (s->side) cudaStreamDestroy(s->side);
    if (s->side2) cudaStreamDestroy(s->side2);
    if (s->side3) cudaStreamDestroy(s->side3);
    if (s->fast) cudaStreamDestroy(s->fast);
    if (s->ev_done) cudaEventDestroy(s->ev_done);
    delete s;
}

void check_eval(ce_session* s, int plant, int64_t n) {
    if (!s) fail("null session");
    if (plant < 0 || plant >= s->n_plants) fail("plant index {} out of range [0, {})", plant, s->n_plants);
    if (n < 0) fail("candidate count {} is negative", n);
}

void check_plants(ce_session* s, int first, int64_t n) {
    check_eval(s, first, n);
    if (first + n > s->n_plants)
        fail("plants [{}, {}) exceed the session's {} plants (one plant per candidate)", first, first + n, s->n_plants);
}

void evaluate_host(ce_session* s, int plant, int64_t n, const float* cuda_mx, const float* info_in, float* info_out,
                   const ce_diagnostics* diag, bool per_candidate = false) {
    if (per_candidate) check_plants(s, plant, n);
    else check_eval(s, plant, n);
    if (n == 0) return;
    const ce_config& c = s->cfg;
    const bool traj = diag && diag->yplant;
    ensure_buffers(s, n, traj);
    Buffers& b = s->buf;
    cudaStream_t st = s->stream;
    CE_CUDA(cudaMemcpyAsync(b.gains, cuda_mx, (size_t)n * c.cuda_mx_width * sizeof(float), cudaMemcpyHostToDevice, st));
    CE_CUDA(cudaMemcpyAsync(b.info, info_in, (size_t)n * c.info_mx_width * sizeof(float), cudaMemcpyHostToDevice, st));
    run_pipeline(s, plant, n, b.gains, b.info, st, traj, per_candidate);
    CE_CUDA(cudaMemcpyAsync(info_out, b.info, (size_t)n * c.info_mx_width * sizeof(float), cudaMemcpyDeviceToHost, st));
    const int nt = c.total_dim;
    const BufElems be = buf_elems(s->precision);
    std::vector<double> tmp;
    if (diag) {
        if (diag->yplant)
            CE_CUDA(cudaMemcpyAsync(diag->yplant, b.traj, (size_t)n * c.time * sizeof(float), cudaMemcpyDeviceToHost, st));
    }
    CE_CUDA(cudaStreamSynchronize(st));
    if (diag) {
        auto pull = [&](float* dst, const void* src, size_t count, size_t bytes) {
            if (!dst) return;
            if (bytes == sizeof(float)) {
                CE_CUDA(cudaMemcpy(dst, src, count * sizeof(float), cudaMemcpyDeviceToHost));
            } else {
                tmp.resize(count);
                CE_CUDA(cudaMemcpy(tmp.data(), src, count * sizeof(double), cudaMemcpyDeviceToHost));
                for (size_t i = 0; i < count; ++i) dst[i] = (float)tmp[i];
            }
        };
        pull(diag->lina, b.lina, (size_t)n * nt * nt, be.lina);
        pull(diag->eigen, b.eig, (size_t)n * 2 * nt, be.eig);
        pull(diag->ata, b.ata, (size_t)n * 4 * nt * nt, be.ata);
        pull(diag->atb, b.atb, (size_t)n * 2 * nt, be.ata);
    }
}

// Device buffer of n records of `count` elements (`stride` elements apart,
// `bytes` each: 4 = float, 8 = double) into n x count doubles.
void pull64(double* dst, const void* src, int64_t n, int64_t count, int64_t stride, size_t bytes) {
    if (!dst) return;
    std::vector<char> h((size_t)n * stride * bytes);
    CE_CUDA(cudaMemcpy(h.data(), src, h.size(), cudaMemcpyDeviceToHost));
    for (int64_t c = 0; c < n; ++c)
        for (int64_t k = 0; k < count; ++k) {
            const char* e = h.data() + ((size_t)c * stride + k) * bytes;
            dst[c * count + k] = bytes == 8 ? *(const double*)e : (double)*(const float*)e;
        }
}

void evaluate_host64(ce_session* s, int plant, int64_t n, const float* cuda_mx, const float* info_in,
                     float* info_out, const ce_diagnostics64* diag) {
    evaluate_host(s, plant, n, cuda_mx, info_in, info_out, nullptr);
    if (!diag || n == 0) return;
    const ce_config& c = s->cfg;
    const Buffers& b = s->buf;
    const int64_t nt = c.total_dim;
    const BufElems e = buf_elems(s->precision);
    pull64(diag->ywin, b.ywin, n, c.fit_steps, fit_pitch(c.fit_steps), e.ywin);
    pull64(diag->summ, b.summ, n, 4, 4, e.summ);
    pull64(diag->lina, b.lina, n, nt * nt, nt * nt, e.lina);
    pull64(diag->eigen, b.eig, n, 2 * nt, 2 * nt, e.eig);
    pull64(diag->ata, b.ata, n, 4 * nt * nt, 4 * nt * nt, e.ata);
    pull64(diag->atb, b.atb, n, 2 * nt, 2 * nt, e.ata);
}

// ---- file boundary ----------------------------------------------------------
std::string read_text(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) fail("Cannot open {}", path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

// ref: src/main.cu:294-302 -- exact size check over `slices` stacked copies
template <typename T>
std::vector<T> readbin(size_t count, const std::string& filename, int slices = 1) {
    const size_t nbytes = count * sizeof(T);
    std::ifstream file(filename, std::ios::binary);
    if (!file) fail("Cannot open {}", filename);
    file.seekg(0, std::ios::end);
    const size_t expected = nbytes * slices;
    const std::streamoff actual = file.tellg();
    if (actual != static_cast<std::streamoff>(expected))
        fail("{} is {} bytes, expected {} ({} x {})", filename, (long long)actual, expected, slices, nbytes);
    file.seekg(0, std::ios::beg);
    std::vector<T> v(count * slices);
    if (!v.empty()) {
        file.read(reinterpret_cast<char*>(v.data()), expected);
        if (!file) fail("Cannot read {} (intended {}-byte allocation)", filename, nbytes);
    }
    return v;
}

void write_bin(const std::string& name, const void* p, size_t bytes) {
    std::ofstream f(name, std::ios::binary);
    if (!f) fail("Cannot open {}", name);
    f.write(reinterpret_cast<const char*>(p), (std::streamsize)bytes);
}

// The rounds of a file run without diagnostics, double-buffered: while round
// r is on the GPU (H2D, the pipeline and D2H enqueued on the session stream),
// the host writes round r-1's rows to INFO_MX_OUT.bin and reads round r+1 from
// CUDA_MX.bin / INFO_MX.bin into the other pinned slot.  Rounds are written in
// order; a read failure of round r+1 surfaces after round r has been written,
// as in a sequential run.
template <typename Read>
void stream_rounds(ce_session* s, const ce_config& c, Read&& read_round, std::ofstream& out) {
    const size_t nthr = (size_t)c.n_threads, cw = c.cuda_mx_width, iw = c.info_mx_width;
    struct Slot {
        float *hg = nullptr, *hi = nullptr, *dg = nullptr, *di = nullptr;
        cudaEvent_t done = nullptr;
    } slot[2];
    auto release = [&] {
        for (Slot& k : slot) {
            if (k.hg) cudaFreeHost(k.hg);
            if (k.hi) cudaFreeHost(k.hi);
            if (k.dg) cudaFree(k.dg);
            if (k.di) cudaFree(k.di);
            if (k.done) cudaEventDestroy(k.done);
        }
    };
    std::unique_ptr<Slot, std::function<void(Slot*)>> guard(slot, [&](Slot*) {
        cudaStreamSynchronize(s->stream);
        release();
    });
    for (Slot& k : slot) {
        CE_CUDA(cudaMallocHost((void**)&k.hg, nthr * cw * sizeof(float)));
        CE_CUDA(cudaMallocHost((void**)&k.hi, nthr * iw * sizeof(float)));
        CE_CUDA(cudaMalloc((void**)&k.dg, nthr * cw * sizeof(float)));
        CE_CUDA(cudaMalloc((void**)&k.di, nthr * iw * sizeof(float)));
        CE_CUDA(cudaEventCreateWithFlags(&k.done, cudaEventDisableTiming));
    }
    cudaStream_t st = s->stream;
    auto write_round = [&](Slot& k) {
        CE_CUDA(cudaEventSynchronize(k.done));
        out.write(reinterpret_cast<char*>(k.hi), nthr * iw * sizeof(float));
    };
    read_round(0, slot[0].hg, slot[0].hi);
    for (int round = 0; round < c.n_rounds; round++) {
        Slot& k = slot[round & 1];
        CE_CUDA(cudaMemcpyAsync(k.dg, k.hg, nthr * cw * sizeof(float), cudaMemcpyHostToDevice, st));
        CE_CUDA(cudaMemcpyAsync(k.di, k.hi, nthr * iw * sizeof(float), cudaMemcpyHostToDevice, st));
        run_pipeline(s, c.serial ? round : 0, (int64_t)nthr, k.dg, k.di, st, false);
        CE_CUDA(cudaMemcpyAsync(k.hi, k.di, nthr * iw * sizeof(float), cudaMemcpyDeviceToHost, st));
        CE_CUDA(cudaEventRecord(k.done, st));
        if (round + 1 < c.n_rounds) {
            Slot& other = slot[(round + 1) & 1];
            if (round >= 1) write_round(other);  // round - 1
            read_round(round + 1, other.hg, other.hi);
        }
    }
    if (c.n_rounds >= 2) write_round(slot[(c.n_rounds - 2) & 1]);
    if (c.n_rounds >= 1) write_round(slot[(c.n_rounds - 1) & 1]);
}

void run_files() {
    ce_config c;
    parse_config(read_text("ControllerEngine.config"), "ControllerEngine.config", c);
    const int ns = c.statespace_dim, nd = c.discrete_dim;
    const int slices = c.serial ? c.n_rounds : 1;
    // same read order as init64KB / upload_plant (ref: src/main.cu:341-399)
    auto ssa = readbin<float>((size_t)ns * ns, "STATESPACE_A.bin");
    auto ssai = readbin<float>((size_t)ns * ns, "STATESPACE_A_I.bin");
    auto ssb = readbin<float>((size_t)ns, "STATESPACE_B.bin");
    auto ssc = readbin<float>((size_t)ns, "STATESPACE_C.bin");
    auto ssd = readbin<float>(1, "STATESPACE_D.bin");
    auto da = readbin<float>((size_t)nd * nd, "DISCRETE_A.bin", slices);
    auto dbu = readbin<float>((size_t)nd, "DISCRETE_BU.bin", slices);
    auto dbw = readbin<float>((size_t)nd * c.nonlin_dim, "DISCRETE_BW.bin", slices);
    auto dc = readbin<float>((size_t)nd, "DISCRETE_C.bin", slices);
    auto dai = readbin<float>((size_t)nd * nd, "DISCRETE_A_I.bin", slices);
    auto bp = readbin<float>((size_t)c.n_params, "BASE_PARAMS.bin", slices);
    auto dci = readbin<int32_t>((size_t)c.dc_dim * c.dc_instructions, "DC_INFO.bin");
    auto ui = readbin<int32_t>((size_t)c.u_dim * c.u_instructions, "U_INFO.bin");
    auto nli = readbin<int32_t>((size_t)c.nl_dim * c.nl_instructions_total, "NL_INFO.bin");
    ce_plant pl{ssa.data(), ssai.data(), ssb.data(), ssc.data(), ssd.data(), da.data(), dai.data(), dbu.data(),
                dbw.data(), dc.data(), bp.data(), dci.data(), ui.data(), nli.data()};
    ce_session* raw = nullptr;
    create_session(&c, &pl, slices, &raw);
    std::unique_ptr<ce_session, void (*)(ce_session*)> s(raw, destroy_session);

    {
        std::ofstream plog("params.log");
        plog << std::scientific << std::setprecision(9);
        for (int i = 0; i < c.n_params; i++) plog << "BASE_PARAMS_HOST[" << i << "] = " << bp[i] << "\n";
        plog << "ref amplitude = " << c.ref_amplitude << "\n";
    }
    const size_t nthr = (size_t)c.n_threads;
    const size_t cw = c.cuda_mx_width, iw = c.info_mx_width;
    std::ifstream cudamx("CUDA_MX.bin", std::ios::binary);
    if (!cudamx) fail("Cannot open CUDA_MX.bin");
    cudamx.seekg(0, std::ios::end);
    const std::streamoff cexp = (std::streamoff)((size_t)c.n_rounds * nthr * cw * sizeof(float));
    if (cudamx.tellg() != cexp)
        fail("CUDA_MX.bin is {} bytes, expected {} ({} rounds x {} candidates)", (long long)cudamx.tellg(),
             (long long)cexp, c.n_rounds, c.n_threads);
    cudamx.seekg(0, std::ios::beg);
    std::ifstream infomx("INFO_MX.bin", std::ios::binary);
    if (!infomx) fail("Cannot open INFO_MX.bin");
    infomx.seekg(0, std::ios::end);
    const std::streamoff iexp = (std::streamoff)((size_t)c.n_rounds * nthr * iw * sizeof(float));
    if (infomx.tellg() != iexp)
        fail("INFO_MX.bin is {} bytes, expected {} ({} rounds x {} candidates)", (long long)infomx.tellg(),
             (long long)iexp, c.n_rounds, c.n_threads);
    infomx.seekg(0, std::ios::beg);
    std::ofstream infoout("INFO_MX_OUT.bin", std::ios::binary);
    if (!infoout) fail("Cannot open INFO_MX_OUT.bin");

    float *hc_mx = nullptr, *hinfo = nullptr;
    CE_CUDA(cudaMallocHost((void**)&hc_mx, nthr * cw * sizeof(float)));
    CE_CUDA(cudaMallocHost((void**)&hinfo, nthr * iw * sizeof(float)));
    std::unique_ptr<float, cudaError_t (*)(void*)> g1(hc_mx, cudaFreeHost), g2(hinfo, cudaFreeHost);
    const int nt = c.total_dim;
    std::vector<float> dy, dl, de, da2, db;
    ce_diagnostics dg{};
    if (c.dump_diagnostics) {
        dy.resize(nthr * c.time);
        dl.resize(nthr * nt * nt);
        de.resize(nthr * 2 * nt);
        da2.resize(nthr * 4 * nt * nt);
        db.resize(nthr * 2 * nt);
        dg = ce_diagnostics{dy.data(), dl.data(), de.data(), da2.data(), db.data()};
    }
    auto read_round = [&](int round, float* g, float* info) {
        cudamx.read(reinterpret_cast<char*>(g), nthr * cw * sizeof(float));
        if (!cudamx) fail("Cannot read CUDA_MX.bin round {} (intended {}-byte allocation)", round, nthr * cw * sizeof(float));
        infomx.read(reinterpret_cast<char*>(info), nthr * iw * sizeof(float));
        if (!infomx) fail("Cannot read INFO_MX.bin round {} (intended {}-byte allocation)", round, nthr * iw * sizeof(float));
    };
    if (!c.dump_diagnostics) {
        stream_rounds(s.get(), c, read_round, infoout);
        return;
    }
    for (int round = 0; round < c.n_rounds; round++) {
        read_round(round, hc_mx, hinfo);
        evaluate_host(s.get(), c.serial ? round : 0, (int64_t)nthr, hc_mx, hinfo, hinfo,
                      c.dump_diagnostics ? &dg : nullptr);
        if (c.dump_diagnostics) {
            write_bin("YPLANT_OUT.bin", dy.data(), dy.size() * sizeof(float));
            write_bin("LINA_MX_OUT.bin", dl.data(), dl.size() * sizeof(float));
            write_bin("EIGEN_MX_OUT.bin", de.data(), de.size() * sizeof(float));
            write_bin("ATA_MX_OUT.bin", da2.data(), da2.size() * sizeof(float));
            write_bin("ATB_MX_OUT.bin", db.data(), db.size() * sizeof(float));
        }
        infoout.write(reinterpret_cast<char*>(hinfo), nthr * iw * sizeof(float));
    }
}

void destroy_ragged(ce_ragged* r) {
    if (!r) return;
    if (r->d_plants) cudaFree(r->d_plants);
    if (r->d_runs) cudaFree(r->d_runs);
    if (r->d_inst) cudaFree(r->d_inst);
    if (r->d_tab) cudaFree(r->d_tab);
    if (r->h_gains) cudaFreeHost(r->h_gains);
    if (r->h_info) cudaFreeHost(r->h_info);
    for (void* p : {(void*)r->d_g_in, (void*)r->d_i_in, (void*)r->d_i_out, (void*)r->d_goff, (void*)r->d_ioff,
                    (void*)r->d_wid})
        if (p) cudaFree(p);
    destroy_session(r->s);
    delete r;
}

// Instances of any shapes, horizons and sweeps: per-instance plants, margin
// plants, sweep grids and plant scalings (one grid kernel over all instances),
// and per-instance Runs whose strides and slots are the batch's maxima.
void create_ragged(int n_inst, const ce_config* cfgs, const ce_plant* plants, ce_ragged** out) {
    if (!cfgs || !plants || !out) fail("ce_ragged_create: null argument");
    if (n_inst < 1) fail("ce_ragged_create: n_inst must be >= 1, got {}", n_inst);
    std::unique_ptr<ce_ragged, void (*)(ce_ragged*)> r(new ce_ragged, destroy_ragged);
    r->cfg.assign(cfgs, cfgs + n_inst);
    ce_config L = cfgs[0];
    for (int i = 0; i < n_inst; ++i) {
        const ce_config& c = cfgs[i];
        const std::string who = std::format("ce_ragged_create: instance {}", i);
        check_config(c, who.c_str());
        if (c.observer != CE_OBSERVER_LUENBERGER) fail("{}: a ragged batch runs the Luenberger observer", who);
        L.statespace_dim = std::max(L.statespace_dim, c.statespace_dim);
        L.discrete_dim = std::max(L.discrete_dim, c.discrete_dim);
        L.nonlin_dim = std::max(L.nonlin_dim, c.nonlin_dim);
        L.total_dim = std::max(L.total_dim, c.total_dim);
        L.cuda_mx_width = std::max(L.cuda_mx_width, c.cuda_mx_width);
        L.info_mx_width = std::max(L.info_mx_width, c.info_mx_width);
        L.fit_steps = std::max(L.fit_steps, c.fit_steps);
        L.freq = std::max(L.freq, c.freq);
        L.time = std::max(L.time, c.time);
    }
    r->layout = L;
    std::vector<Plant> P(n_inst);
    const int ms = margin_plant_stride();
    std::vector<float> mp((size_t)n_inst * ms, 0.0f), zg;
    std::vector<int> n_of(n_inst), F_of(n_inst), row_inst, row_w;
    std::vector<int64_t> zoff(n_inst), goff(n_inst);
    int64_t gtot = 0;
    r->sig.assign(n_inst, {});
    for (int i = 0; i < n_inst; ++i) {
        const ce_config& c = cfgs[i];
        build_plant(c, plants[i], 0, P[i]);
        auto& g = r->sig[i];
        for (int w = 0; w < MAXW; ++w)
            for (int k = 0; k < P[i].n_nl[w] && k < MAX_NL; ++k) g[w * MAX_NL + k] = (uint8_t)P[i].nl[w][k].op;
        for (int k = 0; k < P[i].n_dc && k < MAX_DC; ++k) g[MAXW * MAX_NL + k] = (uint8_t)P[i].dc[k].op;
        for (int k = 0; k < P[i].n_u && k < MAX_U; ++k) g[MAXW * MAX_NL + MAX_DC + k] = (uint8_t)P[i].u[k].op;
        float* m = mp.data() + (size_t)i * ms;
        std::memcpy(m, P[i].m_a, sizeof(P[i].m_a));
        std::memcpy(m + MAXS * MAXS, P[i].m_b, sizeof(P[i].m_b));
        std::memcpy(m + MAXS * MAXS + MAXS, P[i].m_c, sizeof(P[i].m_c));
        m[MAXS * MAXS + 2 * MAXS] = P[i].m_d;
        n_of[i] = c.serial ? c.discrete_dim : c.statespace_dim;
        F_of[i] = c.freq;
        zoff[i] = (int64_t)zg.size();
        const std::vector<float> z = zgrid32(c);
        zg.insert(zg.end(), z.begin(), z.end());
        goff[i] = gtot;
        gtot += (int64_t)c.freq * 8;
        for (int w = 0; w <= c.freq; ++w) {
            row_inst.push_back(i);
            row_w.push_back(w);
        }
    }
    // the pipeline's session: no plant of its own (every candidate's comes from the tables)
    r->s = new ce_session();
    ce_session* s = r->s;
    s->cfg = L;
    s->n_plants = 1;
    s->plants.assign(1, Plant{});
    s->plant_err.assign(1, std::string());
    s->grid_np = 1;
    s->alpha32.assign(1, 1.0f);
    s->sim_kernel.assign(1, SimKernels{});
    s->sim_kind = CE_SIM_TABLE;
    init_streams(s);
    // sweep grids and plant scalings of all instances
    std::vector<void*> tmp;
    auto up = [&](const auto& v) {
        void* d = nullptr;
        const size_t bytes = v.size() * sizeof(v[0]);
        CE_CUDA(cudaMalloc(&d, bytes ? bytes : 1));
        if (bytes) CE_CUDA(cudaMemcpy(d, v.data(), bytes, cudaMemcpyHostToDevice));
        tmp.push_back(d);
        return d;
    };
    struct Free {
        std::vector<void*>& t;
        ~Free() {
            for (void* p : t) cudaFree(p);
        }
    } freer{tmp};
    float* d_grid = nullptr;
    CE_CUDA(cudaMalloc((void**)&d_grid, (size_t)gtot * sizeof(float)));
    s->d_fgrid32 = d_grid;
    float* d_alpha = (float*)up(std::vector<float>(n_inst, 0.0f));
    int* d_bad = (int*)up(std::vector<int>(n_inst, 0));
    launch_plant_grid_rows((int64_t)row_inst.size(), (const int*)up(row_inst), (const int*)up(row_w),
                           (const int*)up(n_of), (const int*)up(F_of), (const int64_t*)up(zoff),
                           (const int64_t*)up(goff), (const float*)up(mp), (const float*)up(zg), d_grid, d_alpha,
                           d_bad, s->stream);
    std::vector<float> alpha(n_inst);
    std::vector<int> bad(n_inst);
    CE_CUDA(cudaMemcpyAsync(alpha.data(), d_alpha, (size_t)n_inst * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    CE_CUDA(cudaMemcpyAsync(bad.data(), d_bad, (size_t)n_inst * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CE_CUDA(cudaStreamSynchronize(s->stream));
    for (int i = 0; i < n_inst; ++i)
        if (bad[i])
            fail("ce_ragged_create: instance {}: allmargin: plant has no finite nonzero gain at crossover = {} rad/s",
                 i, cfgs[i].crossover);
    std::vector<Run> runs(n_inst);
    for (int i = 0; i < n_inst; ++i) {
        runs[i] = run_from_config(cfgs[i], L, 0, alpha[i], 0.0);
        runs[i].grid_off = goff[i];
    }
    CE_CUDA(cudaMalloc((void**)&r->d_runs, (size_t)n_inst * sizeof(Run)));
    CE_CUDA(cudaMemcpy(r->d_runs, runs.data(), (size_t)n_inst * sizeof(Run), cudaMemcpyHostToDevice));
    CE_CUDA(cudaMalloc((void**)&r->d_plants, (size_t)n_inst * sizeof(Plant)));
    CE_CUDA(cudaMemcpy(r->d_plants, P.data(), (size_t)n_inst * sizeof(Plant), cudaMemcpyHostToDevice));
    *out = r.release();
}

// n_cand[i] candidates of instance i, rows packed instance after instance at
// each instance's own widths (CUDA_MX and INFO_MX rows as its sessions take them).
// Lanes per candidate of a ragged batch's simulation under its tuning.
int ragged_lanes(const ce_ragged* r) {
    return r->tuning.sim_lanes == 1 || r->tuning.sim_lanes == SW_LANES ? r->tuning.sim_lanes
                                                                      : ragged_lanes_per_candidate();
}

// Everything an evaluation of n_cand[i] candidates per instance needs before
// it runs: the device order of the candidates, their simulation table, the
// caller-row maps and the session scratch.  Synchronous; the order is rebuilt
// only when the counts or the order's settings change.
void ragged_prepare(ce_ragged* r, const int64_t* n_cand) {
    if (!r || !n_cand) fail("ce_ragged_prepare: null argument");
    const int I = (int)r->cfg.size();
    int64_t N = 0;
    for (int i = 0; i < I; ++i) {
        if (n_cand[i] < 0) fail("ce_ragged_evaluate: instance {} has a negative candidate count {}", i, n_cand[i]);
        N += n_cand[i];
    }
    if (N > INT32_MAX) fail("ce_ragged_evaluate: {} candidates exceed the 32-bit candidate index", N);
    const std::vector<int64_t> counts(n_cand, n_cand + I);
    const int lanes = ragged_lanes(r), inst_order = r->tuning.instance_order;
    if (r->prepared && counts == r->prep_counts && lanes == r->prep_lanes && inst_order == r->prep_inst_order)
        return;
    r->prepared = false;
    ce_session* s = r->s;
    if (r->tuning.eig_blocks_per_sm >= 0) s->tuning.eig_blocks_per_sm = r->tuning.eig_blocks_per_sm;
    // the caller's row offsets of each instance
    std::vector<int64_t> goff(I), ioff(I);
    int64_t gi = 0, ii = 0;
    for (int i = 0; i < I; ++i) {
        goff[i] = gi;
        ioff[i] = ii;
        gi += n_cand[i] * r->cfg[i].cuda_mx_width;
        ii += n_cand[i] * r->cfg[i].info_mx_width;
    }
    r->h_inst.resize((size_t)N);
    r->dev_k.resize((size_t)N);
    // The device order (instance_order):
    // 0 (default): grouped by program.  Instances are sorted by the dimension
    //   class of their simulation (4 or 8 observer / plant rows), then by the
    //   operation sequence of their programs, then by decreasing horizon, and
    //   each instance's candidates stay together.  A warp's lanes then interpret
    //   the same operations in the same slots (one path per slot instead of one
    //   per program), run the dimension class of their own plants, and have
    //   similar horizons, so few lanes idle after their horizon ends.
    // 1: the caller's order.
    // 2: dealt by horizon.  Candidates sorted by decreasing horizon are dealt to
    //   the W warps of the simulation (32 / lanes candidates each) in turn: warp w
    //   holds sorted candidates w, W + w, 2W + w, ..., one from each horizon tier,
    //   each tier ordered by program.
    auto sim_class = [&](int i) {
        return (r->cfg[i].statespace_dim > 4 ? 2 : 0) + (r->cfg[i].discrete_dim > 4 ? 1 : 0);
    };
    std::vector<int> sorted_inst;
    std::vector<int64_t> sorted_k;
    sorted_inst.reserve((size_t)N);
    sorted_k.reserve((size_t)N);
    {
        std::vector<int> order(I);
        for (int i = 0; i < I; ++i) order[i] = i;
        if (inst_order == 0)
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
                const int ca = sim_class(a), cb = sim_class(b);
                if (ca != cb) return ca < cb;
                if (r->sig[a] != r->sig[b]) return r->sig[a] < r->sig[b];
                return r->cfg[a].time > r->cfg[b].time;
            });
        else if (inst_order == 2)
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return r->cfg[a].time > r->cfg[b].time; });
        for (int i : order)
            for (int64_t k = 0; k < n_cand[i]; ++k) {
                sorted_inst.push_back(i);
                sorted_k.push_back(k);
            }
    }
    if (inst_order != 2) {
        for (int64_t q = 0; q < N; ++q) {
            r->h_inst[(size_t)q] = sorted_inst[(size_t)q];
            r->dev_k[(size_t)q] = sorted_k[(size_t)q];
        }
    } else {
        const int64_t per_warp = 32 / lanes;
        const int64_t W = std::max<int64_t>(1, (N + per_warp - 1) / per_warp);
        // Within each tier of W consecutive candidates, order by the programs'
        // operation sequences, so that the candidates dealt to one warp (the same
        // rank in every tier) tend to interpret the same operations in the same
        // slots and the warp executes fewer distinct paths per slot.
        std::vector<int64_t> idx((size_t)N);
        for (int64_t q = 0; q < N; ++q) idx[(size_t)q] = q;
        for (int64_t t0 = 0; t0 < N; t0 += W) {
            const int64_t t1 = std::min(N, t0 + W);
            std::stable_sort(idx.begin() + t0, idx.begin() + t1, [&](int64_t a, int64_t b) {
                return r->sig[sorted_inst[(size_t)a]] < r->sig[sorted_inst[(size_t)b]];
            });
        }
        int64_t p = 0;
        for (int64_t w = 0; w < W; ++w)
            for (int64_t l = 0; l < per_warp; ++l) {
                const int64_t q = l * W + w;  // (l, w) <-> q is a bijection onto [0, per_warp W)
                if (q >= N) continue;
                r->h_inst[(size_t)p] = sorted_inst[(size_t)idx[(size_t)q]];
                r->dev_k[(size_t)p] = sorted_k[(size_t)idx[(size_t)q]];
                ++p;
            }
    }
    // per device position: the caller's row offsets and the instance's widths
    std::vector<int64_t> hg((size_t)N), hi((size_t)N);
    std::vector<int2> hw((size_t)N);
    for (int64_t c = 0; c < N; ++c) {
        const int i = r->h_inst[(size_t)c];
        const int64_t k = r->dev_k[(size_t)c];
        const int cw = r->cfg[i].cuda_mx_width, iw = r->cfg[i].info_mx_width;
        hg[(size_t)c] = goff[i] + k * cw;
        hi[(size_t)c] = ioff[i] + k * iw;
        hw[(size_t)c] = int2{cw, iw};
    }
    if (N > r->inst_cap) {
        if (r->d_inst) cudaFree(r->d_inst);
        if (r->d_tab) cudaFree(r->d_tab);
        r->d_inst = nullptr;
        r->d_tab = nullptr;
        r->inst_cap = 0;
        CE_CUDA(cudaMalloc((void**)&r->d_inst, (size_t)N * sizeof(int)));
        CE_CUDA(cudaMalloc((void**)&r->d_tab, (size_t)RT_FIELDS * N * sizeof(float)));
        r->inst_cap = N;
    }
    if (N > r->map_cap) {
        for (void* p : {(void*)r->d_goff, (void*)r->d_ioff, (void*)r->d_wid})
            if (p) cudaFree(p);
        r->d_goff = r->d_ioff = nullptr;
        r->d_wid = nullptr;
        r->map_cap = 0;
        CE_CUDA(cudaMalloc((void**)&r->d_goff, (size_t)N * sizeof(int64_t)));
        CE_CUDA(cudaMalloc((void**)&r->d_ioff, (size_t)N * sizeof(int64_t)));
        CE_CUDA(cudaMalloc((void**)&r->d_wid, (size_t)N * sizeof(int2)));
        r->map_cap = N;
    }
    if (N > 0) {
        CE_CUDA(cudaMemcpyAsync(r->d_inst, r->h_inst.data(), (size_t)N * sizeof(int), cudaMemcpyHostToDevice, s->stream));
        CE_CUDA(cudaMemcpyAsync(r->d_goff, hg.data(), (size_t)N * sizeof(int64_t), cudaMemcpyHostToDevice, s->stream));
        CE_CUDA(cudaMemcpyAsync(r->d_ioff, hi.data(), (size_t)N * sizeof(int64_t), cudaMemcpyHostToDevice, s->stream));
        CE_CUDA(cudaMemcpyAsync(r->d_wid, hw.data(), (size_t)N * sizeof(int2), cudaMemcpyHostToDevice, s->stream));
        launch_ragged_table(N, r->d_plants, r->d_inst, r->d_tab, r->inst_cap, s->stream);
        s->launches += 1;
        ensure_buffers(s, N, false);
    }
    CE_CUDA(cudaStreamSynchronize(s->stream));
    r->prep_counts = counts;
    r->prep_lanes = lanes;
    r->prep_inst_order = inst_order;
    r->prep_n = N;
    r->g_total = gi;
    r->i_total = ii;
    r->prepared = true;
}

// One prepared evaluation on device rows packed as the host API packs them:
// gather into the device order, one launch per stage, scatter the INFO rows
// back.  Enqueued on st; no allocation, no synchronisation.
void ragged_enqueue(ce_ragged* r, const float* d_cuda_mx, const float* d_info_in, float* d_info_out,
                    cudaStream_t st) {
    const int64_t N = r->prep_n;
    if (N == 0) return;
    ce_session* s = r->s;
    Buffers& b = s->buf;
    const int LW = r->layout.cuda_mx_width, LI = r->layout.info_mx_width;
    launch_ragged_gather(N, r->d_goff, r->d_ioff, r->d_wid, LW, LI, d_cuda_mx, d_info_in, b.gains, b.info, st);
    const Ragged rg{r->d_runs, r->d_plants, r->d_inst, r->d_tab, r->inst_cap, r->prep_lanes,
                    r->tuning.sim_width == 8 ? 1 : 0};
    run_pipeline(s, 0, N, b.gains, b.info, st, false, false, &rg);
    launch_ragged_scatter(N, r->d_ioff, r->d_wid, LI, b.info, d_info_out, st);
    s->launches += 2;
}

void ragged_evaluate_device(ce_ragged* r, const float* d_cuda_mx, const float* d_info_in, float* d_info_out,
                            void* stream) {
    if (!r) fail("ce_ragged_evaluate_device: null ragged batch");
    if (!r->prepared) fail("ce_ragged_evaluate_device: no prepared candidate counts (call ce_ragged_prepare first)");
    if (r->prep_n > 0 && (!d_cuda_mx || !d_info_in || !d_info_out)) fail("ce_ragged_evaluate_device: null buffer");
    ragged_enqueue(r, d_cuda_mx, d_info_in, d_info_out, (cudaStream_t)stream);
}

void ragged_evaluate(ce_ragged* r, const int64_t* n_cand, const float* cuda_mx, const float* info_in,
                     float* info_out) {
    if (!r || !n_cand) fail("ce_ragged_evaluate: null argument");
    ragged_prepare(r, n_cand);
    if (r->prep_n == 0) return;
    if (!cuda_mx || !info_in || !info_out) fail("ce_ragged_evaluate: null buffer");
    const int64_t G = r->g_total, Iw = r->i_total;
    if (G > r->host_g_cap) {
        if (r->h_gains) cudaFreeHost(r->h_gains);
        r->h_gains = nullptr;
        r->host_g_cap = 0;
        CE_CUDA(cudaMallocHost((void**)&r->h_gains, (size_t)G * sizeof(float)));
        r->host_g_cap = G;
    }
    if (Iw > r->host_i_cap) {
        if (r->h_info) cudaFreeHost(r->h_info);
        r->h_info = nullptr;
        r->host_i_cap = 0;
        CE_CUDA(cudaMallocHost((void**)&r->h_info, (size_t)Iw * sizeof(float)));
        r->host_i_cap = Iw;
    }
    if (G > r->dev_g_cap) {
        if (r->d_g_in) cudaFree(r->d_g_in);
        r->d_g_in = nullptr;
        r->dev_g_cap = 0;
        CE_CUDA(cudaMalloc((void**)&r->d_g_in, (size_t)G * sizeof(float)));
        r->dev_g_cap = G;
    }
    if (Iw > r->dev_i_cap) {
        for (float* p : {r->d_i_in, r->d_i_out})
            if (p) cudaFree(p);
        r->d_i_in = r->d_i_out = nullptr;
        r->dev_i_cap = 0;
        CE_CUDA(cudaMalloc((void**)&r->d_i_in, (size_t)Iw * sizeof(float)));
        CE_CUDA(cudaMalloc((void**)&r->d_i_out, (size_t)Iw * sizeof(float)));
        r->dev_i_cap = Iw;
    }
    ce_session* s = r->s;
    std::memcpy(r->h_gains, cuda_mx, (size_t)G * sizeof(float));
    std::memcpy(r->h_info, info_in, (size_t)Iw * sizeof(float));
    CE_CUDA(cudaMemcpyAsync(r->d_g_in, r->h_gains, (size_t)G * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    CE_CUDA(cudaMemcpyAsync(r->d_i_in, r->h_info, (size_t)Iw * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    ragged_enqueue(r, r->d_g_in, r->d_i_in, r->d_i_out, s->stream);
    CE_CUDA(cudaMemcpyAsync(r->h_info, r->d_i_out, (size_t)Iw * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    CE_CUDA(cudaStreamSynchronize(s->stream));
    collect_stage_times(s);
    std::memcpy(info_out, r->h_info, (size_t)Iw * sizeof(float));
}

// The ragged autotuner: coordinate descent over the simulation form (the wide
// four-lane form or one thread per candidate), the device order (grouped by
// program, the caller's order, or dealt by horizon) and the FP64 eigensolves'
// blocks per SM, each
// setting timed over three evaluations of the prepared batch on the caller's
// rows; the fastest is kept.  Results do not depend on the setting.
void ragged_autotune(ce_ragged* r, const float* d_cuda_mx, const float* d_info_in, float* d_info_out, void* stream,
                     ce_ragged_tuning* best) {
    if (!r) fail("ce_ragged_autotune: null ragged batch");
    if (!r->prepared) fail("ce_ragged_autotune: no prepared candidate counts (call ce_ragged_prepare first)");
    cudaStream_t st = (cudaStream_t)stream;
    const std::vector<int64_t> counts = r->prep_counts;
    cudaEvent_t e0, e1;
    CE_CUDA(cudaEventCreate(&e0));
    CE_CUDA(cudaEventCreate(&e1));
    std::unique_ptr<CUevent_st, cudaError_t (*)(cudaEvent_t)> g0(e0, cudaEventDestroy), g1(e1, cudaEventDestroy);
    auto time_of = [&](const ce_ragged_tuning& t) {
        r->tuning = t;
        ragged_prepare(r, counts.data());
        ragged_enqueue(r, d_cuda_mx, d_info_in, d_info_out, st);  // warm
        CE_CUDA(cudaEventRecord(e0, st));
        for (int k = 0; k < 3; ++k) ragged_enqueue(r, d_cuda_mx, d_info_in, d_info_out, st);
        CE_CUDA(cudaEventRecord(e1, st));
        CE_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        CE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        return (double)ms / 3.0;
    };
    ce_ragged_tuning cur = r->tuning;
    if (cur.sim_lanes != 1 && cur.sim_lanes != SW_LANES) cur.sim_lanes = ragged_lanes_per_candidate();
    if (cur.eig_blocks_per_sm <= 0) cur.eig_blocks_per_sm = 5;
    cur.ms_per_evaluation = time_of(cur);
    auto try_set = [&](ce_ragged_tuning t) {
        t.ms_per_evaluation = time_of(t);
        if (t.ms_per_evaluation < cur.ms_per_evaluation) cur = t;
    };
    {
        ce_ragged_tuning t = cur;
        t.sim_lanes = cur.sim_lanes == 1 ? SW_LANES : 1;
        try_set(t);
    }
    for (int o = 1; o <= 2; ++o) {
        ce_ragged_tuning t = cur;
        t.instance_order = (cur.instance_order + o) % 3;
        try_set(t);
    }
    for (int b : {cur.eig_blocks_per_sm - 1, cur.eig_blocks_per_sm + 1})
        if (b >= 1 && b <= 8) {
            ce_ragged_tuning t = cur;
            t.eig_blocks_per_sm = b;
            try_set(t);
        }
    r->tuning = cur;
    ragged_prepare(r, counts.data());
    if (best) *best = cur;
}

}  // namespace
}  // namespace ce

namespace ce {
// One plant per candidate, candidate c on plant h_idx[c] (host array, pinned
// for an asynchronous copy): the serving front end's batches of Monte Carlo
// requests.  Device rows, the caller's stream.
void session_evaluate_plants_indexed(ce_session* s, const int* h_idx, int64_t n, const float* d_cuda_mx,
                                     const float* d_info_in, float* d_info_out, cudaStream_t st) {
    check_eval(s, 0, n);
    for (int64_t c = 0; c < n; ++c) {
        const int p = h_idx[c];
        if (p < 0 || p >= s->n_plants) fail("plant index {} out of range [0, {})", p, s->n_plants);
        if (!s->plant_err[p].empty()) throw std::runtime_error(s->plant_err[p]);
    }
    if (n == 0) return;
    ensure_buffers(s, n, false);
    CE_CUDA(cudaMemcpyAsync(s->buf.plant_idx, h_idx, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, st));
    if (d_info_out != d_info_in)
        CE_CUDA(cudaMemcpyAsync(d_info_out, d_info_in, (size_t)n * s->cfg.info_mx_width * sizeof(float),
                                cudaMemcpyDeviceToDevice, st));
    run_pipeline(s, 0, n, d_cuda_mx, d_info_out, st, false, true, nullptr, s->buf.plant_idx);
}

// Read-only views of a session for other translation units of the library.
const Plant* session_plant(const ce_session* s, int plant) { return &s->plants[plant]; }
const ce_config* session_config(const ce_session* s) { return &s->cfg; }
int session_plants(const ce_session* s) { return s->n_plants; }
const std::string& session_plant_error(const ce_session* s, int plant) { return s->plant_err[plant]; }
void session_set_small_batch_forms(ce_session* s, bool on) { s->small_forms = on; }

// Everything an evaluation of up to n candidates would otherwise allocate or
// build on first use: the scratch buffers (none for n = 0), the FP64 sweep
// grids of an FP64 session and, with `plants`, the per-candidate plant table
// (and its simulation kernel).  A server prepares its sessions at creation so that no
// batch waits on an allocation.
void session_prepare(ce_session* s, int64_t n, bool plants) {
    if (n > 0) ensure_buffers(s, n, false);
    if (grids64(s->precision) && !s->d_fgrid64) build_grids(s, CE_PRECISION_FP64);
    if (plants) ensure_plant_table(s, sim_precision(s->precision));
    CE_CUDA(cudaDeviceSynchronize());
}
Run session_run(const ce_session* s, int plant, int64_t n) { return make_run(s, plant, n); }
void session_count_launches(ce_session* s, int k) { s->launches += k; }
}  // namespace ce

// ============================================================================
// C ABI
// ============================================================================
using namespace ce;

extern "C" {

CE_EXPORT const char* ce_last_error(void) { return g_last_error.c_str(); }

CE_EXPORT const char* ce_version(void) { return "controllerengine-gb300 0.1 (sm_103a)"; }

CE_EXPORT int ce_parse_config(const char* text, const char* filename, ce_config* out) {
    return guarded([&] {
        if (!text || !out) fail("ce_parse_config: null argument");
        parse_config(text, filename ? filename : "ControllerEngine.config", *out);
    });
}

CE_EXPORT int ce_decode_instructions(const int32_t* info, int32_t dim, int32_t count, const float* base_params,
                                     int32_t n_params, ce_instruction* out) {
    return guarded([&] {
        if (count > 0 && (!info || !out || !base_params)) fail("ce_decode_instructions: null argument");
        decode_instructions(info, dim, count, base_params, n_params, out);
    });
}

CE_EXPORT int ce_session_create(const ce_config* cfg, const ce_plant* plant, int32_t n_plants, ce_session** out) {
    return guarded([&] { create_session(cfg, plant, n_plants, out); });
}

CE_EXPORT void ce_session_destroy(ce_session* s) { destroy_session(s); }

CE_EXPORT int ce_ragged_create(int32_t n_inst, const ce_config* cfgs, const ce_plant* plants, ce_ragged** out) {
    return guarded([&] { create_ragged(n_inst, cfgs, plants, out); });
}

CE_EXPORT int ce_ragged_evaluate(ce_ragged* r, const int64_t* n_cand, const float* cuda_mx, const float* info_in,
                                 float* info_out) {
    return guarded([&] { ragged_evaluate(r, n_cand, cuda_mx, info_in, info_out); });
}

CE_EXPORT void ce_ragged_destroy(ce_ragged* r) { destroy_ragged(r); }

CE_EXPORT int ce_ragged_prepare(ce_ragged* r, const int64_t* n_cand) {
    return guarded([&] { ragged_prepare(r, n_cand); });
}

CE_EXPORT int ce_ragged_evaluate_device(ce_ragged* r, const float* d_cuda_mx, const float* d_info_in,
                                        float* d_info_out, void* stream) {
    return guarded([&] { ragged_evaluate_device(r, d_cuda_mx, d_info_in, d_info_out, stream); });
}

CE_EXPORT int ce_ragged_set_tuning(ce_ragged* r, const ce_ragged_tuning* t) {
    return guarded([&] {
        if (!r || !t) fail("null argument");
        if (t->sim_lanes != 0 && t->sim_lanes != 1 && t->sim_lanes != SW_LANES)
            fail("sim_lanes must be 0, 1 or {}, got {}", SW_LANES, t->sim_lanes);
        if (t->instance_order < 0 || t->instance_order > 2)
            fail("instance_order must be 0, 1 or 2, got {}", t->instance_order);
        if (t->eig_blocks_per_sm < 0 || t->eig_blocks_per_sm > 32)
            fail("eig_blocks_per_sm must be in [0, 32], got {}", t->eig_blocks_per_sm);
        if (t->sim_width != 0 && t->sim_width != 8) fail("sim_width must be 0 or 8, got {}", t->sim_width);
        r->tuning = *t;
        r->tuning.ms_per_evaluation = 0.0;
        r->prepared = false;  // the next evaluation rebuilds the device order
    });
}

CE_EXPORT int ce_ragged_get_tuning(const ce_ragged* r, ce_ragged_tuning* t) {
    return guarded([&] {
        if (!r || !t) fail("null argument");
        *t = r->tuning;
    });
}

CE_EXPORT int ce_ragged_autotune(ce_ragged* r, const float* d_cuda_mx, const float* d_info_in, float* d_info_out,
                                 void* stream, ce_ragged_tuning* best) {
    return guarded([&] { ragged_autotune(r, d_cuda_mx, d_info_in, d_info_out, stream, best); });
}

CE_EXPORT int64_t ce_ragged_kernel_launches(const ce_ragged* r) { return r && r->s ? r->s->launches : -1; }

CE_EXPORT int ce_ragged_set_profiling(ce_ragged* r, int32_t on) {
    return guarded([&] {
        if (!r) fail("null ragged batch");
        if (ce_session_set_profiling(r->s, on)) fail("{}", g_last_error);
    });
}

CE_EXPORT int ce_ragged_stage_times(ce_ragged* r, double* ms, int64_t* launches) {
    return guarded([&] {
        if (!r) fail("null ragged batch");
        if (ce_session_stage_times(r->s, ms, launches)) fail("{}", g_last_error);
    });
}

CE_EXPORT int ce_session_set_eig_arith(ce_session* s, int32_t arith) {
    return guarded([&] {
        if (!s) fail("null session");
        if (arith != CE_EIG_ARITH_SEPARATE && arith != CE_EIG_ARITH_FUSED) fail("unknown eigensolve arithmetic {}", arith);
        s->eig_arith = arith;
    });
}

CE_EXPORT int ce_session_get_eig_arith(const ce_session* s, int32_t* arith) {
    return guarded([&] {
        if (!s || !arith) fail("null argument");
        *arith = s->eig_arith;
    });
}

CE_EXPORT int ce_session_set_precision(ce_session* s, int32_t precision) {
    return guarded([&] {
        if (!s) fail("null session");
        if (precision != CE_PRECISION_MIXED && precision != CE_PRECISION_FP64 && precision != CE_PRECISION_COMPENSATED &&
            precision != CE_PRECISION_COMPENSATED_TRAJ64 && precision != CE_PRECISION_COMPENSATED_DF)
            fail("unknown precision {}", precision);
        if (sim_precision(precision) != CE_PRECISION_MIXED && s->cfg.observer == CE_OBSERVER_KALMAN)
            fail("the Kalman observer (observer = kalman) simulates in FP32 only (mixed or compensated precision)");
        s->precision = precision;
    });
}

CE_EXPORT int ce_session_get_config(const ce_session* s, ce_config* out) {
    return guarded([&] {
        if (!s || !out) fail("null argument");
        *out = s->cfg;
    });
}

CE_EXPORT int ce_evaluate(ce_session* s, int32_t plant_index, int64_t n, const float* cuda_mx, const float* info_in,
                          float* info_out) {
    return guarded([&] { evaluate_host(s, plant_index, n, cuda_mx, info_in, info_out, nullptr); });
}

CE_EXPORT int ce_evaluate_diagnostics(ce_session* s, int32_t plant_index, int64_t n, const float* cuda_mx,
                                      const float* info_in, float* info_out, const ce_diagnostics* diag) {
    return guarded([&] { evaluate_host(s, plant_index, n, cuda_mx, info_in, info_out, diag); });
}

CE_EXPORT int ce_evaluate_diagnostics64(ce_session* s, int32_t plant_index, int64_t n, const float* cuda_mx,
                                        const float* info_in, float* info_out, const ce_diagnostics64* diag) {
    return guarded([&] { evaluate_host64(s, plant_index, n, cuda_mx, info_in, info_out, diag); });
}

CE_EXPORT int ce_evaluate_device(ce_session* s, int32_t plant_index, int64_t n, const float* d_cuda_mx,
                                 const float* d_info_in, float* d_info_out, void* stream) {
    return guarded([&] {
        check_eval(s, plant_index, n);
        if (n == 0) return;
        cudaStream_t st = (cudaStream_t)stream;
        if (d_info_out != d_info_in)
            CE_CUDA(cudaMemcpyAsync(d_info_out, d_info_in, (size_t)n * s->cfg.info_mx_width * sizeof(float),
                                    cudaMemcpyDeviceToDevice, st));
        run_pipeline(s, plant_index, n, d_cuda_mx, d_info_out, st, false);
    });
}

CE_EXPORT int ce_evaluate_plants(ce_session* s, int32_t first_plant, int64_t n, const float* cuda_mx,
                                 const float* info_in, float* info_out) {
    return guarded([&] { evaluate_host(s, first_plant, n, cuda_mx, info_in, info_out, nullptr, true); });
}

CE_EXPORT int ce_evaluate_plants_device(ce_session* s, int32_t first_plant, int64_t n, const float* d_cuda_mx,
                                        const float* d_info_in, float* d_info_out, void* stream) {
    return guarded([&] {
        check_plants(s, first_plant, n);
        if (n == 0) return;
        cudaStream_t st = (cudaStream_t)stream;
        if (d_info_out != d_info_in)
            CE_CUDA(cudaMemcpyAsync(d_info_out, d_info_in, (size_t)n * s->cfg.info_mx_width * sizeof(float),
                                    cudaMemcpyDeviceToDevice, st));
        run_pipeline(s, first_plant, n, d_cuda_mx, d_info_out, st, false, true);
    });
}

CE_EXPORT int64_t ce_session_kernel_launches(const ce_session* s) { return s ? s->launches : 0; }

CE_EXPORT int ce_session_set_tuning(ce_session* s, const ce_tuning* t) {
    return guarded([&] {
        if (!s || !t) fail("null argument");
        if (t->eig_lanes != 0 && t->eig_lanes != 1 && t->eig_lanes != 2 && t->eig_lanes != 4 && t->eig_lanes != 8 &&
            t->eig_lanes != 16)
            fail("eig_lanes must be 0, 1, 2, 4, 8 or 16, got {}", t->eig_lanes);
        if (t->eig_blocks_per_sm < 0 || t->eig_blocks_per_sm > 32)
            fail("eig_blocks_per_sm must be in [0, 32], got {}", t->eig_blocks_per_sm);
        if (t->chunks < 0 || t->chunks > MAX_CHUNKS) fail("chunks must be in [0, {}], got {}", MAX_CHUNKS, t->chunks);
        s->tuning = *t;
    });
}

CE_EXPORT int ce_session_get_tuning(const ce_session* s, ce_tuning* t) {
    return guarded([&] {
        if (!s || !t) fail("null argument");
        *t = s->tuning;
    });
}

// The session autotuner: coordinate descent over the chunk count, the lanes per
// matrix and the blocks per SM of the FP64 eigensolves, each setting timed with
// CUDA events on one evaluation of the caller's batch (device buffers, the
// output rows are overwritten).  None of the settings changes a result.
CE_EXPORT int ce_session_autotune(ce_session* s, int32_t plant_index, int64_t n, const float* d_cuda_mx,
                                  const float* d_info_in, float* d_info_out, void* stream, ce_tuning* best) {
    return guarded([&] {
        check_eval(s, plant_index, n);
        if (n == 0) fail("ce_session_autotune: empty batch");
        cudaStream_t st = (cudaStream_t)stream;
        cudaEvent_t e0, e1;
        CE_CUDA(cudaEventCreate(&e0));
        CE_CUDA(cudaEventCreate(&e1));
        std::unique_ptr<CUevent_st, cudaError_t (*)(cudaEvent_t)> g0(e0, cudaEventDestroy), g1(e1, cudaEventDestroy);
        auto time_it = [&](const ce_tuning& t) {
            s->tuning = t;
            float best_ms = 1e30f;
            for (int rep = 0; rep < 3; ++rep) {  // first one warms the setting up
                CE_CUDA(cudaMemcpyAsync(d_info_out, d_info_in, (size_t)n * s->cfg.info_mx_width * sizeof(float),
                                        cudaMemcpyDeviceToDevice, st));
                CE_CUDA(cudaEventRecord(e0, st));
                run_pipeline(s, plant_index, n, d_cuda_mx, d_info_out, st, false);
                CE_CUDA(cudaEventRecord(e1, st));
                CE_CUDA(cudaEventSynchronize(e1));
                float ms = 0.0f;
                CE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                if (rep > 0) best_ms = std::min(best_ms, ms);
            }
            return best_ms;
        };
        ce_tuning cur{2, 5, 2, 0.0};
        float cur_ms = time_it(cur);
        auto try_set = [&](ce_tuning t) {
            const float ms = time_it(t);
            if (ms < cur_ms) {
                cur = t;
                cur_ms = ms;
            }
        };
        for (int c : {1, 4}) try_set(ce_tuning{cur.eig_lanes, cur.eig_blocks_per_sm, c, 0.0});
        for (int l : {1, 4}) {
            const int b = l == 1 ? 3 : 10;  // a full share of shared memory for that width
            try_set(ce_tuning{l, b, cur.chunks, 0.0});
        }
        const int lanes = cur.eig_lanes;
        const int bmax = lanes == 1 ? 3 : lanes == 2 ? 6 : 12;
        for (int b = std::max(1, cur.eig_blocks_per_sm - 1); b <= std::min(bmax, cur.eig_blocks_per_sm + 1); ++b)
            if (b != cur.eig_blocks_per_sm) try_set(ce_tuning{lanes, b, cur.chunks, 0.0});
        cur.ms_per_evaluation = cur_ms;
        s->tuning = cur;
        if (best) *best = cur;
    });
}

CE_EXPORT int ce_session_set_sim_kernel(ce_session* s, int32_t kind) {
    return guarded([&] {
        if (!s) fail("null session");
        if (kind != CE_SIM_TABLE && kind != CE_SIM_SPECIALISED) fail("unknown simulation kernel kind {}", kind);
        select_sim_kernel(s, kind);
    });
}

CE_EXPORT int32_t ce_session_sim_kernel(const ce_session* s) { return s ? s->sim_kind : -1; }

CE_EXPORT const char* ce_session_sim_log(const ce_session* s) { return s ? s->sim_log.c_str() : ""; }

CE_EXPORT int ce_sim_specialised_source(const ce_session* s, int32_t plant_index, char* buf, int64_t cap,
                                        int64_t* size) {
    return guarded([&] {
        if (!s) fail("null session");
        if (plant_index < 0 || plant_index >= s->n_plants)
            fail("plant index {} out of range [0, {})", plant_index, s->n_plants);
        const std::string src = specialised_source(s->plants[plant_index], s->cfg.statespace_dim <= 4 ? 4 : 8,
                                                   s->cfg.discrete_dim <= 4 ? 4 : 8,
                                                   s->cfg.observer == CE_OBSERVER_KALMAN);
        if (size) *size = (int64_t)src.size() + 1;
        if (buf && cap > 0) {
            const size_t k = std::min<size_t>(src.size(), (size_t)cap - 1);
            std::memcpy(buf, src.data(), k);
            buf[k] = '\0';
        }
    });
}

CE_EXPORT int ce_session_set_profiling(ce_session* s, int32_t on) {
    return guarded([&] {
        if (!s) fail("null session");
        collect_stage_times(s);
        s->profiling = on != 0;
        for (int i = 0; i < CE_NUM_STAGES; ++i) {
            s->stage_ms[i] = 0.0;
            s->stage_n[i] = 0;
        }
    });
}

CE_EXPORT int ce_session_stage_times(ce_session* s, double* ms, int64_t* launches) {
    return guarded([&] {
        if (!s) fail("null session");
        collect_stage_times(s);
        for (int i = 0; i < CE_NUM_STAGES; ++i) {
            if (ms) ms[i] = s->stage_ms[i];
            if (launches) launches[i] = s->stage_n[i];
        }
    });
}

CE_EXPORT int ce_measure_fma_rate(int32_t fp64, double* ops_per_second) {
    return guarded([&] {
        if (!ops_per_second) fail("null argument");
        *ops_per_second = measure_fma_rate(fp64 != 0);
    });
}

CE_EXPORT int RunControllerEngine(void) {
    try {
        run_files();
        return 0;
    } catch (const std::exception& e) {
        std::ofstream elog("error.log", std::ios::app);
        elog << "ControllerEngine error: " << e.what() << std::endl;
        g_last_error = e.what();
        return 1;
    }
}

}  // extern "C"
