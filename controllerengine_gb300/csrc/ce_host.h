// ce_host.h -- host-side declarations of the engine library (C++20).
#pragma once

#include <format>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/controller_engine.h"
#include "ce_internal.h"

namespace ce {

extern thread_local std::string g_last_error;

// Every failure is an exception carrying the message; the C ABI catches it,
// stores it for ce_last_error() and returns nonzero (ref: src/main.cu:22-33).
template <typename... Args>
[[noreturn]] void fail(std::format_string<Args...> fmt, Args&&... args) {
    throw std::runtime_error(std::format(fmt, std::forward<Args>(args)...));
}

#define CE_CUDA(x)                                                                                  \
    do {                                                                                            \
        cudaError_t err_ = (x);                                                                     \
        if (err_ != cudaSuccess) ::ce::fail("CUDA error {} at {}:{}", cudaGetErrorString(err_), __FILE__, __LINE__); \
    } while (0)

// Every kernel of the pipeline asks for the largest shared-memory carveout.
// An SM holds blocks of several kernels at once only under one L1/shared
// split; with the default (per-kernel) preference the small-footprint FP32
// kernels get SMs configured for little shared memory, on which the FP64
// eigensolves' blocks (35 KB each) cannot be placed, and the two streams
// serialise instead of sharing the SMs.
inline void prefer_shared(const void* fn) {
    CE_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared));
}

void derive(ce_config& c);
void parse_config(const std::string& text, const std::string& filename, ce_config& out);
void decode_instructions(const int32_t* info, int dim, int count, const float* base_params, int n_params,
                         ce_instruction* out);

// Response of `np` margin plants (margin_plant_stride() floats each: m_a,
// m_b, m_c, m_d) on the z grid zg ((F + 1) x 4: z, arg z; row F the crossover)
// -> grid (np x F x 8 rows), alpha = 1/|P(crossover)| and bad (no finite
// nonzero gain there), all in the session precision.
void launch_plant_grid(int precision, int np, int n, int F, const float* mp, const void* zg, void* grid, void* alpha,
                       int* bad, cudaStream_t st);
int margin_plant_stride();
// The same for a ragged batch in mixed precision: grid row t is row row_w[t] of
// instance row_inst[t] (n_of: its margin-plant dimension, F_of: its frequency
// count; zoff / goff: element offsets of its z grid and its sweep grid).
void launch_plant_grid_rows(int64_t rows, const int* row_inst, const int* row_w, const int* n_of, const int* F_of,
                            const int64_t* zoff, const int64_t* goff, const float* mp, const float* zg, float* grid,
                            float* alpha, int* bad, cudaStream_t st);

// Kernel launchers (ce_k_*.cu); all enqueue on `st`.
void launch_sim(const Run& run, const Plant& P, int precision, const float* gains, void* ywin, void* summ, float* traj,
                cudaStream_t st);
// LIN_A (float; double in the FP64 form) and its FP64 eigenvalues; candidates that pass the modal stability
// test are appended to list, the others get nominal = -1.  count holds three
// ints (reset here): the listed count and the work counters of both kernels.
// list null: no list of stable candidates (the nominal eigensolve then runs on all);
// clear: zero the work counters first (else the caller has).
void launch_lina_eig(const Run& run, const Plant& P, int precision, const float* gains, void* lina, void* eig,
                     int* nominal, int* list, int* count, cudaStream_t st, bool clear = true);
// Nominal closed-loop stability (nominal = 1 / 0) of the listed candidates.
void launch_nominal(const Run& run, const Plant& P, int precision, const float* gains, const void* lina,
                    const int* list, const int* count, int* nominal, cudaStream_t st);
// counts (MAXT + 1 ints) and order ((MAXT + 1) * n ints) bucket the candidates
// by fit class before the fit; both null: candidates in index order.
void launch_fit(const Run& run, int precision, const void* eig, const void* ywin, const void* summ, void* ata,
                void* atb, float* info, int* counts, int* order, cudaStream_t st);
void launch_modal(const Run& run, int precision, const void* eig, const void* ata, const void* atb, float* info,
                  cudaStream_t st);
// The modal setup of the compensated precision: eig, ata, atb double; ywin float and summ SimSummary
// (traj64: ywin double and summ 4 doubles per candidate, the FP64 simulation's).
void launch_fit_comp(const Run& run, bool traj64, const void* eig, const void* ywin, const void* summ, void* ata,
                     void* atb, float* info, int* counts, int* order, cudaStream_t st);
// Scratch of the margin sweep for up to `cap` listed candidates: |PG| and
// arg(PG) per frequency (freq x cap values each, float or double as the
// precision), and per frequency group the b(w) minimum and the first failure.
struct SweepScratch {
    void* mag;
    void* arg;
    void* bpc;
    int* fail;
};
// The margin sweep; list (n ints) and count (1 int) are scratch for the
// candidates that run the frequency loop.
void launch_sweep(const Run& run, int precision, const float* gains, const void* lina, const int* nominal,
                  const void* fgrid, float* info, int* list, int* count, const SweepScratch& sw, cudaStream_t st);

double measure_fma_rate(bool fp64);

// Simulation kernels specialised to a plant's instruction program
// (ce_jit.cpp), cached per program: `main` (the Luenberger loop, or the Kalman
// loop with per-candidate covariance) and, for the Kalman observer, `shared`
// (the shared-noise form).  main == nullptr: failed, with `log` set.
struct SimKernels {
    const void* main = nullptr;
    const void* shared = nullptr;
    const void* sched = nullptr;  // Kalman: the gains from the candidate's schedule
    const void* quad = nullptr;   // Kalman: the covariance split over four lanes
    const void* wide = nullptr;  // four lanes per candidate (Luenberger, one plant)
    explicit operator bool() const { return main != nullptr; }
};
SimKernels specialise_sim(const Plant& P, int ns, int nd, std::string& log, bool mc = false, bool kalman = false);
std::string specialised_source(const Plant& P, int ns, int nd, bool kalman = false);
// Launches kernel (main or shared; with `wide`, the wide form) over the candidates `run` selects.
void launch_sim_specialised(const void* kernel, const Run& run, const Plant& P, const float* gains, float* ywin,
                            SimSummary* summ, float* traj, cudaStream_t st, bool wide = false);
// Whether an evaluation of n candidates of dimension classes (nsc, ndc) runs the
// wide simulation form: not for the 4/4 class, and only when the one-thread grid
// would occupy fewer than half the SMs (CE_SIM_WIDE=0 never, =1 always).
bool use_wide_sim(int64_t n, int nsc, int ndc);
// Whether a single-chunk evaluation of n candidates runs the nominal eigensolve on all
// candidates beside LIN_A's (small batches; CE_NOMINAL_ALL=0 never).
bool concurrent_nominal(int64_t n);

// Blocks of SIM_BLOCK threads that cover the candidates (or list slots) of `run`.
int sim_grid(const Run& run);
// A ragged batch's rows between the caller's packing and the device order (see ce_k_sim.cu).
void launch_ragged_gather(int64_t n, const int64_t* goff, const int64_t* ioff, const int2* wid, int LW, int LI,
                          const float* g_in, const float* i_in, float* g_dev, float* i_dev, cudaStream_t st);
void launch_ragged_scatter(int64_t n, const int64_t* ioff, const int2* wid, int LI, const float* i_dev, float* i_out,
                           cudaStream_t st);
// The per-candidate table of a ragged batch (RT_FIELDS x stride floats) for n candidates.
void launch_ragged_table(int64_t n, const Plant* plants, const int* inst, float* tab, int64_t stride,
                         cudaStream_t st);

// Grouping of a Kalman evaluation's candidates by their noise weights (R and
// the diagonal of Q, bit for bit) for the shared-noise simulation form
// (ce_k_kalman.cu).  Groups of at least KAL_MIN_GROUP candidates fill whole
// warps of the shared list (padded with -1); the others form the per-candidate
// list.
constexpr int KAL_BUCKETS = 1 << 16;
constexpr int KAL_MIN_GROUP = 8;
inline int64_t kal_shared_slots(int64_t n) { return n + 31 * (n / KAL_MIN_GROUP) + 32; }
inline int64_t kal_order_size(int64_t n) { return kal_shared_slots(n) + 2 * n; }
struct KalGroups {
    unsigned* bucket = nullptr;  // n: hash bucket of each candidate
    int* cnt = nullptr;          // KAL_BUCKETS: candidates per bucket
    int* fill = nullptr;         // KAL_BUCKETS: scatter counters
    int* hoff = nullptr;         // KAL_BUCKETS: offset in the shared list
    int* poff = nullptr;         // KAL_BUCKETS: offset in the per-candidate list
    int* totals = nullptr;       // KAL_TOTALS: shared slots, per-candidate count, deferred count,
                                 // scheduled count, straggler count
    int* order = nullptr;        // kal_order_size(n)
    // the per-candidate list's gain schedules (k_kal_schedule): the gains of the
    // first KAL_SCHED_STEPS steps, [step][gain][list position]; per position
    // (t0, p) -- the gains repeat with period p from step t0, or t0 = -1; and the
    // positions whose schedule is periodic, then those whose is not
    float* sched = nullptr;      // KAL_SCHED_STEPS * MAXS * n
    int2* meta = nullptr;        // n
    int* lists = nullptr;        // 2n: scheduled positions at [0, n), stragglers at [n, 2n)
};
constexpr int KAL_TOTALS = 8;
// Steps of covariance recursion a candidate of the per-candidate list gets to
// turn periodic (bit for bit); 87% of the distinct-noise eight-state batch do
// within 2,048 steps (79% within 1,024), the rest run the recursion in full.
constexpr int KAL_SCHED_STEPS = 2048;
// Fills g.order / g.totals for the n candidates of `run` (4 launches incl. a memset).
void launch_kalman_groups(const Run& run, const float* gains, const KalGroups& g, cudaStream_t st);
// The gain schedules of the per-candidate list (`run` with kal_list = 2; one launch): each
// position's recursion for up to min(time, KAL_SCHED_STEPS) steps, stopping once periodic; the
// periodic positions go to g.lists[0, ...) (count totals[3]), the others to g.lists[n, ...)
// (count totals[4]).
void launch_kalman_schedule(const Run& run, const Plant& P, const float* gains, const KalGroups& g,
                            cudaStream_t st);

const Plant* session_plant(const ce_session* s, int plant);
const ce_config* session_config(const ce_session* s);
int session_plants(const ce_session* s);
// Empty, or why plant `plant` cannot be evaluated (its sweep grid failed at creation).
const std::string& session_plant_error(const ce_session* s, int plant);
// Allocate and build, now, what an evaluation of up to n candidates (n = 0: no scratch; with
// `plants`: on per-candidate plants) would otherwise set up on first use.
void session_prepare(ce_session* s, int64_t n, bool plants);
// The latency forms of small batches (on by default): the wide simulation, more lanes per
// matrix in the FP64 eigensolves, the nominal eigensolve beside LIN_A's.  They shorten an
// evaluation on an idle GPU and cost throughput when batches share it, so a server turns them off.
void session_set_small_batch_forms(ce_session* s, bool on);
// Lanes per candidate of a ragged batch's simulation (4: the wide form; 1: one thread each).
int ragged_lanes_per_candidate();
Run session_run(const ce_session* s, int plant, int64_t n);
void session_count_launches(ce_session* s, int k);
void session_evaluate_plants_indexed(ce_session* s, const int* h_idx, int64_t n, const float* d_cuda_mx,
                                     const float* d_info_in, float* d_info_out, cudaStream_t st);

}  // namespace ce
