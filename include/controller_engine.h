/*
 * controller_engine.h -- C ABI of the GB300 batch controller-tuning engine.
 *
 * Drop-in boundary.  The reference exports exactly one symbol,
 *   int RunControllerEngine(void)             (ref: src/main.cu:592, src/ControllerEngine.h:11)
 * which reads ControllerEngine.config and the *.bin plant/gain files from the
 * current directory and writes INFO_MX_OUT.bin.  This library exports the same
 * symbol with the same file semantics, and adds an in-memory session API on
 * which RunControllerEngine is built.  Every entry point takes plain pointers
 * and sizes; none takes a C++ or torch type.
 *
 * Error convention (ref: src/main.cu:22-33, 592-602): entry points return 0 on
 * success and nonzero on failure; the message of the last failure on the
 * calling thread is returned by ce_last_error().  RunControllerEngine also
 * appends "ControllerEngine error: <message>" to error.log, as the reference does.
 * Candidate-level numeric failures are not errors: they become the unstable /
 * eig-fail penalties in the cost vector, exactly as in the reference.
 */
#ifndef CONTROLLER_ENGINE_H
#define CONTROLLER_ENGINE_H

#ifndef __CUDACC_RTC__
#include <stdint.h>
#endif

#if defined(_WIN32)
#define CE_EXPORT __declspec(dllexport)
#else
#define CE_EXPORT __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Shape envelope, identical to the reference's compile-time limits (ref: src/main.cu:44-52). */
#define CE_MAX_STATESPACE_DIM 8
#define CE_MAX_DISCRETE_DIM 8
#define CE_MAX_NONLIN_DIM 4
#define CE_MAX_TOTAL_DIM 16
#define CE_MAX_NL_DIM 9
#define CE_MAX_DC_INSTRUCTIONS 4
#define CE_MAX_U_INSTRUCTIONS 4
#define CE_MAX_NL_INSTRUCTIONS 8
#define CE_MAX_PARAMS 34

/* Operand kinds of a decoded instruction (ref: src/main.cu:73). */
#define CE_OPERAND_CONST 0
#define CE_OPERAND_STATE 1
#define CE_OPERAND_PREV 2

/* Observer of the simulated loop (ce_config.observer). */
#define CE_OBSERVER_LUENBERGER 0
#define CE_OBSERVER_KALMAN 1

/* Arithmetic of a session. */
#define CE_PRECISION_MIXED 0 /* reference arithmetic: FP32 double-float simulation, FP32 fit and sweep, FP64 eigensolves */
#define CE_PRECISION_FP64 1  /* the plain FP64 form of the same method: every stage in FP64 */
/* FP32 simulation with a compensated steady-state sum; FP64 LIN_A, eigenvalues, nominal check and
 * sweep; the fit's normal matrix in closed form (FP64) and its right-hand side by a double-float
 * projection of the FP32 trajectory; FP64 LDLT solve with one step of iterative refinement */
#define CE_PRECISION_COMPENSATED 2
/* A diagnostic form: the compensated form's fit, solve, eigensolves and sweep on the FP64 form's
 * trajectory.  Against the FP64 form it isolates how much of the compensated form's difference
 * is the FP32 trajectory's own. */
#define CE_PRECISION_COMPENSATED_TRAJ64 3
/* The compensated form with the simulation in double-float arithmetic (pairs of FP32 values, about
 * 48 significant bits, on the FP32 pipe) instead of the FP32 recurrence: the trajectory then agrees
 * with the FP64 form's to ~1e-12 rather than ~1e-7, and the rest is the compensated form's. */
#define CE_PRECISION_COMPENSATED_DF 4

/*
 * Parsed ControllerEngine.config plus the sizes derived from it.
 * Fields and derivations follow EngineConfig (ref: src/config.cu:5-79) and
 * make_engine_params (ref: src/config.cu:93-104).
 */
typedef struct ce_config {
    /* sizing */
    int32_t statespace_dim, discrete_dim, nonlin_dim, n_params, input_size;
    int32_t dc_instructions, u_instructions;
    int32_t nl_instructions[CE_MAX_NONLIN_DIM];
    /* launch */
    int32_t n_cores, n_rounds, serial;
    /* simulation */
    int32_t time;
    float duration;
    double ref_step_time;
    float ref_amplitude;
    /* scoring / fit */
    float fit_start, fit_end, steady_start;
    float bandwidth, damping, overshoot, steady_state_error, crossover_coeff, target_gm, target_pm, target_b;
    float eig_fail_err, unstable_err;
    int32_t freq;
    float freq_min;
    int32_t dump_diagnostics;
    /* extension: upper end of the frequency sweep in rad/s; 0 = Nyquist (the reference's only choice) */
    float freq_max_key;
    /* derived (ref: src/config.cu:40-78, 99-100) */
    int32_t n_threads;
    float freq_max;
    int32_t total_dim, dc_dim, u_dim, nl_dim, nl_instructions_total;
    int32_t cuda_mx_width, info_scoring, info_freqresp, info_allmargin, info_modal, info_mx_width;
    int32_t eigen_mx_width, lina_mx_width, ata_mx_width, atb_mx_width;
    float ts, fit_t0, fit_t1, damping2, damping4, crossover;
    int32_t fit_start_id, steady_start_id;
    int32_t fit_steps;   /* number of fit samples: #{t >= 0 : (float)t < (fit_end-fit_start)*time} (ref: src/modalsetup.cu:75-76) */
    int32_t ref_step_id; /* first t with !(t < ref_step_time*time) (ref: src/main.cu:414) */
    /* extension: observer of the simulated loop (key `observer`, default luenberger).
       CE_OBSERVER_KALMAN runs the time-varying Kalman filter of discrete_solve<Kalman>
       (ref: src/discrete_solves.cu:83-185), which the reference never launches; its rows are
       [K(ns), L(ns), N, R, Q(ns)] (cuda_mx_width = 3ns+2): the simulation uses K, N, R and
       diag(Q); LIN_A, the eigensolve and the margin sweep use the [K, L, N] prefix as for the
       Luenberger loop. */
    int32_t observer;
} ce_config;

/* A decoded instruction (ref: src/main.cu:75-82). */
typedef struct ce_instruction {
    int32_t op;    /* 0 SKIP, 1 ADD, 2 SUB, 3 MUL, 4 DIV, 5 SAT, 6 SGN; other values: no-op that still starts the chain */
    int32_t col;   /* column of the row's last nonzero entry */
    int32_t akind; /* CE_OPERAND_* */
    int32_t bkind;
    float aval;    /* BASE_PARAMS value when akind == CE_OPERAND_CONST */
    float bval;
} ce_instruction;

/*
 * Plant, observer model and instruction tables, in the compact row-major
 * layouts of the reference's .bin files (ref: src/main.cu:341-383, 385-400).
 * For n_plants > 1 (mode = serial: one plant per round; or one plant per
 * candidate), discrete_* and base_params hold n_plants stacked copies, as the
 * stacked .bin files do (ref: src/main.cu:294-302, 343-354).
 */
typedef struct ce_plant {
    const float* statespace_a;   /* ns*ns   STATESPACE_A.bin   */
    const float* statespace_a_i; /* ns*ns   STATESPACE_A_I.bin */
    const float* statespace_b;   /* ns      STATESPACE_B.bin   */
    const float* statespace_c;   /* ns      STATESPACE_C.bin   */
    const float* statespace_d;   /* 1       STATESPACE_D.bin   */
    const float* discrete_a;     /* nd*nd   DISCRETE_A.bin     (x n_plants) */
    const float* discrete_a_i;   /* nd*nd   DISCRETE_A_I.bin   (x n_plants) */
    const float* discrete_bu;    /* nd      DISCRETE_BU.bin    (x n_plants) */
    const float* discrete_bw;    /* nd*nw   DISCRETE_BW.bin    (x n_plants) */
    const float* discrete_c;     /* nd      DISCRETE_C.bin     (x n_plants) */
    const float* base_params;    /* n_params BASE_PARAMS.bin   (x n_plants) */
    const int32_t* dc_info;      /* dc_instructions*nd          DC_INFO.bin */
    const int32_t* u_info;       /* u_instructions*ns           U_INFO.bin  */
    const int32_t* nl_info;      /* sum(nl_instructions)*(nd+1) NL_INFO.bin */
} ce_plant;

/* Optional per-candidate intermediates (the reference's dump_diagnostics set,
 * ref: src/main.cu:483-548).  Each pointer may be NULL.  Host memory. */
typedef struct ce_diagnostics {
    float* yplant; /* n * time          candidate-major trajectory   (YPLANT_OUT.bin)   */
    float* lina;   /* n * nt*nt         linearised closed loop      (LINA_MX_OUT.bin)  */
    float* eigen;  /* n * 2nt           eigenvalues (re,im) as float (EIGEN_MX_OUT.bin) */
    float* ata;    /* n * (2nt)^2       modal normal matrix         (ATA_MX_OUT.bin)   */
    float* atb;    /* n * 2nt           modal right-hand side       (ATB_MX_OUT.bin)   */
} ce_diagnostics;

/* The same intermediates in double, as the session's precision computed them
 * (no counterpart in the reference): the FP64 form's values unrounded, the
 * mixed form's floats widened.  For pinning the FP64 form against an FP64
 * restatement of the method.  Any pointer may be NULL. */
typedef struct ce_diagnostics64 {
    double* ywin;  /* n * fit_steps     the trajectory's fit window, y(fit_start_id + w) */
    double* summ;  /* n * 4             sum of y over [steady_start_id, time), max y, min y, and the
                                        sum's rounding-error compensation (FP32 simulation; 0 in FP64) */
    double* lina;  /* n * nt*nt         linearised closed loop */
    double* eigen; /* n * 2nt           eigenvalues (re, im) */
    double* ata;   /* n * (2nt)^2       modal normal matrix */
    double* atb;   /* n * 2nt           modal right-hand side */
} ce_diagnostics64;

typedef struct ce_session ce_session;

/* The functions are host API; device code compiled at run time (NVRTC) sees
 * only the constants and structures above. */
#ifndef __CUDACC_RTC__

/* Message of the last failed call on this thread ("" if none). */
CE_EXPORT const char* ce_last_error(void);

/* Library version string. */
CE_EXPORT const char* ce_version(void);

/* Parse ControllerEngine.config text with the reference's keys, defaults,
 * validation and error messages, then derive the sizes.
 * Replaces load_config + EngineConfig::derive (ref: src/config.cu:106-244, 40-78).
 * `filename` is only used in error messages. */
CE_EXPORT int ce_parse_config(const char* text, const char* filename, ce_config* out);

/* Decode `count` base-36 instruction rows of width `dim`: the last nonzero
 * entry of a row is the instruction, digits 0 / 35 / 1..34 select state /
 * running value / BASE_PARAMS[d-1].  Replaces decode_instructions
 * (ref: src/main.cu:317-337).  NL chains additionally remap col == discrete_dim
 * to CE_MAX_DISCRETE_DIM (the plant output slot); that remap is done by
 * ce_session_create (ref: src/main.cu:374-378), not here. */
CE_EXPORT int ce_decode_instructions(const int32_t* info, int32_t dim, int32_t count,
                                     const float* base_params, int32_t n_params, ce_instruction* out);

/* Create a session: validates the plant, decodes the instruction tables of
 * every plant, uploads everything to the current CUDA device and computes the
 * plant's frequency response on the sweep grid.  Replaces init64KB /
 * upload_plant and the plant half of allmargin (ref: src/main.cu:341-400,
 * src/allmargin.cu:11-41).  n_plants = 1 for mode = batch, n_rounds for
 * mode = serial. */
CE_EXPORT int ce_session_create(const ce_config* cfg, const ce_plant* plant, int32_t n_plants, ce_session** out);
CE_EXPORT void ce_session_destroy(ce_session* s);
CE_EXPORT int ce_session_set_precision(ce_session* s, int32_t precision);
CE_EXPORT int ce_session_get_config(const ce_session* s, ce_config* out);

/* Evaluate n candidates against plant `plant_index` (the round in mode =
 * serial).  cuda_mx: n rows of cuda_mx_width floats [K(ns), L(ns), N];
 * info_in / info_out: n rows of info_mx_width floats (info_out may alias
 * info_in).  Host memory; synchronous.  One call = one round of
 * orchestrate_sims (ref: src/main.cu:467-559). */
CE_EXPORT int ce_evaluate(ce_session* s, int32_t plant_index, int64_t n,
                          const float* cuda_mx, const float* info_in, float* info_out);

/* As ce_evaluate, and also returns the intermediates requested in `diag`. */
CE_EXPORT int ce_evaluate_diagnostics(ce_session* s, int32_t plant_index, int64_t n,
                                      const float* cuda_mx, const float* info_in, float* info_out,
                                      const ce_diagnostics* diag);

/* As ce_evaluate, and also returns the intermediates requested in `diag` in
 * double (no counterpart in the reference). */
CE_EXPORT int ce_evaluate_diagnostics64(ce_session* s, int32_t plant_index, int64_t n,
                                        const float* cuda_mx, const float* info_in, float* info_out,
                                        const ce_diagnostics64* diag);

/* Device-memory variant: pointers are device pointers, work is enqueued on
 * `stream` (a cudaStream_t; NULL = legacy default stream) and the call returns
 * without synchronising.  The session owns its scratch; calls on one session
 * must not overlap. */
CE_EXPORT int ce_evaluate_device(ce_session* s, int32_t plant_index, int64_t n,
                                 const float* d_cuda_mx, const float* d_info_in, float* d_info_out,
                                 void* stream);

/* One plant per candidate (no counterpart in the reference, whose mode =
 * serial runs one plant per round, ref: src/main.cu:341-383, 467-559):
 * candidate c of the batch uses plant first_plant + c of the session
 * (first_plant + n <= n_plants).  The plants share the instruction structure
 * and the observer model; their discrete matrices and BASE_PARAMS differ.  In
 * mode = serial the margin check and the sweep use each candidate's own plant,
 * as a serial round would.  Rows are bit-identical to evaluating each
 * candidate with ce_evaluate(s, first_plant + c, 1, ...), in either precision
 * (mixed: the specialised simulation kernel, compiled for the plant table on
 * first use; FP64: the plain form reading the table). */
CE_EXPORT int ce_evaluate_plants(ce_session* s, int32_t first_plant, int64_t n, const float* cuda_mx,
                                 const float* info_in, float* info_out);
CE_EXPORT int ce_evaluate_plants_device(ce_session* s, int32_t first_plant, int64_t n, const float* d_cuda_mx,
                                        const float* d_info_in, float* d_info_out, void* stream);

/* Launches of this library's kernels since the session was created. */
CE_EXPORT int64_t ce_session_kernel_launches(const ce_session* s);

/*
 * Ragged batches (no counterpart in the reference, which runs one configuration
 * per call): n_inst instances, each with its own configuration (dimensions,
 * nonlinear terms, instruction programs, horizon, sweep) and plant, evaluated
 * together -- one launch per stage over the candidates of all instances, each
 * candidate with its instance's sizes and plant.  Every instance's rows equal,
 * bit for bit, what a session of its own configuration and plant returns.
 * Mixed precision and the Luenberger observer; plants[i] holds one plant.
 * ce_ragged_evaluate takes n_cand[i] candidates of instance i, the CUDA_MX and
 * INFO_MX rows packed instance after instance at each instance's own widths,
 * and writes the INFO rows the same way (host buffers, synchronous).
 */
typedef struct ce_ragged ce_ragged;
CE_EXPORT int ce_ragged_create(int32_t n_inst, const ce_config* cfgs, const ce_plant* plants, ce_ragged** out);
CE_EXPORT int ce_ragged_evaluate(ce_ragged* r, const int64_t* n_cand, const float* cuda_mx, const float* info_in,
                                 float* info_out);
CE_EXPORT void ce_ragged_destroy(ce_ragged* r);
CE_EXPORT int64_t ce_ragged_kernel_launches(const ce_ragged* r);
/* Stage timing of a ragged batch, as ce_session_set_profiling / ce_session_stage_times. */
CE_EXPORT int ce_ragged_set_profiling(ce_ragged* r, int32_t on);
CE_EXPORT int ce_ragged_stage_times(ce_ragged* r, double* ms, int64_t* launches);

/* Device-buffer form of a ragged evaluation (no counterpart in the reference).
 * ce_ragged_prepare fixes the candidate counts n_cand[i] and sets up, once and
 * synchronously, everything an evaluation of those counts needs: the device
 * order of the candidates, their simulation table, the maps of the caller's
 * rows and the scratch.  ce_ragged_evaluate_device then takes device rows packed
 * as ce_ragged_evaluate's host rows (instance after instance, each at its own
 * widths; d_info_out may alias d_info_in), enqueues on `stream` a gather into
 * the device order, one launch per pipeline stage and a scatter of the INFO rows,
 * and returns without synchronising.  It allocates nothing, so a call can be
 * captured into a CUDA graph (stream capture) and replayed; calls on one
 * ragged batch must not overlap.  ce_ragged_evaluate prepares its counts the
 * same way (keeping the preparation while the counts repeat). */
CE_EXPORT int ce_ragged_prepare(ce_ragged* r, const int64_t* n_cand);
CE_EXPORT int ce_ragged_evaluate_device(ce_ragged* r, const float* d_cuda_mx, const float* d_info_in,
                                        float* d_info_out, void* stream);

/* Launch settings of a ragged batch and its autotuner (no counterpart in the
 * reference).  None of them changes a result.  ce_ragged_autotune times, on the
 * prepared counts and the caller's device rows, by coordinate descent: the
 * simulation form, the device order and the FP64 eigensolves' blocks per SM;
 * it keeps the fastest and returns it (with its time per evaluation). */
typedef struct ce_ragged_tuning {
    int32_t sim_lanes;         /* lanes per candidate of the simulation: 4 (the wide form), 1, or 0: the default */
    int32_t instance_order;    /* device order of the candidates: 0 (default) grouped by dimension class, program
                                  and decreasing horizon; 1: the caller's order; 2: dealt to warps by horizon tier */
    int32_t eig_blocks_per_sm; /* FP64 eigensolves: one-warp blocks per SM (0: the library default) */
    int32_t sim_width;         /* the wide simulation's row count: 0 (default) each warp at the dimension class (4 or
                                  8) of its candidates; 8: every candidate at the padded 8/8 width */
    double ms_per_evaluation;  /* ce_ragged_autotune: the chosen setting's time */
} ce_ragged_tuning;
CE_EXPORT int ce_ragged_set_tuning(ce_ragged* r, const ce_ragged_tuning* t);
CE_EXPORT int ce_ragged_get_tuning(const ce_ragged* r, ce_ragged_tuning* t);
CE_EXPORT int ce_ragged_autotune(ce_ragged* r, const float* d_cuda_mx, const float* d_info_in, float* d_info_out,
                                 void* stream, ce_ragged_tuning* best);

/* Launch tuning of a session (no counterpart in the reference).  0 fields take
 * the library defaults (2 lanes per matrix, 5 blocks per SM, 2 chunks for
 * batches of >= 32,768 candidates).  No setting changes a result.
 * ce_session_autotune times settings on one batch of the caller's (device
 * buffers; d_info_out is overwritten) by coordinate descent over the chunk
 * count, the lanes per matrix and the blocks per SM of the FP64 eigensolves,
 * keeps the fastest and returns it with its time. */
typedef struct ce_tuning {
    int32_t eig_lanes;         /* lanes per matrix of the FP64 eigensolves: 1, 2, 4, 8 or 16 (0: by batch size) */
    int32_t eig_blocks_per_sm; /* their persistent one-warp blocks per SM */
    int32_t chunks;            /* chunks a batch of >= 32,768 candidates is cut into (<= 8) */
    double ms_per_evaluation;  /* ce_session_autotune: the time of the chosen setting */
} ce_tuning;
CE_EXPORT int ce_session_set_tuning(ce_session* s, const ce_tuning* t);
CE_EXPORT int ce_session_get_tuning(const ce_session* s, ce_tuning* t);

/* Arithmetic of the FP64 eigensolves, LIN_A's and the nominal closed loop's
 * (no counterpart in the reference, whose Eigen stage on the host rounds every
 * product and every sum, ref: src/eigensolve.cu:6-16, src/allmargin.cu:66-79).
 * CE_EIG_ARITH_FUSED (the default): each multiply-add of the Householder and
 * Givens updates is one DFMA, half the FP64 instructions of the separate form;
 * CE_EIG_ARITH_SEPARATE: every product and sum rounded on its own, as the
 * reference's host code computes them.  The two forms run the same algorithm
 * in the same order and differ by rounding alone (eigenvalues within ~1e-14
 * relative of each other on the eight-state workload). */
#define CE_EIG_ARITH_SEPARATE 0
#define CE_EIG_ARITH_FUSED 1
CE_EXPORT int ce_session_set_eig_arith(ce_session* s, int32_t arith);
CE_EXPORT int ce_session_get_eig_arith(const ce_session* s, int32_t* arith);
CE_EXPORT int ce_session_autotune(ce_session* s, int32_t plant_index, int64_t n, const float* d_cuda_mx,
                                  const float* d_info_in, float* d_info_out, void* stream, ce_tuning* best);

/* Simulation kernel selection (no counterpart in the reference, whose kernel
 * always interprets the decoded instruction tables).
 * CE_SIM_SPECIALISED: the plant's DC/U/NL programs are compiled at session
 * creation (NVRTC, once per distinct program per process) into straight-line
 * code; results are bit-identical to the table-driven kernel's.
 * CE_SIM_TABLE: the table-driven kernel, which needs no compile step.
 * Sessions start specialised unless the environment sets
 * CE_SIM_KERNEL=table or compiling fails (then ce_session_sim_log holds the
 * reason).  ce_session_set_sim_kernel fails, leaving the selection unchanged,
 * if compiling fails.  FP64 precision always uses its own table-driven kernel. */
#define CE_SIM_TABLE 0
#define CE_SIM_SPECIALISED 1
CE_EXPORT int ce_session_set_sim_kernel(ce_session* s, int32_t kind);
CE_EXPORT int32_t ce_session_sim_kernel(const ce_session* s);
CE_EXPORT const char* ce_session_sim_log(const ce_session* s);
/* The CUDA source generated for one plant's program (NUL-terminated; *size
 * receives the length including the NUL).  Copies at most cap-1 characters. */
CE_EXPORT int ce_sim_specialised_source(const ce_session* s, int32_t plant_index, char* buf, int64_t cap,
                                        int64_t* size);

/* Measurement hooks (no counterpart in the reference).  With profiling on,
 * every stage launch is bracketed by CUDA events on the stream it runs on;
 * ce_session_stage_times waits for them and returns, per stage, the summed
 * milliseconds and the launch count since profiling was switched on.
 * Stages, in order: 0 lina+eigensolve, 1 simulation, 2 modal fit,
 * 3 modal solve, 4 nominal closed loop, 5 margin sweep. */
#define CE_NUM_STAGES 6
CE_EXPORT int ce_session_set_profiling(ce_session* s, int32_t on);
CE_EXPORT int ce_session_stage_times(ce_session* s, double* ms, int64_t* launches);

/* FMA-issue throughput of the current device in operations per second,
 * measured with a register-resident dependent-chain kernel (fp64 = 0: FP32
 * FFMA, 1: FP64 DFMA).  Used as the roofline denominator for the FP32/FP64
 * pipes, which the HBM/tensor peak file does not cover. */
CE_EXPORT int ce_measure_fma_rate(int32_t fp64, double* ops_per_second);

/* Allocation-free variant of the modal-fit path.  No counterpart in the
 * reference.  For callers that must not allocate device memory when they
 * evaluate: a real-time tuning loop that cannot afford cudaMalloc's latency
 * (it may synchronise the device), or a host application whose device memory
 * belongs to its own allocator or is budgeted up front.  It runs the simulation and the modal
 * setup (the same kernels as the session pipeline) for n candidates of plant
 * `plant_index`: d_cuda_mx (n x cuda_mx_width gains) and d_eigen (n x 2nt float
 * eigenvalues, e.g. from a previous evaluation) in; d_ata (n x (2nt)^2), d_atb
 * (n x 2nt) out; d_info (n x info_mx_width) in/out, receiving the steady-state
 * value, the overshoot and the unstable penalty.  Device pointers, enqueued on
 * `stream`, no synchronisation.
 * Its only scratch, the fit window and trajectory summaries, is a static
 * device array of CE_NOALLOC_SCRATCH_FLOATS floats (32 MiB, held by every
 * device that loads the library until exit); a call needs
 * n * (round_up(fit_steps, 8) + 4) floats and is rejected with an error if that
 * is more.  It calls no cudaMalloc/cudaFree.  The first call on a device looks
 * up the array's address once (cudaGetSymbolAddress, with that device
 * current; safe from several host threads): make it before any stream capture.
 * All calls share the array, which keeps the last call's contents (nothing in
 * it must start at zero: the simulation writes every element the fit reads):
 * calls whose work overlaps on the GPU race; serialise them.  A plant whose
 * sweep grid failed at session creation is refused, as in ce_evaluate_device. */
#define CE_NOALLOC_SCRATCH_FLOATS (8 * 1024 * 1024)
CE_EXPORT int ce_modal_fit_noalloc(ce_session* s, int32_t plant_index, int64_t n, const float* d_cuda_mx,
                                   const float* d_eigen, float* d_ata, float* d_atb, float* d_info, void* stream);

/* ---- Serving (no counterpart in the reference, which serves one synchronous
 * file round per call, ref: src/main.cu:467-582) ----------------------------
 * A server holds `lanes` sessions of one configuration and a scheduler thread.
 * Requests of any size queue in arrival order; the scheduler packs the oldest
 * request's plant with the queued requests of the same plant into a batch of
 * up to `capacity` candidates (a larger request is served in pieces) and runs
 * it on a free lane; lanes run concurrently on the GPU.  A request's rows do
 * not depend on the batch they are packed into.  The caller's buffers must
 * stay valid until ce_server_wait reports the request done; every request must
 * be waited for once. */
typedef struct ce_server ce_server;

typedef struct ce_server_options {
    int32_t max_batch;        /* candidates per batch (0: 65,536) */
    int32_t lanes;            /* concurrent batches (0: 2, at most 8) */
    int64_t hbm_budget_bytes; /* device memory for all lanes (0: no limit); capacity shrinks to fit */
    int32_t max_wait_us;      /* a partial batch waits up to this long for more requests (0: none) */
    int32_t precision;        /* CE_PRECISION_MIXED (0, the default), _FP64, _COMPENSATED or _COMPENSATED_DF for every lane */
    int64_t max_batch_work;   /* candidate-steps (candidates x horizon) per batch (0: no cap); a request
                                 above it is served in pieces on several lanes at once */
} ce_server_options;

typedef struct ce_server_stats {
    int64_t capacity;           /* candidates per batch after admission */
    int32_t lanes;
    int64_t completed;          /* requests completed since creation / the last reset */
    int64_t batches;            /* batches dispatched */
    int64_t batched_candidates; /* candidates in those batches */
    int64_t queued;             /* requests waiting for dispatch */
    double latency_p50_ms, latency_p99_ms, latency_max_ms; /* submit -> results in the caller's buffer */
    /* where a request's latency goes: queue = submit -> its first piece dispatched to a lane;
     * service = that dispatch -> done (staging, copies, the evaluation and the GPU it shares) */
    double queue_p50_ms, queue_p99_ms, service_p50_ms, service_p99_ms;
    /* per batch: its work on the lane's stream, H2D start to D2H end (CUDA events) */
    double batch_p50_ms, batch_p99_ms, batch_max_ms;
    /* the requests at or above the p99 latency: their count, mean queue and service time, and the
     * mean number of lanes busy when their first piece was dispatched */
    int64_t tail_requests;
    double tail_queue_ms, tail_service_ms, tail_busy_lanes;
} ce_server_stats;

#define CE_PENDING 2 /* ce_server_wait: the timeout passed first */

CE_EXPORT int ce_server_create(const ce_config* cfg, const ce_plant* plant, int32_t n_plants,
                               const ce_server_options* options, ce_server** out);
/* Several models (configurations with their plants) in one server: every lane
 * holds a session per model; a batch holds requests of one model (on any of
 * its plants: a batch on several plants evaluates each row on its own plant). */
CE_EXPORT int ce_server_create_models(const ce_config* cfgs, const ce_plant* plants, const int32_t* n_plants,
                                      int32_t n_models, const ce_server_options* options, ce_server** out);
CE_EXPORT void ce_server_destroy(ce_server* s); /* serves what is queued, then stops */
CE_EXPORT int ce_server_submit(ce_server* s, int32_t plant_index, int64_t n, const float* cuda_mx,
                               const float* info_in, float* info_out, int64_t* request_id);
CE_EXPORT int ce_server_submit_model(ce_server* s, int32_t model, int32_t plant_index, int64_t n,
                                     const float* cuda_mx, const float* info_in, float* info_out, int64_t* request_id);
/* A Monte Carlo request: row k is evaluated on plant first_plant + k of the model (as
 * ce_evaluate_plants, in the server's precision).  Such requests batch with the model's
 * other Monte Carlo requests whatever their plants. */
CE_EXPORT int ce_server_submit_plants(ce_server* s, int32_t model, int32_t first_plant, int64_t n,
                                      const float* cuda_mx, const float* info_in, float* info_out,
                                      int64_t* request_id);
/* 0: done (info_out filled); CE_PENDING: timeout (timeout_ms < 0 waits forever); 1: error. */
CE_EXPORT int ce_server_wait(ce_server* s, int64_t request_id, int32_t timeout_ms);
CE_EXPORT int ce_server_get_stats(ce_server* s, ce_server_stats* out);
CE_EXPORT int ce_server_reset_stats(ce_server* s);

/* The drop-in entry point (ref: src/main.cu:592-602, src/ControllerEngine.h:11):
 * reads ControllerEngine.config and the .bin files from the current
 * directory, streams n_rounds rounds of n_threads candidates, writes
 * INFO_MX_OUT.bin and params.log (and the *_OUT.bin diagnostics when
 * dump_diagnostics is set).  Returns 0, or 1 after appending the message to
 * error.log. */
CE_EXPORT int RunControllerEngine(void);

#endif /* __CUDACC_RTC__ */

#ifdef __cplusplus
}
#endif

#endif /* CONTROLLER_ENGINE_H */
