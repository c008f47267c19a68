// ce_internal.h -- layouts shared by the host orchestrator and the kernels.
//
// The plant, observer model and decoded instruction tables of one plant are
// passed to every kernel BY VALUE as a __grid_constant__ parameter, so they sit
// in the launch's constant bank: warp-uniform operands that FFMA reads straight
// from the constant cache, and a per-launch copy, so sessions with different
// plants can run concurrently on different streams (the reference keeps one
// global __constant__ copy, ref: src/main.cu:56-87, which makes it non-reentrant).
#pragma once

#ifdef __CUDACC_RTC__
typedef int int32_t;
typedef long long int64_t;
#else
#include <stdint.h>
#include <cuda_runtime.h>
#endif
#include "../../include/controller_engine.h"

namespace ce {

constexpr int SIM_BLOCK = 64;   // threads per simulation block (one candidate per thread)
// the wide simulation forms: lanes per candidate and candidates per block
constexpr int SW_LANES = 4, SW_CPB = SIM_BLOCK / SW_LANES;
constexpr int MAX_CHUNKS = 8;  // largest number of chunks one evaluation is cut into
constexpr int SWEEP_FG = 16;   // frequencies per thread in the LU pass of the margin sweep

constexpr int MAXS = CE_MAX_STATESPACE_DIM;   // 8
constexpr int MAXD = CE_MAX_DISCRETE_DIM;     // 8
constexpr int MAXW = CE_MAX_NONLIN_DIM;       // 4
constexpr int MAXT = CE_MAX_TOTAL_DIM;        // 16
constexpr int MAXNC = 2 * CE_MAX_TOTAL_DIM;   // 32: modal basis columns
constexpr int MAX_DC = CE_MAX_DC_INSTRUCTIONS;
constexpr int MAX_U = CE_MAX_U_INSTRUCTIONS;
constexpr int MAX_NL = CE_MAX_NL_INSTRUCTIONS;

// One decoded, SKIP-free instruction.  Removing the SKIP rows of a chain
// changes nothing: the reference interpreter passes over them without touching
// `started` or `result` (ref: src/main.cu:266-268).
struct Instr {
    int op, col, akind, bkind;
    float aval, bval;
};

// Plant + observer model of one round, zero-padded to the MAX dims with row
// stride 8 (the reference's padded __constant__ layout, ref: src/main.cu:304-315).
struct Plant {
    float ss_a[MAXS * MAXS], ss_ai[MAXS * MAXS], ss_b[MAXS], ss_c[MAXS], ss_d;
    float d_a[MAXD * MAXD], d_ai[MAXD * MAXD], d_bu[MAXD], d_bw[MAXD * MAXW], d_c[MAXD];
    // margin plant: observer model in batch mode, true linear plant in serial
    // mode (ref: src/allmargin.cu:11-15); compact ns x ns (row stride MAXS).
    float m_a[MAXS * MAXS], m_b[MAXS], m_c[MAXS], m_d;
    int n_dc, n_u, n_nl[MAXW];
    Instr dc[MAX_DC];
    Instr u[MAX_U];
    Instr nl[MAXW][MAX_NL];  // NL columns: 0..nd-1 plant states, MAXD = plant output y
};

// One plant per candidate (Monte Carlo over plants, or the serial mode's
// per-round plants evaluated in one launch).  The plants' values live on the
// device as a structure of arrays -- field f of plant p at tab[f * np + p] --
// so consecutive candidates read consecutive words; the instruction structure
// (ops, columns, operand kinds) and the observer model are the launch Plant's,
// shared by all plants.  Candidate c of an evaluation uses plant first + c.
constexpr int MC_AI = 0;                      // d_a - I, row stride MAXD
constexpr int MC_A = MC_AI + MAXD * MAXD;     // d_a
constexpr int MC_BU = MC_A + MAXD * MAXD;     // d_bu
constexpr int MC_BW = MC_BU + MAXD;           // d_bw, row stride MAXW
constexpr int MC_C = MC_BW + MAXD * MAXW;     // d_c
constexpr int MC_CST = MC_C + MAXD;           // instruction constants, (a, b) per slot
constexpr int MC_SLOTS = MAX_DC + MAX_U + MAXW * MAX_NL;  // DC k: k; U k: MAX_DC + k; NL w, k: MAX_DC + MAX_U + w MAX_NL + k
constexpr int MC_FIELDS = MC_CST + 2 * MC_SLOTS;

struct McPlants {
    const float* tab;    // null: every candidate uses the launch's Plant
    int64_t np;          // plants in the table (the field stride)
    int64_t first;       // plant of candidate 0
    int64_t grid_stride; // elements between consecutive plants' sweep grids (0: one grid for all)
    const void* alpha;   // per sweep grid: the plant scaling (float or double as the precision)
    int margin;          // 1: the margin plant is the candidate's plant (serial mode), 0: the Plant's
    const int* idx;      // non-null: candidate c uses plant idx[c] (first is then 0)
};

struct Run;

// A ragged batch: instances of different configurations and plants evaluated
// together.  Candidate c belongs to instance inst[c]; that instance's sizes and
// scalars are runs[inst[c]] (whose row strides and slot sizes are the batch's
// common maxima) and its plant plants[inst[c]].
struct Ragged {
    const Run* runs;      // null: a uniform evaluation (the launch's Run and Plant for every candidate)
    const Plant* plants;
    const int* inst;
    // the simulation's plant values per candidate, field-major: field f of
    // candidate c at tab[f * tab_stride + c] (consecutive candidates read
    // consecutive words whatever their instances)
    const float* tab;
    int64_t tab_stride;
    int lanes;  // lanes per candidate of the simulation: SW_LANES (the wide form) or 1
    int full_width;  // 1: the wide form runs every warp at the padded 8/8 width
};

// Fields of that table: observer model, plant, instruction counts and slots.
constexpr int RT_SAI = 0;                       // ss_a - I, row stride MAXS
constexpr int RT_SB = RT_SAI + MAXS * MAXS;     // ss_b
constexpr int RT_SC = RT_SB + MAXS;             // ss_c
constexpr int RT_SD = RT_SC + MAXS;             // ss_d
constexpr int RT_DAI = RT_SD + 1;               // d_a - I, row stride MAXD
constexpr int RT_DBU = RT_DAI + MAXD * MAXD;    // d_bu
constexpr int RT_DBW = RT_DBU + MAXD;           // d_bw, row stride MAXW
constexpr int RT_CNT = RT_DBW + MAXD * MAXW;    // counts: n_dc | n_u << 8 | n_nl[0] << 16 | n_nl[1] << 24, then n_nl[2] | n_nl[3] << 8
constexpr int RT_INS = RT_CNT + 2;              // per slot: code (op | col << 8 | akind << 16 | bkind << 24), aval, bval
constexpr int RT_SLOTS = MAX_DC + MAX_U + MAXW * MAX_NL;  // DC k: k; U k: MAX_DC + k; NL w, k: MAX_DC + MAX_U + w MAX_NL + k
constexpr int RT_FIELDS = RT_INS + 3 * RT_SLOTS;

// Sizes and scalars of one evaluation (the slice of the config the kernels read,
// cf. EngineParams, ref: src/config.cu:84-104).
struct Run {
    int64_t n;  // candidates
    int ns, nd, nt, nw;
    int time, fit_start_id, fit_steps, fit_pitch, steady_start_id, ref_step_id;
    int cuda_w, info_w, info_scoring, info_freqresp, info_allmargin, info_modal;
    int freq;
    float ts, ref_amp, fit_t0, fit_t1, unstable_err, eig_fail_err;
    float bandwidth, damping, overshoot, sse, target_gm, target_pm, target_b, alpha;
    double alpha64;  // alpha of the FP64 form
    int store_traj;  // also write the full trajectory (diagnostics)
    int kalman;      // 1: time-varying Kalman observer (rows [K, L, N, R, Q]), 0: Luenberger
    // Kalman candidate lists (kal_list 0: thread i simulates candidate i).  1: the
    // shared-noise list kal_order[0, kal_totals[0]) in whole warps (-1: padding);
    // 2: the per-candidate list kal_order[kal_totals[0], + kal_totals[1]), then
    // the kal_totals[2] candidates deferred by the shared form at kal_order[kal_defer];
    // 3: the positions of list 2 whose gain schedule turned periodic,
    // kal_lists[0, kal_totals[3]); 4: the others, kal_lists[n, + kal_totals[4])
    int kal_list;
    int* kal_order;
    int* kal_totals;
    int64_t kal_defer;
    const float* kal_sched;  // the gain schedules ([step][gain][position], stride kal_sched_n)
    const int2* kal_meta;    // per position: (t0, p), the gains repeat with period p from step t0
    const int* kal_lists;
    int64_t kal_sched_n;     // positions per schedule row (the buffers' capacity)
    McPlants mc;     // per-candidate plants (mc.tab == null: the Plant for all)
    int eig_lanes;   // FP64 eigensolves: lanes per matrix (1, 2, 4, 8 or 16; 0: by batch size)
    int eig_blocks;  // FP64 eigensolves: one-warp blocks per SM (0: the default)
    int eig_fused;   // FP64 eigensolves: 1 fuses each multiply-add into one DFMA, 0 rounds both
    // floats (or reals) per candidate in the LIN_A, eigenvalue, AtA and Atb buffers:
    // nt^2, 2nt, (2nt)^2, 2nt for a uniform evaluation, the maxima for a ragged one
    int lina_slot, eig_slot, ata_slot, atb_slot;
    int64_t grid_off;  // elements from the sweep grid argument to this run's grid
    Ragged rg;
};

// Per-candidate simulation summary (the parts of the trajectory that modalsetup
// reads besides the fit window).
struct SimSummary {
    float ysum;   // plain float sum of y over [steady_start_id, time), in t order
    float ymax;   // NaN-ignoring max of y over [0, time)
    float ymin;   // NaN-ignoring min of y over [0, time)
    float ycomp;  // the rounding errors of that sum (TwoSum): ysum + ycomp is the compensated sum
};

}  // namespace ce
