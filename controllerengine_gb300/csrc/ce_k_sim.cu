// ce_k_sim.cu -- closed-loop simulation of every candidate (the hot loop).
//
// k_sim_mixed: the step loop of ce_sim_body.cuh with the instruction tables
// interpreted (TableChains); it runs any program with no compile step.  A
// session whose plant program has been compiled into straight-line code
// (ce_jit.cpp) launches that kernel instead.  k_sim_ext is the recurrence in
// FP64 (the plain FP64 form) or in double-float arithmetic (the compensated_df
// form).
#include <cstdlib>

#include "ce_sim_body.cuh"
#include "ce_host.h"

namespace ce {

template <int NSC, int NDC, int KMODE, bool RG = false>
__global__ void __launch_bounds__(SIM_BLOCK) k_sim_mixed(const Run run, const __grid_constant__ Plant P,
                                                         const float* __restrict__ gains, float* __restrict__ ywin,
                                                         SimSummary* __restrict__ summ, float* __restrict__ traj) {
    sim_run<NSC, NDC, TableChains, KMODE, RG>(run, P, gains, ywin, summ, traj);
}

// A ragged batch: every candidate with its instance's sizes, its plant and
// instruction program from the per-candidate table, at the reference's padded width.
__global__ void __launch_bounds__(SIM_BLOCK) k_sim_ragged(const Run run, const __grid_constant__ Plant P,
                                                          const float* __restrict__ gains, float* __restrict__ ywin,
                                                          SimSummary* __restrict__ summ, float* __restrict__ traj) {
    sim_run<MAXS, MAXD, RagChains, SIM_LUENBERGER, true>(run, P, gains, ywin, summ, traj);
}

// The wide form of a ragged batch.  One thread per candidate runs the whole
// horizon as one chain of dependent steps, reloading the plant from shared
// memory every step; at the sizes of an uneven batch too few warps are resident
// to hide that latency, and the longest horizons set the launch's length.
// Here four lanes (a quad) share a candidate, eight candidates per warp.
// Lane q owns rows 2q and 2q+1 of the observer and plant updates, with their
// matrix rows in registers, and NL chain q.  Every lane of the quad forms the
// step's scalars itself -- y (the DC chain), K.xh, u (the U chain), C.xh --
// from the same state and in the same order.  Each value is therefore formed by
// one lane with the operations and order of the one-thread form, so the
// results are bit-identical to it.  The quad exchanges y, W and its new state
// rows through the candidate's slot in shared memory: three quad barriers per
// step.  A warp whose candidates all have ns <= 4 (nd <= 4) runs the 4-row
// observer (plant) step, one row per lane, with the padding beyond 4 virtual.
// words between consecutive fields of the block's table columns: with 17 the
// four lanes of a quad, reading fields of their NL chains 24 fields apart, and
// the warp's eight candidates, reading one field, fall on 32 different banks
constexpr int WIDE_TS = SW_CPB + 1;  // SW_LANES lanes per candidate, SW_CPB candidates per block
// slot layout: the plant-side chains read xp_hi as columns 0..MAXD-1 (their
// column MAXD, y, comes from a register; word WS_XP_HI + MAXD is a zero pad);
// rows are 16-byte aligned, and a stride of 52 words puts the 16-byte loads of
// a warp's eight candidates on disjoint banks
constexpr int WS_XH_HI = 0, WS_XH_LO = 8, WS_XP_HI = 16, WS_XP_LO = 28, WS_W = 36, WS_STRIDE = 52;
static_assert(MAXS == 8 && MAXD == 8 && MAXW == SW_LANES, "the quad splits 8 rows and 4 NL chains");

// The quad's row arithmetic at dimension class NC (4 or 8 rows): lane q owns
// NC / 4 rows.  Loops run to the class, with the padding beyond it virtual as
// in sim_run: `pad` stands for the reference's zero-coefficient terms over the
// padded states (+0, or NaN once a padded state has turned NaN), so every
// class gives the padded 8/8 result bit for bit.
// K.x over the double-float state (hi terms, then lo terms)
template <int NC>
__device__ __forceinline__ float rw_dot(const float* k, const float* hi, const float* lo, float pad) {
    float a = 0.0f;
#pragma unroll
    for (int i = 0; i < NC; ++i) a = __fmaf_rn(k[i], hi[i], a);
    if (NC < MAXS) a = __fadd_rn(a, pad);
#pragma unroll
    for (int i = 0; i < NC; ++i) a = __fmaf_rn(k[i], lo[i], a);
    if (NC < MAXS) a = __fadd_rn(a, pad);
    return a;
}
// K.x and C.x together: two independent chains, each in its own order
template <int NC>
__device__ __forceinline__ void rw_dot2(const float* k, const float* c, const float* hi, const float* lo, float pad,
                                        float& kx, float& cx) {
    float a = 0.0f, b = 0.0f;
#pragma unroll
    for (int i = 0; i < NC; ++i) {
        a = __fmaf_rn(k[i], hi[i], a);
        b = __fmaf_rn(c[i], hi[i], b);
    }
    if (NC < MAXS) {
        a = __fadd_rn(a, pad);
        b = __fadd_rn(b, pad);
    }
#pragma unroll
    for (int i = 0; i < NC; ++i) {
        a = __fmaf_rn(k[i], lo[i], a);
        b = __fmaf_rn(c[i], lo[i], b);
    }
    if (NC < MAXS) {
        a = __fadd_rn(a, pad);
        b = __fadd_rn(b, pad);
    }
    kx = a;
    cx = b;
}
// the lo-part sums of this lane's rows (sum_j M(i,j) x_lo[j], then the
// padding term): independent of this step's inputs, formed ahead of them
template <int NC, int MC>
__device__ __forceinline__ void rw_lo(const float (*m)[MC], const float* lo, float pad, float* out) {
#pragma unroll
    for (int rr = 0; rr < NC / SW_LANES; ++rr) {
        float l = 0.0f;
#pragma unroll
        for (int j = 0; j < NC; ++j) l = __fmaf_rn(m[rr][j], lo[j], l);
        if (NC < MC) l = __fadd_rn(l, pad);
        out[rr] = l;
    }
}
// this lane's observer rows: the increment (A-I)xh + B u + L yerr, then the
// double-float add onto the row's old value (old_hi / old_lo in, new out)
template <int NC>
__device__ __forceinline__ void rw_obs(const float (*sai)[MAXS], const float* sb, const float* Lr, float u, float yerr,
                                       const float* xh_hi, const float* lsum, float pad, float* nh, float* nlo) {
#pragma unroll
    for (int rr = 0; rr < NC / SW_LANES; ++rr) {
        float h = __fmaf_rn(Lr[rr], yerr, __fmul_rn(sb[rr], u));
#pragma unroll
        for (int j = 0; j < NC; ++j) h = __fmaf_rn(sai[rr][j], xh_hi[j], h);
        if (NC < MAXS) h = __fadd_rn(h, pad);
        df_add(nh[rr], nlo[rr], h, lsum[rr]);
    }
}
// this lane's plant rows: (Ad-I)xp + Bu u + Bw W, then the double-float add
template <int NC>
__device__ __forceinline__ void rw_plant(const float (*dai)[MAXD], const float (*dbw)[MAXW], const float* dbu,
                                         float u, const float* W, const float* xp_hi, const float* lsum, float pad,
                                         float* ph, float* plo) {
#pragma unroll
    for (int rr = 0; rr < NC / SW_LANES; ++rr) {
        float h = __fmul_rn(dbu[rr], u);
#pragma unroll
        for (int k = 0; k < MAXW; ++k) h = __fmaf_rn(dbw[rr][k], W[k], h);
#pragma unroll
        for (int j = 0; j < NC; ++j) h = __fmaf_rn(dai[rr][j], xp_hi[j], h);
        if (NC < MAXD) h = __fadd_rn(h, pad);
        df_add(ph[rr], plo[rr], h, lsum[rr]);
    }
}
// a padded state turns NaN once a zero coefficient meets a non-finite operand
template <int NC>
__device__ __forceinline__ bool rw_bad(const float* hi, const float* lo) {
    bool bad = false;
#pragma unroll
    for (int j = 0; j < NC; ++j) bad = bad || !isfinite(hi[j]) || !isfinite(lo[j]);
    return bad;
}

// The chain interpreter of the wide form.  Each slot forms add, subtract and
// multiply as one fused multiply-add (a + b = fma(b, 1, a), a - b = fma(b, -1, a),
// a b = fma(a, b, -0): each rounds once, exactly as the separate operation, -0
// included), the saturation and the sign without branches, and the quotient
// only in lanes whose slot divides.  Lanes interpreting different operations
// (a quad's four NL chains) then execute one path instead of one per
// operation.  Source column MAXD of the plant-side chains is the plant output
// y, taken from a register (yv).
template <bool HAS_SEED, int MAXC, bool YCOL>
__device__ __forceinline__ float chain_sel(const float* __restrict__ t, int slot0, int n, const float* src, float yv,
                                           float seed) {
    float result = 0.0f;
#pragma unroll
    for (int r = 0; r < MAXC; ++r) {
        if (r >= n) break;
        const int f = RT_INS + 3 * (slot0 + r);
        const unsigned code = __float_as_uint(t[f * WIDE_TS]);
        const int op = (int)(code & 0xFFu), col = (int)((code >> 8) & 0xFFu);
        const int ak = (int)((code >> 16) & 0xFFu), bk = (int)(code >> 24);
        float pos = src[col];
        if (YCOL && col == MAXD) pos = yv;
        const float prev = r == 0 ? ((HAS_SEED && !isnan(seed)) ? seed : pos) : result;
        const float a = ak == CE_OPERAND_CONST ? t[(f + 1) * WIDE_TS] : (ak == CE_OPERAND_STATE ? pos : prev);
        const float b = bk == CE_OPERAND_CONST ? t[(f + 2) * WIDE_TS] : (bk == CE_OPERAND_STATE ? pos : prev);
        const bool m = op == 3;
        const float f3 = __fmaf_rn(m ? a : b, m ? b : (op == 1 ? 1.0f : -1.0f), m ? -0.0f : a);
        const float sat = fmin(fmax(prev, a), b);
        const float sg = (float)((0.0f < a) - (a < 0.0f));
        float v = (op >= 1 && op <= 3) ? f3 : op == 5 ? sat : op == 6 ? sg : result;
        if (op == 4) v = rdiv(a, b);
        result = v;
    }
    return result;
}

// The quad's steps.  s8 / d8: the warp's observer / plant class is 8 rows
// (two per lane) rather than 4 (one per lane); both are warp-uniform, so the
// class only selects the row arithmetic and the chain interpreters, the bulk
// of the code, exist once.
__device__ __forceinline__ void ragged_wide_steps(const Run& run, const float* t, float* st, float (*stage)[SW_CPB],
                                                  const int cl, const int q, const unsigned qm, const bool s8,
                                                  const bool d8, const float* __restrict__ row,
                                                  float* __restrict__ wrow, SimSummary* __restrict__ out) {
    const int rs = s8 ? 2 : 1, rd = d8 ? 2 : 1;  // rows per lane
    const int rs0 = q * rs, rd0 = q * rd;
    const int ns = run.ns;
    float sai[2][MAXS], dai[2][MAXD], sb[2], dbu[2], Lr[2], K[MAXS];
#pragma unroll
    for (int rr = 0; rr < 2; ++rr) {
        const int i = rs0 + (rr < rs ? rr : 0);  // a second row only in class 8
#pragma unroll
        for (int j = 0; j < MAXS; ++j) sai[rr][j] = t[(RT_SAI + i * MAXS + j) * WIDE_TS];
        sb[rr] = t[(RT_SB + i) * WIDE_TS];
        Lr[rr] = i < ns ? row[ns + i] : 0.0f;
        const int d = rd0 + (rr < rd ? rr : 0);
#pragma unroll
        for (int j = 0; j < MAXD; ++j) dai[rr][j] = t[(RT_DAI + d * MAXD + j) * WIDE_TS];
        dbu[rr] = t[(RT_DBU + d) * WIDE_TS];
    }
#pragma unroll
    for (int j = 0; j < MAXS; ++j) K[j] = j < ns ? row[j] : 0.0f;
    const float sd = t[RT_SD * WIDE_TS];
    const unsigned cnt0 = __float_as_uint(t[RT_CNT * WIDE_TS]), cnt1 = __float_as_uint(t[(RT_CNT + 1) * WIDE_TS]);
    const int n_dc = (int)(cnt0 & 0xFFu), n_u = (int)((cnt0 >> 8) & 0xFFu);
    const int n_nl = q == 0 ? (int)((cnt0 >> 16) & 0xFFu) : q == 1 ? (int)(cnt0 >> 24)
                   : q == 2 ? (int)(cnt1 & 0xFFu) : (int)((cnt1 >> 8) & 0xFFu);
    const float N = row[2 * ns];

    float xh_hi[MAXS], xh_lo[MAXS], xp_hi[MAXD], xp_lo[MAXD];
#pragma unroll
    for (int i = 0; i < MAXS; ++i) xh_hi[i] = xh_lo[i] = xp_hi[i] = xp_lo[i] = 0.0f;
    bool poisS = false, poisD = false;
    float ysum = 0.0f, ycomp = 0.0f, ymax = -CUDART_INF_F, ymin = CUDART_INF_F;
    // the instance's scalars in registers: its Run lives in global memory, and
    // the fit-window stores could alias it, so reads inside the loop would be
    // reloaded every step
    const int T = run.time, fit0 = run.fit_start_id, fitn = run.fit_steps, ss0 = run.steady_start_id,
              rstep = run.ref_step_id;
    const float ramp = run.ref_amp;
    float y = 0.0f;  // the plant output of the previous step (a DC source column MAXD reads it)
    for (int tt = 0; tt < T; ++tt) {
        const float padS = poisS ? CUDART_NAN_F : 0.0f;
        const float padD = poisD ? CUDART_NAN_F : 0.0f;
        // the sums that do not depend on this step's y, u or W first (independent
        // chains the warp can overlap with the interpreted ones)
        float sc[MAXS];  // C of the observer model, from the table (registers are short here)
#pragma unroll
        for (int j = 0; j < MAXS; ++j) sc[j] = t[(RT_SC + j) * WIDE_TS];
        float kx, cx, lo_s[2], lo_d[2];
        if (s8) {
            rw_dot2<8>(K, sc, xh_hi, xh_lo, padS, kx, cx);
            rw_lo<8, MAXS>(sai, xh_lo, padS, lo_s);
        } else {
            rw_dot2<4>(K, sc, xh_hi, xh_lo, padS, kx, cx);
            rw_lo<4, MAXS>(sai, xh_lo, padS, lo_s);
        }
        if (d8) rw_lo<8, MAXD>(dai, xp_lo, padD, lo_d);
        else rw_lo<4, MAXD>(dai, xp_lo, padD, lo_d);
        // plant output
        y = chain_sel<false, MAX_DC, true>(t, 0, n_dc, st + WS_XP_HI, y, 0.0f);
        // fit window (lane 0), steady-state sum and extremes (every lane keeps
        // them, lane 0 stores them)
        {
            const int w = tt - fit0;
            if (q == 0 && w >= 0 && w < fitn) {
                stage[w & 7][cl] = y;
                if ((w & 7) == 7 || w == fitn - 1 || tt == T - 1) {
                    float4 a, b;
                    a.x = stage[0][cl]; a.y = stage[1][cl]; a.z = stage[2][cl]; a.w = stage[3][cl];
                    b.x = stage[4][cl]; b.y = stage[5][cl]; b.z = stage[6][cl]; b.w = stage[7][cl];
                    float4* dst = reinterpret_cast<float4*>(wrow + (w & ~7));
                    dst[0] = a;
                    dst[1] = b;
                }
            }
            if (tt >= ss0) ysum_add(ysum, ycomp, y);
            ymax = fmaxf(ymax, y);
            ymin = fminf(ymin, y);
        }
        // controller output
        const float ref = tt < rstep ? 0.0f : ramp;
        const float u_raw = __fmaf_rn(N, ref, -kx);
        const float u = chain_sel<true, MAX_U, false>(t, MAX_DC, n_u, st + WS_XH_HI, 0.0f, u_raw);
        // observer output error
        const float yh = __fmaf_rn(sd, u, cx);
        const float yerr = __fsub_rn(y, yh);
        // this lane's nonlinear term over [xp_hi, y]
        st[WS_W + q] = chain_sel<false, MAX_NL, true>(t, MAX_DC + MAX_U + q * MAX_NL, n_nl, st + WS_XP_HI, y, 0.0f);
        // this lane's observer rows; the rows' old values from the slot (an index
        // by lane would put the state arrays in local memory); nothing writes the
        // slot's state before the barrier below
        float nh[2], nlo[2];
        nh[0] = st[WS_XH_HI + rs0];
        nlo[0] = st[WS_XH_LO + rs0];
        if (s8) {
            nh[1] = st[WS_XH_HI + rs0 + 1];
            nlo[1] = st[WS_XH_LO + rs0 + 1];
            rw_obs<8>(sai, sb, Lr, u, yerr, xh_hi, lo_s, padS, nh, nlo);
        } else {
            rw_obs<4>(sai, sb, Lr, u, yerr, xh_hi, lo_s, padS, nh, nlo);
            poisS = poisS || !isfinite(yerr) || !isfinite(u) || rw_bad<4>(xh_hi, xh_lo);
        }
        __syncwarp(qm);  // every W is in the slot; every read of this step's state is done
        float W[MAXW], dbw[2][MAXW];  // Bw rows from the table (registers are short here)
#pragma unroll
        for (int k = 0; k < MAXW; ++k) W[k] = st[WS_W + k];
#pragma unroll
        for (int rr = 0; rr < 2; ++rr)
#pragma unroll
            for (int k = 0; k < MAXW; ++k) dbw[rr][k] = t[(RT_DBW + (rd0 + (rr < rd ? rr : 0)) * MAXW + k) * WIDE_TS];
        // this lane's plant rows
        float ph[2], plo[2];
        ph[0] = st[WS_XP_HI + rd0];
        plo[0] = st[WS_XP_LO + rd0];
        if (d8) {
            ph[1] = st[WS_XP_HI + rd0 + 1];
            plo[1] = st[WS_XP_LO + rd0 + 1];
            rw_plant<8>(dai, dbw, dbu, u, W, xp_hi, lo_d, padD, ph, plo);
        } else {
            rw_plant<4>(dai, dbw, dbu, u, W, xp_hi, lo_d, padD, ph, plo);
            bool bad = !isfinite(u);
#pragma unroll
            for (int k = 0; k < MAXW; ++k) bad = bad || !isfinite(W[k]);
            poisD = poisD || bad || rw_bad<4>(xp_hi, xp_lo);
        }
        // publish this lane's rows, then read the whole new state
        st[WS_XH_HI + rs0] = nh[0];
        st[WS_XH_LO + rs0] = nlo[0];
        if (s8) {
            st[WS_XH_HI + rs0 + 1] = nh[1];
            st[WS_XH_LO + rs0 + 1] = nlo[1];
        }
        st[WS_XP_HI + rd0] = ph[0];
        st[WS_XP_LO + rd0] = plo[0];
        if (d8) {
            st[WS_XP_HI + rd0 + 1] = ph[1];
            st[WS_XP_LO + rd0 + 1] = plo[1];
        }
        __syncwarp(qm);
        // rows 4..7 stay zero in class 4 (no lane owns them)
#pragma unroll
        for (int i = 0; i < MAXS; i += 4) {
            const float4 a = *reinterpret_cast<const float4*>(st + WS_XH_HI + i);
            const float4 b = *reinterpret_cast<const float4*>(st + WS_XH_LO + i);
            const float4 e = *reinterpret_cast<const float4*>(st + WS_XP_HI + i);
            const float4 f = *reinterpret_cast<const float4*>(st + WS_XP_LO + i);
            xh_hi[i] = a.x; xh_hi[i + 1] = a.y; xh_hi[i + 2] = a.z; xh_hi[i + 3] = a.w;
            xh_lo[i] = b.x; xh_lo[i + 1] = b.y; xh_lo[i + 2] = b.z; xh_lo[i + 3] = b.w;
            xp_hi[i] = e.x; xp_hi[i + 1] = e.y; xp_hi[i + 2] = e.z; xp_hi[i + 3] = e.w;
            xp_lo[i] = f.x; xp_lo[i + 1] = f.y; xp_lo[i + 2] = f.z; xp_lo[i + 3] = f.w;
        }
    }
    if (q == 0) {
        SimSummary sm;
        sm.ysum = ysum;
        sm.ymax = ymax;
        sm.ymin = ymin;
        sm.ycomp = ycomp;
        *out = sm;
    }
}

__global__ void __launch_bounds__(SIM_BLOCK, 8) k_sim_ragged_wide(const Run launch, const float* __restrict__ gains,
                                                               float* __restrict__ ywin,
                                                               SimSummary* __restrict__ summ) {
    __shared__ float tab[RT_FIELDS * WIDE_TS];
    __shared__ __align__(16) float slots[SW_CPB * WS_STRIDE];
    __shared__ float stage[8][SW_CPB];
    const int q = threadIdx.x & 3, cl = threadIdx.x >> 2;
    const unsigned qm = 0xFu << (threadIdx.x & 28);
    const int64_t c = (int64_t)blockIdx.x * SW_CPB + cl;
    if (c >= launch.n) return;  // the whole quad leaves together
    const Run& run = run_of<true>(launch, c);
    {
        // the candidate's table column, copied once by its quad
        const float* __restrict__ g = launch.rg.tab + c;
        const int64_t gs = launch.rg.tab_stride;
        for (int f = q; f < RT_FIELDS; f += SW_LANES) tab[f * WIDE_TS + cl] = g[(int64_t)f * gs];
    }
    float* st = slots + cl * WS_STRIDE;
    // the state slot starts at zero, padded rows included (they stay zero for a
    // class below 8: no lane owns them, and no program reads them)
    for (int k = q; k < WS_STRIDE; k += SW_LANES) st[k] = 0.0f;
    // The warp runs the largest dimension class among its candidates (any
    // class at least the candidate's own gives its result), so its quads do
    // not diverge; a device order grouped by class keeps most warps at their
    // candidates' own class.  The lanes still here are whole quads.
    const unsigned live = __activemask();
    const bool s8 = launch.rg.full_width || __any_sync(live, run.ns > 4);
    const bool d8 = launch.rg.full_width || __any_sync(live, run.nd > 4);
    __syncwarp(qm);
    const float* t = tab + cl;  // field f at t[f * WIDE_TS]
    const float* row = gains + c * run.cuda_w;
    float* wrow = ywin + c * (int64_t)run.fit_pitch;
    ragged_wide_steps(run, t, st, stage, cl, q, qm, s8, d8, row, wrow, summ + c);
}

// The per-candidate table of a ragged batch (the RT_* fields) from the
// instances' plants: one thread per candidate, each field a coalesced store.
__global__ void __launch_bounds__(128) k_ragged_table(int64_t n, const Plant* __restrict__ plants,
                                                      const int* __restrict__ inst, float* __restrict__ tab,
                                                      int64_t stride) {
    const int64_t c = (int64_t)blockIdx.x * 128 + threadIdx.x;
    if (c >= n) return;
    const Plant& P = plants[inst[c]];
    auto put = [&](int f, float v) { tab[(int64_t)f * stride + c] = v; };
    auto put_u = [&](int f, unsigned v) { put(f, __uint_as_float(v)); };
    for (int e = 0; e < MAXS * MAXS; ++e) put(RT_SAI + e, P.ss_ai[e]);
    for (int i = 0; i < MAXS; ++i) {
        put(RT_SB + i, P.ss_b[i]);
        put(RT_SC + i, P.ss_c[i]);
    }
    put(RT_SD, P.ss_d);
    for (int e = 0; e < MAXD * MAXD; ++e) put(RT_DAI + e, P.d_ai[e]);
    for (int i = 0; i < MAXD; ++i) put(RT_DBU + i, P.d_bu[i]);
    for (int e = 0; e < MAXD * MAXW; ++e) put(RT_DBW + e, P.d_bw[e]);
    put_u(RT_CNT, (unsigned)P.n_dc | (unsigned)P.n_u << 8 | (unsigned)P.n_nl[0] << 16 | (unsigned)P.n_nl[1] << 24);
    put_u(RT_CNT + 1, (unsigned)P.n_nl[2] | (unsigned)P.n_nl[3] << 8);
    auto slot = [&](int sl, const Instr& I) {
        // an op outside 1..6 leaves the result unchanged whatever its value
        const unsigned op = (I.op >= 1 && I.op <= 6) ? (unsigned)I.op : 7u;
        put_u(RT_INS + 3 * sl, op | (unsigned)I.col << 8 | (unsigned)I.akind << 16 | (unsigned)I.bkind << 24);
        put(RT_INS + 3 * sl + 1, I.aval);
        put(RT_INS + 3 * sl + 2, I.bval);
    };
    // every slot defined: unused ones are empty instructions (code 0, column 0)
    for (int sl = 0; sl < RT_SLOTS; ++sl) {
        put_u(RT_INS + 3 * sl, 0u);
        put(RT_INS + 3 * sl + 1, 0.0f);
        put(RT_INS + 3 * sl + 2, 0.0f);
    }
    for (int k = 0; k < P.n_dc; ++k) slot(k, P.dc[k]);
    for (int k = 0; k < P.n_u; ++k) slot(MAX_DC + k, P.u[k]);
    for (int w = 0; w < MAXW; ++w)
        for (int k = 0; k < P.n_nl[w]; ++k) slot(MAX_DC + MAX_U + w * MAX_NL + k, P.nl[w][k]);
}

// Rows of a ragged batch between the caller's packing (instance after
// instance, each row at its instance's widths) and the device order at the
// batch's widths LW / LI (padding written as 0).  Device position c holds the
// caller's gains row at goff[c] and INFO row at ioff[c], wid[c] = (cuda_w, info_w).
// One thread per element of the device rows: the stores are coalesced.
__global__ void __launch_bounds__(256) k_ragged_gather(int64_t n, const int64_t* __restrict__ goff,
                                                       const int64_t* __restrict__ ioff, const int2* __restrict__ wid,
                                                       int LW, int LI, const float* __restrict__ g_in,
                                                       const float* __restrict__ i_in, float* __restrict__ g_dev,
                                                       float* __restrict__ i_dev) {
    const int64_t t = (int64_t)blockIdx.x * 256 + threadIdx.x;
    const int64_t per = LW + LI;
    if (t >= n * per) return;
    const int64_t c = t / per;
    const int e = (int)(t - c * per);
    const int2 w = wid[c];
    if (e < LW) g_dev[c * LW + e] = e < w.x ? g_in[goff[c] + e] : 0.0f;
    else i_dev[c * LI + (e - LW)] = e - LW < w.y ? i_in[ioff[c] + (e - LW)] : 0.0f;
}

__global__ void __launch_bounds__(256) k_ragged_scatter(int64_t n, const int64_t* __restrict__ ioff,
                                                        const int2* __restrict__ wid, int LI,
                                                        const float* __restrict__ i_dev, float* __restrict__ i_out) {
    const int64_t t = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (t >= n * LI) return;
    const int64_t c = t / LI;
    const int e = (int)(t - c * LI);
    if (e < wid[c].y) i_out[ioff[c] + e] = i_dev[c * LI + e];
}

void launch_ragged_gather(int64_t n, const int64_t* goff, const int64_t* ioff, const int2* wid, int LW, int LI,
                          const float* g_in, const float* i_in, float* g_dev, float* i_dev, cudaStream_t st) {
    const int64_t total = n * (LW + LI);
    k_ragged_gather<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(n, goff, ioff, wid, LW, LI, g_in, i_in, g_dev,
                                                                      i_dev);
    CE_CUDA(cudaGetLastError());
}

void launch_ragged_scatter(int64_t n, const int64_t* ioff, const int2* wid, int LI, const float* i_dev, float* i_out,
                           cudaStream_t st) {
    const int64_t total = n * LI;
    k_ragged_scatter<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(n, ioff, wid, LI, i_dev, i_out);
    CE_CUDA(cudaGetLastError());
}

void launch_ragged_table(int64_t n, const Plant* plants, const int* inst, float* tab, int64_t stride,
                         cudaStream_t st) {
    k_ragged_table<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(n, plants, inst, tab, stride);
    CE_CUDA(cudaGetLastError());
}

// The discrete-plant values and instruction constants the FP64 step reads: the
// launch's Plant, or with per-candidate plants (MC) the candidate's row of the
// plant table -- matrices staged once into this thread's column of dynamic
// shared memory (FIELDS x SIM_BLOCK words), constants read from the table
// where an instruction uses one.
template <int NDC, bool MC>
struct F64Plant {
    static constexpr int F_BU = NDC * NDC, F_BW = F_BU + NDC, FIELDS = F_BW + NDC * MAXW;
    const Plant& P;
    const float* col = nullptr;
    const float* cst = nullptr;
    int64_t cs = 0;
    __device__ __forceinline__ F64Plant(const Run& run, const Plant& plant, int64_t c) : P(plant) {
        if constexpr (MC) {
            extern __shared__ float f64_cols[];
            const float* __restrict__ t = run.mc.tab;
            const int64_t np = run.mc.np, pc = mc_plant(run.mc, c);
            float* w = f64_cols + threadIdx.x;
#pragma unroll
            for (int i = 0; i < NDC; ++i) {
#pragma unroll
                for (int j = 0; j < NDC; ++j) w[(i * NDC + j) * SIM_BLOCK] = t[(int64_t)(MC_AI + i * MAXD + j) * np + pc];
                w[(F_BU + i) * SIM_BLOCK] = t[(int64_t)(MC_BU + i) * np + pc];
#pragma unroll
                for (int k = 0; k < MAXW; ++k)
                    w[(F_BW + i * MAXW + k) * SIM_BLOCK] = t[(int64_t)(MC_BW + i * MAXW + k) * np + pc];
            }
            col = w;
            cst = t + (int64_t)MC_CST * np + pc;
            cs = np;
        }
    }
    // the plant values, floats as stored
    __device__ __forceinline__ float ai(int i, int j) const {
        return MC ? col[(i * NDC + j) * SIM_BLOCK] : P.d_ai[i * MAXD + j];
    }
    __device__ __forceinline__ float bu(int i) const { return MC ? col[(F_BU + i) * SIM_BLOCK] : P.d_bu[i]; }
    __device__ __forceinline__ float bw(int i, int k) const {
        return MC ? col[(F_BW + i * MAXW + k) * SIM_BLOCK] : P.d_bw[i * MAXW + k];
    }
    // the constants of the chain whose first instruction is constant slot slot0
    __device__ __forceinline__ const float* k(int slot0) const { return MC ? cst + (int64_t)2 * slot0 * cs : nullptr; }
};

// The extended-precision forms of the same recurrence, one value per state (no
// hi/lo split of the mixed form): R = double is the plain FP64 form; R = ddf
// (double-float) the simulation of the compensated_df precision, the same
// operations in double-float arithmetic on the FP32 pipe.  The float
// coefficients enter exactly in both; the trajectory and the summaries are
// written as doubles.
template <typename R>
__device__ __forceinline__ double as_double(R v) { return (double)v; }

// The running sums of the recurrence (x + sum_k a_k v_k with float
// coefficients a_k): for double one fused multiply-add per term, in order; for
// double-float a compensated dot product (Ogita, Rump and Oishi's Dot2): the
// float running sum s, each product's exact error and each addition's exact
// error (TwoProduct, TwoSum) gathered in c, and s + c normalised once at the
// end -- as accurate as double-float arithmetic per term, with one float
// addition on the dependent chain per term instead of a full double-float add.
template <typename R> struct Acc;
template <> struct Acc<double> {
    double v;
    __device__ __forceinline__ explicit Acc(double x) : v(x) {}
    __device__ __forceinline__ void add(float a, double x) { v = __fma_rn((double)a, x, v); }
    __device__ __forceinline__ double get() const { return v; }
};
template <> struct Acc<ddf> {
    float s, c;
    __device__ __forceinline__ explicit Acc(ddf x) : s(x.hi), c(x.lo) {}
    __device__ __forceinline__ void add(float a, ddf x) {
        const float p = __fmul_rn(a, x.hi);
        const float e = __fmaf_rn(a, x.lo, __fmaf_rn(a, x.hi, -p));
        const ddf t = dd::dd_two_sum(s, p);
        s = t.hi;
        c = __fadd_rn(c, __fadd_rn(t.lo, e));
    }
    __device__ __forceinline__ ddf get() const {
        if (!isfinite(s)) return ddf(s, 0.0f);
        const ddf r = dd::dd_fast_sum(s, c);
        return isfinite(r.hi) ? r : ddf(r.hi, 0.0f);
    }
};

template <typename R, int NSC, int NDC, bool MC = false>
__global__ void __launch_bounds__(SIM_BLOCK) k_sim_ext(const Run run, const __grid_constant__ Plant P,
                                                       const float* __restrict__ gains, double* __restrict__ ywin,
                                                       double* __restrict__ summ) {
    const int tid = threadIdx.x;
    const int64_t c = (int64_t)blockIdx.x * SIM_BLOCK + tid;
    if (c >= run.n) return;
    const F64Plant<NDC, MC> pv(run, P, c);
    const int ns = run.ns;
    const float* row = gains + c * run.cuda_w;
    float K[NSC], L[NSC];
#pragma unroll
    for (int i = 0; i < NSC; ++i) {
        K[i] = i < ns ? row[i] : 0.0f;
        L[i] = i < ns ? row[ns + i] : 0.0f;
    }
    const R N = R(row[2 * ns]);
    R xh[NSC], xp[NDC];
#pragma unroll
    for (int i = 0; i < NSC; ++i) xh[i] = R(0);
#pragma unroll
    for (int i = 0; i < NDC; ++i) xp[i] = R(0);
    R ysum = R(0), ymax = rneg(rinf<R>()), ymin = rinf<R>();
    double* wrow = ywin + c * (int64_t)run.fit_pitch;
    const int T = run.time;
    for (int t = 0; t < T; ++t) {
        const R y = run_chain<R, NDC, MAX_DC, false, MC>(P.dc, P.n_dc, xp, -1, R(0), R(0), pv.k(0), pv.cs);
        const int w = t - run.fit_start_id;
        if (w >= 0 && w < run.fit_steps) wrow[w] = as_double(y);
        if (t >= run.steady_start_id) ysum = radd(ysum, y);
        ymax = fmax(ymax, y);
        ymin = fmin(ymin, y);
        Acc<R> kx(R(0));
#pragma unroll
        for (int i = 0; i < NSC; ++i) kx.add(K[i], xh[i]);
        const R ref = t < run.ref_step_id ? R(0) : R(run.ref_amp);
        const R u = run_chain<R, NSC, MAX_U, true, MC>(P.u, P.n_u, xh, -1, R(0), rfma(N, ref, rneg(kx.get())),
                                                        pv.k(MAX_DC), pv.cs);
        Acc<R> yh(R(0));
#pragma unroll
        for (int i = 0; i < NSC; ++i) yh.add(P.ss_c[i], xh[i]);
        yh.add(P.ss_d, u);
        const R yerr = rsub(y, yh.get());
        R dh[NSC];
#pragma unroll
        for (int i = 0; i < NSC; ++i) {
            Acc<R> h(rmul(P.ss_b[i], u));
            h.add(L[i], yerr);
#pragma unroll
            for (int j = 0; j < NSC; ++j) h.add(P.ss_ai[i * MAXS + j], xh[j]);
            dh[i] = h.get();
        }
#pragma unroll
        for (int i = 0; i < NSC; ++i) xh[i] = radd(xh[i], dh[i]);
        R W[MAXW];
#pragma unroll
        for (int k = 0; k < MAXW; ++k)
            W[k] = run_chain<R, NDC, MAX_NL, false, MC>(P.nl[k], P.n_nl[k], xp, MAXD, y, R(0),
                                                        pv.k(MAX_DC + MAX_U + k * MAX_NL), pv.cs);
        R ph[NDC];
#pragma unroll
        for (int i = 0; i < NDC; ++i) {
            Acc<R> h(rmul(pv.bu(i), u));
#pragma unroll
            for (int k = 0; k < MAXW; ++k) h.add(pv.bw(i, k), W[k]);
#pragma unroll
            for (int j = 0; j < NDC; ++j) h.add(pv.ai(i, j), xp[j]);
            ph[i] = h.get();
        }
#pragma unroll
        for (int i = 0; i < NDC; ++i) xp[i] = radd(xp[i], ph[i]);
    }
    summ[4 * c + 0] = as_double(ysum);
    summ[4 * c + 1] = as_double(ymax);
    summ[4 * c + 2] = as_double(ymin);
    summ[4 * c + 3] = 0.0;
}

// The gain schedules of the Kalman per-candidate list.  The covariance
// recursion reads only the observer model, R and diag(Q), so a candidate's
// gains can be computed ahead of its trajectory: one thread per list position
// runs the per-candidate form's recursion (kalman_cov_lane, the same
// operations) for up to KAL_SCHED_STEPS steps and stores each step's gain.  A
// snapshot of P every KAL_SCHED_SNAP steps is compared bit for bit with
// P_{t+1}; once equal, the recursion is periodic -- P_{t+1} = P_{t0} makes
// every later gain the one p = t + 1 - t0 steps earlier -- and the thread
// stops.  Periodic positions are listed for the scheduled simulation form;
// the others (no period within the schedule) for the quad form, which runs
// their recursion in full.

__global__ void __launch_bounds__(SIM_BLOCK) k_kal_schedule(const Run run, const __grid_constant__ Plant P,
                                                            const float* __restrict__ gains, float* __restrict__ sched,
                                                            int2* __restrict__ meta, int* __restrict__ lists,
                                                            int* __restrict__ totals) {
    __shared__ float snap[MAXS * MAXS][SIM_BLOCK];
    const int tid = threadIdx.x;
    const int64_t lp = (int64_t)blockIdx.x * SIM_BLOCK + tid;
    if (lp >= (int64_t)run.kal_totals[1] + run.kal_totals[2]) return;
    const int64_t c = kal_list_candidate(run, lp);
    const int ns = run.ns;
    const float* row = gains + c * run.cuda_w;
    const float Rn = row[2 * ns + 1];
    float Qd[MAXS], Pm[MAXS * MAXS], KG[MAXS];
#pragma unroll
    for (int i = 0; i < MAXS; ++i) Qd[i] = i < ns ? row[2 * ns + 2 + i] : 0.0f;
#pragma unroll
    for (int e = 0; e < MAXS * MAXS; ++e) Pm[e] = 0.0f;
    const int64_t S = run.kal_sched_n;
    const int steps = min(run.time, KAL_SCHED_STEPS);
    int t_snap = 0;
    int2 m = make_int2(-1, 0);
    for (int t = 0; t < steps; ++t) {
        if (t - t_snap == KAL_SCHED_SNAP || t == 0) {
#pragma unroll
            for (int e = 0; e < MAXS * MAXS; ++e) snap[e][tid] = Pm[e];
            t_snap = t;
        }
        kalman_cov_lane(P, Pm, Qd, Rn, KG);
#pragma unroll
        for (int k = 0; k < MAXS; ++k) sched[((int64_t)t * MAXS + k) * S + lp] = KG[k];
        bool same = true;
#pragma unroll
        for (int e = 0; e < MAXS * MAXS; ++e) same = same && __float_as_uint(Pm[e]) == __float_as_uint(snap[e][tid]);
        if (same) {
            m = make_int2(t_snap, t + 1 - t_snap);
            break;
        }
    }
    meta[lp] = m;
    if (m.x >= 0) lists[atomicAdd(&totals[3], 1)] = (int)lp;
    else lists[S + atomicAdd(&totals[4], 1)] = (int)lp;
}

void launch_kalman_schedule(const Run& run, const Plant& P, const float* gains, const KalGroups& g,
                            cudaStream_t st) {
    const int grid = (int)((run.n + SIM_BLOCK - 1) / SIM_BLOCK);
    k_kal_schedule<<<grid, SIM_BLOCK, 0, st>>>(run, P, gains, g.sched, g.meta, g.lists, g.totals);
    CE_CUDA(cudaGetLastError());
}

static int dim_class(int d) { return d <= 4 ? 4 : 8; }

// Lanes per candidate of a ragged batch's simulation: 4 (the wide form,
// default) or 1 (CE_RAGGED_WIDE=0).  The host deals a batch's candidates to
// warps of 32 / lanes.
int ragged_lanes_per_candidate() {
    static const int v = [] {
        const char* e = std::getenv("CE_RAGGED_WIDE");
        return (e && e[0] == '0') ? 1 : SW_LANES;
    }();
    return v;
}

template <int NSC, int NDC, int KMODE = SIM_LUENBERGER>
static void sim_launch(const Run& run, const Plant& P, int precision, const float* gains, void* ywin, void* summ,
                       float* traj, cudaStream_t st) {
    const int grid = sim_grid(run);
    if (precision == CE_PRECISION_FP64 || precision == CE_PRECISION_COMPENSATED_DF) {
        if (KMODE != SIM_LUENBERGER) throw std::runtime_error("the Kalman observer runs in mixed precision only");
        auto go = [&](auto r) {
            using R = decltype(r);
            if (run.mc.tab) {
                // per-candidate plants: each thread's plant matrices in its shared-memory column
                const size_t cols = (size_t)F64Plant<NDC, true>::FIELDS * SIM_BLOCK * sizeof(float);
                prefer_shared((const void*)k_sim_ext<R, NSC, NDC, true>);
                k_sim_ext<R, NSC, NDC, true><<<grid, SIM_BLOCK, cols, st>>>(run, P, gains, (double*)ywin,
                                                                            (double*)summ);
                return;
            }
            prefer_shared((const void*)k_sim_ext<R, NSC, NDC>);
            k_sim_ext<R, NSC, NDC><<<grid, SIM_BLOCK, 0, st>>>(run, P, gains, (double*)ywin, (double*)summ);
        };
        if (precision == CE_PRECISION_FP64) go(0.0);
        else go(ddf(0.0f));
    } else {
        prefer_shared((const void*)k_sim_mixed<NSC, NDC, KMODE>);
        k_sim_mixed<NSC, NDC, KMODE><<<grid, SIM_BLOCK, 0, st>>>(run, P, gains, (float*)ywin, (SimSummary*)summ, traj);
    }
}

void launch_sim(const Run& run, const Plant& P, int precision, const float* gains, void* ywin, void* summ, float* traj,
                cudaStream_t st) {
    const int cs = dim_class(run.ns), cd = dim_class(run.nd);
    if (run.rg.runs) {
        // a ragged batch: every instance's plant and program from the table; the
        // wide form runs each warp at the dimension class of its candidates
        if (precision != CE_PRECISION_MIXED || run.kalman)
            throw std::runtime_error("a ragged batch runs the Luenberger loop in mixed precision");
        if (run.rg.lanes == SW_LANES && !traj) {
            prefer_shared((const void*)k_sim_ragged_wide);
            k_sim_ragged_wide<<<(unsigned)((run.n + SW_CPB - 1) / SW_CPB), SIM_BLOCK, 0, st>>>(
                run, gains, (float*)ywin, (SimSummary*)summ);
        } else {
            const size_t cols = (size_t)RT_FIELDS * SIM_BLOCK * sizeof(float);  // the candidates' table columns
            CE_CUDA(cudaFuncSetAttribute((const void*)k_sim_ragged, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)cols));
            prefer_shared((const void*)k_sim_ragged);
            k_sim_ragged<<<sim_grid(run), SIM_BLOCK, cols, st>>>(run, P, gains, (float*)ywin, (SimSummary*)summ,
                                                                 traj);
        }
    } else if (run.kalman && run.kal_list == 1) {
        // the shared-noise form; the Kalman loop always runs the full padded observer width
        if (cd == 4) sim_launch<8, 4, SIM_KALMAN_SHARED>(run, P, precision, gains, ywin, summ, traj, st);
        else sim_launch<8, 8, SIM_KALMAN_SHARED>(run, P, precision, gains, ywin, summ, traj, st);
    } else if (run.kalman && run.kal_list == 3) {
        // the per-candidate list's positions whose gain schedule turned periodic
        if (cd == 4) sim_launch<8, 4, SIM_KALMAN_SCHED>(run, P, precision, gains, ywin, summ, traj, st);
        else sim_launch<8, 8, SIM_KALMAN_SCHED>(run, P, precision, gains, ywin, summ, traj, st);
    } else if (run.kalman && run.kal_list == 4) {
        // the positions whose schedule did not turn periodic: the quad form
        if (cd == 4) sim_launch<8, 4, SIM_KALMAN_QUAD>(run, P, precision, gains, ywin, summ, traj, st);
        else sim_launch<8, 8, SIM_KALMAN_QUAD>(run, P, precision, gains, ywin, summ, traj, st);
    } else if (run.kalman) {
        if (cd == 4) sim_launch<8, 4, SIM_KALMAN_LANE>(run, P, precision, gains, ywin, summ, traj, st);
        else sim_launch<8, 8, SIM_KALMAN_LANE>(run, P, precision, gains, ywin, summ, traj, st);
    } else if (cs == 4 && cd == 4) sim_launch<4, 4>(run, P, precision, gains, ywin, summ, traj, st);
    else if (cs == 4 && cd == 8) sim_launch<4, 8>(run, P, precision, gains, ywin, summ, traj, st);
    else if (cs == 8 && cd == 4) sim_launch<8, 4>(run, P, precision, gains, ywin, summ, traj, st);
    else sim_launch<8, 8>(run, P, precision, gains, ywin, summ, traj, st);
    CE_CUDA(cudaGetLastError());
}

}  // namespace ce
