// ce_sim_body.cuh -- the simulation step loop, shared by the table-driven
// kernel (ce_k_sim.cu) and the kernels specialised at run time to one plant's
// instruction program (ce_jit.cpp compiles this header with NVRTC).
//
// Restates discrete_solve<Luenberger> (ref: src/discrete_solves.cu:12-79):
// per step t
//   y      = DC(xp_hi)                                   plant output chain
//   u      = U(xh_hi, seed = N*ref[t] - K.(xh_hi,xh_lo)) controller output chain
//   yhat   = C.(xh_hi,xh_lo) + D*u
//   xh    += (A-I)xh + B*u + L*(y - yhat)                double-float add
//   W      = NL_k([xp_hi, y]), k < 4                     nonlinear terms
//   xp    += (Ad-I)xp + Bu*u + Bw*W                      double-float add
// with the reference's operation order and roundings, so trajectories are
// bit-identical to the reference kernel's.
//
// One thread per candidate with all state in registers; the plant comes from
// the launch's constant bank.  Only the fit window is stored, staged 8 samples
// at a time in shared memory and written as two 16-byte vectors per lane (one
// full 32-byte sector per lane); yss and the overshoot extremes are reduced in
// registers.
//
// Padding: the reference always loops to the MAX dims (8/8/4) with zero
// padding.  Here loops run to NSC/NDC >= the actual dims (padding inside is
// real, zero-filled state).  The padding between NSC/NDC and 8 is virtual: a
// zero-coefficient term adds +0 (which turns a -0 accumulator into +0) or, once
// the padded state has become NaN, NaN.  `padS`/`padD` hold that value, and the
// poison flags reproduce when the reference's padded states turn NaN (a zero
// coefficient times a non-finite operand).
//
// Chains policy: Chains::kSmem says whether the chains read their sources from
// the per-thread shared-memory rows srcP (plant states, y in row MAXD) and srcH
// (observer states); dc / u / nl evaluate the DC, U and NL_k chains;
// Chains::Local<NDC> supplies the candidate's plant values (BankLocal: the
// launch's Plant; McLocal: the candidate's row of the per-candidate plant table).
#pragma once
#include "ce_device.cuh"

namespace ce {

// The plant values of one candidate: the launch's Plant (the constant bank)...
template <int NDC>
struct BankLocal {
    const Plant& P;
    __device__ __forceinline__ BankLocal(const Run&, const Plant& p, int64_t) : P(p) {}
    __device__ __forceinline__ float ai(int i, int j) const { return P.d_ai[i * MAXD + j]; }
    __device__ __forceinline__ float bu(int i) const { return P.d_bu[i]; }
    __device__ __forceinline__ float bw(int i, int k) const { return P.d_bw[i * MAXW + k]; }
};

// ...or the candidate's own plant from the per-candidate plant table, loaded
// into registers once per candidate (instruction constants that the program
// never uses are never loaded).
template <int NDC>
struct McLocal {
    float ai_[NDC * NDC], bu_[NDC], bw_[NDC * MAXW], cst_[2 * MC_SLOTS];
    __device__ __forceinline__ McLocal(const Run& run, const Plant&, int64_t c) {
        const float* __restrict__ t = run.mc.tab;
        const int64_t np = run.mc.np, p = run.mc.first + c;
#pragma unroll
        for (int i = 0; i < NDC; ++i) {
#pragma unroll
            for (int j = 0; j < NDC; ++j) ai_[i * NDC + j] = t[(int64_t)(MC_AI + i * MAXD + j) * np + p];
            bu_[i] = t[(int64_t)(MC_BU + i) * np + p];
#pragma unroll
            for (int k = 0; k < MAXW; ++k) bw_[i * MAXW + k] = t[(int64_t)(MC_BW + i * MAXW + k) * np + p];
        }
#pragma unroll
        for (int k = 0; k < 2 * MC_SLOTS; ++k) cst_[k] = t[(int64_t)(MC_CST + k) * np + p];
    }
    __device__ __forceinline__ float ai(int i, int j) const { return ai_[i * NDC + j]; }
    __device__ __forceinline__ float bu(int i) const { return bu_[i]; }
    __device__ __forceinline__ float bw(int i, int k) const { return bw_[i * MAXW + k]; }
    __device__ __forceinline__ float c(int k) const { return cst_[k]; }
};

template <int NSC, int NDC, class Chains>
__device__ __forceinline__ void sim_run(const Run& run, const Plant& P, const float* __restrict__ gains,
                                        float* __restrict__ ywin, SimSummary* __restrict__ summ,
                                        float* __restrict__ traj) {
    __shared__ float stage[8][SIM_BLOCK];
    __shared__ float srcP[Chains::kSmem ? MAXD + 1 : 1][SIM_BLOCK];
    __shared__ float srcH[Chains::kSmem ? MAXS : 1][SIM_BLOCK];
    const int tid = threadIdx.x;
    const int64_t c = (int64_t)blockIdx.x * SIM_BLOCK + tid;
    if (c >= run.n) return;  // each thread only touches its own column of the shared rows
    const typename Chains::template Local<NDC> Lc(run, P, c);

    const int ns = run.ns;
    const float* row = gains + c * run.cuda_w;
    float K[NSC], L[NSC];
#pragma unroll
    for (int i = 0; i < NSC; ++i) {
        K[i] = i < ns ? row[i] : 0.0f;
        L[i] = i < ns ? row[ns + i] : 0.0f;
    }
    const float N = row[2 * ns];

    float xh_hi[NSC], xh_lo[NSC], xp_hi[NDC], xp_lo[NDC];
#pragma unroll
    for (int i = 0; i < NSC; ++i) xh_hi[i] = xh_lo[i] = 0.0f;
#pragma unroll
    for (int i = 0; i < NDC; ++i) xp_hi[i] = xp_lo[i] = 0.0f;
    bool poisS = false, poisD = false;

    float ysum = 0.0f, ymax = -CUDART_INF_F, ymin = CUDART_INF_F;
    float* wrow = ywin + c * (int64_t)run.fit_pitch;
    const int T = run.time;

    for (int t = 0; t < T; ++t) {
        const float padS = poisS ? CUDART_NAN_F : 0.0f;
        const float padD = poisD ? CUDART_NAN_F : 0.0f;

        if constexpr (Chains::kSmem) {
#pragma unroll
            for (int i = 0; i < NDC; ++i) srcP[i][tid] = xp_hi[i];
#pragma unroll
            for (int i = 0; i < NSC; ++i) srcH[i][tid] = xh_hi[i];
        }

        // plant output
        const float y = Chains::dc(P, Lc, xp_hi, &srcP[0][tid]);
        if constexpr (Chains::kSmem) srcP[Chains::kSmem ? MAXD : 0][tid] = y;

        // outputs: fit window, steady-state sum, extremes, optional full trajectory
        {
            const int w = t - run.fit_start_id;
            if (w >= 0 && w < run.fit_steps) {
                stage[w & 7][tid] = y;
                if ((w & 7) == 7 || w == run.fit_steps - 1 || t == T - 1) {
                    float4 a, b;
                    a.x = stage[0][tid]; a.y = stage[1][tid]; a.z = stage[2][tid]; a.w = stage[3][tid];
                    b.x = stage[4][tid]; b.y = stage[5][tid]; b.z = stage[6][tid]; b.w = stage[7][tid];
                    float4* dst = reinterpret_cast<float4*>(wrow + (w & ~7));
                    dst[0] = a;
                    dst[1] = b;
                }
            }
            if (t >= run.steady_start_id) ysum = __fadd_rn(ysum, y);
            ymax = fmaxf(ymax, y);
            ymin = fminf(ymin, y);
            if (run.store_traj) traj[c * (int64_t)T + t] = y;
        }

        // controller output
        float kx = 0.0f;
#pragma unroll
        for (int i = 0; i < NSC; ++i) kx = __fmaf_rn(K[i], xh_hi[i], kx);
        if (NSC < MAXS) kx = __fadd_rn(kx, padS);
#pragma unroll
        for (int i = 0; i < NSC; ++i) kx = __fmaf_rn(K[i], xh_lo[i], kx);
        if (NSC < MAXS) kx = __fadd_rn(kx, padS);
        const float ref = t < run.ref_step_id ? 0.0f : run.ref_amp;
        const float u_raw = __fmaf_rn(N, ref, -kx);
        const float u = Chains::u(P, Lc, xh_hi, &srcH[0][tid], u_raw);

        // observer output error
        float yh = 0.0f;
#pragma unroll
        for (int i = 0; i < NSC; ++i) yh = __fmaf_rn(P.ss_c[i], xh_hi[i], yh);
        if (NSC < MAXS) yh = __fadd_rn(yh, padS);
#pragma unroll
        for (int i = 0; i < NSC; ++i) yh = __fmaf_rn(P.ss_c[i], xh_lo[i], yh);
        if (NSC < MAXS) yh = __fadd_rn(yh, padS);
        yh = __fmaf_rn(P.ss_d, u, yh);
        const float yerr = __fsub_rn(y, yh);

        // observer increment (A-I)xh + B u + L yerr, then double-float add
        float dh[NSC], dl[NSC];
#pragma unroll
        for (int i = 0; i < NSC; ++i) {
            float h = __fmaf_rn(L[i], yerr, __fmul_rn(P.ss_b[i], u));
            float l = 0.0f;
#pragma unroll
            for (int j = 0; j < NSC; ++j) h = __fmaf_rn(P.ss_ai[i * MAXS + j], xh_hi[j], h);
#pragma unroll
            for (int j = 0; j < NSC; ++j) l = __fmaf_rn(P.ss_ai[i * MAXS + j], xh_lo[j], l);
            if (NSC < MAXS) {
                h = __fadd_rn(h, padS);
                l = __fadd_rn(l, padS);
            }
            dh[i] = h;
            dl[i] = l;
        }
        if (NSC < MAXS) {
            bool bad = !isfinite(yerr) || !isfinite(u);
#pragma unroll
            for (int j = 0; j < NSC; ++j) bad = bad || !isfinite(xh_hi[j]) || !isfinite(xh_lo[j]);
            poisS = poisS || bad;
        }
#pragma unroll
        for (int i = 0; i < NSC; ++i) df_add(xh_hi[i], xh_lo[i], dh[i], dl[i]);

        // nonlinear terms over [xp_hi, y]
        float W[MAXW];
        Chains::nl(P, Lc, xp_hi, y, &srcP[0][tid], W);

        // plant increment (Ad-I)xp + Bu u + Bw W, then double-float add
        float ph[NDC], pl[NDC];
#pragma unroll
        for (int i = 0; i < NDC; ++i) {
            float h = __fmul_rn(Lc.bu(i), u);
#pragma unroll
            for (int k = 0; k < MAXW; ++k) h = __fmaf_rn(Lc.bw(i, k), W[k], h);
            float l = 0.0f;
#pragma unroll
            for (int j = 0; j < NDC; ++j) h = __fmaf_rn(Lc.ai(i, j), xp_hi[j], h);
#pragma unroll
            for (int j = 0; j < NDC; ++j) l = __fmaf_rn(Lc.ai(i, j), xp_lo[j], l);
            if (NDC < MAXD) {
                h = __fadd_rn(h, padD);
                l = __fadd_rn(l, padD);
            }
            ph[i] = h;
            pl[i] = l;
        }
        if (NDC < MAXD) {
            bool bad = !isfinite(u);
#pragma unroll
            for (int k = 0; k < MAXW; ++k) bad = bad || !isfinite(W[k]);
#pragma unroll
            for (int j = 0; j < NDC; ++j) bad = bad || !isfinite(xp_hi[j]) || !isfinite(xp_lo[j]);
            poisD = poisD || bad;
        }
#pragma unroll
        for (int i = 0; i < NDC; ++i) df_add(xp_hi[i], xp_lo[i], ph[i], pl[i]);
    }

    SimSummary sm;
    sm.ysum = ysum;
    sm.ymax = ymax;
    sm.ymin = ymin;
    sm.pad = 0.0f;
    summ[c] = sm;
}

// The instruction tables of the plant, interpreted (any program, no compile step).
struct TableChains {
    static constexpr bool kSmem = true;
    template <int NDC>
    using Local = BankLocal<NDC>;
    template <int NDC, class Lc>
    __device__ static __forceinline__ float dc(const Plant& P, const Lc&, const float (&)[NDC], const float* sp) {
        return run_chain_sm<float, MAX_DC, false>(P.dc, P.n_dc, sp, SIM_BLOCK, 0.0f);
    }
    template <int NSC, class Lc>
    __device__ static __forceinline__ float u(const Plant& P, const Lc&, const float (&)[NSC], const float* sh,
                                              float seed) {
        return run_chain_sm<float, MAX_U, true>(P.u, P.n_u, sh, SIM_BLOCK, seed);
    }
    template <int NDC, class Lc>
    __device__ static __forceinline__ void nl(const Plant& P, const Lc&, const float (&)[NDC], float, const float* sp,
                                              float (&W)[MAXW]) {
#pragma unroll
        for (int k = 0; k < MAXW; ++k) W[k] = run_chain_sm<float, MAX_NL, false>(P.nl[k], P.n_nl[k], sp, SIM_BLOCK, 0.0f);
    }
};

}  // namespace ce
