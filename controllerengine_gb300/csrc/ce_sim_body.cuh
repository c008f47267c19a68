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
// Kalman observer (KMODE 1 and 2, ref: src/discrete_solves.cu:83-185): the prediction
// xh += (A-I)xh + B u, the covariance P = A P A^T + diag(Q), the gain
// KG = P C^T / (C P C^T + R), the correction xh += KG (y - C xh) in double-float
// and the Joseph update P = (I - KG C) P (I - KG C)^T + KG R KG^T replace the
// Luenberger increment, with the reference's fma chains over the full padded
// width (NSC = 8).  Two of the reference's defects are fixed: its Joseph
// product writes over its own left factor while reading it (:160), here it
// has its own storage; its 1/(C P C^T + R) is the approximate __fdividef
// (:136), here the correctly rounded quotient.  Rows are [K, L, N, R, Q].
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
    // the observer model
    __device__ __forceinline__ float sai(int i, int j) const { return P.ss_ai[i * MAXS + j]; }
    __device__ __forceinline__ float sb(int i) const { return P.ss_b[i]; }
    __device__ __forceinline__ float sc(int i) const { return P.ss_c[i]; }
    __device__ __forceinline__ float sd() const { return P.ss_d; }
};

// ...or, in a ragged batch, the candidate's column of the per-candidate table
// (observer model, plant and instruction program alike), copied once into this
// thread's column of the block's dynamic shared memory (RT_FIELDS x SIM_BLOCK
// words), where every step reads it.
template <int NDC>
struct RagLocal {
    const float* t;
    int s;
    __device__ __forceinline__ RagLocal(const Run& run, const Plant&, int64_t c) : s(SIM_BLOCK) {
        extern __shared__ float rag_cols[];
        const float* __restrict__ g = run.rg.tab + c;
        const int64_t gs = run.rg.tab_stride;
        float* col = rag_cols + threadIdx.x;
        for (int f = 0; f < RT_FIELDS; ++f) col[f * SIM_BLOCK] = g[(int64_t)f * gs];
        t = col;
    }
    __device__ __forceinline__ float f(int field) const { return t[field * s]; }
    __device__ __forceinline__ float ai(int i, int j) const { return f(RT_DAI + i * MAXD + j); }
    __device__ __forceinline__ float bu(int i) const { return f(RT_DBU + i); }
    __device__ __forceinline__ float bw(int i, int k) const { return f(RT_DBW + i * MAXW + k); }
    __device__ __forceinline__ float sai(int i, int j) const { return f(RT_SAI + i * MAXS + j); }
    __device__ __forceinline__ float sb(int i) const { return f(RT_SB + i); }
    __device__ __forceinline__ float sc(int i) const { return f(RT_SC + i); }
    __device__ __forceinline__ float sd() const { return f(RT_SD); }
};

// ...or the candidate's own plant from the per-candidate plant table, loaded
// into registers once per candidate (instruction constants that the program
// never uses are never loaded).
template <int NDC>
struct McLocal {
    float ai_[NDC * NDC], bu_[NDC], bw_[NDC * MAXW], cst_[2 * MC_SLOTS];
    __device__ __forceinline__ McLocal(const Run& run, const Plant& plant, int64_t c) : P(plant) {
        const float* __restrict__ t = run.mc.tab;
        const int64_t np = run.mc.np, p = mc_plant(run.mc, c);
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
    // the observer model is the launch's, shared by all plants
    const Plant& P;
    __device__ __forceinline__ float sai(int i, int j) const { return P.ss_ai[i * MAXS + j]; }
    __device__ __forceinline__ float sb(int i) const { return P.ss_b[i]; }
    __device__ __forceinline__ float sc(int i) const { return P.ss_c[i]; }
    __device__ __forceinline__ float sd() const { return P.ss_d; }
};

// P <- (M P) M^T over the padded 8 x 8 covariance, in place (ABATf, ref:
// src/main.cu:190-212).  Column j of M P needs only column j of P and row i of
// (M P) M^T only row i of M P, so eight temporaries suffice.  Every element is
// the reference's fma chain in k order from 0.
template <class Mat>
__device__ __forceinline__ void abat_in_place(float (&Pm)[MAXS * MAXS], const Mat& M) {
#pragma unroll
    for (int j = 0; j < MAXS; ++j) {
        float col[MAXS];
#pragma unroll
        for (int i = 0; i < MAXS; ++i) {
            float a = 0.0f;
#pragma unroll
            for (int k = 0; k < MAXS; ++k) a = __fmaf_rn(M(i, k), Pm[k * MAXS + j], a);
            col[i] = a;
        }
#pragma unroll
        for (int i = 0; i < MAXS; ++i) Pm[i * MAXS + j] = col[i];
    }
#pragma unroll
    for (int i = 0; i < MAXS; ++i) {
        float r[MAXS];
#pragma unroll
        for (int j = 0; j < MAXS; ++j) {
            float a = 0.0f;
#pragma unroll
            for (int k = 0; k < MAXS; ++k) a = __fmaf_rn(Pm[i * MAXS + k], M(j, k), a);
            r[j] = a;
        }
#pragma unroll
        for (int j = 0; j < MAXS; ++j) Pm[i * MAXS + j] = r[j];
    }
}

// Kalman prediction xh += (A-I) xh + B u, then double-float add (ref: src/discrete_solves.cu:118-126).
__device__ __forceinline__ void kalman_predict(const Plant& P, float (&xh_hi)[MAXS], float (&xh_lo)[MAXS], float u) {
    float dh[MAXS], dl[MAXS];
#pragma unroll
    for (int i = 0; i < MAXS; ++i) {
        float h = __fmul_rn(P.ss_b[i], u), l = 0.0f;
#pragma unroll
        for (int j = 0; j < MAXS; ++j) h = __fmaf_rn(P.ss_ai[i * MAXS + j], xh_hi[j], h);
#pragma unroll
        for (int j = 0; j < MAXS; ++j) l = __fmaf_rn(P.ss_ai[i * MAXS + j], xh_lo[j], l);
        dh[i] = h;
        dl[i] = l;
    }
#pragma unroll
    for (int i = 0; i < MAXS; ++i) df_add(xh_hi[i], xh_lo[i], dh[i], dl[i]);
}

// Kalman correction xh += KG (y - C xh): the residual as a (hi, lo) pair and
// exact products (ref: src/discrete_solves.cu:140-149).
__device__ __forceinline__ void kalman_correct(const Plant& P, float (&xh_hi)[MAXS], float (&xh_lo)[MAXS], float y,
                                               const float (&KG)[MAXS]) {
    float zh = -y, zl = 0.0f;
#pragma unroll
    for (int k = 0; k < MAXS; ++k) zh = __fmaf_rn(P.ss_c[k], xh_hi[k], zh);
#pragma unroll
    for (int k = 0; k < MAXS; ++k) zl = __fmaf_rn(P.ss_c[k], xh_lo[k], zl);
    zh = __fmul_rn(-1.0f, zh);
    zl = __fmul_rn(-1.0f, zl);
#pragma unroll
    for (int i = 0; i < MAXS; ++i) {
        const float s = __fmul_rn(KG[i], zh);
        float e = __fmaf_rn(KG[i], zh, -s);
        e = __fmaf_rn(KG[i], zl, e);
        df_add(xh_hi[i], xh_lo[i], s, e);
    }
}

// -(KG_i C_k - [i == k]): element (i, k) of I - KG C as the reference forms it
// (matmul, diagonal minus one, negation; ref: src/discrete_solves.cu:152-158).
__device__ __forceinline__ float ikh(float kg_i, float c_k, bool diag) {
    float m = __fmaf_rn(kg_i, c_k, 0.0f);
    if (diag) m = __fsub_rn(m, 1.0f);
    return -m;
}

// One candidate's covariance step, all in its own registers (ref:
// src/discrete_solves.cu:128-163): P = A P A^T + diag(Q); KG = P C^T /
// (C P C^T + R); P = (I - KG C) P (I - KG C)^T + KG R KG^T.
__device__ __forceinline__ void kalman_cov_lane(const Plant& P, float (&Pm)[MAXS * MAXS], const float (&Qd)[MAXS],
                                                float Rn, float (&KG)[MAXS]) {
    abat_in_place(Pm, [&](int i, int k) { return P.ss_a[i * MAXS + k]; });
#pragma unroll
    for (int i = 0; i < MAXS; ++i) Pm[i * (MAXS + 1)] = __fadd_rn(Pm[i * (MAXS + 1)], Qd[i]);
    {
        float pht[MAXS], cp[MAXS];
#pragma unroll
        for (int i = 0; i < MAXS; ++i) {
            float a = 0.0f;
#pragma unroll
            for (int k = 0; k < MAXS; ++k) a = __fmaf_rn(Pm[i * MAXS + k], P.ss_c[k], a);
            pht[i] = a;
        }
#pragma unroll
        for (int j = 0; j < MAXS; ++j) {
            float a = 0.0f;
#pragma unroll
            for (int k = 0; k < MAXS; ++k) a = __fmaf_rn(P.ss_c[k], Pm[k * MAXS + j], a);
            cp[j] = a;
        }
        float hphr = 0.0f;
#pragma unroll
        for (int k = 0; k < MAXS; ++k) hphr = __fmaf_rn(cp[k], P.ss_c[k], hphr);
        hphr = __fdiv_rn(1.0f, __fadd_rn(hphr, Rn));
#pragma unroll
        for (int i = 0; i < MAXS; ++i) KG[i] = __fmul_rn(pht[i], hphr);
    }
    float M[MAXS * MAXS];
#pragma unroll
    for (int i = 0; i < MAXS; ++i)
#pragma unroll
        for (int j = 0; j < MAXS; ++j) M[i * MAXS + j] = ikh(KG[i], P.ss_c[j], i == j);
    abat_in_place(Pm, [&](int i, int k) { return M[i * MAXS + k]; });
#pragma unroll
    for (int i = 0; i < MAXS; ++i) {
        const float kr = __fmaf_rn(KG[i], Rn, 0.0f);
#pragma unroll
        for (int j = 0; j < MAXS; ++j) Pm[i * MAXS + j] = __fadd_rn(Pm[i * MAXS + j], __fmaf_rn(kr, KG[j], 0.0f));
    }
}

// The covariance recursion depends only on A, C, Q and R, so candidates with
// the same noise weights share it.  In the shared form a whole warp holds
// such candidates and computes the recursion once, cooperatively: P lives in
// shared memory and lane l forms elements l and l + 32 (rows i0 = l/8 and
// i1 = i0 + 4, column j = l%8) of each product, every element by the same fma
// chain as in the per-candidate form, so the gains are bit-identical.  The
// gains of the last KAL_PERIOD steps are kept in a ring, and every
// KAL_PERIOD steps a snapshot of P is taken.  Once P_{t+1} equals the
// snapshot P_{t0} bit for bit the recursion is periodic with period
// p = t + 1 - t0 (p = 1: a fixed point), every later gain is the one p steps
// earlier, and the recursion stops.
constexpr int KAL_PERIOD = 24;

// Shared memory of one warp in the shared form.
struct KalWarp {
    float P[MAXS * MAXS], T[MAXS * MAXS];
    float A[MAXS * (MAXS + 1)];  // the observer's A, rows padded to 9 (no bank conflicts)
    float kg[KAL_PERIOD][MAXS];  // KG_s of the last KAL_PERIOD steps s, by slot s % KAL_PERIOD
};

struct KalShared {
    float q0, q1, r;  // Q[i0], Q[i1], R
    float snap0, snap1;  // own elements of the snapshot of P
    int t, t_snap;    // steps recursed; step of the snapshot
    int slot;         // ring slot of the current step
    int period;       // 0: recursing; p: the gains repeat with period p
    int rslot;        // periodic: ring slot of the gain p steps back
};

// The gain KG_s of the current step s into KG; advances the recursion while it runs.
__device__ __forceinline__ void kalman_gain_shared(const Plant& P, KalShared& S, KalWarp& W, int lane,
                                                   float (&KG)[MAXS]) {
    constexpr unsigned FULL = 0xffffffffu;
    const int slot = S.slot;
    S.slot = slot + 1 == KAL_PERIOD ? 0 : slot + 1;
    if (S.period) {
        // KG_s = KG_{s-p}; written to this step's slot so the ring stays the last KAL_PERIOD gains
        const int rs = S.rslot;
        S.rslot = rs + 1 == KAL_PERIOD ? 0 : rs + 1;
#pragma unroll
        for (int i = 0; i < MAXS; ++i) KG[i] = W.kg[rs][i];
        const float mine = W.kg[rs][lane & (MAXS - 1)];
        __syncwarp();
        if (lane < MAXS) W.kg[slot][lane] = mine;
        __syncwarp();
        return;
    }
    if (S.t - S.t_snap == KAL_PERIOD || S.t == 0) {
        S.snap0 = W.P[lane];
        S.snap1 = W.P[lane + 32];
        S.t_snap = S.t;
    }
    {
        const int j = lane & (MAXS - 1), i0 = lane >> 3, i1 = i0 + 4;
        constexpr int AS = MAXS + 1;
        // T = A P (column j of P)
        float pc[MAXS];
#pragma unroll
        for (int k = 0; k < MAXS; ++k) pc[k] = W.P[k * MAXS + j];
        float t0 = 0.0f, t1 = 0.0f;
#pragma unroll
        for (int k = 0; k < MAXS; ++k) {
            t0 = __fmaf_rn(W.A[i0 * AS + k], pc[k], t0);
            t1 = __fmaf_rn(W.A[i1 * AS + k], pc[k], t1);
        }
        W.T[lane] = t0;
        W.T[lane + 32] = t1;
        __syncwarp();
        // P = T A^T + diag(Q)
        float u0 = 0.0f, u1 = 0.0f;
#pragma unroll
        for (int k = 0; k < MAXS; ++k) {
            const float a = W.A[j * AS + k];
            u0 = __fmaf_rn(W.T[i0 * MAXS + k], a, u0);
            u1 = __fmaf_rn(W.T[i1 * MAXS + k], a, u1);
        }
        if (i0 == j) u0 = __fadd_rn(u0, S.q0);
        if (i1 == j) u1 = __fadd_rn(u1, S.q1);
        W.P[lane] = u0;
        W.P[lane + 32] = u1;
        __syncwarp();
        // gain: lanes 0-7 form (P C^T)_l, lanes 8-15 (C P)_{l-8}; every lane forms C P C^T + R
        float v = 0.0f;
        if (lane < MAXS) {
#pragma unroll
            for (int k = 0; k < MAXS; ++k) v = __fmaf_rn(W.P[lane * MAXS + k], P.ss_c[k], v);
        } else if (lane < 2 * MAXS) {
#pragma unroll
            for (int k = 0; k < MAXS; ++k) v = __fmaf_rn(P.ss_c[k], W.P[k * MAXS + lane - MAXS], v);
        }
        float h = 0.0f;
#pragma unroll
        for (int k = 0; k < MAXS; ++k) h = __fmaf_rn(__shfl_sync(FULL, v, MAXS + k), P.ss_c[k], h);
        h = __fdiv_rn(1.0f, __fadd_rn(h, S.r));
        const float kgl = __fmul_rn(v, h);
        if (lane < MAXS) W.kg[slot][lane] = kgl;
        const float kgi0 = __shfl_sync(FULL, kgl, i0), kgi1 = __shfl_sync(FULL, kgl, i1);
        const float kgj = __shfl_sync(FULL, kgl, j);
        // T = (I - KG C) P
#pragma unroll
        for (int k = 0; k < MAXS; ++k) pc[k] = W.P[k * MAXS + j];
        float w0 = 0.0f, w1 = 0.0f;
#pragma unroll
        for (int k = 0; k < MAXS; ++k) {
            w0 = __fmaf_rn(ikh(kgi0, P.ss_c[k], k == i0), pc[k], w0);
            w1 = __fmaf_rn(ikh(kgi1, P.ss_c[k], k == i1), pc[k], w1);
        }
        W.T[lane] = w0;
        W.T[lane + 32] = w1;
        __syncwarp();
        // P = T (I - KG C)^T + KG R KG^T
        float z0 = 0.0f, z1 = 0.0f;
#pragma unroll
        for (int k = 0; k < MAXS; ++k) {
            const float m = ikh(kgj, P.ss_c[k], k == j);
            z0 = __fmaf_rn(W.T[i0 * MAXS + k], m, z0);
            z1 = __fmaf_rn(W.T[i1 * MAXS + k], m, z1);
        }
        z0 = __fadd_rn(z0, __fmaf_rn(__fmaf_rn(kgi0, S.r, 0.0f), kgj, 0.0f));
        z1 = __fadd_rn(z1, __fmaf_rn(__fmaf_rn(kgi1, S.r, 0.0f), kgj, 0.0f));
        // P_{t+1} against the snapshot (own elements)
        const bool same = __float_as_uint(z0) == __float_as_uint(S.snap0) &&
                          __float_as_uint(z1) == __float_as_uint(S.snap1);
        // every lane read P for the last time before the barrier above
        W.P[lane] = z0;
        W.P[lane + 32] = z1;
        if (__all_sync(FULL, same)) {
            const int p = S.t + 1 - S.t_snap;  // 1 .. KAL_PERIOD
            S.period = p;
            S.rslot = (slot + 1 - p + KAL_PERIOD) % KAL_PERIOD;
        }
        ++S.t;
        __syncwarp();
    }
#pragma unroll
    for (int i = 0; i < MAXS; ++i) KG[i] = W.kg[slot][i];
}

// Simulation forms: KMODE 0 the Luenberger observer; 1 the Kalman observer
// with each candidate's covariance in its own registers; 2 the Kalman observer
// with the covariance shared by the warp (all 32 lanes hold the same R and Q).
// 3: the Kalman observer with the candidate's gains read from its gain
// schedule (k_kal_schedule), no covariance recursion in the loop; 4: the
// per-candidate covariance split over a quad of lanes (kalman_cov_quad).
constexpr int SIM_LUENBERGER = 0, SIM_KALMAN_LANE = 1, SIM_KALMAN_SHARED = 2, SIM_KALMAN_SCHED = 3,
              SIM_KALMAN_QUAD = 4;

// The quad form: four lanes share a candidate.  Each lane runs the whole
// trajectory (every value the same in the four; lane 0 writes the outputs) and
// owns rows 2q and 2q+1 of every covariance product; P, the rows of P C^T and
// the columns of C P meet in the candidate's slot of shared memory.  Every
// element is formed by one lane with the per-candidate form's fma chain, so
// the gains are bit-identical to it, at a quarter of the dependent chain per
// step -- for the candidates whose recursion never turns periodic, which run
// it for the whole horizon.
struct KalQuadSlot {
    float P[MAXS * MAXS];
    float v[2 * MAXS];  // (P C^T)_i, then (C P)_j
};
struct KalQuadSmem {
    KalQuadSlot s[SIM_BLOCK / SW_LANES];
};
struct KalQuadRef {
    KalQuadSlot& s;
    int q;
    unsigned qm;
};
__device__ __forceinline__ void kalman_cov_quad(const Plant& P, const KalQuadRef& Q, const float (&Qd)[MAXS],
                                                float Rn, float (&KG)[MAXS]) {
    KalQuadSlot& S = Q.s;
    const int i0 = 2 * Q.q;
    float t[2][MAXS], p[2][MAXS];
    // P <- A P A^T + diag(Q), own rows: row i of A P from all of P, then of (A P) A^T
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int j = 0; j < MAXS; ++j) {
            float a = 0.0f;
#pragma unroll
            for (int k = 0; k < MAXS; ++k) a = __fmaf_rn(P.ss_a[(i0 + r) * MAXS + k], S.P[k * MAXS + j], a);
            t[r][j] = a;
        }
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int j = 0; j < MAXS; ++j) {
            float a = 0.0f;
#pragma unroll
            for (int k = 0; k < MAXS; ++k) a = __fmaf_rn(t[r][k], P.ss_a[j * MAXS + k], a);
            p[r][j] = j == i0 + r ? __fadd_rn(a, Qd[i0 + r]) : a;
        }
    __syncwarp(Q.qm);  // every read of the old P is done
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int j = 0; j < MAXS; ++j) S.P[(i0 + r) * MAXS + j] = p[r][j];
    __syncwarp(Q.qm);
    // gain: own rows of P C^T, own columns of C P
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        float a = 0.0f;
#pragma unroll
        for (int k = 0; k < MAXS; ++k) a = __fmaf_rn(p[r][k], P.ss_c[k], a);
        S.v[i0 + r] = a;
        float b = 0.0f;
#pragma unroll
        for (int k = 0; k < MAXS; ++k) b = __fmaf_rn(P.ss_c[k], S.P[k * MAXS + i0 + r], b);
        S.v[MAXS + i0 + r] = b;
    }
    __syncwarp(Q.qm);
    float hphr = 0.0f;
#pragma unroll
    for (int k = 0; k < MAXS; ++k) hphr = __fmaf_rn(S.v[MAXS + k], P.ss_c[k], hphr);
    hphr = __fdiv_rn(1.0f, __fadd_rn(hphr, Rn));
#pragma unroll
    for (int i = 0; i < MAXS; ++i) KG[i] = __fmul_rn(S.v[i], hphr);
    // P <- (I - KG C) P (I - KG C)^T + KG R KG^T, own rows
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int j = 0; j < MAXS; ++j) {
            float a = 0.0f;
#pragma unroll
            for (int k = 0; k < MAXS; ++k) a = __fmaf_rn(ikh(KG[i0 + r], P.ss_c[k], i0 + r == k), S.P[k * MAXS + j], a);
            t[r][j] = a;
        }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const float kr = __fmaf_rn(KG[i0 + r], Rn, 0.0f);
#pragma unroll
        for (int j = 0; j < MAXS; ++j) {
            float a = 0.0f;
#pragma unroll
            for (int k = 0; k < MAXS; ++k) a = __fmaf_rn(t[r][k], ikh(KG[j], P.ss_c[k], j == k), a);
            p[r][j] = __fadd_rn(a, __fmaf_rn(kr, KG[j], 0.0f));
        }
    }
    __syncwarp(Q.qm);  // every read of P and of v is done
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int j = 0; j < MAXS; ++j) S.P[(i0 + r) * MAXS + j] = p[r][j];
    __syncwarp(Q.qm);
}

template <bool Q> struct QuadSmemOf { using type = KalQuadSmem; };
template <> struct QuadSmemOf<false> { struct type {}; };

// The per-candidate list position of the Kalman list `pos` of a scheduled (3)
// or straggler (4) launch, or pos itself for the per-candidate list (2); -1
// past the list's end.
__device__ __forceinline__ int64_t kal_list_position(const Run& run, int64_t pos) {
    if (run.kal_list == 2) return pos < (int64_t)run.kal_totals[1] + run.kal_totals[2] ? pos : -1;
    const int64_t cnt = run.kal_totals[run.kal_list == 3 ? 3 : 4];
    return pos < cnt ? run.kal_lists[(run.kal_list == 3 ? 0 : run.kal_sched_n) + pos] : -1;
}
// The candidate at position lp of the per-candidate list: the list proper, then
// the candidates deferred by the shared form.
__device__ __forceinline__ int64_t kal_list_candidate(const Run& run, int64_t lp) {
    const int64_t np = run.kal_totals[1];
    return lp < np ? run.kal_order[run.kal_totals[0] + lp] : run.kal_order[run.kal_defer + lp - np];
}

// Snapshots of P every KAL_SCHED_SNAP steps in the gain schedules: periods of
// up to this many steps are found.
constexpr int KAL_SCHED_SNAP = 8;

// The gain of step t from a candidate's schedule: KG_t for t below t0 + p, then
// the period [t0, t0 + p) again and again (a running index, no division).  The
// schedule is read in step with the warp's other candidates (one coalesced row
// per gain); the period, which each candidate enters at its own step, is kept
// in the thread's column of shared memory once reached.
struct KalSchedSmem {
    float g[KAL_SCHED_SNAP * MAXS][SIM_BLOCK];
};
struct KalSched {
    const float* g;   // the candidate's column: gain k of schedule step s at g[(s * MAXS + k) * stride]
    int64_t stride;
    int idx, t0, end;  // index of the current step's gain; the period's first step and end
    float* ring;       // the period's gains, gain k of period step s at ring[(s * MAXS + k) * SIM_BLOCK]
    bool cyc;          // the period has been reached (gains from the ring)
    __device__ __forceinline__ void next(float (&KG)[MAXS]) {
        if (cyc) {
#pragma unroll
            for (int k = 0; k < MAXS; ++k) KG[k] = ring[((idx - t0) * MAXS + k) * SIM_BLOCK];
        } else {
#pragma unroll
            for (int k = 0; k < MAXS; ++k) KG[k] = g[((int64_t)idx * MAXS + k) * stride];
        }
        if (++idx == end) {
            if (!cyc) {
                for (int s = t0; s < end; ++s)
#pragma unroll
                    for (int k = 0; k < MAXS; ++k)
                        ring[((s - t0) * MAXS + k) * SIM_BLOCK] = g[((int64_t)s * MAXS + k) * stride];
                cyc = true;
            }
            idx = t0;
        }
    }
};
template <bool S> struct SchedSmemOf { using type = KalSchedSmem; };
template <> struct SchedSmemOf<false> { struct type {}; };

template <int NSC, int NDC, class Chains, int KMODE, bool RG, class Stage, class SrcP, class SrcH, class KW>
__device__ __forceinline__ void sim_candidate(const Run& launch, const Run& run, const Plant& P, int64_t c,
                                              bool writer, const float* __restrict__ gains, float* __restrict__ ywin,
                                              SimSummary* __restrict__ summ, float* __restrict__ traj, Stage& stage,
                                              SrcP& srcP, SrcH& srcH, KW& kw);

// Maps the thread to its candidate (its own index, or an entry of a Kalman
// candidate list) and runs that candidate with its sizes and plant.
template <int NSC, int NDC, class Chains, int KMODE = SIM_LUENBERGER, bool RG = false>
__device__ __forceinline__ void sim_run(const Run& run_in, const Plant& P_in, const float* __restrict__ gains,
                                        float* __restrict__ ywin, SimSummary* __restrict__ summ,
                                        float* __restrict__ traj) {
    const Run& run = run_in;
    constexpr bool KAL = KMODE != SIM_LUENBERGER;
    constexpr bool SHARED = KMODE == SIM_KALMAN_SHARED;
    __shared__ float stage[8][SIM_BLOCK];
    __shared__ float srcP[Chains::kSmem ? MAXD + 1 : 1][SIM_BLOCK];
    __shared__ float srcH[Chains::kSmem ? MAXS : 1][SIM_BLOCK];
    __shared__ KalWarp kw[SHARED ? SIM_BLOCK / 32 : 1];
    __shared__ typename QuadSmemOf<KMODE == SIM_KALMAN_QUAD>::type kq;
    __shared__ typename SchedSmemOf<KMODE == SIM_KALMAN_SCHED>::type ksr;
    const int tid = threadIdx.x;
    // each thread only touches its own column of the shared rows; the quad form
    // gives a candidate to four consecutive threads
    constexpr bool QUAD = KMODE == SIM_KALMAN_QUAD;
    const int64_t pos = ((int64_t)blockIdx.x * SIM_BLOCK + tid) / (QUAD ? SW_LANES : 1);
    int64_t c = pos;
    bool writer = !QUAD || (tid & 3) == 0;
    if constexpr (SHARED) {
        // the shared-noise list: whole warps of one group; a padding slot (-1)
        // shadows the warp's first candidate and writes nothing
        const int64_t wbase = pos & ~(int64_t)31;
        if (wbase >= run.kal_totals[0]) return;  // warp-uniform
        const int own = run.kal_order[pos];
        writer = own >= 0;
        c = writer ? own : run.kal_order[wbase];
    } else if (KAL && run.kal_list >= 2) {
        // the per-candidate list (then the candidates of warps deferred by the
        // shared form), or its scheduled or straggling positions
        const int64_t lp = kal_list_position(run, pos);
        if (lp < 0) return;
        c = kal_list_candidate(run, lp);
        if constexpr (KMODE == SIM_KALMAN_SCHED) {
            const int2 m = run.kal_meta[lp];
            KalSched ks{run.kal_sched + lp, run.kal_sched_n, 0, m.x, m.x + m.y, &ksr.g[0][tid], false};
            return sim_candidate<NSC, NDC, Chains, KMODE, RG>(run_in, run_of<RG>(run_in, c),
                                                               plant_of<RG>(run_in, P_in, c), c, writer, gains, ywin,
                                                               summ, traj, stage, srcP, srcH, ks);
        }
        if constexpr (QUAD) {
            KalQuadRef kr{kq.s[tid >> 2], tid & 3, 0xFu << (tid & 28)};
            return sim_candidate<NSC, NDC, Chains, KMODE, RG>(run_in, run_of<RG>(run_in, c),
                                                               plant_of<RG>(run_in, P_in, c), c, writer, gains, ywin,
                                                               summ, traj, stage, srcP, srcH, kr);
        }
    } else {
        if (c >= run.n) return;
    }
    if constexpr (KMODE == SIM_KALMAN_SCHED || QUAD) {
        return;  // the scheduled and quad forms run only over their lists (kal_list 3, 4)
    } else {
        return sim_candidate<NSC, NDC, Chains, KMODE, RG>(run_in, run_of<RG>(run_in, c),
                                                           plant_of<RG>(run_in, P_in, c), c, writer, gains, ywin,
                                                           summ, traj, stage, srcP, srcH, kw);
    }
}

template <int NSC, int NDC, class Chains, int KMODE, bool RG, class Stage, class SrcP, class SrcH, class KW>
__device__ __forceinline__ void sim_candidate(const Run& launch, const Run& run, const Plant& P, int64_t c,
                                              bool writer, const float* __restrict__ gains, float* __restrict__ ywin,
                                              SimSummary* __restrict__ summ, float* __restrict__ traj, Stage& stage,
                                              SrcP& srcP, SrcH& srcH, KW& kw) {
    constexpr bool KAL = KMODE != SIM_LUENBERGER;
    constexpr bool SHARED = KMODE == SIM_KALMAN_SHARED;
    const int tid = threadIdx.x;
    const typename Chains::template Local<NDC> Lc(launch, P, c);

    const int ns = run.ns;
    const float* row = gains + c * run.cuda_w;
    float K[NSC], L[NSC];
#pragma unroll
    for (int i = 0; i < NSC; ++i) {
        K[i] = i < ns ? row[i] : 0.0f;
        L[i] = i < ns ? row[ns + i] : 0.0f;
    }
    const float N = row[2 * ns];
    static_assert(!KAL || NSC == MAXS, "the Kalman observer runs the full padded width");
    // Kalman: noise weights and covariance (ref: src/discrete_solves.cu:88-101,
    // at the row offsets of [K, L, N, R, Q])
    float Qd[KMODE == SIM_KALMAN_LANE || KMODE == SIM_KALMAN_QUAD ? MAXS : 1],
        Pm[KMODE == SIM_KALMAN_LANE ? MAXS * MAXS : 1];
    float KG[KAL ? MAXS : 1];
    float Rn = 0.0f;
    KalShared S;
    const int lane = tid & 31;
    if constexpr (KMODE == SIM_KALMAN_QUAD) {
        Rn = row[2 * ns + 1];
#pragma unroll
        for (int i = 0; i < MAXS; ++i) Qd[i] = i < ns ? row[2 * ns + 2 + i] : 0.0f;
#pragma unroll
        for (int j = 0; j < 2 * MAXS; ++j) kw.s.P[2 * kw.q * MAXS + j] = 0.0f;  // own rows of P
        __syncwarp(kw.qm);
    }
    if constexpr (KMODE == SIM_KALMAN_LANE) {
        Rn = row[2 * ns + 1];
#pragma unroll
        for (int i = 0; i < MAXS; ++i) Qd[i] = i < ns ? row[2 * ns + 2 + i] : 0.0f;
#pragma unroll
        for (int i = 0; i < MAXS * MAXS; ++i) Pm[i] = 0.0f;
    }
    if constexpr (SHARED) {
        // the warp must hold one set of noise weights bit for bit; if not (two
        // sets in one hash bucket), its candidates go to the per-candidate form
        unsigned eq = 1u, pred;
        Rn = row[2 * ns + 1];
        __match_all_sync(0xffffffffu, __float_as_uint(Rn), (int*)&pred);
        eq &= pred ? 1u : 0u;
        for (int i = 0; i < ns; ++i) {
            __match_all_sync(0xffffffffu, __float_as_uint(row[2 * ns + 2 + i]), (int*)&pred);
            eq &= pred ? 1u : 0u;
        }
        if (!eq) {
            if (writer) run.kal_order[run.kal_defer + atomicAdd(&run.kal_totals[2], 1)] = (int)c;
            return;  // warp-uniform
        }
        const int i0 = lane >> 3, i1 = i0 + 4;
        KalWarp& W = kw[tid >> 5];
        for (int e = lane; e < MAXS * MAXS; e += 32) W.A[(e >> 3) * (MAXS + 1) + (e & 7)] = P.ss_a[e];
        S.q0 = i0 < ns ? row[2 * ns + 2 + i0] : 0.0f;
        S.q1 = i1 < ns ? row[2 * ns + 2 + i1] : 0.0f;
        S.r = Rn;
        S.t = S.t_snap = 0;
        S.slot = S.rslot = 0;
        S.period = 0;
        S.snap0 = S.snap1 = 0.0f;
        W.P[lane] = 0.0f;
        W.P[lane + 32] = 0.0f;
        __syncwarp();
    }

    float xh_hi[NSC], xh_lo[NSC], xp_hi[NDC], xp_lo[NDC];
#pragma unroll
    for (int i = 0; i < NSC; ++i) xh_hi[i] = xh_lo[i] = 0.0f;
#pragma unroll
    for (int i = 0; i < NDC; ++i) xp_hi[i] = xp_lo[i] = 0.0f;
    bool poisS = false, poisD = false;

    float ysum = 0.0f, ycomp = 0.0f, ymax = -CUDART_INF_F, ymin = CUDART_INF_F;
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
                    if (writer) {
                        dst[0] = a;
                        dst[1] = b;
                    }
                }
            }
            if (t >= run.steady_start_id) ysum_add(ysum, ycomp, y);
            ymax = fmaxf(ymax, y);
            ymin = fminf(ymin, y);
            if (run.store_traj && writer) traj[c * (int64_t)T + t] = y;
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

        if constexpr (KAL) {
            kalman_predict(P, xh_hi, xh_lo, u);
            if constexpr (SHARED) {
                kalman_gain_shared(P, S, kw[tid >> 5], lane, KG);
            } else if constexpr (KMODE == SIM_KALMAN_SCHED) {
                kw.next(KG);
            } else if constexpr (KMODE == SIM_KALMAN_QUAD) {
                kalman_cov_quad(P, kw, Qd, Rn, KG);
            } else {
                kalman_cov_lane(P, Pm, Qd, Rn, KG);
            }
            kalman_correct(P, xh_hi, xh_lo, y, KG);
        } else {
            // observer output error
            float yh = 0.0f;
#pragma unroll
            for (int i = 0; i < NSC; ++i) yh = __fmaf_rn(Lc.sc(i), xh_hi[i], yh);
            if (NSC < MAXS) yh = __fadd_rn(yh, padS);
#pragma unroll
            for (int i = 0; i < NSC; ++i) yh = __fmaf_rn(Lc.sc(i), xh_lo[i], yh);
            if (NSC < MAXS) yh = __fadd_rn(yh, padS);
            yh = __fmaf_rn(Lc.sd(), u, yh);
            const float yerr = __fsub_rn(y, yh);

            // observer increment (A-I)xh + B u + L yerr, then double-float add
            float dh[NSC], dl[NSC];
#pragma unroll
            for (int i = 0; i < NSC; ++i) {
                float h = __fmaf_rn(L[i], yerr, __fmul_rn(Lc.sb(i), u));
                float l = 0.0f;
#pragma unroll
                for (int j = 0; j < NSC; ++j) h = __fmaf_rn(Lc.sai(i, j), xh_hi[j], h);
#pragma unroll
                for (int j = 0; j < NSC; ++j) l = __fmaf_rn(Lc.sai(i, j), xh_lo[j], l);
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
        }

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
    sm.ycomp = ycomp;
    if (writer) summ[c] = sm;
}

// ---- the wide form of a session's simulation --------------------------------
// One thread per candidate runs its horizon as one chain of dependent steps;
// a batch too small to fill the GPU (a served request, a small tuning batch)
// leaves that latency exposed.  Here four lanes (a quad) share a candidate,
// sixteen candidates per block.  Lane q holds rows q*RS.. of the observer
// update and q*RD.. of the plant update, with their matrix rows in registers;
// every lane forms the step's scalars itself -- y and u (the compiled DC and U
// programs), K.xh, C.xh, the NL terms -- from the same state in the same
// order, so every value is formed by one lane with the operations and order of
// sim_candidate and the rows are bit-identical to it.  The quad exchanges its
// new state rows through a double-buffered slot in shared memory, one quad
// barrier per step.  Luenberger observer, compiled programs, one plant for
// all candidates.
// slot: xh_hi, xh_lo (MAXS each), xp_hi, xp_lo (MAXD each); a stride of 36 words
// keeps rows 16-byte aligned and the 16-byte loads of a warp's eight candidates
// on disjoint banks
constexpr int SW_XH_HI = 0, SW_XH_LO = MAXS, SW_XP_HI = 2 * MAXS, SW_XP_LO = 2 * MAXS + MAXD, SW_STRIDE = 36;

template <int NSC, int NDC, class Chains>
__device__ __forceinline__ void sim_wide(const Run& run, const Plant& P, const float* __restrict__ gains,
                                         float* __restrict__ ywin, SimSummary* __restrict__ summ,
                                         float* __restrict__ traj) {
    static_assert(!Chains::kSmem, "the wide form runs compiled programs");
    static_assert(NSC % SW_LANES == 0 && NDC % SW_LANES == 0, "the rows split evenly over the quad");
    constexpr int RS = NSC / SW_LANES, RD = NDC / SW_LANES;
    __shared__ __align__(16) float slots[2][SW_CPB * SW_STRIDE];
    __shared__ float stage[8][SW_CPB];
    const int q = threadIdx.x & 3, cl = threadIdx.x >> 2;
    const unsigned qm = 0xFu << (threadIdx.x & 28);
    const int64_t c = (int64_t)blockIdx.x * SW_CPB + cl;
    if (c >= run.n) return;  // the whole quad leaves together
    const typename Chains::template Local<NDC> Lc(run, P, c);
    const int ns = run.ns;
    const float* row = gains + c * run.cuda_w;
    float K[NSC], sc[NSC], Lr[RS], sb[RS], sai[RS][NSC], dbu[RD], dai[RD][NDC], dbw[RD][MAXW];
#pragma unroll
    for (int i = 0; i < NSC; ++i) {
        K[i] = i < ns ? row[i] : 0.0f;
        sc[i] = Lc.sc(i);
    }
#pragma unroll
    for (int rr = 0; rr < RS; ++rr) {
        const int i = q * RS + rr;
        Lr[rr] = i < ns ? row[ns + i] : 0.0f;
        sb[rr] = Lc.sb(i);
#pragma unroll
        for (int j = 0; j < NSC; ++j) sai[rr][j] = Lc.sai(i, j);
    }
#pragma unroll
    for (int rr = 0; rr < RD; ++rr) {
        const int i = q * RD + rr;
        dbu[rr] = Lc.bu(i);
#pragma unroll
        for (int k = 0; k < MAXW; ++k) dbw[rr][k] = Lc.bw(i, k);
#pragma unroll
        for (int j = 0; j < NDC; ++j) dai[rr][j] = Lc.ai(i, j);
    }
    const float N = row[2 * ns], sd = Lc.sd();
    {
        float* s0 = slots[0] + cl * SW_STRIDE;
#pragma unroll
        for (int rr = 0; rr < RS; ++rr) s0[SW_XH_HI + q * RS + rr] = s0[SW_XH_LO + q * RS + rr] = 0.0f;
#pragma unroll
        for (int rr = 0; rr < RD; ++rr) s0[SW_XP_HI + q * RD + rr] = s0[SW_XP_LO + q * RD + rr] = 0.0f;
    }
    __syncwarp(qm);
    float xh_hi[NSC], xh_lo[NSC], xp_hi[NDC], xp_lo[NDC];
#pragma unroll
    for (int i = 0; i < NSC; ++i) xh_hi[i] = xh_lo[i] = 0.0f;
#pragma unroll
    for (int i = 0; i < NDC; ++i) xp_hi[i] = xp_lo[i] = 0.0f;
    bool poisS = false, poisD = false;
    float ysum = 0.0f, ycomp = 0.0f, ymax = -CUDART_INF_F, ymin = CUDART_INF_F;
    float* wrow = ywin + c * (int64_t)run.fit_pitch;
    const int T = run.time;
    for (int t = 0; t < T; ++t) {
        const float* cur = slots[t & 1] + cl * SW_STRIDE;
        float* nxt = slots[(t + 1) & 1] + cl * SW_STRIDE;
        const float padS = poisS ? CUDART_NAN_F : 0.0f;
        const float padD = poisD ? CUDART_NAN_F : 0.0f;
        // plant output
        const float y = Chains::dc(P, Lc, xp_hi, nullptr);
        if (q == 0) {
            // fit window, steady-state sum, extremes, optional full trajectory
            const int w = t - run.fit_start_id;
            if (w >= 0 && w < run.fit_steps) {
                stage[w & 7][cl] = y;
                if ((w & 7) == 7 || w == run.fit_steps - 1 || t == T - 1) {
                    float4 a, b;
                    a.x = stage[0][cl]; a.y = stage[1][cl]; a.z = stage[2][cl]; a.w = stage[3][cl];
                    b.x = stage[4][cl]; b.y = stage[5][cl]; b.z = stage[6][cl]; b.w = stage[7][cl];
                    float4* dst = reinterpret_cast<float4*>(wrow + (w & ~7));
                    dst[0] = a;
                    dst[1] = b;
                }
            }
            if (t >= run.steady_start_id) ysum_add(ysum, ycomp, y);
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
        const float u = Chains::u(P, Lc, xh_hi, nullptr, u_raw);
        // observer output error
        float yh = 0.0f;
#pragma unroll
        for (int i = 0; i < NSC; ++i) yh = __fmaf_rn(sc[i], xh_hi[i], yh);
        if (NSC < MAXS) yh = __fadd_rn(yh, padS);
#pragma unroll
        for (int i = 0; i < NSC; ++i) yh = __fmaf_rn(sc[i], xh_lo[i], yh);
        if (NSC < MAXS) yh = __fadd_rn(yh, padS);
        yh = __fmaf_rn(sd, u, yh);
        const float yerr = __fsub_rn(y, yh);
        // this lane's observer rows: increment, then double-float add on the
        // row's old value (read from the slot: an index by lane would put the
        // state arrays in local memory)
        float nh[RS], nlo[RS];
#pragma unroll
        for (int rr = 0; rr < RS; ++rr) {
            float h = __fmaf_rn(Lr[rr], yerr, __fmul_rn(sb[rr], u));
            float l = 0.0f;
#pragma unroll
            for (int j = 0; j < NSC; ++j) h = __fmaf_rn(sai[rr][j], xh_hi[j], h);
#pragma unroll
            for (int j = 0; j < NSC; ++j) l = __fmaf_rn(sai[rr][j], xh_lo[j], l);
            if (NSC < MAXS) {
                h = __fadd_rn(h, padS);
                l = __fadd_rn(l, padS);
            }
            nh[rr] = cur[SW_XH_HI + q * RS + rr];
            nlo[rr] = cur[SW_XH_LO + q * RS + rr];
            df_add(nh[rr], nlo[rr], h, l);
        }
        if (NSC < MAXS) {
            bool bad = !isfinite(yerr) || !isfinite(u);
#pragma unroll
            for (int j = 0; j < NSC; ++j) bad = bad || !isfinite(xh_hi[j]) || !isfinite(xh_lo[j]);
            poisS = poisS || bad;
        }
        // nonlinear terms over [xp_hi, y]
        float W[MAXW];
        Chains::nl(P, Lc, xp_hi, y, nullptr, W);
        // this lane's plant rows
        float ph[RD], plo[RD];
#pragma unroll
        for (int rr = 0; rr < RD; ++rr) {
            float h = __fmul_rn(dbu[rr], u);
#pragma unroll
            for (int k = 0; k < MAXW; ++k) h = __fmaf_rn(dbw[rr][k], W[k], h);
            float l = 0.0f;
#pragma unroll
            for (int j = 0; j < NDC; ++j) h = __fmaf_rn(dai[rr][j], xp_hi[j], h);
#pragma unroll
            for (int j = 0; j < NDC; ++j) l = __fmaf_rn(dai[rr][j], xp_lo[j], l);
            if (NDC < MAXD) {
                h = __fadd_rn(h, padD);
                l = __fadd_rn(l, padD);
            }
            ph[rr] = cur[SW_XP_HI + q * RD + rr];
            plo[rr] = cur[SW_XP_LO + q * RD + rr];
            df_add(ph[rr], plo[rr], h, l);
        }
        if (NDC < MAXD) {
            bool bad = !isfinite(u);
#pragma unroll
            for (int k = 0; k < MAXW; ++k) bad = bad || !isfinite(W[k]);
#pragma unroll
            for (int j = 0; j < NDC; ++j) bad = bad || !isfinite(xp_hi[j]) || !isfinite(xp_lo[j]);
            poisD = poisD || bad;
        }
        // publish this lane's rows into the other buffer, then read the new state
#pragma unroll
        for (int rr = 0; rr < RS; ++rr) {
            nxt[SW_XH_HI + q * RS + rr] = nh[rr];
            nxt[SW_XH_LO + q * RS + rr] = nlo[rr];
        }
#pragma unroll
        for (int rr = 0; rr < RD; ++rr) {
            nxt[SW_XP_HI + q * RD + rr] = ph[rr];
            nxt[SW_XP_LO + q * RD + rr] = plo[rr];
        }
        __syncwarp(qm);
#pragma unroll
        for (int i = 0; i < NSC; i += 4) {
            const float4 a = *reinterpret_cast<const float4*>(nxt + SW_XH_HI + i);
            const float4 b = *reinterpret_cast<const float4*>(nxt + SW_XH_LO + i);
            xh_hi[i] = a.x; xh_hi[i + 1] = a.y; xh_hi[i + 2] = a.z; xh_hi[i + 3] = a.w;
            xh_lo[i] = b.x; xh_lo[i + 1] = b.y; xh_lo[i + 2] = b.z; xh_lo[i + 3] = b.w;
        }
#pragma unroll
        for (int i = 0; i < NDC; i += 4) {
            const float4 a = *reinterpret_cast<const float4*>(nxt + SW_XP_HI + i);
            const float4 b = *reinterpret_cast<const float4*>(nxt + SW_XP_LO + i);
            xp_hi[i] = a.x; xp_hi[i + 1] = a.y; xp_hi[i + 2] = a.z; xp_hi[i + 3] = a.w;
            xp_lo[i] = b.x; xp_lo[i + 1] = b.y; xp_lo[i + 2] = b.z; xp_lo[i + 3] = b.w;
        }
    }
    if (q == 0) {
        SimSummary sm;
        sm.ysum = ysum;
        sm.ymax = ymax;
        sm.ymin = ymin;
        sm.ycomp = ycomp;
        summ[c] = sm;
    }
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

// A ragged batch: each candidate's own instruction program, read from its
// column of the per-candidate table (the interpreter of run_chain_sm, with the
// instruction fields unpacked from the table words).  Source column k is
// src[k * SS].
template <bool HAS_SEED, int MAXC, int SS = SIM_BLOCK>
__device__ __forceinline__ float run_chain_tab(const float* t, int s, int slot0, int n, const float* src,
                                               float seed) {
    float result = 0.0f;
#pragma unroll
    for (int r = 0; r < MAXC; ++r) {
        if (r >= n) break;
        const int f = RT_INS + 3 * (slot0 + r);
        const unsigned code = __float_as_uint(t[f * s]);
        const int op = (int)(code & 0xFFu), col = (int)((code >> 8) & 0xFFu);
        const int ak = (int)((code >> 16) & 0xFFu), bk = (int)(code >> 24);
        const float pos = src[col * SS];
        float prev;
        if (r == 0) prev = (HAS_SEED && !isnan(seed)) ? seed : pos;
        else prev = result;
        const float a = ak == CE_OPERAND_CONST ? t[(f + 1) * s] : (ak == CE_OPERAND_STATE ? pos : prev);
        const float b = bk == CE_OPERAND_CONST ? t[(f + 2) * s] : (bk == CE_OPERAND_STATE ? pos : prev);
        switch (op) {
            case 1: result = radd(a, b); break;
            case 2: result = rsub(a, b); break;
            case 3: result = rmul(a, b); break;
            case 4: result = rdiv(a, b); break;
            case 5: result = fmin(fmax(prev, a), b); break;
            case 6: result = (float)((0.0f < a) - (a < 0.0f)); break;
            default: break;
        }
    }
    return result;
}

struct RagChains {
    static constexpr bool kSmem = true;
    template <int NDC>
    using Local = RagLocal<NDC>;
    template <int NDC>
    __device__ static __forceinline__ float dc(const Plant&, const RagLocal<NDC>& L, const float (&)[NDC],
                                               const float* sp) {
        const unsigned cnt = __float_as_uint(L.f(RT_CNT));
        return run_chain_tab<false, MAX_DC>(L.t, L.s, 0, (int)(cnt & 0xFFu), sp, 0.0f);
    }
    template <int NSC, int NDC>
    __device__ static __forceinline__ float u(const Plant&, const RagLocal<NDC>& L, const float (&)[NSC],
                                              const float* sh, float seed) {
        const unsigned cnt = __float_as_uint(L.f(RT_CNT));
        return run_chain_tab<true, MAX_U>(L.t, L.s, MAX_DC, (int)((cnt >> 8) & 0xFFu), sh, seed);
    }
    template <int NDC>
    __device__ static __forceinline__ void nl(const Plant&, const RagLocal<NDC>& L, const float (&)[NDC], float,
                                              const float* sp, float (&W)[MAXW]) {
        const unsigned c0 = __float_as_uint(L.f(RT_CNT)), c1 = __float_as_uint(L.f(RT_CNT + 1));
        const int n[MAXW] = {(int)((c0 >> 16) & 0xFFu), (int)(c0 >> 24), (int)(c1 & 0xFFu), (int)((c1 >> 8) & 0xFFu)};
#pragma unroll
        for (int k = 0; k < MAXW; ++k)
            W[k] = run_chain_tab<false, MAX_NL>(L.t, L.s, MAX_DC + MAX_U + k * MAX_NL, n[k], sp, 0.0f);
    }
};

}  // namespace ce
