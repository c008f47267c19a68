// ce_k_modal.cu -- modal fit of the step response and the behaviour score.
//
// k_fit restates modalsetup (ref: src/modalsetup.cu:1-97): eigenvalues -> s
// plane, instability flag, dedupe of consecutive eigenvalues, yss, overshoot,
// and the normal equations AtA/Atb of the least-squares fit of
// y - yss to e^{sigma t - shift} cos/sin(omega t) over the fit window, with the
// reference's float roundings (the same expf/cosf/sinf arguments, the same
// fused multiply-adds, the same sequential order in t), so AtA/Atb equal the
// reference kernel's.
//
// GB300 layout: the reference keeps the 32x32 AtA in a per-thread local array
// (4.6 KB stack, ref: src/modalsetup.cu:67).  Here 16 lanes own one candidate
// and work through the window in chunks of 8 steps: first the chunk's
// 8 x unique basis pairs (one expf + one sin/cos pair each) are spread evenly
// over the lanes and written to shared memory, then every lane accumulates its
// 4x4 tiles of the lower triangle over the 8 steps with two 16-byte shared
// loads and 16 fused multiply-adds per tile and step.  The fit window is read
// as 32 contiguous bytes per chunk.  The small chunk keeps the shared-memory
// footprint (1.2 KB per candidate) low enough for the FP64 eigensolves that
// run alongside on the same SMs.

// k_modal restates modalsolve (ref: src/modalsolve.cu:1-108): diagonal
// scaling, LDLT with symmetric pivoting of the 2nt x 2nt system, per-mode
// energies, energy-weighted wn/zeta of the oscillatory modes and the behaviour
// error.  One warp per candidate, lane i owning row i of the factorisation.
#include <cfloat>

#include "ce_device.cuh"
#include "ce_host.h"

namespace ce {

constexpr float TINY_E6 = 0x1.0c6f7ap-20f;   // ~1e-6, the reference's threshold constant
constexpr float SENT = 0x1.2a05f2p+33f;      // 1e10 sentinel of the dedupe scan
constexpr float LOGFLOOR = 0x1.a484cp-100f;  // ~1e-30 floor of |lambda| before the log
constexpr float PI_F = 0x1.921fb6p+1f;

__device__ __forceinline__ float rexp(float x) { return expf(x); }
__device__ __forceinline__ double rexp(double x) { return exp(x); }
__device__ __forceinline__ float rcos(float x) { return cosf(x); }
__device__ __forceinline__ double rcos(double x) { return cos(x); }
__device__ __forceinline__ float rsin(float x) { return sinf(x); }
__device__ __forceinline__ double rsin(double x) { return sin(x); }
__device__ __forceinline__ void rsincos(float x, float& s, float& c) { sincosf(x, &s, &c); }
__device__ __forceinline__ void rsincos(double x, double& s, double& c) { sincos(x, &s, &c); }
__device__ __forceinline__ float rlog(float x) { return logf(x); }
__device__ __forceinline__ double rlog(double x) { return log(x); }
__device__ __forceinline__ float rsqrt_(float x) { return sqrtf(x); }
__device__ __forceinline__ double rsqrt_(double x) { return sqrt(x); }
__device__ __forceinline__ float rhypot(float a, float b) { return hypotf(a, b); }
__device__ __forceinline__ double rhypot(double a, double b) { return hypot(a, b); }
__device__ __forceinline__ float ratan2(float a, float b) { return atan2f(a, b); }
__device__ __forceinline__ double ratan2(double a, double b) { return atan2(a, b); }

// Modes of one candidate from its eigenvalues (ref: src/modalsetup.cu:8-50,
// src/modalsolve.cu:114-148).  Every lane computes the same values.
template <typename R>
struct Modes {
    R Re[MAXT], Im[MAXT];
    bool dup[MAXT];
    R max_mag;
    int unique;
};

template <typename R>
__device__ __forceinline__ void load_modes(const R* eig, int nt, R ts, Modes<R>& m) {
    m.max_mag = R(0);
#pragma unroll
    for (int i = 0; i < MAXT; ++i) {
        m.Re[i] = R(0);
        m.Im[i] = R(0);
        m.dup[i] = false;
        if (i < nt) {
            const R re = eig[2 * i], im = eig[2 * i + 1];
            const R mag = rhypot(re, im);
            m.max_mag = fmax(m.max_mag, mag);
            m.Re[i] = rdiv(rlog(fmax(mag, R(LOGFLOOR))), ts);
            m.Im[i] = rdiv(ratan2(im, re), ts);
        }
    }
    R pre = R(SENT), pim = R(SENT);
    int unique = nt;
#pragma unroll
    for (int i = 0; i < MAXT; ++i) {
        if (i < nt) {
            if (fabs(rsub(m.Re[i], pre)) < R(TINY_E6) && fabs(rsub(fabs(m.Im[i]), fabs(pim))) < R(TINY_E6)) {
                m.dup[i] = true;
                unique--;
            }
            pre = m.Re[i];
            pim = m.Im[i];
        }
    }
    m.unique = unique;
}

// sigma and |omega| of unique mode number `e`.
template <typename R>
__device__ __forceinline__ void mode_of(const Modes<R>& m, int nt, int e, R& sigma, R& omega) {
    sigma = R(0);
    omega = R(0);
    int slot = 0;
#pragma unroll
    for (int i = 0; i < MAXT; ++i) {
        if (i < nt && !m.dup[i]) {
            if (slot == e) {
                sigma = m.Re[i];
                omega = fabs(m.Im[i]);
            }
            slot++;
        }
    }
}

constexpr int FIT_BLOCK = 128;            // 8 candidates per block
constexpr int FIT_CPB = FIT_BLOCK / 16;
constexpr int FIT_CHUNK = 8;              // window steps per chunk (shared memory: 1.2 KB per candidate)
constexpr int FIT_PITCH = 36;             // basis row: nc values, y at index nc, zeros up to 4*ceil((nc+1)/4)
constexpr int FIT_ROUNDS = 2;             // 4x4 tiles per lane and pass (32 tiles: nc <= 27 in one pass)
constexpr int FIT_CLASSES = MAXT + 1;     // 0: modal-unstable, u = 1..MAXT: stable with u unique modes

// four consecutive basis values (16-byte aligned) from shared memory
__device__ __forceinline__ void ld4(const float* p, float (&v)[4]) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&v)[4]) {
    const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

// Fit classes: the work of a candidate's fit is set by its unique-mode count,
// and a modal-unstable candidate only writes its penalty.  Candidates are
// bucketed by class (counts[cls], order[cls * n + slot]) so that the two
// candidates sharing a warp in k_fit run the same loop trip counts.  The slot
// order inside a class is whatever the atomics give; every candidate's result
// is computed by one half-warp alone, so it does not depend on that order.
template <typename R, bool RG = false>
__global__ void __launch_bounds__(128) k_fit_classify(const Run run_in, const R* __restrict__ eig,
                                                      int* __restrict__ counts, int* __restrict__ order) {
    const int64_t c = (int64_t)blockIdx.x * 128 + threadIdx.x;
    if (c >= run_in.n) return;
    const Run& run = run_of<RG>(run_in, c);
    Modes<R> m;
    load_modes<R>(eig + c * (int64_t)run.eig_slot, run.nt, R(run.ts), m);
    const int cls = m.max_mag > R(1) ? 0 : m.unique;
    const int slot = atomicAdd(&counts[cls], 1);
    order[(int64_t)cls * run_in.n + slot] = (int)c;
}

// Candidate of half-warp h: classes in order of decreasing work (MAXT unique
// modes first, the unstable class last), identity order without a class table.
__device__ __forceinline__ int64_t fit_candidate(const Run& run, const int* counts, const int* order, int64_t h) {
    if (!counts) return h;
    int64_t start = 0;
    for (int cls = MAXT; cls >= 0; --cls) {
        const int k = counts[cls];
        if (h < start + k) return order[(int64_t)cls * run.n + (h - start)];
        start += k;
    }
    return run.n;
}

// CH window steps per chunk: each chunk spreads the basis of its steps over the
// lanes, then accumulates them step by step, so every entry still takes one
// fused multiply-add per step in the order of t whatever CH is.  Large batches
// use 8 (small shared-memory footprint beside the FP64 eigensolves); a batch
// too small to fill the GPU uses 32, which pays the chunk's basis latency and
// barriers once per 32 steps of its latency-bound loop.
template <typename R, typename Sum, bool RG = false, int CH = FIT_CHUNK>
__global__ void __launch_bounds__(FIT_BLOCK) k_fit(const Run run_in, const R* __restrict__ eig, const R* __restrict__ ywin,
                                                   const Sum* __restrict__ summ, R* __restrict__ ata,
                                                   R* __restrict__ atb, float* __restrict__ info,
                                                   const int* __restrict__ counts, const int* __restrict__ order) {
    __shared__ __align__(16) R cb[FIT_CPB][CH][FIT_PITCH];
    __shared__ __align__(16) R mp[FIT_CPB][MAXT][4];
    const int lane = threadIdx.x & 15;
    const int g = threadIdx.x >> 4;
    const unsigned hmask = 0xFFFFu << (threadIdx.x & 16);
    const int64_t h = (int64_t)blockIdx.x * FIT_CPB + g;
    if (h >= run_in.n) return;  // the whole half-warp leaves together
    const int64_t c = fit_candidate(run_in, counts, order, h);
    if (c >= run_in.n) return;
    const Run& run = run_of<RG>(run_in, c);
    const int nt = run.nt;
    const R ts = R(run.ts);

    Modes<R> m;
    load_modes<R>(eig + c * (int64_t)run.eig_slot, nt, ts, m);
    float* out = info + c * (int64_t)run.info_w;
    const int n2 = 2 * nt;
    R* arow = ata + c * (int64_t)run.ata_slot;
    R* brow = atb + c * (int64_t)run.atb_slot;
    // AtA is 2nt x 2nt with row stride 2nt; entries outside j <= i < nc stay
    // zero, as after the reference's memset (ref: src/main.cu:520-521)
    for (int e = lane; e < n2 * n2; e += 16) arow[e] = R(0);
    for (int e = lane; e < n2; e += 16) brow[e] = R(0);
    if (m.max_mag > R(1)) {
        if (lane == 0) {
            const float v = (float)radd(R(run.unstable_err), rdiv(rlog(m.max_mag), ts));
            out[run.info_scoring] = v;
            out[run.info_scoring + 1] = v;
        }
        return;
    }
    const int unique = m.unique, nc = 2 * unique;
    {
        R sig, om;
        mode_of<R>(m, nt, lane, sig, om);
        mp[g][lane][0] = sig;
        mp[g][lane][1] = om;
        mp[g][lane][2] = fmax(rmul(sig, R(run.fit_t0)), rmul(sig, R(run.fit_t1)));
        mp[g][lane][3] = R(0);
    }

    // steady-state value and overshoot (ref: src/modalsetup.cu:52-62); the
    // running max of y*yss equals max(y)*yss (yss >= 0) or min(y)*yss (yss < 0)
    // because rounding is monotone; NaN samples are ignored either way.
    R ysum, ymax, ymin;
    if constexpr (sizeof(R) == 4) {
        ysum = summ[c].ysum; ymax = summ[c].ymax; ymin = summ[c].ymin;
    } else {
        ysum = summ[4 * c]; ymax = summ[4 * c + 1]; ymin = summ[4 * c + 2];
    }
    const R yss = rdiv(ysum, R(run.time - run.steady_start_id));
    if (lane == 0) {
        const R pk = fmax(R(0), yss >= R(0) ? rmul(ymax, yss) : rmul(ymin, yss));
        out[run.info_freqresp + 2] = (float)rsub(rdiv(pk, fmax(rmul(yss, yss), R(TINY_E6))), R(1));
        out[run.info_freqresp + 3] = (float)yss;
    }

    // Normal equations (ref: src/modalsetup.cu:64-94).  The basis vector of a
    // step is extended by the sample y at index nc, so AtA (j <= i < nc) and
    // Atb (row nc) are the lower triangle of one rank-1 accumulation of size
    // N = nc + 1, tiled into 4x4 blocks spread over the 16 lanes.  Each entry
    // is still one fused multiply-add per step in the order of t.
    for (int e = lane; e < CH * FIT_PITCH; e += 16) (&cb[g][0][0])[e] = R(0);
    const int N = nc + 1, NB = (N + 3) >> 2, nblk = NB * (NB + 1) / 2;
    // basis work item k = (step k / unique, mode k % unique) of a chunk; lane l
    // takes k = l, l + 16, ... < CH * unique
    const int s0 = lane / unique, m0 = lane - s0 * unique;
    const int ds = 16 / unique, dm = 16 - ds * unique;
    const int items = CH * unique;
    const R* wrow = ywin + c * (int64_t)run.fit_pitch;
    const int wlimit = run.time - run.fit_start_id;  // window samples past the horizon read as 0
    const int steps = run.fit_steps;
    __syncwarp(hmask);
    // one pass over the window per 32 tiles (a second pass only when nc > 27)
    for (int t0 = 0; t0 < nblk; t0 += 16 * FIT_ROUNDS) {
        int bi[FIT_ROUNDS], bj[FIT_ROUNDS];
#pragma unroll
        for (int r = 0; r < FIT_ROUNDS; ++r) {
            const int blk = t0 + lane + 16 * r;
            int i = 0;
            while ((i + 1) * (i + 2) / 2 <= blk) ++i;
            bi[r] = 4 * i;
            bj[r] = 4 * (blk - i * (i + 1) / 2);
        }
        const bool act0 = t0 + lane < nblk, act1 = t0 + lane + 16 < nblk;
        const bool any1 = t0 + 16 < nblk;  // the same in every lane of the half-warp
        R acc[FIT_ROUNDS][16];
#pragma unroll
        for (int r = 0; r < FIT_ROUNDS; ++r)
#pragma unroll
            for (int k = 0; k < 16; ++k) acc[r][k] = R(0);
        // the window samples of a chunk are loaded one chunk ahead, so that their
        // global-memory latency passes under the previous chunk's work
        constexpr int YL = (CH + 15) / 16;  // samples per lane and chunk
        auto window = [&](int w0, R (&y)[YL]) {
#pragma unroll
            for (int u = 0; u < YL; ++u) {
                const int k = lane + 16 * u, idx = w0 + k;
                y[u] = (k < CH && idx < steps && idx < wlimit) ? wrow[idx] : R(0);
            }
        };
        R ynext[YL];
        window(0, ynext);
        for (int w0 = 0; w0 < steps; w0 += CH) {
#pragma unroll
            for (int u = 0; u < YL; ++u) {
                const int k = lane + 16 * u;
                if (k < CH) cb[g][k][nc] = rsub(ynext[u], yss);
            }
            window(w0 + CH, ynext);
            int s = s0, md = m0;
            for (int k = lane; k < items; k += 16) {
                const int w = w0 + s;
                if (w < steps) {
                    const R sig = mp[g][md][0], om = mp[g][md][1], shift = mp[g][md][2];
                    const R tval = rmul(R(run.fit_start_id + w), ts);
                    const R decay = rexp(rfma(sig, tval, -shift));
                    R sn, cs;
                    rsincos(rmul(om, tval), sn, cs);  // one argument reduction for both
                    cb[g][s][2 * md] = rmul(decay, cs);
                    cb[g][s][2 * md + 1] = rmul(decay, sn);
                }
                s += ds;
                md += dm;
                if (md >= unique) {
                    md -= unique;
                    ++s;
                }
            }
            __syncwarp(hmask);
            const int cnt = min(CH, steps - w0);
            for (int st = 0; st < cnt; ++st) {
                const R* row = &cb[g][st][0];
                if (act0) {
                    R a[4], b[4];
                    ld4(row + bi[0], a);
                    ld4(row + bj[0], b);
#pragma unroll
                    for (int p = 0; p < 4; ++p)
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc[0][4 * p + q] = rfma(a[p], b[q], acc[0][4 * p + q]);
                }
                if (any1 && act1) {
                    R a[4], b[4];
                    ld4(row + bi[1], a);
                    ld4(row + bj[1], b);
#pragma unroll
                    for (int p = 0; p < 4; ++p)
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc[1][4 * p + q] = rfma(a[p], b[q], acc[1][4 * p + q]);
                }
            }
            __syncwarp(hmask);
        }
        // owners write their entries over the zeros
#pragma unroll
        for (int r = 0; r < FIT_ROUNDS; ++r) {
            if (t0 + lane + 16 * r < nblk) {
#pragma unroll
                for (int p = 0; p < 4; ++p)
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int i = bi[r] + p, j = bj[r] + q;
                        if (j < nc && j <= i) {
                            if (i < nc) arow[i * n2 + j] = acc[r][4 * p + q];
                            else if (i == nc) brow[j] = acc[r][4 * p + q];
                        }
                    }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// The modal setup of the compensated precision (CE_PRECISION_COMPENSATED).
//
// Same quantities as k_fit -- yss, overshoot, AtA and Atb of the fit of
// y - yss to e^{sigma t - shift} (cos, sin)(omega t) over the window -- from
// the FP32 trajectory, with the modes from the FP64 eigenvalues (never cast
// to float), and with no unstructured rounding in the normal equations:
//  * yss from the compensated steady-state sum (ysum + ycomp) in double;
//  * AtA in closed form.  Every entry is a sum over the window of a product
//    of two basis functions, i.e. of e^{(s_m + s_k) t} or e^{(conj(s_m) + s_k) t}
//    (s = sigma + i omega), and such a sum is geometric:
//      sum_{w<n} e^{s (t0 + w ts)} = e^{s t0} expm1(n s ts) / expm1(s ts),
//    evaluated in FP64 with complex expm1 so that ratios near 1 lose nothing;
//  * Atb = sum_w b(t_w) (y_w - yss) = sum_w b(t_w) y_w - yss sum_w b(t_w): the
//    second sum geometric as above, the first a projection of the trajectory
//    onto e^{s t}, accumulated by a complex recurrence z <- z e^{s ts} in
//    double-float arithmetic on the FP32 pipe (two floats per real; products
//    exact by FMA, sums by TwoSum), the accumulator as a TwoSum high part with
//    a float low part collecting every error term; z is re-anchored from an
//    FP64 exp / sincos every FC_ANCHOR steps, so its drift stays below
//    FC_ANCHOR x 2^-47 relative.
// AtA and the projection agree with the exact values of the same basis to
// ~1e-14 relative, so the solve sees no rounding of the normal equations that
// its conditioning could amplify; what remains is the FP32 trajectory itself.
//
// Layout: 16 lanes per candidate (the k_fit layout and its class order).  A
// mode's projection is split into 16 / unique contiguous window segments, one
// lane each, combined in segment order; the Gram pairs are spread over the
// lanes.

// double-float number h + l on the FP32 pipe
struct dff {
    float h, l;
};
__device__ __forceinline__ dff dff_of(double x) {
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(__dsub_rn(x, (double)h))};
}
__device__ __forceinline__ dff dff_norm(float a, float b) {  // TwoSum renormalisation of a + b
    float s, e;
    df_two_sum(a, b, s, e);
    return {s, e};
}
__device__ __forceinline__ dff dff_mul(dff a, dff b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return dff_norm(p, e);
}
__device__ __forceinline__ dff dff_add(dff a, dff b) {
    float s, e;
    df_two_sum(a.h, b.h, s, e);
    return dff_norm(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dff dff_neg(dff a) { return {-a.h, -a.l}; }
struct cdff {
    dff re, im;
};
__device__ __forceinline__ cdff cdff_mul(cdff a, cdff b) {
    return {dff_add(dff_mul(a.re, b.re), dff_neg(dff_mul(a.im, b.im))),
            dff_add(dff_mul(a.re, b.im), dff_mul(a.im, b.re))};
}
// sum of y * z (y a float, z double-float): TwoSum high part, every error
// term into the float low part
struct acc2 {
    float h, l;
};
__device__ __forceinline__ void acc2_add(acc2& s, float y, dff z) {
    const float p = __fmul_rn(y, z.h);
    float e = __fmaf_rn(y, z.h, -p);
    e = __fmaf_rn(y, z.l, e);
    float t, err;
    df_two_sum(s.h, p, t, err);
    s.h = t;
    s.l = __fadd_rn(s.l, __fadd_rn(err, e));
}

// complex e^z - 1, accurate near 0: (expm1(x) cos y - 2 sin^2(y/2), e^x sin y)
__device__ __forceinline__ cplx<double> cexpm1_(double x, double y) {
    double sy, cy, sh, ch;
    sincos(y, &sy, &cy);
    sincos(0.5 * y, &sh, &ch);
    const double em = expm1(x);
    return {__dsub_rn(__dmul_rn(em, cy), __dmul_rn(2.0, __dmul_rn(sh, sh))), __dmul_rn(exp(x), sy)};
}

// sum_{w<n} e^{(x + i y) (t0 + w ts) - sh}
__device__ __forceinline__ cplx<double> geo_sum(double x, double y, double t0, double ts, int n, double sh) {
    double sy, cy;
    sincos(__dmul_rn(y, t0), &sy, &cy);
    const double a = exp(__fma_rn(x, t0, -sh));
    const cplx<double> first{__dmul_rn(a, cy), __dmul_rn(a, sy)};
    if (x == 0.0 && y == 0.0) return {__dmul_rn(first.re, (double)n), __dmul_rn(first.im, (double)n)};
    const cplx<double> num = cexpm1_(__dmul_rn((double)n, __dmul_rn(x, ts)), __dmul_rn((double)n, __dmul_rn(y, ts)));
    const cplx<double> den = cexpm1_(__dmul_rn(x, ts), __dmul_rn(y, ts));
    return cmul(first, cdiv(num, den));
}

constexpr int FC_ANCHOR = 256;  // window steps between FP64 re-anchorings of the projection recurrence

// YT: the trajectory's type -- float (the FP32 simulation), or double (the
// FP64 simulation of CE_PRECISION_COMPENSATED_TRAJ64 or the double-float one of
// CE_PRECISION_COMPENSATED_DF: each sample split into two floats, hi + lo,
// both projected).
template <typename YT>
__global__ void __launch_bounds__(FIT_BLOCK) k_fit_comp(const Run run, const double* __restrict__ eig,
                                                       const YT* __restrict__ ywin, const void* __restrict__ summ,
                                                       double* __restrict__ ata, double* __restrict__ atb,
                                                       float* __restrict__ info, const int* __restrict__ counts,
                                                       const int* __restrict__ order) {
    __shared__ float part[FIT_CPB][16][4];
    __shared__ double ms[FIT_CPB][MAXT][3];  // per unique mode: sigma, |omega|, shift
    const int lane = threadIdx.x & 15;
    const int g = threadIdx.x >> 4;
    const unsigned hmask = 0xFFFFu << (threadIdx.x & 16);
    const int64_t h = (int64_t)blockIdx.x * FIT_CPB + g;
    if (h >= run.n) return;
    const int64_t c = fit_candidate(run, counts, order, h);
    if (c >= run.n) return;
    const int nt = run.nt, n2 = 2 * nt;
    const double ts = (double)run.ts;
    Modes<double> m;
    load_modes<double>(eig + c * (int64_t)run.eig_slot, nt, ts, m);
    float* out = info + c * (int64_t)run.info_w;
    double* arow = ata + c * (int64_t)run.ata_slot;
    double* brow = atb + c * (int64_t)run.atb_slot;
    for (int e = lane; e < n2 * n2; e += 16) arow[e] = 0.0;
    for (int e = lane; e < n2; e += 16) brow[e] = 0.0;
    if (m.max_mag > 1.0) {
        if (lane == 0) {
            const float v = (float)__dadd_rn((double)run.unstable_err, __ddiv_rn(log(m.max_mag), ts));
            out[run.info_scoring] = v;
            out[run.info_scoring + 1] = v;
        }
        return;
    }
    const int unique = m.unique, nc = 2 * unique;
    {
        double sig, om;
        mode_of<double>(m, nt, lane, sig, om);
        ms[g][lane][0] = sig;
        ms[g][lane][1] = om;
        ms[g][lane][2] = fmax(__dmul_rn(sig, (double)run.fit_t0), __dmul_rn(sig, (double)run.fit_t1));
    }
    // steady state from the compensated sum (the plain sum alone where the
    // compensation is not finite, i.e. the trajectory overflowed); the FP64
    // simulation's summary is (sum, max, min, 0) in double
    double ysum, ymax, ymin;
    if constexpr (sizeof(YT) == 4) {
        const SimSummary sm = static_cast<const SimSummary*>(summ)[c];
        ysum = isfinite(sm.ycomp) ? __dadd_rn((double)sm.ysum, (double)sm.ycomp) : (double)sm.ysum;
        ymax = sm.ymax;
        ymin = sm.ymin;
    } else {
        const double* sd = static_cast<const double*>(summ) + 4 * c;
        ysum = sd[0];
        ymax = sd[1];
        ymin = sd[2];
    }
    const double yss = __ddiv_rn(ysum, (double)(run.time - run.steady_start_id));
    if (lane == 0) {
        const double pk = fmax(0.0, yss >= 0.0 ? __dmul_rn(ymax, yss) : __dmul_rn(ymin, yss));
        out[run.info_freqresp + 2] = (float)__dsub_rn(__ddiv_rn(pk, fmax(__dmul_rn(yss, yss), (double)TINY_E6)), 1.0);
        out[run.info_freqresp + 3] = (float)yss;
    }
    __syncwarp(hmask);
    const int steps = run.fit_steps;
    const double t0 = __dmul_rn((double)run.fit_start_id, ts);

    // projection of the trajectory: mode md, window segment sg of nseg
    const int nseg = unique > 0 ? 16 / unique : 1;
    const int md = lane / nseg, sg = lane - md * nseg;
    acc2 gre{0.0f, 0.0f}, gim{0.0f, 0.0f};
    if (md < unique) {
        const double sig = ms[g][md][0], om = ms[g][md][1], sh = ms[g][md][2];
        double rs, rc;
        sincos(__dmul_rn(om, ts), &rs, &rc);
        const double ra = exp(__dmul_rn(sig, ts));
        const cdff rho{dff_of(__dmul_rn(ra, rc)), dff_of(__dmul_rn(ra, rs))};
        const int seg = (((steps + nseg - 1) / nseg) + 7) & ~7;
        const int wb = sg * seg, we = min(steps, wb + seg);
        const int wlimit = run.time - run.fit_start_id;  // window samples past the horizon read as 0
        const YT* wrow = ywin + c * (int64_t)run.fit_pitch;
        for (int w0 = wb; w0 < we; w0 += FC_ANCHOR) {
            const double tw = __dmul_rn((double)(run.fit_start_id + w0), ts);
            double zs, zc;
            sincos(__dmul_rn(om, tw), &zs, &zc);
            const double za = exp(__fma_rn(sig, tw, -sh));
            cdff z{dff_of(__dmul_rn(za, zc)), dff_of(__dmul_rn(za, zs))};
            const int w1 = min(we, w0 + FC_ANCHOR);
            for (int w = w0; w < w1; w += 4) {
                YT yv[4];
                if constexpr (sizeof(YT) == 4) {
                    const float4 y4 = *reinterpret_cast<const float4*>(wrow + w);  // w is a multiple of 4
                    yv[0] = y4.x; yv[1] = y4.y; yv[2] = y4.z; yv[3] = y4.w;
                } else {
                    const double2 a = reinterpret_cast<const double2*>(wrow + w)[0];
                    const double2 b = reinterpret_cast<const double2*>(wrow + w)[1];
                    yv[0] = a.x; yv[1] = a.y; yv[2] = b.x; yv[3] = b.y;
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (w + k < w1) {
                        const YT y = (w + k < wlimit) ? yv[k] : YT(0);
                        if constexpr (sizeof(YT) == 4) {
                            acc2_add(gre, y, z.re);
                            acc2_add(gim, y, z.im);
                        } else {
                            const dff ys = dff_of(y);
                            acc2_add(gre, ys.h, z.re);
                            acc2_add(gim, ys.h, z.im);
                            acc2_add(gre, ys.l, z.re);
                            acc2_add(gim, ys.l, z.im);
                        }
                        z = cdff_mul(z, rho);
                    }
                }
            }
        }
    }
    part[g][lane][0] = gre.h;
    part[g][lane][1] = gre.l;
    part[g][lane][2] = gim.h;
    part[g][lane][3] = gim.l;
    __syncwarp(hmask);
    if (lane < unique) {
        double pre = 0.0, pim = 0.0;
        for (int k = 0; k < nseg; ++k) {
            const float* q = part[g][lane * nseg + k];
            pre = __dadd_rn(pre, __dadd_rn((double)q[0], (double)q[1]));
            pim = __dadd_rn(pim, __dadd_rn((double)q[2], (double)q[3]));
        }
        const double sig = ms[g][lane][0], om = ms[g][lane][1], sh = ms[g][lane][2];
        const cplx<double> bs = geo_sum(sig, om, t0, ts, steps, sh);  // sum of the basis over the window
        brow[2 * lane] = __dsub_rn(pre, __dmul_rn(yss, bs.re));
        brow[2 * lane + 1] = __dsub_rn(pim, __dmul_rn(yss, bs.im));
    }
    // the Gram matrix: pair (a, b), a >= b, of unique modes
    const int npairs = unique * (unique + 1) / 2;
    for (int pidx = lane; pidx < npairs; pidx += 16) {
        int a = 0;
        while ((a + 1) * (a + 2) / 2 <= pidx) ++a;
        const int b = pidx - a * (a + 1) / 2;
        const double sa = ms[g][a][0], oa = ms[g][a][1], sha = ms[g][a][2];
        const double sb = ms[g][b][0], ob = ms[g][b][1], shb = ms[g][b][2];
        const double x = __dadd_rn(sa, sb), sh = __dadd_rn(sha, shb);
        // A = sum e^{(s_a + s_b) t}, B = sum e^{(conj(s_a) + s_b) t}
        const cplx<double> A = geo_sum(x, __dadd_rn(oa, ob), t0, ts, steps, sh);
        const cplx<double> B = geo_sum(x, __dsub_rn(ob, oa), t0, ts, steps, sh);
        // Re a Re b, Im a Im b, Re a Im b, Im a Re b (a, b the two modes' e^{s t})
        const double cc = __dmul_rn(0.5, __dadd_rn(A.re, B.re));
        const double ss = __dmul_rn(0.5, __dsub_rn(B.re, A.re));
        const double cs = __dmul_rn(0.5, __dadd_rn(A.im, B.im));
        const double sc = __dmul_rn(0.5, __dsub_rn(A.im, B.im));
        arow[(2 * a) * n2 + 2 * b] = cc;
        arow[(2 * a + 1) * n2 + 2 * b] = sc;
        arow[(2 * a + 1) * n2 + 2 * b + 1] = ss;
        if (a != b) arow[(2 * a) * n2 + 2 * b + 1] = cs;
    }
    (void)nc;
}

void launch_fit_comp(const Run& run, bool traj64, const void* eig, const void* ywin, const void* summ, void* ata,
                     void* atb, float* info, int* counts, int* order, cudaStream_t st) {
    const int grid = (int)((run.n + FIT_CPB - 1) / FIT_CPB);
    if (counts) {
        CE_CUDA(cudaMemsetAsync(counts, 0, FIT_CLASSES * sizeof(int), st));
        prefer_shared((const void*)k_fit_classify<double>);
        k_fit_classify<double><<<(int)((run.n + 127) / 128), 128, 0, st>>>(run, (const double*)eig, counts, order);
        CE_CUDA(cudaGetLastError());
    }
    if (traj64) {
        prefer_shared((const void*)k_fit_comp<double>);
        k_fit_comp<double><<<grid, FIT_BLOCK, 0, st>>>(run, (const double*)eig, (const double*)ywin, summ,
                                                       (double*)ata, (double*)atb, info, counts, order);
    } else {
        prefer_shared((const void*)k_fit_comp<float>);
        k_fit_comp<float><<<grid, FIT_BLOCK, 0, st>>>(run, (const double*)eig, (const float*)ywin, summ,
                                                      (double*)ata, (double*)atb, info, counts, order);
    }
    CE_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
constexpr int MODAL_WARPS = 4;

template <typename R>
__device__ __forceinline__ R rmin_normal();
template <>
__device__ __forceinline__ float rmin_normal<float>() { return FLT_MIN; }
template <>
__device__ __forceinline__ double rmin_normal<double>() { return DBL_MIN; }

// REFINE (the compensated precision): after the solve, one step of iterative
// refinement in FP64 -- the residual of the scaled system from the unfactored
// normal equations, solved with the same factors and added to the solution.
template <typename R, bool RG = false, bool REFINE = false>
__global__ void __launch_bounds__(32 * MODAL_WARPS) k_modal(const Run run_in, const R* __restrict__ eig,
                                                            const R* __restrict__ ata, const R* __restrict__ atb,
                                                            float* __restrict__ info) {
    __shared__ R Ms[MODAL_WARPS][MAXNC][MAXNC + 1];
    __shared__ R xs[MODAL_WARPS][MAXNC];
    __shared__ R rs[MODAL_WARPS][REFINE ? MAXNC : 1];
    __shared__ R cs[MODAL_WARPS][MAXNC];
    __shared__ int trans[MODAL_WARPS][MAXNC];
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const int64_t c = (int64_t)blockIdx.x * MODAL_WARPS + wi;
    if (c >= run_in.n) return;  // whole warp
    const Run& run = run_of<RG>(run_in, c);
    float* out = info + c * (int64_t)run.info_w;
    float* sc = out + run.info_scoring;
    float* fr = out + run.info_freqresp;
    float* md = out + run.info_modal;
    if (sc[0] != 0.0f) return;  // pre-flagged or unstable (ref: src/modalsolve.cu:112)
    const int nt = run.nt, n = 2 * nt;
    const R ts = R(run.ts);
    Modes<R> m;
    load_modes<R>(eig + c * (int64_t)run.eig_slot, nt, ts, m);
    if (m.max_mag > R(1)) {
        if (lane == 0) {
            const float v = (float)radd(R(run.unstable_err), rdiv(rlog(m.max_mag), ts));
            sc[0] = v;
            sc[1] = v;
        }
        return;
    }
    R (*M)[MAXNC + 1] = Ms[wi];
    const R* A = ata + c * (int64_t)run.ata_slot;
    // full symmetric copy of the lower triangle, then D^-1 A D^-1 with
    // D = diag(sqrt(a_ii) or 1) (ref: src/modalsolve.cu:154-162)
    if (lane < n)
        for (int j = 0; j < n; ++j) M[lane][j] = j <= lane ? A[lane * n + j] : A[j * n + lane];
    __syncwarp();
    if (lane < n) {
        const R s = rsqrt_(M[lane][lane]);
        cs[wi][lane] = s > R(TINY_E6) ? s : R(1);
    }
    __syncwarp();
    if (lane < n) {
        const R inv_i = rdiv(R(1), cs[wi][lane]);
        for (int j = 0; j < n; ++j) M[lane][j] = rmul(rmul(inv_i, M[lane][j]), rdiv(R(1), cs[wi][j]));
        xs[wi][lane] = rdiv(atb[c * (int64_t)run.atb_slot + lane], cs[wi][lane]);
    }
    __syncwarp();

    // LDLT with symmetric pivoting, left-looking, lower triangle
    // (Eigen's LDLT<Lower> algorithm: pivot = largest remaining |diagonal|)
    bool stop = false;
    for (int k = 0; k < n && !stop; ++k) {
        // pivot: first index of the largest |M(i,i)|, i >= k (a NaN never wins
        // unless it sits at k, like a sequential `if (v > best)` scan)
        R v = (lane >= k && lane < n) ? fabs(M[lane][lane]) : -rnan<R>();
        if (lane == k && isnan(v)) v = CUDART_INF;
        if (isnan(v)) v = -CUDART_INF;
        int idx = (lane >= k && lane < n) ? lane : 1 << 20;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const R ov = __shfl_down_sync(0xffffffffu, v, off);
            const int oi = __shfl_down_sync(0xffffffffu, idx, off);
            if (ov > v || (ov == v && oi < idx)) {
                v = ov;
                idx = oi;
            }
        }
        const int p = __shfl_sync(0xffffffffu, idx, 0);
        if (lane == 0) trans[wi][k] = p;
        if (p != k) {
            if (lane < k) {
                const R t = M[k][lane];
                M[k][lane] = M[p][lane];
                M[p][lane] = t;
            }
            if (lane > p && lane < n) {
                const R t = M[lane][k];
                M[lane][k] = M[lane][p];
                M[lane][p] = t;
            }
            if (lane > k && lane < p) {
                const R t = M[lane][k];
                M[lane][k] = M[p][lane];
                M[p][lane] = t;
            }
            __syncwarp();
            if (lane == 0) {
                const R t = M[k][k];
                M[k][k] = M[p][p];
                M[p][p] = t;
            }
        }
        __syncwarp();
        if (k > 0) {
            // temp_j = d_j * l_kj; a_kk -= sum_j l_kj temp_j; a_ik -= sum_j l_ij temp_j
            R tk = R(0);
            if (lane == k) {
                R acc = R(0);
                for (int j = 0; j < k; ++j) acc = radd(acc, rmul(M[k][j], rmul(M[j][j], M[k][j])));
                tk = acc;
            }
            R ti = R(0);
            const bool below = lane > k && lane < n;
            if (below) {
                R acc = R(0);
                for (int j = 0; j < k; ++j) acc = radd(acc, rmul(M[lane][j], rmul(M[j][j], M[k][j])));
                ti = acc;
            }
            __syncwarp();
            if (lane == k) M[k][k] = rsub(M[k][k], tk);
            if (below) M[lane][k] = rsub(M[lane][k], ti);
            __syncwarp();
        }
        const R akk = M[k][k];
        const bool valid = fabs(akk) > R(0);
        if (k == 0 && !valid) {
            if (lane < n) trans[wi][lane] = lane;
            stop = true;  // all-zero diagonal: nothing left to factor, the solve yields 0
        } else if (valid && lane > k && lane < n) {
            M[lane][k] = rdiv(M[lane][k], akk);
        }
        __syncwarp();
    }

    // solve: P, L, D^+, L^T, P^T, in place on v
    auto solve = [&](R* v) {
        if (lane == 0)
            for (int k = 0; k < n; ++k) {
                const int p = trans[wi][k];
                const R t = v[k];
                v[k] = v[p];
                v[p] = t;
            }
        __syncwarp();
        for (int i = 0; i < n; ++i) {
            const R xi = v[i];
            if (lane > i && lane < n) v[lane] = rsub(v[lane], rmul(xi, M[lane][i]));
            __syncwarp();
        }
        if (lane < n) {
            const R d = M[lane][lane];
            v[lane] = fabs(d) > rmin_normal<R>() ? rdiv(v[lane], d) : R(0);
        }
        __syncwarp();
        for (int i = n - 1; i >= 0; --i) {
            const R xi = v[i];
            if (lane < i) v[lane] = rsub(v[lane], rmul(M[i][lane], xi));
            __syncwarp();
        }
        if (lane == 0)
            for (int k = n - 1; k >= 0; --k) {
                const int p = trans[wi][k];
                const R t = v[k];
                v[k] = v[p];
                v[p] = t;
            }
        __syncwarp();
    };
    solve(xs[wi]);
    if constexpr (REFINE) {
        // r = D^-1 Atb - (D^-1 AtA D^-1) x, the scaled entries formed as above
        if (lane < n) {
            const R inv_i = rdiv(R(1), cs[wi][lane]);
            R r = rdiv(atb[c * (int64_t)run.atb_slot + lane], cs[wi][lane]);
            for (int j = 0; j < n; ++j) {
                const R a = j <= lane ? A[lane * n + j] : A[j * n + lane];
                r = rsub(r, rmul(rmul(rmul(inv_i, a), rdiv(R(1), cs[wi][j])), xs[wi][j]));
            }
            rs[wi][lane] = r;
        }
        __syncwarp();
        solve(rs[wi]);
        if (lane < n) xs[wi][lane] = radd(xs[wi][lane], rs[wi][lane]);
        __syncwarp();
    }
    if (lane < n) xs[wi][lane] = rdiv(xs[wi][lane], cs[wi][lane]);
    __syncwarp();

    // energies and the behaviour error (ref: src/modalsolve.cu:167-203)
    if (lane == 0) {
        R esum = R(0), logwn = R(0), zw = R(0);
        int e = 0;
        for (int i = 0; i < nt; ++i) {
            if (m.dup[i]) continue;
            const int id = 2 * e;
            const R c0 = xs[wi][id], c1 = xs[wi][id + 1];
            const R g00 = A[id * n + id], g01 = A[(id + 1) * n + id], g11 = A[(id + 1) * n + id + 1];
            const R energy = radd(radd(rmul(rmul(c0, c0), g00), rmul(rmul(rmul(R(2), c0), c1), g01)), rmul(rmul(c1, c1), g11));
            const R re = m.Re[i], im = fabs(m.Im[i]);
            const R wn_e = fmax(rsqrt_(radd(rmul(re, re), rmul(im, im))), R(TINY_E6));
            const R ze = rdiv(-re, wn_e);
            md[id] = (float)wn_e;
            md[id + 1] = (float)ze;
            md[2 * nt + e] = (float)energy;
            e++;
            if (im < R(TINY_E6)) continue;
            esum = radd(esum, energy);
            logwn = radd(logwn, rmul(energy, rlog(wn_e)));
            zw = radd(zw, rmul(energy, ze));
        }
        md[3 * nt] = (float)m.unique;
        R wn, zeta;
        if (esum <= R(TINY_E6)) {
            wn = R(TINY_E6);
            zeta = R(0);
        } else {
            wn = rexp(rdiv(logwn, esum));
            zeta = rdiv(zw, esum);
        }
        const R D = R(run.damping), d2 = rmul(D, D);
        const R targetwn = rdiv(rmul(rmul(R(2), R(PI_F)), R(run.bandwidth)),
                                rsqrt_(radd(rsub(R(1), rmul(R(2), d2)),
                                            rsqrt_(radd(rsub(rmul(rmul(R(4), d2), d2), rmul(R(4), d2)), R(2))))));
        const R lw = rlog(rdiv(wn, targetwn));
        const R dz = rsub(zeta, D);
        R berr = radd(rmul(lw, lw), rdiv(rdiv(rmul(dz, dz), D), D));
        const R OS = R(run.overshoot), SSE = R(run.sse);
        const R eos = rdiv(fmax(R(0), rsub(R(fr[2]), OS)), OS);
        berr = radd(berr, rmul(eos, eos));
        const R ess = rdiv(fmax(R(0), rsub(fabs(rsub(rdiv(R(fr[3]), R(run.ref_amp)), R(1))), SSE)), SSE);
        berr = radd(berr, rmul(ess, ess));
        const float b32 = (float)berr;
        sc[0] = isfinite(b32) ? b32 : run.eig_fail_err;
        sc[1] = sc[0];
        fr[0] = (float)wn;
        fr[1] = (float)zeta;
    }
}

// A batch whose fit grid holds at most two blocks per SM (n <= ~2,400
// candidates at 8 per block) is latency-bound and runs 32-step chunks.
static bool fit_long_chunks(int64_t n) {
    static const int sms = [] {
        int dev = 0, k = 0;
        CE_CUDA(cudaGetDevice(&dev));
        CE_CUDA(cudaDeviceGetAttribute(&k, cudaDevAttrMultiProcessorCount, dev));
        return k;
    }();
    return (n + FIT_CPB - 1) / FIT_CPB <= 2 * (int64_t)sms;
}

void launch_fit(const Run& run, int precision, const void* eig, const void* ywin, const void* summ, void* ata,
                void* atb, float* info, int* counts, int* order, cudaStream_t st) {
    const int grid = (int)((run.n + FIT_CPB - 1) / FIT_CPB);
    if (counts) {
        CE_CUDA(cudaMemsetAsync(counts, 0, FIT_CLASSES * sizeof(int), st));
        const int cgrid = (int)((run.n + 127) / 128);
        if (precision == CE_PRECISION_FP64) {
            prefer_shared((const void*)k_fit_classify<double>);
            k_fit_classify<double><<<cgrid, 128, 0, st>>>(run, (const double*)eig, counts, order);
        } else if (run.rg.runs) {
            prefer_shared((const void*)k_fit_classify<float, true>);
            k_fit_classify<float, true><<<cgrid, 128, 0, st>>>(run, (const float*)eig, counts, order);
        } else {
            prefer_shared((const void*)k_fit_classify<float>);
            k_fit_classify<float><<<cgrid, 128, 0, st>>>(run, (const float*)eig, counts, order);
        }
        CE_CUDA(cudaGetLastError());
    }
    prefer_shared(precision == CE_PRECISION_FP64 ? (const void*)k_fit<double, double>
                  : run.rg.runs                  ? (const void*)k_fit<float, SimSummary, true>
                                                 : (const void*)k_fit<float, SimSummary>);
    if (run.rg.runs && precision != CE_PRECISION_FP64)
        k_fit<float, SimSummary, true><<<grid, FIT_BLOCK, 0, st>>>(run, (const float*)eig, (const float*)ywin,
                                                                  (const SimSummary*)summ, (float*)ata, (float*)atb,
                                                                  info, counts, order);
    else if (precision == CE_PRECISION_FP64)
        k_fit<double, double><<<grid, FIT_BLOCK, 0, st>>>(run, (const double*)eig, (const double*)ywin,
                                                         (const double*)summ, (double*)ata, (double*)atb, info,
                                                         counts, order);
    else if (fit_long_chunks(run.n)) {
        prefer_shared((const void*)k_fit<float, SimSummary, false, 32>);
        k_fit<float, SimSummary, false, 32><<<grid, FIT_BLOCK, 0, st>>>(
            run, (const float*)eig, (const float*)ywin, (const SimSummary*)summ, (float*)ata, (float*)atb, info, counts,
            order);
    } else
        k_fit<float, SimSummary><<<grid, FIT_BLOCK, 0, st>>>(run, (const float*)eig, (const float*)ywin,
                                                            (const SimSummary*)summ, (float*)ata, (float*)atb, info,
                                                            counts, order);
    CE_CUDA(cudaGetLastError());
}

void launch_modal(const Run& run, int precision, const void* eig, const void* ata, const void* atb, float* info,
                  cudaStream_t st) {
    const int grid = (int)((run.n + MODAL_WARPS - 1) / MODAL_WARPS);
    if (precision == CE_PRECISION_COMPENSATED || precision == CE_PRECISION_COMPENSATED_TRAJ64 ||
        precision == CE_PRECISION_COMPENSATED_DF) {
        prefer_shared((const void*)k_modal<double, false, true>);
        k_modal<double, false, true><<<grid, 32 * MODAL_WARPS, 0, st>>>(run, (const double*)eig, (const double*)ata,
                                                                       (const double*)atb, info);
        CE_CUDA(cudaGetLastError());
        return;
    }
    prefer_shared(precision == CE_PRECISION_FP64 ? (const void*)k_modal<double>
                  : run.rg.runs                  ? (const void*)k_modal<float, true>
                                                 : (const void*)k_modal<float>);
    if (run.rg.runs && precision != CE_PRECISION_FP64)
        k_modal<float, true><<<grid, 32 * MODAL_WARPS, 0, st>>>(run, (const float*)eig, (const float*)ata,
                                                               (const float*)atb, info);
    else if (precision == CE_PRECISION_FP64)
        k_modal<double><<<grid, 32 * MODAL_WARPS, 0, st>>>(run, (const double*)eig, (const double*)ata,
                                                          (const double*)atb, info);
    else
        k_modal<float><<<grid, 32 * MODAL_WARPS, 0, st>>>(run, (const float*)eig, (const float*)ata,
                                                         (const float*)atb, info);
    CE_CUDA(cudaGetLastError());
}

}  // namespace ce
