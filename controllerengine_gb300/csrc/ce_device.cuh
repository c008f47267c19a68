// ce_device.cuh -- device arithmetic shared by the kernels.
//
// Rounding discipline: every operation whose result must equal the
// reference's is written with an explicit round-to-nearest intrinsic
// (__fadd_rn, __fmul_rn, __fmaf_rn, ...), so the compiler can neither
// contract a multiply-add the reference keeps separate nor split one it
// fuses.  The reference's device code uses __fmaf_rn / __fadd_rn explicitly
// in the simulation (ref: src/main.cu:122-155, src/discrete_solves.cu); its
// host stages (Eigen on x86) never fuse.
#pragma once

#ifndef __CUDACC_RTC__
#include <cuda_runtime.h>
#endif
#include <math_constants.h>
#include "ce_internal.h"

namespace ce {

// The sizes and plant of candidate c: the launch's in a uniform evaluation, its
// instance's in a ragged one.
template <bool RG>
__device__ __forceinline__ const Run& run_of(const Run& run, int64_t c) {
    if constexpr (RG) return run.rg.runs[run.rg.inst[c]];
    else return run;
}
template <bool RG>
__device__ __forceinline__ const Plant& plant_of(const Run& run, const Plant& P, int64_t c) {
    if constexpr (RG) return run.rg.plants[run.rg.inst[c]];
    else return P;
}

// The plant of candidate c in a per-candidate-plant evaluation.
__device__ __forceinline__ int64_t mc_plant(const McPlants& m, int64_t c) {
    return m.idx ? (int64_t)m.idx[c] : m.first + c;
}

// ---- scalar ops in a type-generic, contraction-proof form -------------------
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float rfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double rfma(double a, double b, double c) { return __fma_rn(a, b, c); }

// ---- double-float numbers: an unevaluated sum hi + lo of two floats ---------
// (|lo| <= half an ulp of hi), about 48 significant bits on the FP32 pipe.
// The operations are the classical error-free transformations (Knuth's
// TwoSum, Dekker's Fast2Sum, the fused-multiply-add TwoProduct) composed into
// the usual double-double add, multiply and divide; each result is within a
// few units of 2^-48 relative.  Used by the simulation of the compensated_df
// precision, where FP32 products would bound the trajectory at ~1e-7.
// The type and its operations live in namespace dd and are found by
// argument-dependent lookup, so they never hide the float and double
// overloads (fmax, radd, ...) that code in this namespace calls.
namespace dd {
struct ddf {
    float hi, lo;
    ddf() = default;
    __device__ __forceinline__ constexpr ddf(float h, float l) : hi(h), lo(l) {}
    __device__ __forceinline__ constexpr ddf(float h) : hi(h), lo(0.0f) {}
    __device__ __forceinline__ constexpr ddf(int h) : hi((float)h), lo(0.0f) {}
    __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
};
__device__ __forceinline__ ddf dd_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return ddf(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ ddf dd_fast_sum(float a, float b) {  // |a| >= |b| or a == 0
    const float s = __fadd_rn(a, b);
    return ddf(s, __fsub_rn(b, __fsub_rn(s, a)));
}
// A sum or product that overflows (or meets an infinity or NaN) is returned as
// (hi, 0) with hi the plain float result, as a double would be inf or NaN.
__device__ __forceinline__ ddf radd(ddf x, ddf y) {
    const ddf s = dd_two_sum(x.hi, y.hi), t = dd_two_sum(x.lo, y.lo);
    if (!isfinite(s.hi)) return ddf(s.hi, 0.0f);
    ddf r = dd_fast_sum(s.hi, __fadd_rn(s.lo, t.hi));
    r = dd_fast_sum(r.hi, __fadd_rn(r.lo, t.lo));
    return isfinite(r.hi) ? r : ddf(r.hi, 0.0f);
}
__device__ __forceinline__ ddf rneg(ddf x) { return ddf(-x.hi, -x.lo); }
__device__ __forceinline__ ddf rsub(ddf x, ddf y) { return radd(x, rneg(y)); }
__device__ __forceinline__ ddf rmul(ddf x, ddf y) {
    const float p = __fmul_rn(x.hi, y.hi);
    if (!isfinite(p)) return ddf(p, 0.0f);
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fmaf_rn(x.hi, y.lo, e);
    e = __fmaf_rn(x.lo, y.hi, e);
    return dd_fast_sum(p, e);
}
// a float coefficient times a double-float: the exact product of a and hi plus a lo
__device__ __forceinline__ ddf rmul(float a, ddf y) {
    const float p = __fmul_rn(a, y.hi);
    if (!isfinite(p)) return ddf(p, 0.0f);
    return dd_fast_sum(p, __fmaf_rn(a, y.lo, __fmaf_rn(a, y.hi, -p)));
}
__device__ __forceinline__ ddf rdiv(ddf x, ddf y) {
    // long division: three float quotient digits, each remainder formed in double-float
    const float q1 = __fdiv_rn(x.hi, y.hi);
    if (!isfinite(q1) || q1 == 0.0f) return ddf(q1, 0.0f);
    ddf r = rsub(x, rmul(q1, y));
    const float q2 = __fdiv_rn(r.hi, y.hi);
    r = rsub(r, rmul(q2, y));
    const float q3 = __fdiv_rn(r.hi, y.hi);
    const ddf q = dd_fast_sum(q1, q2);
    return radd(q, ddf(q3));
}
__device__ __forceinline__ ddf rfma(ddf a, ddf b, ddf c) { return radd(rmul(a, b), c); }
__device__ __forceinline__ ddf rfma(float a, ddf b, ddf c) { return radd(rmul(a, b), c); }
__device__ __forceinline__ bool operator<(ddf a, ddf b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(ddf a, ddf b) { return b < a; }
// (a self-comparison: inside this namespace the name isnan would find this
// overload again, not the float one)
__device__ __forceinline__ bool isnan(ddf a) { return a.hi != a.hi || a.lo != a.lo; }
__device__ __forceinline__ ddf fmax(ddf a, ddf b) { return isnan(a) ? b : isnan(b) ? a : a < b ? b : a; }
__device__ __forceinline__ ddf fmin(ddf a, ddf b) { return isnan(a) ? b : isnan(b) ? a : b < a ? b : a; }
}  // namespace dd
using dd::ddf;
__device__ __forceinline__ double rfma(float a, double b, double c) { return __fma_rn((double)a, b, c); }
__device__ __forceinline__ double rmul(float a, double b) { return __dmul_rn((double)a, b); }
__device__ __forceinline__ double rneg(double x) { return -x; }

template <typename R> __device__ __forceinline__ R rnan();
template <> __device__ __forceinline__ float rnan<float>() { return CUDART_NAN_F; }
template <> __device__ __forceinline__ double rnan<double>() { return CUDART_NAN; }
template <> __device__ __forceinline__ ddf rnan<ddf>() { return ddf(CUDART_NAN_F, CUDART_NAN_F); }
template <typename R> __device__ __forceinline__ R rinf();
template <> __device__ __forceinline__ double rinf<double>() { return CUDART_INF; }
template <> __device__ __forceinline__ ddf rinf<ddf>() { return ddf(CUDART_INF_F, 0.0f); }

// ---- double-float accumulation (ref: src/main.cu:129-155) --------------------
// TwoSum of a and b.
__device__ __forceinline__ void df_two_sum(float a, float b, float& hi, float& lo) {
    hi = __fadd_rn(a, b);
    const float b0 = __fsub_rn(hi, a);
    lo = __fadd_rn(__fsub_rn(a, __fsub_rn(hi, b0)), __fsub_rn(b, b0));
}
// (HI,LO) += (hi,lo): TwoSum of the high parts, low parts folded in, renormalised.
__device__ __forceinline__ void df_add(float& HI, float& LO, float hi, float lo) {
    float sh, sl;
    df_two_sum(HI, hi, sh, sl);
    const float v = __fadd_rn(__fadd_rn(LO, lo), sl);
    HI = __fadd_rn(sh, v);
    LO = __fsub_rn(v, __fsub_rn(HI, sh));
}

// Steady-state sum of the trajectory.  s is the plain float sum in t order
// (the reference's, ref: src/modalsetup.cu:54-56), unchanged; comp collects
// the exact rounding error of each addition (TwoSum), so s + comp is the
// compensated sum (the Kahan-Babuska / Neumaier form) that the compensated
// precision reads.
__device__ __forceinline__ void ysum_add(float& s, float& comp, float y) {
    const float t = __fadd_rn(s, y);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(y, bp));
    comp = __fadd_rn(comp, err);
    s = t;
}

// ---- the instruction interpreter (ref: src/main.cu:260-291) ------------------
// Evaluates one SKIP-free chain of `n` instructions.  `src` holds the NSRC
// source values addressed by the instruction column; column `ycol` (if >= 0)
// addresses `yval` instead (the NL chains' plant-output slot).  The first
// instruction's running value is the seed when HAS_SEED and the seed is not NaN,
// else the state under its column; later ones use the running result.  With
// TAB the constant operands come from a per-candidate table instead of the
// instructions: instruction r's (a, b) at cst[2 r * cs] and cst[(2 r + 1) * cs].
template <typename R, int NSRC, int MAXC, bool HAS_SEED, bool TAB = false>
__device__ __forceinline__ R run_chain(const Instr* __restrict__ ins, int n, const R* src, int ycol, R yval, R seed,
                                       const float* __restrict__ cst = nullptr, int64_t cs = 0) {
    R result = R(0);
#pragma unroll
    for (int r = 0; r < MAXC; ++r) {
        if (r >= n) break;
        const int op = ins[r].op, col = ins[r].col, ak = ins[r].akind, bk = ins[r].bkind;
        R pos = R(0);
#pragma unroll
        for (int c = 0; c < NSRC; ++c)
            if (col == c) pos = src[c];
        if (col == ycol) pos = yval;
        R prev;
        if (r == 0) prev = (HAS_SEED && !isnan(seed)) ? seed : pos;
        else prev = result;
        const float av = !TAB ? ins[r].aval : ak == CE_OPERAND_CONST ? cst[2 * r * cs] : 0.0f;
        const float bv = !TAB ? ins[r].bval : bk == CE_OPERAND_CONST ? cst[(2 * r + 1) * cs] : 0.0f;
        const R a = ak == CE_OPERAND_CONST ? R(av) : (ak == CE_OPERAND_STATE ? pos : prev);
        const R b = bk == CE_OPERAND_CONST ? R(bv) : (bk == CE_OPERAND_STATE ? pos : prev);
        switch (op) {
            case 1: result = radd(a, b); break;
            case 2: result = rsub(a, b); break;
            case 3: result = rmul(a, b); break;
            case 4: result = rdiv(a, b); break;
            case 5: result = fmin(fmax(prev, a), b); break;
            case 6: result = R((R(0) < a) - (a < R(0))); break;
            default: break;  // op outside 1..6: no change, but the chain counts as started
        }
    }
    return result;
}

// The same chain with its sources in shared memory: source column c of this
// thread is src[c * stride].  The column is warp-uniform, so each interpreted
// instruction reads its state with one load instead of a select over every
// column; the loads do not depend on the chain and issue ahead of it.
template <typename R, int MAXC, bool HAS_SEED>
__device__ __forceinline__ R run_chain_sm(const Instr* __restrict__ ins, int n, const R* src, int stride, R seed) {
    R result = R(0);
#pragma unroll
    for (int r = 0; r < MAXC; ++r) {
        if (r >= n) break;
        const int op = ins[r].op, ak = ins[r].akind, bk = ins[r].bkind;
        const R pos = src[ins[r].col * stride];
        R prev;
        if (r == 0) prev = (HAS_SEED && !isnan(seed)) ? seed : pos;
        else prev = result;
        const R a = ak == CE_OPERAND_CONST ? R(ins[r].aval) : (ak == CE_OPERAND_STATE ? pos : prev);
        const R b = bk == CE_OPERAND_CONST ? R(ins[r].bval) : (bk == CE_OPERAND_STATE ? pos : prev);
        switch (op) {
            case 1: result = radd(a, b); break;
            case 2: result = rsub(a, b); break;
            case 3: result = rmul(a, b); break;
            case 4: result = rdiv(a, b); break;
            case 5: result = fmin(fmax(prev, a), b); break;
            case 6: result = R((R(0) < a) - (a < R(0))); break;
            default: break;
        }
    }
    return result;
}

// ---- complex arithmetic in a fixed operation order ---------------------------
template <typename R>
struct cplx {
    R re, im;
};
template <typename R>
__device__ __forceinline__ cplx<R> cmul(cplx<R> a, cplx<R> b) {
    return {rsub(rmul(a.re, b.re), rmul(a.im, b.im)), radd(rmul(a.re, b.im), rmul(a.im, b.re))};
}
template <typename R>
__device__ __forceinline__ cplx<R> csub(cplx<R> a, cplx<R> b) {
    return {rsub(a.re, b.re), rsub(a.im, b.im)};
}
// a / b as a*conj(b) / |b|^2, each part divided by |b|^2.
template <typename R>
__device__ __forceinline__ cplx<R> cdiv(cplx<R> a, cplx<R> b) {
    const R d = radd(rmul(b.re, b.re), rmul(b.im, b.im));
    const R nr = radd(rmul(a.re, b.re), rmul(a.im, b.im));
    const R ni = rsub(rmul(a.im, b.re), rmul(a.re, b.im));
    return {rdiv(nr, d), rdiv(ni, d)};
}
__device__ __forceinline__ float cabs_(cplx<float> a) { return hypotf(a.re, a.im); }
__device__ __forceinline__ double cabs_(cplx<double> a) { return hypot(a.re, a.im); }
__device__ __forceinline__ float carg_(cplx<float> a) { return atan2f(a.im, a.re); }
__device__ __forceinline__ double carg_(cplx<double> a) { return atan2(a.im, a.re); }
// squared modulus; orders pivots like the modulus does, without a libm call
template <typename R>
__device__ __forceinline__ R cnorm2(cplx<R> a) {
    return radd(rmul(a.re, a.re), rmul(a.im, a.im));
}
template <typename R>
__device__ __forceinline__ bool cfinite(cplx<R> a) {
    return isfinite(a.re) && isfinite(a.im);
}

// Solve (z I - A) x = b for an NS x NS real A (row stride NS) by complex LU
// with partial pivoting (largest modulus, compared as re^2+im^2; first on ties), unit-lower forward
// and column-oriented backward substitution.  Restates the partialPivLu().solve
// call sites of the reference (ref: src/allmargin.cu:24-29, 37, 103-104).
// A is read as A[(i*NS + j) * astride].  An exactly zero pivot is left in
// place, so the solve then produces non-finite values.
//
// The forward substitution is carried along with the elimination: at step k
// the right-hand side takes the row interchange and then x[i] -= x[k] l_ik for
// i > k.  Every element of x receives the same operations in the same order
// as in "x = P b, then column-oriented forward substitution" (interchanges do
// not change values, and x[k] is final when it is used), so the results are
// identical; the multipliers are dead after their step, which keeps the
// factorisation in registers.
template <typename R, int NS>
__device__ __forceinline__ void lu_solve_shifted(cplx<R> z, const R* A, int astride, const R* b, cplx<R>* x) {
    cplx<R> M[NS][NS];
#pragma unroll
    for (int i = 0; i < NS; ++i)
#pragma unroll
        for (int j = 0; j < NS; ++j) {
            // z*I - A, with z*I formed as z times (1,0) / (0,0)
            const cplx<R> zi = (i == j) ? cplx<R>{rsub(rmul(z.re, R(1)), rmul(z.im, R(0))), radd(rmul(z.re, R(0)), rmul(z.im, R(1)))}
                                        : cplx<R>{rsub(rmul(z.re, R(0)), rmul(z.im, R(0))), radd(rmul(z.re, R(0)), rmul(z.im, R(0)))};
            M[i][j] = csub(zi, cplx<R>{A[(i * NS + j) * astride], R(0)});
        }
#pragma unroll
    for (int i = 0; i < NS; ++i) x[i] = cplx<R>{b[i], R(0)};
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        // pivot: largest |M(i,k)|, i >= k, first maximum wins
        int p = k;
        R best = cnorm2(M[k][k]);
#pragma unroll
        for (int i = k + 1; i < NS; ++i) {
            const R s = cnorm2(M[i][k]);
            if (s > best) { best = s; p = i; }
        }
        // row interchange (the multiplier columns j < k are not used again),
        // as selects over the candidate rows so that M stays in registers
#pragma unroll
        for (int j = k; j <= NS; ++j) {
            cplx<R>& top = j < NS ? M[k][j] : x[k];
            cplx<R> piv = top;
#pragma unroll
            for (int i = k + 1; i < NS; ++i) {
                cplx<R>& e = j < NS ? M[i][j] : x[i];
                const bool hit = i == p;
                const cplx<R> old = e;
                e.re = hit ? top.re : e.re;
                e.im = hit ? top.im : e.im;
                piv.re = hit ? old.re : piv.re;
                piv.im = hit ? old.im : piv.im;
            }
            top = piv;
        }
        if (best != R(0)) {
#pragma unroll
            for (int i = k + 1; i < NS; ++i) M[i][k] = cdiv(M[i][k], M[k][k]);
        }
#pragma unroll
        for (int i = k + 1; i < NS; ++i) {
#pragma unroll
            for (int j = k + 1; j < NS; ++j) M[i][j] = csub(M[i][j], cmul(M[i][k], M[k][j]));
            x[i] = csub(x[i], cmul(x[k], M[i][k]));
        }
    }
    // upper, column oriented
#pragma unroll
    for (int i = NS - 1; i >= 0; --i) {
        x[i] = cdiv(x[i], M[i][i]);
#pragma unroll
        for (int s = 0; s < i; ++s) x[s] = csub(x[s], cmul(x[i], M[s][i]));
    }
}

}  // namespace ce
