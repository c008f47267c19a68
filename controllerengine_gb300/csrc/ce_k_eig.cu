// ce_k_eig.cu -- linearised closed loop and the FP64 eigensolves.
//
// k_lina_eig: builds LIN_A (ref: src/eigensetup.cu:1-57) in float with the
// reference's roundings, then computes its eigenvalues in FP64 and stores them
// as float (re, im) pairs (ref: src/eigensolve.cu:1-19).
// k_nominal: for candidates still in the running after the modal stage, the
// FP64 eigenvalues of the nominal closed loop Acl_nom of the margin check
// (ref: src/allmargin.cu:61-87): stable iff the solve succeeds and every
// |lambda| < 1.
//
// The eigensolver restates the algorithm of the reference's dependency, Eigen's
// EigenSolver<double> with computeEigenvectors=false (Eigen 3.3/3.4; the
// submodule commit is not recorded): scale by max|a_ij|, Householder reduction
// to upper Hessenberg form, Francis double-shift QR with Wilkinson's ad-hoc
// shift at iteration 10 and the MATLAB-style shift at iteration 30 of an
// eigenvalue, at most 40*n iterations, deflation when
// |h(i,i-1)| <= max(eps*(|h(i-1,i-1)|+|h(i,i)|), max(norm*eps^2, DBL_MIN)),
// 2x2 blocks with real eigenvalues split by a Givens rotation; eigenvalues read
// off the quasi-triangular T in diagonal order, a complex pair as
// (t + p, +z), (t + p, -z).  (EISPACK hqr / JAMA hqr2 are the published forms of
// the same iteration.)  Sums are accumulated in index order without fused
// multiply-adds.  Failure (no convergence, or a non-finite eigenvalue) yields
// NaN for the unset eigenvalues; the reference reads unset storage there.
//
// Only the eigenvalues are wanted, so the updates of the Schur form are limited
// to the active window [il, iu]: the reference's full-width updates also
// transform the rows above il and the columns right of iu, but no later step
// that determines an eigenvalue reads those entries (every entry the window's
// steps read lies inside the window, a deflated block is never touched again,
// and the final extraction reads the diagonal band), so the eigenvalues are
// bit-identical with less than the reference's work.  The exceptional shifts
// still update the whole diagonal 0..iu, as in the reference.
//
// GB300 layout: FP64 is a low-rate pipe on this part (2 lanes per clock per
// SM, 1/64 of FP32).  Each matrix lives in shared memory as [element][matrix]
// and is owned by EQ lanes that split the row / column loops (every element is
// still updated by exactly one lane in the sequential order, so results do not
// depend on EQ).  A 16x16 matrix takes 2 KB, so shared memory bounds the
// matrices resident per SM (about 100) and with them the warps that keep the
// FP64 pipe fed: EQ = 1 issues the fewest FP64 instructions per matrix but
// leaves 3 warps per SM; EQ = 2 or 4 gives 6 or 12 warps at the price of
// computing the scalar steps (Householder vectors, shifts) redundantly in
// every lane of the group.  The scans that only read T -- the deflation test
// of every subdiagonal and the search for the row where a Francis step starts
// -- are split over the group's lanes (the first hit from the top is taken,
// which is the sequential scan's answer), and so are the independent divisions
// of a Householder vector.
#include <cfloat>
#include <algorithm>
#include <cstdlib>

#include "ce_device.cuh"
#include "ce_host.h"

namespace ce {

// One warp per block; EQ lanes per matrix, so M = 32 / EQ matrices per block,
// interleaved in shared memory element by element: element e of matrix m at
// double e * M + m.  Matrix m is owned by lanes m, m + M, m + 2M, ..: the lanes
// of a half-warp belong to different matrices and, when they access the same
// element of their matrices (the lanes of a warp run the same loop with the
// same indices), hit 16 different bank pairs -- no conflict and no padding.
constexpr int EIG_LANES_DEFAULT = 2;
constexpr int EIG_BLOCKS_PER_SM_DEFAULT = 5;
// The persistent eigensolve blocks share their SMs with the FP32 stages of the
// other stream, so their registers come out of the fit's and the simulation's
// share.  Bounding them as if 20 one-warp blocks were resident caps them at
// 80-94 registers (no spills), which leaves room for a fifth fit block beside
// the five eigensolve blocks: left unbounded (104 registers) the eigensolve
// itself is ~2% faster but the fit loses a block and the step gets slower.
// With the Kalman observer the other stream runs the register-heavy
// covariance forms instead, and there the unbounded kernels make the step
// shorter (per-candidate noise weights: 93 against 103 ms per 65,536
// candidates), so Kalman sessions launch unbounded instantiations of the
// default form (two lanes per matrix, fused arithmetic).
constexpr int EIG_REG_BLOCKS = 20;
constexpr int EIG_REG_UNBOUNDED = 1;
template <int EQ> constexpr int eig_mats() { return 32 / EQ; }
template <int EQ> constexpr int eig_stride() { return 32 / EQ; }
constexpr double DEPS = 2.220446049250313080847e-16;
constexpr double DMIN_ = 2.2250738585072013831e-308;

struct SMat {
    double* p;  // element (i,j) at p[(i*n + j) * B]
    int n, B;
    __device__ __forceinline__ double& operator()(int i, int j) const { return p[(i * n + j) * B]; }
};

// A group of EQ lanes owns one matrix: loops over rows / columns are split
// over the group, scalar decisions are computed redundantly by all its lanes
// (they read the same values after each __syncwarp), and single-element writes
// are made by the group's lane 0.  Every element is updated by exactly one
// lane with the same operation sequence as a sequential code, so the results
// do not depend on the split.
template <int EQ>
struct Quad {
    static constexpr int N = EQ;       // lanes per matrix
    static constexpr int M = 32 / EQ;  // matrices per warp
    int q;                             // 0..EQ-1, the lane's place in its group
    int m;                             // the matrix slot; the group is lanes m, m + M, ..
    unsigned mask;                     // the group's lanes
    __device__ __forceinline__ void sync() const { __syncwarp(mask); }
    __device__ __forceinline__ bool lead() const { return q == 0; }
    // The first k (in the group's lane order) for which p holds, or -1.
    __device__ __forceinline__ int first(bool p) const {
        const unsigned b = __ballot_sync(mask, p) & mask;
        return b ? (__ffs(b) - 1 - m) / M : -1;
    }
    // v of the group's lane k, in every lane of the group.
    __device__ __forceinline__ double bcast(double v, int k) const { return __shfl_sync(mask, v, m + k * M); }
};

// The eigensolver's arithmetic: F = false rounds every product and every sum
// separately (the reference's Eigen stages compiled without contraction, a
// multiply and an add per multiply-add); F = true fuses each x + a b and
// x - a b into one DFMA, which halves the FP64 instructions of the reflector
// updates.  The operation sequence is otherwise the same in both forms.
template <bool F>
__device__ __forceinline__ double mac(double x, double a, double b) {
    if constexpr (F) return __fma_rn(a, b, x);
    else return __dadd_rn(x, __dmul_rn(a, b));
}
template <bool F>
__device__ __forceinline__ double nmac(double x, double a, double b) {
    if constexpr (F) return __fma_rn(-a, b, x);
    else return __dsub_rn(x, __dmul_rn(a, b));
}

// Householder of the column segment T(r0 .. r0+m-1, col): returns tau and beta
// (read phase only; the caller writes the essential part).
template <bool F>
__device__ __forceinline__ void house_coeffs(const SMat& T, int r0, int m, int col, double& tau, double& beta,
                                             double& d) {
    const double c0 = T(r0, col);
    double tail = 0.0;
    for (int k = r0 + 1; k < r0 + m; ++k) tail = mac<F>(tail, T(k, col), T(k, col));
    if (m == 1) tail = 0.0;
    if (tail <= DMIN_) {
        tau = 0.0;
        beta = c0;
        d = 0.0;
    } else {
        beta = sqrt(mac<F>(tail, c0, c0));
        if (c0 >= 0.0) beta = -beta;
        d = __dsub_rn(c0, beta);
        tau = __ddiv_rn(__dsub_rn(beta, c0), beta);
    }
}

// Householder of a short register vector v[0..m-1] (m = 2 or 3).
template <bool F>
__device__ __forceinline__ void house_vec(const double* v, int m, double* ess, double& tau, double& beta) {
    const double c0 = v[0];
    double tail = __dmul_rn(v[1], v[1]);
    if (m == 3) tail = mac<F>(tail, v[2], v[2]);
    if (tail <= DMIN_) {
        tau = 0.0;
        beta = c0;
        ess[0] = 0.0;
        ess[1] = 0.0;
    } else {
        beta = sqrt(mac<F>(tail, c0, c0));
        if (c0 >= 0.0) beta = -beta;
        const double d = __dsub_rn(c0, beta);
        ess[0] = __ddiv_rn(v[1], d);
        ess[1] = m == 3 ? __ddiv_rn(v[2], d) : 0.0;
        tau = __ddiv_rn(__dsub_rn(beta, c0), beta);
    }
}

// house_vec computed by a group of lanes: the three quotients (v1 / d, v2 / d,
// (beta - c0) / beta) are independent, so the group's lanes divide different
// operands in one division and exchange the results -- the same quotients in
// fewer FP64 instructions per warp (one division of a 2-lane group's three is
// done by both lanes).
template <bool F, class Qd>
__device__ __forceinline__ void house_vec_g(const Qd& Q, const double* v, int m, double* ess, double& tau,
                                            double& beta) {
    if constexpr (Qd::N == 1) {
        house_vec<F>(v, m, ess, tau, beta);
    } else {
        const double c0 = v[0];
        const double v2 = m == 3 ? v[2] : 0.0;
        double tail = __dmul_rn(v[1], v[1]);
        if (m == 3) tail = mac<F>(tail, v2, v2);
        if (tail <= DMIN_) {
            tau = 0.0;
            beta = c0;
            ess[0] = 0.0;
            ess[1] = 0.0;
            return;
        }
        beta = sqrt(mac<F>(tail, c0, c0));
        if (c0 >= 0.0) beta = -beta;
        const double d = __dsub_rn(c0, beta);
        const double nb = __dsub_rn(beta, c0);
        if constexpr (Qd::N == 2) {
            const double x = __ddiv_rn(Q.q == 0 ? v[1] : nb, Q.q == 0 ? d : beta);
            ess[0] = Q.bcast(x, 0);
            tau = Q.bcast(x, 1);
            ess[1] = m == 3 ? __ddiv_rn(v2, d) : 0.0;
        } else {
            // lane 0: v1 / d, lane 1: v2 / d, lanes 2..: (beta - c0) / beta
            const double x = __ddiv_rn(Q.q == 0 ? v[1] : Q.q == 1 ? v2 : nb, Q.q >= 2 ? beta : d);
            ess[0] = Q.bcast(x, 0);
            const double e1 = Q.bcast(x, 1);
            ess[1] = m == 3 ? e1 : 0.0;
            tau = Q.bcast(x, 2);
        }
    }
}

// The deflation point of the Francis iteration: the largest il <= iu with
// il == 0 or |T(il, il-1)| <= max(eps (|T(il-1, il-1)| + |T(il, il)|), zero_tol).
// The tests read T only, so the group's lanes take every N-th row each and
// the first hit from the top is the sequential scan's answer.
template <class Qd>
__device__ __forceinline__ int deflation_row(const SMat& T, const Qd& Q, int iu, double zero_tol) {
    auto small_sub = [&](int il) {
        double s = __dadd_rn(fabs(T(il - 1, il - 1)), fabs(T(il, il)));
        s = fmax(__dmul_rn(s, DEPS), zero_tol);
        return fabs(T(il, il - 1)) <= s;
    };
    if constexpr (Qd::N == 1) {
        int il = iu;
        while (il > 0 && !small_sub(il)) il--;
        return il;
    } else {
        for (int top = iu;; top -= Qd::N) {
            const int il = top - Q.q;
            const int k = Q.first(il == 0 || (il > 0 && small_sub(il)));
            if (k >= 0) return top - k;
        }
    }
}

// The row im in [il, iu-2] where the Francis step starts, and the first
// Householder vector v there: the largest im at which the bulge would not
// disturb a negligible subdiagonal (or il).  Each candidate row's test reads
// T only, so the group's lanes take every N-th row and the first hit from the
// top is the sequential search's row, with v from the lane that found it.
template <bool F, class Qd>
__device__ __forceinline__ int francis_start(const SMat& T, const Qd& Q, int il, int iu, double sh0, double sh1,
                                             double sh2, double* v) {
    auto first_vec = [&](int im, double* w) {
        const double Tmm = T(im, im);
        const double r = __dsub_rn(sh0, Tmm);
        const double s = __dsub_rn(sh1, Tmm);
        w[0] = __dadd_rn(__ddiv_rn(__dsub_rn(__dmul_rn(r, s), sh2), T(im + 1, im)), T(im, im + 1));
        w[1] = __dsub_rn(__dsub_rn(__dsub_rn(T(im + 1, im + 1), Tmm), r), s);
        w[2] = T(im + 2, im + 1);
        if (im == il) return true;
        const double lhs = __dmul_rn(T(im, im - 1), __dadd_rn(fabs(w[1]), fabs(w[2])));
        const double rhs =
            __dmul_rn(w[0], __dadd_rn(__dadd_rn(fabs(T(im - 1, im - 1)), fabs(Tmm)), fabs(T(im + 1, im + 1))));
        return fabs(lhs) < __dmul_rn(DEPS, rhs);
    };
    if constexpr (Qd::N == 1) {
        int im = iu - 2;
        while (!first_vec(im, v)) --im;
        return im;
    } else {
        for (int top = iu - 2;; top -= Qd::N) {
            const int im = top - Q.q;
            double w[3] = {0.0, 0.0, 0.0};
            const int k = Q.first(im >= il && first_vec(im, w));
            if (k >= 0) {
                v[0] = Q.bcast(w[0], k);
                v[1] = Q.bcast(w[1], k);
                v[2] = Q.bcast(w[2], k);
                return top - k;
            }
        }
    }
}

// H = I - tau [1;ess][1;ess]^T from the left on rows r0..r0+m-1, columns
// c0..c1-1 (columns split over the group).  Per column: tmp = ess.T(r0+1..) +
// T(r0), T(r0) -= tau tmp, T(r0+k+1) -= tmp (tau ess_k).  Four columns are
// processed per iteration so that their independent chains overlap; each
// column's operations and their order are unchanged.
template <bool F, class Qd, typename E>
__device__ __forceinline__ void house_left(const SMat& T, const Qd& Q, int r0, int m, int c0, int c1, E ess_at,
                                           double tau) {
    constexpr int S = Qd::N;
    if (m == 1) {
        const double f = __dsub_rn(1.0, tau);
        for (int j = c0 + Q.q; j < c1; j += S) T(r0, j) = __dmul_rn(T(r0, j), f);
        return;
    }
    if (tau == 0.0) return;
    int j = c0 + Q.q;
    for (; j + 3 * S < c1; j += 4 * S) {
        double t[4];
        const double e = ess_at(0);
#pragma unroll
        for (int u = 0; u < 4; ++u) t[u] = __dmul_rn(e, T(r0 + 1, j + u * S));
        for (int k = 1; k < m - 1; ++k) {
            const double ek = ess_at(k);
#pragma unroll
            for (int u = 0; u < 4; ++u) t[u] = mac<F>(t[u], ek, T(r0 + 1 + k, j + u * S));
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            t[u] = __dadd_rn(t[u], T(r0, j + u * S));
            T(r0, j + u * S) = nmac<F>(T(r0, j + u * S), tau, t[u]);
        }
        for (int k = 0; k < m - 1; ++k) {
            const double te = __dmul_rn(tau, ess_at(k));
#pragma unroll
            for (int u = 0; u < 4; ++u)
                T(r0 + 1 + k, j + u * S) = nmac<F>(T(r0 + 1 + k, j + u * S), t[u], te);
        }
    }
    if (j + S < c1) {
        double t[2];
        const double e = ess_at(0);
#pragma unroll
        for (int u = 0; u < 2; ++u) t[u] = __dmul_rn(e, T(r0 + 1, j + u * S));
        for (int k = 1; k < m - 1; ++k) {
            const double ek = ess_at(k);
#pragma unroll
            for (int u = 0; u < 2; ++u) t[u] = mac<F>(t[u], ek, T(r0 + 1 + k, j + u * S));
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            t[u] = __dadd_rn(t[u], T(r0, j + u * S));
            T(r0, j + u * S) = nmac<F>(T(r0, j + u * S), tau, t[u]);
        }
        for (int k = 0; k < m - 1; ++k) {
            const double te = __dmul_rn(tau, ess_at(k));
#pragma unroll
            for (int u = 0; u < 2; ++u)
                T(r0 + 1 + k, j + u * S) = nmac<F>(T(r0 + 1 + k, j + u * S), t[u], te);
        }
        j += 2 * S;
    }
    for (; j < c1; j += S) {
        double tmp = __dmul_rn(ess_at(0), T(r0 + 1, j));
        for (int k = 1; k < m - 1; ++k) tmp = mac<F>(tmp, ess_at(k), T(r0 + 1 + k, j));
        tmp = __dadd_rn(tmp, T(r0, j));
        T(r0, j) = nmac<F>(T(r0, j), tau, tmp);
        for (int k = 0; k < m - 1; ++k) T(r0 + 1 + k, j) = nmac<F>(T(r0 + 1 + k, j), tmp, __dmul_rn(tau, ess_at(k)));
    }
}

// H from the right on rows r0..r1-1 (split over the group), columns
// c0..c0+m-1.  Per row: tmp = T(i,c0+1..).ess + T(i,c0), T(i,c0) -= tau tmp,
// T(i,c0+k+1) -= ess_k (tau tmp).  Four rows per iteration.
template <bool F, class Qd, typename E>
__device__ __forceinline__ void house_right(const SMat& T, const Qd& Q, int r0, int r1, int c0, int m, E ess_at,
                                            double tau) {
    constexpr int S = Qd::N;
    if (m == 1) {
        const double f = __dsub_rn(1.0, tau);
        for (int i = r0 + Q.q; i < r1; i += S) T(i, c0) = __dmul_rn(T(i, c0), f);
        return;
    }
    if (tau == 0.0) return;
    int i = r0 + Q.q;
    for (; i + 3 * S < r1; i += 4 * S) {
        double t[4];
        const double e = ess_at(0);
#pragma unroll
        for (int u = 0; u < 4; ++u) t[u] = __dmul_rn(T(i + u * S, c0 + 1), e);
        for (int k = 1; k < m - 1; ++k) {
            const double ek = ess_at(k);
#pragma unroll
            for (int u = 0; u < 4; ++u) t[u] = mac<F>(t[u], T(i + u * S, c0 + 1 + k), ek);
        }
        double tt[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            t[u] = __dadd_rn(t[u], T(i + u * S, c0));
            T(i + u * S, c0) = nmac<F>(T(i + u * S, c0), tau, t[u]);
            tt[u] = __dmul_rn(tau, t[u]);
        }
        for (int k = 0; k < m - 1; ++k) {
            const double ek = ess_at(k);
#pragma unroll
            for (int u = 0; u < 4; ++u)
                T(i + u * S, c0 + 1 + k) = nmac<F>(T(i + u * S, c0 + 1 + k), ek, tt[u]);
        }
    }
    if (i + S < r1) {
        double t[2];
        const double e = ess_at(0);
#pragma unroll
        for (int u = 0; u < 2; ++u) t[u] = __dmul_rn(T(i + u * S, c0 + 1), e);
        for (int k = 1; k < m - 1; ++k) {
            const double ek = ess_at(k);
#pragma unroll
            for (int u = 0; u < 2; ++u) t[u] = mac<F>(t[u], T(i + u * S, c0 + 1 + k), ek);
        }
        double tt[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            t[u] = __dadd_rn(t[u], T(i + u * S, c0));
            T(i + u * S, c0) = nmac<F>(T(i + u * S, c0), tau, t[u]);
            tt[u] = __dmul_rn(tau, t[u]);
        }
        for (int k = 0; k < m - 1; ++k) {
            const double ek = ess_at(k);
#pragma unroll
            for (int u = 0; u < 2; ++u)
                T(i + u * S, c0 + 1 + k) = nmac<F>(T(i + u * S, c0 + 1 + k), ek, tt[u]);
        }
        i += 2 * S;
    }
    for (; i < r1; i += S) {
        double tmp = __dmul_rn(T(i, c0 + 1), ess_at(0));
        for (int k = 1; k < m - 1; ++k) tmp = mac<F>(tmp, T(i, c0 + 1 + k), ess_at(k));
        tmp = __dadd_rn(tmp, T(i, c0));
        T(i, c0) = nmac<F>(T(i, c0), tau, tmp);
        const double tt = __dmul_rn(tau, tmp);
        for (int k = 0; k < m - 1; ++k) T(i, c0 + 1 + k) = nmac<F>(T(i, c0 + 1 + k), ess_at(k), tt);
    }
}

// The Francis-step reflectors (m = 3, and m = 2 for the last one) with the
// essential part in registers; same per-column / per-row operations as above.
// Several columns (rows) per step: the work per element is a short chain of
// dependent FP64 operations, and independent chains per lane hide most of
// their latency.
template <bool F, int M>
__device__ __forceinline__ void left_col(double& a0, double& a1, double& a2, double e0, double e1, double tau,
                                         double te0, double te1) {
    double t = __dmul_rn(e0, a1);
    if (M == 3) t = mac<F>(t, e1, a2);
    t = __dadd_rn(t, a0);
    a0 = nmac<F>(a0, tau, t);
    a1 = nmac<F>(a1, t, te0);
    if (M == 3) a2 = nmac<F>(a2, t, te1);
}

template <bool F, int M>
__device__ __forceinline__ void right_row(double& a0, double& a1, double& a2, double e0, double e1, double tau) {
    double t = __dmul_rn(a1, e0);
    if (M == 3) t = mac<F>(t, a2, e1);
    t = __dadd_rn(t, a0);
    a0 = nmac<F>(a0, tau, t);
    const double tt = __dmul_rn(tau, t);
    a1 = nmac<F>(a1, e0, tt);
    if (M == 3) a2 = nmac<F>(a2, e1, tt);
}

// U columns j, j+S, .., j+(U-1)S of the left reflector.
template <bool F, int M, int U, int S>
__device__ __forceinline__ void left_cols(const SMat& T, int r0, int j, double e0, double e1, double tau, double te0,
                                          double te1) {
    double a[U][3];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        a[u][0] = T(r0, j + u * S);
        a[u][1] = T(r0 + 1, j + u * S);
        a[u][2] = M == 3 ? T(r0 + 2, j + u * S) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) left_col<F, M>(a[u][0], a[u][1], a[u][2], e0, e1, tau, te0, te1);
#pragma unroll
    for (int u = 0; u < U; ++u) {
        T(r0, j + u * S) = a[u][0];
        T(r0 + 1, j + u * S) = a[u][1];
        if (M == 3) T(r0 + 2, j + u * S) = a[u][2];
    }
}

// U rows i, i+S, .., i+(U-1)S of the right reflector.
template <bool F, int M, int U, int S>
__device__ __forceinline__ void right_rows(const SMat& T, int i, int c0, double e0, double e1, double tau) {
    double a[U][3];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        a[u][0] = T(i + u * S, c0);
        a[u][1] = T(i + u * S, c0 + 1);
        a[u][2] = M == 3 ? T(i + u * S, c0 + 2) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) right_row<F, M>(a[u][0], a[u][1], a[u][2], e0, e1, tau);
#pragma unroll
    for (int u = 0; u < U; ++u) {
        T(i + u * S, c0) = a[u][0];
        T(i + u * S, c0 + 1) = a[u][1];
        if (M == 3) T(i + u * S, c0 + 2) = a[u][2];
    }
}

// Columns (rows) go four at a time, then a pair, then one.
template <bool F, class Qd, int M>
__device__ __forceinline__ void house_left_small(const SMat& T, const Qd& Q, int r0, int c0, int c1, double e0,
                                                 double e1, double tau) {
    if (tau == 0.0) return;
    const double te0 = __dmul_rn(tau, e0), te1 = __dmul_rn(tau, e1);
    constexpr int S = Qd::N;
    int j = c0 + Q.q;
    for (; j + 3 * S < c1; j += 4 * S) left_cols<F, M, 4, S>(T, r0, j, e0, e1, tau, te0, te1);
    if (j + S < c1) {
        left_cols<F, M, 2, S>(T, r0, j, e0, e1, tau, te0, te1);
        j += 2 * S;
    }
    if (j < c1) left_cols<F, M, 1, S>(T, r0, j, e0, e1, tau, te0, te1);
}

template <bool F, class Qd, int M>
__device__ __forceinline__ void house_right_small(const SMat& T, const Qd& Q, int r0, int r1, int c0, double e0,
                                                  double e1, double tau) {
    if (tau == 0.0) return;
    constexpr int S = Qd::N;
    int i = r0 + Q.q;
    for (; i + 3 * S < r1; i += 4 * S) right_rows<F, M, 4, S>(T, i, c0, e0, e1, tau);
    if (i + S < r1) {
        right_rows<F, M, 2, S>(T, i, c0, e0, e1, tau);
        i += 2 * S;
    }
    if (i < r1) right_rows<F, M, 1, S>(T, i, c0, e0, e1, tau);
}

// Givens rotation (c, s) with [c -s; s c] [p; q] = [r; 0].
template <bool F>
__device__ __forceinline__ void make_givens(double p, double q, double& c, double& s) {
    if (q == 0.0) {
        c = p < 0.0 ? -1.0 : 1.0;
        s = 0.0;
    } else if (p == 0.0) {
        c = 0.0;
        s = q < 0.0 ? 1.0 : -1.0;
    } else if (fabs(p) > fabs(q)) {
        const double t = __ddiv_rn(q, p);
        double u = sqrt(mac<F>(1.0, t, t));
        if (p < 0.0) u = -u;
        c = __ddiv_rn(1.0, u);
        s = __dmul_rn(-t, c);
    } else {
        const double t = __ddiv_rn(p, q);
        double u = sqrt(mac<F>(1.0, t, t));
        if (q < 0.0) u = -u;
        s = __ddiv_rn(-1.0, u);
        c = __dmul_rn(-t, s);
    }
}

// x' = c x - s y, y' = s x + c y (the rotation's adjoint applied to the pair).
template <bool F>
__device__ __forceinline__ void rot_pair(double& x, double& y, double c, double s) {
    const double xi = x, yi = y;
    x = mac<F>(__dmul_rn(c, xi), -s, yi);
    y = mac<F>(__dmul_rn(s, xi), c, yi);
}

// Eigenvalues of the n x n matrix in T (overwritten), computed by a quad.
// emit(i, re, im) is called by the quad's lane 0 for i = 0..n-1 in Schur
// order; returns true on success (the same value in every lane).
template <bool F, class Qd, typename Emit>
__device__ bool eig_real(const SMat& T, const Qd& Q, int n, Emit emit) {
    const int nn = n * n;
    double scale = 0.0;
    for (int e = 0; e < nn; ++e) scale = fmax(scale, fabs(T(e / n, e % n)));
    Q.sync();
    bool ok = true;
    if (scale < DMIN_) {
        for (int e = Q.q; e < nn; e += Qd::N) T(e / n, e % n) = 0.0;
        Q.sync();
    } else {
        for (int e = Q.q; e < nn; e += Qd::N) T(e / n, e % n) = __ddiv_rn(T(e / n, e % n), scale);
        Q.sync();
        // Hessenberg reduction
        for (int i = 0; i < n - 1; ++i) {
            const int rs = n - i - 1;
            double tau, beta, d;
            house_coeffs<F>(T, i + 1, rs, i, tau, beta, d);
            Q.sync();
            for (int k = i + 2 + Q.q; k < n; k += Qd::N) T(k, i) = d == 0.0 ? 0.0 : __ddiv_rn(T(k, i), d);
            if (Q.lead()) T(i + 1, i) = beta;
            Q.sync();
            auto ess = [&](int k) { return T(i + 2 + k, i); };
            house_left<F>(T, Q, i + 1, rs, i + 1, n, ess, tau);
            Q.sync();
            house_right<F>(T, Q, 0, n, i + 1, rs, ess, tau);
            Q.sync();
        }
        for (int e = Q.q; e < nn; e += Qd::N)
            if (e % n + 1 < e / n) T(e / n, e % n) = 0.0;
        Q.sync();
        // Francis double-shift QR
        double norm = 0.0;
        for (int j = 0; j < n; ++j) {
            const int last = min(j + 1, n - 1);
            for (int i = 0; i <= last; ++i) norm = __dadd_rn(norm, fabs(T(i, j)));
        }
        const double zero_tol = fmax(__dmul_rn(norm, __dmul_rn(DEPS, DEPS)), DMIN_);
        int iu = n - 1, iter = 0, total = 0;
        const int max_iter = 40 * n;
        double exshift = 0.0;
        if (norm != 0.0) {
            while (iu >= 0) {
                const int il = deflation_row(T, Q, iu, zero_tol);
                Q.sync();
                if (il == iu) {
                    if (Q.lead()) {
                        T(iu, iu) = __dadd_rn(T(iu, iu), exshift);
                        if (iu > 0) T(iu, iu - 1) = 0.0;
                    }
                    Q.sync();
                    iu--;
                    iter = 0;
                } else if (il == iu - 1) {
                    const double p = __dmul_rn(0.5, __dsub_rn(T(iu - 1, iu - 1), T(iu, iu)));
                    const double q = mac<F>(__dmul_rn(p, p), T(iu, iu - 1), T(iu - 1, iu));
                    const double sub = T(iu, iu - 1);
                    Q.sync();
                    if (Q.lead()) {
                        T(iu, iu) = __dadd_rn(T(iu, iu), exshift);
                        T(iu - 1, iu - 1) = __dadd_rn(T(iu - 1, iu - 1), exshift);
                    }
                    Q.sync();
                    if (q >= 0.0) {
                        const double z = sqrt(fabs(q));
                        double c, s;
                        make_givens<F>(p >= 0.0 ? __dadd_rn(p, z) : __dsub_rn(p, z), sub, c, s);
                        if (!(c == 1.0 && s == 0.0)) {
                            for (int j = iu - 1 + Q.q; j <= iu; j += Qd::N) {
                                double x = T(iu - 1, j), y = T(iu, j);
                                rot_pair<F>(x, y, c, s);
                                T(iu - 1, j) = x;
                                T(iu, j) = y;
                            }
                            Q.sync();
                            for (int i = iu - 1 + Q.q; i <= iu; i += Qd::N) {
                                double x = T(i, iu - 1), y = T(i, iu);
                                rot_pair<F>(x, y, c, s);
                                T(i, iu - 1) = x;
                                T(i, iu) = y;
                            }
                            Q.sync();
                        }
                        if (Q.lead()) T(iu, iu - 1) = 0.0;
                    }
                    if (Q.lead() && iu > 1) T(iu - 1, iu - 2) = 0.0;
                    Q.sync();
                    iu -= 2;
                    iter = 0;
                } else {
                    double sh0 = T(iu, iu), sh1 = T(iu - 1, iu - 1), sh2 = __dmul_rn(T(iu, iu - 1), T(iu - 1, iu));
                    Q.sync();
                    if (iter == 10) {
                        exshift = __dadd_rn(exshift, sh0);
                        for (int i = Q.q; i <= iu; i += Qd::N) T(i, i) = __dsub_rn(T(i, i), sh0);
                        Q.sync();
                        const double s = __dadd_rn(fabs(T(iu, iu - 1)), fabs(T(iu - 1, iu - 2)));
                        sh0 = __dmul_rn(0.75, s);
                        sh1 = __dmul_rn(0.75, s);
                        sh2 = __dmul_rn(__dmul_rn(-0.4375, s), s);
                    }
                    if (iter == 30) {
                        double s = __ddiv_rn(__dsub_rn(sh1, sh0), 2.0);
                        s = mac<F>(sh2, s, s);
                        if (s > 0.0) {
                            s = sqrt(s);
                            if (sh1 < sh0) s = -s;
                            s = __dadd_rn(s, __ddiv_rn(__dsub_rn(sh1, sh0), 2.0));
                            s = __dsub_rn(sh0, __ddiv_rn(sh2, s));
                            exshift = __dadd_rn(exshift, s);
                            for (int i = Q.q; i <= iu; i += Qd::N) T(i, i) = __dsub_rn(T(i, i), s);
                            Q.sync();
                            sh0 = sh1 = sh2 = 0.964;
                        }
                    }
                    iter++;
                    total++;
                    if (total > max_iter) break;
                    // first Householder vector
                    double v[3] = {0.0, 0.0, 0.0};
                    const int im = francis_start<F>(T, Q, il, iu, sh0, sh1, sh2, v);
                    // the QR step
                    for (int k = im; k <= iu - 2; ++k) {
                        const bool first = (k == im);
                        double w[3];
                        if (first) {
                            w[0] = v[0]; w[1] = v[1]; w[2] = v[2];
                        } else {
                            w[0] = T(k, k - 1); w[1] = T(k + 1, k - 1); w[2] = T(k + 2, k - 1);
                        }
                        double ess[2], tau, beta;
                        house_vec_g<F>(Q, w, 3, ess, tau, beta);
                        Q.sync();
                        if (beta != 0.0) {
                            if (Q.lead()) {
                                if (first && k > il) T(k, k - 1) = -T(k, k - 1);
                                else if (!first) T(k, k - 1) = beta;
                            }
                            house_left_small<F, Qd, 3>(T, Q, k, k, iu + 1, ess[0], ess[1], tau);
                            Q.sync();
                            house_right_small<F, Qd, 3>(T, Q, il, min(iu, k + 3) + 1, k, ess[0], ess[1], tau);
                            Q.sync();
                        }
                    }
                    {
                        double w[2] = {T(iu - 1, iu - 2), T(iu, iu - 2)};
                        double ess[2], tau, beta;
                        house_vec_g<F>(Q, w, 2, ess, tau, beta);
                        Q.sync();
                        if (beta != 0.0) {
                            if (Q.lead()) T(iu - 1, iu - 2) = beta;
                            house_left_small<F, Qd, 2>(T, Q, iu - 1, iu - 1, iu + 1, ess[0], 0.0, tau);
                            Q.sync();
                            house_right_small<F, Qd, 2>(T, Q, il, iu + 1, iu - 1, ess[0], 0.0, tau);
                            Q.sync();
                        }
                    }
                    for (int i = im + 2 + Q.q; i <= iu; i += Qd::N) {
                        T(i, i - 2) = 0.0;
                        if (i > im + 2) T(i, i - 3) = 0.0;
                    }
                    Q.sync();
                }
            }
        }
        ok = total <= max_iter;
        if (ok) {
            // the extraction below reads the diagonal band only
            for (int i = Q.q; i < n; i += Qd::N) {
                T(i, i) = __dmul_rn(T(i, i), scale);
                if (i + 1 < n) {
                    T(i + 1, i) = __dmul_rn(T(i + 1, i), scale);
                    T(i, i + 1) = __dmul_rn(T(i, i + 1), scale);
                }
            }
            Q.sync();
        }
    }
    if (!ok) {
        if (Q.lead())
            for (int i = 0; i < n; ++i) emit(i, CUDART_NAN, CUDART_NAN);
        return false;
    }
    int i = 0;
    while (i < n) {
        if (i == n - 1 || T(i + 1, i) == 0.0) {
            const double re = T(i, i);
            if (!isfinite(re)) {
                if (Q.lead())
                    for (int k = i; k < n; ++k) emit(k, CUDART_NAN, CUDART_NAN);
                return false;
            }
            if (Q.lead()) emit(i, re, 0.0);
            ++i;
        } else {
            const double p = __dmul_rn(0.5, __dsub_rn(T(i, i), T(i + 1, i + 1)));
            double t0 = T(i + 1, i), t1 = T(i, i + 1);
            const double maxval = fmax(fabs(p), fmax(fabs(t0), fabs(t1)));
            t0 = __ddiv_rn(t0, maxval);
            t1 = __ddiv_rn(t1, maxval);
            const double p0 = __ddiv_rn(p, maxval);
            const double z = __dmul_rn(maxval, sqrt(fabs(mac<F>(__dmul_rn(p0, p0), t0, t1))));
            const double re = __dadd_rn(T(i + 1, i + 1), p);
            if (!(isfinite(re) && isfinite(z))) {
                if (Q.lead())
                    for (int k = i; k < n; ++k) emit(k, CUDART_NAN, CUDART_NAN);
                return false;
            }
            if (Q.lead()) {
                emit(i, re, z);
                emit(i + 1, re, -z);
            }
            i += 2;
        }
    }
    return true;
}

// Plant values (discrete A, B_u, C) of a candidate: the launch's Plant, or the
// candidate's row of the per-candidate plant table.
struct BankPlantValues {
    const Plant& P;
    __device__ __forceinline__ float a(int i, int j) const { return P.d_a[i * MAXD + j]; }
    __device__ __forceinline__ float bu(int i) const { return P.d_bu[i]; }
    __device__ __forceinline__ float c(int j) const { return P.d_c[j]; }
};
struct TablePlantValues {
    const float* t;
    int64_t np, p;
    __device__ __forceinline__ float f(int field) const { return t[(int64_t)field * np + p]; }
    __device__ __forceinline__ float a(int i, int j) const { return f(MC_A + i * MAXD + j); }
    __device__ __forceinline__ float bu(int i) const { return f(MC_BU + i); }
    __device__ __forceinline__ float c(int j) const { return f(MC_C + j); }
};

// LIN_A = [A - B K - L (C - D K),  L Cd ;  -Bu K,  Ad]   (ref: src/eigensetup.cu:19-42)
template <class PV>
__device__ __forceinline__ float lina_entry(const Plant& P, const PV& pv, const float* K, const float* L, int ns,
                                            int i, int j) {
    if (i < ns && j < ns) {
        const float pbk = __fmaf_rn(P.ss_b[i], K[j], 0.0f);
        const float pdk = __fmaf_rn(P.ss_d, K[j], 0.0f);
        const float pcpd = __fsub_rn(P.ss_c[j], pdk);
        const float lpc = __fmaf_rn(L[i], pcpd, 0.0f);
        return __fsub_rn(__fsub_rn(P.ss_a[i * MAXS + j], pbk), lpc);
    }
    if (i < ns) return __fmaf_rn(L[i], pv.c(j - ns), 0.0f);
    if (j < ns) return -__fmaf_rn(pv.bu(i - ns), K[j], 0.0f);
    return pv.a(i - ns, j - ns);
}

template <int EQ>
__device__ __forceinline__ Quad<EQ> make_quad() {
    constexpr int M = 32 / EQ;
    unsigned rep = 0;  // bits 0, M, 2M, ..
#pragma unroll
    for (int k = 0; k < EQ; ++k) rep |= 1u << (k * M);
    const int lane = threadIdx.x & 31;
    return Quad<EQ>{lane / M, lane % M, rep << (lane % M)};
}
// First index of the next 32 / EQ matrices for the calling warp (one-warp
// blocks); called by all 32 lanes together, so the loop around it decides to
// stop for the whole warp at once.
template <int EQ>
__device__ __forceinline__ int64_t take_work(int* next) {
    int base = 0;
    if ((threadIdx.x & 31) == 0) base = atomicAdd(next, eig_mats<EQ>());
    return (int64_t)__shfl_sync(0xFFFFFFFFu, base, 0);
}

// Candidates whose LIN_A eigenvalues pass the modal stability test (no
// |lambda| > 1, the test k_fit and k_modal apply) go on the list that k_nominal
// works through; the others get nominal = -1 (the sweep never reads it).
__device__ __forceinline__ void list_if_stable(bool unstable, int64_t c, int* nominal, int* list, int* count) {
    if (unstable) {
        nominal[c] = -1;
    } else {
        list[atomicAdd(count, 1)] = (int)c;
    }
}

template <int EQ, bool RG = false, bool F = false, int RB = EIG_REG_BLOCKS>
__global__ void __launch_bounds__(32, RB) k_lina_eig(const Run run, const __grid_constant__ Plant P,
                                                        const float* __restrict__ gains, float* __restrict__ lina,
                                                        float* __restrict__ eig32, int* __restrict__ nominal,
                                                        int* __restrict__ list, int* __restrict__ count,
                                                        int* __restrict__ next) {
    extern __shared__ double smem[];
    const auto Q = make_quad<EQ>();
    const int m = Q.m;
    // persistent: the grid covers a fixed number of blocks per SM; each warp
    // takes the next 32 / EQ matrices from a counter when it is done (the
    // iteration count varies a lot between matrices, a static split would
    // leave the slowest warp's share as the tail)
    for (;;) {
        const int64_t base = take_work<EQ>(next);  // the same in every lane
        if (base >= run.n) break;
        const int64_t c = base + m;
        if (c < run.n) {
            const Run& rn = run_of<RG>(run, c);
            const Plant& PP = plant_of<RG>(run, P, c);
            const int ns = rn.ns, nt = rn.nt;
            const float* row = gains + c * rn.cuda_w;
            float K[MAXS], L[MAXS];
#pragma unroll
            for (int i = 0; i < MAXS; ++i) {
                K[i] = i < ns ? row[i] : 0.0f;
                L[i] = i < ns ? row[ns + i] : 0.0f;
            }
            SMat T{smem + m, nt, eig_stride<EQ>()};
            float* lrow = lina + c * (int64_t)rn.lina_slot;
            auto fill = [&](const auto& pv) {
                for (int e = Q.q; e < nt * nt; e += EQ) {
                    const int i = e / nt, j = e % nt;
                    const float v = lina_entry(PP, pv, K, L, ns, i, j);
                    lrow[e] = v;
                    T(i, j) = (double)v;
                }
            };
            if (run.mc.tab) fill(TablePlantValues{run.mc.tab, run.mc.np, mc_plant(run.mc, c)});
            else fill(BankPlantValues{PP});
            Q.sync();
            float* out = eig32 + c * (int64_t)rn.eig_slot;
            float mx = 0.0f;
            eig_real<F>(T, Q, nt, [&](int i, double re, double im) {
                const float fr = (float)re, fi = (float)im;
                out[2 * i] = fr;
                out[2 * i + 1] = fi;
                mx = fmaxf(mx, hypotf(fr, fi));
            });
            if (Q.lead() && list) list_if_stable(mx > 1.0f, c, nominal, list, count);  // no list: nominal runs on all
        }
        __syncwarp();  // the slots are rewritten for the next matrices
    }
}

// FP64-form LIN_A: the same blocks formed in double from the float inputs,
// every product and difference rounded on its own, and kept in double.
__device__ __forceinline__ double lina_entry64(const Plant& P, double Kj, double Li, int i, int j) {
    const double pbk = __dmul_rn((double)P.ss_b[i], Kj);
    const double pdk = __dmul_rn((double)P.ss_d, Kj);
    const double lpc = __dmul_rn(Li, __dsub_rn((double)P.ss_c[j], pdk));
    return __dsub_rn(__dsub_rn((double)P.ss_a[i * MAXS + j], pbk), lpc);
}

template <int EQ, bool F = false>
__global__ void __launch_bounds__(32, EIG_REG_BLOCKS) k_lina_eig64(const Run run, const __grid_constant__ Plant P,
                                                          const float* __restrict__ gains, double* __restrict__ lina,
                                                          double* __restrict__ eig64, int* __restrict__ nominal,
                                                          int* __restrict__ list, int* __restrict__ count,
                                                          int* __restrict__ next) {
    extern __shared__ double smem[];
    const auto Q = make_quad<EQ>();
    const int m = Q.m;
    for (;;) {
        const int64_t base = take_work<EQ>(next);
        if (base >= run.n) break;
        const int64_t c = base + m;
        if (c < run.n) {
            const int ns = run.ns, nt = run.nt;
            const float* row = gains + c * run.cuda_w;
            SMat T{smem + m, nt, eig_stride<EQ>()};
            double* lrow = lina + c * (int64_t)run.lina_slot;
            auto fill = [&](const auto& pv) {
                for (int e = Q.q; e < nt * nt; e += EQ) {
                    const int i = e / nt, j = e % nt;
                    double v;
                    if (i < ns && j < ns) {
                        v = lina_entry64(P, (double)row[j], (double)row[ns + i], i, j);
                    } else if (i < ns) {
                        v = __dmul_rn((double)row[ns + i], (double)pv.c(j - ns));
                    } else if (j < ns) {
                        v = -__dmul_rn((double)pv.bu(i - ns), (double)row[j]);
                    } else {
                        v = pv.a(i - ns, j - ns);
                    }
                    lrow[e] = v;
                    T(i, j) = v;
                }
            };
            if (run.mc.tab) fill(TablePlantValues{run.mc.tab, run.mc.np, mc_plant(run.mc, c)});
            else fill(BankPlantValues{P});
            Q.sync();
            double* out = eig64 + c * (int64_t)run.eig_slot;
            double mx = 0.0;
            eig_real<F>(T, Q, nt, [&](int i, double re, double im) {
                out[2 * i] = re;
                out[2 * i + 1] = im;
                mx = fmax(mx, hypot(re, im));
            });
            if (Q.lead()) list_if_stable(mx > 1.0, c, nominal, list, count);
        }
        __syncwarp();
    }
}

// Nominal closed loop of the margin check (ref: src/allmargin.cu:50-87):
// Acl_nom = [OPEN_A - (D L) K^T, -L C^T; B K^T, A] with OPEN_A = LIN_A[:ns,:ns]
// and (A, B, C, D) the margin plant.  nominal[c] = 1 if stable, 0 if not.
// Only the candidates k_lina_eig listed (those the modal stage does not flag
// unstable, so the only ones the sweep reads) are solved, packed into full
// warps; the work is independent of the modal stage, so this kernel runs
// concurrently with it.  With no list (a small batch) every candidate is
// solved, OPEN_A is formed here with LIN_A's own float operations, and the
// kernel runs concurrently with k_lina_eig (which then lists nothing): the
// flags of the candidates the modal stage flags are computed but never read.
template <int EQ, bool RG = false, bool F = false, int RB = EIG_REG_BLOCKS>
__global__ void __launch_bounds__(32, RB) k_nominal(const Run run, const __grid_constant__ Plant P,
                                                       const float* __restrict__ gains, const void* __restrict__ lina,
                                                       const int* __restrict__ list, const int* __restrict__ count,
                                                       int* __restrict__ nominal, int fp64_form, int* __restrict__ next) {
    extern __shared__ double smem[];
    const auto Q = make_quad<EQ>();
    const int m = Q.m;
    const int64_t listed = list ? (int64_t)*count : run.n;
    for (;;) {
        const int64_t base = take_work<EQ>(next);
        if (base >= listed) break;
        const int64_t idx = base + m;
        if (idx < listed) {
            const int64_t c = list ? (int64_t)list[idx] : idx;
            const Run& rn = run_of<RG>(run, c);
            const Plant& PP = plant_of<RG>(run, P, c);
            const int ns = rn.ns, nt = rn.nt, n2 = 2 * ns;
            const float* row = gains + c * rn.cuda_w;
            const float* la = (const float*)lina + c * (int64_t)rn.lina_slot;
            const double* la64 = (const double*)lina + c * (int64_t)rn.lina_slot;  // the FP64 form's LIN_A
            SMat T{smem + m, n2, eig_stride<EQ>()};
            // margin plant: the Plant's (observer model in batch mode, the round's plant in
            // serial mode), or in serial mode with per-candidate plants the candidate's own
            const TablePlantValues tv{run.mc.tab, run.mc.np, run.mc.tab ? mc_plant(run.mc, c) : 0};
            const bool own = run.mc.tab && run.mc.margin;
            for (int e = Q.q; e < ns * ns; e += EQ) {
                const int i = e / ns, j = e % ns;
                const float Li = row[ns + i];
                const float Kj = row[j];
                const float md = own ? 0.0f : PP.m_d, mcj = own ? tv.c(j) : PP.m_c[j], mbi = own ? tv.bu(i) : PP.m_b[i];
                const float maij = own ? tv.a(i, j) : PP.m_a[i * MAXS + j];
                if (fp64_form) {
                    // OPEN_A from the FP64 form's double LIN_A
                    const double oa = la64[i * nt + j];
                    T(i, j) = __dsub_rn(oa, __dmul_rn(__dmul_rn((double)md, (double)Li), (double)Kj));
                    T(i, ns + j) = -__dmul_rn((double)Li, (double)mcj);
                    T(ns + i, j) = __dmul_rn((double)mbi, (double)Kj);
                } else {
                    // OPEN_A: LIN_A's entry as k_lina_eig stored it, or formed here by the same
                    // function when the two kernels run concurrently (mixed precision only)
                    const float oa = list ? la[i * nt + j] : lina_entry(PP, BankPlantValues{PP}, row, row + ns, ns, i, j);
                    T(i, j) = (double)__fsub_rn(oa, __fmul_rn(__fmul_rn(md, Li), Kj));
                    T(i, ns + j) = (double)(-__fmul_rn(Li, mcj));
                    T(ns + i, j) = (double)__fmul_rn(mbi, Kj);
                }
                T(ns + i, ns + j) = (double)maij;
            }
            Q.sync();
            bool stable = true;
            const bool ok = eig_real<F>(T, Q, n2, [&](int, double re, double im) {
                if (hypot(re, im) >= 1.0) stable = false;
            });
            if (Q.lead()) nominal[c] = (ok && stable) ? 1 : 0;
        }
        __syncwarp();
    }
}

static void set_smem(const void* fn, size_t bytes) {
    CE_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    prefer_shared(fn);
}

// Blocks (one warp each) per SM of the persistent FP64 kernels.  Their
// footprint is mostly shared memory (16 matrices x 2 KB per warp with two
// lanes per matrix); a fixed number per SM keeps the FP64 pipe of every SM
// fed while leaving the rest of the SM to the FP32 stages that run alongside
// on the other stream.  CE_EIG_BLOCKS_PER_SM overrides.
static int eig_blocks_per_sm(const Run& run) {
    static const int dflt = [] {
        const char* e = std::getenv("CE_EIG_BLOCKS_PER_SM");
        const int k = e ? std::atoi(e) : 0;
        return (k >= 1 && k <= 32) ? k : EIG_BLOCKS_PER_SM_DEFAULT;
    }();
    return (run.eig_blocks >= 1 && run.eig_blocks <= 32) ? run.eig_blocks : dflt;
}

static int sm_count() {
    int dev = 0, sms = 0;
    CE_CUDA(cudaGetDevice(&dev));
    CE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    return sms;
}

static int eig_grid(const Run& run, int64_t work, int mats) {
    const int64_t need = (work + mats - 1) / mats;
    return (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)eig_blocks_per_sm(run) * sm_count()));
}

static bool valid_lanes(int k) { return k == 1 || k == 2 || k == 4 || k == 8 || k == 16; }

// Lanes per matrix of the FP64 eigensolves of n matrices.  An FP64 warp
// instruction occupies the pipe for its full time whatever its active lanes,
// so the lanes of a matrix cost nothing extra while they are spare: they split
// the row and column loops (every element is still updated by exactly one
// lane in the same order, so results do not depend on the split) and compute
// the scalar steps redundantly.  A large batch fills the persistent grid with
// two lanes per matrix (LIN_A eigensolve of 65,536 16x16 matrices: 21.9 ms
// with one lane, 18.4 ms with two); a batch too small to fill it gets more
// lanes per matrix, up to 16 -- the most that still hold every matrix in one
// resident pass -- which shortens each matrix's chain of instructions.  A
// session's tuning (Run::eig_lanes) or CE_EIG_LANES=1|2|4|8|16 overrides.
static int eig_lanes(const Run& run, int64_t n) {
    static const int env = [] {
        const char* e = std::getenv("CE_EIG_LANES");
        const int k = e ? std::atoi(e) : 0;
        return valid_lanes(k) ? k : 0;
    }();
    if (valid_lanes(run.eig_lanes)) return run.eig_lanes;
    if (env) return env;
    const int64_t warps = (int64_t)eig_blocks_per_sm(run) * sm_count();
    int eq = EIG_LANES_DEFAULT;
    while (eq < 16 && (n * (2 * eq) + 31) / 32 <= warps) eq *= 2;
    return eq;
}

template <int EQ, bool F>
static void lina_eig_qf(const Run& run, const Plant& P, int precision, const float* gains, void* lina, void* eig,
                        int* nominal, int* list, int* count, cudaStream_t st) {
    const int grid = eig_grid(run, run.n, eig_mats<EQ>());
    const size_t smem = (size_t)run.nt * run.nt * eig_stride<EQ>() * sizeof(double);
    if (precision == CE_PRECISION_FP64) {
        set_smem((const void*)k_lina_eig64<EQ, F>, smem);
        k_lina_eig64<EQ, F><<<grid, 32, smem, st>>>(run, P, gains, (double*)lina, (double*)eig, nominal, list, count,
                                                     count + 1);
    } else if (run.rg.runs) {
        set_smem((const void*)k_lina_eig<EQ, true, F>, smem);
        k_lina_eig<EQ, true, F><<<grid, 32, smem, st>>>(run, P, gains, (float*)lina, (float*)eig, nominal, list,
                                                         count, count + 1);
    } else {
        if constexpr (EQ == 2 && F) {
            if (run.kalman) {
                auto* k = k_lina_eig<EQ, false, F, EIG_REG_UNBOUNDED>;
                set_smem((const void*)k, smem);
                k<<<grid, 32, smem, st>>>(run, P, gains, (float*)lina, (float*)eig, nominal, list, count, count + 1);
                return;
            }
        }
        set_smem((const void*)k_lina_eig<EQ, false, F>, smem);
        k_lina_eig<EQ, false, F><<<grid, 32, smem, st>>>(run, P, gains, (float*)lina, (float*)eig, nominal, list,
                                                          count, count + 1);
    }
}

template <int EQ>
static void lina_eig_q(const Run& run, const Plant& P, int precision, const float* gains, void* lina, void* eig,
                       int* nominal, int* list, int* count, cudaStream_t st) {
    if (run.eig_fused) lina_eig_qf<EQ, true>(run, P, precision, gains, lina, eig, nominal, list, count, st);
    else lina_eig_qf<EQ, false>(run, P, precision, gains, lina, eig, nominal, list, count, st);
}

template <int EQ, bool F>
static void nominal_qf(const Run& run, const Plant& P, int precision, const float* gains, const void* lina,
                       const int* list, const int* count, int* nominal, cudaStream_t st) {
    const int grid = eig_grid(run, run.n, eig_mats<EQ>());  // the listed count is only known on the device
    const size_t smem = (size_t)(2 * run.ns) * (2 * run.ns) * eig_stride<EQ>() * sizeof(double);
    if (run.rg.runs) {
        set_smem((const void*)k_nominal<EQ, true, F>, smem);
        k_nominal<EQ, true, F><<<grid, 32, smem, st>>>(run, P, gains, lina, list, count, nominal, 0,
                                                       const_cast<int*>(count) + 2);
    } else {
        if constexpr (EQ == 2 && F) {
            if (run.kalman) {
                auto* k = k_nominal<EQ, false, F, EIG_REG_UNBOUNDED>;
                set_smem((const void*)k, smem);
                k<<<grid, 32, smem, st>>>(run, P, gains, lina, list, count, nominal, precision == CE_PRECISION_FP64,
                                          const_cast<int*>(count) + 2);
                return;
            }
        }
        set_smem((const void*)k_nominal<EQ, false, F>, smem);
        k_nominal<EQ, false, F><<<grid, 32, smem, st>>>(run, P, gains, lina, list, count, nominal,
                                                        precision == CE_PRECISION_FP64, const_cast<int*>(count) + 2);
    }
}

template <int EQ>
static void nominal_q(const Run& run, const Plant& P, int precision, const float* gains, const void* lina,
                      const int* list, const int* count, int* nominal, cudaStream_t st) {
    if (run.eig_fused) nominal_qf<EQ, true>(run, P, precision, gains, lina, list, count, nominal, st);
    else nominal_qf<EQ, false>(run, P, precision, gains, lina, list, count, nominal, st);
}

void launch_lina_eig(const Run& run, const Plant& P, int precision, const float* gains, void* lina, void* eig,
                     int* nominal, int* list, int* count, cudaStream_t st, bool clear) {
    if (clear) CE_CUDA(cudaMemsetAsync(count, 0, 3 * sizeof(int), st));  // listed, lina work, nominal work
    switch (eig_lanes(run, run.n)) {
        case 1: lina_eig_q<1>(run, P, precision, gains, lina, eig, nominal, list, count, st); break;
        case 2: lina_eig_q<2>(run, P, precision, gains, lina, eig, nominal, list, count, st); break;
        case 4: lina_eig_q<4>(run, P, precision, gains, lina, eig, nominal, list, count, st); break;
        case 8: lina_eig_q<8>(run, P, precision, gains, lina, eig, nominal, list, count, st); break;
        default: lina_eig_q<16>(run, P, precision, gains, lina, eig, nominal, list, count, st); break;
    }
    CE_CUDA(cudaGetLastError());
}

void launch_nominal(const Run& run, const Plant& P, int precision, const float* gains, const void* lina,
                    const int* list, const int* count, int* nominal, cudaStream_t st) {
    // the listed count is only known on the device: lanes as for all n candidates
    switch (eig_lanes(run, run.n)) {
        case 1: nominal_q<1>(run, P, precision, gains, lina, list, count, nominal, st); break;
        case 2: nominal_q<2>(run, P, precision, gains, lina, list, count, nominal, st); break;
        case 4: nominal_q<4>(run, P, precision, gains, lina, list, count, nominal, st); break;
        case 8: nominal_q<8>(run, P, precision, gains, lina, list, count, nominal, st); break;
        default: nominal_q<16>(run, P, precision, gains, lina, list, count, nominal, st); break;
    }
    CE_CUDA(cudaGetLastError());
}

}  // namespace ce
