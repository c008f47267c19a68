/* ce_oracle_eig.h -- the oracle's FP64 eigensolver, included twice by
 * ce_oracle.c: EIGN(name) names the copy and MAC / NMAC give its multiply-add
 * arithmetic (x + a b and x - a b rounded twice, or fused into one fma).  Test
 * infrastructure only.
 *
 * Householder reduction to upper Hessenberg form and Francis double-shift QR
 * with exceptional shifts at iterations 10 and 30 and at most 40 n iterations,
 * the algorithm of Eigen's EigenSolver<double> without eigenvectors (ref:
 * src/eigensolve.cu:6-16, the reference's only call into it), restated from
 * the published algorithm; eigenvalues in Schur order, a complex pair as
 * (re, +z), (re, -z). */
#define T_(i, j) T[(i) * MT + (j)]

static void EIGN(house)(const double* v, int m, double* ess, double* tau, double* beta) {
    /* v[0..m-1] -> essential v[1..]/(v0-beta), tau, beta */
    const double c0 = v[0];
    double tail = 0.0;
    for (int k = 1; k < m; k++) tail = MAC(tail, v[k], v[k]);
    if (tail <= DBL_MIN) {
        *tau = 0.0;
        *beta = c0;
        for (int k = 1; k < m; k++) ess[k - 1] = 0.0;
    } else {
        double b = sqrt(MAC(tail, c0, c0));
        if (c0 >= 0.0) b = -b;
        for (int k = 1; k < m; k++) ess[k - 1] = v[k] / (c0 - b);
        *tau = (b - c0) / b;
        *beta = b;
    }
}

/* apply I - tau [1;ess][1;ess]^T from the left to rows r0..r0+m-1, cols c0..c1-1 */
static void EIGN(hleft)(double* T, int r0, int m, int c0, int c1, const double* ess, double tau) {
    if (m == 1) {
        for (int j = c0; j < c1; j++) T_(r0, j) = T_(r0, j) * (1.0 - tau);
        return;
    }
    if (tau == 0.0) return;
    for (int j = c0; j < c1; j++) {
        double tmp = ess[0] * T_(r0 + 1, j);
        for (int k = 1; k < m - 1; k++) tmp = MAC(tmp, ess[k], T_(r0 + 1 + k, j));
        tmp = tmp + T_(r0, j);
        T_(r0, j) = NMAC(T_(r0, j), tau, tmp);
        for (int k = 0; k < m - 1; k++) T_(r0 + 1 + k, j) = NMAC(T_(r0 + 1 + k, j), tmp, tau * ess[k]);
    }
}

/* apply from the right to rows r0..r1-1, cols c0..c0+m-1 */
static void EIGN(hright)(double* T, int r0, int r1, int c0, int m, const double* ess, double tau) {
    if (m == 1) {
        for (int i = r0; i < r1; i++) T_(i, c0) = T_(i, c0) * (1.0 - tau);
        return;
    }
    if (tau == 0.0) return;
    for (int i = r0; i < r1; i++) {
        double tmp = T_(i, c0 + 1) * ess[0];
        for (int k = 1; k < m - 1; k++) tmp = MAC(tmp, T_(i, c0 + 1 + k), ess[k]);
        tmp = tmp + T_(i, c0);
        T_(i, c0) = NMAC(T_(i, c0), tau, tmp);
        const double tt = tau * tmp;
        for (int k = 0; k < m - 1; k++) T_(i, c0 + 1 + k) = NMAC(T_(i, c0 + 1 + k), ess[k], tt);
    }
}

static void EIGN(givens)(double p, double q, double* c, double* s) {
    if (q == 0.0) {
        *c = p < 0.0 ? -1.0 : 1.0;
        *s = 0.0;
    } else if (p == 0.0) {
        *c = 0.0;
        *s = q < 0.0 ? 1.0 : -1.0;
    } else if (fabs(p) > fabs(q)) {
        const double t = q / p;
        double u = sqrt(MAC(1.0, t, t));
        if (p < 0.0) u = -u;
        *c = 1.0 / u;
        *s = -t * *c;
    } else {
        const double t = p / q;
        double u = sqrt(MAC(1.0, t, t));
        if (q < 0.0) u = -u;
        *s = -1.0 / u;
        *c = -t * *s;
    }
}

/* eigenvalues of the n x n matrix A (row stride MT, overwritten) in Schur order;
   returns 1 on success; on failure the unset entries are NaN */
int EIGN(oracle_eig)(double* T, int n, double* wr, double* wi) {
    double scale = 0.0;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) scale = fmax(scale, fabs(T_(i, j)));
    int ok = 1;
    if (scale < DBL_MIN) {
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) T_(i, j) = 0.0;
    } else {
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) T_(i, j) = T_(i, j) / scale;
        for (int i = 0; i < n - 1; i++) {
            const int rs = n - i - 1;
            double v[MT], ess[MT], tau, beta;
            for (int k = 0; k < rs; k++) v[k] = T_(i + 1 + k, i);
            EIGN(house)(v, rs, ess, &tau, &beta);
            for (int k = 0; k < rs - 1; k++) T_(i + 2 + k, i) = ess[k];
            T_(i + 1, i) = beta;
            EIGN(hleft)(T, i + 1, rs, i + 1, n, ess, tau);
            EIGN(hright)(T, 0, n, i + 1, rs, ess, tau);
        }
        for (int i = 0; i < n; i++)
            for (int j = 0; j + 1 < i; j++) T_(i, j) = 0.0;
        double norm = 0.0;
        for (int j = 0; j < n; j++) {
            const int last = j + 1 < n - 1 ? j + 1 : n - 1;
            for (int i = 0; i <= last; i++) norm = norm + fabs(T_(i, j));
        }
        const double ztol = fmax(norm * (EPS_D * EPS_D), DBL_MIN);
        int iu = n - 1, iter = 0, total = 0;
        const int maxit = 40 * n;
        double exshift = 0.0;
        if (norm != 0.0) {
            while (iu >= 0) {
                int il = iu;
                while (il > 0) {
                    double s = fabs(T_(il - 1, il - 1)) + fabs(T_(il, il));
                    s = fmax(s * EPS_D, ztol);
                    if (fabs(T_(il, il - 1)) <= s) break;
                    il--;
                }
                if (il == iu) {
                    T_(iu, iu) = T_(iu, iu) + exshift;
                    if (iu > 0) T_(iu, iu - 1) = 0.0;
                    iu--;
                    iter = 0;
                } else if (il == iu - 1) {
                    const double p = 0.5 * (T_(iu - 1, iu - 1) - T_(iu, iu));
                    const double q = MAC(p * p, T_(iu, iu - 1), T_(iu - 1, iu));
                    T_(iu, iu) = T_(iu, iu) + exshift;
                    T_(iu - 1, iu - 1) = T_(iu - 1, iu - 1) + exshift;
                    if (q >= 0.0) {
                        const double z = sqrt(fabs(q));
                        double cs, sn;
                        EIGN(givens)(p >= 0.0 ? p + z : p - z, T_(iu, iu - 1), &cs, &sn);
                        if (!(cs == 1.0 && sn == 0.0)) {
                            for (int j = iu - 1; j < n; j++) {
                                const double x = T_(iu - 1, j), y = T_(iu, j);
                                T_(iu - 1, j) = MAC(cs * x, -sn, y);
                                T_(iu, j) = MAC(sn * x, cs, y);
                            }
                            for (int i = 0; i <= iu; i++) {
                                const double x = T_(i, iu - 1), y = T_(i, iu);
                                T_(i, iu - 1) = MAC(cs * x, -sn, y);
                                T_(i, iu) = MAC(sn * x, cs, y);
                            }
                        }
                        T_(iu, iu - 1) = 0.0;
                    }
                    if (iu > 1) T_(iu - 1, iu - 2) = 0.0;
                    iu -= 2;
                    iter = 0;
                } else {
                    double s0 = T_(iu, iu), s1 = T_(iu - 1, iu - 1), s2 = T_(iu, iu - 1) * T_(iu - 1, iu);
                    if (iter == 10) {
                        exshift = exshift + s0;
                        for (int i = 0; i <= iu; i++) T_(i, i) = T_(i, i) - s0;
                        const double s = fabs(T_(iu, iu - 1)) + fabs(T_(iu - 1, iu - 2));
                        s0 = 0.75 * s;
                        s1 = 0.75 * s;
                        s2 = -0.4375 * s * s;
                    }
                    if (iter == 30) {
                        double s = (s1 - s0) / 2.0;
                        s = MAC(s2, s, s);
                        if (s > 0.0) {
                            s = sqrt(s);
                            if (s1 < s0) s = -s;
                            s = s + (s1 - s0) / 2.0;
                            s = s0 - s2 / s;
                            exshift = exshift + s;
                            for (int i = 0; i <= iu; i++) T_(i, i) = T_(i, i) - s;
                            s0 = s1 = s2 = 0.964;
                        }
                    }
                    iter++;
                    total++;
                    if (total > maxit) break;
                    double v[3] = {0.0, 0.0, 0.0};
                    int im;
                    for (im = iu - 2; im >= il; --im) {
                        const double Tmm = T_(im, im);
                        const double r = s0 - Tmm, s = s1 - Tmm;
                        v[0] = (r * s - s2) / T_(im + 1, im) + T_(im, im + 1);
                        v[1] = T_(im + 1, im + 1) - Tmm - r - s;
                        v[2] = T_(im + 2, im + 1);
                        if (im == il) break;
                        const double lhs = T_(im, im - 1) * (fabs(v[1]) + fabs(v[2]));
                        const double rhs = v[0] * (fabs(T_(im - 1, im - 1)) + fabs(Tmm) + fabs(T_(im + 1, im + 1)));
                        if (fabs(lhs) < EPS_D * rhs) break;
                    }
                    for (int k = im; k <= iu - 2; k++) {
                        const int first = k == im;
                        double w[3], ess[2], tau, beta;
                        if (first) {
                            w[0] = v[0]; w[1] = v[1]; w[2] = v[2];
                        } else {
                            w[0] = T_(k, k - 1); w[1] = T_(k + 1, k - 1); w[2] = T_(k + 2, k - 1);
                        }
                        EIGN(house)(w, 3, ess, &tau, &beta);
                        if (beta != 0.0) {
                            if (first && k > il) T_(k, k - 1) = -T_(k, k - 1);
                            else if (!first) T_(k, k - 1) = beta;
                            EIGN(hleft)(T, k, 3, k, n, ess, tau);
                            EIGN(hright)(T, 0, (iu < k + 3 ? iu : k + 3) + 1, k, 3, ess, tau);
                        }
                    }
                    {
                        double w[2] = {T_(iu - 1, iu - 2), T_(iu, iu - 2)}, ess[2], tau, beta;
                        EIGN(house)(w, 2, ess, &tau, &beta);
                        if (beta != 0.0) {
                            T_(iu - 1, iu - 2) = beta;
                            EIGN(hleft)(T, iu - 1, 2, iu - 1, n, ess, tau);
                            EIGN(hright)(T, 0, iu + 1, iu - 1, 2, ess, tau);
                        }
                    }
                    for (int i = im + 2; i <= iu; i++) {
                        T_(i, i - 2) = 0.0;
                        if (i > im + 2) T_(i, i - 3) = 0.0;
                    }
                }
            }
        }
        ok = total <= maxit;
        if (ok)
            for (int i = 0; i < n; i++)
                for (int j = 0; j < n; j++) T_(i, j) = T_(i, j) * scale;
    }
    for (int i = 0; i < n; i++) wr[i] = wi[i] = NAN;
    if (!ok) return 0;
    int i = 0;
    while (i < n) {
        if (i == n - 1 || T_(i + 1, i) == 0.0) {
            if (!isfinite(T_(i, i))) return 0;
            wr[i] = T_(i, i);
            wi[i] = 0.0;
            i++;
        } else {
            const double p = 0.5 * (T_(i, i) - T_(i + 1, i + 1));
            double t0 = T_(i + 1, i), t1 = T_(i, i + 1);
            const double mx = fmax(fabs(p), fmax(fabs(t0), fabs(t1)));
            t0 = t0 / mx;
            t1 = t1 / mx;
            const double p0 = p / mx;
            const double z = mx * sqrt(fabs(MAC(p0 * p0, t0, t1)));
            const double re = T_(i + 1, i + 1) + p;
            if (!(isfinite(re) && isfinite(z))) return 0;
            wr[i] = re;
            wi[i] = z;
            wr[i + 1] = re;
            wi[i + 1] = -z;
            i += 2;
        }
    }
    return 1;
}
#undef T_
