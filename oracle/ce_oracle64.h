/* ce_oracle64.h -- the plain FP64 form of the reference's method, restated
 * on the CPU for checking the engine's CE_PRECISION_FP64 pipeline.  Test
 * infrastructure only; included at the end of ce_oracle.c (it shares that
 * file's decoded plant and configuration helpers).
 *
 * The method is the reference's -- discrete_solve<Luenberger>
 * (ref: src/discrete_solves.cu:12-79), eigensetup (ref: src/eigensetup.cu:1-57),
 * eigensolve (ref: src/eigensolve.cu:1-19), modalsetup (ref:
 * src/modalsetup.cu:1-97), modalsolve (ref: src/modalsolve.cu:1-108) and
 * allmargin (ref: src/allmargin.cu:1-182) -- with every quantity in double:
 * the state without the hi/lo split, LIN_A, the eigenvalues (never cast to
 * float), the fit basis, the normal equations and their LDLT solve, the
 * plant and loop responses and the margin scan.  Inputs (gains, plant, the
 * configuration's floats) are the float values widened; outputs are the INFO
 * row's floats.  Each operation follows the engine's FP64 kernels in kind
 * and order (fused where they fuse, rounded separately where they do not),
 * so that what differs is only the libm of the transcendental functions
 * (exp, log, sin, cos, atan2, hypot: glibc here, CUDA's there, each within
 * an ulp or two). */

/* the dimension class the engine's kernels loop over: 4 or 8 */
static int dim_class64(int d) { return d <= 4 ? 4 : 8; }

/* one chain of the interpreter in double (ref: src/main.cu:260-291); src has
   MNL entries, src[MD] the plant output y */
static double interp64(const oc_ins* info, int count, const double* src, int has_seed, double seed) {
    double result = 0.0;
    int started = 0;
    for (int r = 0; r < count; r++) {
        const oc_ins in = info[r];
        if (in.op == 0) continue;
        double pos = 0.0;
        for (int c = 0; c < MNL; c++)
            if (c == in.col) pos = src[c];
        const double prev = started ? result : ((has_seed && !isnan(seed)) ? seed : pos);
        const double a = in.akind == 0 ? (double)in.aval : (in.akind == 1 ? pos : prev);
        const double b = in.bkind == 0 ? (double)in.bval : (in.bkind == 1 ? pos : prev);
        switch (in.op) {
            case 1: result = a + b; break;
            case 2: result = a - b; break;
            case 3: result = a * b; break;
            case 4: result = a / b; break;
            case 5: result = fmin(fmax(prev, a), b); break;
            case 6: result = (double)((0.0 < a) - (a < 0.0)); break;
            default: break;
        }
        started = 1;
    }
    return result;
}

/* simulation: the fit window ywin[fit_steps] and (sum of y over the steady
   window, max y, min y) */
static void sim64_one(const oc_cfg* c, const oc_der* d, const oc_pp* P, const float* row, int fit_steps,
                      double* ywin, double* summ) {
    const int ns = c->ns, NSC = dim_class64(c->ns), NDC = dim_class64(c->nd);
    double K[MS] = {0}, L[MS] = {0};
    for (int i = 0; i < NSC; i++) {
        K[i] = i < ns ? (double)row[i] : 0.0;
        L[i] = i < ns ? (double)row[ns + i] : 0.0;
    }
    const double N = row[2 * ns];
    double xh[MS] = {0}, xp[MD] = {0};
    double ysum = 0.0, ymax = -INFINITY, ymin = INFINITY;
    for (int t = 0; t < c->time; t++) {
        double src[MNL] = {0};
        for (int i = 0; i < NDC; i++) src[i] = xp[i];
        const double y = interp64(P->dc, MDC, src, 0, 0.0);
        const int w = t - d->fit_start_id;
        if (w >= 0 && w < fit_steps) ywin[w] = y;
        if (t >= d->steady_start_id) ysum = ysum + y;
        ymax = fmax(ymax, y);
        ymin = fmin(ymin, y);
        double kx = 0.0;
        for (int i = 0; i < NSC; i++) kx = fma(K[i], xh[i], kx);
        const double ref = ((double)t < c->ref_step_time * (double)c->time) ? 0.0 : (double)c->ref_amplitude;
        double hs[MNL] = {0};
        for (int i = 0; i < NSC; i++) hs[i] = xh[i];
        const double u = interp64(P->u, MU, hs, 1, fma(N, ref, -kx));
        double yh = 0.0;
        for (int i = 0; i < NSC; i++) yh = fma((double)P->ss_c[i], xh[i], yh);
        yh = fma((double)P->ss_d, u, yh);
        const double yerr = y - yh;
        double dh[MS];
        for (int i = 0; i < NSC; i++) {
            double h = fma(L[i], yerr, (double)P->ss_b[i] * u);
            for (int j = 0; j < NSC; j++) h = fma((double)P->ss_ai[i * MS + j], xh[j], h);
            dh[i] = h;
        }
        for (int i = 0; i < NSC; i++) xh[i] = xh[i] + dh[i];
        src[MD] = y;
        double W[MW];
        for (int k = 0; k < MW; k++) W[k] = interp64(&P->nl[k * MNLI], MNLI, src, 0, 0.0);
        double ph[MD];
        for (int i = 0; i < NDC; i++) {
            double h = (double)P->d_bu[i] * u;
            for (int k = 0; k < MW; k++) h = fma((double)P->d_bw[i * MW + k], W[k], h);
            for (int j = 0; j < NDC; j++) h = fma((double)P->d_ai[i * MD + j], xp[j], h);
            ph[i] = h;
        }
        for (int i = 0; i < NDC; i++) xp[i] = xp[i] + ph[i];
    }
    summ[0] = ysum;
    summ[1] = ymax;
    summ[2] = ymin;
}

/* LIN_A in double (ref: src/eigensetup.cu:19-42): every product and
   difference rounded on its own */
static void lina64_one(const oc_cfg* c, const oc_pp* P, const float* row, double* out) {
    const int ns = c->ns, nd = c->nd, nt = ns + nd;
    for (int i = 0; i < nt; i++)
        for (int j = 0; j < nt; j++) {
            double v;
            if (i < ns && j < ns) {
                const double Kj = row[j], Li = row[ns + i];
                const double pbk = (double)P->ss_b[i] * Kj;
                const double pdk = (double)P->ss_d * Kj;
                const double lpc = Li * ((double)P->ss_c[j] - pdk);
                v = ((double)P->ss_a[i * MS + j] - pbk) - lpc;
            } else if (i < ns) {
                v = (double)row[ns + i] * (double)P->d_c[j - ns];
            } else if (j < ns) {
                v = -((double)P->d_bu[i - ns] * (double)row[j]);
            } else {
                v = P->d_a[(i - ns) * MD + (j - ns)];
            }
            out[i * nt + j] = v;
        }
}

typedef struct oc_modes64 {
    double Re[MT], Im[MT], max_mag;
    int dup[MT], unique;
} oc_modes64;

/* modes from the double eigenvalues (ref: src/modalsetup.cu:8-50) */
static void modes64_of(const double* eig, int nt, double ts, oc_modes64* m) {
    m->max_mag = 0.0;
    for (int i = 0; i < nt; i++) {
        const double re = eig[2 * i], im = eig[2 * i + 1];
        const double mag = hypot(re, im);
        m->max_mag = fmax(m->max_mag, mag);
        m->Re[i] = log(fmax(mag, (double)LFLOOR)) / ts;
        m->Im[i] = atan2(im, re) / ts;
        m->dup[i] = 0;
    }
    double pre = (double)SENT, pim = (double)SENT;
    int unique = nt;
    for (int i = 0; i < nt; i++) {
        if (fabs(m->Re[i] - pre) < (double)TINY6 && fabs(fabs(m->Im[i]) - fabs(pim)) < (double)TINY6) {
            m->dup[i] = 1;
            unique--;
        }
        pre = m->Re[i];
        pim = m->Im[i];
    }
    m->unique = unique;
}

/* modal setup in double (ref: src/modalsetup.cu:52-94): yss, overshoot and the
   normal equations, each entry one fused multiply-add per window step in t order */
static void modalsetup64_one(const oc_cfg* c, const oc_der* d, int fit_steps, const double* ywin,
                             const double* summ, const double* eig, double* ata, double* atb, float* out) {
    const int nt = d->nt, n2 = 2 * nt;
    const double ts = d->ts;
    for (int e = 0; e < n2 * n2; e++) ata[e] = 0.0;
    for (int e = 0; e < n2; e++) atb[e] = 0.0;
    oc_modes64 m;
    modes64_of(eig, nt, ts, &m);
    float* sc = out + d->info_scoring;
    float* fr = out + d->info_freqresp;
    if (m.max_mag > 1.0) {
        const float v = (float)((double)c->unstable_err + log(m.max_mag) / ts);
        sc[0] = v;
        sc[1] = v;
        return;
    }
    const int unique = m.unique, nc = 2 * unique;
    double sig[MT], om[MT], shift[MT];
    for (int i = 0, e = 0; i < nt; i++) {
        if (m.dup[i]) continue;
        sig[e] = m.Re[i];
        om[e] = fabs(m.Im[i]);
        shift[e] = fmax(sig[e] * (double)d->fit_t0, sig[e] * (double)d->fit_t1);
        e++;
    }
    const double yss = summ[0] / (double)(c->time - d->steady_start_id);
    {
        const double pk = fmax(0.0, yss >= 0.0 ? summ[1] * yss : summ[2] * yss);
        fr[2] = (float)(pk / fmax(yss * yss, (double)TINY6) - 1.0);
        fr[3] = (float)yss;
    }
    const int wlimit = c->time - d->fit_start_id;
    double A[(2 * MT + 1) * (2 * MT + 1)];
    const int N = nc + 1;
    for (int e = 0; e < N * N; e++) A[e] = 0.0;
    for (int w = 0; w < fit_steps; w++) {
        double v[2 * MT + 1];
        for (int e = 0; e < unique; e++) {
            const double tval = (double)(d->fit_start_id + w) * ts;
            const double decay = exp(fma(sig[e], tval, -shift[e]));
            const double arg = om[e] * tval;
            v[2 * e] = decay * cos(arg);
            v[2 * e + 1] = decay * sin(arg);
        }
        v[nc] = (w < wlimit ? ywin[w] : 0.0) - yss;
        for (int i = 0; i < N; i++)
            for (int j = 0; j <= i; j++) A[i * N + j] = fma(v[i], v[j], A[i * N + j]);
    }
    for (int i = 0; i < nc; i++)
        for (int j = 0; j <= i; j++) ata[i * n2 + j] = A[i * N + j];
    for (int j = 0; j < nc; j++) atb[j] = A[nc * N + j];
}

/* LDLT with symmetric pivoting on the largest remaining |diagonal| in double,
   the engine's k_modal<double> step for step; A full symmetric, overwritten;
   x: right-hand side in, solution out */
static void ldlt64_solve(double* A, int n, double* x) {
    int tr[2 * MT];
    int stop = 0;
    for (int k = 0; k < n && !stop; k++) {
        int p = k;
        double best = fabs(A[k * n + k]);
        if (isnan(best)) best = INFINITY;
        for (int i = k + 1; i < n; i++) {
            double v = fabs(A[i * n + i]);
            if (isnan(v)) v = -INFINITY;
            if (v > best) {
                best = v;
                p = i;
            }
        }
        tr[k] = p;
        if (p != k) {
            for (int j = 0; j < k; j++) {
                const double t = A[k * n + j];
                A[k * n + j] = A[p * n + j];
                A[p * n + j] = t;
            }
            for (int i = p + 1; i < n; i++) {
                const double t = A[i * n + k];
                A[i * n + k] = A[i * n + p];
                A[i * n + p] = t;
            }
            for (int i = k + 1; i < p; i++) {
                const double t = A[i * n + k];
                A[i * n + k] = A[p * n + i];
                A[p * n + i] = t;
            }
            const double t = A[k * n + k];
            A[k * n + k] = A[p * n + p];
            A[p * n + p] = t;
        }
        if (k > 0) {
            double tk = 0.0, col[2 * MT];
            for (int j = 0; j < k; j++) tk = tk + A[k * n + j] * (A[j * n + j] * A[k * n + j]);
            for (int i = k + 1; i < n; i++) {
                double acc = 0.0;
                for (int j = 0; j < k; j++) acc = acc + A[i * n + j] * (A[j * n + j] * A[k * n + j]);
                col[i] = acc;
            }
            A[k * n + k] = A[k * n + k] - tk;
            for (int i = k + 1; i < n; i++) A[i * n + k] = A[i * n + k] - col[i];
        }
        const double akk = A[k * n + k];
        const int valid = fabs(akk) > 0.0;
        if (k == 0 && !valid) {
            for (int j = 0; j < n; j++) tr[j] = j;
            stop = 1;
        } else if (valid) {
            for (int i = k + 1; i < n; i++) A[i * n + k] = A[i * n + k] / akk;
        }
    }
    for (int k = 0; k < n; k++) {
        const double t = x[k];
        x[k] = x[tr[k]];
        x[tr[k]] = t;
    }
    for (int i = 0; i < n; i++)
        for (int s = i + 1; s < n; s++) x[s] = x[s] - x[i] * A[s * n + i];
    for (int i = 0; i < n; i++) {
        const double dd = A[i * n + i];
        x[i] = fabs(dd) > DBL_MIN ? x[i] / dd : 0.0;
    }
    for (int i = n - 1; i >= 0; i--)
        for (int s = 0; s < i; s++) x[s] = x[s] - A[i * n + s] * x[i];
    for (int k = n - 1; k >= 0; k--) {
        const double t = x[k];
        x[k] = x[tr[k]];
        x[tr[k]] = t;
    }
}

/* modal solve and the behaviour score in double (ref: src/modalsolve.cu:1-108) */
static void modalsolve64_one(const oc_cfg* c, const oc_der* d, const double* ata, const double* atb,
                             const double* eig, float* out) {
    const int nt = d->nt, n = 2 * nt;
    const double ts = d->ts;
    float* sc = out + d->info_scoring;
    float* fr = out + d->info_freqresp;
    float* md = out + d->info_modal;
    if (sc[0] != 0.0f) return;
    oc_modes64 m;
    modes64_of(eig, nt, ts, &m);
    if (m.max_mag > 1.0) {
        const float v = (float)((double)c->unstable_err + log(m.max_mag) / ts);
        sc[0] = v;
        sc[1] = v;
        return;
    }
    double S[4 * MT * MT], cs[2 * MT], x[2 * MT];
    for (int i = 0; i < n; i++) {
        const double s = sqrt(ata[i * n + i]);
        cs[i] = s > (double)TINY6 ? s : 1.0;
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            const double a = j <= i ? ata[i * n + j] : ata[j * n + i];
            S[i * n + j] = ((1.0 / cs[i]) * a) * (1.0 / cs[j]);
        }
    for (int i = 0; i < n; i++) x[i] = atb[i] / cs[i];
    ldlt64_solve(S, n, x);
    for (int i = 0; i < n; i++) x[i] = x[i] / cs[i];
    double esum = 0.0, logwn = 0.0, zw = 0.0;
    int e = 0;
    for (int i = 0; i < nt; i++) {
        if (m.dup[i]) continue;
        const int id = 2 * e;
        const double c0 = x[id], c1 = x[id + 1];
        const double g00 = ata[id * n + id], g01 = ata[(id + 1) * n + id], g11 = ata[(id + 1) * n + id + 1];
        const double energy = ((c0 * c0) * g00 + ((2.0 * c0) * c1) * g01) + (c1 * c1) * g11;
        const double re = m.Re[i], im = fabs(m.Im[i]);
        const double wn_e = fmax(sqrt(re * re + im * im), (double)TINY6);
        const double ze = -re / wn_e;
        md[id] = (float)wn_e;
        md[id + 1] = (float)ze;
        md[2 * nt + e] = (float)energy;
        e++;
        if (im < (double)TINY6) continue;
        esum = esum + energy;
        logwn = logwn + energy * log(wn_e);
        zw = zw + energy * ze;
    }
    md[3 * nt] = (float)m.unique;
    double wn, zeta;
    if (esum <= (double)TINY6) {
        wn = (double)TINY6;
        zeta = 0.0;
    } else {
        wn = exp(logwn / esum);
        zeta = zw / esum;
    }
    const double D = c->damping, d2 = D * D;
    const double twn = ((2.0 * (double)PI_F) * (double)c->bandwidth) /
                       sqrt((1.0 - 2.0 * d2) + sqrt((((4.0 * d2) * d2) - 4.0 * d2) + 2.0));
    const double lw = log(wn / twn);
    const double dz = zeta - D;
    double berr = lw * lw + ((dz * dz) / D) / D;
    const double OS = c->overshoot, SSE = c->sse;
    const double eos = fmax(0.0, (double)fr[2] - OS) / OS;
    berr = berr + eos * eos;
    const double ess = fmax(0.0, fabs((double)fr[3] / (double)c->ref_amplitude - 1.0) - SSE) / SSE;
    berr = berr + ess * ess;
    const float b32 = (float)berr;
    sc[0] = isfinite(b32) ? b32 : c->eig_fail_err;
    sc[1] = sc[0];
    fr[0] = (float)wn;
    fr[1] = (float)zeta;
}

/* ---- margins in double (ref: src/allmargin.cu:1-182) ---- */
typedef struct cd {
    double re, im;
} cd;
static cd cmul64(cd a, cd b) {
    cd r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static cd csub64(cd a, cd b) {
    cd r = {a.re - b.re, a.im - b.im};
    return r;
}
static cd cdiv64(cd a, cd b) {
    const double d = b.re * b.re + b.im * b.im;
    cd r = {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
    return r;
}

/* x = (z I - A)^{-1} b for the n x n row-major A by complex LU with partial
   pivoting; returns 1 if x is finite */
static int lu64_solve(cd z, const double* A, const double* b, int n, cd* x) {
    cd M[MS][MS];
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            cd zi;
            if (i == j) {
                zi.re = z.re * 1.0 - z.im * 0.0;
                zi.im = z.re * 0.0 + z.im * 1.0;
            } else {
                zi.re = z.re * 0.0 - z.im * 0.0;
                zi.im = z.re * 0.0 + z.im * 0.0;
            }
            const cd a = {A[i * n + j], 0.0};
            M[i][j] = csub64(zi, a);
        }
    int perm[MS];
    for (int k = 0; k < n; k++) {
        int p = k;
        double best = M[k][k].re * M[k][k].re + M[k][k].im * M[k][k].im;
        for (int i = k + 1; i < n; i++) {
            const double s = M[i][k].re * M[i][k].re + M[i][k].im * M[i][k].im;
            if (s > best) {
                best = s;
                p = i;
            }
        }
        perm[k] = p;
        if (p != k)
            for (int j = 0; j < n; j++) {
                const cd t = M[k][j];
                M[k][j] = M[p][j];
                M[p][j] = t;
            }
        if (best != 0.0)
            for (int i = k + 1; i < n; i++) M[i][k] = cdiv64(M[i][k], M[k][k]);
        for (int i = k + 1; i < n; i++)
            for (int j = k + 1; j < n; j++) M[i][j] = csub64(M[i][j], cmul64(M[i][k], M[k][j]));
    }
    for (int i = 0; i < n; i++) {
        x[i].re = b[i];
        x[i].im = 0.0;
    }
    for (int k = 0; k < n; k++) {
        const cd t = x[k];
        x[k] = x[perm[k]];
        x[perm[k]] = t;
    }
    for (int i = 0; i < n; i++)
        for (int s = i + 1; s < n; s++) x[s] = csub64(x[s], cmul64(x[i], M[s][i]));
    for (int i = n - 1; i >= 0; i--) {
        x[i] = cdiv64(x[i], M[i][i]);
        for (int s = 0; s < i; s++) x[s] = csub64(x[s], cmul64(x[i], M[s][i]));
    }
    for (int i = 0; i < n; i++)
        if (!isfinite(x[i].re) || !isfinite(x[i].im)) return 0;
    return 1;
}

/* C^T x + D, accumulated in index order */
static cd ctx64(const double* C, const cd* x, int n, double D) {
    cd acc = {0.0, 0.0};
    for (int i = 0; i < n; i++) {
        const cd k = {C[i], 0.0};
        const cd t = cmul64(k, x[i]);
        acc.re = acc.re + t.re;
        acc.im = acc.im + t.im;
    }
    acc.re = acc.re + D;
    return acc;
}

typedef struct oc_grid64 {
    int F;
    double *z, *th, *pr, *pm, alpha;
    int* pok;
} oc_grid64;

/* the double sweep grid (z_w from double libm on the float configuration) and
   the margin plant's response on it; 0, or -1 if alpha fails */
static int plant_grid64(const oc_cfg* c, const oc_der* d, const oc_mp* mp, oc_grid64* g) {
    const int F = c->freq, n = mp->n;
    double A[MS * MS], B[MS], C[MS];
    for (int i = 0; i < n * n; i++) A[i] = mp->A[i];
    for (int i = 0; i < n; i++) {
        B[i] = mp->B[i];
        C[i] = mp->C[i];
    }
    const double inc = (log((double)d->freq_max) - log((double)c->freq_min)) / (double)(F - 1);
    for (int w = 0; w < F; w++) {
        const double th = exp(log((double)c->freq_min) + inc * (double)w) * (double)d->ts;
        const cd z = {cos(th), sin(th)};
        cd x[MS];
        const int ok = lu64_solve(z, A, B, n, x);
        cd p = {0.0, 0.0};
        if (ok) p = ctx64(C, x, n, (double)mp->D);
        g->z[2 * w] = z.re;
        g->z[2 * w + 1] = z.im;
        g->th[w] = atan2(z.im, z.re);
        g->pr[2 * w] = p.re;
        g->pr[2 * w + 1] = p.im;
        g->pm[w] = hypot(p.re, p.im);
        g->pok[w] = ok;
    }
    const double t = (double)d->crossover * (double)d->ts;
    const cd zc = {cos(t), sin(t)};
    cd x[MS];
    const int ok = lu64_solve(zc, A, B, n, x);
    cd p = {0.0, 0.0};
    if (ok) p = ctx64(C, x, n, (double)mp->D);
    const double pmag = hypot(p.re, p.im);
    g->alpha = 1.0 / pmag;
    if (!ok || !(pmag > 0.0) || !isfinite(pmag)) return -1;
    return 0;
}

static void allmargin64_one(const oc_cfg* c, const oc_der* d, const oc_mp* mp, const oc_grid64* g,
                            const double* lina, const float* row, float* out) {
    const int NS = c->ns, nt = d->nt;
    float* sc = out + d->info_scoring;
    float* am = out + d->info_allmargin;
    const float UN = c->unstable_err, EF = c->eig_fail_err;
    const float sc0 = sc[0];
    if (sc0 >= UN) {
        sc[1] = sc0;
        sc[2] = sc0;
        am[0] = am[1] = am[2] = am[3] = am[4] = 0.0f;
        return;
    }
    double OA[MS * MS], K[MS], L[MS];
    for (int i = 0; i < NS; i++) {
        for (int j = 0; j < NS; j++) OA[i * NS + j] = lina[i * nt + j];
        K[i] = row[i];
        L[i] = row[NS + i];
    }
    /* nominal closed loop from the double OPEN_A */
    {
        double T[MT * MT], wr[MT], wi[MT];
        const int n2 = 2 * NS;
        for (int i = 0; i < NS; i++)
            for (int j = 0; j < NS; j++) {
                T[i * MT + j] = OA[i * NS + j] - ((double)mp->D * L[i]) * K[j];
                T[i * MT + NS + j] = -(L[i] * (double)mp->C[j]);
                T[(NS + i) * MT + j] = (double)mp->B[i] * K[j];
                T[(NS + i) * MT + NS + j] = (double)mp->A[i * NS + j];
            }
        int stable = eig_any(T, n2, wr, wi);
        if (stable)
            for (int i = 0; i < n2; i++)
                if (hypot(wr[i], wi[i]) >= 1.0) {
                    stable = 0;
                    break;
                }
        if (!stable) {
            sc[1] = sc0;
            sc[2] = UN;
            am[0] = am[1] = am[2] = am[3] = am[4] = 0.0f;
            const float total = logf(sc0 + UN + LFLOOR);
            sc[0] = isfinite(total) ? total : EF;
            return;
        }
    }
    const double PI = 3.141592653589793238462643, TWO_PI = 2.0 * PI, R2D = 180.0 / PI, D2R = PI / 180.0;
    const double TS = d->ts;
    double PM = FLT_MAX, GM = FLT_MAX, DM = FLT_MAX, BPC = 1.0;
    int crossed = 0, ok = 1;
    double prevMag = 0.0, prevPhase = 0.0, prevRaw = 0.0, prevTheta = 0.0;
    for (int w = 0; w < c->freq; w++) {
        if (!g->pok[w]) {
            ok = 0;
            break;
        }
        const cd z = {g->z[2 * w], g->z[2 * w + 1]};
        cd x[MS];
        if (!lu64_solve(z, OA, L, NS, x)) {
            ok = 0;
            break;
        }
        cd G = ctx64(K, x, NS, 0.0);
        const cd P = {g->pr[2 * w], g->pr[2 * w + 1]};
        const cd resp = cmul64(P, G);
        const double mg = hypot(resp.re, resp.im);
        const double raw = atan2(resp.im, resp.re);
        const double theta = g->th[w];
        {
            const double Ps = g->alpha * g->pm[w], Cs = hypot(G.re, G.im) / g->alpha;
            const double num = hypot(1.0 + resp.re, resp.im);
            const double den = sqrt(1.0 + Ps * Ps) * sqrt(1.0 + Cs * Cs);
            BPC = fmin(BPC, num / den);
        }
        if (w > 0) {
            double delta = raw - prevRaw;
            if (delta > PI) delta = delta - TWO_PI;
            else if (delta < -PI) delta = delta + TWO_PI;
            const double ph = prevPhase + delta;
            if ((prevMag - 1.0) * (mg - 1.0) <= 0.0 && mg != prevMag) {
                const double frac = (1.0 - prevMag) / (mg - prevMag);
                const double phase_c = prevPhase + frac * (ph - prevPhase);
                crossed = 1;
                double pm_deg = 180.0 + phase_c * R2D;
                pm_deg = pm_deg - 360.0 * floor((pm_deg + 180.0) / 360.0);
                PM = fmin(PM, pm_deg);
                const double theta_c = prevTheta + frac * (theta - prevTheta);
                const double pm_rad_c = pm_deg * D2R;
                if (theta_c > (double)TINY6 && pm_rad_c >= 0.0) DM = fmin(DM, ((pm_rad_c / theta_c) * TS) * 1000.0);
            }
            {
                const double a = prevPhase + PI, b = ph + PI;
                const int ka = (int)floor(a / TWO_PI), kb = (int)floor(b / TWO_PI);
                if (ka != kb && b != a) {
                    const double target = TWO_PI * (double)(b > a ? kb : ka);
                    const double frac = (target - a) / (b - a);
                    const double magp = prevMag + frac * (mg - prevMag);
                    GM = fmin(GM, -20.0 * log10(magp));
                }
            }
            prevPhase = ph;
        } else {
            prevPhase = raw;
        }
        prevMag = mg;
        prevRaw = raw;
        prevTheta = theta;
    }
    if (!ok) {
        sc[1] = sc0;
        sc[2] = EF;
        sc[0] = EF;
        am[0] = 0.0f; am[1] = 0.0f; am[2] = 0.0f; am[3] = 1.0f; am[4] = 0.0f;
        return;
    }
    const double TGM = c->target_gm, TPM = c->target_pm, TB = c->target_b;
    const double egm = fmax(0.0, TGM - GM) / TGM;
    const double epm = crossed ? fmax(0.0, TPM - PM) / TPM : 0.0;
    const double eb = fmax(0.0, TB - BPC) / TB;
    const float merr32 = (float)((egm * egm + epm * epm) + eb * eb);
    sc[1] = sc0;
    sc[2] = merr32;
    am[0] = (float)GM;
    am[1] = (float)PM;
    am[2] = (float)DM;
    am[3] = 1.0f;
    am[4] = (float)BPC;
    const float total = logf(sc0 + merr32 + LFLOOR);
    sc[0] = isfinite(total) ? total : EF;
}

/* One round in the plain FP64 form; info is in/out (n x info_w); the double
   intermediates go to the outputs that are not NULL: ywin (n x fit_steps),
   summ (n x 3), lina (n x nt^2), eig (n x 2nt), ata (n x (2nt)^2), atb (n x 2nt).
   Returns 0, a decode error (1 + digit) or -1 (alpha failure). */
int oracle64_evaluate(const oc_cfg* c, const oc_plant* p, int64_t n, const float* cuda_mx, float* info,
                      double* ywin_out, double* summ_out, double* lina_out, double* eig_out, double* ata_out,
                      double* atb_out, int threads) {
    oc_der d;
    derive(c, &d);
    oc_pp P;
    int rc = pad_plant(c, p, &P);
    if (rc) return rc;
    const int nt = d.nt;
    const int fit_steps = d.fit_len > 0.0f ? (int)ceilf(d.fit_len) : 0;
    oc_mp mp;
    margin_plant(c, p, &mp);
    oc_grid64 g;
    const int F = c->freq;
    g.F = F;
    g.z = (double*)malloc(sizeof(double) * 2 * F);
    g.th = (double*)malloc(sizeof(double) * F);
    g.pr = (double*)malloc(sizeof(double) * 2 * F);
    g.pm = (double*)malloc(sizeof(double) * F);
    g.pok = (int*)malloc(sizeof(int) * F);
    rc = plant_grid64(c, &d, &mp, &g);
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
    for (int64_t k = 0; k < n; k++) {
        double ywin[fit_steps > 0 ? fit_steps : 1], summ[3];
        double lina[MT * MT], T[MT * MT], wr[MT], wi[MT], eig[2 * MT];
        double ata[4 * MT * MT], atb[2 * MT];
        const float* row = cuda_mx + k * d.cuda_w;
        float* out = info + k * d.info_w;
        sim64_one(c, &d, &P, row, fit_steps, ywin, summ);
        lina64_one(c, &P, row, lina);
        for (int i = 0; i < nt; i++)
            for (int j = 0; j < nt; j++) T[i * MT + j] = lina[i * nt + j];
        eig_any(T, nt, wr, wi);
        for (int i = 0; i < nt; i++) {
            eig[2 * i] = wr[i];
            eig[2 * i + 1] = wi[i];
        }
        /* the modal setup runs for every candidate (a pre-flagged one included:
           ref: src/modalsetup.cu:18-26); the modal solve skips the flagged ones */
        modalsetup64_one(c, &d, fit_steps, ywin, summ, eig, ata, atb, out);
        modalsolve64_one(c, &d, ata, atb, eig, out);
        if (rc == 0) allmargin64_one(c, &d, &mp, &g, lina, row, out);
        if (ywin_out)
            for (int w = 0; w < fit_steps; w++) ywin_out[k * fit_steps + w] = ywin[w];
        if (summ_out)
            for (int e = 0; e < 3; e++) summ_out[k * 3 + e] = summ[e];
        if (lina_out)
            for (int e = 0; e < nt * nt; e++) lina_out[k * nt * nt + e] = lina[e];
        if (eig_out)
            for (int e = 0; e < 2 * nt; e++) eig_out[k * 2 * nt + e] = eig[e];
        if (ata_out)
            for (int e = 0; e < 4 * nt * nt; e++) ata_out[k * 4 * nt * nt + e] = ata[e];
        if (atb_out)
            for (int e = 0; e < 2 * nt; e++) atb_out[k * 2 * nt + e] = atb[e];
    }
    free(g.z);
    free(g.th);
    free(g.pr);
    free(g.pm);
    free(g.pok);
    return rc;
}
