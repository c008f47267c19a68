/*
 * ce_oracle.c -- CPU oracle of the ControllerEngine tuning path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the reference's
 * algorithm for one round of RunControllerEngine (ref: src/main.cu:402-559):
 * simulation, LIN_A, FP64 eigensolve, modal setup, modal solve and the
 * margin sweep.  It is the checker the parity tests and bench.py's CPU
 * baseline use; the library never links or calls it.
 *
 * It follows the reference's code structure, not the GPU kernels': every loop
 * runs over the padded MAX dimensions (8 / 8 / 4) exactly as the reference's
 * kernels do, the interpreter walks SKIP rows, the overshoot is the running
 * max of y*yss, and AtA is accumulated as a full 2nt x 2nt array.  Roundings:
 * fmaf() wherever the reference calls __fmaf_rn or where nvcc contracts a
 * multiply-add in the reference kernels (modalsetup: the exponent argument and
 * the AtA/Atb updates); separate multiply and add everywhere else.  Build with
 * -ffp-contract=off.
 *
 * The three Eigen stages restate the published algorithms of the reference's
 * (absent, unpinned) dependency Eigen: EigenSolver<double> (Householder
 * Hessenberg + Francis double-shift QR, EISPACK hqr), LDLT<Lower> with
 * symmetric pivoting, PartialPivLU<complex<float>>.  Sums inside those are
 * accumulated in index order; Eigen's vectorised kernels may round
 * differently in the last bits, so parity with the reference there is to a
 * tolerance, not bitwise.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MS 8   /* MAX_STATESPACE_DIM */
#define MD 8   /* MAX_DISCRETE_DIM */
#define MW 4   /* MAX_NONLIN_DIM */
#define MT 16  /* MAX_TOTAL_DIM */
#define MNL 9  /* MAX_NL_DIM */
#define MDC 4
#define MU 4
#define MNLI 8
#define MP 34

static const float PI_F = 0x1.921fb6p+1f;
static const float TINY6 = 0x1.0c6f7ap-20f;
static const float SENT = 0x1.2a05f2p+33f;
static const float LFLOOR = 0x1.a484cp-100f;

/* raw config values (the keys of ControllerEngine.config) */
typedef struct oc_cfg {
    int32_t ns, nd, nw, n_params, input_size, dc_instr, u_instr, nl_instr[4];
    int32_t serial, time;
    float duration;
    double ref_step_time;
    float ref_amplitude, fit_start, fit_end, steady_start;
    float bandwidth, damping, overshoot, sse, crossover_coeff, target_gm, target_pm, target_b;
    float eig_fail_err, unstable_err;
    int32_t freq;
    float freq_min, freq_max_key;
    int32_t observer; /* 0 Luenberger, 1 time-varying Kalman (key `observer`) */
} oc_cfg;

/* one round's plant, compact row-major as in the .bin files */
typedef struct oc_plant {
    const float *ss_a, *ss_ai, *ss_b, *ss_c, *ss_d;
    const float *d_a, *d_ai, *d_bu, *d_bw, *d_c, *base_params;
    const int32_t *dc_info, *u_info, *nl_info;
} oc_plant;

typedef struct oc_ins {
    int op, col, akind, bkind;
    float aval, bval;
} oc_ins;

/* derived values (ref: src/config.cu:40-78, 99-100) */
typedef struct oc_der {
    float ts, freq_max, fit_t0, fit_t1, crossover;
    int nt, cuda_w, info_scoring, info_freqresp, info_allmargin, info_modal, info_w;
    int fit_start_id, steady_start_id;
    float fit_len;
} oc_der;

static void derive(const oc_cfg* c, oc_der* d) {
    d->ts = c->duration / (float)c->time;
    d->freq_max = c->freq_max_key > 0.0f ? c->freq_max_key : PI_F / d->ts;
    d->nt = c->ns + c->nd;
    d->cuda_w = c->observer ? 3 * c->ns + 2 : 2 * c->ns + 1;
    d->info_scoring = c->input_size;
    d->info_freqresp = d->info_scoring + 3;
    d->info_allmargin = d->info_freqresp + 4;
    d->info_modal = d->info_allmargin + 5;
    d->info_w = d->info_modal + 3 * d->nt + 1;
    d->fit_t0 = c->fit_start * c->duration;
    d->fit_t1 = (c->fit_end * (float)c->time - 1.0f) * d->ts;
    {
        const float d2 = c->damping * c->damping, d4 = d2 * d2;
        const float wn = 2.0f * PI_F * c->bandwidth / sqrtf((1.0f - 2.0f * d2) + sqrtf(4.0f * d4 - 4.0f * d2 + 2.0f));
        d->crossover = c->crossover_coeff * wn * sqrtf(sqrtf(4.0f * d4 + 1.0f) - 2.0f * d2);
    }
    d->fit_start_id = (int)(c->fit_start * (float)c->time);
    d->steady_start_id = (int)(c->steady_start * (float)c->time);
    d->fit_len = (c->fit_end - c->fit_start) * (float)c->time;
}

/* ---- decode (ref: src/main.cu:317-337) ---------------------------------- */
/* returns 0, or 1 + the offending digit if a digit needs a missing BASE_PARAMS entry */
int oracle_decode(const int32_t* info, int dim, int count, const float* bp, int n_params, oc_ins* out) {
    for (int r = 0; r < count; r++) {
        const int32_t* row = &info[(size_t)r * dim];
        int packed = 0, col = 0;
        for (int c = 0; c < dim; c++)
            if (row[c] != 0) {
                packed = row[c];
                col = c;
            }
        out[r].op = 0;
        out[r].col = 0;
        out[r].akind = 0;
        out[r].bkind = 0;
        out[r].aval = 0.0f;
        out[r].bval = 0.0f;
        if (packed == 0) continue;
        int dg[2] = {(packed / 36) % 36, packed % 36};
        int kinds[2];
        float vals[2];
        for (int k = 0; k < 2; k++) {
            const int g = dg[k];
            kinds[k] = g == 0 ? 1 : (g == 35 ? 2 : 0);
            if (g == 0 || g == 35) vals[k] = 0.0f;
            else {
                if (g - 1 >= n_params) return 1 + g;
                vals[k] = g < 1 ? 0.0f : bp[g - 1];
            }
        }
        out[r].op = packed / 1296;
        out[r].col = col;
        out[r].akind = kinds[0];
        out[r].bkind = kinds[1];
        out[r].aval = vals[0];
        out[r].bval = vals[1];
    }
    return 0;
}

/* ---- padded plant, as the reference's __constant__ tables ---------------- */
typedef struct oc_pp {
    float ss_a[MS * MS], ss_ai[MS * MS], ss_b[MS], ss_c[MS], ss_d;
    float d_a[MD * MD], d_ai[MD * MD], d_bu[MD], d_bw[MD * MW], d_c[MD];
    oc_ins dc[MDC], u[MU], nl[MW * MNLI];
} oc_pp;

static int pad_plant(const oc_cfg* c, const oc_plant* p, oc_pp* P) {
    memset(P, 0, sizeof(*P));
    const int ns = c->ns, nd = c->nd, nw = c->nw;
    for (int i = 0; i < ns; i++) {
        for (int j = 0; j < ns; j++) {
            P->ss_a[i * MS + j] = p->ss_a[i * ns + j];
            P->ss_ai[i * MS + j] = p->ss_ai[i * ns + j];
        }
        P->ss_b[i] = p->ss_b[i];
        P->ss_c[i] = p->ss_c[i];
    }
    P->ss_d = p->ss_d[0];
    for (int i = 0; i < nd; i++) {
        for (int j = 0; j < nd; j++) {
            P->d_a[i * MD + j] = p->d_a[i * nd + j];
            P->d_ai[i * MD + j] = p->d_ai[i * nd + j];
        }
        P->d_bu[i] = p->d_bu[i];
        for (int k = 0; k < nw; k++) P->d_bw[i * MW + k] = p->d_bw[i * nw + k];
        P->d_c[i] = p->d_c[i];
    }
    int rc = oracle_decode(p->dc_info, nd, c->dc_instr, p->base_params, c->n_params, P->dc);
    if (rc) return rc;
    rc = oracle_decode(p->u_info, ns, c->u_instr, p->base_params, c->n_params, P->u);
    if (rc) return rc;
    for (int i = 0, row = 0; i < nw; row += c->nl_instr[i], i++) {
        oc_ins* chain = &P->nl[i * MNLI];
        rc = oracle_decode(&p->nl_info[(size_t)row * (nd + 1)], nd + 1, c->nl_instr[i], p->base_params, c->n_params, chain);
        if (rc) return rc;
        for (int r = 0; r < c->nl_instr[i]; r++)
            if (chain[r].col == nd) chain[r].col = MD;
    }
    return 0;
}

/* ---- interpreter (ref: src/main.cu:260-291) ------------------------------- */
static float interp(const oc_ins* info, int count, const float* src, int dim, int has_seed, float seed) {
    float result = 0.0f;
    int started = 0;
    for (int r = 0; r < count; r++) {
        const oc_ins in = info[r];
        if (in.op == 0) continue;
        float pos = 0.0f;
        for (int c = 0; c < dim; c++)
            if (c == in.col) pos = src[c];
        const float prev = started ? result : ((has_seed && !isnan(seed)) ? seed : pos);
        const float a = in.akind == 0 ? in.aval : (in.akind == 1 ? pos : prev);
        const float b = in.bkind == 0 ? in.bval : (in.bkind == 1 ? pos : prev);
        switch (in.op) {
            case 1: result = a + b; break;
            case 2: result = a - b; break;
            case 3: result = a * b; break;
            case 4: result = a / b; break;
            case 5: result = fminf(fmaxf(prev, a), b); break;
            case 6: result = (float)((0 < a) - (a < 0)); break;
            default: break;
        }
        started = 1;
    }
    return result;
}

static float vdot(const float* a, const float* b, int n, float acc) {
    for (int k = 0; k < n; k++) acc = fmaf(a[k], b[k], acc);
    return acc;
}

static void dfadd(float* HI, float* LO, float hi, float lo) {
    const float sh = *HI + hi;
    const float b0 = sh - *HI;
    const float sl = (*HI - (sh - b0)) + (hi - b0);
    const float v = (*LO + lo) + sl;
    *HI = sh + v;
    *LO = v - (*HI - sh);
}

/* ---- simulation (ref: src/discrete_solves.cu:12-79), one candidate -------- */
static void sim_one(const oc_cfg* c, const oc_der* d, const oc_pp* P, const float* row, float* y_out) {
    const int n = c->ns;
    float K[MS] = {0}, L[MS] = {0};
    for (int i = 0; i < MS; i++) {
        K[i] = i < n ? row[i] : 0.0f;
        L[i] = i < n ? row[n + i] : 0.0f;
    }
    const float N = row[2 * n];
    float xh_hi[MS] = {0}, xh_lo[MS] = {0}, xp_hi[MD] = {0}, xp_lo[MD] = {0};
    for (int t = 0; t < c->time; t++) {
        const float y = interp(P->dc, MDC, xp_hi, MD, 0, 0.0f);
        y_out[t] = y;
        const float ref = ((double)t < c->ref_step_time * (double)c->time) ? 0.0f : c->ref_amplitude;
        const float kx = vdot(K, xh_lo, MS, vdot(K, xh_hi, MS, 0.0f));
        const float u_raw = fmaf(N, ref, -kx);
        const float u = interp(P->u, MU, xh_hi, MS, 1, u_raw);
        const float yhat = fmaf(P->ss_d, u, vdot(P->ss_c, xh_lo, MS, vdot(P->ss_c, xh_hi, MS, 0.0f)));
        const float yerr = y - yhat;
        float dh[MS], dl[MS];
        for (int i = 0; i < MS; i++) {
            const float base = fmaf(L[i], yerr, P->ss_b[i] * u);
            dh[i] = vdot(&P->ss_ai[i * MS], xh_hi, MS, base);
            dl[i] = vdot(&P->ss_ai[i * MS], xh_lo, MS, 0.0f);
        }
        for (int i = 0; i < MS; i++) dfadd(&xh_hi[i], &xh_lo[i], dh[i], dl[i]);
        float src[MNL];
        for (int i = 0; i < MD; i++) src[i] = xp_hi[i];
        src[MD] = y;
        float W[MW];
        for (int i = 0; i < MW; i++) W[i] = interp(&P->nl[i * MNLI], MNLI, src, MNL, 0, 0.0f);
        float ph[MD], pl[MD];
        for (int i = 0; i < MD; i++) {
            const float base = vdot(&P->d_bw[i * MW], W, MW, P->d_bu[i] * u);
            ph[i] = vdot(&P->d_ai[i * MD], xp_hi, MD, base);
            pl[i] = vdot(&P->d_ai[i * MD], xp_lo, MD, 0.0f);
        }
        for (int i = 0; i < MD; i++) dfadd(&xp_hi[i], &xp_lo[i], ph[i], pl[i]);
    }
}

/* ---- Kalman observer simulation (ref: src/discrete_solves.cu:83-185) ------
   The reference's discrete_solve<Kalman>, restated with three changes:
   - the row is [K(ns), L(ns), N, R, Q(ns)] (3ns+2 floats; the Luenberger row
     [K, L, N] followed by the noise weights), where the reference reads
     [K, N, R, Q] (2ns+2 floats) from a row 2ns+1 wide, one float into the
     next candidate's row (:88-95 against src/config.cu:51);
   - the Joseph product (I - KG C) P (I - KG C)^T goes to its own buffer; the
     reference passes IKHP as both the left factor and the output of ABATf
     (:160), so its rows are overwritten while still being read;
   - 1/(C P C^T + R) is the correctly rounded quotient; the reference calls
     the approximate __fdividef (:136), whose last bits are not specified.
   Everything else -- the 8-wide padded loops, the fma chains in k order from
   0, the rounded (not fused) products -- is the reference's.  `literal` = 1
   instead runs the reference's row layout [K, N, R, Q] and its in-place
   Joseph product in source order (each element written before the next is
   read), for checking this restatement against the reference's own kernel. */
/* out = (A B) A^T over the padded 8 x 8 arrays (ref: src/main.cu:190-212, ABATf<8,8>);
   out may be B.  abat8_inplace_a writes the result over A, each element as
   soon as it is formed, as the reference's source does for ABATf(IKHP,P,IKHP). */
static void abat8(const float* A, const float* B, float* out) {
    float C0[MS * MS];
    for (int i = 0; i < MS; i++)
        for (int j = 0; j < MS; j++) {
            float c = 0.0f;
            for (int k = 0; k < MS; k++) c = fmaf(A[i * MS + k], B[k * MS + j], c);
            C0[i * MS + j] = c;
        }
    float R[MS * MS];
    for (int i = 0; i < MS; i++)
        for (int j = 0; j < MS; j++) {
            float c = 0.0f;
            for (int k = 0; k < MS; k++) c = fmaf(C0[i * MS + k], A[j * MS + k], c);
            R[i * MS + j] = c;
        }
    memcpy(out, R, sizeof(R));
}

static void abat8_inplace_a(float* A, const float* B) {
    float C0[MS * MS];
    for (int i = 0; i < MS; i++)
        for (int j = 0; j < MS; j++) {
            float c = 0.0f;
            for (int k = 0; k < MS; k++) c = fmaf(A[i * MS + k], B[k * MS + j], c);
            C0[i * MS + j] = c;
        }
    for (int i = 0; i < MS; i++)
        for (int j = 0; j < MS; j++) {
            float c = 0.0f;
            for (int k = 0; k < MS; k++) c = fmaf(C0[i * MS + k], A[j * MS + k], c);
            A[i * MS + j] = c;
        }
}

static void sim_kalman_one(const oc_cfg* c, const oc_pp* P, const float* row, float* y_out, int literal,
                           int* steady_step) {
    const int n = c->ns;
    float K[MS] = {0}, Q[MS] = {0};
    const int oN = literal ? n : 2 * n;
    for (int i = 0; i < MS; i++) {
        K[i] = i < n ? row[i] : 0.0f;
        Q[i] = i < n ? row[oN + 2 + i] : 0.0f;
    }
    const float N = row[oN], R = row[oN + 1];
    float xh_hi[MS] = {0}, xh_lo[MS] = {0}, xp_hi[MD] = {0}, xp_lo[MD] = {0};
    float Pm[MS * MS] = {0}, KG[MS] = {0}, PHT[MS], IKHP[MS * MS], J[MS * MS], C0[MS];
    if (steady_step) *steady_step = -1;
    for (int t = 0; t < c->time; t++) {
        const float y = interp(P->dc, MDC, xp_hi, MD, 0, 0.0f);
        y_out[t] = y;
        const float ref = ((double)t < c->ref_step_time * (double)c->time) ? 0.0f : c->ref_amplitude;
        const float kx = vdot(K, xh_lo, MS, vdot(K, xh_hi, MS, 0.0f));
        const float u_raw = fmaf(N, ref, -kx);
        const float u = interp(P->u, MU, xh_hi, MS, 1, u_raw);
        /* prediction: xh += (A-I) xh + B u */
        float dh[MS], dl[MS];
        for (int i = 0; i < MS; i++) {
            dh[i] = vdot(&P->ss_ai[i * MS], xh_hi, MS, P->ss_b[i] * u);
            dl[i] = vdot(&P->ss_ai[i * MS], xh_lo, MS, 0.0f);
        }
        for (int i = 0; i < MS; i++) dfadd(&xh_hi[i], &xh_lo[i], dh[i], dl[i]);
        float P0[MS * MS];
        memcpy(P0, Pm, sizeof(Pm));
        /* P = A P A^T + diag(Q) */
        abat8(P->ss_a, Pm, Pm);
        for (int i = 0; i < MS; i++) Pm[i * MS + i] = Pm[i * MS + i] + Q[i];
        /* gain: PHT = P C^T, HPHR = 1/(C P C^T + R), KG = PHT HPHR */
        for (int i = 0; i < MS; i++) PHT[i] = vdot(&Pm[i * MS], P->ss_c, MS, 0.0f);
        for (int j = 0; j < MS; j++) {
            float a = 0.0f;
            for (int k = 0; k < MS; k++) a = fmaf(P->ss_c[k], Pm[k * MS + j], a);
            C0[j] = a;
        }
        const float hphr = 1.0f / (vdot(C0, P->ss_c, MS, 0.0f) + R);
        for (int i = 0; i < MS; i++) KG[i] = PHT[i] * hphr;
        /* correction: xh += KG (y - C xh) as double-float products */
        const float dzh = -1.0f * vdot(P->ss_c, xh_hi, MS, -y);
        const float dzl = -1.0f * vdot(P->ss_c, xh_lo, MS, 0.0f);
        for (int i = 0; i < MS; i++) {
            const float s = KG[i] * dzh;
            float e = fmaf(KG[i], dzh, -s);
            e = fmaf(KG[i], dzl, e);
            dfadd(&xh_hi[i], &xh_lo[i], s, e);
        }
        /* P = (I - KG C) P (I - KG C)^T + KG R KG^T, IKHP formed as the reference forms it */
        for (int i = 0; i < MS; i++)
            for (int j = 0; j < MS; j++) {
                float m = fmaf(KG[i], P->ss_c[j], 0.0f);
                if (i == j) m = m - 1.0f;
                IKHP[i * MS + j] = -m;
            }
        if (literal) {
            abat8_inplace_a(IKHP, Pm);
            memcpy(J, IKHP, sizeof(J));
        } else {
            abat8(IKHP, Pm, J);
        }
        for (int i = 0; i < MS; i++) {
            const float kr = fmaf(KG[i], R, 0.0f);
            for (int j = 0; j < MS; j++) Pm[i * MS + j] = J[i * MS + j] + fmaf(kr, KG[j], 0.0f);
        }
        if (steady_step && *steady_step < 0 && memcmp(P0, Pm, sizeof(Pm)) == 0) *steady_step = t;
        /* nonlinear terms and plant, as the Luenberger loop */
        float src[MNL];
        for (int i = 0; i < MD; i++) src[i] = xp_hi[i];
        src[MD] = y;
        float W[MW];
        for (int i = 0; i < MW; i++) W[i] = interp(&P->nl[i * MNLI], MNLI, src, MNL, 0, 0.0f);
        float ph[MD], pl[MD];
        for (int i = 0; i < MD; i++) {
            const float base = vdot(&P->d_bw[i * MW], W, MW, P->d_bu[i] * u);
            ph[i] = vdot(&P->d_ai[i * MD], xp_hi, MD, base);
            pl[i] = vdot(&P->d_ai[i * MD], xp_lo, MD, 0.0f);
        }
        for (int i = 0; i < MD; i++) dfadd(&xp_hi[i], &xp_lo[i], ph[i], pl[i]);
    }
}

/* ---- LIN_A (ref: src/eigensetup.cu:1-57), one candidate ------------------- */
static void lina_one(const oc_cfg* c, const oc_pp* P, const float* row, float* out) {
    const int ns = c->ns, nd = c->nd, nt = ns + nd;
    float K[MS] = {0}, L[MS] = {0};
    for (int i = 0; i < MS; i++) {
        K[i] = i < ns ? row[i] : 0.0f;
        L[i] = i < ns ? row[ns + i] : 0.0f;
    }
    float pbk[MS * MS], pdk[MS], pcpd[MS], lpc[MS * MS], bduk[MD * MS], A1[MS * MS], A2[MS * MD], A3[MD * MS];
    for (int i = 0; i < MS; i++)
        for (int j = 0; j < MS; j++) pbk[i * MS + j] = fmaf(P->ss_b[i], K[j], 0.0f);
    for (int j = 0; j < MS; j++) pdk[j] = fmaf(P->ss_d, K[j], 0.0f);
    for (int j = 0; j < MS; j++) pcpd[j] = P->ss_c[j] - pdk[j];
    for (int i = 0; i < MS; i++)
        for (int j = 0; j < MS; j++) lpc[i * MS + j] = fmaf(L[i], pcpd[j], 0.0f);
    for (int i = 0; i < MD; i++)
        for (int j = 0; j < MS; j++) bduk[i * MS + j] = fmaf(P->d_bu[i], K[j], 0.0f);
    for (int k = 0; k < MS * MS; k++) A1[k] = P->ss_a[k] - pbk[k] - lpc[k];
    for (int i = 0; i < MS; i++)
        for (int j = 0; j < MD; j++) A2[i * MD + j] = fmaf(L[i], P->d_c[j], 0.0f);
    for (int k = 0; k < MD * MS; k++) A3[k] = -bduk[k];
    for (int i = 0; i < ns; i++) {
        for (int j = 0; j < ns; j++) out[i * nt + j] = A1[i * MS + j];
        for (int j = 0; j < nd; j++) out[i * nt + ns + j] = A2[i * MD + j];
    }
    for (int i = 0; i < nd; i++) {
        for (int j = 0; j < ns; j++) out[(ns + i) * nt + j] = A3[i * MS + j];
        for (int j = 0; j < nd; j++) out[(ns + i) * nt + ns + j] = P->d_a[i * MD + j];
    }
}

/* ---- FP64 eigenvalues: Householder Hessenberg + Francis double-shift QR ---- */
static const double EPS_D = 2.220446049250313080847e-16;
/* the reference's arithmetic: every product and sum rounded (no contraction) */
#define EIGN(name) name
#define MAC(x, a, b) ((x) + (a) * (b))
#define NMAC(x, a, b) ((x) - (a) * (b))
#include "ce_oracle_eig.h"
#undef EIGN
#undef MAC
#undef NMAC
/* the fused form of the engine's eigensolves: each x +- a b one fma */
#define EIGN(name) name##_fused
#define MAC(x, a, b) fma((a), (b), (x))
#define NMAC(x, a, b) fma(-(a), (b), (x))
#include "ce_oracle_eig.h"
#undef EIGN
#undef MAC
#undef NMAC

static int g_eig_fused = 0;
void oracle_set_eig_fused(int fused) { g_eig_fused = fused; }
static int eig_any(double* T, int n, double* wr, double* wi) {
    return g_eig_fused ? oracle_eig_fused(T, n, wr, wi) : oracle_eig(T, n, wr, wi);
}

/* ---- modal setup (ref: src/modalsetup.cu:1-97), one candidate ------------- */
typedef struct oc_modes {
    float Re[MT], Im[MT], mr[2 * MT], max_mag;
    int unique, dup[MT];
} oc_modes;

static void modes_of(const float* eig, int nt, float ts, oc_modes* m) {
    m->max_mag = 0.0f;
    for (int i = 0; i < nt; i++) {
        const float re = eig[2 * i], im = eig[2 * i + 1];
        const float mag = hypotf(re, im);
        m->max_mag = fmaxf(m->max_mag, mag);
        m->Re[i] = logf(fmaxf(mag, LFLOOR)) / ts;
        m->Im[i] = atan2f(im, re) / ts;
    }
    float pr = SENT, pi = SENT;
    int unique = nt;
    for (int i = 0; i < nt; i++) {
        m->dup[i] = 0;
        if (fabsf(m->Re[i] - pr) < TINY6 && fabsf(fabsf(m->Im[i]) - fabsf(pi)) < TINY6) {
            m->dup[i] = 1;
            unique--;
        }
        pr = m->Re[i];
        pi = m->Im[i];
    }
    memset(m->mr, 0, sizeof(m->mr));
    unique = 0;
    for (int i = 0; i < nt; i++)
        if (!m->dup[i]) {
            m->mr[2 * unique] = m->Re[i];
            m->mr[2 * unique + 1] = fabsf(m->Im[i]);
            unique++;
        }
    m->unique = unique;
}

static void modalsetup_one(const oc_cfg* c, const oc_der* d, const float* yrow, const float* eig, float* ata,
                           float* atb, float* out) {
    const int nt = d->nt, w = 2 * nt;
    oc_modes m;
    modes_of(eig, nt, d->ts, &m);
    float* sc = out + d->info_scoring;
    memset(ata, 0, sizeof(float) * w * w);
    memset(atb, 0, sizeof(float) * w);
    if (m.max_mag > 1.0f) {
        sc[0] = c->unstable_err + logf(m.max_mag) / d->ts;
        sc[1] = sc[0];
        return;
    }
    const int unique = m.unique, nc = 2 * unique;
    float shift[MT] = {0};
    for (int e = 0; e < unique; e++) shift[e] = fmaxf(m.mr[2 * e] * d->fit_t0, m.mr[2 * e] * d->fit_t1);
    float yss = 0.0f;
    for (int t = d->steady_start_id; t < c->time; t++) yss += yrow[t];
    yss /= (float)(c->time - d->steady_start_id);
    float peak = 0.0f;
    for (int t = 0; t < c->time; t++) peak = fmaxf(peak, yrow[t] * yss);
    out[d->info_freqresp + 2] = peak / fmaxf(yss * yss, TINY6) - 1.0f;
    out[d->info_freqresp + 3] = yss;
    float coeffs[2 * MT] = {0};
    for (int t = 0; t < d->fit_len; t++) {
        const float tval = (float)(d->fit_start_id + t) * d->ts;
        for (int e = 0; e < unique; e++) {
            const float decay = expf(fmaf(m.mr[2 * e], tval, -shift[e]));
            coeffs[2 * e] = decay * cosf(m.mr[2 * e + 1] * tval);
            coeffs[2 * e + 1] = decay * sinf(m.mr[2 * e + 1] * tval);
        }
        const int idx = d->fit_start_id + t;
        const float y = (idx < c->time ? yrow[idx] : 0.0f) - yss;
        for (int i = 0; i < nc; i++) {
            for (int j = 0; j <= i; j++) ata[i * w + j] = fmaf(coeffs[i], coeffs[j], ata[i * w + j]);
            atb[i] = fmaf(coeffs[i], y, atb[i]);
        }
    }
}

/* ---- modal solve (ref: src/modalsolve.cu:1-108), one candidate ------------ */
static void ldlt_solve(float* A, int n, float* x) {
    /* A: n x n full symmetric (row stride n), overwritten; x: rhs in, solution out */
    int tr[2 * MT];
    float temp[2 * MT];
    int stop = 0;
    for (int k = 0; k < n && !stop; k++) {
        int p = k;
        float best = fabsf(A[k * n + k]);
        for (int i = k + 1; i < n; i++)
            if (fabsf(A[i * n + i]) > best) {
                best = fabsf(A[i * n + i]);
                p = i;
            }
        tr[k] = p;
        if (p != k) {
            for (int j = 0; j < k; j++) {
                const float t = A[k * n + j];
                A[k * n + j] = A[p * n + j];
                A[p * n + j] = t;
            }
            for (int i = p + 1; i < n; i++) {
                const float t = A[i * n + k];
                A[i * n + k] = A[i * n + p];
                A[i * n + p] = t;
            }
            {
                const float t = A[k * n + k];
                A[k * n + k] = A[p * n + p];
                A[p * n + p] = t;
            }
            for (int i = k + 1; i < p; i++) {
                const float t = A[i * n + k];
                A[i * n + k] = A[p * n + i];
                A[p * n + i] = t;
            }
        }
        if (k > 0) {
            for (int j = 0; j < k; j++) temp[j] = A[j * n + j] * A[k * n + j];
            float acc = 0.0f;
            for (int j = 0; j < k; j++) acc = acc + A[k * n + j] * temp[j];
            float col[2 * MT];
            for (int i = k + 1; i < n; i++) {
                float a2 = 0.0f;
                for (int j = 0; j < k; j++) a2 = a2 + A[i * n + j] * temp[j];
                col[i] = a2;
            }
            A[k * n + k] = A[k * n + k] - acc;
            for (int i = k + 1; i < n; i++) A[i * n + k] = A[i * n + k] - col[i];
        }
        const float akk = A[k * n + k];
        const int valid = fabsf(akk) > 0.0f;
        if (k == 0 && !valid) {
            for (int j = 0; j < n; j++) tr[j] = j;
            stop = 1;
        } else if (valid) {
            for (int i = k + 1; i < n; i++) A[i * n + k] = A[i * n + k] / akk;
        }
    }
    for (int k = 0; k < n; k++) {
        const float t = x[k];
        x[k] = x[tr[k]];
        x[tr[k]] = t;
    }
    for (int i = 0; i < n; i++)
        for (int s = i + 1; s < n; s++) x[s] = x[s] - x[i] * A[s * n + i];
    for (int i = 0; i < n; i++) {
        const float dd = A[i * n + i];
        x[i] = fabsf(dd) > FLT_MIN ? x[i] / dd : 0.0f;
    }
    for (int i = n - 1; i >= 0; i--)
        for (int s = 0; s < i; s++) x[s] = x[s] - A[i * n + s] * x[i];
    for (int k = n - 1; k >= 0; k--) {
        const float t = x[k];
        x[k] = x[tr[k]];
        x[tr[k]] = t;
    }
}

static void modalsolve_one(const oc_cfg* c, const oc_der* d, const float* ata, const float* atb, const float* eig,
                           float* out) {
    const int nt = d->nt, n = 2 * nt;
    float* sc = out + d->info_scoring;
    float* fr = out + d->info_freqresp;
    float* md = out + d->info_modal;
    if (sc[0] != 0.0f) return;
    oc_modes m;
    modes_of(eig, nt, d->ts, &m);
    if (m.max_mag > 1.0f) {
        sc[0] = c->unstable_err + logf(m.max_mag) / d->ts;
        sc[1] = sc[0];
        return;
    }
    float S[4 * MT * MT], cs[2 * MT], x[2 * MT];
    for (int i = 0; i < n; i++) {
        const float s = sqrtf(ata[i * n + i]);
        cs[i] = s > TINY6 ? s : 1.0f;
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            const float a = j <= i ? ata[i * n + j] : ata[j * n + i];
            S[i * n + j] = ((1.0f / cs[i]) * a) * (1.0f / cs[j]);
        }
    for (int i = 0; i < n; i++) x[i] = atb[i] / cs[i];
    ldlt_solve(S, n, x);
    for (int i = 0; i < n; i++) x[i] = x[i] / cs[i];
    float esum = 0.0f, logwn = 0.0f, zw = 0.0f;
    for (int e = 0; e < m.unique; e++) {
        const int id = 2 * e;
        const float c0 = x[id], c1 = x[id + 1];
        const float g00 = ata[id * n + id], g01 = ata[(id + 1) * n + id], g11 = ata[(id + 1) * n + id + 1];
        const float energy = c0 * c0 * g00 + 2.0f * c0 * c1 * g01 + c1 * c1 * g11;
        const float re = m.mr[id], im = m.mr[id + 1];
        const float wn_e = fmaxf(sqrtf(re * re + im * im), TINY6);
        md[id] = wn_e;
        md[id + 1] = -re / wn_e;
        md[2 * nt + e] = energy;
        if (im < TINY6) continue;
        esum += energy;
        logwn += energy * logf(wn_e);
        zw += energy * (-re / wn_e);
    }
    md[3 * nt] = (float)m.unique;
    float wn, zeta;
    if (esum <= TINY6) {
        wn = TINY6;
        zeta = 0.0f;
    } else {
        wn = expf(logwn / esum);
        zeta = zw / esum;
    }
    const float D = c->damping, d2 = D * D;
    const float twn = 2.0f * PI_F * c->bandwidth / sqrtf((1.0f - 2.0f * d2) + sqrtf(4.0f * d2 * d2 - 4.0f * d2 + 2.0f));
    float be = logf(wn / twn) * logf(wn / twn) + (zeta - D) * (zeta - D) / D / D;
    const float eos = fmaxf(0.0f, fr[2] - c->overshoot) / c->overshoot;
    be += eos * eos;
    const float ess = fmaxf(0.0f, fabsf(fr[3] / c->ref_amplitude - 1.0f) - c->sse) / c->sse;
    be += ess * ess;
    sc[0] = isfinite(be) ? be : c->eig_fail_err;
    sc[1] = sc[0];
    fr[0] = wn;
    fr[1] = zeta;
}

/* ---- complex float LU (PartialPivLU) ------------------------------------- */
typedef struct cf {
    float re, im;
} cf;
static cf cmulf_(cf a, cf b) {
    cf r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static cf csubf_(cf a, cf b) {
    cf r = {a.re - b.re, a.im - b.im};
    return r;
}
static cf cdivf_(cf a, cf b) {
    const float d = b.re * b.re + b.im * b.im;
    cf r = {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
    return r;
}

/* x = (z I - A)^{-1} b for the n x n row-major A; returns 1 if x is finite */
static int lu_solve(cf z, const float* A, const float* b, int n, cf* x) {
    cf M[MS][MS];
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            cf zi;
            if (i == j) {
                zi.re = z.re * 1.0f - z.im * 0.0f;
                zi.im = z.re * 0.0f + z.im * 1.0f;
            } else {
                zi.re = z.re * 0.0f - z.im * 0.0f;
                zi.im = z.re * 0.0f + z.im * 0.0f;
            }
            cf a = {A[i * n + j], 0.0f};
            M[i][j] = csubf_(zi, a);
        }
    int perm[MS];
    for (int k = 0; k < n; k++) {
        int p = k;
        float best = M[k][k].re * M[k][k].re + M[k][k].im * M[k][k].im;
        for (int i = k + 1; i < n; i++) {
            const float s = M[i][k].re * M[i][k].re + M[i][k].im * M[i][k].im;
            if (s > best) {
                best = s;
                p = i;
            }
        }
        perm[k] = p;
        if (best != 0.0f) {
            if (p != k)
                for (int j = 0; j < n; j++) {
                    const cf t = M[k][j];
                    M[k][j] = M[p][j];
                    M[p][j] = t;
                }
            for (int i = k + 1; i < n; i++) M[i][k] = cdivf_(M[i][k], M[k][k]);
        }
        for (int i = k + 1; i < n; i++)
            for (int j = k + 1; j < n; j++) M[i][j] = csubf_(M[i][j], cmulf_(M[i][k], M[k][j]));
    }
    for (int i = 0; i < n; i++) {
        x[i].re = b[i];
        x[i].im = 0.0f;
    }
    for (int k = 0; k < n; k++) {
        const cf t = x[k];
        x[k] = x[perm[k]];
        x[perm[k]] = t;
    }
    for (int i = 0; i < n; i++)
        for (int s = i + 1; s < n; s++) x[s] = csubf_(x[s], cmulf_(x[i], M[s][i]));
    for (int i = n - 1; i >= 0; i--) {
        x[i] = cdivf_(x[i], M[i][i]);
        for (int s = 0; s < i; s++) x[s] = csubf_(x[s], cmulf_(x[i], M[s][i]));
    }
    for (int i = 0; i < n; i++)
        if (!isfinite(x[i].re) || !isfinite(x[i].im)) return 0;
    return 1;
}

static cf ctx_(const float* C, const cf* x, int n, float D) {
    cf acc = {0.0f, 0.0f};
    for (int i = 0; i < n; i++) {
        const cf k = {C[i], 0.0f};
        const cf t = cmulf_(k, x[i]);
        acc.re = acc.re + t.re;
        acc.im = acc.im + t.im;
    }
    acc.re = acc.re + D;
    return acc;
}

/* ---- margins (ref: src/allmargin.cu:1-182) -------------------------------- */
typedef struct oc_margin_plant {
    int n;
    float A[MS * MS], B[MS], C[MS], D;
} oc_mp;

/* sweep grid + plant response: z (2F), theta (F), presp (2F), pmag (F), pok (F); returns 0 or -1 if alpha fails */
static int plant_grid(const oc_cfg* c, const oc_der* d, const oc_mp* mp, float* z, float* th, float* pr, float* pm,
                      int* pok, float* alpha) {
    const int F = c->freq;
    const float inc = (logf(d->freq_max) - logf(c->freq_min)) / (float)(F - 1);
    for (int w = 0; w < F; w++) {
        const float theta = expf(logf(c->freq_min) + inc * (float)w) * d->ts;
        const cf zz = {cosf(theta), sinf(theta)};
        cf x[MS];
        const int ok = lu_solve(zz, mp->A, mp->B, mp->n, x);
        cf p = {0.0f, 0.0f};
        if (ok) p = ctx_(mp->C, x, mp->n, mp->D);
        z[2 * w] = zz.re;
        z[2 * w + 1] = zz.im;
        th[w] = atan2f(zz.im, zz.re);
        pr[2 * w] = p.re;
        pr[2 * w + 1] = p.im;
        pm[w] = hypotf(p.re, p.im);
        pok[w] = ok;
    }
    const float t = d->crossover * d->ts;
    const cf zc = {1.0f * cosf(t), 1.0f * sinf(t)};
    cf x[MS];
    const int ok = lu_solve(zc, mp->A, mp->B, mp->n, x);
    const cf p = ctx_(mp->C, x, mp->n, mp->D);
    const float pmag = hypotf(p.re, p.im);
    *alpha = 1.0f / pmag;
    if (!ok || !(pmag > 0.0f) || !isfinite(pmag)) return -1;
    return 0;
}

static void allmargin_one(const oc_cfg* c, const oc_der* d, const oc_mp* mp, const float* z, const float* th,
                          const float* pr, const float* pm, const int* pok, float alpha, const float* lina,
                          const float* row, float* out) {
    const int NS = c->ns, nt = d->nt;
    float* sc = out + d->info_scoring;
    float* am = out + d->info_allmargin;
    const float UN = c->unstable_err, EF = c->eig_fail_err;
    if (sc[0] >= UN) {
        sc[1] = sc[0];
        sc[2] = sc[0];
        am[0] = am[1] = am[2] = am[3] = am[4] = 0.0f;
        return;
    }
    float OA[MS * MS], K[MS], L[MS];
    for (int i = 0; i < NS; i++) {
        for (int j = 0; j < NS; j++) OA[i * NS + j] = lina[i * nt + j];
        K[i] = row[i];
        L[i] = row[NS + i];
    }
    /* nominal closed loop, FP64 eigensolve */
    {
        double T[MT * MT];
        double wr[MT], wi[MT];
        const int n2 = 2 * NS;
        for (int i = 0; i < NS; i++)
            for (int j = 0; j < NS; j++) {
                T[i * MT + j] = (double)(OA[i * NS + j] - (mp->D * L[i]) * K[j]);
                T[i * MT + NS + j] = (double)(-(L[i] * mp->C[j]));
                T[(NS + i) * MT + j] = (double)(mp->B[i] * K[j]);
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
            sc[1] = sc[0];
            sc[2] = UN;
            am[0] = am[1] = am[2] = am[3] = am[4] = 0.0f;
            const float total = logf(sc[0] + UN + LFLOOR);
            sc[0] = isfinite(total) ? total : EF;
            return;
        }
    }
    float PM = FLT_MAX, GM = FLT_MAX, DM = FLT_MAX, BPC = 1.0f;
    int crossed = 0, ok = 1;
    float prevMag = 0.0f, prevPhase = 0.0f, prevRaw = 0.0f, prevTheta = 0.0f;
    for (int w = 0; w < c->freq; w++) {
        if (!pok[w]) {
            ok = 0;
            break;
        }
        const cf zz = {z[2 * w], z[2 * w + 1]};
        cf x[MS];
        if (!lu_solve(zz, OA, L, NS, x)) {
            ok = 0;
            break;
        }
        const cf G = ctx_(K, x, NS, 0.0f);
        const cf P = {pr[2 * w], pr[2 * w + 1]};
        const cf resp = cmulf_(P, G);
        const float mg = hypotf(resp.re, resp.im);
        const float raw = atan2f(resp.im, resp.re);
        const float theta = th[w];
        {
            const float Ps = alpha * pm[w], Cs = hypotf(G.re, G.im) / alpha;
            BPC = fminf(BPC, hypotf(1.0f + resp.re, resp.im) / (sqrtf(1.0f + Ps * Ps) * sqrtf(1.0f + Cs * Cs)));
        }
        if (w > 0) {
            float delta = raw - prevRaw;
            if (delta > PI_F) delta -= 2.0f * PI_F;
            else if (delta < -PI_F) delta += 2.0f * PI_F;
            const float ph = prevPhase + delta;
            if ((prevMag - 1.0f) * (mg - 1.0f) <= 0.0f && mg != prevMag) {
                const float frac = (1.0f - prevMag) / (mg - prevMag);
                const float phase_c = prevPhase + frac * (ph - prevPhase);
                crossed = 1;
                float pm_deg = 180.0f + phase_c * (180.0f / PI_F);
                pm_deg -= 360.0f * floorf((pm_deg + 180.0f) / 360.0f);
                PM = fminf(PM, pm_deg);
                const float theta_c = prevTheta + frac * (theta - prevTheta);
                const float pm_rad_c = pm_deg * (PI_F / 180.0f);
                if (theta_c > TINY6 && pm_rad_c >= 0.0f) DM = fminf(DM, (pm_rad_c / theta_c) * d->ts * 1000.0f);
            }
            {
                const float a = prevPhase + PI_F, b = ph + PI_F;
                const int ka = (int)floorf(a / (2.0f * PI_F)), kb = (int)floorf(b / (2.0f * PI_F));
                if (ka != kb && b != a) {
                    const float target = 2.0f * PI_F * (float)(b > a ? kb : ka);
                    const float frac = (target - a) / (b - a);
                    const float magp = prevMag + frac * (mg - prevMag);
                    GM = fminf(GM, -20.0f * log10f(magp));
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
        sc[1] = sc[0];
        sc[2] = EF;
        sc[0] = EF;
        am[0] = 0.0f; am[1] = 0.0f; am[2] = 0.0f; am[3] = 1.0f; am[4] = 0.0f;
        return;
    }
    const float egm = fmaxf(0.0f, c->target_gm - GM) / c->target_gm;
    const float epm = crossed ? fmaxf(0.0f, c->target_pm - PM) / c->target_pm : 0.0f;
    const float eb = fmaxf(0.0f, c->target_b - BPC) / c->target_b;
    const float merr = egm * egm + epm * epm + eb * eb;
    sc[1] = sc[0];
    sc[2] = merr;
    am[0] = GM;
    am[1] = PM;
    am[2] = DM;
    am[3] = 1.0f;
    am[4] = BPC;
    const float total = logf(sc[0] + merr + LFLOOR);
    sc[0] = isfinite(total) ? total : EF;
}

/* ===================== exported stage entry points ======================== */

void oracle_derived(const oc_cfg* c, oc_der* d) { derive(c, d); }

int oracle_info_width(const oc_cfg* c) {
    oc_der d;
    derive(c, &d);
    return d.info_w;
}

/* y: n x time */
int oracle_sim(const oc_cfg* c, const oc_plant* p, int64_t n, const float* cuda_mx, float* y, int threads) {
    oc_der d;
    derive(c, &d);
    oc_pp P;
    const int rc = pad_plant(c, p, &P);
    if (rc) return rc;
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
    for (int64_t k = 0; k < n; k++) {
        if (c->observer) sim_kalman_one(c, &P, cuda_mx + k * d.cuda_w, y + k * (int64_t)c->time, 0, NULL);
        else sim_one(c, &d, &P, cuda_mx + k * d.cuda_w, y + k * (int64_t)c->time);
    }
    return 0;
}

/* The Kalman loop in the reference's literal form (row [K, N, R, Q] of
   `width` floats, in-place Joseph product), or the engine's form (literal 0,
   rows of the config's width); steady[k] = first step whose covariance update
   left P bit for bit unchanged (-1: none). */
int oracle_sim_kalman(const oc_cfg* c, const oc_plant* p, int64_t n, const float* rows, int width, int literal,
                      float* y, int32_t* steady, int threads) {
    oc_pp P;
    const int rc = pad_plant(c, p, &P);
    if (rc) return rc;
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
    for (int64_t k = 0; k < n; k++)
        sim_kalman_one(c, &P, rows + k * width, y + k * (int64_t)c->time, literal, steady ? &steady[k] : NULL);
    return 0;
}

/* lina: n x nt*nt */
int oracle_lina(const oc_cfg* c, const oc_plant* p, int64_t n, const float* cuda_mx, float* lina, int threads) {
    oc_der d;
    derive(c, &d);
    oc_pp P;
    const int rc = pad_plant(c, p, &P);
    if (rc) return rc;
#pragma omp parallel for num_threads(threads)
    for (int64_t k = 0; k < n; k++) lina_one(c, &P, cuda_mx + k * d.cuda_w, lina + k * (int64_t)d.nt * d.nt);
    return 0;
}

/* eig: n x 2nt floats (re, im), or eig64 (doubles) when non-NULL */
void oracle_eigensolve(int64_t n, int nt, const float* lina, float* eig, double* eig64, int threads) {
#pragma omp parallel for num_threads(threads)
    for (int64_t k = 0; k < n; k++) {
        double T[MT * MT], wr[MT], wi[MT];
        for (int i = 0; i < nt; i++)
            for (int j = 0; j < nt; j++) T[i * MT + j] = (double)lina[k * nt * nt + i * nt + j];
        eig_any(T, nt, wr, wi);
        for (int i = 0; i < nt; i++) {
            if (eig) {
                eig[k * 2 * nt + 2 * i] = (float)wr[i];
                eig[k * 2 * nt + 2 * i + 1] = (float)wi[i];
            }
            if (eig64) {
                eig64[k * 2 * nt + 2 * i] = wr[i];
                eig64[k * 2 * nt + 2 * i + 1] = wi[i];
            }
        }
    }
}

/* eigenvalues of one general n x n double matrix (row-major), for tests */
int oracle_eig_matrix(const double* A, int n, double* wr, double* wi) {
    double T[MT * MT];
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) T[i * MT + j] = A[i * n + j];
    return eig_any(T, n, wr, wi);
}

/* info (in/out): n x info_w; y: n x time; ata: n x (2nt)^2; atb: n x 2nt */
void oracle_modalsetup(const oc_cfg* c, int64_t n, const float* y, const float* eig, float* ata, float* atb,
                       float* info, int threads) {
    oc_der d;
    derive(c, &d);
    const int nt = d.nt;
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
    for (int64_t k = 0; k < n; k++)
        modalsetup_one(c, &d, y + k * (int64_t)c->time, eig + k * 2 * nt, ata + k * 4 * nt * nt, atb + k * 2 * nt,
                       info + k * d.info_w);
}

void oracle_modalsolve(const oc_cfg* c, int64_t n, const float* ata, const float* atb, const float* eig, float* info,
                       int threads) {
    oc_der d;
    derive(c, &d);
    const int nt = d.nt;
#pragma omp parallel for num_threads(threads)
    for (int64_t k = 0; k < n; k++)
        modalsolve_one(c, &d, ata + k * 4 * nt * nt, atb + k * 2 * nt, eig + k * 2 * nt, info + k * d.info_w);
}

/* margin plant: batch -> statespace model, serial -> the true linear plant (D = 0) */
static void margin_plant(const oc_cfg* c, const oc_plant* p, oc_mp* mp) {
    const int n = c->serial ? c->nd : c->ns;
    mp->n = n;
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < n; j++) mp->A[i * n + j] = c->serial ? p->d_a[i * n + j] : p->ss_a[i * n + j];
        mp->B[i] = c->serial ? p->d_bu[i] : p->ss_b[i];
        mp->C[i] = c->serial ? p->d_c[i] : p->ss_c[i];
    }
    mp->D = c->serial ? 0.0f : p->ss_d[0];
}

/* returns 0, or -1 if the plant has no finite nonzero gain at the crossover */
int oracle_allmargin(const oc_cfg* c, const oc_plant* p, int64_t n, const float* lina, const float* cuda_mx,
                     float* info, int threads) {
    oc_der d;
    derive(c, &d);
    oc_mp mp;
    margin_plant(c, p, &mp);
    const int F = c->freq;
    float* z = (float*)malloc(sizeof(float) * 2 * F);
    float* th = (float*)malloc(sizeof(float) * F);
    float* pr = (float*)malloc(sizeof(float) * 2 * F);
    float* pm = (float*)malloc(sizeof(float) * F);
    int* pok = (int*)malloc(sizeof(int) * F);
    float alpha;
    const int rc = plant_grid(c, &d, &mp, z, th, pr, pm, pok, &alpha);
    if (rc == 0) {
#pragma omp parallel for schedule(dynamic, 8) num_threads(threads)
        for (int64_t k = 0; k < n; k++)
            allmargin_one(c, &d, &mp, z, th, pr, pm, pok, alpha, lina + k * d.nt * d.nt, cuda_mx + k * d.cuda_w,
                          info + k * d.info_w);
    }
    free(z);
    free(th);
    free(pr);
    free(pm);
    free(pok);
    return rc;
}

/* the plant response on the sweep grid (for tests of the host-side grid) */
int oracle_plant_grid(const oc_cfg* c, const oc_plant* p, float* z, float* th, float* pr, float* pm, int* pok,
                      float* alpha) {
    oc_der d;
    derive(c, &d);
    oc_mp mp;
    margin_plant(c, p, &mp);
    return plant_grid(c, &d, &mp, z, th, pr, pm, pok, alpha);
}

/* one full round; info is in/out (n x info_w); diagnostic outputs may be NULL.
   Returns 0, a decode error (1 + digit) or -1 (alpha failure). */
int oracle_evaluate(const oc_cfg* c, const oc_plant* p, int64_t n, const float* cuda_mx, float* info, float* y_out,
                    float* lina_out, float* eig_out, float* ata_out, float* atb_out, int threads) {
    oc_der d;
    derive(c, &d);
    const int nt = d.nt;
    float* y = y_out ? y_out : (float*)malloc(sizeof(float) * n * c->time);
    float* lina = lina_out ? lina_out : (float*)malloc(sizeof(float) * n * nt * nt);
    float* eig = eig_out ? eig_out : (float*)malloc(sizeof(float) * n * 2 * nt);
    float* ata = ata_out ? ata_out : (float*)malloc(sizeof(float) * n * 4 * nt * nt);
    float* atb = atb_out ? atb_out : (float*)malloc(sizeof(float) * n * 2 * nt);
    int rc = oracle_sim(c, p, n, cuda_mx, y, threads);
    if (!rc) rc = oracle_lina(c, p, n, cuda_mx, lina, threads);
    if (!rc) {
        oracle_eigensolve(n, nt, lina, eig, NULL, threads);
        oracle_modalsetup(c, n, y, eig, ata, atb, info, threads);
        oracle_modalsolve(c, n, ata, atb, eig, info, threads);
        rc = oracle_allmargin(c, p, n, lina, cuda_mx, info, threads);
    }
    if (!y_out) free(y);
    if (!lina_out) free(lina);
    if (!eig_out) free(eig);
    if (!ata_out) free(ata);
    if (!atb_out) free(atb);
    return rc;
}

/* the plain FP64 form of the method (the engine's CE_PRECISION_FP64) */
#include "ce_oracle64.h"
