// ce_k_sweep.cu -- loop frequency sweep, stability margins and the total score.
//
// Restates the per-candidate part of allmargin_fixed<NS>
// (ref: src/allmargin.cu:43-181): candidates flagged by the modal stage get
// zero margins; a nominal closed loop that the FP64 eigensolve finds unstable
// gets the unstable penalty; otherwise the compensator
// G(z) = K^T (zI - OPEN_A)^{-1} L is evaluated on the logspace grid by complex
// LU, the loop P*G is unwrapped in phase, gain crossovers give PM (and the delay
// margin), phase crossovers at odd multiples of pi give GM, b(w) =
// |1+PG| / (sqrt(1+|aP|^2) sqrt(1+|G/a|^2)) gives the Vinnicombe margin b_PC, and
// the margin error is added to the behaviour error in log form.
//
// The plant response P(z_w), |P(z_w)|, arg z_w and the plant scaling alpha are
// per-plant values computed once by the host (ref: src/allmargin.cu:20-41).
// One thread per candidate; OPEN_A lives in shared memory ([element][thread]),
// the LU works in registers with the dimension class NSC as its compile-time
// size (zero padding inside the class is exact: padded rows are decoupled
// z*I rows whose right-hand side is zero).
#include <cfloat>
#include <climits>

#include "ce_device.cuh"
#include "ce_host.h"

namespace ce {

constexpr int SWEEP_BLOCK = 64;
constexpr float TINY_E6 = 0x1.0c6f7ap-20f;
constexpr float LOGFLOOR = 0x1.a484cp-100f;

template <typename R> __device__ __forceinline__ R pi_();
template <> __device__ __forceinline__ float pi_<float>() { return 0x1.921fb6p+1f; }
template <> __device__ __forceinline__ double pi_<double>() { return 3.141592653589793238462643; }
__device__ __forceinline__ float rlog10(float x) { return log10f(x); }
__device__ __forceinline__ double rlog10(double x) { return log10(x); }
__device__ __forceinline__ float rlogf_(float x) { return logf(x); }
__device__ __forceinline__ double rlogf_(double x) { return log(x); }
__device__ __forceinline__ float rsqrtf_(float x) { return sqrtf(x); }
__device__ __forceinline__ double rsqrtf_(double x) { return sqrt(x); }

// Candidates that skip the sweep get their outputs here: flagged by the
// modal stage (zero margins), or a nominal closed loop that is not stable
// (the unstable penalty).  The rest are listed for k_sweep, so its warps hold
// only candidates that run the frequency loop.
template <bool RG = false>
__global__ void __launch_bounds__(128) k_sweep_select(const Run run_in, const int* __restrict__ nominal,
                                                      float* __restrict__ info, int* __restrict__ list,
                                                      int* __restrict__ count) {
    const int64_t c = (int64_t)blockIdx.x * 128 + threadIdx.x;
    if (c >= run_in.n) return;
    const Run& run = run_of<RG>(run_in, c);
    float* out = info + c * (int64_t)run.info_w;
    float* sc = out + run.info_scoring;
    float* am = out + run.info_allmargin;
    const float sc0 = sc[0];
    const float UNST = run.unstable_err, EIGF = run.eig_fail_err;
    if (sc0 >= UNST) {
        sc[1] = sc0;
        sc[2] = sc0;
        am[0] = am[1] = am[2] = am[3] = am[4] = 0.0f;
        return;
    }
    if (nominal[c] != 1) {
        sc[1] = sc0;
        sc[2] = UNST;
        am[0] = am[1] = am[2] = am[3] = am[4] = 0.0f;
        const float total = logf(__fadd_rn(__fadd_rn(sc0, UNST), LOGFLOOR));
        sc[0] = isfinite(total) ? total : EIGF;
        return;
    }
    list[atomicAdd(count, 1)] = (int)c;
}

// The sweep in two passes.  k_sweep_resp: one thread per (listed candidate,
// group of SWEEP_FG frequencies) solves the complex LU of every frequency of
// its group and stores |P G| and arg(P G) (layout [w][candidate]), the
// minimum of the b(w) terms and the first frequency that fails (no plant
// response or a non-finite solve).  k_sweep_scan: one thread per listed
// candidate walks the frequencies in order for the phase unwrap, the
// crossovers and the margins (ref: src/allmargin.cu:100-181).  Each value is
// computed with the same operations as in one sequential loop; the minimum
// is exact in any order, and the frequencies after the first failure, which
// the sequential loop never reaches, only feed values that the failure path
// discards.

// fgrid row per frequency: z.re, z.im, arg z, P.re, P.im, |P|, ok, 0
template <typename R, int NSC, bool RG = false>
__global__ void __launch_bounds__(SWEEP_BLOCK) k_sweep_resp(const Run run_in, const float* __restrict__ gains,
                                                            const R* __restrict__ lina,
                                                            const int* __restrict__ list, const int* __restrict__ count,
                                                            const R* __restrict__ fgrid, R* __restrict__ mag,
                                                            R* __restrict__ arg, R* __restrict__ bpc,
                                                            int* __restrict__ fail) {
    __shared__ R As[NSC * NSC][SWEEP_BLOCK];
    const int tid = threadIdx.x;
    const int64_t idx = (int64_t)blockIdx.x * SWEEP_BLOCK + tid;
    const int64_t listed = *count;
    if (idx >= listed) return;
    const int g = blockIdx.y;
    const int64_t c = list[idx];
    const Run& run = run_of<RG>(run_in, c);
    const int w0 = g * SWEEP_FG, w1 = min(run.freq, w0 + SWEEP_FG);
    const int ns = run.ns, nt = run.nt;
    const float* row = gains + c * run.cuda_w;
    const R* la = lina + c * (int64_t)run.lina_slot;  // OPEN_A = LIN_A[:ns, :ns]
    R K[NSC], L[NSC];
#pragma unroll
    for (int i = 0; i < NSC; ++i) {
        K[i] = i < ns ? R(row[i]) : R(0);
        L[i] = i < ns ? R(row[ns + i]) : R(0);
#pragma unroll
        for (int j = 0; j < NSC; ++j) As[i * NSC + j][tid] = (i < ns && j < ns) ? R(la[i * nt + j]) : R(0);
    }
    // per-candidate plants in serial mode: the candidate's own grid and scaling
    const bool own = run.mc.tab && run.mc.grid_stride;
    const int64_t pc = own ? mc_plant(run.mc, c) : 0;  // the candidate's plant
    const R ALPHA = own ? ((const R*)run.mc.alpha)[pc] : (sizeof(R) == 4 ? R(run.alpha) : R(run.alpha64));
    // the grid argument is the grid of plant mc.first
    const R* fgc = fgrid + run.grid_off + (own ? (pc - run.mc.first) * run.mc.grid_stride : 0);
    R bmin = R(1);
    int first_bad = INT_MAX;
    for (int w = w0; w < w1; ++w) {
        const R* fg = fgc + 8 * (int64_t)w;
        if (fg[6] == R(0)) {
            first_bad = w;
            break;
        }
        const cplx<R> z{fg[0], fg[1]};
        cplx<R> x[NSC];
        lu_solve_shifted<R, NSC>(z, &As[0][tid], SWEEP_BLOCK, L, x);
        bool fin = true;
#pragma unroll
        for (int i = 0; i < NSC; ++i) fin = fin && cfinite(x[i]);
        if (!fin) {
            first_bad = w;
            break;
        }
        cplx<R> G{R(0), R(0)};
#pragma unroll
        for (int i = 0; i < NSC; ++i) {
            const cplx<R> t = cmul(cplx<R>{K[i], R(0)}, x[i]);
            G = cplx<R>{radd(G.re, t.re), radd(G.im, t.im)};
        }
        G.re = radd(G.re, R(0));
        const cplx<R> P{fg[3], fg[4]};
        const cplx<R> resp = cmul(P, G);
        mag[(int64_t)w * listed + idx] = cabs_(resp);
        arg[(int64_t)w * listed + idx] = carg_(resp);
        const R Ps = rmul(ALPHA, fg[5]), Cs = rdiv(cabs_(G), ALPHA);
        const R num = cabs_(cplx<R>{radd(R(1), resp.re), resp.im});
        const R den = rmul(rsqrtf_(radd(R(1), rmul(Ps, Ps))), rsqrtf_(radd(R(1), rmul(Cs, Cs))));
        bmin = fmin(bmin, rdiv(num, den));
    }
    bpc[(int64_t)g * listed + idx] = bmin;
    fail[(int64_t)g * listed + idx] = first_bad;
}

template <typename R, bool RG = false>
__global__ void __launch_bounds__(128) k_sweep_scan(const Run run_in, const int* __restrict__ list,
                                                    const int* __restrict__ count, const R* __restrict__ fgrid,
                                                    const R* __restrict__ mag, const R* __restrict__ arg,
                                                    const R* __restrict__ bpc, const int* __restrict__ fail,
                                                    float* __restrict__ info) {
    const int64_t idx = (int64_t)blockIdx.x * 128 + threadIdx.x;
    const int64_t listed = *count;
    if (idx >= listed) return;
    const int64_t c = list[idx];
    const Run& run = run_of<RG>(run_in, c);
    float* out = info + c * (int64_t)run.info_w;
    float* sc = out + run.info_scoring;
    float* am = out + run.info_allmargin;
    const float sc0 = sc[0];
    const float EIGF = run.eig_fail_err;
    const R* fgc = fgrid + run.grid_off;
    const int groups = (run.freq + SWEEP_FG - 1) / SWEEP_FG;
    int first_bad = INT_MAX;
    R BPC = R(1);
    for (int g = 0; g < groups; ++g) {
        first_bad = min(first_bad, fail[(int64_t)g * listed + idx]);
        BPC = fmin(BPC, bpc[(int64_t)g * listed + idx]);
    }
    if (first_bad < run.freq) {
        sc[1] = sc0;
        sc[2] = EIGF;
        sc[0] = EIGF;
        am[0] = 0.0f; am[1] = 0.0f; am[2] = 0.0f; am[3] = 1.0f; am[4] = 0.0f;
        return;
    }
    const R PI = pi_<R>(), TWO_PI = rmul(R(2), PI), R2D = rdiv(R(180), PI), D2R = rdiv(PI, R(180));
    const R TS = R(run.ts);
    R PM = R(FLT_MAX), GM = R(FLT_MAX), DM = R(FLT_MAX);
    bool gain_crossed = false;
    R prevMag = R(0), prevPhase = R(0), prevRaw = R(0), prevTheta = R(0);
    for (int w = 0; w < run.freq; ++w) {
        const R m = mag[(int64_t)w * listed + idx];
        const R raw = arg[(int64_t)w * listed + idx];
        const R theta = fgc[8 * (int64_t)w + 2];
        if (w > 0) {
            R delta = rsub(raw, prevRaw);
            if (delta > PI) delta = rsub(delta, TWO_PI);
            else if (delta < -PI) delta = radd(delta, TWO_PI);
            const R ph = radd(prevPhase, delta);
            // gain crossover
            if (rmul(rsub(prevMag, R(1)), rsub(m, R(1))) <= R(0) && m != prevMag) {
                const R frac = rdiv(rsub(R(1), prevMag), rsub(m, prevMag));
                const R phase_c = radd(prevPhase, rmul(frac, rsub(ph, prevPhase)));
                gain_crossed = true;
                R pm_deg = radd(R(180), rmul(phase_c, R2D));
                pm_deg = rsub(pm_deg, rmul(R(360), floor(rdiv(radd(pm_deg, R(180)), R(360)))));
                PM = fmin(PM, pm_deg);
                const R theta_c = radd(prevTheta, rmul(frac, rsub(theta, prevTheta)));
                const R pm_rad_c = rmul(pm_deg, D2R);
                if (theta_c > R(TINY_E6) && pm_rad_c >= R(0)) DM = fmin(DM, rmul(rmul(rdiv(pm_rad_c, theta_c), TS), R(1000)));
            }
            // phase crossover at odd multiples of pi
            {
                const R a = radd(prevPhase, PI), b = radd(ph, PI);
                const int ka = (int)floor(rdiv(a, TWO_PI)), kb = (int)floor(rdiv(b, TWO_PI));
                if (ka != kb && b != a) {
                    const R target = rmul(TWO_PI, R(b > a ? kb : ka));
                    const R frac = rdiv(rsub(target, a), rsub(b, a));
                    const R mag_p = radd(prevMag, rmul(frac, rsub(m, prevMag)));
                    GM = fmin(GM, rmul(R(-20), rlog10(mag_p)));
                }
            }
            prevPhase = ph;
        } else {
            prevPhase = raw;
        }
        prevMag = m;
        prevRaw = raw;
        prevTheta = theta;
    }
    const R TGM = R(run.target_gm), TPM = R(run.target_pm), TB = R(run.target_b);
    const R egm = rdiv(fmax(R(0), rsub(TGM, GM)), TGM);
    const R epm = gain_crossed ? rdiv(fmax(R(0), rsub(TPM, PM)), TPM) : R(0);
    const R eb = rdiv(fmax(R(0), rsub(TB, BPC)), TB);
    const R merr = radd(radd(rmul(egm, egm), rmul(epm, epm)), rmul(eb, eb));
    const float merr32 = (float)merr;
    sc[1] = sc0;
    sc[2] = merr32;
    am[0] = (float)GM;
    am[1] = (float)PM;
    am[2] = (float)DM;
    am[3] = 1.0f;
    am[4] = (float)BPC;
    const float total = logf(__fadd_rn(__fadd_rn(sc0, merr32), LOGFLOOR));
    sc[0] = isfinite(total) ? total : EIGF;
}

template <typename R>
static void sweep_dispatch(const Run& run, const float* gains, const R* lina, const int* list, const int* count,
                           const R* fgrid, float* info, const SweepScratch& sw, cudaStream_t st) {
    // the listed count is only known on the device: grids cover all n
    const dim3 grid((unsigned)((run.n + SWEEP_BLOCK - 1) / SWEEP_BLOCK), (unsigned)((run.freq + SWEEP_FG - 1) / SWEEP_FG));
    R* mag = (R*)sw.mag;
    R* arg = (R*)sw.arg;
    R* bpc = (R*)sw.bpc;
    if constexpr (sizeof(R) == 4) {
        if (run.rg.runs) {
            // a ragged batch: every instance in the 8-wide class (the padding is exact)
            prefer_shared((const void*)k_sweep_resp<R, 8, true>);
            k_sweep_resp<R, 8, true><<<grid, SWEEP_BLOCK, 0, st>>>(run, gains, lina, list, count, fgrid, mag, arg, bpc,
                                                                   sw.fail);
            prefer_shared((const void*)k_sweep_scan<R, true>);
            k_sweep_scan<R, true><<<(unsigned)((run.n + 127) / 128), 128, 0, st>>>(run, list, count, fgrid, mag, arg,
                                                                                  bpc, sw.fail, info);
            return;
        }
    }
    if (run.ns <= 2) {
        prefer_shared((const void*)k_sweep_resp<R, 2>);
        k_sweep_resp<R, 2><<<grid, SWEEP_BLOCK, 0, st>>>(run, gains, lina, list, count, fgrid, mag, arg, bpc, sw.fail);
    } else if (run.ns <= 4) {
        prefer_shared((const void*)k_sweep_resp<R, 4>);
        k_sweep_resp<R, 4><<<grid, SWEEP_BLOCK, 0, st>>>(run, gains, lina, list, count, fgrid, mag, arg, bpc, sw.fail);
    } else {
        prefer_shared((const void*)k_sweep_resp<R, 8>);
        k_sweep_resp<R, 8><<<grid, SWEEP_BLOCK, 0, st>>>(run, gains, lina, list, count, fgrid, mag, arg, bpc, sw.fail);
    }
    prefer_shared((const void*)k_sweep_scan<R>);
    k_sweep_scan<R><<<(unsigned)((run.n + 127) / 128), 128, 0, st>>>(run, list, count, fgrid, mag, arg, bpc, sw.fail,
                                                                     info);
}

void launch_sweep(const Run& run, int precision, const float* gains, const void* lina, const int* nominal,
                  const void* fgrid, float* info, int* list, int* count, const SweepScratch& sw, cudaStream_t st) {
    CE_CUDA(cudaMemsetAsync(count, 0, sizeof(int), st));
    if (run.rg.runs) {
        prefer_shared((const void*)k_sweep_select<true>);
        k_sweep_select<true><<<(int)((run.n + 127) / 128), 128, 0, st>>>(run, nominal, info, list, count);
    } else {
        prefer_shared((const void*)k_sweep_select<false>);
        k_sweep_select<false><<<(int)((run.n + 127) / 128), 128, 0, st>>>(run, nominal, info, list, count);
    }
    if (precision == CE_PRECISION_FP64)
        sweep_dispatch<double>(run, gains, (const double*)lina, list, count, (const double*)fgrid, info, sw, st);
    else
        sweep_dispatch<float>(run, gains, (const float*)lina, list, count, (const float*)fgrid, info, sw, st);
    CE_CUDA(cudaGetLastError());
}

}  // namespace ce
