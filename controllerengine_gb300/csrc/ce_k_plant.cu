// ce_k_plant.cu -- the margin plant's frequency response on the sweep grid and
// its scaling at the spec crossover (ref: src/allmargin.cu:11-41).
//
// The reference evaluates P(z_w) = C (z_w I - A)^{-1} B + D on the host with a
// complex-float partial-pivot LU for every grid point and alpha =
// 1/|P(e^{j w_c ts})|, fatal if not finite.  Here one thread per (plant,
// frequency) runs the same LU (lu_solve_shifted, zero-padded to the dimension
// class) for all plants of a session at once; the z grid itself (float libm,
// shared by every plant) is formed on the host as in the reference.
#include <cfloat>

#include "ce_device.cuh"
#include "ce_host.h"

namespace ce {

// margin plant of one plant: m_a (row stride MAXS), m_b, m_c, m_d
constexpr int MP_A = 0, MP_B = MAXS * MAXS, MP_C = MP_B + MAXS, MP_D = MP_C + MAXS, MP_STRIDE = MP_D + 1;

template <typename R, int NS>
__global__ void __launch_bounds__(128) k_plant_grid(int np, int n, int F, const float* __restrict__ mp,
                                                    const R* __restrict__ zg, R* __restrict__ grid,
                                                    R* __restrict__ alpha, int* __restrict__ bad) {
    const int64_t t = (int64_t)blockIdx.x * 128 + threadIdx.x;
    if (t >= (int64_t)np * (F + 1)) return;
    const int p = (int)(t / (F + 1)), w = (int)(t % (F + 1));
    const float* m = mp + (int64_t)p * MP_STRIDE;
    R A[NS * NS], b[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) {
#pragma unroll
        for (int j = 0; j < NS; ++j) A[i * NS + j] = (i < n && j < n) ? R(m[MP_A + i * MAXS + j]) : R(0);
        b[i] = i < n ? R(m[MP_B + i]) : R(0);
    }
    const cplx<R> z{zg[4 * w], zg[4 * w + 1]};
    cplx<R> x[NS];
    lu_solve_shifted<R, NS>(z, A, 1, b, x);
    bool ok = true;
#pragma unroll
    for (int i = 0; i < NS; ++i) ok = ok && (i >= n || cfinite(x[i]));
    // C^T x + D, accumulated in index order
    cplx<R> P{R(0), R(0)};
    if (ok) {
#pragma unroll
        for (int i = 0; i < NS; ++i)
            if (i < n) {
                const cplx<R> tt = cmul(cplx<R>{R(m[MP_C + i]), R(0)}, x[i]);
                P = cplx<R>{radd(P.re, tt.re), radd(P.im, tt.im)};
            }
        P.re = radd(P.re, R(m[MP_D]));
    }
    if (w < F) {
        R* g = grid + ((int64_t)p * F + w) * 8;
        g[0] = z.re;
        g[1] = z.im;
        g[2] = zg[4 * w + 2];
        g[3] = P.re;
        g[4] = P.im;
        g[5] = cabs_(P);
        g[6] = ok ? R(1) : R(0);
        g[7] = R(0);
    } else {
        const R pmag = cabs_(P);
        alpha[p] = rdiv(R(1), pmag);
        bad[p] = (!ok || !(pmag > R(0)) || !isfinite(pmag)) ? 1 : 0;
    }
}

template <typename R>
static void grid_dispatch(int np, int n, int F, const float* mp, const R* zg, R* grid, R* alpha, int* bad,
                          cudaStream_t st) {
    const int64_t total = (int64_t)np * (F + 1);
    const int blocks = (int)((total + 127) / 128);
    if (n <= 2) k_plant_grid<R, 2><<<blocks, 128, 0, st>>>(np, n, F, mp, zg, grid, alpha, bad);
    else if (n <= 4) k_plant_grid<R, 4><<<blocks, 128, 0, st>>>(np, n, F, mp, zg, grid, alpha, bad);
    else k_plant_grid<R, 8><<<blocks, 128, 0, st>>>(np, n, F, mp, zg, grid, alpha, bad);
}

void launch_plant_grid(int precision, int np, int n, int F, const float* mp, const void* zg, void* grid, void* alpha,
                       int* bad, cudaStream_t st) {
    if (precision == CE_PRECISION_FP64)
        grid_dispatch<double>(np, n, F, mp, (const double*)zg, (double*)grid, (double*)alpha, bad, st);
    else
        grid_dispatch<float>(np, n, F, mp, (const float*)zg, (float*)grid, (float*)alpha, bad, st);
    CE_CUDA(cudaGetLastError());
}

int margin_plant_stride() { return MP_STRIDE; }

// A ragged batch: grid row t belongs to instance row_inst[t] at frequency
// row_w[t] (row F of an instance: its crossover); every instance in the 8-wide
// class (the zero padding of the shifted LU is exact).
__global__ void __launch_bounds__(128) k_plant_grid_rows(int64_t rows, const int* __restrict__ row_inst,
                                                         const int* __restrict__ row_w, const int* __restrict__ n_of,
                                                         const int* __restrict__ F_of, const int64_t* __restrict__ zoff,
                                                         const int64_t* __restrict__ goff, const float* __restrict__ mp,
                                                         const float* __restrict__ zg, float* __restrict__ grid,
                                                         float* __restrict__ alpha, int* __restrict__ bad) {
    constexpr int NS = MAXS;
    const int64_t t = (int64_t)blockIdx.x * 128 + threadIdx.x;
    if (t >= rows) return;
    const int p = row_inst[t], w = row_w[t], n = n_of[p], F = F_of[p];
    const float* m = mp + (int64_t)p * MP_STRIDE;
    const float* zr = zg + zoff[p] + 4 * (int64_t)w;
    float A[NS * NS], b[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) {
#pragma unroll
        for (int j = 0; j < NS; ++j) A[i * NS + j] = (i < n && j < n) ? m[MP_A + i * MAXS + j] : 0.0f;
        b[i] = i < n ? m[MP_B + i] : 0.0f;
    }
    const cplx<float> z{zr[0], zr[1]};
    cplx<float> x[NS];
    lu_solve_shifted<float, NS>(z, A, 1, b, x);
    bool ok = true;
#pragma unroll
    for (int i = 0; i < NS; ++i) ok = ok && (i >= n || cfinite(x[i]));
    cplx<float> P{0.0f, 0.0f};
    if (ok) {
#pragma unroll
        for (int i = 0; i < NS; ++i)
            if (i < n) {
                const cplx<float> tt = cmul(cplx<float>{m[MP_C + i], 0.0f}, x[i]);
                P = cplx<float>{radd(P.re, tt.re), radd(P.im, tt.im)};
            }
        P.re = radd(P.re, m[MP_D]);
    }
    if (w < F) {
        float* g = grid + goff[p] + 8 * (int64_t)w;
        g[0] = z.re;
        g[1] = z.im;
        g[2] = zr[2];
        g[3] = P.re;
        g[4] = P.im;
        g[5] = cabs_(P);
        g[6] = ok ? 1.0f : 0.0f;
        g[7] = 0.0f;
    } else {
        const float pmag = cabs_(P);
        alpha[p] = rdiv(1.0f, pmag);
        bad[p] = (!ok || !(pmag > 0.0f) || !isfinite(pmag)) ? 1 : 0;
    }
}

void launch_plant_grid_rows(int64_t rows, const int* row_inst, const int* row_w, const int* n_of, const int* F_of,
                            const int64_t* zoff, const int64_t* goff, const float* mp, const float* zg, float* grid,
                            float* alpha, int* bad, cudaStream_t st) {
    k_plant_grid_rows<<<(unsigned)((rows + 127) / 128), 128, 0, st>>>(rows, row_inst, row_w, n_of, F_of, zoff, goff,
                                                                      mp, zg, grid, alpha, bad);
    CE_CUDA(cudaGetLastError());
}

}  // namespace ce
