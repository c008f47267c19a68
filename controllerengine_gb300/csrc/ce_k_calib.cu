// ce_k_calib.cu -- FMA-issue throughput of the device (roofline denominator for
// the FP32 and FP64 pipes).  Each thread runs 8 independent dependent chains
// of FMAs in registers, so the measurement is issue-bound, not latency-bound.
#include "ce_device.cuh"
#include "ce_host.h"

namespace ce {

template <typename R>
__global__ void __launch_bounds__(256) k_fma_rate(R* out, int iters, R a, R b) {
    R x0 = R(threadIdx.x), x1 = x0 + R(1), x2 = x0 + R(2), x3 = x0 + R(3);
    R x4 = x0 + R(4), x5 = x0 + R(5), x6 = x0 + R(6), x7 = x0 + R(7);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = rfma(x0, a, b); x1 = rfma(x1, a, b); x2 = rfma(x2, a, b); x3 = rfma(x3, a, b);
            x4 = rfma(x4, a, b); x5 = rfma(x5, a, b); x6 = rfma(x6, a, b); x7 = rfma(x7, a, b);
        }
    }
    const R s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == R(-12345)) out[0] = s;  // keeps the chains live
}

double measure_fma_rate(bool fp64) {
    int dev = 0, sms = 0;
    CE_CUDA(cudaGetDevice(&dev));
    CE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    void* out = nullptr;
    CE_CUDA(cudaMalloc(&out, 64));
    const int blocks = sms * 8, threads = 256;
    const int iters = fp64 ? 64 : 2048;
    cudaEvent_t e0, e1;
    CE_CUDA(cudaEventCreate(&e0));
    CE_CUDA(cudaEventCreate(&e1));
    auto launch = [&] {
        if (fp64) k_fma_rate<double><<<blocks, threads>>>((double*)out, iters, 0.999999, 1e-7);
        else k_fma_rate<float><<<blocks, threads>>>((float*)out, iters, 0.999999f, 1e-7f);
    };
    launch();
    CE_CUDA(cudaDeviceSynchronize());
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
        CE_CUDA(cudaEventRecord(e0));
        launch();
        CE_CUDA(cudaEventRecord(e1));
        CE_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        CE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        best = std::min(best, ms);
    }
    CE_CUDA(cudaGetLastError());
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    const double ops = (double)blocks * threads * iters * 16.0 * 8.0;
    return ops / (best * 1e-3);
}

}  // namespace ce
