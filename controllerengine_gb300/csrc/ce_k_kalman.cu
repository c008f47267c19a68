// ce_k_kalman.cu -- grouping of a Kalman evaluation's candidates by noise
// weights, for the shared-noise simulation form (ce_sim_body.cuh).
//
// The covariance recursion of the time-varying Kalman observer (ref:
// src/discrete_solves.cu:128-163) reads only the observer model and the
// candidate's R and diag(Q), so candidates with the same weights, bit for bit,
// run the same recursion.  Three kernels sort them into warps that share it:
//   k_kal_hist     hash (R, Q[0..ns)) to one of KAL_BUCKETS buckets, count;
//   k_kal_scan     per bucket: a group of >= KAL_MIN_GROUP candidates takes
//                  ceil(L/32) whole warps of the shared list, a smaller one
//                  joins the per-candidate list; exclusive offsets of both;
//   k_kal_scatter  place each candidate (its rank in the bucket by atomic
//                  counter) in its list.
// Two weight sets that hash to one bucket land in the same warps; the shared
// form checks every warp bit for bit and defers a mixed warp's candidates to
// the per-candidate form, so grouping only ever affects speed.  Results do not
// depend on the placement: each candidate's recursion is the same wherever it
// is computed.
#include "ce_host.h"

namespace ce {

namespace {

__device__ __forceinline__ unsigned mix(unsigned h, unsigned v) {
    // one round of the 32-bit MurmurHash3 block mix
    v *= 0xcc9e2d51u;
    v = (v << 15) | (v >> 17);
    v *= 0x1b873593u;
    h ^= v;
    h = (h << 13) | (h >> 19);
    return h * 5u + 0xe6546b64u;
}

__device__ __forceinline__ unsigned fmix(unsigned h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

__global__ void __launch_bounds__(256) k_kal_hist(const Run run, const float* __restrict__ gains,
                                                  unsigned* __restrict__ bucket, int* __restrict__ cnt) {
    const int64_t c = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (c >= run.n) return;
    const int ns = run.ns;
    const float* row = gains + c * run.cuda_w + 2 * ns + 1;  // R, Q[0..ns)
    unsigned h = 0x9747b28cu;
    for (int i = 0; i <= ns; ++i) h = mix(h, __float_as_uint(row[i]));
    const unsigned b = fmix(h ^ (unsigned)(ns + 1)) & (KAL_BUCKETS - 1);
    bucket[c] = b;
    atomicAdd(&cnt[b], 1);
}

constexpr int SCAN_THREADS = 1024, SCAN_PER = KAL_BUCKETS / SCAN_THREADS;

__global__ void __launch_bounds__(SCAN_THREADS) k_kal_scan(const int* __restrict__ cnt, int* __restrict__ hoff,
                                                           int* __restrict__ poff, int* __restrict__ totals) {
    __shared__ int sh[SCAN_THREADS], sp[SCAN_THREADS];
    const int t = threadIdx.x, b0 = t * SCAN_PER;
    int h = 0, p = 0;
    for (int k = 0; k < SCAN_PER; ++k) {
        const int L = cnt[b0 + k];
        if (L >= KAL_MIN_GROUP) h += (L + 31) & ~31;
        else p += L;
    }
    sh[t] = h;
    sp[t] = p;
    __syncthreads();
    // inclusive Hillis-Steele scan of the per-thread sums
    for (int d = 1; d < SCAN_THREADS; d <<= 1) {
        const int ah = t >= d ? sh[t - d] : 0, ap = t >= d ? sp[t - d] : 0;
        __syncthreads();
        sh[t] += ah;
        sp[t] += ap;
        __syncthreads();
    }
    int oh = sh[t] - h, op = sp[t] - p;
    for (int k = 0; k < SCAN_PER; ++k) {
        const int L = cnt[b0 + k];
        hoff[b0 + k] = oh;
        poff[b0 + k] = op;
        if (L >= KAL_MIN_GROUP) oh += (L + 31) & ~31;
        else op += L;
    }
    if (t == SCAN_THREADS - 1) {
        totals[0] = sh[t];
        totals[1] = sp[t];
    }
}

__global__ void __launch_bounds__(256) k_kal_scatter(const Run run, const unsigned* __restrict__ bucket,
                                                     const int* __restrict__ cnt, const int* __restrict__ hoff,
                                                     const int* __restrict__ poff, int* __restrict__ fill,
                                                     const int* __restrict__ totals, int* __restrict__ order) {
    const int64_t c = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (c >= run.n) return;
    const unsigned b = bucket[c];
    const int r = atomicAdd(&fill[b], 1);
    if (cnt[b] >= KAL_MIN_GROUP) order[hoff[b] + r] = (int)c;
    else order[totals[0] + poff[b] + r] = (int)c;
}

}  // namespace

void launch_kalman_groups(const Run& run, const float* gains, const KalGroups& g, cudaStream_t st) {
    // cnt, fill and totals are one contiguous block
    CE_CUDA(cudaMemsetAsync(g.cnt, 0, (2 * (size_t)KAL_BUCKETS + KAL_TOTALS) * sizeof(int), st));
    CE_CUDA(cudaMemsetAsync(g.order, 0xff, (size_t)kal_shared_slots(run.n) * sizeof(int), st));
    const int blocks = (int)((run.n + 255) / 256);
    k_kal_hist<<<blocks, 256, 0, st>>>(run, gains, g.bucket, g.cnt);
    k_kal_scan<<<1, SCAN_THREADS, 0, st>>>(g.cnt, g.hoff, g.poff, g.totals);
    k_kal_scatter<<<blocks, 256, 0, st>>>(run, g.bucket, g.cnt, g.hoff, g.poff, g.fill, g.totals, g.order);
    CE_CUDA(cudaGetLastError());
}

int sim_grid(const Run& run) {
    // the shared list's slots; the stragglers' quad form: four lanes per candidate
    const int64_t slots = run.kal_list == 1 ? kal_shared_slots(run.n) : run.kal_list == 4 ? 4 * run.n : run.n;
    return (int)((slots + SIM_BLOCK - 1) / SIM_BLOCK);
}

}  // namespace ce
