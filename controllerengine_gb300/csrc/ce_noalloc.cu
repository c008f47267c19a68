// ce_noalloc.cu -- the modal-fit path without any device allocation.
//
// Who needs this: callers that must not allocate device memory at the time
// they evaluate -- a real-time tuning loop that cannot take the latency and
// jitter of cudaMalloc (it may synchronise the device), or a host application
// whose device memory is owned entirely by its own allocator or budgeted up
// front.  The session API (ce_evaluate_device) grows its scratch with
// cudaMalloc when a batch is larger than any before it; this entry point never
// allocates: no cudaMalloc, no cudaFree, no allocating library routine.
//
// What it computes: the simulation and the modal setup of the fit window for
// n candidates (k_sim + k_fit, the same kernels the session pipeline runs):
// AtA, Atb, the steady-state value and overshoot, and the unstable penalty,
// from caller-provided gains and eigenvalues.  The only scratch of that path,
// the candidate-major fit window and the per-candidate trajectory summaries,
// lives in the file-scope array below instead of cudaMalloc'd memory.
//
// Limits and sharing:
//  * The array holds CE_NOALLOC_SCRATCH_FLOATS floats (32 MiB), allocated by
//    the CUDA runtime when the library's module loads on a device and held by
//    every device that loads it until the process exits.  A call needs
//    n * (fit window rounded up to 8 samples + 4) floats; larger calls are
//    rejected with an error, before anything is launched.
//  * All calls on a device share the one array.  Nothing in it must start at
//    zero: every element the fit reads is written by the simulation of the
//    same call.  Two calls whose work overlaps on the GPU (different streams,
//    or different host threads) race on the array and produce garbage: the
//    caller serialises them (one stream, or events).
//  * The first call on a device (whichever host thread makes it) looks up the
//    array's device address with cudaGetSymbolAddress, with that device
//    current, once, and keeps it; make that first call before any stream
//    capture.  In host code the array's name is only a host-side stand-in,
//    never a device address, so the kernels get the looked-up address.
//  * The session's plant must be usable: a plant whose sweep grid failed at
//    session creation is refused with its message, as ce_evaluate_device
//    refuses it.
#include <mutex>

#include "ce_device.cuh"
#include "ce_host.h"

namespace ce {

static __device__ __align__(256) float g_fit_scratch[CE_NOALLOC_SCRATCH_FLOATS];

namespace {

constexpr int MAX_DEVICES = 64;
// Per device: the array's device address, looked up once.  Concurrent first
// calls from several host threads run the lookup once (std::call_once) and all
// read the published address.
std::once_flag g_scratch_once[MAX_DEVICES];
float* g_scratch_ptr[MAX_DEVICES] = {};
cudaError_t g_scratch_rc[MAX_DEVICES] = {};

float* scratch_address() {
    int dev = 0;
    CE_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES) fail("ce_modal_fit_noalloc: device {} out of range", dev);
    std::call_once(g_scratch_once[dev], [dev] {
        void* p = nullptr;
        g_scratch_rc[dev] = cudaGetSymbolAddress(&p, g_fit_scratch);
        g_scratch_ptr[dev] = static_cast<float*>(p);
    });
    if (g_scratch_rc[dev] != cudaSuccess || !g_scratch_ptr[dev])
        fail("ce_modal_fit_noalloc: cudaGetSymbolAddress of the static scratch failed: {}",
             cudaGetErrorString(g_scratch_rc[dev]));
    return g_scratch_ptr[dev];
}

}  // namespace
}  // namespace ce

extern "C" CE_EXPORT int ce_modal_fit_noalloc(ce_session* s, int32_t plant_index, int64_t n, const float* d_cuda_mx,
                                              const float* d_eigen, float* d_ata, float* d_atb, float* d_info,
                                              void* stream) {
    using namespace ce;
    try {
        if (!s) fail("ce_modal_fit_noalloc: null session");
        if (plant_index < 0 || plant_index >= session_plants(s))
            fail("ce_modal_fit_noalloc: plant index {} out of range [0, {})", plant_index, session_plants(s));
        if (n < 0) fail("ce_modal_fit_noalloc: candidate count {} is negative", n);
        if (n == 0) return 0;
        if (const std::string& e = session_plant_error(s, plant_index); !e.empty())
            fail("ce_modal_fit_noalloc: plant {}: {}", plant_index, e);
        Run r = session_run(s, plant_index, n);
        // the limit is checked by division first, so that no product can overflow
        const int64_t per = (int64_t)r.fit_pitch + 4;
        const int64_t cap = (int64_t)CE_NOALLOC_SCRATCH_FLOATS / per;
        if (n > cap)
            fail("ce_modal_fit_noalloc: {} candidates need {} scratch floats each (fit window {} + 4), more than "
                 "the {} that fit; the static scratch holds {} floats",
                 n, per, r.fit_pitch, cap, (int64_t)CE_NOALLOC_SCRATCH_FLOATS);
        const int64_t win = n * (int64_t)r.fit_pitch;
        float* base = scratch_address();
        float* ywin = base;
        SimSummary* summ = reinterpret_cast<SimSummary*>(base + win);  // win is a multiple of 8 floats: 32-byte aligned
        cudaStream_t st = (cudaStream_t)stream;
        r.store_traj = 0;
        launch_sim(r, *session_plant(s, plant_index), CE_PRECISION_MIXED, d_cuda_mx, ywin, summ, nullptr, st);
        launch_fit(r, CE_PRECISION_MIXED, d_eigen, ywin, summ, d_ata, d_atb, d_info, nullptr, nullptr, st);
        session_count_launches(s, 2);
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}
