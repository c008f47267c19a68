// ref_kernel_runner.cpp -- runs the REFERENCE's own kernels (discrete_solve<Luenberger>,
// eigensetup, modalsetup and the unlaunched discrete_solve<Kalman> from src/main.cu, compiled into oracle/_ref/ref_kernels.cubin by
// oracle/Makefile) through the CUDA driver API, with the reference's launch shape
// (256 threads per block, one thread per candidate, ref: src/main.cu:408-409) and
// its __constant__ tables set exactly as init64KB/upload_plant set them.
//
// TEST INFRASTRUCTURE ONLY: the GPU parity tests use it to compare the engine's
// kernels with the reference's on the same inputs.  Built on the GPU host:
//   g++ -O2 -shared -fPIC -I/usr/local/cuda/include ref_kernel_runner.cpp -lcuda
#include <cuda.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

std::string g_err;

#define CK(x)                                                                   \
    do {                                                                        \
        CUresult r_ = (x);                                                      \
        if (r_ != CUDA_SUCCESS) {                                               \
            const char* s_ = nullptr;                                           \
            cuGetErrorString(r_, &s_);                                          \
            g_err = std::string(#x) + ": " + (s_ ? s_ : "?");                   \
            return 1;                                                           \
        }                                                                       \
    } while (0)

// one loaded module per cubin path (the plain build and the one with the correctly rounded reciprocal)
struct Module {
    CUmodule mod = nullptr;
    CUfunction sim = nullptr, setup = nullptr, modal = nullptr, kalman = nullptr;
};
std::map<std::string, Module> g_mods;
CUcontext g_ctx = nullptr;
CUmodule g_mod = nullptr;
CUfunction g_sim = nullptr, g_setup = nullptr, g_modal = nullptr, g_kalman = nullptr;

int set_global(const char* name, const void* src, size_t bytes) {
    CUdeviceptr p;
    size_t sz = 0;
    CK(cuModuleGetGlobal(&p, &sz, g_mod, name));
    if (sz != bytes) {
        g_err = std::string("size mismatch for ") + name + ": module " + std::to_string(sz) + " vs " +
                std::to_string(bytes);
        return 1;
    }
    CK(cuMemcpyHtoD(p, src, bytes));
    return 0;
}

int load(const char* cubin) {
    auto it = g_mods.find(cubin);
    if (it != g_mods.end()) {
        g_mod = it->second.mod;
        g_sim = it->second.sim;
        g_setup = it->second.setup;
        g_modal = it->second.modal;
        g_kalman = it->second.kalman;
        return 0;
    }
    g_sim = g_setup = g_modal = g_kalman = nullptr;
    if (!g_ctx) {
        CK(cuInit(0));
        CUdevice dev;
        CK(cuDeviceGet(&dev, 0));
        CK(cuDevicePrimaryCtxRetain(&g_ctx, dev));
    }
    CK(cuCtxSetCurrent(g_ctx));
    CK(cuModuleLoad(&g_mod, cubin));
    unsigned int count = 0;
    CK(cuModuleGetFunctionCount(&count, g_mod));
    std::vector<CUfunction> fns(count);
    CK(cuModuleEnumerateFunctions(fns.data(), count, g_mod));
    for (CUfunction f : fns) {
        const char* nm = nullptr;
        CK(cuFuncGetName(&nm, f));
        const std::string s = nm ? nm : "";
        if (s.find("discrete_solve") != std::string::npos && s.find("ControllerType0") != std::string::npos) g_sim = f;
        else if (s.find("discrete_solve") != std::string::npos && s.find("ControllerType1") != std::string::npos)
            g_kalman = f;
        else if (s.find("eigensetup") != std::string::npos) g_setup = f;
        else if (s.find("modalsetup") != std::string::npos) g_modal = f;
    }
    if (!g_sim || !g_setup || !g_modal) {
        g_err = "kernels not found in " + std::string(cubin);
        return 1;
    }
    g_mods[cubin] = Module{g_mod, g_sim, g_setup, g_modal, g_kalman};
    return 0;
}

}  // namespace

extern "C" {

const char* ref_runner_error() { return g_err.c_str(); }

// engine: the EngineParams bytes; tables: padded constant arrays in the order
// STATESPACE_A, _A_I, _B, _C, _D, DISCRETE_A, _A_I, _BU, _BW, _C, BASE_PARAMS
// (sizes 64,64,8,8,1,64,64,8,32,8,34 floats); ops: DC_OPS (4), U_OPS (4), NL_OPS (32)
// Instruction records of 24 bytes.  eigen: the float eigenvalues modalsetup reads.
// times (optional, 5 floats): milliseconds of discrete_solve, eigensetup and modalsetup (CUDA
// events), of the input copies and of the output copies (host clock).  yplant may be null (the
// trajectory stays on the device, as in the reference without dump_diagnostics).
int ref_run(const char* cubin, const void* engine, int engine_bytes, const float* const* tables, const void* dc_ops,
            const void* u_ops, const void* nl_ops, int n, int time, int cuda_w, int nt, int info_w,
            const float* cuda_mx, const float* ref, const float* eigen, const float* info_in, float* yplant,
            float* lina, float* ata, float* atb, float* info_out, float* times) {
    if (load(cubin)) return 1;
    CK(cuCtxSetCurrent(g_ctx));
    if (set_global("ENGINE", engine, engine_bytes)) return 1;
    const char* names[11] = {"STATESPACE_A", "STATESPACE_A_I", "STATESPACE_B", "STATESPACE_C", "STATESPACE_D",
                             "DISCRETE_A",   "DISCRETE_A_I",   "DISCRETE_BU",  "DISCRETE_BW",  "DISCRETE_C",
                             "BASE_PARAMS"};
    const size_t sizes[11] = {64, 64, 8, 8, 1, 64, 64, 8, 32, 8, 34};
    for (int i = 0; i < 11; ++i)
        if (set_global(names[i], tables[i], sizes[i] * sizeof(float))) return 1;
    if (set_global("DC_OPS", dc_ops, 4 * 24) || set_global("U_OPS", u_ops, 4 * 24) ||
        set_global("NL_OPS", nl_ops, 32 * 24))
        return 1;
    const size_t ysz = (size_t)n * time, lsz = (size_t)n * nt * nt, asz = (size_t)n * 4 * nt * nt,
                 bsz = (size_t)n * 2 * nt, isz = (size_t)n * info_w, esz = (size_t)n * 2 * nt,
                 gsz = (size_t)n * cuda_w;
    CUdeviceptr d_g, d_ref, d_y, d_l, d_e, d_a, d_b, d_i;
    CK(cuMemAlloc(&d_g, gsz * 4));
    CK(cuMemAlloc(&d_ref, (size_t)time * 4));
    CK(cuMemAlloc(&d_y, ysz * 4));
    CK(cuMemAlloc(&d_l, lsz * 4));
    CK(cuMemAlloc(&d_e, esz * 4));
    CK(cuMemAlloc(&d_a, asz * 4));
    CK(cuMemAlloc(&d_b, bsz * 4));
    CK(cuMemAlloc(&d_i, isz * 4));
    CK(cuMemsetD8(d_y, 0, ysz * 4));
    CK(cuMemsetD8(d_l, 0, lsz * 4));
    CK(cuMemsetD8(d_a, 0, asz * 4));
    CK(cuMemsetD8(d_b, 0, bsz * 4));
    CK(cuCtxSynchronize());
    auto now = [] { return std::chrono::steady_clock::now(); };
    const auto h0 = now();
    CK(cuMemcpyHtoD(d_g, cuda_mx, gsz * 4));
    CK(cuMemcpyHtoD(d_ref, ref, (size_t)time * 4));
    CK(cuMemcpyHtoD(d_e, eigen, esz * 4));
    CK(cuMemcpyHtoD(d_i, info_in, isz * 4));
    const auto h1 = now();
    CUevent ev[4];
    for (auto& e : ev) CK(cuEventCreate(&e, CU_EVENT_DEFAULT));
    const unsigned tpb = 256, blocks = (n + tpb - 1) / tpb;
    CK(cuEventRecord(ev[0], nullptr));
    {
        void* args[] = {&d_g, &d_ref, &d_y};
        CK(cuLaunchKernel(g_sim, blocks, 1, 1, tpb, 1, 1, 0, nullptr, args, nullptr));
    }
    CK(cuEventRecord(ev[1], nullptr));
    {
        void* args[] = {&d_g, &d_l};
        CK(cuLaunchKernel(g_setup, blocks, 1, 1, tpb, 1, 1, 0, nullptr, args, nullptr));
    }
    CK(cuEventRecord(ev[2], nullptr));
    {
        void* args[] = {&d_y, &d_e, &d_a, &d_b, &d_i};
        CK(cuLaunchKernel(g_modal, blocks, 1, 1, tpb, 1, 1, 0, nullptr, args, nullptr));
    }
    CK(cuEventRecord(ev[3], nullptr));
    CK(cuCtxSynchronize());
    const auto d0 = now();
    if (yplant) CK(cuMemcpyDtoH(yplant, d_y, ysz * 4));
    CK(cuMemcpyDtoH(lina, d_l, lsz * 4));
    CK(cuMemcpyDtoH(ata, d_a, asz * 4));
    CK(cuMemcpyDtoH(atb, d_b, bsz * 4));
    CK(cuMemcpyDtoH(info_out, d_i, isz * 4));
    const auto d1 = now();
    if (times) {
        for (int k = 0; k < 3; ++k) CK(cuEventElapsedTime(&times[k], ev[k], ev[k + 1]));
        times[3] = std::chrono::duration<float, std::milli>(h1 - h0).count();
        times[4] = std::chrono::duration<float, std::milli>(d1 - d0).count();
    }
    for (auto& e : ev) cuEventDestroy(e);
    for (CUdeviceptr p : {d_g, d_ref, d_y, d_l, d_e, d_a, d_b, d_i}) cuMemFree(p);
    return 0;
}

// The reference's discrete_solve<Kalman> (src/discrete_solves.cu:83-185, never
// launched by the reference itself) on rows of its own layout [K(ns), N, R,
// Q(ns)]: the caller sets ENGINE.cuda_mx_width = cuda_w = 2ns+2, so every row
// the kernel reads lies inside `rows`.  Only the trajectory is produced.
int ref_run_kalman(const char* cubin, const void* engine, int engine_bytes, const float* const* tables,
                   const void* dc_ops, const void* u_ops, const void* nl_ops, int n, int time, int cuda_w,
                   const float* rows, const float* ref, float* yplant) {
    if (load(cubin)) return 1;
    if (!g_kalman) {
        g_err = "discrete_solve<Kalman> not found in " + std::string(cubin);
        return 1;
    }
    CK(cuCtxSetCurrent(g_ctx));
    if (set_global("ENGINE", engine, engine_bytes)) return 1;
    const char* names[11] = {"STATESPACE_A", "STATESPACE_A_I", "STATESPACE_B", "STATESPACE_C", "STATESPACE_D",
                             "DISCRETE_A",   "DISCRETE_A_I",   "DISCRETE_BU",  "DISCRETE_BW",  "DISCRETE_C",
                             "BASE_PARAMS"};
    const size_t sizes[11] = {64, 64, 8, 8, 1, 64, 64, 8, 32, 8, 34};
    for (int i = 0; i < 11; ++i)
        if (set_global(names[i], tables[i], sizes[i] * sizeof(float))) return 1;
    if (set_global("DC_OPS", dc_ops, 4 * 24) || set_global("U_OPS", u_ops, 4 * 24) ||
        set_global("NL_OPS", nl_ops, 32 * 24))
        return 1;
    const size_t ysz = (size_t)n * time, gsz = (size_t)n * cuda_w;
    CUdeviceptr d_g, d_ref, d_y;
    CK(cuMemAlloc(&d_g, gsz * 4));
    CK(cuMemAlloc(&d_ref, (size_t)time * 4));
    CK(cuMemAlloc(&d_y, ysz * 4));
    CK(cuMemcpyHtoD(d_g, rows, gsz * 4));
    CK(cuMemcpyHtoD(d_ref, ref, (size_t)time * 4));
    CK(cuMemsetD8(d_y, 0, ysz * 4));
    const unsigned tpb = 256, blocks = (n + tpb - 1) / tpb;
    void* args[] = {&d_g, &d_ref, &d_y};
    CK(cuLaunchKernel(g_kalman, blocks, 1, 1, tpb, 1, 1, 0, nullptr, args, nullptr));
    CK(cuCtxSynchronize());
    CK(cuMemcpyDtoH(yplant, d_y, ysz * 4));
    for (CUdeviceptr p : {d_g, d_ref, d_y}) cuMemFree(p);
    return 0;
}
}
