// ce_jit.cpp -- the simulation kernel specialised to one plant's instruction
// program, compiled at session creation with NVRTC.
//
// The decoded DC / U / NL chains are fixed for a session, so instead of
// interpreting them every step (operand-kind selects, an op switch and a
// shared-memory read of the source state per instruction) they are emitted as
// straight-line CUDA over the register-resident states and compiled together
// with the shared step loop (ce_sim_body.cuh) for the exact plant dimensions.
// The instruction *structure* (op, column, operand kinds) is compiled in; the
// constant operands stay in the launch parameters, so every round of a serial
// run (same program, different BASE_PARAMS) shares one compiled kernel.  The
// per-candidate-plant form (`mc`) reads the constants and the plant matrices
// from the candidate's row of the plant table instead.  Each
// generated instruction performs exactly the operations of the interpreter
// (ref: src/main.cu:260-291) with the same roundings, so results are
// bit-identical to the table-driven kernel's.  Compiled kernels are cached per
// process by their source text.
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <nvrtc.h>

#include "ce_host.h"

namespace ce {

namespace {

// Header texts compiled into the library by build.py (ce_jit_src.inc defines
// kJitHeaders[] = {name, text} pairs).
#include "ce_jit_src.inc"

std::mutex g_jit_mu;
std::map<std::string, SimKernels> g_jit_cache;  // source -> compiled kernels

// One chain as straight-line code.  Constant operands come from the launch's
// Plant, or with `mc` from the candidate's plant-table row (slot numbering of
// MC_CST: `slot0` is the chain's first slot).
std::string fmt_chain(const char* fname, const Instr* ins, int n, bool seed, bool nl, const char* table, int slot0,
                      bool mc) {
    std::ostringstream o;
    o << "template <int NSRC, class Lc>\n__device__ __forceinline__ float " << fname
      << "(const ce::Plant& P, const Lc& L, const float (&xs)[NSRC], float y, float seed) {\n    float r = 0.0f;\n";
    for (int k = 0; k < n; ++k) {
        const Instr& I = ins[k];
        o << "    {  // op " << I.op << " col " << I.col << " kinds " << I.akind << "," << I.bkind << "\n";
        if (nl && I.col == MAXD) o << "        const float pos = y;\n";
        else o << "        const float pos = xs[" << I.col << "];\n";
        if (k == 0) o << (seed ? "        const float prev = isnan(seed) ? pos : seed;\n" : "        const float prev = pos;\n");
        else o << "        const float prev = r;\n";
        auto operand = [&](int kind, const char* field) {
            std::ostringstream e;
            if (kind == CE_OPERAND_CONST && mc) e << "L.c(" << 2 * (slot0 + k) + (field[0] == 'b' ? 1 : 0) << ")";
            else if (kind == CE_OPERAND_CONST) e << "P." << table << "[" << k << "]." << field;
            else if (kind == CE_OPERAND_STATE) e << "pos";
            else e << "prev";
            return e.str();
        };
        const std::string a = operand(I.akind, "aval"), b = operand(I.bkind, "bval");
        switch (I.op) {
            case 1: o << "        r = __fadd_rn(" << a << ", " << b << ");\n"; break;
            case 2: o << "        r = __fsub_rn(" << a << ", " << b << ");\n"; break;
            case 3: o << "        r = __fmul_rn(" << a << ", " << b << ");\n"; break;
            case 4: o << "        r = __fdiv_rn(" << a << ", " << b << ");\n"; break;
            case 5: o << "        r = fminf(fmaxf(prev, " << a << "), " << b << ");\n"; break;
            case 6: o << "        r = (float)((0.0f < " << a << ") - (" << a << " < 0.0f));\n"; break;
            default: o << "        (void)prev;  // outside 1..6: no change, the chain counts as started\n"; break;
        }
        o << "        (void)pos;\n    }\n";
    }
    o << "    (void)seed; (void)y; (void)xs; (void)P; (void)L;\n    return r;\n}\n\n";
    return o.str();
}

std::string jit_source(const Plant& P, int ns, int nd, bool mc, bool kalman) {
    std::ostringstream o;
    o << "#include \"ce_sim_body.cuh\"\n\nnamespace cejit {\n\n";
    o << fmt_chain("dc", P.dc, P.n_dc, false, false, "dc", 0, mc);
    o << fmt_chain("u", P.u, P.n_u, true, false, "u", MAX_DC, mc);
    for (int k = 0; k < MAXW; ++k) {
        const std::string fn = "nl" + std::to_string(k), tab = "nl[" + std::to_string(k) + "]";
        o << fmt_chain(fn.c_str(), P.nl[k], P.n_nl[k], false, true, tab.c_str(), MAX_DC + MAX_U + k * MAX_NL, mc);
    }
    o << "struct Chains {\n"
         "    static constexpr bool kSmem = false;\n"
         "    template <int NDC>\n"
      << (mc ? "    using Local = ce::McLocal<NDC>;\n" : "    using Local = ce::BankLocal<NDC>;\n")
      << "    template <int NDC, class Lc>\n"
         "    __device__ static __forceinline__ float dc(const ce::Plant& P, const Lc& L, const float (&xp)[NDC], const float*) {\n"
         "        return cejit::dc(P, L, xp, 0.0f, 0.0f);\n    }\n"
         "    template <int NSC, class Lc>\n"
         "    __device__ static __forceinline__ float u(const ce::Plant& P, const Lc& L, const float (&xh)[NSC], const float*,\n"
         "                                              float seed) {\n"
         "        return cejit::u(P, L, xh, 0.0f, seed);\n    }\n"
         "    template <int NDC, class Lc>\n"
         "    __device__ static __forceinline__ void nl(const ce::Plant& P, const Lc& L, const float (&xp)[NDC], float y,\n"
         "                                              const float*, float (&W)[ce::MAXW]) {\n"
         "        W[0] = cejit::nl0(P, L, xp, y, 0.0f);\n        W[1] = cejit::nl1(P, L, xp, y, 0.0f);\n"
         "        W[2] = cejit::nl2(P, L, xp, y, 0.0f);\n        W[3] = cejit::nl3(P, L, xp, y, 0.0f);\n    }\n};\n\n"
         "}  // namespace cejit\n\n";
    auto kernel = [&](const char* name, int nsc, const char* mode) {
        o << "extern \"C\" __global__ void __launch_bounds__(ce::SIM_BLOCK) " << name << "(\n"
             "    const ce::Run run, const __grid_constant__ ce::Plant P, const float* __restrict__ gains,\n"
             "    float* __restrict__ ywin, ce::SimSummary* __restrict__ summ, float* __restrict__ traj) {\n"
          << "    ce::sim_run<" << nsc << ", " << nd << ", cejit::Chains, " << mode
          << ">(run, P, gains, ywin, summ, traj);\n}\n";
    };
    // the Kalman loop always runs the full padded observer width
    if (kalman) {
        kernel("ce_sim_specialised", MAXS, "ce::SIM_KALMAN_LANE");
        kernel("ce_sim_kalman_shared", MAXS, "ce::SIM_KALMAN_SHARED");
        kernel("ce_sim_kalman_sched", MAXS, "ce::SIM_KALMAN_SCHED");
        kernel("ce_sim_kalman_quad", MAXS, "ce::SIM_KALMAN_QUAD");
    } else {
        kernel("ce_sim_specialised", ns, "ce::SIM_LUENBERGER");
        if (!mc) {
            // the wide form (four lanes per candidate) for batches too small to fill the GPU
            o << "extern \"C\" __global__ void __launch_bounds__(ce::SIM_BLOCK) ce_sim_wide(\n"
                 "    const ce::Run run, const __grid_constant__ ce::Plant P, const float* __restrict__ gains,\n"
                 "    float* __restrict__ ywin, ce::SimSummary* __restrict__ summ, float* __restrict__ traj) {\n"
              << "    ce::sim_wide<" << ns << ", " << nd << ", cejit::Chains>(run, P, gains, ywin, summ, traj);\n}\n";
        }
    }
    return o.str();
}

SimKernels compile(const std::string& src, std::string& log, bool kalman) {
    std::vector<const char*> names, texts;
    for (const auto& h : kJitHeaders) {
        names.push_back(h.name);
        texts.push_back(h.text);
    }
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, src.c_str(), "ce_sim_specialised.cu", (int)names.size(), texts.data(),
                           names.data()) != NVRTC_SUCCESS) {
        log = "nvrtcCreateProgram failed";
        return {};
    }
    const std::string inc = std::string("-I") + CE_CUDA_INCLUDE;
    const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "--fmad=true", inc.c_str(), "-lineinfo"};
    const nvrtcResult rc = nvrtcCompileProgram(prog, (int)(sizeof(opts) / sizeof(opts[0])), opts);
    size_t lsz = 0;
    nvrtcGetProgramLogSize(prog, &lsz);
    std::string plog(lsz, '\0');
    if (lsz) nvrtcGetProgramLog(prog, plog.data());
    if (rc != NVRTC_SUCCESS) {
        log = std::string("NVRTC: ") + nvrtcGetErrorString(rc) + "\n" + plog;
        nvrtcDestroyProgram(&prog);
        return {};
    }
    size_t csz = 0;
    nvrtcGetCUBINSize(prog, &csz);
    std::vector<char> cubin(csz);
    nvrtcGetCUBIN(prog, cubin.data());
    nvrtcDestroyProgram(&prog);
    cudaLibrary_t lib;
    cudaError_t e = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) {
        log = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(e);
        return {};
    }
    SimKernels out;
    std::vector<std::pair<const char*, const void**>> wanted{{"ce_sim_specialised", &out.main}};
    if (kalman) {
        wanted.push_back({"ce_sim_kalman_shared", &out.shared});
        wanted.push_back({"ce_sim_kalman_sched", &out.sched});
        wanted.push_back({"ce_sim_kalman_quad", &out.quad});
    }
    if (src.find("ce_sim_wide(") != std::string::npos) wanted.push_back({"ce_sim_wide", &out.wide});
    for (const auto& [name, slot] : wanted) {
        cudaKernel_t k;
        e = cudaLibraryGetKernel(&k, lib, name);
        if (e != cudaSuccess) {
            log = std::string("cudaLibraryGetKernel: ") + cudaGetErrorString(e);
            return {};
        }
        e = cudaFuncSetAttribute(reinterpret_cast<const void*>(k), cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) {
            log = std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e);
            return {};
        }
        *slot = reinterpret_cast<const void*>(k);
    }
    return out;
}

}  // namespace

SimKernels specialise_sim(const Plant& P, int ns, int nd, std::string& log, bool mc, bool kalman) {
    const std::string src = jit_source(P, ns, nd, mc, kalman);
    std::lock_guard<std::mutex> g(g_jit_mu);
    auto it = g_jit_cache.find(src);
    if (it != g_jit_cache.end()) return it->second;
    const SimKernels k = compile(src, log, kalman);
    if (k) g_jit_cache.emplace(src, k);
    return k;
}

std::string specialised_source(const Plant& P, int ns, int nd, bool kalman) {
    return jit_source(P, ns, nd, false, kalman);
}

bool use_wide_sim(int64_t n, int nsc, int ndc) {
    static const int mode = [] {
        const char* e = std::getenv("CE_SIM_WIDE");
        return e ? (e[0] == '0' ? 0 : 1) : -1;
    }();
    if (mode >= 0) return mode == 1;
    static const int sms = [] {
        int dev = 0, k = 0;
        CE_CUDA(cudaGetDevice(&dev));
        CE_CUDA(cudaDeviceGetAttribute(&k, cudaDevAttrMultiProcessorCount, dev));
        return k;
    }();
    // measured: faster up to ~4,096 candidates with an 8-class observer or plant
    // (one 8-state candidate: 4.0 -> 2.8 ms for 10,000 steps), slower at 16,384,
    // and slower for the 4/4 class at any size (one row per lane is too little
    // work to pay for the exchange)
    return !(nsc == 4 && ndc == 4) && 2 * ((n + SIM_BLOCK - 1) / SIM_BLOCK) < (int64_t)sms;
}

void launch_sim_specialised(const void* kernel, const Run& run, const Plant& P, const float* gains, float* ywin,
                            SimSummary* summ, float* traj, cudaStream_t st, bool wide) {
    const int grid = wide ? (int)((run.n + SW_CPB - 1) / SW_CPB) : sim_grid(run);
    void* args[] = {(void*)&run, (void*)&P, (void*)&gains, (void*)&ywin, (void*)&summ, (void*)&traj};
    CE_CUDA(cudaLaunchKernel(kernel, dim3(grid), dim3(SIM_BLOCK), args, 0, st));
}

}  // namespace ce
