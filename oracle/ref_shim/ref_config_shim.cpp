// ref_config_shim.cpp -- builds the reference's own config parser (src/config.cu,
// compiled from the reference tree by oracle/Makefile, never copied) into
// oracle/_ref/libref_config.so, so tests can pin the engine's parser against it.
//
// config.cu is #included into the reference's main.cu; standalone it needs the
// few names main.cu defines before that include (src/main.cu:22-52): the error
// helper CUDAERR (throws std::runtime_error with a std::format message), PI and
// the MAX_* limits, and the CUDA `__host__` qualifier.  They are provided here
// with the same meaning.
#include <cmath>
#include <cstring>
#include <format>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>

#define __host__
template <typename... A>
[[noreturn]] static void ref_throw(std::format_string<A...> f, A&&... a) {
    throw std::runtime_error(std::format(f, std::forward<A>(a)...));
}
#define CUDAERR(...) ref_throw(__VA_ARGS__)
constexpr float PI = 0x1.921fb6p+1f;
constexpr int MAX_STATESPACE_DIM = 8;
constexpr int MAX_DISCRETE_DIM = 8;
constexpr int MAX_NONLIN_DIM = 4;
constexpr int MAX_TOTAL_DIM = MAX_STATESPACE_DIM + MAX_DISCRETE_DIM;
constexpr int MAX_NL_DIM = MAX_DISCRETE_DIM + 1;
constexpr int MAX_DC_INSTRUCTIONS = 4;
constexpr int MAX_U_INSTRUCTIONS = 4;
constexpr int MAX_NL_INSTRUCTIONS = 8;
constexpr int MAX_PARAMS = 34;

#include "config.cu"

// Flat view of the reference's EngineConfig + EngineParams for ctypes.
extern "C" {
struct ref_cfg_out {
    int statespace_dim, discrete_dim, nonlin_dim, n_params, input_size, dc_instructions, u_instructions;
    int nl_instructions[4];
    int n_cores, n_rounds, serial, time;
    float duration;
    double ref_step_time;
    float ref_amplitude, fit_start, fit_end, steady_start, bandwidth, damping, overshoot, steady_state_error,
        crossover_coeff, target_gm, target_pm, target_b, eig_fail_err, unstable_err;
    int freq;
    float freq_min;
    int dump_diagnostics, n_threads;
    float freq_max;
    int total_dim, dc_dim, u_dim, nl_dim, cuda_mx_width, info_scoring, info_freqresp, info_allmargin, info_modal,
        info_mx_width, eigen_mx_width, lina_mx_width, ata_mx_width, atb_mx_width, nl_instructions_total;
    float ts, fit_t0, fit_t1, damping2, damping4, crossover;
    int fit_start_id, steady_start_id;
};

// Parses `path` with the reference's load_config.  Returns 0, or 1 with the
// exception text in err.
int ref_load_config(const char* path, ref_cfg_out* o, char* err, int errlen) {
    try {
        EngineConfig c = load_config(path);
        EngineParams p = make_engine_params(c);
        std::memset(o, 0, sizeof(*o));
        o->statespace_dim = c.statespace_dim; o->discrete_dim = c.discrete_dim; o->nonlin_dim = c.nonlin_dim;
        o->n_params = c.n_params; o->input_size = c.input_size; o->dc_instructions = c.dc_instructions;
        o->u_instructions = c.u_instructions;
        for (int i = 0; i < c.nonlin_dim; i++) o->nl_instructions[i] = c.nl_instructions[i];
        o->n_cores = c.n_cores; o->n_rounds = c.n_rounds; o->serial = c.serial; o->time = c.time;
        o->duration = c.duration; o->ref_step_time = c.ref_step_time; o->ref_amplitude = c.ref_amplitude;
        o->fit_start = c.fit_start; o->fit_end = c.fit_end; o->steady_start = c.steady_start;
        o->bandwidth = c.bandwidth; o->damping = c.damping; o->overshoot = c.overshoot;
        o->steady_state_error = c.steady_state_error; o->crossover_coeff = c.crossover_coeff;
        o->target_gm = c.target_gm; o->target_pm = c.target_pm; o->target_b = c.target_b;
        o->eig_fail_err = c.eig_fail_err; o->unstable_err = c.unstable_err; o->freq = c.freq;
        o->freq_min = c.freq_min; o->dump_diagnostics = c.dump_diagnostics; o->n_threads = c.n_threads;
        o->freq_max = c.freq_max; o->total_dim = c.total_dim; o->dc_dim = c.dc_dim; o->u_dim = c.u_dim;
        o->nl_dim = c.nl_dim; o->cuda_mx_width = c.cuda_mx_width; o->info_scoring = c.info_scoring;
        o->info_freqresp = c.info_freqresp; o->info_allmargin = c.info_allmargin; o->info_modal = c.info_modal;
        o->info_mx_width = c.info_mx_width; o->eigen_mx_width = c.eigen_mx_width; o->lina_mx_width = c.lina_mx_width;
        o->ata_mx_width = c.ata_mx_width; o->atb_mx_width = c.atb_mx_width;
        o->nl_instructions_total = c.nl_instructions_total;
        o->ts = c.ts; o->fit_t0 = c.fit_t0; o->fit_t1 = c.fit_t1; o->damping2 = c.damping2; o->damping4 = c.damping4;
        o->crossover = c.crossover; o->fit_start_id = p.fit_start_id; o->steady_start_id = p.steady_start_id;
        return 0;
    } catch (const std::exception& e) {
        std::snprintf(err, errlen, "%s", e.what());
        return 1;
    }
}
}
