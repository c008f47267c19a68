// ce_config.cpp -- ControllerEngine.config parser, size derivation and the
// base-36 instruction decoder.
//
// Same keys, defaults, validation order and error texts as the reference's
// load_config (ref: src/config.cu:106-244), EngineConfig::derive
// (ref: src/config.cu:40-78), make_engine_params (ref: src/config.cu:93-104)
// and decode_instructions (ref: src/main.cu:317-337), so a caller that feeds
// a config or an instruction table the reference rejects gets the same
// message here.  One additive key, `freq_max`, is accepted (see below).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <format>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>

#include "ce_host.h"

namespace ce {

namespace {

constexpr float PI = 0x1.921fb6p+1f;  // float pi (ref: src/main.cu:41)

std::string trim(const std::string& s) {
    const size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// (int)d with the x86/MSVC result for out-of-range values (the "integer
// indefinite" INT_MIN), so the range-check message that follows prints the
// value the reference build prints.
int to_int(double d) {
    if (!(d >= -2147483648.0 && d < 2147483648.0)) return INT32_MIN;
    return (int)d;
}

}  // namespace

void derive(ce_config& c) {
    // ref: src/config.cu:40-78; float arithmetic in the same order.
    c.n_threads = (c.n_cores / 128) * 1536;
    c.ts = c.duration / (float)c.time;
    const float nyquist = PI / c.ts;
    c.freq_max = c.freq_max_key > 0.0f ? c.freq_max_key : nyquist;
    c.total_dim = c.statespace_dim + c.discrete_dim;
    c.dc_dim = c.discrete_dim;
    c.u_dim = c.statespace_dim;
    c.nl_dim = c.discrete_dim + 1;
    c.nl_instructions_total = 0;
    for (int i = 0; i < c.nonlin_dim; i++) c.nl_instructions_total += c.nl_instructions[i];

    // the Kalman row appends R and diag(Q) to the Luenberger row [K, L, N]
    c.cuda_mx_width = c.observer == CE_OBSERVER_KALMAN ? 3 * c.statespace_dim + 2 : 2 * c.statespace_dim + 1;
    c.info_scoring = c.input_size;
    c.info_freqresp = c.info_scoring + 3;
    c.info_allmargin = c.info_freqresp + 4;
    c.info_modal = c.info_allmargin + 5;
    c.info_mx_width = c.info_modal + 3 * c.total_dim + 1;
    c.eigen_mx_width = 2 * c.total_dim;
    c.lina_mx_width = c.total_dim * c.total_dim;
    c.ata_mx_width = 2 * c.total_dim * 2 * c.total_dim;
    c.atb_mx_width = 2 * c.total_dim;

    c.fit_t0 = c.fit_start * c.duration;
    c.fit_t1 = (c.fit_end * (float)c.time - 1.0f) * c.ts;

    c.damping2 = c.damping * c.damping;
    c.damping4 = c.damping2 * c.damping2;
    const float wn = 2.0f * PI * c.bandwidth /
                     sqrtf((1.0f - 2.0f * c.damping2) + sqrtf(4.0f * c.damping4 - 4.0f * c.damping2 + 2.0f));
    c.crossover = c.crossover_coeff * wn * sqrtf(sqrtf(4.0f * c.damping4 + 1.0f) - 2.0f * c.damping2);

    // ref: src/config.cu:99-100
    c.fit_start_id = (int)(c.fit_start * (float)c.time);
    c.steady_start_id = (int)(c.steady_start * (float)c.time);
    // ref: src/modalsetup.cu:75-76 -- `for (int t=0; t<fit_len; t++)` with a float bound
    const float fit_len = (c.fit_end - c.fit_start) * (float)c.time;
    c.fit_steps = fit_len > 0.0f ? (int)ceilf(fit_len) : 0;
    // ref: src/main.cu:414 -- reference is 0 while t < ref_step_time*time (double compare)
    const double step_at = c.ref_step_time * (double)c.time;
    int rid = 0;
    if (step_at > 0.0) rid = step_at >= (double)c.time ? c.time : (int)std::ceil(step_at);
    c.ref_step_id = rid;
}

void parse_config(const std::string& text, const std::string& filename, ce_config& out) {
    std::map<std::string, std::string> kv;
    std::istringstream file(text);
    std::string line;
    int lineno = 0;
    while (std::getline(file, line)) {
        lineno++;
        line = trim(line.substr(0, line.find('#')));
        if (line.empty()) continue;
        const size_t eq = line.find('=');
        if (eq == std::string::npos) fail("{}:{}: expected `key = value`, got `{}`", filename, lineno, line);
        const std::string key = trim(line.substr(0, eq));
        if (kv.count(key)) fail("{}:{}: `{}` is set twice", filename, lineno, key);
        kv[key] = trim(line.substr(eq + 1));
    }

    // every key read is erased; what is left at the end is unknown
    auto take = [&](const std::string& key, const char* fallback = nullptr) {
        auto it = kv.find(key);
        if (it == kv.end()) {
            if (fallback) return std::string(fallback);
            fail("{}: missing `{}`", filename, key);
        }
        std::string v = it->second;
        kv.erase(it);
        return v;
    };
    auto as_double = [&](const std::string& key, const std::string& v) {
        char* end = nullptr;
        const double d = std::strtod(v.c_str(), &end);
        if (v.empty() || *end != '\0') fail("{}: `{}` should be a number, got `{}`", filename, key, v);
        return d;
    };
    auto as_int = [&](const std::string& key, const std::string& v) {
        const double d = as_double(key, v);
        if (d != std::floor(d)) fail("{}: `{}` should be an integer, got `{}`", filename, key, v);
        return to_int(d);
    };
    auto get_int = [&](const std::string& key, const char* fallback = nullptr) { return as_int(key, take(key, fallback)); };
    auto get_float = [&](const std::string& key, const char* fallback = nullptr) {
        return (float)as_double(key, take(key, fallback));
    };
    auto in_range = [&](const char* key, double v, double lo, double hi) {
        if (v < lo || v > hi) fail("{}: `{}` = {} is outside [{}, {}]", filename, key, v, lo, hi);
    };

    ce_config c;
    std::memset(&c, 0, sizeof(c));
    c.statespace_dim = get_int("statespace_dim");
    c.discrete_dim = get_int("discrete_dim");
    c.nonlin_dim = get_int("nonlin_dim");
    c.n_params = get_int("n_params");
    c.input_size = get_int("input_size");
    c.dc_instructions = get_int("dc_instructions");
    c.u_instructions = get_int("u_instructions");
    in_range("statespace_dim", c.statespace_dim, 1, CE_MAX_STATESPACE_DIM);
    in_range("discrete_dim", c.discrete_dim, 1, CE_MAX_DISCRETE_DIM);
    in_range("nonlin_dim", c.nonlin_dim, 0, CE_MAX_NONLIN_DIM);
    in_range("n_params", c.n_params, 1, CE_MAX_PARAMS);
    in_range("input_size", c.input_size, 0, 1 << 20);
    in_range("dc_instructions", c.dc_instructions, 0, CE_MAX_DC_INSTRUCTIONS);
    in_range("u_instructions", c.u_instructions, 0, CE_MAX_U_INSTRUCTIONS);

    {
        std::stringstream list(take("nl_instructions", ""));
        std::string item;
        int n = 0;
        while (std::getline(list, item, ',')) {
            item = trim(item);
            if (item.empty()) continue;
            if (n >= CE_MAX_NONLIN_DIM)
                fail("{}: `nl_instructions` has more than MAX_NONLIN_DIM = {} entries", filename, CE_MAX_NONLIN_DIM);
            c.nl_instructions[n] = as_int("nl_instructions", item);
            in_range("nl_instructions", c.nl_instructions[n], 0, CE_MAX_NL_INSTRUCTIONS);
            n++;
        }
        if (n != c.nonlin_dim)
            fail("{}: `nl_instructions` has {} entries but nonlin_dim is {}", filename, n, c.nonlin_dim);
    }

    c.n_cores = get_int("n_cores");
    c.n_rounds = get_int("n_rounds", "1");
    in_range("n_cores", c.n_cores, 128, 1 << 20);
    if (c.n_cores % 128 != 0) fail("{}: `n_cores` = {} should be a multiple of 128 (cores per SM)", filename, c.n_cores);
    in_range("n_rounds", c.n_rounds, 1, 1 << 20);
    {
        const std::string v = take("mode", "batch");
        if (v == "batch") c.serial = 0;
        else if (v == "serial") c.serial = 1;
        else fail("{}: `mode` should be batch/serial, got `{}`", filename, v);
        if (c.serial && c.statespace_dim != c.discrete_dim)
            fail("{}: mode = serial needs statespace_dim ({}) == discrete_dim ({})", filename, c.statespace_dim,
                 c.discrete_dim);
    }

    c.time = get_int("time");
    c.ref_step_time = as_double("ref_step_time", take("ref_step_time"));
    c.ref_amplitude = get_float("ref_amplitude");
    if (!(c.ref_amplitude != 0.0f)) fail("{}: need ref_amplitude != 0", filename);
    in_range("time", c.time, 2, 1 << 24);
    c.duration = get_float("duration", "1.0");
    if (!(c.duration > 0.0f)) fail("{}: need duration > 0", filename);
    in_range("ref_step_time", c.ref_step_time, 0.0, 1.0);

    c.fit_start = get_float("fit_start");
    c.fit_end = get_float("fit_end");
    c.steady_start = get_float("steady_start");
    in_range("fit_start", c.fit_start, 0.0, 1.0);
    in_range("fit_end", c.fit_end, 0.0, 1.0);
    in_range("steady_start", c.steady_start, 0.0, 1.0);
    if (!(c.fit_start < c.fit_end))
        fail("{}: fit_start ({}) must be below fit_end ({})", filename, c.fit_start, c.fit_end);
    if ((int)(c.steady_start * (float)c.time) >= c.time) fail("{}: steady_start leaves no samples to average", filename);

    c.bandwidth = get_float("bandwidth");
    c.damping = get_float("damping");
    c.overshoot = get_float("overshoot");
    c.steady_state_error = get_float("steady_state_error");
    c.crossover_coeff = get_float("crossover_coeff");
    c.target_gm = get_float("target_gm");
    c.target_pm = get_float("target_pm");
    c.target_b = get_float("target_b");
    if (!(c.overshoot > 0.0f)) fail("{}: need overshoot > 0", filename);
    if (!(c.steady_state_error > 0.0f)) fail("{}: need steady_state_error > 0", filename);
    if (!(c.crossover_coeff > 0.0f)) fail("{}: need crossover_coeff > 0", filename);
    if (!(c.target_b > 0.0f && c.target_b < 1.0f)) fail("{}: need 0 < target_b < 1", filename);
    c.eig_fail_err = get_float("eig_fail_err", "1.0e18");
    c.unstable_err = get_float("unstable_err", "1.0e6");

    c.freq = get_int("freq");
    c.freq_min = get_float("freq_min");
    in_range("freq", c.freq, 2, 1 << 20);
    if (!(c.freq_min > 0.0f && c.freq_min < PI * (float)c.time / c.duration))
        fail("{}: need 0 < freq_min < pi*time/duration (Nyquist)", filename);

    {
        const std::string v = take("dump_diagnostics", "false");
        if (v == "true" || v == "1") c.dump_diagnostics = 1;
        else if (v == "false" || v == "0") c.dump_diagnostics = 0;
        else fail("{}: `dump_diagnostics` should be true/false, got `{}`", filename, v);
    }

    // Additive key (not in the reference): end of the sweep in rad/s, 0 = Nyquist.
    c.freq_max_key = get_float("freq_max", "0");
    if (c.freq_max_key != 0.0f &&
        !(c.freq_max_key > c.freq_min && c.freq_max_key <= PI * (float)c.time / c.duration))
        fail("{}: need freq_min < freq_max <= pi*time/duration (Nyquist)", filename);

    // Additive key: the time-varying Kalman observer (ref: src/discrete_solves.cu:83-185).
    {
        const std::string v = take("observer", "luenberger");
        if (v == "luenberger") c.observer = CE_OBSERVER_LUENBERGER;
        else if (v == "kalman") c.observer = CE_OBSERVER_KALMAN;
        else fail("{}: `observer` should be luenberger/kalman, got `{}`", filename, v);
    }

    if (!kv.empty()) fail("{}: unknown key `{}`", filename, kv.begin()->first);

    derive(c);
    const float nyquist = PI / c.ts;
    if (!(c.crossover > 0.0f && c.crossover < nyquist))
        fail("{}: crossover {} rad/s (from bandwidth, damping, crossover_coeff) must be in (0, Nyquist = {})", filename,
             c.crossover, nyquist);
    out = c;
}

// ref: src/main.cu:317-337.  `base_params` is the round's BASE_PARAMS.
void decode_instructions(const int32_t* info, int dim, int count, const float* base_params, int n_params,
                         ce_instruction* out) {
    auto kind = [](int digit) {
        return digit == 0 ? CE_OPERAND_STATE : (digit == 35 ? CE_OPERAND_PREV : CE_OPERAND_CONST);
    };
    auto val = [&](int digit) {
        if (digit == 0 || digit == 35) return 0.0f;
        if (digit - 1 >= n_params)
            fail("instruction digit {} needs BASE_PARAMS[{}] but n_params is {}", digit, digit - 1, n_params);
        // A negative packed entry gives a negative digit, which the reference
        // looks up below BASE_PARAMS; its op is then <= 0 (a SKIP or a no-op),
        // so the value is never read.  0 is stored instead of reading out of bounds.
        if (digit < 1) return 0.0f;
        return base_params[digit - 1];
    };
    for (int r = 0; r < count; r++) {
        const int32_t* row = &info[(size_t)r * dim];
        int packed = 0, col = 0;
        for (int c = 0; c < dim; c++)
            if (row[c] != 0) {
                packed = row[c];
                col = c;
            }
        out[r] = ce_instruction{0, 0, CE_OPERAND_CONST, CE_OPERAND_CONST, 0.0f, 0.0f};
        if (packed == 0) continue;
        const int i1 = (packed / 36) % 36;
        const int i2 = packed % 36;
        // braced initialisation evaluates left to right: digit 1 is checked first
        const int op = packed / 1296;
        const int k1 = kind(i1), k2 = kind(i2);
        const float v1 = val(i1);
        const float v2 = val(i2);
        out[r] = ce_instruction{op, col, k1, k2, v1, v2};
    }
}

}  // namespace ce
