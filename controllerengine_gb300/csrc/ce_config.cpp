// ce_config.cpp -- ControllerEngine.config parser, size derivation and the
// base-36 instruction decoder.
//
// The file format, its keys, defaults and error texts, and the order in which
// problems are reported are the reference's interface (ref:
// src/config.cu:106-244, load_config), as are the derived sizes
// (ref: src/config.cu:40-78, 93-104) and the base-36 decoding
// (ref: src/main.cu:317-337): a caller that feeds a config or an instruction
// table the reference rejects gets the same message here.  The parser itself
// is table-driven (key table + check schedule, below).  Two additive keys,
// `freq_max` and `observer`, are accepted.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <format>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

#include "ce_host.h"

namespace ce {

namespace {

constexpr float PI = 0x1.921fb6p+1f;  // float pi (ref: src/main.cu:41)

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

// ---------------------------------------------------------------------------
// The parser is data: a table of keys (how each value is read and where it is
// stored) and a schedule of steps walked in order.  A step reads one key,
// range-checks one field, or tests one rule across fields.  The order of the
// schedule is part of the interface -- a file with several problems must
// report the same one first as the reference does -- and is pinned by the
// golden cases of the reference's own parser.

namespace {

struct Word {
    const char* text;
    int value;
};

// How a key's text becomes a value.
enum class Kind { Int, Float, Double, Words, IntList };

struct KeySpec {
    const char* name;
    Kind kind;
    const char* dflt;  // nullptr: the key must be present
    // destination: exactly one of these, by kind
    int32_t ce_config::* i = nullptr;
    float ce_config::* f = nullptr;
    double ce_config::* d = nullptr;
    const Word* words = nullptr;  // Words: accepted spellings, ended by {nullptr, 0}
    const char* spelled = nullptr;  // Words: how the error message lists them
};

constexpr Word kModeWords[] = {{"batch", 0}, {"serial", 1}, {nullptr, 0}};
constexpr Word kFlagWords[] = {{"true", 1}, {"1", 1}, {"false", 0}, {"0", 0}, {nullptr, 0}};
constexpr Word kObserverWords[] = {
    {"luenberger", CE_OBSERVER_LUENBERGER}, {"kalman", CE_OBSERVER_KALMAN}, {nullptr, 0}};

KeySpec int_key(const char* n, int32_t ce_config::* m, const char* dflt = nullptr) {
    KeySpec k{n, Kind::Int, dflt};
    k.i = m;
    return k;
}
KeySpec float_key(const char* n, float ce_config::* m, const char* dflt = nullptr) {
    KeySpec k{n, Kind::Float, dflt};
    k.f = m;
    return k;
}
KeySpec words_key(const char* n, int32_t ce_config::* m, const char* dflt, const Word* w, const char* spelled) {
    KeySpec k{n, Kind::Words, dflt};
    k.i = m;
    k.words = w;
    k.spelled = spelled;
    return k;
}

const std::vector<KeySpec>& key_table() {
    static const std::vector<KeySpec> keys = [] {
        std::vector<KeySpec> k;
        k.push_back(int_key("statespace_dim", &ce_config::statespace_dim));
        k.push_back(int_key("discrete_dim", &ce_config::discrete_dim));
        k.push_back(int_key("nonlin_dim", &ce_config::nonlin_dim));
        k.push_back(int_key("n_params", &ce_config::n_params));
        k.push_back(int_key("input_size", &ce_config::input_size));
        k.push_back(int_key("dc_instructions", &ce_config::dc_instructions));
        k.push_back(int_key("u_instructions", &ce_config::u_instructions));
        k.push_back(KeySpec{"nl_instructions", Kind::IntList, ""});
        k.push_back(int_key("n_cores", &ce_config::n_cores));
        k.push_back(int_key("n_rounds", &ce_config::n_rounds, "1"));
        k.push_back(words_key("mode", &ce_config::serial, "batch", kModeWords, "batch/serial"));
        k.push_back(int_key("time", &ce_config::time));
        {
            KeySpec r{"ref_step_time", Kind::Double, nullptr};
            r.d = &ce_config::ref_step_time;
            k.push_back(r);
        }
        k.push_back(float_key("ref_amplitude", &ce_config::ref_amplitude));
        k.push_back(float_key("duration", &ce_config::duration, "1.0"));
        k.push_back(float_key("fit_start", &ce_config::fit_start));
        k.push_back(float_key("fit_end", &ce_config::fit_end));
        k.push_back(float_key("steady_start", &ce_config::steady_start));
        k.push_back(float_key("bandwidth", &ce_config::bandwidth));
        k.push_back(float_key("damping", &ce_config::damping));
        k.push_back(float_key("overshoot", &ce_config::overshoot));
        k.push_back(float_key("steady_state_error", &ce_config::steady_state_error));
        k.push_back(float_key("crossover_coeff", &ce_config::crossover_coeff));
        k.push_back(float_key("target_gm", &ce_config::target_gm));
        k.push_back(float_key("target_pm", &ce_config::target_pm));
        k.push_back(float_key("target_b", &ce_config::target_b));
        k.push_back(float_key("eig_fail_err", &ce_config::eig_fail_err, "1.0e18"));
        k.push_back(float_key("unstable_err", &ce_config::unstable_err, "1.0e6"));
        k.push_back(int_key("freq", &ce_config::freq));
        k.push_back(float_key("freq_min", &ce_config::freq_min));
        k.push_back(words_key("dump_diagnostics", &ce_config::dump_diagnostics, "false", kFlagWords, "true/false"));
        // additive keys (no counterpart in the reference's file): the end of the
        // sweep in rad/s (0 = Nyquist) and the observer of the simulated loop
        k.push_back(float_key("freq_max", &ce_config::freq_max_key, "0"));
        k.push_back(words_key("observer", &ce_config::observer, "luenberger", kObserverWords, "luenberger/kalman"));
        return k;
    }();
    return keys;
}

const KeySpec& spec_of(std::string_view name) {
    for (const KeySpec& k : key_table())
        if (name == k.name) return k;
    throw std::logic_error("config schedule names an unlisted key");
}

// The parsed state the rules look at: the configuration so far and the
// number of entries the nl_instructions list had.
struct State {
    ce_config c;
    int nl_entries = 0;
};

using Rule = bool (*)(const State&);
using Why = std::string (*)(const State&);

struct Step {
    enum Op { Read, Range, Check } op;
    const char* key = nullptr;  // Read, Range
    double lo = 0, hi = 0;      // Range (inclusive)
    Rule holds = nullptr;       // Check
    Why why = nullptr;          // Check: the message after "<file>: "
};

Step read(const char* k) { return Step{Step::Read, k}; }
Step range(const char* k, double lo, double hi) { return Step{Step::Range, k, lo, hi}; }
Step check(Rule r, Why w) { return Step{Step::Check, nullptr, 0, 0, r, w}; }

// The time axis and the sweep bound derived from a partially read file.
float nyquist_of(const ce_config& c) { return PI * (float)c.time / c.duration; }

const std::vector<Step>& schedule() {
    static const std::vector<Step> steps = {
        read("statespace_dim"), read("discrete_dim"), read("nonlin_dim"), read("n_params"), read("input_size"),
        read("dc_instructions"), read("u_instructions"),
        range("statespace_dim", 1, CE_MAX_STATESPACE_DIM), range("discrete_dim", 1, CE_MAX_DISCRETE_DIM),
        range("nonlin_dim", 0, CE_MAX_NONLIN_DIM), range("n_params", 1, CE_MAX_PARAMS),
        range("input_size", 0, 1 << 20), range("dc_instructions", 0, CE_MAX_DC_INSTRUCTIONS),
        range("u_instructions", 0, CE_MAX_U_INSTRUCTIONS),
        read("nl_instructions"),
        check([](const State& s) { return s.nl_entries == s.c.nonlin_dim; },
              [](const State& s) {
                  return std::format("`nl_instructions` has {} entries but nonlin_dim is {}", s.nl_entries,
                                     s.c.nonlin_dim);
              }),
        read("n_cores"), read("n_rounds"),
        range("n_cores", 128, 1 << 20),
        check([](const State& s) { return s.c.n_cores % 128 == 0; },
              [](const State& s) {
                  return std::format("`n_cores` = {} should be a multiple of 128 (cores per SM)", s.c.n_cores);
              }),
        range("n_rounds", 1, 1 << 20),
        read("mode"),
        // the margin sweep of the serial mode puts the true plant where the observer model was
        check([](const State& s) { return !s.c.serial || s.c.statespace_dim == s.c.discrete_dim; },
              [](const State& s) {
                  return std::format("mode = serial needs statespace_dim ({}) == discrete_dim ({})",
                                     s.c.statespace_dim, s.c.discrete_dim);
              }),
        read("time"), read("ref_step_time"), read("ref_amplitude"),
        check([](const State& s) { return s.c.ref_amplitude != 0.0f; },
              [](const State&) { return std::string("need ref_amplitude != 0"); }),
        range("time", 2, 1 << 24),
        read("duration"),
        check([](const State& s) { return s.c.duration > 0.0f; },
              [](const State&) { return std::string("need duration > 0"); }),
        range("ref_step_time", 0.0, 1.0),
        read("fit_start"), read("fit_end"), read("steady_start"),
        range("fit_start", 0.0, 1.0), range("fit_end", 0.0, 1.0), range("steady_start", 0.0, 1.0),
        check([](const State& s) { return s.c.fit_start < s.c.fit_end; },
              [](const State& s) {
                  return std::format("fit_start ({}) must be below fit_end ({})", s.c.fit_start, s.c.fit_end);
              }),
        check([](const State& s) { return (int)(s.c.steady_start * (float)s.c.time) < s.c.time; },
              [](const State&) { return std::string("steady_start leaves no samples to average"); }),
        read("bandwidth"), read("damping"), read("overshoot"), read("steady_state_error"), read("crossover_coeff"),
        read("target_gm"), read("target_pm"), read("target_b"),
        check([](const State& s) { return s.c.overshoot > 0.0f; },
              [](const State&) { return std::string("need overshoot > 0"); }),
        check([](const State& s) { return s.c.steady_state_error > 0.0f; },
              [](const State&) { return std::string("need steady_state_error > 0"); }),
        check([](const State& s) { return s.c.crossover_coeff > 0.0f; },
              [](const State&) { return std::string("need crossover_coeff > 0"); }),
        check([](const State& s) { return s.c.target_b > 0.0f && s.c.target_b < 1.0f; },
              [](const State&) { return std::string("need 0 < target_b < 1"); }),
        read("eig_fail_err"), read("unstable_err"),
        read("freq"), read("freq_min"),
        range("freq", 2, 1 << 20),
        check([](const State& s) { return s.c.freq_min > 0.0f && s.c.freq_min < nyquist_of(s.c); },
              [](const State&) { return std::string("need 0 < freq_min < pi*time/duration (Nyquist)"); }),
        read("dump_diagnostics"),
        read("freq_max"),
        check([](const State& s) {
                  const float f = s.c.freq_max_key;
                  return f == 0.0f || (f > s.c.freq_min && f <= nyquist_of(s.c));
              },
              [](const State&) { return std::string("need freq_min < freq_max <= pi*time/duration (Nyquist)"); }),
        read("observer"),
    };
    return steps;
}

bool blank(char ch) { return ch == ' ' || ch == '\t' || ch == '\r' || ch == '\n'; }

std::string_view strip(std::string_view s) {
    size_t a = 0, b = s.size();
    while (a < b && blank(s[a])) ++a;
    while (b > a && blank(s[b - 1])) --b;
    return s.substr(a, b - a);
}

// The file as key -> value text; a line is `key = value`, text from `#` on is
// a comment, blank lines are skipped.
std::map<std::string, std::string> split_entries(const std::string& text, const std::string& file) {
    std::map<std::string, std::string> kv;
    size_t pos = 0;
    int lineno = 0;
    while (pos < text.size()) {
        size_t end = text.find('\n', pos);
        if (end == std::string::npos) end = text.size();
        std::string_view line(text.data() + pos, end - pos);
        pos = end + 1;
        ++lineno;
        line = strip(line.substr(0, line.find('#')));
        if (line.empty()) continue;
        const size_t eq = line.find('=');
        if (eq == std::string_view::npos) fail("{}:{}: expected `key = value`, got `{}`", file, lineno, line);
        std::string key(strip(line.substr(0, eq)));
        if (kv.contains(key)) fail("{}:{}: `{}` is set twice", file, lineno, key);
        kv.emplace(std::move(key), std::string(strip(line.substr(eq + 1))));
    }
    return kv;
}

// A number as strtod reads it (hex floats included), the whole text consumed.
double number(const std::string& file, const char* key, const std::string& v) {
    const char* s = v.c_str();
    char* stop = nullptr;
    const double d = std::strtod(s, &stop);
    if (v.empty() || *stop != '\0') fail("{}: `{}` should be a number, got `{}`", file, key, v);
    return d;
}

int integer(const std::string& file, const char* key, const std::string& v) {
    const double d = number(file, key, v);
    if (std::floor(d) != d) fail("{}: `{}` should be an integer, got `{}`", file, key, v);
    return to_int(d);
}

void fail_range(const std::string& file, const char* key, double v, double lo, double hi) {
    fail("{}: `{}` = {} is outside [{}, {}]", file, key, v, lo, hi);
}

// The nl_instructions list: comma-separated counts, empty items skipped.
int read_list(const std::string& file, const std::string& v, int32_t* out) {
    int n = 0;
    size_t pos = 0;
    while (pos <= v.size()) {
        size_t comma = v.find(',', pos);
        if (comma == std::string::npos) comma = v.size();
        const std::string item(strip(std::string_view(v).substr(pos, comma - pos)));
        pos = comma + 1;
        if (item.empty()) continue;
        if (n == CE_MAX_NONLIN_DIM)
            fail("{}: `nl_instructions` has more than MAX_NONLIN_DIM = {} entries", file, CE_MAX_NONLIN_DIM);
        const int k = integer(file, "nl_instructions", item);
        if (k < 0 || k > CE_MAX_NL_INSTRUCTIONS) fail_range(file, "nl_instructions", k, 0, CE_MAX_NL_INSTRUCTIONS);
        out[n++] = k;
    }
    return n;
}

double field_value(const ce_config& c, const KeySpec& k) {
    if (k.i) return c.*k.i;
    if (k.f) return c.*k.f;
    return c.*k.d;
}

}  // namespace

void parse_config(const std::string& text, const std::string& filename, ce_config& out) {
    const std::map<std::string, std::string> kv = split_entries(text, filename);
    std::set<std::string> used;
    State s;
    std::memset(&s.c, 0, sizeof(s.c));
    for (const Step& st : schedule()) {
        if (st.op == Step::Check) {
            if (!st.holds(s)) fail("{}: {}", filename, st.why(s));
            continue;
        }
        const KeySpec& k = spec_of(st.key);
        if (st.op == Step::Range) {
            const double v = field_value(s.c, k);
            if (v < st.lo || v > st.hi) fail_range(filename, k.name, v, st.lo, st.hi);
            continue;
        }
        std::string v;
        if (const auto it = kv.find(k.name); it != kv.end()) {
            v = it->second;
            used.insert(it->first);
        } else if (k.dflt) {
            v = k.dflt;
        } else {
            fail("{}: missing `{}`", filename, k.name);
        }
        switch (k.kind) {
            case Kind::Int: s.c.*k.i = integer(filename, k.name, v); break;
            case Kind::Float: s.c.*k.f = (float)number(filename, k.name, v); break;
            case Kind::Double: s.c.*k.d = number(filename, k.name, v); break;
            case Kind::IntList: s.nl_entries = read_list(filename, v, s.c.nl_instructions); break;
            case Kind::Words: {
                const Word* w = k.words;
                while (w->text && v != w->text) ++w;
                if (!w->text) fail("{}: `{}` should be {}, got `{}`", filename, k.name, k.spelled, v);
                s.c.*k.i = w->value;
                break;
            }
        }
    }
    // a key no step read is a typo or a stale key: the first one in name order is reported
    for (const auto& [key, value] : kv)
        if (!used.contains(key)) fail("{}: unknown key `{}`", filename, key);

    derive(s.c);
    const float nyquist = PI / s.c.ts;
    if (!(s.c.crossover > 0.0f && s.c.crossover < nyquist))
        fail("{}: crossover {} rad/s (from bandwidth, damping, crossover_coeff) must be in (0, Nyquist = {})", filename,
             s.c.crossover, nyquist);
    out = s.c;
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
