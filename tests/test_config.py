"""Config parser: keys, defaults, derived sizes and the reference's error texts
(ref: src/config.cu:106-244, 40-78).  CPU only."""
import numpy as np
import pytest

import controllerengine_gb300 as ce
from controllerengine_gb300 import synth

F = np.float32
BASE = synth.mass_spring(1536).config_text
NEXT = len(BASE.splitlines()) + 1  # line number of an appended line


def parse(text):
    return ce.EngineConfig.parse(text)


def with_key(text, key, value):
    out, found = [], False
    for line in text.splitlines():
        k = line.split("=", 1)[0].strip()
        if k == key:
            found = True
            if value is None:
                continue
            line = f"{key} = {value}"
        out.append(line)
    if not found and value is not None:
        out.append(f"{key} = {value}")
    return "\n".join(out) + "\n"


def test_derived_sizes(lib):
    c = parse(BASE)
    assert (c.statespace_dim, c.discrete_dim, c.nonlin_dim, c.total_dim) == (3, 2, 1, 5)
    assert c.n_threads == 1536 and c.n_rounds == 1 and c.serial == 0
    assert c.cuda_mx_width == 7
    assert (c.info_scoring, c.info_freqresp, c.info_allmargin, c.info_modal) == (7, 10, 14, 19)
    assert c.info_mx_width == 19 + 3 * 5 + 1
    assert (c.eigen_mx_width, c.lina_mx_width, c.ata_mx_width, c.atb_mx_width) == (10, 25, 100, 10)
    # float arithmetic of derive(), in the reference's order
    ts = F(2.0) / F(2000)
    assert c.ts == ts
    assert c.freq_max == F(F(np.pi)) / ts
    assert c.fit_t0 == F(0.05) * F(2.0)
    assert c.fit_t1 == (F(0.75) * F(2000) - F(1.0)) * ts
    assert c.fit_start_id == int(F(0.05) * F(2000)) == 100
    assert c.steady_start_id == 1500
    assert c.fit_steps == 1400
    assert c.ref_step_id == 100
    d2 = F(0.59) * F(0.59)
    d4 = d2 * d2
    wn = F(2.0) * F(np.pi) * F(0.5) / np.sqrt((F(1) - F(2) * d2) + np.sqrt(F(4) * d4 - F(4) * d2 + F(2)), dtype=F)
    xo = F(1.0) * wn * np.sqrt(np.sqrt(F(4) * d4 + F(1), dtype=F) - F(2) * d2, dtype=F)
    assert abs(c.crossover - xo) <= 2 * np.spacing(xo)


def test_defaults(lib):
    c = parse(with_key(with_key(BASE, "eig_fail_err", None), "unstable_err", None))
    assert c.eig_fail_err == F(1e18) and c.unstable_err == F(1e6)
    c = parse(with_key(BASE, "duration", None).replace("ref_step_time = 0.05", "ref_step_time = 0.05"))
    assert c.duration == 1.0
    assert c.dump_diagnostics == 0


def test_comments_whitespace_hex(lib):
    t = "# comment line\n" + BASE.replace("time = 2000", "  time   =   2000   # trailing")
    t = t.replace("ref_amplitude = 1.0", "ref_amplitude = 0x1p+0")
    c = parse(t)
    assert c.time == 2000 and c.ref_amplitude == 1.0


ERRORS = [
    (lambda t: t + "bogus\n", f"ControllerEngine.config:{NEXT}: expected `key = value`, got `bogus`"),
    (lambda t: t + "time = 10\n", f"ControllerEngine.config:{NEXT}: `time` is set twice"),
    (lambda t: with_key(t, "freq", None), "ControllerEngine.config: missing `freq`"),
    (lambda t: with_key(t, "time", "abc"), "ControllerEngine.config: `time` should be a number, got `abc`"),
    (lambda t: with_key(t, "time", "2000.5"), "ControllerEngine.config: `time` should be an integer, got `2000.5`"),
    (lambda t: with_key(t, "statespace_dim", "9"), "ControllerEngine.config: `statespace_dim` = 9 is outside [1, 8]"),
    (lambda t: with_key(t, "nonlin_dim", "2"), "ControllerEngine.config: `nl_instructions` has 1 entries but nonlin_dim is 2"),
    (lambda t: with_key(t, "nl_instructions", "9"), "ControllerEngine.config: `nl_instructions` = 9 is outside [0, 8]"),
    (lambda t: with_key(t, "nl_instructions", "1,1,1,1,1"), "ControllerEngine.config: `nl_instructions` has more than MAX_NONLIN_DIM = 4 entries"),
    (lambda t: with_key(t, "n_cores", "200"), "ControllerEngine.config: `n_cores` = 200 should be a multiple of 128 (cores per SM)"),
    (lambda t: with_key(t, "mode", "fast"), "ControllerEngine.config: `mode` should be batch/serial, got `fast`"),
    (lambda t: with_key(t, "mode", "serial"), "ControllerEngine.config: mode = serial needs statespace_dim (3) == discrete_dim (2)"),
    (lambda t: with_key(t, "ref_amplitude", "0"), "ControllerEngine.config: need ref_amplitude != 0"),
    (lambda t: with_key(t, "time", "1"), "ControllerEngine.config: `time` = 1 is outside [2, 16777216]"),
    (lambda t: with_key(t, "duration", "-1"), "ControllerEngine.config: need duration > 0"),
    (lambda t: with_key(t, "ref_step_time", "1.5"), "ControllerEngine.config: `ref_step_time` = 1.5 is outside [0, 1]"),
    (lambda t: with_key(t, "fit_end", "0.01"), "ControllerEngine.config: fit_start (0.05) must be below fit_end (0.01)"),
    (lambda t: with_key(t, "steady_start", "1.0"), "ControllerEngine.config: steady_start leaves no samples to average"),
    (lambda t: with_key(t, "overshoot", "0"), "ControllerEngine.config: need overshoot > 0"),
    (lambda t: with_key(t, "steady_state_error", "0"), "ControllerEngine.config: need steady_state_error > 0"),
    (lambda t: with_key(t, "crossover_coeff", "0"), "ControllerEngine.config: need crossover_coeff > 0"),
    (lambda t: with_key(t, "target_b", "1"), "ControllerEngine.config: need 0 < target_b < 1"),
    (lambda t: with_key(t, "freq", "1"), "ControllerEngine.config: `freq` = 1 is outside [2, 1048576]"),
    (lambda t: with_key(t, "freq_min", "5000"), "ControllerEngine.config: need 0 < freq_min < pi*time/duration (Nyquist)"),
    (lambda t: with_key(t, "dump_diagnostics", "yes"), "ControllerEngine.config: `dump_diagnostics` should be true/false, got `yes`"),
    (lambda t: t + "zeta = 1\n", "ControllerEngine.config: unknown key `zeta`"),
    (lambda t: with_key(t, "bandwidth", "2000"),
     "ControllerEngine.config: crossover"),
]


@pytest.mark.parametrize("mutate,msg", ERRORS)
def test_errors(lib, mutate, msg):
    with pytest.raises(ce.ControllerEngineError) as e:
        parse(mutate(BASE))
    assert str(e.value).startswith(msg), str(e.value)


def test_fit_steps_rounding(lib):
    # `for (int t=0; t<fit_len; t++)` with a float bound: ceil for a fractional bound
    t = with_key(with_key(BASE, "time", "1000"), "fit_end", "0.7")
    c = parse(t)
    fit_len = (F(0.7) - F(0.05)) * F(1000)
    assert c.fit_steps == int(np.ceil(fit_len))
