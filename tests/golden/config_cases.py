"""Config cases (valid and invalid) shared by the fixture generator and the test."""
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parents[2]))


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


def cases():
    from controllerengine_gb300 import synth
    a = synth.mass_spring(1536).config_text
    b = synth.eight_state(n=1536, time=10000).config_text
    out = {"mass_spring": a, "eight_state": b}
    muts = {
        "comment_and_spaces": "# header\n" + a.replace("time = 2000", "   time\t=  2000  # trailing"),
        "hex_float": with_key(a, "ref_amplitude", "0x1.8p+0"),
        "defaults": with_key(with_key(with_key(a, "eig_fail_err", None), "unstable_err", None), "duration", None),
        "serial_ok": with_key(with_key(b, "mode", "serial"), "n_rounds", "3"),
        "dump_1": with_key(a, "dump_diagnostics", "1"),
        "fractional_fit": with_key(with_key(a, "time", "1000"), "fit_end", "0.7"),
        "fit_end_one": with_key(a, "fit_end", "1.0"),
        "nl_empty_entries": with_key(a, "nl_instructions", " 3 , "),
        "ref_step_zero": with_key(a, "ref_step_time", "0"),
        "n_cores_big": with_key(a, "n_cores", "5504"),
        "err_no_eq": a + "bogus\n",
        "err_twice": a + "time = 10\n",
        "err_missing": with_key(a, "freq", None),
        "err_nan_int": with_key(a, "time", "nan"),
        "err_not_number": with_key(a, "time", "12abc"),
        "err_fraction": with_key(a, "time", "2000.5"),
        "err_huge_int": with_key(a, "time", "1e30"),
        "err_ns": with_key(a, "statespace_dim", "9"),
        "err_nd0": with_key(a, "discrete_dim", "0"),
        "err_nlcount": with_key(a, "nonlin_dim", "2"),
        "err_nl_range": with_key(a, "nl_instructions", "9"),
        "err_nl_many": with_key(a, "nl_instructions", "1,1,1,1,1"),
        "err_params": with_key(a, "n_params", "35"),
        "err_cores_mult": with_key(a, "n_cores", "200"),
        "err_rounds": with_key(a, "n_rounds", "0"),
        "err_mode": with_key(a, "mode", "fast"),
        "err_serial_dims": with_key(a, "mode", "serial"),
        "err_ref_amp": with_key(a, "ref_amplitude", "0"),
        "err_time": with_key(a, "time", "1"),
        "err_duration": with_key(a, "duration", "0"),
        "err_ref_step": with_key(a, "ref_step_time", "1.5"),
        "err_fit_order": with_key(a, "fit_end", "0.01"),
        "err_fit_range": with_key(a, "fit_start", "-0.1"),
        "err_steady": with_key(a, "steady_start", "1.0"),
        "err_overshoot": with_key(a, "overshoot", "0"),
        "err_sse": with_key(a, "steady_state_error", "-1"),
        "err_xo_coeff": with_key(a, "crossover_coeff", "0"),
        "err_target_b": with_key(a, "target_b", "1"),
        "err_freq": with_key(a, "freq", "1"),
        "err_freq_min": with_key(a, "freq_min", "5000"),
        "err_dump": with_key(a, "dump_diagnostics", "yes"),
        "err_unknown": a + "zeta = 1\n",
        "err_crossover": with_key(a, "bandwidth", "2000"),
        "err_input_size": with_key(a, "input_size", "-1"),
    }
    out.update(muts)
    return out
