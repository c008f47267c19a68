"""Generates tests/golden/config_golden.json by running the REFERENCE's own
config parser (src/config.cu, built into oracle/_ref/libref_config.so by
`make -C oracle ref`) on every case of config_cases.py.  Run in the container
that has the reference tree; the JSON is committed and read by the tests."""
import ctypes as C
import json
import os
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
from config_cases import cases  # noqa: E402

FIELDS = ["statespace_dim", "discrete_dim", "nonlin_dim", "n_params", "input_size", "dc_instructions",
          "u_instructions"]


class RefOut(C.Structure):
    _fields_ = ([(f, C.c_int) for f in FIELDS] + [("nl_instructions", C.c_int * 4)] +
                [(f, C.c_int) for f in ("n_cores", "n_rounds", "serial", "time")] + [("duration", C.c_float),
                ("ref_step_time", C.c_double)] +
                [(f, C.c_float) for f in ("ref_amplitude", "fit_start", "fit_end", "steady_start", "bandwidth",
                                          "damping", "overshoot", "steady_state_error", "crossover_coeff",
                                          "target_gm", "target_pm", "target_b", "eig_fail_err", "unstable_err")] +
                [("freq", C.c_int), ("freq_min", C.c_float), ("dump_diagnostics", C.c_int), ("n_threads", C.c_int),
                 ("freq_max", C.c_float)] +
                [(f, C.c_int) for f in ("total_dim", "dc_dim", "u_dim", "nl_dim", "cuda_mx_width", "info_scoring",
                                        "info_freqresp", "info_allmargin", "info_modal", "info_mx_width",
                                        "eigen_mx_width", "lina_mx_width", "ata_mx_width", "atb_mx_width",
                                        "nl_instructions_total")] +
                [(f, C.c_float) for f in ("ts", "fit_t0", "fit_t1", "damping2", "damping4", "crossover")] +
                [("fit_start_id", C.c_int), ("steady_start_id", C.c_int)])


def main():
    lib = C.CDLL(str(HERE.parents[1] / "oracle" / "_ref" / "libref_config.so"))
    out = {}
    with tempfile.TemporaryDirectory() as d:
        old = os.getcwd()
        os.chdir(d)
        try:
            for name, text in cases().items():
                Path("ControllerEngine.config").write_text(text)
                o = RefOut()
                err = C.create_string_buffer(4096)
                rc = lib.ref_load_config(b"ControllerEngine.config", C.byref(o), err, 4096)
                if rc:
                    out[name] = {"error": err.value.decode()}
                else:
                    rec = {}
                    for f, t in RefOut._fields_:
                        v = getattr(o, f)
                        if f == "nl_instructions":
                            v = list(v)
                        elif t == C.c_float:
                            v = float(v).hex()  # exact
                        elif t == C.c_double:
                            v = float(v).hex()
                        rec[f] = v
                    out[name] = {"config": rec}
        finally:
            os.chdir(old)
    (HERE / "config_golden.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"{len(out)} cases, {sum('error' in v for v in out.values())} errors")


if __name__ == "__main__":
    main()
