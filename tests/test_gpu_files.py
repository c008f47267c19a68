"""The drop-in file boundary: RunControllerEngine() on the reference's file set
(ref: src/main.cu:385-602), its outputs, diagnostics and error.log behaviour."""
import numpy as np
import pytest

import controllerengine_gb300 as ce
from controllerengine_gb300 import synth

pytestmark = pytest.mark.gpu


def test_run_controller_engine_matches_session(lib, mass_spring, tmp_path):
    p = mass_spring
    p.write(tmp_path)
    assert ce.run_controller_engine(tmp_path) == 0
    cfg = ce.EngineConfig.parse(p.config_text)
    out = np.fromfile(tmp_path / "INFO_MX_OUT.bin", np.float32).reshape(-1, cfg.info_mx_width)
    with ce.Session(cfg, p.plant) as s:
        ref = s.evaluate(p.cuda_mx, p.info_mx)
    assert np.array_equal(out, ref, equal_nan=True)
    log = (tmp_path / "params.log").read_text().splitlines()
    assert log[0] == "BASE_PARAMS_HOST[0] = 5.000000000e-01"
    assert log[-1] == "ref amplitude = 1.000000000e+00"


def test_dump_diagnostics_and_rounds(lib, mass_spring, tmp_path):
    p = mass_spring
    text = p.config_text.replace("n_rounds = 1", "n_rounds = 2") + "dump_diagnostics = true\n"
    g = np.vstack([p.cuda_mx, p.cuda_mx[::-1]])
    info = np.vstack([p.info_mx, p.info_mx[::-1]])
    synth.Problem("two_rounds", text, p.plant, g, info).write(tmp_path)
    assert ce.run_controller_engine(tmp_path) == 0
    cfg = ce.EngineConfig.parse(text)
    out = np.fromfile(tmp_path / "INFO_MX_OUT.bin", np.float32).reshape(2, 1536, cfg.info_mx_width)
    with ce.Session(cfg, p.plant) as s:
        r1, d = s.evaluate_diagnostics(p.cuda_mx[::-1].copy(), p.info_mx[::-1].copy())
    assert np.array_equal(out[1], r1, equal_nan=True)
    # diagnostics hold the last round
    y = np.fromfile(tmp_path / "YPLANT_OUT.bin", np.float32).reshape(1536, cfg.time)
    assert np.array_equal(y, d["yplant"], equal_nan=True)
    for name, key, w in (("LINA_MX_OUT.bin", "lina", 25), ("EIGEN_MX_OUT.bin", "eigen", 10),
                         ("ATA_MX_OUT.bin", "ata", 100), ("ATB_MX_OUT.bin", "atb", 10)):
        a = np.fromfile(tmp_path / name, np.float32).reshape(1536, w)
        assert np.array_equal(a, d[key], equal_nan=True), name


@pytest.mark.parametrize("breakage,msg", [
    (lambda d: (d / "CUDA_MX.bin").write_bytes((d / "CUDA_MX.bin").read_bytes()[:-4]),
     "ControllerEngine error: CUDA_MX.bin is"),
    (lambda d: (d / "DISCRETE_BW.bin").unlink(), "ControllerEngine error: Cannot open DISCRETE_BW.bin"),
    (lambda d: (d / "STATESPACE_A.bin").write_bytes(b"\0" * 8),
     "ControllerEngine error: STATESPACE_A.bin is 8 bytes, expected 36 (1 x 36)"),
    (lambda d: (d / "ControllerEngine.config").write_text("time = 5\n"),
     "ControllerEngine error: ControllerEngine.config: missing `statespace_dim`"),
])
def test_errors_go_to_error_log(lib, mass_spring, tmp_path, breakage, msg):
    mass_spring.write(tmp_path)
    breakage(tmp_path)
    assert ce.run_controller_engine(tmp_path) == 1
    lines = (tmp_path / "error.log").read_text().splitlines()
    assert lines[-1].startswith(msg), lines[-1]


def test_streamed_rounds_match_sessions(lib, tmp_path):
    """Three rounds without diagnostics go through the double-buffered path; in
    mode = serial every round has its own plant (stacked DISCRETE_* and
    BASE_PARAMS, ref: src/main.cu:341-354).  Each round's rows must equal a
    session evaluation of that round's plant."""
    import dataclasses
    p = synth.eight_state(n=1536, time=2000, freq=100)
    pl = p.plant
    rounds = 3
    bps = [pl.base_params.copy() for _ in range(rounds)]
    for r in range(rounds):
        bps[r][1] *= 1.0 + 0.5 * r  # Coulomb friction coefficient differs per round
    stack = lambda a: np.concatenate([np.asarray(a).ravel()] * rounds)
    pl3 = dataclasses.replace(pl, discrete_a=stack(pl.discrete_a), discrete_a_i=stack(pl.discrete_a_i),
                              discrete_bu=stack(pl.discrete_bu), discrete_bw=stack(pl.discrete_bw),
                              discrete_c=stack(pl.discrete_c), base_params=np.concatenate(bps))
    text = p.config_text.replace("n_rounds = 1", f"n_rounds = {rounds}").replace("mode = batch", "mode = serial")
    rng = np.random.default_rng(5)
    perms = [rng.permutation(1536) for _ in range(rounds)]
    g = np.vstack([p.cuda_mx[q] for q in perms])
    info = np.vstack([p.info_mx[q] for q in perms])
    synth.Problem("serial_rounds", text, pl3, g, info).write(tmp_path)
    assert ce.run_controller_engine(tmp_path) == 0
    cfg = ce.EngineConfig.parse(text)
    out = np.fromfile(tmp_path / "INFO_MX_OUT.bin", np.float32).reshape(rounds, 1536, cfg.info_mx_width)
    with ce.Session(cfg, pl3, n_plants=rounds) as s:
        for r in range(rounds):
            ref = s.evaluate(g[r * 1536:(r + 1) * 1536], info[r * 1536:(r + 1) * 1536], plant_index=r)
            assert np.array_equal(out[r], ref, equal_nan=True), f"round {r}"
    assert not np.array_equal(out[0], out[1], equal_nan=True)  # the plants differ
