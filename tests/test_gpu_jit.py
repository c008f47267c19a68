"""The simulation kernel compiled for a plant's instruction program (NVRTC) against
the table-driven kernel that interprets the same program.

The table-driven kernel is pinned bit-exactly to the reference's own kernels
(test_gpu_reference_kernels.py); the specialised kernel performs the same
operations in the same order, so every output must be bit-identical: the full
trajectory, the fit-window normal equations and the INFO rows.  Random programs
cover every opcode (including the no-op codes outside 1..6 and SKIP rows), all
three operand kinds, the plant-output slot of the NL chains and both padded
(dims < 8) and unpadded plants.
"""
import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from controllerengine_gb300 import EngineConfig, Session, synth  # noqa: E402


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _both(prob, want=("yplant", "ata", "atb")):
    cfg = EngineConfig.parse(prob.config_text)
    with Session(cfg, prob.plant) as s:
        assert s.sim_kernel == "specialised", s.sim_log
        out_s, d_s = s.evaluate_diagnostics(prob.cuda_mx, prob.info_mx, want=want)
        s.set_sim_kernel("table")
        assert s.sim_kernel == "table"
        out_t, d_t = s.evaluate_diagnostics(prob.cuda_mx, prob.info_mx, want=want)
    return (out_s, d_s), (out_t, d_t)


def _assert_identical(a, b):
    (out_s, d_s), (out_t, d_t) = a, b
    for k in d_s:
        bad = np.flatnonzero(_bits(d_s[k]) != _bits(d_t[k]))
        assert bad.size == 0, f"{k}: {bad.size} values differ, first at {bad[:5]}"
    bad = np.flatnonzero(_bits(out_s) != _bits(out_t))
    assert bad.size == 0, f"INFO: {bad.size} values differ, first at {bad[:5]}"


@pytest.mark.parametrize("name", ["mass_spring", "eight_state_small"])
def test_specialised_matches_table(name, request):
    prob = request.getfixturevalue(name)
    a, b = _both(prob)
    _assert_identical(a, b)
    # the case is not vacuous: trajectories move and most candidates are scored
    assert np.isfinite(a[1]["yplant"]).mean() > 0.5
    assert np.abs(a[1]["yplant"][np.isfinite(a[1]["yplant"])]).max() > 0.1


def _random_chain(rng, n_rows, cols, n_params):
    """(packed rows) for one chain: digits 0 (state), 35 (running value) or 1..n_params."""
    digits = [0, 35] + list(range(1, n_params + 1))
    chain = []
    for _ in range(n_rows):
        r = rng.random()
        op = 0 if r < 0.08 else (7 if r < 0.14 else int(rng.integers(1, 7)))
        d1, d2 = (int(rng.choice(digits)) for _ in range(2))
        chain.append((op, int(rng.integers(0, cols)), d1, d2))
    return chain


def _config_with(text, **kv):
    lines = []
    for ln in text.splitlines():
        key = ln.split("=")[0].strip()
        if key in kv:
            v = kv.pop(key)
            v = ",".join(str(x) for x in v) if isinstance(v, (list, tuple)) else v
            ln = f"{key} = {v}"
        lines.append(ln)
    assert not kv
    return "\n".join(lines) + "\n"


def _random_program(prob, seed):
    rng = np.random.default_rng(seed)
    cfg = EngineConfig.parse(prob.config_text)
    ns, nd, nw, npar = cfg.statespace_dim, cfg.discrete_dim, cfg.nonlin_dim, cfg.n_params
    n_dc, n_u = int(rng.integers(1, 5)), int(rng.integers(1, 5))
    n_nl = [int(rng.integers(1, 9)) for _ in range(nw)]
    dc = synth.instr_rows(_random_chain(rng, n_dc, nd, npar), nd)
    u = synth.instr_rows(_random_chain(rng, n_u, ns, npar), ns)
    nl = np.vstack([synth.instr_rows(_random_chain(rng, k, nd + 1, npar), nd + 1) for k in n_nl])
    plant = dataclasses.replace(prob.plant, dc_info=dc, u_info=u, nl_info=nl)
    text = _config_with(prob.config_text, dc_instructions=n_dc, u_instructions=n_u, nl_instructions=n_nl)
    return dataclasses.replace(prob, config_text=text, plant=plant)


@pytest.mark.parametrize("seed", range(6))
def test_random_programs_padded_plant(seed, mass_spring):
    prob = _random_program(mass_spring, 100 + seed)
    a, b = _both(prob, want=("yplant",))
    _assert_identical(a, b)


@pytest.mark.parametrize("seed", range(4))
def test_random_programs_eight_state(seed, eight_state_small):
    prob = _random_program(eight_state_small, 200 + seed)
    a, b = _both(prob, want=("yplant",))
    _assert_identical(a, b)


def test_generated_source_names_the_program(mass_spring):
    cfg = EngineConfig.parse(mass_spring.config_text)
    with Session(cfg, mass_spring.plant) as s:
        src = s.specialised_source(0)
    assert "ce_sim_specialised" in src and "ce::sim_run<4, 4, cejit::Chains, ce::SIM_LUENBERGER>" in src
    assert "ce_sim_kalman_shared" not in src
    # the mass-spring NL chain is k3 * x0^3: three multiplies on x0
    assert src.count("__fmul_rn") >= 4


def test_kalman_source_has_both_forms(mass_spring):
    """A Kalman session's program holds the per-candidate and the shared-noise forms, both
    over the full padded observer width."""
    from controllerengine_gb300 import synth
    p = synth.with_kalman(mass_spring)
    with Session(EngineConfig.parse(p.config_text), p.plant) as s:
        src = s.specialised_source(0)
    assert "ce::sim_run<8, 4, cejit::Chains, ce::SIM_KALMAN_LANE>" in src
    assert "ce_sim_kalman_shared" in src and "ce::SIM_KALMAN_SHARED" in src


_WIDE_SCRIPT = r"""
import sys, numpy as np
import controllerengine_gb300 as ce
from controllerengine_gb300 import synth
probs = [synth.mass_spring(300), synth.eight_state(n=200, time=1500, freq=60)]
probs += [synth.random_shape(700 + k, n=150, time=900, freq=50) for k in range(6)]
outs = []
for p in probs:
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant) as s:
        _, d = s.evaluate_diagnostics(p.cuda_mx, p.info_mx, want=("yplant",))
        outs.append(d["yplant"].ravel())
        outs.append(s.evaluate(p.cuda_mx, p.info_mx).ravel())
np.save(sys.argv[1], np.concatenate(outs))
"""


def test_wide_simulation_form_equals_one_thread_form(tmp_path):
    """The wide simulation form (four lanes per candidate; CE_SIM_WIDE=1 forces it, =0 forbids it,
    read once per process) gives the one-thread form's trajectories and rows bit for bit, for
    every dimension class including the padded 4/4 class."""
    import os
    import subprocess
    import sys
    script = tmp_path / "wide_form.py"
    script.write_text(_WIDE_SCRIPT)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    res = {}
    for mode in ("1", "0"):
        out = tmp_path / f"wide{mode}.npy"
        subprocess.run([sys.executable, str(script), str(out)], check=True, cwd=root,
                       env={**os.environ, "CE_SIM_WIDE": mode, "PYTHONPATH": root})
        res[mode] = np.load(out)
    assert np.array_equal(res["1"].view(np.uint32), res["0"].view(np.uint32))
