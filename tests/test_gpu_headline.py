"""Parity on the headline configuration itself: the first 2,048 candidates of the 65,536-candidate
eight-state workload (the throughput benchmark's batch, seed 2) at its full horizon (T = 10,000
steps, fit window 7,000) and sweep (F = 400 points).

Stage by stage against the oracle (the comparisons and tolerances of parity_helpers._stagewise:
trajectories, LIN_A, eigenvalues, yss and overshoot bit-exact; AtA/Atb within 1e-3 of the row
scale; margins within 1e-3 dB / deg), and end to end against an independent oracle run: every
classification (modal-unstable, nominal-unstable, eig-fail, margin status) identical, gain and
phase margins within 1e-3 dB / deg, b_PC within 1e-4 relative (ref: src/modalsetup.cu:18-26 and
src/allmargin.cu:72-87 for the classes, src/allmargin.cu:125-150 for the margins)."""
import numpy as np
import pytest

import controllerengine_gb300 as ce
from controllerengine_gb300 import synth
from parity_helpers import _classes, _close, _cols, _stagewise

pytestmark = pytest.mark.gpu

N = 2048


@pytest.fixture(scope="module")
def headline_slice():
    p = synth.eight_state()  # 65,536 candidates, T = 10,000, F = 400
    assert p.cuda_mx.shape[0] == 65536
    cfg = ce.EngineConfig.parse(p.config_text)
    assert (cfg.time, cfg.freq, cfg.fit_steps) == (10000, 400, 7000)
    return synth.Problem(name="eight_state_headline_slice", config_text=p.config_text, plant=p.plant,
                         cuda_mx=np.ascontiguousarray(p.cuda_mx[:N]), info_mx=np.ascontiguousarray(p.info_mx[:N]))


def test_headline_slice_stagewise(lib, oracle_mod, headline_slice):
    cfg, info = _stagewise(headline_slice, oracle_mod)
    cls = _classes(info, cfg)
    assert cls[:, 3].sum() > 0  # candidates reach the margin sweep


def test_headline_slice_end_to_end(lib, oracle_mod, headline_slice):
    p = headline_slice
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant) as s:
        info = s.evaluate(p.cuda_mx, p.info_mx)
        fused = s.eig_arith == "fused"
    ref = oracle_mod.Oracle(p.config_text, p.plant, eig_fused=fused).evaluate(p.cuda_mx, p.info_mx)
    ca, cb = _classes(info, cfg), _classes(ref, cfg)
    assert np.array_equal(ca, cb), f"classification mismatches: {int((ca != cb).any(axis=1).sum())}"
    am = _cols(cfg)["am"]
    a, b = info[:, am], ref[:, am]
    scored = a[:, 3] == 1
    assert scored.sum() > 0
    assert np.all(_close(a[scored, 0], b[scored, 0], 0, 1e-3)), "gain margin (dB)"
    assert np.all(_close(a[scored, 1], b[scored, 1], 0, 1e-3)), "phase margin (deg)"
    assert np.all(_close(a[scored, 4], b[scored, 4], 1e-4, 1e-7)), "b_PC"
