"""The plain FP64 form (precision "fp64") against the oracle's FP64 restatement of the method
(oracle/ce_oracle64.h), which follows the engine's FP64 kernels operation by operation.

What can differ is only the libm of the transcendental functions (exp, log, sin, cos, atan2,
hypot, log10: CUDA's on the GPU, glibc's here, each within an ulp or two), so:
* the trajectory's fit window and its summaries, LIN_A and the eigenvalues involve none of them
  and are compared to 1e-12 relative (they come out bit-identical);
* AtA / Atb (the basis calls exp, sin and cos) within 1e-12 of each row's scale;
* every pass/fail class (modal-unstable, nominal-unstable, eig-fail, margin status) identical;
* the INFO row's cost terms, the double results rounded to float, within 1e-6 relative, and
  all but a few per mille of them identical (a double difference of ~1e-14, amplified by the
  fit's normal-equation conditioning, crosses a float rounding boundary now and then).
The same form against the mixed form: identical classes on these workloads."""
import numpy as np
import pytest

import controllerengine_gb300 as ce
from controllerengine_gb300 import synth
from parity_helpers import _classes, _cols

pytestmark = pytest.mark.gpu


def _rel(a, b):
    """max over rows of |a - b| / (max |b| of the row)"""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = np.maximum(np.abs(b).max(axis=1, keepdims=True), 1e-300)
    d = np.abs(a - b) / scale
    d[np.isnan(a) & np.isnan(b)] = 0.0
    return float(np.nanmax(d)) if d.size else 0.0


def _problems():
    return {"mass_spring": synth.mass_spring(1536), "eight_state": synth.eight_state(n=512, time=3000, freq=160)}


@pytest.mark.parametrize("name", ["mass_spring", "eight_state"])
def test_fp64_form_against_fp64_oracle(lib, oracle_mod, name):
    p = _problems()[name]
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, precision="fp64") as s:
        info, d = s.evaluate_diagnostics64(p.cuda_mx, p.info_mx)
        fused = s.eig_arith == "fused"
    ref, o = oracle_mod.Oracle(p.config_text, p.plant, eig_fused=fused).evaluate64(p.cuda_mx, p.info_mx)
    d["summ"] = d["summ"][:, :3]  # the fourth column, the FP32 sum's compensation, is 0 in FP64
    for k in ("ywin", "summ", "lina", "eigen"):
        assert _rel(d[k], o[k]) <= 1e-12, (k, _rel(d[k], o[k]))
    for k in ("ata", "atb"):
        assert _rel(d[k], o[k]) <= 1e-12, (k, _rel(d[k], o[k]))
    ca, cb = _classes(info, cfg), _classes(ref, cfg)
    assert np.array_equal(ca, cb), f"{int((ca != cb).any(axis=1).sum())} candidates classified differently"
    c = _cols(cfg)
    cols = np.r_[c["sc"], c["fr"], c["am"], c["md"]]
    a, b = info[:, cols].astype(np.float64), ref[:, cols].astype(np.float64)
    both = np.isfinite(a) & np.isfinite(b)
    assert np.array_equal(np.isfinite(a), np.isfinite(b))
    rel = np.abs(a - b)[both] / np.maximum(np.abs(b)[both], 1e-30)
    assert rel.max() <= 1e-6, rel.max()
    assert (rel == 0).mean() >= 0.99, (rel == 0).mean()


def test_fp64_form_classes_equal_mixed(lib, eight_state_small):
    """The mixed form (the reference's arithmetic) and the FP64 form classify every candidate the
    same on the small eight-state workload (the 65,536-candidate headline batch: 100% in the
    benchmark's fp64_form.mixed_vs_fp64)."""
    p = eight_state_small
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, precision="fp64") as s:
        f64 = s.evaluate(p.cuda_mx, p.info_mx)
    with ce.Session(cfg, p.plant) as s:
        mix = s.evaluate(p.cuda_mx, p.info_mx)
    ca, cb = _classes(mix, cfg), _classes(f64, cfg)
    assert np.array_equal(ca, cb), f"{int((ca != cb).any(axis=1).sum())} candidates classified differently"
