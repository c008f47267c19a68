"""The plain FP64 form (precision "fp64") against the oracle's FP64 restatement of the method
(oracle/ce_oracle64.h), which follows the engine's FP64 kernels operation by operation.

What can differ is only the libm of the transcendental functions (exp, log, sin, cos, atan2,
hypot, log10: CUDA's on the GPU, glibc's here, each within an ulp or two), so:
* the trajectory's fit window and its summaries, LIN_A and the eigenvalues involve none of them
  and are compared to 1e-12 relative (they come out bit-identical);
* AtA / Atb (the basis calls exp, sin and cos) within 1e-12 of each row's scale;
* every pass/fail class (modal-unstable, nominal-unstable, eig-fail, margin status) identical;
* the INFO row's cost terms, the double results rounded to float: the terms no fit enters
  (yss, overshoot, the margins) identical for at least 99% of the values, and every term within
  1e-6 relative, except the fit-derived terms (wn, zeta, the behaviour error and the total score,
  the modal columns) of candidates whose scaled normal matrix has a condition number above 1e9,
  where the libm's last-ulp differences in the basis (1e-16) are amplified beyond 1e-7 -- two
  correct FP64 evaluations disagree there.
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


def _fit_condition(info, ata, cfg):
    """Condition number of each candidate's diagonally scaled normal matrix (the system the modal
    solve factors); 0 for a candidate the fit does not model."""
    nt = cfg.total_dim
    uniq = info[:, cfg.info_modal + 3 * nt].astype(int)
    out = np.zeros(info.shape[0])
    for k in range(info.shape[0]):
        nc = 2 * uniq[k]
        if nc == 0 or info[k, cfg.info_scoring + 1] >= cfg.unstable_err:
            continue
        A = ata[k].reshape(2 * nt, 2 * nt)[:nc, :nc]
        A = np.tril(A) + np.tril(A, -1).T
        dg = np.sqrt(np.abs(np.diag(A)))
        dg[dg <= 1e-6] = 1.0
        out[k] = np.linalg.cond(A / dg[:, None] / dg[None, :])
    return out


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
    assert np.array_equal(np.isfinite(a), np.isfinite(b))
    with np.errstate(invalid="ignore"):
        rel = np.where(np.isfinite(a) & np.isfinite(b), np.abs(a - b) / np.maximum(np.abs(b), 1e-30), 0.0)
    fr = c["fr"].start
    fit_cols = np.isin(cols, np.r_[c["sc"], fr, fr + 1, c["md"]])
    # the terms no fit enters (yss, overshoot, the margins): the same floats, all but a few
    assert (rel[:, ~fit_cols] == 0).mean() >= 0.99, (rel[:, ~fit_cols] == 0).mean()
    cond = _fit_condition(info, d["ata"], cfg)
    ill = (cond > 1e9)[:, None] & fit_cols[None, :]
    assert rel[~ill].max() <= 1e-6, (rel[~ill].max(), np.unravel_index(np.argmax(np.where(ill, 0, rel)), rel.shape))


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
