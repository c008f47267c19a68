"""The compensated_df precision: the compensated form with the simulation in double-float
arithmetic (each state an unevaluated pair of FP32 values, about 48 significant bits, on the FP32
pipe) instead of the FP32 recurrence.  Against the plain FP64 form:
* LIN_A, the eigenvalues and every margin are identical (the same FP64 kernels, which do not read
  the trajectory), and so is every pass/fail class;
* the fit window agrees within 1e-9 of the window's largest |y| for every candidate whose loop is
  modal-stable (each double-float operation is within a few 2^-48; the FP64 form's own rounding
  is 2^-53; the differences grow along the horizon with the loop's sensitivity), and yss, the
  double result rounded to float, equal or one float apart;
* the fit-derived terms (wn, zeta, the behaviour error) agree within 1e-6 wherever the scaled
  normal matrix is conditioned below 1e8 -- the bound the compensated arithmetic meets on the FP64
  form's own trajectory -- where the compensated form's FP32 trajectory leaves ~1e-5."""
import numpy as np
import pytest

import controllerengine_gb300 as ce
from controllerengine_gb300 import synth
from parity_helpers import _classes, _cols

pytestmark = pytest.mark.gpu


def _problems():
    return {"mass_spring": synth.mass_spring(1536), "eight_state": synth.eight_state(n=512, time=3000, freq=160)}


def _fit_condition(info, ata, cfg):
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


@pytest.mark.parametrize("name", ["mass_spring", "eight_state"])
def test_compensated_df_against_fp64_form(lib, name):
    p = _problems()[name]
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, precision="fp64") as s:
        f64, d64 = s.evaluate_diagnostics64(p.cuda_mx, p.info_mx)
    with ce.Session(cfg, p.plant, precision="compensated_df") as s:
        cdf, dd = s.evaluate_diagnostics64(p.cuda_mx, p.info_mx)
    with ce.Session(cfg, p.plant, precision="compensated") as s:
        cmp_ = s.evaluate(p.cuda_mx, p.info_mx)
    for k in ("lina", "eigen"):
        assert np.array_equal(dd[k], d64[k]), k
    ca, cb = _classes(cdf, cfg), _classes(f64, cfg)
    assert np.array_equal(ca, cb), f"{int((ca != cb).any(axis=1).sum())} candidates classified differently"
    c = _cols(cfg)
    assert np.array_equal(cdf[:, c["am"]], f64[:, c["am"]], equal_nan=True), "margins"
    stable = f64[:, cfg.info_scoring + 1] < cfg.unstable_err
    assert stable.sum() > 50
    y, y64 = dd["ywin"][stable], d64["ywin"][stable]
    scale = np.maximum(np.abs(y64).max(axis=1), 1e-30)
    traj = np.abs(y - y64).max(axis=1) / scale
    assert traj.max() <= 1e-9, traj.max()
    fr = c["fr"].start
    yss, yss64 = cdf[stable, fr + 3].astype(np.float64), f64[stable, fr + 3].astype(np.float64)
    # both are the double results rounded to float: equal, or one float apart at a rounding boundary
    ulp = np.spacing(np.abs(yss64).astype(np.float32)).astype(np.float64)
    assert (np.abs(yss - yss64) <= ulp).all()
    cond = _fit_condition(f64, d64["ata"], cfg)
    good = stable & (cond > 0) & (cond < 1e8)
    if good.sum() == 0:
        pytest.skip("no well-conditioned fit in this workload")
    for col in (fr, fr + 1, cfg.info_scoring + 1):
        a, b = cdf[good, col].astype(np.float64), f64[good, col].astype(np.float64)
        rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-30)
        assert rel.max() <= 1e-6, (col, rel.max(), int(good.sum()))
        # and no worse than the compensated form's, whose trajectory is FP32
        rc = np.abs(cmp_[good, col].astype(np.float64) - b) / np.maximum(np.abs(b), 1e-30)
        assert np.median(rel) <= np.median(rc), (col, np.median(rel), np.median(rc))


def test_compensated_df_rows_do_not_depend_on_the_batch(lib):
    p = synth.eight_state(n=512, time=3000, freq=160)
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, precision="compensated_df") as s:
        full = s.evaluate(p.cuda_mx, p.info_mx)
        part = np.vstack([s.evaluate(p.cuda_mx[a:a + 97], p.info_mx[a:a + 97]) for a in range(0, 512, 97)])
    assert np.array_equal(full, part, equal_nan=True)


@pytest.mark.parametrize("serial", [False, True])
def test_compensated_df_per_candidate_plants(lib, serial):
    """One plant per candidate: the double-float simulation reads the candidate's plant from the
    plant table; rows equal each candidate alone with its plant, classes equal the FP64 form's."""
    p = synth.monte_carlo(n_plants=64, time=1200, freq=60, serial=serial)
    rng = np.random.default_rng(12)
    p.cuda_mx[:, :8] *= rng.uniform(0.5, 3.0, (64, 1)).astype(np.float32)
    p.info_mx[:, :8] = p.cuda_mx[:, :8]
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, n_plants=64, precision="compensated_df") as s:
        rows = s.evaluate_plants(p.cuda_mx, p.info_mx)
        part = s.evaluate_plants(p.cuda_mx[10:30], p.info_mx[10:30], first_plant=10)
        s.set_precision("fp64")
        f64 = s.evaluate_plants(p.cuda_mx, p.info_mx)
    assert np.array_equal(rows[10:30].view(np.uint32), part.view(np.uint32))
    assert np.array_equal(_classes(rows, cfg), _classes(f64, cfg))


def test_compensated_df_refuses_kalman(lib):
    p = synth.eight_state(n=64, time=500, freq=40, observer="kalman")
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant) as s:
        with pytest.raises(ce.ControllerEngineError, match="simulates in FP32 only"):
            s.set_precision("compensated_df")
