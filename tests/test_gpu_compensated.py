"""The compensated precision (precision "compensated") against the plain FP64 form and against an
independent float64 evaluation of its own normal equations.

The compensated form simulates in FP32 (the mixed form's kernels, so its trajectory is the
mixed form's, bit for bit) and runs LIN_A, the eigensolves, the nominal check and the sweep in
FP64 (the FP64 form's kernels).  So, against the FP64 form:
* eigenvalues, LIN_A and every margin (GM, PM, DM, b_PC, margin status) are identical;
* every pass/fail class is identical;
* the normal matrix AtA -- from the closed form of its geometric sums here, from per-step FP64
  accumulation there -- agrees to 1e-10 of the scale of the two modes involved, sqrt(sum |z_m|^2)
  sqrt(sum |z_k|^2) with z_m = e^{s_m t} over the window (the two differ by the FP64 form's
  rounding of the sample times and of its 7,000-term sums; a sine column that is 0 in exact
  arithmetic -- a real or a Nyquist mode -- is exactly 0 or ~1e-16 of its mode in the closed
  form and rounding noise of that size in a direct sum);
* the steady state yss agrees to 1e-6 relative: what remains is the FP32 trajectory's own
  difference from the FP64 one, which the compensated sum no longer adds to.
The right-hand side Atb, the projection of the FP32 trajectory onto the basis by a double-float
recurrence, is checked against a float64 evaluation in numpy of the same sum on the same FP32
trajectory: within 1e-11 of sum_w |z_m(t_w)| |y_w - yss| for mode m's two entries."""
import numpy as np
import pytest

import controllerengine_gb300 as ce
from controllerengine_gb300 import synth
from parity_helpers import _classes, _cols

pytestmark = pytest.mark.gpu

# the engine's float constants of the mode extraction (ref: src/modalsetup.cu:8-50)
TINY = float.fromhex("0x1.0c6f7ap-20")
LOGFLOOR = float.fromhex("0x1.a484cp-100")
SENT = float.fromhex("0x1.2a05f2p+33")


def _problems():
    return {"mass_spring": synth.mass_spring(1536), "eight_state": synth.eight_state(n=512, time=3000, freq=160)}


def _modes(eig, nt, ts):
    """sigma, |omega| of the unique modes (the engine's dedupe of consecutive eigenvalues)."""
    re, im = eig[0::2], eig[1::2]
    mag = np.hypot(re, im)
    Re = np.log(np.maximum(mag, LOGFLOOR)) / ts
    Im = np.arctan2(im, re) / ts
    out, pre, pim = [], SENT, SENT
    for i in range(nt):
        if not (abs(Re[i] - pre) < TINY and abs(abs(Im[i]) - abs(pim)) < TINY):
            out.append((Re[i], abs(Im[i])))
        pre, pim = Re[i], Im[i]
    return out


@pytest.mark.parametrize("name", ["mass_spring", "eight_state"])
def test_compensated_against_fp64_form(lib, name):
    p = _problems()[name]
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, precision="fp64") as s:
        f64, d64 = s.evaluate_diagnostics64(p.cuda_mx, p.info_mx)
    with ce.Session(cfg, p.plant, precision="compensated") as s:
        cmp_, dc = s.evaluate_diagnostics64(p.cuda_mx, p.info_mx)
    with ce.Session(cfg, p.plant) as s:
        mix, dm = s.evaluate_diagnostics64(p.cuda_mx, p.info_mx, want=("ywin", "summ"))
    # the simulation is the mixed form's
    assert np.array_equal(dc["ywin"], dm["ywin"]) and np.array_equal(dc["summ"], dm["summ"])
    for k in ("lina", "eigen"):
        assert np.array_equal(dc[k], d64[k]), k
    ca, cb = _classes(cmp_, cfg), _classes(f64, cfg)
    assert np.array_equal(ca, cb), f"{int((ca != cb).any(axis=1).sum())} candidates classified differently"
    c = _cols(cfg)
    assert np.array_equal(cmp_[:, c["am"]], f64[:, c["am"]], equal_nan=True), "margins"
    nt = cfg.total_dim
    stable = cmp_[:, cfg.info_scoring + 1] < cfg.unstable_err
    a = dc["ata"].reshape(-1, 2 * nt, 2 * nt)[stable]
    b = d64["ata"].reshape(-1, 2 * nt, 2 * nt)[stable]
    dg = np.abs(np.einsum("kii->ki", b))
    mode = np.sqrt(dg[:, 0::2] + dg[:, 1::2])  # per mode: sqrt(sum |z_m|^2)
    mode = np.repeat(mode, 2, axis=1)
    scale = np.maximum(mode[:, :, None] * mode[:, None, :], 1e-300)
    err = np.abs(a - b) / scale
    assert err.max() <= 1e-10, err.max()
    fr = cfg.info_freqresp
    yc, y64, ym = (x[stable, fr + 3].astype(np.float64) for x in (cmp_, f64, mix))
    rel_c = np.abs(yc - y64) / np.abs(y64)
    rel_m = np.abs(ym - y64) / np.abs(y64)
    assert rel_c.max() <= 1e-6, rel_c.max()
    assert np.median(rel_c) < np.median(rel_m), (np.median(rel_c), np.median(rel_m))


@pytest.mark.parametrize("name", ["mass_spring", "eight_state"])
def test_compensated_normal_equations_against_float64(lib, name):
    p = _problems()[name]
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, precision="compensated") as s:
        info, d = s.evaluate_diagnostics64(p.cuda_mx, p.info_mx)
    nt, ts = cfg.total_dim, float(np.float32(cfg.ts))
    steps, w0 = cfg.fit_steps, cfg.fit_start_id
    t = (w0 + np.arange(steps)) * ts
    wlimit = cfg.time - w0
    uniq = info[:, cfg.info_modal + 3 * nt]
    checked = 0
    for k in range(0, info.shape[0], max(1, info.shape[0] // 64)):
        if info[k, cfg.info_scoring + 1] >= cfg.unstable_err:
            continue
        modes = _modes(d["eigen"][k], nt, ts)
        if len(modes) != int(uniq[k]):
            continue  # a dedupe decided on a last-ulp difference of the libm
        cols = []
        for sig, om in modes:
            sh = max(sig * float(np.float32(cfg.fit_t0)), sig * float(np.float32(cfg.fit_t1)))
            e = np.exp(sig * t - sh)
            cols += [e * np.cos(om * t), e * np.sin(om * t)]
        B = np.array(cols).T
        nc = B.shape[1]
        ysum = d["summ"][k, 0] + d["summ"][k, 3]
        yss = ysum / (cfg.time - cfg.steady_start_id)
        y = np.where(np.arange(steps) < wlimit, d["ywin"][k], 0.0)
        r = y - yss
        atb = B.T @ r
        got = d["atb"][k, :nc]
        zmag = np.hypot(B[:, 0::2], B[:, 1::2])  # |z_m(t_w)| per mode
        bound = np.repeat(1e-11 * (zmag * np.abs(r)[:, None]).sum(0), 2)
        assert (np.abs(got - atb) <= bound + 1e-300).all(), (k, np.abs(got - atb).max(), bound.min())
        ata = B.T @ B
        A = d["ata"][k].reshape(2 * nt, 2 * nt)[:nc, :nc]
        mode = np.repeat(np.sqrt((zmag ** 2).sum(0)), 2)
        low = np.tril_indices(nc)
        err = (np.abs(A - ata) / np.maximum(np.outer(mode, mode), 1e-300))[low]
        assert err.max() <= 1e-12, (k, err.max())
        checked += 1
    assert checked >= 8, checked


def test_compensated_rows_do_not_depend_on_the_batch(lib):
    p = synth.eight_state(n=512, time=3000, freq=160)
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, precision="compensated") as s:
        full = s.evaluate(p.cuda_mx, p.info_mx)
        part = np.vstack([s.evaluate(p.cuda_mx[a:a + 97], p.info_mx[a:a + 97]) for a in range(0, 512, 97)])
    assert np.array_equal(full, part, equal_nan=True)


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
def test_compensated_arithmetic_on_the_fp64_trajectory(lib, name):
    """The diagnostic precision "compensated_traj64": the compensated form's fit, solve,
    eigensolves and sweep fed with the FP64 form's trajectory.  Against the FP64 form, everything
    that does not pass through the fit is identical (classes, yss, overshoot, margins), and the fit
    terms agree within 1e-6 wherever the scaled normal matrix is conditioned below 1e8 -- so the
    compensated form's larger differences on those candidates are its FP32 trajectory's."""
    p = _problems()[name]
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, precision="fp64") as s:
        f64, d64 = s.evaluate_diagnostics64(p.cuda_mx, p.info_mx, want=("ata",))
    with ce.Session(cfg, p.plant, precision="compensated_traj64") as s:
        t64 = s.evaluate(p.cuda_mx, p.info_mx)
    assert np.array_equal(_classes(t64, cfg), _classes(f64, cfg))
    c = _cols(cfg)
    fr = c["fr"].start
    for col in (fr + 2, fr + 3):
        assert np.array_equal(t64[:, col], f64[:, col], equal_nan=True)
    assert np.array_equal(t64[:, c["am"]], f64[:, c["am"]], equal_nan=True)
    cond = _fit_condition(f64, d64["ata"], cfg)
    good = (cond > 0) & (cond < 1e8) & (f64[:, cfg.info_scoring + 1] < cfg.unstable_err)
    if good.sum() == 0:
        pytest.skip("no well-conditioned fit in this workload")
    for col in (fr, fr + 1, cfg.info_scoring + 1):
        a, b = t64[good, col].astype(np.float64), f64[good, col].astype(np.float64)
        rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-30)
        assert rel.max() <= 1e-6, (col, rel.max(), int(good.sum()))
