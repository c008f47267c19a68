"""Stage-wise GPU-vs-oracle comparison shared by the parity tests (see
test_gpu_parity.py for what is bit-exact and what is compared to a tolerance)."""
import numpy as np

import controllerengine_gb300 as ce


def _eq(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


def _mismatch(a, b):
    a, b = np.asarray(a), np.asarray(b)
    bad = ~((a == b) | (np.isnan(a) & np.isnan(b)))
    return int(bad.sum())


def _cols(cfg):
    s = cfg.info_scoring
    return dict(sc=slice(s, s + 3), fr=slice(s + 3, s + 7), am=slice(s + 7, s + 12),
                md=slice(s + 12, s + 12 + 3 * cfg.total_dim + 1))


def _classes(info, cfg):
    c = _cols(cfg)
    sc, am = info[:, c["sc"]], info[:, c["am"]]
    return np.stack([sc[:, 1] >= cfg.unstable_err, sc[:, 2] == np.float32(cfg.unstable_err),
                     sc[:, 2] == np.float32(cfg.eig_fail_err), am[:, 3]], axis=1)


def _close(a, b, rtol, atol=0.0):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    ok = both_nan | (np.abs(a - b) <= atol + rtol * np.abs(b)) | (a == b)
    return ok


def _stagewise(problem, oracle_mod, score_atol=1e-6, eig_arith=None):
    """eig_arith: the session's eigensolve arithmetic ("fused" / "separate"; None: the library
    default); the oracle's eigensolves use the same one, so eigenvalues compare bit for bit."""
    cfg = ce.EngineConfig.parse(problem.config_text)
    with ce.Session(cfg, problem.plant) as s:
        if eig_arith:
            s.set_eig_arith(eig_arith)
        arith = s.eig_arith
        info, d = s.evaluate_diagnostics(problem.cuda_mx, problem.info_mx)
        launches = s.kernel_launches
    # lina+eig, sim, fit classes, fit, modal, nominal, sweep selection, LU pass, scan; the
    # Kalman observer adds three grouping kernels, the per-candidate list's gain schedules and
    # two more simulation forms
    assert launches == (15 if cfg.observer else 9)
    orc = oracle_mod.Oracle(problem.config_text, problem.plant, eig_fused=arith == "fused")
    g = problem.cuda_mx

    y_o = orc.sim(g)
    assert _eq(d["yplant"], y_o), f"trajectory mismatches: {_mismatch(d['yplant'], y_o)}"
    lina_o = orc.lina(g)
    assert _eq(d["lina"], lina_o), f"LIN_A mismatches: {_mismatch(d['lina'], lina_o)}"
    eig_o = orc.eigensolve(d["lina"])
    assert _eq(d["eigen"], eig_o), f"eigenvalue mismatches: {_mismatch(d['eigen'], eig_o)}"

    ata_o, atb_o, info1 = orc.modalsetup(d["yplant"], d["eigen"], problem.info_mx)
    c = _cols(cfg)
    fr = c["fr"]
    # yss and overshoot involve no libm call: bit-exact
    assert _eq(info[:, fr][:, 2:4], info1[:, fr][:, 2:4])
    # sigma = log|lambda|/ts turns a 1-ulp hypotf difference near |lambda| = 1 into a
    # relative error of ~6e-8/|log|lambda||; the engine matches the reference's own
    # kernel bit for bit here (test_gpu_reference_kernels), glibc differs by that much
    scale = np.maximum(np.abs(ata_o).max(axis=1, keepdims=True), 1e-30)
    assert np.all(_close(d["ata"], ata_o, 0, 1e-3 * scale)), "AtA"
    bscale = np.maximum(np.abs(atb_o).max(axis=1, keepdims=True), 1e-30)
    assert np.all(_close(d["atb"], atb_o, 0, 1e-3 * bscale)), "Atb"

    # modal solve + margins in the oracle on the engine's own intermediates
    info2 = orc.modalsolve(d["ata"], d["atb"], d["eigen"], info1)
    info3 = orc.allmargin(d["lina"], g, info2)
    assert _eq(_classes(info, cfg), _classes(info3, cfg)), "classification differs"
    sc, am, md = c["sc"], c["am"], c["md"]
    # the oracle recomputes the modes with glibc (see above): 1e-3 relative
    assert np.all(_close(info[:, sc], info3[:, sc], 1e-3, score_atol)), "scores"
    assert np.all(_close(info[:, fr][:, :2], info3[:, fr][:, :2], 1e-3, 1e-6)), "wn, zeta"
    assert np.all(_close(info[:, md], info3[:, md], 1e-3, 1e-6)), "modal columns"
    a, b = info[:, am], info3[:, am]
    assert np.all(_close(a[:, 0], b[:, 0], 0, 1e-3)), "gain margin (dB)"
    assert np.all(_close(a[:, 1], b[:, 1], 0, 1e-3)), "phase margin (deg)"
    assert np.all(_close(a[:, 2], b[:, 2], 1e-4, 1e-6)), "delay margin"
    assert _eq(a[:, 3], b[:, 3])
    assert np.all(_close(a[:, 4], b[:, 4], 1e-5, 1e-7)), "b_PC"
    # the user columns pass through untouched
    assert _eq(info[:, :cfg.input_size], problem.info_mx[:, :cfg.input_size])
    return cfg, info


def closed_form_margins(problem, oa, crossover, row=0):
    """Margins of synth.first_order_loop's loop L(z) = c b k l / ((z - a)(z - a_cl)) in float64 from
    its float32 coefficients (a_cl = oa, the observer block of LIN_A as computed): the gain
    crossover |L| = 1 and the phase crossover arg L = -pi solved by bracketing on (0, pi); GM (dB),
    PM (deg), DM (ms) there.  b_PC is the minimum over the sweep's own grid (theta_w in float32 as
    the sweep forms it) of |1 + L| / (sqrt(1 + |alpha P|^2) sqrt(1 + |G / alpha|^2)), alpha =
    1 / |P| at the crossover frequency."""
    from scipy.optimize import brentq
    cfg = ce.EngineConfig.parse(problem.config_text)
    pl = problem.plant
    a, b, c = (np.float64(x[0]) for x in (pl.statespace_a, pl.statespace_b, pl.statespace_c))
    k, l = (np.float64(x) for x in problem.cuda_mx[row, :2])
    oa = np.float64(oa)
    P = lambda th: c * b / (np.exp(1j * th) - a)
    G = lambda th: k * l / (np.exp(1j * th) - oa)
    phase = lambda th: -(np.angle(np.exp(1j * th) - a) + np.angle(np.exp(1j * th) - oa))
    ts = np.float64(np.float32(cfg.ts))
    th_g = brentq(lambda t: abs(P(t) * G(t)) - 1.0, 1e-9, np.pi - 1e-9, xtol=1e-15)
    th_p = brentq(lambda t: phase(t) + np.pi, 1e-9, np.pi - 1e-9, xtol=1e-15)
    pm = 180.0 + np.degrees(phase(th_g))
    gm = -20.0 * np.log10(abs(P(th_p) * G(th_p)))
    dm = np.radians(pm) / th_g * ts * 1000.0
    F = cfg.freq
    f32 = np.float32
    inc = (np.log(f32(cfg.freq_max)) - np.log(f32(cfg.freq_min))) / f32(F - 1)
    th = np.exp(np.log(f32(cfg.freq_min)) + inc * np.arange(F, dtype=f32)).astype(f32) * f32(ts)
    th = th.astype(np.float64)
    alpha = 1.0 / abs(P(np.float64(crossover) * ts))
    bw = abs(1.0 + P(th) * G(th)) / (np.sqrt(1.0 + (alpha * abs(P(th))) ** 2) * np.sqrt(1.0 + (abs(G(th)) / alpha) ** 2))
    return dict(gm=gm, pm=pm, dm=dm, bpc=min(1.0, bw.min()))
