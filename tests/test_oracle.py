"""Pins of the CPU oracle itself: the FP64 eigensolver against LAPACK and closed
forms, the simulation against an independent float64 recurrence, the margins
against a loop with a closed form, and the workload generator's invariants.
CPU only."""
import numpy as np
import pytest
from scipy.linalg import expm

import controllerengine_gb300 as ce
from controllerengine_gb300 import synth


def test_eig_matches_lapack(oracle_mod):
    rng = np.random.default_rng(3)
    for n in list(range(1, 17)) * 4:
        A = rng.standard_normal((n, n))
        if rng.random() < 0.3:
            A = A @ np.diag(rng.uniform(0.01, 10.0, n))
        ok, ev = oracle_mod.eig_matrix(A)
        assert ok
        ref = np.linalg.eigvals(A)
        # same multiset of eigenvalues
        key = lambda z: (round(z.real, 6), round(abs(z.imag), 6), np.sign(z.imag))
        a = sorted(ev, key=key)
        b = sorted(ref, key=key)
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-9 * max(1.0, np.abs(ref).max()))


def test_eig_pair_convention(oracle_mod):
    # complex pairs are adjacent with the positive imaginary part first (Schur-diagonal order)
    rng = np.random.default_rng(4)
    for _ in range(50):
        A = rng.standard_normal((8, 8))
        ok, ev = oracle_mod.eig_matrix(A)
        i = 0
        while i < 8:
            if ev[i].imag != 0:
                assert ev[i].imag > 0 and ev[i + 1] == np.conj(ev[i])
                i += 2
            else:
                i += 1


def test_eig_zoh_closed_form(oracle_mod):
    # ZOH of a damped oscillator: eigenvalues exp(s dt), s = -zeta wn +- i wn sqrt(1-zeta^2)
    Ac = np.array([[0.0, 1.0], [-4.0, -0.4]])
    Ad = expm(Ac * 1e-3)
    ok, ev = oracle_mod.eig_matrix(Ad)
    s = np.roots([1.0, 0.4, 4.0])
    np.testing.assert_allclose(sorted(ev, key=lambda z: z.imag), sorted(np.exp(s * 1e-3), key=lambda z: z.imag),
                               rtol=1e-13)


def test_eig_zero_and_triangular(oracle_mod):
    ok, ev = oracle_mod.eig_matrix(np.zeros((4, 4)))
    assert ok and np.all(ev == 0)
    T = np.triu(np.arange(1.0, 17.0).reshape(4, 4))
    ok, ev = oracle_mod.eig_matrix(T)
    assert ok and sorted(ev.real) == [1.0, 6.0, 11.0, 16.0]


def test_sim_linear_matches_float64(oracle_mod):
    """No nonlinearity, K = L = 0: y is the plant's step response to u = N r."""
    from controllerengine_gb300 import synth
    p = synth.mass_spring(1536)
    p.plant.nl_info[:] = 0
    g = np.zeros((1, 7), np.float32)
    g[0, 6] = 2.0
    y = oracle_mod.Oracle(p.config_text, p.plant).sim(g)[0]
    A = p.plant.discrete_a.reshape(2, 2).astype(np.float64)
    B = p.plant.discrete_bu.astype(np.float64)
    x = np.zeros(2)
    ref = np.empty(2000)
    for t in range(2000):
        ref[t] = x[0]
        u = 0.0 if t < 100 else 2.0
        x = A @ x + B * u
    np.testing.assert_allclose(y, ref, rtol=1e-5, atol=1e-9)


def test_generator_invariants():
    from controllerengine_gb300 import synth
    p = synth.eight_state(n=64, time=500, freq=50)
    A = p.plant.discrete_a.reshape(8, 8).astype(np.float64)
    r = np.abs(np.linalg.eigvals(A))
    assert np.all((r > 0.899) & (r < 0.9951))
    np.testing.assert_array_equal(p.plant.discrete_a_i, p.plant.discrete_a - np.eye(8, dtype=np.float32).reshape(-1))
    assert p.cuda_mx.shape == (64, 17) and np.all(np.isfinite(p.cuda_mx))


@pytest.mark.parametrize("observer", ["luenberger", "kalman"])
def test_oracle_ref_config_equals_engine_parse(oracle_mod, observer):
    """The fields the reference's kernels read, derived by the oracle alone (used to launch
    them without the engine) equal the engine's parse, for both observers."""
    import controllerengine_gb300 as ce
    from controllerengine_gb300 import synth
    for p in (synth.eight_state(n=8, time=1000, freq=50, observer=observer), synth.random_shape(3, n=8)):
        rc = oracle_mod.Oracle(p.config_text, p.plant).ref_config()
        cfg = ce.EngineConfig.parse(p.config_text)
        for k, v in vars(rc).items():
            assert getattr(cfg, k) == v, k


def test_margins_closed_form(oracle_mod):
    """The margin restatement (ref: src/allmargin.cu:1-182) against a loop with a closed form,
    synth.first_order_loop: GM, PM and DM from the sweep's interpolated crossovers converge to the
    exact margins at second order in the grid spacing (linear interpolation between grid points),
    and lie within 1e-3 dB / deg / ms of them at 2,000 points; b_PC equals the minimum over the
    same grid."""
    from parity_helpers import closed_form_margins
    errs = {}
    for F in (200, 400, 2000):
        p = synth.first_order_loop(freq=F, gains=((5.0, 0.05), (20.0, 0.2)))
        cfg = ce.EngineConfig.parse(p.config_text)
        orc = oracle_mod.Oracle(p.config_text, p.plant)
        lina = orc.lina(p.cuda_mx)
        out = orc.allmargin(lina, p.cuda_mx, p.info_mx)
        for r in range(2):
            am = out[r, cfg.info_allmargin:cfg.info_allmargin + 5]
            want = closed_form_margins(p, lina[r, 0], cfg.crossover, row=r)
            assert am[3] == 1.0  # nominal loop stable
            errs[F, r] = np.abs(am[[0, 1, 2]] - [want["gm"], want["pm"], want["dm"]])
            assert abs(am[4] - want["bpc"]) <= 1e-5 * want["bpc"], (am[4], want["bpc"])
    for r in range(2):
        assert (errs[2000, r] < 1e-3).all(), errs[2000, r]
        # second order while the interpolation error dominates (at 2,000 points float32
        # rounding is of the same size): twice the points, ~4x smaller error (at least 3x)
        assert (errs[200, r] > 3 * errs[400, r]).all(), (errs[200, r], errs[400, r])


def test_fused_eigensolve_lapack(oracle_mod):
    """The fused eigensolve arithmetic (one fma per multiply-add) against LAPACK, as the separate
    form is above."""
    rng = np.random.default_rng(4)
    for n in list(range(1, 17)) * 2:
        A = rng.standard_normal((n, n))
        ok, ev = oracle_mod.eig_matrix(A, fused=True)
        assert ok
        ref = np.linalg.eigvals(A)
        key = lambda z: (round(z.real, 6), round(abs(z.imag), 6), np.sign(z.imag))
        np.testing.assert_allclose(sorted(ev, key=key), sorted(ref, key=key), rtol=1e-9,
                                   atol=1e-9 * max(1.0, np.abs(ref).max()))


def test_fused_eigensolve_agrees_with_separate_on_the_eight_state_workload(oracle_mod):
    """The engine's default eigensolve arithmetic against the reference's, both restated in the
    oracle, on every candidate of the 65,536-candidate eight-state workload (T = 10,000, F = 400):
    LIN_A's FP64 eigenvalues within 1e-9 of each other relative to the matrix's largest |lambda|
    (they are ~1e-14 apart), the same modal-stability class for every candidate, and the same
    nominal closed-loop verdict and margins (the margin stage on every candidate, none pre-flagged).
    For a few matrices (82 of 65,536) the QR iteration deflates two eigenvalues in the other order,
    so they are compared as matched sets and the reordered ones are bounded."""
    p = synth.eight_state()
    sep = oracle_mod.Oracle(p.config_text, p.plant, eig_fused=False)
    fus = oracle_mod.Oracle(p.config_text, p.plant, eig_fused=True)
    lina = sep.lina(p.cuda_mx)
    a = sep.eigensolve(lina, fp64=True).reshape(len(lina), -1, 2)
    b = fus.eigensolve(lina, fp64=True).reshape(len(lina), -1, 2)
    za, zb = a[..., 0] + 1j * a[..., 1], b[..., 0] + 1j * b[..., 1]
    assert np.isfinite(za).all() and np.isfinite(zb).all()
    scale = np.abs(za).max(axis=1)
    rel = np.abs(za - zb).max(axis=1) / scale
    reordered = np.where(rel > 1e-9)[0]
    assert len(reordered) <= 0.005 * len(za), len(reordered)
    for k in reordered:  # the same eigenvalues in another Schur order
        d = np.abs(za[k][:, None] - zb[k][None, :])
        assert d.min(axis=1).max() <= 1e-9 * scale[k] and d.min(axis=0).max() <= 1e-9 * scale[k], k
    # modal stability as the modal stage tests it, on the float eigenvalues
    fa = np.hypot(a[..., 0].astype(np.float32), a[..., 1].astype(np.float32)).max(axis=1) > 1
    fb = np.hypot(b[..., 0].astype(np.float32), b[..., 1].astype(np.float32)).max(axis=1) > 1
    assert np.array_equal(fa, fb)
    # the nominal closed loop's verdict (and with it the margins) on every candidate
    ra = sep.allmargin(lina, p.cuda_mx, p.info_mx)
    rb = fus.allmargin(lina, p.cuda_mx, p.info_mx)
    assert np.array_equal(ra, rb, equal_nan=True)


def test_fp64_sim_linear_matches_float64_recurrence(oracle_mod):
    """The oracle's FP64 form of the simulation, with no nonlinearity and K = L = 0, is the plant's
    step response to u = N r computed in float64 (the same recurrence, fused as the engine fuses
    it): 1e-12 relative, against 1e-5 for the float form above."""
    p = synth.mass_spring(1536)
    p.plant.nl_info[:] = 0
    g = np.zeros((1, 7), np.float32)
    g[0, 6] = 2.0
    cfg = ce.EngineConfig.parse(p.config_text)
    _, d = oracle_mod.Oracle(p.config_text, p.plant).evaluate64(g, p.info_mx[:1])
    A = p.plant.discrete_a.reshape(2, 2).astype(np.float64)
    B = p.plant.discrete_bu.astype(np.float64)
    x = np.zeros(2)
    ref = np.empty(cfg.time)
    for t in range(cfg.time):
        ref[t] = x[0]
        u = 0.0 if t < cfg.ref_step_id else 2.0
        x = A @ x + B * u
    w = ref[cfg.fit_start_id:cfg.fit_start_id + cfg.fit_steps]
    np.testing.assert_allclose(d["ywin"][0], w, rtol=1e-12, atol=1e-15 * np.abs(w).max())
    np.testing.assert_allclose(d["summ"][0, 0], ref[cfg.steady_start_id:].sum(), rtol=1e-12)


def test_fp64_margins_closed_form(oracle_mod):
    """The oracle's FP64 margins on the loop with a closed form converge to the exact margins at
    second order in the grid spacing, like the float restatement, and sit within 1e-3 of them at
    2,000 points; the remaining error is the linear interpolation between grid points."""
    from parity_helpers import closed_form_margins
    errs = {}
    for F in (200, 400, 2000):
        p = synth.first_order_loop(freq=F, gains=((5.0, 0.05), (20.0, 0.2)))
        cfg = ce.EngineConfig.parse(p.config_text)
        orc = oracle_mod.Oracle(p.config_text, p.plant)
        out, d = orc.evaluate64(p.cuda_mx, p.info_mx)
        for r in range(2):
            am = out[r, cfg.info_allmargin:cfg.info_allmargin + 5]
            want = closed_form_margins(p, d["lina"][r, 0], cfg.crossover, row=r)
            if am[3] != 1.0:
                continue
            errs[F, r] = np.abs(am[[0, 1]] - [want["gm"], want["pm"]])
    assert errs, "no candidate reached the margin sweep"
    for (F, r), e in errs.items():
        if F == 2000:
            assert (e < 1e-3).all(), e
        if F == 200 and (400, r) in errs:
            assert (e > 3 * errs[400, r]).all(), (e, errs[400, r])
