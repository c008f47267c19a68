"""The Kalman observer (`observer = kalman`, ref: src/discrete_solves.cu:83-185) on the CPU:
the config key and row width, and the oracle's restatement of the Kalman loop checked
against an independent float64 Kalman filter written here with numpy (the same method,
none of the reference's float32 roundings), so the restatement is the filter it claims to
be.  The GPU kernel is compared with the oracle bit for bit in test_gpu_kalman.py, and the
oracle with the reference's own compiled Kalman kernel in test_gpu_reference_kernels.py."""
import numpy as np
import pytest

import controllerengine_gb300 as ce
from controllerengine_gb300 import synth


def test_config_observer_key_and_row_width():
    p = synth.mass_spring(8)
    cfg = ce.EngineConfig.parse(p.config_text)
    assert cfg.observer == 0 and cfg.cuda_mx_width == 2 * cfg.statespace_dim + 1
    k = synth.with_kalman(p)
    cfg = ce.EngineConfig.parse(k.config_text)
    assert cfg.observer == 1 and cfg.cuda_mx_width == 3 * cfg.statespace_dim + 2
    assert k.cuda_mx.shape[1] == cfg.cuda_mx_width
    with pytest.raises(ce.ControllerEngineError, match="observer"):
        ce.EngineConfig.parse(p.config_text + "observer = extended\n")


def _chain(decoded):
    return [tuple(r) for r in decoded if r[0] != 0]


def _interp(chain, src, seed=None):
    """The instruction interpreter (ref: src/main.cu:260-291) in float64, vectorised over rows."""
    res = None
    for op, col, ak, bk, av, bv in chain:
        pos = src[:, col]
        if res is None:
            prev = pos if seed is None else np.where(np.isnan(seed), pos, seed)
        else:
            prev = res
        a = av if ak == 0 else (pos if ak == 1 else prev)
        b = bv if bk == 0 else (pos if bk == 1 else prev)
        a = np.broadcast_to(np.asarray(a, np.float64), pos.shape)
        b = np.broadcast_to(np.asarray(b, np.float64), pos.shape)
        if op == 1:
            res = a + b
        elif op == 2:
            res = a - b
        elif op == 3:
            res = a * b
        elif op == 4:
            res = a / b
        elif op == 5:
            res = np.minimum(np.maximum(prev, a), b)
        elif op == 6:
            res = np.sign(a)
    return np.zeros(src.shape[0]) if res is None else res


def kalman_f64(problem):
    """The time-varying Kalman loop in plain float64: predict, covariance, gain, correction,
    Joseph update, then the nonlinear plant step; rows [K, L, N, R, Q]."""
    cfg = ce.EngineConfig.parse(problem.config_text)
    pl = problem.plant
    ns, nd, nw = cfg.statespace_dim, cfg.discrete_dim, cfg.nonlin_dim
    g = problem.cuda_mx.astype(np.float64)
    n = g.shape[0]
    K, N, R, Q = g[:, :ns], g[:, 2 * ns], g[:, 2 * ns + 1], g[:, 2 * ns + 2:3 * ns + 2]
    A = np.asarray(pl.statespace_a, np.float64).reshape(ns, ns)
    B = np.asarray(pl.statespace_b, np.float64).reshape(ns)
    C = np.asarray(pl.statespace_c, np.float64).reshape(ns)
    Ad = np.asarray(pl.discrete_a, np.float64)[:nd * nd].reshape(nd, nd)
    Bu = np.asarray(pl.discrete_bu, np.float64)[:nd]
    Bw = np.asarray(pl.discrete_bw, np.float64)[:nd * nw].reshape(nd, nw)
    bp = np.asarray(pl.base_params, np.float32)[:cfg.n_params]
    dc = _chain(ce.decode_instructions(pl.dc_info, nd, cfg.dc_instructions, bp))
    u_ch = _chain(ce.decode_instructions(pl.u_info, ns, cfg.u_instructions, bp))
    rows = np.asarray(pl.nl_info, np.int32).reshape(-1, nd + 1)
    nl, r0 = [], 0
    for k in range(nw):
        cnt = cfg.nl_instructions[k]
        nl.append(_chain(ce.decode_instructions(rows[r0:r0 + cnt], nd + 1, cnt, bp)))
        r0 += cnt
    xh, xp = np.zeros((n, ns)), np.zeros((n, nd))
    P = np.zeros((n, ns, ns))
    eye = np.eye(ns)
    y_out = np.empty((n, cfg.time))
    for t in range(cfg.time):
        y = _interp(dc, xp)
        y_out[:, t] = y
        ref = 0.0 if t < cfg.ref_step_time * cfg.time else float(np.float32(cfg.ref_amplitude))
        u = _interp(u_ch, xh, seed=N * ref - np.einsum("ni,ni->n", K, xh))
        xh = xh @ A.T + B[None] * u[:, None]
        P = A[None] @ P @ A.T[None] + Q[:, :, None] * eye[None]
        pc = P @ C
        kg = pc / (pc @ C + R)[:, None]
        xh = xh + kg * (y - xh @ C)[:, None]
        M = eye[None] - kg[:, :, None] * C[None, None, :]
        P = M @ P @ M.transpose(0, 2, 1) + R[:, None, None] * kg[:, :, None] * kg[:, None, :]
        src = np.hstack([xp, y[:, None]])
        W = np.stack([_interp(c, src) for c in nl], axis=1) if nw else np.zeros((n, 0))
        xp = xp @ Ad.T + Bu[None] * u[:, None] + (W @ Bw.T if nw else 0.0)
    return y_out


@pytest.mark.parametrize("make", [lambda: synth.with_kalman(synth.mass_spring(24), seed=5),
                                  lambda: synth.eight_state(n=24, time=600, freq=40, observer="kalman")],
                         ids=["mass_spring_3_state", "eight_state"])
def test_oracle_kalman_is_the_kalman_filter(oracle_mod, make):
    p = make()
    if p.name.startswith("mass_spring"):
        p.config_text = p.config_text.replace("time = 2000", "time = 800")
    orc = oracle_mod.Oracle(p.config_text, p.plant)
    y = orc.sim(p.cuda_mx)
    y64 = kalman_f64(p)
    assert np.isfinite(y).all()
    scale = np.abs(y64).max(axis=1, keepdims=True)
    err = (np.abs(y - y64) / scale).max(axis=1)
    if p.name.startswith("mass_spring"):
        assert err.max() < 2e-4, err.max()  # a smooth loop: every row
    else:
        # the Coulomb-friction sign and the rate clamp are discontinuous, so a 1-ulp
        # difference at a switching instant can send a row elsewhere; the rest agree
        # to float32 rounding
        assert np.median(err) < 1e-6 and (err < 1e-4).mean() >= 0.75, err


def test_oracle_kalman_entry_points_agree(oracle_mod):
    """oracle_sim on a Kalman config and oracle_sim_kalman on the same rows are one loop; the
    reference's literal form (rows [K, N, R, Q], in-place Joseph product) differs."""
    p = synth.eight_state(n=16, time=1500, freq=40, observer="kalman")
    orc = oracle_mod.Oracle(p.config_text, p.plant)
    y = orc.sim(p.cuda_mx)
    y2, steady = orc.sim_kalman(p.cuda_mx)
    assert np.array_equal(y.view(np.uint32), y2.view(np.uint32))
    assert (steady >= 0).any()  # the covariance recursion reaches a fixed point
    ns = 8
    lit = np.hstack([p.cuda_mx[:, :ns], p.cuda_mx[:, 2 * ns:]])  # [K, N, R, Q]
    y3, _ = orc.sim_kalman(lit, literal=True)
    assert np.array_equal(y[:, :4], y3[:, :4])  # the covariance reaches y only after a few steps
    assert not np.array_equal(y, y3)
