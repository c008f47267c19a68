"""Seeded synthetic tuning workloads in the reference's file format.

The reference ships no sample inputs, so every workload is generated from a
seed: a ControllerEngine.config text, the plant/observer/instruction .bin set
and the CUDA_MX / INFO_MX candidate rows.  Shapes and distributions follow the
benchmark configurations of this port:

* ``mass_spring``   -- 2-state mass-spring-damper (m=1, k=4, c=0.4, ZOH at
  dt=1e-3) with a cubic spring term k3*x0^3 (k3=0.5) written as NL multiply
  instructions, y = x0, a 3-state observer model (plant + leaky integrator of
  the input disturbance, pole 0.999), u clamped to [-10, 10], gains log-uniform in [0.1, 10];
  2000 steps, unit step at 0.1 s, fit 0.1-1.5 s, steady from 1.5 s, 200 sweep
  points from 1e-2 rad/s.
* ``eight_state``   -- 8-state plant with a seeded stable spectrum (4 complex
  pairs, |z| ~ U[0.90, 0.995], angle ~ U[0.01, 0.5] rad) in a random orthogonal
  basis, B_u and C ~ N(0, 1); four nonlinear terms (cubic stiffness, Coulomb
  friction, a rate clamp, a division by 1 + a x_k^2); an 8-state observer with a
  steady-state Kalman gain per candidate (from a seeded pool of Q, R); u
  saturated to [-5, 5]; 10,000 steps, 400 sweep points.

The instruction interpreter can only read single states, so the output
y = C x cannot be written as a DC chain; the eight-state plant is therefore
stored in the coordinates z = T x with first row of T equal to C (the rest an
orthonormal complement), where C z-coordinates is e_0 and the DC chain is
y = z_0.  The spectrum and the input/output behaviour are those of the drawn
(A, B_u, C).

The sweep always ends at Nyquist (pi/ts), as in the reference.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
from scipy.linalg import expm, solve_discrete_are

from .engine import PlantFiles

F32 = np.float32


def pack(op: int, d1: int, d2: int) -> int:
    """Base-36 instruction entry: op*36^2 + d1*36 + d2 (digit 0 = state, 35 = running value, k = BASE_PARAMS[k-1])."""
    return op * 1296 + d1 * 36 + d2


ADD, SUB, MUL, DIV, SAT, SGN = 1, 2, 3, 4, 5, 6
STATE, PREV = 0, 35


def instr_rows(chain: list[tuple[int, int, int, int]], dim: int) -> np.ndarray:
    """Rows of width `dim`, one per (op, col, d1, d2)."""
    rows = np.zeros((len(chain), dim), np.int32)
    for r, (op, col, d1, d2) in enumerate(chain):
        rows[r, col] = pack(op, d1, d2)
    return rows


@dataclass
class Problem:
    name: str
    config_text: str
    plant: PlantFiles
    cuda_mx: np.ndarray   # n x (2ns+1), or n x (3ns+2) with the Kalman observer
    info_mx: np.ndarray   # n x info_w
    n_plants: int = 1

    def write(self, directory):
        from pathlib import Path
        d = Path(directory)
        d.mkdir(parents=True, exist_ok=True)
        (d / "ControllerEngine.config").write_text(self.config_text)
        self.plant.write(d)
        self.cuda_mx.astype(F32).tofile(d / "CUDA_MX.bin")
        self.info_mx.astype(F32).tofile(d / "INFO_MX.bin")


def _config_text(**kv) -> str:
    lines = []
    for k, v in kv.items():
        if isinstance(v, (list, tuple)):
            v = ",".join(str(x) for x in v)
        lines.append(f"{k} = {v}")
    return "\n".join(lines) + "\n"


def info_width(ns: int, nd: int, input_size: int) -> int:
    return input_size + 3 + 4 + 5 + 3 * (ns + nd) + 1


def zoh(Ac: np.ndarray, Bc: np.ndarray, dt: float):
    n, m = Ac.shape[0], Bc.shape[1]
    M = np.zeros((n + m, n + m))
    M[:n, :n] = Ac
    M[:n, n:] = Bc
    E = expm(M * dt)
    return E[:n, :n], E[:n, n:]


def mass_spring(n: int = 1536, seed: int = 1, preflag: bool = True) -> Problem:
    rng = np.random.default_rng(seed)
    m, k, c, k3, dt = 1.0, 4.0, 0.4, 0.5, 1e-3
    Ac = np.array([[0.0, 1.0], [-k / m, -c / m]])
    Bc = np.array([[0.0], [1.0 / m]])
    Ad, Bd = zoh(Ac, Bc, dt)
    Bw = -Bd  # the cubic spring force opposes the displacement
    # observer model: plant + a slowly leaking input-disturbance integrator
    # (x' = Ax + B(u + d), d' = 0.999 d); a pole exactly at 1 would sit,
    # uncontrollable, in every nominal closed loop of the margin check
    As = np.zeros((3, 3))
    As[:2, :2] = Ad
    As[:2, 2:] = Bd
    As[2, 2] = 0.999
    Bs = np.array([Bd[0, 0], Bd[1, 0], 0.0])
    Cs = np.array([1.0, 0.0, 0.0])
    # BASE_PARAMS: k3, umax, umin, one, minus one, zero
    bp = np.array([k3, 10.0, -10.0, 1.0, -1.0, 0.0], F32)
    dc = instr_rows([(MUL, 0, STATE, 4)], 2)                              # y = x0 * 1
    u = instr_rows([(SAT, 0, 3, 2)], 3)                                   # clamp(u_raw, -10, 10)
    nl = instr_rows([(MUL, 0, STATE, STATE), (MUL, 0, PREV, STATE), (MUL, 0, PREV, 1)], 3)  # k3 x0^3
    plant = PlantFiles(
        statespace_a=As.astype(F32), statespace_a_i=(As.astype(F32) - np.eye(3, dtype=F32)),
        statespace_b=Bs.astype(F32), statespace_c=Cs.astype(F32), statespace_d=np.zeros(1, F32),
        discrete_a=Ad.astype(F32), discrete_a_i=(Ad.astype(F32) - np.eye(2, dtype=F32)),
        discrete_bu=Bd[:, 0].astype(F32), discrete_bw=Bw.astype(F32), discrete_c=np.array([1.0, 0.0], F32),
        base_params=bp, dc_info=dc, u_info=u, nl_info=nl)
    gains = np.exp(rng.uniform(np.log(0.1), np.log(10.0), size=(n, 7))).astype(F32)
    iw = info_width(3, 2, 7)
    info = np.zeros((n, iw), F32)
    info[:, :7] = gains
    if preflag and n >= 8:
        info[3, 7] = 5.0      # pre-flagged below unstable_err: margins still scored
        info[5, 7] = 2.0e6    # pre-flagged above unstable_err: margins zeroed
    text = _config_text(
        statespace_dim=3, discrete_dim=2, nonlin_dim=1, n_params=6, input_size=7, dc_instructions=1,
        u_instructions=1, nl_instructions=[3], n_cores=128 * max(1, n // 1536), n_rounds=1, mode="batch",
        time=2000, duration=2.0, ref_step_time=0.05, ref_amplitude=1.0, fit_start=0.05, fit_end=0.75,
        steady_start=0.75, bandwidth=0.5, damping=0.59, overshoot=0.10, steady_state_error=0.05,
        crossover_coeff=1.0, target_gm=9.0, target_pm=55.0, target_b=0.2, eig_fail_err=1.0e18,
        unstable_err=1.0e6, freq=200, freq_min=0.01)
    return Problem("mass_spring_2state", text, plant, gains, info)


def stable_spectrum_matrix(rng, n: int = 8, rmin=0.90, rmax=0.995, thmin=0.01, thmax=0.5) -> np.ndarray:
    """Real n x n matrix with n/2 complex pole pairs r e^{+-i theta} in a Haar-random orthogonal basis."""
    blocks = np.zeros((n, n))
    for p in range(n // 2):
        r, th = rng.uniform(rmin, rmax), rng.uniform(thmin, thmax)
        blocks[2 * p:2 * p + 2, 2 * p:2 * p + 2] = r * np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
    G = rng.standard_normal((n, n))
    Q, R = np.linalg.qr(G)
    Q = Q * np.sign(np.diag(R))
    return Q @ blocks @ Q.T


def output_first_basis(A, B, C):
    """Similarity z = T x with T[0] = C, other rows an orthonormal basis of C's complement."""
    n = A.shape[0]
    c = C.reshape(1, n)
    _, _, Vt = np.linalg.svd(c)
    T = np.vstack([c, Vt[1:]])
    Ti = np.linalg.inv(T)
    return T @ A @ Ti, T @ B, (c @ Ti).reshape(n)


def eight_state(n: int = 65536, seed: int = 2, time: int = 10000, freq: int = 400, pool: int = 64,
                input_size: int = 17, observer: str = "luenberger") -> Problem:
    """The eight-state workload.  observer="kalman" runs the time-varying Kalman filter in the
    simulation: each row becomes [K, L, N, R, Q] with the noise weights (R, diag Q) that L was
    computed from, and the config says `observer = kalman`."""
    rng = np.random.default_rng(seed)
    ns = nd = 8
    A0 = stable_spectrum_matrix(rng, 8)
    B0 = rng.standard_normal((8, 1))
    C0 = rng.standard_normal(8)
    A, B, C = output_first_basis(A0, B0, C0)
    Cz = np.zeros(8)
    Cz[0] = 1.0
    Bw = 1e-3 * rng.standard_normal((8, 4))
    i, j, k, m_ = (int(v) for v in rng.choice(8, size=4, replace=False))
    c_fric, r_clamp, a_div = rng.uniform(0.01, 0.1), rng.uniform(0.5, 2.0), rng.uniform(0.0, 1.0)
    # BASE_PARAMS: 1 one, 2 Coulomb c, 3 -r, 4 r, 5 a, 6 umin, 7 umax, 8 zero
    bp = np.array([1.0, c_fric, -r_clamp, r_clamp, a_div, -5.0, 5.0, 0.0], F32)
    dc = instr_rows([(MUL, 0, STATE, 1)], nd)
    u = instr_rows([(SAT, 0, 6, 7)], ns)
    nl_chains = [
        [(MUL, i, STATE, STATE), (MUL, i, PREV, STATE)],                          # x_i^3
        [(SGN, j, STATE, STATE), (MUL, j, PREV, 2)],                              # c sign(x_j)
        [(SAT, k, 3, 4), (SUB, k, PREV, STATE)],                                  # clamp(x_k,-r,r) - x_k
        [(MUL, k, STATE, STATE), (MUL, k, PREV, 5), (ADD, k, PREV, 1), (DIV, m_, STATE, PREV)],  # x_m/(1+a x_k^2)
    ]
    nl = np.vstack([instr_rows(ch, nd + 1) for ch in nl_chains])
    Af, Bf = A.astype(F32), B[:, 0].astype(F32)
    plant = PlantFiles(
        statespace_a=Af, statespace_a_i=Af - np.eye(8, dtype=F32), statespace_b=Bf, statespace_c=Cz.astype(F32),
        statespace_d=np.zeros(1, F32), discrete_a=Af, discrete_a_i=Af - np.eye(8, dtype=F32), discrete_bu=Bf,
        discrete_bw=Bw.astype(F32), discrete_c=Cz.astype(F32), base_params=bp, dc_info=dc, u_info=u, nl_info=nl)
    # a pool of LQR state-feedback and steady-state Kalman predictor gains from seeded weights
    Ks, Ls, Rs, Qs = [], [], [], []
    for _ in range(pool):
        Qk = np.diag(np.exp(rng.uniform(np.log(1e-2), np.log(1e1), 8)))
        Rk = np.array([[np.exp(rng.uniform(np.log(1e-1), np.log(1e1)))]])
        P = solve_discrete_are(A, B, Qk, Rk)
        Ks.append(np.linalg.solve(Rk + B.T @ P @ B, B.T @ P @ A).reshape(8))
        Qo = np.diag(np.exp(rng.uniform(np.log(1e-3), np.log(1e0), 8)))
        Ro = np.array([[np.exp(rng.uniform(np.log(1e-2), np.log(1e0)))]])
        S = solve_discrete_are(A.T, Cz.reshape(8, 1), Qo, Ro)
        Ls.append((A @ S @ Cz / (Cz @ S @ Cz + Ro[0, 0])).reshape(8))
        Rs.append(Ro[0, 0])
        Qs.append(np.diag(Qo))
    Ks, Ls, Rs, Qs = np.array(Ks), np.array(Ls), np.array(Rs), np.array(Qs)
    ki = rng.integers(0, pool, n)
    li = rng.integers(0, pool, n)
    scale = np.exp(rng.uniform(np.log(0.3), np.log(4.0), (n, 1)))
    K = Ks[ki] * scale
    L = Ls[li]
    # prefilter N = 1 / closed-loop DC gain of the linear loop, perturbed
    Acl = A[None] - B[None] * K[:, None, :]
    dcg = np.einsum("j,njk,k->n", Cz, np.linalg.inv(np.eye(8)[None] - Acl), B[:, 0])
    N = (1.0 / np.where(np.abs(dcg) > 1e-6, dcg, 1.0)) * rng.uniform(0.8, 1.2, n)
    gains = np.hstack([K, L, N[:, None]]).astype(F32)
    extra = {}
    if observer == "kalman":
        gains = np.hstack([gains, Rs[li][:, None].astype(F32), Qs[li].astype(F32)])
        extra["observer"] = "kalman"
    elif observer != "luenberger":
        raise ValueError(f"observer {observer!r}")
    iw = info_width(ns, nd, input_size)
    info = np.zeros((n, iw), F32)
    info[:, :min(input_size, 17)] = gains[:, :min(input_size, 17)]
    text = _config_text(
        statespace_dim=8, discrete_dim=8, nonlin_dim=4, n_params=8, input_size=input_size, dc_instructions=1,
        u_instructions=1, nl_instructions=[2, 2, 2, 4], n_cores=128 * max(1, -(-n // 1536)), n_rounds=1,
        mode="batch", time=time, duration=time * 1e-3, ref_step_time=0.05, ref_amplitude=1.0, fit_start=0.05,
        fit_end=0.75, steady_start=0.75, bandwidth=10.0, damping=0.6, overshoot=0.10, steady_state_error=0.05,
        crossover_coeff=1.0, target_gm=9.0, target_pm=55.0, target_b=0.2, eig_fail_err=1.0e18, unstable_err=1.0e6,
        freq=freq, freq_min=0.1, **extra)
    return Problem("eight_state" if observer == "luenberger" else "eight_state_kalman", text, plant, gains, info)


def stable_matrix(rng, n: int, rmin=0.85, rmax=0.995, thmin=0.01, thmax=0.5) -> np.ndarray:
    """Real n x n matrix with floor(n/2) complex pole pairs and, for odd n, one real pole, all of
    modulus in [rmin, rmax], in a Haar-random orthogonal basis."""
    blocks = np.zeros((n, n))
    for p in range(n // 2):
        r, th = rng.uniform(rmin, rmax), rng.uniform(thmin, thmax)
        blocks[2 * p:2 * p + 2, 2 * p:2 * p + 2] = r * np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
    if n % 2:
        blocks[n - 1, n - 1] = rng.uniform(rmin, rmax)
    Q, R = np.linalg.qr(rng.standard_normal((n, n)))
    Q = Q * np.sign(np.diag(R))
    return Q @ blocks @ Q.T


def random_shape(seed: int, n: int = 256, time: int | None = None, freq: int | None = None) -> Problem:
    """One instance of the uneven-shape workload: statespace and discrete dimensions U{2..8},
    0-4 nonlinear terms with 1-8 instructions each (no-op and SKIP rows included), horizon
    log-uniform in [1e3, 2e4] steps and 50-400 sweep points unless given.  The observer model
    (ns states) is a separately drawn stable system with y = z_0; the plant (nd states) is drawn
    the same way; K is an LQR gain and L a steady-state Kalman predictor gain of the model, both
    from seeded weights and scaled per candidate, so the batch holds stable and unstable loops."""
    rng = np.random.default_rng(seed)
    ns, nd, nw = int(rng.integers(2, 9)), int(rng.integers(2, 9)), int(rng.integers(0, 5))
    if time is None:
        time = int(np.exp(rng.uniform(np.log(1e3), np.log(2e4))))
    if freq is None:
        freq = int(rng.integers(50, 401))
    ts = 1e-3
    # observer model in output-first coordinates
    Am, Bm, Cm = output_first_basis(stable_matrix(rng, ns), rng.standard_normal((ns, 1)), rng.standard_normal(ns))
    e0s = np.zeros(ns)
    e0s[0] = 1.0
    Ap, Bp, _ = output_first_basis(stable_matrix(rng, nd), rng.standard_normal((nd, 1)), rng.standard_normal(nd))
    e0d = np.zeros(nd)
    e0d[0] = 1.0
    Bw = 1e-3 * rng.standard_normal((nd, nw))
    # BASE_PARAMS: 1 one, 2 small coefficient, 3 -r, 4 r, 5 umin, 6 umax, 7 second coefficient
    c1, c2, r = rng.uniform(0.01, 0.5), rng.uniform(-0.5, 0.5), rng.uniform(0.2, 2.0)
    bp = np.array([1.0, c1, -r, r, -5.0, 5.0, c2], F32)
    dc_chain = [(MUL, 0, STATE, 1)]
    if rng.random() < 0.5:
        dc_chain.append((7, 0, STATE, STATE))  # an op outside 1..6: no change
    u_chain = [(SAT, 0, 5, 6)]
    nl_rows, nl_counts = [], []
    for _ in range(nw):
        i, j = int(rng.integers(0, nd)), int(rng.integers(0, nd + 1))  # j == nd reads the plant output
        kind = int(rng.integers(0, 4))
        if kind == 0:
            ch = [(MUL, i, STATE, STATE), (MUL, i, PREV, STATE), (MUL, i, PREV, 2)]
        elif kind == 1:
            ch = [(SGN, j, STATE, STATE), (MUL, j, PREV, 2)]
        elif kind == 2:
            ch = [(SAT, i, 3, 4), (SUB, i, PREV, STATE)]
        else:
            ch = [(MUL, j, STATE, 7), (ADD, i, PREV, STATE), (DIV, i, PREV, 1)]
        while len(ch) < 8 and rng.random() < 0.3:
            ch.insert(int(rng.integers(0, len(ch) + 1)), (0, int(rng.integers(0, nd + 1)), 0, 0))  # SKIP row
        rows = instr_rows(ch, nd + 1)
        nl_rows.append(rows)
        nl_counts.append(len(ch))
    nl = np.vstack(nl_rows) if nl_rows else np.zeros((0, nd + 1), np.int32)
    Amf, Bmf, Apf, Bpf = Am.astype(F32), Bm[:, 0].astype(F32), Ap.astype(F32), Bp[:, 0].astype(F32)
    plant = PlantFiles(
        statespace_a=Amf, statespace_a_i=Amf - np.eye(ns, dtype=F32), statespace_b=Bmf,
        statespace_c=e0s.astype(F32), statespace_d=np.zeros(1, F32), discrete_a=Apf,
        discrete_a_i=Apf - np.eye(nd, dtype=F32), discrete_bu=Bpf, discrete_bw=Bw.astype(F32),
        discrete_c=e0d.astype(F32), base_params=bp, dc_info=instr_rows(dc_chain, nd),
        u_info=instr_rows(u_chain, ns), nl_info=nl)
    Qk = np.diag(np.exp(rng.uniform(np.log(1e-2), np.log(1e1), ns)))
    Rk = np.array([[np.exp(rng.uniform(np.log(1e-1), np.log(1e1)))]])
    P = solve_discrete_are(Am, Bm, Qk, Rk)
    K0 = np.linalg.solve(Rk + Bm.T @ P @ Bm, Bm.T @ P @ Am).reshape(ns)
    Qo = np.diag(np.exp(rng.uniform(np.log(1e-3), np.log(1e0), ns)))
    S = solve_discrete_are(Am.T, e0s.reshape(ns, 1), Qo, np.array([[0.1]]))
    L0 = (Am @ S @ e0s / (e0s @ S @ e0s + 0.1)).reshape(ns)
    K = K0[None] * np.exp(rng.uniform(np.log(0.2), np.log(5.0), (n, 1)))
    L = L0[None] * np.exp(rng.uniform(np.log(0.5), np.log(2.0), (n, 1)))
    Nn = np.exp(rng.uniform(np.log(0.5), np.log(2.0), (n, 1)))
    gains = np.hstack([K, L, Nn]).astype(F32)
    input_size = 2 * ns + 1
    info = np.zeros((n, info_width(ns, nd, input_size)), F32)
    info[:, :input_size] = gains
    text = _config_text(
        statespace_dim=ns, discrete_dim=nd, nonlin_dim=nw, n_params=len(bp), input_size=input_size,
        dc_instructions=len(dc_chain), u_instructions=len(u_chain), nl_instructions=nl_counts,
        n_cores=128 * max(1, -(-n // 1536)), n_rounds=1, mode="batch", time=time, duration=time * ts,
        ref_step_time=0.05, ref_amplitude=1.0, fit_start=0.05, fit_end=0.75, steady_start=0.75,
        bandwidth=float(np.exp(rng.uniform(np.log(0.5), np.log(20.0)))), damping=0.6, overshoot=0.10,
        steady_state_error=0.05, crossover_coeff=1.0, target_gm=6.0, target_pm=45.0, target_b=0.2,
        eig_fail_err=1.0e18, unstable_err=1.0e6, freq=freq, freq_min=0.1)
    return Problem(f"random_shape_{seed}", text, plant, gains, info)


def first_order_loop(freq: int = 2000, a: float = 0.99, b: float = 0.01, gains=((5.0, 0.05),)) -> Problem:
    """A loop whose margins have a closed form: a first-order observer model P(z) = c b / (z - a)
    (c = 1, d = 0; batch mode, so the margin check uses this model) and per row gains (k, l, N = 1),
    whose compensator is G(z) = k l / (z - a_cl) with a_cl = a - b k - l c, the observer block of
    LIN_A.  The loop P G = c b k l / ((z - a)(z - a_cl)) has one gain crossover and one phase
    crossover in (0, pi).  The simulated plant is a first-order lag; no nonlinear terms."""
    bp = np.array([1.0, -1e6, 1e6], F32)
    dc = instr_rows([(MUL, 0, STATE, 1)], 1)                                   # y = x0 * 1
    u = instr_rows([(SAT, 0, 2, 3)], 1)                                        # clamp(u_raw, -1e6, 1e6)
    plant = PlantFiles(
        statespace_a=np.array([a], F32), statespace_a_i=np.array([a], F32) - F32(1),
        statespace_b=np.array([b], F32), statespace_c=np.array([1.0], F32), statespace_d=np.zeros(1, F32),
        discrete_a=np.array([0.95], F32), discrete_a_i=np.array([0.95], F32) - F32(1),
        discrete_bu=np.array([0.05], F32), discrete_bw=np.zeros(0, F32), discrete_c=np.array([1.0], F32),
        base_params=bp, dc_info=dc, u_info=u, nl_info=np.zeros((0, 2), np.int32))
    g = np.array([[k, l, 1.0] for k, l in gains], F32)
    info = np.zeros((g.shape[0], info_width(1, 1, 3)), F32)
    info[:, :3] = g
    text = _config_text(
        statespace_dim=1, discrete_dim=1, nonlin_dim=0, n_params=3, input_size=3, dc_instructions=1,
        u_instructions=1, nl_instructions="", n_cores=128, n_rounds=1, mode="batch", time=2000, duration=2.0,
        ref_step_time=0.05, ref_amplitude=1.0, fit_start=0.05, fit_end=0.75, steady_start=0.75, bandwidth=2.0,
        damping=0.6, overshoot=0.1, steady_state_error=0.05, crossover_coeff=1.0, target_gm=6.0, target_pm=45.0,
        target_b=0.2, eig_fail_err=1.0e18, unstable_err=1.0e6, freq=freq, freq_min=0.01)
    return Problem(f"first_order_loop_{freq}", text, plant, g, info)


def perturbed_plants(pl: PlantFiles, n_plants: int, seed: int) -> PlantFiles:
    """n_plants copies of plant `pl` stacked as the plant files of a multi-plant session: A and
    B_u scaled elementwise by (1 + 0.1 N(0,1)) and BASE_PARAMS by U[0.8, 1.2] per plant (A_I
    recomputed), B_w and C kept; the observer model and the instruction tables are shared."""
    rng = np.random.default_rng(seed)
    nd = int(np.sqrt(pl.discrete_a.size))
    A0 = pl.discrete_a.reshape(nd, nd).astype(np.float64)
    Bu0 = pl.discrete_bu.astype(np.float64)
    A = A0[None] * (1.0 + 0.1 * rng.standard_normal((n_plants, nd, nd)))
    Bu = Bu0[None] * (1.0 + 0.1 * rng.standard_normal((n_plants, nd)))
    bp = pl.base_params.astype(np.float64)[None] * rng.uniform(0.8, 1.2, (n_plants, pl.base_params.size))
    Af = A.astype(F32)
    return PlantFiles(
        statespace_a=pl.statespace_a, statespace_a_i=pl.statespace_a_i, statespace_b=pl.statespace_b,
        statespace_c=pl.statespace_c, statespace_d=pl.statespace_d,
        discrete_a=Af.ravel(), discrete_a_i=(Af - np.eye(nd, dtype=F32)[None]).ravel(),
        discrete_bu=Bu.astype(F32).ravel(), discrete_bw=np.tile(pl.discrete_bw, n_plants),
        discrete_c=np.tile(pl.discrete_c, n_plants), base_params=bp.astype(F32).ravel(),
        dc_info=pl.dc_info, u_info=pl.u_info, nl_info=pl.nl_info)


def monte_carlo(n_plants: int = 262144, seed: int = 3, time: int = 8000, freq: int = 400, serial: bool = True,
                base_seed: int = 2) -> Problem:
    """Monte Carlo over plants: the eight-state plant with A and B_u scaled elementwise by
    (1 + 0.1 N(0,1)) and BASE_PARAMS by U[0.8, 1.2] per plant (A_I recomputed), one fixed gain
    set for every plant (the first candidate of the eight-state pool), gain and phase targets
    6 dB / 45 deg.  In `serial` mode (the reference's per-round plants) the margin check uses
    each plant itself.  Returns a Problem whose plant files hold n_plants stacked plants and
    whose CUDA_MX / INFO_MX hold one row per plant."""
    base = eight_state(n=1, seed=base_seed, time=time, freq=freq)
    plant = perturbed_plants(base.plant, n_plants, seed)
    gains = np.repeat(base.cuda_mx[:1], n_plants, axis=0)
    info = np.repeat(base.info_mx[:1], n_plants, axis=0)
    text = base.config_text.replace("mode = batch", "mode = serial" if serial else "mode = batch")
    text = text.replace("target_gm = 9.0", "target_gm = 6.0").replace("target_pm = 55.0", "target_pm = 45.0")
    return Problem(f"monte_carlo_{n_plants}", text, plant, gains, info, n_plants=n_plants)


def with_kalman(p: Problem, seed: int = 7, r_range=(1e-2, 1.0), q_range=(1e-4, 1e-1)) -> Problem:
    """`p` with the time-varying Kalman observer: every row gets a measurement weight R and
    the diagonal of Q appended (log-uniform in the given ranges, seeded), and the config says
    `observer = kalman`.  K, L, N are kept, so LIN_A and the margin sweep see the same loop."""
    import dataclasses
    kv = {k.strip(): v.strip() for k, v in (line.split("=", 1) for line in p.config_text.splitlines() if "=" in line)}
    ns = int(kv["statespace_dim"])
    rng = np.random.default_rng(seed)
    n = p.cuda_mx.shape[0]
    lg = lambda lo, hi, size: np.exp(rng.uniform(np.log(lo), np.log(hi), size))
    rq = np.hstack([lg(*r_range, (n, 1)), lg(*q_range, (n, ns))]).astype(F32)
    return dataclasses.replace(p, name=p.name + "_kalman", config_text=p.config_text + "observer = kalman\n",
                               cuda_mx=np.hstack([p.cuda_mx.astype(F32), rq]))


def _with_keys(text: str, **kv) -> str:
    """`text` with the given config keys set (replaced where present, appended otherwise)."""
    lines, seen = [], set()
    for line in text.splitlines():
        key = line.split("=", 1)[0].strip() if "=" in line else None
        if key in kv:
            lines.append(f"{key} = {kv[key]}")
            seen.add(key)
        else:
            lines.append(line)
    lines += [f"{k} = {v}" for k, v in kv.items() if k not in seen]
    return "\n".join(lines) + "\n"


def uneven(n_inst: int = 16384, seed: int = 9, bases: int = 512) -> list:
    """The uneven-size workload: n_inst instances of one candidate each.  `bases` plants and
    candidate pools are drawn as in random_shape (dimensions U{2..8}, 0-4 nonlinear terms with
    1-8 instructions, observer model, plant, LQR and Kalman-predictor gains); each instance takes
    one of them with its own horizon (log-uniform in [1e3, 2e4] steps), sweep size (U{50..400})
    and one of the base's candidate gain sets."""
    rng = np.random.default_rng(seed)
    per = -(-n_inst // bases)
    out = []
    for b in range(bases):
        base = random_shape(seed * 100003 + b, n=per)
        for k in range(per):
            if len(out) == n_inst:
                break
            T = int(np.exp(rng.uniform(np.log(1e3), np.log(2e4))))
            F = int(rng.integers(50, 401))
            text = _with_keys(base.config_text, time=T, duration=T * 1e-3, freq=F, n_cores=128)
            out.append(Problem(f"uneven_{len(out)}", text, base.plant, base.cuda_mx[k:k + 1].copy(),
                               base.info_mx[k:k + 1].copy()))
    return out
