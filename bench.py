#!/usr/bin/env python
"""Throughput of the GB300 tuning engine: candidates/s on the 8-state, 65,536-candidate workload.

A step is one full evaluation of 65,536 candidate gain sets on the 8-state
nonlinear plant (10,000 simulation steps, 400 sweep frequencies): simulation,
LIN_A + FP64 eigensolve, modal fit, modal solve, nominal closed-loop check and
margin sweep, producing the INFO cost rows.

* value -- candidates/s with gains and INFO rows resident in HBM (ce_evaluate_device);
* e2e   -- candidates/s through the C ABI with pinned host buffers (ce_evaluate:
           H2D gains + INFO rows, the pipeline, D2H INFO rows, every step);
* roofline -- the dominant kernel, timed live with CUDA events on its stream;
* cpu_baseline -- the CPU oracle (a C port of the reference method, OpenMP) on a
           bounded sample of the same workload on this host's cores;
* fp64_form -- the same pipeline with every stage in FP64 (the plain FP64 form);
* monte_carlo, kalman, serving -- the per-candidate-plant, Kalman-observer and
           request-serving workloads.

`--impl reference` times the reference method on the host cores instead: the
reference's Eigen host path does not build here (Eigen is not vendored), so the
C port of its method in oracle/ stands in for it.  Its line also carries
`reference_gpu_build`: the reference's own kernels (compiled from its sources
for sm_103a) on the GPU with its Eigen stages restated on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "tuning candidates/s (8-state, 64K batch)"
UNIT = "candidates/s"


def workload_args(a):
    return dict(n=a.candidates, time=a.time, freq=a.freq)


def precision_report(rows, fp64, cfg):
    """Cost rows of one form (the mixed form: the reference's arithmetic; or the compensated
    form) against the plain FP64 form of the same method on the same candidates: agreement of
    the pass/fail classes, and per cost term, over the candidates both forms score, the
    relative error (median, p99, max, and the fraction within 1e-6).  The overshoot is a
    fraction that is often ~0, so its error is absolute."""
    s, am, fr = cfg.info_scoring, cfg.info_allmargin, cfg.info_freqresp
    def classes(x):
        return np.stack([x[:, s + 1] >= cfg.unstable_err, x[:, s + 2] == np.float32(cfg.unstable_err),
                         x[:, s + 2] == np.float32(cfg.eig_fail_err), x[:, am + 3] == 1.0], axis=1)
    cm, cf = classes(rows), classes(fp64)
    same = (cm == cf).all(axis=1)
    scored = same & ~cm[:, 0] & ~cm[:, 1] & ~cm[:, 2]
    terms = {"total_score": s, "behaviour_err": s + 1, "margin_err": s + 2, "wn": fr, "zeta": fr + 1,
             "overshoot_abs": fr + 2, "yss": fr + 3, "gm_db": am, "pm_deg": am + 1, "dm_ms": am + 2,
             "b_pc": am + 4}
    rel = {}
    for name, col in terms.items():
        a_, b_ = rows[scored, col].astype(np.float64), fp64[scored, col].astype(np.float64)
        ok = np.isfinite(a_) & np.isfinite(b_) & (np.abs(b_) < 1e30)
        den = 1.0 if name.endswith("_abs") else np.maximum(np.abs(b_[ok]), 1e-30)
        e = np.abs(a_[ok] - b_[ok]) / den
        rel[name] = ({"median": float(np.median(e)), "p99": float(np.quantile(e, 0.99)), "max": float(e.max()),
                      "within_1e-6": float((e <= 1e-6).mean())} if e.size else None)
    return {"class_agreement": float(same.mean()), "candidates_compared": int(scored.sum()), "relative_error": rel}


def precision_floor(sess, problem, cfg, sample: int = 4096):
    """Where the compensated form's fit-derived terms miss 1e-6 of the FP64 form: on a sample of
    the batch, per candidate, the FP32 trajectory's difference from the FP64 one (max over the
    fit window, relative to the window's largest |y|) and the condition number of the scaled
    normal matrix (the system the modal solve factors, from the FP64 form); then, binned by that
    condition number, the median relative error of wn, zeta and the behaviour error for the
    compensated and the mixed forms.  Error ~ condition x trajectory difference marks the FP32
    trajectory as the floor; beside them the compensated arithmetic on the FP64 trajectory and the
    compensated_df form (the same arithmetic on a double-float trajectory)."""
    g, info = problem.cuda_mx[:sample], problem.info_mx[:sample]
    nt = cfg.total_dim
    out = {}
    prev = sess.precision
    for form in ("fp64", "compensated", "mixed", "compensated_traj64", "compensated_df"):
        sess.set_precision(form)
        out[form] = sess.evaluate_diagnostics64(g, info, want=("ywin", "ata"))
    sess.set_precision(prev)
    (f64, d64), (cmp_, dc), (mix, _) = out["fp64"], out["compensated"], out["mixed"]
    # the compensated form's arithmetic on the FP64 trajectory: what remains against the FP64 form
    # once the FP32 trajectory is taken out
    t64 = precision_report(out["compensated_traj64"][0], f64, cfg)
    dfr, ddf_ = out["compensated_df"]
    s, fr, md = cfg.info_scoring, cfg.info_freqresp, cfg.info_modal
    yscale = np.maximum(np.abs(d64["ywin"]).max(axis=1), 1e-30)
    traj = np.abs(dc["ywin"] - d64["ywin"]).max(axis=1) / yscale
    traj_df = np.abs(ddf_["ywin"] - d64["ywin"]).max(axis=1) / yscale
    uniq = f64[:, md + 3 * nt].astype(int)
    cond = np.full(len(g), np.inf)
    ata = d64["ata"].reshape(-1, 2 * nt, 2 * nt)
    for u in np.unique(uniq):
        if u <= 0:
            continue
        idx = np.where(uniq == u)[0]
        A = ata[idx, :2 * u, :2 * u]
        A = np.tril(A) + np.transpose(np.tril(A, -1), (0, 2, 1))
        dg = np.sqrt(np.abs(np.einsum("kii->ki", A)))
        dg[dg <= 1e-6] = 1.0
        with np.errstate(all="ignore"):
            cond[idx] = np.linalg.cond(A / dg[:, :, None] / dg[:, None, :])
    scored = (f64[:, s + 1] < cfg.unstable_err) & (cmp_[:, s + 1] < cfg.unstable_err) & np.isfinite(cond)
    def rel(x, col):
        a_, b_ = x[:, col].astype(np.float64), f64[:, col].astype(np.float64)
        return np.abs(a_ - b_) / np.maximum(np.abs(b_), 1e-30)
    bins = []
    for lo in range(0, 12, 2):
        sel = scored & (cond >= 10.0 ** lo) & (cond < 10.0 ** (lo + 2))
        if sel.sum() < 4:
            continue
        row = {"cond": f"1e{lo}..1e{lo + 2}", "candidates": int(sel.sum()),
               "trajectory_rel_diff_median": float(np.median(traj[sel]))}
        for name, col in (("wn", fr), ("zeta", fr + 1), ("behaviour_err", s + 1)):
            row[f"{name}_compensated"] = float(np.median(rel(cmp_, col)[sel]))
            row[f"{name}_mixed"] = float(np.median(rel(mix, col)[sel]))
            e = rel(out["compensated_traj64"][0], col)[sel]
            row[f"{name}_compensated_on_fp64_trajectory"] = float(np.median(e))
            row[f"{name}_compensated_on_fp64_trajectory_within_1e-6"] = float((e <= 1e-6).mean())
            e = rel(dfr, col)[sel]
            row[f"{name}_compensated_df"] = float(np.median(e))
            row[f"{name}_compensated_df_within_1e-6"] = float((e <= 1e-6).mean())
        bins.append(row)
    # the same errors binned by the trajectory's own difference from the FP64 one
    tbins = []
    for lo in range(-9, 1):
        sel = scored & (traj >= 10.0 ** lo) & (traj < 10.0 ** (lo + 1))
        if sel.sum() < 4:
            continue
        row = {"trajectory_rel_diff": f"1e{lo}..1e{lo + 1}", "candidates": int(sel.sum())}
        for name, col in (("wn", fr), ("zeta", fr + 1), ("behaviour_err", s + 1)):
            e = rel(cmp_, col)[sel]
            row[f"{name}_compensated_median"] = float(np.median(e))
            row[f"{name}_compensated_within_1e-6"] = float((e <= 1e-6).mean())
        tbins.append(row)
    return {"sample": int(len(g)), "trajectory_rel_diff": {"median": float(np.median(traj)),
                                                            "p99": float(np.quantile(traj, 0.99))},
            "df_trajectory_rel_diff": {"median": float(np.median(traj_df)),
                                       "p99": float(np.quantile(traj_df, 0.99))},
            "compensated_df_vs_fp64": precision_report(dfr, f64, cfg),
            "by_condition": bins, "by_trajectory_difference": tbins,
            "compensated_on_fp64_trajectory_vs_fp64": t64}


def fit_ops(eigen, steps):
    """FP32 operations of the modal fit over one batch: for each stable candidate,
    per window step, the normal-equation FMAs nc(nc+1)/2 + nc and 5 operations per
    mode for the basis arguments and products (expf and sin/cos counted as 0).
    `eigen` is (n, nt, 2); a mode equal in (re, |im|) to its predecessor is a
    conjugate duplicate and does not enter the basis."""
    re, im = eigen[..., 0].astype(np.float64), eigen[..., 1].astype(np.float64)
    dup = np.zeros(re.shape, bool)
    dup[:, 1:] = (re[:, 1:] == re[:, :-1]) & (np.abs(im[:, 1:]) == np.abs(im[:, :-1]))
    unique = re.shape[1] - dup.sum(1)
    stable = modal_stable(eigen)
    nc = 2 * unique[stable]
    return float(steps * (nc * (nc + 1) // 2 + nc + 5 * unique[stable]).sum())


def modal_stable(eigen):
    """Candidates whose LIN_A eigenvalues all satisfy |lambda| <= 1 (the ones the fit
    models and the nominal closed loop is solved for)."""
    return np.hypot(eigen[..., 0].astype(np.float64), eigen[..., 1].astype(np.float64)).max(1) <= 1.0


def eig_ops(n):
    """Eigenvalues of a real n x n matrix by Householder-Hessenberg reduction and
    Francis double-shift QR: 10 n^3 flops (Golub and Van Loan, Matrix
    Computations, 4th ed., table 7.5.2), i.e. 5 n^3 fused multiply-adds -- counted
    here as FP64 pipe operations, the unit of the measured DFMA issue rate."""
    return 5 * n ** 3


def sim_ops_per_step(ns, nd, nw, n_instr):
    """FP32 operations of one simulation step (FMA, add and mul each count 1)."""
    dots = 4 * ns + 2                      # K.(hi,lo), C.(hi,lo), D u, u_raw
    observer = ns * (2 * ns + 2)           # (A-I)(hi,lo), B u, L yerr
    plant = nd * (2 * nd + nw + 1)         # (Ad-I)(hi,lo), Bw W, Bu u
    dfadd = 11 * (ns + nd)                 # double-float accumulation
    return dots + observer + plant + dfadd + 5 + n_instr


class ClockSampler:
    def __init__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms",
                                       "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self, gpu_index=0):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = []
        for line in Path(self.f.name).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9 and parts[0] == str(gpu_index):
                rows.append(parts)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def cpu_baseline(problem, seconds: float, threads: int):
    from oracle import oracle as O
    orc = O.Oracle(problem.config_text, problem.plant, threads=threads)
    n_total = problem.cuda_mx.shape[0]
    probe = min(64, n_total)
    t0 = time.perf_counter()
    orc.evaluate(problem.cuda_mx[:probe], problem.info_mx[:probe])
    rate = probe / max(time.perf_counter() - t0, 1e-6)
    n_s = int(min(n_total, max(probe, rate * seconds)))
    t0 = time.perf_counter()
    rows = orc.evaluate(problem.cuda_mx[:n_s], problem.info_mx[:n_s])
    dt = time.perf_counter() - t0
    return {"value": n_s / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n_s} of the {n_total} candidates, full horizon, oracle C port with OpenMP ({dt:.1f} s)"}, rows


def parity_report(gpu, ref, cfg):
    """The engine's rows against the oracle's (the reference method restated on the CPU, its own
    trajectories, eigenvalues and libm) on the same candidates: identity of the pass/fail classes
    (modal-unstable, nominal-unstable, eig-fail, margin status), the gain / phase margins in dB /
    deg, and the per-term difference of the scored candidates.  Fit-derived terms (wn, zeta,
    behaviour error) carry the FP32 normal equations' sensitivity to last-ulp libm differences."""
    s, am, fr = cfg.info_scoring, cfg.info_allmargin, cfg.info_freqresp
    def classes(x):
        return np.stack([x[:, s + 1] >= cfg.unstable_err, x[:, s + 2] == np.float32(cfg.unstable_err),
                         x[:, s + 2] == np.float32(cfg.eig_fail_err), x[:, am + 3] == 1.0], axis=1)
    cg, co = classes(gpu), classes(ref)
    same = (cg == co).all(axis=1)
    scored = same & (gpu[:, am + 3] == 1.0) & ~cg[:, 0]
    def stats(e):
        e = e[np.isfinite(e)]
        return {"median": float(np.median(e)), "p99": float(np.quantile(e, 0.99)), "max": float(e.max())} if e.size \
            else None
    g64, r64 = gpu.astype(np.float64), ref.astype(np.float64)
    absd = {"gm_db": stats(np.abs(g64[scored, am] - r64[scored, am])),
            "pm_deg": stats(np.abs(g64[scored, am + 1] - r64[scored, am + 1]))}
    terms = {"total_score": s, "behaviour_err": s + 1, "margin_err": s + 2, "wn": fr, "zeta": fr + 1,
             "overshoot": fr + 2, "yss": fr + 3, "gm_db": am, "pm_deg": am + 1, "dm_ms": am + 2, "b_pc": am + 4}
    rel = {k: stats(np.abs(g64[scored, c] - r64[scored, c]) / np.maximum(np.abs(r64[scored, c]), 1e-6))
           for k, c in terms.items()}
    return {"candidates": int(len(gpu)), "class_identity": float(same.mean()),
            "rows_bit_identical": float((gpu.view(np.uint32) == ref.view(np.uint32)).all(axis=1).mean()),
            "class_mismatches": int((~same).sum()), "scored_compared": int(scored.sum()),
            "margin_abs_diff": absd, "relative_diff": rel,
            "margins_within_1e-3": bool(all(v is None or v["max"] <= 1e-3 for v in absd.values()))}


def reference_gpu_build(problem, threads: int, sample: int = 4096):
    """The reference as it runs, in candidates/s: its own kernels (discrete_solve<Luenberger>,
    eigensetup, modalsetup from src/main.cu, compiled for sm_103a where the reference lies and
    launched with its launch shape and constant tables by oracle/ref_kernels.py) on the GPU over
    the whole batch, and its Eigen host stages (eigensolve, modalsolve, allmargin; Eigen itself
    is not vendored, so their C restatement in oracle/) on all host cores -- eigensolve and
    modalsolve over the whole batch, allmargin over `sample` candidates, scaled.  The trajectory
    stays on the device, as in the reference without dump_diagnostics."""
    from oracle import oracle as O, ref_kernels as RK
    if not RK.available():
        return {"unavailable": "oracle/_ref/ref_kernels.cubin not built (make -C oracle ref needs the reference tree)"}
    orc = O.Oracle(problem.config_text, problem.plant, threads=threads)
    cfg = orc.ref_config()
    g, info = problem.cuda_mx, problem.info_mx
    n = g.shape[0]
    zero = np.zeros((n, 2 * cfg.total_dim), np.float32)
    RK.run(cfg, problem.plant, g[:256], zero[:256], info[:256], want_y=False)  # module load
    _, lina, _, _, _ = RK.run(cfg, problem.plant, g, zero, info, want_y=False)
    t0 = time.perf_counter()
    eig = orc.eigensolve(lina)
    t_eig = time.perf_counter() - t0
    tm = {}
    _, _, ata, atb, info1 = RK.run(cfg, problem.plant, g, eig, info, want_y=False, times=tm)
    t0 = time.perf_counter()
    info2 = orc.modalsolve(ata, atb, eig, info1)
    t_ms = time.perf_counter() - t0
    m = min(n, sample)
    t0 = time.perf_counter()
    orc.allmargin(lina[:m], g[:m], info2[:m])
    t_am = (time.perf_counter() - t0) * n / m
    gpu_s = (tm["discrete_solve"] + tm["eigensetup"] + tm["modalsetup"]) * 1e-3
    copy_s = (tm["h2d"] + tm["d2h"]) * 1e-3
    total = gpu_s + copy_s + t_eig + t_ms + t_am
    return {"value": n / total, "unit": UNIT, "candidates": n, "cores": threads,
            "seconds": {"gpu_kernels": gpu_s, "copies": copy_s, "eigensolve_cpu": t_eig, "modalsolve_cpu": t_ms,
                        "allmargin_cpu": t_am},
            "gpu_kernels_ms": {k: tm[k] for k in ("discrete_solve", "eigensetup", "modalsetup")},
            "sample": f"GPU stages and eigensolve/modalsolve on all {n} candidates, allmargin on {m} (scaled)"}


def run_reference(a, rank, world):
    from controllerengine_gb300 import synth
    if rank != 0:
        return
    problem = synth.eight_state(**workload_args(a))
    threads = os.cpu_count() or 1
    from oracle import oracle as O
    orc = O.Oracle(problem.config_text, problem.plant, threads=threads)
    probe = 64
    t0 = time.perf_counter()
    orc.evaluate(problem.cuda_mx[:probe], problem.info_mx[:probe])
    rate = probe / max(time.perf_counter() - t0, 1e-6)
    n_s = int(min(problem.cuda_mx.shape[0], max(probe, rate * a.ref_step_seconds)))
    for _ in range(a.warmup):
        orc.evaluate(problem.cuda_mx[:min(n_s, 256)], problem.info_mx[:min(n_s, 256)])
    t0 = time.perf_counter()
    for k in range(a.steps):
        sl = slice((k * n_s) % (problem.cuda_mx.shape[0] - n_s + 1), None)
        g = problem.cuda_mx[sl][:n_s]
        orc.evaluate(g, problem.info_mx[sl][:g.shape[0]])
    dt = time.perf_counter() - t0
    value = n_s * a.steps / dt
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * dt / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (f64 eigensolve)", "data": "synthetic (seeded eight_state workload)", "impl": "reference",
            "config": {"workload": "eight_state: 65536 candidates, 8-state plant, 4 nonlinear terms, 10000 steps, "
                                   "400 sweep points; each step a bounded sample",
                       "candidates_per_step": n_s, "time": a.time, "freq": a.freq},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{n_s} candidates per step, full horizon; the reference's Eigen host "
                                       "path is not buildable here (Eigen not vendored), its method is timed "
                                       "through the C port in oracle/"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if a.ref_gpu_build:
        line["reference_gpu_build"] = reference_gpu_build(problem, threads)
    print(json.dumps(line), flush=True)


def serving_models(k: int = 16, seed: int = 5):
    """The serving mix: k plants drawn as in the uneven-shape workload (dimensions 2..8, 0-4
    nonlinear terms, 50-400 sweep points) with horizons log-uniform in [1e3, 1e4] steps, each
    with 16,384 candidate rows."""
    from controllerengine_gb300 import synth
    rng = np.random.default_rng(seed)
    out = []
    for m in range(k):
        T = int(np.exp(rng.uniform(np.log(1e3), np.log(1e4))))
        out.append(synth.random_shape(1000 + m, n=16384, time=T, freq=int(rng.integers(50, 401))))
    return out


def serving_bench(problems, seconds: float, lanes: int = 3, max_batch: int = 16384, seed: int = 7,
                  precision: str = "mixed", n_plants: int = 16384, mc_fraction: float = 0.25,
                  max_wait_us: int = 0, max_batch_work: int = 0, runs: int = 1):
    """Request serving (ce_server_*): every model of `problems` holds n_plants perturbed copies
    of its plant (synth.perturbed_plants); a request carries U[256, 16384] candidates on a model
    drawn uniformly -- with probability mc_fraction a Monte Carlo request (one gain set on as
    many consecutive plants, ce_server_submit_plants), else a tuning request (distinct gain
    sets on one plant).  Saturation: 256 requests submitted at once, candidates/s until all are
    done.  Latency: Poisson arrivals at 70% of that rate for `seconds`, then at 50 requests/s
    (light load, when below that) for half as long; p50/p99 of submit ->
    results in the caller's buffer (measured by the server).  The loaded runs draw their requests
    and arrival times beforehand and keep Python's garbage collector off, so the generator itself
    adds no bursts."""
    import controllerengine_gb300 as ce
    from controllerengine_gb300 import synth
    rng = np.random.default_rng(seed)
    cfgs = [ce.EngineConfig.parse(p.config_text) for p in problems]
    plant_sets = [synth.perturbed_plants(p.plant, n_plants, 200 + k) for k, p in enumerate(problems)]
    mc_rows = [(np.repeat(p.cuda_mx[:1], 16384, axis=0), np.repeat(p.info_mx[:1], 16384, axis=0)) for p in problems]

    def draw():
        k = int(rng.integers(0, len(problems)))
        p = problems[k]
        m = int(rng.integers(256, 16385))
        if rng.random() < mc_fraction:
            first = int(rng.integers(0, n_plants - m + 1))
            return k, True, first, mc_rows[k][0][:m], mc_rows[k][1][:m]
        a = int(rng.integers(0, p.cuda_mx.shape[0] - m + 1))
        return k, False, int(rng.integers(0, n_plants)), p.cuda_mx[a:a + m], p.info_mx[a:a + m]

    def submit(srv, req, out=None):
        k, mc, plant, g, i = req
        if mc:
            return srv.submit_plants(g, i, first_plant=plant, model=k, out=out)
        return srv.submit(g, i, plant_index=plant, model=k, out=out)

    def draw_submit(srv):
        # a request naming a plant whose sweep grid failed is refused at submit: draw again
        for _ in range(100):
            req = draw()
            try:
                return req, submit(srv, req)
            except ce.ControllerEngineError:
                refused[0] += 1
        raise RuntimeError("no servable request in 100 draws")

    refused = [0]
    models = [(c, ps, n_plants) for c, ps in zip(cfgs, plant_sets)]
    with ce.Server(None, None, models=models, max_batch=max_batch, lanes=lanes, precision=precision,
                   max_wait_us=max_wait_us, max_batch_work=max_batch_work) as srv:
        # warm-up: every lane sizes its scratch for a full batch of every model, and compiles
        # the per-candidate-plant kernels of every model
        for _ in range(lanes):
            hs = []
            for k, p in enumerate(problems):
                hs.append(srv.submit(p.cuda_mx[:max_batch], p.info_mx[:max_batch], model=k))
                for first in (0, n_plants // 2):
                    try:
                        hs.append(srv.submit_plants(mc_rows[k][0][:4096], mc_rows[k][1][:4096], first_plant=first,
                                                    model=k))
                    except ce.ControllerEngineError:
                        pass
            for h in hs:
                h.wait()
        refused[0] = 0
        reqs = [draw() for _ in range(256)]
        total = sum(r[3].shape[0] for r in reqs)
        t0 = time.perf_counter()
        hs = []
        for r in reqs:
            try:
                hs.append(submit(srv, r))
            except ce.ControllerEngineError:
                total -= r[3].shape[0]
                refused[0] += 1
        for h in hs:
            h.wait()
        sat = total / (time.perf_counter() - t0)
        mean_size = (256 + 16384) / 2
        rate = 0.7 * sat / mean_size  # requests/s
        # consecutive loaded runs; the line's main figures are the last run's, every run's are listed
        per_run = []
        import gc
        for _ in range(max(1, runs)):
            arrivals = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * seconds * 1.5) + 16))
            arrivals = arrivals[arrivals < seconds]
            plan = [draw() for _ in range(len(arrivals))]
            # the result buffers, allocated and touched before the run (a serving client reuses
            # its buffers; fresh ones would fault their pages in during the result copy)
            outs = [np.zeros_like(req[4]) for req in plan]
            srv.reset_stats()
            hs, offered, n_mc = [], 0, 0
            gc.disable()
            try:
                t0 = time.perf_counter()
                for t_at, req, out in zip(arrivals, plan, outs):
                    now = time.perf_counter() - t0
                    if now < t_at:
                        time.sleep(t_at - now)
                    try:
                        h = submit(srv, req, out)
                    except ce.ControllerEngineError:
                        refused[0] += 1  # a plant whose sweep grid failed: refused at submit
                        continue
                    offered += req[3].shape[0]
                    n_mc += req[1]
                    hs.append(h)
                for h in hs:
                    h.wait()
                wall = time.perf_counter() - t0
            finally:
                gc.enable()
            st = srv.stats()
            per_run.append({"requests": st["completed"], "latency_p50_ms": st["latency_p50_ms"],
                            "latency_p99_ms": st["latency_p99_ms"], "latency_max_ms": st["latency_max_ms"],
                            "queue_p99_ms": st["queue_p99_ms"], "service_p99_ms": st["service_p99_ms"],
                            "batch_p99_ms": st["batch_p99_ms"], "tail_queue_ms": st["tail_queue_ms"],
                            "tail_service_ms": st["tail_service_ms"], "tail_busy_lanes": st["tail_busy_lanes"]})
        # light load: 50 requests/s, the low end of the serving configuration's arrival rates
        # (when that is below 70% of saturation), where a request is mostly served alone
        light = None
        if 50.0 < rate:
            srv.reset_stats()
            hs = []
            t0 = time.perf_counter()
            t_next = t0
            while t_next - t0 < max(3.0, seconds / 2):
                now = time.perf_counter()
                if now < t_next:
                    time.sleep(t_next - now)
                hs.append(draw_submit(srv)[1])
                t_next += rng.exponential(1.0 / 50.0)
            for h in hs:
                h.wait()
            sl = srv.stats()
            light = {"offered_requests_per_s": 50.0, "requests": sl["completed"],
                     "mean_batch": sl["batched_candidates"] / max(1, sl["batches"]),
                     "latency_p50_ms": sl["latency_p50_ms"], "latency_p99_ms": sl["latency_p99_ms"],
                     "latency_max_ms": sl["latency_max_ms"]}
    shapes = sorted({(c.statespace_dim, c.discrete_dim, c.time, c.freq) for c in cfgs})
    return {"request_mix": f"U[256, 16384] candidates on one of {len(problems)} models of the uneven-shape "
                           f"workload (dims 2..8, horizons 1e3..1e4, 50..400 sweep points), each with {n_plants} "
                           f"perturbed plants; {mc_fraction:.0%} Monte Carlo requests (one gain set on as many "
                           "consecutive plants), the rest tuning requests (distinct gain sets on one plant)",
            "precision": precision,
            "models": [list(x) for x in shapes],
            "lanes": lanes, "max_batch": st["capacity"], "max_wait_us": max_wait_us,
            "max_batch_work": max_batch_work, "loaded_runs": per_run,
            "p99_all_runs_ms": max(r["latency_p99_ms"] for r in per_run),
            "saturation_candidates_per_s": sat,
            "offered_requests_per_s": rate, "offered_load": "70% of saturation, Poisson arrivals",
            "requests": st["completed"], "monte_carlo_requests": n_mc, "refused_requests": refused[0],
            "achieved_candidates_per_s": offered / wall,
            "batches": st["batches"], "mean_batch": st["batched_candidates"] / max(1, st["batches"]),
            "latency_p50_ms": st["latency_p50_ms"], "latency_p99_ms": st["latency_p99_ms"],
            "latency_max_ms": st["latency_max_ms"],
            "breakdown": {k: st[k] for k in ("queue_p50_ms", "queue_p99_ms", "service_p50_ms", "service_p99_ms",
                                             "batch_p50_ms", "batch_p99_ms", "batch_max_ms", "tail_requests",
                                             "tail_queue_ms", "tail_service_ms", "tail_busy_lanes")},
            "light_load": light}


def monte_carlo_bench(n_plants: int, steps: int, warmup: int):
    """Monte Carlo over plants (one plant per candidate, serial-mode margins): candidates/s of
    ce_evaluate_plants_device over n_plants plants, inputs resident, CUDA events."""
    import torch
    import controllerengine_gb300 as ce
    from controllerengine_gb300 import synth
    t0 = time.perf_counter()
    p = synth.monte_carlo(n_plants=n_plants)
    cfg = ce.EngineConfig.parse(p.config_text)
    sess = ce.Session(cfg, p.plant, n_plants=n_plants)
    setup = time.perf_counter() - t0
    dev = torch.device("cuda", torch.cuda.current_device())
    g = torch.from_numpy(p.cuda_mx).to(dev)
    info = torch.from_numpy(p.info_mx).to(dev)
    out = torch.empty_like(info)
    st = torch.cuda.current_stream(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for _ in range(warmup):
        sess.evaluate_plants_device(n_plants, g.data_ptr(), info.data_ptr(), out.data_ptr(), stream=st.cuda_stream)
    torch.cuda.synchronize()
    ms = 0.0
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        sess.evaluate_plants_device(n_plants, g.data_ptr(), info.data_ptr(), out.data_ptr(), stream=st.cuda_stream)
        e1.record(st)
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
    o = out.cpu().numpy()
    sess.close()
    sc = o[:, cfg.info_scoring]
    return {"workload": f"{n_plants} plants: eight-state A, B_u x (1 + 0.1 N(0,1)), BASE_PARAMS x U[0.8, 1.2], "
                        f"one gain set, T = {cfg.time}, F = {cfg.freq}, serial-mode margins",
            "candidates_per_s": n_plants * steps / (ms * 1e-3), "ms_per_step": ms / steps, "steps": steps,
            "session_setup_s": setup, "scored_fraction": float(np.mean(sc < cfg.unstable_err))}


def uneven_bench(n_inst: int, steps: int, warmup: int, sample: int = 24):
    """The uneven-size workload (synth.uneven: n_inst instances of one candidate each, dimensions
    2..8, 0-4 nonlinear terms with their own instruction programs, horizons 1e3..2e4 steps,
    50..400 sweep points): instances/s of one ragged batch (ce_ragged_evaluate, host buffers, every
    stage one launch over all instances), beside (a) the same instances evaluated one session each
    (a sample of them, sessions created beforehand), (b) padded to max: the same instances with
    every horizon and sweep raised to the largest (20,000 steps, 400 points), and (c) n_inst
    candidates of one 8-state plant at that size in one session."""
    import controllerengine_gb300 as ce
    from controllerengine_gb300 import synth
    t0 = time.perf_counter()
    probs = synth.uneven(n_inst)
    cfgs = [ce.EngineConfig.parse(p.config_text) for p in probs]
    rb = ce.Ragged([(c, p.plant) for c, p in zip(cfgs, probs)])
    setup = time.perf_counter() - t0
    # the C ABI's packed rows (instance after instance at each instance's widths)
    counts = [p.cuda_mx.shape[0] for p in probs]
    g_all = np.concatenate([p.cuda_mx.reshape(-1) for p in probs])
    i_all = np.concatenate([p.info_mx.reshape(-1) for p in probs])
    for _ in range(warmup):
        rb.evaluate_packed(counts, g_all, i_all)
    l0 = rb.kernel_launches
    rb.set_profiling(True)
    t0 = time.perf_counter()
    for _ in range(steps):
        out = rb.evaluate_packed(counts, g_all, i_all)
    wall = (time.perf_counter() - t0) / steps
    stages = {k: v[0] / steps for k, v in rb.stage_times().items() if v[1]}
    launches = (rb.kernel_launches - l0) // steps
    rb.set_profiling(False)
    # the device path: rows resident, the autotuner's setting, one evaluation captured into a CUDA
    # graph and replayed (CUDA events on the replay stream)
    import torch
    dg = torch.from_numpy(g_all).cuda()
    di = torch.from_numpy(i_all).cuda()
    do = torch.empty_like(di)
    rb.prepare(counts)
    tuned = rb.autotune(dg.data_ptr(), di.data_ptr(), do.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        rb.evaluate_device(dg.data_ptr(), di.data_ptr(), do.data_ptr(), stream=side.cuda_stream)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        rb.evaluate_device(dg.data_ptr(), di.data_ptr(), do.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
    for _ in range(warmup):
        graph.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        graph.replay()
    e1.record()
    torch.cuda.synchronize()
    graph_ms = e0.elapsed_time(e1) / steps
    same = bool(np.array_equal(do.cpu().numpy().view(np.uint32), out.view(np.uint32)))
    del graph
    rb.close()
    offs = np.cumsum([0] + [c.info_mx_width for c in cfgs])
    scored = float(np.mean([out[offs[k] + c.info_scoring] < c.unstable_err for k, c in enumerate(cfgs)]))
    # (a) one session per instance, on a sample (table-driven simulation: no compile per instance)
    rng = np.random.default_rng(3)
    pick = rng.choice(n_inst, size=min(sample, n_inst), replace=False)
    prev = os.environ.get("CE_SIM_KERNEL")
    os.environ["CE_SIM_KERNEL"] = "table"
    try:
        sess = [ce.Session(cfgs[k], probs[k].plant) for k in pick]
    finally:
        if prev is None:
            os.environ.pop("CE_SIM_KERNEL")
        else:
            os.environ["CE_SIM_KERNEL"] = prev
    for s_, k in zip(sess, pick):
        s_.evaluate(probs[k].cuda_mx, probs[k].info_mx)
    t0 = time.perf_counter()
    for s_, k in zip(sess, pick):
        s_.evaluate(probs[k].cuda_mx, probs[k].info_mx)
    per_inst = (time.perf_counter() - t0) / len(pick)
    for s_ in sess:
        s_.close()
    # (b) padded to max: the same instances (their own plants and programs) with the simulation at
    # the padded 8/8 width, every horizon raised to the largest, 20,000 steps at the instance's own
    # step size, and every sweep to 400 points, through the same ragged path
    import re

    def pad(p, c):
        t = re.sub(r"(?m)^time = .*$", "time = 20000", p.config_text)
        t = re.sub(r"(?m)^duration = .*$", f"duration = {20000 * float(c.ts)!r}", t)
        return re.sub(r"(?m)^freq = .*$", "freq = 400", t)

    pcfgs = [ce.EngineConfig.parse(pad(p, c)) for p, c in zip(probs, cfgs)]
    assert all(c.time == 20000 and c.freq == 400 for c in pcfgs)
    with ce.Ragged([(c, p.plant) for c, p in zip(pcfgs, probs)]) as rp:
        rp.set_tuning(sim_width=8)  # every candidate at the padded 8/8 width, as the reference pads
        for _ in range(warmup):
            rp.evaluate_packed(counts, g_all, i_all)
        t0 = time.perf_counter()
        for _ in range(steps):
            rp.evaluate_packed(counts, g_all, i_all)
        padded = (time.perf_counter() - t0) / steps
    # (c) one uniform plant at the largest shape (8-state, 4 NL terms, 20,000 steps, 400 points):
    # another problem, run by one compiled program with no interpretation
    pm = synth.eight_state(n=n_inst, time=20000, freq=400)
    pc = ce.EngineConfig.parse(pm.config_text)
    with ce.Session(pc, pm.plant) as s_:
        for _ in range(warmup):
            s_.evaluate(pm.cuda_mx, pm.info_mx)
        t0 = time.perf_counter()
        for _ in range(steps):
            s_.evaluate(pm.cuda_mx, pm.info_mx)
        uniform = (time.perf_counter() - t0) / steps
    shapes = {(c.statespace_dim, c.discrete_dim, c.nonlin_dim) for c in cfgs}
    return {"workload": f"{n_inst} instances x 1 candidate: dims 2..8 ({len(shapes)} distinct (ns, nd, nw)), "
                        "0-4 NL terms, horizons 1e3..2e4, 50..400 sweep points",
            "instances_per_s": n_inst / wall, "ms_per_step": 1e3 * wall, "steps": steps,
            "launches_per_step": launches, "stages_ms_per_step": stages, "setup_s": setup,
            "scored_fraction": scored,
            "graph": {"instances_per_s": n_inst / (graph_ms * 1e-3), "ms_per_step": graph_ms, "tuning": tuned,
                      "rows_equal_host_path": same,
                      "what": "ce_ragged_evaluate_device captured in one CUDA graph (gather, one launch per "
                              "stage, scatter), device-resident rows, the ragged autotuner's setting"},
            "one_session_per_instance": {"instances_per_s": 1.0 / per_inst, "ms_per_instance": 1e3 * per_inst,
                                         "sample": len(pick)},
            "padded_to_max": {"instances_per_s": n_inst / padded, "ms_per_step": 1e3 * padded,
                              "padding": "the same instances, every horizon 20000 steps and every sweep 400 "
                                         "points, the simulation at the padded 8/8 width (ce_ragged_tuning.sim_width = 8)"},
            "uniform_max_plant": {"instances_per_s": n_inst / uniform, "ms_per_step": 1e3 * uniform,
                                  "shape": "one 8-state, 4 NL-term plant and program for every candidate, "
                                           "20000 steps, 400 points (a different problem)"},
            "timing": "wall clock around the synchronous host-buffer call ce_ragged_evaluate (packing to the "
                      "device layout, copies and kernels)"}


def small_bench(steps: int, warmup: int, cpu: bool):
    """The small mass-spring case (1,024 candidates, 3-state observer, 2,000 steps, 200 sweep
    points: the reference's CPU-runnable configuration): candidates/s of the mixed and the FP64
    form (ce_evaluate_device, inputs resident, CUDA events) and of the oracle port on all host
    cores (bounded sample)."""
    import torch
    import controllerengine_gb300 as ce
    from controllerengine_gb300 import synth
    p = synth.mass_spring(1024)
    cfg = ce.EngineConfig.parse(p.config_text)
    dev = torch.device("cuda", torch.cuda.current_device())
    g = torch.from_numpy(p.cuda_mx).to(dev)
    info = torch.from_numpy(p.info_mx).to(dev)
    out = torch.empty_like(info)
    st = torch.cuda.current_stream(dev)
    res = {"workload": "mass_spring: 1024 candidates, 2-state plant + cubic spring, 3-state observer, "
                       "T = 2000, F = 200"}
    for prec in ("mixed", "fp64"):
        with ce.Session(cfg, p.plant, precision=prec) as s_:
            for _ in range(warmup):
                s_.evaluate_device(1024, g.data_ptr(), info.data_ptr(), out.data_ptr(), stream=st.cuda_stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(st)
            for _ in range(steps):
                s_.evaluate_device(1024, g.data_ptr(), info.data_ptr(), out.data_ptr(), stream=st.cuda_stream)
            e1.record(st)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / steps
        res[prec] = {"candidates_per_s": 1024 / (ms * 1e-3), "ms_per_step": ms}
    if cpu:
        res["cpu_baseline"] = cpu_baseline(p, 5.0, os.cpu_count() or 1)[0]
    return res


def _kalman_time(p, n: int, steps: int, warmup: int, autotune: bool = True):
    import torch
    import controllerengine_gb300 as ce
    cfg = ce.EngineConfig.parse(p.config_text)
    sess = ce.Session(cfg, p.plant)
    dev = torch.device("cuda", torch.cuda.current_device())
    g = torch.from_numpy(p.cuda_mx).to(dev)
    info = torch.from_numpy(p.info_mx).to(dev)
    out = torch.empty_like(info)
    st = torch.cuda.current_stream(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    # the session autotuner picks the launch settings on this batch, as for the headline (untimed)
    tuning = (sess.autotune(n, g.data_ptr(), info.data_ptr(), out.data_ptr(), stream=st.cuda_stream) if autotune
              else None)
    for _ in range(warmup):
        sess.evaluate_device(n, g.data_ptr(), info.data_ptr(), out.data_ptr(), stream=st.cuda_stream)
    torch.cuda.synchronize()
    ms = 0.0
    sess.set_profiling(True)
    l0 = sess.kernel_launches
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        sess.evaluate_device(n, g.data_ptr(), info.data_ptr(), out.data_ptr(), stream=st.cuda_stream)
        e1.record(st)
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
    launches = (sess.kernel_launches - l0) // steps
    stages = {k: v[0] / steps for k, v in sess.stage_times().items() if v[1]}
    sess.close()
    keys, counts = np.unique(p.cuda_mx[:, 2 * cfg.statespace_dim + 1:], axis=0, return_counts=True)
    return {"candidates_per_s": n * steps / (ms * 1e-3), "ms_per_step": ms / steps, "steps": steps,
            "launches_per_step": launches, "stages_ms_per_step": stages, "noise_weight_sets": len(keys),
            "shared_noise_fraction": float(counts[counts >= 8].sum() / n), "tuning": tuning}


def kalman_bench(n: int, steps: int, warmup: int, cpu_seconds: float, autotune: bool = True):
    """The eight-state workload with the time-varying Kalman observer (rows [K, L, N, R, Q]):
    candidates/s of ce_evaluate_device at the session autotuner's launch settings (chosen untimed
    on the batch, as for the headline), inputs resident, CUDA events, L2 flushed between steps,
    with the simulation stage's share.  Twice: noise weights from the 64-set pool the gains were
    designed with (candidates share covariance recursions: the shared-noise form), and with R
    perturbed per candidate by a factor 1 + U[0, 1e-3] (every recursion distinct: the
    per-candidate form).  The oracle port on the host cores on a bounded sample beside it."""
    from controllerengine_gb300 import synth
    p = synth.eight_state(n=n, observer="kalman")
    res = {"workload": f"eight_state with observer = kalman: {n} candidates, T = 10000, F = 400",
           "pooled_noise": _kalman_time(p, n, steps, warmup, autotune)}
    q = synth.Problem(p.name, p.config_text, p.plant, p.cuda_mx.copy(), p.info_mx)
    rng = np.random.default_rng(17)
    q.cuda_mx[:, 17] *= (1.0 + 1e-3 * rng.random(n)).astype(np.float32)
    res["distinct_noise"] = _kalman_time(q, n, max(1, steps - 1), 1, autotune)
    res["candidates_per_s"] = res["pooled_noise"]["candidates_per_s"]
    if cpu_seconds > 0:
        res["cpu_baseline"] = cpu_baseline(p, cpu_seconds, os.cpu_count() or 1)[0]
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--candidates", type=int, default=65536)
    ap.add_argument("--time", type=int, default=10000)
    ap.add_argument("--freq", type=int, default=400)
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-step-seconds", type=float, default=8.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--sim-kernel", default="specialised", choices=["specialised", "table"])
    ap.add_argument("--no-autotune", action="store_true", help="keep the library's default launch settings")
    ap.add_argument("--serve-seconds", type=float, default=10.0, help="Poisson serving run (0: skip)")
    ap.add_argument("--serve-runs", type=int, default=5, help="consecutive loaded serving runs")
    ap.add_argument("--serve-lanes", type=int, default=3)
    ap.add_argument("--serve-max-work", type=int, default=0,
                    help="serving: candidate-steps per batch (0: no cap)")
    ap.add_argument("--serve-max-wait-us", type=int, default=0,
                    help="serving: how long a partial batch may wait for more requests")
    ap.add_argument("--mc-plants", type=int, default=262144, help="Monte Carlo plants, one per candidate (0: skip)")
    ap.add_argument("--ref-gpu-build", type=int, default=1,
                    help="reference arm: also time the reference's own kernels + host stages (0: skip)")
    ap.add_argument("--kalman-candidates", type=int, default=65536, help="Kalman-observer workload (0: skip)")
    ap.add_argument("--uneven-instances", type=int, default=16384, help="uneven-size ragged batch (0: skip)")
    ap.add_argument("--small-steps", type=int, default=10, help="the small mass-spring case (0: skip)")
    ap.add_argument("--floor-sample", type=int, default=4096,
                    help="candidates of the precision-floor analysis (trajectory difference, conditioning; 0: skip)")
    ap.add_argument("--eig-compare", type=int, default=1,
                    help="also run the other eigensolve arithmetic on the batch and compare rows (0: skip)")
    a = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if a.impl == "reference":
        run_reference(a, rank, world)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from controllerengine_gb300 import build, synth
    build.build()
    import controllerengine_gb300 as ce
    from controllerengine_gb300.engine import measure_fma_rate

    problem = synth.eight_state(seed=2 + rank, **workload_args(a))  # each rank its own candidates (weak scaling)
    n = problem.cuda_mx.shape[0]
    cfg = ce.EngineConfig.parse(problem.config_text)
    sess = ce.Session(cfg, problem.plant)
    if sess.sim_kernel != a.sim_kernel:
        sess.set_sim_kernel(a.sim_kernel)  # raises with the compiler's log if specialising fails

    dev = torch.device("cuda", local)
    g = torch.from_numpy(problem.cuda_mx).to(dev)
    info_in = torch.from_numpy(problem.info_mx).to(dev)
    info_out = torch.empty_like(info_in)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2 (129 MB)

    def step():
        sess.evaluate_device(n, g.data_ptr(), info_in.data_ptr(), info_out.data_ptr(), stream=stream.cuda_stream)

    # the session autotuner picks the launch settings on this batch (untimed; results do not depend on them)
    if a.no_autotune:
        tuning = sess.tuning
    else:
        tuning = sess.autotune(n, g.data_ptr(), info_in.data_ptr(), info_out.data_ptr(), stream=stream.cuda_stream)
    # eigenvalues of every candidate (untimed): the fit's work depends on the mode count
    _, diag = sess.evaluate_diagnostics(problem.cuda_mx, problem.info_mx, want=("eigen",))
    eig_all = diag["eigen"].reshape(n, cfg.total_dim, 2)
    fit_work = fit_ops(eig_all, cfg.fit_steps)
    n_listed = int(modal_stable(eig_all).sum())
    del diag, eig_all

    for _ in range(a.warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize()

    # ---- device-resident timed region ----
    sess.set_profiling(True)
    l0 = sess.kernel_launches
    clocks = ClockSampler()
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    t_wall = time.perf_counter()
    for k in range(a.steps):
        flush.zero_()  # L2 flush between timed iterations, outside the events
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    wall = time.perf_counter() - t_wall
    clk = clocks.stop(local)
    launches = sess.kernel_launches - l0
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev)
    stages = sess.stage_times()
    sess.set_profiling(False)
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / a.steps
    value = world * n * a.steps / (ms * 1e-3)
    value_rows = info_out.cpu().numpy()  # the rows of the timed steps (identical in every step)

    # ---- e2e through the C ABI with pinned host buffers ----
    pin_g = torch.from_numpy(problem.cuda_mx).pin_memory().numpy()
    pin_i = torch.from_numpy(problem.info_mx).pin_memory().numpy()
    pin_o = torch.empty(problem.info_mx.shape, dtype=torch.float32).pin_memory().numpy()
    lib = ce.load_library()
    import ctypes as C
    from controllerengine_gb300 import _ffi
    fp = lambda arr: arr.ctypes.data_as(_ffi._FP)
    lib.ce_evaluate(sess._h, 0, n, fp(pin_g), fp(pin_i), fp(pin_o))  # warm
    e2e_steps = a.steps  # the same step count as the device-resident value
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        rc = lib.ce_evaluate(sess._h, 0, n, fp(pin_g), fp(pin_i), fp(pin_o))
        assert rc == 0, _ffi.last_error(lib)
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * n * e2e_steps / e2e_s
    h2d = n * (cfg.cuda_mx_width + cfg.info_mx_width) * 4
    d2h = n * cfg.info_mx_width * 4

    # ---- FP64 form ----
    fp64 = None
    if a.fp64_steps > 0:
        mixed_rows = info_out.cpu().numpy()
        sess.set_precision("fp64")
        step()
        torch.cuda.synchronize()
        fp64_rows = info_out.cpu().numpy()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(a.fp64_steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        f_ms = e0.elapsed_time(e1) / a.fp64_steps
        fp64 = {"value": world * n / (f_ms * 1e-3), "unit": UNIT, "ms_per_step": f_ms,
                "speedup_of_mixed": (world * n / (ms_per_step * 1e-3)) / (world * n / (f_ms * 1e-3)),
                "mixed_vs_fp64": precision_report(mixed_rows, fp64_rows, cfg)}
        # the compensated form on the same batch, against the same FP64 rows
        sess.set_precision("compensated")
        step()
        torch.cuda.synchronize()
        comp_rows = info_out.cpu().numpy()
        sess.set_profiling(True)
        e0.record(stream)
        for _ in range(a.fp64_steps + 1):
            flush.zero_()
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        c_stages = {k: v[0] / (a.fp64_steps + 1) for k, v in sess.stage_times().items()}
        sess.set_profiling(False)
        c_ms = e0.elapsed_time(e1) / (a.fp64_steps + 1)
        fp64["compensated"] = {"value": world * n / (c_ms * 1e-3), "unit": UNIT, "ms_per_step": c_ms,
                               "speedup_of_fp64_form": f_ms / c_ms, "stages_ms_per_step": c_stages,
                               "compensated_vs_fp64": precision_report(comp_rows, fp64_rows, cfg)}
        # the compensated form with the double-float simulation, on the same batch
        sess.set_precision("compensated_df")
        step()
        torch.cuda.synchronize()
        df_rows = info_out.cpu().numpy()
        sess.set_profiling(True)
        e0.record(stream)
        for _ in range(a.fp64_steps + 1):
            flush.zero_()
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        d_stages = {k: v[0] / (a.fp64_steps + 1) for k, v in sess.stage_times().items()}
        sess.set_profiling(False)
        d_ms = e0.elapsed_time(e1) / (a.fp64_steps + 1)
        fp64["compensated_df"] = {"value": world * n / (d_ms * 1e-3), "unit": UNIT, "ms_per_step": d_ms,
                                  "speedup_of_fp64_form": f_ms / d_ms, "stages_ms_per_step": d_stages,
                                  "compensated_df_vs_fp64": precision_report(df_rows, fp64_rows, cfg),
                                  "what": "the compensated form with the simulation in double-float arithmetic "
                                          "(pairs of FP32 values) instead of FP32"}
        sess.set_precision("mixed")
        if a.floor_sample > 0:
            fp64["precision_floor"] = precision_floor(sess, problem, cfg, a.floor_sample)

    # ---- eigensolve arithmetic: the separate (reference) form on the same batch ----
    eig_cmp = None
    if a.eig_compare:
        arith0 = sess.eig_arith
        other = "separate" if arith0 == "fused" else "fused"
        sess.set_eig_arith(other)
        for _ in range(2):
            flush.zero_()
            step()
        torch.cuda.synchronize()
        o_rows = info_out.cpu().numpy()
        sess.set_profiling(True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(2):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        o_stages = {k: v[0] / 2 for k, v in sess.stage_times().items()}
        sess.set_profiling(False)
        sess.set_eig_arith(arith0)
        rep = parity_report(value_rows, o_rows, cfg)
        other_rows = o_rows
        eig_cmp = {"default": arith0, "other": other, "other_ms_per_step": e0.elapsed_time(e1) / 2,
                   "other_stages_ms_per_step": o_stages,
                   "rows_bit_identical": float((value_rows.view(np.uint32) == o_rows.view(np.uint32)).all(axis=1).mean()),
                   "class_identity": rep["class_identity"], "margin_abs_diff": rep["margin_abs_diff"]}

    # ---- roofline of the dominant kernel ----
    per_launch = {k: (v[0] / v[1] if v[1] else 0.0) for k, v in stages.items()}
    # a large batch runs each stage as several chunk launches: per step = sum over its chunks
    per_step = {k: v[0] / a.steps for k, v in stages.items()}
    dom = max(per_step, key=per_step.get)
    fp32_rate = measure_fma_rate(False)
    fp64_rate = measure_fma_rate(True)
    n_instr = 1 + 1 + 10  # DC, U and the NL instructions of this workload
    peak = fp32_rate / 1e12
    src = "measured FP32 FFMA issue rate (ce_measure_fma_rate), not in MEASURED_PEAKS"
    sim_name = "ce_sim_specialised (8,8)" if sess.sim_kernel == "specialised" else "k_sim_mixed<8,8>"
    work = {"sim": (sim_name, sim_ops_per_step(8, 8, 4, n_instr) * a.time * n,
                    f"{sim_ops_per_step(8, 8, 4, n_instr)} FP32 ops/step x {a.time} steps x {n} candidates"),
            "fit": ("k_fit<float>", fit_work,
                    f"normal-equation FMAs + 5 basis ops per mode-step, {cfg.fit_steps} window steps, "
                    f"summed over the stable candidates ({fit_work / 1e9:.2f} G ops)")}
    nt, n2 = cfg.total_dim, 2 * cfg.statespace_dim
    work64 = {"lina_eig": ("k_lina_eig<2>", eig_ops(nt) * n,
                           f"5 n^3 FP64 FMAs (10 n^3 flops) of a {nt}x{nt} real eigensolve x {n} candidates"),
              "nominal": ("k_nominal<2>", eig_ops(n2) * n_listed,
                          f"5 n^3 FP64 FMAs (10 n^3 flops) of a {n2}x{n2} real eigensolve x {n_listed} "
                          "listed candidates")}
    src64 = "measured FP64 DFMA issue rate (ce_measure_fma_rate), not in MEASURED_PEAKS"
    # DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of each stage's launch over one
    # 16,384-candidate chunk of this workload, from ncu captures (summaries in the profiles
    # directory); scaled to this step's candidates in proportion.  Writes still resident in L2
    # when a kernel ends are not counted (the fit window: 459 MB written per chunk, 404 MB seen).
    dram_mb_16k = {"sim": 2.33 + 403.96, "fit": 358.21 + 84.60, "lina_eig": 1.29 + 0.03, "nominal": 7.62,
                   "sweep": 7.57 + 0.66}
    rooflines = {}
    for group, bound, pk, sname in ((work, "fp32", peak, src), (work64, "fp64", fp64_rate / 1e12, src64)):
        for st, (kname, ops, desc) in group.items():
            ach = ops / (per_step[st] * 1e-3) / 1e12 if per_step.get(st) else None
            rooflines[st] = {"kernel": kname, "bound": bound, "achieved": ach, "peak": pk, "unit": "Tops/s",
                             "frac": ach / pk if ach else None,
                             "traffic": dram_mb_16k[st] * 1e6 * n / 16384 if st in dram_mb_16k else None,
                             "traffic_unit": "bytes per step (ncu capture of a 16,384-candidate launch, scaled)",
                             "work_per_launch": desc, "peak_source": sname}
            if bound == "fp64" and ach:
                # the reference's Eigen stages run unfused (separate multiply and add), so a
                # bit-exact restatement issues two FP64 instructions per multiply-add
                rooflines[st]["frac_of_unfused_ceiling"] = ach / (pk / 2)
    roof = rooflines.get(dom) or {"kernel": dom, "bound": "fp32", "achieved": None, "peak": None, "unit": "Tops/s",
                                  "frac": None, "traffic": None}
    peaks_file = ROOT / "MEASURED_PEAKS.json"
    hbm_peak = json.loads(peaks_file.read_text())["hbm_gbs"] if peaks_file.exists() else 6800.0
    win_bytes = n * cfg.fit_steps * 4 * 2  # fit window written by k_sim and read by k_fit
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (f64 eigensolve)", "data": "synthetic (seeded eight_state workload, random-draw plant)",
        "config": {"workload": "eight_state: 65536 candidates, 8-state plant, 4 nonlinear terms, 10000 steps, "
                               "400 sweep points", "candidates_per_gpu": n, "time": a.time, "freq": a.freq,
                   "l2": "256 MB buffer written between timed steps (outside the events)",
                   "sim_kernel": sess.sim_kernel, "tuning": tuning},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "roofline": roof,
        "rooflines_by_stage": rooflines,
        "stages_ms_per_step": per_step,
        "stages_ms_per_launch": per_launch,
        "fit_window_hbm": {"bytes_per_step": win_bytes, "gbs_if_overlapped": win_bytes / (ms_per_step * 1e-3) / 1e9,
                           "peak_gbs": hbm_peak},
        "peaks_measured": {"fp32_tops": fp32_rate / 1e12, "fp64_tops": fp64_rate / 1e12},
        "fp64_form": fp64,
        "eig_arith": eig_cmp,
        "clocks": clk,
        "wall_s_timed": wall,
    }
    if rank == 0 and a.mc_plants > 0:
        line["monte_carlo"] = monte_carlo_bench(a.mc_plants, 2, 1)
    if rank == 0 and a.small_steps > 0:
        line["small"] = small_bench(a.small_steps, 3, not a.no_cpu)
    if rank == 0 and a.uneven_instances > 0:
        line["uneven"] = uneven_bench(a.uneven_instances, 3, 2)
    if rank == 0 and a.kalman_candidates > 0:
        line["kalman"] = kalman_bench(a.kalman_candidates, 3, 3, 0.0 if a.no_cpu else 5.0, not a.no_autotune)
    if rank == 0 and a.serve_seconds > 0:
        models = serving_models()
        line["serving"] = serving_bench(models, a.serve_seconds, lanes=a.serve_lanes, max_wait_us=a.serve_max_wait_us,
                                        max_batch_work=a.serve_max_work, runs=a.serve_runs)
        # the same request stream served by the plain FP64 form (at its own 70% load)
        line["serving"]["fp64_form"] = {k: v for k, v in serving_bench(models, a.serve_seconds / 2,
                                                                       precision="fp64").items()
                                        if k in ("saturation_candidates_per_s", "offered_requests_per_s",
                                                 "achieved_candidates_per_s", "latency_p50_ms", "latency_p99_ms",
                                                 "latency_max_ms", "requests", "monte_carlo_requests")}
    if rank == 0 and not a.no_cpu:
        line["cpu_baseline"], orc_rows = cpu_baseline(problem, a.cpu_seconds, os.cpu_count() or 1)
        # the rows the oracle computed for the baseline, against the engine's rows of the timed steps
        line["parity"] = parity_report(value_rows[:len(orc_rows)], orc_rows, cfg)
        line["parity"]["what"] = ("engine rows of the timed headline batch (default eigensolve arithmetic: "
                                  f"{sess.eig_arith}) vs the oracle's rows (the reference's separate arithmetic) "
                                  "on the cpu_baseline sample")
        if eig_cmp is not None and eig_cmp["other"] == "separate":
            # the same sample evaluated with the reference's own (separate) eigensolve arithmetic
            sep = parity_report(other_rows[:len(orc_rows)], orc_rows, cfg)
            sep["what"] = ("engine rows of the same headline batch with the separate eigensolve arithmetic "
                           "(the oracle's) vs the oracle's rows on the cpu_baseline sample")
            line["parity"]["separate_arithmetic"] = sep
    if rank == 0:
        print(json.dumps(line), flush=True)
    sess.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
