"""The engine's kernels against the REFERENCE's own kernels on the GPU.

oracle/_ref/ref_kernels.cubin is the reference's src/main.cu compiled for
sm_103a where it lies (`make -C oracle ref`, with a type-level stand-in for
the absent Eigen headers); oracle/ref_kernels.py launches its discrete_solve,
eigensetup and modalsetup with the reference's launch shape and constant
tables.  Same inputs in, bit-identical outputs expected: trajectories, LIN_A,
and (fed the engine's own FP64 eigenvalues) AtA, Atb, yss, overshoot and the
unstable penalty."""
import numpy as np
import pytest

import controllerengine_gb300 as ce

pytestmark = pytest.mark.gpu


def _eq(a, b):
    return np.array_equal(a, b, equal_nan=True)


def _bad(a, b):
    return int((~((a == b) | (np.isnan(a) & np.isnan(b)))).sum())


@pytest.fixture(scope="module")
def refk():
    from oracle import ref_kernels
    if not ref_kernels.available():
        pytest.skip("reference cubin not built (needs the reference tree: make -C oracle ref)")
    return ref_kernels


@pytest.mark.parametrize("which", ["mass_spring", "eight_state_small"])
def test_engine_kernels_equal_reference_kernels(lib, refk, which, request):
    p = request.getfixturevalue(which)
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant) as s:
        info, d = s.evaluate_diagnostics(p.cuda_mx, p.info_mx)
    y, lina, ata, atb, rinfo = refk.run(cfg, p.plant, p.cuda_mx, d["eigen"], p.info_mx)
    assert _eq(d["yplant"], y), f"trajectory: {_bad(d['yplant'], y)} of {y.size} differ"
    assert _eq(d["lina"], lina), f"LIN_A: {_bad(d['lina'], lina)} differ"
    assert _eq(d["ata"], ata), f"AtA: {_bad(d['ata'], ata)} differ"
    assert _eq(d["atb"], atb), f"Atb: {_bad(d['atb'], atb)} differ"
    fr = cfg.info_freqresp
    assert _eq(info[:, fr + 2:fr + 4], rinfo[:, fr + 2:fr + 4]), "yss / overshoot"
    s0 = cfg.info_scoring
    unst = rinfo[:, s0] != p.info_mx[:, s0]  # rows the reference's modalsetup flagged unstable
    assert unst.any()
    assert _eq(info[unst, s0:s0 + 2], rinfo[unst, s0:s0 + 2]), "unstable penalty"


def test_oracle_kalman_against_reference_kalman_kernel(refk, oracle_mod):
    """The reference never launches discrete_solve<Kalman> (src/discrete_solves.cu:83-185);
    here its compiled kernel runs on rows of its own layout [K, N, R, Q], given to it as the
    row width so that no read leaves the row, against the oracle's literal form of it (that
    layout, and the Joseph product written over its own left factor in source order).  The
    one remaining difference is the reciprocal -- the kernel's approximate __fdividef, the
    oracle's correctly rounded quotient -- so whole trajectories are compared row by row: at
    least half must be identical, and the rows that blow up must be the same rows; the same
    kernel built with __fdividef read as the correctly rounded quotient must match every row.
    The engine's form (own storage for the Joseph product) stays finite where the reference's
    diverges."""
    from controllerengine_gb300 import synth
    for name, p in (("mass", synth.with_kalman(synth.mass_spring(256), seed=5)),
                    ("eight", synth.eight_state(n=256, time=3000, freq=40, observer="kalman"))):
        cfg = ce.EngineConfig.parse(p.config_text)
        ns = cfg.statespace_dim
        lit = np.ascontiguousarray(np.hstack([p.cuda_mx[:, :ns], p.cuda_mx[:, 2 * ns:]]))
        y_ref = refk.run_kalman(cfg, p.plant, lit)
        orc = oracle_mod.Oracle(p.config_text, p.plant)
        y_lit, _ = orc.sim_kalman(lit, literal=True)
        same = np.array([_eq(a, b) for a, b in zip(y_ref, y_lit)])
        assert same.mean() >= 0.5, f"{name}: {same.sum()} of {len(same)} rows identical"
        assert _eq(y_ref[:, :2], y_lit[:, :2])
        blown_ref = ~np.isfinite(y_ref).all(axis=1)
        assert np.array_equal(blown_ref, ~np.isfinite(y_lit).all(axis=1)), name
        assert np.isfinite(orc.sim(p.cuda_mx)).all(), name
        if name == "eight":
            assert blown_ref.mean() > 0.5  # the in-place Joseph product diverges
        # the reference's kernel with its reciprocal correctly rounded (built beside the plain
        # one by `make -C oracle ref`): every row identical
        assert refk.CUBIN_RN.exists()
        y_rn = refk.run_kalman(cfg, p.plant, lit, rounded_reciprocal=True)
        assert _eq(y_rn, y_lit), f"{name}: {_bad(y_rn, y_lit)} values differ"

