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
