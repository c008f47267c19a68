"""Uneven shapes: random statespace / discrete dimensions (2..8), 0-4 nonlinear
terms with SKIP and no-op rows, and assorted horizons and sweep lengths, checked
stage by stage against the oracle with the same bars as test_gpu_parity.py
(trajectories, LIN_A, eigenvalues, yss / overshoot and classifications bit-exact).
Covers every simulation dimension class (4, 8, with the padding emulation) and
every sweep class (2, 4, 8)."""
import pytest

from controllerengine_gb300 import EngineConfig, synth
from parity_helpers import _stagewise

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", range(12))
def test_random_shape_stagewise(seed, lib, oracle_mod):
    rng_time = [700, 1500, 2500, 1000][seed % 4]
    prob = synth.random_shape(seed, n=256, time=rng_time, freq=40 + 10 * (seed % 7))
    _stagewise(prob, oracle_mod)


def test_random_shapes_cover_the_classes():
    dims = [EngineConfig.parse(synth.random_shape(s, n=8, time=700, freq=40).config_text) for s in range(12)]
    ns = {c.statespace_dim for c in dims}
    nd = {c.discrete_dim for c in dims}
    assert any(d <= 2 for d in ns) and any(2 < d <= 4 for d in ns) and any(d > 4 for d in ns)
    assert any(d <= 4 for d in nd) and any(d > 4 for d in nd)
    assert any(c.nonlin_dim == 0 for c in dims) and any(c.nonlin_dim >= 3 for c in dims)
