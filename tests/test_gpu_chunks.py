"""A large batch is evaluated in chunks (eigensolves of later chunks overlap the
fit of earlier ones).  Every candidate is computed independently, so the INFO
rows must not depend on how the batch is cut: one 49,152-candidate call (cut
into chunks) must equal three 16,384-candidate calls (one chunk each), bit for
bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from controllerengine_gb300 import EngineConfig, Session, synth  # noqa: E402


def test_chunked_batch_equals_separate_calls():
    prob = synth.eight_state(n=49152, time=2000, freq=100)
    cfg = EngineConfig.parse(prob.config_text)
    with Session(cfg, prob.plant) as s:
        l0 = s.kernel_launches
        whole = s.evaluate(prob.cuda_mx, prob.info_mx)
        assert s.kernel_launches - l0 > 9  # the batch was cut into chunks
        parts = [s.evaluate(prob.cuda_mx[k:k + 16384], prob.info_mx[k:k + 16384]) for k in range(0, 49152, 16384)]
    sep = np.vstack(parts)
    bad = np.flatnonzero(whole.view(np.uint32) != sep.view(np.uint32))
    assert bad.size == 0, f"{bad.size} INFO values differ, first at {bad[:5]}"
    # not vacuous: most candidates carry a finite total score
    assert np.isfinite(whole[:, cfg.info_scoring]).mean() > 0.5
