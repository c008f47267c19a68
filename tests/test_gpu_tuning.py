"""Launch tuning (ce_session_set_tuning / ce_session_autotune): every setting of
lanes per matrix, blocks per SM and chunk count gives bit-identical rows, and the
autotuner returns one of the settings it tried with its time."""
import numpy as np
import pytest

import controllerengine_gb300 as ce
from controllerengine_gb300 import synth

pytestmark = pytest.mark.gpu


def test_tuning_does_not_change_results():
    import torch
    p = synth.eight_state(n=40000, time=1200, freq=60)
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant) as s:
        ref = s.evaluate(p.cuda_mx, p.info_mx)
        for lanes, blocks, chunks in [(1, 3, 1), (4, 10, 2), (2, 6, 2), (2, 4, 1), (8, 5, 2), (16, 5, 1)]:
            s.set_tuning(lanes, blocks, chunks)
            out = s.evaluate(p.cuda_mx, p.info_mx)
            assert np.array_equal(out.view(np.uint32), ref.view(np.uint32)), (lanes, blocks, chunks)
        with pytest.raises(ce.ControllerEngineError, match="eig_lanes"):
            s.set_tuning(3, 0, 0)
        g = torch.from_numpy(p.cuda_mx).cuda()
        i = torch.from_numpy(p.info_mx).cuda()
        o = torch.empty_like(i)
        best = s.autotune(g.shape[0], g.data_ptr(), i.data_ptr(), o.data_ptr(),
                          stream=torch.cuda.current_stream().cuda_stream)
        assert best["eig_lanes"] in (1, 2, 4) and best["chunks"] in (1, 2, 4) and best["ms_per_evaluation"] > 0
        assert s.tuning["eig_lanes"] == best["eig_lanes"]
        after = s.evaluate(p.cuda_mx, p.info_mx)
    assert np.array_equal(after.view(np.uint32), ref.view(np.uint32))


def test_small_batch_lanes_do_not_change_results():
    """A batch too small to fill the persistent eigensolve grid gets more lanes per matrix by
    default (up to 16); its rows equal those of every explicit setting."""
    p = synth.eight_state(n=700, time=1500, freq=80)
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant) as s:
        auto = s.evaluate(p.cuda_mx, p.info_mx)
        for lanes in (1, 2, 4, 8, 16):
            s.set_tuning(lanes, 0, 0)
            out = s.evaluate(p.cuda_mx, p.info_mx)
            assert np.array_equal(out.view(np.uint32), auto.view(np.uint32)), lanes


def test_kalman_session_lanes_do_not_change_results():
    """Kalman-observer sessions launch their own instantiations of the default eigensolve form
    (two lanes per matrix, fused arithmetic, no register bound); its rows equal those of the other
    lane counts."""
    p = synth.eight_state(n=700, time=1500, freq=80, pool=4, observer="kalman")
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant) as s:
        s.set_tuning(2, 0, 0)
        two = s.evaluate(p.cuda_mx, p.info_mx)
        for lanes in (1, 4, 16):
            s.set_tuning(lanes, 0, 0)
            out = s.evaluate(p.cuda_mx, p.info_mx)
            assert np.array_equal(out.view(np.uint32), two.view(np.uint32)), lanes
