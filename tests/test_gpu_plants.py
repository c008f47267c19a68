"""One plant per candidate (ce_evaluate_plants): a batch in which candidate c uses
plant first + c of the session must give, row for row and bit for bit, what
evaluating each candidate alone with its plant gives -- in serial mode (the margin
check and the sweep on each candidate's own plant) and in batch mode (on the
shared observer model)."""
import numpy as np
import pytest

import controllerengine_gb300 as ce
from controllerengine_gb300 import synth

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _alone(s, p, first, n):
    return np.vstack([s.evaluate(p.cuda_mx[k:k + 1], p.info_mx[k:k + 1], plant_index=first + k) for k in range(n)])


@pytest.mark.parametrize("serial", [True, False])
def test_per_candidate_plants_equal_alone(serial):
    p = synth.monte_carlo(n_plants=96, time=1500, freq=80, serial=serial)
    # vary the gains too, so the batch holds stable and unstable loops
    rng = np.random.default_rng(11)
    p.cuda_mx[:, :8] *= rng.uniform(0.5, 3.0, (96, 1)).astype(np.float32)
    p.info_mx[:, :8] = p.cuda_mx[:, :8]
    cfg = ce.EngineConfig.parse(p.config_text)
    assert cfg.serial == (1 if serial else 0)
    with ce.Session(cfg, p.plant, n_plants=96) as s:
        mc = s.evaluate_plants(p.cuda_mx, p.info_mx)
        ref = _alone(s, p, 0, 96)
        # an offset window of plants
        part = s.evaluate_plants(p.cuda_mx[40:70], p.info_mx[40:70], first_plant=40)
    assert np.array_equal(_bits(mc), _bits(ref))
    assert np.array_equal(_bits(part), _bits(ref[40:70]))
    sc = mc[:, cfg.info_scoring:cfg.info_scoring + 3]
    assert len(np.unique(sc[:, 0])) > 48  # the plants differ
    assert (sc[:, 1] < cfg.unstable_err).sum() > 10  # and many loops are scored


def test_per_candidate_plants_errors():
    p = synth.monte_carlo(n_plants=8, time=500, freq=40)
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, n_plants=8) as s:
        with pytest.raises(ce.ControllerEngineError, match="exceed the session"):
            s.evaluate_plants(p.cuda_mx, p.info_mx, first_plant=1)


@pytest.mark.parametrize("serial", [True, False])
def test_per_candidate_plants_fp64_form(serial):
    """The plain FP64 form with one plant per candidate: rows equal the FP64 form of each
    candidate alone with its plant, and differ from the mixed form's."""
    p = synth.monte_carlo(n_plants=64, time=1200, freq=60, serial=serial)
    rng = np.random.default_rng(12)
    p.cuda_mx[:, :8] *= rng.uniform(0.5, 3.0, (64, 1)).astype(np.float32)
    p.info_mx[:, :8] = p.cuda_mx[:, :8]
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, n_plants=64) as s:
        mixed = s.evaluate_plants(p.cuda_mx, p.info_mx)
        s.set_precision("fp64")
        f64 = s.evaluate_plants(p.cuda_mx, p.info_mx)
        part = s.evaluate_plants(p.cuda_mx[10:30], p.info_mx[10:30], first_plant=10)
        ref = _alone(s, p, 0, 64)
    assert np.array_equal(_bits(f64), _bits(ref))
    assert np.array_equal(_bits(part), _bits(ref[10:30]))
    assert not np.array_equal(_bits(f64), _bits(mixed))
    sc = f64[:, cfg.info_scoring:cfg.info_scoring + 3]
    assert len(np.unique(sc[:, 0])) > 32 and (sc[:, 1] < cfg.unstable_err).sum() > 5


def test_per_candidate_device_api():
    import torch
    p = synth.monte_carlo(n_plants=64, time=800, freq=50)
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, n_plants=64) as s:
        host = s.evaluate_plants(p.cuda_mx, p.info_mx)
        g = torch.from_numpy(p.cuda_mx).cuda()
        i = torch.from_numpy(p.info_mx).cuda()
        o = torch.empty_like(i)
        st = torch.cuda.current_stream()
        s.evaluate_plants_device(64, g.data_ptr(), i.data_ptr(), o.data_ptr(), stream=st.cuda_stream)
        torch.cuda.synchronize()
    assert np.array_equal(_bits(host), _bits(o.cpu().numpy()))
