"""Ragged batches (ce_ragged_*): instances of different shapes -- dimensions 2..8, 0..4
nonlinear terms with their own instruction programs, horizons, sweep sizes, batch and serial
margin plants -- evaluated together with one launch per stage must give every instance's rows
bit for bit as a session of its own configuration and plant does."""
import numpy as np
import pytest

import controllerengine_gb300 as ce
from controllerengine_gb300 import synth

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _instances():
    rng = np.random.default_rng(21)
    probs = []
    for k in range(10):
        probs.append(synth.random_shape(300 + k, n=int(rng.integers(1, 60)), time=int(rng.integers(400, 2500)),
                                        freq=int(rng.integers(30, 160))))
    probs.append(synth.mass_spring(40))
    mc = synth.monte_carlo(n_plants=1, time=900, freq=50, serial=True)
    probs.append(synth.Problem(mc.name, mc.config_text, mc.plant, np.repeat(mc.cuda_mx, 7, 0),
                               np.repeat(mc.info_mx, 7, 0)))
    return probs


def test_ragged_equals_own_sessions():
    probs = _instances()
    cfgs = [ce.EngineConfig.parse(p.config_text) for p in probs]
    assert len({(c.statespace_dim, c.discrete_dim, c.nonlin_dim) for c in cfgs}) >= 6
    assert any(c.serial for c in cfgs)
    with ce.Ragged([(c, p.plant) for c, p in zip(cfgs, probs)]) as rb:
        l0 = rb.kernel_launches
        outs = rb.evaluate([(p.cuda_mx, p.info_mx) for p in probs])
        # the candidate table (once per candidate counts), the gather into the device order, one
        # launch per stage for all instances, the scatter of the INFO rows
        assert rb.kernel_launches - l0 == 12
        l1 = rb.kernel_launches
        again = rb.evaluate([(p.cuda_mx, p.info_mx) for p in probs])
        assert rb.kernel_launches - l1 == 11
    for c, p, o, o2 in zip(cfgs, probs, outs, again):
        with ce.Session(c, p.plant) as s:
            ref = s.evaluate(p.cuda_mx, p.info_mx)
        assert np.array_equal(_bits(o), _bits(ref)), p.name
        assert np.array_equal(_bits(o2), _bits(ref)), p.name
    sc = np.concatenate([o[:, c.info_scoring] for c, o in zip(cfgs, outs)])
    assert (sc < 1e6).sum() > 20 and (sc >= 1e6).sum() > 0  # scored and unstable loops both present


def test_ragged_many_single_candidate_instances():
    """One candidate per instance, as in the uneven-size configuration; a sample of the
    instances against their own sessions."""
    probs = [synth.random_shape(2000 + k, n=1, time=int(400 + 37 * k % 1500), freq=int(30 + 7 * k % 120))
             for k in range(400)]
    cfgs = [ce.EngineConfig.parse(p.config_text) for p in probs]
    with ce.Ragged([(c, p.plant) for c, p in zip(cfgs, probs)]) as rb:
        outs = rb.evaluate([(p.cuda_mx, p.info_mx) for p in probs])
    for k in range(0, 400, 23):
        with ce.Session(cfgs[k], probs[k].plant) as s:
            ref = s.evaluate(probs[k].cuda_mx, probs[k].info_mx)
        assert np.array_equal(_bits(outs[k]), _bits(ref)), k


def test_ragged_empty_and_uneven_counts():
    probs = _instances()[:4]
    cfgs = [ce.EngineConfig.parse(p.config_text) for p in probs]
    with ce.Ragged([(c, p.plant) for c, p in zip(cfgs, probs)]) as rb:
        outs = rb.evaluate([(p.cuda_mx[:0], p.info_mx[:0]) if k % 2 else (p.cuda_mx, p.info_mx)
                            for k, p in enumerate(probs)])
        none = rb.evaluate([(p.cuda_mx[:0], p.info_mx[:0]) for p in probs])
    assert all(o.shape[0] == 0 for k, o in enumerate(outs) if k % 2)
    assert all(o.shape[0] == 0 for o in none)
    for k in (0, 2):
        with ce.Session(cfgs[k], probs[k].plant) as s:
            assert np.array_equal(_bits(outs[k]), _bits(s.evaluate(probs[k].cuda_mx, probs[k].info_mx)))


def test_ragged_order_reused_across_calls():
    """The device order is kept while the candidate counts repeat: one ragged batch evaluated
    with counts A, then B, then A again on other gains, every time equal to the sessions."""
    probs = _instances()
    cfgs = [ce.EngineConfig.parse(p.config_text) for p in probs]
    rng = np.random.default_rng(5)

    def rows(sub, scale):
        # K and L scaled (N kept); the INFO rows' user columns pass through unchanged
        out = []
        for p, m in zip(probs, sub):
            g = p.cuda_mx[:m].copy()
            g[:, :-1] *= np.float32(scale)
            out.append((g, p.info_mx[:m].copy()))
        return out

    full = [p.cuda_mx.shape[0] for p in probs]
    part = [max(0, m - int(rng.integers(0, 3))) for m in full]
    with ce.Ragged([(c, p.plant) for c, p in zip(cfgs, probs)]) as rb:
        for sub, scale in ((full, 1.0), (part, 1.0), (full, 0.9)):
            batch = rows(sub, scale)
            outs = rb.evaluate(batch)
            for c, p, (g, i), o in zip(cfgs, probs, batch, outs):
                if g.shape[0] == 0:
                    continue
                with ce.Session(c, p.plant) as s:
                    ref = s.evaluate(g, i)
                assert np.array_equal(_bits(o), _bits(ref)), (p.name, scale, g.shape[0])


_ONE_THREAD_SCRIPT = r"""
import sys, numpy as np
import controllerengine_gb300 as ce
from controllerengine_gb300 import synth
probs = [synth.random_shape(2000 + k, n=3, time=int(400 + 37 * k % 1500), freq=int(30 + 7 * k % 120))
         for k in range(120)]
cfgs = [ce.EngineConfig.parse(p.config_text) for p in probs]
with ce.Ragged([(c, p.plant) for c, p in zip(cfgs, probs)]) as rb:
    outs = rb.evaluate([(p.cuda_mx, p.info_mx) for p in probs])
np.save(sys.argv[1], np.concatenate([o.ravel() for o in outs]))
"""


def test_ragged_one_thread_form_equals_wide_form(tmp_path):
    """The one-thread simulation form (CE_RAGGED_WIDE=0, read once per process) and the default
    wide form give the same rows bit for bit."""
    import os
    import subprocess
    import sys
    script = tmp_path / "ragged_form.py"
    script.write_text(_ONE_THREAD_SCRIPT)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    res = {}
    for form, env in (("wide", {}), ("one", {"CE_RAGGED_WIDE": "0"})):
        out = tmp_path / f"{form}.npy"
        subprocess.run([sys.executable, str(script), str(out)], check=True, cwd=root,
                       env={**os.environ, **env, "PYTHONPATH": root})
        res[form] = np.load(out)
    assert np.array_equal(_bits(res["wide"]), _bits(res["one"]))


def _dims_of(seed):
    rng = np.random.default_rng(seed)
    return int(rng.integers(2, 9)), int(rng.integers(2, 9))


def test_ragged_dimension_classes_with_diverging_loops():
    """Warps of small plants run the 4-row steps with the padding beyond 4 virtual: rows equal the
    instances' own sessions bit for bit, also for loops whose gains are scaled until the trajectory
    overflows (the padded states of the reference then turn NaN and poison every row)."""
    want = {(4, 4): 3, (4, 8): 1, (8, 4): 1, (8, 8): 1}
    seeds = []
    for seed in range(5000, 5400):
        ns, nd = _dims_of(seed)
        cls = (4 if ns <= 4 else 8, 4 if nd <= 4 else 8)
        if want.get(cls, 0) > 0:
            want[cls] -= 1
            seeds.append(seed)
    assert not any(want.values())
    probs = []
    for seed in seeds:
        p = synth.random_shape(seed, n=48, time=1500, freq=60)
        g = p.cuda_mx.copy()
        ns = _dims_of(seed)[0]
        g[::2, :2 * ns] *= np.float32(30.0)  # K and L of every other candidate
        probs.append(synth.Problem(p.name, p.config_text, p.plant, g, p.info_mx))
    cfgs = [ce.EngineConfig.parse(p.config_text) for p in probs]
    with ce.Ragged([(c, p.plant) for c, p in zip(cfgs, probs)]) as rb:
        outs = rb.evaluate([(p.cuda_mx, p.info_mx) for p in probs])
    unstable = 0
    for c, p, o in zip(cfgs, probs, outs):
        with ce.Session(c, p.plant) as s:
            ref = s.evaluate(p.cuda_mx, p.info_mx)
        assert np.array_equal(_bits(o), _bits(ref)), p.name
        unstable += int((o[:, c.info_scoring + 1] >= c.unstable_err).sum())
    assert unstable > 20, unstable
