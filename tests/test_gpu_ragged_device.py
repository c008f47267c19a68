"""The ragged batch's device path: ce_ragged_prepare + ce_ragged_evaluate_device on device rows,
captured into a CUDA graph and replayed, and the ragged autotuner.  Every result must equal the
host path's (ce_ragged_evaluate) bit for bit: the device order, the simulation form and the
launch settings change where and how a candidate is computed, never its result."""
import numpy as np
import pytest

import controllerengine_gb300 as ce
from controllerengine_gb300 import synth

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _batch():
    rng = np.random.default_rng(33)
    probs = [synth.random_shape(700 + k, n=int(rng.integers(1, 40)), time=int(rng.integers(400, 2000)),
                                freq=int(rng.integers(30, 140))) for k in range(14)]
    probs.append(synth.mass_spring(25))
    cfgs = [ce.EngineConfig.parse(p.config_text) for p in probs]
    return probs, cfgs


def _packed(probs, scale=1.0):
    g = np.concatenate([(p.cuda_mx * np.float32(scale)).astype(np.float32).reshape(-1) for p in probs])
    i = np.concatenate([p.info_mx.reshape(-1) for p in probs])
    return g, i


def test_ragged_device_path_in_a_cuda_graph():
    import torch
    probs, cfgs = _batch()
    counts = [p.cuda_mx.shape[0] for p in probs]
    g1, i1 = _packed(probs)
    g2, _ = _packed(probs, 1.2)
    with ce.Ragged([(c, p.plant) for c, p in zip(cfgs, probs)]) as rb:
        ref1 = rb.evaluate_packed(counts, g1, i1)
        ref2 = rb.evaluate_packed(counts, g2, i1)
        dg = torch.from_numpy(g1).cuda()
        di = torch.from_numpy(i1).cuda()
        do = torch.empty_like(di)
        rb.prepare(counts)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):  # an uncaptured call first: kernels loaded
            rb.evaluate_device(dg.data_ptr(), di.data_ptr(), do.data_ptr(), stream=side.cuda_stream)
        torch.cuda.synchronize()
        direct = do.cpu().numpy()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            rb.evaluate_device(dg.data_ptr(), di.data_ptr(), do.data_ptr(),
                               stream=torch.cuda.current_stream().cuda_stream)
        do.zero_()
        graph.replay()
        torch.cuda.synchronize()
        out1 = do.cpu().numpy()
        dg.copy_(torch.from_numpy(g2))
        graph.replay()
        torch.cuda.synchronize()
        out2 = do.cpu().numpy()
    assert np.array_equal(_bits(direct), _bits(ref1))
    assert np.array_equal(_bits(out1), _bits(ref1))
    assert np.array_equal(_bits(out2), _bits(ref2))


def test_ragged_tunings_and_autotune_keep_results():
    import torch
    probs, cfgs = _batch()
    counts = [p.cuda_mx.shape[0] for p in probs]
    g, i = _packed(probs)
    with ce.Ragged([(c, p.plant) for c, p in zip(cfgs, probs)]) as rb:
        ref = rb.evaluate_packed(counts, g, i)
        for t in ({"sim_lanes": 1}, {"instance_order": 1}, {"instance_order": 2}, {"sim_lanes": 1, "instance_order": 1},
                  {"sim_lanes": 1, "instance_order": 2}, {"eig_blocks_per_sm": 3},
                  {"sim_width": 8}, {"sim_width": 8, "instance_order": 2}):
            rb.set_tuning(**t)
            assert np.array_equal(_bits(rb.evaluate_packed(counts, g, i)), _bits(ref)), t
        rb.set_tuning()
        dg = torch.from_numpy(g).cuda()
        di = torch.from_numpy(i).cuda()
        do = torch.empty_like(di)
        rb.prepare(counts)
        best = rb.autotune(dg.data_ptr(), di.data_ptr(), do.data_ptr(),
                           stream=torch.cuda.current_stream().cuda_stream)
        assert best["sim_lanes"] in (1, 4) and best["instance_order"] in (0, 1, 2) and best["ms_per_evaluation"] > 0
        assert rb.tuning["sim_lanes"] == best["sim_lanes"]
        torch.cuda.synchronize()
        assert np.array_equal(_bits(do.cpu().numpy()), _bits(ref))
        assert np.array_equal(_bits(rb.evaluate_packed(counts, g, i)), _bits(ref))
