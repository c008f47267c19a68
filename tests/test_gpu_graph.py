"""One evaluation captured into a CUDA graph (torch.cuda.graph on the caller's
stream) and replayed: the session's fork/join streams join the capture, no
allocation happens inside it (the first, uncaptured call sizes the scratch),
and replays on new inputs in the same buffers equal direct evaluations."""
import numpy as np
import pytest

import controllerengine_gb300 as ce

pytestmark = pytest.mark.gpu


def test_graph_capture_and_replay(eight_state_small):
    import torch
    p = eight_state_small
    cfg = ce.EngineConfig.parse(p.config_text)
    n = p.cuda_mx.shape[0]
    with ce.Session(cfg, p.plant) as s:
        ref1 = s.evaluate(p.cuda_mx, p.info_mx)
        g2 = (p.cuda_mx * np.float32(1.3)).astype(np.float32)
        ref2 = s.evaluate(g2, p.info_mx)
        dg = torch.from_numpy(p.cuda_mx).cuda()
        di = torch.from_numpy(p.info_mx).cuda()
        do = torch.empty_like(di)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):  # first call outside the capture: scratch sized, kernels loaded
            s.evaluate_device(n, dg.data_ptr(), di.data_ptr(), do.data_ptr(), stream=side.cuda_stream)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            s.evaluate_device(n, dg.data_ptr(), di.data_ptr(), do.data_ptr(),
                              stream=torch.cuda.current_stream().cuda_stream)
        graph.replay()
        torch.cuda.synchronize()
        out1 = do.cpu().numpy()
        dg.copy_(torch.from_numpy(g2))
        graph.replay()
        torch.cuda.synchronize()
        out2 = do.cpu().numpy()
    assert np.array_equal(out1.view(np.uint32), ref1.view(np.uint32))
    assert np.array_equal(out2.view(np.uint32), ref2.view(np.uint32))
