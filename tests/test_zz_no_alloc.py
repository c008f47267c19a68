"""ce_modal_fit_noalloc: the modal-fit path for callers that cannot allocate
device memory when they evaluate (a real-time loop that cannot take
cudaMalloc's latency, an application whose device memory belongs to its own
allocator).  Its fit-window scratch is a
static device array instead of cudaMalloc'd memory.

Checked through the C ABI against the session pipeline (ce_evaluate_diagnostics,
the existing entry point) on two calls in a row that reuse the shared array,
with the tolerance of the other kernel tests for these stages (they are the
same kernels: bit-exact).  This file sorts last so that a run stopping at the
first failure has run everything else first."""
import ctypes as C

import numpy as np
import pytest

import controllerengine_gb300 as ce
from controllerengine_gb300 import _ffi, synth

pytestmark = pytest.mark.gpu


def _noalloc(lib, sess, n, g, eig, ata, atb, info, stream):
    rc = lib.ce_modal_fit_noalloc(sess._h, 0, n, C.c_void_p(g.data_ptr()), C.c_void_p(eig.data_ptr()),
                                  C.c_void_p(ata.data_ptr()), C.c_void_p(atb.data_ptr()),
                                  C.c_void_p(info.data_ptr()), C.c_void_p(stream))
    assert rc == 0, _ffi.last_error(lib)


@pytest.mark.parametrize("observer", ["luenberger", "kalman"])
def test_noalloc_matches_session_pipeline_twice(lib, observer):
    import torch
    p = synth.mass_spring(1536)
    if observer == "kalman":
        p = synth.with_kalman(p, seed=5)
    cfg = ce.EngineConfig.parse(p.config_text)
    nt = cfg.total_dim
    fr, s0 = cfg.info_freqresp, cfg.info_scoring
    with ce.Session(cfg, p.plant) as sess:
        ref_info, d = sess.evaluate_diagnostics(p.cuda_mx, p.info_mx, want=("eigen", "ata", "atb"))
        stream = torch.cuda.current_stream().cuda_stream
        # two calls in a row on the shared scratch: a small batch, then a larger one
        for lo, hi in ((0, 600), (600, 1536)):
            n = hi - lo
            g = torch.from_numpy(np.ascontiguousarray(p.cuda_mx[lo:hi])).cuda()
            eig = torch.from_numpy(np.ascontiguousarray(d["eigen"][lo:hi])).cuda()
            info = torch.from_numpy(np.ascontiguousarray(p.info_mx[lo:hi])).cuda()
            ata = torch.full((n, 4 * nt * nt), float("nan"), device="cuda")
            atb = torch.full((n, 2 * nt), float("nan"), device="cuda")
            _noalloc(lib, sess, n, g, eig, ata, atb, info, stream)
            torch.cuda.synchronize()
            np.testing.assert_array_equal(ata.cpu().numpy(), d["ata"][lo:hi])
            np.testing.assert_array_equal(atb.cpu().numpy(), d["atb"][lo:hi])
            out = info.cpu().numpy()
            # yss and overshoot of the stable candidates, the penalty of the unstable ones
            np.testing.assert_array_equal(out[:, fr + 2:fr + 4], ref_info[lo:hi, fr + 2:fr + 4])
            unst = out[:, s0] != p.info_mx[lo:hi, s0]
            assert unst.any()
            np.testing.assert_array_equal(out[unst, s0:s0 + 2], ref_info[lo:hi][unst, s0:s0 + 2])


def test_noalloc_leaves_free_device_memory_unchanged(lib):
    """After a first call (which may load the module that holds the static array), further calls
    change nothing in the device's free memory: they allocate nothing."""
    import torch
    p = synth.mass_spring(1536)
    cfg = ce.EngineConfig.parse(p.config_text)
    nt, n = cfg.total_dim, 512
    with ce.Session(cfg, p.plant) as sess:
        _, d = sess.evaluate_diagnostics(p.cuda_mx[:n], p.info_mx[:n], want=("eigen",))
        g = torch.from_numpy(np.ascontiguousarray(p.cuda_mx[:n])).cuda()
        eig = torch.from_numpy(np.ascontiguousarray(d["eigen"])).cuda()
        info = torch.from_numpy(np.ascontiguousarray(p.info_mx[:n])).cuda()
        ata = torch.empty((n, 4 * nt * nt), device="cuda")
        atb = torch.empty((n, 2 * nt), device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        _noalloc(lib, sess, n, g, eig, ata, atb, info, stream)
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        for _ in range(3):
            _noalloc(lib, sess, n, g, eig, ata, atb, info, stream)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_batches_beyond_the_static_scratch(lib):
    import torch
    p = synth.mass_spring(1536)
    cfg = ce.EngineConfig.parse(p.config_text)
    per = ((cfg.fit_steps + 7) // 8) * 8 + 4
    too_many = (8 * 1024 * 1024) // per + 1
    with ce.Session(cfg, p.plant) as sess:
        z = torch.zeros(1, device="cuda")
        for n in (too_many, 1 << 62):  # the second would overflow n * per in 64 bits
            rc = lib.ce_modal_fit_noalloc(sess._h, 0, n, *(C.c_void_p(z.data_ptr()),) * 5, C.c_void_p(0))
            assert rc == 1
            assert "the static scratch holds 8388608 floats" in _ffi.last_error(lib)


def test_noalloc_refuses_an_unusable_plant_like_the_session(lib):
    """A plant whose sweep grid failed at session creation (C = 0: no gain at the crossover) is
    refused with its message, as the session pipeline refuses it; nothing is launched."""
    import torch
    p = synth.monte_carlo(n_plants=8, time=600, freq=40, serial=True)
    p.plant.discrete_c[5 * 8:6 * 8] = 0.0
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, n_plants=8) as sess:
        z = torch.zeros(1, device="cuda")
        rc = lib.ce_modal_fit_noalloc(sess._h, 5, 4, *(C.c_void_p(z.data_ptr()),) * 5, C.c_void_p(0))
        assert rc == 1
        assert "plant 5" in _ffi.last_error(lib) and "crossover" in _ffi.last_error(lib)
