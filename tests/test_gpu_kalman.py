"""The time-varying Kalman observer on the GPU (`observer = kalman`, ref:
src/discrete_solves.cu:83-185 with its row layout and in-place Joseph product fixed):
trajectories bit-identical to the oracle's restatement for the full eight-state
observer and for a 3-state observer inside the padded 8-wide loop, with the
table-driven and the specialised simulation kernels; the whole INFO row stage by
stage as for the Luenberger loop; per-candidate plants; and the FP64 form refused."""
import numpy as np
import pytest

import controllerengine_gb300 as ce
from controllerengine_gb300 import synth
from parity_helpers import _eq, _mismatch, _stagewise

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="module")
def eight_kalman():
    return synth.eight_state(n=512, time=3000, freq=160, observer="kalman")


@pytest.fixture(scope="module")
def mass_kalman():
    return synth.with_kalman(synth.mass_spring(1536), seed=5)


@pytest.mark.parametrize("kernel", ["table", "specialised"])
@pytest.mark.parametrize("which", ["eight", "mass"])
def test_kalman_trajectories_bit_exact(oracle_mod, eight_kalman, mass_kalman, kernel, which):
    p = eight_kalman if which == "eight" else mass_kalman
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant) as s:
        s.set_sim_kernel(kernel)
        _, d = s.evaluate_diagnostics(p.cuda_mx, p.info_mx)
    y_o = oracle_mod.Oracle(p.config_text, p.plant).sim(p.cuda_mx)
    assert _eq(d["yplant"], y_o), f"trajectory mismatches: {_mismatch(d['yplant'], y_o)}"
    assert np.isfinite(d["yplant"]).mean() > 0.9


@pytest.mark.parametrize("kernel", ["table", "specialised"])
@pytest.mark.parametrize("time", [800, 3000])
def test_kalman_distinct_noise_schedules_bit_exact(oracle_mod, kernel, time):
    """Every candidate with its own noise weights (R scaled by 1 + U[0, 1e-3]): the per-candidate
    list's gain schedules (periodic within 1,024 steps: the scheduled form; the rest: the full
    per-candidate recursion; with T = 800 the schedule covers the whole horizon) give the oracle's
    trajectories bit for bit."""
    p = synth.eight_state(n=384, time=time, freq=80, observer="kalman")
    g = p.cuda_mx.copy()
    g[:, 17] *= (1.0 + 1e-3 * np.random.default_rng(17).random(g.shape[0])).astype(np.float32)
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant) as s:
        s.set_sim_kernel(kernel)
        _, d = s.evaluate_diagnostics(g, p.info_mx)
    y_o = oracle_mod.Oracle(p.config_text, p.plant).sim(g)
    assert _eq(d["yplant"], y_o), f"trajectory mismatches: {_mismatch(d['yplant'], y_o)}"
    assert np.isfinite(d["yplant"]).mean() > 0.9


@pytest.mark.parametrize("which", ["eight", "mass"])
def test_kalman_stagewise(oracle_mod, eight_kalman, mass_kalman, which):
    # one mass-spring row has a score of -2.0e-3 that the oracle's glibc-recomputed modes
    # move by 1.5e-5 (the modal-fit sensitivity the stagewise check describes): 1e-4 absolute
    _stagewise(eight_kalman if which == "eight" else mass_kalman, oracle_mod,
               score_atol=1e-6 if which == "eight" else 1e-4)


def test_kalman_differs_from_luenberger(eight_kalman):
    """The same K, L, N with the Kalman loop: other trajectories, same LIN_A."""
    p = eight_kalman
    lue = synth.eight_state(n=512, time=3000, freq=160)
    outs = {}
    for q in (p, lue):
        cfg = ce.EngineConfig.parse(q.config_text)
        with ce.Session(cfg, q.plant) as s:
            outs[q.name] = s.evaluate_diagnostics(q.cuda_mx, q.info_mx)[1]
    a, b = outs[p.name], outs[lue.name]
    assert _eq(a["lina"], b["lina"])
    assert not _eq(a["yplant"], b["yplant"])


def test_kalman_per_candidate_plants():
    p = synth.with_kalman(synth.monte_carlo(n_plants=64, time=1200, freq=60, serial=True), seed=9)
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, n_plants=64) as s:
        mc = s.evaluate_plants(p.cuda_mx, p.info_mx)
        alone = np.vstack([s.evaluate(p.cuda_mx[k:k + 1], p.info_mx[k:k + 1], plant_index=k) for k in range(64)])
    assert np.array_equal(_bits(mc), _bits(alone))


def test_kalman_fp64_form_refused(mass_kalman):
    cfg = ce.EngineConfig.parse(mass_kalman.config_text)
    with ce.Session(cfg, mass_kalman.plant) as s:
        with pytest.raises(ce.ControllerEngineError, match="simulates in FP32 only"):
            s.set_precision("fp64")
        s.set_precision("compensated")  # the compensated form simulates in FP32: accepted


def _bucket(r, q):
    """The grouping hash of ce_k_kalman.cu (k_kal_hist) for one row's R and Q[0..ns)."""
    M = 0xffffffff
    rotl = lambda x, k: ((x << k) | (x >> (32 - k))) & M
    h = 0x9747b28c
    for w in np.asarray([r, *q], np.float32).view(np.uint32):
        v = (int(w) * 0xcc9e2d51) & M
        v = (rotl(v, 15) * 0x1b873593) & M
        h = (rotl(h ^ v, 13) * 5 + 0xe6546b64) & M
    h ^= len(q) + 1
    h ^= h >> 16
    h = (h * 0x85ebca6b) & M
    h ^= h >> 13
    h = (h * 0xc2b2ae35) & M
    h ^= h >> 16
    return h & 0xffff


def test_kalman_shared_noise_groups(oracle_mod):
    """Few noise-weight sets, so whole warps share a covariance recursion (and reach its
    fixed point or two-cycle within the horizon): every trajectory equals the oracle's."""
    p = synth.eight_state(n=1000, time=4000, freq=80, pool=3, observer="kalman")
    cfg = ce.EngineConfig.parse(p.config_text)
    assert len(np.unique(p.cuda_mx[:, 17:], axis=0)) == 3
    with ce.Session(cfg, p.plant) as s:
        _, d = s.evaluate_diagnostics(p.cuda_mx, p.info_mx, want=("yplant",))
        launches = s.kernel_launches
    # the nine of the Luenberger pipeline, three grouping kernels, the gain schedules and two more
    # simulation forms
    assert launches == 15
    y_o = oracle_mod.Oracle(p.config_text, p.plant).sim(p.cuda_mx)
    assert _eq(d["yplant"], y_o), f"trajectory mismatches: {_mismatch(d['yplant'], y_o)}"


def test_kalman_hash_collision_is_deferred(oracle_mod):
    """Two noise-weight sets that hash to one bucket share warps; the shared form sees the
    mismatch and hands those candidates to the per-candidate form: results unchanged."""
    base = synth.eight_state(n=96, time=1500, freq=60, pool=1, observer="kalman")
    q = base.cuda_mx[0, 18:26].copy()
    seen, pair = {}, None
    for k in range(1, 20000):
        r = np.float32(0.05 + 1e-4 * k)
        b = _bucket(r, q)
        if b in seen:
            pair = (seen[b], r)
            break
        seen[b] = r
    assert pair is not None
    g = base.cuda_mx.copy()
    g[:48, 17] = pair[0]
    g[48:, 17] = pair[1]
    g = g[np.random.default_rng(0).permutation(96)]
    p = synth.Problem(base.name, base.config_text, base.plant, g, base.info_mx)
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant) as s:
        for kernel in ("specialised", "table"):
            s.set_sim_kernel(kernel)
            _, d = s.evaluate_diagnostics(p.cuda_mx, p.info_mx, want=("yplant",))
            y_o = oracle_mod.Oracle(p.config_text, p.plant).sim(p.cuda_mx)
            assert _eq(d["yplant"], y_o), f"{kernel}: {_mismatch(d['yplant'], y_o)} mismatches"


def test_kalman_file_boundary(tmp_path):
    """RunControllerEngine() with `observer = kalman` in ControllerEngine.config."""
    p = synth.eight_state(n=1536, time=1200, freq=60, pool=5, observer="kalman")
    p.write(tmp_path)
    assert ce.run_controller_engine(tmp_path) == 0
    cfg = ce.EngineConfig.parse(p.config_text)
    out = np.fromfile(tmp_path / "INFO_MX_OUT.bin", np.float32).reshape(-1, cfg.info_mx_width)
    with ce.Session(cfg, p.plant) as s:
        ref = s.evaluate(p.cuda_mx, p.info_mx)
    assert np.array_equal(_bits(out), _bits(ref))


def test_kalman_server_and_chunks():
    """Served requests of assorted sizes, and one chunked batch against its pieces: every row
    equals the same candidates evaluated alone (the grouping is per evaluation)."""
    p = synth.eight_state(n=40000, time=800, freq=40, pool=6, observer="kalman")
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant) as s:
        whole = s.evaluate(p.cuda_mx, p.info_mx)
        parts = np.vstack([s.evaluate(p.cuda_mx[a:a + 10000], p.info_mx[a:a + 10000]) for a in range(0, 40000, 10000)])
    assert np.array_equal(_bits(whole), _bits(parts))
    cuts = [0, 37, 3037, 3100, 9000]
    with ce.Server(cfg, p.plant, max_batch=4096, lanes=2) as srv:
        reqs = [srv.submit(p.cuda_mx[a:b], p.info_mx[a:b]) for a, b in zip(cuts, cuts[1:])]
        got = np.vstack([r.wait() for r in reqs])
    assert np.array_equal(_bits(got), _bits(whole[:9000]))


def test_kalman_graph_capture():
    import torch
    p = synth.eight_state(n=2048, time=1000, freq=40, pool=4, observer="kalman")
    cfg = ce.EngineConfig.parse(p.config_text)
    n = p.cuda_mx.shape[0]
    with ce.Session(cfg, p.plant) as s:
        ref = s.evaluate(p.cuda_mx, p.info_mx)
        dg = torch.from_numpy(p.cuda_mx).cuda()
        di = torch.from_numpy(p.info_mx).cuda()
        do = torch.empty_like(di)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            s.evaluate_device(n, dg.data_ptr(), di.data_ptr(), do.data_ptr(), stream=side.cuda_stream)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            s.evaluate_device(n, dg.data_ptr(), di.data_ptr(), do.data_ptr(),
                              stream=torch.cuda.current_stream().cuda_stream)
        do.zero_()
        graph.replay()
        torch.cuda.synchronize()
    assert np.array_equal(_bits(do.cpu().numpy()), _bits(ref))
