"""The serving front end (ce_server_*): requests of assorted sizes are packed into
batches per model (on any of its plants), split when larger than a batch, and run on
concurrent lanes;
every request's rows must equal the rows of the same candidates evaluated alone,
bit for bit.  Also: several plants in one server, submissions from several
threads, HBM-budget admission and the latency statistics."""
import dataclasses
import threading

import numpy as np
import pytest

import controllerengine_gb300 as ce

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _alone(prob, plant_files=None, n_plants=1, plant_index=0, rows=slice(None)):
    cfg = ce.EngineConfig.parse(prob.config_text)
    with ce.Session(cfg, plant_files or prob.plant, n_plants=n_plants) as s:
        return s.evaluate(prob.cuda_mx[rows], prob.info_mx[rows], plant_index=plant_index)


def test_mixed_sizes_equal_alone(eight_state_small):
    p = eight_state_small
    cfg = ce.EngineConfig.parse(p.config_text)
    ref = _alone(p)
    cuts = [0, 37, 237, 242, 512]  # 37, 200, 5 and 270 candidates; batches hold 300
    with ce.Server(cfg, p.plant, max_batch=300, lanes=2) as srv:
        reqs = [srv.submit(p.cuda_mx[a:b], p.info_mx[a:b]) for a, b in zip(cuts, cuts[1:])]
        outs = [r.wait() for r in reqs]
        st = srv.stats()
    got = np.vstack(outs)
    assert np.array_equal(_bits(got), _bits(ref))
    assert st["completed"] == 4 and st["capacity"] == 300
    assert st["batched_candidates"] == 512 and st["batches"] >= 2  # the 270-candidate request is split
    assert 0 < st["latency_p50_ms"] <= st["latency_p99_ms"] <= st["latency_max_ms"]


def test_request_larger_than_a_batch_is_split(mass_spring):
    p = mass_spring
    cfg = ce.EngineConfig.parse(p.config_text)
    ref = _alone(p)
    with ce.Server(cfg, p.plant, max_batch=256, lanes=3) as srv:
        out = srv.submit(p.cuda_mx, p.info_mx).wait()
        st = srv.stats()
    assert np.array_equal(_bits(out), _bits(ref))
    assert st["batches"] == 6  # 1536 candidates in batches of 256


def _two_plants(p):
    """The mass-spring plant twice, the second copy with another cubic stiffness (BASE_PARAMS[0])."""
    pl = p.plant
    bp2 = pl.base_params.copy()
    bp2[0] *= 3.0
    stack = lambda a: np.concatenate([a.ravel(), a.ravel()])
    return dataclasses.replace(pl, discrete_a=stack(pl.discrete_a), discrete_a_i=stack(pl.discrete_a_i),
                               discrete_bu=stack(pl.discrete_bu), discrete_bw=stack(pl.discrete_bw),
                               discrete_c=stack(pl.discrete_c), base_params=np.concatenate([pl.base_params, bp2]))


def test_two_plants_in_one_server(mass_spring):
    p = mass_spring
    cfg = ce.EngineConfig.parse(p.config_text)
    pl2 = _two_plants(p)
    refs = [_alone(p, pl2, 2, k) for k in range(2)]
    assert not np.array_equal(refs[0], refs[1])  # the plants differ
    with ce.Server(cfg, pl2, n_plants=2, max_batch=512, lanes=2) as srv:
        reqs = [(k, a, srv.submit(p.cuda_mx[a:a + 192], p.info_mx[a:a + 192], plant_index=k))
                for a in range(0, 1536, 192) for k in range(2)]
        for k, a, r in reqs:
            assert np.array_equal(_bits(r.wait()), _bits(refs[k][a:a + 192]))
    # one lane that waits for full batches: requests on both plants share every batch
    with ce.Server(cfg, pl2, n_plants=2, max_batch=512, lanes=1, max_wait_us=200000) as srv:
        reqs = [(k, a, srv.submit(p.cuda_mx[a:a + 192], p.info_mx[a:a + 192], plant_index=k))
                for a in range(0, 1536, 192) for k in range(2)]
        for k, a, r in reqs:
            assert np.array_equal(_bits(r.wait()), _bits(refs[k][a:a + 192]))
        assert srv.stats()["batches"] == 6  # 16 x 192 rows in batches of 512


def test_concurrent_submitters(eight_state_small):
    p = eight_state_small
    cfg = ce.EngineConfig.parse(p.config_text)
    ref = _alone(p)
    results, errors = {}, []
    with ce.Server(cfg, p.plant, max_batch=200, lanes=2) as srv:
        def client(t):
            try:
                for a in range(t * 64, 512, 4 * 64):
                    results[a] = srv.submit(p.cuda_mx[a:a + 64], p.info_mx[a:a + 64]).wait()
            except Exception as e:  # reported below
                errors.append(e)
        th = [threading.Thread(target=client, args=(t,)) for t in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
    assert not errors
    got = np.vstack([results[a] for a in sorted(results)])
    assert np.array_equal(_bits(got), _bits(ref))


def test_hbm_budget_admission(eight_state_small):
    p = eight_state_small
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Server(cfg, p.plant, max_batch=65536, lanes=2, hbm_budget_bytes=64 << 20) as srv:
        cap = srv.stats()["capacity"]
        assert 0 < cap < 65536
        out = srv.submit(p.cuda_mx, p.info_mx).wait()
    assert np.array_equal(_bits(out), _bits(_alone(p)))
    with pytest.raises(ce.ControllerEngineError, match="HBM budget"):
        ce.Server(cfg, p.plant, lanes=2, hbm_budget_bytes=1024)


def test_timeout_and_empty_request(mass_spring):
    p = mass_spring
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Server(cfg, p.plant, max_batch=1536) as srv:
        empty = srv.submit(p.cuda_mx[:0], p.info_mx[:0])
        assert empty.wait(0).shape == (0, cfg.info_mx_width)
        r = srv.submit(p.cuda_mx, p.info_mx)
        first = r.wait(0)  # usually still running; either way no error
        out = first if first is not None else r.wait()
    assert np.array_equal(_bits(out), _bits(_alone(p)))


def test_several_models(mass_spring):
    """Two configurations in one server (ce_server_create_models): requests of both
    interleave; each equals its own model's session evaluated alone."""
    from controllerengine_gb300 import synth
    a = mass_spring
    b = synth.random_shape(4, n=600, time=900, freq=60)
    cfg_a, cfg_b = ce.EngineConfig.parse(a.config_text), ce.EngineConfig.parse(b.config_text)
    ref_a, ref_b = _alone(a), _alone(b)
    with ce.Server(None, None, models=[(cfg_a, a.plant, 1), (cfg_b, b.plant, 1)], max_batch=400, lanes=2) as srv:
        reqs = []
        for k in range(6):
            reqs.append((0, k * 256, srv.submit(a.cuda_mx[k * 256:(k + 1) * 256], a.info_mx[k * 256:(k + 1) * 256])))
            reqs.append((1, k * 100, srv.submit(b.cuda_mx[k * 100:(k + 1) * 100], b.info_mx[k * 100:(k + 1) * 100],
                                                model=1)))
        for m, a0, r in reqs:
            ref = ref_a if m == 0 else ref_b
            rows = 256 if m == 0 else 100
            assert np.array_equal(_bits(r.wait()), _bits(ref[a0:a0 + rows]))


def test_fp64_server_equals_fp64_session(mass_spring):
    """Every lane of a server created with the FP64 form runs it; rows equal an FP64 session's."""
    p = mass_spring
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, precision="fp64") as s:
        ref = s.evaluate(p.cuda_mx, p.info_mx)
    mixed = _alone(p)
    with ce.Server(cfg, p.plant, max_batch=700, lanes=2, precision="fp64") as srv:
        got = np.vstack([srv.submit(p.cuda_mx[a:a + 512], p.info_mx[a:a + 512]).wait() for a in range(0, 1536, 512)])
    assert np.array_equal(_bits(got), _bits(ref))
    assert not np.array_equal(_bits(got), _bits(mixed))


@pytest.mark.parametrize("precision", ["compensated", "compensated_df"])
def test_compensated_servers_equal_their_sessions(mass_spring, precision):
    """A server created with a compensated form runs it in every lane; rows equal a session's."""
    p = mass_spring
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, precision=precision) as s:
        ref = s.evaluate(p.cuda_mx, p.info_mx)
    with ce.Server(cfg, p.plant, max_batch=700, lanes=2, precision=precision) as srv:
        got = np.vstack([srv.submit(p.cuda_mx[a:a + 512], p.info_mx[a:a + 512]).wait() for a in range(0, 1536, 512)])
    assert np.array_equal(_bits(got), _bits(ref))


def test_monte_carlo_requests_batch_with_each_other():
    """Monte Carlo requests (row k on plant first + k) of assorted plant ranges are packed into
    the same batches, between ordinary requests on one plant; every row equals ce_evaluate_plants
    (or ce_evaluate for the ordinary ones)."""
    from controllerengine_gb300 import synth
    p = synth.monte_carlo(n_plants=600, time=900, freq=50, serial=True)
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, n_plants=600) as s:
        ref_mc = s.evaluate_plants(p.cuda_mx, p.info_mx)
        ref_one = s.evaluate(p.cuda_mx[:90], p.info_mx[:90], plant_index=7)
    ranges = [(0, 120), (300, 450), (120, 125), (500, 600), (125, 300)]
    with ce.Server(cfg, p.plant, n_plants=600, max_batch=256, lanes=2) as srv:
        reqs = []
        for k, (a, b) in enumerate(ranges):
            reqs.append(("mc", a, b, srv.submit_plants(p.cuda_mx[a:b], p.info_mx[a:b], first_plant=a)))
            if k % 2 == 0:
                reqs.append(("one", 0, 90, srv.submit(p.cuda_mx[:90], p.info_mx[:90], plant_index=7)))
        for kind, a, b, r in reqs:
            out = r.wait()
            ref = ref_mc[a:b] if kind == "mc" else ref_one
            assert np.array_equal(_bits(out), _bits(ref)), (kind, a, b)
        st = srv.stats()
    assert st["batches"] < len(reqs)  # Monte Carlo requests of different plant ranges shared batches
    with ce.Server(cfg, p.plant, n_plants=600, max_batch=256, lanes=1) as srv:
        with pytest.raises(ce.ControllerEngineError, match="exceed the model"):
            srv.submit_plants(p.cuda_mx[:10], p.info_mx[:10], first_plant=595)


def test_monte_carlo_batch_in_two_chunks():
    """A Monte Carlo batch of 40,000 rows runs as two chunks; in serial mode every row's sweep
    reads its own plant's grid, in the second chunk as in the first."""
    from controllerengine_gb300 import synth
    p = synth.monte_carlo(n_plants=40000, time=300, freq=40, serial=True)
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, n_plants=40000) as s:
        ref = s.evaluate_plants(p.cuda_mx, p.info_mx)
    with ce.Server(cfg, p.plant, n_plants=40000, max_batch=40000, lanes=1) as srv:
        got = srv.submit_plants(p.cuda_mx, p.info_mx, first_plant=0).wait()
    assert np.array_equal(_bits(got), _bits(ref))


def test_monte_carlo_requests_fp64_server():
    """Monte Carlo requests on a server of the FP64 form equal the FP64 form of
    ce_evaluate_plants, beside ordinary requests."""
    from controllerengine_gb300 import synth
    p = synth.monte_carlo(n_plants=300, time=900, freq=50, serial=True)
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, n_plants=300, precision="fp64") as s:
        ref_mc = s.evaluate_plants(p.cuda_mx, p.info_mx)
        ref_one = s.evaluate(p.cuda_mx[:50], p.info_mx[:50], plant_index=3)
    with ce.Server(cfg, p.plant, n_plants=300, max_batch=128, lanes=2, precision="fp64") as srv:
        a = srv.submit_plants(p.cuda_mx[:200], p.info_mx[:200], first_plant=0)
        b = srv.submit(p.cuda_mx[:50], p.info_mx[:50], plant_index=3)
        c = srv.submit_plants(p.cuda_mx[250:300], p.info_mx[250:300], first_plant=250)
        assert np.array_equal(_bits(a.wait()), _bits(ref_mc[:200]))
        assert np.array_equal(_bits(b.wait()), _bits(ref_one))
        assert np.array_equal(_bits(c.wait()), _bits(ref_mc[250:300]))


def test_request_on_unusable_plant_fails_alone():
    """A plant whose sweep grid failed (here: C = 0, no gain at the crossover) fails the requests
    that name it when they are submitted; requests on the other plants are served."""
    from controllerengine_gb300 import synth
    p = synth.monte_carlo(n_plants=64, time=600, freq=40, serial=True)
    p.plant.discrete_c[5 * 8:6 * 8] = 0.0
    cfg = ce.EngineConfig.parse(p.config_text)
    with ce.Session(cfg, p.plant, n_plants=64) as s:
        ref = s.evaluate_plants(p.cuda_mx[10:], p.info_mx[10:], first_plant=10)
        with pytest.raises(ce.ControllerEngineError, match="crossover"):
            s.evaluate_plants(p.cuda_mx[:10], p.info_mx[:10])
    with ce.Server(cfg, p.plant, n_plants=64, max_batch=256, lanes=1) as srv:
        with pytest.raises(ce.ControllerEngineError, match="plant 5"):
            srv.submit_plants(p.cuda_mx[:10], p.info_mx[:10], first_plant=0)
        with pytest.raises(ce.ControllerEngineError, match="plant 5"):
            srv.submit(p.cuda_mx[:3], p.info_mx[:3], plant_index=5)
        got = srv.submit_plants(p.cuda_mx[10:], p.info_mx[10:], first_plant=10).wait()
    assert np.array_equal(_bits(got), _bits(ref))
