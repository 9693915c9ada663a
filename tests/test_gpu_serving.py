"""GPU: the request loop (SimulationServer) serves a mixed trace -- TP06,
Courtemanche, Aliev-Panfilov and Fenton-Karma, 2D and 3D, float32 and
float64 -- under an HBM budget that forces queueing, and every request's
tracker outputs equal those of the same model run alone; requests on their
own streams run on the device at the same time (their device spans
overlap) and still give each request's results alone, bit for bit."""
import copy

import numpy as np
import pytest
import torch

import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    import finitewave_gb300 as fg
    fg._ffi.load()
    import gpu_cases
    return fg, gpu_cases


def _trace_cases():
    tp06, _ = cases.tp06(2)
    crn, _ = cases.courtemanche(3)
    ap, _ = cases.ap2d_cfg1()
    fk, _ = cases.models_2d("fk", True)
    out = []
    for c, prec in ((tp06, "float32"), (crn, "float64"), (ap, "float32"),
                    (fk, "float64"), (copy.deepcopy(tp06), "float64")):
        c = copy.copy(c)
        c["t_max"] = min(c["t_max"], 12)
        c["trackers"] = [dict(kind="at", threshold=0.5 if c["model"] in
                              ("ap", "fk") else -20.0)] + \
            [t for t in c.get("trackers", []) if t["kind"] == "probe"]
        out.append((c, prec))
    return out


def test_serving_matches_alone(env):
    fg, gc = env
    alone = []
    for c, prec in _trace_cases():
        m, objs = gc.build(c, npfloat=prec)
        m.run()
        alone.append([copy.deepcopy(o.output) for o in objs])
    reqs, objs_all = [], []
    for i, (c, prec) in enumerate(_trace_cases()):
        m, objs = gc.build(c, npfloat=prec)
        reqs.append(fg.Request(m, arrival=0.001 * i, name=str(i)))
        objs_all.append(objs)
    fp = [fg.device_footprint(r.model) for r in reqs]
    # room for the two largest only: later requests wait for admission
    budget = sum(sorted(fp)[-2:])
    server = fg.SimulationServer(hbm_budget=budget, chunk=250)
    done = server.serve(reqs, realtime=False)
    assert len(done) == len(reqs) and not server.rejected
    st = server.stats()
    assert st["completed"] == len(reqs)
    assert st["latency_p99_s"] >= st["latency_p50_s"] > 0
    assert any(r.queueing > 0 for r in reqs)
    for i, (objs, ref) in enumerate(zip(objs_all, alone)):
        assert reqs[i].steps > 0
        got = [o.output for o in objs]
        for g, r in zip(got, ref):
            if isinstance(r, dict):
                for k in r:
                    assert np.array_equal(g[k], r[k]), (i, k)
            else:
                assert np.array_equal(np.asarray(g), np.asarray(r)), i


def test_rejects_request_over_budget(env):
    fg, gc = env
    c, _ = cases.ap2d_cfg1()
    m, _ = gc.build(c, npfloat="float32")
    server = fg.SimulationServer(hbm_budget=1024, chunk=100)
    done = server.serve([fg.Request(m)], realtime=False)
    assert done == [] and len(server.rejected) == 1


def _tp06_sheet(fg, n, t_max, seed):
    rng = np.random.default_rng(seed)
    mesh = (1 + (rng.random((n, n)) <= 0.1)).astype(np.int8)
    mesh[0, :] = mesh[-1, :] = mesh[:, 0] = mesh[:, -1] = 0
    tissue = fg.CardiacTissue2D((n, n))
    tissue.mesh = mesh
    m = fg.TP062D()
    m.dt, m.dr, m.t_max = 0.01, 0.25, t_max
    m.npfloat = "float64"
    m.cardiac_tissue = tissue
    seq = fg.StimSequence()
    seq.add_stim(fg.StimCurrentCoord2D(0, 100, 1.0, 0, n, 1, 6))
    m.stim_sequence = seq
    at = fg.ActivationTime2DTracker()
    at.threshold = -20.0
    trs = fg.TrackerSequence()
    trs.add_tracker(at)
    m.tracker_sequence = trs
    return m, at


def test_requests_overlap_on_device(env):
    """Three float64 TP06 sheets, each too small to fill the GPU, served
    together on separate streams: their device spans overlap (the sum of
    the spans exceeds their union) and each request's activation map
    equals its run alone."""
    fg, _ = env
    cfg = [(192, 0.6, 1), (160, 0.6, 2), (176, 0.6, 3)]
    alone = []
    for n, t_max, seed in cfg:
        m, at = _tp06_sheet(fg, n, t_max, seed)
        m.run()
        alone.append(at.output.copy())
    reqs, ats = [], []
    for i, (n, t_max, seed) in enumerate(cfg):
        m, at = _tp06_sheet(fg, n, t_max, seed)
        reqs.append(fg.Request(m, arrival=0.0, name=str(i)))
        ats.append(at)
    server = fg.SimulationServer(chunk=15, streams=4, in_flight=2)
    server.serve(reqs, realtime=False)
    st = server.stats()
    assert st["completed"] == 3
    spans = sorted(server.device_spans(), key=lambda x: x[1])
    assert len(spans) == 3
    assert any(spans[i + 1][1] < spans[i][2] for i in range(2)), spans
    assert st["device_overlap"] > 1.0, st
    for r, at, act in zip(reqs, ats, alone):
        assert r.steps == 60
        assert np.array_equal(at.output, act), r.name
        assert r.snapshot() is not None
