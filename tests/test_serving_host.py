"""CPU: the serving loop's scheduling (SimulationServer.serve) with fake
models and a fake CUDA stream -- admission by the HBM budget, requests
waiting for memory and admitted as it frees up (continuous batching),
rejection of requests larger than the budget, chunked advancing to each
request's own step count, and the statistics.  No device work happens: the
fake model only records which requests advanced in each scheduling round.
"""

import numpy as np
import pytest
import torch

from finitewave_gb300 import serving


class _FakeStream:
    def __init__(self, log):
        self.log = log

    def wait_stream(self, other):
        pass

    def synchronize(self):
        # the server synchronises the compute stream once per scheduling
        # round, after advancing every active request
        self.log.append("|")


class _FakeModel:
    dt = 0.5

    def __init__(self, name, steps, log):
        self.name = name
        self.t = 0.0
        self.t_max = steps * self.dt
        self.log = log
        self.initialized = 0
        self.state_loader = None
        self.state_saver = None
        self.command_sequence = None
        self.tracker_sequence = None
        self._myo_d = torch.ones(10, dtype=torch.int8)
        self.advanced = []

    def initialize(self):
        self.initialized += 1

    def _run_segment(self, n, sync=True):
        assert not sync
        self.advanced.append(n)
        self.log.append(self.name)
        return n

    def check_termination(self):
        return False

    def _check_status(self):
        pass


@pytest.fixture
def fake_cuda(monkeypatch):
    log = []
    stream = _FakeStream(log)
    monkeypatch.setattr(torch.cuda, "Stream", lambda *a, **k: _FakeStream([]))
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a, **k: stream)
    monkeypatch.setattr(torch.cuda, "current_device", lambda: 0)
    sizes = {}
    monkeypatch.setattr(serving, "device_footprint", lambda m: sizes[m.name])
    return log, sizes


def _rounds(log):
    out, cur = [], []
    for e in log:
        if e == "|":
            out.append(cur)
            cur = []
        else:
            cur.append(e)
    return out


def test_admission_by_budget_and_chunks(fake_cuda):
    log, sizes = fake_cuda
    steps = {"a": 7, "b": 3, "c": 5, "big": 2}
    models = {k: _FakeModel(k, v, log) for k, v in steps.items()}
    sizes.update(a=40, b=40, c=40, big=1000)
    reqs = [serving.Request(models[k], arrival=0.0, name=k)
            for k in ("a", "b", "c", "big")]
    srv = serving.SimulationServer(hbm_budget=100, chunk=2)
    done = srv.serve(reqs, realtime=False)

    # the oversized request is rejected, the others all complete
    assert [r.name for r in srv.rejected] == ["big"]
    assert sorted(r.name for r in done) == ["a", "b", "c"]
    # at most two 40-byte requests fit the 100-byte budget at once
    rounds = _rounds(log)
    assert all(len(r) <= 2 for r in rounds)
    assert len(rounds[0]) == 2
    # c waits for memory and is admitted once b (3 steps = 2 rounds) leaves
    first_c = next(i for i, r in enumerate(rounds) if "c" in r)
    last_b = max(i for i, r in enumerate(rounds) if "b" in r)
    assert first_c == last_b + 1
    # every request advances exactly its own step count, in chunks of <= 2
    for k in ("a", "b", "c"):
        m = models[k]
        assert sum(m.advanced) == steps[k]
        assert all(0 < n <= 2 for n in m.advanced)
        assert m.initialized == 1
        # released: device arrays dropped
        assert m._dev == {} and m.weights is None
    assert models["big"].initialized == 0
    # completion order follows the remaining work
    assert [r.name for r in done] == ["b", "a", "c"]
    for r in done:
        assert r.steps == steps[r.name]
        assert r.arrival <= r.admitted <= r.finished


def test_stats(fake_cuda):
    log, sizes = fake_cuda
    models = [_FakeModel(str(i), 2 + i, log) for i in range(5)]
    for m in models:
        sizes[m.name] = 10
    srv = serving.SimulationServer(hbm_budget=1000, chunk=3)
    srv.serve([serving.Request(m, arrival=0.0, name=m.name) for m in models],
              realtime=False)
    st = srv.stats()
    assert st["completed"] == 5 and st["rejected"] == 0
    lat = np.array([r.latency for r in srv.completed])
    assert st["latency_p50_s"] == pytest.approx(np.percentile(lat, 50))
    assert st["latency_p99_s"] == pytest.approx(np.percentile(lat, 99))
    assert st["latency_p50_s"] <= st["latency_p99_s"]
    # myocyte-steps: 10 myocytes per fake tissue
    assert st["myocyte_steps"] == 10 * sum(2 + i for i in range(5))
    empty = serving.SimulationServer(hbm_budget=1).stats()
    assert empty == {"completed": 0, "rejected": 0}
