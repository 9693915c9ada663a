"""CPU: the serving loop's scheduling (SimulationServer.serve) with fake
models and stand-in device operations -- admission by the HBM budget,
requests waiting for memory and admitted as it frees up (continuous
batching), rejection of requests larger than the budget, chunked advancing
to each request's own step count, host work after a completed chunk, and
the statistics.  No device work happens: the fake model only records when
it is initialised, advanced and finished.
"""
import contextlib

import numpy as np
import pytest
import torch

from finitewave_gb300 import serving


class _FakeOps:
    """Stand-in for the loop's device operations: every event has completed
    when it is polled, host copies are plain copies."""

    def stream(self):
        return object()

    def using(self, s):
        return contextlib.nullcontext()

    def record(self, s, timing=False):
        return "event"

    def done(self, ev):
        return True

    def wait(self, s, ev):
        pass

    def to_host(self, t, s):
        return t.clone()

    def elapsed_ms(self, a, b):
        return 0.0


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
        self._n_myo = 10
        self._status = torch.zeros(1, dtype=torch.int32)
        self._dev = {"u": None}
        self.weights = "w"
        self.advanced = []

    def initialize(self):
        self.initialized += 1
        self.log.append(("init", self.name))

    def _run_segment(self, n, sync=True):
        assert not sync
        self.advanced.append(n)
        self.log.append(("step", self.name))
        return n

    def check_termination(self):
        return False

    def _check_status(self, st=None):
        self.log.append(("done", self.name))


@pytest.fixture
def fake_cuda(monkeypatch):
    log = []
    monkeypatch.setattr(torch.cuda, "current_device", lambda: 0)
    sizes = {}
    monkeypatch.setattr(serving, "device_footprint", lambda m: sizes[m.name])

    def server(**kw):
        srv = serving.SimulationServer(prep_threads=0, in_flight=1, **kw)
        srv._ops = _FakeOps()
        return srv
    return log, sizes, server


def test_admission_by_budget_and_chunks(fake_cuda):
    log, sizes, server = fake_cuda
    steps = {"a": 7, "b": 3, "c": 5, "big": 2}
    models = {k: _FakeModel(k, v, log) for k, v in steps.items()}
    sizes.update(a=40, b=40, c=40, big=1000)
    reqs = [serving.Request(models[k], arrival=0.0, name=k)
            for k in ("a", "b", "c", "big")]
    srv = server(hbm_budget=100, chunk=2)
    done = srv.serve(reqs, realtime=False)

    # the oversized request is rejected, the others all complete
    assert [r.name for r in srv.rejected] == ["big"]
    assert sorted(r.name for r in done) == ["a", "b", "c"]
    # at most two 40-byte requests are admitted (initialised, not yet
    # released) at any time
    live, most = set(), 0
    for kind, name in log:
        if kind == "init":
            live.add(name)
        elif kind == "done":
            live.discard(name)
        most = max(most, len(live))
    assert most == 2
    # c waits for memory and is admitted once b has been released
    assert log.index(("init", "c")) > log.index(("done", "b"))
    # a and b advance together before that (continuous batching)
    first = [n for k, n in log[:log.index(("done", "b"))] if k == "step"]
    assert set(first) == {"a", "b"}
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
        assert r.arrival <= r.admitted <= r.started <= r.finished


def test_in_flight_limit_and_host_work(fake_cuda):
    """A request with a command sequence runs its commands after each
    completed chunk, before the next chunk is issued."""
    log, sizes, server = fake_cuda

    class _Seq:
        def __init__(self, model):
            self.model = model
            self.seen = []

        def execute_next(self):
            self.seen.append(sum(self.model.advanced))

    m = _FakeModel("cmd", 6, log)
    m.command_sequence = _Seq(m)
    sizes["cmd"] = 10
    srv = server(hbm_budget=100, chunk=2)
    srv.serve([serving.Request(m, name="cmd")], realtime=False)
    assert m.advanced == [2, 2, 2]
    assert m.command_sequence.seen == [2, 4, 6]


def test_stats(fake_cuda):
    log, sizes, server = fake_cuda
    models = [_FakeModel(str(i), 2 + i, log) for i in range(5)]
    for m in models:
        sizes[m.name] = 10
    srv = server(hbm_budget=1000, chunk=3)
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
