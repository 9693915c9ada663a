"""GPU: a batch of tissues of different models, stencils, sizes, stimuli,
trackers and run lengths advanced together by the persistent ragged kernel
(TissueBatch / fw_batch_run) equals each tissue run on its own in the fused
form with the same region shape and K (cp.async variant, K = 4): every node
is computed by the same float32 expression on the same inputs, whichever
tile or launch computes it, so the comparison is exact."""
import copy

import numpy as np
import pytest
import torch

import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gc():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from finitewave_gb300 import _ffi
    _ffi.load()
    import gpu_cases
    return gpu_cases


def _no_probes(case, keep_at=1):
    """The case's trackers the batch takes (one activation-time tracker),
    plus a local activation tracker at u = 0.5 where it has none, so that
    every tissue also stages and writes back activation flags (with rows
    padded to the pitch in the TMA form)."""
    c = copy.copy(case)
    out, n_at = [], 0
    for t in case.get("trackers", []):
        if t["kind"] == "at":
            if n_at >= keep_at:
                continue
            n_at += 1
        elif t["kind"] != "lat":
            continue
        out.append(t)
    if not any(t["kind"] == "lat" for t in out):
        out.append(dict(kind="lat", threshold=0.5))
    c["trackers"] = out
    return c


def _batch_cases():
    """Tissues of every batched kind: AP / MS / FK, iso5 / aniso9, sizes
    from 34 to 102 nodes a side and a 3 x 200 cable, 600 to 10000 steps."""
    out = [_no_probes(cases.ap2d_cfg1()[0]),
           _no_probes(cases.ap2d_aniso_spiral()[0])]
    for name in ("ms", "fk"):
        for aniso in (False, True):
            out.append(_no_probes(cases.models_2d(name, aniso)[0]))
    cable = _no_probes(cases.trackers_cable()[0])
    out.append(cable)
    st = _no_probes(cases.stimuli_2d()[0])
    out.append(st)
    return out


def _outputs(model, objs):
    r = {"u": model.u, "step": model.step, "t": model.t}
    for name in model._state_names:
        r[name] = getattr(model, name)
    r["trackers"] = [o.output for o in objs]
    return r


def _same(a, b, where):
    if isinstance(a, list):
        assert len(a) == len(b), where
        for i, (x, y) in enumerate(zip(a, b)):
            _same(x, y, f"{where}[{i}]")
    elif isinstance(a, dict):
        assert a.keys() == b.keys(), where
        for k in a:
            _same(a[k], b[k], f"{where}.{k}")
    else:
        assert np.array_equal(np.asarray(a), np.asarray(b)), where


@pytest.mark.parametrize("kernel", ["tma", "pairs", "cp.async"])
def test_batch_equals_single_fused(gc, kernel):
    import finitewave_gb300 as fg
    cs = _batch_cases()
    single = []
    for c in cs:
        m, objs = gc.build(c, npfloat="float32", form="fused", fused_k=4,
                           fused_variant=1)
        m.run()
        single.append(_outputs(m, objs))
    built = [gc.build(c, npfloat="float32") for c in cs]
    batch = fg.TissueBatch([m for m, _ in built], kernel=kernel)
    launches0 = fg._ffi.load().fw_launch_count()
    batch.run()
    torch.cuda.synchronize()
    assert fg._ffi.load().fw_launch_count() > launches0
    assert batch._batch.kernel == {"tma": 2, "pairs": 3, "cp.async": 1}[kernel]
    for i, ((m, objs), ref) in enumerate(zip(built, single)):
        got = _outputs(m, objs)
        assert got["step"] == ref["step"] and got["t"] == ref["t"], i
        _same(got, ref, f"tissue {i}")


def test_batch_rejects_unsupported(gc):
    import finitewave_gb300 as fg
    case, _ = cases.ap2d_aniso_spiral()   # has probe trackers
    m, _ = gc.build(case, npfloat="float32")
    with pytest.raises(ValueError, match="probe"):
        fg.TissueBatch([m]).run()
    case, _ = cases.ap2d_cfg1()
    m, _ = gc.build(case, npfloat="float64")
    with pytest.raises(ValueError, match="float32"):
        fg.TissueBatch([m]).run()


class _Restimulate:
    """Command: u = 1 on the first interior columns at time t."""

    def __init__(self, t):
        self.t, self.passed = t, False

    def update_status(self, model):
        self.passed = model.t >= self.t
        return self.passed

    def execute(self, model):
        model.u[1:-1, 1:4] = 1.0


def test_batch_graph_chunks_equal_direct(gc):
    """Fixed chunks replayed from captured CUDA graphs give the same result
    as direct launches (and as one long run)."""
    import finitewave_gb300 as fg
    cs = _batch_cases()[:4]
    out = []
    for chunk, graphs in ((None, False), (150, False), (150, True)):
        built = [gc.build(c, npfloat="float32") for c in cs]
        b = fg.TissueBatch([m for m, _ in built], chunk=chunk, graphs=graphs)
        # a command on the first tissue rewrites part of its potential in
        # mid-run: its state must leave the batch's row-padded copies for
        # the command and return afterwards
        seq = fg.CommandSequence()
        seq.add_command(_Restimulate(3.0))
        built[0][0].command_sequence = seq
        b.run()
        torch.cuda.synchronize()
        if graphs:
            assert b._graphs, "no graph was captured"
        out.append([_outputs(m, o) for m, o in built])
    for i in range(len(cs)):
        _same(out[1][i], out[0][i], f"chunked {i}")
        _same(out[2][i], out[0][i], f"graphs {i}")
