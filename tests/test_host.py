"""CPU-side tests: the C ABI library loads and exports what fwgpu.h declares,
argument validation, and the host scheduling logic (stimulus and tracker
windows, time accumulation, LAT layer reconstruction) against naive
restatements of the reference's per-step rules."""
import ctypes
import os
import re

import numpy as np
import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from finitewave_gb300 import _ffi
    return _ffi.load()


def _declared():
    with open(os.path.join(ROOT, "include", "fwgpu.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"FW_API\s+[\w\s\*]+?\b(fw_\w+)\s*\(", src)))


def test_exports_every_declared_symbol(lib):
    names = _declared()
    assert "fw_step" in names and "fw_build_weights" in names
    for name in names:
        assert hasattr(lib, name), name


def test_struct_layout_matches(lib):
    from finitewave_gb300 import _ffi
    for which, st in _ffi._STRUCTS.items():
        assert lib.fw_struct_size(which) == ctypes.sizeof(st)


def test_version_and_model_info(lib):
    from finitewave_gb300 import _ffi
    assert lib.fw_version() >= 100
    assert _ffi.model_info(_ffi.MODEL_AP) == (1, 5)
    assert _ffi.model_info(_ffi.MODEL_FK) == (2, 11)
    assert _ffi.model_info(_ffi.MODEL_TP06) == (19, 49)
    assert _ffi.model_info(_ffi.MODEL_CRN) == (21, 39)
    with pytest.raises(_ffi.FwError) as e:
        _ffi.model_info(99)
    assert e.value.code == _ffi.FW_ERR_UNSUPPORTED


def test_step_rejects_bad_args(lib):
    """Validation happens before any CUDA call, so it runs without a GPU."""
    from finitewave_gb300 import _ffi
    assert lib.fw_step(None, 0, 1, None) == _ffi.FW_ERR_ARG
    a = _ffi.StepArgs()
    a.model, a.stencil, a.precision = _ffi.MODEL_AP, _ffi.ISO5, _ffi.F64
    a.ni, a.nj, a.nk = 10, 10, 1
    rc = lib.fw_step(ctypes.byref(a), 0, 1, None)
    assert rc == _ffi.FW_ERR_ARG
    assert b"missing" in lib.fw_last_error()
    a.stencil = 77
    assert lib.fw_step(ctypes.byref(a), 0, 1, None) == _ffi.FW_ERR_ARG
    a.stencil, a.nk = _ffi.ISO7, 1
    assert lib.fw_step(ctypes.byref(a), 0, 1, None) == _ffi.FW_ERR_ARG
    assert b"does not fit" in lib.fw_last_error()


def _times(t0, dt, n):
    ts, t = [], t0
    for _ in range(n):
        ts.append(t)
        t += dt
    return np.array(ts), t


def test_time_accumulation_matches_python_loop():
    """np.add.accumulate replays `t += dt` exactly (cardiac_model.py:176)."""
    for dt in (0.01, 0.0015, 0.001, 0.02):
        n = 100000
        acc = np.empty(n + 1)
        acc[0] = 0
        acc[1:] = dt
        a = np.add.accumulate(acc)
        ref, last = _times(0, dt, n)
        assert np.array_equal(a[:n], ref)
        assert a[n] == last


def _naive_stim_steps(t_stim, dur, ts):
    passed, out = False, []
    for n, t in enumerate(ts):
        if t >= t_stim and not passed:
            out.append(n)
            passed = t >= t_stim + dur
    return out


@pytest.mark.parametrize("t_stim,dur", [(0, 0.0), (31, 0.0), (5, 0.5),
                                         (2.5, 0.7), (0.004, 0.01)])
def test_stim_windows(t_stim, dur):
    from finitewave_gb300.stimulation import StimCurrentCoord2D
    ts, _ = _times(0, 0.01, 5000)
    expect = _naive_stim_steps(t_stim, dur, ts)
    s = StimCurrentCoord2D(t_stim, 1.0, dur, 0, 3, 0, 3)
    got = []
    # two segments, to cover a window that spans a segment boundary
    cut = expect[len(expect) // 2] if expect else 100
    for lo, hi in ((0, cut), (cut, len(ts))):
        for first, last, _ in s._windows(ts[lo:hi], lo):
            got.extend(range(first, last + 1))
    assert got == expect


def test_tracker_windows():
    from finitewave_gb300.tracker import ActivationTime2DTracker
    ts, _ = _times(0, 0.01, 3000)
    tr = ActivationTime2DTracker()
    tr.start_time, tr.end_time, tr.step = 1.0, 20.0, 7
    first, last, count = tr._window(ts[500:], 500)
    expect = [n for n, t in enumerate(ts) if n >= 500 and 1.0 <= t <= 20.0
              and n % 7 == 0]
    assert (first, last, count) == (expect[0], expect[-1], len(expect))


class _FakeModel:
    def __init__(self, shape, ts):
        self.shape, self.ts = shape, ts

    def _shape(self):
        return self.shape

    def _device(self):
        return torch.device("cpu")

    def _np_dtype(self):
        return np.float64

    def _time_of_steps(self, steps):
        return self.ts[np.asarray(steps)]


def test_lat_layer_reconstruction():
    """Rebuild the reference's LAT layers from per-node crossing lists and
    compare with a direct restatement of local_activation_time_2d_tracker.py
    :58-89 on random crossing sequences."""
    from finitewave_gb300.tracker import LocalActivationTime2DTracker
    rng = np.random.default_rng(3)
    shape = (6, 7)
    n = 42
    nsteps = 400
    ts, _ = _times(0, 0.01, nsteps)
    above = rng.random((nsteps, n)) < 0.08
    # smear crossings into plateaus so nodes cross, stay, return
    for k in range(1, nsteps):
        above[k] |= above[k - 1] & (rng.random(n) < 0.8)
    # reference semantics
    act = [-np.ones(n)]
    activated = np.zeros(n, bool)
    events = [[] for _ in range(n)]
    for k in range(nsteps):
        cross = above[k] & ~activated
        activated = np.where(cross, True, activated)
        back = ~above[k] & activated
        activated = np.where(back, False, activated)
        if np.any(act[-1][cross] > -1):
            act.append(-np.ones(n))
        act[-1] = np.where(cross, ts[k], act[-1])
        for c in np.flatnonzero(cross):
            events[c].append(k)
    tr = LocalActivationTime2DTracker()
    tr.capacity = max(len(e) for e in events)
    tr.initialize(_FakeModel(shape, ts))
    for c, ev in enumerate(events):
        tr._count[c] = len(ev)
        for j, k in enumerate(ev):
            tr._steps[j, c] = k
    out = tr.output
    assert out.shape == (len(act), *shape)
    assert np.array_equal(out, np.array(act).reshape(len(act), *shape))


def test_detailed_model_layout(lib):
    """TP06 / Courtemanche / Luo-Rudy 1991: state and parameter lists agree
    with the library's counts; under float64 every state array is float64,
    under float32 exactly the ion concentrations are compensated pairs."""
    import finitewave_gb300 as fg
    from finitewave_gb300 import _ffi
    conc = {fg.TP062D: {"cai", "casr", "cass", "nai", "Ki"},
            fg.Courtemanche2D: {"nai", "ki", "cai", "caup", "carel"},
            fg.LuoRudy912D: {"cai"}}
    for cls, names in conc.items():
        m = cls()
        ns, npar = _ffi.model_info(m._model_id)
        assert (len(m._state_names), len(m._param_names)) == (ns, npar)
        for i, name in enumerate(m._state_names):
            assert _ffi.state_is_f64(m._model_id, _ffi.F64, i) == 1
            assert _ffi.state_is_f64(m._model_id, _ffi.F32, i) == 0
            assert _ffi.state_is_pair(m._model_id, _ffi.F64, i) == 0
            assert _ffi.state_is_pair(m._model_id, _ffi.F32, i) == \
                (name in names), name
        assert m.state_vars == ["u"] + list(m._state_names)


def test_compensated_pair_split():
    """Host conversion of float64 values to (hi, lo) float32 pairs: hi is
    the value rounded to float32, hi + lo recovers it to ~2^-48."""
    from finitewave_gb300.model import _split_pair
    rng = np.random.default_rng(3)
    v = np.concatenate([rng.uniform(1e-5, 1e-3, 100),
                        rng.uniform(5, 150, 100), [0.0, 1.3, 138.3]])
    p = _split_pair(v)
    assert p.dtype == np.float32 and p.shape == v.shape + (2,)
    assert np.array_equal(p[..., 0], v.astype(np.float32))
    back = p[..., 0].astype(np.float64) + p[..., 1]
    assert np.all(np.abs(back - v) <= np.abs(v) * 2.0 ** -46)


def test_batch_plan_checks(lib):
    """fw_batch_plan_size validates each tissue on the host (no device
    work): supported models / precision / trackers, and sizes the plan by
    the tissues' tile counts."""
    from finitewave_gb300 import _ffi

    def tissue(ni, nj, model=_ffi.MODEL_AP, prec=_ffi.F32, n_probe=0):
        a = _ffi.StepArgs()
        a.model, a.stencil, a.precision = model, _ffi.ISO5, prec
        a.ni, a.nj, a.nk = ni, nj, 1
        a.weights = a.myo = a.u[0] = a.u[1] = 0x1000
        a.state[0] = a.state[1] = 0x1000
        a.state_b[0] = a.state_b[1] = 0x2000
        a.n_probe = n_probe
        return a

    def size(ts):
        arr = (ctypes.c_void_p * len(ts))(*[ctypes.addressof(t) for t in ts])
        out = ctypes.c_int64()
        rc = lib.fw_batch_plan_size(arr, len(ts), ctypes.byref(out))
        return rc, out.value

    rc, one = size([tissue(100, 100)])
    assert rc == _ffi.FW_OK and one > 0
    # the fused batch needs a second buffer per state variable
    t = tissue(100, 100)
    t.state_b[0] = 0
    assert size([t])[0] == _ffi.FW_ERR_ARG
    rc, two = size([tissue(100, 100), tissue(100, 100)])
    assert rc == _ffi.FW_OK and two > one
    rc, big = size([tissue(1000, 1000)])
    assert rc == _ffi.FW_OK and big > one
    assert size([tissue(64, 64, model=_ffi.MODEL_TP06)])[0] == \
        _ffi.FW_ERR_UNSUPPORTED
    assert size([tissue(64, 64, prec=_ffi.F64)])[0] == \
        _ffi.FW_ERR_UNSUPPORTED
    assert size([tissue(64, 64, n_probe=1)])[0] == _ffi.FW_ERR_UNSUPPORTED
    assert size([tissue(2, 64)])[0] == _ffi.FW_ERR_ARG
    nb = ctypes.c_int64()
    assert lib.fw_batch_scratch_size(ctypes.byref(nb)) == _ffi.FW_OK
    assert nb.value >= 8


def test_diffuse_patterns_match_reference():
    """Diffuse2DPattern / Diffuse3DPattern draw the reference's random
    numbers: same seed, same mesh (tests/golden/fibrosis.npz)."""
    import finitewave_gb300 as fg
    g = np.load(os.path.join(ROOT, "tests", "golden", "fibrosis.npz"))
    np.random.seed(2024)
    assert np.array_equal(fg.Diffuse2DPattern(0.3).generate(shape=(20, 30)),
                          g["d2_full"])
    np.random.seed(2025)
    assert np.array_equal(
        fg.Diffuse2DPattern(0.5, 3, 15, 4, 22).generate(shape=(20, 30)),
        g["d2_box"])
    np.random.seed(2026)
    got = fg.Diffuse2DPattern(0.2).generate(mesh=g["d2_mesh_in"].copy())
    assert np.array_equal(got, g["d2_mesh"])
    np.random.seed(2027)
    assert np.array_equal(
        fg.Diffuse3DPattern(2, 10, 1, 8, 0, 5, 0.25).generate((12, 9, 6)),
        g["d3_box"])
    np.random.seed(2028)
    assert np.array_equal(
        fg.Diffuse3DPattern(None, None, None, None, None, None,
                            0.1).generate((8, 7, 6)), g["d3_full"])
    t = fg.CardiacTissue2D((20, 30))
    np.random.seed(2024)
    fg.Diffuse2DPattern(0.3).apply(t)
    ref = g["d2_full"].copy()
    ref[0, :] = ref[-1, :] = ref[:, 0] = ref[:, -1] = 0
    assert np.array_equal(np.asarray(t.mesh), ref)


def test_device_footprint():
    """The admission estimate of the request loop: bytes per node of u,
    u_new, mesh, myo, state (float64 concentrations under float32 for the
    detailed models), weights, packed weights and trackers."""
    import finitewave_gb300 as fg
    t = fg.CardiacTissue2D((50, 40))
    t.fibers = np.zeros((50, 40, 2))
    t.fibers[..., 0] = 1
    m = fg.AlievPanfilov2D()
    m.npfloat = "float32"
    m.cardiac_tissue = t
    trs = fg.TrackerSequence()
    trs.add_tracker(fg.ActivationTime2DTracker())
    m.tracker_sequence = trs
    assert fg.device_footprint(m) == 50 * 40 * (2 * 4 + 2 + 4 + 9 * 4 +
                                                8 * 4 + 4)
    t3 = fg.CardiacTissue3D((10, 12, 14))
    m3 = fg.TP063D()
    m3.npfloat = "float32"
    m3.cardiac_tissue = t3
    assert fg.device_footprint(m3) == 10 * 12 * 14 * (
        2 * 4 + 2 + 5 * 8 + 14 * 4 + 7 * 4)


def test_autotune_cache_logic(tmp_path, monkeypatch):
    """The autotuner's cache without a GPU: the key names the GPU, model
    class, stencil, dimension and size class; a configuration is timed once,
    then served from memory, then from the JSON file; an unreadable file
    means a re-tune, not an error."""
    import json
    import torch
    from finitewave_gb300 import autotune

    path = tmp_path / "tune.json"
    monkeypatch.setenv("FWGPU_AUTOTUNE_CACHE", str(path))
    monkeypatch.setattr(torch.cuda, "get_device_name", lambda dev=None: "GPU-X")
    calls = []

    def fake_tune(model, steps=96):
        calls.append(model)
        return {"variant": 3, "k": 4, "ms": {"3/4": 1.0}, "steps": steps}

    monkeypatch.setattr(autotune, "tune", fake_tune)

    class _Stencil:
        kind = 2

    class AlievPanfilov2D:
        stencil = _Stencil()

        def __init__(self, shape):
            self.shape = shape

        def _shape(self):
            return self.shape

        def _device(self):
            return 0

    m = AlievPanfilov2D((4096, 4096))
    assert autotune.key(m) == "GPU-X|AlievPanfilov2D|2|2D|2^24"
    # the size class is the power of two of the node count
    assert autotune.key(AlievPanfilov2D((4000, 4000))).endswith("|2^23")
    assert autotune.key(AlievPanfilov2D((64, 64, 64))).endswith("|3D|2^18")

    autotune._memo.clear()
    assert autotune.choose(m) == (3, 4) and len(calls) == 1
    assert autotune.choose(m) == (3, 4) and len(calls) == 1       # memory
    table = json.loads(path.read_text())
    assert table[autotune.key(m)]["variant"] == 3
    autotune._memo.clear()
    assert autotune.choose(m) == (3, 4) and len(calls) == 1       # file
    path.write_text("{ not json")
    autotune._memo.clear()
    assert autotune.choose(m) == (3, 4) and len(calls) == 2       # re-tuned
    assert json.loads(path.read_text())[autotune.key(m)]["k"] == 4
    autotune._memo.clear()
    # TMA candidates (variants 3 and 4) come first, cp.async ones after
    assert {v for v, _ in autotune._TMA} == {3, 4}
    assert all(k % 2 == 0 for v, k in autotune._TMA if v == 4)


def _fmaf(a, b, c):
    """float32 fused multiply-add: the exact product (fits float64) plus c,
    rounded to float32 (double rounding at most half an ulp off fmaf)."""
    return (a.astype(np.float64) * b + c).astype(np.float32)


def test_ap_float32_update_rearrangement():
    """The float32 Aliev-Panfilov update of the fused kernels (u - a - 1
    formed once, the cubic as ((u - (a + 1)) u + a) u, FMAs) against the
    reference's expression in float64 (aliev_panfilov_2d.py:133-202) on a
    grid of (u, v, diffusion) values over the model's range: the new v and
    u agree within float32 rounding."""
    f32 = np.float32
    a, k, eap, mu1, mu2 = 0.1, 8.0, 0.01, 0.2, 0.3
    dt = 0.01
    u, v, un = np.meshgrid(np.linspace(-0.1, 1.1, 121),
                           np.linspace(0.0, 2.5, 101),
                           np.array([-0.05, 0.0, 0.3]), indexing="ij")
    # reference, float64
    v64 = v + (-dt) * (eap + (mu1 * v) / (mu2 + u)) * (v + k * u * (u - a - 1.0))
    u64 = (u + un) + dt * ((-k) * u * (u - a) * (u - 1.0) - u * v64)
    # the float32 form
    U, V, UN = (x.astype(f32) for x in (u, v, u + un))
    A, K, EAP, MU1, MU2, DT = (f32(x) for x in (a, k, eap, mu1, mu2, dt))
    ua1 = U - (A + f32(1.0))
    q = (MU1 * V) / (MU2 + U)
    g = _fmaf(K * U, ua1, V)
    V32 = _fmaf((-DT) * (EAP + q), g, V)
    cub = _fmaf(ua1, U, A) * U
    U32 = _fmaf(np.full_like(U, DT), _fmaf(np.full_like(U, -K), cub, -(U * V32)), UN)
    scale_v = np.maximum(np.abs(v64), 1.0)
    scale_u = np.maximum(np.abs(u64), 1.0)
    # about one float32 ulp measured (1.1e-7); two allowed
    assert np.max(np.abs(V32 - v64) / scale_v) < 2.5e-7
    assert np.max(np.abs(U32 - u64) / scale_u) < 2.5e-7


class _HostModel:
    """Stand-in for a model on the host side of commands and checkpoints."""
    state_vars = ["u", "v"]

    def __init__(self, t_max=10.0):
        self.t = 0.0
        self.t_max = t_max
        self.u = np.arange(6.0).reshape(2, 3)
        self.v = -np.arange(6.0).reshape(2, 3)


def test_command_sequence_runs_each_command_once_when_due():
    """core/command/command_sequence.py: a command runs at the first check
    with t >= its time, once; initialize re-arms every command."""
    from finitewave_gb300.command import Command, CommandSequence

    ran = []

    class Mark(Command):
        def execute(self, model):
            ran.append((self.t, model.t))

    m = _HostModel()
    seq = CommandSequence()
    for t in (1.0, 2.0, 3.0):
        seq.add_command(Mark(t))
    seq.initialize(m)
    m.t = 0.5
    seq.execute_next()
    assert ran == []
    m.t = 2.0
    seq.execute_next()
    seq.execute_next()
    assert ran == [(1.0, 2.0), (2.0, 2.0)]
    m.t = 7.0
    seq.execute_next()
    assert [c for c, _ in ran] == [1.0, 2.0, 3.0]
    seq.initialize(m)
    seq.execute_next()
    assert len(ran) == 6
    seq.remove_commands()
    assert seq.sequence == []


def test_state_saver_and_loader_round_trip(tmp_path):
    """core/state/state_saver.py, state_loader.py: one <var>.npy per state
    variable, written once t reaches the saver's time (or t_max for a
    negative time), read back by the loader; an empty path disables both and
    a missing directory is a FileNotFoundError."""
    from finitewave_gb300.state import (StateLoader, StateSaver,
                                        StateSaverCollection)

    m = _HostModel(t_max=5.0)
    end = StateSaver(str(tmp_path / "end"))          # time -1: at the end
    at3 = StateSaver(str(tmp_path / "at3"), time=3.0)
    coll = StateSaverCollection()
    coll.savers = [end, at3]
    coll.initialize(m)
    m.t = 2.0
    coll.save()
    assert not (tmp_path / "end").exists() and not (tmp_path / "at3").exists()
    m.t = 3.0
    coll.save()
    assert (tmp_path / "at3" / "u.npy").exists() and at3.passed
    m.u = m.u + 100.0                                  # later state
    coll.save()                                        # at3 does not re-save
    assert np.array_equal(np.load(tmp_path / "at3" / "u.npy"),
                          np.arange(6.0).reshape(2, 3))
    m.t = 5.0
    coll.save()
    assert np.array_equal(np.load(tmp_path / "end" / "u.npy"), m.u)

    off = StateSaver("")
    off.initialize(m)
    off.save()
    assert off.passed

    m2 = _HostModel()
    m2.u = np.zeros((2, 3))
    m2.v = np.zeros((2, 3))
    loader = StateLoader(str(tmp_path / "at3"))
    loader.initialize(m2)
    loader.load()
    assert np.array_equal(m2.u, np.arange(6.0).reshape(2, 3))
    assert np.array_equal(m2.v, -np.arange(6.0).reshape(2, 3))
    m2.u = None
    loader.load()                                      # once only
    assert m2.u is None
    with pytest.raises(FileNotFoundError):
        StateLoader(str(tmp_path / "missing")).initialize(m2)


def test_tissue_mesh_rules():
    """core/tissue/cardiac_tissue.py and the 2D/3D tissues: assigning a mesh
    zeroes its outer ring, a mesh of the wrong dimension is a ValueError,
    myocyte indices are the flat indices of code 1 outside special
    boundaries, clean() turns fibrosis back into myocytes, clone() copies."""
    import finitewave_gb300 as fg

    t = fg.CardiacTissue2D((5, 6))
    mesh = np.full((5, 6), 1, dtype=np.int8)
    mesh[2, 3] = 2
    t.mesh = mesh
    ring = np.ones((5, 6), bool)
    ring[1:-1, 1:-1] = False
    assert (t.mesh[ring] == 0).all() and t.mesh[2, 3] == 2
    t.compute_myo_indexes()
    want = np.flatnonzero(t.mesh == 1)
    assert np.array_equal(t.myo_indexes, want) and len(want) == 3 * 4 - 1
    t.special_boundaries = np.zeros((5, 6), np.int8)
    t.special_boundaries[1, 1] = 1
    t.compute_myo_indexes()
    assert 1 * 6 + 1 not in t.myo_indexes and len(t.myo_indexes) == 10
    c = t.clone()
    c.clean()
    assert c.mesh[2, 3] == 1 and t.mesh[2, 3] == 2
    with pytest.raises(ValueError):
        t.mesh = np.ones((5, 6, 2), np.int8)

    t3 = fg.CardiacTissue3D((4, 5, 6))
    assert t3.mesh.sum() == 2 * 3 * 4
    assert (t3.mesh[0] == 0).all() and (t3.mesh[:, :, -1] == 0).all()


def test_plugin_classification_and_host_steps():
    """User subclasses with their own ``stimulate`` / ``_track`` / ``track``
    run on the host; this package's classes run in the kernels.  The run
    loop finds the next step on which a host plug-in is due with the
    reference's rules (stim_sequence.py:65-77, tracker.py:70-83)."""
    import finitewave_gb300 as fg
    from finitewave_gb300 import stimulation, tracker

    class MyStim(fg.Stim):
        def initialize(self, model):
            pass

        def stimulate(self, model):
            pass

    class MyCoord(fg.StimVoltageCoord2D):
        def stimulate(self, model):
            pass

    class MyTracker(fg.Tracker):
        def initialize(self, model):
            self.model = model

        def _track(self):
            pass

    class MyAT(fg.ActivationTime2DTracker):
        def _track(self):
            pass

    class EveryStep(fg.Tracker):
        def initialize(self, model):
            self.model = model

        def track(self):
            pass

    assert stimulation.is_native(fg.StimVoltageCoord2D(0, 1, 0, 5, 0, 5))
    assert stimulation.is_native(fg.StimCurrentMatrix2D(0, 1, 1,
                                                        np.ones((4, 4))))
    assert not stimulation.is_native(MyStim(1.0))
    assert not stimulation.is_native(MyCoord(0, 1, 0, 5, 0, 5))
    assert tracker.is_native(fg.ActivationTime2DTracker())
    assert tracker.is_native(fg.MultiVariable2DTracker())
    assert tracker.is_native(fg.Period2DTracker())
    assert not tracker.is_native(MyTracker())
    assert not tracker.is_native(MyAT())
    assert not tracker.is_native(EveryStep())

    m = fg.AlievPanfilov2D()
    m.dt, m.t, m.step = 0.01, 0.0, 0
    s = MyStim(0.5, 0.1)
    assert m._steps_before_host(200, [s], []) == 50
    s.passed = True
    assert m._steps_before_host(200, [s], []) == 200
    tr = MyTracker()
    tr.start_time, tr.step = 0.3, 7
    # first step n with t_n >= 0.3 and n % 7 == 0: t_35 = 0.35 (t_28 < 0.3)
    assert m._steps_before_host(200, [], [tr]) == 35
    m.step, m.t = 35, 0.35
    assert m._steps_before_host(200, [], [tr]) == 0
    assert m._steps_before_host(200, [], [EveryStep()]) == 0


def test_batched_restitution_ranges_match_measurement():
    """The batched configuration draws each tissue's S1-S2 coupling interval
    from its model's restitution range; the ranges in bench.py are the ones
    tests/golden/make_restitution.py measured with the float64 oracle."""
    import importlib.util
    import json
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location(
        "bench_for_test", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    with open(os.path.join(root, "tests", "golden", "restitution.json")) as f:
        meas = json.load(f)["models"]
    for m, (lo, hi) in bench.RESTITUTION.items():
        assert hi == meas[m]["bcl"] == bench.BCL[m]
        assert lo == meas[m]["erp"] and 0 < lo < hi
    specs = bench.batched_specs(64)
    for s in specs:
        lo, hi = bench.RESTITUTION[s["model"]]
        assert lo <= s["ci"] <= hi


def test_restitution_protocol_reproduces_recorded_travel_time():
    """The float64 pacing protocol of tests/golden/make_restitution.py
    (oracle kernels, one thread) reproduces the recorded arrival of the
    first Aliev-Panfilov S1 wave at the probe node, and an S2 one BCL after
    the last S1 is a ninth crossing (a propagated response)."""
    import importlib.util
    import json
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location(
        "make_restitution", os.path.join(root, "tests", "golden",
                                         "make_restitution.py"))
    mr = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mr)
    with open(os.path.join(root, "tests", "golden", "restitution.json")) as f:
        rec = json.load(f)["models"]["ap"]
    first = mr._pace("ap", None, stop_after=mr.BCL["ap"])
    assert first and abs(first[0] - rec["travel_to_probe"]) < 1e-6
    bcl = mr.BCL["ap"]
    late = mr._pace("ap", bcl, stop_after=8 * bcl + 3 * first[0])
    assert len(late) >= 9
