"""Trackers: device buffers filled inside the step loop, host-side outputs.

Mirrors ``core/tracker/`` and the activation-time, local-activation-time and
probe trackers of the reference.  ``Tracker.track`` in the reference runs
after the ionic kernel and before the buffer swap, on steps where
``start_time <= t <= end_time`` and ``step % self.step == 0``
(``core/tracker/tracker.py:70-83``).  Here the model turns that condition
into a window of step indices (``fwgpu.h: fw_window``) and the kernels do
the per-node work; ``output`` converts the device record into the
reference's output format on demand.
"""
import copy
from pathlib import Path

import numpy as np
import torch

from . import _ffi


class Tracker:
    """Base tracker (core/tracker/tracker.py:8-101)."""

    def __init__(self):
        self.model = None
        self.file_name = "tracked_data"
        self.path = "."
        self.start_time = 0
        self.end_time = np.inf
        self.step = 1

    def initialize(self, model):
        raise NotImplementedError

    def _track(self):
        """Record one sample (the reference's abstract ``Tracker._track``).
        This package's own trackers record inside the kernels instead; a
        user subclass that implements ``_track`` runs on the host."""
        raise NotImplementedError

    def track(self):
        """Call ``_track`` on the steps where the tracker is active
        (core/tracker/tracker.py:70-83): start_time <= t <= end_time and
        step % self.step == 0."""
        if self.start_time > self.model.t or self.model.t > self.end_time:
            return
        if self.model.step % self.step != 0:
            return
        self._track()

    def clone(self):
        return copy.deepcopy(self)

    def write(self):
        np.save(Path(self.path, self.file_name).with_suffix(".npy"),
                self.output)

    # -- scheduling ------------------------------------------------------
    def _window(self, ts, n0):
        """Active steps of this tracker among steps n0.. with times ts:
        (first, last, count) or None."""
        ns = n0 + np.arange(len(ts), dtype=np.int64)
        ok = (self.start_time <= ts) & (ts <= self.end_time)
        ok &= (ns % int(self.step)) == 0
        if not ok.any():
            return None
        idx = np.flatnonzero(ok)
        return int(ns[idx[0]]), int(ns[idx[-1]]), int(idx.size)


class TrackerSequence:
    """Ordered list of trackers (core/tracker/tracker_sequence.py)."""

    def __init__(self):
        self.sequence = []
        self.model = None

    def initialize(self, model):
        self.model = model
        for tracker in self.sequence:
            tracker.initialize(model)

    def add_tracker(self, tracker):
        self.sequence.append(tracker)

    def remove_trackers(self):
        self.sequence = []


class ActivationTime2DTracker(Tracker):
    """First time each node's u exceeds ``threshold``
    (cpuwave2D/tracker/activation_time_2d_tracker.py:7-75).

    The device keeps the step index of the first crossing (int32, -1 when
    none); ``act_t`` maps it to the model time of that step.
    """

    def __init__(self):
        super().__init__()
        self.threshold = -40
        self.file_name = "act_time_2d"
        self._act_step = None

    def initialize(self, model):
        self.model = model
        self._act_step = torch.full(model._shape(), -1, dtype=torch.int32,
                                    device=model._device())
        self._np_dtype = model._np_dtype()

    @property
    def act_t(self):
        if self._act_step is None:
            return np.ndarray
        steps = self._act_step.cpu().numpy()
        times = self.model._time_of_steps(np.maximum(steps, 0))
        out = np.where(steps >= 0, times, -1.0)
        return out.astype(self._np_dtype)

    @property
    def output(self):
        return self.act_t


class ActivationTime3DTracker(ActivationTime2DTracker):
    """(cpuwave3D/tracker/activation_time_3d_tracker.py)"""

    def __init__(self):
        super().__init__()
        self.file_name = "act_time_3d"


class LocalActivationTime2DTracker(Tracker):
    """Every threshold crossing of every node
    (cpuwave2D/tracker/local_activation_time_2d_tracker.py:6-101).

    The device records each node's crossing steps (up to ``capacity`` per
    node); ``output`` rebuilds the reference's list of layers: a new layer
    starts whenever a crossing node already has a time in the last layer.
    """

    def __init__(self):
        super().__init__()
        self.threshold = -40
        self.file_name = "local_act_time_2d"
        self.capacity = 64

    def initialize(self, model):
        self.model = model
        shape = model._shape()
        dev = model._device()
        n = int(np.prod(shape))
        self._n = n
        self._shape = shape
        self._activated = torch.zeros(n, dtype=torch.uint8, device=dev)
        self._count = torch.zeros(n, dtype=torch.int32, device=dev)
        self._steps = torch.zeros((int(self.capacity), n), dtype=torch.int32,
                                  device=dev)
        self._np_dtype = model._np_dtype()

    @property
    def act_t(self):
        count = self._count.cpu().numpy()
        if (count > self.capacity).any():
            raise RuntimeError(
                "LocalActivationTimeTracker: a node crossed the threshold "
                f"more than capacity={self.capacity} times; raise capacity")
        steps = self._steps.cpu().numpy()
        cells = np.concatenate([np.flatnonzero(count > k)
                                for k in range(int(count.max(initial=0)))]
                               ) if count.max(initial=0) > 0 else np.zeros(0, np.int64)
        ks = np.concatenate([np.full(int((count > k).sum()), k)
                             for k in range(int(count.max(initial=0)))]
                            ) if count.max(initial=0) > 0 else np.zeros(0, np.int64)
        ev_steps = steps[ks, cells] if cells.size else np.zeros(0, np.int32)
        order = np.lexsort((cells, ev_steps))
        ev_steps, cells = ev_steps[order], cells[order]
        layers = [-np.ones(self._n)]
        last = np.full(self._n, -1, dtype=np.int64)
        g = 0
        if cells.size:
            bounds = np.flatnonzero(np.diff(ev_steps)) + 1
            starts = np.concatenate([[0], bounds])
            ends = np.concatenate([bounds, [cells.size]])
            times = self.model._time_of_steps(ev_steps[starts])
            for s, e, t in zip(starts, ends, times):
                c = cells[s:e]
                if (last[c] == g).any():
                    g += 1
                    layers.append(-np.ones(self._n))
                layers[g][c] = t
                last[c] = g
        return [lay.reshape(self._shape) for lay in layers]

    @property
    def output(self):
        return np.array(self.act_t)


class LocalActivationTime3DTracker(LocalActivationTime2DTracker):
    """(cpuwave3D/tracker/local_activation_time_3d_tracker.py)"""

    def __init__(self):
        super().__init__()
        self.file_name = "local_act_time_3d"


class _ProbeTracker(Tracker):
    """Values of variables at given cells on every active step."""

    def _vars(self):
        raise NotImplementedError

    def initialize(self, model):
        self.model = model
        names = ["u"] + list(model._state_names)
        for var in self._vars():
            if var not in names:
                raise ValueError(f"Variable '{var}' not found in model.")
        self._var_ids = [names.index(v) for v in self._vars()]
        cells = np.atleast_2d(np.asarray(self.cell_ind, dtype=np.int64))
        shape = model._shape()
        if cells.shape[1] != len(shape):
            raise ValueError(f"cell_ind must hold {len(shape)} indices per "
                             "cell")
        for d, n in enumerate(shape):
            if ((cells[:, d] < -n) | (cells[:, d] >= n)).any():
                raise IndexError("cell_ind out of bounds")
        flat = np.ravel_multi_index(tuple((cells % np.array(shape)).T), shape)
        self._cells = torch.as_tensor(flat.astype(np.int64),
                                      device=model._device())
        self._n_cells = len(flat)
        self._chunks = []
        self._samples = 0
        self._np_dtype = model._np_dtype()

    def _reserve(self, count):
        nv = len(self._var_ids)
        buf = torch.empty((count, nv, self._n_cells), dtype=torch.float64,
                          device=self.model._device())
        self._chunks.append(buf)
        return buf

    def _collect(self):
        if not self._chunks:
            return np.zeros((0, len(self._var_ids), self._n_cells))
        return torch.cat(self._chunks).cpu().numpy()


class ActionPotential2DTracker(_ProbeTracker):
    """u at ``cell_ind`` (cpuwave2D/tracker/action_potential_2d_tracker.py)."""

    def __init__(self):
        super().__init__()
        self.cell_ind = [1, 1]
        self.file_name = "act_pot"

    def _vars(self):
        return ["u"]

    @property
    def output(self):
        return np.squeeze(self._collect()[:, 0, :].astype(self._np_dtype))


class ActionPotential3DTracker(ActionPotential2DTracker):
    """(cpuwave3D/tracker/action_potential_3d_tracker.py)"""

    def __init__(self):
        super().__init__()
        self.cell_ind = [1, 1, 1]


class MultiVariable2DTracker(_ProbeTracker):
    """Several state variables at ``cell_ind``
    (cpuwave2D/tracker/multi_variable_2d_tracker.py)."""

    def __init__(self):
        super().__init__()
        self.var_list = []
        self.cell_ind = [1, 1]
        self.dir_name = "multi_vars"

    def _vars(self):
        return list(self.var_list)

    @property
    def output(self):
        data = self._collect()
        return {var: np.squeeze(data[:, i, :].astype(self._np_dtype))
                for i, var in enumerate(self.var_list)}

    def write(self):
        if not Path(self.path, self.dir_name).is_dir():
            Path(self.path, self.dir_name).mkdir(parents=True)
        out = self.output
        for var in self.var_list:
            np.save(Path(self.path, self.dir_name, f"{var}.npy"), out[var])


class MultiVariable3DTracker(MultiVariable2DTracker):
    """(cpuwave3D/tracker/multi_variable_3d_tracker.py)"""

    def __init__(self):
        super().__init__()
        self.cell_ind = [1, 1, 1]


class Variable2DTracker(MultiVariable2DTracker):
    """One variable at ``cell_ind`` (cpuwave2D/tracker/variable_2d_tracker.py)."""

    @property
    def var_name(self):
        return self.var_list[0]

    @var_name.setter
    def var_name(self, value):
        self.var_list = [value]

    @property
    def output(self):
        return MultiVariable2DTracker.output.fget(self)[self.var_name]

    def write(self):
        if not Path(self.path, self.dir_name).exists():
            Path(self.path, self.dir_name).mkdir(parents=True)
        np.save(Path(self.path, self.dir_name, self.var_name).with_suffix(
            ".npy"), self.output)


class Variable3DTracker(Variable2DTracker):
    """(cpuwave3D/tracker/variable_3d_tracker.py)"""

    def __init__(self):
        super().__init__()
        self.cell_ind = [1, 1, 1]


class ECG2DTracker(Tracker):
    """Pseudo-ECG at measurement points (cpuwave2D/tracker/ecg_2d_tracker.py:
    6-153): on each tracked step, for every point (x, y, z) the sum over
    myocytes (i, j) of (diffuse(u) - u) / (d * dr) with
    d = (x - i)^2 + (y - j)^2 + z^2.  Computed on the device by a reduction
    kernel (fw_ecg_tracker); the model runs in the plain form while one is
    attached.  ``output`` is the (samples, points) array."""

    def __init__(self, measure_coords=None):
        super().__init__()
        self.measure_coords = measure_coords
        self.file_name = "ecg.npy"
        self._chunks = []

    def initialize(self, model):
        self.model = model
        self.measure_coords = np.atleast_2d(
            np.asarray(self.measure_coords, dtype=np.float64))
        if self.measure_coords.shape[1] != 3:
            raise ValueError("measure_coords must hold (x, y, z) per point")
        if not 1 <= len(self.measure_coords) <= _ffi.MAX_ECG_LEADS:
            raise ValueError(f"1..{_ffi.MAX_ECG_LEADS} measurement points")
        self._chunks = []

    def _reserve(self, count):
        buf = torch.zeros((count, len(self.measure_coords)),
                          dtype=torch.float64, device=self.model._device())
        self._chunks.append(buf)
        return buf

    @property
    def output(self):
        if not self._chunks:
            return np.zeros((0, len(np.atleast_2d(self.measure_coords))))
        return torch.cat([c.cpu() if c.is_cuda else c
                          for c in self._chunks]).numpy()

    def write(self):
        Path(self.path).mkdir(parents=True, exist_ok=True)
        np.save(Path(self.path).joinpath(self.file_name).with_suffix(".npy"),
                self.output)


class ECG3DTracker(ECG2DTracker):
    """(cpuwave3D/tracker/ecg_3d_tracker.py: d includes (z - k)^2)"""


class SpiralWaveCore2DTracker(Tracker):
    """Spiral-wave tips (cpuwave2D/tracker/spiral_wave_core_2d_tracker.py:
    9-249): on each tracked step, the cells whose ``threshold`` isoline is
    crossed both at the previous tracked step and now, refined to the
    intersection of the two bilinear isolines.  Found on the device
    (fw_tip_tracker); the model runs in the plain form while one is
    attached.  ``output`` is a pandas DataFrame with columns x, y, time,
    step (x, y, z, time, step in 3D) when pandas is installed, else a dict
    of the same columns as numpy arrays."""

    _columns = ("x", "y")

    def __init__(self):
        super().__init__()
        self.threshold = 0.5
        self.file_name = "spiral_wave_core"
        self.capacity = 1 << 16   # tips held per run() segment

    def initialize(self, model):
        self.model = model
        # the reference copies model.u when the trackers are initialised,
        # before the model sets its initial potential (zeros)
        self._u_prev = model._dev["u"].clone()
        self._count = torch.zeros(1, dtype=torch.int32,
                                  device=model._device())
        self._chunks = []   # (tips tensor, count snapshot, first step, stride)

    def _reserve(self, first, stride):
        self._close_chunk()
        buf = torch.empty((int(self.capacity), 4), dtype=torch.float64,
                          device=self.model._device())
        self._count.zero_()
        self._chunks.append([buf, None, first, stride])
        return buf

    def _close_chunk(self):
        if self._chunks and self._chunks[-1][1] is None:
            self._chunks[-1][1] = self._count.clone()

    def _records(self):
        self._close_chunk()
        recs = []
        for buf, count, first, stride in self._chunks:
            c = int(count.item())
            if c > self.capacity:
                raise RuntimeError("SpiralWaveCore tracker: more tips than "
                                   f"capacity={self.capacity} in one run "
                                   "segment; raise capacity")
            raw = buf[:c].cpu().numpy()
            ints = raw[:, :2].copy().view(np.int32).reshape(c, 4)
            sample, k, i, j = (ints[:, q].astype(np.int64) for q in range(4))
            steps = first + sample * stride
            recs.append((steps, k, i, j, raw[:, 2], raw[:, 3]))
        if not recs:
            z = np.zeros(0)
            return (z.astype(np.int64),) * 4 + (z, z)
        return tuple(np.concatenate(c) for c in zip(*recs))

    @property
    def output(self):
        steps, k, i, j, x, y = self._records()
        order = np.lexsort((j, i, k, steps))
        steps, k, x, y = steps[order], k[order], x[order], y[order]
        times = self.model._time_of_steps(steps) if steps.size else \
            np.zeros(0)
        cols = {"x": x, "y": y}
        if len(self._columns) == 3:
            cols["z"] = k
        cols["time"] = times
        cols["step"] = steps
        try:
            import pandas as pd
        except ImportError:
            return cols
        return pd.DataFrame(cols)

    def write(self):
        out = self.output
        path = Path(self.path, self.file_name).with_suffix(".csv")
        if hasattr(out, "to_csv"):
            out.to_csv(path)
        else:
            names = list(out)
            np.savetxt(path, np.column_stack([out[n] for n in names]),
                       delimiter=",", header=",".join(names), comments="")


class SpiralWaveCore3DTracker(SpiralWaveCore2DTracker):
    """(cpuwave3D/tracker/spiral_wave_core_3d_tracker.py): the 2D search in
    every z layer; tips carry their layer as z."""

    _columns = ("x", "y", "z")


class Period2DTracker(LocalActivationTime2DTracker):
    """Activation periods at given cells (cpuwave2D/tracker/
    period_2d_tracker.py:7-95): the differences of each cell's successive
    threshold crossings, from the device's crossing record.  ``output`` is a
    pandas Series of arrays (one per cell) when pandas is installed, else a
    list of arrays."""

    def __init__(self):
        super().__init__()
        self.cell_ind = []
        self.file_name = "period"

    def _cells_flat(self):
        cells = np.atleast_2d(np.asarray(self.cell_ind, dtype=np.int64))
        return np.ravel_multi_index(tuple(cells.T), self._shape)

    @property
    def output(self):
        flat = self._cells_flat()
        count = self._count.cpu().numpy()[flat]
        if (count > self.capacity).any():
            raise RuntimeError("Period tracker: a cell crossed the threshold "
                               f"more than capacity={self.capacity} times")
        steps = self._steps.cpu().numpy()[:, flat]
        periods = []
        for c in range(len(flat)):
            t = self.model._time_of_steps(steps[:count[c], c].astype(np.int64))
            periods.append(np.diff(t))
        try:
            import pandas as pd
        except ImportError:
            return periods
        return pd.Series(periods)

    def write(self):
        out = self.output
        path = Path(self.path, self.file_name).with_suffix(".csv")
        if hasattr(out, "to_csv"):
            out.to_csv(path)
        else:
            with open(path, "w") as f:
                for c, p in enumerate(out):
                    f.write(f"{c}," + ",".join(repr(float(x)) for x in p) + "\n")


class Period3DTracker(Period2DTracker):
    """(cpuwave3D/tracker/period_3d_tracker.py)"""


_NATIVE = (ActivationTime2DTracker, LocalActivationTime2DTracker,
           _ProbeTracker, ECG2DTracker, SpiralWaveCore2DTracker)


def is_native(tracker):
    """True when the kernels record `tracker` themselves: one of this
    package's tracker classes, with neither ``track`` nor ``_track``
    replaced by a subclass.  Any other tracker with the reference's
    interface (``initialize``, ``track`` / ``_track``, ``start_time``,
    ``end_time``, ``step``) runs on the host."""
    return (isinstance(tracker, _NATIVE) and
            type(tracker)._track is Tracker._track and
            type(tracker).track is Tracker.track)
