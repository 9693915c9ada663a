"""Stimuli: host-side schedule, device-side application.

Mirrors ``core/stimulation/`` and the 2D / 3D stimulus classes of the
reference.  The reference applies a stimulus from Python on every step where
``model.t >= stim.t and not stim.passed`` and then sets
``passed = model.t >= stim.t + duration`` (``stim_sequence.py:65-77``,
``stim.py:52-56``).  Here the model replays that float64 schedule on the host
and hands each stimulus to the GPU as a window of step indices plus a region
(half-open box, optional node mask), so the stimulus is applied on the
device inside the step loop (``fwgpu.h: fw_stim``).
"""
import numpy as np
import torch

from . import _ffi


class Stim:
    """Base stimulus (core/stimulation/stim.py:4-56)."""

    def __init__(self, time, duration=0.0):
        self.t = time
        self.duration = duration
        self.passed = False

    def initialize(self, model):
        self.passed = False

    def update_status(self, model):
        self.passed = model.t >= (self.t + self.duration)

    def stimulate(self, model):
        """Apply this stimulus once to ``model.u`` on the device (the
        reference's ``Stim.stimulate``).  The run loop calls it only on the
        steps whose stimuli run on the host, in the sequence's order, because
        a stimulus of another kind (a user subclass with its own
        ``stimulate``) is due on that step; on every other step the stimulus
        is applied inside the kernels.  Same arithmetic as the kernels:
        nodes of the region with mesh == 1, u = value (voltage) or
        u = min(u + dt * current, u_max) (current)."""
        lo, hi, mask = self._region(model)
        kind, value, has_umax, u_max = self._kind_value(
            model, self._host_application())
        if any(b <= a for a, b in zip(lo, hi)):
            return
        box = tuple(slice(a, b) for a, b in zip(lo, hi))
        u = model._dev["u"][box]
        sel = model._mesh_d[box] == 1
        if mask is not None:
            sel &= mask[box] != 0
        if kind == _ffi.STIM_VOLTAGE:
            u.masked_fill_(sel, value)
        else:
            x = u + value
            if has_umax:
                x = torch.where(x > u_max, torch.full_like(x, u_max), x)
            u.copy_(torch.where(sel, x, u))
        model._nonmyo_equal = None

    def _host_application(self):
        """Index of the application made by a host-side ``stimulate``."""
        return 0

    # -- lowering -------------------------------------------------------
    def _region(self, model):
        """(lo, hi, mask_tensor_or_None) in grid coordinates."""
        raise NotImplementedError

    def _kind_value(self, model, k):
        """(kind, value, has_umax, u_max) of the k-th application."""
        raise NotImplementedError

    def _windows(self, ts, n0):
        """Replay the reference's schedule over the segment times ``ts``
        (time at steps n0, n0+1, ...).  Returns a list of (first, last,
        application index) step windows and advances ``passed``."""
        if self.passed:
            return []
        ok = ts >= self.t
        if not ok.any():
            return []
        a = int(np.argmax(ok))
        done = ts[a:] >= (self.t + self.duration)
        if done.any():
            b = a + int(np.argmax(done))
            self.passed = True
        else:
            b = len(ts) - 1
        return [(n0 + a, n0 + b, 0)]


class StimVoltage(Stim):
    """Set u to a value (core/stimulation/stim_voltage.py)."""

    def __init__(self, time, volt_value, duration=0.0):
        super().__init__(time, duration)
        self.volt_value = volt_value

    def _kind_value(self, model, k):
        return _ffi.STIM_VOLTAGE, float(self.volt_value), 0, 0.0


class StimCurrent(Stim):
    """Add dt * current to u (core/stimulation/stim_current.py)."""

    def __init__(self, time, curr_value, duration):
        super().__init__(time, duration)
        self.curr_value = curr_value
        self.u_max = None

    def _kind_value(self, model, k):
        u_max = getattr(self, "u_max", None)
        return (_ffi.STIM_CURRENT, float(model.dt * self.curr_value),
                int(u_max is not None),
                float(u_max) if u_max is not None else 0.0)


def is_native(stim):
    """True when the kernels apply `stim` themselves: one of this package's
    stimulus classes whose region and value the library understands, and
    whose ``stimulate`` is not replaced by a subclass.  Any other object
    with the reference's interface (``t``, ``passed``, ``initialize``,
    ``stimulate``, ``update_status``) runs on the host."""
    return (isinstance(stim, Stim) and type(stim)._region is not Stim._region
            and type(stim).stimulate is Stim.stimulate)


class StimSequence:
    """Ordered list of stimuli (core/stimulation/stim_sequence.py)."""

    def __init__(self):
        self.sequence = []
        self.model = None

    def initialize(self, model):
        self.model = model
        for stim in self.sequence:
            stim.initialize(model)

    def add_stim(self, stim):
        self.sequence.append(stim)

    def remove_stim(self):
        self.sequence = []


def _slice_bounds(bounds, shape):
    lo, hi = [], []
    for (a, b), n in zip(bounds, shape):
        s, e, _ = slice(a, b).indices(n)
        lo.append(s)
        hi.append(max(s, e))
    return lo, hi


def _mask_region(mask, model):
    mask = np.asarray(mask, dtype=bool)
    shape = model.cardiac_tissue.mesh.shape
    if mask.shape != shape:
        mask = np.broadcast_to(mask, shape)
    nz = np.nonzero(mask)
    if len(nz[0]) == 0:
        return [0] * len(shape), [0] * len(shape), None
    lo = [int(a.min()) for a in nz]
    hi = [int(a.max()) + 1 for a in nz]
    dev = torch.as_tensor(np.ascontiguousarray(mask, dtype=np.int8),
                          device=model._device())
    return lo, hi, dev


class _Coord:
    def _region(self, model):
        shape = model.cardiac_tissue.mesh.shape
        lo, hi = _slice_bounds(self._bounds(), shape)
        return lo, hi, None


class StimVoltageCoord2D(_Coord, StimVoltage):
    """Voltage on mesh==1 nodes of a box (stim_voltage_coord_2d.py)."""

    def __init__(self, time, volt_value, x1, x2, y1, y2):
        super().__init__(time, volt_value)
        self.x1, self.x2, self.y1, self.y2 = x1, x2, y1, y2

    def _bounds(self):
        return [(self.x1, self.x2), (self.y1, self.y2)]


class StimCurrentCoord2D(_Coord, StimCurrent):
    """Current on mesh==1 nodes of a box (stim_current_coord_2d.py)."""

    def __init__(self, time, curr_value, duration, x1, x2, y1, y2,
                 u_max=None):
        super().__init__(time, curr_value, duration)
        self.x1, self.x2, self.y1, self.y2 = x1, x2, y1, y2
        self.u_max = u_max

    def _bounds(self):
        return [(self.x1, self.x2), (self.y1, self.y2)]


class StimVoltageCoord3D(_Coord, StimVoltage):
    """(stim_voltage_coord_3d.py)"""

    def __init__(self, time, volt_value, x1, x2, y1, y2, z1, z2):
        super().__init__(time, volt_value)
        self.x1, self.x2, self.y1, self.y2 = x1, x2, y1, y2
        self.z1, self.z2 = z1, z2

    def _bounds(self):
        return [(self.x1, self.x2), (self.y1, self.y2), (self.z1, self.z2)]


class StimCurrentCoord3D(_Coord, StimCurrent):
    """(stim_current_coord_3d.py)"""

    def __init__(self, time, curr_value, duration, x1, x2, y1, y2, z1, z2,
                 u_max=None):
        super().__init__(time, curr_value, duration)
        self.x1, self.x2, self.y1, self.y2 = x1, x2, y1, y2
        self.z1, self.z2 = z1, z2
        self.u_max = u_max

    def _bounds(self):
        return [(self.x1, self.x2), (self.y1, self.y2), (self.z1, self.z2)]


class _Matrix:
    def _region(self, model):
        return _mask_region(np.asarray(self.matrix) > 0, model)


class StimVoltageMatrix2D(_Matrix, StimVoltage):
    """Voltage where matrix > 0 and mesh == 1 (stim_voltage_matrix_2d.py)."""

    def __init__(self, time, volt_value, matrix):
        super().__init__(time, volt_value)
        self.matrix = matrix


class StimCurrentMatrix2D(_Matrix, StimCurrent):
    """Current where matrix > 0 and mesh == 1 (stim_current_matrix_2d.py)."""

    def __init__(self, time, curr_value, duration, matrix, u_max=None):
        super().__init__(time, curr_value, duration)
        self.matrix = matrix
        self.u_max = u_max


class StimVoltageMatrix3D(StimVoltageMatrix2D):
    """(stim_voltage_matrix_3d.py)"""


class StimCurrentMatrix3D(StimCurrentMatrix2D):
    """(stim_current_matrix_3d.py)"""


class StimCurrentArea2D(StimCurrent):
    """Current on a list of node coordinates (stim_current_area_2d.py)."""

    def __init__(self, time, curr_value, duration, coords=None, u_max=None):
        super().__init__(time, curr_value, duration)
        self.coords = coords
        self.u_max = u_max

    def add_stim_point(self, coord, mesh, size=None):
        self._coord = coord
        if size is None:
            self.coords = np.atleast_2d(coord)
            return
        tissue_points = np.argwhere(mesh == 1)
        dist = np.linalg.norm(tissue_points - coord, axis=1)
        self.coords = tissue_points[dist < size]

    def initialize(self, model):
        coords = np.asarray(self.coords)
        mask = (model.cardiac_tissue.mesh[tuple(coords.T)] == 1)
        if mask.sum() == 0:
            raise ValueError("The specified area does not have healthy cells.")
        self._coords = coords[mask]
        return super().initialize(model)

    def _region(self, model):
        m = np.zeros(model.cardiac_tissue.mesh.shape, dtype=bool)
        m[tuple(self._coords.T)] = True
        return _mask_region(m, model)


class StimCurrentArea3D(StimCurrentArea2D):
    """(stim_current_area_3d.py)"""


class StimVoltageListMatrix3D(StimVoltage):
    """Per-step voltage sequence on a mask (stim_voltage_list_matrix_3d.py).

    Application k (k = 0, 1, ...) sets u = volt_value[k] on
    ``matrix > 0 & mesh == 1``; each application is its own step window.
    """

    def __init__(self, time, volt_values, duration, matrix):
        super().__init__(time, volt_values, duration)
        self.matrix = matrix
        self.step = 0

    def initialize(self, model):
        super().initialize(model)
        total_steps = int(self.duration / model.dt) + 1
        if len(self.volt_value) < total_steps:
            raise ValueError("The length of the voltage values array should "
                             "be greater than the total number of steps.")

    def _region(self, model):
        return _mask_region(np.asarray(self.matrix) > 0, model)

    def _kind_value(self, model, k):
        return _ffi.STIM_VOLTAGE, float(self.volt_value[k]), 0, 0.0

    def _host_application(self):
        k = self.step
        self.step += 1
        return k

    def _windows(self, ts, n0):
        out = []
        for w_first, w_last, _ in Stim._windows(self, ts, n0):
            for n in range(w_first, w_last + 1):
                out.append((n, n, self.step))
                self.step += 1
        return out
