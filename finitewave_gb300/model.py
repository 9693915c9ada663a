"""Cardiac models: device-resident state and the chunked run loop.

``CardiacModel.run`` keeps the reference's semantics (``core/model/
cardiac_model.py:130-189``) -- per step: stimuli, diffusion, ionic update,
trackers, ``t += dt``, ``step += 1``, swap, commands, state saver,
termination -- but runs the steps on the GPU in segments: the host replays
the float64 time accumulation, cuts the run at every step where host-side
work is due (a command, a state save, termination), and hands each segment
to ``fw_step`` with the stimulus windows and tracker windows that fall into
it.  Between segments nothing is copied back unless a host object asks for
a state variable.

State variables (``u``, ``v``, ...) live in device tensors; reading
``model.u`` returns a host numpy copy and assigning ``model.u = array``
uploads it, so state loaders, savers and commands work unchanged.
"""
import copy
import ctypes
import warnings

import numpy as np
import torch

from . import _ffi
from .stencil import (AsymmetricStencil2D, AsymmetricStencil3D,
                      IsotropicStencil2D, IsotropicStencil3D)
from . import stimulation, tracker as _tracker
from .tracker import (ActivationTime2DTracker, ECG2DTracker,
                      LocalActivationTime2DTracker, SpiralWaveCore2DTracker,
                      Tracker, _ProbeTracker)

_NP = {"float64": np.float64, "float32": np.float32}
_MAX_SEGMENT = 1 << 20


def _np_name(npfloat):
    name = np.dtype(npfloat).name
    if name not in _NP:
        raise ValueError(f"npfloat must be float64 or float32, got {npfloat}")
    return name


class _DeviceArray(np.ndarray):
    """Host copy of a device state array whose item assignments write
    through: ``model.u[1:-1, 1:-1] = 1`` (as the reference's commands do on
    its numpy state) updates the device array.  Views write through as
    well; copies (``.copy()``, arithmetic results) are plain arrays."""

    def __array_finalize__(self, obj):
        if self.base is None or obj is None:
            self._owner = self._name = self._root = None
            return
        self._owner = getattr(obj, "_owner", None)
        self._name = getattr(obj, "_name", None)
        self._root = getattr(obj, "_root", None)

    def __setitem__(self, key, value):
        super().__setitem__(key, value)
        owner = getattr(self, "_owner", None)
        if owner is not None and self._root is not None:
            setattr(owner, self._name, np.asarray(self._root))

    def __array_wrap__(self, arr, context=None, return_scalar=False):
        # ufunc results are new arrays: plain numpy
        out = np.asarray(arr)
        if return_scalar and out.ndim == 0:
            return out[()]
        return out


def _device_array(owner, name, host):
    a = host.view(_DeviceArray)
    a._owner, a._name, a._root = owner, name, a
    return a


class _StateVar:
    """Descriptor: a state variable held on the device, seen as numpy."""

    def __init__(self, name):
        self.name = name

    def __get__(self, obj, cls=None):
        if obj is None:
            return self
        dev = obj.__dict__.get("_dev")
        if dev and self.name in dev:
            t = dev[self.name]
            if self.name in obj.__dict__.get("_pairs", ()):
                h = t.cpu().numpy()
                host = h[..., 0].astype(np.float64) + h[..., 1]
            else:
                host = t.cpu().numpy()
            return _device_array(obj, self.name, host)
        return obj.__dict__.get("_host", {}).get(self.name, np.ndarray)

    def __set__(self, obj, value):
        dev = obj.__dict__.get("_dev")
        if dev and self.name in dev and isinstance(value, np.ndarray):
            t = dev[self.name]
            pair = self.name in obj.__dict__.get("_pairs", ())
            shape = tuple(t.shape[:-1]) if pair else tuple(t.shape)
            if value.shape != shape:
                raise ValueError(f"{self.name}: shape {value.shape} != "
                                 f"{shape}")
            if pair:
                t.copy_(torch.as_tensor(_split_pair(value)))
            else:
                t.copy_(torch.as_tensor(np.ascontiguousarray(value))
                        .to(t.dtype))
            other = obj.__dict__.get("_stateb", {}).get(self.name)
            if other is not None:
                # the fused form's second buffer equals the state at
                # non-myocytes (and is overwritten at myocytes)
                other.copy_(t)
            obj.__dict__["_nonmyo_equal"] = None
            return
        obj.__dict__.setdefault("_host", {})[self.name] = value


def _split_pair(value):
    """float64 values as compensated float32 pairs (hi, lo), hi the value
    rounded to float32 and lo the rest rounded to float32: (..., 2)."""
    v = np.asarray(value, dtype=np.float64)
    hi = v.astype(np.float32)
    lo = (v - hi.astype(np.float64)).astype(np.float32)
    return np.ascontiguousarray(np.stack([hi, lo], axis=-1))


class CardiacModel:
    """Base class of the GPU models (core/model/cardiac_model.py:9-239).

    Subclasses define ``_model_id`` (fwgpu.h fw_model), ``_state_names``
    (state variables after ``u``, in the library's order), ``_param_names``
    (parameters in the library's order) and ``select_stencil``.

    Extra attributes over the reference: ``device`` (CUDA device, default
    the current one), ``form`` ('plain', 'fused' or None for automatic:
    fused for float32 where the library has it, plain otherwise),
    ``fused_k`` / ``fused_variant`` (the fused kernel's time steps per
    launch and kernel; 0 = chosen by ``autotune``) and ``autotune`` (time
    the fused candidates once per configuration, finitewave_gb300.autotune).
    """

    _model_id = None
    _state_names = ()
    _param_names = ()
    _reset_u_new = False
    _init_names = {}   # state variable -> suffix of its init_* attribute

    u = _StateVar("u")
    u_new = _StateVar("u_new")

    def __init_subclass__(cls, **kw):
        super().__init_subclass__(**kw)
        for name in cls._state_names:
            if not isinstance(cls.__dict__.get(name), _StateVar):
                setattr(cls, name, _StateVar(name))

    def __init__(self):
        self.meta = {}
        self.cardiac_tissue = None
        self.stim_sequence = None
        self.tracker_sequence = None
        self.command_sequence = None
        self.state_loader = None
        self.state_saver = None
        self.stencil = None
        self.diffusion_kernel = None
        self.ionic_kernel = None
        self.weights = None
        self.dt = 0.
        self.dr = 0.
        self.t_max = 0.
        self.t = 0
        self.step = 0
        self.D_model = 1.
        self.prog_bar = True
        self.npfloat = np.float64
        self.state_vars = []
        self.device = None
        self.form = None
        self.fused_k = 0
        self.fused_variant = 0
        self.autotune = True
        self._dev = {}
        self._t_hist = []

    # ------------------------------------------------------------ helpers
    def _device(self):
        if self.device is not None:
            return torch.device(self.device)
        if not torch.cuda.is_available():
            raise RuntimeError("finitewave_gb300 needs a CUDA device")
        return torch.device("cuda", torch.cuda.current_device())

    def _np_dtype(self):
        return _NP[_np_name(self.npfloat)]

    def _precision(self):
        return _ffi.F64 if _np_name(self.npfloat) == "float64" else _ffi.F32

    def _torch_dtype(self, state_index=None):
        if state_index is not None and _ffi.state_is_f64(
                self._model_id, self._precision(), state_index):
            return torch.float64
        return torch.float64 if self._precision() == _ffi.F64 \
            else torch.float32

    def _shape(self):
        return tuple(np.asarray(self.cardiac_tissue.mesh).shape)

    def _params(self):
        return [float(getattr(self, n)) for n in self._param_names]

    def _time_of_steps(self, steps):
        """Model time t at the given global step indices (the float64
        accumulation t += dt, as the reference computes it)."""
        hist = self._t_hist_array()
        return hist[np.asarray(steps, dtype=np.int64)]

    def _t_hist_array(self):
        if len(self._t_hist) != 1:
            self._t_hist = [np.concatenate(self._t_hist)] if self._t_hist \
                else [np.zeros(0)]
        return self._t_hist[0]

    # ---------------------------------------------------------- lifecycle
    def initialize(self):
        """Allocate state on the device, build weights, set up stimuli,
        trackers, commands and state I/O (cardiac_model.py:91-117) and
        then the model's initial values."""
        dev = self._device()
        shape = self._shape()
        dtype = self._torch_dtype()
        self._dev = {}
        u = torch.zeros(shape, dtype=dtype, device=dev)
        self._dev["u"] = u
        self._dev["u_new"] = u.clone()
        self.step = 0
        self.t = 0
        self._t_hist = []
        self._status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.compute_weights()
        self.diffusion_kernel = self.stencil.select_diffusion_kernel()
        if self.stim_sequence:
            self.stim_sequence.initialize(self)
        if self.tracker_sequence:
            self.tracker_sequence.initialize(self)
        if self.command_sequence:
            self.command_sequence.initialize(self)
        if self.state_loader:
            self.state_loader.initialize(self)
        if self.state_saver:
            self.state_saver.initialize(self)
        init_u = float(getattr(self, "init_u", 0.0))
        self._dev["u"].fill_(init_u)
        if self._reset_u_new:
            self._dev["u_new"].copy_(self._dev["u"])
        prec = self._precision()
        self._pairs = {n for i, n in enumerate(self._state_names)
                       if _ffi.state_is_pair(self._model_id, prec, i)}
        for i, name in enumerate(self._state_names):
            v = float(getattr(self, "init_" + self._init_names.get(name, name)))
            if name in self._pairs:
                hi, lo = _split_pair(v)
                t = torch.empty(shape + (2,), dtype=torch.float32, device=dev)
                t[..., 0].fill_(float(hi))
                t[..., 1].fill_(float(lo))
            else:
                t = torch.empty(shape, dtype=self._torch_dtype(i), device=dev)
                t.fill_(v)
            self._dev[name] = t
        # second state buffers of the fused form (fw_step_args.state_b): a
        # fused launch reads the state from one and writes the other
        self._stateb = {}
        if (prec == _ffi.F32 and len(shape) == 2 and
                self._model_id in self._FUSED_MODELS):
            self._stateb = {n: self._dev[n].clone() for n in self._state_names}

    def compute_weights(self):
        """Myocyte indices, stencil choice and device weights
        (cardiac_model.py:119-128)."""
        tissue = self.cardiac_tissue
        tissue.compute_myo_indexes()
        mesh = np.asarray(tissue.mesh)
        myo = mesh == 1
        if tissue.special_boundaries is not None:
            myo &= np.asarray(tissue.special_boundaries) == 0
        ring = np.zeros(mesh.shape, dtype=bool)
        for ax in range(mesh.ndim):
            sl = [slice(None)] * mesh.ndim
            sl[ax] = 0
            ring[tuple(sl)] = True
            sl[ax] = -1
            ring[tuple(sl)] = True
        if (myo & ring).any():
            raise ValueError("myocytes (mesh == 1) on the outer ring of the "
                             "grid are not supported: the stencil would "
                             "read outside the grid")
        dev = self._device()
        self._n_myo = int(myo.sum())
        self._mesh_d = torch.as_tensor(np.ascontiguousarray(mesh, np.int8),
                                       device=dev)
        self._myo_d = torch.as_tensor(myo.astype(np.int8), device=dev)
        self._special = tissue.special_boundaries is not None and bool(
            (np.asarray(tissue.special_boundaries)[mesh == 1] != 0).any())
        if self.stencil is None:
            self.stencil = self.select_stencil(tissue)
        self.weights = self.stencil.compute_weights(self, tissue)
        self._step_stencil = self.stencil.kind
        if self.stencil.kind == _ffi.ANISO19 and not bool(
                self.weights[list(_ffi.ANISO19_XY_ZERO)].any()):
            # fibers with no z component: the eight planes coupling k +- 1
            # with i +- 1 or j +- 1 are zero, and the step skips them
            self._step_stencil = _ffi.ANISO19_XY
        self._pack_weights()
        self._weight_rows()

    def _weight_rows(self, force=False):
        """FW_STENCIL_ANISO19_XY steps read the eleven weight planes 0-8,
        11 and 12.  When the grid's nodes share few distinct rows of them
        (one per fiber layer and myocyte neighbourhood in a slab with
        layered fibers), keep the distinct rows (padded to 12 values) and
        each node's row instead: the step then reads a 4-byte row index per
        node from HBM and the rows from L2, with the same sums.  Kept when
        the rows take at most a quarter of the planes' bytes and 32 MB
        (`force`: whenever the form applies, for tests)."""
        self._wrows = self._widx = None
        self._wrows_src = self.weights
        if getattr(self, "_step_stencil", None) != _ffi.ANISO19_XY:
            return
        w = self.weights
        n = w[0].numel()
        planes = w[[0, 1, 2, 3, 4, 5, 6, 7, 8, 11, 12]].reshape(11, n)
        ibits = torch.int32 if w.dtype == torch.float32 else torch.int64
        bits = planes.t().contiguous().view(ibits)
        uniq, inv = torch.unique(bits, dim=0, return_inverse=True)
        row_bytes = uniq.shape[0] * 12 * w.element_size()
        if not force and (row_bytes * 4 > n * 11 * w.element_size() or
                          row_bytes > 32 << 20):
            return   # little sharing: the planes themselves
        rows = torch.zeros((uniq.shape[0], 12), dtype=w.dtype, device=w.device)
        rows[:, :11] = uniq.view(w.dtype)
        self._wrows = rows
        self._widx = inv.to(torch.int32).contiguous()

    def _pack_weights(self):
        """Node-major copy of the off-centre weights for the TMA form of the
        fused kernel (fw_pack_weights); only for 2D float32 grids whose row
        length is a multiple of 16 nodes."""
        self._wpack = None
        kind = self.stencil.kind
        shape = self._shape()
        if (self._precision() != _ffi.F32 or kind not in (_ffi.ISO5, _ffi.ANISO9)
                or self._model_id not in self._FUSED_MODELS
                or shape[1] % 16 != 0 or self.form == "plain"):
            return
        nwo = 4 if kind == _ffi.ISO5 else 8
        n = shape[0] * shape[1]
        self._wpack = torch.empty(n * nwo, dtype=torch.float32,
                                  device=self._device())
        _ffi.call("fw_pack_weights", kind, self.weights.data_ptr(), n,
                  self._wpack.data_ptr(),
                  torch.cuda.current_stream().cuda_stream)

    def select_stencil(self, cardiac_tissue):
        raise NotImplementedError

    def run_diffusion_kernel(self):
        """One diffusion pass u_new = W u over the myocytes
        (cardiac_model.py:205-211)."""
        idx = torch.as_tensor(self.cardiac_tissue.myo_indexes,
                              device=self._device())
        self.diffusion_kernel(self._dev["u_new"], self._dev["u"],
                              self.weights, idx)

    def run_ionic_kernel(self):
        """One ionic pass over the myocytes (the models' run_ionic_kernel)."""
        idx = torch.as_tensor(
            np.asarray(self.cardiac_tissue.myo_indexes, dtype=np.int64),
            device=self._device())
        ptrs = [self._dev[n].data_ptr() for n in self._state_names]
        arr = (ctypes.c_void_p * max(1, len(ptrs)))(*ptrs)
        par = (ctypes.c_double * max(1, len(self._param_names)))(
            *self._params())
        _ffi.call("fw_ionic", self._model_id, self._precision(),
                  self._dev["u_new"].data_ptr(), self._dev["u"].data_ptr(),
                  arr, idx.data_ptr(), idx.numel(), float(self.dt), par,
                  torch.cuda.current_stream().cuda_stream)

    def check_termination(self):
        max_iters = int(np.ceil(self.t_max / self.dt))
        return (self.t > self.t_max) or (self.step > max_iters)

    def clone(self):
        return copy.deepcopy(self)

    # ---------------------------------------------------------------- run
    def run(self, initialize=True, num_of_theads=None):
        """Run the simulation to t_max (cardiac_model.py:130-189).

        ``num_of_theads`` is accepted for interface compatibility; the work
        runs on the GPU.
        """
        if initialize:
            self.initialize()
        if self.t_max < self.t:
            raise ValueError("t_max must be greater than current t.")
        if self.state_loader:
            self.state_loader.load()
        self._nonmyo_equal = None
        host_stims, host_trs = self._host_plugins()
        iters = int(np.ceil((self.t_max - self.t) / self.dt))
        remaining = iters
        while remaining > 0:
            limit = min(remaining, _MAX_SEGMENT)
            if host_stims or host_trs:
                k = self._steps_before_host(limit, host_stims, host_trs)
                n_seg = self._host_step(host_stims, host_trs) if k == 0 \
                    else self._run_segment(k, sync=False)
            else:
                n_seg = self._run_segment(limit, sync=False)
            remaining -= n_seg
            if self.command_sequence:
                self.command_sequence.execute_next()
            if self.state_saver:
                self.state_saver.save()
            if self.check_termination():
                if self.state_saver:
                    self.state_saver.save()
                break
        self._check_status()

    def _times(self, limit):
        """Times t_n of the next `limit` steps and the time after them (the
        float64 accumulation t += dt)."""
        acc = np.empty(limit + 1)
        acc[0] = self.t
        acc[1:] = self.dt
        return np.add.accumulate(acc)

    # ------------------------------------------- host round-trip plug-ins
    def _host_plugins(self):
        """Stimuli and trackers the kernels do not apply themselves: user
        subclasses written against the reference's plug-in interface
        (``Stim.stimulate``, ``Tracker._track`` / ``track``)."""
        stims = [s for s in (self.stim_sequence.sequence
                             if self.stim_sequence else [])
                 if not stimulation.is_native(s)]
        trs = [t for t in (self.tracker_sequence.sequence
                           if self.tracker_sequence else [])
               if not _tracker.is_native(t)]
        return stims, trs

    def _steps_before_host(self, limit, stims, trs):
        """Steps (at most `limit`) before the next step on which a host
        stimulus or tracker is due: a stimulus on steps with t >= stim.t
        while it has not passed (stim_sequence.py:65-77), a tracker on the
        steps of Tracker.track (tracker.py:70-83), or on every step when a
        subclass replaces ``track``."""
        ts = self._times(limit)[:limit]
        ns = self.step + np.arange(limit, dtype=np.int64)
        due = np.zeros(limit, dtype=bool)
        for s in stims:
            if not s.passed:
                due |= ts >= s.t
        for tr in trs:
            if isinstance(tr, Tracker) and type(tr).track is not Tracker.track:
                return 0
            due |= ((tr.start_time <= ts) & (ts <= tr.end_time) &
                    (ns % int(tr.step) == 0))
        return int(np.argmax(due)) if due.any() else limit

    def _host_step(self, stims, trs):
        """One step with host plug-ins, in the reference's order
        (cardiac_model.py:164-178).  When a host stimulus is due, every
        stimulus of the step runs on the host in the sequence's order
        (this package's own through ``Stim.stimulate`` on the device
        array); then one plain-form step on the device, with this package's
        trackers inside it; then the host trackers, which see the state as
        the reference's do: ``model.u`` after the stimuli, ``model.u_new``
        and the state variables after the update, ``model.t`` and
        ``model.step`` of this step."""
        host_stim = any(self.t >= s.t and not s.passed for s in stims)
        if host_stim:
            for s in self.stim_sequence.sequence:
                if self.t >= s.t and not s.passed:
                    s.stimulate(self)
                    s.update_status(self)
        form = self.form
        self.form = "plain"
        try:
            seg = self._prepare_segment(1, skip_stims=host_stim)
        finally:
            self.form = form
        stream = torch.cuda.current_stream().cuda_stream
        _ffi.call("fw_step", ctypes.byref(seg.args), seg.n0, seg.n_seg,
                  stream)
        if trs:
            with _HostView(self):
                for tr in self.tracker_sequence.sequence:
                    if any(tr is h for h in trs):
                        tr.track()
        self._finish_segment(seg)
        return seg.n_seg

    def _segment_times(self, limit):
        """Times t_n of the next `limit` steps and the segment length: the
        first step after which a command, a state save or termination is
        due ends the segment."""
        ts_all = self._times(limit)
        after = ts_all[1:]
        steps_after = self.step + 1 + np.arange(limit)
        stop = (after > self.t_max) | (steps_after >
                                       int(np.ceil(self.t_max / self.dt)))
        if self.command_sequence:
            for c in self.command_sequence.sequence:
                if not c.passed and c.t is not None:
                    stop |= after >= c.t
        saver = self.state_saver
        if saver is not None:
            savers = getattr(saver, "savers", None) or [saver]
            for s in savers:
                if getattr(s, "passed", True):
                    continue
                if s.time < 0:
                    stop |= after >= self.t_max
                else:
                    stop |= after >= s.time
        n_seg = int(np.argmax(stop)) + 1 if stop.any() else limit
        return ts_all[:n_seg], float(ts_all[n_seg]), n_seg

    _FUSED_MODELS = (_ffi.MODEL_AP, _ffi.MODEL_MS, _ffi.MODEL_FK,
                     _ffi.MODEL_BK)

    def _fused_ok(self):
        """The fused form covers 2D float32 AP/MS/FK without special
        boundaries, with u and u_new equal at non-myocytes."""
        if (self._precision() != _ffi.F32 or self._special or
                self._model_id not in self._FUSED_MODELS or
                self.stencil.kind not in (_ffi.ISO5, _ffi.ANISO9)):
            return False
        trs = self.tracker_sequence.sequence if self.tracker_sequence else []
        if any(isinstance(t, (ECG2DTracker, SpiralWaveCore2DTracker))
               for t in trs):
            return False
        if (sum(isinstance(t, ActivationTime2DTracker) for t in trs) > 2 or
                sum(isinstance(t, LocalActivationTime2DTracker)
                    for t in trs) > 1):
            return False
        if getattr(self, "_nonmyo_equal", None) is None:
            off = self._myo_d == 0
            self._nonmyo_equal = bool(torch.equal(self._dev["u"][off],
                                                  self._dev["u_new"][off]))
        return self._nonmyo_equal

    def _form(self):
        if self.form == "plain":
            return _ffi.FORM_PLAIN
        if self.form == "fused":
            if not self._fused_ok():
                raise ValueError("form='fused' needs a 2D float32 Aliev-"
                                 "Panfilov / Mitchell-Schaeffer / Fenton-"
                                 "Karma model without special boundaries")
            return _ffi.FORM_FUSED
        return _ffi.FORM_FUSED if self._fused_ok() else _ffi.FORM_PLAIN

    def _check_status(self, st=None):
        """Raise (or warn) for the bits set in the device status word; `st`
        is a copy of it already on the host, else it is read (a device
        synchronisation)."""
        if st is None:
            st = int(self._status.item())
        if st & _ffi.FW_DEV_TIMEOUT:
            raise RuntimeError(f"{type(self).__name__}: a bounded on-chip "
                               "wait of the fused kernel gave up; the state "
                               "after this run is not defined")
        if st & _ffi.FW_DEV_BATCH_FAULT:
            raise RuntimeError(f"{type(self).__name__}: a batch tile "
                               "descriptor was out of range; the state after "
                               "this run is not defined")
        if st & _ffi.FW_DEV_NONFINITE:
            # the reference carries on with NaN silently; keep its results
            # and say so
            warnings.warn(f"{type(self).__name__}: the potential became inf "
                          "or NaN (time step too large for the model?)",
                          RuntimeWarning, stacklevel=3)
        if st & _ffi.FW_DEV_TIP_OVERFLOW:
            raise RuntimeError("SpiralWaveCore tracker: more tips than its "
                               "capacity in one run segment")
        if st & _ffi.FW_DEV_PROBE_OVERFLOW:
            raise RuntimeError("probe tracker buffer overflow")
        if st & _ffi.FW_DEV_LAT_OVERFLOW:
            raise RuntimeError("LocalActivationTimeTracker: a node crossed "
                               "the threshold more often than its capacity")

    def _run_segment(self, limit, sync=True):
        """Advance up to `limit` steps on the device (one fw_step call);
        returns the number of steps taken.  With sync=False the device
        status word is not read back (no host synchronisation)."""
        seg = self._prepare_segment(limit)
        stream = torch.cuda.current_stream().cuda_stream
        _ffi.call("fw_step", ctypes.byref(seg.args), seg.n0, seg.n_seg,
                  stream)
        if sync:
            self._check_status()
        self._finish_segment(seg)
        return seg.n_seg

    def _bare_args(self):
        """fw_step_args with the model's arrays, parameters and kernel
        choice, and no stimuli or trackers."""
        a = _ffi.StepArgs()
        a.model = self._model_id
        a.stencil = getattr(self, "_step_stencil", self.stencil.kind)
        a.precision = self._precision()
        shape = self._shape()
        a.ni, a.nj = shape[0], shape[1]
        a.nk = shape[2] if len(shape) == 3 else 1
        a.mesh = self._mesh_d.data_ptr()
        a.myo = self._myo_d.data_ptr()
        a.weights = self.weights.data_ptr()
        if getattr(self, "_wrows", None) is not None:
            if self.weights is not self._wrows_src:
                self._weight_rows()   # the weights were replaced
            if self._wrows is not None and a.stencil == _ffi.ANISO19_XY:
                a.weight_rows = self._wrows.data_ptr()
                a.weight_row_index = self._widx.data_ptr()
        wpack = getattr(self, "_wpack", None)
        a.weights_packed = wpack.data_ptr() if wpack is not None else None
        a.u[0] = self._dev["u"].data_ptr()
        a.u[1] = self._dev["u_new"].data_ptr()
        for i, name in enumerate(self._state_names):
            a.state[i] = self._dev[name].data_ptr()
            t = getattr(self, "_stateb", {}).get(name)
            if t is not None:
                a.state_b[i] = t.data_ptr()
        for i, p in enumerate(self._params()):
            a.params[i] = p
        a.dt = float(self.dt)
        a.form = self._form()
        a.fused_k = int(self.fused_k)
        a.fused_variant = int(self.fused_variant)
        a.debug_flags = int(getattr(self, "_debug_flags", 0))
        if a.fused_variant == 5 and a.form == _ffi.FORM_FUSED:
            self._fly_args(a)
        if (a.form == _ffi.FORM_FUSED and not a.fused_k and
                not a.fused_variant and self.autotune):
            from . import autotune
            a.fused_variant, a.fused_k = autotune.choose(self)
        self._fused_choice = (a.fused_variant, a.fused_k) \
            if a.form == _ffi.FORM_FUSED else None
        return a

    def _fly_args(self, a):
        """fused_variant 5 forms the AsymmetricStencil2D weights on chip:
        the tissue's fibers as float32 pairs (made once) and the stencil's
        constants."""
        fly = getattr(self, "_fly", None)
        tissue = self.cardiac_tissue
        if fly is None or fly[0] is not tissue.fibers:
            if (self.stencil.kind != _ffi.ANISO9 or tissue.fibers is None or
                    np.ndim(tissue.conductivity) != 0):
                raise ValueError("fused_variant 5 needs an AsymmetricStencil2D "
                                 "tissue with fibers and a scalar "
                                 "conductivity")
            fib = torch.as_tensor(np.ascontiguousarray(
                np.asarray(tissue.fibers, dtype=np.float32)),
                device=self._device())
            fly = (tissue.fibers, fib)
            self._fly = fly
        a.fibers_f32 = fly[1].data_ptr()
        a.fly_D_al = float(self.stencil.D_al)
        a.fly_D_ac = float(self.stencil.D_ac)
        a.fly_cond = float(tissue.conductivity)
        a.fly_scale = float(self.D_model) * float(self.dt) / float(self.dr) ** 2

    def _prepare_segment(self, limit, skip_stims=False):
        """The fw_step_args of the next segment of at most `limit` steps
        (stimulus and tracker windows in global step indices).  Stimuli and
        trackers that run on the host are left out, and so are all stimuli
        with skip_stims (a host step that has applied them already)."""
        a = self._bare_args()
        ts, t_end, n_seg = self._segment_times(limit)
        n0 = int(self.step)
        self._t_hist.append(ts)
        keep = []

        # stimuli (stim_sequence.py:65-77)
        n_st = 0
        if self.stim_sequence and not skip_stims:
            for stim in self.stim_sequence.sequence:
                if not stimulation.is_native(stim):
                    continue
                wins = stim._windows(ts, n0)
                if not wins:
                    continue
                lo, hi, mask = stim._region(self)
                if mask is not None:
                    keep.append(mask)
                for first, last, k in wins:
                    if n_st >= _ffi.MAX_STIMS:
                        raise RuntimeError("too many stimulus windows in one "
                                           "segment")
                    kind, value, has_umax, u_max = stim._kind_value(self, k)
                    s = a.stims[n_st]
                    s.kind, s.value = kind, value
                    s.has_umax, s.u_max = has_umax, u_max
                    s.first, s.last = first, last
                    for d in range(3):
                        s.lo[d] = lo[d] if d < len(lo) else 0
                        s.hi[d] = hi[d] if d < len(hi) else 1
                    s.mask = mask.data_ptr() if mask is not None else None
                    n_st += 1
        a.n_stims = n_st

        # trackers (tracker.py:70-83)
        n_at = n_lat = n_pr = n_ecg = n_tip = 0
        if self.tracker_sequence:
            for tr in self.tracker_sequence.sequence:
                if not _tracker.is_native(tr):
                    continue
                win = tr._window(ts, n0)
                if win is None:
                    continue
                first, last, count = win
                if isinstance(tr, ActivationTime2DTracker):
                    d = a.at[n_at]
                    n_at += 1
                    d.win.first, d.win.last, d.win.stride = first, last, \
                        int(tr.step)
                    d.threshold = float(tr.threshold)
                    d.act_step = tr._act_step.data_ptr()
                elif isinstance(tr, LocalActivationTime2DTracker):
                    d = a.lat[n_lat]
                    n_lat += 1
                    d.win.first, d.win.last, d.win.stride = first, last, \
                        int(tr.step)
                    d.threshold = float(tr.threshold)
                    d.activated = tr._activated.data_ptr()
                    d.cross_steps = tr._steps.data_ptr()
                    d.cross_count = tr._count.data_ptr()
                    d.capacity = int(tr.capacity)
                elif isinstance(tr, ECG2DTracker):
                    if n_ecg >= _ffi.MAX_ECG:
                        raise RuntimeError("too many ECG trackers")
                    buf = tr._reserve(count)
                    d = a.ecg[n_ecg]
                    n_ecg += 1
                    d.win.first, d.win.last, d.win.stride = first, last, \
                        int(tr.step)
                    d.n_leads = len(tr.measure_coords)
                    for c, xyz in enumerate(tr.measure_coords):
                        for q in range(3):
                            d.coords[c][q] = float(xyz[q])
                    d.dr = float(self.dr)
                    d.out = buf.data_ptr()
                    d.sample_offset = 0
                    d.capacity = count
                elif isinstance(tr, SpiralWaveCore2DTracker):
                    if n_tip >= _ffi.MAX_TIP:
                        raise RuntimeError("at most one spiral-wave core "
                                           "tracker per model")
                    buf = tr._reserve(first, int(tr.step))
                    d = a.tip[n_tip]
                    n_tip += 1
                    d.win.first, d.win.last, d.win.stride = first, last, \
                        int(tr.step)
                    d.threshold = float(tr.threshold)
                    d.u_prev = tr._u_prev.data_ptr()
                    d.out = buf.data_ptr()
                    d.count = tr._count.data_ptr()
                    d.capacity = int(tr.capacity)
                    d.sample_offset = 0
                elif isinstance(tr, _ProbeTracker):
                    buf = tr._reserve(count)
                    d = a.probe[n_pr]
                    n_pr += 1
                    d.win.first, d.win.last, d.win.stride = first, last, \
                        int(tr.step)
                    d.n_cells = tr._n_cells
                    d.n_vars = len(tr._var_ids)
                    for i, v in enumerate(tr._var_ids):
                        d.var_ids[i] = v
                    d.cells = tr._cells.data_ptr()
                    d.out = buf.data_ptr()
                    d.sample_offset = 0
                    d.capacity = count
                else:
                    raise TypeError(f"{type(tr).__name__} is not a "
                                    "finitewave_gb300 tracker")
        a.n_at, a.n_lat, a.n_probe = n_at, n_lat, n_pr
        a.n_ecg = n_ecg
        a.n_tip = n_tip
        a.status = self._status.data_ptr()
        return _Segment(a, n0, n_seg, t_end, keep)

    def _finish_segment(self, seg):
        """Account for a segment the device has been given: swap u / u_new
        (and, after a fused segment, the two state buffers) after an odd
        step count, advance t and step."""
        if seg.n_seg % 2 == 1:
            self._dev["u"], self._dev["u_new"] = (self._dev["u_new"],
                                                  self._dev["u"])
            if seg.args.form == _ffi.FORM_FUSED:
                sb = self._stateb
                for n in self._state_names:
                    self._dev[n], sb[n] = sb[n], self._dev[n]
        self.t = seg.t_end
        self.step = seg.n0 + seg.n_seg


class _HostView:
    """While host trackers run: host copies of the state variables also in
    ``model.__dict__``, where the reference's trackers may read them
    (``model.__dict__[var]``, multi_variable_2d_tracker.py:54,68); removed
    afterwards.  Attribute access (``model.u``) reads the device arrays
    through the state-variable descriptors either way."""

    def __init__(self, model):
        self.model = model
        self.names = ["u", "u_new"] + list(model._state_names)

    def __enter__(self):
        d = self.model.__dict__
        snap = {n: np.asarray(getattr(self.model, n)) for n in self.names}
        d.update(snap)
        return self

    def __exit__(self, *exc):
        for n in self.names:
            self.model.__dict__.pop(n, None)
        return False


class _Segment:
    """One segment's fw_step_args and bookkeeping (`keep` holds host-side
    objects whose device memory the args point to)."""

    __slots__ = ("args", "n0", "n_seg", "t_end", "keep")

    def __init__(self, args, n0, n_seg, t_end, keep):
        self.args, self.n0, self.n_seg = args, n0, n_seg
        self.t_end, self.keep = t_end, keep


# ------------------------------------------------------------------ models

def _stencil_2d(tissue):
    return IsotropicStencil2D() if tissue.fibers is None \
        else AsymmetricStencil2D()


def _stencil_3d(tissue):
    return IsotropicStencil3D() if tissue.fibers is None \
        else AsymmetricStencil3D()


class AlievPanfilov2D(CardiacModel):
    """Aliev-Panfilov (cpuwave2D/model/aliev_panfilov_2d.py:10-335)."""

    _model_id = _ffi.MODEL_AP
    _state_names = ("v",)
    _param_names = ("a", "k", "eap", "mu_1", "mu_2")

    def __init__(self):
        super().__init__()
        self.D_model = 1.
        self.state_vars = ["u", "v"]
        self.npfloat = "float64"
        self.a = 0.1
        self.k = 8.0
        self.eap = 0.01
        self.mu_1 = 0.2
        self.mu_2 = 0.3
        self.init_u = 0.0
        self.init_v = 0.0

    def select_stencil(self, cardiac_tissue):
        return _stencil_2d(cardiac_tissue)


class AlievPanfilov3D(AlievPanfilov2D):
    """(cpuwave3D/model/aliev_panfilov_3d.py)"""

    def select_stencil(self, cardiac_tissue):
        return _stencil_3d(cardiac_tissue)


class MitchellSchaeffer2D(CardiacModel):
    """Mitchell-Schaeffer (cpuwave2D/model/mitchell_schaeffer_2d.py)."""

    _model_id = _ffi.MODEL_MS
    _state_names = ("h",)
    _param_names = ("tau_close", "tau_open", "tau_in", "tau_out", "u_gate")

    def __init__(self):
        super().__init__()
        self.D_model = 1.
        self.state_vars = ["u", "h"]
        self.npfloat = "float64"
        self.tau_close = 150
        self.tau_open = 120
        self.tau_out = 6
        self.tau_in = 0.3
        self.u_gate = 0.13
        self.init_u = 0.0
        self.init_h = 1.0

    def select_stencil(self, cardiac_tissue):
        return _stencil_2d(cardiac_tissue)


class MitchellSchaeffer3D(MitchellSchaeffer2D):
    """(cpuwave3D/model/mitchell_schaeffer_3d.py)"""

    def select_stencil(self, cardiac_tissue):
        return _stencil_3d(cardiac_tissue)


class FentonKarma2D(CardiacModel):
    """Fenton-Karma MLR-I (cpuwave2D/model/fenton_karma_2d.py)."""

    _model_id = _ffi.MODEL_FK
    _state_names = ("v", "w")
    _param_names = ("tau_d", "tau_o", "tau_r", "tau_si", "tau_v_m",
                    "tau_v_p", "tau_w_m", "tau_w_p", "k", "u_c", "uc_si")

    def __init__(self):
        super().__init__()
        self.D_model = 1.
        self.state_vars = ["u", "v", "w"]
        self.npfloat = "float64"
        self.tau_r = 130
        self.tau_o = 12.5
        self.tau_d = 0.172
        self.tau_si = 127
        self.tau_v_m = 18.2
        self.tau_v_p = 10
        self.tau_w_m = 80
        self.tau_w_p = 1020
        self.k = 10
        self.u_c = 0.13
        self.uc_si = 0.85
        self.init_u = 0.0
        self.init_v = 1.0
        self.init_w = 1.0

    def select_stencil(self, cardiac_tissue):
        return _stencil_2d(cardiac_tissue)


class FentonKarma3D(FentonKarma2D):
    """(cpuwave3D/model/fenton_karma_3d.py)"""

    def select_stencil(self, cardiac_tissue):
        return _stencil_3d(cardiac_tissue)


class TP062D(CardiacModel):
    """ten Tusscher-Panfilov 2006 epicardial model (cpuwave2D/model/
    tp06_2d.py:10-240).  Parameters in the order of ionic_kernel_2d's
    signature (:1003-1012), defaults from :81-148, initial values :151-170.
    Under npfloat float32 the ion concentrations (cai, casr, cass, nai, Ki)
    stay float64; the reference's frozen Ca_i (:1098) is kept."""

    _model_id = _ffi.MODEL_TP06
    _reset_u_new = True
    _state_names = ("cai", "casr", "cass", "nai", "Ki", "m", "h", "j", "xr1",
                    "xr2", "xs", "r", "s", "d", "f", "f2", "fcass", "rr",
                    "oo")
    _param_names = ("ko", "cao", "nao", "Vc", "Vsr", "Vss", "Bufc", "Kbufc",
                    "Bufsr", "Kbufsr", "Bufss", "Kbufss", "Vmaxup", "Kup",
                    "Vrel", "k1_", "k2_", "k3", "k4", "EC", "maxsr", "minsr",
                    "Vleak", "Vxfer", "R", "F", "T", "RTONF", "CAPACITANCE",
                    "gkr", "pKNa", "gk1", "gna", "gbna", "KmK", "KmNa",
                    "knak", "gcal", "gbca", "knaca", "KmNai", "KmCa", "ksat",
                    "n_", "gpca", "KpCa", "gpk", "gto", "gks")

    def __init__(self):
        super().__init__()
        self.D_model = 0.154
        self.state_vars = ["u"] + list(self._state_names)
        self.npfloat = "float64"
        self.ko, self.cao, self.nao = 5.4, 2.0, 140.0
        self.Vc, self.Vsr, self.Vss = 0.016404, 0.001094, 0.00005468
        self.Bufc, self.Kbufc = 0.2, 0.001
        self.Bufsr, self.Kbufsr = 10.0, 0.3
        self.Bufss, self.Kbufss = 0.4, 0.00025
        self.Vmaxup, self.Kup, self.Vrel = 0.006375, 0.00025, 0.102
        self.k1_, self.k2_, self.k3, self.k4 = 0.15, 0.045, 0.060, 0.005
        self.EC, self.maxsr, self.minsr = 1.5, 2.5, 1.0
        self.Vleak, self.Vxfer = 0.00036, 0.0038
        self.R, self.F, self.T = 8314.472, 96485.3415, 310.0
        self.RTONF = 26.71376
        self.CAPACITANCE = 0.185
        self.gkr, self.pKNa, self.gk1, self.gna = 0.153, 0.03, 5.405, 14.838
        self.gbna, self.KmK, self.KmNa, self.knak = 0.00029, 1.0, 40.0, 2.724
        self.gcal, self.gbca, self.knaca = 0.00003980, 0.000592, 1000
        self.KmNai, self.KmCa, self.ksat, self.n_ = 87.5, 1.38, 0.1, 0.35
        self.gpca, self.KpCa, self.gpk = 0.1238, 0.0005, 0.0146
        self.gto, self.gks = 0.294, 0.392
        self.init_u = -84.5
        self.init_cai, self.init_casr, self.init_cass = 0.00007, 1.3, 0.00007
        self.init_nai, self.init_Ki = 7.67, 138.3
        self.init_m, self.init_h, self.init_j = 0.0, 0.75, 0.75
        self.init_xr1, self.init_xr2, self.init_xs = 0.0, 1.0, 0.0
        self.init_r, self.init_s, self.init_d = 0.0, 1.0, 0.0
        self.init_f, self.init_f2, self.init_fcass = 1.0, 1.0, 1.0
        self.init_rr, self.init_oo = 1.0, 0.0

    def select_stencil(self, cardiac_tissue):
        return _stencil_2d(cardiac_tissue)


class TP063D(TP062D):
    """(cpuwave3D/model/tp06_3d.py:36-83)"""

    def select_stencil(self, cardiac_tissue):
        return _stencil_3d(cardiac_tissue)


class Courtemanche2D(CardiacModel):
    """Courtemanche-Ramirez-Nattel 1998 atrial model (cpuwave2D/model/
    courtemanche_2d.py:10-178).  Parameters in the order of
    ionic_kernel_2d's signature (:569-577), defaults :32-83, initial values
    :85-106.  Under npfloat float32 the concentrations (nai, ki, cai, caup,
    carel) stay float64.  As in the reference, the model's ``xs`` array
    holds the IKr gate and ``xr`` the IKs gate (:152-160 against :581), and
    IKr uses the fixed conductance 0.0294 (:420-422) whatever ``gkr`` is."""

    _model_id = _ffi.MODEL_CRN
    _reset_u_new = True
    _state_names = ("nai", "ki", "cai", "caup", "carel", "m", "h", "j_", "d",
                    "f", "oa", "oi", "ua", "ui", "xr", "xs", "fca", "irel",
                    "vrel", "urel", "wrel")
    _init_names = {"j_": "j"}
    _param_names = ("gna", "gnab", "gk1", "gkr", "gks", "gto", "gcal", "gcab",
                    "gkur_coeff", "F", "T", "R", "Vc", "Vj", "Vup", "Vrel",
                    "ibk", "cao", "nao", "ko", "caupmax", "kup", "kmnai",
                    "kmko", "kmnancx", "kmcancx", "ksatncx", "kmcmdn",
                    "kmtrpn", "kmcsqn", "trpnmax", "cmdnmax", "csqnmax",
                    "inacamax", "inakmax", "ipcamax", "krel", "iupmax",
                    "kq10")

    def __init__(self):
        super().__init__()
        self.D_model = 0.154
        self.state_vars = ["u"] + list(self._state_names)
        self.npfloat = "float64"
        self.gna, self.gnab, self.gk1 = 7.8, 0.000674, 0.09
        self.gkr, self.gks, self.gto = 0.0294, 0.129, 0.1652
        self.gcal, self.gcab, self.gkur_coeff = 0.1238, 0.00113, 1
        self.F, self.T, self.R = 96485.0, 310.0, 8314.0
        self.Vc = 20100
        self.Vj = self.Vc * 0.68
        self.Vup = self.Vj * 0.06 * 0.92
        self.Vrel = self.Vj * 0.06 * 0.08
        self.ibk, self.cao, self.nao, self.ko = 0.0, 1.8, 140, 5.4
        self.caupmax, self.kup = 15, 0.00092
        self.kmnai, self.kmko = 10, 1.5
        self.kmnancx, self.kmcancx, self.ksatncx = 87.5, 1.38, 0.1
        self.kmcmdn, self.kmtrpn, self.kmcsqn = 0.00238, 0.0005, 0.8
        self.trpnmax, self.cmdnmax, self.csqnmax = 0.07, 0.05, 10.0
        self.inacamax, self.inakmax, self.ipcamax = 1600, 0.6, 0.275
        self.krel, self.iupmax, self.kq10 = 30, 0.005, 3
        self.init_u = -84.5
        self.init_nai, self.init_ki, self.init_cai = 11.2, 139, 0.000102
        self.init_caup, self.init_carel = 1.6, 1.1
        self.init_m, self.init_h, self.init_j = 0.00291, 0.965, 0.978
        self.init_d, self.init_f = 0.000137, 0.999837
        self.init_oa, self.init_oi = 0.000592, 0.9992
        self.init_ua, self.init_ui = 0.003519, 0.9987
        self.init_xs, self.init_xr, self.init_fca = 0.0187, 0.0000329, 0.775
        self.init_irel, self.init_vrel = 0, 1
        self.init_urel, self.init_wrel = 0, 0.9

    def select_stencil(self, cardiac_tissue):
        return _stencil_2d(cardiac_tissue)


class Courtemanche3D(Courtemanche2D):
    """(cpuwave3D/model/courtemanche_3d.py:40-88)"""

    def select_stencil(self, cardiac_tissue):
        return _stencil_3d(cardiac_tissue)


class Barkley2D(CardiacModel):
    """Barkley (cpuwave2D/model/barkley_2d.py:8-170)."""

    _model_id = _ffi.MODEL_BK
    _state_names = ("v",)
    _param_names = ("a", "b", "eap")

    def __init__(self):
        super().__init__()
        self.D_model = 1.
        self.state_vars = ["u", "v"]
        self.npfloat = "float64"
        self.a = 0.75
        self.b = 0.02
        self.eap = 0.02
        self.init_u = 0.0
        self.init_v = 0

    def select_stencil(self, cardiac_tissue):
        return _stencil_2d(cardiac_tissue)


class Barkley3D(Barkley2D):
    """(cpuwave3D/model/barkley_3d.py)"""

    def select_stencil(self, cardiac_tissue):
        return _stencil_3d(cardiac_tissue)


class BuenoOrovio2D(CardiacModel):
    """Bueno-Orovio minimal ventricular model (cpuwave2D/model/
    bueno_orovio_2d.py:13-180); parameters in ionic_kernel_2d's order."""

    _model_id = _ffi.MODEL_BO
    _state_names = ("v", "w", "s")
    _param_names = ("u_o", "u_u", "theta_v", "theta_w", "theta_v_m",
                    "theta_o", "tau_v1_m", "tau_v2_m", "tau_v_p", "tau_w1_m",
                    "tau_w2_m", "k_w_m", "u_w_m", "tau_w_p", "tau_fi",
                    "tau_o1", "tau_o2", "tau_so1", "tau_so2", "k_so", "u_so",
                    "tau_s1", "tau_s2", "k_s", "u_s", "tau_si", "tau_w_inf",
                    "w_inf_")

    def __init__(self):
        super().__init__()
        self.D_model = 1.
        self.state_vars = ["u", "v", "w", "s"]
        self.npfloat = "float64"
        self.u_o, self.u_u = 0.0, 1.55
        self.theta_v, self.theta_w = 0.3, 0.13
        self.theta_v_m, self.theta_o = 0.006, 0.006
        self.tau_v1_m, self.tau_v2_m, self.tau_v_p = 60, 1150, 1.4506
        self.tau_w1_m, self.tau_w2_m = 60, 15
        self.k_w_m, self.u_w_m, self.tau_w_p = 65, 0.03, 200
        self.tau_fi, self.tau_o1, self.tau_o2 = 0.11, 400, 6
        self.tau_so1, self.tau_so2 = 30.0181, 0.9957
        self.k_so, self.u_so = 2.0458, 0.65
        self.tau_s1, self.tau_s2 = 2.7342, 16
        self.k_s, self.u_s = 2.0994, 0.9087
        self.tau_si, self.tau_w_inf, self.w_inf_ = 1.8875, 0.07, 0.94
        self.init_u, self.init_v, self.init_w, self.init_s = 0.0, 1.0, 1.0, 0.0

    def select_stencil(self, cardiac_tissue):
        return _stencil_2d(cardiac_tissue)


class BuenoOrovio3D(BuenoOrovio2D):
    """(cpuwave3D/model/bueno_orovio_3d.py)"""

    def select_stencil(self, cardiac_tissue):
        return _stencil_3d(cardiac_tissue)


class LuoRudy912D(CardiacModel):
    """Luo-Rudy 1991 (cpuwave2D/model/luo_rudy91_2d.py); parameters in
    ionic_kernel_2d's order.  Under npfloat float32, cai stays float64."""

    _model_id = _ffi.MODEL_LR91
    _reset_u_new = True
    _state_names = ("m", "h", "j", "d", "f", "x", "cai")
    _param_names = ("gna", "gsi", "gk", "gk1", "gkp", "gb", "ko", "ki",
                    "nai", "nao", "cao", "R", "T", "F", "PR_NaK")

    def __init__(self):
        super().__init__()
        self.D_model = 0.1
        self.state_vars = ["u"] + list(self._state_names)
        self.npfloat = "float64"
        self.gna, self.gsi, self.gk = 23.0, 0.09, 0.282
        self.gk1, self.gkp, self.gb = 0.6047, 0.0183, 0.03921
        self.ko, self.ki, self.nai = 5.4, 145.0, 18.0
        self.nao, self.cao = 140.0, 1.8
        self.R, self.T, self.F = 8.314, 310.0, 96.5
        self.PR_NaK = 0.01833
        self.init_u = -84.5
        self.init_m, self.init_h, self.init_j = 0.0017, 0.9832, 0.995484
        self.init_d, self.init_f, self.init_x = 0.000003, 1.0, 0.0057
        self.init_cai = 0.0002

    def select_stencil(self, cardiac_tissue):
        return _stencil_2d(cardiac_tissue)


class LuoRudy913D(LuoRudy912D):
    """(cpuwave3D/model/luo_rudy91_3d.py)"""

    def select_stencil(self, cardiac_tissue):
        return _stencil_3d(cardiac_tissue)
