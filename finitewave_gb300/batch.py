"""Many independent 2D tissues advanced together on one GPU.

The reference runs one ``CardiacModel.run`` loop per tissue
(core/model/cardiac_model.py:130-189).  ``TissueBatch`` takes any number of
already configured float32 2D models -- Aliev-Panfilov, Mitchell-Schaeffer or
Fenton-Karma, isotropic or anisotropic, each with its own tissue, size,
parameters, stimuli and trackers -- and advances all of them through one
persistent kernel per K time steps over a ragged list of tiles
(``fw_batch_plan`` / ``fw_batch_run``).  Each model ends exactly as its own
``model.run()`` would leave it (same time accumulation, stimulus and tracker
windows, commands, state saver and termination checks between segments).

Per tissue: at most one activation-time and one local-activation-time
tracker, no probe trackers.
"""
import ctypes

import numpy as np
import torch

from . import _ffi, stimulation, tracker
from .model import _MAX_SEGMENT
from .tracker import (ActivationTime2DTracker, LocalActivationTime2DTracker)

_BATCH_MODELS = (_ffi.MODEL_AP, _ffi.MODEL_MS, _ffi.MODEL_FK)


class _Mirror:
    """Copies of one model's arrays that the TMA form of the batched kernel
    reads through tensor maps -- the two potential buffers, the two buffers
    of each state variable, the myocyte flags, the weights (plus their
    node-major packing) and the local activation tracker's flags -- with
    rows padded to a multiple of 16 nodes (the row pitch a tensor map
    needs).  The padding columns are non-myocytes holding zero in both
    potential buffers.  The batch advances the copies; `sync_in` and
    `sync_out` move the model's state between them and the model's own
    arrays, and `swap` follows the model's u / u_new exchange."""

    def __init__(self, m):
        ni, nj = m._shape()
        self.model, self.nj = m, nj
        self.pitch = -(-nj // 16) * 16
        self.weights_src = m.weights
        dev = m._device()
        f32 = torch.float32
        nw = m.weights.shape[0]
        self.w = torch.zeros((nw, ni, self.pitch), dtype=f32, device=dev)
        self.w[:, :, :nj] = m.weights.view(nw, ni, nj)
        nwo = 4 if m.stencil.kind == _ffi.ISO5 else 8
        self.wpack = torch.empty(ni * self.pitch * nwo, dtype=f32, device=dev)
        _ffi.call("fw_pack_weights", m.stencil.kind, self.w.data_ptr(),
                  ni * self.pitch, self.wpack.data_ptr(),
                  torch.cuda.current_stream(dev).cuda_stream)
        self.myo = torch.zeros((ni, self.pitch), dtype=torch.int8, device=dev)
        self.myo[:, :nj] = m._myo_d
        self.u = [torch.zeros((ni, self.pitch), dtype=f32, device=dev)
                  for _ in range(2)]
        self.state = [torch.zeros((ni, self.pitch), dtype=f32, device=dev)
                      for _ in m._state_names]
        self.state_b = [torch.zeros((ni, self.pitch), dtype=f32, device=dev)
                        for _ in m._state_names]
        # device address of a tracker's flags -> (flags, padded copy)
        self.act = {}

    def valid_for(self, m):
        return m is self.model and m.weights is self.weights_src

    def _lat_flags(self):
        seq = self.model.tracker_sequence
        if not seq:
            return []
        return [tr._activated for tr in seq.sequence
                if isinstance(tr, LocalActivationTime2DTracker)
                and tracker.is_native(tr)
                and getattr(tr, "_activated", None) is not None]

    def sync_in(self):
        m, nj = self.model, self.nj
        ni = self.u[0].shape[0]
        self.u[0][:, :nj].copy_(m._dev["u"])
        self.u[1][:, :nj].copy_(m._dev["u_new"])
        for t, tb, name in zip(self.state, self.state_b, m._state_names):
            t[:, :nj].copy_(m._dev[name])
            tb[:, :nj].copy_(m._dev[name])
        act = {}
        for f in self._lat_flags():
            old = self.act.get(f.data_ptr())
            if old is not None and old[0] is f:
                pad = old[1]
            else:
                pad = torch.zeros((ni, self.pitch), dtype=torch.uint8,
                                  device=f.device)
            pad[:, :nj].copy_(f.view(ni, nj))
            act[f.data_ptr()] = (f, pad)
        self.act = act

    def sync_out(self):
        m, nj = self.model, self.nj
        ni = self.u[0].shape[0]
        m._dev["u"].copy_(self.u[0][:, :nj])
        m._dev["u_new"].copy_(self.u[1][:, :nj])
        for t, name in zip(self.state, m._state_names):
            m._dev[name].copy_(t[:, :nj])
        for f, pad in self.act.values():
            f.view(ni, nj).copy_(pad[:, :nj])

    def swap(self):
        self.u.reverse()
        self.state, self.state_b = self.state_b, self.state

    def apply(self, a):
        """Point a tissue's fw_step_args at the copies."""
        a.u[0], a.u[1] = self.u[0].data_ptr(), self.u[1].data_ptr()
        for i, (t, tb) in enumerate(zip(self.state, self.state_b)):
            a.state[i] = t.data_ptr()
            a.state_b[i] = tb.data_ptr()
        a.myo = self.myo.data_ptr()
        a.weights = self.w.data_ptr()
        a.weights_packed = self.wpack.data_ptr()
        for k in range(a.n_lat):
            pad = self.act.get(a.lat[k].activated)
            if pad is None:
                raise RuntimeError("TissueBatch: a local activation tracker "
                                   "was not set up before the run")
            a.lat[k].activated = pad[1].data_ptr()
        a.pitch = self.pitch
        a.fused_variant = 0


class TissueBatch:
    """A batch of models run together (see the module docstring).

    chunk: advance the batch in chunks of at most this many steps (None: as
    long as every model allows).  graphs: replay each chunk's launches from
    a captured CUDA graph -- the launches of a chunk depend only on its
    length and on the plan and scratch buffers (each chunk is planned at
    offset 0 into the same plan buffer), so equal chunks replay one graph
    and the per-launch host cost disappears.  kernel: "tma" (default) runs
    the TMA pipeline over row-padded copies of the tissues' arrays (made
    once per model and kept by the batch, about 90 bytes per node), state
    copied in at the start of run() and out at its end and around host-side
    commands and state savers; "pairs" runs the same pipeline with 2 x 2
    nodes per thread advanced in two-wide float32 instructions (the same
    bits as "tma"); "cp.async" runs the kernel that stages with 4-byte
    asynchronous copies straight from the models' arrays."""

    def __init__(self, models=(), chunk=None, graphs=True, kernel="tma"):
        if kernel not in ("tma", "pairs", "cp.async"):
            raise ValueError("kernel must be 'tma', 'pairs' or 'cp.async'")
        self.models = list(models)
        self.chunk = chunk
        self.graphs = graphs
        self.kernel = kernel
        self._plan = None
        self._scratch = None
        self._batch = None   # the last plan's fw_batch handle
        self._graphs = {}
        self._mirrors = {}

    def _mirror(self, m):
        mir = self._mirrors.get(id(m))
        if mir is None or not mir.valid_for(m):
            mir = _Mirror(m)
            self._mirrors[id(m)] = mir
        return mir

    def add(self, model):
        self.models.append(model)

    # ---------------------------------------------------------------- checks
    @staticmethod
    def _check(model):
        name = type(model).__name__
        if (model._precision() != _ffi.F32 or
                model._model_id not in _BATCH_MODELS or
                model.stencil.kind not in (_ffi.ISO5, _ffi.ANISO9)):
            raise ValueError(f"{name}: a batch takes 2D float32 Aliev-Panfilov"
                             " / Mitchell-Schaeffer / Fenton-Karma models")
        if model._special:
            raise ValueError(f"{name}: special boundaries are not supported "
                             "in a batch")
        trs = model.tracker_sequence.sequence if model.tracker_sequence \
            else []
        n_at = sum(isinstance(t, ActivationTime2DTracker) for t in trs)
        n_lat = sum(isinstance(t, LocalActivationTime2DTracker) for t in trs)
        if (n_at > 1 or n_lat > 1 or n_at + n_lat != len(trs) or
                not all(tracker.is_native(t) for t in trs)):
            raise ValueError(f"{name}: a batched tissue takes at most one "
                             "activation-time and one local-activation-time "
                             "tracker, and no probe trackers")
        stims = model.stim_sequence.sequence if model.stim_sequence else []
        if not all(stimulation.is_native(s) for s in stims):
            raise ValueError(f"{name}: a batched tissue takes only this "
                             "package's stimulus classes (a stimulus with "
                             "its own stimulate() needs model.run())")
        if not model._fused_ok():
            raise ValueError(f"{name}: u and u_new must be equal at the "
                             "non-myocyte nodes")

    def _device(self):
        devs = {str(m._device()) for m in self.models}
        if len(devs) != 1:
            raise ValueError(f"batched models are on several devices: {devs}")
        return self.models[0]._device()

    def _buffers(self, plan_bytes, dev):
        if self._plan is None or self._plan.numel() < plan_bytes or \
                self._plan.device != dev:
            self._plan = torch.empty(max(2 * plan_bytes, 1 << 16),
                                     dtype=torch.uint8, device=dev)
            self._graphs = {}     # captured against the old buffer
        if self._scratch is None or self._scratch.device != dev:
            nb = ctypes.c_int64()
            _ffi.call("fw_batch_scratch_size", ctypes.byref(nb))
            # zero once; every launch leaves it zero
            self._scratch = torch.zeros(nb.value, dtype=torch.uint8,
                                        device=dev)
        return self._plan, self._scratch

    def _launch(self, b, scratch, n, dev):
        """fw_batch_run(b, scratch, 0, n), replayed from a CUDA graph when
        the same launches were captured before."""
        stream = torch.cuda.current_stream(dev)
        if not self.graphs:
            _ffi.call("fw_batch_run", ctypes.byref(b), scratch.data_ptr(), 0,
                      n, stream.cuda_stream)
            return
        key = (n, b.plan, b.n_tissues, b.n_tiles, b.ksteps, b.grid,
               scratch.data_ptr())
        g = self._graphs.get(key)
        if g is None:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                _ffi.call("fw_batch_run", ctypes.byref(b),
                          scratch.data_ptr(), 0, n,
                          torch.cuda.current_stream().cuda_stream)
            self._graphs[key] = g
        g.replay()

    # ------------------------------------------------------------------ run
    def run(self, initialize=True):
        """Run every model to its own t_max (cardiac_model.py:130-189 per
        model, all models on the device together)."""
        ms = self.models
        if not ms:
            return
        if initialize:
            for m in ms:
                m.initialize()
        for m in ms:
            if m.t_max < m.t:
                raise ValueError("t_max must be greater than current t.")
            if m.state_loader:
                m.state_loader.load()
            m._nonmyo_equal = None
            self._check(m)
        dev = self._device()
        remaining = [int(np.ceil((m.t_max - m.t) / m.dt)) for m in ms]
        active = [i for i in range(len(ms)) if remaining[i] > 0]
        stream = torch.cuda.current_stream(dev).cuda_stream
        tma = self.kernel in ("tma", "pairs")
        mirrors = [self._mirror(m) for m in ms] if tma else None
        if tma:
            for mir in mirrors:
                mir.sync_in()
        while active:
            limit = min(_MAX_SEGMENT, min(remaining[i] for i in active))
            if self.chunk:
                limit = min(limit, int(self.chunk))
            n = min(ms[i]._segment_times(limit)[2] for i in active)
            segs = [ms[i]._prepare_segment(n) for i in active]
            for i, seg in zip(active, segs):
                if tma:
                    mirrors[i].apply(seg.args)
                    if self.kernel == "pairs":
                        seg.args.fused_variant = 6
                else:
                    seg.args.fused_variant = 1
            k = len(segs)
            ptrs = (ctypes.c_void_p * k)(
                *[ctypes.addressof(s.args) for s in segs])
            n_begin = (ctypes.c_int64 * k)(*[s.n0 for s in segs])
            size = ctypes.c_int64()
            _ffi.call("fw_batch_plan_size", ptrs, k, ctypes.byref(size))
            plan, scratch = self._buffers(size.value, dev)
            b = _ffi.Batch()
            _ffi.call("fw_batch_plan", ptrs, k, n_begin, plan.data_ptr(),
                      plan.numel(), ctypes.byref(b), stream)
            self._launch(b, scratch, n, dev)
            self._batch = b
            still = []
            for i, seg in zip(active, segs):
                m = ms[i]
                m._finish_segment(seg)
                if tma and seg.n_seg % 2 == 1:
                    mirrors[i].swap()
                remaining[i] -= n
                host = tma and (m.command_sequence or m.state_saver)
                if host:
                    mirrors[i].sync_out()
                if m.command_sequence:
                    m.command_sequence.execute_next()
                if m.state_saver:
                    m.state_saver.save()
                if host:
                    mirrors[i].sync_in()
                if m.check_termination():
                    if m.state_saver:
                        m.state_saver.save()
                    continue
                if remaining[i] > 0:
                    still.append(i)
            active = still
        if tma:
            for mir in mirrors:
                mir.sync_out()
        for m in ms:
            m._check_status()
