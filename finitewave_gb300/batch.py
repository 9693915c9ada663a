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


class TissueBatch:
    """A batch of models run together (see the module docstring).

    chunk: advance the batch in chunks of at most this many steps (None: as
    long as every model allows).  graphs: replay each chunk's launches from
    a captured CUDA graph -- the launches of a chunk depend only on its
    length and on the plan and scratch buffers (each chunk is planned at
    offset 0 into the same plan buffer), so equal chunks replay one graph
    and the per-launch host cost disappears."""

    def __init__(self, models=(), chunk=None, graphs=True):
        self.models = list(models)
        self.chunk = chunk
        self.graphs = graphs
        self._plan = None
        self._scratch = None
        self._batch = None   # the last plan's fw_batch handle
        self._graphs = {}

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
        while active:
            limit = min(_MAX_SEGMENT, min(remaining[i] for i in active))
            if self.chunk:
                limit = min(limit, int(self.chunk))
            n = min(ms[i]._segment_times(limit)[2] for i in active)
            segs = [ms[i]._prepare_segment(n) for i in active]
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
                remaining[i] -= n
                if m.command_sequence:
                    m.command_sequence.execute_next()
                if m.state_saver:
                    m.state_saver.save()
                if m.check_termination():
                    if m.state_saver:
                        m.state_saver.save()
                    continue
                if remaining[i] > 0:
                    still.append(i)
            active = still
        for m in ms:
            m._check_status()
