"""A request loop serving many simulations on one GPU.

The reference runs one simulation per ``model.run()`` call.  The server
takes simulation requests -- configured models of any family, 2D or 3D, each
with its own tissue, stimuli, trackers and ``t_max`` -- as they arrive, and

* admits them first come, first served while the device footprint of the
  admitted requests (state, weights, mesh and tracker buffers: bytes per node
  x nodes, `device_footprint`) stays within an HBM budget;
* keeps every admitted request's state resident in device memory and
  advances all of them chunk by chunk (continuous batching: a request joins
  at the next chunk boundary after its admission and leaves at the chunk
  boundary where it finishes);
* streams a finished request's tracker buffers back to pinned host memory on
  a separate copy stream (the trackers' ``output`` then reads the host
  copies) and releases its device memory;
* records arrival, admission and finish times, from which `stats` reports
  the latency percentiles (p50 / p99), the queueing / service split and the
  node-steps per second served.

Each request advances exactly as its own ``model.run()`` would (the same
segments, commands, state saver and termination checks), so its outputs do
not depend on what else is being served.
"""
import collections
import time

import numpy as np
import torch

from . import _ffi

_STATE_BYTES = {_ffi.F64: 8, _ffi.F32: 4}


def device_footprint(model):
    """Device bytes a model will hold once initialised: u and u_new, the
    state variables, the stencil weights (and the packed copy of the fused
    form), mesh and myocyte flags, and its trackers' buffers."""
    shape = tuple(np.asarray(model.cardiac_tissue.mesh).shape)
    n = int(np.prod(shape))
    prec = model._precision()
    b = _STATE_BYTES[prec]
    per_node = 2 * b + 2                                   # u, u_new, mesh, myo
    for i in range(len(model._state_names)):
        per_node += 8 if _ffi.state_is_f64(model._model_id, prec, i) else b
    stencil = model.stencil if model.stencil is not None else \
        model.select_stencil(model.cardiac_tissue)
    nw = _ffi.STENCIL_NW[stencil.kind]
    per_node += nw * b
    if prec == _ffi.F32 and len(shape) == 2:
        per_node += (nw - 1) * 4                           # packed weights
    trs = model.tracker_sequence.sequence if model.tracker_sequence else []
    for tr in trs:
        name = type(tr).__name__
        if name.startswith("ActivationTime"):
            per_node += 4
        elif name.startswith("LocalActivationTime"):
            per_node += 1 + 4 + 4 * int(getattr(tr, "capacity", 16))
    return n * per_node


class Request:
    """One simulation request: a configured model and its arrival time
    (seconds after the start of serving)."""

    def __init__(self, model, arrival=0.0, name=None):
        self.model = model
        self.arrival = float(arrival)
        self.name = name
        self.footprint = None
        self.admitted = None
        self.finished = None
        self.steps = 0
        self.myocytes = 0
        self._remaining = 0

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival

    @property
    def queueing(self):
        return None if self.admitted is None else self.admitted - self.arrival

    @property
    def service(self):
        return None if self.finished is None else self.finished - self.admitted


def _to_host(obj, copy_stream, keep):
    """Replace every CUDA tensor attribute of obj (and in its lists) by a
    pinned host copy made on copy_stream."""
    for key, val in list(vars(obj).items()):
        if isinstance(val, torch.Tensor) and val.is_cuda:
            h = torch.empty(val.shape, dtype=val.dtype, pin_memory=True)
            with torch.cuda.stream(copy_stream):
                h.copy_(val, non_blocking=True)
            keep.append(val)
            setattr(obj, key, h)
        elif isinstance(val, list):
            new = []
            for x in val:
                if isinstance(x, torch.Tensor) and x.is_cuda:
                    h = torch.empty(x.shape, dtype=x.dtype, pin_memory=True)
                    with torch.cuda.stream(copy_stream):
                        h.copy_(x, non_blocking=True)
                    keep.append(x)
                    new.append(h)
                else:
                    new.append(x)
            setattr(obj, key, new)


class SimulationServer:
    """Serve a trace of requests (see the module docstring).

    hbm_budget: bytes of device memory the admitted requests may hold
    (default: 80 % of the device's free memory at start); chunk: time steps
    a request advances between scheduling points."""

    def __init__(self, hbm_budget=None, chunk=1000, device=None):
        self.hbm_budget = hbm_budget
        self.chunk = int(chunk)
        self.device = device
        self.completed = []
        self.rejected = []
        self.t_start = None
        self.t_end = None

    def _release(self, req, copy_stream):
        m = req.model
        compute = torch.cuda.current_stream()
        copy_stream.wait_stream(compute)
        keep = []
        if m.tracker_sequence:
            for tr in m.tracker_sequence.sequence:
                _to_host(tr, copy_stream, keep)
        copy_stream.synchronize()
        del keep
        m._dev = {}
        m.weights = None
        m._wpack = None
        m._mesh_d = m._myo_d = None

    def serve(self, requests, realtime=True):
        """Run the trace; returns the completed requests in finishing
        order.  With realtime=False, arrivals are taken as already due."""
        dev = torch.device(self.device) if self.device is not None else \
            torch.device("cuda", torch.cuda.current_device())
        budget = self.hbm_budget
        if budget is None:
            free, _ = torch.cuda.mem_get_info(dev)
            budget = int(0.8 * free)
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        queue = collections.deque()
        active = []
        used = 0
        copy_stream = torch.cuda.Stream(dev)
        self.t_start = t0 = time.perf_counter()

        def now():
            return time.perf_counter() - t0

        while pending or queue or active:
            t = now()
            while pending and (not realtime or pending[0].arrival <= t):
                r = pending.popleft()
                r.footprint = device_footprint(r.model)
                if r.footprint > budget:
                    self.rejected.append(r)
                    continue
                queue.append(r)
            while queue and used + queue[0].footprint <= budget:
                r = queue.popleft()
                m = r.model
                m.initialize()
                if m.state_loader:
                    m.state_loader.load()
                r._remaining = int(np.ceil((m.t_max - m.t) / m.dt))
                r.myocytes = int(m._myo_d.sum().item())
                r.admitted = now()
                used += r.footprint
                active.append(r)
            if not active:
                if pending and realtime:
                    time.sleep(max(0.0, min(pending[0].arrival - now(), 0.01)))
                continue
            for r in active:
                m = r.model
                n = m._run_segment(min(self.chunk, r._remaining), sync=False)
                r._remaining -= n
                r.steps += n
                if m.command_sequence:
                    m.command_sequence.execute_next()
                if m.state_saver:
                    m.state_saver.save()
                if m.check_termination():
                    r._remaining = 0
            torch.cuda.current_stream().synchronize()
            still = []
            for r in active:
                if r._remaining > 0:
                    still.append(r)
                    continue
                r.model._check_status()
                self._release(r, copy_stream)
                r.finished = now()
                used -= r.footprint
                self.completed.append(r)
            active = still
        self.t_end = now()
        return self.completed

    def stats(self):
        """Latency percentiles and throughput of the completed requests."""
        done = self.completed
        if not done:
            return {"completed": 0, "rejected": len(self.rejected)}
        lat = np.array([r.latency for r in done])
        q = np.array([r.queueing for r in done])
        s = np.array([r.service for r in done])
        work = sum(r.myocytes * r.steps for r in done)
        span = max(r.finished for r in done) - min(r.arrival for r in done)
        return {
            "completed": len(done), "rejected": len(self.rejected),
            "latency_p50_s": float(np.percentile(lat, 50)),
            "latency_p99_s": float(np.percentile(lat, 99)),
            "latency_mean_s": float(lat.mean()),
            "queueing_mean_s": float(q.mean()),
            "service_mean_s": float(s.mean()),
            "myocyte_steps": int(work),
            "makespan_s": float(span),
            "value": float(work / span) if span > 0 else None,
        }
