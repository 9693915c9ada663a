"""A request loop serving many simulations on one GPU.

The reference runs one simulation per ``model.run()`` call.  The server
takes simulation requests -- configured models of any family, 2D or 3D, each
with its own tissue, stimuli, trackers and ``t_max`` -- as they arrive, and

* admits them first come, first served while the device footprint of the
  admitted requests (state, weights, mesh and tracker buffers: bytes per node
  x nodes, `device_footprint`) stays within an HBM budget;
* prepares an admitted request (``initialize()``: host mesh work, uploads,
  the weight build) on a worker thread and on the request's own CUDA stream,
  so the loop keeps issuing work for the running requests meanwhile;
* keeps every admitted request's state resident in device memory and
  advances it chunk by chunk on its own stream (continuous batching: a
  request joins as soon as it is prepared and leaves when it finishes), so
  the kernels of different requests run on the GPU at the same time; the
  loop never synchronises the device, it polls CUDA events, with at most
  `in_flight` chunks queued per request;
* streams each request's activation maps back to pinned host memory on a
  copy stream after every chunk (``Request.snapshot``) and, when it
  finishes, all its tracker buffers and its status word; its device memory
  is released once those copies have landed;
* records arrival, admission, start and finish times, and device-side
  start and end events per request, from which `stats` reports the latency
  percentiles (p50 / p99), the queueing / service split, the node-steps per
  second served and how much the requests overlapped on the device.

Each request advances exactly as its own ``model.run()`` would (the same
segments, commands, state saver and termination checks; commands and state
savers run on the host once the segment before them has completed), so its
outputs do not depend on what else is being served.
"""
import collections
import concurrent.futures
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
        per_node += 8 if (_ffi.state_is_f64(model._model_id, prec, i) or
                          _ffi.state_is_pair(model._model_id, prec, i)) else b
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
        self.started = None
        self.finished = None
        self.steps = 0
        self.myocytes = 0
        self._remaining = 0
        self._stream = None
        self._inflight = collections.deque()
        self._hostwork = False
        self._snap = []          # [(pinned host tensors, copy event)]
        self._span = None        # (start event, end event) on the device

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival

    @property
    def queueing(self):
        return None if self.admitted is None else self.admitted - self.arrival

    @property
    def service(self):
        return None if self.finished is None else self.finished - self.admitted

    def snapshot(self):
        """The most recent activation maps streamed back while the request
        runs (one host array per activation-time tracker, the tracker's
        step indices, -1 where not activated yet), or None before the first
        copy has landed."""
        for host, ev in reversed(self._snap):
            if ev is None or ev.query():
                return [h.numpy() for h in host]
        return None


class _Cuda:
    """The device operations of the loop, kept apart from the scheduling
    (which the CPU tests drive with a stand-in)."""

    def __init__(self, dev):
        self.dev = dev

    def stream(self):
        return torch.cuda.Stream(self.dev)

    def using(self, s):
        return torch.cuda.stream(s)

    def record(self, s, timing=False):
        ev = torch.cuda.Event(enable_timing=timing)
        ev.record(s)
        return ev

    def done(self, ev):
        return ev.query()

    def wait(self, s, ev):
        s.wait_event(ev)

    def to_host(self, t, s):
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        with torch.cuda.stream(s):
            h.copy_(t, non_blocking=True)
        return h

    def elapsed_ms(self, a, b):
        return a.elapsed_time(b)


def _device_tensors(obj):
    """(name, index or None, tensor) of the CUDA tensor attributes of obj,
    including those held in list attributes."""
    out = []
    for key, val in list(vars(obj).items()):
        if isinstance(val, torch.Tensor) and val.is_cuda:
            out.append((key, None, val))
        elif isinstance(val, list):
            for i, x in enumerate(val):
                if isinstance(x, torch.Tensor) and x.is_cuda:
                    out.append((key, i, x))
    return out


class SimulationServer:
    """Serve a trace of requests (see the module docstring).

    hbm_budget: bytes of device memory the admitted requests may hold
    (default: 80 % of the device's free memory at start); chunk: time steps
    a request advances per scheduling step; streams: CUDA streams the
    requests are spread over; in_flight: chunks a request may have queued
    on the device; prep_threads: worker threads preparing admitted
    requests (0: prepare in the loop); stream_back: copy the activation
    maps to the host after every chunk."""

    def __init__(self, hbm_budget=None, chunk=1000, device=None, streams=8,
                 in_flight=2, prep_threads=1, stream_back=True):
        self.hbm_budget = hbm_budget
        self.chunk = int(chunk)
        self.device = device
        self.n_streams = max(1, int(streams))
        self.in_flight = max(1, int(in_flight))
        self.prep_threads = int(prep_threads)
        self.stream_back = stream_back
        self.completed = []
        self.rejected = []
        self.t_start = None
        self.t_end = None
        self._ops = None
        self._origin = None

    # ------------------------------------------------------------ helpers
    def _prepare(self, r):
        """initialize() on the request's stream (worker thread)."""
        m = r.model
        with self._ops.using(r._stream):
            m.initialize()
            if m.state_loader:
                m.state_loader.load()
        r._remaining = int(np.ceil((m.t_max - m.t) / m.dt))
        r.myocytes = int(getattr(m, "_n_myo", 0))
        return r

    def _at_buffers(self, m):
        from .tracker import ActivationTime2DTracker
        trs = m.tracker_sequence.sequence if m.tracker_sequence else []
        return [t._act_step for t in trs
                if isinstance(t, ActivationTime2DTracker) and
                getattr(t, "_act_step", None) is not None]

    def _issue(self, r, now):
        """Queue the request's next chunk on its stream."""
        ops, m = self._ops, r.model
        if r._span is None:
            r._span = [ops.record(r._stream, timing=True), None]
            r.started = now()
        with ops.using(r._stream):
            n = m._run_segment(min(self.chunk, r._remaining), sync=False)
        r._remaining -= n
        r.steps += n
        ev = ops.record(r._stream)
        r._inflight.append(ev)
        if self.stream_back:
            bufs = self._at_buffers(m)
            if bufs:
                ops.wait(self._copy, ev)
                host = [ops.to_host(b, self._copy) for b in bufs]
                r._snap = (r._snap + [(host, ops.record(self._copy))])[-2:]
        if m.command_sequence or m.state_saver:
            # commands and savers see the state after this chunk: they run
            # when it has completed
            r._hostwork = True
        elif m.check_termination():
            r._remaining = 0

    def _host_work(self, r):
        m = r.model
        if m.command_sequence:
            m.command_sequence.execute_next()
        if m.state_saver:
            m.state_saver.save()
        if m.check_termination():
            if m.state_saver:
                m.state_saver.save()
            r._remaining = 0
        r._hostwork = False

    def _begin_release(self, r):
        """Copy the tracker buffers and the status word to pinned host
        memory on the copy stream once the request's work is done; drop
        the model's other device arrays.  Returns the copy event."""
        ops, m = self._ops, r.model
        last = ops.record(r._stream, timing=True)
        r._span[1] = last
        ops.wait(self._copy, last)
        keep = []
        if m.tracker_sequence:
            for tr in m.tracker_sequence.sequence:
                for key, i, t in _device_tensors(tr):
                    h = ops.to_host(t, self._copy)
                    keep.append(t)
                    if i is None:
                        setattr(tr, key, h)
                    else:
                        getattr(tr, key)[i] = h
        status = getattr(m, "_status", None)
        r._status_host = ops.to_host(status, self._copy) \
            if status is not None else None
        keep.append(status)
        r._keep = keep
        m._dev = {}
        m.weights = None
        m._wpack = None
        m._mesh_d = m._myo_d = None
        return ops.record(self._copy)

    def _finish_release(self, r):
        st = r._status_host
        r._keep = None
        if st is not None:
            r.model._check_status(int(st.reshape(-1)[0]))

    # ------------------------------------------------------------- serving
    def serve(self, requests, realtime=True):
        """Run the trace; returns the completed requests in finishing
        order.  With realtime=False, arrivals are taken as already due."""
        dev = torch.device(self.device) if self.device is not None else \
            torch.device("cuda", torch.cuda.current_device())
        if self._ops is None:
            self._ops = _Cuda(dev)
        ops = self._ops
        budget = self.hbm_budget
        if budget is None:
            free, _ = torch.cuda.mem_get_info(dev)
            budget = int(0.8 * free)
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        queue = collections.deque()
        preparing, active, releasing = [], [], []
        used = 0
        streams = [ops.stream() for _ in range(self.n_streams)]
        self._copy = ops.stream()
        self._origin = ops.record(streams[0], timing=True)
        pool = concurrent.futures.ThreadPoolExecutor(self.prep_threads) \
            if self.prep_threads > 0 else None
        k_stream = 0
        self.t_start = t0 = time.perf_counter()

        def now():
            return time.perf_counter() - t0

        try:
            while pending or queue or preparing or active or releasing:
                progress = False
                t = now()
                while pending and (not realtime or pending[0].arrival <= t):
                    r = pending.popleft()
                    r.footprint = device_footprint(r.model)
                    if r.footprint > budget:
                        self.rejected.append(r)
                    else:
                        queue.append(r)
                    progress = True
                while queue and used + queue[0].footprint <= budget:
                    r = queue.popleft()
                    r.admitted = now()
                    used += r.footprint
                    r._stream = streams[k_stream % len(streams)]
                    k_stream += 1
                    if pool is not None:
                        preparing.append((r, pool.submit(self._prepare, r)))
                    else:
                        preparing.append((r, None))
                        self._prepare(r)
                    progress = True
                still = []
                for r, fut in preparing:
                    if fut is None or fut.done():
                        if fut is not None:
                            fut.result()
                        active.append(r)
                        progress = True
                    else:
                        still.append((r, fut))
                preparing = still
                still = []
                for r in active:
                    while r._inflight and ops.done(r._inflight[0]):
                        r._inflight.popleft()
                        progress = True
                    if r._hostwork and not r._inflight:
                        self._host_work(r)
                        progress = True
                    if (r._remaining > 0 and not r._hostwork and
                            len(r._inflight) < self.in_flight):
                        self._issue(r, now)
                        progress = True
                    if r._remaining > 0 or r._inflight or r._hostwork:
                        still.append(r)
                    else:
                        releasing.append((r, self._begin_release(r)))
                        progress = True
                active = still
                still = []
                for r, ev in releasing:
                    if ops.done(ev):
                        self._finish_release(r)
                        r.finished = now()
                        used -= r.footprint
                        self.completed.append(r)
                        progress = True
                    else:
                        still.append((r, ev))
                releasing = still
                if not progress:
                    if pending and realtime and not (queue or preparing or
                                                     active or releasing):
                        time.sleep(max(0.0, min(pending[0].arrival - now(),
                                                0.01)))
                    else:
                        time.sleep(5e-5)
        finally:
            if pool is not None:
                pool.shutdown(wait=True)
        self.t_end = now()
        return self.completed

    def device_spans(self):
        """(name, start ms, end ms) of every completed request on the
        device timeline: from before its first chunk to after its last,
        relative to the start of serving."""
        out = []
        for r in self.completed:
            if r._span is None or r._span[1] is None:
                continue
            a = self._ops.elapsed_ms(self._origin, r._span[0])
            b = self._ops.elapsed_ms(self._origin, r._span[1])
            out.append((r.name, a, b))
        return out

    def stats(self):
        """Latency percentiles, throughput and device overlap of the
        completed requests."""
        done = self.completed
        if not done:
            return {"completed": 0, "rejected": len(self.rejected)}
        lat = np.array([r.latency for r in done])
        q = np.array([r.queueing for r in done])
        s = np.array([r.service for r in done])
        work = sum(r.myocytes * r.steps for r in done)
        span = max(r.finished for r in done) - min(r.arrival for r in done)
        out = {
            "completed": len(done), "rejected": len(self.rejected),
            "latency_p50_s": float(np.percentile(lat, 50)),
            "latency_p99_s": float(np.percentile(lat, 99)),
            "latency_mean_s": float(lat.mean()),
            "queueing_p50_s": float(np.percentile(q, 50)),
            "queueing_p99_s": float(np.percentile(q, 99)),
            "queueing_mean_s": float(q.mean()),
            "service_p50_s": float(np.percentile(s, 50)),
            "service_mean_s": float(s.mean()),
            "service_sum_s": float(s.sum()),
            "myocyte_steps": int(work),
            "makespan_s": float(span),
            "value": float(work / span) if span > 0 else None,
        }
        spans = self.device_spans() if self._origin is not None else []
        if spans:
            iv = sorted((a, b) for _, a, b in spans)
            union, cur_a, cur_b = 0.0, iv[0][0], iv[0][1]
            for a, b in iv[1:]:
                if a > cur_b:
                    union += cur_b - cur_a
                    cur_a, cur_b = a, b
                else:
                    cur_b = max(cur_b, b)
            union += cur_b - cur_a
            total = sum(b - a for a, b in iv)
            out["device_span_sum_ms"] = float(total)
            out["device_span_union_ms"] = float(union)
            out["device_overlap"] = float(total / union) if union > 0 else None
        return out
