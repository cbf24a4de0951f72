"""Continuous-batching PSF server (serving form; lentil has no server).

Requests (one broadband PSF each: pupil amplitude and OPD, wavelengths and
weights, optics) are queued by any thread and scheduled by one GPU thread:

- plans (the resident DFT matrices and operand buffers of one optics /
  wavelength set) live in an LRU cache whose device bytes are admitted
  against an HBM budget; idle plans are evicted to make room, a request that
  alone exceeds the budget fails with MemoryError;
- every scheduling pass takes the oldest request whose plan is idle,
  batches the queued requests with the same plan (up to the plan's batch
  capacity) and launches them on a free CUDA stream, so requests that arrive
  while others run are admitted as plans and streams free up, and different
  plans' work overlaps on the device;
- each (plan, batch count) launch sequence is captured once into a CUDA
  graph and replayed;
- completion is detected with CUDA events; latency is submit -> result.
"""
import collections
import concurrent.futures
import threading
import time

import numpy as np
import torch

from . import _device as dv
from . import _lib
from . import util
from .broadband import make_plan, plan_geometry
from .ptype import pupil as PUPIL


class PSFRequest:
    """One broadband PSF: sum_lambda w * |propagate_dft(Wavefront(lambda) * pupil)|^2."""

    def __init__(self, amp, opd, wavelengths, weights, pixelscale_in, focal_length,
                 det_pixelscale, det_shape, oversample=2):
        self.amp = np.ascontiguousarray(amp, dtype=np.float64)   # mask applied
        self.opd = np.ascontiguousarray(opd, dtype=np.float64)
        self.wavelengths = np.atleast_1d(np.asarray(wavelengths, dtype=np.float64))
        self.weights = np.atleast_1d(np.asarray(weights, dtype=np.float64))
        self.pixelscale_in = float(pixelscale_in)
        self.focal_length = float(focal_length)
        self.det_pixelscale = float(det_pixelscale)
        self.det_shape = int(det_shape)
        self.oversample = int(oversample)
        self.future = concurrent.futures.Future()
        self.t_submit = self.t_done = None

    def key(self, precision):
        k = getattr(self, '_key', None)
        if k is None or k[0] != precision:
            s = util.boundary_slice(self.amp)
            k = (precision, (self.amp.shape, self.wavelengths.tobytes(), self.pixelscale_in,
                             self.focal_length, self.det_pixelscale, self.det_shape,
                             self.oversample, precision,
                             (s[0].start, s[0].stop, s[1].start, s[1].stop)))
            self._key = k
        return k[1]

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_submit


def plan_bytes_estimate(plane_shape, fslice, window, L, batch, precision):
    """Device bytes of a plan (mirrors the plan's own carve-out)."""
    m, n = fslice[2], fslice[3]
    M, N = window
    ru = lambda a, b: (a + b - 1) // b * b
    if precision == 'fp64':
        return 16 * (L * (M * m + n * N) + batch * L * (m * n + M * n + M * N))
    kp1, kp2 = ru(m, 32), ru(n, 32)
    e = L * ((ru(M, 64) // 64 * 128) * 2 * kp1 + (ru(N, 128) // 128 * 256) * 2 * kp2) * 4
    ops = batch * L * (n * 2 * kp1 + M * 2 * kp2) * 4 + batch * M * ru(N, 4) * 4
    return e + ops


class _Slot:
    """A cached plan with static device/pinned buffers and captured graphs."""

    def __init__(self, key, geo, batch, precision, device):
        self.key, self.geo, self.batch = key, geo, batch
        self.plan = make_plan(geo, batch=batch, precision=precision)
        H, W = geo.plane_shape
        L = len(geo.wavelengths)
        self.A = torch.zeros((batch, H, W), dtype=torch.float64, device=device)
        self.O = torch.zeros_like(self.A)
        self.Wt = torch.zeros((batch, L), dtype=torch.float64, device=device)
        self.out = torch.zeros((batch,) + geo.shape_out, dtype=torch.float64, device=device)
        self.hA = torch.zeros((batch, H, W), dtype=torch.float64).pin_memory()
        self.hO = torch.zeros_like(self.hA).pin_memory()
        self.hW = torch.zeros((batch, L), dtype=torch.float64).pin_memory()
        self.hout = torch.zeros((batch,) + geo.shape_out, dtype=torch.float64).pin_memory()
        self.bytes = (self.plan.nbytes + 8 * (self.A.numel() * 2 + self.Wt.numel() + self.out.numel()))
        self.graphs = {}
        self.busy = False

    def run(self, n, stream, use_graphs):
        """Launch the first n PSFs on ``stream`` (inputs already staged)."""
        with torch.cuda.stream(stream):
            self.A[:n].copy_(self.hA[:n], non_blocking=True)
            self.O[:n].copy_(self.hO[:n], non_blocking=True)
            self.Wt[:n].copy_(self.hW[:n], non_blocking=True)
            if use_graphs:
                g = self.graphs.get(n)
                if g is None:
                    # warm up once outside capture, then capture the launch sequence
                    self.plan.execute(self.A[:n], self.O[:n], self.Wt[:n], out=self.out[:n], check=False)
                    g = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g, stream=stream):
                        self.plan.execute(self.A[:n], self.O[:n], self.Wt[:n], out=self.out[:n],
                                          check=False)
                    self.graphs[n] = g
                g.replay()
            else:
                self.plan.execute(self.A[:n], self.O[:n], self.Wt[:n], out=self.out[:n], check=False)
            self.hout[:n].copy_(self.out[:n], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        return ev


class PSFServer:
    """Continuous-batching broadband PSF server on one GPU."""

    def __init__(self, hbm_budget=None, streams=4, max_batch=4, precision='split',
                 use_graphs=True, device=None):
        self.device = device or dv.device()
        free, total = torch.cuda.mem_get_info(self.device)
        self.budget = int(hbm_budget) if hbm_budget else int(0.7 * free)
        self.precision = precision
        self.max_batch = max_batch
        self.use_graphs = use_graphs
        self.n_streams = streams
        self._queue = collections.deque()
        self._cv = threading.Condition()
        self._slots = collections.OrderedDict()     # key -> _Slot, LRU order
        self._bytes = 0
        self._inflight = []                          # (event, slot, requests, stream index)
        self._free_streams = list(range(streams))
        self._streams = []
        self._stop = False
        self.stats = collections.Counter()
        self._error = None
        self._thread = threading.Thread(target=self._loop, name='psf-server', daemon=True)
        self._thread.start()

    # ------------------------------------------------------------ public
    def submit(self, req):
        if req.future.done():                      # a request object may be submitted again
            req.future = concurrent.futures.Future()
            req.t_done = None
        req.t_submit = time.perf_counter()
        with self._cv:
            if self._stop:
                raise RuntimeError('server closed')
            self._queue.append(req)
            self._cv.notify()
        return req.future

    def cancel(self, req):
        """Remove a queued (not yet launched) request; True if it was removed."""
        with self._cv:
            try:
                self._queue.remove(req)
            except ValueError:
                return False
        req.future.cancel()
        self.stats['cancelled'] += 1
        return True

    def close(self, wait=True):
        with self._cv:
            self._stop = True
            self._cv.notify()
        if wait:
            self._thread.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---------------------------------------------------------- scheduler
    def _loop(self):
        torch.cuda.set_device(self.device)
        self._streams = [torch.cuda.Stream(device=self.device) for _ in range(self.n_streams)]
        while True:
            progressed = self._poll()
            progressed |= self._admit()
            with self._cv:
                if self._stop and not self._queue and not self._inflight:
                    return
                if not progressed:
                    self._cv.wait(timeout=0.0002)

    def _poll(self):
        done = [x for x in self._inflight if x[0].query()]
        for item in done:
            ev, slot, reqs, si = item
            self._inflight.remove(item)
            now = time.perf_counter()
            try:
                _lib.call('lgb_psf_plan_status', slot.plan._h, self._streams[si].cuda_stream)
                err = None
            except Exception as e:                     # device timeout or CUDA error
                err = e
            for k, r in enumerate(reqs):
                r.t_done = now
                if r.future.done():
                    continue
                if err is None:
                    r.future.set_result(slot.hout[k].numpy().copy())
                else:
                    r.future.set_exception(err)
            slot.busy = False
            self._free_streams.append(si)
            self.stats['completed'] += len(reqs)
        return bool(done)

    def _geometry(self, req):
        s = util.boundary_slice(req.amp)
        return plan_geometry(req.amp.shape, s, [], np.broadcast_to(req.pixelscale_in, (2,)),
                             req.focal_length, PUPIL, req.wavelengths, req.det_pixelscale,
                             shape=req.det_shape, oversample=req.oversample)

    def _make_room(self, need):
        for key in list(self._slots):
            if self._bytes + need <= self.budget:
                break
            slot = self._slots[key]
            if not slot.busy:
                del self._slots[key]
                self._bytes -= slot.bytes
                del slot
                self.stats['evicted'] += 1
        return self._bytes + need <= self.budget

    def _slot_for(self, req):
        key = req.key(self.precision)
        slot = self._slots.get(key)
        if slot is not None:
            self._slots.move_to_end(key)
            self.stats['plan_hits'] += 1
            return slot, key
        geo = self._geometry(req)
        if geo.window_shape is None:
            return 'empty', key
        L = len(geo.wavelengths)
        batch = self.max_batch
        est = plan_bytes_estimate(geo.plane_shape, geo.fslice, geo.window_shape, L, batch,
                                  self.precision)
        while batch > 1 and est > self.budget // 4:
            batch //= 2
            est = plan_bytes_estimate(geo.plane_shape, geo.fslice, geo.window_shape, L, batch,
                                      self.precision)
        if est > self.budget:
            return 'too_big', key
        if not self._make_room(int(est * 1.1)):
            return None, key                          # wait for running work to finish
        slot = _Slot(key, geo, batch, self.precision, self.device)
        self._slots[key] = slot
        self._bytes += slot.bytes
        self.stats['plans_built'] += 1
        return slot, key

    def _admit(self):
        progressed = False
        while self._free_streams:
            with self._cv:
                pending = list(self._queue)
            if not pending:
                break
            chosen = None
            for req in pending:                       # oldest request whose plan is free
                key = req.key(self.precision)
                s = self._slots.get(key)
                if s is not None and s.busy:
                    continue
                slot, key = self._slot_for(req)
                if slot == 'too_big':
                    with self._cv:
                        self._queue.remove(req)
                    req.future.set_exception(MemoryError(
                        'request needs more device memory than the server budget'))
                    self.stats['rejected'] += 1
                    progressed = True
                    continue
                if slot == 'empty':
                    with self._cv:
                        self._queue.remove(req)
                    req.t_done = time.perf_counter()
                    req.future.set_result(np.zeros((req.det_shape * req.oversample,) * 2))
                    progressed = True
                    continue
                if slot is None:
                    continue
                chosen = (slot, key)
                break
            if chosen is None:
                break
            slot, key = chosen
            with self._cv:
                batch = [r for r in self._queue if r.key(self.precision) == key][:slot.batch]
                for r in batch:
                    self._queue.remove(r)
            keep = slot.geo.keep
            for k, r in enumerate(batch):
                slot.hA[k].numpy()[...] = r.amp
                slot.hO[k].numpy()[...] = r.opd
                slot.hW[k].numpy()[...] = r.weights[keep]
            si = self._free_streams.pop(0)
            slot.busy = True
            ev = slot.run(len(batch), self._streams[si], self.use_graphs)
            self._inflight.append((ev, slot, batch, si))
            self.stats['launches'] += 1
            self.stats['batched'] += len(batch)
            progressed = True
        return progressed
