"""Continuous-batching PSF server (serving form; lentil has no server).

Requests (one broadband PSF each: pupil amplitude and OPD, wavelengths and
weights, optics) are queued by any thread and scheduled by one GPU thread:

- the server holds a spectral grid; a plan built on the grid (the resident
  DFT matrices of every grid wavelength for one optics geometry) serves every
  request whose wavelengths lie on the grid, by wavelength subset -- a
  device-resident DFT-matrix cache.  Requests off the grid get a plan of
  their own wavelengths;
- plans live in an LRU cache whose device bytes are admitted against an HBM
  budget; plans without launches in flight are evicted to make room, a
  request whose plan alone exceeds the budget fails with MemoryError;
- every scheduling pass takes the oldest request, batches the queued
  requests with the same plan and wavelength subset (up to ``max_batch``)
  and launches them on a free CUDA stream with operand buffers of their own,
  so requests that arrive while others run are admitted as streams free up,
  and launches (of the same plan or of different plans) overlap on the
  device;
- a launch issued while others are in flight shares the GPU, so it runs the
  tensor-core tile with the best throughput per SM (256 columns); a launch
  issued onto an idle GPU takes the autotuner's width for its launch class
  (``lentil_gb300.tuner``), which may be the narrower tile when it alone
  cannot occupy every CTA pair;
- a small launch shape seen twice keeps its buffers and is captured into a
  CUDA graph (one per tile width; for the tuned width only once the tuner has
  decided the launch class) that later launches replay;
- completion is detected with CUDA events; latency is submit -> result;
- pupils and OPD bases can be made device-resident once
  (``PSFServer.resident_pupil`` / ``resident_basis``): a request that names
  a resident pupil and gives its OPD as modal coefficients of a resident
  basis sends only its coefficients to the device (the OPD map is expanded
  there by ``lgb_basis_expand``), and its geometry key needs no scan of the
  amplitude; requests with plain arrays are staged through pinned memory;
- a request whose plan cannot be built, or a launch whose buffers cannot be
  allocated, fails with that exception while the server keeps serving; any
  other error of the scheduling loop fails the queued requests instead of
  leaving their futures waiting.
"""
import itertools
import collections
import concurrent.futures
import threading
import time

import numpy as np
import torch

from . import _device as dv
from . import _lib
from . import tuner
from . import util
from .broadband import make_plan, plan_geometry
from .ptype import pupil as PUPIL


_resident_ids = itertools.count(1)


class Resident:
    """A pupil-plane array held on the device for the life of the object:
    a pupil amplitude (float64 [H, W], mask applied, with its boundary slice
    computed once) or an OPD basis (float32 [K, H, W]).  Made by
    ``PSFServer.resident_pupil`` / ``resident_basis``; requests refer to it
    instead of carrying the array."""

    def __init__(self, array, dtype, device, slice_=None):
        self.tensor = torch.as_tensor(np.ascontiguousarray(array), dtype=dtype).to(device)
        torch.cuda.current_stream(device).synchronize()   # on the device before any launch reads it
        self.shape = tuple(self.tensor.shape)
        self.key = next(_resident_ids)
        self.slice = slice_


class PSFRequest:
    """One broadband PSF: sum_lambda w * |propagate_dft(Wavefront(lambda) * pupil)|^2.

    ``amp``: amplitude array (mask applied) or a resident pupil.  ``opd``:
    OPD map (metres), or, with ``opd_basis`` (a resident basis of K modes),
    the K modal coefficients of the OPD."""

    def __init__(self, amp, opd, wavelengths, weights, pixelscale_in, focal_length,
                 det_pixelscale, det_shape, oversample=2, opd_basis=None):
        self.amp = amp if isinstance(amp, Resident) else np.ascontiguousarray(amp, dtype=np.float64)
        self.opd_basis = opd_basis
        if opd_basis is not None:
            if not isinstance(opd_basis, Resident) or len(opd_basis.shape) != 3:
                raise TypeError('opd_basis must be a resident basis (PSFServer.resident_basis)')
            self.opd = np.ascontiguousarray(opd, dtype=np.float64).reshape(-1)
            if self.opd.size != opd_basis.shape[0]:
                raise ValueError('one OPD coefficient per basis mode')
            if opd_basis.shape[1:] != self.plane_shape:
                raise ValueError('OPD basis and pupil shapes differ')
        else:
            self.opd = np.ascontiguousarray(opd, dtype=np.float64)
            if self.opd.shape != self.plane_shape:
                raise ValueError('OPD and pupil shapes differ')
        self.wavelengths = np.atleast_1d(np.asarray(wavelengths, dtype=np.float64))
        self.weights = np.atleast_1d(np.asarray(weights, dtype=np.float64))
        if self.weights.shape != self.wavelengths.shape:
            raise ValueError('one weight per wavelength')
        self.pixelscale_in = float(pixelscale_in)
        self.focal_length = float(focal_length)
        self.det_pixelscale = float(det_pixelscale)
        self.det_shape = int(det_shape)
        self.oversample = int(oversample)
        self.future = concurrent.futures.Future()
        self.t_submit = self.t_launch = self.t_done = None
        self._geo_key = None

    @property
    def plane_shape(self):
        return tuple(self.amp.shape)

    def field_slice(self):
        if isinstance(self.amp, Resident):
            return self.amp.slice
        return util.boundary_slice(self.amp)

    def geometry_key(self):
        if self._geo_key is None:
            s = self.field_slice()
            self._geo_key = (self.plane_shape, self.pixelscale_in, self.focal_length,
                             self.det_pixelscale, self.det_shape, self.oversample,
                             (s[0].start, s[0].stop, s[1].start, s[1].stop))
        return self._geo_key

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_submit

    @property
    def queue_wait(self):
        """Seconds from submission to the launch that computed the request."""
        return None if self.t_launch is None else self.t_launch - self.t_submit


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
    flags = batch * (kp1 // 32) * 8 * ((kp2 + 255) // 256)    # field nonzero flags
    return e + ops + flags


class _Buffers:
    """Device and pinned host buffers of one launch shape (n PSFs, n_sel
    wavelengths), optionally with the launch captured as a CUDA graph."""

    KMAX = 1024                   # modal coefficients per PSF (lgb_basis_expand's limit)

    def __init__(self, slot, n, n_sel, device):
        H, W = slot.geo.plane_shape
        self.n, self.n_sel = n, n_sel
        self.shape_out = (n,) + slot.geo.shape_out
        self.A = torch.empty((n, H, W), dtype=torch.float64, device=device)
        self.O = torch.empty_like(self.A)
        self.Wt = torch.empty(n * n_sel, dtype=torch.float64, device=device)
        self.lam = torch.empty(n_sel, dtype=torch.int32, device=device)
        self.C = torch.empty((n, self.KMAX), dtype=torch.float64, device=device)
        self.out = torch.empty(self.shape_out, dtype=torch.float64, device=device)
        self.ws = torch.empty(max(1, slot.plan.workspace_bytes(n, n_sel)), dtype=torch.uint8,
                              device=device)
        self.hA = self.hO = None      # pinned staging of plain arrays, made when first needed
        self.hW = torch.empty(n * n_sel, dtype=torch.float64, pin_memory=True)
        self.hlam = torch.empty(n_sel, dtype=torch.int32, pin_memory=True)
        self.hC = torch.empty((n, self.KMAX), dtype=torch.float64, pin_memory=True)
        self.hout = None              # this launch's results (pinned, handed to the requests)
        self.reqs = []
        self.graphs = {}              # tile width -> captured launch
        self.busy = False

    def stage(self, slot, batch):
        """Host side of a launch: plain arrays into pinned staging, modal
        coefficients, weights and the wavelength subset."""
        self.reqs = batch
        hW = self.hW.view(len(batch), self.n_sel).numpy()
        hC = self.hC.numpy()
        for k, r in enumerate(batch):
            if not isinstance(r.amp, Resident):
                if self.hA is None:
                    self.hA = torch.empty(tuple(self.A.shape), dtype=torch.float64, pin_memory=True)
                self.hA[k].numpy()[...] = r.amp
            if r.opd_basis is not None:
                hC[k, :r.opd.size] = r.opd
            else:
                if self.hO is None:
                    self.hO = torch.empty(tuple(self.O.shape), dtype=torch.float64, pin_memory=True)
                self.hO[k].numpy()[...] = r.opd
            hW[k] = r.weights if slot.grid else r.weights[slot.geo.keep]
        if slot.grid:
            self.hlam.numpy()[...] = batch[0]._subset
        # results land in a block of torch's caching host allocator that the
        # requests keep (no copy on the scheduling thread)
        self.hout = torch.empty(self.shape_out, dtype=torch.float64, pin_memory=True)

    def load(self, slot, stream):
        """Device side of the inputs, on ``stream``: resident pupils copied
        on the device, plain arrays from pinned staging, modal OPDs expanded
        from their coefficients."""
        P = self.A.shape[1] * self.A.shape[2]
        if any(r.opd_basis is not None for r in self.reqs):
            self.C.copy_(self.hC, non_blocking=True)
        for k, r in enumerate(self.reqs):
            if isinstance(r.amp, Resident):
                self.A[k].copy_(r.amp.tensor, non_blocking=True)
            else:
                self.A[k].copy_(self.hA[k], non_blocking=True)
            if r.opd_basis is not None:
                _lib.call('lgb_basis_expand', r.opd_basis.tensor.data_ptr(), self.C[k].data_ptr(),
                          int(r.opd.size), P, self.O[k].data_ptr(), stream.cuda_stream)
            else:
                self.O[k].copy_(self.hO[k], non_blocking=True)
        self.Wt.copy_(self.hW, non_blocking=True)
        if slot.grid:
            self.lam.copy_(self.hlam, non_blocking=True)

    @property
    def nbytes(self):
        return 8 * (2 * self.A.numel() + self.Wt.numel() + self.C.numel() + self.out.numel()) + \
            self.ws.numel()

    def launch(self, slot):
        lam = self.lam if slot.grid else None
        slot.plan.execute(self.A, self.O, self.Wt, out=self.out, check=False, lam_idx=lam,
                          workspace=self.ws)


class _Slot:
    """A cached plan: the resident DFT matrices of one optics geometry (and
    wavelength grid); launches bring their own operand buffers."""

    STATIC_LIMIT = 256 << 20      # launch shapes up to this size keep buffers + a graph

    def __init__(self, key, geo, precision, grid):
        self.key, self.geo, self.grid = key, geo, grid
        self.precision = precision
        self.plan = make_plan(geo, batch=0, precision=precision)
        self.bytes = self.plan.nbytes
        self.static = {}              # (n, n_sel) -> _Buffers reused across launches
        self.seen = collections.Counter()
        self.inflight = 0

    def buffers(self, n, n_sel, device, use_graphs):
        key = (n, n_sel)
        self.seen[key] += 1
        b = self.static.get(key)
        if b is not None and not b.busy:
            return b, True
        b = _Buffers(self, n, n_sel, device)
        if use_graphs and key not in self.static and self.seen[key] >= 2 and \
                b.nbytes <= self.STATIC_LIMIT:
            self.static[key] = b
            return b, True
        return b, False

    def tile_decided(self, b):
        """Whether the autotuner has settled the tile width of this launch's
        class (a graph captured before that would keep the model's width)."""
        if self.precision == 'fp64':
            return True
        m, n = self.geo.fslice[2], self.geo.fslice[3]
        M, N = self.geo.window_shape
        return tuner.lookup(m, n, M, N, b.n * b.n_sel, self.precision, 'intensity') != 0

    def run(self, b, stream, reuse, tile):
        """Launch buffers ``b`` (host inputs already staged) on ``stream``
        with pair-tile width ``tile`` (0: the autotuner's)."""
        self.plan.set_tile(tile)
        with torch.cuda.stream(stream):
            b.load(self, stream)
            g = b.graphs.get(tile)
            if reuse and g is None and (tile != 0 or self.tile_decided(b)):
                b.launch(self)                       # warm-up outside capture
                # capture_begin/end rather than the torch.cuda.graph context,
                # whose entry synchronises the device, collects garbage and
                # empties the caching allocator: the scheduling thread would
                # wait for every launch in flight
                g = torch.cuda.CUDAGraph()
                g.capture_begin(capture_error_mode='thread_local')
                try:
                    b.launch(self)
                finally:
                    g.capture_end()
                b.graphs[tile] = g
            if g is not None:
                g.replay()
            else:
                b.launch(self)
            b.hout.copy_(b.out, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        return ev


class PSFServer:
    """Continuous-batching broadband PSF server on one GPU.

    ``grid``: the spectral grid (metres) whose wavelengths share resident DFT
    matrices; default 128 points over 400-1000 nm."""

    SHARED_TILE = 256     # tile width of launches issued while others are in flight
    EVENTS = 4096         # plan build / eviction records kept

    def __init__(self, hbm_budget=None, streams=4, max_batch=8, precision='split',
                 use_graphs=True, grid=None, device=None, tuner_cache=None):
        self.device = device or dv.device()
        self.tuner_cache = tuner_cache       # tile widths loaded now, saved on close
        if tuner_cache:
            tuner.load(tuner_cache)
        free, total = torch.cuda.mem_get_info(self.device)
        # budget for resident plans; launch buffers come on top, from the
        # caching allocator, at most one launch per stream
        self.budget = int(hbm_budget) if hbm_budget else int(0.55 * free)
        self.precision = precision
        self.max_batch = max_batch
        self.use_graphs = use_graphs
        self.grid = np.asarray(np.linspace(400e-9, 1000e-9, 128) if grid is None else grid, float)
        if precision == 'fp64':
            self.grid = np.zeros(0)                   # wavelength subsets need split plans
        self.n_streams = streams
        self._alloc_failures = 0
        self._queue = collections.deque()
        self._cv = threading.Condition()
        self._slots = collections.OrderedDict()     # key -> _Slot, LRU order
        self._bytes = 0
        self._inflight = []                          # (event, slot, requests, stream index)
        self._free_streams = list(range(streams))
        self._streams = []
        self._stop = False
        self.stats = collections.Counter()
        # the last EVENTS (perf_counter time, kind, value): 'build' (plan
        # build seconds on the scheduler thread), 'evict' (plan bytes released)
        self.events = collections.deque(maxlen=self.EVENTS)
        self._thread = threading.Thread(target=self._loop, name='psf-server', daemon=True)
        self._thread.start()

    # ------------------------------------------------------------ public
    def resident_pupil(self, amp):
        """Keep a pupil amplitude (mask applied) on the device; requests
        that name it copy it on the device instead of sending it."""
        a = np.ascontiguousarray(amp, dtype=np.float64)
        return Resident(a, torch.float64, self.device, util.boundary_slice(a))

    def resident_basis(self, modes):
        """Keep an OPD basis ([K, H, W], K <= 1024) on the device as FP32;
        requests give their OPD as K coefficients of it."""
        m = np.asarray(modes)
        if m.ndim != 3 or not 1 <= m.shape[0] <= _Buffers.KMAX:
            raise ValueError('an OPD basis is [K, H, W] with 1 <= K <= 1024')
        return Resident(m, torch.float32, self.device)

    def submit(self, req):
        if req.future.done():                      # a request object may be submitted again
            req.future = concurrent.futures.Future()
            req.t_done = None
        self._classify(req)
        req.t_submit = time.perf_counter()
        with self._cv:
            if self._stop:
                raise RuntimeError('server closed')
            self._queue.append(req)
            self._cv.notify()
        return req.future

    def inject_allocation_failures(self, n):
        """Test hook: the next ``n`` launch allocations fail on the host (as
        ``torch.cuda.OutOfMemoryError``); their requests fail with it and the
        server keeps serving."""
        self._alloc_failures = int(n)

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
        if self.tuner_cache:
            tuner.save(self.tuner_cache)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---------------------------------------------------------- requests
    def _classify(self, req):
        """Plan key, wavelength subset on the grid (or None) and batch key."""
        idx = None
        if len(self.grid):
            pos = np.clip(np.searchsorted(self.grid, req.wavelengths), 0, len(self.grid) - 1)
            lo = np.clip(pos - 1, 0, len(self.grid) - 1)
            pick = np.where(np.abs(self.grid[lo] - req.wavelengths) <
                            np.abs(self.grid[pos] - req.wavelengths), lo, pos)
            on = np.abs(self.grid[pick] - req.wavelengths) <= 1e-9 * req.wavelengths
            if np.all(on) and len(np.unique(pick)) == len(pick):
                idx = pick.astype(np.int32)
        req._subset = idx
        if idx is not None:
            req._plan_key = ('grid', req.geometry_key(), self.precision)
            req._batch_key = (req._plan_key, idx.tobytes())
        else:
            req._plan_key = ('own', req.geometry_key(), req.wavelengths.tobytes(), self.precision)
            req._batch_key = (req._plan_key, b'')

    # ---------------------------------------------------------- scheduler
    def _loop(self):
        torch.cuda.set_device(self.device)
        self._streams = [torch.cuda.Stream(device=self.device) for _ in range(self.n_streams)]
        while True:
            try:
                progressed = self._poll()
                progressed |= self._admit()
            except Exception as e:                   # never leave futures hanging
                self.stats['loop_errors'] += 1
                with self._cv:
                    stuck = list(self._queue)
                    self._queue.clear()
                for r in stuck:
                    if not r.future.done():
                        r.future.set_exception(e)
                progressed = True
            with self._cv:
                if self._stop and not self._queue and not self._inflight:
                    return
                if not progressed:
                    self._cv.wait(timeout=0.0002)

    def _poll(self):
        done = [x for x in self._inflight if x[0].query()]
        for item in done:
            ev, slot, b, reqs, si = item
            self._inflight.remove(item)
            now = time.perf_counter()
            try:
                _lib.call('lgb_dft2_status', b.ws.data_ptr(), self._streams[si].cuda_stream)
                err = None
            except Exception as e:                     # device timeout or CUDA error
                err = e
            hout, b.hout = b.hout, None
            b.busy = False
            slot.inflight -= 1
            self._free_streams.append(si)
            self.stats['completed'] += len(reqs)      # before any future completes
            for k, r in enumerate(reqs):
                r.t_done = now
                if r.future.done():
                    continue
                if err is None:
                    r.future.set_result(hout[k].numpy())
                else:
                    r.future.set_exception(err)
        return bool(done)

    def _make_room(self, need):
        for key in list(self._slots):
            if self._bytes + need <= self.budget:
                break
            slot = self._slots[key]
            if slot.inflight == 0:
                del self._slots[key]
                self._bytes -= slot.bytes
                self.events.append((time.perf_counter(), 'evict', slot.bytes))
                del slot
                self.stats['evicted'] += 1
        return self._bytes + need <= self.budget

    def _slot_for(self, req):
        key = req._plan_key
        slot = self._slots.get(key)
        if slot is not None:
            self._slots.move_to_end(key)
            self.stats['plan_hits'] += 1
            return slot
        grid = req._subset is not None
        wl = self.grid if grid else req.wavelengths
        s = req.field_slice()
        geo = plan_geometry(req.plane_shape, s, [], np.broadcast_to(req.pixelscale_in, (2,)),
                            req.focal_length, PUPIL, wl, req.det_pixelscale,
                            shape=req.det_shape, oversample=req.oversample)
        if geo.window_shape is None or (grid and len(geo.keep) != len(wl)):
            return 'empty'
        L = len(geo.wavelengths)
        est = plan_bytes_estimate(geo.plane_shape, geo.fslice, geo.window_shape, L, 0,
                                  self.precision)
        if est > self.budget:
            return 'too_big'
        if not self._make_room(int(est * 1.05)):
            return None                               # wait for running work to finish
        t0 = time.perf_counter()
        slot = _Slot(key, geo, self.precision, grid)
        self.events.append((t0, 'build', time.perf_counter() - t0))
        self._slots[key] = slot
        self._bytes += slot.bytes
        self.stats['plans_built'] += 1
        return slot

    def _admit(self):
        progressed = False
        while self._free_streams:
            with self._cv:
                pending = list(self._queue)
            if not pending:
                break
            chosen = None
            for req in pending:                       # oldest request first
                try:
                    slot = self._slot_for(req)
                except (MemoryError, RuntimeError) as e:   # plan allocation or build failed
                    with self._cv:
                        if req in self._queue:
                            self._queue.remove(req)
                    req.t_done = time.perf_counter()
                    self.stats['failed'] += 1
                    req.future.set_exception(e)
                    progressed = True
                    continue
                if isinstance(slot, str):             # 'too_big' or 'empty'
                    with self._cv:
                        self._queue.remove(req)
                    if slot == 'too_big':
                        self.stats['rejected'] += 1
                        req.future.set_exception(MemoryError(
                            'request needs more device memory than the server budget'))
                    else:
                        req.t_done = time.perf_counter()
                        req.future.set_result(np.zeros((req.det_shape * req.oversample,) * 2))
                    progressed = True
                    continue
                if slot is None:
                    continue
                chosen = (slot, req._batch_key)
                break
            if chosen is None:
                break
            slot, bkey = chosen
            with self._cv:
                batch = [r for r in self._queue if r._batch_key == bkey][:self.max_batch]
                for r in batch:
                    self._queue.remove(r)
            n_sel = len(batch[0].wavelengths) if slot.grid else len(slot.geo.wavelengths)
            si = self._free_streams.pop(0)
            slot.inflight += 1
            b = None
            try:
                if self._alloc_failures > 0:         # test hook: the allocation fails
                    self._alloc_failures -= 1
                    raise torch.cuda.OutOfMemoryError('injected allocation failure')
                b, reuse = slot.buffers(len(batch), n_sel, self.device, self.use_graphs)
                b.stage(slot, batch)
                b.busy = True
                t_launch = time.perf_counter()
                for r in batch:
                    r.t_launch = t_launch
                tile = self.SHARED_TILE if self._inflight else 0
                ev = slot.run(b, self._streams[si], reuse, tile)
            except (MemoryError, RuntimeError) as e:     # torch OOM is a RuntimeError
                if b is not None:
                    b.busy = False
                slot.inflight -= 1
                self._free_streams.append(si)
                now = time.perf_counter()
                self.stats['failed'] += len(batch)
                for r in batch:
                    r.t_done = now
                    r.future.set_exception(e)
                progressed = True
                continue
            self._inflight.append((ev, slot, b, batch, si))
            self.stats['launches'] += 1
            self.stats['batched'] += len(batch)
            self.stats['tuned_tile_launches' if tile == 0 else 'shared_gpu_launches'] += 1
            if tile in b.graphs:
                self.stats['graph_launches'] += 1
            progressed = True
        return progressed
