"""Fused broadband PSFs: lentil's documented user loop

    for lam, w in zip(wavelengths, weights):
        img = propagate_dft(Wavefront(lam) * pupil, pixelscale, ...).insert(img, w)

(docs/user/performance.rst:44-49) as one plan execution on the GPU for a
batch of PSFs that share optics.  The plan keeps the DFT matrices of every
wavelength resident, builds the phasor of every (PSF, wavelength) straight
into the tensor-core operand layout, and accumulates w * |E|^2 in the MFT
epilogue.

Fields that share one window and one shift per wavelength are summed before
the transform (the MFT is linear and lentil's ``Wavefront.intensity`` sums
overlapping fields coherently), so a segmented pupil without per-segment
tilts is one dense field.  Pupils whose segments carry their own tilts are
propagated field by field through ``propagate_dft`` (same kernels, one
launch sequence per field) and overlap-added on the device.
"""
import concurrent.futures
import ctypes
import os
import threading

import numpy as np
import torch

from . import _device as dv
from . import _lib
from . import util
from .propagate import plan_fields


class _ProbeField:
    """Geometry-only stand-in for a Field (offset, shape, tilts)."""

    def __init__(self, offset, shape, tilt):
        self.offset, self.shape, self.tilt = offset, shape, tilt

    shift = None  # bound below


def _probe_shift(self, z, wavelength, pixelscale, oversample, indexing='ij'):
    from .field import Field
    return Field.shift(self, z, wavelength, pixelscale, oversample, indexing)


_ProbeField.shift = _probe_shift


class _ProbeWavefront:
    def __init__(self, wavelength, pixelscale, focal_length, shape, data, ptype):
        self.wavelength, self.pixelscale, self.focal_length = wavelength, pixelscale, focal_length
        self.shape, self.data, self.ptype = shape, data, ptype


class CapturedExecute:
    """A PSFPlan execute captured as a CUDA graph (see ``PSFPlan.capture``)."""

    def __init__(self, plan, amp, opd, weights, out, lam_idx=None):
        self.plan, self.amp, self.opd, self.weights, self.out = plan, amp, opd, weights, out
        self.lam_idx = lam_idx
        count = int(amp.shape[0])
        n_sel = None if lam_idx is None else int(lam_idx.numel())
        self.ws = torch.empty(max(1, plan.workspace_bytes(count, n_sel)), dtype=torch.uint8,
                              device=amp.device)
        run = lambda: plan.execute(amp, opd, weights, out=out, check=False, lam_idx=lam_idx,
                                   workspace=self.ws)
        s = torch.cuda.Stream(device=amp.device)
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            run()                         # warm-up outside the capture (tuner, attributes)
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph, stream=s):
                run()
        torch.cuda.current_stream().wait_stream(s)

    def replay(self):
        """Rerun the captured execute on the current stream; returns ``out``."""
        self.graph.replay()
        return self.out

    def status(self):
        _lib.call('lgb_dft2_status', self.ws.data_ptr(), dv.stream_ptr())


class PSFPlan:
    """Device plan for a batch of broadband PSFs with fixed optics.

    Parameters mirror the user loop: pupil-plane shape and field slice, the
    wavelengths, per-wavelength MFT sampling ``alpha`` and output shift, the
    MFT window inside the output image, the batch size and the precision."""

    def __init__(self, plane_shape, field_slice, field_offset, wavelengths, alphas, shifts,
                 window_shape, image_shape, window_origin, batch=1, precision='split'):
        lib = _lib.load()
        dv.device()
        self.plane_shape = tuple(int(x) for x in plane_shape)
        self.field_slice = tuple(int(x) for x in field_slice)
        self.image_shape = tuple(int(x) for x in image_shape)
        self.wavelengths = np.ascontiguousarray(wavelengths, dtype=np.float64)
        self.L = len(self.wavelengths)
        self.batch = int(batch)
        self.precision = precision
        ar = np.ascontiguousarray([a[0] for a in alphas], dtype=np.float64)
        ac = np.ascontiguousarray([a[1] for a in alphas], dtype=np.float64)
        sr = np.ascontiguousarray([s[0] for s in shifts], dtype=np.float64)
        sc = np.ascontiguousarray([s[1] for s in shifts], dtype=np.float64)
        r0, c0, m, n = self.field_slice
        d = _lib.PsfDesc()
        d.H, d.W = self.plane_shape
        d.r0, d.c0, d.m, d.n = r0, c0, m, n
        d.offset_r, d.offset_c = float(field_offset[0]), float(field_offset[1])
        d.M, d.N = int(window_shape[0]), int(window_shape[1])
        d.out_rows, d.out_cols = self.image_shape
        d.win_r0, d.win_c0 = int(window_origin[0]), int(window_origin[1])
        d.n_wavelengths = self.L
        keep = (self.wavelengths, ar, ac, sr, sc)
        d.wavelengths, d.alpha_r, d.alpha_c, d.shift_r, d.shift_c = [a.ctypes.data for a in keep]
        d.batch = self.batch
        d.precision = _lib.precision_code(precision)
        self.desc = d
        # plan memory is a block of torch's caching allocator: a plan built
        # where an earlier one was released reuses its memory without
        # mapping new device memory; executes on other streams are recorded
        # on the block so that it outlives their work
        nbytes = lib.lgb_psf_plan_size(ctypes.byref(d))
        if nbytes == 0:                  # an invalid description: the size call recorded why
            _lib.check(_lib.EINVAL)
        self._home = torch.cuda.current_stream()
        self._foreign = set()
        self._mem = dv.workspace(nbytes)
        h = ctypes.c_void_p()
        _lib.check(lib.lgb_psf_plan_create_in(ctypes.byref(d), self._mem.data_ptr(), nbytes,
                                              ctypes.byref(h), self._home.cuda_stream))
        self._h = h
        self.nbytes = lib.lgb_psf_plan_bytes(h)
        # executes without a caller workspace share the plan's own operand
        # buffers and status word: they are issued one at a time (lock) and
        # each waits on the device for the previous one (event), whatever
        # stream or thread it comes from
        self._own_lock = threading.Lock()
        self._own_done = None
        # the DFT matrices are built on the creating stream; executes on any
        # other stream wait for them on the device
        self._built = torch.cuda.Event()
        self._built.record(self._home)
        self._lanes = None               # execute_streams: [(stream, workspace)] x LANES

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and h.value:
            try:
                _lib.load().lgb_psf_plan_destroy(h)
            except Exception:
                pass
            self._h = None

    def set_tile(self, tile):
        """Pair-tile width of this plan's tensor-core launches: 0 = the
        autotuner's choice (``lentil_gb300.tuner``), 256 or 128 = that width."""
        _lib.call('lgb_psf_plan_set_tile', self._h, int(tile))

    def capture(self, amp, opd, weights, out, lam_idx=None):
        """The execute of these device tensors, captured once as a CUDA graph.

        Returns a ``CapturedExecute`` whose ``replay()`` reruns it with
        whatever the tensors hold at that moment (write new inputs into them in
        place) and no host work per kernel; ``status()`` waits and raises a
        device-side failure.  The plan must outlive the capture."""
        return CapturedExecute(self, amp, opd, weights, out, lam_idx)

    LANES = 2

    def execute_streams(self, amp, opd, weights, out, check=True):
        """``execute`` of n PSFs one at a time, alternating them over two CUDA
        streams with a workspace each, both forked from and joined back to the
        caller's stream.  A PSF's kernels then start on the SMs that the
        previous PSF's last wave of MFT CTA pairs leaves idle (+1-2 % PSFs/s
        on the 1024^2 64-wavelength workload).  amp [1 or n, H, W], opd
        [n, H, W], weights [1 or n, L], out [n, rows, cols]; ``check=False``
        leaves the status to ``stream_status()``.  Inside a CUDA-graph capture,
        and for complex128 plans (whose executes use the plan's own buffers),
        the PSFs run in order on the caller's stream."""
        count = int(opd.shape[0])
        if tuple(out.shape[:1]) != (count,):
            raise ValueError(f'out must hold {count} images')
        pick = lambda t, k: t if t.shape[0] == 1 else t[k:k + 1]
        cur = torch.cuda.current_stream()
        capturing = torch.cuda.is_current_stream_capturing()
        if count == 1 or capturing or _lib.precision_code(self.precision) == _lib.FP64:
            for k in range(count):        # (no status wait inside a capture)
                self.execute(pick(amp, k), opd[k:k + 1], pick(weights, k), out=out[k:k + 1],
                             check=check and not capturing)
            return out
        if self._lanes is None:
            nbytes = max(1, self.workspace_bytes(1))
            self._lanes = [(torch.cuda.Stream(device=cur.device), dv.workspace(nbytes))
                           for _ in range(self.LANES)]
        fork = torch.cuda.Event()
        fork.record(cur)
        for st, ws in self._lanes:
            st.wait_event(fork)          # inputs written and workspaces free (earlier joins)
        for k in range(count):
            st, ws = self._lanes[k % self.LANES]
            with torch.cuda.stream(st):
                self.execute(pick(amp, k), opd[k:k + 1], pick(weights, k), out=out[k:k + 1],
                             check=False, workspace=ws)
        for st, ws in self._lanes:
            join = torch.cuda.Event()
            join.record(st)
            cur.wait_event(join)
        if check:
            self.stream_status()
        return out

    def stream_status(self):
        """Wait for the caller's stream and raise a device-side failure that
        an ``execute_streams`` call recorded in its workspaces."""
        for st, ws in self._lanes or ():
            _lib.call('lgb_dft2_status', ws.data_ptr(), dv.stream_ptr())

    def workspace_bytes(self, count, n_sel=None):
        """Bytes of a caller workspace for ``execute(..., workspace=...)``."""
        return _lib.load().lgb_psf_execute_workspace_size(self._h, count,
                                                          self.L if n_sel is None else n_sel)

    def execute(self, amp, opd, weights, out=None, accumulate=False, check=True, lam_idx=None,
                workspace=None):
        """amp (mask applied), opd: [n, H, W] float64 CUDA tensors (n <= batch);
        weights: [n, L] (or [n, len(lam_idx)]); returns out [n, rows, cols]
        float64.  ``lam_idx`` (int32 CUDA tensor) restricts the PSFs to those
        of the plan's wavelengths."""
        dev = dv.device()
        amp = amp if amp.dtype == torch.float64 and amp.is_contiguous() else amp.double().contiguous()
        opd = opd if opd.dtype == torch.float64 and opd.is_contiguous() else opd.double().contiguous()
        weights = dv.to_device(weights, torch.float64)
        count = int(amp.shape[0])
        shp = (count,) + self.plane_shape
        cap = self.batch if workspace is None else count
        if not 1 <= count <= cap or tuple(amp.shape) != shp or tuple(opd.shape) != shp:
            raise ValueError(f'amp/opd must have shape (n,) + {self.plane_shape}, n <= {cap}')
        n_sel = self.L if lam_idx is None else int(lam_idx.numel())
        if weights.numel() < count * n_sel:
            raise ValueError(f'weights must have {count * n_sel} entries')
        if out is None:
            out = torch.empty((count,) + self.image_shape, dtype=torch.float64, device=dev)
            accumulate = False
        cur = torch.cuda.current_stream()
        if cur != self._home and not torch.cuda.is_current_stream_capturing():
            cur.wait_event(self._built)
            if cur.cuda_stream not in self._foreign:
                self._mem.record_stream(cur)
                self._foreign.add(cur.cuda_stream)
        if workspace is not None:
            if lam_idx is not None and (lam_idx.dtype != torch.int32 or not lam_idx.is_cuda):
                raise TypeError('lam_idx must be an int32 CUDA tensor')
            _lib.call('lgb_psf_execute_ws', self._h, count, dv.ptr(lam_idx), n_sel,
                      amp.data_ptr(), opd.data_ptr(), weights.data_ptr(), out.data_ptr(),
                      int(bool(accumulate)), workspace.data_ptr(), workspace.numel(),
                      dv.stream_ptr())
            if check:
                _lib.call('lgb_dft2_status', workspace.data_ptr(), dv.stream_ptr())
            return out
        if lam_idx is not None and (lam_idx.dtype != torch.int32 or not lam_idx.is_cuda):
            raise TypeError('lam_idx must be an int32 CUDA tensor')
        with self._own_lock:
            cur = torch.cuda.current_stream()
            capturing = torch.cuda.is_current_stream_capturing()
            if self._own_done is not None and not capturing:
                cur.wait_event(self._own_done)
            if lam_idx is None:
                _lib.call('lgb_psf_execute_batch', self._h, count, amp.data_ptr(),
                          opd.data_ptr(), weights.data_ptr(), out.data_ptr(),
                          int(bool(accumulate)), cur.cuda_stream)
            else:
                _lib.call('lgb_psf_execute_subset', self._h, count, lam_idx.data_ptr(), n_sel,
                          amp.data_ptr(), opd.data_ptr(), weights.data_ptr(), out.data_ptr(),
                          int(bool(accumulate)), cur.cuda_stream)
            if not capturing:
                self._own_done = torch.cuda.Event()
                self._own_done.record(cur)
            if check:
                _lib.call('lgb_psf_plan_status', self._h, cur.cuda_stream)
        return out


_HOST_POOL = None
_HOST_POOL_LOCK = threading.Lock()
_HOST_WORKERS = max(1, min(8, os.cpu_count() or 1))
_HOST_PARALLEL_MIN = 1 << 22          # elements below which one thread is faster


def _host_pool():
    global _HOST_POOL
    with _HOST_POOL_LOCK:
        if _HOST_POOL is None:
            _HOST_POOL = concurrent.futures.ThreadPoolExecutor(max_workers=_HOST_WORKERS,
                                                               thread_name_prefix='lgb-host')
        return _HOST_POOL


def _forget_host_pool():
    # a forked child inherits the pool object but not its threads
    global _HOST_POOL, _HOST_POOL_LOCK
    _HOST_POOL, _HOST_POOL_LOCK = None, threading.Lock()


if hasattr(os, 'register_at_fork'):
    os.register_at_fork(after_in_child=_forget_host_pool)


def _by_rows(fn, rows, size):
    """fn(r0, r1) over blocks of rows in the host pool (numpy releases the GIL
    in its loops, so the blocks run in parallel), or in one call when the
    array is small."""
    parts = min(_HOST_WORKERS, rows) if size >= _HOST_PARALLEL_MIN else 1
    if parts <= 1:
        fn(0, rows)
        return
    edges = np.linspace(0, rows, parts + 1).round().astype(int)
    list(_host_pool().map(lambda k: fn(edges[k], edges[k + 1]), range(parts)))


def _summed_mask(mask):
    """mask.sum(axis=0) of an (S, H, W) mask by row blocks: each pixel adds
    its S values in the same order, so the result is the same array."""
    out = np.empty(mask.shape[1:], dtype=np.add.reduce(mask[:, :1, :1], axis=0).dtype)
    _by_rows(lambda r0, r1: np.sum(mask[:, r0:r1], axis=0, out=out[r0:r1]), mask.shape[1],
             mask.size)
    return out


def _product(a, b):
    out = np.empty(np.broadcast_shapes(a.shape, b.shape), dtype=np.result_type(a, b))
    _by_rows(lambda r0, r1: np.multiply(a[r0:r1], b[r0:r1], out=out[r0:r1]), out.shape[0],
             out.size)
    return out


def dense_field(pupil):
    """Merged single field of a pupil without per-segment tilts: the slice
    covering every segment and amp*sum(masks) over it (lentil/plane.py:494-514
    summed over segments).  Returns (slice, amp_eff, opd) on the host."""
    amp = np.asarray(dv.to_host(pupil.amplitude) if dv.is_tensor(pupil.amplitude) else pupil.amplitude,
                     dtype=float)
    opd = np.asarray(dv.to_host(pupil.opd) if dv.is_tensor(pupil.opd) else pupil.opd, dtype=float)
    mask = pupil.mask
    mask = np.asarray(dv.to_host(mask) if dv.is_tensor(mask) else mask, dtype=float)
    if amp.ndim != 2:
        raise NotImplementedError('broadband plan needs an amplitude array')
    gmask = mask if mask.ndim == 2 else _summed_mask(mask)
    # the union of the segments' bounding boxes: segment masks are
    # transmissions (>= 0), so a pixel lies in some segment exactly where
    # their sum is positive -- one scan of the summed mask instead of one
    # per segment
    s = util.boundary_slice(gmask)
    opd_full = np.broadcast_to(opd, amp.shape) if opd.size == 1 else opd
    amp_eff = _product(amp, gmask) if amp.shape == gmask.shape else amp * gmask
    return s, amp_eff, np.ascontiguousarray(opd_full, dtype=float)


def _device_field(pupil):
    """(slice, amp_eff, opd) of ``dense_field`` with amp_eff and opd as CUDA
    tensors.  A frozen plane cannot change its amplitude or OPD (lentil's
    freeze contract), so its merged field is kept on the device with the
    plane and later calls reuse it (keyed on the mask object as well)."""
    frozen = bool(getattr(pupil, 'frozen', False))
    key = id(getattr(pupil, '_mask', None))
    cache = getattr(pupil, '_lgb_device_field', None) if frozen else None
    if cache is not None and cache[0] == key:
        return cache[1]
    s, amp_eff, opd = dense_field(pupil)
    shp = (1,) + amp_eff.shape
    field = (s, dv.to_device(amp_eff, torch.float64).reshape(shp),
             dv.to_device(opd, torch.float64).reshape(shp))
    if frozen:
        try:
            pupil._lgb_device_field = (key, field)
        except AttributeError:           # a plane class with __slots__: no cache
            pass
    return field


def broadband_psf(pupil, wavelengths, weights, pixelscale, shape=None, prop_shape=None,
                  oversample=2, mask=None, precision='split', out=None):
    """Sum over wavelengths of weight * propagate_dft(Wavefront(lam) * pupil).intensity.

    Equivalent to lentil's broadband loop; returns a float64 image (numpy, or
    a CUDA tensor when the pupil holds tensors).  ``out`` (optional) is added
    to, as ``Wavefront.insert`` does."""
    from .wavefront import Wavefront
    from . import propagate as prop
    wavelengths = np.atleast_1d(np.asarray(wavelengths, dtype=float))
    weights = np.atleast_1d(np.asarray(weights, dtype=float))
    tensor_io = pupil._tensor_io() if hasattr(pupil, '_tensor_io') else False
    if len(pupil.tilt) > 1:
        # per-segment tilts: every segment is its own field with its own window
        img = None
        dev_out = None if out is None else dv.to_device(out, torch.float64)
        for lam, w in zip(wavelengths, weights):
            wf = prop.propagate_dft(Wavefront(lam) * pupil, pixelscale, shape=shape,
                                    prop_shape=prop_shape, oversample=oversample, mask=mask,
                                    precision=precision)
            if dev_out is None:
                dev_out = torch.zeros(tuple(int(s) for s in wf.shape), dtype=torch.float64,
                                      device=dv.device())
            dev_out = wf.insert(dev_out, weight=w)
        img = dev_out
        return _deliver(img, out, tensor_io)

    s, a, o = _device_field(pupil)
    plane_shape = tuple(a.shape[1:])
    geo = plan_geometry(plane_shape, s, list(pupil.tilt), pupil.pixelscale, pupil.focal_length,
                        pupil.ptype, wavelengths, pixelscale, shape, prop_shape, oversample, mask)
    dev = dv.device()
    img = torch.zeros(geo.shape_out, dtype=torch.float64, device=dev) if out is None else \
        dv.to_device(out, torch.float64)
    if not geo.keep:
        return _deliver(img, out, tensor_io)
    plan = _cached_plan(geo, precision)
    w = dv.to_device(weights[geo.keep], torch.float64).reshape(1, -1)
    plan.execute(a, o, w, out=img.reshape((1,) + geo.shape_out), accumulate=True)
    return _deliver(img, out, tensor_io)


class Geometry:
    """Where one merged field lands for every wavelength of a broadband PSF."""
    __slots__ = ('plane_shape', 'fslice', 'offset', 'wavelengths', 'alphas', 'shifts',
                 'window_shape', 'window_origin', 'shape_out', 'keep')


def plan_geometry(plane_shape, s, tilts, dx, focal_length, ptype, wavelengths, du, shape=None,
                  prop_shape=None, oversample=2, mask=None):
    """Window maths of propagate_dft (lentil/propagate.py:175-240) for one
    field slice ``s`` of the pupil plane and every wavelength; wavelengths
    whose window misses the output are dropped (``keep`` lists the rest)."""
    off = util.slice_offset(s, plane_shape)
    r0, c0 = int(s[0].start), int(s[1].start)
    m, n = int(s[0].stop) - r0, int(s[1].stop) - c0
    g = Geometry()
    g.plane_shape, g.fslice, g.offset = tuple(plane_shape), (r0, c0, m, n), off
    g.alphas, g.shifts, g.keep = [], [], []
    window, shape_out = None, None
    for i, lam in enumerate(np.atleast_1d(wavelengths)):
        probe = _ProbeWavefront(lam, dx, focal_length, plane_shape,
                                [_ProbeField(off, (m, n), list(tilts))], ptype)
        _, shape_out, _, jobs = plan_fields(probe, du, shape, prop_shape, oversample, mask)
        if not jobs:
            continue
        j = jobs[0]
        win = (tuple(int(x) for x in j.shape), tuple(int(x) for x in j.offset_out))
        if window is not None and win != window:
            raise NotImplementedError('wavelength-dependent output windows are not fused')
        window = win
        g.keep.append(i)
        g.alphas.append(tuple(float(a) for a in j.alpha))
        g.shifts.append(tuple(float(x) for x in j.shift))
    g.shape_out = tuple(int(x) for x in shape_out)
    g.wavelengths = np.atleast_1d(np.asarray(wavelengths, dtype=float))[g.keep]
    if window is not None:
        wshape, woff = window
        # window origin inside the image: the placement rule of lentil/field.py:267
        g.window_shape = wshape
        g.window_origin = (g.shape_out[0] // 2 - wshape[0] // 2 + woff[0],
                           g.shape_out[1] // 2 - wshape[1] // 2 + woff[1])
    else:
        g.window_shape = g.window_origin = None
    return g


def make_plan(geo, batch=1, precision='split'):
    """PSFPlan for a Geometry."""
    return PSFPlan(geo.plane_shape, geo.fslice, geo.offset, geo.wavelengths, geo.alphas, geo.shifts,
                   geo.window_shape, geo.shape_out, geo.window_origin, batch=batch,
                   precision=precision)


def _deliver(img, out, tensor_io):
    if out is not None and not dv.is_tensor(out):
        out[...] = dv.to_host(img)
        return out
    if out is not None:
        if img.data_ptr() != out.data_ptr():
            out.copy_(img)
        return out
    return img if tensor_io else dv.to_host(img)


_PLANS = {}
_PLANS_LOCK = threading.Lock()


def _cached_plan(geo, precision, batch=1):
    """The PSF plan of a geometry, from an 8-entry FIFO shared by the
    process's threads (a plan evicted while another thread still uses it
    lives until that thread drops it)."""
    key = (geo.plane_shape, geo.fslice, tuple(geo.offset), tuple(geo.wavelengths.tolist()),
           tuple(geo.alphas), tuple(geo.shifts), geo.window_shape, geo.shape_out,
           geo.window_origin, precision, batch)
    with _PLANS_LOCK:
        p = _PLANS.get(key)
        if p is None:
            if len(_PLANS) >= 8:
                _PLANS.pop(next(iter(_PLANS)))
            p = make_plan(geo, batch=batch, precision=precision)
            _PLANS[key] = p
    return p
