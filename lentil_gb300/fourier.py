"""Matrix triple product DFT on the GPU, drop-in for ``lentil.fourier``.

``dft2``/``idft2`` keep lentil's signatures, argument meaning and errors
(lentil/fourier.py:5-198) and add ``precision``: ``'fp64'`` (complex128,
parity with lentil) or ``'split-bf16'``/``'split-fp16'`` (tensor cores,
16-bit hi/lo operand split with FP32 accumulation).  ``npix`` is accepted as
an alias of ``shape``.  numpy in -> numpy out; CUDA tensor in -> tensor out.
The DFT matrices of recently used geometries stay on the device (a plan
cache, ``plan_cache_info``/``clear_plan_cache``); split-precision device
failures of a transform returned as a tensor are raised by the next
transform of that geometry or by ``plan_status()``.
"""
import collections
import ctypes
import threading

import numpy as np
import torch

from . import _device as dv
from . import _lib

# Device-resident DFT matrices of recently used geometries (lgb_dft2_plan_*):
# a repeated transform of one geometry builds no matrices and copies nothing
# from the host.  Least recently used plans are destroyed beyond either bound.
PLAN_CACHE_ENTRIES = 32
PLAN_CACHE_BYTES = 1 << 30


class _Dft2Plan:
    """One dft2 geometry with its DFT matrices on the device, in a block of
    the caching allocator (dropping the plan frees it stream-safely)."""

    def __init__(self, key):
        m, n, M, N, ar, ac, sr, sc, orow, ocol, unitary, prec, _dev = key
        lib = self._lib = _lib.load()
        self.nbytes = int(lib.lgb_dft2_plan_size(m, n, M, N, prec))
        self._mem = dv.workspace(self.nbytes)
        self._home = torch.cuda.current_stream()
        self._foreign = set()
        h = ctypes.c_void_p()
        _lib.call('lgb_dft2_plan_create_in', m, n, M, N, ar, ac, sr, sc, orow, ocol, unitary, prec,
                  self._mem.data_ptr(), self.nbytes, dv.stream_ptr(), ctypes.byref(h))
        self._h = h
        self._built = torch.cuda.Event()      # the matrix build, on the creating stream
        self._built.record(self._home)
        self.shape_out = (M, N)
        self.split = prec != _lib.FP64
        self.pins = 0                 # > 0 while a captured CUDA graph holds its pointers

    def execute(self, fd):
        """fd: [count, m, n] contiguous complex128 CUDA tensor -> [count, M, N].
        A device-side failure of an earlier execute is raised here."""
        count = int(fd.shape[0])
        s = torch.cuda.current_stream()
        if s != self._home and not torch.cuda.is_current_stream_capturing():
            s.wait_event(self._built)         # the matrices are built before s reads them
            if s.cuda_stream not in self._foreign:
                self._mem.record_stream(s)    # keep the matrices until s is done with them
                self._foreign.add(s.cuda_stream)
        F = torch.empty((count,) + self.shape_out, dtype=torch.complex128, device=fd.device)
        nbytes = self._lib.lgb_dft2_plan_workspace_size(self._h, count)
        ws = dv.workspace(nbytes)
        _lib.call('lgb_dft2_plan_execute', self._h, fd.data_ptr(), count, F.data_ptr(),
                  ws.data_ptr(), nbytes, dv.stream_ptr())
        return F

    def status(self):
        """Wait for the stream and raise a device-side failure of this plan."""
        _lib.call('lgb_dft2_plan_status', self._h, dv.stream_ptr())

    def destroy(self):
        if self._h is not None and self._h.value:
            self._lib.lgb_dft2_plan_destroy(self._h)
        self._h = None
        self._mem = None


_plans = collections.OrderedDict()
_seen = set()                 # geometries transformed once without a plan
_plans_lock = threading.Lock()


def _plan(m, n, M, N, ar, ac, sr, sc, orow, ocol, unitary, prec):
    """The cached plan of a geometry, created on its second use (None on the
    first: a one-off transform builds its matrices in its own workspace)."""
    key = (m, n, M, N, ar, ac, sr, sc, orow, ocol, int(bool(unitary)), prec,
           torch.cuda.current_device())
    with _plans_lock:
        p = _plans.get(key)
        if p is not None:
            _plans.move_to_end(key)
            return p
        if key not in _seen or torch.cuda.is_current_stream_capturing():
            if len(_seen) > 65536:
                _seen.clear()
            _seen.add(key)
            return None
        _seen.discard(key)
        p = _plans[key] = _Dft2Plan(key)
        if not torch.cuda.is_current_stream_capturing():
            total = sum(q.nbytes for q in _plans.values())
            for k in list(_plans):
                if len(_plans) <= 1 or (len(_plans) <= PLAN_CACHE_ENTRIES and
                                        total <= PLAN_CACHE_BYTES):
                    break
                old = _plans[k]
                if old.pins or old is p:
                    continue
                del _plans[k]
                total -= old.nbytes
                old.destroy()
        return p


class pinned_plans:
    """Context manager: every plan used inside the block stays cached (and
    its device memory alive) until ``release()`` -- for CUDA graphs that
    capture transforms, whose replays reuse the plans' pointers."""

    def __init__(self):
        self._held = []

    def __enter__(self):
        _pin_sinks.append(self._held)
        return self

    def __exit__(self, *exc):
        _pin_sinks.remove(self._held)
        return False

    def release(self):
        with _plans_lock:
            for p in self._held:
                p.pins -= 1
            self._held.clear()


_pin_sinks = []


def _note_use(p):
    for sink in _pin_sinks:
        if p not in sink:
            p.pins += 1
            sink.append(p)


def plan_cache_info():
    """(entries, device bytes) of the dft2 plan cache."""
    with _plans_lock:
        return len(_plans), sum(p.nbytes for p in _plans.values())


def clear_plan_cache():
    """Destroy every cached dft2 plan that no captured CUDA graph holds (see
    ``pinned_plans``) and forget the geometries seen once."""
    with _plans_lock:
        for k in list(_plans):
            if not _plans[k].pins:
                _plans.pop(k).destroy()
        _seen.clear()


def plan_status():
    """Wait for the current stream and raise any device-side failure of a
    cached split-precision plan (executes report it one call later)."""
    with _plans_lock:
        plans = list(_plans.values())
    for p in plans:
        if p.split:
            p.status()


class _OneOff:
    """Result holder of a transform that ran without a plan (status checked)."""
    split = False

    def status(self):
        pass


def _transform(fd, M, N, alpha, shift, offset, unitary, precision):
    """[count, m, n] CUDA complex128 -> ([count, M, N], plan) through the
    plan cache; a geometry's first transform builds its matrices in a
    workspace of its own (and reports its split-path status at once)."""
    count, m, n = (int(x) for x in fd.shape)
    ar, ac = _pair(alpha, 'alpha')
    sr, sc = _pair(shift, 'shift')
    orow, ocol = _pair(offset, 'offset')
    prec = _lib.precision_code(precision)
    if m < 1 or n < 1 or M < 1 or N < 1:
        raise ValueError('dft2: sizes must be positive')
    fd = fd.contiguous()
    p = _plan(m, n, M, N, ar, ac, sr, sc, orow, ocol, unitary, prec)
    if p is None and torch.cuda.is_current_stream_capturing():
        # a plan's memory and matrix build must not land inside a graph
        raise RuntimeError('dft2: a geometry first met under stream capture has no plan; '
                           'run it twice outside the capture first')
    if p is not None:
        with _plans_lock:
            _note_use(p)
        return p.execute(fd), p
    F = torch.empty((count, M, N), dtype=torch.complex128, device=fd.device)
    nbytes = _lib.load().lgb_dft2_batch_workspace_size(count, m, n, M, N, prec)
    ws = dv.workspace(nbytes)
    _lib.call('lgb_dft2_batch', fd.data_ptr(), count, m, n, F.data_ptr(), M, N, ar, ac, sr, sc,
              orow, ocol, int(bool(unitary)), prec, ws.data_ptr(), nbytes, dv.stream_ptr())
    if prec != _lib.FP64:
        _lib.call('lgb_dft2_status', ws.data_ptr(), dv.stream_ptr())
    return F, _OneOff()


def _pair(x, name):
    v = np.broadcast_to(np.asarray(x, dtype=float), (2,))
    return float(v[0]), float(v[1])


def _shape(shape, npix, f_shape):
    if npix is not None:
        if shape is not None:
            raise TypeError("dft2 got both 'shape' and its alias 'npix'")
        shape = npix
    if shape is None:
        return int(f_shape[0]), int(f_shape[1])
    M, N = np.broadcast_to(np.asarray(shape), (2,))
    return int(M), int(N)


def _check_out(out):
    if out is None:
        return
    dt = out.dtype
    if dv.is_tensor(out):
        ok = dt in (torch.complex128, torch.complex64)
        name = str(dt)
    else:
        ok = np.can_cast(complex, dt)
        name = str(dt)
    if not ok:
        raise TypeError(f"Cannot cast complex output to dtype('{name}')")


def _finish(F_dev, out, host):
    """Deliver a device result as lentil does: into ``out`` when given."""
    if out is not None:
        if dv.is_tensor(out):
            if tuple(out.shape) != tuple(F_dev.shape):
                raise ValueError(f'out has shape {tuple(out.shape)}, expected {tuple(F_dev.shape)}')
            out.copy_(F_dev)
        else:
            if out.shape != tuple(F_dev.shape):
                raise ValueError(f'out has shape {out.shape}, expected {tuple(F_dev.shape)}')
            out[...] = dv.to_host(F_dev)
        return out
    return dv.to_host(F_dev) if host else F_dev


def dft2_matrices(m, n, M, N, alpha, shift=(0, 0), offset=(0, 0)):
    """E1 (M x m) and E2 (n x N) as CUDA complex128 tensors
    (lentil/fourier.py:106-110)."""
    ar, ac = _pair(alpha, 'alpha')
    sr, sc = _pair(shift, 'shift')
    orow, ocol = _pair(offset, 'offset')
    dev = dv.device()
    E1 = torch.empty((M, m), dtype=torch.complex128, device=dev)
    E2 = torch.empty((n, N), dtype=torch.complex128, device=dev)
    _lib.call('lgb_dft2_matrices', m, n, M, N, ar, ac, sr, sc, orow, ocol, E1.data_ptr(),
              E2.data_ptr(), dv.stream_ptr())
    return E1, E2


def dft2(f, alpha, shape=None, shift=(0, 0), offset=(0, 0), unitary=True, out=None, npix=None,
         precision='fp64'):
    """2-D DFT by matrix triple product ``E1 . f . E2`` (lentil/fourier.py:5-103).

    Parameters follow lentil: ``alpha`` output sampling (scalar or (row, col)),
    ``shape`` (alias ``npix``) output shape, ``shift`` DC shift in output
    pixels, ``offset`` input-plane offset, ``unitary`` energy normalisation,
    ``out`` complex array written in place and returned.
    """
    host = not dv.is_tensor(f)
    _check_out(out)
    fd = dv.to_device(f, torch.complex128)
    if fd.dim() != 2:
        raise ValueError('dft2 expects a 2-D array')
    M, N = _shape(shape, npix, fd.shape)
    F, plan = _transform(fd.unsqueeze(0), M, N, alpha, shift, offset, unitary, precision)
    res = _finish(F[0], out, host)
    if plan.split and (host or (out is not None and not dv.is_tensor(out))):
        plan.status()                     # the result is on the host: report at once
    return res


def dft2_batch(f, alpha, shape=None, shift=(0, 0), offset=(0, 0), unitary=True, npix=None,
               precision='fp64'):
    """``dft2`` of every field of a stack ``f`` [count, m, n] with one
    geometry (an extension of lentil's dft2, which takes one array): the DFT
    matrices come from the plan cache and the split path transforms the whole
    stack in one pair of tensor-core launches.  Returns [count, M, N], on the
    device for CUDA input, else as numpy."""
    host = not dv.is_tensor(f)
    fd = dv.to_device(f, torch.complex128)
    if fd.dim() != 3:
        raise ValueError('dft2_batch expects a 3-D stack [count, m, n]')
    M, N = _shape(shape, npix, fd.shape[1:])
    F, plan = _transform(fd, M, N, alpha, shift, offset, unitary, precision)
    if host:
        res = dv.to_host(F)
        if plan.split:
            plan.status()                 # the result is on the host: report at once
        return res
    return F


def idft2(F, alpha, shape=None, shift=(0, 0), unitary=True, out=None, npix=None,
          precision='fp64'):
    """Inverse DFT ``conj(dft2(conj(F))) / F.size`` (lentil/fourier.py:124-198)."""
    host = not dv.is_tensor(F)
    _check_out(out)
    Fd = dv.to_device(F, torch.complex128)
    if Fd.dim() != 2:
        raise ValueError('idft2 expects a 2-D array')
    m, n = (int(x) for x in Fd.shape)
    M, N = _shape(shape, npix, (m, n))
    # conj(dft2(conj(F), offset 0)) * (1 / F.size), the dft2 from the plan cache
    G, plan = _transform(Fd.conj().resolve_conj().unsqueeze(0), M, N, alpha, shift, (0, 0),
                         unitary, precision)
    f = G[0].conj() * (1.0 / (m * n))
    res = _finish(f, out, host)
    if plan.split and (host or (out is not None and not dv.is_tensor(out))):
        plan.status()
    return res
