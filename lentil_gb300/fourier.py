"""Matrix triple product DFT on the GPU, drop-in for ``lentil.fourier``.

``dft2``/``idft2`` keep lentil's signatures, argument meaning and errors
(lentil/fourier.py:5-198) and add ``precision``: ``'fp64'`` (complex128,
parity with lentil) or ``'split-bf16'``/``'split-fp16'`` (tensor cores,
16-bit hi/lo operand split with FP32 accumulation).  ``npix`` is accepted as
an alias of ``shape``.  numpy in -> numpy out; CUDA tensor in -> tensor out.
"""
import numpy as np
import torch

from . import _device as dv
from . import _lib


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
    m, n = fd.shape
    M, N = _shape(shape, npix, (m, n))
    ar, ac = _pair(alpha, 'alpha')
    sr, sc = _pair(shift, 'shift')
    orow, ocol = _pair(offset, 'offset')
    prec = _lib.precision_code(precision)
    F = torch.empty((M, N), dtype=torch.complex128, device=fd.device)
    nbytes = _lib.load().lgb_dft2_workspace_size(m, n, M, N, prec)
    ws = dv.workspace(nbytes)
    _lib.call('lgb_dft2', fd.data_ptr(), m, n, F.data_ptr(), M, N, ar, ac, sr, sc, orow, ocol,
              int(bool(unitary)), prec, ws.data_ptr(), nbytes, dv.stream_ptr())
    if prec != _lib.FP64:
        _lib.call('lgb_dft2_status', ws.data_ptr(), dv.stream_ptr())
    return _finish(F, out, host)


def dft2_batch(f, alpha, shape=None, shift=(0, 0), offset=(0, 0), unitary=True, npix=None,
               precision='fp64'):
    """``dft2`` of every field of a stack ``f`` [count, m, n] with one
    geometry (an extension of lentil's dft2, which takes one array): the DFT
    matrices are built once and the split path transforms the whole stack in
    one pair of tensor-core launches.  Returns [count, M, N], on the device
    for CUDA input, else as numpy."""
    host = not dv.is_tensor(f)
    fd = dv.to_device(f, torch.complex128)
    if fd.dim() != 3:
        raise ValueError('dft2_batch expects a 3-D stack [count, m, n]')
    count, m, n = (int(x) for x in fd.shape)
    M, N = _shape(shape, npix, (m, n))
    ar, ac = _pair(alpha, 'alpha')
    sr, sc = _pair(shift, 'shift')
    orow, ocol = _pair(offset, 'offset')
    prec = _lib.precision_code(precision)
    F = torch.empty((count, M, N), dtype=torch.complex128, device=fd.device)
    nbytes = _lib.load().lgb_dft2_batch_workspace_size(count, m, n, M, N, prec)
    ws = dv.workspace(nbytes)
    _lib.call('lgb_dft2_batch', fd.data_ptr(), count, m, n, F.data_ptr(), M, N, ar, ac, sr, sc,
              orow, ocol, int(bool(unitary)), prec, ws.data_ptr(), nbytes, dv.stream_ptr())
    if prec != _lib.FP64:
        _lib.call('lgb_dft2_status', ws.data_ptr(), dv.stream_ptr())
    return dv.to_host(F) if host else F


def idft2(F, alpha, shape=None, shift=(0, 0), unitary=True, out=None, npix=None,
          precision='fp64'):
    """Inverse DFT ``conj(dft2(conj(F))) / F.size`` (lentil/fourier.py:124-198)."""
    host = not dv.is_tensor(F)
    _check_out(out)
    Fd = dv.to_device(F, torch.complex128)
    if Fd.dim() != 2:
        raise ValueError('idft2 expects a 2-D array')
    m, n = Fd.shape
    M, N = _shape(shape, npix, (m, n))
    ar, ac = _pair(alpha, 'alpha')
    sr, sc = _pair(shift, 'shift')
    prec = _lib.precision_code(precision)
    f = torch.empty((M, N), dtype=torch.complex128, device=Fd.device)
    nbytes = _lib.load().lgb_idft2_workspace_size(m, n, M, N, prec)
    ws = dv.workspace(nbytes)
    _lib.call('lgb_idft2', Fd.data_ptr(), m, n, f.data_ptr(), M, N, ar, ac, sr, sc,
              int(bool(unitary)), prec, ws.data_ptr(), nbytes, dv.stream_ptr())
    if prec != _lib.FP64:
        _lib.call('lgb_dft2_status', ws.data_ptr(), dv.stream_ptr())
    return _finish(f, out, host)
