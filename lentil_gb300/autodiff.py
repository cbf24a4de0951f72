"""Differentiable MFT intensity for phase retrieval (no counterpart in
lentil, which has no gradients).

``mft_intensity(opd, amp, ...)`` is lentil's monochromatic PSF
(``propagate_dft(Wavefront(lam) * Pupil(amp, opd)).intensity``, one field,
no tilt) as a ``torch.autograd.Function`` of the OPD map.  Forward: phasor
kernel, MFT (complex128 or split tensor-core), |F|^2.  Backward, with the
field recomputed instead of stored: dL/dF* = dL/dI * F, the adjoint MFT
(a dft2 of its conjugate with offset and shift swapped and negated), and
dL/dopd = (2 pi / lambda) 2 Im(g conj(f)) from the phasor-adjoint kernel.
"""
from collections import namedtuple

import numpy as np
import torch

from . import _device as dv
from . import _lib
from . import fourier
from . import util
from .propagate import _dft_alpha

Geometry = namedtuple('Geometry', 'wavelength alpha shape shift offset slc plane precision')


def geometry(amp, wavelength, pixelscale_in, focal_length, pixelscale_out, shape,
             oversample=2, precision='fp64'):
    """MFT geometry of ``propagate_dft`` for an untilted single-field pupil
    whose support is ``amp != 0`` (lentil/propagate.py:175-240,
    lentil/plane.py:494-510): full output window, zero shift, slice offset."""
    a = dv.to_host(amp) if dv.is_tensor(amp) else np.asarray(amp)
    slc = util.boundary_slice(a != 0)
    off = util.slice_offset(slc, a.shape)
    dx = np.broadcast_to(pixelscale_in, (2,))
    du = np.broadcast_to(pixelscale_out, (2,))
    shp = np.broadcast_to(shape, (2,)) * oversample
    alpha = _dft_alpha(dx, du, wavelength, focal_length, oversample)
    r0, c0 = int(slc[0].start), int(slc[1].start)
    m, n = int(slc[0].stop) - r0, int(slc[1].stop) - c0
    return Geometry(float(wavelength), tuple(float(x) for x in alpha),
                    (int(shp[0]), int(shp[1])), (0.0, 0.0), tuple(int(x) for x in off),
                    (r0, c0, m, n), tuple(a.shape), precision)


def _phasor_stack(amp, opd, g):
    """Fields f [K, m, n] of a stack opd [K, H, W] in one launch; the split
    precisions take the FP32-sine form, whose 1e-7 error is below the 16-bit
    operand split that follows."""
    r0, c0, m, n = g.slc
    H, W = g.plane
    K = int(opd.shape[0])
    f = torch.empty((K, m, n), dtype=torch.complex128, device=amp.device)
    _lib.call('lgb_phasor_stack', amp.data_ptr(), opd.data_ptr(), K, H, W, r0, c0, m, n,
              g.wavelength, int(g.precision != 'fp64'), f.data_ptr(), dv.stream_ptr())
    return f


def _forward_field(amp, opd, g):
    """Fields f [K, m, n] of a stack of OPD maps opd [K, H, W] and their
    transforms F [K, M, N] (one batched MFT for the whole stack)."""
    f = _phasor_stack(amp, opd.contiguous(), g)
    F = fourier.dft2_batch(f, g.alpha, shape=g.shape, shift=g.shift, offset=g.offset,
                           unitary=True, precision=g.precision)
    return f, F


class MFTIntensity(torch.autograd.Function):
    """I = |dft2(amp exp(2 pi i opd / lambda))|^2, differentiable in opd.
    ``opd`` is one map [H, W] or a stack [K, H, W] sharing ``amp`` and the
    geometry (e.g. focus-diverse images); the stack is transformed in one
    batched MFT, forward and backward."""

    @staticmethod
    def forward(ctx, opd, amp, g):
        single = opd.dim() == 2
        opd = opd.detach().to(torch.float64).contiguous()
        opd = opd.unsqueeze(0) if single else opd
        amp = amp.detach().to(torch.float64).contiguous()
        _, F = _forward_field(amp, opd, g)
        I = torch.empty(F.shape, dtype=torch.float64, device=F.device)
        _lib.call('lgb_abs2', F.data_ptr(), I.data_ptr(), F.numel(), dv.stream_ptr())
        ctx.save_for_backward(opd, amp)
        ctx.g, ctx.single = g, single
        return I[0] if single else I

    @staticmethod
    def backward(ctx, grad_I):
        opd, amp = ctx.saved_tensors
        g = ctx.g
        f, F = _forward_field(amp, opd, g)                 # recomputed, not stored
        gI = grad_I.detach().to(torch.float64).contiguous().reshape(F.shape)
        Hc = torch.empty_like(F)
        _lib.call('lgb_intensity_adjoint', F.data_ptr(), gI.data_ptr(), Hc.data_ptr(), F.numel(),
                  dv.stream_ptr())
        r0, c0, m, n = g.slc
        q = fourier.dft2_batch(Hc, g.alpha, shape=(m, n), shift=(-g.offset[0], -g.offset[1]),
                               offset=(-g.shift[0], -g.shift[1]), unitary=True,
                               precision=g.precision)
        grad = torch.zeros_like(opd)
        for k in range(opd.shape[0]):
            _lib.call('lgb_phasor_adjoint', q[k].data_ptr(), f[k].data_ptr(), m, n, g.wavelength,
                      grad[k].data_ptr(), g.plane[1], r0, c0, dv.stream_ptr())
        return (grad[0] if ctx.single else grad), None, None


def mft_intensity(opd, amp, g):
    """Differentiable PSF intensity of ``amp * exp(2 pi i opd / lambda)``
    for one OPD map or a stack of them."""
    return MFTIntensity.apply(opd, amp, g)


class _BasisOPD(torch.autograd.Function):
    """OPD = sum_k c_k B_k over an FP32 basis [K, H, W], differentiable in c
    (lgb_basis_expand / lgb_basis_project: one pass over the basis each)."""

    @staticmethod
    def forward(ctx, coeffs, basis32):
        K, P = int(basis32.shape[0]), int(basis32[0].numel())
        c = coeffs.detach().to(torch.float64).contiguous()
        out = torch.empty(tuple(basis32.shape[1:]), dtype=torch.float64, device=c.device)
        _lib.call('lgb_basis_expand', basis32.data_ptr(), c.data_ptr(), K, P, out.data_ptr(),
                  dv.stream_ptr())
        ctx.save_for_backward(basis32)
        return out

    @staticmethod
    def backward(ctx, grad):
        (basis32,) = ctx.saved_tensors
        K, P = int(basis32.shape[0]), int(basis32[0].numel())
        g = grad.detach().to(torch.float64).contiguous()
        out = torch.empty(K, dtype=torch.float64, device=g.device)
        nb = _lib.load().lgb_basis_project_workspace_size(K)
        ws = dv.workspace(nb)
        _lib.call('lgb_basis_project', basis32.data_ptr(), g.data_ptr(), K, P, out.data_ptr(),
                  ws.data_ptr(), nb, dv.stream_ptr())
        return out, None


class _StackedOPD(torch.autograd.Function):
    """OPD_i = sum_k c_k B_k + D_i for the diversity maps D [n, H, W] in one
    pass over the FP32 basis, and dL/dc = B . sum_i dL/dOPD_i in one more
    (lgb_basis_expand_stack / lgb_basis_project_stack), in place of a
    broadcast add and a reduction over the images."""

    @staticmethod
    def forward(ctx, coeffs, basis32, add):
        K, P = int(basis32.shape[0]), int(basis32[0].numel())
        n = int(add.shape[0])
        c = coeffs.detach().to(torch.float64).contiguous()
        d = add.detach().to(torch.float64).contiguous()
        out = torch.empty((n,) + tuple(basis32.shape[1:]), dtype=torch.float64, device=c.device)
        _lib.call('lgb_basis_expand_stack', basis32.data_ptr(), c.data_ptr(), K, P, d.data_ptr(),
                  n, out.data_ptr(), dv.stream_ptr())
        ctx.save_for_backward(basis32)
        ctx.n = n
        return out

    @staticmethod
    def backward(ctx, grad):
        (basis32,) = ctx.saved_tensors
        K, P = int(basis32.shape[0]), int(basis32[0].numel())
        g = grad.detach().to(torch.float64).contiguous()
        out = torch.empty(K, dtype=torch.float64, device=g.device)
        nb = _lib.load().lgb_basis_project_workspace_size(K)
        ws = dv.workspace(nb)
        _lib.call('lgb_basis_project_stack', basis32.data_ptr(), g.data_ptr(), ctx.n, K, P,
                  out.data_ptr(), ws.data_ptr(), nb, dv.stream_ptr())
        return out, None, (grad if ctx.needs_input_grad[2] else None)


class _SquaredError(torch.autograd.Function):
    """sum (I - T)^2 and its gradient 2 (I - T) dL in one kernel pass each
    (lgb_sq_error, lgb_sq_error_grad), in place of a chain of FP64
    elementwise kernels and reductions."""

    @staticmethod
    def forward(ctx, I, T):
        if I.shape != T.shape:
            raise ValueError(f'images {tuple(I.shape)} and targets {tuple(T.shape)} differ')
        I = I.to(torch.float64).contiguous()
        T = T.to(torch.float64).contiguous()
        loss = torch.empty((), dtype=torch.float64, device=I.device)
        ws = torch.empty(_lib.load().lgb_sq_error_workspace_size(), dtype=torch.uint8,
                         device=I.device)
        _lib.call('lgb_sq_error', I.data_ptr(), T.data_ptr(), I.numel(), loss.data_ptr(),
                  ws.data_ptr(), ws.numel(), dv.stream_ptr())
        ctx.save_for_backward(I, T)
        return loss

    @staticmethod
    def backward(ctx, grad):
        I, T = ctx.saved_tensors
        g = grad.to(torch.float64).contiguous()
        dI = torch.empty_like(I)
        _lib.call('lgb_sq_error_grad', I.data_ptr(), T.data_ptr(), I.numel(), g.data_ptr(),
                  dI.data_ptr(), dv.stream_ptr())
        return dI, (-dI if ctx.needs_input_grad[1] else None)


def squared_error(I, T):
    """sum((I - T) ** 2) as one device pass, differentiable in I and T."""
    return _SquaredError.apply(I, T)


class PhaseRetrieval:
    """Focus-diverse phase-retrieval loss sum_k sum (PSF_k - target_k)^2 over
    OPD = basis . coeffs (+ an optional free-form map), with the diversity
    OPD maps added per image.

    ``loss`` runs eagerly.  ``graphed_loss`` is the same function of the
    coefficients captured once as two CUDA graphs (forward, backward) with
    ``torch.cuda.make_graphed_callables`` and replayed on later calls: the
    transforms run from cached, pinned dft2 plans and every launch goes to
    the current stream, so a replay issues no host work per kernel.  The
    diversity maps, targets and basis are read where they lie when the graphs
    are captured (assign new targets in place).  ``check()`` raises a
    device-side failure of the transforms."""

    def __init__(self, amp, basis, diversity, targets, g):
        dev = dv.device()
        self.amp = dv.to_device(amp, torch.float64)
        self.basis = dv.to_device(basis, torch.float64)          # (K, H, W)
        self.diversity = [dv.to_device(d, torch.float64) for d in diversity]
        self.targets = [dv.to_device(t, torch.float64) for t in targets]
        self.g = g
        self.device = dev
        self._graphed = None
        self._pins = None
        # the split precisions expand the modes from an FP32 copy of the
        # basis (half the bytes, FP32 multiply-adds); fp64 keeps torch's FP64 sum
        self._basis32 = None if g.precision == 'fp64' else self.basis.float().contiguous()

    def opd(self, coeffs, free=None):
        if self._basis32 is not None:
            o = _BasisOPD.apply(coeffs, self._basis32)
        else:
            o = torch.einsum('k,khw->hw', coeffs, self.basis)
        return o if free is None else o + free

    def _stack(self, coeffs, div, free=None):
        """The OPD maps of all diversity images, [n, H, W] (one batched MFT)."""
        if self._basis32 is not None and free is None:
            return _StackedOPD.apply(coeffs, self._basis32, div)
        return self.opd(coeffs, free).unsqueeze(0) + div

    def loss(self, coeffs, free=None):
        stack = self._stack(coeffs, torch.stack(self.diversity), free)
        return squared_error(mft_intensity(stack, self.amp, self.g), torch.stack(self.targets))

    def graphed_loss(self, coeffs):
        """``loss(coeffs)`` replayed from CUDA graphs (captured on first use)."""
        if self._graphed is None:
            div = torch.stack(self.diversity)
            tgt = torch.stack(self.targets)

            def fn(c):
                return squared_error(mft_intensity(self._stack(c, div), self.amp, self.g), tgt)

            sample = coeffs.detach().clone().requires_grad_(True)
            with fourier.pinned_plans() as pins:
                self._graphed = torch.cuda.make_graphed_callables(fn, (sample,))
            self._pins = pins
            self._static = (div, tgt)
        return self._graphed(coeffs)

    def release_graphs(self):
        """Drop the captured graphs and unpin their dft2 plans."""
        self._graphed = None
        if self._pins is not None:
            self._pins.release()
            self._pins = None

    def check(self):
        """Wait for the device and raise a failure of a split-precision transform."""
        fourier.plan_status()
