"""Far-field propagation, drop-in for ``lentil.propagate_dft`` and
``lentil.propagate_fft`` (lentil/propagate.py:9-272).

The window algebra (tilt -> integer + subpixel shift, output/mask window
intersection, lentil's centring of the clipped window, the FFT padding) runs
on the host in integers; every transform runs on the GPU through
``fourier.dft2``.  lentil's FFT propagation is a centred, ortho-normalised
FFT of the field zero-padded to ``round(1/alpha)``: exactly a centred DFT
with alpha = 1/N, which the MFT kernels evaluate over the field's support
only (no padded array is formed) at any N, not just FFT-friendly sizes.
"""
import numpy as np
import torch

from . import _device as dv
from . import extent as ext
from . import field as fld
from . import fourier
from . import util
from .field import Field
from .ptype import pupil, image


def _dft_alpha(dx, du, wavelength, z, oversample):
    """lentil/propagate.py:121-123."""
    return ((dx[0] * du[0]) / (wavelength * z * oversample),
            (dx[1] * du[1]) / (wavelength * z * oversample))


def _propagate_ptype(ptype, method='fraunhofer'):
    """lentil/propagate.py:263-272."""
    if ptype not in (pupil, image):
        raise TypeError("Wavefront must have ptype 'pupil' or 'image'")
    return image if ptype == pupil else pupil


def _mask_window(mask):
    """Shape and centre shift of the nonzero region of an output mask
    (lentil/propagate.py:245-260)."""
    rmin, rmax, cmin, cmax = util.boundary(mask, 0)
    shape = (rmax - rmin + 1, cmax - cmin + 1)
    shift = (rmin + shape[0] // 2 - mask.shape[0] // 2, cmin + shape[1] // 2 - mask.shape[1] // 2)
    return shape, shift


class FieldJob:
    """One field's MFT: its data and where its window lands."""
    __slots__ = ('field', 'alpha', 'shape', 'shift', 'offset_out')

    def __init__(self, field, alpha, shape, shift, offset_out):
        self.field, self.alpha, self.shape, self.shift, self.offset_out = (
            field, alpha, shape, shift, offset_out)


def plan_fields(wavefront, pixelscale, shape=None, prop_shape=None, oversample=2, mask=None):
    """Window maths of propagate_dft for every field (lentil/propagate.py:175-240).

    Returns (ptype_out, shape_out, du, jobs); a field whose window misses the
    output produces no job, as in lentil."""
    ptype_out = _propagate_ptype(wavefront.ptype, method='fraunhofer')
    shape = np.asarray(wavefront.shape) if shape is None else np.broadcast_to(shape, (2,))
    prop_shape = np.asarray(shape) if prop_shape is None else np.broadcast_to(prop_shape, (2,))
    shape_out = shape * oversample
    prop_shape_out = prop_shape * oversample
    if mask is not None:
        mask = np.asarray(mask)
        if np.all(mask.shape != shape_out):
            raise ValueError(f'shape mismatch: mask shape {mask.shape} != output shape {tuple(shape_out)}')
        mshape, mshift = _mask_window(mask)
        out_extent = ext.array_extent(mshape, mshift)
    else:
        out_extent = ext.array_extent(shape_out, shift=(0, 0))
    dx = wavefront.pixelscale
    du = np.broadcast_to(pixelscale, (2,))
    z = wavefront.focal_length
    jobs = []
    for field in wavefront.data:
        shift = field.shift(z=z, wavelength=wavefront.wavelength, pixelscale=du,
                            oversample=oversample, indexing='ij')
        whole = np.trunc(shift)
        subpx = np.asarray(shift, dtype=float) - whole
        prop_extent = ext.array_extent(prop_shape_out, whole)
        if not ext.intersect(out_extent, prop_extent):
            continue
        ishape = ext.intersection_shape(out_extent, prop_extent)
        ishift = ext.intersection_shift(out_extent, prop_extent)
        iextent = ext.array_extent(ishape, ishift)
        # extra shift that re-centres a clipped window (lentil/propagate.py:221-230)
        pshift = np.array(ext.array_center(prop_extent)) - np.array(ext.array_center(iextent))
        alpha = _dft_alpha(dx, du, wavefront.wavelength, z, oversample)
        jobs.append(FieldJob(field, alpha, ishape, pshift + subpx, ishift))
    return ptype_out, shape_out, du, jobs


def propagate_dft(wavefront, pixelscale, shape=None, prop_shape=None, oversample=2, mask=None,
                  precision='fp64'):
    """Propagate a Wavefront to the far field with the MFT
    (lentil/propagate.py:147-242).  ``precision`` selects the complex128
    path (default, lentil parity) or the split tensor-core path."""
    from .wavefront import Wavefront
    ptype_out, shape_out, du, jobs = plan_fields(wavefront, pixelscale, shape, prop_shape,
                                                 oversample, mask)
    out = Wavefront.empty(wavelength=wavefront.wavelength, pixelscale=du / oversample,
                          focal_length=wavefront.focal_length, shape=shape_out, ptype=ptype_out)
    out._tensor_io = wavefront._tensor_io
    for j in jobs:
        data = fourier.dft2(j.field.data, alpha=j.alpha, shape=j.shape, shift=j.shift,
                            offset=j.field.offset, unitary=True, precision=precision)
        out.data.append(Field(data=data, pixelscale=du / oversample, offset=j.offset_out))
    return out


# --------------------------------------------------------------------------
# FFT propagation
# --------------------------------------------------------------------------
def _fft_shape(dx, du, z, wavelength, oversample):
    """Padded FFT shape and the propagation wavelength it implies
    (lentil/propagate.py:126-132)."""
    alpha = _dft_alpha(dx, du, z, wavelength, oversample)
    fft_shape = np.round(np.reciprocal(alpha)).astype(int)
    prop_wavelength = np.min((fft_shape / oversample * dx * du) / z)
    return fft_shape, prop_wavelength


def scratch_shape(wavelength, dx, du, z, oversample):
    """Scratch shape an FFT propagation over ``wavelength`` needs
    (lentil/propagate.py:91-118)."""
    dx = np.broadcast_to(dx, (2,))
    du = np.broadcast_to(du, (2,))
    fft_shape, _ = _fft_shape(dx, du, z, np.max(wavelength), oversample)
    return tuple(fft_shape)


def _has_tilt(wavefront):
    """lentil/propagate.py:139-144."""
    return any(f.tilt for f in wavefront.data)


def _centred_dft_coords(g_shape, start, fft_shape):
    """dft2 offset and shift that make a DFT with alpha = 1/N of ``g`` (placed
    at ``start`` in an otherwise zero N_r x N_c array) equal the centred ortho
    FFT ifftshift(fft2(fftshift(x), norm='ortho')) of that array.  Per axis
    the FFT's phase is (u - c)(r - c)/N with c = N//2 for even N and N//2 + 1
    for odd N (fftshift and ifftshift differ by one sample there): offset
    start + m//2 - c on the input, shift N - 2*(N//2) on the output."""
    offset, shift = [], []
    for ax in range(2):
        N, m = int(fft_shape[ax]), int(g_shape[ax])
        odd = N % 2
        offset.append(int(start[ax]) + m // 2 - N // 2 - odd)
        shift.append(float(odd))
    return tuple(offset), tuple(shift)


def _centred_dft(g, start, fft_shape, precision):
    """Centred ortho DFT of the N_r x N_c array holding ``g`` at ``start``."""
    offset, shift = _centred_dft_coords(g.shape, start, fft_shape)
    return fourier.dft2(g, (1.0 / fft_shape[0], 1.0 / fft_shape[1]),
                        shape=(int(fft_shape[0]), int(fft_shape[1])), shift=shift,
                        offset=offset, unitary=True, precision=precision)


def _pad_geometry(n, N):
    """Source slice start/stop and destination start of lentil's centred
    pad/crop along one axis (lentil/util.py:31-90)."""
    if N - n <= 0:
        s0 = (n - N) // 2
        return s0, s0 + N, 0
    return 0, n, (N - n) // 2


def _insert_box(wavefront, fft_shape):
    """Bounding rows/columns, inside an array of ``fft_shape``, that the
    wavefront's fields cover when inserted centred (lentil/field.py:231-305)."""
    r0, r1, c0, c1 = int(fft_shape[0]), 0, int(fft_shape[1]), 0
    for f in wavefront.data:
        if f.size == 0:
            continue
        fs = (1, 1) if f.data.dim() < 2 else f.shape
        ul = (int(fft_shape[0]) // 2 - fs[0] // 2 + int(f.offset[0]),
              int(fft_shape[1]) // 2 - fs[1] // 2 + int(f.offset[1]))
        r0, r1 = min(r0, max(ul[0], 0)), max(r1, min(ul[0] + fs[0], int(fft_shape[0])))
        c0, c1 = min(c0, max(ul[1], 0)), max(c1, min(ul[1] + fs[1], int(fft_shape[1])))
    return r0, r1, c0, c1


def propagate_fft(wavefront, pixelscale, shape=None, oversample=2, scratch=None,
                  precision='fp64'):
    """Propagate a Wavefront to the far field as lentil's zero-padded FFT
    does (lentil/propagate.py:9-88): the output Wavefront holds one Field of
    the full FFT shape ``round(1/alpha)``, its wavelength is recomputed for
    the integer padding, and ``scratch`` (numpy array or CUDA tensor larger
    than the FFT shape in both dimensions) receives the padded field, as in
    lentil.  ``precision`` selects the complex128 path (default, parity with
    numpy's FFT) or a split tensor-core path."""
    from .wavefront import Wavefront
    if _has_tilt(wavefront):
        raise NotImplementedError('propagate_fft does not support Wavefronts with fitted tilt. '
                                  'Use propagate_dft instead.')
    ptype_out = _propagate_ptype(wavefront.ptype, method='fraunhofer')
    pixelscale = np.broadcast_to(pixelscale, (2,))
    fft_shape, prop_wavelength = _fft_shape(wavefront.pixelscale, pixelscale,
                                            wavefront.focal_length, wavefront.wavelength,
                                            oversample)
    if shape is None:
        shape_out = tuple(int(x) for x in fft_shape)
    else:
        shape = tuple(np.broadcast_to(shape, (2,)))
        if np.any(np.asarray(shape) > fft_shape / oversample):
            raise ValueError(f'requested shape {tuple(shape)} is larger in at least one '
                             f'dimension than maximum propagation shape '
                             f'{tuple(fft_shape // oversample)}')
        shape_out = (shape[0] * oversample, shape[1] * oversample)
    out = Wavefront.empty(wavelength=prop_wavelength, pixelscale=pixelscale / oversample,
                          focal_length=wavefront.focal_length, shape=shape_out, ptype=ptype_out)
    out._tensor_io = wavefront._tensor_io
    Nr, Nc = int(fft_shape[0]), int(fft_shape[1])
    if scratch is not None:
        if not all(np.asarray(scratch.shape) > fft_shape):
            raise ValueError(f'scratch must have shape greater than or equal to {tuple(fft_shape)}')
        region = torch.zeros((Nr, Nc), dtype=torch.complex128, device=dv.device())
        for f in wavefront.data:
            fld.insert(f, region)
        if dv.is_tensor(scratch):
            scratch[:Nr, :Nc] = region
        else:
            scratch[:Nr, :Nc] = dv.to_host(region)
        r0, r1, c0, c1 = _insert_box(wavefront, fft_shape)
        if r1 > r0 and c1 > c0:
            data = _centred_dft(region[r0:r1, c0:c1].contiguous(), (r0, c0), fft_shape, precision)
        else:
            data = torch.zeros((Nr, Nc), dtype=torch.complex128, device=dv.device())
    else:
        full = wavefront.field_tensor()
        (a0, a1, d0), (b0, b1, e0) = (_pad_geometry(int(full.shape[0]), Nr),
                                      _pad_geometry(int(full.shape[1]), Nc))
        data = _centred_dft(full[a0:a1, b0:b1].contiguous(), (d0, e0), fft_shape, precision)
    out.data.append(Field(data=data, pixelscale=pixelscale / oversample))
    return out
