"""Far-field propagation by MFT, drop-in for ``lentil.propagate_dft``
(lentil/propagate.py:147-272).

The window algebra (tilt -> integer + subpixel shift, output/mask window
intersection, lentil's centring of the clipped window) runs on the host in
integers; every field's transform runs on the GPU through ``fourier.dft2``.
"""
import numpy as np

from . import extent as ext
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
