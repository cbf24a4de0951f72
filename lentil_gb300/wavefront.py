"""Monochromatic wavefront with device-resident fields, drop-in for
``lentil.Wavefront`` (lentil/wavefront.py:12-165)."""
import numpy as np
import torch

from . import _device as dv
from . import field as fld
from .field import Field
from .ptype import ptype as _ptype, none, pupil, image


class Wavefront:
    """Parameters and attributes as lentil's Wavefront.  ``.field`` and
    ``.intensity`` return numpy arrays unless the wavefront was built from
    CUDA tensors (then CUDA tensors); ``.insert`` updates ``out`` in place."""

    def __init__(self, wavelength, pixelscale=None, diameter=None, focal_length=None,
                 tilt=None, ptype=None):
        from .plane import Tilt
        self.focal_length = focal_length if focal_length else None
        self.diameter = diameter
        self.shape = ()
        self._wavelength = wavelength
        self._pixelscale = None if pixelscale is None else np.broadcast_to(pixelscale, (2,))
        self.ptype = ptype
        self._tensor_io = False
        if tilt is not None:
            if len(tilt) != 2:
                raise ValueError('tilt must be specified as [rx, ry]')
            tilt = [Tilt(x=tilt[0], y=tilt[1])]
        self.data = [Field(data=np.array(1, dtype=complex), offset=None, tilt=tilt)]

    def __mul__(self, plane):
        return plane.__mul__(self)

    def __rmul__(self, other):
        return self.__mul__(other)

    @property
    def wavelength(self):
        return self._wavelength

    @property
    def pixelscale(self):
        return self._pixelscale

    @property
    def ptype(self):
        return self._ptype

    @ptype.setter
    def ptype(self, value):
        p = _ptype(value)
        if p not in (none, pupil, image):
            raise TypeError(f"invalid ptype '{value}' for Wavefront")
        self._ptype = p

    def _deliver(self, t):
        return t if self._tensor_io else dv.to_host(t)

    def field_tensor(self):
        """Complex field as a CUDA complex128 tensor (lentil/wavefront.py:101-112)."""
        out = torch.zeros(tuple(int(s) for s in self.shape), dtype=torch.complex128,
                          device=dv.device())
        for f in self.data:
            fld.insert(f, out)
        return out

    def intensity_tensor(self):
        """Intensity as a CUDA float64 tensor (lentil/wavefront.py:114-125)."""
        out = torch.zeros(tuple(int(s) for s in self.shape), dtype=torch.float64,
                          device=dv.device())
        for f in fld.reduce(self.data):
            fld.insert(f, out, intensity=True)
        return out

    @property
    def field(self):
        return self._deliver(self.field_tensor())

    @property
    def intensity(self):
        return self._deliver(self.intensity_tensor())

    @classmethod
    def empty(cls, wavelength, pixelscale=None, diameter=None, focal_length=None, tilt=None,
              shape=None, ptype=None):
        """Wavefront with no fields (lentil/wavefront.py:127-142)."""
        w = cls(wavelength=wavelength, pixelscale=pixelscale, diameter=diameter,
                focal_length=focal_length, tilt=tilt, ptype=ptype)
        w.data = []
        w.shape = () if shape is None else shape
        return w

    def insert(self, out, weight=1):
        """out += weight * intensity, in place (lentil/wavefront.py:145-165)."""
        for f in fld.reduce(self.data):
            out = fld.insert(f, out, intensity=True, weight=weight)
        return out
