"""Optical planes, drop-in for ``lentil.Plane``/``Pupil``/``Image``/``Tilt``.

The extension protocol is lentil's: subclasses override ``__amp__``,
``__opd__``, ``__mask__`` (lentil/plane.py:40-50) and ``__mul__``; tilt
objects implement ``__shift__(xs, ys, z, wavelength)``.  ``Plane.__mul__``
builds the per-segment phasor amp*mask*exp(2 pi i opd/lambda)
(lentil/plane.py:477-516) with the library's phasor kernel; masks, slices
and tilt fits are host-side bookkeeping as in lentil.
"""
import copy

import numpy as np
import torch

from . import _device as dv
from . import _lib
from . import util
from .field import Field
from .ptype import ptype as _ptype, none, pupil, image, tilt as tilt_t, transform

# Wavefront ptype -> {Plane ptype -> result ptype}; a missing entry means the
# product is not allowed (lentil/plane.py:632-668)
_MUL_PTYPE = {
    none: {none: none, pupil: pupil, image: image, tilt_t: none, transform: none},
    pupil: {pupil: pupil, tilt_t: pupil, transform: pupil},
    image: {image: image, tilt_t: pupil, transform: pupil},
}


def _np(x):
    """Host view of an array-like (tensors are copied back once)."""
    return dv.to_host(x) if dv.is_tensor(x) else np.asarray(x)


def _asarray(x):
    return x if dv.is_tensor(x) else np.asarray(x)


def _size(x):
    return int(x.numel()) if dv.is_tensor(x) else int(np.asarray(x).size)


def _scalar(x):
    return float(_np(x).reshape(-1)[0])


class _PlaneBase:
    """lentil/plane.py:19-396 (the parts on the diffraction path)."""

    def __new__(cls, *args, **kwargs):
        self = super().__new__(cls)
        self._amplitude = np.array(1)
        self._opd = np.array(0)
        self._mask = None
        self._pixelscale = None
        self._ptype = _ptype(None)
        self._diameter = None
        self.tilt = []
        self._frozen = False
        self.__freeze_attrs__ = ['amplitude', 'opd']
        return self

    def __repr__(self):
        return f'{self.__class__.__name__}()'

    def __amp__(self):
        return self._amplitude

    def __mask__(self):
        if self._mask is None:
            a = self.amplitude
            return (a != 0) if dv.is_tensor(a) else np.copy(a).astype(bool)
        return self._mask

    def _mask_is_amplitude(self):
        """True when the mask is the amplitude's nonzero pattern: no mask was
        given and ``__mask__`` is not overridden.  Its shape and rank are then
        the amplitude's, and amplitude * mask is the amplitude itself."""
        return self._mask is None and type(self).__mask__ is _PlaneBase.__mask__

    def __opd__(self):
        return self._opd

    def __mul__(self, wavefront):
        raise NotImplementedError

    def __rmul__(self, other):
        return self.__mul__(other)

    @property
    def ptype(self):
        return self._ptype

    @ptype.setter
    def ptype(self, value):
        self._ptype = _ptype(value)

    @property
    def amplitude(self):
        return self._amplitude if self.frozen else self.__amp__()

    @amplitude.setter
    def amplitude(self, value):
        if self.frozen:
            raise RuntimeError("Can't set amplitude while Plane is frozen")
        self._amplitude = _asarray(value)

    @property
    def opd(self):
        return self._opd if self.frozen else self.__opd__()

    @opd.setter
    def opd(self, value):
        if self.frozen:
            raise RuntimeError("Can't set opd while Plane is frozen")
        self._opd = _asarray(value)

    @property
    def mask(self):
        return self.__mask__()

    @property
    def global_mask(self):
        m = self.mask
        return m if self.size < 2 else (m.sum(0) if dv.is_tensor(m) else np.sum(m, axis=0))

    @property
    def pixelscale(self):
        return self._pixelscale

    @property
    def diameter(self):
        """lentil/plane.py:147-171."""
        if self._diameter is not None:
            return self._diameter
        rmin, rmax, cmin, cmax = util.boundary(_np(self.global_mask))
        return np.max(np.max((rmax - rmin, cmax - cmin)) * np.asarray(self.pixelscale))

    def _mask_meta(self):
        """(shape, rank) of the mask, without building an amplitude-derived one."""
        m = self.amplitude if self._mask_is_amplitude() else self.mask
        shp = tuple(m.shape) if hasattr(m, 'shape') else np.shape(m)
        return shp, len(shp)

    @property
    def shape(self):
        shp, nd = self._mask_meta()
        return shp if nd in (0, 1, 2) else shp[1:]

    @property
    def size(self):
        shp, nd = self._mask_meta()
        return 1 if nd in (0, 1, 2) else int(shp[0])

    @property
    def frozen(self):
        return self._frozen

    def freeze(self, inplace=True):
        """Cache ``__freeze_attrs__`` (lentil/plane.py:218-257)."""
        if self.frozen:
            raise RuntimeError('Plane is already frozen. Call thaw() to unfreeze.')
        p = self if inplace else copy.deepcopy(self)
        for attr in p.__freeze_attrs__:
            setattr(p, f'_{attr}', getattr(p, attr))
        p._frozen = True
        return None if inplace else p

    def thaw(self):
        self._frozen = False
        self.__dict__.pop('_lgb_device_field', None)    # device copy kept while frozen


class Plane(_PlaneBase):
    """lentil/plane.py:414-611."""

    def __init__(self, amplitude=None, opd=None, mask=None, pixelscale=None, diameter=None,
                 ptype=None, **kwargs):
        if 'amp' in kwargs:
            if amplitude is not None:
                raise AttributeError("Got both 'amplitude' and 'amp', which are aliases of one another")
            amplitude = kwargs['amp']
        if amplitude is not None:
            self._amplitude = _asarray(amplitude)
        if opd is not None:
            self._opd = _asarray(opd)
        if mask is not None:
            self._mask = _asarray(mask)
        if pixelscale is not None:
            self._pixelscale = np.broadcast_to(pixelscale, (2,))
        if diameter is not None:
            self._diameter = diameter
        if ptype is not None:
            self._ptype = _ptype(ptype)

    @property
    def _slice(self):
        return _plane_slice(self.mask)

    def _tensor_io(self):
        return any(dv.is_tensor(x) for x in (self.amplitude, self.opd, self._mask))

    def __mul__(self, wavefront):
        """Per-segment phasor times every incoming field (lentil/plane.py:477-516)."""
        if self.ptype not in _MUL_PTYPE[wavefront.ptype]:
            raise TypeError(f"can't multiply Wavefront with ptype '{wavefront.ptype}' by Plane "
                            f"with ptype '{self.ptype}'")
        from .wavefront import Wavefront
        pixelscale = _mul_pixelscale(self.pixelscale, wavefront.pixelscale)
        shape = wavefront.shape if self.shape == () else self.shape
        out = Wavefront.empty(wavelength=wavefront.wavelength, pixelscale=pixelscale,
                              focal_length=wavefront.focal_length, shape=shape,
                              ptype=_MUL_PTYPE[wavefront.ptype][self.ptype])
        out._tensor_io = wavefront._tensor_io or self._tensor_io()
        amp, opd, mask = self.amplitude, self.opd, self.mask
        amp_arr = _size(amp) > 1
        opd_arr = _size(opd) > 1
        amp_d = dv.to_device(amp, torch.float64) if amp_arr else None
        opd_d = dv.to_device(opd, torch.float64) if opd_arr else None
        amp_v = 0.0 if amp_arr else _scalar(amp)
        opd_v = 0.0 if opd_arr else _scalar(opd)
        # an amplitude-derived mask multiplies the amplitude by one where it
        # is nonzero and by zero where it is zero: nothing to apply
        mask_d = dv.to_device(mask, torch.float64) if amp_arr and not self._mask_is_amplitude() \
            else None
        plane_shape = tuple(self.shape)
        slices = _plane_slice(mask)
        for f in wavefront.data:
            for n, s in enumerate(slices):
                phasor = self._phasor(n, s, amp_d, amp_v, opd_d, opd_v, mask_d, plane_shape,
                                      wavefront.wavelength)
                pf = Field(data=phasor, pixelscale=self.pixelscale,
                           offset=util.slice_offset(s, plane_shape),
                           tilt=[self.tilt[n]] if self.tilt else [])
                res = f * pf
                if res.size > 0:
                    out.data.append(res)
        return out

    def _phasor(self, n, s, amp_d, amp_v, opd_d, opd_v, mask_d, plane_shape, wavelength):
        dev = dv.device()
        arr = amp_d if amp_d is not None else opd_d
        if arr is None:
            # both scalars: lentil's 0-d phasor
            ph = torch.empty((1, 1), dtype=torch.complex128, device=dev)
            _lib.call('lgb_phasor', None, amp_v, None, None, opd_v, 1, 1, 0, 0, 1, 1,
                      float(wavelength), ph.data_ptr(), dv.stream_ptr())
            return ph.reshape(())
        H, W = arr.shape[-2], arr.shape[-1]
        if s is Ellipsis or s == Ellipsis:
            r0, c0, m, nn = 0, 0, H, W
        else:
            r0, c0 = int(s[0].start), int(s[1].start)
            m, nn = int(s[0].stop) - r0, int(s[1].stop) - c0
        mptr = None
        if mask_d is not None:
            mk = mask_d if mask_d.dim() < 3 else mask_d[n]
            if mk.dim() == 2:
                mptr = mk.contiguous().data_ptr()
                mask_keep = mk
            elif float(mk.reshape(-1)[0]) == 0.0:
                amp_v, amp_d = 0.0, None
        ph = torch.empty((m, nn), dtype=torch.complex128, device=dev)
        _lib.call('lgb_phasor', dv.ptr(amp_d), amp_v, mptr if amp_d is not None else None,
                  dv.ptr(opd_d), opd_v, H, W, r0, c0, m, nn, float(wavelength), ph.data_ptr(),
                  dv.stream_ptr())
        return ph

    def ptt_vector(self):
        """Masked piston/x-tilt/y-tilt basis (lentil/plane.py:522-562)."""
        if self.shape == () or self.shape is None:
            return None
        if self.pixelscale is None:
            raise ValueError("can't create ptt_vector with pixelscale = ()")
        ps = np.broadcast_to(self.pixelscale, (2,))
        r, c = util.mesh(self.shape)
        base = np.stack([np.ones(r.size), r.ravel() * ps[0], -c.ravel() * ps[1]])
        mask = _np(self.mask)
        if self.size == 1:
            return base * mask.ravel()[None, :]
        v = np.empty((self.size * 3, int(np.prod(self.shape))))
        for k in range(self.size):
            v[3 * k:3 * k + 3] = base * mask[k].ravel()[None, :]
        return v

    def fit_tilt(self, inplace=False):
        """Least-squares tilt removal into Tilt objects (lentil/plane.py:564-611).

        The fit runs on the GPU without forming ``ptt_vector``: one kernel
        sums each mask's 3x3 normal equations of lentil's least-squares
        problem (deterministic FP64), the host solves them with ``lstsq``
        (the minimum-norm solution lentil's ``lstsq`` returns), and a second
        kernel removes the tilts with lentil's one-mask / several-mask rules.
        The OPD keeps its kind (numpy stays numpy, a CUDA tensor stays one)."""
        plane = self if inplace else copy.deepcopy(self)
        if plane.shape == () or plane.shape is None:
            return plane                       # no mask: ptt_vector is None
        if plane.pixelscale is None:
            raise ValueError("can't create ptt_vector with pixelscale = ()")
        opd_in = plane.opd
        if _size(opd_in) == 1:
            return plane
        H, W = (int(x) for x in plane.shape)
        S = plane.size
        ps = np.broadcast_to(plane.pixelscale, (2,)).astype(float)
        dev = dv.device()
        opd_d = dv.to_device(opd_in, torch.float64).reshape(H, W).contiguous()
        mask_d = dv.to_device(plane.mask, torch.float64).reshape(S, H, W).contiguous()
        sums = torch.empty((S, 9), dtype=torch.float64, device=dev)
        ws = dv.workspace(_lib.load().lgb_ptt_normal_workspace_size(S))
        _lib.call('lgb_ptt_normal', opd_d.data_ptr(), mask_d.data_ptr(), S, H, W, float(ps[0]),
                  float(ps[1]), sums.data_ptr(), ws.data_ptr(), ws.numel(), dv.stream_ptr())
        q = dv.to_host(sums)
        t = np.empty((S, 3))
        for k in range(S):
            a00, a01, a02, a11, a12, a22, y0, y1, y2 = q[k]
            A = np.array([[a00, a01, a02], [a01, a11, a12], [a02, a12, a22]])
            t[k] = np.linalg.lstsq(A, np.array([y0, y1, y2]), rcond=None)[0]
        t_d = torch.as_tensor(t, device=dev).contiguous()
        out = torch.empty((H, W), dtype=torch.float64, device=dev)
        _lib.call('lgb_remove_tilt', opd_d.data_ptr(), mask_d.data_ptr(), S, H, W, float(ps[0]),
                  float(ps[1]), t_d.data_ptr(), out.data_ptr(), dv.stream_ptr())
        plane.opd = out if dv.is_tensor(opd_in) else dv.to_host(out)
        plane.tilt.extend([Tilt(x=t[k, 1], y=t[k, 2]) for k in range(S)])
        return plane


def _mul_pixelscale(a, b):
    """lentil/plane.py:614-629."""
    a = None if a is None else np.broadcast_to(a, (2,))
    b = None if b is None else np.broadcast_to(b, (2,))
    if a is None:
        return b
    if b is None:
        return a
    if all(a == b):
        return a
    raise ValueError(f"can't multiply with inconsistent pixelscales: {a} != {b}")


def _plane_slice(mask):
    """Bounding-box slices of each mask layer (lentil/plane.py:671-705)."""
    if mask is None:
        return [Ellipsis]
    m = _np(mask)
    if m.ndim < 2:
        return [Ellipsis]
    if m.ndim == 2:
        return [util.boundary_slice(m)]
    if m.ndim == 3:
        return [util.boundary_slice(x) for x in m]
    raise ValueError('mask has invalid dimensions')


class Pupil(Plane):
    """Pupil plane carrying a focal length (lentil/plane.py:708-771)."""

    def __new__(cls, *args, **kwargs):
        self = super().__new__(cls, *args, **kwargs)
        self._focal_length = None
        self._ptype = pupil
        return self

    def __init__(self, amplitude=None, opd=None, mask=None, pixelscale=None, focal_length=None,
                 diameter=None, **kwargs):
        super().__init__(amplitude=amplitude, opd=opd, mask=mask, pixelscale=pixelscale,
                         diameter=diameter, ptype=pupil, **kwargs)
        if focal_length is not None:
            self._focal_length = focal_length

    def __mul__(self, wavefront):
        w = super().__mul__(wavefront)
        w.focal_length = self.focal_length
        return w

    @property
    def focal_length(self):
        return self._focal_length


class Image(Plane):
    """Image plane (lentil/plane.py:774-820)."""

    def __new__(cls, *args, **kwargs):
        self = super().__new__(cls, *args, **kwargs)
        self._ptype = image
        return self

    def __init__(self, amplitude=None, opd=None, mask=None, pixelscale=None, **kwargs):
        super().__init__(amplitude=amplitude, opd=opd, mask=mask, pixelscale=pixelscale,
                         ptype=image, **kwargs)

    def __mul__(self, wavefront):
        w = super().__mul__(wavefront)
        w.ptype = image
        return w

    def fit_tilt(self, *args, **kwargs):
        return self


class _TiltBase(Plane):
    """Planes implementing the tilt interface (lentil/plane.py:823-881)."""

    def __new__(cls, *args, **kwargs):
        self = super().__new__(cls, *args, **kwargs)
        self._ptype = _ptype(kwargs['ptype']) if 'ptype' in kwargs else tilt_t
        return self

    def __mul__(self, wavefront):
        w = super().__mul__(wavefront)
        for f in w.data:
            f.tilt.append(self)
        return w

    def __shift__(self, wavelength, x0, y0, **kwargs):
        raise NotImplementedError


class Tilt(_TiltBase):
    """Angular tilt; image shift -z*angle (lentil/plane.py:884-923).  As in
    lentil, the tilt about x moves the image in y and vice versa."""

    def __init__(self, x, y, **kwargs):
        super().__init__(**kwargs)
        self.x = y
        self.y = x

    def __shift__(self, xs=0, ys=0, z=0, **kwargs):
        return xs - z * self.x, ys - z * self.y


_GL_NODES, _GL_WEIGHTS = np.polynomial.legendre.leggauss(32)


class DispersiveTilt(_TiltBase):
    """Spectral dispersion as a wavelength-dependent image shift
    (lentil/plane.py:926-1097).

    The light of wavelength ``lam`` lands at distance ``d`` along the
    spectral trace, with ``lam = polyval(dispersion, d)``, at the trace
    point ``(x, polyval(trace, x))`` whose arc length from ``x = 0`` is
    ``d``; the shift adds that point to the incoming one.  Both polynomials
    are in decreasing powers, lengths in meters on the focal plane.

    First-order polynomials are solved in closed form, with lentil's
    arithmetic.  For higher orders ``d`` is the real root of
    ``polyval(dispersion, d) - lam`` nearest zero (companion-matrix roots
    polished by Newton steps) and ``x`` inverts the arc length
    ``s(x) = integral_0^x sqrt(1 + trace'(t)^2) dt`` by Newton's method over
    32-point Gauss-Legendre quadrature.  (lentil reaches the same points by
    least squares from 0; under numpy 2 its higher-order trace raises a
    TypeError there.)"""

    def __init__(self, trace=None, dispersion=None, **kwargs):
        super().__init__(**kwargs)
        if trace is not None:
            self.trace = np.asarray(trace)
        if dispersion is not None:
            self.dispersion = np.asarray(dispersion)

    def __shift__(self, wavelength, xs=0., ys=0., **kwargs):
        trace = np.asarray(self.trace, dtype=float)
        x = self._trace_x(trace, self._distance(np.asarray(self.dispersion, dtype=float),
                                                float(wavelength)))
        return x + xs, np.polyval(trace, x) + ys

    @staticmethod
    def _distance(disp, lam):
        if disp.size == 2:
            return (lam - disp[1]) / disp[0]
        if disp.size < 2:
            raise ValueError('dispersion needs order >= 1')
        c = disp.copy()
        c[-1] -= lam
        r = np.roots(c)
        r = r[np.abs(r.imag) <= 1e-9 * np.maximum(np.abs(r), 1e-300)].real
        if r.size == 0:
            raise ValueError(f'no distance along the trace has wavelength {lam}')
        d = r[np.argmin(np.abs(r))]
        dc = np.polyder(c)
        for _ in range(3):
            g = np.polyval(dc, d)
            if g == 0:
                break
            d = d - np.polyval(c, d) / g
        return float(d)

    @staticmethod
    def _trace_x(trace, d):
        if trace.size == 2:
            return d / np.sqrt(1 + trace[0] ** 2)
        slope = np.polyder(trace) if trace.size > 1 else np.zeros(1)

        def speed(t):
            return np.sqrt(1.0 + np.polyval(slope, t) ** 2)

        def arc(x):
            h = 0.5 * x
            return h * np.dot(_GL_WEIGHTS, speed(h * (_GL_NODES + 1.0)))

        x = d / speed(0.0)
        for _ in range(60):
            step = (arc(x) - d) / speed(x)
            x -= step
            if abs(step) <= 4e-16 * max(abs(x), 1e-300):
                break
        return float(x)


class Grism(DispersiveTilt):
    """Deprecated alias of :class:`DispersiveTilt` (lentil/plane.py:1099-1169)."""

    def __init__(self, trace, dispersion, **kwargs):
        import warnings
        warnings.warn('lentil.Grism will be deprecated in v1.0.0, it is replaced by '
                      'lentil.DispersiveTilt.', DeprecationWarning, stacklevel=2)
        super().__init__(trace=trace, dispersion=dispersion, **kwargs)
