"""numpy restatement of lentil 0.8.8's far-field MFT path (the oracle).

TEST INFRASTRUCTURE ONLY: used by tests, the smoke check and the CPU
baseline legs of bench.py.  Never imported by ``lentil_gb300``.

Parity: pinned against golden vectors generated by lentil 0.8.8 itself
(``tests/golden/make_golden.py`` -> ``tests/golden/*.npz``), checked by
``tests/test_oracle_golden.py``.

All citations are paths inside the lentil project.
"""
from __future__ import annotations

import copy
import functools
import itertools
from math import factorial

import numpy as np

# --------------------------------------------------------------------------
# plane types (lentil/ptype.py:1-50)
# --------------------------------------------------------------------------
NONE, PUPIL, IMAGE, TILT, TRANSFORM = 'none', 'pupil', 'image', 'tilt', 'transform'


def _ptype(p):
    p = 'none' if p is None else p
    if p not in (NONE, PUPIL, IMAGE, TILT, TRANSFORM):
        raise TypeError(f"plane type '{p}' not understood")
    return p


# --------------------------------------------------------------------------
# fourier (lentil/fourier.py)
# --------------------------------------------------------------------------
@functools.lru_cache(maxsize=32)
def _coords(m, n, M, N):
    """Centred index vectors, lentil/fourier.py:113-121."""
    return (np.arange(m) - np.floor(m / 2.0), np.arange(n) - np.floor(n / 2.0),
            np.arange(M) - np.floor(M / 2.0), np.arange(N) - np.floor(N / 2.0))


def dft2_matrices(m, n, M, N, ar, ac, sr, sc, orow, ocol):
    """E1 (M x m), E2 (n x N); lentil/fourier.py:106-110."""
    R, S, U, V = _coords(m, n, M, N)
    E1 = np.exp(-2.0 * 1j * np.pi * ar * np.outer(R + orow, U - sr)).T
    E2 = np.exp(-2.0 * 1j * np.pi * ac * np.outer(S + ocol, V - sc))
    return E1, E2


def dft2(f, alpha, shape=None, shift=(0, 0), offset=(0, 0), unitary=True, out=None):
    """Matrix triple product E1 . f . E2; lentil/fourier.py:5-103."""
    ar, ac = np.broadcast_to(alpha, (2,))
    f = np.asarray(f)
    m, n = f.shape
    M, N = np.broadcast_to([m, n] if shape is None else shape, (2,))
    sr, sc = np.broadcast_to(shift, (2,))
    orow, ocol = np.broadcast_to(offset, (2,))
    if out is not None and not np.can_cast(complex, out.dtype):
        raise TypeError(f"Cannot cast complex output to dtype('{out.dtype}')")
    E1, E2 = dft2_matrices(m, n, M, N, ar, ac, sr, sc, orow, ocol)
    F = np.dot(E1.dot(f), E2, out=out)
    if unitary:
        np.multiply(F, np.sqrt(np.abs(ar * ac)), out=F)
    return F


def idft2(F, alpha, shape=None, shift=(0, 0), unitary=True, out=None):
    """conj(dft2(conj(F)))/F.size; lentil/fourier.py:124-198."""
    F = np.asarray(F)
    size = F.size
    f = dft2(np.conj(F), alpha, shape, shift, unitary=unitary, out=out)
    np.conj(f, out=f)
    return np.divide(f, size, out=f)


# --------------------------------------------------------------------------
# extent algebra (lentil/extent.py)
# --------------------------------------------------------------------------
def array_extent(shape, shift, parent_shape=None):
    """lentil/extent.py:5-40."""
    if len(shape) < 2:
        shape = (1, 1)
    rmin = int(-(shape[0] // 2) + shift[0])
    cmin = int(-(shape[1] // 2) + shift[1])
    rmax = int(rmin + shape[0] - 1)
    cmax = int(cmin + shape[1] - 1)
    if parent_shape is not None:
        pc = np.asarray(parent_shape) // 2
        rmin, rmax, cmin, cmax = rmin + pc[0], rmax + pc[0], cmin + pc[1], cmax + pc[1]
    return rmin, rmax, cmin, cmax


def array_center(extent):
    """lentil/extent.py:43-59."""
    rmin, rmax, cmin, cmax = extent
    return rmin + (rmax - rmin + 1) // 2, cmin + (cmax - cmin + 1) // 2


def intersect(a, b):
    """lentil/extent.py:62-77."""
    return a[0] <= b[1] and a[1] >= b[0] and a[2] <= b[3] and a[3] >= b[2]


def intersection_extent(a, b):
    """lentil/extent.py:80-99."""
    return max(a[0], b[0]), min(a[1], b[1]), max(a[2], b[2]), min(a[3], b[3])


def intersection_shape(a, b):
    """lentil/extent.py:102-124."""
    rmin, rmax, cmin, cmax = intersection_extent(a, b)
    nr, nc = rmax - rmin + 1, cmax - cmin + 1
    return () if (nr <= 0 or nc <= 0) else (nr, nc)


def intersection_slices(a, b):
    """lentil/extent.py:127-150."""
    rmin, rmax, cmin, cmax = intersection_extent(a, b)
    return ((slice(rmin - a[0], rmax - a[0] + 1), slice(cmin - a[2], cmax - a[2] + 1)),
            (slice(rmin - b[0], rmax - b[0] + 1), slice(cmin - b[2], cmax - b[2] + 1)))


def intersection_shift(a, b):
    """lentil/extent.py:153-168."""
    return array_center(intersection_extent(a, b))


# --------------------------------------------------------------------------
# helpers (lentil/helper.py, lentil/util.py)
# --------------------------------------------------------------------------
def mesh(shape, shift=(0, 0), angle=0):
    """lentil/helper.py:7-17."""
    nr, nc = shape[0], shape[1]
    rr, cc = np.meshgrid(np.arange(nr) - np.floor(nr / 2.0) - shift[0],
                         np.arange(nc) - np.floor(nc / 2.0) - shift[1], indexing='ij')
    a = np.deg2rad(angle)
    return rr * np.cos(a) + cc * np.sin(a), rr * -np.sin(a) + cc * np.cos(a)


def boundary(x, threshold=0):
    """lentil/util.py:190-218."""
    x = np.asarray(x) > threshold
    rows = np.where(np.any(x, axis=1))[0]
    cols = np.where(np.any(x, axis=0))[0]
    return rows[0], rows[-1], cols[0], cols[-1]


def boundary_slice(x, threshold=0, pad=(0, 0)):
    """lentil/helper.py:27-62."""
    pad = np.asarray(pad)
    if pad.shape == ():
        pad = np.append(pad, pad)
    rmin, rmax, cmin, cmax = boundary(x, threshold)
    rmin = np.max((rmin - pad[0], 0))
    rmax = np.min((rmax + pad[0] + 1, x.shape[0]))
    cmin = np.max((cmin - pad[1], 0))
    cmax = np.min((cmax + pad[1] + 1, x.shape[1]))
    return np.s_[rmin:rmax, cmin:cmax]


def slice_offset(slc, shape):
    """lentil/helper.py:65-123."""
    if slc == Ellipsis:
        return (0, 0)
    if Ellipsis in slc:
        if slice(None, None, None) in slc:
            return (0, 0)
        raise ValueError(f"Can't compute offset from slice {slc}")
    ss = np.array((slc[0].stop - slc[0].start, slc[1].stop - slc[1].start))
    off = np.array((slc[0].start + ss[0] // 2, slc[1].start + ss[1] // 2)) - np.asarray(shape) // 2
    return (0, 0) if np.all(off == 0) else tuple(off)


def centroid(img):
    """lentil/util.py:6-28."""
    img = np.asarray(img)
    img = img / np.sum(img)
    nr, nc = img.shape
    rr, cc = np.mgrid[0:nr, 0:nc]
    return np.dot(rr.ravel(), img.ravel()), np.dot(cc.ravel(), img.ravel())


def normalize_power(array, power=1):
    """lentil/util.py:378-411."""
    array = np.asarray(array)
    return array * np.sqrt(power / np.sum(np.abs(array) ** 2))


def pad(array, shape):
    """Centre zero-pad / crop of a 2-D array; lentil/util.py:31-90."""
    array = np.asarray(array)
    out = np.zeros((shape[0], shape[1]), dtype=array.dtype)
    src, dst = [], []
    for ax in (0, 1):
        a, s = array.shape[ax], shape[ax]
        if s - a <= 0:
            lo = (a - s) // 2
            src.append(slice(lo, lo + s)); dst.append(slice(0, s))
        else:
            lo = (s - a) // 2
            src.append(slice(0, a)); dst.append(slice(lo, lo + a))
    out[dst[0], dst[1]] = array[src[0], src[1]]
    return out


def rescale(img, scale, shape=None, mask=None, order=3, mode='nearest', unitary=True):
    """Spline resampling; lentil/util.py:261-349."""
    from scipy.ndimage import map_coordinates
    img = np.asarray(img)
    if mask is None:
        mask = np.zeros_like(img).real
        mask[img != 0] = 1
    if shape is None:
        shape = np.ceil((img.shape[0] * scale, img.shape[1] * scale)).astype(int)
    elif np.isscalar(shape):
        shape = np.ceil((shape * scale, shape * scale)).astype(int)
    else:
        shape = np.ceil((shape[0] * scale, shape[1] * scale)).astype(int)
    x = (np.arange(shape[1], dtype=np.float64) - shape[1] / 2.) / scale + img.shape[1] / 2.
    y = (np.arange(shape[0], dtype=np.float64) - shape[0] / 2.) / scale + img.shape[0] / 2.
    xx, yy = np.meshgrid(x, y)
    mask = map_coordinates(mask, [yy, xx], order=1, mode='nearest')
    mask[mask < np.finfo(mask.dtype).eps] = 0
    out = map_coordinates(img, [yy, xx], order=order, mode=mode)
    if unitary:
        out *= np.sum(img) / np.sum(out)
    out *= mask
    return out


# --------------------------------------------------------------------------
# Field (lentil/field.py)
# --------------------------------------------------------------------------
class Field:
    """Sparse complex tile with integer offset and tilt list; lentil/field.py:7-194."""
    __slots__ = ('data', 'offset', 'tilt', 'pixelscale', 'extent')

    def __init__(self, data, pixelscale=None, offset=None, tilt=None):
        self.data = np.asarray(data, dtype=complex)
        self.pixelscale = pixelscale
        self.offset = offset if offset is not None else [0, 0]
        self.tilt = tilt if tilt else []
        self.extent = array_extent(self.shape, self.offset)

    @property
    def shape(self):
        return self.data.shape

    @property
    def size(self):
        return self.data.size

    def __mul__(self, other):
        """lentil/field.py:80-147."""
        tilt = self.tilt + other.tilt
        if self.size == 1 and other.size == 1:
            if np.array_equal(self.offset, other.offset):
                data, offset = self.data * other.data, self.offset
            else:
                data, offset = [], None
        else:
            a, ao, b, bo = self.data, self.offset, other.data, other.offset
            if a.shape != b.shape:              # lentil/field.py:464-484
                if a.size == 1:
                    a, ao = np.broadcast_to(a, b.shape), bo
                if b.size == 1:
                    b, bo = np.broadcast_to(b, a.shape), ao
            ea, eb = array_extent(a.shape, ao), array_extent(b.shape, bo)
            if intersect(ea, eb):
                sa, sb = intersection_slices(ea, eb)
                data, offset = a[sa] * b[sb], intersection_shift(ea, eb)
            else:
                data, offset = [], None
        return Field(data=data, offset=offset, tilt=tilt)

    def shift(self, z, wavelength, pixelscale, oversample, indexing='ij'):
        """Tilt -> output pixel shift; lentil/field.py:149-194."""
        if indexing not in ('xy', 'ij'):
            raise ValueError("Valid values for `indexing` are 'xy' and 'ij'")
        if pixelscale is None:
            raise ValueError('pixelscale must be defined to compute shift')
        x, y = 0, 0
        for t in self.tilt:
            x, y = t.__shift__(xs=x, ys=y, z=z, wavelength=wavelength)
        ps = np.broadcast_to(pixelscale, (2,))
        out = x / ps[0] * oversample, y / ps[1] * oversample
        if indexing == 'ij':
            out = -out[1], out[0]
        return out


def field_boundary(fields):
    """lentil/field.py:196-229."""
    import sys
    rmin, rmax, cmin, cmax = sys.maxsize, 0, sys.maxsize, 0
    for f in fields:
        a, b, c, d = f.extent
        rmin, rmax, cmin, cmax = min(rmin, a), max(rmax, b), min(cmin, c), max(cmax, d)
    return rmin, rmax, cmin, cmax


def insert(field, out, intensity=False, weight=1):
    """Clipped overlap-add of a Field into an array; lentil/field.py:231-305."""
    if field.shape == out.shape and np.array_equal(field.offset, [0, 0]):
        fs = os_ = Ellipsis
    else:
        osh, fsh, fo = np.asarray(out.shape), np.asarray(field.shape), np.asarray(field.offset)
        ul = (osh // 2) - (fsh // 2) + fo
        fr0, fr1, fc0, fc1 = 0, int(fsh[0]), 0, int(fsh[1])
        or0, or1 = int(ul[0]), int(ul[0] + fsh[0])
        oc0, oc1 = int(ul[1]), int(ul[1] + fsh[1])
        if or0 < 0:
            fr0, or0 = -or0, 0
        if or1 > osh[0]:
            fr1 -= or1 - osh[0]; or1 = osh[0]
        if oc0 < 0:
            fc0, oc0 = -oc0, 0
        if oc1 > osh[1]:
            fc1 -= oc1 - osh[1]; oc1 = osh[1]
        os_ = slice(or0, or1), slice(oc0, oc1)
        fs = slice(fr0, fr1), slice(fc0, fc1)
    if intensity:
        out[os_] += np.abs(field.data[fs] ** 2) * weight
    else:
        out[os_] += field.data[fs] * weight
    return out


def _merge(fields):
    """lentil/field.py:331-386."""
    if not np.all([f.pixelscale == fields[0].pixelscale for f in fields]):
        raise ValueError("Can't merge: pixelscales must be equal")
    rmin, rmax, cmin, cmax = field_boundary(fields)
    if rmin == 0 and rmax == 0 and cmin == 0 and cmax == 0:
        out = np.zeros((), dtype=complex)
        slices = [Ellipsis]
    else:
        out = np.zeros((rmax - rmin + 1, cmax - cmin + 1), dtype=complex)
        slices = [(slice(f.extent[0] - rmin, f.extent[1] - rmin + 1),
                   slice(f.extent[2] - cmin, f.extent[3] - cmin + 1)) for f in fields]
    for f, s in zip(fields, slices):
        out[s] += f.data
    nrow, ncol = rmax - rmin + 1, cmax - cmin + 1
    return Field(data=out, pixelscale=fields[0].pixelscale,
                 offset=(rmin + nrow // 2, cmin + ncol // 2))


def merge(a, b, enforce_overlap=True):
    """lentil/field.py:308-327."""
    if enforce_overlap and not intersect(a.extent, b.extent):
        raise ValueError("Can't merge non-overlapping fields")
    return _merge((a, b))


def _disjoint(groups):
    """lentil/field.py:451-461 (iterative form of the same pairwise scan)."""
    while True:
        for m, n in itertools.combinations(range(len(groups)), 2):
            if intersect(groups[m]['extent'], groups[n]['extent']):
                groups[m]['field'].extend(groups[n]['field'])
                groups[m]['extent'] = field_boundary(groups[m]['field'])
                groups.pop(n)
                break
        else:
            return groups


def reduce(fields):
    """lentil/field.py:413-448."""
    groups = _disjoint([{'field': [f], 'extent': f.extent} for f in fields])
    return [_merge(g['field']) if len(g['field']) > 1 else g['field'][0] for g in groups]


# --------------------------------------------------------------------------
# Wavefront (lentil/wavefront.py)
# --------------------------------------------------------------------------
class Wavefront:
    """lentil/wavefront.py:12-165."""

    def __init__(self, wavelength, pixelscale=None, diameter=None, focal_length=None,
                 tilt=None, ptype=None):
        self.focal_length = focal_length if focal_length else None
        self.diameter = diameter
        self.shape = ()
        self.wavelength = wavelength
        self.pixelscale = None if pixelscale is None else np.broadcast_to(pixelscale, (2,))
        p = _ptype(ptype)
        if p not in (NONE, PUPIL, IMAGE):
            raise TypeError(f"invalid ptype '{p}' for Wavefront")
        self.ptype = p
        if tilt is not None:
            if len(tilt) != 2:
                raise ValueError('tilt must be specified as [rx, ry]')
            tilt = [Tilt(x=tilt[0], y=tilt[1])]
        self.data = [Field(data=np.array(1, dtype=complex), offset=None, tilt=tilt)]

    def __mul__(self, plane):
        return plane.__mul__(self)

    @classmethod
    def empty(cls, wavelength, pixelscale=None, diameter=None, focal_length=None,
              tilt=None, shape=None, ptype=None):
        w = cls(wavelength=wavelength, pixelscale=pixelscale, diameter=diameter,
                focal_length=focal_length, tilt=tilt, ptype=ptype)
        w.data = []
        w.shape = () if shape is None else shape
        return w

    @property
    def field(self):
        out = np.zeros(self.shape, dtype=complex)
        for f in self.data:
            out = insert(f, out)
        return out

    @property
    def intensity(self):
        out = np.zeros(self.shape, dtype=float)
        for f in reduce(self.data):
            out = insert(f, out, intensity=True)
        return out

    def insert(self, out, weight=1):
        for f in reduce(self.data):
            out = insert(f, out, intensity=True, weight=weight)
        return out


# --------------------------------------------------------------------------
# Planes (lentil/plane.py)
# --------------------------------------------------------------------------
_MUL_PTYPE = {                                         # lentil/plane.py:634-652
    NONE: {NONE: NONE, PUPIL: PUPIL, IMAGE: IMAGE, TILT: NONE, TRANSFORM: NONE},
    PUPIL: {PUPIL: PUPIL, TILT: PUPIL, TRANSFORM: PUPIL},
    IMAGE: {IMAGE: IMAGE, TILT: PUPIL, TRANSFORM: PUPIL},
}


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


class Plane:
    """lentil/plane.py:19-611 (the parts on the diffraction path)."""
    default_ptype = NONE

    def __init__(self, amplitude=None, opd=None, mask=None, pixelscale=None,
                 diameter=None, ptype=None, **kwargs):
        if 'amp' in kwargs:
            if amplitude is not None:
                raise AttributeError("Got both 'amplitude' and 'amp'")
            amplitude = kwargs['amp']
        self.amplitude = np.asarray(1 if amplitude is None else amplitude)
        self.opd = np.asarray(0 if opd is None else opd)
        self._mask = None if mask is None else np.asarray(mask)
        self.pixelscale = None if pixelscale is None else np.broadcast_to(pixelscale, (2,))
        self._diameter = diameter
        self.ptype = _ptype(ptype if ptype is not None else self.default_ptype)
        self.tilt = []

    @property
    def mask(self):
        """lentil/plane.py:43-47."""
        return np.copy(self.amplitude).astype(bool) if self._mask is None else self._mask

    @property
    def size(self):
        return 1 if self.mask.ndim in (0, 1, 2) else self.mask.shape[0]

    @property
    def shape(self):
        return self.mask.shape if self.size == 1 else self.mask.shape[1:]

    @property
    def diameter(self):
        """lentil/plane.py:147-171."""
        if self._diameter is not None:
            return self._diameter
        gm = self.mask if self.size < 2 else np.sum(self.mask, axis=0)
        rmin, rmax, cmin, cmax = boundary(gm)
        return np.max(np.max((rmax - rmin, cmax - cmin)) * np.asarray(self.pixelscale))

    def _slices(self):
        """lentil/plane.py:671-705."""
        mask = self.mask
        if mask is None or mask.ndim < 2:
            return [Ellipsis]
        if mask.ndim == 2:
            return [boundary_slice(mask)]
        return [boundary_slice(m) for m in mask]

    def __mul__(self, wavefront):
        """Phasor construction amp*exp(2*pi*i*opd/lambda); lentil/plane.py:477-516."""
        if self.ptype not in _MUL_PTYPE[wavefront.ptype]:
            raise TypeError(f"can't multiply Wavefront with ptype '{wavefront.ptype}' "
                            f"by Plane with ptype '{self.ptype}'")
        pixelscale = _mul_pixelscale(self.pixelscale, wavefront.pixelscale)
        shape = wavefront.shape if self.shape == () else self.shape
        out = Wavefront.empty(wavelength=wavefront.wavelength, pixelscale=pixelscale,
                              focal_length=wavefront.focal_length, shape=shape,
                              ptype=_MUL_PTYPE[wavefront.ptype][self.ptype])
        for field in wavefront.data:
            for n, s in enumerate(self._slices()):
                mask = self.mask if self.size == 1 else self.mask[n]
                amp = self.amplitude if self.amplitude.size == 1 else self.amplitude[s] * mask[s]
                opd = self.opd if self.opd.size == 1 else self.opd[s]
                phasor = Field(data=amp * np.exp(2 * np.pi * 1j * opd / wavefront.wavelength),
                               pixelscale=self.pixelscale,
                               offset=slice_offset(s, self.shape),
                               tilt=[self.tilt[n]] if self.tilt else [])
                res = field * phasor
                if res.size > 0:
                    out.data.append(res)
        return out

    def ptt_vector(self):
        """lentil/plane.py:522-562."""
        if self.shape == () or self.shape is None:
            return None
        if self.pixelscale is None:
            raise ValueError("can't create ptt_vector with pixelscale = ()")
        ps = np.broadcast_to(self.pixelscale, (2,))
        r, c = mesh(self.shape)
        unmasked = np.einsum('ij,i->ij', [np.ones(r.size), r.ravel(), -c.ravel()], [1, ps[0], ps[1]])
        if self.size == 1:
            return np.einsum('ij,j->ij', unmasked, self.mask.ravel())
        v = np.empty((self.size * 3, int(np.prod(self.shape))))
        for k in range(self.size):
            v[3 * k:3 * k + 3] = unmasked * self.mask[k].ravel()
        return v

    def fit_tilt(self, inplace=False):
        """Least-squares tilt removal into Tilt objects; lentil/plane.py:564-611."""
        plane = self if inplace else copy.deepcopy(self)
        v = plane.ptt_vector()
        if v is None or plane.opd.size == 1:
            return plane
        if self.size == 1:
            t = np.linalg.lstsq(v.T, plane.opd.ravel(), rcond=None)[0]
            plane.opd = plane.opd - np.einsum('ij,i->j', v[1:3], t[1:3]).reshape(plane.opd.shape)
            plane.tilt.append(Tilt(x=t[1], y=t[2]))
        else:
            t = np.empty((self.size, 3))
            parts = np.empty((self.size,) + plane.opd.shape)
            for k in range(self.size):
                t[k] = np.linalg.lstsq(v[3 * k:3 * k + 3].T, plane.opd.ravel(), rcond=None)[0]
                seg = np.einsum('ij,i->j', v[3 * k + 1:3 * k + 3], t[k, 1:3])
                parts[k] = (plane.opd - seg.reshape(plane.opd.shape)) * self.mask[k]
            plane.opd = np.sum(parts, axis=0)
            plane.tilt.extend([Tilt(x=t[k, 1], y=t[k, 2]) for k in range(self.size)])
        return plane


class Pupil(Plane):
    """lentil/plane.py:708-771."""
    default_ptype = PUPIL

    def __init__(self, amplitude=None, opd=None, mask=None, pixelscale=None,
                 focal_length=None, diameter=None, **kwargs):
        super().__init__(amplitude=amplitude, opd=opd, mask=mask, pixelscale=pixelscale,
                         diameter=diameter, ptype=PUPIL, **kwargs)
        self.focal_length = focal_length

    def __mul__(self, wavefront):
        w = super().__mul__(wavefront)
        w.focal_length = self.focal_length
        return w


class Image(Plane):
    """lentil/plane.py:774-820."""
    default_ptype = IMAGE

    def __init__(self, amplitude=None, opd=None, mask=None, pixelscale=None, **kwargs):
        super().__init__(amplitude=amplitude, opd=opd, mask=mask, pixelscale=pixelscale,
                         ptype=IMAGE, **kwargs)

    def __mul__(self, wavefront):
        w = super().__mul__(wavefront)
        w.ptype = IMAGE
        return w


class Tilt:
    """Angular tilt (x/y swapped at construction); lentil/plane.py:884-923."""

    def __init__(self, x, y):
        self.x = y
        self.y = x

    def __shift__(self, xs=0, ys=0, z=0, **kwargs):
        return xs - z * self.x, ys - z * self.y


# --------------------------------------------------------------------------
# propagation (lentil/propagate.py)
# --------------------------------------------------------------------------
def _dft_alpha(dx, du, wavelength, z, oversample):
    """lentil/propagate.py:121-123."""
    return ((dx[0] * du[0]) / (wavelength * z * oversample),
            (dx[1] * du[1]) / (wavelength * z * oversample))


def _mask_shape(x, threshold=0):
    """lentil/propagate.py:245-248."""
    rmin, rmax, cmin, cmax = boundary(x, threshold)
    return rmax - rmin + 1, cmax - cmin + 1


def _mask_shift(x, threshold=0):
    """lentil/propagate.py:251-260."""
    rcf, ccf = x.shape[0] // 2, x.shape[1] // 2
    rmin, rmax, cmin, cmax = boundary(x, threshold)
    sh = (rmax - rmin + 1, cmax - cmin + 1)
    return rmin + sh[0] // 2 - rcf, cmin + sh[1] // 2 - ccf


def _propagate_ptype(ptype):
    """lentil/propagate.py:263-272."""
    if ptype not in (PUPIL, IMAGE):
        raise TypeError("Wavefront must have ptype 'pupil' or 'image'")
    return IMAGE if ptype == PUPIL else PUPIL


def propagate_plan(wavefront, pixelscale, shape=None, prop_shape=None, oversample=2, mask=None):
    """Host-side window maths of propagate_dft, lentil/propagate.py:147-242.

    Returns (ptype_out, shape_out, du, list of per-field jobs) where a job is
    (field, alpha, intersect_shape, shift, intersect_shift)."""
    ptype_out = _propagate_ptype(wavefront.ptype)
    shape = np.asarray(wavefront.shape) if shape is None else np.broadcast_to(shape, (2,))
    prop_shape = np.asarray(shape) if prop_shape is None else np.broadcast_to(prop_shape, (2,))
    shape_out = shape * oversample
    prop_shape_out = prop_shape * oversample
    if mask is not None:
        mask = np.asarray(mask)
        if np.all(mask.shape != shape_out):
            raise ValueError(f'shape mismatch: mask shape {mask.shape} != output shape {tuple(shape_out)}')
        out_extent = array_extent(_mask_shape(mask), _mask_shift(mask))
    else:
        out_extent = array_extent(shape_out, shift=(0, 0))
    dx = wavefront.pixelscale
    du = np.broadcast_to(pixelscale, (2,))
    z = wavefront.focal_length
    jobs = []
    for field in wavefront.data:
        shift = field.shift(z=z, wavelength=wavefront.wavelength, pixelscale=du,
                            oversample=oversample, indexing='ij')
        fix = np.trunc(shift)
        subpx = np.asarray(shift) - fix
        prop_extent = array_extent(prop_shape_out, fix)
        if intersect(out_extent, prop_extent):
            ishape = intersection_shape(out_extent, prop_extent)
            ishift = intersection_shift(out_extent, prop_extent)
            iext = array_extent(ishape, ishift)
            pshift = np.array(array_center(prop_extent)) - np.array(array_center(iext))
            alpha = _dft_alpha(dx, du, wavefront.wavelength, z, oversample)
            jobs.append((field, alpha, ishape, pshift + subpx, ishift))
    return ptype_out, shape_out, du, jobs


def propagate_dft(wavefront, pixelscale, shape=None, prop_shape=None, oversample=2, mask=None):
    """lentil/propagate.py:147-242."""
    ptype_out, shape_out, du, jobs = propagate_plan(wavefront, pixelscale, shape, prop_shape,
                                                    oversample, mask)
    out = Wavefront.empty(wavelength=wavefront.wavelength, pixelscale=du / oversample,
                          focal_length=wavefront.focal_length, shape=shape_out, ptype=ptype_out)
    for field, alpha, ishape, shift, ishift in jobs:
        data = dft2(field.data, alpha, shape=ishape, shift=shift, offset=field.offset, unitary=True)
        out.data.append(Field(data=data, pixelscale=du / oversample, offset=ishift))
    return out


def _fft_shape(dx, du, z, wavelength, oversample):
    """Padded FFT shape and the propagation wavelength it implies;
    lentil/propagate.py:126-132 (``_dft_alpha`` is symmetric in wavelength
    and z, so lentil's swapped argument order is harmless)."""
    alpha = _dft_alpha(dx, du, z, wavelength, oversample)
    fft_shape = np.round(np.reciprocal(alpha)).astype(int)
    prop_wavelength = np.min((fft_shape / oversample * dx * du) / z)
    return fft_shape, prop_wavelength


def _fft2c(x):
    """Centred ortho FFT; lentil/propagate.py:135-136."""
    return np.fft.ifftshift(np.fft.fft2(np.fft.fftshift(x), norm='ortho'))


def _has_tilt(wavefront):
    """lentil/propagate.py:139-144."""
    return any(f.tilt for f in wavefront.data)


def scratch_shape(wavelength, dx, du, z, oversample):
    """lentil/propagate.py:91-118."""
    dx = np.broadcast_to(dx, (2,))
    du = np.broadcast_to(du, (2,))
    fft_shape, _ = _fft_shape(dx, du, z, np.max(wavelength), oversample)
    return tuple(fft_shape)


def propagate_fft(wavefront, pixelscale, shape=None, oversample=2, scratch=None):
    """Far-field propagation by a zero-padded centred FFT;
    lentil/propagate.py:9-88."""
    if _has_tilt(wavefront):
        raise NotImplementedError('propagate_fft does not support Wavefronts with fitted tilt. '
                                  'Use propagate_dft instead.')
    ptype_out = _propagate_ptype(wavefront.ptype)
    pixelscale = np.broadcast_to(pixelscale, (2,))
    fft_shape, prop_wavelength = _fft_shape(wavefront.pixelscale, pixelscale,
                                            wavefront.focal_length, wavefront.wavelength,
                                            oversample)
    if shape is None:
        shape_out = tuple(fft_shape)
    else:
        shape = tuple(np.broadcast_to(shape, (2,)))
        if np.any(shape > fft_shape / oversample):
            raise ValueError(f'requested shape {tuple(shape)} is larger in at least one '
                             f'dimension than maximum propagation shape '
                             f'{tuple(fft_shape // oversample)}')
        shape_out = (shape[0] * oversample, shape[1] * oversample)
    out = Wavefront.empty(wavelength=prop_wavelength, pixelscale=pixelscale / oversample,
                          focal_length=wavefront.focal_length, shape=shape_out, ptype=ptype_out)
    if scratch is not None:
        if not all(np.asarray(scratch.shape) > fft_shape):
            raise ValueError(f'scratch must have shape greater than or equal to {tuple(fft_shape)}')
        view = scratch[0:fft_shape[0], 0:fft_shape[1]]
        view[...] = 0
        for f in wavefront.data:
            view[...] = insert(f, view)
        field = _fft2c(view)
    else:
        field = _fft2c(pad(wavefront.field, fft_shape))
    out.data.append(Field(data=field, pixelscale=pixelscale / oversample))
    return out


def broadband_psf(pupil, wavelengths, weights, pixelscale, shape=None, prop_shape=None,
                  oversample=2, mask=None, out=None):
    """The documented user broadband loop (docs/user/performance.rst:44-49):
    for each wavelength, Wavefront(lam) * pupil -> propagate_dft -> insert(out, w)."""
    for lam, w in zip(wavelengths, weights):
        wf = propagate_dft(Wavefront(lam) * pupil, pixelscale, shape=shape,
                           prop_shape=prop_shape, oversample=oversample, mask=mask)
        if out is None:
            out = np.zeros(wf.shape, dtype=float)
        out = wf.insert(out, weight=w)
    return out


# --------------------------------------------------------------------------
# detector (lentil/detector.py)
# --------------------------------------------------------------------------
def pixel(img, oversample=1):
    """Sinc pixel MTF by FFT convolution; lentil/detector.py:167-222."""
    img = np.asarray(img)
    mx = np.sinc(np.fft.fftfreq(img.shape[1]) * oversample)
    my = np.sinc(np.fft.fftfreq(img.shape[0]) * oversample)
    kernel = np.dot(mx[:, np.newaxis], my[np.newaxis, :])
    return np.abs(np.fft.ifft2(np.fft.fft2(img) * kernel))


def pixelate(img, oversample):
    """lentil/detector.py:225-251."""
    return rescale(pixel(img, oversample), 1 / oversample, order=3, mode='nearest', unitary=True)


# The cubic-spline resampling of rescale (scipy.ndimage.map_coordinates,
# order=3, mode='nearest', at lentil's points, lentil/util.py:323-340)
# restated as one banded linear operator per axis, the form the library's
# off-grid pixelate evaluates.  scipy pads the input with RS_PAD edge copies,
# prefilters with a half-sample-symmetric boundary and sums four cubic
# B-spline coefficients around x + RS_PAD; the prefilter is the convolution
# with sqrt(3) z^|t| (z = sqrt(3) - 2; Unser, Aldroubi & Eden 1993),
# truncated here at |t| <= RS_TAPS.  Checked against scipy in the tests.
RS_PAD, RS_TAPS = 12, 30
RS_BW = 2 * RS_TAPS + 4


def _reflect_half(r, L):
    r = np.mod(r, 2 * L)
    return np.where(r >= L, 2 * L - 1 - r, r)


def _beta3(t):
    t = np.abs(t)
    return np.where(t < 1, 2 / 3 - t * t + t ** 3 / 2, np.where(t < 2, (2 - t) ** 3 / 6, 0.0))


def resample_operator(n, oversample):
    """(S, x, q0, G): output sample k = sum_b G[k, b] s[q0[k] + b] for a
    length-n signal s resampled at lentil's points x."""
    S = int(np.ceil(n * (1 / oversample)))
    x = (np.arange(S, dtype=np.float64) - S / 2.) / (1 / oversample) + n / 2.
    Np = n + 2 * RS_PAD
    xp = x + RS_PAD
    i0 = np.floor(xp).astype(np.int64) - 1
    q0 = np.clip(i0 - RS_TAPS - RS_PAD, 0, max(0, n - RS_BW))
    t = np.arange(-RS_TAPS, RS_TAPS + 1)
    z = np.sqrt(3) - 2
    h = np.sqrt(3) * z ** np.abs(t)
    G = np.zeros((S, RS_BW))
    for k in range(S):
        for j in range(i0[k], i0[k] + 4):
            q = np.clip(_reflect_half(_reflect_half(j, Np) - t, Np) - RS_PAD, 0, n - 1) - q0[k]
            if q.min() < 0 or q.max() >= RS_BW:
                raise AssertionError('resample window too narrow')
            np.add.at(G[k], q, _beta3(xp[k] - j) * h)
    return S, x, q0, G


def pixelate_banded(img, oversample):
    """pixelate with the resampling evaluated as G . p . G^T."""
    p = pixel(img, oversample)
    n = p.shape[0]
    S, x, q0, G = resample_operator(n, oversample)
    nb = min(RS_BW, n)
    T = np.stack([p[:, q0[l]:q0[l] + nb] @ G[l, :nb] for l in range(S)], axis=1)
    raw = np.stack([G[k, :nb] @ T[q0[k]:q0[k] + nb, :] for k in range(S)], axis=0)
    from scipy.ndimage import map_coordinates
    xx, yy = np.meshgrid(x, x)
    mask = map_coordinates((p != 0).astype(float), [yy, xx], order=1, mode='nearest')
    mask[mask < np.finfo(float).eps] = 0
    return raw * (np.sum(p) / np.sum(raw)) * mask


# --------------------------------------------------------------------------
# input generators (lentil/zernike.py, lentil/wfe.py)
# --------------------------------------------------------------------------
def noll_to_nm(j):
    """lentil/zernike.py:348-391 (row of the triangle, then the position in it)."""
    if j < 1:
        raise ValueError('Noll index must be greater than zero')
    n = int(np.ceil((-1 + np.sqrt(1 + 8 * j)) / 2) - 1)
    if n == 0:
        return 0, 0
    r = int(j - (n + 1) * (n + 2) / 2 - 1)
    row = [1, 1] if n & 1 else [0]
    for _ in range(n // 2):
        row.append(row[-1] + 2)
        row.append(row[-1])
    return int(n), int(row[r] * (-1 if j & 1 else 1))


def ansi_to_nm(j):
    """lentil/zernike.py:394-415."""
    if j < 0:
        raise ValueError('ANSI index must be zero or larger')
    n = np.floor((np.sqrt(8 * j + 1) - 1) / 2)
    return int(n), int(2 * j - n * (n + 2))


def fringe_to_nm(j):
    """lentil/zernike.py:418-441."""
    if j < 1:
        raise ValueError('Fringe index must be greater than zero')
    m_n = 2 * (np.ceil(np.sqrt(j)) - 1)
    g_s = (m_n / 2) ** 2 + 1
    n = m_n / 2 + np.floor((j - g_s) / 2)
    return int(n), int((m_n - n) * (1 - np.mod(j - g_s, 2) * 2))


def zernike_radial(n, m, rho):
    """lentil/zernike.py:96-109."""
    m, n = abs(int(m)), abs(int(n))
    if (n - m) & 1:
        return 0
    out = np.zeros(rho.shape)
    for k in range((n - m) // 2 + 1):
        rk = ((-1) ** k * factorial(n - k) /
              (factorial(k) * factorial((n + m) // 2 - k) * factorial((n - m) // 2 - k)))
        out += rk * rho ** (n - 2 * k)
    return out


def zernike_coordinates(mask, shift=None, rotate=0):
    """lentil/zernike.py:444-480."""
    mask = np.asarray(mask, dtype=bool)
    if shift is None:
        center = np.asarray(mask.shape) / 2
        cen = centroid(mask)
        shift = (cen[0] - center[0], cen[1] - center[1])
    rr, cc = mesh(mask.shape, shift)
    r = np.abs(rr + 1j * cc)
    rho = r / np.max(r * mask)
    angle = (90 - rotate) * np.pi / 180
    theta = np.angle(-rr * np.exp(1j * angle) + 1j * cc * np.exp(1j * angle))
    return rho, theta


def zernike(mask, index, normalize=True, order='noll', rho=None, theta=None):
    """lentil/zernike.py:11-93."""
    mask = np.asarray(mask, dtype=bool)
    n, m = {'noll': noll_to_nm, 'fringe': fringe_to_nm, 'ansi': ansi_to_nm}[order](index)
    if rho is None:
        rho, theta = zernike_coordinates(mask)
    elif theta is None:
        raise ValueError('Both rho and theta must be specified')
    if m == 0:
        if n == 0:
            return mask
        return (np.sqrt(n + 1) if normalize else 1) * zernike_radial(n, m, rho) * mask
    ang = np.cos(m * theta) if m > 0 else np.sin(m * theta)
    if normalize:
        return np.sqrt(2) * np.sqrt(n + 1) * zernike_radial(n, m, rho) * ang * mask
    return zernike_radial(n, m, rho) * ang * mask


def zernike_compose(mask, coeffs, normalize=True, order='noll', rho=None, theta=None):
    """lentil/zernike.py:112-180."""
    mask = np.asarray(mask)
    opd = np.zeros(mask.shape)
    for index, coeff in np.ndenumerate(np.asarray(coeffs)):
        opd += coeff * zernike(mask, index[0] + 1, normalize, order, rho, theta)
    return opd


def zernike_basis(mask, modes, vectorize=False, normalize=True, order='noll', rho=None,
                  theta=None):
    """lentil/zernike.py:183-234."""
    modes = np.asarray(modes)
    if modes.shape == ():
        modes = modes[..., np.newaxis]
    mask = np.asarray(mask)
    basis = np.zeros(modes.shape + mask.shape)
    for index, mode in np.ndenumerate(modes):
        basis[index] = zernike(mask, mode, normalize, order, rho, theta)
    return basis.reshape(basis.shape[0], -1) if vectorize else basis


def power_spectrum(mask, pixelscale, rms, half_power_freq, exp, seed=None):
    """lentil/wfe.py:8-70 (Sidick 2009 PSD filter of seeded white noise)."""
    mask = np.asarray(mask)
    rng = np.random.default_rng(seed)
    n, m = mask.shape
    yy, xx = np.mgrid[0:m, 0:n]
    yy = (yy - (np.floor(m / 2) + 1)) / m
    xx = (xx - (np.floor(n / 2) + 1)) / n
    dr = np.sqrt(xx * xx + yy * yy)
    half_power_freq = half_power_freq * pixelscale / np.sqrt(m ** 2 + n ** 2)
    psd = 1 / (1 + (dr / half_power_freq) ** exp)
    psd[dr == 0] = 0
    psd = psd / np.sum(psd)
    H = np.fft.fftshift(np.sqrt(psd))
    noise = rng.normal(size=[n, m])
    opd = np.real(np.fft.ifft2(np.fft.fft2(noise) * H)) * np.sqrt(m * n)
    opd *= mask
    return opd * np.sqrt(np.count_nonzero(opd) / np.sum(np.abs(opd) ** 2)) * rms


# --------------------------------------------------------------------------
# error metric used throughout the parity tests
# --------------------------------------------------------------------------
def peak_normalised_error(test, ref):
    """max|test - ref| / max|ref|."""
    test = np.asarray(test)
    ref = np.asarray(ref)
    den = np.max(np.abs(ref))
    return float(np.max(np.abs(test - ref)) / (den if den > 0 else 1.0))
