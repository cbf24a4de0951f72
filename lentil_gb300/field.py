"""Sparse complex fields on the GPU, drop-in for ``lentil.field``.

A Field is a device complex128 tile plus lentil's integer ``offset`` of its
centre from the plane centre and a ``tilt`` list (lentil/field.py:7-194).
Extents, windows and merge bookkeeping stay on the host (integer algebra);
the pixels are multiplied, overlap-added and squared by library kernels.
"""
import sys

import numpy as np
import torch

from . import _device as dv
from . import _lib
from . import extent as ext


class Field:
    """Two-dimensional sampled complex field (lentil/field.py:7-78)."""
    __slots__ = ('data', 'offset', 'tilt', 'pixelscale', 'extent')

    def __init__(self, data, pixelscale=None, offset=None, tilt=None):
        if isinstance(data, (list, tuple)) and len(data) == 0:
            data = np.zeros((0,), dtype=complex)
        self.data = dv.to_device(data, torch.complex128)
        self.pixelscale = pixelscale
        self.offset = offset if offset is not None else [0, 0]
        self.tilt = tilt if tilt else []
        self.extent = ext.array_extent(self.shape, self.offset)

    @property
    def shape(self):
        return tuple(self.data.shape)

    @property
    def size(self):
        return int(self.data.numel())

    def __mul__(self, other):
        """Intersection product with lentil's broadcast rules
        (lentil/field.py:80-147, 464-484)."""
        tilt = self.tilt + other.tilt
        if self.size == 1 and other.size == 1:
            if np.array_equal(self.offset, other.offset):
                data = _multiply(self.data.reshape(1, 1), (0, 0), other.data.reshape(1, 1), (0, 0), (1, 1))
                return Field(data=data.reshape(self.data.shape if self.data.dim() >= other.data.dim()
                                               else other.data.shape),
                             offset=self.offset, tilt=tilt)
            return Field(data=[], offset=None, tilt=tilt)
        a, ao, b, bo = self.data, self.offset, other.data, other.offset
        a_shape, b_shape = tuple(a.shape), tuple(b.shape)
        if a_shape != b_shape:
            if a.numel() == 1:
                a_shape, ao = b_shape, bo
            if b.numel() == 1:
                b_shape, bo = a_shape, ao
        ea, eb = ext.array_extent(a_shape, ao), ext.array_extent(b_shape, bo)
        if not ext.intersect(ea, eb):
            return Field(data=[], offset=None, tilt=tilt)
        sa, sb = ext.intersection_slices(ea, eb)
        om, on = sa[0].stop - sa[0].start, sa[1].stop - sa[1].start
        data = _multiply(a if a.numel() > 1 else a.reshape(1, 1), (sa[0].start, sa[1].start),
                         b if b.numel() > 1 else b.reshape(1, 1), (sb[0].start, sb[1].start),
                         (om, on))
        return Field(data=data, offset=ext.intersection_shift(ea, eb), tilt=tilt)

    def shift(self, z, wavelength, pixelscale, oversample, indexing='ij'):
        """Output-pixel shift of the field from its tilts
        (lentil/field.py:149-194)."""
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


def _multiply(a, a0, b, b0, oshape):
    """out = a[a0 + window] * b[b0 + window]; size-1 operands broadcast."""
    om, on = oshape
    out = torch.empty((om, on), dtype=torch.complex128, device=a.device)
    lda = 0 if a.numel() == 1 else a.shape[1]
    ldb = 0 if b.numel() == 1 else b.shape[1]
    _lib.call('lgb_field_multiply', a.data_ptr(), lda, a0[0], a0[1], b.data_ptr(), ldb, b0[0], b0[1],
              out.data_ptr(), om, on, dv.stream_ptr())
    return out


def boundary(fields):
    """Bounding extent of several fields (lentil/field.py:196-229)."""
    rmin, rmax, cmin, cmax = sys.maxsize, 0, sys.maxsize, 0
    for f in fields:
        a, b, c, d = f.extent
        rmin, rmax, cmin, cmax = min(rmin, a), max(rmax, b), min(cmin, c), max(cmax, d)
    return rmin, rmax, cmin, cmax


def _as2d(t):
    return t.reshape(1, 1) if t.dim() < 2 else t


def insert(field, out, intensity=False, weight=1):
    """Clipped overlap-add of ``field`` into ``out`` (lentil/field.py:231-305).

    ``out`` is a CUDA tensor (updated in place) or a numpy array (updated in
    place through one round trip); with ``intensity`` the added quantity is
    ``|field|^2 * weight``."""
    host = not dv.is_tensor(out)
    od = dv.to_device(out, torch.float64 if intensity else torch.complex128) if host else out
    if not host:
        want = torch.float64 if intensity else torch.complex128
        if od.dtype != want or not od.is_contiguous():
            raise TypeError(f'insert needs a contiguous {want} tensor for out')
    if field.size > 0 and od.numel() > 0:
        f2, o2 = _as2d(field.data), _as2d(od)
        off = (0, 0) if field.data.dim() == 0 and od.dim() == 0 else field.offset
        _lib.call('lgb_field_insert', f2.data_ptr(), f2.shape[0], f2.shape[1], int(off[0]),
                  int(off[1]), o2.data_ptr(), o2.shape[0], o2.shape[1], float(weight),
                  int(bool(intensity)), dv.stream_ptr())
    if host:
        out[...] = dv.to_host(od)
        return out
    return od


def _merge(fields):
    """Union of fields as one field (lentil/field.py:331-386)."""
    if not np.all([np.array_equal(f.pixelscale, fields[0].pixelscale) for f in fields]):
        raise ValueError("Can't merge: pixelscales must be equal")
    rmin, rmax, cmin, cmax = boundary(fields)
    dev = fields[0].data.device
    if rmin == 0 and rmax == 0 and cmin == 0 and cmax == 0:
        out = torch.zeros((), dtype=torch.complex128, device=dev)
        for f in fields:
            insert(Field(f.data.reshape(()) if f.size == 1 else f.data), out)
        return Field(data=out, pixelscale=fields[0].pixelscale, offset=(0, 0))
    nr, nc = rmax - rmin + 1, cmax - cmin + 1
    out = torch.zeros((nr, nc), dtype=torch.complex128, device=dev)
    off = (rmin + nr // 2, cmin + nc // 2)
    for f in fields:
        # placing f at its own offset inside the union reproduces the union
        # slices of lentil/field.py:361-376
        g = Field.__new__(Field)
        g.data, g.offset, g.tilt, g.pixelscale = f.data, (f.offset[0] - off[0], f.offset[1] - off[1]), [], None
        g.extent = f.extent
        insert(g, out)
    return Field(data=out, pixelscale=fields[0].pixelscale, offset=off)


def merge(a, b, enforce_overlap=True):
    """lentil/field.py:308-327."""
    if enforce_overlap and not overlap((a, b)):
        raise ValueError("Can't merge non-overlapping fields")
    return _merge((a, b))


def _disjoint(groups):
    """Pairwise merge of overlapping groups until disjoint (lentil/field.py:451-461)."""
    merged = True
    while merged:
        merged = False
        for i in range(len(groups)):
            for j in range(i + 1, len(groups)):
                if ext.intersect(groups[i]['extent'], groups[j]['extent']):
                    groups[i]['field'].extend(groups[j]['field'])
                    groups[i]['extent'] = boundary(groups[i]['field'])
                    groups.pop(j)
                    merged = True
                    break
            if merged:
                break
    return groups


def overlap(fields):
    """lentil/field.py:389-410."""
    if len(fields) == 2:
        return ext.intersect(fields[0].extent, fields[1].extent)
    return len(_disjoint([{'field': [f], 'extent': f.extent} for f in fields])) <= 1


def reduce(fields):
    """Disjoint set of coherently merged fields (lentil/field.py:413-448)."""
    groups = _disjoint([{'field': [f], 'extent': f.extent} for f in fields])
    return [_merge(g['field']) if len(g['field']) > 1 else g['field'][0] for g in groups]
