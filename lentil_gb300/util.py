"""Host-side array helpers with lentil's conventions (lentil/util.py,
lentil/helper.py).  Pure numpy; they prepare inputs and window geometry and
never touch the GPU."""
import numpy as np


def mesh(shape, shift=(0, 0), angle=0):
    """Centred (row, col) coordinate grids, optionally rotated by ``angle``
    degrees (lentil/helper.py:7-17)."""
    nr, nc = int(shape[0]), int(shape[1])
    r = (np.arange(nr) - np.floor(nr / 2.0) - shift[0])[:, None] * np.ones((1, nc))
    c = np.ones((nr, 1)) * (np.arange(nc) - np.floor(nc / 2.0) - shift[1])[None, :]
    a = np.deg2rad(angle)
    ca, sa = np.cos(a), np.sin(a)
    return r * ca + c * sa, c * ca - r * sa


def boundary(x, threshold=0):
    """(rmin, rmax, cmin, cmax) of the entries above ``threshold``
    (lentil/util.py:190-218)."""
    x = np.asarray(x) > threshold
    rows = np.flatnonzero(x.any(axis=1))
    cols = np.flatnonzero(x.any(axis=0))
    return rows[0], rows[-1], cols[0], cols[-1]


def boundary_slice(x, threshold=0, pad=(0, 0)):
    """Bounding box of ``x > threshold`` as a slice pair
    (lentil/helper.py:27-62)."""
    pad = np.broadcast_to(np.asarray(pad), (2,))
    rmin, rmax, cmin, cmax = boundary(x, threshold)
    return np.s_[max(rmin - pad[0], 0):min(rmax + pad[0] + 1, x.shape[0]),
                 max(cmin - pad[1], 0):min(cmax + pad[1] + 1, x.shape[1])]


def slice_offset(slc, shape):
    """Offset of a slice's centre from the centre of ``shape``
    (lentil/helper.py:65-123)."""
    if slc is Ellipsis or slc == Ellipsis:
        return (0, 0)
    if Ellipsis in slc:
        if slice(None, None, None) in slc:
            return (0, 0)
        raise ValueError(f"Can't compute offset from slice {slc}")
    off = []
    for ax in (0, 1):
        n = slc[ax].stop - slc[ax].start
        off.append(int(slc[ax].start + n // 2 - int(shape[ax]) // 2))
    return (0, 0) if off == [0, 0] else tuple(off)


def centroid(img):
    """Intensity centroid in (row, col) (lentil/util.py:6-28)."""
    img = np.asarray(img, dtype=float)
    img = img / img.sum()
    return (float(np.sum(img.sum(axis=1) * np.arange(img.shape[0]))),
            float(np.sum(img.sum(axis=0) * np.arange(img.shape[1]))))


def normalize_power(array, power=1):
    """Scale so that sum |array|^2 == power (lentil/util.py:378-411)."""
    array = np.asarray(array)
    return array * np.sqrt(power / np.sum(np.abs(array) ** 2))


def pad(array, shape):
    """Centred zero-pad or crop of a 2-D array (lentil/util.py:31-90)."""
    array = np.asarray(array)
    out = np.zeros((int(shape[0]), int(shape[1])), dtype=array.dtype)
    src, dst = [], []
    for ax in (0, 1):
        a, s = array.shape[ax], int(shape[ax])
        lo = abs(s - a) // 2
        if s <= a:
            src.append(slice(lo, lo + s)); dst.append(slice(0, s))
        else:
            src.append(slice(0, a)); dst.append(slice(lo, lo + a))
    out[dst[0], dst[1]] = array[src[0], src[1]]
    return out
