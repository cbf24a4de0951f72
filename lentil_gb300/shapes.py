"""Aperture generators (host-side numpy, input preparation only).

Same names, arguments and pixel conventions as lentil's ``lentil/shape.py``
and ``lentil/segmented.py``; they build the pupils the diffraction path
consumes and are not on the GPU path themselves.
"""
import numpy as np

from .util import mesh


def circle(shape, radius, shift=(0, 0), antialias=True):
    """Disk of ``radius`` px; edge antialiased by a one-pixel linear ramp
    (lentil/shape.py:6-30)."""
    rr, cc = mesh(shape)
    dist = np.hypot(rr - shift[0], cc - shift[1])
    out = np.clip(radius + 0.5 - dist, 0.0, 1.0)
    if not antialias:
        out[out > 0] = 1
    return out


def hexagon(shape, radius, shift=(0, 0), rotate=False, antialias=True):
    """Regular hexagon, circumradius ``radius`` px, as the intersection of six
    half-planes (lentil/shape.py:33-75)."""
    shape = np.broadcast_to(shape, (2,))
    r, c = mesh(shape, shift)
    apothem = radius * np.sqrt(3) / 2
    out = np.ones(shape)
    for k in range(6):
        ang = k * np.pi / 3 + (0.0 if rotate else np.pi / 6)
        d = r * np.sin(ang) + c * np.cos(ang)
        if antialias:
            edge = np.clip(apothem + 0.5 - d, 0.0, 1.0)
        else:
            edge = (d <= apothem).astype(float)
        out = np.minimum(out, edge)
    return out


def rectangle(shape, width, height, shift=(0, 0), angle=0, antialias=True):
    """Rotated rectangle (lentil/shape.py:78-114)."""
    shape = np.broadcast_to(shape, (2,))
    rr, cc = mesh(shape, shift, angle)
    out = np.minimum(np.clip(0.5 + width / 2 - np.abs(cc), 0, 1),
                     np.clip(0.5 + height / 2 - np.abs(rr), 0, 1))
    out = np.minimum(np.ones(shape), out)
    if not antialias:
        out[out > 0] = 1
    return out


def spider(shape, width, angle=0, shift=(0, 0), antialias=True):
    """Half-line vane of ``width`` px leaving the centre at ``angle`` degrees
    (lentil/shape.py:117-145)."""
    shape = np.broadcast_to(shape, (2,))
    length = np.sqrt(2) * np.max(shape) / 2
    a = np.deg2rad(angle)
    centre = (shift[0] - length / 2 * np.sin(a), shift[1] + length / 2 * np.cos(a))
    return 1 - rectangle(shape, length, width, centre, angle, antialias)


# axial hex-grid directions, walked in this order around each ring
_HEX_STEPS = ((1, 0), (1, -1), (0, -1), (-1, 0), (-1, 1), (0, 1))


def _ring(k):
    """Axial (q, r) cells of hex ring ``k`` in walk order (start at (-k, k))."""
    q, r = -k, k
    cells = []
    for dq, dr in _HEX_STEPS:
        for _ in range(k):
            cells.append((q, r))
            q, r = q + dq, r + dr
    return cells


def hex_segments(rings, seg_radius, seg_gap, rotate=False, antialias=True,
                 flatten=False, pad=2, drop=(0,)):
    """Cube of hexagonal segment masks (lentil/segmented.py:8-80).

    Segment 0 is the centre, then rings outward; ``drop`` removes segments
    by that index (the default drops the centre)."""
    apothem = seg_radius * np.sqrt(3) / 2
    size = int(np.ceil((rings * 2 + 1) * apothem * 2 + rings * 2 * seg_gap + pad * 2))
    shape = (size, size)
    pitch = seg_radius + seg_gap / 2
    out = []
    if 0 not in drop:
        out.append(hexagon(shape, seg_radius, shift=(0, 0), antialias=antialias, rotate=rotate))
    idx = 1
    for k in range(1, rings + 1):
        for q, r in _ring(k):
            if rotate:
                x = pitch * (np.sqrt(3) * q + np.sqrt(3) / 2 * r)
                y = pitch * 1.5 * r
            else:
                x = pitch * 1.5 * q
                y = pitch * (np.sqrt(3) / 2 * q + np.sqrt(3) * r)
            if idx not in drop:
                out.append(hexagon(shape, seg_radius, shift=(-y, x), antialias=antialias,
                                   rotate=rotate))
            idx += 1
    out = np.asarray(out)
    return np.sum(out, axis=0) if flatten else out
