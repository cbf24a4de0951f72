"""Integer window algebra (rmin, rmax, cmin, cmax), inclusive bounds, with
lentil's centring convention (lentil/extent.py:5-169).  Host-side: these
decide which output pixels a propagation computes and where a Field lands;
the pixels themselves are produced on the GPU."""


def array_extent(shape, shift, parent_shape=None):
    """Extent of a ``shape`` array whose centre (index shape//2) sits at
    ``shift`` (lentil/extent.py:5-40)."""
    if len(shape) < 2:
        shape = (1, 1)
    # truncation toward zero of (shift - shape//2), as lentil does for
    # non-integer shifts
    r0 = int(shift[0] - int(shape[0]) // 2)
    c0 = int(shift[1] - int(shape[1]) // 2)
    ext = (r0, r0 + int(shape[0]) - 1, c0, c0 + int(shape[1]) - 1)
    if parent_shape is not None:
        pr, pc = int(parent_shape[0]) // 2, int(parent_shape[1]) // 2
        ext = (ext[0] + pr, ext[1] + pr, ext[2] + pc, ext[3] + pc)
    return ext


def array_center(extent):
    """Index of the centre pixel (lentil/extent.py:43-59)."""
    r0, r1, c0, c1 = extent
    return r0 + (r1 - r0 + 1) // 2, c0 + (c1 - c0 + 1) // 2


def intersect(a, b):
    """True when two extents overlap (lentil/extent.py:62-77)."""
    return a[0] <= b[1] and b[0] <= a[1] and a[2] <= b[3] and b[2] <= a[3]


def intersection_extent(a, b):
    """lentil/extent.py:80-99."""
    return max(a[0], b[0]), min(a[1], b[1]), max(a[2], b[2]), min(a[3], b[3])


def intersection_shape(a, b):
    """Shape of the overlap, () when empty (lentil/extent.py:102-124)."""
    r0, r1, c0, c1 = intersection_extent(a, b)
    nr, nc = r1 - r0 + 1, c1 - c0 + 1
    return (nr, nc) if nr > 0 and nc > 0 else ()


def intersection_slices(a, b):
    """Slices of the overlap inside ``a`` and inside ``b``
    (lentil/extent.py:127-150)."""
    r0, r1, c0, c1 = intersection_extent(a, b)
    return ((slice(r0 - a[0], r1 - a[0] + 1), slice(c0 - a[2], c1 - a[2] + 1)),
            (slice(r0 - b[0], r1 - b[0] + 1), slice(c0 - b[2], c1 - b[2] + 1)))


def intersection_shift(a, b):
    """Centre of the overlap (lentil/extent.py:153-168)."""
    return array_center(intersection_extent(a, b))
