"""Plane-type tags (lentil/ptype.py:1-50): same names, equality and errors."""

PTYPES = ('none', 'pupil', 'image', 'tilt', 'transform')


class PType:
    __slots__ = ('_key',)

    def __init__(self, key):
        if key not in PTYPES:
            raise TypeError(f"plane type '{key}' not understood")
        self._key = key

    def __eq__(self, other):
        return isinstance(other, PType) and self._key == other._key

    def __hash__(self):
        return hash(self._key)

    def __repr__(self):
        return f"ptype('{self._key}')"

    def __str__(self):
        return self._key


def ptype(value):
    """Coerce None / str / PType to a PType."""
    if value is None:
        value = 'none'
    return value if isinstance(value, PType) else PType(value)


none = ptype('none')
pupil = ptype('pupil')
image = ptype('image')
tilt = ptype('tilt')
transform = ptype('transform')
