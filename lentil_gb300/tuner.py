"""Tile-shape autotuner of the split-precision (tensor-core) MFT.

Every split launch runs its CTA-pair tiles 256 or 128 output columns wide:
256 feeds each shared-memory A tile into twice the MMA work and wins on large
transforms; 128 makes twice the tiles, which wins when a launch is too small
to occupy every CTA pair.  The library picks the width per launch class
(precision, field m x n, window M x N, epilogue, and the occupancy the
problem count gives) and caches it for the process.  In ``'measure'`` mode
(the default) a class is tuned online on real launches: the first runs the
occupancy model's width, the second the other, both timed with CUDA events,
and a later launch keeps the faster -- no relaunch, no host wait.  In
``'model'`` mode the occupancy model decides.  See ``lgb_tuner_*`` in
include/lentil_gb300.h.
"""
import contextlib

from . import _lib

MODES = {'model': 0, 'measure': 1}
EPILOGUES = {'intensity': 0, 'complex': 1}


def set_mode(mode):
    """'measure' (time both widths on first use of a shape) or 'model'."""
    if mode not in MODES:
        raise ValueError(f'unknown tuner mode {mode!r}; expected one of {sorted(MODES)}')
    _lib.call('lgb_tuner_set_mode', MODES[mode])


def force_tile(tile=0):
    """Run every split launch with this tile width (256 or 128); 0 restores tuning."""
    _lib.call('lgb_tuner_force_tile', int(tile))


@contextlib.contextmanager
def forced(tile):
    """Context manager: ``force_tile(tile)`` inside the block."""
    force_tile(tile)
    try:
        yield
    finally:
        force_tile(0)


def clear():
    """Forget every cached choice."""
    _lib.load().lgb_tuner_clear()


def entries():
    """Number of launch classes with a decided width."""
    return _lib.load().lgb_tuner_entries()


def lookup(m, n, M, N, count, precision='split', epilogue='intensity'):
    """Decided width of the class of a launch (count = PSFs x wavelengths), or 0."""
    return _lib.load().lgb_tuner_lookup(int(m), int(n), int(M), int(N), int(count),
                                        _lib.precision_code(precision), EPILOGUES[epilogue])


def last_tile():
    """Width used by this thread's last split launch (0 before any)."""
    return _lib.load().lgb_tuner_last_tile()
