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
import json
import os

import numpy as np

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


def _device_tag():
    import torch
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return {'name': p.name, 'sm_count': int(p.multi_processor_count)}


def save(path):
    """Write the decided launch classes to a JSON cache file (atomically)."""
    lib = _lib.load()
    n = lib.lgb_tuner_export(None, 0)
    rows = np.zeros((max(n, 1), 9), dtype=np.int32)
    n = min(n, lib.lgb_tuner_export(rows.ctypes.data, rows.shape[0]))
    doc = {'version': 1, 'device': _device_tag(), 'classes': rows[:n].tolist()}
    tmp = f'{path}.tmp{os.getpid()}'
    with open(tmp, 'w') as fh:
        json.dump(doc, fh)
    os.replace(tmp, path)
    return n


def load(path):
    """Add the classes of a cache file written by ``save`` on the same kind of
    GPU (same name and SM count: the classes are counted in waves over its
    CTA pairs); returns how many were loaded (0 for a missing, foreign or
    unreadable file)."""
    try:
        with open(path) as fh:
            doc = json.load(fh)
    except (OSError, ValueError):
        return 0
    if doc.get('version') != 1 or doc.get('device') != _device_tag():
        return 0
    rows = np.asarray(doc.get('classes', []), dtype=np.int32).reshape(-1, 9)
    rows = np.ascontiguousarray(rows)
    _lib.call('lgb_tuner_import', rows.ctypes.data, rows.shape[0])
    return int(rows.shape[0])
