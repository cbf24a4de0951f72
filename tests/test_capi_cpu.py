"""C ABI checks that need no GPU: the library builds, loads and exports every
symbol include/lentil_gb300.h declares; host-side validation errors map to
lentil's exception types."""
import ctypes
import os
import re

import numpy as np
import pytest

from lentil_gb300 import _build, _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'include',
                      'lentil_gb300.h')


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(lgb_[a-z0-9_]+)\s*\(', text)))


@pytest.fixture(scope='module')
def lib():
    return _lib.load()


def test_header_declares_entry_points():
    names = header_functions()
    assert 'lgb_dft2' in names and 'lgb_psf_execute' in names and 'lgb_phasor' in names


def test_library_exports_every_header_symbol(lib):
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header():
    assert set(header_functions()) == set(_lib.SIGNATURES)


def test_version_and_error_string(lib):
    assert lib.lgb_version() >> 16 == 1
    assert isinstance(lib.lgb_last_error(), bytes)


def test_invalid_sizes_raise_valueerror(lib):
    # rejected by host-side validation before any CUDA call
    st = lib.lgb_dft2(None, 0, 4, None, 4, 4, 0.1, 0.1, 0, 0, 0, 0, 1, 0, None, 0, None)
    assert st == _lib.EINVAL
    with pytest.raises(ValueError):
        _lib.check(st)
    assert b'positive' in lib.lgb_last_error()


def test_unknown_precision_rejected(lib):
    with pytest.raises(ValueError):
        _lib.precision_code('fp8')
    assert lib.lgb_dft2_workspace_size(0, 1, 1, 1, 0) == 0


def test_workspace_sizes_are_consistent(lib):
    a = lib.lgb_dft2_workspace_size(100, 90, 128, 120, _lib.FP64)
    assert a >= 16 * (128 * 100 + 90 * 120)
    b = lib.lgb_dft2_workspace_size(100, 90, 128, 120, _lib.SPLIT_BF16)
    assert b > 0
    assert lib.lgb_idft2_workspace_size(100, 90, 128, 120, 0) >= a + 16 * 100 * 90


@pytest.mark.parametrize('n,os_', [(2048, 3), (1000, 3), (64, 5), (75, 2), (5, 2)])
def test_pixel_workspace_covers_off_grid_buffers(lib, n, os_):
    # the size query must count every buffer the off-grid pixelate carves:
    # the MTF product (two N x N planes on the FFT path, three real planes on
    # the GEMM path), the banded operator, both resampling passes
    S = lib.lgb_pixelate_size(n, os_)
    assert S == int(np.ceil(n * (1 / os_)))
    fft = n >= 2 and n & (n - 1) == 0
    need = 2 * 8 * n * n if fft else 3 * 8 * n * n
    need += 8 * (64 * S + n * S + S * S) + 4 * S
    assert lib.lgb_pixel_workspace_size(n, os_) >= need
    assert lib.lgb_pixelate_size(0, 2) == -1 and lib.lgb_pixelate_size(10, 0) == -1


def test_tuner_controls_without_a_gpu(lib):
    # mode / forced width / cache controls touch no device
    assert lib.lgb_tuner_set_mode(0) == _lib.OK and lib.lgb_tuner_set_mode(1) == _lib.OK
    assert lib.lgb_tuner_set_mode(7) == _lib.EINVAL
    assert lib.lgb_tuner_force_tile(128) == _lib.OK and lib.lgb_tuner_force_tile(0) == _lib.OK
    assert lib.lgb_tuner_force_tile(96) == _lib.EINVAL
    lib.lgb_tuner_clear()
    assert lib.lgb_tuner_entries() == 0
    assert lib.lgb_tuner_lookup(64, 64, 64, 64, 1, _lib.SPLIT_BF16, 0) == 0
    assert lib.lgb_tuner_last_tile() == 0


def test_dft2_plan_argument_errors_without_a_gpu(lib):
    # invalid geometries are rejected before any device call
    h = ctypes.c_void_p()
    assert lib.lgb_dft2_plan_create(0, 4, 4, 4, .1, .1, 0, 0, 0, 0, 1, 0, None,
                                    ctypes.byref(h)) == _lib.EINVAL
    assert lib.lgb_dft2_plan_create(4, 4, 4, 4, .1, .1, 0, 0, 0, 0, 1, 9, None,
                                    ctypes.byref(h)) == _lib.EINVAL
    assert not h.value
    assert lib.lgb_dft2_plan_bytes(None) == 0 and lib.lgb_dft2_plan_workspace_size(None, 1) == 0
    assert lib.lgb_dft2_plan_destroy(None) == _lib.OK
    assert lib.lgb_dft2_plan_execute(None, None, 1, None, None, 0, None) == _lib.EINVAL


def test_build_is_up_to_date():
    assert _build.up_to_date()


def test_no_cpu_fallback():
    # without a CUDA device every entry of the path raises instead of
    # computing on the host (this container has no GPU)
    import torch
    if torch.cuda.is_available():
        pytest.skip('a CUDA device is present')
    import lentil_gb300 as lg
    f = np.ones((8, 8), dtype=complex)
    for call in (lambda: lg.fourier.dft2(f, 0.1),
                 lambda: lg.fourier.dft2_batch(f[None], 0.1, precision='split-bf16'),
                 lambda: lg.detector.pixelate(np.ones((8, 8)), 2),
                 lambda: lg.zernike_compose(np.ones((8, 8)), [0, 1e-8])):
        with pytest.raises(RuntimeError, match='CUDA device'):
            call()


def test_psf_plan_size_rejects_a_bad_description(lib):
    # lgb_psf_plan_size returns 0 for an invalid description and records the
    # reason, which the Python plan raises as ValueError (no device needed)
    lam = np.array([6e-7]); ar = np.array([1e-3]); sh = np.zeros(1)
    d = _lib.PsfDesc()
    d.H = d.W = 64
    d.r0 = d.c0 = 0
    d.m, d.n = 80, 64                          # field slice taller than the pupil plane
    d.M = d.N = d.out_rows = d.out_cols = 32
    d.n_wavelengths = 1
    d.wavelengths, d.alpha_r, d.alpha_c = lam.ctypes.data, ar.ctypes.data, ar.ctypes.data
    d.shift_r = d.shift_c = sh.ctypes.data
    d.batch, d.precision = 1, _lib.SPLIT_BF16
    assert lib.lgb_psf_plan_size(ctypes.byref(d)) == 0
    assert b'field slice outside the pupil plane' in lib.lgb_last_error()
    with pytest.raises(ValueError, match='field slice'):
        _lib.check(_lib.EINVAL)
    d.m = 64                                   # valid: a positive size
    assert lib.lgb_psf_plan_size(ctypes.byref(d)) > 0
