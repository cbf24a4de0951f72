"""Pin the numpy oracle to lentil 0.8.8's own outputs (golden vectors)."""
import numpy as np
import pytest

from oracle import lentil_oracle as lo
from tests.golden_cases import (FFT_CASES, PROPAGATE_CASES, build_pupil, fft_case, fft_field_crop,
                                propagate_kwargs)


def test_dft2_cases(golden):
    g = golden('dft2')
    for name in g['names']:
        F = lo.dft2(g[f'{name}_f'], g[f'{name}_alpha'], shape=tuple(g[f'{name}_shape']),
                    shift=g[f'{name}_shift'], offset=g[f'{name}_offset'],
                    unitary=bool(g[f'{name}_unitary']))
        assert lo.peak_normalised_error(F, g[f'{name}_F']) < 1e-13, name


def test_dft2_shift_and_offset(golden):
    g = golden('dft2')
    n = 100
    F = lo.dft2(np.ones((n, n)), 1 / n, shift=g['shift100_shift'])
    assert lo.peak_normalised_error(F, g['shift100_F']) < 1e-13
    c = np.asarray(lo.centroid(np.abs(F) ** 2)) - n // 2
    assert np.allclose(c, g['shift100_shift'], atol=1e-9)
    f = g['offset_f']
    r0, r1, c0, c1 = g['offset_slice']
    FF = lo.dft2(f[r0:r1, c0:c1], alpha=1 / 3, shape=10, offset=g['offset_offset'])
    assert lo.peak_normalised_error(FF, g['offset_F']) < 1e-13


def test_idft2(golden):
    g = golden('dft2')
    for name, n in (('ieven', 10), ('iodd', 11)):
        f = lo.idft2(g[f'{name}_F'], 1 / n, unitary=False)
        assert lo.peak_normalised_error(f, g[f'{name}_f']) < 1e-13


@pytest.mark.parametrize('name', PROPAGATE_CASES)
def test_propagate_cases(golden, name):
    g = golden('propagate')
    pl = build_pupil(lo, g, name)
    w = lo.propagate_dft(lo.Wavefront(float(g[f'{name}_wavelength'])) * pl,
                         **propagate_kwargs(g, name))
    assert len(w.data) == int(g[f'{name}_nfields'])
    ref = g[f'{name}_intensity']
    I = w.intensity
    assert I.shape == ref.shape
    if np.max(ref) == 0:
        assert np.all(I == 0)
    else:
        assert lo.peak_normalised_error(I, ref) < 1e-12


def test_broadband_insert(golden):
    g = golden('propagate')
    pl = lo.Pupil(amplitude=g['bb_amp'], opd=g['bb_opd'], pixelscale=g['bb_pixelscale_in'].tolist(),
                  focal_length=10)
    img = lo.broadband_psf(pl, g['bb_wl'], g['bb_wt'], 6e-6, shape=24, oversample=2)
    assert lo.peak_normalised_error(img, g['bb_img']) < 1e-12


def test_field_merge_reduce_insert(golden):
    g = golden('field')
    a = lo.Field(np.ones((5, 4)), pixelscale=1, offset=[-2, -2])
    b = lo.Field(np.ones((3, 3)), pixelscale=1, offset=[0, -1])
    c = lo.merge(a, b)
    assert np.array_equal(c.data, g['merge_data'])
    assert np.array_equal(c.offset, g['merge_offset'])
    fs = [lo.Field(g[f'reduce_in{k}_data'], pixelscale=1, offset=list(g[f'reduce_in{k}_offset']))
          for k in range(4)]
    red = lo.reduce(fs)
    assert len(red) == int(g['reduce_n'])
    for k, f in enumerate(red):
        assert np.array_equal(f.data, g[f'reduce_out{k}_data'])
        assert np.array_equal(f.offset, g[f'reduce_out{k}_offset'])
    out = np.zeros((9, 8))
    for f in fs:
        out = lo.insert(f, out, intensity=True, weight=0.7)
    assert np.allclose(out, g['insert_intensity'], rtol=1e-14, atol=0)
    out = np.zeros((9, 8), dtype=complex)
    for f in fs:
        out = lo.insert(f, out)
    assert np.array_equal(out, g['insert_complex'])


PIXELATE_CASES = ['px64os2', 'px90os3', 'px128os4',                     # grid samples
                  'px100os3', 'px75os2', 'px61os7', 'px128os3', 'px64os5']  # off grid


@pytest.mark.parametrize('name', PIXELATE_CASES)
def test_pixelate(golden, name):
    g = golden('detector')
    img, os_ = g[f'{name}_img'], int(g[f'{name}_os'])
    assert lo.peak_normalised_error(lo.pixel(img, os_), g[f'{name}_pixel']) < 1e-13
    assert lo.peak_normalised_error(lo.pixelate(img, os_), g[f'{name}_pixelate']) < 1e-12
    # the banded-operator restatement the off-grid kernels follow
    assert lo.peak_normalised_error(lo.pixelate_banded(img, os_), g[f'{name}_pixelate']) < 1e-13


@pytest.mark.parametrize('n,os_', [(5, 2), (10, 3), (33, 4), (200, 16), (97, 3)])
def test_resample_operator_matches_scipy(n, os_):
    # G . s . G^T == map_coordinates(order=3, mode='nearest') at lentil's points,
    # including sizes below the window width and large oversampling
    from scipy.ndimage import map_coordinates
    s = np.random.default_rng(n).uniform(0, 1, (n, n)) ** 3
    S, x, q0, G = lo.resample_operator(n, os_)
    nb = min(lo.RS_BW, n)
    rows = np.stack([s[:, q0[l]:q0[l] + nb] @ G[l, :nb] for l in range(S)], axis=1)
    out = np.stack([G[k, :nb] @ rows[q0[k]:q0[k] + nb, :] for k in range(S)], axis=0)
    xx, yy = np.meshgrid(x, x)
    ref = map_coordinates(s, [yy, xx], order=3, mode='nearest')
    assert out.shape == (int(np.ceil(n * (1 / os_))),) * 2
    assert lo.peak_normalised_error(out, ref) < 1e-14


@pytest.mark.parametrize('name', FFT_CASES)
def test_propagate_fft_cases(golden, name):
    g = golden('propagate_fft')
    wf, kw, scratch = fft_case(lo, g, name)
    w = lo.propagate_fft(wf, scratch=scratch, **kw)
    assert tuple(w.shape) == tuple(g[f'{name}_out_shape'])
    assert w.wavelength == float(g[f'{name}_out_wavelength'])
    assert np.array_equal(w.pixelscale, g[f'{name}_out_pixelscale'])
    field = w.data[0].data
    assert field.shape == tuple(g[f'{name}_field_shape'])
    assert lo.peak_normalised_error(fft_field_crop(g, name, field), g[f'{name}_field_crop']) < 1e-12
    assert lo.peak_normalised_error(w.intensity, g[f'{name}_intensity']) < 1e-12
    if scratch is not None:                  # lentil leaves the padded field in scratch
        reg = scratch[:field.shape[0], :field.shape[1]]
        assert np.isclose(reg.sum(), complex(g[f'{name}_scratch_sum']), rtol=1e-12)
        assert np.array_equal(fft_field_crop(g, name, reg), g[f'{name}_scratch_crop'])


def test_scratch_shape(golden):
    g = golden('propagate_fft')
    dx, du, z, os_ = g['scratch_shape_args']
    assert lo.scratch_shape(g['scratch_shape_wl'], dx, du, z, os_) == tuple(g['scratch_shape'])
