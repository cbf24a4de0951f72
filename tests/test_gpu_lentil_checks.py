"""The physical checks lentil's own propagation tests make (lentil
tests/test_propagate.py:8-141), restated here and run through the GPU path:
power conservation, the Airy pattern of a circular pupil, the centroid's
invariance under fit_tilt, the analytic image shift of a pupil tilt, and an
all-zero image when the tilt moves the PSF out of the window.  Seeded, and
in both the complex128 and the split tensor-core forms where the check is
not an exact equality."""
import numpy as np
import pytest
import scipy.special

import lentil_gb300 as lg
from oracle import lentil_oracle as lo

pytestmark = pytest.mark.gpu

PRECISIONS = ['fp64', 'split-bf16']


def _pupil(npix, radius, coeffs=None, focal_length=10.0, diameter=1.0):
    """Circular pupil of unit power with a Zernike OPD, `diameter` across
    2 * radius pixels."""
    amp = lo.normalize_power(lg.circle((npix, npix), radius))
    opd = np.zeros((npix, npix)) if coeffs is None else lg.zernike_compose(amp > 0, coeffs)
    return lg.Pupil(amplitude=amp, opd=opd, pixelscale=diameter / (2 * radius),
                    focal_length=focal_length)


def _psf(p, lam, shape, pixelscale, oversample, precision):
    w = lg.propagate_dft(lg.Wavefront(lam) * p, pixelscale=pixelscale, shape=shape,
                         oversample=oversample, precision=precision)
    return w.intensity


def _airy(diameter, focal_length, lam, pixelscale, n):
    """(2 J1(x) / x)^2 with x = pi q D / (lam f), centred on pixel (n-1)/2."""
    c = (n - 1) / 2.0
    y, x = np.indices((n, n), dtype=float)
    q = np.hypot((x - c) * pixelscale, (y - c) * pixelscale)
    arg = np.pi * q * diameter / (lam * focal_length)
    arg[arg == 0] = np.finfo(float).eps
    return (2 * scipy.special.j1(arg) / arg) ** 2


@pytest.mark.parametrize('precision', PRECISIONS)
@pytest.mark.parametrize('oversample', [1, 2])
def test_power_is_conserved(cuda_device, precision, oversample):
    psf = _psf(_pupil(256, 120), 650e-9, (64, 64), 5e-6, oversample, precision)
    assert 0.95 <= psf.sum() <= 1.0 + 1e-9


@pytest.mark.parametrize('precision', PRECISIONS)
def test_airy_pattern(cuda_device, precision):
    p = _pupil(512, 250)
    psf = _psf(p, 650e-9, 511, 5e-6, 1, precision)          # odd: the DC pixel is central
    ref = _airy(1.0, 10.0, 650e-9, 5e-6, 511)
    assert np.allclose(psf / psf.max(), ref / ref.max(), atol=1e-3)


def _tilt_coeffs(seed):
    c = 5e-6 * np.random.default_rng(seed).uniform(-0.5, 0.5, 3)
    c[0] = 0.0
    return c


@pytest.mark.parametrize('seed', [1, 2, 3])
def test_fit_tilt_keeps_the_centroid(cuda_device, seed):
    coeffs = _tilt_coeffs(seed)
    p = _pupil(256, 120, coeffs)
    psf = _psf(p, 650e-9, 128, 5e-6, 2, 'fp64')
    p.fit_tilt(inplace=True)
    psf_fit = _psf(p, 650e-9, 128, 5e-6, 2, 'fp64')
    psf[psf < 1e-5] = 0
    psf_fit[psf_fit < 1e-5] = 0
    delta = np.abs(np.asarray(lo.centroid(psf)) - np.asarray(lo.centroid(psf_fit)))
    assert np.all(delta <= 1e-10)


@pytest.mark.parametrize('fit', [False, True])
@pytest.mark.parametrize('seed', [4, 5])
def test_tilt_shift_matches_geometry(cuda_device, fit, seed):
    # a Noll Z2/Z3 coefficient c tilts the wavefront by 4c peak-to-valley
    # across the diameter: the image moves by (4c / D) f / pixel, (x, y) ->
    # (row, col) = (y, -x)
    os_, ps, npix = 10, 5e-6, 64
    coeffs = _tilt_coeffs(seed)
    p = _pupil(256, 120, coeffs)
    if fit:
        p.fit_tilt(inplace=True)
    psf = _psf(p, 650e-9, (npix, npix), ps, os_, 'fp64')
    psf = psf / psf.max()
    psf[psf < 0.2] = 0
    shift = np.asarray(lo.centroid(psf)) - npix // 2 * os_
    tilt = coeffs[1:3]
    expect = (tilt / 1.0) * 10.0 / ps * os_ * 4
    expect = np.array([expect[1], -expect[0]])
    assert np.all(np.abs(shift - expect) / os_ < 0.2)


def test_tilt_out_of_the_window_gives_no_image(cuda_device):
    p = _pupil(255, 120, [0, 1e-3])
    p.fit_tilt(inplace=True)
    img = _psf(p, 650e-9, (64, 64), 5e-6, 2, 'fp64')
    assert np.all(img == 0)


@pytest.mark.parametrize('precision', PRECISIONS)
@pytest.mark.parametrize('coeffs,size', [(None, 128), ([0, 1e-6, 2e-6], 64)])
def test_mask_equals_masked_psf(cuda_device, precision, coeffs, size):
    # lentil tests/test_propagate_mask.py:4-37: propagating into a detector
    # mask gives the unmasked PSF times the mask (with and without tilt)
    p = _pupil(256, 120, coeffs)
    mask = lg.rectangle((256, 256), size, size, shift=(20, -30), antialias=False)
    psf = _psf(p, 650e-9, 128, 5e-6, 2, precision)
    w = lg.propagate_dft(lg.Wavefront(650e-9) * p, pixelscale=5e-6, shape=128, oversample=2,
                         mask=mask, precision=precision)
    if precision == 'fp64':
        assert np.allclose(w.intensity, psf * mask)
    else:
        # two different transform sizes, each within 2e-6 of the exact PSF
        assert lo.peak_normalised_error(w.intensity, psf * mask) < 4e-6


@pytest.mark.parametrize('precision', PRECISIONS)
@pytest.mark.parametrize('seed', [0, 3])
def test_rescaled_pupil_gives_the_same_psf(cuda_device, precision, seed):
    # lentil tests/test_propagate.py:144-163: a pupil resampled 3x finer
    # (lentil Plane.rescale: cubic spline, amplitude / scale, pixelscale /
    # scale; prepared here with the oracle's rescale) gives a PSF whose
    # cross-correlation with the original peaks at zero lag and whose power
    # agrees to 1%
    coeffs = np.random.default_rng(seed).uniform(-200e-9, 200e-9, 6)
    amp = lo.normalize_power(lg.circle((256, 256), 120))
    opd = lo.zernike_compose(amp > 0, coeffs)
    amp2 = lo.rescale(amp, 3, order=3, mode='nearest', unitary=False) / 3
    opd2 = lo.rescale(opd, 3, order=3, mode='nearest', unitary=False)
    psfs = []
    for a, o, ps in ((amp, opd, 1.0 / 240), (amp2, opd2, 1.0 / 720)):
        p = lg.Pupil(amplitude=a, opd=o, pixelscale=ps, focal_length=10.0)
        psfs.append(_psf(p, 650e-9, (64, 64), 5e-6, 10, precision))
    xc = np.fft.ifftshift(np.conj(np.fft.fft2(psfs[0])) * np.fft.fft2(psfs[1]))
    assert np.allclose(lo.centroid(np.abs(xc)), [320, 320])
    assert np.isclose(psfs[0].sum(), psfs[1].sum(), rtol=1e-2)


def test_error_behaviour(cuda_device):
    # the exception types lentil raises on the path: ptype misuse
    # (lentil/plane.py:478-481, wavefront.py:96-97, propagate.py:266-267),
    # mask shape (propagate.py:184-185), out dtype (fourier.py:91-93), FFT
    # propagation with tilt (propagate.py:36-38)
    with pytest.raises(TypeError):
        lg.Wavefront(650e-9, ptype=lg.image) * lg.Pupil()
    with pytest.raises(TypeError):
        lg.Wavefront(650e-9, ptype=lg.tilt)
    with pytest.raises(TypeError):
        lg.propagate_dft(lg.Wavefront(650e-9), 5e-6, shape=32)
    p = _pupil(64, 30)
    with pytest.raises(ValueError):
        lg.propagate_dft(lg.Wavefront(650e-9) * p, 5e-6, shape=32, oversample=2,
                         mask=np.ones((10, 10)))
    with pytest.raises(TypeError):
        lg.fourier.dft2(np.ones((4, 4)), 0.1, out=np.zeros((4, 4)))
    with pytest.raises(NotImplementedError):
        lg.propagate_fft(lg.Wavefront(650e-9) * p * lg.Tilt(1e-6, 0), 5e-6, shape=32)
