"""lentil itself, routed through this library as a user would route it.

Where lentil is installed beside the repository (``baseline/_ref``, an
offline install of lentil 0.8.8), these tests import it, compute results with
its stock numpy path, then replace its entry points by this library's as the
integration guide shows and run the same calls again:

* only ``lentil.fourier.dft2`` replaced: lentil's own ``propagate_dft``
  (lentil/propagate.py:235-238 calls ``lentil.fourier.dft2``), Plane and
  Field code then run the transform on the GPU;
* the whole path replaced (planes, wavefront, field, dft2/idft2,
  propagate_dft): lentil-style user code runs on the GPU end to end.

Both must give lentil's results to 1e-12 (peak-normalised, complex128).  The
last test restates the known-answer properties lentil's own suite checks for
dft2/idft2 and propagate_dft (tests/test_fourier.py:7-111,
tests/test_propagate.py:8-163) through the patched ``lentil`` names.  Without
the install the tests skip."""
import os
import sys

import numpy as np
import pytest

import lentil_gb300 as lg
from oracle import lentil_oracle as lo

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LENTIL_DIR = os.path.join(ROOT, 'baseline', '_ref')


@pytest.fixture(scope='module')
def lentil():
    if not os.path.isfile(os.path.join(LENTIL_DIR, 'lentil', '__init__.py')):
        pytest.skip('lentil is not installed under baseline/_ref')
    if LENTIL_DIR not in sys.path:
        sys.path.append(LENTIL_DIR)
    import lentil as mod
    return mod


def _full_patch(lentil, mp):
    """The drop-in of the integration guide, undone after the test."""
    for name in ('Plane', 'Pupil', 'Image', 'Tilt', 'Wavefront'):
        mp.setattr(lentil, name, getattr(lg, name))
    mp.setattr(lentil.field, 'Field', lg.Field)
    mp.setattr(lentil.fourier, 'dft2', lg.fourier.dft2)
    mp.setattr(lentil.fourier, 'idft2', lg.fourier.idft2)
    mp.setattr(lentil, 'propagate_dft', lg.propagate_dft)


def _pupil_inputs(seed, npix=256, radius=120, segments=False):
    rng = np.random.default_rng(seed)
    amp = lg.normalize_power(lg.circle((npix, npix), radius))
    opd = lg.zernike_compose(amp > 0, np.r_[0, rng.normal(0, 100e-9, 10)])
    mask = None
    if segments:
        segs = lg.hex_segments(rings=1, seg_radius=npix / 7, seg_gap=2)
        mask = np.asarray([lg.pad(s, (npix, npix)) for s in segs])
        amp = lg.normalize_power(mask.sum(axis=0))
    return amp, opd, mask


def _user_psfs(L):
    """lentil-style user code (everything through the ``L`` module)."""
    out = {}
    amp, opd, _ = _pupil_inputs(1)
    p = L.Pupil(amplitude=amp, opd=opd, pixelscale=1 / 240, focal_length=10)
    out['mono'] = L.propagate_dft(L.Wavefront(650e-9) * p, pixelscale=5e-6, shape=128,
                                  oversample=2).intensity
    p2 = L.Pupil(amplitude=amp, opd=opd + 2e-6 * (np.arange(256)[None, :] / 256),
                 pixelscale=1 / 240, focal_length=10)
    p2.fit_tilt(inplace=True)
    out['fit_tilt'] = L.propagate_dft(L.Wavefront(700e-9) * p2, pixelscale=5e-6, shape=(96, 80),
                                      oversample=3).intensity
    amp_s, opd_s, mask = _pupil_inputs(2, segments=True)
    ps = L.Pupil(amplitude=amp_s, opd=opd_s, mask=mask, pixelscale=1 / 240, focal_length=10)
    img = None
    for lam, w in zip(np.linspace(500e-9, 800e-9, 3), (0.2, 0.5, 0.3)):
        wf = L.propagate_dft(L.Wavefront(lam) * ps, pixelscale=5e-6, shape=64, oversample=2)
        img = wf.insert(np.zeros(wf.shape) if img is None else img, weight=w)
    out['segmented_broadband'] = img
    return out


def test_dft2_only_inside_stock_lentil(lentil, monkeypatch, cuda_device):
    stock = _user_psfs(lentil)
    calls = []

    def gpu_dft2(*a, **k):
        calls.append(1)
        return lg.fourier.dft2(*a, **k)

    monkeypatch.setattr(lentil.fourier, 'dft2', gpu_dft2)
    routed = _user_psfs(lentil)
    assert calls, 'lentil did not call the replaced dft2'
    for k, ref in stock.items():
        assert isinstance(routed[k], np.ndarray) and routed[k].shape == ref.shape
        assert lo.peak_normalised_error(routed[k], ref) <= 1e-12, k


def test_full_dropin_user_code(lentil, monkeypatch, cuda_device):
    stock = _user_psfs(lentil)
    _full_patch(lentil, monkeypatch)
    assert lentil.Pupil is lg.Pupil and lentil.propagate_dft is lg.propagate_dft
    routed = _user_psfs(lentil)
    for k, ref in stock.items():
        assert isinstance(routed[k], np.ndarray) and routed[k].shape == ref.shape
        assert lo.peak_normalised_error(routed[k], ref) <= 1e-12, k


def test_known_answers_through_patched_lentil(lentil, monkeypatch, cuda_device):
    _full_patch(lentil, monkeypatch)
    rng = np.random.default_rng(3)
    for n in (10, 11):                                   # even and odd: the centred FFT
        f = rng.random((n, n)) + 1j * rng.random((n, n))
        F = lentil.fourier.dft2(f, 1 / n, unitary=False)
        np.testing.assert_allclose(F, np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(f))),
                                   rtol=0, atol=1e-12 * np.abs(F).max())
        g = lentil.fourier.idft2(F, 1 / n, unitary=False)
        np.testing.assert_allclose(g, f, rtol=0, atol=1e-12)
    f = rng.random((10, 11)) + 1j * rng.random((10, 11))  # unitary: power is kept
    F = lentil.fourier.dft2(f, (1 / 10, 1 / 11), unitary=True)
    assert abs(np.sum(np.abs(F) ** 2) - np.sum(np.abs(f) ** 2)) < 1e-12 * np.sum(np.abs(f) ** 2)
    out = np.zeros((10, 11), dtype=complex)              # out= is written and returned
    assert lentil.fourier.dft2(f, (1 / 10, 1 / 11), out=out) is out
    # power through propagate_dft at oversample 1 and 2 (a normalised pupil)
    amp, _, _ = _pupil_inputs(0)
    p = lentil.Pupil(amplitude=amp, opd=np.zeros_like(amp), pixelscale=1 / 256, focal_length=10)
    for os_ in (1, 2):
        s = lentil.propagate_dft(lentil.Wavefront(650e-9) * p, shape=(64, 64), pixelscale=5e-6,
                                 oversample=os_).intensity.sum()
        assert 0.95 <= s <= 1
    # a tilt that lands outside the window gives an all-zero image
    pt = lentil.Pupil(amplitude=amp, opd=lg.zernike_compose(amp > 0, [0, 1e-3]),
                      pixelscale=1 / 256, focal_length=10)
    pt.fit_tilt(inplace=True)
    img = lentil.propagate_dft(lentil.Wavefront(650e-9) * pt, shape=(64, 64), pixelscale=5e-6,
                               oversample=2).intensity
    assert np.all(img == 0)
