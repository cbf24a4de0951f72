"""Seeded random sweeps of the transform geometry against the oracle:
dft2 over sizes, sampling, shifts, offsets and normalisation in both
precision forms, and propagate_dft over pupils, output shapes, oversampling,
tilts and output masks.  Bounds: complex128 1e-12 peak-normalised; the split
forms on random complex fields 3e-5 (bf16) / 2e-6 (fp16), on PSFs 2e-6."""
import numpy as np
import pytest

import lentil_gb300 as lg
from oracle import lentil_oracle as lo

pytestmark = pytest.mark.gpu

FIELD_TOL = {'fp64': 1e-12, 'split-bf16': 3e-5, 'split-fp16': 2e-6}


def _geometry(rng):
    m, n = (int(x) for x in rng.integers(1, 160, 2))
    M, N = (int(x) for x in rng.integers(1, 200, 2))
    alpha = tuple(float(a) for a in rng.uniform(0.2, 1.5, 2) / np.array([max(m, 2), max(n, 2)]))
    if rng.random() < 0.3:
        alpha = alpha[0]                          # scalar form
    shift = tuple(float(x) for x in rng.uniform(-3, 3, 2).round(rng.integers(0, 3)))
    offset = tuple(float(x) for x in rng.uniform(-4, 4, 2).round(rng.integers(0, 3)))
    return m, n, M, N, alpha, shift, offset, bool(rng.random() < 0.7)


@pytest.mark.parametrize('seed', range(12))
def test_dft2_random_geometry(cuda_device, seed):
    rng = np.random.default_rng(1000 + seed)
    m, n, M, N, alpha, shift, offset, unitary = _geometry(rng)
    f = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
    kw = dict(shape=(M, N), shift=shift, offset=offset, unitary=unitary)
    ref = lo.dft2(f, alpha, **kw)
    for precision, tol in FIELD_TOL.items():
        F = lg.fourier.dft2(f, alpha, precision=precision, **kw)
        assert F.shape == (M, N)
        assert lo.peak_normalised_error(F, ref) < tol, (precision, m, n, M, N, alpha, shift,
                                                        offset, unitary)


@pytest.mark.parametrize('seed', range(8))
def test_propagate_dft_random_setup(cuda_device, seed):
    rng = np.random.default_rng(2000 + seed)
    npix = int(rng.integers(24, 96))
    amp = lo.normalize_power(lg.circle((npix, npix), npix * rng.uniform(0.3, 0.5)))
    opd = lg.zernike_compose(amp > 0, np.r_[0, rng.normal(0, 40e-9, 8)])
    os_ = int(rng.integers(1, 4))
    shape = tuple(int(x) for x in rng.integers(8, 40, 2))
    prop_shape = None
    if rng.random() < 0.4:
        prop_shape = tuple(max(2, s // 2 + int(rng.integers(0, 3))) for s in shape)
    ps_out = 5e-6 * rng.uniform(0.5, 2.0)
    lam = float(rng.uniform(450e-9, 950e-9))
    tilt = None
    if rng.random() < 0.5:
        tilt = [float(x) for x in rng.normal(0, 3e-6, 2)]
    mask = None
    if rng.random() < 0.3:
        mask = (rng.uniform(size=(shape[0] * os_, shape[1] * os_)) > 0.2).astype(float)
    out = {}
    for mod in (lg, lo):
        pl = mod.Pupil(amplitude=amp, opd=opd, pixelscale=1.0 / npix, focal_length=10.0)
        wf = mod.Wavefront(lam) * pl if tilt is None else mod.Wavefront(lam, tilt=tilt) * pl
        w = mod.propagate_dft(wf, ps_out, shape=shape, prop_shape=prop_shape, oversample=os_,
                              mask=mask)
        out[mod] = w.intensity
    ref = out[lo]
    assert out[lg].shape == ref.shape
    if ref.max() == 0:                            # the PSF fell outside the window
        assert np.all(out[lg] == 0)
    else:
        assert lo.peak_normalised_error(out[lg], ref) < 1e-12
