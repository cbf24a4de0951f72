"""Host logic of propagate_fft (no GPU): the padding geometry and the
centred-DFT coordinates that let the MFT kernels evaluate lentil's centred
FFT (lentil/propagate.py:9-136), checked with the oracle's dft2 against
numpy's FFT, and scratch_shape against lentil's golden value."""
import numpy as np
import pytest

from lentil_gb300 import propagate as lgp
from oracle import lentil_oracle as lo


@pytest.mark.parametrize('fshape,N', [((20, 20), (32, 32)), ((21, 20), (33, 32)),
                                      ((19, 23), (35, 37)), ((40, 41), (33, 30)),
                                      ((7, 8), (9, 9)), ((1, 5), (4, 7))])
def test_centred_dft_coords_reproduce_numpy_fft(fshape, N):
    rng = np.random.default_rng(sum(fshape) + sum(N))
    f = rng.standard_normal(fshape) + 1j * rng.standard_normal(fshape)
    ref = lo._fft2c(lo.pad(f, N))
    (a0, a1, d0), (b0, b1, e0) = (lgp._pad_geometry(fshape[0], N[0]),
                                  lgp._pad_geometry(fshape[1], N[1]))
    g = f[a0:a1, b0:b1]
    offset, shift = lgp._centred_dft_coords(g.shape, (d0, e0), N)
    got = lo.dft2(g, (1 / N[0], 1 / N[1]), shape=N, shift=shift, offset=offset, unitary=True)
    assert np.max(np.abs(got - ref)) < 1e-13


@pytest.mark.parametrize('n,N', [(10, 16), (11, 16), (10, 15), (16, 10), (17, 10), (9, 9)])
def test_pad_geometry_matches_lentil_pad(n, N):
    x = np.arange(1, n + 1, dtype=float)[:, None] * np.ones((1, 3))
    ref = lo.pad(x, (N, 3))[:, 0]
    s0, s1, d0 = lgp._pad_geometry(n, N)
    out = np.zeros(N)
    out[d0:d0 + (s1 - s0)] = x[s0:s1, 0]
    assert np.array_equal(out, ref)


def test_scratch_shape_golden(golden):
    g = golden('propagate_fft')
    dx, du, z, os_ = g['scratch_shape_args']
    assert lgp.scratch_shape(g['scratch_shape_wl'], dx, du, z, os_) == tuple(g['scratch_shape'])
    fs, lam = lgp._fft_shape(np.array([dx, dx]), np.array([du, du]), z, 650e-9, os_)
    assert tuple(fs) == (666, 666) and lam == pytest.approx(6.50390625e-07, rel=1e-15)
