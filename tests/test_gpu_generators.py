"""Zernike generators on the GPU (lgb_zernike_coordinates / lgb_zernike_eval)
against lentil 0.8.8's golden outputs and the oracle's restatement of
lentil/zernike.py.  Tolerances: OPDs to 1e-12 of their peak, coordinates to
1e-12 absolute (hypot / atan2 on the GPU vs numpy)."""
import importlib

import numpy as np
import pytest
import torch

import lentil_gb300 as lg
from oracle import lentil_oracle as lo

lz = importlib.import_module('lentil_gb300.zernike')

pytestmark = pytest.mark.gpu


def _close(a, b, tol=1e-12):
    a, b = np.asarray(a, float), np.asarray(b, float)
    assert a.shape == b.shape
    assert np.max(np.abs(a - b)) <= tol * max(np.max(np.abs(b)), 1e-300)


def test_zernike_compose_golden(golden, cuda_device):
    g = golden('generators')
    m = lg.circle((64, 64), 30)
    _close(lg.zernike_compose(m, g['zcoeffs']), g['zcompose'])


def test_zernike_coordinates_golden(golden, cuda_device):
    g = golden('generators')
    mm = g['hexseg'][4]
    rho, theta = lg.zernike_coordinates(mm)
    assert np.max(np.abs(rho - g['zcoord_rho'])) < 1e-12
    assert np.max(np.abs(theta - g['zcoord_theta'])) < 1e-12
    seg = lg.zernike_compose(mm, [1e-8, 2e-8, -3e-8], rho=g['zcoord_rho'], theta=g['zcoord_theta'])
    _close(seg, g['zcompose_seg'])


@pytest.mark.parametrize('order', ['noll', 'fringe', 'ansi'])
@pytest.mark.parametrize('normalize', [True, False])
def test_zernike_orders_vs_oracle(cuda_device, order, normalize):
    rng = np.random.default_rng(4)
    mask = lg.circle((100, 90), 40, shift=(3, -2)) > 0.5
    c = rng.normal(0, 1e-7, 36)
    _close(lg.zernike_compose(mask, c, normalize=normalize, order=order),
           lo.zernike_compose(mask, c, normalize=normalize, order=order))


def test_zernike_basis_and_single_modes(cuda_device):
    mask = lg.hexagon((80, 80), 35) > 0
    modes = [1, 2, 3, 4, 7, 11, 16, 22, 37]
    B = lg.zernike_basis(mask, modes)
    Bo = lo.zernike_basis(mask, modes)
    _close(B, Bo)
    Bv = lg.zernike_basis(mask, modes, vectorize=True)
    assert Bv.shape == (len(modes), 80 * 80)
    _close(Bv, Bo.reshape(len(modes), -1))
    for j in (1, 5, 12):
        _close(lg.zernike(mask, j), lo.zernike(mask, j))


def test_zernike_coordinates_shift_rotate(cuda_device):
    mask = lg.circle((70, 64), 28) > 0
    for shift, rot in ((None, 30.0), ((2.5, -1.0), 0.0), ((0.0, 3.0), -45.0)):
        rho, theta = lg.zernike_coordinates(mask, shift=shift, rotate=rot)
        ro, to = lo.zernike_coordinates(mask, shift=shift, rotate=rot)
        assert np.max(np.abs(rho - ro)) < 1e-12
        # theta at the origin itself (rho == 0) is atan2 of signed zeros; no
        # Zernike term depends on it (R_n^m(0) = 0 for m != 0)
        off = ro > 0
        assert np.max(np.abs(np.angle(np.exp(1j * (theta - to)))[off])) < 1e-12


def test_zernike_tensor_in_tensor_out(cuda_device):
    mask = torch.as_tensor(lg.circle((64, 64), 30) > 0.5, device='cuda')
    z = lg.zernike_compose(mask, [0, 1e-7, -2e-7, 5e-8])
    assert isinstance(z, torch.Tensor) and z.is_cuda
    _close(z.cpu().numpy(), lo.zernike_compose(mask.cpu().numpy(), [0, 1e-7, -2e-7, 5e-8]))


def test_zernike_empty_mask_raises(cuda_device):
    with pytest.raises(ValueError):
        lg.zernike_coordinates(np.zeros((16, 16)))


def test_power_spectrum_golden(golden, cuda_device):
    # 64 x 64: the radix-2 FFT path
    g = golden('generators')
    psd = lg.power_spectrum(lg.circle((64, 64), 30), 1 / 64, 25e-9, 8, 2, seed=7)
    _close(psd, g['psd'])


@pytest.mark.parametrize('N', [90, 256])
def test_power_spectrum_vs_oracle(cuda_device, N):
    # 90: DFT-matrix path (not a power of two); 256: FFT path
    mask = lg.circle((N, N), 0.45 * N)
    _close(lg.power_spectrum(mask, 1 / N, 20e-9, 10.0, 2.5, seed=N),
           lo.power_spectrum(mask, 1 / N, 20e-9, 10.0, 2.5, seed=N))


def test_power_spectrum_tensor_and_errors(cuda_device):
    mask = torch.as_tensor(lg.circle((32, 32), 14), device='cuda')
    z = lg.power_spectrum(mask, 1 / 32, 10e-9, 5.0, 2, seed=1)
    assert isinstance(z, torch.Tensor) and z.is_cuda
    _close(z.cpu().numpy(), lo.power_spectrum(mask.cpu().numpy(), 1 / 32, 10e-9, 5.0, 2, seed=1))
    with pytest.raises(ValueError):
        lg.power_spectrum(np.ones((16, 20)), 1 / 16, 1e-8, 4.0, 2, seed=0)
