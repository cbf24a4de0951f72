"""Phase retrieval and the large oversampled workload at their stated sizes.

Phase retrieval: 512 x 512 circular pupil, OPD = Noll 2-37 ~ N(0, 30 nm)
plus 18-segment piston/tip/tilt ~ N(0, 40 nm), three images at defocus -1, 0
and +1 wave P-V (633 nm), 256 x 256 detector at oversample 2 (512 x 512
output), loss = sum (PSF - target)^2 with targets from a seeded true OPD plus
N(0, 1e-4 peak) noise.  The gradient with respect to the OPD map and to the
modal coefficients is checked against a complex128 numpy adjoint written
here (lentil has no gradients) and against central finite differences of the
loss.

Large oversampled: 4096 x 4096 obscured 18-hex pupil with three spiders,
Noll 2-22 + 25 nm rms PSD error and a 50 lambda/D tilt removed by fit_tilt
(an output shift), 1024 x 1024 detector at oversample 4, then pixelate; 2 of
the 32 wavelengths against the oracle's lentil loop and pixelate
(lentil/propagate.py:147-242, lentil/detector.py:225-251)."""
import numpy as np
import pytest
import torch

import lentil_gb300 as lg
from lentil_gb300 import autodiff, workloads
from oracle import lentil_oracle as lo

pytestmark = pytest.mark.gpu

WL = 633e-9


def _phase_retrieval_setup(precision='fp64'):
    npix = 512
    amp = lg.normalize_power(lg.circle((npix, npix), npix // 2))
    support = amp > 0
    segs = lg.hex_segments(rings=2, seg_radius=116.8 * npix / 1024, seg_gap=2)
    segs = np.asarray([lg.pad(x, (npix, npix)) for x in segs]) * support
    rho, th = lg.zernike_coordinates(support)
    basis, sigma = [], []
    for j in range(2, 38):
        basis.append(lg.zernike(support, j, rho=rho, theta=th)); sigma.append(30e-9)
    for sg in segs:
        if sg.sum() == 0:
            continue
        r2, t2 = lg.zernike_coordinates(sg)
        for j in (1, 2, 3):
            basis.append(lg.zernike(sg, j, rho=r2, theta=t2)); sigma.append(40e-9)
    basis, sigma = np.asarray(basis), np.asarray(sigma)
    assert len(sigma) == 36 + 3 * 18
    g64 = autodiff.geometry(amp, WL, 1.0 / npix, 10.0, 5e-6, shape=256, oversample=2,
                            precision='fp64')
    g = g64._replace(precision=precision)
    assert g.shape == (512, 512)
    z4 = lg.zernike(support, 4)
    div = [k * WL / (z4.max() - z4.min()) * z4 for k in (-1, 0, 1)]
    rng = np.random.default_rng(4)
    true_c = rng.normal(0, 1, len(sigma)) * sigma
    pr = autodiff.PhaseRetrieval(amp, basis, div, [np.zeros(g.shape)] * 3, g)
    with torch.no_grad():                       # targets from the complex128 forward
        t = [autodiff.mft_intensity(pr.opd(torch.as_tensor(true_c, device='cuda')) + d, pr.amp, g64)
             for d in pr.diversity]
    pr.targets = [x + 1e-4 * x.max() * torch.as_tensor(rng.normal(size=g.shape), device='cuda')
                  for x in t]
    c0 = rng.normal(0, 1, len(sigma)) * sigma * 0.5          # an iterate away from the truth
    return amp, basis, div, g, pr, c0


def _numpy_loss_grad(amp, basis, div, g, targets, c):
    """complex128 loss and dL/dopd (full map) of the focus-diverse loss."""
    r0, c0, m, n = g.slc
    E1, E2 = lo.dft2_matrices(m, n, g.shape[0], g.shape[1], g.alpha[0], g.alpha[1], 0, 0,
                              g.offset[0], g.offset[1])
    s = np.sqrt(abs(g.alpha[0] * g.alpha[1]))
    opd0 = np.tensordot(c, basis, 1)
    a = amp[r0:r0 + m, c0:c0 + n]
    L, grad = 0.0, np.zeros_like(opd0)
    for d, T in zip(div, targets):
        o = (opd0 + d)[r0:r0 + m, c0:c0 + n]
        f = a * np.exp(2j * np.pi * o / g.wavelength)
        F = s * (E1 @ f @ E2)
        I = np.abs(F) ** 2
        L += np.sum((I - T) ** 2)
        gf = s * (E1.conj().T @ (2 * (I - T) * F) @ E2.conj().T)
        grad[r0:r0 + m, c0:c0 + n] += (2 * np.pi / g.wavelength) * 2 * np.imag(gf * np.conj(f))
    return L, grad


def test_phase_retrieval_full_size_vs_complex128(cuda_device):
    amp, basis, div, g, pr, c0 = _phase_retrieval_setup()
    targets = [t.cpu().numpy() for t in pr.targets]
    L_ref, gopd_ref = _numpy_loss_grad(amp, basis, div, g, targets, c0)
    gc_ref = np.tensordot(basis, gopd_ref, 2)                 # dL/dc = B . dL/dopd
    # the OPD-map gradient through the autograd function, one diversity at a time
    opd0 = torch.as_tensor(np.tensordot(c0, basis, 1), device='cuda').requires_grad_(True)
    a = torch.as_tensor(amp, device='cuda')
    L = sum(((autodiff.mft_intensity(opd0 + torch.as_tensor(d, device='cuda'), a, g)
              - torch.as_tensor(T, device='cuda')) ** 2).sum() for d, T in zip(div, targets))
    L.backward()
    assert abs(L.item() - L_ref) <= 1e-10 * abs(L_ref)
    assert lo.peak_normalised_error(opd0.grad.cpu().numpy(), gopd_ref) < 1e-10
    # the coefficient gradient through the batched loss, eager and graphed
    c = torch.as_tensor(c0, device='cuda').requires_grad_(True)
    Lc = pr.loss(c)
    Lc.backward()
    assert abs(Lc.item() - L_ref) <= 1e-10 * abs(L_ref)
    assert lo.peak_normalised_error(c.grad.cpu().numpy(), gc_ref) < 1e-10
    c.grad = None
    pr.graphed_loss(c).backward()
    assert lo.peak_normalised_error(c.grad.cpu().numpy(), gc_ref) < 1e-10


def test_phase_retrieval_full_size_finite_differences(cuda_device):
    amp, basis, div, g, pr, c0 = _phase_retrieval_setup()
    c = torch.as_tensor(c0, device='cuda').requires_grad_(True)
    pr.loss(c).backward()
    grad = c.grad.cpu().numpy()
    eps = 1e-12
    # Zernike modes (Noll 2, 4, 11, 37) and piston/tip/tilt of two segments
    for k in (0, 2, 9, 35, 36, 38, 52, 53):
        e = torch.zeros_like(c)
        e[k] = eps
        with torch.no_grad():
            fd = (pr.loss(c + e) - pr.loss(c - e)).item() / (2 * eps)
        assert abs(fd - grad[k]) <= 1e-5 * np.max(np.abs(grad)), (k, fd, grad[k])


@pytest.mark.parametrize('precision,tol', [('split-fp16', 1e-4), ('split-bf16', 5e-4)])
def test_phase_retrieval_full_size_split_gradient(cuda_device, precision, tol):
    amp, basis, div, g, pr, c0 = _phase_retrieval_setup()
    _, _, _, gs, prs, _ = _phase_retrieval_setup(precision)
    c = torch.as_tensor(c0, device='cuda').requires_grad_(True)
    pr.loss(c).backward()
    ref = c.grad.cpu().numpy()
    c.grad = None
    prs.loss(c).backward()
    assert lo.peak_normalised_error(c.grad.cpu().numpy(), ref) < tol


@pytest.mark.parametrize('precision,tol', [('fp64', 1e-11), ('split-bf16', 2e-6)])
def test_large_oversampled_full_size_two_wavelengths(cuda_device, precision, tol):
    wl, mask, opd = workloads.large_segmented(npix=4096, n_wavelengths=32)
    idx = [0, 31]
    lam, w = wl.wavelengths[idx], wl.weights[idx]
    kw = dict(shape=wl.det_shape, oversample=wl.oversample)
    pg = lg.Pupil(amplitude=wl.amp, opd=opd.copy(), pixelscale=wl.pixelscale_in, focal_length=10)
    pg.fit_tilt(inplace=True)
    assert len(pg.tilt) == 1
    img = lg.detector.pixelate(lg.broadband_psf(pg, lam, w, wl.det_pixelscale,
                                                precision=precision, **kw), wl.oversample)
    ref = _large_reference(wl, opd, lam, w, kw)
    assert img.shape == ref.shape == (1024, 1024)
    assert lo.peak_normalised_error(img, ref) < tol


_LARGE_REF = {}


def _large_reference(wl, opd, lam, w, kw):
    key = tuple(lam)
    if key not in _LARGE_REF:
        po = lo.Pupil(amplitude=wl.amp, opd=opd.copy(), pixelscale=wl.pixelscale_in,
                      focal_length=10)
        po.fit_tilt(inplace=True)
        _LARGE_REF[key] = lo.pixelate(lo.broadband_psf(po, lam, w, wl.det_pixelscale, **kw),
                                      wl.oversample)
    return _LARGE_REF[key]
