"""Gradients of the MFT intensity (phase retrieval): against a complex128
numpy reference gradient written here and against finite differences."""
import numpy as np
import pytest
import torch

import lentil_gb300 as lg
from lentil_gb300 import autodiff
from oracle import lentil_oracle as lo

pytestmark = pytest.mark.gpu


def _setup(npix=64, seed=0):
    rng = np.random.default_rng(seed)
    amp = lo.normalize_power(lg.circle((npix, npix), npix * 0.45))
    opd = lg.zernike_compose(amp, np.r_[0, rng.normal(0, 30e-9, 14)])
    g = autodiff.geometry(amp, 633e-9, 1.0 / npix, 10.0, 5e-6 * 4, shape=24, oversample=2)
    target = rng.uniform(0, 1e-3, g.shape)
    return amp, opd, g, target


def _numpy_grad(amp, opd, g, target):
    """dL/dopd of L = sum(|F|^2 - T)^2 in complex128 numpy."""
    r0, c0, m, n = g.slc
    f = amp[r0:r0 + m, c0:c0 + n] * np.exp(2j * np.pi * opd[r0:r0 + m, c0:c0 + n] / g.wavelength)
    E1, E2 = lo.dft2_matrices(m, n, g.shape[0], g.shape[1], g.alpha[0], g.alpha[1], 0, 0,
                              g.offset[0], g.offset[1])
    c = np.sqrt(abs(g.alpha[0] * g.alpha[1]))
    F = c * E1 @ f @ E2
    I = np.abs(F) ** 2
    G = 2 * (I - target)
    gf = c * E1.conj().T @ (G * F) @ E2.conj().T
    grad = np.zeros_like(opd)
    grad[r0:r0 + m, c0:c0 + n] = (2 * np.pi / g.wavelength) * 2 * np.imag(gf * np.conj(f))
    return np.sum((I - target) ** 2), grad


def _gpu_loss_grad(amp, opd, g, target):
    o = torch.as_tensor(opd, device='cuda').requires_grad_(True)
    a = torch.as_tensor(amp, device='cuda')
    t = torch.as_tensor(target, device='cuda')
    L = ((autodiff.mft_intensity(o, a, g) - t) ** 2).sum()
    L.backward()
    return L.item(), o.grad.cpu().numpy()


def test_forward_matches_propagate(cuda_device):
    amp, opd, g, _ = _setup()
    I = autodiff.mft_intensity(torch.as_tensor(opd, device='cuda'), torch.as_tensor(amp, device='cuda'), g)
    pl = lo.Pupil(amplitude=amp, opd=opd, pixelscale=1 / 64, focal_length=10)
    ref = lo.propagate_dft(lo.Wavefront(633e-9) * pl, 5e-6 * 4, shape=24, oversample=2).intensity
    assert lo.peak_normalised_error(I.cpu().numpy(), ref) < 1e-12


def test_gradient_vs_complex128_reference(cuda_device):
    amp, opd, g, target = _setup()
    L_ref, grad_ref = _numpy_grad(amp, opd, g, target)
    L, grad = _gpu_loss_grad(amp, opd, g, target)
    assert abs(L - L_ref) <= 1e-10 * abs(L_ref)
    assert lo.peak_normalised_error(grad, grad_ref) < 1e-10


def test_gradient_finite_differences(cuda_device):
    amp, opd, g, target = _setup(seed=1)
    _, grad = _gpu_loss_grad(amp, opd, g, target)
    rng = np.random.default_rng(5)
    idx = np.argwhere(amp > 0)
    eps = 1e-11
    for r, c in idx[rng.choice(len(idx), 6, replace=False)]:
        p, m_ = opd.copy(), opd.copy()
        p[r, c] += eps
        m_[r, c] -= eps
        Lp, _ = _numpy_grad(amp, p, g, target)
        Lm, _ = _numpy_grad(amp, m_, g, target)
        fd = (Lp - Lm) / (2 * eps)
        assert abs(fd - grad[r, c]) <= 1e-5 * np.max(np.abs(grad)), (r, c, fd, grad[r, c])


@pytest.mark.parametrize('precision,tol', [('split-fp16', 1e-4), ('split-bf16', 5e-4)])
def test_split_gradient_close_to_fp64(cuda_device, precision, tol):
    amp, opd, g, target = _setup(npix=128, seed=2)
    _, grad64 = _gpu_loss_grad(amp, opd, g, target)
    _, grads = _gpu_loss_grad(amp, opd, g._replace(precision=precision), target)
    assert lo.peak_normalised_error(grads, grad64) < tol


def test_phase_retrieval_coefficient_gradients(cuda_device):
    # focus-diverse loss on Zernike + segment piston/tip/tilt coefficients
    npix = 64
    amp = lo.normalize_power(lg.circle((npix, npix), npix * 0.45))
    segs = lg.hex_segments(rings=1, seg_radius=8, seg_gap=1)
    segs = np.asarray([lg.pad(s, (npix, npix)) for s in segs]) * (amp > 0)
    basis = [lg.zernike(amp > 0, j) for j in range(2, 12)]
    for s in segs:
        rho, th = lg.zernike_coordinates(s)
        basis += [lg.zernike(s, j, rho=rho, theta=th) for j in (1, 2, 3)]
    basis = np.asarray(basis)
    g = autodiff.geometry(amp, 633e-9, 1.0 / npix, 10.0, 5e-6 * 4, shape=24, oversample=2)
    z4 = lg.zernike(amp > 0, 4)
    div = [k * 633e-9 / (z4.max() - z4.min()) * z4 for k in (-1, 0, 1)]
    rng = np.random.default_rng(3)
    true_c = rng.normal(0, 30e-9, len(basis))
    pr = autodiff.PhaseRetrieval(amp, basis, div, [np.zeros(g.shape)] * 3, g)
    with torch.no_grad():
        tgts = [autodiff.mft_intensity(pr.opd(torch.as_tensor(true_c, device='cuda')) + d, pr.amp, g)
                for d in pr.diversity]
    pr.targets = [t + 1e-4 * t.max() * torch.as_tensor(rng.normal(size=g.shape), device='cuda')
                  for t in tgts]
    c0 = torch.zeros(len(basis), dtype=torch.float64, device='cuda', requires_grad=True)
    L = pr.loss(c0)
    L.backward()
    grad = c0.grad.cpu().numpy()
    eps = 1e-12
    for k in (0, 3, 11, 15):
        e = torch.zeros_like(c0)
        e[k] = eps
        with torch.no_grad():
            fd = (pr.loss(c0 + e) - pr.loss(c0 - e)).item() / (2 * eps)
        assert abs(fd - grad[k]) <= 1e-5 * np.max(np.abs(grad)), (k, fd, grad[k])


@pytest.mark.parametrize('precision', ['fp64', 'split-bf16'])
def test_stacked_images_match_single_images(cuda_device, precision):
    # a stack of OPD maps (focus-diverse images) goes through one batched MFT
    # forward and backward; images and gradients equal the one-map results
    amp, opd, g, target = _setup()
    g = g._replace(precision=precision)
    rng = np.random.default_rng(9)
    stack = np.stack([opd + k * 40e-9 * lg.zernike_compose(amp, [0, 0, 0, 1]) for k in (-1, 0, 1)])
    targets = rng.uniform(0, 1e-3, (3,) + g.shape)
    a = torch.as_tensor(amp, device='cuda')
    o = torch.as_tensor(stack, device='cuda').requires_grad_(True)
    L = ((autodiff.mft_intensity(o, a, g) - torch.as_tensor(targets, device='cuda')) ** 2).sum()
    L.backward()
    total, grads = 0.0, []
    for k in range(3):
        Lk, gk = _gpu_loss_grad(amp, stack[k], g, targets[k])
        total += Lk
        grads.append(gk)
    tol = 1e-12 if precision == 'fp64' else 1e-10
    assert abs(L.item() - total) <= tol * abs(total)
    gs = np.stack(grads)
    assert np.max(np.abs(o.grad.cpu().numpy() - gs)) <= tol * np.max(np.abs(gs))


@pytest.mark.parametrize('precision', ['fp64', 'split-bf16'])
def test_graphed_loss_matches_eager(cuda_device, precision):
    # the loss and coefficient gradient replayed from CUDA graphs equal the
    # eager evaluation, across several replays with different coefficients;
    # the captured transforms' plans stay cached until the graphs are released
    npix = 64
    amp = lo.normalize_power(lg.circle((npix, npix), npix * 0.45))
    basis = np.asarray([lg.zernike(amp > 0, j) for j in range(2, 16)])
    g = autodiff.geometry(amp, 633e-9, 1.0 / npix, 10.0, 5e-6 * 4, shape=24, oversample=2,
                          precision=precision)
    z4 = lg.zernike(amp > 0, 4)
    div = [k * 633e-9 / (z4.max() - z4.min()) * z4 for k in (-1, 0, 1)]
    rng = np.random.default_rng(8)
    tg = [rng.uniform(0, 1e-3, g.shape) for _ in range(3)]
    pr = autodiff.PhaseRetrieval(amp, basis, div, tg, g)
    lg.fourier.clear_plan_cache()
    c = torch.zeros(len(basis), dtype=torch.float64, device='cuda', requires_grad=True)
    for trial in range(3):
        with torch.no_grad():
            c.copy_(torch.as_tensor(rng.normal(0, 20e-9, len(basis)), device='cuda'))
        c.grad = None
        Lg = pr.graphed_loss(c)
        Lg.backward()
        gg = c.grad.clone()
        c.grad = None
        Le = pr.loss(c)
        Le.backward()
        assert abs(Lg.item() - Le.item()) <= 1e-12 * abs(Le.item()), trial
        assert torch.allclose(gg, c.grad, rtol=1e-10, atol=1e-12 * gg.abs().max().item()), trial
    n_pinned = lg.fourier.plan_cache_info()[0]
    assert n_pinned >= 2                        # forward and adjoint geometries
    old = lg.fourier.PLAN_CACHE_ENTRIES
    try:
        lg.fourier.PLAN_CACHE_ENTRIES = 1       # pinned plans are not evicted
        f = rng.standard_normal((20, 20)) + 0j
        for _ in range(2):
            lg.fourier.dft2(f, 0.05, precision=precision)
        assert lg.fourier.plan_cache_info()[0] == n_pinned + 1
        c.grad = None
        pr.graphed_loss(c).backward()           # replays on the pinned plans
        g2 = c.grad.clone()
        c.grad = None
        pr.loss(c).backward()
        assert torch.allclose(g2, c.grad, rtol=1e-10, atol=1e-12 * g2.abs().max().item())
    finally:
        lg.fourier.PLAN_CACHE_ENTRIES = old
    lg.fourier.clear_plan_cache()               # pinned plans survive a clear
    assert lg.fourier.plan_cache_info()[0] == n_pinned
    c.grad = None
    pr.graphed_loss(c).backward()
    assert torch.isfinite(c.grad).all()
    pr.check()
    pr.release_graphs()
    lg.fourier.clear_plan_cache()
    assert lg.fourier.plan_cache_info()[0] == 0


def test_phasor_stack_forms(cuda_device):
    # the exact form equals lgb_phasor bitwise; the FP32-sine form used by
    # the split precisions stays within 1e-6 of it (large OPDs included)
    from lentil_gb300 import _lib
    rng = np.random.default_rng(14)
    H, W, K, r0, c0, m, n = 40, 36, 3, 2, 3, 31, 29
    amp = torch.as_tensor(rng.uniform(0, 1, (H, W)), device='cuda')
    opd = torch.as_tensor(rng.normal(0, 2e-6, (K, H, W)), device='cuda')
    s = torch.cuda.current_stream().cuda_stream
    out = {}
    for fast in (0, 1):
        f = torch.empty((K, m, n), dtype=torch.complex128, device='cuda')
        _lib.call('lgb_phasor_stack', amp.data_ptr(), opd.data_ptr(), K, H, W, r0, c0, m, n,
                  633e-9, fast, f.data_ptr(), s)
        out[fast] = f
    for k in range(K):
        one = torch.empty((m, n), dtype=torch.complex128, device='cuda')
        _lib.call('lgb_phasor', amp.data_ptr(), 0.0, None, opd[k].data_ptr(), 0.0, H, W, r0, c0,
                  m, n, 633e-9, one.data_ptr(), s)
        assert torch.equal(out[0][k], one)
    assert (out[1] - out[0]).abs().max().item() < 1e-6 * amp.max().item()


def test_basis_expand_and_project(cuda_device):
    # the FP32-basis modal OPD and its adjoint against torch's FP64 sums of
    # the same FP32 basis values (ragged sizes; deterministic repeats)
    from lentil_gb300 import _lib
    rng = np.random.default_rng(15)
    for K, H, W in ((1, 7, 5), (13, 33, 31), (90, 128, 96)):
        B = torch.as_tensor(rng.normal(size=(K, H, W)), device='cuda').float()
        c = torch.as_tensor(rng.normal(size=K), device='cuda')
        out = torch.empty((H, W), dtype=torch.float64, device='cuda')
        s = torch.cuda.current_stream().cuda_stream
        _lib.call('lgb_basis_expand', B.data_ptr(), c.data_ptr(), K, H * W, out.data_ptr(), s)
        ref = torch.einsum('k,khw->hw', c, B.double())
        assert (out - ref).abs().max().item() < 1e-5 * ref.abs().max().item()
        g = torch.as_tensor(rng.normal(size=(H, W)), device='cuda')
        nb = _lib.load().lgb_basis_project_workspace_size(K)
        ws = torch.empty(nb, dtype=torch.uint8, device='cuda')
        res = []
        for _ in range(2):
            pr = torch.empty(K, dtype=torch.float64, device='cuda')
            _lib.call('lgb_basis_project', B.data_ptr(), g.data_ptr(), K, H * W, pr.data_ptr(),
                      ws.data_ptr(), nb, s)
            res.append(pr)
        assert torch.equal(res[0], res[1])
        refp = torch.einsum('khw,hw->k', B.double(), g)
        assert (res[0] - refp).abs().max().item() < 1e-5 * refp.abs().max().item() + 1e-12


def test_squared_error_matches_torch(cuda_device):
    # the fused loss kernel and its gradient against torch's own expression
    g = torch.Generator(device='cuda').manual_seed(5)
    for shape in ((3, 64, 64), (1000,), (0,), (2, 1, 7)):
        I = torch.rand(shape, dtype=torch.float64, device='cuda', generator=g).requires_grad_(True)
        T = torch.rand(shape, dtype=torch.float64, device='cuda', generator=g).requires_grad_(True)
        L = autodiff.squared_error(I, T)
        L.backward(torch.tensor(1.7, dtype=torch.float64, device='cuda'))
        gI, gT = I.grad.clone(), T.grad.clone()
        I.grad = T.grad = None
        R = ((I - T) ** 2).sum()
        R.backward(torch.tensor(1.7, dtype=torch.float64, device='cuda'))
        assert abs(L.item() - R.item()) <= 1e-13 * max(1.0, abs(R.item()))
        assert torch.allclose(gI, I.grad, rtol=1e-15, atol=0)
        assert torch.allclose(gT, T.grad, rtol=1e-15, atol=0)


def test_stacked_opd_matches_broadcast_add(cuda_device):
    # OPD_i = B . c + D_i and dL/dc = B . sum_i dL/dOPD_i in one pass each,
    # against the modal OPD, a broadcast add and autograd's sum over images
    rng = np.random.default_rng(8)
    K, H, W, n = 21, 96, 80, 3
    B = torch.as_tensor(rng.normal(size=(K, H, W)), device='cuda').float().contiguous()
    D = torch.as_tensor(rng.normal(size=(n, H, W)) * 1e-7, device='cuda')
    G = torch.as_tensor(rng.normal(size=(n, H, W)), device='cuda')
    c1 = torch.as_tensor(rng.normal(size=K) * 1e-8, device='cuda').requires_grad_(True)
    c2 = c1.detach().clone().requires_grad_(True)
    s1 = autodiff._StackedOPD.apply(c1, B, D)
    s2 = autodiff._BasisOPD.apply(c2, B).unsqueeze(0) + D
    assert torch.equal(s1, s2)
    (s1 * G).sum().backward()
    (s2 * G).sum().backward()
    assert float((c1.grad - c2.grad).abs().max()) <= 1e-6 * float(c2.grad.abs().max())
