"""propagate_dft, Plane phasors, field algebra and the fused broadband plan on
the GPU against lentil's golden vectors and the oracle."""
import numpy as np
import pytest
import torch

import lentil_gb300 as lg
from oracle import lentil_oracle as lo
from tests.golden_cases import PROPAGATE_CASES, build_pupil, propagate_kwargs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('name', PROPAGATE_CASES)
def test_propagate_fp64_golden(golden, cuda_device, name):
    g = golden('propagate')
    pl = build_pupil(lg, g, name)
    w = lg.propagate_dft(lg.Wavefront(float(g[f'{name}_wavelength'])) * pl,
                         **propagate_kwargs(g, name))
    assert len(w.data) == int(g[f'{name}_nfields'])
    I = w.intensity
    ref = g[f'{name}_intensity']
    assert isinstance(I, np.ndarray) and I.shape == ref.shape
    if np.max(ref) == 0:
        assert np.all(I == 0)
    else:
        assert lo.peak_normalised_error(I, ref) < 1e-12


# split tolerances: two 16-bit planes give 16 (bf16) or 22 (fp16) significant
# bits per operand, and the FP32 tensor-core accumulation is folded into
# round-to-nearest registers after every 64-wide K block
SPLIT_TOL = {'split-bf16': 3e-5, 'split-fp16': 2e-6}


@pytest.mark.parametrize('precision', ['split-bf16', 'split-fp16'])
@pytest.mark.parametrize('name', ['config1', 'tilt_fit1', 'oddrect', 'seg_fit0', 'seg_fit1'])
def test_propagate_split_golden(golden, cuda_device, name, precision):
    g = golden('propagate')
    pl = build_pupil(lg, g, name)
    w = lg.propagate_dft(lg.Wavefront(float(g[f'{name}_wavelength'])) * pl,
                         precision=precision, **propagate_kwargs(g, name))
    e = lo.peak_normalised_error(w.intensity, g[f'{name}_intensity'])
    assert e < SPLIT_TOL[precision], e


def test_plane_phasor_matches_oracle(cuda_device):
    rng = np.random.default_rng(1)
    amp = rng.uniform(size=(10, 10))
    opd = rng.uniform(size=(10, 10))
    p = lg.Plane(pixelscale=1, amplitude=amp, opd=opd)
    w = lg.Wavefront(650e-9) * p
    slc = lo.boundary_slice(amp.astype(bool))
    ref = amp[slc] * np.exp(2 * np.pi * 1j * opd[slc] / 650e-9)
    d = w.data[0].data.cpu().numpy()
    # lentil's own test uses OPDs of up to 1 m: the phase argument reaches
    # 1e7 rad, so both evaluations carry ~1e-16 * 1e7 absolute phase error
    phase_max = 2 * np.pi * np.max(opd) / 650e-9
    assert np.max(np.abs(d - ref)) < 4e-16 * phase_max * np.max(np.abs(ref))


def test_overlapping_segment_slices(cuda_device):
    # lentil tests/test_plane.py:117-131
    seg = lg.hexagon((64, 64), 32, antialias=False)[5:60, :]
    segmask = np.zeros((2, 128, 128))
    segmask[0, 0:55, 2:66] = seg
    segmask[1, 29:84, 55:119] = seg
    mask = np.sum(segmask, axis=0)
    pupil = lg.Pupil(amplitude=mask, mask=segmask, pixelscale=1 / 256, focal_length=10)
    w = lg.Wavefront(500e-9)
    w *= pupil
    assert np.allclose(mask, w.intensity, rtol=0, atol=1e-12)


def test_field_algebra_golden(golden, cuda_device):
    g = golden('field')
    a = lg.Field(np.ones((5, 4)), pixelscale=1, offset=[-2, -2])
    b = lg.Field(np.ones((3, 3)), pixelscale=1, offset=[0, -1])
    c = lg.field.merge(a, b)
    assert np.array_equal(c.data.cpu().numpy(), g['merge_data'])
    assert np.array_equal(c.offset, g['merge_offset'])
    fs = [lg.Field(g[f'reduce_in{k}_data'], pixelscale=1, offset=list(g[f'reduce_in{k}_offset']))
          for k in range(4)]
    red = lg.field.reduce(fs)
    assert len(red) == int(g['reduce_n'])
    for k, f in enumerate(red):
        assert np.allclose(f.data.cpu().numpy(), g[f'reduce_out{k}_data'], rtol=0, atol=1e-15)
        assert np.array_equal(f.offset, g[f'reduce_out{k}_offset'])
    out = np.zeros((9, 8))
    for f in fs:
        out = lg.field.insert(f, out, intensity=True, weight=0.7)
    assert np.allclose(out, g['insert_intensity'], rtol=1e-14, atol=0)
    out = np.zeros((9, 8), dtype=complex)
    for f in fs:
        out = lg.field.insert(f, out)
    assert np.allclose(out, g['insert_complex'], rtol=0, atol=1e-15)


@pytest.mark.parametrize('case', [
    (1, [0, 0], 1, [0, 0], 1 + 0j, [0, 0]),
    (1, [0, 0], 1, [1, 0], [], [0, 0]),
    (np.ones((2, 2)), [0, 0], np.ones((2, 2)), [0, 0], np.ones((2, 2)), [0, 0]),
    (np.ones((2, 2)), [0, 0], np.ones((2, 2)), [4, 4], [], [0, 0]),
    (1, [0, 0], np.ones((3, 3)), [-5, -5], np.ones((3, 3)), [-5, -5]),
    (np.ones((5, 4)), [-2, -2], np.ones((3, 3)), [0, -1], np.ones((2, 2)), [0, -1]),
])
def test_field_multiply(cuda_device, case):
    # lentil tests/test_field.py:7-24
    a_data, a_off, b_data, b_off, data, off = case
    c = lg.Field(a_data, pixelscale=1, offset=a_off) * lg.Field(b_data, pixelscale=1, offset=b_off)
    assert np.array_equal(c.data.cpu().numpy(), np.asarray(data, dtype=complex))
    if c.size:
        assert np.array_equal(c.offset, off)


def test_default_wavefront(cuda_device):
    w = lg.Wavefront(wavelength=500e-9)
    assert np.array_equal(w.field, 1 + 0j)
    assert np.array_equal(w.intensity, 1)
    with pytest.raises(TypeError):
        lg.propagate_dft(w, shape=(64, 64), pixelscale=5e-6)


def _bb_pupil(golden):
    g = golden('propagate')
    return g, dict(amplitude=g['bb_amp'], opd=g['bb_opd'], pixelscale=g['bb_pixelscale_in'].tolist(),
                   focal_length=10)


@pytest.mark.parametrize('precision,tol', [('fp64', 1e-12), ('split-bf16', 2e-6),
                                           ('split-fp16', 5e-7)])
def test_broadband_plan_golden(golden, cuda_device, precision, tol):
    g, kw = _bb_pupil(golden)
    img = lg.broadband_psf(lg.Pupil(**kw), g['bb_wl'], g['bb_wt'], 6e-6, shape=24, oversample=2,
                           precision=precision)
    e = lo.peak_normalised_error(img, g['bb_img'])
    assert e < tol, e


def test_broadband_loop_equals_plan(golden, cuda_device):
    # the user loop through propagate_dft + Wavefront.insert and the fused plan
    g, kw = _bb_pupil(golden)
    pl = lg.Pupil(**kw)
    img = np.zeros((48, 48))
    for lam, w in zip(g['bb_wl'], g['bb_wt']):
        img = lg.propagate_dft(lg.Wavefront(lam) * pl, 6e-6, shape=24, oversample=2).insert(img, w)
    assert lo.peak_normalised_error(img, g['bb_img']) < 1e-12
    fused = lg.broadband_psf(pl, g['bb_wl'], g['bb_wt'], 6e-6, shape=24, oversample=2,
                             precision='fp64')
    assert lo.peak_normalised_error(fused, img) < 1e-12


@pytest.mark.parametrize('fit', [False, True])
def test_broadband_segmented(golden, cuda_device, fit):
    # 3-D segment mask: merged dense field (no tilts) or per-segment fields
    g = golden('propagate')
    name = f'seg_fit{int(fit)}'
    wl = np.array([500e-9, 550e-9, 640e-9])
    wt = np.array([0.3, 0.3, 0.4])
    pl = build_pupil(lg, g, name)
    po = build_pupil(lo, g, name)
    kw = propagate_kwargs(g, name)
    ref = lo.broadband_psf(po, wl, wt, **kw)
    for prec, tol in (('fp64', 1e-12), ('split-bf16', 2e-5)):
        img = lg.broadband_psf(pl, wl, wt, precision=prec, **kw)
        assert lo.peak_normalised_error(img, ref) < tol, prec


def test_plan_batch_matches_single(cuda_device):
    # PSFs of a batch equal the same PSFs computed alone
    rng = np.random.default_rng(9)
    H = 96
    amp = lo.normalize_power(lg.circle((H, H), 44))
    wl = np.linspace(500e-9, 800e-9, 5)
    alphas = [((1 / 88) * 5e-6 / (l * 10 * 2),) * 2 for l in wl]
    shifts = [(0.0, 0.0)] * len(wl)
    B = 3
    opd = np.stack([lg.zernike_compose(amp, np.r_[0, rng.normal(0, 30e-9, 10)]) for _ in range(B)])
    wts = rng.uniform(0.5, 1.5, (B, len(wl)))
    A = torch.as_tensor(np.broadcast_to(amp, (B, H, H)).copy(), device='cuda')
    O = torch.as_tensor(opd, device='cuda')
    for prec in ('fp64', 'split-bf16'):
        plan = lg.PSFPlan((H, H), (0, 0, H, H), (0, 0), wl, alphas, shifts, (80, 72), (80, 72),
                          (0, 0), batch=B, precision=prec)
        outb = plan.execute(A, O, wts).cpu().numpy()
        one = lg.PSFPlan((H, H), (0, 0, H, H), (0, 0), wl, alphas, shifts, (80, 72), (80, 72),
                         (0, 0), batch=1, precision=prec)
        for b in range(B):
            o1 = one.execute(A[b:b + 1].contiguous(), O[b:b + 1].contiguous(), wts[b:b + 1]).cpu().numpy()
            # the split path reduces wavelengths into FP32 with atomic adds,
            # whose order is not fixed: equal to FP32 rounding, not bitwise
            tol = 1e-12 if prec == 'fp64' else 1e-6
            assert lo.peak_normalised_error(outb[b], o1[0]) < tol


def test_execute_streams_matches_execute(cuda_device):
    # PSFs alternating over two streams with a workspace each equal the same
    # PSFs executed one by one on the caller's stream
    rng = np.random.default_rng(15)
    H = 96
    amp = lo.normalize_power(lg.circle((H, H), 44))
    wl = np.linspace(500e-9, 800e-9, 20)
    alphas = [((1 / 88) * 5e-6 / (l * 10 * 2),) * 2 for l in wl]
    shifts = [(0.0, 0.0)] * len(wl)
    n = 5
    O = torch.as_tensor(np.stack([lg.zernike_compose(amp, np.r_[0, rng.normal(0, 30e-9, 10)])
                                  for _ in range(n)]), device='cuda')
    A1 = torch.as_tensor(amp[None].copy(), device='cuda')
    An = torch.as_tensor(np.stack([amp * rng.uniform(0.5, 1.5) for _ in range(n)]), device='cuda')
    W1 = torch.as_tensor(rng.uniform(0.5, 1.5, (1, len(wl))), device='cuda')
    Wn = torch.as_tensor(rng.uniform(0.5, 1.5, (n, len(wl))), device='cuda')
    for prec in ('split-bf16', 'fp64'):
        plan = lg.PSFPlan((H, H), (0, 0, H, H), (0, 0), wl, alphas, shifts, (80, 72), (80, 72),
                          (0, 0), batch=1, precision=prec)
        for A, W in ((A1, W1), (An, Wn)):
            one = torch.stack([plan.execute(A if A.shape[0] == 1 else A[k:k + 1], O[k:k + 1],
                                            W if W.shape[0] == 1 else W[k:k + 1])[0]
                               for k in range(n)])
            out = torch.full((n, 80, 72), 7.0, dtype=torch.float64, device='cuda')
            got = plan.execute_streams(A, O, W, out)
            assert got is out
            plan.stream_status()
            tol = (1e-13 if prec == 'fp64' else 1e-6) * float(one.abs().max())
            assert float((out - one).abs().max()) <= tol, prec
        # one PSF, and inside a CUDA-graph capture: in order on the caller's stream
        out1 = plan.execute_streams(A1, O[:1], W1, torch.empty((1, 80, 72), dtype=torch.float64,
                                                               device='cuda'))
        ref1 = plan.execute(A1, O[:1], W1)
        assert float((out1 - ref1).abs().max()) <= 1e-6 * float(ref1.abs().max())
        if prec != 'fp64':
            outg = torch.empty((n, 80, 72), dtype=torch.float64, device='cuda')
            plan.execute_streams(A1, O, W1, outg)            # warm: plan memory, tuner decided
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                g.capture_begin(capture_error_mode='thread_local')
                plan.execute_streams(A1, O, W1, outg)
                g.capture_end()
            torch.cuda.current_stream().wait_stream(side)
            outg.zero_()
            g.replay()
            torch.cuda.synchronize()
            ref = plan.execute_streams(A1, O, W1, torch.empty_like(outg))
            assert float((outg - ref).abs().max()) <= 1e-6 * float(ref.abs().max())


def test_split_phase_of_a_large_opd(cuda_device):
    # tens of waves of OPD: the split operand's phase (the float64 OPD split
    # into a float pair by integer operations, times 1/lambda as a float-float
    # product, reduced to a cycle) must hold the field to the split's own
    # precision, as the complex128 plan does
    H = 128
    amp = lo.normalize_power(lg.circle((H, H), 60))
    rho, theta = lg.zernike_coordinates(amp > 0)
    opd = (30e-6 * lg.zernike(amp > 0, 4, rho=rho, theta=theta)           # ~60 waves P-V
           + 8e-6 * lg.zernike(amp > 0, 2, rho=rho, theta=theta)
           + 3e-9 * np.random.default_rng(16).normal(size=(H, H)))
    wl = np.linspace(500e-9, 700e-9, 6)
    wt = np.full(len(wl), 1 / len(wl))
    kw = dict(shape=64, oversample=2)
    pl = lg.Pupil(amplitude=amp, opd=opd, pixelscale=1 / 120, focal_length=10)
    ref = lg.broadband_psf(pl, wl, wt, 5e-6, precision='fp64', **kw)
    po = lo.Pupil(amplitude=amp, opd=opd, pixelscale=1 / 120, focal_length=10)
    assert lo.peak_normalised_error(ref, lo.broadband_psf(po, wl, wt, 5e-6, **kw)) < 1e-12
    # fp16 (22 bits, the default split form) holds 1e-6 however far the
    # defocus lowers the peak; bf16's 16 bits are ~1e-5 of the field, and
    # against a peak ~1e-3 of the focused one that shows as ~5e-6
    for prec, tol in (('split-fp16', 1e-6), ('split', 1e-6), ('split-bf16', 2e-5)):
        img = lg.broadband_psf(pl, wl, wt, 5e-6, precision=prec, **kw)
        assert lo.peak_normalised_error(img, ref) < tol, prec


def test_broadband_many_wavelengths(cuda_device):
    # 520 wavelengths: the phasor operand kernel's blocks then take more than
    # 32 wavelengths each (16 groups at most), so they reload their
    # wavelength factors part-way through the loop
    rng = np.random.default_rng(14)
    H = 40
    amp = lo.normalize_power(lg.circle((H, H), 18))
    opd = lg.zernike_compose(amp, np.r_[0, rng.normal(0, 40e-9, 10)])
    wl = np.linspace(500e-9, 900e-9, 520)
    wt = rng.uniform(0.5, 1.5, len(wl))
    wt /= wt.sum()
    kw = dict(shape=16, oversample=2)
    po = lo.Pupil(amplitude=amp, opd=opd, pixelscale=1 / 36, focal_length=10)
    ref = lo.broadband_psf(po, wl, wt, 5e-6, **kw)
    for prec, tol in (('fp64', 1e-12), ('split-bf16', 2e-6)):
        pl = lg.Pupil(amplitude=amp, opd=opd, pixelscale=1 / 36, focal_length=10)
        img = lg.broadband_psf(pl, wl, wt, 5e-6, precision=prec, **kw)
        assert lo.peak_normalised_error(img, ref) < tol, prec


@pytest.mark.parametrize('image,origin', [((80, 72), (0, 0)),        # the window is the image
                                          ((100, 90), (7, 11))])    # a window inside the image
def test_plan_output_overwrite_and_accumulate(cuda_device, image, origin):
    # accumulate=False replaces whatever the output held (a window that
    # covers the image is stored without clearing it first); accumulate=True
    # adds the PSF to it
    rng = np.random.default_rng(12)
    H = 96
    amp = lo.normalize_power(lg.circle((H, H), 44))
    wl = np.linspace(500e-9, 800e-9, 4)
    alphas = [((1 / 88) * 5e-6 / (l * 10 * 2),) * 2 for l in wl]
    shifts = [(0.0, 0.0)] * len(wl)
    A = torch.as_tensor(amp[None].copy(), device='cuda')
    O = torch.as_tensor(lg.zernike_compose(amp, np.r_[0, rng.normal(0, 30e-9, 10)])[None],
                        device='cuda')
    W = torch.as_tensor(rng.uniform(0.5, 1.5, (1, len(wl))), device='cuda')
    for prec in ('fp64', 'split-bf16'):
        plan = lg.PSFPlan((H, H), (0, 0, H, H), (0, 0), wl, alphas, shifts, (80, 72), image,
                          origin, batch=1, precision=prec)
        fresh = plan.execute(A, O, W).cpu().numpy()
        assert fresh.shape == (1,) + image
        r0, c0 = origin
        outside = np.ones(image, bool)
        outside[r0:r0 + 80, c0:c0 + 72] = False
        assert np.all(fresh[0][outside] == 0)
        garbage = torch.as_tensor(rng.uniform(-5, 5, (1,) + image), device='cuda')
        over = plan.execute(A, O, W, out=garbage.clone()).cpu().numpy()
        added = plan.execute(A, O, W, out=garbage.clone(), accumulate=True).cpu().numpy()
        tol = (1e-13 if prec == 'fp64' else 1e-6) * fresh.max()  # split: FP32 atomics, order not fixed
        assert np.abs(over - fresh).max() <= tol, prec
        assert np.abs(added - (garbage.cpu().numpy() + fresh)).max() <= tol + 1e-12, prec


@pytest.mark.parametrize('name', ['px64os2', 'px90os3', 'px128os4',          # grid samples
                                  'px100os3', 'px75os2', 'px61os7', 'px128os3', 'px64os5'])
def test_pixel_pixelate_golden(golden, cuda_device, name):
    # lentil/detector.py:167-251 against lentil's own outputs
    g = golden('detector')
    img, os_ = g[f'{name}_img'], int(g[f'{name}_os'])
    assert lo.peak_normalised_error(lg.detector.pixel(img, os_), g[f'{name}_pixel']) < 1e-12
    assert lo.peak_normalised_error(lg.detector.pixelate(img, os_), g[f'{name}_pixelate']) < 1e-12


def test_pixel_unitary_and_errors(cuda_device):
    # lentil tests/test_detector.py:86-97
    a = np.random.default_rng(2).uniform(0, 1, (100, 100))
    assert np.isclose(np.sum(a), np.sum(lg.detector.pixel(a, oversample=1)), rtol=1e-12)
    assert lg.detector.pixelate(np.ones((10, 10)), 2).shape == (5, 5)
    assert lg.detector.pixelate(np.ones((10, 10)), 3).shape == (4, 4)     # ceil(10/3)
    with pytest.raises(ValueError):
        lg.detector.pixel(np.ones((10, 12)), 2)
    with pytest.raises(NotImplementedError):
        lg.detector.pixelate(np.ones((10, 10)), 2.5)


@pytest.mark.parametrize('n,os_', [(5, 2), (33, 4), (200, 16), (1000, 3), (2048, 3)])
def test_pixelate_off_grid_matches_oracle(cuda_device, n, os_):
    # off-grid cubic resampling (N % os != 0; both pixel-MTF paths: FFT for
    # 2048, circulant GEMMs otherwise) against the oracle; numpy in -> numpy
    # out, CUDA tensor in -> CUDA tensor out
    img = np.random.default_rng(n).uniform(0, 1, (n, n)) ** 4
    ref = lo.pixelate(img, os_)
    out = lg.detector.pixelate(img, os_)
    assert isinstance(out, np.ndarray) and out.shape == ref.shape
    assert lo.peak_normalised_error(out, ref) < 1e-12
    assert np.isclose(out.sum(), ref.sum(), rtol=1e-12)
    t = lg.detector.pixelate(torch.as_tensor(img, device='cuda'), os_)
    assert t.is_cuda and lo.peak_normalised_error(t.cpu().numpy(), ref) < 1e-12


@pytest.mark.parametrize('precision,tol', [('fp64', 1e-11), ('split-bf16', 3e-6)])
def test_large_oversampled_pixelated_small_scale(cuda_device, precision, tol):
    # the large oversampled workload at reduced size: obscured 18-hex pupil
    # with spiders, PSD error and a large tilt removed by fit_tilt (output
    # shift), oversample 4, then pixelate
    from lentil_gb300 import workloads
    wl, mask, opd = workloads.large_segmented(npix=256, n_wavelengths=3, tilt_lambda_d=6.0)
    lam, w = wl.wavelengths, wl.weights
    kw = dict(shape=64, oversample=4)
    po = lo.Pupil(amplitude=wl.amp, opd=opd.copy(), pixelscale=wl.pixelscale_in, focal_length=10)
    po.fit_tilt(inplace=True)
    ref = lo.pixelate(lo.broadband_psf(po, lam, w, wl.det_pixelscale, **kw), 4)
    pg = lg.Pupil(amplitude=wl.amp, opd=opd.copy(), pixelscale=wl.pixelscale_in, focal_length=10)
    pg.fit_tilt(inplace=True)
    assert len(pg.tilt) == 1
    img = lg.detector.pixelate(lg.broadband_psf(pg, lam, w, wl.det_pixelscale,
                                                precision=precision, **kw), 4)
    assert img.shape == ref.shape == (64, 64)
    assert lo.peak_normalised_error(img, ref) < tol


def test_image_to_pupil_round_trip(cuda_device):
    # pupil -> image -> field stop (Image plane) -> propagate_dft back to a
    # pupil plane (lentil/propagate.py:263-272 flips the ptype), complex128,
    # against the oracle at every plane
    rng = np.random.default_rng(17)
    amp = lg.normalize_power(lg.circle((96, 96), 44))
    opd = lg.zernike_compose(amp > 0, np.r_[0, rng.normal(0, 40e-9, 10)])
    stop = lg.circle((64, 64), 20)
    out = {}
    for mod in (lg, lo):
        pl = mod.Pupil(amplitude=amp, opd=opd, pixelscale=1 / 96, focal_length=10)
        w = mod.propagate_dft(mod.Wavefront(700e-9) * pl, pixelscale=8e-6, shape=32, oversample=2)
        assert w.ptype == (lg.image if mod is lg else lo.IMAGE)
        w = mod.Image(amplitude=stop, pixelscale=4e-6) * w
        back = mod.propagate_dft(w, pixelscale=1 / 96, shape=96, oversample=1)
        assert back.ptype == (lg.pupil if mod is lg else lo.PUPIL)
        f = back.field
        out[mod.__name__] = f.cpu().numpy() if isinstance(f, torch.Tensor) else np.asarray(f)
    got, ref = out['lentil_gb300'], out[lo.__name__]
    assert got.shape == ref.shape == (96, 96)
    assert lo.peak_normalised_error(got, ref) < 1e-12


@pytest.mark.parametrize('name', ['lin', 'steep', 'tilt'])
@pytest.mark.parametrize('precision,tol', [('fp64', 1e-12), ('split-bf16', 2e-6)])
def test_tilt_planes_golden(golden, cuda_device, name, precision, tol):
    # Wavefront * pupil * (DispersiveTilt | Tilt) through lentil's broadband
    # loop: each wavelength lands at its own window (a dispersed spectrum)
    g = golden('tilt')
    pl = lg.Pupil(amplitude=g['img_amp'], opd=g['img_opd'], pixelscale=1 / 60, focal_length=10)
    if name == 'tilt':
        tp = lg.Tilt(x=2.3e-6, y=-1.1e-6)
    else:
        tp = lg.DispersiveTilt(trace=g[f'{name}_trace'], dispersion=g[f'{name}_dispersion'])
    img = np.zeros((96, 96))
    budget = 0.0                  # each wavelength's error is bounded by its own peak
    for lam, wt in zip(g['img_wl'], g['img_wt']):
        w = lg.propagate_dft(lg.Wavefront(lam) * pl * tp, pixelscale=6e-6, shape=48, oversample=2,
                             precision=precision)
        img = w.insert(img, weight=wt)
        budget += wt * w.intensity.max()
    ref = g[f'img_{name}']
    assert lo.peak_normalised_error(img, ref) < tol * budget / ref.max()


@pytest.mark.parametrize('tile', [256, 128])
def test_zero_field_blocks_are_skipped_exactly(cuda_device, tile):
    # Two discs 870 columns apart: the field's bounding box (671 x 991) holds
    # whole column tiles without a nonzero entry and many all-zero 64-row K
    # blocks, which the tensor-core stage 1 skips (an odd count of 21 K
    # blocks, so one block straddles the real and imaginary rows).  The
    # result must match the complex128 oracle as a dense field does.
    H = 1024
    amp = lg.circle((H, H), 60, shift=(-300, -440)) + lg.circle((H, H), 60, shift=(250, 430))
    amp = lo.normalize_power(amp)
    opd = lo.zernike_compose(amp > 0, [0, 0, 0, 80e-9, 30e-9, -20e-9])
    wl = np.array([600e-9, 700e-9, 800e-9])
    wt = np.array([0.3, 0.3, 0.4])
    kw = dict(pixelscale=5e-6, shape=64, oversample=2)
    ref = lo.broadband_psf(lo.Pupil(amplitude=amp, opd=opd, pixelscale=1 / H, focal_length=10),
                           wl, wt, **kw)
    pl = lg.Pupil(amplitude=amp, opd=opd, pixelscale=1 / H, focal_length=10)
    with lg.tuner.forced(tile):
        img = lg.broadband_psf(pl, wl, wt, precision='split-bf16', **kw)
    assert lo.peak_normalised_error(img, ref) < 2e-6


def test_frozen_pupil_keeps_its_field_on_the_device(cuda_device):
    # a frozen pupil's merged field is cached on the device across broadband
    # calls; thawing drops it, so a changed OPD is seen after re-freezing
    rng = np.random.default_rng(23)
    segs = lg.hex_segments(rings=1, seg_radius=18, seg_gap=2)
    mask = np.asarray([lg.pad(s_, (128, 128)) for s_ in segs])
    amp = lg.normalize_power(mask.sum(axis=0))
    opd1 = lg.zernike_compose(amp > 0, np.r_[0, rng.normal(0, 40e-9, 10)])
    opd2 = lg.zernike_compose(amp > 0, np.r_[0, rng.normal(0, 40e-9, 10)])
    wl, wt = np.linspace(500e-9, 800e-9, 3), np.array([0.3, 0.4, 0.3])
    kw = dict(shape=32, oversample=2, precision='fp64')

    def ref(opd):
        po = lo.Pupil(amplitude=amp, opd=opd, mask=mask, pixelscale=1 / 128, focal_length=10)
        return lo.broadband_psf(po, wl, wt, 5e-6, shape=32, oversample=2)

    p = lg.Pupil(amplitude=amp, opd=opd1, mask=mask, pixelscale=1 / 128, focal_length=10)
    p.freeze()
    first = lg.broadband_psf(p, wl, wt, 5e-6, **kw)
    assert getattr(p, '_lgb_device_field', None) is not None
    again = lg.broadband_psf(p, wl, wt, 5e-6, **kw)
    assert np.array_equal(first, again)
    assert lo.peak_normalised_error(first, ref(opd1)) < 1e-12
    p.thaw()
    assert getattr(p, '_lgb_device_field', None) is None
    p.opd = opd2
    p.freeze()
    assert lo.peak_normalised_error(lg.broadband_psf(p, wl, wt, 5e-6, **kw), ref(opd2)) < 1e-12
