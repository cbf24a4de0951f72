"""propagate_fft / scratch_shape on the GPU against lentil's golden vectors
(lentil/propagate.py:9-136).  The centred FFT of the padded field is
evaluated by the library's MFT kernels as a DFT with alpha = 1/N.
Tolerances: complex128 path <= 1e-12 peak-normalised (numpy's FFT and the
complex128 MFT agree to rounding); split tensor-core path <= 2e-6."""
import numpy as np
import pytest
import torch

import lentil_gb300 as lg
from oracle import lentil_oracle as lo
from tests.golden_cases import FFT_CASES, fft_case, fft_field_crop

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('name', FFT_CASES)
def test_propagate_fft_fp64_golden(golden, cuda_device, name):
    g = golden('propagate_fft')
    wf, kw, scratch = fft_case(lg, g, name)
    w = lg.propagate_fft(wf, scratch=scratch, **kw)
    assert tuple(w.shape) == tuple(g[f'{name}_out_shape'])
    assert w.wavelength == float(g[f'{name}_out_wavelength'])
    assert np.array_equal(w.pixelscale, g[f'{name}_out_pixelscale'])
    assert w.ptype == lg.image
    assert len(w.data) == 1
    field = w.data[0].data.cpu().numpy()
    assert field.shape == tuple(g[f'{name}_field_shape'])
    assert lo.peak_normalised_error(fft_field_crop(g, name, field), g[f'{name}_field_crop']) < 1e-12
    I = w.intensity
    assert isinstance(I, np.ndarray)
    assert lo.peak_normalised_error(I, g[f'{name}_intensity']) < 1e-12
    if scratch is not None:                 # lentil leaves the padded field in scratch
        reg = scratch[:field.shape[0], :field.shape[1]]
        # the padded pupil field (GPU phasor vs numpy's exp: equal to rounding)
        assert np.isclose(reg.sum(), complex(g[f'{name}_scratch_sum']), rtol=1e-12)
        assert lo.peak_normalised_error(fft_field_crop(g, name, reg),
                                        g[f'{name}_scratch_crop']) < 1e-13
        assert np.all(scratch[field.shape[0]:, :] == 7)     # outside the region: untouched


@pytest.mark.parametrize('name', ['c1', 'odd', 'crop'])
def test_propagate_fft_split_golden(golden, cuda_device, name):
    g = golden('propagate_fft')
    wf, kw, _ = fft_case(lg, g, name)
    w = lg.propagate_fft(wf, precision='split-bf16', **kw)
    assert lo.peak_normalised_error(w.intensity, g[f'{name}_intensity']) < 2e-6


def test_propagate_fft_tensor_scratch(golden, cuda_device):
    # a CUDA scratch tensor is filled in place like lentil's numpy scratch
    g = golden('propagate_fft')
    wf, kw, scratch = fft_case(lg, g, 'odd_scratch')
    t = torch.as_tensor(scratch, device='cuda')
    w = lg.propagate_fft(wf, scratch=t, **kw)
    assert lo.peak_normalised_error(w.intensity, g['odd_scratch_intensity']) < 1e-12
    reg = t[:153, :191].cpu().numpy()
    assert lo.peak_normalised_error(fft_field_crop(g, 'odd_scratch', reg),
                                    g['odd_scratch_scratch_crop']) < 1e-13


def test_propagate_fft_matches_oracle_random(cuda_device):
    # random rectangular pupil, even x odd FFT shape, against numpy's FFT
    rng = np.random.default_rng(11)
    amp = lg.normalize_power(lg.circle((90, 70), 33))
    opd = rng.normal(0, 5e-8, amp.shape) * (amp > 0)
    lam = (1 / 90) * 6e-6 * 120 / 8
    for mod in (lg, lo):
        pl = mod.Pupil(amplitude=amp, opd=opd, pixelscale=1 / 90, focal_length=8)
        w = mod.propagate_fft(mod.Wavefront(lam) * pl, pixelscale=(6e-6, 5e-6), shape=(50, 40),
                              oversample=2)
        if mod is lg:
            I = w.intensity
        else:
            ref = w.intensity
    assert lo.peak_normalised_error(I, ref) < 1e-12


def test_propagate_fft_errors(cuda_device):
    amp = lg.normalize_power(lg.circle((64, 64), 30))
    pl = lg.Pupil(amplitude=amp, opd=np.zeros_like(amp), pixelscale=1 / 64, focal_length=10)
    wf = lg.Wavefront(600e-9) * pl
    with pytest.raises(ValueError):                # shape beyond fft_shape / oversample
        lg.propagate_fft(wf, pixelscale=5e-6, shape=1000, oversample=2)
    fs = lg.scratch_shape(600e-9, 1 / 64, 5e-6, 10, 2)
    with pytest.raises(ValueError):                # scratch must exceed the FFT shape
        lg.propagate_fft(wf, pixelscale=5e-6, oversample=2,
                         scratch=np.zeros(fs, dtype=complex))
    tilted = lg.Wavefront(600e-9, tilt=[1e-6, 2e-6]) * pl
    with pytest.raises(NotImplementedError):       # tilt needs propagate_dft
        lg.propagate_fft(tilted, pixelscale=5e-6, oversample=2)
    img = lg.Wavefront(600e-9, ptype=lg.image)
    img.data, img.shape = [], (8, 8)
    img.ptype = lg.none
    with pytest.raises(TypeError):                 # ptype must be pupil or image
        lg.propagate_fft(img, pixelscale=5e-6, oversample=2)
