"""The broadband segmented workload at its full size against the oracle.

1024 x 1024 pupil of 18 hexagonal segments (two rings, empty centre, 2 px
gaps), per-segment piston/tip/tilt ~ N(0, 50 nm), Noll 2-22 ~ N(0, 15 nm),
5800 K blackbody weights over 500-900 nm, 512 x 512 detector at oversample 2
(1024 x 1024 output).  The oracle runs lentil's per-segment user loop
(lentil/propagate.py:147-242, lentil/field.py:413-439, lentil/plane.py:494-514:
one field per segment mask, windowed MFT, overlap-add of the intensities) on
4 of the 64 wavelengths; the GPU runs the fused plan (one merged field) in
complex128 and both split precisions on the same inputs.  The 64-wavelength
split PSF is compared with the complex128 plan.

Error metric: max|I - I_ref| / max(I_ref) (peak-normalised), the metric the
split precision is specified against (<= 1e-6 versus FP64); complex128 must
agree with numpy to 1e-12."""
import numpy as np
import pytest
import torch

import lentil_gb300 as lg
from lentil_gb300 import broadband, workloads
from oracle import lentil_oracle as lo

pytestmark = pytest.mark.gpu

SEEDS = [2, 7, 19]
SUBSET = [0, 21, 42, 63]          # 4 of the 64 wavelengths, spread over the band
TOL = {'fp64': 1e-12, 'split-bf16': 1e-6, 'split-fp16': 1e-6}


def _inputs(seed):
    wl = workloads.broadband_segmented(1024, 64, seed=seed)
    opd = wl.opds(1)[0]
    return wl, opd


def _pupils(wl, opd):
    kw = dict(amplitude=wl.amp, opd=opd, mask=wl.mask3d, pixelscale=wl.pixelscale_in,
              focal_length=wl.focal_length)
    return lg.Pupil(**kw), lo.Pupil(**kw)


@pytest.mark.parametrize('seed', SEEDS)
def test_full_size_subset_vs_oracle(cuda_device, seed):
    wl, opd = _inputs(seed)
    pg, po = _pupils(wl, opd)
    lam, w = wl.wavelengths[SUBSET], wl.weights[SUBSET]
    kw = dict(shape=wl.det_shape, oversample=wl.oversample)
    ref = lo.broadband_psf(po, lam, w, wl.det_pixelscale, **kw)
    assert ref.shape == (1024, 1024)
    errs = {}
    for prec in TOL:
        img = lg.broadband_psf(pg, lam, w, wl.det_pixelscale, precision=prec, **kw)
        assert img.shape == ref.shape
        errs[prec] = lo.peak_normalised_error(img, ref)
    print(f'seed {seed}: peak-normalised error vs oracle (4 wavelengths) {errs}')
    for prec, tol in TOL.items():
        assert errs[prec] <= tol, (prec, errs[prec])


def test_full_size_64_wavelengths_split_vs_fp64(cuda_device):
    """All 64 wavelengths through the fused plan as the benchmark runs it
    (device-resident inputs, one merged field): split vs complex128."""
    wl, opd = _inputs(SEEDS[0])
    gmask = wl.mask3d.sum(axis=0)
    amp_eff = wl.amp * gmask
    s = lg.util.boundary_slice(gmask)
    geo = broadband.plan_geometry(wl.plane_shape, s, [], np.broadcast_to(wl.pixelscale_in, (2,)),
                                  wl.focal_length, lg.pupil, wl.wavelengths, wl.det_pixelscale,
                                  shape=wl.det_shape, oversample=wl.oversample)
    assert len(geo.keep) == 64
    A = torch.as_tensor(amp_eff[None], device='cuda')
    O = torch.as_tensor(opd[None], device='cuda')
    W = torch.as_tensor(wl.weights[None], device='cuda')
    ref = broadband.make_plan(geo, precision='fp64').execute(A, O, W).cpu().numpy()
    errs = {}
    for prec in ('split-bf16', 'split-fp16'):
        img = broadband.make_plan(geo, precision=prec).execute(A, O, W).cpu().numpy()
        errs[prec] = lo.peak_normalised_error(img, ref)
    print(f'64 wavelengths, peak-normalised error vs the complex128 plan {errs}')
    for prec, e in errs.items():
        assert e <= TOL[prec], (prec, e)


@pytest.mark.parametrize('lam_index', [0, 63])
def test_full_size_single_wavelength(cuda_device, lam_index):
    """One wavelength alone (no averaging over the band): complex128 to
    1e-12, both split forms to 1e-6.  (bf16 operands chain two K blocks per
    accumulator only when a PSF carries 16 or more wavelengths; a single
    wavelength drains every block, as fp16 always does.)"""
    wl, opd = _inputs(SEEDS[0])
    pg, po = _pupils(wl, opd)
    lam, w = wl.wavelengths[[lam_index]], np.ones(1)
    kw = dict(shape=wl.det_shape, oversample=wl.oversample)
    ref = lo.broadband_psf(po, lam, w, wl.det_pixelscale, **kw)
    errs = {prec: lo.peak_normalised_error(
        lg.broadband_psf(pg, lam, w, wl.det_pixelscale, precision=prec, **kw), ref)
        for prec in TOL}
    print(f'one wavelength ({lam[0] * 1e9:.0f} nm): peak-normalised error vs oracle {errs}')
    assert errs['fp64'] <= 1e-12
    assert errs['split-fp16'] <= 1e-6
    assert errs['split-bf16'] <= 1e-6
