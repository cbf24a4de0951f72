"""Plane.fit_tilt on the GPU (normal equations + tilt removal kernels)
against the oracle's restatement of lentil's lstsq fit
(lentil/plane.py:522-611).  The end-to-end golden cases with fit_tilt
(tilt_fit1, seg_fit1, nooutput in test_gpu_propagate.py) pin it to lentil.
Tolerance: the fitted tilts to 1e-10 relative and the tilt-free OPD to
1e-12 of its peak (FP64 normal equations vs lentil's SVD lstsq)."""
import numpy as np
import pytest
import torch

import lentil_gb300 as lg
from oracle import lentil_oracle as lo

pytestmark = pytest.mark.gpu


def _fit_both(amp, opd, mask, pixelscale):
    """Both fits plus the OPD scale the residuals are measured against."""
    pg = lg.Pupil(amplitude=amp, opd=opd.copy(), mask=mask, pixelscale=pixelscale, focal_length=10)
    po = lo.Pupil(amplitude=amp, opd=opd.copy(), mask=mask, pixelscale=pixelscale, focal_length=10)
    pg.fit_tilt(inplace=True)
    po.fit_tilt(inplace=True)
    tg = np.array([[t.x, t.y] for t in pg.tilt])
    to = np.array([[t.x, t.y] for t in po.tilt])
    return pg, po, tg, to, np.max(np.abs(opd))


def _check(pg, po, tg, to, opd_scale):
    # tilts relative to the largest fitted tilt, OPD relative to the input
    # OPD (a residual that is only rounding noise has no scale of its own)
    assert tg.shape == to.shape
    scale = np.max(np.abs(to)) or 1.0
    assert np.max(np.abs(tg - to)) <= 1e-10 * scale
    og, oo = np.asarray(pg.opd), np.asarray(po.opd)
    assert isinstance(pg.opd, np.ndarray) and og.shape == oo.shape
    assert np.max(np.abs(og - oo)) <= 1e-12 * opd_scale


def test_fit_tilt_single_antialiased_mask(cuda_device):
    rng = np.random.default_rng(3)
    amp = lg.circle((96, 110), 40, shift=(3, -5))             # fractional edge values
    opd = lg.zernike_compose(amp > 0, rng.normal(0, 1e-7, 8)) + 3e-7 * lg.util.mesh(amp.shape)[0] / 96
    _check(*_fit_both(amp, opd, amp, (1 / 96, 1.2 / 110)))


def test_fit_tilt_golden_segments(golden, cuda_device):
    g = golden('propagate')
    _check(*_fit_both(g['seg_fit1_amp'], g['seg_fit1_opd'], g['seg_fit1_mask'],
                      g['seg_fit1_pixelscale_in'].tolist()))


def test_fit_tilt_18_segments(cuda_device):
    rng = np.random.default_rng(5)
    segs = lg.hex_segments(rings=2, seg_radius=58.4, seg_gap=1)
    segs = np.asarray([lg.pad(s, (512, 512)) for s in segs])
    amp = lg.normalize_power(segs.sum(axis=0))
    r, c = lg.util.mesh(amp.shape)
    opd = np.zeros_like(amp)
    for k in range(segs.shape[0]):
        p = rng.normal(0, 50e-9, 3)
        opd += segs[k] * (p[0] + p[1] * r / 512 + p[2] * c / 512)
    _check(*_fit_both(amp, opd, segs, 1 / 512))


def test_fit_tilt_empty_segment_gives_zero_tilt(cuda_device):
    amp = lg.circle((64, 64), 25)
    masks = np.stack([amp > 0.5, np.zeros((64, 64), bool)]).astype(float)
    opd = 1e-7 * lg.util.mesh((64, 64))[1] / 64
    pg, po, tg, to, sc = _fit_both(amp, opd, masks, 1 / 64)
    assert np.all(tg[1] == 0) and np.all(to[1] == 0)
    _check(pg, po, tg, to, sc)


def test_fit_tilt_keeps_tensor_opd(cuda_device):
    amp = lg.circle((64, 64), 25)
    opd = 2e-7 * lg.util.mesh((64, 64))[0] / 64
    pg = lg.Pupil(amplitude=amp, opd=torch.as_tensor(opd, device='cuda'), pixelscale=1 / 64,
                  focal_length=10)
    pg.fit_tilt(inplace=True)
    assert isinstance(pg.opd, torch.Tensor) and pg.opd.is_cuda
    po = lo.Pupil(amplitude=amp, opd=opd.copy(), pixelscale=1 / 64, focal_length=10)
    po.fit_tilt(inplace=True)
    assert np.max(np.abs(pg.opd.cpu().numpy() - po.opd)) <= 1e-12 * np.max(np.abs(opd))
    tg = np.array([pg.tilt[0].x, pg.tilt[0].y])
    to = np.array([po.tilt[0].x, po.tilt[0].y])
    assert np.max(np.abs(tg - to)) <= 1e-10 * np.max(np.abs(to))
