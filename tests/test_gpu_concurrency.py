"""Concurrent callers of the drop-in API.

Two host threads, each on its own CUDA stream, compute broadband PSFs of the
same optics (so they share one cached plan and its operand buffers) with
different OPD maps.  Every result must equal the one computed alone and match
the oracle."""
import threading

import numpy as np
import pytest
import torch

import lentil_gb300 as lg
from oracle import lentil_oracle as lo

pytestmark = pytest.mark.gpu

NPIX, L = 192, 8
WL = np.linspace(500e-9, 800e-9, L)
WT = np.linspace(1.0, 2.0, L) / np.linspace(1.0, 2.0, L).sum()


def _opds(count, seed):
    amp = lg.normalize_power(lg.circle((NPIX, NPIX), NPIX // 2 - 4))
    rng = np.random.default_rng(seed)
    return amp, [lg.zernike_compose(amp, np.r_[0, rng.normal(0, 40e-9, 10)]) for _ in range(count)]


def _psf(amp, opd, precision):
    p = lg.Pupil(amplitude=amp, opd=opd, pixelscale=1 / NPIX, focal_length=10)
    return lg.broadband_psf(p, WL, WT, 5e-6, shape=96, oversample=2, precision=precision)


@pytest.mark.parametrize('precision', ['split-bf16', 'fp64'])
def test_two_threads_two_streams_share_a_plan(cuda_device, precision):
    amp, opds = _opds(6, seed=5)
    alone = [_psf(amp, o, precision) for o in opds]          # sequential, default stream
    got = [None] * len(opds)
    errors = []

    def worker(k0):
        try:
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                for rep in range(3):
                    for k in range(k0, len(opds), 2):
                        got[k] = _psf(amp, opds[k], precision)
        except Exception as e:          # surfaced below
            errors.append(e)

    th = [threading.Thread(target=worker, args=(i,)) for i in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    # the split form sums wavelengths with FP32 reduce-adds whose order varies
    # from run to run; the complex128 form is deterministic
    same = 1e-12 if precision == 'fp64' else 1e-6
    tol = 1e-12 if precision == 'fp64' else 3e-5
    for k, o in enumerate(opds):
        assert lo.peak_normalised_error(got[k], alone[k]) <= same
        ref = lo.broadband_psf(lo.Pupil(amplitude=amp, opd=o, pixelscale=1 / NPIX, focal_length=10),
                               WL, WT, 5e-6, shape=96, oversample=2)
        assert lo.peak_normalised_error(got[k], ref) <= tol
