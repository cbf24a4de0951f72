"""Continuous-batching server: every result equals the same PSF computed
alone (fused plan and oracle) while requests of different sizes overlap."""
import numpy as np
import pytest

import lentil_gb300 as lg
from lentil_gb300 import serving
from oracle import lentil_oracle as lo

pytestmark = pytest.mark.gpu

TOL = 2e-6    # split-precision PSF vs its own result computed alone / the oracle


def _request(rng, npix, det, L, segmented=False):
    if segmented:
        segs = lg.hex_segments(rings=2, seg_radius=npix * 0.114, seg_gap=1)
        amp = lg.pad(np.sum(segs, axis=0), (npix, npix))
    else:
        amp = lg.circle((npix, npix), npix * 0.45)
    amp = lg.normalize_power(amp)
    opd = lg.zernike_compose(amp > 0, np.r_[0, rng.normal(0, 20e-9, 10)])
    wl = np.linspace(400e-9, 1000e-9, L) if L > 1 else np.array([700e-9])
    w = rng.uniform(0.5, 1.5, L)
    return serving.PSFRequest(amp, opd, wl, w / w.sum(), 1.0 / npix, 10.0, 5e-6 * 256 / npix,
                              det, oversample=2)


def _alone(req):
    pl = lo.Pupil(amplitude=req.amp, opd=req.opd, pixelscale=req.pixelscale_in,
                  focal_length=req.focal_length)
    return lo.broadband_psf(pl, req.wavelengths, req.weights, req.det_pixelscale,
                            shape=req.det_shape, oversample=req.oversample)


def test_results_same_alone_and_in_mix(cuda_device):
    rng = np.random.default_rng(7)
    reqs = [_request(rng, npix, det, L, seg) for npix, det, L, seg in
            [(64, 16, 3, False), (96, 24, 5, True), (64, 16, 3, False), (128, 32, 2, False),
             (64, 16, 3, False), (96, 24, 5, True), (128, 20, 1, True), (64, 16, 3, False)]]
    with serving.PSFServer(streams=3, max_batch=2, precision='split') as srv:
        futs = [srv.submit(r) for r in reqs]
        results = [f.result(timeout=120) for f in futs]
        stats = dict(srv.stats)
    assert stats['completed'] == len(reqs)
    assert stats['batched'] == len(reqs)
    assert stats['launches'] < len(reqs)          # same-plan requests were batched
    # every launch either had the GPU to itself (autotuned tile width) or
    # shared it with launches in flight (the 256-wide throughput tile)
    assert stats['tuned_tile_launches'] + stats['shared_gpu_launches'] == stats['launches']
    assert stats['tuned_tile_launches'] >= 1      # the first launch found the GPU idle
    for r, img in zip(reqs, results):
        ref = _alone(r)
        assert img.shape == ref.shape
        assert lo.peak_normalised_error(img, ref) < TOL
    # alone through a fresh server (no mix) gives the same image within tolerance
    with serving.PSFServer(streams=1, max_batch=1, precision='split') as srv:
        solo = [srv.submit(r).result(timeout=120) for r in reqs[:3]]
    for a, b in zip(solo, results[:3]):
        assert lo.peak_normalised_error(a, b) < TOL


def test_budget_rejects_oversize_and_cancel(cuda_device):
    rng = np.random.default_rng(8)
    with serving.PSFServer(hbm_budget=64 << 20, streams=1, max_batch=1) as srv:
        big = _request(rng, 512, 256, 64)            # needs far more than 64 MB
        f = srv.submit(big)
        with pytest.raises(MemoryError):
            f.result(timeout=120)
        small = _request(rng, 64, 16, 2)
        assert lo.peak_normalised_error(srv.submit(small).result(timeout=120), _alone(small)) < TOL
    with serving.PSFServer(streams=1, max_batch=1) as srv:
        reqs = [_request(rng, 64, 16, 2) for _ in range(4)]
        futs = [srv.submit(r) for r in reqs]
        srv.cancel(reqs[-1])
        for f in futs[:-1]:
            f.result(timeout=120)
        assert futs[-1].cancelled() or futs[-1].done()


def test_eviction_under_budget(cuda_device):
    rng = np.random.default_rng(9)
    reqs = [_request(rng, 64, 16, L) for L in (2, 3, 4, 5, 6)]
    one = serving.plan_bytes_estimate((64, 64), (0, 0, 58, 58), (32, 32), 6, 0, 'split')
    with serving.PSFServer(hbm_budget=int(2.5 * one), streams=1, max_batch=1,
                           grid=np.zeros(0)) as srv:
        out = [srv.submit(r).result(timeout=120) for r in reqs]
        assert srv.stats['evicted'] >= 1
    for r, img in zip(reqs, out):
        assert lo.peak_normalised_error(img, _alone(r)) < TOL


def test_grid_plans_serve_wavelength_subsets(cuda_device):
    # requests whose wavelengths lie on the server grid share one resident
    # plan per optics geometry (DFT-matrix cache) whatever their subset
    rng = np.random.default_rng(10)
    grid = np.linspace(400e-9, 1000e-9, 16)
    reqs = []
    for L in (1, 3, 5, 16, 2, 7):
        r = _request(rng, 64, 16, L)
        idx = np.sort(rng.choice(16, L, replace=False))
        r.wavelengths, r.weights = grid[idx], rng.uniform(0.5, 1.5, L)
        reqs.append(r)
    with serving.PSFServer(streams=2, max_batch=2, grid=grid) as srv:
        out = [f.result(timeout=120) for f in [srv.submit(r) for r in reqs]]
        stats = dict(srv.stats)
    assert stats['plans_built'] == 1
    for r, img in zip(reqs, out):
        assert lo.peak_normalised_error(img, _alone(r)) < TOL


def test_allocation_failure_fails_only_its_launch(cuda_device):
    # a launch whose buffers cannot be allocated (made on the host through the
    # test hook) fails its requests with the allocation error; the server
    # keeps its stream and slot accounting and serves the following requests
    import torch
    rng = np.random.default_rng(9)
    with serving.PSFServer(streams=1, max_batch=1, precision='split') as srv:
        srv.inject_allocation_failures(1)
        first = _request(rng, 64, 16, 2)
        with pytest.raises(torch.cuda.OutOfMemoryError):
            srv.submit(first).result(timeout=120)
        later = [_request(rng, 64, 16, 2) for _ in range(3)]
        out = [srv.submit(r).result(timeout=120) for r in later]
        stats = dict(srv.stats)
    assert stats['failed'] == 1 and stats['completed'] == 3
    for r, img in zip(later, out):
        assert lo.peak_normalised_error(img, _alone(r)) < TOL


def test_server_tuner_cache_file(cuda_device, tmp_path):
    # PSFServer(tuner_cache=path) writes the tile widths it decided on close
    # and a later server loads them
    import json
    from lentil_gb300 import tuner
    path = tmp_path / 'tiles.json'
    rng = np.random.default_rng(10)
    tuner.clear()
    with serving.PSFServer(streams=1, max_batch=1, precision='split', tuner_cache=str(path)) as srv:
        for _ in range(6):                  # one launch class, tuned while the GPU is idle
            srv.submit(_request(rng, 64, 16, 2)).result(timeout=120)
        decided = tuner.entries()
    doc = json.loads(path.read_text())
    assert len(doc['classes']) == decided >= 1
    tuner.clear()
    with serving.PSFServer(streams=1, max_batch=1, precision='split', tuner_cache=str(path)):
        assert tuner.entries() == decided


def test_resident_pupil_and_modal_opd(cuda_device):
    # requests naming a device-resident pupil and giving their OPD as
    # coefficients of a resident Zernike basis (expanded on the GPU) equal
    # the same requests carrying the arrays, and the oracle
    rng = np.random.default_rng(11)
    npix = 96
    amp = lg.normalize_power(lg.circle((npix, npix), npix * 0.45))
    support = amp > 0
    rho, th = lg.zernike_coordinates(support)
    basis = np.asarray([lg.zernike(support, j, rho=rho, theta=th) for j in range(2, 12)])
    basis32 = basis.astype(np.float32)
    with serving.PSFServer(streams=2, max_batch=2, precision='split') as srv:
        pup, bas = srv.resident_pupil(amp), srv.resident_basis(basis32)
        modal, raw = [], []
        for L in (3, 5, 3, 1):
            c = rng.normal(0, 30e-9, 10)
            wl = np.linspace(450e-9, 900e-9, L) if L > 1 else np.array([650e-9])
            w = np.full(L, 1.0 / L)
            args = (wl, w, 1.0 / npix, 10.0, 5e-6 * 256 / npix, 24)
            modal.append(serving.PSFRequest(pup, c, *args, opd_basis=bas))
            raw.append(serving.PSFRequest(amp, np.tensordot(c, basis32.astype(np.float64), 1), *args))
        out_m = [f.result(timeout=120) for f in [srv.submit(r) for r in modal]]
        out_r = [f.result(timeout=120) for f in [srv.submit(r) for r in raw]]
    for r, a, b in zip(raw, out_m, out_r):
        assert lo.peak_normalised_error(a, b) < TOL
        assert lo.peak_normalised_error(a, _alone(r)) < TOL
    with pytest.raises(ValueError):
        serving.PSFRequest(pup, np.zeros(3), np.array([6e-7]), np.ones(1), 1.0 / npix, 10.0, 5e-6,
                           24, opd_basis=bas)
