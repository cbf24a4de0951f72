"""Host preparation of the broadband plan's merged field (no GPU): the
row-block parallel mask sum and amplitude product equal numpy's own
(lentil/plane.py:494-514 summed over segments)."""
import numpy as np
import pytest

from lentil_gb300 import broadband, shapes, util


def _segments(npix):
    segs = shapes.hex_segments(rings=2, seg_radius=116.8 * npix / 1024, seg_gap=2)
    return np.asarray([util.pad(s, (npix, npix)) for s in segs])


def test_summed_mask_is_numpys_sum():
    for npix in (64, 1024):                 # below and above the parallel threshold
        segs = _segments(npix)
        assert np.array_equal(broadband._summed_mask(segs), segs.sum(axis=0))
        b = segs > 0.5
        got = broadband._summed_mask(b)
        assert got.dtype == b.sum(axis=0).dtype and np.array_equal(got, b.sum(axis=0))


def test_dense_field_matches_numpy():
    import lentil_gb300 as lg
    segs = _segments(1024)
    g = segs.sum(axis=0)
    amp = util.normalize_power(g)
    opd = np.random.default_rng(3).normal(0, 1e-7, amp.shape)
    pup = lg.Pupil(amplitude=amp, opd=opd, mask=segs, pixelscale=1 / 1024, focal_length=10)
    s, amp_eff, o = broadband.dense_field(pup)
    assert s == util.boundary_slice(g)
    assert np.array_equal(amp_eff, amp * g)
    assert np.array_equal(o, opd)


@pytest.mark.filterwarnings('ignore:This process .* is multi-threaded:DeprecationWarning')
def test_host_pool_after_fork():
    # a child forked after the pool started gets a fresh pool, not dead threads
    import multiprocessing as mp
    segs = _segments(1024)
    broadband._summed_mask(segs)                      # the parent's pool is running
    ctx = mp.get_context('fork')
    with ctx.Pool(1) as pool:
        ok = pool.apply(_child_sum_ok, ())
    assert ok


def _child_sum_ok():
    segs = _segments(1024)
    return bool(np.array_equal(broadband._summed_mask(segs), segs.sum(axis=0)))
