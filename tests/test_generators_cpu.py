"""Input generators without a GPU: the oracle's Zernike / PSD restatements
and the host-side aperture shapes against lentil 0.8.8's golden outputs
(tests/golden/generators.npz), and the Zernike index maps of lentil_gb300
against lentil's (lentil/zernike.py:348-441)."""
import importlib

import numpy as np
import pytest

import lentil_gb300 as lg
from oracle import lentil_oracle as lo

lz = importlib.import_module('lentil_gb300.zernike')    # the module (the package exports the function)


def test_oracle_zernike_golden(golden):
    g = golden('generators')
    m = lg.circle((64, 64), 30)
    assert np.max(np.abs(lo.zernike_compose(m, g['zcoeffs']) - g['zcompose'])) <= \
        1e-12 * np.max(np.abs(g['zcompose']))
    mm = g['hexseg'][4]
    rho, theta = lo.zernike_coordinates(mm)
    assert np.allclose(rho, g['zcoord_rho'], rtol=0, atol=1e-13)
    assert np.allclose(theta, g['zcoord_theta'], rtol=0, atol=1e-13)
    seg = lo.zernike_compose(mm, [1e-8, 2e-8, -3e-8], rho=rho, theta=theta)
    assert np.max(np.abs(seg - g['zcompose_seg'])) <= 1e-12 * np.max(np.abs(g['zcompose_seg']))


def test_oracle_power_spectrum_golden(golden):
    g = golden('generators')
    psd = lo.power_spectrum(lg.circle((64, 64), 30), 1 / 64, 25e-9, 8, 2, seed=7)
    assert np.max(np.abs(psd - g['psd'])) <= 1e-12 * np.max(np.abs(g['psd']))


@pytest.mark.parametrize('name,fn', [
    ('circle', lambda: lg.circle((64, 70), 20.3, shift=(1.5, -2.25))),
    ('circle_noaa', lambda: lg.circle((64, 64), 20, antialias=False)),
    ('hexagon', lambda: lg.hexagon((64, 64), 20, shift=(2, -3))),
    ('hexagon_rot', lambda: lg.hexagon((64, 64), 20, rotate=True)),
    ('rectangle', lambda: lg.rectangle((64, 64), 30, 12, shift=(3, 4), angle=30)),
    ('spider', lambda: lg.spider((64, 64), 3, angle=210)),
    ('hexseg', lambda: lg.hex_segments(rings=2, seg_radius=10, seg_gap=1)),
])
def test_shapes_golden(golden, name, fn):
    ref = golden('generators')[name]
    out = np.asarray(fn(), dtype=float)
    assert out.shape == ref.shape
    assert np.max(np.abs(out - ref)) <= 1e-12


def test_zernike_index_maps_match_lentil():
    for j in range(1, 232):
        assert lz.noll_to_nm(j) == lo.noll_to_nm(j), j
        assert lz.fringe_to_nm(j) == lo.fringe_to_nm(j), j
    for j in range(0, 232):
        assert lz.ansi_to_nm(j) == lo.ansi_to_nm(j), j
    for bad in (lambda: lz.noll_to_nm(0), lambda: lz.fringe_to_nm(0), lambda: lz.ansi_to_nm(-1)):
        with pytest.raises(ValueError):
            bad()


def test_zernike_radial_terms_match_lentil():
    rho = np.linspace(0, 1, 97)
    for n in range(0, 12):
        for m in range(-n, n + 1):
            want = lo.zernike_radial(n, m, rho)
            got = sum(a * rho ** p for a, p in lz.radial_terms(n, m)) if lz.radial_terms(n, m) else 0
            assert np.array_equal(np.asarray(got), np.asarray(want)), (n, m)

