"""Host-side plane semantics (no GPU): lentil's extension protocol
(``__amp__``/``__opd__``/``__mask__`` overrides, freeze/thaw, ptypes;
lentil tests/test_plane.py:18-71,189-218) and the tilt planes' ``__shift__``
(Tilt, DispersiveTilt, Grism; lentil tests/test_plane.py:163-187,213-218),
the latter pinned to lentil's own outputs in tests/golden/tilt.npz."""
import warnings

import numpy as np
import pytest
import scipy.integrate

import lentil_gb300 as lg
from lentil_gb300 import plane as lgp


def test_default_plane():
    p = lg.Plane()
    assert p.pixelscale is None
    assert np.all(p.amplitude == 1)
    assert np.all(p.opd == 0)
    assert p.mask == p.amplitude


def test_amp_alias_and_error():
    assert lg.Plane(amp=10).amplitude == 10
    with pytest.raises(AttributeError):
        lg.Plane(amplitude=10, amp=10)


def test_overridden_hooks_are_used():
    class Custom(lg.Plane):
        def __amp__(self):
            return np.array(1)

        def __opd__(self):
            return np.array(2)

        def __mask__(self):
            return np.array(3)

    p = Custom()
    assert p.amplitude == 1 and p.opd == 2 and p.mask == 3


def test_opd_override_may_read_the_mask():
    class Custom(lg.Plane):
        def __opd__(self):
            return 2 * self.mask

        def __mask__(self):
            return 3

    assert Custom().opd == 6


def test_freeze_caches_and_thaw_releases():
    class Random(lg.Plane):
        def __opd__(self):
            return np.random.default_rng().uniform()

    p = Random()
    assert p.opd != p.opd
    p.freeze()
    a, b = p.opd, p.opd
    assert a == b
    with pytest.raises(RuntimeError):
        p.opd = 1.0
    with pytest.raises(RuntimeError):
        p.freeze()
    p.thaw()
    assert p.opd != a
    q = p.freeze(inplace=False)
    assert q is not p and q.frozen and not p.frozen


@pytest.mark.parametrize('cls,ptype', [(lg.Plane, lg.ptype(None)), (lg.Pupil, lg.pupil),
                                       (lg.Image, lg.image), (lgp._TiltBase, lg.tilt)])
def test_default_ptype(cls, ptype):
    assert cls().ptype == ptype


def test_tilt_ptype_overload():
    assert lgp._TiltBase(ptype=lg.pupil).ptype == lg.pupil


def test_tilt_shift_swaps_axes():
    t = lg.Tilt(x=2e-6, y=-3e-6)
    assert t.__shift__(xs=1.0, ys=2.0, z=10.0) == (1.0 + 3e-5, 2.0 - 2e-5)


@pytest.mark.parametrize('name', ['lin', 'steep', 'quad_disp', 'cubic_disp'])
def test_dispersive_tilt_golden(golden, name):
    g = golden('tilt')
    dt = lg.DispersiveTilt(trace=g[f'{name}_trace'], dispersion=g[f'{name}_dispersion'])
    got = np.array([[dt.__shift__(wavelength=lam, xs=s[0], ys=s[1]) for lam in g['wl']]
                    for s in g['starts']])
    ref = g[f'{name}_xy']
    if len(g[f'{name}_dispersion']) == 2:
        assert np.array_equal(got, ref)           # closed form, lentil's arithmetic
    else:
        # lentil's least-squares root vs the polished polynomial root
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_dispersive_tilt_center():
    dt = lg.DispersiveTilt(dispersion=[1, 650e-9], trace=[2, 0])
    x0, y0 = np.random.default_rng(7).uniform(-5, 5, 2)
    x, y = dt.__shift__(wavelength=650e-9, xs=x0, ys=y0)
    assert x == x0 and y == y0


def test_dispersive_tilt_shift():
    dt = lg.DispersiveTilt(trace=[1, 1], dispersion=[1, 650e-9])
    wave = 900e-9
    x, y = dt.__shift__(wavelength=wave)
    assert x == (wave - dt.dispersion[1]) / np.sqrt(2)
    assert y == 1 + x


def test_dispersive_tilt_class_attributes():
    class Custom(lg.DispersiveTilt):
        dispersion = [1, 0]
        trace = [1, 0]

    assert np.allclose(Custom().__shift__(1), np.sqrt(2) / 2)


@pytest.mark.parametrize('trace', [[400.0, 0.2, 0.0], [-3e5, 50.0, 0.1, 0.0], [5e-6]])
def test_dispersive_tilt_higher_order_trace(trace):
    # the point's arc length along the trace from x = 0 equals the dispersed
    # distance (checked with adaptive quadrature), and it lies on the trace
    dt = lg.DispersiveTilt(trace=trace, dispersion=[1e-3, 650e-9])
    slope = np.polyder(np.asarray(trace, float)) if len(trace) > 1 else np.zeros(1)
    for lam in (550e-9, 640e-9, 650e-9, 780e-9):
        d = (lam - 650e-9) / 1e-3
        x, y = dt.__shift__(wavelength=lam, xs=0.0, ys=0.0)
        s = scipy.integrate.quad(lambda u: np.sqrt(1 + np.polyval(slope, u) ** 2), 0, x,
                                 epsabs=0, epsrel=1e-13)[0]
        assert abs(s - d) <= 1e-13 * max(abs(d), 1e-9)
        assert y == np.polyval(trace, x)


def test_dispersion_needs_order_one():
    with pytest.raises(ValueError):
        lg.DispersiveTilt(trace=[1, 0], dispersion=[650e-9]).__shift__(wavelength=600e-9)


def test_grism_is_a_deprecated_dispersive_tilt():
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter('always')
        g = lg.Grism(trace=[0.3, 0], dispersion=[1e-3, 650e-9])
    assert any(issubclass(x.category, DeprecationWarning) for x in w)
    d = lg.DispersiveTilt(trace=[0.3, 0], dispersion=[1e-3, 650e-9])
    assert g.__shift__(wavelength=700e-9) == d.__shift__(wavelength=700e-9)


def test_shape_and_size_follow_the_mask_hooks():
    # a plane without a mask reads its mask's shape and rank from the
    # amplitude; a given mask or an overridden __mask__ (or __amp__) decides
    # them, as lentil's Plane.shape/size do (lentil/plane.py:173-201)
    a = np.zeros((40, 30))
    a[5:20, 3:25] = 1
    p = lg.Plane(amplitude=a)
    assert p._mask_is_amplitude() and p.shape == (40, 30) and p.size == 1
    assert np.array_equal(p.mask, a != 0)
    m3 = np.stack([a, a, a])
    q = lg.Plane(amplitude=a, mask=m3)
    assert not q._mask_is_amplitude() and q.shape == (40, 30) and q.size == 3

    class Masked(lg.Plane):
        def __mask__(self):
            return np.ones((2, 8, 9))

    r = Masked(amplitude=np.ones((8, 9)))
    assert not r._mask_is_amplitude() and r.shape == (8, 9) and r.size == 2

    class Amp(lg.Plane):
        def __amp__(self):
            return np.ones((6, 7))

    s = Amp()
    assert s._mask_is_amplitude() and s.shape == (6, 7) and s.size == 1
    assert lg.Plane(amplitude=3.0).shape == () and lg.Plane(amplitude=3.0).size == 1
