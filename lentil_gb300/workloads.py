"""Seeded synthetic inputs of the benchmark workloads (host-side numpy).

``broadband_segmented`` builds the broadband segmented PSF workload: a
1024 x 1024 pupil of 18 hexagonal segments (two rings around an empty
centre, 2 px gaps), per-segment piston/tip/tilt ~ N(0, 50 nm) on each
segment's own Zernike coordinates, global Noll 2-22 ~ N(0, 15 nm),
64 wavelengths uniform over 500-900 nm weighted by a 5800 K blackbody
(photon units, normalised), a 1 m aperture over the pupil grid, f = 10 m,
5 um detector pixels, 512 x 512 detector at oversample 2.

``monochromatic_circle`` builds the monochromatic 256 x 256 circular
pupil (diameter 256 px = 1 m, f = 10 m), Noll 2-11 ~ N(0, 20 nm) at
650 nm onto a 128 x 128 detector of 5 um pixels at oversample 2.
"""
import numpy as np

from . import shapes, util
from .wfe import blackbody_photlam
from .zernike import zernike_basis, zernike_compose, zernike_coordinates


class Workload:
    """Pupil geometry, OPD basis and spectrum of one benchmark case."""

    def __init__(self, name, amp, mask3d, opd_basis, coeff_sigma, wavelengths, weights,
                 pixelscale_in, focal_length, det_pixelscale, det_shape, oversample, seed):
        self.name = name
        self.amp = amp                  # amplitude, mask applied, power normalised
        self.mask3d = mask3d            # (S, H, W) segment masks or None
        self.opd_basis = opd_basis      # (K, H, W) float32 OPD modes
        self.coeff_sigma = coeff_sigma  # (K,) metres rms per mode
        self.wavelengths = wavelengths
        self.weights = weights
        self.pixelscale_in = pixelscale_in
        self.focal_length = focal_length
        self.det_pixelscale = det_pixelscale
        self.det_shape = det_shape
        self.oversample = oversample
        self.seed = seed

    @property
    def plane_shape(self):
        return self.amp.shape

    def opds(self, count, seed=None):
        """``count`` seeded OPD maps (float64, metres)."""
        rng = np.random.default_rng(self.seed if seed is None else seed)
        c = rng.normal(0.0, 1.0, (count, len(self.coeff_sigma))) * self.coeff_sigma[None, :]
        K, H, W = self.opd_basis.shape
        out = (c.astype(np.float32) @ self.opd_basis.reshape(K, H * W)).reshape(count, H, W)
        return out.astype(np.float64)


def broadband_segmented(npix=1024, n_wavelengths=64, seed=2, seg_radius=None, basis=None):
    """The broadband segmented workload (see module docstring).  ``basis``
    evaluates Zernike modes (``zernike_basis`` signature); the default runs
    on the GPU, a host implementation can stand in where no GPU is used."""
    basis = zernike_basis if basis is None else basis
    if seg_radius is None:
        seg_radius = 116.8 * npix / 1024
    segs = shapes.hex_segments(rings=2, seg_radius=seg_radius, seg_gap=2)
    segs = np.asarray([util.pad(s, (npix, npix)) for s in segs])
    gmask = segs.sum(axis=0)
    amp = util.normalize_power(gmask)
    modes, sigma = [], []
    for s in segs:                                # piston, tip, tilt of each segment
        modes.extend(np.asarray(basis(s, [1, 2, 3]), dtype=np.float32))
        sigma.extend([50e-9] * 3)
    modes.extend(np.asarray(basis(gmask, list(range(2, 23))), dtype=np.float32))  # Noll 2-22
    sigma.extend([15e-9] * 21)
    wl_nm = np.linspace(500.0, 900.0, n_wavelengths)
    w = blackbody_photlam(wl_nm, 5800.0)
    return Workload('broadband_segmented', amp, segs, np.asarray(modes), np.asarray(sigma),
                    wl_nm * 1e-9, w / w.sum(), 1.0 / npix, 10.0, 5e-6, npix // 2, 2, seed)


def monochromatic_circle(seed=1, basis=None):
    """The monochromatic circular-pupil workload (see module docstring)."""
    basis = zernike_basis if basis is None else basis
    npix = 256
    amp = util.normalize_power(shapes.circle((npix, npix), npix // 2, antialias=False))
    modes = np.asarray(basis(amp, list(range(2, 12))), dtype=np.float32)
    return Workload('monochromatic_circle', amp, None, modes, np.full(10, 20e-9),
                    np.array([650e-9]), np.array([1.0]), 1.0 / npix, 10.0, 5e-6, 128, 2, seed)


def large_segmented(npix=4096, n_wavelengths=32, seed=5, tilt_lambda_d=50.0):
    """Large oversampled broadband workload: ``npix``^2 pupil of the 18-hex
    segmented aperture (gaps 2 px per 1024) with a central obscuration of 20 %
    of the diameter and 3 spider vanes 8 px wide at 90/210/330 degrees; OPD =
    Noll 2-22 N(0, 15 nm) + a seeded 1/f^2 PSD surface of 25 nm rms + a
    global tilt of ``tilt_lambda_d`` lambda/D (at 800 nm) that fit_tilt turns
    into an output shift; 32 wavelengths over 600-1000 nm with 5800 K
    blackbody weights; 1024^2 detector at oversample 4 (scaled with npix),
    then pixelated.  Returns (Workload, 2-D mask, opd with the tilt)."""
    scale = npix / 1024
    segs = shapes.hex_segments(rings=2, seg_radius=116.8 * scale, seg_gap=2 * scale)
    gmask = util.pad(np.sum(segs, axis=0), (npix, npix))
    obsc = shapes.circle((npix, npix), 0.2 * npix / 2)
    mask = np.clip(gmask - obsc, 0, 1)
    for ang in (90, 210, 330):
        mask = mask * shapes.spider((npix, npix), 8 * scale, angle=ang)
    amp = util.normalize_power(mask)
    rng = np.random.default_rng(seed)
    support = mask > 0
    rho, theta = zernike_coordinates(support)
    opd = zernike_compose(support, np.r_[0.0, rng.normal(0, 15e-9, 21)], rho=rho, theta=theta)
    from .wfe import power_spectrum
    opd += power_spectrum(support, 1.0 / npix, 25e-9, 10.0, 2, seed=seed)
    # tilt of tilt_lambda_d lambda/D at 800 nm in a random direction: Noll
    # Z2/Z3 = 2 rho cos/sin, so a coefficient c gives 4c of OPD across D
    ang = rng.uniform(0, 2 * np.pi)
    c = tilt_lambda_d * 800e-9 / 4
    opd += zernike_compose(support, [0.0, c * np.cos(ang), c * np.sin(ang)], rho=rho, theta=theta)
    wl_nm = np.linspace(600.0, 1000.0, n_wavelengths)
    w = blackbody_photlam(wl_nm, 5800.0)
    wl = Workload('large_segmented', amp, None, np.zeros((0, npix, npix), np.float32),
                  np.zeros(0), wl_nm * 1e-9, w / w.sum(), 1.0 / npix, 10.0, 5e-6,
                  npix // 4, 4, seed)
    return wl, mask, opd
