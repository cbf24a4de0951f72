"""Wavefront-error and source-spectrum generators (host-side numpy, input
preparation only)."""
import numpy as np

# lentil/radiometry.py:12-14
_H = 6.62606957e-34
_C = 299792456
_K = 1.3806488e-23


def power_spectrum(mask, pixelscale, rms, half_power_freq, exp, seed=None):
    """Seeded 1/f^exp surface error, masked and scaled to ``rms`` over the
    nonzero pixels (lentil/wfe.py:8-70; Sidick 2009 PSD filter)."""
    mask = np.asarray(mask)
    rng = np.random.default_rng(seed)
    n, m = mask.shape
    fy = (np.arange(m) - (np.floor(m / 2) + 1)) / m
    fx = (np.arange(n) - (np.floor(n / 2) + 1)) / n
    dr = np.hypot(fy[:, None], fx[None, :])
    f0 = half_power_freq * pixelscale / np.sqrt(m ** 2 + n ** 2)
    psd = 1.0 / (1.0 + (dr / f0) ** exp)
    psd[dr == 0] = 0
    psd = psd / psd.sum()
    filt = np.fft.fftshift(np.sqrt(psd))
    noise = rng.normal(size=[n, m])
    opd = np.real(np.fft.ifft2(np.fft.fft2(noise) * filt)) * np.sqrt(m * n)
    opd = opd * mask
    return opd * np.sqrt(np.count_nonzero(opd) / np.sum(np.abs(opd) ** 2)) * rms


def blackbody_photlam(wave_nm, temp):
    """Planck photon radiance (photons s^-1 m^-2 sr^-1 nm^-1) at ``wave_nm``;
    the default ``valueunit='photlam'`` of lentil's Blackbody
    (lentil/radiometry.py:932-971, 1226-1263)."""
    lam = np.asarray(wave_nm, float) * 1e-9
    energy = 2 * _H * _C ** 2 / (lam ** 5 * (np.exp(_H * _C / (lam * _K * temp)) - 1))
    return energy * lam / (_H * _C) * 1e-9
