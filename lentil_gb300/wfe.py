"""Wavefront-error and source-spectrum generators.

``power_spectrum`` filters seeded white noise on the GPU
(``lgb_power_spectrum``); the noise itself is drawn with numpy's generator
from the same seed so that the surface matches lentil's.  The blackbody
weights are a few host-side numbers."""
import numpy as np
import torch

from . import _device as dv
from . import _lib

# lentil/radiometry.py:12-14
_H = 6.62606957e-34
_C = 299792456
_K = 1.3806488e-23


def power_spectrum(mask, pixelscale, rms, half_power_freq, exp, seed=None):
    """Seeded 1/f^exp surface error, masked and scaled to ``rms`` over the
    nonzero pixels (lentil/wfe.py:8-70; Sidick 2009 PSD filter).  lentil's
    frequency grid is only consistent for square masks; numpy masks give a
    numpy OPD, CUDA tensors a CUDA tensor."""
    n, m = (int(x) for x in (mask.shape if dv.is_tensor(mask) else np.shape(mask)))
    if n != m:
        raise ValueError(f'power_spectrum needs a square mask, got {(n, m)}')
    rng = np.random.default_rng(seed)
    noise = dv.to_device(rng.normal(size=[n, m]), torch.float64)
    mask_d = dv.to_device(mask, torch.float64)
    out = torch.empty((n, m), dtype=torch.float64, device=noise.device)
    ws = dv.workspace(_lib.load().lgb_power_spectrum_workspace_size(n))
    _lib.call('lgb_power_spectrum', noise.data_ptr(), mask_d.data_ptr(), n, float(pixelscale),
              float(rms), float(half_power_freq), float(exp), out.data_ptr(), ws.data_ptr(),
              ws.numel(), dv.stream_ptr())
    return out if dv.is_tensor(mask) else dv.to_host(out)


def blackbody_photlam(wave_nm, temp):
    """Planck photon radiance (photons s^-1 m^-2 sr^-1 nm^-1) at ``wave_nm``;
    the default ``valueunit='photlam'`` of lentil's Blackbody
    (lentil/radiometry.py:932-971, 1226-1263)."""
    lam = np.asarray(wave_nm, float) * 1e-9
    energy = 2 * _H * _C ** 2 / (lam ** 5 * (np.exp(_H * _C / (lam * _K * temp)) - 1))
    return energy * lam / (_H * _C) * 1e-9
