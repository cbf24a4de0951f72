"""Rebuild the golden propagate scenarios as oracle objects (test helper)."""
import numpy as np

from oracle import lentil_oracle as lo


def propagate_kwargs(g, name):
    kw = {}
    for k in ('pixelscale', 'shape', 'prop_shape', 'oversample'):
        v = g[f'{name}_{k}']
        if not (v.ndim == 0 and v == -1):
            kw[k] = v.item() if v.ndim == 0 else tuple(v.tolist())
    if f'{name}_outmask' in g:
        kw['mask'] = g[f'{name}_outmask']
    return kw


def build_pupil(mod, g, name):
    """Pupil of module ``mod`` (oracle or product API) from fixture arrays."""
    amp, opd = g[f'{name}_amp'], g[f'{name}_opd']
    mask = g.get(f'{name}_mask')
    pl = mod.Pupil(amplitude=amp, opd=opd.copy(), mask=mask,
                   pixelscale=g[f'{name}_pixelscale_in'].tolist(),
                   focal_length=float(g[f'{name}_focal_length']))
    if bool(g[f'{name}_fit_tilt']):
        pl.fit_tilt(inplace=True)
    return pl


PROPAGATE_CASES = ['config1', 'tilt_fit0', 'tilt_fit1', 'outmask', 'nooutput', 'oddrect',
                   'seg_fit0', 'seg_fit1']


FFT_CASES = ['c1', 'odd', 'odd_scratch', 'crop']


def fft_case(mod, g, name):
    """(wavefront, propagate_fft kwargs, scratch or None) of a golden
    propagate_fft case, built with the plane classes of ``mod``."""
    pl = mod.Pupil(amplitude=g[f'{name}_amp'], opd=g[f'{name}_opd'],
                   pixelscale=g[f'{name}_pixelscale_in'].tolist(),
                   focal_length=float(g[f'{name}_focal_length']))
    wf = mod.Wavefront(float(g[f'{name}_wavelength'])) * pl
    shape = g[f'{name}_shape']
    kw = dict(pixelscale=g[f'{name}_pixelscale'].tolist(),
              shape=None if np.all(shape == -1) else tuple(np.broadcast_to(shape, (2,)).tolist()),
              oversample=int(g[f'{name}_oversample']))
    sshape = g[f'{name}_scratch']
    scratch = None if np.all(sshape == -1) else np.full(tuple(sshape), 7 + 0j)
    return wf, kw, scratch


def fft_field_crop(g, name, field):
    """The centre crop of a propagate_fft field that the golden case stores."""
    r0, c0 = (int(x) for x in g[f'{name}_field_crop_origin'])
    k = g[f'{name}_field_crop'].shape[0]
    return field[r0:r0 + k, c0:c0 + k]
