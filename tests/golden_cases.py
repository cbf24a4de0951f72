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
