"""Detector sampling on the GPU, drop-in for ``lentil.detector.pixel`` and
``lentil.detector.pixelate`` (lentil/detector.py:167-251)."""
import torch

from . import _device as dv
from . import _lib


def _run(name, img, oversample, out_shape):
    host = not dv.is_tensor(img)
    d = dv.to_device(img, torch.float64)
    if d.dim() != 2:
        raise ValueError(f'{name} expects a 2-D image')
    rows, cols = d.shape
    nbytes = _lib.load().lgb_pixel_workspace_size(int(rows), int(oversample))
    ws = dv.workspace(nbytes)
    out = torch.empty(out_shape(rows), dtype=torch.float64, device=d.device)
    _lib.call('lgb_' + name, d.data_ptr(), int(rows), int(cols), int(oversample), out.data_ptr(),
              ws.data_ptr(), nbytes, dv.stream_ptr())
    return dv.to_host(out) if host else out


def pixel(img, oversample=1):
    """Apply the square-pixel MTF sinc(f*oversample) (lentil/detector.py:167-222)."""
    return _run('pixel', img, oversample, lambda n: (n, n))


def pixelate(img, oversample):
    """Pixel MTF, then cubic-spline resampling to native pixels
    (lentil/detector.py:225-251, lentil/util.py:261-349): an
    ceil(N / oversample)-square image."""
    os_ = int(oversample)
    if os_ != oversample or os_ < 1:
        raise NotImplementedError('pixelate needs a positive integer oversample')
    size = _lib.load().lgb_pixelate_size
    return _run('pixelate', img, os_, lambda n: (size(int(n), os_),) * 2)
