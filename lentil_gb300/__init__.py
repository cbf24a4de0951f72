"""lentil_gb300: lentil's far-field MFT diffraction path on one GB300 (sm_103a).

Drop-in API of the path (same names and arguments as lentil 0.8.8):
``fourier.dft2``/``idft2``, ``propagate_dft``, ``propagate_fft``, ``Wavefront``, ``Plane``,
``Pupil``, ``Image``, ``Tilt``, ``field`` helpers and ``detector.pixelate``,
plus the fused ``broadband_psf``/``PSFPlan``.  Every transform, phasor,
overlap-add, tilt fit, pixelation and Zernike/power-spectrum generation runs
in the library's own CUDA kernels (``liblentil_gb300.so``, C ABI in
``include/lentil_gb300.h``); there is no CPU fallback.  The aperture shapes
are host-side numpy helpers for building inputs, as in lentil.
``tuner`` controls the tile-shape autotuner of the tensor-core MFT.
"""
__version__ = '0.1.0'

from .ptype import ptype, none, pupil, image, tilt, transform
from . import fourier
from . import detector
from . import field
from .field import Field
from .plane import Plane, Pupil, Image, Tilt, DispersiveTilt, Grism
from .wavefront import Wavefront
from .propagate import propagate_dft, propagate_fft, scratch_shape
from .broadband import broadband_psf, PSFPlan
from .shapes import circle, hexagon, rectangle, spider, hex_segments
from .util import boundary, centroid, normalize_power, pad
from .zernike import zernike, zernike_compose, zernike_basis, zernike_coordinates
from .wfe import power_spectrum
from . import _lib
from . import tuner
