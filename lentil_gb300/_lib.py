"""ctypes binding of ``liblentil_gb300.so`` (declared in include/lentil_gb300.h).

The library is built in-tree by ``lentil_gb300._build``.  There is no CPU
fallback: every entry of the diffraction path goes through this library and
raises if it cannot be loaded or no CUDA device is present.
"""
import ctypes
import os
import threading

from . import _build

OK, EINVAL, ETYPE, ECUDA, EUNSUPPORTED, ETIMEOUT, EWORKSPACE = range(7)
FP64, SPLIT_BF16, SPLIT_FP16 = 0, 1, 2

PRECISIONS = {'fp64': FP64, 'split-bf16': SPLIT_BF16, 'split-fp16': SPLIT_FP16,
              'split': SPLIT_FP16}

c_int, c_double, c_size_t, c_void_p = ctypes.c_int, ctypes.c_double, ctypes.c_size_t, ctypes.c_void_p
c_int64 = ctypes.c_int64


class PsfDesc(ctypes.Structure):
    """Mirror of ``lgb_psf_desc``."""
    _fields_ = [('H', c_int), ('W', c_int), ('r0', c_int), ('c0', c_int), ('m', c_int), ('n', c_int),
                ('offset_r', c_double), ('offset_c', c_double), ('M', c_int), ('N', c_int),
                ('out_rows', c_int), ('out_cols', c_int), ('win_r0', c_int), ('win_c0', c_int),
                ('n_wavelengths', c_int), ('wavelengths', c_void_p), ('alpha_r', c_void_p),
                ('alpha_c', c_void_p), ('shift_r', c_void_p), ('shift_c', c_void_p),
                ('batch', c_int), ('precision', c_int)]


# name -> (restype, argtypes); every symbol of include/lentil_gb300.h
SIGNATURES = {
    'lgb_last_error': (ctypes.c_char_p, []),
    'lgb_version': (c_int, []),
    'lgb_mempool_usage': (c_int, [c_int, c_int, ctypes.POINTER(ctypes.c_ulonglong)]),
    'lgb_test_stall_tma': (c_int, [c_int, c_int, c_double]),
    'lgb_dft2_matrices': (c_int, [c_int, c_int, c_int, c_int, c_double, c_double, c_double,
                                  c_double, c_double, c_double, c_void_p, c_void_p, c_void_p]),
    'lgb_dft2_workspace_size': (c_size_t, [c_int, c_int, c_int, c_int, c_int]),
    'lgb_dft2': (c_int, [c_void_p, c_int, c_int, c_void_p, c_int, c_int, c_double, c_double,
                         c_double, c_double, c_double, c_double, c_int, c_int, c_void_p, c_size_t,
                         c_void_p]),
    'lgb_dft2_status': (c_int, [c_void_p, c_void_p]),
    'lgb_dft2_batch_workspace_size': (c_size_t, [c_int, c_int, c_int, c_int, c_int, c_int]),
    'lgb_dft2_batch': (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_int, c_int, c_double,
                               c_double, c_double, c_double, c_double, c_double, c_int, c_int,
                               c_void_p, c_size_t, c_void_p]),
    'lgb_dft2_noalloc': (c_int, [c_void_p, c_int, c_int, c_void_p, c_int, c_int, c_double,
                                 c_double, c_double, c_double, c_double, c_double, c_int,
                                 c_void_p]),
    'lgb_idft2_workspace_size': (c_size_t, [c_int, c_int, c_int, c_int, c_int]),
    'lgb_idft2': (c_int, [c_void_p, c_int, c_int, c_void_p, c_int, c_int, c_double, c_double,
                          c_double, c_double, c_int, c_int, c_void_p, c_size_t, c_void_p]),
    'lgb_phasor': (c_int, [c_void_p, c_double, c_void_p, c_void_p, c_double, c_int, c_int, c_int,
                           c_int, c_int, c_int, c_double, c_void_p, c_void_p]),
    'lgb_field_insert': (c_int, [c_void_p, c_int, c_int, c_int64, c_int64, c_void_p, c_int, c_int,
                                 c_double, c_int, c_void_p]),
    'lgb_field_multiply': (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_int, c_int, c_int,
                                   c_void_p, c_int, c_int, c_void_p]),
    'lgb_pixel_workspace_size': (c_size_t, [c_int, c_int]),
    'lgb_pixel': (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_size_t, c_void_p]),
    'lgb_pixelate_size': (c_int, [c_int, c_int]),
    'lgb_psf_plan_set_tile': (c_int, [c_void_p, c_int]),
    'lgb_dft2_plan_create': (c_int, [c_int, c_int, c_int, c_int, c_double, c_double, c_double,
                                     c_double, c_double, c_double, c_int, c_int, c_void_p,
                                     ctypes.POINTER(c_void_p)]),
    'lgb_dft2_plan_size': (c_size_t, [c_int, c_int, c_int, c_int, c_int]),
    'lgb_dft2_plan_create_in': (c_int, [c_int, c_int, c_int, c_int, c_double, c_double, c_double,
                                        c_double, c_double, c_double, c_int, c_int, c_void_p,
                                        c_size_t, c_void_p, ctypes.POINTER(c_void_p)]),
    'lgb_dft2_plan_bytes': (c_size_t, [c_void_p]),
    'lgb_dft2_plan_workspace_size': (c_size_t, [c_void_p, c_int]),
    'lgb_dft2_plan_execute': (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_size_t,
                                      c_void_p]),
    'lgb_dft2_plan_status': (c_int, [c_void_p, c_void_p]),
    'lgb_dft2_plan_inject_status': (c_int, [c_void_p, c_int, c_void_p]),
    'lgb_basis_expand': (c_int, [c_void_p, c_void_p, c_int, c_size_t, c_void_p, c_void_p]),
    'lgb_basis_project_workspace_size': (c_size_t, [c_int]),
    'lgb_basis_project': (c_int, [c_void_p, c_void_p, c_int, c_size_t, c_void_p, c_void_p,
                                  c_size_t, c_void_p]),
    'lgb_basis_expand_stack': (c_int, [c_void_p, c_void_p, c_int, c_size_t, c_void_p, c_int,
                                       c_void_p, c_void_p]),
    'lgb_basis_project_stack': (c_int, [c_void_p, c_void_p, c_int, c_int, c_size_t, c_void_p,
                                        c_void_p, c_size_t, c_void_p]),
    'lgb_sq_error_workspace_size': (c_size_t, []),
    'lgb_sq_error': (c_int, [c_void_p, c_void_p, c_size_t, c_void_p, c_void_p, c_size_t, c_void_p]),
    'lgb_sq_error_grad': (c_int, [c_void_p, c_void_p, c_size_t, c_void_p, c_void_p, c_void_p]),
    'lgb_phasor_stack': (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_int,
                                 c_int, c_double, c_int, c_void_p, c_void_p]),
    'lgb_dft2_plan_destroy': (c_int, [c_void_p]),
    'lgb_tuner_set_mode': (c_int, [c_int]),
    'lgb_tuner_force_tile': (c_int, [c_int]),
    'lgb_tuner_clear': (None, []),
    'lgb_tuner_entries': (c_int, []),
    'lgb_tuner_lookup': (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_int]),
    'lgb_tuner_last_tile': (c_int, []),
    'lgb_tuner_export': (c_int, [c_void_p, c_int]),
    'lgb_tuner_import': (c_int, [c_void_p, c_int]),
    'lgb_pixelate': (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_size_t,
                             c_void_p]),
    'lgb_ptt_normal_workspace_size': (c_size_t, [c_int]),
    'lgb_ptt_normal': (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_double, c_double,
                               c_void_p, c_void_p, c_size_t, c_void_p]),
    'lgb_remove_tilt': (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_double, c_double,
                                c_void_p, c_void_p, c_void_p]),
    'lgb_power_spectrum_workspace_size': (c_size_t, [c_int]),
    'lgb_power_spectrum': (c_int, [c_void_p, c_void_p, c_int, c_double, c_double, c_double,
                                   c_double, c_void_p, c_void_p, c_size_t, c_void_p]),
    'lgb_zernike_workspace_size': (c_size_t, []),
    'lgb_zernike_coordinates': (c_int, [c_void_p, c_int, c_int, c_int, c_double, c_double,
                                        c_double, c_void_p, c_void_p, c_void_p, c_size_t,
                                        c_void_p]),
    'lgb_zernike_eval': (c_int, [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p, c_int, c_int,
                                 c_void_p, c_int, c_void_p]),
    'lgb_abs2': (c_int, [c_void_p, c_void_p, c_size_t, c_void_p]),
    'lgb_intensity_adjoint': (c_int, [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    'lgb_phasor_adjoint': (c_int, [c_void_p, c_void_p, c_int, c_int, c_double, c_void_p, c_int,
                                   c_int, c_int, c_void_p]),
    'lgb_psf_plan_create': (c_int, [ctypes.POINTER(PsfDesc), ctypes.POINTER(c_void_p), c_void_p]),
    'lgb_psf_plan_bytes': (c_size_t, [c_void_p]),
    'lgb_psf_plan_size': (c_size_t, [ctypes.POINTER(PsfDesc)]),
    'lgb_psf_plan_create_in': (c_int, [ctypes.POINTER(PsfDesc), c_void_p, c_size_t,
                                       ctypes.POINTER(c_void_p), c_void_p]),
    'lgb_psf_execute': (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    'lgb_psf_execute_batch': (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_int, c_void_p]),
    'lgb_psf_execute_subset': (c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p,
                                       c_void_p, c_void_p, c_int, c_void_p]),
    'lgb_psf_execute_workspace_size': (c_size_t, [c_void_p, c_int, c_int]),
    'lgb_psf_execute_ws': (c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    'lgb_psf_plan_status': (c_int, [c_void_p, c_void_p]),
    'lgb_psf_plan_destroy': (c_int, [c_void_p]),
    'lgb_psf_plan_profile': (c_int, [c_void_p, c_int]),
    'lgb_psf_plan_kernel_times': (c_int, [c_void_p, ctypes.POINTER(c_double),
                                          ctypes.POINTER(c_int), c_int]),
}
PROFILE_SLOTS = ('phasor', 'mft_stage1', 'mft_stage2', 'other')

_lock = threading.Lock()
_lib = None


class LentilGpuError(RuntimeError):
    """A CUDA failure inside the library."""


class DeviceTimeout(LentilGpuError):
    """A bounded device-side wait expired; the results of the call are invalid."""


_EXC = {EINVAL: ValueError, ETYPE: TypeError, ECUDA: LentilGpuError,
        EUNSUPPORTED: NotImplementedError, ETIMEOUT: DeviceTimeout, EWORKSPACE: ValueError}


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load (building first if needed) the CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing and not _build.up_to_date():
            _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f'lentil_gb300 CUDA library missing: {path}')
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status):
    """Raise the exception lentil raises for the same condition."""
    if status == OK:
        return
    msg = load().lgb_last_error().decode(errors='replace')
    raise _EXC.get(status, LentilGpuError)(msg)


def call(name, *args):
    check(getattr(load(), name)(*args))


def precision_code(precision):
    try:
        return PRECISIONS[precision]
    except KeyError:
        raise ValueError(f"unknown precision {precision!r}; expected one of {sorted(PRECISIONS)}")
