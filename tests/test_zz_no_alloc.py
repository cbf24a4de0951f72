"""lgb_dft2_noalloc: the complex128 dft2 for callers that cannot allocate
device memory at call time (fixed-budget control loops, work issued under
stream capture).  It must give the same transform as lgb_dft2 with a
caller-provided workspace, call after call, while drawing all of its scratch
(the GEMMs' split-K partial products included) from the library's fixed
device array, so the device's stream-ordered pool sees no allocation.
Collected last on purpose (file name)."""
import ctypes

import numpy as np
import pytest
import torch

from lentil_gb300 import _lib
from oracle import lentil_oracle as lo

pytestmark = pytest.mark.gpu

TOL = 1e-12   # peak-normalised, the complex128 parity tolerance of the suite


def _with_workspace(lib, f, M, N, args):
    m, n = f.shape
    F = torch.empty((M, N), dtype=torch.complex128, device='cuda')
    nbytes = lib.lgb_dft2_workspace_size(m, n, M, N, _lib.FP64)
    ws = torch.empty(nbytes, dtype=torch.uint8, device='cuda')
    _lib.check(lib.lgb_dft2(f.data_ptr(), m, n, F.data_ptr(), M, N, *args, 1, _lib.FP64,
                            ws.data_ptr(), nbytes, torch.cuda.current_stream().cuda_stream))
    return F


def _no_alloc(lib, f, M, N, args):
    m, n = f.shape
    F = torch.empty((M, N), dtype=torch.complex128, device='cuda')
    _lib.check(lib.lgb_dft2_noalloc(f.data_ptr(), m, n, F.data_ptr(), M, N, *args, 1,
                                    torch.cuda.current_stream().cuda_stream))
    return F


def _pool(lib, reset=False):
    """(reserved, reserved high, used, used high) of the device's default pool."""
    out = (ctypes.c_ulonglong * 4)()
    _lib.check(lib.lgb_mempool_usage(torch.cuda.current_device(), int(reset), out))
    return list(out)


def test_no_alloc_matches_workspace_entry_point(cuda_device):
    lib = _lib.load()
    rng = np.random.default_rng(11)
    cases = [((37, 29), (41, 33), (0.0123, -0.0071, 3.25, -7.5, -4.5, 2.0)),
             ((64, 48), (80, 72), (0.004, 0.006, 0.5, -1.0, 3.0, -2.0))]
    for (m, n), (M, N), args in cases:          # two calls in a row, same scratch
        f_np = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
        f = torch.as_tensor(f_np, device='cuda')
        got = _no_alloc(lib, f, M, N, args).cpu().numpy()
        want = _with_workspace(lib, f, M, N, args).cpu().numpy()
        assert lo.peak_normalised_error(got, want) < TOL
        ref = lo.dft2(f_np, args[0:2], shape=(M, N), shift=args[2:4], offset=args[4:6])
        assert lo.peak_normalised_error(got, ref) < TOL


def test_no_alloc_allocates_nothing(cuda_device):
    """64 x 64 -> 128 x 128 is two output tiles of 64 x 64 with K = 64, a size
    at which the FP64 GEMM splits K: the workspace entry takes the partials
    from the stream-ordered pool (the control below), the allocation-free
    entry from its fixed array, so the pool's high-water mark stays put."""
    lib = _lib.load()
    rng = np.random.default_rng(12)
    args = (0.0031, 0.0027, 1.5, -2.0, 0.5, 1.0)
    f_np = rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))
    f = torch.as_tensor(f_np, device='cuda')
    F1 = torch.empty((128, 128), dtype=torch.complex128, device='cuda')
    F2 = torch.empty_like(F1)
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    before = _pool(lib, reset=True)
    for F in (F1, F2):                          # two calls in a row
        _lib.check(lib.lgb_dft2_noalloc(f.data_ptr(), 64, 64, F.data_ptr(), 128, 128, *args, 1,
                                        stream))
    torch.cuda.synchronize()
    after = _pool(lib)
    assert after[3] == before[2], f'pool used high-water mark moved: {before} -> {after}'
    assert after[1] == before[0], f'pool reserved high-water mark moved: {before} -> {after}'
    # control: the same transform with a caller workspace splits K into pool memory
    _pool(lib, reset=True)
    want = _with_workspace(lib, f, 128, 128, args)
    torch.cuda.synchronize()
    ctl = _pool(lib)
    assert ctl[3] > before[2], 'control: the workspace entry did not split K at this size'
    want = want.cpu().numpy()
    ref = lo.dft2(f_np, args[0:2], shape=(128, 128), shift=args[2:4], offset=args[4:6])
    for F in (F1, F2):
        got = F.cpu().numpy()
        assert lo.peak_normalised_error(got, want) < TOL
        assert lo.peak_normalised_error(got, ref) < TOL


def test_no_alloc_rejects_oversize(cuda_device):
    lib = _lib.load()
    st = lib.lgb_dft2_noalloc(None, 1024, 1024, None, 1024, 1024, 0.001, 0.001, 0, 0, 0, 0, 1,
                              None)
    assert st == _lib.EINVAL
    assert b'scratch' in lib.lgb_last_error()
