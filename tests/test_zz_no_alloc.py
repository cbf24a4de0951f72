"""lgb_dft2_noalloc: the complex128 dft2 for callers that cannot allocate
device memory at call time (fixed-budget control loops, work issued under
stream capture).  It must give the same transform as lgb_dft2 with a
caller-provided workspace, call after call, while drawing its scratch from
the library's fixed device array.  Collected last on purpose (file name)."""
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


def test_no_alloc_rejects_oversize(cuda_device):
    lib = _lib.load()
    st = lib.lgb_dft2_noalloc(None, 1024, 1024, None, 1024, 1024, 0.001, 0.001, 0, 0, 0, 0, 1,
                              None)
    assert st == _lib.EINVAL
    assert b'scratch' in lib.lgb_last_error()
