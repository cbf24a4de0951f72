"""The tensor-core MFT's bounded waits, run out on the GPU.

A one-shot test hook makes the next stage-1 launch arrive on one stage's
full barrier without issuing its TMA loads, so the MMA issuer's wait on that
barrier (and then every other role's) runs out after 1 ms.  The kernel must
record LGB_ETIMEOUT, retire what it issued and return: the entry's status
call reports the time-out, the GPU stays usable, and the next transform of
the same workspace is correct."""
import time

import numpy as np
import pytest
import torch

from lentil_gb300 import _lib
from oracle import lentil_oracle as lo

pytestmark = pytest.mark.gpu


def _dft2(lib, f, M, N, args, prec, ws):
    m, n = f.shape
    F = torch.empty((M, N), dtype=torch.complex128, device='cuda')
    st = lib.lgb_dft2(f.data_ptr(), m, n, F.data_ptr(), M, N, *args, 1, prec, ws.data_ptr(),
                      ws.numel(), torch.cuda.current_stream().cuda_stream)
    return st, F


@pytest.mark.parametrize('precision', ['split-bf16', 'split-fp16'])
def test_withheld_load_times_out_then_next_launch_is_correct(cuda_device, precision):
    lib = _lib.load()
    prec = _lib.PRECISIONS[precision]
    rng = np.random.default_rng(21)
    m, n, M, N = 300, 280, 256, 240
    args = (0.0021, 0.0023, 0.5, -1.5, 2.0, -3.0)
    f_np = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
    f = torch.as_tensor(f_np, device='cuda')
    nbytes = lib.lgb_dft2_workspace_size(m, n, M, N, prec)
    ws = torch.empty(nbytes, dtype=torch.uint8, device='cuda')
    stream = torch.cuda.current_stream().cuda_stream
    # warm: kernels loaded and the tile width of this launch class decided
    for _ in range(6):
        st, _ = _dft2(lib, f, M, N, args, prec, ws)
        assert st == _lib.OK
    assert lib.lgb_dft2_status(ws.data_ptr(), stream) == _lib.OK

    _lib.check(lib.lgb_test_stall_tma(0, 1, 1.0))     # item 0, K block 1, 1 ms bound
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st, _ = _dft2(lib, f, M, N, args, prec, ws)
    assert st == _lib.OK                               # the launch itself is accepted
    st = lib.lgb_dft2_status(ws.data_ptr(), stream)    # waits for the stream
    elapsed = time.perf_counter() - t0
    assert st == _lib.ETIMEOUT, (st, lib.lgb_last_error())
    assert b'expired' in lib.lgb_last_error()
    assert elapsed < 1.0, elapsed                      # ran out after ~1 ms, not the 2 s default
    torch.cuda.synchronize()                           # the context is still usable

    st, F = _dft2(lib, f, M, N, args, prec, ws)        # the next launch runs normally
    assert st == _lib.OK
    assert lib.lgb_dft2_status(ws.data_ptr(), stream) == _lib.OK
    ref = lo.dft2(f_np, args[0:2], shape=(M, N), shift=args[2:4], offset=args[4:6])
    assert lo.peak_normalised_error(F.cpu().numpy(), ref) < 3e-5
