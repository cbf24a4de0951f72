"""Write-bounds checks of the C ABI (compute-sanitizer is closed on the GPU
pool): every output and workspace buffer handed to the library sits inside a
larger allocation whose margins hold a sentinel byte pattern, and after each
call on small ragged shapes the margins must be unchanged.  A kernel writing
past either end of its buffer (by up to the guard width) fails the test
instead of corrupting a neighbour silently."""
import ctypes

import numpy as np
import pytest
import torch

from lentil_gb300 import _lib
from oracle import lentil_oracle as lo

pytestmark = pytest.mark.gpu

GUARD = 1 << 20              # bytes of sentinel on each side
PATTERN = 0xA5


class Guarded:
    """A device buffer of ``nbytes`` between two sentinel margins."""

    def __init__(self, nbytes):
        self.nbytes = max(int(nbytes), 1)
        n = self.nbytes + 2 * GUARD + 256
        self.raw = torch.full((n,), PATTERN, dtype=torch.uint8, device='cuda')
        base = self.raw.data_ptr()
        self.off = GUARD + (-(base + GUARD)) % 256          # 256-byte aligned data start
        self.ptr = base + self.off

    def view(self, dtype, shape):
        count = int(np.prod(shape))
        itemsize = torch.empty((), dtype=dtype).element_size()
        assert count * itemsize <= self.nbytes
        return self.raw[self.off:self.off + count * itemsize].view(dtype).view(shape)

    def check(self):
        torch.cuda.synchronize()
        head = self.raw[:self.off]
        tail = self.raw[self.off + self.nbytes:]
        assert bool((head == PATTERN).all()), 'write before the buffer'
        assert bool((tail == PATTERN).all()), 'write past the end of the buffer'


def _s():
    return torch.cuda.current_stream().cuda_stream


def _c128(shape, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    return torch.as_tensor(a, device='cuda')


@pytest.mark.parametrize('shape', [(1, 1), (7, 5), (33, 65), (130, 97)])
def test_phasor_and_field_insert(cuda_device, shape):
    m, n = shape
    H, W = m + 6, n + 3
    rng = np.random.default_rng(m)
    amp = torch.as_tensor(rng.uniform(0, 1, (H, W)), device='cuda')
    opd = torch.as_tensor(rng.normal(0, 1e-7, (H, W)), device='cuda')
    out = Guarded(16 * m * n)
    _lib.call('lgb_phasor', amp.data_ptr(), 0.0, None, opd.data_ptr(), 0.0, H, W, 4, 2, m, n,
              600e-9, out.ptr, _s())
    out.check()
    f = out.view(torch.complex128, (m, n)).clone()
    for intensity in (0, 1):
        om, on = m + 5, n - 1 if n > 1 else 1
        dst = Guarded((8 if intensity else 16) * om * on)
        dst.view(torch.uint8, (dst.nbytes,)).zero_()
        for off in ((0, 0), (3, -2), (-om, on), (om // 2 + 1, -(on // 2) - 2)):
            _lib.call('lgb_field_insert', f.data_ptr(), m, n, off[0], off[1], dst.ptr, om, on,
                      0.5, intensity, _s())
        dst.check()


@pytest.mark.parametrize('precision', [_lib.FP64, _lib.SPLIT_BF16, _lib.SPLIT_FP16])
@pytest.mark.parametrize('geom', [(1, 2, 3, 5), (37, 29, 41, 23), (70, 130, 129, 65)])
def test_dft2_batch_outputs_and_workspace(cuda_device, precision, geom):
    m, n, M, N = geom
    count = 3
    lib = _lib.load()
    f = _c128((count, m, n), m * n)
    F = Guarded(16 * count * M * N)
    nbytes = lib.lgb_dft2_batch_workspace_size(count, m, n, M, N, precision)
    ws = Guarded(nbytes)
    _lib.call('lgb_dft2_batch', f.data_ptr(), count, m, n, F.ptr, M, N, 0.021, 0.017, 0.5,
              -1.0, 1.0, 2.0, 1, precision, ws.ptr, nbytes, _s())
    F.check()
    ws.check()


@pytest.mark.parametrize('precision', [_lib.FP64, _lib.SPLIT_BF16])
def test_dft2_plan_execute(cuda_device, precision):
    lib = _lib.load()
    m, n, M, N = 45, 61, 77, 38
    size = lib.lgb_dft2_plan_size(m, n, M, N, precision)
    mem = Guarded(size)
    h = ctypes.c_void_p()
    _lib.call('lgb_dft2_plan_create_in', m, n, M, N, 0.03, 0.02, 0.0, 0.5, -1.0, 0.0, 1,
              precision, mem.ptr, size, _s(), ctypes.byref(h))
    try:
        for count in (1, 4):
            f = _c128((count, m, n), count)
            F = Guarded(16 * count * M * N)
            nbytes = lib.lgb_dft2_plan_workspace_size(h, count)
            ws = Guarded(nbytes)
            _lib.call('lgb_dft2_plan_execute', h, f.data_ptr(), count, F.ptr, ws.ptr, nbytes, _s())
            F.check()
            ws.check()
        mem.check()
    finally:
        torch.cuda.synchronize()
        lib.lgb_dft2_plan_destroy(h)


@pytest.mark.parametrize('n,os_', [(64, 2), (75, 2), (61, 7), (128, 3), (90, 3)])
def test_pixel_and_pixelate(cuda_device, n, os_):
    lib = _lib.load()
    img = torch.as_tensor(np.random.default_rng(n).uniform(0, 1, (n, n)) ** 4, device='cuda')
    nbytes = lib.lgb_pixel_workspace_size(n, os_)
    S = lib.lgb_pixelate_size(n, os_)
    for name, out_n in (('lgb_pixel', n), ('lgb_pixelate', S)):
        out = Guarded(8 * out_n * out_n)
        ws = Guarded(nbytes)
        _lib.call(name, img.data_ptr(), n, n, os_, out.ptr, ws.ptr, nbytes, _s())
        out.check()
        ws.check()
        if name == 'lgb_pixelate':
            res = out.view(torch.float64, (S, S)).cpu().numpy()
            assert lo.peak_normalised_error(res, lo.pixelate(img.cpu().numpy(), os_)) < 1e-12


def test_zernike_tilt_and_power_spectrum(cuda_device):
    lib = _lib.load()
    H, W = 53, 47
    rng = np.random.default_rng(4)
    mask = torch.as_tensor((rng.uniform(size=(H, W)) > 0.3).astype(float), device='cuda')
    rho = Guarded(8 * H * W)
    theta = Guarded(8 * H * W)
    zws = Guarded(lib.lgb_zernike_workspace_size())
    _lib.call('lgb_zernike_coordinates', mask.data_ptr(), H, W, 1, 0.0, 0.0, 10.0, rho.ptr,
              theta.ptr, zws.ptr, lib.lgb_zernike_workspace_size(), _s())
    for g in (rho, theta, zws):
        g.check()
    # mode table rows [m, scale, nterms, (coef, power) x 2]
    table = torch.as_tensor(np.array([[1, 2.0, 1, 1.0, 1, 0, 0], [0, 1.5, 2, 2.0, 2, -1.0, 0]]),
                            device='cuda')
    out = Guarded(8 * 2 * H * W)
    _lib.call('lgb_zernike_eval', rho.ptr, theta.ptr, mask.data_ptr(), H * W, table.data_ptr(), 2,
              2, out.ptr, 1, _s())
    out.check()
    S = 3
    masks = torch.as_tensor(np.stack([(rng.uniform(size=(H, W)) > 0.5).astype(float)
                                      for _ in range(S)]), device='cuda')
    opd = torch.as_tensor(rng.normal(size=(H, W)), device='cuda')
    nb = lib.lgb_ptt_normal_workspace_size(S)
    nrm = Guarded(8 * S * 9)                     # {A00 A01 A02 A11 A12 A22 y0 y1 y2} per mask
    tws = Guarded(nb)
    _lib.call('lgb_ptt_normal', opd.data_ptr(), masks.data_ptr(), S, H, W, 0.1, 0.1, nrm.ptr,
              tws.ptr, nb, _s())
    nrm.check()
    tws.check()
    t = torch.zeros(3 * S, dtype=torch.float64, device='cuda')
    rem = Guarded(8 * H * W)
    _lib.call('lgb_remove_tilt', opd.data_ptr(), masks.data_ptr(), S, H, W, 0.1, 0.1,
              t.data_ptr(), rem.ptr, _s())
    rem.check()
    for N in (48, 64):
        noise = torch.as_tensor(rng.normal(size=(N, N)), device='cuda')
        pm = torch.ones((N, N), dtype=torch.float64, device='cuda')
        pb = lib.lgb_power_spectrum_workspace_size(N)
        psd = Guarded(8 * N * N)
        pws = Guarded(pb)
        _lib.call('lgb_power_spectrum', noise.data_ptr(), pm.data_ptr(), N, 1e-3, 1e-8, 8.0,
                  3.0, psd.ptr, pws.ptr, pb, _s())
        psd.check()
        pws.check()


@pytest.mark.parametrize('precision', [_lib.FP64, _lib.SPLIT_BF16])
def test_idft2_c_entry(cuda_device, precision):
    # lgb_idft2 (the C entry; Python's idft2 composes the cached dft2 instead)
    lib = _lib.load()
    m, n, M, N = 33, 47, 40, 29
    F = _c128((m, n), 5)
    out = Guarded(16 * M * N)
    nbytes = lib.lgb_idft2_workspace_size(m, n, M, N, precision)
    ws = Guarded(nbytes)
    _lib.call('lgb_idft2', F.data_ptr(), m, n, out.ptr, M, N, 0.03, 0.025, 0.5, -1.0, 1,
              precision, ws.ptr, nbytes, _s())
    out.check()
    ws.check()
    got = out.view(torch.complex128, (M, N)).cpu().numpy()
    ref = lo.idft2(F.cpu().numpy(), (0.03, 0.025), shape=(M, N), shift=(0.5, -1.0), unitary=True)
    assert lo.peak_normalised_error(got, ref) < (1e-12 if precision == _lib.FP64 else 3e-5)
