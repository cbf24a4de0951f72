"""Device plumbing: torch supplies device memory and the current stream; all
arithmetic of the path runs in the library's own kernels."""
import numpy as np
import torch

from . import _lib


_ready = False


def device():
    """The current CUDA device; raises when there is none (no CPU fallback).
    The availability check and the library load run once per process."""
    global _ready
    if not _ready:
        if not torch.cuda.is_available():
            raise RuntimeError('lentil_gb300 needs a CUDA device (GB300, sm_103a); none is available')
        _lib.load()
        _ready = True
    return torch.device('cuda', torch.cuda.current_device())


def stream_ptr():
    return torch.cuda.current_stream().cuda_stream


def is_tensor(x):
    return isinstance(x, torch.Tensor)


PINNED_COPY_LIMIT = 64 << 20     # host arrays up to this size are staged through pinned memory


def to_device(x, dtype):
    """numpy / scalar / tensor -> contiguous CUDA tensor of ``dtype`` (one copy at most).

    Host data never makes the host wait for the GPU: a single value becomes a
    device fill (no copy), an array up to ``PINNED_COPY_LIMIT`` is copied into
    a pinned block of torch's caching host allocator (read before this call
    returns, so the caller may reuse its array) and sent with an asynchronous
    copy on the current stream."""
    dev = device()
    if is_tensor(x):
        t = x.to(device=dev, dtype=dtype)
    else:
        a = np.asarray(x)
        if dtype == torch.complex128:
            a = a.astype(np.complex128, copy=False)
        elif dtype == torch.float64:
            a = a.astype(np.float64, copy=False)
        if a.size == 1 and a.dtype.kind in 'fc':
            return torch.full(a.shape, a.item(), dtype=dtype, device=dev)
        # np.ascontiguousarray would turn a 0-d array into shape (1,)
        a = a if a.flags.c_contiguous else a.copy(order='C')
        h = torch.from_numpy(a)
        if 0 < a.nbytes <= PINNED_COPY_LIMIT and h.dtype == dtype:
            t = h.pin_memory().to(device=dev, non_blocking=True)
        else:
            t = h.to(device=dev, dtype=dtype)
    return t.contiguous()


def ptr(t):
    return t.data_ptr() if t is not None else None


def workspace(nbytes):
    """256-byte-aligned device workspace (the caching allocator aligns to 512)."""
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device())


def to_host(t):
    return t.detach().cpu().numpy()
