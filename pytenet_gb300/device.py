"""
Device plumbing: PyTorch is used only for device memory, streams and graph
capture. All arithmetic happens in the CUDA kernels of libptn_gb300.so.
"""

import numpy as np
import torch

from . import _lib

CDT = torch.complex128


def device():
    if not torch.cuda.is_available():
        raise RuntimeError("pytenet_gb300 needs a CUDA GPU (GB300, sm_103a); no CPU fallback exists")
    return torch.device("cuda", torch.cuda.current_device())


def lib():
    return _lib.load()


def stream_ptr():
    return torch.cuda.current_stream().cuda_stream


def ptr(t):
    return t.data_ptr() if t is not None else None


def to_dev(x):
    """Host array (or device tensor) -> contiguous complex128 device tensor."""
    if isinstance(x, torch.Tensor):
        t = x.to(device=device(), dtype=CDT)
        return t.contiguous()
    a = np.ascontiguousarray(np.asarray(x), dtype=np.complex128)
    return torch.from_numpy(a).to(device(), non_blocking=False)


def to_host(t):
    return t.detach().cpu().numpy()


def empty(shape):
    return torch.empty(tuple(int(s) for s in shape), dtype=CDT, device=device())


def zeros(shape):
    return torch.zeros(tuple(int(s) for s in shape), dtype=CDT, device=device())


class Workspace:
    """Grow-only device scratch buffer (bytes)."""

    def __init__(self):
        self.buf = None

    def get(self, nbytes):
        nbytes = max(int(nbytes), 256)
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = torch.empty(nbytes, dtype=torch.uint8, device=device())
        return self.buf

    def ptr(self, nbytes):
        return self.get(nbytes).data_ptr(), max(int(nbytes), 256)


def call(fn, *args):
    """Invoke a C entry point and raise on a non-OK status."""
    _lib.check(fn(*args))
