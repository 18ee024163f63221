"""Device plumbing: torch tensors as device storage, streams, axis views."""
import numpy as np
import torch

from . import _lib


def require_cuda():
    """The product computes on the GPU only; fail loudly without one."""
    if not torch.cuda.is_available():
        raise _lib.SgpuError(_lib.ERR_UNSUPPORTED,
                             "shenfun_gb300 needs a CUDA device (no CPU fallback)")
    _lib.load()


def stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def ptr(t, dtypes=(torch.float64, torch.complex128)):
    if not isinstance(t, torch.Tensor):
        raise TypeError("expected a torch tensor")
    if not t.is_cuda:
        raise _lib.SgpuError(_lib.ERR_ARG, "tensor is not on a CUDA device")
    if t.dtype not in dtypes:
        raise _lib.SgpuError(_lib.ERR_ARG, f"unsupported dtype {t.dtype}")
    if not t.is_contiguous():
        raise _lib.SgpuError(_lib.ERR_ARG, "tensor must be C-contiguous")
    return t.data_ptr()


def data_kind(t):
    return _lib.COMPLEX if t.is_complex() else _lib.REAL


def view3(shape, axis):
    """(outer, n, inner) of a C-contiguous array around `axis`."""
    axis = axis % len(shape)
    outer = int(np.prod(shape[:axis], dtype=np.int64))
    inner = int(np.prod(shape[axis + 1:], dtype=np.int64))
    return outer, int(shape[axis]), inner


def as_device(a, dtype=None, device=None):
    """numpy / list / tensor -> contiguous CUDA tensor."""
    device = device or torch.device("cuda", torch.cuda.current_device())
    if isinstance(a, torch.Tensor):
        t = a.to(device=device, dtype=dtype) if dtype is not None else a.to(device=device)
    else:
        t = torch.as_tensor(np.asarray(a), device=device)
        if dtype is not None:
            t = t.to(dtype)
    return t.contiguous()
