"""Per-axis transform plans: owners of the C-ABI ``sgpu_plan`` handles.

The counterpart of the serial FFTW plan objects the reference creates in each
basis' ``plan()`` (mpi4py_fft.fftw.dctn/rfftn/irfftn/fftn/ifftn,
chebyshev/bases.py:407-469, fourier/bases.py:218-279): built once per
(kind, n, basis) and reused; the tables live on the device.
"""
import ctypes

import torch

from . import _lib
from .device import ptr, stream_handle, view3, data_kind

_cache = {}


class LinePlan:
    def __init__(self, kind, n, basis=_lib.BASIS_ORTHO, form=_lib.PLAIN_F64):
        self.kind, self.n, self.basis, self.form = kind, n, basis, form
        h = ctypes.c_void_p()
        _lib.call("sgpu_plan_create", ctypes.byref(h), kind, n, basis, form)
        self._h = h

    def __del__(self):
        try:
            if self._h:
                _lib.load().sgpu_plan_destroy(self._h)
                self._h = None
        except Exception:
            pass

    @property
    def variant(self):
        """The plan's kernel variant (sgpu_plan_get_variant; 0 where the plan
        has a single kernel)."""
        v = ctypes.c_int()
        _lib.call("sgpu_plan_get_variant", self._h, ctypes.byref(v))
        return v.value

    @variant.setter
    def variant(self, v):
        _lib.call("sgpu_plan_set_variant", self._h, int(v))

    def __call__(self, inp, out, axis, scale=1.0, stream=None):
        """Transform `inp` into `out` along `axis` (both C-contiguous CUDA tensors)."""
        outer, n_in, inner = view3(tuple(inp.shape), axis)
        o2, n_out, i2 = view3(tuple(out.shape), axis)
        if (outer, inner) != (o2, i2):
            raise _lib.SgpuError(_lib.ERR_ARG, "input/output shapes differ off the axis")
        kind = data_kind(inp)
        from . import autotune
        if autotune.enabled():
            lay = (outer, inner, kind)
            tuned = self.__dict__.setdefault("_tuned", {})
            if lay not in tuned:
                tuned[lay] = None  # the tuner's own calls of this plan run as set
                tuned[lay] = autotune.apply(self, outer, inner, kind)
            elif tuned[lay] is not None and self.variant != tuned[lay]:
                self.variant = tuned[lay]
        nb = ctypes.c_size_t()
        _lib.call("sgpu_plan_workspace_size", self._h, outer, inner, kind, ctypes.byref(nb))
        work = None
        if nb.value:
            # tensor-core form on strided lines: scratch for the split input
            # from torch's caching allocator (512-byte aligned, reused)
            work = torch.empty(nb.value, dtype=torch.uint8, device=inp.device)
        dst = out
        if (self.form == _lib.MIXED_DF and inner == 1 and n_in > 130 and inp.data_ptr() == out.data_ptr()
                and self.kind in (_lib.XF_CHEB_SCALAR, _lib.XF_CHEB_FORWARD, _lib.XF_CHEB_BACKWARD)):
            # the fused tensor-core kernel does not run in place for n > 130
            dst = torch.empty_like(out)
        _lib.call("sgpu_plan_execute_ws", self._h, ptr(inp), ptr(dst), outer, inner, kind,
                  float(scale), work.data_ptr() if work is not None else None, nb.value,
                  stream_handle(stream))
        if dst is not out:
            out.copy_(dst)
        return out


def get_plan(kind, n, basis=_lib.BASIS_ORTHO, form=_lib.PLAIN_F64):
    key = (kind, n, basis, form)
    p = _cache.get(key)
    if p is None:
        p = LinePlan(kind, n, basis, form)
        _cache[key] = p
    return p
