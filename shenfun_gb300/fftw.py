"""Per-axis transform plan objects with the interface of the FFTW plans the
reference's bases build in ``plan()``: ``mpi4py_fft.fftw.dctn / rfftn /
irfftn / fftn / ifftn`` (chebyshev/bases.py:407-469, fourier/bases.py:218-279)
and call through ``Transform`` (spectralbase.py:2398-2416) as
``self.forward.xfftn()`` / ``self.backward.xfftn(normalise_idft=False)``.

A plan is made once over fixed input and output arrays and then called
without arguments (or with arrays to copy in and out), exactly as there:

* ``input_array`` / ``output_array``: the planned arrays (CUDA tensors here,
  C-contiguous, made by ``aligned``/``aligned_like`` or given by the caller);
* ``__call__(input_array=None, output_array=None, implicit=True,
  normalize=False, **kw)``: one line-kernel launch on the current stream;
  ``normalize=True`` applies ``get_normalization()`` inside that launch;
* ``get_normalization()``: 1/N for the Fourier plans, 1/(2N) for DCT types 2
  and 3 (FFTW's logical transform sizes).

The outputs follow FFTW's unnormalised conventions: ``dctn`` type 2 is
REDFT10 (y_k = 2 sum_n x_n cos(pi k (2n + 1) / 2N)), type 3 is REDFT01
(y_k = x_0 + 2 sum_{n>=1} x_n cos(pi n (2k + 1) / 2N)), ``fftn``/``rfftn``
are the unnormalised forward DFT and ``ifftn``/``irfftn`` the unnormalised
backward one.  Complex input to ``dctn`` transforms the real and imaginary
parts alike (what the reference's ``DCTWrap`` does with two real plans).
One transformed axis per plan, as every basis of the reference uses.  DCT
types 1 and 4 and the DSTs (the Gauss-Lobatto Chebyshev points and other
bases, outside the transforms this library runs) raise ``SgpuError``
(unsupported).  ``form="mixed"`` runs the Fourier plans of length 256 in the
mixed form's fixed-point kernels; the default is the FP64 form.
"""
import numpy as np
import torch

from . import _lib
from .device import require_cuda
from .plans import get_plan

# FFTW's planner flags (fftw3.h values), for call sites that pass them
flag_dict = {"FFTW_MEASURE": 0, "FFTW_DESTROY_INPUT": 1, "FFTW_UNALIGNED": 2, "FFTW_CONSERVE_MEMORY": 4,
             "FFTW_EXHAUSTIVE": 8, "FFTW_PRESERVE_INPUT": 16, "FFTW_PATIENT": 32, "FFTW_ESTIMATE": 64}

_TORCH = {np.dtype("float64"): torch.float64, np.dtype("complex128"): torch.complex128}


def _tdtype(dtype):
    if isinstance(dtype, torch.dtype):
        return dtype
    t = _TORCH.get(np.dtype(dtype))
    if t is None:
        raise _lib.SgpuError(_lib.ERR_UNSUPPORTED, "plans run on float64 and complex128 arrays")
    return t


def aligned(shape, n=8, dtype=np.dtype("d"), fill=None):
    """A C-contiguous device array of `shape` (the allocator's blocks are
    512-byte aligned, above any `n`)."""
    require_cuda()
    a = torch.empty(tuple(shape), dtype=_tdtype(dtype), device="cuda")
    if fill is not None:
        a.fill_(fill)
    return a


def aligned_like(z, fill=None):
    """A device array of z's shape and dtype (z a tensor or a numpy array)."""
    if not isinstance(z, torch.Tensor):
        return aligned(np.shape(z), dtype=np.asarray(z).dtype, fill=fill)
    require_cuda()
    a = torch.empty_like(z, memory_format=torch.contiguous_format, device="cuda")
    if fill is not None:
        a.fill_(fill)
    return a


class FFT:
    """A planned transform of `input_array` into `output_array` along one
    axis (the interface of mpi4py_fft.fftw's plan objects)."""

    def __init__(self, kind, input_array, output_array, axis, n, M, form):
        for a in (input_array, output_array):
            if not (isinstance(a, torch.Tensor) and a.is_cuda and a.is_contiguous()):
                raise _lib.SgpuError(_lib.ERR_ARG, "plans take C-contiguous CUDA arrays")
        want = {_lib.XF_R2C: (torch.float64, torch.complex128), _lib.XF_C2R: (torch.complex128, torch.float64),
                _lib.XF_C2C_FWD: (torch.complex128, torch.complex128),
                _lib.XF_C2C_BWD: (torch.complex128, torch.complex128)}.get(
                    kind, (input_array.dtype, input_array.dtype))
        if (input_array.dtype, output_array.dtype) != want or want[0] not in (torch.float64, torch.complex128):
            raise _lib.SgpuError(_lib.ERR_ARG, "array dtypes do not match the transform")
        self.kind = kind
        self.axis = axis % input_array.dim()
        self._input_array = input_array
        self._output_array = output_array
        self._M = M
        self._plan = get_plan(kind, n, form=_lib.FORMS[form])

    @property
    def input_array(self):
        return self._input_array

    @property
    def output_array(self):
        return self._output_array

    def get_normalization(self):
        return self._M

    def __call__(self, input_array=None, output_array=None, implicit=True, normalize=False, **kw):
        if input_array is not None and input_array is not self._input_array:
            self._input_array.copy_(torch.as_tensor(input_array, device=self._input_array.device))
        self._plan(self._input_array, self._output_array, self.axis, self._M if normalize else 1.0)
        if output_array is not None and output_array is not self._output_array:
            if isinstance(output_array, torch.Tensor):
                output_array.copy_(self._output_array)
            else:
                output_array[...] = self._output_array.cpu().numpy()
            return output_array
        return self._output_array


def _axis(input_array, axes):
    if axes is None or len(tuple(np.atleast_1d(axes))) != 1:
        raise _lib.SgpuError(_lib.ERR_UNSUPPORTED, "one transformed axis per plan")
    return int(np.atleast_1d(axes)[0]) % input_array.dim()


def _output(output_array, shape, dtype, like):
    if output_array is not None:
        if tuple(output_array.shape) != tuple(shape) or output_array.dtype != dtype:
            raise _lib.SgpuError(_lib.ERR_ARG, "output array has the wrong shape or dtype")
        return output_array
    return torch.zeros(tuple(shape), dtype=dtype, device=like.device)


def dctn(input_array, s=None, axes=(-1,), type=2, threads=1, flags=(0,), output_array=None, form="plain"):
    """DCT type 2 (REDFT10) or 3 (REDFT01) along one axis."""
    require_cuda()
    ax = _axis(input_array, axes)
    if type not in (2, 3):
        raise _lib.SgpuError(_lib.ERR_UNSUPPORTED, "DCT types 2 and 3 only")
    n = input_array.shape[ax]
    out = _output(output_array, input_array.shape, input_array.dtype, input_array)
    return FFT(_lib.XF_DCT2 if type == 2 else _lib.XF_DCT3, input_array, out, ax, n, 1.0 / (2 * n), form)


def fftn(input_array, s=None, axes=(-1,), threads=1, flags=(0,), output_array=None, form="plain"):
    """Unnormalised forward complex DFT along one axis."""
    require_cuda()
    ax = _axis(input_array, axes)
    n = input_array.shape[ax]
    out = _output(output_array, input_array.shape, torch.complex128, input_array)
    return FFT(_lib.XF_C2C_FWD, input_array, out, ax, n, 1.0 / n, form)


def ifftn(input_array, s=None, axes=(-1,), threads=1, flags=(0,), output_array=None, form="plain"):
    """Unnormalised backward complex DFT along one axis."""
    require_cuda()
    ax = _axis(input_array, axes)
    n = input_array.shape[ax]
    out = _output(output_array, input_array.shape, torch.complex128, input_array)
    return FFT(_lib.XF_C2C_BWD, input_array, out, ax, n, 1.0 / n, form)


def rfftn(input_array, s=None, axes=(-1,), threads=1, flags=(0,), output_array=None, form="plain"):
    """Unnormalised real-to-complex forward DFT along one axis (N // 2 + 1
    outputs)."""
    require_cuda()
    ax = _axis(input_array, axes)
    n = input_array.shape[ax]
    shape = list(input_array.shape)
    shape[ax] = n // 2 + 1
    out = _output(output_array, shape, torch.complex128, input_array)
    return FFT(_lib.XF_R2C, input_array, out, ax, n, 1.0 / n, form)


def irfftn(input_array, s=None, axes=(-1,), threads=1, flags=(0,), output_array=None, form="plain"):
    """Unnormalised complex-to-real backward DFT along one axis; the real
    length is `s` (or the output array's), else 2 (M - 1) for M inputs."""
    require_cuda()
    ax = _axis(input_array, axes)
    if s is not None:
        n = int(np.atleast_1d(s)[-1])
    elif output_array is not None:
        n = output_array.shape[ax]
    else:
        n = 2 * (input_array.shape[ax] - 1)
    if n // 2 + 1 != input_array.shape[ax]:
        raise _lib.SgpuError(_lib.ERR_ARG, "real length does not match the complex input")
    shape = list(input_array.shape)
    shape[ax] = n
    out = _output(output_array, shape, torch.float64, input_array)
    return FFT(_lib.XF_C2R, input_array, out, ax, n, 1.0 / n, form)
