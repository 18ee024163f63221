"""Serial transform plans with FFTW's unnormalised conventions, via scipy.fft.

Conventions (FFTW manual, "What FFTW Really Computes"):
  dct type 1 = REDFT00, type 2 = REDFT10, type 3 = REDFT01, type 4 = REDFT11
  dst type 1 = RODFT00, ...; scipy.fft's norm=None dct/dst match these exactly.
  fftn/rfftn: unnormalised forward; ifftn/irfftn: unnormalised backward.
"""
import numpy as np
import scipy.fft as sfft

from .utilities import *  # noqa: F401,F403
from .utilities import flag_dict  # noqa: F401


def aligned(shape, n=8, dtype=np.dtype("d"), fill=None):
    a = np.empty(shape, dtype=dtype)
    if fill is not None:
        a.fill(fill)
    return a


def aligned_like(z, fill=None):
    a = np.empty_like(np.asarray(z))
    if fill is not None:
        a.fill(fill)
    return a


class FFT:
    """A planned serial transform over fixed input/output arrays."""

    def __init__(self, kind, input_array, s, axes, output_array, type=None):
        self.kind = kind
        self.type = type
        self.axes = tuple(axes)
        self.s = s
        self.input_array = input_array
        self.output_array = output_array
        self._M = self._normalization()

    def _normalization(self):
        shp = self.output_array.shape if self.kind in ("irfft",) else self.input_array.shape
        if self.kind in ("irfft",):
            n = [self.output_array.shape[a] for a in self.axes]
        else:
            n = [self.input_array.shape[a] for a in self.axes]
        if self.kind in ("dct", "dst"):
            t = self.type
            if self.kind == "dct" and t == 1:
                return 1.0 / np.prod([2 * (m - 1) for m in n])
            if self.kind == "dst" and t == 1:
                return 1.0 / np.prod([2 * (m + 1) for m in n])
            return 1.0 / np.prod([2 * m for m in n])
        del shp
        return 1.0 / np.prod(n)

    def get_normalization(self):
        return self._M

    def _run(self):
        x = self.input_array
        ax = self.axes
        if self.kind == "fft":
            y = sfft.fftn(x, axes=ax)
        elif self.kind == "ifft":
            y = sfft.ifftn(x, axes=ax, norm="forward")
        elif self.kind == "rfft":
            y = sfft.rfftn(x, axes=ax)
        elif self.kind == "irfft":
            s = [self.output_array.shape[a] for a in ax]
            y = sfft.irfftn(x, s=s, axes=ax, norm="forward")
        elif self.kind == "dct":
            y = sfft.dctn(x, type=self.type, axes=ax)
        elif self.kind == "dst":
            y = sfft.dstn(x, type=self.type, axes=ax)
        else:
            raise NotImplementedError(self.kind)
        self.output_array[...] = y

    def __call__(self, input_array=None, output_array=None, implicit=True,
                 normalize=False, **kw):
        if input_array is not None and input_array is not self.input_array:
            self.input_array[...] = input_array
        self._run()
        if normalize:
            self.output_array *= self._M
        if output_array is not None and output_array is not self.output_array:
            output_array[...] = self.output_array
            return output_array
        return self.output_array


def _out(input_array, output_array, shape, dtype):
    if output_array is not None:
        return output_array
    return np.zeros(shape, dtype=dtype)


def fftn(input_array, s=None, axes=(-1,), threads=1, flags=(0,), output_array=None):
    out = _out(input_array, output_array, input_array.shape, np.complex128)
    return FFT("fft", input_array, s, axes, out)


def ifftn(input_array, s=None, axes=(-1,), threads=1, flags=(0,), output_array=None):
    out = _out(input_array, output_array, input_array.shape, np.complex128)
    return FFT("ifft", input_array, s, axes, out)


def rfftn(input_array, s=None, axes=(-1,), threads=1, flags=(0,), output_array=None):
    shp = list(input_array.shape)
    shp[axes[-1]] = shp[axes[-1]] // 2 + 1
    out = _out(input_array, output_array, shp, np.complex128)
    return FFT("rfft", input_array, s, axes, out)


def irfftn(input_array, s=None, axes=(-1,), threads=1, flags=(0,), output_array=None):
    shp = list(input_array.shape)
    if s is not None:
        for a, n in zip(axes, s):
            shp[a] = n
    else:
        shp[axes[-1]] = 2 * (shp[axes[-1]] - 1)
    out = _out(input_array, output_array, shp, np.float64)
    return FFT("irfft", input_array, s, axes, out)


def dctn(input_array, s=None, axes=(-1,), type=2, threads=1, flags=(0,), output_array=None):
    out = _out(input_array, output_array, input_array.shape, input_array.dtype)
    return FFT("dct", input_array, s, axes, out, type=type)


def idctn(input_array, s=None, axes=(-1,), type=2, threads=1, flags=(0,), output_array=None):
    inv = {1: 1, 2: 3, 3: 2, 4: 4}[type]
    return dctn(input_array, s, axes, inv, threads, flags, output_array)


def dstn(input_array, s=None, axes=(-1,), type=2, threads=1, flags=(0,), output_array=None):
    out = _out(input_array, output_array, input_array.shape, input_array.dtype)
    return FFT("dst", input_array, s, axes, out, type=type)


def idstn(input_array, s=None, axes=(-1,), type=2, threads=1, flags=(0,), output_array=None):
    inv = {1: 1, 2: 3, 3: 2, 4: 4}[type]
    return dstn(input_array, s, axes, inv, threads, flags, output_array)
