"""numpy-backed DistArray for one rank."""
from numbers import Number
import numpy as np
from .pencil import Pencil, Subcomm


class DistArray(np.ndarray):
    def __new__(cls, global_shape, subcomm=None, val=None, dtype=float,
                buffer=None, alignment=None, rank=0):
        global_shape = tuple(global_shape)
        if isinstance(buffer, np.ndarray) and buffer.shape == global_shape:
            buffer = np.ascontiguousarray(buffer, dtype=dtype)
            obj = np.ndarray.__new__(cls, global_shape, dtype=dtype, buffer=buffer)
        else:
            obj = np.ndarray.__new__(cls, global_shape, dtype=dtype, buffer=buffer)
        if buffer is None and isinstance(val, Number):
            obj.fill(val)
        ndim = len(global_shape) - rank
        sub = subcomm if subcomm is not None else Subcomm(None, [0] * max(ndim, 1))
        al = alignment if alignment is not None else ndim - 1
        obj._p0 = Pencil(sub, global_shape[rank:], al)
        obj._rank = rank
        return obj

    def __array_finalize__(self, obj):
        if obj is None:
            return
        self._p0 = getattr(obj, "_p0", None)
        self._rank = getattr(obj, "_rank", 0)

    @property
    def v(self):
        return self.__array__()

    @property
    def global_shape(self):
        return self.shape

    @property
    def substart(self):
        return (0,) * self.ndim

    @property
    def subcomm(self):
        return self._p0.subcomm if self._p0 is not None else None

    @property
    def commsizes(self):
        return [1] * (self.ndim - self.rank)

    @property
    def pencil(self):
        return self._p0

    @property
    def rank(self):
        return self._rank

    @property
    def dimensions(self):
        return self.ndim - self.rank

    @property
    def alignment(self):
        return self._p0.axis if self._p0 is not None else self.ndim - 1

    def local_slice(self):
        return tuple(slice(0, n) for n in self.shape)

    def get_global_slice(self, gslice):
        return np.asarray(self)[gslice]

    def redistribute(self, axis=None, out=None):
        if out is not None:
            out[...] = self
            return out
        return self

    def get_pencil_and_transfer(self, axis):
        p1 = Pencil(self.subcomm, self.shape[self.rank:], axis)
        return p1, self._p0.transfer(p1, self.dtype)


def newDistArray(pfft, forward_output=True, val=0, rank=0, view=False):
    shape = pfft.shape(forward_output)
    dtype = pfft.dtype(forward_output)
    a = DistArray(shape, val=val, dtype=dtype, rank=0)
    return a.v if view else a
