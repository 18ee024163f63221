"""Single-rank pencils: every pencil holds the whole array; transfers copy."""
import numpy as np
from mpi4py import MPI


class Subcomm(tuple):
    def __new__(cls, comm=None, dims=None, reorder=True):
        if isinstance(dims, int):
            dims = [0] * dims
        dims = list(dims) if dims is not None else [0]
        return tuple.__new__(cls, [MPI.Comm() for _ in dims])

    def destroy(self):
        pass


class Transfer:
    def __init__(self, comm, shape, dtype, subshapeA, axisA, subshapeB, axisB):
        self.comm = comm
        self.shape = tuple(shape)
        self.dtype = np.dtype(dtype)
        self.subshapeA = tuple(subshapeA)
        self.subshapeB = tuple(subshapeB)
        self.axisA = axisA
        self.axisB = axisB

    def forward(self, arrayA, arrayB):
        arrayB[...] = arrayA

    def backward(self, arrayB, arrayA):
        arrayA[...] = arrayB

    def destroy(self):
        pass


class Pencil:
    def __init__(self, subcomm, shape, axis=-1):
        self.subcomm = subcomm
        self.shape = tuple(shape)
        self.axis = axis % len(shape) if len(shape) else 0
        self.subshape = tuple(shape)
        self.substart = (0,) * len(shape)

    def pencil(self, axis):
        return Pencil(self.subcomm, self.shape, axis)

    def transfer(self, pencil, dtype):
        return Transfer(MPI.Comm(), self.shape, dtype, self.subshape, self.axis,
                        pencil.subshape, pencil.axis)
