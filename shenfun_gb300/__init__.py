"""shenfun_gb300: the tensor-product spectral-Galerkin hot path of shenfun on
one GB300 GPU (sm_103a CUDA kernels behind a C ABI, torch tensors as storage).

The Python API mirrors shenfun's for this path::

    from shenfun_gb300 import *
    T = TensorProductSpace(comm, (FunctionSpace(N, 'F', dtype='D'),
                                  FunctionSpace(N, 'F', dtype='d'),
                                  FunctionSpace(N + 1, 'C', bc=(0, 0))))
    u, v = TrialFunction(T), TestFunction(T)
    H = chebyshev.la.Helmholtz(*inner(v, -div(grad(u)) + c*u))
    u_hat = H(inner(v, f), Function(T))
    u = u_hat.backward()
"""
from . import _lib  # noqa: F401
from ._lib import SgpuError, check_device  # noqa: F401
from .spaces import FunctionSpace, TensorProductSpace, R2C, C2C  # noqa: F401
from .forms import (Array, Function, TestFunction, TrialFunction, inner, project,  # noqa: F401
                    div, grad, Dx, TPMatrix)
from . import la, chebyshev  # noqa: F401
from .integrators import PDEIMEXRK, IMEXRK011, IMEXRK111, IMEXRK222, IMEXRK443  # noqa: F401

comm = None  # single GPU, single process: no MPI communicator

__version__ = "0.1.0"
