"""Legendre spaces (LG quadrature) on the GPU path."""
from . import _lib


def space(N, nbcs, quad="LG", domain=(-1.0, 1.0)):
    raise _lib.SgpuError(_lib.ERR_UNSUPPORTED, "Legendre spaces are not built yet")
