"""Recursive Legendre transforms of the gb300 optimization mode: the two
names spectralbase.py imports from ``shenfun.optimization.<mode>.transforms``
for ``kind='recursive'`` (spectralbase.py:485-491, 551-558), with the
reference's signatures (optimization/cython/transforms.pyx:175-216).  Each
call builds the point-by-degree matrix from the recursion matrix on the GPU
and applies it to every line with an FP64 GEMM (``sgpu_scalar_product`` /
``sgpu_evaluate_expansion_all``).
"""
from . import _Dev, _call, _f64
from ..device import stream_handle, view3

__all__ = ["scalar_product", "evaluate_expansion_all"]


def _recursion(a):
    ad = _f64(a)
    if ad.t.dim() != 2 or ad.t.shape[0] not in (2, 3):
        raise ValueError("recursion matrix data must have 2 or 3 rows")
    return ad


def scalar_product(input_array, output_array, x, w, axis, a):
    """transforms.pyx:175 scalar_product(input, output, x, w, axis, a):
    output[i] = sum_j P_i(x_j) w_j input[j] along ``axis``."""
    ind = _Dev(input_array)
    outd = _Dev(output_array, ind.t.dtype)
    outer, N, inner = view3(tuple(ind.t.shape), axis)
    if tuple(outd.t.shape) != tuple(ind.t.shape):
        raise ValueError("scalar_product: input and output must have the same shape")
    xd, wd, ad = _f64(x), _f64(w), _recursion(a)
    if xd.t.numel() < N or wd.t.numel() < N:
        raise ValueError("scalar_product: fewer points than the axis length")
    _call("sgpu_scalar_product", ind.ptr, outd.ptr, xd.ptr, wd.ptr, ad.ptr, ad.t.shape[0], ad.t.shape[1], outer,
          N, inner, ind.kind, None, 0, stream_handle())
    outd.back()
    return output_array


def evaluate_expansion_all(input_array, output_array, x, axis, a):
    """transforms.pyx:199 evaluate_expansion_all(input, output, x, axis, a):
    output[j] = sum_i P_i(x_j) input[i] along ``axis``."""
    ind = _Dev(input_array)
    outd = _Dev(output_array, ind.t.dtype)
    outer, N, inner = view3(tuple(ind.t.shape), axis)
    o2, Nx, i2 = view3(tuple(outd.t.shape), axis)
    if (o2, i2) != (outer, inner):
        raise ValueError("evaluate_expansion_all: input and output differ off the axis")
    xd, ad = _f64(x), _recursion(a)
    if xd.t.numel() < Nx:
        raise ValueError("evaluate_expansion_all: fewer points than the output axis")
    _call("sgpu_evaluate_expansion_all", ind.ptr, outd.ptr, xd.ptr, ad.ptr, ad.t.shape[0], ad.t.shape[1], outer,
          N, Nx, inner, ind.kind, None, 0, stream_handle())
    outd.back()
    return output_array
