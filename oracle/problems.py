"""Tensor-product round trips (CPU oracle): forward/scalar product over every
axis, per-wavenumber banded solve, backward.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

A space is a list of 1D bases, one per axis, each ``(family, kind, N)`` with
family in {"fourier", "chebyshev", "legendre"} and kind in {"C2C", "R2C"} for
Fourier or {"T", "SD", "SB", "L"} for the polynomial families.  The reference
transforms the last axis of ``axes`` first (tensorproductspace.py:417-447) and
runs the backward chain in the opposite order (tensorproductspace.py:45-96).
"""
import numpy as np

from . import spectral as S
from . import la


def _scalar_1d(f, basis, axis, kind="recursive"):
    fam, b, N = basis
    if fam == "fourier":
        return S.r2c_forward(f, axis) if b == "R2C" else S.c2c_forward(f, axis)
    if fam == "chebyshev":
        return S.cheb_scalar_product(f, b, axis)
    return S.leg_scalar_product(f, b, axis, kind)


def _forward_1d(f, basis, axis, kind="recursive"):
    fam, b, N = basis
    if fam == "fourier":
        return _scalar_1d(f, basis, axis)
    if fam == "chebyshev":
        return S.cheb_forward(f, b, axis)
    return S.leg_forward(f, b, axis, kind)


def _backward_1d(u, basis, axis, kind="recursive"):
    fam, b, N = basis
    if fam == "fourier":
        return S.r2c_backward(u, N, axis) if b == "R2C" else S.c2c_backward(u, axis)
    if fam == "chebyshev":
        return S.cheb_backward(u, b, axis)
    return S.leg_backward(u, b, axis, kind)


def scalar_product(f, bases, axes=None, kind="recursive"):
    """ScalarTransform.__call__ (tensorproductspace.py:146-191)."""
    axes = list(range(len(bases))) if axes is None else list(axes)
    out = f
    for ax in reversed(axes):
        out = _scalar_1d(out, bases[ax], ax, kind)
    return out


def forward(f, bases, axes=None, kind="recursive"):
    """ForwardTransform.__call__ (tensorproductspace.py:205-259)."""
    axes = list(range(len(bases))) if axes is None else list(axes)
    out = f
    for ax in reversed(axes):
        out = _forward_1d(out, bases[ax], ax, kind)
    return out


def backward(u, bases, axes=None, kind="recursive"):
    """BackwardTransform.__call__ (tensorproductspace.py:45-96)."""
    axes = list(range(len(bases))) if axes is None else list(axes)
    out = u
    for ax in axes:
        out = _backward_1d(out, bases[ax], ax, kind)
    return out


def fourier_k2(bases, solve_axis):
    """sum over Fourier axes of k^2, broadcast to the spectral shape with the
    solve axis collapsed (TPMatrix scale arrays, matrixbase.py:1328-1365)."""
    shape = []
    ks = []
    for ax, (fam, b, N) in enumerate(bases):
        if ax == solve_axis:
            shape.append(1)
            continue
        k = S.r2c_wavenumbers(N) if b == "R2C" else S.c2c_wavenumbers(N)
        shape.append(len(k))
        ks.append((ax, k.astype(float)))
    k2 = np.zeros(shape)
    for ax, k in ks:
        s = [1] * len(bases)
        s[ax] = len(k)
        k2 = k2 + (k ** 2).reshape(s)
    return k2


def _systems(u, axis):
    """View the solve axis last and flatten the others: (S, N)."""
    um = np.moveaxis(u, axis, -1)
    return um.reshape(-1, um.shape[-1]), um.shape


def helmholtz_solve(f_hat, bases, c, axis):
    """Solve (-lap + c) u = f with alfa = -1, beta = k^2 + c per wavenumber,
    Chebyshev SD via LU_Helmholtz/Solve_Helmholtz (chebyshev/la.py:223-317)."""
    N = bases[axis][2]
    beta = fourier_k2(bases, axis) + c
    bsys = np.moveaxis(np.broadcast_to(beta, beta.shape), axis, -1).reshape(-1)
    fs, shp = _systems(f_hat, axis)
    d0, d1, d2, L = la.helmholtz_lu(N, -np.ones_like(bsys), bsys)
    us = la.helmholtz_solve(fs, d0, d1, d2, L)
    return np.moveaxis(us.reshape(shp), -1, axis)


def biharmonic_solve(f_hat, bases, axis):
    """Solve lap^2 u = f for Chebyshev SB along axis: a0 S + alfa A + beta B
    with a0 = 1, alfa = -2 k^2, beta = k^4 (inner(v, div(grad(div(grad(u))))),
    chebyshev/la.py:442-502), one dense direct solve per wavenumber (the
    reference's odd-N path, la.SolverGeneric1ND with splu)."""
    N = bases[axis][2]
    k2 = fourier_k2(bases, axis)
    k2s = np.moveaxis(k2, axis, -1).reshape(-1)
    fs, shp = _systems(f_hat, axis)
    Sm, Am, Bm = la.cheb_sb_dense(N)
    us = la.dense_solve_systems([Sm, Am, Bm], [np.ones_like(k2s), -2 * k2s, k2s ** 2], fs)
    return np.moveaxis(us.reshape(shp), -1, axis)


def helmholtz_roundtrip(f, bases, c, axis, axes=None):
    """scalar product -> Helmholtz solve -> backward (the hot path's step)."""
    fh = scalar_product(f, bases, axes)
    uh = helmholtz_solve(fh, bases, c, axis)
    return backward(uh, bases, axes), fh, uh
