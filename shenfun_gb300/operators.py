"""Host-side 1D operators of linear forms and projections of expressions
(forms/inner.py:356-491 with a Function as trial argument,
forms/project.py:124-199), built once per (test space, trial space,
derivative order) in FP64 and applied along an axis on the GPU by
``sgpu_line_gemm``.

Every polynomial basis on the path is a stencil over the orthogonal
polynomials P_m (Chebyshev T_m or Legendre L_m): phi_k = sum_m S[k][m] P_m.
With D the derivative matrix of orthogonal coefficient vectors and h the
norms (P_m, P_m)_w:

    linear form   W_c = S_test diag(h) (D^c S_trial^T)     (phi_k, d^c u / dx^c)_w
    projection    P_c = B^{-1} W_c,  B = S_test diag(h) S_test^T

exact in exact arithmetic (the reference assembles the same inner products
from closed forms and solves with its mass matrix).  A Fourier axis carries
the factor (i k)^c of its wavenumbers, with the reference's normalisation
(the mass matrix of a Fourier space is the identity, fourier/bases.py).
"""
import functools

import numpy as np
from numpy.polynomial import chebyshev as npcheb
from numpy.polynomial import legendre as npleg


def stencil(base):
    """S (dim x N) of a polynomial basis; spectralbase.py:1504-1526 and the
    bases' stencils (chebyshev/bases.py, legendre/bases.py)."""
    fam, name, N = base.family(), base.short_name(), base.N
    k = np.arange(N, dtype=float)
    if name in ("T", "L"):
        return np.eye(N)
    n = base.dim()
    S = np.zeros((n, N))
    S[np.arange(n), np.arange(n)] = 1.0
    r = np.arange(n)
    if name == "SD":
        S[r, r + 2] = -1.0
    elif name == "SN":
        S[r, r + 2] = -(k[:n] / (k[:n] + 2)) ** 2
    elif name == "SB" and fam == "chebyshev":
        S[r, r + 2] = -(2 * k[:n] + 4) / (k[:n] + 3)
        S[r, r + 4] = (k[:n] + 1) / (k[:n] + 3)
    elif name == "SB" and fam == "legendre":
        S[r, r + 2] = -2 * (2 * k[:n] + 5) / (2 * k[:n] + 7)
        S[r, r + 4] = (2 * k[:n] + 3) / (2 * k[:n] + 7)
    else:
        raise NotImplementedError(f"{fam} {name}")
    return S


def norms(fam, N):
    if fam == "chebyshev":
        h = np.full(N, np.pi / 2)
        h[0] = np.pi
        return h
    return 2.0 / (2 * np.arange(N) + 1.0)


def derivative(fam, N, c):
    """D^c (N x N): column m holds the orthogonal coefficients of P_m^(c)."""
    D = np.zeros((N, N))
    der = npcheb.chebder if fam == "chebyshev" else npleg.legder
    for m in range(c, N):
        e = np.zeros(N)
        e[m] = 1.0
        d = der(e, c)
        D[:d.size, m] = d
    return D


@functools.lru_cache(maxsize=64)
def _polynomial_operator(key_test, key_trial, c, solve):
    (fam, N_t, name_t, dim_t), (fam_u, N_u, name_u, dim_u) = key_test, key_trial
    if fam != fam_u:
        raise NotImplementedError("projection between polynomial families")
    test, trial = _Base(fam, name_t, N_t, dim_t), _Base(fam, name_u, N_u, dim_u)
    St, Su = stencil(test), stencil(trial)
    M = max(N_t, N_u)
    h = norms(fam, M)
    Du = derivative(fam, N_u, c) @ Su.T            # (N_u, dim_u): P-coefficients of phi_j^(c)
    Dfull = np.zeros((M, dim_u))
    Dfull[:N_u] = Du
    Stf = np.zeros((dim_t, M))
    Stf[:, :N_t] = St
    W = Stf @ (h[:, None] * Dfull)                 # (dim_t, dim_u)
    if not solve:
        return W
    B = Stf @ (h[:, None] * Stf.T)
    return np.linalg.solve(B, W)


class _Base:
    def __init__(self, fam, name, N, dim):
        self._fam, self._name, self.N, self._dim = fam, name, N, dim

    def family(self):
        return self._fam

    def short_name(self):
        return self._name

    def dim(self):
        return self._dim


def _key(base):
    return (base.family(), base.N, base.short_name(), base.dim())


def axis_operator(test_base, trial_base, c, solve):
    """(M, factor) of one axis: M (trial N x test N, row-major) maps a line of
    trial coefficients to test coefficients, as ``sgpu_line_gemm`` applies
    it, and ``factor`` is the complex number multiplying it (i^c on a Fourier
    axis, 1 otherwise)."""
    if test_base.family() == "fourier":
        if trial_base.family() != "fourier" or trial_base.N != test_base.N:
            raise NotImplementedError("projection between different Fourier spaces")
        k = np.asarray(test_base.wavenumbers(scaled=True), dtype=float)
        return np.diag(k ** c), 1j ** c
    P = _polynomial_operator(_key(test_base), _key(trial_base), int(c), bool(solve))
    M = np.zeros((trial_base.N, test_base.N))
    M[:P.shape[1], :P.shape[0]] = P.T
    return M, 1.0


def expr_plan(T, U, terms, solve, src_complex):
    """Host plan of a linear form / projection of sum_t c_t d^{d_t} uh, uh in
    U, onto T: (line axis, output shape, complex?, [(M, line scales)]) with
    one entry per derivative order along the line axis (the one non-periodic
    axis, else the last).  M (U's N x T's N) is that axis' operator; the
    line scales hold, per line in (outer, inner) order, the sum of c_t times
    the Fourier factors (i k)^d of the other axes and the line axis' own
    factor, as re/im pairs when complex."""
    from .spaces import TensorProductSpace
    bases_T = list(T.bases) if isinstance(T, TensorProductSpace) else [T]
    bases_U = list(U.bases) if isinstance(U, TensorProductSpace) else [U]
    if len(bases_T) != len(bases_U):
        raise NotImplementedError("projection between spaces of different dimensions")
    nd = len(bases_T)
    np_axes = [i for i, b in enumerate(bases_T) if b.family() != "fourier"]
    if len(np_axes) > 1:
        raise NotImplementedError("more than one non-periodic axis")
    ax = np_axes[0] if np_axes else nd - 1
    for b in bases_T + bases_U:
        if b.family() != "fourier" and tuple(getattr(b, "domain", (-1.0, 1.0))) != (-1.0, 1.0):
            raise NotImplementedError("only the reference domain [-1, 1] is on the GPU path")
        if getattr(b, "has_nonhomogeneous_bcs", False):
            raise NotImplementedError("expressions of a Function with non-homogeneous boundary values")
    for i in range(nd):
        if i != ax and (bases_T[i].family() != "fourier" or bases_U[i].N != bases_T[i].N):
            raise NotImplementedError("the periodic axes of the two spaces must agree")
    out_shape = list(T.shape(True)) if isinstance(T, TensorProductSpace) else [T.shape(True)]
    sys_shape = list(out_shape)
    sys_shape[ax] = 1
    groups = {}
    for coef, d in terms:
        sc = np.full(sys_shape, complex(coef))
        for i, b in enumerate(bases_T):
            if i != ax and d[i]:
                k = np.asarray(b.wavenumbers(scaled=True), dtype=float)
                sh = [1] * nd
                sh[i] = len(k)
                sc = sc * (1j * k.reshape(sh)) ** d[i]
        groups[d[ax]] = groups.get(d[ax], 0) + sc
    ops = {c: axis_operator(bases_T[ax], bases_U[ax], c, solve) for c in groups}
    scales = {c: (sc * ops[c][1]).reshape(-1) for c, sc in groups.items()}
    cplx = bool(src_complex) or any(np.abs(sc.imag).max() > 0 for sc in scales.values())
    out = []
    for c in groups:
        sc = scales[c]
        lines = np.ascontiguousarray(np.stack([sc.real, sc.imag], -1).reshape(-1)) if cplx else sc.real.copy()
        out.append((ops[c][0], lines))
    return ax, out_shape, cplx, out
