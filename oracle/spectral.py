"""1D spectral transforms along one axis of an N-D array (CPU oracle, numpy).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Every function restates the reference (shenfun 4.3.0) with numpy/scipy; the
file:line citations are paths inside the reference project.  FFTW's
unnormalised conventions (REDFT10 = DCT-II, REDFT01 = DCT-III, DFT) are the
ones ``scipy.fft`` uses with ``norm=None`` for dct and the forward fft.
"""
import numpy as np
import scipy.fft as sfft


# ---------------------------------------------------------------------------
# helpers
def _bshape(arr, axis, n):
    s = [1] * arr.ndim
    s[axis] = n
    return s


def _take(arr, axis, sl):
    idx = [slice(None)] * arr.ndim
    idx[axis] = sl
    return tuple(idx)


# ---------------------------------------------------------------------------
# Chebyshev, Gauss-Chebyshev quadrature (chebyshev/bases.py:155, :213-214)
def cheb_gc_points_weights(N):
    """x_j = cos(pi (2j+1) / (2N)), w_j = pi / N  (numpy chebgauss order)."""
    j = np.arange(N)
    return np.cos(np.pi * (2 * j + 1) / (2 * N)), np.full(N, np.pi / N)


def cheb_scalar_product_ortho(f, axis=-1):
    """(f, T_k)_w at GC nodes: FFTW REDFT10 scaled by pi/(2N).

    chebyshev/bases.py:340-347 (``out *= pi/(2 N)``), plan :426-434.
    """
    N = f.shape[axis]
    if np.iscomplexobj(f):
        # DCTWrap: real and imaginary parts transformed separately (:100-115)
        return cheb_scalar_product_ortho(f.real, axis) + 1j * cheb_scalar_product_ortho(f.imag, axis)
    return sfft.dct(f, type=2, axis=axis) * (np.pi / (2 * N))


def cheb_backward_ortho(c, axis=-1):
    """sum_k c_k T_k(x_j): FFTW REDFT01, then *0.5 + c_0/2 (chebyshev/bases.py:315-329)."""
    if np.iscomplexobj(c):
        return cheb_backward_ortho(c.real, axis) + 1j * cheb_backward_ortho(c.imag, axis)
    out = sfft.dct(c, type=3, axis=axis) * 0.5
    out += c[_take(c, axis, slice(0, 1))] / 2
    return out


# ---------------------------------------------------------------------------
# Shen composite stencils, phi_k = sum_m K_m(k) P_{k+m}
# (spectralbase.py:1504-1526: entries k >= dim are zeroed)
def stencil(family, basis, N):
    """Return {offset m: K_m (length N-m)}.

    The reference builds the stencil SparseMatrix by evaluating each entry's
    sympy expression over k (spectralbase.py:1504-1526) and zeroes rows
    k >= dim only when the result is an array; entries that are plain
    constants (the 1 and -1 of ShenDirichlet, the leading 1 of ShenBiharmonic)
    stay nonzero on every row.  The scalar product therefore leaves the
    orthogonal coefficients c_k in the tail rows k >= dim, and this
    restatement keeps that.
    """
    k = np.arange(N, dtype=float)
    if basis == "T" or basis == "L":
        return {0: np.ones(N)}
    if basis == "SD":
        # chebyshev/bases.py:546 {0: 1, 2: -1}; legendre/bases.py:374 (unscaled)
        return {0: np.ones(N), 2: -np.ones(N - 2)}
    if basis == "SN" and family == "chebyshev":
        # chebyshev/bases.py:937 {0: 1, 2: -(n/(n+2))**2}; the array diagonal
        # has N-2 entries, all kept (rows k >= N-2 do not exist in it)
        return {0: np.ones(N), 2: -(k[:N - 2] / (k[:N - 2] + 2)) ** 2}
    if basis == "SB" and family == "chebyshev":
        # chebyshev/bases.py:1249 {0: 1, 2: -(2n+4)/(n+3), 4: (n+1)/(n+3)}
        d = {0: np.ones(N), 2: -(2 * k[:N - 2] + 4) / (k[:N - 2] + 3),
             4: (k[:N - 4] + 1) / (k[:N - 4] + 3)}
    elif basis == "SB" and family == "legendre":
        # legendre/bases.py:564 {0: 1, 2: -(4n+10)/(2n+7), 4: (2n+3)/(2n+7)}
        d = {0: np.ones(N), 2: -(4 * k[:N - 2] + 10) / (2 * k[:N - 2] + 7),
             4: (2 * k[:N - 4] + 3) / (2 * k[:N - 4] + 7)}
    else:
        raise NotImplementedError((family, basis))
    d[2][N - 4:] = 0
    d[4][N - 4:] = 0
    return d


def num_bcs(basis):
    return {"T": 0, "L": 0, "SD": 2, "SN": 2, "SB": 4}[basis]


def apply_stencil(c, K, axis=-1):
    """out_k = sum_m K_m(k) c_{k+m}  (CompositeBase._evaluate_scalar_product,
    spectralbase.py:1462-1474, via SparseMatrix.matvec matrixbase.py:87-144)."""
    N = c.shape[axis]
    out = np.zeros_like(c)
    for m, v in K.items():
        n = N - m
        out[_take(out, axis, slice(0, n))] += v.reshape(_bshape(c, axis, n)) * c[_take(c, axis, slice(m, N))]
    return out


def to_ortho(u, K, dim, axis=-1):
    """c_{k+m} += K_m(k) u_k for k < dim (CompositeBase.to_ortho,
    spectralbase.py:1616-1634)."""
    out = np.zeros_like(u)
    for m, v in K.items():
        out[_take(out, axis, slice(m, m + dim))] += v[:dim].reshape(_bshape(u, axis, dim)) * u[_take(u, axis, slice(0, dim))]
    return out


# ---------------------------------------------------------------------------
# Mass matrices (band dicts over the dim = N - nbcs dofs)
def cheb_norm_sq(N):
    """(T_k, T_k)_w = c_k pi/2, c_0 = 2 (chebyshev.Orthogonal.L2_norm_sq)."""
    h = np.full(N, np.pi / 2)
    h[0] = np.pi
    return h


def leg_norm_sq(N):
    """(L_k, L_k) = 2/(2k+1) (legendre.Orthogonal.L2_norm_sq)."""
    return 2.0 / (2 * np.arange(N) + 1.0)


def mass_bands(family, basis, N):
    """Band dict of the Shen mass matrix B_kj = (phi_j, phi_k)_w.

    Chebyshev SD: chebyshev/matrices.py:238-246; SB: :515-528.
    Legendre SD: legendre/matrices.py:121-135; SB: legendre/matrices.py:179-192.
    """
    if basis in ("T", "L"):
        h = cheb_norm_sq(N) if family == "chebyshev" else leg_norm_sq(N)
        return {0: h}
    if family == "chebyshev" and basis == "SD":
        h = cheb_norm_sq(N)
        return {-2: np.full(N - 4, -h[1]), 0: h[:-2] + h[2:], 2: np.full(N - 4, -h[1])}
    if family == "chebyshev" and basis == "SN":
        # BSNSNmat (chebyshev/matrices.py:377-401): alpha = (k/(k+2))^2,
        # {0: h + alpha^2 h_{k+2}, +-2: -alpha h_{k+2}}
        h = cheb_norm_sq(N)
        k = np.arange(N, dtype=float)
        alpha = (k / (k + 2)) ** 2
        d = {0: h[:-2] + alpha[:-2] ** 2 * h[2:], 2: -alpha[:N - 4] * h[2:N - 2]}
        d[-2] = d[2].copy()
        return d
    if family == "legendre" and basis == "SD":
        d0 = leg_norm_sq(N)
        return {0: d0[:-2] + d0[2:], -2: -d0[2:-2], 2: -d0[2:-2]}
    if family == "chebyshev" and basis == "SB":
        h = cheb_norm_sq(N)
        S = stencil("chebyshev", "SB", N)
        d = {0: h[:-4] + h[2:-2] * S[2][:-2] ** 2 + h[4:] * S[4] ** 2,
             2: h[2:-4] * S[2][:-4] + h[4:-2] * S[4][:-2] * S[2][2:-2],
             4: h[4:-4] * S[4][:-4]}
        d[0] = d[0][:N - 4]
        d[2] = d[2][:N - 6]
        d[4] = d[4][:N - 8]
        d[-2] = d[2].copy()
        d[-4] = d[4].copy()
        return d
    if family == "legendre" and basis == "SB":
        d0 = leg_norm_sq(N)
        i = np.arange(N - 4, dtype=float)
        d = {0: (-4 * i - 10) ** 2 * d0[2:-2] / (2 * i + 7) ** 2 + (2 * i + 3) ** 2 * d0[4:] / (2 * i + 7) ** 2 + d0[:-4],
             2: (-4 * i[:-2] - 18) * (2 * i[:-2] + 3) * d0[4:-2] / ((2 * i[:-2] + 7) * (2 * i[:-2] + 11)) + (-4 * i[:-2] - 10) * d0[2:-4] / (2 * i[:-2] + 7),
             4: (2 * i[:-4] + 3) * d0[4:-4] / (2 * i[:-4] + 7)}
        d[-2] = d[2].copy()
        d[-4] = d[4].copy()
        return d
    raise NotImplementedError((family, basis))


def mass_solve(b, family, basis, axis=-1):
    """Apply B^{-1} on the first dim entries along axis (apply_inverse_mass,
    spectralbase.py:560-577 -> TDMA/PDMA, la.py:331-543)."""
    from . import la
    N = b.shape[axis]
    nb = num_bcs(basis)
    out = b.copy()
    if nb == 0:
        h = mass_bands(family, basis, N)[0]
        return out / h.reshape(_bshape(b, axis, N))
    dim = N - nb
    bands = mass_bands(family, basis, N)
    sub = np.moveaxis(out, axis, 0)[:dim].copy()
    if nb == 2:
        data = np.zeros((3, dim))
        data[0, :-2] = bands[-2]
        data[1] = bands[0]
        data[2, 2:] = bands[2]
        la.tdma_lu(data)
        sub = la.tdma_solve(sub, data, axis=0)
    else:
        data = np.zeros((5, dim))
        data[0, :-4] = bands[-4]
        data[1, :-2] = bands[-2]
        data[2] = bands[0]
        data[3, 2:] = bands[2]
        data[4, 4:] = bands[4]
        la.pdma_lu(data)
        sub = la.pdma_solve(sub, data, axis=0)
    o = np.moveaxis(out, axis, 0)
    o[:dim] = sub
    o[dim:] = 0  # homogeneous boundary dofs (tensorproductspace.py:2108-2128)
    return out


# ---------------------------------------------------------------------------
# Chebyshev composite transforms (GC quadrature, 'fast' kind)
def cheb_scalar_product(f, basis="SD", axis=-1):
    c = cheb_scalar_product_ortho(f, axis)
    if basis == "T":
        return c
    return apply_stencil(c, stencil("chebyshev", basis, f.shape[axis]), axis)


def cheb_forward(f, basis="SD", axis=-1):
    return mass_solve(cheb_scalar_product(f, basis, axis), "chebyshev", basis, axis)


def cheb_backward(u, basis="SD", axis=-1):
    """to_ortho then ortho backward (CompositeBase._evaluate_expansion_all,
    spectralbase.py:1450-1460)."""
    if basis == "T":
        return cheb_backward_ortho(u, axis)
    N = u.shape[axis]
    return cheb_backward_ortho(to_ortho(u, stencil("chebyshev", basis, N), N - num_bcs(basis), axis), axis)


# ---------------------------------------------------------------------------
# Fourier (fourier/bases.py:131-162 forward *1/N; :380-407, :526-533 backward
# unnormalised)
def r2c_forward(f, axis=-1):
    return sfft.rfft(f, axis=axis) / f.shape[axis]


def r2c_backward(u, N, axis=-1):
    return sfft.irfft(u, n=N, axis=axis, norm="forward")


def c2c_forward(f, axis=-1):
    return sfft.fft(f, axis=axis) / f.shape[axis]


def c2c_backward(u, axis=-1):
    return sfft.ifft(u, axis=axis, norm="forward")


def r2c_wavenumbers(N):
    return np.fft.rfftfreq(N, 1.0 / N).astype(int)   # fourier/bases.py:334-342


def c2c_wavenumbers(N):
    return np.fft.fftfreq(N, 1.0 / N).astype(int)


# ---------------------------------------------------------------------------
# Legendre, Gauss-Legendre quadrature
def leg_lg_points_weights(N):
    """LG nodes/weights in ascending order.  The reference computes them with
    Bogaert's iteration-free method (legendre/fastgl/fastgl.cpp, wrapped at
    fastgl_wrap.pyx:31-53); numpy's Golub-Welsch + Newton polish agrees to
    O(1e-16) and is pinned against the reference's values in the tests."""
    x, w = np.polynomial.legendre.leggauss(N)
    return x, w


def _leg_recursion_coeffs(M):
    """x P_n = anm_n P_{n+1} + anp_n P_{n-1}: anm_n = (n+1)/(2n+1), anp_n = n/(2n+1)."""
    n = np.arange(M, dtype=float)
    return (n + 1) / (2 * n + 1), n / (2 * n + 1)


def leg_scalar_product_ortho(f, axis=-1, kind="recursive"):
    """sum_j w_j f_j L_k(x_j).

    'recursive': on-the-fly three-term recurrence (transforms.pyx:262-325).
    'vandermonde': dot with legvander (spectralbase.py:539-549).
    """
    N = f.shape[axis]
    x, w = leg_lg_points_weights(N)
    fm = np.moveaxis(f, axis, -1)
    if kind == "vandermonde":
        P = np.polynomial.legendre.legvander(x, N - 1)
        out = np.dot(fm * w, P)
        return np.moveaxis(out, -1, axis)
    anm, anp = _leg_recursion_coeffs(N + 3)
    out = np.zeros(fm.shape, dtype=np.result_type(fm, float))
    Lnm = np.ones(N)
    Ln = x / anm[0]
    Lnp = x / anm[1] * Ln - anp[1] / anm[1] * Lnm
    wf = fm * w
    for i in range(N):
        s1 = 1 / anm[i + 2]
        s2 = anp[i + 2] / anm[i + 2]
        out[..., i] = wf @ Lnm
        Lnm, Ln, Lnp = Ln, Lnp, s1 * x * Lnp - s2 * Ln
    return np.moveaxis(out, -1, axis)


def leg_backward_ortho(c, axis=-1, kind="recursive"):
    """sum_k c_k L_k(x_j) (transforms.pyx:214-260; vandermonde spectralbase.py:472-483)."""
    N = c.shape[axis]
    x, _ = leg_lg_points_weights(N)
    P = np.polynomial.legendre.legvander(x, N - 1)
    cm = np.moveaxis(c, axis, -1)
    if kind == "vandermonde":
        return np.moveaxis(cm @ P.T, -1, axis)
    anm, anp = _leg_recursion_coeffs(N + 3)
    out = np.zeros(cm.shape, dtype=np.result_type(cm, float))
    Lnm = np.ones(N)
    Ln = x / anm[0]
    Lnp = x / anm[1] * Ln - anp[1] / anm[1] * Lnm
    for i in range(N):
        s1 = 1 / anm[i + 2]
        s2 = anp[i + 2] / anm[i + 2]
        out += cm[..., i:i + 1] * Lnm
        Lnm, Ln, Lnp = Ln, Lnp, s1 * x * Lnp - s2 * Ln
    return np.moveaxis(out, -1, axis)


def leg_scalar_product(f, basis="SD", axis=-1, kind="recursive"):
    c = leg_scalar_product_ortho(f, axis, kind)
    if basis == "L":
        return c
    N = f.shape[axis]
    out = apply_stencil(c, stencil("legendre", basis, N), axis)
    if kind == "vandermonde":
        # composite Vandermonde path zeroes the tail rows (spectralbase.py:1466-1469)
        out[_take(out, axis, slice(N - num_bcs(basis), N))] = 0
    return out


def leg_forward(f, basis="SD", axis=-1, kind="recursive"):
    return mass_solve(leg_scalar_product(f, basis, axis, kind), "legendre", basis, axis)


def leg_backward(u, basis="SD", axis=-1, kind="recursive"):
    if basis == "L":
        return leg_backward_ortho(u, axis, kind)
    N = u.shape[axis]
    return leg_backward_ortho(to_ortho(u, stencil("legendre", basis, N), N - num_bcs(basis), axis), axis, kind)
