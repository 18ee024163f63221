"""Banded solvers of the spectral-Galerkin path (CPU oracle, numpy).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Sequential recurrences are restated exactly as the reference's Cython loops,
vectorised over the independent systems (one system per Fourier wavenumber),
so the per-system operation order - and therefore the rounding - follows the
reference.  Citations are paths inside the reference project.
"""
import numpy as np

from . import spectral


def _mv(u, axis):
    return np.moveaxis(u, axis, 0)


# ---------------------------------------------------------------------------
# TDMA: offsets (-2, 0, 2); data[0, :-2] = ld, data[1] = d, data[2, 2:] = ud
def tdma_lu(data):
    """In-place LU (la.pyx:243-252; la.py:344-352)."""
    ld = data[0, :-2]
    d = data[1, :]
    ud = data[2, 2:]
    n = d.shape[0]
    for i in range(2, n):
        ld[i - 2] = ld[i - 2] / d[i - 2]
        d[i] = d[i] - ld[i - 2] * ud[i - 2]
    return data


def tdma_solve(u, data, axis=0):
    """Solve along axis with LU'd data (TDMA_inner_solve_ptr, la.pyx:516-532)."""
    u = np.array(u, copy=True)
    v = _mv(u, axis)
    n = data.shape[1]
    ld = data[0, :-2]
    d = data[1, :]
    ud = data[2, 2:]
    bs = (slice(None),) + (None,) * (v.ndim - 1)
    del bs
    for i in range(2, n):
        v[i] -= ld[i - 2] * v[i - 2]
    v[n - 1] = v[n - 1] / d[n - 1]
    v[n - 2] = v[n - 2] / d[n - 2]
    for i in range(n - 3, -1, -1):
        v[i] = (v[i] - ud[i] * v[i + 2]) / d[i]
    return u


# ---------------------------------------------------------------------------
# PDMA: offsets (-4, -2, 0, 2, 4); data rows a, b, d, e, f (la.pyx:213-241)
def pdma_lu(data):
    a = data[0, :-4]
    b = data[1, :-2]
    d = data[2, :]
    e = data[3, 2:]
    f = data[4, 4:]
    n = d.shape[0]
    m = e.shape[0]
    k = n - m
    for i in range(n - 2 * k):
        lam = b[i] / d[i]
        d[i + k] -= lam * e[i]
        e[i + k] -= lam * f[i]
        b[i] = lam
        lam = a[i] / d[i]
        b[i + k] -= lam * e[i]
        d[i + 2 * k] -= lam * f[i]
        a[i] = lam
    i = n - 4
    lam = b[i] / d[i]
    d[i + k] -= lam * e[i]
    b[i] = lam
    i = n - 3
    lam = b[i] / d[i]
    d[i + k] -= lam * e[i]
    b[i] = lam
    return data


def pdma_solve(u, data, axis=0):
    """PDMA_inner_solve_ptr (la.pyx:496-514)."""
    u = np.array(u, copy=True)
    v = _mv(u, axis)
    n = data.shape[1]
    a = data[0]
    b = data[1]
    d = data[2]
    e = data[3, 2:]
    f = data[4, 4:]
    v[2] -= b[0] * v[0]
    v[3] -= b[1] * v[1]
    for k in range(4, n):
        v[k] -= (b[k - 2] * v[k - 2] + a[k - 4] * v[k - 4])
    v[n - 1] /= d[n - 1]
    v[n - 2] /= d[n - 2]
    v[n - 3] = (v[n - 3] - e[n - 3] * v[n - 1]) / d[n - 3]
    v[n - 4] = (v[n - 4] - e[n - 4] * v[n - 2]) / d[n - 4]
    for k in range(n - 5, -1, -1):
        v[k] = (v[k] - e[k] * v[k + 2] - f[k] * v[k + 4]) / d[k]
    return u


# ---------------------------------------------------------------------------
# Chebyshev Dirichlet Helmholtz (alfa A + beta B) u = f, A = ASDSD, B = BSDSD
def cheb_sd_stiffness(N):
    """ASDSD diagonals used by the solver: A[0], A[2] (= A[k], k>=2 constant
    rows), A[4] (chebyshev/matrices.py:1061-1079)."""
    k = np.arange(N, dtype=float)
    return {0: -2 * np.pi * (k[:N - 2] + 1) * (k[:N - 2] + 2),
            2: -4 * np.pi * (k[:N - 4] + 1),
            4: -4 * np.pi * (k[:N - 6] + 1)}


def helmholtz_lu(N, alfa, beta):
    """LU of alfa*A + beta*B for many systems (LU_Helmholtz_1D, la.pyx:717-763).

    alfa, beta: arrays of shape (S,).  Returns d0, d1, d2, L of shape (S, N)
    (the reference's factor arrays have the basis length N; entries beyond the
    N-2 dofs stay zero).
    """
    alfa = np.asarray(alfa, float).reshape(-1)
    beta = np.asarray(beta, float).reshape(-1)
    S = max(alfa.size, beta.size)
    alfa = np.broadcast_to(alfa, (S,))
    beta = np.broadcast_to(beta, (S,))
    A = cheb_sd_stiffness(N)
    B = spectral.mass_bands("chebyshev", "SD", N)
    A0, A2, A4 = A[0], A[2], A[4]
    Bm2, B0, B2 = B[-2], B[0], B[2]
    M = N - 2
    d0 = np.zeros((S, N))
    d1 = np.zeros((S, N))
    d2 = np.zeros((S, N))
    L = np.zeros((S, N))
    d0[:, 0] = alfa * A0[0] + beta * B0[0]
    d0[:, 1] = alfa * A0[1] + beta * B0[1]
    d1[:, 0] = alfa * A2[0] + beta * B2[0]
    d1[:, 1] = alfa * A2[1] + beta * B2[1]
    d2[:, 0] = alfa * A4[0]
    d2[:, 1] = alfa * A4[1]
    for i in range(2, M):
        L[:, i - 2] = beta * Bm2[i - 2] / d0[:, i - 2]
        d0[:, i] = alfa * A0[i] + beta * B0[i] - L[:, i - 2] * d1[:, i - 2]
        if i < M - 2:
            d1[:, i] = alfa * A2[i] + beta * B2[i] - L[:, i - 2] * d2[:, i - 2]
        if i < M - 4:
            d2[:, i] = alfa * A4[i] - L[:, i - 2] * d2[:, i - 2]
    return d0, d1, d2, L


def helmholtz_solve(f, d0, d1, d2, L):
    """Solve_Helmholtz_1D_ptr (la.pyx:871-912) for systems along the last axis.

    f: (S, N) (complex or real); d*: (S, N).  Returns u (S, N), tail zeros.
    """
    S, Nb = d0.shape
    N = Nb - 2
    y = np.zeros(f.shape[:-1] + (N,), dtype=f.dtype)
    u = np.zeros_like(f)
    y[:, 0] = f[:, 0]
    y[:, 1] = f[:, 1]
    for i in range(2, N):
        y[:, i] = f[:, i] - L[:, i - 2] * y[:, i - 2]
    u[:, N - 1] = y[:, N - 1] / d0[:, N - 1]
    u[:, N - 2] = y[:, N - 2] / d0[:, N - 2]
    u[:, N - 3] = (y[:, N - 3] - d1[:, N - 3] * u[:, N - 1]) / d0[:, N - 3]
    u[:, N - 4] = (y[:, N - 4] - d1[:, N - 4] * u[:, N - 2]) / d0[:, N - 4]
    se = np.zeros(S, dtype=f.dtype)
    so = np.zeros(S, dtype=f.dtype)
    for i in range(N - 5, -1, -1):
        ui = y[:, i] - d1[:, i] * u[:, i + 2]
        if i % 2 == 0:
            se = se + u[:, i + 4]
            ui = ui - d2[:, i] * se
        else:
            so = so + u[:, i + 4]
            ui = ui - d2[:, i] * so
        u[:, i] = ui / d0[:, i]
    return u


def helmholtz_matvec(v, alfa, beta):
    """b = (alfa A + beta B) v for systems along the last axis
    (Helmholtz_matvec_ptr, Matvec.pyx:656-695)."""
    S, Nb = v.shape
    M = Nb - 2
    A = cheb_sd_stiffness(Nb)
    dd, ud = A[0], A[2]
    bd = spectral.mass_bands("chebyshev", "SD", Nb)[0]
    alf = np.broadcast_to(np.asarray(alfa, float).reshape(-1), (S,))
    bet = np.broadcast_to(np.asarray(beta, float).reshape(-1), (S,))
    b = np.zeros_like(v)
    h = np.pi / 2
    k = M - 1
    b[:, k] = (dd[k] * alf + bd[k] * bet) * v[:, k] - h * bet * v[:, k - 2]
    b[:, k - 1] = (dd[k - 1] * alf + bd[k - 1] * bet) * v[:, k - 1] - h * bet * v[:, k - 3]
    s1 = np.zeros(S, dtype=v.dtype)
    s2 = np.zeros(S, dtype=v.dtype)
    for k in range(M - 3, 1, -1):
        p = ud[k] * alf
        if k % 2 == 0:
            s2 = s2 + v[:, k + 2]
            b[:, k] = (dd[k] * alf + bd[k] * bet) * v[:, k] - h * bet * (v[:, k - 2] + v[:, k + 2]) + p * s2
        else:
            s1 = s1 + v[:, k + 2]
            b[:, k] = (dd[k] * alf + bd[k] * bet) * v[:, k] - h * bet * (v[:, k - 2] + v[:, k + 2]) + p * s1
    k = 1
    s1 = s1 + v[:, k + 2]
    s2 = s2 + v[:, k + 1]
    b[:, k] = (dd[k] * alf + bd[k] * bet) * v[:, k] - h * bet * v[:, k + 2] + ud[k] * alf * s1
    b[:, k - 1] = (dd[k - 1] * alf + bd[k - 1] * bet) * v[:, k - 1] - h * bet * v[:, k + 1] + ud[k - 1] * alf * s2
    return b


# ---------------------------------------------------------------------------
# Dense reference matrices (for biharmonic / generic per-wavenumber solves)
def cheb_sd_dense(N):
    """Dense (N-2)x(N-2) A (ASDSD) and B (BSDSD)."""
    M = N - 2
    k = np.arange(M, dtype=float)
    A = np.zeros((M, M))
    for i in range(M):
        A[i, i] = -2 * np.pi * (k[i] + 1) * (k[i] + 2)
        A[i, i + 2::2] = -4 * np.pi * (k[i] + 1)
    Bd = spectral.mass_bands("chebyshev", "SD", N)
    B = np.diag(Bd[0]) + np.diag(Bd[2], 2) + np.diag(Bd[-2], -2)
    return A, B


def cheb_sb_dense(N):
    """Dense (N-4)x(N-4) S (SSBSB, chebyshev/matrices.py:1444-1458), A (ASBSB,
    :1008-1017) and B (BSBSB, :515-528)."""
    M = N - 4
    ki = np.arange(M, dtype=float)
    S = np.zeros((M, M))
    for i in range(M):
        S[i, i] = np.pi * 8 * (ki[i] + 1) ** 2 * (ki[i] + 2) * (ki[i] + 4)
        for j in range(i + 2, M, 2):
            S[i, j] = 8 * (ki[i] + 1) * (ki[i] + 2) * (ki[i] * (ki[i] + 4) + 3 * (ki[j] + 2) ** 2) * np.pi / (ki[j] + 3)
    A = np.diag(-4 * ((ki + 1) * (ki + 2) ** 2) / (ki + 3) * np.pi)
    A += np.diag(2 * (ki[:-2] + 1) * (ki[:-2] + 2) * np.pi, 2)
    A += np.diag(2 * (ki[2:] - 1) * (ki[2:] + 2) * np.pi, -2)
    Bd = spectral.mass_bands("chebyshev", "SB", N)
    B = np.diag(Bd[0]) + np.diag(Bd[2], 2) + np.diag(Bd[-2], -2) + np.diag(Bd[4], 4) + np.diag(Bd[-4], -4)
    return S, A, B


def dense_solve_systems(mats, scales, f):
    """Solve (sum_i scales[i][s] * mats[i]) u_s = f_s for every system s.

    mats: list of (M, M); scales: list of arrays (S,); f: (S, Nb) with the
    first M entries the dofs.  Equivalent to the reference's per-wavenumber
    SolverGeneric1ND with a direct LU (la.py:1183-1434, splu per system).
    """
    S = f.shape[0]
    M = mats[0].shape[0]
    Amat = np.zeros((S, M, M))
    for m, sc in zip(mats, scales):
        Amat += np.broadcast_to(np.asarray(sc, float).reshape(-1), (S,))[:, None, None] * m
    u = np.zeros_like(f)
    u[:, :M] = np.linalg.solve(Amat, f[:, :M, None])[..., 0]
    return u


# ---------------------------------------------------------------------------
# Legendre Dirichlet: (alfa A + beta B) with A = diag(4k+6), B tridiagonal
# (legendre/matrices.py:121-135, :285-292) -> TDMA per system
def leg_sd_bands(N):
    k = np.arange(N - 2, dtype=float)
    B = spectral.mass_bands("legendre", "SD", N)
    return {0: 4 * k + 6}, B


def leg_helmholtz_solve(f, alfa, beta):
    """Solve (alfa A + beta B) u = f per system (SolverGeneric1ND -> TDMA,
    la.py:1346-1364, la.pyx:516-532), systems along the first axis of f."""
    S, Nb = f.shape
    M = Nb - 2
    A, B = leg_sd_bands(Nb)
    alf = np.broadcast_to(np.asarray(alfa, float).reshape(-1), (S,))
    bet = np.broadcast_to(np.asarray(beta, float).reshape(-1), (S,))
    u = np.zeros_like(f)
    for s in range(S):
        data = np.zeros((3, M))
        data[0, :-2] = bet[s] * B[-2]
        data[1] = alf[s] * A[0] + bet[s] * B[0]
        data[2, 2:] = bet[s] * B[2]
        tdma_lu(data)
        u[s, :M] = tdma_solve(f[s, :M], data)
    return u
