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


def cheb_sn_stiffness(N):
    """ASNSN diagonals 0, 2, 4 as the reference evaluates them
    (chebyshev/matrices.py:1110-1122): a_kk = -2 pi k^2 (k+1)/(k+2),
    a_{k,k+i} = -4 pi (k+i)^2 (k+1)/(k+2)^2."""
    k = np.arange(N - 2, dtype=float)

    def key(i):
        if i == 0:
            return -2 * np.pi * k ** 2 * (k + 1) / (k + 2)
        return -4 * np.pi * (k[:-i] + i) ** 2 * (k[:-i] + 1) / (k[:-i] + 2) ** 2
    return {0: key(0), 2: key(2), 4: key(4)}


def helmholtz_lu(N, alfa, beta, neumann=False):
    """LU of alfa*A + beta*B for many systems (LU_Helmholtz_1D, la.pyx:717-763).

    alfa, beta: arrays of shape (S,).  Returns d0, d1, d2, L of shape (S, N)
    (the reference's factor arrays have the basis length N; entries beyond the
    N-2 dofs stay zero).  neumann: A = ASNSN, B = BSNSN with the Neumann
    branch (la.pyx:735-751): columns j >= 1 divided by j^2, and for
    |beta| < 1e-8 the singular row 0 replaced by a_00 = 1/alfa, b_00 = 0.
    """
    alfa = np.asarray(alfa, float).reshape(-1)
    beta = np.asarray(beta, float).reshape(-1)
    S = max(alfa.size, beta.size)
    alfa = np.broadcast_to(alfa, (S,))
    beta = np.broadcast_to(beta, (S,))
    M = N - 2
    if neumann:
        A = cheb_sn_stiffness(N)
        B = spectral.mass_bands("chebyshev", "SN", N)
        i2 = np.arange(M, dtype=float) ** 2
        A0 = np.tile(A[0], (S, 1))
        B0 = np.tile(B[0], (S, 1))
        sing = np.abs(beta) < 1e-8
        A0[sing, 0] = 1.0 / alfa[sing]
        B0[sing, 0] = 0.0
        A0[:, 1:] /= i2[1:]
        B0[:, 1:] /= i2[1:]
        A2 = A[2] / i2[2:]
        B2 = B[2] / i2[2:M]
        A4 = A[4] / i2[4:]
        Bm2 = B[-2].copy()
        Bm2[1:] /= i2[1:M - 2]
        A0c = lambda i: A0[:, i]  # noqa: E731
        B0c = lambda i: B0[:, i]  # noqa: E731
    else:
        A = cheb_sd_stiffness(N)
        B = spectral.mass_bands("chebyshev", "SD", N)
        A2, A4 = A[2], A[4]
        Bm2, B2 = B[-2], B[2]
        A0c = lambda i: A[0][i]  # noqa: E731
        B0c = lambda i: B[0][i]  # noqa: E731
    d0 = np.zeros((S, N))
    d1 = np.zeros((S, N))
    d2 = np.zeros((S, N))
    L = np.zeros((S, N))
    d0[:, 0] = alfa * A0c(0) + beta * B0c(0)
    d0[:, 1] = alfa * A0c(1) + beta * B0c(1)
    d1[:, 0] = alfa * A2[0] + beta * B2[0]
    d1[:, 1] = alfa * A2[1] + beta * B2[1]
    d2[:, 0] = alfa * A4[0]
    d2[:, 1] = alfa * A4[1]
    for i in range(2, M):
        L[:, i - 2] = beta * Bm2[i - 2] / d0[:, i - 2]
        d0[:, i] = alfa * A0c(i) + beta * B0c(i) - L[:, i - 2] * d1[:, i - 2]
        if i < M - 2:
            d1[:, i] = alfa * A2[i] + beta * B2[i] - L[:, i - 2] * d2[:, i - 2]
        if i < M - 4:
            d2[:, i] = alfa * A4[i] - L[:, i - 2] * d2[:, i - 2]
    return d0, d1, d2, L


def helmholtz_solve(f, d0, d1, d2, L, neumann=False):
    """Solve_Helmholtz_1D_ptr (la.pyx:871-912) for systems along the last axis.

    f: (S, N) (complex or real); d*: (S, N).  Returns u (S, N), tail zeros.
    neumann: the unknowns are w_j = j^2 u_j; u_0 = 0 where d0[0] == 1 to 1e-8
    (la.pyx:907-912).
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
    if neumann:
        u[(d0[:, 0] - 1.0) ** 2 < 1e-16, 0] = 0.0
        for i in range(1, N):
            u[:, i] /= i * i
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


# ---------------------------------------------------------------------------
# Chebyshev ShenNeumann matrices and the Poisson solvers
def cheb_sn_dense(N):
    """Dense ASNSN and BSNSN (chebyshev/matrices.py:1096-1122, :377-401) of
    the N-2 dofs: a_kj = -4 pi j^2 (k+1)/(k+2)^2 for j = k+2, k+4, ..."""
    M = N - 2
    k = np.arange(M, dtype=float)
    A = np.zeros((M, M))
    A[k.astype(int), k.astype(int)] = -2 * np.pi * k ** 2 * (k + 1) / (k + 2)
    for i in range(M):
        for j in range(i + 2, M, 2):
            A[i, j] = -4 * np.pi * j ** 2 * (i + 1) / (i + 2) ** 2
    Bb = spectral.mass_bands("chebyshev", "SN", N)
    B = np.diag(Bb[0]) + np.diag(Bb[2], 2) + np.diag(Bb[-2], -2)
    return A, B


def helmholtz_neumann_matvec(v, alfa, beta):
    """b = (alfa ASNSN + beta BSNSN) v along the last axis, tail entries zero:
    the definition Helmholtz_Neumann_matvec (Matvec.pyx:722-800) evaluates
    (it does not run under numpy 2, so the dense product stands in)."""
    S, Nb = v.shape
    A, B = cheb_sn_dense(Nb)
    alf = np.broadcast_to(np.asarray(alfa, float).reshape(-1), (S,))
    bet = np.broadcast_to(np.asarray(beta, float).reshape(-1), (S,))
    b = np.zeros_like(v)
    b[:, :Nb - 2] = alf[:, None] * (v[:, :Nb - 2] @ A.T) + bet[:, None] * (v[:, :Nb - 2] @ B.T)
    return b


def add_solve(b, A0, A2, scale, axis=0):
    """Poisson_Solve_ADD_1D_ptr (la.pyx:671-706) along axis: d = A[0],
    d1 = A[2] (one value per row), N = len(d) dofs; the boundary rows keep
    b's values (ADDSolver.solve copies b into u, chebyshev/la.py:17-20; a
    Function's set_boundary_dofs zeroes them afterwards)."""
    u = np.array(b, copy=True)
    uv, bv = _mv(u, axis), _mv(np.asarray(b), axis)
    N = len(A0)
    d, d1 = np.asarray(A0, float), np.broadcast_to(np.asarray(A2, float), (N - 2,))
    se = np.zeros(uv.shape[1:], dtype=u.dtype)
    so = np.zeros(uv.shape[1:], dtype=u.dtype)
    uv[N - 1] = bv[N - 1] / d[N - 1]
    uv[N - 2] = bv[N - 2] / d[N - 2]
    for k in range(N - 3, -1, -1):
        if k % 2 == 0:
            se = se + uv[k + 2]
            uv[k] = bv[k] - d1[k] * se
        else:
            so = so + uv[k + 2]
            uv[k] = bv[k] - d1[k] * so
        uv[k] /= d[k]
    if not abs(scale - 1) < 1e-8:
        uv[:N] /= scale
    return u


def ann_solve(b, A0, A2, scale, axis=0, u0=0.0):
    """ANNSolver.__call__ (chebyshev/la.py:77-128) along axis: columns scaled
    by 1/j^2, back substitution for k = N-3 .. 1, u = w / j^2 / scale, the
    constraint u_0 = u0, boundary dofs 0."""
    u = np.array(b, copy=True)
    uv, bv = _mv(u, axis), _mv(np.asarray(b), axis)
    M = len(A0)
    j2 = np.arange(M, dtype=float) ** 2
    j2[0] = 1
    j2 = 1.0 / j2
    d = np.asarray(A0, float) * j2
    d1 = np.asarray(A2, float) * j2[2:]
    se = np.zeros(uv.shape[1:], dtype=u.dtype)
    so = np.zeros(uv.shape[1:], dtype=u.dtype)
    us = uv[:M]
    us[-1] = bv[M - 1] / d[-1]
    us[-2] = bv[M - 2] / d[-2]
    for k in range(M - 3, 0, -1):
        if k % 2 == 0:
            se = se + us[k + 2]
            us[k] = bv[k] - d1[k] * se
        else:
            so = so + us[k + 2]
            us[k] = bv[k] - d1[k] * so
        us[k] /= d[k]
    us *= j2.reshape((M,) + (1,) * (us.ndim - 1))
    uv /= scale
    uv[0] = u0
    uv[M:] = 0
    return u


# ---------------------------------------------------------------------------
# The other banded solvers: DiagMA, TwoDMA, ThreeDMA, FDMA, HeptaDMA
# (la.py:291-800).  data in the reference's column-aligned DIA layout:
# row r holds M[i][i + off[r]] at column i + off[r].
def dia_dense(data, offsets):
    n = data.shape[1]
    M = np.zeros((n, n))
    for r, o in enumerate(offsets):
        for i in range(n):
            if 0 <= i + o < n:
                M[i, i + o] = data[r, i + o]
    return M


def threedma_effective(data):
    """ThreeDMA.inner_solve reads its offset-4 coefficient of row i from the
    offset-2 row's storage (u2 = data[1, 4:], la.py:686-689, la.pyx:569-580):
    u2[i] = data[1, i + 4].  Returns the DIA data of the matrix it solves."""
    eff = np.array(data, copy=True)
    n = data.shape[1]
    eff[2, 4:] = data[1, 4:n]
    return eff


def banded_lu(data, offsets):
    """Doolittle LU without pivoting, in place in the DIA layout (the
    reference's *_LU recurrences are this elimination for their bands)."""
    n = data.shape[1]
    row = {o: r for r, o in enumerate(offsets)}
    for i in range(n):
        piv = data[row[0], i]
        for l in offsets:
            if l >= 0 or i - l >= n:
                continue
            m = data[row[l], i] / piv
            data[row[l], i] = m
            for u in offsets:
                if u <= 0 or i + u >= n:
                    continue
                data[row[u + l], i + u] -= m * data[row[u], i + u]
    return data


def banded_solve(u, data, offsets, axis=0):
    """Forward then back substitution with the LU of banded_lu (*_Solve)."""
    u = np.array(u, copy=True)
    v = np.moveaxis(u, axis, 0)
    n = data.shape[1]
    for i in range(n):
        for r, l in enumerate(offsets):
            if l < 0 and i + l >= 0:
                v[i] = v[i] - data[r, i + l] * v[i + l]
    r0 = list(offsets).index(0)
    for i in range(n - 1, -1, -1):
        for r, o in enumerate(offsets):
            if o > 0 and i + o < n:
                v[i] = v[i] - data[r, i + o] * v[i + o]
        v[i] = v[i] / data[r0, i]
    return u
