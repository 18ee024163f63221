"""1D Galerkin matrices of the spaces on the hot path (setup, host side).

Closed-form band coefficients restated from the reference's implemented
matrices; they are evaluated once on the host in FP64 and consumed by the
solvers (which copy what they need to the device).

  Chebyshev ShenDirichlet: B = BSDSD (chebyshev/matrices.py:238-246),
                           A = ASDSD (chebyshev/matrices.py:1061-1079)
  Chebyshev ShenBiharmonic: B = BSBSB (:515-528), A = ASBSB (:1008-1017),
                            S = SSBSB (:1444-1458)
  Legendre ShenDirichlet: B = BSDSD (legendre/matrices.py:121-135),
                          A = ASDSD (legendre/matrices.py:285-292)
  Legendre ShenBiharmonic: B = BSBSB (legendre/matrices.py:179-192)
"""
import numpy as np


class SpectralMatrix(dict):
    """Banded 1D matrix as {offset: diagonal}; ``key`` names it like the
    reference's matrix classes (e.g. 'ASDSDmat').  ``upper_rows`` marks the
    Chebyshev stiffness/biharmonic matrices whose upper triangle is dense with
    a closed form per row (they are never stored densely)."""

    def __init__(self, key, diags, shape, test=None, trial=None, upper_rows=None):
        dict.__init__(self, diags)
        self.key = key
        self.shape = shape
        self.testfunction = (test, 0)
        self.trialfunction = (trial, 0)
        self.upper_rows = upper_rows
        self.scale = 1.0

    def get_key(self):
        return self.key

    def todense(self):
        M = np.zeros(self.shape)
        n = self.shape[0]
        for off, d in self.items():
            d = np.broadcast_to(np.atleast_1d(d), (n - abs(off),))
            M += np.diag(d, off)
        if self.upper_rows is not None:
            for i in range(n):
                for j in range(i + 2, n, 2):
                    if j - i not in self:
                        M[i, j] = self.upper_rows(i, j)
        return M


def cheb_norm_sq(N):
    h = np.full(N, np.pi / 2)
    h[0] = np.pi
    return h


def leg_norm_sq(N):
    return 2.0 / (2 * np.arange(N) + 1.0)


def cheb_sd_B(N, space=None):
    h = cheb_norm_sq(N)
    return SpectralMatrix("BSDSDmat", {-2: -h[1], 0: h[:-2] + h[2:], 2: -h[1]}, (N - 2, N - 2),
                          space, space)


def cheb_sd_A(N, space=None):
    k = np.arange(N, dtype=float)
    d = {0: -2 * np.pi * (k[:N - 2] + 1) * (k[:N - 2] + 2),
         2: -4 * np.pi * (k[:-4] + 1),
         4: -4 * np.pi * (k[:N - 6] + 1)}
    return SpectralMatrix("ASDSDmat", d, (N - 2, N - 2), space, space,
                          upper_rows=lambda i, j: -4 * np.pi * (i + 1))


def cheb_sb_stencil(N):
    k = np.arange(N, dtype=float)
    K2 = -(2 * k[:N - 2] + 4) / (k[:N - 2] + 3)
    K4 = (k[:N - 4] + 1) / (k[:N - 4] + 3)
    K2[N - 4:] = 0
    return K2, K4


def cheb_sb_B(N, space=None):
    h = cheb_norm_sq(N)
    K2, K4 = cheb_sb_stencil(N)
    d = {0: h[:-4] + h[2:-2] * K2[:-2] ** 2 + h[4:] * K4 ** 2,
         2: h[2:-4] * K2[:-4] + h[4:-2] * K4[:-2] * K2[2:-2],
         4: h[4:-4] * K4[:-4]}
    d[-2] = d[2].copy()
    d[-4] = d[4].copy()
    return SpectralMatrix("BSBSBmat", d, (N - 4, N - 4), space, space)


def cheb_sb_A(N, space=None):
    k = np.arange(N - 4, dtype=float)
    d = {-2: 2 * (k[2:] - 1) * (k[2:] + 2) * np.pi,
         0: -4 * ((k + 1) * (k + 2) ** 2) / (k + 3) * np.pi,
         2: 2 * (k[:-2] + 1) * (k[:-2] + 2) * np.pi}
    return SpectralMatrix("ASBSBmat", d, (N - 4, N - 4), space, space)


def cheb_sb_S(N, space=None):
    ki = np.arange(N - 4, dtype=float)

    def row(i, j):
        return 8 * (ki[i] + 1) * (ki[i] + 2) * (ki[i] * (ki[i] + 4) + 3 * (ki[j] + 2) ** 2) * np.pi / (ki[j] + 3)
    d = {0: np.pi * 8 * (ki + 1) ** 2 * (ki + 2) * (ki + 4)}
    return SpectralMatrix("SSBSBmat", d, (N - 4, N - 4), space, space, upper_rows=row)


def leg_sd_B(N, space=None):
    d0 = leg_norm_sq(N)
    return SpectralMatrix("BSDSDmat", {0: d0[:-2] + d0[2:], -2: -d0[2:-2], 2: -d0[2:-2]},
                          (N - 2, N - 2), space, space)


def leg_sd_A(N, space=None):
    k = np.arange(N - 2, dtype=float)
    return SpectralMatrix("ASDSDmat", {0: 4 * k + 6}, (N - 2, N - 2), space, space)


def leg_sb_B(N, space=None):
    d0 = leg_norm_sq(N)
    i = np.arange(N - 4, dtype=float)
    d = {0: (-4 * i - 10) ** 2 * d0[2:-2] / (2 * i + 7) ** 2 + (2 * i + 3) ** 2 * d0[4:] / (2 * i + 7) ** 2 + d0[:-4],
         2: (-4 * i[:-2] - 18) * (2 * i[:-2] + 3) * d0[4:-2] / ((2 * i[:-2] + 7) * (2 * i[:-2] + 11)) + (-4 * i[:-2] - 10) * d0[2:-4] / (2 * i[:-2] + 7),
         4: (2 * i[:-4] + 3) * d0[4:-4] / (2 * i[:-4] + 7)}
    d[-2] = d[2].copy()
    d[-4] = d[4].copy()
    return SpectralMatrix("BSBSBmat", d, (N - 4, N - 4), space, space)


def galerkin_matrix(space, order):
    """(phi_j^{(order)}, phi_k)_w for the polynomial spaces on the hot path."""
    fam, name, N = space.family(), space.short_name(), space.N
    table = {
        ("chebyshev", "SD", 0): cheb_sd_B, ("chebyshev", "SD", 2): cheb_sd_A,
        ("chebyshev", "SB", 0): cheb_sb_B, ("chebyshev", "SB", 2): cheb_sb_A,
        ("chebyshev", "SB", 4): cheb_sb_S,
        ("legendre", "SD", 0): leg_sd_B,
        ("legendre", "SB", 0): leg_sb_B,
    }
    if (fam, name, order) == ("legendre", "SD", 2):
        # (phi''_j, phi_k) = -(phi'_j, phi'_k) = -A (integration by parts)
        M = leg_sd_A(N, space)
        M[0] = -M[0]
        M.key = "ASDSDmat"
        M.sign = -1
        return M
    fn = table.get((fam, name, order))
    if fn is None:
        raise NotImplementedError(f"matrix of order {order} for {fam} {name}")
    return fn(N, space)
