"""1D Galerkin matrices of the spaces on the hot path (setup, host side).

Closed-form band coefficients restated from the reference's implemented
matrices; they are evaluated once on the host in FP64 and consumed by the
solvers (which copy what they need to the device).

  Chebyshev ShenDirichlet: B = BSDSD (chebyshev/matrices.py:238-246),
                           A = ASDSD (chebyshev/matrices.py:1061-1079)
  Chebyshev ShenBiharmonic: B = BSBSB (:515-528), A = ASBSB (:1008-1017),
                            S = SSBSB (:1444-1458)
  Chebyshev ShenNeumann: B = BSNSN (:377-401), A = ASNSN (:1096-1122)
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
        self.solver = None
        self.constrained_rows = ()

    def get_key(self):
        return self.key

    @property
    def issymmetric(self):
        offs = set(self.keys())
        if any(-o not in offs for o in offs) or self.upper_rows is not None:
            return False
        n = self.shape[0]
        return all(np.allclose(np.broadcast_to(np.atleast_1d(self[o]), (n - abs(o),)),
                               np.broadcast_to(np.atleast_1d(self[-o]), (n - abs(o),))) for o in offs if o > 0)

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
        for row in self.constrained_rows:
            diag = M[row, row]
            M[row, :] = 0.0
            M[row, row] = diag
        return M

    def get_solver(self):
        """The solver class for this matrix (matrixbase.py:439-474): the
        overrides of the Chebyshev / Legendre matrix classes
        (chebyshev/matrices.py:248, 403, 530, 1081, 1124; legendre/matrices.py:
        136, 191), else by band pattern, else the generic ``la.Solve``."""
        from . import la
        if np.all(np.asarray(self.scale) == 0):
            return la.Solve
        space = self.testfunction[0]
        fam = space.family() if space is not None else None
        over = {"chebyshev": {"BSDSDmat": la.TDMA, "BSNSNmat": la.TDMA, "BSBSBmat": la.PDMA,
                              "ASDSDmat": la.ADDSolver, "ASNSNmat": la.ANNSolver},
                "legendre": {"BSDSDmat": la.TDMA, "BSBSBmat": la.PDMA}}.get(fam, {})
        if self.key in over:
            return over[self.key]
        if self.upper_rows is not None:
            return la.Solve
        keys = tuple(sorted(int(k) for k in self.keys()))
        if keys == (-1, 0, 1) and self.issymmetric:
            return la.TDMA_O
        return {(0,): la.DiagMA, (0, 2): la.TwoDMA, (-2, 0, 2): la.TDMA, (0, 2, 4): la.ThreeDMA,
                (-2, 0, 2, 4): la.FDMA, (-4, -2, 0, 2, 4): la.PDMA,
                (-4, -2, 0, 2, 4, 6, 8): la.HeptaDMA}.get(keys, la.Solve)

    def solve(self, b, u=None, axis=0, constraints=()):
        """Solve self u = b along axis (matrixbase.py:410-437); the solver is
        created on the first call and kept."""
        if self.solver is None:
            self.solver = self.get_solver()(self)
        return self.solver(b, u=u, axis=axis, constraints=constraints)


def constrained(mat, constraints):
    """A copy of ``mat`` with the rows of ``constraints`` ((row, value)
    pairs) made identity rows, as SparseMatrixSolver.apply_constraints does
    for a SparseMatrix (la.py:77-130): the row's diagonal entry becomes
    1/scale and its other stored entries 0 (a dense upper part too)."""
    n = mat.shape[0]
    d = {k: np.array(np.broadcast_to(np.atleast_1d(np.asarray(v, dtype=float)), (n - abs(k),)))
         for k, v in mat.items()}
    A = SpectralMatrix(mat.key, d, mat.shape, mat.testfunction[0], mat.trialfunction[0], mat.upper_rows)
    A.scale = mat.scale
    for attr in ("order", "sign"):
        if hasattr(mat, attr):
            setattr(A, attr, getattr(mat, attr))
    sc = float(np.asarray(mat.scale).reshape(-1)[0])
    rows = []
    for row, _ in constraints:
        row = int(row)
        for key, v in A.items():
            if key >= 0:
                if row < n - key:
                    v[row] = float(key == 0) / sc
            elif 0 < row + key < n + key:
                v[row + key] = 0.0
        rows.append(row)
    A.constrained_rows = tuple(rows)
    return A


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


def cheb_sn_B(N, space=None):
    h = cheb_norm_sq(N)
    k = np.arange(N, dtype=float)
    al = (k / (k + 2)) ** 2
    d = {0: h[:-2] + al[:-2] ** 2 * h[2:], 2: -al[:N - 4] * h[2:N - 2]}
    d[-2] = d[2].copy()
    return SpectralMatrix("BSNSNmat", d, (N - 2, N - 2), space, space)


def cheb_sn_A(N, space=None):
    k = np.arange(N - 2, dtype=float)
    d = {0: -2 * np.pi * k ** 2 * (k + 1) / (k + 2),
         2: -4 * np.pi * (k[:-2] + 2) ** 2 * (k[:-2] + 1) / (k[:-2] + 2) ** 2,
         4: -4 * np.pi * (k[:-4] + 4) ** 2 * (k[:-4] + 1) / (k[:-4] + 2) ** 2}
    return SpectralMatrix("ASNSNmat", d, (N - 2, N - 2), space, space,
                          upper_rows=lambda i, j: -4 * np.pi * j ** 2 * (i + 1) / (i + 2) ** 2)


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
        ("chebyshev", "SN", 0): cheb_sn_B, ("chebyshev", "SN", 2): cheb_sn_A,
        ("legendre", "SD", 0): leg_sd_B,
        ("legendre", "SB", 0): leg_sb_B,
    }
    keys = {0: "B", 2: "A", 4: "S"}
    if (fam, name, order) == ("legendre", "SD", 2):
        # (phi''_j, phi_k) = -(phi'_j, phi'_k) = -A (integration by parts)
        M = leg_sd_A(N, space)
        M[0] = -M[0]
        M.key = "ASDSDmat"
        M.sign = -1
    elif (fam, name, order) in table:
        M = table[(fam, name, order)](N, space)
    elif fam == "legendre" and name == "SB" and order in (2, 4):
        b, _ = band_sep_term(space, order)
        n = b.shape[1]
        diags = {off: b[r, max(0, -off):n - max(0, off)] for r, off in enumerate((-4, -2, 0, 2, 4))
                 if np.any(b[r])}
        M = SpectralMatrix(keys[order] + "SBSBmat", diags, (n, n), space, space)
    else:
        raise NotImplementedError(f"matrix of order {order} for {fam} {name}")
    M.order = order
    return M


# ---------------------------------------------------------------------------
# Banded + semiseparable description of (phi_j^{(order)}, phi_k) for the
# per-wavenumber solver (sgpu_band_sep_*): bands[5][n] at offsets -4..4 (row
# k holds M[k][k+off]) and, for the one term with a dense upper part, the
# generators p, q, r, t with M[k][j] = p_k q_j + r_k t_j for j >= k+2.
def band_sep_dense(bands, gens):
    """Dense matrix of one band/semiseparable term (for tests and checks)."""
    n = bands.shape[1]
    M = np.zeros((n, n))
    for r, off in enumerate((-4, -2, 0, 2, 4)):
        for k in range(n):
            if 0 <= k + off < n:
                M[k, k + off] += bands[r, k]
    if gens is not None:
        for k in range(n):
            for j in range(k + 2, n, 2):
                M[k, j] += gens[0, k] * gens[1, j] + gens[2, k] * gens[3, j]
    return M


def band_sep_term(space, order):
    """(bands (5, n), gens (4, n) or None) for one Galerkin matrix."""
    fam, name, N = space.family(), space.short_name(), space.N
    nb = {"SD": 2, "SB": 4}[name]
    n = N - nb
    k = np.arange(n, dtype=float)
    bands = np.zeros((5, n))
    gens = None
    if fam == "chebyshev" and name == "SD":
        if order == 0:
            h = cheb_norm_sq(N)
            bands[2] = h[:-2] + h[2:]
            bands[1, 2:] = -h[1]      # M[k][k-2]
            bands[3, :-2] = -h[1]     # M[k][k+2]
        elif order == 2:
            bands[2] = -2 * np.pi * (k + 1) * (k + 2)
            gens = np.zeros((4, n))
            gens[0] = -4 * np.pi * (k + 1)
            gens[1] = 1.0
        else:
            raise NotImplementedError(order)
    elif fam == "chebyshev" and name == "SB":
        if order == 0:
            B = cheb_sb_B(N)
            bands[2] = B[0]
            bands[3, :-2] = B[2]
            bands[4, :-4] = B[4]
            bands[1, 2:] = B[-2]
            bands[0, 4:] = B[-4]
        elif order == 2:
            bands[2] = -4 * ((k + 1) * (k + 2) ** 2) / (k + 3) * np.pi
            bands[3, :-2] = 2 * (k[:-2] + 1) * (k[:-2] + 2) * np.pi
            bands[1, 2:] = 2 * (k[2:] - 1) * (k[2:] + 2) * np.pi
        elif order == 4:
            bands[2] = np.pi * 8 * (k + 1) ** 2 * (k + 2) * (k + 4)
            gens = np.zeros((4, n))
            gens[0] = 8 * np.pi * (k + 1) * (k + 2) * k * (k + 4)
            gens[1] = 1.0 / (k + 3)
            gens[2] = 24 * np.pi * (k + 1) * (k + 2)
            gens[3] = (k + 2) ** 2 / (k + 3)
        else:
            raise NotImplementedError(order)
    elif fam == "legendre" and name == "SD":
        h = leg_norm_sq(N)
        if order == 0:
            bands[2] = h[:-2] + h[2:]
            bands[3, :-2] = -h[2:-2]        # M[k][k+2] = -h_{k+2}
            bands[1, 2:] = -h[2:-2]         # M[k][k-2] = -h_k
        elif order == 2:
            bands[2] = -(4 * k + 6)
        else:
            raise NotImplementedError(order)
    elif fam == "legendre" and name == "SB":
        if order == 0:
            B = leg_sb_B(N)
            bands[2] = B[0]
            bands[3, :-2] = B[2]
            bands[4, :-4] = B[4]
            bands[1, 2:] = B[-2]
            bands[0, 4:] = B[-4]
        elif order == 2:
            # -(phi'_j, phi'_k): ASBSB {0: 2(2k+3)(1+g_k), +-2: -2(2k+3)} (legendre/matrices.py:318-340)
            g = (2 * k + 3) / (2 * k + 7)
            bands[2] = -2 * (2 * k + 3) * (1 + g)
            bands[3, :-2] = 2 * (2 * k[:-2] + 3)
            bands[1, 2:] = 2 * (2 * k[:-2] + 3)
        elif order == 4:
            # (phi''_j, phi''_k) = 2 (2k+3)^2 (2k+5) (legendre/matrices.py:425-440)
            bands[2] = 2 * (2 * k + 3) ** 2 * (2 * k + 5)
        else:
            raise NotImplementedError(order)
    else:
        raise NotImplementedError(f"{fam} {name}")
    return bands, gens
