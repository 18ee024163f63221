"""IMEX Runge-Kutta steps of u_t = nu lap(u) + f (CPU oracle, numpy).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates PDEIMEXRK.assemble / compute_rhs / solve_step
(utilities/integrators.py:782-817) and the tableaux of IMEXRK111/222/443
(:836-900) for a Fourier x ... x Chebyshev ShenDirichlet space: every linear
form is alfa A + beta B per wavenumber (Helmholtz_matvec, Matvec.pyx:656-695;
inner(v, lap u) = A - k^2 B), every solve LU_Helmholtz/Solve_Helmholtz
(la.pyx:717-912), and the Nyquist modes of even Fourier axes are zeroed in
each right-hand side (tensorproductspace.py:1054-1080).
"""
import numpy as np

from . import la, problems as P, spectral as S


def tableau(name):
    if name == "IMEXRK111":
        return np.array([[0, 0], [0, 1.0]]), np.array([[0, 0], [1.0, 0]])
    if name == "IMEXRK222":
        g = (2 - np.sqrt(2)) / 2
        d = 1 - 1 / (2 * g)
        return (np.array([[0, 0, 0], [0, g, 0], [0, 1 - g, g]]),
                np.array([[0, 0, 0], [g, 0, 0], [d, 1 - d, 0]]))
    if name == "IMEXRK443":
        a = np.array([[0, 0, 0, 0, 0], [0, 1 / 2, 0, 0, 0], [0, 1 / 6, 1 / 2, 0, 0],
                      [0, -1 / 2, 1 / 2, 1 / 2, 0], [0, 3 / 2, -3 / 2, 1 / 2, 1 / 2]])
        b = np.array([[0, 0, 0, 0, 0], [1 / 2, 0, 0, 0, 0], [11 / 18, 1 / 18, 0, 0, 0],
                      [5 / 6, -5 / 6, 1 / 2, 0, 0], [1 / 4, 7 / 4, 3 / 4, -7 / 4, 0]])
        return a, b
    raise ValueError(name)


def nyquist_mask(bases):
    shape = []
    for fam, b, N in bases:
        shape.append(N // 2 + 1 if b == "R2C" else N)
    mask = np.ones(shape)
    for ax, (fam, b, N) in enumerate(bases):
        if fam == "fourier" and N % 2 == 0:
            idx = [slice(None)] * len(bases)
            idx[ax] = -1 if b == "R2C" else N // 2
            mask[tuple(idx)] = 0
    return mask


def imex_run(u_hat0, f_hat, nu, dt, name, nsteps, bases, axis):
    """u_hat after each of `nsteps` steps of scheme `name`."""
    a, b = tableau(name)
    steps = a.shape[0] - 1
    N = bases[axis][2]
    k2 = P.fourier_k2(bases, axis)
    ks = np.moveaxis(np.broadcast_to(k2, k2.shape), axis, -1).reshape(-1)
    one = np.ones_like(ks)

    # a ShenNeumann axis takes the Neumann branch of the Helmholtz LU / solve
    # and the ASNSN / BSNSN product (la.pyx:735-751, 907-912)
    nm = bases[axis][1] == "SN"
    matvec = la.helmholtz_neumann_matvec if nm else la.helmholtz_matvec

    def mv(v, alfa, beta):
        vs, shp = P._systems(v, axis)
        return np.moveaxis(matvec(vs, alfa, beta).reshape(shp), -1, axis)

    d = la.helmholtz_lu(N, -dt * a[1, 1] * nu * one, one + dt * a[1, 1] * nu * ks, neumann=nm)

    def solve(f):
        fs, shp = P._systems(f, axis)
        return np.moveaxis(la.helmholtz_solve(fs, *d, neumann=nm).reshape(shp), -1, axis)

    mask = nyquist_mask(bases)
    u = u_hat0.copy()
    out = []
    for _ in range(nsteps):
        K = [None] * steps
        Lr = [None] * (steps - 1)
        for rk in range(steps):
            K[rk] = mv(f_hat, 0 * one, one)
            if rk == 0:
                u0 = mv(u, 0 * one, one)
            rhs = u0.copy()
            for j in range(rk + 1):
                rhs = rhs + dt * b[rk + 1, j] * K[j]
            if rk > 0:
                Lr[rk - 1] = mv(u, nu * one, -nu * ks)
                for j in range(rk):
                    rhs = rhs + dt * a[rk + 1, j + 1] * Lr[j]
            rhs = rhs * mask
            u = solve(rhs)
        out.append(u.copy())
    return out
