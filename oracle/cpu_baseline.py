"""CPU timing legs for bench.py (the reported baselines and the reference arm).

TEST/MEASUREMENT INFRASTRUCTURE ONLY: bench.py's ``cpu_baseline`` entries and
``--impl reference`` leg are the only users.

When the reference's own Cython kernels are built in ``oracle/_ref``
(``oracle/build_ref.py``), every leg runs the reference's compiled functions
on the path, the same ones shenfun calls; otherwise the numpy restatements in
``oracle`` stand in (``kind`` says which).  The reference's transform library
(FFTW through its own wrappers) is not installed: scipy.fft stands in for the
Fourier and Chebyshev (DCT) transforms.

* ``HelmholtzRoundTrip``: Fourier x Fourier x Chebyshev Dirichlet round trip,
  ``inner(v, f)`` (Chebyshev GC scalar product, rfft, fft) -> Helmholtz solve
  with ``LU_Helmholtz`` / ``Solve_Helmholtz`` (la.pyx:708-947) -> backward.
* ``Poisson2D``: Fourier (R2C) x Chebyshev Dirichlet 2D Poisson, the same
  kernels on one 2D grid.
* ``BiharmonicRoundTrip``: Fourier x Fourier x Chebyshev ShenBiharmonic,
  the solve with ``LU_Biharmonic`` / ``Biharmonic_factor_pr`` (setup) and
  ``Biharmonic_Solve`` (la.pyx, called from chebyshev/la.py:499-547).
* ``LegendreLines``: the recursive Legendre transforms
  ``evaluate_expansion_all`` / ``scalar_product`` (transforms.pyx:175-325,
  called from spectralbase.py:448-575) on a sample of lines.
"""
import importlib.util
import os
import sys
import sysconfig
import time

import numpy as np
import scipy.fft as sfft

from . import spectral as S, la as OL, problems as P

HERE = os.path.dirname(os.path.abspath(__file__))


def load_ref(name):
    """The reference's compiled Cython module `name` from oracle/_ref, or None."""
    so = os.path.join(HERE, "_ref", name + sysconfig.get_config_var("EXT_SUFFIX"))
    if not os.path.exists(so):
        return None
    try:
        # the module keeps the fully qualified name it was compiled with
        spec = importlib.util.spec_from_file_location("shenfun.optimization.cython." + name, so)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        return mod
    except Exception:
        return None


def load_ref_la():
    return load_ref("la")


class HelmholtzRoundTrip:
    """cfg: Fourier Nx (C2C) x Fourier Ny (R2C) x Chebyshev SD Nz."""

    def __init__(self, Nx, Ny, Nz, c, workers=1, use_reference=True):
        self.shape = (Nx, Ny, Nz)
        self.c = c
        self.workers = workers
        self.bases = [("fourier", "C2C", Nx), ("fourier", "R2C", Ny), ("chebyshev", "SD", Nz)]
        self.ref = load_ref_la() if use_reference else None
        self.kind = "reference" if self.ref is not None else "port"
        beta = P.fourier_k2(self.bases, 2) + c          # (Nx, Ny//2+1, 1)
        self.alfa = -np.ones_like(beta)
        self.beta = beta
        t0 = time.perf_counter()
        if self.ref is not None:
            shp = (Nx, Ny // 2 + 1, Nz)
            self.d = [np.zeros(shp) for _ in range(4)]
            A = {0: None, 2: None, 4: None}
            Am = OL.cheb_sd_stiffness(Nz)
            Bm = S.mass_bands("chebyshev", "SD", Nz)
            A = {k: v for k, v in Am.items()}

            class _B(dict):
                pass
            B = _B({-2: np.broadcast_to(Bm[-2], Am[2].shape).copy(), 0: Bm[0],
                    2: np.broadcast_to(Bm[2], Am[2].shape).copy()})
            self.ref.LU_Helmholtz(A, B, self.alfa, self.beta, False, *self.d, 2)
        else:
            bsys = beta.reshape(-1)
            self.fac = OL.helmholtz_lu(Nz, -np.ones_like(bsys), bsys)
        self.setup_s = time.perf_counter() - t0

    def scalar_product(self, f):
        w = self.workers
        Nz = self.shape[2]
        c = sfft.dct(f, type=2, axis=2, workers=w) * (np.pi / (2 * Nz))
        c = S.apply_stencil(c, S.stencil("chebyshev", "SD", Nz), 2)
        c = sfft.rfft(c, axis=1, workers=w) / self.shape[1]
        return sfft.fft(c, axis=0, workers=w) / self.shape[0]

    def backward(self, uh):
        w = self.workers
        Nz = self.shape[2]
        c = sfft.ifft(uh, axis=0, norm="forward", workers=w)
        c = sfft.irfft(c, n=self.shape[1], axis=1, norm="forward", workers=w)
        c = S.to_ortho(c, S.stencil("chebyshev", "SD", Nz), Nz - 2, 2)
        out = sfft.dct(c, type=3, axis=2, workers=w) * 0.5
        out += c[..., :1] / 2
        return out

    def solve(self, fh):
        if self.ref is not None:
            u = np.zeros_like(fh)
            self.ref.Solve_Helmholtz(fh, u, False, *self.d, 2)
            return u
        Nz = self.shape[2]
        us = OL.helmholtz_solve(fh.reshape(-1, Nz), *self.fac)
        return us.reshape(fh.shape)

    def step(self, f):
        return self.backward(self.solve(self.scalar_product(f)))


def time_steps(rt, f, steps, warmup=1):
    for _ in range(warmup):
        rt.step(f)
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        rt.step(f)
        ts.append(time.perf_counter() - t0)
    return ts


def _helmholtz_mats(N):
    """Chebyshev Dirichlet stiffness {offset: diagonal} and mass bands in the
    dict layout LU_Helmholtz reads (chebyshev/la.py:219-231)."""
    A = dict(OL.cheb_sd_stiffness(N))
    Bm = S.mass_bands("chebyshev", "SD", N)
    B = {-2: Bm[-2], 0: Bm[0], 2: Bm[2]}
    return A, B


class Poisson2D:
    """2D Poisson -lap u = f on Fourier Nx (R2C along axis 0, [0, 2 pi)) x
    Chebyshev ShenDirichlet Ny (axis 1): scalar product -> per-wavenumber
    Helmholtz solve (alpha = -1, beta = k^2) -> backward."""

    def __init__(self, Nx, Ny, use_reference=True):
        self.shape = (Nx, Ny)
        self.ref = load_ref_la() if use_reference else None
        self.kind = "reference" if self.ref is not None else "port"
        k = np.fft.rfftfreq(Nx, 1.0 / Nx)
        self.beta = (k ** 2)[:, None].copy()
        self.alfa = -np.ones_like(self.beta)
        t0 = time.perf_counter()
        if self.ref is not None:
            A, B = _helmholtz_mats(Ny)
            B = {o: np.broadcast_to(v, A[2].shape).copy() if o else v for o, v in B.items()}
            self.d = [np.zeros((Nx // 2 + 1, Ny)) for _ in range(4)]
            self.ref.LU_Helmholtz(A, B, self.alfa, self.beta, False, *self.d, 1)
        else:
            self.fac = OL.helmholtz_lu(Ny, self.alfa.reshape(-1), self.beta.reshape(-1))
        self.setup_s = time.perf_counter() - t0

    def scalar_product(self, f):
        Nx, Ny = self.shape
        c = sfft.dct(f, type=2, axis=1) * (np.pi / (2 * Ny))
        c = S.apply_stencil(c, S.stencil("chebyshev", "SD", Ny), 1)
        return sfft.rfft(c, axis=0) / Nx

    def backward(self, uh):
        Nx, Ny = self.shape
        c = sfft.irfft(uh, n=Nx, axis=0, norm="forward")
        c = S.to_ortho(c, S.stencil("chebyshev", "SD", Ny), Ny - 2, 1)
        out = sfft.dct(c, type=3, axis=1) * 0.5
        out += c[:, :1] / 2
        return out

    def solve(self, fh):
        if self.ref is not None:
            u = np.zeros_like(fh)
            self.ref.Solve_Helmholtz(fh, u, False, *self.d, 1)
            return u
        return OL.helmholtz_solve(fh, *self.fac).reshape(fh.shape)

    def step(self, f):
        return self.backward(self.solve(self.scalar_product(f)))


class BiharmonicRoundTrip:
    """Fourier Nx (C2C) x Fourier Ny (R2C) x Chebyshev ShenBiharmonic Nz:
    scalar product -> biharmonic solve (a0 = 1, alpha = -2 k^2, beta = k^4;
    chebyshev/la.py:412-440) -> backward."""

    def __init__(self, Nx, Ny, Nz, use_reference=True):
        from . import refabi as RA
        self.shape = (Nx, Ny, Nz)
        self.ref = load_ref_la() if use_reference else None
        self.kind = "reference" if self.ref is not None else "port"
        bases = [("fourier", "C2C", Nx), ("fourier", "R2C", Ny), ("chebyshev", "SB", Nz)]
        k2 = P.fourier_k2(bases, 2)
        self.alfa = -2 * k2
        self.beta = k2 ** 2
        Sd, Ad, Bd = OL.cheb_sb_dense(Nz)
        diags = [np.diag(Sd, 0), np.diag(Sd, 2), np.diag(Sd, 4), np.diag(Ad, -2), np.diag(Ad, 0),
                 np.diag(Ad, 2), np.diag(Bd, -4), np.diag(Bd, -2), np.diag(Bd, 0), np.diag(Bd, 2),
                 np.diag(Bd, 4)]
        diags = [np.ascontiguousarray(d) for d in diags]
        M = diags[0][::2].shape[0]
        ss = (2, Nx, Ny // 2 + 1, M)
        self.f = [np.zeros(ss) for _ in range(7)]  # u0, u1, u2, l0, l1, ak, bk
        t0 = time.perf_counter()
        u0, u1, u2, l0, l1, ak, bk = self.f
        if self.ref is not None:
            self.ref.LU_Biharmonic(1.0, self.alfa, self.beta, *diags, u0, u1, u2, l0, l1, 2)
            self.ref.Biharmonic_factor_pr(ak, bk, l0, l1, 2)
        else:
            RA.lu_biharmonic(1.0, self.alfa, self.beta, *diags, u0, u1, u2, l0, l1, 2)
            RA.biharmonic_factor_pr(ak, bk, l0, l1, 2)
        self.setup_s = time.perf_counter() - t0

    def scalar_product(self, f):
        Nx, Ny, Nz = self.shape
        c = sfft.dct(f, type=2, axis=2) * (np.pi / (2 * Nz))
        c = S.apply_stencil(c, S.stencil("chebyshev", "SB", Nz), 2)
        c = sfft.rfft(c, axis=1) / Ny
        return sfft.fft(c, axis=0) / Nx

    def backward(self, uh):
        Nx, Ny, Nz = self.shape
        c = sfft.ifft(uh, axis=0, norm="forward")
        c = sfft.irfft(c, n=Ny, axis=1, norm="forward")
        c = S.to_ortho(c, S.stencil("chebyshev", "SB", Nz), Nz - 4, 2)
        out = sfft.dct(c, type=3, axis=2) * 0.5
        out += c[..., :1] / 2
        return out

    def solve(self, fh):
        u = np.zeros_like(fh)
        u0, u1, u2, l0, l1, ak, bk = self.f
        if self.ref is not None:
            self.ref.Biharmonic_Solve(fh, u, u0, u1, u2, l0, l1, ak, bk, 1.0, 2)
        else:
            from . import refabi as RA
            RA.biharmonic_solve(fh, u, u0, u1, u2, l0, l1, ak, bk, 1.0, 2)
        return u

    def step(self, f):
        return self.backward(self.solve(self.scalar_product(f)))


def legendre_recursion(M):
    """The dia-format data of the Legendre recursion matrix
    (legendre/bases.py:239-242, ``get_recursion_matrix(M, M).diags('dia').data``):
    row 0 the sub-diagonal (k+1)/(2k+1) aligned by column (last entry 0),
    row 1 the super-diagonal j/(2j+1) (first entry 0)."""
    k = np.arange(M, dtype=float)
    a = np.zeros((2, M))
    a[0, :-1] = (k[:-1] + 1) / (2 * k[:-1] + 1)
    a[1, 1:] = k[1:] / (2 * k[1:] + 1)
    return a


class LegendreLines:
    """The reference's recursive Legendre transforms on `lines` lines of
    length N (one thread): backward = evaluate_expansion_all of orthogonal
    coefficients, forward = scalar_product (the O(N) Dirichlet stencil and
    mass solve around them are left out: under 1 % of the work at N >= 128)."""

    def __init__(self, N, lines, seed=0, use_reference=True):
        from . import refabi as RA
        self.ref = load_ref("transforms") if use_reference else None
        self.kind = "reference" if self.ref is not None else "port"
        self.lib = self.ref if self.ref is not None else RA
        self.N, self.lines = N, lines
        self.x, self.w = S.leg_lg_points_weights(N)
        self.a = legendre_recursion(N + 3)
        rng = np.random.default_rng(seed)
        self.c = rng.uniform(-1, 1, (lines, N)) * (np.arange(N) + 1.0) ** -2
        self.u = np.zeros_like(self.c)
        self.c2 = np.zeros_like(self.c)

    def backward(self):
        self.lib.evaluate_expansion_all(self.c, self.u, self.x, 1, self.a)

    def forward(self):
        self.lib.scalar_product(self.u, self.c2, self.x, self.w, 1, self.a)


def time_calls(fn, reps, warmup=1):
    for _ in range(warmup):
        fn()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return ts


if __name__ == "__main__":
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 64
    rt = HelmholtzRoundTrip(n, n, n + 1, 1000.0, workers=os.cpu_count())
    f = np.random.default_rng(0).standard_normal(rt.shape)
    print(rt.kind, "setup", rt.setup_s, "steps", time_steps(rt, f, 3))
