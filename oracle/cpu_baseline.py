"""CPU timing leg for bench.py (the reported baseline and the reference arm).

TEST/MEASUREMENT INFRASTRUCTURE ONLY: bench.py's ``cpu_baseline`` and
``--impl reference`` legs are the only users.

One step is the reference's Helmholtz round trip on the host:
``inner(v, f)`` (Chebyshev GC scalar product, rfft, fft) -> Chebyshev
Dirichlet Helmholtz solve -> ``backward``.  When the reference's own Cython
kernels are built in ``oracle/_ref`` (``oracle/build_ref.py``), the solve runs
the reference's compiled ``LU_Helmholtz`` / ``Solve_Helmholtz``
(la.pyx:708-947), the same functions shenfun calls; the transforms then use
scipy.fft standing in for FFTW (the reference's own transform library is not
installed).  Otherwise the numpy restatement in ``oracle.la`` is used.
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


def load_ref_la():
    so = os.path.join(HERE, "_ref", "la" + sysconfig.get_config_var("EXT_SUFFIX"))
    if not os.path.exists(so):
        return None
    try:
        # the module keeps the fully qualified name it was compiled with
        spec = importlib.util.spec_from_file_location("shenfun.optimization.cython.la", so)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        return mod
    except Exception:
        return None


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


if __name__ == "__main__":
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 64
    rt = HelmholtzRoundTrip(n, n, n + 1, 1000.0, workers=os.cpu_count())
    f = np.random.default_rng(0).standard_normal(rt.shape)
    print(rt.kind, "setup", rt.setup_s, "steps", time_steps(rt, f, 3))
