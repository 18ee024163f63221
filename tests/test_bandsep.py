"""Per-wavenumber banded + semiseparable solver (CPU: kernel block program in
the harness; matrix descriptions against the oracle's dense matrices)."""
import numpy as np
import pytest

from oracle import la as OL, spectral as S
from shenfun_gb300 import matrices as MX
from test_kernel_emu import emu, run  # noqa: F401

rng = np.random.default_rng(5)


class _Space:
    def __init__(self, fam, name, N):
        self._f, self._n, self.N = fam, name, N

    def family(self):
        return self._f

    def short_name(self):
        return self._n


@pytest.mark.parametrize("N", [12, 17, 33, 64])
def test_descriptions_match_oracle(N):
    Sm, Am, Bm = OL.cheb_sb_dense(N)
    sp = _Space("chebyshev", "SB", N)
    for order, ref in ((4, Sm), (2, Am), (0, Bm)):
        b, g = MX.band_sep_term(sp, order)
        assert np.abs(MX.band_sep_dense(b, g) - ref).max() <= 1e-12 * np.abs(ref).max()
    A, B = OL.cheb_sd_dense(N)
    sp = _Space("chebyshev", "SD", N)
    for order, ref in ((2, A), (0, B)):
        b, g = MX.band_sep_term(sp, order)
        assert np.abs(MX.band_sep_dense(b, g) - ref).max() <= 1e-12 * np.abs(ref).max()
    sp = _Space("legendre", "SD", N)
    b, g = MX.band_sep_term(sp, 0)
    Bd = S.mass_bands("legendre", "SD", N)
    ref = np.diag(Bd[0]) + np.diag(Bd[2], 2) + np.diag(Bd[-2], -2)
    assert np.abs(MX.band_sep_dense(b, g) - ref).max() <= 1e-14


def _systems(emu, fam, name, N, orders, coefs, cplx):  # noqa: F811
    sp = _Space(fam, name, N)
    terms = [MX.band_sep_term(sp, o) for o in orders]
    gen_term = next((i for i, (_, g) in enumerate(terms) if g is not None), -1)
    n = terms[0][0].shape[1]
    bands = np.stack([b for b, _ in terms])
    gens = terms[gen_term][1] if gen_term >= 0 else np.zeros((4, n))
    nsys = coefs.shape[1]
    f = rng.standard_normal((nsys, N))
    if cplx:
        f = f + 1j * rng.standard_normal(f.shape)
    cnt = nsys * N * (2 if cplx else 1)
    out = run(emu, ["bandsep", n, len(orders), gen_term, nsys, N, int(cplx)],
              [bands, gens, coefs, f], 2 * cnt)
    out = out.view(np.complex128) if cplx else out
    u = out[:out.size // 2].reshape(nsys, N)
    mv = out[out.size // 2:].reshape(nsys, N)
    for s in range(nsys):
        M = sum(coefs[t, s] * MX.band_sep_dense(*terms[t]) for t in range(len(orders)))
        ref = np.linalg.solve(M, f[s, :n])
        err = np.abs(u[s, :n] - ref).max() / np.abs(ref).max()
        assert err < 1e-11, (s, err)
        # the matvec (Biharmonic_matvec's product) of the solution, and its tail
        mref = M @ u[s, :n]
        assert np.abs(mv[s, :n] - mref).max() <= 1e-13 * np.abs(mref).max() + 1e-300
        assert np.all(mv[s, n:] == 0)


@pytest.mark.parametrize("N", [16, 17, 33])
@pytest.mark.parametrize("cplx", [False, True])
def test_chebyshev_biharmonic(emu, N, cplx):  # noqa: F811
    k2 = rng.uniform(0, 500, 5)
    coefs = np.stack([np.ones(5), -2 * k2, k2 ** 2])
    _systems(emu, "chebyshev", "SB", N, (4, 2, 0), coefs, cplx)


@pytest.mark.parametrize("N", [16, 17, 64])
def test_chebyshev_helmholtz(emu, N):  # noqa: F811
    coefs = np.stack([-np.ones(4), rng.uniform(0.1, 2000, 4)])
    _systems(emu, "chebyshev", "SD", N, (2, 0), coefs, True)


@pytest.mark.parametrize("N", [16, 17, 64])
@pytest.mark.parametrize("name,orders", [("SD", (2, 0)), ("SB", (4, 2, 0))])
def test_legendre(emu, N, name, orders):  # noqa: F811
    k2 = rng.uniform(0, 300, 4)
    coefs = np.stack([np.ones(4), k2]) if name == "SD" else np.stack([np.ones(4), -2 * k2, k2 ** 2])
    if name == "SD":
        coefs[0] = -1.0
    _systems(emu, "legendre", name, N, orders, coefs, False)
