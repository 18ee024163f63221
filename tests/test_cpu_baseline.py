"""The CPU timing legs behind bench.py's cpu_baseline entries: each leg's
output against the oracle (and the reference's compiled kernels, when built,
against the numpy restatement), so that a timed baseline computes the
workload it claims to."""
import warnings

import numpy as np
import pytest

from oracle import cpu_baseline as CB, problems as P, spectral as S


def _manufactured_2d(Nx, Ny):
    x = 2 * np.pi * np.arange(Nx) / Nx
    y = np.cos(np.pi * (2 * np.arange(Ny) + 1) / (2 * Ny))
    X, Y = np.meshgrid(x, y, indexing="ij")
    cy, sy = np.cos(np.pi * Y / 2), np.sin(np.pi * Y / 2)
    g = (1 - Y ** 2) * cy
    gpp = -2 * cy + 2 * np.pi * Y * sy - (np.pi ** 2 / 4) * (1 - Y ** 2) * cy
    return np.sin(2 * X) * g, np.sin(2 * X) * (4 * g - gpp)


@pytest.mark.parametrize("use_ref", [True, False])
def test_poisson2d_manufactured(use_ref):
    u, f = _manufactured_2d(64, 64)
    pz = CB.Poisson2D(64, 64, use_reference=use_ref)
    got = pz.step(f)
    assert np.abs(got - u).max() / np.abs(u).max() < 1e-13


@pytest.mark.parametrize("use_ref", [True, False])
def test_biharmonic_roundtrip_even(use_ref):
    Nx, Ny, Nz = 8, 6, 24
    f = np.random.default_rng(3).standard_normal((Nx, Ny, Nz))
    rt = CB.BiharmonicRoundTrip(Nx, Ny, Nz, use_reference=use_ref)
    bases = [("fourier", "C2C", Nx), ("fourier", "R2C", Ny), ("chebyshev", "SB", Nz)]
    ref = P.backward(P.biharmonic_solve(P.scalar_product(f, bases), bases, 2), bases)
    got = rt.step(f)
    assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-12


def test_biharmonic_manufactured():
    Nx, Ny, Nz = 8, 8, 24
    x = 2 * np.pi * np.arange(Nx) / Nx
    z = np.cos(np.pi * (2 * np.arange(Nz) + 1) / (2 * Nz))
    X, Y, Z = np.meshgrid(x, x, z, indexing="ij")
    u = np.sin(X) * np.cos(Y) * (1 - Z ** 2) ** 2
    f = np.sin(X) * np.cos(Y) * (44 - 56 * Z ** 2 + 4 * Z ** 4)
    got = CB.BiharmonicRoundTrip(Nx, Ny, Nz).step(f)
    assert np.abs(got - u).max() / np.abs(u).max() < 1e-12


def test_biharmonic_odd_dofs_mirrors_reference():
    """Odd N - 4: the reference's 2D/3D LU factors len(sii) // 2 rows per
    parity, leaving the last even row zero; the restatement keeps that, and
    both give the same (non-finite) solve."""
    Nx, Ny, Nz = 4, 4, 21
    f = np.random.default_rng(4).standard_normal((Nx, Ny, Nz))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        port = CB.BiharmonicRoundTrip(Nx, Ny, Nz, use_reference=False)
        assert np.all(port.f[0][0, ..., -1] == 0)        # u0, even parity, last row
        assert np.all(port.f[0][1, ..., :-1] != 0)
        assert not np.isfinite(port.step(f)).all()
        ref = CB.BiharmonicRoundTrip(Nx, Ny, Nz)
        if ref.kind == "reference":
            for a, b in zip(ref.f, port.f):
                np.testing.assert_allclose(a, b, rtol=1e-12, atol=0)


def test_legendre_recursion_matches_fixture_layout():
    a = CB.legendre_recursion(18)
    k = np.arange(18.0)
    assert np.allclose(a[0, :-1], (k[:-1] + 1) / (2 * k[:-1] + 1)) and a[0, -1] == 0
    assert np.allclose(a[1], k / (2 * k + 1))


@pytest.mark.parametrize("use_ref", [True, False])
def test_legendre_lines(use_ref):
    L = CB.LegendreLines(48, 5, use_reference=use_ref)
    L.backward()
    L.forward()
    np.testing.assert_allclose(L.u, S.leg_backward_ortho(L.c, axis=1), rtol=0, atol=1e-13)
    np.testing.assert_allclose(L.c2, S.leg_scalar_product_ortho(L.u, axis=1), rtol=0, atol=1e-13)


def test_rhs_pool_bounded_and_deterministic():
    from shenfun_gb300.serving import RhsPool
    pool = RhsPool(per_shape=2, seed=1, pinned=False)
    a = pool((4, 5), 10)
    b = pool((4, 5), 12)
    c = pool((4, 5), 11)
    assert a is b and a is not c
    assert len(pool.arrays) == 2 and pool.nbytes == 2 * 4 * 5 * 8
    np.testing.assert_array_equal(RhsPool(per_shape=2, seed=1, pinned=False)((4, 5), 0), a)


def test_dlt_term_count():
    """The Taylor-term count behind bench.py's DLT bound: the terms fall off
    like (N max|dtheta|)^n / n!, so the count is nearly independent of N
    (14-16 for 1e-16 on 4096 lines), and a loose tolerance stops at term 1."""
    import bench
    counts = [bench.dlt_terms(N, 4096) for N in (512, 2048)]
    assert all(12 <= c <= 18 for c in counts)
    assert bench.dlt_terms(512, 4096, tol=1e3) == 1
