"""GPU: FP32 banded solves with FP64 iterative refinement (the chosen form of
the per-wavenumber solves) against the FP64 direct solves and the oracle.

Tolerances: the refined solution against the FP64 direct one <= 1e-12
(relative, max-abs over max-abs); the channel-grid round trip with refined
solves against the FP64 oracle <= 1e-10 (the mixed form's bound)."""
import numpy as np
import pytest
import torch

from oracle import la as OL, problems as P

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def sg():
    from shenfun_gb300 import build
    build.build()
    import shenfun_gb300
    return shenfun_gb300


def channel_space(sg, shape, form):
    return sg.TensorProductSpace(None, (sg.FunctionSpace(shape[0], "F", dtype="D"),
                                        sg.FunctionSpace(shape[1], "F", dtype="d"),
                                        sg.FunctionSpace(shape[2], "C", bc=(0, 0))), form=form)


@pytest.mark.parametrize("shape", [(16, 12, 33), (256, 256, 257)])
@pytest.mark.parametrize("residual", ["fp64", "df"])
def test_helmholtz_refined_matches_direct(sg, shape, residual):
    T = channel_space(sg, shape, "plain")
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    mats = sg.inner(v, -sg.div(sg.grad(u)) + 1000.0 * u)
    Hd = sg.chebyshev.la.Helmholtz(*mats)
    Hr = sg.chebyshev.la.Helmholtz(*mats, form="refined", residual=residual)
    f = sg.inner(v, sg.Array(T, buffer=np.random.default_rng(0).standard_normal(shape)))
    ud = Hd(f, sg.Function(T))
    ur = Hr(f, sg.Function(T))
    assert rel(ur.v[..., :-2], ud.v[..., :-2]) < 1e-12
    it = Hr.last_iterations.cpu().numpy()
    assert it.min() >= 1 and it.max() <= Hr.max_it
    # in place (the right-hand side is re-read every correction: kept)
    g = f.v.clone()
    Hr(g, g)
    assert rel(g[..., :-2], ud.v[..., :-2]) < 1e-12


def test_channel_round_trip_refined_vs_oracle(sg):
    shape = (64, 48, 65)
    T = channel_space(sg, shape, "mixed")
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + 1000.0 * u), form="refined")
    f = np.random.default_rng(1).standard_normal(shape)
    uq = H(sg.inner(v, sg.Array(T, buffer=f)), sg.Function(T)).backward()
    bases = [("fourier", "C2C", shape[0]), ("fourier", "R2C", shape[1]), ("chebyshev", "SD", shape[2])]
    ref, _, _ = P.helmholtz_roundtrip(f, bases, 1000.0, 2)
    assert rel(uq.v, ref) < 1e-10


@pytest.mark.parametrize("shape", [(16, 12, 17), (128, 128, 129)])
def test_biharmonic_refined_matches_direct(sg, shape):
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(shape[0], "F", dtype="D"),
                                     sg.FunctionSpace(shape[1], "F", dtype="d"),
                                     sg.FunctionSpace(shape[2], "C", bc=(0, 0, 0, 0))))
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    mats = sg.inner(v, sg.div(sg.grad(sg.div(sg.grad(u)))))
    Hd = sg.chebyshev.la.Biharmonic(mats)
    Hr = sg.chebyshev.la.Biharmonic(mats, form="refined")
    f = sg.inner(v, sg.Array(T, buffer=np.random.default_rng(2).standard_normal(shape)))
    ud = Hd(f, sg.Function(T))
    ur = Hr(f, sg.Function(T))
    assert rel(ur.v[..., :-4], ud.v[..., :-4]) < 1e-12
    it = Hr.last_iterations.cpu().numpy()
    assert it.min() >= 1 and it.max() <= Hr.max_it


@pytest.mark.parametrize("key,shape", [("h8x8x17", (8, 8, 17, None)), ("h6x4x16", (6, 4, 16, None))])
def test_helmholtz_refined_golden(sg, golden, key, shape):
    """The reference's Helmholtz solves (fixture recorded from shenfun's own
    LU_Helmholtz / Solve_Helmholtz) through the refined path."""
    d = golden("helmholtz")
    Nx, Ny, Nz, _ = shape
    c = float(d[key + "_c"])
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(Nx, "F", dtype="D"), sg.FunctionSpace(Ny, "F", dtype="d"),
                                     sg.FunctionSpace(Nz, "C", bc=(0, 0))))
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    for residual in ("fp64", "df"):
        H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + c * u), form="refined", residual=residual)
        uh = H(torch.as_tensor(d[key + "_f"], device="cuda"), sg.Function(T))
        assert rel(uh.v[..., :-2], d[key + "_u"][..., :-2]) < 1e-12


def test_helmholtz_refined_oracle_lu(sg):
    """Seven systems with shifts up to 4000 through (A, B, alfa, beta), against
    the oracle's restatement of LU_Helmholtz / Solve_Helmholtz."""
    from shenfun_gb300.matrices import galerkin_matrix
    from shenfun_gb300.spaces import ChebyshevShenDirichlet
    N = 33
    alfa = -np.ones(7)
    beta = np.linspace(1.0, 4000.0, 7)
    f = np.random.default_rng(3).standard_normal((N, 7))
    uref = OL.helmholtz_solve(f.T, *OL.helmholtz_lu(N, alfa, beta)).T
    V = ChebyshevShenDirichlet(N)
    A, B = galerkin_matrix(V, 2), galerkin_matrix(V, 0)
    H = sg.chebyshev.la.Helmholtz(A, B, alfa.reshape(1, 7), beta.reshape(1, 7), form="refined")
    u = H(torch.as_tensor(f, device="cuda"))
    assert rel(u[:N - 2], uref[:N - 2]) < 1e-12
