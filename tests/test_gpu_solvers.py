"""GPU parity: Legendre spaces, per-wavenumber banded/semiseparable solves
(SolverGeneric1ND, Biharmonic) against the reference's golden fixtures and
the oracle.  Plain FP64 form, relative error (max-abs over max-abs)."""
import numpy as np
import pytest
import torch

from oracle import spectral as S, problems as P

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda")


@pytest.fixture(scope="module")
def sg():
    from shenfun_gb300 import build
    build.build()
    import shenfun_gb300
    return shenfun_gb300


@pytest.mark.parametrize("N", [16, 33, 64])
@pytest.mark.parametrize("kind", ["recursive", "vandermonde"])
def test_legendre_1d_golden(sg, golden, N, kind):
    from shenfun_gb300.legendre import LegendreOrthogonal, LegendreShenDirichlet
    d = golden("legendre")
    for tag, C in (("L", LegendreOrthogonal), ("LD", LegendreShenDirichlet)):
        V = C(N)
        assert rel(V.scalar_product(dev(d[f"{tag}{N}_f"]), kind=kind), d[f"{tag}{N}_sp_{kind}"]) < 1e-13
        assert rel(V.backward(dev(d[f"{tag}{N}_uh"]), kind=kind), d[f"{tag}{N}_bw_{kind}"]) < 1e-13
        assert rel(V.forward(dev(d[f"{tag}{N}_f"]), kind=kind), d[f"{tag}{N}_fw_{kind}"]) < 1e-12


@pytest.mark.parametrize("N", [12, 64, 129])
@pytest.mark.parametrize("basis", ["L", "SD", "SB"])
@pytest.mark.parametrize("cplx", [False, True])
def test_legendre_axis(sg, N, basis, cplx):
    from shenfun_gb300 import legendre as L
    V = {"L": L.LegendreOrthogonal, "SD": L.LegendreShenDirichlet, "SB": L.LegendreShenBiharmonic}[basis](N)
    rng = np.random.default_rng(N)
    for shape, axis in (((3, 5, N), 2), ((4, N, 3), 1)):
        x = rng.standard_normal(shape)
        if cplx:
            x = x + 1j * rng.standard_normal(shape)
        assert rel(V.scalar_product(dev(x), axis=axis), S.leg_scalar_product(x, basis, axis)) < 1e-12
        fw = S.leg_forward(x, basis, axis)
        assert rel(V.forward(dev(x), axis=axis), fw) < (1e-11 if basis != "SB" else 1e-9)
        assert rel(V.backward(dev(fw), axis=axis), S.leg_backward(fw, basis, axis)) < 1e-12


def test_legendre_poisson2d_golden(sg, golden):
    d = golden("legendre")
    K0 = sg.FunctionSpace(16, "F", dtype="d")
    LD = sg.FunctionSpace(24, "L", bc=(0, 0))
    T = sg.TensorProductSpace(None, (K0, LD), axes=(1, 0))
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    f_hat = sg.inner(v, sg.Array(T, buffer=d["p2d_fj"]))
    assert rel(f_hat, d["p2d_fhat"]) < 1e-13
    sol = sg.la.SolverGeneric1ND(sg.inner(v, -sg.div(sg.grad(u)) + 3.0 * u))
    u_hat = sol(f_hat, sg.Function(T))
    assert rel(u_hat, d["p2d_uhat"]) < 1e-12
    assert rel(u_hat.backward(), d["p2d_uq"]) < 1e-12


@pytest.mark.parametrize("Nz", [16, 17])
def test_biharmonic_golden(sg, golden, Nz):
    d = golden(f"biharmonic_8x8x{Nz}")
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(8, "F", dtype="D"),
                                     sg.FunctionSpace(8, "F", dtype="d"),
                                     sg.FunctionSpace(Nz, "C", bc=(0, 0, 0, 0))))
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    f_hat = sg.inner(v, sg.Array(T, buffer=d["fj"]))
    assert rel(f_hat, d["f_hat"]) < 1e-13
    mats = sg.inner(v, sg.div(sg.grad(sg.div(sg.grad(u)))))
    for solver in (sg.la.SolverGeneric1ND(mats), sg.chebyshev.la.Biharmonic(mats)):
        u_hat = solver(f_hat, sg.Function(T))
        assert rel(u_hat, d["u_hat_generic"]) < 1e-12
        assert rel(u_hat.backward(), d["uq"]) < 1e-12
        assert rel(u_hat.backward(), d["uj"]) < 1e-10   # manufactured solution


def test_cfg3_biharmonic_full_size(sg):
    """Fourier 128 x Fourier 128 x Chebyshev ShenBiharmonic 129, manufactured
    u = sin(x) cos(y) (1 - z^2)^2: GPU round trip against the oracle (one dense
    direct solve per wavenumber) and against the exact solution."""
    import sympy as sp
    Nx, Ny, Nz = 128, 128, 129
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(Nx, "F", dtype="D"),
                                     sg.FunctionSpace(Ny, "F", dtype="d"),
                                     sg.FunctionSpace(Nz, "C", bc=(0, 0, 0, 0))))
    x, y, z = sp.symbols("x,y,z", real=True)
    ue = sp.sin(x) * sp.cos(y) * (1 - z ** 2) ** 2
    fe = ue.diff(x, 4) + ue.diff(y, 4) + ue.diff(z, 4) + 2 * ue.diff(x, 2, y, 2) + \
        2 * ue.diff(x, 2, z, 2) + 2 * ue.diff(y, 2, z, 2)
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    fj = sg.Array(T, buffer=fe)
    f_hat = sg.inner(v, fj)
    H = sg.chebyshev.la.Biharmonic(sg.inner(v, sg.div(sg.grad(sg.div(sg.grad(u))))))
    uq = H(f_hat, sg.Function(T)).backward()
    bases = [("fourier", "C2C", Nx), ("fourier", "R2C", Ny), ("chebyshev", "SB", Nz)]
    fnp = fj.v.cpu().numpy()
    ref_fh = P.scalar_product(fnp, bases)
    assert rel(f_hat, ref_fh) < 1e-12
    ref = P.backward(P.biharmonic_solve(ref_fh, bases, 2), bases)
    assert rel(uq, ref) < 1e-10
    assert rel(uq, sg.Array(T, buffer=ue).v) < 1e-10


@pytest.mark.parametrize("Nz", [16, 17, 65])
def test_biharmonic_matvec(sg, Nz):
    """Biharmonic.matvec (the residual Biharmonic_matvec, Matvec.pyx:908):
    the product of the oracle's dense SSBSB / ASBSB / BSBSB per wavenumber
    (scales 1, -2 k^2, k^4 of inner(v, div(grad(div(grad(u)))))), and it
    undoes the solve on the dofs; also for a Legendre ShenDirichlet system."""
    from oracle import la as OL
    Nx, Ny = 8, 6
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(Nx, "F", dtype="D"), sg.FunctionSpace(Ny, "F", dtype="d"),
                                     sg.FunctionSpace(Nz, "C", bc=(0, 0, 0, 0))))
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    H = sg.chebyshev.la.Biharmonic(sg.inner(v, sg.div(sg.grad(sg.div(sg.grad(u))))))
    rng = np.random.default_rng(Nz)
    shape = (Nx, Ny // 2 + 1, Nz)
    w = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    w[..., Nz - 4:] = 0
    c = H.matvec(dev(w), torch.zeros(shape, dtype=torch.complex128, device="cuda"))
    Sm, Am, Bm = OL.cheb_sb_dense(Nz)
    k2 = P.fourier_k2([("fourier", "C2C", Nx), ("fourier", "R2C", Ny), ("chebyshev", "SB", Nz)], 2)
    k2 = np.broadcast_to(k2, (Nx, Ny // 2 + 1, 1)).reshape(-1)
    ws = w.reshape(-1, Nz)[:, :Nz - 4]
    ref = np.zeros_like(w.reshape(-1, Nz))
    for s in range(ws.shape[0]):
        ref[s, :Nz - 4] = (Sm - 2 * k2[s] * Am + k2[s] ** 2 * Bm) @ ws[s]
    assert rel(c.reshape(-1, Nz), ref) < 1e-12
    x = H(c, torch.zeros_like(c))
    assert rel(x, w) < 1e-10


DMA_OFFSETS = {"DiagMA": (0,), "TwoDMA": (0, 2), "ThreeDMA": (0, 2, 4), "FDMA": (-2, 0, 2, 4),
               "HeptaDMA": (-4, -2, 0, 2, 4, 6, 8)}


@pytest.mark.parametrize("name", sorted(DMA_OFFSETS))
@pytest.mark.parametrize("n", [12, 17])
def test_banded_solvers_golden(sg, golden, name, n):
    """The reference's other banded solvers through sgpu_banded_LU / _Solve:
    every recorded right-hand side (1D, and 2D along either axis) against the
    reference's own solution, and complex right-hand sides against the
    oracle."""
    from oracle import la as OL
    from shenfun_gb300.matrices import SpectralMatrix
    d = golden("dma")
    D = d[f"{name}{n}_dense"]
    offs = DMA_OFFSETS[name]
    mat = SpectralMatrix(name, {o: np.diagonal(D, o).copy() for o in offs}, (n, n))
    solver = getattr(sg.la, name)(mat)
    keys = [k[:-2] for k in d if k.startswith(f"{name}{n}_") and k.endswith("_b")]
    for key in keys:
        u = solver(dev(d[key + "_b"]), axis=int(key[-1]))
        assert rel(u, d[key + "_u"]) < 1e-12
    rng = np.random.default_rng(n)
    b = rng.standard_normal((3, n, 4)) + 1j * rng.standard_normal((3, n, 4))
    data = np.zeros((len(offs), n))
    for r, o in enumerate(offs):
        for i in range(n):
            if 0 <= i + o < n:
                data[r, i + o] = D[i, i + o]
    if name == "ThreeDMA":
        data = OL.threedma_effective(data)
    OL.banded_lu(data, offs)
    assert rel(solver(dev(b), axis=1), OL.banded_solve(b, data, offs, axis=1)) < 1e-12
