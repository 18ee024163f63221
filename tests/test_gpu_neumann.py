"""GPU parity for the Chebyshev ShenNeumann row: SN transforms, the Neumann
branch of the Helmholtz solver (reference layout and factor cache, both
forms), the Neumann matvec, the ADD / ANN Poisson solvers, and a full
Neumann round trip, against the oracle and the reference's fixtures
(tests/golden/neumann.npz).  Plain form: relative error <= 1e-12; mixed
form <= 1e-10 (max-abs error over max-abs reference)."""
import numpy as np
import pytest
import torch

from oracle import spectral as S, la as OL, problems as P

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL_MIXED = 1e-10


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def sg():
    from shenfun_gb300 import build
    build.build()
    import shenfun_gb300
    from shenfun_gb300 import _lib
    assert _lib.load().sgpu_device_ok() == 1
    return shenfun_gb300


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda")


rng = np.random.default_rng(71)
BCN = {"left": {"N": 0}, "right": {"N": 0}}


@pytest.mark.parametrize("N", [8, 9, 16, 17, 33])
def test_sn_golden_1d(sg, N, golden):
    d = golden("neumann")
    V = sg.FunctionSpace(N, "C", bc=BCN)
    assert V.short_name() == "SN"
    f = d[f"sn{N}_f"]
    assert rel(V.scalar_product(dev(f)), d[f"sn{N}_sp"]) < TOL
    assert rel(V.forward(dev(f)), d[f"sn{N}_fw"]) < TOL
    assert rel(V.backward(dev(d[f"sn{N}_uh"])), d[f"sn{N}_bw"]) < TOL


@pytest.mark.parametrize("n", [12, 16, 17, 33, 64, 129, 257, 1100])
@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_sn_axis_transforms(sg, n, cplx, form):
    from shenfun_gb300 import _lib
    from shenfun_gb300.spaces import ChebyshevShenNeumann
    V = ChebyshevShenNeumann(n)
    V.form = _lib.FORMS[form]
    x = rng.standard_normal((3, n, 5))
    if cplx:
        x = x + 1j * rng.standard_normal(x.shape)
    tol = TOL if form == "plain" else TOL_MIXED
    assert rel(V.scalar_product(dev(x), axis=1), S.cheb_scalar_product(x, "SN", 1)) < tol
    fw = V.forward(dev(x), axis=1)
    assert rel(fw, S.cheb_forward(x, "SN", 1)) < tol
    ref_fw = S.cheb_forward(x, "SN", 1)
    assert rel(V.backward(dev(ref_fw), axis=1), S.cheb_backward(ref_fw, "SN", 1)) < tol


@pytest.mark.parametrize("key", ["h6x4x16", "h4x6x17", "h8x8x33"])
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_helmholtz_neumann_golden(sg, key, form, golden):
    """Helmholtz(*inner(v, -div(grad(u)) + c u)) on Fourier x Fourier x
    ShenNeumann against the reference's factors and solution; c = 0 holds
    the singular zero mode (u_0 = 0)."""
    d = golden("neumann")
    Nx, Ny, Nz = (int(t) for t in key[1:].split("x"))
    c = float(d[key + "_c"])
    F0 = sg.FunctionSpace(Nx, "F", dtype="D")
    F1 = sg.FunctionSpace(Ny, "F", dtype="d")
    SN = sg.FunctionSpace(Nz, "C", bc=BCN)
    T = sg.TensorProductSpace(None, (F0, F1, SN), form=form)
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    H = sg.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + c * u))
    assert H.neumann
    assert rel(H.u0, d[key + "_d0"]) < TOL
    assert rel(H.u1, d[key + "_d1"]) < TOL
    assert rel(H.L, d[key + "_L"]) < TOL
    f = dev(d[key + "_f"])
    x = H(f, torch.zeros_like(f))
    assert rel(x, d[key + "_u"]) < (TOL if form == "plain" else TOL_MIXED)
    x2 = H.solve_reference_layout(f, torch.zeros_like(f))
    assert rel(x2, d[key + "_u"]) < TOL
    mv = H.matvec(x2, torch.zeros_like(f))
    ref = OL.helmholtz_neumann_matvec(d[key + "_u"].reshape(-1, Nz),
                                      np.broadcast_to(d[key + "_alfa"], (Nx, Ny // 2 + 1, 1)).reshape(-1),
                                      np.broadcast_to(d[key + "_beta"], (Nx, Ny // 2 + 1, 1)).reshape(-1))
    assert rel(mv.reshape(-1, Nz), ref) < TOL


@pytest.mark.parametrize("N,shape,axis", [(16, (16,), 0), (17, (17, 6), 0), (33, (5, 33), 1),
                                          (257, (4, 257, 3), 1)])
@pytest.mark.parametrize("cplx", [False, True])
def test_poisson_solvers(sg, N, shape, axis, cplx):
    from shenfun_gb300 import chebyshev
    b = rng.standard_normal(shape)
    if cplx:
        b = b + 1j * rng.standard_normal(shape)
    SD = sg.FunctionSpace(N, "C", bc=(0, 0))
    A = sg.inner(sg.TestFunction(SD), sg.div(sg.grad(sg.TrialFunction(SD))))
    u = chebyshev.la.ADDSolver(A)(dev(b), torch.zeros(shape, dtype=dev(b).dtype, device="cuda"), axis=axis)
    a = OL.cheb_sd_stiffness(N)
    assert rel(u, OL.add_solve(b, a[0], a[2], 1.0, axis=axis)) < TOL
    SN = sg.FunctionSpace(N, "C", bc=BCN)
    A = sg.inner(sg.TestFunction(SN), -sg.div(sg.grad(sg.TrialFunction(SN))))
    u = chebyshev.la.ANNSolver(A)(dev(b), torch.zeros(shape, dtype=dev(b).dtype, device="cuda"), axis=axis)
    a = OL.cheb_sn_stiffness(N)
    assert rel(u, OL.ann_solve(b, a[0], a[2], -1.0, axis=axis)) < TOL


@pytest.mark.parametrize("N", [16, 17, 32])
def test_poisson_golden(sg, N, golden):
    from shenfun_gb300 import chebyshev
    d = golden("neumann")
    SD = sg.FunctionSpace(N, "C", bc=(0, 0))
    A = sg.inner(sg.TestFunction(SD), sg.div(sg.grad(sg.TrialFunction(SD))))
    assert rel(chebyshev.la.ADDSolver(A)(dev(d[f"add{N}_b"])), d[f"add{N}_u"]) < TOL
    SN = sg.FunctionSpace(N, "C", bc=BCN)
    A = sg.inner(sg.TestFunction(SN), -sg.div(sg.grad(sg.TrialFunction(SN))))
    assert rel(chebyshev.la.ANNSolver(A)(dev(d[f"ann{N}_b"])), d[f"ann{N}_u"]) < TOL


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_neumann_roundtrip_channel(sg, form):
    """forward -> Helmholtz (Neumann) -> backward on Fourier 32 x Fourier 32 x
    ShenNeumann 65, against the oracle chain; the solution satisfies the
    Neumann condition u'(+-1) = 0 by construction of the basis."""
    Nx, Ny, Nz, c = 32, 32, 65, 10.0
    F0 = sg.FunctionSpace(Nx, "F", dtype="D")
    F1 = sg.FunctionSpace(Ny, "F", dtype="d")
    SN = sg.FunctionSpace(Nz, "C", bc=BCN)
    T = sg.TensorProductSpace(None, (F0, F1, SN), form=form)
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    H = sg.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + c * u))
    f = rng.standard_normal((Nx, Ny, Nz))
    fh = T.scalar_product(dev(f))
    uh = H(fh, torch.zeros_like(fh))
    ua = T.backward(uh)
    bases = [("fourier", "C2C", Nx), ("fourier", "R2C", Ny), ("chebyshev", "SN", Nz)]
    fh_ref = P.scalar_product(f, bases)
    assert rel(fh, fh_ref) < (TOL if form == "plain" else TOL_MIXED)
    alfa = -np.ones(Nx * (Ny // 2 + 1))
    k = np.fft.fftfreq(Nx, 1 / Nx)[:, None] ** 2 + np.fft.rfftfreq(Ny, 1 / Ny)[None, :] ** 2
    beta = (k + c).reshape(-1)
    fac = OL.helmholtz_lu(Nz, alfa, beta, neumann=True)
    uh_ref = OL.helmholtz_solve(fh_ref.reshape(-1, Nz), *fac, neumann=True).reshape(fh_ref.shape)
    ua_ref = P.backward(uh_ref, bases)
    assert rel(ua, ua_ref) < (1e-11 if form == "plain" else 1e-9)
