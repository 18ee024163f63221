"""GPU parity: the CUDA path through the C ABI against the oracle and the
reference's golden fixtures.  Plain form: FP64, relative error <= 1e-12
(max-abs error over max-abs reference) unless a case states otherwise."""
import numpy as np
import pytest
import torch

from oracle import spectral as S, la as OL, problems as P

pytestmark = pytest.mark.gpu

TOL = 1e-12


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


rng = np.random.default_rng(11)


@pytest.mark.parametrize("n", [8, 9, 16, 17, 43, 64, 129, 256, 257])
def test_fourier_axis_transforms(sg, n):
    from shenfun_gb300.spaces import R2C, C2C
    x = rng.standard_normal((4, n, 6))
    R = R2C(n)
    y = R.forward(dev(x), axis=1)
    assert rel(y, S.r2c_forward(x, axis=1)) < TOL
    z = R.backward(y, axis=1)
    assert rel(z, S.r2c_backward(y.cpu().numpy(), n, axis=1)) < TOL
    xc = x + 1j * rng.standard_normal(x.shape)
    C = C2C(n)
    yc = C.forward(dev(xc), axis=1)
    assert rel(yc, S.c2c_forward(xc, axis=1)) < TOL
    assert rel(C.backward(yc, axis=1), xc) < TOL


@pytest.mark.parametrize("n", [12, 16, 17, 33, 64, 129, 257])
@pytest.mark.parametrize("basis", ["T", "SD", "SB"])
@pytest.mark.parametrize("cplx", [False, True])
def test_chebyshev_axis_transforms(sg, n, basis, cplx):
    from shenfun_gb300.spaces import (ChebyshevOrthogonal, ChebyshevShenDirichlet,
                                      ChebyshevShenBiharmonic)
    V = {"T": ChebyshevOrthogonal, "SD": ChebyshevShenDirichlet, "SB": ChebyshevShenBiharmonic}[basis](n)
    for shape, axis in (((5, 3, n), 2), ((3, n, 7), 1)):
        x = rng.standard_normal(shape)
        if cplx:
            x = x + 1j * rng.standard_normal(shape)
        assert rel(V.scalar_product(dev(x), axis=axis), S.cheb_scalar_product(x, basis, axis)) < TOL
        fw = V.forward(dev(x), axis=axis)
        assert rel(fw, S.cheb_forward(x, basis, axis)) < (TOL if basis != "SB" else 5e-11)
        fwn = fw.cpu().numpy()
        assert rel(V.backward(fw, axis=axis), S.cheb_backward(fwn, basis, axis)) < TOL


def test_golden_1d(sg, golden):
    from shenfun_gb300.spaces import (ChebyshevOrthogonal, ChebyshevShenDirichlet,
                                      ChebyshevShenBiharmonic, R2C, C2C)
    d = golden("cheb_1d")
    cls = {"T": ChebyshevOrthogonal, "SD": ChebyshevShenDirichlet, "SB": ChebyshevShenBiharmonic}
    for N in (8, 9, 16, 17, 33, 64):
        for tag, C in cls.items():
            if f"{tag}{N}_f" not in d:
                continue
            V = C(N)
            assert rel(V.scalar_product(dev(d[f"{tag}{N}_f"])), d[f"{tag}{N}_sp"]) < TOL
            assert rel(V.forward(dev(d[f"{tag}{N}_f"])), d[f"{tag}{N}_fw"]) < TOL
            assert rel(V.backward(dev(d[f"{tag}{N}_uh"])), d[f"{tag}{N}_bw"]) < TOL
    d = golden("fourier_1d")
    for N in (8, 9, 16, 64):
        assert rel(R2C(N).forward(dev(d[f"R{N}_f"])), d[f"R{N}_fw"]) < TOL
        assert rel(R2C(N).backward(dev(d[f"R{N}_uh"])), d[f"R{N}_bw"]) < TOL
        assert rel(C2C(N).forward(dev(d[f"C{N}_f"])), d[f"C{N}_fw"]) < TOL
        assert rel(C2C(N).backward(dev(d[f"C{N}_uh"])), d[f"C{N}_bw"]) < TOL


@pytest.mark.parametrize("shape", [(8, 8, 17, 1000.0), (6, 4, 16, 0.0), (4, 6, 33, 50.0)])
def test_golden_helmholtz(sg, golden, shape):
    Nx, Ny, Nz, c = shape
    d = golden("helmholtz")
    k = f"h{Nx}x{Ny}x{Nz}"
    F0 = sg.FunctionSpace(Nx, "F", dtype="D")
    F1 = sg.FunctionSpace(Ny, "F", dtype="d")
    SD = sg.FunctionSpace(Nz, "C", bc=(0, 0))
    T = sg.TensorProductSpace(None, (F0, F1, SD))
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + c * u))
    assert rel(H.alfa, d[k + "_alfa"]) == 0 and rel(H.beta, d[k + "_beta"]) == 0
    for name, arr in (("_d0", H.u0), ("_d1", H.u1), ("_d2", H.u2), ("_L", H.L)):
        assert rel(arr, d[k + name]) < 1e-14, name
    uh = H(dev(d[k + "_f"]), sg.Function(T))
    assert rel(uh, d[k + "_u"]) < TOL
    mv = H.matvec(dev(d[k + "_u"]), torch.zeros_like(dev(d[k + "_u"])))
    assert rel(mv, d[k + "_mv"]) < TOL


def test_golden_helmholtz_axis0(sg, golden):
    d = golden("helmholtz")
    SD = sg.FunctionSpace(20, "C", bc=(0, 0))
    F1 = sg.FunctionSpace(6, "F", dtype="d")
    T = sg.TensorProductSpace(None, (SD, F1), axes=(0, 1))
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + 7.5 * u))
    assert rel(H.u0, d["h2d_d0"]) < 1e-14
    uh = H(dev(d["h2d_f"]), sg.Function(T))
    assert rel(uh, d["h2d_u"]) < TOL


def test_golden_cfg1_poisson2d(sg, golden):
    d = golden("cfg1_poisson2d")
    K0 = sg.FunctionSpace(64, "F", dtype="d")
    SD = sg.FunctionSpace(64, "C", bc=(0, 0))
    T = sg.TensorProductSpace(None, (K0, SD), axes=(1, 0))
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    fj = sg.Array(T, buffer=d["fj"])
    f_hat = sg.inner(v, fj)
    assert rel(f_hat, d["f_hat"]) < TOL
    H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u))))
    u_hat = H(f_hat, sg.Function(T))
    assert rel(u_hat, d["u_hat"]) < TOL
    g = sg.la.SolverGeneric1ND(sg.inner(v, -sg.div(sg.grad(u))))
    assert rel(g(f_hat, sg.Function(T)), d["u_hat_generic"]) < TOL
    uq = u_hat.backward()
    assert rel(uq, d["uq"]) < TOL
    assert rel(uq, d["uj"]) < 1e-12
    assert rel(sg.Array(T, buffer=d["uj"]).forward(), d["fw"]) < TOL


@pytest.mark.parametrize("shape", [(8, 8, 17), (16, 12, 24)])
def test_golden_cfg2_small(sg, golden, shape):
    d = golden("cfg2_%dx%dx%d" % shape)
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(shape[0], "F", dtype="D"),
                                     sg.FunctionSpace(shape[1], "F", dtype="d"),
                                     sg.FunctionSpace(shape[2], "C", bc=(0, 0))))
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + 1000.0 * u))
    f_hat = sg.inner(v, sg.Array(T, buffer=d["fj"]))
    assert rel(f_hat, d["f_hat"]) < TOL
    u_hat = H(f_hat, sg.Function(T))
    assert rel(u_hat, d["u_hat"]) < TOL
    assert rel(u_hat.backward(), d["uq"]) < TOL
    fw = sg.Array(T, buffer=d["fj"]).forward()
    assert rel(fw, d["fw"]) < TOL
    assert rel(fw.backward(), d["fwbw"]) < TOL


def test_cfg2_full_size(sg):
    """Fourier 256 x Fourier 256 x Chebyshev SD 257, alpha = k^2 + 1/(nu dt),
    nu dt = 1e-3, RHS N(0,1) from seed 0: GPU round trip against the oracle,
    plus the size-independent checks (H u_hat reproduces f_hat on the dofs;
    forward o backward is the identity on spectral space)."""
    Nx, Ny, Nz = 256, 256, 257
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(Nx, "F", dtype="D"),
                                     sg.FunctionSpace(Ny, "F", dtype="d"),
                                     sg.FunctionSpace(Nz, "C", bc=(0, 0))))
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + 1000.0 * u))
    f = np.random.default_rng(0).standard_normal((Nx, Ny, Nz))
    fj = sg.Array(T, buffer=f)
    f_hat = sg.inner(v, fj)
    u_hat = H(f_hat, sg.Function(T))
    uq = u_hat.backward()
    bases = [("fourier", "C2C", Nx), ("fourier", "R2C", Ny), ("chebyshev", "SD", Nz)]
    ref_u, ref_fh, ref_uh = P.helmholtz_roundtrip(f, bases, 1000.0, 2)
    assert rel(f_hat, ref_fh) < TOL
    assert rel(u_hat, ref_uh) < TOL
    assert rel(uq, ref_u) < TOL
    mv = H.matvec(u_hat.v, torch.zeros_like(u_hat.v))
    assert rel(mv[..., :-2], f_hat.v[..., :-2]) < 1e-11
    fw = uq.forward()
    assert rel(fw[..., :-2], u_hat.v[..., :-2]) < 1e-11


def test_reference_layout_solve_entry(sg, golden):
    """sgpu_Solve_Helmholtz (reference-layout factors) agrees with the cache path."""
    d = golden("helmholtz")
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(8, "F", dtype="D"),
                                     sg.FunctionSpace(8, "F", dtype="d"),
                                     sg.FunctionSpace(17, "C", bc=(0, 0))))
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + 1000.0 * u))
    f = dev(d["h8x8x17_f"])
    out = torch.zeros_like(f)
    H.solve_reference_layout(f, out)
    assert rel(out, d["h8x8x17_u"]) < TOL


MIXED_TOL = 1e-10   # the mixed form's bound against the FP64 oracle


@pytest.mark.parametrize("shape", [(8, 8, 17), (16, 12, 24)])
def test_mixed_form_small(sg, golden, shape):
    d = golden("cfg2_%dx%dx%d" % shape)
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(shape[0], "F", dtype="D"),
                                     sg.FunctionSpace(shape[1], "F", dtype="d"),
                                     sg.FunctionSpace(shape[2], "C", bc=(0, 0))), form="mixed")
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + 1000.0 * u))
    f_hat = sg.inner(v, sg.Array(T, buffer=d["fj"]))
    assert rel(f_hat, d["f_hat"]) < MIXED_TOL
    u_hat = H(f_hat, sg.Function(T))
    assert rel(u_hat, d["u_hat"]) < MIXED_TOL
    assert rel(u_hat.backward(), d["uq"]) < MIXED_TOL


def test_mixed_form_cfg2_full_size(sg):
    Nx, Ny, Nz = 256, 256, 257
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(Nx, "F", dtype="D"),
                                     sg.FunctionSpace(Ny, "F", dtype="d"),
                                     sg.FunctionSpace(Nz, "C", bc=(0, 0))), form="mixed")
    u, v = sg.TrialFunction(T), sg.TestFunction(T)
    H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + 1000.0 * u))
    f = np.random.default_rng(0).standard_normal((Nx, Ny, Nz))
    uq = H(sg.inner(v, sg.Array(T, buffer=f)), sg.Function(T)).backward()
    bases = [("fourier", "C2C", Nx), ("fourier", "R2C", Ny), ("chebyshev", "SD", Nz)]
    ref, _, _ = P.helmholtz_roundtrip(f, bases, 1000.0, 2)
    err = rel(uq, ref)
    assert err < MIXED_TOL, err
