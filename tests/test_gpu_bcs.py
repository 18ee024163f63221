"""GPU parity for non-homogeneous boundary values on a Chebyshev axis
(ShenDirichlet bc=(a, b), ShenNeumann {'left': {'N': a}, 'right': {'N': b}}):
forward, backward and the Helmholtz solve with boundary matrices, in 1D and on
tensor-product grids, against the reference's fixtures
(tests/golden/nonhomog.npz) and the oracle.  Plain form: relative error
<= 1e-12; mixed form <= 1e-10."""
import numpy as np
import pytest
import torch

from oracle import bcs as BC, problems as P

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL_MIXED = 1e-10
BCV = {"SD": (1.5, -0.5), "SN": (0.7, -0.3)}


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


def space(sg, tag, N, vals=None):
    vals = BCV[tag] if vals is None else vals
    if tag == "SD":
        return sg.FunctionSpace(N, "C", bc=vals)
    return sg.FunctionSpace(N, "C", bc={"left": {"N": vals[0]}, "right": {"N": vals[1]}})


@pytest.mark.parametrize("tag", ["SD", "SN"])
@pytest.mark.parametrize("N", [12, 17])
def test_nonhomog_1d_golden(sg, golden, tag, N):
    d = golden("nonhomog")
    V = space(sg, tag, N)
    assert V.has_nonhomogeneous_bcs
    f = d[f"{tag}{N}_f"]
    assert rel(V.scalar_product(dev(f)), d[f"{tag}{N}_sp"]) < TOL
    assert rel(V.forward(dev(f)), d[f"{tag}{N}_fw"]) < TOL
    assert rel(V.backward(dev(d[f"{tag}{N}_uh"])), d[f"{tag}{N}_bw"]) < TOL
    u = sg.Function(V)
    u.set_boundary_dofs()
    assert rel(u[-2:], np.array(BCV[tag])) == 0


@pytest.mark.parametrize("tag", ["SD", "SN"])
@pytest.mark.parametrize("shape", [(8, 6, 17), (16, 6)])
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_nonhomog_tensor_golden(sg, golden, tag, shape, form):
    d = golden("nonhomog")
    key = tag + "_" + "x".join(str(n) for n in shape)
    if len(shape) == 3:
        bases = (sg.FunctionSpace(shape[0], "F", dtype="D"), sg.FunctionSpace(shape[1], "F", dtype="d"),
                 space(sg, tag, shape[2]))
    else:
        bases = (space(sg, tag, shape[0]), sg.FunctionSpace(shape[1], "F", dtype="d"))
    T = sg.TensorProductSpace(None, bases, form=form)
    tol = TOL if form == "plain" else TOL_MIXED
    fa = sg.Array(T, buffer=d[key + "_f"])
    assert rel(fa.forward(), d[key + "_fw"]) < tol
    v, u = sg.TestFunction(T), sg.TrialFunction(T)
    fh = sg.inner(v, fa)
    assert rel(fh, d[key + "_sp"]) < tol
    uh = sg.Function(T, buffer=d[key + "_uh"])
    assert rel(uh.backward(), d[key + "_bw"]) < tol
    H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + 5.0 * u))
    x = H(sg.Function(T, buffer=d[key + "_rhs"]), sg.Function(T))
    assert rel(x, d[key + "_sol"]) < tol
    assert rel(x.backward(), d[key + "_solx"]) < tol


@pytest.mark.parametrize("tag", ["SD", "SN"])
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_nonhomog_channel_poisson(sg, tag, form):
    """-div(grad(u)) + u = f on Fourier 32 x Fourier 32 x Chebyshev 65 with
    wall values: the GPU chain (scalar product, solve with boundary
    matrices, backward) against the oracle; for Dirichlet walls the backward
    solution takes the wall values at x = +-1 (evaluated through the
    Chebyshev series of the mean mode)."""
    Nx, Ny, Nz = 32, 32, 65
    vals = (2.0, -1.0)
    bases = (sg.FunctionSpace(Nx, "F", dtype="D"), sg.FunctionSpace(Ny, "F", dtype="d"),
             space(sg, tag, Nz, vals))
    T = sg.TensorProductSpace(None, bases, form=form)
    rng = np.random.default_rng(5)
    f = rng.standard_normal((Nx, Ny, Nz))
    v, u = sg.TestFunction(T), sg.TrialFunction(T)
    H = sg.chebyshev.la.Helmholtz(*sg.inner(v, -sg.div(sg.grad(u)) + 1.0 * u))
    fh = sg.inner(v, sg.Array(T, buffer=f))
    uh = H(fh, sg.Function(T))
    ua = uh.backward()
    ob = [("fourier", "C2C", Nx), ("fourier", "R2C", Ny), ("chebyshev", tag, Nz)]
    fh_ref = P.scalar_product(f, ob)
    uh_ref = BC.helmholtz_bc_solve(fh_ref, ob, 1.0, 2, vals)
    tol = TOL if form == "plain" else TOL_MIXED
    assert rel(uh, uh_ref) < tol
    assert rel(ua, BC.tp_backward(uh_ref, ob, 2)) < tol * 10
    if tag == "SD":
        # u(+-1) of the mean mode from its coefficients: the wall values
        c = uh_ref[0, 0]
        from oracle import spectral as S
        K = S.stencil("chebyshev", "SD", Nz)
        t = S.to_ortho(c, K, Nz - 2)
        t = BC.add_to_orthogonal(t, c, "SD")
        k = np.arange(Nz)
        assert abs(np.sum(t * (-1.0) ** k) - vals[0]) < 1e-12
        assert abs(np.sum(t) - vals[1]) < 1e-12
