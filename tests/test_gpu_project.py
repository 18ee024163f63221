"""project() of Functions and expressions, linear forms of expressions, and
SpectralMatrix.solve / get_solver, against fixtures recorded from the
unmodified reference (tests/golden/project.npz)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def sg():
    import shenfun_gb300 as sg
    return sg


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def fn(sg, space, values):
    return sg.Function(space, buffer=values)


def test_project_1d_chebyshev_legendre(sg, golden):
    d = golden("project")
    SD = sg.FunctionSpace(14, "C", bc=(0, 0))
    SB = sg.FunctionSpace(16, "C", bc=(0, 0, 0, 0))
    SN = sg.FunctionSpace(14, "C", bc={"left": {"N": 0}, "right": {"N": 0}})
    T14, T16 = sg.FunctionSpace(14, "C"), sg.FunctionSpace(16, "C")
    u = fn(sg, SD, d["sd_u"])
    assert rel(sg.project(sg.Dx(u, 0, 1), T14), d["sd_dx_T"]) < TOL
    assert rel(sg.project(sg.Dx(u, 0, 2), SD), d["sd_dxx_SD"]) < TOL
    assert rel(sg.project(u, T14), d["sd_u_T"]) < TOL
    assert rel(sg.project(sg.div(sg.grad(u)), T14), d["sd_lap_T"]) < TOL
    assert rel(sg.inner(sg.TestFunction(SD), sg.Dx(u, 0, 2)), d["sd_inner_dxx"]) < TOL
    assert rel(sg.inner(sg.TestFunction(T14), u), d["sd_inner_u_T"]) < TOL
    ub = fn(sg, SB, d["sb_u"])
    assert rel(sg.project(sg.Dx(ub, 0, 3), T16), d["sb_d3_T"]) < TOL
    assert rel(sg.project(sg.div(sg.grad(ub)), SB), d["sb_lap_SB"]) < TOL
    un = fn(sg, SN, d["sn_u"])
    assert rel(sg.project(sg.Dx(un, 0, 1), T14), d["sn_dx_T"]) < TOL
    LSD, L14 = sg.FunctionSpace(14, "L", bc=(0, 0)), sg.FunctionSpace(14, "L")
    ul = fn(sg, LSD, d["l_u"])
    assert rel(sg.project(sg.Dx(ul, 0, 1), L14), d["l_dx_L"]) < TOL
    assert rel(sg.project(sg.Dx(ul, 0, 2), LSD), d["l_dxx_SD"]) < TOL


def test_project_tensor_product(sg, golden):
    d = golden("project")
    F0 = sg.FunctionSpace(6, "F", dtype="D")
    F1 = sg.FunctionSpace(8, "F", dtype="d")
    SD, T14 = sg.FunctionSpace(14, "C", bc=(0, 0)), sg.FunctionSpace(14, "C")
    T3 = sg.TensorProductSpace(sg.comm, (F0, F1, SD))
    T3o = sg.TensorProductSpace(sg.comm, (F0, F1, T14))
    u3 = fn(sg, T3, d["t3_u"])
    assert rel(sg.project(sg.Dx(u3, 2, 1), T3o), d["t3_dz_T"]) < TOL
    assert rel(sg.project(sg.div(sg.grad(u3)), T3), d["t3_lap"]) < TOL
    assert rel(sg.project(sg.Dx(u3, 0, 1) + 2 * sg.Dx(u3, 1, 2), T3), d["t3_mix"]) < TOL
    assert rel(sg.inner(sg.TestFunction(T3), sg.div(sg.grad(u3))), d["t3_inner_lap"]) < TOL
    FF = sg.TensorProductSpace(sg.comm, (F0, F1))
    uf = fn(sg, FF, d["ff_u"])
    assert rel(sg.project(sg.Dx(uf, 1, 1) - sg.Dx(uf, 0, 2), FF), d["ff_d"]) < TOL


def test_project_derivative_identities_large(sg):
    """Size-independent checks at N = 257 on the channel-like grid: the
    projected Laplacian of u equals the backward / forward transform route
    (exact for Gauss quadrature), and projecting u on the orthogonal basis then
    back reproduces u on the mesh."""
    g = np.random.default_rng(3)
    F0 = sg.FunctionSpace(16, "F", dtype="D")
    F1 = sg.FunctionSpace(16, "F", dtype="d")
    SD, T = sg.FunctionSpace(257, "C", bc=(0, 0)), sg.FunctionSpace(257, "C")
    TS = sg.TensorProductSpace(sg.comm, (F0, F1, SD))
    TO = sg.TensorProductSpace(sg.comm, (F0, F1, T))
    # a smooth field: decaying spectrum on every axis
    shape = TS.shape(True)
    c = (g.standard_normal(shape) + 1j * g.standard_normal(shape)) / (1.0 + np.arange(shape[2])) ** 3
    c[..., 255:] = 0
    u = sg.Function(TS, buffer=c)
    uo = sg.project(u, TO)
    x1 = u.backward()
    x2 = uo.backward()
    assert rel(x2, x1) < 1e-12
    du = sg.project(sg.Dx(u, 2, 1), TO)
    # d/dz of the orthogonal expansion by the Chebyshev recurrence (host)
    co = uo.detach().cpu().numpy()
    dref = np.polynomial.chebyshev.chebder(np.moveaxis(co, 2, 0), 1)
    dref = np.concatenate([dref, np.zeros((1,) + dref.shape[1:])], 0)
    assert rel(du, np.moveaxis(dref, 0, 2)) < 1e-11


MS = [("csd", ("C", (0, 0), 14)), ("csb", ("C", (0, 0, 0, 0), 16)),
      ("csn", ("C", {"left": {"N": 0}, "right": {"N": 0}}, 14)), ("lsd", ("L", (0, 0), 14))]


@pytest.mark.parametrize("name,spec", MS, ids=[m[0] for m in MS])
def test_spectral_matrix_solve(sg, golden, name, spec):
    d = golden("project")
    fam, bc, N = spec
    space = sg.FunctionSpace(N, fam, bc=bc)
    v, w = sg.TestFunction(space), sg.TrialFunction(space)
    forms = {"B": lambda: sg.inner(v, w), "A": lambda: sg.inner(v, sg.div(sg.grad(w))),
             "S": lambda: sg.inner(v, sg.div(sg.grad(sg.div(sg.grad(w)))))}
    ran = 0
    for key, make in forms.items():
        for tag in (f"ms_{name}{key}_1d0", f"ms_{name}{key}_2d0", f"ms_{name}{key}_2d1"):
            if tag + "_b" not in d:
                continue
            mat = make()
            assert type(mat).__name__ == "SpectralMatrix"
            ax = int(tag[-1])
            want = str(d[tag + "_solver"])
            assert mat.get_solver().__name__ == want, (tag, mat.get_solver().__name__, want)
            b = torch.as_tensor(d[tag + "_b"], device="cuda")
            cons = ((0, 0),) if (name == "csn" and key == "A") else ()
            x = mat.solve(b, axis=ax, constraints=cons).detach().cpu().numpy()
            ref = d[tag + "_x"]
            bad = ~np.isfinite(ref)
            if bad.any():
                # the reference's DiagMA_Solve_2D/3D divides all N entries of a
                # line by the diagonal (la.pyx:128-146), reading past its n
                # entries for the boundary rows; only those rows may differ
                rows = np.nonzero(np.moveaxis(bad, ax, 0).reshape(bad.shape[ax], -1).any(1))[0]
                assert rows.min() >= mat.shape[0], (tag, rows)
                keep = [slice(None)] * ref.ndim
                keep[ax] = slice(0, mat.shape[0])
                x, ref = x[tuple(keep)], ref[tuple(keep)]
            assert rel(x, ref) < TOL, tag
            ran += 1
    assert ran
