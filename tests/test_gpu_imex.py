"""GPU: IMEX Runge-Kutta time stepping (PDEIMEXRK, utilities/integrators.py:702-900)
against the reference's own run (golden fixture) and the oracle; a CUDA-graph
replay of a whole step equals the eager step bit for bit."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

BASES = [("fourier", "C2C", 8), ("fourier", "R2C", 8), ("chebyshev", "SD", 17)]


@pytest.fixture(scope="module")
def sg():
    from shenfun_gb300 import build
    build.build()
    import shenfun_gb300
    return shenfun_gb300


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else a
    return np.abs(a - b).max() / np.abs(b).max()


def make(sg, d, name, form="plain"):
    from shenfun_gb300 import integrators as I
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(8, "F", dtype="D"), sg.FunctionSpace(8, "F", dtype="d"),
                                     sg.FunctionSpace(17, "C", bc=(0, 0))), form=form)
    nu, dt = float(d["nu"]), float(d["dt"])
    u_hat = sg.Function(T, buffer=d["u_hat0"])
    f_hat = sg.Function(T, buffer=d["f_hat"])
    sol = getattr(I, name)(sg.TestFunction(T), u_hat, lambda u: nu * sg.div(sg.grad(u)), f_hat, dt)
    sol.assemble()
    return sol, u_hat


@pytest.mark.parametrize("name", ["IMEXRK111", "IMEXRK222", "IMEXRK443"])
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_imex_golden(sg, golden, name, form):
    d = golden("imex")
    sol, u_hat = make(sg, d, name, form)
    tol = 1e-12 if form == "plain" else 1e-10
    for step in range(3):
        sol.step()
        assert rel(u_hat, d[f"{name}_step{step}"]) < tol, step


def test_imex_graph_replay(sg, golden):
    """capture_step (2 eager warm-up steps, then one captured) + 3 replays
    gives bit for bit the state of 5 eager steps."""
    d = golden("imex")
    eager, ue = make(sg, d, "IMEXRK443")
    for _ in range(5):
        eager.step()
    graph, ug = make(sg, d, "IMEXRK443")
    graph.capture_step(warmup=2)
    for _ in range(3):
        graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(ue, ug)


def test_imex_oracle_longer(sg, golden):
    """Ten steps against the oracle's restatement (the fixture holds three)."""
    from oracle import imex
    d = golden("imex")
    sol, u_hat = make(sg, d, "IMEXRK222")
    ref = imex.imex_run(d["u_hat0"], d["f_hat"], float(d["nu"]), float(d["dt"]), "IMEXRK222", 10, BASES, 2)
    for step in range(10):
        sol.step()
    assert rel(u_hat, ref[-1]) < 1e-12


def test_imex_nonlinear_graph(sg):
    """A nonlinear term through the transforms, N(u) = inner(v, u^2) (backward,
    square, scalar product, mixed form), stepped eagerly and by graph replay:
    equal bit for bit."""
    from shenfun_gb300 import integrators as I
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(16, "F", dtype="D"), sg.FunctionSpace(12, "F", dtype="d"),
                                     sg.FunctionSpace(33, "C", bc=(0, 0))), form="mixed")
    v = sg.TestFunction(T)
    work = sg.Array(T)

    def N(u_hat, out):
        T.backward(u_hat.v, work.v)
        work.v.mul_(work.v)
        T.scalar_product(work.v, out)

    a = sg.Array(T)
    a.v.copy_(torch.randn(a.shape, dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(3)))
    u0 = a.forward()
    res = []
    for graph in (False, True):
        u_hat = sg.Function(T)
        u_hat.v.copy_(u0.v)
        sol = I.IMEXRK443(v, u_hat, lambda u: 0.1 * sg.div(sg.grad(u)), N, 1e-3)
        sol.assemble()
        if graph:
            sol.capture_step(warmup=1)
            for _ in range(3):
                sol.replay()
        else:
            for _ in range(4):
                sol.step()
        torch.cuda.synchronize()
        res.append(u_hat.v.clone())
    assert torch.isfinite(res[0]).all()
    assert torch.equal(res[0], res[1])


@pytest.mark.parametrize("name", ["IMEXRK111", "IMEXRK222", "IMEXRK443"])
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_imex_neumann_oracle(sg, name, form):
    """The IMEX caller on a ShenNeumann axis (the Neumann Helmholtz branch for
    every stage's solve, the Neumann matvec for the linear forms): three
    steps against the oracle's scheme with the Neumann LU and product."""
    from oracle import imex as OI
    from shenfun_gb300 import integrators as I
    nb = [("fourier", "C2C", 8), ("fourier", "R2C", 8), ("chebyshev", "SN", 17)]
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(8, "F", dtype="D"), sg.FunctionSpace(8, "F", dtype="d"),
                                     sg.FunctionSpace(17, "C", bc={"left": {"N": 0}, "right": {"N": 0}})),
                              form=form)
    rng = np.random.default_rng(41)
    shape = (8, 5, 17)
    u0 = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    f0 = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    u0[..., -2:] = 0
    f0[..., -2:] = 0
    nu, dt = 0.1, 0.01
    u_hat = sg.Function(T, buffer=u0)
    sol = getattr(I, name)(sg.TestFunction(T), u_hat, lambda u: nu * sg.div(sg.grad(u)),
                           sg.Function(T, buffer=f0), dt)
    sol.assemble()
    ref = OI.imex_run(u0, f0, nu, dt, name, 3, nb, 2)
    tol = 1e-12 if form == "plain" else 1e-10
    for step in range(3):
        sol.step()
        assert rel(u_hat, ref[step]) < tol, step
