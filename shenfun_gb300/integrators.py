"""IMEX Runge-Kutta time stepping on the GPU path (utilities/integrators.py:702-900).

``PDEIMEXRK`` solves u_t = N + L u with the implicit-explicit Runge-Kutta
schemes of Ascher, Ruuth and Spiteri (Appl. Numer. Math. 25, 1997) in the
reference's form: one implicit solve per stage with the matrix of
``inner(v, u - dt a_kk L(u))`` (a_kk is the same for every stage), explicit
right-hand sides assembled from the stored nonlinear and linear terms, the
Nyquist modes of the Fourier axes masked out of every right-hand side.

Supported here: a tensor-product space with one Chebyshev ShenDirichlet or
ShenNeumann axis and Fourier axes, L of Helmholtz type (a combination of ``div(grad(u))`` and
``u``, e.g. ``lambda u: nu*div(grad(u))``), so that every linear form is a
``sgpu_Helmholtz_matvec`` call and every solve a cached Helmholtz solve.  The
nonlinear term N is a spectral ``Function`` (a forcing: its linear form is
the mass matrix times it, as the reference's ``Inner(v, f_hat)``) or a
callable ``N(u_hat, out)`` that fills ``out`` with the linear form of the
nonlinear term (for instance ``inner(v, nonlinear_array(u_hat.backward()))``).

Every array is preallocated and every step is a fixed sequence of kernel
launches on the current stream, so a whole time step can be captured once in
a CUDA graph and replayed (``capture_step`` / ``replay``).
"""
import numpy as np
import torch

from . import _lib
from .device import ptr, stream_handle, view3, data_kind
from .forms import Function, TrialFunction, TPMatrix, inner
from .la import SolverGeneric1ND
from .spaces import C2C, R2C

__all__ = ["PDEIMEXRK", "IMEXRK011", "IMEXRK111", "IMEXRK222", "IMEXRK443"]


class _HelmholtzForm:
    """c = (alfa A + beta B) v along the Chebyshev ShenDirichlet (or
    ShenNeumann) axis: the linear form ``inner(v, L(u))`` of an L of Helmholtz
    type, from its TPMatrix list (A = ASDSDmat / ASNSNmat of the second
    derivative, B = BSDSDmat / BSNSNmat)."""

    def __init__(self, mats, T):
        mats = [mats] if isinstance(mats, TPMatrix) else list(mats)
        keys = {m.get_key() for m in mats}
        self.neumann = keys <= {"ASNSNmat", "BSNSNmat"}
        if not (keys <= {"ASDSDmat", "BSDSDmat"} or self.neumann):
            raise NotImplementedError(f"linear operator with matrices {sorted(keys)}")
        ax = mats[0].axis
        shape = list(T.shape(True))
        shape[ax] = 1
        alfa = np.zeros(shape)
        beta = np.zeros(shape)
        for m in mats:
            if m.get_key() in ("ASDSDmat", "ASNSNmat"):
                alfa = alfa + m.scale
            else:
                beta = beta + m.scale
        self.alfa = torch.as_tensor(np.array(np.broadcast_to(alfa, shape), dtype=float), device="cuda")
        self.beta = torch.as_tensor(np.array(np.broadcast_to(beta, shape), dtype=float), device="cuda")
        self.axis = ax

    def __call__(self, v, c):
        """c = operator(v); rows past the basis dimension are zero."""
        c.zero_()
        outer, n, inner_ = view3(tuple(v.shape), self.axis)
        entry = "sgpu_Helmholtz_Neumann_matvec" if self.neumann else "sgpu_Helmholtz_matvec"
        _lib.call(entry, ptr(v), ptr(c), ptr(self.alfa), ptr(self.beta), outer, n, inner_,
                  data_kind(v), stream_handle())
        return c


def _nyquist_mask(T):
    """1 everywhere but the Nyquist coefficients of the even Fourier axes
    (tensorproductspace.py:1054-1080, fourier/bases.py:344-360, 545-550);
    None when there are none."""
    shape = T.shape(True)
    mask = None
    for i, b in enumerate(T.bases):
        if isinstance(b, (R2C, C2C)) and b.N % 2 == 0:
            m = np.ones(shape[i])
            m[b.N // 2 if isinstance(b, C2C) else -1] = 0
            s = [1] * len(shape)
            s[i] = shape[i]
            m = m.reshape(s)
            mask = m if mask is None else mask * m
    if mask is None:
        return None
    return torch.as_tensor(np.ascontiguousarray(mask), dtype=torch.float64, device="cuda")


class PDEIMEXRK:
    """u_t = N + L u by an IMEX Runge-Kutta scheme (integrators.py:702-817).

    Parameters mirror the reference: ``v`` the TestFunction, ``u`` the
    Function holding the solution (updated in place by ``solve_step``), ``L``
    a callable on an expression, ``N`` a Function or a callable
    ``N(u_hat, out)``, ``dt`` the time step, ``solver`` optional.
    """

    def __init__(self, v, u, L, N, dt, solver=None, name="U-equation", latex=None):
        self.v = v
        self.u_ = u
        self.L = L
        self.N = N
        self.dt = float(dt)
        self._solver = solver if solver is not None else SolverGeneric1ND
        self.solvers = []
        self.name = name
        self.latex = latex
        T = self.T = v.function_space()
        self.rhs = Function(T)
        self.Krhs = [Function(T) for _ in range(self.steps())]
        self.Lrhs = [Function(T) for _ in range(max(self.steps() - 1, 0))]
        self.u0_out = Function(T)
        self.mask = _nyquist_mask(T)
        self._graph = None

    @classmethod
    def steps(cls):
        raise NotImplementedError

    def stages(self):
        raise NotImplementedError

    def assemble(self):
        a = self.stages()[0]
        ul = TrialFunction(self.T)
        self.solvers.append(self._solver(inner(self.v, ul - self.dt * a[1, 1] * self.L(ul))))
        self.linear_rhs = _HelmholtzForm(inner(self.v, self.L(ul)), self.T)
        self.u0_rhs = _HelmholtzForm(inner(self.v, 1.0 * ul), self.T)
        if isinstance(self.N, torch.Tensor):
            f = self.N
            self.nonlinear_rhs = lambda out: self.u0_rhs(f.v if hasattr(f, "v") else f, out)
        elif callable(self.N):
            self.nonlinear_rhs = lambda out: self.N(self.u_, out)
        else:
            raise RuntimeError("Wrong type of nonlinear expression")
        # stage coefficients as Python floats, so that a step launches the same
        # kernels every time (and can be captured)
        a, b = self.stages()[:2]
        self._a = [[float(x) for x in row] for row in np.asarray(a)]
        self._b = [[float(x) for x in row] for row in np.asarray(b)]

    def compute_rhs(self, rk=0):
        """Assemble the right-hand side of stage rk (integrators.py:798-813)."""
        a, b, dt = self._a, self._b, self.dt
        rhs = self.rhs.v
        self.nonlinear_rhs(self.Krhs[rk].v)
        if rk == 0:
            self.u0_rhs(self.u_.v, self.u0_out.v)  # only at the start of a step
        rhs.copy_(self.u0_out.v)
        for j in range(rk + 1):
            rhs.add_(self.Krhs[j].v, alpha=dt * b[rk + 1][j])
        if rk > 0:
            self.linear_rhs(self.u_.v, self.Lrhs[rk - 1].v)
            for j in range(rk):
                rhs.add_(self.Lrhs[j].v, alpha=dt * a[rk + 1][j + 1])
        if self.mask is not None:
            rhs.mul_(self.mask)
        return self.rhs

    def solve_step(self, rk=0):
        # one solver: the diagonal of a is constant
        return self.solvers[0](self.rhs, self.u_)

    def step(self):
        """One time step: every stage's right-hand side and solve."""
        for rk in range(self.steps()):
            self.compute_rhs(rk)
            self.solve_step(rk)
        return self.u_

    # -- CUDA graph of a whole time step -------------------------------------
    def capture_step(self, warmup=2):
        """Record one time step in a CUDA graph (after `warmup` eager steps,
        which also advance the solution) and return it; ``replay`` then runs a
        step with a single launch.  The captured step reads and writes the
        same arrays as the eager one."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            for _ in range(warmup):
                self.step()
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step()
        self._graph = g
        return g

    def replay(self):
        if self._graph is None:
            raise RuntimeError("capture_step() first")
        self._graph.replay()
        return self.u_


class IMEXRK011(PDEIMEXRK):
    @classmethod
    def steps(cls):
        return 1

    def stages(self):
        a = np.array([[0, 0], [0, 0]])
        b = np.array([[0, 0], [1, 0]])
        return a, b, (1, 0)


class IMEXRK111(PDEIMEXRK):
    @classmethod
    def steps(cls):
        return 1

    def stages(self):
        a = np.array([[0, 0], [0, 1]])
        b = np.array([[0, 0], [1, 0]])
        return a, b, (0, 1)


class IMEXRK222(PDEIMEXRK):
    @classmethod
    def steps(cls):
        return 2

    def stages(self):
        gamma = (2 - np.sqrt(2)) / 2
        delta = 1 - 1 / (2 * gamma)
        a = np.array([[0, 0, 0], [0, gamma, 0], [0, 1 - gamma, gamma]])
        b = np.array([[0, 0, 0], [gamma, 0, 0], [delta, 1 - delta, 0]])
        return a, b, (0, gamma, 1)


class IMEXRK443(PDEIMEXRK):
    @classmethod
    def steps(cls):
        return 4

    def stages(self):
        a = np.array([[0, 0, 0, 0, 0],
                      [0, 1 / 2, 0, 0, 0],
                      [0, 1 / 6, 1 / 2, 0, 0],
                      [0, -1 / 2, 1 / 2, 1 / 2, 0],
                      [0, 3 / 2, -3 / 2, 1 / 2, 1 / 2]])
        b = np.array([[0, 0, 0, 0, 0],
                      [1 / 2, 0, 0, 0, 0],
                      [11 / 18, 1 / 18, 0, 0, 0],
                      [5 / 6, -5 / 6, 1 / 2, 0, 0],
                      [1 / 4, 7 / 4, 3 / 4, -7 / 4, 0]])
        return a, b, (0, 1 / 2, 2 / 3, 1 / 2, 1)
