"""Forms API on the GPU path: Array/Function, Test/TrialFunction, div/grad/Dx,
inner and project (forms/arguments.py, forms/inner.py, forms/project.py).

Only what the hot path needs is provided: linear forms ``inner(v, Array)``
(the scalar product transform) and ``inner(v, expr)`` with ``expr`` a
constant-coefficient combination of derivatives of a Function, bilinear forms
built from constant multiples of derivatives of the trial function, which
assemble into ``TPMatrix`` objects with per-wavenumber scale arrays (the
reference's ``get_simplified_tpmatrices`` result, matrixbase.py:1648-1678),
and ``project`` of Arrays, Functions and such expressions.
"""
import numbers

import numpy as np
import torch

from . import _lib
from .spaces import TensorProductSpace, FourierBase, SpectralBase
from . import matrices as M


# ---------------------------------------------------------------------------
class _ShenfunArray(torch.Tensor):
    """torch.Tensor subclass bound to a function space (DistArray analogue)."""

    _space = None

    @staticmethod
    def _new(cls, space, data):
        obj = torch.Tensor._make_subclass(cls, data, False)
        obj._space = space
        return obj

    def function_space(self):
        return self._space

    @property
    def v(self):
        return self.as_subclass(torch.Tensor)

    def __array__(self, dtype=None):
        a = self.detach().cpu().as_subclass(torch.Tensor).numpy()
        return a.astype(dtype) if dtype is not None else a

    @classmethod
    def __torch_function__(cls, func, types, args=(), kwargs=None):
        # results of torch ops are plain tensors (no space attached)
        kwargs = kwargs or {}
        with torch._C.DisableTorchFunctionSubclass():
            return func(*args, **kwargs)


def _fill(space, forward_output, val, buffer):
    shape = space.shape(forward_output)
    dt = space.torch_dtype(forward_output) if isinstance(space, TensorProductSpace) else \
        (torch.complex128 if (forward_output and isinstance(space, FourierBase)) else torch.float64)
    t = torch.empty(shape, dtype=dt, device="cuda")
    if buffer is None:
        t.fill_(val)
        return t, None
    if hasattr(buffer, "free_symbols"):
        return t, buffer  # sympy expression: evaluate on the mesh
    src = torch.as_tensor(np.asarray(buffer)) if not isinstance(buffer, torch.Tensor) else buffer
    t.copy_(src.to(device="cuda", dtype=dt).reshape(shape))
    return t, None


def _eval_sympy(space, expr):
    import sympy as sp
    syms = sorted(expr.free_symbols, key=lambda s: "xyzrs".index(str(s)))
    mesh = space.mesh() if isinstance(space, TensorProductSpace) else [space.mesh()]
    args = [mesh["xyzrs".index(str(s))] for s in syms]
    vals = sp.lambdify(syms, expr, "numpy")(*args)
    return np.broadcast_to(vals, space.shape(False)).astype(float)


class Array(_ShenfunArray):
    """Physical-space values on the quadrature mesh (forms/arguments.py:1891)."""

    def __new__(cls, space, val=0, buffer=None):
        t, sym = _fill(space, False, val, buffer)
        if sym is not None:
            t.copy_(torch.as_tensor(_eval_sympy(space, sym), device="cuda"))
        return _ShenfunArray._new(cls, space, t)

    def forward(self, output_array=None, kind=None):
        if output_array is None:
            output_array = Function(self._space)
        self._space.forward(self.v, output_array.v if isinstance(output_array, _ShenfunArray) else output_array)
        return output_array


class Function(_ShenfunArray):
    """Spectral expansion coefficients (forms/arguments.py:1427)."""

    def __new__(cls, space, val=0, buffer=None):
        t, sym = _fill(space, True, val, buffer)
        obj = _ShenfunArray._new(cls, space, t)
        if sym is not None:
            a = Array(space, buffer=sym)
            a.forward(obj)
        return obj

    def set_boundary_dofs(self):
        """Boundary dofs of a non-homogeneous Chebyshev axis set to their
        final values (BoundaryValues.set_boundary_dofs(u, final=True),
        tensorproductspace.py:2108-2128)."""
        T = self._space
        bases = T.bases if isinstance(T, TensorProductSpace) else (T,)
        for ax, b in enumerate(bases):
            if getattr(b, "has_nonhomogeneous_bcs", False):
                b._apply_bcs(self.v, ax, lift=False)
        return self

    def backward(self, output_array=None, kind=None, mesh=None):
        if output_array is None:
            output_array = Array(self._space)
        self._space.backward(self.v, output_array.v if isinstance(output_array, _ShenfunArray) else output_array)
        return output_array


# ---------------------------------------------------------------------------
class Expr:
    """Linear combination of derivatives of a basis function:
    terms = [(coefficient, derivative order per axis)]."""

    def __init__(self, basis, terms):
        self.basis = basis
        self.terms = list(terms)

    def function_space(self):
        return self.basis.function_space()

    def __add__(self, other):
        other = _as_expr(other)
        a, b = getattr(self.basis, "function", None), getattr(other.basis, "function", None)
        if (a is None) != (b is None) or (a is not None and a.data_ptr() != b.data_ptr()):
            raise NotImplementedError("a sum of expressions of different arguments")
        assert other.basis is self.basis or other.basis.space is self.basis.space
        return Expr(self.basis, self.terms + other.terms)

    def __sub__(self, other):
        return self + (-_as_expr(other))

    def __neg__(self):
        return Expr(self.basis, [(-c, d) for c, d in self.terms])

    def __mul__(self, a):
        if not isinstance(a, numbers.Number):
            return NotImplemented
        return Expr(self.basis, [(a * c, d) for c, d in self.terms])

    __rmul__ = __mul__


class BasisFunction(Expr):
    def __init__(self, space, argument):
        self.space = space
        self.argument = argument
        nd = space.dimensions if isinstance(space, TensorProductSpace) else 1
        Expr.__init__(self, self, [(1.0, (0,) * nd)])

    def function_space(self):
        return self.space


def TestFunction(space):
    return BasisFunction(space, 0)


def TrialFunction(space):
    return BasisFunction(space, 1)


class FunctionBasis(BasisFunction):
    """A Function in a form: argument 2, the expansion it holds
    (forms/arguments.py:1204-1230, Function as a BasisFunction)."""

    def __init__(self, function):
        self.function = function
        BasisFunction.__init__(self, function.function_space(), 2)


def _as_expr(e):
    if isinstance(e, Expr):
        return e
    if isinstance(e, Function):
        return FunctionBasis(e)
    raise TypeError(f"cannot use {type(e)} in a form")


def Dx(e, axis=0, k=1):
    e = _as_expr(e)
    out = []
    for c, d in e.terms:
        d = list(d)
        d[axis] += k
        out.append((c, tuple(d)))
    return Expr(e.basis, out)


class _Grad:
    def __init__(self, e):
        self.e = _as_expr(e)


def grad(e):
    return _Grad(e)


def div(g):
    if not isinstance(g, _Grad):
        raise NotImplementedError("div of a general vector expression")
    e = g.e
    nd = len(e.terms[0][1])
    out = None
    for ax in range(nd):
        t = Dx(e, ax, 2)
        out = t if out is None else out + t
    return out


# ---------------------------------------------------------------------------
class TPMatrix:
    """scale * (identity on the Fourier axes) x pmat on the non-periodic axis.

    ``scale`` has the spectral shape with the non-periodic axis collapsed to
    one; it carries the Fourier factors (i k)^d of every term that shares
    ``pmat`` (TPMatrix / get_simplified_tpmatrices, matrixbase.py:1275-1678).
    """

    def __init__(self, pmat, scale, space, axis):
        self.pmat = pmat
        self.scale = scale
        self.space = space
        self.axis = axis
        self.mats = pmat

    def get_key(self):
        return self.pmat.key

    @property
    def tensorproductspace(self):
        return self.space

    def __repr__(self):
        return f"TPMatrix({self.pmat.key}, axis={self.axis})"


def _bilinear(test, expr):
    T = test.function_space()
    if isinstance(T, SpectralBase):
        # 1D: plain SpectralMatrix list
        out = {}
        for c, d in expr.terms:
            m = M.galerkin_matrix(T, d[0])
            key = d[0]
            if key in out:
                out[key][1] += c
            else:
                out[key] = [m, c]
        res = []
        for m, c in out.values():
            m.scale = c
            res.append(m)
        return res[0] if len(res) == 1 else res
    np_axes = T.get_nonperiodic_axes()
    if len(np_axes) != 1:
        raise NotImplementedError("exactly one non-periodic axis is on the GPU path")
    ax = np_axes[0]
    shape = list(T.shape(True))
    shape[ax] = 1
    ks = []
    for i, b in enumerate(T.bases):
        if isinstance(b, FourierBase):
            k = np.asarray(b.wavenumbers(scaled=True), dtype=float)
            s = [1] * len(shape)
            s[i] = len(k)
            ks.append((i, k.reshape(s)))
    groups = {}
    for c, d in expr.terms:
        sc = np.full(shape, c, dtype=complex)
        for i, k in ks:
            if d[i]:
                sc = sc * (1j * k) ** d[i]
        key = d[ax]
        groups[key] = groups.get(key, 0) + sc
    out = []
    base = T.bases[ax]
    for order, sc in sorted(groups.items(), key=lambda kv: -kv[0]):
        if np.abs(sc.imag).max() > 0:
            raise NotImplementedError("odd derivatives along Fourier axes")
        out.append(TPMatrix(M.galerkin_matrix(base, order), np.ascontiguousarray(sc.real), T, ax))
    return out[0] if len(out) == 1 else out


def _expr_apply(T, expr, solve, output_array=None):
    """The linear form (phi_k, expr)_w of an expression of one Function uh
    (forms/inner.py:483-497, the matvecs of the assembled matrices) or, with
    ``solve``, its projection u = B^{-1} (phi_k, expr)_w (forms/project.py:
    124-199), on the GPU: one line GEMM (sgpu_line_gemm, per-line scales,
    accumulating) per derivative order along the line axis, with the host
    operators of operators.expr_plan."""
    from .device import ptr, stream_handle, view3, require_cuda
    from .operators import expr_plan
    require_cuda()
    fb = expr.basis
    src = fb.function.v
    ax, out_shape, cplx, terms = expr_plan(T, fb.space, expr.terms, solve, src.is_complex())
    dt = torch.complex128 if cplx else torch.float64
    if src.dtype != dt:
        src = src.to(dt)
    src = src.contiguous()
    if output_array is None:
        output_array = Function(T)
    out = torch.zeros(out_shape, dtype=dt, device=src.device)
    o_in, n_in, i_in = view3(tuple(src.shape), ax)
    o_out, n_out, i_out = view3(tuple(out.shape), ax)
    if (o_in, i_in) != (o_out, i_out):
        raise _lib.SgpuError(_lib.ERR_ARG, "the Function does not match the space off the line axis")
    for Mat, scale in terms:
        Md = torch.as_tensor(np.ascontiguousarray(Mat), device=src.device)
        sd = torch.as_tensor(scale, device=src.device)
        # Md, sd live on the current stream: the caching allocator reuses their
        # memory only after this launch in stream order
        _lib.call("sgpu_line_gemm", ptr(src), ptr(out), ptr(Md), n_in, n_out, o_in, i_in,
                  _lib.COMPLEX if cplx else _lib.REAL, ptr(sd), 1, stream_handle())
    dst = output_array.v if isinstance(output_array, _ShenfunArray) else output_array
    dst.copy_(out if dst.is_complex() else out.real)
    return output_array


def inner(test, trial, output_array=None, kind=None):
    """Scalar product (linear form) or matrix assembly (bilinear form)
    (forms/inner.py:16-511)."""
    if isinstance(test, BasisFunction) and isinstance(trial, (Function, FunctionBasis)) or (
            isinstance(test, BasisFunction) and isinstance(trial, Expr) and
            getattr(trial.basis, "argument", 1) == 2):
        return _expr_apply(test.function_space(), _as_expr(trial), False, output_array)
    if isinstance(test, BasisFunction) and isinstance(trial, torch.Tensor):
        T = test.function_space()
        if output_array is None:
            output_array = Function(T)
        out = output_array.v if isinstance(output_array, _ShenfunArray) else output_array
        inp = trial.v if isinstance(trial, _ShenfunArray) else trial
        T.scalar_product(inp, out)
        return output_array
    if isinstance(test, BasisFunction) and isinstance(trial, (Expr, BasisFunction)):
        return _bilinear(test, trial)
    if isinstance(trial, BasisFunction) and isinstance(test, (Expr,)):
        return _bilinear(trial, test)
    raise NotImplementedError("inner of these arguments")


def project(uh, T, output_array=None):
    """Projection on T (forms/project.py:16-199): an Array on T's mesh is
    forward transformed (:117-122); a Function or an expression of one
    (derivatives with constant coefficients) is projected with the mass
    solve, u = B^{-1} (v, uh) (:124-199), on the GPU."""
    if isinstance(uh, (Function, Expr)):
        expr = _as_expr(uh)
        if getattr(expr.basis, "argument", None) != 2:
            raise ValueError("project takes an Array, a Function or an expression of a Function")
        return _expr_apply(T, expr, True, output_array)
    if output_array is None:
        output_array = Function(T)
    src = uh.v if isinstance(uh, _ShenfunArray) else uh
    T.forward(src, output_array.v if isinstance(output_array, _ShenfunArray) else output_array)
    return output_array
