"""Linear-algebra solvers on the GPU (la.py and chebyshev/la.py of the
reference): TDMA, PDMA, SolverGeneric1ND and the Chebyshev Helmholtz solver.

Factorisations happen once at construction (on the device) and are reused by
every call, like the reference's ``perform_lu`` / ``LU_Helmholtz``.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .device import ptr, stream_handle, view3, data_kind, require_cuda
from .forms import Function, TPMatrix, _ShenfunArray
from .matrices import SpectralMatrix


def _raw(t):
    return t.v if isinstance(t, _ShenfunArray) else t


def _band_data(mat, offsets):
    """Pack a banded SpectralMatrix into the reference's (len(offsets), n)
    data layout: row r holds offset offsets[r] starting at column max(0, off)."""
    n = mat.shape[0]
    data = np.zeros((len(offsets), n))
    for r, off in enumerate(offsets):
        d = mat.get(off, 0.0)
        d = np.broadcast_to(np.atleast_1d(np.asarray(d, dtype=float)), (n - abs(off),))
        if not np.isscalar(mat.scale) and np.asarray(mat.scale).size != 1:
            # per-row scales belong to a TPMatrix's solver, not to one band
            raise _lib.SgpuError(_lib.ERR_ARG, "banded solver: the matrix scale must be a scalar")
        s = float(np.asarray(mat.scale).reshape(-1)[0]) if not np.isscalar(mat.scale) else mat.scale
        if off >= 0:
            data[r, off:] = d * s
        else:
            data[r, :n + off] = d * s
    return data


def _as_list(mats):
    """A form's matrices: inner() returns one matrix for a one-term form and a
    list otherwise (forms/inner.py:497-499)."""
    if isinstance(mats, (TPMatrix, SpectralMatrix)):
        return [mats]
    return list(mats)


def _constraint_rows(b, axis, constraints):
    """b[T.si[row]] = val for every constraint (la.py:124-129)."""
    for row, val in constraints:
        b.select(axis, int(row)).fill_(val)


class _Constrained:
    """Solvers factorise at construction; a call with constraints refactors
    once from the matrix with those rows made identity rows
    (SparseMatrixSolver.apply_constraints, la.py:77-130)."""

    _cons = ()

    def _check_constraints(self, constraints):
        cons = tuple((int(r), v) for r, v in constraints)
        if cons and tuple(r for r, _ in cons) != tuple(r for r, _ in self._cons):
            from .matrices import constrained
            self._factor(constrained(self.mat, cons))
            self._cons = cons
        return cons


class _BandedSolver(_Constrained):
    offsets = None
    lu_entry = None
    solve_entry = None

    def __init__(self, mat):
        require_cuda()
        if isinstance(mat, list):
            mat = mat[0] if len(mat) == 1 else _sum_mats(mat)
        self.mat = mat
        self.n = mat.shape[0]
        self._factor(mat)

    def _factor(self, mat):
        data = _band_data(mat, self.offsets)
        self._lu = torch.as_tensor(data, device="cuda").contiguous()
        _lib.call(self.lu_entry, ptr(self._lu), self.n, stream_handle())

    def __call__(self, b, u=None, axis=0, constraints=()):
        b = _raw(b)
        _constraint_rows(b, axis, self._check_constraints(constraints))
        if u is None:
            u = b
        else:
            u = _raw(u)
            if u.data_ptr() != b.data_ptr():
                u.copy_(b)
        shape = tuple(u.shape)
        outer, n, inner = view3(shape, axis)
        if n < self.n:
            raise _lib.SgpuError(_lib.ERR_ARG, "array shorter than the matrix along axis")
        if n == self.n:
            _lib.call(self.solve_entry, ptr(u), ptr(self._lu), outer, n, inner, data_kind(u),
                      stream_handle())
        else:
            # the first n entries along axis are the dofs (the rest are boundary dofs)
            sub = u.narrow(axis, 0, self.n).contiguous()
            _lib.call(self.solve_entry, ptr(sub), ptr(self._lu), outer, self.n, inner,
                      data_kind(sub), stream_handle())
            u.narrow(axis, 0, self.n).copy_(sub)
        return u


class TDMA(_BandedSolver):
    """Offsets (-2, 0, 2) (la.py:331-393; kernels la.pyx:77, 243, 516)."""

    offsets = (-2, 0, 2)
    lu_entry = "sgpu_TDMA_LU"
    solve_entry = "sgpu_TDMA_Solve"


class PDMA(_BandedSolver):
    """Offsets (-4, -2, 0, 2, 4) (la.py:450-543; kernels la.pyx:61, 213, 496)."""

    offsets = (-4, -2, 0, 2, 4)
    lu_entry = "sgpu_PDMA_LU"
    solve_entry = "sgpu_PDMA_Solve"


class _GeneralBanded(_Constrained):
    """Banded solver for the reference's other band patterns (la.py:291-800):
    LU once on the device (sgpu_banded_LU), solve per call (sgpu_banded_Solve)
    along any axis, in place; the dofs are the first n entries along it."""

    offsets = None

    def __init__(self, mat):
        require_cuda()
        if isinstance(mat, list):
            mat = mat[0] if len(mat) == 1 else _sum_mats(mat)
        self.mat = mat
        self.n = mat.shape[0]
        self._factor(mat)

    def _factor(self, mat):
        data = self._prepare(_band_data(mat, self.offsets))
        self._lu = torch.as_tensor(data, device="cuda").contiguous()
        self._off = (ctypes.c_int * len(self.offsets))(*self.offsets)
        _lib.call("sgpu_banded_LU", ptr(self._lu), len(self.offsets), self._off, self.n, stream_handle())

    @staticmethod
    def _prepare(data):
        return data

    def __call__(self, b, u=None, axis=0, constraints=()):
        b = _raw(b)
        _constraint_rows(b, axis, self._check_constraints(constraints))
        if u is None:
            u = b
        else:
            u = _raw(u)
            if u.data_ptr() != b.data_ptr():
                u.copy_(b)
        outer, n, inner = view3(tuple(u.shape), axis)
        if n != self.n:
            sub = u.narrow(axis, 0, self.n).contiguous()
            o2, _, i2 = view3(tuple(sub.shape), axis)
            _lib.call("sgpu_banded_Solve", ptr(sub), ptr(self._lu), len(self.offsets), self._off, o2, self.n,
                      i2, data_kind(sub), stream_handle())
            u.narrow(axis, 0, self.n).copy_(sub)
            return u
        _lib.call("sgpu_banded_Solve", ptr(u), ptr(self._lu), len(self.offsets), self._off, outer, n, inner,
                  data_kind(u), stream_handle())
        return u


class DiagMA(_GeneralBanded):
    """Diagonal (la.py:291-328)."""
    offsets = (0,)


class TwoDMA(_GeneralBanded):
    """Offsets 0, 2 (la.py:615-659)."""
    offsets = (0, 2)


class ThreeDMA(_GeneralBanded):
    """Offsets 0, 2, 4 (la.py:661-709).  The reference's solve reads the
    offset-4 coefficient of row i from the offset-2 diagonal's storage
    (u2 = data[1, 4:], la.py:686-689 and la.pyx:569-580), i.e. it solves the
    matrix whose offset-4 entries are M[i + 2][i + 4]; kept for parity."""
    offsets = (0, 2, 4)

    @staticmethod
    def _prepare(data):
        data = data.copy()
        data[2, 4:] = data[1, 4:]
        return data


class FDMA(_GeneralBanded):
    """Offsets -2, 0, 2, 4 (la.py:545-613)."""
    offsets = (-2, 0, 2, 4)


class HeptaDMA(_GeneralBanded):
    """Offsets -4, -2, 0, 2, 4, 6, 8 (la.py:711-800)."""
    offsets = (-4, -2, 0, 2, 4, 6, 8)


class TDMA_O(_GeneralBanded):
    """Symmetric tridiagonal with offsets -1, 0, 1 (la.py:396-447)."""
    offsets = (-1, 0, 1)


class Solve(_Constrained):
    """Generic solver for a matrix without a tailored band pattern
    (la.py:823-840).  The reference factorises with scipy's splu and solves
    on the host; here the (constrained) matrix is inverted once on the host in
    FP64 and every solve applies the inverse along the axis with the FP64 line
    GEMM on the GPU (sgpu_line_gemm); the dofs are the first n entries."""

    def __init__(self, mats, format=None):
        require_cuda()
        if isinstance(mats, list):
            mats = mats[0] if len(mats) == 1 else _sum_mats(mats)
        self.mat = mats
        self.n = mats.shape[0]
        self._factor(mats)

    def _factor(self, mat):
        sc = np.asarray(mat.scale, dtype=float)
        if sc.size != 1:
            raise _lib.SgpuError(_lib.ERR_ARG, "Solve: the matrix scale must be a scalar")
        dense = mat.todense() * float(sc.reshape(-1)[0])
        inv = np.linalg.inv(dense)
        # sgpu_line_gemm computes out(l, k) = sum_j in(l, j) M[j][k]
        self._M = torch.as_tensor(np.ascontiguousarray(inv.T), device="cuda")

    def __call__(self, b, u=None, axis=0, constraints=()):
        b = _raw(b)
        _constraint_rows(b, axis, self._check_constraints(constraints))
        ur = b if u is None else _raw(u)
        outer, N, inner = view3(tuple(b.shape), axis)
        if N < self.n:
            raise _lib.SgpuError(_lib.ERR_ARG, "array shorter than the matrix along axis")
        src = b.narrow(axis, 0, self.n).contiguous()
        if src.data_ptr() == b.data_ptr() and ur.data_ptr() == b.data_ptr():
            src = src.clone()
        dst = torch.empty_like(src)
        o2, _, i2 = view3(tuple(src.shape), axis)
        _lib.call("sgpu_line_gemm", ptr(src), ptr(dst), ptr(self._M), self.n, self.n, o2, i2, data_kind(src),
                  None, 0, stream_handle())
        ur.narrow(axis, 0, self.n).copy_(dst)
        return b if u is None else u


def _sum_mats(mats):
    d = {}
    for m in mats:
        s = m.scale if np.isscalar(m.scale) else 1.0
        for off, v in m.items():
            d[off] = d.get(off, 0.0) + s * np.asarray(v, dtype=float)
    out = SpectralMatrix(mats[0].key, d, mats[0].shape)
    return out


# ---------------------------------------------------------------------------
class Helmholtz:
    """Chebyshev Dirichlet / Neumann Helmholtz solver (chebyshev/la.py:131-351):
    (alfa A + beta B) u = b along one axis, one system per Fourier wavenumber.
    A, B are ASDSD, BSDSD (ShenDirichlet) or ASNSN, BSNSN (ShenNeumann: the
    Neumann branch, la.pyx:735-751, 907-912).

    Accepts the two TPMatrix objects of ``inner(v, -div(grad(u)) + c*u)`` (or
    ``(A, B, alfa, beta)`` with SpectralMatrix A, B and scalars/arrays).

    ``form``: "plain" (FP64 factor cache and sweeps), "mixed" (double-float),
    or "refined" (Dirichlet only): FP32 factor cache (half the bytes) and
    FP32 sweeps refined by an FP64-level residual until the correction is
    below ``tol`` of the solution (at most ``max_it`` corrections); the
    residual runs in FP64 (``residual="fp64"``) or double-float on the FP32
    pipes (``residual="df"``).  ``last_iterations`` then holds each
    (system, parity) chain's correction count.
    """

    def __init__(self, *args, form=None, tol=1e-13, max_it=8, residual="fp64"):
        require_cuda()
        if len(args) == 1:
            args = tuple(args[0])
        keys = {a.get_key() for a in args[:2]}
        self.neumann = bool(keys & {"ASNSNmat", "BSNSNmat"})
        akey, bkey = ("ASNSNmat", "BSNSNmat") if self.neumann else ("ASDSDmat", "BSDSDmat")
        if len(args) == 2 and all(isinstance(a, TPMatrix) for a in args):
            by = {a.get_key(): a for a in args}
            A, B = by[akey], by[bkey]
            self.T = A.space
            self.axis = A.axis
            alfa, beta = A.scale, B.scale
            self.N = self.T.bases[self.axis].N
        elif len(args) == 4:
            A, B, alfa, beta = args
            self.T = None
            self.axis = 0
            self.N = A.shape[0] + 2
            alfa = np.atleast_1d(np.asarray(alfa, dtype=float))
            beta = np.atleast_1d(np.asarray(beta, dtype=float))
        else:
            raise ValueError("Helmholtz(A_tp, B_tp) or Helmholtz(A, B, alfa, beta)")
        alfa = np.asarray(alfa, dtype=float)
        beta = np.asarray(beta, dtype=float)
        shape = np.broadcast_shapes(alfa.shape, beta.shape)
        self.alfa = torch.as_tensor(np.array(np.broadcast_to(alfa, shape)), device="cuda")
        self.beta = torch.as_tensor(np.array(np.broadcast_to(beta, shape)), device="cuda")
        self._scale_shape = shape
        fshape = list(shape) if len(shape) else [1]
        if self.T is not None:
            fshape[self.axis] = self.N
        else:
            fshape = [self.N] + list(shape[1:]) if len(shape) > 1 else [self.N]
        self.u0 = torch.zeros(fshape, dtype=torch.float64, device="cuda")
        self.u1 = torch.zeros_like(self.u0)
        self.u2 = torch.zeros_like(self.u0)
        self.L = torch.zeros_like(self.u0)
        outer, _, inner = view3(tuple(fshape), self.axis)
        if outer * inner != self.alfa.numel():
            raise _lib.SgpuError(_lib.ERR_ARG, "scale arrays do not match the systems")
        self._outer, self._inner = outer, inner
        _lib.call("sgpu_LU_Helmholtz", self.N, ptr(self.alfa), ptr(self.beta), int(self.neumann),
                  ptr(self.u0), ptr(self.u1), ptr(self.u2), ptr(self.L), outer, inner, stream_handle())
        # factorisation cache used by __call__: reciprocal pivots, interleaved
        # [q][k][system] layout, FP64 (plain), double-float pairs (mixed) or
        # FP32 (refined)
        self.refined = form == "refined"
        if self.refined and self.neumann:
            raise _lib.SgpuError(_lib.ERR_UNSUPPORTED, "refined solves: Dirichlet systems only")
        self.tol, self.max_it = float(tol), int(max_it)
        self.residual_form = {"fp64": _lib.PLAIN_F64, "df": _lib.MIXED_DF}[residual]
        self.form = _lib.FP32_REFINED if self.refined else (_lib.FORMS[form] if form is not None else (
            self.T.form if self.T is not None else _lib.PLAIN_F64))
        self.last_iterations = None
        self._r = None
        nsys = outer * inner
        # boundary matrices of a non-homogeneous trial space (extract_bc_matrices,
        # chebyshev/la.py:222-231): subtracted from the right-hand side
        base = self.T.bases[self.axis] if self.T is not None else None
        self._bcbase = base if getattr(base, "has_nonhomogeneous_bcs", False) else None
        self._fac = torch.empty(4 * (self.N - 2) * nsys, dtype=torch.float32 if self.refined else torch.float64,
                                device="cuda")
        _lib.call("sgpu_helmholtz_factor", self.N, ptr(self.alfa), ptr(self.beta), int(self.neumann),
                  outer, inner, self.form, self._fac.data_ptr(), stream_handle())

    def __call__(self, b, u=None, constraints=()):
        b = _raw(b)
        if u is None:
            u = torch.zeros_like(b)
        ur = _raw(u)
        outer, n, inner = view3(tuple(b.shape), self.axis)
        if n != self.N or (outer, inner) != (self._outer, self._inner):
            raise _lib.SgpuError(_lib.ERR_ARG, "array shape does not match the solver")
        bb = self._bcbase
        if bb is not None:
            # u.set_boundary_dofs(); b -= bc_mat.matvec(u) (chebyshev/la.py:302-306)
            g = bb.bc_lines(tuple(b.shape), self.axis, [a for a in range(b.dim()) if a != self.axis],
                            b.dtype)
            _lib.call("sgpu_bc_apply", ptr(b), ptr(bb._bc_table("A")), ptr(self.alfa),
                      ptr(bb._bc_table("B")), ptr(self.beta), ptr(g), outer, n, inner, 0,
                      data_kind(b), stream_handle())
        if self.refined:
            self._solve_refined(b, ur, outer, n, inner)
        else:
            _lib.call("sgpu_helmholtz_solve_cached", ptr(b), ptr(ur), ptr(self._fac), int(self.neumann),
                      outer, n, inner, data_kind(b), self.form, stream_handle())
        if bb is not None:
            _lib.call("sgpu_bc_apply", ptr(ur), None, None, None, None, ptr(g), outer, n, inner, 1,
                      data_kind(ur), stream_handle())
        if constraints:
            idx = [0] * ur.dim()
            ur[tuple(idx)] = constraints[0][1]
        return u

    def _solve_refined(self, b, ur, outer, n, inner):
        if self._r is None or self._r.shape != b.shape or self._r.dtype != b.dtype:
            self._r = torch.empty_like(b)
            self.last_iterations = torch.zeros(2 * outer * inner, dtype=torch.int32, device="cuda")
        src = b
        if b.data_ptr() == ur.data_ptr():  # the refinement re-reads b: keep it
            src = b.clone()
        _lib.call("sgpu_helmholtz_solve_refined", ptr(src), ptr(ur), ptr(self._r), self._fac.data_ptr(),
                  ptr(self.alfa), ptr(self.beta), outer, n, inner, data_kind(b), self.tol, self.max_it,
                  self.residual_form, self.last_iterations.data_ptr(), stream_handle())

    def solve_reference_layout(self, b, u):
        """Solve through the reference-layout factors u0, u1, u2, L
        (Solve_Helmholtz, la.pyx:845) instead of the cache."""
        b, ur = _raw(b), _raw(u)
        outer, n, inner = view3(tuple(b.shape), self.axis)
        _lib.call("sgpu_Solve_Helmholtz", ptr(b), ptr(ur), int(self.neumann), ptr(self.u0),
                  ptr(self.u1), ptr(self.u2), ptr(self.L), outer, n, inner, data_kind(b),
                  stream_handle())
        return u

    def matvec(self, v, c):
        v, cr = _raw(v), _raw(c)
        outer, n, inner = view3(tuple(v.shape), self.axis)
        entry = "sgpu_Helmholtz_Neumann_matvec" if self.neumann else "sgpu_Helmholtz_matvec"
        _lib.call(entry, ptr(v), ptr(cr), ptr(self.alfa), ptr(self.beta), outer, n, inner,
                  data_kind(v), stream_handle())
        return c


class SolverGeneric1ND:
    """One non-periodic axis, one banded system per Fourier wavenumber
    (la.py:1183-1434).  Dispatches on the basis of the non-periodic axis:
    Chebyshev ShenDirichlet / ShenNeumann -> the Helmholtz kernels (the
    reference falls back to a sparse LU per wavenumber there,
    la.py:1299-1364)."""

    def __init__(self, mats):
        mats = _as_list(mats)
        T = mats[0].space
        ax = mats[0].axis
        base = T.bases[ax]
        keys = {m.get_key() for m in mats}
        self.T, self.axis = T, ax
        sn = base.short_name()
        if base.family() == "chebyshev" and sn in ("SD", "SN") and keys <= {f"A{sn}{sn}mat", f"B{sn}{sn}mat"}:
            by = {m.get_key(): m for m in mats}
            shape = list(T.shape(True))
            shape[ax] = 1
            A = by.get(f"A{sn}{sn}mat")
            B = by.get(f"B{sn}{sn}mat")
            alfa = A.scale if A is not None else np.zeros(shape)
            beta = B.scale if B is not None else np.zeros(shape)
            self._impl = Helmholtz(_tp(f"A{sn}{sn}mat", alfa, T, ax), _tp(f"B{sn}{sn}mat", beta, T, ax))
        else:
            self._impl = BandSepSolver(mats)

    def __call__(self, b, u=None, constraints=()):
        return self._impl(b, u, constraints)


class BandSepSolver:
    """Per-wavenumber systems sum_t scale_t M_t with banded + rank-2 upper
    semiseparable M_t, factorised once on the device (sgpu_band_sep_factor)
    and solved per call (sgpu_band_sep_solve).  Used for Legendre
    ShenDirichlet / ShenBiharmonic and Chebyshev ShenBiharmonic.

    ``form="refined"``: an FP32 factor cache and FP32 sweeps refined by the
    FP64 residual of the matvec below, as Helmholtz(form="refined")."""

    def __init__(self, mats, form="plain", tol=1e-13, max_it=8):
        from .matrices import band_sep_term
        require_cuda()
        mats = sorted(_as_list(mats), key=lambda m: -m.pmat.order)
        T, ax = mats[0].space, mats[0].axis
        base = T.bases[ax]
        self.T, self.axis, self.N = T, ax, base.N
        terms = [band_sep_term(base, m.pmat.order) for m in mats]
        self.n = terms[0][0].shape[1]
        self.gen_term = next((i for i, (_, g) in enumerate(terms) if g is not None), -1)
        if sum(g is not None for _, g in terms) > 1:
            raise NotImplementedError("more than one semiseparable term")
        bands = np.ascontiguousarray(np.stack([b for b, _ in terms]))
        shape = list(T.shape(True))
        shape[ax] = 1
        coefs = np.stack([np.broadcast_to(np.asarray(m.scale, dtype=float), shape).reshape(-1)
                          for m in mats])
        self.nsys = coefs.shape[1]
        self._outer, _, self._inner = view3(tuple(T.shape(True)), ax)
        self._bands = torch.as_tensor(bands, device="cuda")
        self._coef = torch.as_tensor(np.ascontiguousarray(coefs), device="cuda")
        self._gens = (torch.as_tensor(np.ascontiguousarray(terms[self.gen_term][1]), device="cuda")
                      if self.gen_term >= 0 else None)
        m = (self.n + 1) // 2
        self.refined = form == "refined"
        self.tol, self.max_it = float(tol), int(max_it)
        self.last_iterations = None
        self._r = None
        self._fac = torch.empty(7 * m * 2 * self.nsys, dtype=torch.float32 if self.refined else torch.float64,
                                device="cuda")
        _lib.call("sgpu_band_sep_factor32" if self.refined else "sgpu_band_sep_factor", self.n, len(mats),
                  self.gen_term, ptr(self._bands), ptr(self._gens) if self._gens is not None else None,
                  ptr(self._coef), self.nsys, self._fac.data_ptr(), stream_handle())

    def __call__(self, b, u=None, constraints=()):
        b = _raw(b)
        if u is None:
            u = torch.zeros_like(b)
        ur = _raw(u)
        outer, Nb, inner = view3(tuple(b.shape), self.axis)
        if (outer, inner) != (self._outer, self._inner) or Nb != self.N:
            raise _lib.SgpuError(_lib.ERR_ARG, "array shape does not match the solver")
        if self.refined:
            if self._r is None or self._r.shape != b.shape or self._r.dtype != b.dtype:
                self._r = torch.empty_like(b)
                self.last_iterations = torch.zeros(2 * self.nsys, dtype=torch.int32, device="cuda")
            src = b.clone() if b.data_ptr() == ur.data_ptr() else b
            _lib.call("sgpu_band_sep_solve_refined", ptr(src), ptr(ur), ptr(self._r), self._fac.data_ptr(),
                      self.n, self._coef.shape[0], self.gen_term, ptr(self._bands),
                      ptr(self._gens) if self._gens is not None else None, ptr(self._coef), outer, Nb, inner,
                      data_kind(b), self.tol, self.max_it, self.last_iterations.data_ptr(), stream_handle())
            return u
        _lib.call("sgpu_band_sep_solve", ptr(b), ptr(ur), ptr(self._fac),
                  ptr(self._gens) if self._gens is not None else None, self.n, outer, Nb, inner,
                  data_kind(b), stream_handle())
        return u

    def matvec(self, v, c):
        """c = (sum_t scale_t M_t) v per wavenumber (Biharmonic.matvec,
        chebyshev/la.py:552-558: the residual of the solve); v must not be c."""
        v, cr = _raw(v), _raw(c)
        outer, Nb, inner = view3(tuple(v.shape), self.axis)
        if (outer, inner) != (self._outer, self._inner) or Nb != self.N:
            raise _lib.SgpuError(_lib.ERR_ARG, "array shape does not match the solver")
        _lib.call("sgpu_band_sep_matvec", ptr(v), ptr(cr), self.n, self._coef.shape[0], self.gen_term,
                  ptr(self._bands), ptr(self._gens) if self._gens is not None else None, ptr(self._coef),
                  outer, Nb, inner, data_kind(v), stream_handle())
        return c


class Biharmonic(BandSepSolver):
    """Chebyshev ShenBiharmonic solver for a0 S + alfa A + beta B
    (chebyshev/la.py:354-558): the same structured per-wavenumber LU, valid for
    even and odd N.  The reference's 2D/3D kernels assume equal even/odd
    lengths: with N - 4 odd its LU factors len(sii) // 2 rows per parity
    (la.pyx:1651, 1950) and its solve divides by the unfactored last even row
    (la.pyx:1356-1362), so its output is non-finite there (checked against
    the unmodified reference at N = 21 and 33)."""


def _tp(key, scale, T, ax):
    from .matrices import galerkin_matrix
    order = {"ASDSDmat": 2, "BSDSDmat": 0, "ASNSNmat": 2, "BSNSNmat": 0}[key]
    return TPMatrix(galerkin_matrix(T.bases[ax], order), np.asarray(scale, dtype=float), T, ax)


class _PoissonSolver:
    """scale * A u = b along one axis for a single Chebyshev stiffness matrix
    (SparseMatrixSolver.__call__, la.py:199-270)."""

    key = None
    entry = None

    def __init__(self, mats):
        require_cuda()
        mats = mats if isinstance(mats, (list, tuple)) else [mats]
        if len(mats) != 1 or mats[0].get_key() != self.key:
            raise ValueError(f"{type(self).__name__} takes one {self.key}")
        self.mat = mats[0]
        sc = self.mat.scale
        if isinstance(self.mat, TPMatrix) or not np.isscalar(sc) and np.size(sc) != 1:
            raise NotImplementedError("a scalar-scaled 1D stiffness matrix")
        self.scale = float(np.asarray(sc).reshape(-1)[0]) * getattr(self.mat, "sign", 1)
        self.N = self.mat.shape[0] + 2

    def _run(self, b, u, axis, extra=()):
        b = _raw(b)
        if u is None:
            u = b
        ur = _raw(u)
        outer, n, inner = view3(tuple(b.shape), axis)
        if n != self.N or tuple(ur.shape) != tuple(b.shape):
            raise _lib.SgpuError(_lib.ERR_ARG, "array shape does not match the solver")
        _lib.call(self.entry, ptr(b), ptr(ur), self.scale, *extra, outer, n, inner, data_kind(b),
                  stream_handle())
        return u


class ADDSolver(_PoissonSolver):
    """Chebyshev ShenDirichlet Poisson solve, A = ASDSD (chebyshev/la.py:11-71,
    Poisson_Solve_ADD la.pyx:614-706): back substitution with running sums."""

    key = "ASDSDmat"
    entry = "sgpu_Poisson_Solve_ADD"

    def __call__(self, b, u=None, axis=0, constraints=()):
        out = self._run(b, u, axis)
        if isinstance(out, Function) and not getattr(out.function_space(), "has_nonhomogeneous_bcs", False):
            # u.set_boundary_dofs() of a homogeneous space (la.py:265-266)
            _raw(out).narrow(axis, self.N - 2, 2).zero_()
        return out


class ANNSolver(_PoissonSolver):
    """Chebyshev ShenNeumann Poisson solve, A = ASNSN (chebyshev/la.py:74-128):
    the mean mode is fixed by the constraint u_0 = value (default 0)."""

    key = "ASNSNmat"
    entry = "sgpu_Poisson_Solve_ANN"

    def __call__(self, b, u=None, axis=0, constraints=((0, 0),)):
        cons = tuple(constraints)
        if len(cons) != 1 or cons[0][0] != 0:
            raise NotImplementedError("one constraint on row 0")
        return self._run(b, u, axis, (float(cons[0][1]),))


Solver = SolverGeneric1ND
