"""1D function spaces and the tensor-product space, on the GPU.

Mirrors the reference's L3a/L4 layers (spectralbase.py, fourier/bases.py,
chebyshev/bases.py, tensorproductspace.py) for the spaces on the hot path:
Fourier R2C/C2C, Chebyshev Orthogonal / ShenDirichlet / ShenBiharmonic (GC
quadrature) and Legendre (see legendre.py).  Arrays are CUDA tensors; each
per-axis transform is one kernel launch of a cached ``LinePlan``.
"""
import copy

import numpy as np
import torch

from . import _lib
from .device import require_cuda, ptr, stream_handle, view3, data_kind
from .plans import get_plan


class Domain(tuple):
    pass


# ---------------------------------------------------------------------------
class SpectralBase:
    """Common 1D space interface (spectralbase.py:200-648)."""

    family_name = None
    padding_factor = 1
    # arithmetic of the transforms: _lib.PLAIN_F64 (FP64) or _lib.MIXED_DF
    # (double-float on the FP32 pipes); set by TensorProductSpace(form=...)
    form = _lib.PLAIN_F64

    def __init__(self, N, dtype=float):
        self.N = int(N)
        self.axis = 0
        self.tensorproductspace = None
        self._dtype = np.dtype(dtype)

    # -- shape / meta --------------------------------------------------------
    def family(self):
        return self.family_name

    def dim(self):
        return self.N

    def shape(self, forward_output=True):
        return self.N

    @property
    def dtype(self):
        return self._dtype

    def dimensions(self):
        return 1

    def num_bcs(self):
        return 0

    def get_unplanned(self, **kw):
        return copy.copy(self)

    # -- 1D transforms along self.axis of a tensor ---------------------------
    def _out(self, inp, forward_output, output_array, axis=None):
        if output_array is not None:
            return output_array
        shape = list(inp.shape)
        ax = self.axis if axis is None else axis
        shape[ax % inp.dim()] = self.shape(forward_output)
        return torch.empty(shape, dtype=self._out_dtype(inp, forward_output), device=inp.device)

    def _out_dtype(self, inp, forward_output):
        return inp.dtype


# ---------------------------------------------------------------------------
class FourierBase(SpectralBase):
    """fourier/bases.py:44-279.  With ``padding_factor`` > 1 the physical
    grid has M = floor(padding_factor N) points: backward pads the N
    coefficients (sgpu_fourier_pad) and runs the length-M inverse transform,
    forward / scalar_product run the length-M transform scaled by 1/M and
    truncate (sgpu_fourier_truncate) - the 3/2-rule dealiasing of
    fourier/bases.py:409-435, 570-598."""

    family_name = "fourier"

    def __init__(self, N, dtype, domain=(0.0, 2 * np.pi), padding_factor=1):
        SpectralBase.__init__(self, N, dtype)
        self.domain = Domain(domain)
        self.padding_factor = padding_factor

    @property
    def M(self):
        """points of the (padded) physical grid"""
        return int(np.floor(self.padding_factor * self.N))

    @property
    def padded(self):
        return self.M != self.N

    def get_dealiased(self, padding_factor=1.5, **kw):
        b = copy.copy(self)
        b.padding_factor = padding_factor
        return b

    def _spectral_len(self, n):
        return n

    def _fwd(self, kind, input_array, output_array, axis):
        """forward / scalar product, padded or not"""
        require_cuda()
        ax = self.axis if axis is None else axis
        out = self._out(input_array, True, output_array, ax)
        if not self.padded:
            return get_plan(kind, self.N, form=self.form)(input_array, out, ax, 1.0 / self.N)
        shape = list(input_array.shape)
        shape[ax % len(shape)] = self._spectral_len(self.M)
        work = torch.empty(shape, dtype=torch.complex128, device=input_array.device)
        get_plan(kind, self.M, form=self.form)(input_array, work, ax, 1.0 / self.M)
        outer, _, inner = view3(tuple(work.shape), ax)
        _lib.call("sgpu_fourier_truncate", ptr(work), ptr(out), outer, self.N, self.M, inner, kind,
                  stream_handle())
        return out

    def _bwd(self, kind, input_array, output_array, axis):
        require_cuda()
        ax = self.axis if axis is None else axis
        out = self._out(input_array, False, output_array, ax)
        if not self.padded:
            return get_plan(kind, self.N, form=self.form)(input_array, out, ax, 1.0)
        shape = list(input_array.shape)
        shape[ax % len(shape)] = self._spectral_len(self.M)
        work = torch.empty(shape, dtype=torch.complex128, device=input_array.device)
        outer, _, inner = view3(tuple(input_array.shape), ax)
        _lib.call("sgpu_fourier_pad", ptr(input_array), ptr(work), outer, self.N, self.M, inner, kind,
                  stream_handle())
        return get_plan(kind, self.M, form=self.form)(work, out, ax, 1.0)

    def domain_factor(self):
        a, b = self.domain
        return 2 * np.pi / (b - a)

    def points_and_weights(self, N=None, map_true_domain=False, **kw):
        N = self.M if N is None else N
        points = np.arange(N, dtype=float) * 2 * np.pi / N
        if map_true_domain:
            points = points / self.domain_factor() + self.domain[0]
        return points, np.full(N, 2 * np.pi / N)

    def mesh(self, bcast=True, map_true_domain=True):
        return self.points_and_weights(map_true_domain=map_true_domain)[0]

    def get_normalization(self):
        return 1.0 / self.N

    @staticmethod
    def boundary_condition():
        return "Periodic"


class R2C(FourierBase):
    """Real-to-complex Fourier space (fourier/bases.py:282-475)."""

    def __init__(self, N, domain=(0.0, 2 * np.pi), padding_factor=1, **kw):
        FourierBase.__init__(self, N, float, domain, padding_factor)

    def shape(self, forward_output=True):
        return self.N // 2 + 1 if forward_output else self.M

    def _spectral_len(self, n):
        return n // 2 + 1

    def wavenumbers(self, bcast=False, scaled=False, eliminate_highest_freq=False):
        k = np.fft.rfftfreq(self.N, 1.0 / self.N).astype(int)
        if self.N % 2 == 0 and eliminate_highest_freq:
            k[-1] = 0
        return k * self.domain_factor() if scaled else k

    @staticmethod
    def short_name():
        return "R2C"

    def _out_dtype(self, inp, forward_output):
        return torch.complex128 if forward_output else torch.float64

    def scalar_product(self, input_array, output_array=None, axis=None):
        return self._fwd(_lib.XF_R2C, input_array, output_array, axis)

    forward = scalar_product

    def backward(self, input_array, output_array=None, axis=None):
        return self._bwd(_lib.XF_C2R, input_array, output_array, axis)


class C2C(FourierBase):
    """Complex-to-complex Fourier space (fourier/bases.py:478-641)."""

    def __init__(self, N, domain=(0.0, 2 * np.pi), padding_factor=1, **kw):
        FourierBase.__init__(self, N, complex, domain, padding_factor)

    def shape(self, forward_output=True):
        return self.N if forward_output else self.M

    def wavenumbers(self, bcast=False, scaled=False, eliminate_highest_freq=False):
        k = np.fft.fftfreq(self.N, 1.0 / self.N).astype(int)
        if self.N % 2 == 0 and eliminate_highest_freq:
            k[self.N // 2] = 0
        return k * self.domain_factor() if scaled else k

    @staticmethod
    def short_name():
        return "C2C"

    def scalar_product(self, input_array, output_array=None, axis=None):
        return self._fwd(_lib.XF_C2C_FWD, input_array, output_array, axis)

    forward = scalar_product

    def backward(self, input_array, output_array=None, axis=None):
        return self._bwd(_lib.XF_C2C_BWD, input_array, output_array, axis)


# ---------------------------------------------------------------------------
class ChebyshevBase(SpectralBase):
    """Chebyshev spaces with Gauss-Chebyshev quadrature (chebyshev/bases.py).

    scalar_product / forward / backward run the fused GC transforms: the DCT
    with the pi/(2N) scale and the Shen stencil epilogue, the TDMA/PDMA mass
    solve (forward), or the to_ortho prologue with the DCT-III (backward).
    """

    family_name = "chebyshev"
    basis_id = _lib.BASIS_ORTHO
    quad = "GC"
    bc_values = None  # constant boundary values (left, right) of SD / SN

    def __init__(self, N, quad="GC", domain=(-1.0, 1.0), dtype=float, bc=None, **kw):
        if quad != "GC":
            raise NotImplementedError("only Gauss-Chebyshev quadrature is on the GPU path")
        SpectralBase.__init__(self, N, dtype)
        self.domain = Domain(domain)
        if bc is not None:
            vals = tuple(float(v) for v in bc)
            if any(vals):
                if self.basis_id not in (_lib.BASIS_SD, _lib.BASIS_SN) or len(vals) != 2:
                    raise NotImplementedError("non-homogeneous values on ShenDirichlet / ShenNeumann only")
                self.bc_values = vals
        self._bc_tables = {}

    @property
    def has_nonhomogeneous_bcs(self):
        return self.bc_values is not None

    def _plan_basis(self, kind):
        if kind == _lib.XF_CHEB_BACKWARD and self.has_nonhomogeneous_bcs:
            return self.basis_id | _lib.BASIS_BC
        return self.basis_id

    # -- non-homogeneous boundary values (tensorproductspace.py:1909-2128) ---
    def bc_matrices(self):
        """(A_bc, B_bc): (phi''_{N-2+i}, phi_k)_w and (phi_{N-2+i}, phi_k)_w
        for the dofs k, (N-2) x 2, of the boundary basis SD (T0 -+ T1)/2,
        SN T1/2 -+ T2/8 (BCGeneric, spectralbase.py:1702-1790)."""
        N = self.N
        h = np.full(N, np.pi / 2)
        h[0] = np.pi
        A = np.zeros((N - 2, 2))
        B = np.zeros((N - 2, 2))
        if self.basis_id == _lib.BASIS_SD:
            B[0] = [h[0] / 2, h[0] / 2]
            B[1] = [-h[1] / 2, h[1] / 2]
        else:
            B[1] = [h[1] / 2, h[1] / 2]
            B[2] = [-h[2] / 8, h[2] / 8]
            A[0] = [-h[0] / 2, h[0] / 2]
        return A, B

    def _bc_table(self, name):
        t = self._bc_tables.get(name)
        if t is None:
            A, B = self.bc_matrices()
            if name == "lift":
                # B^{-1} B_bc: the forward transform's correction of the dofs
                from .la import TDMA
                from .matrices import galerkin_matrix
                rhs = torch.as_tensor(B, device="cuda").contiguous()
                t = TDMA(galerkin_matrix(self, 0))(rhs, axis=0)
            else:
                t = torch.as_tensor(A if name == "A" else B, device="cuda").contiguous()
            self._bc_tables[name] = t
        return t

    def bc_lines(self, shape, axis, spectral_axes, dtype):
        """Boundary values of every line of an array of `shape` (the axis
        holds the two values): the constants, on the zero-mode lines of the
        Fourier axes in spectral space (set_tensor_bcs,
        tensorproductspace.py:1928-2036)."""
        key = ("g", tuple(shape), axis, tuple(sorted(spectral_axes)), dtype)
        g = self._bc_tables.get(key)
        if g is None:
            gs = list(shape)
            gs[axis] = 2
            g = torch.zeros(gs, dtype=dtype, device="cuda")
            idx = [slice(None)] * len(gs)
            for a in spectral_axes:
                idx[a] = slice(0, 1)
            for i in range(2):
                idx[axis] = i
                g[tuple(idx)] = self.bc_values[i]
            self._bc_tables[key] = g
        return g

    def _spectral_axes_before(self):
        T = self.tensorproductspace
        if T is None:
            return []
        order = list(reversed(T.axes))
        return order[:order.index(self.axis)]

    def _apply_bcs(self, arr, axis, lift):
        ax = (self.axis if axis is None else axis) % arr.dim()
        g = self.bc_lines(tuple(arr.shape), ax, self._spectral_axes_before() if lift else
                          [a for a in range(arr.dim()) if a != ax], arr.dtype)
        outer, n, inner = view3(tuple(arr.shape), ax)
        _lib.call("sgpu_bc_apply", ptr(arr), ptr(self._bc_table("lift")) if lift else None, None, None,
                  None, ptr(g), outer, n, inner, 1, data_kind(arr), stream_handle())
        return arr

    def domain_factor(self):
        a, b = self.domain
        return 2.0 / (b - a)

    def points_and_weights(self, N=None, map_true_domain=False, **kw):
        N = self.N if N is None else N
        j = np.arange(N)
        x = np.cos(np.pi * (2 * j + 1) / (2 * N))
        if map_true_domain:
            a, b = self.domain
            x = (x + 1) * (b - a) / 2 + a
        return x, np.full(N, np.pi / N)

    def mesh(self, bcast=True, map_true_domain=True):
        return self.points_and_weights(map_true_domain=map_true_domain)[0]

    def dim(self):
        return self.N - self.num_bcs()

    def _run(self, kind, input_array, output_array, axis):
        require_cuda()
        if self.domain_factor() != 1:
            raise NotImplementedError("only the reference domain [-1, 1] is on the GPU path")
        ax = self.axis if axis is None else axis
        out = self._out(input_array, True, output_array, ax)
        return get_plan(kind, self.N, self._plan_basis(kind), self.form)(input_array, out, ax)

    def scalar_product(self, input_array, output_array=None, axis=None):
        return self._run(_lib.XF_CHEB_SCALAR, input_array, output_array, axis)

    def forward(self, input_array, output_array=None, axis=None):
        out = self._run(_lib.XF_CHEB_FORWARD, input_array, output_array, axis)
        if self.has_nonhomogeneous_bcs:
            # _add_mass_rhs + mass solve (spectralbase.py:255-259) by linearity:
            # dofs -= B^{-1} B_bc g, boundary dofs = g
            self._apply_bcs(out, axis, lift=True)
        return out

    def backward(self, input_array, output_array=None, axis=None):
        return self._run(_lib.XF_CHEB_BACKWARD, input_array, output_array, axis)


class ChebyshevOrthogonal(ChebyshevBase):
    """chebyshev/bases.py:118-470."""

    @staticmethod
    def short_name():
        return "T"

    @staticmethod
    def boundary_condition():
        return ""


class ChebyshevShenDirichlet(ChebyshevBase):
    """phi_k = T_k - T_{k+2} (chebyshev/bases.py:476-581)."""

    basis_id = _lib.BASIS_SD

    def num_bcs(self):
        return 2

    @staticmethod
    def short_name():
        return "SD"

    @staticmethod
    def boundary_condition():
        return "Dirichlet"


class ChebyshevShenNeumann(ChebyshevBase):
    """phi_k = T_k - (k/(k+2))^2 T_{k+2} (chebyshev/bases.py:863-945):
    u'(-1) = u'(1) = 0."""

    basis_id = _lib.BASIS_SN

    def num_bcs(self):
        return 2

    @staticmethod
    def short_name():
        return "SN"

    @staticmethod
    def boundary_condition():
        return "Neumann"


class ChebyshevShenBiharmonic(ChebyshevBase):
    """phi_k = T_k - 2(k+2)/(k+3) T_{k+2} + (k+1)/(k+3) T_{k+4}
    (chebyshev/bases.py:1175-1258)."""

    basis_id = _lib.BASIS_SB

    def num_bcs(self):
        return 4

    @staticmethod
    def short_name():
        return "SB"

    @staticmethod
    def boundary_condition():
        return "Biharmonic"


# ---------------------------------------------------------------------------
def _bc_kinds(bc):
    """(ordered condition names, values) of a boundary-condition argument:
    a tuple of Dirichlet values (2: left/right, 4: biharmonic) or the
    reference's dict form {'left': {'D': a, 'N': b}, 'right': {...}}
    (spectralbase.py BoundaryConditions, forms/arguments.py:155-188)."""
    if bc is None:
        return "", ()
    if isinstance(bc, dict):
        names, vals = [], []
        for side, tag in (("left", "L"), ("right", "R")):
            for key, v in (bc.get(side) or {}).items():
                names.append(tag + key)
                vals.append(v)
        return "".join(names), tuple(vals)
    vals = tuple(bc)
    return {0: "", 2: "LDRD", 4: "LDLNRDRN"}.get(len(vals), "?"), vals


def FunctionSpace(N, family="Fourier", bc=None, dtype="d", quad=None, domain=None, **kw):
    """Pick the 1D space from family and boundary conditions
    (forms/arguments.py:30-418; bc tuples of zeros only - homogeneous)."""
    fam = family.lower()
    if fam in ("f", "fourier"):
        dom = domain if domain is not None else (0.0, 2 * np.pi)
        pf = kw.get("padding_factor", 1)
        if np.dtype(dtype).char in "FDG":
            return C2C(N, domain=dom, padding_factor=pf)
        return R2C(N, domain=dom, padding_factor=pf)
    kinds, vals = _bc_kinds(bc)
    nb = len(vals)
    if any(v != 0 for v in vals) and kinds not in ("LDRD", "LNRN"):
        raise NotImplementedError("non-homogeneous values on ShenDirichlet / ShenNeumann only")
    dom = domain if domain is not None else (-1.0, 1.0)
    basis = kw.get("basis")
    if fam in ("c", "chebyshev"):
        q = quad or "GC"
        if basis == "ShenNeumann" or kinds == "LNRN":
            return ChebyshevShenNeumann(N, quad=q, domain=dom, bc=vals or None)
        if basis not in (None, "ShenDirichlet", "ShenBiharmonic", "Orthogonal") or kinds not in ("", "LDRD", "LDLNRDRN"):
            raise NotImplementedError(f"Chebyshev basis {basis or kinds!r}")
        if nb == 0:
            return ChebyshevOrthogonal(N, quad=q, domain=dom)
        if nb == 2:
            return ChebyshevShenDirichlet(N, quad=q, domain=dom, bc=vals)
        if nb == 4:
            return ChebyshevShenBiharmonic(N, quad=q, domain=dom)
    if fam in ("l", "legendre"):
        if any(v != 0 for v in vals):
            raise NotImplementedError("non-homogeneous values on a Legendre space")
        from . import legendre
        return legendre.space(N, nb, quad=quad or "LG", domain=dom)
    raise NotImplementedError(f"family {family!r} with {nb} boundary conditions")


# ---------------------------------------------------------------------------
class _Chain:
    """A chain of per-axis transforms with preallocated work arrays, the
    counterpart of Forward/Backward/ScalarTransform (tensorproductspace.py:45-259)."""

    def __init__(self, T, op):
        self.T = T
        self.op = op  # 'forward' | 'scalar_product' | 'backward'
        self._input = None
        self._output = None

    @property
    def input_array(self):
        if self._input is None:
            fo = self.op == "backward"
            self._input = torch.zeros(self.T.shape(fo), dtype=self.T.torch_dtype(fo), device="cuda")
        return self._input

    @property
    def output_array(self):
        if self._output is None:
            fo = self.op != "backward"
            self._output = torch.zeros(self.T.shape(fo), dtype=self.T.torch_dtype(fo), device="cuda")
        return self._output

    def __call__(self, input_array=None, output_array=None, kind=None, **kw):
        require_cuda()
        inp = self.input_array if input_array is None else input_array
        out = self.output_array if output_array is None else output_array
        if isinstance(inp, torch.Tensor) and not inp.is_cuda:
            inp = inp.cuda()
        return self.T._execute(self.op, inp, out, kind)


class TensorProductSpace:
    """Tensor product of 1D spaces on one GPU (tensorproductspace.py:262-469).

    The last axis of ``axes`` is transformed first in forward/scalar_product
    and last in backward, as in the reference.  There is no pencil
    decomposition: every axis transform reads and writes the whole array.
    """

    def __init__(self, comm=None, bases=(), axes=None, dtype=None, form="plain", **kw):
        self.comm = comm
        self.bases = tuple(b.get_unplanned() for b in bases)
        self.form = _lib.FORMS[form]
        nd = len(self.bases)
        for i, b in enumerate(self.bases):
            b.axis = i
            b.tensorproductspace = self
            b.form = self.form
        self.axes = tuple(range(nd)) if axes is None else tuple(int(a) % nd for a in axes)
        first = self.bases[self.axes[-1]]
        if dtype is None:
            dtype = complex if isinstance(first, C2C) else float
        self._dtype = np.dtype(dtype)
        if isinstance(first, R2C):
            assert self._dtype.char in "fdg"
        # the R2C axis needs real data: it must come before every C2C axis in
        # the forward order (last axis of `axes` first)
        order = list(reversed(self.axes))
        r2c = [order.index(i) for i, b in enumerate(self.bases) if isinstance(b, R2C)]
        c2c = [order.index(i) for i, b in enumerate(self.bases) if isinstance(b, C2C)]
        if len(r2c) > 1 or (r2c and c2c and min(c2c) < r2c[0]):
            raise ValueError("the R2C axis must be transformed before every C2C axis")
        if r2c and self._dtype.char in "FDG":
            raise ValueError("an R2C axis needs real physical data")
        self.forward = _Chain(self, "forward")
        self.backward = _Chain(self, "backward")
        self.scalar_product = _Chain(self, "scalar_product")
        self._work = {}

    def get_dealiased(self, padding_factor=1.5, dealias_direct=False, **kw):
        """The space with padded Fourier axes (3/2-rule dealiasing,
        tensorproductspace.py:543): one factor for every axis or a tuple.
        Polynomial axes keep factor 1 (padding them is not on the GPU path)."""
        if dealias_direct:
            raise NotImplementedError("dealias_direct (2/3-rule truncation) is not on the GPU path")
        nd = len(self.bases)
        fac = tuple(padding_factor) if isinstance(padding_factor, (tuple, list)) else (padding_factor,) * nd
        bases = []
        for b, f in zip(self.bases, fac):
            if isinstance(b, FourierBase):
                bases.append(b.get_dealiased(f))
            elif f == 1:
                bases.append(copy.copy(b))
            else:
                raise NotImplementedError("padding along polynomial axes")
        return TensorProductSpace(self.comm, bases, axes=self.axes, dtype=self._dtype, form=self.form)

    # -- meta ----------------------------------------------------------------
    def __len__(self):
        return len(self.bases)

    @property
    def dimensions(self):
        return len(self.bases)

    def shape(self, forward_output=False):
        return tuple(b.shape(forward_output) for b in self.bases)

    def global_shape(self, forward_output=False):
        return self.shape(forward_output)

    def dims(self):
        return self.shape(True)

    def dtype(self, forward_output=False):
        if forward_output:
            if any(isinstance(b, FourierBase) for b in self.bases) or self._dtype.char in "FDG":
                return np.dtype(complex)
            return np.dtype(float)
        return self._dtype

    def torch_dtype(self, forward_output=False):
        return torch.complex128 if self.dtype(forward_output).char in "FDG" else torch.float64

    def local_slice(self, forward_output=True):
        return tuple(slice(0, n) for n in self.shape(forward_output))

    def get_nonperiodic_axes(self):
        return [i for i, b in enumerate(self.bases) if not isinstance(b, FourierBase)]

    def local_wavenumbers(self, broadcast=False, scaled=False, eliminate_highest_freq=False):
        ks = []
        nd = len(self.bases)
        for i, b in enumerate(self.bases):
            if isinstance(b, FourierBase):
                k = b.wavenumbers(scaled=scaled, eliminate_highest_freq=eliminate_highest_freq)
            else:
                k = np.arange(b.N)
            s = [1] * nd
            s[i] = len(k)
            k = np.asarray(k).reshape(s)
            ks.append(np.broadcast_to(k, self.shape(True)) if broadcast else k)
        return ks

    def mesh(self, map_true_domain=True):
        out = []
        nd = len(self.bases)
        for i, b in enumerate(self.bases):
            x = b.mesh(map_true_domain=map_true_domain)
            s = [1] * nd
            s[i] = len(x)
            out.append(x.reshape(s))
        return out

    local_mesh = mesh

    # -- execution -----------------------------------------------------------
    def _buf(self, key, shape, dtype):
        t = self._work.get(key)
        if t is None or tuple(t.shape) != tuple(shape) or t.dtype != dtype:
            t = torch.empty(shape, dtype=dtype, device="cuda")
            self._work[key] = t
        return t

    def _execute(self, op, inp, out, kind=None):
        order = list(reversed(self.axes)) if op != "backward" else list(self.axes)
        shape = list(inp.shape)
        cur = inp
        nsteps = len(order)
        for step, ax in enumerate(order):
            b = self.bases[ax]
            fo = op != "backward"
            new_shape = list(shape)
            new_shape[ax] = b.shape(fo)
            if isinstance(b, R2C):
                dt = torch.complex128 if fo else torch.float64
            else:
                dt = cur.dtype
            last = step == nsteps - 1
            if last:
                dst = out
            elif (cur is not inp and tuple(new_shape) == tuple(cur.shape) and dt == cur.dtype
                  and getattr(b, "inplace_ok", True)):
                dst = cur  # same-size transform: in place on a work array
            else:
                dst = self._buf(("w", step % 2, tuple(new_shape), dt), new_shape, dt)
                if dst is cur:
                    dst = self._buf(("w", (step + 1) % 2, tuple(new_shape), dt), new_shape, dt)
            getattr(b, op)(cur, dst, axis=ax)
            cur = dst
            shape = new_shape
        return out
