"""Non-homogeneous boundary values on a Chebyshev axis (CPU oracle, numpy).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates, for constant boundary values on a ShenDirichlet ('SD') or
ShenNeumann ('SN') axis:

* the boundary basis (BCGeneric.stencil_matrix, spectralbase.py:1724-1730,
  from utilities get_bc_basis): SD phi_{N-2} = (T0 - T1)/2,
  phi_{N-1} = (T0 + T1)/2; SN phi_{N-2} = T1/2 - T2/8, phi_{N-1} = T1/2 + T2/8;
* backward: to_ortho plus the boundary functions of the two boundary dofs
  (BoundaryValues._add_to_orthogonal, tensorproductspace.py:2072-2089);
* forward: scalar product, the boundary dofs set to the values of the stage
  (set_boundary_dofs, :2108-2128), minus the boundary mass matrix times them
  (_add_mass_rhs, :2091-2106), then the mass solve of the dofs;
* the Helmholtz solve with boundary matrices (chebyshev/la.py:302-306):
  b -= (alfa A_bc + beta B_bc) g, solve, boundary dofs = g.

In a tensor-product space with Fourier axes the boundary values of a stage
are the constants on every line while the Chebyshev axis is transformed
before the Fourier axes (set_tensor_bcs, tensorproductspace.py:1928-2036),
and only on the lines of the zero Fourier modes after them (the forward
transform of a constant).
"""
import numpy as np

from . import spectral as S, la, problems as P

BC_STENCIL = {"SD": np.array([[0.5, -0.5], [0.5, 0.5]]),
              "SN": np.array([[0.0, 0.5, -0.125], [0.0, 0.5, 0.125]])}


def bc_mass(basis, N):
    """B_bc[k, i] = (phi_{N-2+i}, phi_k)_w for the dofs k < N-2."""
    h = S.cheb_norm_sq(N)
    K = S.stencil("chebyshev", basis, N)
    M = BC_STENCIL[basis]
    dim = N - 2
    B = np.zeros((dim, 2))
    for k in range(dim):
        for m, v in K.items():
            j = k + m
            if j < M.shape[1] and j < N:
                B[k] += v[k] * h[j] * M[:, j]
    return B


def bc_stiffness(basis, N):
    """A_bc[k, i] = (phi''_{N-2+i}, phi_k)_w: zero for SD (linear boundary
    functions); for SN phi'' = -+ T2''/8 = -+ 1/2, so only row 0."""
    A = np.zeros((N - 2, 2))
    if basis == "SN":
        A[0] = [-np.pi / 2, np.pi / 2]
    return A


def add_to_orthogonal(c, u, basis, axis=-1):
    """c_j += sum_i M[i, j] u_{N-2+i} along axis."""
    M = BC_STENCIL[basis]
    cv, uv = np.moveaxis(c, axis, 0), np.moveaxis(u, axis, 0)
    N = uv.shape[0]
    for j in range(M.shape[1]):
        cv[j] = cv[j] + (M[0, j] * uv[N - 2] + M[1, j] * uv[N - 1])
    return c


def backward_1d(u, basis, axis=-1):
    N = u.shape[axis]
    c = S.to_ortho(u, S.stencil("chebyshev", basis, N), N - 2, axis)
    c = add_to_orthogonal(c, u, basis, axis)
    return S.cheb_backward_ortho(c, axis)


def forward_1d(f, basis, g, axis=-1):
    """g: boundary values broadcastable to f with the axis of length 2."""
    N = f.shape[axis]
    s = S.cheb_scalar_product(f, basis, axis)
    sv = np.moveaxis(s, axis, 0)
    gv = np.moveaxis(np.broadcast_to(g, _gshape(s.shape, axis)), axis, 0)
    sv[N - 2] = gv[0]
    sv[N - 1] = gv[1]
    B = bc_mass(basis, N)
    sv[:N - 2] -= B[:, 0].reshape((-1,) + (1,) * (sv.ndim - 1)) * gv[0] + \
        B[:, 1].reshape((-1,) + (1,) * (sv.ndim - 1)) * gv[1]
    out = S.mass_solve(s, "chebyshev", basis, axis)
    ov = np.moveaxis(out, axis, 0)
    ov[N - 2] = gv[0]
    ov[N - 1] = gv[1]
    return out


def _gshape(shape, axis):
    sh = list(shape)
    sh[axis] = 2
    return tuple(sh)


def stage_values(shape, axis, bc, spectral_axes, dtype=float):
    """Boundary values of every line at a stage: the constants, restricted to
    the zero mode along the Fourier axes already in spectral space."""
    g = np.zeros(_gshape(shape, axis), dtype=dtype)
    idx = [slice(None)] * len(shape)
    for a in spectral_axes:
        idx[a] = slice(0, 1)
    for i in range(2):
        ii = list(idx)
        ii[axis] = i
        g[tuple(ii)] = bc[i]
    return g


def tp_forward(f, bases, bc, axis):
    """ForwardTransform of a tensor-product space with the non-homogeneous
    Chebyshev axis `axis` (bases as in oracle.problems), default axes order."""
    out = f
    done = []
    for ax in reversed(range(len(bases))):
        if ax == axis:
            g = stage_values(out.shape, ax, bc, done, out.dtype)
            out = forward_1d(out, bases[ax][1], g, ax)
        else:
            out = P._forward_1d(out, bases[ax], ax)
        done.append(ax)
    return out


def tp_backward(u, bases, axis):
    out = u
    for ax in range(len(bases)):
        out = backward_1d(out, bases[ax][1], ax) if ax == axis else P._backward_1d(out, bases[ax], ax)
    return out


def helmholtz_bc_solve(f_hat, bases, c, axis, bc):
    """-div(grad(u)) + c u = f: alfa = -1, beta = k^2 + c per wavenumber,
    f_hat - (alfa A_bc + beta B_bc) g, solve, boundary dofs g (the final
    boundary values: the constants on the zero-mode line)."""
    b, N = bases[axis][1], bases[axis][2]
    beta = P.fourier_k2(bases, axis) + c
    bsys = np.moveaxis(np.broadcast_to(beta, beta.shape), axis, -1).reshape(-1)
    alfa = -np.ones_like(bsys)
    fs, shp = P._systems(f_hat, axis)
    g = stage_values(f_hat.shape, axis, bc, [a for a in range(len(bases)) if a != axis], f_hat.dtype)
    gl, _ = P._systems(g, axis)
    A, B = bc_stiffness(b, N), bc_mass(b, N)
    rhs = fs.copy()
    rhs[:, :N - 2] -= alfa[:, None] * (gl @ A.T) + bsys[:, None] * (gl @ B.T)
    fac = la.helmholtz_lu(N, alfa, bsys, neumann=(b == "SN"))
    us = la.helmholtz_solve(rhs, *fac, neumann=(b == "SN"))
    us[:, N - 2:] = gl
    return np.moveaxis(us.reshape(shp), -1, axis)
