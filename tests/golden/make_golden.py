"""Generate golden fixtures by running the unmodified reference (shenfun 4.3.0).

TEST INFRASTRUCTURE ONLY.  Run in a container that has the reference checkout
and the compiled reference kernels (``python oracle/build_ref.py`` first):

    python tests/golden/make_golden.py

Every fixture is a small ``.npz`` written next to this script.  The inputs are
seeded (numpy ``default_rng``), so re-running reproduces the files.  FFTW is
absent here; the shims reproduce its unnormalised conventions with scipy.fft,
so the transform fixtures pin the reference's scaling, stencil and solver
arithmetic, not FFTW's own rounding.
"""
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
warnings.simplefilter("ignore")

from refimport import import_reference  # noqa: E402

sf = import_reference()
from shenfun import (FunctionSpace, TensorProductSpace, Array, Function,  # noqa: E402
                     TrialFunction, TestFunction, inner, div, grad, la, chebyshev,
                     comm, Dx)
import sympy as sp  # noqa: E402

OUT = {}


def put(name, **arrays):
    OUT.setdefault(name, {}).update({k: np.asarray(v) for k, v in arrays.items()})


def save():
    for name, d in OUT.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        size = os.path.getsize(os.path.join(HERE, name + ".npz"))
        print(f"{name}.npz: {len(d)} arrays, {size/1024:.1f} KiB")


rng = np.random.default_rng(20261204)


# --------------------------------------------------------------------------
# 1D Chebyshev transforms: Orthogonal (T), ShenDirichlet (SD), ShenBiharmonic (SB)
# chebyshev/bases.py:315-353 (DCT scaling), spectralbase.py:1450-1474 (stencil)
def cheb_1d():
    for N in (8, 9, 16, 17, 33, 64):
        for tag, bc in (("T", None), ("SD", (0, 0)), ("SB", (0, 0, 0, 0))):
            if tag == "SB" and N < 12:
                continue
            V = FunctionSpace(N, "C", bc=bc) if bc else FunctionSpace(N, "C")
            f = rng.standard_normal(N)
            sp_ = V.scalar_product(f.copy(), np.zeros(N)).copy()
            fw = V.forward(f.copy(), np.zeros(N)).copy()
            dim = V.dim()
            uh = np.zeros(N)
            uh[:dim] = rng.standard_normal(dim)
            bw = V.backward(uh.copy(), np.zeros(N)).copy()
            x, w = V.points_and_weights()
            put("cheb_1d", **{f"{tag}{N}_f": f, f"{tag}{N}_sp": sp_,
                               f"{tag}{N}_fw": fw, f"{tag}{N}_uh": uh,
                               f"{tag}{N}_bw": bw, f"{tag}{N}_x": x,
                               f"{tag}{N}_w": w})


# --------------------------------------------------------------------------
# 1D Fourier: fourier/bases.py:131-162 (forward 1/N), :380-407 (backward)
def fourier_1d():
    for N in (8, 9, 16, 64):
        R = FunctionSpace(N, "F", dtype="d")
        f = rng.standard_normal(N)
        fw = R.forward(f.copy(), np.zeros(N // 2 + 1, complex)).copy()
        uh = rng.standard_normal(N // 2 + 1) + 1j * rng.standard_normal(N // 2 + 1)
        uh[0] = uh[0].real
        if N % 2 == 0:
            uh[-1] = uh[-1].real
        bw = R.backward(uh.copy(), np.zeros(N)).copy()
        C = FunctionSpace(N, "F", dtype="D")
        fc = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        fwc = C.forward(fc.copy(), np.zeros(N, complex)).copy()
        uhc = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        bwc = C.backward(uhc.copy(), np.zeros(N, complex)).copy()
        put("fourier_1d", **{f"R{N}_f": f, f"R{N}_fw": fw, f"R{N}_uh": uh,
                              f"R{N}_bw": bw, f"C{N}_f": fc, f"C{N}_fw": fwc,
                              f"C{N}_uh": uhc, f"C{N}_bw": bwc,
                              f"R{N}_k": R.wavenumbers(bcast=False),
                              f"C{N}_k": C.wavenumbers(bcast=False)})


# --------------------------------------------------------------------------
# Banded solvers: la.py:331-393 (TDMA), :450-543 (PDMA); la.pyx:213-252,496-532
def banded():
    for N in (16, 17, 32):
        SD = FunctionSpace(N, "C", bc=(0, 0))
        u, v = TrialFunction(SD), TestFunction(SD)
        B = inner(u, v)
        data = np.zeros((3, N - 2))
        data[0, :-2] = B[-2] if np.ndim(B[-2]) else B[-2] * np.ones(N - 4)
        data[1] = B[0]
        data[2, 2:] = B[2] if np.ndim(B[2]) else B[2] * np.ones(N - 4)
        raw = data.copy()
        sol = la.TDMA(B)
        b1 = rng.standard_normal(N - 2)
        x1 = sol(b1.copy())
        b2 = rng.standard_normal((N - 2, 5)) + 1j * rng.standard_normal((N - 2, 5))
        x2 = la.TDMA(B)(b2.copy(), axis=0)
        b3 = rng.standard_normal((4, N - 2))
        x3 = la.TDMA(B)(b3.copy(), axis=1)
        lu = data.copy()
        la.TDMA.LU(lu)
        put("banded", **{f"tdma{N}_raw": raw, f"tdma{N}_lu": lu, f"tdma{N}_b1": b1,
                         f"tdma{N}_x1": x1, f"tdma{N}_b2": b2, f"tdma{N}_x2": x2,
                         f"tdma{N}_b3": b3, f"tdma{N}_x3": x3})
        SB = FunctionSpace(N, "C", bc=(0, 0, 0, 0))
        u, v = TrialFunction(SB), TestFunction(SB)
        B = inner(u, v)
        n = N - 4
        data = np.zeros((5, n))
        data[0, :-4] = B[-4]
        data[1, :-2] = B[-2]
        data[2] = B[0]
        data[3, 2:] = B[2]
        data[4, 4:] = B[4]
        raw = data.copy()
        b1 = rng.standard_normal(n)
        x1 = la.PDMA(B)(b1.copy())
        b2 = rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3))
        x2 = la.PDMA(B)(b2.copy(), axis=0)
        lu = data.copy()
        la.PDMA.LU(lu)
        put("banded", **{f"pdma{N}_raw": raw, f"pdma{N}_lu": lu, f"pdma{N}_b1": b1,
                         f"pdma{N}_x1": x1, f"pdma{N}_b2": b2, f"pdma{N}_x2": x2})


# --------------------------------------------------------------------------
# Chebyshev Dirichlet Helmholtz: chebyshev/la.py:131-351, la.pyx:717-947
def helmholtz():
    for (Nx, Ny, Nz, c) in ((8, 8, 17, 1000.0), (6, 4, 16, 0.0), (4, 6, 33, 50.0)):
        F0 = FunctionSpace(Nx, "F", dtype="D")
        F1 = FunctionSpace(Ny, "F", dtype="d")
        SD = FunctionSpace(Nz, "C", bc=(0, 0))
        T = TensorProductSpace(comm, (F0, F1, SD))
        u, v = TrialFunction(T), TestFunction(T)
        mats = inner(v, -div(grad(u)) + c * u)
        H = chebyshev.la.Helmholtz(*mats)
        fh = Function(T)
        shp = fh.shape
        fh[:] = rng.standard_normal(shp) + 1j * rng.standard_normal(shp)
        fh[..., -2:] = 0
        if c == 0.0:
            fh[0, 0] = 0
        uh = Function(T)
        uh = H(fh.copy(), uh)
        mv = np.zeros_like(uh)
        mv = H.matvec(uh.copy(), mv)
        key = f"h{Nx}x{Ny}x{Nz}"
        put("helmholtz", **{key + "_c": c, key + "_alfa": H.alfa, key + "_beta": H.beta,
                            key + "_d0": H.u0, key + "_d1": H.u1, key + "_d2": H.u2,
                            key + "_L": H.L, key + "_f": fh, key + "_u": uh,
                            key + "_mv": mv})
    # 2D case with the solve axis first (the reference's 1D entry converts a
    # 1-element scale array to a scalar, which numpy 2 rejects: la.pyx:718)
    SD = FunctionSpace(20, "C", bc=(0, 0))
    F1 = FunctionSpace(6, "F", dtype="d")
    T = TensorProductSpace(comm, (SD, F1), axes=(0, 1))
    u, v = TrialFunction(T), TestFunction(T)
    mats = inner(v, -div(grad(u)) + 7.5 * u)
    H = chebyshev.la.Helmholtz(*mats)
    f = Function(T)
    f[:] = rng.standard_normal(f.shape) + 1j * rng.standard_normal(f.shape)
    f[-2:] = 0
    x = H(f.copy(), Function(T))
    put("helmholtz", h2d_f=f, h2d_u=x, h2d_d0=H.u0, h2d_d1=H.u1, h2d_d2=H.u2,
        h2d_L=H.L, h2d_alfa=H.alfa, h2d_beta=H.beta)


# --------------------------------------------------------------------------
# Full round trips (forward -> solve -> backward) on tensor-product spaces.
def roundtrips():
    # cfg1: 2D Poisson, F64 x SD64, manufactured solution.
    N = (64, 64)
    K0 = FunctionSpace(N[0], "F", dtype="d")
    SD = FunctionSpace(N[1], "C", bc=(0, 0))
    T = TensorProductSpace(comm, (K0, SD), axes=(1, 0))
    u, v = TrialFunction(T), TestFunction(T)
    x, y = sp.symbols("x,y", real=True)
    ue = sp.sin(2 * x) * (1 - y ** 2) * sp.cos(sp.pi * y / 2)
    fe = -(ue.diff(x, 2) + ue.diff(y, 2))
    fj = Array(T, buffer=fe)
    f_hat = inner(v, fj)
    mats = inner(v, -div(grad(u)))
    H = chebyshev.la.Helmholtz(*mats)
    u_hat = H(f_hat.copy(), Function(T))
    g = la.SolverGeneric1ND(mats)
    u_hat2 = g(f_hat.copy(), Function(T))
    uq = u_hat.backward()
    uj = Array(T, buffer=ue)
    mesh = T.local_mesh(True)
    put("cfg1_poisson2d", fj=fj, f_hat=f_hat, u_hat=u_hat, u_hat_generic=u_hat2,
        uq=uq, uj=uj, x=mesh[0], y=mesh[1], fw=uj.forward())

    # cfg2 shape family at small size: C2C x R2C x SD, alpha=k^2+1/(nu dt)
    for (Nx, Ny, Nz) in ((8, 8, 17), (16, 12, 24)):
        F0 = FunctionSpace(Nx, "F", dtype="D")
        F1 = FunctionSpace(Ny, "F", dtype="d")
        SD = FunctionSpace(Nz, "C", bc=(0, 0))
        T = TensorProductSpace(comm, (F0, F1, SD))
        u, v = TrialFunction(T), TestFunction(T)
        mats = inner(v, -div(grad(u)) + 1000.0 * u)
        H = chebyshev.la.Helmholtz(*mats)
        fj = Array(T)
        fj[:] = rng.standard_normal(fj.shape)
        f_hat = inner(v, fj)
        u_hat = H(f_hat.copy(), Function(T))
        uq = u_hat.backward()
        fw = fj.forward()
        put(f"cfg2_{Nx}x{Ny}x{Nz}", fj=fj, f_hat=f_hat, u_hat=u_hat, uq=uq, fw=fw,
            fwbw=fw.backward())


# --------------------------------------------------------------------------
# Biharmonic: chebyshev/la.py:354-558 (even N), la.SolverGeneric1ND (odd N)
def biharmonic():
    x, y, z = sp.symbols("x,y,z", real=True)
    ue = sp.sin(x) * sp.cos(y) * (1 - z ** 2) ** 2
    fe = ue.diff(x, 4) + ue.diff(y, 4) + ue.diff(z, 4) + 2 * ue.diff(x, 2, y, 2) + \
        2 * ue.diff(x, 2, z, 2) + 2 * ue.diff(y, 2, z, 2)
    for (Nx, Ny, Nz) in ((8, 8, 16), (8, 8, 17)):
        F0 = FunctionSpace(Nx, "F", dtype="D")
        F1 = FunctionSpace(Ny, "F", dtype="d")
        SB = FunctionSpace(Nz, "C", bc=(0, 0, 0, 0))
        T = TensorProductSpace(comm, (F0, F1, SB))
        u, v = TrialFunction(T), TestFunction(T)
        fj = Array(T, buffer=fe)
        f_hat = inner(v, fj)
        mats = inner(v, div(grad(div(grad(u)))))
        g = la.SolverGeneric1ND(mats)
        u_hat = g(f_hat.copy(), Function(T))
        d = dict(fj=fj, f_hat=f_hat, u_hat_generic=u_hat, uq=u_hat.backward(),
                 uj=Array(T, buffer=ue))
        if Nz % 2 == 0:
            Hb = chebyshev.la.Biharmonic(*mats)
            u_hat_b = Hb(f_hat.copy(), Function(T))
            d["u_hat_biharmonic"] = u_hat_b
        put(f"biharmonic_{Nx}x{Ny}x{Nz}", **d)


# --------------------------------------------------------------------------
# Legendre: nodes/weights (fastgl), SD transforms (recursive + vandermonde),
# Fourier x Legendre Poisson via SolverGeneric1ND/TDMA.
def legendre():
    for N in (4, 8, 16, 33, 100):
        L = FunctionSpace(N, "L")
        xw = L.points_and_weights()
        put("legendre", **{f"xw{N}_x": xw[0], f"xw{N}_w": xw[1]})
    for N in (16, 33, 64):
        for tag, bc in (("L", None), ("LD", (0, 0))):
            V = FunctionSpace(N, "L", bc=bc) if bc else FunctionSpace(N, "L")
            f = rng.standard_normal(N)
            dim = V.dim()
            uh = np.zeros(N)
            uh[:dim] = rng.uniform(-1, 1, dim) * (np.arange(dim) + 1.0) ** -2
            d = {f"{tag}{N}_f": f, f"{tag}{N}_uh": uh}
            for kind in ("recursive", "vandermonde"):
                d[f"{tag}{N}_sp_{kind}"] = V.scalar_product(f.copy(), np.zeros(N), kind=kind).copy()
                d[f"{tag}{N}_bw_{kind}"] = V.backward(uh.copy(), np.zeros(N), kind=kind).copy()
                d[f"{tag}{N}_fw_{kind}"] = V.forward(f.copy(), np.zeros(N), kind=kind).copy()
            put("legendre", **d)
    # 2D Fourier x Legendre Dirichlet Helmholtz via SolverGeneric1ND
    K0 = FunctionSpace(16, "F", dtype="d")
    LD = FunctionSpace(24, "L", bc=(0, 0))
    T = TensorProductSpace(comm, (K0, LD), axes=(1, 0))
    u, v = TrialFunction(T), TestFunction(T)
    fj = Array(T)
    fj[:] = rng.standard_normal(fj.shape)
    f_hat = inner(v, fj)
    mats = inner(v, -div(grad(u)) + 3.0 * u)
    g = la.SolverGeneric1ND(mats)
    u_hat = g(f_hat.copy(), Function(T))
    put("legendre", p2d_fj=fj, p2d_fhat=f_hat, p2d_uhat=u_hat, p2d_uq=u_hat.backward())


# --------------------------------------------------------------------------
# IMEX Runge-Kutta time stepping of u_t = nu lap(u) + f (utilities/integrators.py:702-900)
# on C2C x R2C x ShenDirichlet, with a fixed spectral forcing f_hat as the
# "nonlinear" term; three steps of each scheme from the same start.  Own rng,
# so that the other fixtures keep their draws.
def imex():
    from shenfun.utilities.integrators import IMEXRK111, IMEXRK222, IMEXRK443
    r = np.random.default_rng(31)
    T = TensorProductSpace(comm, (FunctionSpace(8, "F", dtype="D"), FunctionSpace(8, "F", dtype="d"),
                                  FunctionSpace(17, "C", bc=(0, 0))))
    nu, dt = 0.05, 0.01
    a = Array(T)
    a[:] = r.standard_normal(a.shape)
    u_hat0 = a.forward()
    a[:] = r.standard_normal(a.shape)
    f_hat = a.forward()
    d = {"u_hat0": u_hat0.copy(), "f_hat": f_hat.copy(), "nu": nu, "dt": dt}
    for cls in (IMEXRK111, IMEXRK222, IMEXRK443):
        u_hat = Function(T)
        u_hat[:] = u_hat0
        sol = cls(TestFunction(T), u_hat, lambda u: nu * div(grad(u)), f_hat, dt)
        sol.assemble()
        for step in range(3):
            for rk in range(sol.steps()):
                sol.compute_rhs(rk)
                sol.solve_step(rk)
            d[f"{cls.__name__}_step{step}"] = u_hat.copy()
    put("imex", **d)


# --------------------------------------------------------------------------
# Padded (3/2-rule) transforms on the Fourier axes (TensorProductSpace.get_dealiased,
# tensorproductspace.py:543; fourier/bases.py:409-435, 570-598): backward of
# spectral data onto the padded grid, forward of padded-grid data, for even
# and odd Fourier lengths.  Own rng.
def dealias():
    r = np.random.default_rng(43)
    d = {}
    for (Nx, Ny, Nz) in ((8, 8, 17), (9, 7, 12)):
        T = TensorProductSpace(comm, (FunctionSpace(Nx, "F", dtype="D"), FunctionSpace(Ny, "F", dtype="d"),
                                      FunctionSpace(Nz, "C", bc=(0, 0))))
        TD = T.get_dealiased((1.5, 1.5, 1))
        a = Array(T)
        a[:] = r.standard_normal(a.shape)
        u_hat = a.forward()
        up = Array(TD)
        up = TD.backward(u_hat, up)
        b = Array(TD)
        b[:] = r.standard_normal(b.shape)
        fh = Function(TD)
        fh = TD.forward(b, fh)
        sh = Function(TD)
        sh = TD.scalar_product(b, sh)
        tag = f"{Nx}x{Ny}x{Nz}"
        d.update({f"{tag}_u_hat": u_hat.copy(), f"{tag}_padded_backward": up.copy(),
                  f"{tag}_padded_in": b.copy(), f"{tag}_padded_forward": fh.copy(),
                  f"{tag}_padded_scalar": sh.copy()})
    put("dealias", **d)


# --------------------------------------------------------------------------
# Chebyshev ShenNeumann and the Poisson solvers: SN transforms
# (chebyshev/bases.py:863-945), the Neumann branch of LU_Helmholtz /
# Solve_Helmholtz (la.pyx:733-751, 907-912) with Helmholtz_Neumann_matvec
# (Matvec.pyx:722-800), ADDSolver (chebyshev/la.py:11-71, la.pyx:614-706) and
# ANNSolver (chebyshev/la.py:74-128).  Own rng, so the group reproduces alone.
def neumann():
    g = np.random.default_rng(59)
    d = {}
    bcN = {"left": {"N": 0}, "right": {"N": 0}}
    for N in (8, 9, 16, 17, 33):
        V = FunctionSpace(N, "C", bc=bcN)
        assert V.short_name() == "SN"
        f = g.standard_normal(N)
        d[f"sn{N}_f"] = f
        d[f"sn{N}_sp"] = V.scalar_product(f.copy(), np.zeros(N)).copy()
        d[f"sn{N}_fw"] = V.forward(f.copy(), np.zeros(N)).copy()
        uh = np.zeros(N)
        uh[:N - 2] = g.standard_normal(N - 2)
        d[f"sn{N}_uh"] = uh
        d[f"sn{N}_bw"] = V.backward(uh.copy(), np.zeros(N)).copy()
    for (Nx, Ny, Nz, c) in ((6, 4, 16, 0.0), (4, 6, 17, 50.0), (8, 8, 33, 1000.0)):
        F0 = FunctionSpace(Nx, "F", dtype="D")
        F1 = FunctionSpace(Ny, "F", dtype="d")
        SN = FunctionSpace(Nz, "C", bc=bcN)
        T = TensorProductSpace(comm, (F0, F1, SN))
        u, v = TrialFunction(T), TestFunction(T)
        mats = inner(v, -div(grad(u)) + c * u)
        H = chebyshev.la.Helmholtz(*mats)
        assert H.neumann
        fh = Function(T)
        fh[:] = g.standard_normal(fh.shape) + 1j * g.standard_normal(fh.shape)
        fh[..., -2:] = 0
        uh = H(fh.copy(), Function(T))
        key = f"h{Nx}x{Ny}x{Nz}"
        d.update({key + "_c": c, key + "_alfa": H.alfa, key + "_beta": H.beta,
                  key + "_d0": H.u0, key + "_d1": H.u1, key + "_d2": H.u2, key + "_L": H.L,
                  key + "_f": fh, key + "_u": uh})
    # Helmholtz_Neumann_matvec does not run under numpy 2 (its 1/j2 lands in
    # an integer array, Matvec.pyx:785-788): record the reference's own
    # ASNSN / BSNSN matrices instead, the matvec's definition
    for N in (16, 17):
        SN = FunctionSpace(N, "C", bc=bcN)
        A = inner(TestFunction(SN), div(grad(TrialFunction(SN))))
        B = inner(TestFunction(SN), TrialFunction(SN))
        d.update({f"snA{N}": A.diags("csr").toarray(), f"snB{N}": B.diags("csr").toarray()})
    # Poisson solvers along one axis
    for N in (16, 17, 32):
        SD = FunctionSpace(N, "C", bc=(0, 0))
        A = inner(TestFunction(SD), div(grad(TrialFunction(SD))))
        sol = chebyshev.la.ADDSolver(A)
        b = Function(SD)
        b[:] = g.standard_normal(N)
        b[-2:] = 0
        x = sol(b.copy(), Function(SD))
        d.update({f"add{N}_b": b, f"add{N}_u": x, f"add{N}_scale": A.scale,
                  f"add{N}_A0": np.asarray(A[0]), f"add{N}_A2": np.broadcast_to(A[2], (N - 4,)).copy()})
        SN = FunctionSpace(N, "C", bc=bcN)
        A = inner(TestFunction(SN), -div(grad(TrialFunction(SN))))
        sol = chebyshev.la.ANNSolver(A)
        b = Function(SN)
        b[:] = g.standard_normal(N)
        b[-2:] = 0
        x = sol(b.copy(), Function(SN))
        d.update({f"ann{N}_b": b, f"ann{N}_u": x, f"ann{N}_scale": A.scale,
                  f"ann{N}_A0": np.asarray(A[0]), f"ann{N}_A2": np.asarray(A[2])})
    # ADD on a 2D array along either axis (the compiled kernel, la.pyx:614-629)
    from shenfun.optimization.cython import la as cla
    SD = FunctionSpace(20, "C", bc=(0, 0))
    A = inner(TestFunction(SD), div(grad(TrialFunction(SD))))
    for ax in (0, 1):
        shape = (20, 5) if ax == 0 else (5, 20)
        b = g.standard_normal(shape) + 1j * g.standard_normal(shape)
        u = np.zeros_like(b)
        cla.Poisson_Solve_ADD(A, b.copy(), u, ax)
        d.update({f"add2d{ax}_b": b, f"add2d{ax}_u": u})
    put("neumann", **d)


# --------------------------------------------------------------------------
# Non-homogeneous boundary values on a Chebyshev axis (constants): the
# boundary basis (utilities get_bc_basis via BCGeneric, spectralbase.py:
# 1702-1790), BoundaryValues (tensorproductspace.py:1909-2106: set_tensor_bcs,
# _add_to_orthogonal, _add_mass_rhs, set_boundary_dofs) and the Helmholtz
# solve with boundary matrices (chebyshev/la.py:222-317).  Own rng.
def nonhomog():
    g = np.random.default_rng(67)
    d = {}
    cases = {"SD": (1.5, -0.5), "SN": {"left": {"N": 0.7}, "right": {"N": -0.3}}}
    for tag, bc in cases.items():
        for N in (12, 17):
            V = FunctionSpace(N, "C", bc=bc)
            assert V.short_name() == tag and V.has_nonhomogeneous_bcs
            f = g.standard_normal(N)
            d[f"{tag}{N}_f"] = f
            d[f"{tag}{N}_sp"] = V.scalar_product(f.copy(), np.zeros(N)).copy()
            d[f"{tag}{N}_fw"] = V.forward(f.copy(), np.zeros(N)).copy()
            uh = Function(V)
            uh[:N - 2] = g.standard_normal(N - 2)
            uh.set_boundary_dofs()
            d[f"{tag}{N}_uh"] = np.array(uh)
            d[f"{tag}{N}_bw"] = V.backward(np.array(uh), np.zeros(N)).copy()
    # channel grids: Fourier x Fourier x Chebyshev with constant wall values,
    # and a 2D grid with the Chebyshev axis first
    for tag, bc in cases.items():
        for shape, order in (((8, 6, 17), "last"), ((16, 6), "first")):
            if order == "last":
                Nx, Ny, Nz = shape
                bases = (FunctionSpace(Nx, "F", dtype="D"), FunctionSpace(Ny, "F", dtype="d"),
                         FunctionSpace(Nz, "C", bc=bc))
            else:
                Nz, Ny = shape
                bases = (FunctionSpace(Nz, "C", bc=bc), FunctionSpace(Ny, "F", dtype="d"))
            T = TensorProductSpace(comm, bases)
            key = f"{tag}_" + "x".join(str(n) for n in shape)
            fa = Array(T)
            fa[:] = g.standard_normal(fa.shape)
            d[key + "_f"] = np.array(fa)
            d[key + "_fw"] = np.array(fa.forward(Function(T)))
            d[key + "_sp"] = np.array(inner(TestFunction(T), fa))
            uh = Function(T)
            uh[:] = g.standard_normal(uh.shape) + 1j * g.standard_normal(uh.shape)
            uh.set_boundary_dofs()
            d[key + "_uh"] = np.array(uh)
            d[key + "_bw"] = np.array(uh.backward(Array(T)))
            u, v = TrialFunction(T), TestFunction(T)
            c = 5.0
            mats = inner(v, -div(grad(u)) + c * u)
            H = chebyshev.la.Helmholtz(*mats)
            fh = inner(v, fa)
            x = H(fh.copy(), Function(T))
            d[key + "_rhs"] = np.array(fh)
            d[key + "_sol"] = np.array(x)
            d[key + "_solx"] = np.array(x.backward(Array(T)))
    put("nonhomog", **d)


# --------------------------------------------------------------------------
# The other banded solvers of the kernel dispatch list: DiagMA, TwoDMA,
# ThreeDMA, FDMA, HeptaDMA (la.py:291-800, la.pyx), on diagonally dominant
# random bands, solved along each axis of a 2D array.  Own rng.
def dma():
    from shenfun.matrixbase import SparseMatrix
    g = np.random.default_rng(73)
    d = {}
    kinds = {"DiagMA": (0,), "TwoDMA": (0, 2), "ThreeDMA": (0, 2, 4), "FDMA": (-2, 0, 2, 4),
             "HeptaDMA": (-4, -2, 0, 2, 4, 6, 8)}
    for name, offs in kinds.items():
        for n in (12, 17):
            diags = {}
            for o in offs:
                m = n - abs(o)
                diags[o] = (4.0 + g.uniform(0, 1, m)) if o == 0 else g.uniform(-0.5, 0.5, m)
            M = SparseMatrix(dict(diags), (n, n))
            dense = M.diags("csr").toarray()
            for ax, shape in ((0, (n,)), (0, (n, 3)), (1, (4, n))):
                b = g.standard_normal(shape)
                sol = getattr(la, name)(SparseMatrix(dict(diags), (n, n)))
                try:
                    u = sol(b.copy(), axis=ax)
                except ValueError:
                    continue  # the reference's DiagMA solve takes 1D right-hand sides only
                key = f"{name}{n}_{len(shape)}d_ax{ax}"
                d.update({key + "_b": b, key + "_u": np.array(u)})
            d[f"{name}{n}_dense"] = dense
    put("dma", **d)


# --------------------------------------------------------------------------
# The kernel dispatch boundary (optimization/__init__.py:37-84): every call
# the reference's own classes make to its compiled kernels by name, recorded
# with its arguments before and after (the kernels write in place).  The
# replays in tests/test_optimization_mode.py and test_gpu_optimization_mode.py
# feed the same arguments to the gb300 optimization module and to the oracle.
# Own rng.
OPT_NAMES = ("TDMA_LU", "TDMA_Solve", "PDMA_LU", "PDMA_Solve", "FDMA_LU", "FDMA_Solve", "TwoDMA_Solve",
             "ThreeDMA_Solve", "DiagMA_Solve", "HeptaDMA_LU", "HeptaDMA_Solve", "TDMA_O_LU", "TDMA_O_Solve",
             "SolverGeneric1ND_solve_data", "LU_Helmholtz", "Solve_Helmholtz", "Helmholtz_matvec",
             "LU_Biharmonic", "Biharmonic_factor_pr", "Biharmonic_Solve", "Biharmonic_matvec")
OPT_TRANSFORMS = ("scalar_product", "evaluate_expansion_all")


def optmode():
    import functools
    import json
    import shenfun.optimization as opt
    from shenfun.matrixbase import SparseMatrix, SpectralMatrix
    g = np.random.default_rng(4099)
    cy = opt.cython
    tr = sys.modules["shenfun.optimization.cython.transforms"]
    calls = []
    arrays = {}

    def snap(a, key):
        if isinstance(a, (bool, np.bool_)):
            return {"t": "bool", "v": bool(a)}
        if isinstance(a, (int, float, np.integer, np.floating)) and not isinstance(a, np.ndarray):
            return {"t": "num", "v": float(a), "int": isinstance(a, (int, np.integer))}
        if callable(a) and not isinstance(a, np.ndarray):
            return {"t": "fn", "v": a.__name__}
        if isinstance(a, (SparseMatrix, SpectralMatrix)) or (isinstance(a, dict)):
            offs = sorted(int(k) for k in a.keys())
            for o in offs:
                arrays[f"{key}_d{o}"] = np.atleast_1d(np.asarray(a[o], dtype=float)).copy()
            return {"t": "mat", "offsets": offs, "key": key}
        arr = np.asarray(a)
        if arr.ndim == 0:
            return {"t": "num", "v": float(arr), "int": False}
        arrays[key] = arr.copy()
        return {"t": "arr", "key": key}

    def recorder(name, fn):
        @functools.wraps(fn)
        def wrapped(*args):
            i = len(calls)
            spec = [snap(a, f"c{i:03d}_a{j}") for j, a in enumerate(args)]
            before = [np.array(a, copy=True) if s["t"] == "arr" else None for a, s in zip(args, spec)]
            r = fn(*args)
            for a, s, b0 in zip(args, spec, before):
                if s["t"] == "arr" and not np.array_equal(np.asarray(a), b0, equal_nan=True):
                    s["out"] = s["key"] + "_out"
                    arrays[s["out"]] = np.array(a, copy=True)
            calls.append({"name": name, "args": spec})
            return r
        return wrapped

    saved = {}
    for n in OPT_NAMES:
        saved[(cy, n)] = getattr(cy, n)
        setattr(cy, n, recorder(n, getattr(cy, n)))
    for n in OPT_TRANSFORMS:
        saved[(tr, n)] = getattr(tr, n)
        setattr(tr, n, recorder("transforms." + n, getattr(tr, n)))
    try:
        # banded solvers through the reference's own classes (la.py:291-800)
        kinds = {"TDMA": (-2, 0, 2), "PDMA": (-4, -2, 0, 2, 4), "FDMA": (-2, 0, 2, 4), "TwoDMA": (0, 2),
                 "ThreeDMA": (0, 2, 4), "HeptaDMA": (-4, -2, 0, 2, 4, 6, 8), "TDMA_O": (-1, 0, 1)}
        for name, offs in kinds.items():
            n = 14
            diags = {o: (4.0 + g.uniform(0, 1, n - abs(o))) if o == 0 else g.uniform(-0.5, 0.5, n - abs(o))
                     for o in offs}
            for ax, shape in ((0, (n, 3)), (1, (4, n))):
                sol = getattr(la, name)(SparseMatrix(dict(diags), (n, n)))
                b = g.standard_normal(shape) + 1j * g.standard_normal(shape)
                sol(b.copy(), axis=ax)
        # the reference's DiagMA solve takes 1D right-hand sides only
        n = 14
        sol = la.DiagMA(SparseMatrix({0: 2.0 + g.uniform(0, 1, n)}, (n, n)))
        sol(g.standard_normal(n) + 1j * g.standard_normal(n), axis=0)
        # Chebyshev Dirichlet / Neumann Helmholtz (chebyshev/la.py:131-351)
        for basis, bc in (("SD", (0, 0)), ("SN", {"left": ("N", 0), "right": ("N", 0)})):
            F0 = FunctionSpace(6, "F", dtype="D")
            F1 = FunctionSpace(6, "F", dtype="d")
            C = FunctionSpace(16, "C", bc=bc)
            T = TensorProductSpace(comm, (F0, F1, C))
            u, v = TrialFunction(T), TestFunction(T)
            mats = inner(v, -div(grad(u)) + 10 * u)
            H = chebyshev.la.Helmholtz(*mats)
            fh = Function(T, buffer=g.standard_normal(T.shape(True)) + 1j * g.standard_normal(T.shape(True)))
            H(fh.copy(), Function(T))
            if basis == "SD":
                H.matvec(fh.copy(), Function(T))
        # Chebyshev biharmonic (chebyshev/la.py:354-558), even N
        F0 = FunctionSpace(6, "F", dtype="D")
        F1 = FunctionSpace(6, "F", dtype="d")
        SB = FunctionSpace(20, "C", bc=(0, 0, 0, 0))
        T = TensorProductSpace(comm, (F0, F1, SB))
        u, v = TrialFunction(T), TestFunction(T)
        mats = inner(v, div(grad(div(grad(u)))) + 5 * div(grad(u)) + 3 * u)
        Hb = chebyshev.la.Biharmonic(*mats)
        fh = Function(T, buffer=g.standard_normal(T.shape(True)) + 1j * g.standard_normal(T.shape(True)))
        Hb(fh.copy(), Function(T))
        Hb.matvec(fh.copy(), Function(T))
        # SolverGeneric1ND on Fourier x Legendre (la.py:1183-1434): one TDMA /
        # PDMA per wavenumber through SolverGeneric1ND_solve_data
        for bc in ((0, 0), (0, 0, 0, 0)):
            F0 = FunctionSpace(6, "F", dtype="D")
            L = FunctionSpace(18, "L", bc=bc)
            T = TensorProductSpace(comm, (F0, L))
            u, v = TrialFunction(T), TestFunction(T)
            op = -div(grad(u)) + u if len(bc) == 2 else div(grad(div(grad(u)))) + u
            S = la.SolverGeneric1ND(inner(v, op))
            fh = Function(T, buffer=g.standard_normal(T.shape(True)) + 1j * g.standard_normal(T.shape(True)))
            S(fh.copy(), Function(T))
        # recursive Legendre transforms (spectralbase.py:485-491, 551-558)
        for N, bc in ((12, None), (17, (0, 0))):
            L = FunctionSpace(N, "L", bc=bc) if bc else FunctionSpace(N, "L")
            fj = g.standard_normal(N)
            L.scalar_product(fj, np.zeros(N), kind="recursive")
            L.backward(g.standard_normal(N), np.zeros(N), kind="recursive")
    finally:
        for (mod, n), fn in saved.items():
            setattr(mod, n, fn)
    arrays["manifest"] = np.array(json.dumps(calls))
    put("optmode", **arrays)
    print("optmode:", len(calls), "calls:", sorted({c["name"] for c in calls}))


# --------------------------------------------------------------------------
# project of Functions and of expressions (forms/project.py:124-199), linear
# forms of expressions (forms/inner.py:483-497), and SpectralMatrix.solve
# through get_solver (matrixbase.py:410-474).  Own rng.
def project_group():
    from shenfun import project
    g = np.random.default_rng(515)
    d = {}

    def fn(space, ndof):
        uh = Function(space)
        uh[:ndof] = g.standard_normal(ndof)
        return uh

    SD = FunctionSpace(14, "C", bc=(0, 0))
    SB = FunctionSpace(16, "C", bc=(0, 0, 0, 0))
    SN = FunctionSpace(14, "C", bc={"left": {"N": 0}, "right": {"N": 0}})
    T14, T16 = FunctionSpace(14, "C"), FunctionSpace(16, "C")
    u = fn(SD, 12)
    d.update(sd_u=u, sd_dx_T=project(Dx(u, 0, 1), T14), sd_dxx_SD=project(Dx(u, 0, 2), SD),
             sd_u_T=project(u, T14), sd_lap_T=project(div(grad(u)), T14),
             sd_inner_dxx=inner(TestFunction(SD), Dx(u, 0, 2)), sd_inner_u_T=inner(TestFunction(T14), u))
    ub = fn(SB, 12)
    d.update(sb_u=ub, sb_d3_T=project(Dx(ub, 0, 3), T16), sb_lap_SB=project(div(grad(ub)), SB))
    un = fn(SN, 12)
    d.update(sn_u=un, sn_dx_T=project(Dx(un, 0, 1), T14))
    LSD, L14 = FunctionSpace(14, "L", bc=(0, 0)), FunctionSpace(14, "L")
    ul = fn(LSD, 12)
    d.update(l_u=ul, l_dx_L=project(Dx(ul, 0, 1), L14), l_dxx_SD=project(Dx(ul, 0, 2), LSD))
    F0 = FunctionSpace(6, "F", dtype="D")
    F1 = FunctionSpace(8, "F", dtype="d")
    T3 = TensorProductSpace(comm, (F0, F1, SD))
    T3o = TensorProductSpace(comm, (F0, F1, T14))
    u3 = Function(T3)
    u3[..., :12] = g.standard_normal(u3[..., :12].shape) + 1j * g.standard_normal(u3[..., :12].shape)
    d.update(t3_u=u3, t3_dz_T=project(Dx(u3, 2, 1), T3o), t3_lap=project(div(grad(u3)), T3),
             t3_mix=project(Dx(u3, 0, 1) + 2 * Dx(u3, 1, 2), T3),
             t3_inner_lap=inner(TestFunction(T3), div(grad(u3))))
    FF = TensorProductSpace(comm, (F0, F1))
    uf = Function(FF, buffer=g.standard_normal(FF.shape(True)) + 1j * g.standard_normal(FF.shape(True)))
    d.update(ff_u=uf, ff_d=project(Dx(uf, 1, 1) - Dx(uf, 0, 2), FF))
    # SpectralMatrix.solve through get_solver
    for name, space in (("csd", SD), ("csb", SB), ("csn", SN), ("lsd", LSD)):
        v, w = TestFunction(space), TrialFunction(space)
        forms = {"B": inner(v, w), "A": inner(v, div(grad(w)))}
        if name == "csb":
            forms["S"] = inner(v, div(grad(div(grad(w)))))
        for key, mat in forms.items():
            N = space.N
            for shape, ax in (((N,), 0), ((N, 3), 0), ((4, N), 1)):
                b = g.standard_normal(shape) + 1j * g.standard_normal(shape)
                cons = ((0, 0),) if (name == "csn" and key == "A") else ()
                try:
                    x = mat.solve(b.copy(), axis=ax, constraints=cons) if cons else mat.solve(b.copy(), axis=ax)
                except Exception:
                    continue
                tag = f"ms_{name}{key}_{len(shape)}d{ax}"
                d.update({tag + "_b": b, tag + "_x": np.array(x)})
                d[tag + "_solver"] = np.array(type(mat.solver).__name__)
                mat.solver = None
    put("project", **d)


GROUPS = {"cheb_1d": cheb_1d, "fourier_1d": fourier_1d, "banded": banded, "helmholtz": helmholtz,
          "roundtrips": roundtrips, "biharmonic": biharmonic, "legendre": legendre, "imex": imex,
          "dealias": dealias, "neumann": neumann,
          "nonhomog": nonhomog, "dma": dma, "optmode": optmode,
          "project": project_group}

if __name__ == "__main__":
    # no arguments: every group (the shared rng makes the earlier groups depend
    # on their order); with names: only those groups (those with their own rng
    # reproduce exactly)
    for name in (sys.argv[1:] or list(GROUPS)):
        GROUPS[name]()
    save()
