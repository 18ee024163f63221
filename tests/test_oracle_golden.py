"""Pin the CPU oracle against fixtures recorded from the unmodified reference
(tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from oracle import spectral as S, la, problems as P

TOL = 1e-13


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("N", [8, 9, 16, 17, 33, 64])
@pytest.mark.parametrize("tag", ["T", "SD", "SB"])
def test_chebyshev_1d(golden, N, tag):
    d = golden("cheb_1d")
    if f"{tag}{N}_f" not in d:
        pytest.skip("not recorded")
    f = d[f"{tag}{N}_f"]
    assert rel(S.cheb_scalar_product(f, tag), d[f"{tag}{N}_sp"]) < TOL
    assert rel(S.cheb_forward(f, tag), d[f"{tag}{N}_fw"]) < TOL
    assert rel(S.cheb_backward(d[f"{tag}{N}_uh"], tag), d[f"{tag}{N}_bw"]) < TOL
    assert rel(S.cheb_gc_points_weights(N)[0], d[f"{tag}{N}_x"]) < TOL


@pytest.mark.parametrize("N", [8, 9, 16, 64])
def test_fourier_1d(golden, N):
    d = golden("fourier_1d")
    assert rel(S.r2c_forward(d[f"R{N}_f"]), d[f"R{N}_fw"]) < TOL
    assert rel(S.r2c_backward(d[f"R{N}_uh"], N), d[f"R{N}_bw"]) < TOL
    assert rel(S.c2c_forward(d[f"C{N}_f"]), d[f"C{N}_fw"]) < TOL
    assert rel(S.c2c_backward(d[f"C{N}_uh"]), d[f"C{N}_bw"]) < TOL
    assert np.array_equal(S.r2c_wavenumbers(N), d[f"R{N}_k"])
    assert np.array_equal(S.c2c_wavenumbers(N), d[f"C{N}_k"])


@pytest.mark.parametrize("N", [16, 17, 32])
def test_tdma_pdma(golden, N):
    d = golden("banded")
    lu = la.tdma_lu(d[f"tdma{N}_raw"].copy())
    assert rel(lu, d[f"tdma{N}_lu"]) < TOL
    assert rel(la.tdma_solve(d[f"tdma{N}_b1"], lu), d[f"tdma{N}_x1"]) < TOL
    assert rel(la.tdma_solve(d[f"tdma{N}_b2"], lu), d[f"tdma{N}_x2"]) < TOL
    assert rel(la.tdma_solve(d[f"tdma{N}_b3"], lu, axis=1), d[f"tdma{N}_x3"]) < TOL
    lu = la.pdma_lu(d[f"pdma{N}_raw"].copy())
    assert rel(lu, d[f"pdma{N}_lu"]) < TOL
    assert rel(la.pdma_solve(d[f"pdma{N}_b1"], lu), d[f"pdma{N}_x1"]) < TOL
    assert rel(la.pdma_solve(d[f"pdma{N}_b2"], lu), d[f"pdma{N}_x2"]) < TOL


@pytest.mark.parametrize("shape", [(8, 8, 17, 1000.0), (6, 4, 16, 0.0), (4, 6, 33, 50.0)])
def test_helmholtz(golden, shape):
    Nx, Ny, Nz, c = shape
    d = golden("helmholtz")
    k = f"h{Nx}x{Ny}x{Nz}"
    bases = [("fourier", "C2C", Nx), ("fourier", "R2C", Ny), ("chebyshev", "SD", Nz)]
    assert np.all(d[k + "_alfa"] == -1.0)
    assert rel(P.fourier_k2(bases, 2) + c, d[k + "_beta"]) == 0.0
    d0, d1, d2, L = la.helmholtz_lu(Nz, d[k + "_alfa"].reshape(-1), d[k + "_beta"].reshape(-1))
    for name, arr in (("_d0", d0), ("_d1", d1), ("_d2", d2), ("_L", L)):
        assert rel(arr, d[k + name].reshape(-1, Nz)) < TOL
    u = la.helmholtz_solve(d[k + "_f"].reshape(-1, Nz), d0, d1, d2, L)
    assert rel(u, d[k + "_u"].reshape(-1, Nz)) < TOL
    mv = la.helmholtz_matvec(d[k + "_u"].reshape(-1, Nz), d[k + "_alfa"].reshape(-1),
                             d[k + "_beta"].reshape(-1))
    assert rel(mv, d[k + "_mv"].reshape(-1, Nz)) < TOL


def test_helmholtz_solve_axis0(golden):
    d = golden("helmholtz")
    f = np.moveaxis(d["h2d_f"], 0, -1)
    d0, d1, d2, L = la.helmholtz_lu(20, d["h2d_alfa"].reshape(-1), d["h2d_beta"].reshape(-1))
    assert rel(d0, np.moveaxis(d["h2d_d0"], 0, -1)) < TOL
    u = la.helmholtz_solve(f, d0, d1, d2, L)
    assert rel(u, np.moveaxis(d["h2d_u"], 0, -1)) < TOL


def test_cfg1_poisson2d(golden):
    d = golden("cfg1_poisson2d")
    bases = [("fourier", "R2C", 64), ("chebyshev", "SD", 64)]
    assert rel(P.scalar_product(d["fj"], bases, axes=(1, 0)), d["f_hat"]) < TOL
    assert rel(P.helmholtz_solve(d["f_hat"], bases, 0.0, 1), d["u_hat"]) < TOL
    assert rel(P.backward(d["u_hat"], bases, axes=(1, 0)), d["uq"]) < TOL
    assert rel(P.forward(d["uj"], bases, axes=(1, 0)), d["fw"]) < TOL
    assert np.abs(d["uq"] - d["uj"]).max() < 1e-12   # manufactured solution


@pytest.mark.parametrize("shape", [(8, 8, 17), (16, 12, 24)])
def test_cfg2_roundtrip(golden, shape):
    d = golden("cfg2_%dx%dx%d" % shape)
    bases = [("fourier", "C2C", shape[0]), ("fourier", "R2C", shape[1]), ("chebyshev", "SD", shape[2])]
    u, fh, uh = P.helmholtz_roundtrip(d["fj"], bases, 1000.0, 2)
    assert rel(fh, d["f_hat"]) < TOL
    assert rel(uh, d["u_hat"]) < TOL
    assert rel(u, d["uq"]) < TOL
    fw = P.forward(d["fj"], bases)
    assert rel(fw, d["fw"]) < TOL
    assert rel(P.backward(d["fw"], bases), d["fwbw"]) < TOL


@pytest.mark.parametrize("Nz", [16, 17])
def test_biharmonic(golden, Nz):
    d = golden(f"biharmonic_8x8x{Nz}")
    bases = [("fourier", "C2C", 8), ("fourier", "R2C", 8), ("chebyshev", "SB", Nz)]
    assert rel(P.scalar_product(d["fj"], bases), d["f_hat"]) < TOL
    uh = P.biharmonic_solve(d["f_hat"], bases, 2)
    assert rel(uh, d["u_hat_generic"]) < 1e-12
    assert rel(P.backward(uh, bases), d["uq"]) < 1e-12
    if "u_hat_biharmonic" in d:
        assert rel(uh, d["u_hat_biharmonic"]) < 1e-12


@pytest.mark.parametrize("N", [4, 8, 16, 33, 100])
def test_legendre_nodes(golden, N):
    d = golden("legendre")
    x, w = S.leg_lg_points_weights(N)
    assert rel(x, d[f"xw{N}_x"]) < 1e-15
    assert rel(w, d[f"xw{N}_w"]) < 1e-13


@pytest.mark.parametrize("N", [16, 33, 64])
@pytest.mark.parametrize("kind", ["recursive", "vandermonde"])
def test_legendre_1d(golden, N, kind):
    d = golden("legendre")
    for tag, b in (("L", "L"), ("LD", "SD")):
        assert rel(S.leg_scalar_product(d[f"{tag}{N}_f"], b, kind=kind), d[f"{tag}{N}_sp_{kind}"]) < 1e-13
        assert rel(S.leg_backward(d[f"{tag}{N}_uh"], b, kind=kind), d[f"{tag}{N}_bw_{kind}"]) < 1e-14
        assert rel(S.leg_forward(d[f"{tag}{N}_f"], b, kind=kind), d[f"{tag}{N}_fw_{kind}"]) < 1e-12


def test_legendre_poisson2d(golden):
    d = golden("legendre")
    bases = [("fourier", "R2C", 16), ("legendre", "SD", 24)]
    assert rel(P.scalar_product(d["p2d_fj"], bases, axes=(1, 0)), d["p2d_fhat"]) < 1e-13
    beta = P.fourier_k2(bases, 1) + 3.0
    fs, shp = P._systems(d["p2d_fhat"], 1)
    us = la.leg_helmholtz_solve(fs, np.ones(fs.shape[0]), beta.reshape(-1))
    assert rel(np.moveaxis(us.reshape(shp), -1, 1), d["p2d_uhat"]) < 1e-13


@pytest.mark.parametrize("name", ["IMEXRK111", "IMEXRK222", "IMEXRK443"])
def test_imex_oracle(golden, name):
    """IMEX Runge-Kutta steps of u_t = nu lap(u) + f on C2C x R2C x SD
    (utilities/integrators.py:702-900) against the reference's own run."""
    from oracle import imex
    d = golden("imex")
    bases = [("fourier", "C2C", 8), ("fourier", "R2C", 8), ("chebyshev", "SD", 17)]
    out = imex.imex_run(d["u_hat0"], d["f_hat"], float(d["nu"]), float(d["dt"]), name, 3, bases, 2)
    for step in range(3):
        ref = d[f"{name}_step{step}"]
        assert np.abs(out[step] - ref).max() / np.abs(ref).max() < 1e-13


@pytest.mark.parametrize("shape", [(8, 8, 17), (9, 7, 12)])
def test_dealias_oracle(golden, shape):
    """Padded (3/2-rule) Fourier transforms (get_dealiased((1.5, 1.5, 1)))
    against the reference: backward onto the padded grid, forward and scalar
    product from it, even and odd Fourier lengths."""
    from oracle import dealias as D
    d = golden("dealias")
    tag = "%dx%dx%d" % shape
    bases = [("fourier", "C2C", shape[0]), ("fourier", "R2C", shape[1]), ("chebyshev", "SD", shape[2])]
    fac = (1.5, 1.5, 1)
    up = D.padded_backward(d[f"{tag}_u_hat"], bases, fac)
    assert np.abs(up - d[f"{tag}_padded_backward"]).max() < 1e-13 * np.abs(up).max()
    fh = D.padded_forward(d[f"{tag}_padded_in"], bases, fac)
    assert np.abs(fh - d[f"{tag}_padded_forward"]).max() < 1e-13 * np.abs(fh).max()
    sh = D.padded_forward(d[f"{tag}_padded_in"], bases, fac, scalar=True)
    assert np.abs(sh - d[f"{tag}_padded_scalar"]).max() < 1e-13 * np.abs(sh).max()


# --------------------------------------------------------------------------
# Chebyshev ShenNeumann and the Poisson solvers (neumann.npz)
@pytest.mark.parametrize("N", [8, 9, 16, 17, 33])
def test_shen_neumann_1d(golden, N):
    d = golden("neumann")
    f = d[f"sn{N}_f"]
    assert rel(S.cheb_scalar_product(f, "SN"), d[f"sn{N}_sp"]) < TOL
    assert rel(S.cheb_forward(f, "SN"), d[f"sn{N}_fw"]) < TOL
    assert rel(S.cheb_backward(d[f"sn{N}_uh"], "SN"), d[f"sn{N}_bw"]) < TOL


@pytest.mark.parametrize("N", [16, 17])
def test_shen_neumann_matrices(golden, N):
    A, B = la.cheb_sn_dense(N)
    d = golden("neumann")
    assert rel(A, d[f"snA{N}"]) < TOL
    assert rel(B, d[f"snB{N}"]) < TOL


@pytest.mark.parametrize("key", ["h6x4x16", "h4x6x17", "h8x8x33"])
def test_helmholtz_neumann(golden, key):
    d = golden("neumann")
    f = d[key + "_f"]
    N = f.shape[-1]
    sys = f.shape[:-1] + (1,)
    alfa = np.broadcast_to(d[key + "_alfa"], sys).reshape(-1)
    beta = np.broadcast_to(d[key + "_beta"], sys).reshape(-1)
    fac = la.helmholtz_lu(N, alfa, beta, neumann=True)
    for got, name in zip(fac, ("_d0", "_d1", "_d2", "_L")):
        assert np.array_equal(got, d[key + name].reshape(-1, N))  # bit-exact LU
    u = la.helmholtz_solve(f.reshape(-1, N), *fac, neumann=True)
    assert rel(u, d[key + "_u"].reshape(-1, N)) < TOL
    # the definition of the matvec undoes the solve (zero mode excluded)
    mv = la.helmholtz_neumann_matvec(u, alfa, beta)
    reg = np.abs(beta) >= 1e-8
    assert rel(mv[reg, :N - 2], f.reshape(-1, N)[reg, :N - 2]) < 1e-11


@pytest.mark.parametrize("N", [16, 17, 32])
def test_poisson_add_ann(golden, N):
    d = golden("neumann")
    u = la.add_solve(d[f"add{N}_b"], d[f"add{N}_A0"], d[f"add{N}_A2"], float(d[f"add{N}_scale"]))
    assert rel(u, d[f"add{N}_u"]) < TOL
    u = la.ann_solve(d[f"ann{N}_b"], d[f"ann{N}_A0"], d[f"ann{N}_A2"], float(d[f"ann{N}_scale"]))
    assert rel(u, d[f"ann{N}_u"]) < TOL


@pytest.mark.parametrize("axis", [0, 1])
def test_poisson_add_2d(golden, axis):
    d = golden("neumann")
    A = la.cheb_sd_stiffness(20)
    u = la.add_solve(d[f"add2d{axis}_b"], A[0], A[2], 1.0, axis=axis)
    ref = d[f"add2d{axis}_u"]
    sl = [slice(None)] * 2
    sl[axis] = slice(0, 18)  # the compiled kernel writes the dofs only
    assert rel(u[tuple(sl)], ref[tuple(sl)]) < TOL


# --------------------------------------------------------------------------
# non-homogeneous boundary values (nonhomog.npz)
BCV = {"SD": (1.5, -0.5), "SN": (0.7, -0.3)}


def _nh_bases(tag, shape):
    if len(shape) == 3:
        return [("fourier", "C2C", shape[0]), ("fourier", "R2C", shape[1]), ("chebyshev", tag, shape[2])], 2
    return [("chebyshev", tag, shape[0]), ("fourier", "R2C", shape[1])], 0


@pytest.mark.parametrize("tag", ["SD", "SN"])
@pytest.mark.parametrize("N", [12, 17])
def test_nonhomog_1d(golden, tag, N):
    from oracle import bcs as BC
    d = golden("nonhomog")
    f = d[f"{tag}{N}_f"]
    assert rel(S.cheb_scalar_product(f, tag), d[f"{tag}{N}_sp"]) < TOL
    assert rel(BC.forward_1d(f, tag, np.array(BCV[tag])), d[f"{tag}{N}_fw"]) < TOL
    assert rel(BC.backward_1d(d[f"{tag}{N}_uh"], tag), d[f"{tag}{N}_bw"]) < TOL


@pytest.mark.parametrize("tag", ["SD", "SN"])
@pytest.mark.parametrize("shape", [(8, 6, 17), (16, 6)])
def test_nonhomog_tensor(golden, tag, shape):
    from oracle import bcs as BC
    d = golden("nonhomog")
    key = tag + "_" + "x".join(str(n) for n in shape)
    bases, ax = _nh_bases(tag, shape)
    f = d[key + "_f"]
    assert rel(BC.tp_forward(f, bases, BCV[tag], ax), d[key + "_fw"]) < TOL
    assert rel(P.scalar_product(f, bases), d[key + "_sp"]) < TOL
    assert rel(BC.tp_backward(d[key + "_uh"], bases, ax), d[key + "_bw"]) < TOL
    sol = BC.helmholtz_bc_solve(d[key + "_rhs"], bases, 5.0, ax, BCV[tag])
    assert rel(sol, d[key + "_sol"]) < TOL
    assert rel(BC.tp_backward(sol, bases, ax), d[key + "_solx"]) < TOL


# --------------------------------------------------------------------------
# DiagMA / TwoDMA / ThreeDMA / FDMA / HeptaDMA (dma.npz)
DMA_OFFSETS = {"DiagMA": (0,), "TwoDMA": (0, 2), "ThreeDMA": (0, 2, 4), "FDMA": (-2, 0, 2, 4),
               "HeptaDMA": (-4, -2, 0, 2, 4, 6, 8)}


def dma_data(D, offsets):
    n = D.shape[0]
    data = np.zeros((len(offsets), n))
    for r, o in enumerate(offsets):
        for i in range(n):
            if 0 <= i + o < n:
                data[r, i + o] = D[i, i + o]
    return data


@pytest.mark.parametrize("name", sorted(DMA_OFFSETS))
@pytest.mark.parametrize("n", [12, 17])
def test_banded_solvers(golden, name, n):
    d = golden("dma")
    offs = DMA_OFFSETS[name]
    keys = [k[:-2] for k in d if k.startswith(f"{name}{n}_") and k.endswith("_b")]
    assert keys
    for key in keys:
        data = dma_data(d[f"{name}{n}_dense"], offs)
        if name == "ThreeDMA":
            data = la.threedma_effective(data)
        la.banded_lu(data, offs)
        u = la.banded_solve(d[key + "_b"], data, offs, axis=int(key[-1]))
        assert rel(u, d[key + "_u"]) < TOL
