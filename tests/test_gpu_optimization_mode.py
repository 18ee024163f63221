"""The gb300 optimization mode on the GPU, called the way the reference's own
classes call its compiled kernels.

* Every kernel-dispatch call recorded from the unmodified reference
  (la.TDMA/PDMA/FDMA/TwoDMA/ThreeDMA/HeptaDMA/TDMA_O/DiagMA,
  chebyshev.la.Helmholtz (Dirichlet and Neumann), chebyshev.la.Biharmonic,
  la.SolverGeneric1ND on Fourier x Legendre, the recursive Legendre
  transforms) is replayed through ``shenfun_gb300.optimization`` with the
  recorded arguments, as numpy arrays (the adapter copies them) and as CUDA
  tensors (in place); what each call writes must match the reference's.
* At sizes past the fixtures the C-ABI entry points are compared with the
  oracle restatements, along every axis layout, and the biharmonic chain is
  checked by a size-independent property: the matvec of the solution gives
  back the right-hand side.
"""
import numpy as np
import pytest
import torch

import optmode_replay as R
from oracle import refabi as RA

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _resolve(rec):
    import shenfun_gb300.optimization as opt
    import shenfun_gb300.optimization.transforms as tr
    if rec.name.startswith("transforms."):
        return getattr(tr, rec.name.split(".", 1)[1])
    return getattr(opt, rec.name)


def _fix_fn_args(rec):
    import shenfun_gb300.optimization as opt
    if rec.name == "SolverGeneric1ND_solve_data":
        rec.args[2] = getattr(opt, rec.args[2])
    return rec


RECORDS = R.calls()


@pytest.mark.parametrize("device", [False, True], ids=["numpy", "cuda"])
@pytest.mark.parametrize("i", range(len(RECORDS)), ids=[f"{i}-{r.name}" for i, r in enumerate(RECORDS)])
def test_replay_reference_dispatch(i, device):
    rec = _fix_fn_args(R.calls(device=device)[i])
    _resolve(rec)(*rec.args)
    torch.cuda.synchronize()
    errs = rec.rel_errors()
    assert errs
    for j, e in errs.items():
        assert e < TOL, (rec.name, j, e)


def test_whole_reference_sequences_on_device_tensors():
    """The recorded sequences in order on CUDA tensors: LU_Biharmonic ->
    Biharmonic_factor_pr -> Biharmonic_Solve with the device factors the
    earlier calls produced (not the recorded ones)."""
    import shenfun_gb300.optimization as opt
    recs = {r.name: r for r in R.calls(device=True)}
    lu, pr, sv = recs["LU_Biharmonic"], recs["Biharmonic_factor_pr"], recs["Biharmonic_Solve"]
    u0, u1, u2, l0, l1 = [torch.zeros_like(t) for t in lu.args[14:19]]
    opt.LU_Biharmonic(*lu.args[:14], u0, u1, u2, l0, l1, lu.args[19])
    ak, bk = torch.zeros_like(u0), torch.zeros_like(u0)
    opt.Biharmonic_factor_pr(ak, bk, l0, l1, pr.args[4])
    b = sv.args[0]
    u = torch.zeros_like(b)
    opt.Biharmonic_Solve(b, u, u0, u1, u2, l0, l1, ak, bk, sv.args[9], sv.args[10])
    ref = sv.outputs[1]
    got = u.cpu().numpy()
    assert np.abs(got - ref).max() / np.abs(ref).max() < TOL


# ---- beyond the fixtures: the C ABI against the oracle ------------------------
def _cheb_sb_diags(N):
    """sii, siu, siuu, ail, aii, aiu, bill, bil, bii, biu, biuu of the
    Chebyshev biharmonic SBB / ABB / BBB matrices (chebyshev/matrices.py)."""
    from shenfun_gb300 import matrices as MM
    S, A, B = MM.cheb_sb_S(N), MM.cheb_sb_A(N), MM.cheb_sb_B(N)
    n = N - 4
    k = np.arange(n, dtype=float)
    row = lambda i, j: 8 * (k[i] + 1) * (k[i] + 2) * (k[i] * (k[i] + 4) + 3 * (k[j] + 2) ** 2) * np.pi / (k[j] + 3)  # noqa: E731
    siu = np.array([row(i, i + 2) for i in range(n - 2)])
    siuu = np.array([row(i, i + 4) for i in range(n - 4)])
    return [np.asarray(S[0]), siu, siuu, A[-2], A[0], A[2], B[-4], B[-2], B[0], B[2], B[4]]


def test_cheb_sb_diagonals_match_the_recorded_reference():
    rec = R.calls(names={"LU_Biharmonic"})[0]
    N = 2 * rec.args[14].shape[-1] + 4
    for q, (mine, ref) in enumerate(zip(_cheb_sb_diags(N), rec.args[3:14])):
        assert np.allclose(mine, ref, rtol=1e-14, atol=0), q


@pytest.mark.parametrize("shape,axis", [((12, 7, 130), 2), ((66, 5, 3), 0), ((4, 98, 6), 1)])
def test_biharmonic_chain_against_oracle_and_matvec(shape, axis):
    import shenfun_gb300.optimization as opt
    g = np.random.default_rng(sum(shape))
    N = shape[axis]
    M = (N - 4) // 2
    diags = _cheb_sb_diags(N)
    sys_shape = list(shape)
    sys_shape[axis] = 1
    kk = g.uniform(0, 30, sys_shape)
    alfa, beta, a0 = -2 * kk, kk ** 2, 1.0
    fshape = [2] + list(shape)
    fshape[axis + 1] = M
    fac = [torch.zeros(fshape, dtype=torch.float64, device="cuda") for _ in range(7)]
    opt.LU_Biharmonic(a0, alfa, beta, *diags, *fac[:5], axis)
    opt.Biharmonic_factor_pr(fac[5], fac[6], fac[3], fac[4], axis)
    ref = [np.zeros(fshape) for _ in range(7)]
    RA.lu_biharmonic(a0, alfa, beta, *diags, *ref[:5], axis=axis)
    RA.biharmonic_factor_pr(ref[5], ref[6], ref[3], ref[4], axis=axis)
    for q in range(7):
        got = fac[q].cpu().numpy()
        assert np.abs(got - ref[q]).max() <= 1e-12 * np.abs(ref[q]).max(), q
    f = g.standard_normal(shape) + 1j * g.standard_normal(shape)
    sl = [slice(None)] * 3
    sl[axis] = slice(2 * M, None)
    f[tuple(sl)] = 0
    fd = torch.from_numpy(f).cuda()
    u = torch.zeros_like(fd)
    opt.Biharmonic_Solve(fd, u, *fac, a0, axis)
    uo = np.zeros_like(f)
    RA.biharmonic_solve(f, uo, *ref, a0, axis=axis)
    un = u.cpu().numpy()
    assert np.abs(un - uo).max() <= 1e-11 * np.abs(uo).max()
    # size-independent: (a0 S + alfa A + beta B) u reproduces f on the dofs
    b = torch.zeros_like(fd)
    opt.Biharmonic_matvec(u, b, a0, alfa, beta, *diags[:3], *diags[3:], axis)
    bn = b.cpu().numpy()
    sl[axis] = slice(0, 2 * M)
    assert np.abs(bn[tuple(sl)] - f[tuple(sl)]).max() <= 1e-10 * np.abs(f).max()


@pytest.mark.parametrize("kind,rows", [("TDMA", 3), ("PDMA", 5), ("FDMA", 4), ("HeptaDMA", 7), ("TDMA_O", 3),
                                       ("ThreeDMA", 3), ("TwoDMA", 2), ("DiagMA", 1)])
@pytest.mark.parametrize("naxes", [0, 1, 2])
def test_solve_data_layouts(kind, rows, naxes):
    import shenfun_gb300.optimization as opt
    g = np.random.default_rng(rows * 10 + naxes)
    shape = [9, 10, 11]
    shape[naxes] = 40
    cols = 38
    others = [s for a, s in enumerate(shape) if a != naxes]
    data = g.uniform(-0.3, 0.3, others + [rows, cols])
    mid = {"DiagMA": 0, "TwoDMA": 0, "ThreeDMA": 0, "TDMA": 1, "TDMA_O": 1, "PDMA": 2, "FDMA": 1,
           "HeptaDMA": 2}[kind]
    data[..., mid, :] = 2.0 + g.uniform(0, 1, others + [cols])
    u = g.standard_normal(shape) + 1j * g.standard_normal(shape)
    ud = torch.from_numpy(u).cuda()
    opt.SolverGeneric1ND_solve_data(ud, data, getattr(opt, kind + "_inner_solve"), naxes, True)
    ref = u.copy()
    RA.solve_data(ref, data, kind, naxes, True)
    got = ud.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    s0 = [0, 0, 0]
    s0[naxes] = slice(None)
    assert np.array_equal(got[tuple(s0)], u[tuple(s0)])  # system 0 skipped


@pytest.mark.parametrize("N,bc", [(64, None), (129, (0, 0)), (300, None)])
@pytest.mark.parametrize("axis", [0, 1])
def test_recursive_legendre_against_oracle(N, bc, axis):
    import shenfun_gb300.optimization.transforms as tr
    from shenfun_gb300.legendre import leggauss
    g = np.random.default_rng(N + axis)
    x, w = leggauss(N)
    k = np.arange(N + 3, dtype=float)
    a = np.zeros((2, N + 3))
    a[0] = (k + 1) / (2 * k + 1)
    a[1] = k / (2 * k + 1)
    shape = (N, 7) if axis == 0 else (5, N)
    fj = g.standard_normal(shape) + 1j * g.standard_normal(shape)
    out = torch.zeros(shape, dtype=torch.complex128, device="cuda")
    tr.scalar_product(torch.from_numpy(fj).cuda(), out, x, w, axis, a)
    ref = np.zeros_like(fj)
    RA.scalar_product(fj, ref, x, w, axis, a)
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-12 * np.abs(ref).max()
    c = g.standard_normal(shape) / (1 + np.arange(N)).reshape((-1, 1) if axis == 0 else (1, -1))
    out2 = np.zeros(shape)
    tr.evaluate_expansion_all(c, out2, x, axis, a)
    ref2 = np.zeros(shape)
    RA.evaluate_expansion_all(c, ref2, x, axis, a)
    assert np.abs(out2 - ref2).max() <= 1e-12 * np.abs(ref2).max()
