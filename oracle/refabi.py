"""CPU restatement of the reference kernels behind the reference-signature
entry points: the Chebyshev biharmonic LU / factor / solve / matvec, the
banded *_inner_solve kernels SolverGeneric1ND_solve_data dispatches to, and
the recursive Legendre scalar product / evaluation.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Each function follows the cited Cython loop step for step (the biharmonic LU
eliminates whole rows, O(M^2) per system, as the reference does), vectorised
over the independent systems.  Citations are paths inside the reference
project (shenfun/optimization/cython/...).
"""
import numpy as np


def _sys(a, axis):
    """(..., M along axis, ...) -> (M, nsys) view order used below."""
    a = np.moveaxis(a, axis, -1)
    return a.reshape(-1, a.shape[-1]).T


def _unsys(flat, shape, axis):
    moved = list(shape)
    moved.append(moved.pop(axis))
    return np.moveaxis(flat.T.reshape(moved), -1, axis)


# ---------------------------------------------------------------------------
# Chebyshev biharmonic: la.pyx:975-1290
def lu_biharmonic_oe(odd, a, b, c, sii, siu, siuu, ail, aii, aiu, bill, bil, bii, biu, biuu, M):
    """la.pyx:1018-1125 (LU_oe_Biharmonic_1D) for the parity-`odd` diagonals
    (sii = full_sii[odd::2] etc.); b, c arrays over systems.  Returns u0, u1,
    u2, l0, l1 of shape (M, nsys)."""
    b = np.atleast_1d(np.asarray(b, dtype=float))
    c = np.atleast_1d(np.asarray(c, dtype=float))
    ns = max(b.size, c.size)
    b = np.broadcast_to(b, (ns,))
    c = np.broadcast_to(c, (ns,))
    pi = np.pi
    c0 = np.zeros((M, ns))
    c1 = np.zeros((M, ns))
    c2 = np.zeros((M, ns))
    u0, u1, u2, l0, l1 = (np.zeros((M, ns)) for _ in range(5))

    def mform(k, j):
        return 8 * (k + 1) * (k + 2) * (k * (k + 4) + 3 * (j + 2) * (j + 2))

    c0[0] = a * sii[0] + b * aii[0] + c * bii[0]
    c0[1] = a * siu[0] + b * aiu[0] + c * biu[0]
    c0[2] = a * siuu[0] + c * biuu[0]
    c0[3] = mform(odd, 6 + odd) * a * pi / (6 + odd + 3.)
    c0[4] = mform(odd, 8 + odd) * a * pi / (8 + odd + 3.)
    c1[0] = b * ail[0] + c * bil[0]
    c1[1] = a * sii[1] + b * aii[1] + c * bii[1]
    c1[2] = a * siu[1] + b * aiu[1] + c * biu[1]
    c1[3] = a * siuu[1] + c * biuu[1]
    c1[4] = mform(odd + 2, 8 + odd) * a * pi / (8 + odd + 3.)
    c2[0] = c * bill[0]
    c2[1] = b * ail[1] + c * bil[1]
    c2[2] = a * sii[2] + b * aii[2] + c * bii[2]
    c2[3] = a * siu[2] + b * aiu[2] + c * biu[2]
    c2[4] = a * siuu[2] + c * biuu[2]
    for i in range(5, M):
        j = 2 * i + odd
        c0[i] = mform(odd, j) * a * pi / (j + 3.)
        c1[i] = mform(odd + 2, j) * a * pi / (j + 3.)
        c2[i] = mform(odd + 4, j) * a * pi / (j + 3.)
    u0[0] = c0[0]
    u1[0] = c0[1]
    u2[0] = c0[2]
    for kk in range(1, M):
        l0[kk - 1] = c1[kk - 1] / u0[kk - 1]
        if kk < M - 1:
            l1[kk - 1] = c2[kk - 1] / u0[kk - 1]
        c1[kk:] = c1[kk:] - l0[kk - 1] * c0[kk:]
        if kk < M - 1:
            c2[kk:] = c2[kk:] - l1[kk - 1] * c0[kk:]
        c0[kk:] = c1[kk:]
        c1[kk:] = c2[kk:]
        if kk < M - 2:
            c2[kk] = c * bill[kk]
            c2[kk + 1] = b * ail[kk + 1] + c * bil[kk + 1]
            c2[kk + 2] = a * sii[kk + 2] + b * aii[kk + 2] + c * bii[kk + 2]
            if kk < M - 3:
                c2[kk + 3] = a * siu[kk + 2] + b * aiu[kk + 2] + c * biu[kk + 2]
            if kk < M - 4:
                c2[kk + 4] = a * siuu[kk + 2] + c * biuu[kk + 2]
            if kk < M - 5:
                k = 2 * (kk + 2) + odd
                for i in range(kk + 5, M):
                    j = 2 * i + odd
                    c2[i] = mform(k, j) * a * pi / (j + 3.)
        u0[kk] = c0[kk]
        if kk < M - 1:
            u1[kk] = c0[kk + 1]
        if kk < M - 2:
            u2[kk] = c0[kk + 2]
    return u0, u1, u2, l0, l1


def lu_biharmonic(a0, alfa, beta, sii, siu, siuu, ail, aii, aiu, bill, bil, bii, biu, biuu, u0, u1, u2, l0, l1,
                  axis=0):
    """la.pyx:975 LU_Biharmonic: fills the (2, ..., M, ...) factor arrays in place.

    Rows per parity: the 1D kernel (la.pyx:991-1016) factors the length of
    each parity's slice of sii; the 2D and 3D kernels (la.pyx:1651, 1950)
    factor len(sii) // 2 rows for both parities.  With an odd number of dofs
    the 2D/3D kernels therefore leave the last even row at zero (and the
    reference's solve then divides by it), which this restatement keeps."""
    shape = u0.shape[1:]
    M = shape[axis]
    sys_shape = list(shape)
    sys_shape[axis] = 1
    b = np.broadcast_to(np.asarray(alfa, dtype=float), sys_shape).reshape(-1)
    c = np.broadcast_to(np.asarray(beta, dtype=float), sys_shape).reshape(-1)
    diags = (sii, siu, siuu, ail, aii, aiu, bill, bil, bii, biu, biuu)
    nd = np.asarray(sii).shape[0]
    for odd in (0, 1):
        Mp = (nd - odd + 1) // 2 if len(shape) == 1 else nd // 2
        res = lu_biharmonic_oe(odd, float(a0), b, c, *[np.asarray(d)[odd::2] for d in diags], Mp)
        for arr, r in zip((u0, u1, u2, l0, l1), res):
            full = np.zeros((M, r.shape[1]))
            full[:Mp] = r
            arr[odd] = _unsys(full, shape, axis)


def biharmonic_factor_pr(ak, bk, l0, l1, axis=0):
    """la.pyx:1195-1233 Biharmonic_factor_pr (rows 0 .. M-3 per parity)."""
    shape = l0.shape[1:]
    M = shape[axis]
    for odd in (0, 1):
        L0, L1 = _sys(l0[odd], axis), _sys(l1[odd], axis)
        a = _sys(ak[odd], axis).copy()
        b = _sys(bk[odd], axis).copy()
        k = odd
        a[0] = 8 * k * (k + 1) * (k + 2) * (k + 4) * np.pi
        b[0] = 24 * (k + 1) * (k + 2) * np.pi
        k = 2 + odd
        a[1] = 8 * k * (k + 1) * (k + 2) * (k + 4) * np.pi - L0[0] * a[0]
        b[1] = 24 * (k + 1) * (k + 2) * np.pi - L0[0] * b[0]
        for k in range(2, M + 1 - 3):
            kk = 2 * k + odd
            pp = 8 * kk * (kk + 1) * (kk + 2) * (kk + 4)
            rr = 24 * (kk + 1) * (kk + 2)
            a[k] = pp * np.pi - L0[k - 1] * a[k - 1] - L1[k - 2] * a[k - 2]
            b[k] = rr * np.pi - L0[k - 1] * b[k - 1] - L1[k - 2] * b[k - 2]
        ak[odd] = _unsys(a, shape, axis)
        bk[odd] = _unsys(b, shape, axis)


def biharmonic_solve(b, u, u0, u1, u2, l0, l1, ak, bk, a0, axis=0):
    """la.pyx:1235-1290 Biharmonic_Solve: u[:2M] along axis; u[2M:] untouched."""
    M = u0.shape[1:][axis]
    fb = np.moveaxis(b, axis, 0)
    ub = np.moveaxis(u, axis, 0)
    y = np.zeros_like(fb[:2 * M])
    res = np.zeros_like(fb[:2 * M])
    for odd in (0, 1):
        U0, U1, U2, L0, L1, A, B = (np.moveaxis(x[odd], axis, 0) for x in (u0, u1, u2, l0, l1, ak, bk))
        f = fb[odd:2 * M:2]
        yy = y[odd::2]
        yy[0] = f[0]
        yy[1] = f[1] - L0[0] * yy[0]
        for i in range(2, M):
            yy[i] = f[i] - L0[i - 1] * yy[i - 1] - L1[i - 2] * yy[i - 2]
        uk = res[odd::2]
        uk[M - 1] = yy[M - 1] / U0[M - 1]
        uk[M - 2] = (yy[M - 2] - U1[M - 2] * uk[M - 1]) / U0[M - 2]
        uk[M - 3] = (yy[M - 3] - U1[M - 3] * uk[M - 2] - U2[M - 3] * uk[M - 1]) / U0[M - 3]
        s1 = np.zeros_like(yy[0])
        s2 = np.zeros_like(yy[0])
        for kk in range(M - 4, -1, -1):
            j = 2 * kk + odd + 6
            s1 = s1 + uk[kk + 3] / (j + 3.)
            s2 = s2 + (uk[kk + 3] / (j + 3.)) * ((j + 2.) * (j + 2.))
            uk[kk] = (yy[kk] - U1[kk] * uk[kk + 1] - U2[kk] * uk[kk + 2] - A[kk] * a0 * s1 - B[kk] * a0 * s2) / U0[kk]
    ub[:2 * M] = res
    return u


def biharmonic_matvec(v, b, a0, alfa, beta, sii, siu, siuu, ail, aii, aiu, bill, bil, bii, biu, biuu, axis=0):
    """Matvec.pyx:820-920 Biharmonic_matvec: b[:M] = (a0 S + alfa A + beta B) v, M = len(sii)."""
    M = len(sii)
    shape = list(v.shape)
    shape[axis] = 1
    alf = np.moveaxis(np.broadcast_to(np.asarray(alfa, dtype=float), shape), axis, 0)[0]
    bet = np.moveaxis(np.broadcast_to(np.asarray(beta, dtype=float), shape), axis, 0)[0]
    vv = np.moveaxis(v, axis, 0)
    bb = np.moveaxis(b, axis, 0)
    sii, siu, siuu, ail, aii, aiu, bill, bil, bii, biu, biuu = (
        np.asarray(d, dtype=float) for d in (sii, siu, siuu, ail, aii, aiu, bill, bil, bii, biu, biuu))
    dd = [a0 * sii[i] + alf * aii[i] + bet * bii[i] for i in range(M)]
    ld = [alf * ail[i] + bet * bil[i] for i in range(M - 2)]
    ldd = [bet * bill[i] for i in range(M - 4)]
    ud = [a0 * siu[i] + alf * aiu[i] + bet * biu[i] for i in range(M - 2)]
    udd = [a0 * siuu[i] + bet * biuu[i] for i in range(M - 4)]
    for i in (M - 1, M - 2):
        bb[i] = ldd[i - 4] * vv[i - 4] + ld[i - 2] * vv[i - 2] + dd[i] * vv[i]
    for i in (M - 3, M - 4):
        bb[i] = ldd[i - 4] * vv[i - 4] + ld[i - 2] * vv[i - 2] + dd[i] * vv[i] + ud[i] * vv[i + 2]
    for i in (M - 5, M - 6):
        bb[i] = (ldd[i - 4] * vv[i - 4] + ld[i - 2] * vv[i - 2] + dd[i] * vv[i] + ud[i] * vv[i + 2]
                 + udd[i] * vv[i + 4])
    s1 = np.zeros_like(vv[0])
    s2 = np.zeros_like(vv[0])
    o1 = np.zeros_like(vv[0])
    o2 = np.zeros_like(vv[0])
    for k in range(M - 7, -1, -1):
        j = k + 6
        p = k * sii[k] / (k + 1.)
        r = 24 * (k + 1) * (k + 2) * np.pi
        d = vv[j] / (j + 3.)
        if k % 2 == 0:
            s1 = s1 + d
            s2 = s2 + (j + 2) * (j + 2) * d
            bb[k] = (p * s1 + r * s2) * a0
        else:
            o1 = o1 + d
            o2 = o2 + (j + 2) * (j + 2) * d
            bb[k] = (p * o1 + r * o2) * a0
        if k > 3:
            bb[k] += ldd[k - 4] * vv[k - 4] + ld[k - 2] * vv[k - 2] + dd[k] * vv[k] + ud[k] * vv[k + 2] + udd[k] * vv[k + 4]
        elif k > 1:
            bb[k] += ld[k - 2] * vv[k - 2] + dd[k] * vv[k] + ud[k] * vv[k + 2] + udd[k] * vv[k + 4]
        else:
            bb[k] += dd[k] * vv[k] + ud[k] * vv[k + 2] + udd[k] * vv[k + 4]
    return b


# ---------------------------------------------------------------------------
# banded inner solves (la.pyx:466-613) on one line u (first data.shape[1] entries)
def inner_solve(kind, u, data):
    n = data.shape[1]
    D = data.reshape(-1)
    if kind == "DiagMA":
        u[:n] /= data[0, :n]
    elif kind == "TwoDMA":
        d, u1 = D[0:], D[n + 2:]
        u[n - 1] /= d[n - 1]
        u[n - 2] /= d[n - 2]
        for i in range(n - 3, -1, -1):
            u[i] = (u[i] - u1[i] * u[i + 2]) / d[i]
    elif kind in ("ThreeDMA", "FDMA"):
        if kind == "ThreeDMA":
            d, u1, u2 = D[0:], D[n + 2:], D[n + 4:]
        else:
            ld, d, u1, u2 = D[0:], D[n:], D[2 * n + 2:], D[3 * n + 4:]
            for i in range(2, n):
                u[i] -= ld[i - 2] * u[i - 2]
        u[n - 1] /= d[n - 1]
        u[n - 2] /= d[n - 2]
        u[n - 3] = (u[n - 3] - u1[n - 3] * u[n - 1]) / d[n - 3]
        u[n - 4] = (u[n - 4] - u1[n - 4] * u[n - 2]) / d[n - 4]
        for i in range(n - 5, -1, -1):
            u[i] = (u[i] - u1[i] * u[i + 2] - u2[i] * u[i + 4]) / d[i]
    elif kind == "TDMA":
        ld, d, ud = D[0:], D[n:], D[2 * n + 2:]
        for i in range(2, n):
            u[i] -= ld[i - 2] * u[i - 2]
        u[n - 1] /= d[n - 1]
        u[n - 2] /= d[n - 2]
        for i in range(n - 3, -1, -1):
            u[i] = (u[i] - ud[i] * u[i + 2]) / d[i]
    elif kind == "TDMA_O":
        ld, d, ud = D[0:], D[n:], D[2 * n + 1:]
        for i in range(1, n):
            u[i] -= ld[i - 1] * u[i - 1]
        u[n - 1] /= d[n - 1]
        for i in range(n - 2, -1, -1):
            u[i] = (u[i] - ud[i] * u[i + 1]) / d[i]
    elif kind in ("PDMA", "HeptaDMA"):
        a, b, d, e, f = D[0:], D[n:], D[2 * n:], D[3 * n + 2:], D[4 * n + 4:]
        u[2] -= b[0] * u[0]
        u[3] -= b[1] * u[1]
        for k in range(4, n):
            u[k] -= (b[k - 2] * u[k - 2] + a[k - 4] * u[k - 4])
        u[n - 1] /= d[n - 1]
        u[n - 2] /= d[n - 2]
        u[n - 3] = (u[n - 3] - e[n - 3] * u[n - 1]) / d[n - 3]
        u[n - 4] = (u[n - 4] - e[n - 4] * u[n - 2]) / d[n - 4]
        if kind == "PDMA":
            for k in range(n - 5, -1, -1):
                u[k] = (u[k] - e[k] * u[k + 2] - f[k] * u[k + 4]) / d[k]
        else:
            g, h = D[5 * n + 6:], D[6 * n + 8:]
            u[n - 5] = (u[n - 5] - e[n - 5] * u[n - 3] - f[n - 5] * u[n - 1]) / d[n - 5]
            u[n - 6] = (u[n - 6] - e[n - 6] * u[n - 4] - f[n - 6] * u[n - 2]) / d[n - 6]
            u[n - 7] = (u[n - 7] - e[n - 7] * u[n - 5] - f[n - 7] * u[n - 3] - g[n - 7] * u[n - 1]) / d[n - 7]
            u[n - 8] = (u[n - 8] - e[n - 8] * u[n - 6] - f[n - 8] * u[n - 4] - g[n - 8] * u[n - 2]) / d[n - 8]
            for k in range(n - 9, -1, -1):
                u[k] = (u[k] - e[k] * u[k + 2] - f[k] * u[k + 4] - g[k] * u[k + 6] - h[k] * u[k + 8]) / d[k]
    else:
        raise ValueError(kind)
    return u


def solve_data(u, data, kind, naxes, is_zero_index):
    """la.pyx:371-427 SolverGeneric1ND_solve_data: system (i, j) of the axes
    other than naxes, in order, solved with data[i, j]."""
    um = np.moveaxis(u, naxes, -1)
    lines = um.reshape(-1, um.shape[-1])
    dat = data.reshape(-1, *data.shape[-2:])
    for s in range(lines.shape[0]):
        if s == 0 and is_zero_index:
            continue
        line = lines[s].copy()
        inner_solve(kind, line, dat[s])
        lines[s] = line
    u[...] = np.moveaxis(lines.reshape(um.shape), -1, naxes)
    return u


# ---------------------------------------------------------------------------
# recursive Legendre transforms (transforms.pyx:218-325)
def _recursion(a):
    a = np.asarray(a, dtype=float)
    if a.shape[0] == 2:
        return a[0], np.zeros(a.shape[1]), a[1]
    return a[0], a[1], a[2]


def legendre_matrix(x, a, n):
    """P[i, j] = P_i(x_j), i < n, by the reference's recurrence."""
    anm, ann, anp = _recursion(a)
    x = np.asarray(x, dtype=float)
    P = np.zeros((n, x.size))
    Lm = np.ones_like(x)
    L = (x - ann[0]) / anm[0]
    Lp = (x - ann[1]) / anm[1] * L - anp[1] / anm[1] * Lm
    for i in range(n):
        P[i] = Lm
        s1 = 1 / anm[i + 2]
        s2 = anp[i + 2] / anm[i + 2]
        Lm, L = L, Lp
        Lp = s1 * (x - ann[i + 2]) * L - s2 * Lm
    return P


def scalar_product(input_array, output_array, x, w, axis, a):
    """transforms.pyx:175 (_scalar_product_ptr, :275-325)."""
    N = input_array.shape[axis]
    P = legendre_matrix(x[:N], a, N)
    fin = np.moveaxis(input_array, axis, -1)
    res = (fin * np.asarray(w)[:N]) @ P.T
    output_array[...] = np.moveaxis(res, -1, axis)
    return output_array


def evaluate_expansion_all(input_array, output_array, x, axis, a):
    """transforms.pyx:199 (_evaluate_expansion_all_ptr, :218-273)."""
    N = input_array.shape[axis]
    Nx = output_array.shape[axis]
    P = legendre_matrix(x[:Nx], a, N)
    fin = np.moveaxis(input_array, axis, -1)
    output_array[...] = np.moveaxis(fin @ P, -1, axis)
    return output_array
