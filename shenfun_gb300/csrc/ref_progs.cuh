// Block programs of the reference-signature entry points (ref_abi.cu): the
// entry points shenfun's optimization modules export by name, on the
// reference's own argument arrays and layouts.
//
//  * Chebyshev biharmonic LU / factor / solve / matvec in the reference's
//    factor layout (la.pyx:975-1290, Matvec.pyx:820-906): per Fourier system
//    and parity p, the parity-p rows of a0 SBB + alfa ABB + beta BBB (banded
//    in the two lower and two upper parity neighbours, plus a full upper part
//    whose entries are m(k, j) a0 pi / (j + 3) with the integer
//    m = 8 (k+1)(k+2)(k(k+4) + 3 (j+2)^2)).  The reference eliminates whole
//    rows (O(M^2) per system); here every row's upper part is kept as the two
//    coefficients (P, Q) of (P + Q (j+2)^2) a0 pi / (j + 3), so the
//    elimination is O(M) and runs in registers.  The LU factors of a matrix
//    without pivoting are unique, so the stored u0, u1, u2, l0, l1 are the
//    reference's to rounding.
//  * the banded solves of SolverGeneric1ND_solve_data (la.pyx:371-427) and
//    the *_inner_solve kernels it dispatches to by name (la.pyx:466-613),
//    each in the reference's data layout, one system per thread.
//  * the three-term recurrence of the recursive Legendre transforms
//    (transforms.pyx:218-325), evaluated once per point to build the matrix
//    the line GEMM applies.
#pragma once

#include "solvers.cuh"

namespace sgpu {
namespace ref {

const double PI = 3.141592653589793;

// ---- Chebyshev biharmonic ---------------------------------------------------
// the reference's diagonals (full index space of the N - 4 dofs): SBB main,
// +2, +4; ABB -2, main, +2; BBB -4, -2, main, +2, +4
struct BihDiags {
  const double *sii, *siu, *siuu, *ail, *aii, *aiu, *bill, *bil, *bii, *biu, *biuu;
};

// entry (k, j) of the full upper part, from the row's coefficients (P, Q);
// for unreduced rows P + Q (j+2)^2 is the reference's integer m exactly
SGPU_HD double bih_far(double P, double Q, int64_t j, double a0) {
  const double jj = (double)((j + 2) * (j + 2));
  return (P + Q * jj) * a0 * PI / (j + 3.0);
}

// Row r of parity p (global index g = 2 r + p): E[q] = entry at parity column
// r - 2 + q for q = 0..4 (0 outside [0, M)), and the coefficients of its full
// upper part (columns >= r + 3).  la.pyx:1017-1052 (LU_oe_Biharmonic_1D).
SGPU_HD void bih_row(const BihDiags& d, double a, double b, double c, int64_t r, int p, int64_t M, double E[5],
                     double& P, double& Q) {
  const int64_t g = 2 * r + p;
  E[0] = r >= 2 ? c * d.bill[g - 4] : 0.0;
  E[1] = r >= 1 ? b * d.ail[g - 2] + c * d.bil[g - 2] : 0.0;
  E[2] = a * d.sii[g] + b * d.aii[g] + c * d.bii[g];
  E[3] = r + 1 < M ? a * d.siu[g] + b * d.aiu[g] + c * d.biu[g] : 0.0;
  E[4] = r + 2 < M ? a * d.siuu[g] + c * d.biuu[g] : 0.0;
  P = (double)(8 * g * (g + 1) * (g + 2) * (g + 4));
  Q = (double)(24 * (g + 1) * (g + 2));
}

// LU of one (system, parity) chain: the factor arrays are pre-offset to the
// chain, entry r at f[r * fs].  l0[r] (r < M-1), l1[r] (r < M-2) are the two
// subdiagonals of L, u0, u1, u2 the first three diagonals of U (la.pyx:991-1125).
SGPU_HD void bih_lu_prog(const BihDiags& d, double a, double b, double c, int p, int64_t M, double* u0,
                         double* u1, double* u2, double* l0, double* l1, int64_t fs) {
  double E[5], P0, Q0, P1, Q1, P2, Q2;
  // pivot row: columns kk-1 .. kk+1; next rows: kk-1 .. kk+2 and kk-1 .. kk+3
  double x0[3], x1[4], x2[5];
  bih_row(d, a, b, c, 0, p, M, E, P0, Q0);
  x0[0] = E[2], x0[1] = E[3], x0[2] = E[4];
  bih_row(d, a, b, c, 1, p, M, E, P1, Q1);
  for (int q = 0; q < 4; ++q) x1[q] = E[q + 1];
  bih_row(d, a, b, c, 2, p, M, E, P2, Q2);
  for (int q = 0; q < 5; ++q) x2[q] = E[q];
  u0[0] = x0[0];
  u1[0] = x0[1];
  u2[0] = x0[2];
  for (int64_t kk = 1; kk < M; ++kk) {
    const double piv = x0[0];
    // the pivot row's full upper part at columns kk+2 and kk+3
    const double f2 = kk + 2 < M ? bih_far(P0, Q0, 2 * (kk + 2) + p, a) : 0.0;
    const double f3 = kk + 3 < M ? bih_far(P0, Q0, 2 * (kk + 3) + p, a) : 0.0;
    const double lz = x1[0] / piv;
    l0[(kk - 1) * fs] = lz;
    x1[1] -= lz * x0[1];
    x1[2] -= lz * x0[2];
    x1[3] -= lz * f2;
    P1 -= lz * P0;
    Q1 -= lz * Q0;
    if (kk < M - 1) {
      const double lo = x2[0] / piv;
      l1[(kk - 1) * fs] = lo;
      x2[1] -= lo * x0[1];
      x2[2] -= lo * x0[2];
      x2[3] -= lo * f2;
      x2[4] -= lo * f3;
      P2 -= lo * P0;
      Q2 -= lo * Q0;
    }
    x0[0] = x1[1], x0[1] = x1[2], x0[2] = x1[3];
    P0 = P1, Q0 = Q1;
    for (int q = 0; q < 4; ++q) x1[q] = x2[q + 1];
    P1 = P2, Q1 = Q2;
    if (kk < M - 2) {
      bih_row(d, a, b, c, kk + 2, p, M, E, P2, Q2);
      for (int q = 0; q < 5; ++q) x2[q] = E[q];
    }
    u0[kk * fs] = x0[0];
    if (kk < M - 1) u1[kk * fs] = x0[1];
    if (kk < M - 2) u2[kk * fs] = x0[2];
  }
}

// coefficients of U's full upper part from L (la.pyx:1213-1233,
// Biharmonic_factor_oe_pr): ak, bk for rows 0 .. M-3
SGPU_HD void bih_factor_pr_prog(int p, int64_t M, double* ak, double* bk, const double* l0, const double* l1,
                                int64_t fs) {
  int64_t k = p;
  ak[0] = (double)(8 * k * (k + 1) * (k + 2) * (k + 4)) * PI;
  bk[0] = (double)(24 * (k + 1) * (k + 2)) * PI;
  k = 2 + p;
  ak[fs] = (double)(8 * k * (k + 1) * (k + 2) * (k + 4)) * PI - l0[0] * ak[0];
  bk[fs] = (double)(24 * (k + 1) * (k + 2)) * PI - l0[0] * bk[0];
  for (int64_t r = 2; r < M - 2; ++r) {
    const int64_t g = 2 * r + p;
    const double pp = (double)(8 * g * (g + 1) * (g + 2) * (g + 4)), rr = (double)(24 * (g + 1) * (g + 2));
    ak[r * fs] = pp * PI - l0[(r - 1) * fs] * ak[(r - 1) * fs] - l1[(r - 2) * fs] * ak[(r - 2) * fs];
    bk[r * fs] = rr * PI - l0[(r - 1) * fs] * bk[(r - 1) * fs] - l1[(r - 2) * fs] * bk[(r - 2) * fs];
  }
}

// Solve of one (system, parity) chain (la.pyx:1252-1290, Solve_Biharmonic_3D_n):
// L y = f, then U u = y with the full upper part as two running sums.  The
// forward sweep writes y into u (entry i is read from f before it is
// written), so u may alias f.  fv / uv: the line's even or odd entries.
template <class T>
SGPU_HD void bih_solve_prog(Line<T> fv, Line<T> uv, int p, int64_t M, const double* u0, const double* u1,
                            const double* u2, const double* l0, const double* l1, const double* ak,
                            const double* bk, double a0, int64_t fs) {
  T y2 = fv[0], y1;
  uv[0] = y2;
  y1 = fv[1] - mulr(y2, l0[0]);
  uv[1] = y1;
  for (int64_t i = 2; i < M; ++i) {
    const T y = fv[i] - mulr(y1, l0[(i - 1) * fs]) - mulr(y2, l1[(i - 2) * fs]);
    uv[i] = y;
    y2 = y1;
    y1 = y;
  }
  T w1 = divr(uv[M - 1], u0[(M - 1) * fs]);  // u[kk+1], u[kk+2], u[kk+3] while kk descends
  uv[M - 1] = w1;
  T w0 = divr(uv[M - 2] - mulr(w1, u1[(M - 2) * fs]), u0[(M - 2) * fs]);
  uv[M - 2] = w0;
  T wm = divr(uv[M - 3] - mulr(w0, u1[(M - 3) * fs]) - mulr(w1, u2[(M - 3) * fs]), u0[(M - 3) * fs]);
  uv[M - 3] = wm;
  T s1 = zero_of(T()), s2 = zero_of(T());
  T n1 = wm, n2 = w0, n3 = w1;  // u[kk+1], u[kk+2], u[kk+3]
  for (int64_t kk = M - 4; kk >= 0; --kk) {
    const int64_t j = 2 * kk + p + 6;
    const T dj = divr(n3, j + 3.0);
    s1 = s1 + dj;
    s2 = s2 + mulr(dj, (double)(j + 2) * (double)(j + 2));
    const T v = divr(uv[kk] - mulr(n1, u1[kk * fs]) - mulr(n2, u2[kk * fs]) - mulr(s1, ak[kk * fs] * a0) -
                         mulr(s2, bk[kk * fs] * a0),
                     u0[kk * fs]);
    uv[kk] = v;
    n3 = n2;
    n2 = n1;
    n1 = v;
  }
}

// b = (a0 SBB + alf ABB + bet BBB) v on the first M = N - 4 entries of a line
// (Matvec.pyx:820-906, Biharmonic_matvec_ptr); the other entries of b are
// left as they are.  Needs M >= 10.
template <class T>
SGPU_HD void bih_matvec_prog(Line<T> v, Line<T> b, const BihDiags& d, double a0, double alf, double bet,
                             int64_t M) {
  auto dd = [&](int64_t i) { return a0 * d.sii[i] + alf * d.aii[i] + bet * d.bii[i]; };
  auto ld = [&](int64_t i) { return alf * d.ail[i] + bet * d.bil[i]; };
  auto ldd = [&](int64_t i) { return bet * d.bill[i]; };
  auto ud = [&](int64_t i) { return a0 * d.siu[i] + alf * d.aiu[i] + bet * d.biu[i]; };
  auto udd = [&](int64_t i) { return a0 * d.siuu[i] + bet * d.biuu[i]; };
  for (int64_t i = M - 1; i >= M - 6; --i) {
    T s = mulr(v[i - 4], ldd(i - 4)) + mulr(v[i - 2], ld(i - 2)) + mulr(v[i], dd(i));
    if (i <= M - 3) s = s + mulr(v[i + 2], ud(i));
    if (i <= M - 5) s = s + mulr(v[i + 4], udd(i));
    b[i] = s;
  }
  T s1 = zero_of(T()), s2 = zero_of(T()), o1 = zero_of(T()), o2 = zero_of(T());
  for (int64_t k = M - 7; k >= 0; --k) {
    const int64_t j = k + 6;
    const double pk = k * d.sii[k] / (k + 1.0);
    const double rk = (double)(24 * (k + 1) * (k + 2)) * PI;
    const T dj = divr(v[j], j + 3.0);
    const double jj = (double)((j + 2) * (j + 2));
    T s;
    if (k % 2 == 0) {
      s1 = s1 + dj;
      s2 = s2 + mulr(dj, jj);
      s = mulr(mulr(s1, pk) + mulr(s2, rk), a0);
    } else {
      o1 = o1 + dj;
      o2 = o2 + mulr(dj, jj);
      s = mulr(mulr(o1, pk) + mulr(o2, rk), a0);
    }
    T t;
    if (k > 3)
      t = mulr(v[k - 4], ldd(k - 4)) + mulr(v[k - 2], ld(k - 2)) + mulr(v[k], dd(k)) + mulr(v[k + 2], ud(k)) +
          mulr(v[k + 4], udd(k));
    else if (k > 1)
      t = mulr(v[k - 2], ld(k - 2)) + mulr(v[k], dd(k)) + mulr(v[k + 2], ud(k)) + mulr(v[k + 4], udd(k));
    else
      t = mulr(v[k], dd(k)) + mulr(v[k + 2], ud(k)) + mulr(v[k + 4], udd(k));
    b[k] = s + t;
  }
}

// ---- banded solves by name (la.pyx:466-613) --------------------------------
enum DmaKind { DMA_DIAG = 0, DMA_TWO = 1, DMA_THREE = 2, DMA_T = 3, DMA_T_O = 4, DMA_P = 5, DMA_F = 6, DMA_HEPTA = 7 };

// smallest number of columns a kind's solve reads without leaving the data
SGPU_HD int dma_min_cols(int kind) {
  switch (kind) {
    case DMA_DIAG: return 1;
    case DMA_T_O: return 2;
    case DMA_TWO: case DMA_T: return 3;
    case DMA_THREE: case DMA_P: case DMA_F: return 5;
    case DMA_HEPTA: return 9;
  }
  return 1 << 30;
}
SGPU_HD int dma_rows(int kind) {
  switch (kind) {
    case DMA_DIAG: return 1;
    case DMA_TWO: return 2;
    case DMA_THREE: case DMA_T: case DMA_T_O: return 3;
    case DMA_F: return 4;
    case DMA_P: return 5;
    case DMA_HEPTA: return 7;
  }
  return 0;
}

// one system: n = columns of data (the first n entries of the line are solved)
template <class T>
SGPU_HD void dma_solve_prog(int kind, Line<T> u, const double* data, int64_t n) {
  switch (kind) {
    case DMA_DIAG:
      for (int64_t i = 0; i < n; ++i) u[i] = divr(u[i], data[i]);
      return;
    case DMA_TWO: {
      const double* d = data;
      const double* u1 = data + n + 2;
      u[n - 1] = divr(u[n - 1], d[n - 1]);
      u[n - 2] = divr(u[n - 2], d[n - 2]);
      for (int64_t i = n - 3; i >= 0; --i) u[i] = divr(u[i] - mulr(u[i + 2], u1[i]), d[i]);
      return;
    }
    case DMA_THREE: {
      // the offset-4 coefficients are read from the offset-2 row, four
      // columns on (la.pyx:569-584)
      const double* d = data;
      const double* u1 = data + n + 2;
      const double* u2 = data + n + 4;
      u[n - 1] = divr(u[n - 1], d[n - 1]);
      u[n - 2] = divr(u[n - 2], d[n - 2]);
      u[n - 3] = divr(u[n - 3] - mulr(u[n - 1], u1[n - 3]), d[n - 3]);
      u[n - 4] = divr(u[n - 4] - mulr(u[n - 2], u1[n - 4]), d[n - 4]);
      for (int64_t i = n - 5; i >= 0; --i)
        u[i] = divr(u[i] - mulr(u[i + 2], u1[i]) - mulr(u[i + 4], u2[i]), d[i]);
      return;
    }
    case DMA_T: {
      const double* ld = data;
      const double* d = data + n;
      const double* ud = data + 2 * n + 2;
      for (int64_t i = 2; i < n; ++i) u[i] = u[i] - mulr(u[i - 2], ld[i - 2]);
      u[n - 1] = divr(u[n - 1], d[n - 1]);
      u[n - 2] = divr(u[n - 2], d[n - 2]);
      for (int64_t i = n - 3; i >= 0; --i) u[i] = divr(u[i] - mulr(u[i + 2], ud[i]), d[i]);
      return;
    }
    case DMA_T_O: {
      const double* ld = data;
      const double* d = data + n;
      const double* ud = data + 2 * n + 1;
      for (int64_t i = 1; i < n; ++i) u[i] = u[i] - mulr(u[i - 1], ld[i - 1]);
      u[n - 1] = divr(u[n - 1], d[n - 1]);
      for (int64_t i = n - 2; i >= 0; --i) u[i] = divr(u[i] - mulr(u[i + 1], ud[i]), d[i]);
      return;
    }
    case DMA_F: {
      const double* ld = data;
      const double* d = data + n;
      const double* u1 = data + 2 * n + 2;
      const double* u2 = data + 3 * n + 4;
      for (int64_t i = 2; i < n; ++i) u[i] = u[i] - mulr(u[i - 2], ld[i - 2]);
      u[n - 1] = divr(u[n - 1], d[n - 1]);
      u[n - 2] = divr(u[n - 2], d[n - 2]);
      u[n - 3] = divr(u[n - 3] - mulr(u[n - 1], u1[n - 3]), d[n - 3]);
      u[n - 4] = divr(u[n - 4] - mulr(u[n - 2], u1[n - 4]), d[n - 4]);
      for (int64_t i = n - 5; i >= 0; --i)
        u[i] = divr(u[i] - mulr(u[i + 2], u1[i]) - mulr(u[i + 4], u2[i]), d[i]);
      return;
    }
    case DMA_P:
    case DMA_HEPTA: {
      const double* a = data;
      const double* b = data + n;
      const double* d = data + 2 * n;
      const double* e = data + 3 * n + 2;
      const double* f = data + 4 * n + 4;
      u[2] = u[2] - mulr(u[0], b[0]);
      u[3] = u[3] - mulr(u[1], b[1]);
      for (int64_t k = 4; k < n; ++k) u[k] = u[k] - (mulr(u[k - 2], b[k - 2]) + mulr(u[k - 4], a[k - 4]));
      u[n - 1] = divr(u[n - 1], d[n - 1]);
      u[n - 2] = divr(u[n - 2], d[n - 2]);
      u[n - 3] = divr(u[n - 3] - mulr(u[n - 1], e[n - 3]), d[n - 3]);
      u[n - 4] = divr(u[n - 4] - mulr(u[n - 2], e[n - 4]), d[n - 4]);
      if (kind == DMA_P) {
        for (int64_t k = n - 5; k >= 0; --k)
          u[k] = divr(u[k] - mulr(u[k + 2], e[k]) - mulr(u[k + 4], f[k]), d[k]);
        return;
      }
      const double* g = data + 5 * n + 6;
      const double* h = data + 6 * n + 8;
      u[n - 5] = divr(u[n - 5] - mulr(u[n - 3], e[n - 5]) - mulr(u[n - 1], f[n - 5]), d[n - 5]);
      u[n - 6] = divr(u[n - 6] - mulr(u[n - 4], e[n - 6]) - mulr(u[n - 2], f[n - 6]), d[n - 6]);
      u[n - 7] = divr(u[n - 7] - mulr(u[n - 5], e[n - 7]) - mulr(u[n - 3], f[n - 7]) - mulr(u[n - 1], g[n - 7]),
                      d[n - 7]);
      u[n - 8] = divr(u[n - 8] - mulr(u[n - 6], e[n - 8]) - mulr(u[n - 4], f[n - 8]) - mulr(u[n - 2], g[n - 8]),
                      d[n - 8]);
      for (int64_t k = n - 9; k >= 0; --k)
        u[k] = divr(u[k] - mulr(u[k + 2], e[k]) - mulr(u[k + 4], f[k]) - mulr(u[k + 6], g[k]) -
                        mulr(u[k + 8], h[k]),
                    d[k]);
      return;
    }
  }
}

// ---- recursive Legendre transforms (transforms.pyx:218-325) -----------------
// Column j of the matrix of the point x: P_i(x) for i < n by the three-term
// recurrence of the recursion matrix's DIA data a (rows x cols; two rows:
// sub- and super-diagonal, three: sub, main, super).  out[i * ld] = P_i(x) w.
SGPU_HD void legendre_recursion_column(double x, double w, const double* a, int rows, int64_t cols, int64_t n,
                                       double* out, int64_t ld) {
  const double* anm = a;
  const double* ann = rows == 2 ? nullptr : a + cols;
  const double* anp = rows == 2 ? a + cols : a + 2 * cols;
  auto nn = [&](int64_t i) { return ann ? ann[i] : 0.0; };
  double Lm = 1.0;
  double L = (x - nn(0)) / anm[0];
  double Lp = (x - nn(1)) / anm[1] * L - anp[1] / anm[1] * Lm;
  for (int64_t i = 0; i < n; ++i) {
    out[i * ld] = Lm * w;
    const double s1 = 1.0 / anm[i + 2];
    const double s2 = anp[i + 2] / anm[i + 2];
    Lm = L;
    L = Lp;
    Lp = s1 * (x - nn(i + 2)) * L - s2 * Lm;
  }
}

// ---- per-thread drivers (the kernels of ref_abi.cu and the CPU emulator) ---
// factor arrays of shape (2, outer, M, inner): chain c = p * nsys + s
SGPU_HD int64_t chain_base(int64_t c, int64_t nsys, int64_t M, int64_t inner) {
  const int64_t p = c / nsys, s = c - p * nsys;
  const int64_t o = s / inner, i = s - o * inner;
  return (p * (nsys / inner) + o) * M * inner + i;
}

SGPU_HD void bih_lu_chain(int64_t c, int64_t nsys, const BihDiags& d, double a0, const double* alfa,
                          const double* beta, double* u0, double* u1, double* u2, double* l0, double* l1,
                          int64_t M, int64_t inner) {
  const int p = (int)(c / nsys);
  const int64_t s = c - p * nsys;
  const int64_t b = chain_base(c, nsys, M, inner);
  bih_lu_prog(d, a0, alfa[s], beta[s], p, M, u0 + b, u1 + b, u2 + b, l0 + b, l1 + b, inner);
}

SGPU_HD void bih_factor_pr_chain(int64_t c, int64_t nsys, double* ak, double* bk, const double* l0,
                                 const double* l1, int64_t M, int64_t inner) {
  const int64_t b = chain_base(c, nsys, M, inner);
  bih_factor_pr_prog((int)(c / nsys), M, ak + b, bk + b, l0 + b, l1 + b, inner);
}

// chain c reads entries p, p + 2, ... of line s of f (outer, N, inner)
template <class T>
SGPU_HD void bih_solve_chain(int64_t c, int64_t nsys, const T* f, T* u, const double* u0, const double* u1,
                             const double* u2, const double* l0, const double* l1, const double* ak,
                             const double* bk, double a0, int64_t N, int64_t M, int64_t inner) {
  const int p = (int)(c / nsys);
  const int64_t s = c - p * nsys;
  const int64_t lb = sys_base(s, N, inner) + p * inner;
  const int64_t b = chain_base(c, nsys, M, inner);
  Line<T> fv{const_cast<T*>(f) + lb, 2 * inner}, uv{u + lb, 2 * inner};
  bih_solve_prog<T>(fv, uv, p, M, u0 + b, u1 + b, u2 + b, l0 + b, l1 + b, ak + b, bk + b, a0, inner);
}

template <class T>
SGPU_HD void bih_matvec_sys(int64_t s, const T* v, T* b, const BihDiags& d, double a0, const double* alfa,
                            const double* beta, int64_t N, int64_t M, int64_t inner) {
  const int64_t lb = sys_base(s, N, inner);
  Line<T> vv{const_cast<T*>(v) + lb, inner}, bv{b + lb, inner};
  bih_matvec_prog<T>(vv, bv, d, a0, alfa[s], beta[s], M);
}

// system s of u (outer, N, inner) with its matrix at data + s * dstride
template <class T>
SGPU_HD void dma_solve_sys(int64_t s, int kind, T* u, const double* data, int64_t dstride, int64_t cols, int64_t N,
                           int64_t inner) {
  Line<T> uv{u + sys_base(s, N, inner), inner};
  dma_solve_prog<T>(kind, uv, data + s * dstride, cols);
}

// point j of the recursive Legendre matrix: scalar product M[j][i] =
// P_i(x_j) w_j (npts x n), evaluation M[i][j] = P_i(x_j) (n x npts)
SGPU_HD void legendre_matrix_point(int64_t j, int scalar, const double* x, const double* w, const double* a,
                                   int rows, int64_t cols, int64_t n, int64_t npts, double* M) {
  if (scalar)
    legendre_recursion_column(x[j], w[j], a, rows, cols, n, M + j * n, 1);
  else
    legendre_recursion_column(x[j], 1.0, a, rows, cols, n, M + j, npts);
}

}  // namespace ref
}  // namespace sgpu
