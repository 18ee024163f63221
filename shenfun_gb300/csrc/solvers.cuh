// Batched banded solvers, one system per (outer, inner) index of a
// (outer, n, inner) array: TDMA / PDMA (la.pyx:213-252, 496-532) and the
// Chebyshev Dirichlet Helmholtz LU / solve / matvec (la.pyx:717-912,
// Matvec.pyx:656-695).  One thread owns one system and runs the reference's
// sequential recurrence, so the per-system operation order follows the
// reference.  With inner > 1 consecutive threads own consecutive systems and
// every step of the recurrence is a coalesced row access.
#pragma once

#include <cmath>

#include "dfloat.cuh"

namespace sgpu {

SGPU_HD double mulr(double a, double s) { return a * s; }
SGPU_HD cd mulr(cd a, double s) { return scale(a, s); }
SGPU_HD double zero_of(double) { return 0.0; }
SGPU_HD cd zero_of(cd) { return cx<double>(0.0, 0.0); }
SGPU_HD double divr(double a, double s) { return a / s; }
SGPU_HD cd divr(cd a, double s) { return cx<double>(a.re / s, a.im / s); }
SGPU_HD double real_of(double, double c) { return c; }
SGPU_HD cd real_of(cd, double c) { return cx<double>(c, 0.0); }

// strided line view: element k of system s
template <class T>
struct Line {
  T* base;
  int64_t st;
  SGPU_HD T& operator[](int64_t k) const { return base[k * st]; }
};

SGPU_HD int64_t sys_base(int64_t s, int64_t n, int64_t inner) {
  int64_t o = s / inner, i = s - o * inner;
  return o * n * inner + i;
}

// ---- TDMA / PDMA ----------------------------------------------------------
SGPU_HD void tdma_lu_prog(double* data, int64_t n) {
  double* ld = data;
  double* d = data + n;
  double* ud = data + 2 * n + 2;
  for (int64_t i = 2; i < n; ++i) {
    ld[i - 2] = ld[i - 2] / d[i - 2];
    d[i] = d[i] - ld[i - 2] * ud[i - 2];
  }
}

template <class T>
SGPU_HD void tdma_solve_prog(T* u_all, const double* data, int64_t n, int64_t inner, int64_t s) {
  Line<T> u{u_all + sys_base(s, n, inner), inner};
  const double* ld = data;
  const double* d = data + n;
  const double* ud = data + 2 * n + 2;
  for (int64_t i = 2; i < n; ++i) u[i] = u[i] - mulr(u[i - 2], ld[i - 2]);
  u[n - 1] = mulr(u[n - 1], 1.0 / d[n - 1]);
  u[n - 2] = mulr(u[n - 2], 1.0 / d[n - 2]);
  for (int64_t i = n - 3; i >= 0; --i) u[i] = mulr(u[i] - mulr(u[i + 2], ud[i]), 1.0 / d[i]);
}

SGPU_HD void pdma_lu_prog(double* data, int64_t n) {
  double* a = data;
  double* b = data + n;
  double* d = data + 2 * n;
  double* e = data + 3 * n + 2;
  double* f = data + 4 * n + 4;
  const int64_t k = 2;
  for (int64_t i = 0; i < n - 2 * k; ++i) {
    double lam = b[i] / d[i];
    d[i + k] -= lam * e[i];
    e[i + k] -= lam * f[i];
    b[i] = lam;
    lam = a[i] / d[i];
    b[i + k] -= lam * e[i];
    d[i + 2 * k] -= lam * f[i];
    a[i] = lam;
  }
  for (int64_t i = n - 4; i <= n - 3; ++i) {
    double lam = b[i] / d[i];
    d[i + k] -= lam * e[i];
    b[i] = lam;
  }
}

template <class T>
SGPU_HD void pdma_solve_prog(T* u_all, const double* data, int64_t n, int64_t inner, int64_t s) {
  Line<T> u{u_all + sys_base(s, n, inner), inner};
  const double* a = data;
  const double* b = data + n;
  const double* d = data + 2 * n;
  const double* e = data + 3 * n + 2;
  const double* f = data + 4 * n + 4;
  u[2] = u[2] - mulr(u[0], b[0]);
  u[3] = u[3] - mulr(u[1], b[1]);
  for (int64_t k = 4; k < n; ++k) u[k] = u[k] - (mulr(u[k - 2], b[k - 2]) + mulr(u[k - 4], a[k - 4]));
  u[n - 1] = mulr(u[n - 1], 1.0 / d[n - 1]);
  u[n - 2] = mulr(u[n - 2], 1.0 / d[n - 2]);
  u[n - 3] = mulr(u[n - 3] - mulr(u[n - 1], e[n - 3]), 1.0 / d[n - 3]);
  u[n - 4] = mulr(u[n - 4] - mulr(u[n - 2], e[n - 4]), 1.0 / d[n - 4]);
  for (int64_t k = n - 5; k >= 0; --k)
    u[k] = mulr(u[k] - mulr(u[k + 2], e[k]) - mulr(u[k + 4], f[k]), 1.0 / d[k]);
}

// ---- general banded LU / solve (DiagMA, TwoDMA, ThreeDMA, FDMA, HeptaDMA) --
// The reference's other banded solvers (la.py:291-800, la.pyx) differ only in
// their band offsets.  Storage is theirs (scipy DIA, column aligned): row r of
// data holds offset off[r], M[i][i + off[r]] at data[r * n + i + off[r]].
// The offsets are even, ascending, include 0 and every even offset between
// the lowest and the highest, so elimination without pivoting fills in only
// inside the band.  LU in place (Doolittle: the multipliers replace the lower
// entries), then per line forward and back substitution.
struct BandDesc {
  int nd;
  int off[9];
};

SGPU_HD int band_row(const BandDesc& b, int o) {
  for (int r = 0; r < b.nd; ++r)
    if (b.off[r] == o) return r;
  return -1;
}

SGPU_HD void banded_lu_prog(double* data, const BandDesc& b, int64_t n) {
  const int r0 = band_row(b, 0);
  for (int64_t i = 0; i < n; ++i) {
    const double piv = data[r0 * n + i];
    for (int rl = 0; rl < b.nd; ++rl) {
      const int l = b.off[rl];
      if (l >= 0) continue;
      const int64_t k = i - l;  // row eliminated
      if (k >= n) continue;
      double& mk = data[rl * n + i];  // M[k][i] (offset l of row k, column i)
      const double m = mk / piv;
      mk = m;
      for (int ru = 0; ru < b.nd; ++ru) {
        const int u = b.off[ru];
        if (u <= 0 || i + u >= n) continue;
        const int rt = band_row(b, u + l);  // offset of (k, i + u)
        data[(int64_t)rt * n + i + u] -= m * data[(int64_t)ru * n + i + u];
      }
    }
  }
}

template <class T>
SGPU_HD void banded_solve_prog(T* u_all, const double* data, const BandDesc& b, int64_t n,
                               int64_t inner, int64_t s) {
  Line<T> u{u_all + sys_base(s, n, inner), inner};
  const int r0 = band_row(b, 0);
  for (int64_t i = 0; i < n; ++i) {
    T y = u[i];
    for (int r = 0; r < b.nd; ++r) {
      const int l = b.off[r];
      if (l < 0 && i + l >= 0) y = y - mulr(u[i + l], data[r * n + i + l]);  // row i's multiplier
    }
    u[i] = y;
  }
  for (int64_t i = n - 1; i >= 0; --i) {
    T x = u[i];
    for (int r = 0; r < b.nd; ++r) {
      const int o = b.off[r];
      if (o > 0 && i + o < n) x = x - mulr(u[i + o], data[r * n + i + o]);
    }
    u[i] = divr(x, data[r0 * n + i]);
  }
}

// ---- Chebyshev Dirichlet / Neumann Helmholtz -------------------------------
// ASDSD / BSDSD coefficients in the reference's evaluation order
// (chebyshev/matrices.py:1061-1079, :238-246).
SGPU_HD double hA0(int64_t k) { return ((-2.0 * 3.141592653589793) * (k + 1.0)) * (k + 2.0); }
SGPU_HD double hA2(int64_t k) { return (-4.0 * 3.141592653589793) * (k + 1.0); }
SGPU_HD double hB0(int64_t k) { return k == 0 ? 3.141592653589793 + 1.5707963267948966 : 3.141592653589793; }
SGPU_HD double hB2() { return -1.5707963267948966; }

// ShenNeumann phi_k = T_k - (k/(k+2))^2 T_{k+2} (chebyshev/bases.py:863-937):
// A = ASNSN (chebyshev/matrices.py:1096-1122), a_kk = -2 pi k^2 (k+1)/(k+2),
// a_kj = -4 pi j^2 (k+1)/(k+2)^2 for j = k+2, k+4, ...; B = BSNSN
// (chebyshev/matrices.py:377-401), b_kk = h_k + (k/(k+2))^4 h_{k+2},
// b_{k,k+2} = b_{k+2,k} = -(k/(k+2))^2 h_{k+2}, h_0 = pi, h_k = pi/2.  The
// Neumann branch of LU_Helmholtz_1D (la.pyx:735-751) divides column j >= 1 of
// both matrices by j^2: every strictly-upper row of the scaled A is then one
// constant, -4 pi (k+1)/(k+2)^2, and the Dirichlet recurrences solve for
// w_j = j^2 u_j.  For a pure stiffness system (|beta| < 1e-8) the singular
// row 0 gets a_00 = 1/alfa, b_00 = 0, and the solve sets u_0 = 0.
SGPU_HD double sn_h(int64_t k) { return k == 0 ? 3.141592653589793 : 1.5707963267948966; }
SGPU_HD double sn_K2sq(int64_t k) {
  const double r = k / (k + 2.0);
  return r * r;
}
SGPU_HD double sn_col(int64_t j) { return (double)j * (double)j; }

// Row i of the (column-scaled) matrices: A(i,i), A(i,i+2), A(i,i+4),
// B(i,i), B(i,i+2), B(i+2,i).
struct HelmRow {
  double A0, A2, A4, B0, B2, Bm2;
};

SGPU_HD HelmRow helm_row(int64_t i, int neumann) {
  HelmRow r;
  if (!neumann) {
    r.A0 = hA0(i);
    r.A2 = hA2(i);
    r.A4 = hA2(i);
    r.B0 = hB0(i);
    r.B2 = hB2();
    r.Bm2 = hB2();
    return r;
  }
  const double k = (double)i, m4pi = -4.0 * 3.141592653589793;
  const double a2 = ((m4pi * ((k + 2) * (k + 2))) * (k + 1)) / ((k + 2) * (k + 2));
  const double a4 = ((m4pi * ((k + 4) * (k + 4))) * (k + 1)) / ((k + 2) * (k + 2));
  const double al = sn_K2sq(i);
  r.A0 = i == 0 ? 0.0 : ((((-2.0 * 3.141592653589793) * (k * k)) * (k + 1)) / (k + 2)) / sn_col(i);
  r.A2 = a2 / sn_col(i + 2);
  r.A4 = a4 / sn_col(i + 4);
  r.B0 = sn_h(i) + (al * al) * sn_h(i + 2);
  if (i >= 1) r.B0 /= sn_col(i);
  r.B2 = (-al * sn_h(i + 2)) / sn_col(i + 2);
  r.Bm2 = i >= 1 ? (-al * sn_h(i + 2)) / sn_col(i) : 0.0;
  return r;
}

// the pure-stiffness test of the Neumann branch (la.pyx:736, 908)
SGPU_HD bool sn_singular(double beta) { return beta < 1e-8 && beta > -1e-8; }
SGPU_HD bool sn_zero_mode(double d00) { return (d00 - 1.0) * (d00 - 1.0) < 1e-16; }

// LU_Helmholtz_1D (la.pyx:717-763); N = number of basis functions, the
// factor lines have N entries with the last two untouched.
SGPU_HD void helmholtz_lu_prog(int64_t N, const double* alfa, const double* beta, int neumann,
                               double* d0_all, double* d1_all, double* d2_all, double* L_all,
                               int64_t inner, int64_t s) {
  const int64_t b0 = sys_base(s, N, inner);
  Line<double> d0{d0_all + b0, inner}, d1{d1_all + b0, inner}, d2{d2_all + b0, inner},
      L{L_all + b0, inner};
  const double a = alfa[s], b = beta[s];
  const int64_t M = N - 2;
  HelmRow r0 = helm_row(0, neumann), r1 = helm_row(1, neumann);
  if (neumann && sn_singular(b)) {
    r0.A0 = 1.0 / a;
    r0.B0 = 0.0;
  }
  d0[0] = a * r0.A0 + b * r0.B0;
  d0[1] = a * r1.A0 + b * r1.B0;
  d1[0] = a * r0.A2 + b * r0.B2;
  d1[1] = a * r1.A2 + b * r1.B2;
  d2[0] = a * r0.A4;
  d2[1] = a * r1.A4;
  for (int64_t i = 2; i < M; ++i) {
    const HelmRow r = helm_row(i, neumann);
    double l = b * helm_row(i - 2, neumann).Bm2 / d0[i - 2];
    L[i - 2] = l;
    d0[i] = a * r.A0 + b * r.B0 - l * d1[i - 2];
    if (i < M - 2) d1[i] = a * r.A2 + b * r.B2 - l * d2[i - 2];
    if (i < M - 4) d2[i] = a * r.A4 - l * d2[i - 2];
  }
}

// Solve_Helmholtz_1D_ptr (la.pyx:871-912).  y is kept in u.
template <class T>
SGPU_HD void helmholtz_solve_prog(const T* b_all, T* u_all, int neumann, const double* d0_all,
                                  const double* d1_all, const double* d2_all, const double* L_all,
                                  int64_t Nb, int64_t inner, int64_t s) {
  const int64_t b0 = sys_base(s, Nb, inner);
  Line<const T> f{b_all + b0, inner};
  Line<T> u{u_all + b0, inner};
  Line<const double> d0{d0_all + b0, inner}, d1{d1_all + b0, inner}, d2{d2_all + b0, inner},
      L{L_all + b0, inner};
  const int64_t N = Nb - 2;
  T y0 = f[0], y1 = f[1];
  u[0] = y0;
  u[1] = y1;
  for (int64_t i = 2; i < N; ++i) {
    T y = f[i] - mulr(y0, L[i - 2]);
    u[i] = y;
    y0 = y1;
    y1 = y;
  }
  T un1 = mulr(u[N - 1], 1.0 / d0[N - 1]);
  T un2 = mulr(u[N - 2], 1.0 / d0[N - 2]);
  u[N - 1] = un1;
  u[N - 2] = un2;
  T un3 = mulr(u[N - 3] - mulr(un1, d1[N - 3]), 1.0 / d0[N - 3]);
  T un4 = mulr(u[N - 4] - mulr(un2, d1[N - 4]), 1.0 / d0[N - 4]);
  u[N - 3] = un3;
  u[N - 4] = un4;
  // running state: u[i+2], u[i+4] of each parity
  T se = zero_of(T()), so = zero_of(T());
  T up2 = un3, up4 = un1;  // parity of N-5: u[N-3], u[N-1]
  T uq2 = un4, uq4 = un2;  // other parity: u[N-4], u[N-2]
  for (int64_t i = N - 5; i >= 0; --i) {
    T ui = u[i] - mulr(up2, d1[i]);
    if (i % 2 == 0) {
      se = se + up4;
      ui = ui - mulr(se, d2[i]);
    } else {
      so = so + up4;
      ui = ui - mulr(so, d2[i]);
    }
    ui = mulr(ui, 1.0 / d0[i]);
    u[i] = ui;
    // shift: the next i (i-1) has the other parity
    T t2 = uq2, t4 = uq4;
    uq4 = up2;
    uq2 = ui;
    up2 = t2;
    up4 = t4;
  }
  if (neumann) {
    // back from w_j = j^2 u_j (la.pyx:907-912)
    if (sn_zero_mode(d0[0])) u[0] = zero_of(T());
    for (int64_t i = 1; i < N; ++i) u[i] = divr(u[i], sn_col(i));
  }
}

// Helmholtz_Neumann_matvec (Matvec.pyx:722-800): b = (alfa A + beta B) v with
// A = ASNSN, B = BSNSN on the N-2 dofs, tail zero.  Row k needs
// S_k = sum_{j = k+2, k+4, ...} j^2 v_j, kept per parity while k descends.
template <class T>
SGPU_HD void helmholtz_neumann_matvec_prog(const T* v_all, T* b_all, const double* alfa,
                                           const double* beta, int64_t Nb, int64_t inner,
                                           int64_t s) {
  const int64_t b0 = sys_base(s, Nb, inner);
  Line<const T> v{v_all + b0, inner};
  Line<T> b{b_all + b0, inner};
  const int64_t M = Nb - 2;
  const double alf = alfa[s], bet = beta[s];
  const double pi = 3.141592653589793;
  T S[2] = {zero_of(T()), zero_of(T())};
  for (int64_t k = M - 1; k >= 0; --k) {
    const double kk = (double)k;
    const double akk = ((((-2.0 * pi) * (kk * kk)) * (kk + 1)) / (kk + 2));
    const double bkk = sn_h(k) + (sn_K2sq(k) * sn_K2sq(k)) * sn_h(k + 2);
    T acc = mulr(v[k], alf * akk + bet * bkk);
    if (k + 2 < M) {
      S[k & 1] = S[k & 1] + mulr(v[k + 2], sn_col(k + 2));
      acc = acc + mulr(v[k + 2], bet * (-sn_K2sq(k) * sn_h(k + 2)));
      acc = acc + mulr(S[k & 1], alf * (((-4.0 * pi) * (kk + 1)) / ((kk + 2) * (kk + 2))));
    }
    if (k >= 2) acc = acc + mulr(v[k - 2], bet * (-sn_K2sq(k - 2) * sn_h(k)));
    b[k] = acc;
  }
  b[M] = zero_of(T());
  b[M + 1] = zero_of(T());
}

// Poisson_Solve_ADD_1D_ptr (la.pyx:671-706): A u = b with A = scale * ASDSD,
// upper triangular, back substitution with one running sum per parity; the
// two boundary dofs are set to zero (homogeneous boundary values).
template <class T>
SGPU_HD void poisson_add_prog(const T* b_all, T* u_all, double scale, int64_t Nb, int64_t inner,
                              int64_t s) {
  const int64_t b0 = sys_base(s, Nb, inner);
  Line<const T> b{b_all + b0, inner};
  Line<T> u{u_all + b0, inner};
  const int64_t N = Nb - 2;
  T S[2] = {zero_of(T()), zero_of(T())};
  T up[2] = {zero_of(T()), zero_of(T())};  // last u of each parity
  for (int64_t k = N - 1; k >= 0; --k) {
    T uk = b[k];
    if (k <= N - 3) {
      S[k & 1] = S[k & 1] + up[k & 1];
      uk = uk - mulr(S[k & 1], hA2(k));
    }
    uk = divr(uk, hA0(k));
    up[k & 1] = uk;
    u[k] = uk;
  }
  if (!(scale - 1.0 < 1e-8 && scale - 1.0 > -1e-8))
    for (int64_t k = 0; k < N; ++k) u[k] = divr(u[k], scale);
  // ADDSolver.solve copies b into u and the kernel solves the N - 2 dofs
  // (chebyshev/la.py:17-20, la.pyx:671-706): the two boundary rows keep b's
  u[N] = b[N];
  u[N + 1] = b[N + 1];
}

// ANNSolver.__call__ (chebyshev/la.py:77-128): A u = b with A = scale * ASNSN,
// columns scaled by 1/j^2 (j >= 1), back substitution for k = N-1 .. 1 with
// one running sum per parity, u_k = w_k / k^2, then u /= scale and the
// constraint u_0 = c0; boundary dofs zero.
template <class T>
SGPU_HD void poisson_ann_prog(const T* b_all, T* u_all, double scale, double c0, int64_t Nb,
                              int64_t inner, int64_t s) {
  const int64_t b0 = sys_base(s, Nb, inner);
  Line<const T> b{b_all + b0, inner};
  Line<T> u{u_all + b0, inner};
  const int64_t N = Nb - 2;
  const double pi = 3.141592653589793;
  T S[2] = {zero_of(T()), zero_of(T())};
  T up[2] = {zero_of(T()), zero_of(T())};
  for (int64_t k = N - 1; k >= 1; --k) {
    const double kk = (double)k;
    const double d = ((((-2.0 * pi) * (kk * kk)) * (kk + 1)) / (kk + 2)) * (1.0 / sn_col(k));
    T wk = b[k];
    if (k <= N - 3) {
      const double d1 = ((-4.0 * pi) * (kk + 1)) * (1.0 / sn_col(k + 2));
      S[k & 1] = S[k & 1] + up[k & 1];
      wk = wk - mulr(S[k & 1], d1);
    }
    wk = divr(wk, d);
    up[k & 1] = wk;
    u[k] = divr(mulr(wk, 1.0 / sn_col(k)), scale);
  }
  u[0] = real_of(T(), c0);
  u[N] = zero_of(T());
  u[N + 1] = zero_of(T());
}

// Helmholtz_matvec_ptr (Matvec.pyx:656-695): b = (alfa A + beta B) v, tail zero.
template <class T>
SGPU_HD void helmholtz_matvec_prog(const T* v_all, T* b_all, const double* alfa,
                                   const double* beta, int64_t Nb, int64_t inner, int64_t s) {
  const int64_t b0 = sys_base(s, Nb, inner);
  Line<const T> v{v_all + b0, inner};
  Line<T> b{b_all + b0, inner};
  const int64_t M = Nb - 2;
  const double alf = alfa[s], bet = beta[s];
  const double h = 1.5707963267948966;
  int64_t k = M - 1;
  b[k] = mulr(v[k], hA0(k) * alf + hB0(k) * bet) - mulr(v[k - 2], h * bet);
  b[k - 1] = mulr(v[k - 1], hA0(k - 1) * alf + hB0(k - 1) * bet) - mulr(v[k - 3], h * bet);
  T s1 = zero_of(T()), s2 = zero_of(T());
  for (k = M - 3; k > 1; --k) {
    double p = hA2(k) * alf;
    if (k % 2 == 0) {
      s2 = s2 + v[k + 2];
      b[k] = mulr(v[k], hA0(k) * alf + hB0(k) * bet) - mulr(v[k - 2] + v[k + 2], h * bet) + mulr(s2, p);
    } else {
      s1 = s1 + v[k + 2];
      b[k] = mulr(v[k], hA0(k) * alf + hB0(k) * bet) - mulr(v[k - 2] + v[k + 2], h * bet) + mulr(s1, p);
    }
  }
  k = 1;
  s1 = s1 + v[k + 2];
  s2 = s2 + v[k + 1];
  b[k] = mulr(v[k], hA0(k) * alf + hB0(k) * bet) - mulr(v[k + 2], h * bet) + mulr(s1, hA2(k) * alf);
  b[k - 1] = mulr(v[k - 1], hA0(k - 1) * alf + hB0(k - 1) * bet) - mulr(v[k + 1], h * bet) +
             mulr(s2, hA2(k - 1) * alf);
  b[M] = zero_of(T());
  b[M + 1] = zero_of(T());
}

// ---- non-homogeneous boundary values (sgpu_bc_apply) -----------------------
// Line s of u: u[k] -= (alfa_s CA[k][0] + beta_s CB[k][0]) g0 + (...[1]) g1
// for the dofs k < N-2 (tables row-major (N-2) x 2, NULL = absent, NULL
// scales = 1), then optionally the boundary dofs u[N-2], u[N-1] = g0, g1.
// g holds the two values of every line as g[o][0|1][i].
SGPU_HD bool is_zero(double a) { return a == 0.0; }
SGPU_HD bool is_zero(cd a) { return a.re == 0.0 && a.im == 0.0; }

template <class T>
SGPU_HD void bc_apply_prog(T* u, const double* CA, const double* alfa, const double* CB,
                           const double* beta, const T* g, int64_t N, int64_t inner, int64_t s,
                           int set_dofs) {
  const int64_t o = s / inner, i = s - o * inner;
  const T g0 = g[(o * 2) * inner + i], g1 = g[(o * 2 + 1) * inner + i];
  Line<T> line{u + sys_base(s, N, inner), inner};
  const int64_t dim = N - 2;
  if (set_dofs) {
    line[dim] = g0;
    line[dim + 1] = g1;
  }
  if (!(CA || CB) || (is_zero(g0) && is_zero(g1))) return;
  const double a = alfa ? alfa[s] : 1.0, b = beta ? beta[s] : 1.0;
  for (int64_t k = 0; k < dim; ++k) {
    double c0 = 0.0, c1 = 0.0;
    if (CA) {
      c0 = a * CA[2 * k];
      c1 = a * CA[2 * k + 1];
    }
    if (CB) {
      c0 += b * CB[2 * k];
      c1 += b * CB[2 * k + 1];
    }
    if (c0 != 0.0 || c1 != 0.0) line[k] = line[k] - (mulr(g0, c0) + mulr(g1, c1));
  }
}

// ---- banded + rank-2 upper semiseparable systems ---------------------------
// One system per Fourier wavenumber: M = sum_t c_t M_t over up to 3 terms,
// where every M_t has even offsets in {-4, -2, 0, 2, 4} and at most one term
// (gen_term) also has a strictly-upper part of the form
//   M_t[k][j] = p_k q_j + r_k t_j     for j >= k + 2, j - k even.
// This covers every per-wavenumber system of the Galerkin spaces here:
// Chebyshev ShenBiharmonic a0 S + alpha A + beta B (S = SSBSB: rank-2 upper,
// chebyshev/matrices.py:1444-1458), Chebyshev ShenDirichlet alpha A + beta B
// (A = ASDSD: constant rows, rank 1), Legendre ShenDirichlet/ShenBiharmonic
// (banded only, la.py TDMA/PDMA).  Even and odd unknowns decouple; each
// parity is a chain with offsets -2..2 in chain index.
//
// Gaussian elimination without pivoting keeps the structure: row c of U is
// diag_c, band entries corr1_c (column c+1), corr2_c (column c+2) and the
// generator part P_c q_j + R_c t_j for j >= c+1; L has two sub-diagonals
// (L1, L0).  Eliminating column c from rows c+1 and c+2 only rescales their
// generator coefficients (P, R) and touches O(1) band entries, so factor and
// solve are O(n) per chain.  (The reference's tailored Chebyshev solvers
// LU_Helmholtz / LU_Biharmonic, la.pyx:717-763 and la.pyx:975-1233, exploit
// the same structure with running sums; the reference's generic path for
// these systems is a sparse LU per wavenumber, la.py:1231-1364.)
//
template <class R>
SGPU_HD R store_cast(double x);
template <>
SGPU_HD double store_cast<double>(double x) { return x; }
template <>
SGPU_HD df store_cast<df>(double x) { return df_from_double(x); }
template <>
SGPU_HD float store_cast<float>(double x) {
  // round to nearest (a one-off cost of the factorisation)
  return (float)x;
}

// Factor cache: fac[q][c][chain], q = L0, L1, 1/diag, corr1, corr2, P, R,
// chain = 2 * system + parity, c < m = (n + 1) / 2.
struct BandSepDesc {
  int n;                 // unknowns (dofs) per system
  int nterms;            // <= 3
  int gen_term;          // term with the semiseparable upper part, -1 if none
  const double* bands;   // [nterms][5][n]: offsets -4, -2, 0, 2, 4 at row k
  const double* gens;    // [4][n]: p_k, q_j, r_k, t_j of gen_term
  const double* coef;    // [nterms][nsys]
};

SGPU_HD double bs_band(const BandSepDesc& d, int64_t nsys, int64_t s, int off_idx, int k) {
  double v = 0.0;
  for (int t = 0; t < d.nterms; ++t)
    v += d.coef[t * nsys + s] * d.bands[((size_t)t * 5 + off_idx) * d.n + k];
  return v;
}

template <class F = double>
SGPU_HD void band_sep_factor_prog(const BandSepDesc& d, F* fac, int64_t nsys, int64_t chain) {
  const int64_t s = chain >> 1;
  const int par = (int)(chain & 1);
  const int n = d.n;
  const int m = (n + 1) / 2;
  const int64_t nch = 2 * nsys;
  const double cg = d.gen_term >= 0 ? d.coef[d.gen_term * nsys + s] : 0.0;
  const double* gp = d.gens;
  const double* gq = d.gens ? d.gens + n : nullptr;
  const double* gr = d.gens ? d.gens + 2 * n : nullptr;
  const double* gt = d.gens ? d.gens + 3 * n : nullptr;
  // window rows c, c+1, c+2: sub2, sub1, diag, corr1, corr2, P, R
  double W[3][7];
  auto load_row = [&](double* r, int c) {
    const int k = 2 * c + par;
    if (k >= n) {
      for (int i = 0; i < 7; ++i) r[i] = 0.0;
      return;
    }
    r[0] = bs_band(d, nsys, s, 0, k);
    r[1] = bs_band(d, nsys, s, 1, k);
    r[2] = bs_band(d, nsys, s, 2, k);
    r[3] = bs_band(d, nsys, s, 3, k);
    r[4] = bs_band(d, nsys, s, 4, k);
    r[5] = d.gens ? cg * gp[k] : 0.0;
    r[6] = d.gens ? cg * gr[k] : 0.0;
  };
  auto Q = [&](int c) { const int k = 2 * c + par; return (d.gens && k < n) ? gq[k] : 0.0; };
  auto T = [&](int c) { const int k = 2 * c + par; return (d.gens && k < n) ? gt[k] : 0.0; };
  load_row(W[0], 0);
  load_row(W[1], 1);
  load_row(W[2], 2);
  for (int c = 0; c < m; ++c) {
    double* r0 = W[c % 3];
    double* r1 = W[(c + 1) % 3];
    double* r2 = W[(c + 2) % 3];
    const double piv = r0[2];
    const double dinv = 1.0 / piv;
    const double u1 = r0[3] + r0[5] * Q(c + 1) + r0[6] * T(c + 1);  // U(c, c+1)
    const double u2 = r0[4] + r0[5] * Q(c + 2) + r0[6] * T(c + 2);  // U(c, c+2)
    double l1 = 0.0, l0 = 0.0;
    if (c + 1 < m) {
      l1 = r1[1] * dinv;
      r1[2] -= l1 * u1;
      r1[3] -= l1 * r0[4];
      r1[5] -= l1 * r0[5];
      r1[6] -= l1 * r0[6];
    }
    if (c + 2 < m) {
      l0 = r2[0] * dinv;
      r2[1] -= l0 * u1;
      r2[2] -= l0 * u2;
      r2[5] -= l0 * r0[5];
      r2[6] -= l0 * r0[6];
    }
    // multipliers belong to the rows they eliminate
    if (c + 1 < m) fac[((size_t)1 * m + c + 1) * nch + chain] = store_cast<F>(l1);
    if (c + 2 < m) fac[((size_t)0 * m + c + 2) * nch + chain] = store_cast<F>(l0);
    if (c == 0) {
      fac[((size_t)1 * m + 0) * nch + chain] = store_cast<F>(0.0);
      fac[((size_t)0 * m + 0) * nch + chain] = store_cast<F>(0.0);
      if (m > 1) fac[((size_t)0 * m + 1) * nch + chain] = store_cast<F>(0.0);
    }
    fac[((size_t)2 * m + c) * nch + chain] = store_cast<F>(dinv);
    fac[((size_t)3 * m + c) * nch + chain] = store_cast<F>(r0[3]);
    fac[((size_t)4 * m + c) * nch + chain] = store_cast<F>(r0[4]);
    fac[((size_t)5 * m + c) * nch + chain] = store_cast<F>(r0[5]);
    fac[((size_t)6 * m + c) * nch + chain] = store_cast<F>(r0[6]);
    load_row(r0, c + 3);  // slot of row c becomes row c+3
  }
}

template <class T>
SGPU_HD void band_sep_solve_prog(const T* b_all, T* u_all, const double* fac, const double* gens,
                                 int n, int64_t Nb, int64_t inner, int64_t nsys, int64_t chain) {
  // rows prefetched PF at a time, as in the Helmholtz cached solve (the loads
  // do not depend on the recurrence; each row is read before it is written)
  constexpr int PF = 4;
  const int64_t s = chain >> 1;
  const int par = (int)(chain & 1);
  const int m = (n + 1) / 2;
  const int64_t nch = 2 * nsys;
  const int64_t base = sys_base(s, Nb, inner);
  const T* f = b_all + base;
  T* u = u_all + base;
  auto F = [&](int q, int c) { return fac[((size_t)q * m + c) * nch + chain]; };
  const int cend = (n - par + 1) / 2;  // chain rows k = 2c + par < n
  T y1 = zero_of(T()), y2 = zero_of(T());  // y_{c-1}, y_{c-2}
  for (int c0 = 0; c0 < cend; c0 += PF) {
    T fv[PF];
    double l1[PF], l0[PF];
#pragma unroll
    for (int j = 0; j < PF; ++j) {
      const int c = c0 + j;
      if (c < cend) {
        fv[j] = f[(2 * c + par) * inner];
        l1[j] = F(1, c);
        l0[j] = F(0, c);
      }
    }
#pragma unroll
    for (int j = 0; j < PF; ++j) {
      const int c = c0 + j;
      if (c < cend) {
        T y = fv[j] - mulr(y1, l1[j]) - mulr(y2, l0[j]);
        u[(2 * c + par) * inner] = y;
        y2 = y1;
        y1 = y;
      }
    }
  }
  T sq = zero_of(T()), st = zero_of(T());  // sum_{j >= c+1} q_j u_j, t_j u_j
  T up1 = zero_of(T()), up2 = zero_of(T());
  for (int c0 = cend - 1; c0 >= 0; c0 -= PF) {
    T yv[PF];
    double dv[PF], e1[PF], e2[PF], p5[PF], p6[PF], gq[PF], gt[PF];
#pragma unroll
    for (int j = 0; j < PF; ++j) {
      const int c = c0 - j;
      if (c >= 0) {
        const int k = 2 * c + par;
        yv[j] = u[k * inner];
        dv[j] = F(2, c);
        e1[j] = F(3, c);
        e2[j] = F(4, c);
        if (gens) {
          p5[j] = F(5, c);
          p6[j] = F(6, c);
          gq[j] = gens[n + k];
          gt[j] = gens[3 * n + k];
        }
      }
    }
#pragma unroll
    for (int j = 0; j < PF; ++j) {
      const int c = c0 - j;
      if (c >= 0) {
        T v = yv[j] - mulr(up1, e1[j]) - mulr(up2, e2[j]);
        if (gens) v = v - mulr(sq, p5[j]) - mulr(st, p6[j]);
        v = mulr(v, dv[j]);
        u[(2 * c + par) * inner] = v;
        if (gens) {
          sq = sq + mulr(v, gq[j]);
          st = st + mulr(v, gt[j]);
        }
        up2 = up1;
        up1 = v;
      }
    }
  }
}

// c = M v with M = sum_t coef_t M_t (the matrix the factor/solve above
// inverts): the residual Biharmonic_matvec (Matvec.pyx:908-1010) computes for
// Chebyshev ShenBiharmonic, and the same product for every other
// per-wavenumber system here.  One thread per (system, parity) chain, rows
// descending so that the semiseparable part is two running sums
// sum_{j >= k+2} q_j v_j and t_j v_j.  Entries k >= n of each line are zeroed.
template <class T>
SGPU_HD void band_sep_matvec_prog(const BandSepDesc& d, const T* v_all, T* c_all, int64_t Nb,
                                  int64_t inner, int64_t nsys, int64_t chain) {
  const int64_t s = chain >> 1;
  const int par = (int)(chain & 1);
  const int n = d.n;
  const int64_t base = sys_base(s, Nb, inner);
  const T* v = v_all + base;
  T* c = c_all + base;
  const double cg = d.gen_term >= 0 ? d.coef[d.gen_term * nsys + s] : 0.0;
  const double* gp = d.gens;
  const double* gq = d.gens ? d.gens + n : nullptr;
  const double* gr = d.gens ? d.gens + 2 * n : nullptr;
  const double* gt = d.gens ? d.gens + 3 * n : nullptr;
  T sq = zero_of(T()), st = zero_of(T());
  int top = n - 1;
  if ((top & 1) != par) --top;
  for (int k = top; k >= 0; k -= 2) {
    if (d.gens && k + 2 < n) {
      const T vk2 = v[(k + 2) * inner];
      sq = sq + mulr(vk2, gq[k + 2]);
      st = st + mulr(vk2, gt[k + 2]);
    }
    T acc = zero_of(T());
#pragma unroll
    for (int o = 0; o < 5; ++o) {
      const int j = k + 2 * o - 4;
      if (j >= 0 && j < n) acc = acc + mulr(v[j * inner], bs_band(d, nsys, s, o, k));
    }
    if (d.gens) acc = acc + mulr(sq, cg * gp[k]) + mulr(st, cg * gr[k]);
    c[k * inner] = acc;
  }
  for (int64_t k = n + par; k < Nb; k += 2) c[k * inner] = zero_of(T());
}

// ---- factorisation cache: interleaved, reciprocal-pivot layout -------------
// fac[q][k][s] for q = 0..3 (L, 1/d0, d1, d2), k in [0, M), s a system:
// consecutive systems are contiguous, so thread s reads row k coalesced.
// Entries are FP64 (plain form) or double-float pairs (mixed form); both are
// 8 bytes.  The LU itself is computed in FP64 in the reference's order
// (la.pyx:717-763) and only then stored.
template <class R>
SGPU_HD void helmholtz_factor_prog(int64_t N, const double* alfa, const double* beta, int neumann,
                                   R* fac, int64_t nsys, int64_t s) {
  const int64_t M = N - 2;
  const double a = alfa[s], b = beta[s];
  R* FL = fac;
  R* FD = fac + M * nsys;
  R* F1 = fac + 2 * M * nsys;
  R* F2 = fac + 3 * M * nsys;
  double d0m2 = 0, d1m2 = 0, d2m2 = 0, d0m1 = 0, d1m1 = 0, d2m1 = 0;  // rows i-2, i-1
  double bm2m2 = 0, bm2m1 = 0;  // B(i, i-2) of rows i-2, i-1 (column-scaled)
  for (int64_t i = 0; i < M; ++i) {
    HelmRow r = helm_row(i, neumann);
    if (i == 0 && neumann && sn_singular(b)) {
      r.A0 = 1.0 / a;
      r.B0 = 0.0;
    }
    double l = 0, d0, d1 = 0, d2 = 0;
    if (i < 2) {
      d0 = a * r.A0 + b * r.B0;
      d1 = a * r.A2 + b * r.B2;
      d2 = a * r.A4;
    } else {
      l = b * bm2m2 / d0m2;
      d0 = a * r.A0 + b * r.B0 - l * d1m2;
      if (i < M - 2) d1 = a * r.A2 + b * r.B2 - l * d2m2;
      if (i < M - 4) d2 = a * r.A4 - l * d2m2;
    }
    FL[i * nsys + s] = store_cast<R>(l);
    // a Neumann zero mode is solved as u_0 = 0 (la.pyx:907-909): a zero
    // reciprocal pivot gives exactly that
    const bool zero_mode = neumann && i == 0 && sn_zero_mode(d0);
    FD[i * nsys + s] = store_cast<R>(zero_mode ? 0.0 : 1.0 / d0);
    F1[i * nsys + s] = store_cast<R>(d1);
    F2[i * nsys + s] = store_cast<R>(d2);
    d0m2 = d0m1; d1m2 = d1m1; d2m2 = d2m1;
    d0m1 = d0; d1m1 = d1; d2m1 = d2;
    bm2m2 = bm2m1;
    bm2m1 = r.Bm2;
  }
}

// Solve with cached factors, one thread per (system, parity): the even and
// odd unknowns of a Chebyshev Dirichlet Helmholtz system are decoupled, so
// each parity chain runs Solve_Helmholtz_1D_ptr's recurrences (la.pyx:871-912)
// independently.  T is the element type in memory (double or complex
// double), R the arithmetic (double or df).
template <class R, class T>
struct ElemOps;
// acc - a s with one rounding in FP64 (an explicit FMA: the result does not
// depend on how a compiler contracts it in each kernel that inlines the
// program, so every kernel running a program gives the same bits)
SGPU_HD double fms(double acc, double a, double s) {
#ifdef __CUDA_ARCH__
  return __fma_rn(-a, s, acc);
#else
  return std::fma(-a, s, acc);
#endif
}
SGPU_HD df fms(df acc, df a, df s) { return acc - a * s; }
// the FP32 sweeps of the refined solves: one FP32 FMA (without this overload
// the float arguments would promote to the FP64 one)
SGPU_HD float fms(float acc, float a, float s) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(-a, s, acc);
#else
  return std::fmaf(-a, s, acc);
#endif
}

template <class R>
struct ElemOps<R, double> {
  typedef R V;
  static SGPU_HD V load(const double* p) { return from_f64<R>(*p); }
  static SGPU_HD void store(double* p, V v) { *p = to_f64(v); }
  static SGPU_HD V zero() { return R(0.0); }
  static SGPU_HD V mul(V a, R s) { return a * s; }
  static SGPU_HD V msub(V acc, V a, R s) { return fms(acc, a, s); }
};
template <class R>
struct ElemOps<R, cd> {
  typedef Cx<R> V;
  static SGPU_HD V load(const cd* p) { return cx<R>(from_f64<R>(p->re), from_f64<R>(p->im)); }
  static SGPU_HD void store(cd* p, V v) { *p = cx<double>(to_f64(v.re), to_f64(v.im)); }
  static SGPU_HD V zero() { return cx<R>(R(0.0), R(0.0)); }
  static SGPU_HD V mul(V a, R s) { return scale(a, s); }
  static SGPU_HD V msub(V acc, V a, R s) { return cx<R>(fms(acc.re, a.re, s), fms(acc.im, a.im, s)); }
};

template <class R>
SGPU_HD R fac_at(const R* fac, int64_t q, int64_t k, int64_t M, int64_t nsys, int64_t s) {
  return fac[(q * M + k) * nsys + s];
}

// Both sweeps prefetch SOLVE_PF rows of their chain into registers before
// running the recurrence over them: the loads do not depend on the
// recurrence, so a thread keeps SOLVE_PF requests in flight instead of one
// (the solve is bound by memory latency, not bandwidth, with one thread per
// chain).  Rows are read before they are written in both sweeps, so b may
// alias u.
constexpr int SOLVE_PF = 8;

template <class R, class T>
SGPU_HD void helmholtz_cached_solve_prog(const T* b_all, T* u_all, const R* fac, int neumann,
                                         int64_t Nb, int64_t inner, int64_t nsys, int64_t s,
                                         int par) {
  typedef ElemOps<R, T> E;
  typedef typename E::V V;
  const int64_t M = Nb - 2;
  const int64_t base = sys_base(s, Nb, inner);
  const T* f = b_all + base;
  T* u = u_all + base;
  // forward sweep y_i = f_i - L_{i-2} y_{i-2} along the chain i = par, par+2, ...
  // (row i stores the multiplier the reference keeps in L[i-2])
  V y = E::zero();
  int64_t top = par;
  for (int64_t i0 = par; i0 < M; i0 += 2 * SOLVE_PF) {
    V fv[SOLVE_PF];
    R lv[SOLVE_PF];
#pragma unroll
    for (int j = 0; j < SOLVE_PF; ++j) {
      const int64_t i = i0 + 2 * j;
      if (i < M) {
        fv[j] = E::load(f + i * inner);
        lv[j] = fac_at(fac, 0, i, M, nsys, s);
      }
    }
#pragma unroll
    for (int j = 0; j < SOLVE_PF; ++j) {
      const int64_t i = i0 + 2 * j;
      if (i < M) {
        V fi = fv[j];
        if (i >= 2) fi = E::msub(fi, y, lv[j]);
        y = fi;
        E::store(u + i * inner, y);
        top = i;
      }
    }
  }
  // back substitution from the top of the chain
  V up2 = E::zero(), S = E::zero(), pend = E::zero();  // u_{i+2}; sum of u_{>=i+4}
  bool have2 = false;
  for (int64_t i0 = top; i0 >= 0; i0 -= 2 * SOLVE_PF) {
    V yv[SOLVE_PF];
    R dv[SOLVE_PF], d1v[SOLVE_PF], d2v[SOLVE_PF];
#pragma unroll
    for (int j = 0; j < SOLVE_PF; ++j) {
      const int64_t i = i0 - 2 * j;
      if (i >= 0) {
        yv[j] = E::load(u + i * inner);
        dv[j] = fac_at(fac, 1, i, M, nsys, s);
        d1v[j] = fac_at(fac, 2, i, M, nsys, s);
        d2v[j] = fac_at(fac, 3, i, M, nsys, s);
      }
    }
#pragma unroll
    for (int j = 0; j < SOLVE_PF; ++j) {
      const int64_t i = i0 - 2 * j;
      if (i >= 0) {
        V ui = yv[j];
        if (have2) ui = E::msub(ui, up2, d1v[j]);
        if (i <= M - 5) {
          S = S + pend;
          ui = E::msub(ui, S, d2v[j]);
        }
        ui = E::mul(ui, dv[j]);
        // Neumann: the recurrences run on w_i = i^2 u_i
        E::store(u + i * inner, (neumann && i >= 1) ? E::mul(ui, from_f64<R>(1.0 / sn_col(i))) : ui);
        pend = up2;
        up2 = ui;
        have2 = true;
      }
    }
  }
}

// ---- FP32 solves with FP64 iterative refinement ------------------------------
// The chosen form of the banded solves: the factor cache is FP32 (half the
// bytes of the FP64 one; the LU is still computed in FP64 and rounded once),
// the sweeps run in FP32, and a residual in FP64-level arithmetic (R = double
// on the FP64 pipe, or R = df, double-float on the FP32 pipes) drives the
// correction: u = A32^-1 f; repeat r = f - A u, d = A32^-1 r, u += d until
// max|d| <= tol max|u| (or max_it corrections).  One thread per (system,
// parity) chain: the Chebyshev Dirichlet Helmholtz and ShenBiharmonic
// systems decouple by parity, so the whole loop runs on the chain.

// magnitude bound used by the stopping test (max of |re|, |im|)
SGPU_HD double mag(double a) { return a < 0 ? -a : a; }
SGPU_HD double mag(cd a) {
  const double x = a.re < 0 ? -a.re : a.re, y = a.im < 0 ? -a.im : a.im;
  return x > y ? x : y;
}

// r = f - (alfa A + beta B) u on the chain k = par, par+2, .. < M of a
// ShenDirichlet Helmholtz line (the rows of helmholtz_matvec_prog), in
// arithmetic R; rows descending so that sum_{j >= k+2} u_j is a running sum
template <class R, class T>
SGPU_HD void helmholtz_residual_chain(const T* f, const T* u, T* r, double alf, double bet, int64_t M,
                                      int64_t inner, int par) {
  typedef ElemOps<R, T> E;
  typedef typename E::V V;
  const double h = 1.5707963267948966;
  int64_t top = M - 1;
  if ((top & 1) != par) --top;
  V S = E::zero();                  // sum of u_j, j >= k+2 on the chain
  V up2 = E::zero(), uk = E::zero();
  bool have = false;
  if (top >= 0) uk = E::load(u + top * inner);
  for (int64_t k = top; k >= 0; k -= 2) {
    const V um2 = k >= 2 ? E::load(u + (k - 2) * inner) : E::zero();
    V acc = E::mul(uk, from_f64<R>(hA0(k) * alf + hB0(k) * bet));
    if (k >= 2) acc = acc - E::mul(um2, from_f64<R>(h * bet));
    if (have) {
      S = S + up2;
      acc = acc - E::mul(up2, from_f64<R>(h * bet)) + E::mul(S, from_f64<R>(hA2(k) * alf));
    }
    E::store(r + k * inner, E::load(f + k * inner) - acc);
    up2 = uk;
    uk = um2;
    have = true;
  }
}

// u += d on the chain (FP64), returning max|d| and max|u| (after the update)
template <class T>
SGPU_HD void chain_update(T* u, const T* d, int64_t M, int64_t inner, int par, double& dmax, double& umax) {
  dmax = 0.0;
  umax = 0.0;
  for (int64_t k = par; k < M; k += 2) {
    const T dk = d[k * inner];
    const T uk = u[k * inner] + dk;
    u[k * inner] = uk;
    const double a = mag(dk), b = mag(uk);
    dmax = a > dmax ? a : dmax;
    umax = b > umax ? b : umax;
  }
}

// the whole refinement of one Helmholtz chain; returns the corrections applied
template <class R, class T>
SGPU_HD int helmholtz_refine_prog(const T* f_all, T* u_all, T* r_all, const float* fac32, const double* alfa,
                                  const double* beta, int64_t Nb, int64_t inner, int64_t nsys, int64_t s,
                                  int par, double tol, int max_it) {
  const int64_t M = Nb - 2;
  const int64_t base = sys_base(s, Nb, inner);
  helmholtz_cached_solve_prog<float, T>(f_all, u_all, fac32, 0, Nb, inner, nsys, s, par);
  int it = 0;
  while (it < max_it) {
    helmholtz_residual_chain<R, T>(f_all + base, u_all + base, r_all + base, alfa[s], beta[s], M, inner, par);
    helmholtz_cached_solve_prog<float, T>(r_all, r_all, fac32, 0, Nb, inner, nsys, s, par);
    double dmax, umax;
    chain_update(u_all + base, r_all + base, M, inner, par, dmax, umax);
    ++it;
    if (dmax <= tol * umax) break;
  }
  return it;
}

// band_sep_solve_prog in arithmetic R from a factor cache of R entries (the
// FP32 sweeps of the refined biharmonic / generic solves)
template <class R, class T>
SGPU_HD void band_sep_solve_gen(const T* b_all, T* u_all, const R* fac, const double* gens, int n, int64_t Nb,
                                int64_t inner, int64_t nsys, int64_t chain) {
  typedef ElemOps<R, T> E;
  typedef typename E::V V;
  const int64_t s = chain >> 1;
  const int par = (int)(chain & 1);
  const int m = (n + 1) / 2;
  const int64_t nch = 2 * nsys;
  const int64_t base = sys_base(s, Nb, inner);
  const T* f = b_all + base;
  T* u = u_all + base;
  auto F = [&](int q, int c) { return fac[((size_t)q * m + c) * nch + chain]; };
  const int cend = (n - par + 1) / 2;
  V y1 = E::zero(), y2 = E::zero();
  for (int c = 0; c < cend; ++c) {
    const V y = E::load(f + (2 * c + par) * inner) - E::mul(y1, F(1, c)) - E::mul(y2, F(0, c));
    E::store(u + (2 * c + par) * inner, y);
    y2 = y1;
    y1 = y;
  }
  V sq = E::zero(), st = E::zero(), up1 = E::zero(), up2 = E::zero();
  for (int c = cend - 1; c >= 0; --c) {
    const int k = 2 * c + par;
    V v = E::load(u + k * inner) - E::mul(up1, F(3, c)) - E::mul(up2, F(4, c));
    if (gens) v = v - E::mul(sq, F(5, c)) - E::mul(st, F(6, c));
    v = E::mul(v, F(2, c));
    E::store(u + k * inner, v);
    if (gens) {
      sq = sq + E::mul(v, from_f64<R>(gens[n + k]));
      st = st + E::mul(v, from_f64<R>(gens[3 * n + k]));
    }
    up2 = up1;
    up1 = v;
  }
}

// the whole refinement of one banded + semiseparable chain (biharmonic,
// Legendre, generic systems): FP32 sweeps, FP64 residual from the matvec
template <class T>
SGPU_HD int band_sep_refine_prog(const BandSepDesc& d, const T* f_all, T* u_all, T* r_all, const float* fac32,
                                 int64_t Nb, int64_t inner, int64_t nsys, int64_t chain, double tol, int max_it) {
  const int64_t s = chain >> 1;
  const int par = (int)(chain & 1);
  const int64_t base = sys_base(s, Nb, inner);
  band_sep_solve_gen<float, T>(f_all, u_all, fac32, d.gens, d.n, Nb, inner, nsys, chain);
  int it = 0;
  while (it < max_it) {
    band_sep_matvec_prog<T>(d, u_all, r_all, Nb, inner, nsys, chain);  // r = M u on the chain
    for (int64_t k = par; k < d.n; k += 2) r_all[base + k * inner] = f_all[base + k * inner] - r_all[base + k * inner];
    band_sep_solve_gen<float, T>(r_all, r_all, fac32, d.gens, d.n, Nb, inner, nsys, chain);
    double dmax, umax;
    chain_update(u_all + base, r_all + base, d.n, inner, par, dmax, umax);
    ++it;
    if (dmax <= tol * umax) break;
  }
  return it;
}

}  // namespace sgpu
