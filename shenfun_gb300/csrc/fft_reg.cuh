// Register-resident two-pass FFT for line lengths m = P * Q (P, Q in
// {4, 8, 16, 32}): the fast path of the line transforms for the common
// power-of-two lengths (64 ... 1024, and 256 inside Rader's length-257 DFT).
//
// With n = Q n1 + n2 and k = k1 + P k2 (Cooley-Tukey "four-step" inside one
// line):  X[k1 + P k2] = sum_n2 W_m^{n2 k1} W_Q^{n2 k2} sum_n1 x[Q n1 + n2] W_P^{n1 k1}.
//   pass 1: thread (line, n2) loads x[Q n1 + n2] (n1 = 0..P-1, consecutive
//           threads read consecutive words), runs a P-point DFT in registers,
//           multiplies by W_m^{n2 k1} and stores Z[k1][n2] with a padded row
//           stride Q + 1 (conflict-free for the transposed read that follows);
//   pass 2: thread (line, k1) loads Z[k1][0..Q-1], runs a Q-point DFT in
//           registers and stores X[k1 + P k2].
// Two shared-memory exchanges and two barriers per line instead of one per
// radix-4 stage, no integer division in the inner loops, compile-time DFT
// constants.
//
// Included by fft_line.cuh after LinePlan, the table accessors and the small
// DFT kernels are defined.
#pragma once

namespace sgpu {

// exp(-2 pi i j / 16) for j = 0..15 as compile-time constants
template <class R>
SGPU_HD Cx<R> w16(int j) {
  // cos / sin of 2 pi j / 16 (correctly rounded decimal expansions)
  const double c1 = 0.92387953251128675612818318939678829;
  const double s1 = 0.38268343236508977172845998403039887;
  const double h = 0.70710678118654752440084436210484904;
  switch (j & 15) {
    case 0: return cx<R>(R(1.0), R(0.0));
    case 1: return cx<R>(R(c1), R(-s1));
    case 2: return cx<R>(R(h), R(-h));
    case 3: return cx<R>(R(s1), R(-c1));
    case 4: return cx<R>(R(0.0), R(-1.0));
    case 5: return cx<R>(R(-s1), R(-c1));
    case 6: return cx<R>(R(-h), R(-h));
    case 7: return cx<R>(R(-c1), R(-s1));
    case 8: return cx<R>(R(-1.0), R(0.0));
    case 9: return cx<R>(R(-c1), R(s1));
    case 10: return cx<R>(R(-h), R(h));
    case 11: return cx<R>(R(-s1), R(c1));
    case 12: return cx<R>(R(0.0), R(1.0));
    case 13: return cx<R>(R(s1), R(c1));
    case 14: return cx<R>(R(h), R(h));
    default: return cx<R>(R(c1), R(s1));
  }
}

// multiply by exp(-2 pi i j / 16) with the trivial cases specialised
template <class R>
SGPU_HD Cx<R> mul_w16(Cx<R> a, int j) {
  switch (j & 15) {
    case 0: return a;
    case 4: return mul_mi(a);
    case 8: return cx<R>(-a.re, -a.im);
    case 12: return mul_pi(a);
    default: return a * w16<R>(j);
  }
}

// In-register forward DFTs of size 2, 4, 8, 16, 32 on v[0..P-1] (natural order).
template <class R, int P>
struct RegDFT;

template <class R>
struct RegDFT<R, 2> {
  static SGPU_HD void run(Cx<R>* v) { dft2(v); }
};

template <class R>
struct RegDFT<R, 4> {
  static SGPU_HD void run(Cx<R>* v) { dft4(v); }
};

// size 8 = 2 x 4: n = 4 n1 + n2 -> k = k1 + 2 k2
template <class R>
struct RegDFT<R, 8> {
  static SGPU_HD void run(Cx<R>* v) {
    Cx<R> a[4][2];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
      Cx<R> t[2] = {v[n2], v[4 + n2]};
      dft2(t);
      a[n2][0] = t[0];
      a[n2][1] = mul_w16<R>(t[1], 2 * n2);  // W_8^{n2 k1}, k1 = 1
    }
#pragma unroll
    for (int k1 = 0; k1 < 2; ++k1) {
      Cx<R> t[4] = {a[0][k1], a[1][k1], a[2][k1], a[3][k1]};
      dft4(t);
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) v[k1 + 2 * k2] = t[k2];
    }
  }
};

// size 16 = 4 x 4: n = 4 n1 + n2 -> k = k1 + 4 k2
template <class R>
struct RegDFT<R, 16> {
  static SGPU_HD void run(Cx<R>* v) {
    Cx<R> a[4][4];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
      Cx<R> t[4] = {v[n2], v[4 + n2], v[8 + n2], v[12 + n2]};
      dft4(t);
#pragma unroll
      for (int k1 = 0; k1 < 4; ++k1) a[n2][k1] = mul_w16<R>(t[k1], n2 * k1);
    }
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
      Cx<R> t[4] = {a[0][k1], a[1][k1], a[2][k1], a[3][k1]};
      dft4(t);
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[k2];
    }
  }
};

// Two-pass FFT of `lines` lines of length P*Q in src (stride ld); the padded
// exchange buffer tmp holds lines * P * (Q + 1) entries.  Result in src.
template <class R, int P, int Q>
SGPU_HD void fft_two_pass(const LinePlan& p, Cx<R>* src, Cx<R>* tmp, int lines, int tid,
                          int nth) {
  const int QP = Q + 1;
  // pass 1: P-point DFTs over n1
  for (int e = tid; e < lines * Q; e += nth) {
    const int t = e / Q, n2 = e - t * Q;
    const Cx<R>* x = src + (size_t)t * p.ld;
    Cx<R> v[P];
#pragma unroll
    for (int n1 = 0; n1 < P; ++n1) v[n1] = x[Q * n1 + n2];
    RegDFT<R, P>::run(v);
    Cx<R>* z = tmp + (size_t)t * P * QP;
    z[n2] = v[0];
#pragma unroll
    for (int k1 = 1; k1 < P; ++k1) z[k1 * QP + n2] = v[k1] * tw_at<R>(p, n2 * k1);
  }
  SGPU_SYNC();
  // pass 2: Q-point DFTs over n2
  for (int e = tid; e < lines * P; e += nth) {
    const int t = e / P, k1 = e - t * P;
    const Cx<R>* z = tmp + (size_t)t * P * QP + k1 * QP;
    Cx<R> v[Q];
#pragma unroll
    for (int n2 = 0; n2 < Q; ++n2) v[n2] = z[n2];
    RegDFT<R, Q>::run(v);
    Cx<R>* X = src + (size_t)t * p.ld;
#pragma unroll
    for (int k2 = 0; k2 < Q; ++k2) X[k1 + P * k2] = v[k2];
  }
  SGPU_SYNC();
}

// Returns true (and transforms src in place) when m has a two-pass split.
template <class R>
SGPU_HD bool fft_fast(const LinePlan& p, Cx<R>* src, Cx<R>* tmp, int lines, int tid, int nth) {
  switch (p.m) {
    case 16: fft_two_pass<R, 4, 4>(p, src, tmp, lines, tid, nth); return true;
    case 32: fft_two_pass<R, 4, 8>(p, src, tmp, lines, tid, nth); return true;
    case 64: fft_two_pass<R, 8, 8>(p, src, tmp, lines, tid, nth); return true;
    case 128: fft_two_pass<R, 8, 16>(p, src, tmp, lines, tid, nth); return true;
    case 256: fft_two_pass<R, 16, 16>(p, src, tmp, lines, tid, nth); return true;
    default: return false;
  }
}

}  // namespace sgpu
