// Length-256 Fourier transforms along a strided axis (inner >= 16): the x
// and y passes of a Fourier x Fourier x Chebyshev grid.  Same results as the
// generic line programs (fft_progs.cuh); a different schedule.
//
// The generic programs stage a tile of lines in shared memory, run the FFT
// there and write it back, with a barrier between every phase.  Here a CTA
// of 256 threads owns 16 complex lines (32 real lines for R2C / C2R) and:
//   pass 1  thread (line, n2) reads x[16 n1 + n2], n1 = 0..15, straight from
//           global memory (for fixed (n1, n2) the 16 lines of a half-warp are
//           consecutive addresses: coalesced), runs a 16-point DFT in
//           registers, multiplies by W_256^{n2 k1} and writes Z[line][k1][n2]
//           to shared memory;
//   barrier
//   pass 2  thread (line, k1) reads Z[line][k1][0..15], runs the second
//           16-point DFT in registers and writes X[k1 + 16 k2] straight to
//           global memory (coalesced the same way).
// One barrier for C2C and C2R; R2C adds one exchange (two barriers) to pair
// Z_k with Z_{256-k}.  The shared line stride (273 entries) is odd in 16-byte
// units, so the quarter-warps of both passes hit distinct bank groups.
//
// Real data go two lines at a time as one complex line (z = p + i q), as in
// the generic programs; inverse transforms conjugate on the way in and out
// (IDFT(X) = conj(DFT(conj X))).  The phases are __host__ __device__
// functions of a thread index so the CPU harness can run them thread by
// thread between the barriers.
#pragma once

#include "fft_line.cuh"

namespace sgpu {
namespace f256 {

const int N = 256;
const int TL = 16;    // complex lines per CTA
const int NT = 256;   // threads per CTA
const int LDZ = 273;  // shared-memory line stride (complex entries)

enum Kind { C2C_FWD = 0, C2C_BWD = 1, R2C = 2, C2R = 3 };

template <class R>
SGPU_HD size_t smem_bytes() {
  return sizeof(Cx<R>) * (size_t)TL * LDZ;
}

// element k of line l in an array with n_arr entries along the axis:
// base_off(l) + k * inner
SGPU_HD int64_t base_off(int64_t l, int64_t n_arr, int64_t inner) {
  const int64_t o = l / inner, i = l - o * inner;
  return o * n_arr * inner + i;
}

struct Args {
  const double* in;
  double* out;
  int64_t nlines;  // lines of the transform: complex lines (C2C) or real lines (R2C / C2R)
  int64_t inner;
  double scl;
  int64_t pb;      // R2C / C2R: lines pair up only within blocks of pb lines (0: one block)
};

// R2C / C2R: the two real lines of complex slot C (pairs never cross a block
// of pb lines); live flags for lines past a block or the array
SGPU_HD void pair_lines(const Args& a, int64_t C, int64_t& lp, bool& lvp, bool& lvq) {
  const int64_t B = a.pb > 0 ? a.pb : a.nlines;
  const int64_t hp = (B + 1) / 2;
  const int64_t b = C / hp, j = C - b * hp;
  lp = b * B + 2 * j;
  lvp = 2 * j < B && lp < a.nlines;
  lvq = 2 * j + 1 < B && lp + 1 < a.nlines;
}

#ifdef __CUDA_ARCH__
SGPU_HD double ldg(const double* p) { return __ldg(p); }
#else
SGPU_HD double ldg(const double* p) { return *p; }
#endif

// load one complex entry (re, im at p[0], p[1]) or a real pair
template <class R>
SGPU_HD Cx<R> ld_cx(const double* p) {
  return cx<R>(from_f64<R>(ldg(p)), from_f64<R>(ldg(p + 1)));
}

// -- pass 1: thread t = (n2 << 4) | line --------------------------------------
template <class R, int KIND>
SGPU_HD void pass1(const LinePlan& p, const Args& a, int64_t blk, Cx<R>* Z, int t) {
  const int line = t & 15, n2 = t >> 4;
  Cx<R> v[16];
  const Cx<R> zero = cx<R>(R(0.0), R(0.0));
  if (KIND == C2C_FWD || KIND == C2C_BWD) {
    const int64_t l = blk * TL + line;
    const bool live = l < a.nlines;
    const double* src = a.in + 2 * (live ? base_off(l, N, a.inner) : 0);
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) {
      v[n1] = live ? ld_cx<R>(src + 2 * (int64_t)(16 * n1 + n2) * a.inner) : zero;
      if (KIND == C2C_BWD) v[n1] = conj(v[n1]);
    }
  } else if (KIND == R2C) {
    int64_t lp;
    bool lvp, lvq;
    pair_lines(a, blk * TL + line, lp, lvp, lvq);
    const int64_t lq = lp + 1;
    const double* sp = a.in + (lvp ? base_off(lp, N, a.inner) : 0);
    const double* sq = a.in + (lvq ? base_off(lq, N, a.inner) : 0);
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) {
      const int64_t k = (int64_t)(16 * n1 + n2) * a.inner;
      v[n1] = cx<R>(lvp ? from_f64<R>(ldg(sp + k)) : R(0.0), lvq ? from_f64<R>(ldg(sq + k)) : R(0.0));
    }
  } else {  // C2R: Z_j = P_j + i Q_j with the Hermitian extension, conjugated
    int64_t lp;
    bool lvp, lvq;
    pair_lines(a, blk * TL + line, lp, lvp, lvq);
    const int64_t lq = lp + 1;
    const int nh = N / 2 + 1;
    const double* sp = a.in + 2 * (lvp ? base_off(lp, nh, a.inner) : 0);
    const double* sq = a.in + 2 * (lvq ? base_off(lq, nh, a.inner) : 0);
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) {
      const int j = 16 * n1 + n2;
      const bool up = j > N / 2;
      const int64_t k = (int64_t)(up ? N - j : j) * a.inner;
      Cx<R> P = lvp ? ld_cx<R>(sp + 2 * k) : zero;
      Cx<R> Q = lvq ? ld_cx<R>(sq + 2 * k) : zero;
      if (j == 0 || j == N / 2) {
        P.im = R(0.0);
        Q.im = R(0.0);
      }
      if (up) {
        P = conj(P);
        Q = conj(Q);
      }
      v[n1] = conj(P + mul_pi(Q));
    }
  }
  RegDFT<R, 16>::run(v);
  Cx<R>* z = Z + (size_t)line * LDZ + n2;
  z[0] = v[0];
#pragma unroll
  for (int k1 = 1; k1 < 16; ++k1) z[k1 * 17] = v[k1] * tw_at<R>(p, n2 * k1);
}

// -- pass 2: thread t = (k1 << 4) | line; X[k1 + 16 k2] in v[k2] ---------------
template <class R>
SGPU_HD void pass2_dft(const Cx<R>* Z, int t, Cx<R>* v) {
  const int line = t & 15, k1 = t >> 4;
  const Cx<R>* z = Z + (size_t)line * LDZ + k1 * 17;
#pragma unroll
  for (int n2 = 0; n2 < 16; ++n2) v[n2] = z[n2];
  RegDFT<R, 16>::run(v);
}

template <class R, int KIND>
SGPU_HD void pass2_store(const Args& a, int64_t blk, int t, const Cx<R>* v) {
  const int line = t & 15, k1 = t >> 4;
  const R sc = from_f64<R>(a.scl);
  if (KIND == C2C_FWD || KIND == C2C_BWD) {
    const int64_t l = blk * TL + line;
    if (l >= a.nlines) return;
    double* dst = a.out + 2 * base_off(l, N, a.inner);
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) {
      const Cx<R> x = v[k2];
      double* d = dst + 2 * (int64_t)(k1 + 16 * k2) * a.inner;
      d[0] = to_f64(x.re * sc);
      d[1] = to_f64(KIND == C2C_BWD ? -(x.im * sc) : x.im * sc);
    }
  } else {  // C2R: conj(X) * scale -> real lines 2c (re) and 2c + 1 (im)
    int64_t lp;
    bool lvp, lvq;
    pair_lines(a, blk * TL + line, lp, lvp, lvq);
    double* dp = lvp ? a.out + base_off(lp, N, a.inner) : nullptr;
    double* dq = lvq ? a.out + base_off(lp + 1, N, a.inner) : nullptr;
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) {
      const int64_t k = (int64_t)(k1 + 16 * k2) * a.inner;
      if (dp) dp[k] = to_f64(v[k2].re * sc);
      if (dq) dq[k] = to_f64(-(v[k2].im * sc));
    }
  }
}

// R2C, after the pass-2 DFTs: W[line][k] = X[k] (shared memory, reusing Z
// behind a barrier), then thread t forms P_k, Q_k for the entries e = t,
// t + 256, ... of the 16 x 129 outputs.
template <class R>
SGPU_HD void r2c_stash(Cx<R>* W, int t, const Cx<R>* v) {
  const int line = t & 15, k1 = t >> 4;
  Cx<R>* w = W + (size_t)line * LDZ;
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) w[k1 + 16 * k2] = v[k2];
}

template <class R>
SGPU_HD void r2c_post(const Args& a, int64_t blk, const Cx<R>* W, int t, int nth) {
  const int nh = N / 2 + 1;
  const R h = R(0.5) * from_f64<R>(a.scl);
  for (int e = t; e < TL * nh; e += nth) {
    const int line = e & 15, k = e >> 4;
    const Cx<R>* w = W + (size_t)line * LDZ;
    const Cx<R> z = w[k];
    const Cx<R> zc = conj(w[k == 0 ? 0 : N - k]);
    const Cx<R> P = scale(z + zc, h);
    const Cx<R> Q = scale(mul_mi(z - zc), h);
    int64_t lp;
    bool lvp, lvq;
    pair_lines(a, blk * TL + line, lp, lvp, lvq);
    if (lvp) {
      double* d = a.out + 2 * (base_off(lp, nh, a.inner) + (int64_t)k * a.inner);
      d[0] = to_f64(P.re);
      d[1] = to_f64(P.im);
    }
    if (lvq) {
      double* d = a.out + 2 * (base_off(lp + 1, nh, a.inner) + (int64_t)k * a.inner);
      d[0] = to_f64(Q.re);
      d[1] = to_f64(Q.im);
    }
  }
}

// tiles of a launch: complex lines (slots of real line pairs) / 16
SGPU_HD int64_t tiles(int kind, int64_t nlines, int64_t pb) {
  int64_t cl = nlines;
  if (kind == R2C || kind == C2R) {
    const int64_t B = pb > 0 ? pb : nlines;
    const int64_t full = B > 0 ? nlines / B : 0, r = nlines - full * B;
    cl = full * ((B + 1) / 2) + (r + 1) / 2;
  }
  return (cl + TL - 1) / TL;
}

}  // namespace f256
}  // namespace sgpu
