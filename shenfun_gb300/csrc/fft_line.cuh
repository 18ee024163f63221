// Line transforms along one axis of a (outer, n, inner) array: Fourier
// R2C/C2R/C2C and Chebyshev DCT-II/III with the Shen stencil, scaling and
// mass-matrix solve fused around them.
//
// One CTA owns a tile of lines.  It stages them from HBM into shared memory
// with row-coalesced loads (consecutive threads read consecutive addresses),
// runs a mixed-radix Stockham FFT of length m on every line of the tile, and
// writes the results back the same way.  Real data are processed two lines at
// a time as one complex line (z = p + i q).  DCT-II/III use Makhoul's
// reordering so that a length-n DCT costs one length-n complex FFT plus an
// O(n) twiddle pass.  A prime length n >= 11 is computed with Rader's
// algorithm (a cyclic convolution of length n-1, i.e. two FFTs of length n-1
// against a precomputed kernel spectrum), so n = 257 costs two 256-point FFTs.
//
// All block programs are __host__ __device__ (see sgpu_common.cuh): the CPU
// harness in tests/kernel_emu runs the same code to check indices and bounds.
#pragma once

#include "dfloat.cuh"

namespace sgpu {

#define SGPU_MAX_STAGES 24
#define SGPU_MAX_GENERIC_RADIX 4096

struct LinePlan {
  int kind;          // SGPU_XF_*
  int basis;         // SGPU_BASIS_* (Chebyshev kinds)
  int n;             // transform length along the axis
  int n_in, n_out;   // elements along the axis in the input / output arrays
  int m;             // complex FFT length (n, or n-1 with Rader)
  int rader;         // 1: length-n DFT through Rader's algorithm
  int nstages;
  int radix[SGPU_MAX_STAGES];
  int tlc;           // complex lines per CTA
  int ld;            // shared-memory line stride (complex elements) >= max(n, m)
  int nthreads;      // threads per CTA
  size_t smem;       // dynamic shared memory bytes per CTA
  // device tables
  const cd* tw;      // tw[e] = exp(-2 pi i e / m), e in [0, m)
  const cd* rk;      // Rader: DFT_m(b) / m, b_q = exp(-2 pi i g^{-q} / n)
  const int* rin;    // Rader gather:  a_q = z[rin[q]],  rin[q] = g^q mod n
  const int* rout;   // Rader scatter: X[rout[p]] = z_0 + c_p, rout[p] = g^{-p} mod n
  const cd* post;    // Chebyshev: post[k] = exp(-i pi k / (2 n)), k in [0, n)
  const double* mass;  // Chebyshev forward: LU'd mass bands (TDMA 3 x dim or PDMA 5 x dim)
  const double* sten;  // SB stencil rows: sten[k] = K2(k), sten[n + k] = K4(k)
  // the same tables as double-float pairs (mixed form)
  const Cx<df>* tw_f;
  const Cx<df>* rk_f;
  const Cx<df>* post_f;
  const df* sten_f;
  // m = 256: exp(-2 pi i e / 256) in Q0.62, each part split as h 2^31 + l
  // (tw_q[4 e .. 4 e + 3] = re h, re l, im h, im l; +1 saturates, the
  // fixed-point passes never use it)
  const int* tw_q;
  int form;          // SGPU_PLAIN_F64 or SGPU_MIXED_DF
  int64_t pb;        // real data: lines pair up (one complex FFT per pair)
                     // only within blocks of pb lines (0: one block of all
                     // lines), so that a stack of independent arrays gives
                     // each array's bits
  int bcfun;         // Chebyshev backward: add the boundary functions of the
                     // two boundary dofs (non-homogeneous SD / SN)
};

// typed table access: FP64 tables for R = double, df tables for R = df
template <class R>
SGPU_HD Cx<R> tw_at(const LinePlan& p, int e);
template <>
SGPU_HD Cx<double> tw_at<double>(const LinePlan& p, int e) { return p.tw[e]; }
template <>
SGPU_HD Cx<df> tw_at<df>(const LinePlan& p, int e) { return p.tw_f[e]; }
template <class R>
SGPU_HD Cx<R> rk_at(const LinePlan& p, int e);
template <>
SGPU_HD Cx<double> rk_at<double>(const LinePlan& p, int e) { return p.rk[e]; }
template <>
SGPU_HD Cx<df> rk_at<df>(const LinePlan& p, int e) { return p.rk_f[e]; }
template <class R>
SGPU_HD Cx<R> post_at(const LinePlan& p, int e);
template <>
SGPU_HD Cx<double> post_at<double>(const LinePlan& p, int e) { return p.post[e]; }
template <>
SGPU_HD Cx<df> post_at<df>(const LinePlan& p, int e) { return p.post_f[e]; }
template <class R>
SGPU_HD R sten_at(const LinePlan& p, int e);
template <>
SGPU_HD double sten_at<double>(const LinePlan& p, int e) { return p.sten[e]; }
template <>
SGPU_HD df sten_at<df>(const LinePlan& p, int e) { return p.sten_f[e]; }

// ---------------------------------------------------------------------------
// R-point DFT kernels (forward sign, y_s = sum_r v_r exp(-2 pi i r s / R))
template <class R>
SGPU_HD void dft2(Cx<R>* v) {
  Cx<R> a = v[0], b = v[1];
  v[0] = a + b;
  v[1] = a - b;
}

template <class R>
SGPU_HD void dft4(Cx<R>* v) {
  Cx<R> s02 = v[0] + v[2], d02 = v[0] - v[2];
  Cx<R> s13 = v[1] + v[3], d13 = mul_mi(v[1] - v[3]);
  v[0] = s02 + s13;
  v[1] = d02 + d13;
  v[2] = s02 - s13;
  v[3] = d02 - d13;
}

template <class R>
SGPU_HD void dft3(Cx<R>* v) {
  const R c = R(-0.5);
  const R s = R(0.86602540378443864676372317075294);  // sin(2 pi / 3)
  Cx<R> t = v[1] + v[2];
  Cx<R> d = v[1] - v[2];
  Cx<R> a = v[0] + scale(t, c);
  Cx<R> b = mul_mi(scale(d, s));
  v[0] = v[0] + t;
  v[1] = a + b;
  v[2] = a - b;
}

template <class R>
SGPU_HD void dft5(Cx<R>* v) {
  const R c1 = R(0.30901699437494742410229341718282);   // cos(2 pi/5)
  const R c2 = R(-0.80901699437494742410229341718282);  // cos(4 pi/5)
  const R s1 = R(0.95105651629515357211643933337938);   // sin(2 pi/5)
  const R s2 = R(0.58778525229247312916870595463907);   // sin(4 pi/5)
  Cx<R> t1 = v[1] + v[4], t2 = v[2] + v[3];
  Cx<R> d1 = v[1] - v[4], d2 = v[2] - v[3];
  Cx<R> a1 = v[0] + scale(t1, c1) + scale(t2, c2);
  Cx<R> a2 = v[0] + scale(t1, c2) + scale(t2, c1);
  Cx<R> b1 = mul_mi(scale(d1, s1) + scale(d2, s2));
  Cx<R> b2 = mul_mi(scale(d1, s2) - scale(d2, s1));
  v[0] = v[0] + t1 + t2;
  v[1] = a1 + b1;
  v[4] = a1 - b1;
  v[2] = a2 + b2;
  v[3] = a2 - b2;
}

// One Stockham butterfly: radix R_, stride Ns, butterfly j of a length-m line.
template <class R, int R_>
SGPU_HD void stockham_fixed(const Cx<R>* in, Cx<R>* out, int m, int Ns, int j, const LinePlan& p) {
  Cx<R> v[R_];
  const int mr = m / R_;
  const int k = j % Ns;
  const int st = mr / Ns;  // = m / (Ns * R_)
#pragma unroll
  for (int r = 0; r < R_; ++r) v[r] = in[j + r * mr];
  if (k != 0) {
#pragma unroll
    for (int r = 1; r < R_; ++r) {
      v[r] = v[r] * tw_at<R>(p, r * k * st);
    }
  }
  if (R_ == 2) dft2(v);
  if (R_ == 3) dft3(v);
  if (R_ == 4) dft4(v);
  if (R_ == 5) dft5(v);
  const int idx = (j / Ns) * Ns * R_ + k;
#pragma unroll
  for (int r = 0; r < R_; ++r) out[idx + r * Ns] = v[r];
}

// Generic odd-prime radix: direct O(R^2) DFT from the m-th roots table.
template <class R>
SGPU_HD void stockham_generic(const Cx<R>* in, Cx<R>* out, int m, int Rr, int Ns, int j,
                              const LinePlan& p) {
  const int mr = m / Rr;
  const int k = j % Ns;
  const int st = mr / Ns;
  const int idx = (j / Ns) * Ns * Rr + k;
  for (int s = 0; s < Rr; ++s) {
    Cx<R> acc = cx<R>(R(0), R(0));
    for (int r = 0; r < Rr; ++r) {
      Cx<R> x = in[j + r * mr];
      // twiddle W_m^{r k st} then DFT root W_R^{r s} = W_m^{(r s mod R) mr}
      int e = (r * k * st + ((r * s) % Rr) * mr) % m;
      acc = acc + x * tw_at<R>(p, e);
    }
    out[idx + s * Ns] = acc;
  }
}

}  // namespace sgpu

#include "fft_reg.cuh"

namespace sgpu {

// Run all stages of a length-m FFT on `lines` lines stored with stride ld.
// src holds the input; returns the buffer holding the output (src or dst).
template <class R>
SGPU_HD Cx<R>* fft_stages(const LinePlan& p, Cx<R>* src, Cx<R>* dst, int lines, int tid,
                          int nth) {
  const int m = p.m;
  int Ns = 1;
  for (int s = 0; s < p.nstages; ++s) {
    const int Rr = p.radix[s];
    const int nb = m / Rr;
    const int total = lines * nb;
    for (int idx = tid; idx < total; idx += nth) {
      const int t = idx / nb, j = idx - t * nb;
      const Cx<R>* in = src + (size_t)t * p.ld;
      Cx<R>* out = dst + (size_t)t * p.ld;
      switch (Rr) {
        case 2: stockham_fixed<R, 2>(in, out, m, Ns, j, p); break;
        case 3: stockham_fixed<R, 3>(in, out, m, Ns, j, p); break;
        case 4: stockham_fixed<R, 4>(in, out, m, Ns, j, p); break;
        case 5: stockham_fixed<R, 5>(in, out, m, Ns, j, p); break;
        default: stockham_generic<R>(in, out, m, Rr, Ns, j, p); break;
      }
    }
    SGPU_SYNC();
    Cx<R>* t = src;
    src = dst;
    dst = t;
    Ns *= Rr;
  }
  return src;
}

// Forward DFT of length n of every line in X (stride ld), result back in X.
// A and B are scratch line buffers of the same shape; slot holds 2 complex
// values per line.
template <class R>
SGPU_HD void dft_lines(const LinePlan& p, Cx<R>* X, Cx<R>* A, Cx<R>* B, Cx<R>* slot, int lines,
                       int tid, int nth) {
  const int n = p.n, m = p.m, ld = p.ld;
  if (!p.rader) {
    if (fft_fast<R>(p, X, A, lines, tid, nth)) return;
    Cx<R>* res = fft_stages<R>(p, X, A, lines, tid, nth);
    if (res != X) {
      for (int e = tid; e < lines * n; e += nth) {
        int t = e / n, k = e - t * n;
        X[(size_t)t * ld + k] = res[(size_t)t * ld + k];
      }
      SGPU_SYNC();
    }
    return;
  }
  // Rader: a_q = z[g^q], conv with b, X[g^-p] = z0 + c_p, X[0] = z0 + sum a
  for (int e = tid; e < lines * m; e += nth) {
    int t = e / m, q = e - t * m;
    A[(size_t)t * ld + q] = X[(size_t)t * ld + p.rin[q]];
  }
  for (int t = tid; t < lines; t += nth) slot[2 * t] = X[(size_t)t * ld];
  SGPU_SYNC();
  Cx<R>* r1 = A;
  if (!fft_fast<R>(p, A, B, lines, tid, nth)) r1 = fft_stages<R>(p, A, B, lines, tid, nth);
  for (int t = tid; t < lines; t += nth) slot[2 * t + 1] = r1[(size_t)t * ld];
  SGPU_SYNC();
  // multiply by the kernel spectrum, conjugate: IDFT(y) = conj(DFT(conj(y)))
  for (int e = tid; e < lines * m; e += nth) {
    int t = e / m, q = e - t * m;
    r1[(size_t)t * ld + q] = conj(r1[(size_t)t * ld + q] * rk_at<R>(p, q));
  }
  SGPU_SYNC();
  Cx<R>* other = (r1 == A) ? B : A;
  Cx<R>* r2 = r1;
  if (!fft_fast<R>(p, r1, other, lines, tid, nth)) r2 = fft_stages<R>(p, r1, other, lines, tid, nth);
  for (int e = tid; e < lines * m; e += nth) {
    int t = e / m, q = e - t * m;
    X[(size_t)t * ld + p.rout[q]] = slot[2 * t] + conj(r2[(size_t)t * ld + q]);
  }
  for (int t = tid; t < lines; t += nth) X[(size_t)t * ld] = slot[2 * t] + slot[2 * t + 1];
  SGPU_SYNC();
}

}  // namespace sgpu

#include "fft_progs.cuh"
