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
#define SGPU_MAX_GENERIC_RADIX 127

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
  int form;          // SGPU_PLAIN_F64 or SGPU_MIXED_DF
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

// ---------------------------------------------------------------------------
// Tile addressing.  Lines are l = o * inner + i; a tile is TL consecutive
// lines.  Element (l, k) of an array with n_arr entries along the axis lives
// at o * n_arr * inner + k * inner + i.
SGPU_HD int64_t elem_off(int64_t l, int64_t k, int64_t n_arr, int64_t inner) {
  int64_t o = l / inner, i = l - o * inner;
  return (o * n_arr + k) * inner + i;
}

// Map a flat index e over a TL x n_arr tile to (t, k) so that consecutive e
// touch consecutive addresses: along k when lines are contiguous (inner == 1),
// along t otherwise.
SGPU_HD void tile_map(int64_t e, int TL, int n_arr, int64_t inner, int& t, int& k) {
  if (inner == 1) {
    t = (int)(e / n_arr);
    k = (int)(e - (int64_t)t * n_arr);
  } else {
    k = (int)(e / TL);
    t = (int)(e - (int64_t)k * TL);
  }
}

// Stencil coefficient K_m(k) of the Shen basis (offsets 0, 2, 4).  Constant
// entries (the 1 and -1 of ShenDirichlet, the leading 1 of ShenBiharmonic)
// apply to every row, as in the reference's stencil matrix
// (spectralbase.py:1504-1526); k-dependent entries are zero for k >= dim.
template <class R>
SGPU_HD R stencil_coef(const LinePlan& p, int off, int k) {
  if (p.basis == SGPU_BASIS_ORTHO) return off == 0 ? R(1.0) : R(0.0);
  if (p.basis == SGPU_BASIS_SD) return off == 0 ? R(1.0) : (off == 2 ? R(-1.0) : R(0.0));
  // SB
  if (off == 0) return R(1.0);
  if (off == 2) return sten_at<R>(p, k);
  if (off == 4) return sten_at<R>(p, p.n + k);
  return R(0.0);
}

SGPU_HD int basis_nbcs(int basis) {
  return basis == SGPU_BASIS_SD ? 2 : (basis == SGPU_BASIS_SB ? 4 : 0);
}

// ---------------------------------------------------------------------------
// Block programs.  smem layout: X | A | B (tlc * ld complex each) | slot (2 tlc)
template <class R>
struct Smem {
  Cx<R>* X;
  Cx<R>* A;
  Cx<R>* B;
  Cx<R>* slot;
};

template <class R>
SGPU_HD Smem<R> carve(const LinePlan& p, void* smem) {
  Smem<R> s;
  Cx<R>* base = (Cx<R>*)smem;
  size_t L = (size_t)p.tlc * p.ld;
  s.X = base;
  s.A = base + L;
  s.B = base + 2 * L;
  s.slot = base + 3 * L;
  return s;
}

template <class R>
SGPU_HD size_t smem_bytes(int tlc, int ld) {
  return sizeof(Cx<R>) * ((size_t)3 * tlc * ld + 2 * (size_t)tlc);
}

// Load a tile of lines into X.  Real data: line pair (2c, 2c+1) -> complex
// line c (re, im); complex data: line c -> complex line c.  Lines past the end
// of the array are zero.
template <class R>
SGPU_HD void load_tile(const LinePlan& p, const void* in, int in_complex, int64_t l0,
                       int64_t nlines, int64_t inner, Cx<R>* X, int tid, int nth) {
  const int n_arr = p.n_in;
  const int TL = in_complex ? p.tlc : 2 * p.tlc;
  const int64_t total = (int64_t)TL * n_arr;
  for (int64_t e = tid; e < total; e += nth) {
    int t, k;
    tile_map(e, TL, n_arr, inner, t, k);
    int64_t l = l0 + t;
    if (in_complex) {
      Cx<R> v = cx<R>(R(0), R(0));
      if (l < nlines) {
        const double* src = (const double*)in + 2 * elem_off(l, k, n_arr, inner);
        v = cx<R>(from_f64<R>(src[0]), from_f64<R>(src[1]));
      }
      X[(size_t)t * p.ld + k] = v;
    } else {
      R v = R(0);
      if (l < nlines) v = from_f64<R>(((const double*)in)[elem_off(l, k, n_arr, inner)]);
      Cx<R>& z = X[(size_t)(t >> 1) * p.ld + k];
      if (t & 1)
        z.im = v;
      else
        z.re = v;
    }
  }
  SGPU_SYNC();
}

// Store a tile from Y (complex lines, or real line pairs packed re/im).
template <class R>
SGPU_HD void store_tile(const LinePlan& p, void* out, int out_complex, int64_t l0,
                        int64_t nlines, int64_t inner, const Cx<R>* Y, int tid, int nth) {
  const int n_arr = p.n_out;
  const int TL = out_complex ? p.tlc : 2 * p.tlc;
  const int64_t total = (int64_t)TL * n_arr;
  for (int64_t e = tid; e < total; e += nth) {
    int t, k;
    tile_map(e, TL, n_arr, inner, t, k);
    int64_t l = l0 + t;
    if (l >= nlines) continue;
    if (out_complex) {
      Cx<R> v = Y[(size_t)t * p.ld + k];
      double* dst = (double*)out + 2 * elem_off(l, k, n_arr, inner);
      dst[0] = to_f64(v.re);
      dst[1] = to_f64(v.im);
    } else {
      const Cx<R>& z = Y[(size_t)(t >> 1) * p.ld + k];
      ((double*)out)[elem_off(l, k, n_arr, inner)] = to_f64((t & 1) ? z.im : z.re);
    }
  }
}

// Fourier R2C: pairs of real lines -> half spectra, times `scale`.
template <class R>
SGPU_HD void prog_r2c(const LinePlan& p, const double* in, double* out, int64_t nlines,
                      int64_t inner, double scl, int64_t blk, void* smem, int tid, int nth) {
  Smem<R> s = carve<R>(p, smem);
  const int64_t l0 = blk * 2 * p.tlc;
  load_tile<R>(p, in, 0, l0, nlines, inner, s.X, tid, nth);
  dft_lines<R>(p, s.X, s.A, s.B, s.slot, p.tlc, tid, nth);
  // separate: P_k = (Z_k + conj Z_{n-k}) / 2, Q_k = (Z_k - conj Z_{n-k}) / (2i)
  const int n = p.n, nh = n / 2 + 1;
  const R h = R(0.5) * from_f64<R>(scl);
  for (int e = tid; e < p.tlc * nh; e += nth) {
    int c = e / nh, k = e - c * nh;
    Cx<R> z = s.X[(size_t)c * p.ld + k];
    Cx<R> zc = conj(s.X[(size_t)c * p.ld + (k == 0 ? 0 : n - k)]);
    s.A[(size_t)(2 * c) * p.ld + k] = scale(z + zc, h);
    s.A[(size_t)(2 * c + 1) * p.ld + k] = scale(mul_mi(z - zc), h);
  }
  SGPU_SYNC();
  // A now holds 2*tlc complex lines: store as complex output lines
  LinePlan q = p;
  q.tlc = 2 * p.tlc;
  store_tile<R>(q, out, 1, l0, nlines, inner, s.A, tid, nth);
}

// Fourier C2R: pairs of half spectra -> real lines (unnormalised), times scale.
template <class R>
SGPU_HD void prog_c2r(const LinePlan& p, const double* in, double* out, int64_t nlines,
                      int64_t inner, double scl, int64_t blk, void* smem, int tid, int nth) {
  Smem<R> s = carve<R>(p, smem);
  const int64_t l0 = blk * 2 * p.tlc;
  LinePlan q = p;
  q.tlc = 2 * p.tlc;  // load 2*tlc complex half-spectrum lines into A (ld stride)
  load_tile<R>(q, in, 1, l0, nlines, inner, s.A, tid, nth);
  const int n = p.n, nh = n / 2 + 1;
  // Z_k = P_k + i Q_k with Hermitian extension; DC and (even n) Nyquist real.
  for (int e = tid; e < p.tlc * n; e += nth) {
    int c = e / n, k = e - c * n;
    const Cx<R>* P = s.A + (size_t)(2 * c) * p.ld;
    const Cx<R>* Q = s.A + (size_t)(2 * c + 1) * p.ld;
    Cx<R> pk, qk;
    if (k < nh) {
      pk = P[k];
      qk = Q[k];
      if (k == 0 || 2 * k == n) {
        pk.im = R(0);
        qk.im = R(0);
      }
    } else {
      pk = conj(P[n - k]);
      qk = conj(Q[n - k]);
    }
    // conj for the inverse transform: IDFT(Z) = conj(DFT(conj(Z)))
    s.X[(size_t)c * p.ld + k] = conj(pk + mul_pi(qk));
  }
  SGPU_SYNC();
  dft_lines<R>(p, s.X, s.A, s.B, s.slot, p.tlc, tid, nth);
  const R sc = from_f64<R>(scl);
  for (int e = tid; e < p.tlc * n; e += nth) {
    int c = e / n, k = e - c * n;
    Cx<R> z = s.X[(size_t)c * p.ld + k];
    s.X[(size_t)c * p.ld + k] = cx<R>(z.re * sc, -(z.im * sc));
  }
  SGPU_SYNC();
  store_tile<R>(p, out, 0, l0, nlines, inner, s.X, tid, nth);
}

// Fourier C2C forward / backward (unnormalised), times scale.
template <class R>
SGPU_HD void prog_c2c(const LinePlan& p, const double* in, double* out, int64_t nlines,
                      int64_t inner, double scl, int64_t blk, void* smem, int tid, int nth) {
  Smem<R> s = carve<R>(p, smem);
  const int64_t l0 = blk * p.tlc;
  const bool bwd = p.kind == SGPU_XF_C2C_BWD;
  load_tile<R>(p, in, 1, l0, nlines, inner, s.X, tid, nth);
  if (bwd) {
    for (int e = tid; e < p.tlc * p.n; e += nth) {
      int c = e / p.n, k = e - c * p.n;
      s.X[(size_t)c * p.ld + k] = conj(s.X[(size_t)c * p.ld + k]);
    }
    SGPU_SYNC();
  }
  dft_lines<R>(p, s.X, s.A, s.B, s.slot, p.tlc, tid, nth);
  const R sc = from_f64<R>(scl);
  for (int e = tid; e < p.tlc * p.n; e += nth) {
    int c = e / p.n, k = e - c * p.n;
    Cx<R> z = s.X[(size_t)c * p.ld + k];
    s.X[(size_t)c * p.ld + k] = bwd ? cx<R>(z.re * sc, -(z.im * sc)) : scale(z, sc);
  }
  SGPU_SYNC();
  store_tile<R>(p, out, 1, l0, nlines, inner, s.X, tid, nth);
}

// Chebyshev forward kinds: DCT-II (REDFT10) and the GC scalar product with the
// stencil epilogue (+ inverse mass for SGPU_XF_CHEB_FORWARD).
template <class R>
SGPU_HD void prog_dct2(const LinePlan& p, const double* in, double* out, int in_complex,
                       int64_t nlines, int64_t inner, double scl, int64_t blk, void* smem,
                       int tid, int nth) {
  Smem<R> s = carve<R>(p, smem);
  const int TL = in_complex ? p.tlc : 2 * p.tlc;
  const int64_t l0 = blk * TL;
  const int n = p.n, h = (n + 1) / 2;
  load_tile<R>(p, in, in_complex, l0, nlines, inner, s.A, tid, nth);
  // Makhoul reorder: v_j = x_{2j} (j < h), v_{n-1-j} = x_{2j+1}
  for (int e = tid; e < p.tlc * n; e += nth) {
    int c = e / n, j = e - c * n;
    int src = j < h ? 2 * j : 2 * (n - 1 - j) + 1;
    s.X[(size_t)c * p.ld + j] = s.A[(size_t)c * p.ld + src];
  }
  SGPU_SYNC();
  dft_lines<R>(p, s.X, s.A, s.B, s.slot, p.tlc, tid, nth);
  // Y_k = 2 Re(exp(-i pi k / 2n) V_k) for each of the two packed real lines.
  R fac;
  if (p.kind == SGPU_XF_DCT2)
    fac = from_f64<R>(2.0 * scl);
  else
    fac = from_f64<R>(3.14159265358979323846264338327950288 / n);  // (pi / 2n) * 2
  for (int e = tid; e < p.tlc * n; e += nth) {
    int c = e / n, k = e - c * n;
    Cx<R> z = s.X[(size_t)c * p.ld + k];
    Cx<R> zc = conj(s.X[(size_t)c * p.ld + (k == 0 ? 0 : n - k)]);
    Cx<R> P = scale(z + zc, R(0.5));
    Cx<R> Q = scale(mul_mi(z - zc), R(0.5));
    Cx<R> w = post_at<R>(p, k);
    R yp = (w.re * P.re - w.im * P.im) * fac;
    R yq = (w.re * Q.re - w.im * Q.im) * fac;
    s.A[(size_t)c * p.ld + k] = cx<R>(yp, yq);
  }
  SGPU_SYNC();
  Cx<R>* Y = s.A;
  if (p.kind == SGPU_XF_CHEB_SCALAR || p.kind == SGPU_XF_CHEB_FORWARD) {
    // out_k = sum_m K_m(k) y_{k+m}
    for (int e = tid; e < p.tlc * n; e += nth) {
      int c = e / n, k = e - c * n;
      const Cx<R>* y = s.A + (size_t)c * p.ld;
      Cx<R> acc = y[k];
      for (int off = 2; off <= 4; off += 2) {
        if (k + off < n) {
          acc = acc + scale(y[k + off], stencil_coef<R>(p, off, k));
        }
      }
      s.B[(size_t)c * p.ld + k] = acc;
    }
    SGPU_SYNC();
    Y = s.B;
  }
  if (p.kind == SGPU_XF_CHEB_FORWARD) {
    // B^{-1} on the first dim entries (TDMA_inner_solve_ptr / PDMA_inner_solve_ptr,
    // la.pyx:496-532), boundary dofs zero (homogeneous BCs).  The plan's mass
    // table holds the LU'd bands with the diagonal row replaced by its
    // reciprocal, so the solve multiplies instead of dividing.
    const int nb = basis_nbcs(p.basis), dim = n - nb;
    for (int c = tid; c < p.tlc; c += nth) {
      Cx<R>* u = Y + (size_t)c * p.ld;
      if (nb == 2) {
        const double* ld_ = p.mass;
        const double* di = p.mass + dim;
        const double* ud = p.mass + 2 * dim + 2;
        for (int i = 2; i < dim; ++i) u[i] = u[i] - scale(u[i - 2], from_f64<R>(ld_[i - 2]));
        u[dim - 1] = scale(u[dim - 1], from_f64<R>(di[dim - 1]));
        u[dim - 2] = scale(u[dim - 2], from_f64<R>(di[dim - 2]));
        for (int i = dim - 3; i >= 0; --i)
          u[i] = scale(u[i] - scale(u[i + 2], from_f64<R>(ud[i])), from_f64<R>(di[i]));
      } else if (nb == 4) {
        const double* a = p.mass;
        const double* b = p.mass + dim;
        const double* di = p.mass + 2 * dim;
        const double* ee = p.mass + 3 * dim + 2;
        const double* f = p.mass + 4 * dim + 4;
        u[2] = u[2] - scale(u[0], from_f64<R>(b[0]));
        u[3] = u[3] - scale(u[1], from_f64<R>(b[1]));
        for (int k = 4; k < dim; ++k)
          u[k] = u[k] - (scale(u[k - 2], from_f64<R>(b[k - 2])) + scale(u[k - 4], from_f64<R>(a[k - 4])));
        u[dim - 1] = scale(u[dim - 1], from_f64<R>(di[dim - 1]));
        u[dim - 2] = scale(u[dim - 2], from_f64<R>(di[dim - 2]));
        u[dim - 3] = scale(u[dim - 3] - scale(u[dim - 1], from_f64<R>(ee[dim - 3])), from_f64<R>(di[dim - 3]));
        u[dim - 4] = scale(u[dim - 4] - scale(u[dim - 2], from_f64<R>(ee[dim - 4])), from_f64<R>(di[dim - 4]));
        for (int k = dim - 5; k >= 0; --k)
          u[k] = scale(u[k] - scale(u[k + 2], from_f64<R>(ee[k])) - scale(u[k + 4], from_f64<R>(f[k])), from_f64<R>(di[k]));
      } else {
        // orthogonal basis: diagonal mass; the table holds 1 / (c_k pi / 2)
        for (int k = 0; k < n; ++k) u[k] = scale(u[k], from_f64<R>(p.mass[k]));
      }
      for (int k = dim; k < n; ++k) u[k] = cx<R>(R(0), R(0));
    }
    SGPU_SYNC();
  }
  store_tile<R>(p, out, in_complex, l0, nlines, inner, Y, tid, nth);
}

// Chebyshev backward kinds: DCT-III (REDFT01) and the GC backward with the
// to_ortho prologue (0.5 * REDFT01 + c_0 / 2).
template <class R>
SGPU_HD void prog_dct3(const LinePlan& p, const double* in, double* out, int in_complex,
                       int64_t nlines, int64_t inner, double scl, int64_t blk, void* smem,
                       int tid, int nth) {
  Smem<R> s = carve<R>(p, smem);
  const int TL = in_complex ? p.tlc : 2 * p.tlc;
  const int64_t l0 = blk * TL;
  const int n = p.n, h = (n + 1) / 2;
  load_tile<R>(p, in, in_complex, l0, nlines, inner, s.A, tid, nth);
  Cx<R>* C = s.A;
  if (p.kind == SGPU_XF_CHEB_BACKWARD && p.basis != SGPU_BASIS_ORTHO) {
    // to_ortho: c_{k+m} += K_m(k) u_k for k < dim (spectralbase.py:1616-1634)
    const int dim = n - basis_nbcs(p.basis);
    for (int e = tid; e < p.tlc * n; e += nth) {
      int c = e / n, k = e - c * n;
      const Cx<R>* u = s.A + (size_t)c * p.ld;
      Cx<R> acc = cx<R>(R(0), R(0));
      if (k < dim) acc = u[k];
      for (int off = 2; off <= 4; off += 2) {
        int j = k - off;
        if (j >= 0 && j < dim) acc = acc + scale(u[j], stencil_coef<R>(p, off, j));
      }
      s.B[(size_t)c * p.ld + k] = acc;
    }
    SGPU_SYNC();
    C = s.B;
  }
  // W_k = f (c_k - i c_{n-k}) exp(i pi k / 2n), c_n = 0; for the GC backward
  // f = 1/2 and W_0 = c_0 (0.5 REDFT01 + c_0/2); for raw REDFT01 f = 1.
  // Two real lines p, q packed: Z = W_p + i W_q, then conj for the IDFT.
  const bool gc = p.kind == SGPU_XF_CHEB_BACKWARD;
  const R f = gc ? R(0.5) : R(1.0);
  for (int e = tid; e < p.tlc * n; e += nth) {
    int c = e / n, k = e - c * n;
    const Cx<R>* cl = C + (size_t)c * p.ld;
    Cx<R> a = cl[k];
    Cx<R> b = k == 0 ? cx<R>(R(0), R(0)) : cl[n - k];
    // line p uses .re parts, line q uses .im parts
    Cx<R> wp = cx<R>(a.re, -b.re);
    Cx<R> wq = cx<R>(a.im, -b.im);
    Cx<R> z;
    if (k == 0) {
      z = cx<R>(a.re, a.im);  // W_0 = c_0 (both lines)
      if (!gc) z = cx<R>(a.re, a.im);
    } else {
      Cx<R> tw = conj(post_at<R>(p, k));  // exp(+i pi k / 2n)
      wp = scale(wp * tw, f);
      wq = scale(wq * tw, f);
      z = wp + mul_pi(wq);
    }
    s.X[(size_t)c * p.ld + k] = conj(z);
  }
  SGPU_SYNC();
  dft_lines<R>(p, s.X, s.A, s.B, s.slot, p.tlc, tid, nth);
  // y_{2j} = w_j, y_{2j+1} = w_{n-1-j}; w = conj(result); real line p = Re w, q = Im w
  const R sc = gc ? R(1) : R(scl);
  for (int e = tid; e < p.tlc * n; e += nth) {
    int c = e / n, i = e - c * n;
    int j = (i & 1) ? (n - 1 - (i >> 1)) : (i >> 1);
    Cx<R> z = conj(s.X[(size_t)c * p.ld + j]);
    s.A[(size_t)c * p.ld + i] = scale(z, sc);
  }
  (void)h;
  SGPU_SYNC();
  store_tile<R>(p, out, in_complex, l0, nlines, inner, s.A, tid, nth);
}

template <class R>
SGPU_HD void prog_dispatch(const LinePlan& p, const double* in, double* out, int data_complex,
                           int64_t nlines, int64_t inner, double scl, int64_t blk, void* smem,
                           int tid, int nth) {
  switch (p.kind) {
    case SGPU_XF_R2C: prog_r2c<R>(p, in, out, nlines, inner, scl, blk, smem, tid, nth); break;
    case SGPU_XF_C2R: prog_c2r<R>(p, in, out, nlines, inner, scl, blk, smem, tid, nth); break;
    case SGPU_XF_C2C_FWD:
    case SGPU_XF_C2C_BWD: prog_c2c<R>(p, in, out, nlines, inner, scl, blk, smem, tid, nth); break;
    case SGPU_XF_DCT2:
    case SGPU_XF_CHEB_SCALAR:
    case SGPU_XF_CHEB_FORWARD:
      prog_dct2<R>(p, in, out, data_complex, nlines, inner, scl, blk, smem, tid, nth);
      break;
    case SGPU_XF_DCT3:
    case SGPU_XF_CHEB_BACKWARD:
      prog_dct3<R>(p, in, out, data_complex, nlines, inner, scl, blk, smem, tid, nth);
      break;
    default: break;
  }
}

// whether the lines are complex: fixed by the Fourier kinds, chosen by the
// caller for the Chebyshev kinds
SGPU_HD int data_complex_for(const LinePlan& p, int data_kind) {
  if (p.kind == SGPU_XF_R2C) return 0;
  if (p.kind == SGPU_XF_C2R || p.kind == SGPU_XF_C2C_FWD || p.kind == SGPU_XF_C2C_BWD) return 1;
  return data_kind == SGPU_COMPLEX ? 1 : 0;
}

// number of lines one CTA handles for this plan and data kind
SGPU_HD int lines_per_block(const LinePlan& p, int data_complex) {
  switch (p.kind) {
    case SGPU_XF_R2C:
    case SGPU_XF_C2R: return 2 * p.tlc;
    case SGPU_XF_C2C_FWD:
    case SGPU_XF_C2C_BWD: return p.tlc;
    default: return data_complex ? p.tlc : 2 * p.tlc;
  }
}

}  // namespace sgpu
