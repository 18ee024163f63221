// Length-256 Fourier passes of the mixed form in 64-bit fixed point: the
// schedule of fft256.cuh (pass 1 = 16-point DFTs over n1 in registers +
// twiddles, one shared-memory transpose, pass 2 = 16-point DFTs over n2),
// with every value an integer on a per-line grid instead of a double-float.
//
// Format.  A line (a real line, for R2C / C2R) is scaled by a power of two
// chosen from its largest FP64 exponent E: X = round(x 2^S), S = 1076 - E - hr,
// so that |X| < 2^(54 - hr) (hr = 1 for R2C and C2R: their pairs add two
// lines' transforms before separating them).  A length-256 DFT grows moduli
// at most 256-fold, so every intermediate stays below 2^62.5 < 2^63:
// additions are exact 64-bit integer additions and cannot overflow.
// Twiddle factors are Q0.62 integers w = round(2^62 c) split as
// w = wh 2^31 + wl (wl in [0, 2^31)); with y = yh 2^31 + yl the product
// y c = yh wh + (yh wl + yl wh) / 2^31 + yl wl / 2^62 takes three 32 x 32 ->
// 64-bit multiply-adds, dropping the last term and the fraction of the
// middle one (below 2 units).  Each value
// therefore carries about 53 bits relative to its line's largest entry - the
// normwise accuracy of an FP64 FFT - at 2 integer instructions per addition
// instead of ~11 FP32 instructions for a double-float addition.
//
// Lines of a complex pair (R2C: z = p + i q; C2R: z = conj(P + i Q)) keep
// separate scales 2^Sp and 2^Sq: the DFT is linear, so the pair's transform
// is 2^Sp DFT(p) + i 2^Sq DFT(q) on one integer grid, and each line is
// unscaled on its own at the end.  The scales need the line's maximum
// exponent before any value is converted: each thread reduces the exponents
// of its 16 values, the 16 threads of a line meet in shared memory (one
// barrier), and the values are then loaded again (from L1 or L2) and
// converted: held in registers across the barrier they would spill.
//
// A line holding Inf or NaN comes out as NaN (an FP64 transform spreads it
// over the line the same way); subnormal inputs count as zero, and outputs
// below the FP64 normal range flush to zero.
#pragma once

#include "fft256.cuh"

namespace sgpu {
namespace f256 {

struct Cq {
  long long re, im;
};

SGPU_HD Cq cq(long long r, long long i) {
  Cq c;
  c.re = r;
  c.im = i;
  return c;
}
SGPU_HD Cq operator+(Cq a, Cq b) { return cq(a.re + b.re, a.im + b.im); }
SGPU_HD Cq operator-(Cq a, Cq b) { return cq(a.re - b.re, a.im - b.im); }
SGPU_HD Cq q_mul_mi(Cq a) { return cq(a.im, -a.re); }  // x (-i)
SGPU_HD Cq q_mul_pi(Cq a) { return cq(-a.im, a.re); }  // x (+i)
SGPU_HD Cq q_conj(Cq a) { return cq(a.re, -a.im); }

// a Q0.62 factor split for q62: w = h 2^31 + l, l in [0, 2^31)
struct Tw {
  int h, l;
};
SGPU_HD constexpr Tw tsplit(long long q) { return Tw{(int)(q >> 31), (int)(q & 0x7FFFFFFFLL)}; }

// y w / 2^62, |y| < 2^62 (every value a twiddle multiplies is below 2^61)
SGPU_HD long long q62(long long y, Tw w) {
  const int yh = (int)(y >> 31);
  const int yl = (int)(y & 0x7FFFFFFFLL);
  const long long mid = (long long)yh * w.l + (long long)yl * w.h;
  return (long long)yh * w.h + (mid >> 31);
}

SGPU_HD Cq q_mul(Cq a, Tw wr, Tw wi) {
  return cq(q62(a.re, wr) - q62(a.im, wi), q62(a.re, wi) + q62(a.im, wr));
}

// round(2^62 x) of cos(pi / 8), sin(pi / 8) and cos(pi / 4)
const long long kQc1 = 4260642322793532497LL;
const long long kQs1 = 1764815834521887442LL;
const long long kQh = 3260954456333195553LL;

// x exp(-2 pi i j / 16) for the j a 4 x 4 DFT uses (n2 k1, n2, k1 < 4)
SGPU_HD Cq q_mul_w16(Cq a, int j) {
  const Tw h = tsplit(kQh);
  switch (j) {
    case 0: return a;
    case 1: return q_mul(a, tsplit(kQc1), tsplit(-kQs1));
    case 2: return cq(q62(a.re + a.im, h), q62(a.im - a.re, h));    // (h, -h)
    case 3: return q_mul(a, tsplit(kQs1), tsplit(-kQc1));
    case 4: return q_mul_mi(a);
    case 6: return cq(q62(a.im - a.re, h), -q62(a.re + a.im, h));   // (-h, -h)
    default: return q_mul(a, tsplit(-kQc1), tsplit(kQs1));           // 9: (-c1, s1)
  }
}

SGPU_HD void q_dft4(Cq* v) {
  const Cq t0 = v[0] + v[2], t1 = v[0] - v[2], t2 = v[1] + v[3], t3 = v[1] - v[3];
  v[0] = t0 + t2;
  v[2] = t0 - t2;
  v[1] = t1 + q_mul_mi(t3);
  v[3] = t1 + q_mul_pi(t3);
}

// 16-point forward DFT in place, natural order (4 x 4: n = 4 n1 + n2,
// k = k1 + 4 k2), as RegDFT<R, 16>
SGPU_HD void q_dft16(Cq* v) {
  Cq a[4][4];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    Cq t[4] = {v[n2], v[4 + n2], v[8 + n2], v[12 + n2]};
    q_dft4(t);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) a[n2][k1] = q_mul_w16(t[k1], n2 * k1);
  }
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    Cq t[4] = {a[0][k1], a[1][k1], a[2][k1], a[3][k1]};
    q_dft4(t);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[k2];
  }
}

// one complex entry (16-byte aligned) as one 16-byte load / store
SGPU_HD void ldg2(const double* p, double& re, double& im) {
#ifdef __CUDA_ARCH__
  const double2 v = __ldg((const double2*)p);
  re = v.x;
  im = v.y;
#else
  re = p[0];
  im = p[1];
#endif
}
SGPU_HD void st2(double* p, double re, double im) {
#ifdef __CUDA_ARCH__
  *(double2*)p = make_double2(re, im);
#else
  p[0] = re;
  p[1] = im;
#endif
}

// biased FP64 exponent (0 for zero and subnormals, 0x7ff for Inf / NaN)
SGPU_HD int bexp(double x) { return (int)((d2u(x) >> 52) & 0x7ff); }

// round(x 2^(1076 - Eh)) for |x| < 2^(Eh - 1022), Eh >= the value's biased
// exponent: the 53-bit significand doubled and shifted right by Eh - e
// (at most 63), rounded half up; zero and subnormals give 0 (Inf / NaN give
// a bounded value, and their line is flagged instead).  Branch-free.
SGPU_HD long long fx_from_f64(double x, int Eh) {
  const unsigned long long b = d2u(x);
  const int e = (int)((b >> 52) & 0x7ff);
  const unsigned long long M = e ? (((b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull) << 1) : 0ull;
  const int d = Eh - e;
  const int sft = d < 63 ? d : 63;
  const unsigned long long X = (M + ((1ull << sft) >> 1)) >> sft;
  const long long m = (long long)b >> 63;  // 0 or -1: the sign
  return ((long long)X ^ m) - m;
}

// X 2^(k - 1075) as an FP64 value (round half up; below the normal range
// flushes to zero)
SGPU_HD double fx_to_f64(long long X, int k) {
  const long long m = X >> 63;
  unsigned long long a = (unsigned long long)((X ^ m) - m);  // |X|
#ifdef __CUDA_ARCH__
  const int n = __clzll((long long)a);
#else
  const int n = a ? __builtin_clzll(a) : 64;
#endif
  a <<= (n & 63);  // leading one at bit 63 (a = 0 stays 0)
  const unsigned long long t0 = a + 1024ull;  // round at bit 10
  const bool carry = t0 < a;  // out of bit 63: the significand is 2^53
  const unsigned long long t = carry ? 0x8000000000000000ull : t0;
  const int be = k + 11 - n + (carry ? 1 : 0);  // biased exponent
  unsigned long long bits = ((unsigned long long)be << 52) | ((t >> 11) & 0xFFFFFFFFFFFFFull);
  bits = (a == 0 || be <= 0) ? 0ull : (be >= 0x7ff ? 0x7ff0000000000000ull : bits);
  return u2d(bits | ((unsigned long long)m & 0x8000000000000000ull));
}

// X / 2^d rounded half up (d >= 0; beyond 62 every value here rounds to 0)
SGPU_HD long long q_shr(long long X, int d) {
  const int sft = d < 62 ? d : 62;
  return (X + ((1LL << sft) >> 1)) >> sft;
}

// shared memory beyond the exchange buffer: per (line, n2) the local
// maximum exponents of the line's values (R2C / C2R: of p and of q), per
// line their maximum, then per line the element offsets of its first
// entries in the input and the output (R2C / C2R: of p and of q; -1 for
// lines past the array or block)
const int EX = TL * 16;
SGPU_HD size_t fx_smem_bytes() {
  return sizeof(Cq) * (size_t)TL * LDZ + sizeof(int) * (2 * EX + 2 * TL) + sizeof(long long) * 4 * TL;
}
struct FxShared {
  Cq* Z;
  int* Ez;          // [2][TL][16]
  int* El;          // [2][TL]: written in pass 1, read after its barrier
  long long* Lin;   // [2 TL]: p (or the complex line), q
  long long* Lout;  // [2 TL]
};
SGPU_HD FxShared fx_shared(unsigned char* base) {
  FxShared f;
  f.Z = (Cq*)base;
  f.Ez = (int*)(base + sizeof(Cq) * (size_t)TL * LDZ);
  f.El = f.Ez + 2 * EX;
  f.Lin = (long long*)(f.El + 2 * TL);
  f.Lout = f.Lin + 2 * TL;
  return f;
}

// the maximum over the 16 threads of `line` (Ez: [line][n2])
SGPU_HD int line_exp(const int* Ez, int line) {
  int E = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) E = Ez[line * 16 + i] > E ? Ez[line * 16 + i] : E;
  return E;
}

// -- phase A: the maximum exponents of the thread's inputs and (threads
// n2 = 0) the line offsets --------------------------------------------------
template <int KIND>
SGPU_HD void fx_load(const Args& a, int64_t blk, int t, const FxShared& sh) {
  const int line = t & 15, n2 = t >> 4;
  int ep = 0, eq = 0;
  if (KIND == C2C_FWD || KIND == C2C_BWD) {
    // C2C needs no common exponent before its first DFT (fx_c2c_pass1)
  } else {
    int64_t lp;
    bool lvp, lvq;
    pair_lines(a, blk * TL + line, lp, lvp, lvq);
    const int nh = N / 2 + 1;
    const int64_t n_in = KIND == R2C ? N : nh, n_out = KIND == R2C ? nh : N;
    if (n2 == 0) {
      sh.Lin[line] = lvp ? base_off(lp, n_in, a.inner) : -1;
      sh.Lin[TL + line] = lvq ? base_off(lp + 1, n_in, a.inner) : -1;
      sh.Lout[line] = lvp ? base_off(lp, n_out, a.inner) : -1;
      sh.Lout[TL + line] = lvq ? base_off(lp + 1, n_out, a.inner) : -1;
    }
    if (KIND == R2C) {
      const double* sp = a.in + (lvp ? base_off(lp, N, a.inner) : 0);
      const double* sq = a.in + (lvq ? base_off(lp + 1, N, a.inner) : 0);
#pragma unroll
      for (int n1 = 0; n1 < 16; ++n1) {
        const int64_t k = (int64_t)(16 * n1 + n2) * a.inner;
        const int e0 = lvp ? bexp(ldg(sp + k)) : 0, e1 = lvq ? bexp(ldg(sq + k)) : 0;
        ep = e0 > ep ? e0 : ep;
        eq = e1 > eq ? e1 : eq;
      }
    } else {  // C2R: exponents only (the values are loaded again in pass 1)
      const double* sp = a.in + 2 * (lvp ? base_off(lp, nh, a.inner) : 0);
      const double* sq = a.in + 2 * (lvq ? base_off(lp + 1, nh, a.inner) : 0);
#pragma unroll
      for (int n1 = 0; n1 < 16; ++n1) {
        const int j = 16 * n1 + n2;
        if (j > N / 2) continue;  // the conjugate half repeats entries 1..127
        const int64_t k = (int64_t)j * a.inner;
        const bool edge = j == 0 || j == N / 2;
        if (lvp) {
          double re, im;
          ldg2(sp + 2 * k, re, im);
          const int e0 = bexp(re), e1 = edge ? 0 : bexp(im);
          ep = e0 > ep ? e0 : ep;
          ep = e1 > ep ? e1 : ep;
        }
        if (lvq) {
          double re, im;
          ldg2(sq + 2 * k, re, im);
          const int e0 = bexp(re), e1 = edge ? 0 : bexp(im);
          eq = e0 > eq ? e0 : eq;
          eq = e1 > eq ? e1 : eq;
        }
      }
    }
  }
  sh.Ez[line * 16 + n2] = ep;
  sh.Ez[EX + line * 16 + n2] = eq;
}

// -- pass 1: convert on the line grid, 16-point DFT, twiddle, Z[line][k1][n2]
template <int KIND>
SGPU_HD void fx_pass1(const LinePlan& p, const Args& a, const FxShared& sh, int t) {
  const int line = t & 15, n2 = t >> 4;
  Cq v[16];
  if (KIND == C2C_FWD || KIND == C2C_BWD) {
    return;  // fx_c2c_pass1
  } else if (KIND == R2C) {
    const int Ep = line_exp(sh.Ez, line) + 1, Eq = line_exp(sh.Ez + EX, line) + 1;
    if (n2 == 0) {
      sh.El[line] = Ep - 1;
      sh.El[TL + line] = Eq - 1;
    }
    const long long bp = sh.Lin[line], bq = sh.Lin[TL + line];
    const double* sp = a.in + (bp >= 0 ? bp : 0);
    const double* sq = a.in + (bq >= 0 ? bq : 0);
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) {
      const int64_t k = (int64_t)(16 * n1 + n2) * a.inner;
      v[n1] = cq(bp >= 0 ? fx_from_f64(ldg(sp + k), Ep) : 0, bq >= 0 ? fx_from_f64(ldg(sq + k), Eq) : 0);
    }
  } else {  // C2R: z_j = conj(P_j + i Q_j), Hermitian extension, P and Q on their own grids
    const int Ep = line_exp(sh.Ez, line) + 1, Eq = line_exp(sh.Ez + EX, line) + 1;
    if (n2 == 0) {
      sh.El[line] = Ep - 1;
      sh.El[TL + line] = Eq - 1;
    }
    const long long bp = sh.Lin[line], bq = sh.Lin[TL + line];
    const double* sp = a.in + 2 * (bp >= 0 ? bp : 0);
    const double* sq = a.in + 2 * (bq >= 0 ? bq : 0);
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) {
      const int j = 16 * n1 + n2;
      const bool up = j > N / 2;
      const int64_t k = (int64_t)(up ? N - j : j) * a.inner;
      const bool edge = j == 0 || j == N / 2;
      long long pr = 0, pi = 0, qr = 0, qi = 0;
      if (bp >= 0) {
        double re, im;
        ldg2(sp + 2 * k, re, im);
        pr = fx_from_f64(re, Ep);
        pi = edge ? 0 : fx_from_f64(im, Ep);
      }
      if (bq >= 0) {
        double re, im;
        ldg2(sq + 2 * k, re, im);
        qr = fx_from_f64(re, Eq);
        qi = edge ? 0 : fx_from_f64(im, Eq);
      }
      if (up) {
        pi = -pi;
        qi = -qi;
      }
      // P + i Q = (pr - qi) + i (pi + qr), conjugated
      v[n1] = cq(pr - qi, -(pi + qr));
    }
  }
  q_dft16(v);
  Cq* z = sh.Z + (size_t)line * LDZ + n2;
  z[0] = v[0];
  const int* tw = p.tw_q;
#pragma unroll
  for (int k1 = 1; k1 < 16; ++k1) {
    const int e = n2 * k1;
    const Tw wr{tw[4 * e], tw[4 * e + 1]}, wi{tw[4 * e + 2], tw[4 * e + 3]};
    z[k1 * 17] = e == 0 ? v[k1] : q_mul(v[k1], wr, wi);
  }
}

// output scaling: value = X 2^(sx + Eh - 1076) (sm: a remaining FP64
// factor when the scale is not a power of two, else 1)
struct FxScale {
  int sx;
  double sm;
};

SGPU_HD double fx_out(long long X, int Eh, const FxScale& s) {
  const double d = fx_to_f64(X, s.sx + Eh - 1);
  return s.sm == 1.0 ? d : d * s.sm;
}

// -- C2C: pass 1 on the thread's own grid ----------------------------------
// Thread (line, n2) converts its 16 values with its own maximum exponent e_t
// (no barrier before the first DFT), and pass 2 puts the 16 threads' results
// on the line's grid E = max e_t by rounding shifts of E - e_t: a DFT of
// scaled subsequences, aligned before they are combined.
template <int KIND>
SGPU_HD void fx_c2c_pass1(const LinePlan& p, const Args& a, int64_t blk, const FxShared& sh, int t) {
  const int line = t & 15, n2 = t >> 4;
  const int64_t l = blk * TL + line;
  const bool live = l < a.nlines;
  const int64_t b = live ? base_off(l, N, a.inner) : 0;
  if (n2 == 0) sh.Lout[line] = live ? b : -1;
  const double* src = a.in + 2 * b;
  double x[32];
  int et = 0;
#pragma unroll
  for (int n1 = 0; n1 < 16; ++n1) {
    x[2 * n1] = 0.0;
    x[2 * n1 + 1] = 0.0;
    if (live) ldg2(src + 2 * (int64_t)(16 * n1 + n2) * a.inner, x[2 * n1], x[2 * n1 + 1]);
    const int e0 = bexp(x[2 * n1]), e1 = bexp(x[2 * n1 + 1]);
    et = e0 > et ? e0 : et;
    et = e1 > et ? e1 : et;
  }
  Cq v[16];
#pragma unroll
  for (int n1 = 0; n1 < 16; ++n1) {
    const long long im = fx_from_f64(x[2 * n1 + 1], et);
    v[n1] = cq(fx_from_f64(x[2 * n1], et), KIND == C2C_BWD ? -im : im);
  }
  sh.Ez[line * 16 + n2] = et;
  q_dft16(v);
  Cq* z = sh.Z + (size_t)line * LDZ + n2;
  z[0] = v[0];
  const int* tw = p.tw_q;
#pragma unroll
  for (int k1 = 1; k1 < 16; ++k1) {
    const int e = n2 * k1;
    const Tw wr{tw[4 * e], tw[4 * e + 1]}, wi{tw[4 * e + 2], tw[4 * e + 3]};
    z[k1 * 17] = e == 0 ? v[k1] : q_mul(v[k1], wr, wi);
  }
}

// C2C pass 2: align to the line grid, DFT; returns the line's exponent
SGPU_HD int fx_c2c_pass2(const FxShared& sh, int t, Cq* v) {
  const int line = t & 15, k1 = t >> 4;
  const int E = line_exp(sh.Ez, line);
  const int* ez = sh.Ez + line * 16;
  const Cq* z = sh.Z + (size_t)line * LDZ + k1 * 17;
#pragma unroll
  for (int n2 = 0; n2 < 16; ++n2) {
    const int d = E - ez[n2];
    v[n2] = cq(q_shr(z[n2].re, d), q_shr(z[n2].im, d));
  }
  q_dft16(v);
  return E;
}

template <int KIND>
SGPU_HD void fx_c2c_store(const Args& a, int t, const Cq* v, int Eh, const FxShared& sh, const FxScale& s) {
  const int line = t & 15, k1 = t >> 4;
  const long long b = sh.Lout[line];
  if (b < 0) return;
  const double qnan = u2d(0x7ff8000000000000ull);
  double* dst = a.out + 2 * b;
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) {
    double* d = dst + 2 * (int64_t)(k1 + 16 * k2) * a.inner;
    if (Eh == 0x7ff)
      st2(d, qnan, qnan);
    else
      st2(d, fx_out(v[k2].re, Eh, s), fx_out(KIND == C2C_BWD ? -v[k2].im : v[k2].im, Eh, s));
  }
}

// -- pass 2: thread (line, k1); X[k1 + 16 k2] in v[k2] ----------------------
SGPU_HD void fx_pass2_dft(const Cq* Z, int t, Cq* v) {
  const int line = t & 15, k1 = t >> 4;
  const Cq* z = Z + (size_t)line * LDZ + k1 * 17;
#pragma unroll
  for (int n2 = 0; n2 < 16; ++n2) v[n2] = z[n2];
  q_dft16(v);
}

// C2R: conj(X) -> real lines 2c (re) and 2c + 1 (im)
SGPU_HD void fx_c2r_store(const Args& a, int t, const Cq* v, const FxShared& sh, const FxScale& s) {
  const int line = t & 15, k1 = t >> 4;
  const double qnan = u2d(0x7ff8000000000000ull);
  const long long bp = sh.Lout[line], bq = sh.Lout[TL + line];
  const int Ep = sh.El[line], Eq = sh.El[TL + line];
  double* dp = bp >= 0 ? a.out + bp : nullptr;
  double* dq = bq >= 0 ? a.out + bq : nullptr;
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) {
    const int64_t k = (int64_t)(k1 + 16 * k2) * a.inner;
    if (dp) dp[k] = Ep == 0x7ff ? qnan : fx_out(v[k2].re, Ep + 1, s);
    if (dq) dq[k] = Eq == 0x7ff ? qnan : fx_out(-v[k2].im, Eq + 1, s);
  }
}

// R2C, after the pass-2 DFTs: W[line][k] = X[k] in shared memory (reusing Z
// behind a barrier), then P_k = (Z_k + conj Z_{N-k}) / 2 on p's grid and
// Q_k = -i (Z_k - conj Z_{N-k}) / 2 on q's (the halving folds into the
// exponent: the grids were 2^(1076 - E - 1), so E - 1 + 1)
SGPU_HD void fx_r2c_stash(Cq* W, int t, const Cq* v) {
  const int line = t & 15, k1 = t >> 4;
  Cq* w = W + (size_t)line * LDZ;
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) w[k1 + 16 * k2] = v[k2];
}

SGPU_HD void fx_r2c_post(const Args& a, const FxShared& sh, int t, int nth, const FxScale& s) {
  const int nh = N / 2 + 1;
  const double qnan = u2d(0x7ff8000000000000ull);
  for (int e = t; e < TL * nh; e += nth) {
    const int line = e & 15, k = e >> 4;
    const Cq* w = sh.Z + (size_t)line * LDZ;
    const Cq z = w[k];
    const Cq zc = q_conj(w[k == 0 ? 0 : N - k]);
    // z + zc = 2 DFT(p') and -i (z - zc) = 2 DFT(q'), each below 2 * 256 * 2^53
    const Cq P = z + zc;
    const Cq Q = q_mul_mi(z - zc);
    const long long bp = sh.Lout[line], bq = sh.Lout[TL + line];
    if (bp >= 0) {
      const int Ep = sh.El[line];
      double* d = a.out + 2 * (bp + (int64_t)k * a.inner);
      st2(d, Ep == 0x7ff ? qnan : fx_out(P.re, Ep, s), Ep == 0x7ff ? qnan : fx_out(P.im, Ep, s));
    }
    if (bq >= 0) {
      const int Eq = sh.El[TL + line];
      double* d = a.out + 2 * (bq + (int64_t)k * a.inner);
      st2(d, Eq == 0x7ff ? qnan : fx_out(Q.re, Eq, s), Eq == 0x7ff ? qnan : fx_out(Q.im, Eq, s));
    }
  }
}

// the output scale as a power of two and a remaining factor
inline FxScale fx_scale(double scl) {
  FxScale s;
  int e = 0;
  const double m = std::frexp(scl, &e);  // scl = m 2^e, m in [0.5, 1)
  if (m == 0.5) {
    s.sx = e - 1;
    s.sm = 1.0;
  } else {
    s.sx = 0;
    s.sm = scl;
  }
  return s;
}

}  // namespace f256
}  // namespace sgpu
