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
// Grids.  C2C: thread (line, n2) converts its 16 values on its own grid
// (its largest exponent) before the first DFT; pass 2 aligns the 16 threads'
// results to the line's grid by rounding shifts.  R2C / C2R transform each
// real line alone as a half-length complex FFT (z_n = x_2n + i x_2n+1, 128
// points: DFT16 x DFT8 four-step, 32 lines per CTA) with the same per-thread
// grids, so no line shares a grid with another and no exponent pass or
// barrier comes before the first DFT.  R2C separates the even / odd spectra
// after the FFT (X_k = E_k + W^k O_k from Z_k and Z_{128-k}), C2R combines
// them before it (Z_k = X_k + conj X_{128-k} + i W^-k (X_k - conj X_{128-k})).
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

// C2C shared memory: the exchange buffer, per (line, n2) the pass-1 grid
// exponents, per line its exponent and output offset (-1 past the array)
SGPU_HD size_t fx_smem_bytes() {
  return sizeof(Cq) * (size_t)TL * LDZ + sizeof(int) * (16 * TL + TL) + sizeof(long long) * TL + 8;
}
struct FxShared {
  Cq* Z;
  int* Ez;          // [TL][16]
  int* El;          // [TL]
  long long* Lout;  // [TL]
};
SGPU_HD FxShared fx_shared(unsigned char* base) {
  FxShared f;
  f.Z = (Cq*)base;
  f.Ez = (int*)(base + sizeof(Cq) * (size_t)TL * LDZ);
  f.El = f.Ez + 16 * TL;
  f.Lout = (long long*)(f.El + TL);  // 17 TL = 272 ints: 8-byte aligned
  return f;
}

// the maximum over the 16 threads of `line` (Ez: [line][n2])
SGPU_HD int line_exp(const int* Ez, int line) {
  int E = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) E = Ez[line * 16 + i] > E ? Ez[line * 16 + i] : E;
  return E;
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

// Thread (line, n2)'s 16 values x[16 n1 + n2] (real, imaginary) straight
// from global memory, and their largest exponent
SGPU_HD int fx_c2c_load(const Args& a, int64_t blk, const FxShared& sh, int t, double (&x)[32]) {
  const int line = t & 15, n2 = t >> 4;
  const int64_t l = blk * TL + line;
  const bool live = l < a.nlines;
  const int64_t b = live ? base_off(l, N, a.inner) : 0;
  if (n2 == 0) sh.Lout[line] = live ? b : -1;
  const double* src = a.in + 2 * b;
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
  return et;
}

// The same values from a tile of the block's TL lines staged in shared
// memory, row-major [256][TL] complex (a tensor copy's box; lines past the
// array arrive as zeros)
SGPU_HD int fx_c2c_load_tile(const Args& a, int64_t blk, const FxShared& sh, const double* tile, int t,
                             double (&x)[32]) {
  const int line = t & 15, n2 = t >> 4;
  const int64_t l = blk * TL + line;
  if (n2 == 0) sh.Lout[line] = l < a.nlines ? base_off(l, N, a.inner) : -1;
  int et = 0;
#pragma unroll
  for (int n1 = 0; n1 < 16; ++n1) {
    const double* q = tile + 2 * ((16 * n1 + n2) * TL + line);
    x[2 * n1] = q[0];
    x[2 * n1 + 1] = q[1];
    const int e0 = bexp(x[2 * n1]), e1 = bexp(x[2 * n1 + 1]);
    et = e0 > et ? e0 : et;
    et = e1 > et ? e1 : et;
  }
  return et;
}

// -- C2C: pass 1 on the thread's own grid ----------------------------------
// Thread (line, n2) converts its 16 values with its own maximum exponent e_t
// (no barrier before the first DFT), and pass 2 puts the 16 threads' results
// on the line's grid E = max e_t by rounding shifts of E - e_t: a DFT of
// scaled subsequences, aligned before they are combined.
template <int KIND>
SGPU_HD void fx_c2c_pass1_regs(const LinePlan& p, const FxShared& sh, int t, const double (&x)[32], int et) {
  const int line = t & 15, n2 = t >> 4;
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

template <int KIND>
SGPU_HD void fx_c2c_pass1(const LinePlan& p, const Args& a, int64_t blk, const FxShared& sh, int t) {
  double x[32];
  const int et = fx_c2c_load(a, blk, sh, t, x);
  fx_c2c_pass1_regs<KIND>(p, sh, t, x, et);
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

// -- R2C / C2R: one real line as a 128-point complex FFT ------------------
const int TH = 32;    // real lines per CTA
const int MH = 128;   // complex FFT length
const int LDH = 129;  // shared-memory line stride (odd in 16-byte units)

struct FxHalf {
  Cq* Z;            // [TH][LDH]: entry (k1, n2) of pass 1 at k1 * 8 + n2; spectrum k after pass 2
  int* Ez;          // [TH][8]: pass-1 grid exponents
  int* El;          // [TH]: line exponents
  long long* Lout;  // [TH]: output offset of each line (-1 past the array)
};
SGPU_HD size_t fxh_smem_bytes() {
  return sizeof(Cq) * (size_t)TH * LDH + sizeof(int) * (8 * TH + TH) + sizeof(long long) * TH + 8;
}
SGPU_HD FxHalf fxh_shared(unsigned char* base) {
  FxHalf f;
  f.Z = (Cq*)base;
  f.Ez = (int*)(base + sizeof(Cq) * (size_t)TH * LDH);
  f.El = f.Ez + 8 * TH;
  // 8-byte aligned: the int arrays hold 9 TH = 288 entries
  f.Lout = (long long*)(f.El + TH);
  return f;
}

// 8-point forward DFT in place, natural order (2 x 4: n = 4 n1 + n2, k = k1 + 2 k2)
SGPU_HD void q_dft8(Cq* v) {
  Cq a[4][2];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    const Cq t0 = v[n2], t1 = v[4 + n2];
    a[n2][0] = t0 + t1;
    a[n2][1] = q_mul_w16(t0 - t1, 2 * n2);  // W_8^{n2}
  }
#pragma unroll
  for (int k1 = 0; k1 < 2; ++k1) {
    Cq t[4] = {a[0][k1], a[1][k1], a[2][k1], a[3][k1]};
    q_dft4(t);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 2 * k2] = t[k2];
  }
}

SGPU_HD Tw tw_re(const LinePlan& p, int e) { return Tw{p.tw_q[4 * e], p.tw_q[4 * e + 1]}; }
SGPU_HD Tw tw_im(const LinePlan& p, int e) { return Tw{p.tw_q[4 * e + 2], p.tw_q[4 * e + 3]}; }

// pass-1 tail shared by R2C and C2R: 16-point DFT over n1, twiddle
// W_128^{n2 k1} (= W_256^{2 n2 k1}), Z[line][k1][n2]
SGPU_HD void fxh_store_pass1(const LinePlan& p, const FxHalf& sh, int line, int n2, Cq* v) {
  q_dft16(v);
  Cq* z = sh.Z + (size_t)line * LDH + n2;
  z[0] = v[0];
#pragma unroll
  for (int k1 = 1; k1 < 16; ++k1) {
    const int e = 2 * n2 * k1;
    z[k1 * 8] = e == 0 ? v[k1] : q_mul(v[k1], tw_re(p, e), tw_im(p, e));
  }
}

// R2C pass 1: thread t = (n2 << 5) | line loads x[16 n1 + 2 n2] and
// x[16 n1 + 2 n2 + 1] (z_{8 n1 + n2}) of its line, on its own grid
SGPU_HD void fxh_r2c_pass1(const LinePlan& p, const Args& a, int64_t blk, const FxHalf& sh, int t) {
  const int line = t & 31, n2 = t >> 5;
  const int64_t l = blk * TH + line;
  const bool live = l < a.nlines;
  const int64_t bi = live ? base_off(l, N, a.inner) : 0;
  if (n2 == 0) sh.Lout[line] = live ? base_off(l, N / 2 + 1, a.inner) : -1;
  const double* src = a.in + bi;
  double x[32];
  int et = 0;
#pragma unroll
  for (int n1 = 0; n1 < 16; ++n1) {
    const int64_t k = (int64_t)(16 * n1 + 2 * n2) * a.inner;
    x[2 * n1] = live ? ldg(src + k) : 0.0;
    x[2 * n1 + 1] = live ? ldg(src + k + a.inner) : 0.0;
    const int e0 = bexp(x[2 * n1]), e1 = bexp(x[2 * n1 + 1]);
    et = e0 > et ? e0 : et;
    et = e1 > et ? e1 : et;
  }
  Cq v[16];
#pragma unroll
  for (int n1 = 0; n1 < 16; ++n1) v[n1] = cq(fx_from_f64(x[2 * n1], et + 1), fx_from_f64(x[2 * n1 + 1], et + 1));
  sh.Ez[line * 8 + n2] = et;
  fxh_store_pass1(p, sh, line, n2, v);
}

// C2R pass 1: Z'_k = X_k + conj X_{128-k} + i W^-k (X_k - conj X_{128-k})
// for k = 8 n1 + n2 (the imaginary parts of X_0 and X_128 are ignored, as
// an FP64 C2R does), conjugated for the inverse DFT; the inputs are read
// once for the thread's exponent and again (L1) to convert
SGPU_HD void fxh_c2r_pass1(const LinePlan& p, const Args& a, int64_t blk, const FxHalf& sh, int t) {
  const int line = t & 31, n2 = t >> 5;
  const int nh = N / 2 + 1;
  const int64_t l = blk * TH + line;
  const bool live = l < a.nlines;
  const int64_t bi = live ? base_off(l, nh, a.inner) : 0;
  if (n2 == 0) sh.Lout[line] = live ? base_off(l, N, a.inner) : -1;
  const double* src = a.in + 2 * bi;
  int et = 0;
  if (live) {
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) {
      const int k = 8 * n1 + n2, m = MH - k;
      double r0, i0, r1, i1;
      ldg2(src + 2 * (int64_t)k * a.inner, r0, i0);
      ldg2(src + 2 * (int64_t)m * a.inner, r1, i1);
      const int e0 = bexp(r0), e1 = k == 0 ? 0 : bexp(i0), e2 = bexp(r1), e3 = m == MH ? 0 : bexp(i1);
      et = e0 > et ? e0 : et;
      et = e1 > et ? e1 : et;
      et = e2 > et ? e2 : et;
      et = e3 > et ? e3 : et;
    }
  }
  const int Eh = et + 1;
  Cq v[16];
#pragma unroll
  for (int n1 = 0; n1 < 16; ++n1) {
    const int k = 8 * n1 + n2, m = MH - k;
    double r0 = 0.0, i0 = 0.0, r1 = 0.0, i1 = 0.0;
    if (live) {
      ldg2(src + 2 * (int64_t)k * a.inner, r0, i0);
      ldg2(src + 2 * (int64_t)m * a.inner, r1, i1);
    }
    const Cq xk = cq(fx_from_f64(r0, Eh), k == 0 ? 0 : fx_from_f64(i0, Eh));
    const Cq xm = cq(fx_from_f64(r1, Eh), m == MH ? 0 : -fx_from_f64(i1, Eh));  // conj X_{128-k}
    const Cq S = xk + xm, D = xk - xm;
    // D W^-k = conj(conj(D) W^k) with the table's W^k (its -1 is exact)
    const Cq DW = k == 0 ? D : q_conj(q_mul(q_conj(D), tw_re(p, k), tw_im(p, k)));
    v[n1] = q_conj(S + q_mul_pi(DW));
  }
  sh.Ez[line * 8 + n2] = et;
  fxh_store_pass1(p, sh, line, n2, v);
}

// pass 2 of one item (line, k1): align the 8 pass-1 threads of the line to
// its grid, DFT8 over n2; v[k2] = spectrum index k1 + 16 k2.  Returns the
// line's exponent (without the headroom bit).
SGPU_HD int fxh_pass2(const FxHalf& sh, int line, int k1, Cq* v) {
  const int* ez = sh.Ez + line * 8;
  int E = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) E = ez[i] > E ? ez[i] : E;
  const Cq* z = sh.Z + (size_t)line * LDH + k1 * 8;
#pragma unroll
  for (int n2 = 0; n2 < 8; ++n2) {
    const int d = E - ez[n2];
    v[n2] = cq(q_shr(z[n2].re, d), q_shr(z[n2].im, d));
  }
  q_dft8(v);
  return E;
}

// R2C after pass 2 (a barrier in between): W[line][k] = Z_k
SGPU_HD void fxh_r2c_stash(const FxHalf& sh, int line, int k1, const Cq* v, int E) {
  Cq* w = sh.Z + (size_t)line * LDH;
#pragma unroll
  for (int k2 = 0; k2 < 8; ++k2) w[k1 + 16 * k2] = v[k2];
  if (k1 == 0) sh.El[line] = E;
}

// R2C after the stash (a barrier in between): 2 X_k = A - i W^k B with
// A = Z_k + conj Z_{128-k}, B = Z_k - conj Z_{128-k}, k = 0..128, on the
// line's grid (the halving folds into the exponent)
SGPU_HD void fxh_r2c_post(const LinePlan& p, const Args& a, const FxHalf& sh, int t, int nth, const FxScale& s) {
  const int nh = N / 2 + 1;
  const double qnan = u2d(0x7ff8000000000000ull);
  for (int e = t; e < TH * nh; e += nth) {
    const int line = e & 31, k = e >> 5;
    const long long b = sh.Lout[line];
    if (b < 0) continue;
    const Cq* w = sh.Z + (size_t)line * LDH;
    const Cq zk = w[k & (MH - 1)];
    const Cq zm = q_conj(w[(MH - k) & (MH - 1)]);
    const Cq A = zk + zm, B = zk - zm;
    const Cq WB = k == 0 ? B : q_mul(B, tw_re(p, k), tw_im(p, k));
    const Cq X2 = A + q_mul_mi(WB);
    const int E = sh.El[line];
    double* d = a.out + 2 * (b + (int64_t)k * a.inner);
    if (E == 0x7ff)
      st2(d, qnan, qnan);
    else
      st2(d, fx_out(X2.re, E, s), fx_out(X2.im, E, s));
  }
}

// C2R after pass 2: z_n = conj(v) at n = k1 + 16 k2 -> x_2n = Re, x_2n+1 = Im
SGPU_HD void fxh_c2r_store(const Args& a, const FxHalf& sh, int line, int k1, const Cq* v, int E,
                           const FxScale& s) {
  const long long b = sh.Lout[line];
  if (b < 0) return;
  const double qnan = u2d(0x7ff8000000000000ull);
  double* dst = a.out + b;
#pragma unroll
  for (int k2 = 0; k2 < 8; ++k2) {
    const int64_t n = k1 + 16 * k2;
    double* d = dst + 2 * n * a.inner;
    if (E == 0x7ff) {
      d[0] = qnan;
      d[a.inner] = qnan;
    } else {
      d[0] = fx_out(v[k2].re, E + 1, s);
      d[a.inner] = fx_out(-v[k2].im, E + 1, s);
    }
  }
}

// CTAs of a fixed-point launch
SGPU_HD int64_t fx_tiles(int kind, int64_t nlines) {
  return kind == R2C || kind == C2R ? (nlines + TH - 1) / TH : (nlines + TL - 1) / TL;
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
