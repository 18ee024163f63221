// Fused split-BF16 line contraction on the tensor cores: the building blocks
// (host + device) of k_lc_fused (lc_fused.cu), shared with the CPU emulator.
//
//   out(l, n) = sum_k in(l, k) M[k][n]     lines l of length N, K active entries
//
// The earlier contraction (ozaki.cuh) wrote BF16 digit slices of the whole
// input to HBM in one kernel and read them back in another.  This one splits
// the lines inside the GEMM kernel, so a pass moves the algorithmic bytes
// only (read the input, write the output).  The problem is set up transposed:
//
//   D[n][line] = sum_k Mt[n][k] X[line][k]
//
// MMA M = 128 output indices n (MT CTAs share a tile of lines: CTA r of the
// group owns outputs 128 r .. 128 r + 127), MMA N = lines, K = entries.
// Every CTA of a group splits the tile's lines into digits in its own shared
// memory (the second read of the lines hits L2); all synchronisation stays
// inside the CTA.  The matrix digits (A operand) are split on the host and
// streamed from L2 with bulk copies.  Outputs past the last full 128-row tile
// (at most two: N = 257 has output 256 left over) are FP64 dot products that
// the digit threads accumulate while they read the lines, each CTA of the
// group taking a share of the tile's lines.
//
// Digits.  Every line (and every matrix column) is scaled by a power of two
// 2^e with all |x| < 2^e and cut to a P-bit fixed-point integer X < 2^P
// (the matrix rounded, the lines truncated), P = W S - H (H bits of
// headroom), which is cut
// into S balanced W-bit digits: X = sum_s d_s 2^{W(S-1-s)}, d_s in
// [-2^{W-1}, 2^{W-1}) for s >= 1 and |d_0| <= 2^{W-H} + 1.  The digits are
// stored as integers in BF16 (exact: at most 8 significant bits).  Products
// d_s d'_t with s + t <= S - 1 are kept; all S digit groups g = s + t get an
// accumulator of their own in TMEM.  For A_s (matrix digit s) one MMA
// multiplies it by the line digits of t = 0 .. S-1-s laid side by side along
// N, whose D columns are exactly groups s .. S-1 (N = (S - s) BN, cut into
// MMAs of at most 256 columns): S(S+1)/2 digit products in few wide MMAs.
// Group sums are integers; a group's FP32 accumulator is exact while its
// worst-case magnitude stays below 2^24 (checked by exact_groups() below).
// The epilogue adds the groups in 64-bit fixed point and assembles the FP64
// result with integer instructions (no FP64 arithmetic per element).
//
// Configuration: W = 8, S = 7, H = 2 (54 bits, 28 digit products).  Groups
// 0..3 are exact for every input with K <= 339; groups 4..6 (2^-32 .. 2^-48
// below the leading one) are exact as long as their sums stay below 2^24,
// which only digit patterns aligned along a whole line could break.  The
// dropped products (s + t >= 7) leave a normwise error ~2e-15 of
// |x| |M| - the FP64 level the Chebyshev Dirichlet Helmholtz recurrence needs
// (it magnifies its input's perturbations up to ~4000x).  More headroom
// makes more groups exact but loses two bits of product precision per bit
// (H = 3 measured 1e-14).  Tiles of BN = 64 lines (7 x 64 accumulator
// columns, one set in TMEM) or BN = 32 (two sets of 7 x 32: the next tile's
// MMAs run while this tile's epilogue reads the other set).
#pragma once

#include <cmath>
#include <cstring>

#include "sgpu_common.cuh"
#include "tc_ptx.cuh"

namespace sgpu {
namespace lc {

const int MROWS = 128;    // outputs per CTA = MMA M
const int KSTEP = 16;     // K per MMA (kind::f16)
const int A_BLOCK = MROWS * KSTEP;  // elements of one matrix-digit block (4 KB)
const int LBO_A = MROWS * 16;       // bytes between the two 8-wide K core-matrix columns of A
const int SBO = 128;                // bytes between adjacent 8-row core matrices
const int MAX_MT = 4;               // CTAs per tile group (outputs <= 512 + 2)
const int MAX_NX = 2;               // outputs computed as FP64 dot products

template <int W_, int S_, int H_, int BN_>
struct Cfg {
  static const int W = W_, S = S_, H = H_, BN = BN_;
  static const int P = W * S - H;  // fixed-point bits of a scaled entry
  static const int NBUF = 2 * S * BN <= 512 ? 2 : 1;
  static const int A_STAGE = S * A_BLOCK * 2;  // bytes of one K step of matrix digits
  static const int B_STAGE = S * BN * KSTEP * 2;
  static const int LBO_B = S * BN * 16;
  // fractional bits of the epilogue's fixed-point sum T = sum_g G_g 2^{F-Wg}:
  // |G_0| <= (2^{W-H}+1)^2 K < 2^20.5 for K <= KMAX keeps |T| < 2^62, and the
  // resolution of T is 2^-53 of 2^{ex+em} (the scale of the line times the
  // scale of the matrix column)
  static const int F = 41;
  static const int KMAX = 339;
  static_assert(S * BN <= 512, "accumulators exceed TMEM");
  static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256, "MMA N");
  static_assert(W * S - H <= 60 && W <= 8, "digit layout");
};
typedef Cfg<8, 7, 2, 64> CfgWide;    // one accumulator set, 64-line tiles
typedef Cfg<8, 7, 2, 32> CfgNarrow;  // two accumulator sets, 32-line tiles

// largest |sum over K of group g| in units of the digit products
SGPU_HD double group_bound(int W, int S, int H, int g, int K) {
  const double d0 = (double)((1 << (W - H)) + 1), d = (double)(1 << (W - 1));
  double b = 0;
  for (int s = 0; s <= g; ++s) {
    const int t = g - s;
    if (s > S - 1 || t > S - 1) continue;
    b += (s == 0 ? d0 : d) * (t == 0 ? d0 : d);
  }
  return b * K;
}

// number of leading digit groups whose FP32 sums are exact for K entries
SGPU_HD int exact_groups(int W, int S, int H, int K) {
  int g = 0;
  while (g < S && group_bound(W, S, H, g, K) < 16777216.0) ++g;
  return g;
}

SGPU_HD uint32_t exp_field(double x) {
  uint64_t b;
  memcpy(&b, &x, 8);
  return (uint32_t)((b >> 52) & 0x7ff);
}

// e with every |x| of the line below 2^e, from the largest biased exponent
// field (0 for an all-zero line; subnormal entries count as zero)
SGPU_HD int exp_from_field(uint32_t maxfield) { return maxfield ? (int)maxfield - 1022 : 0; }

// balanced digits of x at scale e as BF16 bit patterns of the integers d_s
template <class C>
SGPU_HD void split_digits(double x, int e, uint16_t (&out)[C::S]) {
  constexpr int W = C::W, S = C::S, P = C::P;
  uint64_t b;
  memcpy(&b, &x, 8);
  const int field = (int)((b >> 52) & 0x7ff);
  uint64_t X = 0;
  if (field != 0) {
    const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    // X = round(|x| 2^{P-e}) = round(m 2^{-sh}), |x| = m 2^{field-1075}
    const int sh = 1075 + e - P - field;
    if (sh <= 0)
      X = m << (-sh);
    else if (sh < 64)
      X = (m + (1ull << (sh - 1))) >> sh;
  }
  int d[S];
  int carry = 0;
#pragma unroll
  for (int s = S - 1; s >= 1; --s) {
    int u = (int)((uint32_t)(X >> (W * (S - 1 - s))) & ((1u << W) - 1)) + carry;
    carry = u >= (1 << (W - 1)) ? 1 : 0;
    d[s] = u - (carry << W);
  }
  d[0] = (int)(X >> (W * (S - 1))) + carry;
  const uint32_t neg = (uint32_t)(b >> 63);
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const int v = neg ? -d[s] : d[s];
    // exact float of v (|v| <= 2^8) by the 1.5 * 2^23 bias; its top 16 bits
    // are the BF16 value
    const uint32_t biased = 0x4B400000u + (uint32_t)v;
    float f;
    memcpy(&f, &biased, 4);
    f -= 12582912.0f;
    uint32_t fb;
    memcpy(&fb, &f, 4);
    out[s] = (uint16_t)(fb >> 16);
  }
}

// byte permute (the device PRMT): result byte i = byte sel[4i+3:4i] of the
// eight-byte pool {b, a} (a = bytes 0..3, b = bytes 4..7)
SGPU_HD uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel) {
#if defined(__CUDA_ARCH__)
  return __byte_perm(a, b, sel);
#else
  const uint64_t pool = ((uint64_t)b << 32) | a;
  uint32_t r = 0;
  for (int i = 0; i < 4; ++i) r |= (uint32_t)((pool >> (8 * ((sel >> (4 * i)) & 7))) & 0xff) << (8 * i);
  return r;
#endif
}

SGPU_HD float fma_rn(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}

// The digits of eight consecutive entries of one line (one 16-byte
// core-matrix row per digit slice): out[s] = BF16 d_s of x[0..7], little end
// first.  W = 8 digits are bytes: adding 0x80 to every byte below the top
// one turns X into Y whose bytes y_s give the balanced digits d_s = y_s - 128
// (the carries of the addition are exactly the balancing carries), and the
// top digit is Y's top byte.  A digit becomes an FP32 by the 1.5 * 2^23 bias
// (one byte permute builds the biased float, one FMA removes the bias and
// applies the sign); its top 16 bits are the BF16 value, and one more byte
// permute packs two entries' digits into a word.
template <class C>
SGPU_HD void split8(const double (&x)[8], int e, uint4 (&out)[C::S]) {
  static_assert(C::W == 8 && C::S == 7 && C::P <= 62, "byte digits");
  float v[8][C::S];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    uint64_t b;
    memcpy(&b, &x[q], 8);
    const uint32_t hi = (uint32_t)(b >> 32);
    const int field = (int)((hi >> 20) & 0x7ff);
    const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    // X = floor(|x| 2^{P-e}) = m 2^{-sh} truncated (at most one unit of
    // 2^{e-P} below the exact value); sh >= 53 - P = -1 because |x| < 2^e,
    // and X = 0 for zeros, subnormals and shifts past the mantissa
    const int sh = 1075 + e - C::P - field;
    uint64_t X = sh < 0 ? (m << 1) : (m >> (sh & 63));
    X = (field == 0 || sh > 62) ? 0 : X;
    const uint64_t Y = X + 0x0000808080808080ull;
    const uint32_t ylo = (uint32_t)Y, yhi = (uint32_t)(Y >> 32);
    const uint32_t sbit = hi & 0x80000000u;
    uint32_t ub;
    float sgn, c1, c0;
    ub = 0x3F800000u | sbit;
    memcpy(&sgn, &ub, 4);
    ub = 0xCB400080u ^ sbit;  // -(1.5 * 2^23 + 128), sign-flipped for negative x
    memcpy(&c1, &ub, 4);
    ub = 0xCB400000u ^ sbit;  // -(1.5 * 2^23)
    memcpy(&c0, &ub, 4);
    // digit s sits in byte 6 - s of Y: s = 0..2 in yhi bytes 2, 1, 0; s = 3..6
    // in ylo bytes 3, 2, 1, 0
#pragma unroll
    for (int sd = 0; sd < C::S; ++sd) {
      const int byte = 6 - sd;
      const uint32_t word = byte >= 4 ? yhi : ylo;
      const uint32_t fb = prmt(word, 0x4B400000u, 0x7640u | (uint32_t)(byte & 3));
      float f;
      memcpy(&f, &fb, 4);
      v[q][sd] = fma_rn(f, sgn, sd == 0 ? c0 : c1);
    }
  }
#pragma unroll
  for (int sd = 0; sd < C::S; ++sd) {
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 8; q += 2) {
      uint32_t a, b;
      memcpy(&a, &v[q][sd], 4);
      memcpy(&b, &v[q + 1][sd], 4);
      w[q >> 1] = prmt(a, b, 0x7632u);
    }
    out[sd].x = w[0];
    out[sd].y = w[1];
    out[sd].z = w[2];
    out[sd].w = w[3];
  }
}

SGPU_HD int32_t f2i_rn(float v) {
#if defined(__CUDA_ARCH__)
  return __float2int_rn(v);
#else
  return (int32_t)lrintf(v);
#endif
}

SGPU_HD int clz64(uint64_t a) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)a);
#else
  return a ? __builtin_clzll(a) : 64;
#endif
}

// One output from the S = 7 group accumulators (FP32 bit patterns of
// integers below 2^25 in magnitude):
//   value = 2^{W(2S-2) + ex + em - 2P} sum_g G_g 2^{-W g}
//         = T 2^{ex + em + W(2S-2) - 2P - F},  T = sum_g G_g 2^{F - W g}
// with T rounded at 2^-1 (group 6 enters as round(G_6 / 2^7)).  The groups
// become int32 exactly; G_0 2^8 + G_1 fits in int32 (|G_0| < 2^20.5), the
// rest are 32 x 32 -> 64-bit multiply-adds; T (|T| < 2^62) becomes FP64 bits
// round-to-nearest-even with integer instructions: a mantissa that rounds up
// to 2^53 carries into the exponent field by itself.
template <class C>
SGPU_HD double combine(const uint32_t (&gb)[C::S], int ex, int em) {
  static_assert(C::W == 8 && C::S == 7 && C::F == 41, "byte digits, 7 groups");
  int32_t gi[C::S];
#pragma unroll
  for (int g = 0; g < C::S; ++g) {
    float f;
    memcpy(&f, &gb[g], 4);
    gi[g] = f2i_rn(f);
  }
  const int32_t A = gi[0] * 256 + gi[1];
  int64_t T = (int64_t)A * ((int64_t)1 << 33);
  T += (int64_t)gi[2] * ((int64_t)1 << 25);
  T += (int64_t)gi[3] * ((int64_t)1 << 17);
  T += (int64_t)gi[4] * ((int64_t)1 << 9);
  T += (int64_t)gi[5] * 2;
  T += (int64_t)((gi[6] + 64) >> 7);
  const int E = ex + em + C::W * (2 * C::S - 2) - 2 * C::P - C::F;
  if (T == 0) return 0.0;
  const uint64_t sbit = (uint64_t)T & 0x8000000000000000ull;
  const uint64_t a = T < 0 ? (uint64_t)(-T) : (uint64_t)T;
  const int sh = 11 - clz64(a);  // puts the leading bit at 2^52
  uint64_t mant;
  if (sh > 0) {
    mant = a >> sh;
    const uint64_t rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    mant += (rem > half || (rem == half && (mant & 1))) ? 1 : 0;
  } else {
    mant = a << (-sh);
  }
  const int biased = E + sh + 1075;
  if (biased <= 0 || biased >= 2047) {  // outside the normal range: rare
    const double r = ldexp((double)mant, E + sh);
    return sbit ? -r : r;
  }
  const uint64_t bits = sbit | (((uint64_t)(biased - 1) << 52) + mant);
  double r;
  memcpy(&r, &bits, 8);
  return r;
}

// 32 x 32 -> 64-bit multiply-add (one wide integer multiply-add on the
// device)
SGPU_HD int64_t mad_wide(int32_t a, int32_t b, int64_t c) {
#if defined(__CUDA_ARCH__)
  int64_t d;
  asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
  return d;
#else
  return (int64_t)a * b + c;
#endif
}

// T 2^E as FP64 (|T| < 2^62), round-to-nearest-even, the same value as
// combine()'s conversion: the hardware's integer -> FP64 conversion rounds T
// to 53 bits (to nearest, ties to even; one instruction on the FP64 pipe,
// which the contraction otherwise leaves mostly idle, in place of ~30
// integer ones), and 2^E is added to the exponent field while the result
// stays normal (ldexp for the rare rest)
SGPU_HD double fixed62_to_double(int64_t T, int E) {
  const double v = (double)T;
  uint64_t b;
  memcpy(&b, &v, 8);
  const int eb = (int)((b >> 52) & 0x7ff) + E;
  if (T == 0) return 0.0;
  if (eb <= 0 || eb >= 2047) return ldexp(v, E);  // outside the normal range: rare
  b += (uint64_t)(int64_t)E << 52;
  double r;
  memcpy(&r, &b, 8);
  return r;
}

// Eight outputs at once (the eight lines of one TMEM load), written step by
// step across the outputs so that their independent integer chains
// interleave: a[g][j] = group g of output j, ex[j] the line scales, em the
// matrix column's scale.  The same integers and the same rounding as
// combine(), with the group terms as wide multiply-adds by their powers of
// two.
template <class C>
SGPU_HD void combine8(const uint32_t (&a)[C::S][8], const int (&ex)[8], int em, double (&out)[8]) {
  static_assert(C::W == 8 && C::S == 7 && C::F == 41, "byte digits, 7 groups");
  int64_t T[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float f0, f1;
    memcpy(&f0, &a[0][j], 4);
    memcpy(&f1, &a[1][j], 4);
    T[j] = (int64_t)(f2i_rn(f0) * 256 + f2i_rn(f1)) * ((int64_t)1 << 33);
  }
#pragma unroll
  for (int g = 2; g < C::S; ++g)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float f;
      memcpy(&f, &a[g][j], 4);
      const int32_t gi = f2i_rn(f);
      // weights 2^25, 2^17, 2^9, 2^1 and a rounded 2^-7
      T[j] = g < 6 ? mad_wide(gi, 1 << (C::F - C::W * g), T[j]) : mad_wide((gi + 64) >> 7, 1, T[j]);
    }
#pragma unroll
  for (int j = 0; j < 8; ++j)
    out[j] = fixed62_to_double(T[j], ex[j] + em + C::W * (2 * C::S - 2) - 2 * C::P - C::F);
}

// geometry of one contraction over contiguous lines: rows are lines (complex
// lines give two rows, real and imaginary parts, at element stride 2)
struct Geom {
  int64_t nrows;
  int N;        // line length (input and output)
  int K;        // leading input entries the matrix uses
  int cplx;
  int nsteps;   // MMA K steps of 16 (K rounded up)
  int MT;       // CTAs per tile group = 128-output tiles on the tensor cores
  int Nmma;     // outputs on the tensor cores (the rest: FP64 dot products)
  int NX;       // outputs as FP64 dot products (N - Nmma, at most 2)
  int64_t tiles;  // tiles of BN rows
};

SGPU_HD int64_t row_base(const Geom& g, int64_t row) {
  return g.cplx ? (row >> 1) * 2 * (int64_t)g.N + (row & 1) : row * (int64_t)g.N;
}
SGPU_HD int kstride(const Geom& g) { return g.cplx ? 2 : 1; }

// outputs on the tensor cores: whole 128-row tiles, plus the last partial
// tile unless at most two outputs spill past a multiple of 128
inline void output_split(int N, int& MT, int& Nmma, int& NX) {
  const int rem = N % MROWS;
  if (N > MROWS && rem >= 1 && rem <= MAX_NX) {
    Nmma = N - rem;
    NX = rem;
  } else {
    Nmma = N;
    NX = 0;
  }
  MT = (Nmma + MROWS - 1) / MROWS;
}

inline bool supported_nk(int N, int K) {
  if (N < 16 || K < 1 || K > N) return false;
  int MT, Nmma, NX;
  output_split(N, MT, Nmma, NX);
  return MT <= MAX_MT && K <= CfgWide::KMAX && exact_groups(CfgWide::W, CfgWide::S, CfgWide::H, K) >= 4;
}

// index of element (row n, k) inside one 128 x 16 matrix-digit block,
// canonical K-major no-swizzle layout [k / 8][n / 8][n % 8][k % 8]
SGPU_HD int a_index(int n, int k) { return (k >> 3) * (MROWS * 8) + (n >> 3) * 64 + (n & 7) * 8 + (k & 7); }

// byte offset of the 16-byte core-matrix row (line row j, K half h) of digit
// slice t inside a B stage: rows t BN + j laid side by side along N,
// [h][row / 8][row % 8][8 elements]
template <class C>
SGPU_HD uint32_t b_offset(int t, int j, int h) {
  const int row = t * C::BN + j;
  return (uint32_t)((h * (C::S * C::BN / 8) + (row >> 3)) * 128 + (row & 7) * 16);
}

// host: matrix digits for a geometry, tiles [mt][kstep][s][128 x 16] (zero
// past K and past Nmma), per-output exponents em[MT * 128], and the FP64
// columns of the dot-product outputs xcol[NX][K]
template <class C>
inline void split_matrix_host(const double* M, const Geom& g, uint16_t* tiles, int* em, double* xcol) {
  const size_t nt = (size_t)g.MT * g.nsteps * C::S * A_BLOCK;
  memset(tiles, 0, nt * sizeof(uint16_t));
  for (int n = 0; n < g.MT * MROWS; ++n) em[n] = 0;
  for (int n = 0; n < g.Nmma; ++n) {
    uint32_t mf = 0;
    for (int k = 0; k < g.K; ++k) {
      const uint32_t f = exp_field(M[(size_t)k * g.N + n]);
      mf = f > mf ? f : mf;
    }
    em[n] = exp_from_field(mf);
    const int mt = n / MROWS, nl = n % MROWS;
    for (int k = 0; k < g.K; ++k) {
      uint16_t d[C::S];
      split_digits<C>(M[(size_t)k * g.N + n], em[n], d);
      const int ks = k / KSTEP, kl = k % KSTEP;
      for (int s = 0; s < C::S; ++s)
        tiles[(((size_t)mt * g.nsteps + ks) * C::S + s) * A_BLOCK + a_index(nl, kl)] = d[s];
    }
  }
  for (int c = 0; c < g.NX; ++c)
    for (int k = 0; k < g.K; ++k) xcol[(size_t)c * g.K + k] = M[(size_t)k * g.N + g.Nmma + c];
}

template <class C>
inline size_t matrix_tile_elems(const Geom& g) {
  return (size_t)g.MT * g.nsteps * C::S * A_BLOCK;
}

template <class C>
inline Geom make_geom(int N, int K, int64_t nlines, int cplx) {
  Geom g;
  g.N = N;
  g.K = K;
  g.cplx = cplx;
  g.nrows = nlines * (1 + cplx);
  g.nsteps = (K + KSTEP - 1) / KSTEP;
  output_split(N, g.MT, g.Nmma, g.NX);
  g.tiles = (g.nrows + C::BN - 1) / C::BN;
  return g;
}

}  // namespace lc
}  // namespace sgpu
