// Dense FP64 line contractions on the BF16 tensor cores (tcgen05), exact to
// about 42 bits, by splitting both operands into BF16 "digit" slices
// (the Ozaki scheme: Ozaki, Ogita, Oishi & Rump, Numer. Algorithms 59, 2012;
// on FP16/BF16 tensor cores: Ootomo & Yokota, IJHPCA 2022).
//
//   out(l, n) = sum_k A(l, k) B(k, n)       A: lines x K (FP64), B: K x Nout
//
// Each row of A (and each column of B) is scaled by a power of two 2^e with
// |x| < 2^{e-1} (one bit of headroom) and rounded to a W*S-bit fixed-point
// integer X < 2^{WS-1}, which is cut into S balanced digits:
// X = sum_s d_s 2^{W(S-1-s)},  |d_s| <= 2^{W-1}.  Slice s stores d_s 2^{-W s}
// in BF16 (exact: at most 8 significant bits).  Then
//   A B = 2^{eA+eB-2W} sum_{s,t} A_s B_t,
// and the products with s + t <= S - 1 are kept (W = 7, S = 7: 28 products,
// 48 bits).  The tensor core sums them into five FP32 accumulators in TMEM:
// G0 (s+t=0), G1, G2, G3 and G4 (s+t>=4).  Group g holds multiples of
// 2^{-W g} of magnitude at most (g+1) 2^{2W-2} K units, below 2^24 for
// g <= 3 when K <= 2^{26-2W}/4 (W=7: K <= 1024), so those FP32 sums are
// exact (longer contractions run in chunks of 1024 whose FP64 results are
// added); G4 carries terms below 2^{-4W} relative, where FP32 rounding is
// harmless (a fourth exact group lowers the error ~50x against folding
// s+t=3 into the rounded one).  The
// epilogue adds the four in 64-bit fixed point with integer instructions and
// assembles the FP64 result bit by bit (the FP64 pipe is ~1/64 of FP32 on
// this part, so no FP64 arithmetic runs per element).
//
// Data layout: the split slices are written pre-tiled in the tensor core's
// canonical no-swizzle K-major layout, one block per (slice, row tile,
// 32-wide K block): [kgroup 4][rowgroup][row 8][8 elements] (8 KB for the
// 128-row A tiles, 6 KB for the 96-row B tiles).  A pipeline stage is then
// 2S plain bulk copies (cp.async.bulk).
#pragma once

#include <cmath>
#include <cstring>

#include "sgpu_common.cuh"
#include "tc_ptx.cuh"

namespace sgpu {
namespace oz {

const int BM = 128;       // rows (lines) per tile = MMA M
const int BK = 32;        // K per split block (the pre-tiled layout)
const int STAGES = 4;     // pipeline stages of 16 K each (half a split block)
const int W = 7;          // bits per digit
const int A_ELEMS = BM * BK;            // 4096 bf16 = 8 KB per A slice block
const int A_BYTES = A_ELEMS * 2;
const int LBO_A = BM * 16;              // K-direction core-matrix stride (bytes)
const int SBO = 128;                    // row-direction core-matrix stride (bytes)

// A digit configuration: S digits per operand, products with s + t <= S - 1,
// NACC FP32 accumulators (groups 0..NACC-2 separately, the rest combined) and
// BN output columns per tile (NACC * BN <= 512 TMEM columns).
// NBUF accumulator sets: with two (2 NACC BN <= 512 TMEM columns) the
// epilogue of one tile overlaps the main loop of the next; with one the
// producer still prefetches the next tile's operands during the epilogue.
// Wider tiles read the A operand from shared memory less often per flop
// (measured on the channel grid's z axis: BN = 96 with one set beat BN = 48
// with two).
// ATMEM: the A slices of a K step are copied once into TMEM (tcgen05.cp,
// two buffers of S x 8 columns after the accumulators) and every digit
// product reads A from there; only B is read from shared memory per MMA.
// Measured on the channel grid's z pass: correct, but no faster per MMA
// than both operands in shared memory (~120 cycles per 128 x N x 16 MMA
// including the epilogue's share, N = 64 .. 96): the MMAs are bound by an
// instruction cadence, not by operand reads, and the smaller N it needs
// (TMEM budget) adds tiles.  Both configurations below keep A in shared
// memory; the TMEM variant stays selectable and tested.
template <int S_, int NACC_, int BN_, int ATMEM_ = 0>
struct Cfg {
  static const int S = S_, NACC = NACC_, BN = BN_, ATMEM = ATMEM_;
  static const int ACOLS = ATMEM ? 2 * S * 8 : 0;  // TMEM columns of the A buffers
  static const int NBUF = 2 * NACC * BN + ACOLS <= 512 ? 2 : 1;
  static const int B_ELEMS = BN * BK, B_BYTES = B_ELEMS * 2;
  static const int LBO_B = BN * 16;
  static const int NPROD = S * (S + 1) / 2;
  static_assert(NACC * BN + ACOLS <= 512, "accumulators and A buffers exceed TMEM");
  static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256, "MMA N");
};
// 7 digits (48 bits), 28 products, groups 0..3 exact: normwise ~1e-13
typedef Cfg<7, 5, 96> CfgStd;
// 8 digits (55 bits), 36 products, groups 0..4 exact: normwise ~1e-15, for
// contractions whose result a later step amplifies (the Chebyshev Dirichlet
// Helmholtz recurrence magnifies input perturbations up to ~4000x at large
// shifts, so its mixed form needs FP64-level transforms)
typedef Cfg<8, 6, 80> CfgPrec;
// the TMEM-A variant of CfgPrec (BN = 64: 6 x 64 accumulator + 2 x 64 A columns)
typedef Cfg<8, 6, 64, 1> CfgPrecTmemA;

// index of element (row r, k in the K block) inside a block of `rows` rows:
// [k / 8][r / 8][r % 8][k % 8]
SGPU_HD int tile_index(int rows, int r, int k) {
  return (k >> 3) * rows * 8 + (r >> 3) * 64 + (r & 7) * 8 + (k & 7);
}

// exponent of a row/column: e with max|x| < 2^{e-1} (one bit of headroom),
// from the largest biased exponent field (0 for an all-zero or all-subnormal
// line)
SGPU_HD int exp_from_field(uint32_t maxfield) { return maxfield ? (int)maxfield - 1021 : 0; }

SGPU_HD uint32_t exp_field(double x) {
  uint64_t b;
  memcpy(&b, &x, 8);
  return (uint32_t)((b >> 52) & 0x7ff);
}

// balanced digits of x (|x| < 2^{e-1}) at W*S bits: BF16 bit patterns of
// d_s 2^{-W s}.  Integer arithmetic (and exact FP32 adds) only: the W-bit
// fields of the fixed-point magnitude X are read off with shifts, then made
// balanced from the least significant end (a field >= 2^{W-1} becomes
// field - 2^W with a carry into the next one), which gives the unique
// representation with d_s in [-2^{W-1}, 2^{W-1}) for s >= 1.
template <int W, int S>
SGPU_HD void split_digits(double x, int e, uint16_t (&out)[S]) {
  static_assert(W * S <= 60, "fixed point beyond 64 bits");
  uint64_t b;
  memcpy(&b, &x, 8);
  const int field = (int)((b >> 52) & 0x7ff);
  uint64_t X = 0;
  if (field != 0) {
    const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    // X = round(|x| 2^{WS-e}) = round(m 2^{-sh}); sh >= 54 - W*S since
    // |x| < 2^{e-1} (> 0 for 7 digits, >= -2 for 8), and X < 2^{WS-1}
    const int sh = 1075 + e - W * S - field;
    if (sh <= 0)
      X = m << (-sh);
    else if (sh < 64)
      X = (m + (1ull << (sh - 1))) >> sh;
  }
  int d[S];
  int carry = 0;
#pragma unroll
  for (int s = S - 1; s >= 0; --s) {
    int u = (int)((uint32_t)(X >> (W * (S - 1 - s))) & ((1u << W) - 1)) + carry;
    if (s > 0) {
      carry = u >= (1 << (W - 1)) ? 1 : 0;
      u -= carry << W;
    }
    d[s] = u;
  }
  const uint32_t sign = (uint32_t)(b >> 63);
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const int v = sign ? -d[s] : d[s];
    // exact float of v (|v| <= 2^W) by the 1.5 * 2^23 bias, scaled by 2^{-W s};
    // its top 16 bits are the BF16 value
    const uint32_t biased = 0x4B400000u + (uint32_t)v;
    float f;
    memcpy(&f, &biased, 4);
    f -= 12582912.0f;
    const uint32_t pb = (uint32_t)(127 - W * s) << 23;  // 2^{-W s}
    float p;
    memcpy(&p, &pb, 4);
    f *= p;
    uint32_t fb;
    memcpy(&fb, &f, 4);
    out[s] = (uint16_t)(fb >> 16);
  }
}

// round(v * 2^sh) for an FP32 v, as int64, integer instructions only
// (FP32 subnormals count as zero)
SGPU_HD int64_t f32_fixed(uint32_t b, int sh) {
  const int ex = (int)((b >> 23) & 0xff);
  if (ex == 0) return 0;
  const int64_t m = (int64_t)((b & 0x7fffffu) | 0x800000u);
  const int e = ex - 150 + sh;  // v 2^sh = m 2^e
  int64_t r;
  if (e >= 0)
    r = e < 39 ? (m << e) : 0;  // callers keep |v 2^sh| < 2^62
  else if (e > -40)
    r = (m + ((int64_t)1 << (-e - 1))) >> (-e);
  else
    r = 0;
  return (b >> 31) ? -r : r;
}

// T * 2^E as an FP64 bit pattern, round to nearest even; integer instructions
// except for results outside the normal range (rare, handled with ldexp)
SGPU_HD double fixed_to_double(int64_t T, int E) {
  if (T == 0) return 0.0;
  const uint64_t sign = T < 0 ? (1ull << 63) : 0;
  const uint64_t a = T < 0 ? (uint64_t)(-T) : (uint64_t)T;
#if defined(__CUDA_ARCH__)
  const int msb = 63 - __clzll((long long)a);
#else
  const int msb = 63 - __builtin_clzll(a);
#endif
  uint64_t mant;
  int e2;
  if (msb > 52) {
    const int s = msb - 52;
    const uint64_t rem = a & ((1ull << s) - 1), half = 1ull << (s - 1);
    mant = a >> s;
    if (rem > half || (rem == half && (mant & 1))) ++mant;
    e2 = s;
    if (mant >> 53) {
      mant >>= 1;
      ++e2;
    }
  } else {
    mant = a << (52 - msb);
    e2 = msb - 52;
  }
  const int biased = e2 + E + 52 + 1023;
  if (biased <= 0 || biased >= 2047) {
    const double v = ldexp((double)mant, e2 + E);
    return sign ? -v : v;
  }
  const uint64_t bits = sign | ((uint64_t)biased << 52) | (mant & 0xFFFFFFFFFFFFFull);
  double r;
  memcpy(&r, &bits, 8);
  return r;
}

// FP32 -> int32, round to nearest (exact for the integer-valued sums)
SGPU_HD int32_t f2i_rn(float v) {
#if defined(__CUDA_ARCH__)
  return __float2int_rn(v);
#else
  return (int32_t)lrintf(v);
#endif
}

// one output element from the NACC FP32 accumulators (bit patterns) of digit
// groups 0..NACC-2 (exact: G_g 2^{Wg} are integers below 2^24 in magnitude)
// and >= NACC-1 (rounded); E = eA + eB - 2W.  The groups are added in 64-bit
// fixed point T = sum_g G_g 2^F (F = 33 for five accumulators, 36 for six,
// both keeping |T| < 2^63 for K <= 1024 and resolving the last exact group),
// and T 2^{E-F} is assembled as FP64 bits.
template <int NACC>
SGPU_HD double combine_groups(const uint32_t (&gb)[NACC], int E) {
  static_assert((NACC == 5 || NACC == 6) && W == 7, "five or six accumulators of 7-bit digits");
  constexpr int F = NACC == 5 ? 33 : 36;
  float g[NACC];
  for (int i = 0; i < NACC; ++i) memcpy(&g[i], &gb[i], 4);
  int64_t T = f2i_rn(g[0]);
  float sc = 1.0f;
  for (int i = 1; i < NACC - 1; ++i) {
    sc *= 128.0f;
    T = T * 128 + f2i_rn(g[i] * sc);
  }
  // the rounded group at 2^-F: T so far is in units of 2^{-7 (NACC-2)}
  constexpr int rest = F - 7 * (NACC - 2);
  const uint32_t fb = (uint32_t)(127 + F) << 23;  // 2^F
  float pF;
  memcpy(&pF, &fb, 4);
  T = T * ((int64_t)1 << rest) + f2i_rn(g[NACC - 1] * pF);
  return fixed_to_double(T, E - F);
}

// geometry of one contraction over lines of a (outer, N, inner) array:
// rows are lines (complex lines give two rows: real and imaginary parts)
struct Geom {
  int64_t nrows;   // rows of A (lines x (1 + cplx))
  int64_t inner;
  int N;           // line length (= Nout, and the K extent of the tiles)
  int K;           // leading input entries the matrix uses (its other rows are zero)
  int cplx;
  int nkb;         // K blocks of BK the contraction runs over: the K active
                   // input entries, padded (the A slices hold these blocks)
  int nkb_b;       // K blocks of the matrix tiles: all N rows, padded
  int mtiles;      // row tiles of BM
  int ntiles;      // output-column tiles of BN
  // one GEMM launch sums the K blocks [kb0, kb1): at most KCHUNK_MAX blocks,
  // so that its FP32 group sums stay exact; a launch with accum adds its
  // FP64 result to the output of the previous chunks
  int kb0, kb1, accum;
  int kchunk;      // K blocks per launch (KCHUNK_MAX; smaller in tests)
};

// K blocks per GEMM launch: 1024 / BK (the exactness bound K <= 1024 above)
constexpr int KCHUNK_MAX = 1024 / 32;
// largest contraction length: K chunks of 1024, each exact, added in FP64
constexpr int OZ_MAX_K = 8192;

SGPU_HD int64_t row_offset(const Geom& g, int64_t row, int64_t j) {
  const int64_t l = g.cplx ? (row >> 1) : row;
  const int64_t part = g.cplx ? (row & 1) : 0;
  const int64_t o = l / g.inner, i = l - o * g.inner;
  const int64_t e = (o * g.N + j) * g.inner + i;
  return g.cplx ? 2 * e + part : e;
}

// bytes of the split operand A (slices + row exponents) for a geometry
inline size_t a_split_bytes(const Geom& g, int S) {
  return (size_t)S * g.mtiles * g.nkb * A_BYTES + (size_t)g.mtiles * BM * sizeof(int);
}

inline Geom make_geom(int N, int64_t nlines, int64_t inner, int cplx, int BN, int K) {
  Geom g;
  g.N = N;
  g.K = K;
  g.inner = inner;
  g.cplx = cplx;
  g.nrows = nlines * (1 + cplx);
  // rows >= K of the matrix are zero: their input entries need no slices and
  // their K steps no MMAs (a backward transform skips the boundary dofs)
  g.nkb = ((K > 0 ? K : 1) + BK - 1) / BK;
  g.nkb_b = (N + BK - 1) / BK;
  g.mtiles = (int)((g.nrows + BM - 1) / BM);
  g.ntiles = (N + BN - 1) / BN;
  g.kb0 = 0;
  g.kb1 = g.nkb;
  g.accum = 0;
  g.kchunk = KCHUNK_MAX;
  return g;
}

// the launch of chunk c: K blocks [c kchunk, min(nkb, (c+1) kchunk))
inline Geom chunk_geom(const Geom& g, int c) {
  Geom h = g;
  h.kb0 = c * g.kchunk;
  h.kb1 = h.kb0 + g.kchunk < g.nkb ? h.kb0 + g.kchunk : g.nkb;
  h.accum = c > 0;
  return h;
}
inline int num_chunks(const Geom& g) { return (g.nkb + g.kchunk - 1) / g.kchunk; }

// MMA K steps (16 wide) of one launch: the chunk's blocks, cut at the last
// active entry K; at least one (a zero contraction still initialises the
// accumulators)
SGPU_HD int oz_steps(const Geom& g) {
  const int kend = g.kb1 * BK < g.K ? g.kb1 * BK : g.K;
  const int n = (kend - g.kb0 * BK + 15) / 16;
  return n < 1 ? 1 : n;
}

// largest exponent field of row `row` over the lanes' strided share
// (lane, lane + nlane, ...) of the K entries the matrix uses (entries it
// ignores, such as the boundary dofs a backward transform skips, must not
// set the scale); rows past nrows give 0
SGPU_HD uint32_t rowexp_partial(const double* in, const Geom& g, int64_t row, int lane, int nlane) {
  uint32_t mf = 0;
  if (row < g.nrows)
    for (int j = lane; j < g.K; j += nlane) {
      const uint32_t f = exp_field(in[row_offset(g, row, j)]);
      mf = f > mf ? f : mf;
    }
  return mf;
}

// split block (mt, kb): the 128 x 32 input block of row tile mt and K block
// kb -> S slice blocks of 8 KB.  Phase 1: each work item is one row and eight
// consecutive k (one 16-byte core-matrix row per slice); it loads its eight
// inputs first (independent loads in flight), splits them and stores 16 bytes
// per slice to shared memory in the tiled order.  Items are numbered so that
// global reads coalesce: a warp covers whole 256-byte line segments for
// contiguous lines, consecutive lines otherwise.  Phase 2 copies the S blocks
// out with 16-byte stores.  smem: S * A_BYTES bytes, 16-byte aligned.
template <int S>
SGPU_HD void split_block(const double* in, const int* eA, uint16_t* At, const Geom& g, int mt, int kb,
                         void* smem, int tid, int nth) {
  uint16_t* sm = (uint16_t*)smem;
  const int nitem = BM * (BK / 8);
  for (int it = tid; it < nitem; it += nth) {
    // contiguous lines: a warp takes 8 rows x 4 chunks (each row's 256 bytes
    // read together), lanes 8j..8j+7 on 8 different rows so that their
    // 16-byte shared stores hit different banks
    const int r = g.inner == 1 ? 8 * (it >> 5) + (it & 7) : it % BM;
    const int kc = g.inner == 1 ? (it >> 3) & 3 : it / BM;
    const int64_t row = (int64_t)mt * BM + r;
    const int k0 = kb * BK + kc * 8;
    double x[8];
    if (row < g.nrows) {
      const int64_t base = row_offset(g, row, 0);
      const int64_t st = g.inner * (g.cplx ? 2 : 1);
      for (int q = 0; q < 8; ++q) x[q] = k0 + q < g.K ? in[base + (int64_t)(k0 + q) * st] : 0.0;
    } else {
      for (int q = 0; q < 8; ++q) x[q] = 0.0;
    }
    const int e = eA[row];
    uint16_t d[8][S];
    for (int q = 0; q < 8; ++q) split_digits<W, S>(x[q], e, d[q]);
    const int ti = tile_index(BM, r, kc * 8);  // a multiple of 8 elements: 16-byte aligned
    for (int s = 0; s < S; ++s) {
      uint4 v;
      v.x = (uint32_t)d[0][s] | ((uint32_t)d[1][s] << 16);
      v.y = (uint32_t)d[2][s] | ((uint32_t)d[3][s] << 16);
      v.z = (uint32_t)d[4][s] | ((uint32_t)d[5][s] << 16);
      v.w = (uint32_t)d[6][s] | ((uint32_t)d[7][s] << 16);
      *reinterpret_cast<uint4*>(sm + (size_t)s * A_ELEMS + ti) = v;
    }
  }
  SGPU_SYNC();
  const int nvec = S * A_BYTES / 16;
  const uint4* src = reinterpret_cast<const uint4*>(sm);
  for (int v = tid; v < nvec; v += nth) {
    const int s = v / (A_BYTES / 16), off = v % (A_BYTES / 16);
    uint4* dst = reinterpret_cast<uint4*>(At + (((int64_t)s * g.mtiles + mt) * g.nkb + kb) * A_ELEMS) + off;
    *dst = src[v];
  }
}

// host: split column n of a fixed N x N matrix M (out = in . M, so output
// column n is M[:, n]) into the tiled slices [S][ntiles][nkb][BN x BK] and its
// exponent; the tiles start zeroed
template <class C>
void split_matrix_column(const double* M, int N, int n, uint16_t* tiles, int* ex) {
  const int S = C::S, BN = C::BN, B_ELEMS = C::B_ELEMS;
  const int nkb = (N + BK - 1) / BK, ntiles = (N + BN - 1) / BN;
  uint32_t mf = 0;
  for (int k = 0; k < N; ++k) {
    const uint32_t f = exp_field(M[(size_t)k * N + n]);
    mf = f > mf ? f : mf;
  }
  ex[n] = exp_from_field(mf);
  const int nt = n / BN, r = n % BN;
  for (int k = 0; k < N; ++k) {
    uint16_t d[C::S];
    split_digits<W, C::S>(M[(size_t)k * N + n], ex[n], d);
    for (int s = 0; s < S; ++s)
      tiles[(((size_t)s * ntiles + nt) * nkb + k / BK) * B_ELEMS + tile_index(BN, r, k % BK)] = d[s];
  }
}

template <class C>
void split_matrix_host(const double* M, int N, uint16_t* tiles, int* ex) {
  const int nkb = (N + BK - 1) / BK, ntiles = (N + C::BN - 1) / C::BN;
  memset(tiles, 0, sizeof(uint16_t) * (size_t)C::S * ntiles * nkb * C::B_ELEMS);
  memset(ex, 0, sizeof(int) * (size_t)ntiles * C::BN);
  for (int n = 0; n < N; ++n) split_matrix_column<C>(M, N, n, tiles, ex);
}

template <class C>
inline size_t matrix_tile_elems(int N) {
  return (size_t)C::S * ((N + C::BN - 1) / C::BN) * ((N + BK - 1) / BK) * C::B_ELEMS;
}

}  // namespace oz
}  // namespace sgpu
