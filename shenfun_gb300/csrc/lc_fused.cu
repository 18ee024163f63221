// The fused split-BF16 line contraction (lc_fused.cuh has the scheme), two
// kernels per pass:
//
// k_lc_scales   one warp per line, lines visited last to first: the line's
//               power-of-two scale (4 bytes of scratch per line).  Visiting
//               the lines backwards leaves the first ones in L2 for the
//               contraction, which starts with them.
// k_lc_fused    persistent, one CTA per SM, 20 warps.  CTA c computes output
//               rows 128 r .. 128 r + 127 (r = c % MT) of the tiles of 64
//               lines assigned to its group c / MT; the MT CTAs of a group work
//               on the same tiles at about the same time, so the second read of
//               a tile's lines hits L2.  Roles:
//   warp 0        lane 0 streams the CTA's matrix digits (one bulk copy of
//                 S x 4 KB per K step, L2-resident) through an RA-deep ring;
//                 the warp owns the TMEM allocation
//   warp 1        lane 0 issues the MMAs: per K step and matrix digit s one
//                 MMA (or two, past 256 columns) against the line digits of
//                 t = 0 .. S-1-s side by side, into accumulator groups s..S-1
//   warps 2..11   digits: 8-entry pieces of the lines -> S digit rows in the
//                 B ring, K step by K step (the next piece's loads in flight
//                 while the current one is split); a thread keeps to one line,
//                 so it also accumulates that line's FP64 dot products for the
//                 outputs past the last 128-row tile (lines split between the
//                 MT CTAs by whole warps)
//   warps 12..19  epilogue: TMEM -> registers -> integer combine -> FP64
//                 outputs (lane = output index, so a warp's stores for one line
//                 are 256 contiguous bytes), and the dot-product outputs
// All synchronisation is CTA-local (mbarriers, named barriers).  Every wait
// is bounded: a wait that gives up sets the CTA's abort flag and the launch's
// error word, the roles leave their loops at uniform points, and the copies
// and MMAs in flight are waited for before the CTA exits.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <mutex>
#include <new>
#include <vector>

#include "lc_fused.cuh"
#include "lc_fused.h"

using namespace sgpu;
using namespace sgpu::lc;

// bounded waits of this kernel that gave up (added to the other tensor-core
// kernels' count by sgpu_wait_timeouts)
__device__ unsigned int g_lc_timeouts = 0;

namespace {

const int THREADS = 640;
const int DIGIT_W0 = 2, NDIGIT = 10;  // digit warps 2..11
const int EPI_W0 = 12, NEPI = 8;     // epilogue warps 12..19
static_assert(NEPI % 4 == 0 && EPI_W0 == DIGIT_W0 + NDIGIT && THREADS == 32 * (EPI_W0 + NEPI), "warp roles");
const int RA = 4;                    // matrix-digit ring stages
const uint64_t DRAIN_NS = 2000000000ull;  // limit of waits for work already issued
const uint32_t BAR_DIGIT = 1;             // named barrier of the digit warps
const int KW = (CfgWide::KMAX + 31) / 32;  // loads per lane of one line (scales)
const uint32_t NAP_NS = 200;                  // probe spacing of long waits

template <class C>
struct Roles {
  static const int NPART = NDIGIT * 32 / C::BN;  // digit threads per line (dot-product partials)
  static_assert((2 * C::BN) % 32 == 0, "a digit warp's pieces belong to one K step");
  static_assert((NDIGIT * 32) % C::BN == 0, "a digit thread keeps to one line");
};

template <class C>
struct Smem {
  static const int RB = 6;  // line-digit ring stages
  static const size_t a_off = 0;
  static const size_t b_off = a_off + (size_t)RA * C::A_STAGE;
  static const size_t x_off = b_off + (size_t)RB * C::B_STAGE;  // double [2][NPART][BN][MAX_NX]
  static const size_t bar_off = x_off + (size_t)2 * Roles<C>::NPART * C::BN * MAX_NX * 8;
  // a_full, a_empty [RA], b_full, b_empty [RB], tfull, tempty, x_full,
  // x_free [2], mdone, then the TMEM address and the abort flag
  static const int NBARS = 2 * RA + 2 * RB + 8 + 1;
  static const size_t end = bar_off + (size_t)NBARS * 8 + 16;
  static const size_t bytes = end + 1024;  // alignment slack
};
static_assert(Smem<CfgWide>::bytes <= 232448, "shared memory");
static_assert(Smem<CfgNarrow>::bytes <= 232448, "shared memory");
// the digit threads of one round write the pieces of NDIGIT * 32 / (2 BN) K
// steps; with more than RB - 1 of them in flight, a thread checking a stage's
// previous use could see the parity of the use before that and overwrite
// digits an MMA still reads
static_assert(NDIGIT * 32 <= (Smem<CfgWide>::RB - 1) * 2 * CfgWide::BN &&
                  NDIGIT * 32 <= (Smem<CfgNarrow>::RB - 1) * 2 * CfgNarrow::BN,
              "digit rounds span fewer K steps than the ring has stages");

__device__ __forceinline__ void set_abort(volatile int* flag) { *flag = 1; }

__global__ void __launch_bounds__(256) k_lc_scales(const double* __restrict__ in, Geom g, int* __restrict__ eg) {
  const int lane = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= g.nrows) return;
  const int64_t row = g.nrows - 1 - w;
  const double* src = in + row_base(g, row);
  const int ksd = kstride(g);
  double x[KW];
#pragma unroll
  for (int j = 0; j < KW; ++j) {
    const int k = lane + 32 * j;
    x[j] = k < g.K ? src[(int64_t)k * ksd] : 0.0;
  }
  uint32_t mf = 0;
#pragma unroll
  for (int j = 0; j < KW; ++j) {
    const uint32_t f = exp_field(x[j]);
    mf = f > mf ? f : mf;
  }
  mf = __reduce_max_sync(0xffffffffu, mf);
  if (lane == 0) eg[row] = exp_from_field(mf);
}

template <class C>
__global__ void __launch_bounds__(THREADS, 1)
    k_lc_fused(const double* __restrict__ in, double* __restrict__ out, const uint16_t* __restrict__ At,
               const int* __restrict__ em, const int* __restrict__ eg, const double* __restrict__ xcol, Geom g,
               int* err, uint64_t wait_ns) {
  constexpr int S = C::S, BN = C::BN, NBUF = C::NBUF, RB = Smem<C>::RB, NPART = Roles<C>::NPART;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* a_ring = smem + Smem<C>::a_off;
  uint8_t* b_ring = smem + Smem<C>::b_off;
  uint64_t* bars = (uint64_t*)(smem + Smem<C>::bar_off);
  uint64_t* a_full = bars;
  uint64_t* a_empty = a_full + RA;
  uint64_t* b_full = a_empty + RA;
  uint64_t* b_empty = b_full + RB;
  uint64_t* tfull = b_empty + RB;
  uint64_t* tempty = tfull + 2;
  uint64_t* x_full = tempty + 2;  // [2] dot-product partials of a tile written
  uint64_t* x_free = x_full + 2;  // [2] ... read by the epilogue
  uint64_t* mdone = x_free + 2;
  double* xpart = (double*)(smem + Smem<C>::x_off);
  uint32_t* tmem_holder = (uint32_t*)(mdone + 1);
  volatile int* s_abort = (volatile int*)(tmem_holder + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int MT = g.MT;
  const int rank = (int)(blockIdx.x % (unsigned)MT);
  const int64_t grp = blockIdx.x / MT, ngrp = gridDim.x / MT;

  if (threadIdx.x == 0) {
    for (int i = 0; i < RA; ++i) {
      tc::mbar_init(&a_full[i], 1);
      tc::mbar_init(&a_empty[i], 1);
    }
    for (int i = 0; i < RB; ++i) {
      tc::mbar_init(&b_full[i], 2 * BN);  // every (line, K half) piece of the step
      tc::mbar_init(&b_empty[i], 1);      // the MMA commit
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&tfull[i], 1);
      tc::mbar_init(&tempty[i], NEPI);
      tc::mbar_init(&x_full[i], 1);
      tc::mbar_init(&x_free[i], NEPI);
    }
    tc::mbar_init(mdone, 1);
    *s_abort = 0;
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tmem_holder, 512);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_holder;
  bool ok = true;
  const int ksd = kstride(g);

  if (warp == 0) {
    if (lane == 0) {
      // producer: matrix digits of this CTA's 128 outputs, K step by K step
      int64_t q = 0;
      const uint8_t* Ab = (const uint8_t*)At + (size_t)rank * g.nsteps * C::A_STAGE;
      for (int64_t T = grp; T < g.tiles && ok; T += ngrp) {
        for (int ks = 0; ks < g.nsteps; ++ks, ++q) {
          const int st = (int)(q % RA);
          if (q >= RA && !tc::mbar_wait_try(&a_empty[st], (uint32_t)((q / RA) - 1) & 1u, wait_ns)) {
            ok = false;
            break;
          }
          tc::mbar_arrive_expect_tx(&a_full[st], (uint32_t)C::A_STAGE);
          tc::bulk_g2s(a_ring + (size_t)st * C::A_STAGE, Ab + (size_t)ks * C::A_STAGE, (uint32_t)C::A_STAGE,
                       &a_full[st]);
        }
        if (*s_abort) ok = false;
      }
      // every copy issued must land before the CTA may exit
      for (int64_t r = q - RA; r < q; ++r) {
        if (r < 0) continue;
        if (!tc::mbar_wait_try(&a_full[r % RA], (uint32_t)(r / RA) & 1u, DRAIN_NS)) ok = false;
      }
      if (!ok) set_abort(s_abort);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer
      int64_t qa = 0, qb = 0, i = 0;
      for (int64_t T = grp; T < g.tiles && ok; T += ngrp, ++i) {
        const int b = (int)(i % NBUF);
        const int64_t use = i / NBUF;
        if (use >= 1 && !tc::mbar_wait_try(&tempty[b], (uint32_t)(use - 1) & 1u, wait_ns)) {
          ok = false;
          break;
        }
        tc::fence_after_sync();
        const uint32_t dbase = tmem + (uint32_t)(b * S * BN);
        for (int ks = 0; ks < g.nsteps; ++ks, ++qa, ++qb) {
          const int sa = (int)(qa % RA), sb = (int)(qb % RB);
          if (!tc::mbar_wait_try(&a_full[sa], (uint32_t)(qa / RA) & 1u, wait_ns) ||
              !tc::mbar_wait_try(&b_full[sb], (uint32_t)(qb / RB) & 1u, wait_ns)) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint32_t a0 = tc::smem_u32(a_ring + (size_t)sa * C::A_STAGE);
          const uint32_t b0 = tc::smem_u32(b_ring + (size_t)sb * C::B_STAGE);
#pragma unroll
          for (int s = 0; s < S; ++s) {
            const uint64_t ad = tc::sdesc_interleave(a0 + (uint32_t)(s * A_BLOCK * 2), LBO_A, SBO);
            const int rows = (S - s) * BN;
#pragma unroll
            for (int c0 = 0; c0 < rows; c0 += 256) {
              const int n = rows - c0 < 256 ? rows - c0 : 256;
              const uint64_t bd = tc::sdesc_interleave(b0 + (uint32_t)(c0 * 16), C::LBO_B, SBO);
              tc::mma_f16(dbase + (uint32_t)(s * BN + c0), ad, bd, tc::idesc_bf16_f32(MROWS, n),
                          (ks > 0 || s > 0) ? 1u : 0u);
            }
          }
          tc::mma_commit(&a_empty[sa]);
          tc::mma_commit(&b_empty[sb]);
        }
        tc::mma_commit(&tfull[b]);  // also after an early exit: the epilogue must not wait in vain
        if (*s_abort) ok = false;
      }
      tc::mma_commit(mdone);
      if (!ok) set_abort(s_abort);
    }
  } else if (warp < DIGIT_W0 + NDIGIT) {
    // digit warps: pieces (K step, K half h, line jj), line fastest, so that a
    // warp's 32 pieces share one K step and its 16-byte stores are contiguous.
    // Loop exits are decided by a vote at their named barrier.
    const int ts = threadIdx.x - DIGIT_W0 * 32;
    const int per = 2 * BN;
    // this thread's line within every tile, its share of the dot products
    const int my_jj = ts % BN, part = ts / BN;
    const bool dots = g.NX > 0 && (my_jj / 32) % MT == rank;
    bool bad = false;
    int64_t qb0 = 0, i = 0;
    auto load = [&](int it, int64_t row0, double (&x)[8]) {
      const int ks = it / per, rem = it - ks * per;
      const int h = rem / BN, jj = rem - h * BN;
      const int64_t row = row0 + jj;
      const int k0 = ks * KSTEP + h * 8;
      if (row < g.nrows) {
        const double* src = in + row_base(g, row);
#pragma unroll
        for (int qq = 0; qq < 8; ++qq) x[qq] = k0 + qq < g.K ? src[(int64_t)(k0 + qq) * ksd] : 0.0;
      } else {
#pragma unroll
        for (int qq = 0; qq < 8; ++qq) x[qq] = 0.0;
      }
    };
    for (int64_t T = grp; T < g.tiles; T += ngrp, ++i) {
      const int64_t row0 = T * BN;
      const int total = g.nsteps * per;
      double acc[MAX_NX] = {0.0, 0.0};
      double xn[8];
      if (ts < total) load(ts, row0, xn);
      for (int base = 0; base < total; base += NDIGIT * 32) {
        const int it = base + ts;
        const bool act = it < total && !bad;
        double x[8];
#pragma unroll
        for (int qq = 0; qq < 8; ++qq) x[qq] = xn[qq];
        if (it + NDIGIT * 32 < total) load(it + NDIGIT * 32, row0, xn);  // the next piece in flight
        const int ks = it / per, rem = it - ks * per;
        const int h = rem / BN, jj = rem - h * BN;
        const int64_t q = qb0 + ks;
        const int st = (int)(q % RB);
        bool wrote = false;
        if (act && dots) {
          const int k0 = ks * KSTEP + h * 8;
#pragma unroll
          for (int c = 0; c < MAX_NX; ++c)
            if (c < g.NX)
#pragma unroll
              for (int qq = 0; qq < 8; ++qq)
                if (k0 + qq < g.K) acc[c] = fma(x[qq], __ldg(xcol + (size_t)c * g.K + k0 + qq), acc[c]);
        }
        if (act) {
          if (q >= RB && !tc::mbar_wait_try_nap(&b_empty[st], (uint32_t)((q / RB) - 1) & 1u, wait_ns, 64)) {
            bad = true;
          } else {
            const int64_t row = row0 + jj;
            const int e = row < g.nrows ? __ldg(eg + row) : 0;
            uint4 dg[S];
            split8<C>(x, e, dg);
            uint8_t* bst = b_ring + (size_t)st * C::B_STAGE;
#pragma unroll
            for (int t = 0; t < S; ++t) *reinterpret_cast<uint4*>(bst + b_offset<C>(t, jj, h)) = dg[t];
            wrote = true;
          }
        }
        // the pieces are read by the tensor cores (async proxy)
        tc::fence_proxy_async_shared_cta();
        const uint32_t wmask = __ballot_sync(0xffffffffu, wrote);
        if (lane == 0 && wmask) tc::mbar_arrive_count(&b_full[st], (uint32_t)__popc(wmask));
      }
      qb0 += g.nsteps;
      if (g.NX > 0) {
        // the partials of this tile into slot i % 2, once the epilogue has
        // read that slot's previous tile
        const int xs = (int)(i & 1);
        if (i >= 2 && !tc::mbar_wait_try(&x_free[xs], (uint32_t)((i / 2) - 1) & 1u, wait_ns)) bad = true;
#pragma unroll
        for (int c = 0; c < MAX_NX; ++c) xpart[((xs * NPART + part) * BN + my_jj) * MAX_NX + c] = acc[c];
      }
      if (tc::named_sync_or(BAR_DIGIT, NDIGIT * 32, bad || *s_abort)) break;
      if (g.NX > 0 && ts == 0) tc::mbar_arrive(&x_full[i & 1]);
    }
    if (bad) ok = false;
    // no MMA may still read this CTA's ring when it exits
    if (ts == 0 && ok && !*s_abort) {
      for (int64_t r = qb0 - RB; r < qb0; ++r) {
        if (r < 0) continue;
        if (!tc::mbar_wait_try(&b_empty[r % RB], (uint32_t)(r / RB) & 1u, DRAIN_NS)) ok = false;
      }
    }
    if (!ok) set_abort(s_abort);
  } else {
    // epilogue
    const int quarter = warp & 3, part = (warp - EPI_W0) >> 2;  // part 0 .. NEPI / 4 - 1
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    const int nl = quarter * 32 + lane;
    const int n = rank * MROWS + nl;
    const bool n_ok = n < g.Nmma;
    const int emn = n_ok ? em[n] : 0;
    int64_t i = 0;
    for (int64_t T = grp; T < g.tiles; T += ngrp, ++i) {
      const int b = (int)(i % NBUF);
      const bool mine = tc::mbar_wait_try_nap(&tfull[b], (uint32_t)(i / NBUF) & 1u, wait_ns, NAP_NS) && !*s_abort;
      if (!__all_sync(0xffffffffu, mine)) {  // warp-uniform exit
        ok = false;
        break;
      }
      tc::fence_after_sync();
      const int64_t row0 = T * BN;
      for (int c8 = part; c8 < BN / 8; c8 += NEPI / 4) {
        uint32_t a[S][8];
#pragma unroll
        for (int gg = 0; gg < S; ++gg)
          tc::tmem_ld8(tmem + lane_base + (uint32_t)(b * S * BN + gg * BN + c8 * 8), a[gg]);
        int ex[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int64_t row = row0 + c8 * 8 + j;
          ex[j] = row < g.nrows ? __ldg(eg + row) : 0;
        }
        tc::tmem_ld_wait();
        double v[8];
        combine8<C>(a, ex, emn, v);
        if (n_ok) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int64_t row = row0 + c8 * 8 + j;
            if (row < g.nrows) out[row_base(g, row) + (int64_t)n * ksd] = v[j];
          }
        }
      }
      // the dot-product outputs of this CTA's share of the lines (the tile's
      // lines are all read by now: in-place contractions stay correct)
      if (g.NX > 0) {
        const int xs = (int)(i & 1);
        const bool got = tc::mbar_wait_try(&x_full[xs], (uint32_t)(i / 2) & 1u, wait_ns);
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        if (warp - EPI_W0 < BN / 32) {
          const int jj = (warp - EPI_W0) * 32 + lane;
          const int64_t row = row0 + jj;
          if ((jj / 32) % MT == rank && row < g.nrows)
            for (int c = 0; c < g.NX; ++c) {
              double sum = 0.0;
              for (int p = 0; p < NPART; ++p) sum += xpart[((xs * NPART + p) * BN + jj) * MAX_NX + c];
              out[row_base(g, row) + (int64_t)(g.Nmma + c) * ksd] = sum;
            }
        }
      }
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) {
        tc::mbar_arrive(&tempty[b]);
        if (g.NX > 0) tc::mbar_arrive(&x_free[i & 1]);
      }
    }
    if (!ok) set_abort(s_abort);
  }
  // every MMA must have completed before TMEM is released
  __syncwarp();
  if (warp == 0 && !tc::mbar_wait_try(mdone, 0, DRAIN_NS)) ok = false;
  tc::fence_before_sync();
  __syncthreads();
  if ((!ok && lane == 0) || (*s_abort && threadIdx.x == 0)) {
    atomicAdd(&g_lc_timeouts, 1u);
    if (err) atomicOr(err, 1);
  }
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 512);
  }
}

// per-device launch attributes (the large dynamic shared memory) and SM counts
struct DevState {
  std::once_flag attr[2];
  int attr_rc[2] = {0, 0};
  int nctas[2] = {};  // resident CTAs per device and tile width
};
const int MAX_DEV = 64;
DevState g_dev[MAX_DEV];

template <class C>
int cfg_index() { return C::BN == 64 ? 0 : 1; }

template <class C>
int prepare(int dev, int& nctas) {
  DevState& d = g_dev[dev];
  const int ci = cfg_index<C>();
  std::call_once(d.attr[ci], [&]() {
    d.attr_rc[ci] = cudaFuncSetAttribute(k_lc_fused<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)Smem<C>::bytes) == cudaSuccess
                        ? 1
                        : -1;
    cudaGetLastError();
  });
  if (d.attr_rc[ci] != 1) return SGPU_ERR_CUDA;
  int n = __atomic_load_n(&d.nctas[ci], __ATOMIC_ACQUIRE);
  if (n <= 0) {
    int per_sm = 0, nsm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lc_fused<C>, THREADS, Smem<C>::bytes) != cudaSuccess ||
        per_sm <= 0)
      per_sm = 1;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0) nsm = 1;
    cudaGetLastError();
    n = per_sm * nsm;
    __atomic_store_n(&d.nctas[ci], n, __ATOMIC_RELEASE);
  }
  nctas = n;
  return SGPU_OK;
}

template <class C>
int launch(const Matrix& m, const double* in, double* out, int64_t nlines, int cplx, void* work, size_t work_bytes,
           int* err, uint64_t wait_ns, cudaStream_t stream) {
  const Geom g = make_geom<C>(m.N, m.K, nlines, cplx);
  if (g.MT != m.MT || g.Nmma != m.Nmma || g.NX != m.NX) return SGPU_ERR_ARG;
  if (g.tiles == 0) return SGPU_OK;
  if (!work || work_bytes < workspace_bytes(m, nlines, cplx) || ((uintptr_t)work & 255)) return SGPU_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return SGPU_ERR_CUDA;
  }
  if (dev < 0 || dev >= MAX_DEV) return SGPU_ERR_UNSUPPORTED;
  int nctas = 0;
  int st = prepare<C>(dev, nctas);
  if (st != SGPU_OK) return st;
  int* eg = (int*)work;
  const int64_t sblocks = (g.nrows + 7) / 8;
  if (sblocks > 0x7fffffffLL) return SGPU_ERR_ARG;
  k_lc_scales<<<(unsigned)sblocks, 256, 0, stream>>>(in, g, eg);
  // groups of MT CTAs (one per 128 outputs) share a tile sequence
  const int64_t ngrp = std::max<int64_t>(1, std::min<int64_t>(nctas / g.MT, g.tiles));
  k_lc_fused<C><<<(unsigned)(ngrp * g.MT), THREADS, Smem<C>::bytes, stream>>>(
      in, out, (const uint16_t*)m.tiles, (const int*)m.em, eg, (const double*)m.xcol, g, err, wait_ns);
  if (cudaGetLastError() != cudaSuccess) return SGPU_ERR_CUDA;
  return SGPU_OK;
}

}  // namespace

namespace sgpu {
namespace lc {

bool supported(int N, int K) { return supported_nk(N, K); }

int matrix_create(const double* M, int N, int K, Matrix* out) {
  if (!out || !M) return SGPU_ERR_ARG;
  if (!supported_nk(N, K)) return SGPU_ERR_UNSUPPORTED;
  typedef CfgWide C;  // both tile widths share the matrix layout
  const Geom g = make_geom<C>(N, K, 0, 0);
  std::vector<uint16_t> tiles(matrix_tile_elems<C>(g));
  std::vector<int> em((size_t)g.MT * MROWS);
  std::vector<double> xcol((size_t)std::max(1, g.NX) * K);
  split_matrix_host<C>(M, g, tiles.data(), em.data(), xcol.data());
  const size_t tb = tiles.size() * 2, eb = em.size() * 4, xb = xcol.size() * 8;
  const size_t eo = (tb + 255) & ~(size_t)255, xo = (eo + eb + 255) & ~(size_t)255;
  void* dev = nullptr;
  if (cudaMalloc(&dev, xo + xb) != cudaSuccess) {
    cudaGetLastError();
    return SGPU_ERR_NOMEM;
  }
  if (cudaMemcpy(dev, tiles.data(), tb, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy((char*)dev + eo, em.data(), eb, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy((char*)dev + xo, xcol.data(), xb, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(dev);
    cudaGetLastError();
    return SGPU_ERR_CUDA;
  }
  out->N = N;
  out->K = K;
  out->MT = g.MT;
  out->Nmma = g.Nmma;
  out->NX = g.NX;
  out->tiles = (uint16_t*)dev;
  out->em = (int*)((char*)dev + eo);
  out->xcol = (double*)((char*)dev + xo);
  return SGPU_OK;
}

void matrix_destroy(Matrix* m) {
  if (m && m->tiles) cudaFree(m->tiles);
  if (m) m->tiles = nullptr;
}

// pipeline-wait limit of the fused kernel (0: one second); a test sets a
// short one to make the waits run out
std::atomic<unsigned long long> g_wait_limit_ns{0};

int read_timeouts(unsigned int* count) {
  return cudaMemcpyFromSymbol(count, g_lc_timeouts, sizeof(unsigned int)) == cudaSuccess ? SGPU_OK : SGPU_ERR_CUDA;
}

size_t workspace_bytes(const Matrix& m, int64_t nlines, int cplx) {
  (void)m;
  const size_t nrows = (size_t)nlines * (1 + cplx);
  return (nrows * 4 + 255) & ~(size_t)255;
}

int contract(const Matrix& m, const double* in, double* out, int64_t nlines, int cplx, void* work, size_t work_bytes,
             int* err, uint64_t wait_ns, cudaStream_t stream) {
  if (nlines == 0) return SGPU_OK;
  if (!m.tiles || !in || !out || nlines < 0) return SGPU_ERR_ARG;
  if ((((uintptr_t)in) & 7) || (((uintptr_t)out) & 7)) return SGPU_ERR_ARG;
  if (wait_ns == 0) wait_ns = g_wait_limit_ns.load(std::memory_order_relaxed);
  if (wait_ns == 0) wait_ns = 1000000000ull;
  return m.variant == 2 ? launch<CfgNarrow>(m, in, out, nlines, cplx, work, work_bytes, err, wait_ns, stream)
                        : launch<CfgWide>(m, in, out, nlines, cplx, work, work_bytes, err, wait_ns, stream);
}

}  // namespace lc
}  // namespace sgpu

extern "C" int sgpu_set_wait_limit_ns(unsigned long long ns) {
  sgpu::lc::g_wait_limit_ns.store(ns, std::memory_order_relaxed);
  return SGPU_OK;
}
