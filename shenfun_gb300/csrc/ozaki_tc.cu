// Split-BF16 tensor-core contraction along lines (the mixed form of the
// Legendre Vandermonde transforms).  Kernels:
//   k_oz_rowexp   one warp per row: the row's power-of-two scale
//   k_oz_split    one CTA per (128-row tile, 32-wide K block): S digit slices
//                 staged in shared memory, written out pre-tiled (16-byte stores)
//   k_oz_gemm     persistent, one CTA per SM over 128 x BN output tiles: a
//                 producer thread streams 2S slice half blocks per K step with
//                 bulk copies, one thread issues tcgen05.mma for the S(S+1)/2
//                 slice products into NACC TMEM accumulators (two sets where
//                 TMEM holds them, so that the next tile's MMAs overlap this
//                 tile's epilogue), and twelve warps run the integer epilogue
//                 (TMEM -> registers -> FP64 bits -> global).
// The split matrix operand (B) is built once on the host with the same digit
// code and uploaded with the plan.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "lc_fused.h"
#include "ozaki.cuh"
#include "ozaki_tc.h"

using namespace sgpu;
using namespace sgpu::oz;

// count of bounded waits in these kernels that gave up (read by
// sgpu_wait_timeouts); stays 0 unless a pipeline stalls
__device__ unsigned int g_oz_timeouts = 0;

__global__ void __launch_bounds__(256) k_oz_rowexp(const double* __restrict__ in, int* __restrict__ eA, Geom g) {
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= (int64_t)g.mtiles * BM) return;
  uint32_t mf = rowexp_partial(in, g, warp, threadIdx.x & 31, 32);
  mf = __reduce_max_sync(0xffffffffu, mf);
  if ((threadIdx.x & 31) == 0) eA[warp] = exp_from_field(mf);
}

template <int S>
__global__ void __launch_bounds__(256) k_oz_split(const double* __restrict__ in, const int* __restrict__ eA,
                                                  uint16_t* __restrict__ At, Geom g) {
  extern __shared__ __align__(16) unsigned char split_smem[];
  const int mt = (int)(blockIdx.x / (unsigned)g.nkb), kb = (int)(blockIdx.x % (unsigned)g.nkb);
  split_block<S>(in, eA, At, g, mt, kb, split_smem, (int)threadIdx.x, (int)blockDim.x);
}

// shared memory: STAGES x (S half blocks of A, S half blocks of B), then the
// barriers.  A stage is one MMA K step (16): the first or second half of a
// split block ([kgroup 4][rowgroup][8][8]: kgroups 0-1 or 2-3, contiguous).
template <class C>
struct GemmSmem {
  static const size_t stage_bytes = (size_t)C::S * (A_BYTES + C::B_BYTES) / 2;
  static const size_t bar_off = STAGES * stage_bytes;
  // barriers + alignment slack, rounded up to the 227 KB per-CTA maximum so
  // that every descriptor-addressed operand read stays inside the allocation
  static const size_t need = bar_off + 1024 + 1024;
  static const size_t bytes = need < 232448 ? 232448 : need;
};
static_assert(GemmSmem<CfgStd>::need <= 232448, "stages exceed shared memory");
static_assert(GemmSmem<CfgPrec>::need <= 232448, "stages exceed shared memory");

// Persistent kernel, one CTA per SM, 16 warps.  Warp 0 lane 0 streams the
// operands' half blocks through the STAGES-deep ring for every tile this CTA
// owns (tiles blockIdx.x, blockIdx.x + gridDim.x, ...; output-column tiles
// fastest so that concurrent CTAs share row tiles in L2); warp 1 lane 0
// issues the MMAs of tile i into accumulator set i % NBUF; warps 4..15 run
// the epilogue of tile i (warp w reads TMEM lane quarter w % 4 - the hardware
// ties a warp to lanes 32 (w % 4) .. +31 - and a third of the BN columns),
// while the MMAs of tile i + 1 fill the other set (NBUF = 2) or the producer
// prefetches its operands (NBUF = 1).
const int GEMM_THREADS = 512;
const int EPI_WARPS = 12;

template <class C>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    k_oz_gemm(const uint16_t* __restrict__ At, const int* __restrict__ eA, const uint16_t* __restrict__ Bt,
              const int* __restrict__ eB, double* __restrict__ out, Geom g) {
  constexpr int S = C::S, NACC = C::NACC, BN = C::BN, NBUF = C::NBUF;
  static_assert(BN % 8 == 0, "8-column epilogue chunks");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + GemmSmem<C>::bar_off);  // [STAGES]
  uint64_t* empty = full + STAGES;                              // [STAGES]
  uint64_t* tfull = empty + STAGES;                             // [2] accumulators ready
  uint64_t* tempty = tfull + 2;                                 // [2] accumulators read out
  uint64_t* mdone = tempty + 2;                                 // every MMA finished
  uint32_t* tmem_holder = (uint32_t*)(mdone + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ntile = (int64_t)g.mtiles * g.ntiles;

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&tfull[i], 1);
      tc::mbar_init(&tempty[i], EPI_WARPS);
    }
    tc::mbar_init(mdone, 1);
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

  constexpr int AH = A_BYTES / 2, BH = C::B_BYTES / 2;  // half blocks
  auto sA = [&](int st, int s) { return smem + (size_t)st * GemmSmem<C>::stage_bytes + (size_t)s * AH; };
  auto sB = [&](int st, int s) {
    return smem + (size_t)st * GemmSmem<C>::stage_bytes + (size_t)S * AH + (size_t)s * BH;
  };
  // K steps of 16 per tile in this launch's chunk, up to the last active
  // input entry (a 257-long contraction runs 17 steps, not 18)
  const int nsteps = oz_steps(g);

  if (warp == 0 && lane == 0) {
    // producer
    int64_t q = 0;  // ring position over all tiles
    // the A slices miss L2 on first touch (the matrix's B slices stay
    // resident): prefetch them into L2 PF_STEPS K steps ahead, across the
    // boundary into this CTA's next tile, so that the ring's bulk copies
    // (STAGES steps deep) hit L2
    constexpr int PF_STEPS = 8;
    auto prefetch_a = [&](int64_t tt, int ks) {
      const int mtp = (int)(tt / g.ntiles), kb = g.kb0 + (ks >> 1), hf = ks & 1;
      for (int s = 0; s < S; ++s)
        tc::bulk_prefetch_l2(At + (((int64_t)s * g.mtiles + mtp) * g.nkb + kb) * A_ELEMS + hf * (A_ELEMS / 2),
                             AH);
    };
    if (blockIdx.x < ntile)
      for (int ks = 0; ks < PF_STEPS && ks < nsteps; ++ks) prefetch_a(blockIdx.x, ks);
    for (int64_t t = blockIdx.x; t < ntile && ok; t += gridDim.x) {
      const int nt = (int)(t % g.ntiles), mt = (int)(t / g.ntiles);
      for (int ks = 0; ks < nsteps; ++ks, ++q) {
        const int st = (int)(q % STAGES);
        const uint32_t ph = (uint32_t)(q / STAGES) & 1u;
        if (ks + PF_STEPS < nsteps)
          prefetch_a(t, ks + PF_STEPS);
        else if (t + gridDim.x < ntile && ks + PF_STEPS - nsteps < nsteps)
          prefetch_a(t + gridDim.x, ks + PF_STEPS - nsteps);
        if (q >= STAGES && !tc::mbar_wait(&empty[st], ph ^ 1u)) {
          ok = false;
          break;
        }
        const int kb = g.kb0 + (ks >> 1), hf = ks & 1;
        tc::mbar_arrive_expect_tx(&full[st], (uint32_t)(S * (AH + BH)));
        for (int s = 0; s < S; ++s) {
          tc::bulk_g2s(sA(st, s), At + (((int64_t)s * g.mtiles + mt) * g.nkb + kb) * A_ELEMS + hf * (A_ELEMS / 2),
                       AH, &full[st]);
          tc::bulk_g2s(sB(st, s),
                       Bt + (((int64_t)s * g.ntiles + nt) * g.nkb_b + kb) * C::B_ELEMS + hf * (C::B_ELEMS / 2),
                       BH, &full[st]);
        }
      }
    }
    // drain: every copy issued must have landed before the CTA may exit
    for (int64_t r = q - STAGES; r < q; ++r) {
      if (r < 0) continue;
      if (!tc::mbar_wait(&full[r % STAGES], (uint32_t)(r / STAGES) & 1u)) ok = false;
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    const uint32_t idesc = tc::idesc_bf16_f32(BM, BN);
    int64_t q = 0;
    int64_t i = 0;  // local tile count
    for (int64_t t = blockIdx.x; t < ntile && ok; t += gridDim.x, ++i) {
      const int b = (int)(i % NBUF);
      const int64_t use = i / NBUF;  // uses of set b before this one
      if (use >= 1 && !tc::mbar_wait(&tempty[b], (uint32_t)(use - 1) & 1u)) {
        ok = false;
        break;
      }
      tc::fence_after_sync();
      const uint32_t dbase = tmem + (uint32_t)(b * NACC * BN);
      uint32_t inited = 0;
      for (int ks = 0; ks < nsteps; ++ks, ++q) {
        const int st = (int)(q % STAGES);
        const uint32_t ph = (uint32_t)(q / STAGES) & 1u;
        if (!tc::mbar_wait(&full[st], ph)) {
          ok = false;
          break;
        }
        if (C::ATMEM && q >= 2) {
          // A buffer (q & 1) was last read by the MMAs of step q - 2: their
          // commit completed that step's phase of its stage's empty barrier
          const int64_t q2 = q - 2;
          if (!tc::mbar_wait(&empty[q2 % STAGES], (uint32_t)(q2 / STAGES) & 1u)) {
            ok = false;
            break;
          }
        }
        tc::fence_after_sync();
        const uint32_t abuf = tmem + (uint32_t)(NACC * BN + (q & 1) * S * 8);
        if (C::ATMEM) {
#pragma unroll
          for (int s = 0; s < S; ++s)
            tc::tmem_cp_128x256b(abuf + (uint32_t)(s * 8),
                                 tc::sdesc_interleave(tc::smem_u32(sA(st, s)), LBO_A, SBO));
        }
#pragma unroll
        for (int s = 0; s < S; ++s) {
          const uint64_t ad = tc::sdesc_interleave(tc::smem_u32(sA(st, s)), LBO_A, SBO);
#pragma unroll
          for (int tt = 0; tt + s < S; ++tt) {
            const uint64_t bd = tc::sdesc_interleave(tc::smem_u32(sB(st, tt)), C::LBO_B, SBO);
            const int acc = s + tt < NACC - 1 ? s + tt : NACC - 1;
            if (C::ATMEM)
              tc::mma_f16_ts(dbase + (uint32_t)(acc * BN), abuf + (uint32_t)(s * 8), bd, idesc,
                             (inited >> acc) & 1u);
            else
              tc::mma_f16(dbase + (uint32_t)(acc * BN), ad, bd, idesc, (inited >> acc) & 1u);
            inited |= 1u << acc;
          }
        }
        tc::mma_commit(&empty[st]);  // frees the stage once these MMAs (and copies) have read it
      }
      tc::mma_commit(&tfull[b]);  // set b final (also after an early exit)
    }
    tc::mma_commit(mdone);
  } else if (warp >= 4) {
    // epilogue
    const int quarter = warp & 3, part = (warp >> 2) - 1;  // part 0..2: 8-column chunks part, part + 3, ...
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    const int64_t ostride = g.inner * (g.cplx ? 2 : 1);
    int64_t i = 0;
    for (int64_t t = blockIdx.x; t < ntile; t += gridDim.x, ++i) {
      const int nt = (int)(t % g.ntiles), mt = (int)(t / g.ntiles);
      const int b = (int)(i % NBUF);
      // a warp-uniform outcome keeps the .sync.aligned loads below convergent
      const bool got =
          __all_sync(0xffffffffu, tc::mbar_wait_sleep(&tfull[b], (uint32_t)(i / NBUF) & 1u));
      if (!got) ok = false;
      tc::fence_after_sync();
      const int64_t row = (int64_t)mt * BM + quarter * 32 + lane;
      const bool row_ok = row < g.nrows;
      const int erow = eA[row] - 2 * W;
      const int64_t obase = row_offset(g, row_ok ? row : 0, 0);
      for (int ch = part; ch < BN / 8 && ok; ch += 3) {
        uint32_t a[NACC][8];
#pragma unroll
        for (int qq = 0; qq < NACC; ++qq)
          tc::tmem_ld8(tmem + lane_base + (uint32_t)(b * NACC * BN + qq * BN + ch * 8), a[qq]);
        tc::tmem_ld_wait();
        if (row_ok) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int col = nt * BN + ch * 8 + j;
            if (col < g.N) {
              uint32_t gb[NACC];
#pragma unroll
              for (int qq = 0; qq < NACC; ++qq) gb[qq] = a[qq][j];
              const double v = combine_groups<NACC>(gb, erow + eB[col]);
              double* o = out + obase + (int64_t)col * ostride;
              *o = g.accum ? *o + v : v;
            }
          }
        }
        __syncwarp();
      }
      // the set may be refilled once every epilogue warp has read it
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&tempty[b]);
      if (!ok) break;
    }
  }
  // every MMA must have completed before TMEM is released
  __syncwarp();
  if (warp == 0 && !tc::mbar_wait_sleep(mdone, 0)) ok = false;
  tc::fence_before_sync();
  __syncthreads();
  if (!ok && lane == 0) atomicAdd(&g_oz_timeouts, 1u);
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 512);
  }
}

namespace sgpu {
namespace oz {

int pick_digits(int K) { return K >= 1 && K <= OZ_MAX_K ? SGPU_OK : SGPU_ERR_UNSUPPORTED; }

template <class C>
static int matrix_create_cfg(const double* M, int N, Matrix* out) {
  std::vector<uint16_t> tiles(matrix_tile_elems<C>(N));
  std::vector<int> ex((size_t)((N + C::BN - 1) / C::BN) * C::BN);
  // columns split independently: spread them over the host's cores (the
  // plan's set-up cost grows as N^2 x digits)
  const unsigned hw = std::thread::hardware_concurrency();
  const int nth = (int)std::max(1u, std::min(hw ? hw : 1u, 16u));
  std::vector<std::thread> pool;
  for (int t = 0; t < nth; ++t)
    pool.emplace_back([&, t]() {
      for (int n = t; n < N; n += nth) split_matrix_column<C>(M, N, n, tiles.data(), ex.data());
    });
  for (auto& th : pool) th.join();
  const size_t tb = tiles.size() * sizeof(uint16_t), eb = ex.size() * sizeof(int);
  void* dev = nullptr;
  if (cudaMalloc(&dev, tb + eb) != cudaSuccess) {
    cudaGetLastError();
    return SGPU_ERR_NOMEM;
  }
  out->tiles = (uint16_t*)dev;
  out->exps = (int*)((char*)dev + tb);
  if (cudaMemcpy(out->tiles, tiles.data(), tb, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(out->exps, ex.data(), eb, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(dev);
    cudaGetLastError();
    out->tiles = nullptr;
    return SGPU_ERR_CUDA;
  }
  return SGPU_OK;
}

int matrix_create(const double* M, int N, int precise, Matrix* out) {
  if (pick_digits(N) != SGPU_OK) return SGPU_ERR_UNSUPPORTED;
  out->N = N;
  out->precise = precise ? 1 : 0;
  out->S = precise ? CfgPrec::S : CfgStd::S;
  out->K = 0;
  for (int k = 0; k < N; ++k)
    for (int n = 0; n < N; ++n)
      if (M[(size_t)k * N + n] != 0.0) out->K = k + 1;
  return precise ? matrix_create_cfg<CfgPrec>(M, N, out) : matrix_create_cfg<CfgStd>(M, N, out);
}

void matrix_destroy(Matrix* m) {
  if (m && m->tiles) cudaFree(m->tiles);
  if (m) m->tiles = nullptr;
}

size_t workspace_bytes(const Matrix& m, int64_t nlines, int64_t inner, int cplx) {
  const Geom g = make_geom(m.N, nlines, inner, cplx, m.precise ? CfgPrec::BN : CfgStd::BN, m.K);
  return a_split_bytes(g, m.S);
}

// per-device launch state: the large dynamic shared memory attributes (set
// once per device and configuration) and the SM count
struct OzDevState {
  std::once_flag attr[2];
  int attr_rc[2] = {0, 0};
  std::once_flag sm_once;
  int nsm = 0;
};
static OzDevState g_oz_dev[64];

template <class C>
static int run(const Matrix& m, const Geom& g, const double* in, double* out, void* work, cudaStream_t stream) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return SGPU_ERR_CUDA;
  }
  OzDevState& ds = g_oz_dev[dev];
  const int ci = m.precise ? 1 : 0;
  std::call_once(ds.attr[ci], [&]() {
    ds.attr_rc[ci] = (cudaFuncSetAttribute(k_oz_gemm<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)GemmSmem<C>::bytes) == cudaSuccess &&
                      cudaFuncSetAttribute(k_oz_split<C::S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           C::S * A_BYTES) == cudaSuccess)
                         ? 1
                         : -1;
    cudaGetLastError();
  });
  if (ds.attr_rc[ci] != 1) return SGPU_ERR_CUDA;
  std::call_once(ds.sm_once, [&]() {
    if (cudaDeviceGetAttribute(&ds.nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || ds.nsm <= 0) ds.nsm = 1;
    cudaGetLastError();
  });
  const int nsm = ds.nsm;
  uint16_t* At = (uint16_t*)work;
  int* eA = (int*)((char*)work + (size_t)C::S * g.mtiles * g.nkb * A_BYTES);
  const int64_t nrow_pad = (int64_t)g.mtiles * BM;
  k_oz_rowexp<<<(unsigned)((nrow_pad * 32 + 255) / 256), 256, 0, stream>>>(in, eA, g);
  k_oz_split<C::S><<<(unsigned)((int64_t)g.mtiles * g.nkb), 256, C::S * A_BYTES, stream>>>(in, eA, At, g);
  const int64_t ntile = (int64_t)g.mtiles * g.ntiles;
  const unsigned nctas = (unsigned)(ntile < nsm ? ntile : nsm);
  // one launch per K chunk of at most 1024 (stream-ordered: a chunk adds to
  // the previous chunks' output)
  for (int c = 0; c < num_chunks(g); ++c)
    k_oz_gemm<C><<<nctas, GEMM_THREADS, GemmSmem<C>::bytes, stream>>>(At, eA, m.tiles, m.exps, out,
                                                                      chunk_geom(g, c));
  return cudaGetLastError() == cudaSuccess ? SGPU_OK : SGPU_ERR_CUDA;
}

int contract(const Matrix& m, const double* in, double* out, int64_t nlines, int64_t inner, int cplx,
             void* work, size_t work_bytes, cudaStream_t stream) {
  if (nlines == 0) return SGPU_OK;
  if (!m.tiles) return SGPU_ERR_ARG;
  const Geom g = make_geom(m.N, nlines, inner, cplx, m.precise ? CfgPrec::BN : CfgStd::BN, m.K);
  // one-dimensional grids: tiles x K blocks stay below 2^31
  if ((int64_t)g.mtiles * (g.nkb > g.ntiles ? g.nkb : g.ntiles) > 0x7fffffff || (int64_t)g.mtiles * 16 > 0x7fffffff)
    return SGPU_ERR_ARG;
  if (work_bytes < a_split_bytes(g, m.S) || ((uintptr_t)work & 255)) return SGPU_ERR_ARG;
  return m.precise ? run<CfgPrec>(m, g, in, out, work, stream) : run<CfgStd>(m, g, in, out, work, stream);
}

}  // namespace oz
}  // namespace sgpu

namespace sgpu {
int f256_read_timeouts(unsigned int* count);  // fft256.cu
}

extern "C" int sgpu_wait_timeouts(unsigned int* count) {
  if (!count) return SGPU_ERR_ARG;
  unsigned int a = 0, b = 0;
  if (cudaMemcpyFromSymbol(&a, g_oz_timeouts, sizeof(unsigned int)) != cudaSuccess) {
    cudaGetLastError();
    return SGPU_ERR_CUDA;
  }
  int st = sgpu::lc::read_timeouts(&b);
  unsigned int c = 0;
  if (st == SGPU_OK) st = sgpu::f256_read_timeouts(&c);
  if (st != SGPU_OK) {
    cudaGetLastError();
    return st;
  }
  *count = a + b + c;
  return SGPU_OK;
}

// the timeout counters as last seen by sgpu_last_error (process-wide)
static std::atomic<unsigned int> g_seen_timeouts{0};

extern "C" int sgpu_last_error(cudaStream_t stream) {
  if (cudaStreamSynchronize(stream) != cudaSuccess) {
    cudaGetLastError();
    return SGPU_ERR_CUDA;
  }
  unsigned int now = 0;
  const int st = sgpu_wait_timeouts(&now);
  if (st != SGPU_OK) return st;
  const unsigned int seen = g_seen_timeouts.exchange(now);
  return now != seen ? SGPU_ERR_TIMEOUT : SGPU_OK;
}
