// Kernels of the strided length-256 Fourier passes (fft256.cuh has the
// schedule), FP64 and double-float, and their launcher.
#include <cuda.h>  // CUtensorMap and its enums; the encoder comes from the driver at run time

#include <mutex>
#include <type_traits>

#include "fft256.cuh"
#include "fft256_fx.cuh"
#include "tc_ptx.cuh"

// bounded waits of the tensor-copy kernels that gave up (added to the other
// kernels' count by sgpu_wait_timeouts)
__device__ unsigned int g_f256_timeouts = 0;

namespace sgpu {
namespace f256 {

// CTAs per SM (MINB): 2 gives 128 registers a thread (the 16 complex values
// of a thread's register DFT and the DFT's temporaries stay in registers),
// 3 gives 85 registers and more warps to hide latency, at the cost of spills
template <class R, int KIND, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_fft256(LinePlan p, Args a) {
  extern __shared__ __align__(16) unsigned char f256_smem[];
  Cx<R>* Z = (Cx<R>*)f256_smem;
  const int64_t blk = (int64_t)blockIdx.x;
  const int t = (int)threadIdx.x;
  pass1<R, KIND>(p, a, blk, Z, t);
  __syncthreads();
  Cx<R> v[16];
  pass2_dft<R>(Z, t, v);
  if (KIND == R2C) {
    __syncthreads();
    r2c_stash<R>(Z, t, v);
    __syncthreads();
    r2c_post<R>(a, blk, Z, t, NT);
  } else {
    pass2_store<R, KIND>(a, blk, t, v);
  }
}

// the mixed form in 64-bit fixed point (fft256_fx.cuh)
template <int KIND, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_fft256_fx(LinePlan p, Args a, FxScale s) {
  extern __shared__ __align__(16) unsigned char f256_smem[];
  const int t = (int)threadIdx.x;
  const int64_t blk = (int64_t)blockIdx.x;
  if (KIND == C2C_FWD || KIND == C2C_BWD) {
    const FxShared sh = fx_shared(f256_smem);
    Cq v[16];
    fx_c2c_pass1<KIND>(p, a, blk, sh, t);
    __syncthreads();
    const int E = fx_c2c_pass2(sh, t, v);
    fx_c2c_store<KIND>(a, t, v, E, sh, s);
    return;
  }
  const FxHalf sh = fxh_shared(f256_smem);
  if (KIND == R2C)
    fxh_r2c_pass1(p, a, blk, sh, t);
  else
    fxh_c2r_pass1(p, a, blk, sh, t);
  __syncthreads();
  // pass 2: two (line, k1) items per thread
  Cq v[2][8];
  int E[2];
#pragma unroll
  for (int j = 0; j < 2; ++j) E[j] = fxh_pass2(sh, (t + NT * j) & 31, (t + NT * j) >> 5, v[j]);
  if (KIND == R2C) {
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 2; ++j) fxh_r2c_stash(sh, (t + NT * j) & 31, (t + NT * j) >> 5, v[j], E[j]);
    __syncthreads();
    fxh_r2c_post(p, a, sh, t, NT, s);
  } else {
#pragma unroll
    for (int j = 0; j < 2; ++j) fxh_c2r_store(a, sh, (t + NT * j) & 31, (t + NT * j) >> 5, v[j], E[j], s);
  }
}

// C2C in fixed point with the block's input staged by one tensor copy
// (cp.async.bulk.tensor): lines l0 .. l0 + TL - 1 (l0 = TL blk, all in one
// outer block) are the box {2 TL doubles, 256 rows, 1} at (2 (l0 mod inner),
// 0, l0 / inner) of the map {2 inner, 256, outer} doubles, row-major in the
// exchange buffer's space; each thread reads its 16 values there, and after
// a barrier the buffer serves the pass-1 -> pass-2 exchange as before.  The
// arithmetic is fx_c2c_pass1's: the same bits.
const size_t FX_TILE_BYTES = (size_t)2 * TL * N * sizeof(double);  // 64 KB
const uint64_t FX_TMA_WAIT_NS = 1000000000ull;
static_assert(FX_TILE_BYTES <= sizeof(Cq) * (size_t)TL * LDZ, "the tile fits the exchange buffer");
SGPU_HD size_t fx_tma_bar_off() { return (fx_smem_bytes() + 15) & ~(size_t)15; }
SGPU_HD size_t fx_tma_smem_bytes() { return fx_tma_bar_off() + 16 + 128; }  // + the mbarrier, 128-byte alignment

template <int KIND, int MINB>
__global__ void __launch_bounds__(NT, MINB)
    k_fft256_fx_tma(LinePlan p, Args a, FxScale s, const __grid_constant__ CUtensorMap tmap) {
  extern __shared__ __align__(16) unsigned char f256_smem[];
  unsigned char* base = (unsigned char*)(((uintptr_t)f256_smem + 127) & ~(uintptr_t)127);
  const FxShared sh = fx_shared(base);
  uint64_t* bar = (uint64_t*)(base + fx_tma_bar_off());
  const int t = (int)threadIdx.x;
  const int64_t blk = (int64_t)blockIdx.x;
  if (t == 0) {
    tc::mbar_init(bar, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  if (t == 0) {
    const int64_t l0 = blk * TL;
    tc::mbar_arrive_expect_tx(bar, (uint32_t)FX_TILE_BYTES);
    tc::tma_load_3d(sh.Z, &tmap, (int)(2 * (l0 % a.inner)), 0, (int)(l0 / a.inner), bar);
  }
  const bool got = tc::mbar_wait_try(bar, 0, FX_TMA_WAIT_NS);
  if (!got && t == 0) atomicAdd(&g_f256_timeouts, 1u);
  double x[32];
  const int et = fx_c2c_load_tile(a, blk, sh, (const double*)sh.Z, t, x);
  __syncthreads();  // every value is in registers: the buffer is the exchange buffer from here on
  fx_c2c_pass1_regs<KIND>(p, sh, t, x, et);
  __syncthreads();
  Cq v[16];
  const int E = fx_c2c_pass2(sh, t, v);
  fx_c2c_store<KIND>(a, t, v, E, sh, s);
  // a copy that outlived the wait must land before the CTA's shared memory goes
  if (!got) tc::mbar_wait_try(bar, 0, FX_TMA_WAIT_NS);
}

// per device: the large dynamic shared memory of every instantiation, set
// once ([arithmetic: FP64, double-float, fixed point][kind][occupancy])
struct DevAttr {
  std::once_flag once[3][4][2];
  int rc[3][4][2] = {};
  std::once_flag tma_once[4][2];  // the tensor-copy C2C kernels
  int tma_rc[4][2] = {};
};
const int MAX_DEV = 64;
DevAttr g_dev[MAX_DEV];

template <class R, int KIND, int MINB>
int launch_kind(const LinePlan& p, const Args& a, unsigned nblocks, cudaStream_t s) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEV) return SGPU_ERR_CUDA;
  DevAttr& d = g_dev[dev];
  const int ri = std::is_same<R, df>::value ? 1 : 0, mi = MINB == 3 ? 1 : 0;
  std::call_once(d.once[ri][KIND][mi], [&]() {
    d.rc[ri][KIND][mi] = cudaFuncSetAttribute(k_fft256<R, KIND, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem_bytes<R>()) == cudaSuccess
                             ? 1
                             : -1;
    cudaGetLastError();
  });
  if (d.rc[ri][KIND][mi] != 1) return SGPU_ERR_CUDA;
  k_fft256<R, KIND, MINB><<<nblocks, NT, smem_bytes<R>(), s>>>(p, a);
  return cudaGetLastError() == cudaSuccess ? SGPU_OK : SGPU_ERR_CUDA;
}

template <int KIND, int MINB>
int launch_fx(const LinePlan& p, const Args& a, const FxScale& sc, unsigned nblocks, cudaStream_t s) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEV) return SGPU_ERR_CUDA;
  DevAttr& d = g_dev[dev];
  const int mi = MINB == 3 ? 1 : 0;
  const size_t smem = (KIND == R2C || KIND == C2R) ? fxh_smem_bytes() : fx_smem_bytes();
  std::call_once(d.once[2][KIND][mi], [&]() {
    d.rc[2][KIND][mi] = cudaFuncSetAttribute(k_fft256_fx<KIND, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem) == cudaSuccess
                            ? 1
                            : -1;
    cudaGetLastError();
  });
  if (d.rc[2][KIND][mi] != 1) return SGPU_ERR_CUDA;
  k_fft256_fx<KIND, MINB><<<nblocks, NT, smem, s>>>(p, a, sc);
  return cudaGetLastError() == cudaSuccess ? SGPU_OK : SGPU_ERR_CUDA;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [&]() {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)f;
    cudaGetLastError();
  });
  return fn;
}

// SGPU_ERR_UNSUPPORTED when the layout does not suit the tensor copy (a
// block's lines would straddle two outer blocks, or the driver has no
// encoder): the caller then runs the kernel that loads its own values
template <int KIND, int MINB>
int launch_fx_tma(const LinePlan& p, const Args& a, const FxScale& sc, unsigned nblocks, cudaStream_t s) {
  const int64_t outer = a.nlines / a.inner;
  if (outer * a.inner != a.nlines || (outer > 1 && a.inner % TL != 0)) return SGPU_ERR_UNSUPPORTED;
  if (((uintptr_t)a.in & 15) || 2 * a.inner > 0x7fffffffLL || outer > 0x7fffffffLL) return SGPU_ERR_UNSUPPORTED;
  const EncodeTiledFn enc = encode_tiled();
  if (!enc) return SGPU_ERR_UNSUPPORTED;
  CUtensorMap tm;
  const cuuint64_t dims[3] = {(cuuint64_t)(2 * a.inner), (cuuint64_t)N, (cuuint64_t)outer};
  const cuuint64_t strides[2] = {(cuuint64_t)(2 * a.inner * sizeof(double)),
                                 (cuuint64_t)(2 * a.inner * sizeof(double)) * N};  // bytes, multiples of 16
  const cuuint32_t box[3] = {2 * TL, N, 1};                                         // 256 x 256 bytes
  const cuuint32_t estr[3] = {1, 1, 1};
  if (enc(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, (void*)a.in, dims, strides, box, estr,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return SGPU_ERR_UNSUPPORTED;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEV) return SGPU_ERR_CUDA;
  DevAttr& d = g_dev[dev];
  const int mi = MINB == 3 ? 1 : 0;
  std::call_once(d.tma_once[KIND][mi], [&]() {
    d.tma_rc[KIND][mi] = cudaFuncSetAttribute(k_fft256_fx_tma<KIND, MINB>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)fx_tma_smem_bytes()) == cudaSuccess
                             ? 1
                             : -1;
    cudaGetLastError();
  });
  if (d.tma_rc[KIND][mi] != 1) return SGPU_ERR_CUDA;
  k_fft256_fx_tma<KIND, MINB><<<nblocks, NT, fx_tma_smem_bytes(), s>>>(p, a, sc, tm);
  return cudaGetLastError() == cudaSuccess ? SGPU_OK : SGPU_ERR_CUDA;
}

template <int MINB>
int launch_fx_kind(int kind, const LinePlan& p, const Args& a, const FxScale& sc, unsigned nb, cudaStream_t s) {
  switch (kind) {
    case C2C_FWD: return launch_fx<C2C_FWD, MINB>(p, a, sc, nb, s);
    case C2C_BWD: return launch_fx<C2C_BWD, MINB>(p, a, sc, nb, s);
    case R2C: return launch_fx<R2C, MINB>(p, a, sc, nb, s);
    case C2R: return launch_fx<C2R, MINB>(p, a, sc, nb, s);
  }
  return SGPU_ERR_ARG;
}

template <class R, int MINB>
int launch_r(int kind, const LinePlan& p, const Args& a, unsigned nb, cudaStream_t s) {
  switch (kind) {
    case C2C_FWD: return launch_kind<R, C2C_FWD, MINB>(p, a, nb, s);
    case C2C_BWD: return launch_kind<R, C2C_BWD, MINB>(p, a, nb, s);
    case R2C: return launch_kind<R, R2C, MINB>(p, a, nb, s);
    case C2R: return launch_kind<R, C2R, MINB>(p, a, nb, s);
  }
  return SGPU_ERR_ARG;
}

}  // namespace f256

// The plan's length-256 Fourier pass along a strided axis, or
// SGPU_ERR_UNSUPPORTED when the plan or layout does not qualify; ctas_per_sm
// 2 or 3 picks the register budget (above); fixed: 1 the mixed form in 64-bit
// fixed point instead of double-float (SGPU_ERR_UNSUPPORTED for the plain
// form, whose arithmetic is FP64), 2 the same with the C2C input staged by a
// tensor copy.
int f256_launch(const LinePlan& p, const double* in, double* out, int64_t nlines, int64_t inner, double scl,
                int ctas_per_sm, int fixed, cudaStream_t s) {
  using namespace f256;
  if (p.n != N || p.m != N || p.rader || inner < 16) return SGPU_ERR_UNSUPPORTED;
  int kind;
  switch (p.kind) {
    case SGPU_XF_C2C_FWD: kind = C2C_FWD; break;
    case SGPU_XF_C2C_BWD: kind = C2C_BWD; break;
    case SGPU_XF_R2C: kind = R2C; break;
    case SGPU_XF_C2R: kind = C2R; break;
    default: return SGPU_ERR_UNSUPPORTED;
  }
  if (in == out && (kind == R2C || kind == C2R)) return SGPU_ERR_ARG;
  const int64_t nt = tiles(kind, nlines, p.pb);
  if (nt == 0) return SGPU_OK;
  if (nt > 0x7fffffffLL) return SGPU_ERR_ARG;
  Args a{in, out, nlines, inner, scl, p.pb};
  if (fixed) {
    if (p.form != SGPU_MIXED_DF || !p.tw_q) return SGPU_ERR_UNSUPPORTED;
    // complex entries move as 16-byte loads and stores: complex arrays must
    // be 16-byte aligned (else the caller runs the generic programs)
    const bool cin = kind != R2C, cout = kind != C2R;
    if ((cin && ((uintptr_t)in & 15)) || (cout && ((uintptr_t)out & 15))) return SGPU_ERR_UNSUPPORTED;
    const FxScale sc = fx_scale(scl);
    const int64_t nx = fx_tiles(kind, nlines);  // R2C / C2R: 32 real lines per CTA, no pairs
    if (nx > 0x7fffffffLL) return SGPU_ERR_ARG;
    if (fixed == 2 && (kind == C2C_FWD || kind == C2C_BWD)) {
      // the input tile staged by a tensor copy (where the layout allows one)
      int st;
      if (kind == C2C_FWD)
        st = ctas_per_sm == 3 ? launch_fx_tma<C2C_FWD, 3>(p, a, sc, (unsigned)nx, s)
                              : launch_fx_tma<C2C_FWD, 2>(p, a, sc, (unsigned)nx, s);
      else
        st = ctas_per_sm == 3 ? launch_fx_tma<C2C_BWD, 3>(p, a, sc, (unsigned)nx, s)
                              : launch_fx_tma<C2C_BWD, 2>(p, a, sc, (unsigned)nx, s);
      if (st != SGPU_ERR_UNSUPPORTED) return st;
    }
    return ctas_per_sm == 3 ? launch_fx_kind<3>(kind, p, a, sc, (unsigned)nx, s)
                            : launch_fx_kind<2>(kind, p, a, sc, (unsigned)nx, s);
  }
  if (ctas_per_sm == 3)
    return p.form == SGPU_MIXED_DF ? launch_r<df, 3>(kind, p, a, (unsigned)nt, s)
                                   : launch_r<double, 3>(kind, p, a, (unsigned)nt, s);
  return p.form == SGPU_MIXED_DF ? launch_r<df, 2>(kind, p, a, (unsigned)nt, s)
                                 : launch_r<double, 2>(kind, p, a, (unsigned)nt, s);
}

}  // namespace sgpu

namespace sgpu {
// the tensor-copy kernels' given-up waits (sgpu_wait_timeouts adds them up)
int f256_read_timeouts(unsigned int* count) {
  return cudaMemcpyFromSymbol(count, g_f256_timeouts, sizeof(unsigned int)) == cudaSuccess ? SGPU_OK
                                                                                             : SGPU_ERR_CUDA;
}
}  // namespace sgpu
