// Kernels of the strided length-256 Fourier passes (fft256.cuh has the
// schedule), FP64 and double-float, and their launcher.
#include <mutex>
#include <type_traits>

#include "fft256.cuh"
#include "fft256_fx.cuh"

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

// per device: the large dynamic shared memory of every instantiation, set
// once ([arithmetic: FP64, double-float, fixed point][kind][occupancy])
struct DevAttr {
  std::once_flag once[3][4][2];
  int rc[3][4][2] = {};
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
// 2 or 3 picks the register budget (above); fixed: the mixed form in 64-bit
// fixed point instead of double-float (SGPU_ERR_UNSUPPORTED for the plain
// form, whose arithmetic is FP64).
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
