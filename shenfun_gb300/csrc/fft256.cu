// Kernels of the strided length-256 Fourier passes (fft256.cuh has the
// schedule), FP64 and double-float, and their launcher.
#include "fft256.cuh"

namespace sgpu {
namespace f256 {

// CTAs per SM: 2 (128 registers a thread: the 16 complex values of a
// thread's register DFT stay in registers) for double-float; FP64 values are
// pairs of FP64 registers, so the same budget holds
template <class R, int KIND>
__global__ void __launch_bounds__(NT, 2) k_fft256(LinePlan p, Args a) {
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

template <class R, int KIND>
int launch_kind(const LinePlan& p, const Args& a, unsigned nblocks, cudaStream_t s) {
  static bool attr = false;  // benign race: every caller sets the same value
  if (!attr) {
    if (cudaFuncSetAttribute(k_fft256<R, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_bytes<R>()) != cudaSuccess) {
      cudaGetLastError();
      return SGPU_ERR_CUDA;
    }
    attr = true;
  }
  k_fft256<R, KIND><<<nblocks, NT, smem_bytes<R>(), s>>>(p, a);
  return cudaGetLastError() == cudaSuccess ? SGPU_OK : SGPU_ERR_CUDA;
}

template <class R>
int launch_r(int kind, const LinePlan& p, const Args& a, unsigned nb, cudaStream_t s) {
  switch (kind) {
    case C2C_FWD: return launch_kind<R, C2C_FWD>(p, a, nb, s);
    case C2C_BWD: return launch_kind<R, C2C_BWD>(p, a, nb, s);
    case R2C: return launch_kind<R, R2C>(p, a, nb, s);
    case C2R: return launch_kind<R, C2R>(p, a, nb, s);
  }
  return SGPU_ERR_ARG;
}

}  // namespace f256

// The plan's length-256 Fourier pass along a strided axis, or
// SGPU_ERR_UNSUPPORTED when the plan or layout does not qualify.
int f256_launch(const LinePlan& p, const double* in, double* out, int64_t nlines, int64_t inner, double scl,
                cudaStream_t s) {
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
  const int64_t nt = tiles(kind, nlines);
  if (nt == 0) return SGPU_OK;
  if (nt > 0x7fffffffLL) return SGPU_ERR_ARG;
  Args a{in, out, nlines, inner, scl};
  return p.form == SGPU_MIXED_DF ? launch_r<df>(kind, p, a, (unsigned)nt, s)
                                 : launch_r<double>(kind, p, a, (unsigned)nt, s);
}

}  // namespace sgpu
