// The line-transform kernel, one instantiation per (arithmetic, program
// group), so that each compiles as a separate, smaller function and the two
// arithmetic forms and two program families build in parallel translation
// units (xf_fourier_f64.cu, xf_fourier_df.cu, xf_cheb_f64.cu, xf_cheb_df.cu).
//   G = 0 R2C, 1 C2R, 2 C2C, 3 DCT-II family (DCT2, Chebyshev scalar
//   product, forward), 4 DCT-III family (DCT3, Chebyshev backward)
#pragma once

#include <mutex>

#include "fft_line.cuh"

namespace sgpu {

enum { XF_G_R2C = 0, XF_G_C2R = 1, XF_G_C2C = 2, XF_G_DCT2 = 3, XF_G_DCT3 = 4 };

inline int xf_group(int kind) {
  switch (kind) {
    case SGPU_XF_R2C: return XF_G_R2C;
    case SGPU_XF_C2R: return XF_G_C2R;
    case SGPU_XF_C2C_FWD:
    case SGPU_XF_C2C_BWD: return XF_G_C2C;
    case SGPU_XF_DCT3:
    case SGPU_XF_CHEB_BACKWARD: return XF_G_DCT3;
    default: return XF_G_DCT2;
  }
}

#ifdef __CUDACC__
// CTAs per SM: the line programs are latency-bound (long scoreboard and
// barrier stalls at two CTAs, 118 registers); capping registers (80 for
// three CTAs, 64 for four) costs a few hundred bytes of L1-cached spills and
// measured 20-25 % faster Fourier passes on the channel grid; four CTAs
// measured best for FP64, three for double-float
template <class R>
struct LineMinBlocks {
  static const int value = 3;
};
template <>
struct LineMinBlocks<double> {
  static const int value = 4;
};

template <class R, int G>
__global__ void __launch_bounds__(256, LineMinBlocks<R>::value) sgpu_line_kernel(LinePlan p, const double* in,
                                                                                double* out,
                                                        int data_complex, int64_t nlines,
                                                        int64_t inner, double scl) {
  extern __shared__ __align__(16) unsigned char sgpu_smem[];
  const int64_t blk = (int64_t)blockIdx.x;
  const int tid = (int)threadIdx.x, nth = (int)blockDim.x;
  if (G == XF_G_R2C)
    prog_r2c<R>(p, in, out, nlines, inner, scl, blk, sgpu_smem, tid, nth);
  else if (G == XF_G_C2R)
    prog_c2r<R>(p, in, out, nlines, inner, scl, blk, sgpu_smem, tid, nth);
  else if (G == XF_G_C2C)
    prog_c2c<R>(p, in, out, nlines, inner, scl, blk, sgpu_smem, tid, nth);
  else if (G == XF_G_DCT2)
    prog_dct2<R>(p, in, out, data_complex, nlines, inner, scl, blk, sgpu_smem, tid, nth);
  else
    prog_dct3<R>(p, in, out, data_complex, nlines, inner, scl, blk, sgpu_smem, tid, nth);
}

// the large dynamic shared memory attribute, set once per device and
// instantiation
template <class R, int G>
struct XfAttr {
  std::once_flag once[64];
  int rc[64] = {};
};

template <class R, int G>
int xf_launch_group(const LinePlan& p, const double* in, double* out, int dc, int64_t nlines,
                    int64_t inner, double scl, unsigned nblocks, cudaStream_t stream) {
  static XfAttr<R, G> attr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return SGPU_ERR_CUDA;
  }
  std::call_once(attr.once[dev], [&]() {
    attr.rc[dev] = cudaFuncSetAttribute(sgpu_line_kernel<R, G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        220 * 1024) == cudaSuccess ? 1 : -1;
    cudaGetLastError();
  });
  if (attr.rc[dev] != 1) return SGPU_ERR_CUDA;
  sgpu_line_kernel<R, G><<<nblocks, p.nthreads, p.smem, stream>>>(p, in, out, dc, nlines, inner, scl);
  return cudaGetLastError() == cudaSuccess ? SGPU_OK : SGPU_ERR_CUDA;
}
#endif

// per-TU launchers (group G of the family)
int xf_launch_fourier_f64(int G, const LinePlan& p, const double* in, double* out, int dc,
                          int64_t nlines, int64_t inner, double scl, unsigned nblocks, cudaStream_t s);
int xf_launch_fourier_df(int G, const LinePlan& p, const double* in, double* out, int dc,
                         int64_t nlines, int64_t inner, double scl, unsigned nblocks, cudaStream_t s);
int xf_launch_cheb_f64(int G, const LinePlan& p, const double* in, double* out, int dc,
                       int64_t nlines, int64_t inner, double scl, unsigned nblocks, cudaStream_t s);
int xf_launch_cheb_df(int G, const LinePlan& p, const double* in, double* out, int dc,
                      int64_t nlines, int64_t inner, double scl, unsigned nblocks, cudaStream_t s);

}  // namespace sgpu
