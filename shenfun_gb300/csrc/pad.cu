// Zero padding and truncation of Fourier coefficients for the padded
// (3/2-rule dealiased) transforms (fourier/bases.py:409-435 for R2C,
// :570-598 for C2C; TensorProductSpace.get_dealiased,
// tensorproductspace.py:543).  A padded backward transform is
// pad (N -> M coefficients) + the unnormalised length-M inverse transform; a
// padded forward transform is the length-M transform scaled by 1/M +
// truncate (M -> N).  An even N's Nyquist coefficient is shared between the
// +N/2 and -N/2 slots of the padded array: halved on the way out (made real
// for R2C), summed (twice the real part for R2C) on the way back.
//
// One thread per output element of a (outer, n, inner) complex array:
// HBM-bound copies, consecutive threads along `inner` (coalesced).
#include "sgpu_common.cuh"

using namespace sgpu;

namespace {

SGPU_HD void pad_elem(const cd* in, cd* out, int64_t t, int64_t outer, int N, int M, int64_t inner, int r2c) {
  const int nin = r2c ? N / 2 + 1 : N;
  const int nout = r2c ? M / 2 + 1 : M;
  const int64_t i = t % inner;
  const int64_t oj = t / inner;
  const int j = (int)(oj % nout);
  const int64_t o = oj / nout;
  int src = -1;
  if (j <= N / 2)
    src = j;
  else if (!r2c && j >= M - N / 2)
    src = j - M + N;
  cd v = cx<double>(0.0, 0.0);
  if (src >= 0 && src < nin) {
    v = in[(o * nin + src) * inner + i];
    if (N % 2 == 0 && (src == N / 2 || (!r2c && j == M - N / 2))) {
      v.re *= 0.5;
      v.im = r2c ? 0.0 : v.im * 0.5;
    }
  }
  out[t] = v;
}

SGPU_HD void truncate_elem(const cd* in, cd* out, int64_t t, int64_t outer, int N, int M, int64_t inner,
                           int r2c) {
  const int nin = r2c ? M / 2 + 1 : M;
  const int nout = r2c ? N / 2 + 1 : N;
  const int64_t i = t % inner;
  const int64_t oj = t / inner;
  const int j = (int)(oj % nout);
  const int64_t o = oj / nout;
  cd v = cx<double>(0.0, 0.0);
  if (j <= N / 2) v = in[(o * nin + j) * inner + i];
  if (!r2c && j >= N - N / 2) {
    const cd w = in[(o * nin + (j - N + M)) * inner + i];
    v.re += w.re;
    v.im += w.im;
  }
  if (r2c && N % 2 == 0 && j == N / 2) {
    v.re *= 2.0;
    v.im = 0.0;
  }
  out[t] = v;
}

__global__ void __launch_bounds__(256) k_fourier_pad(const cd* __restrict__ in, cd* __restrict__ out, int64_t outer,
                                                     int N, int M, int64_t inner, int r2c, int64_t total) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
    pad_elem(in, out, t, outer, N, M, inner, r2c);
}

__global__ void __launch_bounds__(256) k_fourier_truncate(const cd* __restrict__ in, cd* __restrict__ out,
                                                          int64_t outer, int N, int M, int64_t inner, int r2c,
                                                          int64_t total) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
    truncate_elem(in, out, t, outer, N, M, inner, r2c);
}

int launch_args(int kind, int N, int M, int* r2c) {
  if (kind == SGPU_XF_R2C || kind == SGPU_XF_C2R)
    *r2c = 1;
  else if (kind == SGPU_XF_C2C_FWD || kind == SGPU_XF_C2C_BWD)
    *r2c = 0;
  else
    return SGPU_ERR_ARG;
  if (N < 1 || M < N) return SGPU_ERR_ARG;
  return SGPU_OK;
}

unsigned grid_for(int64_t total) {
  int64_t b = (total + 255) / 256;
  const int64_t cap = 152 * 16;  // grid-stride beyond 16 CTAs per SM
  return (unsigned)(b < cap ? (b < 1 ? 1 : b) : cap);
}

}  // namespace

extern "C" int sgpu_fourier_pad(const void* in, void* out, int64_t outer, int N, int M, int64_t inner, int kind,
                                cudaStream_t stream) {
  int r2c = 0;
  if (!in || !out || outer < 0 || inner < 1 || in == out) return SGPU_ERR_ARG;
  const int st = launch_args(kind, N, M, &r2c);
  if (st != SGPU_OK) return st;
  const int64_t total = outer * (r2c ? M / 2 + 1 : M) * inner;
  if (total == 0) return SGPU_OK;
  k_fourier_pad<<<grid_for(total), 256, 0, stream>>>((const cd*)in, (cd*)out, outer, N, M, inner, r2c, total);
  return cudaGetLastError() == cudaSuccess ? SGPU_OK : SGPU_ERR_CUDA;
}

extern "C" int sgpu_fourier_truncate(const void* in, void* out, int64_t outer, int N, int M, int64_t inner,
                                     int kind, cudaStream_t stream) {
  int r2c = 0;
  if (!in || !out || outer < 0 || inner < 1 || in == out) return SGPU_ERR_ARG;
  const int st = launch_args(kind, N, M, &r2c);
  if (st != SGPU_OK) return st;
  const int64_t total = outer * (r2c ? N / 2 + 1 : N) * inner;
  if (total == 0) return SGPU_OK;
  k_fourier_truncate<<<grid_for(total), 256, 0, stream>>>((const cd*)in, (cd*)out, outer, N, M, inner, r2c,
                                                          total);
  return cudaGetLastError() == cudaSuccess ? SGPU_OK : SGPU_ERR_CUDA;
}
