// C ABI of the batched banded solvers (see solvers.cuh for the algorithms).
#include <mutex>

#include "solvers.cuh"

using namespace sgpu;

namespace {

const int kThreads = 128;

inline int finish() {
  return cudaGetLastError() == cudaSuccess ? SGPU_OK : SGPU_ERR_CUDA;
}

inline unsigned nblk(int64_t nsys) { return (unsigned)((nsys + kThreads - 1) / kThreads); }

}  // namespace

__global__ void k_tdma_lu(double* data, int64_t n) { tdma_lu_prog(data, n); }
__global__ void k_pdma_lu(double* data, int64_t n) { pdma_lu_prog(data, n); }

template <class T>
__global__ void k_tdma_solve(T* u, const double* data, int64_t n, int64_t inner, int64_t nsys) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) tdma_solve_prog<T>(u, data, n, inner, s);
}

template <class T>
__global__ void k_pdma_solve(T* u, const double* data, int64_t n, int64_t inner, int64_t nsys) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) pdma_solve_prog<T>(u, data, n, inner, s);
}

__global__ void k_helmholtz_lu(int64_t N, const double* alfa, const double* beta, int neumann,
                               double* d0, double* d1, double* d2, double* L, int64_t inner,
                               int64_t nsys) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) helmholtz_lu_prog(N, alfa, beta, neumann, d0, d1, d2, L, inner, s);
}

template <class T>
__global__ void k_helmholtz_solve(const T* b, T* u, int neumann, const double* d0, const double* d1,
                                  const double* d2, const double* L, int64_t N, int64_t inner,
                                  int64_t nsys) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) helmholtz_solve_prog<T>(b, u, neumann, d0, d1, d2, L, N, inner, s);
}

template <class T>
__global__ void k_helmholtz_neumann_matvec(const T* v, T* b, const double* alfa, const double* beta,
                                           int64_t N, int64_t inner, int64_t nsys) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) helmholtz_neumann_matvec_prog<T>(v, b, alfa, beta, N, inner, s);
}

template <class T>
__global__ void k_poisson_add(const T* b, T* u, double scale, int64_t N, int64_t inner, int64_t nsys) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) poisson_add_prog<T>(b, u, scale, N, inner, s);
}

template <class T>
__global__ void k_poisson_ann(const T* b, T* u, double scale, double c0, int64_t N, int64_t inner,
                              int64_t nsys) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) poisson_ann_prog<T>(b, u, scale, c0, N, inner, s);
}

template <class T>
__global__ void k_helmholtz_matvec(const T* v, T* b, const double* alfa, const double* beta,
                                   int64_t N, int64_t inner, int64_t nsys) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) helmholtz_matvec_prog<T>(v, b, alfa, beta, N, inner, s);
}

__global__ void k_banded_lu(double* data, BandDesc b, int64_t n) { banded_lu_prog(data, b, n); }

template <class T>
__global__ void k_banded_solve(T* u, const double* data, BandDesc b, int64_t n, int64_t inner, int64_t nsys) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) banded_solve_prog<T>(u, data, b, n, inner, s);
}

namespace {
// offsets: 1..9 values, ascending, with 0 and every value between the first
// and the last, all even (steps of 2) or consecutive (steps of 1, as
// TDMA_O's -1, 0, 1): elimination fills in only inside the band
int band_desc(int ndiag, const int* offsets, int64_t n, BandDesc* b) {
  if (!offsets || ndiag < 1 || ndiag > 9 || n < 1) return SGPU_ERR_ARG;
  b->nd = ndiag;
  bool even = true;
  for (int r = 0; r < ndiag; ++r) even = even && offsets[r] % 2 == 0;
  const int step = even ? 2 : 1;
  for (int r = 0; r < ndiag; ++r) {
    const int o = offsets[r];
    if ((r > 0 && o != offsets[r - 1] + step) || (o < 0 ? -o : o) >= n) return SGPU_ERR_ARG;
    b->off[r] = o;
  }
  if (offsets[0] > 0 || offsets[ndiag - 1] < 0) return SGPU_ERR_ARG;
  return SGPU_OK;
}
}  // namespace

extern "C" int sgpu_banded_LU(double* data, int ndiag, const int* offsets, int64_t n, cudaStream_t stream) {
  BandDesc b;
  if (!data) return SGPU_ERR_ARG;
  const int st = band_desc(ndiag, offsets, n, &b);
  if (st != SGPU_OK) return st;
  k_banded_lu<<<1, 1, 0, stream>>>(data, b, n);
  return finish();
}

extern "C" int sgpu_banded_Solve(void* u, const double* data, int ndiag, const int* offsets, int64_t outer,
                                 int64_t n, int64_t inner, int data_kind, cudaStream_t stream) {
  BandDesc b;
  if (!u || !data || outer < 0 || inner < 1) return SGPU_ERR_ARG;
  const int st = band_desc(ndiag, offsets, n, &b);
  if (st != SGPU_OK) return st;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  if (data_kind == SGPU_COMPLEX)
    k_banded_solve<cd><<<nblk(nsys), kThreads, 0, stream>>>((cd*)u, data, b, n, inner, nsys);
  else if (data_kind == SGPU_REAL)
    k_banded_solve<double><<<nblk(nsys), kThreads, 0, stream>>>((double*)u, data, b, n, inner, nsys);
  else
    return SGPU_ERR_ARG;
  return finish();
}

extern "C" int sgpu_TDMA_LU(double* data, int64_t n, cudaStream_t stream) {
  if (!data || n < 3) return SGPU_ERR_ARG;
  k_tdma_lu<<<1, 1, 0, stream>>>(data, n);
  return finish();
}

extern "C" int sgpu_PDMA_LU(double* data, int64_t n, cudaStream_t stream) {
  if (!data || n < 5) return SGPU_ERR_ARG;
  k_pdma_lu<<<1, 1, 0, stream>>>(data, n);
  return finish();
}

extern "C" int sgpu_TDMA_Solve(void* u, const double* data, int64_t outer, int64_t n,
                               int64_t inner, int data_kind, cudaStream_t stream) {
  if (!u || !data || n < 3 || outer < 0 || inner < 1) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  if (data_kind == SGPU_COMPLEX)
    k_tdma_solve<cd><<<nblk(nsys), kThreads, 0, stream>>>((cd*)u, data, n, inner, nsys);
  else if (data_kind == SGPU_REAL)
    k_tdma_solve<double><<<nblk(nsys), kThreads, 0, stream>>>((double*)u, data, n, inner, nsys);
  else
    return SGPU_ERR_ARG;
  return finish();
}

extern "C" int sgpu_PDMA_Solve(void* u, const double* data, int64_t outer, int64_t n,
                               int64_t inner, int data_kind, cudaStream_t stream) {
  if (!u || !data || n < 5 || outer < 0 || inner < 1) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  if (data_kind == SGPU_COMPLEX)
    k_pdma_solve<cd><<<nblk(nsys), kThreads, 0, stream>>>((cd*)u, data, n, inner, nsys);
  else if (data_kind == SGPU_REAL)
    k_pdma_solve<double><<<nblk(nsys), kThreads, 0, stream>>>((double*)u, data, n, inner, nsys);
  else
    return SGPU_ERR_ARG;
  return finish();
}

extern "C" int sgpu_LU_Helmholtz(int64_t N, const double* alfa, const double* beta, int neumann,
                                 double* d0, double* d1, double* d2, double* L, int64_t outer,
                                 int64_t inner, cudaStream_t stream) {
  if (!alfa || !beta || !d0 || !d1 || !d2 || !L || N < 8 || outer < 0 || inner < 1 ||
      (neumann != 0 && neumann != 1))
    return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  k_helmholtz_lu<<<nblk(nsys), kThreads, 0, stream>>>(N, alfa, beta, neumann, d0, d1, d2, L, inner, nsys);
  return finish();
}

extern "C" int sgpu_Solve_Helmholtz(const void* b, void* u, int neumann, const double* d0,
                                    const double* d1, const double* d2, const double* L,
                                    int64_t outer, int64_t N, int64_t inner, int data_kind,
                                    cudaStream_t stream) {
  if (!b || !u || !d0 || !d1 || !d2 || !L || N < 8 || outer < 0 || inner < 1 ||
      (neumann != 0 && neumann != 1))
    return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  if (data_kind == SGPU_COMPLEX)
    k_helmholtz_solve<cd><<<nblk(nsys), kThreads, 0, stream>>>((const cd*)b, (cd*)u, neumann, d0, d1,
                                                               d2, L, N, inner, nsys);
  else if (data_kind == SGPU_REAL)
    k_helmholtz_solve<double><<<nblk(nsys), kThreads, 0, stream>>>(
        (const double*)b, (double*)u, neumann, d0, d1, d2, L, N, inner, nsys);
  else
    return SGPU_ERR_ARG;
  return finish();
}

extern "C" int sgpu_Helmholtz_matvec(const void* v, void* b, const double* alfa,
                                     const double* beta, int64_t outer, int64_t N, int64_t inner,
                                     int data_kind, cudaStream_t stream) {
  if (!v || !b || !alfa || !beta || N < 8 || outer < 0 || inner < 1) return SGPU_ERR_ARG;
  if (v == b) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  if (data_kind == SGPU_COMPLEX)
    k_helmholtz_matvec<cd><<<nblk(nsys), kThreads, 0, stream>>>((const cd*)v, (cd*)b, alfa, beta,
                                                                N, inner, nsys);
  else if (data_kind == SGPU_REAL)
    k_helmholtz_matvec<double><<<nblk(nsys), kThreads, 0, stream>>>(
        (const double*)v, (double*)b, alfa, beta, N, inner, nsys);
  else
    return SGPU_ERR_ARG;
  return finish();
}

extern "C" int sgpu_Helmholtz_Neumann_matvec(const void* v, void* b, const double* alfa,
                                             const double* beta, int64_t outer, int64_t N,
                                             int64_t inner, int data_kind, cudaStream_t stream) {
  if (!v || !b || !alfa || !beta || N < 8 || outer < 0 || inner < 1) return SGPU_ERR_ARG;
  if (v == b) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  if (data_kind == SGPU_COMPLEX)
    k_helmholtz_neumann_matvec<cd><<<nblk(nsys), kThreads, 0, stream>>>((const cd*)v, (cd*)b, alfa,
                                                                        beta, N, inner, nsys);
  else if (data_kind == SGPU_REAL)
    k_helmholtz_neumann_matvec<double><<<nblk(nsys), kThreads, 0, stream>>>(
        (const double*)v, (double*)b, alfa, beta, N, inner, nsys);
  else
    return SGPU_ERR_ARG;
  return finish();
}

extern "C" int sgpu_Poisson_Solve_ADD(const void* b, void* u, double scale, int64_t outer, int64_t N,
                                      int64_t inner, int data_kind, cudaStream_t stream) {
  if (!b || !u || N < 5 || outer < 0 || inner < 1 || !(scale != 0.0)) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  if (data_kind == SGPU_COMPLEX)
    k_poisson_add<cd><<<nblk(nsys), kThreads, 0, stream>>>((const cd*)b, (cd*)u, scale, N, inner, nsys);
  else if (data_kind == SGPU_REAL)
    k_poisson_add<double><<<nblk(nsys), kThreads, 0, stream>>>((const double*)b, (double*)u, scale, N,
                                                              inner, nsys);
  else
    return SGPU_ERR_ARG;
  return finish();
}

extern "C" int sgpu_Poisson_Solve_ANN(const void* b, void* u, double scale, double u0, int64_t outer,
                                      int64_t N, int64_t inner, int data_kind, cudaStream_t stream) {
  if (!b || !u || N < 5 || outer < 0 || inner < 1 || !(scale != 0.0)) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  if (data_kind == SGPU_COMPLEX)
    k_poisson_ann<cd><<<nblk(nsys), kThreads, 0, stream>>>((const cd*)b, (cd*)u, scale, u0, N, inner,
                                                           nsys);
  else if (data_kind == SGPU_REAL)
    k_poisson_ann<double><<<nblk(nsys), kThreads, 0, stream>>>((const double*)b, (double*)u, scale, u0,
                                                              N, inner, nsys);
  else
    return SGPU_ERR_ARG;
  return finish();
}

// ---- factorisation cache + cached solve (both forms) -----------------------
template <class R>
__global__ void k_helmholtz_factor(int64_t N, const double* alfa, const double* beta, int neumann,
                                   R* fac, int64_t nsys) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) helmholtz_factor_prog<R>(N, alfa, beta, neumann, fac, nsys, s);
}

template <class R, class T>
__global__ void k_helmholtz_cached(const T* b, T* u, const R* fac, int neumann, int64_t N,
                                   int64_t inner, int64_t nsys) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 2 * nsys)
    helmholtz_cached_solve_prog<R, T>(b, u, fac, neumann, N, inner, nsys, t >> 1, (int)(t & 1));
}

template <class R, class T>
__global__ void k_helmholtz_refine(const T* b, T* u, T* r, const float* fac, const double* alfa, const double* beta,
                                   int64_t N, int64_t inner, int64_t nsys, double tol, int max_it, int* iters) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 2 * nsys) {
    const int it = helmholtz_refine_prog<R, T>(b, u, r, fac, alfa, beta, N, inner, nsys, t >> 1, (int)(t & 1), tol,
                                               max_it);
    if (iters) iters[t] = it;
  }
}

extern "C" int sgpu_helmholtz_solve_refined(const void* b, void* u, void* r, const void* fac32, const double* alfa,
                                            const double* beta, int64_t outer, int64_t N, int64_t inner,
                                            int data_kind, double tol, int max_it, int residual_form, int* iters,
                                            cudaStream_t stream) {
  if (!b || !u || !r || !fac32 || !alfa || !beta || N < 8 || outer < 0 || inner < 1 || max_it < 0 || !(tol >= 0))
    return SGPU_ERR_ARG;
  if (b == u || b == r || u == r) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  const unsigned nb = nblk(2 * nsys);
  const float* f32 = (const float*)fac32;
  if (residual_form == SGPU_PLAIN_F64 && data_kind == SGPU_COMPLEX)
    k_helmholtz_refine<double, cd><<<nb, kThreads, 0, stream>>>((const cd*)b, (cd*)u, (cd*)r, f32, alfa, beta, N, inner,
                                                               nsys, tol, max_it, iters);
  else if (residual_form == SGPU_PLAIN_F64 && data_kind == SGPU_REAL)
    k_helmholtz_refine<double, double><<<nb, kThreads, 0, stream>>>((const double*)b, (double*)u, (double*)r, f32, alfa,
                                                                   beta, N, inner, nsys, tol, max_it, iters);
  else if (residual_form == SGPU_MIXED_DF && data_kind == SGPU_COMPLEX)
    k_helmholtz_refine<df, cd><<<nb, kThreads, 0, stream>>>((const cd*)b, (cd*)u, (cd*)r, f32, alfa, beta, N, inner,
                                                           nsys, tol, max_it, iters);
  else if (residual_form == SGPU_MIXED_DF && data_kind == SGPU_REAL)
    k_helmholtz_refine<df, double><<<nb, kThreads, 0, stream>>>((const double*)b, (double*)u, (double*)r, f32, alfa,
                                                               beta, N, inner, nsys, tol, max_it, iters);
  else
    return SGPU_ERR_ARG;
  return finish();
}

extern "C" int sgpu_helmholtz_factor(int64_t N, const double* alfa, const double* beta, int neumann,
                                     int64_t outer, int64_t inner, int form, void* fac,
                                     cudaStream_t stream) {
  if (!alfa || !beta || !fac || N < 8 || outer < 0 || inner < 1 || (neumann != 0 && neumann != 1))
    return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  if (form == SGPU_PLAIN_F64)
    k_helmholtz_factor<double><<<nblk(nsys), kThreads, 0, stream>>>(N, alfa, beta, neumann, (double*)fac, nsys);
  else if (form == SGPU_MIXED_DF)
    k_helmholtz_factor<df><<<nblk(nsys), kThreads, 0, stream>>>(N, alfa, beta, neumann, (df*)fac, nsys);
  else if (form == SGPU_FP32_REFINED && neumann == 0)
    k_helmholtz_factor<float><<<nblk(nsys), kThreads, 0, stream>>>(N, alfa, beta, neumann, (float*)fac, nsys);
  else
    return SGPU_ERR_ARG;
  return finish();
}

// Problems of few systems: one CTA of 64 threads per system.  The system's
// right-hand side and factor rows are gathered into shared memory (every
// thread a few independent loads: one memory round trip), threads 0 and 1
// run the two parity chains' program from there, and the dof rows are
// written back (rows M, M+1 of u keep their contents, as in the one-thread-
// per-chain kernel).  With few systems that kernel runs all chains on one or
// a few SMs, each chain a sequence of dependent memory round trips and all
// of them sharing an SM's FP64 units; here every system gets an SM's share.
template <class R, class T>
__global__ void __launch_bounds__(64) k_helmholtz_cached_sys(const T* b, T* u, const R* fac, int neumann, int64_t N,
                                                             int64_t inner, int64_t nsys) {
  extern __shared__ __align__(16) unsigned char hs_smem[];
  const int64_t s = (int64_t)blockIdx.x, M = N - 2;
  T* sb = (T*)hs_smem;
  T* su = sb + N;
  R* sf = (R*)(su + N);
  const int64_t base = sys_base(s, N, inner);
  const int tid = (int)threadIdx.x, nth = (int)blockDim.x;
  for (int64_t i0 = 0; i0 < N; i0 += 4 * nth) {
    T v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t i = i0 + tid + j * nth;
      if (i < N) v[j] = b[base + i * inner];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t i = i0 + tid + j * nth;
      if (i < N) sb[i] = v[j];
    }
  }
  for (int64_t i0 = 0; i0 < 4 * M; i0 += 4 * nth) {
    R v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t i = i0 + tid + j * nth;
      if (i < 4 * M) v[j] = fac[i * nsys + s];  // row (q, k) = i of the interleaved cache
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t i = i0 + tid + j * nth;
      if (i < 4 * M) sf[i] = v[j];
    }
  }
  __syncthreads();
  if (tid < 2) helmholtz_cached_solve_prog<R, T>(sb, su, sf, neumann, N, 1, 1, 0, tid);
  __syncthreads();
  for (int64_t i = tid; i < M; i += nth) u[base + i * inner] = su[i];
}

// the per-system kernel for up to 4,096 systems (SGPU_ERR_UNSUPPORTED above)
template <class R, class T>
int launch_sys_solve(const T* b, T* u, const R* fac, int neumann, int64_t N, int64_t inner, int64_t nsys,
                     cudaStream_t stream) {
  const size_t smem = 2 * (size_t)N * sizeof(T) + 4 * (size_t)(N - 2) * sizeof(R);
  if (nsys > 4096 || smem > 48 * 1024) return SGPU_ERR_UNSUPPORTED;
  k_helmholtz_cached_sys<R, T><<<(unsigned)nsys, 64, smem, stream>>>(b, u, fac, neumann, N, inner, nsys);
  return finish();
}

extern "C" int sgpu_helmholtz_solve_cached(const void* b, void* u, const void* fac, int neumann,
                                           int64_t outer, int64_t N, int64_t inner, int data_kind,
                                           int form, cudaStream_t stream) {
  if (!b || !u || !fac || N < 8 || outer < 0 || inner < 1 || (neumann != 0 && neumann != 1))
    return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  const unsigned nb = nblk(2 * nsys);
  const int nm = neumann;
  {
    int st = SGPU_ERR_UNSUPPORTED;
    if (form == SGPU_PLAIN_F64 && data_kind == SGPU_COMPLEX)
      st = launch_sys_solve<double, cd>((const cd*)b, (cd*)u, (const double*)fac, nm, N, inner, nsys, stream);
    else if (form == SGPU_PLAIN_F64 && data_kind == SGPU_REAL)
      st = launch_sys_solve<double, double>((const double*)b, (double*)u, (const double*)fac, nm, N, inner, nsys,
                                            stream);
    else if (form == SGPU_MIXED_DF && data_kind == SGPU_COMPLEX)
      st = launch_sys_solve<df, cd>((const cd*)b, (cd*)u, (const df*)fac, nm, N, inner, nsys, stream);
    else if (form == SGPU_MIXED_DF && data_kind == SGPU_REAL)
      st = launch_sys_solve<df, double>((const double*)b, (double*)u, (const df*)fac, nm, N, inner, nsys, stream);
    if (st != SGPU_ERR_UNSUPPORTED) return st;
  }
  if (form == SGPU_PLAIN_F64 && data_kind == SGPU_COMPLEX)
    k_helmholtz_cached<double, cd><<<nb, kThreads, 0, stream>>>((const cd*)b, (cd*)u, (const double*)fac, nm, N, inner, nsys);
  else if (form == SGPU_PLAIN_F64 && data_kind == SGPU_REAL)
    k_helmholtz_cached<double, double><<<nb, kThreads, 0, stream>>>((const double*)b, (double*)u, (const double*)fac, nm, N, inner, nsys);
  else if (form == SGPU_MIXED_DF && data_kind == SGPU_COMPLEX)
    k_helmholtz_cached<df, cd><<<nb, kThreads, 0, stream>>>((const cd*)b, (cd*)u, (const df*)fac, nm, N, inner, nsys);
  else if (form == SGPU_MIXED_DF && data_kind == SGPU_REAL)
    k_helmholtz_cached<df, double><<<nb, kThreads, 0, stream>>>((const double*)b, (double*)u, (const df*)fac, nm, N, inner, nsys);
  else
    return SGPU_ERR_ARG;
  return finish();
}

// Batches of problems of one shape (serving): member k's systems are at
// b + k nsys N with their own factor cache facs[k] (a device array of K
// pointers); one thread per (system, parity) of every member.
template <class R, class T>
__global__ void k_helmholtz_cached_batch(const T* b, T* u, const void* const* facs, int neumann, int64_t N,
                                         int64_t inner, int64_t nsys, int K) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * nsys * K) return;
  const int64_t c = t >> 1;
  const int k = (int)(c / nsys);
  const int64_t s = c - (int64_t)k * nsys, off = (int64_t)k * nsys * N;
  helmholtz_cached_solve_prog<R, T>(b + off, u + off, (const R*)facs[k], neumann, N, inner, nsys, s, (int)(t & 1));
}

extern "C" int sgpu_helmholtz_solve_cached_batch(const void* b, void* u, const void* const* facs, int K, int neumann,
                                                 int64_t outer, int64_t N, int64_t inner, int data_kind, int form,
                                                 cudaStream_t stream) {
  if (!b || !u || !facs || K < 1 || N < 8 || outer < 0 || inner < 1 || (neumann != 0 && neumann != 1))
    return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  const unsigned nb = nblk(2 * nsys * K);
  if (form == SGPU_PLAIN_F64 && data_kind == SGPU_COMPLEX)
    k_helmholtz_cached_batch<double, cd><<<nb, kThreads, 0, stream>>>((const cd*)b, (cd*)u, facs, neumann, N, inner,
                                                                      nsys, K);
  else if (form == SGPU_PLAIN_F64 && data_kind == SGPU_REAL)
    k_helmholtz_cached_batch<double, double><<<nb, kThreads, 0, stream>>>((const double*)b, (double*)u, facs, neumann,
                                                                          N, inner, nsys, K);
  else if (form == SGPU_MIXED_DF && data_kind == SGPU_COMPLEX)
    k_helmholtz_cached_batch<df, cd><<<nb, kThreads, 0, stream>>>((const cd*)b, (cd*)u, facs, neumann, N, inner, nsys,
                                                                  K);
  else if (form == SGPU_MIXED_DF && data_kind == SGPU_REAL)
    k_helmholtz_cached_batch<df, double><<<nb, kThreads, 0, stream>>>((const double*)b, (double*)u, facs, neumann, N,
                                                                      inner, nsys, K);
  else
    return SGPU_ERR_ARG;
  return finish();
}

// ---- banded + semiseparable per-wavenumber systems --------------------------
template <class F>
__global__ void k_band_sep_factor(BandSepDesc d, F* fac, int64_t nsys) {
  int64_t ch = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (ch < 2 * nsys) band_sep_factor_prog<F>(d, fac, nsys, ch);
}

template <class T>
__global__ void k_band_sep_refine(BandSepDesc d, const T* b, T* u, T* r, const float* fac, int64_t Nb, int64_t inner,
                                  int64_t nsys, double tol, int max_it, int* iters) {
  int64_t ch = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (ch < 2 * nsys) {
    const int it = band_sep_refine_prog<T>(d, b, u, r, fac, Nb, inner, nsys, ch, tol, max_it);
    if (iters) iters[ch] = it;
  }
}

template <class T>
__global__ void k_band_sep_solve(const T* b, T* u, const double* fac, const double* gens, int n,
                                 int64_t Nb, int64_t inner, int64_t nsys) {
  int64_t ch = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (ch < 2 * nsys) band_sep_solve_prog<T>(b, u, fac, gens, n, Nb, inner, nsys, ch);
}

extern "C" int sgpu_band_sep_factor(int n, int nterms, int gen_term, const double* bands,
                                    const double* gens, const double* coef, int64_t nsys,
                                    double* fac, cudaStream_t stream) {
  if (n < 2 || nterms < 1 || nterms > 3 || gen_term >= nterms || !bands || !coef || !fac ||
      nsys < 0)
    return SGPU_ERR_ARG;
  if ((gen_term >= 0) != (gens != nullptr)) return SGPU_ERR_ARG;
  if (nsys == 0) return SGPU_OK;
  BandSepDesc d{n, nterms, gen_term, bands, gens, coef};
  k_band_sep_factor<double><<<nblk(2 * nsys), kThreads, 0, stream>>>(d, fac, nsys);
  return finish();
}

extern "C" int sgpu_band_sep_factor32(int n, int nterms, int gen_term, const double* bands, const double* gens,
                                      const double* coef, int64_t nsys, float* fac, cudaStream_t stream) {
  if (n < 2 || nterms < 1 || nterms > 3 || gen_term >= nterms || !bands || !coef || !fac || nsys < 0)
    return SGPU_ERR_ARG;
  if ((gen_term >= 0) != (gens != nullptr)) return SGPU_ERR_ARG;
  if (nsys == 0) return SGPU_OK;
  BandSepDesc d{n, nterms, gen_term, bands, gens, coef};
  k_band_sep_factor<float><<<nblk(2 * nsys), kThreads, 0, stream>>>(d, fac, nsys);
  return finish();
}

extern "C" int sgpu_band_sep_solve_refined(const void* b, void* u, void* r, const float* fac32, int n, int nterms,
                                           int gen_term, const double* bands, const double* gens, const double* coef,
                                           int64_t outer, int64_t Nb, int64_t inner, int data_kind, double tol,
                                           int max_it, int* iters, cudaStream_t stream) {
  if (!b || !u || !r || !fac32 || n < 2 || Nb < n || nterms < 1 || nterms > 3 || gen_term >= nterms || !bands ||
      !coef || outer < 0 || inner < 1 || max_it < 0 || !(tol >= 0))
    return SGPU_ERR_ARG;
  if ((gen_term >= 0) != (gens != nullptr)) return SGPU_ERR_ARG;
  if (b == u || b == r || u == r) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  BandSepDesc d{n, nterms, gen_term, bands, gens, coef};
  if (data_kind == SGPU_COMPLEX)
    k_band_sep_refine<cd><<<nblk(2 * nsys), kThreads, 0, stream>>>(d, (const cd*)b, (cd*)u, (cd*)r, fac32, Nb, inner,
                                                                   nsys, tol, max_it, iters);
  else if (data_kind == SGPU_REAL)
    k_band_sep_refine<double><<<nblk(2 * nsys), kThreads, 0, stream>>>(d, (const double*)b, (double*)u, (double*)r,
                                                                       fac32, Nb, inner, nsys, tol, max_it, iters);
  else
    return SGPU_ERR_ARG;
  return finish();
}

template <class T>
__global__ void k_band_sep_matvec(BandSepDesc d, const T* v, T* c, int64_t Nb, int64_t inner, int64_t nsys) {
  int64_t ch = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (ch < 2 * nsys) band_sep_matvec_prog<T>(d, v, c, Nb, inner, nsys, ch);
}

extern "C" int sgpu_band_sep_matvec(const void* v, void* c, int n, int nterms, int gen_term,
                                    const double* bands, const double* gens, const double* coef,
                                    int64_t outer, int64_t Nb, int64_t inner, int data_kind,
                                    cudaStream_t stream) {
  if (!v || !c || v == c || n < 2 || Nb < n || nterms < 1 || nterms > 3 || gen_term >= nterms ||
      !bands || !coef || outer < 0 || inner < 1)
    return SGPU_ERR_ARG;
  if ((gen_term >= 0) != (gens != nullptr)) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  BandSepDesc d{n, nterms, gen_term, bands, gens, coef};
  if (data_kind == SGPU_COMPLEX)
    k_band_sep_matvec<cd><<<nblk(2 * nsys), kThreads, 0, stream>>>(d, (const cd*)v, (cd*)c, Nb, inner, nsys);
  else if (data_kind == SGPU_REAL)
    k_band_sep_matvec<double><<<nblk(2 * nsys), kThreads, 0, stream>>>(d, (const double*)v, (double*)c, Nb,
                                                                       inner, nsys);
  else
    return SGPU_ERR_ARG;
  return finish();
}

extern "C" int sgpu_band_sep_solve(const void* b, void* u, const double* fac, const double* gens,
                                   int n, int64_t outer, int64_t Nb, int64_t inner, int data_kind,
                                   cudaStream_t stream) {
  if (!b || !u || !fac || n < 2 || Nb < n || outer < 0 || inner < 1) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  if (data_kind == SGPU_COMPLEX)
    k_band_sep_solve<cd><<<nblk(2 * nsys), kThreads, 0, stream>>>((const cd*)b, (cd*)u, fac, gens, n, Nb, inner, nsys);
  else if (data_kind == SGPU_REAL)
    k_band_sep_solve<double><<<nblk(2 * nsys), kThreads, 0, stream>>>((const double*)b, (double*)u, fac, gens, n, Nb, inner, nsys);
  else
    return SGPU_ERR_ARG;
  return finish();
}

template <class T>
__global__ void k_band_sep_solve_batch(const T* b, T* u, const double* const* facs, const double* gens, int n,
                                       int64_t Nb, int64_t inner, int64_t nsys, int K) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * nsys * K) return;
  const int k = (int)(t / (2 * nsys));
  const int64_t ch = t - (int64_t)k * 2 * nsys, off = (int64_t)k * nsys * Nb;
  band_sep_solve_prog<T>(b + off, u + off, facs[k], gens, n, Nb, inner, nsys, ch);
}

extern "C" int sgpu_band_sep_solve_batch(const void* b, void* u, const double* const* facs, const double* gens, int K,
                                         int n, int64_t outer, int64_t Nb, int64_t inner, int data_kind,
                                         cudaStream_t stream) {
  if (!b || !u || !facs || K < 1 || n < 2 || Nb < n || outer < 0 || inner < 1) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  const unsigned nb = nblk(2 * nsys * K);
  if (data_kind == SGPU_COMPLEX)
    k_band_sep_solve_batch<cd><<<nb, kThreads, 0, stream>>>((const cd*)b, (cd*)u, facs, gens, n, Nb, inner, nsys, K);
  else if (data_kind == SGPU_REAL)
    k_band_sep_solve_batch<double><<<nb, kThreads, 0, stream>>>((const double*)b, (double*)u, facs, gens, n, Nb, inner,
                                                                nsys, K);
  else
    return SGPU_ERR_ARG;
  return finish();
}
