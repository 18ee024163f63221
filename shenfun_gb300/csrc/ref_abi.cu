// C ABI of the reference-signature entry points (ref_progs.cuh has the
// algorithms): the names shenfun's optimization modules export for the
// biharmonic solver, SolverGeneric1ND's per-wavenumber banded solves and the
// recursive Legendre transforms, taking the reference's argument arrays in
// its layouts (device pointers; one thread per system or per (system,
// parity) chain).
#include "ref_progs.cuh"
#include "shenfun_gb300.h"

using namespace sgpu;
using namespace sgpu::ref;

namespace sgpu {
int line_gemm_f64(const double* in, double* out, const double* M, int Nin, int Nout, int64_t nrows,
                  int64_t inner, int cplx, cudaStream_t stream, const double* lscale, int accumulate);
}

namespace {

const int kThreads = 128;

inline int finish() { return cudaGetLastError() == cudaSuccess ? SGPU_OK : SGPU_ERR_CUDA; }
inline unsigned nblk(int64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

bool diags_ok(const BihDiags& d) {
  return d.sii && d.siu && d.siuu && d.ail && d.aii && d.aiu && d.bill && d.bil && d.bii && d.biu && d.biuu;
}

}  // namespace

__global__ void k_ref_bih_lu(BihDiags d, double a0, const double* alfa, const double* beta, double* u0,
                             double* u1, double* u2, double* l0, double* l1, int64_t M, int64_t inner,
                             int64_t nsys) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < 2 * nsys) bih_lu_chain(c, nsys, d, a0, alfa, beta, u0, u1, u2, l0, l1, M, inner);
}

__global__ void k_ref_bih_factor_pr(double* ak, double* bk, const double* l0, const double* l1, int64_t M,
                                    int64_t inner, int64_t nsys) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < 2 * nsys) bih_factor_pr_chain(c, nsys, ak, bk, l0, l1, M, inner);
}

template <class T>
__global__ void k_ref_bih_solve(const T* f, T* u, const double* u0, const double* u1, const double* u2,
                                const double* l0, const double* l1, const double* ak, const double* bk,
                                double a0, int64_t N, int64_t M, int64_t inner, int64_t nsys) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < 2 * nsys) bih_solve_chain<T>(c, nsys, f, u, u0, u1, u2, l0, l1, ak, bk, a0, N, M, inner);
}

template <class T>
__global__ void k_ref_bih_matvec(const T* v, T* b, BihDiags d, double a0, const double* alfa,
                                 const double* beta, int64_t N, int64_t M, int64_t inner, int64_t nsys) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) bih_matvec_sys<T>(s, v, b, d, a0, alfa, beta, N, M, inner);
}

template <class T>
__global__ void k_ref_dma_solve(int kind, T* u, const double* data, int64_t dstride, int64_t cols, int64_t N,
                                int64_t inner, int64_t nsys, int skip_first) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys && !(skip_first && s == 0)) dma_solve_sys<T>(s, kind, u, data, dstride, cols, N, inner);
}

__global__ void k_ref_leg_matrix(const double* x, const double* w, const double* a, int rows, int64_t cols,
                                 int64_t n, int64_t npts, double* M, int scalar) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < npts) legendre_matrix_point(j, scalar, x, w, a, rows, cols, n, npts, M);
}

extern "C" int sgpu_LU_Biharmonic(double a0, const double* alfa, const double* beta, const double* sii,
                                  const double* siu, const double* siuu, const double* ail, const double* aii,
                                  const double* aiu, const double* bill, const double* bil, const double* bii,
                                  const double* biu, const double* biuu, double* u0, double* u1, double* u2,
                                  double* l0, double* l1, int64_t outer, int64_t M, int64_t inner,
                                  cudaStream_t stream) {
  const BihDiags d{sii, siu, siuu, ail, aii, aiu, bill, bil, bii, biu, biuu};
  if (!diags_ok(d) || !alfa || !beta || !u0 || !u1 || !u2 || !l0 || !l1) return SGPU_ERR_ARG;
  if (outer < 0 || inner < 1 || M < 5) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  k_ref_bih_lu<<<nblk(2 * nsys), kThreads, 0, stream>>>(d, a0, alfa, beta, u0, u1, u2, l0, l1, M, inner, nsys);
  return finish();
}

extern "C" int sgpu_Biharmonic_factor_pr(double* ak, double* bk, const double* l0, const double* l1,
                                         int64_t outer, int64_t M, int64_t inner, cudaStream_t stream) {
  if (!ak || !bk || !l0 || !l1 || outer < 0 || inner < 1 || M < 5) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  k_ref_bih_factor_pr<<<nblk(2 * nsys), kThreads, 0, stream>>>(ak, bk, l0, l1, M, inner, nsys);
  return finish();
}

extern "C" int sgpu_Biharmonic_Solve(const void* b, void* u, const double* u0, const double* u1,
                                     const double* u2, const double* l0, const double* l1, const double* ak,
                                     const double* bk, double a0, int64_t outer, int64_t N, int64_t inner,
                                     int64_t M, int data_kind, cudaStream_t stream) {
  if (!b || !u || !u0 || !u1 || !u2 || !l0 || !l1 || !ak || !bk) return SGPU_ERR_ARG;
  if (outer < 0 || inner < 1 || M < 5 || 2 * M > N) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  const unsigned g = nblk(2 * nsys);
  if (data_kind == SGPU_COMPLEX)
    k_ref_bih_solve<cd><<<g, kThreads, 0, stream>>>((const cd*)b, (cd*)u, u0, u1, u2, l0, l1, ak, bk, a0, N, M,
                                                    inner, nsys);
  else if (data_kind == SGPU_REAL)
    k_ref_bih_solve<double><<<g, kThreads, 0, stream>>>((const double*)b, (double*)u, u0, u1, u2, l0, l1, ak,
                                                        bk, a0, N, M, inner, nsys);
  else
    return SGPU_ERR_ARG;
  return finish();
}

extern "C" int sgpu_Biharmonic_matvec(const void* v, void* b, double a0, const double* alfa, const double* beta,
                                      const double* sii, const double* siu, const double* siuu, const double* ail,
                                      const double* aii, const double* aiu, const double* bill, const double* bil,
                                      const double* bii, const double* biu, const double* biuu, int64_t outer,
                                      int64_t N, int64_t inner, int64_t M, int data_kind, cudaStream_t stream) {
  const BihDiags d{sii, siu, siuu, ail, aii, aiu, bill, bil, bii, biu, biuu};
  if (!v || !b || v == b || !alfa || !beta || !diags_ok(d)) return SGPU_ERR_ARG;
  if (outer < 0 || inner < 1 || M < 10 || M > N) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  if (data_kind == SGPU_COMPLEX)
    k_ref_bih_matvec<cd><<<nblk(nsys), kThreads, 0, stream>>>((const cd*)v, (cd*)b, d, a0, alfa, beta, N, M, inner,
                                                              nsys);
  else if (data_kind == SGPU_REAL)
    k_ref_bih_matvec<double><<<nblk(nsys), kThreads, 0, stream>>>((const double*)v, (double*)b, d, a0, alfa, beta,
                                                                  N, M, inner, nsys);
  else
    return SGPU_ERR_ARG;
  return finish();
}

namespace {
int dma_launch(int sol, void* u, const double* data, int64_t dstride, int64_t rows, int64_t cols, int64_t outer,
               int64_t N, int64_t inner, int skip_first, int data_kind, cudaStream_t stream) {
  if (!u || !data || sol < SGPU_SOL_DIAGMA || sol > SGPU_SOL_HEPTADMA) return SGPU_ERR_ARG;
  if (outer < 0 || inner < 1 || rows < dma_rows(sol) || cols < dma_min_cols(sol) || cols > N) return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  if (data_kind == SGPU_COMPLEX)
    k_ref_dma_solve<cd><<<nblk(nsys), kThreads, 0, stream>>>(sol, (cd*)u, data, dstride, cols, N, inner, nsys,
                                                             skip_first);
  else if (data_kind == SGPU_REAL)
    k_ref_dma_solve<double><<<nblk(nsys), kThreads, 0, stream>>>(sol, (double*)u, data, dstride, cols, N, inner,
                                                                 nsys, skip_first);
  else
    return SGPU_ERR_ARG;
  return finish();
}
}  // namespace

extern "C" int sgpu_SolverGeneric1ND_solve_data(void* u, const double* data, int sol, int is_zero_index,
                                                int64_t outer, int64_t N, int64_t inner, int64_t rows,
                                                int64_t cols, int data_kind, cudaStream_t stream) {
  return dma_launch(sol, u, data, rows * cols, rows, cols, outer, N, inner, is_zero_index ? 1 : 0, data_kind,
                    stream);
}

extern "C" int sgpu_DMA_Solve(int sol, void* u, const double* data, int64_t rows, int64_t cols, int64_t outer,
                              int64_t N, int64_t inner, int data_kind, cudaStream_t stream) {
  return dma_launch(sol, u, data, 0, rows, cols, outer, N, inner, 0, data_kind, stream);
}

namespace {
int legendre_recursive(int scalar, const void* in, void* out, const double* x, const double* w, const double* a,
                       int a_rows, int64_t a_cols, int64_t outer, int64_t Nin, int64_t Nout, int64_t inner,
                       int data_kind, void* work, size_t work_bytes, cudaStream_t stream) {
  if (!in || !out || in == out || !x || !a || (scalar && !w)) return SGPU_ERR_ARG;
  if (a_rows != 2 && a_rows != 3) return SGPU_ERR_ARG;
  if (outer < 0 || inner < 1 || Nin < 1 || Nout < 1 || Nin > 0x7fffffff || Nout > 0x7fffffff) return SGPU_ERR_ARG;
  if (data_kind != SGPU_REAL && data_kind != SGPU_COMPLEX) return SGPU_ERR_ARG;
  const int64_t n = scalar ? Nout : Nin;      // polynomial degrees
  const int64_t npts = scalar ? Nin : Nout;   // points
  if (a_cols < n + 2) return SGPU_ERR_ARG;
  const size_t mbytes = (size_t)n * (size_t)npts * sizeof(double);
  double* M = (double*)work;
  bool own = false;
  if (!M) {
    if (cudaMallocAsync((void**)&M, mbytes, stream) != cudaSuccess) {
      cudaGetLastError();
      return SGPU_ERR_NOMEM;
    }
    own = true;
  } else if (work_bytes < mbytes) {
    return SGPU_ERR_ARG;
  }
  k_ref_leg_matrix<<<nblk(npts), kThreads, 0, stream>>>(x, w, a, a_rows, a_cols, n, npts, M, scalar);
  int st = finish();
  const int64_t nrows = outer * inner * (data_kind == SGPU_COMPLEX ? 2 : 1);
  if (st == SGPU_OK)
    st = line_gemm_f64((const double*)in, (double*)out, M, (int)Nin, (int)Nout, nrows, inner,
                       data_kind == SGPU_COMPLEX, stream, nullptr, 0);
  if (own && cudaFreeAsync(M, stream) != cudaSuccess && st == SGPU_OK) st = SGPU_ERR_CUDA;
  return st;
}
}  // namespace

extern "C" int sgpu_scalar_product(const void* input, void* output, const double* x, const double* w,
                                   const double* a, int a_rows, int64_t a_cols, int64_t outer, int64_t N,
                                   int64_t inner, int data_kind, void* work, size_t work_bytes,
                                   cudaStream_t stream) {
  return legendre_recursive(1, input, output, x, w, a, a_rows, a_cols, outer, N, N, inner, data_kind, work,
                            work_bytes, stream);
}

extern "C" int sgpu_evaluate_expansion_all(const void* input, void* output, const double* x, const double* a,
                                           int a_rows, int64_t a_cols, int64_t outer, int64_t N, int64_t Nx,
                                           int64_t inner, int data_kind, void* work, size_t work_bytes,
                                           cudaStream_t stream) {
  return legendre_recursive(0, input, output, x, nullptr, a, a_rows, a_cols, outer, N, Nx, inner, data_kind,
                            work, work_bytes, stream);
}
