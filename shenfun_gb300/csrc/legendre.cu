// Legendre spaces (Gauss-Legendre quadrature): nodes/weights and the dense
// Vandermonde transforms of the plain FP64 form.
//
// The reference evaluates Legendre transforms with an O(N^2) three-term
// recurrence per line (transforms.pyx:175-325, the default 'recursive' kind)
// or a Vandermonde dot product (spectralbase.py:472-483, 539-549).  Both are
// the same dense contraction; here it is one GEMM per direction with the
// Shen stencil folded into a precomputed N x N matrix:
//   scalar product:  out = f . diag(w) V K^T      (V_jk = L_k(x_j))
//   backward:        u   = c . K V^T              (to_ortho folded in)
// K is the stencil matrix with the reference's convention that the constant
// entries of ShenDirichlet apply to every row (spectralbase.py:1504-1526), so
// the scalar product keeps the orthogonal coefficients in the tail rows.
// The matrices are built on the host in double-double (ddouble.h) and
// stored in FP64.
// Plain form: FP64 tiled GEMM (k_line_gemm_f64).  Mixed form: the same
// matrices split into BF16 digit slices and contracted on the tensor cores
// (ozaki_tc.cu), about 48 bits, for N <= 8192 (above 1024 as one exact
// contraction per K chunk of 1024, the chunks' results added in FP64).  The
// reference's fast transform for large N (Hale & Townsend's DLT, legendre/
// dlt.py:20-206: leg2cheb plus ~20 Taylor-term DCT/DSTs in FP64) does not
// pay on this part at these lengths: FP64 runs at ~1 TFLOP/s against
// ~0.6 PFLOP/s for the split-BF16 contraction.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "ddouble.h"
#include "lc_fused.h"
#include "ozaki_tc.h"
#include "solvers.cuh"

using namespace sgpu;

using ddm::dd;
using ddm::to_double;

namespace {
// run body(i) for i in [0, n) on up to 16 host threads (independent
// iterations only): the plan's double-double set-up is O(N^2)
template <class F>
void parallel_for(int n, F body) {
  const unsigned hw = std::thread::hardware_concurrency();
  const int nth = std::min(n, (int)std::max(1u, std::min(hw ? hw : 1u, 16u)));
  if (nth <= 1 || n < 64) {
    for (int i = 0; i < n; ++i) body(i);
    return;
  }
  std::vector<std::thread> pool;
  for (int t = 0; t < nth; ++t)
    pool.emplace_back([=]() {
      for (int i = t; i < n; i += nth) body(i);
    });
  for (auto& th : pool) th.join();
}
}  // namespace

// Gauss-Legendre nodes (ascending) and weights: Newton iteration on P_N from
// Tricomi's asymptotic initial guesses, P_N and P_N' by the three-term
// recurrence, first in FP64 and then two steps in double-double (Newton
// doubles the correct digits per step); Golub & Welsch 1969 give the same
// rule, the reference uses Bogaert's 2014 iteration-free method
// (legendre/fastgl).
namespace {
// P_N(z) and P_{N-1}(z)
template <class T>
void legendre_pn(int N, const T& z, T& pn, T& pm) {
  T p0 = T(1.0), p1 = z;
  for (int k = 2; k <= N; ++k) {
    T p2 = ((double)(2 * k - 1) * z * p1 - (double)(k - 1) * p0) / (double)k;
    p0 = p1;
    p1 = p2;
  }
  if (N == 1) {
    p1 = z;
    p0 = T(1.0);
  }
  pn = p1;
  pm = p0;
}
}  // namespace

extern "C" int sgpu_leggauss(int N, double* x, double* w) {
  if (N < 1 || !x || !w) return SGPU_ERR_ARG;
  const double pi = 3.14159265358979323846;
  parallel_for((N + 1) / 2, [=](int i) {
    // i-th largest root
    const double th = pi * (4.0 * (i + 1) - 1) / (4.0 * N + 2);
    double z = std::cos(th) * (1 - (N - 1.0) / (8.0 * N * N * N));
    for (int it = 0; it < 100; ++it) {
      double pn, pm;
      legendre_pn(N, z, pn, pm);
      const double dz = pn / (N * (z * pn - pm) / (z * z - 1));
      z -= dz;
      if (std::fabs(dz) < 1e-14) break;
    }
    dd zd(z), pn, pm;
    for (int it = 0; it < 2; ++it) {
      legendre_pn(N, zd, pn, pm);
      const dd pp = (double)N * (zd * pn - pm) / (zd * zd - dd(1.0));
      zd = zd - pn / pp;
    }
    // the derivative at the converged root
    legendre_pn(N, zd, pn, pm);
    const dd pp = (double)N * (zd * pn - pm) / (zd * zd - dd(1.0));
    const dd wt = dd(2.0) / ((dd(1.0) - zd * zd) * pp * pp);
    x[N - 1 - i] = to_double(zd);
    x[i] = -to_double(zd);
    w[i] = w[N - 1 - i] = to_double(wt);
  });
  if (N % 2 == 1) x[N / 2] = 0.0;
  return SGPU_OK;
}

namespace {

// V_jk = L_k(x_j) in double-double, x from the FP64 nodes
void vandermonde(int N, const double* x, std::vector<dd>& V) {
  V.assign((size_t)N * N, dd());
  dd* v = V.data();
  parallel_for(N, [=](int j) {
    dd z = x[j], p0 = 1.0, p1 = z;
    v[(size_t)j * N + 0] = 1.0;
    if (N > 1) v[(size_t)j * N + 1] = z;
    for (int k = 2; k < N; ++k) {
      dd p2 = ((double)(2 * k - 1) * z * p1 - (double)(k - 1) * p0) / (double)k;
      v[(size_t)j * N + k] = p2;
      p0 = p1;
      p1 = p2;
    }
  });
}

// stencil K[k][m] (row k, offset m = 0, 2, 4) of the Legendre bases
void stencil(int basis, int N, std::vector<dd>& K2, std::vector<dd>& K4) {
  K2.assign(N, dd());
  K4.assign(N, dd());
  if (basis == SGPU_BASIS_SD) {
    for (int k = 0; k < N - 2; ++k) K2[k] = -1.0;  // constant: every row
  } else if (basis == SGPU_BASIS_SB) {
    // legendre/bases.py:564 {0: 1, 2: -(4n+10)/(2n+7), 4: (2n+3)/(2n+7)}, zero for k >= N-4
    for (int k = 0; k < N - 4; ++k) {
      K2[k] = -(dd(4.0 * k + 10) / (2.0 * k + 7));
      K4[k] = dd(2.0 * k + 3) / (2.0 * k + 7);
    }
  }
}

// Forward-transform matrix of the mixed form: F = Ms B^{-T}, so that
// forward(f) = f . F in one contraction (scalar product and mass solve
// together).  B_kl = sum_m K_km h_m K_lm (k, l < dim) is the mass matrix of
// the basis (stencil K, h_m = 2 / (2m + 1); legendre/matrices.py:110-192 give
// the same bands); F[j][k] = (B^{-1} Ms[j, :dim])_k, built in double-double
// with a banded LU (half-bandwidth 2 or 4, B is symmetric positive
// definite).  Columns k >= dim are zero, as the forward transform leaves them.
void forward_matrix(int N, int dim, const std::vector<dd>& K2, const std::vector<dd>& K4,
                    const std::vector<dd>& MsL, std::vector<double>& F) {
  const int bw = dim == N ? 0 : (dim == N - 2 ? 2 : 4);
  std::vector<dd> h(N);
  for (int m = 0; m < N; ++m) h[m] = dd(2.0) / (double)(2 * m + 1);
  // row k of K: entries at k, k+2, k+4
  auto kent = [&](int k, int m) -> dd {
    if (m == k) return 1.0;
    if (m == k + 2) return K2[k];
    if (m == k + 4) return K4[k];
    return 0.0;
  };
  const int W = 2 * bw + 1;
  std::vector<dd> A((size_t)dim * W, dd());  // A[k][bw + (l - k)]
  for (int k = 0; k < dim; ++k)
    for (int l = k - bw; l <= k + bw; ++l) {
      if (l < 0 || l >= dim) continue;
      dd v = 0.0;
      for (int m = (k > l ? k : l); m <= (k < l ? k : l) + 4 && m < N; ++m) v += kent(k, m) * h[m] * kent(l, m);
      A[(size_t)k * W + bw + (l - k)] = v;
    }
  // banded LU without pivoting: L unit lower (stored below), U upper
  for (int k = 0; k < dim; ++k) {
    const dd piv = A[(size_t)k * W + bw];
    for (int i = k + 1; i <= k + bw && i < dim; ++i) {
      const dd f = A[(size_t)i * W + bw + (k - i)] / piv;
      A[(size_t)i * W + bw + (k - i)] = f;
      for (int l = k + 1; l <= k + bw && l < dim; ++l) A[(size_t)i * W + bw + (l - i)] -= f * A[(size_t)k * W + bw + (l - k)];
    }
  }
  F.assign((size_t)N * N, 0.0);
  double* Fp = F.data();
  const dd* Ap = A.data();
  const dd* Msp = MsL.data();
  parallel_for(N, [=](int j) {
    std::vector<dd> y(dim);
    const dd* A = Ap;
    for (int k = 0; k < dim; ++k) y[k] = Msp[(size_t)j * N + k];
    for (int i = 0; i < dim; ++i)
      for (int k = i - bw; k < i; ++k)
        if (k >= 0) y[i] -= A[(size_t)i * W + bw + (k - i)] * y[k];
    for (int i = dim - 1; i >= 0; --i) {
      for (int l = i + 1; l <= i + bw && l < dim; ++l) y[i] -= A[(size_t)i * W + bw + (l - i)] * y[l];
      y[i] /= A[(size_t)i * W + bw];
    }
    for (int k = 0; k < dim; ++k) Fp[(size_t)j * N + k] = to_double(y[k]);
  });
}

}  // namespace

struct sgpu_legendre_plan {
  int N, basis, form;
  double* d_scalar;  // N x N: out = f . Ms
  double* d_back;    // N x N: u = c . Mb
  double* d_mass;    // LU'd mass bands (reciprocal diagonal), forward transform
  double* d_nodes;   // x, w (2N)
  std::vector<double> x, w;
  oz::Matrix tc_scalar, tc_forward, tc_back;  // mixed form: split Ms, Ms B^{-T}, Mb
  // mixed form, contiguous lines, N <= 339: the same three operators for the
  // fused contraction (the digit split inside the GEMM kernel, 54 bits)
  lc::Matrix fc[3];
  bool fused = false;
};

extern "C" int sgpu_legendre_plan_create(sgpu_legendre_plan** out, int N, int basis, int form) {
  if (!out) return SGPU_ERR_ARG;
  *out = nullptr;
  if (N < 2 || N > 8192) return SGPU_ERR_ARG;
  if (basis < SGPU_BASIS_ORTHO || basis > SGPU_BASIS_SB) return SGPU_ERR_ARG;
  if (form != SGPU_PLAIN_F64 && form != SGPU_MIXED_DF) return SGPU_ERR_UNSUPPORTED;
  if (form == SGPU_MIXED_DF) {
    if (oz::pick_digits(N) != SGPU_OK) return SGPU_ERR_UNSUPPORTED;
  }
  if (basis == SGPU_BASIS_SD && N < 4) return SGPU_ERR_ARG;
  if (basis == SGPU_BASIS_SB && N < 8) return SGPU_ERR_ARG;
  sgpu_legendre_plan* p = new (std::nothrow) sgpu_legendre_plan;
  if (!p) return SGPU_ERR_NOMEM;
  p->N = N;
  p->basis = basis;
  p->form = form;
  p->x.resize(N);
  p->w.resize(N);
  sgpu_leggauss(N, p->x.data(), p->w.data());
  std::vector<dd> V, K2, K4;
  vandermonde(N, p->x.data(), V);
  stencil(basis, N, K2, K4);
  const int nb = basis == SGPU_BASIS_SD ? 2 : (basis == SGPU_BASIS_SB ? 4 : 0);
  const int dim = N - nb;
  // Ms[j][k] = w_j (V_jk + K2_k V_j,k+2 + K4_k V_j,k+4)
  std::vector<double> Ms((size_t)N * N), Mb((size_t)N * N, 0.0);
  std::vector<dd> MsL(form == SGPU_MIXED_DF ? (size_t)N * N : 0);
  {
    const dd* Vp = V.data();
    const dd* K2p = K2.data();
    const dd* K4p = K4.data();
    const double* wp = p->w.data();
    double* Msp = Ms.data();
    double* Mbp = Mb.data();
    dd* MsLp = MsL.empty() ? nullptr : MsL.data();
    parallel_for(N, [=](int j) {
      for (int k = 0; k < N; ++k) {
        dd v = Vp[(size_t)j * N + k];
        if (k + 2 < N) v += K2p[k] * Vp[(size_t)j * N + k + 2];
        if (k + 4 < N) v += K4p[k] * Vp[(size_t)j * N + k + 4];
        const dd wv = wp[j] * v;
        Msp[(size_t)j * N + k] = to_double(wv);
        if (MsLp) MsLp[(size_t)j * N + k] = wv;
        // Mb[k][j] = V_jk + K2_k V_j,k+2 + K4_k V_j,k+4 for k < dim (rows k >= dim zero)
        if (k < dim) Mbp[(size_t)k * N + j] = to_double(v);
      }
    });
  }
  // mass matrix (legendre/matrices.py:121-135, :179-192) LU'd with TDMA/PDMA_LU
  std::vector<double> mass;
  std::vector<dd> h(N);
  for (int k = 0; k < N; ++k) h[k] = dd(2.0) / (double)(2 * k + 1);
  if (nb == 0) {
    mass.resize(N);
    for (int k = 0; k < N; ++k) mass[k] = to_double(dd(1.0) / h[k]);
  } else if (nb == 2) {
    mass.assign(3 * (size_t)dim, 0.0);
    double* ld = &mass[0];
    double* d = &mass[dim];
    double* ud = &mass[2 * dim + 2];
    for (int k = 0; k < dim; ++k) d[k] = to_double(h[k] + h[k + 2]);
    for (int k = 0; k < dim - 2; ++k) ld[k] = ud[k] = -to_double(h[k + 2]);
    tdma_lu_prog(mass.data(), dim);
    for (int k = 0; k < dim; ++k) d[k] = 1.0 / d[k];
  } else {
    mass.assign(5 * (size_t)dim, 0.0);
    double* a = &mass[0];
    double* b = &mass[dim];
    double* d = &mass[2 * dim];
    double* e = &mass[3 * dim + 2];
    double* f = &mass[4 * dim + 4];
    // the integer factors below are exact in FP64 (|i| < 2^20)
    for (int i = 0; i < dim; ++i) {
      const double I = i;
      d[i] = to_double(((-4 * I - 10) * (-4 * I - 10)) * h[i + 2] / ((2 * I + 7) * (2 * I + 7)) +
                       ((2 * I + 3) * (2 * I + 3)) * h[i + 4] / ((2 * I + 7) * (2 * I + 7)) + h[i]);
    }
    for (int i = 0; i < dim - 2; ++i) {
      const double I = i;
      b[i] = e[i] = to_double(((-4 * I - 18) * (2 * I + 3)) * h[i + 4] / ((2 * I + 7) * (2 * I + 11)) +
                              (-4 * I - 10) * h[i + 2] / (2 * I + 7));
    }
    for (int i = 0; i < dim - 4; ++i) {
      const double I = i;
      a[i] = f[i] = to_double((2 * I + 3) * h[i + 4] / (2 * I + 7));
    }
    pdma_lu_prog(mass.data(), dim);
    for (int k = 0; k < dim; ++k) d[k] = 1.0 / d[k];
  }
  size_t nbytes = sizeof(double) * (2 * (size_t)N * N + mass.size() + 2 * (size_t)N);
  void* dev = nullptr;
  if (cudaMalloc(&dev, nbytes) != cudaSuccess) {
    cudaGetLastError();
    delete p;
    return SGPU_ERR_NOMEM;
  }
  double* b = (double*)dev;
  p->d_scalar = b;
  p->d_back = b + (size_t)N * N;
  p->d_mass = b + 2 * (size_t)N * N;
  p->d_nodes = p->d_mass + mass.size();
  cudaError_t e1 = cudaMemcpy(p->d_scalar, Ms.data(), sizeof(double) * Ms.size(), cudaMemcpyHostToDevice);
  cudaError_t e2 = cudaMemcpy(p->d_back, Mb.data(), sizeof(double) * Mb.size(), cudaMemcpyHostToDevice);
  cudaError_t e3 = cudaMemcpy(p->d_mass, mass.data(), sizeof(double) * mass.size(), cudaMemcpyHostToDevice);
  cudaError_t e4 = cudaMemcpy(p->d_nodes, p->x.data(), sizeof(double) * N, cudaMemcpyHostToDevice);
  cudaError_t e5 = cudaMemcpy(p->d_nodes + N, p->w.data(), sizeof(double) * N, cudaMemcpyHostToDevice);
  if (e1 || e2 || e3 || e4 || e5) {
    cudaFree(dev);
    cudaGetLastError();
    delete p;
    return SGPU_ERR_CUDA;
  }
  if (form == SGPU_MIXED_DF) {
    // the forward transform contracts with F = Ms B^{-T} directly: a scalar
    // product followed by the mass solve would magnify the scalar product's
    // normwise error ~N-fold in the high modes
    std::vector<double> F;
    forward_matrix(N, dim, K2, K4, MsL, F);
    int st = oz::matrix_create(Ms.data(), N, 0, &p->tc_scalar);
    if (st == SGPU_OK) st = oz::matrix_create(F.data(), N, 0, &p->tc_forward);
    if (st == SGPU_OK) st = oz::matrix_create(Mb.data(), N, 0, &p->tc_back);
    // contiguous lines: the fused contraction where it applies (all three
    // directions, so one scratch size serves every call)
    const oz::Matrix* tcs[3] = {&p->tc_scalar, &p->tc_forward, &p->tc_back};
    const double* hm[3] = {Ms.data(), F.data(), Mb.data()};
    if (st == SGPU_OK && lc::supported(N, tcs[0]->K) && lc::supported(N, tcs[1]->K) && lc::supported(N, tcs[2]->K)) {
      for (int d = 0; d < 3 && st == SGPU_OK; ++d) st = lc::matrix_create(hm[d], N, tcs[d]->K, &p->fc[d]);
      p->fused = st == SGPU_OK;
    }
    if (st != SGPU_OK) {
      oz::matrix_destroy(&p->tc_scalar);
      oz::matrix_destroy(&p->tc_forward);
      oz::matrix_destroy(&p->tc_back);
      for (int d = 0; d < 3; ++d) lc::matrix_destroy(&p->fc[d]);
      cudaFree(dev);
      delete p;
      return st;
    }
  }
  *out = p;
  return SGPU_OK;
}

extern "C" int sgpu_legendre_plan_destroy(sgpu_legendre_plan* p) {
  if (!p) return SGPU_OK;
  cudaFree(p->d_scalar);
  oz::matrix_destroy(&p->tc_scalar);
  oz::matrix_destroy(&p->tc_forward);
  oz::matrix_destroy(&p->tc_back);
  for (int d = 0; d < 3; ++d) lc::matrix_destroy(&p->fc[d]);
  delete p;
  return SGPU_OK;
}

extern "C" int sgpu_legendre_nodes(const sgpu_legendre_plan* p, double* x, double* w) {
  if (!p || !x || !w) return SGPU_ERR_ARG;
  std::memcpy(x, p->x.data(), sizeof(double) * p->N);
  std::memcpy(w, p->w.data(), sizeof(double) * p->N);
  return SGPU_OK;
}

// ---------------------------------------------------------------------------
// FP64 GEMM along lines: out(l, k) = sum_j in(l, j) M[j][k] for every line l
// of an (outer, Nin, inner) input and (outer, Nout, inner) output (complex
// lines: real and imaginary parts are two rows); M is Nin x Nout.  64 x 64
// output tiles, K steps of 16, 256 threads with 4 x 4 register blocks; rows
// are (line, part) pairs.
namespace {
const int TM = 64, TN = 64, TK = 16;
}

// lscale (optional): one factor per line (complex lines: a complex factor,
// re/im pairs) multiplying the line's result; accumulate: out += result.
__global__ void __launch_bounds__(256) k_line_gemm_f64(const double* in, double* out, const double* M,
                                                       int Nin, int Nout, int64_t nrows, int64_t inner,
                                                       int cplx, const double* lscale, int accumulate) {
  __shared__ double As[TK][TM + 1];
  __shared__ double Bs[TK][TN + 1];
  const int tid = threadIdx.x;
  const int64_t row0 = (int64_t)blockIdx.x * TM;
  const int col0 = blockIdx.y * TN;
  const int tr = tid / 16, tc = tid % 16;  // 16 x 16 threads, 4 x 4 each
  double acc[4][4] = {};
  // element (row, j) of a line of length N: row = line * (1 + cplx) + part
  auto off = [&](int64_t row, int64_t j, int N) -> int64_t {
    int64_t l = cplx ? (row >> 1) : row;
    int part = cplx ? (int)(row & 1) : 0;
    int64_t o = l / inner, i = l - o * inner;
    int64_t e = (o * N + j) * inner + i;
    return cplx ? 2 * e + part : e;
  };
  for (int k0 = 0; k0 < Nin; k0 += TK) {
    // A tile: TM rows x TK columns (4 per thread)
    for (int e = tid; e < TM * TK; e += 256) {
      int r = e / TK, kk = e % TK;
      int64_t row = row0 + r;
      int j = k0 + kk;
      As[kk][r] = (row < nrows && j < Nin) ? in[off(row, j, Nin)] : 0.0;
    }
    for (int e = tid; e < TK * TN; e += 256) {
      int kk = e / TN, c = e % TN;
      int j = k0 + kk, col = col0 + c;
      Bs[kk][c] = (j < Nin && col < Nout) ? M[(size_t)j * Nout + col] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tr * 4 + i];
#pragma unroll
      for (int i = 0; i < 4; ++i) b[i] = Bs[kk][tc * 4 + i];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[i][q] = fma(a[i], b[q], acc[i][q]);
    }
    __syncthreads();
  }
  if (lscale) {
    // a thread's 4 rows start at an even row, so (re, im) of a complex line
    // are rows (0, 1) or (2, 3) of its block
    if (cplx) {
#pragma unroll
      for (int pr = 0; pr < 2; ++pr) {
        const int64_t row = row0 + tr * 4 + 2 * pr;
        if (row >= nrows) continue;
        const double sr = lscale[row], si = lscale[row + 1];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const double re = acc[2 * pr][q], im = acc[2 * pr + 1][q];
          acc[2 * pr][q] = sr * re - si * im;
          acc[2 * pr + 1][q] = sr * im + si * re;
        }
      }
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int64_t row = row0 + tr * 4 + i;
        if (row >= nrows) continue;
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[i][q] *= lscale[row];
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int64_t row = row0 + tr * 4 + i;
    if (row >= nrows) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int col = col0 + tc * 4 + q;
      if (col < Nout) {
        double* o = out + off(row, col, Nout);
        *o = accumulate ? *o + acc[i][q] : acc[i][q];
      }
    }
  }
}

namespace sgpu {
int line_gemm_f64(const double* in, double* out, const double* M, int Nin, int Nout, int64_t nrows,
                  int64_t inner, int cplx, cudaStream_t stream, const double* lscale, int accumulate) {
  if (nrows == 0) return SGPU_OK;
  if ((nrows + TM - 1) / TM > 0x7fffffff || Nin < 1 || Nout < 1) return SGPU_ERR_ARG;
  dim3 grid((unsigned)((nrows + TM - 1) / TM), (unsigned)((Nout + TN - 1) / TN));
  k_line_gemm_f64<<<grid, 256, 0, stream>>>(in, out, M, Nin, Nout, nrows, inner, cplx, lscale, accumulate);
  return cudaGetLastError() == cudaSuccess ? SGPU_OK : SGPU_ERR_CUDA;
}
}  // namespace sgpu

extern "C" int sgpu_line_gemm(const void* in, void* out, const double* M, int64_t Nin, int64_t Nout,
                              int64_t outer, int64_t inner, int data_kind, const double* line_scale,
                              int accumulate, cudaStream_t stream) {
  if (!in || !out || !M || in == out || outer < 0 || inner < 1 || Nin < 1 || Nout < 1) return SGPU_ERR_ARG;
  if (Nin > 0x7fffffff || Nout > 0x7fffffff) return SGPU_ERR_ARG;
  if (data_kind != SGPU_REAL && data_kind != SGPU_COMPLEX) return SGPU_ERR_ARG;
  const int cplx = data_kind == SGPU_COMPLEX;
  return sgpu::line_gemm_f64((const double*)in, (double*)out, M, (int)Nin, (int)Nout, outer * inner * (1 + cplx),
                             inner, cplx, stream, line_scale, accumulate ? 1 : 0);
}

// mass solve along lines after the scalar product (forward transform)
template <class T>
__global__ void k_legendre_mass(T* u, const double* mass, int N, int basis, int64_t nlines,
                                int64_t inner) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nlines) return;
  const int nb = basis == SGPU_BASIS_SD ? 2 : (basis == SGPU_BASIS_SB ? 4 : 0);
  const int dim = N - nb;
  T* base = u + sys_base(s, N, inner);
  Line<T> v{base, inner};
  if (nb == 0) {
    for (int k = 0; k < N; ++k) v[k] = mulr(v[k], mass[k]);
    return;
  }
  if (nb == 2) {
    const double* ld = mass;
    const double* di = mass + dim;
    const double* ud = mass + 2 * dim + 2;
    for (int i = 2; i < dim; ++i) v[i] = v[i] - mulr(v[i - 2], ld[i - 2]);
    v[dim - 1] = mulr(v[dim - 1], di[dim - 1]);
    v[dim - 2] = mulr(v[dim - 2], di[dim - 2]);
    for (int i = dim - 3; i >= 0; --i) v[i] = mulr(v[i] - mulr(v[i + 2], ud[i]), di[i]);
  } else {
    const double* a = mass;
    const double* b = mass + dim;
    const double* di = mass + 2 * dim;
    const double* e = mass + 3 * dim + 2;
    const double* f = mass + 4 * dim + 4;
    v[2] = v[2] - mulr(v[0], b[0]);
    v[3] = v[3] - mulr(v[1], b[1]);
    for (int k = 4; k < dim; ++k) v[k] = v[k] - (mulr(v[k - 2], b[k - 2]) + mulr(v[k - 4], a[k - 4]));
    v[dim - 1] = mulr(v[dim - 1], di[dim - 1]);
    v[dim - 2] = mulr(v[dim - 2], di[dim - 2]);
    v[dim - 3] = mulr(v[dim - 3] - mulr(v[dim - 1], e[dim - 3]), di[dim - 3]);
    v[dim - 4] = mulr(v[dim - 4] - mulr(v[dim - 2], e[dim - 4]), di[dim - 4]);
    for (int k = dim - 5; k >= 0; --k)
      v[k] = mulr(v[k] - mulr(v[k + 2], e[k]) - mulr(v[k + 4], f[k]), di[k]);
  }
  for (int k = dim; k < N; ++k) v[k] = zero_of(T());
}

// direction: 0 = scalar product, 1 = forward (scalar product + mass solve), 2 = backward
static int legendre_run(const sgpu_legendre_plan* p, int direction, const void* in, void* out,
                        int64_t outer, int64_t inner, int data_kind, void* work, size_t work_bytes,
                        cudaStream_t stream) {
  if (!p || !in || !out || outer < 0 || inner < 1) return SGPU_ERR_ARG;
  if (direction < 0 || direction > 2) return SGPU_ERR_ARG;
  if (data_kind != SGPU_REAL && data_kind != SGPU_COMPLEX) return SGPU_ERR_ARG;
  if (in == out) return SGPU_ERR_ARG;  // the GEMM reads every input row of a tile
  const int64_t nlines = outer * inner;
  if (nlines == 0) return SGPU_OK;
  const int cplx = data_kind == SGPU_COMPLEX;
  if (p->form == SGPU_MIXED_DF && p->fused && inner == 1) {
    const int st = lc::contract(p->fc[direction], (const double*)in, (double*)out, nlines, cplx, work, work_bytes,
                                nullptr, 0, stream);
    if (st != SGPU_OK) return st;
  } else if (p->form == SGPU_MIXED_DF) {
    const oz::Matrix& M = direction == 2 ? p->tc_back : (direction == 1 ? p->tc_forward : p->tc_scalar);
    const int st = oz::contract(M, (const double*)in, (double*)out, nlines, inner, cplx, work, work_bytes, stream);
    if (st != SGPU_OK) return st;
  } else {
    const int64_t nrows = nlines * (1 + cplx);
    dim3 grid((unsigned)((nrows + TM - 1) / TM), (unsigned)((p->N + TN - 1) / TN));
    if ((nrows + TM - 1) / TM > 0x7fffffff) return SGPU_ERR_ARG;
    const double* M = direction == 2 ? p->d_back : p->d_scalar;
    k_line_gemm_f64<<<grid, 256, 0, stream>>>((const double*)in, (double*)out, M, p->N, p->N, nrows, inner, cplx,
                                              nullptr, 0);
  }
  if (direction == 1 && p->form != SGPU_MIXED_DF) {
    const unsigned nb = (unsigned)((nlines + 127) / 128);
    if (cplx)
      k_legendre_mass<cd><<<nb, 128, 0, stream>>>((cd*)out, p->d_mass, p->N, p->basis, nlines, inner);
    else
      k_legendre_mass<double><<<nb, 128, 0, stream>>>((double*)out, p->d_mass, p->N, p->basis, nlines, inner);
  }
  return cudaGetLastError() == cudaSuccess ? SGPU_OK : SGPU_ERR_CUDA;
}

extern "C" int sgpu_legendre_workspace_size(const sgpu_legendre_plan* p, int64_t outer, int64_t inner,
                                            int data_kind, size_t* bytes) {
  if (!p || !bytes || outer < 0 || inner < 1) return SGPU_ERR_ARG;
  if (data_kind != SGPU_REAL && data_kind != SGPU_COMPLEX) return SGPU_ERR_ARG;
  if (p->form != SGPU_MIXED_DF) {
    *bytes = 0;
    return SGPU_OK;
  }
  *bytes = p->fused && inner == 1
               ? lc::workspace_bytes(p->fc[0], outer, data_kind == SGPU_COMPLEX)
               : oz::workspace_bytes(p->tc_scalar, outer * inner, inner, data_kind == SGPU_COMPLEX);
  return SGPU_OK;
}

extern "C" int sgpu_legendre_execute_ws(const sgpu_legendre_plan* p, int direction, const void* in,
                                        void* out, int64_t outer, int64_t inner, int data_kind,
                                        void* work, size_t work_bytes, cudaStream_t stream) {
  return legendre_run(p, direction, in, out, outer, inner, data_kind, work, work_bytes, stream);
}

// without a caller workspace the mixed form takes its scratch from the
// stream-ordered allocator for the duration of the call
extern "C" int sgpu_legendre_execute(const sgpu_legendre_plan* p, int direction, const void* in,
                                     void* out, int64_t outer, int64_t inner, int data_kind,
                                     cudaStream_t stream) {
  if (!p || p->form != SGPU_MIXED_DF)
    return legendre_run(p, direction, in, out, outer, inner, data_kind, nullptr, 0, stream);
  size_t nb = 0;
  int st = sgpu_legendre_workspace_size(p, outer, inner, data_kind, &nb);
  if (st != SGPU_OK) return st;
  if (nb == 0 || outer * inner == 0)
    return legendre_run(p, direction, in, out, outer, inner, data_kind, nullptr, 0, stream);
  void* work = nullptr;
  if (cudaMallocAsync(&work, nb, stream) != cudaSuccess) {
    cudaGetLastError();
    return SGPU_ERR_NOMEM;
  }
  st = legendre_run(p, direction, in, out, outer, inner, data_kind, work, nb, stream);
  cudaFreeAsync(work, stream);
  return st;
}
