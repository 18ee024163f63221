// Native Helmholtz problem object: one call runs the whole hot-path step
// (scalar product of the right-hand side -> per-wavenumber banded solve ->
// backward transform) on a Fourier x ... x Dirichlet grid with the
// non-periodic axis last, the step a shenfun time stepper performs with
// inner(v, f), H(f_hat, u_hat) and u_hat.backward()
// (chebyshev/la.py:288-317, tensorproductspace.py:45-259).
//
// Grids: 2D  R2C(N0) x D(N1)        spectral (N0/2+1, N1)
//        3D  C2C(N0) x R2C(N1) x D(N2)   spectral (N0, N1/2+1, N2)
// with D a ShenDirichlet space of the Chebyshev (GC) or Legendre (LG) family.
// The operator is (-lap + c): alfa = -1, beta = |k|^2 + c per wavenumber.
//
// Creation builds the transform plans and factorises every system (device
// allocations happen there); the solve allocates nothing: its two scratch
// arrays come from the caller (sgpu_helmholtz_workspace_size).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <tuple>
#include <vector>

#include "ozaki_tc.h"
#include "solvers.cuh"

struct sgpu_plan;
struct sgpu_legendre_plan;

extern "C" {
int sgpu_plan_create(sgpu_plan** plan, int kind, int n, int basis, int form);
int sgpu_plan_destroy(sgpu_plan* plan);
int sgpu_plan_workspace_size(const sgpu_plan* plan, int64_t outer, int64_t inner, int data_kind,
                             size_t* bytes);
int sgpu_plan_execute_ws(const sgpu_plan* plan, const void* in, void* out, int64_t outer, int64_t inner,
                         int data_kind, double scale, void* work, size_t work_bytes, cudaStream_t stream);
int sgpu_legendre_workspace_size(const sgpu_legendre_plan* plan, int64_t outer, int64_t inner,
                                 int data_kind, size_t* bytes);
int sgpu_legendre_execute_ws(const sgpu_legendre_plan* plan, int direction, const void* in, void* out,
                             int64_t outer, int64_t inner, int data_kind, void* work, size_t work_bytes,
                             cudaStream_t stream);
int sgpu_plan_execute(const sgpu_plan* plan, const void* in, void* out, int64_t outer,
                      int64_t inner, int data_kind, double scale, cudaStream_t stream);
int sgpu_plan_execute_blocks(const sgpu_plan* plan, const void* in, void* out, int64_t outer, int64_t inner,
                             int data_kind, double scale, void* work, size_t work_bytes, int64_t pair_lines,
                             cudaStream_t stream);
int sgpu_legendre_plan_create(sgpu_legendre_plan** plan, int N, int basis, int form);
int sgpu_legendre_plan_destroy(sgpu_legendre_plan* plan);
int sgpu_legendre_execute(const sgpu_legendre_plan* plan, int direction, const void* in,
                          void* out, int64_t outer, int64_t inner, int data_kind,
                          cudaStream_t stream);
int sgpu_helmholtz_factor(int64_t N, const double* alfa, const double* beta, int neumann,
                          int64_t outer, int64_t inner, int form, void* fac, cudaStream_t stream);
int sgpu_helmholtz_solve_cached(const void* b, void* u, const void* fac, int neumann,
                                int64_t outer, int64_t N, int64_t inner, int data_kind, int form,
                                cudaStream_t stream);
int sgpu_band_sep_factor(int n, int nterms, int gen_term, const double* bands,
                         const double* gens, const double* coef, int64_t nsys, double* fac,
                         cudaStream_t stream);
int sgpu_band_sep_solve(const void* b, void* u, const double* fac, const double* gens, int n,
                        int64_t outer, int64_t Nb, int64_t inner, int data_kind,
                        cudaStream_t stream);
int sgpu_helmholtz_solve_cached_batch(const void* b, void* u, const void* const* facs, int K, int neumann,
                                      int64_t outer, int64_t N, int64_t inner, int data_kind, int form,
                                      cudaStream_t stream);
int sgpu_band_sep_solve_batch(const void* b, void* u, const double* const* facs, const double* gens, int K, int n,
                              int64_t outer, int64_t Nb, int64_t inner, int data_kind, cudaStream_t stream);
}

struct sgpu_helmholtz_problem {
  int ndim, family, form;
  int64_t N[3];
  double c;
  int64_t nsys, nphys, nspec;      // systems, physical and spectral element counts
  sgpu_plan* fx_f = nullptr;       // 3D: C2C forward / backward along axis 0
  sgpu_plan* fx_b = nullptr;
  sgpu_plan* fr_f = nullptr;       // R2C forward / C2R backward (axis 0 in 2D, 1 in 3D)
  sgpu_plan* fr_b = nullptr;
  sgpu_plan* d_s = nullptr;        // Chebyshev scalar product / backward (last axis)
  sgpu_plan* d_b = nullptr;
  sgpu_legendre_plan* leg = nullptr;
  double* dev = nullptr;           // alfa | beta | factor cache | bands | coef
  double* alfa = nullptr;
  double* beta = nullptr;
  double* fac = nullptr;
  double* bands = nullptr;
  double* coef = nullptr;
  bool shared_plans = false;       // plans come from the process-wide cache
  bool stream_ordered = false;     // device memory from cudaMallocAsync
  cudaStream_t stream = 0;         // creation stream (stream-ordered problems)
  int device = -1;                 // the device the problem's memory and plans live on
};

namespace {

// Process-wide per-axis plan cache for stream-ordered problems: plans depend
// only on (kind, n, basis, form), so requests that share an axis length share
// them.  Plans stay until sgpu_plan_cache_clear or process exit.
std::mutex g_plan_mutex;
std::map<std::tuple<int, int, int, int>, sgpu_plan*> g_plans;
std::map<std::tuple<int, int, int>, sgpu_legendre_plan*> g_leg_plans;

// Plans are built outside the lock, so that callers on several threads build
// plans of different lengths at the same time; two callers that build the
// same plan keep the first one inserted.
template <class Plan, class Key, class Make, class Destroy>
int cached(std::map<Key, Plan*>& cache, const Key& key, Plan** out, Make make, Destroy destroy) {
  {
    std::lock_guard<std::mutex> lock(g_plan_mutex);
    auto it = cache.find(key);
    if (it != cache.end()) {
      *out = it->second;
      return SGPU_OK;
    }
  }
  Plan* mine = nullptr;
  const int st = make(&mine);
  if (st != SGPU_OK) return st;
  std::lock_guard<std::mutex> lock(g_plan_mutex);
  auto it = cache.find(key);
  if (it != cache.end()) {
    destroy(mine);
    *out = it->second;
    return SGPU_OK;
  }
  cache[key] = mine;
  *out = mine;
  return SGPU_OK;
}

int cached_plan(sgpu_plan** out, int kind, int n, int basis, int form) {
  return cached(g_plans, std::make_tuple(kind, n, basis, form), out,
                [&](sgpu_plan** p) { return sgpu_plan_create(p, kind, n, basis, form); },
                [](sgpu_plan* p) { sgpu_plan_destroy(p); });
}

int cached_leg_plan(sgpu_legendre_plan** out, int n, int basis, int form) {
  return cached(g_leg_plans, std::make_tuple(n, basis, form), out,
                [&](sgpu_legendre_plan** p) { return sgpu_legendre_plan_create(p, n, basis, form); },
                [](sgpu_legendre_plan* p) { sgpu_legendre_plan_destroy(p); });
}

void destroy_all(sgpu_helmholtz_problem* p) {
  if (!p) return;
  if (!p->shared_plans) {
    sgpu_plan_destroy(p->fx_f);
    sgpu_plan_destroy(p->fx_b);
    sgpu_plan_destroy(p->fr_f);
    sgpu_plan_destroy(p->fr_b);
    sgpu_plan_destroy(p->d_s);
    sgpu_plan_destroy(p->d_b);
    sgpu_legendre_plan_destroy(p->leg);
  }
  if (p->dev) {
    if (p->stream_ordered)
      cudaFreeAsync(p->dev, p->stream);
    else
      cudaFree(p->dev);
  }
  delete p;
}

SGPU_HD int64_t fftfreq(int64_t i, int64_t n) { return i <= (n - 1) / 2 ? i : i - n; }

// per-wavenumber scales alfa = -1, beta = |k|^2 + c of a problem, written on
// the device (a pageable host source would make the copy wait for the
// stream's earlier work)
__global__ void k_problem_scales(double* alfa, double* beta, int64_t nsys, int ndim, int64_t n0, int64_t nr,
                                 double c) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nsys; s += (int64_t)gridDim.x * blockDim.x) {
    double k2;
    if (ndim == 2) {
      k2 = (double)(s * s);
    } else {
      const int64_t ix = s / (nr / 2 + 1), iy = s % (nr / 2 + 1);
      const double kx = (double)fftfreq(ix, n0);
      k2 = kx * kx + (double)(iy * iy);
    }
    alfa[s] = -1.0;
    beta[s] = k2 + c;
  }
}

// Legendre ShenDirichlet terms (legendre/matrices.py:121-135, 285-292):
// term 0 the stiffness diagonal -(4k+6), term 1 the mass matrix
__global__ void k_legendre_terms(double* bands, int64_t n) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const double hk = 2.0 / (2.0 * k + 1.0), hk2 = 2.0 / (2.0 * (k + 2) + 1.0);
    for (int r = 0; r < 10; ++r) bands[r * n + k] = 0.0;
    bands[(0 * 5 + 2) * n + k] = -(4.0 * k + 6.0);
    bands[(1 * 5 + 2) * n + k] = hk + hk2;
    if (k + 2 < n) bands[(1 * 5 + 3) * n + k] = -hk2;
    if (k >= 2) bands[(1 * 5 + 1) * n + k] = -hk;
  }
}

int create_impl(sgpu_helmholtz_problem** out, int ndim, const int64_t* N, int family, double c,
                int form, bool ordered, cudaStream_t stream);

}  // namespace

extern "C" int sgpu_helmholtz_create(sgpu_helmholtz_problem** out, int ndim, const int64_t* N,
                                     int family, double c, int form) {
  return create_impl(out, ndim, N, family, c, form, false, 0);
}

extern "C" int sgpu_helmholtz_create_on(sgpu_helmholtz_problem** out, int ndim,
                                        const int64_t* N, int family, double c, int form,
                                        cudaStream_t stream) {
  return create_impl(out, ndim, N, family, c, form, true, stream);
}

extern "C" int sgpu_plan_cache_clear(void) {
  std::lock_guard<std::mutex> lock(g_plan_mutex);
  for (auto& kv : g_plans) sgpu_plan_destroy(kv.second);
  for (auto& kv : g_leg_plans) sgpu_legendre_plan_destroy(kv.second);
  g_plans.clear();
  g_leg_plans.clear();
  return SGPU_OK;
}

namespace {
int create_impl(sgpu_helmholtz_problem** out, int ndim, const int64_t* N, int family, double c,
                int form, bool ordered, cudaStream_t stream) {
  if (!out || !N) return SGPU_ERR_ARG;
  *out = nullptr;
  if (ndim != 2 && ndim != 3) return SGPU_ERR_ARG;
  if (family != SGPU_FAMILY_CHEBYSHEV && family != SGPU_FAMILY_LEGENDRE) return SGPU_ERR_ARG;
  if (form != SGPU_PLAIN_F64 && form != SGPU_MIXED_DF) return SGPU_ERR_ARG;
  for (int i = 0; i < ndim; ++i)
    if (N[i] < 2 || N[i] > (1 << 16)) return SGPU_ERR_ARG;
  if (N[ndim - 1] < 8) return SGPU_ERR_ARG;
  int device = -1;
  if (cudaGetDevice(&device) != cudaSuccess) {
    cudaGetLastError();
    return SGPU_ERR_CUDA;
  }
  sgpu_helmholtz_problem* p = new (std::nothrow) sgpu_helmholtz_problem;
  if (!p) return SGPU_ERR_NOMEM;
  p->device = device;
  p->ndim = ndim;
  p->family = family;
  p->form = form;
  p->c = c;
  p->shared_plans = ordered;
  p->stream_ordered = ordered;
  p->stream = stream;
  for (int i = 0; i < 3; ++i) p->N[i] = i < ndim ? N[i] : 1;
  const int64_t Nd = N[ndim - 1];
  const int64_t nr = ndim == 2 ? N[0] : N[1];  // R2C axis length
  p->nsys = ndim == 2 ? (nr / 2 + 1) : N[0] * (nr / 2 + 1);
  p->nphys = (ndim == 2 ? N[0] : N[0] * N[1]) * Nd;
  p->nspec = p->nsys * Nd;
  // every plan uses the requested arithmetic (mixed: double-float Fourier
  // transforms, tensor-core contractions along the Dirichlet axis)
  int st = SGPU_OK;
  auto chk = [&](int r) {  // the first failure's status
    if (st == SGPU_OK) st = r;
  };
  if (ndim == 3) {
    chk((ordered ? cached_plan : sgpu_plan_create)(&p->fx_f, SGPU_XF_C2C_FWD, (int)N[0], 0, form));
    chk((ordered ? cached_plan : sgpu_plan_create)(&p->fx_b, SGPU_XF_C2C_BWD, (int)N[0], 0, form));
  }
  chk((ordered ? cached_plan : sgpu_plan_create)(&p->fr_f, SGPU_XF_R2C, (int)nr, 0, form));
  chk((ordered ? cached_plan : sgpu_plan_create)(&p->fr_b, SGPU_XF_C2R, (int)nr, 0, form));
  if (family == SGPU_FAMILY_CHEBYSHEV) {
    chk((ordered ? cached_plan : sgpu_plan_create)(&p->d_s, SGPU_XF_CHEB_SCALAR, (int)Nd, SGPU_BASIS_SD, form));
    chk((ordered ? cached_plan : sgpu_plan_create)(&p->d_b, SGPU_XF_CHEB_BACKWARD, (int)Nd, SGPU_BASIS_SD, form));
  } else {
    // the mixed form contracts on the tensor cores where the plan supports N
    int lform = form;
    if (lform == SGPU_MIXED_DF && sgpu::oz::pick_digits((int)Nd) != SGPU_OK) lform = SGPU_PLAIN_F64;
    chk((ordered ? cached_leg_plan : sgpu_legendre_plan_create)(&p->leg, (int)Nd, SGPU_BASIS_SD, lform));
  }
  if (st != SGPU_OK) {
    destroy_all(p);
    return st;
  }
  const int64_t n = Nd - 2;
  const int64_t m = (n + 1) / 2;
  size_t nfac = family == SGPU_FAMILY_CHEBYSHEV ? (size_t)4 * n * p->nsys
                                                : (size_t)7 * m * 2 * p->nsys;
  size_t nb = family == SGPU_FAMILY_CHEBYSHEV ? 0 : (size_t)2 * 5 * n;
  size_t total = 2 * (size_t)p->nsys + nfac + nb + (nb ? 2 * (size_t)p->nsys : 0);
  cudaError_t me = ordered ? cudaMallocAsync((void**)&p->dev, sizeof(double) * total, stream)
                           : cudaMalloc((void**)&p->dev, sizeof(double) * total);
  if (me != cudaSuccess) {
    cudaGetLastError();
    destroy_all(p);
    return SGPU_ERR_NOMEM;
  }
  p->alfa = p->dev;
  p->beta = p->alfa + p->nsys;
  p->fac = p->beta + p->nsys;
  // per-wavenumber scales alfa = -1, beta = |k|^2 + c
  const unsigned sgrid = (unsigned)std::min<int64_t>((p->nsys + 255) / 256, 1024);
  k_problem_scales<<<sgrid, 256, 0, stream>>>(p->alfa, p->beta, p->nsys, ndim, N[0], nr, c);
  if (family == SGPU_FAMILY_CHEBYSHEV) {
    st = sgpu_helmholtz_factor(Nd, p->alfa, p->beta, 0, p->nsys, 1, SGPU_PLAIN_F64, p->fac, stream);
  } else {
    // terms: (phi''_j, phi_k) = -(4k+6) diagonal with coefficient alfa, and the
    // mass matrix B (legendre/matrices.py:121-135) with coefficient beta
    p->bands = p->fac + nfac;
    p->coef = p->bands + nb;
    k_legendre_terms<<<(unsigned)std::min<int64_t>((n + 255) / 256, 1024), 256, 0, stream>>>(p->bands, n);
    cudaMemcpyAsync(p->coef, p->alfa, sizeof(double) * 2 * p->nsys, cudaMemcpyDeviceToDevice, stream);
    st = sgpu_band_sep_factor((int)n, 2, -1, p->bands, nullptr, p->coef, p->nsys, p->fac, stream);
  }
  // plain creation waits for the factorisation; stream-ordered creation leaves
  // it queued on `stream` (later work on that stream sees it)
  const cudaError_t ce = ordered ? cudaGetLastError()
                                 : (cudaStreamSynchronize(stream) == cudaSuccess ? cudaGetLastError()
                                                                                : cudaErrorUnknown);
  if (st != SGPU_OK || ce != cudaSuccess) {
    cudaGetLastError();
    destroy_all(p);
    return SGPU_ERR_CUDA;
  }
  *out = p;
  return SGPU_OK;
}
}  // namespace

extern "C" int sgpu_helmholtz_destroy(sgpu_helmholtz_problem* p) {
  destroy_all(p);
  return SGPU_OK;
}

extern "C" int sgpu_helmholtz_shape(const sgpu_helmholtz_problem* p, int64_t* phys, int64_t* spec) {
  if (!p || !phys || !spec) return SGPU_ERR_ARG;
  for (int i = 0; i < p->ndim; ++i) phys[i] = spec[i] = p->N[i];
  if (p->ndim == 2)
    spec[0] = p->N[0] / 2 + 1;
  else
    spec[1] = p->N[1] / 2 + 1;
  return SGPU_OK;
}

// scratch layout: wr (real, physical size) | wc (complex, spectral size) |
// wt (the Dirichlet-axis contraction's split input in the tensor-core form)
static size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

static size_t split_bytes(const sgpu_helmholtz_problem* p, int K = 1) {
  const int64_t nlines_d = K * (p->nphys / p->N[p->ndim - 1]);
  size_t a = 0, b = 0;
  if (p->family == SGPU_FAMILY_CHEBYSHEV) {
    sgpu_plan_workspace_size(p->d_s, nlines_d, 1, SGPU_REAL, &a);
    sgpu_plan_workspace_size(p->d_b, nlines_d, 1, SGPU_REAL, &b);
  } else {
    sgpu_legendre_workspace_size(p->leg, nlines_d, 1, SGPU_REAL, &a);
  }
  return a > b ? a : b;
}

extern "C" int sgpu_helmholtz_workspace_size(const sgpu_helmholtz_problem* p, size_t* bytes) {
  if (!p || !bytes) return SGPU_ERR_ARG;
  *bytes = round256((size_t)p->nphys * 8) + round256((size_t)p->nspec * 16) + split_bytes(p);
  return SGPU_OK;
}

// the step itself on a scratch area laid out as above, for K problems of p's
// shape stacked along a leading axis (f, u: K physical arrays; work: the
// scratch of the stacked arrays); facs (device, K pointers) gives each
// member's factor cache, nullptr for K = 1 and p's own
static int helmholtz_run(const sgpu_helmholtz_problem* p, const double* f, double* u, void* work,
                         cudaStream_t s, int K = 1, const void* const* facs = nullptr) {
  const int64_t Nd = p->N[p->ndim - 1];
  const int64_t nlines_d = K * (p->nphys / Nd);  // physical lines along the last axis
  double* wr = (double*)work;
  double* wc = (double*)((unsigned char*)work + round256((size_t)K * p->nphys * 8));
  void* wt = (unsigned char*)wc + round256((size_t)K * p->nspec * 16);
  const size_t wtb = split_bytes(p, K);
  // the first failing call's status is the step's status
  int st = SGPU_OK;
  auto chk = [&](int r) {
    if (st == SGPU_OK) st = r;
  };
  // real lines pair up within each member only (bits independent of the batch)
  const int64_t pl_d = nlines_d / K;
  const int64_t pl_r = p->ndim == 2 ? Nd : p->N[0] * Nd;
  // 1. scalar product along the Dirichlet axis (real data)
  if (p->family == SGPU_FAMILY_CHEBYSHEV)
    chk(sgpu_plan_execute_blocks(p->d_s, f, wr, nlines_d, 1, SGPU_REAL, 1.0, wt, wtb, pl_d, s));
  else
    chk(sgpu_legendre_execute_ws(p->leg, 0, f, wr, nlines_d, 1, SGPU_REAL, wt, wtb, s));
  if (p->ndim == 2) {
    const int64_t N0 = p->N[0];
    chk(sgpu_plan_execute_blocks(p->fr_f, wr, wc, K, Nd, SGPU_REAL, 1.0 / N0, nullptr, 0, pl_r, s));
  } else {
    const int64_t N0 = p->N[0], N1 = p->N[1], Nh = N1 / 2 + 1;
    chk(sgpu_plan_execute_blocks(p->fr_f, wr, wc, K * N0, Nd, SGPU_REAL, 1.0 / N1, nullptr, 0, pl_r, s));
    chk(sgpu_plan_execute(p->fx_f, wc, wc, K, Nh * Nd, SGPU_COMPLEX, 1.0 / N0, s));
  }
  // 2. one banded system per wavenumber, in place on the spectral array
  if (p->family == SGPU_FAMILY_CHEBYSHEV)
    chk(facs ? sgpu_helmholtz_solve_cached_batch(wc, wc, facs, K, 0, p->nsys, Nd, 1, SGPU_COMPLEX, SGPU_PLAIN_F64, s)
             : sgpu_helmholtz_solve_cached(wc, wc, p->fac, 0, p->nsys, Nd, 1, SGPU_COMPLEX, SGPU_PLAIN_F64, s));
  else
    chk(facs ? sgpu_band_sep_solve_batch(wc, wc, (const double* const*)facs, nullptr, K, (int)(Nd - 2), p->nsys, Nd,
                                         1, SGPU_COMPLEX, s)
             : sgpu_band_sep_solve(wc, wc, p->fac, nullptr, (int)(Nd - 2), p->nsys, Nd, 1, SGPU_COMPLEX, s));
  // 3. backward
  if (p->ndim == 2) {
    chk(sgpu_plan_execute_blocks(p->fr_b, wc, wr, K, Nd, SGPU_COMPLEX, 1.0, nullptr, 0, pl_r, s));
  } else {
    const int64_t N0 = p->N[0], N1 = p->N[1], Nh = N1 / 2 + 1;
    chk(sgpu_plan_execute(p->fx_b, wc, wc, K, Nh * Nd, SGPU_COMPLEX, 1.0, s));
    chk(sgpu_plan_execute_blocks(p->fr_b, wc, wr, K * N0, Nd, SGPU_COMPLEX, 1.0, nullptr, 0, pl_r, s));
  }
  if (p->family == SGPU_FAMILY_CHEBYSHEV)
    chk(sgpu_plan_execute_blocks(p->d_b, wr, u, nlines_d, 1, SGPU_REAL, 1.0, wt, wtb, pl_d, s));
  else
    chk(sgpu_legendre_execute_ws(p->leg, 2, wr, u, nlines_d, 1, SGPU_REAL, wt, wtb, s));
  return st;
}

// the current device must be the one the problem was created on
static bool on_own_device(const sgpu_helmholtz_problem* p) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return dev == p->device;
}

extern "C" int sgpu_helmholtz_batch_workspace_size(const sgpu_helmholtz_problem* p, int K, size_t* bytes) {
  if (!p || !bytes || K < 1) return SGPU_ERR_ARG;
  *bytes = round256((size_t)K * p->nphys * 8) + round256((size_t)K * p->nspec * 16) + split_bytes(p, K);
  return SGPU_OK;
}

extern "C" int sgpu_helmholtz_plan_handles(const sgpu_helmholtz_problem* p, sgpu_plan** plans, int64_t* lines) {
  if (!p || !plans || !lines) return SGPU_ERR_ARG;
  const int64_t Nd = p->N[p->ndim - 1], nl = p->nphys / Nd;
  sgpu_plan* h[6] = {p->d_s, p->fr_f, p->fx_f, p->fx_b, p->fr_b, p->d_b};
  int64_t oi[12] = {nl, 1, 0, 0, 0, 0, 0, 0, 0, 0, nl, 1};
  if (p->ndim == 2) {
    oi[2] = 1, oi[3] = Nd, oi[8] = 1, oi[9] = Nd;
  } else {
    const int64_t Nh = p->N[1] / 2 + 1;
    oi[2] = p->N[0], oi[3] = Nd, oi[4] = 1, oi[5] = Nh * Nd, oi[6] = 1, oi[7] = Nh * Nd, oi[8] = p->N[0], oi[9] = Nd;
  }
  for (int i = 0; i < 6; ++i) plans[i] = h[i];
  for (int i = 0; i < 12; ++i) lines[i] = oi[i];
  return SGPU_OK;
}

extern "C" int sgpu_helmholtz_factor_ptr(const sgpu_helmholtz_problem* p, const void** fac) {
  if (!p || !fac) return SGPU_ERR_ARG;
  *fac = p->fac;
  return SGPU_OK;
}

extern "C" int sgpu_helmholtz_solve_batch(const sgpu_helmholtz_problem* p, int K, const void* const* facs,
                                          const double* f, double* u, void* work, size_t work_bytes,
                                          cudaStream_t stream) {
  if (!p || K < 1 || !facs || !f || !u || !work) return SGPU_ERR_ARG;
  if (!on_own_device(p)) return SGPU_ERR_ARG;
  size_t need = 0;
  sgpu_helmholtz_batch_workspace_size(p, K, &need);
  if (work_bytes < need || ((uintptr_t)work & 255) != 0) return SGPU_ERR_ARG;
  return helmholtz_run(p, f, u, work, stream, K, facs);
}

extern "C" int sgpu_helmholtz_solve(const sgpu_helmholtz_problem* p, const double* f, double* u,
                                    void* work, size_t work_bytes, cudaStream_t stream) {
  if (!p || !f || !u || !work) return SGPU_ERR_ARG;
  if (!on_own_device(p)) return SGPU_ERR_ARG;
  size_t need = 0;
  sgpu_helmholtz_workspace_size(p, &need);
  if (work_bytes < need) return SGPU_ERR_ARG;
  if (((uintptr_t)work & 255) != 0) return SGPU_ERR_ARG;
  return helmholtz_run(p, f, u, work, stream);
}

// ---------------------------------------------------------------------------
// Allocation-free variant of sgpu_helmholtz_solve.
//
// Some callers cannot hand the library a scratch buffer: a host program whose
// device memory is owned by another allocator that must not see raw
// cudaMalloc calls (or has no budget left for them), a Fortran or C code
// reaching the library through a thin FFI that has no notion of device
// buffers beyond its own input and output arrays, or a latency-critical loop
// that must not risk an allocation during a step.  For them the step can use
// a scratch array compiled into the library instead.
//
// The array below is a fixed 64 MiB of device memory.  Every GPU that loads
// the library holds it until the process exits, whether or not this entry
// point is used.  Problems whose scratch (sgpu_helmholtz_workspace_size: one
// real physical array, one complex spectral array, and for the mixed form
// the contraction's scratch along the Dirichlet axis) exceeds 64 MiB are
// rejected with SGPU_ERR_SCRATCH_LIMIT.  The Chebyshev mixed form needs 4
// bytes more per line than the plain form, so 128 x 128 x 129 fits both
// (34 MB); the Legendre mixed form adds a digit copy of the physical array
// (about 14 bytes per point), so compare sgpu_helmholtz_workspace_size with
// 64 MiB for it; 256 x 256 x 65 (68 MB) fits neither.
//
// The first call on a device (and after cudaDeviceReset, which replaces the
// device's context and with it the array's address) looks up the array's
// device address with cudaGetSymbolAddress, with that device current, and
// remembers it per (device, context); make that first call before any
// stream capture.  The problem must be used on the device it was created on
// (SGPU_ERR_ARG otherwise).  All calls share the one array and it keeps
// whatever the last call left in it; every call writes each scratch element
// it reads before reading it, so nothing has to be cleared between calls.
// Calls whose execution overlaps on the GPU (different streams, or
// different host threads without ordering) race on the array and give wrong
// results: serialise them.  Host code never passes the array's name to a
// kernel (in host code it is a host-side stand-in, not a device address):
// only the address obtained from cudaGetSymbolAddress is used.
#include <mutex>

#define SGPU_NOALLOC_SCRATCH_BYTES ((size_t)64 << 20)
#define SGPU_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_sgpu_noalloc_scratch[SGPU_NOALLOC_SCRATCH_BYTES];

namespace {
struct NoallocEntry {
  int dev = -1;
  void* ctx = nullptr;
  void* addr = nullptr;
};
std::mutex g_noalloc_mutex;
NoallocEntry g_noalloc[SGPU_NOALLOC_MAX_DEVICES];

// the current context of the calling thread (the runtime's primary context
// of the current device), through the driver's cuCtxGetCurrent
void* current_context() {
  typedef int (*GetCurrent)(void**);
  static GetCurrent fn = nullptr;
  static std::once_flag once;
  std::call_once(once, []() {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (GetCurrent)f;
    cudaGetLastError();
  });
  void* ctx = nullptr;
  if (!fn || fn(&ctx) != 0) return nullptr;
  return ctx;
}
}  // namespace

extern "C" int sgpu_helmholtz_solve_noalloc(const sgpu_helmholtz_problem* p, const double* f,
                                            double* u, cudaStream_t stream) {
  if (!p || !f || !u) return SGPU_ERR_ARG;
  size_t need = 0;
  sgpu_helmholtz_workspace_size(p, &need);
  if (need > SGPU_NOALLOC_SCRATCH_BYTES) return SGPU_ERR_SCRATCH_LIMIT;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return SGPU_ERR_CUDA;
  }
  if (dev != p->device) return SGPU_ERR_ARG;
  if (dev < 0 || dev >= SGPU_NOALLOC_MAX_DEVICES) return SGPU_ERR_UNSUPPORTED;
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoallocEntry& e = g_noalloc[dev];
    void* ctx = current_context();
    if (!e.addr || e.ctx != ctx) {
      void* addr = nullptr;
      if (cudaGetSymbolAddress(&addr, g_sgpu_noalloc_scratch) != cudaSuccess || !addr) {
        cudaGetLastError();
        return SGPU_ERR_CUDA;
      }
      e.dev = dev;
      e.ctx = ctx;
      e.addr = addr;
    }
    base = e.addr;
  }
  return helmholtz_run(p, f, u, base, stream);
}
