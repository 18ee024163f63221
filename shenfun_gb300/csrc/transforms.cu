// Transform plans (C ABI: sgpu_plan_*); the kernels are in xf_*.cu.
//
// In the mixed form the Chebyshev kinds (scalar product, forward, backward
// of a basis) run as a dense line contraction on the tensor cores
// (ozaki_tc.cu) instead of the double-float FFT: the operator is linear in
// the line, so its N x N matrix is the FP64 line kernel applied to the
// identity (on the device), and one split-BF16 contraction applies it (about 48
// bits; the forward matrix includes the mass solve, so its error is not
// magnified by it).  On GB300 the O(N^2) contraction on the tensor cores
// beats the O(N log N) transform on the FP32/FP64 pipes for N up to ~1000.
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "lc_fused.h"
#include "ozaki_tc.h"
#include "plan_host.cuh"
#include "xf_kernels.cuh"

using namespace sgpu;

struct sgpu_plan {
  LinePlan lp;
  void* dev_tables;  // one allocation holding every device table
  bool tensor = false;
  oz::Matrix tc;     // tensor form: the line operator, split (any line layout)
  bool fused = false;
  lc::Matrix fm;     // the same operator for the fused contraction (contiguous lines)
  int fvariant = 1;  // length-256 Fourier plans: 1 strided-pass kernel, its default arithmetic and occupancy
                     // (3 CTAs per SM for double-float, 2 for FP64: measured best on the channel
                     // grid), 2 generic line programs, 3 / 4 strided-pass kernel at 2 / 3 CTAs per SM,
                     // 5 / 6 fixed point at 2 / 3 CTAs per SM, 7 fixed point with tensor-copy input (C2C)
};

namespace sgpu {
int f256_launch(const LinePlan& p, const double* in, double* out, int64_t nlines, int64_t inner, double scl,
                int ctas_per_sm, int fixed, cudaStream_t s);
}

namespace {

bool tensor_kind(int kind, int n, int form) {
  // Chebyshev lengths above 1024 stay on the double-float FFT line kernels:
  // the dense contraction's n^2 cost overtakes them there
  return form == SGPU_MIXED_DF && n >= 16 && n <= 1024 &&
         (kind == SGPU_XF_CHEB_SCALAR || kind == SGPU_XF_CHEB_FORWARD || kind == SGPU_XF_CHEB_BACKWARD);
}

__global__ void k_identity(double* I, int n) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)n * n;
       t += (int64_t)gridDim.x * blockDim.x)
    I[t] = (t / n == t % n) ? 1.0 : 0.0;
}

// M[j][k] = output k of the FP64 transform of the unit line e_j (n x n): the
// FP64 line kernel applied to the n x n identity on the device, on a private
// non-blocking stream with stream-ordered scratch, so that building a plan
// does not wait for work on the caller's streams (the same block program on
// the host took 3-40 ms for n = 129-1024)
int operator_matrix(int kind, int n, int basis, std::vector<double>& M) {
  LinePlan p;
  HostTables T;
  int st = build_plan_host(kind, n, basis, SGPU_PLAIN_F64, p, T);
  if (st != SGPU_OK) return st;
  if (p.n_in != n || p.n_out != n) return SGPU_ERR_UNSUPPORTED;
  size_t off[SGPU_NTAB];
  const size_t tb = table_layout(T, off);
  std::vector<unsigned char> img(tb, 0);
  table_image(T, off, img.data());
  const size_t tbr = (tb + 255) & ~(size_t)255, mb = (size_t)n * n * sizeof(double);
  cudaStream_t s;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return SGPU_ERR_CUDA;
  }
  unsigned char* dev = nullptr;
  st = SGPU_OK;
  if (cudaMallocAsync((void**)&dev, tbr + 2 * mb, s) != cudaSuccess) {
    st = SGPU_ERR_NOMEM;
  } else {
    double* I = (double*)(dev + tbr);
    double* O = I + (size_t)n * n;
    bind_tables(p, T, off, dev);
    M.assign((size_t)n * n, 0.0);
    const int lpb = lines_per_block(p, 0);
    const unsigned nb = (unsigned)((n + lpb - 1) / lpb);
    if (cudaMemcpyAsync(dev, img.data(), tb, cudaMemcpyHostToDevice, s) != cudaSuccess) st = SGPU_ERR_CUDA;
    if (st == SGPU_OK) {
      k_identity<<<(unsigned)(((int64_t)n * n + 255) / 256 < 4096 ? ((int64_t)n * n + 255) / 256 : 4096), 256, 0,
                   s>>>(I, n);
      st = xf_launch_cheb_f64(xf_group(p.kind), p, I, O, 0, n, 1, 1.0, nb, s);
    }
    if (st == SGPU_OK && cudaMemcpyAsync(M.data(), O, mb, cudaMemcpyDeviceToHost, s) != cudaSuccess)
      st = SGPU_ERR_CUDA;
    cudaFreeAsync(dev, s);
  }
  if (cudaStreamSynchronize(s) != cudaSuccess && st == SGPU_OK) st = SGPU_ERR_CUDA;
  cudaStreamDestroy(s);
  cudaGetLastError();
  return st;
}

}  // namespace

extern "C" int sgpu_plan_create(sgpu_plan** out, int kind, int n, int basis, int form) {
  if (!out) return SGPU_ERR_ARG;
  *out = nullptr;
  if (tensor_kind(kind, n, form)) {
    std::vector<double> M;
    int st = operator_matrix(kind, n, basis, M);
    if (st != SGPU_OK) return st;
    sgpu_plan* plan = new (std::nothrow) sgpu_plan;
    if (!plan) return SGPU_ERR_NOMEM;
    // the Chebyshev Dirichlet Helmholtz recurrence magnifies perturbations
    // of its input up to ~4000x at large shifts: FP64-level transforms
    st = oz::matrix_create(M.data(), n, 1, &plan->tc);
    if (st != SGPU_OK) {
      delete plan;
      return st;
    }
    // contiguous lines take the fused contraction where it applies (no
    // scratch, one pass over the data)
    if (lc::supported(n, plan->tc.K)) {
      st = lc::matrix_create(M.data(), n, plan->tc.K, &plan->fm);
      if (st != SGPU_OK) {
        oz::matrix_destroy(&plan->tc);
        delete plan;
        return st;
      }
      plan->fused = true;
    }
    std::memset(&plan->lp, 0, sizeof(plan->lp));
    plan->lp.kind = kind;
    plan->lp.basis = basis;
    plan->lp.form = form;
    plan->lp.n = plan->lp.n_in = plan->lp.n_out = n;
    plan->dev_tables = nullptr;
    plan->tensor = true;
    *out = plan;
    return SGPU_OK;
  }
  LinePlan p;
  HostTables T;
  int st = build_plan_host(kind, n, basis, form, p, T);
  if (st != SGPU_OK) return st;
  size_t off[SGPU_NTAB];
  const size_t sz = table_layout(T, off);
  std::vector<unsigned char> img(sz, 0);
  table_image(T, off, img.data());
  void* dev = nullptr;
  if (cudaMalloc(&dev, sz) != cudaSuccess) {
    cudaGetLastError();
    return SGPU_ERR_NOMEM;
  }
  if (cudaMemcpy(dev, img.data(), sz, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(dev);
    cudaGetLastError();
    return SGPU_ERR_CUDA;
  }
  bind_tables(p, T, off, (unsigned char*)dev);
  sgpu_plan* plan = new (std::nothrow) sgpu_plan;
  if (!plan) {
    cudaFree(dev);
    return SGPU_ERR_NOMEM;
  }
  plan->lp = p;
  plan->dev_tables = dev;
  *out = plan;
  return SGPU_OK;
}

extern "C" int sgpu_plan_destroy(sgpu_plan* plan) {
  if (!plan) return SGPU_OK;
  if (plan->dev_tables) cudaFree(plan->dev_tables);
  oz::matrix_destroy(&plan->tc);
  lc::matrix_destroy(&plan->fm);
  delete plan;
  return SGPU_OK;
}

extern "C" int sgpu_plan_workspace_size(const sgpu_plan* plan, int64_t outer, int64_t inner, int data_kind,
                                        size_t* bytes) {
  if (!plan || !bytes || outer < 0 || inner < 1) return SGPU_ERR_ARG;
  if (data_kind != SGPU_REAL && data_kind != SGPU_COMPLEX) return SGPU_ERR_ARG;
  if (!plan->tensor)
    *bytes = 0;
  else if (plan->fused && inner == 1)
    *bytes = lc::workspace_bytes(plan->fm, outer, data_kind == SGPU_COMPLEX);
  else
    *bytes = oz::workspace_bytes(plan->tc, outer * inner, inner, data_kind == SGPU_COMPLEX);
  return SGPU_OK;
}


namespace {
// SMs of the current device (cached per device)
int sm_count() {
  static std::once_flag once[64];
  static int n[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return 1;
  }
  std::call_once(once[dev], [&]() {
    if (cudaDeviceGetAttribute(&n[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n[dev] <= 0) n[dev] = 1;
    cudaGetLastError();
  });
  return n[dev];
}

bool fourier256(const sgpu_plan* plan) {
  const LinePlan& p = plan->lp;
  return !plan->tensor && p.n == 256 && p.m == 256 && !p.rader &&
         (p.kind == SGPU_XF_R2C || p.kind == SGPU_XF_C2R || p.kind == SGPU_XF_C2C_FWD || p.kind == SGPU_XF_C2C_BWD);
}
}  // namespace

extern "C" int sgpu_plan_set_variant(sgpu_plan* plan, int variant) {
  if (!plan || variant < 0 || variant > 7) return SGPU_ERR_ARG;
  if (plan->fused) {
    if (variant > 2) return SGPU_ERR_ARG;
    plan->fm.variant = variant == 0 ? 1 : variant;
    return SGPU_OK;
  }
  if (fourier256(plan)) {
    if (variant >= 5 && plan->lp.form != SGPU_MIXED_DF) return SGPU_ERR_UNSUPPORTED;
    if (variant == 7 && plan->lp.kind != SGPU_XF_C2C_FWD && plan->lp.kind != SGPU_XF_C2C_BWD)
      return SGPU_ERR_UNSUPPORTED;
    plan->fvariant = variant == 0 ? 1 : variant;
    return SGPU_OK;
  }
  return variant == 0 ? SGPU_OK : SGPU_ERR_UNSUPPORTED;
}

extern "C" int sgpu_plan_get_variant(const sgpu_plan* plan, int* variant) {
  if (!plan || !variant) return SGPU_ERR_ARG;
  *variant = plan->fused ? plan->fm.variant : (fourier256(plan) ? plan->fvariant : 0);
  return SGPU_OK;
}

static int plan_run(const sgpu_plan* plan, const void* in, void* out, int64_t outer, int64_t inner,
                    int data_kind, double scale, void* work, size_t work_bytes, cudaStream_t stream,
                    int64_t pair_lines = 0) {
  if (!plan || !in || !out) return SGPU_ERR_ARG;
  if (outer < 0 || inner < 1) return SGPU_ERR_ARG;
  if (data_kind != SGPU_REAL && data_kind != SGPU_COMPLEX) return SGPU_ERR_ARG;
  if (plan->tensor) {
    // contiguous lines: the fused kernel.  Its CTAs for different 128-output
    // parts of a line do not wait for one another, so it runs in place only
    // when one CTA covers every output (n <= 130); the split-copy kernels
    // (strided lines) run in place by construction
    if (plan->fused && inner == 1) {
      if (in == out && plan->fm.MT > 1) return SGPU_ERR_ARG;
      return lc::contract(plan->fm, (const double*)in, (double*)out, outer, data_kind == SGPU_COMPLEX, work,
                          work_bytes, nullptr, 0, stream);
    }
    return oz::contract(plan->tc, (const double*)in, (double*)out, outer * inner, inner,
                        data_kind == SGPU_COMPLEX, work, work_bytes, stream);
  }
  LinePlan p = plan->lp;  // per call: the pairing blocks of real lines
  p.pb = pair_lines > 0 && pair_lines < outer * inner ? pair_lines : 0;
  if (in == out && p.n_in != p.n_out) return SGPU_ERR_ARG;
  const int64_t nlines = outer * inner;
  if (nlines == 0) return SGPU_OK;
  if (plan->fvariant != 2 && fourier256(plan) && inner >= 16) {
    // variant 1: plain FP64, or the mixed form in fixed point, at 2 CTAs per
    // SM (the 3-CTA register budget spills)
    const int fv = plan->fvariant;
    const bool mixed = p.form == SGPU_MIXED_DF;
    const int ctas = (fv == 4 || fv == 6) ? 3 : 2;
    const int fixed = fv == 7 ? 2 : ((fv >= 5 || (fv == 1 && mixed)) ? 1 : 0);
    const int st = f256_launch(p, (const double*)in, (double*)out, nlines, inner, scale, ctas, fixed, stream);
    if (st != SGPU_ERR_UNSUPPORTED) return st;
  }
  const int dcx = data_complex_for(p, data_kind);
  // real data: one CTA per tlc complex slots (pairs of real lines)
  auto blocks_for = [&](const LinePlan& q) -> int64_t {
    const int lpb = lines_per_block(q, dcx);
    return dcx ? (nlines + lpb - 1) / lpb : (pair_slots(nlines, q.pb) + q.tlc - 1) / q.tlc;
  };
  // small launches (fewer tiles than twice the SMs): fewer lines per CTA,
  // so that a small array spreads over more SMs; every line's arithmetic is
  // the same at any tile size, so the results do not change
  {
    const int64_t target = 2 * (int64_t)sm_count();
    bool shrunk = false;
    while (p.tlc > 1 && blocks_for(p) < target) {
      p.tlc >>= 1;
      shrunk = true;
    }
    if (shrunk) p.smem = smem_bytes<double>(p.tlc, p.ld);
  }
  const int64_t nblocks = blocks_for(p);
  if (nblocks > 0x7fffffffLL) return SGPU_ERR_ARG;
  const int dc = data_complex_for(p, data_kind);
  const int G = xf_group(p.kind);
  const bool fourier = G == XF_G_R2C || G == XF_G_C2R || G == XF_G_C2C;
  const double* src = (const double*)in;
  double* dst = (double*)out;
  const unsigned nb = (unsigned)nblocks;
  if (p.form == SGPU_MIXED_DF)
    return fourier ? xf_launch_fourier_df(G, p, src, dst, dc, nlines, inner, scale, nb, stream)
                   : xf_launch_cheb_df(G, p, src, dst, dc, nlines, inner, scale, nb, stream);
  return fourier ? xf_launch_fourier_f64(G, p, src, dst, dc, nlines, inner, scale, nb, stream)
                 : xf_launch_cheb_f64(G, p, src, dst, dc, nlines, inner, scale, nb, stream);
}

extern "C" int sgpu_plan_execute_blocks(const sgpu_plan* plan, const void* in, void* out, int64_t outer,
                                        int64_t inner, int data_kind, double scale, void* work, size_t work_bytes,
                                        int64_t pair_lines, cudaStream_t stream) {
  if (pair_lines < 0) return SGPU_ERR_ARG;
  return plan_run(plan, in, out, outer, inner, data_kind, scale, work, work_bytes, stream, pair_lines);
}

extern "C" int sgpu_plan_execute_ws(const sgpu_plan* plan, const void* in, void* out, int64_t outer,
                                    int64_t inner, int data_kind, double scale, void* work, size_t work_bytes,
                                    cudaStream_t stream) {
  return plan_run(plan, in, out, outer, inner, data_kind, scale, work, work_bytes, stream);
}

// without a caller workspace the tensor form takes its scratch from the
// stream-ordered allocator for the duration of the call
extern "C" int sgpu_plan_execute(const sgpu_plan* plan, const void* in, void* out, int64_t outer,
                                 int64_t inner, int data_kind, double scale, cudaStream_t stream) {
  if (!plan || !plan->tensor || outer * inner == 0)
    return plan_run(plan, in, out, outer, inner, data_kind, scale, nullptr, 0, stream);
  size_t nb = 0;
  int st = sgpu_plan_workspace_size(plan, outer, inner, data_kind, &nb);
  if (st != SGPU_OK) return st;
  // the fused kernel on more than 128 outputs runs in place through a
  // temporary output appended to the scratch
  const bool tmp_out = plan->fused && inner == 1 && in == out && plan->fm.MT > 1;
  const size_t ob = tmp_out ? (size_t)outer * plan->lp.n_out * (data_kind == SGPU_COMPLEX ? 16 : 8) : 0;
  const size_t nb_r = (nb + 255) & ~(size_t)255;
  void* work = nullptr;
  if (cudaMallocAsync(&work, nb_r + ob, stream) != cudaSuccess) {
    cudaGetLastError();
    return SGPU_ERR_NOMEM;
  }
  void* dst = tmp_out ? (void*)((char*)work + nb_r) : out;
  st = plan_run(plan, in, dst, outer, inner, data_kind, scale, work, nb, stream);
  if (st == SGPU_OK && tmp_out && cudaMemcpyAsync(out, dst, ob, cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
    st = SGPU_ERR_CUDA;
  cudaFreeAsync(work, stream);
  cudaGetLastError();
  return st;
}
