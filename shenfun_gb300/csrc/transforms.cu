// Transform plans (C ABI: sgpu_plan_*); the kernels are in xf_*.cu.
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "plan_host.cuh"
#include "xf_kernels.cuh"

using namespace sgpu;

struct sgpu_plan {
  LinePlan lp;
  void* dev_tables;  // one allocation holding every device table
};

extern "C" int sgpu_plan_create(sgpu_plan** out, int kind, int n, int basis, int form) {
  if (!out) return SGPU_ERR_ARG;
  *out = nullptr;
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
  delete plan;
  return SGPU_OK;
}

extern "C" int sgpu_plan_execute(const sgpu_plan* plan, const void* in, void* out, int64_t outer,
                                 int64_t inner, int data_kind, double scale, cudaStream_t stream) {
  if (!plan || !in || !out) return SGPU_ERR_ARG;
  if (outer < 0 || inner < 1) return SGPU_ERR_ARG;
  if (data_kind != SGPU_REAL && data_kind != SGPU_COMPLEX) return SGPU_ERR_ARG;
  const LinePlan& p = plan->lp;
  if (in == out && p.n_in != p.n_out) return SGPU_ERR_ARG;
  const int64_t nlines = outer * inner;
  if (nlines == 0) return SGPU_OK;
  const int lpb = lines_per_block(p, data_complex_for(p, data_kind));
  const int64_t nblocks = (nlines + lpb - 1) / lpb;
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
