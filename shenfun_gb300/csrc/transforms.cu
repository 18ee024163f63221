// Transform plans and the line-transform kernel (C ABI: sgpu_plan_*).
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "plan_host.cuh"

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

template <class R>
__global__ void __launch_bounds__(256) sgpu_line_kernel(LinePlan p, const double* in, double* out,
                                                        int data_complex, int64_t nlines,
                                                        int64_t inner, double scl) {
  extern __shared__ __align__(16) unsigned char sgpu_smem[];
  prog_dispatch<R>(p, in, out, data_complex, nlines, inner, scl, (int64_t)blockIdx.x, sgpu_smem,
                   (int)threadIdx.x, (int)blockDim.x);
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
  static bool attr_set = false;
  if (!attr_set) {
    if (cudaFuncSetAttribute(sgpu_line_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             220 * 1024) != cudaSuccess ||
        cudaFuncSetAttribute(sgpu_line_kernel<df>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             220 * 1024) != cudaSuccess) {
      cudaGetLastError();
      return SGPU_ERR_CUDA;
    }
    attr_set = true;
  }
  const int dc = data_complex_for(p, data_kind);
  if (p.form == SGPU_MIXED_DF)
    sgpu_line_kernel<df><<<(unsigned)nblocks, p.nthreads, p.smem, stream>>>(
        p, (const double*)in, (double*)out, dc, nlines, inner, scale);
  else
    sgpu_line_kernel<double><<<(unsigned)nblocks, p.nthreads, p.smem, stream>>>(
        p, (const double*)in, (double*)out, dc, nlines, inner, scale);
  if (cudaGetLastError() != cudaSuccess) return SGPU_ERR_CUDA;
  return SGPU_OK;
}
