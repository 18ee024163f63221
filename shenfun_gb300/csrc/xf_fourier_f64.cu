// Fourier line-transform kernels (R2C, C2R, C2C), f64 arithmetic.
#include "xf_kernels.cuh"

namespace sgpu {
int xf_launch_fourier_f64(int G, const LinePlan& p, const double* in, double* out, int dc,
                          int64_t nlines, int64_t inner, double scl, unsigned nblocks, cudaStream_t s) {
  switch (G) {
    case XF_G_R2C: return xf_launch_group<double, XF_G_R2C>(p, in, out, dc, nlines, inner, scl, nblocks, s);
    case XF_G_C2R: return xf_launch_group<double, XF_G_C2R>(p, in, out, dc, nlines, inner, scl, nblocks, s);
    case XF_G_C2C: return xf_launch_group<double, XF_G_C2C>(p, in, out, dc, nlines, inner, scl, nblocks, s);
    default: return SGPU_ERR_ARG;
  }
}
}  // namespace sgpu
