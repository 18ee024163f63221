// Chebyshev line-transform kernels (DCT-II and DCT-III families with the
// fused scaling, Shen stencil, mass solve and to_ortho), df arithmetic.
#include "xf_kernels.cuh"

namespace sgpu {
int xf_launch_cheb_df(int G, const LinePlan& p, const double* in, double* out, int dc,
                       int64_t nlines, int64_t inner, double scl, unsigned nblocks, cudaStream_t s) {
  switch (G) {
    case XF_G_DCT2: return xf_launch_group<df, XF_G_DCT2>(p, in, out, dc, nlines, inner, scl, nblocks, s);
    case XF_G_DCT3: return xf_launch_group<df, XF_G_DCT3>(p, in, out, dc, nlines, inner, scl, nblocks, s);
    default: return SGPU_ERR_ARG;
  }
}
}  // namespace sgpu
