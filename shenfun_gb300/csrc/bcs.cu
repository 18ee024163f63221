// Non-homogeneous boundary values on a Chebyshev ShenDirichlet / ShenNeumann
// axis: the right-hand-side correction of the two boundary dofs
// (BoundaryValues._add_mass_rhs, tensorproductspace.py:2091-2106, and the
// boundary matrices a Helmholtz solve subtracts, chebyshev/la.py:302-306)
// and the boundary dofs themselves (set_boundary_dofs, :2108-2128).
//
// One thread per line of a (outer, N, inner) array: consecutive threads own
// consecutive inner indices, so every row access is coalesced.  Lines whose
// two boundary values are zero (every Fourier mode but the mean for constant
// wall values) only read g.
#include "solvers.cuh"

using namespace sgpu;

template <class T>
__global__ void __launch_bounds__(128)
    k_bc_apply(T* u, const double* CA, const double* alfa, const double* CB, const double* beta,
               const T* g, int64_t N, int64_t inner, int64_t nsys, int set_dofs) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) bc_apply_prog<T>(u, CA, alfa, CB, beta, g, N, inner, s, set_dofs);
}

extern "C" int sgpu_bc_apply(void* u, const double* CA, const double* alfa, const double* CB,
                             const double* beta, const void* g, int64_t outer, int64_t N,
                             int64_t inner, int set_dofs, int data_kind, cudaStream_t stream) {
  if (!u || !g || N < 4 || outer < 0 || inner < 1 || (set_dofs != 0 && set_dofs != 1))
    return SGPU_ERR_ARG;
  const int64_t nsys = outer * inner;
  if (nsys == 0) return SGPU_OK;
  const unsigned nb = (unsigned)((nsys + 127) / 128);
  if (data_kind == SGPU_COMPLEX)
    k_bc_apply<cd><<<nb, 128, 0, stream>>>((cd*)u, CA, alfa, CB, beta, (const cd*)g, N, inner, nsys,
                                           set_dofs);
  else if (data_kind == SGPU_REAL)
    k_bc_apply<double><<<nb, 128, 0, stream>>>((double*)u, CA, alfa, CB, beta, (const double*)g, N,
                                               inner, nsys, set_dofs);
  else
    return SGPU_ERR_ARG;
  return cudaGetLastError() == cudaSuccess ? SGPU_OK : SGPU_ERR_CUDA;
}
