// Internal C++ interface of the fused split-BF16 line contraction
// (lc_fused.cu), used by the mixed-form Chebyshev plans for contiguous lines.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace sgpu {
namespace lc {

// a fixed N x N matrix M (row-major, out(l, n) = sum_k in(l, k) M[k][n]) with
// K leading nonzero rows, split into BF16 digits for the tensor cores
struct Matrix {
  int N = 0, K = 0;
  int MT = 0;     // CTAs per tile group (128-output tiles)
  int Nmma = 0;   // outputs on the tensor cores
  int NX = 0;     // outputs as FP64 dot products
  uint16_t* tiles = nullptr;  // device: digit tiles | exponents | dot-product columns
  int* em = nullptr;
  double* xcol = nullptr;     // dot-product columns [NX][K]
  int variant = 1;            // tiles: 1 = 64 lines, one accumulator set; 2 = 32 lines, two sets
};

// true when the fused contraction handles (N, K): 16 <= N <= 514 and
// K <= 339 (the exactness bound of its leading digit groups)
bool supported(int N, int K);
int matrix_create(const double* M_host, int N, int K, Matrix* out);
void matrix_destroy(Matrix* m);
// device scratch of a contraction: 4 bytes per row (the line scales)
size_t workspace_bytes(const Matrix& m, int64_t nlines, int cplx);
// out = in . M along contiguous lines (inner = 1) of a (nlines, N) real or
// (nlines, N) complex array; in may alias out when MT = 1 (N <= 130).  work:
// workspace_bytes of scratch, 256-byte aligned.  err (device int, may be
// null) gets bit 0 set when a bounded wait of the launch gave up; wait_ns
// (0: one second) bounds each pipeline wait.
// bounded waits of the fused kernel that gave up since the library was loaded
int read_timeouts(unsigned int* count);
int contract(const Matrix& m, const double* in, double* out, int64_t nlines, int cplx, void* work, size_t work_bytes,
             int* err, uint64_t wait_ns, cudaStream_t stream);

}  // namespace lc
}  // namespace sgpu
