// Internal C++ interface of the split-BF16 tensor-core line contraction
// (ozaki_tc.cu), used by the Legendre plans.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace sgpu {
namespace oz {

// a fixed N x N matrix M (row-major, out(l, n) = sum_k in(l, k) M[k][n]),
// split into BF16 digit slices and tiled on the device
struct Matrix {
  int N = 0, S = 0;
  int K = 0;                  // 1 + the last nonzero row: input entries the contraction reads
  int precise = 0;            // 0: 7 digits (~1e-13 normwise), 1: 8 digits (~1e-15)
  uint16_t* tiles = nullptr;  // device: slices, then per-column exponents
  int* exps = nullptr;
};

// OK for contraction lengths 1 <= K <= 8192: each GEMM launch sums at most
// 1024 of them (the FP32 sums of the exact digit groups stay below 2^24)
// and longer contractions add the launches' FP64 results; else UNSUPPORTED
int pick_digits(int K);
int matrix_create(const double* M_host, int N, int precise, Matrix* out);
void matrix_destroy(Matrix* m);
// device scratch one contraction of `nlines` lines needs (256-byte aligned)
size_t workspace_bytes(const Matrix& m, int64_t nlines, int64_t inner, int cplx);
// out = in . M along lines of a (outer, N, inner) array (in != out)
int contract(const Matrix& m, const double* in, double* out, int64_t nlines, int64_t inner, int cplx,
             void* work, size_t work_bytes, cudaStream_t stream);

}  // namespace oz
}  // namespace sgpu
