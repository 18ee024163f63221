// Common definitions for the shenfun_gb300 kernels.
//
// Every kernel body in this library is written as a __host__ __device__
// "block program": a function of (block index, thread index, thread count,
// shared-memory pointer) whose phases are thread-strided loops separated by
// SGPU_SYNC().  The CUDA kernels call it with threadIdx/blockDim; the CPU
// index-check harness (tests/kernel_emu) calls the same function with one
// "thread" per block, so every index and buffer bound is exercised on the
// CPU before a GPU ever runs the code.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#ifdef __CUDA_ARCH__
#define SGPU_SYNC() __syncthreads()
#else
#define SGPU_SYNC() ((void)0)
#endif

#ifdef __CUDACC__
#define SGPU_HD __host__ __device__ __forceinline__
#else
// plain host compilers (the CPU harness): ordinary inline functions, so the
// sanitizer build stays small
#define SGPU_HD inline
#endif

#include "../../include/shenfun_gb300.h"

namespace sgpu {

// ---------------------------------------------------------------------------
// complex arithmetic on a real type R (double for the plain form)
template <class R>
struct Cx {
  R re, im;
};

template <class R>
SGPU_HD Cx<R> cx(R a, R b) {
  Cx<R> z;
  z.re = a;
  z.im = b;
  return z;
}
template <class R>
SGPU_HD Cx<R> operator+(Cx<R> a, Cx<R> b) { return cx<R>(a.re + b.re, a.im + b.im); }
template <class R>
SGPU_HD Cx<R> operator-(Cx<R> a, Cx<R> b) { return cx<R>(a.re - b.re, a.im - b.im); }
template <class R>
SGPU_HD Cx<R> operator*(Cx<R> a, Cx<R> b) {
  return cx<R>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <class R>
SGPU_HD Cx<R> scale(Cx<R> a, R s) { return cx<R>(a.re * s, a.im * s); }
template <class R>
SGPU_HD Cx<R> conj(Cx<R> a) { return cx<R>(a.re, -a.im); }
// multiply by -i
template <class R>
SGPU_HD Cx<R> mul_mi(Cx<R> a) { return cx<R>(a.im, -a.re); }
// multiply by +i
template <class R>
SGPU_HD Cx<R> mul_pi(Cx<R> a) { return cx<R>(-a.im, a.re); }

// specialisation of the complex product with fused multiply-adds
SGPU_HD Cx<double> operator*(Cx<double> a, Cx<double> b) {
  Cx<double> z;
  z.re = fma(a.re, b.re, -a.im * b.im);
  z.im = fma(a.re, b.im, a.im * b.re);
  return z;
}

typedef Cx<double> cd;

SGPU_HD int imin(int a, int b) { return a < b ? a : b; }
SGPU_HD int imax(int a, int b) { return a > b ? a : b; }

}  // namespace sgpu
