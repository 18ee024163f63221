// Library-level C ABI: status strings, version, device check.
#include "sgpu_common.cuh"

extern "C" const char* sgpu_status_string(int status) {
  switch (status) {
    case SGPU_OK: return "ok";
    case SGPU_ERR_ARG: return "invalid argument (shape, pointer or enum)";
    case SGPU_ERR_UNSUPPORTED: return "unsupported request";
    case SGPU_ERR_CUDA: return "CUDA runtime error";
    case SGPU_ERR_NOMEM: return "out of device memory for plan tables";
    case SGPU_ERR_NONFINITE: return "non-finite input";
    case SGPU_ERR_ZERO_PIVOT: return "zero pivot";
    case SGPU_ERR_TIMEOUT: return "bounded device wait ran out";
    case SGPU_ERR_SCRATCH_LIMIT:
      return "problem needs more scratch than the allocation-free entry point's 64 MiB";
    default: return "unknown status";
  }
}

extern "C" int sgpu_version(void) { return 100; }

__global__ void k_probe(int* flag) { *flag = 103; }

extern "C" int sgpu_device_ok(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return 0;
  }
  int* d = nullptr;
  if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  k_probe<<<1, 1>>>(d);
  int h = 0;
  cudaError_t e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return h == 103;
}
