// Shared helpers for the yastn_gb300 CUDA kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <cuComplex.h>
#include "../../include/yastn_gb300.h"

namespace yb {

// Records the last CUDA error for yb_last_cuda_error().
void set_cuda_error(int code);

// Checks the launch that was just enqueued; returns YB_OK or YB_ERR_CUDA.
inline int check_launch() {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_cuda_error((int)e);
    return YB_ERR_CUDA;
  }
  return YB_OK;
}

// Division by a run-time constant d (1 <= d < 2^31) for dividends n < 2^31:
// q = (umulhi(n, magic) + n) >> shift, with shift = ceil(log2 d) and
// magic = floor(2^32 (2^shift - d) / d) + 1 (Granlund-Montgomery round-up method).
__device__ __forceinline__ uint32_t fast_div(uint32_t n, uint32_t magic, uint32_t shift) {
  return (__umulhi(n, magic) + n) >> shift;
}

// Complex helpers on double2 (x = real, y = imag).
struct cplx {
  double re, im;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

}  // namespace yb
