// Device-resident Lanczos vector operations (the Krylov expansion of YASTN's eigs,
// yastn/tensor/_krylov.py:17-46 with yastn/krylov/_krylov.py:177-238, on the backend's
// vdot / add / norm, yastn/backend/backend_np.py:553-577).
//
// The Krylov basis is one (ncv + 1) x n matrix in HBM and the tridiagonal coefficients are
// device scalars, so a whole expansion runs without a host synchronisation and can be
// captured in a CUDA graph. Reductions are deterministic: a fixed grid of kParts CTAs writes
// per-CTA partial sums (each CTA sums a fixed strided set of elements in a fixed order, then
// a fixed shared-memory tree), and one warp adds the partials in a fixed order.
//
//   yb_krylov_dot:    s = sum_i conj(x_i) y_i                      (alpha_j = <V_j, w>)
//   yb_krylov_update: w <- w - alpha V_j - beta V_{j-1}, s = |w|    (one pass over w)
//   yb_krylov_norm:   s = |x|                                       (|v0|)
//   yb_krylov_scale:  v <- w / beta                                (V_{j+1} = w / beta_j)
//   yb_krylov_combine: y = sum_i c_i V_i                           (Ritz vectors)
#include "yb_common.cuh"

namespace yb {
namespace {

constexpr int kParts = 304;  // 2 CTAs per SM
constexpr int kThr = 256;

struct R64 {
  using T = double;
  __device__ static T zero() { return 0.0; }
  __device__ static T cdot(T a, T b) { return a * b; }  // conj(a) b
  __device__ static T add(T a, T b) { return a + b; }
  __device__ static double norm2(T a) { return a * a; }
  __device__ static T mul(T a, T b) { return a * b; }
  __device__ static T scale(T a, double s) { return a * s; }
  __device__ static T shfl(T v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
};

struct C128 {
  using T = double2;
  __device__ static T zero() { return make_double2(0.0, 0.0); }
  __device__ static T cdot(T a, T b) { return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x); }
  __device__ static T add(T a, T b) { return make_double2(a.x + b.x, a.y + b.y); }
  __device__ static double norm2(T a) { return a.x * a.x + a.y * a.y; }
  __device__ static T mul(T a, T b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
  __device__ static T scale(T a, double s) { return make_double2(a.x * s, a.y * s); }
  __device__ static T shfl(T v, int o) {
    return make_double2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
  }
};

// fixed-order block reduction of one value per thread
template <class F>
__device__ __forceinline__ typename F::T block_sum(typename F::T v) {
  using T = typename F::T;
  __shared__ T sh[kThr / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = F::add(v, F::shfl(v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  T s = F::zero();
  if (threadIdx.x == 0)
    for (int i = 0; i < kThr / 32; ++i) s = F::add(s, sh[i]);
  return s;  // valid in thread 0
}

template <class F>
__global__ void __launch_bounds__(kThr) dot_parts_kernel(const typename F::T* __restrict__ x,
                                                         const typename F::T* __restrict__ y, int64_t n,
                                                         typename F::T* __restrict__ parts) {
  using T = typename F::T;
  T acc = F::zero();
  for (int64_t i = (int64_t)blockIdx.x * kThr + threadIdx.x; i < n; i += (int64_t)kParts * kThr)
    acc = F::add(acc, F::cdot(x[i], y[i]));
  const T s = block_sum<F>(acc);
  if (threadIdx.x == 0) parts[blockIdx.x] = s;
}

// w <- w - alpha v1 - beta v0 (beta real, v0 optional), partial sums of |w|^2
template <class F>
__global__ void __launch_bounds__(kThr) update_kernel(typename F::T* __restrict__ w, const typename F::T* __restrict__ v1,
                                                      const typename F::T* __restrict__ v0,
                                                      const typename F::T* __restrict__ alpha,
                                                      const double* __restrict__ beta, int64_t n,
                                                      double* __restrict__ parts) {
  using T = typename F::T;
  const T a = *alpha;
  const double b = v0 ? *beta : 0.0;
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThr + threadIdx.x; i < n; i += (int64_t)kParts * kThr) {
    T t = F::add(w[i], F::scale(F::mul(a, v1[i]), -1.0));
    if (v0) t = F::add(t, F::scale(v0[i], -b));
    w[i] = t;
    acc += F::norm2(t);
  }
  const double s = block_sum<R64>(acc);
  if (threadIdx.x == 0) parts[blockIdx.x] = s;
}

// out = the sum of the parts (one warp: lane l adds parts l, l + 32, ... in order, then a fixed
// shuffle tree, so the result does not depend on timing); finish_norm_kernel: out = sqrt(sum)
template <class F>
__global__ void finish_kernel(const typename F::T* __restrict__ parts, typename F::T* __restrict__ out, int n_parts) {
  using T = typename F::T;
  T s = F::zero();
  for (int i = threadIdx.x; i < n_parts; i += 32) s = F::add(s, parts[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s = F::add(s, F::shfl(s, o));
  if (threadIdx.x == 0) *out = s;
}

__global__ void finish_norm_kernel(const double* __restrict__ parts, double* __restrict__ out, int n_parts) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n_parts; i += 32) s += parts[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (threadIdx.x == 0) *out = sqrt(s);
}

template <class F>
__global__ void __launch_bounds__(kThr) norm_parts_kernel(const typename F::T* __restrict__ x, int64_t n,
                                                          double* __restrict__ parts) {
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThr + threadIdx.x; i < n; i += (int64_t)kParts * kThr) acc += F::norm2(x[i]);
  const double s = block_sum<R64>(acc);
  if (threadIdx.x == 0) parts[blockIdx.x] = s;
}

template <class F>
__global__ void __launch_bounds__(kThr) scale_kernel(const typename F::T* __restrict__ w, const double* __restrict__ beta,
                                                     int64_t n, typename F::T* __restrict__ out) {
  const double inv = 1.0 / *beta;
  for (int64_t i = (int64_t)blockIdx.x * kThr + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThr)
    out[i] = F::scale(w[i], inv);
}

// y = sum_{i < m} c_i V_i, V row-major m x n (row stride ldv elements)
template <class F>
__global__ void __launch_bounds__(kThr) combine_kernel(const typename F::T* __restrict__ V, int64_t ldv,
                                                       const typename F::T* __restrict__ c, int m, int64_t n,
                                                       typename F::T* __restrict__ y) {
  using T = typename F::T;
  for (int64_t i = (int64_t)blockIdx.x * kThr + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThr) {
    T acc = F::zero();
    for (int r = 0; r < m; ++r) acc = F::add(acc, F::mul(c[r], V[r * ldv + i]));
    y[i] = acc;
  }
}

inline unsigned grid_for(int64_t n) {
  const int64_t g = (n + kThr - 1) / kThr;
  return (unsigned)(g < 4 * kParts ? (g > 0 ? g : 1) : 4 * kParts);
}

}  // namespace
}  // namespace yb

extern "C" {

int yb_krylov_parts(void) { return yb::kParts; }

int yb_krylov_dot(const void* x, const void* y, int64_t n, int dtype, void* parts, void* out, void* stream) {
  if (!x || !y || !parts || !out || n < 0) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64) {
    yb::dot_parts_kernel<yb::R64><<<yb::kParts, yb::kThr, 0, s>>>((const double*)x, (const double*)y, n, (double*)parts);
    yb::finish_kernel<yb::R64><<<1, 32, 0, s>>>((const double*)parts, (double*)out, yb::kParts);
  } else if (dtype == YB_C128) {
    yb::dot_parts_kernel<yb::C128><<<yb::kParts, yb::kThr, 0, s>>>((const double2*)x, (const double2*)y, n,
                                                                  (double2*)parts);
    yb::finish_kernel<yb::C128><<<1, 32, 0, s>>>((const double2*)parts, (double2*)out, yb::kParts);
  } else {
    return YB_ERR_INVALID;
  }
  return yb::check_launch();
}

int yb_krylov_update(void* w, const void* v1, const void* v0, const void* alpha, const double* beta, int64_t n,
                     int dtype, double* parts, double* norm_out, void* stream) {
  if (!w || !v1 || !alpha || !parts || !norm_out || n < 0 || (v0 && !beta)) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64)
    yb::update_kernel<yb::R64><<<yb::kParts, yb::kThr, 0, s>>>((double*)w, (const double*)v1, (const double*)v0,
                                                             (const double*)alpha, beta, n, parts);
  else if (dtype == YB_C128)
    yb::update_kernel<yb::C128><<<yb::kParts, yb::kThr, 0, s>>>((double2*)w, (const double2*)v1, (const double2*)v0,
                                                              (const double2*)alpha, beta, n, parts);
  else
    return YB_ERR_INVALID;
  yb::finish_norm_kernel<<<1, 32, 0, s>>>(parts, norm_out, yb::kParts);
  return yb::check_launch();
}

int yb_krylov_norm(const void* x, int64_t n, int dtype, double* parts, double* out, void* stream) {
  if (!x || !parts || !out || n < 0) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64)
    yb::norm_parts_kernel<yb::R64><<<yb::kParts, yb::kThr, 0, s>>>((const double*)x, n, parts);
  else if (dtype == YB_C128)
    yb::norm_parts_kernel<yb::C128><<<yb::kParts, yb::kThr, 0, s>>>((const double2*)x, n, parts);
  else
    return YB_ERR_INVALID;
  yb::finish_norm_kernel<<<1, 32, 0, s>>>(parts, out, yb::kParts);
  return yb::check_launch();
}

int yb_krylov_scale(const void* w, const double* beta, int64_t n, int dtype, void* out, void* stream) {
  if (!w || !beta || !out || n < 0) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64)
    yb::scale_kernel<yb::R64><<<yb::grid_for(n), yb::kThr, 0, s>>>((const double*)w, beta, n, (double*)out);
  else if (dtype == YB_C128)
    yb::scale_kernel<yb::C128><<<yb::grid_for(n), yb::kThr, 0, s>>>((const double2*)w, beta, n, (double2*)out);
  else
    return YB_ERR_INVALID;
  return yb::check_launch();
}

int yb_krylov_combine(const void* V, int64_t ldv, const void* coeffs, int m, int64_t n, int dtype, void* y,
                      void* stream) {
  if (!V || !coeffs || !y || m < 0 || n < 0) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64)
    yb::combine_kernel<yb::R64><<<yb::grid_for(n), yb::kThr, 0, s>>>((const double*)V, ldv, (const double*)coeffs, m,
                                                                   n, (double*)y);
  else if (dtype == YB_C128)
    yb::combine_kernel<yb::C128><<<yb::grid_for(n), yb::kThr, 0, s>>>((const double2*)V, ldv,
                                                                    (const double2*)coeffs, m, n, (double2*)y);
  else
    return YB_ERR_INVALID;
  return yb::check_launch();
}

}  // extern "C"
