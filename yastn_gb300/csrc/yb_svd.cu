// Family (c): batched one-sided (Hestenes) Jacobi SVD of all charge-sector blocks.
//
// Each block A (m x n, row-major) is handled in its "wide" orientation: the k=min(m,n)
// vectors to orthogonalise are the rows of A (m <= n) or of A^T (m > n), each of
// length L=max(m,n), copied into a workspace X. A parallel round-robin ordering
// (circle method over N = k rounded up to even) pairs all vectors in N-1 rounds of
// N/2 disjoint pairs; one warp rotates one pair, all blocks advance in the same
// launch. Rotations are accumulated in W (k x k, starting at I), so that
// X_final = W X_0 with orthogonal rows; then S = row norms, the normalised rows give
// Vh (wide) or U (tall), and W^T gives the other factor. The host launches sweeps
// until no rotation was applied in a sweep or the sweep cap is hit (reported as
// YB_ERR_NOT_CONVERGED by the host layer). No kernel waits on another CTA.
//
// A rotation is applied when |x_p.x_q| > tol * ||x_p|| ||x_q|| with tol = sqrt(L) * eps
// (the threshold of LAPACK's one-sided Jacobi); the angle follows Rutishauser's
// stable formula with hypot to avoid overflow.
#include <float.h>
#include "yb_common.cuh"

namespace yb {
namespace {

constexpr int kWarps = 8;

// record fields
enum { R_A = 0, R_M, R_N, R_U, R_S, R_V, R_X, R_W, R_P, R_K, R_L, R_NP, R_T };

// Per-block Frobenius norm -> shift[b] (used to make a symmetric block positive definite).
__global__ void block_fro_kernel(const double* __restrict__ A, const int64_t* __restrict__ blocks,
                                 double* __restrict__ shift) {
  __shared__ double red[32];
  const int64_t* r = blocks + (int64_t)blockIdx.x * YB_SVD_REC;
  const int64_t cnt = r[R_M] * r[R_N];
  const double* a = A + r[R_A];
  double acc = 0.0;
  for (int64_t e = threadIdx.x; e < cnt; e += blockDim.x) acc = fma(a[e], a[e], acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    // ||A||_2 <= ||A||_F: A + shift*I is positive definite; the +1 keeps an all-zero block regular
    shift[blockIdx.x] = sqrt(tot) + 1.0;
  }
}

__global__ void svd_init_kernel(const double* __restrict__ A, double* __restrict__ work,
                                const int64_t* __restrict__ blocks, int64_t* __restrict__ counters,
                                int n_blocks, const double* __restrict__ shift) {
  const int64_t* r = blocks + (int64_t)blockIdx.y * YB_SVD_REC;
  const int64_t m = r[R_M], n = r[R_N], k = r[R_K], L = r[R_L];
  const bool tall = m > n;
  const int64_t xs = k * L, ws = k * k;
  double* X = work + r[R_X];
  double* W = work + r[R_W];
  const double* a = A + r[R_A];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < xs + ws;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (e < xs) {
      const int64_t i = e / L, l = e - i * L;
      double v = tall ? a[l * n + i] : a[e];
      if (shift != nullptr && i == l) v += shift[blockIdx.y];
      X[e] = v;
    } else {
      const int64_t f = e - xs;
      const int64_t i = f / k, j = f - i * k;
      W[f] = (i == j) ? 1.0 : 0.0;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    counters[blockIdx.y] = 1;             // rotations in the last completed sweep (1 = active)
    counters[n_blocks + blockIdx.y] = 0;  // rotations in the sweep in progress
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(kWarps * 32) svd_round_kernel(double* __restrict__ work,
                                                                const int64_t* __restrict__ blocks,
                                                                const int32_t* __restrict__ pair_items,
                                                                int n_items, int round, double tol_scale,
                                                                int64_t* __restrict__ counters,
                                                                int n_blocks) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int item = blockIdx.x * kWarps + warp;
  if (item >= n_items) return;
  const int b = pair_items[2 * item];
  const int pi = pair_items[2 * item + 1];
  if (counters[b] == 0) return;  // block converged in the previous sweep
  const int64_t* r = blocks + (int64_t)b * YB_SVD_REC;
  const int64_t k = r[R_K], L = r[R_L], N = r[R_NP];
  if (round >= N - 1) return;
  int64_t p, q;
  if (pi == 0) {
    p = N - 1;
    q = round;
  } else {
    p = (round + pi) % (N - 1);
    q = (round - pi + (N - 1)) % (N - 1);
  }
  if (p >= k || q >= k) return;  // dummy vector of an odd count
  if (p > q) { int64_t t = p; p = q; q = t; }
  double* X = work + r[R_X];
  double* W = work + r[R_W];
  double* xp = X + p * L;
  double* xq = X + q * L;
  double al = 0.0, be = 0.0, ga = 0.0;
  for (int64_t l = lane; l < L; l += 32) {
    const double u = xp[l], v = xq[l];
    al = fma(u, u, al);
    be = fma(v, v, be);
    ga = fma(u, v, ga);
  }
  al = warp_sum(al);
  be = warp_sum(be);
  ga = warp_sum(ga);
  const double tol = tol_scale * sqrt((double)L) * DBL_EPSILON;
  if (!(fabs(ga) > tol * sqrt(al) * sqrt(be))) return;  // also skips zero vectors
  const double zeta = (be - al) / (2.0 * ga);
  const double t = copysign(1.0, zeta) / (fabs(zeta) + hypot(1.0, zeta));
  const double c = 1.0 / sqrt(fma(t, t, 1.0));
  const double s = c * t;
  for (int64_t l = lane; l < L; l += 32) {
    const double u = xp[l], v = xq[l];
    xp[l] = fma(c, u, -s * v);
    xq[l] = fma(s, u, c * v);
  }
  double* wp = W + p * k;
  double* wq = W + q * k;
  for (int64_t l = lane; l < k; l += 32) {
    const double u = wp[l], v = wq[l];
    wp[l] = fma(c, u, -s * v);
    wq[l] = fma(s, u, c * v);
  }
  if (lane == 0) atomicAdd((unsigned long long*)&counters[n_blocks + b], 1ull);
}

__global__ void svd_sweep_end_kernel(int64_t* counters, int n_blocks) {
  for (int b = threadIdx.x; b < n_blocks; b += blockDim.x) {
    if (counters[b] != 0) counters[b] = counters[n_blocks + b];
    counters[n_blocks + b] = 0;
  }
}

// One CTA per block: singular values = row norms, sort descending (index tie-break),
// write U, S, Vh; vectors of zero norm are completed to an orthonormal set.
// mode 0: SVD (S descending). mode 1/2: symmetric eigendecomposition of a block that
// was shifted by shift[b] (lambda = sigma - shift), eigenvectors = columns of W^T,
// ordered ascending (1) or by |lambda| descending (2); Vh is not written.
__global__ void __launch_bounds__(1024) svd_finalize_kernel(const double* __restrict__ work,
                                                            double* __restrict__ U, double* __restrict__ S,
                                                            double* __restrict__ Vh,
                                                            const int64_t* __restrict__ blocks, int pow2,
                                                            int mode, const double* __restrict__ shift) {
  extern __shared__ unsigned char smem_raw[];
  double* sig = reinterpret_cast<double*>(smem_raw);
  int* idx = reinterpret_cast<int*>(sig + pow2);
  __shared__ int n_zero;
  const int64_t* r = blocks + (int64_t)blockIdx.x * YB_SVD_REC;
  const int64_t m = r[R_M], n = r[R_N], k = r[R_K], L = r[R_L];
  const bool tall = m > n;
  const double* X = work + r[R_X];
  const double* W = work + r[R_W];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) n_zero = 0;
  for (int i = threadIdx.x; i < pow2; i += blockDim.x) {
    sig[i] = -1.0;  // padding sorts last
    idx[i] = i;
  }
  __syncthreads();
  for (int64_t i = warp; i < k; i += nw) {
    double acc = 0.0;
    for (int64_t l = lane; l < L; l += 32) acc = fma(X[i * L + l], X[i * L + l], acc);
    acc = warp_sum(acc);
    if (lane == 0) {
      const double sv = sqrt(acc);
      sig[i] = (mode == 0) ? sv : (mode == 1 ? -(sv - shift[blockIdx.x]) : fabs(sv - shift[blockIdx.x]));
    }
  }
  __syncthreads();
  if (mode != 0) {
    // sort keys may be negative: shift them so that the -1 padding still sorts last
    __shared__ double kmin;
    if (threadIdx.x == 0) {
      double mn = 0.0;
      for (int64_t i = 0; i < k; ++i) mn = fmin(mn, sig[i]);
      kmin = mn;
    }
    __syncthreads();
    for (int64_t i = threadIdx.x; i < k; i += blockDim.x) sig[i] -= kmin;
    __syncthreads();
  }
  // bitonic sort, descending by value, ascending index on ties
  for (int size = 2; size <= pow2; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < pow2; i += blockDim.x) {
        const int j = i ^ stride;
        if (j > i) {
          const bool up = ((i & size) == 0);
          const double vi = sig[i], vj = sig[j];
          const int ii = idx[i], ij = idx[j];
          const bool i_first = (vi > vj) || (vi == vj && ii < ij);
          if (up != i_first) {
            sig[i] = vj; sig[j] = vi;
            idx[i] = ij; idx[j] = ii;
          }
        }
      }
      __syncthreads();
    }
  }
  double* Sb = S + r[R_S];
  double* Ub = U + r[R_U];
  double* Vb = Vh + r[R_V];
  if (mode != 0) {
    // eigenvalue = (row norm) - shift, recomputed from X to avoid the key transform
    for (int64_t j = warp; j < k; j += nw) {
      const int64_t i = idx[j];
      double acc = 0.0;
      for (int64_t l = lane; l < L; l += 32) acc = fma(X[i * L + l], X[i * L + l], acc);
      acc = warp_sum(acc);
      if (lane == 0) Sb[j] = sqrt(acc) - shift[blockIdx.x];
    }
    for (int64_t e = threadIdx.x; e < k * k; e += blockDim.x) {
      const int64_t j = e / k, c = e - j * k;
      Ub[c * k + j] = W[(int64_t)idx[j] * k + c];
    }
    return;
  }
  for (int j = threadIdx.x; j < k; j += blockDim.x) {
    Sb[j] = sig[j];
    if (!(sig[j] > 0.0)) atomicAdd(&n_zero, 1);
  }
  // normalised rows -> Vh (wide) or U columns (tall); W rows -> U columns (wide) or Vh rows (tall)
  for (int64_t e = threadIdx.x; e < k * L; e += blockDim.x) {
    const int64_t j = e / L, l = e - j * L;
    const double sv = sig[j];
    const double v = (sv > 0.0) ? X[(int64_t)idx[j] * L + l] / sv : 0.0;
    if (tall) Ub[l * k + j] = v; else Vb[j * n + l] = v;
  }
  for (int64_t e = threadIdx.x; e < k * k; e += blockDim.x) {
    const int64_t j = e / k, c = e - j * k;
    const double w = W[(int64_t)idx[j] * k + c];
    if (tall) Vb[j * n + c] = w; else Ub[c * k + j] = w;
  }
  __syncthreads();
  if (n_zero == 0) return;
  // completion: zero singular values sit at the end (positions k - n_zero .. k-1); replace
  // their vectors by unit vectors orthogonalised (twice) against all earlier ones.
  __shared__ double red[32];
  __shared__ double coef;
  const int64_t stride_v = tall ? k : 1;     // distance between consecutive entries of one vector
  const int64_t stride_j = tall ? 1 : n;     // distance between vectors
  double* base = tall ? Ub : Vb;
  for (int64_t j = k - n_zero; j < k; ++j) {
    for (int64_t cand = 0; cand < L; ++cand) {
      double* vj = base + j * stride_j;
      for (int64_t l = threadIdx.x; l < L; l += blockDim.x) vj[l * stride_v] = (l == cand) ? 1.0 : 0.0;
      __syncthreads();
      for (int pass = 0; pass < 2; ++pass) {
        for (int64_t i = 0; i < j; ++i) {
          const double* vi = base + i * stride_j;
          double acc = 0.0;
          for (int64_t l = threadIdx.x; l < L; l += blockDim.x) acc = fma(vi[l * stride_v], vj[l * stride_v], acc);
          acc = warp_sum(acc);
          if (lane == 0) red[warp] = acc;
          __syncthreads();
          if (threadIdx.x == 0) {
            double tot = 0.0;
            for (int w = 0; w < nw; ++w) tot += red[w];
            coef = tot;
          }
          __syncthreads();
          const double cf = coef;
          for (int64_t l = threadIdx.x; l < L; l += blockDim.x) vj[l * stride_v] -= cf * vi[l * stride_v];
          __syncthreads();
        }
      }
      double acc = 0.0;
      for (int64_t l = threadIdx.x; l < L; l += blockDim.x) acc = fma(vj[l * stride_v], vj[l * stride_v], acc);
      acc = warp_sum(acc);
      if (lane == 0) red[warp] = acc;
      __syncthreads();
      if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < nw; ++w) tot += red[w];
        coef = sqrt(tot);
      }
      __syncthreads();
      const double nrm = coef;
      if (nrm > 0.5) {
        for (int64_t l = threadIdx.x; l < L; l += blockDim.x) vj[l * stride_v] /= nrm;
        __syncthreads();
        break;
      }
      __syncthreads();
    }
  }
}

}  // namespace
}  // namespace yb

extern "C" {

int yb_svd_init(const void* a, void* work, const int64_t* blocks, int n_blocks, int dtype, int64_t* counters,
                double* shift, void* stream) {
  if (n_blocks == 0) return YB_OK;
  if (dtype != YB_F64) return YB_ERR_INVALID;
  if (!a || !work || !blocks || !counters) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (shift != nullptr) {
    yb::block_fro_kernel<<<n_blocks, 256, 0, s>>>((const double*)a, blocks, shift);
  }
  dim3 grid(64, (unsigned)n_blocks);
  yb::svd_init_kernel<<<grid, 256, 0, s>>>((const double*)a, (double*)work, blocks, counters, n_blocks, shift);
  return yb::check_launch();
}

int yb_svd_sweep(void* work, const int64_t* blocks, int n_blocks, const int32_t* pair_items, int n_pair_items,
                 int max_rounds, int dtype, double tol, int64_t* counters, void* stream) {
  if (n_blocks == 0 || n_pair_items == 0) return YB_OK;
  if (dtype != YB_F64) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const int grid = (n_pair_items + yb::kWarps - 1) / yb::kWarps;
  for (int rd = 0; rd < max_rounds; ++rd) {
    yb::svd_round_kernel<<<grid, yb::kWarps * 32, 0, s>>>((double*)work, blocks, pair_items, n_pair_items, rd, tol,
                                                          counters, n_blocks);
  }
  yb::svd_sweep_end_kernel<<<1, 256, 0, s>>>(counters, n_blocks);
  return yb::check_launch();
}

int yb_svd_finalize(const void* work, void* U, double* S, void* Vh, const int64_t* blocks, int n_blocks, int dtype,
                    int max_k, int mode, const double* shift, void* stream) {
  if (n_blocks == 0) return YB_OK;
  if (dtype != YB_F64) return YB_ERR_INVALID;
  if (mode < 0 || mode > 2 || (mode != 0 && shift == nullptr)) return YB_ERR_INVALID;
  if (max_k > 8192) return YB_ERR_TOO_LARGE;
  int pow2 = 1;
  while (pow2 < max_k) pow2 <<= 1;
  const size_t smem = (size_t)pow2 * (sizeof(double) + sizeof(int));
  cudaStream_t s = (cudaStream_t)stream;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(yb::svd_finalize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) { yb::set_cuda_error((int)e); return YB_ERR_CUDA; }
  }
  yb::svd_finalize_kernel<<<n_blocks, 1024, smem, s>>>((const double*)work, (double*)U, S, (double*)Vh, blocks, pow2,
                                                       mode, shift);
  return yb::check_launch();
}

}  // extern "C"
