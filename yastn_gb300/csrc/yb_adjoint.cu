// Adjoint of the block SVD (regularised as in yastn/backend/linalg/torch_svd_gesdd.py:296-428).
//
// For a block A = U diag(s) Vh (m x n, k = min(m, n)) with cotangents gU, gS, gVh and
// P = U^H gU, Q = Vh gVh^H (both k x k, computed by the grouped GEMM), this kernel forms
//
//   K_ij = (F+G)_ij (P_ij - conj P_ji)/2 + (F-G)_ij (Q_ij - conj Q_ji)/2
//          + delta_ij (gS_i + i Im(P_ii) sinv_i [complex])
//          - [n > k] sinv_i conj(Q_ji) - [m > k] P_ij sinv_j
//
// with F_ij = r(s_j - s_i), G_ij = r(s_j + s_i) off the diagonal (zero on it),
// sinv_i = r(s_i) and r(x) = x / (x^2 + 1e-12), and initialises the work matrix TR:
// wide blocks TR = diag(sinv) gVh, square TR = 0, tall TR = gU diag(sinv). The host
// then finishes with grouped GEMMs: TR += K Vh, dA = U TR (square/wide) or
// TR += U K, dA = TR Vh (tall), which equals the reference's u_term + sigma_term +
// v_term (+ imaginary term).
#include "yb_common.cuh"

namespace yb {
namespace {

__device__ __forceinline__ double rinv(double x) { return x / (x * x + 1.0e-12); }

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <bool Cx>
struct Elt;
template <>
struct Elt<false> {
  using T = double;
};
template <>
struct Elt<true> {
  using T = double2;
};

__device__ __forceinline__ double re(double a) { return a; }
__device__ __forceinline__ double re(double2 a) { return a.x; }

template <bool Cx>
__global__ void svd_adjoint_core_kernel(const typename Elt<Cx>::T* __restrict__ P,
                                        const typename Elt<Cx>::T* __restrict__ Q, const double* __restrict__ S,
                                        const double* __restrict__ gS, typename Elt<Cx>::T* __restrict__ K,
                                        const typename Elt<Cx>::T* __restrict__ gU,
                                        const typename Elt<Cx>::T* __restrict__ gVh,
                                        typename Elt<Cx>::T* __restrict__ TR, const int64_t* __restrict__ blocks) {
  using T = typename Elt<Cx>::T;
  const int64_t* r = blocks + (int64_t)blockIdx.y * YB_ADJ_REC;
  const int64_t m = r[1], n = r[2], k = r[8], kind = r[9];
  const double* s = S + r[4];
  const T* Pb = P + r[6];
  const T* Qb = Q + r[6];
  T* Kb = K + r[6];
  const int64_t kk = k * k;
  const int64_t ntr = (kind == 2) ? m * k : k * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < kk + ntr;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (e < kk) {
      const int64_t i = e / k, j = e - i * k;
      const double si = s[i], sj = s[j];
      if constexpr (Cx) {
        const double2 pij = Pb[i * k + j], pji = Pb[j * k + i];
        const double2 qij = Qb[i * k + j], qji = Qb[j * k + i];
        double2 out = make_double2(0.0, 0.0);
        if (i != j) {
          const double f = rinv(sj - si), g = rinv(sj + si);
          const double a = 0.5 * (f + g), b = 0.5 * (f - g);
          out.x = a * (pij.x - pji.x) + b * (qij.x - qji.x);
          out.y = a * (pij.y + pji.y) + b * (qij.y + qji.y);
        } else {
          out.x = (gS ? gS[r[4] + i] : 0.0);
          out.y = pij.y * rinv(si);
        }
        if (kind == 1) {  // - sinv_i conj(Q_ji)
          out.x -= rinv(si) * qji.x;
          out.y += rinv(si) * qji.y;
        } else if (kind == 2) {  // - P_ij sinv_j
          out.x -= pij.x * rinv(sj);
          out.y -= pij.y * rinv(sj);
        }
        Kb[i * k + j] = out;
      } else {
        const double pij = Pb[i * k + j], pji = Pb[j * k + i];
        const double qij = Qb[i * k + j], qji = Qb[j * k + i];
        double out = 0.0;
        if (i != j) {
          const double f = rinv(sj - si), g = rinv(sj + si);
          out = 0.5 * (f + g) * (pij - pji) + 0.5 * (f - g) * (qij - qji);
        } else {
          out = gS ? gS[r[4] + i] : 0.0;
        }
        if (kind == 1) out -= rinv(si) * qji;
        else if (kind == 2) out -= pij * rinv(sj);
        Kb[i * k + j] = out;
      }
    } else {
      const int64_t f = e - kk;
      T* tr = TR + r[7];
      if (kind == 0) {
        if constexpr (Cx) tr[f] = make_double2(0.0, 0.0); else tr[f] = 0.0;
      } else if (kind == 1) {  // k x n: row i scaled by sinv_i
        const int64_t i = f / n;
        const double w = rinv(s[i]);
        const T g = gVh[r[5] + f];
        if constexpr (Cx) tr[f] = make_double2(g.x * w, g.y * w); else tr[f] = g * w;
      } else {  // m x k: column j scaled by sinv_j
        const int64_t j = f % k;
        const double w = rinv(s[j]);
        const T g = gU[r[3] + f];
        if constexpr (Cx) tr[f] = make_double2(g.x * w, g.y * w); else tr[f] = g * w;
      }
    }
  }
}

// Adjoint of the block Hermitian eigendecomposition A = U diag(d) U^H. X = op(U)^T gU
// (k x k per block, from the grouped GEMM) becomes the inner matrix K of dA = U K op(U)^T:
//   symeig (order by magnitude, yastn/backend/linalg/torch_eig_sym.py:43-54; op(U) = U):
//     K_ij = r_eps(d_j - d_i) X_ij off the diagonal, K_ii = gd_i
//   torch.linalg.eigh (op(U) = conj(U)):
//     K_ij = (X_ij - conj X_ji) / (2 (d_j - d_i)) off the diagonal, K_ii = gd_i, or
//     i Im(X_ii) without gd
// with r_eps(x) = x / (x^2 + eps). Record per block: [0] X/K offset [1] k [2] d offset.
template <bool Cx>
__global__ void eigh_adjoint_core_kernel(const typename Elt<Cx>::T* __restrict__ X, const double* __restrict__ D,
                                         const double* __restrict__ gD, typename Elt<Cx>::T* __restrict__ K,
                                         const int64_t* __restrict__ blocks, int symeig, double eps) {
  using T = typename Elt<Cx>::T;
  const int64_t* r = blocks + (int64_t)blockIdx.y * 4;
  const int64_t off = r[0], k = r[1];
  const double* d = D + r[2];
  const T* Xb = X + off;
  T* Kb = K + off;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < k * k; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / k, j = e - i * k;
    T v;
    if (i == j) {
      const double g = gD ? gD[r[2] + i] : 0.0;
      if constexpr (Cx) v = make_double2(g, (symeig || gD) ? 0.0 : Xb[e].y);
      else v = g;
    } else {
      const double x = d[j] - d[i];
      if (symeig) {
        const double f = x / (x * x + eps);
        if constexpr (Cx) v = make_double2(f * Xb[e].x, f * Xb[e].y);
        else v = f * Xb[e];
      } else {
        const double f = 0.5 / x;
        if constexpr (Cx) {
          const double2 a = Xb[e], b = Xb[j * k + i];
          v = make_double2(f * (a.x - b.x), f * (a.y + b.y));
        } else {
          v = f * (Xb[e] - Xb[j * k + i]);
        }
      }
    }
    Kb[e] = v;
  }
}

// QR adjoint: records YB_QRADJ_REC int64 per block: [0] M offset (k x k) [1] k
// [2] B offset (rows x k, row-major, leading dimension [4]) [3] rows [4] ldb
// [5] R offset (k x k upper triangle, leading dimension [6]) [6] ldr.
// copyltu: M <- tril(M, -1) + tril(M, -1)^H + Re diag(M) (the upper triangle mirrored from
// the lower, conjugated for complex data, whose diagonal keeps its real part).
template <bool Cx>
__global__ void qr_copyltu_kernel(double* __restrict__ M, const int64_t* __restrict__ recs) {
  const int64_t* r = recs + (int64_t)blockIdx.y * YB_QRADJ_REC;
  const int64_t k = r[1];
  double* m = M + (Cx ? 2 : 1) * r[0];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < k * k; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / k, j = e - i * k;
    if (Cx) {
      if (i < j) {  // writes the upper triangle only, reads the lower
        m[2 * e] = m[2 * (j * k + i)];
        m[2 * e + 1] = -m[2 * (j * k + i) + 1];
      } else if (i == j) {
        m[2 * e + 1] = 0.0;
      }
    } else {
      if (i < j) m[e] = m[j * k + i];
    }
  }
}

// B <- B R^{-H} row by row (R upper triangular with a real diagonal): x R^H = b, i.e.
// x_j = (b_j - sum_{l > j} x_l conj(R_jl)) / R_jj by back substitution, one warp per row, in
// place. Entries of x already solved are re-read from L2 (written by lane 0 of the same warp,
// ordered by __syncwarp).
template <bool Cx>
__global__ void trsm_rt_kernel(double* __restrict__ B, const double* __restrict__ Rm, const int64_t* __restrict__ recs) {
  constexpr int W = Cx ? 2 : 1;
  const int64_t* r = recs + (int64_t)blockIdx.y * YB_QRADJ_REC;
  const int64_t k = r[1], rows = r[3], ldb = r[4], ldr = r[6];
  double* b = B + W * r[2];
  const double* R = Rm + W * r[5];
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row = warp; row < rows; row += nwarps) {
    double* x = b + W * row * ldb;
    for (int64_t j = k - 1; j >= 0; --j) {
      double ar = 0.0, ai = 0.0;
      for (int64_t l = j + 1 + lane; l < k; l += 32) {
        if (Cx) {  // x_l conj(R_jl)
          const double rr = R[2 * (j * ldr + l)], ri = R[2 * (j * ldr + l) + 1];
          const double xr = __ldcg(x + 2 * l), xi = __ldcg(x + 2 * l + 1);
          ar = fma(xr, rr, fma(xi, ri, ar));
          ai = fma(xi, rr, fma(-xr, ri, ai));
        } else {
          ar = fma(R[j * ldr + l], __ldcg(x + l), ar);
        }
      }
      ar = warp_sum(ar);
      if (Cx) ai = warp_sum(ai);
      if (lane == 0) {
        const double d = R[W * (j * ldr + j)];  // real and positive
        x[W * j] = (__ldcg(x + W * j) - ar) / d;
        if (Cx) x[2 * j + 1] = (__ldcg(x + 2 * j + 1) - ai) / d;
      }
      __syncwarp();
    }
  }
}

}  // namespace
}  // namespace yb

extern "C" int yb_qr_adjoint_sym(void* M, const int64_t* recs, int n_blocks, int dtype, void* stream) {
  if (n_blocks == 0) return YB_OK;
  if (!M || !recs) return YB_ERR_INVALID;
  const dim3 grid(16, (unsigned)n_blocks);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64) yb::qr_copyltu_kernel<false><<<grid, 256, 0, s>>>((double*)M, recs);
  else if (dtype == YB_C128) yb::qr_copyltu_kernel<true><<<grid, 256, 0, s>>>((double*)M, recs);
  else return YB_ERR_INVALID;
  return yb::check_launch();
}

extern "C" int yb_trsm_rt(void* B, const void* R, const int64_t* recs, int n_blocks, int dtype, void* stream) {
  if (n_blocks == 0) return YB_OK;
  if (!B || !R || !recs) return YB_ERR_INVALID;
  const dim3 grid(32, (unsigned)n_blocks);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64) yb::trsm_rt_kernel<false><<<grid, 256, 0, s>>>((double*)B, (const double*)R, recs);
  else if (dtype == YB_C128) yb::trsm_rt_kernel<true><<<grid, 256, 0, s>>>((double*)B, (const double*)R, recs);
  else return YB_ERR_INVALID;
  return yb::check_launch();
}

extern "C" int yb_eigh_adjoint_core(const void* X, const double* D, const double* gD, void* K,
                                    const int64_t* blocks, int n_blocks, int dtype, int symeig, double eps,
                                    void* stream) {
  if (n_blocks == 0) return YB_OK;
  if (!X || !D || !K || !blocks) return YB_ERR_INVALID;
  dim3 grid(16, (unsigned)n_blocks);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64)
    yb::eigh_adjoint_core_kernel<false><<<grid, 256, 0, s>>>((const double*)X, D, gD, (double*)K, blocks, symeig, eps);
  else if (dtype == YB_C128)
    yb::eigh_adjoint_core_kernel<true><<<grid, 256, 0, s>>>((const double2*)X, D, gD, (double2*)K, blocks, symeig,
                                                            eps);
  else
    return YB_ERR_INVALID;
  return yb::check_launch();
}

extern "C" int yb_svd_adjoint_core(const void* P, const void* Q, const double* S, const double* gS, void* K,
                                   const void* gU, const void* gVh, void* TR, const int64_t* blocks, int n_blocks,
                                   int dtype, void* stream) {
  if (n_blocks == 0) return YB_OK;
  if (!P || !Q || !S || !K || !gU || !gVh || !TR || !blocks) return YB_ERR_INVALID;
  dim3 grid(32, (unsigned)n_blocks);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64)
    yb::svd_adjoint_core_kernel<false><<<grid, 256, 0, s>>>((const double*)P, (const double*)Q, S, gS, (double*)K,
                                                            (const double*)gU, (const double*)gVh, (double*)TR,
                                                            blocks);
  else if (dtype == YB_C128)
    yb::svd_adjoint_core_kernel<true><<<grid, 256, 0, s>>>((const double2*)P, (const double2*)Q, S, gS, (double2*)K,
                                                           (const double2*)gU, (const double2*)gVh, (double2*)TR,
                                                           blocks);
  else
    return YB_ERR_INVALID;
  return yb::check_launch();
}
