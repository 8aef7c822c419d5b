// Masks, truncation and gauge fixing on the device.
//
//  * yb_mask_gather: apply_mask / its adjoint (gather or scatter of kept indices along
//    one axis of every block), one launch for all blocks.
//  * yb_truncation_mask: the truncation rule of yastn/tensor/linalg.py:637-735 fused
//    into one single-CTA launch (per-block tol_block/D_block cut, global tol/D_total cut
//    by ranking S*mask, optional multiplet-gap extension), so the caller needs one
//    device->host copy of the kept counts instead of a sync per block.
//  * yb_fix_signs: the gauge of yastn/backend/backend_np.py:447-458 (largest-|U| entry
//    of each column made real positive; magnitudes compared as int64(|U| * 2^40)).
#include <float.h>
#include "yb_common.cuh"

namespace yb {
namespace {

// ------------------------------------------------------------------ apply_mask
template <typename Unit>
__global__ void mask_gather_kernel(const Unit* __restrict__ A, Unit* __restrict__ out,
                                   const int64_t* __restrict__ recs, const int64_t* __restrict__ items,
                                   const int64_t* __restrict__ idx, int scatter) {
  const int64_t* it = items + 2 * (int64_t)blockIdx.x;
  const int64_t* r = recs + it[0] * YB_MASK_REC;
  const int64_t first = it[1];
  const int64_t sln = r[0], sla = r[1], pre = r[2], da = r[3], dn = r[4], post = r[5], ioff = r[6];
  const int64_t total = pre * dn * post;
  const int64_t n = min((int64_t)YB_COPY_ITEM_UNITS, total - first);
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    const int64_t g = first + e;
    const int64_t p = g / (dn * post);
    const int64_t rem = g - p * dn * post;
    const int64_t i = rem / post;
    const int64_t q = rem - i * post;
    const int64_t s = sla + (p * da + idx[ioff + i]) * post + q;
    if (scatter) out[s] = A[sln + g];
    else out[sln + g] = A[s];
  }
}

// ------------------------------------------------------------------ truncation
constexpr int kTruncThreads = 1024;
constexpr int kMaxBlk = 1024;

__device__ __forceinline__ int block_of(const int64_t* blk, int n_blk, int64_t i) {
  int lo = 0, hi = n_blk - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (blk[4 * mid] <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(kTruncThreads) truncation_kernel(const double* __restrict__ S, int64_t n,
                                                                   const int64_t* __restrict__ blk,
                                                                   const double* __restrict__ tol_block, int n_blk,
                                                                   double tol, int64_t D_total, int multiplets,
                                                                   uint8_t* __restrict__ mask_out,
                                                                   int64_t* __restrict__ kept, int pow2) {
  extern __shared__ unsigned char smem_raw[];
  double* val = reinterpret_cast<double*>(smem_raw);
  int* idx = reinterpret_cast<int*>(val + pow2);
  uint8_t* mask = reinterpret_cast<uint8_t*>(idx + pow2);
  __shared__ unsigned long long bmax_bits[kMaxBlk];
  __shared__ int bcnt[kMaxBlk];
  __shared__ unsigned long long gmax_bits;
  __shared__ int gcnt;
  __shared__ long long dt_shared;

  const int tid = threadIdx.x;
  for (int b = tid; b < n_blk; b += blockDim.x) { bmax_bits[b] = 0ull; bcnt[b] = 0; }
  if (tid == 0) { gmax_bits = 0ull; gcnt = 0; }
  for (int64_t i = tid; i < n; i += blockDim.x) mask[i] = 1;
  __syncthreads();
  // per-block max |S| (non-negative doubles order like their bit patterns)
  for (int64_t i = tid; i < n; i += blockDim.x) {
    const int b = block_of(blk, n_blk, i);
    atomicMax(&bmax_bits[b], (unsigned long long)__double_as_longlong(fabs(S[i])));
  }
  __syncthreads();
  for (int64_t i = tid; i < n; i += blockDim.x) {
    const int b = block_of(blk, n_blk, i);
    if (S[i] > tol_block[b] * __longlong_as_double((long long)bmax_bits[b])) atomicAdd(&bcnt[b], 1);
  }
  __syncthreads();
  // per-block cut: keep the D_bl largest (ascending rank >= len - D_bl, stable ranks)
  for (int64_t i = tid; i < n; i += blockDim.x) {
    const int b = block_of(blk, n_blk, i);
    const int64_t lo = blk[4 * b], hi = blk[4 * b + 1], dblock = blk[4 * b + 2];
    const int64_t len = hi - lo;
    int64_t dbl = bcnt[b];
    if (dblock >= 0 && dblock < dbl) dbl = dblock;
    if (dbl == 0) {
      mask[i] = 0;
    } else if (dbl < len) {
      const double v = S[i];
      int64_t rank = 0;
      for (int64_t j = lo; j < hi; ++j) {
        const double w = S[j];
        rank += (w < v) || (w == v && j < i);
      }
      if (rank < len - dbl) mask[i] = 0;
    }
  }
  __syncthreads();
  // global cut on temp = S * mask
  for (int64_t i = tid; i < pow2; i += blockDim.x) {
    if (i < n) {
      const double t = mask[i] ? S[i] : 0.0 * S[i];
      val[i] = t;
      atomicMax(&gmax_bits, (unsigned long long)__double_as_longlong(fabs(t)));
    } else {
      val[i] = __longlong_as_double(0x7ff0000000000000LL);  // +inf padding; index tie-break puts it last
    }
    idx[i] = (int)i;
  }
  __syncthreads();
  const double gmax = __longlong_as_double((long long)gmax_bits);
  for (int64_t i = tid; i < n; i += blockDim.x)
    if (val[i] > tol * gmax) atomicAdd(&gcnt, 1);
  __syncthreads();
  int64_t dt = gcnt;
  if (D_total >= 0 && D_total < dt) dt = D_total;
  if (dt == 0) {
    for (int64_t i = tid; i < n; i += blockDim.x) mask_out[i] = 0;
    for (int b = tid; b < n_blk; b += blockDim.x) kept[b] = 0;
    return;
  }
  // ascending bitonic sort of (val, idx)
  for (int size = 2; size <= pow2; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = tid; i < pow2; i += blockDim.x) {
        const int j = i ^ stride;
        if (j > i) {
          const bool up = ((i & size) == 0);
          const double vi = val[i], vj = val[j];
          const int ii = idx[i], ij = idx[j];
          const bool in_order = (vi < vj) || (vi == vj && ii < ij);
          if (up != in_order) {
            val[i] = vj; val[j] = vi;
            idx[i] = ij; idx[j] = ii;
          }
        }
      }
      __syncthreads();
    }
  }
  if (tid == 0) {
    long long d = dt;
    if (multiplets && d < n) {
      // inds[-p] is position n - p of the ascending order
      double gap = -1.0;
      for (long long p = d; p < n; ++p) {
        const double a = S[idx[n - p]], b = S[idx[n - p - 1]];
        const double gp = fabs(a - b);
        if (gp > gap) { d = p; gap = gp; }
        if (gap > fabs(a)) break;
      }
    }
    dt_shared = d;
  }
  __syncthreads();
  const int64_t keep_from = n - dt_shared;
  for (int64_t p = tid; p < keep_from; p += blockDim.x) mask[idx[p]] = 0;
  __syncthreads();
  for (int b = tid; b < n_blk; b += blockDim.x) bcnt[b] = 0;
  __syncthreads();
  for (int64_t i = tid; i < n; i += blockDim.x) {
    mask_out[i] = mask[i];
    if (mask[i]) atomicAdd(&bcnt[block_of(blk, n_blk, i)], 1);
  }
  __syncthreads();
  for (int b = tid; b < n_blk; b += blockDim.x) kept[b] = bcnt[b];
}

// ------------------------------------------------------------------ fix_svd_signs
template <bool Cx>
__global__ void fix_signs_kernel(const double* __restrict__ Uin, const double* __restrict__ Vin,
                                 double* __restrict__ Uout, double* __restrict__ Vout, double* __restrict__ phases,
                                 const int64_t* __restrict__ blocks, int apply_given) {
  constexpr int W = Cx ? 2 : 1;
  const int64_t* r = blocks + (int64_t)blockIdx.y * YB_SVD_REC;
  const int64_t m = r[1], n = r[2], k = r[9];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t c = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  if (c >= k) return;
  const double* U = Uin + W * r[3];
  const double* V = Vin + W * r[5];
  double* Uo = Uout + W * r[3];
  double* Vo = Vout + W * r[5];
  double pr, pi = 0.0;
  if (apply_given) {
    pr = phases[W * (r[4] + c)];
    if (Cx) pi = phases[W * (r[4] + c) + 1];
  } else {
    long long best = -1;
    int64_t brow = 0;
    for (int64_t row = lane; row < m; row += 32) {
      double a;
      if (Cx) a = hypot(U[2 * (row * k + c)], U[2 * (row * k + c) + 1]);
      else a = fabs(U[row * k + c]);
      const long long amp = (long long)(a * 1099511627776.0);  // truncation toward zero, as astype(int64)
      if (amp > best) { best = amp; brow = row; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int64_t orow = __shfl_xor_sync(0xffffffffu, brow, o);
      if (ob > best || (ob == best && orow < brow)) { best = ob; brow = orow; }
    }
    if (Cx) {
      const double ur = U[2 * (brow * k + c)], ui = U[2 * (brow * k + c) + 1];
      const double a = hypot(ur, ui);
      pr = ur / a;
      pi = ui / a;
    } else {
      const double u = U[brow * k + c];
      pr = u / fabs(u);
    }
    if (lane == 0 && phases) {
      phases[W * (r[4] + c)] = pr;
      if (Cx) phases[W * (r[4] + c) + 1] = pi;
    }
    __syncwarp();
  }
  // U[:, c] *= conj(phase); Vh[c, :] *= phase
  for (int64_t row = lane; row < m; row += 32) {
    if (Cx) {
      const double ur = U[2 * (row * k + c)], ui = U[2 * (row * k + c) + 1];
      Uo[2 * (row * k + c)] = ur * pr + ui * pi;
      Uo[2 * (row * k + c) + 1] = ui * pr - ur * pi;
    } else {
      Uo[row * k + c] = U[row * k + c] * pr;
    }
  }
  for (int64_t col = lane; col < n; col += 32) {
    if (Cx) {
      const double vr = V[2 * (c * n + col)], vi = V[2 * (c * n + col) + 1];
      Vo[2 * (c * n + col)] = vr * pr - vi * pi;
      Vo[2 * (c * n + col) + 1] = vr * pi + vi * pr;
    } else {
      Vo[c * n + col] = V[c * n + col] * pr;
    }
  }
}


// Adjoint of the gauge fix (torch's autograd of the reference's fix_svd_signs,
// backend_torch.py:353-366; complex gradients in torch's convention): per column c, with
// p = U[r*, c] / |U[r*, c]| at the forward's row choice r* (recomputed from U by the same rule),
// dU[:, c] = gU[:, c] p, dVh[c, :] = gVh[c, :] conj(p), and for complex data
// dU[r*, c] += -i (p / |U[r*, c]|) Im(conj(G) p), G = sum_i U[i, c] conj(gU[i, c]) +
// sum_j conj(Vh[c, j]) gVh[c, j] (the gradient through the phase).
template <bool Cx>
__global__ void fix_signs_adjoint_kernel(const double* __restrict__ Uin, const double* __restrict__ Vin,
                                         const double* __restrict__ gU, const double* __restrict__ gV,
                                         double* __restrict__ dU, double* __restrict__ dV,
                                         const int64_t* __restrict__ blocks) {
  constexpr int W = Cx ? 2 : 1;
  const int64_t* r = blocks + (int64_t)blockIdx.y * YB_SVD_REC;
  const int64_t m = r[1], n = r[2], k = r[9];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t c = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  if (c >= k) return;
  const int64_t uo = W * r[3], vo = W * r[5];
  const double* U = Uin + uo;
  const double* V = Vin + vo;
  long long best = -1;
  int64_t brow = 0;
  for (int64_t row = lane; row < m; row += 32) {
    const double a = Cx ? hypot(U[2 * (row * k + c)], U[2 * (row * k + c) + 1]) : fabs(U[row * k + c]);
    const long long amp = (long long)(a * 1099511627776.0);  // as the forward's int64(|U| 2^40)
    if (amp > best) { best = amp; brow = row; }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int64_t orow = __shfl_xor_sync(0xffffffffu, brow, o);
    if (ob > best || (ob == best && orow < brow)) { best = ob; brow = orow; }
  }
  double pr, pi = 0.0, au;
  if (Cx) {
    const double ur = U[2 * (brow * k + c)], ui = U[2 * (brow * k + c) + 1];
    au = hypot(ur, ui);
    pr = ur / au;
    pi = ui / au;
  } else {
    const double u = U[brow * k + c];
    au = fabs(u);
    pr = u / au;
  }
  double Gr = 0.0, Gi = 0.0;
  for (int64_t row = lane; row < m; row += 32) {
    const int64_t e = row * k + c;
    if (Cx) {  // U conj(gU)
      const double ur = U[2 * e], ui = U[2 * e + 1], gr = gU[uo + 2 * e], gi = gU[uo + 2 * e + 1];
      Gr += ur * gr + ui * gi;
      Gi += ui * gr - ur * gi;
      dU[uo + 2 * e] = gr * pr - gi * pi;
      dU[uo + 2 * e + 1] = gr * pi + gi * pr;
    } else {
      dU[uo + e] = gU[uo + e] * pr;
    }
  }
  for (int64_t col = lane; col < n; col += 32) {
    const int64_t e = c * n + col;
    if (Cx) {  // conj(V) gV
      const double vr = V[2 * e], vi = V[2 * e + 1], gr = gV[vo + 2 * e], gi = gV[vo + 2 * e + 1];
      Gr += vr * gr + vi * gi;
      Gi += vr * gi - vi * gr;
      dV[vo + 2 * e] = gr * pr + gi * pi;
      dV[vo + 2 * e + 1] = gi * pr - gr * pi;
    } else {
      dV[vo + e] = gV[vo + e] * pr;
    }
  }
  if (Cx) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      Gr += __shfl_xor_sync(0xffffffffu, Gr, o);
      Gi += __shfl_xor_sync(0xffffffffu, Gi, o);
    }
    __syncwarp();
    if (lane == (int)(brow & 31)) {  // the lane that wrote dU[r*, c]
      const double t = (Gr * pi - Gi * pr) / au;  // Im(conj(G) p) / |u|
      const int64_t e = brow * k + c;
      dU[uo + 2 * e] += pi * t;
      dU[uo + 2 * e + 1] -= pr * t;
    }
  }
}

}  // namespace
}  // namespace yb

extern "C" {

int yb_mask_gather(const void* A, void* out, int unit_bytes, const int64_t* recs, const int64_t* items, int n_items,
                   const int64_t* idx, int scatter, void* stream) {
  if (n_items == 0) return YB_OK;
  if (!A || !out || !recs || !items || !idx || n_items < 0) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  switch (unit_bytes) {  // raw units of the element size
    case 8:
      yb::mask_gather_kernel<double><<<(unsigned)n_items, 256, 0, s>>>((const double*)A, (double*)out, recs, items, idx,
                                                                       scatter);
      break;
    case 16:
      yb::mask_gather_kernel<double2><<<(unsigned)n_items, 256, 0, s>>>((const double2*)A, (double2*)out, recs, items,
                                                                        idx, scatter);
      break;
    case 4:
      yb::mask_gather_kernel<uint32_t><<<(unsigned)n_items, 256, 0, s>>>((const uint32_t*)A, (uint32_t*)out, recs,
                                                                         items, idx, scatter);
      break;
    case 2:
      yb::mask_gather_kernel<uint16_t><<<(unsigned)n_items, 256, 0, s>>>((const uint16_t*)A, (uint16_t*)out, recs,
                                                                         items, idx, scatter);
      break;
    case 1:
      yb::mask_gather_kernel<uint8_t><<<(unsigned)n_items, 256, 0, s>>>((const uint8_t*)A, (uint8_t*)out, recs, items,
                                                                        idx, scatter);
      break;
    default: return YB_ERR_INVALID;
  }
  return yb::check_launch();
}

int yb_truncation_mask(const double* S, int64_t n, const int64_t* blk, const double* tol_block, int n_blk, double tol,
                       int64_t D_total, int truncate_multiplets, uint8_t* mask, int64_t* kept, void* stream) {
  if (n < 0 || n_blk < 0) return YB_ERR_INVALID;
  if (n > YB_TRUNC_MAX || n_blk > yb::kMaxBlk) return YB_ERR_TOO_LARGE;
  if (n_blk == 0) return YB_OK;
  int pow2 = 1;
  while (pow2 < n) pow2 <<= 1;
  const size_t smem = (size_t)pow2 * (sizeof(double) + sizeof(int)) + (size_t)pow2;
  cudaError_t e = cudaFuncSetAttribute(yb::truncation_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(smem < 48 * 1024 ? 48 * 1024 : smem));
  if (e != cudaSuccess) { yb::set_cuda_error((int)e); return YB_ERR_CUDA; }
  yb::truncation_kernel<<<1, yb::kTruncThreads, smem, (cudaStream_t)stream>>>(
      S, n, blk, tol_block, n_blk, tol, D_total, truncate_multiplets, mask, kept, pow2);
  return yb::check_launch();
}

int yb_fix_signs(const void* Uin, const void* Vin, void* Uout, void* Vout, void* phase_out, const int64_t* blocks,
                 int n_blocks, int max_k, int dtype, int apply_given, void* stream) {
  if (n_blocks == 0 || max_k == 0) return YB_OK;
  if (!Uin || !Vin || !Uout || !Vout || !blocks || max_k < 0) return YB_ERR_INVALID;
  if (apply_given && !phase_out) return YB_ERR_INVALID;
  dim3 grid((unsigned)((max_k + 7) / 8), (unsigned)n_blocks);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64)
    yb::fix_signs_kernel<false><<<grid, 256, 0, s>>>((const double*)Uin, (const double*)Vin, (double*)Uout,
                                                     (double*)Vout, (double*)phase_out, blocks, apply_given);
  else if (dtype == YB_C128)
    yb::fix_signs_kernel<true><<<grid, 256, 0, s>>>((const double*)Uin, (const double*)Vin, (double*)Uout,
                                                    (double*)Vout, (double*)phase_out, blocks, apply_given);
  else
    return YB_ERR_INVALID;
  return yb::check_launch();
}

int yb_fix_signs_adjoint(const void* Uin, const void* Vin, const void* gU, const void* gV, void* dU, void* dV,
                         const int64_t* blocks, int n_blocks, int max_k, int dtype, void* stream) {
  if (n_blocks == 0 || max_k == 0) return YB_OK;
  if (!Uin || !Vin || !gU || !gV || !dU || !dV || !blocks || max_k < 0) return YB_ERR_INVALID;
  dim3 grid((unsigned)((max_k + 7) / 8), (unsigned)n_blocks);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64)
    yb::fix_signs_adjoint_kernel<false><<<grid, 256, 0, s>>>((const double*)Uin, (const double*)Vin,
                                                             (const double*)gU, (const double*)gV, (double*)dU,
                                                             (double*)dV, blocks);
  else if (dtype == YB_C128)
    yb::fix_signs_adjoint_kernel<true><<<grid, 256, 0, s>>>((const double*)Uin, (const double*)Vin,
                                                            (const double*)gU, (const double*)gV, (double*)dU,
                                                            (double*)dV, blocks);
  else
    return YB_ERR_INVALID;
  return yb::check_launch();
}

}  // extern "C"
