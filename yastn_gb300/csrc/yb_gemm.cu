// Family (b): grouped sum-of-products GEMM over charge sectors, native FP64 / complex128.
//
//   C_o = alpha * sum_{t in terms(o)} op(A_t) op(B_t) + beta * C_o
//
// One launch covers every 64x64 output tile of every sector; the host orders tiles
// largest-K first so that the long tiles start early. Outputs with few rows (the
// contractions with a small MPO block, for instance) use "skinny" tiles instead: all rows x
// 1024 columns, four columns per thread, op(A) staged in shared memory (up to 16 rows, above 8
// with 256 columns, one per thread; the host sends outputs of up to 8 rows, and of 9..16 rows
// only when they are wide). Outputs of at most 16 columns and many rows take "tall" tiles
// (256 rows, one per thread, all columns). On GB300 FP64 arithmetic runs at
// about 1.2 TFLOP/s on the DFMA pipe (the DMMA m8n8k4 tensor path measured slower),
// so a register-tiled DFMA kernel with shared-memory staging is FP64-bound: each thread
// owns a 4x4 sub-tile and issues 16 independent FMAs per staged k.
#include "yb_common.cuh"

namespace yb {
namespace {

constexpr int kTile = YB_GEMM_TILE;  // 64
constexpr int kK = 16;
constexpr int kThreads = 256;
constexpr int kPad = 2;
constexpr int kSkinnyK = 64;     // K-chunk of op(A) staged for a skinny tile (64 x 16 <= 16 x 66)

struct Real {
  using T = double;
  __device__ static T zero() { return 0.0; }
  __device__ static T conj(T a) { return a; }
  __device__ static void fma(T& acc, T a, T b) { acc = ::fma(a, b, acc); }
  __device__ static T scale(T a, double s) { return a * s; }
  __device__ static T add(T a, T b) { return a + b; }
};

struct Cplx {
  using T = double2;
  __device__ static T zero() { return make_double2(0.0, 0.0); }
  __device__ static T conj(T a) { return make_double2(a.x, -a.y); }
  __device__ static void fma(T& acc, T a, T b) {
    acc.x = ::fma(a.x, b.x, acc.x);
    acc.x = ::fma(-a.y, b.y, acc.x);
    acc.y = ::fma(a.x, b.y, acc.y);
    acc.y = ::fma(a.y, b.x, acc.y);
  }
  __device__ static T scale(T a, double s) { return make_double2(a.x * s, a.y * s); }
  __device__ static T add(T a, T b) { return make_double2(a.x + b.x, a.y + b.y); }
};

// Skinny tile: C (M x kThreads*CPT slice) = alpha sum_t op(A_t) op(B_t) + beta C for at
// most M rows (the block's mr <= M rows; M is the compiled bound). op(A) is staged in shared
// memory K-chunk by K-chunk ([kSkinnyK][M], broadcast reads); each thread owns CPT columns,
// kThreads apart, so B loads and C stores coalesce.
template <class F, int M, int CPT>
__device__ __forceinline__ void skinny_tile(const typename F::T* __restrict__ A, const typename F::T* __restrict__ B,
                                            typename F::T* __restrict__ C, const int64_t* __restrict__ orec,
                                            const int64_t* __restrict__ terms, int tcol, double alpha, double beta,
                                            typename F::T* Ak) {
  using T = typename F::T;
  const int64_t c_off = orec[0], ldc = orec[3], t0 = orec[4], t1 = orec[5];
  const int64_t mr = orec[1], nc = orec[2];
  const int64_t j0 = (int64_t)tcol * (kThreads * CPT) + threadIdx.x;
  T acc[CPT][M];
#pragma unroll
  for (int u = 0; u < CPT; ++u)
#pragma unroll
    for (int i = 0; i < M; ++i) acc[u][i] = F::zero();
  for (int64_t t = t0; t < t1; ++t) {
    const int64_t* trec = terms + t * YB_GEMM_TERM_REC;
    const int64_t K = trec[2];
    const T* La = A + trec[0];
    const T* Ra = B + trec[1];
    const int64_t l_is = trec[3], l_ls = trec[4], r_ls = trec[5], r_js = trec[6];
    const int flags = (int)trec[7];
    const bool conjL = flags & 1, conjR = flags & 2;
    for (int64_t k0 = 0; k0 < K; k0 += kSkinnyK) {
      __syncthreads();
      for (int e = threadIdx.x; e < kSkinnyK * M; e += kThreads) {
        const int i = e % M, l = e / M;
        T v = F::zero();
        if (k0 + l < K && i < mr) {
          v = La[i * l_is + (k0 + l) * l_ls];
          if (conjL) v = F::conj(v);
        }
        Ak[l * M + i] = v;
      }
      __syncthreads();
      const int64_t kn = min((int64_t)kSkinnyK, K - k0);
      const T* Rk = Ra + k0 * r_ls;
      for (int64_t l = 0; l < kn; ++l) {
        T b[CPT];
#pragma unroll
        for (int u = 0; u < CPT; ++u) {
          const int64_t j = j0 + u * kThreads;
          b[u] = (j < nc) ? Rk[l * r_ls + j * r_js] : F::zero();
          if (conjR) b[u] = F::conj(b[u]);
        }
#pragma unroll
        for (int i = 0; i < M; ++i) {
          const T a = Ak[l * M + i];
#pragma unroll
          for (int u = 0; u < CPT; ++u) F::fma(acc[u][i], a, b[u]);
        }
      }
    }
  }
#pragma unroll
  for (int u = 0; u < CPT; ++u) {
    const int64_t j = j0 + u * kThreads;
    if (j >= nc) continue;
#pragma unroll
    for (int i = 0; i < M; ++i) {
      if (i >= mr) break;
      T* p = C + c_off + i * ldc + j;
      T v = alpha == 1.0 ? acc[u][i] : F::scale(acc[u][i], alpha);  // no FP64 multiply for alpha = 1
      if (beta != 0.0) v = F::add(v, F::scale(*p, beta));
      *p = v;
    }
  }
}

template <class F>
__device__ __forceinline__ void skinny_dispatch(int64_t mr, const typename F::T* __restrict__ A,
                                                const typename F::T* __restrict__ B, typename F::T* __restrict__ C,
                                                const int64_t* __restrict__ orec, const int64_t* __restrict__ terms,
                                                int tcol, double alpha, double beta, typename F::T* Ak) {
  // FP64 issue rate, not bandwidth, bounds these tiles: no FMA is spent on padding rows up to 8
  switch (mr) {
    case 1: skinny_tile<F, 1, 4>(A, B, C, orec, terms, tcol, alpha, beta, Ak); break;
    case 2: skinny_tile<F, 2, 4>(A, B, C, orec, terms, tcol, alpha, beta, Ak); break;
    case 3: skinny_tile<F, 3, 4>(A, B, C, orec, terms, tcol, alpha, beta, Ak); break;
    case 4: skinny_tile<F, 4, 4>(A, B, C, orec, terms, tcol, alpha, beta, Ak); break;
    case 5: skinny_tile<F, 5, 4>(A, B, C, orec, terms, tcol, alpha, beta, Ak); break;
    case 6: skinny_tile<F, 6, 4>(A, B, C, orec, terms, tcol, alpha, beta, Ak); break;
    case 7: skinny_tile<F, 7, 4>(A, B, C, orec, terms, tcol, alpha, beta, Ak); break;
    case 8: skinny_tile<F, 8, 4>(A, B, C, orec, terms, tcol, alpha, beta, Ak); break;
    case 9: skinny_tile<F, 9, 1>(A, B, C, orec, terms, tcol, alpha, beta, Ak); break;
    case 10: skinny_tile<F, 10, 1>(A, B, C, orec, terms, tcol, alpha, beta, Ak); break;
    case 11: skinny_tile<F, 11, 1>(A, B, C, orec, terms, tcol, alpha, beta, Ak); break;
    case 12: skinny_tile<F, 12, 1>(A, B, C, orec, terms, tcol, alpha, beta, Ak); break;
    case 13: case 14: skinny_tile<F, 14, 1>(A, B, C, orec, terms, tcol, alpha, beta, Ak); break;
    default: skinny_tile<F, 16, 1>(A, B, C, orec, terms, tcol, alpha, beta, Ak); break;
  }
}

// Tall skinny tile (kind 3): 256 rows x all n <= 16 columns of an output, one row per thread.
// op(B) is staged in shared memory K-chunk by K-chunk ([kTallK][N], broadcast reads); each
// thread reads its own op(A) row (a row's K-contiguous entries come from L1 after the first
// touch) and keeps its N accumulators in registers, so no FMA is spent on padding columns (a
// 64x64 tile of an n = 9 output runs 9 of each warp's 32 columns). N is the exact column count.
constexpr int kTallK = 64;
constexpr int kTallRows = kThreads;

template <class F, int N>
__device__ __forceinline__ void tall_tile(const typename F::T* __restrict__ A, const typename F::T* __restrict__ B,
                                          typename F::T* __restrict__ C, const int64_t* __restrict__ orec,
                                          const int64_t* __restrict__ terms, int trow, double alpha, double beta,
                                          typename F::T* Bk) {
  using T = typename F::T;
  const int64_t c_off = orec[0], m = orec[1], ldc = orec[3], t0 = orec[4], t1 = orec[5];
  const int64_t i = (int64_t)trow * kTallRows + threadIdx.x;
  const bool live = i < m;
  T acc[N];
#pragma unroll
  for (int j = 0; j < N; ++j) acc[j] = F::zero();
  for (int64_t t = t0; t < t1; ++t) {
    const int64_t* trec = terms + t * YB_GEMM_TERM_REC;
    const int64_t K = trec[2];
    const int64_t l_is = trec[3], l_ls = trec[4], r_ls = trec[5], r_js = trec[6];
    const int flags = (int)trec[7];
    const bool conjL = flags & 1, conjR = flags & 2;
    const T* Arow = A + trec[0] + (live ? i * l_is : 0);
    const T* Rb = B + trec[1];
    for (int64_t k0 = 0; k0 < K; k0 += kTallK) {
      __syncthreads();
      for (int e = threadIdx.x; e < kTallK * N; e += kThreads) {
        const int j = e % N, l = e / N;
        T v = F::zero();
        if (k0 + l < K) {
          v = Rb[(k0 + l) * r_ls + j * r_js];
          if (conjR) v = F::conj(v);
        }
        Bk[l * N + j] = v;
      }
      __syncthreads();
      if (!live) continue;
      const int kn = (int)min((int64_t)kTallK, K - k0);
      for (int l0 = 0; l0 < kn; l0 += 8) {
        T a[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          a[u] = (l0 + u < kn) ? Arow[(k0 + l0 + u) * l_ls] : F::zero();
          if (conjL) a[u] = F::conj(a[u]);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          if (l0 + u < kn) {
#pragma unroll
            for (int j = 0; j < N; ++j) F::fma(acc[j], a[u], Bk[(l0 + u) * N + j]);
          }
        }
      }
    }
  }
  if (!live) return;
  T* crow = C + c_off + i * ldc;
#pragma unroll
  for (int j = 0; j < N; ++j) {
    T v = alpha == 1.0 ? acc[j] : F::scale(acc[j], alpha);
    if (beta != 0.0) v = F::add(v, F::scale(crow[j], beta));
    crow[j] = v;
  }
}

template <class F>
__device__ __forceinline__ void tall_dispatch(int64_t nc, const typename F::T* __restrict__ A,
                                              const typename F::T* __restrict__ B, typename F::T* __restrict__ C,
                                              const int64_t* __restrict__ orec, const int64_t* __restrict__ terms,
                                              int trow, double alpha, double beta, typename F::T* Bk) {
  switch (nc) {
#define YB_TALL_CASE(NN) \
    case NN: tall_tile<F, NN>(A, B, C, orec, terms, trow, alpha, beta, Bk); break;
    YB_TALL_CASE(1) YB_TALL_CASE(2) YB_TALL_CASE(3) YB_TALL_CASE(4) YB_TALL_CASE(5) YB_TALL_CASE(6)
    YB_TALL_CASE(7) YB_TALL_CASE(8) YB_TALL_CASE(9) YB_TALL_CASE(10) YB_TALL_CASE(11) YB_TALL_CASE(12)
    YB_TALL_CASE(13) YB_TALL_CASE(14) YB_TALL_CASE(15) YB_TALL_CASE(16)
#undef YB_TALL_CASE
    default: break;
  }
}

// Short skinny outputs (one term, at most 8 rows, K <= 8; the contractions with a small
// MPO block): C (mr rows x a strip of YB_GEMM_SHORT_COLS columns) = alpha op(A) op(B) + beta C.
// GB300 issues 2 DFMA per SM per cycle, so the m K FMAs per column bound these strips rather
// than their bytes, and the pipe stays fed only while enough warps have their loads back: a
// strip's record reads are one round trip (the tile names both the output and its term), a
// thread keeps few registers (eight warps per SM scheduler) and issues its loads of op(B)
// before the barrier that publishes op(A) in shared memory. NT threads own
// YB_GEMM_SHORT_COLS / NT columns each, NT apart (every load and store instruction of a warp
// is coalesced), in passes of G columns. The epilogue of alpha = 1, beta = 0 is compiled
// apart: an if-converted alpha multiply would cost one DMUL per output on the FP64 pipe.
__host__ __device__ constexpr int short_pass(int elem_bytes, int M, int KB, int cpt) {
  int g = cpt;  // columns per pass: op(B) and accumulators within 32 registers
  while (g > 1 && (KB + M) * g * elem_bytes / 4 > 32) g >>= 1;
  return g;
}

template <class F, int M, int KB, bool PLAIN, int NT>
__device__ __forceinline__ void short_tile(const typename F::T* __restrict__ A, const typename F::T* __restrict__ B,
                                           typename F::T* __restrict__ C, const int64_t* __restrict__ orec,
                                           const int64_t* __restrict__ trec, int tcol, double alpha, double beta,
                                           typename F::T* Ak) {
  using T = typename F::T;
  constexpr int CPT = YB_GEMM_SHORT_COLS / NT;  // columns per thread
  constexpr int G = short_pass((int)sizeof(T), M, KB, CPT);
  const int64_t c_off = orec[0], ldc = orec[3], nc = orec[2];
  const int mr = M <= 4 ? M : (int)orec[1];  // M is exact below 5 rows
  const int K = (int)trec[2];
  const int64_t l_is = trec[3], l_ls = trec[4], r_ls = trec[5], r_js = trec[6];
  const int flags = (int)trec[7];
  const bool conjL = flags & 1, conjR = flags & 2;
  if (threadIdx.x < KB * M) {
    const int i = threadIdx.x % M, l = threadIdx.x / M;
    T v = F::zero();
    if (l < K && i < mr) {
      v = __ldg(A + trec[0] + i * l_is + l * l_ls);
      if (conjL) v = F::conj(v);
    }
    Ak[l * M + i] = v;
  }
  const int64_t j0 = (int64_t)tcol * YB_GEMM_SHORT_COLS + threadIdx.x;
  const T* __restrict__ Rb = B + trec[1];
  T b[KB][G];
  auto load_b = [&](int u0) {
#pragma unroll
    for (int u = 0; u < G; ++u) {
      const int64_t j = j0 + (u0 + u) * NT;
      const bool live = j < nc;
      const T* col = Rb + (live ? j * r_js : 0);
#pragma unroll
      for (int l = 0; l < KB; ++l) {
        b[l][u] = (live && l < K) ? __ldg(col + l * r_ls) : F::zero();
        if (conjR) b[l][u] = F::conj(b[l][u]);
      }
    }
  };
  load_b(0);
  __syncthreads();  // op(A) staged
#pragma unroll
  for (int u0 = 0; u0 < CPT; u0 += G) {
    if (u0) load_b(u0);
    T acc[G][M];
#pragma unroll
    for (int u = 0; u < G; ++u)
#pragma unroll
      for (int i = 0; i < M; ++i) acc[u][i] = F::zero();
#pragma unroll
    for (int l = 0; l < KB; ++l) {
      if (l < K) {
#pragma unroll
        for (int i = 0; i < M; ++i) {
          const T ai = Ak[l * M + i];
#pragma unroll
          for (int u = 0; u < G; ++u) F::fma(acc[u][i], ai, b[l][u]);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < G; ++u) {
      const int64_t j = j0 + (u0 + u) * NT;
      if (j >= nc) continue;
#pragma unroll
      for (int i = 0; i < M; ++i) {
        if (i >= mr) break;
        T* p = C + c_off + i * ldc + j;
        if (PLAIN) {
          *p = acc[u][i];
        } else {
          T v = F::scale(acc[u][i], alpha);
          if (beta != 0.0) v = F::add(v, F::scale(*p, beta));  // C is not read for beta = 0
          *p = v;
        }
      }
    }
  }
}

template <class F, bool PLAIN, int NT>
__device__ __forceinline__ void short_rows(const typename F::T* __restrict__ A, const typename F::T* __restrict__ B,
                                           typename F::T* __restrict__ C, const int64_t* __restrict__ orec,
                                           const int64_t* __restrict__ trec, int tcol, double alpha, double beta,
                                           typename F::T* Ak) {
  const bool k4 = trec[2] <= 4;
  switch ((int)orec[1]) {
    case 1: k4 ? short_tile<F, 1, 4, PLAIN, NT>(A, B, C, orec, trec, tcol, alpha, beta, Ak)
               : short_tile<F, 1, 8, PLAIN, NT>(A, B, C, orec, trec, tcol, alpha, beta, Ak); break;
    case 2: k4 ? short_tile<F, 2, 4, PLAIN, NT>(A, B, C, orec, trec, tcol, alpha, beta, Ak)
               : short_tile<F, 2, 8, PLAIN, NT>(A, B, C, orec, trec, tcol, alpha, beta, Ak); break;
    case 3: k4 ? short_tile<F, 3, 4, PLAIN, NT>(A, B, C, orec, trec, tcol, alpha, beta, Ak)
               : short_tile<F, 3, 8, PLAIN, NT>(A, B, C, orec, trec, tcol, alpha, beta, Ak); break;
    case 4: k4 ? short_tile<F, 4, 4, PLAIN, NT>(A, B, C, orec, trec, tcol, alpha, beta, Ak)
               : short_tile<F, 4, 8, PLAIN, NT>(A, B, C, orec, trec, tcol, alpha, beta, Ak); break;
    default: short_tile<F, 8, 8, PLAIN, NT>(A, B, C, orec, trec, tcol, alpha, beta, Ak); break;
  }
}

// A kind-2 tile (output, term index, strip, 2): both records are read at once.
template <class F, int NT>
__device__ __forceinline__ void short_dispatch(const typename F::T* __restrict__ A, const typename F::T* __restrict__ B,
                                               typename F::T* __restrict__ C, const int64_t* __restrict__ outs,
                                               const int64_t* __restrict__ terms, int4 tl, double alpha, double beta,
                                               typename F::T* Ak) {
  const int64_t* orec = outs + (int64_t)tl.x * YB_GEMM_OUT_REC;
  const int64_t* trec = terms + (int64_t)tl.y * YB_GEMM_TERM_REC;
  if (alpha == 1.0 && beta == 0.0)  // once per strip (FP64 compares)
    short_rows<F, true, NT>(A, B, C, orec, trec, tl.z, alpha, beta, Ak);
  else
    short_rows<F, false, NT>(A, B, C, orec, trec, tl.z, alpha, beta, Ak);
}

// Kernel of the short skinny strips only (tile kind 2): 256 threads x 2 columns; at most 64
// registers for FP64 (four CTAs, 32 warps per SM), 128 for complex128.
constexpr int kShortThreads = YB_GEMM_SHORT_COLS / 2;

template <class F>
__global__ void __launch_bounds__(kShortThreads, sizeof(typename F::T) == 8 ? 4 : 2) short_gemm_kernel(
    const typename F::T* __restrict__ A, const typename F::T* __restrict__ B, typename F::T* __restrict__ C,
    const int64_t* __restrict__ outs, const int64_t* __restrict__ terms, const int32_t* __restrict__ tiles,
    double alpha, double beta) {
  __shared__ typename F::T Ak[8 * 8];
  const int4 tl = reinterpret_cast<const int4*>(tiles)[blockIdx.x];
  short_dispatch<F, kShortThreads>(A, B, C, outs, terms, tl, alpha, beta, Ak);
}

template <class F>
__global__ void __launch_bounds__(kThreads) grouped_gemm_kernel(const typename F::T* __restrict__ A,
                                                                 const typename F::T* __restrict__ B,
                                                                 typename F::T* __restrict__ C,
                                                                 const int64_t* __restrict__ outs,
                                                                 const int64_t* __restrict__ terms,
                                                                 const int32_t* __restrict__ tiles,
                                                                 double alpha, double beta) {
  using T = typename F::T;
  __shared__ T As[kK][kTile + kPad];
  __shared__ T Bs[kK][kTile + kPad];

  const int4 tl = reinterpret_cast<const int4*>(tiles)[blockIdx.x];
  const int64_t* orec = outs + (int64_t)tl.x * YB_GEMM_OUT_REC;
  const int64_t c_off = orec[0], m = orec[1], n = orec[2], ldc = orec[3];
  const int64_t t0 = orec[4], t1 = orec[5];
  if (tl.w == 1) {  // skinny: the m <= 16 rows x 1024 (256) columns
    skinny_dispatch<F>(m, A, B, C, orec, terms, tl.z, alpha, beta, &As[0][0]);
    return;
  }
  if (tl.w == 2) {  // short skinny: m <= 8 rows, one term with K <= 8, 512 columns
    short_dispatch<F, kThreads>(A, B, C, outs, terms, tl, alpha, beta, &As[0][0]);
    return;
  }
  if (tl.w == 3) {  // tall skinny: 256 rows x all n <= 16 columns
    tall_dispatch<F>(n, A, B, C, orec, terms, tl.y, alpha, beta, &As[0][0]);
    return;
  }

  const int64_t row0 = (int64_t)tl.y * kTile, col0 = (int64_t)tl.z * kTile;

  // thread (ty, tx) owns rows 4ty..4ty+3 and columns 4tx..4tx+3; a warp covers 16 rows x 32
  // columns, so the warps of a small sector's tile that fall outside it skip the FMAs
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ty = (warp >> 1) * 4 + (lane >> 3);  // row group
  const int tx = (warp & 1) * 8 + (lane & 7);    // column group
  const bool active = (row0 + (warp >> 1) * 16 < m) && (col0 + (warp & 1) * 32 < n);
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = F::zero();

  for (int64_t t = t0; t < t1; ++t) {
    const int64_t* trec = terms + t * YB_GEMM_TERM_REC;
    const int64_t a_off = trec[0], b_off = trec[1], K = trec[2];
    const int64_t a_rs = trec[3], a_cs = trec[4], b_rs = trec[5], b_cs = trec[6];
    const int flags = (int)trec[7];
    const bool conjA = flags & 1, conjB = flags & 2;
    const bool a_kfast = (a_cs == 1);  // k is the contiguous index of A
    const bool b_jfast = (b_cs == 1) || (b_rs != 1);
    for (int64_t k0 = 0; k0 < K; k0 += kK) {
      // stage A tile: 64 rows x 16 k
#pragma unroll
      for (int r = 0; r < (kTile * kK) / kThreads; ++r) {
        const int e = threadIdx.x + r * kThreads;
        int i, l;
        if (a_kfast) { l = e % kK; i = e / kK; } else { i = e % kTile; l = e / kTile; }
        const int64_t gi = row0 + i, gl = k0 + l;
        T v = F::zero();
        if (gi < m && gl < K) {
          v = A[a_off + gi * a_rs + gl * a_cs];
          if (conjA) v = F::conj(v);
        }
        As[l][i] = v;
      }
      // stage B tile: 16 k x 64 cols
#pragma unroll
      for (int r = 0; r < (kTile * kK) / kThreads; ++r) {
        const int e = threadIdx.x + r * kThreads;
        int j, l;
        if (b_jfast) { j = e % kTile; l = e / kTile; } else { l = e % kK; j = e / kK; }
        const int64_t gj = col0 + j, gl = k0 + l;
        T v = F::zero();
        if (gj < n && gl < K) {
          v = B[b_off + gl * b_rs + gj * b_cs];
          if (conjB) v = F::conj(v);
        }
        Bs[l][j] = v;
      }
      __syncthreads();
      const int kn = (int)min((int64_t)kK, K - k0);
#pragma unroll
      for (int l = 0; l < kK; ++l) {
        if (!active || l >= kn) break;
        T a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[l][ty * 4 + i];
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = Bs[l][tx * 4 + j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) F::fma(acc[i][j], a[i], b[j]);
      }
      __syncthreads();
    }
  }
  // epilogue
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t gi = row0 + ty * 4 + i;
    if (gi >= m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t gj = col0 + tx * 4 + j;
      if (gj >= n) continue;
      T* p = C + c_off + gi * ldc + gj;
      T v = F::scale(acc[i][j], alpha);
      if (beta != 0.0) v = F::add(v, F::scale(*p, beta));
      *p = v;
    }
  }
}

// Split-K reduction: C_o = alpha * sum_{c < chunks} P[p_off + c m n + i n + j] + beta * C_o,
// the partial products summed in chunk order (deterministic). One CTA per task of
// YB_GEMM_RED_ITEM consecutive elements of one output.
template <class F>
__global__ void __launch_bounds__(kThreads) gemm_reduce_kernel(typename F::T* __restrict__ C,
                                                                const typename F::T* __restrict__ P,
                                                                const int64_t* __restrict__ recs,
                                                                const int32_t* __restrict__ tasks, double alpha,
                                                                double beta) {
  using T = typename F::T;
  const int2 tk = reinterpret_cast<const int2*>(tasks)[blockIdx.x];
  const int64_t* r = recs + (int64_t)tk.x * YB_GEMM_RED_REC;
  const int64_t c_off = r[0], n = r[2], ldc = r[3], p_off = r[4], chunks = r[5];
  const int64_t mn = r[1] * n;
  const int64_t e0 = (int64_t)tk.y * YB_GEMM_RED_ITEM;
  const int64_t e1 = min(e0 + (int64_t)YB_GEMM_RED_ITEM, mn);
  for (int64_t e = e0 + threadIdx.x; e < e1; e += kThreads) {
    T acc = F::zero();
    for (int64_t c = 0; c < chunks; ++c) acc = F::add(acc, P[p_off + c * mn + e]);
    const int64_t i = e / n, j = e - i * n;
    T* p = C + c_off + i * ldc + j;
    T v = F::scale(acc, alpha);
    if (beta != 0.0) v = F::add(v, F::scale(*p, beta));
    *p = v;
  }
}

}  // namespace
}  // namespace yb

extern "C" int yb_gemm_reduce(void* c, const void* p, int dtype, const int64_t* recs, const int32_t* tasks,
                              int n_tasks, double alpha, double beta, void* stream) {
  if (n_tasks == 0) return YB_OK;
  if (!c || !p || !recs || !tasks || n_tasks < 0) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64) {
    yb::gemm_reduce_kernel<yb::Real><<<n_tasks, yb::kThreads, 0, s>>>((double*)c, (const double*)p, recs, tasks,
                                                                      alpha, beta);
  } else if (dtype == YB_C128) {
    yb::gemm_reduce_kernel<yb::Cplx><<<n_tasks, yb::kThreads, 0, s>>>((double2*)c, (const double2*)p, recs,
                                                                      tasks, alpha, beta);
  } else {
    return YB_ERR_INVALID;
  }
  return yb::check_launch();
}

extern "C" int yb_grouped_gemm(const void* a, const void* b, void* c, int dtype, const int64_t* outs,
                               const int64_t* terms, const int32_t* tiles, int n_tiles, double alpha,
                               double beta, void* stream) {
  if (n_tiles == 0) return YB_OK;
  if (!a || !b || !c || !outs || !tiles || n_tiles < 0) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64) {
    yb::grouped_gemm_kernel<yb::Real><<<n_tiles, yb::kThreads, 0, s>>>(
        (const double*)a, (const double*)b, (double*)c, outs, terms, tiles, alpha, beta);
  } else if (dtype == YB_C128) {
    yb::grouped_gemm_kernel<yb::Cplx><<<n_tiles, yb::kThreads, 0, s>>>(
        (const double2*)a, (const double2*)b, (double2*)c, outs, terms, tiles, alpha, beta);
  } else {
    return YB_ERR_INVALID;
  }
  return yb::check_launch();
}

extern "C" int yb_grouped_gemm_short(const void* a, const void* b, void* c, int dtype, const int64_t* outs,
                                     const int64_t* terms, const int32_t* tiles, int n_tiles, double alpha,
                                     double beta, void* stream) {
  if (n_tiles == 0) return YB_OK;
  if (!a || !b || !c || !outs || !terms || !tiles || n_tiles < 0) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64) {
    yb::short_gemm_kernel<yb::Real><<<n_tiles, yb::kShortThreads, 0, s>>>(
        (const double*)a, (const double*)b, (double*)c, outs, terms, tiles, alpha, beta);
  } else if (dtype == YB_C128) {
    yb::short_gemm_kernel<yb::Cplx><<<n_tiles, yb::kShortThreads, 0, s>>>(
        (const double2*)a, (const double2*)b, (double2*)c, outs, terms, tiles, alpha, beta);
  } else {
    return YB_ERR_INVALID;
  }
  return yb::check_launch();
}
