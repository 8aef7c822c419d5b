// Family (b'): FP64 sector GEMMs emulated with split operands on BF16 tensor cores
// (Ozaki scheme, error-free splitting with per-row / per-column exponents).
//
// Splitting: every row i of A (and every column j of B) is scaled by a power of two
// 2^-e so that its entries lie in (-1, 1), then written as s signed integer digits
//     v = sum_{t<s} d_t 2^{-7(t+1)},  d_0 in [-128, 128], d_t in [-64, 63] (t > 0),
// (balanced base-128 digits of rint(v 2^{7s}), integer arithmetic). Every digit is an
// integer of at most 8 significant bits and is stored exactly as BF16. A slice pair (t_a, t_b)
// contributes 2^{e_i + f_j - 14 - 7 (t_a + t_b)} (D_A[t_a] D_B[t_b])_ij; pairs with
// t_a + t_b <= s - 1 are kept (s(s+1)/2 products), the rest are below the FP64 rounding
// of the result for s = 8 (57 bits of each operand are represented).
//
// Exactness of the tensor-core products: a digit product is an integer of magnitude
// <= 2^14 (<= 2^13 unless both digits are leading ones); all pairs of one diagonal
// t = t_a + t_b share one FP32 accumulator over a K-chunk of 400, so every partial sum is
// an integer below 2^24 and is exact in FP32. After each chunk the diagonals are folded
// exactly into two int64 halves, which are added to FP64 accumulators; the final scale
// is an exponent-field add.
//
// GEMM kernel: 64x64 output tile per CTA, 8 warps each owning a 32x16 sub-tile (2x2
// mma.sync.m16n8k16 tiles), K-step 16 staged in shared memory with cp.async (double
// buffered, rows padded to 48 bytes so ldmatrix is bank-conflict free).
#include <atomic>
#include <type_traits>
#include <mutex>
#include "yb_ozaki_common.cuh"

namespace yb {
namespace {
using oz::scaled_rint;
using oz::scale_pow2;
using oz::fold_round;

constexpr int kTile = 64;
constexpr int kK = 16;
constexpr int kRow = 24;  // smem row stride in bf16 elements (16 data + 8 pad = 48 bytes)
// K-chunk of 25 * 16 = 400: on diagonal t the per-k sum of digit products is at most
// 2 * 2^13 + (t - 1) * 2^12 = (t + 3) 2^12 <= 10 * 2^12 (t <= 7), so a chunk sum stays
// below 400 * 10 * 2^12 < 2^24 and is exact in FP32.
constexpr int kChunkSteps = 25;
constexpr int kThreads = 256;

// ------------------------------------------------------------------ splitting
// Split record (YB_OZ_SPLIT_REC = 10 int64):
//   [0] source offset [1] rows [2] K (length of the real rows) [3] row stride [4] mode
//   [5] destination offset (BF16 elements) [6] exponent offset [7] Kp (K rounded up to 16)
//   [8] stride between consecutive k [9] operand (bit 0: 0 = A, 1 = B) | tile rows << 8
// Element k of row i is read at source offset [0] + i*[3] + k*[8] (FP64 elements for mode 0,
// complex elements for modes 1-3), so an A block (rows contiguous, [8] = 1) and a B block
// read by columns ([3] = 1, [8] = n: the rows of B^T, no transposed copy) are split alike.
// mode 0: a real row; modes 1-3: a complex128 row of K/2 values read as the real row
// [re | im] (1), [re | -im] (2) or [im | re] (3), the operands of the two real products
// C_r = [A_r, A_i][B_r; -B_i] and C_i = [A_r, A_i][B_i; B_r] of a complex GEMM.
// Destination layouts (padding zero-filled):
//   tile rows 0: planes [slice][row][Kp] (the mma.sync kernel);
//   tile rows TH (64 or 128): per slice, the rows padded to a multiple of TH, in blocks of
//   TH rows x 16 k ordered (row tile, K step), each block in the canonical K-major
//   core-matrix order of the tcgen05 descriptors (element offset of (row r, k) in a block:
//   (r/8)*128 + (k/8)*64 + (r%8)*8 + k%8).
//
// The digits are extracted with integer arithmetic only (GB300's FP64 pipe is narrow):
// Q = rint(a 2^{7s-e}) (|Q| < 2^{7s}) is formed from a's mantissa and exponent bits by a
// shift with round-half-to-even, then the balanced base-128 digits follow from
// U = Q + 64 (1 + 128 + ... + 128^{s-2}): d_t = ((U >> 7(s-1-t)) & 127) - 64 for t >= 1 and
// the leading digit d_0 = U >> 7(s-1) in [-128, 128] (arithmetic shift). This represents
// a 2^-e = sum_t d_t 2^{-7(t+1)} up to the rounding of Q (half a unit of the last digit).
// A digit d (|d| <= 128, at most 8 significant bits) becomes its BF16 pattern without a
// conversion instruction: the FP32 value 1.5*2^23 + d has the bit pattern 0x4B400000 + d,
// subtracting 1.5*2^23 leaves d exactly, and the upper half of d's FP32 pattern is its BF16.
constexpr int kSplitRec = 10;
constexpr int kSplitRows = 8;       // rows per CTA
constexpr int kSplitThreads = 256;  // thread t: row t % 8, chunk lane t / 8
constexpr int kSplitLanes = kSplitThreads / kSplitRows;  // 32 chunk lanes: chunks c = lane, lane + 32, ...

__host__ __device__ constexpr long long digit_bias(int s) {
  return s <= 1 ? 0 : (digit_bias(s - 1) << 7) | 64;
}

__device__ __forceinline__ uint32_t digit_f32(int field_plus_magic) {
  return __float_as_uint(__int_as_float(field_plus_magic) - 12582912.0f);
}

// The S digits of one element as FP32 bit patterns (BF16 in the upper halves).
template <int S>
__device__ __forceinline__ void digit_words(long long bits, int e, uint32_t* w) {
  constexpr long long kBias = digit_bias(S);
  const long long u = scaled_rint(bits, e, S) + kBias;
  const uint32_t lo = (uint32_t)u, hi = (uint32_t)((unsigned long long)u >> 32);
  w[0] = digit_f32(0x4B400000 + ((int)hi >> (7 * (S - 1) - 32)));
#pragma unroll
  for (int t = 1; t < S; ++t) {
    const int o = 7 * (S - 1 - t);
    uint32_t f;
    if (o >= 32) f = hi >> (o - 32);
    else if (o + 7 <= 32) f = lo >> o;
    else f = __funnelshift_r(lo, hi, o);
    w[t] = digit_f32(0x4B400000 - 64 + (int)(f & 127u));
  }
}


// One CTA per 8 rows of a record (groups: int32 pairs (record, first row)); the 256 threads
// are 8 rows x 32 chunk lanes, each lane taking the row's 8-long K chunks lane, lane + 32, ...:
// the row maxima first (exponents), then the digits, each chunk stored as one 16-byte word
// per slice (8 consecutive rows of a tile-layout block are 128 contiguous bytes). Real rows
// with at most two chunks per lane (K <= 512) keep their values in registers between the two
// passes; a group wholly in the row padding of the tile layout only writes zeros.
template <int S>
__device__ __forceinline__ void store_chunk(__nv_bfloat16* dst, int64_t slice_stride, int64_t off, const long long* x,
                                           int e) {
  uint32_t pk[S][4];
#pragma unroll
  for (int u = 0; u < 8; u += 2) {
    uint32_t w0[S], w1[S];
    digit_words<S>(x[u], e, w0);
    digit_words<S>(x[u + 1], e, w1);
#pragma unroll
    for (int t = 0; t < S; ++t) pk[t][u >> 1] = __byte_perm(w0[t], w1[t], 0x7632);
  }
#pragma unroll
  for (int t = 0; t < S; ++t)
    *reinterpret_cast<uint4*>(dst + t * slice_stride + off) = make_uint4(pk[t][0], pk[t][1], pk[t][2], pk[t][3]);
}

template <int S>
__global__ void __launch_bounds__(kSplitThreads, 3) split_kernel(
    const double* __restrict__ a_src, const double* __restrict__ b_src, __nv_bfloat16* __restrict__ a_dst,
    __nv_bfloat16* __restrict__ b_dst, int* __restrict__ a_exps, int* __restrict__ b_exps,
    const int64_t* __restrict__ recs, const int32_t* __restrict__ groups) {
  __shared__ long long smax[kSplitLanes][kSplitRows];
  __shared__ int sexp[kSplitRows];
  const int2 g = reinterpret_cast<const int2*>(groups)[blockIdx.x];
  const int64_t* r = recs + (int64_t)g.x * kSplitRec;
  const int64_t rows = r[1], K = r[2], Kp = r[7];
  const int flags = (int)r[9];
  const bool opb = flags & 1;
  const int TH = flags >> 8;
  const int ri = threadIdx.x % kSplitRows, cl = threadIdx.x / kSplitRows;
  const int64_t row = (int64_t)g.y + ri;
  const bool live = row < rows;
  const int64_t nck = Kp / 8;  // chunks of the padded row
  // destination of chunk c of this row
  int64_t slice_stride, row_base;
  int in_tile = 0;
  if (TH == 0) {
    slice_stride = rows * Kp;
    row_base = row * Kp;
  } else {
    slice_stride = (rows + TH - 1) / TH * TH * Kp;
    const int rr = (int)(row % TH);
    row_base = (row / TH) * (Kp / 16) * (int64_t)TH * 16;
    in_tile = (rr >> 3) * 128 + (rr & 7) * 8;
  }
  auto offset = [&](int64_t c) -> int64_t {
    return TH == 0 ? row_base + 8 * c : row_base + (c >> 1) * (int64_t)TH * 16 + in_tile + (c & 1) * 64;
  };
  __nv_bfloat16* dst = (opb ? b_dst : a_dst) + r[5];
  if (g.y >= rows) {  // all 8 rows are padding rows of the tile layout: zeros
    const uint4 z = make_uint4(0u, 0u, 0u, 0u);
    for (int64_t c = cl; c < nck; c += kSplitLanes)
#pragma unroll
      for (int t = 0; t < S; ++t) *reinterpret_cast<uint4*>(dst + t * slice_stride + offset(c)) = z;
    return;
  }
  const int mode = (int)r[4];
  const int64_t ks = r[8];
  const long long* base =
      reinterpret_cast<const long long*>(opb ? b_src : a_src) + (mode == 0 ? 1 : 2) * (r[0] + (live ? row : 0) * r[3]);
  // bit pattern of element k (k < K) of this row
  auto elem = [&](int64_t k) -> long long {
    if (mode == 0) return __ldg(base + k * ks);
    const int64_t half = K / 2;
    const bool first = k < half;
    const long long* c = base + 2 * (first ? k : k - half) * ks;
    const long long re = __ldg(c), im = __ldg(c + 1);
    if (mode == 1) return first ? re : im;
    if (mode == 2) return first ? re : (long long)((unsigned long long)im ^ 0x8000000000000000ull);
    return first ? im : re;
  };
  auto load_chunk = [&](int64_t c, long long* x) {
    const int64_t k0 = 8 * c;
    if (mode == 0 && live && k0 + 8 <= K) {
      const long long* p = base + k0 * ks;
#pragma unroll
      for (int u = 0; u < 8; ++u) x[u] = __ldg(p + u * ks);
    } else {
#pragma unroll
      for (int u = 0; u < 8; ++u) x[u] = (live && k0 + u < K) ? elem(k0 + u) : 0ll;
    }
  };
  auto rowmax = [&](const long long* x, long long mx) {
#pragma unroll
    for (int u = 0; u < 8; ++u) mx = max(mx, x[u] & 0x7fffffffffffffffll);
    return mx;
  };
  auto exponent = [&](long long mx) {
    smax[cl][ri] = mx;
    __syncthreads();
    if (threadIdx.x < kSplitRows) {
#pragma unroll 8
      for (int w = 1; w < kSplitLanes; ++w) mx = max(mx, smax[w][ri]);
      int e = 0;  // max |a| = f 2^e, f in [0.5, 1): |a| < 2^e
      if (mx >= (1ll << 52)) e = (int)(mx >> 52) - 1022;
      else if (mx > 0) frexp(__longlong_as_double(mx), &e);
      sexp[ri] = e;
      if (live) (opb ? b_exps : a_exps)[r[6] + row] = e;
    }
    __syncthreads();
    return sexp[ri];
  };
  const bool pad_row = TH == 0 && !live;  // planes layout: rows past the record are not stored
  if (nck <= 2 * kSplitLanes) {
    // at most two chunks per lane: values held in registers between the passes
    long long x0[8], x1[8];
    const int64_t c0 = cl, c1 = cl + kSplitLanes;
    load_chunk(c0 < nck ? c0 : 0, x0);
    load_chunk(c1 < nck ? c1 : 0, x1);
    long long mx = 0;
    if (c0 < nck) mx = rowmax(x0, mx);
    if (c1 < nck) mx = rowmax(x1, mx);
    const int e = exponent(mx);
    if (pad_row) return;
    if (c0 < nck) store_chunk<S>(dst, slice_stride, offset(c0), x0, e);
    if (c1 < nck) store_chunk<S>(dst, slice_stride, offset(c1), x1, e);
    return;
  }
  long long mx = 0;
  for (int64_t c = cl; c < nck; c += kSplitLanes) {
    long long x[8];
    load_chunk(c, x);
    mx = rowmax(x, mx);
  }
  const int e = exponent(mx);
  if (pad_row) return;
  for (int64_t c = cl; c < nck; c += kSplitLanes) {
    long long x[8];
    load_chunk(c, x);
    store_chunk<S>(dst, slice_stride, offset(c), x, e);
  }
}

template <int S>
int launch_split(const double* a_src, const double* b_src, void* a_dst, void* b_dst, int* a_exps, int* b_exps,
                 const int64_t* recs, const int32_t* groups, int n_groups, cudaStream_t s) {
  split_kernel<S><<<n_groups, kSplitThreads, 0, s>>>(a_src, b_src, (__nv_bfloat16*)a_dst,
                                                                  (__nv_bfloat16*)b_dst, a_exps, b_exps, recs, groups);
  return check_launch();
}

// ------------------------------------------------------------------ GEMM
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
  const unsigned saddr = (unsigned)__cvta_generic_to_shared(smem);
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(saddr), "l"(gmem), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }

__device__ __forceinline__ void ldmatrix_x4(unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3, const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(a));
}
__device__ __forceinline__ void ldmatrix_x2(unsigned& r0, unsigned& r1, const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(a));
}
__device__ __forceinline__ void mma_bf16(float* c, const unsigned* a, const unsigned* b) {
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
               "{%0,%1,%2,%3};\n"
               : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// out record: [0] c offset [1] m [2] n [3] ldc [4] A slices offset [5] A exp offset
//             [6] B slices offset [7] B exp offset [8] K [9] Kp [10] output column stride
//             (0 or 1: contiguous; 2: the real or imaginary part of complex output)
template <int S>
__global__ void __launch_bounds__(kThreads, 1) ozaki_gemm_kernel(const __nv_bfloat16* __restrict__ As,
                                                                 const int* __restrict__ Ae,
                                                                 const __nv_bfloat16* __restrict__ Bs,
                                                                 const int* __restrict__ Be, double* __restrict__ C,
                                                                 const int64_t* __restrict__ outs,
                                                                 const int32_t* __restrict__ tiles) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16* sA = reinterpret_cast<__nv_bfloat16*>(smem_raw);          // [2][S][64][kRow]
  __nv_bfloat16* sB = sA + 2 * S * kTile * kRow;                           // [2][S][64][kRow]
  const int4 tl = reinterpret_cast<const int4*>(tiles)[blockIdx.x];
  const int64_t* o = outs + (int64_t)tl.x * 16;
  const int64_t c_off = o[0], m = o[1], n = o[2], ldc = o[3];
  const int64_t a_sl = o[4], a_ex = o[5], b_sl = o[6], b_ex = o[7], Kp = o[9];
  const int64_t ccs = o[10] > 0 ? o[10] : 1;  // output column stride (2: one part of complex data)
  const int64_t row0 = (int64_t)tl.y * kTile, col0 = (int64_t)tl.z * kTile;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = warp & 1, wn = warp >> 1;  // warp sub-tile: rows wm*32.., cols wn*16..
  // a warp whose sub-tile lies wholly outside the sector (small m or n) only helps staging
  const bool active = (row0 + wm * 32 < m) && (col0 + wn * 16 < n);

  const int64_t a_stride = m * Kp, b_stride = n * Kp;
  auto stage = [&](int buf, int64_t k0) {
    // S slices x 64 rows x 16 k = S*128 chunks of 16 bytes for each operand
    for (int c = threadIdx.x; c < S * kTile * 2; c += kThreads) {
      const int t = c / (kTile * 2), rem = c % (kTile * 2), rr = rem >> 1, half = rem & 1;
      const int64_t ga = row0 + rr, gb = col0 + rr;
      const bool va = ga < m, vb = gb < n;
      const __nv_bfloat16* srcA = As + a_sl + t * a_stride + (va ? ga : 0) * Kp + k0 + half * 8;
      const __nv_bfloat16* srcB = Bs + b_sl + t * b_stride + (vb ? gb : 0) * Kp + k0 + half * 8;
      cp_async16(sA + ((buf * S + t) * kTile + rr) * kRow + half * 8, srcA, va);
      cp_async16(sB + ((buf * S + t) * kTile + rr) * kRow + half * 8, srcB, vb);
    }
    cp_async_commit();
  };

  float acc[S][2][2][4];
  double acc64[2][2][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc64[i][j][v] = 0.0;
#pragma unroll
  for (int d = 0; d < S; ++d)
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[d][i][j][v] = 0.f;

  const int64_t nsteps = Kp / kK;
  if (nsteps > 0) stage(0, 0);
  for (int64_t st = 0; st < nsteps; ++st) {
    const int buf = st & 1;
    cp_async_wait_all();
    __syncthreads();
    if (st + 1 < nsteps) stage(buf ^ 1, (st + 1) * kK);
    if (!active) continue;
#pragma unroll
    for (int ta = 0; ta < S; ++ta) {
      unsigned af[2][4];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const __nv_bfloat16* p = sA + ((buf * S + ta) * kTile + wm * 32 + i * 16 + (lane & 15)) * kRow + (lane >> 4) * 8;
        ldmatrix_x4(af[i][0], af[i][1], af[i][2], af[i][3], p);
      }
#pragma unroll
      for (int tb = 0; tb < S - ta; ++tb) {
        unsigned bf[2][2];
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const __nv_bfloat16* p =
              sB + ((buf * S + tb) * kTile + wn * 16 + j * 8 + (lane & 7)) * kRow + ((lane >> 3) & 1) * 8;
          ldmatrix_x2(bf[j][0], bf[j][1], p);
        }
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int j = 0; j < 2; ++j) mma_bf16(acc[ta + tb][i][j], af[i], bf[j]);
      }
    }
    if (((st + 1) % kChunkSteps) == 0 || st + 1 == nsteps) {
      // fold the diagonal sums (exact integers below 2^24 in FP32) into FP64: the weighted
      // sum sum_d acc_d 2^(-7d) is formed exactly in two int64 halves (diagonals 0..3 and
      // 4..7, each below 2^46) and rounded once (fold_round), on the integer pipe, which
      // keeps the fold off GB300's narrow FP64 pipe; the first chunk is assigned, later ones
      // added (two copies of the loop, so that the first issues no FP64 add)
      auto fold = [&](auto first_tag) {
        constexpr bool kFirst = decltype(first_tag)::value;
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int v = 0; v < 4; ++v) {
              int qi[S];
#pragma unroll
              for (int d = 0; d < S; ++d) {
                qi[d] = __float2int_rn(acc[d][i][j][v]);
                acc[d][i][j][v] = 0.f;
              }
              long long hi, lo;
              oz::fold_halves<S>(qi, hi, lo);
              const double x = fold_round(hi, lo, 7 * (S - 4), -7 * (S - 1));
              if (kFirst) acc64[i][j][v] = x;
              else acc64[i][j][v] += x;
            }
      };
      if (st < kChunkSteps) fold(std::true_type{});
      else fold(std::false_type{});
    }
  }
  // epilogue: C = acc64 * 2^(e_i + f_j - 14)
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int64_t gi = row0 + wm * 32 + i * 16 + (lane >> 2) + (v >= 2 ? 8 : 0);
        const int64_t gj = col0 + wn * 16 + j * 8 + (lane & 3) * 2 + (v & 1);
        if (gi < m && gj < n)
          C[c_off + gi * ldc + gj * ccs] = scale_pow2(acc64[i][j][v], Ae[a_ex + gi] + Be[b_ex + gj] - 14);
      }
}

template <int S>
int launch_gemm(const void* As, const int* Ae, const void* Bs, const int* Be, double* C, const int64_t* outs,
                const int32_t* tiles, int n_tiles, cudaStream_t s) {
  const size_t smem = (size_t)2 * 2 * S * kTile * kRow * sizeof(__nv_bfloat16);
  cudaError_t e = cudaFuncSetAttribute(ozaki_gemm_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) { set_cuda_error((int)e); return YB_ERR_CUDA; }
  ozaki_gemm_kernel<S><<<n_tiles, kThreads, smem, s>>>((const __nv_bfloat16*)As, Ae, (const __nv_bfloat16*)Bs, Be, C,
                                                       outs, tiles);
  return check_launch();
}

}  // namespace
}  // namespace yb

extern "C" {

int yb_ozaki_split(const double* a_src, const double* b_src, void* a_slices, void* b_slices, int* a_exps,
                   int* b_exps, const int64_t* recs, const int32_t* groups, int n_groups, int slices_count,
                   void* stream) {
  if (n_groups == 0) return YB_OK;
  if (!recs || !groups || n_groups < 0) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  switch (slices_count) {
    case 6: return yb::launch_split<6>(a_src, b_src, a_slices, b_slices, a_exps, b_exps, recs, groups, n_groups, s);
    case 7: return yb::launch_split<7>(a_src, b_src, a_slices, b_slices, a_exps, b_exps, recs, groups, n_groups, s);
    case 8: return yb::launch_split<8>(a_src, b_src, a_slices, b_slices, a_exps, b_exps, recs, groups, n_groups, s);
    default: return YB_ERR_INVALID;
  }
}

int yb_ozaki_gemm(const void* a_slices, const int* a_exps, const void* b_slices, const int* b_exps, double* c,
                  const int64_t* outs, const int32_t* tiles, int n_tiles, int slices_count, void* stream) {
  if (n_tiles == 0) return YB_OK;
  if (!a_slices || !a_exps || !b_slices || !b_exps || !c || !outs || !tiles) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  switch (slices_count) {
    case 6: return yb::launch_gemm<6>(a_slices, a_exps, b_slices, b_exps, c, outs, tiles, n_tiles, s);
    case 7: return yb::launch_gemm<7>(a_slices, a_exps, b_slices, b_exps, c, outs, tiles, n_tiles, s);
    case 8: return yb::launch_gemm<8>(a_slices, a_exps, b_slices, b_exps, c, outs, tiles, n_tiles, s);
    default: return YB_ERR_INVALID;
  }
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// yb_ozaki_dot_static: the same emulated dot with its scratch (digit planes, exponents and
// the transposed B blocks) in a file-scope device array instead of caller memory, for
// callers that cannot allocate device memory. Every GPU that loads the library holds the
// array (YB_STATIC_SCRATCH_BYTES) until the process exits. All calls share it and it keeps
// the last call's contents: every region is fully rewritten before it is read, and calls
// that overlap on the GPU (different streams, or threads) race on it.
static __device__ __align__(256) unsigned char g_ozaki_static_scratch[YB_STATIC_SCRATCH_BYTES];

namespace yb {
namespace {
constexpr int kMaxDevices = 64;
std::atomic<unsigned char*> g_static_ptr[kMaxDevices];
std::mutex g_static_mu;

// Device address of the static scratch for the current device. The first call on a device
// resolves it with cudaGetSymbolAddress (with that device current) and caches it.
int static_scratch(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) { set_cuda_error((int)e); return YB_ERR_CUDA; }
  if (dev < 0 || dev >= kMaxDevices) return YB_ERR_INVALID;
  unsigned char* p = g_static_ptr[dev].load(std::memory_order_acquire);
  if (p == nullptr) {
    std::lock_guard<std::mutex> lock(g_static_mu);
    p = g_static_ptr[dev].load(std::memory_order_acquire);
    if (p == nullptr) {
      void* q = nullptr;
      e = cudaGetSymbolAddress(&q, g_ozaki_static_scratch);
      if (e != cudaSuccess || q == nullptr) { set_cuda_error((int)e); return YB_ERR_CUDA; }
      p = static_cast<unsigned char*>(q);
      g_static_ptr[dev].store(p, std::memory_order_release);
    }
  }
  *out = p;
  return YB_OK;
}

inline int64_t align256(int64_t x) { return (x + 255) & ~(int64_t)255; }
}  // namespace
}  // namespace yb

extern "C" int yb_ozaki_dot_static(const double* A, const double* B, double* C, int dtype,
                                   const int64_t* split_recs, const int32_t* split_groups, int n_groups,
                                   const int64_t* outs, const int32_t* tiles, int n_tiles, const int64_t* nat_outs,
                                   const int64_t* nat_terms, const int32_t* nat_tiles, int n_nat_tiles,
                                   int slices_count, int64_t a_slice_elems, int64_t b_slice_elems, int64_t a_exp_count,
                                   int64_t b_exp_count, void* stream) {
  if (dtype != YB_F64) return YB_ERR_INVALID;  // complex split records are not accepted here
  if (n_tiles == 0 && n_nat_tiles == 0) return YB_OK;
  if (!A || !B || !C || n_groups < 0 || n_tiles < 0 || n_nat_tiles < 0) return YB_ERR_INVALID;
  if (n_tiles > 0 && (!split_recs || !split_groups || !outs || !tiles)) return YB_ERR_INVALID;
  if (n_nat_tiles > 0 && (!nat_outs || !nat_terms || !nat_tiles)) return YB_ERR_INVALID;
  if (a_slice_elems < 0 || b_slice_elems < 0 || a_exp_count < 0 || b_exp_count < 0) return YB_ERR_INVALID;
  const int64_t off_a = 0;
  const int64_t off_b = yb::align256(off_a + 2 * a_slice_elems);
  const int64_t off_ea = yb::align256(off_b + 2 * b_slice_elems);
  const int64_t off_eb = yb::align256(off_ea + 4 * a_exp_count);
  const int64_t total = yb::align256(off_eb + 4 * b_exp_count);
  if (total > (int64_t)YB_STATIC_SCRATCH_BYTES) return YB_ERR_TOO_LARGE;
  // sectors with K < 16 or skinny outputs: the native FP64 kernel, which needs no scratch
  int st = yb_grouped_gemm(A, B, C, YB_F64, nat_outs, nat_terms, nat_tiles, n_nat_tiles, 1.0, 0.0, stream);
  if (st != YB_OK || n_tiles == 0) return st;
  unsigned char* base = nullptr;
  st = yb::static_scratch(&base);
  if (st != YB_OK) return st;
  int* ea = reinterpret_cast<int*>(base + off_ea);
  int* eb = reinterpret_cast<int*>(base + off_eb);
  st = yb_ozaki_split(A, B, base + off_a, base + off_b, ea, eb, split_recs, split_groups, n_groups, slices_count,
                      stream);
  if (st != YB_OK) return st;
  return yb_ozaki_gemm(base + off_a, ea, base + off_b, eb, C, outs, tiles, n_tiles, slices_count, stream);
}
