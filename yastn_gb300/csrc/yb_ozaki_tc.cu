// Family (b'), tensor-core form: FP64 sector GEMMs emulated on the tcgen05 tensor cores with
// the operand split fused into the GEMM (no digit planes in global memory).
//
// Each CTA computes a 128 x 64 output tile. Eight converter warps read the FP64 operand tiles
// of a 16-long K step straight from the merged operands (A: 128 rows x 16, row-major blocks;
// B: 16 rows x 64 columns of a K x n row-major block, so no transposed copy of B is needed),
// write every value as S balanced base-128 digits in BF16 (the integer digit split of
// yb_ozaki_split, with the per-row / per-column exponents of yb_ozaki_exponents) directly in
// the canonical K-major core-matrix layout of the UMMA shared-memory descriptors, and hand
// the stage to the MMA warp through an mbarrier. One thread of the MMA warp issues the
// S(S+1)/2 tcgen05.mma (M=128, N=64, K=16, BF16 -> FP32) of a step into the S digit-diagonal
// accumulators in tensor memory (S x 64 of the 512 TMEM columns) and frees the stage with
// tcgen05.commit. At the end of every 400-long K chunk (exact FP32 integer sums, as in the
// mma.sync kernel) the converter warps read the accumulators back (warp w: TMEM lanes
// 32 (w mod 4).., 32 of the 64 columns), combine the diagonals exactly into a 128-bit integer
// on the integer pipe, round it once to FP64 and add it to the tile's FP64 accumulators, so
// the result is bit-identical to the mma.sync kernel's. Complex sectors (two real products
// with doubled K, C_r = [A_r, A_i][B_r; -B_i], C_i = [A_r, A_i][B_i; B_r]) read the real-part
// and imaginary-part segments of K in turn. Every wait is bounded; a CTA that gives up
// records the status word of yb_ozaki_device_error, waits (bounded) for its MMAs, frees its
// tensor memory and writes nothing.
#include "yb_ozaki_common.cuh"

namespace yb {
namespace {
using namespace oz;

constexpr int kM = 128, kN = 64, kK = 16, kStages = 4;
constexpr int kConv = 256;             // converter / fold threads (8 warps)
constexpr int kThreadsF = kConv + 32;  // + the MMA warp
constexpr int kChunkSteps = 25;        // 400-long K chunks: exact FP32 diagonal sums
constexpr long long kSpin = 1ll << 24;
constexpr uint32_t kATile = kM * kK * 2;  // one slice's 128 x 16 digit tile, bytes
constexpr uint32_t kBTile = kN * kK * 2;  // 64 x 16

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void conv_bar() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

// Digits of slice T of the 8 A values (one 16-byte core-matrix row) and of the 4 B values
// (8 bytes), stored for every slice T < S.
template <int S, int T>
struct StoreDigits {
  __device__ __forceinline__ static void run(unsigned char* stage, uint32_t a_dst, uint32_t b_dst,
                                             const long long* au, const long long* bu) {
    uint4 v;
    v.x = pack_bf16(digit_bits<S, T>(au[0]), digit_bits<S, T>(au[1]));
    v.y = pack_bf16(digit_bits<S, T>(au[2]), digit_bits<S, T>(au[3]));
    v.z = pack_bf16(digit_bits<S, T>(au[4]), digit_bits<S, T>(au[5]));
    v.w = pack_bf16(digit_bits<S, T>(au[6]), digit_bits<S, T>(au[7]));
    *reinterpret_cast<uint4*>(stage + T * kATile + a_dst) = v;
    uint2 w;
    w.x = pack_bf16(digit_bits<S, T>(bu[0]), digit_bits<S, T>(bu[1]));
    w.y = pack_bf16(digit_bits<S, T>(bu[2]), digit_bits<S, T>(bu[3]));
    *reinterpret_cast<uint2*>(stage + b_dst + T * kBTile) = w;
    StoreDigits<S, T + 1>::run(stage, a_dst, b_dst, au, bu);
  }
};
template <int S>
struct StoreDigits<S, S> {
  __device__ __forceinline__ static void run(unsigned char*, uint32_t, uint32_t, const long long*,
                                             const long long*) {}
};

// out record (16 int64): [0] c offset (FP64 words) [1] m [2] n [3] ldc (FP64 words)
// [4] A offset (elements) [5] A exponents offset [6] B offset (elements) [7] B exponents offset
// [8] K [9] lda (elements) [10] output column stride (FP64 words) [11] complex part
// (0: real part, 1: imaginary part) [12] 1 for complex operands [13] ldb (elements)
template <int S>
__global__ void __launch_bounds__(kThreadsF, 1)
    ozaki_fused_kernel(const double* __restrict__ A, const double* __restrict__ B, const int* __restrict__ exps,
                       double* __restrict__ C, const int64_t* __restrict__ outs, const int32_t* __restrict__ tiles,
                       int* __restrict__ err) {
  constexpr uint32_t kStage = S * (kATile + kBTile);
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint32_t tmem_slot;
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], accb, tfree, drain;
  __shared__ int failed_s;
  volatile int* failed = &failed_s;

  const int4 tl = reinterpret_cast<const int4*>(tiles)[blockIdx.x];
  const int64_t* o = outs + (int64_t)tl.x * 16;
  const int64_t c_off = o[0], m = o[1], n = o[2], ldc = o[3], a_off = o[4], a_ex = o[5], b_off = o[6];
  const int64_t b_ex = o[7], K = o[8], lda = o[9], ccs = o[10] > 0 ? o[10] : 1, ldb = o[13];
  const int part = (int)o[11], cplx = (int)o[12];
  const int64_t row0 = (int64_t)tl.y * kM, col0 = (int64_t)tl.z * kN;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t sbase = smem_u32(smem);
  const int64_t kseg = (K + kK - 1) / kK;         // K steps of one segment
  const int64_t ksteps = cplx ? 2 * kseg : kseg;  // complex: real-part segment, then imaginary-part one
  const int64_t nchunks = (ksteps + kChunkSteps - 1) / kChunkSteps;

  if (warp == 8) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == kConv) {
    for (int i = 0; i < kStages; ++i) {
      mbar_init(smem_u32(&full[i]), kConv);
      mbar_init(smem_u32(&empty[i]), 1);
    }
    mbar_init(smem_u32(&accb), 1);
    mbar_init(smem_u32(&tfree), kConv);
    mbar_init(smem_u32(&drain), 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
    *failed = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;

  if (warp == 8) {
    // ---------------------------------------------------------------- MMA issue (one thread)
    if (lane == 0) {
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kN >> 3) << 17) |
                             ((uint32_t)(kM >> 4) << 24);  // F32 accumulate, BF16 A/B, K-major, N=64, M=128
      bool ok = true;
      for (int64_t ch = 0; ch < nchunks && ok; ++ch) {
        if (ch > 0) {  // the previous chunk's fold has read the accumulators this chunk overwrites
          if (!mbar_wait(smem_u32(&tfree), (uint32_t)((ch - 1) & 1), kSpin)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;");
        }
        const int64_t s0 = ch * kChunkSteps, s1 = min(ksteps, s0 + kChunkSteps);
        for (int64_t st = s0; st < s1; ++st) {
          const int stage = (int)(st % kStages);
          if (*failed || !mbar_wait(smem_u32(&full[stage]), (uint32_t)((st / kStages) & 1), kSpin)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t a0 = sbase + (uint32_t)stage * kStage, b0 = a0 + S * kATile;
#pragma unroll
          for (int ta = 0; ta < S; ++ta)
#pragma unroll
            for (int tb = 0; tb < S - ta; ++tb)
              tc_mma(tmem + (uint32_t)((ta + tb) * kN), umma_desc(a0 + ta * kATile), umma_desc(b0 + tb * kBTile), idesc,
                     (st == s0 && ta == 0) ? 0u : 1u);
          tc_commit(smem_u32(&empty[stage]));
        }
        if (!ok) break;
        tc_commit(smem_u32(&accb));  // this chunk's accumulators are complete once its MMAs are
      }
      if (!ok) {
        *failed = 1;
        atomicExch(err, 1);
      }
      // every MMA issued has completed before the tensor memory is released
      tc_commit(smem_u32(&drain));
      if (!mbar_wait(smem_u32(&drain), 0u, kSpin)) atomicExch(err, 1);
    }
    __syncwarp();
  } else {
    // ---------------------------------------------------------------- convert, fold, store
    const int ar = tid >> 1, ah = tid & 1;  // A: row ar of the tile, k half ah of the step
    const int bj = tid >> 2, bg = tid & 3;  // B: column bj of the tile, k quarter bg of the step
    const int64_t arow = row0 + ar, bcol = col0 + bj;
    const bool a_live = arow < m, b_live = bcol < n;
    const int ea = a_live ? __ldg(exps + a_ex + arow) : 0;
    const int eb = b_live ? __ldg(exps + b_ex + bcol) : 0;
    const long long* Ab = reinterpret_cast<const long long*>(A);
    const long long* Bb = reinterpret_cast<const long long*>(B);
    const uint32_t a_dst = (uint32_t)((ar >> 3) * 256 + ah * 128 + (ar & 7) * 16);
    const uint32_t b_dst = (uint32_t)(S * kATile + (bj >> 3) * 256 + (bg >> 1) * 128 + (bj & 7) * 16 + (bg & 1) * 8);
    const int q = warp & 3, chalf = warp >> 2;  // fold: TMEM lane quarter, half of the 64 columns
    double acc[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) acc[j] = 0.0;
    bool ok = true;
    for (int64_t st = 0; st < ksteps && ok; ++st) {
      const int stage = (int)(st % kStages);
      if (st >= kStages) {  // the MMAs that read this stage's previous contents have completed
        if (*failed || !mbar_wait(smem_u32(&empty[stage]), (uint32_t)(((st / kStages) - 1) & 1), kSpin)) {
          ok = false;
          break;
        }
      }
      const int seg = st >= kseg ? 1 : 0;
      const int64_t k0 = (st - seg * kseg) * kK;
      long long au[8], bu[4];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int64_t k = k0 + 8 * ah + i;
        long long v = 0;
        if (a_live && k < K) {
          const int64_t e = a_off + arow * lda + k;
          v = __ldg(Ab + (cplx ? 2 * e + seg : e));
        }
        au[i] = v;
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int64_t k = k0 + 4 * bg + i;
        long long v = 0;
        if (b_live && k < K) {
          const int64_t e = b_off + k * ldb + bcol;
          if (cplx) {
            v = __ldg(Bb + 2 * e + (part ^ seg));
            if (part == 0 && seg == 1) v ^= (long long)0x8000000000000000ull;  // [B_r; -B_i]
          } else {
            v = __ldg(Bb + e);
          }
        }
        bu[i] = v;
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) au[i] = digit_word<S>(au[i], ea);
#pragma unroll
      for (int i = 0; i < 4; ++i) bu[i] = digit_word<S>(bu[i], eb);
      StoreDigits<S, 0>::run(smem + (size_t)stage * kStage, a_dst, b_dst, au, bu);
      fence_proxy_async();  // the digits are visible to the tensor cores' reads
      mbar_arrive(smem_u32(&full[stage]));

      if ((st + 1) % kChunkSteps == 0 || st + 1 == ksteps) {
        const int64_t ch = st / kChunkSteps;
        if (!mbar_wait(smem_u32(&accb), (uint32_t)(ch & 1), kSpin)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        // exact fold: the diagonal sums are integers below 2^24 in FP32; their weighted sum
        // sum_d q_d 2^{7(S-1-d)} is formed in two int64 halves and one 128-bit integer, then
        // rounded once to FP64 (the same rounding as the mma.sync kernel's fold)
#pragma unroll
        for (int cb = 0; cb < 4; ++cb) {
          long long hi[8], lo[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) hi[j] = lo[j] = 0;
#pragma unroll
          for (int d = 0; d < S; ++d) {
            uint32_t v[8];
            tc_ld8(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(d * kN + chalf * 32 + cb * 8), v);
            asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const long long qv = (long long)__float2int_rn(__uint_as_float(v[j]));
              if (d < 4) hi[j] += qv << (7 * (3 - d));
              else lo[j] += qv << (7 * (S - 1 - d));
            }
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const __int128 tot = (__int128)hi[j] * ((__int128)1 << (7 * (S - 4))) + (__int128)lo[j];
            const double t = i128_to_double_scaled(tot, -7 * (S - 1));
            acc[cb * 8 + j] = ch == 0 ? t : acc[cb * 8 + j] + t;
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        mbar_arrive(smem_u32(&tfree));
      }
    }
    if (!ok) {
      *failed = 1;
      atomicExch(err, 1);
    }
    conv_bar();  // all converters are past their last step: the stages are free
    if (!*failed) {
      double* tileC = reinterpret_cast<double*>(smem);
      const int r = 32 * q + lane;
#pragma unroll
      for (int j = 0; j < 32; ++j) tileC[r * (kN + 1) + chalf * 32 + j] = acc[j];
      conv_bar();
      for (int e = tid; e < kM * kN; e += kConv) {
        const int rr = e / kN, cc = e % kN;
        const int64_t gi = row0 + rr, gj = col0 + cc;
        if (gi < m && gj < n)
          C[c_off + gi * ldc + gj * ccs] =
              scale_pow2(tileC[rr * (kN + 1) + cc], __ldg(exps + a_ex + gi) + __ldg(exps + b_ex + gj) - 14);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 8) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

template <int S>
int launch_fused(const double* A, const double* B, const int* exps, double* C, const int64_t* outs,
                 const int32_t* tiles, int n_tiles, int* err, cudaStream_t s) {
  const size_t smem = (size_t)kStages * S * (kATile + kBTile);
  static_assert((size_t)kM * (kN + 1) * 8 <= (size_t)kStages * 6 * (kATile + kBTile),
                "epilogue tile must fit in the stage buffers");
  auto kern = ozaki_fused_kernel<S>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) { set_cuda_error((int)e); return YB_ERR_CUDA; }
  kern<<<n_tiles, kThreadsF, smem, s>>>(A, B, exps, C, outs, tiles, err);
  return check_launch();
}

// Per-row (axis 0) or per-column (axis 1) exponents: rec (8 int64): [0] offset (elements)
// [1] rows [2] cols [3] ld (elements) [4] 1 for complex data (a complex row counts its real
// and imaginary parts) [5] exponents offset. Axis 0: one warp per row; axis 1: 32 columns
// per CTA, its 8 warps walking down the rows (coalesced along the columns).
__global__ void ozaki_exps_kernel(const double* __restrict__ X, int* __restrict__ exps,
                                  const int64_t* __restrict__ recs, int axis) {
  const int64_t* r = recs + (int64_t)blockIdx.y * 8;
  const int64_t off = r[0], rows = r[1], cols = r[2], ld = r[3], eoff = r[5];
  const int cplx = (int)r[4];
  const long long* Xb = reinterpret_cast<const long long*>(X);
  const long long kMag = 0x7fffffffffffffffll;
  if (axis == 0) {
    const int lane = threadIdx.x & 31;
    const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= rows) return;
    const int64_t len = cplx ? 2 * cols : cols;
    const long long* p = Xb + (cplx ? 2 * (off + row * ld) : off + row * ld);
    long long mx = 0;
    for (int64_t l = lane; l < len; l += 32) mx = max(mx, __ldg(p + l) & kMag);
#pragma unroll
    for (int w = 16; w > 0; w >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, w));
    if (lane == 0) exps[eoff + row] = exponent_of(mx);
  } else {
    // 32 columns per CTA, the 8 warps walk down the rows (coalesced along the columns)
    __shared__ long long red[8][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t col = (int64_t)blockIdx.x * 32 + lane;
    if ((int64_t)blockIdx.x * 32 >= cols) return;
    long long mx = 0;
    if (col < cols)
      for (int64_t k = warp; k < rows; k += 8) {
        const int64_t e = off + k * ld + col;
        if (cplx) mx = max(mx, max(__ldg(Xb + 2 * e) & kMag, __ldg(Xb + 2 * e + 1) & kMag));
        else mx = max(mx, __ldg(Xb + e) & kMag);
      }
    red[warp][lane] = mx;
    __syncthreads();
    if (warp == 0 && col < cols) {
      for (int w = 1; w < 8; ++w) mx = max(mx, red[w][lane]);
      exps[eoff + col] = exponent_of(mx);
    }
  }
}

}  // namespace
}  // namespace yb

// Status word of the tcgen05 kernel (1 after a CTA gave up on a bounded wait).
static __device__ int g_ozaki_tc_error;

extern "C" {

int yb_ozaki_exponents(const void* x, int* exps, const int64_t* recs, int n_recs, int max_len, int axis,
                       void* stream) {
  if (n_recs == 0 || max_len == 0) return YB_OK;
  if (!x || !exps || !recs || n_recs < 0 || max_len < 0 || (axis != 0 && axis != 1)) return YB_ERR_INVALID;
  const unsigned gx = axis == 0 ? (unsigned)((max_len + 7) / 8) : (unsigned)((max_len + 31) / 32);
  yb::ozaki_exps_kernel<<<dim3(gx, (unsigned)n_recs), 256, 0, (cudaStream_t)stream>>>((const double*)x, exps, recs,
                                                                                       axis);
  return yb::check_launch();
}

int yb_ozaki_gemm_fused(const void* a, const void* b, const int* exps, double* c, const int64_t* outs,
                        const int32_t* tiles, int n_tiles, int slices_count, void* stream) {
  if (n_tiles == 0) return YB_OK;
  if (!a || !b || !exps || !c || !outs || !tiles || n_tiles < 0) return YB_ERR_INVALID;
  int* err = nullptr;
  cudaError_t e = cudaGetSymbolAddress((void**)&err, g_ozaki_tc_error);
  if (e != cudaSuccess) { yb::set_cuda_error((int)e); return YB_ERR_CUDA; }
  cudaStream_t s = (cudaStream_t)stream;
  const double* A = (const double*)a;
  const double* B = (const double*)b;
  switch (slices_count) {
    case 8: return yb::launch_fused<8>(A, B, exps, c, outs, tiles, n_tiles, err, s);
    case 7: return yb::launch_fused<7>(A, B, exps, c, outs, tiles, n_tiles, err, s);
    case 6: return yb::launch_fused<6>(A, B, exps, c, outs, tiles, n_tiles, err, s);
    default: return YB_ERR_INVALID;
  }
}

int yb_ozaki_device_error(int* out, int reset, void* stream) {
  if (!out) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyFromSymbolAsync(out, g_ozaki_tc_error, sizeof(int), 0, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && reset) {
    const int zero = 0;
    e = cudaMemcpyToSymbolAsync(g_ozaki_tc_error, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  if (e != cudaSuccess) { yb::set_cuda_error((int)e); return YB_ERR_CUDA; }
  return YB_OK;
}

}  // extern "C"
