// Family (b'), tensor-core form: FP64 sector GEMMs emulated on the tcgen05 tensor cores from
// the digit planes that yb_ozaki_split_tiled writes in the tile layout of the UMMA
// shared-memory descriptors.
//
// A persistent kernel (one CTA per SM) walks its share of the 128 x NT output tiles (NT = 64
// or 32; tiles sorted by decreasing K, or grouped by CTA by the host) with three warp roles:
//  - warp 0 (one thread) streams the S digit tiles of A (128 x 16) and of B (64 x 16) of each
//    16-long K step into a 4-stage shared-memory ring with cp.async.bulk copies completing on
//    the stage's mbarrier, refilling a stage as soon as the MMAs that read it have completed,
//    straight on into the next tile's steps;
//  - warp 1 (one thread) issues the S(S+1)/2 slice products of a step (BF16 -> FP32, M=128,
//    K=16) into the S digit-diagonal accumulators in tensor memory (S x 64 of the 512 TMEM
//    columns), up to four products per tcgen05.mma (N = 64 per B slice: slices tb..tb+3 are
//    one operand, diagonals ta+tb..ta+tb+3 adjacent accumulators; 13 MMAs per step for S = 8),
//    and frees the stage with tcgen05.commit; with NT = 32 the S x 32 accumulator columns of
//    a chunk fit twice in the 512 columns, and consecutive chunks alternate between the two
//    buffers, so the MMAs of the next chunk (and tile) need not wait for this chunk's fold;
//  - 16 fold warps (4 per TMEM lane quarter, NT/4 columns each) read the accumulators back at
//    the end of every 400-long K chunk (exact FP32 integer sums), combine the diagonals exactly
//    into a 128-bit integer on the integer pipe, round it once to FP64 into the tile's FP64
//    accumulators (bit-identical to the mma.sync kernel's fold), release the tensor memory to
//    the next chunk's MMAs and, after a tile's last chunk, write the tile from registers while
//    the next tile's MMAs run. Warps whose rows or columns lie wholly outside the sector (the
//    padding of small sectors) skip their reads and folds.
// Every wait is bounded; a CTA that gives up records the status word of yb_ozaki_device_error,
// waits (bounded) for its copies and MMAs, frees its tensor memory and stops writing.
#include <type_traits>
#include "yb_ozaki_common.cuh"

namespace yb {
namespace {
using namespace oz;

constexpr int kM = 128, kK = 16, kStages = 4;
constexpr int kFoldWarps = 16;              // 4 per TMEM lane quarter
constexpr int kFold = 32 * kFoldWarps;      // fold / epilogue threads (warps 2-17)
constexpr int kThreadsT = 64 + kFold;       // producer warp, MMA warp, fold warps
constexpr int kChunkSteps = 25;             // 400-long K chunks: exact FP32 diagonal sums
constexpr long long kSpin = 1ll << 24;
constexpr uint32_t kATile = kM * kK * 2;  // one slice's 128 x 16 digit tile, bytes

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}

// out record (16 int64): [0] c offset [1] m [2] n [3] ldc [4] A slices offset (tile layout)
// [5] A exponents offset [6] B slices offset (tile layout) [7] B exponents offset [8] K [9] Kp
// [10] output column stride (2: one part of complex data)
// NT: output tile width (64, or 32: then the S diagonal accumulators of a chunk take S x 32 of
// the 512 TMEM columns and two chunks alternate between two buffers, so that the fold of one
// tile overlaps the MMAs of the next).
template <int S, int NT>
__global__ void __launch_bounds__(kThreadsT, 1)
    ozaki_gemm_tc_kernel(const __nv_bfloat16* __restrict__ As, const int* __restrict__ Ae,
                         const __nv_bfloat16* __restrict__ Bs, const int* __restrict__ Be, double* __restrict__ C,
                         const int64_t* __restrict__ outs, const int32_t* __restrict__ tiles, int n_tiles,
                         const int32_t* __restrict__ cta_tiles, int* __restrict__ err) {
  constexpr int kN = NT;
  constexpr uint32_t kBTile = kN * kK * 2;          // one slice's NT x 16 digit tile, bytes
  constexpr int kFoldCols = kN / (kFoldWarps / 4);  // columns per fold warp (16 or 8)
  constexpr int kBufCols = S * kN;                  // TMEM columns of one chunk's accumulators
  constexpr int kBufs = 2 * kBufCols <= 512 ? 2 : 1;
  constexpr uint32_t kStage = S * (kATile + kBTile);
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint32_t tmem_slot;
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], accb[2], tfree[2], drain;
  __shared__ int failed_s;
  volatile int* failed = &failed_s;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t sbase = smem_u32(smem);
  // this CTA's tiles: [t0, t1) of a schedule grouped by CTA, or every gridDim.x-th tile
  const bool sched = cta_tiles != nullptr;
  const int t0 = sched ? cta_tiles[blockIdx.x] : (int)blockIdx.x;
  const int t1 = sched ? cta_tiles[blockIdx.x + 1] : n_tiles;
  const int dt = sched ? 1 : (int)gridDim.x;

  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int i = 0; i < kStages; ++i) {
      mbar_init(smem_u32(&full[i]), 1);
      mbar_init(smem_u32(&empty[i]), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(smem_u32(&accb[i]), 1);
      mbar_init(smem_u32(&tfree[i]), kFold);
    }
    mbar_init(smem_u32(&drain), 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
    *failed = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    // ---------------------------------------------------------------- producer
    if (lane == 0) {
      int64_t gs = 0;  // K steps issued by this CTA (all its tiles): the ring position
      bool ok = true;
      for (int t = t0; t < t1 && ok; t += dt) {
        const int4 tl = reinterpret_cast<const int4*>(tiles)[t];
        const int64_t* o = outs + (int64_t)tl.x * 16;
        const int64_t m = o[1], n = o[2], a_sl = o[4], b_sl = o[6], Kp = o[9];
        const int64_t ksteps = Kp / kK;
        // digit planes in tile layout: per slice, (row tile, K step) blocks of 128 x 16 (A) / 64 x 16 (B)
        const int64_t a_slice = (m + kM - 1) / kM * kM * Kp, b_slice = (n + kN - 1) / kN * kN * Kp;
        const __nv_bfloat16* a_tiles = As + a_sl + (int64_t)tl.y * ksteps * (kM * kK);
        const __nv_bfloat16* b_tiles = Bs + b_sl + (int64_t)tl.z * ksteps * (kN * kK);
        for (int64_t st = 0; st < ksteps; ++st, ++gs) {
          const int stage = (int)(gs % kStages);
          if (gs >= kStages) {  // the MMAs that read this stage's previous contents have completed
            if (*failed || !mbar_wait(smem_u32(&empty[stage]), (uint32_t)(((gs / kStages) - 1) & 1), kSpin)) {
              *failed = 1;
              atomicExch(err, 1);
              ok = false;
              break;
            }
          }
          const uint32_t fb = smem_u32(&full[stage]);
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(kStage) : "memory");
          const uint32_t d0 = sbase + (uint32_t)stage * kStage;
          for (int s = 0; s < S; ++s) {
            bulk_load(d0 + s * kATile, a_tiles + s * a_slice + st * (kM * kK), kATile, fb);
            bulk_load(d0 + S * kATile + s * kBTile, b_tiles + s * b_slice + st * (kN * kK), kBTile, fb);
          }
        }
      }
      // no copy may still be landing in shared memory when the CTA exits: the last issued
      // step of each stage is that stage's latest phase
      for (int64_t j = max((int64_t)0, gs - kStages); j < gs; ++j)
        if (!mbar_wait(smem_u32(&full[j % kStages]), (uint32_t)((j / kStages) & 1), kSpin)) atomicExch(err, 1);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------------------------------------------------------- MMA issue
    if (lane == 0) {
      // F32 accumulate, BF16 A/B, K-major, M=128; N = 64 x (slices in one MMA) is set per MMA
      const uint32_t idesc0 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kM >> 4) << 24);
      bool ok = true;
      int64_t gs = 0, gch = 0;  // steps and chunks of this CTA
      for (int t = t0; t < t1 && ok; t += dt) {
        const int4 tl = reinterpret_cast<const int4*>(tiles)[t];
        const int64_t ksteps = outs[(int64_t)tl.x * 16 + 9] / kK;
        const int64_t nchunks = (ksteps + kChunkSteps - 1) / kChunkSteps;
        for (int64_t ch = 0; ch < nchunks && ok; ++ch, ++gch) {
          const int buf = (int)(gch % kBufs);
          const int64_t use = gch / kBufs;  // earlier chunks in this buffer
          const uint32_t acc_base = tmem + (uint32_t)(buf * kBufCols);
          if (use > 0) {  // the fold of this buffer's previous chunk has read the accumulators
            if (*failed || !mbar_wait(smem_u32(&tfree[buf]), (uint32_t)((use - 1) & 1), kSpin)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;");
          }
          const int64_t s1 = min(ksteps, (ch + 1) * kChunkSteps);
          for (int64_t st = ch * kChunkSteps; st < s1; ++st, ++gs) {
            const int stage = (int)(gs % kStages);
            if (*failed || !mbar_wait(smem_u32(&full[stage]), (uint32_t)((gs / kStages) & 1), kSpin)) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t a0 = sbase + (uint32_t)stage * kStage, b0 = a0 + S * kATile;
            const bool first = st == ch * kChunkSteps;
            // A_ta times up to four B slices at once: the B slices lie one after the other in
            // the stage (64 rows each, the same core-matrix strides), so B_tb..B_tb+k-1 is one
            // operand of N = 64k rows, and the diagonals ta+tb..ta+tb+k-1 are adjacent 64-column
            // accumulators: one MMA of N = 64k does the k slice products
#pragma unroll
            for (int ta = 0; ta < S; ++ta)
#pragma unroll
              for (int tb = 0; tb < S - ta; tb += 4) {
                const int k = (S - ta - tb) < 4 ? (S - ta - tb) : 4;
                tc_mma(acc_base + (uint32_t)((ta + tb) * kN), umma_desc(a0 + ta * kATile), umma_desc(b0 + tb * kBTile),
                       idesc0 | ((uint32_t)((kN * k) >> 3) << 17), (first && ta == 0) ? 0u : 1u);
              }
            tc_commit(smem_u32(&empty[stage]));
          }
          if (!ok) break;
          tc_commit(smem_u32(&accb[buf]));  // this chunk's accumulators are complete once its MMAs are
        }
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
    // ---------------------------------------------------------------- fold and store
    const int q = warp & 3;             // TMEM lane quarter of this warp
    const int cg = (warp - 2) >> 2;     // its 16-column group
    const int r = 32 * q + lane;        // tile row of this thread
    int64_t gch = 0;
    bool ok = true;
    for (int t = t0; t < t1 && ok; t += dt) {
      const int4 tl = reinterpret_cast<const int4*>(tiles)[t];
      const int64_t* o = outs + (int64_t)tl.x * 16;
      const int64_t c_off = o[0], m = o[1], n = o[2], ldc = o[3], a_ex = o[5], b_ex = o[7], Kp = o[9];
      const int64_t ccs = o[10] > 0 ? o[10] : 1;
      const int64_t row0 = (int64_t)tl.y * kM, col0 = (int64_t)tl.z * kN + kFoldCols * cg;
      const int64_t nchunks = (Kp / kK + kChunkSteps - 1) / kChunkSteps;
      // warps wholly in the padding of a small sector skip the reads and the fold
      const bool busy = (row0 + 32 * q < m) && (col0 < n);
      double acc[kFoldCols];
      for (int64_t ch = 0; ch < nchunks; ++ch, ++gch) {
        const int buf = (int)(gch % kBufs);
        const uint32_t acc_base = tmem + (uint32_t)(buf * kBufCols);
        if (*failed || !mbar_wait(smem_u32(&accb[buf]), (uint32_t)((gch / kBufs) & 1), kSpin)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        // exact fold: the diagonal sums are integers below 2^24 in FP32; their weighted sum
        // sum_d q_d 2^{7(S-1-d)} = hi 2^{7(S-4)} + lo is formed in two int64 halves and
        // rounded once to FP64 (the same rounding as the mma.sync kernel's fold). The S
        // diagonals of 4 columns are read with one wait. The first chunk is assigned, later
        // ones added (two copies of the loop, so that the first issues no FP64 add).
        auto fold = [&](auto first_tag) {
          constexpr bool kFirst = decltype(first_tag)::value;
#pragma unroll
          for (int cb = 0; cb < kFoldCols / 4; ++cb) {
            uint32_t v[S][4];
#pragma unroll
            for (int d = 0; d < S; ++d)
              tc_ld4(acc_base + ((uint32_t)(32 * q) << 16) + (uint32_t)(d * kN + kFoldCols * cg + cb * 4), v[d]);
            asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              int qi[S];
#pragma unroll
              for (int d = 0; d < S; ++d) qi[d] = __float2int_rn(__uint_as_float(v[d][j]));
              long long hi, lo;
              fold_halves<S>(qi, hi, lo);
              const double x = fold_round(hi, lo, 7 * (S - 4), -7 * (S - 1));
              if (kFirst) acc[cb * 4 + j] = x;
              else acc[cb * 4 + j] += x;
            }
          }
        };
        if (busy) {
          if (ch == 0) fold(std::true_type{});
          else fold(std::false_type{});
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        mbar_arrive(smem_u32(&tfree[buf]));
      }
      if (!ok) break;
      // the tile, straight from registers (the next tile's MMAs proceed meanwhile)
      const int64_t gi = row0 + r;
      if (busy && gi < m) {
        const int ea = Ae[a_ex + gi] - 14;
        double* crow = C + c_off + gi * ldc;
#pragma unroll
        for (int j = 0; j < kFoldCols; ++j) {
          const int64_t gj = col0 + j;
          if (gj < n) crow[gj * ccs] = scale_pow2(acc[j], ea + Be[b_ex + gj]);
        }
      }
    }
    if (!ok) {
      *failed = 1;
      atomicExch(err, 1);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

int sm_count() {
  static int sms[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  if (sms[dev] == 0) cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
  return sms[dev];
}

template <int S, int NT>
int launch_gemm_tc(const void* As, const int* Ae, const void* Bs, const int* Be, double* C, const int64_t* outs,
                   const int32_t* tiles, int n_tiles, const int32_t* cta_tiles, int n_ctas, int* err,
                   cudaStream_t s) {
  const size_t smem = (size_t)kStages * S * (kATile + (uint32_t)(NT * kK * 2));
  auto kern = ozaki_gemm_tc_kernel<S, NT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) { set_cuda_error((int)e); return YB_ERR_CUDA; }
  const int sms = sm_count();
  if (sms <= 0) return YB_ERR_CUDA;
  // one CTA per SM (its shared memory and all 512 TMEM columns): a schedule may not ask for more
  if (cta_tiles && (n_ctas < 1 || n_ctas > sms)) return YB_ERR_INVALID;
  const int grid = cta_tiles ? n_ctas : (n_tiles < sms ? n_tiles : sms);
  kern<<<grid, kThreadsT, smem, s>>>((const __nv_bfloat16*)As, Ae, (const __nv_bfloat16*)Bs, Be, C, outs, tiles,
                                     n_tiles, cta_tiles, err);
  return check_launch();
}

}  // namespace
}  // namespace yb

// Status word of the tcgen05 kernel (1 after a CTA gave up on a bounded wait).
static __device__ int g_ozaki_tc_error;

extern "C" {

int yb_ozaki_gemm_tc(const void* a_slices, const int* a_exps, const void* b_slices, const int* b_exps, double* c,
                     const int64_t* outs, const int32_t* tiles, int n_tiles, const int32_t* cta_tiles, int n_ctas,
                     int tile_n, int slices_count, void* stream) {
  if (n_tiles == 0) return YB_OK;
  if (!a_slices || !a_exps || !b_slices || !b_exps || !c || !outs || !tiles || n_tiles < 0) return YB_ERR_INVALID;
  if (tile_n != 64 && tile_n != 32) return YB_ERR_INVALID;
  int* err = nullptr;
  cudaError_t e = cudaGetSymbolAddress((void**)&err, g_ozaki_tc_error);
  if (e != cudaSuccess) { yb::set_cuda_error((int)e); return YB_ERR_CUDA; }
  cudaStream_t s = (cudaStream_t)stream;
#define YB_TC_LAUNCH(SS, NN) \
  return yb::launch_gemm_tc<SS, NN>(a_slices, a_exps, b_slices, b_exps, c, outs, tiles, n_tiles, cta_tiles, n_ctas, err, s)
  switch (slices_count * 100 + tile_n) {
    case 864: YB_TC_LAUNCH(8, 64);
    case 832: YB_TC_LAUNCH(8, 32);
    case 764: YB_TC_LAUNCH(7, 64);
    case 732: YB_TC_LAUNCH(7, 32);
    case 664: YB_TC_LAUNCH(6, 64);
    case 632: YB_TC_LAUNCH(6, 32);
    default: return YB_ERR_INVALID;
  }
#undef YB_TC_LAUNCH
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
