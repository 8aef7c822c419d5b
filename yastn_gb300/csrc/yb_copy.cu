// Family (a): one-launch strided block copies (merge / unmerge / their adjoints).
//
// The host compiles YASTN's merge metadata (meta_new/meta_mrg of transpose_and_merge,
// the unmerge records) into copy tasks: each task is an n-dim strided copy whose
// extents are the transposed source block and whose source/destination strides map
// the permutation, the reshape to the fused block and its sub-slice offset. Dims that
// are contiguous in both source and destination are collapsed on the host, and pairs
// of FP64 elements are moved as one 16-byte unit when every offset and stride allows.
//
// Work is split into items of up to YB_COPY_ITEM_UNITS units of one task; one CTA
// handles one item. Within an item consecutive threads take consecutive units of the
// innermost dim (destination-contiguous after collapsing), so stores are coalesced.
// Tasks that transpose (source contiguous along another dim) are tiled instead.
#include <type_traits>
#include "yb_common.cuh"

namespace yb {

static thread_local int g_last_cuda_error = 0;
void set_cuda_error(int code) { g_last_cuda_error = code; }

namespace {

constexpr int kThreads = 256;
constexpr int kIlp = 4;

// Kind-0 tasks with ND <= 4 dims: the task's extents, strides and division constants are read
// into registers once per item; every unit then costs ND - 1 fast divisions (the outermost
// coordinate is what remains) and two index updates per dim.
template <typename Unit, int ND>
__device__ __forceinline__ void copy_units(const Unit* __restrict__ src, Unit* __restrict__ dst, const int64_t* rec,
                                           int64_t first) {
  uint32_t size[ND], magic[ND], shift[ND];
  int64_t sstr[ND], dstr[ND];
#pragma unroll
  for (int d = 0; d < ND; ++d) {
    size[d] = (uint32_t)rec[YB_CP_SIZE + d];
    magic[d] = (uint32_t)rec[YB_CP_MAGIC + d];
    shift[d] = (uint32_t)rec[YB_CP_SHIFT + d];
    sstr[d] = rec[YB_CP_SSTR + d];
    dstr[d] = rec[YB_CP_DSTR + d];
  }
  const int64_t count = rec[YB_CP_COUNT];
  const int64_t n = min((int64_t)YB_COPY_ITEM_UNITS, count - first);
  const int64_t sbase = rec[YB_CP_SRC];
  const int64_t dbase = rec[YB_CP_DST];
  for (int64_t e0 = threadIdx.x; e0 < n; e0 += (int64_t)kThreads * kIlp) {
    Unit v[kIlp];
    int64_t doff[kIlp];
#pragma unroll
    for (int j = 0; j < kIlp; ++j) {
      const int64_t e = e0 + (int64_t)j * kThreads;
      doff[j] = -1;
      if (e < n) {
        uint32_t idx = (uint32_t)(first + e);
        int64_t so = sbase, dof = dbase;
#pragma unroll
        for (int d = ND - 1; d >= 1; --d) {
          const uint32_t q = fast_div(idx, magic[d], shift[d]);
          const int64_t r = (int64_t)(idx - q * size[d]);
          so += r * sstr[d];
          dof += r * dstr[d];
          idx = q;
        }
        so += (int64_t)idx * sstr[0];
        dof += (int64_t)idx * dstr[0];
        v[j] = __ldg(src + so);
        doff[j] = dof;
      }
    }
#pragma unroll
    for (int j = 0; j < kIlp; ++j)
      if (doff[j] >= 0) dst[doff[j]] = v[j];
  }
}

// Tasks with more than 4 dims (rare: the host collapses every dim contiguous on both sides).
template <typename Unit>
__device__ __forceinline__ void copy_units_generic(const Unit* __restrict__ src, Unit* __restrict__ dst,
                                                   const int64_t* rec, int64_t first) {
  const int ndim = (int)rec[YB_CP_NDIM];
  const int64_t n = min((int64_t)YB_COPY_ITEM_UNITS, rec[YB_CP_COUNT] - first);
  for (int64_t e = threadIdx.x; e < n; e += kThreads) {
    uint32_t idx = (uint32_t)(first + e);
    int64_t so = rec[YB_CP_SRC], dof = rec[YB_CP_DST];
    for (int d = ndim - 1; d >= 0; --d) {
      const uint32_t size = (uint32_t)rec[YB_CP_SIZE + d];
      const uint32_t q = fast_div(idx, (uint32_t)rec[YB_CP_MAGIC + d], (uint32_t)rec[YB_CP_SHIFT + d]);
      const int64_t r = (int64_t)(idx - q * size);
      so += r * rec[YB_CP_SSTR + d];
      dof += r * rec[YB_CP_DSTR + d];
      idx = q;
    }
    dst[dof] = __ldg(src + so);
  }
}

template <typename Unit>
__device__ __forceinline__ void copy_units_any(const Unit* __restrict__ src, Unit* __restrict__ dst, const int64_t* rec,
                                               int64_t first) {
  switch ((int)rec[YB_CP_NDIM]) {
    case 1: copy_units<Unit, 1>(src, dst, rec, first); break;
    case 2: copy_units<Unit, 2>(src, dst, rec, first); break;
    case 3: copy_units<Unit, 3>(src, dst, rec, first); break;
    case 4: copy_units<Unit, 4>(src, dst, rec, first); break;
    default: copy_units_generic<Unit>(src, dst, rec, first); break;
  }
}

// Kind-1 tasks: tiles of YB_COPY_TILE x YB_COPY_TILE elements staged in shared memory.
// The tile index is decomposed over the record's dims like a unit index; the remainders
// of the last two dims are the tile's y and x positions. Each warp reads tile rows along
// y (source-contiguous) and, after the barrier, writes tile rows along x
// (destination-contiguous), so both sides are coalesced.
template <typename Elem>
__device__ __forceinline__ void copy_tiles(const Elem* __restrict__ src, Elem* __restrict__ dst, const int64_t* rec,
                                           int64_t first, Elem (*tile)[YB_COPY_TILE + 1]) {
  constexpr int T = YB_COPY_TILE;
  const int ndim = (int)rec[YB_CP_NDIM];
  const int64_t count = rec[YB_CP_COUNT];
  const int64_t nx = rec[YB_CP_NX], ny = rec[YB_CP_NY];
  const int64_t ss_x = rec[YB_CP_SSTR + ndim - 1] / T, ds_y = rec[YB_CP_DSTR + ndim - 2] / T;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = kThreads >> 5;
  const int64_t last = min(count, first + (int64_t)YB_COPY_ITEM_TILES);
  for (int64_t t = first; t < last; ++t) {
    uint32_t idx = (uint32_t)t;
    int64_t so = rec[YB_CP_SRC], dof = rec[YB_CP_DST], tx = 0, ty = 0;
#pragma unroll
    for (int d = YB_CP_MAXD - 1; d >= 0; --d) {
      if (d < ndim) {
        const uint32_t size = (uint32_t)rec[YB_CP_SIZE + d];
        const uint32_t q = fast_div(idx, (uint32_t)rec[YB_CP_MAGIC + d], (uint32_t)rec[YB_CP_SHIFT + d]);
        const int64_t r = (int64_t)(idx - q * size);
        so += r * rec[YB_CP_SSTR + d];
        dof += r * rec[YB_CP_DSTR + d];
        if (d == ndim - 1) tx = r;
        if (d == ndim - 2) ty = r;
        idx = q;
      }
    }
    const int ex = (int)min((int64_t)T, nx - tx * T), ey = (int)min((int64_t)T, ny - ty * T);
    __syncthreads();  // the previous tile has been written out
    for (int xi = warp; xi < ex; xi += nwarps)
      if (lane < ey) tile[xi][lane] = __ldg(src + so + xi * ss_x + lane);
    __syncthreads();
    for (int yi = warp; yi < ey; yi += nwarps)
      if (lane < ex) dst[dof + yi * ds_y + lane] = tile[lane][yi];
  }
}

// Elem is the element type of the data (double for FP64, double2 for complex128). FP64
// tasks flagged YB_CP_VEC move pairs of elements as one 16-byte unit.
template <typename Elem>
__global__ void __launch_bounds__(kThreads) block_copy_kernel(const Elem* __restrict__ src, Elem* __restrict__ dst,
                                                               const int64_t* __restrict__ tasks,
                                                               const int64_t* __restrict__ items) {
  __shared__ int64_t rec[YB_COPY_REC];
  __shared__ Elem tile[YB_COPY_TILE][YB_COPY_TILE + 1];
  const int64_t* item = items + 2 * (int64_t)blockIdx.x;
  const int64_t task = item[0];
  const int64_t first = item[1];
  if (threadIdx.x < YB_COPY_REC) rec[threadIdx.x] = tasks[task * YB_COPY_REC + threadIdx.x];
  __syncthreads();
  if (rec[YB_CP_KIND] == 1)
    copy_tiles<Elem>(src, dst, rec, first, tile);
  else if (std::is_same<Elem, double>::value && rec[YB_CP_VEC] != 0)
    copy_units_any<double2>(reinterpret_cast<const double2*>(src), reinterpret_cast<double2*>(dst), rec, first);
  else
    copy_units_any<Elem>(src, dst, rec, first);
}


// Composed copies: dst[i] = src[|map[i]| - 1], negated where map[i] < 0 and conjugated when
// `conj` is set, zero where map[i] == 0. The map (int32, one entry per destination element) is
// the composition of a chain of merges, unmerges, transposes and block negations, so one pass
// replaces the chain. Map reads and stores are coalesced; the loads follow the map (runs of the
// source's innermost dims; a transposed run reuses its sectors from L2). Negation and
// conjugation flip IEEE sign bits, as -x and conj(x) do. Words = 8-byte words per element
// (1: float64, 2: complex128).
template <int Words>
__global__ void __launch_bounds__(kThreads) map_gather_kernel(const uint64_t* __restrict__ src,
                                                               uint64_t* __restrict__ dst,
                                                               const int32_t* __restrict__ map, int64_t n,
                                                               uint64_t conj_hi) {
  constexpr uint64_t kSign = 0x8000000000000000ull;
  const int64_t base = (int64_t)blockIdx.x * (kThreads * kIlp) + threadIdx.x;
  int32_t m[kIlp];
#pragma unroll
  for (int j = 0; j < kIlp; ++j) {
    const int64_t e = base + (int64_t)j * kThreads;
    m[j] = e < n ? __ldg(map + e) : 0;
  }
  uint64_t v[kIlp][Words];
#pragma unroll
  for (int j = 0; j < kIlp; ++j) {
    const int32_t a = m[j] < 0 ? -m[j] : m[j];
    const uint64_t neg = m[j] < 0 ? kSign : 0ull;
    if (Words == 2) {
      ulonglong2 w = make_ulonglong2(0ull, 0ull);
      if (a != 0) w = __ldg(reinterpret_cast<const ulonglong2*>(src) + (a - 1));
      v[j][0] = a != 0 ? (w.x ^ neg) : 0ull;
      v[j][Words - 1] = a != 0 ? (w.y ^ neg ^ conj_hi) : 0ull;
    } else {
      v[j][0] = a != 0 ? (__ldg(src + (a - 1)) ^ neg) : 0ull;
    }
  }
#pragma unroll
  for (int j = 0; j < kIlp; ++j) {
    const int64_t e = base + (int64_t)j * kThreads;
    if (e < n) {
      if (Words == 2)
        reinterpret_cast<ulonglong2*>(dst)[e] = make_ulonglong2(v[j][0], v[j][Words - 1]);
      else
        dst[e] = v[j][0];
    }
  }
}

}  // namespace
}  // namespace yb

extern "C" {

int yb_abi_version(void) { return 100; }
int yb_last_cuda_error(void) { return yb::g_last_cuda_error; }

int yb_block_copy(const void* src, void* dst, int unit_bytes, const int64_t* tasks, int n_tasks,
                  const int64_t* items, int n_items, void* stream) {
  if (n_items == 0) return YB_OK;
  if (!src || !dst || !tasks || !items || n_tasks <= 0 || n_items < 0) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  dim3 grid((unsigned)n_items);
  // the copy moves elements as raw units: 8 bytes (float64, complex64), 16 (complex128), and
  // 1, 2, 4 for the other dtypes a tensor may hold (bool masks, float32, ...)
  switch (unit_bytes) {
    case 8: yb::block_copy_kernel<double><<<grid, yb::kThreads, 0, s>>>((const double*)src, (double*)dst, tasks, items); break;
    case 16:
      yb::block_copy_kernel<double2><<<grid, yb::kThreads, 0, s>>>((const double2*)src, (double2*)dst, tasks, items);
      break;
    case 4:
      yb::block_copy_kernel<uint32_t><<<grid, yb::kThreads, 0, s>>>((const uint32_t*)src, (uint32_t*)dst, tasks, items);
      break;
    case 2:
      yb::block_copy_kernel<uint16_t><<<grid, yb::kThreads, 0, s>>>((const uint16_t*)src, (uint16_t*)dst, tasks, items);
      break;
    case 1:
      yb::block_copy_kernel<uint8_t><<<grid, yb::kThreads, 0, s>>>((const uint8_t*)src, (uint8_t*)dst, tasks, items);
      break;
    default: return YB_ERR_INVALID;
  }
  return yb::check_launch();
}


int yb_map_gather(const void* src, void* dst, int dtype, const int32_t* map, int64_t n, int conj, void* stream) {
  if (n == 0) return YB_OK;
  if (!src || !dst || !map || n < 0 || n >= ((int64_t)1 << 40)) return YB_ERR_INVALID;
  if (dtype != YB_F64 && dtype != YB_C128) return YB_ERR_INVALID;
  if (dtype == YB_C128 && ((((uintptr_t)src) | ((uintptr_t)dst)) & 15u)) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t per_cta = (int64_t)yb::kThreads * yb::kIlp;
  const dim3 grid((unsigned)((n + per_cta - 1) / per_cta));
  if (dtype == YB_C128)
    yb::map_gather_kernel<2><<<grid, yb::kThreads, 0, s>>>((const uint64_t*)src, (uint64_t*)dst, map, n,
                                                           conj ? 0x8000000000000000ull : 0ull);
  else
    yb::map_gather_kernel<1><<<grid, yb::kThreads, 0, s>>>((const uint64_t*)src, (uint64_t*)dst, map, n, 0ull);
  return yb::check_launch();
}

}  // extern "C"
