// Helpers shared by the split-operand (Ozaki) emulated GEMM kernels: the scaled rounding of
// the integer digit split, exact integer-built conversions, and the tcgen05 / mbarrier
// primitives of the tensor-core kernel.
#pragma once
#include <cuda_bf16.h>
#include "yb_common.cuh"

namespace yb {
namespace oz {

// Q = rint(a 2^{7s-e}) (|Q| < 2^{7s}) from a's mantissa and exponent bits, by a shift with
// round-half-to-even (a = the double with bit pattern ``bits``; |a| < 2^e), without branches:
// elements near the row maximum (left shift, up to 3 bits for s = 8) and smaller ones (right
// shift with rounding) take the same instructions.
__host__ __device__ __forceinline__ long long scaled_rint(long long bits, int e, int s) {
  const unsigned long long mag = (unsigned long long)bits & 0x7fffffffffffffffull;
  const int E = (int)(mag >> 52);
  const unsigned long long M = (mag & 0xfffffffffffffull) | (E ? (1ull << 52) : 0ull);
  const int up = (E ? E - 1075 : -1074) + 7 * s - e;  // Q = rint(M 2^up)
  const int shl = up > 0 ? up : 0;
  const int shr = up < 0 ? (-up < 63 ? -up : 63) : 0;
  unsigned long long q = (M << shl) >> shr;
  const unsigned long long rem = M & ((1ull << shr) - 1ull);
  const unsigned long long half = (1ull << shr) >> 1;
  q += (unsigned long long)((rem > half) | ((rem == half) & (shr != 0) & ((q & 1ull) != 0)));
  return bits < 0 ? -(long long)q : (long long)q;
}

// x 2^E by an exponent-field add when x and the result are normal doubles.
__device__ __forceinline__ double scale_pow2(double x, int E) {
  const long long b = __double_as_longlong(x);
  const int be = (int)((b >> 52) & 0x7ff);
  if (be == 0 || be == 0x7ff || be + E < 1 || be + E > 2046) return scalbn(x, E);
  return __longlong_as_double(b + ((long long)E << 52));
}

// Correctly rounded (to nearest, ties to even) double of W 2^E for W = hi 2^L + lo, the exact
// value of a folded tile element (|hi|, |lo| < 2^46, 6 <= L <= 40), without branches so that
// the compiler can interleave the conversions of several elements; the integer pipe only.
// W = H 2^L + r with 0 <= r < 2^L is brought to sign and magnitude Hm 2^L + rm, whose leading
// bit p gives the shift to 53 bits; every result lies in the normal range for the exponents
// of the fold (1023 + p + E in [1, 2046]).
__host__ __device__ __forceinline__ int clz64(unsigned long long x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

__host__ __device__ __forceinline__ double fold_round(long long hi, long long lo, int L, int E) {
  const unsigned long long mask = (1ull << L) - 1ull;
  const long long H = hi + (lo >> L);                  // arithmetic shift: floor(lo / 2^L)
  const unsigned long long r = (unsigned long long)lo & mask;
  const bool neg = H < 0;
  const unsigned long long Hm = neg ? (unsigned long long)(-H) - (r != 0 ? 1ull : 0ull) : (unsigned long long)H;
  const unsigned long long rm = neg ? (0ull - r) & mask : r;
  const int pH = 63 - clz64(Hm), pr = 63 - clz64(rm);  // -1 for zero
  const int p = Hm ? pH + L : pr;                       // leading bit of Hm 2^L + rm (-1: zero)
  const int sh = p > 52 ? p - 52 : 0;                   // bits below the 53 kept (sh < L)
  unsigned long long V = (Hm << (L - sh)) | (rm >> sh);
  const unsigned long long rem = rm & ((1ull << sh) - 1ull);
  const unsigned long long half = sh ? (1ull << (sh - 1)) : 0ull;
  const unsigned long long up = (rem > half) | ((rem == half) & (V & 1ull) & (sh != 0 ? 1ull : 0ull));
  V += up;
  const int carry = (int)(V >> 53);                     // rounded up to 2^53
  V >>= carry;
  const int lead = p > 52 ? 52 : p;                     // leading bit of V before the rounding
  const unsigned long long frac = (lead >= 0 ? (V << (52 - lead)) : 0ull) & 0xfffffffffffffull;
  const unsigned long long bits = (neg ? 0x8000000000000000ull : 0ull) |
                                  ((unsigned long long)(1023 + p + carry + E) << 52) | frac;
  union {
    unsigned long long u;
    double d;
  } cv;
  cv.u = bits;
  return p < 0 ? 0.0 : cv.d;
}

// The two int64 halves of a fold from the S exact diagonal sums q_d (|q_d| <= 400 * 10 * 2^12,
// chunks of at most 400): hi = sum_{d<4} q_d 2^{7(3-d)}, lo = sum_{d>=4} q_d 2^{7(S-1-d)}.
// The last two terms of each half are combined in 32 bits (|128 q + q'| < 2^31 by that bound)
// and the rest with 32 x 32 -> 64-bit multiply-adds.
template <int S>
__device__ __forceinline__ void fold_halves(const int* q, long long& hi, long long& lo) {
  hi = (long long)q[0] * (1ll << 21) + (long long)q[1] * (1ll << 14) + (long long)(q[2] * 128 + q[3]);
  long long l = (long long)(q[S - 2] * 128 + q[S - 1]);
#pragma unroll
  for (int d = 4; d < S - 2; ++d) l += (long long)q[d] * (1ll << (7 * (S - 1 - d)));
  lo = l;
}

// ------------------------------------------------------------------ tcgen05 / mbarrier
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: canonical K-major, no swizzle, LBO = 128 B (between the two
// 8-element core matrices of a 16-long K step), SBO = 256 B (between 8-row groups)
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
         ((uint64_t)1 << 46);
}

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on an mbarrier phase: false after ``limit`` polls.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, long long limit) {
  for (long long it = 0; it < limit; ++it)
    if (mbar_try(mbar, parity)) return true;
  return false;
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar));
}

__device__ __forceinline__ void tc_ld4(uint32_t taddr, uint32_t* r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
}

__device__ __forceinline__ void tc_ld8(uint32_t taddr, uint32_t* r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}

}  // namespace oz
}  // namespace yb
