// Helpers shared by the split-operand (Ozaki) emulated GEMM kernels: the scaled rounding of
// the integer digit split, exact integer-built conversions, and the tcgen05 / mbarrier
// primitives of the tensor-core kernel.
#pragma once
#include <cuda_bf16.h>
#include "yb_common.cuh"

namespace yb {
namespace oz {

// Q = rint(a 2^{7s-e}) (|Q| < 2^{7s}) from a's mantissa and exponent bits, by a shift with
// round-half-to-even (a = the double with bit pattern ``bits``; |a| < 2^e).
__device__ __forceinline__ long long scaled_rint(long long bits, int e, int s) {
  const long long mag = bits & 0x7fffffffffffffffll;
  if (mag == 0) return 0;
  const int E = (int)(mag >> 52);
  long long M = mag & 0xfffffffffffffll;
  int ex = -1074;  // a = M 2^ex
  if (E != 0) {
    M |= 1ll << 52;
    ex = E - 1075;
  }
  const int up = ex + 7 * s - e;  // Q = rint(M 2^up)
  long long q;
  if (up >= 0) {
    q = M << up;  // |Q| < 2^{7s}: up <= 7s - 53
  } else {
    const int sh = min(-up, 63);
    q = M >> sh;
    const unsigned long long rem = (unsigned long long)M & ((1ull << sh) - 1ull);
    const unsigned long long half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (q & 1))) ++q;
  }
  return bits < 0 ? -q : q;
}

// x 2^E by an exponent-field add when x and the result are normal doubles.
__device__ __forceinline__ double scale_pow2(double x, int E) {
  const long long b = __double_as_longlong(x);
  const int be = (int)((b >> 52) & 0x7ff);
  if (be == 0 || be == 0x7ff || be + E < 1 || be + E > 2046) return scalbn(x, E);
  return __longlong_as_double(b + ((long long)E << 52));
}

// Correctly rounded (to nearest, ties to even) double of the integer v times 2^E, on the
// integer pipe; results outside the normal range go through scalbn.
__device__ __forceinline__ double i128_to_double_scaled(__int128 v, int E) {
  if (v == 0) return 0.0;
  const unsigned long long sgn = v < 0 ? 0x8000000000000000ull : 0ull;
  unsigned __int128 m = v < 0 ? (unsigned __int128)(-v) : (unsigned __int128)v;
  const unsigned long long mh = (unsigned long long)(m >> 64), ml = (unsigned long long)m;
  int p = mh ? 127 - __clzll((long long)mh) : 63 - __clzll((long long)ml);  // leading bit
  unsigned long long mant;
  if (p <= 52) {
    mant = ml << (52 - p);
  } else {
    const int sh = p - 52;
    mant = (unsigned long long)(m >> sh);
    const unsigned __int128 rem = m & (((unsigned __int128)1 << sh) - 1);
    const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
    if (rem > half || (rem == half && (mant & 1ull))) ++mant;
    if (mant >> 53) {
      mant >>= 1;
      ++p;
    }
  }
  const unsigned long long frac = mant & 0xfffffffffffffull;
  const int be = 1023 + p + E;
  if (be >= 1 && be <= 2046) return __longlong_as_double((long long)(sgn | ((unsigned long long)be << 52) | frac));
  return scalbn(__longlong_as_double((long long)(sgn | ((1023ull + (unsigned long long)p) << 52) | frac)), E);
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

__device__ __forceinline__ void tc_ld8(uint32_t taddr, uint32_t* r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}

}  // namespace oz
}  // namespace yb
