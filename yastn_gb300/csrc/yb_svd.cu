// Family (c): batched one-sided (Hestenes) Jacobi SVD / Hermitian eigendecomposition of
// all charge-sector blocks, mixed precision, real (FP64) or complex (complex128) data.
//
// Each block A (m x n, row-major) is handled in its "wide" orientation: the k=min(m,n)
// vectors to orthogonalise are the rows of A (m <= n) or of A^H (m > n), each of length
// L=max(m,n), held in a workspace X; rotations are accumulated in W (k x k), so that
// X = W X_0 at every step. A parallel round-robin ordering (circle method over
// N = k rounded up to even) pairs all vectors in N-1 rounds of N/2 disjoint pairs; one
// warp rotates one pair and all blocks advance together.
//
// GB300 has ~60x more FP32 than FP64 throughput, so the sweeps run in two phases:
//   1. FP32 sweeps on (X32, W32) (float or complex64) until the rows are orthogonal to
//      about 1e-4 (a blocked variant keeps super-vectors of rows in shared memory);
//   2. the host orthonormalises W = widen(W32) with Newton-Schulz steps and forms
//      X = W X_0 with the FP64 grouped GEMM; then FP64 sweeps polish (X, W) until a
//      sweep whose largest |cos| was below tol_stop (typically 2-3 sweeps).
// One persistent cooperative launch runs all the sweeps of a phase; rounds are separated
// by a grid barrier whose spin is bounded (an error flag is raised and the kernel exits
// if it ever times out). Finally S = row norms (descending), the normalised rows give Vh
// (wide) or U (tall, conjugated), and W^H gives the other factor.
//
// A rotation is applied when |<x_p, x_q>| > sqrt(L) eps ||x_p|| ||x_q|| (the threshold of
// LAPACK's one-sided Jacobi); the angle follows Rutishauser's formula with hypot. For
// complex rows the phase u = g/|g| of g = <x_p, x_q> = sum_l x_p[l] conj(x_q[l]) is first
// moved onto x_q, which makes the pair's inner product real, and the real rotation of
// (|x_p|^2, |x_q|^2, |g|) follows: x_p <- c x_p - s u x_q, x_q <- s x_p + c u x_q (unitary).
#include <float.h>
#include "yb_common.cuh"

namespace yb {
namespace {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;
constexpr long long kSpinLimit = 1ll << 22;

// record fields
enum { R_A = 0, R_M, R_N, R_U, R_S, R_V, R_X, R_W, R_P, R_K, R_L, R_NP, R_T, R_X32, R_W32, R_NSUP,
       R_QR, R_LQ, R_Z, R_VQ, R_TAU, R_RR, R_WS, R_NSUP64 };
// per-block state (int64): [0] max |cos| of the sweep in progress (double bits),
// [1] converged flag, [2] sweeps run in the current phase, [3] largest |cos| of the last sweep,
// [4], [5] squared row norms (double bits) at or below which a row is rounding noise in the
// FP32 / FP64 phase: a pair with such a row is neither rotated nor counted for convergence,
// and the finalisation completes the vectors of those rows like those of zero values
enum { ST_MAXCOS = 0, ST_CONV = 1, ST_SWEEPS = 2, ST_LASTCOS = 3, ST_THR32 = 4, ST_THR64 = 5, ST_REC = 6 };
constexpr double kNoise32 = 1e-5;   // noise row norm relative to ||A||_F in the FP32 phase
constexpr double kNoise64 = 1e-14;  // idem in the FP64 phase (a few FP64 roundings of ||A||_F)
// control words after the per-block state: [0] barrier count [1] barrier generation
// [2] error flag [3] all-converged flag
enum { C_COUNT = 0, C_GEN = 1, C_ERR = 2, C_DONE = 3, C_REC = 4 };

template <typename T>
struct Eps;
template <>
struct Eps<float> {
  static constexpr double v = 5.9604644775390625e-08;  // 2^-24
};
template <>
struct Eps<double> {
  static constexpr double v = 1.1102230246251565e-16;  // 2^-53
};

// Numeric traits of the four working types: float, double, complex64 (float2) and
// complex128 (double2). R is the real type; fmac(x, y, acc) = acc + x conj(y).
template <typename T>
struct Num;
template <>
struct Num<float> {
  using R = float;
  static constexpr bool cplx = false;
  __device__ static float zero() { return 0.f; }
  __device__ static float one() { return 1.f; }
  __device__ static float abs2(float x) { return x * x; }
  __device__ static float fmac(float x, float y, float acc) { return fmaf(x, y, acc); }
  __device__ static float fma_(float a, float b, float acc) { return fmaf(a, b, acc); }
  __device__ static float mul(float a, float b) { return a * b; }
  __device__ static float scale(float s, float a) { return s * a; }
  __device__ static float conj(float a) { return a; }
  __device__ static float add(float a, float b) { return a + b; }
  __device__ static float sub(float a, float b) { return a - b; }
};
template <>
struct Num<double> {
  using R = double;
  static constexpr bool cplx = false;
  __device__ static double zero() { return 0.0; }
  __device__ static double one() { return 1.0; }
  __device__ static double abs2(double x) { return x * x; }
  __device__ static double fmac(double x, double y, double acc) { return fma(x, y, acc); }
  __device__ static double fma_(double a, double b, double acc) { return fma(a, b, acc); }
  __device__ static double mul(double a, double b) { return a * b; }
  __device__ static double scale(double s, double a) { return s * a; }
  __device__ static double conj(double a) { return a; }
  __device__ static double add(double a, double b) { return a + b; }
  __device__ static double sub(double a, double b) { return a - b; }
};
template <>
struct Num<float2> {
  using R = float;
  static constexpr bool cplx = true;
  __device__ static float2 zero() { return make_float2(0.f, 0.f); }
  __device__ static float2 one() { return make_float2(1.f, 0.f); }
  __device__ static float abs2(float2 x) { return fmaf(x.x, x.x, x.y * x.y); }
  __device__ static float2 fmac(float2 x, float2 y, float2 acc) {
    return make_float2(fmaf(x.x, y.x, fmaf(x.y, y.y, acc.x)), fmaf(x.y, y.x, fmaf(-x.x, y.y, acc.y)));
  }
  __device__ static float2 fma_(float2 a, float2 b, float2 acc) {
    return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y)));
  }
  __device__ static float2 mul(float2 a, float2 b) { return fma_(a, b, zero()); }
  __device__ static float2 scale(float s, float2 a) { return make_float2(s * a.x, s * a.y); }
  __device__ static float2 conj(float2 a) { return make_float2(a.x, -a.y); }
  __device__ static float2 add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
  __device__ static float2 sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
};
template <>
struct Num<double2> {
  using R = double;
  static constexpr bool cplx = true;
  __device__ static double2 zero() { return make_double2(0.0, 0.0); }
  __device__ static double2 one() { return make_double2(1.0, 0.0); }
  __device__ static double abs2(double2 x) { return fma(x.x, x.x, x.y * x.y); }
  __device__ static double2 fmac(double2 x, double2 y, double2 acc) {
    return make_double2(fma(x.x, y.x, fma(x.y, y.y, acc.x)), fma(x.y, y.x, fma(-x.x, y.y, acc.y)));
  }
  __device__ static double2 fma_(double2 a, double2 b, double2 acc) {
    return make_double2(fma(a.x, b.x, fma(-a.y, b.y, acc.x)), fma(a.x, b.y, fma(a.y, b.x, acc.y)));
  }
  __device__ static double2 mul(double2 a, double2 b) { return fma_(a, b, zero()); }
  __device__ static double2 scale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
  __device__ static double2 conj(double2 a) { return make_double2(a.x, -a.y); }
  __device__ static double2 add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
  __device__ static double2 sub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
};

// conversions between the storage types
__device__ __forceinline__ float to32(double v) { return (float)v; }
__device__ __forceinline__ float2 to32(double2 v) { return make_float2((float)v.x, (float)v.y); }
__device__ __forceinline__ double to64(float v) { return (double)v; }
__device__ __forceinline__ double2 to64(float2 v) { return make_double2((double)v.x, (double)v.y); }
__device__ __forceinline__ double cabs2(double v) { return v * v; }
__device__ __forceinline__ double cabs2(double2 v) { return fma(v.x, v.x, v.y * v.y); }
__device__ __forceinline__ double cconj_(double v) { return v; }
__device__ __forceinline__ double2 cconj_(double2 v) { return make_double2(v.x, -v.y); }
__device__ __forceinline__ double add_real(double v, double c) { return v + c; }
__device__ __forceinline__ double2 add_real(double2 v, double c) { return make_double2(v.x + c, v.y); }
__device__ __forceinline__ double rscale(double v, double s) { return v * s; }
__device__ __forceinline__ double2 rscale(double2 v, double s) { return make_double2(v.x * s, v.y * s); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Jacobi rotation of a row pair from its warp-local partial sums al_ = |x_p|^2, be_ =
// |x_q|^2, ga_ = <x_p, x_q> (Rutishauser's formulas): returns true (every lane) if the pair
// is rotated, with (c, s) and the phase u (1 for real rows). |cos| of the pair goes to the
// block's running maximum. GB300 runs FP64 at 1/64 of the FP32 rate, so the FP32 phase
// keeps the whole computation in FP32, and the FP64 phase does the scalar part on lane 0
// only and broadcasts the result.
template <typename T>
__device__ __forceinline__ void warp_sum_t(T& v);
template <>
__device__ __forceinline__ void warp_sum_t<float>(float& v) { v = warp_sum(v); }
template <>
__device__ __forceinline__ void warp_sum_t<double>(double& v) { v = warp_sum(v); }
template <>
__device__ __forceinline__ void warp_sum_t<float2>(float2& v) { v.x = warp_sum(v.x); v.y = warp_sum(v.y); }
template <>
__device__ __forceinline__ void warp_sum_t<double2>(double2& v) { v.x = warp_sum(v.x); v.y = warp_sum(v.y); }

__device__ __forceinline__ float gabs(float g) { return fabsf(g); }
__device__ __forceinline__ double gabs(double g) { return fabs(g); }
__device__ __forceinline__ float gabs(float2 g) { return hypotf(g.x, g.y); }
__device__ __forceinline__ double gabs(double2 g) { return hypot(g.x, g.y); }

template <typename T>
struct Rotation {
  using R = typename Num<T>::R;
  // scalar part: from the summed (al, be, g) to (c, s, u); |cos| to the running maximum
  __device__ static bool scalar(R al, R be, T ga, int64_t L, int64_t* st, R& c, R& s, T& u, R thr2) {
    if (!(al > thr2 && be > thr2 && al > R(0) && be > R(0))) return false;
    const R g = gabs(ga);
    const R cosv = g / (sqrt(al) * sqrt(be));
    atomicMax((unsigned long long*)st, (unsigned long long)__double_as_longlong((double)cosv));
    if (!(cosv > sqrt((R)L) * (R)Eps<R>::v)) return false;
    R zeta;
    if constexpr (Num<T>::cplx) {
      u.x = ga.x / g;
      u.y = ga.y / g;
      zeta = (be - al) / (R(2) * g);
    } else {
      u = R(1);
      zeta = (be - al) / (R(2) * ga);
    }
    const R t = copysign(R(1), zeta) / (fabs(zeta) + hypot(R(1), zeta));
    c = R(1) / sqrt(fma(t, t, R(1)));
    s = c * t;
    return true;
  }
  // thr2: squared noise norm of the phase; a pair with a row at or below it is left alone
  __device__ static bool get(R al_, R be_, T ga_, int64_t L, int lane, int64_t* st, R& c, R& s, T& u, R thr2) {
    const R al = warp_sum(al_), be = warp_sum(be_);
    warp_sum_t<T>(ga_);
    if constexpr (sizeof(R) == 4) {
      // FP32: every lane computes the same (cheap) scalar part; one lane records |cos|
      if (!(al > thr2 && be > thr2 && al > R(0) && be > R(0))) return false;
      const R g = gabs(ga_);
      const R cosv = g / (sqrtf(al) * sqrtf(be));
      if (lane == 0) atomicMax((unsigned long long*)st, (unsigned long long)__double_as_longlong((double)cosv));
      if (!(cosv > sqrtf((float)L) * 5.9604645e-08f)) return false;
      R zeta;
      if constexpr (Num<T>::cplx) {
        u.x = ga_.x / g;
        u.y = ga_.y / g;
        zeta = (be - al) / (2.f * g);
      } else {
        u = 1.f;
        zeta = (be - al) / (2.f * ga_);
      }
      const R t = copysignf(1.f, zeta) / (fabsf(zeta) + hypotf(1.f, zeta));
      c = 1.f / sqrtf(fmaf(t, t, 1.f));
      s = c * t;
      return true;
    } else {
      int rot = 0;
      if (lane == 0) rot = scalar(al, be, ga_, L, st, c, s, u, thr2) ? 1 : 0;
      rot = __shfl_sync(0xffffffffu, rot, 0);
      if (!rot) return false;
      c = __shfl_sync(0xffffffffu, c, 0);
      s = __shfl_sync(0xffffffffu, s, 0);
      if constexpr (Num<T>::cplx) {
        u.x = __shfl_sync(0xffffffffu, u.x, 0);
        u.y = __shfl_sync(0xffffffffu, u.y, 0);
      } else {
        u = 1.0;
      }
      return true;
    }
  }
};

// (a, b) <- (c a - s u b, s a + c u b)
template <typename T>
__device__ __forceinline__ void rot2(T& a, T& b, typename Num<T>::R c, typename Num<T>::R s, T u) {
  T bu = b;
  if constexpr (Num<T>::cplx) bu = Num<T>::mul(u, b);
  const T na = Num<T>::sub(Num<T>::scale(c, a), Num<T>::scale(s, bu));
  const T nb = Num<T>::add(Num<T>::scale(s, a), Num<T>::scale(c, bu));
  a = na;
  b = nb;
}

// Per-block Frobenius norm -> shift[b] (eigh: makes a symmetric block positive definite)
// and scale[b], a power of two that brings the FP32 copy of the block (shift included)
// below 1 in magnitude, so that FP32 squares and dot products neither overflow nor lose
// the block to underflow. The rotations, and so W, do not depend on the scale.
template <typename TI>
__global__ void block_fro_kernel(const TI* __restrict__ A, const int64_t* __restrict__ blocks,
                                 double* __restrict__ shift, double* __restrict__ scale,
                                 int64_t* __restrict__ state) {
  // QR-preconditioned blocks start the FP32 phase from the rows of R, where small singular
  // values are explicit row norms rather than cancellations: its noise norm is FP64's
  __shared__ double red[32];
  const int64_t* r = blocks + (int64_t)blockIdx.x * YB_SVD_REC;
  const int64_t cnt = r[R_M] * r[R_N];
  const TI* a = A + r[R_A];
  double acc = 0.0;
  for (int64_t e = threadIdx.x; e < cnt; e += blockDim.x) acc += cabs2(a[e]);
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    // ||A||_2 <= ||A||_F: A + shift I is positive definite; +1 keeps an all-zero block regular
    const double fro = sqrt(tot);
    double bound = fro;
    if (shift != nullptr) {
      shift[blockIdx.x] = fro + 1.0;
      bound = 2.0 * fro + 1.0;
    }
    int e = 0;
    if (bound > 0.0 && bound <= 1.0e300) frexp(bound, &e);
    scale[blockIdx.x] = ldexp(1.0, -e);
    // the FP32 phase works on scale * A, the FP64 phase on A itself
    const double t32 = (r[R_QR] ? kNoise64 : kNoise32) * fro * ldexp(1.0, -e), t64 = kNoise64 * fro;
    state[(int64_t)blockIdx.x * ST_REC + ST_THR32] = __double_as_longlong(t32 * t32);
    state[(int64_t)blockIdx.x * ST_REC + ST_THR64] = __double_as_longlong(t64 * t64);
  }
}

// X32 = scale_b (A or A^H) (+ shift on the diagonal) in FP32, W32 = I; resets the state.
template <typename TI, typename T32>
__global__ void svd_init_kernel(const TI* __restrict__ A, T32* __restrict__ work32,
                                const int64_t* __restrict__ blocks, int64_t* __restrict__ state,
                                const double* __restrict__ shift, const double* __restrict__ scale) {
  const double sc = scale[blockIdx.y];
  const int64_t* r = blocks + (int64_t)blockIdx.y * YB_SVD_REC;
  const int64_t m = r[R_M], n = r[R_N], k = r[R_K], L = r[R_L];
  const bool tall = m > n;
  const int64_t xs = k * L, ws = k * k;
  T32* X = work32 + r[R_X32];
  T32* W = work32 + r[R_W32];
  const TI* a = A + r[R_A];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < xs + ws;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (e < xs) {
      const int64_t i = e / L, l = e - i * L;
      TI v = tall ? cconj_(a[l * n + i]) : a[e];
      if (shift != nullptr && i == l) v = add_real(v, shift[blockIdx.y]);
      X[e] = to32(rscale(v, sc));
    } else {
      const int64_t f = e - xs;
      const int64_t i = f / k, j = f - i * k;
      W[f] = (i == j) ? Num<T32>::one() : Num<T32>::zero();
    }
  }
  if (blockIdx.x == 0 && threadIdx.x < ST_THR32) state[blockIdx.y * ST_REC + threadIdx.x] = 0;
}

// Resets the sweep words (0..3) of each block's state (the noise norms stay).
__global__ void svd_state_reset_kernel(int64_t* __restrict__ state) {
  if (threadIdx.x < ST_THR32) state[blockIdx.x * ST_REC + threadIdx.x] = 0;
}

// W64 = widen(W32) (the host orthonormalises it next); resets the per-block state.
template <typename T32, typename T64>
__global__ void svd_widen_kernel(const T32* __restrict__ work32, T64* __restrict__ work64,
                                 const int64_t* __restrict__ blocks, int64_t* __restrict__ state) {
  const int64_t* r = blocks + (int64_t)blockIdx.y * YB_SVD_REC;
  const int64_t k = r[R_K];
  const T32* W32 = work32 + r[R_W32];
  T64* W = work64 + r[R_W];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < k * k; e += (int64_t)gridDim.x * blockDim.x)
    W[e] = to64(W32[e]);
  if (blockIdx.x == 0 && threadIdx.x < ST_THR32) state[blockIdx.y * ST_REC + threadIdx.x] = 0;
}

// X = shift_b * W (eigh: the FP64 phase then adds W A with the grouped GEMM, X = W (A + shift I)).
template <typename T64>
__global__ void svd_shift_prefill_kernel(T64* __restrict__ work64, const int64_t* __restrict__ blocks,
                                         const double* __restrict__ shift) {
  const int64_t* r = blocks + (int64_t)blockIdx.y * YB_SVD_REC;
  const int64_t k = r[R_K];
  const double c = shift[blockIdx.y];
  const T64* W = work64 + r[R_W];
  T64* X = work64 + r[R_X];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < k * k; e += (int64_t)gridDim.x * blockDim.x)
    X[e] = rscale(W[e], c);
}

// Grid barrier for a cooperative launch (all CTAs co-resident). The spin is bounded: on
// timeout the error flag is raised and false is returned, and the caller exits.
__device__ bool grid_barrier(unsigned long long* ctrl, unsigned nblocks) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned long long* gen = ctrl + C_GEN;
    const unsigned long long g = *gen;
    __threadfence();
    const unsigned long long arrived = atomicAdd(ctrl + C_COUNT, 1ull) + 1ull;
    if (arrived == nblocks) {
      ctrl[C_COUNT] = 0ull;
      __threadfence();
      atomicAdd(ctrl + C_GEN, 1ull);
    } else {
      long long spins = 0;
      while (*gen == g) {
        __nanosleep(32);
        if (++spins > kSpinLimit) {
          atomicExch(ctrl + C_ERR, 1ull);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

constexpr int kChunk = 8;  // elements per lane per row kept in flight
constexpr int kLoadBatch = 8;  // independent loads per thread when a CTA stages rows
constexpr int kRowRegs = 16;   // row elements per lane kept in registers in a blocked inner round

// Rotates rows (p, q) of X and W by one Jacobi rotation. Loads are issued a chunk at a
// time (kChunk per lane and row, all before any store of the chunk) so that the L2
// latency is paid once per chunk rather than once per element. Rows are rewritten by
// other SMs between rounds, so loads bypass L1 (ld.global.cg).
template <typename T>
__device__ __forceinline__ void rotate_rows(T* __restrict__ a, T* __restrict__ b, int64_t len, int lane,
                                            typename Num<T>::R c, typename Num<T>::R s, T u) {
  for (int64_t base = 0; base < len; base += 32 * kChunk) {
    T x[kChunk], y[kChunk];
#pragma unroll
    for (int j = 0; j < kChunk; ++j) {
      const int64_t i = base + j * 32 + lane;
      x[j] = (i < len) ? __ldcg(a + i) : Num<T>::zero();
      y[j] = (i < len) ? __ldcg(b + i) : Num<T>::zero();
    }
#pragma unroll
    for (int j = 0; j < kChunk; ++j) {
      const int64_t i = base + j * 32 + lane;
      if (i < len) {
        rot2<T>(x[j], y[j], c, s, u);
        a[i] = x[j];
        b[i] = y[j];
      }
    }
  }
}

template <typename T>
__device__ __forceinline__ void rotate_pair(T* __restrict__ X, T* __restrict__ W, int64_t k, int64_t L, int64_t p,
                                            int64_t q, int lane, int64_t* st) {
  using R = typename Num<T>::R;
  T* xp = X + p * L;
  T* xq = X + q * L;
  // partial sums in the working precision (FP32 in the FP32 phase keeps the FP64 pipe free)
  R al_ = 0, be_ = 0;
  T ga_ = Num<T>::zero();
  for (int64_t base = 0; base < L; base += 32 * kChunk) {
    T x[kChunk], y[kChunk];
#pragma unroll
    for (int j = 0; j < kChunk; ++j) {
      const int64_t i = base + j * 32 + lane;
      x[j] = (i < L) ? __ldcg(xp + i) : Num<T>::zero();
      y[j] = (i < L) ? __ldcg(xq + i) : Num<T>::zero();
    }
#pragma unroll
    for (int j = 0; j < kChunk; ++j) {
      al_ += Num<T>::abs2(x[j]);
      be_ += Num<T>::abs2(y[j]);
      ga_ = Num<T>::fmac(x[j], y[j], ga_);
    }
  }
  R c = 0, s = 0;
  T u = Num<T>::one();
  const R thr2 = (R)__longlong_as_double((long long)st[sizeof(R) == 4 ? ST_THR32 : ST_THR64]);
  if (!Rotation<T>::get(al_, be_, ga_, L, lane, st + ST_MAXCOS, c, s, u, thr2)) return;
  rotate_rows<T>(xp, xq, L, lane, c, s, u);
  rotate_rows<T>(W + p * k, W + q * k, k, lane, c, s, u);
}

// All sweeps of one precision phase in one cooperative launch.
template <typename T>
__global__ void __launch_bounds__(kThreads) svd_sweeps_kernel(T* __restrict__ work, const int64_t* __restrict__ blocks,
                                                              int n_blocks, const int32_t* __restrict__ pair_items,
                                                              int n_items, int max_rounds, int max_sweeps,
                                                              double tol_stop, int64_t* __restrict__ state) {
  unsigned long long* ctrl = reinterpret_cast<unsigned long long*>(state + (int64_t)n_blocks * ST_REC);
  __shared__ int any_active;
  const int lane = threadIdx.x & 31;
  const int64_t gwarp = (int64_t)blockIdx.x * kWarps + (threadIdx.x >> 5);
  const int64_t nwarps = (int64_t)gridDim.x * kWarps;
  const int rx = sizeof(typename Num<T>::R) == 4 ? R_X32 : R_X;
  const int rw = sizeof(typename Num<T>::R) == 4 ? R_W32 : R_W;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    for (int round = 0; round < max_rounds; ++round) {
      for (int64_t item = gwarp; item < n_items; item += nwarps) {
        const int b = pair_items[2 * item];
        const int pi = pair_items[2 * item + 1];
        int64_t* st = state + (int64_t)b * ST_REC;
        if (((volatile int64_t*)st)[ST_CONV]) continue;
        const int64_t* r = blocks + (int64_t)b * YB_SVD_REC;
        const int64_t k = r[R_K], L = r[R_L], N = r[R_NP];
        if (round >= N - 1) continue;
        int64_t p, q;
        if (pi == 0) {
          p = N - 1;
          q = round;
        } else {
          p = (round + pi) % (N - 1);
          q = (round - pi + (N - 1)) % (N - 1);
        }
        if (p >= k || q >= k) continue;  // the dummy vector of an odd count
        if (p > q) { const int64_t tq = p; p = q; q = tq; }
        rotate_pair<T>(work + r[rx], work + r[rw], k, L, p, q, lane, st);
      }
      if (!grid_barrier(ctrl, gridDim.x)) return;
    }
    // sweep end: a block whose largest |cos| in this sweep was <= tol_stop is converged
    if (blockIdx.x == 0) {
      if (threadIdx.x == 0) any_active = 0;
      __syncthreads();
      for (int b = threadIdx.x; b < n_blocks; b += blockDim.x) {
        int64_t* st = state + (int64_t)b * ST_REC;
        if (st[ST_CONV]) continue;
        const double mc = __longlong_as_double((long long)st[ST_MAXCOS]);
        st[ST_SWEEPS] += 1;
        st[ST_LASTCOS] = st[ST_MAXCOS];
        st[ST_MAXCOS] = 0;
        if (mc <= tol_stop) st[ST_CONV] = 1; else any_active = 1;
      }
      __syncthreads();
      if (threadIdx.x == 0) ctrl[C_DONE] = any_active ? 0ull : 1ull;
      __threadfence();
    }
    if (!grid_barrier(ctrl, gridDim.x)) return;
    if (((volatile unsigned long long*)ctrl)[C_DONE]) return;
  }
}

// ---------------------------------------------------------------------------------------
// Blocked variant for the FP32 phase: rows are grouped into super-vectors of BR rows; the
// circle method pairs super-vectors (R_NSUP of them, even), and one CTA per pair loads the
// 2*BR rows into shared memory, runs up to inner_sweeps one-sided Jacobi sweeps among them
// (circle method over the 2*BR rows, one warp per pair, rotations accumulated in a
// 2BR x 2BR matrix Q), writes the rows back and applies Q to the matching rows of W
// (column by column, in place). Outer rounds are separated by the grid barrier.
template <typename T, int BR>
__global__ void __launch_bounds__(BR * 32) svd_block_sweeps_kernel(T* __restrict__ work,
                                                                   const int64_t* __restrict__ blocks, int n_blocks,
                                                                   const int32_t* __restrict__ super_items,
                                                                   int n_items, int max_rounds, int max_sweeps,
                                                                   int inner_sweeps, double tol_stop, int lmax,
                                                                   int64_t* __restrict__ state) {
  constexpr int R2 = 2 * BR;
  using R = typename Num<T>::R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* Xs = reinterpret_cast<T*>(smem_raw);   // [R2][lmax]
  T* Qs = Xs + (size_t)R2 * lmax;           // [R2][R2]
  __shared__ int any_rot, any_active;
  __shared__ int64_t grow[R2];              // global row of each local row (-1: absent)
  unsigned long long* ctrl = reinterpret_cast<unsigned long long*>(state + (int64_t)n_blocks * ST_REC);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int rx = sizeof(typename Num<T>::R) == 4 ? R_X32 : R_X;
  const int rw = sizeof(typename Num<T>::R) == 4 ? R_W32 : R_W;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    for (int round = 0; round < max_rounds; ++round) {
      for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
        const int b = super_items[2 * item];
        const int pi = super_items[2 * item + 1];
        int64_t* st = state + (int64_t)b * ST_REC;
        if (((volatile int64_t*)st)[ST_CONV]) continue;
        const int64_t* r = blocks + (int64_t)b * YB_SVD_REC;
        const int64_t k = r[R_K], L = r[R_L], NS = r[sizeof(R) == 4 ? R_NSUP : R_NSUP64];
        if (round >= NS - 1) continue;
        int64_t P, Q;
        if (pi == 0) { P = NS - 1; Q = round; }
        else { P = (round + pi) % (NS - 1); Q = (round - pi + (NS - 1)) % (NS - 1); }
        T* X = work + r[rx];
        T* W = work + r[rw];
        __syncthreads();
        if (threadIdx.x < R2) {
          const int sv = threadIdx.x < BR ? (int)P : (int)Q;
          const int64_t g = (int64_t)sv * BR + (threadIdx.x % BR);
          grow[threadIdx.x] = (g < k) ? g : -1;
        }
        for (int e = threadIdx.x; e < R2 * R2; e += blockDim.x)
          Qs[e] = (e / R2 == e % R2) ? Num<T>::one() : Num<T>::zero();
        if (threadIdx.x == 0) any_rot = 0;
        __syncthreads();
        {
          // the rows of the pair: kLoadBatch independent L2 loads in flight per thread
          const unsigned tot = (unsigned)(R2 * L), Lu = (unsigned)L;
          for (unsigned e0 = threadIdx.x; e0 < tot; e0 += blockDim.x * kLoadBatch) {
            T v[kLoadBatch];
#pragma unroll
            for (int u = 0; u < kLoadBatch; ++u) {
              const unsigned e = e0 + u * blockDim.x;
              v[u] = Num<T>::zero();
              if (e < tot) {
                const unsigned i = e / Lu, l = e - i * Lu;
                const int64_t g = grow[i];
                if (g >= 0) v[u] = __ldcg(X + g * L + l);
              }
            }
#pragma unroll
            for (int u = 0; u < kLoadBatch; ++u) {
              const unsigned e = e0 + u * blockDim.x;
              if (e < tot) {
                const unsigned i = e / Lu, l = e - i * Lu;
                Xs[(size_t)i * lmax + l] = v[u];
              }
            }
          }
        }
        __syncthreads();
        for (int inner = 0; inner < inner_sweeps; ++inner) {
          __shared__ int rot_this;
          if (threadIdx.x == 0) rot_this = 0;
          __syncthreads();
          for (int ir = 0; ir < R2 - 1; ++ir) {
            int p, q;
            if (warp == 0) { p = R2 - 1; q = ir; }
            else { p = (ir + warp) % (R2 - 1); q = (ir - warp + (R2 - 1)) % (R2 - 1); }
            if (p > q) { const int t = p; p = q; q = t; }
            if (grow[p] >= 0 && grow[q] >= 0) {
              T* xp = Xs + (size_t)p * lmax;
              T* xq = Xs + (size_t)q * lmax;
              R al_ = 0, be_ = 0;
              T ga_ = Num<T>::zero();
              // rows of at most 32 kRowRegs elements stay in registers between the inner
              // products and the rotation (one shared-memory read and write per element)
              // (only for CTAs of up to 256 threads: wider ones have 128 registers per thread)
              constexpr int RR = (BR <= 8 && sizeof(T) * BR <= 64) ? kRowRegs : 1;
              const bool in_regs = RR == kRowRegs && L <= 32 * kRowRegs;
              T ra[RR], rb[RR];
              if (in_regs) {
#pragma unroll
                for (int u = 0; u < RR; ++u) {
                  const int l = lane + 32 * u;
                  ra[u] = (l < L) ? xp[l] : Num<T>::zero();
                  rb[u] = (l < L) ? xq[l] : Num<T>::zero();
                  al_ += Num<T>::abs2(ra[u]);
                  be_ += Num<T>::abs2(rb[u]);
                  ga_ = Num<T>::fmac(ra[u], rb[u], ga_);
                }
              } else {
                for (int64_t l = lane; l < L; l += 32) {
                  const T a = xp[l], b = xq[l];
                  al_ += Num<T>::abs2(a);
                  be_ += Num<T>::abs2(b);
                  ga_ = Num<T>::fmac(a, b, ga_);
                }
              }
              R c = 0, s = 0;
              T u = Num<T>::one();
              const R thr2 = (R)__longlong_as_double((long long)st[sizeof(R) == 4 ? ST_THR32 : ST_THR64]);
              if (Rotation<T>::get(al_, be_, ga_, L, lane, st + ST_MAXCOS, c, s, u, thr2)) {
                if (in_regs) {
#pragma unroll
                  for (int v = 0; v < RR; ++v) {
                    const int l = lane + 32 * v;
                    if (l < L) {
                      rot2<T>(ra[v], rb[v], c, s, u);
                      xp[l] = ra[v];
                      xq[l] = rb[v];
                    }
                  }
                } else {
                  for (int64_t l = lane; l < L; l += 32) {
                    T a = xp[l], b = xq[l];
                    rot2<T>(a, b, c, s, u);
                    xp[l] = a;
                    xq[l] = b;
                  }
                }
                for (int l = lane; l < R2; l += 32) {
                  T a = Qs[p * R2 + l], b = Qs[q * R2 + l];
                  rot2<T>(a, b, c, s, u);
                  Qs[p * R2 + l] = a;
                  Qs[q * R2 + l] = b;
                }
                if (lane == 0) { rot_this = 1; any_rot = 1; }
              }
            }
            __syncthreads();
          }
          const int rotated = rot_this;
          __syncthreads();  // every thread has read rot_this before the next sweep resets it
          if (!rotated) break;
        }
        if (any_rot) {
          const unsigned tot = (unsigned)(R2 * L), Lu = (unsigned)L;
          for (unsigned e = threadIdx.x; e < tot; e += blockDim.x) {
            const unsigned i = e / Lu, l = e - i * Lu;
            const int64_t g = grow[i];
            if (g >= 0) X[g * L + l] = Xs[(size_t)i * lmax + l];
          }
          // W rows: W_new = Q W_old for the 2*BR rows, one column per thread at a time
          for (int64_t c = threadIdx.x; c < k; c += blockDim.x) {
            T old[R2];
#pragma unroll
            for (int j = 0; j < R2; ++j) old[j] = (grow[j] >= 0) ? __ldcg(W + grow[j] * k + c) : Num<T>::zero();
#pragma unroll
            for (int i = 0; i < R2; ++i) {
              if (grow[i] < 0) continue;
              T acc = Num<T>::zero();
#pragma unroll
              for (int j = 0; j < R2; ++j) acc = Num<T>::fma_(Qs[i * R2 + j], old[j], acc);
              W[grow[i] * k + c] = acc;
            }
          }
        }
      }
      if (!grid_barrier(ctrl, gridDim.x)) return;
    }
    if (blockIdx.x == 0) {
      if (threadIdx.x == 0) any_active = 0;
      __syncthreads();
      for (int b = threadIdx.x; b < n_blocks; b += blockDim.x) {
        int64_t* st = state + (int64_t)b * ST_REC;
        if (st[ST_CONV]) continue;
        const double mc = __longlong_as_double((long long)st[ST_MAXCOS]);
        st[ST_SWEEPS] += 1;
        st[ST_LASTCOS] = st[ST_MAXCOS];
        st[ST_MAXCOS] = 0;
        if (mc <= tol_stop) st[ST_CONV] = 1; else any_active = 1;
      }
      __syncthreads();
      if (threadIdx.x == 0) ctrl[C_DONE] = any_active ? 0ull : 1ull;
      __threadfence();
    }
    if (!grid_barrier(ctrl, gridDim.x)) return;
    if (((volatile unsigned long long*)ctrl)[C_DONE]) return;
  }
}

template <typename T, int BR>
int launch_block_sweeps(T* work, const int64_t* blocks, int n_blocks, const int32_t* items, int n_items,
                        int max_rounds, int max_sweeps, int inner_sweeps, double tol_stop, int lmax, int64_t* state,
                        cudaStream_t s) {
  const size_t smem = ((size_t)2 * BR * lmax + (size_t)4 * BR * BR) * sizeof(T);
  int dev = 0, sms = 0, per_sm = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) { set_cuda_error((int)e); return YB_ERR_CUDA; }
  if (smem > (size_t)optin) return YB_ERR_TOO_LARGE;
  e = cudaFuncSetAttribute(svd_block_sweeps_kernel<T, BR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, svd_block_sweeps_kernel<T, BR>, BR * 32, smem);
  if (e != cudaSuccess) { set_cuda_error((int)e); return YB_ERR_CUDA; }
  if (per_sm < 1) return YB_ERR_TOO_LARGE;
  int grid = sms * per_sm;
  if (grid > n_items) grid = n_items;
  if (grid < 1) grid = 1;
  e = cudaMemsetAsync(state + (int64_t)n_blocks * ST_REC, 0, sizeof(int64_t) * C_REC, s);
  if (e != cudaSuccess) { set_cuda_error((int)e); return YB_ERR_CUDA; }
  void* args[] = {&work, &blocks, &n_blocks, &items, &n_items, &max_rounds, &max_sweeps, &inner_sweeps, &tol_stop,
                  &lmax, &state};
  e = cudaLaunchCooperativeKernel((const void*)svd_block_sweeps_kernel<T, BR>, dim3(grid), dim3(BR * 32), args, smem,
                                  s);
  if (e != cudaSuccess) { set_cuda_error((int)e); return YB_ERR_CUDA; }
  return YB_OK;
}

// One CTA per block: singular values = row norms, sort descending (index tie-break),
// write U, S, Vh; vectors of zero norm are completed to an orthonormal set.
// mode 0: SVD. mode 1/2: Hermitian eigendecomposition of a block shifted by shift[b]
// (lambda = sigma - shift), eigenvectors = columns of W^H, ordered ascending (1) or by
// |lambda| descending (2); Vh is not written.
// ---------------------------------------------------------------- QR preconditioning
// A block whose spectrum is graded (singular values spread over many decades, as in the
// projector blocks of a corner transfer matrix step) keeps one-sided Jacobi busy for tens of
// FP64 sweeps when started from the rows of A, where the small singular values are hidden
// in cancellations. Started from the rows of the triangular factor R of a Householder QR,
// they are explicit (graded row norms): the FP32 phase then resolves the whole spectrum and
// FP64 needs a few sweeps. With M = X_0^T (A^T for wide/square blocks, conj(A) for tall
// ones; M's columns are the rows of X_0) and M = Q R:
//   wide:  A = R^T Q^T;      W R = S Y  =>  U = Y^T,  Vh = conj(W) Q^T
//   tall:  A = conj(Q R);                 =>  U = conj(Q) W^T,  Vh = conj(Y)
// (Y: rows of X = W R normalised, W: the accumulated rotations). Z holds M's columns as
// rows (Z = X_0, k rows of length L); the factorisation leaves R in Z's upper part and the
// Householder vectors below the diagonal (LAPACK's geqr2 layout, transposed); Q^T is then
// formed in place (org2r, backward accumulation).

// Z = X_0 in FP64 (A, or A^H for tall blocks). Records with [16] = 2 (yb_qr, M = A): Z's
// rows are the first k columns of A (length L = m).
template <typename T>
__global__ void svd_qr_load_kernel(const T* __restrict__ A, T* __restrict__ work, const int64_t* __restrict__ blocks) {
  const int64_t* r = blocks + (int64_t)blockIdx.y * YB_SVD_REC;
  if (!r[R_QR]) return;
  const int64_t m = r[R_M], n = r[R_N], k = r[R_K], L = r[R_LQ];
  const bool tall = m > n, plain = r[R_QR] == 2;
  const T* a = A + r[R_A];
  T* Z = work + r[R_Z];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < k * L; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / L, l = e - i * L;
    Z[e] = plain ? a[l * n + i] : (tall ? cconj_(a[l * n + i]) : a[e]);
  }
}

template <typename T>
__device__ __forceinline__ T ldcg_t(const T* p) { return __ldcg(p); }

// Householder reflector of row j of Z on its elements [j, L) (LAPACK larfg): beta real,
// tau = (beta - alpha) / beta, v = x / (alpha - beta) with v_0 = 1 implicit; Z[j] = beta,
// v stored in Z[j+1..L), tau in tau[j]. One warp.
template <typename T>
__device__ void qr_reflector(T* __restrict__ z, T* __restrict__ tau, int64_t j, int64_t L, int lane) {
  __syncwarp();  // the row was just rewritten by other lanes of this warp
  double xn = 0.0;
  for (int64_t l = j + 1 + lane; l < L; l += 32) xn += cabs2(ldcg_t(z + l));
  xn = warp_sum(xn);
  const T alpha = ldcg_t(z + j);
  double ar, ai;
  if constexpr (Num<T>::cplx) { ar = alpha.x; ai = alpha.y; } else { ar = alpha; ai = 0.0; }
  if (xn == 0.0 && ai == 0.0) {
    if (lane == 0) tau[j] = Num<T>::zero();
    return;
  }
  const double beta = -copysign(sqrt(ar * ar + ai * ai + xn), ar);
  T tv, sc;
  if constexpr (Num<T>::cplx) {
    tv = make_double2((beta - ar) / beta, -ai / beta);
    // 1 / (alpha - beta)
    const double dr = ar - beta, di = ai, d2 = dr * dr + di * di;
    sc = make_double2(dr / d2, -di / d2);
  } else {
    tv = (beta - ar) / beta;
    sc = 1.0 / (ar - beta);
  }
  for (int64_t l = j + 1 + lane; l < L; l += 32) z[l] = Num<T>::mul(sc, ldcg_t(z + l));
  if (lane == 0) {
    if constexpr (Num<T>::cplx) z[j] = make_double2(beta, 0.0); else z[j] = beta;
    tau[j] = tv;
  }
}

// Applies I - t v v^H (v_0 = 1 at element j, v_l at elements l > j of vrow) to a row segment
// x[j..L) of Z: w = x_j + sum_l conj(v_l) x_l; x_j -= t w; x_l -= t w v_l. One warp.
template <typename T>
__device__ __forceinline__ void qr_apply(T* __restrict__ x, const T* __restrict__ vrow, T t, int64_t j, int64_t L,
                                         int lane) {
  const T xj = ldcg_t(x + j);
  T w = Num<T>::zero();
  for (int64_t l = j + 1 + lane; l < L; l += 32) w = Num<T>::fmac(ldcg_t(x + l), ldcg_t(vrow + l), w);
  warp_sum_t<T>(w);
  w = Num<T>::add(w, xj);
  const T tw = Num<T>::mul(t, w);
  if (lane == 0) x[j] = Num<T>::sub(xj, tw);
  for (int64_t l = j + 1 + lane; l < L; l += 32) x[l] = Num<T>::sub(ldcg_t(x + l), Num<T>::mul(tw, ldcg_t(vrow + l)));
  __syncwarp();
}

// Waits (lane 0 polls, bounded) until *flag >= target; on timeout raises *err and returns
// (the caller carries on with whatever it reads: the host sees the error word and fails).
__device__ __forceinline__ void qr_wait(const unsigned long long* flag, unsigned long long target,
                                        unsigned long long* err, int lane) {
  if (lane == 0) {
    long long spins = 0;
    while (*(volatile const unsigned long long*)flag < target) {
      __nanosleep(32);
      if (++spins > kSpinLimit) {
        atomicExch(err, 1ull);
        break;
      }
    }
    __threadfence();
  }
  __syncwarp();
}

__device__ __forceinline__ void qr_publish(unsigned long long* flag, unsigned long long value, int lane) {
  __syncwarp();
  if (lane == 0) {
    __threadfence();
    atomicMax(flag, value);
  }
}

// One cooperative launch: groups of `group` CTAs factor one block at a time. Row c of Z is
// handled by warp c mod (8 group) of the group throughout, so a row is only ever rewritten by
// the warp that reads it, and the only exchange is each reflector: the warp owning row j+1
// updates it first in step j, makes reflector j+1 and publishes it through the block's
// ready counter (flags[b] = number of reflectors published); every warp waits for reflector j
// before applying it, so warps run ahead of each other as far as the data allows. Then (one
// group barrier) R's rows, the FP32 start X32 = scale R, W32 = I and the reflectors are
// written; after a second barrier every warp forms its own columns of Q independently
// (Q e_c = H_0 ... H_c e_c), in place of its rows of Z.
template <typename T, typename T32>
__global__ void __launch_bounds__(kThreads) svd_qr_kernel(T* __restrict__ work, T32* __restrict__ work32,
                                                          const int64_t* __restrict__ blocks, int n_blocks,
                                                          int group, unsigned long long* __restrict__ qctrl,
                                                          const double* __restrict__ scale) {
  const int g = blockIdx.x / group, rank = blockIdx.x % group;
  const int n_groups = gridDim.x / group;
  if (g >= n_groups) return;
  unsigned long long* flags = qctrl;  // [n_blocks ready counters][C_REC words per group]
  unsigned long long* ctrl = qctrl + n_blocks + (int64_t)g * C_REC;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t gw = (int64_t)rank * kWarps + warp, nwg = (int64_t)group * kWarps;
  const int64_t gt = (int64_t)rank * kThreads + threadIdx.x, ngt = (int64_t)group * kThreads;
  for (int b = g; b < n_blocks; b += n_groups) {
    const int64_t* r = blocks + (int64_t)b * YB_SVD_REC;
    if (!r[R_QR]) continue;
    const int64_t k = r[R_K], L = r[R_LQ];
    T* Z = work + r[R_Z];
    T* V = work + r[R_VQ];
    T* tau = work + r[R_TAU];
    T* RR = work + r[R_RR];
    T32* X32 = work32 + r[R_X32];
    T32* W32 = work32 + r[R_W32];
    unsigned long long* ready = flags + b;
    const double sc = scale ? scale[b] : 0.0;  // no FP32 Jacobi start for yb_qr
    // factorisation
    if (gw == 0) {
      qr_reflector<T>(Z, tau, 0, L, lane);
      qr_publish(ready, 1ull, lane);
    }
    for (int64_t j = 0; j < k; ++j) {
      const int64_t first = j + 1 + ((gw - (j + 1)) % nwg + nwg) % nwg;
      if (first >= k) break;  // no rows of this warp below row j: none below any later row either
      qr_wait(ready, (unsigned long long)(j + 1), ctrl + C_ERR, lane);
      const T* vrow = Z + j * L;
      const T t = Num<T>::conj(ldcg_t(tau + j));  // M <- H^H M
      for (int64_t c = first; c < k; c += nwg) {
        qr_apply<T>(Z + c * L, vrow, t, j, L, lane);
        if (c == j + 1) {
          qr_reflector<T>(Z + c * L, tau, j + 1, L, lane);
          qr_publish(ready, (unsigned long long)(j + 2), lane);
        }
      }
    }
    if (!grid_barrier(ctrl, group)) return;
    // R rows, the FP32 start, the reflectors
    for (int64_t e = gt; e < k * k; e += ngt) {
      const int64_t i = e / k, c = e - i * k;
      const T v = (c >= i) ? ldcg_t(Z + c * L + i) : Num<T>::zero();
      RR[e] = v;
      if (scale) {
        X32[e] = to32(rscale(v, sc));
        W32[e] = (i == c) ? Num<T32>::one() : Num<T32>::zero();
      }
    }
    for (int64_t e = gt; e < k * L; e += ngt) {
      const int64_t j = e / L, l = e - j * L;
      V[e] = (l > j) ? ldcg_t(Z + e) : Num<T>::zero();
    }
    if (!grid_barrier(ctrl, group)) return;
    // Q's columns: row c of Z becomes (H_0 ... H_c e_c)^T
    for (int64_t c = gw; c < k; c += nwg) {
      T* x = Z + c * L;
      for (int64_t l = lane; l < L; l += 32) x[l] = (l == c) ? Num<T>::one() : Num<T>::zero();
      __syncwarp();
      for (int64_t j = c; j >= 0; --j) qr_apply<T>(x, V + j * L, ldcg_t(tau + j), j, L, lane);
    }
    if (!grid_barrier(ctrl, group)) return;
  }
}

// Candidate vectors of the blocked completion: G (L x nz, row-major per record) filled with
// values uniform in [-1, 1) from a counter-based hash of (record, element) (deterministic;
// any full-rank draw works: the candidates are projected and orthonormalised afterwards).
// recs: int64 pairs (offset, count) per record.
template <typename T>
__global__ void fill_candidates_kernel(T* __restrict__ G, const int64_t* __restrict__ recs) {
  const int64_t off = recs[2 * blockIdx.y], cnt = recs[2 * blockIdx.y + 1];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x) {
    uint64_t h = (uint64_t)(off + e) * 0x9E3779B97F4A7C15ull + (uint64_t)blockIdx.y * 0xD1B54A32D192ED03ull;
    h ^= h >> 31; h *= 0xBF58476D1CE4E5B9ull; h ^= h >> 29; h *= 0x94D049BB133111EBull; h ^= h >> 32;
    const double u = (double)(h >> 11) * 0x1.0p-52 - 1.0;
    if constexpr (Num<T>::cplx) {
      const uint64_t h2 = h * 0x2545F4914F6CDD1Dull;
      G[off + e] = make_double2(u, (double)(h2 >> 11) * 0x1.0p-52 - 1.0);
    } else {
      G[off + e] = u;
    }
  }
}

// yb_qr output: Q (m x k, row-major) from Z = Q^T and the square part of R (k x k of the
// k x n rows) from R's rows, both with the signs that make R's diagonal positive (LAPACK's
// diagonal is beta = -sign(Re alpha) |x|: s_c = -1 where it is negative, as the reference's
// sign(diag(R)) fix; a zero diagonal keeps +1). R's entries below the diagonal are zero.
template <typename T>
__global__ void qr_finalize_kernel(const T* __restrict__ work, T* __restrict__ Q, T* __restrict__ Rout,
                                   const int64_t* __restrict__ blocks) {
  const int64_t* r = blocks + (int64_t)blockIdx.y * YB_SVD_REC;
  const int64_t n = r[R_N], k = r[R_K], L = r[R_LQ];
  const T* Z = work + r[R_Z];
  const T* RR = work + r[R_RR];
  T* q = Q + r[R_U];
  T* rr = Rout + r[R_V];
  auto sgn = [&](int64_t c) -> double {
    const T d = RR[c * k + c];
    double re;
    if constexpr (Num<T>::cplx) re = d.x; else re = d;
    return re < 0.0 ? -1.0 : 1.0;
  };
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < L * k; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t l = e / k, c = e - l * k;
    q[e] = rscale(Z[c * L + l], sgn(c));
  }
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < k * k; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / k, c = e - i * k;
    rr[i * n + c] = (c >= i) ? rscale(RR[e], sgn(i)) : Num<T>::zero();
  }
}

template <typename T>
__global__ void __launch_bounds__(1024) svd_finalize_kernel(T* __restrict__ work, T* __restrict__ U,
                                                            double* __restrict__ S, T* __restrict__ Vh,
                                                            const int64_t* __restrict__ blocks, int pow2,
                                                            int mode, const double* __restrict__ shift,
                                                            const int64_t* __restrict__ state,
                                                            int64_t* __restrict__ n_small) {
  extern __shared__ unsigned char smem_raw[];
  // [sig: pow2 doubles][complex: pow2 doubles][idx: pow2 ints]
  double* sig = reinterpret_cast<double*>(smem_raw);
  double* cim = sig + pow2;
  int* idx = reinterpret_cast<int*>(cim + (Num<T>::cplx ? pow2 : 0));
  __shared__ int n_zero;
  __shared__ double kmin;
  const int64_t* r = blocks + (int64_t)blockIdx.x * YB_SVD_REC;
  const int64_t m = r[R_M], n = r[R_N], k = r[R_K], L = r[R_L];
  const bool tall = m > n;
  const T* X = work + r[R_X];
  const T* W = work + r[R_W];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) n_zero = 0;
  for (int i = threadIdx.x; i < pow2; i += blockDim.x) {
    sig[i] = -1.0;  // padding sorts last
    idx[i] = i;
  }
  __syncthreads();
  for (int64_t i = warp; i < k; i += nw) {
    double acc = 0.0;
    for (int64_t l = lane; l < L; l += 32) acc += cabs2(X[i * L + l]);
    acc = warp_sum(acc);
    if (lane == 0) {
      const double sv = sqrt(acc);
      sig[i] = (mode == 0) ? sv : (mode == 1 ? -(sv - shift[blockIdx.x]) : fabs(sv - shift[blockIdx.x]));
    }
  }
  __syncthreads();
  if (mode != 0) {
    // eigh sort keys may be negative: shift them so that the -1 padding still sorts last
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
  T* Ub = U + r[R_U];
  T* Vb = Vh + r[R_V];
  if (mode != 0) {
    for (int64_t j = warp; j < k; j += nw) {
      const int64_t i = idx[j];
      double acc = 0.0;
      for (int64_t l = lane; l < L; l += 32) acc += cabs2(X[i * L + l]);
      acc = warp_sum(acc);
      if (lane == 0) Sb[j] = sqrt(acc) - shift[blockIdx.x];
    }
    for (int64_t e = threadIdx.x; e < k * k; e += blockDim.x) {
      const int64_t j = e / k, c = e - j * k;
      Ub[c * k + j] = cconj_(W[(int64_t)idx[j] * k + c]);
    }
    return;
  }
  // rows at the rounding-noise level were not rotated: their vectors are completed like
  // those of zero values (the values themselves are kept)
  const double zthr = state ? sqrt(__longlong_as_double((long long)state[(int64_t)blockIdx.x * ST_REC + ST_THR64]))
                            : 0.0;
  for (int j = threadIdx.x; j < k; j += blockDim.x) {
    Sb[j] = sig[j];
    if (!(sig[j] > zthr && sig[j] > 0.0)) atomicAdd(&n_zero, 1);
  }
  // wide (X_0 = A): Vh rows = x_j / s_j, U = W^H; tall (X_0 = A^H): U columns = conj(x_j) / s_j,
  // Vh = W. QR-preconditioned (X_0 = R): wide: U columns = x_j / s_j, and the sorted conj(W)
  // goes to WS for Vh = conj(W) Q^T; tall: Vh rows = conj(x_j) / s_j, WS = sorted W for
  // U = conj(Q) W^T (both products follow as grouped GEMMs).
  const bool qr = r[R_QR] != 0;
  const bool to_u = tall != qr;  // the factor built from the rows of X
  for (int64_t e = threadIdx.x; e < k * L; e += blockDim.x) {
    const int64_t j = e / L, l = e - j * L;
    const double sv = sig[j];
    const T x = X[(int64_t)idx[j] * L + l];
    T v = (sv > zthr && sv > 0.0) ? rscale(x, 1.0 / sv) : rscale(x, 0.0);
    if (tall) v = cconj_(v);
    if (to_u) Ub[l * k + j] = v; else Vb[j * n + l] = v;
  }
  T* WS = work + r[R_WS];
  for (int64_t e = threadIdx.x; e < k * k; e += blockDim.x) {
    const int64_t j = e / k, c = e - j * k;
    const T w = W[(int64_t)idx[j] * k + c];
    if (qr) WS[e] = tall ? w : cconj_(w);
    else if (tall) Vb[j * n + c] = w;
    else Ub[c * k + j] = cconj_(w);
  }
  __syncthreads();
  if (n_zero == 0) return;
  // large completions (n_zero k L above 2^22) are left to the host's blocked completion
  // (random candidates projected with grouped GEMMs and orthonormalised by yb_qr): the count
  // goes to n_small[b] and the vectors stay as written
  if (n_small != nullptr && (double)n_zero * (double)k * (double)L > 4194304.0) {
    if (threadIdx.x == 0) n_small[blockIdx.x] = n_zero;
    return;
  }
  // completion: the small values sit at the end (positions k - n_zero .. k-1); each of their
  // vectors becomes a unit vector e_c orthogonalised against all earlier vectors by two passes
  // of classical Gram-Schmidt (all coefficients of a pass at once). The candidate is the
  // coordinate least covered by the earlier (orthonormal) vectors, c = argmin_l
  // sum_{i<j} |v_i[l]|^2: its residual norm^2 is 1 minus that sum, at least (L - j) / L since
  // the sums over l add up to j. The coefficients of a pass live in shared memory: real parts
  // in the sig array (no longer needed), imaginary parts in the complex area.
  const int64_t stride_v = to_u ? k : 1;  // distance between consecutive entries of one vector
  const int64_t stride_j = to_u ? 1 : n;  // distance between vectors
  T* base = to_u ? Ub : Vb;
  __shared__ double red[32];
  __shared__ int64_t redi[32];
  __shared__ double nrm_s;
  __shared__ int64_t cand_s;
  double* cre = sig;
  for (int64_t j = k - n_zero; j < k; ++j) {
    T* vj = base + j * stride_j;
    {
      // coverage of each coordinate by v_0..v_{j-1}; block argmin (ties: the smaller l)
      double bv = 3.0e300;
      int64_t bl = L;
      if (to_u) {
        for (int64_t l = warp; l < L; l += nw) {
          double acc = 0.0;
          for (int64_t i = lane; i < j; i += 32) acc += cabs2(base[l * stride_v + i]);
          acc = warp_sum(acc);
          if (acc < bv) { bv = acc; bl = l; }
        }
      } else {
        for (int64_t l = threadIdx.x; l < L; l += blockDim.x) {
          double acc = 0.0;
          for (int64_t i = 0; i < j; ++i) acc += cabs2(base[i * stride_j + l]);
          if (acc < bv) { bv = acc; bl = l; }
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const long long ol = __shfl_xor_sync(0xffffffffu, (long long)bl, o);
        if (ov < bv || (ov == bv && ol < bl)) { bv = ov; bl = ol; }
      }
      if (lane == 0) { red[warp] = bv; redi[warp] = bl; }
      __syncthreads();
      if (threadIdx.x == 0) {
        double v = red[0];
        int64_t c = redi[0];
        for (int w = 1; w < nw; ++w)
          if (red[w] < v || (red[w] == v && redi[w] < c)) { v = red[w]; c = redi[w]; }
        cand_s = c < L ? c : 0;
      }
      __syncthreads();
    }
    const int64_t cand = cand_s;
    {
      for (int64_t l = threadIdx.x; l < L; l += blockDim.x)
        vj[l * stride_v] = (l == cand) ? Num<T>::one() : Num<T>::zero();
      __syncthreads();
      for (int pass = 0; pass < 2; ++pass) {
        // coefficients c_i = <v_i, v_j> = sum_l conj(v_i[l]) v_j[l], i < j
        if (to_u) {
          // vectors are contiguous across i for a fixed l: one thread per i
          for (int64_t i = threadIdx.x; i < j; i += blockDim.x) {
            T acc = Num<T>::zero();
            for (int64_t l = 0; l < L; ++l) acc = Num<T>::fmac(vj[l * stride_v], base[l * stride_v + i], acc);
            if constexpr (Num<T>::cplx) {
              cre[i] = acc.x;
              cim[i] = acc.y;
            } else {
              cre[i] = acc;
            }
          }
        } else {
          // vectors are contiguous along l: one warp per i
          for (int64_t i = warp; i < j; i += nw) {
            T acc = Num<T>::zero();
            for (int64_t l = lane; l < L; l += 32) acc = Num<T>::fmac(vj[l], base[i * stride_j + l], acc);
            warp_sum_t<T>(acc);
            if (lane == 0) {
              if constexpr (Num<T>::cplx) {
                cre[i] = acc.x;
                cim[i] = acc.y;
              } else {
                cre[i] = acc;
              }
            }
          }
        }
        __syncthreads();
        // v_j -= sum_i c_i v_i
        if (to_u) {
          // row l of U holds entry l of every vector: one warp per l
          for (int64_t l = warp; l < L; l += nw) {
            T acc = Num<T>::zero();
            for (int64_t i = lane; i < j; i += 32) {
              T cf;
              if constexpr (Num<T>::cplx) cf = make_double2(cre[i], cim[i]);
              else cf = cre[i];
              acc = Num<T>::add(acc, Num<T>::mul(cf, base[l * stride_v + i]));
            }
            warp_sum_t<T>(acc);
            if (lane == 0) vj[l * stride_v] = Num<T>::sub(vj[l * stride_v], acc);
          }
        } else {
          for (int64_t l = threadIdx.x; l < L; l += blockDim.x) {
            T v = vj[l];
            for (int64_t i = 0; i < j; ++i) {
              T cf;
              if constexpr (Num<T>::cplx) cf = make_double2(cre[i], cim[i]);
              else cf = cre[i];
              v = Num<T>::sub(v, Num<T>::mul(cf, base[i * stride_j + l]));
            }
            vj[l] = v;
          }
        }
        __syncthreads();
      }
      double acc = 0.0;
      for (int64_t l = threadIdx.x; l < L; l += blockDim.x) acc += cabs2(vj[l * stride_v]);
      acc = warp_sum(acc);
      if (lane == 0) red[warp] = acc;
      __syncthreads();
      if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < nw; ++w) tot += red[w];
        nrm_s = sqrt(tot);
      }
      __syncthreads();
      const double nrm = nrm_s;
      for (int64_t l = threadIdx.x; l < L; l += blockDim.x)
        vj[l * stride_v] = nrm > 0.0 ? rscale(vj[l * stride_v], 1.0 / nrm) : Num<T>::zero();
      __syncthreads();
    }
  }
}

template <typename T>
int launch_sweeps(T* work, const int64_t* blocks, int n_blocks, const int32_t* pair_items, int n_items,
                  int max_rounds, int max_sweeps, double tol_stop, int64_t* state, cudaStream_t s) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, svd_sweeps_kernel<T>, kThreads, 0);
  if (e != cudaSuccess) { set_cuda_error((int)e); return YB_ERR_CUDA; }
  const int need = (n_items + kWarps - 1) / kWarps;
  int grid = sms * per_sm;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  // zero the barrier/control words (stream-ordered)
  e = cudaMemsetAsync(state + (int64_t)n_blocks * ST_REC, 0, sizeof(int64_t) * C_REC, s);
  if (e != cudaSuccess) { set_cuda_error((int)e); return YB_ERR_CUDA; }
  void* args[] = {&work, &blocks, &n_blocks, &pair_items, &n_items, &max_rounds, &max_sweeps, &tol_stop, &state};
  e = cudaLaunchCooperativeKernel((const void*)svd_sweeps_kernel<T>, dim3(grid), dim3(kThreads), args, 0, s);
  if (e != cudaSuccess) { set_cuda_error((int)e); return YB_ERR_CUDA; }
  return YB_OK;
}

}  // namespace
}  // namespace yb

namespace yb {

template <typename T>
int block_sweeps_t(T* w, const int64_t* blocks, int n_blocks, const int32_t* super_items, int n_items,
                          int max_rounds, int rows_per_super, int max_sweeps, int inner_sweeps, double tol_stop,
                          int lmax, int64_t* state, cudaStream_t s) {
  constexpr bool fp64 = sizeof(typename Num<T>::R) == 8;
  switch (rows_per_super) {
    case 16:
      if constexpr (fp64) return YB_ERR_INVALID;
      else return yb::launch_block_sweeps<T, 16>(w, blocks, n_blocks, super_items, n_items, max_rounds, max_sweeps,
                                                 inner_sweeps, tol_stop, lmax, state, s);
    case 8: return yb::launch_block_sweeps<T, 8>(w, blocks, n_blocks, super_items, n_items, max_rounds, max_sweeps,
                                                inner_sweeps, tol_stop, lmax, state, s);
    case 4: return yb::launch_block_sweeps<T, 4>(w, blocks, n_blocks, super_items, n_items, max_rounds, max_sweeps,
                                                inner_sweeps, tol_stop, lmax, state, s);
    default: return YB_ERR_INVALID;
  }
}

template <typename T, typename T32>
int qr_t(const void* a, void* work, void* work32, const int64_t* blocks, int n_blocks, int64_t* state, double* scale,
         int64_t* qctrl, int qctrl_words, cudaStream_t s) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, yb::svd_qr_kernel<T, T32>, yb::kThreads, 0);
  if (e != cudaSuccess) { yb::set_cuda_error((int)e); return YB_ERR_CUDA; }
  const int capacity = sms * (per_sm < 1 ? 1 : per_sm);
  int group = capacity / n_blocks;
  group = group < 1 ? 1 : (group > 64 ? 64 : group);
  int n_groups = capacity / group;
  if (n_groups > n_blocks) n_groups = n_blocks;
  if ((int64_t)n_groups * yb::C_REC + n_blocks > qctrl_words) n_groups = (qctrl_words - n_blocks) / yb::C_REC;
  if (n_groups < 1) return YB_ERR_INVALID;
  if (state) yb::block_fro_kernel<T><<<n_blocks, 256, 0, s>>>((const T*)a, blocks, nullptr, scale, state);
  yb::svd_qr_load_kernel<T><<<dim3(64, (unsigned)n_blocks), 256, 0, s>>>((const T*)a, (T*)work, blocks);
  e = cudaMemsetAsync(qctrl, 0, sizeof(int64_t) * ((size_t)n_groups * yb::C_REC + n_blocks), s);
  if (e != cudaSuccess) { yb::set_cuda_error((int)e); return YB_ERR_CUDA; }
  T* w = (T*)work;
  T32* w32 = (T32*)work32;
  unsigned long long* qc = (unsigned long long*)qctrl;
  void* args[] = {&w, &w32, &blocks, &n_blocks, &group, &qc, &scale};
  e = cudaLaunchCooperativeKernel((const void*)yb::svd_qr_kernel<T, T32>, dim3(n_groups * group), dim3(yb::kThreads),
                                  args, 0, s);
  if (e != cudaSuccess) { yb::set_cuda_error((int)e); return YB_ERR_CUDA; }
  if (state) yb::svd_state_reset_kernel<<<n_blocks, 32, 0, s>>>(state);
  return yb::check_launch();
}

template <typename T>
int finalize_t(void* work, void* U, double* S, void* Vh, const int64_t* blocks, int n_blocks, int pow2,
                      int mode, const double* shift, const int64_t* state, int64_t* n_small, cudaStream_t s) {
  const size_t smem = (size_t)pow2 * (sizeof(double) * (Num<T>::cplx ? 2 : 1) + sizeof(int));
  if (smem > 32 * 1024) {  // with the kernel's static shared memory the total passes 48 KB earlier
    cudaError_t e = cudaFuncSetAttribute(yb::svd_finalize_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) { yb::set_cuda_error((int)e); return YB_ERR_CUDA; }
  }
  yb::svd_finalize_kernel<T><<<n_blocks, 1024, smem, s>>>((T*)work, (T*)U, S, (T*)Vh, blocks, pow2, mode,
                                                          shift, state, n_small);
  return yb::check_launch();
}

}  // namespace yb

extern "C" {

int yb_svd_init(const void* a, void* work32, const int64_t* blocks, int n_blocks, int dtype, int64_t* state,
                double* shift, double* scale, void* stream) {
  if (n_blocks == 0) return YB_OK;
  if (dtype != YB_F64 && dtype != YB_C128) return YB_ERR_INVALID;
  if (!a || !work32 || !blocks || !state || !scale) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  dim3 grid(64, (unsigned)n_blocks);
  if (dtype == YB_F64) {
    yb::block_fro_kernel<double><<<n_blocks, 256, 0, s>>>((const double*)a, blocks, shift, scale, state);
    yb::svd_init_kernel<double, float><<<grid, 256, 0, s>>>((const double*)a, (float*)work32, blocks, state, shift,
                                                            scale);
  } else {
    yb::block_fro_kernel<double2><<<n_blocks, 256, 0, s>>>((const double2*)a, blocks, shift, scale, state);
    yb::svd_init_kernel<double2, float2><<<grid, 256, 0, s>>>((const double2*)a, (float2*)work32, blocks, state,
                                                              shift, scale);
  }
  return yb::check_launch();
}

int yb_svd_qr(const void* a, void* work64, void* work32, const int64_t* blocks, int n_blocks, int dtype,
              int64_t* state, double* scale, int64_t* qctrl, int qctrl_words, void* stream) {
  if (n_blocks == 0) return YB_OK;
  if (dtype != YB_F64 && dtype != YB_C128) return YB_ERR_INVALID;
  if (!a || !work64 || !work32 || !blocks || !state || !scale || !qctrl) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64)
    return yb::qr_t<double, float>(a, work64, work32, blocks, n_blocks, state, scale, qctrl, qctrl_words, s);
  return yb::qr_t<double2, float2>(a, work64, work32, blocks, n_blocks, state, scale, qctrl, qctrl_words, s);
}

int yb_fill_candidates(void* G, const int64_t* recs, int n_recs, int dtype, void* stream) {
  if (n_recs == 0) return YB_OK;
  if (!G || !recs) return YB_ERR_INVALID;
  const dim3 grid(32, (unsigned)n_recs);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64) yb::fill_candidates_kernel<double><<<grid, 256, 0, s>>>((double*)G, recs);
  else if (dtype == YB_C128) yb::fill_candidates_kernel<double2><<<grid, 256, 0, s>>>((double2*)G, recs);
  else return YB_ERR_INVALID;
  return yb::check_launch();
}

int yb_qr(const void* a, void* Q, void* R, void* work64, const int64_t* blocks, int n_blocks, int dtype,
          int64_t* qctrl, int qctrl_words, void* stream) {
  if (n_blocks == 0) return YB_OK;
  if (dtype != YB_F64 && dtype != YB_C128) return YB_ERR_INVALID;
  if (!a || !Q || !R || !work64 || !blocks || !qctrl) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const dim3 grid(64, (unsigned)n_blocks);
  int st;
  if (dtype == YB_F64) {
    st = yb::qr_t<double, float>(a, work64, nullptr, blocks, n_blocks, nullptr, nullptr, qctrl, qctrl_words, s);
    if (st != YB_OK) return st;
    yb::qr_finalize_kernel<double><<<grid, 256, 0, s>>>((const double*)work64, (double*)Q, (double*)R, blocks);
  } else {
    st = yb::qr_t<double2, float2>(a, work64, nullptr, blocks, n_blocks, nullptr, nullptr, qctrl, qctrl_words, s);
    if (st != YB_OK) return st;
    yb::qr_finalize_kernel<double2><<<grid, 256, 0, s>>>((const double2*)work64, (double2*)Q, (double2*)R, blocks);
  }
  return yb::check_launch();
}

int yb_svd_sweeps(void* work, const int64_t* blocks, int n_blocks, const int32_t* pair_items, int n_pair_items,
                  int max_rounds, int precision, int dtype, int max_sweeps, double tol_stop, int64_t* state,
                  void* stream) {
  if (n_blocks == 0 || n_pair_items == 0 || max_sweeps <= 0) return YB_OK;
  if (!work || !blocks || !pair_items || !state) return YB_ERR_INVALID;
  if (dtype != YB_F64 && dtype != YB_C128) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const bool c = dtype == YB_C128;
  if (precision == 32 && !c)
    return yb::launch_sweeps<float>((float*)work, blocks, n_blocks, pair_items, n_pair_items, max_rounds, max_sweeps,
                                    tol_stop, state, s);
  if (precision == 32 && c)
    return yb::launch_sweeps<float2>((float2*)work, blocks, n_blocks, pair_items, n_pair_items, max_rounds,
                                     max_sweeps, tol_stop, state, s);
  if (precision == 64 && !c)
    return yb::launch_sweeps<double>((double*)work, blocks, n_blocks, pair_items, n_pair_items, max_rounds,
                                     max_sweeps, tol_stop, state, s);
  if (precision == 64 && c)
    return yb::launch_sweeps<double2>((double2*)work, blocks, n_blocks, pair_items, n_pair_items, max_rounds,
                                      max_sweeps, tol_stop, state, s);
  return YB_ERR_INVALID;
}

int yb_svd_block_sweeps(void* work32, const int64_t* blocks, int n_blocks, const int32_t* super_items,
                        int n_items, int max_rounds, int rows_per_super, int precision, int dtype, int max_sweeps,
                        int inner_sweeps, double tol_stop, int lmax, int64_t* state, void* stream) {
  if (n_blocks == 0 || n_items == 0 || max_sweeps <= 0) return YB_OK;
  if (!work32 || !blocks || !super_items || !state || lmax <= 0 || inner_sweeps <= 0) return YB_ERR_INVALID;
  if (precision != 32 && precision != 64) return YB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == 64) {
    if (rows_per_super != 4 && rows_per_super != 8) return YB_ERR_INVALID;
    if (dtype == YB_F64)
      return yb::block_sweeps_t<double>((double*)work32, blocks, n_blocks, super_items, n_items, max_rounds,
                                        rows_per_super, max_sweeps, inner_sweeps, tol_stop, lmax, state, s);
    if (dtype == YB_C128)
      return yb::block_sweeps_t<double2>((double2*)work32, blocks, n_blocks, super_items, n_items, max_rounds,
                                         rows_per_super, max_sweeps, inner_sweeps, tol_stop, lmax, state, s);
    return YB_ERR_INVALID;
  }
  if (dtype == YB_F64)
    return yb::block_sweeps_t<float>((float*)work32, blocks, n_blocks, super_items, n_items, max_rounds, rows_per_super,
                                 max_sweeps, inner_sweeps, tol_stop, lmax, state, s);
  if (dtype == YB_C128)
    return yb::block_sweeps_t<float2>((float2*)work32, blocks, n_blocks, super_items, n_items, max_rounds,
                                  rows_per_super, max_sweeps, inner_sweeps, tol_stop, lmax, state, s);
  return YB_ERR_INVALID;
}

int yb_svd_widen(const void* work32, void* work64, const int64_t* blocks, int n_blocks, int dtype, int64_t* state,
                 void* stream) {
  if (n_blocks == 0) return YB_OK;
  if (!work32 || !work64 || !blocks || !state) return YB_ERR_INVALID;
  dim3 grid(64, (unsigned)n_blocks);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64)
    yb::svd_widen_kernel<float, double><<<grid, 256, 0, s>>>((const float*)work32, (double*)work64, blocks, state);
  else if (dtype == YB_C128)
    yb::svd_widen_kernel<float2, double2><<<grid, 256, 0, s>>>((const float2*)work32, (double2*)work64, blocks,
                                                               state);
  else
    return YB_ERR_INVALID;
  return yb::check_launch();
}

int yb_svd_shift_prefill(void* work64, const int64_t* blocks, int n_blocks, int dtype, const double* shift,
                         void* stream) {
  if (n_blocks == 0) return YB_OK;
  if (!work64 || !blocks || !shift) return YB_ERR_INVALID;
  dim3 grid(64, (unsigned)n_blocks);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64)
    yb::svd_shift_prefill_kernel<double><<<grid, 256, 0, s>>>((double*)work64, blocks, shift);
  else if (dtype == YB_C128)
    yb::svd_shift_prefill_kernel<double2><<<grid, 256, 0, s>>>((double2*)work64, blocks, shift);
  else
    return YB_ERR_INVALID;
  return yb::check_launch();
}

int yb_svd_finalize(void* work, void* U, double* S, void* Vh, const int64_t* blocks, int n_blocks, int dtype,
                    int max_k, int mode, const double* shift, const int64_t* state, int64_t* n_small,
                    void* stream) {
  if (n_blocks == 0) return YB_OK;
  if (dtype != YB_F64 && dtype != YB_C128) return YB_ERR_INVALID;
  if (mode < 0 || mode > 2 || (mode != 0 && shift == nullptr)) return YB_ERR_INVALID;
  if (max_k > 8192) return YB_ERR_TOO_LARGE;
  int pow2 = 1;
  while (pow2 < max_k) pow2 <<= 1;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == YB_F64)
    return yb::finalize_t<double>(work, U, S, Vh, blocks, n_blocks, pow2, mode, shift, state, n_small, s);
  return yb::finalize_t<double2>(work, U, S, Vh, blocks, n_blocks, pow2, mode, shift, state, n_small, s);
}

}  // extern "C"
