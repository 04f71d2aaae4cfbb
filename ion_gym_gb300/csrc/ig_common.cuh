// ig_common.cuh -- shared device helpers for the ion_gym field-solve kernels.
//
// Exactness contract of the FP64 kernels: every FP64 operation is an explicit
// round-to-nearest intrinsic (__dadd_rn, __dmul_rn, __fma_rn, __ddiv_rn,
// __drcp_rn), so nothing is contracted or reassociated and each kernel returns
// the bits of the reference's float64 arithmetic (left-to-right evaluation,
// float32 theta products kept in float32, as the compiled reference types
// them).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ig {

// Even-reflection neighbour rule at every outer face (the ghost at -1 is
// node 1, the ghost at n is node n-2; a size-1 axis uses the node itself).
__host__ __device__ __forceinline__ long lo_nb(long i, long n) {
  return i > 0 ? i - 1 : (n > 1 ? 1 : i);
}
__host__ __device__ __forceinline__ long hi_nb(long i, long n) {
  return i < n - 1 ? i + 1 : (n > 1 ? n - 2 : i);
}

// x / 6.0 correctly rounded, in two FP64 operations instead of a full
// division: q = RN(x*zh + RN(x*zl)) with zh = RN(1/6), zl = RN(1/6 - zh)
// (Brisebarre, Muller, Raina, "Accelerating correctly rounded floating-point
// division when the divisor is known in advance", IEEE Trans. Comput. 53(8),
// 2004).  Why it is exact for the divisor 6: x = M*2^e with an integer
// 53-bit M, so the bits of x/6 beyond the 53rd are r/3 ulp with r in
// {0,1,2}; the true quotient is therefore never closer than 1/6 ulp to a
// rounding midpoint, while the unrounded x*zh + RN(x*zl) is within about
// 2^-100 relative of x/6.  Rounding it once gives RN(x/6).  Subnormal and
// huge magnitudes, and non-finite x, take the hardware division.  Checked
// bit-for-bit against x/6.0 by the test-suite.
__device__ __forceinline__ double div6(double x) {
  const unsigned e = (static_cast<unsigned>(__double2hiint(x)) >> 20) & 0x7ffu;
  if (e < 64u || e > 2000u) {
    // +-0 / 6 is +-0 (sign kept): cold starts are mostly zeros
    if ((static_cast<unsigned long long>(__double_as_longlong(x)) << 1) == 0ULL) return x;
    return __ddiv_rn(x, 6.0);
  }
  const double zh = 0x1.5555555555555p-3;
  const double zl = 0x1.5555555555555p-57;
  return __fma_rn(x, zh, __dmul_rn(x, zl));
}

// |d| as an order-preserving 64-bit key (d >= 0, so the IEEE bit pattern
// orders like the value).  NaN maps to 0: the reference's "if d > dmax"
// never takes a NaN.
__device__ __forceinline__ unsigned long long absbits(double d) {
  unsigned long long b =
      static_cast<unsigned long long>(__double_as_longlong(d)) & 0x7fffffffffffffffULL;
  return b > 0x7ff0000000000000ULL ? 0ULL : b;
}

// Warp max of a 64-bit key with two 32-bit warp reductions (REDUX): the
// largest high word, then the largest low word among the lanes holding it.
// Every lane of the warp must call it.
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
  const unsigned hi = __reduce_max_sync(0xffffffffu, (unsigned)(v >> 32));
  const unsigned lo =
      __reduce_max_sync(0xffffffffu, (unsigned)(v >> 32) == hi ? (unsigned)v : 0u);
  return ((unsigned long long)hi << 32) | lo;
}

// Block-wide max of a 64-bit key, then one atomicMax into *dst -- only when
// it beats the value already there, so the tens of thousands of blocks of a
// launch do not all queue atomics on one address.  Every thread of the
// block must call it.
__device__ __forceinline__ void block_max_to(unsigned long long v,
                                             unsigned long long* dst) {
  __shared__ unsigned long long red[32];
  v = warp_max_u64(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? red[lane] : 0ULL;
    v = warp_max_u64(v);
    if (lane == 0 && v && v > *reinterpret_cast<volatile unsigned long long*>(dst))
      atomicMax(dst, v);
  }
}

__host__ __device__ __forceinline__ double bits_to_double(unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(static_cast<long long>(b));
#else
  double d;
  __builtin_memcpy(&d, &b, 8);
  return d;
#endif
}

}  // namespace ig
