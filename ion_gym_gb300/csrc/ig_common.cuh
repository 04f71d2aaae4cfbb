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

// x / 6.0 correctly rounded without the FP64 pipe (GB300 runs FP64 at
// about 1/64 of its integer rate, and the theta-free sweep is bound by it).
// x = M * 2^(E-52) with a 53-bit integer significand M, so x/6 =
// (N/3) * 2^(E-53-k) with N = M * 2^k, k = 1 when M >= 1.5 * 2^52 and 2
// otherwise, which puts N/3 in [2^52, 2^53).  Q = floor(N/3) (one 64-bit
// multiply-high by ceil(2^65/3)) and the remainder r = N - 3Q is 0, 1 or 2:
// the discarded fraction r/3 is never one half, so RN(N/3) is Q + (r == 2),
// and Q + 1 never reaches 2^53 (that would need N = 3*2^53 - 1, odd).  The
// result is Q with the biased exponent lowered by 1 + k.  Zeros return
// themselves (sign kept; cold starts are mostly zeros); exponents whose
// quotient would be subnormal (biased below 4), infinities and NaNs take the
// hardware division.  Checked bit-for-bit against x/6.0 by the test-suite.
__device__ __forceinline__ double div6(double x) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned eb = (static_cast<unsigned>(b >> 32) >> 20) & 0x7ffu;
  if (eb - 4u > 2042u) {
    if ((b << 1) == 0ULL) return x;
    return __ddiv_rn(x, 6.0);
  }
  const unsigned long long m = (b & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
  const unsigned k = m >= 0x0018000000000000ULL ? 1u : 2u;
  const unsigned long long n = m << k;
  const unsigned long long q0 = __umul64hi(n, 0xAAAAAAAAAAAAAAABULL) >> 1;
  const unsigned r = static_cast<unsigned>(n) - 3u * static_cast<unsigned>(q0);
  const unsigned long long q = q0 + (r == 2u ? 1ULL : 0ULL);
  // q carries the implicit bit 2^52, so adding it to the exponent field
  // (eb - 2 - k) << 52 sets the exponent to eb - 1 - k
  const unsigned long long mag =
      (static_cast<unsigned long long>(eb - 2u - k) << 52) + q;
  return __longlong_as_double(static_cast<long long>((b & 0x8000000000000000ULL) | mag));
}

// RN(omega * RN(q - old)), the SOR step of every sweep, on the integer pipe
// where that is exact.  With q = Mq*2^(eq-1075) and old = Mo*2^(eo-1075)
// (53-bit integer significands, biased exponents no more than one apart) the
// difference is the exact integer D = +-Mq*2^(eq-e) -+ Mo*2^(eo-e), e the
// smaller exponent; when |D| < 2^53 it is RN(q - old) itself.  The product
// W*|D| (W omega's significand) is exact in 128 bits and is rounded once to
// 53 bits, to nearest, ties to even -- RN(omega * d).  Lanes outside that
// window (zeros, subnormals, exponents more than one apart, a difference
// that would round, a subnormal or overflowing product, omega not a
// positive normal number) take the two FP64 operations.  q == old gives +0,
// as q - old does.  Checked bit-for-bit against the FP64 expression by the
// test-suite.
__device__ __forceinline__ double omega_step(double old, double q, double omega) {
  constexpr unsigned long long kFrac = 0x000fffffffffffffULL, kHid = 0x0010000000000000ULL;
  const unsigned long long bq = static_cast<unsigned long long>(__double_as_longlong(q));
  const unsigned long long bo = static_cast<unsigned long long>(__double_as_longlong(old));
  const unsigned long long bw = static_cast<unsigned long long>(__double_as_longlong(omega));
  const unsigned eq = static_cast<unsigned>(bq >> 52) & 0x7ffu;
  const unsigned eo = static_cast<unsigned>(bo >> 52) & 0x7ffu;
  const unsigned ew = static_cast<unsigned>(bw >> 52);  // sign bit included
  const unsigned emin = min(eq, eo);
  bool ok = eq - 1u < 2046u && eo - 1u < 2046u && max(eq, eo) - emin <= 1u &&
            ew - 1u < 2046u;
  unsigned long long out = 0;
  if (ok) {
    long long a = static_cast<long long>(((bq & kFrac) | kHid) << (eq - emin));
    long long b = static_cast<long long>(((bo & kFrac) | kHid) << (eo - emin));
    if (static_cast<long long>(bq) < 0) a = -a;
    if (static_cast<long long>(bo) < 0) b = -b;
    const long long dd = a - b;
    if (dd == 0) return 0.0;
    const unsigned long long ad = static_cast<unsigned long long>(dd < 0 ? -dd : dd);
    ok = (ad >> 53) == 0ULL;
    if (ok) {
      const unsigned long long w = (bw & kFrac) | kHid;
      const unsigned long long lo = w * ad, hi = __umul64hi(w, ad);
      int sh = (hi ? 128 - __clzll(static_cast<long long>(hi))
                   : 64 - __clzll(static_cast<long long>(lo))) - 53;  // 0..53
      unsigned long long m = lo;
      if (sh > 0) {
        m = (lo >> sh) | (hi << (64 - sh));
        const unsigned long long rem = lo & ((1ULL << sh) - 1ULL), half = 1ULL << (sh - 1);
        m += (rem > half || (rem == half && (m & 1ULL))) ? 1ULL : 0ULL;
        if (m >> 53) {
          m >>= 1;
          sh++;
        }
      }
      const int eu = sh + static_cast<int>(ew) + static_cast<int>(emin) - 1075;
      ok = eu >= 1 && eu <= 2046;
      // m carries the implicit bit: (eu - 1) << 52 plus m has exponent eu
      out = (dd < 0 ? 0x8000000000000000ULL : 0ULL) |
            ((static_cast<unsigned long long>(eu - 1) << 52) + m);
    }
  }
  if (!ok) return __dmul_rn(omega, __dsub_rn(q, old));
  return __longlong_as_double(static_cast<long long>(out));
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
