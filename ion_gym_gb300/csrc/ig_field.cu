// ig_field.cu -- from solved bases to the flight's fields on the device:
// unit bases (build_stl3d.py:835-849, (phi / v_basis).astype(float32)),
// drive superposition (build_stl3d.py:547-568, A = sum float32(v_i) * b_i
// and group potentials = sum of member bases, in float32) and the
// electrode-aware E-field (tracer3d.py:55-117, numpy.gradient with the
// one-sided rule at metal nodes beside vacuum), bit-identical to the
// reference.
//
// Rounding follows the reference's typing exactly:
//  * superposition: float32 multiply, then float32 add into an accumulator
//    that starts at +0, terms in electrode order; zero drive terms are
//    skipped as the reference skips them;
//  * numpy.gradient on a float32 potential divides in float32 when the
//    spacing is a Python float (NEP 50 "weak" scalar: RN32(2h), RN32(h))
//    and in float64 then rounds to float32 when the spacing is a numpy
//    float64 (h_is_f64);
//  * the metal-node correction is compiled with a float64 spacing: the
//    float32 difference is divided in float64 and rounded to float32.
// Every operation is an explicit round-to-nearest intrinsic, so no fused
// multiply-add can change a bit.
#include <cmath>
#include <cstdint>
#include <string>
#include <type_traits>
#include <vector>

#include "ig_common.cuh"
#include "ig_internal.h"
#include "../../include/igsolve.h"

namespace ig {
namespace {

constexpr int kMaxSteps = IG_FIELD_MAX_STEPS;
constexpr int kMaxCh = IG_FIELD_MAX_CHANNELS;

// One superposition launch: channels [0, nch) over steps [0, nsteps).
// Step s reads the basis at src[s]; channel c adds mult[c][s] times
// RN32(w[c][s] * basis).
struct SupPlan {
  int nsteps, nch, accumulate, pad;
  const float* src[kMaxSteps];
  float w[kMaxCh][kMaxSteps];
  uint8_t mult[kMaxCh][kMaxSteps];
};
static_assert(sizeof(SupPlan) < 4000, "superposition plan must fit the kernel parameters");

// Superposition.  Each thread keeps NCH float32 accumulators and reads
// the bases B steps at a time (B = 8, fewer for wide float4 accumulators so
// the registers suffice; the B loads are issued before any is used, so a
// warp has B independent DRAM reads in flight).  k_superpose4 works on
// float4 groups [0, n4) when every basis and output row is 16-byte aligned;
// k_superpose1 on single nodes [first, n).
template <int NCH, typename V>
__device__ __forceinline__ void sup_steps(V* acc, const SupPlan& plan, long long t);

__device__ __forceinline__ void sup_add(float& a, float w, float x) {
  a = __fadd_rn(a, __fmul_rn(w, x));
}
__device__ __forceinline__ void sup_add(float4& a, float w, float4 x) {
  sup_add(a.x, w, x.x);
  sup_add(a.y, w, x.y);
  sup_add(a.z, w, x.z);
  sup_add(a.w, w, x.w);
}
__device__ __forceinline__ float sup_load(const float* p, long long t) { return __ldcs(p + t); }
__device__ __forceinline__ float4 sup_load4(const float* p, long long t) {
  return __ldcs(reinterpret_cast<const float4*>(p) + t);
}

template <int NCH, bool VEC>
__global__ void __launch_bounds__(256)
k_superpose(long long first, long long n, const SupPlan plan, float* __restrict__ out,
            long long ostride) {
  using V = typename std::conditional<VEC, float4, float>::type;
  for (long long t = first + (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    V acc[NCH];
#pragma unroll
    for (int c = 0; c < NCH; c++) {
      if (plan.accumulate)
        acc[c] = reinterpret_cast<const V*>(out + c * ostride)[t];
      else
        acc[c] = V{};
    }
    constexpr int B = !VEC ? 8 : (NCH <= 2 ? 8 : (NCH <= 4 ? 4 : 2));
    for (int s0 = 0; s0 < plan.nsteps; s0 += B) {
      V x[B];
#pragma unroll
      for (int u = 0; u < B; u++) {
        if (s0 + u < plan.nsteps) {
          if constexpr (VEC)
            x[u] = sup_load4(plan.src[s0 + u], t);
          else
            x[u] = sup_load(plan.src[s0 + u], t);
        }
      }
#pragma unroll
      for (int u = 0; u < B; u++) {
        const int s = s0 + u;
        if (s < plan.nsteps) {
#pragma unroll
          for (int c = 0; c < NCH; c++) {
            const float w = plan.w[c][s];
            for (int m = 0; m < plan.mult[c][s]; m++) sup_add(acc[c], w, x[u]);
          }
        }
      }
    }
#pragma unroll
    for (int c = 0; c < NCH; c++) reinterpret_cast<V*>(out + c * ostride)[t] = acc[c];
  }
}

// (phi / v_basis).astype(float32): float64 division, then round to float32.
__global__ void __launch_bounds__(256)
k_unit_basis(const double* __restrict__ phi, long long n, double vb, float* __restrict__ out) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    out[t] = __double2float_rn(__ddiv_rn(__ldcs(phi + t), vb));
}

// ---- exact divisions ------------------------------------------------------
// Dv: RN32(d / c) for a float32 divisor c fixed per launch, with y =
// RN32(1/c) (chosen on the host as the float nearest 1/c).  q0 = RN(d*y) is
// within 1.5 ulp of d/c; one FMA correction makes q1 faithful, so the
// remainder d - q1*c is exact (one FMA) and q1 + r*y rounded once is the
// correctly rounded quotient (Markstein's theorem: a faithful quotient and a
// correctly rounded reciprocal give RN(d/c) after one correction).  Inputs
// outside [2^-100, 2^100] (zeros, subnormals, inf, NaN) and divisors outside
// [2^-20, 2^20] take the IEEE division instead.
struct Dv {
  float c, y;
  int ok;
};

__device__ __forceinline__ float div32(float d, const Dv& D) {
  const float ad = fabsf(d);
  if (D.ok && ad >= 0x1p-100f && ad <= 0x1p100f) {
    const float q0 = __fmul_rn(d, D.y);
    const float r0 = __fmaf_rn(-q0, D.c, d);
    const float q1 = __fmaf_rn(r0, D.y, q0);
    const float r1 = __fmaf_rn(-q1, D.c, d);
    return __fmaf_rn(r1, D.y, q1);
  }
  if (D.ok && d == 0.f) return __fmul_rn(d, D.y);
  return __fdiv_rn(d, D.c);
}

// Dh: RN32(RN64(d / h)) for a float32 d and a float64 h, as compiled numpy
// and numba code computes a float32 difference over a float64 spacing.  With
// hh = RN32(h), hl = RN32(h - hh): q0 = RN32(d / hh) exactly (div32), the
// remainder r = d - q0*hh exactly (one FMA), and c = (r - q0*hl) / hh
// approximates d/h - q0 to within 2^-44 |q0|.  s = RN32(q0 + c) is the
// answer unless q0 + c lies within 2^-42 |s| of a rounding boundary of s
// (the half-way points to its float32 neighbours); then, and for inputs
// outside the checked ranges, the float64 division decides.
struct Dh {
  double h;
  float hh, hl, rh;
  Dv dh;
  int ok;
};

__device__ __noinline__ float div64_slow(float d, double h) {
  return __double2float_rn(__ddiv_rn((double)d, h));
}

__device__ __forceinline__ float div64(float d, const Dh& H) {
  if (H.ok) {
    const float q0 = div32(d, H.dh);
    if (d == 0.f) return q0;  // +-0 / h (h > 0) keeps the sign of d
    const float aq = fabsf(q0);
    if (aq >= 0x1p-40f && aq <= 0x1p40f) {
      const float r = __fmaf_rn(-q0, H.hh, d);
      const float num = __fmaf_rn(-q0, H.hl, r);
      const float c = __fmul_rn(num, H.rh);
      const float s = __fadd_rn(q0, c);
      const float t = __fadd_rn(__fsub_rn(q0, s), c);
      const float as = fabsf(s);
      const unsigned bits = __float_as_uint(as);
      const float away = __fsub_rn(__uint_as_float(bits + 1u), as);
      const float toward = __fsub_rn(as, __uint_as_float(bits - 1u));
      const float tp = s < 0.f ? -t : t;
      const float g = __fmul_rn(as, 0x1p-42f);
      if (tp < __fmul_rn(0.5f, away) - g && tp > g - __fmul_rn(0.5f, toward)) return s;
    }
  }
  return div64_slow(d, H.h);
}

// Spacing of one launch: the float32 divisors RN32(2h), RN32(h) (a Python
// float spacing), the float64 divisors 2h, h (a numpy float64 spacing) and
// the float64 h of the metal rule.
struct Spacing {
  double h2, h1;
  Dv d2, d1;
  Dh e2, e1;
  int f64div;
};

__device__ __forceinline__ float grad_div(float d, bool central, const Spacing& s) {
  if (s.f64div) return div64(d, central ? s.e2 : s.e1);
  return div32(d, central ? s.d2 : s.d1);
}

template <bool F64DIV>
__device__ __forceinline__ float grad_div_t(float d, bool central, const Spacing& s) {
  if constexpr (F64DIV)
    return div64(d, central ? s.e2 : s.e1);
  else
    return div32(d, central ? s.d2 : s.d1);
}

// Self-check of the two division emulations against the hardware's IEEE
// divisions: div32 over every float32 bit pattern for one divisor, div64 on
// `samples` hashed inputs (half of them with exponents near the quotient
// range that the fast path serves).
__global__ void k_check_div32(Dv D, unsigned long long* bad) {
  unsigned long long local = 0;
  for (unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
       t < (1ULL << 32); t += (unsigned long long)gridDim.x * blockDim.x) {
    const float d = __uint_as_float((unsigned)t);
    if (!(fabsf(d) <= 3.4028235e38f)) continue;
    if (__float_as_uint(div32(d, D)) != __float_as_uint(__fdiv_rn(d, D.c))) local++;
  }
  if (local) atomicAdd(bad, local);
}

__global__ void k_check_div64(Dh H, unsigned long long samples, unsigned seed,
                              unsigned long long* bad) {
  unsigned long long local = 0;
  for (unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
       t < samples; t += (unsigned long long)gridDim.x * blockDim.x) {
    unsigned x = (unsigned)(t * 2654435761ULL) ^ seed ^ (unsigned)(t >> 32);
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    float d = __uint_as_float(x);
    if (t & 1) d = __uint_as_float((x & 0x807fffffu) | ((97u + (x >> 24) % 62u) << 23));
    if (!(fabsf(d) <= 3.4028235e38f)) continue;
    if (__float_as_uint(div64(d, H)) != __float_as_uint(div64_slow(d, H.h))) local++;
  }
  if (local) atomicAdd(bad, local);
}

constexpr int kBX = 32, kBY = 8, kPlanes = 8;

// tracer3d._fa3d_correct at one metal node (o = (i, j, k)) for NC
// channels, after the plain gradient was stored there: along each axis with
// vacuum on exactly one side, the field becomes minus the one-sided
// difference into the vacuum divided (float64) by h.
template <int NC>
__device__ __forceinline__ void metal_fix(const float* __restrict__ phi, long long pstride,
                                          const uint8_t* __restrict__ metal, int o, int i, int j,
                                          int k, int nx, int ny, int nz, const Dh& e1,
                                          float* ex, float* ey, float* ez, long long ostride) {
  const int sx = ny * nz, sy = nz;
  const int step[3] = {sx, sy, 1};
  const bool lo[3] = {i > 0, j > 0, k > 0};
  const bool hi[3] = {i + 1 < nx, j + 1 < ny, k + 1 < nz};
  float* out[3] = {ex, ey, ez};
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const bool vp = hi[a] && !metal[o + step[a]];
    const bool vm = lo[a] && !metal[o - step[a]];
    if (vp == vm) continue;
    const int up = vp ? o + step[a] : o;
    const int dn = vp ? o : o - step[a];
    float u[NC], v[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) {
      u[c] = phi[c * pstride + up];
      v[c] = phi[c * pstride + dn];
    }
#pragma unroll
    for (int c = 0; c < NC; c++) out[a][c * ostride + o] = -div64(__fsub_rn(u[c], v[c]), e1);
  }
}

// E = -grad(phi) for float32 potentials, NC channels per thread.  Thread
// (j, k) marches over kPlanes x-planes of the chunk blockIdx.z % nchunks
// for channels [NC*g, NC*g + NC), g = blockIdx.z / nchunks, with the
// x-neighbours in registers; the y/z neighbours come through L1 from the
// block's own loads.  Every node gets numpy.gradient's value.  Metal nodes
// (one mask byte, read with the potentials) are queued in shared memory
// and, after the block's gradient is stored, the whole block applies
// metal_fix to the queue, so a lone metal lane (a box face across the
// contiguous axis) does not hold its warp.  In-channel offsets are 32-bit
// (the host checks nx*ny*nz + 2*ny*nz < 2^31).
template <int NC, bool F64DIV>
__global__ void __launch_bounds__(kBX * kBY)
k_field32(const float* __restrict__ phi, long long pstride, const uint8_t* __restrict__ metal,
          int nx, int ny, int nz, Spacing sp, int nchunks, float* __restrict__ ex,
          float* __restrict__ ey, float* __restrict__ ez, long long ostride) {
  __shared__ unsigned short queue[kBX * kBY * kPlanes];
  __shared__ int queued;
  const int k = blockIdx.x * kBX + threadIdx.x;
  const int j = blockIdx.y * kBY + threadIdx.y;
  const int g = blockIdx.z / nchunks;
  const int i0 = (blockIdx.z % nchunks) * kPlanes;
  const int i1 = min(i0 + kPlanes, nx);
  if (threadIdx.x == 0 && threadIdx.y == 0) queued = 0;
  __syncthreads();
  const int sx = ny * nz, sy = nz;
  const float* p = phi + (long long)g * NC * pstride;
  const long long ob = (long long)g * NC * ostride;
  if (k < nz && j < ny && i0 < nx) {
    const bool jlo = j > 0, jhi = j + 1 < ny, klo = k > 0, khi = k + 1 < nz;
    const bool ycen = jlo && jhi, zcen = klo && khi;
    int o = i0 * sx + j * sy + k;
    float vm[NC], vc[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) {
      vm[c] = i0 > 0 ? p[c * pstride + o - sx] : 0.f;
      vc[c] = p[c * pstride + o];
    }
    for (int i = i0; i < i1; i++, o += sx) {
      float vp[NC], ya[NC], yb[NC], za[NC], zb[NC];
#pragma unroll
      for (int c = 0; c < NC; c++) {
        const float* q = p + c * pstride + o;
        vp[c] = i + 1 < nx ? q[sx] : 0.f;
        ya[c] = jlo ? q[-sy] : vc[c];
        yb[c] = jhi ? q[sy] : vc[c];
        za[c] = klo ? q[-1] : vc[c];
        zb[c] = khi ? q[1] : vc[c];
      }
      if (metal && metal[o])
        queue[atomicAdd(&queued, 1)] =
            (unsigned short)(((i - i0) << 8) | (threadIdx.y << 5) | threadIdx.x);
      const bool xcen = i > 0 && i + 1 < nx;
#pragma unroll
      for (int c = 0; c < NC; c++) {
        // numpy.gradient: (up - down) / 2h inside, one-sided / h at the
        // faces (the missing y/z neighbour was replaced by the node itself
        // above; x takes a branch that is uniform over the block).
        float dx;
        if (xcen)
          dx = grad_div_t<F64DIV>(__fsub_rn(vp[c], vm[c]), true, sp);
        else
          dx = grad_div_t<F64DIV>(i == 0 ? __fsub_rn(vp[c], vc[c]) : __fsub_rn(vc[c], vm[c]),
                                  false, sp);
        const float dy = grad_div_t<F64DIV>(__fsub_rn(yb[c], ya[c]), ycen, sp);
        const float dz = grad_div_t<F64DIV>(__fsub_rn(zb[c], za[c]), zcen, sp);
        const long long w = ob + c * ostride + o;
        __stcs(ex + w, -dx);
        __stcs(ey + w, -dy);
        __stcs(ez + w, -dz);
        vm[c] = vc[c];
        vc[c] = vp[c];
      }
    }
  }
  if (!metal) return;  // uniform over the grid
  __syncthreads();
  const int nq = queued;
  for (int t = threadIdx.y * kBX + threadIdx.x; t < nq; t += kBX * kBY) {
    const unsigned e = queue[t];
    const int mi = i0 + (int)(e >> 8), mj = blockIdx.y * kBY + (int)((e >> 5) & 7),
              mk = blockIdx.x * kBX + (int)(e & 31);
    metal_fix<NC>(p, pstride, metal, mi * sx + mj * sy + mk, mi, mj, mk, nx, ny, nz, sp.e1,
                  ex + ob, ey + ob, ez + ob, ostride);
  }
}

// E = -grad(phi) for float64 potentials (and for float32 grids of 2^31
// nodes or more): one channel per blockIdx.z / nchunks, 64-bit offsets.
__device__ __forceinline__ double d64_central(double a, double b, const Spacing& s) {
  return __ddiv_rn(__dsub_rn(a, b), s.h2);
}
__device__ __forceinline__ double d64_edge(double a, double b, const Spacing& s) {
  return __ddiv_rn(__dsub_rn(a, b), s.h1);
}
__device__ __forceinline__ float d32_central(float a, float b, const Spacing& s) {
  return grad_div(__fsub_rn(a, b), true, s);
}
__device__ __forceinline__ float d32_edge(float a, float b, const Spacing& s) {
  return grad_div(__fsub_rn(a, b), false, s);
}
__device__ __forceinline__ double onesided(double a, double b, const Spacing& s) {
  return __ddiv_rn(__dsub_rn(a, b), s.h1);
}
__device__ __forceinline__ float onesided(float a, float b, const Spacing& s) {
  return div64(__fsub_rn(a, b), s.e1);
}
__device__ __forceinline__ double central(double a, double b, const Spacing& s) {
  return d64_central(a, b, s);
}
__device__ __forceinline__ float central(float a, float b, const Spacing& s) {
  return d32_central(a, b, s);
}
__device__ __forceinline__ double edge(double a, double b, const Spacing& s) {
  return d64_edge(a, b, s);
}
__device__ __forceinline__ float edge(float a, float b, const Spacing& s) {
  return d32_edge(a, b, s);
}

template <typename T>
__device__ __forceinline__ T axis_deriv(T vm, T vc, T vp, long q, long n, const Spacing& s,
                                        bool metal, bool vac_p, bool vac_m) {
  T d;
  if (q == 0)
    d = edge(vp, vc, s);
  else if (q == n - 1)
    d = edge(vc, vm, s);
  else
    d = central(vp, vm, s);
  if (metal) {
    if (vac_p && !vac_m)
      d = onesided(vp, vc, s);
    else if (vac_m && !vac_p)
      d = onesided(vc, vm, s);
  }
  return d;
}

constexpr int kIChunk = 16;

template <typename T>
__global__ void __launch_bounds__(kBX * kBY)
k_field(const T* __restrict__ phi, long long pstride, const uint8_t* __restrict__ metal,
        long nx, long ny, long nz, Spacing sp, int nchunks, T* __restrict__ ex,
        T* __restrict__ ey, T* __restrict__ ez, long long ostride) {
  const long k = (long)blockIdx.x * kBX + threadIdx.x;
  const long j = (long)blockIdx.y * kBY + threadIdx.y;
  const int ch = blockIdx.z / nchunks;
  const long i0 = (long)(blockIdx.z % nchunks) * kIChunk;
  if (k >= nz || j >= ny || i0 >= nx) return;
  const long i1 = i0 + kIChunk < nx ? i0 + kIChunk : nx;
  const T* p = phi + ch * pstride;
  T* oxp = ex + ch * ostride;
  T* oyp = ey + ch * ostride;
  T* ozp = ez + ch * ostride;
  const long long sx = (long long)ny * nz, sy = nz;
  long long o = (long long)i0 * sx + (long long)j * sy + k;
  T vm = i0 > 0 ? p[o - sx] : T(0);
  T vc = p[o];
  for (long i = i0; i < i1; i++, o += sx) {
    const T vp = i + 1 < nx ? p[o + sx] : T(0);
    const bool m = metal && metal[o];
    bool xp = false, xm = false, yp = false, ym = false, zp = false, zm = false;
    if (m) {
      xp = i + 1 < nx && !metal[o + sx];
      xm = i > 0 && !metal[o - sx];
      yp = j + 1 < ny && !metal[o + sy];
      ym = j > 0 && !metal[o - sy];
      zp = k + 1 < nz && !metal[o + 1];
      zm = k > 0 && !metal[o - 1];
    }
    const T ym_v = j > 0 ? p[o - sy] : T(0);
    const T yp_v = j + 1 < ny ? p[o + sy] : T(0);
    const T zm_v = k > 0 ? p[o - 1] : T(0);
    const T zp_v = k + 1 < nz ? p[o + 1] : T(0);
    oxp[o] = -axis_deriv<T>(vm, vc, vp, i, nx, sp, m, xp, xm);
    oyp[o] = -axis_deriv<T>(ym_v, vc, yp_v, j, ny, sp, m, yp, ym);
    ozp[o] = -axis_deriv<T>(zm_v, vc, zp_v, k, nz, sp, m, zp, zm);
    vm = vc;
    vc = vp;
  }
}

inline unsigned grid_for(long long n) {
  long long b = (n + 255) / 256;
  const long long cap = 152LL * 8;  // 8 resident 256-thread blocks per SM
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

template <int NCH>
void launch_sup(bool vec, long long n, const SupPlan& p, float* out, long long ostride,
                cudaStream_t st) {
  const unsigned grid = 152u * 32u;   // 32 resident-capable blocks per SM, grid-stride
  if (vec) {
    const long long n4 = n / 4;
    if (n4 > 0) k_superpose<NCH, true><<<grid, 256, 0, st>>>(0, n4, p, out, ostride);
    if (n4 * 4 < n) k_superpose<NCH, false><<<1, 256, 0, st>>>(n4 * 4, n, p, out, ostride);
  } else {
    k_superpose<NCH, false><<<grid, 256, 0, st>>>(0, n, p, out, ostride);
  }
}

// One launch per (<= kMaxCh channels) x (<= kMaxSteps steps) block of the
// plan; later step blocks continue the float32 accumulators in `out`.
int superpose(const float* const* src, int n_steps, int n_channels, const float* weights,
              const uint8_t* mult, long long n, float* out, long long ostride,
              cudaStream_t st) {
  bool vec = ostride % 4 == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0;
  for (int s = 0; s < n_steps; s++)
    vec = vec && (reinterpret_cast<uintptr_t>(src[s]) & 15) == 0;
  long launches = 0;
  for (int c0 = 0; c0 < n_channels; c0 += kMaxCh) {
    const int nch = n_channels - c0 < kMaxCh ? n_channels - c0 : kMaxCh;
    // zero steps: still one launch so the channel is written (all +0)
    for (int s0 = 0; s0 == 0 || s0 < n_steps; s0 += kMaxSteps) {
      SupPlan p{};
      p.nsteps = n_steps - s0 < kMaxSteps ? n_steps - s0 : kMaxSteps;
      if (p.nsteps < 0) p.nsteps = 0;
      p.nch = nch;
      p.accumulate = s0 > 0;
      for (int s = 0; s < p.nsteps; s++) {
        p.src[s] = src[s0 + s];
        for (int c = 0; c < nch; c++) {
          p.w[c][s] = weights[(size_t)(c0 + c) * n_steps + s0 + s];
          p.mult[c][s] = mult[(size_t)(c0 + c) * n_steps + s0 + s];
        }
      }
      float* o = out + (long long)c0 * ostride;
      switch (nch) {
        case 1: launch_sup<1>(vec, n, p, o, ostride, st); break;
        case 2: launch_sup<2>(vec, n, p, o, ostride, st); break;
        case 3: launch_sup<3>(vec, n, p, o, ostride, st); break;
        case 4: launch_sup<4>(vec, n, p, o, ostride, st); break;
        case 5: launch_sup<5>(vec, n, p, o, ostride, st); break;
        case 6: launch_sup<6>(vec, n, p, o, ostride, st); break;
        case 7: launch_sup<7>(vec, n, p, o, ostride, st); break;
        default: launch_sup<8>(vec, n, p, o, ostride, st); break;
      }
      launches += (vec && n % 4 != 0 && n >= 4) ? 2 : 1;
      if (n_steps <= 0) break;
    }
  }
  note_launches(launches);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(std::string("superposition launch: ") + cudaGetErrorString(e));
    return IG_CUDA_ERROR;
  }
  return IG_OK;
}

// RN32(1/c): the float nearest 1/c among RN32(RN64(1/c)) and its two
// neighbours (v*c is exact in double, so the comparison is exact).
float nearest_recip(float c) {
  const float y = (float)(1.0 / (double)c);
  const float cand[3] = {std::nextafter(y, 0.0f), y, std::nextafter(y, y > 0 ? 1e30f : -1e30f)};
  float best = y;
  double be = 1e300;
  for (float v : cand) {
    const double e = std::fabs(1.0 - (double)v * (double)c);
    if (e < be) {
      be = e;
      best = v;
    }
  }
  return best;
}

bool in_fast_range(float c) {
  const float a = std::fabs(c);
  return a >= 0x1p-20f && a <= 0x1p20f;
}

Dv make_dv(float c) {
  Dv d;
  d.c = c;
  d.ok = in_fast_range(c) ? 1 : 0;
  d.y = d.ok ? nearest_recip(c) : 0.0f;
  return d;
}

Dh make_dh(double h) {
  Dh d;
  d.h = h;
  d.hh = (float)h;
  d.hl = (float)(h - (double)d.hh);
  d.ok = (h > 0 && in_fast_range(d.hh) && std::isfinite(h)) ? 1 : 0;
  d.rh = d.ok ? nearest_recip(d.hh) : 0.0f;
  d.dh = make_dv(d.hh);
  d.ok = d.ok && d.dh.ok;
  return d;
}

Spacing make_spacing(double h, int h_is_f64) {
  Spacing s;
  s.h2 = 2.0 * h;
  s.h1 = h;
  s.d2 = make_dv((float)(2.0 * h));
  s.d1 = make_dv((float)h);
  s.e2 = make_dh(2.0 * h);
  s.e1 = make_dh(h);
  s.f64div = h_is_f64 ? 1 : 0;
  return s;
}

template <bool F64DIV>
void launch_field32(int nc, dim3 grid, dim3 block, cudaStream_t st, const float* P,
                    long long pstride, const uint8_t* metal, int nx, int ny, int nz,
                    const Spacing& sp, int nchunks, float* X, float* Y, float* Z,
                    long long ostride) {
  switch (nc) {
    case 4:
      k_field32<4, F64DIV><<<grid, block, 0, st>>>(P, pstride, metal, nx, ny, nz, sp, nchunks,
                                                   X, Y, Z, ostride);
      break;
    case 3:
      k_field32<3, F64DIV><<<grid, block, 0, st>>>(P, pstride, metal, nx, ny, nz, sp, nchunks,
                                                   X, Y, Z, ostride);
      break;
    case 2:
      k_field32<2, F64DIV><<<grid, block, 0, st>>>(P, pstride, metal, nx, ny, nz, sp, nchunks,
                                                   X, Y, Z, ostride);
      break;
    default:
      k_field32<1, F64DIV><<<grid, block, 0, st>>>(P, pstride, metal, nx, ny, nz, sp, nchunks,
                                                   X, Y, Z, ostride);
      break;
  }
}

int field(const void* phi, int dtype, long long pstride, int nch, const uint8_t* metal,
          long nx, long ny, long nz, double h, int h_is_f64, void* ex, void* ey, void* ez,
          long long ostride, cudaStream_t st) {
  const Spacing sp = make_spacing(h, h_is_f64);
  const dim3 block(kBX, kBY);
  const long long n = (long long)nx * ny * nz;
  long launches = 0;
  if ((ny + kBY - 1) / kBY > 65535) {
    set_last_error("field: grid too large for one launch (ceil(ny/8) must be <= 65535)");
    return IG_BAD_ARG;
  }
  if (dtype == 0 && n + 2LL * ny * nz < (1LL << 31)) {
    const int nchunks = (int)((nx + kPlanes - 1) / kPlanes);
    const float* P = static_cast<const float*>(phi);
    float* X = static_cast<float*>(ex);
    float* Y = static_cast<float*>(ey);
    float* Z = static_cast<float*>(ez);
    for (int c0 = 0; c0 < nch;) {
      const int left = nch - c0;
      const int nc = left >= 4 ? 4 : left;
      const int groups = nc == 4 ? left / 4 : 1;
      const long long gz = (long long)nchunks * groups;
      if (gz > 65535) {
        set_last_error("field: channels x ceil(nx/8) exceeds one launch (65535)");
        return IG_BAD_ARG;
      }
      const dim3 grid((unsigned)((nz + kBX - 1) / kBX), (unsigned)((ny + kBY - 1) / kBY),
                      (unsigned)gz);
      const float* Pc = P + (long long)c0 * pstride;
      const long long oc = (long long)c0 * ostride;
      if (sp.f64div)
        launch_field32<true>(nc, grid, block, st, Pc, pstride, metal, (int)nx, (int)ny, (int)nz,
                             sp, nchunks, X + oc, Y + oc, Z + oc, ostride);
      else
        launch_field32<false>(nc, grid, block, st, Pc, pstride, metal, (int)nx, (int)ny,
                              (int)nz, sp, nchunks, X + oc, Y + oc, Z + oc, ostride);
      launches++;
      c0 += nc * groups;
    }
  } else {
    const int nchunks = (int)((nx + kIChunk - 1) / kIChunk);
    const long long gz = (long long)nchunks * nch;
    if (gz > 65535) {
      set_last_error("field: channels x ceil(nx/16) exceeds one launch (65535)");
      return IG_BAD_ARG;
    }
    const dim3 grid((unsigned)((nz + kBX - 1) / kBX), (unsigned)((ny + kBY - 1) / kBY),
                    (unsigned)gz);
    if (dtype == 0)
      k_field<float><<<grid, block, 0, st>>>(
          static_cast<const float*>(phi), pstride, metal, nx, ny, nz, sp, nchunks,
          static_cast<float*>(ex), static_cast<float*>(ey), static_cast<float*>(ez), ostride);
    else
      k_field<double><<<grid, block, 0, st>>>(
          static_cast<const double*>(phi), pstride, metal, nx, ny, nz, sp, nchunks,
          static_cast<double*>(ex), static_cast<double*>(ey), static_cast<double*>(ez), ostride);
    launches++;
  }
  note_launches(launches);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(std::string("field launch: ") + cudaGetErrorString(e));
    return IG_CUDA_ERROR;
  }
  return IG_OK;
}

int check_field_args(int dtype, int nch, long nx, long ny, long nz, double h) {
  if (dtype != 0 && dtype != 1) {
    set_last_error("field: dtype must be 0 (float32) or 1 (float64)");
    return IG_BAD_ARG;
  }
  if (nch < 1 || nx < 1 || ny < 1 || nz < 1) {
    set_last_error("field: empty grid or no channel");
    return IG_BAD_ARG;
  }
  if (nx < 2 || ny < 2 || nz < 2) {
    set_last_error("Shape of array too small to calculate a numerical gradient, at least "
                   "(edge_order + 1) elements are required.");
    return IG_BAD_ARG;
  }
  if (!(h == h) || h == 0.0) {
    set_last_error("field: spacing must be a non-zero number");
    return IG_BAD_ARG;
  }
  return IG_OK;
}

int check_plan(int n_steps, const int* rows, int n_channels, const uint8_t* mult, int n_rows) {
  if (n_steps < 0 || n_channels < 1 || (n_steps > 0 && (!rows || !mult))) {
    set_last_error("superposition: invalid plan");
    return IG_BAD_ARG;
  }
  for (int s = 0; s < n_steps; s++)
    if (rows[s] < 0 || (n_rows >= 0 && rows[s] >= n_rows)) {
      set_last_error("superposition: basis row out of range");
      return IG_BAD_ARG;
    }
  return IG_OK;
}

struct Tmp {
  void* p = nullptr;
  ~Tmp() {
    if (p) cudaFree(p);
  }
};

int no_device() {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_last_error("no CUDA device is visible");
    return IG_NO_DEVICE;
  }
  return IG_OK;
}

}  // namespace
}  // namespace ig

using namespace ig;

#define GF(x)                                                            \
  do {                                                                   \
    cudaError_t e_ = (x);                                                \
    if (e_ != cudaSuccess) {                                             \
      set_last_error(std::string(#x) + ": " + cudaGetErrorString(e_));   \
      return IG_CUDA_ERROR;                                              \
    }                                                                    \
  } while (0)

extern "C" int ig_unit_bases_dev(const double* phi, long long n, double v_basis, float* out,
                                 void* stream) {
  set_last_error("");
  if ((!phi || !out) && n > 0) {
    set_last_error("unit bases: null pointer");
    return IG_BAD_ARG;
  }
  if (n <= 0) return IG_OK;
  k_unit_basis<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(phi, n, v_basis,
                                                                           out);
  note_launches(1);
  GF(cudaGetLastError());
  return IG_OK;
}

extern "C" int ig_superpose_dev(const float* const* basis_ptrs, int n_steps, int n_channels,
                                const float* weights, const uint8_t* mult, long long n,
                                float* out, long long out_stride, void* stream) {
  set_last_error("");
  if (n_steps < 0 || n_channels < 1 || (n_steps > 0 && (!basis_ptrs || !weights || !mult))) {
    set_last_error("superposition: invalid plan");
    return IG_BAD_ARG;
  }
  for (int s = 0; s < n_steps; s++)
    if (!basis_ptrs[s]) {
      set_last_error("superposition: null basis pointer");
      return IG_BAD_ARG;
    }
  if (n < 0 || (n > 0 && !out) || out_stride < n) {
    set_last_error("superposition: invalid output or stride");
    return IG_BAD_ARG;
  }
  if (n == 0) return IG_OK;
  return superpose(basis_ptrs, n_steps, n_channels, weights, mult, n, out, out_stride,
                   static_cast<cudaStream_t>(stream));
}

extern "C" int ig_field_aware_dev(const void* phi, int dtype, long long phi_stride,
                                  int n_channels, const uint8_t* metal, long nx, long ny,
                                  long nz, double h, int h_is_f64, void* ex, void* ey, void* ez,
                                  long long out_stride, void* stream) {
  set_last_error("");
  if (int st = check_field_args(dtype, n_channels, nx, ny, nz, h)) return st;
  const long long n = (long long)nx * ny * nz;
  if (!phi || !ex || !ey || !ez || (n_channels > 1 && (phi_stride < n || out_stride < n))) {
    set_last_error("field: invalid buffers or strides");
    return IG_BAD_ARG;
  }
  return field(phi, dtype, phi_stride, n_channels, metal, nx, ny, nz, h, h_is_f64, ex, ey, ez,
               out_stride, static_cast<cudaStream_t>(stream));
}

extern "C" int ig_field_aware_3d(const void* phi, int dtype, const uint8_t* metal, long nx,
                                 long ny, long nz, double h, int h_is_f64, void* ex, void* ey,
                                 void* ez) {
  set_last_error("");
  if (int st = check_field_args(dtype, 1, nx, ny, nz, h)) return st;
  if (!phi || !ex || !ey || !ez) {
    set_last_error("field: null buffer");
    return IG_BAD_ARG;
  }
  if (int st = no_device()) return st;
  const size_t n = (size_t)nx * ny * nz, es = dtype ? 8 : 4;
  Tmp dp, dm, dout;
  GF(cudaMalloc(&dp.p, n * es));
  GF(cudaMemcpy(dp.p, phi, n * es, cudaMemcpyHostToDevice));
  if (metal) {
    GF(cudaMalloc(&dm.p, n));
    GF(cudaMemcpy(dm.p, metal, n, cudaMemcpyHostToDevice));
  }
  GF(cudaMalloc(&dout.p, 3 * n * es));
  char* o = static_cast<char*>(dout.p);
  if (int st = field(dp.p, dtype, (long long)n, 1, static_cast<uint8_t*>(dm.p), nx, ny, nz, h,
                     h_is_f64, o, o + n * es, o + 2 * n * es, (long long)n, nullptr))
    return st;
  GF(cudaMemcpy(ex, o, n * es, cudaMemcpyDeviceToHost));
  GF(cudaMemcpy(ey, o + n * es, n * es, cudaMemcpyDeviceToHost));
  GF(cudaMemcpy(ez, o + 2 * n * es, n * es, cudaMemcpyDeviceToHost));
  return IG_OK;
}

extern "C" int ig_compose_fields(const float* bases, int n_bases, int n_steps, const int* rows,
                                 int n_channels, const float* weights, const uint8_t* mult,
                                 const uint8_t* metal, long nx, long ny, long nz, double h,
                                 int h_is_f64, float* phi_out, float* ex_out, float* ey_out,
                                 float* ez_out) {
  set_last_error("");
  if (int st = check_plan(n_steps, rows, n_channels, mult, n_bases)) return st;
  if (int st = check_field_args(0, n_channels, nx, ny, nz, h)) return st;
  if ((n_bases > 0 && !bases) || !phi_out || !ex_out || !ey_out || !ez_out) {
    set_last_error("compose: null buffer");
    return IG_BAD_ARG;
  }
  if (int st = no_device()) return st;
  const size_t n = (size_t)nx * ny * nz;
  const size_t nc = (size_t)n_channels;
  Tmp db, dm, dphi, de;
  if (n_bases > 0) {
    GF(cudaMalloc(&db.p, (size_t)n_bases * n * 4));
    GF(cudaMemcpy(db.p, bases, (size_t)n_bases * n * 4, cudaMemcpyHostToDevice));
  }
  if (metal) {
    GF(cudaMalloc(&dm.p, n));
    GF(cudaMemcpy(dm.p, metal, n, cudaMemcpyHostToDevice));
  }
  GF(cudaMalloc(&dphi.p, nc * n * 4));
  GF(cudaMalloc(&de.p, 3 * nc * n * 4));
  float* P = static_cast<float*>(dphi.p);
  float* E = static_cast<float*>(de.p);
  std::vector<const float*> src((size_t)n_steps);
  for (int s = 0; s < n_steps; s++) src[s] = static_cast<const float*>(db.p) + (size_t)rows[s] * n;
  if (int st = superpose(src.data(), n_steps, n_channels, weights, mult, (long long)n, P,
                         (long long)n, nullptr))
    return st;
  if (int st = field(P, 0, (long long)n, n_channels, static_cast<uint8_t*>(dm.p), nx, ny, nz, h,
                     h_is_f64, E, E + nc * n, E + 2 * nc * n, (long long)n, nullptr))
    return st;
  GF(cudaMemcpy(phi_out, P, nc * n * 4, cudaMemcpyDeviceToHost));
  GF(cudaMemcpy(ex_out, E, nc * n * 4, cudaMemcpyDeviceToHost));
  GF(cudaMemcpy(ey_out, E + nc * n, nc * n * 4, cudaMemcpyDeviceToHost));
  GF(cudaMemcpy(ez_out, E + 2 * nc * n, nc * n * 4, cudaMemcpyDeviceToHost));
  return IG_OK;
}

extern "C" int ig_field_check_division(double h, unsigned long long samples, unsigned seed,
                                       unsigned long long* mismatches_out) {
  set_last_error("");
  if (!mismatches_out || !(h > 0) || !std::isfinite(h)) {
    set_last_error("division check: h must be a positive finite number");
    return IG_BAD_ARG;
  }
  if (int st = no_device()) return st;
  Tmp bad;
  GF(cudaMalloc(&bad.p, 8));
  GF(cudaMemset(bad.p, 0, 8));
  unsigned long long* b = static_cast<unsigned long long*>(bad.p);
  const Spacing sp = make_spacing(h, 0);
  k_check_div32<<<152 * 32, 256>>>(sp.d1, b);
  k_check_div32<<<152 * 32, 256>>>(sp.d2, b);
  if (samples) {
    k_check_div64<<<152 * 32, 256>>>(sp.e1, samples, seed, b);
    k_check_div64<<<152 * 32, 256>>>(sp.e2, samples, seed ^ 0x9e3779b9u, b);
  }
  note_launches(samples ? 4 : 2);
  GF(cudaGetLastError());
  GF(cudaMemcpy(mismatches_out, b, 8, cudaMemcpyDeviceToHost));
  return IG_OK;
}
