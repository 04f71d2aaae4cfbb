// ig_mixed.cu -- mixed-precision batched solves (FP32 multigrid inside FP64
// iterative refinement) on sm_103a.
//
// Problem: B Dirichlet problems that share one metal mask (the electrode
// bases of a deck, or B voltage sets on one geometry), each solved to an
// absolute accuracy `acc` in the potential:
//
//   phi <- Dirichlet values     (HBM, 64-bit fixed point: units of 2^-56 of
//                                the problem's largest Dirichlet magnitude)
//   repeat:  g32 = -(float) r(phi)          r: the reference's fine-level
//                                           residual (multigrid3d.py:305-354),
//                                           an exact int64 sum, 0 at metal
//            x32 = cg_iters iterations of flexible CG on A x = g (FP32,
//                  A x = sum(nbr x) - 6 x), each preconditioned by one
//                  multigrid V-cycle (block-ANY coarse masks, 13-point
//                  restriction of the colour-0 residual, trilinear
//                  prolongation, red-black Gauss-Seidel, one-CTA bottom)
//            phi += x32;    stop when the geometric tail estimated from
//                           the observed step contraction is below acc
//                           (per problem)
//   (method 0 replaces the CG by `vcycles` plain V-cycles per step)
//
// FP32 data live in a red-black split layout: colour c of row (i, j) holds
// nodes k = 2m + ((i+j+c) & 1) at index m, so one colour's update reads the
// other colour's rows contiguously (the z-neighbours are slots m-1+p, m+p of
// the same row, the x/y-neighbours slot m of the adjacent rows) and writes
// its own rows without touching the other colour: about 13 bytes per node
// update in FP32 against 26 for the natural layout.
//
// Batching: blockIdx.y is the problem index; masks are shared, per-problem
// arrays are strided.  The whole refinement step (CG iterations, FP64
// update, residual) is captured once into a CUDA graph and replayed; the
// host reads only the B step maxima per step.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <vector>
#include <array>
#include <map>
#include <mutex>

#include "ig_common.cuh"
#include "ig_internal.h"
#include "../../include/igsolve.h"

namespace ig {
namespace {

constexpr int kT = 256;
constexpr int kBottomMax = 1024;     // nodes of the coarsest level (one CTA)
constexpr int kBottomThreads = 512;  // k_bottom is always launched with this many
static_assert(kBottomMax % kBottomThreads == 0, "k_bottom: whole nodes per thread");

__device__ __forceinline__ uint32_t fdivu(uint32_t n, const FastDiv& f) {
  return (__umulhi(n, f.m) + n) >> f.s;
}

// Geometry of one level in split layout.
struct SGeo {
  int nx, ny, nz, H;        // H: slots per colour row, (nz + 1) / 2 rounded
                            // up to a multiple of 4 (16-byte aligned rows)
  uint32_t csz;             // nx * ny * H (one colour array)
  uint32_t n;               // nx * ny * nz (natural)
  // per-problem strides of the metal masks (bytes): the split masks of the
  // level and the natural fine mask; 0 when every problem shares one metal
  uint32_t msplit = 0, mnat = 0;
  FastDiv dH, dny, dnz, dH4, dH8;  // dH8: pairs of float4 groups per row
};

SGeo sgeo(const Dims& d) {
  SGeo g;
  g.nx = (int)d.nx;
  g.ny = (int)d.ny;
  g.nz = (int)d.nz;
  g.H = (int)((((d.nz + 1) / 2) + 3) & ~3L);
  g.csz = (uint32_t)(d.nx * d.ny * g.H);
  g.n = (uint32_t)d.n();
  g.dH = FastDiv((uint32_t)g.H);
  g.dH4 = FastDiv((uint32_t)(g.H / 4));
  g.dH8 = FastDiv((uint32_t)((g.H / 4 + 1) / 2));
  g.dny = FastDiv((uint32_t)d.ny);
  g.dnz = FastDiv((uint32_t)d.nz);
  return g;
}

__device__ __forceinline__ int lo_i(int i, int n) { return i > 0 ? i - 1 : (n > 1 ? 1 : i); }
__device__ __forceinline__ int hi_i(int i, int n) { return i < n - 1 ? i + 1 : (n > 1 ? n - 2 : i); }

// split index of natural node (i, j, k): colour and slot
__device__ __forceinline__ uint32_t sidx(const SGeo& g, int i, int j, int k) {
  return ((uint32_t)i * g.ny + j) * g.H + (k >> 1);
}
__device__ __forceinline__ int scol(int i, int j, int k) { return (i + j + k) & 1; }

// Sum of the six neighbours of split slot (i, j, m) of colour c; own = own
// colour array, oth = the other colour's array.  Size-1 axes use the node
// itself (reference even-reflection rule, solver3d.py:156-167).
__device__ __forceinline__ float nbr_sum(const SGeo& g, const float* __restrict__ own,
                                         const float* __restrict__ oth, int i,
                                         int j, int m, int k, uint32_t self) {
  const bool flat = g.nx == 1 || g.ny == 1 || g.nz == 1;
  const float me = flat ? own[self] : 0.f;
  const float xm = g.nx > 1 ? oth[((uint32_t)lo_i(i, g.nx) * g.ny + j) * g.H + m] : me;
  const float xp = g.nx > 1 ? oth[((uint32_t)hi_i(i, g.nx) * g.ny + j) * g.H + m] : me;
  const float ym = g.ny > 1 ? oth[((uint32_t)i * g.ny + lo_i(j, g.ny)) * g.H + m] : me;
  const float yp = g.ny > 1 ? oth[((uint32_t)i * g.ny + hi_i(j, g.ny)) * g.H + m] : me;
  float zm = me, zp = me;
  if (g.nz > 1) {
    const uint32_t row = ((uint32_t)i * g.ny + j) * g.H;
    zm = oth[row + (lo_i(k, g.nz) >> 1)];
    zp = oth[row + (hi_i(k, g.nz) >> 1)];
  }
  return ((xm + xp) + (ym + yp)) + (zm + zp);
}

// ---- FP32 kernels on split arrays (blockIdx.y = problem) ----------------

__device__ __forceinline__ float4 ld4(const float* p) {
  return *reinterpret_cast<const float4*>(p);
}

// Neighbour sums of the four slots m0..m0+3 (k parity p) of row (i, j),
// read from the other colour's array `oth` (grids with no size-1 axis):
// 16-byte loads of the x/y neighbour rows and of the row's own other-colour
// slots.  The z neighbours of slot m (node k = 2m + p) are slots m-1+p and
// m+p of the other colour's row; node 0 reflects k-1 to k+1 (slot 0), node
// nz-1 reflects k+1 to k-1.  The slot past the row's end (p = 1, last
// group) only feeds unused slots, whose results are never kept.  Sum order:
// ((xm + xp) + (ym + yp)) + (zm + zp).
// Values of the other colour's array: plain loads.
struct PlainLd {
  const float* __restrict__ a;
  __device__ __forceinline__ float4 v4(uint32_t o) const { return ld4(a + o); }
  __device__ __forceinline__ float v1(uint32_t o) const { return a[o]; }
};
// Values of the new CG direction z + beta p, formed where they are read
// (the expression k_cg_dir stores).
struct DirLd {
  const float* __restrict__ z;
  const float* __restrict__ p;
  float b;
  __device__ __forceinline__ float4 v4(uint32_t o) const {
    const float4 zz = ld4(z + o), pp = ld4(p + o);
    return make_float4(zz.x + b * pp.x, zz.y + b * pp.y, zz.z + b * pp.z, zz.w + b * pp.w);
  }
  __device__ __forceinline__ float v1(uint32_t o) const { return z[o] + b * p[o]; }
};

template <class L>
__device__ __forceinline__ void nbr4(const L& oth, const SGeo& G, int i, int j, int m0, int p,
                                     uint32_t base, float q[4]) {
  const float4 xm = oth.v4(((uint32_t)lo_i(i, G.nx) * G.ny + j) * G.H + m0);
  const float4 xp = oth.v4(((uint32_t)hi_i(i, G.nx) * G.ny + j) * G.H + m0);
  const float4 ym = oth.v4(((uint32_t)i * G.ny + lo_i(j, G.ny)) * G.H + m0);
  const float4 yp = oth.v4(((uint32_t)i * G.ny + hi_i(j, G.ny)) * G.H + m0);
  const float4 zc = oth.v4(base);
  float z[5];
  if (p == 0) {
    z[0] = m0 > 0 ? oth.v1(base - 1) : zc.x;
    z[1] = zc.x; z[2] = zc.y; z[3] = zc.z; z[4] = zc.w;
  } else {
    z[0] = zc.x; z[1] = zc.y; z[2] = zc.z; z[3] = zc.w;
    z[4] = m0 + 4 < G.H ? oth.v1(base + 4) : 0.f;
  }
  const int utop = G.nz - 1 - p - 2 * m0;  // 2u == utop: node nz-1
  const float sx[4] = {(xm.x + xp.x) + (ym.x + yp.x), (xm.y + xp.y) + (ym.y + yp.y),
                       (xm.z + xp.z) + (ym.z + yp.z), (xm.w + xp.w) + (ym.w + yp.w)};
#pragma unroll
  for (int u = 0; u < 4; u++) q[u] = sx[u] + (z[u] + (2 * u == utop ? z[u] : z[u + 1]));
}

// One float4 group (slots m0..m0+3 of colour c, row ij) of the update.
// FLAT: the grid has a size-1 axis (per-slot neighbour sums).
template <bool FLAT>
__device__ __forceinline__ void gs4_at(float* __restrict__ own, const float* __restrict__ oth,
                                       const float* __restrict__ gp,
                                       const uint8_t* __restrict__ mp, const SGeo& G, int c,
                                       float omega, uint32_t ij, int i, int j, int m0) {
  const int p = (i + j + c) & 1;
  const uint32_t base = ij * (uint32_t)G.H + m0;
  const uchar4 mk = *reinterpret_cast<const uchar4*>(mp + base);
  float q[4];
  // Grids with no size-1 axis take the float4 path for every group, the z
  // faces included, so no warp diverges into a per-slot path at the ends of
  // its rows.  There the loads (in bounds in every group) are issued with
  // the mask's rather than after it, so a group waits for one memory round
  // trip, not two.
  const float4 gg = ld4(gp + base);
  if (!FLAT) nbr4(PlainLd{oth}, G, i, j, m0, p, base, q);
  if (mk.x & mk.y & mk.z & mk.w) return;  // all metal or unused slots
  if (FLAT) {
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int k = 2 * (m0 + u) + p;
      q[u] = k < G.nz ? nbr_sum(G, own, oth, i, j, m0 + u, k, base + u) : 0.f;
    }
  }
  const float gv[4] = {gg.x, gg.y, gg.z, gg.w};
  const uint8_t mv[4] = {mk.x, mk.y, mk.z, mk.w};
  if (omega == 1.0f && (mk.x | mk.y | mk.z | mk.w) == 0) {
    *reinterpret_cast<float4*>(own + base) =
        make_float4((q[0] - gv[0]) * (1.0f / 6.0f), (q[1] - gv[1]) * (1.0f / 6.0f),
                    (q[2] - gv[2]) * (1.0f / 6.0f), (q[3] - gv[3]) * (1.0f / 6.0f));
    return;
  }
#pragma unroll
  for (int u = 0; u < 4; u++) {
    if (mv[u]) continue;
    const float nv = (q[u] - gv[u]) * (1.0f / 6.0f);
    own[base + u] = omega == 1.0f ? nv : own[base + u] + omega * (nv - own[base + u]);
  }
}

template <bool FLAT>
__device__ __forceinline__ void gs4_group(float* __restrict__ own, const float* __restrict__ oth,
                                          const float* __restrict__ gp,
                                          const uint8_t* __restrict__ mp, const SGeo& G,
                                          int c, float omega, uint32_t t) {
  const uint32_t ij = fdivu(t, G.dH4);
  const int m0 = 4 * (int)(t - ij * G.dH4.d);
  const int i = (int)fdivu(ij, G.dny);
  const int j = (int)(ij - (uint32_t)i * G.dny.d);
  gs4_at<FLAT>(own, oth, gp, mp, G, c, omega, ij, i, j, m0);
}

// Red-black Gauss-Seidel half-sweep of colour c on the split layout.  Each
// thread updates NG float4 groups (four consecutive slots of one colour
// row; 16-byte loads of the neighbour rows -- the split layout makes the
// x/y neighbours of slot m the slots m of the adjacent rows, and the z
// neighbours slots m-1+p and m+p of the other colour's own row), the groups
// blockDim apart so every load instruction stays coalesced.  Groups that
// touch a face in z, or grids with a size-1 axis, take the per-slot path.
// NG and the block size are chosen per grid by the session's tuner.
template <int NG, bool FLAT>
__global__ void k_gs4(float* __restrict__ e, const float* __restrict__ g,
                      const uint8_t* __restrict__ mask, SGeo G, int c, float omega,
                      size_t pstride) {
  mask += (size_t)blockIdx.y * G.msplit;
  const uint32_t nq = G.csz >> 2;
  float* eb = e + blockIdx.y * pstride;
  float* own = eb + (size_t)c * G.csz;
  const float* oth = eb + (size_t)(1 - c) * G.csz;
  const float* gp = g + blockIdx.y * pstride + (size_t)c * G.csz;
  const uint8_t* mp = mask + (size_t)c * G.csz;
  const uint32_t t0 = blockIdx.x * blockDim.x * NG + threadIdx.x;
#pragma unroll
  for (int u = 0; u < NG; u++) {
    const uint32_t t = t0 + u * blockDim.x;
    if (t < nq) gs4_group<FLAT>(own, oth, gp, mp, G, c, omega, t);
  }
}

// The same half-sweep with two consecutive float4 groups of one row per
// thread (slots m0..m0+7): one index computation and one mask / z-boundary
// lookup serve eight slots.  A row with an odd number of groups leaves the
// second group of its last pair idle.
template <bool FLAT>
__global__ void k_gs8(float* __restrict__ e, const float* __restrict__ g,
                      const uint8_t* __restrict__ mask, SGeo G, int c, float omega,
                      size_t pstride) {
  mask += (size_t)blockIdx.y * G.msplit;
  const uint32_t H4 = (uint32_t)(G.H >> 2);
  const uint32_t npair = (uint32_t)G.nx * G.ny * G.dH8.d;
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npair) return;
  const uint32_t ij = fdivu(t, G.dH8);
  const uint32_t q0 = 2 * (t - ij * G.dH8.d);
  float* eb = e + blockIdx.y * pstride;
  float* own = eb + (size_t)c * G.csz;
  const float* oth = eb + (size_t)(1 - c) * G.csz;
  const float* gp = g + blockIdx.y * pstride + (size_t)c * G.csz;
  const uint8_t* mp = mask + (size_t)c * G.csz;
  const int i = (int)fdivu(ij, G.dny);
  const int j = (int)(ij - (uint32_t)i * G.dny.d);
  gs4_at<FLAT>(own, oth, gp, mp, G, c, omega, ij, i, j, 4 * (int)q0);
  if (q0 + 1 < H4) gs4_at<FLAT>(own, oth, gp, mp, G, c, omega, ij, i, j, 4 * (int)q0 + 4);
}

// The first Gauss-Seidel pair (omega = 1) of a cycle that starts from e = 0,
// in one pass.  Colour 0 sees zero neighbours, so its new value is
// (0 - g0) / 6 at free nodes and 0 at metal; colour 1 then reads those
// colour-0 values at its six neighbours, which this thread recomputes from
// g0 and the colour-0 mask (five float4 rows and one edge slot, the same
// rows the separate colour-1 launch would read from e).  Every expression
// and its order are those of gs4_at, so the result has the bits of a memset
// and two half-sweeps, at 9 bytes per node (g, mask, both colours of e
// written) instead of 4 + 13.  Grids with a size-1 axis use the separate
// launches.
__device__ __forceinline__ float zero_start_e0(float g, uint8_t m) {
  return m ? 0.f : (0.f - g) * (1.0f / 6.0f);
}
__device__ __forceinline__ float4 zero_start_e0(const float* gp, const uint8_t* mp) {
  const float4 g = ld4(gp);
  const uchar4 m = *reinterpret_cast<const uchar4*>(mp);
  return make_float4(zero_start_e0(g.x, m.x), zero_start_e0(g.y, m.y), zero_start_e0(g.z, m.z),
                     zero_start_e0(g.w, m.w));
}

// The right-hand side a cycle reads: g itself, or (FOLD) g + alpha q -- the
// flexible CG's update of the previous iteration, formed where it is read
// (k_cg_update's expression, so the same bits).
template <bool FOLD>
struct RhsLd {
  const float* __restrict__ g;
  const float* __restrict__ q;
  float al;
  __device__ __forceinline__ float4 v4(uint32_t o) const {
    float4 v = ld4(g + o);
    if (FOLD) {
      const float4 w = ld4(q + o);
      v.x = __fmaf_rn(al, w.x, v.x); v.y = __fmaf_rn(al, w.y, v.y);
      v.z = __fmaf_rn(al, w.z, v.z); v.w = __fmaf_rn(al, w.w, v.w);
    }
    return v;
  }
  __device__ __forceinline__ float v1(uint32_t o) const {
    return FOLD ? __fmaf_rn(al, q[o], g[o]) : g[o];
  }
};
__device__ __forceinline__ float4 zero_start_e0(float4 g, uchar4 m) {
  return make_float4(zero_start_e0(g.x, m.x), zero_start_e0(g.y, m.y), zero_start_e0(g.z, m.z),
                     zero_start_e0(g.w, m.w));
}

// Float4 group t (both colours) of the fused first pair, for one problem:
// e0, g0 and mask its split arrays (colour 1 at + csz).  FOLD: the
// right-hand side is g0 + al q0 (the previous CG iteration's update,
// formed where it is read), and the thread stores it, both colours of its
// slots, to gout (a different array: neighbouring threads still read g0).
template <bool FOLD>
__device__ __forceinline__ void zero_pair_at(float* e0, const float* g0, const uint8_t* mask,
                                             const SGeo& G, uint32_t t,
                                             const float* q0 = nullptr, float al = 0.f,
                                             float* gout = nullptr) {
  const uint32_t ij = fdivu(t, G.dH4);
  const int m0 = 4 * (int)(t - ij * G.dH4.d);
  const int i = (int)fdivu(ij, G.dny);
  const int j = (int)(ij - (uint32_t)i * G.dny.d);
  const uint32_t base = ij * (uint32_t)G.H + m0;
  float* e1 = e0 + G.csz;
  const RhsLd<FOLD> r0{g0, q0, al};
  const RhsLd<FOLD> r1{g0 + G.csz, FOLD ? q0 + G.csz : nullptr, al};
  const uint8_t* k0 = mask;
  const uint8_t* k1 = mask + G.csz;
  auto m4 = [&](uint32_t o) { return *reinterpret_cast<const uchar4*>(k0 + o); };
  // colour 0 of this thread's slots
  const float4 g0own = r0.v4(base);
  const float4 zc = zero_start_e0(g0own, m4(base));
  *reinterpret_cast<float4*>(e0 + base) = zc;
  // colour 1 of this thread's slots, from the colour-0 values around them
  const uint32_t rxm = ((uint32_t)lo_i(i, G.nx) * G.ny + j) * G.H + m0;
  const uint32_t rxp = ((uint32_t)hi_i(i, G.nx) * G.ny + j) * G.H + m0;
  const uint32_t rym = ((uint32_t)i * G.ny + lo_i(j, G.ny)) * G.H + m0;
  const uint32_t ryp = ((uint32_t)i * G.ny + hi_i(j, G.ny)) * G.H + m0;
  const float4 xm = zero_start_e0(r0.v4(rxm), m4(rxm));
  const float4 xp = zero_start_e0(r0.v4(rxp), m4(rxp));
  const float4 ym = zero_start_e0(r0.v4(rym), m4(rym));
  const float4 yp = zero_start_e0(r0.v4(ryp), m4(ryp));
  const int p = (i + j + 1) & 1;
  float z[5];
  if (p == 0) {
    z[0] = m0 > 0 ? zero_start_e0(r0.v1(base - 1), k0[base - 1]) : zc.x;
    z[1] = zc.x; z[2] = zc.y; z[3] = zc.z; z[4] = zc.w;
  } else {
    z[0] = zc.x; z[1] = zc.y; z[2] = zc.z; z[3] = zc.w;
    z[4] = m0 + 4 < G.H ? zero_start_e0(r0.v1(base + 4), k0[base + 4]) : 0.f;
  }
  const int utop = G.nz - 1 - p - 2 * m0;
  const float sx[4] = {(xm.x + xp.x) + (ym.x + yp.x), (xm.y + xp.y) + (ym.y + yp.y),
                       (xm.z + xp.z) + (ym.z + yp.z), (xm.w + xp.w) + (ym.w + yp.w)};
  const float4 gg = r1.v4(base);
  if (FOLD) {
    *reinterpret_cast<float4*>(gout + base) = g0own;
    *reinterpret_cast<float4*>(gout + G.csz + base) = gg;
  }
  const uchar4 mk = *reinterpret_cast<const uchar4*>(k1 + base);
  const float gv[4] = {gg.x, gg.y, gg.z, gg.w};
  const uint8_t mv[4] = {mk.x, mk.y, mk.z, mk.w};
  float o[4];
#pragma unroll
  for (int u = 0; u < 4; u++) {
    const float q = sx[u] + (z[u] + (2 * u == utop ? z[u] : z[u + 1]));
    o[u] = mv[u] ? 0.f : (q - gv[u]) * (1.0f / 6.0f);
  }
  *reinterpret_cast<float4*>(e1 + base) = make_float4(o[0], o[1], o[2], o[3]);
}

__global__ void __launch_bounds__(kT)
k_gs_zero_pair(float* __restrict__ e, const float* __restrict__ g,
               const uint8_t* __restrict__ mask, SGeo G, size_t pstride) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= (G.csz >> 2)) return;
  zero_pair_at<false>(e + blockIdx.y * pstride, g + blockIdx.y * pstride,
                      mask + (size_t)blockIdx.y * G.msplit, G, t);
}

// k_gs_zero_pair on the finest level of a flexible-CG step's later
// iterations: the right-hand side g + alpha q (alpha = scal[4b + 1], the
// previous iteration's step) is formed where it is read and stored to
// gout, which the rest of the iteration reads as its right-hand side --
// the g half of k_cg_update folded in.
__global__ void __launch_bounds__(kT)
k_gs_zero_pair_fold(float* __restrict__ e, const float* __restrict__ g,
                    const float* __restrict__ q, const double* __restrict__ scal,
                    float* __restrict__ gout, const uint8_t* __restrict__ mask, SGeo G,
                    size_t pstride) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= (G.csz >> 2)) return;
  const size_t o = blockIdx.y * pstride;
  zero_pair_at<true>(e + o, g + o, mask + (size_t)blockIdx.y * G.msplit, G, t, q + o,
                     (float)scal[4 * blockIdx.y + 1], gout + o);
}

// ---- temporal blocking: S red-black half-sweeps in one pass -----------------
//
// The fine level's Gauss-Seidel half-sweeps (omega 1) of one smoothing phase
// of the V-cycle run in one launch.  With omega 1 a half-sweep of colour c
// reads only the other colour, so S alternating half-sweeps read one colour
// of e once, g and the mask, and write e once: 11 bytes per node for any S
// (9 when the phase starts from e = 0), against 6.5 per half-sweep.
//
// A CTA owns a tile of TY rows (j) by TMG float4 groups of slots (the split
// layout's rows, both colours) and marches through the x-planes.  Stage s
// (1..S) updates colour c_s = C1 ^ ((s - 1) & 1) on plane t - s + 1 at
// iteration t: each stage lags the one before by one plane, so the planes
// i - 1, i, i + 1 of stage s - 1 that stage s reads at plane i are all
// done.  A thread keeps one float4 position (row j, group gi) through every
// stage: the x-neighbours of its position are its own results of the stage
// before (a three-plane register window per stage), the y-neighbours and the
// z-edge slots come from the neighbouring positions through shared memory,
// where every stage publishes the plane it just computed.  Stage s reads the
// previous iteration's publication (parity t - 1) and writes parity t, so one
// barrier per plane orders everything.  The tile carries a halo of S rows
// and S groups on each side, shrinking by one per stage, so the last stage
// covers exactly the tile.  Faces reflect as in the separate kernels
// (lo_i / hi_i in y and x, the z-face rules of nbr4).
//
// Every node's update is the expression of gs4_at (the same neighbour sum
// order, (q - g) * (1/6), 0 at metal and unused slots), so the result has
// the bits of the S separate launches (checked by ig_mixed_check_fused).
// ZERO: the phase starts from e = 0 (colour C1 = 0 first, as the cycle's
// zero-start pair): nothing of e is read and the first stage is -g/6.
// Otherwise the kernel reads colour 1 - C1 of `ein` and writes both colours
// of the result to `eout`, a different array (tiles read their halo from
// `ein` while neighbouring tiles write their output).
template <int S, int TY, int TMG>
struct TbShape {
  static constexpr int R = TY + 2 * S, GR = TMG + 2 * S, NT = R * GR;
  static constexpr size_t smem = (size_t)S * 2 * NT * sizeof(float4);
};

__device__ __forceinline__ float4 gs_update4(float4 xm, float4 xp, float4 ym, float4 yp,
                                             float4 zc, float z0, float z4, int p, int utop,
                                             float4 gg, uchar4 mk) {
  if (mk.x & mk.y & mk.z & mk.w) return make_float4(0.f, 0.f, 0.f, 0.f);
  float z[5];
  if (p == 0) {
    z[0] = z0; z[1] = zc.x; z[2] = zc.y; z[3] = zc.z; z[4] = zc.w;
  } else {
    z[0] = zc.x; z[1] = zc.y; z[2] = zc.z; z[3] = zc.w; z[4] = z4;
  }
  const float sx[4] = {(xm.x + xp.x) + (ym.x + yp.x), (xm.y + xp.y) + (ym.y + yp.y),
                       (xm.z + xp.z) + (ym.z + yp.z), (xm.w + xp.w) + (ym.w + yp.w)};
  const float gv[4] = {gg.x, gg.y, gg.z, gg.w};
  const uint8_t mv[4] = {mk.x, mk.y, mk.z, mk.w};
  float o[4];
#pragma unroll
  for (int u = 0; u < 4; u++) {
    const float q = sx[u] + (z[u] + (2 * u == utop ? z[u] : z[u + 1]));
    o[u] = mv[u] ? 0.f : (q - gv[u]) * (1.0f / 6.0f);
  }
  return make_float4(o[0], o[1], o[2], o[3]);
}

template <int S, bool ZERO, int C1, int TY, int TMG, int MINB>
__global__ void __launch_bounds__(TbShape<S, TY, TMG>::NT, MINB)
k_gs_tb(const float* __restrict__ ein, float* __restrict__ eout, const float* __restrict__ g,
        const uint8_t* __restrict__ mask, SGeo G, size_t pstride) {
  mask += (size_t)blockIdx.y * G.msplit;
  using Sh = TbShape<S, TY, TMG>;
  constexpr int R = Sh::R, GR = Sh::GR, NT = Sh::NT;
  extern __shared__ float4 tb_sm[];  // [stage 0..S-1][parity][NT]; stage 0 = input
  const int tid = threadIdx.x;
  const int r = tid / GR, q = tid - r * GR;
  const int H4 = G.H >> 2;
  const int ntj = (G.ny + TY - 1) / TY;
  const int tj = (int)(blockIdx.x % (unsigned)ntj), tg = (int)(blockIdx.x / (unsigned)ntj);
  const int j0 = tj * TY, g0 = tg * TMG;
  const int j = j0 - S + r, gi = g0 - S + q;
  const bool indom = j >= 0 && j < G.ny && gi >= 0 && gi < H4;
  const int m0 = 4 * gi;
  const size_t pb = (size_t)blockIdx.y * pstride;
  const uint32_t rowstride = (uint32_t)G.ny * (uint32_t)G.H;
  // shared-memory rows of the y-neighbours (faces reflect into the tile)
  const int rlo = indom ? lo_i(j, G.ny) - (j0 - S) : r;
  const int rhi = indom ? hi_i(j, G.ny) - (j0 - S) : r;
  float4 cur[S], prv[S], pp[S];  // stage s outputs (s = 0: input) at planes t-s+1, t-s, t-s-1
#pragma unroll
  for (int s = 0; s < S; s++)
    cur[s] = prv[s] = pp[s] = make_float4(0.f, 0.f, 0.f, 0.f);
  const int cin = 1 - C1;  // the colour the first stage reads
  if (!ZERO && indom) {   // plane 0 of the input
    cur[0] = ld4(ein + pb + (size_t)cin * G.csz + (uint32_t)j * G.H + m0);
  }
  if (!ZERO) tb_sm[(0 * 2 + 1) * NT + tid] = cur[0];
  __syncthreads();
  const int last = G.nx - 1 + S - 1;
  for (int t = 0; t <= last; t++) {
    const int rd = (t - 1) & 1, wr = t & 1;
    if (!ZERO) {
      pp[0] = prv[0];
      prv[0] = cur[0];
      cur[0] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (indom && t + 1 < G.nx)
        cur[0] = ld4(ein + pb + (size_t)cin * G.csz + (uint32_t)(t + 1) * rowstride +
                     (uint32_t)j * G.H + m0);
      tb_sm[(0 * 2 + wr) * NT + tid] = cur[0];
    }
    float4 out_last = make_float4(0.f, 0.f, 0.f, 0.f);
    // every stage's right-hand side and mask of this iteration, issued
    // together before any stage computes (they depend on nothing computed)
    float4 gq[S];
    uchar4 mq[S];
#pragma unroll
    for (int s = 1; s <= S; s++) {
      const int c = C1 ^ ((s - 1) & 1);
      const int i = t - s + 1;
      const bool act = indom && i >= 0 && i < G.nx && r >= s && r < R - s && q >= s &&
                       q < GR - s;
      gq[s - 1] = make_float4(0.f, 0.f, 0.f, 0.f);
      mq[s - 1] = make_uchar4(1, 1, 1, 1);
      if (act) {
        const uint32_t off = (uint32_t)i * rowstride + (uint32_t)j * G.H + m0;
        gq[s - 1] = ld4(g + pb + (size_t)c * G.csz + off);
        mq[s - 1] = *reinterpret_cast<const uchar4*>(mask + (size_t)c * G.csz + off);
      }
    }
#pragma unroll
    for (int s = 1; s <= S; s++) {
      const int c = C1 ^ ((s - 1) & 1);
      const int i = t - s + 1;
      const bool act = indom && i >= 0 && i < G.nx && r >= s && r < R - s && q >= s &&
                       q < GR - s;
      float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
      if (act) {
        const float4 gg = gq[s - 1];
        const uchar4 mk = mq[s - 1];
        const int p = (i + j + c) & 1;
        const int utop = G.nz - 1 - p - 2 * m0;
        if (ZERO && s == 1) {
          // e = 0 before the phase: colour 0 is -g/6 at free slots
          o = make_float4(zero_start_e0(gg.x, mk.x), zero_start_e0(gg.y, mk.y),
                          zero_start_e0(gg.z, mk.z), zero_start_e0(gg.w, mk.w));
        } else {
          const int sp = s - 1;
          const float4* src = tb_sm + (size_t)(sp * 2 + rd) * NT;
          const float4 xm = i > 0 ? pp[sp] : cur[sp];
          const float4 xp = i < G.nx - 1 ? cur[sp] : pp[sp];
          const float4 zc = prv[sp];
          const float4 ym = src[rlo * GR + q];
          const float4 yp = src[rhi * GR + q];
          const float z0 = p == 0 ? (m0 > 0 ? src[r * GR + q - 1].w : zc.x) : 0.f;
          const float z4 = p == 1 ? (m0 + 4 < G.H ? src[r * GR + q + 1].x : 0.f) : 0.f;
          o = gs_update4(xm, xp, ym, yp, zc, z0, z4, p, utop, gg, mk);
        }
      }
      if (s < S) {
        pp[s] = prv[s];
        prv[s] = cur[s];
        cur[s] = o;
        tb_sm[(size_t)(s * 2 + wr) * NT + tid] = o;
      } else {
        out_last = o;
      }
    }
    // the finished plane: colour c_S from the last stage, colour c_{S-1}
    // from the stage before (its previous plane)
    const int io = t - S + 1;
    if (indom && io >= 0 && r >= S && r < S + TY && q >= S && q < S + TMG) {
      const int cS = C1 ^ ((S - 1) & 1);
      const uint32_t off = (uint32_t)io * rowstride + (uint32_t)j * G.H + m0;
      *reinterpret_cast<float4*>(eout + pb + (size_t)cS * G.csz + off) = out_last;
      *reinterpret_cast<float4*>(eout + pb + (size_t)(1 - cS) * G.csz + off) = prv[S - 1];
    }
    __syncthreads();
  }
}

// Launches the fused smoothing phase of S half-sweeps on level a (S = 2, 4,
// 6).  zero: the phase starts from e = 0 (colours 0, 1, ...), writing ein
// itself; otherwise colours 1, 0, ... from ein into eout.
// Tile of each phase length: TY rows by TG float4 groups, MB CTAs per SM.
template <int S> struct TbTile { static constexpr int TY = 8, TG = 8, MB = 2; };
template <> struct TbTile<6> { static constexpr int TY = 8, TG = 16, MB = 1; };

template <int S, bool ZERO, int C1>
void launch_tb_t(const float* ein, float* eout, const float* g, const uint8_t* mask,
                 const SGeo& G, size_t pstride, int nb, cudaStream_t s) {
  constexpr int TY = TbTile<S>::TY, TG = TbTile<S>::TG;
  using Sh = TbShape<S, TY, TG>;
  const unsigned ntj = (unsigned)((G.ny + TY - 1) / TY);
  const unsigned ntg = (unsigned)(((G.H >> 2) + TG - 1) / TG);
  k_gs_tb<S, ZERO, C1, TY, TG, TbTile<S>::MB><<<dim3(ntj * ntg, nb), Sh::NT, Sh::smem, s>>>(
      ein, eout, g, mask, G, pstride);
}

template <int S, bool ZERO, int C1>
cudaError_t tb_attr() {
  constexpr int TY = TbTile<S>::TY, TG = TbTile<S>::TG;
  return cudaFuncSetAttribute(k_gs_tb<S, ZERO, C1, TY, TG, TbTile<S>::MB>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)TbShape<S, TY, TG>::smem);
}

// The blocked kernels' dynamic shared memory (above the default 48 KB) is
// enabled once, outside any stream capture.
cudaError_t tb_prepare() {
  cudaError_t e = cudaSuccess;
  for (cudaError_t x : {tb_attr<2, true, 0>(), tb_attr<4, true, 0>(), tb_attr<6, true, 0>(),
                        tb_attr<2, false, 1>(), tb_attr<4, false, 1>(),
                        tb_attr<6, false, 1>(), tb_attr<2, false, 0>(),
                        tb_attr<4, false, 0>(), tb_attr<6, false, 0>()})
    if (x != cudaSuccess) e = x;
  return e;
}

// c1: the first stage's colour (0 when zero).
void launch_tb(int S, bool zero, int c1, const float* ein, float* eout, const float* g,
               const uint8_t* mask, const SGeo& G, size_t pstride, int nb, cudaStream_t s) {
  if (zero) {
    if (S == 2) launch_tb_t<2, true, 0>(ein, eout, g, mask, G, pstride, nb, s);
    else if (S == 4) launch_tb_t<4, true, 0>(ein, eout, g, mask, G, pstride, nb, s);
    else launch_tb_t<6, true, 0>(ein, eout, g, mask, G, pstride, nb, s);
  } else if (c1 == 1) {
    if (S == 2) launch_tb_t<2, false, 1>(ein, eout, g, mask, G, pstride, nb, s);
    else if (S == 4) launch_tb_t<4, false, 1>(ein, eout, g, mask, G, pstride, nb, s);
    else launch_tb_t<6, false, 1>(ein, eout, g, mask, G, pstride, nb, s);
  } else {
    if (S == 2) launch_tb_t<2, false, 0>(ein, eout, g, mask, G, pstride, nb, s);
    else if (S == 4) launch_tb_t<4, false, 0>(ein, eout, g, mask, G, pstride, nb, s);
    else launch_tb_t<6, false, 0>(ein, eout, g, mask, G, pstride, nb, s);
  }
}

// Number of 32-bit words that differ between a and b (a check of the fused
// kernels against their separate launches).
__global__ void __launch_bounds__(kT)
k_count_diff(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, size_t n,
             unsigned long long* bad) {
  const size_t t = (size_t)blockIdx.x * kT + threadIdx.x;
  const unsigned d = __syncthreads_count(t < n && a[t] != b[t]);
  if (threadIdx.x == 0 && d) atomicAdd(bad, (unsigned long long)d);
}

// Residual r = g - A e of colour 0 only, in split layout.  After a red-black
// Gauss-Seidel pair that ended on colour 1 the residual of colour 1 is zero
// (each colour-1 node was just solved exactly against its neighbours), so
// colour 0 carries the whole residual.
__global__ void __launch_bounds__(kT)
k_resid0(const float* __restrict__ e, const float* __restrict__ g,
         const uint8_t* __restrict__ mask, SGeo G, float* __restrict__ r,
         size_t pstride) {
  mask += (size_t)blockIdx.y * G.msplit;
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= G.csz) return;
  const uint32_t ij = fdivu(t, G.dH);
  const int m = (int)(t - ij * G.dH.d);
  const int i = (int)fdivu(ij, G.dny);
  const int j = (int)(ij - (uint32_t)i * G.dny.d);
  const int k = 2 * m + ((i + j) & 1);
  float out = 0.f;
  if (k < G.nz && !mask[t]) {
    const float* eb = e + blockIdx.y * pstride;
    const float a = nbr_sum(G, eb, eb + G.csz, i, j, m, k, t) - 6.0f * eb[t];
    out = g[blockIdx.y * pstride + t] - a;
  }
  r[blockIdx.y * (size_t)G.csz + t] = out;
}

// k_resid0 over float4 groups (grids with no size-1 axis): the same
// expressions per slot, 16-byte loads of the colour-1 neighbour rows, one
// float4 store of r.
// Float4 group t of the colour-0 residual, one problem: eb, gb, mask its
// split arrays, rb its colour-0 residual (csz floats).
__device__ __forceinline__ void resid0_4_at(const float* eb, const float* gb,
                                            const uint8_t* mask, const SGeo& G, float* rb,
                                            uint32_t t) {
  const uint32_t ij = fdivu(t, G.dH4);
  const int m0 = 4 * (int)(t - ij * G.dH4.d);
  const int i = (int)fdivu(ij, G.dny);
  const int j = (int)(ij - (uint32_t)i * G.dny.d);
  const uint32_t base = ij * (uint32_t)G.H + m0;
  float4* out = reinterpret_cast<float4*>(rb + base);
  // no early exit on an all-metal group: the loads are in bounds in every
  // group and go out with the mask's; metal slots select 0 below
  const uchar4 mk = *reinterpret_cast<const uchar4*>(mask + base);
  float q[4];
  nbr4(PlainLd{eb + G.csz}, G, i, j, m0, (i + j) & 1, base, q);
  const float4 ev = ld4(eb + base), gg = ld4(gb + base);
  const float es[4] = {ev.x, ev.y, ev.z, ev.w}, gv[4] = {gg.x, gg.y, gg.z, gg.w};
  const uint8_t mv[4] = {mk.x, mk.y, mk.z, mk.w};
  float o[4];
#pragma unroll
  for (int u = 0; u < 4; u++) {
    const float a = q[u] - 6.0f * es[u];
    o[u] = mv[u] ? 0.f : gv[u] - a;
  }
  *out = make_float4(o[0], o[1], o[2], o[3]);
}

__global__ void __launch_bounds__(kT)
k_resid0_4(const float* __restrict__ e, const float* __restrict__ g,
           const uint8_t* __restrict__ mask, SGeo G, float* __restrict__ r,
           size_t pstride) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= (G.csz >> 2)) return;
  resid0_4_at(e + blockIdx.y * pstride, g + blockIdx.y * pstride,
              mask + (size_t)blockIdx.y * G.msplit, G, r + blockIdx.y * (size_t)G.csz, t);
}

// 4 x full weighting when only colour 0 of the fine residual is nonzero:
// around a coarse node (fine centre 2c, colour 0) the colour-0 points are
// the centre (weight 1) and the 12 edge neighbours (weight 1/4); the faces
// and corners are colour 1.  Clamped edges as in the 27-point form.
__global__ void __launch_bounds__(kT)
k_restrict0(const float* __restrict__ r0, SGeo F, float* __restrict__ gc, SGeo C,
            size_t cstride) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= C.n) return;
  const uint32_t ij = fdivu(t, C.dnz);
  const int kc = (int)(t - ij * C.dnz.d);
  const int ic = (int)fdivu(ij, C.dny);
  const int jc = (int)(ij - (uint32_t)ic * C.dny.d);
  const float* rb = r0 + blockIdx.y * (size_t)F.csz;
  float acc = 0.f;
#pragma unroll
  for (int di = -1; di <= 1; di++) {
    const int ii = min(max(2 * ic + di, 0), F.nx - 1);
    const float wi = di == 0 ? 1.f : 0.5f;
#pragma unroll
    for (int dj = -1; dj <= 1; dj++) {
      const int jj = min(max(2 * jc + dj, 0), F.ny - 1);
      const float wj = dj == 0 ? 1.f : 0.5f;
#pragma unroll
      for (int dk = -1; dk <= 1; dk++) {
        const int kk = min(max(2 * kc + dk, 0), F.nz - 1);
        if ((ii + jj + kk) & 1) continue;   // colour 1: zero residual
        const float wk = dk == 0 ? 1.f : 0.5f;
        acc += wi * wj * wk * rb[sidx(F, ii, jj, kk)];
      }
    }
  }
  const int c = scol(ic, jc, kc);
  gc[blockIdx.y * cstride + (size_t)c * C.csz + sidx(C, ic, jc, kc)] = 0.5f * acc;
}

// The 13-tap sum of one coarse node (k_restrict0's loop).
__device__ __forceinline__ float restrict0_node(const float* __restrict__ rb, const SGeo& F,
                                                int ic, int jc, int kc) {
  float acc = 0.f;
#pragma unroll
  for (int di = -1; di <= 1; di++) {
    const int ii = min(max(2 * ic + di, 0), F.nx - 1);
    const float wi = di == 0 ? 1.f : 0.5f;
#pragma unroll
    for (int dj = -1; dj <= 1; dj++) {
      const int jj = min(max(2 * jc + dj, 0), F.ny - 1);
      const float wj = dj == 0 ? 1.f : 0.5f;
#pragma unroll
      for (int dk = -1; dk <= 1; dk++) {
        const int kk = min(max(2 * kc + dk, 0), F.nz - 1);
        if ((ii + jj + kk) & 1) continue;
        const float wk = dk == 0 ? 1.f : 0.5f;
        acc += wi * wj * wk * rb[sidx(F, ii, jj, kk)];
      }
    }
  }
  return acc;
}

// k_restrict0 for four consecutive coarse z nodes kc = 4g .. 4g+3 of one
// coarse row per thread.  Away from the faces (no clamped tap) the 13 taps
// of the four nodes are nine 16-byte row loads and four edge slots: around
// fine centre (2ic, 2jc, 2kc) the colour-0 taps are slot kc of rows (0, 0)
// and (+-1, +-1), and slots kc - 1 and kc of rows (+-1, 0) and (0, +-1)
// (their colour-0 nodes have odd k).  Taps are summed in k_restrict0's
// (di, dj, dk) order with its weights, so the bits are the same; groups
// that touch a face use that loop per node.  The four results go to the
// coarse split layout as two 8-byte stores (kc alternates colour).
// Coarse nodes 4t' .. of the four-node restriction, one problem: rb its
// fine colour-0 residual, gb its coarse right-hand side (split layout);
// t < C.nx * C.ny * ((C.nz + 3) / 4).
__device__ __forceinline__ void restrict0_4_at(const float* rb, const SGeo& F, float* gb,
                                               const SGeo& C, uint32_t t) {
  const uint32_t G4 = (uint32_t)(C.nz + 3) >> 2;
  const uint32_t ij = t / G4;
  const int kc0 = 4 * (int)(t - ij * G4);
  const int ic = (int)fdivu(ij, C.dny);
  const int jc = (int)(ij - (uint32_t)ic * C.dny.d);
  const bool inner = ic >= 1 && 2 * ic + 1 <= F.nx - 1 && jc >= 1 && 2 * jc + 1 <= F.ny - 1 &&
                     kc0 >= 1 && 2 * (kc0 + 3) + 1 <= F.nz - 1;
  if (!inner) {
    for (int u = 0; u < 4; u++) {
      const int kc = kc0 + u;
      if (kc >= C.nz) break;
      gb[(size_t)scol(ic, jc, kc) * C.csz + sidx(C, ic, jc, kc)] =
          0.5f * restrict0_node(rb, F, ic, jc, kc);
    }
    return;
  }
  auto row = [&](int di, int dj) {
    return rb + ((uint32_t)(2 * ic + di) * F.ny + (uint32_t)(2 * jc + dj)) * F.H + kc0;
  };
  float a[4] = {0.f, 0.f, 0.f, 0.f};
  // one tap per node from slot kc of a row, weight w
  auto at = [&](const float* r, float w) {
    const float4 v = ld4(r);
    a[0] += w * v.x;
    a[1] += w * v.y;
    a[2] += w * v.z;
    a[3] += w * v.w;
  };
  // two taps per node from slots kc - 1 and kc of a row (dk = -1, +1)
  auto at2 = [&](const float* r, float w) {
    const float4 v = ld4(r);
    const float m = r[-1];
    a[0] += w * m;
    a[0] += w * v.x;
    a[1] += w * v.x;
    a[1] += w * v.y;
    a[2] += w * v.y;
    a[2] += w * v.z;
    a[3] += w * v.z;
    a[3] += w * v.w;
  };
  at(row(-1, -1), 0.25f);
  at2(row(-1, 0), 0.25f);
  at(row(-1, 1), 0.25f);
  at2(row(0, -1), 0.25f);
  at(row(0, 0), 1.f);
  at2(row(0, 1), 0.25f);
  at(row(1, -1), 0.25f);
  at2(row(1, 0), 0.25f);
  at(row(1, 1), 0.25f);
  // kc0 is even: nodes kc0, kc0 + 2 share a colour (slots kc0/2, kc0/2 + 1),
  // kc0 + 1, kc0 + 3 the other
  const int ca = scol(ic, jc, kc0);
  const uint32_t cs = ((uint32_t)ic * C.ny + jc) * C.H + (kc0 >> 1);
  *reinterpret_cast<float2*>(gb + (size_t)ca * C.csz + cs) = make_float2(0.5f * a[0], 0.5f * a[2]);
  *reinterpret_cast<float2*>(gb + (size_t)(1 - ca) * C.csz + cs) =
      make_float2(0.5f * a[1], 0.5f * a[3]);
}

__global__ void __launch_bounds__(kT)
k_restrict0_4(const float* __restrict__ r0, SGeo F, float* __restrict__ gc, SGeo C,
              size_t cstride) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= (uint32_t)C.nx * C.ny * ((uint32_t)(C.nz + 3) >> 2)) return;
  restrict0_4_at(r0 + blockIdx.y * (size_t)F.csz, F, gc + blockIdx.y * cstride, C, t);
}

// r = g - A e on natural layout (0 at metal).
__global__ void __launch_bounds__(kT)
k_resid(const float* __restrict__ e, const float* __restrict__ g,
        const uint8_t* __restrict__ mask, SGeo G, float* __restrict__ r,
        size_t pstride, size_t rstride) {
  mask += (size_t)blockIdx.y * G.msplit;
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= G.n) return;
  const uint32_t ij = fdivu(t, G.dnz);
  const int k = (int)(t - ij * G.dnz.d);
  const int i = (int)fdivu(ij, G.dny);
  const int j = (int)(ij - (uint32_t)i * G.dny.d);
  const int c = scol(i, j, k);
  const uint32_t s = sidx(G, i, j, k);
  float out = 0.f;
  if (!mask[(size_t)c * G.csz + s]) {
    const float* eb = e + blockIdx.y * pstride;
    const float* own = eb + (size_t)c * G.csz;
    const float* oth = eb + (size_t)(1 - c) * G.csz;
    const float a = nbr_sum(G, own, oth, i, j, k >> 1, k, s) - 6.0f * own[s];
    out = g[blockIdx.y * pstride + (size_t)c * G.csz + s] - a;
  }
  r[blockIdx.y * rstride + t] = out;
}

// Coarse right-hand side: 4 x full weighting of the fine residual
// (27 points, weights 1/2 per off-centre step, clamped edges, /8), written
// to the coarse split layout.
__global__ void __launch_bounds__(kT)
k_restrict(const float* __restrict__ r, SGeo F, float* __restrict__ gc, SGeo C,
           size_t rstride, size_t cstride) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= C.n) return;
  const uint32_t ij = fdivu(t, C.dnz);
  const int kc = (int)(t - ij * C.dnz.d);
  const int ic = (int)fdivu(ij, C.dny);
  const int jc = (int)(ij - (uint32_t)ic * C.dny.d);
  const float* rb = r + blockIdx.y * rstride;
  float acc = 0.f;
#pragma unroll
  for (int di = -1; di <= 1; di++) {
    const int ii = min(max(2 * ic + di, 0), F.nx - 1);
    const float wi = di == 0 ? 1.f : 0.5f;
#pragma unroll
    for (int dj = -1; dj <= 1; dj++) {
      const int jj = min(max(2 * jc + dj, 0), F.ny - 1);
      const float wj = dj == 0 ? 1.f : 0.5f;
      const float* row = rb + ((size_t)ii * F.ny + jj) * F.nz;
      const float a = row[min(max(2 * kc - 1, 0), F.nz - 1)];
      const float b = row[min(2 * kc, F.nz - 1)];
      const float d = row[min(2 * kc + 1, F.nz - 1)];
      acc += wi * wj * (0.5f * (a + d) + b);
    }
  }
  const int c = scol(ic, jc, kc);
  gc[blockIdx.y * cstride + (size_t)c * C.csz + sidx(C, ic, jc, kc)] = 0.5f * acc;
}

struct LerpF {
  int a0, a1;
  float t;
};
// fine coordinate i/2 on the coarse axis of c nodes, low node kept one below
// the top (multigrid3d.py:465-481)
__device__ __forceinline__ LerpF pa(int i, int c) {
  float xf = 0.5f * (float)i;
  if (xf > (float)(c - 1)) xf = (float)(c - 1);
  int x0 = (int)xf;
  if (x0 > c - 2) x0 = c > 1 ? c - 2 : 0;
  LerpF l;
  l.a0 = x0;
  l.a1 = c > 1 ? x0 + 1 : x0;
  l.t = xf - (float)x0;
  return l;
}

__device__ __forceinline__ float cget(const float* eb, const SGeo& C, int i, int j, int k) {
  return eb[(size_t)scol(i, j, k) * C.csz + sidx(C, i, j, k)];
}

// e_fine += trilinear(e_coarse) at free fine nodes.  Each axis weight is 0,
// 1/2 or 1 (fine node i sits at i/2 in coarse units), so a fine node reads
// only the 1, 2, 4 or 8 coarse values whose weight is nonzero.
// Over the split layout: thread = 4 consecutive slots
// of one colour of fine row (i, j) (blockIdx.z = colour), so the 4 nodes
// share their x/y weights and their k parity (one z pattern for the whole
// thread) and the fine correction is read and written as one float4.  The
// per-node sum is formed in x, y, z order.
__global__ void __launch_bounds__(kT)
k_prolong_add4_gather(const float* __restrict__ ec, SGeo C, float* __restrict__ ef,
               const uint8_t* __restrict__ maskf, SGeo F, size_t cstride,
               size_t fstride) {
  maskf += (size_t)blockIdx.y * F.msplit;
  const int c = blockIdx.z;  // gridDim.z = 1: colour 0 only
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= (F.csz >> 2)) return;
  const uint32_t ij = fdivu(t, F.dH4);
  const int m0 = 4 * (int)(t - ij * F.dH4.d);
  const int i = (int)fdivu(ij, F.dny);
  const int j = (int)(ij - (uint32_t)i * F.dny.d);
  const int pc = (i + j + c) & 1;
  const uint32_t base = ij * (uint32_t)F.H + m0;
  const uchar4 mk = *reinterpret_cast<const uchar4*>(maskf + (size_t)c * F.csz + base);
  const uint8_t mv[4] = {mk.x, mk.y, mk.z, mk.w};
  const float* eb = ec + blockIdx.y * cstride;
  const LerpF x = pa(i, C.nx), y = pa(j, C.ny);
  int xi[2], yi[2];
  float xw[2], yw[2];
  int nxw = 0, nyw = 0;
  if (x.t != 1.f) { xi[nxw] = x.a0; xw[nxw++] = 1.f - x.t; }
  if (x.t != 0.f) { xi[nxw] = x.a1; xw[nxw++] = x.t; }
  if (y.t != 1.f) { yi[nyw] = y.a0; yw[nyw++] = 1.f - y.t; }
  if (y.t != 0.f) { yi[nyw] = y.a1; yw[nyw++] = y.t; }
  float add[4];
#pragma unroll
  for (int u = 0; u < 4; u++) {
    add[u] = 0.f;
    const int k = 2 * (m0 + u) + pc;
    if (mv[u] || k >= F.nz) continue;
    const LerpF z = pa(k, C.nz);
    int zi[2];
    float zw[2];
    int nzw = 0;
    if (z.t != 1.f) { zi[nzw] = z.a0; zw[nzw++] = 1.f - z.t; }
    if (z.t != 0.f) { zi[nzw] = z.a1; zw[nzw++] = z.t; }
    float acc = 0.f;
    for (int a = 0; a < nxw; a++)
      for (int b = 0; b < nyw; b++) {
        float zs = 0.f;
        for (int q = 0; q < nzw; q++) zs += zw[q] * cget(eb, C, xi[a], yi[b], zi[q]);
        acc += xw[a] * yw[b] * zs;
      }
    add[u] = acc;
  }
  if (mk.x & mk.y & mk.z & mk.w) return;  // metal or unused: nothing to add
  float4* out = reinterpret_cast<float4*>(ef + fstride * blockIdx.y + (size_t)c * F.csz + base);
  float4 v = *out;
  v.x += add[0];
  v.y += add[1];
  v.z += add[2];
  v.w += add[3];
  *out = v;
}

// The same correction with the coarse values fetched once per thread: the
// fine slots m0..m0+3 of one colour row sit at coarse z positions m0 + u
// (+1/2 for odd k), so all four read coarse nodes kc = m0 .. m0+4 of at most
// four coarse rows -- five values per row, three from one colour array and
// two from the other (kc alternates colour; slot kc >> 1) -- instead of
// locating every coarse node separately.  Per fine node the weights, the
// skipped zero weights and the x, y, z summation order are those of
// k_prolong_add4_gather, so the results are the same bits.  Needs every
// axis of both grids at least 2 nodes long.
// Fine float4 group t of colour c of the windowed prolongation, one
// problem: eb its coarse correction, efb its fine correction and maskf its
// fine split mask.
__device__ __forceinline__ void prolong_add4_at(const float* eb, const SGeo& C, float* efb,
                                                const uint8_t* maskf, const SGeo& F, int c,
                                                uint32_t t) {
  const uint32_t ij = fdivu(t, F.dH4);
  const int m0 = 4 * (int)(t - ij * F.dH4.d);
  const int i = (int)fdivu(ij, F.dny);
  const int j = (int)(ij - (uint32_t)i * F.dny.d);
  const int pc = (i + j + c) & 1;
  const uint32_t base = ij * (uint32_t)F.H + m0;
  // the coarse values are fetched whatever the mask says (in bounds); an
  // all-metal (or unused) group skips only the read-modify-write below
  const uchar4 mk = *reinterpret_cast<const uchar4*>(maskf + (size_t)c * F.csz + base);
  const uint8_t mv[4] = {mk.x, mk.y, mk.z, mk.w};
  const LerpF x = pa(i, C.nx), y = pa(j, C.ny);
  // the nonzero x (y) weights in order: a0 with 1 - t unless t = 1, then a1
  // with t unless t = 0 (t is 0, 1/2 or 1)
  const int xi[2] = {x.t == 1.f ? x.a1 : x.a0, x.a1};
  const float xw[2] = {x.t == 1.f ? x.t : 1.f - x.t, x.t};
  const int nxw = (x.t != 0.f && x.t != 1.f) ? 2 : 1;
  const int yi[2] = {y.t == 1.f ? y.a1 : y.a0, y.a1};
  const float yw[2] = {y.t == 1.f ? y.t : 1.f - y.t, y.t};
  const int nyw = (y.t != 0.f && y.t != 1.f) ? 2 : 1;
  // z weights of the four fine nodes: fine node u reads window slots u
  // (weight wl) and u + 1 (weight wh, skipped when 0).  pa() gives
  // a0 = m0 + u with weights 1 - t, t (t = 0 or 1/2), or at the top face
  // a1 = m0 + u alone with weight 1.
  float wl[4], wh[4];
#pragma unroll
  for (int u = 0; u < 4; u++) {
    const LerpF z = pa(2 * (m0 + u) + pc, C.nz);
    const bool top = z.t == 1.f;
    wl[u] = top ? z.t : 1.f - z.t;
    wh[u] = top ? 0.f : z.t;
  }
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) {
      if (a >= nxw || b >= nyw) continue;
      const uint32_t row = ((uint32_t)xi[a] * C.ny + yi[b]) * C.H + (m0 >> 1);
      const int ca = (xi[a] + yi[b] + m0) & 1;
      const float* A = eb + (size_t)ca * C.csz + row;
      const float* Bc = eb + (size_t)(1 - ca) * C.csz + row;
      // slots (m0 >> 1) and the next of both colours as 8-byte loads (the
      // row offset is even: H and m0 >> 1 are), in bounds even where they
      // lie past the row's last node (padding), which the guards zero
      const float2 a01 = *reinterpret_cast<const float2*>(A);
      const float2 b01 = *reinterpret_cast<const float2*>(Bc);
      float cv[5];
      cv[0] = a01.x;
      cv[1] = m0 + 1 < C.nz ? b01.x : 0.f;
      cv[2] = m0 + 2 < C.nz ? a01.y : 0.f;
      cv[3] = m0 + 3 < C.nz ? b01.y : 0.f;
      cv[4] = m0 + 4 < C.nz ? A[2] : 0.f;
      const float w = xw[a] * yw[b];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        float zs = 0.f;
        zs += wl[u] * cv[u];
        if (wh[u] != 0.f) zs += wh[u] * cv[u + 1];
        acc[u] += w * zs;
      }
    }
  if (mk.x & mk.y & mk.z & mk.w) return;  // metal or unused: nothing to add
  float4* out = reinterpret_cast<float4*>(efb + (size_t)c * F.csz + base);
  float4 v = *out;
  v.x += mv[0] ? 0.f : acc[0];
  v.y += mv[1] ? 0.f : acc[1];
  v.z += mv[2] ? 0.f : acc[2];
  v.w += mv[3] ? 0.f : acc[3];
  *out = v;
}

__global__ void __launch_bounds__(kT)
k_prolong_add4(const float* __restrict__ ec, SGeo C, float* __restrict__ ef,
               const uint8_t* __restrict__ maskf, SGeo F, size_t cstride,
               size_t fstride) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= (F.csz >> 2)) return;
  prolong_add4_at(ec + blockIdx.y * cstride, C, ef + fstride * blockIdx.y,
                  maskf + (size_t)blockIdx.y * F.msplit, F, blockIdx.z, t);
}

// The coarsest level's SOR pairs for one problem, by the calling CTA
// (kBottomThreads threads, all of which must call it): eb (out), gb and
// mask the problem's split arrays, se and sg shared scratch of kBottomMax
// floats each.
__device__ __forceinline__ void bottom_at(float* eb, const float* gb, const uint8_t* mask,
                                          const SGeo& G, float omega, int pairs, float* se,
                                          float* sg) {
  // A thread's nodes (at most kBottomMax / kBottomThreads): their colour,
  // whether they are free, and their six neighbours' slots, worked out once
  // so that the pairs below run on shared memory alone.
  constexpr int NPT = kBottomMax / kBottomThreads;
  int nbr[NPT][6];
  int col[NPT];
#pragma unroll
  for (int u = 0; u < NPT; u++) {
    const uint32_t t = threadIdx.x + (uint32_t)u * kBottomThreads;
    col[u] = -1;  // no node, or metal: never updated
    if (t < G.n) {
      const int k = (int)(t % G.nz);
      const int j = (int)((t / G.nz) % G.ny);
      const int i = (int)(t / ((uint32_t)G.nz * G.ny));
      const int c = scol(i, j, k);
      const uint32_t sl = sidx(G, i, j, k);
      se[t] = 0.f;
      sg[t] = gb[(size_t)c * G.csz + sl];
      if (!mask[(size_t)c * G.csz + sl]) col[u] = c;
      nbr[u][0] = (lo_i(i, G.nx) * G.ny + j) * G.nz + k;
      nbr[u][1] = (hi_i(i, G.nx) * G.ny + j) * G.nz + k;
      nbr[u][2] = (i * G.ny + lo_i(j, G.ny)) * G.nz + k;
      nbr[u][3] = (i * G.ny + hi_i(j, G.ny)) * G.nz + k;
      nbr[u][4] = (i * G.ny + j) * G.nz + lo_i(k, G.nz);
      nbr[u][5] = (i * G.ny + j) * G.nz + hi_i(k, G.nz);
    }
  }
  __syncthreads();
  for (int it = 0; it < pairs; it++) {
    for (int c = 0; c < 2; c++) {
#pragma unroll
      for (int u = 0; u < NPT; u++) {
        if (col[u] != c) continue;
        const uint32_t t = threadIdx.x + (uint32_t)u * kBottomThreads;
        const float q = ((((se[nbr[u][0]] + se[nbr[u][1]]) + (se[nbr[u][2]] + se[nbr[u][3]])) +
                          (se[nbr[u][4]] + se[nbr[u][5]])) -
                         sg[t]) *
                        (1.0f / 6.0f);
        se[t] += omega * (q - se[t]);
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int u = 0; u < NPT; u++) {
    const uint32_t t = threadIdx.x + (uint32_t)u * kBottomThreads;
    if (t < G.n) {
      const int k = (int)(t % G.nz);
      const int j = (int)((t / G.nz) % G.ny);
      const int i = (int)(t / ((uint32_t)G.nz * G.ny));
      eb[(size_t)scol(i, j, k) * G.csz + sidx(G, i, j, k)] = se[t];
    }
  }
}

// Coarsest level: red-black SOR in shared memory, one CTA per problem, a
// fixed number of pairs (the level has at most kBottomMax nodes).
__global__ void __launch_bounds__(kBottomThreads)
k_bottom(float* __restrict__ e, const float* __restrict__ g,
         const uint8_t* __restrict__ mask, SGeo G, float omega, int pairs,
         size_t pstride) {
  __shared__ float se[kBottomMax];
  __shared__ float sg[kBottomMax];
  bottom_at(e + blockIdx.x * pstride, g + blockIdx.x * pstride,
            mask + (size_t)blockIdx.x * G.msplit, G, omega, pairs, se, sg);
}

// The cycle of the level just above the bottom, the bottom solve included,
// by one CTA per problem in shared memory: the level's right-hand side and
// masks are read once and its correction written once, so the dozen
// launches of a few blocks that the separate kernels take on these small
// grids -- each a few microseconds of latency -- become one.  The phases
// are the device code of those kernels (zero_pair_at, gs4_group,
// resid0_4_at, restrict0_4_at, bottom_at, prolong_add4_at) over the CTA's
// threads, in their order, so the result has their bits.  Shared memory:
// the bottom's scratch (2 kBottomMax floats), the level's correction and
// right-hand side (2 csz floats each), its colour-0 residual (csz floats),
// the bottom's correction and right-hand side (2 csz_b floats each), then
// both masks (2 csz + 2 csz_b bytes); tail_smem_bytes() gives the total.
__global__ void __launch_bounds__(kBottomThreads)
k_tail_cycle(float* __restrict__ e, const float* __restrict__ g,
             const uint8_t* __restrict__ mask, SGeo A, size_t apstride,
             const uint8_t* __restrict__ bmask, SGeo Bt, int nu1, int nu2, float omega_b,
             int pairs) {
  extern __shared__ float4 tail_smem[];
  float* se = reinterpret_cast<float*>(tail_smem);
  float* sg = se + kBottomMax;
  float* ae = sg + kBottomMax;
  float* ag = ae + 2 * (size_t)A.csz;
  float* ar = ag + 2 * (size_t)A.csz;
  float* be = ar + (size_t)A.csz;
  float* bg = be + 2 * (size_t)Bt.csz;
  uint8_t* am = reinterpret_cast<uint8_t*>(bg + 2 * (size_t)Bt.csz);
  uint8_t* bm = am + 2 * (size_t)A.csz;
  const uint32_t tid = threadIdx.x;
  const float* gA = g + blockIdx.x * apstride;
  const uint8_t* mA = mask + (size_t)blockIdx.x * A.msplit;
  const uint8_t* mB = bmask + (size_t)blockIdx.x * Bt.msplit;
  const uint32_t na4 = (2 * A.csz) >> 2, nb4 = (2 * Bt.csz) >> 2;
  for (uint32_t q = tid; q < na4; q += kBottomThreads) {
    reinterpret_cast<float4*>(ag)[q] = ld4(gA + 4 * (size_t)q);
    reinterpret_cast<uchar4*>(am)[q] = reinterpret_cast<const uchar4*>(mA)[q];
  }
  for (uint32_t q = tid; q < nb4; q += kBottomThreads)
    reinterpret_cast<uchar4*>(bm)[q] = reinterpret_cast<const uchar4*>(mB)[q];
  __syncthreads();
  const uint32_t nq = A.csz >> 2;
  // pre-smoothing: the fused first pair from e = 0, then nu1 - 1 pairs
  for (uint32_t t = tid; t < nq; t += kBottomThreads) zero_pair_at<false>(ae, ag, am, A, t);
  __syncthreads();
  for (int q = 1; q < nu1; q++)
    for (int c = 0; c < 2; c++) {
      for (uint32_t t = tid; t < nq; t += kBottomThreads)
        gs4_group<false>(ae + (size_t)c * A.csz, ae + (size_t)(1 - c) * A.csz,
                         ag + (size_t)c * A.csz, am + (size_t)c * A.csz, A, c, 1.f, t);
      __syncthreads();
    }
  // the colour-0 residual, restricted to the bottom's right-hand side
  for (uint32_t t = tid; t < nq; t += kBottomThreads) resid0_4_at(ae, ag, am, A, ar, t);
  __syncthreads();
  const uint32_t nr = (uint32_t)Bt.nx * Bt.ny * ((uint32_t)(Bt.nz + 3) >> 2);
  for (uint32_t t = tid; t < nr; t += kBottomThreads) restrict0_4_at(ar, A, bg, Bt, t);
  __syncthreads();
  bottom_at(be, bg, bm, Bt, omega_b, pairs, se, sg);
  __syncthreads();
  // colour 0 takes the prolonged correction (the first post-smoothing
  // half-sweep, colour 1, rewrites every free colour-1 slot)
  for (uint32_t t = tid; t < nq; t += kBottomThreads) prolong_add4_at(be, Bt, ae, am, A, 0, t);
  __syncthreads();
  for (int q = 0; q < nu2; q++)
    for (int c = 1; c >= 0; c--) {
      for (uint32_t t = tid; t < nq; t += kBottomThreads)
        gs4_group<false>(ae + (size_t)c * A.csz, ae + (size_t)(1 - c) * A.csz,
                         ag + (size_t)c * A.csz, am + (size_t)c * A.csz, A, c, 1.f, t);
      __syncthreads();
    }
  float* eA = e + blockIdx.x * apstride;
  for (uint32_t q = tid; q < na4; q += kBottomThreads)
    reinterpret_cast<float4*>(eA)[q] = reinterpret_cast<const float4*>(ae)[q];
}

// Shared bytes k_tail_cycle needs for level A above the bottom Bt.
inline size_t tail_smem_bytes(const SGeo& A, const SGeo& Bt) {
  return 4 * (2 * (size_t)kBottomMax + 5 * (size_t)A.csz + 4 * (size_t)Bt.csz) +
         2 * (size_t)A.csz + 2 * (size_t)Bt.csz;
}
constexpr size_t kTailSmemMax = 200 * 1024;

// Coarse metal of the FP32 correction's hierarchy: injection with a rescue
// of thin metal.  Coarse node (i, j, k) is metal when fine node
// (2i, 2j, 2k) is (injection), or when its fine 2x2x2 block holds metal
// that no injected coarse node within one coarse step represents -- a
// plate or ring thinner than the coarse spacing, which injection alone
// would drop.  (The FP64 V-cycle keeps the reference's block-ANY rule.)
// Block-ANY makes every coarse object up to a fine cell fatter, so the
// coarse correction stops short of each metal surface; injection alone
// loses thin electrodes on the deep levels.  Measured refinement steps
// (block-ANY / injection / this rule): ring stack 7 / 6 / 6, quadrupole
// 6 / 4 / 4, planar boards 6-7 / 9-10 / 7, random decks 5-7 / 5-6 / 5-6,
// with unchanged accuracy.
__global__ void k_coarsen_inject(const uint8_t* __restrict__ fine, SGeo F,
                                 uint8_t* __restrict__ coarse, SGeo C) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= C.n) return;
  const uint32_t ij = fdivu(t, C.dnz);
  const uint32_t kc = t - ij * C.dnz.d;
  const uint32_t ic = fdivu(ij, C.dny);
  const uint32_t jc = ij - ic * C.dny.d;
  coarse[t] = fine[((2 * ic) * (uint32_t)F.ny + 2 * jc) * (uint32_t)F.nz + 2 * kc];
}

__global__ void k_coarsen_rescue(const uint8_t* __restrict__ fine, SGeo F,
                                 const uint8_t* __restrict__ inj, uint8_t* __restrict__ out,
                                 SGeo C) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= C.n) return;
  if (inj[t]) {
    out[t] = 1;
    return;
  }
  const uint32_t ij = fdivu(t, C.dnz);
  const int kc = (int)(t - ij * C.dnz.d);
  const int ic = (int)fdivu(ij, C.dny);
  const int jc = (int)(ij - (uint32_t)ic * C.dny.d);
  bool any = false;
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++)
      for (int q = 0; q < 2; q++) {
        const int i = 2 * ic + a, j = 2 * jc + b, k = 2 * kc + q;
        if (i < F.nx && j < F.ny && k < F.nz &&
            fine[((uint32_t)i * F.ny + j) * (uint32_t)F.nz + k])
          any = true;
      }
  bool near = false;
  if (any)
    for (int a = -1; a <= 1; a++)
      for (int b = -1; b <= 1; b++)
        for (int q = -1; q <= 1; q++) {
          const int i = ic + a, j = jc + b, k = kc + q;
          if (i >= 0 && j >= 0 && k >= 0 && i < C.nx && j < C.ny && k < C.nz &&
              inj[((uint32_t)i * C.ny + j) * (uint32_t)C.nz + k])
            near = true;
        }
  out[t] = any && !near ? 1 : 0;
}

// natural u8 mask -> split u8 mask
__global__ void k_split_mask(const uint8_t* __restrict__ nat, SGeo G, uint8_t* __restrict__ sp) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= G.n) return;
  const uint32_t ij = fdivu(t, G.dnz);
  const int k = (int)(t - ij * G.dnz.d);
  const int i = (int)fdivu(ij, G.dny);
  const int j = (int)(ij - (uint32_t)i * G.dny.d);
  sp[(size_t)scol(i, j, k) * G.csz + sidx(G, i, j, k)] = nat[t];
}

// ---- FP64 refinement kernels (natural phi64, split g32 / e32) -----------

// ---- the refined potential in 64-bit fixed point ---------------------------
//
// Problem b's potential is held as integers Phi in units of
// u_b = 2^(E_b - 56), E_b the binary exponent of its largest Dirichlet
// magnitude (|value| < 2^E_b; E_b in [-60, 60]), so every potential the
// refinement can reach, bounded by the Dirichlet values, is below 2^56 units
// in magnitude and the int64 range leaves 128x headroom.  One unit is
// 2^-56 of the largest value: finer than a float64 ulp there (2^-53).
// Benefits: the reference's fine residual sum(nbr) - 6 phi is an exact
// integer sum (an earlier float64 form had to align the values to a common
// exponent first, about 130 integer operations per node); the
// update adds the rounded correction; the float64 potential is formed once,
// at the end, with the Dirichlet values written exactly at the metal.

// 2^k as a float (k in [-126, 127]) and as a double (k in [-1022, 1023])
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }
__device__ __forceinline__ double pow2d(int k) {
  return __longlong_as_double(static_cast<long long>(1023 + k) << 52);
}

// RN(x) as an int64 on the integer pipe (the hardware conversion runs on
// the FP64 pipe, which this GPU has little of): the IEEE conversion itself,
// rounded once to nearest, ties to even, from the discarded bits and the
// kept integer's last bit.  |x| >= 2^63, infinities and NaN take the
// hardware conversion.  Checked against it bit for bit by
// ig_mixed_check_convert.
__device__ __forceinline__ long long f2ll_rn(float x) {
  const unsigned b = __float_as_uint(x);
  const int ef = static_cast<int>((b >> 23) & 0xffu);
  if (ef < 126) return 0LL;  // |x| < 1/2 (zeros and subnormals included)
  if (ef >= 190) return __float2ll_rn(x);
  const unsigned long long m = (b & 0x7fffffu) | 0x800000u;  // |x| = m * 2^(ef - 150)
  unsigned long long r;
  if (ef >= 150) {
    r = m << (ef - 150);
  } else {
    const int sh = 150 - ef;  // 1..24
    r = m >> sh;
    const unsigned long long rem = m & ((1ULL << sh) - 1ULL), half = 1ULL << (sh - 1);
    r += (rem > half || (rem == half && (r & 1ULL))) ? 1ULL : 0ULL;
  }
  return (b >> 31) ? -static_cast<long long>(r) : static_cast<long long>(r);
}

// g32 = -(float) (scale * r(phi)) at free nodes, 0 at metal; r is the
// reference's fine residual with theta None (kind kPlain: sum - 6 phi; the
// Shortley-Weller form is half of it and is scaled by 2 through nscale =
// -(float) scale, a power of two).  The residual is an exact int64 sum of
// the fixed-point potentials, rounded once to float and scaled by u_b.
// One warp per natural row (i, j): the row's coordinates, its four x/y
// neighbour rows and its two split output rows are worked out once, and
// the lanes walk the row 32 nodes at a time (two steps in flight), so every
// load of the row and of its neighbour rows is 256 contiguous bytes.
constexpr int kRowWarps = kT / 32;
inline unsigned rows_blocks(const SGeo& g) {
  return (unsigned)(((size_t)g.nx * g.ny + kRowWarps - 1) / kRowWarps);
}
__global__ void __launch_bounds__(kT)
k_resid64(const long long* __restrict__ phi, const uint8_t* __restrict__ fixed,
          SGeo G, float* __restrict__ g, const int* __restrict__ fexp, float nscale,
          size_t nstride, size_t pstride) {
  const uint32_t r = blockIdx.x * kRowWarps + (threadIdx.x >> 5);
  if (r >= (uint32_t)G.nx * (uint32_t)G.ny) return;  // whole warps
  const int lane = threadIdx.x & 31;
  const int i = (int)fdivu(r, G.dny);
  const int j = (int)(r - (uint32_t)i * G.dny.d);
  const int nz = G.nz;
  const long long* p = phi + blockIdx.y * nstride;
  const long long* pr = p + (size_t)r * nz;
  const long long* pxm = p + ((size_t)lo_i(i, G.nx) * G.ny + j) * nz;
  const long long* pxp = p + ((size_t)hi_i(i, G.nx) * G.ny + j) * nz;
  const long long* pym = p + ((size_t)i * G.ny + lo_i(j, G.ny)) * nz;
  const long long* pyp = p + ((size_t)i * G.ny + hi_i(j, G.ny)) * nz;
  const uint8_t* fr = fixed + (size_t)blockIdx.y * G.mnat + (size_t)r * nz;
  // the colour of the row's even k, then the split rows of both colours
  const int ce = (i + j) & 1;
  float* gb = g + blockIdx.y * pstride + (size_t)r * G.H;
  float* ge = gb + (size_t)ce * G.csz;
  float* go = gb + (size_t)(1 - ce) * G.csz;
  const float u = pow2f(fexp[blockIdx.y] - 56);
  // every load is in bounds whatever the mask says, so the mask and the
  // seven potentials are fetched together and the mask only selects; four
  // steps of the row in flight (measured: 477 -> 375 us on the 8-basis
  // ring stack against two)
#pragma unroll 4
  for (int k = lane; k < nz; k += 32) {
    const int km = k > 0 ? k - 1 : (nz > 1 ? 1 : k);
    const int kp = k + 1 < nz ? k + 1 : (nz > 1 ? nz - 2 : k);
    const uint8_t metal = fr[k];
    const long long s = ((pxm[k] + pxp[k]) + (pym[k] + pyp[k])) + (pr[km] + pr[kp]);
    const long long c = pr[k];
    const long long rr = s - ((c << 2) + (c << 1));
    ((k & 1) ? go : ge)[k >> 1] = metal ? 0.f : __ll2float_rn(rr) * u * nscale;
  }
}

// k_resid64 for short rows: a warp takes R consecutive natural rows as one
// run of R * nz nodes (each lane's row and k from one division, its plane
// and row-in-plane from another), so a warp has enough of the row's steps
// in flight even when nz is small; the same expressions per node.
__global__ void __launch_bounds__(kT)
k_resid64_flat(const long long* __restrict__ phi, const uint8_t* __restrict__ fixed,
               SGeo G, float* __restrict__ g, const int* __restrict__ fexp, float nscale,
               size_t nstride, size_t pstride, uint32_t R) {
  const uint32_t nrows = (uint32_t)G.nx * (uint32_t)G.ny;
  const uint32_t r0 = (blockIdx.x * kRowWarps + (threadIdx.x >> 5)) * R;
  if (r0 >= nrows) return;  // whole warps
  const uint32_t lane = threadIdx.x & 31;
  const int nz = G.nz;
  const uint32_t span = min(R, nrows - r0) * (uint32_t)nz;
  const long long* p = phi + blockIdx.y * nstride;
  const uint8_t* fb = fixed + (size_t)blockIdx.y * G.mnat;
  float* gb = g + blockIdx.y * pstride;
  const float u = pow2f(fexp[blockIdx.y] - 56);
#pragma unroll 4
  for (uint32_t q = lane; q < span; q += 32) {
    const uint32_t rr = fdivu(q, G.dnz);
    const int k = (int)(q - rr * (uint32_t)nz);
    const uint32_t r = r0 + rr;
    const int i = (int)fdivu(r, G.dny);
    const int j = (int)(r - (uint32_t)i * G.dny.d);
    const size_t o = (size_t)r * nz;
    const int km = k > 0 ? k - 1 : (nz > 1 ? 1 : k);
    const int kp = k + 1 < nz ? k + 1 : (nz > 1 ? nz - 2 : k);
    const uint8_t metal = fb[o + k];
    const long long s =
        ((p[((size_t)lo_i(i, G.nx) * G.ny + j) * nz + k] +
          p[((size_t)hi_i(i, G.nx) * G.ny + j) * nz + k]) +
         (p[((size_t)i * G.ny + lo_i(j, G.ny)) * nz + k] +
          p[((size_t)i * G.ny + hi_i(j, G.ny)) * nz + k])) +
        (p[o + km] + p[o + kp]);
    const long long c = p[o + k];
    const long long rv = s - ((c << 2) + (c << 1));
    gb[(size_t)((i + j + k) & 1) * G.csz + (size_t)r * G.H + (k >> 1)] =
        metal ? 0.f : __ll2float_rn(rv) * u * nscale;
  }
}

// Natural rows per warp for the residual and the update: 1 (one warp per
// row, k_resid64 / k_update64) when rows are long enough to keep a warp's
// loads in flight, else enough rows for about 256 nodes (the _flat forms).
// force: -1 the rule, 0 always one row per warp, 1 always several.
inline uint32_t flat_rows(const SGeo& G, int force) {
  if (force == 0) return 1;
  if (force == 1) return (uint32_t)std::max(2, (256 + G.nz - 1) / G.nz);
  return G.nz >= 192 ? 1u : (uint32_t)std::max(2, (256 + G.nz - 1) / G.nz);
}
inline unsigned flat_blocks(const SGeo& G, uint32_t R) {
  const size_t warps = ((size_t)G.nx * G.ny + R - 1) / R;
  return (unsigned)((warps + kRowWarps - 1) / kRowWarps);
}

// float -> double by its bits for zeros and normal floats (exponent rebias,
// significand moved up 29 bits); subnormals, infinities and NaN convert on
// the FP64 pipe.
__device__ __forceinline__ double widen(float d) {
  const unsigned fb = __float_as_uint(d);
  const unsigned ef = (fb >> 23) & 0xffu;
  if ((fb & 0x7fffffffu) == 0u)
    return __longlong_as_double(static_cast<long long>(static_cast<unsigned long long>(fb) << 32));
  if (ef - 1u < 254u)
    return __longlong_as_double(static_cast<long long>(
        (static_cast<unsigned long long>(fb & 0x80000000u) << 32) |
        (static_cast<unsigned long long>(ef + 896u) << 52) |
        (static_cast<unsigned long long>(fb & 0x7fffffu) << 29)));
  return (double)d;
}

// Phi += e32 / u_b (rounded to the nearest unit) at free nodes; the
// per-problem maximum of |e32| (the applied change, to within half a unit)
// goes to dmax[b] as float64 bits (the refinement's convergence norm, the
// analogue of the V-cycle's full-cycle change, multigrid3d.py:702).  With
// p given, e32 is e + alpha p: the flexible CG's last step x += alpha p
// folded in (k_cg_update's expression; its g half is dead, the residual is
// recomputed next).  One warp per natural row, as k_resid64: lane k's
// potential and mask are 8 and 1 contiguous bytes of the row, its
// correction slot k >> 1 of the colour (i + j + k) & 1, so a warp's loads
// of the corrections are two runs of 16 consecutive floats.
__global__ void __launch_bounds__(kT)
k_update64(long long* __restrict__ phi, const uint8_t* __restrict__ fixed,
           const float* __restrict__ e, SGeo G, unsigned long long* dmax,
           const int* __restrict__ fexp, size_t nstride, size_t pstride,
           const float* __restrict__ p = nullptr, const double* __restrict__ scal = nullptr) {
  const uint32_t r = blockIdx.x * kRowWarps + (threadIdx.x >> 5);
  unsigned key32 = 0;
  if (r < (uint32_t)G.nx * (uint32_t)G.ny) {
    const int lane = threadIdx.x & 31;
    const int i = (int)fdivu(r, G.dny);
    const int j = (int)(r - (uint32_t)i * G.dny.d);
    const int nz = G.nz;
    long long* pr = phi + blockIdx.y * nstride + (size_t)r * nz;
    const uint8_t* fr = fixed + (size_t)blockIdx.y * G.mnat + (size_t)r * nz;
    const size_t ro = blockIdx.y * pstride + (size_t)r * G.H;
    const float* ee = e ? e + ro + (size_t)((i + j) & 1) * G.csz : nullptr;
    const float* eo = e ? e + ro + (size_t)(1 - ((i + j) & 1)) * G.csz : nullptr;
    const float* pe = p ? p + ro + (size_t)((i + j) & 1) * G.csz : nullptr;
    const float* po = p ? p + ro + (size_t)(1 - ((i + j) & 1)) * G.csz : nullptr;
    const float al = p ? (float)scal[4 * blockIdx.y + 1] : 0.f;
    const float to_units = pow2f(56 - fexp[blockIdx.y]);
    // The loads do not wait for the mask (all in bounds) and no lane
    // branches on it: metal nodes compute a zero change and skip only the
    // store (a predicated store).  Measured per launch, 8-basis ring stack /
    // 257^3 quadrupole (a quarter of it metal): 507 / 75 us, against
    // 544 / 195 us when every node was written back and 641 / 87 us when
    // metal lanes left the loop body early.
#pragma unroll 2
    for (int k = lane; k < nz; k += 32) {
      const int m = k >> 1;
      const uint8_t metal = fr[k];
      const long long old = pr[k];
      float ev = e ? ((k & 1) ? eo : ee)[m] : 0.f;
      if (p) ev = __fmaf_rn(al, ((k & 1) ? po : pe)[m], ev);
      ev = metal ? 0.f : ev;
      const long long nv = old + f2ll_rn(ev * to_units);
      if (!metal) pr[k] = nv;
      // |ev| as float bits (ordered like the values); NaN counts as
      // infinity: never converged
      key32 = max(key32, min(__float_as_uint(ev) & 0x7fffffffu, 0x7f800000u));
    }
  }
  // the warp's largest |ev| (float bits order like the values), widened
  // once to float64 bits; a warp whose maximum beats the stored one raises
  // it -- no block barrier, so a warp leaves as soon as its row is done
  const unsigned wmax = __reduce_max_sync(0xffffffffu, key32);
  if ((threadIdx.x & 31) == 0 && wmax) {
    const unsigned long long key =
        static_cast<unsigned long long>(__double_as_longlong(widen(__uint_as_float(wmax))));
    if (key > *reinterpret_cast<volatile unsigned long long*>(dmax + blockIdx.y))
      atomicMax(dmax + blockIdx.y, key);
  }
}

// k_update64 for short rows: R consecutive natural rows per warp as one run
// (see k_resid64_flat); the same expressions per node.
__global__ void __launch_bounds__(kT)
k_update64_flat(long long* __restrict__ phi, const uint8_t* __restrict__ fixed,
                const float* __restrict__ e, SGeo G, unsigned long long* dmax,
                const int* __restrict__ fexp, size_t nstride, size_t pstride,
                const float* __restrict__ p, const double* __restrict__ scal, uint32_t R) {
  const uint32_t nrows = (uint32_t)G.nx * (uint32_t)G.ny;
  const uint32_t r0 = (blockIdx.x * kRowWarps + (threadIdx.x >> 5)) * R;
  unsigned key32 = 0;
  if (r0 < nrows) {
    const uint32_t lane = threadIdx.x & 31;
    const int nz = G.nz;
    const uint32_t span = min(R, nrows - r0) * (uint32_t)nz;
    long long* P = phi + blockIdx.y * nstride + (size_t)r0 * nz;
    const uint8_t* F = fixed + (size_t)blockIdx.y * G.mnat + (size_t)r0 * nz;
    const size_t pb = blockIdx.y * pstride;
    const float al = p ? (float)scal[4 * blockIdx.y + 1] : 0.f;
    const float to_units = pow2f(56 - fexp[blockIdx.y]);
#pragma unroll 2
    for (uint32_t q = lane; q < span; q += 32) {
      const uint32_t rr = fdivu(q, G.dnz);
      const int k = (int)(q - rr * (uint32_t)nz);
      const uint32_t r = r0 + rr;
      const int i = (int)fdivu(r, G.dny);
      const int j = (int)(r - (uint32_t)i * G.dny.d);
      const size_t so = pb + (size_t)((i + j + k) & 1) * G.csz + (size_t)r * G.H + (k >> 1);
      const uint8_t metal = F[q];
      const long long old = P[q];
      float ev = e ? e[so] : 0.f;
      if (p) ev = __fmaf_rn(al, p[so], ev);
      ev = metal ? 0.f : ev;
      const long long nv = old + f2ll_rn(ev * to_units);
      if (!metal) P[q] = nv;
      key32 = max(key32, min(__float_as_uint(ev) & 0x7fffffffu, 0x7f800000u));
    }
  }
  const unsigned wmax = __reduce_max_sync(0xffffffffu, key32);
  if ((threadIdx.x & 31) == 0 && wmax) {
    const unsigned long long key =
        static_cast<unsigned long long>(__double_as_longlong(widen(__uint_as_float(wmax))));
    if (key > *reinterpret_cast<volatile unsigned long long*>(dmax + blockIdx.y))
      atomicMax(dmax + blockIdx.y, key);
  }
}

// Phi[b] = the Dirichlet values of problem b at metal (in units of u_b), 0
// elsewhere; for a basis set v_basis (vfx units) on mask b.
__global__ void k_init_basis(long long* __restrict__ phi, const uint8_t* __restrict__ masks,
                             uint32_t n, long long vfx, size_t nstride) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= n) return;
  phi[blockIdx.y * nstride + t] = masks[(size_t)blockIdx.y * n + t] ? vfx : 0LL;
}

__global__ void k_init_vals(long long* __restrict__ phi, const uint8_t* __restrict__ fixed,
                            const double* __restrict__ val, uint32_t n, size_t nstride,
                            const int* __restrict__ fexp, size_t fstride) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= n) return;
  fixed += blockIdx.y * fstride;
  const double v = val[blockIdx.y * nstride + t];
  phi[blockIdx.y * nstride + t] =
      fixed[t] ? __double2ll_rn(v * pow2d(56 - fexp[blockIdx.y])) : 0LL;
}

// Per problem, the largest |Dirichlet value| at the metal, as float64 bits
// (NaN and infinities count as the largest finite value, so the caller's
// range check refuses them).
__global__ void __launch_bounds__(kT)
k_absmax_vals(const double* __restrict__ val, const uint8_t* __restrict__ fixed, uint32_t n,
              size_t nstride, unsigned long long* out, size_t fstride) {
  fixed += blockIdx.y * fstride;
  unsigned long long key = 0;
  for (uint32_t t = blockIdx.x * kT + threadIdx.x; t < n; t += gridDim.x * kT) {
    if (!fixed[t]) continue;
    unsigned long long kk =
        static_cast<unsigned long long>(__double_as_longlong(val[blockIdx.y * nstride + t])) &
        0x7fffffffffffffffULL;
    if (kk >= 0x7ff0000000000000ULL) kk = 0x7fefffffffffffffULL;
    key = max(key, kk);
  }
  block_max_to(key, out + blockIdx.y);
}

// In place: the float64 potential of problem b from its units (Phi * u_b,
// one rounding when |Phi| >= 2^53), with the Dirichlet values written
// exactly at the metal: vals (n per problem) when given, else the basis
// set's v_basis on mask b (masks, n per problem) and 0 on the rest.
__global__ void k_fixed_out(long long* __restrict__ phi, const uint8_t* __restrict__ fixed,
                            const double* __restrict__ vals, const uint8_t* __restrict__ masks,
                            double v, uint32_t n, size_t nstride,
                            const int* __restrict__ fexp, size_t fstride) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= n) return;
  fixed += blockIdx.y * fstride;
  const size_t o = blockIdx.y * nstride + t;
  // the potential is fetched with the mask, not after it; only metal nodes
  // (few) wait for their Dirichlet value
  const long long q = phi[o];
  const uint8_t metal = fixed[t];
  double r = __ll2double_rn(q) * pow2d(fexp[blockIdx.y] - 56);
  if (metal) r = vals ? vals[o] : (masks[(size_t)blockIdx.y * n + t] ? v : 0.0);
  reinterpret_cast<double*>(phi)[o] = r;
}

// The unit bases of a basis solve as float32: RN32(phi / v_basis), phi the
// float64 potential k_fixed_out would form (v_basis exactly on the basis's
// own electrode, 0 on the other metal) -- the two roundings of the field
// cache's (phi / V_BASIS).astype(float32), so the same bits -- into `out`
// (n floats per problem), for a download of 4 bytes per node instead of 8.
__global__ void k_unit32_out(const long long* __restrict__ phi, const uint8_t* __restrict__ fixed,
                             const uint8_t* __restrict__ masks, double v, uint32_t n,
                             size_t nstride, const int* __restrict__ fexp, float* __restrict__ out) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= n) return;
  const long long q = phi[blockIdx.y * nstride + t];
  const uint8_t metal = fixed[t];
  double r = __ll2double_rn(q) * pow2d(fexp[blockIdx.y] - 56);
  if (metal) r = masks[(size_t)blockIdx.y * n + t] ? v : 0.0;
  out[(size_t)blockIdx.y * n + t] = __double2float_rn(__ddiv_rn(r, v));
}

// f2ll_rn against the hardware conversion: mism counts the inputs whose
// results differ.
__global__ void k_check_convert(const float* __restrict__ fv, uint32_t n,
                                unsigned long long* mism) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= n) return;
  if (f2ll_rn(fv[t]) != __float2ll_rn(fv[t])) atomicAdd(mism, 1ULL);
}

// ---- flexible CG on the FP32 correction (level 0, split layout) --------
//
// Solves L x = r with L = 6 - sum(neighbours) (the negated 7-point operator,
// symmetric positive definite on the free nodes), preconditioned by the
// multigrid cycle (z = V(g) with g = -r, since the cycle solves A e = g with
// A = -L).  Flexible CG, one-term form: alpha = <p, r>/<p, L p>,
// beta = -<z_new, L p_old>/<p_old, L p_old>.  The solver carries g = -r
// instead of r.  Dot products: per-thread FP32 over four slots, per-block
// FP64, then a fixed-order FP64 sum per problem (deterministic).

__device__ __forceinline__ double block_sum_d(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < blockDim.x / 32 ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  return t;  // valid in thread 0
}

// p = z + beta p on valid free slots (p stays 0 on metal).
__global__ void __launch_bounds__(kT)
k_cg_dir(float* __restrict__ p, const float* __restrict__ z,
         const double* __restrict__ scal, size_t pstride, uint32_t n) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= n) return;
  const float b = (float)scal[4 * blockIdx.y + 2];
  const size_t o = blockIdx.y * pstride + t;
  p[o] = z[o] + b * p[o];
}

// Compensated float32 accumulation (Kahan): a thread sums many products
// with about float64 accuracy at float32 cost; the block total is formed in
// float64 once per block.
struct KSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float y = __fsub_rn(v, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// The last half-sweep of the finest level's cycle (k_gs4<NG, false>, the
// same update) with the flexible CG's <z, q_old> formed in the same pass:
// once the colour-c groups are updated, z is final, so each thread adds
// both colours of its slots (the other colour from the half-sweep before)
// against q, and each block writes one partial (part[b * gridDim.x +
// blockIdx.x]) -- k_cg_dot's read of z folded into the sweep that writes
// it.  Summation order differs from k_cg_dot (blocks of the sweep's shape),
// so the partial sums, not the update, may differ in their last bits.
template <int NG>
__global__ void k_gs4_dot(float* __restrict__ e, const float* __restrict__ g,
                          const uint8_t* __restrict__ mask, SGeo G, int c, float omega,
                          size_t pstride, const float* __restrict__ q,
                          double* __restrict__ part) {
  __shared__ double sh[32];
  mask += (size_t)blockIdx.y * G.msplit;
  const uint32_t nq = G.csz >> 2;
  float* eb = e + blockIdx.y * pstride;
  float* own = eb + (size_t)c * G.csz;
  const float* oth = eb + (size_t)(1 - c) * G.csz;
  const float* gp = g + blockIdx.y * pstride + (size_t)c * G.csz;
  const uint8_t* mp = mask + (size_t)c * G.csz;
  const float* qo = q + blockIdx.y * pstride + (size_t)c * G.csz;
  const float* qt = q + blockIdx.y * pstride + (size_t)(1 - c) * G.csz;
  const uint32_t t0 = blockIdx.x * blockDim.x * NG + threadIdx.x;
  KSum acc;
#pragma unroll
  for (int u = 0; u < NG; u++) {
    const uint32_t t = t0 + u * blockDim.x;
    if (t < nq) {
      gs4_group<false>(own, oth, gp, mp, G, c, omega, t);
      const uint32_t ij = fdivu(t, G.dH4);
      const uint32_t base = ij * (uint32_t)G.H + 4 * (t - ij * G.dH4.d);
      const float4 za = ld4(own + base), zb = ld4(oth + base);
      const float4 qa = ld4(qo + base), qb = ld4(qt + base);
      acc.add(za.x * qa.x); acc.add(za.y * qa.y); acc.add(za.z * qa.z); acc.add(za.w * qa.w);
      acc.add(zb.x * qb.x); acc.add(zb.y * qb.y); acc.add(zb.z * qb.z); acc.add(zb.w * qb.w);
    }
  }
  const double tot = block_sum_d(acc.value(), sh);
  if (threadIdx.x == 0) part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = tot;
}

// q = L p (both colours; q = 0 on metal) and block partials of <p, q> and
// <p, g>; blockIdx.y = colour, blockIdx.z = problem.  Grid-stride over
// float4 groups (kCgBlocks blocks per colour and problem), so each block
// reduces once.  Blocks start in (x, y, z) order, so the two colours of a
// problem run side by side over the same rows: the other colour's values
// one colour reads as neighbours are the ones the other is reading as its
// own, and come from L2 rather than from a second pass over DRAM.
constexpr unsigned kCgBlocks = 152 * 2;
__global__ void __launch_bounds__(kT)
k_cg_matvec(const float* __restrict__ p, const float* __restrict__ g,
            const uint8_t* __restrict__ mask, SGeo G, float* __restrict__ q,
            double* __restrict__ part, size_t pstride) {
  mask += (size_t)blockIdx.z * G.msplit;
  __shared__ double sh[kT / 32];
  const int c = blockIdx.y;
  const uint32_t nq = G.csz >> 2;
  KSum spq, spg;
  const float* pb = p + blockIdx.z * pstride;
  const float* own = pb + (size_t)c * G.csz;
  const float* oth = pb + (size_t)(1 - c) * G.csz;
  for (uint32_t t = blockIdx.x * kT + threadIdx.x; t < nq; t += gridDim.x * kT) {
    const uint32_t ij = fdivu(t, G.dH4);
    const int m0 = 4 * (int)(t - ij * G.dH4.d);
    const int i = (int)fdivu(ij, G.dny);
    const int j = (int)(ij - (uint32_t)i * G.dny.d);
    const int pc = (i + j + c) & 1;
    const uint32_t base = ij * (uint32_t)G.H + m0;
    const uchar4 mk = *reinterpret_cast<const uchar4*>(mask + (size_t)c * G.csz + base);
    const uint8_t mv[4] = {mk.x, mk.y, mk.z, mk.w};
    const float4 pv = ld4(own + base);
    const float4 gv = ld4(g + blockIdx.z * pstride + (size_t)c * G.csz + base);
    const float pp[4] = {pv.x, pv.y, pv.z, pv.w};
    const float gg[4] = {gv.x, gv.y, gv.z, gv.w};
    float out[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int k = 2 * (m0 + u) + pc;
      out[u] = 0.f;
      if (!mv[u] && k < G.nz)
        out[u] = 6.0f * pp[u] - nbr_sum(G, own, oth, i, j, m0 + u, k, base + u);
      spq.add(pp[u] * out[u]);
      spg.add(pp[u] * gg[u]);
    }
    *reinterpret_cast<float4*>(q + blockIdx.z * pstride + (size_t)c * G.csz + base) =
        make_float4(out[0], out[1], out[2], out[3]);
  }
  const double a = block_sum_d(spq.value(), sh);
  __syncthreads();
  const double b = block_sum_d(spg.value(), sh);
  if (threadIdx.x == 0) {
    const size_t slot = ((size_t)blockIdx.z * 2 + c) * gridDim.x + blockIdx.x;
    part[2 * slot] = a;
    part[2 * slot + 1] = b;
  }
}

// k_cg_dir and k_cg_matvec in one pass (grids with no size-1 axis): the new
// direction p = z + beta p_old is formed where it is read -- at the thread's
// own slots (stored to pn) and at their six neighbours -- so z and p_old are
// read once and p is written once.  p_old and pn are different arrays (a
// thread of one colour reads the other colour's p_old while that colour's
// threads store theirs).  Same expressions as the two kernels, same bits;
// the same grid (colour in y, problem in z).
// XM: the x half of the previous iteration's k_cg_update folded in at the
// thread's own slots, where p_old is read anyway: 0 none, 1 x = alpha p_old
// (the step's first update: x not read), 2 x += alpha p_old; alpha =
// scal[4b + 1], still the previous iteration's (k_cg_update's expression).
template <int XM>
__global__ void __launch_bounds__(kT, 4)
k_cg_matvec_dir(const float* __restrict__ z, const float* __restrict__ po,
                float* __restrict__ pn, const double* __restrict__ scal,
                const float* __restrict__ g, const uint8_t* __restrict__ mask, SGeo G,
                float* __restrict__ q, double* __restrict__ part, size_t pstride,
                float* __restrict__ x) {
  mask += (size_t)blockIdx.z * G.msplit;
  __shared__ double sh[kT / 32];
  const int c = blockIdx.y;
  const uint32_t nq = G.csz >> 2;
  const float b = (float)scal[4 * blockIdx.z + 2];
  KSum spq, spg;
  const size_t own = blockIdx.z * pstride + (size_t)c * G.csz;
  const size_t oth = blockIdx.z * pstride + (size_t)(1 - c) * G.csz;
  const DirLd on{z + oth, po + oth, b};
  for (uint32_t t = blockIdx.x * kT + threadIdx.x; t < nq; t += gridDim.x * kT) {
    const uint32_t ij = fdivu(t, G.dH4);
    const int m0 = 4 * (int)(t - ij * G.dH4.d);
    const int i = (int)fdivu(ij, G.dny);
    const int j = (int)(ij - (uint32_t)i * G.dny.d);
    const int pc = (i + j + c) & 1;
    const uint32_t base = ij * (uint32_t)G.H + m0;
    const uchar4 mk = *reinterpret_cast<const uchar4*>(mask + (size_t)c * G.csz + base);
    const uint8_t mv[4] = {mk.x, mk.y, mk.z, mk.w};
    const float4 pv = DirLd{z + own, po + own, b}.v4(base);
    *reinterpret_cast<float4*>(pn + own + base) = pv;
    if (XM) {
      const float al = (float)scal[4 * blockIdx.z + 1];
      const float4 pold = ld4(po + own + base);
      float4 xv = XM == 2 ? ld4(x + own + base) : make_float4(0.f, 0.f, 0.f, 0.f);
      xv.x = __fmaf_rn(al, pold.x, xv.x); xv.y = __fmaf_rn(al, pold.y, xv.y);
      xv.z = __fmaf_rn(al, pold.z, xv.z); xv.w = __fmaf_rn(al, pold.w, xv.w);
      *reinterpret_cast<float4*>(x + own + base) = xv;
    }
    const float4 gv = ld4(g + own + base);
    const float pp[4] = {pv.x, pv.y, pv.z, pv.w};
    const float gg[4] = {gv.x, gv.y, gv.z, gv.w};
    // the neighbour loads (in bounds in every group, padding included) do
    // not wait for the mask; it only selects
    float nb[4], out[4];
    nbr4(on, G, i, j, m0, pc, base, nb);
#pragma unroll
    for (int u = 0; u < 4; u++) out[u] = mv[u] ? 0.f : 6.0f * pp[u] - nb[u];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      spq.add(pp[u] * out[u]);
      spg.add(pp[u] * gg[u]);
    }
    *reinterpret_cast<float4*>(q + own + base) = make_float4(out[0], out[1], out[2], out[3]);
  }
  const double a = block_sum_d(spq.value(), sh);
  __syncthreads();
  const double bb = block_sum_d(spg.value(), sh);
  if (threadIdx.x == 0) {
    const size_t slot = ((size_t)blockIdx.z * 2 + c) * gridDim.x + blockIdx.x;
    part[2 * slot] = a;
    part[2 * slot + 1] = bb;
  }
}

// block partials of <z, q>: grid-stride over float4 groups, kCgBlocks
// blocks per problem
__global__ void __launch_bounds__(kT)
k_cg_dot(const float* __restrict__ z, const float* __restrict__ q,
         double* __restrict__ part, size_t pstride, uint32_t n) {
  __shared__ double sh[kT / 32];
  KSum s;
  const float* zb = z + blockIdx.y * pstride;
  const float* qb = q + blockIdx.y * pstride;
  for (uint32_t t = blockIdx.x * kT + threadIdx.x; t < n / 4; t += gridDim.x * kT) {
    const float4 a = ld4(zb + 4 * (size_t)t), b = ld4(qb + 4 * (size_t)t);
    s.add(a.x * b.x);
    s.add(a.y * b.y);
    s.add(a.z * b.z);
    s.add(a.w * b.w);
  }
  const double a = block_sum_d(s.value(), sh);
  if (threadIdx.x == 0) part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = a;
}

// Per-problem fixed-order sums of the partials.  mode 0: alpha from <p,q>
// and <p,g> (also keeps <p,q> for beta); mode 1: beta = -<z,q>/<p,q>.
// scal[4b + 0] = <p,q>, [1] = alpha, [2] = beta.
__global__ void __launch_bounds__(kT)
k_cg_reduce(const double* __restrict__ part, int nparts, int stride,
            double* __restrict__ scal, int mode) {
  __shared__ double sh[kT / 32];
  const int b = blockIdx.x;
  double a = 0.0, c = 0.0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) {
    const size_t o = (size_t)b * nparts + k;
    a += part[stride * o];
    if (stride == 2) c += part[stride * o + 1];
  }
  const double sa = block_sum_d(a, sh);
  __syncthreads();
  const double sc = block_sum_d(c, sh);
  if (threadIdx.x == 0) {
    double* S = scal + 4 * b;
    if (mode == 0) {
      S[0] = sa;
      S[1] = sa > 0.0 ? -sc / sa : 0.0;
    } else {
      S[2] = S[0] > 0.0 ? -sa / S[0] : 0.0;
    }
  }
}

// x += alpha p; g += alpha q (float4).  FIRST: the step's first iteration,
// where x is zero: x = alpha p + 0 (the same bits, without reading x).
template <bool FIRST>
__global__ void __launch_bounds__(kT)
k_cg_update(float* __restrict__ x, float* __restrict__ g, const float* __restrict__ p,
            const float* __restrict__ q, const double* __restrict__ scal,
            size_t pstride, uint32_t n) {
  const uint32_t t = blockIdx.x * kT + threadIdx.x;
  if (t >= n / 4) return;  // n: a multiple of 4 (split rows are)
  const float al = (float)scal[4 * blockIdx.y + 1];
  const size_t o = blockIdx.y * pstride + 4 * (size_t)t;
  float4 xv = FIRST ? make_float4(0.f, 0.f, 0.f, 0.f) : ld4(x + o);
  float4 gv = ld4(g + o);
  const float4 pv = ld4(p + o), qv = ld4(q + o);
  xv.x = __fmaf_rn(al, pv.x, xv.x); xv.y = __fmaf_rn(al, pv.y, xv.y);
  xv.z = __fmaf_rn(al, pv.z, xv.z); xv.w = __fmaf_rn(al, pv.w, xv.w);
  gv.x = __fmaf_rn(al, qv.x, gv.x); gv.y = __fmaf_rn(al, qv.y, gv.y);
  gv.z = __fmaf_rn(al, qv.z, gv.z); gv.w = __fmaf_rn(al, qv.w, gv.w);
  *reinterpret_cast<float4*>(x + o) = xv;
  *reinterpret_cast<float4*>(g + o) = gv;
}

// ---- host side ----------------------------------------------------------

#define MK(x)                                                                \
  do {                                                                       \
    cudaError_t e_ = (x);                                                    \
    if (e_ != cudaSuccess) {                                                 \
      set_last_error(std::string(#x) + ": " + cudaGetErrorString(e_));       \
      throw (int)IG_CUDA_ERROR;                                              \
    }                                                                        \
  } while (0)

// Stream-ordered device buffer, move-only.
template <class T>
struct Buf {
  T* p = nullptr;
  cudaStream_t s = nullptr;
  Buf() = default;
  Buf(const Buf&) = delete;
  Buf& operator=(const Buf&) = delete;
  Buf(Buf&& o) noexcept : p(o.p), s(o.s) { o.p = nullptr; }
  Buf& operator=(Buf&& o) noexcept {
    release();
    p = o.p;
    s = o.s;
    o.p = nullptr;
    return *this;
  }
  void alloc(size_t n, cudaStream_t st) {
    release();
    s = st;
    MK(cudaMallocAsync((void**)&p, std::max<size_t>(n * sizeof(T), 256), st));
  }
  void release() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
  }
  ~Buf() { release(); }
};

struct MLevel {
  Dims d;
  SGeo G;
  Buf<uint8_t> nat;    // natural mask (source of the next coarsening)
  Buf<uint8_t> mask;   // split mask
  Buf<float> e, g, r;  // split e, g (per problem); natural r (per problem)
  size_t pstride = 0;  // 2 * csz
  size_t rstride = 0;  // n
};

unsigned nblk(uint32_t n) { return (n + kT - 1) / kT; }

double omega_of(const Dims& d) {
  double num = 0.0, w = 0.0;
  const long ns[3] = {d.nx, d.ny, d.nz};
  for (long q : ns)
    if (q >= 2) { num += std::cos(M_PI / (double)(q + 1)); w += 1.0; }
  if (w == 0) return 1.0;
  const double rho = std::min(num / w, 1.0 - 1e-15);
  return 2.0 / (1.0 + std::sqrt(1.0 - rho * rho));
}

bool is_bottom(const Dims& d) {
  return d.n() <= (size_t)kBottomMax || (d.nx <= 2 && d.ny <= 2 && d.nz <= 2);
}

// Device bytes a session holds (for admission control by HBM footprint).
size_t session_bytes(Dims fine, int bmax, int nmetal = 1) {
  // fine masks, phi, masks/values staging
  size_t b = fine.n() * ((size_t)nmetal + 8 * (size_t)bmax + (size_t)bmax);
  Dims d = fine;
  while (true) {
    const size_t csz = (size_t)d.nx * d.ny * (size_t)((((d.nz + 1) / 2) + 3) & ~3L);
    b += (d.n() + 2 * csz) * (size_t)nmetal + 2 * (2 * csz * 4 * (size_t)bmax);
    // level 0: the flexible CG's correction, two direction buffers, L p and
    // the second right-hand side buffer
    if (d.n() == fine.n()) b += 5 * (2 * csz * 4 * (size_t)bmax);
    if (is_bottom(d)) break;
    b += std::max(d.n(), 2 * csz) * 4 * (size_t)bmax;
    d = coarse_of(d);
  }
  return b + 8 * (size_t)bmax;
}

// Kernel launches the mixed path issued (graph replays count every node).
std::atomic<long> g_mixed_launches{0};

// Launch shape of the smoother: float4 groups per thread (1, 2, 4 spread a
// block apart; 8 = k_gs8, two consecutive groups of a row) and block size.
struct GsCfg {
  int ng = 1;
  int threads = 256;
  int tb = 0;  // half-sweeps per temporally blocked pass on the finest level; 0: none
  // what the tuner measured (us per half-sweep): the chosen separate shape,
  // and the best blocked depth (0 when none was timed) with its time
  float sep_us = 0.f, tb_us = 0.f;
  int tb_best = 0;
};

// One geometry resident on the device: the FP32 multigrid hierarchy for up
// to bmax problems, the FP64 potentials, and one CUDA graph per batch size.
struct Session {
  cudaStream_t s = nullptr;
  Dims d;
  int bmax = 1;
  int B = 1;  // problems of the current call
  int nmetal = 1;  // 1: one metal for every problem; bmax: problem p on metal p
  std::vector<MLevel> lv;
  Buf<long long> phi;   // refined potentials, fixed point (units 2^(fexp[b] - 56))
  Buf<int> fexp;        // per problem: the unit exponent E_b
  Buf<unsigned long long> vmax;  // per problem: the largest |Dirichlet value|
  Buf<uint8_t> fixed;   // natural fine mask
  Buf<uint8_t> stage;   // per-call staging of basis masks
  Buf<double> vstage;   // per-call staging of Dirichlet values
  Buf<unsigned long long> dmax;
  // flexible CG state (level 0, split FP32): correction x, direction p,
  // q = L p; dot-product partials and per-problem scalars
  Buf<float> xb, pb, qb;
  Buf<float> pb2;  // the other buffer of the direction (fused dir + matvec)
  Buf<float> g2;   // the finest level's other right-hand side buffer (fold)
  bool fold_on = true;     // IG_MIXED_FOLD=0: the separate k_cg_update launches
  bool fold_next = false;  // the next finest-level zero-start pair folds g += alpha q
  bool dot_on = true;      // IG_MIXED_DOT=0: <z, q> by k_cg_dot
  bool dot_next = false;   // the finest level's last half-sweep forms <z, q>
  bool dot_done = false;   // ... and did (its partial count in dot_nparts)
  int dot_nparts = 0;
  Buf<double> part, scal;
  int method = 1;            // 0: defect correction with `vcycles` cycles,
                             // 1: flexible CG preconditioned by one cycle
  int cg_iters = 3;          // CG iterations per FP64 refinement
  int nu1 = 2, nu2 = 2, vcycles = 2, bottom_pairs = 40;
  int gamma = 1;             // 1: V-cycle, 2: W-cycle (coarse levels twice)
  int gamma_levels = 64;     // the second coarse visit only from the finest levels
  // cycles of level l + 1 per visit of level l (the bottom is solved directly,
  // so once is enough there)
  int coarse_visits(size_t l) const {
    return (l + 2 < lv.size() && (int)l < gamma_levels) ? gamma : 1;
  }
  float smooth_omega = 1.f;  // red-black relaxation factor of the smoother
  double resid_scale = 1.0;
  float bottom_omega = 1.f;
  // captured refinement steps, by (batch size, direction parity)
  std::vector<std::pair<int, cudaGraphExec_t>> graphs;
  // which direction buffer holds the search direction at the start of the
  // next step: with an odd number of fused CG iterations a step ends in the
  // other buffer, and the next step (a graph captured with the buffers
  // swapped) starts there instead of copying it back
  bool p_in_b2 = false;
  GsCfg gs_cfg;          // smoother launch shape, from the tuner
  bool gs_tuned = false;
  // levels (finest first) whose smoothing phases run temporally blocked
  // (k_gs_tb: each phase's half-sweeps in one pass); 0 = separate launches.
  // Off by default: on the benchmark decks the blocked passes measured
  // slower than the separate half-sweeps (ring stack 77-86 against 126
  // solves/s; each plane of the march waits on a barrier and on loads that
  // one or two CTAs per SM cannot hide), although they move fewer bytes.
  int tb_levels = 0;
  int tb_max = 6;  // half-sweeps per blocked pass (2, 4 or 6); longer phases split
  bool tb_auto = true;  // the tuner picks tb_levels / tb_max (no environment override)
  bool tail_on = true;   // k_tail_cycle allowed (IG_MIXED_TAIL=0: the separate launches)
  bool tail_ok = false;  // ... and usable on this hierarchy
  double last_solve_bytes = 0.0;  // algorithmic bytes of the last solve's steps
  int rows_force = -1;  // rows per warp of the residual and update: -1 by rule (flat_rows)

  ~Session() {
    for (auto& g : graphs) cudaGraphExecDestroy(g.second);
    lv.clear();
    phi.release();
    fexp.release();
    vmax.release();
    fixed.release();
    stage.release();
    vstage.release();
    dmax.release();
    xb.release();
    pb.release();
    pb2.release();
    g2.release();
    qb.release();
    part.release();
    scal.release();
    if (s) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  }

  // The metal of every level: the fine mask, its coarsenings (injection
  // with the thin-metal rescue) and their split forms, into the level
  // buffers.  Nothing else of a session depends on the metal, so a session
  // can take another geometry of its shape (ig_mixed_rebind) and keep its
  // buffers, tuned smoother shape and captured graphs.
  // metal: nmetal stacked (nx, ny, nz) masks (nmetal = 1: one metal shared
  // by every problem; nmetal = bmax: problem p on metal p).
  void load_metal(const uint8_t* metal) {
    const size_t n = d.n();
    MK(cudaMemcpyAsync(fixed.p, metal, n * nmetal, cudaMemcpyDefault, s));
    Buf<uint8_t> inj;
    if (lv.size() > 1) inj.alloc(lv[1].G.n, s);
    for (int q = 0; q < nmetal; q++)
      for (size_t l = 0; l < lv.size(); l++) {
        MLevel& L = lv[l];
        uint8_t* nat = L.nat.p + (size_t)q * L.G.n;
        if (l == 0) {
          MK(cudaMemcpyAsync(nat, fixed.p + (size_t)q * n, n, cudaMemcpyDeviceToDevice, s));
        } else {
          const MLevel& F = lv[l - 1];
          const uint8_t* fnat = F.nat.p + (size_t)q * F.G.n;
          k_coarsen_inject<<<nblk(L.G.n), kT, 0, s>>>(fnat, F.G, inj.p, L.G);
          MK(cudaGetLastError());
          k_coarsen_rescue<<<nblk(L.G.n), kT, 0, s>>>(fnat, F.G, inj.p, nat, L.G);
          MK(cudaGetLastError());
        }
        uint8_t* mk = L.mask.p + (size_t)q * 2 * L.G.csz;
        MK(cudaMemsetAsync(mk, 1, 2 * (size_t)L.G.csz, s));  // unused slots: metal
        k_split_mask<<<nblk(L.G.n), kT, 0, s>>>(nat, L.G, mk);
        MK(cudaGetLastError());
      }
    g_mixed_launches.fetch_add(3L * (long)lv.size() * nmetal);
  }

  void build(const uint8_t* metal) {
    const size_t n = d.n();
    fixed.alloc(n * nmetal, s);
    Dims c = d;
    while (true) {
      MLevel L;
      L.d = c;
      L.G = sgeo(c);
      if (nmetal > 1) {
        L.G.msplit = 2 * L.G.csz;
        L.G.mnat = (uint32_t)n;  // the natural mask is read on level 0 only
      }
      L.nat.alloc(c.n() * nmetal, s);
      L.mask.alloc(2 * (size_t)L.G.csz * nmetal, s);
      L.pstride = 2 * (size_t)L.G.csz;
      L.rstride = L.G.n;
      L.e.alloc(L.pstride * bmax, s);
      L.g.alloc(L.pstride * bmax, s);
      MK(cudaMemsetAsync(L.e.p, 0, L.pstride * bmax * 4, s));
      MK(cudaMemsetAsync(L.g.p, 0, L.pstride * bmax * 4, s));
      const bool bottom = is_bottom(c);
      L.rstride = std::max<size_t>(L.G.n, L.G.csz);
      // r doubles as the output array of the blocked post-smoothing (the
      // two swap roles), so it holds a whole split correction per problem
      if (!bottom) L.r.alloc(std::max(L.rstride, L.pstride) * bmax, s);
      lv.push_back(std::move(L));
      if (bottom) break;
      c = coarse_of(c);
    }
    load_metal(metal);
    bottom_omega = (float)omega_of(lv.back().d);
    update_tail();
    if (tb_levels > 0) MK(tb_prepare());
    phi.alloc(n * bmax, s);
    fexp.alloc(bmax, s);
    vmax.alloc(bmax, s);
    dmax.alloc(bmax, s);
    if (method == 1) {
      const size_t ps = lv[0].pstride * bmax;
      xb.alloc(ps, s);
      pb.alloc(ps, s);
      if (!flat(lv[0])) {
        pb2.alloc(ps, s);
        g2.alloc(ps, s);
      }
      qb.alloc(ps, s);
      const size_t nb4 = nblk(lv[0].G.csz / 4), nbn = nblk((uint32_t)lv[0].pstride);
      part.alloc(std::max(4 * nb4, nbn) * bmax, s);
      scal.alloc(4 * bmax, s);
    }
    MK(cudaGetLastError());
  }

  // One colour half-sweep of level a for nb problems with the tuned shape.
  void launch_gs(MLevel& a, int c, int nb, float omega) {
    const uint32_t nq = a.G.csz / 4;
    if (a.G.nx == 1 || a.G.ny == 1 || a.G.nz == 1) {
      k_gs4<1, true><<<dim3(nblk(nq), nb), kT, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G, c, omega,
                                                      a.pstride);
      return;
    }
    const unsigned per = (unsigned)(gs_cfg.threads * gs_cfg.ng);
    const dim3 grid((nq + per - 1) / per, nb);
    if (gs_cfg.ng == 8) {
      const uint32_t npair = (uint32_t)a.G.nx * a.G.ny * a.G.dH8.d;
      const dim3 g8((npair + gs_cfg.threads - 1) / gs_cfg.threads, nb);
      k_gs8<false><<<g8, gs_cfg.threads, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G, c, omega,
                                                 a.pstride);
      return;
    }
    switch (gs_cfg.ng) {
      case 4:
        k_gs4<4, false><<<grid, gs_cfg.threads, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G, c, omega,
                                                        a.pstride);
        break;
      case 2:
        k_gs4<2, false><<<grid, gs_cfg.threads, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G, c, omega,
                                                        a.pstride);
        break;
      default:
        k_gs4<1, false><<<grid, gs_cfg.threads, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G, c, omega,
                                                        a.pstride);
        break;
    }
  }

  // The finest level's last half-sweep with <z, q> folded in (k_gs4_dot):
  // its partials go to `part`, their count to dot_nparts.  Returns false
  // (nothing launched) where the tuned shape has no such form.
  bool launch_gs_dot(MLevel& a, int c, int nb, float omega) {
    if (flat(a) || gs_cfg.ng == 8) return false;
    const uint32_t nq = a.G.csz / 4;
    const unsigned per = (unsigned)(gs_cfg.threads * gs_cfg.ng);
    const dim3 grid((nq + per - 1) / per, nb);
    switch (gs_cfg.ng) {
      case 4:
        k_gs4_dot<4><<<grid, gs_cfg.threads, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G, c, omega,
                                                      a.pstride, qb.p, part.p);
        break;
      case 2:
        k_gs4_dot<2><<<grid, gs_cfg.threads, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G, c, omega,
                                                      a.pstride, qb.p, part.p);
        break;
      default:
        k_gs4_dot<1><<<grid, gs_cfg.threads, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G, c, omega,
                                                      a.pstride, qb.p, part.p);
        break;
    }
    dot_nparts = (int)grid.x;
    return true;
  }

  // The smoother's launch shape (groups per thread x block size) and its
  // temporal-block depth, timed on this grid's finest level for nb
  // problems: three red-black pairs per shape after one warm pair, the
  // fastest kept; then passes of 2, 4 and 6 half-sweeps in one temporally
  // blocked launch (k_gs_tb, e into r: two timed after a warm one), taken
  // for the finest level when one costs at least 15 % less per half-sweep
  // than the best separate launch.  Either choice gives the same bits.  Shapes are cached
  // per (grid, problem count) for the process.  Runs before the first graph
  // capture; the level-0 correction and residual it scribbles on are
  // rewritten before use.  IG_MIXED_TB_LEVELS, when set, fixes the blocking
  // instead.
  void apply_tb(const GsCfg& c) {
    if (!tb_auto) return;
    tb_levels = c.tb > 0 ? 1 : 0;
    if (c.tb > 0) tb_max = c.tb;
  }
  void tune_gs(int nb) {
    static std::mutex mu;
    static std::map<std::array<long, 5>, GsCfg> cache;
    const std::array<long, 5> key{d.nx, d.ny, d.nz, (long)nb, tb_auto ? 1L : 0L};
    {
      std::lock_guard<std::mutex> lk(mu);
      auto it = cache.find(key);
      if (it != cache.end()) {
        gs_cfg = it->second;
        apply_tb(gs_cfg);
        gs_tuned = true;
        return;
      }
    }
    MLevel& f = lv[0];
    cudaEvent_t e0, e1;
    MK(cudaEventCreate(&e0));
    MK(cudaEventCreate(&e1));
    GsCfg best;
    float best_ms = 1e30f;
    long launches = 0;
    for (int ng : {1, 2, 4, 8})
      for (int th : {128, 256, 512}) {
        gs_cfg.ng = ng;
        gs_cfg.threads = th;
        for (int c = 0; c < 2; c++) launch_gs(f, c, nb, 1.f);
        MK(cudaEventRecord(e0, s));
        for (int q = 0; q < 3; q++)
          for (int c = 0; c < 2; c++) launch_gs(f, c, nb, 1.f);
        MK(cudaEventRecord(e1, s));
        MK(cudaEventSynchronize(e1));
        float ms = 0.f;
        MK(cudaEventElapsedTime(&ms, e0, e1));
        launches += 8;
        if (ms < best_ms) {
          best_ms = ms;
          best = gs_cfg;
        }
      }
    best.tb = 0;
    best.sep_us = 1e3f * best_ms / 6.f;
    if (tb_auto && lv.size() > 1 && !flat(f) && smooth_omega == 1.f) {
      MK(tb_prepare());
      float best_per = best_ms / 6.f, tb_per = 1e30f;
      for (int S2 : {2, 4, 6}) {
        launch_tb(S2, false, 1, f.e.p, f.r.p, f.g.p, f.mask.p, f.G, f.pstride, nb, s);
        MK(cudaEventRecord(e0, s));
        for (int q = 0; q < 2; q++)
          launch_tb(S2, false, 1, f.e.p, f.r.p, f.g.p, f.mask.p, f.G, f.pstride, nb, s);
        MK(cudaEventRecord(e1, s));
        MK(cudaEventSynchronize(e1));
        float ms = 0.f;
        MK(cudaEventElapsedTime(&ms, e0, e1));
        MK(cudaGetLastError());
        launches += 3;
        const float per = ms / (2.f * S2);
        if (per < tb_per) {
          tb_per = per;
          best.tb_best = S2;
          best.tb_us = 1e3f * per;
        }
        // blocking must win by a clear margin: the separate launches pay a
        // per-launch cost that a concurrent stream or a profiler inflates
        // far more than the blocked pass's, and blocking measured slower on
        // every grid the benchmarks use
        if (per < 0.85f * best_per) {
          best_per = per;
          best.tb = S2;
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    g_mixed_launches.fetch_add(launches);
    gs_cfg = best;
    apply_tb(best);
    gs_tuned = true;
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = best;
  }

  static bool flat(const MLevel& a) { return a.G.nx == 1 || a.G.ny == 1 || a.G.nz == 1; }
  static bool two_or_more(const MLevel& a) { return a.G.nx > 1 && a.G.ny > 1 && a.G.nz > 1; }

  // fine a.e += trilinear(coarse b.e) for colours 0 .. ncol-1
  void launch_prolong(MLevel& b, MLevel& a, int nb, unsigned ncol) {
    const dim3 grid(nblk(a.G.csz / 4), nb, ncol);
    if (two_or_more(a) && two_or_more(b))
      k_prolong_add4<<<grid, kT, 0, s>>>(b.e.p, b.G, a.e.p, a.mask.p, a.G, b.pstride, a.pstride);
    else
      k_prolong_add4_gather<<<grid, kT, 0, s>>>(b.e.p, b.G, a.e.p, a.mask.p, a.G, b.pstride,
                                                a.pstride);
  }

  // the direction update and the operator apply fuse on grids with no
  // size-1 axis (two direction buffers)
  bool fuse_dir() const { return pb2.p != nullptr; }

  // The first pre-smoothing pair from e = 0 runs as one fused pass.
  // The level just above the bottom cycles in one CTA per problem
  // (k_tail_cycle) when its arrays fit in shared memory; set at build and
  // when the cycle changes.
  void update_tail() {
    tail_ok = false;
    if (tail_on && lv.size() >= 2) {
      const MLevel& ta = lv[lv.size() - 2];
      const MLevel& tb = lv.back();
      tail_ok = !flat(ta) && two_or_more(ta) && two_or_more(tb) && smooth_omega == 1.f &&
                nu1 >= 1 && nu2 >= 1 && tail_smem_bytes(ta.G, tb.G) <= kTailSmemMax;
      if (tail_ok)
        MK(cudaFuncSetAttribute(k_tail_cycle, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kTailSmemMax));
    }
  }

  // level l's cycle from zero runs as k_tail_cycle (l the last level above
  // the bottom, no temporal blocking there)
  bool tail_level(size_t l) const { return tail_ok && l + 2 == lv.size() && !use_tb(l); }

  bool fuse_zero_pair(const MLevel& a) const {
    return nu1 >= 1 && smooth_omega == 1.f && !flat(a);
  }

  // Temporally blocked smoothing on level l (k_gs_tb): grids with no
  // size-1 axis, Gauss-Seidel (omega 1), phases of 1..3 pairs.
  bool use_tb(size_t l) const {
    return (int)l < tb_levels && l + 1 < lv.size() && !flat(lv[l]) && smooth_omega == 1.f;
  }

  // One cycle on level l.  zero: the level's correction starts at 0 (the
  // cycle zeroes it, or its first Gauss-Seidel pair writes every slot).
  void vcycle(size_t l, bool zero) {
    MLevel& a = lv[l];
    const dim3 gs(nblk(a.G.csz), B), gn(nblk(a.G.n), B);
    if (l + 1 == lv.size()) {
      k_bottom<<<B, kBottomThreads, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G, bottom_omega,
                                            bottom_pairs, a.pstride);
      return;
    }
    if (zero && tail_level(l)) {
      const MLevel& b = lv[l + 1];
      k_tail_cycle<<<B, kBottomThreads, tail_smem_bytes(a.G, b.G), s>>>(
          a.e.p, a.g.p, a.mask.p, a.G, a.pstride, b.mask.p, b.G, nu1, nu2, bottom_omega,
          bottom_pairs);
      return;
    }
    int q0 = 0;
    if (tb_pre(l, zero)) {
      // the pre-smoothing from e = 0 in passes of up to tb_max half-sweeps:
      // the first reads no e and writes it in place, the others go from e
      // into r, which then serves as the correction
      int left = 2 * nu1;
      bool first = true;
      while (left > 0) {
        const int S2 = std::min(left, tb_max);
        if (first) {
          launch_tb(S2, true, 0, a.e.p, a.e.p, a.g.p, a.mask.p, a.G, a.pstride, B, s);
        } else {
          launch_tb(S2, false, 0, a.e.p, a.r.p, a.g.p, a.mask.p, a.G, a.pstride, B, s);
          std::swap(a.e, a.r);
        }
        first = false;
        left -= S2;
      }
      q0 = nu1;
    } else if (zero && fuse_zero_pair(a) && l == 0 && fold_next) {
      // the previous CG iteration's g += alpha q, folded in: the updated
      // right-hand side goes to the other buffer, which becomes the level's
      k_gs_zero_pair_fold<<<dim3(nblk(a.G.csz / 4), B), kT, 0, s>>>(
          a.e.p, a.g.p, qb.p, scal.p, g2.p, a.mask.p, a.G, a.pstride);
      std::swap(a.g.p, g2.p);
      fold_next = false;
      q0 = 1;
    } else if (zero && fuse_zero_pair(a)) {
      k_gs_zero_pair<<<dim3(nblk(a.G.csz / 4), B), kT, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G,
                                                              a.pstride);
      q0 = 1;
    } else if (zero) {
      MK(cudaMemsetAsync(a.e.p, 0, a.pstride * B * 4, s));
    }
    for (int q = q0; q < nu1; q++)
      for (int c = 0; c < 2; c++) launch_gs(a, c, B, smooth_omega);
    MLevel& b = lv[l + 1];
    if (nu1 > 0 && smooth_omega == 1.f) {
      // Gauss-Seidel ended on colour 1: its residual is zero
      if (flat(a))
        k_resid0<<<gs, kT, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G, a.r.p, a.pstride);
      else
        k_resid0_4<<<dim3(nblk(a.G.csz / 4), B), kT, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G,
                                                            a.r.p, a.pstride);
      k_restrict0_4<<<dim3(nblk((uint32_t)b.G.nx * b.G.ny * ((b.G.nz + 3) / 4)), B), kT, 0, s>>>(
          a.r.p, a.G, b.g.p, b.G, b.pstride);
    } else {
      k_resid<<<gn, kT, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G, a.r.p, a.pstride, a.rstride);
      k_restrict<<<dim3(nblk(b.G.n), B), kT, 0, s>>>(a.r.p, a.G, b.g.p, b.G, a.rstride, b.pstride);
    }
    // the coarse correction: gamma cycles on the coarse equation from 0
    // (the bottom is solved directly, so once is enough there)
    const int reps = coarse_visits(l);
    for (int q = 0; q < reps; q++) vcycle(l + 1, q == 0);
    // The first post-smoothing half-sweep (colour 1, omega 1) overwrites
    // every free colour-1 slot without reading it, so only colour 0 takes
    // the prolonged correction then.
    const unsigned pcol = (nu2 >= 1 && smooth_omega == 1.f) ? 1u : 2u;
    launch_prolong(b, a, B, pcol);
    // post-smoothing in the reverse colour order keeps the cycle symmetric
    if (tb_post(l)) {
      // in passes of up to tb_max half-sweeps, each from e into r, which
      // then serves as the correction
      for (int left = 2 * nu2; left > 0;) {
        const int S2 = std::min(left, tb_max);
        launch_tb(S2, false, 1, a.e.p, a.r.p, a.g.p, a.mask.p, a.G, a.pstride, B, s);
        std::swap(a.e, a.r);
        left -= S2;
      }
      return;
    }
    for (int q = 0; q < nu2; q++)
      for (int c = 1; c >= 0; c--) {
        if (l == 0 && dot_next && q + 1 == nu2 && c == 0 &&
            launch_gs_dot(a, c, B, smooth_omega)) {
          dot_next = false;
          dot_done = true;
          continue;
        }
        launch_gs(a, c, B, smooth_omega);
      }
  }

  // the finest level's FP64 residual and potential update, one warp per
  // natural row or, for short rows, several rows per warp (flat_rows)
  void launch_resid64() {
    MLevel& f = lv[0];
    const uint32_t R = flat_rows(f.G, rows_force);
    if (R == 1)
      k_resid64<<<dim3(rows_blocks(f.G), B), kT, 0, s>>>(phi.p, fixed.p, f.G, f.g.p, fexp.p,
                                                         (float)-resid_scale, f.G.n, f.pstride);
    else
      k_resid64_flat<<<dim3(flat_blocks(f.G, R), B), kT, 0, s>>>(
          phi.p, fixed.p, f.G, f.g.p, fexp.p, (float)-resid_scale, f.G.n, f.pstride, R);
  }
  void launch_update64(const float* e, unsigned long long* dm, const float* p,
                       const double* sc) {
    MLevel& f = lv[0];
    const uint32_t R = flat_rows(f.G, rows_force);
    if (R == 1)
      k_update64<<<dim3(rows_blocks(f.G), B), kT, 0, s>>>(phi.p, fixed.p, e, f.G, dm, fexp.p,
                                                          f.G.n, f.pstride, p, sc);
    else
      k_update64_flat<<<dim3(flat_blocks(f.G, R), B), kT, 0, s>>>(
          phi.p, fixed.p, e, f.G, dm, fexp.p, f.G.n, f.pstride, p, sc, R);
  }

  // one refinement step: FP64 residual, V-cycles on the correction, update
  void step_enqueue() {
    MLevel& f = lv[0];
    launch_resid64();
    for (int v = 0; v < vcycles; v++) vcycle(0, v == 0);
    MK(cudaMemsetAsync(dmax.p, 0, 8 * B, s));
    launch_update64(f.e.p, dmax.p, nullptr, nullptr);
  }

  // the flexible CG: once per solve, the FP64 residual and zero state
  void cg_init() {
    MLevel& f = lv[0];
    launch_resid64();
    MK(cudaMemsetAsync(xb.p, 0, f.pstride * B * 4, s));
    MK(cudaMemsetAsync(pb.p, 0, f.pstride * B * 4, s));
    p_in_b2 = false;
    MK(cudaMemsetAsync(qb.p, 0, f.pstride * B * 4, s));
    MK(cudaMemsetAsync(scal.p, 0, 4 * B * 8, s));
  }

  // cg_iters preconditioned iterations, then the reliable update: the FP32
  // correction is added to the FP64 potential, whose exact FP64 residual
  // replaces the carried one (the search direction is kept)
  void cg_enqueue(bool from_b2) {
    MLevel& f = lv[0];
    const uint32_t n = (uint32_t)f.pstride;
    const dim3 gv(nblk(n), B);
    const unsigned nb4 = std::min(nblk(f.G.csz / 4), kCgBlocks);
    const unsigned nbd = std::min(nblk(n / 4), kCgBlocks);
    float* pcur = from_b2 ? pb2.p : pb.p;
    float* pnext = from_b2 ? pb.p : pb2.p;
    const bool fold = fold_ok();
    for (int it = 0; it < cg_iters; it++) {
      // with fold, iteration it > 0 takes the previous iteration's
      // k_cg_update in two halves: g += alpha q in the finest level's
      // zero-start pair, x += alpha p_old in the direction update
      fold_next = fold && it > 0;
      dot_next = dot_on;
      dot_done = false;
      vcycle(0, true);  // z = f.e
      dot_next = false;
      if (dot_done) {
        // <z, q> was formed by the cycle's last half-sweep
        k_cg_reduce<<<B, kT, 0, s>>>(part.p, dot_nparts, 1, scal.p, 1);
      } else {
        k_cg_dot<<<dim3(nbd, B), kT, 0, s>>>(f.e.p, qb.p, part.p, f.pstride, n);
        k_cg_reduce<<<B, kT, 0, s>>>(part.p, (int)nbd, 1, scal.p, 1);
      }
      if (fuse_dir()) {
        const dim3 gm(nb4, 2, B);
        if (!fold || it == 0)
          k_cg_matvec_dir<0><<<gm, kT, 0, s>>>(f.e.p, pcur, pnext, scal.p, f.g.p, f.mask.p,
                                               f.G, qb.p, part.p, f.pstride, nullptr);
        else if (it == 1)
          k_cg_matvec_dir<1><<<gm, kT, 0, s>>>(f.e.p, pcur, pnext, scal.p, f.g.p, f.mask.p,
                                               f.G, qb.p, part.p, f.pstride, xb.p);
        else
          k_cg_matvec_dir<2><<<gm, kT, 0, s>>>(f.e.p, pcur, pnext, scal.p, f.g.p, f.mask.p,
                                               f.G, qb.p, part.p, f.pstride, xb.p);
        std::swap(pcur, pnext);
      } else {
        k_cg_dir<<<gv, kT, 0, s>>>(pcur, f.e.p, scal.p, f.pstride, n);
        k_cg_matvec<<<dim3(nb4, 2, B), kT, 0, s>>>(pcur, f.g.p, f.mask.p, f.G, qb.p, part.p,
                                                  f.pstride);
      }
      k_cg_reduce<<<B, kT, 0, s>>>(part.p, 2 * (int)nb4, 2, scal.p, 0);
      // the last iteration's x += alpha p is folded into the FP64 update
      // below; the first one writes x = alpha p (no zeroing pass)
      if (fold)
        ;  // taken by the next iteration's zero-start pair and direction update
      else if (it == 0 && cg_iters > 1)
        k_cg_update<true><<<dim3(nblk(n / 4), B), kT, 0, s>>>(xb.p, f.g.p, pcur, qb.p, scal.p,
                                                             f.pstride, n);
      else if (it + 1 < cg_iters)
        k_cg_update<false><<<dim3(nblk(n / 4), B), kT, 0, s>>>(xb.p, f.g.p, pcur, qb.p, scal.p,
                                                              f.pstride, n);
    }
    MK(cudaMemsetAsync(dmax.p, 0, 8 * B, s));
    // phi += x + alpha p (x absent when the step has one iteration)
    launch_update64(cg_iters > 1 ? xb.p : nullptr, dmax.p, pcur, scal.p);
    launch_resid64();
  }

  // a step ends with the direction in the other buffer when the fused CG
  // runs an odd number of iterations
  bool step_swaps() const { return method == 1 && fuse_dir() && (cg_iters & 1); }

  // The CG update folded into the next iteration (k_gs_zero_pair_fold,
  // k_cg_matvec_dir<1|2>): the finest level starts its cycle with the fused
  // zero-start pair, the direction update is fused, and the iterations are
  // odd in number, so the right-hand side buffers swap an even number of
  // times per step and every captured step starts and ends on the same one.
  // <z, q> formed by the finest level's last half-sweep (k_gs4_dot; the
  // conditions under which vcycle reaches launch_gs_dot)
  bool dot_fused() const {
    return dot_on && method == 1 && lv.size() > 1 && !tail_level(0) && !tb_post(0) &&
           nu2 >= 1 && !flat(lv[0]) && gs_cfg.ng != 8;
  }

  bool fold_ok() const {
    return fold_on && method == 1 && fuse_dir() && g2.p != nullptr && cg_iters > 1 &&
           (cg_iters & 1) && fuse_zero_pair(lv[0]) && !tb_pre(0, true) && !tail_level(0) &&
           lv.size() > 1;
  }

  void step() {
    const bool from_b2 = method == 1 && p_in_b2;
    const int key = 2 * B + (from_b2 ? 1 : 0);
    cudaGraphExec_t exec = nullptr;
    for (auto& g : graphs)
      if (g.first == key) exec = g.second;
    if (!exec) {
      if (!gs_tuned) tune_gs(B);
      cudaGraph_t graph;
      MK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      if (method == 1)
        cg_enqueue(from_b2);
      else
        step_enqueue();
      MK(cudaStreamEndCapture(s, &graph));
      MK(cudaGraphInstantiate(&exec, graph, 0));
      MK(cudaGraphDestroy(graph));
      graphs.push_back({key, exec});
    }
    MK(cudaGraphLaunch(exec, s));
    if (step_swaps()) p_in_b2 = !p_in_b2;
  }

  // kernel launches of one cycle on level l (memsets are not kernels)
  bool tb_pre(size_t l, bool zero) const { return zero && nu1 >= 1 && use_tb(l); }
  bool tb_post(size_t l) const { return nu2 >= 1 && use_tb(l); }
  int tb_passes(int stages) const { return (stages + tb_max - 1) / tb_max; }

  long cycle_launches(size_t l, bool zero) const {
    if (l + 1 == lv.size()) return 1;
    if (zero && tail_level(l)) return 1;
    const int reps = coarse_visits(l);
    long n = 3;                                         // residual, restriction, prolongation
    if (tb_pre(l, zero)) n += tb_passes(2 * nu1);
    else n += 2 * nu1 - ((zero && fuse_zero_pair(lv[l])) ? 1 : 0);
    n += tb_post(l) ? tb_passes(2 * nu2) : 2 * nu2;
    for (int q = 0; q < reps; q++) n += cycle_launches(l + 1, q == 0);
    return n;
  }

  // Algorithmic DRAM bytes of one cycle on level l, per problem: the bytes
  // each kernel must move (its inputs read once, its outputs written once),
  // as the kernel table of the design notes counts them.
  double cycle_bytes(size_t l, bool zero) const {
    const MLevel& a = lv[l];
    const double n = (double)a.G.n;
    if (l + 1 == lv.size()) return 9.0 * n;            // g, mask in; e out
    // k_tail_cycle: g and mask in, e out, the bottom's mask in
    if (zero && tail_level(l)) return 9.0 * n + (double)lv[l + 1].G.n;
    double b = 0.0;
    int q0 = 0;
    if (tb_pre(l, zero)) {
      // g, mask in, e out; the later passes read one colour of e too
      b += 9.0 * n + 11.0 * n * (tb_passes(2 * nu1) - 1);
      q0 = nu1;
    } else if (zero && fuse_zero_pair(a)) {
      b += 9.0 * n;
      q0 = 1;
    } else if (zero) {
      b += 4.0 * n;                                     // memset of e
    }
    b += 2.0 * (nu1 - q0) * 6.5 * n;                    // half-sweeps
    const double nc = (double)lv[l + 1].G.n;
    if (nu1 > 0 && smooth_omega == 1.f)
      b += 8.5 * n + 2.0 * n + 4.0 * nc;                // colour-0 residual, restriction
    else
      b += 13.0 * n + 4.0 * n + 4.0 * nc;
    const int reps = coarse_visits(l);
    for (int q = 0; q < reps; q++) b += cycle_bytes(l + 1, q == 0);
    const bool one = nu2 >= 1 && smooth_omega == 1.f;
    b += (one ? 4.5 : 9.0) * n;                         // prolongation
    // blocked: one colour of e, g and the mask in, e out
    b += tb_post(l) ? 11.0 * n * tb_passes(2 * nu2) : 2.0 * nu2 * 6.5 * n;
    return b;
  }

  // Algorithmic bytes of one refinement step for nb problems.
  double step_bytes(int nb) const {
    const double n = (double)lv[0].G.n;
    double b = 0.0;
    if (method == 1) {
      const bool fold = fold_ok();
      for (int it = 0; it < cg_iters; it++) {
        b += cycle_bytes(0, true);
        b += (dot_fused() ? 4.0 : 8.0) * n;             // <z, q> (q only when fused)
        b += (fuse_dir() ? 21.0 : 33.0) * n;            // direction, L p
        if (fold) {
          // q in, the updated g out (zero-start pair); x out / in and out
          if (it > 0) b += 8.0 * n + (it == 1 ? 4.0 : 8.0) * n;
        } else if (it == 0 && cg_iters > 1) {
          b += 20.0 * n;                                // x = a p, g += a q
        } else if (it + 1 < cg_iters) {
          b += 24.0 * n;
        }
      }
      b += (cg_iters > 1 ? 25.0 : 21.0) * n;            // phi += x + a p
    } else {
      for (int v = 0; v < vcycles; v++) b += cycle_bytes(0, v == 0);
      b += 21.0 * n;                                    // phi += e
    }
    b += 13.0 * n;                                      // FP64 residual
    return b * nb;
  }

  long launches_per_step() const {
    // per iteration: dot, two reductions, direction + L p (one launch when
    // fused) and, on all but the last, the CG update; then update64, resid64
    if (method == 1)
      return 2 + cg_iters * (cycle_launches(0, true) + (fuse_dir() ? 4 : 5) -
                             (dot_fused() ? 1 : 0)) +
             (fold_ok() ? 0 : cg_iters - 1);
    long n = 2;
    for (int v = 0; v < vcycles; v++) n += cycle_launches(0, v == 0);
    return n;
  }
};

struct MixedResult {
  int status;
  int steps;
  std::vector<double> dmax;
  long launches;  // kernel launches of the steps
  double bytes;   // algorithmic bytes of the steps
};

// Refinement steps until every problem is within acc of its converged
// potential.  With d_k the max |change| applied by step k and
// rho_k = d_k / d_{k-1} its observed contraction, the error left after step k
// is the sum of the later changes, d_{k+1} + d_{k+2} + ... (measured against
// the converged FP64 solution on the benchmark decks: within a few percent
// of d_{k+1}).  rho_{k+1} is estimated as kRhoSafety times the larger of the
// last two observed ratios, and a problem is done when the geometric tail
// d_k rho / (1 - rho) of that estimate is below acc (or when d_k is 0).  The
// first step has no ratio and never stops a problem with a nonzero change.
constexpr double kRhoSafety = 3.0;

MixedResult run_mixed(Session& M, const double* acc, int max_steps) {
  if (M.method == 1) M.cg_init();
  std::vector<unsigned long long> h(M.B);
  std::vector<double> prev(M.B, INFINITY), prev_rho(M.B, 0.0);
  MixedResult res{IG_NOT_CONVERGED, 0, std::vector<double>(M.B, 0.0), 0, 0.0};
  for (int it = 0; it < max_steps; it++) {
    M.step();
    res.launches += M.launches_per_step();
    res.bytes += M.step_bytes(M.B);
    MK(cudaMemcpyAsync(h.data(), M.dmax.p, 8 * M.B, cudaMemcpyDeviceToHost, M.s));
    MK(cudaStreamSynchronize(M.s));
    res.steps = it + 1;
    bool all = true;
    for (int b = 0; b < M.B; b++) {
      const double d = bits_to_double(h[b]);
      res.dmax[b] = d;
      const double r = std::isfinite(prev[b]) && prev[b] > 0 ? d / prev[b] : 1.0;
      const double rho = std::min(kRhoSafety * std::max(r, prev_rho[b]), 0.95);
      const double tail = d * rho / (1.0 - rho);
      if (!(tail < acc[b]) && !(d == 0.0)) all = false;
      prev[b] = d;
      prev_rho[b] = r;
    }
    if (all) {
      res.status = IG_OK;
      break;
    }
  }
  M.last_solve_bytes = res.bytes;
  return res;
}


// The unit exponent of each problem from its largest |Dirichlet value|
// (|value| < 2^E), uploaded to fexp; refuses magnitudes outside
// [2^-61, 2^60) and non-finite values.
void set_units(Session& S, const std::vector<double>& vmax) {
  std::vector<int> e(S.B);
  for (int b = 0; b < S.B; b++) {
    const double m = vmax[b];
    if (!(m < 1.152921504606846976e18)) {  // 2^60, NaN included
      set_last_error("mixed-precision solve: a Dirichlet value is not finite or of "
                     "magnitude 2^60 or more");
      throw (int)IG_BAD_ARG;
    }
    int ex = 0;
    if (m > 0.0) std::frexp(m, &ex);  // m = f 2^ex, f in [0.5, 1): m < 2^ex
    if (m > 0.0 && ex < -60) {
      set_last_error("mixed-precision solve: the Dirichlet values are all below 2^-61 in "
                     "magnitude");
      throw (int)IG_BAD_ARG;
    }
    e[b] = ex;
  }
  MK(cudaMemcpyAsync(S.fexp.p, e.data(), 4 * S.B, cudaMemcpyHostToDevice, S.s));
  MK(cudaStreamSynchronize(S.s));  // e lives on this stack
}

// The float64 potentials (Dirichlet values exact at the metal: vals, or
// v_basis on the basis masks) into phi_out.
int finish(Session& S, const MixedResult& r, double* phi_out, int* steps_out,
           double* dmax_out, const double* vals, const uint8_t* masks, double v,
           float* unit_out = nullptr) {
  g_mixed_launches.fetch_add(r.launches + 1);
  const uint32_t n = (uint32_t)S.d.n();
  if (unit_out) {
    // float32 unit bases, staged in the finest level's correction buffer
    // (scratch once the refinement is done; it holds pstride >= n floats
    // per problem)
    float* u = S.lv[0].e.p;
    k_unit32_out<<<dim3(nblk(n), S.B), kT, 0, S.s>>>(S.phi.p, S.fixed.p, masks, v, n, n,
                                                     S.fexp.p, u);
    MK(cudaGetLastError());
    MK(cudaMemcpyAsync(unit_out, u, (size_t)n * S.B * 4, cudaMemcpyDefault, S.s));
  } else {
    k_fixed_out<<<dim3(nblk(n), S.B), kT, 0, S.s>>>(S.phi.p, S.fixed.p, vals, masks, v, n, n,
                                                    S.fexp.p, S.lv[0].G.mnat);
    MK(cudaGetLastError());
    MK(cudaMemcpyAsync(phi_out, S.phi.p, S.d.n() * S.B * 8, cudaMemcpyDefault, S.s));
  }
  MK(cudaStreamSynchronize(S.s));
  if (steps_out) *steps_out = r.steps;
  if (dmax_out) std::memcpy(dmax_out, r.dmax.data(), 8 * S.B);
  if (r.status != IG_OK) set_last_error("mixed-precision refinement reached its step cap");
  return r.status;
}

}  // namespace

long mixed_launch_total() { return g_mixed_launches.load(); }

}  // namespace ig

using namespace ig;

extern "C" {

long ig_mixed_launch_count(void) { return mixed_launch_total(); }

long ig_mixed_bytes(long nx, long ny, long nz, int max_problems) {
  if (nx < 1 || ny < 1 || nz < 1 || max_problems < 1) return -1;
  return (long)session_bytes(Dims{nx, ny, nz}, max_problems);
}

int ig_mixed_open(const uint8_t* metal, long nx, long ny, long nz,
                  int max_problems, int stencil, int nu1, int nu2, int vcycles,
                  void** handle) {
  return ig_mixed_open_ex(metal, nx, ny, nz, max_problems, stencil, nu1, nu2,
                          vcycles, 1, 0, 1.0, 1, 3, handle);
}

}  // extern "C"

namespace {
// Opens a session; nmetal = 1 (one metal, `metal`) or max_problems
// (`metal` stacks one mask per problem).
int open_session(const uint8_t* metal, int nmetal, long nx, long ny, long nz,
                 int max_problems, int stencil, int nu1, int nu2, int vcycles, int gamma,
                 int gamma_levels, double smooth_omega, int method, int cg_iters,
                 void** handle) {
  set_last_error("");
  if (!handle || !metal) {
    set_last_error("null argument");
    return IG_BAD_ARG;
  }
  *handle = nullptr;
  if (nx < 1 || ny < 1 || nz < 1 || max_problems < 1 || max_problems > 65535 ||
      (double)nx * ny * nz >= 2147483648.0 ||
      (double)nx * ny * nz * max_problems >= 9.0e18 || (stencil != 0 && stencil != 1)) {
    set_last_error("invalid shape, problem count or stencil");
    return IG_BAD_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_last_error("no CUDA device is visible");
    return IG_NO_DEVICE;
  }
  // an error an earlier call on this thread left behind (and reported
  // itself) is not this session's: start from a clean slate
  cudaGetLastError();
  Session* S = new Session();
  try {
    MK(cudaStreamCreateWithFlags(&S->s, cudaStreamNonBlocking));
    S->d = Dims{nx, ny, nz};
    S->bmax = max_problems;
    S->nmetal = nmetal;
    S->nu1 = std::max(0, nu1);
    S->nu2 = std::max(1, nu2);
    S->vcycles = std::max(1, vcycles);
    S->gamma = std::min(2, std::max(1, gamma));
    S->gamma_levels = gamma_levels > 0 ? gamma_levels : 64;
    S->smooth_omega = (float)std::min(1.9, std::max(0.5, smooth_omega));
    S->method = method == 0 ? 0 : 1;
    S->cg_iters = std::min(64, std::max(1, cg_iters));
    // IG_MIXED_FLAT: 0 = one natural row per warp in the FP64 residual and
    // update, 1 = several rows per warp, unset = by row length
    if (const char* v = std::getenv("IG_MIXED_FLAT")) S->rows_force = std::atoi(v) ? 1 : 0;
    // IG_MIXED_DOT=0: the flexible CG's <z, q> by its own kernel
    if (const char* v = std::getenv("IG_MIXED_DOT")) S->dot_on = std::atoi(v) != 0;
    // IG_MIXED_FOLD=0: the flexible CG's updates by separate launches
    if (const char* v = std::getenv("IG_MIXED_FOLD")) S->fold_on = std::atoi(v) != 0;
    // IG_MIXED_TAIL=0: the last level above the bottom by separate launches
    if (const char* v = std::getenv("IG_MIXED_TAIL")) S->tail_on = std::atoi(v) != 0;
    // IG_MIXED_TB_LEVELS: how many of the finest levels smooth temporally
    // blocked, fixed instead of left to the smoother tuner
    if (const char* v = std::getenv("IG_MIXED_TB_LEVELS")) {
      S->tb_levels = std::max(0, std::atoi(v));
      S->tb_auto = false;
    }
    // IG_MIXED_TB_MAX: half-sweeps per blocked pass (2, 4 or 6)
    if (const char* v = std::getenv("IG_MIXED_TB_MAX"))
      S->tb_max = std::min(6, std::max(2, std::atoi(v) & ~1));
    // the Shortley-Weller residual with unit legs is half the ghost_linear
    // one: scale it so the correction solves the same equation
    S->resid_scale = stencil == 0 ? 1.0 : 2.0;
    S->build(metal);
    MK(cudaStreamSynchronize(S->s));
  } catch (int code) {
    delete S;
    return code;
  }
  *handle = S;
  return IG_OK;
}
}  // namespace

extern "C" {

int ig_mixed_open_ex(const uint8_t* metal, long nx, long ny, long nz,
                     int max_problems, int stencil, int nu1, int nu2,
                     int vcycles, int gamma, int gamma_levels, double smooth_omega,
                     int method, int cg_iters, void** handle) {
  return open_session(metal, 1, nx, ny, nz, max_problems, stencil, nu1, nu2, vcycles, gamma,
                      gamma_levels, smooth_omega, method, cg_iters, handle);
}

int ig_mixed_open_multi(const uint8_t* metals, int n_problems, long nx, long ny, long nz,
                        int stencil, int nu1, int nu2, int vcycles, int gamma,
                        int gamma_levels, double smooth_omega, int method, int cg_iters,
                        void** handle) {
  if (n_problems < 1) {
    set_last_error("ig_mixed_open_multi: n_problems must be >= 1");
    return IG_BAD_ARG;
  }
  return open_session(metals, n_problems, nx, ny, nz, n_problems, stencil, nu1, nu2, vcycles,
                      gamma, gamma_levels, smooth_omega, method, cg_iters, handle);
}

long ig_mixed_bytes_multi(long nx, long ny, long nz, int n_problems) {
  if (nx < 1 || ny < 1 || nz < 1 || n_problems < 1) return -1;
  return (long)session_bytes(Dims{nx, ny, nz}, n_problems, n_problems);
}

void ig_mixed_close(void* handle) { delete static_cast<Session*>(handle); }

int ig_mixed_rebind(void* handle, const uint8_t* metal, long nx, long ny, long nz) {
  set_last_error("");
  Session* S = static_cast<Session*>(handle);
  if (!S || !metal) {
    set_last_error("null argument");
    return IG_BAD_ARG;
  }
  if (nx != S->d.nx || ny != S->d.ny || nz != S->d.nz) {
    set_last_error("ig_mixed_rebind: the new metal's shape differs from the session's");
    return IG_BAD_ARG;
  }
  try {
    S->load_metal(metal);             // nmetal masks for a per-problem session
    MK(cudaStreamSynchronize(S->s));  // the caller may reuse its mask buffer
  } catch (int code) {
    return code;
  }
  return IG_OK;
}

int ig_mixed_set_cycle(void* handle, int nu1, int nu2, int cg_iters) {
  set_last_error("");
  Session* S = static_cast<Session*>(handle);
  if (!S || nu1 < 0 || nu1 > 16 || nu2 < 1 || nu2 > 16 || cg_iters < 1 || cg_iters > 64) {
    set_last_error("null session or smoothing pairs outside 0..16 / 1..16, CG iterations "
                   "outside 1..64");
    return IG_BAD_ARG;
  }
  try {
    MK(cudaStreamSynchronize(S->s));
    for (auto& g : S->graphs) cudaGraphExecDestroy(g.second);
    S->graphs.clear();
    S->nu1 = nu1;
    S->nu2 = nu2;
    S->cg_iters = S->method == 1 ? cg_iters : S->cg_iters;
    S->update_tail();
  } catch (int code) {
    return code;
  }
  return IG_OK;
}

int ig_mixed_check_convert(const float* floats, long n, long long* mismatches) {
  set_last_error("");
  if (!floats || !mismatches || n < 1 || n > (1L << 30)) {
    set_last_error("null argument or count outside 1..2^30");
    return IG_BAD_ARG;
  }
  try {
    cudaStream_t s = nullptr;
    MK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamGuard {
      cudaStream_t s;
      ~StreamGuard() {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
      }
    } guard{s};
    Buf<float> fv;
    Buf<unsigned long long> mm;
    fv.alloc((size_t)n, s);
    mm.alloc(1, s);
    MK(cudaMemcpyAsync(fv.p, floats, 4 * (size_t)n, cudaMemcpyHostToDevice, s));
    MK(cudaMemsetAsync(mm.p, 0, 8, s));
    k_check_convert<<<nblk((uint32_t)n), kT, 0, s>>>(fv.p, (uint32_t)n, mm.p);
    MK(cudaGetLastError());
    unsigned long long h = 0;
    MK(cudaMemcpyAsync(&h, mm.p, 8, cudaMemcpyDeviceToHost, s));
    MK(cudaStreamSynchronize(s));
    *mismatches = (long long)h;
    return IG_OK;
  } catch (int code) {
    return code;
  }
}

int ig_mixed_tuning(void* handle, int n_problems, int* out_ng, int* out_threads,
                    int* out_tb, double* out_us) {
  set_last_error("");
  Session* S = static_cast<Session*>(handle);
  if (!S || !out_ng || !out_threads || !out_tb || !out_us || n_problems < 1 ||
      n_problems > S->bmax) {
    set_last_error("null argument or problem count outside 1..max_problems");
    return IG_BAD_ARG;
  }
  try {
    if (!S->gs_tuned) S->tune_gs(n_problems);
    *out_ng = S->gs_cfg.ng;
    *out_threads = S->gs_cfg.threads;
    out_tb[0] = S->gs_cfg.tb;
    out_tb[1] = S->gs_cfg.tb_best;
    out_us[0] = S->gs_cfg.sep_us;
    out_us[1] = S->gs_cfg.tb_us;
    return IG_OK;
  } catch (int code) {
    return code;
  }
}

int ig_mixed_solve_bytes(void* handle, double* bytes_out) {
  set_last_error("");
  Session* S = static_cast<Session*>(handle);
  if (!S || !bytes_out) {
    set_last_error("null argument");
    return IG_BAD_ARG;
  }
  *bytes_out = S->last_solve_bytes;
  return IG_OK;
}

int ig_mixed_step_bytes(void* handle, int n_problems, double* bytes_out) {
  set_last_error("");
  Session* S = static_cast<Session*>(handle);
  if (!S || n_problems < 1 || n_problems > S->bmax || !bytes_out) {
    set_last_error("bad session, problem count or output pointer");
    return IG_BAD_ARG;
  }
  *bytes_out = S->step_bytes(n_problems);
  return IG_OK;
}

int ig_mixed_time_gs(void* handle, int n_problems, int pairs, double* ms_per_launch,
                     double* bytes_per_launch) {
  set_last_error("");
  Session* S = static_cast<Session*>(handle);
  if (!S || n_problems < 1 || n_problems > S->bmax || pairs < 1) {
    set_last_error("bad session, problem count or pair count");
    return IG_BAD_ARG;
  }
  try {
    MLevel& f = S->lv[0];
    if (!S->gs_tuned) S->tune_gs(n_problems);
    cudaEvent_t e0, e1;
    MK(cudaEventCreate(&e0));
    MK(cudaEventCreate(&e1));
    for (int c = 0; c < 2; c++) S->launch_gs(f, c, n_problems, 1.f);  // warm
    MK(cudaEventRecord(e0, S->s));
    for (int q = 0; q < pairs; q++)
      for (int c = 0; c < 2; c++) S->launch_gs(f, c, n_problems, 1.f);
    MK(cudaEventRecord(e1, S->s));
    MK(cudaEventSynchronize(e1));
    float ms = 0.f;
    MK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    g_mixed_launches.fetch_add(2L * pairs + 2);
    if (ms_per_launch) *ms_per_launch = ms / (2.0 * pairs);
    // algorithmic bytes of one colour launch: per updated node read its
    // right-hand side (4) and mask (1), write e (4); per node of the other
    // colour read e once (4)
    if (bytes_per_launch) *bytes_per_launch = (double)n_problems * (double)S->d.n() * 6.5;
    return (int)IG_OK;
  } catch (int code) {
    return code;
  }
}

int ig_mixed_check_fused(void* handle, int n_problems, long long mismatches[8]) {
  set_last_error("");
  Session* S = static_cast<Session*>(handle);
  if (!S || !mismatches || n_problems < 1 || n_problems > S->bmax || S->method != 1 ||
      !S->qb.p) {
    set_last_error("bad session (flexible-CG sessions only) or problem count");
    return IG_BAD_ARG;
  }
  try {
    if (!S->gs_tuned) S->tune_gs(n_problems);
    const int B = n_problems;
    S->B = B;  // the session's launch helpers run B problems (each solve sets it anew)
    cudaStream_t s = S->s;
    Buf<unsigned long long> bad;
    bad.alloc(8, s);
    MK(cudaMemsetAsync(bad.p, 0, 64, s));
    long launches = 0;
    auto diff = [&](const void* a, const void* b, size_t words, int slot) {
      k_count_diff<<<dim3((unsigned)((words + kT - 1) / kT), 1), kT, 0, s>>>(
          static_cast<const uint32_t*>(a), static_cast<const uint32_t*>(b), words, bad.p + slot);
      launches++;
    };
    float* scrA = S->xb.p;  // the CG vectors are scratch between solves
    float* scrB = S->qb.p;
    for (size_t l = 0; l + 1 < S->lv.size(); l++) {
      MLevel& a = S->lv[l];
      MLevel& b = S->lv[l + 1];
      const size_t words = a.pstride * B;
      const size_t bytes = words * 4;
      // the prolongation, both colours, on the corrections the solve left
      MK(cudaMemcpyAsync(scrA, a.e.p, bytes, cudaMemcpyDeviceToDevice, s));
      S->launch_prolong(b, a, B, 2);
      MK(cudaMemcpyAsync(scrB, a.e.p, bytes, cudaMemcpyDeviceToDevice, s));
      MK(cudaMemcpyAsync(a.e.p, scrA, bytes, cudaMemcpyDeviceToDevice, s));
      k_prolong_add4_gather<<<dim3(nblk(a.G.csz / 4), B, 2), kT, 0, s>>>(
          b.e.p, b.G, a.e.p, a.mask.p, a.G, b.pstride, a.pstride);
      diff(a.e.p, scrB, words, 2);
      launches += 2;
      if (Session::flat(a)) continue;
      // the colour-0 residual after a Gauss-Seidel pair
      k_resid0<<<dim3(nblk(a.G.csz), B), kT, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G, a.r.p,
                                                    a.pstride);
      MK(cudaMemcpyAsync(scrA, a.r.p, (size_t)a.G.csz * B * 4, cudaMemcpyDeviceToDevice, s));
      k_resid0_4<<<dim3(nblk(a.G.csz / 4), B), kT, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G, a.r.p,
                                                          a.pstride);
      diff(a.r.p, scrA, (size_t)a.G.csz * B, 1);
      launches += 2;
      // the restriction of that residual to the coarse right-hand side
      k_restrict0<<<dim3(nblk(b.G.n), B), kT, 0, s>>>(a.r.p, a.G, b.g.p, b.G, b.pstride);
      MK(cudaMemcpyAsync(scrA, b.g.p, b.pstride * B * 4, cudaMemcpyDeviceToDevice, s));
      k_restrict0_4<<<dim3(nblk((uint32_t)b.G.nx * b.G.ny * ((b.G.nz + 3) / 4)), B), kT, 0, s>>>(
          a.r.p, a.G, b.g.p, b.G, b.pstride);
      diff(b.g.p, scrA, b.pstride * B, 4);
      launches += 2;
      // the fused first pair from a zero correction (a stand-in correction
      // left over from an earlier cycle: both ways must overwrite all of it)
      MK(cudaMemsetAsync(a.e.p, 0x7f, bytes, s));
      k_gs_zero_pair<<<dim3(nblk(a.G.csz / 4), B), kT, 0, s>>>(a.e.p, a.g.p, a.mask.p, a.G,
                                                              a.pstride);
      MK(cudaMemcpyAsync(scrA, a.e.p, bytes, cudaMemcpyDeviceToDevice, s));
      MK(cudaMemsetAsync(a.e.p, 0, bytes, s));
      for (int c = 0; c < 2; c++) S->launch_gs(a, c, B, 1.f);
      diff(a.e.p, scrA, words, 0);
      launches += 3;
      // the temporally blocked smoothing phases of 1, 2 and 3 pairs: from
      // e = 0 (colours 0, 1, ...; over a stand-in correction) against a
      // zeroed correction and the separate half-sweeps, and from that
      // result (colours 1, 0, ..., into r) against the separate
      // half-sweeps on the same input
      MK(tb_prepare());
      for (int S2 = 2; S2 <= 6; S2 += 2) {
        MK(cudaMemsetAsync(a.e.p, 0x7f, bytes, s));
        launch_tb(S2, true, 0, a.e.p, a.e.p, a.g.p, a.mask.p, a.G, a.pstride, B, s);
        MK(cudaMemcpyAsync(scrA, a.e.p, bytes, cudaMemcpyDeviceToDevice, s));
        MK(cudaMemsetAsync(a.e.p, 0, bytes, s));
        for (int q = 0; q < S2 / 2; q++)
          for (int c = 0; c < 2; c++) S->launch_gs(a, c, B, 1.f);
        diff(a.e.p, scrA, words, 6);
        MK(cudaMemcpyAsync(scrB, a.e.p, bytes, cudaMemcpyDeviceToDevice, s));   // input
        // continuing colours 0, 1, ... (a later pre-smoothing pass)
        MK(cudaMemsetAsync(a.r.p, 0x7f, bytes, s));
        launch_tb(S2, false, 0, a.e.p, a.r.p, a.g.p, a.mask.p, a.G, a.pstride, B, s);
        for (int q = 0; q < S2 / 2; q++)
          for (int c = 0; c < 2; c++) S->launch_gs(a, c, B, 1.f);
        diff(a.e.p, a.r.p, words, 6);
        MK(cudaMemcpyAsync(a.e.p, scrB, bytes, cudaMemcpyDeviceToDevice, s));
        // colours 1, 0, ... (post-smoothing)
        MK(cudaMemsetAsync(a.r.p, 0x7f, bytes, s));
        launch_tb(S2, false, 1, a.e.p, a.r.p, a.g.p, a.mask.p, a.G, a.pstride, B, s);
        for (int q = 0; q < S2 / 2; q++)
          for (int c = 1; c >= 0; c--) S->launch_gs(a, c, B, 1.f);
        diff(a.e.p, a.r.p, words, 7);
        MK(cudaMemcpyAsync(a.e.p, scrB, bytes, cudaMemcpyDeviceToDevice, s));
        launches += 4 + 4 * S2 + 3;
      }
    }
    // the fused direction update + operator apply on level 0, from the
    // direction, correction and beta the solve left
    if (S->fuse_dir()) {
      MLevel& f = S->lv[0];
      const size_t words = f.pstride * B;
      const unsigned nb4 = std::min(nblk(f.G.csz / 4), kCgBlocks);
      const size_t nparts = 2 * (size_t)B * 2 * nb4;
      Buf<double> part2;
      part2.alloc(nparts, s);
      k_cg_matvec_dir<0><<<dim3(nb4, 2, B), kT, 0, s>>>(f.e.p, S->pb.p, S->pb2.p, S->scal.p,
                                                       f.g.p, f.mask.p, f.G, scrB, part2.p,
                                                       f.pstride, nullptr);
      k_cg_dir<<<dim3(nblk((uint32_t)f.pstride), B), kT, 0, s>>>(S->pb.p, f.e.p, S->scal.p,
                                                                 f.pstride, (uint32_t)f.pstride);
      k_cg_matvec<<<dim3(nb4, 2, B), kT, 0, s>>>(S->pb.p, f.g.p, f.mask.p, f.G, scrA,
                                                S->part.p, f.pstride);
      diff(S->pb.p, S->pb2.p, words, 3);
      diff(scrA, scrB, words, 3);
      diff(S->part.p, part2.p, 2 * nparts, 3);
      launches += 3;
    }
    // the CG update of a step's first iteration (x = alpha p) against a
    // zeroed x and the update, and the last iteration's x += alpha p folded
    // into the FP64 update against the two kernels (potentials and maxima)
    {
      MLevel& f = S->lv[0];
      const size_t words = f.pstride * B;
      const uint32_t n = (uint32_t)f.pstride;
      const dim3 gu(nblk(n / 4), B);
      float* x = S->xb.p;
      float* p = S->pb.p;
      MK(cudaMemsetAsync(x, 0, words * 4, s));
      k_cg_update<false><<<gu, kT, 0, s>>>(x, f.g.p, p, S->qb.p, S->scal.p, f.pstride, n);
      MK(cudaMemcpyAsync(scrA, x, words * 4, cudaMemcpyDeviceToDevice, s));
      k_cg_update<true><<<gu, kT, 0, s>>>(x, f.g.p, p, S->qb.p, S->scal.p, f.pstride, n);
      diff(x, scrA, words, 5);
      const size_t nphi = f.G.n * (size_t)B;
      Buf<long long> phi0, phi1;
      phi0.alloc(nphi, s);
      phi1.alloc(nphi, s);
      Buf<unsigned long long> dm;
      dm.alloc(2 * (size_t)B, s);
      MK(cudaMemsetAsync(dm.p, 0, 16 * (size_t)B, s));
      MK(cudaMemcpyAsync(phi0.p, S->phi.p, nphi * 8, cudaMemcpyDeviceToDevice, s));
      MK(cudaMemcpyAsync(scrB, x, words * 4, cudaMemcpyDeviceToDevice, s));   // x kept
      k_cg_update<false><<<gu, kT, 0, s>>>(x, f.g.p, p, S->qb.p, S->scal.p, f.pstride, n);
      S->launch_update64(x, dm.p, nullptr, nullptr);
      MK(cudaMemcpyAsync(phi1.p, S->phi.p, nphi * 8, cudaMemcpyDeviceToDevice, s));
      MK(cudaMemcpyAsync(S->phi.p, phi0.p, nphi * 8, cudaMemcpyDeviceToDevice, s));
      S->launch_update64(scrB, dm.p + B, p, S->scal.p);
      diff(S->phi.p, phi1.p, 2 * nphi, 5);
      diff(dm.p, dm.p + B, 2 * (size_t)B, 5);
      launches += 6;
    }
    unsigned long long h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    MK(cudaMemcpyAsync(h, bad.p, 64, cudaMemcpyDeviceToHost, s));
    MK(cudaStreamSynchronize(s));
    g_mixed_launches.fetch_add(launches);
    for (int q = 0; q < 8; q++) mismatches[q] = (long long)h[q];
    return (int)IG_OK;
  } catch (int code) {
    return code;
  }
}

}  // extern "C"

namespace {
// The basis solve behind ig_mixed_solve_bases (phi_out) and
// ig_mixed_solve_unit_bases (unit_out).
int solve_bases_to(Session* S, const uint8_t* masks, int n_bases, double v_basis, double acc,
                   int max_steps, double* phi_out, float* unit_out, int* steps_out,
                   double* dmax_out) {
  set_last_error("");
  if (!S || !masks || !(phi_out || unit_out) || n_bases < 1 || n_bases > S->bmax) {
    set_last_error("null argument or basis count outside 1..max_problems");
    return IG_BAD_ARG;
  }
  if (unit_out && !(std::fabs(v_basis) > 0.0 && std::isfinite(v_basis))) {
    set_last_error("ig_mixed_solve_unit_bases: v_basis must be finite and nonzero");
    return IG_BAD_ARG;
  }
  if (S->nmetal > 1) {
    set_last_error("ig_mixed_solve_bases: a session with one metal per problem solves "
                   "values (ig_mixed_solve_values), not the bases of one metal union");
    return IG_BAD_ARG;
  }
  try {
    const size_t n = S->d.n();
    S->B = n_bases;
    if (!S->stage.p) S->stage.alloc(n * S->bmax, S->s);
    MK(cudaMemcpyAsync(S->stage.p, masks, n * n_bases, cudaMemcpyDefault, S->s));
    set_units(*S, std::vector<double>(n_bases, std::fabs(v_basis)));
    int ex = 0;
    if (v_basis != 0.0) std::frexp(std::fabs(v_basis), &ex);
    // v_basis in units 2^(ex - 56): exact (|v_basis| >= 2^(ex - 1))
    const long long vfx = std::llrint(std::ldexp(v_basis, 56 - ex));
    k_init_basis<<<dim3(nblk((uint32_t)n), n_bases), kT, 0, S->s>>>(S->phi.p, S->stage.p,
                                                                   (uint32_t)n, vfx, n);
    MK(cudaGetLastError());
    const std::vector<double> accs(n_bases, acc);
    const MixedResult r = run_mixed(*S, accs.data(), max_steps);
    return finish(*S, r, phi_out, steps_out, dmax_out, nullptr, S->stage.p, v_basis, unit_out);
  } catch (int code) {
    return code;
  }
}
}  // namespace

extern "C" {

int ig_mixed_solve_bases(void* handle, const uint8_t* masks, int n_bases,
                         double v_basis, double acc, int max_steps,
                         double* phi_out, int* steps_out, double* dmax_out) {
  if (!phi_out) {
    set_last_error("null argument or basis count outside 1..max_problems");
    return IG_BAD_ARG;
  }
  return solve_bases_to(static_cast<Session*>(handle), masks, n_bases, v_basis, acc,
                        max_steps, phi_out, nullptr, steps_out, dmax_out);
}

int ig_mixed_solve_unit_bases(void* handle, const uint8_t* masks, int n_bases,
                              double v_basis, double acc, int max_steps, float* unit_out,
                              int* steps_out, double* dmax_out) {
  if (!unit_out) {
    set_last_error("null argument or basis count outside 1..max_problems");
    return IG_BAD_ARG;
  }
  return solve_bases_to(static_cast<Session*>(handle), masks, n_bases, v_basis, acc,
                        max_steps, nullptr, unit_out, steps_out, dmax_out);
}

int ig_mixed_solve_values(void* handle, const double* vals, int n_problems,
                          double acc, int max_steps, double* phi_out,
                          int* steps_out, double* dmax_out) {
  if (n_problems < 1 || n_problems > 65535) {
    set_last_error("problem count outside 1..max_problems");
    return IG_BAD_ARG;
  }
  const std::vector<double> accs(n_problems, acc);
  return ig_mixed_solve_values_acc(handle, vals, n_problems, accs.data(), max_steps, phi_out,
                                   steps_out, dmax_out);
}

int ig_mixed_solve_values_acc(void* handle, const double* vals, int n_problems,
                              const double* acc, int max_steps, double* phi_out,
                              int* steps_out, double* dmax_out) {
  set_last_error("");
  Session* S = static_cast<Session*>(handle);
  if (!S || !vals || !phi_out || !acc || n_problems < 1 || n_problems > S->bmax) {
    set_last_error("null argument or problem count outside 1..max_problems");
    return IG_BAD_ARG;
  }
  try {
    const size_t n = S->d.n();
    S->B = n_problems;
    if (!S->vstage.p) S->vstage.alloc(n * S->bmax, S->s);
    MK(cudaMemcpyAsync(S->vstage.p, vals, n * n_problems * 8, cudaMemcpyDefault, S->s));
    MK(cudaMemsetAsync(S->vmax.p, 0, 8 * (size_t)n_problems, S->s));
    k_absmax_vals<<<dim3(std::min(nblk((uint32_t)n), 1024u), n_problems), kT, 0, S->s>>>(
        S->vstage.p, S->fixed.p, (uint32_t)n, n, S->vmax.p, S->lv[0].G.mnat);
    MK(cudaGetLastError());
    std::vector<unsigned long long> mb(n_problems);
    MK(cudaMemcpyAsync(mb.data(), S->vmax.p, 8 * (size_t)n_problems, cudaMemcpyDeviceToHost,
                       S->s));
    MK(cudaStreamSynchronize(S->s));
    std::vector<double> vm(n_problems);
    for (int b = 0; b < n_problems; b++) vm[b] = bits_to_double(mb[b]);
    set_units(*S, vm);
    k_init_vals<<<dim3(nblk((uint32_t)n), n_problems), kT, 0, S->s>>>(
        S->phi.p, S->fixed.p, S->vstage.p, (uint32_t)n, n, S->fexp.p, S->lv[0].G.mnat);
    MK(cudaGetLastError());
    g_mixed_launches.fetch_add(2);
    const MixedResult r = run_mixed(*S, acc, max_steps);
    return finish(*S, r, phi_out, steps_out, dmax_out, S->vstage.p, nullptr, 0.0);
  } catch (int code) {
    return code;
  }
}

int ig_mixed_bases(const uint8_t* metal, const uint8_t* masks, int n_bases,
                   double v_basis, long nx, long ny, long nz, int stencil,
                   double acc, int max_steps, int nu1, int nu2, int vcycles,
                   double* phi_out, int* steps_out, double* dmax_out) {
  void* h = nullptr;
  int st = ig_mixed_open(metal, nx, ny, nz, n_bases, stencil, nu1, nu2, vcycles, &h);
  if (st != IG_OK) return st;
  st = ig_mixed_solve_bases(h, masks, n_bases, v_basis, acc, max_steps, phi_out,
                            steps_out, dmax_out);
  ig_mixed_close(h);
  return st;
}

}  // extern "C"
