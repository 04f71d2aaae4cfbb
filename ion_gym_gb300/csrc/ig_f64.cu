// ig_f64.cu -- exact FP64 kernels of the 3-D Laplace solve on sm_103a.
//
// Each kernel returns the bits the reference's compiled float64 kernels
// return on the same input (ion_gym physics/solver3d.py and
// physics/multigrid3d.py, cited per kernel).  FP64 is the scarce pipe on
// GB300 (about 1/64 of the FP32 rate), so the kernels spend it only where the
// reference does: masks, indices, maxima and absolute values run on the
// integer pipe, and the theta == 1 stencil divides by 6 on the integer pipe
// (ig::div6) instead of a full division.
//
// Layout: C-order (nx, ny, nz), z contiguous; theta (6, nx, ny, nz) float32.
// Sweeps map one thread to one (i, j, k-pair) cell so a warp reads 64
// consecutive doubles of a row and every lane does useful FP64 work; the
// flattened index is split with 32-bit multiplicative division.
#include <atomic>
#include <mutex>

#include "ig_common.cuh"
#include "ig_internal.h"

namespace ig {

std::atomic<long> g_launches{0};
long launch_total() { return g_launches.load(); }
void note_launches(long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

namespace {

constexpr int kThreads = 256;

inline void counted() { g_launches.fetch_add(1, std::memory_order_relaxed); }

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
  return (__umulhi(n, f.m) + n) >> f.s;
}

struct SweepGeom {
  long nx, ny, nz;
  FastDiv div_kk, div_ny;
  uint32_t total;  // nx*ny*nkk
};

inline SweepGeom sweep_geom(Dims d) {
  SweepGeom g;
  g.nx = d.nx;
  g.ny = d.ny;
  g.nz = d.nz;
  const long nkk = (d.nz + 1) / 2;
  g.div_kk = FastDiv((uint32_t)nkk);
  g.div_ny = FastDiv((uint32_t)d.ny);
  g.total = (uint32_t)(d.nx * d.ny * nkk);
  return g;
}

struct FlatGeom {
  long nx, ny, nz;
  FastDiv div_nz, div_ny;
  uint32_t total;
};

inline FlatGeom flat_geom(Dims d) {
  FlatGeom g;
  g.nx = d.nx;
  g.ny = d.ny;
  g.nz = d.nz;
  g.div_nz = FastDiv((uint32_t)d.nz);
  g.div_ny = FastDiv((uint32_t)d.ny);
  g.total = (uint32_t)d.n();
  return g;
}

inline unsigned blocks_for(size_t n) {
  return (unsigned)((n + kThreads - 1) / kThreads);
}

// Early-exit test of the exact SOR loop (PairCtl in ig_internal.h).  Uniform
// over the block, so a returning block skips the block reduction as a whole.
__device__ __forceinline__ bool pair_skip(PairCtl* ctl, int colour, int lp) {
  volatile PairCtl* c = ctl;
  if (c->done) return true;
  if (lp >= c->limit) return true;
  if (colour == 0) {
    unsigned long long a = 0, b = 0;
    bool have = false;
    if (lp > 0) {
      a = c->slot[2 * lp - 2];
      b = c->slot[2 * lp - 1];
      have = true;
    } else if (c->has_prev) {
      a = c->prev[0];
      b = c->prev[1];
      have = true;
    }
    if (have) {
      const double d = bits_to_double(a > b ? a : b);
      if (d < c->tol) {
        if (blockIdx.x == 0 && threadIdx.x == 0) c->done = 1;
        return true;
      }
    }
  }
  return false;
}

// Node indices fit 32 bits (grids are below 2^31 nodes).
struct Nb {
  uint32_t xm, xp, ym, yp, zm, zp;
};

// The six neighbours of node p = (i, j, k) as offsets from p, with the
// even-reflection rule at the faces (the ghost at -1 is node 1, the ghost at
// n is node n-2; a size-1 axis uses the node itself) as selects, so the
// interior and the faces run the same instructions.
__device__ __forceinline__ Nb neighbours(uint32_t i, uint32_t j, uint32_t k, uint32_t nx,
                                         uint32_t ny, uint32_t nz) {
  const uint32_t sy = nz, sx = ny * nz;
  const uint32_t p = (i * ny + j) * nz + k;
  const uint32_t rx = nx > 1 ? sx : 0u, ry = ny > 1 ? sy : 0u, rz = nz > 1 ? 1u : 0u;
  Nb n;
  n.xm = i > 0 ? p - sx : p + rx;
  n.xp = i + 1 < nx ? p + sx : p - rx;
  n.ym = j > 0 ? p - sy : p + ry;
  n.yp = j + 1 < ny ? p + sy : p - ry;
  n.zm = k > 0 ? p - 1 : p + rz;
  n.zp = k + 1 < nz ? p + 1 : p - rz;
  return n;
}

// num and den of the theta-weighted stencil exactly as the reference forms
// them (solver3d.py:169-191, multigrid3d.py:329-353).
template <int KIND>
__device__ __forceinline__ void theta_num_den(const double v[6],
                                              const float* __restrict__ th,
                                              size_t N, size_t p, double& num,
                                              double& den) {
  const float t0 = th[p], t1 = th[N + p], t2 = th[2 * N + p];
  const float t3 = th[3 * N + p], t4 = th[4 * N + p], t5 = th[5 * N + p];
  if (KIND == kThetaGhost) {
    const double w0 = __drcp_rn((double)t0), w1 = __drcp_rn((double)t1);
    const double w2 = __drcp_rn((double)t2), w3 = __drcp_rn((double)t3);
    const double w4 = __drcp_rn((double)t4), w5 = __drcp_rn((double)t5);
    num = __dmul_rn(v[0], w0);
    num = __dadd_rn(num, __dmul_rn(v[1], w1));
    num = __dadd_rn(num, __dmul_rn(v[2], w2));
    num = __dadd_rn(num, __dmul_rn(v[3], w3));
    num = __dadd_rn(num, __dmul_rn(v[4], w4));
    num = __dadd_rn(num, __dmul_rn(v[5], w5));
    den = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(w0, w1), w2), w3), w4), w5);
  } else {
    const float sx = __fadd_rn(t0, t1), sy = __fadd_rn(t2, t3), sz = __fadd_rn(t4, t5);
    const float a0 = __fmul_rn(t0, sx), a1 = __fmul_rn(t1, sx);
    const float a2 = __fmul_rn(t2, sy), a3 = __fmul_rn(t3, sy);
    const float a4 = __fmul_rn(t4, sz), a5 = __fmul_rn(t5, sz);
    num = __ddiv_rn(v[0], (double)a0);
    num = __dadd_rn(num, __ddiv_rn(v[1], (double)a1));
    num = __dadd_rn(num, __ddiv_rn(v[2], (double)a2));
    num = __dadd_rn(num, __ddiv_rn(v[3], (double)a3));
    num = __dadd_rn(num, __ddiv_rn(v[4], (double)a4));
    num = __dadd_rn(num, __ddiv_rn(v[5], (double)a5));
    const double px = __drcp_rn((double)__fmul_rn(t0, t1));
    const double py = __drcp_rn((double)__fmul_rn(t2, t3));
    const double pz = __drcp_rn((double)__fmul_rn(t4, t5));
    den = __dadd_rn(__dadd_rn(px, py), pz);
  }
}

__device__ __forceinline__ double sum6(const double v[6]) {
  return __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(v[0], v[1]), v[2]), v[3]), v[4]), v[5]);
}

__device__ __forceinline__ void load6(const double* __restrict__ a, const Nb& n,
                                      double v[6]) {
  v[0] = a[n.xm];
  v[1] = a[n.xp];
  v[2] = a[n.ym];
  v[3] = a[n.yp];
  v[4] = a[n.zm];
  v[5] = a[n.zp];
}

// solver3d._sweep (solver3d.py:131-198).
template <int KIND, bool CTL, bool DELTA = true>
__global__ void __launch_bounds__(kThreads)
k_sweep(double* __restrict__ phi, const uint8_t* __restrict__ fixed,
        const float* __restrict__ th, SweepGeom g, double omega, int colour,
        unsigned long long* dslot, PairCtl* ctl, int lp) {
  if (CTL) {
    if (pair_skip(ctl, colour, lp)) return;
    dslot = &ctl->slot[2 * lp + colour];
  }
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  unsigned long long mb = 0;
  if (t < g.total) {
    const uint32_t ij = fdiv(t, g.div_kk);
    const uint32_t kk = t - ij * g.div_kk.d;
    const uint32_t i = fdiv(ij, g.div_ny);
    const uint32_t j = ij - i * g.div_ny.d;
    const uint32_t k = 2 * kk + ((i + j + colour) & 1);
    if (k < (uint32_t)g.nz) {
      const uint32_t p = (i * (uint32_t)g.ny + j) * (uint32_t)g.nz + k;
      if (!fixed[p]) {
        const Nb n = neighbours(i, j, k, g.nx, g.ny, g.nz);
        double v[6];
        load6(phi, n, v);
        const double old = phi[p];
        double q;
        if (KIND == kPlain) {
          q = div6(sum6(v));
        } else {
          double num, den;
          theta_num_den<KIND>(v, th, (size_t)g.nx * g.ny * g.nz, p, num, den);
          q = __ddiv_rn(num, den);
        }
        const double nw = __dadd_rn(old, omega_step(old, q, omega));
        if (DELTA) mb = absbits(__dsub_rn(nw, old));
        phi[p] = nw;
      }
    }
  }
  // without a slot (DELTA false) nobody reads the max |update|: skip the
  // subtraction and the block reduction
  if (DELTA) block_max_to(mb, dslot);
}

// multigrid3d._residual (multigrid3d.py:305-354): num - den*phi, 0 at fixed.
template <int KIND>
__global__ void __launch_bounds__(kThreads)
k_residual(const double* __restrict__ phi, const uint8_t* __restrict__ fixed,
           const float* __restrict__ th, FlatGeom g, double* __restrict__ out,
           unsigned long long* absmax) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  unsigned long long mb = 0;
  if (t < g.total) {
    const uint32_t ij = fdiv(t, g.div_nz);
    const uint32_t k = t - ij * g.div_nz.d;
    const uint32_t i = fdiv(ij, g.div_ny);
    const uint32_t j = ij - i * g.div_ny.d;
    double r = 0.0;
    if (!fixed[t]) {
      const Nb n = neighbours(i, j, k, g.nx, g.ny, g.nz);
      double v[6];
      load6(phi, n, v);
      if (KIND == kPlain) {
        r = __dsub_rn(sum6(v), __dmul_rn(6.0, phi[t]));
      } else if (KIND == kPlainSW) {
        // unit legs: num = sum of v/2 (== sum/2 exactly), den = 3
        r = __dsub_rn(__dmul_rn(sum6(v), 0.5), __dmul_rn(3.0, phi[t]));
      } else {
        double num, den;
        theta_num_den<KIND>(v, th, g.total, t, num, den);
        r = __dsub_rn(num, __dmul_rn(den, phi[t]));
      }
    }
    if (out) out[t] = r;
    mb = absbits(r);
  }
  if (absmax) block_max_to(mb, absmax);
}

// multigrid3d._sweep_rhs (multigrid3d.py:357-391).
template <bool CTL>
__global__ void __launch_bounds__(kThreads)
k_sweep_rhs(double* __restrict__ e, const uint8_t* __restrict__ fixed,
            const double* __restrict__ f, SweepGeom g, double omega,
            int colour, unsigned long long* dslot, PairCtl* ctl, int lp) {
  if (CTL) {
    if (pair_skip(ctl, colour, lp)) return;
    dslot = &ctl->slot[2 * lp + colour];
  }
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  unsigned long long mb = 0;
  if (t < g.total) {
    const uint32_t ij = fdiv(t, g.div_kk);
    const uint32_t kk = t - ij * g.div_kk.d;
    const uint32_t i = fdiv(ij, g.div_ny);
    const uint32_t j = ij - i * g.div_ny.d;
    const uint32_t k = 2 * kk + ((i + j + colour) & 1);
    if (k < (uint32_t)g.nz) {
      const uint32_t p = (i * (uint32_t)g.ny + j) * (uint32_t)g.nz + k;
      if (!fixed[p]) {
        const Nb n = neighbours(i, j, k, g.nx, g.ny, g.nz);
        double v[6];
        load6(e, n, v);
        const double old = e[p];
        const double nv = div6(__dsub_rn(sum6(v), f[p]));
        const double nw = __dadd_rn(old, omega_step(old, nv, omega));
        mb = absbits(__dsub_rn(nw, old));
        e[p] = nw;
      }
    }
  }
  block_max_to(mb, dslot);
}


// multigrid3d._restrict_fw_njit (multigrid3d.py:420-455) at coarse node
// (ic, jc, kc): 27-point full weighting with clamped edges, /8, and
// -4x when neg4 (the caller's scaling).
__device__ __forceinline__ double restrict_node(const double* __restrict__ fine, long nx,
                                                long ny, long nz, long ic, long jc, long kc,
                                                int neg4) {
  const long i = 2 * ic, j = 2 * jc, k = 2 * kc;
  double acc = 0.0;
#pragma unroll
  for (int di = -1; di <= 1; di++) {
    long ii = i + di;
    ii = ii < 0 ? 0 : (ii > nx - 1 ? nx - 1 : ii);
    const double wi = di == 0 ? 1.0 : 0.5;
#pragma unroll
    for (int dj = -1; dj <= 1; dj++) {
      long jj = j + dj;
      jj = jj < 0 ? 0 : (jj > ny - 1 ? ny - 1 : jj);
      const double wj = dj == 0 ? 1.0 : 0.5;
      const double* row = fine + ((size_t)ii * ny + jj) * nz;
#pragma unroll
      for (int dk = -1; dk <= 1; dk++) {
        long kk = k + dk;
        kk = kk < 0 ? 0 : (kk > nz - 1 ? nz - 1 : kk);
        const double wk = dk == 0 ? 1.0 : 0.5;
        // wi*wj*wk is a power of two, folded at compile time
        acc = __dadd_rn(acc, __dmul_rn(wi * wj * wk, row[kk]));
      }
    }
  }
  double r = __dmul_rn(acc, 0.125);  // == acc / 8.0 (power-of-two scale)
  if (neg4) r = -__dmul_rn(r, 4.0);
  return r;
}

struct Lerp {
  long a0, a1;
  double t;
};

// multigrid3d.py:465-481 (prolong-add coordinates)
__device__ __forceinline__ Lerp pa_axis(long i, long c) {
  double xf = __dmul_rn((double)i, 0.5);
  if (xf > (double)(c - 1)) xf = (double)c - 1.0;
  long x0 = (long)xf;
  if (x0 > c - 2) x0 = c > 1 ? c - 2 : 0;
  Lerp l;
  l.a0 = x0;
  l.a1 = c > 1 ? x0 + 1 : x0;
  l.t = __dsub_rn(xf, (double)x0);
  return l;
}

// multigrid3d.py:144-156 (cascadic prolongation coordinates)
__device__ __forceinline__ Lerp pl_axis(long i, long c) {
  double xf = __ddiv_rn((double)i, 2.0);
  if (xf > (double)(c - 1)) xf = (double)(c - 1);
  const long x0 = (long)floor(xf);
  Lerp l;
  l.a0 = x0;
  l.a1 = x0 + 1 < c - 1 ? x0 + 1 : c - 1;
  l.t = __dsub_rn(xf, (double)x0);
  return l;
}

__device__ __forceinline__ double lerp_ref(double a, double b, double t) {
  // a*(1-t) + b*t, evaluated as the reference writes it
  return __dadd_rn(__dmul_rn(a, __dsub_rn(1.0, t)), __dmul_rn(b, t));
}

__device__ __forceinline__ double trilinear(const double* __restrict__ c,
                                            long cy, long cz, const Lerp& x,
                                            const Lerp& y, const Lerp& z) {
#define C(a, b, d) c[((size_t)(a) * cy + (b)) * cz + (d)]
  const double c00 = lerp_ref(C(x.a0, y.a0, z.a0), C(x.a1, y.a0, z.a0), x.t);
  const double c10 = lerp_ref(C(x.a0, y.a1, z.a0), C(x.a1, y.a1, z.a0), x.t);
  const double c01 = lerp_ref(C(x.a0, y.a0, z.a1), C(x.a1, y.a0, z.a1), x.t);
  const double c11 = lerp_ref(C(x.a0, y.a1, z.a1), C(x.a1, y.a1, z.a1), x.t);
#undef C
  const double c0 = lerp_ref(c00, c10, y.t);
  const double c1 = lerp_ref(c01, c11, y.t);
  return lerp_ref(c0, c1, z.t);
}

// One CTA solving the bottom of multigrid3d._solve_err
// (multigrid3d.py:575-580) from shared memory: every node update is the
// launched kernel's arithmetic and the maxima are order-free, so the result
// and the pair count equal the launched loop's, without a launch per pair or
// a host synchronisation per batch.
constexpr int kBottomCta = 1024;

__device__ __forceinline__ unsigned long long cta_max(unsigned long long v,
                                                      unsigned long long* red) {
  v = warp_max_u64(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = lane < (int)(blockDim.x >> 5) ? red[lane] : 0ull;
    v = warp_max_u64(v);
    if (lane == 0) red[32] = v;
  }
  __syncthreads();
  const unsigned long long r = red[32];
  __syncthreads();
  return r;
}

// tol = rel_tol * max(max|f|, 1e-300) / 6 of a level in shared memory (NaN
// in f makes it NaN, as numpy's max does).
__device__ double cta_level_tol(const double* f, long n, double rel_tol,
                                unsigned long long* red) {
  unsigned long long fk = 0;
  bool nan = false;
  for (long t = threadIdx.x; t < n; t += blockDim.x) {
    const unsigned long long x =
        static_cast<unsigned long long>(__double_as_longlong(f[t])) & 0x7fffffffffffffffULL;
    if (x > 0x7ff0000000000000ULL) nan = true;
    else if (x > fk) fk = x;
  }
  nan = __syncthreads_or(nan);
  fk = cta_max(fk, red);
  double scale = nan ? __longlong_as_double(0x7ff8000000000000LL) : bits_to_double(fk);
  scale = (1e-300 > scale) ? 1e-300 : scale;  // max(|f|.max(), 1e-300)
  return __ddiv_rn(__dmul_rn(rel_tol, scale), 6.0);
}

// One colour of _sweep_rhs over a level in shared memory; returns the
// largest |update| key (all threads).
__device__ unsigned long long cta_sweep(double* e, const uint8_t* fx, const double* f,
                                        long nx, long ny, long nz, double omega, int colour,
                                        unsigned long long* red) {
  const long half = nz / 2 + 1;  // slots of one colour in a row
  unsigned long long mb = 0;
  for (long t = threadIdx.x; t < nx * ny * half; t += blockDim.x) {
    const long ij = t / half, kk = t - ij * half;
    const long i = ij / ny, j = ij - i * ny;
    const long k = 2 * kk + ((i + j + colour) & 1);
    if (k >= nz) continue;
    const long p = (i * ny + j) * nz + k;
    if (fx[p]) continue;
    const Nb nb = neighbours(i, j, k, nx, ny, nz);
    double v[6];
    load6(e, nb, v);
    const double old = e[p];
    const double nv = div6(__dsub_rn(sum6(v), f[p]));
    const double nw = __dadd_rn(old, omega_step(old, nv, omega));
    const unsigned long long x = absbits(__dsub_rn(nw, old));
    if (x > mb) mb = x;
    e[p] = nw;
  }
  __syncthreads();
  return cta_max(mb, red);
}

// The bottom: e = 0; SOR pairs at omega until the larger of a pair's two
// max |update| is below 0.02 * tol, at most max_pairs pairs.
__device__ void cta_bottom(double* e, const uint8_t* fx, const double* f, long nx, long ny,
                           long nz, double rel_tol, double omega, long max_pairs,
                           unsigned long long* red) {
  const long n = nx * ny * nz;
  for (long t = threadIdx.x; t < n; t += blockDim.x) e[t] = 0.0;
  const double tol = __dmul_rn(0.02, cta_level_tol(f, n, rel_tol, red));
  for (long pr = 0; pr < max_pairs; pr++) {
    const unsigned long long k0 = cta_sweep(e, fx, f, nx, ny, nz, omega, 0, red);
    const unsigned long long k1 = cta_sweep(e, fx, f, nx, ny, nz, omega, 1, red);
    if (bits_to_double(k0 > k1 ? k0 : k1) < tol) break;
  }
}

__global__ void __launch_bounds__(kBottomCta)
k_bottom_err(double* __restrict__ e_out, const uint8_t* __restrict__ fixed_g,
             const double* __restrict__ f_g, long nx, long ny, long nz, double rel_tol,
             double omega, long max_pairs) {
  extern __shared__ double sm[];
  __shared__ unsigned long long red[33];
  const long n = nx * ny * nz;
  double* e = sm;
  double* f = sm + n;
  uint8_t* fx = reinterpret_cast<uint8_t*>(sm + 2 * n);
  for (long t = threadIdx.x; t < n; t += blockDim.x) {
    f[t] = f_g[t];
    fx[t] = fixed_g[t];
  }
  __syncthreads();
  cta_bottom(e, fx, f, nx, ny, nz, rel_tol, omega, max_pairs, red);
  __syncthreads();
  for (long t = threadIdx.x; t < n; t += blockDim.x) e_out[t] = e[t];
}

// multigrid3d._residual_rhs (multigrid3d.py:394-417).
__global__ void __launch_bounds__(kThreads)
k_residual_rhs(const double* __restrict__ e, const uint8_t* __restrict__ fixed,
               const double* __restrict__ f, FlatGeom g,
               double* __restrict__ out) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= g.total) return;
  const uint32_t ij = fdiv(t, g.div_nz);
  const uint32_t k = t - ij * g.div_nz.d;
  const uint32_t i = fdiv(ij, g.div_ny);
  const uint32_t j = ij - i * g.div_ny.d;
  double r = 0.0;
  if (!fixed[t]) {
    const Nb n = neighbours(i, j, k, g.nx, g.ny, g.nz);
    double v[6];
    load6(e, n, v);
    r = __dsub_rn(__dsub_rn(sum6(v), __dmul_rn(6.0, e[t])), f[t]);
  }
  out[t] = r;
}

__global__ void __launch_bounds__(kThreads)
k_restrict(const double* __restrict__ fine, long nx, long ny, long nz,
           double* __restrict__ out, FlatGeom c, int neg4) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= c.total) return;
  const uint32_t ij = fdiv(t, c.div_nz);
  const long kc = t - ij * c.div_nz.d;
  const long ic = fdiv(ij, c.div_ny);
  const long jc = ij - ic * c.div_ny.d;
  out[t] = restrict_node(fine, nx, ny, nz, ic, jc, kc, neg4);
}

// multigrid3d._prolong_add_njit (multigrid3d.py:458-499).
__global__ void __launch_bounds__(kThreads)
k_prolong_add(const double* __restrict__ coarse, long cx, long cy, long cz,
              double* __restrict__ out, const uint8_t* __restrict__ fixed,
              FlatGeom g) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= g.total) return;
  if (fixed[t]) return;
  const uint32_t ij = fdiv(t, g.div_nz);
  const long k = t - ij * g.div_nz.d;
  const long i = fdiv(ij, g.div_ny);
  const long j = ij - i * g.div_ny.d;
  const Lerp x = pa_axis(i, cx), y = pa_axis(j, cy), z = pa_axis(k, cz);
  out[t] = __dadd_rn(out[t], trilinear(coarse, cy, cz, x, y, z));
}

// multigrid3d._prolongate (multigrid3d.py:138-171).
__global__ void __launch_bounds__(kThreads)
k_prolongate(const double* __restrict__ coarse, long cx, long cy, long cz,
             double* __restrict__ out, FlatGeom g) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= g.total) return;
  const uint32_t ij = fdiv(t, g.div_nz);
  const long k = t - ij * g.div_nz.d;
  const long i = fdiv(ij, g.div_ny);
  const long j = ij - i * g.div_ny.d;
  const Lerp x = pl_axis(i, cx), y = pl_axis(j, cy), z = pl_axis(k, cz);
  out[t] = trilinear(coarse, cy, cz, x, y, z);
}

// multigrid3d._coarsen_fixed_any (multigrid3d.py:507-526).
__global__ void __launch_bounds__(kThreads)
k_coarsen_any(const uint8_t* __restrict__ fixed, long nx, long ny, long nz,
              uint8_t* __restrict__ out, FlatGeom c) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= c.total) return;
  const uint32_t ij = fdiv(t, c.div_nz);
  const long kc = t - ij * c.div_nz.d;
  const long ic = fdiv(ij, c.div_ny);
  const long jc = ij - ic * c.div_ny.d;
  uint8_t any = 0;
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++)
      for (int q = 0; q < 2; q++) {
        const long i = 2 * ic + a, j = 2 * jc + b, k = 2 * kc + q;
        if (i < nx && j < ny && k < nz && fixed[((size_t)i * ny + j) * nz + k]) any = 1;
      }
  out[t] = any;
}

// multigrid3d._coarsen_mask (multigrid3d.py:85-135).
__global__ void __launch_bounds__(kThreads)
k_coarsen_mask(const uint8_t* __restrict__ fixed, const double* __restrict__ val,
               long nx, long ny, long nz, uint8_t* __restrict__ fc,
               double* __restrict__ vc, FlatGeom c) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= c.total) return;
  const uint32_t ij = fdiv(t, c.div_nz);
  const long kc = t - ij * c.div_nz.d;
  const long ic = fdiv(ij, c.div_ny);
  const long jc = ij - ic * c.div_ny.d;
  const size_t p0 = ((size_t)(2 * ic) * ny + 2 * jc) * nz + 2 * kc;
  if (fixed[p0]) {
    fc[t] = 1;
    vc[t] = val[p0];
    return;
  }
  unsigned long long best = 0;
  bool any = false;
  double bv = 0.0;
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++)
      for (int q = 0; q < 2; q++) {
        const long i = 2 * ic + a, j = 2 * jc + b, k = 2 * kc + q;
        if (i >= nx || j >= ny || k >= nz) continue;
        const size_t p = ((size_t)i * ny + j) * nz + k;
        if (!fixed[p]) continue;
        const double v = val[p];
        // |v| compared through its bits (first maximum wins, as argmax)
        const unsigned long long m =
            (static_cast<unsigned long long>(__double_as_longlong(v)) & 0x7fffffffffffffffULL) + 1ULL;
        if (!any || m > best) {
          best = m;
          bv = v;
        }
        any = true;
      }
  fc[t] = any ? 1 : 0;
  vc[t] = any ? bv : val[p0];
}

__global__ void k_set_fixed(double* __restrict__ phi,
                            const uint8_t* __restrict__ fixed,
                            const double* __restrict__ val, size_t n) {
  const size_t t = (size_t)blockIdx.x * kThreads + threadIdx.x;
  if (t < n && fixed[t]) phi[t] = val[t];
}

__global__ void __launch_bounds__(kThreads)
k_absdiff_max(const double* __restrict__ a, const double* __restrict__ b,
              size_t n, unsigned long long* bits, int* nan_flag) {
  unsigned long long mb = 0;
  bool nan = false;
  for (size_t t = (size_t)blockIdx.x * kThreads + threadIdx.x; t < n;
       t += (size_t)gridDim.x * kThreads) {
    const double d = b ? __dsub_rn(a[t], b[t]) : a[t];
    const unsigned long long x =
        static_cast<unsigned long long>(__double_as_longlong(d)) & 0x7fffffffffffffffULL;
    if (x > 0x7ff0000000000000ULL) nan = true;
    else if (x > mb) mb = x;
  }
  if (__syncthreads_or(nan) && threadIdx.x == 0) *nan_flag = 1;
  block_max_to(mb, bits);
}

// phi <- (phi + flip(phi, axis)) * 0.5 (multigrid3d.py:689-691); each thread
// owns a mirror pair, so the in-place update reads both values first.
__global__ void __launch_bounds__(kThreads)
k_sym_project(double* __restrict__ phi, FlatGeom g, int axis) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= g.total) return;
  const uint32_t ij = fdiv(t, g.div_nz);
  const long k = t - ij * g.div_nz.d;
  const long i = fdiv(ij, g.div_ny);
  const long j = ij - i * g.div_ny.d;
  long mi = i, mj = j, mk = k;
  if (axis == 0) mi = g.nx - 1 - i;
  else if (axis == 1) mj = g.ny - 1 - j;
  else mk = g.nz - 1 - k;
  const size_t q = ((size_t)mi * g.ny + mj) * g.nz + mk;
  if (q < t) return;  // the partner with the lower index does the pair
  const double s = __dmul_rn(__dadd_rn(phi[t], phi[q]), 0.5);
  phi[t] = s;
  phi[q] = s;
}

// solver3d._residual_kernel (solver3d.py:366-386): num/den - u.
__global__ void __launch_bounds__(kThreads)
k_residual_audit(const double* __restrict__ u, const uint8_t* __restrict__ fixed,
                 const float* __restrict__ th, FlatGeom g,
                 double* __restrict__ out) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= g.total) return;
  const uint32_t ij = fdiv(t, g.div_nz);
  const uint32_t k = t - ij * g.div_nz.d;
  const uint32_t i = fdiv(ij, g.div_ny);
  const uint32_t j = ij - i * g.div_ny.d;
  double r = 0.0;
  if (!fixed[t]) {
    const Nb n = neighbours(i, j, k, g.nx, g.ny, g.nz);
    double v[6], num, den;
    load6(u, n, v);
    theta_num_den<kThetaGhost>(v, th, g.total, t, num, den);
    r = __dsub_rn(__ddiv_rn(num, den), u[t]);
  }
  out[t] = r;
}

// solver3d._err_sweep (solver3d.py:389-417).
__global__ void __launch_bounds__(kThreads)
k_err_sweep(double* __restrict__ e, const uint8_t* __restrict__ fixed,
            const float* __restrict__ th, const double* __restrict__ rhs,
            SweepGeom g, double omega, int colour, unsigned long long* dslot) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  unsigned long long mb = 0;
  if (t < g.total) {
    const uint32_t ij = fdiv(t, g.div_kk);
    const uint32_t kk = t - ij * g.div_kk.d;
    const uint32_t i = fdiv(ij, g.div_ny);
    const uint32_t j = ij - i * g.div_ny.d;
    const uint32_t k = 2 * kk + ((i + j + colour) & 1);
    if (k < (uint32_t)g.nz) {
      const uint32_t p = (i * (uint32_t)g.ny + j) * (uint32_t)g.nz + k;
      if (!fixed[p]) {
        const Nb n = neighbours(i, j, k, g.nx, g.ny, g.nz);
        double v[6], num, den;
        load6(e, n, v);
        theta_num_den<kThetaGhost>(v, th, (size_t)g.nx * g.ny * g.nz, p, num, den);
        const double old = e[p];
        const double inner = __dsub_rn(__dadd_rn(__ddiv_rn(num, den), rhs[p]), old);
        const double nw = __dadd_rn(old, __dmul_rn(omega, inner));
        mb = absbits(__dsub_rn(nw, old));
        e[p] = nw;
      }
    }
  }
  block_max_to(mb, dslot);
}

__global__ void k_fill_ones_f32(float* a, size_t n) {
  const size_t t = (size_t)blockIdx.x * kThreads + threadIdx.x;
  if (t < n) a[t] = 1.0f;
}

}  // namespace

void launch_sweep(cudaStream_t s, double* phi, const uint8_t* fixed,
                  const float* th, int kind, Dims d, double omega, int colour,
                  unsigned long long* dslot, PairCtl* ctl, int lp) {
  const SweepGeom g = sweep_geom(d);
  const unsigned nb = blocks_for(g.total);
  if (nb == 0) return;
  counted();
#define IG_SWEEP(K)                                                              \
  if (ctl) k_sweep<K, true><<<nb, kThreads, 0, s>>>(phi, fixed, th, g, omega,    \
                                                    colour, dslot, ctl, lp);     \
  else if (dslot) k_sweep<K, false><<<nb, kThreads, 0, s>>>(phi, fixed, th, g,   \
                                                 omega, colour, dslot, ctl, lp); \
  else k_sweep<K, false, false><<<nb, kThreads, 0, s>>>(phi, fixed, th, g,       \
                                                 omega, colour, dslot, ctl, lp);
  if (kind == kPlain) { IG_SWEEP(kPlain) }
  else if (kind == kThetaGhost) { IG_SWEEP(kThetaGhost) }
  else { IG_SWEEP(kThetaSW) }
#undef IG_SWEEP
}

void launch_residual(cudaStream_t s, const double* phi, const uint8_t* fixed,
                     const float* th, int kind, Dims d, double* out,
                     unsigned long long* absmax) {
  const FlatGeom g = flat_geom(d);
  const unsigned nb = blocks_for(g.total);
  if (nb == 0) return;
  counted();
  if (kind == kPlain)
    k_residual<kPlain><<<nb, kThreads, 0, s>>>(phi, fixed, th, g, out, absmax);
  else if (kind == kPlainSW)
    k_residual<kPlainSW><<<nb, kThreads, 0, s>>>(phi, fixed, th, g, out, absmax);
  else if (kind == kThetaGhost)
    k_residual<kThetaGhost><<<nb, kThreads, 0, s>>>(phi, fixed, th, g, out, absmax);
  else
    k_residual<kThetaSW><<<nb, kThreads, 0, s>>>(phi, fixed, th, g, out, absmax);
}

void launch_sweep_rhs(cudaStream_t s, double* e, const uint8_t* fixed,
                      const double* f, Dims d, double omega, int colour,
                      unsigned long long* dslot, PairCtl* ctl, int lp) {
  const SweepGeom g = sweep_geom(d);
  const unsigned nb = blocks_for(g.total);
  if (nb == 0) return;
  counted();
  if (ctl)
    k_sweep_rhs<true><<<nb, kThreads, 0, s>>>(e, fixed, f, g, omega, colour, dslot, ctl, lp);
  else
    k_sweep_rhs<false><<<nb, kThreads, 0, s>>>(e, fixed, f, g, omega, colour, dslot, ctl, lp);
}

bool launch_bottom_err(cudaStream_t s, double* e, const uint8_t* fixed, const double* f,
                       Dims d, double rel_tol, double omega, long max_pairs) {
  const size_t n = d.n();
  const size_t bytes = 17 * n;
  if (n == 0 || bytes > kBottomSmemMax) return false;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaFuncSetAttribute(k_bottom_err, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kBottomSmemMax);
  });
  k_bottom_err<<<1, kBottomCta, (bytes + 7) / 8 * 8, s>>>(e, fixed, f, d.nx, d.ny, d.nz,
                                                         rel_tol, omega, max_pairs);
  counted();
  return true;
}

void launch_residual_rhs(cudaStream_t s, const double* e, const uint8_t* fixed,
                         const double* f, Dims d, double* out) {
  const FlatGeom g = flat_geom(d);
  const unsigned nb = blocks_for(g.total);
  if (nb) {
    k_residual_rhs<<<nb, kThreads, 0, s>>>(e, fixed, f, g, out);
    counted();
  }
}

void launch_restrict(cudaStream_t s, const double* fine, Dims d, double* out,
                     Dims c, int neg4) {
  const FlatGeom g = flat_geom(c);
  const unsigned nb = blocks_for(g.total);
  if (nb) {
    k_restrict<<<nb, kThreads, 0, s>>>(fine, d.nx, d.ny, d.nz, out, g, neg4);
    counted();
  }
}

void launch_prolong_add(cudaStream_t s, const double* coarse, Dims c,
                        double* out, const uint8_t* fixed, Dims d) {
  const FlatGeom g = flat_geom(d);
  const unsigned nb = blocks_for(g.total);
  if (nb) {
    k_prolong_add<<<nb, kThreads, 0, s>>>(coarse, c.nx, c.ny, c.nz, out, fixed, g);
    counted();
  }
}

void launch_prolongate(cudaStream_t s, const double* coarse, Dims c,
                       double* out, Dims d) {
  const FlatGeom g = flat_geom(d);
  const unsigned nb = blocks_for(g.total);
  if (nb) {
    k_prolongate<<<nb, kThreads, 0, s>>>(coarse, c.nx, c.ny, c.nz, out, g);
    counted();
  }
}

void launch_coarsen_any(cudaStream_t s, const uint8_t* fixed, Dims d,
                        uint8_t* out, Dims c) {
  const FlatGeom g = flat_geom(c);
  const unsigned nb = blocks_for(g.total);
  if (nb) {
    k_coarsen_any<<<nb, kThreads, 0, s>>>(fixed, d.nx, d.ny, d.nz, out, g);
    counted();
  }
}

void launch_coarsen_mask(cudaStream_t s, const uint8_t* fixed,
                         const double* val, Dims d, uint8_t* fc, double* vc,
                         Dims c) {
  const FlatGeom g = flat_geom(c);
  const unsigned nb = blocks_for(g.total);
  if (nb) {
    k_coarsen_mask<<<nb, kThreads, 0, s>>>(fixed, val, d.nx, d.ny, d.nz, fc, vc, g);
    counted();
  }
}

void launch_set_fixed(cudaStream_t s, double* phi, const uint8_t* fixed,
                      const double* val, size_t n) {
  const unsigned nb = blocks_for(n);
  if (nb) {
    k_set_fixed<<<nb, kThreads, 0, s>>>(phi, fixed, val, n);
    counted();
  }
}

void launch_absdiff_max(cudaStream_t s, const double* a, const double* b,
                        size_t n, unsigned long long* bits, int* nan_flag) {
  unsigned nb = blocks_for(n);
  if (nb > 152u * 8u) nb = 152u * 8u;
  if (nb) {
    k_absdiff_max<<<nb, kThreads, 0, s>>>(a, b, n, bits, nan_flag);
    counted();
  }
}

void launch_sym_project(cudaStream_t s, double* phi, Dims d, int axis) {
  const FlatGeom g = flat_geom(d);
  const unsigned nb = blocks_for(g.total);
  if (nb) {
    k_sym_project<<<nb, kThreads, 0, s>>>(phi, g, axis);
    counted();
  }
}

void launch_residual_audit(cudaStream_t s, const double* u,
                           const uint8_t* fixed, const float* th, Dims d,
                           double* out) {
  const FlatGeom g = flat_geom(d);
  const unsigned nb = blocks_for(g.total);
  if (nb) {
    k_residual_audit<<<nb, kThreads, 0, s>>>(u, fixed, th, g, out);
    counted();
  }
}

void launch_err_sweep(cudaStream_t s, double* e, const uint8_t* fixed,
                      const float* th, const double* rhs, Dims d, double omega,
                      int colour, unsigned long long* dslot) {
  const SweepGeom g = sweep_geom(d);
  const unsigned nb = blocks_for(g.total);
  if (nb) {
    k_err_sweep<<<nb, kThreads, 0, s>>>(e, fixed, th, rhs, g, omega, colour, dslot);
    counted();
  }
}

void launch_fill_ones_f32(cudaStream_t s, float* a, size_t n) {
  const unsigned nb = blocks_for(n);
  if (nb) {
    k_fill_ones_f32<<<nb, kThreads, 0, s>>>(a, n);
    counted();
  }
}

}  // namespace ig
