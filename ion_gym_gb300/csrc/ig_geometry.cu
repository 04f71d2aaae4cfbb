// ig_geometry.cu -- analytic scenes on the device: the labelled node raster
// (ion_gym physics/rasterize3d.py:45-109) and the fractional-surface legs
// theta (physics/solver3d.py:46-127), bit-identical to the reference's
// float64 numpy evaluation.
//
// A scene arrives as a flat primitive table in grid units.  Each primitive
// carries its electrode (in raster order), its shape, whether it is a
// `within` or a `notin` solid, and its bounds pre-combined on the host with
// the reference's tolerance exactly as the reference writes them
// (r**2 + eps, (z - length) - eps, x1 - eps, ...), so the kernels only form
// (x - cx)**2 + (y - cy)**2 with round-to-nearest operations and compare.
#include <cstdint>
#include <string>

#include "ig_common.cuh"
#include "ig_internal.h"
#include "../../include/igsolve.h"

namespace ig {
namespace {

constexpr int kT = 256;

// One primitive, 8 doubles: kind (0 cylinder, 1 box), electrode slot,
// shape id, role (0 within, 1 notin), then the bounds:
//   cylinder: cx, cy, r2 (r**2 + e), zlo ((z - length) - e), zhi (z + e)
//   box:      x1 - e, x2 + e, y1 - e, y2 + e, z1 - e, z2 + e
// Two copies of the bounds are stored: with e = +eps (inclusive) and with
// e = -eps (strict, used for `notin` solids by the theta inside test).
struct Prim {
  int kind, elec, shape, role;
  double in[6];
  double st[6];
};

__device__ __forceinline__ bool inside(const Prim& p, const double* b, double x,
                                       double y, double z) {
  if (p.kind == 0) {
    const double dx = __dsub_rn(x, b[0]);
    const double dy = __dsub_rn(y, b[1]);
    const double rr = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    return rr <= b[2] && z >= b[3] && z <= b[4];
  }
  return x >= b[0] && x <= b[1] && y >= b[2] && y <= b[3] && z >= b[4] && z <= b[5];
}

// rasterize3d.rasterize: per node, electrodes in order; shapes union, within
// minus notin (inclusive bounds for both); a node claimed by a second
// electrode index is a clash.  Per electrode: node count, clash count and
// the lowest clashing flat index.
__global__ void __launch_bounds__(kT)
k_rasterize(const Prim* __restrict__ prims, int np, const int* __restrict__ eidx,
            int ne, long nx, long ny, long nz, int16_t* __restrict__ lab,
            unsigned long long* __restrict__ count,
            unsigned long long* __restrict__ clash_count,
            unsigned long long* __restrict__ clash_min) {
  const size_t n = (size_t)nx * ny * nz;
  const size_t t = (size_t)blockIdx.x * kT + threadIdx.x;
  if (t >= n) return;
  const long k = (long)(t % nz);
  const long j = (long)((t / nz) % ny);
  const long i = (long)(t / ((size_t)nz * ny));
  const double x = (double)i, y = (double)j, z = (double)k;
  int16_t cur = 0;
  int p = 0;
  for (int e = 0; e < ne; e++) {
    bool m = false;
    while (p < np && prims[p].elec == e) {
      // one shape: its within primitives then its notin primitives
      const int sh = prims[p].shape;
      bool w = false;
      while (p < np && prims[p].elec == e && prims[p].shape == sh) {
        const Prim& q = prims[p];
        const bool hit = inside(q, q.in, x, y, z);
        if (q.role == 0) w = w || hit;
        else w = w && !hit;
        p++;
      }
      m = m || w;
    }
    if (m) {
      const int16_t idx = (int16_t)eidx[e];
      atomicAdd(count + e, 1ULL);
      if (cur != 0 && cur != idx) {
        atomicAdd(clash_count + e, 1ULL);
        atomicMin(clash_min + e, (unsigned long long)t);
      }
      cur = idx;
    }
  }
  lab[t] = cur;
}

// solver3d.inside_scene_pts for one point: union over shapes of (any
// within, inclusive) minus (any notin, strict)
__device__ __forceinline__ bool inside_scene(const Prim* __restrict__ prims, int np,
                                             double x, double y, double z) {
  bool total = false;
  int p = 0;
  while (p < np) {
    const int e = prims[p].elec, sh = prims[p].shape;
    bool w = false;
    while (p < np && prims[p].elec == e && prims[p].shape == sh) {
      const Prim& q = prims[p];
      if (q.role == 0) w = w || inside(q, q.in, x, y, z);
      else w = w && !inside(q, q.st, x, y, z);
      p++;
    }
    total = total || w;
  }
  return total;
}

// solver3d.fractions_from_scene: the leg of direction d at every vacuum
// node whose d-neighbour is metal (a low mirror plane sees node 1 from node
// 0), by `iters` bisections of the exact inside test; theta =
// float32(clip(0.5 (lo + hi), 1e-3, 1)).  blockIdx.y = direction.
__global__ void __launch_bounds__(kT)
k_theta(const Prim* __restrict__ prims, int np, const uint8_t* __restrict__ metal,
        long nx, long ny, long nz, int mirror_bits, int iters,
        float* __restrict__ th) {
  const size_t n = (size_t)nx * ny * nz;
  const size_t t = (size_t)blockIdx.x * kT + threadIdx.x;
  if (t >= n) return;
  const int d = blockIdx.y;
  const int ax = d >> 1;
  const int step = (d & 1) ? 1 : -1;
  const long k = (long)(t % nz);
  const long j = (long)((t / nz) % ny);
  const long i = (long)(t / ((size_t)nz * ny));
  if (metal[t]) return;
  long c[3] = {i, j, k};
  const long len[3] = {nx, ny, nz};
  long q[3] = {i, j, k};
  q[ax] += step;
  const bool mir = (mirror_bits >> ax) & 1;
  if (q[ax] < 0) {
    if (!(mir && step < 0 && len[ax] > 1)) return;
    q[ax] = 1;   // the mirrored solid across the low plane
  }
  if (q[ax] >= len[ax]) return;
  if (!metal[((size_t)q[0] * ny + q[1]) * nz + q[2]]) return;
  const double p0[3] = {(double)c[0], (double)c[1], (double)c[2]};
  double lo = 0.0, hi = 1.0;
  for (int it = 0; it < iters; it++) {
    const double mid = __dmul_rn(0.5, __dadd_rn(lo, hi));
    double pr[3] = {p0[0], p0[1], p0[2]};
    pr[ax] = __dadd_rn(p0[ax], step > 0 ? mid : -mid);
    if (mir && step < 0) pr[ax] = fabs(pr[ax]);
    const bool hit = inside_scene(prims, np, pr[0], pr[1], pr[2]);
    if (hit) hi = mid;
    else lo = mid;
  }
  double v = __dmul_rn(0.5, __dadd_rn(lo, hi));
  v = v < 1e-3 ? 1e-3 : (v > 1.0 ? 1.0 : v);
  th[(size_t)d * n + t] = __double2float_rn(v);
}

__global__ void k_fill_f32(float* a, size_t n, float v) {
  const size_t t = (size_t)blockIdx.x * kT + threadIdx.x;
  if (t < n) a[t] = v;
}

}  // namespace
}  // namespace ig

using namespace ig;

namespace {
struct Tmp {
  void* p = nullptr;
  ~Tmp() {
    if (p) cudaFree(p);
  }
};
#define GK(x)                                                            \
  do {                                                                   \
    cudaError_t e_ = (x);                                                \
    if (e_ != cudaSuccess) {                                             \
      set_last_error(std::string(#x) + ": " + cudaGetErrorString(e_));   \
      return IG_CUDA_ERROR;                                              \
    }                                                                    \
  } while (0)

int check_table(const double* table, int n_prims) {
  for (int p = 0; p < n_prims; p++) {
    const double* r = table + 16 * p;
    if ((r[0] != 0.0 && r[0] != 1.0) || r[1] < 0 || (r[3] != 0.0 && r[3] != 1.0)) {
      set_last_error("malformed primitive table");
      return IG_BAD_ARG;
    }
    if (p > 0 && r[1] < table[16 * (p - 1) + 1]) {
      set_last_error("primitive table not in electrode order");
      return IG_BAD_ARG;
    }
  }
  return IG_OK;
}

int upload_prims(const double* table, int n_prims, Tmp& dev) {
  // table rows: kind, elec, shape, role, in[6], st[6]  (16 doubles)
  Prim* h = new Prim[n_prims > 0 ? n_prims : 1];
  for (int p = 0; p < n_prims; p++) {
    const double* r = table + 16 * p;
    h[p].kind = (int)r[0];
    h[p].elec = (int)r[1];
    h[p].shape = (int)r[2];
    h[p].role = (int)r[3];
    for (int a = 0; a < 6; a++) {
      h[p].in[a] = r[4 + a];
      h[p].st[a] = r[10 + a];
    }
  }
  cudaError_t e = cudaMalloc(&dev.p, sizeof(Prim) * (n_prims > 0 ? n_prims : 1));
  if (e == cudaSuccess)
    e = cudaMemcpy(dev.p, h, sizeof(Prim) * n_prims, cudaMemcpyHostToDevice);
  delete[] h;
  if (e != cudaSuccess) {
    set_last_error(std::string("primitive upload: ") + cudaGetErrorString(e));
    return IG_CUDA_ERROR;
  }
  return IG_OK;
}
}  // namespace

extern "C" int ig_rasterize(const double* table, int n_prims,
                            const int* electrode_index, int n_electrodes,
                            long nx, long ny, long nz, int16_t* labels_out,
                            unsigned long long* counts_out,
                            unsigned long long* clash_counts_out,
                            unsigned long long* clash_first_out) {
  set_last_error("");
  if (!table || !electrode_index || !labels_out || n_prims < 0 || n_electrodes < 1 ||
      nx < 1 || ny < 1 || nz < 1) {
    set_last_error("invalid raster arguments");
    return IG_BAD_ARG;
  }
  if (int st = check_table(table, n_prims)) return st;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_last_error("no CUDA device is visible");
    return IG_NO_DEVICE;
  }
  const size_t n = (size_t)nx * ny * nz;
  Tmp prims, eidx, lab, cnt;
  if (int st = upload_prims(table, n_prims, prims)) return st;
  GK(cudaMalloc(&eidx.p, sizeof(int) * n_electrodes));
  GK(cudaMemcpy(eidx.p, electrode_index, sizeof(int) * n_electrodes, cudaMemcpyHostToDevice));
  GK(cudaMalloc(&lab.p, 2 * n));
  GK(cudaMalloc(&cnt.p, 3 * 8 * (size_t)n_electrodes));
  unsigned long long* c = static_cast<unsigned long long*>(cnt.p);
  GK(cudaMemset(c, 0, 2 * 8 * (size_t)n_electrodes));
  GK(cudaMemset(c + 2 * n_electrodes, 0xff, 8 * (size_t)n_electrodes));
  const unsigned nb = (unsigned)((n + kT - 1) / kT);
  k_rasterize<<<nb, kT>>>(static_cast<Prim*>(prims.p), n_prims,
                          static_cast<int*>(eidx.p), n_electrodes, nx, ny, nz,
                          static_cast<int16_t*>(lab.p), c, c + n_electrodes,
                          c + 2 * n_electrodes);
  GK(cudaGetLastError());
  GK(cudaMemcpy(labels_out, lab.p, 2 * n, cudaMemcpyDeviceToHost));
  if (counts_out) GK(cudaMemcpy(counts_out, c, 8 * n_electrodes, cudaMemcpyDeviceToHost));
  if (clash_counts_out)
    GK(cudaMemcpy(clash_counts_out, c + n_electrodes, 8 * n_electrodes, cudaMemcpyDeviceToHost));
  if (clash_first_out)
    GK(cudaMemcpy(clash_first_out, c + 2 * n_electrodes, 8 * n_electrodes,
                  cudaMemcpyDeviceToHost));
  return IG_OK;
}

extern "C" int ig_theta_scene(const double* table, int n_prims, const uint8_t* metal,
                              long nx, long ny, long nz, int mirror_bits, int iters,
                              float* theta_out) {
  set_last_error("");
  if (!table || !metal || !theta_out || n_prims < 0 || nx < 1 || ny < 1 || nz < 1 ||
      iters < 0) {
    set_last_error("invalid theta arguments");
    return IG_BAD_ARG;
  }
  if (int st = check_table(table, n_prims)) return st;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_last_error("no CUDA device is visible");
    return IG_NO_DEVICE;
  }
  const size_t n = (size_t)nx * ny * nz;
  Tmp prims, m, th;
  if (int st = upload_prims(table, n_prims, prims)) return st;
  GK(cudaMalloc(&m.p, n));
  GK(cudaMemcpy(m.p, metal, n, cudaMemcpyHostToDevice));
  GK(cudaMalloc(&th.p, 6 * n * 4));
  const unsigned nb = (unsigned)((6 * n + kT - 1) / kT);
  k_fill_f32<<<nb, kT>>>(static_cast<float*>(th.p), 6 * n, 1.0f);
  const dim3 g((unsigned)((n + kT - 1) / kT), 6);
  k_theta<<<g, kT>>>(static_cast<Prim*>(prims.p), n_prims, static_cast<uint8_t*>(m.p), nx,
                     ny, nz, mirror_bits, iters, static_cast<float*>(th.p));
  GK(cudaGetLastError());
  GK(cudaMemcpy(theta_out, th.p, 6 * n * 4, cudaMemcpyDeviceToHost));
  return IG_OK;
}
