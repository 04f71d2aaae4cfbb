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
#include <vector>

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

// ---- extruded 2-D cross-sections (build_shapes3d.py, raster2d.py) -------
//
// A shape's cross-section is evaluated on its in-plane node coordinates
// (a_i, b_j) with the reference's float64 expressions (raster2d.py:113-
// 230): a rect (optionally rotated about its centre) or an ellipse with
// every edge moved out by the 1e-9 mm tolerance, or a polygon as a closed
// solid (even-odd interior or within 1e-9 mm of an edge).  The host passes
// the scalars already combined as the reference writes them.
struct XSec {
  int type;          // 0 rect, 1 ellipse, 2 polygon
  int rotated;       // rect
  double p[10];      // rect: cx, cy, ca, sa, xlo, xhi, ylo, yhi
                     // ellipse: cx, cy, rxT, ryT; polygon: tol2
};

__global__ void __launch_bounds__(kT)
k_xsection(XSec S, const double* __restrict__ poly, int npts, const double* __restrict__ a,
           long na, const double* __restrict__ b, long nb, uint8_t* __restrict__ out) {
  const size_t n = (size_t)na * nb;
  const size_t t = (size_t)blockIdx.x * kT + threadIdx.x;
  if (t >= n) return;
  const double X = a[t / nb], Y = b[t % nb];
  bool in = false;
  if (S.type == 0) {
    double xr = X, yr = Y;
    if (S.rotated) {
      const double cx = S.p[0], cy = S.p[1], ca = S.p[2], sa = S.p[3];
      const double dx = __dsub_rn(X, cx), dy = __dsub_rn(Y, cy);
      xr = __dsub_rn(__dadd_rn(cx, __dmul_rn(dx, ca)), __dmul_rn(dy, sa));
      yr = __dadd_rn(__dadd_rn(cy, __dmul_rn(dx, sa)), __dmul_rn(dy, ca));
    }
    in = xr >= S.p[4] && xr <= S.p[5] && yr >= S.p[6] && yr <= S.p[7];
  } else if (S.type == 1) {
    const double u = __ddiv_rn(__dsub_rn(X, S.p[0]), S.p[2]);
    const double v = __ddiv_rn(__dsub_rn(Y, S.p[1]), S.p[3]);
    in = __dadd_rn(__dmul_rn(u, u), __dmul_rn(v, v)) <= 1.0;
  } else {
    // poly rows: x0, y0, x1, y1, ex, ey, seg2 (7 x npts)
    const double* x0 = poly;
    const double* y0 = poly + npts;
    const double* x1 = poly + 2 * npts;
    const double* y1 = poly + 3 * npts;
    const double* ex = poly + 4 * npts;
    const double* ey = poly + 5 * npts;
    const double* sg = poly + 6 * npts;
    bool inside = false;
    for (int e = 0; e < npts; e++) {
      const double ax = x0[e], ay = y0[e], bx = x1[e], by = y1[e];
      if (ay == by) continue;
      const bool straddles = (ay > Y) != (by > Y);
      const double xint = __dadd_rn(
          ax, __ddiv_rn(__dmul_rn(__dsub_rn(Y, ay), __dsub_rn(bx, ax)), __dsub_rn(by, ay)));
      inside ^= straddles && (X < xint);
    }
    double d2 = __longlong_as_double(0x7ff0000000000000LL);  // +inf
    for (int e = 0; e < npts; e++) {
      double dj2;
      const double dx = __dsub_rn(X, x0[e]), dy = __dsub_rn(Y, y0[e]);
      if (sg[e] == 0.0) {
        dj2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
      } else {
        double tt = __ddiv_rn(__dadd_rn(__dmul_rn(dx, ex[e]), __dmul_rn(dy, ey[e])), sg[e]);
        tt = tt < 0.0 ? 0.0 : (tt > 1.0 ? 1.0 : tt);
        const double px = __dadd_rn(x0[e], __dmul_rn(tt, ex[e]));
        const double py = __dadd_rn(y0[e], __dmul_rn(tt, ey[e]));
        const double qx = __dsub_rn(X, px), qy = __dsub_rn(Y, py);
        dj2 = __dadd_rn(__dmul_rn(qx, qx), __dmul_rn(qy, qy));
      }
      d2 = dj2 < d2 ? dj2 : d2;
    }
    in = inside || d2 <= S.p[0];
  }
  out[t] = in ? 1 : 0;
}

// One extruded shape of the 3-D assembly: its electrode slot, extrusion
// axis (in-plane axes are the next two, cyclically), whether it is a
// cutout, and where its cross-section (na x nb bytes) and its range along
// the axis (one byte per node of that axis) start in the shared buffers.
struct ShapeRec {
  int slot, axis, cutout, pad;
  long long xs_off, rng_off;
  int na, nb;
};

// build_shapes3d.shapes_masks_3d + electrode_mask_3d: per node, electrodes
// in order; an electrode's shapes in order, additive shapes OR their
// volume in, cutouts AND NOT theirs; the node's label is the last
// electrode that claims it and a claim over an earlier one is a clash.
__global__ void __launch_bounds__(kT)
k_shapes_label(const ShapeRec* __restrict__ recs, int nrec, const uint8_t* __restrict__ xs,
               const uint8_t* __restrict__ rng, const int* __restrict__ eidx, int ne, long nx,
               long ny, long nz, int16_t* __restrict__ lab, unsigned long long* __restrict__ count,
               unsigned long long* __restrict__ clash_count,
               unsigned long long* __restrict__ clash_min) {
  const size_t n = (size_t)nx * ny * nz;
  const size_t t = (size_t)blockIdx.x * kT + threadIdx.x;
  if (t >= n) return;
  const long idx[3] = {(long)(t / ((size_t)nz * ny)), (long)((t / nz) % ny), (long)(t % nz)};
  int16_t cur = 0;
  int r = 0;
  for (int e = 0; e < ne; e++) {
    bool m = false;
    for (; r < nrec && recs[r].slot == e; r++) {
      const ShapeRec& q = recs[r];
      const int a1 = (q.axis + 1) % 3, a2 = (q.axis + 2) % 3;
      const bool v = rng[q.rng_off + idx[q.axis]] &&
                     xs[q.xs_off + (long long)idx[a1] * q.nb + idx[a2]];
      if (q.cutout)
        m = m && !v;
      else
        m = m || v;
    }
    if (m) {
      const int16_t id = (int16_t)eidx[e];
      atomicAdd(count + e, 1ULL);
      if (cur != 0) {
        atomicAdd(clash_count + e, 1ULL);
        atomicMin(clash_min + e, (unsigned long long)t);
      }
      cur = id;
    }
  }
  lab[t] = cur;
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

extern "C" int ig_shape_xsection(int type, const double* params, int n_params,
                                 const double* poly, int n_points, const double* a, long na,
                                 const double* b, long nb, uint8_t* out) {
  set_last_error("");
  if (type < 0 || type > 2 || !params || n_params < 1 || n_params > 10 || !a || !b || !out ||
      na < 1 || nb < 1 || (type == 2 && (!poly || n_points < 1))) {
    set_last_error("invalid cross-section arguments");
    return IG_BAD_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_last_error("no CUDA device is visible");
    return IG_NO_DEVICE;
  }
  XSec S{};
  S.type = type;
  for (int q = 0; q < n_params; q++) S.p[q] = params[q];
  S.rotated = type == 0 && n_params >= 9 && params[8] != 0.0;
  const size_t n = (size_t)na * nb;
  Tmp dp, da, db, dout;
  if (type == 2) {
    GK(cudaMalloc(&dp.p, 7 * sizeof(double) * n_points));
    GK(cudaMemcpy(dp.p, poly, 7 * sizeof(double) * n_points, cudaMemcpyHostToDevice));
  }
  GK(cudaMalloc(&da.p, 8 * na));
  GK(cudaMalloc(&db.p, 8 * nb));
  GK(cudaMemcpy(da.p, a, 8 * na, cudaMemcpyHostToDevice));
  GK(cudaMemcpy(db.p, b, 8 * nb, cudaMemcpyHostToDevice));
  GK(cudaMalloc(&dout.p, n));
  k_xsection<<<(unsigned)((n + kT - 1) / kT), kT>>>(
      S, static_cast<double*>(dp.p), n_points, static_cast<double*>(da.p), na,
      static_cast<double*>(db.p), nb, static_cast<uint8_t*>(dout.p));
  GK(cudaGetLastError());
  note_launches(1);
  GK(cudaMemcpy(out, dout.p, n, cudaMemcpyDeviceToHost));
  return IG_OK;
}

extern "C" int ig_shapes_label(const long long* table, int n_shapes, const uint8_t* xs,
                               long long xs_len, const uint8_t* rng, long long rng_len,
                               const int* electrode_index, int n_electrodes, long nx, long ny,
                               long nz, int16_t* labels_out, unsigned long long* counts_out,
                               unsigned long long* clash_counts_out,
                               unsigned long long* clash_first_out) {
  set_last_error("");
  if (!table || n_shapes < 0 || !xs || !rng || !electrode_index || n_electrodes < 1 ||
      !labels_out || nx < 1 || ny < 1 || nz < 1) {
    set_last_error("invalid shape-label arguments");
    return IG_BAD_ARG;
  }
  const long len[3] = {nx, ny, nz};
  std::vector<ShapeRec> recs((size_t)(n_shapes > 0 ? n_shapes : 1));
  for (int q = 0; q < n_shapes; q++) {
    // rows: slot, axis, cutout, xs_off, rng_off (7 long longs with na, nb)
    const long long* r = table + 7 * q;
    ShapeRec& R = recs[q];
    R.slot = (int)r[0];
    R.axis = (int)r[1];
    R.cutout = (int)r[2];
    R.xs_off = r[3];
    R.rng_off = r[4];
    R.na = (int)r[5];
    R.nb = (int)r[6];
    const int a1 = (R.axis + 1) % 3, a2 = (R.axis + 2) % 3;
    if (R.axis < 0 || R.axis > 2 || R.slot < 0 || R.slot >= n_electrodes ||
        (q > 0 && R.slot < recs[q - 1].slot) || R.na != len[a1] || R.nb != len[a2] ||
        R.xs_off < 0 || R.xs_off + (long long)R.na * R.nb > xs_len || R.rng_off < 0 ||
        R.rng_off + len[R.axis] > rng_len) {
      set_last_error("malformed shape table");
      return IG_BAD_ARG;
    }
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_last_error("no CUDA device is visible");
    return IG_NO_DEVICE;
  }
  const size_t n = (size_t)nx * ny * nz;
  Tmp drec, dxs, drng, deidx, dlab, dcnt;
  GK(cudaMalloc(&drec.p, sizeof(ShapeRec) * recs.size()));
  GK(cudaMemcpy(drec.p, recs.data(), sizeof(ShapeRec) * recs.size(), cudaMemcpyHostToDevice));
  GK(cudaMalloc(&dxs.p, xs_len > 0 ? xs_len : 1));
  if (xs_len > 0) GK(cudaMemcpy(dxs.p, xs, xs_len, cudaMemcpyHostToDevice));
  GK(cudaMalloc(&drng.p, rng_len > 0 ? rng_len : 1));
  if (rng_len > 0) GK(cudaMemcpy(drng.p, rng, rng_len, cudaMemcpyHostToDevice));
  GK(cudaMalloc(&deidx.p, sizeof(int) * n_electrodes));
  GK(cudaMemcpy(deidx.p, electrode_index, sizeof(int) * n_electrodes, cudaMemcpyHostToDevice));
  GK(cudaMalloc(&dlab.p, 2 * n));
  GK(cudaMalloc(&dcnt.p, 3 * 8 * (size_t)n_electrodes));
  unsigned long long* c = static_cast<unsigned long long*>(dcnt.p);
  GK(cudaMemset(c, 0, 2 * 8 * (size_t)n_electrodes));
  GK(cudaMemset(c + 2 * n_electrodes, 0xff, 8 * (size_t)n_electrodes));
  k_shapes_label<<<(unsigned)((n + kT - 1) / kT), kT>>>(
      static_cast<ShapeRec*>(drec.p), n_shapes, static_cast<uint8_t*>(dxs.p),
      static_cast<uint8_t*>(drng.p), static_cast<int*>(deidx.p), n_electrodes, nx, ny, nz,
      static_cast<int16_t*>(dlab.p), c, c + n_electrodes, c + 2 * n_electrodes);
  GK(cudaGetLastError());
  note_launches(1);
  GK(cudaMemcpy(labels_out, dlab.p, 2 * n, cudaMemcpyDeviceToHost));
  if (counts_out) GK(cudaMemcpy(counts_out, c, 8 * n_electrodes, cudaMemcpyDeviceToHost));
  if (clash_counts_out)
    GK(cudaMemcpy(clash_counts_out, c + n_electrodes, 8 * n_electrodes, cudaMemcpyDeviceToHost));
  if (clash_first_out)
    GK(cudaMemcpy(clash_first_out, c + 2 * n_electrodes, 8 * n_electrodes,
                  cudaMemcpyDeviceToHost));
  return IG_OK;
}
