// ig_solvers.cu -- host drivers of the FP64 solve paths and the C-ABI of
// libigsolve.so (declared in include/igsolve.h).
//
// The drivers restate the reference's Python drivers (solve3d, solve3d_mg,
// solve3d_vmg, _solve_err, the basis loops) with the arrays resident in HBM:
// the host only launches kernels and reads back the few scalars the
// reference branches on (a sweep pair's max |update|, a cycle's max change,
// max |f| of an error level).  Sweep pairs run in batches whose launches
// stop themselves on the device once a pair met the tolerance (PairCtl), so
// the host synchronizes once per batch, not once per pair, and the result is
// still the reference's pair-exact stop.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "ig_common.cuh"
#include "ig_internal.h"
#include "../../include/igsolve.h"

namespace ig {
namespace {

thread_local std::string t_err;
std::atomic<int> g_stop{0};

struct Prof {
  std::atomic<int> on{0};
  double ms = 0.0;
  long launches = 0;
  long nodes = 0;
} g_prof;

struct Status : std::runtime_error {
  int code;
  Status(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CK(x)                                                                  \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess)                                                     \
      throw Status(IG_CUDA_ERROR, std::string(#x) + ": " +                     \
                                      cudaGetErrorString(e_) + " (line " +    \
                                      std::to_string(__LINE__) + ")");         \
  } while (0)

// Per-thread stream and pinned control block, created on first use.
struct ThreadCtx {
  int dev = -1;
  cudaStream_t s = nullptr;
  PairCtl* ctl_h = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  ~ThreadCtx() {
    // process exit: the driver reclaims everything; nothing to do here
  }
};
thread_local ThreadCtx t_ctx;

ThreadCtx& ctx() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
    throw Status(IG_NO_DEVICE, "no CUDA device is visible");
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (t_ctx.dev != dev) {
    t_ctx.dev = dev;
    CK(cudaStreamCreateWithFlags(&t_ctx.s, cudaStreamNonBlocking));
    CK(cudaMallocHost(&t_ctx.ctl_h, sizeof(PairCtl)));
    CK(cudaEventCreate(&t_ctx.ev0));
    CK(cudaEventCreate(&t_ctx.ev1));
    // keep freed stream-ordered allocations cached between solves
    cudaMemPool_t pool;
    CK(cudaDeviceGetDefaultMemPool(&pool, dev));
    uint64_t thr = std::numeric_limits<uint64_t>::max();
    CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  }
  return t_ctx;
}

// Stream-ordered device buffer.
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;
  DBuf() = default;
  DBuf(size_t count, cudaStream_t st) { alloc(count, st); }
  void alloc(size_t count, cudaStream_t st) {
    release();
    s = st;
    n = count;
    if (count) CK(cudaMallocAsync((void**)&p, std::max<size_t>(count * sizeof(T), 16), st));
  }
  void release() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    n = 0;
  }
  ~DBuf() { release(); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), s(o.s) { o.p = nullptr; o.n = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    release();
    p = o.p; n = o.n; s = o.s;
    o.p = nullptr; o.n = 0;
    return *this;
  }
};

void check_dims(long nx, long ny, long nz) {
  if (nx < 1 || ny < 1 || nz < 1)
    throw Status(IG_BAD_ARG, "every axis of the grid must be >= 1");
  const double n = (double)nx * (double)ny * (double)nz;
  if (n >= 2147483648.0)
    throw Status(IG_BAD_ARG, "grids of 2^31 nodes or more are not supported");
}

int stencil_check(int stencil) {
  if (stencil != 0 && stencil != 1)
    throw Status(IG_BAD_ARG, "unknown stencil code (0 = ghost_linear, 1 = sw)");
  return stencil;
}

// Sweep kernel kind for a fine grid: theta None reduces both stencils to
// sum/6 (Shortley-Weller with unit legs halves num and den alike).
int sweep_kind(const float* th, int stencil) {
  if (!th) return kPlain;
  return stencil == 0 ? kThetaGhost : kThetaSW;
}

// Residual kind: with theta None the two stencils differ by a factor of 2
// (ghost_linear: sum - 6 phi; Shortley-Weller: sum/2 - 3 phi).
constexpr int kPlainSWResid = kPlainSW;

double optimal_omega_libm(const Dims& d) {
  // solver3d.optimal_omega (solver3d.py:201-230) for unit spacing
  double num = 0.0, wsum = 0.0;
  const long ns[3] = {d.nx, d.ny, d.nz};
  bool any = false;
  for (long n : ns)
    if (n >= 2) {
      num += std::cos(M_PI / (double)(n + 1));
      wsum += 1.0;
      any = true;
    }
  if (!any) return 1.0;
  double rho = num / wsum;
  rho = std::min(rho, 1.0 - 1e-15);
  return 2.0 / (1.0 + std::sqrt(1.0 - rho * rho));
}

inline double umax(unsigned long long a, unsigned long long b) {
  return bits_to_double(a > b ? a : b);
}

struct PairsResult {
  long pairs;
  double delta;
  bool converged;
};

// The reference's "for s in range(max): d = max(d1, d2); if d < tol: stop"
// loop, in device-terminated batches.  launch_pair(lp, ctl) enqueues the
// colour-0 and colour-1 launches of local pair lp.
template <class F>
PairsResult run_pairs(ThreadCtx& c, PairCtl* ctl_d, double tol, long max_pairs,
                      size_t nodes, F&& launch_pair) {
  PairCtl* h = c.ctl_h;
  long base = 0;
  int has_prev = 0;
  unsigned long long prev[2] = {0, 0};
  double last = std::numeric_limits<double>::quiet_NaN();
  int B = 8;
  const bool prof = g_prof.on.load() != 0;
  while (base < max_pairs) {
    const int lim = (int)std::min<long>(B, max_pairs - base);
    std::memset(h, 0, sizeof(PairCtl));
    h->prev[0] = prev[0];
    h->prev[1] = prev[1];
    h->has_prev = has_prev;
    h->limit = lim;
    h->tol = tol;
    CK(cudaMemcpyAsync(ctl_d, h, sizeof(PairCtl), cudaMemcpyHostToDevice, c.s));
    if (prof) CK(cudaEventRecord(c.ev0, c.s));
    for (int lp = 0; lp < lim; lp++) launch_pair(lp, ctl_d);
    CK(cudaGetLastError());
    if (prof) CK(cudaEventRecord(c.ev1, c.s));
    CK(cudaMemcpyAsync(h, ctl_d, sizeof(PairCtl), cudaMemcpyDeviceToHost, c.s));
    CK(cudaStreamSynchronize(c.s));
    int ran = lim;
    PairsResult res{0, 0.0, false};
    for (int lp = 0; lp < lim; lp++) {
      const double d = umax(h->slot[2 * lp], h->slot[2 * lp + 1]);
      if (d < tol) {
        res = {base + lp + 1, d, true};
        ran = lp + 1;
        break;
      }
      last = d;
    }
    if (prof) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
      g_prof.ms += ms;
      g_prof.launches += 2L * ran;
      g_prof.nodes += (long)nodes * ran;
    }
    if (res.converged) return res;
    prev[0] = h->slot[2 * lim - 2];
    prev[1] = h->slot[2 * lim - 1];
    has_prev = 1;
    base += lim;
    B = std::min(kMaxBatch, 2 * B);
  }
  return {max_pairs, last, false};
}

// Reads back one 64-bit max key (sync) as a double, NaN when flagged.
double read_absmax(ThreadCtx& c, unsigned long long* bits_d, int* nan_d) {
  unsigned long long b = 0;
  int nanf = 0;
  CK(cudaMemcpyAsync(&b, bits_d, 8, cudaMemcpyDeviceToHost, c.s));
  if (nan_d) CK(cudaMemcpyAsync(&nanf, nan_d, 4, cudaMemcpyDeviceToHost, c.s));
  CK(cudaStreamSynchronize(c.s));
  if (nanf) return std::numeric_limits<double>::quiet_NaN();
  return bits_to_double(b);
}

double device_absmax(ThreadCtx& c, const double* a, const double* b, size_t n,
                     DBuf<unsigned long long>& scratch) {
  // scratch: [0] = max bits, [1] = NaN flag (as int in the low word)
  CK(cudaMemsetAsync(scratch.p, 0, 16, c.s));
  launch_absdiff_max(c.s, a, b, n, scratch.p, (int*)(scratch.p + 1));
  CK(cudaGetLastError());
  return read_absmax(c, scratch.p, (int*)(scratch.p + 1));
}

// ---------------------------------------------------------------- SOR
struct FineGrid {
  Dims d;
  DBuf<uint8_t> fixed;
  DBuf<double> phi;
  DBuf<float> th;  // empty when theta is None
  int stencil = 0;
  const float* thp() const { return th.p; }
};

// phi = phi0 (or 0); phi[fixed] = val[fixed]  (solver3d.py:263-265)
void init_phi(ThreadCtx& c, FineGrid& g, const double* val_h,
              const double* phi0_h, DBuf<double>& val_d) {
  const size_t n = g.d.n();
  if (phi0_h)
    CK(cudaMemcpyAsync(g.phi.p, phi0_h, n * 8, cudaMemcpyDefault, c.s));
  else
    CK(cudaMemsetAsync(g.phi.p, 0, n * 8, c.s));
  val_d.alloc(n, c.s);
  CK(cudaMemcpyAsync(val_d.p, val_h, n * 8, cudaMemcpyDefault, c.s));
  launch_set_fixed(c.s, g.phi.p, g.fixed.p, val_d.p, n);
}

PairsResult sor_loop(ThreadCtx& c, double* phi, const uint8_t* fx,
                     const float* th, int stencil, Dims d, double omega,
                     double tol, long max_pairs, PairCtl* ctl_d) {
  const int kind = sweep_kind(th, stencil);
  cudaStream_t s = c.s;
  return run_pairs(c, ctl_d, tol, max_pairs, d.n(), [&](int lp, PairCtl* ctl) {
    launch_sweep(s, phi, fx, th, kind, d, omega, 0, nullptr, ctl, lp);
    launch_sweep(s, phi, fx, th, kind, d, omega, 1, nullptr, ctl, lp);
  });
}

// ---------------------------------------------------------------- V-cycle
struct ErrLevel {
  Dims d;
  DBuf<uint8_t> fixed;
  DBuf<double> e, f, r;
  bool bottom = false;
};

struct VCycle {
  std::vector<ErrLevel> lv;  // lv[0]: the first coarse (error) level
  DBuf<unsigned long long> slots;  // per-pair max keys of fixed-count sweeps
  DBuf<unsigned long long> red;    // absmax scratch
  DBuf<PairCtl> ctl;
  double bottom_omega = 1.0;
  int nu1 = 3, nu2 = 3;
  double rel_tol = 0.05;
  int max_cycles_err = 30;
  int min_coarse = 9;
};

// Builds the error hierarchy below a fine grid: block-ANY masks
// (multigrid3d.py:675 on the fine grid, :578 on every error level).
void build_err_levels(ThreadCtx& c, VCycle& v, const uint8_t* fine_fixed,
                      Dims fine) {
  Dims d = coarse_of(fine);
  const uint8_t* src = fine_fixed;
  Dims sd = fine;
  while (true) {
    ErrLevel L;
    L.d = d;
    L.fixed.alloc(d.n(), c.s);
    launch_coarsen_any(c.s, src, sd, L.fixed.p, d);
    L.e.alloc(d.n(), c.s);
    L.f.alloc(d.n(), c.s);
    L.bottom = std::min({d.nx, d.ny, d.nz}) <= v.min_coarse;
    if (!L.bottom) L.r.alloc(d.n(), c.s);
    v.lv.push_back(std::move(L));
    if (v.lv.back().bottom) break;
    src = v.lv.back().fixed.p;
    sd = d;
    d = coarse_of(d);
  }
  CK(cudaGetLastError());
}

// multigrid3d._solve_err (multigrid3d.py:553-599) on level L; the level's
// right-hand side is already in lv[L].f, the solution lands in lv[L].e.
void solve_err(ThreadCtx& c, VCycle& v, size_t L) {
  ErrLevel& a = v.lv[L];
  const size_t n = a.d.n();
  if (a.bottom && launch_bottom_err(c.s, a.e.p, a.fixed.p, a.f.p, a.d, v.rel_tol,
                                    v.bottom_omega, 20000)) {
    CK(cudaGetLastError());
    return;
  }
  CK(cudaMemsetAsync(a.e.p, 0, n * 8, c.s));
  const double fmax = device_absmax(c, a.f.p, nullptr, n, v.red);
  const double scale = (1e-300 > fmax) ? 1e-300 : fmax;  // max(|f|.max(), 1e-300)
  const double tol = v.rel_tol * scale / 6.0;
  if (a.bottom) {
    const double om = v.bottom_omega;
    double* e = a.e.p;
    const uint8_t* fx = a.fixed.p;
    const double* f = a.f.p;
    const Dims d = a.d;
    cudaStream_t s = c.s;
    run_pairs(c, v.ctl.p, 0.02 * tol, 20000, 0, [&](int lp, PairCtl* ctl) {
      launch_sweep_rhs(s, e, fx, f, d, om, 0, nullptr, ctl, lp);
      launch_sweep_rhs(s, e, fx, f, d, om, 1, nullptr, ctl, lp);
    });
    return;
  }
  ErrLevel& b = v.lv[L + 1];
  unsigned long long* sl = v.slots.p;
  for (int cyc = 0; cyc < v.max_cycles_err; cyc++) {
    for (int q = 0; q < v.nu1; q++) {
      launch_sweep_rhs(c.s, a.e.p, a.fixed.p, a.f.p, a.d, 1.0, 0, sl, nullptr, 0);
      launch_sweep_rhs(c.s, a.e.p, a.fixed.p, a.f.p, a.d, 1.0, 1, sl, nullptr, 0);
    }
    launch_residual_rhs(c.s, a.e.p, a.fixed.p, a.f.p, a.d, a.r.p);
    launch_restrict(c.s, a.r.p, a.d, b.f.p, b.d, 1);
    solve_err(c, v, L + 1);
    launch_prolong_add(c.s, b.e.p, b.d, a.e.p, a.fixed.p, a.d);
    if (v.nu2 > 0) {
      CK(cudaMemsetAsync(sl, 0, 2 * v.nu2 * 8, c.s));
      for (int q = 0; q < v.nu2; q++) {
        launch_sweep_rhs(c.s, a.e.p, a.fixed.p, a.f.p, a.d, 1.0, 0, sl + 2 * q, nullptr, 0);
        launch_sweep_rhs(c.s, a.e.p, a.fixed.p, a.f.p, a.d, 1.0, 1, sl + 2 * q + 1, nullptr, 0);
      }
      CK(cudaGetLastError());
      unsigned long long last[2];
      CK(cudaMemcpyAsync(last, sl + 2 * (v.nu2 - 1), 16, cudaMemcpyDeviceToHost, c.s));
      CK(cudaStreamSynchronize(c.s));
      if (umax(last[0], last[1]) < tol) break;
    } else {
      if (0.0 < tol) break;
    }
  }
}

// Axes along which fixed and val are exactly flip-invariant
// (multigrid3d.py:643-650).  val(p) is read through a callback so a basis
// solve can test v_basis * mask without materialising val.
template <class V>
std::vector<int> sym_axes(const uint8_t* fixed, V&& val, Dims d) {
  std::vector<int> axes;
  const long n[3] = {d.nx, d.ny, d.nz};
  for (int a = 0; a < 3; a++) {
    if (n[a] < 3) continue;
    bool ok = true;
    for (long i = 0; i < d.nx && ok; i++)
      for (long j = 0; j < d.ny && ok; j++)
        for (long k = 0; k < d.nz; k++) {
          long mi = i, mj = j, mk = k;
          if (a == 0) mi = d.nx - 1 - i;
          else if (a == 1) mj = d.ny - 1 - j;
          else mk = d.nz - 1 - k;
          const size_t p = ((size_t)i * d.ny + j) * d.nz + k;
          const size_t q = ((size_t)mi * d.ny + mj) * d.nz + mk;
          if ((fixed[p] != 0) != (fixed[q] != 0) || !(val(p) == val(q))) {
            ok = false;
            break;
          }
        }
    if (ok) axes.push_back(a);
  }
  return axes;
}

struct VmgOut {
  int status;
  long sweeps;
  double delta;
  int cycles;
  double prev;
};

// multigrid3d.solve3d_vmg (multigrid3d.py:602-731) on a prepared fine grid.
VmgOut vmg_loop(ThreadCtx& c, FineGrid& g, VCycle& v, double tol,
                int max_cycles, int accept_stagnation,
                const std::vector<int>& sym) {
  const size_t n = g.d.n();
  const int kind = sweep_kind(g.thp(), g.stencil);
  const int rkind = g.thp() ? kind : (g.stencil == 0 ? kPlain : kPlainSWResid);
  DBuf<double> r(n, c.s), phi_c0(n, c.s);
  ErrLevel& e0 = v.lv[0];
  long sweeps = 0;
  double prev = std::numeric_limits<double>::infinity();
  double cycle_d = std::numeric_limits<double>::infinity();
  for (int cyc = 0; cyc < max_cycles; cyc++) {
    if (g_stop.load()) return {IG_INTERRUPTED, sweeps, prev, cyc, prev};
    CK(cudaMemcpyAsync(phi_c0.p, g.phi.p, n * 8, cudaMemcpyDeviceToDevice, c.s));
    for (int q = 0; q < v.nu1; q++) {
      launch_sweep(c.s, g.phi.p, g.fixed.p, g.thp(), kind, g.d, 1.0, 0, nullptr, nullptr, 0);
      launch_sweep(c.s, g.phi.p, g.fixed.p, g.thp(), kind, g.d, 1.0, 1, nullptr, nullptr, 0);
      sweeps++;
    }
    CK(cudaGetLastError());
    if (g_stop.load()) {
      CK(cudaStreamSynchronize(c.s));
      return {IG_INTERRUPTED, sweeps, prev, cyc, prev};
    }
    launch_residual(c.s, g.phi.p, g.fixed.p, g.thp(), rkind, g.d, r.p, nullptr);
    launch_restrict(c.s, r.p, g.d, e0.f.p, e0.d, 1);
    CK(cudaGetLastError());
    solve_err(c, v, 0);
    launch_prolong_add(c.s, e0.e.p, e0.d, g.phi.p, g.fixed.p, g.d);
    for (int q = 0; q < v.nu2; q++) {
      launch_sweep(c.s, g.phi.p, g.fixed.p, g.thp(), kind, g.d, 1.0, 0, nullptr, nullptr, 0);
      launch_sweep(c.s, g.phi.p, g.fixed.p, g.thp(), kind, g.d, 1.0, 1, nullptr, nullptr, 0);
      sweeps++;
    }
    for (int a : sym) launch_sym_project(c.s, g.phi.p, g.d, a);
    CK(cudaGetLastError());
    cycle_d = device_absmax(c, g.phi.p, phi_c0.p, n, v.red);
    if (cycle_d < tol) return {IG_OK, sweeps, cycle_d, cyc + 1, prev};
    if (cycle_d >= prev) {
      if (accept_stagnation) return {IG_OK, sweeps, cycle_d, cyc + 1, prev};
      return {IG_STAGNATED, sweeps, cycle_d, cyc, prev};
    }
    prev = cycle_d;
  }
  return {IG_CYCLE_CAP, sweeps, cycle_d, max_cycles, prev};
}

void prepare_vcycle(ThreadCtx& c, VCycle& v, FineGrid& g, int nu1, int nu2,
                    double bottom_omega) {
  v.nu1 = nu1;
  v.nu2 = nu2;
  build_err_levels(c, v, g.fixed.p, g.d);
  v.bottom_omega = bottom_omega > 0 ? bottom_omega : optimal_omega_libm(v.lv.back().d);
  v.slots.alloc(2 * std::max(1, std::max(nu1, nu2)) + 2, c.s);
  CK(cudaMemsetAsync(v.slots.p, 0, v.slots.n * 8, c.s));
  v.red.alloc(2, c.s);
  v.ctl.alloc(1, c.s);
}

void load_fine(ThreadCtx& c, FineGrid& g, const uint8_t* fixed,
               const float* theta, long nx, long ny, long nz, int stencil) {
  check_dims(nx, ny, nz);
  g.d = Dims{nx, ny, nz};
  g.stencil = stencil_check(stencil);
  const size_t n = g.d.n();
  g.fixed.alloc(n, c.s);
  CK(cudaMemcpyAsync(g.fixed.p, fixed, n, cudaMemcpyDefault, c.s));
  g.phi.alloc(n, c.s);
  if (theta) {
    g.th.alloc(6 * n, c.s);
    CK(cudaMemcpyAsync(g.th.p, theta, 6 * n * 4, cudaMemcpyDefault, c.s));
  }
}

void copy_out(ThreadCtx& c, const double* d, double* h, size_t n) {
  CK(cudaMemcpyAsync(h, d, n * 8, cudaMemcpyDefault, c.s));
  CK(cudaStreamSynchronize(c.s));
}

// ---------------------------------------------------------------- cascadic
struct MgLevel {
  Dims d;
  DBuf<uint8_t> fixed;
  DBuf<double> val;
};

std::vector<MgLevel> build_mg_levels(ThreadCtx& c, const uint8_t* fixed_h,
                                     const double* val_h, Dims d,
                                     int min_coarse, int max_levels) {
  std::vector<MgLevel> lv;
  MgLevel f0;
  f0.d = d;
  f0.fixed.alloc(d.n(), c.s);
  f0.val.alloc(d.n(), c.s);
  CK(cudaMemcpyAsync(f0.fixed.p, fixed_h, d.n(), cudaMemcpyDefault, c.s));
  CK(cudaMemcpyAsync(f0.val.p, val_h, d.n() * 8, cudaMemcpyDefault, c.s));
  lv.push_back(std::move(f0));
  while ((int)lv.size() < max_levels) {
    const Dims& a = lv.back().d;
    const Dims b = coarse_of(a);
    if (std::min({a.nx, a.ny, a.nz}) <= min_coarse || std::min({b.nx, b.ny, b.nz}) < 3) break;
    MgLevel L;
    L.d = b;
    L.fixed.alloc(b.n(), c.s);
    L.val.alloc(b.n(), c.s);
    launch_coarsen_mask(c.s, lv.back().fixed.p, lv.back().val.p, a, L.fixed.p, L.val.p, b);
    lv.push_back(std::move(L));
  }
  CK(cudaGetLastError());
  return lv;
}

// ---------------------------------------------------------------- C-ABI glue
template <class F>
int guard(F&& f) {
  try {
    t_err.clear();
    return f();
  } catch (const Status& s) {
    t_err = s.what();
    return s.code;
  } catch (const std::exception& e) {
    t_err = e.what();
    return IG_CUDA_ERROR;
  }
}

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

}  // namespace
}  // namespace ig

using namespace ig;

void ig::set_last_error(const std::string& m) { t_err = m; }

extern "C" {

const char* ig_last_error(void) { return t_err.c_str(); }
int ig_abi_version(void) { return 2; }
int ig_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

void ig_request_stop(void) { g_stop.store(1); }
void ig_clear_stop(void) { g_stop.store(0); }
int ig_stop_requested(void) { return g_stop.load(); }

void ig_prof_enable(int on) { g_prof.on.store(on ? 1 : 0); }
void ig_prof_reset(void) {
  g_prof.ms = 0.0;
  g_prof.launches = 0;
  g_prof.nodes = 0;
}
long ig_launch_count(void) { return launch_total(); }
void ig_prof_read(double* ms, long* launches, long* nodes) {
  if (ms) *ms = g_prof.ms;
  if (launches) *launches = g_prof.launches;
  if (nodes) *nodes = g_prof.nodes;
}

int ig_solve3d(const uint8_t* fixed, const double* val, const float* theta,
               long nx, long ny, long nz, double tol, long max_sweeps,
               double omega, const double* phi0, int stencil, double* phi_out,
               long* sweeps_out, double* delta_out) {
  return guard([&] {
    if (!fixed || !val || !phi_out) throw Status(IG_BAD_ARG, "null array");
    ThreadCtx& c = ctx();
    FineGrid g;
    load_fine(c, g, fixed, theta, nx, ny, nz, stencil);
    DBuf<double> val_d;
    init_phi(c, g, val, phi0, val_d);
    DBuf<PairCtl> ctl(1, c.s);
    const PairsResult r = sor_loop(c, g.phi.p, g.fixed.p, g.thp(), g.stencil, g.d,
                                    omega, tol, max_sweeps, ctl.p);
    copy_out(c, g.phi.p, phi_out, g.d.n());
    if (sweeps_out) *sweeps_out = r.pairs;
    if (delta_out) *delta_out = r.delta;
    if (!r.converged) {
      t_err = "SOR reached its sweep cap";
      return (int)IG_NOT_CONVERGED;
    }
    return (int)IG_OK;
  });
}

int ig_solve_basis_sor(const uint8_t* metal, const uint8_t* mask,
                       double v_basis, const float* theta, long nx, long ny,
                       long nz, double tol, long max_sweeps, double omega,
                       int stencil, double* phi_out, long* sweeps_out,
                       double* delta_out) {
  return guard([&] {
    if (!metal || !mask || !phi_out) throw Status(IG_BAD_ARG, "null array");
    check_dims(nx, ny, nz);
    const size_t n = (size_t)nx * ny * nz;
    std::vector<double> val(n);
    for (size_t p = 0; p < n; p++) val[p] = mask[p] ? v_basis : 0.0;
    return ig_solve3d(metal, val.data(), theta, nx, ny, nz, tol, max_sweeps,
                      omega, nullptr, stencil, phi_out, sweeps_out, delta_out);
  });
}

int ig_solve3d_mg(const uint8_t* fixed, const double* val, const float* theta,
                  long nx, long ny, long nz, double tol, long max_sweeps,
                  int stencil, int min_coarse, int max_levels,
                  double level_tol_factor, const double* level_omega,
                  int n_level_omega, double* phi_out, long* sweeps_out,
                  double* delta_out) {
  return guard([&] {
    if (!fixed || !val || !phi_out) throw Status(IG_BAD_ARG, "null array");
    check_dims(nx, ny, nz);
    stencil_check(stencil);
    ThreadCtx& c = ctx();
    const Dims d0{nx, ny, nz};
    std::vector<MgLevel> lv = build_mg_levels(c, fixed, val, d0, min_coarse, std::max(1, max_levels));
    const int nl = (int)lv.size();
    auto omega_of = [&](int L) {
      if (level_omega && L < n_level_omega) return level_omega[L];
      return optimal_omega_libm(lv[L].d);
    };
    DBuf<PairCtl> ctl(1, c.s);
    DBuf<float> th_d;
    if (theta) {
      th_d.alloc(6 * d0.n(), c.s);
      CK(cudaMemcpyAsync(th_d.p, theta, 6 * d0.n() * 4, cudaMemcpyDefault, c.s));
    }
    // coarsest level: cold solve with theta None (multigrid3d.py:200-204);
    // then each finer level from the prolongated guess (multigrid3d.py:206-226)
    DBuf<double> cur;
    Dims cd{0, 0, 0};
    for (int L = nl - 1; L >= 0; L--) {
      MgLevel& M = lv[L];
      const size_t n = M.d.n();
      DBuf<double> phi(n, c.s);
      if (L == nl - 1)
        CK(cudaMemsetAsync(phi.p, 0, n * 8, c.s));
      else
        launch_prolongate(c.s, cur.p, cd, phi.p, M.d);
      launch_set_fixed(c.s, phi.p, M.fixed.p, M.val.p, n);
      // the coarsest solve always uses the plain stencil; with a one-level
      // hierarchy the reference then solves the fine grid again from zero
      // with theta (multigrid3d.py:201-203, 220-226)
      const float* th = (L == 0 && nl > 1) ? th_d.p : nullptr;
      const double ltol = (L == 0 || L == nl - 1) ? tol : tol * level_tol_factor;
      PairsResult r = sor_loop(c, phi.p, M.fixed.p, th, stencil, M.d,
                               omega_of(L), ltol, max_sweeps, ctl.p);
      if (nl == 1 && r.converged && th_d.p) {
        CK(cudaMemsetAsync(phi.p, 0, n * 8, c.s));
        launch_set_fixed(c.s, phi.p, M.fixed.p, M.val.p, n);
        r = sor_loop(c, phi.p, M.fixed.p, th_d.p, stencil, M.d, omega_of(0),
                     tol, max_sweeps, ctl.p);
      }
      if (!r.converged || L == 0) {
        if (sweeps_out) *sweeps_out = r.pairs;
        if (delta_out) *delta_out = r.delta;
      }
      if (!r.converged) {
        if (L == 0) copy_out(c, phi.p, phi_out, n);
        t_err = "SOR reached its sweep cap on cascadic level " + std::to_string(L);
        return (int)IG_NOT_CONVERGED;
      }
      if (L == 0) {
        copy_out(c, phi.p, phi_out, n);
        return (int)IG_OK;
      }
      cur = std::move(phi);
      cd = M.d;
    }
    return (int)IG_OK;
  });
}

int ig_solve3d_vmg(const uint8_t* fixed, const double* val, const float* theta,
                   long nx, long ny, long nz, double tol, int max_cycles,
                   int nu1, int nu2, int stencil, const double* phi0,
                   int accept_stagnation, double bottom_omega, double* phi_out,
                   long* sweeps_out, double* delta_out, int* cycles_out,
                   double* prev_delta_out) {
  return guard([&] {
    if (!fixed || !val || !phi_out) throw Status(IG_BAD_ARG, "null array");
    if (nu1 < 0 || nu2 < 0) throw Status(IG_BAD_ARG, "nu1 and nu2 must be >= 0");
    ThreadCtx& c = ctx();
    FineGrid g;
    load_fine(c, g, fixed, theta, nx, ny, nz, stencil);
    DBuf<double> val_d;
    init_phi(c, g, val, phi0, val_d);
    std::vector<int> sym;
    if (!theta) sym = sym_axes(fixed, [&](size_t p) { return val[p]; }, g.d);
    VCycle v;
    prepare_vcycle(c, v, g, nu1, nu2, bottom_omega);
    const VmgOut o = vmg_loop(c, g, v, tol, max_cycles, accept_stagnation, sym);
    copy_out(c, g.phi.p, phi_out, g.d.n());
    if (sweeps_out) *sweeps_out = o.sweeps;
    if (delta_out) *delta_out = o.delta;
    if (cycles_out) *cycles_out = o.cycles;
    if (prev_delta_out) *prev_delta_out = o.prev;
    if (o.status != IG_OK) t_err = "V-cycle did not reach tol";
    return o.status;
  });
}

int ig_solve_basis_vmg(const uint8_t* metal, const uint8_t* mask,
                       double v_basis, const float* theta, long nx, long ny,
                       long nz, double tol, int max_cycles, int nu1, int nu2,
                       int stencil, double bottom_omega, double* phi_out,
                       long* sweeps_out, double* delta_out, int* cycles_out,
                       double* prev_delta_out) {
  return guard([&] {
    if (!metal || !mask || !phi_out) throw Status(IG_BAD_ARG, "null array");
    check_dims(nx, ny, nz);
    const size_t n = (size_t)nx * ny * nz;
    std::vector<double> val(n);
    for (size_t p = 0; p < n; p++) val[p] = mask[p] ? v_basis : 0.0;
    return ig_solve3d_vmg(metal, val.data(), theta, nx, ny, nz, tol, max_cycles,
                          nu1, nu2, stencil, nullptr, 0, bottom_omega, phi_out,
                          sweeps_out, delta_out, cycles_out, prev_delta_out);
  });
}

int ig_cascadic_relres(const uint8_t* fixed, const double* val, long nx,
                       long ny, long nz, double rel_tol, long max_sweeps,
                       int min_coarse, int max_levels, double level_tol_factor,
                       const double* level_omega, int n_level_omega,
                       int check_every, double* phi_out, long* sweeps_out,
                       double* relres_out, long* total_pairs_out,
                       int* levels_out) {
  return guard([&] {
    if (!fixed || !val || !phi_out) throw Status(IG_BAD_ARG, "null array");
    if (check_every < 1) throw Status(IG_BAD_ARG, "check_every must be >= 1");
    check_dims(nx, ny, nz);
    ThreadCtx& c = ctx();
    const Dims d0{nx, ny, nz};
    std::vector<MgLevel> lv = build_mg_levels(c, fixed, val, d0, min_coarse, std::max(1, max_levels));
    const int nl = (int)lv.size();
    if (levels_out) *levels_out = nl;
    DBuf<unsigned long long> red(2, c.s);
    DBuf<double> cur, nxt;
    Dims cd{0, 0, 0};
    long total = 0;
    const bool prof = g_prof.on.load() != 0;
    for (int L = nl - 1; L >= 0; L--) {
      MgLevel& M = lv[L];
      const size_t n = M.d.n();
      nxt.alloc(n, c.s);
      // ||b||: residual of the Dirichlet values with zeros elsewhere
      CK(cudaMemsetAsync(nxt.p, 0, n * 8, c.s));
      launch_set_fixed(c.s, nxt.p, M.fixed.p, M.val.p, n);
      CK(cudaMemsetAsync(red.p, 0, 16, c.s));
      launch_residual(c.s, nxt.p, M.fixed.p, nullptr, kPlain, M.d, nullptr, red.p);
      const double bnorm = read_absmax(c, red.p, nullptr);
      if (L < nl - 1) {
        launch_prolongate(c.s, cur.p, cd, nxt.p, M.d);
        launch_set_fixed(c.s, nxt.p, M.fixed.p, M.val.p, n);
      }
      const double om = (level_omega && L < n_level_omega) ? level_omega[L] : optimal_omega_libm(M.d);
      const double ltol = (L == 0 || L == nl - 1) ? rel_tol : rel_tol * level_tol_factor;
      long pairs = 0;
      double rr = std::numeric_limits<double>::infinity();
      while (true) {
        CK(cudaMemsetAsync(red.p, 0, 16, c.s));
        launch_residual(c.s, nxt.p, M.fixed.p, nullptr, kPlain, M.d, nullptr, red.p);
        const double rmax = read_absmax(c, red.p, nullptr);
        rr = bnorm > 0 ? rmax / bnorm : rmax;
        if (rr < ltol || pairs >= max_sweeps) break;
        const int chunk = (int)std::min<long>(check_every, max_sweeps - pairs);
        if (prof) CK(cudaEventRecord(c.ev0, c.s));
        for (int q = 0; q < chunk; q++) {
          launch_sweep(c.s, nxt.p, M.fixed.p, nullptr, kPlain, M.d, om, 0, nullptr, nullptr, 0);
          launch_sweep(c.s, nxt.p, M.fixed.p, nullptr, kPlain, M.d, om, 1, nullptr, nullptr, 0);
        }
        CK(cudaGetLastError());
        if (prof) {
          CK(cudaEventRecord(c.ev1, c.s));
          CK(cudaEventSynchronize(c.ev1));
          float ms = 0.f;
          CK(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
          g_prof.ms += ms;
          g_prof.launches += 2L * chunk;
          g_prof.nodes += (long)n * chunk;
        }
        pairs += chunk;
      }
      total += pairs;
      if (L == 0) {
        copy_out(c, nxt.p, phi_out, n);
        if (sweeps_out) *sweeps_out = pairs;
        if (relres_out) *relres_out = rr;
        if (total_pairs_out) *total_pairs_out = total;
        if (!(rr < ltol)) {
          t_err = "cascadic solve reached its sweep cap";
          return (int)IG_NOT_CONVERGED;
        }
        return (int)IG_OK;
      }
      cur = std::move(nxt);
      cd = M.d;
    }
    return (int)IG_OK;
  });
}

// ---- single kernels ----------------------------------------------------

namespace {
struct KScratch {
  int dev = -1;
  unsigned long long* d = nullptr;
};
thread_local KScratch t_ks;

unsigned long long* kscratch() {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (t_ks.dev != dev) {
    CK(cudaMalloc(&t_ks.d, 16));
    t_ks.dev = dev;
  }
  return t_ks.d;
}

double finish_max(cudaStream_t s, unsigned long long* slot) {
  unsigned long long b = 0;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(&b, slot, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return bits_to_double(b);
}
}  // namespace

int ig_sweep_dev(double* phi, const uint8_t* fixed, const float* theta,
                 long nx, long ny, long nz, double omega, int colour,
                 int stencil, double* dmax_out, void* stream) {
  return guard([&] {
    check_dims(nx, ny, nz);
    stencil_check(stencil);
    cudaStream_t s = as_stream(stream);
    unsigned long long* slot = kscratch();
    CK(cudaMemsetAsync(slot, 0, 8, s));
    launch_sweep(s, phi, fixed, theta, sweep_kind(theta, stencil), Dims{nx, ny, nz},
                 omega, colour & 1, slot, nullptr, 0);
    const double d = finish_max(s, slot);
    if (dmax_out) *dmax_out = d;
    return (int)IG_OK;
  });
}

int ig_residual_dev(const double* phi, const uint8_t* fixed, const float* theta,
                    long nx, long ny, long nz, int stencil, double* out,
                    void* stream) {
  return guard([&] {
    check_dims(nx, ny, nz);
    stencil_check(stencil);
    const int kind = theta ? sweep_kind(theta, stencil) : (stencil == 0 ? kPlain : kPlainSWResid);
    launch_residual(as_stream(stream), phi, fixed, theta, kind, Dims{nx, ny, nz}, out, nullptr);
    CK(cudaGetLastError());
    return (int)IG_OK;
  });
}

int ig_sweep_rhs_dev(double* e, const uint8_t* fixed, const double* f, long nx,
                     long ny, long nz, double omega, int colour,
                     double* dmax_out, void* stream) {
  return guard([&] {
    check_dims(nx, ny, nz);
    cudaStream_t s = as_stream(stream);
    unsigned long long* slot = kscratch();
    CK(cudaMemsetAsync(slot, 0, 8, s));
    launch_sweep_rhs(s, e, fixed, f, Dims{nx, ny, nz}, omega, colour & 1, slot, nullptr, 0);
    const double d = finish_max(s, slot);
    if (dmax_out) *dmax_out = d;
    return (int)IG_OK;
  });
}

int ig_residual_rhs_dev(const double* e, const uint8_t* fixed, const double* f,
                        long nx, long ny, long nz, double* out, void* stream) {
  return guard([&] {
    check_dims(nx, ny, nz);
    launch_residual_rhs(as_stream(stream), e, fixed, f, Dims{nx, ny, nz}, out);
    CK(cudaGetLastError());
    return (int)IG_OK;
  });
}

int ig_restrict_fw_dev(const double* fine, long nx, long ny, long nz,
                       double* out, void* stream) {
  return guard([&] {
    check_dims(nx, ny, nz);
    const Dims d{nx, ny, nz};
    launch_restrict(as_stream(stream), fine, d, out, coarse_of(d), 0);
    CK(cudaGetLastError());
    return (int)IG_OK;
  });
}

int ig_prolong_add_dev(const double* coarse, long cx, long cy, long cz,
                       double* out, const uint8_t* fixed, long nx, long ny,
                       long nz, void* stream) {
  return guard([&] {
    check_dims(nx, ny, nz);
    check_dims(cx, cy, cz);
    launch_prolong_add(as_stream(stream), coarse, Dims{cx, cy, cz}, out, fixed, Dims{nx, ny, nz});
    CK(cudaGetLastError());
    return (int)IG_OK;
  });
}

int ig_prolongate_dev(const double* coarse, long cx, long cy, long cz,
                      double* out, long nx, long ny, long nz, void* stream) {
  return guard([&] {
    check_dims(nx, ny, nz);
    check_dims(cx, cy, cz);
    launch_prolongate(as_stream(stream), coarse, Dims{cx, cy, cz}, out, Dims{nx, ny, nz});
    CK(cudaGetLastError());
    return (int)IG_OK;
  });
}

int ig_coarsen_fixed_any_dev(const uint8_t* fixed, long nx, long ny, long nz,
                             uint8_t* out, void* stream) {
  return guard([&] {
    check_dims(nx, ny, nz);
    const Dims d{nx, ny, nz};
    launch_coarsen_any(as_stream(stream), fixed, d, out, coarse_of(d));
    CK(cudaGetLastError());
    return (int)IG_OK;
  });
}

int ig_coarsen_mask_dev(const uint8_t* fixed, const double* val, long nx,
                        long ny, long nz, uint8_t* fc, double* vc,
                        void* stream) {
  return guard([&] {
    check_dims(nx, ny, nz);
    const Dims d{nx, ny, nz};
    launch_coarsen_mask(as_stream(stream), fixed, val, d, fc, vc, coarse_of(d));
    CK(cudaGetLastError());
    return (int)IG_OK;
  });
}

int ig_residual_audit_dev(const double* u, const uint8_t* fixed,
                          const float* theta, long nx, long ny, long nz,
                          double* out, void* stream) {
  return guard([&] {
    check_dims(nx, ny, nz);
    if (nx < 2 || ny < 2 || nz < 2)
      throw Status(IG_BAD_ARG, "the audit residual needs every axis >= 2");
    if (!theta) throw Status(IG_BAD_ARG, "the audit residual needs theta");
    launch_residual_audit(as_stream(stream), u, fixed, theta, Dims{nx, ny, nz}, out);
    CK(cudaGetLastError());
    return (int)IG_OK;
  });
}

int ig_err_sweep_dev(double* e, const uint8_t* fixed, const float* theta,
                     const double* rhs, long nx, long ny, long nz,
                     double omega, int colour, double* dmax_out,
                     void* stream) {
  return guard([&] {
    check_dims(nx, ny, nz);
    if (nx < 2 || ny < 2 || nz < 2)
      throw Status(IG_BAD_ARG, "the error sweep needs every axis >= 2");
    if (!theta) throw Status(IG_BAD_ARG, "the error sweep needs theta");
    cudaStream_t s = as_stream(stream);
    unsigned long long* slot = kscratch();
    CK(cudaMemsetAsync(slot, 0, 8, s));
    launch_err_sweep(s, e, fixed, theta, rhs, Dims{nx, ny, nz}, omega, colour & 1, slot);
    const double d = finish_max(s, slot);
    if (dmax_out) *dmax_out = d;
    return (int)IG_OK;
  });
}

}  // extern "C"

extern "C" long long ig_device_free_bytes(void) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return 0;
  }
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return (long long)free_b;
}
