// ig_noalloc.cu -- ig_cascadic_relres_noalloc: the residual-stopped cascadic
// solve on device-resident arrays without allocating any memory.
//
// Who needs it: a caller that cannot call cudaMalloc (or have a library call
// it on its behalf) while it runs -- a serving process that reserved its HBM
// budget up front and hands the solver only borrowed buffers, a framework
// whose custom-call interface forbids allocations outside its own allocator,
// or a latency-bound loop in which an allocation could block on the driver.
// ig_cascadic_relres allocates the coarse levels, the fine working copy and a
// reduction slot on every call (stream-ordered pool allocations); this entry
// point iterates in the caller's output array and keeps everything else in
// one file-scope device array, g_noalloc_scratch, of IG_NOALLOC_SCRATCH_BYTES.
//
// The array is part of the library image: every GPU that loads the library
// holds it until the process exits.  All calls share it and it keeps the last
// call's contents, so calls that overlap on the GPU (two host threads, or two
// streams) race on it; serialise them.  The reduction slot is cleared before
// every use; every coarse-level array is fully written before it is read.
//
// Set-up: every call resolves the device address of g_noalloc_scratch with
// cudaGetSymbolAddress on the calling thread's current device (host code
// cannot use the symbol itself: on the host it names a stand-in, not device
// memory).  The lookup allocates nothing, and resolving it per call keeps the
// address right after a device reset or a new primary context, where the
// module is loaded again and the array can move.  The solve synchronises the
// stream at every residual check (the stop decision is taken on the host).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>

#include "ig_common.cuh"
#include "ig_internal.h"
#include "../../include/igsolve.h"

// The scratch itself: file scope, internal linkage, one per device context.
static __device__ __align__(256) unsigned char g_noalloc_scratch[IG_NOALLOC_SCRATCH_BYTES];

namespace ig {
namespace {

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

struct Carve {
  unsigned char* base;
  size_t used;
  template <class T>
  T* take(size_t count) {
    T* p = reinterpret_cast<T*>(base + used);
    used += align256(count * sizeof(T));
    return p;
  }
};

struct Level {
  Dims d;
  uint8_t* fixed;
  double* val;
  double* phi;
};

// Bytes of scratch the coarse hierarchy of `fine` needs (levels 1..L-1:
// mask, Dirichlet values and potential) plus the reduction slot.
size_t scratch_need(Dims fine, int min_coarse, int max_levels, int* nlev) {
  size_t need = align256(16);
  int n = 1;
  Dims a = fine;
  while (n < max_levels) {
    const Dims b = coarse_of(a);
    if (std::min({a.nx, a.ny, a.nz}) <= min_coarse ||
        std::min({b.nx, b.ny, b.nz}) < 3)
      break;
    need += align256(b.n()) + 2 * align256(b.n() * 8);
    a = b;
    n++;
  }
  *nlev = n;
  return need;
}

int fail(int code, const std::string& m) {
  set_last_error(m);
  return code;
}

#define NA_CK(x)                                                          \
  do {                                                                    \
    cudaError_t e_ = (x);                                                 \
    if (e_ != cudaSuccess)                                                \
      return fail(IG_CUDA_ERROR, std::string(#x) + ": " +                 \
                                     cudaGetErrorString(e_));             \
  } while (0)

}  // namespace
}  // namespace ig

using namespace ig;

extern "C" int ig_cascadic_relres_noalloc(
    const uint8_t* fixed, const double* val, long nx, long ny, long nz,
    double rel_tol, long max_sweeps, int min_coarse, int max_levels,
    double level_tol_factor, const double* level_omega, int n_level_omega,
    int check_every, double* phi_out, long* sweeps_out, double* relres_out,
    long* total_pairs_out, int* levels_out, void* stream) {
  set_last_error("");
  if (!fixed || !val || !phi_out)
    return fail(IG_BAD_ARG, "null device array");
  if (nx < 1 || ny < 1 || nz < 1)
    return fail(IG_BAD_ARG, "every axis of the grid must be >= 1");
  if ((double)nx * ny * nz >= 2147483648.0)
    return fail(IG_BAD_ARG, "grids of 2^31 nodes or more are not supported");
  if (check_every < 1) return fail(IG_BAD_ARG, "check_every must be >= 1");
  const Dims d0{nx, ny, nz};
  int nl = 1;
  const size_t need = scratch_need(d0, min_coarse, std::min(32, std::max(1, max_levels)), &nl);
  if (need > (size_t)IG_NOALLOC_SCRATCH_BYTES)
    return fail(IG_BAD_ARG,
                "the coarse levels of a " + std::to_string(nx) + "x" +
                    std::to_string(ny) + "x" + std::to_string(nz) +
                    " grid need " + std::to_string(need) +
                    " bytes of scratch; the static scratch holds " +
                    std::to_string((size_t)IG_NOALLOC_SCRATCH_BYTES) +
                    " bytes (use ig_cascadic_relres for larger grids)");
  // the array's address on the current device (see the file header)
  void* sym = nullptr;
  NA_CK(cudaGetSymbolAddress(&sym, g_noalloc_scratch));
  unsigned char* base = static_cast<unsigned char*>(sym);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);

  // carve the hierarchy: level 0 is the caller's arrays, phi iterates in
  // phi_out; levels 1.. live in the static scratch
  Carve cv{base, 0};
  unsigned long long* red = cv.take<unsigned long long>(2);
  Level lv[32];
  lv[0] = Level{d0, const_cast<uint8_t*>(fixed), const_cast<double*>(val), phi_out};
  for (int L = 1; L < nl; L++) {
    const Dims c = coarse_of(lv[L - 1].d);
    lv[L].d = c;
    lv[L].fixed = cv.take<uint8_t>(c.n());
    lv[L].val = cv.take<double>(c.n());
    lv[L].phi = cv.take<double>(c.n());
    launch_coarsen_mask(s, lv[L - 1].fixed, lv[L - 1].val, lv[L - 1].d,
                        lv[L].fixed, lv[L].val, c);
  }
  NA_CK(cudaGetLastError());
  if (levels_out) *levels_out = nl;

  auto absmax_resid = [&](const Level& M, const double* phi, double* out) -> int {
    unsigned long long b = 0;
    NA_CK(cudaMemsetAsync(red, 0, 16, s));
    launch_residual(s, phi, M.fixed, nullptr, kPlain, M.d, nullptr, red);
    NA_CK(cudaGetLastError());
    NA_CK(cudaMemcpyAsync(&b, red, 8, cudaMemcpyDeviceToHost, s));
    NA_CK(cudaStreamSynchronize(s));
    *out = bits_to_double(b);
    return IG_OK;
  };

  long total = 0;
  for (int L = nl - 1; L >= 0; L--) {
    Level& M = lv[L];
    const size_t n = M.d.n();
    // max|r(phi_D)| with phi_D = Dirichlet values, zero elsewhere
    NA_CK(cudaMemsetAsync(M.phi, 0, n * 8, s));
    launch_set_fixed(s, M.phi, M.fixed, M.val, n);
    double bnorm = 0.0;
    int st = absmax_resid(M, M.phi, &bnorm);
    if (st != IG_OK) return st;
    if (L < nl - 1) {
      launch_prolongate(s, lv[L + 1].phi, lv[L + 1].d, M.phi, M.d);
      launch_set_fixed(s, M.phi, M.fixed, M.val, n);
    }
    double om;
    if (level_omega && L < n_level_omega) {
      om = level_omega[L];
    } else {
      double num = 0.0, w = 0.0;
      const long ns[3] = {M.d.nx, M.d.ny, M.d.nz};
      for (long q : ns)
        if (q >= 2) { num += std::cos(M_PI / (double)(q + 1)); w += 1.0; }
      double rho = w > 0 ? std::min(num / w, 1.0 - 1e-15) : 0.0;
      om = w > 0 ? 2.0 / (1.0 + std::sqrt(1.0 - rho * rho)) : 1.0;
    }
    const double ltol = (L == 0 || L == nl - 1) ? rel_tol : rel_tol * level_tol_factor;
    long pairs = 0;
    double rr = INFINITY;
    while (true) {
      double rmax = 0.0;
      st = absmax_resid(M, M.phi, &rmax);
      if (st != IG_OK) return st;
      rr = bnorm > 0 ? rmax / bnorm : rmax;
      if (rr < ltol || pairs >= max_sweeps) break;
      const int chunk = (int)std::min<long>(check_every, max_sweeps - pairs);
      for (int q = 0; q < chunk; q++) {
        launch_sweep(s, M.phi, M.fixed, nullptr, kPlain, M.d, om, 0, nullptr, nullptr, 0);
        launch_sweep(s, M.phi, M.fixed, nullptr, kPlain, M.d, om, 1, nullptr, nullptr, 0);
      }
      NA_CK(cudaGetLastError());
      pairs += chunk;
    }
    total += pairs;
    if (L == 0) {
      NA_CK(cudaStreamSynchronize(s));
      if (sweeps_out) *sweeps_out = pairs;
      if (relres_out) *relres_out = rr;
      if (total_pairs_out) *total_pairs_out = total;
      if (!(rr < ltol)) return fail(IG_NOT_CONVERGED, "cascadic solve reached its sweep cap");
      return IG_OK;
    }
  }
  return IG_OK;
}
