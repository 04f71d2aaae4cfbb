// ig_internal.h -- declarations shared by the CUDA translation units of
// libigsolve.so (kernel launchers, control blocks).  Not part of the C-ABI;
// the public entry points are in include/igsolve.h.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

namespace ig {

struct Dims {
  long nx, ny, nz;
  size_t n() const { return (size_t)nx * (size_t)ny * (size_t)nz; }
};

inline Dims coarse_of(const Dims& d) {
  return Dims{(d.nx + 1) / 2, (d.ny + 1) / 2, (d.nz + 1) / 2};
}

// Unsigned 31-bit division by a run-time constant (Granlund & Montgomery,
// "Division by invariant integers using multiplication", PLDI 1994):
// q = (umulhi(n, m) + n) >> s with s = ceil(log2 d) and
// m = floor(2^32 (2^s - d) / d) + 1, exact for every n < 2^31.
struct FastDiv {
  uint32_t d, m, s;
  FastDiv() : d(1), m(1), s(0) {}
  explicit FastDiv(uint32_t div) : d(div) {
    s = 0;
    while ((1ull << s) < div) ++s;
    m = (uint32_t)(((1ull << 32) * ((1ull << s) - div)) / div + 1);
  }
};

// Per-batch control block of the exact SOR loop.  A batch is up to
// kMaxBatch red-black pairs launched back to back; slot[2p + c] receives the
// max |update| of colour c of pair p (as order-preserving bits).  The colour-0
// launch of pair p first looks at pair p-1 (or at `prev`, the last pair of
// the previous batch) and, when it met `tol`, marks the batch done so every
// later launch returns at once.  The host then reads the slots and finds the
// pair that converged, exactly as the reference's per-pair test does.
constexpr int kMaxBatch = 256;
struct PairCtl {
  unsigned long long slot[2 * kMaxBatch];
  unsigned long long prev[2];
  double tol;
  int has_prev;
  int limit;
  int done;
  int pad_;
};

// Stencil selector for the fine sweeps.
enum StencilKind : int {
  kPlain = 0,        // theta is all ones: every stencil reduces to sum/6
  kThetaGhost = 1,   // theta given, ghost_linear weights
  kThetaSW = 2,      // theta given, Shortley-Weller weights
  kPlainSW = 3,      // theta all ones, Shortley-Weller residual (sum/2 - 3 phi);
                     // its sweeps equal kPlain's
};

// ---- exact FP64 kernels (ig_f64.cu) ----
// One colour of the reference SOR sweep.  dslot: where the max |update| goes
// when ctl == nullptr; with ctl the slot is ctl->slot[2*lp + colour].
void launch_sweep(cudaStream_t s, double* phi, const uint8_t* fixed,
                  const float* th, int kind, Dims d, double omega, int colour,
                  unsigned long long* dslot, PairCtl* ctl, int lp);
void launch_residual(cudaStream_t s, const double* phi, const uint8_t* fixed,
                     const float* th, int kind, Dims d, double* out,
                     unsigned long long* absmax /* nullable */);
// The whole bottom solve of multigrid3d._solve_err (e = 0, tol from
// max|f|, SOR pairs to 0.02 tol, at most max_pairs) in one CTA with the
// level in shared memory; false (nothing launched) when the level does not
// fit in kBottomSmemMax bytes (17 per node).
constexpr size_t kBottomSmemMax = 200 * 1024;
bool launch_bottom_err(cudaStream_t s, double* e, const uint8_t* fixed, const double* f,
                       Dims d, double rel_tol, double omega, long max_pairs);
void launch_sweep_rhs(cudaStream_t s, double* e, const uint8_t* fixed,
                      const double* f, Dims d, double omega, int colour,
                      unsigned long long* dslot, PairCtl* ctl, int lp);
void launch_residual_rhs(cudaStream_t s, const double* e, const uint8_t* fixed,
                         const double* f, Dims d, double* out);
// out = acc/8 (mode 0) or -((acc/8)*4) (mode 1, the coarse right-hand side)
void launch_restrict(cudaStream_t s, const double* fine, Dims d, double* out,
                     Dims c, int neg4);
void launch_prolong_add(cudaStream_t s, const double* coarse, Dims c,
                        double* out, const uint8_t* fixed, Dims d);
void launch_prolongate(cudaStream_t s, const double* coarse, Dims c,
                       double* out, Dims d);
void launch_coarsen_any(cudaStream_t s, const uint8_t* fixed, Dims d,
                        uint8_t* out, Dims c);
void launch_coarsen_mask(cudaStream_t s, const uint8_t* fixed,
                         const double* val, Dims d, uint8_t* fc, double* vc,
                         Dims c);
void launch_set_fixed(cudaStream_t s, double* phi, const uint8_t* fixed,
                      const double* val, size_t n);
// max |a - b| (b nullable: max |a|) into *bits, NaN noted in *nan_flag
void launch_absdiff_max(cudaStream_t s, const double* a, const double* b,
                        size_t n, unsigned long long* bits, int* nan_flag);
void launch_sym_project(cudaStream_t s, double* phi, Dims d, int axis);
void launch_residual_audit(cudaStream_t s, const double* u,
                           const uint8_t* fixed, const float* th, Dims d,
                           double* out);
void launch_err_sweep(cudaStream_t s, double* e, const uint8_t* fixed,
                      const float* th, const double* rhs, Dims d, double omega,
                      int colour, unsigned long long* dslot);
void launch_fill_ones_f32(cudaStream_t s, float* a, size_t n);

// Number of kernel launches this library has issued since it was loaded.
long launch_total();
// Adds n launches issued by another translation unit to that count.
void note_launches(long n);

// Sets the calling thread's ig_last_error() message.
void set_last_error(const std::string& m);

}  // namespace ig
