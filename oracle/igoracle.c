/*
 * igoracle.c -- CPU restatement of the reference ion_gym 3-D Laplace
 * kernels.  TEST INFRASTRUCTURE ONLY: the parity tests, smoke() and the
 * CPU-baseline leg of bench.py link this file as the checker; the library
 * never does.
 *
 * Parity is pinned: tests/test_oracle_golden.py replays every fixture in
 * tests/golden/{kernels,drivers}.npz (made by running the reference itself,
 * tests/golden/make_golden.py) through this file and requires identical
 * bits.
 *
 * Arithmetic follows the compiled (numba) typing of the reference exactly:
 *   - float64 everywhere a float64 operand or a float literal is involved;
 *   - theta is float32, and sums/products of two theta values stay float32
 *     (the Shortley-Weller leg products), then widen when they meet float64;
 *   - left-to-right evaluation, no contraction into FMA (build with
 *     -ffp-contract=off), no reassociation.
 * Within one red-black colour every update is independent, and the maximum
 * over rows is order-free, so the OpenMP loop over x-planes gives the same
 * bits as the reference's prange loop.
 *
 * Arrays are C-order (nx, ny, nz), z contiguous; theta is (6, nx, ny, nz)
 * in the order (-x, +x, -y, +y, -z, +z).  Boundary rule at every outer face:
 * even reflection (the ghost at -1 is node 1, at n is node n-2), and a
 * size-1 axis uses the node itself.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define AT(a, i, j, k) (a)[((size_t)(i) * (size_t)ny + (size_t)(j)) * (size_t)nz + (size_t)(k)]

/* neighbour index below / above with the even-reflection rule
 * (solver3d.py:156-167, multigrid3d.py:317-328) */
static inline long lo_nb(long i, long n) { return i > 0 ? i - 1 : (n > 1 ? 1 : i); }
static inline long hi_nb(long i, long n) { return i < n - 1 ? i + 1 : (n > 1 ? n - 2 : i); }

int ig_or_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void ig_or_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* The 7-point weights of one node: num and den as the reference forms them
 * (solver3d.py:169-191 == multigrid3d.py:329-353). */
static inline void stencil_num_den(const double v[6], const float *th, size_t N,
                                   size_t p, int ghost_linear, double *num,
                                   double *den)
{
    float t0 = th[0 * N + p], t1 = th[1 * N + p], t2 = th[2 * N + p];
    float t3 = th[3 * N + p], t4 = th[4 * N + p], t5 = th[5 * N + p];
    if (ghost_linear) {
        double w0 = 1.0 / (double)t0, w1 = 1.0 / (double)t1;
        double w2 = 1.0 / (double)t2, w3 = 1.0 / (double)t3;
        double w4 = 1.0 / (double)t4, w5 = 1.0 / (double)t5;
        *num = v[0] * w0 + v[1] * w1 + v[2] * w2 + v[3] * w3 + v[4] * w4 + v[5] * w5;
        *den = w0 + w1 + w2 + w3 + w4 + w5;
    } else {
        float sx = t0 + t1, sy = t2 + t3, sz = t4 + t5;     /* float32 */
        float a0 = t0 * sx, a1 = t1 * sx, a2 = t2 * sy;      /* float32 */
        float a3 = t3 * sy, a4 = t4 * sz, a5 = t5 * sz;
        float px = t0 * t1, py = t2 * t3, pz = t4 * t5;
        *num = v[0] / (double)a0 + v[1] / (double)a1 + v[2] / (double)a2
             + v[3] / (double)a3 + v[4] / (double)a4 + v[5] / (double)a5;
        *den = 1.0 / (double)px + 1.0 / (double)py + 1.0 / (double)pz;
    }
}

static inline void gather6(const double *a, long i, long j, long k, long nx,
                           long ny, long nz, double v[6])
{
    v[0] = AT(a, lo_nb(i, nx), j, k);
    v[1] = AT(a, hi_nb(i, nx), j, k);
    v[2] = AT(a, i, lo_nb(j, ny), k);
    v[3] = AT(a, i, hi_nb(j, ny), k);
    v[4] = AT(a, i, j, lo_nb(k, nz));
    v[5] = AT(a, i, j, hi_nb(k, nz));
}

/* solver3d._sweep (solver3d.py:131-198): one colour of SOR, returns max|d|. */
double ig_or_sweep(double *phi, const uint8_t *fixed, const float *th, long nx,
                   long ny, long nz, double omega, int colour, int ghost_linear)
{
    const size_t N = (size_t)nx * ny * nz;
    double gmax = 0.0;
#pragma omp parallel for schedule(static) reduction(max : gmax)
    for (long i = 0; i < nx; i++) {
        double dmax = 0.0;
        for (long j = 0; j < ny; j++) {
            long k0 = (i + j + colour) & 1;
            for (long k = k0; k < nz; k += 2) {
                size_t p = ((size_t)i * ny + j) * nz + k;
                if (fixed[p]) continue;
                double v[6], num, den;
                gather6(phi, i, j, k, nx, ny, nz, v);
                stencil_num_den(v, th, N, p, ghost_linear, &num, &den);
                double old = phi[p];
                double nw = old + omega * (num / den - old);
                double d = fabs(nw - old);
                if (d > dmax) dmax = d;
                phi[p] = nw;
            }
        }
        if (dmax > gmax) gmax = dmax;
    }
    return gmax;
}

/* multigrid3d._residual (multigrid3d.py:305-354): out = num - den*phi, 0 at
 * fixed nodes. */
void ig_or_residual(const double *phi, const uint8_t *fixed, const float *th,
                    long nx, long ny, long nz, int ghost_linear, double *out)
{
    const size_t N = (size_t)nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < nx; i++)
        for (long j = 0; j < ny; j++)
            for (long k = 0; k < nz; k++) {
                size_t p = ((size_t)i * ny + j) * nz + k;
                if (fixed[p]) { out[p] = 0.0; continue; }
                double v[6], num, den;
                gather6(phi, i, j, k, nx, ny, nz, v);
                stencil_num_den(v, th, N, p, ghost_linear, &num, &den);
                out[p] = num - den * phi[p];
            }
}

/* multigrid3d._sweep_rhs (multigrid3d.py:357-391): SOR on
 * sum(nbr) - 6e = f, returns max|d|. */
double ig_or_sweep_rhs(double *e, const uint8_t *fixed, const double *f,
                       long nx, long ny, long nz, double omega, int colour)
{
    double gmax = 0.0;
#pragma omp parallel for schedule(static) reduction(max : gmax)
    for (long i = 0; i < nx; i++) {
        double dmax = 0.0;
        for (long j = 0; j < ny; j++) {
            long k0 = (i + j + colour) & 1;
            for (long k = k0; k < nz; k += 2) {
                size_t p = ((size_t)i * ny + j) * nz + k;
                if (fixed[p]) continue;
                double v[6];
                gather6(e, i, j, k, nx, ny, nz, v);
                double nv = (v[0] + v[1] + v[2] + v[3] + v[4] + v[5] - f[p]) / 6.0;
                double old = e[p];
                double nw = old + omega * (nv - old);
                double d = fabs(nw - old);
                if (d > dmax) dmax = d;
                e[p] = nw;
            }
        }
        if (dmax > gmax) gmax = dmax;
    }
    return gmax;
}

/* multigrid3d._residual_rhs (multigrid3d.py:394-417). */
void ig_or_residual_rhs(const double *e, const uint8_t *fixed, const double *f,
                        long nx, long ny, long nz, double *out)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < nx; i++)
        for (long j = 0; j < ny; j++)
            for (long k = 0; k < nz; k++) {
                size_t p = ((size_t)i * ny + j) * nz + k;
                if (fixed[p]) { out[p] = 0.0; continue; }
                double v[6];
                gather6(e, i, j, k, nx, ny, nz, v);
                out[p] = (v[0] + v[1] + v[2] + v[3] + v[4] + v[5] - 6.0 * e[p]) - f[p];
            }
}

/* multigrid3d._restrict_fw_njit (multigrid3d.py:420-455): 27-point full
 * weighting with clamped edges, divided by 8 (the caller scales by 4). */
void ig_or_restrict_fw(const double *fine, long nx, long ny, long nz,
                       double *out, long cx, long cy, long cz)
{
#pragma omp parallel for schedule(static)
    for (long ic = 0; ic < cx; ic++)
        for (long jc = 0; jc < cy; jc++)
            for (long kc = 0; kc < cz; kc++) {
                long i = 2 * ic, j = 2 * jc, k = 2 * kc;
                double acc = 0.0;
                for (long di = -1; di <= 1; di++) {
                    long ii = i + di;
                    if (ii < 0) ii = 0;
                    if (ii > nx - 1) ii = nx - 1;
                    double wi = di == 0 ? 1.0 : 0.5;
                    for (long dj = -1; dj <= 1; dj++) {
                        long jj = j + dj;
                        if (jj < 0) jj = 0;
                        if (jj > ny - 1) jj = ny - 1;
                        double wj = dj == 0 ? 1.0 : 0.5;
                        for (long dk = -1; dk <= 1; dk++) {
                            long kk = k + dk;
                            if (kk < 0) kk = 0;
                            if (kk > nz - 1) kk = nz - 1;
                            double wk = dk == 0 ? 1.0 : 0.5;
                            acc += wi * wj * wk * AT(fine, ii, jj, kk);
                        }
                    }
                }
                out[((size_t)ic * cy + jc) * cz + kc] = acc / 8.0;
            }
}

/* coordinate split of the V-cycle prolongation (multigrid3d.py:465-481):
 * fine i sits at i/2 in coarse units, clamped, and the low node is kept one
 * below the top so the weight can reach 1 at the high edge. */
static inline void pa_axis(long i, long c, long *a0, long *a1, double *t)
{
    double xf = (double)i * 0.5;
    if (xf > (double)(c - 1)) xf = (double)c - 1.0;
    long x0 = (long)xf;
    if (x0 > c - 2) x0 = c > 1 ? c - 2 : 0;
    *a1 = c > 1 ? x0 + 1 : x0;
    *a0 = x0;
    *t = xf - (double)x0;
}

/* multigrid3d._prolong_add_njit (multigrid3d.py:458-499): trilinear
 * coarse -> fine, added into out, skipping fixed nodes. */
void ig_or_prolong_add(const double *coarse, long cx, long cy, long cz,
                       double *out, const uint8_t *fixed, long nx, long ny,
                       long nz)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < nx; i++) {
        long x0, x1;
        double tx;
        pa_axis(i, cx, &x0, &x1, &tx);
        for (long j = 0; j < ny; j++) {
            long y0, y1;
            double ty;
            pa_axis(j, cy, &y0, &y1, &ty);
            for (long k = 0; k < nz; k++) {
                size_t p = ((size_t)i * ny + j) * nz + k;
                if (fixed[p]) continue;
                long z0, z1;
                double tz;
                pa_axis(k, cz, &z0, &z1, &tz);
#define C(a, b, c_) coarse[((size_t)(a) * cy + (b)) * cz + (c_)]
                double c00 = C(x0, y0, z0) * (1 - tx) + C(x1, y0, z0) * tx;
                double c10 = C(x0, y1, z0) * (1 - tx) + C(x1, y1, z0) * tx;
                double c01 = C(x0, y0, z1) * (1 - tx) + C(x1, y0, z1) * tx;
                double c11 = C(x0, y1, z1) * (1 - tx) + C(x1, y1, z1) * tx;
#undef C
                double c0 = c00 * (1 - ty) + c10 * ty;
                double c1 = c01 * (1 - ty) + c11 * ty;
                out[p] += c0 * (1 - tz) + c1 * tz;
            }
        }
    }
}

/* multigrid3d._prolongate (multigrid3d.py:138-171): cascadic trilinear
 * interpolation; the fine coordinate is clamped to the last coarse node and
 * the upper index is clamped, so the weight is 0 at the high edge. */
static inline void pl_axis(long i, long c, long *a0, long *a1, double *t)
{
    double xf = (double)i / 2.0;
    if (xf > (double)(c - 1)) xf = (double)(c - 1);
    long x0 = (long)floor(xf);
    long x1 = x0 + 1 < c - 1 ? x0 + 1 : c - 1;
    *a0 = x0;
    *a1 = x1;
    *t = xf - (double)x0;
}

void ig_or_prolongate(const double *coarse, long cx, long cy, long cz,
                      double *out, long nx, long ny, long nz)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < nx; i++) {
        long x0, x1;
        double tx;
        pl_axis(i, cx, &x0, &x1, &tx);
        for (long j = 0; j < ny; j++) {
            long y0, y1;
            double ty;
            pl_axis(j, cy, &y0, &y1, &ty);
            for (long k = 0; k < nz; k++) {
                long z0, z1;
                double tz;
                pl_axis(k, cz, &z0, &z1, &tz);
#define C(a, b, c_) coarse[((size_t)(a) * cy + (b)) * cz + (c_)]
                double c00 = C(x0, y0, z0) * (1 - tx) + C(x1, y0, z0) * tx;
                double c10 = C(x0, y1, z0) * (1 - tx) + C(x1, y1, z0) * tx;
                double c01 = C(x0, y0, z1) * (1 - tx) + C(x1, y0, z1) * tx;
                double c11 = C(x0, y1, z1) * (1 - tx) + C(x1, y1, z1) * tx;
#undef C
                double c0 = c00 * (1 - ty) + c10 * ty;
                double c1 = c01 * (1 - ty) + c11 * ty;
                out[((size_t)i * ny + j) * nz + k] = c0 * (1 - tz) + c1 * tz;
            }
        }
    }
}

/* multigrid3d._coarsen_fixed_any (multigrid3d.py:507-526): a coarse node
 * is fixed when any node of its 2x2x2 fine block (low corner 2c) is. */
void ig_or_coarsen_fixed_any(const uint8_t *fixed, long nx, long ny, long nz,
                             uint8_t *out, long cx, long cy, long cz)
{
#pragma omp parallel for schedule(static)
    for (long ic = 0; ic < cx; ic++)
        for (long jc = 0; jc < cy; jc++)
            for (long kc = 0; kc < cz; kc++) {
                uint8_t any = 0;
                for (long a = 0; a < 2; a++)
                    for (long b = 0; b < 2; b++)
                        for (long c = 0; c < 2; c++) {
                            long i = 2 * ic + a, j = 2 * jc + b, k = 2 * kc + c;
                            if (i < nx && j < ny && k < nz && AT(fixed, i, j, k)) any = 1;
                        }
                out[((size_t)ic * cy + jc) * cz + kc] = any;
            }
}

/* multigrid3d._coarsen_mask (multigrid3d.py:85-135): injection at even
 * fine indices; a vacuum injection point whose 2x2x2 block holds fixed
 * nodes becomes fixed with the value of the block's largest-|val| fixed
 * node (first in (di, dj, dk) order on a tie). */
void ig_or_coarsen_mask(const uint8_t *fixed, const double *val, long nx,
                        long ny, long nz, uint8_t *fc, double *vc, long cx,
                        long cy, long cz)
{
#pragma omp parallel for schedule(static)
    for (long ic = 0; ic < cx; ic++)
        for (long jc = 0; jc < cy; jc++)
            for (long kc = 0; kc < cz; kc++) {
                size_t q = ((size_t)ic * cy + jc) * cz + kc;
                long i0 = 2 * ic, j0 = 2 * jc, k0 = 2 * kc;
                if (AT(fixed, i0, j0, k0)) {
                    fc[q] = 1;
                    vc[q] = AT(val, i0, j0, k0);
                    continue;
                }
                double best = -1.0, bv = 0.0;
                int any = 0;
                for (long a = 0; a < 2; a++)
                    for (long b = 0; b < 2; b++)
                        for (long c = 0; c < 2; c++) {
                            long i = i0 + a, j = j0 + b, k = k0 + c;
                            if (i >= nx || j >= ny || k >= nz) continue;
                            if (!AT(fixed, i, j, k)) continue;
                            double v = AT(val, i, j, k);
                            double m = fabs(v);
                            any = 1;
                            if (m > best) { best = m; bv = v; }
                        }
                fc[q] = (uint8_t)any;
                vc[q] = any ? bv : AT(val, i0, j0, k0);
            }
}

/* solver3d._residual_kernel (solver3d.py:366-386): audit residual
 * num/den - u (ghost_linear weights; every axis must be >= 2). */
void ig_or_residual_audit(const double *u, const uint8_t *fixed,
                          const float *th, long nx, long ny, long nz,
                          double *out)
{
    const size_t N = (size_t)nx * ny * nz;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < nx; i++)
        for (long j = 0; j < ny; j++)
            for (long k = 0; k < nz; k++) {
                size_t p = ((size_t)i * ny + j) * nz + k;
                if (fixed[p]) { out[p] = 0.0; continue; }
                double v[6], num, den;
                gather6(u, i, j, k, nx, ny, nz, v);
                stencil_num_den(v, th, N, p, 1, &num, &den);
                out[p] = num / den - u[p];
            }
}

/* solver3d._err_sweep (solver3d.py:389-417): SOR on the error equation
 * with a right-hand side, ghost_linear weights. */
double ig_or_err_sweep(double *e, const uint8_t *fixed, const float *th,
                       const double *rhs, long nx, long ny, long nz,
                       double omega, int colour)
{
    const size_t N = (size_t)nx * ny * nz;
    double gmax = 0.0;
#pragma omp parallel for schedule(static) reduction(max : gmax)
    for (long i = 0; i < nx; i++) {
        double dmax = 0.0;
        for (long j = 0; j < ny; j++) {
            long k0 = (i + j + colour) & 1;
            for (long k = k0; k < nz; k += 2) {
                size_t p = ((size_t)i * ny + j) * nz + k;
                if (fixed[p]) continue;
                double v[6], num, den;
                gather6(e, i, j, k, nx, ny, nz, v);
                stencil_num_den(v, th, N, p, 1, &num, &den);
                double old = e[p];
                double nw = old + omega * ((num / den + rhs[p]) - old);
                double d = fabs(nw - old);
                if (d > dmax) dmax = d;
                e[p] = nw;
            }
        }
        if (dmax > gmax) gmax = dmax;
    }
    return gmax;
}
