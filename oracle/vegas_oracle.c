/*
 * vegas_oracle.c -- CPU restatement of the vegas+ hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA kernels in
 * vegas_gb300/csrc: it is compiled into oracle/_build/libvegas_oracle.so and
 * loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline
 * and reference arm.  The product library never links or calls it.
 *
 * Every function restates the arithmetic of the reference module
 * src/vegas/_vegas.pyx (vegas 6.4.1; "pyx" below) in the same order of
 * floating-point operations, so that in FP64 it reproduces the reference
 * bit for bit where the reference is sequential.  It is compiled with
 * -ffp-contract=off so that x86 and Arm hosts round identically.
 *
 * Multi-threaded drivers (vo_iterate) split the hypercubes into contiguous
 * ranges per thread; partial sums are combined in thread order, so results
 * are deterministic for a given thread count.
 */
#include <complex.h>
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define VO_TINY 1e-257      /* pyx:34  10**(min_10_exp + 50) */
#define VO_EPSILON (DBL_EPSILON * 1e4) /* pyx:36 */

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11 "Parallel random numbers:
 * as easy as 1, 2, 3").  The CUDA kernels use the same counter layout.      */
/* ------------------------------------------------------------------------ */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void vo_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
        uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n1 = lo1;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        uint32_t n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += PHILOX_W0; k1 += PHILOX_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Uniform in [0,1) with 53 random bits for sample i, axis d of iteration itn
 * of integral `stream`.  Counter = (i_lo, i_hi, itn, stream<<8 | 0x80 | d>>1);
 * axis d takes words 2(d&1), 2(d&1)+1.  Identical to the device generator.  */
double vo_uniform_f64(uint64_t seed, uint32_t stream, uint32_t itn, uint64_t i, int d)
{
    uint32_t ctr[4] = {(uint32_t)i, (uint32_t)(i >> 32), itn,
                       (stream << 8) | 0x80u | (uint32_t)(d >> 1)};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    vo_philox4x32_10(ctr, key, o);
    uint32_t hi = o[2 * (d & 1)], lo = o[2 * (d & 1) + 1];
    uint64_t m = ((uint64_t)hi << 21) | (uint64_t)(lo >> 11);
    return (double)m * (1.0 / 9007199254740992.0);
}

/* FP32-mode uniform: 24 random bits, [0,1); counter word 3 = stream<<8 | d>>2. */
float vo_uniform_f32(uint64_t seed, uint32_t stream, uint32_t itn, uint64_t i, int d)
{
    uint32_t ctr[4] = {(uint32_t)i, (uint32_t)(i >> 32), itn, (stream << 8) | (uint32_t)(d >> 2)};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    vo_philox4x32_10(ctr, key, o);
    return (float)(o[d & 3] >> 8) * (1.0f / 16777216.0f);
}

/* Strata per axis, Integrator.set pyx:1348: ``abs(b) ** (1./dim)``.  Cython
 * compiles this double ** double as a C99 complex power (cpow), whose
 * rounding differs from pow(): e.g. b=125000, dim=1 gives 124999.99...  The
 * real part is returned; the caller truncates it with int().               */
double vo_strata_pow(double base, int dim)
{
    double complex z = cpow(CMPLX(fabs(base), 0.0), CMPLX(1. / (double)dim, 0.0));
    return creal(z);
}

/* ------------------------------------------------------------------------ */
/* AdaptiveMap                                                              */
/* ------------------------------------------------------------------------ */

/* AdaptiveMap.make_uniform, pyx:205-241 (numpy.linspace: i*step + start,
 * last node = stop).  grid rows have stride ldg, inc rows stride ldi.      */
void vo_make_uniform(int dim, const double *xl, const double *xu, const int64_t *ninc,
                     double *grid, int64_t ldg, double *inc, int64_t ldi)
{
    for (int d = 0; d < dim; d++) {
        int64_t n = ninc[d];
        double step = (xu[d] - xl[d]) / (double)n;
        for (int64_t i = 0; i < n; i++)
            grid[d * ldg + i] = (double)i * step + xl[d];
        grid[d * ldg + n] = xu[d];
        for (int64_t i = 0; i < n; i++)
            inc[d * ldi + i] = grid[d * ldg + i + 1] - grid[d * ldg + i];
    }
}

/* AdaptiveMap.map, pyx:310-360: y[n,dim] -> x[n,dim], jac[n]. */
void vo_map(int dim, const int64_t *ninc, const double *grid, int64_t ldg, const double *inc,
            int64_t ldi, int64_t n, const double *y, double *x, double *jac)
{
    for (int64_t i = 0; i < n; i++) {
        double j = 1.0;
        for (int d = 0; d < dim; d++) {
            int64_t K = ninc[d];
            double y_ninc = y[i * dim + d] * (double)K;
            int64_t iy = (int64_t)floor(y_ninc);
            double dy_ninc = y_ninc - (double)iy;
            if (iy < K) {
                x[i * dim + d] = grid[d * ldg + iy] + inc[d * ldi + iy] * dy_ninc;
                j *= inc[d * ldi + iy] * (double)K;
            } else {
                x[i * dim + d] = grid[d * ldg + K];
                j *= inc[d * ldi + K - 1] * (double)K;
            }
        }
        jac[i] = j;
    }
}

/* AdaptiveMap.invmap, pyx:362-413: iy = searchsorted(grid[d], x, 'right');
 * y = (iy-1 + (x - grid[iy-1]) / inc[iy-1]) / ninc inside, 0 below, 1 above;
 * jac *= inc * ninc.                                                       */
void vo_invmap(int dim, const int64_t *ninc, const double *grid, int64_t ldg, const double *inc,
               int64_t ldi, int64_t n, const double *x, double *y, double *jac)
{
    for (int64_t i = 0; i < n; i++) jac[i] = 1.;
    for (int d = 0; d < dim; d++) {
        int64_t K = ninc[d];
        const double *gd = grid + d * ldg;
        for (int64_t i = 0; i < n; i++) {
            double xv = x[i * dim + d];
            int64_t lo = 0, hi = K + 1;
            while (lo < hi) {
                int64_t mid = (lo + hi) / 2;
                if (gd[mid] <= xv) lo = mid + 1;
                else hi = mid;
            }
            int64_t iy = lo;
            if (iy > 0 && iy <= K) {
                int64_t iyi = iy - 1;
                y[i * dim + d] = ((double)iyi + (xv - gd[iyi]) / inc[d * ldi + iyi]) / (double)K;
                jac[i] *= inc[d * ldi + iyi] * (double)K;
            } else if (iy <= 0) {
                y[i * dim + d] = 0.;
                jac[i] *= inc[d * ldi] * (double)K;
            } else {
                y[i * dim + d] = 1.0;
                jac[i] *= inc[d * ldi + K - 1] * (double)K;
            }
        }
    }
}

/* AdaptiveMap.add_training_data, pyx:421-464.  sum_f/n_f [dim, ldi] must be
 * initialised by the caller (0 and TINY, pyx:450-452).                      */
void vo_add_training_data(int dim, const int64_t *ninc, int64_t ldi, int64_t n, const double *y,
                          const double *f, double *sum_f, double *n_f)
{
    for (int d = 0; d < dim; d++) {
        int64_t K = ninc[d];
        for (int64_t i = 0; i < n; i++) {
            double yi = y[i * dim + d];
            if (yi > 0 && yi < 1) {
                int64_t iy = (int64_t)floor(yi * (double)K);
                sum_f[d * ldi + iy] += fabs(f[i]);
                n_f[d * ldi + iy] += 1;
            }
        }
    }
}

/* AdaptiveMap.adapt, pyx:467-594.  sum_f == NULL means "no training data".
 * avg_f is ONE buffer of length max(old_ninc) shared by all axes, exactly
 * as at pyx:533 (values carry over between axes when an axis does not
 * overwrite them).  Writes new grid/inc with strides ldg_new/ldi_new.      */
void vo_adapt(int dim, const int64_t *old_ninc, const double *grid, int64_t ldg, const double *inc,
              int64_t ldi, const double *sum_f, const double *n_f, double alpha,
              const int64_t *new_ninc, double *new_grid, int64_t ldg_new, double *new_inc,
              int64_t ldi_new)
{
    int64_t max_new = 0, max_old = 0;
    for (int d = 0; d < dim; d++) {
        if (new_ninc[d] > max_new) max_new = new_ninc[d];
        if (old_ninc[d] > max_old) max_old = old_ninc[d];
    }
    if (max_new == 1) { /* pyx:514-525 */
        for (int d = 0; d < dim; d++) {
            new_grid[d * ldg_new + 0] = grid[d * ldg + 0];
            new_grid[d * ldg_new + 1] = grid[d * ldg + old_ninc[d]];
            new_inc[d * ldi_new] = new_grid[d * ldg_new + 1] - new_grid[d * ldg_new];
        }
        return;
    }
    double *avg_f = (double *)malloc(sizeof(double) * (size_t)(max_old > 0 ? max_old : 1));
    double *tmp_f = (double *)malloc(sizeof(double) * (size_t)(max_old > 0 ? max_old : 1));
    for (int64_t i = 0; i < max_old; i++) avg_f[i] = 1.0;
    for (int d = 0; d < dim; d++) {
        int64_t K = old_ninc[d];
        if (alpha != 0 && K > 1) {
            if (sum_f != NULL) {
                for (int64_t i = 0; i < K; i++) {
                    if (n_f[d * ldi + i] > 0) avg_f[i] = sum_f[d * ldi + i] / n_f[d * ldi + i];
                    else avg_f[i] = 0.;
                }
            }
            if (alpha > 0) {
                double s;
                tmp_f[0] = fabs(7. * avg_f[0] + avg_f[1]) / 8.;
                tmp_f[K - 1] = fabs(7. * avg_f[K - 1] + avg_f[K - 2]) / 8.;
                s = tmp_f[0] + tmp_f[K - 1];
                for (int64_t i = 1; i < K - 1; i++) {
                    tmp_f[i] = fabs(6. * avg_f[i] + avg_f[i - 1] + avg_f[i + 1]) / 8.;
                    s += tmp_f[i];
                }
                if (s > 0) {
                    for (int64_t i = 0; i < K; i++) avg_f[i] = tmp_f[i] / s + VO_TINY;
                } else {
                    for (int64_t i = 0; i < K; i++) avg_f[i] = VO_TINY;
                }
                for (int64_t i = 0; i < K; i++) {
                    if (avg_f[i] > 0 && avg_f[i] <= 0.99999999)
                        avg_f[i] = pow(-(1 - avg_f[i]) / log(avg_f[i]), alpha);
                }
            }
        }
        /* regrid, pyx:563-587 */
        int64_t Kn = new_ninc[d];
        new_grid[d * ldg_new + 0] = grid[d * ldg + 0];
        new_grid[d * ldg_new + Kn] = grid[d * ldg + K];
        int64_t j = -1;
        double acc_f = 0, f_ninc = 0.;
        for (int64_t i = 0; i < K; i++) f_ninc += avg_f[i];
        f_ninc /= (double)Kn;
        for (int64_t i = 1; i < Kn; i++) {
            int out = 0;
            while (acc_f < f_ninc) {
                j += 1;
                if (j < K) acc_f += avg_f[j];
                else { out = 1; break; }
            }
            if (out) break;
            acc_f -= f_ninc;
            new_grid[d * ldg_new + i] = grid[d * ldg + j + 1] - (acc_f / avg_f[j]) * inc[d * ldi + j];
        }
        for (int64_t i = 0; i < Kn; i++)
            new_inc[d * ldi_new + i] = new_grid[d * ldg_new + i + 1] - new_grid[d * ldg_new + i];
    }
    free(avg_f);
    free(tmp_f);
}

/* ------------------------------------------------------------------------ */
/* Integrator                                                               */
/* ------------------------------------------------------------------------ */

/* Integrator._random_batch allocation, pyx:1692-1706 (all batches of one
 * iteration concatenated).  Returns total evaluations; range[0..1] as the
 * reference's neval_hcube_range (note the `elif`, pyx:1701-1704).          */
int64_t vo_alloc(int64_t H, const double *sigf, double neval_sigf, int adaptive,
                 int64_t min_neval_hcube, int64_t max_neval_hcube, int64_t avg_neval_hcube,
                 int64_t *neval_h, int64_t *range)
{
    int64_t tot = 0;
    range[0] = min_neval_hcube;
    range[1] = min_neval_hcube;
    if (max_neval_hcube < min_neval_hcube) max_neval_hcube = min_neval_hcube;
    for (int64_t h = 0; h < H; h++) {
        int64_t n;
        if (adaptive) {
            n = (int64_t)(sigf[h] * neval_sigf) + min_neval_hcube;
            if (n > max_neval_hcube) n = max_neval_hcube;
            if (n < range[0]) range[0] = n;
            else if (n > range[1]) range[1] = n;
        } else {
            n = avg_neval_hcube;
        }
        neval_h[h] = n;
        tot += n;
    }
    return tot;
}

/* Mixed-radix hypercube decode, axis 0 fastest (pyx:1736-1738). */
static inline void vo_hcube_y0(int dim, const int64_t *nstrat, int64_t h, int64_t *y0)
{
    for (int d = 0; d < dim; d++) {
        y0[d] = h % nstrat[d];
        h = (h - y0[d]) / nstrat[d];
    }
}

/* Integrator._random_batch points, pyx:1731-1752, for hypercubes [h0,h1),
 * samples starting at global index i0.  u==NULL draws Philox FP64 uniforms
 * (seed, stream, itn); otherwise u[n,dim] (global sample order) is used.
 * Outputs (any may be NULL except y/x/jac scratch): y, x, wgt, hcube.       */
static void vo_points_range(int dim, const int64_t *nstrat, const int64_t *ninc, const double *grid,
                            int64_t ldg, const double *inc, int64_t ldi, int64_t H,
                            const int64_t *neval_h, int64_t h0, int64_t h1, int64_t i0,
                            const double *u, uint64_t seed, uint32_t stream, uint32_t itn,
                            double *y, double *x, double *wgt, int64_t *hcube)
{
    int64_t y0[64];
    double dv_y = 1. / (double)H;
    int64_t i = i0;
    for (int64_t h = h0; h < h1; h++) {
        vo_hcube_y0(dim, nstrat, h, y0);
        int64_t n = neval_h[h];
        for (int64_t k = 0; k < n; k++, i++) {
            for (int d = 0; d < dim; d++) {
                double ud = u ? u[i * dim + d] : vo_uniform_f64(seed, stream, itn, (uint64_t)i, d);
                y[i * dim + d] = ((double)y0[d] + ud) / (double)nstrat[d];
            }
        }
        /* map + weight (pyx:1743, 1748-1749) */
        vo_map(dim, ninc, grid, ldg, inc, ldi, n, y + (i - n) * dim, x + (i - n) * dim, wgt + (i - n));
        for (int64_t k = i - n; k < i; k++) {
            wgt[k] *= dv_y / (double)n;
            if (hcube) hcube[k] = h;
        }
    }
}

void vo_points(int dim, const int64_t *nstrat, const int64_t *ninc, const double *grid, int64_t ldg,
               const double *inc, int64_t ldi, int64_t H, const int64_t *neval_h, const double *u,
               uint64_t seed, uint32_t stream, uint32_t itn, double *y, double *x, double *wgt,
               int64_t *hcube)
{
    vo_points_range(dim, nstrat, ninc, grid, ldg, inc, ldi, H, neval_h, 0, H, 0, u, seed, stream,
                    itn, y, x, wgt, hcube);
}

/* Per-hypercube two-pass reduction, pyx:2136-2193, for hypercubes [h0,h1)
 * whose samples start at i0.  fx is [n, s] row-major.  mean[s] and
 * var[s*s] (lower triangle, correlate_integrals=True form) are ACCUMULATED.
 * sigf/sum_sigf updated when adaptive.  fdv2[i] written when non-NULL.
 * hc_var[h - h0] = sigf2 = |variance of component 0| (pyx:2181, the
 * adapt_to_errors training value) when non-NULL.                          */
static void vo_reduce_range(int64_t h0, int64_t h1, int64_t i0, const int64_t *neval_h, int s,
                            const double *wgt, const double *fx, int adaptive, double beta,
                            double *mean, double *var, double *sigf, double *sum_sigf, double *fdv2,
                            double *hc_var)
{
    double sum_wf[16], sum_dwf[16], sum_dwf2[256], dwf[16];
    int64_t j = i0;
    for (int64_t h = h0; h < h1; h++) {
        int64_t n = neval_h[h];
        for (int a = 0; a < s; a++) { sum_wf[a] = 0.0; sum_dwf[a] = 0.0; }
        for (int a = 0; a < s * s; a++) sum_dwf2[a] = 0.0;
        for (int64_t k = j; k < j + n; k++)
            for (int a = 0; a < s; a++) sum_wf[a] += wgt[k] * fx[k * s + a];
        for (int64_t k = j; k < j + n; k++) {
            for (int a = 0; a < s; a++) {
                dwf[a] = wgt[k] * fx[k * s + a] - sum_wf[a] / (double)n;
                if (fabs(dwf[a]) < VO_EPSILON * fabs(sum_wf[a] / (double)n)) {
                    dwf[a] = VO_EPSILON * fabs(sum_wf[a] / (double)n);
                    sum_dwf2[a * s + a] += dwf[a] * dwf[a];
                    dwf[a] = 0.;
                } else {
                    sum_dwf2[a * s + a] += dwf[a] * dwf[a];
                }
                sum_dwf[a] += dwf[a];
                for (int b = 0; b < a; b++) sum_dwf2[a * s + b] += dwf[a] * dwf[b];
            }
            if (fdv2) {
                double t = wgt[k] * fx[k * s] * (double)n;
                fdv2[k] = t * t;
            }
        }
        for (int a = 0; a < s; a++) {
            mean[a] += sum_wf[a] + sum_dwf[a];
            for (int b = 0; b <= a; b++)
                var[a * s + b] += ((double)n * sum_dwf2[a * s + b] - sum_dwf[a] * sum_dwf[b]) / ((double)n - 1.);
        }
        double sigf2 = fabs(((double)n * sum_dwf2[0] - sum_dwf[0] * sum_dwf[0]) / ((double)n - 1.));
        if (hc_var) hc_var[h - h0] = sigf2;
        if (adaptive) {
            sigf[h] = pow(sigf2, beta / 2.);
            *sum_sigf += sigf[h];
        }
        j += n;
    }
}

void vo_reduce(int64_t H, const int64_t *neval_h, int s, const double *wgt, const double *fx,
               int adaptive, double beta, double *mean, double *var, double *sigf,
               double *sum_sigf, double *fdv2, double *hc_var)
{
    vo_reduce_range(0, H, 0, neval_h, s, wgt, fx, adaptive, beta, mean, var, sigf, sum_sigf, fdv2,
                    hc_var);
}

/* ------------------------------------------------------------------------ */
/* Built-in integrands (FP64), the synthetic workloads of the benchmarks.   */
/* ------------------------------------------------------------------------ */
enum {
    VO_F_GAUSS = 0,     /* p = {a, c, norm}: norm*exp(-a*sum_d (x_d-c)^2)              */
    VO_F_RIDGE = 1,     /* p = {M, s}: (1/M) sum_j N_dim(x; c_j*1, s), c_j=(j+.5)/M       */
    VO_F_LORENTZ = 2,   /* p = {c[dim], w[dim]}: prod_d (w/pi)/((x-c)^2+w^2)             */
    VO_F_MIXTURE = 3,   /* p = {K, sigma, c[K*dim]}: (1/K) sum_k N_dim(x; c_k, sigma)      */
    VO_F_LATTICE = 4,   /* p = {a, lambda}: exp(-S), periodic chain action                */
    VO_F_CONST = 5,     /* p = {value}                                                   */
};

static double vo_eval1(int kind, const double *p, int dim, const double *x)
{
    const double PI = 3.14159265358979323846;
    switch (kind) {
    case VO_F_GAUSS: {
        double s = 0.0;
        for (int d = 0; d < dim; d++) s += (x[d] - p[1]) * (x[d] - p[1]);
        return p[2] * exp(-p[0] * s);
    }
    case VO_F_RIDGE: {
        int M = (int)p[0];
        double sg = p[1];
        double norm = pow(2 * PI * sg * sg, -0.5 * dim);
        double acc = 0.0;
        for (int j = 0; j < M; j++) {
            double c = (j + 0.5) / M, r2 = 0.0;
            for (int d = 0; d < dim; d++) r2 += (x[d] - c) * (x[d] - c);
            acc += exp(-r2 / (2 * sg * sg));
        }
        return norm * acc / M;
    }
    case VO_F_LORENTZ: {
        double f = 1.0;
        for (int d = 0; d < dim; d++) {
            double c = p[d], w = p[dim + d], dx = x[d] - c;
            f *= (w / PI) / (dx * dx + w * w);
        }
        return f;
    }
    case VO_F_MIXTURE: {
        int K = (int)p[0];
        double sg = p[1];
        double norm = pow(2 * PI * sg * sg, -0.5 * dim);
        double acc = 0.0;
        for (int k = 0; k < K; k++) {
            double r2 = 0.0;
            for (int d = 0; d < dim; d++) {
                double dx = x[d] - p[2 + k * dim + d];
                r2 += dx * dx;
            }
            acc += exp(-r2 / (2 * sg * sg));
        }
        return norm * acc / K;
    }
    case VO_F_LATTICE: {
        double a = p[0], lam = p[1], S = 0.0;
        for (int i = 0; i < dim; i++) {
            double xi = x[i], xn = x[(i + 1) % dim], dx = xn - xi;
            S += dx * dx / (2 * a) + a * (xi * xi / 2 + lam * xi * xi * xi * xi);
        }
        return exp(-S);
    }
    case VO_F_CONST:
        return p[0];
    }
    return NAN;
}

void vo_eval(int kind, const double *p, int dim, int64_t n, const double *x, double *f)
{
    for (int64_t i = 0; i < n; i++) f[i] = vo_eval1(kind, p, dim, x + i * dim);
}

/* ------------------------------------------------------------------------ */
/* One full vegas+ iteration for a built-in integrand (pyx:2086-2217),     */
/* multi-threaded over hypercube ranges.  State is updated in place:       */
/*   sigf[H], *sum_sigf, and (when alpha>0 && adapt) grid/inc via adapt.   */
/* out[0]=mean, out[1]=var, out[2]=last_neval, out[3]=range lo, out[4]=hi. */
/* ------------------------------------------------------------------------ */
typedef struct {
    int dim, kind, adaptive, train, train_hc;
    const double *p;
    const int64_t *nstrat, *ninc;
    const double *grid, *inc;
    int64_t ldg, ldi, H;
    const int64_t *neval_h, *offs;
    int64_t h0, h1;
    uint64_t seed;
    uint32_t stream, itn;
    double beta;
    double *sigf;
    double mean, var, sum_sigf;
    double *sum_f, *n_f; /* per-thread histograms [dim, ldi] */
    int64_t chunk;
} vo_job;

static void *vo_job_run(void *arg)
{
    vo_job *J = (vo_job *)arg;
    int dim = J->dim;
    int64_t maxn = 0;
    for (int64_t h = J->h0; h < J->h1; h++)
        if (J->neval_h[h] > maxn) maxn = J->neval_h[h];
    /* process in chunks of whole hypercubes to bound scratch memory */
    int64_t cap = J->chunk > maxn ? J->chunk : maxn;
    double *y = (double *)malloc(sizeof(double) * (size_t)(cap * dim));
    double *x = (double *)malloc(sizeof(double) * (size_t)(cap * dim));
    double *w = (double *)malloc(sizeof(double) * (size_t)cap);
    double *f = (double *)malloc(sizeof(double) * (size_t)cap);
    double *fdv2 = (double *)malloc(sizeof(double) * (size_t)cap);
    double *hcv = (double *)malloc(sizeof(double) * (size_t)(J->h1 - J->h0 + 1));
    J->mean = 0.0; J->var = 0.0; J->sum_sigf = 0.0;
    int64_t h = J->h0;
    while (h < J->h1) {
        int64_t he = h, cnt = 0;
        while (he < J->h1 && cnt + J->neval_h[he] <= cap) cnt += J->neval_h[he++];
        int64_t i0 = J->offs[h];
        /* local index space: shift pointers so vo_points_range indexes from 0 */
        int64_t y0[64];
        double dv_y = 1. / (double)J->H;
        int64_t k = 0;
        for (int64_t hh = h; hh < he; hh++) {
            vo_hcube_y0(dim, J->nstrat, hh, y0);
            int64_t n = J->neval_h[hh];
            for (int64_t q = 0; q < n; q++, k++)
                for (int d = 0; d < dim; d++) {
                    double ud = vo_uniform_f64(J->seed, J->stream, J->itn, (uint64_t)(i0 + k), d);
                    y[k * dim + d] = ((double)y0[d] + ud) / (double)J->nstrat[d];
                }
            vo_map(dim, J->ninc, J->grid, J->ldg, J->inc, J->ldi, n, y + (k - n) * dim,
                   x + (k - n) * dim, w + (k - n));
            for (int64_t q = k - n; q < k; q++) w[q] *= dv_y / (double)n;
        }
        vo_eval(J->kind, J->p, dim, cnt, x, f);
        double m = 0.0, v = 0.0;
        vo_reduce_range(h, he, 0, J->neval_h, 1, w, f, J->adaptive, J->beta, &m, &v, J->sigf,
                        &J->sum_sigf, fdv2, hcv);
        J->mean += m;
        J->var += v;
        if (J->train)
            vo_add_training_data(dim, J->ninc, J->ldi, cnt, y, fdv2, J->sum_f, J->n_f);
        if (J->train_hc) {   /* adapt_to_errors: sigf2 at each hypercube's last sample, pyx:2187-2193 */
            int64_t klast = -1;
            for (int64_t hh = h; hh < he; hh++) {
                klast += J->neval_h[hh];
                vo_add_training_data(dim, J->ninc, J->ldi, 1, y + klast * dim, &hcv[hh - h], J->sum_f,
                                     J->n_f);
            }
        }
        h = he;
    }
    free(y); free(x); free(w); free(f); free(fdv2); free(hcv);
    return NULL;
}

int vo_iterate(int dim, int kind, const double *p, const int64_t *nstrat, int64_t *ninc,
               double *grid, int64_t ldg, double *inc, int64_t ldi, int64_t H, double *sigf,
               double *sum_sigf, int64_t neval, double neval_frac, int64_t min_neval_hcube,
               int64_t max_neval_hcube, double alpha, double beta, int adapt, int adapt_to_errors,
               uint64_t seed, uint32_t stream, uint32_t itn, int nthreads, double *out)
{
    /* adapt_to_errors: uniform allocation, no sigf, the map trained on each
     * hypercube's variance (pyx:1659, 1675, 2187-2196, 2209)               */
    int adaptive_alloc = (beta > 0 && H > 1 && !adapt_to_errors);
    int adaptive = adaptive_alloc && adapt;
    int train_hc = adapt_to_errors && adapt;
    int train = (adapt && alpha > 0 && !adapt_to_errors) || train_hc;
    int64_t *neval_h = (int64_t *)malloc(sizeof(int64_t) * (size_t)H);
    int64_t *offs = (int64_t *)malloc(sizeof(int64_t) * (size_t)(H + 1));
    int64_t range[2];
    double neval_sigf = (beta > 0 && *sum_sigf > 0 && !adapt_to_errors)
                            ? neval_frac * (double)neval / *sum_sigf : 0.0;
    int64_t tot = vo_alloc(H, sigf, neval_sigf, adaptive_alloc, min_neval_hcube, max_neval_hcube,
                           (int64_t)((double)neval / (double)H), neval_h, range);
    offs[0] = 0;
    for (int64_t h = 0; h < H; h++) offs[h + 1] = offs[h] + neval_h[h];
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    vo_job jobs[256];
    pthread_t th[256];
    int64_t bnd[257];
    size_t hsz = (size_t)dim * (size_t)ldi;
    /* thread t owns hypercubes [bnd[t], bnd[t+1]): equal shares of samples */
    bnd[0] = 0;
    bnd[nthreads] = H;
    for (int t = 1; t < nthreads; t++) {
        int64_t target = tot * t / nthreads, a = 0, b = H;
        while (a < b) { int64_t m = (a + b) / 2; if (offs[m] < target) a = m + 1; else b = m; }
        bnd[t] = a < bnd[t - 1] ? bnd[t - 1] : a;
    }
    for (int t = 0; t < nthreads; t++) {
        vo_job *J = &jobs[t];
        memset(J, 0, sizeof(*J));
        J->dim = dim; J->kind = kind; J->p = p; J->adaptive = adaptive;
        J->train = train && !train_hc; J->train_hc = train_hc;
        J->nstrat = nstrat; J->ninc = ninc; J->grid = grid; J->inc = inc; J->ldg = ldg; J->ldi = ldi;
        J->H = H; J->neval_h = neval_h; J->offs = offs;
        J->h0 = bnd[t];
        J->h1 = bnd[t + 1] < bnd[t] ? bnd[t] : bnd[t + 1];
        J->seed = seed; J->stream = stream; J->itn = itn; J->beta = beta; J->sigf = sigf;
        J->chunk = 65536;
        if (train) {
            J->sum_f = (double *)calloc(hsz, sizeof(double));
            J->n_f = (double *)calloc(hsz, sizeof(double));
        }
    }
    for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, vo_job_run, &jobs[t]);
    vo_job_run(&jobs[0]);
    for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
    double mean = 0.0, var = 0.0, ss = 0.0;
    for (int t = 0; t < nthreads; t++) { mean += jobs[t].mean; var += jobs[t].var; ss += jobs[t].sum_sigf; }
    out[0] = mean; out[1] = var; out[2] = (double)tot; out[3] = (double)range[0]; out[4] = (double)range[1];
    if (adaptive) {
        if (ss > 0) *sum_sigf = ss;
        else { for (int64_t h = 0; h < H; h++) sigf[h] = 1.; *sum_sigf = (double)H; }
    }
    if (train && alpha > 0) {
        double *sum_f = (double *)calloc(hsz, sizeof(double));
        double *n_f = (double *)malloc(sizeof(double) * hsz);
        for (size_t q = 0; q < hsz; q++) n_f[q] = VO_TINY;
        for (int t = 0; t < nthreads; t++) {
            for (size_t q = 0; q < hsz; q++) { sum_f[q] += jobs[t].sum_f[q]; n_f[q] += jobs[t].n_f[q]; }
            free(jobs[t].sum_f); free(jobs[t].n_f);
        }
        double *ng = (double *)malloc(sizeof(double) * (size_t)dim * (size_t)ldg);
        double *ni = (double *)malloc(sizeof(double) * hsz);
        vo_adapt(dim, ninc, grid, ldg, inc, ldi, sum_f, n_f, alpha, ninc, ng, ldg, ni, ldi);
        memcpy(grid, ng, sizeof(double) * (size_t)dim * (size_t)ldg);
        memcpy(inc, ni, sizeof(double) * hsz);
        free(ng); free(ni); free(sum_f); free(n_f);
    } else if (train) {   /* adapt_to_errors with alpha = 0: the map is not adapted */
        for (int t = 0; t < nthreads; t++) { free(jobs[t].sum_f); free(jobs[t].n_f); }
    }
    free(neval_h);
    free(offs);
    return 0;
}
