/*
 * vg_host.c -- host-side logic of the C ABI: error reporting and the
 * stratification sizing of Integrator.set (src/vegas/_vegas.pyx:1335-1407).
 *
 * Compiled with gcc (C11) and -ffp-contract=off so that the floating-point
 * expressions that feed int() truncations round as in the reference.
 */
#include <complex.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "vg_internal.h"

static _Thread_local char vg_err_buf[512];

int vg_fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(vg_err_buf, sizeof(vg_err_buf), fmt, ap);
    va_end(ap);
    return code;
}

void vg_clear_error(void) { vg_err_buf[0] = '\0'; }

const char *vg_last_error(void) { return vg_err_buf; }

int vg_version(void) { return 100; }

size_t vg_struct_size(int which)
{
    return which == 0 ? sizeof(vg_integrator) : (which == 1 ? sizeof(vg_stats) : 0);
}

/*
 * Strata per axis.  The reference writes int(abs(b) ** (1./dim)) (pyx:1348);
 * Cython compiles that double ** double as a C99 complex power, so the value
 * is creal(cpow(b, 1/dim)) = exp(log(b)/dim), which rounds differently from
 * pow() (b=125000, dim=1 gives 124999.99...).  Reproduced exactly here.
 */
static double strata_pow(double base, int dim)
{
    double complex z = cpow(CMPLX(fabs(base), 0.0), CMPLX(1. / (double)dim, 0.0));
    return creal(z);
}

int vg_set_strata(int dim, int mode, int64_t *neval, int neval_given, const int64_t *nstrat_in,
                  double neval_frac, double beta, int adapt_to_errors, int uniform_nstrat,
                  double max_mem, int minimize_mem, int64_t maxinc_axis, int64_t *nstrat_out,
                  int64_t *ninc_out, int64_t *min_neval_hcube_out)
{
    vg_clear_error();
    if (dim < 1 || dim > VG_MAX_DIM)
        return vg_fail(VG_ERR_UNSUPPORTED, "dim = %d outside 1..%d", dim, VG_MAX_DIM);
    double nf = (beta == 0 || adapt_to_errors) ? 0.0 : neval_frac;   /* pyx:1331 */
    int64_t nstrat[VG_MAX_DIM];
    if (mode == 1) {                                                  /* pyx:1335-1345 */
        double nh = 1.0;
        for (int d = 0; d < dim; d++) {
            if (nstrat_in[d] < 1) return vg_fail(VG_ERR_VALUE, "bad nstrat");
            nstrat[d] = nstrat_in[d];
            nh *= (double)nstrat[d];
        }
        if (!neval_given) {
            *neval = (int64_t)(2. * nh / (1. - nf));
        } else if ((double)*neval < 2. * nh / (1. - nf)) {
            return vg_fail(VG_ERR_VALUE, "neval too small: %lld < %.17g", (long long)*neval,
                           2. * nh / (1. - nf));
        }
    } else if (mode == 0) {                                           /* pyx:1346-1366 */
        double base = (1 - nf) * (double)*neval / 2.;
        int64_t ns = (int64_t)strata_pow(base, dim);
        if (ns < 1) ns = 1;
        int64_t d = (int64_t)((log(base) - (double)dim * log((double)ns)) / log(1 + 1. / (double)ns));
        double cells = pow((double)(ns + 1), (double)d) * pow((double)ns, (double)(dim - d));
        if (cells > max_mem && !minimize_mem)
            return vg_fail(VG_ERR_MEMORY, "work arrays larger than max_mem; set minimize_mem=True "
                                          "(and install h5py module) or increase max_mem");
        if (uniform_nstrat) d = 0;
        if (d < 0) d = 0;
        for (int k = 0; k < dim; k++) nstrat[k] = (k < d) ? ns + 1 : ns;
    } else {
        for (int k = 0; k < dim; k++) nstrat[k] = nstrat_in[k];
    }
    /* grid increments, pyx:1369-1386 */
    if (adapt_to_errors) {
        for (int k = 0; k < dim; k++) ninc_out[k] = nstrat[k];
    } else {
        int64_t ni = (int64_t)((double)*neval / 10.);
        if (ni > maxinc_axis) ni = maxinc_axis;
        for (int k = 0; k < dim; k++) {
            if (ni >= nstrat[k]) {
                ninc_out[k] = (int64_t)((double)ni / (double)nstrat[k]) * nstrat[k];
            } else if (nstrat[k] <= maxinc_axis) {
                ninc_out[k] = nstrat[k];
            } else {
                nstrat[k] = (int64_t)((double)nstrat[k] / (double)ni) * ni;
                ninc_out[k] = ni;
            }
        }
    }
    /* min_neval_hcube, pyx:1397-1407 */
    double nhc = 1.0;
    for (int k = 0; k < dim; k++) {
        nstrat_out[k] = nstrat[k];
        nhc *= (double)nstrat[k];
    }
    int64_t mnh;
    if (nhc == 1.0) mnh = *neval;
    else mnh = (int64_t)((1 - nf) * (double)*neval / nhc);
    if (mnh < 2) mnh = 2;
    *min_neval_hcube_out = mnh;
    return VG_OK;
}
