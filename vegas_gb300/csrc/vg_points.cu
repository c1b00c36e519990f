// vg_points.cu -- built-in integrands evaluated at given points, for paths
// that produce their points outside the fused tile kernel (the learned flow
// composed after the AdaptiveMap).  No reference counterpart: the reference
// calls the user's integrand on its batch of points (_vegas.pyx:2126-2129);
// this is the same call for the built-in synthetic integrands.
//
//   f[i] = vol * f(lo + width * z_i) * jac[i] * exp(-logdet[i])
// (jac and logdet optional)
//
// z is FP32 [n, dim] on the unit cube; the evaluation is FP32 as in the fused
// kernels (vg_integrands.cuh).  HBM-bound for cheap integrands: reads 4*dim
// (+4) bytes and writes 4 bytes per point.
#include <string.h>

#include "vg_integrands.cuh"

int vg_build_params(int kind, int dim, const double *params, int nparams, VgParams *Pp, int *tab_len_out);

namespace {

struct PointsArgs {
    int64_t n;
    int dim, tab_len;
    float lo[VG_MAX_DIM], width[VG_MAX_DIM];
    float vol;
    const float *z;
    const float *logdet;
    const float *jac;
    float *f;
};

template <int KIND, int DIMB>
__global__ void __launch_bounds__(256) points_kernel(PointsArgs a, VgParams P)
{
    extern __shared__ __align__(16) float tab[];
    const VgF32Consts k = vg_prepare_f32<KIND>(P, a.dim);
    vg_fill_table_f32<KIND>(P, a.dim, tab, k);
    __syncthreads();
    const int dim = a.dim;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float x[DIMB];
#pragma unroll
        for (int d = 0; d < DIMB; d++)
            x[d] = d < dim ? fmaf(a.width[d], a.z[i * dim + d], a.lo[d]) : 0.f;
        float v = a.vol * vg_eval_f32<KIND, DIMB>(k, tab, a.tab_len, dim, x);
        if (a.jac != nullptr) v *= a.jac[i];
        if (a.logdet != nullptr) v *= __expf(-a.logdet[i]);
        a.f[i] = v;
    }
}

template <int KIND>
int launch_points(const PointsArgs &a, const VgParams &P, cudaStream_t st)
{
    const size_t smem = sizeof(float) * (a.tab_len + 4);
    int grid = vg_num_sms() * 8;
    const int64_t need = (a.n + 255) / 256;
    if (need < grid) grid = (int)need;
    if (a.dim <= 4) points_kernel<KIND, 4><<<grid, 256, smem, st>>>(a, P);
    else if (a.dim <= 8) points_kernel<KIND, 8><<<grid, 256, smem, st>>>(a, P);
    else if (a.dim <= 16) points_kernel<KIND, 16><<<grid, 256, smem, st>>>(a, P);
    else points_kernel<KIND, 64><<<grid, 256, smem, st>>>(a, P);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

__global__ void weight_kernel(int64_t n, const float *__restrict__ f, const float *__restrict__ jac,
                              const float *__restrict__ logdet, float *__restrict__ out)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float v = f[i];
        if (jac != nullptr) v *= jac[i];
        if (logdet != nullptr) v *= __expf(-logdet[i]);
        out[i] = v;
    }
}

}  // namespace

// out[i] = f[i] * jac[i] * exp(-logdet[i]) for integrand values computed
// elsewhere (a torch integrand on the flow path); jac, logdet optional.
extern "C" int vg_weight_points(int64_t n, const float *f, const float *jac, const float *logdet, float *out,
                                void *stream)
{
    VG_RANGE("vg_weight_points");
    vg_clear_error();
    if (n <= 0) return VG_OK;
    int64_t nb = (n + 255) / 256;
    const int64_t cap = (int64_t)vg_num_sms() * 16;
    if (nb > cap) nb = cap;
    weight_kernel<<<(unsigned)nb, 256, 0, (cudaStream_t)stream>>>(n, f, jac, logdet, out);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

extern "C" int vg_eval_points(int kind, const double *params, int nparams, int dim, int64_t n,
                              const float *z, const double *lo, const double *width,
                              const float *logdet, const float *jac, float *f, void *stream)
{
    VG_RANGE("vg_eval_points");
    vg_clear_error();
    if (dim < 1 || dim > VG_MAX_DIM) return vg_fail(VG_ERR_VALUE, "dim %d out of range", dim);
    if (n < 0) return vg_fail(VG_ERR_VALUE, "negative point count");
    VgParams P;   // copied into the kernel arguments at launch
    int tab_len = 0, rc;
    if ((rc = vg_build_params(kind, dim, params, nparams, &P, &tab_len))) return rc;
    if (sizeof(float) * (tab_len + 4) > 48 * 1024) return vg_fail(VG_ERR_UNSUPPORTED, "integrand table too large");
    if (n == 0) return VG_OK;
    PointsArgs a;
    memset(&a, 0, sizeof(a));
    a.n = n;
    a.dim = dim;
    a.tab_len = tab_len;
    double vol = 1.0;
    for (int d = 0; d < dim; d++) {
        a.lo[d] = (float)lo[d];
        a.width[d] = (float)width[d];
        vol *= width[d];
    }
    a.vol = (float)vol;
    a.z = z;
    a.logdet = logdet;
    a.jac = jac;
    a.f = f;
    cudaStream_t st = (cudaStream_t)stream;
    switch (kind) {
    case VG_F_GAUSS: return launch_points<VG_F_GAUSS>(a, P, st);
    case VG_F_RIDGE: return launch_points<VG_F_RIDGE>(a, P, st);
    case VG_F_LORENTZ: return launch_points<VG_F_LORENTZ>(a, P, st);
    case VG_F_MIXTURE: return launch_points<VG_F_MIXTURE>(a, P, st);
    case VG_F_LATTICE: return launch_points<VG_F_LATTICE>(a, P, st);
    default: return launch_points<VG_F_CONST>(a, P, st);
    }
}
