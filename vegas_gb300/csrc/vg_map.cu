// vg_map.cu -- AdaptiveMap on the GPU: make_uniform, map, training data and
// adapt (smoothing, damping, cumulative-sum regrid).
//
// Reference: src/vegas/_vegas.pyx (vegas 6.4.1) AdaptiveMap, pyx:39-832.
// FP64 arithmetic uses explicit round-to-nearest intrinsics where the
// reference's operation order matters, so that no multiply-add is contracted.
#include <math.h>
#include <string.h>

#include "vg_common.cuh"
#include "vg_adapt.cuh"

namespace {

struct MapGeom {
    int dim;
    int ninc[VG_MAX_DIM];
};

// ------------------------------------------------------------ make_uniform
// numpy.linspace semantics (i*step + start, last node = stop), pyx:228-239.
struct Limits {
    double v[2 * VG_MAX_DIM];
};

__global__ void make_uniform_kernel(MapGeom g, Limits lim, double *grid, int64_t ldg, double *inc,
                                    int64_t ldi)
{
    int d = blockIdx.x;
    int K = g.ninc[d];
    double xl = lim.v[2 * d], xu = lim.v[2 * d + 1];
    double step = __ddiv_rn(__dsub_rn(xu, xl), (double)K);
    for (int i = threadIdx.x; i <= K; i += blockDim.x)
        grid[d * ldg + i] = (i == K) ? xu : __dadd_rn(__dmul_rn((double)i, step), xl);
    __syncthreads();
    for (int i = threadIdx.x; i < K; i += blockDim.x) {
        double a = (i == K - 1) ? xu : __dadd_rn(__dmul_rn((double)(i + 1), step), xl);
        double b = __dadd_rn(__dmul_rn((double)i, step), xl);
        inc[d * ldi + i] = __dsub_rn(a, b);
    }
}

// ------------------------------------------------------------------- map
// pyx:346-359: iy = floor(y*ninc); x = grid[iy] + inc[iy]*dy; jac *= inc*ninc;
// iy == ninc maps to grid[ninc] with inc[ninc-1].
template <typename T>
__global__ void map_kernel(MapGeom g, const double *__restrict__ grid,
                           const double *__restrict__ inc, int64_t ldg, int64_t ldi, int64_t n,
                           const T *__restrict__ y, T *__restrict__ x, T *__restrict__ jac)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int dim = g.dim;
    if (sizeof(T) == 8) {
        double j = 1.0;
        for (int d = 0; d < dim; d++) {
            int K = g.ninc[d];
            double yn = __dmul_rn((double)y[i * dim + d], (double)K);
            double fl = floor(yn);
            int64_t iy = (int64_t)fl;
            double dy = __dsub_rn(yn, (double)iy);
            if (iy < K) {
                double w = inc[d * ldi + iy];
                x[i * dim + d] = (T)__dadd_rn(grid[d * ldg + iy], __dmul_rn(w, dy));
                j = __dmul_rn(j, __dmul_rn(w, (double)K));
            } else {
                x[i * dim + d] = (T)grid[d * ldg + K];
                j = __dmul_rn(j, __dmul_rn(inc[d * ldi + K - 1], (double)K));
            }
        }
        jac[i] = (T)j;
    } else {
        float j = 1.0f;
        for (int d = 0; d < dim; d++) {
            int K = g.ninc[d];
            float yn = (float)y[i * dim + d] * (float)K;
            int iy = (int)floorf(yn);
            float dy = yn - (float)iy;
            if (iy < K) {
                float w = (float)inc[d * ldi + iy];
                x[i * dim + d] = (T)fmaf(w, dy, (float)grid[d * ldg + iy]);
                j *= w * (float)K;
            } else {
                x[i * dim + d] = (T)(float)grid[d * ldg + K];
                j *= (float)inc[d * ldi + K - 1] * (float)K;
            }
        }
        jac[i] = (T)j;
    }
}

// ------------------------------------------------------- training data
// pyx:456-463: for 0 < y < 1: sum_f[d, floor(y*ninc)] += |f|, n_f += 1.
template <typename T>
__global__ void train_kernel(MapGeom g, int64_t ldi, int64_t n, const T *__restrict__ y,
                             const T *__restrict__ f, double *sum_f, unsigned long long *n_f)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double fi = fabs((double)f[i]);
    for (int d = 0; d < g.dim; d++) {
        double yi = (double)y[i * g.dim + d];
        if (yi > 0 && yi < 1) {
            int64_t iy = (int64_t)floor(__dmul_rn(yi, (double)g.ninc[d]));
            atomicAdd(&sum_f[d * ldi + iy], fi);
            atomicAdd(&n_f[d * ldi + iy], 1ull);
        }
    }
}

// ------------------------------------------------------------------ adapt
using vgadapt::AdaptArgs;
constexpr int ADAPT_NT = 1024;

__global__ void __launch_bounds__(ADAPT_NT) adapt_kernel(AdaptArgs a)
{
    extern __shared__ double sm[];
    double *avg = sm;                 // [max_old]
    double *tmp = sm + a.max_old;     // [max_old]
    double *part = tmp + a.max_old;   // [ADAPT_NT]
    // in place (new_grid == grid): the axis' old nodes and increments staged
    double *gs = a.new_grid == a.grid ? part + ADAPT_NT : nullptr;   // [max_old + 1]
    double *is = gs != nullptr ? gs + a.max_old + 1 : nullptr;        // [max_old]
    for (int i = threadIdx.x; i < a.max_old; i += ADAPT_NT) avg[i] = 1.0;
    __syncthreads();
    if (a.sequential) {
        for (int d = 0; d < a.dim; d++) vgadapt::adapt_axis<ADAPT_NT>(a, d, avg, tmp, part, gs, is);
    } else {
        vgadapt::adapt_axis<ADAPT_NT>(a, blockIdx.x, avg, tmp, part, gs, is);
    }
}

// pyx:514-525: max(new_ninc) == 1 collapses every axis to one increment.
__global__ void adapt_single_kernel(AdaptArgs a)
{
    int d = threadIdx.x;
    if (d >= a.dim) return;
    double g0 = a.grid[d * a.ldg], g1 = a.grid[d * a.ldg + a.old_ninc[d]];
    a.new_grid[d * a.ldg_new] = g0;
    a.new_grid[d * a.ldg_new + 1] = g1;
    a.new_inc[d * a.ldi_new] = __dsub_rn(g1, g0);
}

int fill_geom(MapGeom &g, int dim, const int64_t *ninc)
{
    if (dim < 1 || dim > VG_MAX_DIM) return vg_fail(VG_ERR_UNSUPPORTED, "dim %d", dim);
    g.dim = dim;
    for (int d = 0; d < dim; d++) {
        if (ninc[d] < 1 || ninc[d] > (1 << 30)) return vg_fail(VG_ERR_VALUE, "bad ninc");
        g.ninc[d] = (int)ninc[d];
    }
    return VG_OK;
}

}  // namespace

// ======================================================================
extern "C" int vg_make_uniform(int dim, const int64_t *ninc, const double *xl, const double *xu,
                               double *grid, int64_t ldg, double *inc, int64_t ldi, void *stream)
{
    VG_RANGE("vg_make_uniform");
    vg_clear_error();
    MapGeom g;
    int rc = fill_geom(g, dim, ninc);
    if (rc) return rc;
    Limits lim;
    for (int d = 0; d < dim; d++) {
        if (ninc[d] + 1 > ldg || ninc[d] > ldi) return vg_fail(VG_ERR_VALUE, "grid too small");
        lim.v[2 * d] = xl[d];
        lim.v[2 * d + 1] = xu[d];
    }
    make_uniform_kernel<<<dim, 256, 0, (cudaStream_t)stream>>>(g, lim, grid, ldg, inc, ldi);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

namespace {
// AdaptiveMap.jac1d (pyx:265-295): dx[d]/dy[d] = inc[d][iy] * ninc[d],
// iy = floor(y ninc) (inc[ninc-1] at y = 1).
template <typename T>
__global__ void jac1d_kernel(MapGeom g, const double *__restrict__ inc, int64_t ldi, int64_t n,
                             const T *__restrict__ y, T *__restrict__ out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int d = 0; d < g.dim; d++) {
        const int K = g.ninc[d];
        int64_t iy;
        if (sizeof(T) == 8) iy = (int64_t)floor(__dmul_rn((double)y[i * g.dim + d], (double)K));
        else iy = (int64_t)floorf((float)y[i * g.dim + d] * (float)K);
        if (iy >= K) iy = K - 1;
        if (iy < 0) iy = 0;
        out[i * g.dim + d] = (T)__dmul_rn(inc[d * ldi + iy], (double)K);
    }
}
}  // namespace

extern "C" int vg_jac1d(int dim, const int64_t *ninc, const double *inc, int64_t ldi, int64_t n,
                        const void *y, void *out, int dtype, void *stream)
{
    VG_RANGE("vg_jac1d");
    vg_clear_error();
    MapGeom g;
    int rc = fill_geom(g, dim, ninc);
    if (rc) return rc;
    if (n <= 0) return VG_OK;
    const int64_t nb = (n + 255) / 256;
    if (dtype == VG_F64)
        jac1d_kernel<double><<<(unsigned)nb, 256, 0, (cudaStream_t)stream>>>(g, inc, ldi, n, (const double *)y,
                                                                              (double *)out);
    else
        jac1d_kernel<float><<<(unsigned)nb, 256, 0, (cudaStream_t)stream>>>(g, inc, ldi, n, (const float *)y,
                                                                             (float *)out);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

extern "C" int vg_map(int dim, const int64_t *ninc, const double *grid, const double *inc,
                      int64_t ldg, int64_t ldi, int64_t n, const void *y, void *x, void *jac,
                      int dtype, void *stream)
{
    VG_RANGE("vg_map");
    vg_clear_error();
    MapGeom g;
    int rc = fill_geom(g, dim, ninc);
    if (rc) return rc;
    if (n <= 0) return VG_OK;
    int nt = 256;
    int64_t nb = (n + nt - 1) / nt;
    if (dtype == VG_F64)
        map_kernel<double><<<(unsigned)nb, nt, 0, (cudaStream_t)stream>>>(
            g, grid, inc, ldg, ldi, n, (const double *)y, (double *)x, (double *)jac);
    else
        map_kernel<float><<<(unsigned)nb, nt, 0, (cudaStream_t)stream>>>(
            g, grid, inc, ldg, ldi, n, (const float *)y, (float *)x, (float *)jac);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

// ---------------------------------------------------------------- invmap
// pyx:362-413: iy = searchsorted(grid[d], x, side='right') (nodes <= x);
// inside: y = (iy-1 + (x - grid[iy-1]) / inc[iy-1]) / ninc, jac *= inc*ninc;
// below the first node y = 0 with inc[0]; above the last y = 1 with
// inc[ninc-1].  FP64 arithmetic for either storage type.
template <typename T>
__global__ void invmap_kernel(MapGeom g, const double *__restrict__ grid,
                              const double *__restrict__ inc, int64_t ldg, int64_t ldi, int64_t n,
                              const T *__restrict__ x, T *__restrict__ y, T *__restrict__ jac)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int dim = g.dim;
    double j = 1.0;
    for (int d = 0; d < dim; d++) {
        const int K = g.ninc[d];
        const double xv = (double)x[i * dim + d];
        const double *gd = grid + d * ldg;
        int lo = 0, hi = K + 1;   // first node > xv, in [0, K+1]
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (gd[mid] <= xv) lo = mid + 1;
            else hi = mid;
        }
        const int iy = lo;
        double yv, w;
        if (iy > 0 && iy <= K) {
            w = inc[d * ldi + iy - 1];
            yv = __ddiv_rn(__dadd_rn((double)(iy - 1), __ddiv_rn(__dsub_rn(xv, gd[iy - 1]), w)), (double)K);
        } else if (iy <= 0) {
            w = inc[d * ldi];
            yv = 0.0;
        } else {
            w = inc[d * ldi + K - 1];
            yv = 1.0;
        }
        y[i * dim + d] = (T)yv;
        j = __dmul_rn(j, __dmul_rn(w, (double)K));
    }
    jac[i] = (T)j;
}

extern "C" int vg_invmap(int dim, const int64_t *ninc, const double *grid, const double *inc,
                         int64_t ldg, int64_t ldi, int64_t n, const void *x, void *y, void *jac,
                         int dtype, void *stream)
{
    VG_RANGE("vg_invmap");
    vg_clear_error();
    MapGeom g;
    int rc = fill_geom(g, dim, ninc);
    if (rc) return rc;
    if (n <= 0) return VG_OK;
    const int nt = 256;
    const int64_t nb = (n + nt - 1) / nt;
    if (dtype == VG_F64)
        invmap_kernel<double><<<(unsigned)nb, nt, 0, (cudaStream_t)stream>>>(
            g, grid, inc, ldg, ldi, n, (const double *)x, (double *)y, (double *)jac);
    else
        invmap_kernel<float><<<(unsigned)nb, nt, 0, (cudaStream_t)stream>>>(
            g, grid, inc, ldg, ldi, n, (const float *)x, (float *)y, (float *)jac);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

extern "C" int vg_add_training_data(int dim, const int64_t *ninc, int64_t ldi, int64_t n,
                                    const void *y, const void *f, int dtype, double *sum_f,
                                    uint64_t *n_f, void *stream)
{
    VG_RANGE("vg_add_training_data");
    vg_clear_error();
    MapGeom g;
    int rc = fill_geom(g, dim, ninc);
    if (rc) return rc;
    if (n <= 0) return VG_OK;
    int nt = 256;
    int64_t nb = (n + nt - 1) / nt;
    if (dtype == VG_F64)
        train_kernel<double><<<(unsigned)nb, nt, 0, (cudaStream_t)stream>>>(
            g, ldi, n, (const double *)y, (const double *)f, sum_f, (unsigned long long *)n_f);
    else
        train_kernel<float><<<(unsigned)nb, nt, 0, (cudaStream_t)stream>>>(
            g, ldi, n, (const float *)y, (const float *)f, sum_f, (unsigned long long *)n_f);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

// Largest old ninc the adapt kernel handles (two FP64 rows in shared memory).
#define VG_ADAPT_MAX_NINC 12288

// In place the kernel also stages the old nodes and increments (two more rows).
int vg_adapt_in_place_ok(int max_old) { return 4 * (size_t)max_old + 1 <= 2 * VG_ADAPT_MAX_NINC; }

// In place (new_grid == grid, new_inc == inc) needs the old ninc to equal
// the new one and vg_adapt_in_place_ok(); zero_hist clears sum_f / n_f once
// read.
int vg_adapt_launch(int dim, const int64_t *old_ninc, const int64_t *new_ninc, const double *grid,
                    const double *inc, int64_t ldg, int64_t ldi, const double *sum_f,
                    const uint64_t *n_f, double alpha, double *new_grid, double *new_inc,
                    int64_t ldg_new, int64_t ldi_new, cudaStream_t st, int fast, int zero_hist)
{
    if (dim < 1 || dim > VG_MAX_DIM) return vg_fail(VG_ERR_UNSUPPORTED, "dim %d", dim);
    AdaptArgs a;
    memset(&a, 0, sizeof(a));
    a.dim = dim;
    int max_old = 0, max_new = 0, any_one = 0;
    for (int d = 0; d < dim; d++) {
        if (old_ninc[d] < 1 || new_ninc[d] < 1)
            return vg_fail(VG_ERR_VALUE, "ninc < 1: new ninc %lld", (long long)new_ninc[d]);
        if (old_ninc[d] > VG_ADAPT_MAX_NINC || new_ninc[d] > (1 << 30))
            return vg_fail(VG_ERR_UNSUPPORTED, "ninc %lld above %d", (long long)old_ninc[d],
                           VG_ADAPT_MAX_NINC);
        if (old_ninc[d] + 1 > ldg || old_ninc[d] > ldi || new_ninc[d] + 1 > ldg_new ||
            new_ninc[d] > ldi_new)
            return vg_fail(VG_ERR_VALUE, "grid arrays too small");
        a.old_ninc[d] = (int)old_ninc[d];
        a.new_ninc[d] = (int)new_ninc[d];
        max_old = old_ninc[d] > max_old ? (int)old_ninc[d] : max_old;
        max_new = new_ninc[d] > max_new ? (int)new_ninc[d] : max_new;
        any_one |= (old_ninc[d] == 1);
    }
    a.grid = grid;
    a.inc = inc;
    a.ldg = ldg;
    a.ldi = ldi;
    a.sum_f = sum_f;
    a.n_f = (const unsigned long long *)n_f;
    a.alpha = alpha;
    a.new_grid = new_grid;
    a.new_inc = new_inc;
    a.ldg_new = ldg_new;
    a.ldi_new = ldi_new;
    a.max_old = max_old;
    a.fast = fast;
    a.zero_hist = zero_hist;
    const int in_place = (new_grid == grid);
    if (in_place) {
        for (int d = 0; d < dim; d++)
            if (old_ninc[d] != new_ninc[d] || new_inc != inc || ldg_new != ldg || ldi_new != ldi)
                return vg_fail(VG_ERR_VALUE, "in-place adapt keeps ninc and strides");
        if (!vg_adapt_in_place_ok(max_old)) return vg_fail(VG_ERR_UNSUPPORTED, "in-place adapt: ninc too large");
    }
    if (max_new == 1) {
        adapt_single_kernel<<<1, 64, 0, st>>>(a);
        VG_LAUNCH_CHECK();
        return VG_OK;
    }
    // Axes are independent unless avg_f values carry over between them:
    // without training data and alpha > 0 (each axis smooths the previous
    // axis' output), or when an axis with a single increment reuses the
    // previous axis' avg_f[0] (pyx:533-564).
    a.sequential = ((sum_f == nullptr && alpha > 0) || (alpha != 0 && any_one)) ? 1 : 0;
    size_t smem = sizeof(double) * (2 * (size_t)max_old + ADAPT_NT);
    if (in_place) smem += sizeof(double) * (2 * (size_t)max_old + 1);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(adapt_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(double) * (2 * VG_ADAPT_MAX_NINC + ADAPT_NT)));
        attr = true;
    }
    adapt_kernel<<<a.sequential ? 1 : dim, ADAPT_NT, smem, st>>>(a);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

extern "C" int vg_adapt(int dim, const int64_t *old_ninc, const int64_t *new_ninc,
                        const double *grid, const double *inc, int64_t ldg, int64_t ldi,
                        const double *sum_f, const uint64_t *n_f, double alpha, double *new_grid,
                        double *new_inc, int64_t ldg_new, int64_t ldi_new, void *stream)
{
    VG_RANGE("vg_adapt");
    vg_clear_error();
    if (new_grid == grid) return vg_fail(VG_ERR_VALUE, "vg_adapt writes a separate grid");
    return vg_adapt_launch(dim, old_ninc, new_ninc, grid, inc, ldg, ldi, sum_f, n_f, alpha,
                           new_grid, new_inc, ldg_new, ldi_new, (cudaStream_t)stream, 0, 0);
}
