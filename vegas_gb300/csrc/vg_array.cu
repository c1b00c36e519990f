// vg_array.cu -- per-hypercube reduction of array-valued integrands.
//
// Reference: Integrator.__call__, src/vegas/_vegas.pyx:2136-2193 (the loops
// over fcn_size s): per hypercube, per component c the sums
//     sum_wf[c]  = sum_j wgt_j f_jc
//     dwf_c      = wgt_j f_jc - sum_wf[c]/n;  |dwf_c| < EPSILON |mean_c| ->
//                  sum_dwf2[c,c] += (EPSILON |mean_c|)^2 and dwf_c = 0
//                  (which removes it from the off-diagonal products)
//     sum_dwf[c] += dwf_c;  sum_dwf2[c,t] += dwf_c dwf_t  (t < c, correlated)
// and the iteration totals mean[c] += sum_wf[c] + sum_dwf[c] (Neely),
// var[c,t] += (n sum_dwf2[c,t] - sum_dwf[c] sum_dwf[t]) / (n - 1).
// sigf and the training histogram come from component 0 only (pyx:2173,
// 2181-2186): the scalar reduction (vg_reduce on column 0) does those.
//
// One warp per hypercube (static assignment), FP64 throughout; per-warp
// totals in a fixed order, then one block sums the warps' partials with
// Neumaier compensation -- deterministic.  Uncorrelated components are
// independent, so more than 16 of them are reduced 16 at a time (one pair
// of launches per group of columns).
#include <string.h>

#include "vg_tile.cuh"

namespace {

constexpr int AW = 8;              // warps per CTA
constexpr int ANT = AW * 32;

struct ArrArgs {
    int64_t H;
    const int64_t *offsets;
    const int32_t *neval_h;
    const double *wgt;
    const void *f;
    int f64;
    int s;                         // components in this launch
    int c0, ld;                    // first column of this launch, row length of f
    double *parts;                 // [nwarps][nval]
    int nval;
};

__device__ __forceinline__ double fval(const ArrArgs &a, int64_t j, int c)
{
    const int64_t i = j * a.ld + a.c0 + c;
    return a.f64 ? ((const double *)a.f)[i] : (double)((const float *)a.f)[i];
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

template <int SM, bool CORR>
__global__ void __launch_bounds__(ANT) array_hcube_kernel(ArrArgs a)
{
    constexpr int NP = CORR ? SM * (SM + 1) / 2 : SM;
    const int lane = threadIdx.x & 31;
    const int64_t gw = ((int64_t)blockIdx.x * ANT + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * ANT) >> 5;
    const int s = a.s;
    double M[SM], V[NP];
#pragma unroll
    for (int c = 0; c < SM; c++) M[c] = 0.0;
#pragma unroll
    for (int p = 0; p < NP; p++) V[p] = 0.0;
    for (int64_t h = gw; h < a.H; h += nw) {
        const int64_t off = a.offsets[h];
        const int n = a.neval_h[h];
        double sw[SM];
#pragma unroll
        for (int c = 0; c < SM; c++) sw[c] = 0.0;
        for (int j = lane; j < n; j += 32) {
            const double w = a.wgt[off + j];
#pragma unroll
            for (int c = 0; c < SM; c++)
                if (c < s) sw[c] = __dadd_rn(sw[c], __dmul_rn(w, fval(a, off + j, c)));
        }
        double mc[SM], thr[SM];
#pragma unroll
        for (int c = 0; c < SM; c++) {
            sw[c] = warp_sum(sw[c]);
            mc[c] = __ddiv_rn(sw[c], (double)n);
            thr[c] = __dmul_rn(VG_EPSILON, fabs(mc[c]));
        }
        double sd[SM], q[NP];
#pragma unroll
        for (int c = 0; c < SM; c++) sd[c] = 0.0;
#pragma unroll
        for (int p = 0; p < NP; p++) q[p] = 0.0;
        for (int j = lane; j < n; j += 32) {
            const double w = a.wgt[off + j];
            double d[SM];
#pragma unroll
            for (int c = 0; c < SM; c++) {
                d[c] = 0.0;
                if (c >= s) continue;
                double dv = __dsub_rn(__dmul_rn(w, fval(a, off + j, c)), mc[c]);
                const int qi = CORR ? c * (c + 1) / 2 + c : c;
                if (fabs(dv) < thr[c]) {
                    q[qi] = __dadd_rn(q[qi], __dmul_rn(thr[c], thr[c]));
                    dv = 0.0;
                } else {
                    q[qi] = __dadd_rn(q[qi], __dmul_rn(dv, dv));
                }
                sd[c] = __dadd_rn(sd[c], dv);
                d[c] = dv;
                if (CORR) {
#pragma unroll
                    for (int t = 0; t < SM; t++)
                        if (t < c) q[c * (c + 1) / 2 + t] = __dadd_rn(q[c * (c + 1) / 2 + t], __dmul_rn(dv, d[t]));
                }
            }
        }
        const double nd = (double)n;
#pragma unroll
        for (int c = 0; c < SM; c++) {
            if (c >= s) continue;
            sd[c] = warp_sum(sd[c]);
            M[c] = __dadd_rn(M[c], __dadd_rn(sw[c], sd[c]));
        }
#pragma unroll
        for (int c = 0; c < SM; c++) {
            if (c >= s) continue;
            if (CORR) {
#pragma unroll
                for (int t = 0; t < SM; t++) {
                    if (t > c) continue;
                    const int p = c * (c + 1) / 2 + t;
                    const double qq = warp_sum(q[p]);
                    V[p] = __dadd_rn(V[p], __ddiv_rn(__dsub_rn(__dmul_rn(nd, qq), __dmul_rn(sd[c], sd[t])),
                                                     __dsub_rn(nd, 1.)));
                }
            } else {
                const double qq = warp_sum(q[c]);
                V[c] = __dadd_rn(V[c], __ddiv_rn(__dsub_rn(__dmul_rn(nd, qq), __dmul_rn(sd[c], sd[c])),
                                                 __dsub_rn(nd, 1.)));
            }
        }
    }
    if (lane == 0) {
        double *P = a.parts + gw * a.nval;
#pragma unroll
        for (int c = 0; c < SM; c++)
            if (c < s) P[c] = M[c];
#pragma unroll
        for (int p = 0; p < NP; p++)
            if (s + p < a.nval) P[s + p] = V[p];
    }
}

// Fixed-order compensated sum of the warps' partials (one thread per value),
// unpacked into mean[s] and the s x s (co)variance matrix.
// Components c0 .. c0+s-1 of an s_all-component integrand; the first launch
// (zero = 1) clears the whole matrix.
__global__ void array_total_kernel(const double *__restrict__ parts, int64_t nw, int nval, int s, int corr,
                                   int c0, int s_all, int zero, double *__restrict__ mean_out,
                                   double *__restrict__ var_out)
{
    if (zero)
        for (int i = threadIdx.x; i < s_all * s_all; i += blockDim.x) var_out[i] = 0.0;
    __syncthreads();
    for (int v = threadIdx.x; v < nval; v += blockDim.x) {
        VgKSum k = {0.0, 0.0};
        for (int64_t w = 0; w < nw; w++) k.add(parts[w * nval + v]);
        const double tot = k.value();
        if (v < s) {
            mean_out[c0 + v] = tot;
        } else if (corr) {
            int p = v - s, c = 0;
            while ((c + 1) * (c + 2) / 2 <= p) c++;
            const int t = p - c * (c + 1) / 2;
            var_out[c * s + t] = tot;
            var_out[t * s + c] = tot;
        } else {
            const int c = c0 + v - s;
            var_out[(int64_t)c * s_all + c] = tot;
        }
    }
}

}  // namespace

// mean_out[s]; var_out[s*s] (correlated: full symmetric matrix; else the
// diagonal in var_out[c*s + c], zeros elsewhere).
extern "C" int vg_reduce_array(const vg_integrator *it, const void *f, int f_dtype, int s, int correlate,
                               const double *wgt, double *mean_out, double *var_out, void *work,
                               size_t work_bytes, void *stream)
{
    VG_RANGE("vg_reduce_array");
    vg_clear_error();
    vg::IterArgs a;
    int rc = vg::fill_iter_args(a, it, 0, nullptr);
    if (rc) return rc;
    if (s < 1) return vg_fail(VG_ERR_VALUE, "s < 1");
    if (correlate && s > 6)
        return vg_fail(VG_ERR_UNSUPPORTED, "array integrands: s <= 6 correlated components");
    const int np = correlate ? s * (s + 1) / 2 : s;
    const int nval = s + np;
    const int grid = vg_num_sms() * 2;
    const int64_t nw = (int64_t)grid * AW;
    const size_t need = sizeof(double) * (size_t)nw * nval;
    if (work_bytes < need) return vg_fail(VG_ERR_VALUE, "array workspace %zu < %zu", work_bytes, need);
    ArrArgs A;
    A.H = it->nhcube;
    A.offsets = a.offsets;
    A.neval_h = a.neval_h;
    A.wgt = wgt;
    A.f = f;
    A.f64 = (f_dtype == VG_F64);
    A.ld = s;
    cudaStream_t st = (cudaStream_t)stream;
    if (correlate) {
        A.s = s;
        A.c0 = 0;
        A.parts = (double *)work;
        A.nval = nval;
        array_hcube_kernel<6, true><<<grid, ANT, 0, st>>>(A);
        VG_LAUNCH_CHECK();
        array_total_kernel<<<1, 128, 0, st>>>((const double *)work, nw, nval, s, 1, 0, s, 1, mean_out, var_out);
        VG_LAUNCH_CHECK();
        return VG_OK;
    }
    for (int c0 = 0; c0 < s; c0 += 16) {   // groups of 16 independent columns
        const int sc = s - c0 < 16 ? s - c0 : 16;
        A.s = sc;
        A.c0 = c0;
        A.nval = 2 * sc;
        A.parts = (double *)work + (size_t)nw * 2 * c0;
        if (sc <= 8) array_hcube_kernel<8, false><<<grid, ANT, 0, st>>>(A);
        else array_hcube_kernel<16, false><<<grid, ANT, 0, st>>>(A);
        VG_LAUNCH_CHECK();
        array_total_kernel<<<1, 128, 0, st>>>(A.parts, nw, A.nval, sc, 0, c0, s, c0 == 0, mean_out, var_out);
        VG_LAUNCH_CHECK();
    }
    return VG_OK;
}

extern "C" size_t vg_reduce_array_work_bytes(int s, int correlate)
{
    const int np = correlate ? s * (s + 1) / 2 : s;
    const int64_t nw = (int64_t)vg_num_sms() * 2 * AW;
    return sizeof(double) * (size_t)nw * (s + np);
}
