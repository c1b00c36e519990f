// vg_adapt.cuh -- AdaptiveMap.adapt for one axis as a block-level device
// function (src/vegas/_vegas.pyx:467-594: average of the training data,
// 3-tap smoothing, normalisation, damping ((1-f)/-ln f)^alpha, regrid).
// Templated on the block size: the adapt kernel runs it with 1024 threads
// per axis, the batched kernel with the 256 threads of its CTA.
#pragma once
#include "vg_common.cuh"

namespace vgadapt {

struct AdaptArgs {
    int dim;
    int old_ninc[VG_MAX_DIM];
    int new_ninc[VG_MAX_DIM];
    const double *grid, *inc;
    int64_t ldg, ldi;
    const double *sum_f;
    const unsigned long long *n_f;
    double alpha;
    double *new_grid, *new_inc;
    int64_t ldg_new, ldi_new;
    int max_old;      // length of the shared avg_f buffer (pyx:533)
    int sequential;   // one block walks all axes, carrying avg_f (pyx:533 semantics)
    int fast;         // FP32 mode: MUFU transcendentals and reciprocal multiplies
};

// ((1 - v) / -ln v)^alpha of the damping step (pyx:560-562), FP32-mode path:
// 1 - v and the exponent split in double, logs/exps on the MUFU.
__device__ __forceinline__ double damp_fast(double v, double alpha)
{
    const double one_m = 1.0 - v;
    float lnv;
    if (one_m < 0.25) lnv = log1pf((float)(v - 1.0));
    else lnv = vg_log2_split(v) * 0.69314718055994531f;
    const float q = (float)one_m / (-lnv);
    return (double)vg_ex2_approx((float)alpha * vg_lg2_approx(q));
}

// a / b in double with one Newton step on a float reciprocal (FP32 mode).
__device__ __forceinline__ double div_fast(double a, double b)
{
    double r = (double)(1.0f / (float)b);
    r = fma(r, fma(-b, r, 1.0), r);
    return a * r;
}

// Block-wide inclusive prefix sum of v[0..n) in place (FP64, fixed order):
// per-thread sequential over a contiguous chunk, then a scan of chunk totals.
template <int ADAPT_NT>
__device__ void block_inclusive_scan(double *v, int n, double *part /* ADAPT_NT */)
{
    int t = threadIdx.x;
    int per = (n + ADAPT_NT - 1) / ADAPT_NT;
    int b = t * per, e = min(n, b + per);
    double s = 0.0;
    for (int i = b; i < e; i++) {
        s = __dadd_rn(s, v[i]);
        v[i] = s;
    }
    part[t] = s;
    __syncthreads();
    // Hillis-Steele on the ADAPT_NT chunk totals
    for (int off = 1; off < ADAPT_NT; off <<= 1) {
        double add = (t >= off) ? part[t - off] : 0.0;
        __syncthreads();
        part[t] = __dadd_rn(part[t], add);
        __syncthreads();
    }
    double carry = (t > 0) ? part[t - 1] : 0.0;
    if (t > 0)
        for (int i = b; i < e; i++) v[i] = __dadd_rn(v[i], carry);
    __syncthreads();
}

// Sum of v[0..n) in a fixed order; result broadcast to all threads.
template <int ADAPT_NT>
__device__ double block_sum(const double *v, int n, double *part)
{
    int t = threadIdx.x;
    double s = 0.0;
    for (int i = t; i < n; i += ADAPT_NT) s = __dadd_rn(s, v[i]);
    part[t] = s;
    __syncthreads();
    for (int off = ADAPT_NT / 2; off > 0; off >>= 1) {
        if (t < off) part[t] = __dadd_rn(part[t], part[t + off]);
        __syncthreads();
    }
    double r = part[0];
    __syncthreads();
    return r;
}

// One axis of AdaptiveMap.adapt.  avg (length >= max_old) holds the carried
// avg_f values on entry, the final ones on exit.
template <int ADAPT_NT>
__device__ void adapt_axis(const AdaptArgs &a, int d, double *avg, double *tmp, double *part)
{
    const int K = a.old_ninc[d];
    const int Kn = a.new_ninc[d];
    const int t = threadIdx.x;
    const double alpha = a.alpha;
    if (alpha != 0 && K > 1) {
        if (a.sum_f != nullptr) {
            for (int i = t; i < K; i += ADAPT_NT) {
                const unsigned long long c = a.n_f[d * a.ldi + i];
                const double nf = __dadd_rn((double)c, VG_TINY);
                if (a.fast) avg[i] = c ? div_fast(a.sum_f[d * a.ldi + i], (double)c) : 0.0;
                else avg[i] = (nf > 0) ? __ddiv_rn(a.sum_f[d * a.ldi + i], nf) : 0.0;
            }
            __syncthreads();
        }
        if (alpha > 0) {
            // smoothing, pyx:548-553
            for (int i = t; i < K; i += ADAPT_NT) {
                double v;
                if (i == 0) v = __dadd_rn(__dmul_rn(7., avg[0]), avg[1]);
                else if (i == K - 1) v = __dadd_rn(__dmul_rn(7., avg[K - 1]), avg[K - 2]);
                else v = __dadd_rn(__dadd_rn(__dmul_rn(6., avg[i]), avg[i - 1]), avg[i + 1]);
                tmp[i] = __ddiv_rn(fabs(v), 8.);
            }
            __syncthreads();
            double s = block_sum<ADAPT_NT>(tmp, K, part);
            // normalise + damp, pyx:554-562
            const double rs = (s > 0) ? 1.0 / s : 0.0;
            for (int i = t; i < K; i += ADAPT_NT) {
                double v;
                if (a.fast) {
                    v = (s > 0) ? tmp[i] * rs + VG_TINY : VG_TINY;
                    if (v > 0 && v <= 0.99999999) v = damp_fast(v, alpha);
                } else {
                    v = (s > 0) ? __dadd_rn(__ddiv_rn(tmp[i], s), VG_TINY) : VG_TINY;
                    if (v > 0 && v <= 0.99999999) v = pow(__ddiv_rn(-(1 - v), log(v)), alpha);
                }
                avg[i] = v;
            }
            __syncthreads();
        }
    }
    // regrid, pyx:563-587: new node i sits where the running sum of avg_f
    // reaches i*f_ninc; found by a block scan + binary search per node.
    double *P = tmp;
    for (int i = t; i < K; i += ADAPT_NT) P[i] = avg[i];
    __syncthreads();
    block_inclusive_scan<ADAPT_NT>(P, K, part);
    double total = P[K - 1];
    double f_ninc = __ddiv_rn(total, (double)Kn);
    const double *gd = a.grid + d * a.ldg;
    const double *id = a.inc + d * a.ldi;
    double *ng = a.new_grid + d * a.ldg_new;
    for (int i = t; i <= Kn; i += ADAPT_NT) {
        double v;
        if (i == 0) v = gd[0];
        else if (i == Kn) v = gd[K];
        else {
            double target = __dmul_rn((double)i, f_ninc);
            int lo = 0, hi = K - 1;   // first j with P[j] >= target
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (P[mid] < target) lo = mid + 1;
                else hi = mid;
            }
            int j = lo;
            double acc = __dsub_rn(P[j], target);
            v = __dsub_rn(gd[j + 1], __dmul_rn(__ddiv_rn(acc, avg[j]), id[j]));
        }
        ng[i] = v;
    }
    __syncthreads();
    double *ni = a.new_inc + d * a.ldi_new;
    for (int i = t; i < Kn; i += ADAPT_NT) ni[i] = __dsub_rn(ng[i + 1], ng[i]);
    __syncthreads();
}


}  // namespace vgadapt
