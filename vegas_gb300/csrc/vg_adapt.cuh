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
    int zero_hist;    // clear sum_f / n_f once read (the end of an iteration)
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
    double r = (double)__frcp_rn((float)b);
    r = fma(r, fma(-b, r, 1.0), r);
    return a * r;
}

// Block-wide inclusive prefix sum of v[0..n) in place (FP64, fixed order):
// per-thread sequential over a contiguous chunk, then a scan of the chunk
// totals by warp shuffles (within each warp, then over the warp totals) --
// few FP64 instructions per thread (GB300 issues FP64 at a low rate).
template <int ADAPT_NT>
__device__ void block_inclusive_scan(double *v, int n, double *part /* >= 32 */)
{
    constexpr int NW = ADAPT_NT / 32;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int per = (n + ADAPT_NT - 1) / ADAPT_NT;
    const int b = t * per, e = min(n, b + per);
    double s = 0.0;
    for (int i = b; i < e; i++) {
        s = __dadd_rn(s, v[i]);
        v[i] = s;
    }
    double x = s;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const double y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x = __dadd_rn(x, y);
    }
    if (lane == 31) part[w] = x;
    __syncthreads();
    if (w == 0) {
        double z = lane < NW ? part[lane] : 0.0;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, z, off);
            if (lane >= off) z = __dadd_rn(z, y);
        }
        if (lane < NW) part[lane] = z;
    }
    __syncthreads();
    double ex = __shfl_up_sync(0xffffffffu, x, 1);   // exclusive prefix within the warp
    if (lane == 0) ex = 0.0;
    if (t > 0) {
        const double carry = (w > 0) ? __dadd_rn(part[w - 1], ex) : ex;
        for (int i = b; i < e; i++) v[i] = __dadd_rn(v[i], carry);
    }
    __syncthreads();
}

// Sum of v[0..n) in a fixed order; result broadcast to all threads.
template <int ADAPT_NT>
__device__ double block_sum(const double *v, int n, double *part /* >= 33 */)
{
    constexpr int NW = ADAPT_NT / 32;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    double s = 0.0;
    for (int i = t; i < n; i += ADAPT_NT) s = __dadd_rn(s, v[i]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s = __dadd_rn(s, __shfl_xor_sync(0xffffffffu, s, off));
    if (lane == 0) part[w] = s;
    __syncthreads();
    if (w == 0) {
        double z = lane < NW ? part[lane] : 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) z = __dadd_rn(z, __shfl_xor_sync(0xffffffffu, z, off));
        if (lane == 0) part[32] = z;
    }
    __syncthreads();
    const double r = part[32];
    __syncthreads();
    return r;
}

// FP32 block reductions (max, sum) over ADAPT_NT threads; f = shared scratch
// of >= 33 floats.  Result broadcast to all threads.
template <int ADAPT_NT, bool MAX>
__device__ float block_reduce_f(float v, float *f)
{
    constexpr int NW = ADAPT_NT / 32;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float o = __shfl_xor_sync(0xffffffffu, v, off);
        v = MAX ? fmaxf(v, o) : v + o;
    }
    if (lane == 0) f[w] = v;
    __syncthreads();
    if (w == 0) {
        float z = lane < NW ? f[lane] : 0.f;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float o = __shfl_xor_sync(0xffffffffu, z, off);
            z = MAX ? fmaxf(z, o) : z + o;
        }
        if (lane == 0) f[32] = z;
    }
    __syncthreads();
    const float r = f[32];
    __syncthreads();
    return r;
}

// FP32 mode, alpha > 0 with training data: the weights of one axis (average,
// 3-tap smoothing, normalisation, damping; pyx:539-562) in FP32 on the MUFU,
// written to avg[] as doubles.  A normalised weight outside the float range
// (or within 1e-5 of 1) is formed and damped in FP64, so tiny weights keep
// the reference's ((1 - v) / -ln v)^alpha.  The cumulative sums and the new
// nodes (regrid) stay FP64.
template <int ADAPT_NT>
__device__ void adapt_weights_fast(const AdaptArgs &a, int d, int K, double *avg, double *tmp, double *part)
{
    const int t = threadIdx.x;
    float *af = reinterpret_cast<float *>(tmp);   // [K] averages
    float *sf = af + K;                           // [K] smoothed (tmp holds 2K floats)
    float *pf = reinterpret_cast<float *>(part);
    for (int i = t; i < K; i += ADAPT_NT) {
        const unsigned long long c = a.n_f[d * a.ldi + i];
        af[i] = c ? (float)div_fast(a.sum_f[d * a.ldi + i], (double)c) : 0.f;
        if (a.zero_hist) {
            const_cast<double *>(a.sum_f)[d * a.ldi + i] = 0.0;
            const_cast<unsigned long long *>(a.n_f)[d * a.ldi + i] = 0ull;
        }
    }
    __syncthreads();
    float mx = 0.f;
    for (int i = t; i < K; i += ADAPT_NT) {
        float v;
        if (i == 0) v = fmaf(7.f, af[0], af[1]);
        else if (i == K - 1) v = fmaf(7.f, af[K - 1], af[K - 2]);
        else v = fmaf(6.f, af[i], af[i - 1] + af[i + 1]);
        v = fabsf(v) * 0.125f;
        sf[i] = v;
        mx = fmaxf(mx, v);
    }
    mx = block_reduce_f<ADAPT_NT, true>(mx, pf);
    const float rmx = mx > 0.f ? 1.f / mx : 0.f;   // sum of values scaled by the max: no overflow
    float sp = 0.f;
    for (int i = t; i < K; i += ADAPT_NT) sp += sf[i] * rmx;
    sp = block_reduce_f<ADAPT_NT, false>(sp, pf);
    const float rs = sp > 0.f ? 1.f / sp : 0.f;
    const float alf = (float)a.alpha;
    for (int i = t; i < K; i += ADAPT_NT) {
        const float vf = sf[i] * rmx * rs;
        double v;
        if (sp > 0.f && vf >= 1.17549435e-38f && vf < 0.99999f) {
            const float one_m = 1.f - vf;
            const float lnv = one_m < 0.25f ? log1pf(-one_m) : vg_lg2_approx(vf) * 0.69314718f;
            const float q = one_m / (-lnv);
            v = (double)vg_ex2_approx(alf * vg_lg2_approx(q));
        } else {
            v = sp > 0.f ? (double)sf[i] * (double)rmx * (double)rs + VG_TINY : VG_TINY;
            if (v > 0 && v <= 0.99999999) v = damp_fast(v, a.alpha);
        }
        avg[i] = v;
    }
    __syncthreads();
}

// One axis of AdaptiveMap.adapt.  avg (length >= max_old) holds the carried
// avg_f values on entry, the final ones on exit.  With gs / is (shared
// memory, max_old + 1 and max_old doubles) the axis' old nodes and
// increments are staged there first, so new_grid / new_inc may be the grid
// itself (adapt in place).
template <int ADAPT_NT>
__device__ void adapt_axis(const AdaptArgs &a, int d, double *avg, double *tmp, double *part,
                           double *gs = nullptr, double *is = nullptr)
{
    const int K = a.old_ninc[d];
    const int Kn = a.new_ninc[d];
    const int t = threadIdx.x;
    const double alpha = a.alpha;
    if (alpha > 0 && K > 1 && a.fast && a.sum_f != nullptr) {
        adapt_weights_fast<ADAPT_NT>(a, d, K, avg, tmp, part);
    } else if (alpha != 0 && K > 1) {
        if (a.sum_f != nullptr) {
            for (int i = t; i < K; i += ADAPT_NT) {
                const unsigned long long c = a.n_f[d * a.ldi + i];
                if (a.fast) {
                    avg[i] = c ? div_fast(a.sum_f[d * a.ldi + i], (double)c) : 0.0;
                } else {
                    const double nf = __dadd_rn((double)c, VG_TINY);
                    avg[i] = (nf > 0) ? __ddiv_rn(a.sum_f[d * a.ldi + i], nf) : 0.0;
                }
                if (a.zero_hist) {
                    const_cast<double *>(a.sum_f)[d * a.ldi + i] = 0.0;
                    const_cast<unsigned long long *>(a.n_f)[d * a.ldi + i] = 0ull;
                }
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
                tmp[i] = __dmul_rn(fabs(v), 0.125);   // == v / 8 exactly
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
    const double *gd = a.grid + d * a.ldg;
    const double *id = a.inc + d * a.ldi;
    for (int i = t; i < K; i += ADAPT_NT) {
        P[i] = avg[i];
        if (gs != nullptr) {
            gs[i] = gd[i];
            is[i] = id[i];
        }
    }
    if (gs != nullptr && t == 0) gs[K] = gd[K];
    __syncthreads();
    if (gs != nullptr) {
        gd = gs;
        id = is;
    }
    block_inclusive_scan<ADAPT_NT>(P, K, part);
    const double total = P[K - 1];
    const double f_ninc = a.fast ? div_fast(total, (double)Kn) : __ddiv_rn(total, (double)Kn);
    double *ng = a.new_grid + d * a.ldg_new;
    for (int i = t; i <= Kn; i += ADAPT_NT) {
        double v;
        if (i == 0) v = gd[0];
        else if (i == Kn) v = gd[K];
        else {
            const double target = __dmul_rn((double)i, f_ninc);
            // first j with P[j] >= target; P and target are >= 0, so their
            // IEEE bit patterns order like the values (integer compares)
            const long long tb = __double_as_longlong(target);
            int lo = 0, hi = K - 1;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (__double_as_longlong(P[mid]) < tb) lo = mid + 1;
                else hi = mid;
            }
            int j = lo;
            double acc = __dsub_rn(P[j], target);
            const double q = a.fast ? div_fast(acc, avg[j]) : __ddiv_rn(acc, avg[j]);
            v = __dsub_rn(gd[j + 1], __dmul_rn(q, id[j]));
        }
        ng[i] = v;
    }
    __syncthreads();
    double *ni = a.new_inc + d * a.ldi_new;
    for (int i = t; i < Kn; i += ADAPT_NT) ni[i] = __dsub_rn(ng[i + 1], ng[i]);
    __syncthreads();
}


}  // namespace vgadapt
