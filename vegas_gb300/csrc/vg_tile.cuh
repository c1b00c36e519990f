// vg_tile.cuh -- the persistent tile kernel of a vegas+ iteration.
//
// Reference: src/vegas/_vegas.pyx (vegas 6.4.1): sampling and map of
// Integrator._random_batch (pyx:1731-1752), the per-hypercube two-pass
// reduction of Integrator.__call__ (pyx:2136-2193), the training feed
// (pyx:2173, 2196-2197 -> AdaptiveMap.add_training_data pyx:421-464).
//
// Samples of an iteration are ordered by hypercube (as in the reference).  A
// tile is NT*S consecutive samples; thread t owns samples [t*S, t*S+S) of the
// tile.  CTAs take tiles from an atomic counter; everything a tile produces
// is indexed by the tile, so results do not depend on which CTA ran it.
//
// Template parameters: T (float | double) is the sampling/map/integrand
// arithmetic; DIMB is a compile-time bound on the dimension (arrays stay in
// registers); S samples per thread; MODE points / reduce / fused; KIND the
// built-in integrand of the fused mode.
#pragma once
#include <math.h>
#include <string.h>

#include "vg_common.cuh"
#include "vg_integrands.cuh"

namespace vg {

constexpr int NT = 256;          // threads per tile CTA
constexpr int BASE_TILE = 256;   // granularity of the tile schedule tile_h0[]
#define VG_WAIT_ITERS_DEFAULT (1u << 24)   // polls of a bounded wait (vg_set_wait_budget)
extern uint32_t g_wait_iters;
constexpr int ALLOC_NT = 256;    // allocation count / offsets blocks
constexpr int ALLOC_PER = 4;     // hypercubes per thread there
constexpr int FIN_NT = 1024;

// POINTS: write points for a torch integrand (optionally also keep each
// sample's Jacobian and training bins); REDUCE: read f and reduce,
// regenerating each sample; REDUCE_KEPT: read f and the kept Jacobians and
// bins and reduce (no Philox, no map: a stream over HBM); FUSED: evaluate a
// built-in integrand and reduce in one kernel; EVAL: evaluate a built-in
// integrand and write f (first half of the split path used for expensive
// integrands, followed by a REDUCE launch).
enum { MODE_POINTS = 0, MODE_REDUCE = 1, MODE_FUSED = 2, MODE_EVAL = 3, MODE_REDUCE_KEPT = 4 };

// Partial statistics of a hypercube cut by a tile boundary.
struct TileRec {
    int64_t h;       // hypercube, -1 if the slot is empty
    double n;        // samples of h inside the tile
    double S;        // sum of wf
    double Q;        // sum of squared deviations about S/n (EPSILON-guarded)
    double D;        // sum of deviations (round-off residue: Neely correction)
    int32_t spans;   // head slot only: h also continues past the tile
    int32_t pad;
};

struct TilePart {
    VgKSum mean, var, sigf;
};

struct IterArgs {
    int dim;
    int nstrat[VG_MAX_DIM];
    int ninc[VG_MAX_DIM];
    const double *grid, *inc;
    int64_t ldg, ldi;
    int64_t H;
    int64_t ncap;
    double *sigf;
    double beta;
    int adaptive;             // update sigf (pyx:2083, 2183-2186)
    int adaptive_alloc;       // allocate from sigf (pyx:1668)
    int train;                // accumulate training histogram (pyx:2196)
    int train_hc;             // adapt_to_errors: train on each hypercube's variance (pyx:2187-2193)
    double *sum_f;
    unsigned long long *n_f;
    vg_stats *stats;
    int32_t *neval_h;
    int64_t *offsets;
    int64_t *bsum;            // allocation: published block totals / prefixes
    int64_t *tile_h0;         // first hypercube of each BASE_TILE samples
    unsigned long long *counter;  // dynamic tile counter (reset by allocation)
    unsigned int *fin_counter;    // finalize blocks done (reset by allocation)
    unsigned int *alloc_sync;     // single-pass allocation: ticket, epoch, error, count maximum
    TileRec *recs;
    TilePart *parts;
    int64_t ntiles_cap;       // in BASE_TILE units
    int64_t neval;
    double neval_frac;
    int64_t min_neval_hcube, max_neval_hcube;
    uint64_t seed;
    uint32_t stream;
    uint32_t itn;
    const double *u;          // injected uniforms [n, dim] or nullptr
    const void *f_in;         // MODE_REDUCE, MODE_REDUCE_KEPT
    void *keep_jac;           // per-sample Jacobian (T): written by MODE_POINTS when set, read by REDUCE_KEPT
    unsigned short *keep_bins;   // per-sample training bins [n, keep_bstride] (0xffff: none), likewise
    int keep_bstride;            // bins per kept sample: dim rounded up to 4 (8-byte aligned rows)
    int f_f64;
    void *x_out, *y_out;      // MODE_POINTS
    float *f_eval;            // MODE_EVAL output / MODE_REDUCE input of the split path
    TilePart *part2;          // finalize: one partial per finalize block
    double *wgt_out;
    int64_t *hc_out;
    float2 *tablef;           // FP32 mode: (x_node, inc) table [dim][maxK+1], built by the allocation
    int table_smem;           // grid table staged in shared memory
    int hist_smem;            // training histogram in shared memory
    int maxK;
    int tab_len;              // integrand table length (floats)
    int T;                    // tile size of the launched kernel
    int ncta;                 // CTAs of the launched reduction kernel (one partial each)
    double dv_y;              // 1 / nhcube (pyx:1639)
    double beta_half;         // beta / 2 (pyx:2185)
    uint32_t wait_iters;      // polls of a bounded wait before it gives up (vg_set_wait_budget)
    uint32_t pad_wait;
};

template <typename T>
struct GridEntry;
template <>
struct GridEntry<float> {
    typedef float2 type;
};
template <>
struct GridEntry<double> {
    typedef double2 type;
};

struct SmemPlan {
    size_t table, hsum, hcnt, bins, win_off, win_n, win_w, seg_S, keyF, keyL, P, red, itab, total;
};

template <typename T>
__host__ __device__ inline SmemPlan smem_plan(int dim, int maxK, int Ttile, int table_smem,
                                              int hist_smem, int tab_len, int bins_smem,
                                              int need_red)
{
    SmemPlan p;
    size_t o = 0;
    p.table = o;
    if (table_smem) o = (o + sizeof(typename GridEntry<T>::type) * (size_t)dim * (maxK + 1) + 15) & ~(size_t)15;
    p.hsum = o;
    if (hist_smem) o = (o + sizeof(T) * (size_t)dim * maxK + 15) & ~(size_t)15;
    p.hcnt = o;
    if (hist_smem) o = (o + sizeof(unsigned int) * (size_t)dim * maxK + 15) & ~(size_t)15;
    p.bins = o;
    if (bins_smem) o = (o + sizeof(unsigned short) * (size_t)Ttile * dim + 15) & ~(size_t)15;
    p.win_off = o; o = (o + sizeof(int) * (Ttile + 2) + 15) & ~(size_t)15;
    p.win_n = o;   o = (o + sizeof(int) * (Ttile + 2) + 15) & ~(size_t)15;
    p.win_w = o;   o = (o + sizeof(float) * (Ttile + 2) + 15) & ~(size_t)15;
    p.seg_S = o;   if (need_red) o = (o + sizeof(double) * (Ttile + 2) + 15) & ~(size_t)15;
    p.keyF = o;    if (need_red) o = (o + sizeof(int) * NT + 15) & ~(size_t)15;
    p.keyL = o;    if (need_red) o = (o + sizeof(int) * NT + 15) & ~(size_t)15;
    p.P = o;       if (need_red) o = (o + sizeof(double2) * NT + 15) & ~(size_t)15;
    p.red = o;     if (need_red) o = (o + sizeof(VgKSum) * (NT / 32) * 3 + 64 + 15) & ~(size_t)15;
    p.itab = o;    o = (o + sizeof(float) * (tab_len + 4) + 15) & ~(size_t)15;
    p.total = o;
    return p;
}

// Inclusive segmented scan over the NT threads of (flag, value2); the result
// for thread t is returned and stored in P[t].
__device__ __forceinline__ double2 seg_scan(int flag, double2 v, double2 *P, double2 *wsum,
                                            int *wflag)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int f = flag;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        double ux = __shfl_up_sync(0xffffffffu, v.x, off);
        double uy = __shfl_up_sync(0xffffffffu, v.y, off);
        int uf = __shfl_up_sync(0xffffffffu, f, off);
        if (lane >= off) {
            if (!f) {
                v.x = ux + v.x;
                v.y = uy + v.y;
            }
            f |= uf;
        }
    }
    if (lane == 31) {
        wsum[w] = v;
        wflag[w] = f;
    }
    __syncthreads();
    if (w == 0) {
        const int NW = NT / 32;
        double2 x = lane < NW ? wsum[lane] : make_double2(0.0, 0.0);
        int g = lane < NW ? wflag[lane] : 1;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            double ux = __shfl_up_sync(0xffffffffu, x.x, off);
            double uy = __shfl_up_sync(0xffffffffu, x.y, off);
            int ug = __shfl_up_sync(0xffffffffu, g, off);
            if (lane >= off) {
                if (!g) {
                    x.x = ux + x.x;
                    x.y = uy + x.y;
                }
                g |= ug;
            }
        }
        if (lane < NW) wsum[lane] = x;
    }
    __syncthreads();
    if (w > 0 && !f) {
        double2 c = wsum[w - 1];
        v.x = c.x + v.x;
        v.y = c.y + v.y;
    }
    P[threadIdx.x] = v;
    __syncthreads();
    return v;
}

// (ah, al) += (bh, bl) in float-float (TwoSum of the heads, tails added,
// renormalised).  Used by the FP32 mode's reduction within a tile.
__device__ __forceinline__ void ff_add_pair(float &ah, float &al, float bh, float bl)
{
    const float s = __fadd_rn(ah, bh);
    const float bb = __fsub_rn(s, ah);
    float e = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    e = __fadd_rn(e, __fadd_rn(al, bl));
    ah = __fadd_rn(s, e);
    al = __fsub_rn(e, __fsub_rn(ah, s));
}

// FP32 mode keeps float-float values in the FP64 fields of the tile records
// and partial sums as bit patterns (low word = head, high word = tail), so
// storing and loading them moves integers -- GB300's FP64 pipe is slow, and
// a single warp waits hundreds of cycles per dependent FP64 instruction.
__device__ __forceinline__ double ff_pack(float h, float l)
{
    return __hiloint2double(__float_as_int(l), __float_as_int(h));
}

__device__ __forceinline__ void ff_unpack(double d, float &h, float &l)
{
    h = __int_as_float(__double2loint(d));
    l = __int_as_float(__double2hiint(d));
}

// Block-wide float-float reduction of six floats (three float-float values)
// in a fixed order; the result is valid in thread 0.  scratch: 6 * NTB/32
// floats of shared memory.
template <int NTB>
__device__ __forceinline__ void ff_block_reduce6(float (&r6)[6], float *scratch)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        float o6[6];
#pragma unroll
        for (int i = 0; i < 6; i++) o6[i] = __shfl_down_sync(0xffffffffu, r6[i], off);
#pragma unroll
        for (int i = 0; i < 6; i += 2) ff_add_pair(r6[i], r6[i + 1], o6[i], o6[i + 1]);
    }
    if (NTB > 32) {
        const int tid = threadIdx.x;
        if ((tid & 31) == 0) {
#pragma unroll
            for (int i = 0; i < 6; i++) scratch[(tid >> 5) * 6 + i] = r6[i];
        }
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < NTB / 32; w++)
#pragma unroll
                for (int i = 0; i < 6; i += 2) ff_add_pair(r6[i], r6[i + 1], scratch[w * 6 + i], scratch[w * 6 + i + 1]);
        }
        __syncthreads();
    }
}

// (h, l) = (ah, al) * b in float-float (the head's product error by fma).
__device__ __forceinline__ void ff_mul_f(float ah, float al, float b, float &h, float &l)
{
    const float p = __fmul_rn(ah, b);
    float e = __fmaf_rn(ah, b, -p);
    e = __fmaf_rn(al, b, e);
    h = __fadd_rn(p, e);
    l = __fsub_rn(e, __fsub_rn(h, p));
}

// (h, l) = (ah, al) * (bh, bl) in float-float.
__device__ __forceinline__ void ff_mul(float ah, float al, float bh, float bl, float &h, float &l)
{
    const float p = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    h = __fadd_rn(p, e);
    l = __fsub_rn(e, __fsub_rn(h, p));
}

// A double as float-float (exact when it came from one).
__device__ __forceinline__ void ff_from_double(double x, float &h, float &l)
{
    h = (float)x;
    l = (float)(x - (double)h);
}

// (h, l) = (ah, al)^2 in float-float.
__device__ __forceinline__ void ff_sqr(float ah, float al, float &h, float &l)
{
    const float p = __fmul_rn(ah, ah);
    float e = __fmaf_rn(ah, ah, -p);
    e = __fmaf_rn(__fmul_rn(2.f, ah), al, e);
    h = __fadd_rn(p, e);
    l = __fsub_rn(e, __fsub_rn(h, p));
}

// (h, l) = (ah, al) / b in float-float: head quotient, its remainder by fma,
// one correction term.
__device__ __forceinline__ void ff_div_f(float ah, float al, float b, float &h, float &l)
{
    const float rb = __frcp_rn(b);   // correctly rounded reciprocal, cheaper than a division
    const float q1 = __fmul_rn(ah, rb);
    const float r = __fadd_rn(__fmaf_rn(-q1, b, ah), al);
    const float q2 = __fmul_rn(r, rb);
    h = __fadd_rn(q1, q2);
    l = __fsub_rn(q2, __fsub_rn(h, q1));
}

// Inclusive segmented scan over the NT threads of float-float values:
// (x, y) is one float-float number, and with K == 2 (z, w) a second one.
template <int K>
__device__ __forceinline__ float4 seg_scan_ff(int flag, float4 v, float4 *P, float4 *wsum, int *wflag)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int f = flag;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const float ux = __shfl_up_sync(0xffffffffu, v.x, off);
        const float uy = __shfl_up_sync(0xffffffffu, v.y, off);
        float uz = 0.f, uw = 0.f;
        if (K == 2) {
            uz = __shfl_up_sync(0xffffffffu, v.z, off);
            uw = __shfl_up_sync(0xffffffffu, v.w, off);
        }
        const int uf = __shfl_up_sync(0xffffffffu, f, off);
        if (lane >= off) {
            if (!f) {
                ff_add_pair(v.x, v.y, ux, uy);
                if (K == 2) ff_add_pair(v.z, v.w, uz, uw);
            }
            f |= uf;
        }
    }
    if (lane == 31) {
        wsum[w] = v;
        wflag[w] = f;
    }
    __syncthreads();
    if (w == 0) {
        const int NW = NT / 32;
        float4 x = lane < NW ? wsum[lane] : make_float4(0.f, 0.f, 0.f, 0.f);
        int g = lane < NW ? wflag[lane] : 1;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const float ux = __shfl_up_sync(0xffffffffu, x.x, off);
            const float uy = __shfl_up_sync(0xffffffffu, x.y, off);
            float uz = 0.f, uw = 0.f;
            if (K == 2) {
                uz = __shfl_up_sync(0xffffffffu, x.z, off);
                uw = __shfl_up_sync(0xffffffffu, x.w, off);
            }
            const int ug = __shfl_up_sync(0xffffffffu, g, off);
            if (lane >= off) {
                if (!g) {
                    ff_add_pair(x.x, x.y, ux, uy);
                    if (K == 2) ff_add_pair(x.z, x.w, uz, uw);
                }
                g |= ug;
            }
        }
        if (lane < NW) wsum[lane] = x;
    }
    __syncthreads();
    if (w > 0 && !f) {
        const float4 c = wsum[w - 1];
        ff_add_pair(v.x, v.y, c.x, c.y);
        if (K == 2) ff_add_pair(v.z, v.w, c.z, c.w);
    }
    P[threadIdx.x] = v;
    __syncthreads();
    return v;
}

// ------------------------------------------------- integrand, batched over S
template <typename T, int KIND, int DIMB, int S>
struct BatchEval {
    static __device__ __forceinline__ void run(const VgParams &prm, const VgF32Consts &kc,
                                               const float *tab, int nterm, int dim,
                                               const T (&x)[S][DIMB], T (&f)[S])
    {
#pragma unroll
        for (int k = 0; k < S; k++) {
            if (sizeof(T) == 8) f[k] = (T)vg_eval_f64<KIND, DIMB>(prm, dim, (const double *)x[k]);
            else f[k] = (T)vg_eval_f32<KIND, DIMB>(kc, tab, nterm, dim, (const float *)x[k]);
        }
    }
};

// Ridge in FP32: all S samples of the thread share each pass over the M term
// offsets v_j (one shared-memory load feeds 4*S exponentials).
template <int DIMB, int S>
struct BatchEval<float, VG_F_RIDGE, DIMB, S> {
    static __device__ __forceinline__ void run(const VgParams &prm, const VgF32Consts &kc,
                                               const float *tab, int nterm, int dim,
                                               const float (&x)[S][DIMB], float (&f)[S])
    {
        float E0[S], w[S], a0[S], a1[S];
#pragma unroll
        for (int k = 0; k < S; k++) {
            float m = 0.f;
#pragma unroll
            for (int d = 0; d < DIMB; d++)
                if (d < dim) m += x[k][d];
            m *= kc.c[3];
            float R = 0.f;
#pragma unroll
            for (int d = 0; d < DIMB; d++)
                if (d < dim) {
                    float t = x[k][d] - m;
                    R = fmaf(t, t, R);
                }
            E0[k] = -kc.c[0] * R;
            w[k] = m * kc.c[1];
            a0[k] = 0.f;
            a1[k] = 0.f;
        }
        const float4 *t4 = reinterpret_cast<const float4 *>(tab);
        const int n4 = nterm >> 2;
        const float rc = 1.f / kc.c[4];
        unsigned int nt = 0;
#pragma unroll
        for (int k = 0; k < S; k++) {
            // This sample's window of groups of 4 terms that can be nonzero: a
            // term with E0 - (w - v_j)^2 < -127 is exactly zero
            // (ex2.approx.ftz flushes it), so skipping whole groups of such
            // terms leaves the sum -- and f -- bit-identical.
            int qlo = n4, qhi = 0;
            const float rad2 = E0[k] + 127.f;
            if (rad2 > 0.f) {
                const float delta = sqrtf(rad2) * 1.0001f + 1e-3f;
                int jlo = (int)floorf((w[k] - delta) * rc - 0.5f) - 1;
                int jhi = (int)ceilf((w[k] + delta) * rc - 0.5f) + 1;
                jlo = jlo < 0 ? 0 : jlo;
                jhi = jhi > nterm - 1 ? nterm - 1 : jhi;
                qlo = jlo >> 2;
                qhi = min(n4, (jhi >> 2) + 1);
            }
            nt += qhi > qlo ? (unsigned int)(4 * (qhi - qlo)) : 0u;
            float b0 = 0.f, b1 = 0.f, b2 = 0.f, b3 = 0.f;
            const float wk = w[k], ek = E0[k];
#pragma unroll 2
            for (int q = qlo; q < qhi; q++) {
                const float4 v = t4[q];
                const float d0 = wk - v.x, d1 = wk - v.y, d2 = wk - v.z, d3 = wk - v.w;
                b0 += vg_ex2(fmaf(-d0, d0, ek));
                b1 += vg_ex2(fmaf(-d1, d1, ek));
                b2 += vg_ex2(fmaf(-d2, d2, ek));
                b3 += vg_ex2(fmaf(-d3, d3, ek));
            }
            for (int j = n4 << 2; j < nterm; j++) {
                const float d0 = wk - tab[j];
                b0 += vg_ex2(fmaf(-d0, d0, ek));
            }
            a0[k] = b0 + b1;
            a1[k] = b2 + b3;
        }
        if (prm.term_count != nullptr) {   // instrumentation: terms evaluated
            const unsigned int tot = __reduce_add_sync(0xffffffffu, nt);
            if ((threadIdx.x & 31) == 0) atomicAdd(prm.term_count, (unsigned long long)tot);
        }
#pragma unroll
        for (int k = 0; k < S; k++) f[k] = kc.c[2] * (a0[k] + a1[k]);
    }
};

// a / b: exact in FP64 mode (reference parity), a reciprocal multiply refined
// by one Newton step in FP32 mode (GB300 FP64 division is expensive).
template <typename T>
__device__ __forceinline__ double vg_div(double a, double b)
{
    if (sizeof(T) == 8) return __ddiv_rn(a, b);
    double r = (double)__frcp_rn((float)b);
    r = fma(r, fma(-b, r, 1.0), r);
    return a * r;
}

// One sample's y along one axis and its map increment index (pyx:1738-1742,
// 325-330): yd = (y0 + u) / nstrat, yn = yd * K, iy = floor(yn); yfl = the
// floor as T.  FP32 mode: the reciprocal of nstrat and K as float are given,
// the floor's integer comes from the float's bits (0 <= yn < 2^23): no
// int <-> float conversion per sample (those share GB300's slow FP64 pipe).
template <typename T>
__device__ __forceinline__ int sample_y(int y0, float y0f, T u, int ns, float rns, int K, float Kf, T &yd,
                                        T &yn, T &yfl)
{
    int iy;
    if (sizeof(T) == 8) {
        yd = (T)__ddiv_rn(__dadd_rn((double)y0, (double)u), (double)ns);
        yn = (T)__dmul_rn((double)yd, (double)K);
        iy = (int)floor((double)yn);
        yfl = (T)iy;
    } else {
        yd = (T)__fmul_rn(__fadd_rn(y0f, (float)u), rns);
        yn = (T)__fmul_rn((float)yd, Kf);
        const float fl = floorf((float)yn);
        iy = __float_as_int(fl + 8388608.f) - 0x4B000000;
        yfl = (T)fl;
    }
    return iy;
}

// Training bin of a sample along one axis: its increment, or 0xffff when y
// is 0 or 1 (add_training_data skips those, pyx:460).
template <typename T>
__device__ __forceinline__ unsigned short sample_bin(T yd, int iy, int K)
{
    return (unsigned short)((yd > (T)0 && yd < (T)1 && iy < K) ? iy : 0xffff);
}

// adapt_to_errors: the hypercube's |variance| into the training histogram
// at its last sample's bins, count 1 (pyx:2187-2193).
__device__ __forceinline__ void train_hcube(const IterArgs &a, const unsigned short *bins, double v)
{
    for (int d = 0; d < a.dim; d++) {
        const unsigned short b = bins[d];
        if (b == 0xffff) continue;
        atomicAdd(&a.sum_f[d * a.ldi + b], v);
        atomicAdd(&a.n_f[d * a.ldi + b], 1ull);
    }
}

// The training bins of hypercube h's last sample, regenerated from its
// uniforms exactly as the tile kernels form them (for hypercubes that the
// finalize merges across tiles).
template <typename T>
static __device__ void last_sample_bins(const IterArgs &a, int64_t h, unsigned short *bins)
{
    const int dim = a.dim;
    const int64_t ig = a.offsets[h] + a.neval_h[h] - 1;
    T u[VG_MAX_DIM];
    if (a.u != nullptr) {
        for (int d = 0; d < dim; d++) u[d] = (T)a.u[ig * dim + d];
    } else {
        VgUniform<T>::template draw<VG_MAX_DIM>(a.seed, a.stream, a.itn, (uint64_t)ig, dim, u);
    }
    int64_t hh = h;
    for (int d = 0; d < dim; d++) {
        const int ns = a.nstrat[d];
        const int y0 = (int)(hh % ns);
        hh /= ns;
        const int K = a.ninc[d];
        T yd, yn, yfl;
        const int iy = sample_y<T>(y0, (float)y0, u[d], ns, 1.f / (float)ns, K, (float)K, yd, yn, yfl);
        bins[d] = sample_bin<T>(yd, iy, K);
    }
}

// FP32 mode: the hypercube whose first piece is the tail record of tile t,
// merged in float-float with its pieces in the following tiles (Chan et
// al.'s parallel-variance update: Q = Q1 + Q2 + (m2 - m1)^2 n1 n2 / (n1 +
// n2)).  Adds its mean S + D and variance (nQ - D^2)/(n - 1) to (m, v), sets
// its sigf and adds it to s, and trains it under adapt_to_errors.
static __device__ __noinline__ void merge_cut_ff(const IterArgs &a, int64_t t, int64_t ntiles, float &mh, float &ml, float &vh_,
                             float &vl_, float &sh, float &sl)
{
    const TileRec r = a.recs[2 * t + 1];
    if (r.h < 0) return;
    float n = (float)r.pad, Sh, Sl, Qh, Ql, Dh, Dl;
    ff_unpack(r.S, Sh, Sl);
    ff_unpack(r.Q, Qh, Ql);
    ff_unpack(r.D, Dh, Dl);
    bool big = !(fabsf(Qh) < 1e30f);
    for (int64_t t2 = t + 1; t2 < ntiles; t2++) {
        const TileRec q = a.recs[2 * t2];
        if (q.h != r.h) break;
        const float qn = (float)q.pad, n2 = n + qn;
        float qSh, qSl, qQh, qQl, qDh, qDl;
        ff_unpack(q.S, qSh, qSl);
        ff_unpack(q.Q, qQh, qQl);
        ff_unpack(q.D, qDh, qDl);
        big |= !(fabsf(qQh) < 1e30f);
        float m1h, m1l, m2h, m2l, wh, wl, ddh, ddl, th, tl;
        ff_div_f(Sh, Sl, n, m1h, m1l);
        ff_div_f(qSh, qSl, qn, m2h, m2l);
        ff_add_pair(m2h, m2l, -m1h, -m1l);
        const float wph = __fmul_rn(n, qn);
        const float wpl = __fmaf_rn(n, qn, -wph);
        ff_div_f(wph, wpl, n2, wh, wl);
        ff_sqr(m2h, m2l, ddh, ddl);
        ff_mul(ddh, ddl, wh, wl, th, tl);
        ff_add_pair(Qh, Ql, qQh, qQl);
        ff_add_pair(Qh, Ql, th, tl);
        ff_add_pair(Sh, Sl, qSh, qSl);
        ff_add_pair(Dh, Dl, qDh, qDl);
        n = n2;
        if (!q.spans) break;
    }
    float vh, vl;
    if (!big) {
        float nqh, nql, d2h, d2l;
        ff_mul_f(Qh, Ql, n, nqh, nql);
        ff_sqr(Dh, Dl, d2h, d2l);
        ff_add_pair(nqh, nql, -d2h, -d2l);
        ff_div_f(nqh, nql, n - 1.f, vh, vl);
    } else {   // squares beyond the float range: this hypercube in FP64
        const double Q = vg_ff_value(Qh, Ql), D = vg_ff_value(Dh, Dl), nd = (double)n;
        const double v = vg_div<float>(__dsub_rn(__dmul_rn(nd, Q), __dmul_rn(D, D)), nd - 1.0);
        vh = (float)v;
        vl = (float)(v - (double)vh);
    }
    if (a.train_hc) {   // adapt_to_errors: train at the hypercube's last sample
        unsigned short b[VG_MAX_DIM];
        last_sample_bins<float>(a, r.h, b);
        train_hcube(a, b, fabs(vg_ff_value(vh, vl)));
    }
    ff_add_pair(Sh, Sl, Dh, Dl);
    ff_add_pair(mh, ml, Sh, Sl);
    ff_add_pair(vh_, vl_, vh, vl);
    if (a.adaptive) {
        const float av = fabsf(vh);
        const float sg = av > 0.f ? vg_ex2_approx((float)a.beta_half * vg_lg2_approx(av)) : 0.f;
        a.sigf[r.h] = (double)sg;
        vg_ff_add(sh, sl, sg);
    }
}

// FP32 mode, rare path: a hypercube whose squared deviations leave the float
// range, finished in FP64.  Returns its (mean, variance, sigf) contributions
// and stores its sigf.
// (With want_var, the third value is |variance| instead: adapt_to_errors.)
static __device__ __noinline__ double3 finish_f64(double Sx, double Dx, double Qx, int nin, double beta_half,
                                                  int adaptive, double *sigf_h, int want_var)
{
    const double nd = (double)nin;
    const double vh = vg_div<float>(__dsub_rn(__dmul_rn(nd, Qx), __dmul_rn(Dx, Dx)), __dsub_rn(nd, 1.));
    double sg = 0.0;
    if (adaptive) {
        sg = vg_pow_fast(fabs(vh), beta_half);
        *sigf_h = sg;
    }
    return make_double3(__dadd_rn(Sx, Dx), vh, want_var ? fabs(vh) : sg);
}

// FP32 mode: the (x_node, inc) table of the grid in FP32, entry K of each
// axis = (grid[K], inc[K-1]) -- built once per iteration by the allocation so
// the tile CTAs copy it instead of converting FP64 nodes themselves.
__device__ __forceinline__ void build_tablef(const IterArgs &a, int64_t first, int64_t stride)
{
    const int W = a.maxK + 1;
    for (int64_t i = first; i < (int64_t)a.dim * W; i += stride) {
        const int d = (int)(i / W), j = (int)(i % W);
        const int K = a.ninc[d];
        float2 e = make_float2(0.f, 1.f);
        if (j < K) e = make_float2((float)a.grid[d * a.ldg + j], (float)a.inc[d * a.ldi + j]);
        else if (j == K) e = make_float2((float)a.grid[d * a.ldg + K], (float)a.inc[d * a.ldi + K - 1]);
        a.tablef[i] = e;
    }
}

// ------------------------------------------------------------------ kernel
// The work of one CTA: reduction modes take tiles first, first + stride, ...
// (static, deterministic); evaluation-only modes take tiles from the atomic
// counter.  The CTA's partial sums go to a.parts[part_slot].  Called by the
// grid-wide tile_kernel (first = blockIdx.x, stride = gridDim.x) and by the
// batched kernel, where G CTAs share an integral (rank, G, rank).
template <typename T, int MODE, int KIND, int DIMB, int S>
__device__ __forceinline__ void tile_body(const IterArgs &a, const VgParams &prm, unsigned char *smem,
                                          int64_t first, int64_t stride, int64_t part_slot)
{
    typedef typename GridEntry<T>::type GE;
    constexpr int TT = NT * S;
    constexpr int KSUB = TT / BASE_TILE;   // base tiles per tile
    const int dim = a.dim;
    const int tid = threadIdx.x;
    constexpr int NEED_RED = (MODE == MODE_REDUCE || MODE == MODE_FUSED || MODE == MODE_REDUCE_KEPT);
    const int use_bins = NEED_RED && (a.train || a.train_hc);   // per-sample bins in shared memory
    const SmemPlan sp = smem_plan<T>(dim, a.maxK, TT, a.table_smem, a.hist_smem, a.tab_len,
                                     use_bins, NEED_RED);
    GE *table = (GE *)(smem + sp.table);
    T *hsum = (T *)(smem + sp.hsum);
    unsigned int *hcnt = (unsigned int *)(smem + sp.hcnt);
    unsigned short *sbins = (unsigned short *)(smem + sp.bins);
    int *win_off = (int *)(smem + sp.win_off);
    int *win_n = (int *)(smem + sp.win_n);
    float *win_w = (float *)(smem + sp.win_w);   // FP32 mode: dv_y / neval_h of the window's hypercubes
    double *seg_S = (double *)(smem + sp.seg_S);
    int *keyF = (int *)(smem + sp.keyF);
    int *keyL = (int *)(smem + sp.keyL);
    double2 *Pv = (double2 *)(smem + sp.P);
    VgKSum *red = (VgKSum *)(smem + sp.red);
    float *itab = (float *)(smem + sp.itab);
    double2 *wsum = (double2 *)red;   // scan scratch (aliases red; used apart)
    int *wflag = (int *)(red + NT / 32 + 1);
    __shared__ int64_t s_tile;

    const int64_t N = a.stats->neval;
    const int64_t ntiles = (N + TT - 1) / TT;
    const int64_t nbase = (N + BASE_TILE - 1) / BASE_TILE;
    if (a.stats->ntiles == 0) return;   // allocation failed: nothing to do

    // ---- per-CTA setup: grid table, histogram, integrand constants
    if (a.table_smem) {
        if (sizeof(T) == 4) {   // FP32 mode: copy the float table built by the allocation
            const int n = dim * (a.maxK + 1);
            const float2 *src = a.tablef;
            float2 *dst = reinterpret_cast<float2 *>(table);
            for (int i = tid; i < n; i += NT) dst[i] = src[i];
        } else {
            for (int d = 0; d < dim; d++) {
                const int K = a.ninc[d];
                for (int i = tid; i <= K; i += NT) {
                    GE e;
                    if (i < K) {
                        e.x = (T)a.grid[d * a.ldg + i];
                        e.y = (T)a.inc[d * a.ldi + i];
                    } else {
                        e.x = (T)a.grid[d * a.ldg + K];
                        e.y = (T)a.inc[d * a.ldi + K - 1];
                    }
                    table[(size_t)d * (a.maxK + 1) + i] = e;
                }
            }
        }
    }
    if (use_bins && a.hist_smem) {
        for (int i = tid; i < dim * a.maxK; i += NT) {
            hsum[i] = (T)0;
            hcnt[i] = 0u;
        }
    }
    VgF32Consts kc;
    if ((MODE == MODE_FUSED || MODE == MODE_EVAL) && sizeof(T) == 4) {
        kc = vg_prepare_f32<KIND>(prm, dim);
        vg_fill_table_f32<KIND>(prm, dim, itab, kc);
    } else {
        for (int i = 0; i < 8; i++) kc.c[i] = 0.f;
    }
    const double dv_y = a.dv_y;
    const float dv_yf = (float)a.dv_y;
    const double beta_half = a.beta_half;
    const float beta_half_f = (float)a.beta_half;
    float Kf[DIMB], rstrat[DIMB];   // FP32 mode: per-axis constants
#pragma unroll
    for (int d = 0; d < DIMB; d++) {
        Kf[d] = d < dim ? (float)a.ninc[d] : 1.f;
        rstrat[d] = d < dim ? 1.f / (float)a.nstrat[d] : 1.f;
    }
    int nan_local = 0;
    // per-thread running sums over every hypercube this thread finalises
    double acc_m = 0.0, acc_v = 0.0, acc_s = 0.0;
    // FP32 mode: the same running sums in float-float, folded in at the end
    float am_h = 0.f, am_l = 0.f, av_h = 0.f, av_l = 0.f, as_h = 0.f, as_l = 0.f;
    int used64 = 0;   // FP32 mode: a hypercube went through the FP64 fallback
    // The running sums -> one compensated block reduction in a fixed order ->
    // a.parts[slot]; the sums restart from zero.
    auto emit_partial = [&](int64_t slot) {
        __syncthreads();
        if constexpr (sizeof(T) == 4) {
            // float-float block reduction (FP32 pipe); the rare FP64
            // finishes are folded in first
            if (used64) {
                float h = (float)acc_m;
                ff_add_pair(am_h, am_l, h, (float)(acc_m - (double)h));
                h = (float)acc_v;
                ff_add_pair(av_h, av_l, h, (float)(acc_v - (double)h));
                h = (float)acc_s;
                ff_add_pair(as_h, as_l, h, (float)(acc_s - (double)h));
            }
            float r6[6] = {am_h, am_l, av_h, av_l, as_h, as_l};
            ff_block_reduce6<NT>(r6, reinterpret_cast<float *>(red));
            if (tid == 0) {   // float-float partials, packed
                TilePart p;
                p.mean = VgKSum{ff_pack(r6[0], r6[1]), 0.0};
                p.var = VgKSum{ff_pack(r6[2], r6[3]), 0.0};
                p.sigf = VgKSum{ff_pack(r6[4], r6[5]), 0.0};
                a.parts[slot] = p;
            }
            am_h = am_l = av_h = av_l = as_h = as_l = 0.f;
            if (used64) acc_m = acc_v = acc_s = 0.0;
            used64 = 0;
        } else {
            const VgKSum m = vg_block_ksum<NT>(VgKSum{acc_m, 0.0}, red);
            const VgKSum v = vg_block_ksum<NT>(VgKSum{acc_v, 0.0}, red);
            const VgKSum sg = vg_block_ksum<NT>(VgKSum{acc_s, 0.0}, red);
            if (tid == 0) {
                TilePart p;
                p.mean = m;
                p.var = v;
                p.sigf = sg;
                a.parts[slot] = p;
            }
            acc_m = acc_v = acc_s = 0.0;
        }
        __syncthreads();
    };
    int64_t next_static = first;

    for (;;) {
        __syncthreads();
        int64_t tile;
        if (NEED_RED) {
            // reduction modes: fixed tile -> CTA assignment, so the per-CTA
            // partial sums (and hence the result) are deterministic
            tile = next_static;
            next_static += stride;
        } else {
            // evaluation-only modes: dynamic tiles for load balance
            if (tid == 0) s_tile = (int64_t)atomicAdd(a.counter, 1ull);
            __syncthreads();
            tile = s_tile;
        }
        if (tile >= ntiles) break;
        const int64_t tile_start = tile * (int64_t)TT;
        const int tile_len = (int)min((int64_t)TT, N - tile_start);
        const int64_t h0 = a.tile_h0[tile * KSUB];
        const int64_t bnext = (tile + 1) * KSUB;            // base tile after this tile
        const int64_t hnext = bnext < nbase ? a.tile_h0[bnext] : a.H;
        const int64_t hlast = (hnext < a.H) ? hnext : a.H - 1;
        const int nwin = (int)(hlast - h0 + 1);
        if (nwin < 1 || nwin > TT) {   // impossible while every count is >= 2
            if (tid == 0) a.stats->status = VG_ERR_UNSUPPORTED;
            break;
        }
        for (int k = tid; k <= nwin; k += NT) {
            int64_t h = h0 + k;
            int64_t o = (h <= a.H) ? a.offsets[h] : N;
            int64_t r = o - tile_start;
            win_off[k] = (int)(r < 0 ? 0 : (r > tile_len ? tile_len : r));
            if (k < nwin) {
                win_n[k] = a.neval_h[h];
                if (sizeof(T) == 4) win_w[k] = dv_yf / (float)win_n[k];
            }
        }
        __syncthreads();

        // ---- pass 0: draw, map, evaluate the thread's samples
        const int li0 = tid * S;
        int nmine = tile_len - li0;
        nmine = nmine < 0 ? 0 : (nmine > S ? S : nmine);
        int lh = 0;
        if (nmine > 0) {
            int lo = 0, hi = nwin - 1;   // last k with win_off[k] <= li0
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (win_off[mid] <= li0) lo = mid;
                else hi = mid - 1;
            }
            lh = lo;
        }
        int y0[DIMB];
        float y0f[DIMB];   // FP32 mode: the stratum coordinates as floats (no per-sample conversion)
        if (a.H <= 0x7fffffff) {   // 32-bit mixed-radix decode
            int hh = (int)(h0 + lh);
#pragma unroll
            for (int d = 0; d < DIMB; d++) {
                if (d < dim) {
                    const int q = hh / a.nstrat[d];
                    y0[d] = hh - q * a.nstrat[d];
                    hh = q;
                } else {
                    y0[d] = 0;
                }
            }
        } else {
            int64_t hh = h0 + lh;
#pragma unroll
            for (int d = 0; d < DIMB; d++) {
                if (d < dim) {
                    int64_t q = hh / a.nstrat[d];
                    y0[d] = (int)(hh - q * a.nstrat[d]);
                    hh = q;
                } else {
                    y0[d] = 0;
                }
            }
        }
#pragma unroll
        for (int d = 0; d < DIMB; d++) y0f[d] = (float)y0[d];
        T xs[S][DIMB];
        T wg[S];   // sampler weight (FP32 in the FP32 mode)
        float jn[S];   // FP32 mode: wgt * neval_h = jac * dv_y
        int lhs[S];
        int cur = lh;
        // the uniforms of all the thread's samples first (into xs): the
        // draws do not depend on the hypercube walk below, so the S samples'
        // Philox rounds interleave instead of waiting on one another
        // (REDUCE_KEPT reads the kept Jacobians instead)
#pragma unroll
        for (int k = 0; k < S && MODE != MODE_REDUCE_KEPT; k++) {
#pragma unroll
            for (int d = 0; d < DIMB; d++) xs[k][d] = (T)0.5;
            if (k < nmine) {
                const int64_t ig = tile_start + li0 + k;
                if (a.u != nullptr) {
#pragma unroll
                    for (int d = 0; d < DIMB; d++)
                        if (d < dim) xs[k][d] = (T)a.u[ig * dim + d];
                } else {
                    VgUniform<T>::template draw<DIMB>(a.seed, a.stream, a.itn, (uint64_t)ig, dim, xs[k]);
#pragma unroll
                    for (int d = 0; d < DIMB; d++)
                        if (d >= dim) xs[k][d] = (T)0.5;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < S; k++) {
            lhs[k] = cur;
            wg[k] = 0.0;
            if (k < nmine) {
                const int li = li0 + k;
                while (li >= win_off[cur + 1]) {   // next hypercube: mixed-radix increment
                    cur++;
                    int carry = 1;
#pragma unroll
                    for (int d = 0; d < DIMB; d++) {
                        if (d < dim && carry) {
                            if (++y0[d] < a.nstrat[d]) {
                                carry = 0;
                                y0f[d] += 1.f;
                            } else {
                                y0[d] = 0;
                                y0f[d] = 0.f;
                            }
                        }
                    }
                }
                lhs[k] = cur;
                const int64_t ig = tile_start + li;
                const int nh = win_n[cur];
                T jac = (T)1;
                T yv[DIMB];
                unsigned short kbin[DIMB];   // MODE_POINTS: the bins to keep
                if constexpr (MODE == MODE_REDUCE_KEPT) {
                    jac = ((const T *)a.keep_jac)[ig];
                    if (use_bins) {   // rows of 4 bins, one 8-byte load each
                        const uint2 *src = reinterpret_cast<const uint2 *>(a.keep_bins + ig * a.keep_bstride);
                        for (int q = 0; q < dim; q += 4) {
                            const uint2 v = src[q >> 2];
                            const unsigned short b4[4] = {(unsigned short)(v.x & 0xffffu), (unsigned short)(v.x >> 16),
                                                          (unsigned short)(v.y & 0xffffu), (unsigned short)(v.y >> 16)};
                            for (int r = 0; r < 4 && q + r < dim; r++) sbins[(li0 + k) * dim + q + r] = b4[r];
                        }
                    }
                }
#pragma unroll
                for (int d = 0; d < DIMB; d++) {
                    if (d >= dim || MODE == MODE_REDUCE_KEPT) continue;
                    const int K = a.ninc[d];
                    T yd, yn, yfl;
                    const int iy = sample_y<T>(y0[d], y0f[d], xs[k][d], a.nstrat[d], rstrat[d], K, Kf[d], yd, yn, yfl);
                    const T dy = yn - yfl;
                    yv[d] = yd;
                    const int clamp = iy >= K;
                    const int ie = clamp ? K : iy;
                    GE e;
                    if (a.table_smem) {
                        e = table[(size_t)d * (a.maxK + 1) + ie];
                    } else if (sizeof(T) == 4) {
                        const float2 t2 = a.tablef[(size_t)d * (a.maxK + 1) + ie];
                        e.x = (T)t2.x;
                        e.y = (T)t2.y;
                    } else if (!clamp) {
                        e.x = (T)a.grid[d * a.ldg + ie];
                        e.y = (T)a.inc[d * a.ldi + ie];
                    } else {
                        e.x = (T)a.grid[d * a.ldg + K];
                        e.y = (T)a.inc[d * a.ldi + K - 1];
                    }
                    if (sizeof(T) == 8) {
                        xs[k][d] = clamp ? e.x
                                         : (T)__dadd_rn((double)e.x, __dmul_rn((double)e.y, (double)dy));
                        jac = (T)__dmul_rn((double)jac, __dmul_rn((double)e.y, (double)K));
                    } else {
                        xs[k][d] = clamp ? e.x : (T)fmaf((float)e.y, (float)dy, (float)e.x);
                        jac = (T)((float)jac * ((float)e.y * Kf[d]));
                    }
                    if (use_bins) sbins[(li0 + k) * dim + d] = sample_bin<T>(yd, iy, K);
                    if (MODE == MODE_POINTS) kbin[d] = sample_bin<T>(yd, iy, K);
                }
                if (MODE == MODE_POINTS && a.keep_bins) {   // rows of 4 bins, one 8-byte store each
                    uint2 *dst = reinterpret_cast<uint2 *>(a.keep_bins + ig * a.keep_bstride);
#pragma unroll
                    for (int q = 0; q < DIMB; q += 4) {
                        if (q >= dim) break;
                        unsigned int w4[4];
#pragma unroll
                        for (int r = 0; r < 4; r++) w4[r] = (q + r < dim && q + r < DIMB) ? kbin[q + r] : 0xffffu;
                        dst[q >> 2] = make_uint2(w4[0] | (w4[1] << 16), w4[2] | (w4[3] << 16));
                    }
                }
                // weight, pyx:1748-1749: jac *= dv_y / neval_hcube
                if (sizeof(T) == 8) wg[k] = (T)__dmul_rn((double)jac, __ddiv_rn(dv_y, (double)nh));
                else {
                    wg[k] = (T)((float)jac * win_w[cur]);
                    jn[k] = (float)jac * dv_yf;   // wgt * neval_h, for fdv2
                }
                if (MODE == MODE_POINTS) {
                    T *xo = (T *)a.x_out;
#pragma unroll
                    for (int d = 0; d < DIMB; d++)
                        if (d < dim) xo[ig * dim + d] = xs[k][d];
                    if (a.y_out) {
                        T *yo = (T *)a.y_out;
#pragma unroll
                        for (int d = 0; d < DIMB; d++)
                            if (d < dim) yo[ig * dim + d] = yv[d];
                    }
                    if (a.wgt_out) a.wgt_out[ig] = (double)wg[k];
                    if (a.hc_out) a.hc_out[ig] = h0 + cur;
                    if (a.keep_jac) ((T *)a.keep_jac)[ig] = jac;
                }
            }
        }
        if (MODE == MODE_POINTS) continue;

        T fv[S];
        if (MODE == MODE_FUSED || MODE == MODE_EVAL) {
            BatchEval<T, KIND, DIMB, S>::run(prm, kc, itab, a.tab_len, dim, xs, fv);
            if (MODE == MODE_EVAL) {
#pragma unroll
                for (int k = 0; k < S; k++)
                    if (k < nmine) a.f_eval[tile_start + li0 + k] = (float)fv[k];
                continue;
            }
        } else {
#pragma unroll
            for (int k = 0; k < S; k++) {
                fv[k] = (T)0;
                if (k < nmine) {
                    const int64_t ig = tile_start + li0 + k;
                    fv[k] = a.f_f64 ? (T)((const double *)a.f_in)[ig]
                                    : (T)((const float *)a.f_in)[ig];
                }
            }
        }
        T wf[S];   // wgt * f, pyx:2143 (FP32 in the FP32 mode)
#pragma unroll
        for (int k = 0; k < S; k++) {
            wf[k] = (T)0;
            if (k >= nmine) continue;
            if (fv[k] != fv[k]) nan_local = 1;
            double w1 = 0.0;
            float wf32 = 0.f;
            if (sizeof(T) == 8) {
                w1 = __dmul_rn((double)wg[k], (double)fv[k]);
                wf[k] = (T)w1;
            } else {
                wf32 = (float)wg[k] * (float)fv[k];
                wf[k] = (T)wf32;
            }
            if (use_bins && a.train) {
                // fdv2 = (wgt*f*neval)^2, pyx:2173; |fdv2| into the bins, pyx:460-463
                T fd;
                if (sizeof(T) == 8) {
                    const double t1 = __dmul_rn(w1, (double)win_n[lhs[k]]);
                    fd = (T)__dmul_rn(t1, t1);
                } else {
                    const float t1 = (float)fv[k] * jn[k];
                    fd = (T)(t1 * t1);
                }
                for (int d = 0; d < dim; d++) {
                    const unsigned short b = sbins[(li0 + k) * dim + d];
                    if (b == 0xffff) continue;
                    if (a.hist_smem) {
                        atomicAdd(&hsum[d * a.maxK + b], fd);
                        atomicAdd(&hcnt[d * a.maxK + b], 1u);
                    } else {
                        atomicAdd(&a.sum_f[d * a.ldi + b], (double)fd);
                        atomicAdd(&a.n_f[d * a.ldi + b], 1ull);
                    }
                }
            }
        }

        if constexpr (sizeof(T) == 4) {
        // ---- FP32 mode: the tile's reduction in float-float (TwoSum/TwoProd,
        // about 2^-48 relative), FP64 once per hypercube -- GB300 runs FP64 at
        // a small fraction of the FP32 rate.  Same two passes as below.
        const int has = nmine > 0;
        const int fk = has ? lhs[0] : 0x7fffffff;
        const int lk = has ? lhs[nmine - 1] : 0x7fffffff;
        float fh = 0.f, fl = 0.f, lh2 = 0.f, ll = 0.f;
#pragma unroll
        for (int k = 0; k < S; k++) {
            if (k < nmine && lhs[k] == fk) vg_ff_add(fh, fl, (float)wf[k]);
            if (k < nmine && lhs[k] == lk) vg_ff_add(lh2, ll, (float)wf[k]);
        }
        keyF[tid] = fk;
        keyL[tid] = lk;
        __syncthreads();
        const int prevL = tid > 0 ? keyL[tid - 1] : -1;
        const int nextF = tid < NT - 1 ? keyF[tid + 1] : -2;
        const int flag = (tid == 0) || (lk != prevL);
        float4 *Pf = reinterpret_cast<float4 *>(Pv);
        float4 *wsf = reinterpret_cast<float4 *>(wsum);
        float2 *segf = reinterpret_cast<float2 *>(seg_S);
        const float4 Pi = seg_scan_ff<1>(flag, make_float4(lh2, ll, 0.f, 0.f), Pf, wsf, wflag);
        const int ends_last = has && (lk != nextF);
        if (has && lk != fk) {
            float ch = fh, cl = fl;
            if (tid > 0 && prevL == fk) ff_add_pair(ch, cl, Pf[tid - 1].x, Pf[tid - 1].y);
            segf[fk] = make_float2(ch, cl);
        }
        if (ends_last) segf[lk] = make_float2(Pi.x, Pi.y);
        __syncthreads();
        // per hypercube: mean S + D, variance (n Q - D^2) / (n - 1) and
        // sigf = |var|^(beta/2) (pyx:2174-2186), in float-float with an FP32
        // sigf; FP64 only where the squares leave the float range
        auto finish = [&](int64_t h, int nin, float Sh, float Sl, float Dh, float Dl, float Qh, float Ql,
                          int big, double Qbig) {
            if (big || !(fabsf(Qh) < 1e30f)) {
                const double3 r = finish_f64(vg_ff_value(Sh, Sl), vg_ff_value(Dh, Dl),
                                             __dadd_rn(vg_ff_value(Qh, Ql), Qbig), nin, beta_half,
                                             a.adaptive, a.sigf + h, a.train_hc);
                acc_m += r.x;
                acc_v += r.y;
                if (!a.train_hc) acc_s += r.z;
                used64 = 1;
                if (a.train_hc) train_hcube(a, sbins + (size_t)(win_off[(int)(h - h0) + 1] - 1) * dim, r.z);
                return;
            }
            const float fn = (float)nin;
            float mh = Sh, ml = Sl;
            ff_add_pair(mh, ml, Dh, Dl);
            ff_add_pair(am_h, am_l, mh, ml);
            float nqh, nql, d2h, d2l, vh, vl;
            ff_mul_f(Qh, Ql, fn, nqh, nql);
            ff_sqr(Dh, Dl, d2h, d2l);
            ff_add_pair(nqh, nql, -d2h, -d2l);
            ff_div_f(nqh, nql, fn - 1.f, vh, vl);
            ff_add_pair(av_h, av_l, vh, vl);
            if (a.adaptive) {
                const float av = fabsf(vh);
                const float sg = av > 0.f ? vg_ex2_approx(beta_half_f * vg_lg2_approx(av)) : 0.f;
                a.sigf[h] = (double)sg;
                vg_ff_add(as_h, as_l, sg);
            }
            if (a.train_hc)
                train_hcube(a, sbins + (size_t)(win_off[(int)(h - h0) + 1] - 1) * dim, fabs(vg_ff_value(vh, vl)));
        };
        // pass 2 over the thread's runs of equal hypercube, unrolled over the
        // S samples so that wf[] and lhs[] stay in registers
        float4 dq_first = make_float4(0.f, 0.f, 0.f, 0.f), dq_last = dq_first;   // (D, Q) float-float
        {
            int key = -1, nin = 1, big = 0, nguard = 0;
            bool is_first = false, is_last = false;
            float sh = 0.f, sl = 0.f, m_hi = 0.f, m_lo = 0.f, thr_f = 0.f;
            float dh_s = 0.f, dl_s = 0.f, qh = 0.f, ql = 0.f;
            double Qbig = 0.0;
#pragma unroll
            for (int k = 0; k < S; k++) {
                if (k >= nmine) continue;
                if (k == 0 || lhs[k] != key) {   // a run starts: its sum, mean and guard
                    key = lhs[k];
                    sh = 0.f;
                    sl = 0.f;
#pragma unroll
                    for (int j = k; j < S; j++)
                        if (j < nmine && lhs[j] == key) vg_ff_add(sh, sl, (float)wf[j]);
                    nin = win_off[key + 1] - win_off[key];
                    is_first = (key == fk);
                    is_last = (key == lk);
                    if (is_first || is_last) {
                        const float2 t2 = segf[key];
                        sh = t2.x;
                        sl = t2.y;
                    }
                    // mean m = S / nin as float-float
                    const float fn = (float)nin;
                    const float rn = __frcp_rn(fn);
                    m_hi = sh * rn;
                    m_lo = (__fadd_rn(fmaf(-m_hi, fn, sh), sl)) * rn;
                    thr_f = (float)VG_EPSILON * fabsf(m_hi);
                    dh_s = dl_s = qh = ql = 0.f;
                    nguard = 0;
                    big = 0;
                    Qbig = 0.0;
                }
                {
                    const float x = (float)wf[k];
                    const float s0 = __fsub_rn(x, m_hi);   // TwoSum(wf, -m_hi), then - m_lo
                    const float bb = __fsub_rn(s0, x);
                    float e0 = __fadd_rn(__fsub_rn(x, __fsub_rn(s0, bb)), __fsub_rn(-m_hi, bb));
                    e0 = __fsub_rn(e0, m_lo);
                    const float d = __fadd_rn(s0, e0);
                    e0 = __fsub_rn(e0, __fsub_rn(d, s0));
                    if (fabsf(d) < thr_f) {   // |dwf| < EPSILON |mean|, pyx:2156
                        nguard++;
                    } else {
                        if (fabsf(d) > 1e18f) {   // squares beyond the float range: FP64
                            const double dd = (double)d + (double)e0;
                            Qbig = __dadd_rn(Qbig, __dmul_rn(dd, dd));
                            big = 1;
                        } else {
                            const float p = __fmul_rn(d, d);
                            const float pe = __fadd_rn(fmaf(d, d, -p), __fmul_rn(2.f * d, e0));
                            ff_add_pair(qh, ql, p, pe);
                        }
                        ff_add_pair(dh_s, dl_s, d, e0);
                    }
                }
                const bool run_end = (k + 1 >= nmine) || lhs[k + 1 < S ? k + 1 : k] != key;
                if (run_end) {
                    if (nguard) ff_add_pair(qh, ql, (float)nguard * thr_f * thr_f, 0.f);
                    if (is_first) dq_first = make_float4(dh_s, dl_s, qh, ql);
                    if (is_last) dq_last = make_float4(dh_s, dl_s, qh, ql);
                    if (!is_first && !is_last)   // hypercube wholly inside this thread
                        finish(h0 + key, nin, sh, sl, dh_s, dl_s, qh, ql, big, Qbig);
                    else if (big) {   // rare: carry the FP64 part through the scan's head
                        if (is_first) dq_first.z = (float)((double)dq_first.z + Qbig);
                        else dq_last.z = (float)((double)dq_last.z + Qbig);
                    }
                }
            }
        }
        __syncthreads();
        const float4 Pq = seg_scan_ff<2>(flag, dq_last, Pf, wsf, wflag);
#pragma unroll
        for (int which = 0; which < 2; which++) {
            int key;
            float4 dq;
            if (which == 0) {
                if (!(has && lk != fk)) continue;
                key = fk;
                dq = dq_first;
                if (tid > 0 && prevL == fk) {
                    const float4 c = Pf[tid - 1];
                    ff_add_pair(dq.x, dq.y, c.x, c.y);
                    ff_add_pair(dq.z, dq.w, c.z, c.w);
                }
            } else {
                if (!ends_last) continue;
                key = lk;
                dq = Pq;
            }
            const int64_t h = h0 + key;
            const int nin = win_off[key + 1] - win_off[key];
            const int nh = win_n[key];
            const float2 sg2 = segf[key];
            const int64_t ostart = a.offsets[h];
            const bool starts_before = ostart < tile_start;
            const bool ends_after = ostart + nh > tile_start + tile_len;
            if (!starts_before && !ends_after) {
                finish(h, nin, sg2.x, sg2.y, dq.x, dq.y, dq.z, dq.w, 0, 0.0);
            } else {   // a piece of a hypercube cut by the tile: float-float record
                TileRec r;
                r.h = h;
                r.n = 0.0;
                r.S = ff_pack(sg2.x, sg2.y);
                r.Q = ff_pack(dq.z, dq.w);
                r.D = ff_pack(dq.x, dq.y);
                r.spans = (starts_before && ends_after) ? 1 : 0;
                r.pad = nin;
                a.recs[2 * tile + (starts_before ? 0 : 1)] = r;
            }
        }
        } else {
        // ---- pass 1: per-run sums of wf; segmented scan across threads
        const int has = nmine > 0;
        const int fk = has ? lhs[0] : 0x7fffffff;
        const int lk = has ? lhs[nmine - 1] : 0x7fffffff;
        double fsum = 0.0, lsum = 0.0;
#pragma unroll
        for (int k = 0; k < S; k++) {
            if (k < nmine && lhs[k] == fk) fsum += (double)wf[k];
            if (k < nmine && lhs[k] == lk) lsum += (double)wf[k];
        }
        keyF[tid] = fk;
        keyL[tid] = lk;
        __syncthreads();
        const int prevL = tid > 0 ? keyL[tid - 1] : -1;
        const int nextF = tid < NT - 1 ? keyF[tid + 1] : -2;
        const int flag = (tid == 0) || (lk != prevL);
        double2 Pi = seg_scan(flag, make_double2(lsum, 0.0), Pv, wsum, wflag);
        const double carry1 = (tid > 0 && prevL == fk && has) ? Pv[tid - 1].x : 0.0;
        const int ends_last = has && (lk != nextF);
        if (has && lk != fk) seg_S[fk] = fsum + carry1;
        if (ends_last) seg_S[lk] = Pi.x;
        __syncthreads();

        // ---- pass 2: deviations about the hypercube mean (pyx:2154-2171)
        double2 dq_first = make_double2(0.0, 0.0), dq_last = make_double2(0.0, 0.0);
        {
            int k = 0;
            while (k < nmine) {
                const int key = lhs[k];
                int k1 = k;
                double Sloc = 0.0;
                while (k1 < nmine && lhs[k1] == key) Sloc += (double)wf[k1++];
                const int nin = win_off[key + 1] - win_off[key];
                const bool is_first = (key == fk), is_last = (key == lk);
                const double Sseg = (is_first || is_last) ? seg_S[key] : Sloc;
                const double m = vg_div<T>(Sseg, (double)nin);
                const double thr = __dmul_rn(VG_EPSILON, fabs(m));
                double Dr = 0.0, Qr = 0.0;
                for (int q = k; q < k1; q++) {
                    const double dwf = __dsub_rn((double)wf[q], m);
                    if (fabs(dwf) < thr) {
                        Qr = __dadd_rn(Qr, __dmul_rn(thr, thr));
                    } else {
                        Qr = __dadd_rn(Qr, __dmul_rn(dwf, dwf));
                        Dr = __dadd_rn(Dr, dwf);
                    }
                }
                if (is_first) dq_first = make_double2(Dr, Qr);
                if (is_last) dq_last = make_double2(Dr, Qr);
                if (!is_first && !is_last) {   // hypercube wholly inside this thread
                    const double nd = (double)nin;
                    const double vh = vg_div<T>(__dsub_rn(__dmul_rn(nd, Qr), __dmul_rn(Dr, Dr)),
                                                __dsub_rn(nd, 1.));
                    acc_m += __dadd_rn(Sseg, Dr);
                    acc_v += vh;
                    if (a.adaptive) {
                        const double sg = (sizeof(T) == 8) ? pow(fabs(vh), beta_half)
                                                           : vg_pow_fast(fabs(vh), beta_half);
                        a.sigf[h0 + key] = sg;
                        acc_s += sg;
                    }
                    if (a.train_hc) train_hcube(a, sbins + (size_t)(win_off[key + 1] - 1) * dim, fabs(vh));
                }
                k = k1;
            }
        }
        __syncthreads();
        double2 Pq = seg_scan(flag, dq_last, Pv, wsum, wflag);
        const double2 carry2 =
            (tid > 0 && prevL == fk && has) ? Pv[tid - 1] : make_double2(0.0, 0.0);
#pragma unroll
        for (int which = 0; which < 2; which++) {
            int key;
            double2 dq;
            if (which == 0) {
                if (!(has && lk != fk)) continue;
                key = fk;
                dq = make_double2(dq_first.x + carry2.x, dq_first.y + carry2.y);
            } else {
                if (!ends_last) continue;
                key = lk;
                dq = Pq;
            }
            const int64_t h = h0 + key;
            const int nin = win_off[key + 1] - win_off[key];
            const int nh = win_n[key];
            const double Sseg = seg_S[key];
            const int64_t ostart = a.offsets[h];
            const bool starts_before = ostart < tile_start;
            const bool ends_after = ostart + nh > tile_start + tile_len;
            if (!starts_before && !ends_after) {
                const double nd = (double)nin;
                const double vh = vg_div<T>(__dsub_rn(__dmul_rn(nd, dq.y), __dmul_rn(dq.x, dq.x)),
                                            __dsub_rn(nd, 1.));
                acc_m += __dadd_rn(Sseg, dq.x);
                acc_v += vh;
                if (a.adaptive) {
                    const double sg = (sizeof(T) == 8) ? pow(fabs(vh), beta_half)
                                                       : vg_pow_fast(fabs(vh), beta_half);
                    a.sigf[h] = sg;
                    acc_s += sg;
                }
                if (a.train_hc) train_hcube(a, sbins + (size_t)(win_off[key + 1] - 1) * dim, fabs(vh));
            } else {
                TileRec r;
                r.h = h;
                r.n = (double)nin;
                r.S = Sseg;
                r.Q = dq.y;
                r.D = dq.x;
                r.spans = (starts_before && ends_after) ? 1 : 0;
                r.pad = 0;
                a.recs[2 * tile + (starts_before ? 0 : 1)] = r;
            }
        }
        }
        if (tid == 0) {   // empty record slots
            const int64_t o0 = a.offsets[h0];
            if (!(o0 < tile_start)) a.recs[2 * tile].h = -1;
            int lastkey = nwin - 1;
            while (lastkey > 0 && win_off[lastkey] >= tile_len) lastkey--;
            const int64_t hL = h0 + lastkey;
            const bool tail = (a.offsets[hL] + a.neval_h[hL] > tile_start + tile_len) &&
                              !(hL == h0 && o0 < tile_start);
            if (!tail) a.recs[2 * tile + 1].h = -1;
        }
    }

    // ---- epilogue: partial sums (unless written per tile), NaN flag,
    // histogram flush
    if (NEED_RED) {
        emit_partial(part_slot);
        if (nan_local) atomicExch((int *)&a.stats->nan_seen, 1);
        if (use_bins && a.hist_smem) {
            __syncthreads();
            for (int d = 0; d < dim; d++) {
                const int K = a.ninc[d];
                for (int i = tid; i < K; i += NT) {
                    const unsigned int c = hcnt[d * a.maxK + i];
                    if (c) {
                        atomicAdd(&a.sum_f[d * a.ldi + i], (double)hsum[d * a.maxK + i]);
                        atomicAdd(&a.n_f[d * a.ldi + i], (unsigned long long)c);
                    }
                }
            }
        }
    }
}

// Resident CTAs per SM the register allocation targets at dim <= 4 in FP32
// for the fused ridge and for the drop-in path's sampling and reduction
// kernels: 4 with 2 samples per thread (64 registers; the shared memory then
// holds no grid table), 2 with 4; 1 (no limit) otherwise.
template <typename T, int MODE, int KIND, int DIMB, int S>
constexpr int tile_min_blocks()
{
    return (sizeof(T) == 4 && DIMB <= 4 &&
            ((MODE == MODE_FUSED && KIND == VG_F_RIDGE) || MODE == MODE_REDUCE || MODE == MODE_POINTS ||
             MODE == MODE_REDUCE_KEPT))
               ? ((S == 2 || (MODE == MODE_POINTS && S == 4)) ? 4 : 2)
               : 1;
}

template <typename T, int MODE, int KIND, int DIMB, int S>
__global__ void __launch_bounds__(NT, tile_min_blocks<T, MODE, KIND, DIMB, S>()) tile_kernel(IterArgs a, VgParams prm)
{
    extern __shared__ __align__(16) unsigned char smem[];
    tile_body<T, MODE, KIND, DIMB, S>(a, prm, smem, blockIdx.x, gridDim.x, blockIdx.x);
}

// ---------------------------------------------------------------- launcher
// Tuning (vg_set_tile_tuning): samples per thread of the fused FP32 kernel
// for dim <= 4 (0 = automatic), grid table / histogram in shared memory
// (-1 automatic, 0 off, 1 on where it fits).
extern int g_tile_s4, g_tile_table, g_tile_hist;

template <typename T, int MODE, int KIND, int DIMB, int S>
int launch_tile(IterArgs &a, const VgParams *prm, int tab_len, cudaStream_t st)
{
    constexpr int TT = NT * S;
    const int dim = a.dim;
    a.tab_len = tab_len;
    a.T = TT;
    constexpr int NEED_RED = (MODE == MODE_REDUCE || MODE == MODE_FUSED || MODE == MODE_REDUCE_KEPT);
    const int bins = NEED_RED && (a.train || a.train_hc);
    const size_t budget = 200 * 1024;
    // the 4-CTA-per-SM configuration reads the FP32 grid table through L1
    // (its shared memory then fits four CTAs); others stage it
    constexpr bool many_ctas = tile_min_blocks<T, MODE, KIND, DIMB, S>() >= 4;
    a.table_smem = g_tile_table == 0 ? 0 : (g_tile_table == 1 ? 1 : (many_ctas ? 0 : 1));
    a.hist_smem = g_tile_hist == 0 ? 0 : (NEED_RED && a.train);
    SmemPlan p = smem_plan<T>(dim, a.maxK, TT, a.table_smem, a.hist_smem, tab_len, bins, NEED_RED);
    if (p.total > budget && a.hist_smem) {
        a.hist_smem = 0;
        p = smem_plan<T>(dim, a.maxK, TT, a.table_smem, a.hist_smem, tab_len, bins, NEED_RED);
    }
    if (p.total > budget) {
        a.table_smem = 0;
        p = smem_plan<T>(dim, a.maxK, TT, a.table_smem, a.hist_smem, tab_len, bins, NEED_RED);
    }
    if (p.total > 220 * 1024) return vg_fail(VG_ERR_UNSUPPORTED, "shared memory plan too large");
    auto kern = tile_kernel<T, MODE, KIND, DIMB, S>;
    static size_t attr_bytes = 0;   // largest dynamic shared memory enabled so far
    if (p.total > attr_bytes) {
        VG_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)p.total));
        attr_bytes = p.total;
    }
    int per_sm = 0;
    VG_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, p.total));
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)vg_num_sms() * per_sm;
    const int64_t tcap = (a.ntiles_cap * BASE_TILE + TT - 1) / TT;
    if (grid > tcap) grid = tcap;
    if (grid < 1) grid = 1;
    if (NEED_RED && grid > a.ntiles_cap) grid = a.ntiles_cap;
    a.ncta = (int)grid;
    static VgParams empty;
    kern<<<(unsigned)grid, NT, p.total, st>>>(a, prm ? *prm : empty);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

// Dispatch on the dimension bucket (DIMB) for a given precision/mode/kind.
template <typename T, int MODE, int KIND>
int launch_dim(IterArgs &a, const VgParams *prm, int tab_len, cudaStream_t st);

int finalize_launch(IterArgs &a, cudaStream_t st, int fast);
int launch_reduce(IterArgs &a, int f64, cudaStream_t st);
int launch_reduce_kept(IterArgs &a, int f64, cudaStream_t st);
// IterArgs of one integral (pointers into its workspace) and its adapt scratch grid
int fill_iter_args(IterArgs &a, const vg_integrator *it, uint32_t itn, const double *u);
void scratch_grid(const vg_integrator *it, double **new_grid, double **new_inc);

}  // namespace vg
