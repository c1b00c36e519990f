// vg_integrands.cuh -- built-in integrands evaluated inside the fused
// iteration kernel.  They are the synthetic workloads of the benchmarks:
// the CPU oracle (oracle/vegas_oracle.c, vo_eval1) defines the same
// functions in FP64.
//
// FP64 versions follow the oracle's direct formulas.  FP32 versions are
// written for the SFU / FP32 pipes: Gaussians are evaluated with exp2 of a
// log2-scaled exponent, and the ridge uses the decomposition
//     |x - c 1|^2 = R + dim (m - c)^2,  m = mean(x), R = sum (x_d - m)^2,
// so each of its M terms costs one subtract, one FMA and one ex2.
#pragma once
#include "vg_common.cuh"

#define VG_MAX_PARAMS 1024

struct VgParams {
    int n;
    float fc[8];                 // FP32 constants, precomputed on the host (vg_prepare_f32_host)
    unsigned long long *term_count;   // optional: Gaussian terms evaluated (ridge, FP32)
    double p[VG_MAX_PARAMS];
};

// Per-CTA precomputed constants (shared memory) for the FP32 integrands.
struct VgIntegrandSmem {
    float k0, k1, k2, k3;  // scalar constants (meaning per integrand)
};

constexpr double VG_PI = 3.14159265358979323846;
constexpr double VG_LOG2E = 1.4426950408889634074;

// ------------------------------------------------------------------ FP64
template <int KIND, int DIMB>
__device__ __forceinline__ double vg_eval_f64(const VgParams &P, int dim, const double *x)
{
    const double *p = P.p;
    if (KIND == VG_F_GAUSS) {
        double s = 0.0;
        for (int d = 0; d < dim; d++) {
            double t = __dsub_rn(x[d], p[1]);
            s = __dadd_rn(s, __dmul_rn(t, t));
        }
        return __dmul_rn(p[2], exp(__dmul_rn(-p[0], s)));
    } else if (KIND == VG_F_RIDGE) {
        int M = (int)p[0];
        double sg = p[1];
        double two_s2 = __dmul_rn(__dmul_rn(2.0, sg), sg);
        double norm = pow(__dmul_rn(__dmul_rn(__dmul_rn(2.0, VG_PI), sg), sg), -0.5 * dim);
        double acc = 0.0;
        for (int j = 0; j < M; j++) {
            double c = __ddiv_rn(__dadd_rn((double)j, 0.5), (double)M);
            double r2 = 0.0;
            for (int d = 0; d < dim; d++) {
                double t = __dsub_rn(x[d], c);
                r2 = __dadd_rn(r2, __dmul_rn(t, t));
            }
            acc = __dadd_rn(acc, exp(__ddiv_rn(-r2, two_s2)));
        }
        return __ddiv_rn(__dmul_rn(norm, acc), (double)M);
    } else if (KIND == VG_F_LORENTZ) {
        double f = 1.0;
        for (int d = 0; d < dim; d++) {
            double c = p[d], w = p[dim + d];
            double t = __dsub_rn(x[d], c);
            f = __dmul_rn(f, __ddiv_rn(__ddiv_rn(w, VG_PI),
                                       __dadd_rn(__dmul_rn(t, t), __dmul_rn(w, w))));
        }
        return f;
    } else if (KIND == VG_F_MIXTURE) {
        int K = (int)p[0];
        double sg = p[1];
        double two_s2 = __dmul_rn(__dmul_rn(2.0, sg), sg);
        double norm = pow(__dmul_rn(__dmul_rn(__dmul_rn(2.0, VG_PI), sg), sg), -0.5 * dim);
        double acc = 0.0;
        for (int k = 0; k < K; k++) {
            double r2 = 0.0;
            for (int d = 0; d < dim; d++) {
                double t = __dsub_rn(x[d], p[2 + k * dim + d]);
                r2 = __dadd_rn(r2, __dmul_rn(t, t));
            }
            acc = __dadd_rn(acc, exp(__ddiv_rn(-r2, two_s2)));
        }
        return __ddiv_rn(__dmul_rn(norm, acc), (double)K);
    } else if (KIND == VG_F_LATTICE) {
        double a = p[0], lam = p[1], S = 0.0;
        for (int i = 0; i < dim; i++) {
            double xi = x[i], xn = x[(i + 1) % dim];
            double dx = __dsub_rn(xn, xi);
            double kin = __ddiv_rn(__dmul_rn(dx, dx), __dmul_rn(2.0, a));
            double x2 = __dmul_rn(xi, xi);
            double pot = __dmul_rn(a, __dadd_rn(__ddiv_rn(x2, 2.0), __dmul_rn(__dmul_rn(lam, x2), x2)));
            S = __dadd_rn(S, __dadd_rn(kin, pot));
        }
        return exp(-S);
    } else {
        return p[0];
    }
}

// ------------------------------------------------------------------ FP32
// Constants precomputed on the host side of the kernel launch (FP64 -> FP32
// once per CTA):  see vg_prepare_f32.
struct VgF32Consts {
    float c[8];
};

// FP32 constants of each integrand, computed once on the host in FP64 (the
// GPU's FP64 rate is too low to recompute them in every thread).
inline void vg_prepare_f32_host(VgParams &P, int kind, int dim)
{
    const double *p = P.p;
    for (int i = 0; i < 8; i++) P.fc[i] = 0.f;
    if (kind == VG_F_GAUSS) {
        P.fc[0] = (float)(p[0] * VG_LOG2E);  // a*log2(e)
        P.fc[1] = (float)p[1];               // centre
        P.fc[2] = (float)p[2];               // norm
    } else if (kind == VG_F_RIDGE) {
        double M = p[0], sg = p[1];
        double kk = 1.0 / (2.0 * sg * sg) * VG_LOG2E;    // log2 units
        double sk = sqrt(kk * dim);
        P.fc[0] = (float)kk;                                // E0 = -kk * R
        P.fc[1] = (float)sk;                                // w = m * sk
        P.fc[2] = (float)(pow(2.0 * VG_PI * sg * sg, -0.5 * dim) / M);
        P.fc[3] = (float)(1.0 / dim);
        P.fc[4] = (float)(sk / M);                          // v_j = (j + 1/2) * sk/M
        P.fc[5] = (float)M;
    } else if (kind == VG_F_MIXTURE) {
        double sg = p[1];
        P.fc[0] = (float)(VG_LOG2E / (2.0 * sg * sg));
        P.fc[1] = (float)(pow(2.0 * VG_PI * sg * sg, -0.5 * dim) / p[0]);
        P.fc[5] = (float)p[0];
    } else if (kind == VG_F_LATTICE) {
        P.fc[0] = (float)(1.0 / (2.0 * p[0]));
        P.fc[1] = (float)p[0];
        P.fc[2] = (float)p[1];
    } else if (kind == VG_F_CONST) {
        P.fc[0] = (float)p[0];
    }
}

template <int KIND>
__device__ __forceinline__ VgF32Consts vg_prepare_f32(const VgParams &P, int dim)
{
    VgF32Consts k;
#pragma unroll
    for (int i = 0; i < 8; i++) k.c[i] = P.fc[i];
    return k;
}

// Fill per-CTA shared tables (ridge term offsets, mixture centres).
template <int KIND>
__device__ __forceinline__ void vg_fill_table_f32(const VgParams &P, int dim, float *tab,
                                                  const VgF32Consts &k)
{
    if (KIND == VG_F_RIDGE) {
        const int M = (int)P.fc[5];
        for (int j = threadIdx.x; j < M; j += blockDim.x) tab[j] = ((float)j + 0.5f) * k.c[4];
    } else if (KIND == VG_F_MIXTURE) {
        const int K = (int)P.fc[5];
        for (int j = threadIdx.x; j < K * dim; j += blockDim.x) tab[j] = (float)P.p[2 + j];
    } else if (KIND == VG_F_LORENTZ) {
        for (int j = threadIdx.x; j < dim; j += blockDim.x) {
            const float c = (float)P.p[j], w = (float)P.p[dim + j];
            tab[j] = c;                                     // centre
            tab[dim + j] = w;                               // width
            tab[2 * dim + j] = w * (float)(1.0 / VG_PI);
            tab[3 * dim + j] = w * w;
        }
    }
}

template <int KIND>
__device__ __forceinline__ int vg_table_len(const VgParams &P, int dim)
{
    if (KIND == VG_F_RIDGE) return (int)P.p[0];
    if (KIND == VG_F_MIXTURE) return (int)P.p[0] * dim;
    if (KIND == VG_F_LORENTZ) return 4 * dim;
    return 0;
}

__device__ __forceinline__ float vg_ex2(float x)
{
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

template <int KIND, int DIMB>
__device__ __forceinline__ float vg_eval_f32(const VgF32Consts &k, const float *__restrict__ tab,
                                             int nterm, int dim, const float *x)
{
    if (KIND == VG_F_GAUSS) {
        float s = 0.f;
#pragma unroll
        for (int d = 0; d < DIMB; d++) {
            if (d >= dim) break;
            float t = x[d] - k.c[1];
            s = fmaf(t, t, s);
        }
        return k.c[2] * vg_ex2(-k.c[0] * s);
    } else if (KIND == VG_F_RIDGE) {
        float m = 0.f;
#pragma unroll
        for (int d = 0; d < DIMB; d++)
            if (d < dim) m += x[d];
        m *= k.c[3];
        float R = 0.f;
#pragma unroll
        for (int d = 0; d < DIMB; d++) {
            if (d >= dim) break;
            float t = x[d] - m;
            R = fmaf(t, t, R);
        }
        const float E0 = -k.c[0] * R;
        const float w = m * k.c[1];
        float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
        // terms with E0 - (w - v_j)^2 < -127 are exactly zero (ex2.approx.ftz
        // flushes them): evaluate the window of the others only, aligned to
        // the 4-way accumulator pattern -- the sum is bit-identical
        int j = 0, jend = nterm & ~3;
        {
            const float rad2 = E0 + 127.f;
            if (rad2 <= 0.f) {
                jend = 0;
            } else {
                const float delta = sqrtf(rad2) * 1.0001f + 1e-3f;
                const float rc = 1.f / k.c[4];
                int jlo = (int)floorf((w - delta) * rc - 0.5f) - 1;
                int jhi = (int)ceilf((w + delta) * rc - 0.5f) + 1;
                jlo = jlo < 0 ? 0 : jlo;
                jhi = jhi > nterm - 1 ? nterm - 1 : jhi;
                j = jlo & ~3;
                const int je = (jhi & ~3) + 4;
                jend = je < jend ? je : jend;
                if (j > jend) j = jend;
            }
        }
        for (; j + 4 <= jend; j += 4) {
            float4 v = *reinterpret_cast<const float4 *>(tab + j);
            float d0 = w - v.x, d1 = w - v.y, d2 = w - v.z, d3 = w - v.w;
            a0 += vg_ex2(fmaf(-d0, d0, E0));
            a1 += vg_ex2(fmaf(-d1, d1, E0));
            a2 += vg_ex2(fmaf(-d2, d2, E0));
            a3 += vg_ex2(fmaf(-d3, d3, E0));
        }
        for (j = nterm & ~3; j < nterm; j++) {
            float d0 = w - tab[j];
            a0 += vg_ex2(fmaf(-d0, d0, E0));
        }
        return k.c[2] * ((a0 + a1) + (a2 + a3));
    } else if (KIND == VG_F_LORENTZ) {
        float f = 1.f;
#pragma unroll
        for (int d = 0; d < DIMB; d++) {
            if (d >= dim) break;
            float t = x[d] - tab[d];
            f *= __fdividef(tab[2 * dim + d], fmaf(t, t, tab[3 * dim + d]));
        }
        return f;
    } else if (KIND == VG_F_MIXTURE) {
        int K = nterm / dim;
        float acc = 0.f;
        for (int q = 0; q < K; q++) {
            float r2 = 0.f;
#pragma unroll
            for (int d = 0; d < DIMB; d++) {
                if (d >= dim) break;
                float t = x[d] - tab[q * dim + d];
                r2 = fmaf(t, t, r2);
            }
            acc += vg_ex2(-k.c[0] * r2);
        }
        return k.c[1] * acc;
    } else if (KIND == VG_F_LATTICE) {
        float S = 0.f;
#pragma unroll
        for (int i = 0; i < DIMB; i++) {
            if (i >= dim) break;
            float xi = x[i], xn = (i + 1 == dim) ? x[0] : x[(i + 1) % DIMB];
            float dx = xn - xi;
            float x2 = xi * xi;
            S = fmaf(dx * dx, k.c[0], S);
            S = fmaf(k.c[1], fmaf(k.c[2] * x2, x2, 0.5f * x2), S);
        }
        return vg_ex2(-S * (float)VG_LOG2E);
    } else {
        return k.c[0];
    }
}
