// vg_common.cuh -- device helpers shared by the vegas+ kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include "vg_internal.h"

// NVTX range around an entry point's enqueue work (host side), so that a
// profiler's timeline groups each call's kernels under the ABI name.  The
// NVTX3 calls are no-ops unless a profiling tool is attached.
struct VgRange {
    explicit VgRange(const char *name) { nvtxRangePushA(name); }
    ~VgRange() { nvtxRangePop(); }
    VgRange(const VgRange &) = delete;
    VgRange &operator=(const VgRange &) = delete;
};
#define VG_RANGE_CAT2(a, b) a##b
#define VG_RANGE_CAT(a, b) VG_RANGE_CAT2(a, b)
#define VG_RANGE(name) VgRange VG_RANGE_CAT(vg_range_, __LINE__)(name)

#define VG_TINY 1e-257                       // _vegas.pyx:34
#define VG_EPSILON (2.220446049250313e-16 * 1e4)  // _vegas.pyx:36

// ---------------------------------------------------------------- Philox
// Philox4x32-10 (Salmon et al., SC'11).  Counter layout shared with the
// oracle: (sample_lo, sample_hi, iteration, stream<<8 | group).
struct VgU4 {
    uint32_t x, y, z, w;
};

__device__ __forceinline__ VgU4 vg_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                          uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return VgU4{c0, c1, c2, c3};
}

// Uniforms for sample i, axes [0, dim) (dim <= DIMB): FP64 takes two words
// per axis (53 bits, counter word 3 = stream<<8 | 0x80 | d>>1), FP32 one word
// per axis (24 bits, counter word 3 = stream<<8 | d>>2).  Same stream as the
// oracle (vo_uniform_f64 / vo_uniform_f32).
template <typename T>
struct VgUniform;

template <>
struct VgUniform<double> {
    template <int DIMB>
    static __device__ __forceinline__ void draw(uint64_t seed, uint32_t stream, uint32_t itn,
                                                uint64_t i, int dim, double *u)
    {
#pragma unroll
        for (int g = 0; 2 * g < DIMB; g++) {
            if (2 * g >= dim) break;
            VgU4 r = vg_philox((uint32_t)i, (uint32_t)(i >> 32), itn,
                               (stream << 8) | 0x80u | (uint32_t)g, (uint32_t)seed,
                               (uint32_t)(seed >> 32));
            uint64_t m0 = ((uint64_t)r.x << 21) | (uint64_t)(r.y >> 11);
            u[2 * g] = (double)m0 * (1.0 / 9007199254740992.0);
            if (2 * g + 1 < DIMB) {
                uint64_t m1 = ((uint64_t)r.z << 21) | (uint64_t)(r.w >> 11);
                u[2 * g + 1] = (double)m1 * (1.0 / 9007199254740992.0);
            }
        }
    }
};

template <>
struct VgUniform<float> {
    template <int DIMB>
    static __device__ __forceinline__ void draw(uint64_t seed, uint32_t stream, uint32_t itn,
                                                uint64_t i, int dim, float *u)
    {
        const float s = 1.0f / 16777216.0f;
#pragma unroll
        for (int g = 0; 4 * g < DIMB; g++) {
            if (4 * g >= dim) break;
            VgU4 r = vg_philox((uint32_t)i, (uint32_t)(i >> 32), itn, (stream << 8) | (uint32_t)g,
                               (uint32_t)seed, (uint32_t)(seed >> 32));
            u[4 * g] = (float)(r.x >> 8) * s;
            if (4 * g + 1 < DIMB) u[4 * g + 1] = (float)(r.y >> 8) * s;
            if (4 * g + 2 < DIMB) u[4 * g + 2] = (float)(r.z >> 8) * s;
            if (4 * g + 3 < DIMB) u[4 * g + 3] = (float)(r.w >> 8) * s;
        }
    }
};

// --------------------------------------------------- fast transcendentals
// FP32-mode replacements for FP64 pow/log on GB300, whose FP64 rate is about
// 1/64 of its FP32 rate.  The binary exponent is split off exactly with
// integer arithmetic, so the full double range is handled; the mantissa's
// log2 and the fraction's exp2 use the MUFU (ex2/lg2.approx).  Relative
// error ~2e-6, enough for the allocation weights and grid damping of the FP32
// mode; the FP64 mode keeps the exact FP64 library functions.
__device__ __forceinline__ float vg_lg2_approx(float x)
{
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float vg_ex2_approx(float x)
{
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// log2(x) for finite x > 0 (FP32 result, exact exponent split).
__device__ __forceinline__ float vg_log2_split(double x)
{
    int hi = __double2hiint(x), lo = __double2loint(x);
    int e = (hi >> 20) & 0x7ff;
    if (e == 0) {   // subnormal: scale by 2^54
        x *= 18014398509481984.0;
        hi = __double2hiint(x);
        lo = __double2loint(x);
        e = ((hi >> 20) & 0x7ff) - 54;
    }
    double m = __hiloint2double((hi & 0x800fffff) | 0x3ff00000, lo);   // [1, 2)
    return (float)(e - 1023) + vg_lg2_approx((float)m);
}

// 2^p for |p| < 2^24 as a double (0 below the normal range, inf above).
__device__ __forceinline__ double vg_exp2_split(float p)
{
    float fl = floorf(p);
    float fr = p - fl;                      // [0, 1)
    int n = (int)fl;
    double r = (double)vg_ex2_approx(fr);   // [1, 2)
    if (n < -1021) return 0.0;
    if (n > 1022) return __longlong_as_double(0x7ff0000000000000LL);
    long long bits = __double_as_longlong(r) + ((long long)n << 52);
    return __longlong_as_double(bits);
}

// x^y for x >= 0 (fast path), falling back to pow for 0, inf and NaN.
__device__ __forceinline__ double vg_pow_fast(double x, double y)
{
    if (!(x > 0.0) || x > 1.7e308) return pow(x, y);
    return vg_exp2_split((float)y * vg_log2_split(x));
}

// ------------------------------------------------------- compensated sum
// Neumaier summation in FP64 for the per-iteration totals.
struct VgKSum {
    double s, c;
    __device__ __forceinline__ void add(double v)
    {
        double t = s + v;
        if (fabs(s) >= fabs(v)) c += (s - t) + v;
        else c += (v - t) + s;
        s = t;
    }
    __device__ __forceinline__ void merge(const VgKSum &o)
    {
        add(o.s);
        c += o.c;
    }
    __device__ __forceinline__ double value() const { return s + c; }
};

__device__ __forceinline__ VgKSum vg_ksum_shfl_down(VgKSum v, int off)
{
    VgKSum o;
    o.s = __shfl_down_sync(0xffffffffu, v.s, off);
    o.c = __shfl_down_sync(0xffffffffu, v.c, off);
    return o;
}

// Fixed-order block reduction of a compensated sum (deterministic).  All
// threads of the block must call it; result valid in thread 0.
template <int NT>
__device__ __forceinline__ VgKSum vg_block_ksum(VgKSum v, VgKSum *smem /* NT/32 */)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        VgKSum o = vg_ksum_shfl_down(v, off);
        v.merge(o);
    }
    if (NT == 32) return v;   // one warp: done (FP64 instructions are costly)
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) smem[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (lane < NT / 32) ? smem[lane] : VgKSum{0.0, 0.0};
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            VgKSum o = vg_ksum_shfl_down(v, off);
            v.merge(o);
        }
    }
    __syncthreads();
    return v;
}

// Float-float (double-single) accumulation: (h, l) += x with Knuth's
// TwoSum (error-free in h, the rounding error carried in l).  The FP32 mode
// accumulates a thread's few samples this way (about 2^-48 relative, close
// to FP64) before the per-hypercube sums continue in FP64.  __fadd_rn /
// __fsub_rn keep the compiler from reassociating or contracting.
__device__ __forceinline__ void vg_ff_add(float &h, float &l, float x)
{
    const float s = __fadd_rn(h, x);
    const float bb = __fsub_rn(s, h);
    const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    h = s;
    l = __fadd_rn(l, e);
}

__device__ __forceinline__ double vg_ff_value(float h, float l) { return (double)h + (double)l; }

#define VG_CUDA_CHECK(expr)                                                                  \
    do {                                                                                     \
        cudaError_t _e = (expr);                                                             \
        if (_e != cudaSuccess)                                                               \
            return vg_fail(VG_ERR_CUDA, "%s: %s (%s:%d)", #expr, cudaGetErrorString(_e),    \
                           __FILE__, __LINE__);                                              \
    } while (0)

#define VG_LAUNCH_CHECK()                                                                    \
    do {                                                                                     \
        cudaError_t _e = cudaGetLastError();                                                 \
        if (_e != cudaSuccess)                                                               \
            return vg_fail(VG_ERR_CUDA, "kernel launch: %s (%s:%d)", cudaGetErrorString(_e), \
                           __FILE__, __LINE__);                                              \
    } while (0)

static inline int vg_num_sms()
{
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 148;
    }
    return n;
}
