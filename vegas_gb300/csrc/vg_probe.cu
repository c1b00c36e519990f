// vg_probe.cu -- throughput probes for roofline denominators.
//
// Each probe runs independent dependency chains per thread (8 per thread,
// enough to cover pipe latency) for `iters` rounds and writes one value per
// thread so nothing is optimised away.  Work per launch:
//   ex2:   nthreads * iters * 8 MUFU.EX2
//   fma:   nthreads * iters * 8 FMA (2 flops each)
#include "vg_common.cuh"

namespace {

__global__ void probe_ex2(float *out, int iters)
{
    float v[8];
    for (int k = 0; k < 8; k++) v[k] = -1e-3f * (float)(threadIdx.x + k);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            float r;
            asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v[k]));
            v[k] = -r;   // stays in (-1, 0]: no overflow
        }
    }
    float s = 0.f;
    for (int k = 0; k < 8; k++) s += v[k];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void probe_dfma(double *out, int iters)
{
    double v[8];
    for (int k = 0; k < 8; k++) v[k] = 1.0 + 1e-9 * (threadIdx.x + k);
    const double a = 0.999999999, b = 1e-12;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = fma(v[k], a, b);
    }
    double s = 0.0;
    for (int k = 0; k < 8; k++) s += v[k];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void probe_ffma(float *out, int iters)
{
    float v[8];
    for (int k = 0; k < 8; k++) v[k] = 1.0f + 1e-6f * (threadIdx.x + k);
    const float a = 0.9999999f, b = 1e-7f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = fmaf(v[k], a, b);
    }
    float s = 0.f;
    for (int k = 0; k < 8; k++) s += v[k];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int vg_probe_mufu_ex2(float *out, int64_t nthreads, int iters, void *stream)
{
    vg_clear_error();
    if (nthreads % 256) return vg_fail(VG_ERR_VALUE, "nthreads must be a multiple of 256");
    probe_ex2<<<(unsigned)(nthreads / 256), 256, 0, (cudaStream_t)stream>>>(out, iters);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

extern "C" int vg_probe_fp64_fma(double *out, int64_t nthreads, int iters, void *stream)
{
    vg_clear_error();
    if (nthreads % 256) return vg_fail(VG_ERR_VALUE, "nthreads must be a multiple of 256");
    probe_dfma<<<(unsigned)(nthreads / 256), 256, 0, (cudaStream_t)stream>>>(out, iters);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

extern "C" int vg_probe_fp32_fma(float *out, int64_t nthreads, int iters, void *stream)
{
    vg_clear_error();
    if (nthreads % 256) return vg_fail(VG_ERR_VALUE, "nthreads must be a multiple of 256");
    probe_ffma<<<(unsigned)(nthreads / 256), 256, 0, (cudaStream_t)stream>>>(out, iters);
    VG_LAUNCH_CHECK();
    return VG_OK;
}
