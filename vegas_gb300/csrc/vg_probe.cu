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

// ------------------------------------------------------------------------
// tcgen05 building-block check: one CTA computes D[128 x N] = A[128 x K] *
// B[N x K]^T (bf16 in, FP32 accumulation in TMEM) with the helpers of
// vg_umma.cuh -- the same descriptors, swizzle and TMEM loads the flow
// kernels use.  status[0] is set to 1 when the bounded wait gave up.
#include "vg_umma.cuh"

namespace {

__global__ void __launch_bounds__(128) probe_umma_kernel(const __nv_bfloat16 *__restrict__ A,
                                                         const __nv_bfloat16 *__restrict__ B,
                                                         float *__restrict__ D, int N, int K,
                                                         uint32_t ncols, int a_mn, int b_mn, int *status)
{
    extern __shared__ uint8_t dsm[];
    __shared__ uint64_t bar;
    __shared__ uint32_t slot;
    uint8_t *base = umma::align1024(dsm);
    uint8_t *sa = base;
    uint8_t *sb = base + 128 * K * 2;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int kc = K / 8;
    if (!a_mn) {
        for (int i = tid; i < 128 * kc; i += blockDim.x) {
            const int r = i / kc, k = (i % kc) * 8;
            *reinterpret_cast<uint4 *>(sa + umma::sw128_offset(128, r, k)) =
                *reinterpret_cast<const uint4 *>(A + (size_t)r * K + k);
        }
    } else {   // A given as [K][128]: the tile of its transpose
        for (int i = tid; i < K * 16; i += blockDim.x) {
            const int k = i / 16, m = (i % 16) * 8;
            *reinterpret_cast<uint4 *>(sa + umma::sw128_offset(K, k, m)) =
                *reinterpret_cast<const uint4 *>(A + (size_t)k * 128 + m);
        }
    }
    if (!b_mn) {
        for (int i = tid; i < N * kc; i += blockDim.x) {
            const int r = i / kc, k = (i % kc) * 8;
            *reinterpret_cast<uint4 *>(sb + umma::sw128_offset(N, r, k)) =
                *reinterpret_cast<const uint4 *>(B + (size_t)r * K + k);
        }
    } else {   // B given as [K][N]
        const int nc = N / 8;
        for (int i = tid; i < K * nc; i += blockDim.x) {
            const int k = i / nc, m = (i % nc) * 8;
            *reinterpret_cast<uint4 *>(sb + umma::sw128_offset(K, k, m)) =
                *reinterpret_cast<const uint4 *>(B + (size_t)k * N + m);
        }
    }
    umma::fence_async_smem();
    if (warp == 0) umma::tmem_alloc(umma::smem_u32(&slot), ncols);
    if (tid == 0) umma::mbar_init(umma::smem_u32(&bar), 1);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = slot;
    if (tid == 0) {
        umma::gemm_128xN_ex(tmem, umma::smem_u32(sa), a_mn, a_mn ? 0 : 128, umma::smem_u32(sb), b_mn, b_mn ? 0 : N, N,
                            K, 0);
        umma::mma_commit(umma::smem_u32(&bar));
    }
    const bool ok = umma::mbar_wait(umma::smem_u32(&bar), 0);
    umma::fence_after_sync();
    if (!ok) {
        if (tid == 0) atomicExch(status, 1);
        umma::mbar_wait(umma::smem_u32(&bar), 0);   // bounded: give the MMAs a second chance to drain
    } else {
        const int row = 32 * warp + (tid & 31);
        for (int c = 0; c < N; c += 16) {
            float v[16];
            umma::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
#pragma unroll
            for (int i = 0; i < 16; i++) D[(size_t)row * N + c + i] = v[i];
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, ncols);
}

}  // namespace

extern "C" int vg_probe_umma_gemm(const void *A, const void *B, float *D, int N, int K, int a_mn, int b_mn,
                                  int *status, void *stream)
{
    vg_clear_error();
    if (N < 16 || N > 256 || N % 16 || K < 64 || K % 64 || K > 256 || (b_mn && N % 64))
        return vg_fail(VG_ERR_VALUE, "umma probe: N in 16..256 (multiple of 16; of 64 for MN-major B), "
                                     "K in 64..256 (multiple of 64)");
    uint32_t ncols = 32;
    while ((int)ncols < N) ncols <<= 1;
    const size_t smem = (size_t)(128 + N) * K * 2 + 1024;
    cudaError_t e = cudaFuncSetAttribute(probe_umma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return vg_fail(VG_ERR_CUDA, "umma probe smem: %s", cudaGetErrorString(e));
    probe_umma_kernel<<<1, 128, smem, (cudaStream_t)stream>>>((const __nv_bfloat16 *)A, (const __nv_bfloat16 *)B,
                                                              D, N, K, ncols, a_mn, b_mn, status);
    VG_LAUNCH_CHECK();
    return VG_OK;
}
