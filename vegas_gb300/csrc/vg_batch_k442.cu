// vg_batch_k442.cu -- batched-kernel instantiation: 4 / 4 / 2 samples per
// thread in the dimension buckets 4 / 8 / 16 (Lorentzian products).
#include "vg_batch.cuh"

namespace vgbatch {
int launch_k442(const BatchJob *jobs, const VgParams *prm, const int *order, int njobs, int nitn, int nwarm,
                uint32_t itn0, unsigned int *queue, size_t smem, int grid, cudaStream_t st)
{
    auto k = batch_kernel<VG_F_LORENTZ, 4, 4, 2, 1>;
    k<<<grid, NT, smem, st>>>(jobs, prm, order, njobs, nitn, nwarm, itn0, queue);
    VG_LAUNCH_CHECK();
    return VG_OK;
}
// sets the kernel's shared-memory attribute (outside any stream capture)
int occupancy_k442(size_t smem, int *per_sm)
{
    VG_CUDA_CHECK(cudaFuncSetAttribute(batch_kernel<VG_F_LORENTZ, 4, 4, 2, 1>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    VG_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, batch_kernel<VG_F_LORENTZ, 4, 4, 2, 1>, NT, smem));
    return VG_OK;
}
}  // namespace vgbatch
