// vg_batch_k442.cu -- batched-kernel instantiation: 4 / 4 / 2 samples per
// thread in the dimension buckets 4 / 8 / 16 (Lorentzian products and the lattice action).
#include "vg_batch.cuh"

namespace vgbatch {
template <int KIND>
static int launch_kind(const BatchJob *jobs, const VgParams *prm, const int *order, int njobs, int nitn, int nwarm,
                       uint32_t itn0, unsigned int *queue, size_t smem, int grid, int group, int *status,
                       cudaStream_t st)
{
    auto k = batch_kernel<KIND, 4, 4, 2, 1>;
    if (group > 1) {   // co-resident groups: cooperative launch
        void *args[] = {(void *)&jobs, (void *)&prm, (void *)&order, (void *)&njobs, (void *)&nitn, (void *)&nwarm,
                        (void *)&itn0, (void *)&queue, (void *)&group, (void *)&status};
        VG_CUDA_CHECK(cudaLaunchCooperativeKernel((const void *)k, dim3((unsigned)grid), dim3(NT), args, smem, st));
        return VG_OK;
    }
    k<<<grid, NT, smem, st>>>(jobs, prm, order, njobs, nitn, nwarm, itn0, queue, group, status);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

template <int KIND>
static int occupancy_kind(size_t smem, int *per_sm)
{
    auto k = batch_kernel<KIND, 4, 4, 2, 1>;
    VG_CUDA_CHECK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    VG_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k, NT, smem));
    return VG_OK;
}

int launch_k442(int kind, const BatchJob *jobs, const VgParams *prm, const int *order, int njobs, int nitn, int nwarm,
                uint32_t itn0, unsigned int *queue, size_t smem, int grid, int group, int *status, cudaStream_t st)
{
    if (kind == VG_F_LATTICE)
        return launch_kind<VG_F_LATTICE>(jobs, prm, order, njobs, nitn, nwarm, itn0, queue, smem, grid, group,
                                         status, st);
    return launch_kind<VG_F_LORENTZ>(jobs, prm, order, njobs, nitn, nwarm, itn0, queue, smem, grid, group, status,
                                     st);
}

// sets the kernel's shared-memory attribute (outside any stream capture)
int occupancy_k442(int kind, size_t smem, int *per_sm)
{
    if (kind == VG_F_LATTICE) return occupancy_kind<VG_F_LATTICE>(smem, per_sm);
    return occupancy_kind<VG_F_LORENTZ>(smem, per_sm);
}
}  // namespace vgbatch
