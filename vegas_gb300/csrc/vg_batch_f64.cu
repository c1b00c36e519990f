// vg_batch_f64.cu -- the FP64 parity configuration of the batched launch:
// Lorentzian products of dim <= 8, sampling, map, evaluation and every sum
// in FP64 (the arithmetic of the single-integral FP64 path), so that each
// integral's iterations can be checked against the CPU oracle.
#include "vg_batch.cuh"

namespace vgbatch {
int launch_f64(const BatchJob *jobs, const VgParams *prm, const int *order, int njobs, int nitn, int nwarm,
               uint32_t itn0, unsigned int *queue, size_t smem, int grid, int group, int *status, cudaStream_t st)
{
    return launch_one<double, VG_F_LORENTZ, F64_DIMB, F64_CONFIG.S, F64_CONFIG.minb>(
        jobs, prm, order, njobs, nitn, nwarm, itn0, queue, smem, grid, group, status, st);
}

int occupancy_f64(size_t smem, int *per_sm)
{
    return occupancy_one<double, VG_F_LORENTZ, F64_DIMB, F64_CONFIG.S, F64_CONFIG.minb>(smem, per_sm);
}
}  // namespace vgbatch
