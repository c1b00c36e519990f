// vg_batch_b16.cu -- batched kernels of the dimension bucket dim <= 16 (its
// three tile configurations, Lorentzian products and the lattice action).
#include "vg_batch.cuh"

namespace vgbatch {
VG_BATCH_BUCKET_ENTRY(16)
}  // namespace vgbatch
