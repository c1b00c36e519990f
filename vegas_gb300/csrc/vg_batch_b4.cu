// vg_batch_b4.cu -- batched kernels of the dimension bucket dim <= 4 (its
// three tile configurations, Lorentzian products and the lattice action).
#include "vg_batch.cuh"

namespace vgbatch {
VG_BATCH_BUCKET_ENTRY(4)
}  // namespace vgbatch
