// vg_batch_b8.cu -- batched kernels of the dimension bucket dim <= 8 (its
// three tile configurations, Lorentzian products and the lattice action).
#include "vg_batch.cuh"

namespace vgbatch {
VG_BATCH_BUCKET_ENTRY(8)
}  // namespace vgbatch
