// vg_fused_gauss.cu -- fused tile-kernel instantiations for the built-in
// integrand VG_F_GAUSS (see vg_integrands.cuh).
#include "vg_fused.cuh"

namespace vg {
int launch_fused_gauss(IterArgs &a, const VgParams &P, int tab_len, int f64, cudaStream_t st)
{
    return launch_fused_kind<VG_F_GAUSS>(a, P, tab_len, f64, st);
}
}  // namespace vg
