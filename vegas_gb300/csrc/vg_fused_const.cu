// vg_fused_const.cu -- fused tile-kernel instantiations for the built-in
// integrand VG_F_CONST (see vg_integrands.cuh).
#include "vg_fused.cuh"

namespace vg {
int launch_fused_const(IterArgs &a, const VgParams &P, int tab_len, int f64, cudaStream_t st)
{
    return launch_fused_kind<VG_F_CONST>(a, P, tab_len, f64, st);
}
}  // namespace vg
