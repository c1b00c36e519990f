// vg_dropin.cu -- tile-kernel instantiations of the drop-in (torch integrand)
// path: MODE_POINTS writes x (and optionally y, weights, hypercubes, and the
// kept Jacobians and training bins) for the integrand; MODE_REDUCE reads the
// integrand values back and reduces, regenerating each sample;
// MODE_REDUCE_KEPT reduces from the kept Jacobians and bins instead.
#include "vg_tile.cuh"

namespace vg {

// Samples per thread of the FP32 sampling and kept-sample reduction kernels
// at dim <= 4 (vg_set_dropin_tuning; 0 = automatic).
int g_dropin_sp = 0, g_dropin_sr = 0;

int launch_points(IterArgs &a, int f64, cudaStream_t st)
{
    if (f64) {
        if (a.dim <= 8) return launch_tile<double, MODE_POINTS, 0, 8, 1>(a, nullptr, 0, st);
        return launch_tile<double, MODE_POINTS, 0, 64, 1>(a, nullptr, 0, st);
    }
    if (a.dim <= 4) {
        if (g_dropin_sp == 4) return launch_tile<float, MODE_POINTS, 0, 4, 4>(a, nullptr, 0, st);
        if (g_dropin_sp == 8) return launch_tile<float, MODE_POINTS, 0, 4, 8>(a, nullptr, 0, st);
        return launch_tile<float, MODE_POINTS, 0, 4, 2>(a, nullptr, 0, st);
    }
    if (a.dim <= 8) return launch_tile<float, MODE_POINTS, 0, 8, 1>(a, nullptr, 0, st);
    if (a.dim <= 16) return launch_tile<float, MODE_POINTS, 0, 16, 1>(a, nullptr, 0, st);
    return launch_tile<float, MODE_POINTS, 0, 64, 1>(a, nullptr, 0, st);
}

int launch_reduce(IterArgs &a, int f64, cudaStream_t st)
{
    if (f64) {
        if (a.dim <= 8) return launch_tile<double, MODE_REDUCE, 0, 8, 2>(a, nullptr, 0, st);
        return launch_tile<double, MODE_REDUCE, 0, 64, 1>(a, nullptr, 0, st);
    }
    if (a.dim <= 4) return launch_tile<float, MODE_REDUCE, 0, 4, 2>(a, nullptr, 0, st);
    if (a.dim <= 8) return launch_tile<float, MODE_REDUCE, 0, 8, 4>(a, nullptr, 0, st);
    if (a.dim <= 16) return launch_tile<float, MODE_REDUCE, 0, 16, 2>(a, nullptr, 0, st);
    return launch_tile<float, MODE_REDUCE, 0, 64, 1>(a, nullptr, 0, st);
}

int launch_reduce_kept(IterArgs &a, int f64, cudaStream_t st)
{
    if (f64) {
        if (a.dim <= 8) return launch_tile<double, MODE_REDUCE_KEPT, 0, 8, 2>(a, nullptr, 0, st);
        return launch_tile<double, MODE_REDUCE_KEPT, 0, 64, 1>(a, nullptr, 0, st);
    }
    if (a.dim <= 4) {
        if (g_dropin_sr == 4) return launch_tile<float, MODE_REDUCE_KEPT, 0, 4, 4>(a, nullptr, 0, st);
        return launch_tile<float, MODE_REDUCE_KEPT, 0, 4, 2>(a, nullptr, 0, st);
    }
    if (a.dim <= 8) return launch_tile<float, MODE_REDUCE_KEPT, 0, 8, 4>(a, nullptr, 0, st);
    if (a.dim <= 16) return launch_tile<float, MODE_REDUCE_KEPT, 0, 16, 2>(a, nullptr, 0, st);
    return launch_tile<float, MODE_REDUCE_KEPT, 0, 64, 1>(a, nullptr, 0, st);
}

}  // namespace vg

// Tuning of the drop-in path's FP32 kernels at dim <= 4: samples per thread
// of the sampler (0 automatic = 2; 2, 4, 8) and of the kept-sample
// reduction (0 automatic = 2; 2, 4).
extern "C" int vg_set_dropin_tuning(int s_points, int s_reduce)
{
    if (s_points != 0 && s_points != 2 && s_points != 4 && s_points != 8)
        return vg_fail(VG_ERR_VALUE, "s_points %d", s_points);
    if (s_reduce != 0 && s_reduce != 2 && s_reduce != 4) return vg_fail(VG_ERR_VALUE, "s_reduce %d", s_reduce);
    vg::g_dropin_sp = s_points;
    vg::g_dropin_sr = s_reduce;
    return VG_OK;
}

#include "vg_fused.cuh"

namespace vg {
int launch_fused(IterArgs &a, int kind, const VgParams &P, int tab_len, int f64, cudaStream_t st)
{
    switch (kind) {
    case VG_F_GAUSS: return launch_fused_gauss(a, P, tab_len, f64, st);
    case VG_F_RIDGE: return launch_fused_ridge(a, P, tab_len, f64, st);
    case VG_F_LORENTZ: return launch_fused_lorentz(a, P, tab_len, f64, st);
    case VG_F_MIXTURE: return launch_fused_mixture(a, P, tab_len, f64, st);
    case VG_F_LATTICE: return launch_fused_lattice(a, P, tab_len, f64, st);
    default: return launch_fused_const(a, P, tab_len, f64, st);
    }
}
}  // namespace vg
