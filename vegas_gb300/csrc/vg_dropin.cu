// vg_dropin.cu -- tile-kernel instantiations of the drop-in (torch integrand)
// path: MODE_POINTS writes x (and optionally y, weights, hypercubes) for the
// integrand; MODE_REDUCE reads the integrand values back and reduces.
#include "vg_tile.cuh"

namespace vg {

int launch_points(IterArgs &a, int f64, cudaStream_t st)
{
    if (f64) {
        if (a.dim <= 8) return launch_tile<double, MODE_POINTS, 0, 8, 1>(a, nullptr, 0, st);
        return launch_tile<double, MODE_POINTS, 0, 64, 1>(a, nullptr, 0, st);
    }
    if (a.dim <= 4) return launch_tile<float, MODE_POINTS, 0, 4, 2>(a, nullptr, 0, st);
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

}  // namespace vg

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
