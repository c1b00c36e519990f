// vg_fused.cuh -- dimension-bucket dispatch of the fused tile kernel for one
// built-in integrand (included by one vg_fused_*.cu file per integrand so the
// instantiations compile in parallel).
#pragma once
#include "vg_tile.cuh"

namespace vg {

// One fused kernel by default.  The split form -- an EVAL kernel without the
// reduction's shared memory and barriers (higher occupancy for an SFU-bound
// loop) writing f, a REDUCE kernel reading it back -- stays selectable for
// the ridge (vg_set_eval_split): it paid while the ridge evaluated all of its
// terms; with the FP32 term window the fused kernel is faster.
extern int g_eval_split;   // 0 automatic, 1 fused, 2 split (vg_set_eval_split)

template <int KIND>
int launch_fused_kind(IterArgs &a, const VgParams &P, int tab_len, int f64, cudaStream_t st)
{
    if (!f64 && KIND == VG_F_RIDGE && g_eval_split == 2) {
        int rc;
        VG_CUDA_CHECK(cudaMemsetAsync(a.counter, 0, sizeof(unsigned long long), st));   // dynamic tiles
        if (a.dim <= 4) rc = launch_tile<float, MODE_EVAL, KIND, 4, 2>(a, &P, tab_len, st);
        else if (a.dim <= 8) rc = launch_tile<float, MODE_EVAL, KIND, 8, 2>(a, &P, tab_len, st);
        else if (a.dim <= 16) rc = launch_tile<float, MODE_EVAL, KIND, 16, 2>(a, &P, tab_len, st);
        else rc = launch_tile<float, MODE_EVAL, KIND, 64, 1>(a, &P, tab_len, st);
        if (rc) return rc;
        VG_CUDA_CHECK(cudaMemsetAsync(a.counter, 0, sizeof(unsigned long long), st));
        a.f_in = a.f_eval;
        a.f_f64 = 0;
        return launch_reduce(a, 0, st);
    }
    if (f64) {
        if (a.dim <= 8) return launch_tile<double, MODE_FUSED, KIND, 8, 2>(a, &P, tab_len, st);
        return launch_tile<double, MODE_FUSED, KIND, 64, 1>(a, &P, tab_len, st);
    }
    if (a.dim <= 4) {
        if constexpr (KIND == VG_F_RIDGE)
            if (g_tile_s4 != 4) return launch_tile<float, MODE_FUSED, KIND, 4, 2>(a, &P, tab_len, st);
        return launch_tile<float, MODE_FUSED, KIND, 4, 4>(a, &P, tab_len, st);
    }
    if (a.dim <= 8) return launch_tile<float, MODE_FUSED, KIND, 8, 4>(a, &P, tab_len, st);
    if (a.dim <= 16) return launch_tile<float, MODE_FUSED, KIND, 16, 2>(a, &P, tab_len, st);
    return launch_tile<float, MODE_FUSED, KIND, 64, 1>(a, &P, tab_len, st);
}

int launch_fused_gauss(IterArgs &a, const VgParams &P, int tab_len, int f64, cudaStream_t st);
int launch_fused_ridge(IterArgs &a, const VgParams &P, int tab_len, int f64, cudaStream_t st);
int launch_fused_lorentz(IterArgs &a, const VgParams &P, int tab_len, int f64, cudaStream_t st);
int launch_fused_mixture(IterArgs &a, const VgParams &P, int tab_len, int f64, cudaStream_t st);
int launch_fused_lattice(IterArgs &a, const VgParams &P, int tab_len, int f64, cudaStream_t st);
int launch_fused_const(IterArgs &a, const VgParams &P, int tab_len, int f64, cudaStream_t st);

}  // namespace vg
