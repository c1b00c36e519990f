// vg_batch.cu -- host side of the batched many-integral launch.
//
// vg_batch_prepare builds the device job table (per integral: its iteration
// arguments, adapt arguments, integrand parameters, output slots) and picks
// the shared-memory plan of a tile-shape variant; vg_batch_launch is one
// persistent kernel over all integrals (no host synchronisation, no
// allocation: it can be captured in a CUDA graph).  No counterpart in the
// reference, which integrates one integrand per Integrator call; each
// integral here runs the same vegas+ iteration as vg_fused_iteration.
#include <string.h>

#include <vector>

#include "vg_batch.cuh"

int vg_build_params(int kind, int dim, const double *params, int nparams, VgParams *Pp, int *tab_len_out);

namespace vgbatch {
int launch_k442(int, const BatchJob *, const VgParams *, const int *, int, int, int, uint32_t, unsigned int *, size_t,
                int, int, int *, cudaStream_t);
int launch_k221(int, const BatchJob *, const VgParams *, const int *, int, int, int, uint32_t, unsigned int *, size_t,
                int, int, int *, cudaStream_t);
int launch_k222(int, const BatchJob *, const VgParams *, const int *, int, int, int, uint32_t, unsigned int *, size_t,
                int, int, int *, cudaStream_t);
int occupancy_k442(int, size_t, int *);
int occupancy_k221(int, size_t, int *);
int occupancy_k222(int, size_t, int *);
}  // namespace vgbatch

namespace {
using namespace vgbatch;

// Tile-shape variants: samples per thread of the dimension buckets 4 / 8 /
// 16, the shared-memory budget of the plan (above about 113 KB one CTA per
// SM; below it two, with a kernel compiled for 128 registers per thread) and
// what leaves shared memory first when the plan is over budget: the training
// histogram (its atomics then go to global memory) or the grid table (then
// read through L1, the histogram keeps shared-memory atomics).
struct Variant {
    int S4, S8, S16;
    size_t budget;
    int table_first;   // over budget: drop the staged grid table before the histogram
    int kernel;        // instantiation: 0 = k442, 1 = k221, 2 = k222
};
const Variant VARIANTS[] = {
    {4, 4, 2, 220 * 1024, 0, 0},   // one CTA per SM, everything staged
    {2, 2, 1, 220 * 1024, 0, 1},   // one CTA per SM, everything staged
    {2, 2, 2, 110 * 1024, 0, 2},   // two CTAs per SM, histogram in global memory
    {2, 2, 2, 110 * 1024, 1, 2},   // two CTAs per SM, grid table through L1
};
constexpr int NVARIANTS = (int)(sizeof(VARIANTS) / sizeof(VARIANTS[0]));

int kernel_of(int v) { return VARIANTS[v].kernel; }

size_t table_jobs_bytes(int njobs) { return ((size_t)njobs * sizeof(BatchJob) + 255) & ~(size_t)255; }

}  // namespace

extern "C" int vg_batch_variants(void) { return NVARIANTS; }

extern "C" size_t vg_batch_table_bytes(int njobs)
{
    return table_jobs_bytes(njobs) + (size_t)njobs * sizeof(VgParams);
}

extern "C" int vg_batch_prepare(const vg_integrator *its, int njobs, int kind, const double *params, int ldp,
                                const int *nparams, int nitn, double *out, double *res, unsigned int *sync,
                                int variant, void *table, size_t table_bytes, size_t *smem_out, int *grid_out,
                                void *stream)
{
    vg_clear_error();
    if (njobs < 1) return vg_fail(VG_ERR_VALUE, "no integrals");
    if (kind != VG_F_LORENTZ && kind != VG_F_LATTICE)
        return vg_fail(VG_ERR_UNSUPPORTED, "batched launch: Lorentzian products and the lattice action only");
    if (variant < 0 || variant >= NVARIANTS) return vg_fail(VG_ERR_VALUE, "variant %d", variant);
    if (nitn < 1) return vg_fail(VG_ERR_VALUE, "nitn < 1");
    if (table_bytes < vg_batch_table_bytes(njobs)) return vg_fail(VG_ERR_VALUE, "job table too small");
    const Variant V = VARIANTS[variant];
    std::vector<BatchJob> jobs((size_t)njobs);
    std::vector<VgParams> prm((size_t)njobs);
    size_t smem_max = 0;
    for (int j = 0; j < njobs; j++) {
        const vg_integrator *it = &its[j];
        if (it->precision != VG_F32) return vg_fail(VG_ERR_UNSUPPORTED, "batched launch computes in FP32");
        BatchJob &J = jobs[(size_t)j];
        memset(&J, 0, sizeof(J));
        int rc = vg::fill_iter_args(J.a, it, 0, nullptr);
        if (rc) return rc;
        int tab_len = 0;
        if ((rc = vg_build_params(kind, it->dim, params + (size_t)j * ldp, nparams[j], &prm[(size_t)j], &tab_len)))
            return rc;
        const int dim = it->dim;
        int S;
        if (dim <= 4) { J.dimb = 4; S = V.S4; }
        else if (dim <= 8) { J.dimb = 8; S = V.S8; }
        else if (dim <= 16) { J.dimb = 16; S = V.S16; }
        else return vg_fail(VG_ERR_UNSUPPORTED, "batched launch: dim %d above 16", dim);
        IterArgs &a = J.a;
        const int TT = vg::NT * S;
        a.tab_len = tab_len;
        a.T = TT;
        a.ncta = 1;
        const int bins = a.train;
        a.table_smem = 1;
        a.hist_smem = bins;
        vg::SmemPlan p = vg::smem_plan<float>(dim, a.maxK, TT, 1, a.hist_smem, tab_len, bins, 1);
        if (V.table_first && p.total > V.budget) {
            a.table_smem = 0;
            p = vg::smem_plan<float>(dim, a.maxK, TT, 0, a.hist_smem, tab_len, bins, 1);
        }
        if (p.total > V.budget && a.hist_smem) {
            a.hist_smem = 0;
            p = vg::smem_plan<float>(dim, a.maxK, TT, a.table_smem, 0, tab_len, bins, 1);
        }
        if (p.total > V.budget && a.table_smem) {
            a.table_smem = 0;
            p = vg::smem_plan<float>(dim, a.maxK, TT, 0, a.hist_smem, tab_len, bins, 1);
        }
        if (p.total > 220 * 1024) return vg_fail(VG_ERR_UNSUPPORTED, "shared memory plan too large");
        size_t need = p.total;
        J.adapt = (it->adapt && it->alpha > 0) ? 1 : 0;
        if (J.adapt) {
            vgadapt::AdaptArgs &ad = J.ad;
            ad.dim = dim;
            int max_old = 0;
            for (int d = 0; d < dim; d++) {
                ad.old_ninc[d] = ad.new_ninc[d] = (int)it->ninc[d];
                max_old = (int)it->ninc[d] > max_old ? (int)it->ninc[d] : max_old;
            }
            if (max_old < 2) J.adapt = 0;   // a single increment per axis: nothing to adapt
            ad.grid = it->grid;
            ad.inc = it->inc;
            ad.ldg = it->ldg;
            ad.ldi = it->ldi;
            ad.sum_f = it->sum_f;
            ad.n_f = (const unsigned long long *)it->n_f;
            ad.alpha = it->alpha;
            vg::scratch_grid(it, &ad.new_grid, &ad.new_inc);
            ad.ldg_new = it->ldg;
            ad.ldi_new = it->ldi;
            ad.max_old = max_old;
            ad.sequential = 1;
            ad.fast = 1;
            const size_t an = sizeof(double) * (2 * (size_t)max_old + vg::NT);
            need = an > need ? an : need;
        }
        J.out = out + (size_t)j * 2 * nitn;
        J.res = res + (size_t)j * 4;
        J.sync = sync != nullptr ? sync + j : nullptr;
        smem_max = need > smem_max ? need : smem_max;
    }
    cudaStream_t st = (cudaStream_t)stream;
    char *tb = (char *)table;
    VG_CUDA_CHECK(cudaMemcpyAsync(tb, jobs.data(), sizeof(BatchJob) * (size_t)njobs, cudaMemcpyHostToDevice, st));
    VG_CUDA_CHECK(cudaMemcpyAsync(tb + table_jobs_bytes(njobs), prm.data(), sizeof(VgParams) * (size_t)njobs,
                                  cudaMemcpyHostToDevice, st));
    VG_CUDA_CHECK(cudaStreamSynchronize(st));   // the host staging buffers go out of scope
    int per_sm = 0, rc = 0;
    switch (kernel_of(variant)) {
    case 0: rc = occupancy_k442(kind, smem_max, &per_sm); break;
    case 1: rc = occupancy_k221(kind, smem_max, &per_sm); break;
    default: rc = occupancy_k222(kind, smem_max, &per_sm); break;
    }
    if (rc) return rc;
    if (per_sm < 1) return vg_fail(VG_ERR_UNSUPPORTED, "batched kernel does not fit on an SM");
    *smem_out = smem_max;
    *grid_out = vg_num_sms() * per_sm;
    return VG_OK;
}

extern "C" int vg_batch_launch(const void *table, int njobs, int kind, int nitn, int nwarm, uint32_t itn0,
                               const int *order, unsigned int *queue, unsigned int *sync, int group, int *status,
                               size_t smem, int grid, int variant, void *stream)
{
    vg_clear_error();
    if (variant < 0 || variant >= NVARIANTS) return vg_fail(VG_ERR_VALUE, "variant %d", variant);
    if (nwarm < 0 || nwarm >= nitn) return vg_fail(VG_ERR_VALUE, "need 0 <= nwarm < nitn");
    cudaStream_t st = (cudaStream_t)stream;
    const BatchJob *jobs = (const BatchJob *)table;
    const VgParams *prm = (const VgParams *)((const char *)table + table_jobs_bytes(njobs));
    int g;
    if (group > 1) {   // njobs groups of `group` co-resident CTAs
        if ((int64_t)njobs * group > grid)
            return vg_fail(VG_ERR_VALUE, "group launch needs njobs*group <= %d co-resident CTAs", grid);
        if (sync == nullptr) return vg_fail(VG_ERR_VALUE, "group launch needs the sync counters");
        g = njobs * group;
        VG_CUDA_CHECK(cudaMemsetAsync(sync, 0, sizeof(unsigned int) * (size_t)njobs, st));
    } else {
        g = grid < njobs ? grid : njobs;
    }
    VG_CUDA_CHECK(cudaMemsetAsync(queue, 0, sizeof(unsigned int), st));
    switch (kernel_of(variant)) {
    case 0: return launch_k442(kind, jobs, prm, order, njobs, nitn, nwarm, itn0, queue, smem, g, group, status, st);
    case 1: return launch_k221(kind, jobs, prm, order, njobs, nitn, nwarm, itn0, queue, smem, g, group, status, st);
    default: return launch_k222(kind, jobs, prm, order, njobs, nitn, nwarm, itn0, queue, smem, g, group, status, st);
    }
}
