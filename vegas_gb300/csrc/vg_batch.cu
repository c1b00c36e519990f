// vg_batch.cu -- host side of the batched many-integral launch.
//
// vg_batch_prepare builds the device job table (per integral: its iteration
// arguments, adapt arguments, integrand parameters, output slots) and the
// shared-memory plan of each dimension bucket's tile configuration;
// vg_batch_launch runs one persistent kernel per bucket present (integrals of
// dim <= 4, <= 8, <= 16), the buckets on forked streams so that the SMs one
// bucket's kernel leaves at its end are taken by the next (no host
// synchronisation, no allocation: it can be captured in a CUDA graph).  No
// counterpart in the reference, which integrates one integrand per Integrator
// call; each integral here runs the same vegas+ iteration as
// vg_fused_iteration.
#include <string.h>

#include <mutex>
#include <vector>

#include "vg_batch.cuh"

int vg_build_params(int kind, int dim, const double *params, int nparams, VgParams *Pp, int *tab_len_out);

namespace vgbatch {
int launch_b4(int, int, const BatchJob *, const VgParams *, const int *, int, int, int, uint32_t, unsigned int *,
              size_t, int, int, int *, cudaStream_t);
int launch_b8(int, int, const BatchJob *, const VgParams *, const int *, int, int, int, uint32_t, unsigned int *,
              size_t, int, int, int *, cudaStream_t);
int launch_b16(int, int, const BatchJob *, const VgParams *, const int *, int, int, int, uint32_t, unsigned int *,
               size_t, int, int, int *, cudaStream_t);
int occupancy_b4(int, int, size_t, int *);
int occupancy_b8(int, int, size_t, int *);
int occupancy_b16(int, int, size_t, int *);
int launch_f64(const BatchJob *, const VgParams *, const int *, int, int, int, uint32_t, unsigned int *, size_t, int,
               int, int *, cudaStream_t);
int occupancy_f64(size_t, int *);
}  // namespace vgbatch

namespace {
using namespace vgbatch;

size_t table_jobs_bytes(int njobs) { return ((size_t)njobs * sizeof(BatchJob) + 255) & ~(size_t)255; }

// Shared-memory budget of a plan for `minb` CTAs per SM: the SM's 228 KB
// less the per-CTA reservation and the kernel's static shared memory.
size_t smem_budget(int minb)
{
    const size_t per = (size_t)228 * 1024 / (size_t)minb;
    const size_t cap = (size_t)220 * 1024;
    const size_t b = per > 6 * 1024 ? per - 6 * 1024 : 0;
    return b < cap ? b : cap;
}

int bucket_of(int dim) { return dim <= 4 ? 0 : (dim <= 8 ? 1 : 2); }

int occupancy_dispatch(int b, int kind, int cfg, size_t smem, int *per_sm)
{
    if (cfg == VG_BATCH_CFG_F64) return occupancy_f64(smem, per_sm);
    if (b == 0) return occupancy_b4(kind, cfg, smem, per_sm);
    if (b == 1) return occupancy_b8(kind, cfg, smem, per_sm);
    return occupancy_b16(kind, cfg, smem, per_sm);
}

int launch_dispatch(int b, int kind, int cfg, const BatchJob *jobs, const VgParams *prm, const int *order, int njobs,
                    int nitn, int nwarm, uint32_t itn0, unsigned int *queue, size_t smem, int grid, int group,
                    int *status, cudaStream_t st)
{
    if (cfg == VG_BATCH_CFG_F64)
        return launch_f64(jobs, prm, order, njobs, nitn, nwarm, itn0, queue, smem, grid, group, status, st);
    if (b == 0)
        return launch_b4(kind, cfg, jobs, prm, order, njobs, nitn, nwarm, itn0, queue, smem, grid, group, status, st);
    if (b == 1)
        return launch_b8(kind, cfg, jobs, prm, order, njobs, nitn, nwarm, itn0, queue, smem, grid, group, status, st);
    return launch_b16(kind, cfg, jobs, prm, order, njobs, nitn, nwarm, itn0, queue, smem, grid, group, status, st);
}

// Streams the bucket kernels run on besides the caller's, and the events of
// the fork and the join, per device ordinal (created once, outside any
// capture, by vg_batch_prepare; never replaced).
struct AuxStreams {
    cudaStream_t s[NBUCKET];
    cudaEvent_t fork, join[NBUCKET];
};
std::mutex g_aux_mutex;
AuxStreams *g_aux[VG_MAX_DEVICES];

int current_device(int *dev)
{
    VG_CUDA_CHECK(cudaGetDevice(dev));
    if (*dev < 0 || *dev >= VG_MAX_DEVICES) return vg_fail(VG_ERR_UNSUPPORTED, "device ordinal %d", *dev);
    return VG_OK;
}

int ensure_aux()
{
    int dev = 0, rc = current_device(&dev);
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(g_aux_mutex);
    if (g_aux[dev] != nullptr) return VG_OK;
    AuxStreams a;
    for (int b = 0; b < NBUCKET; b++) {
        VG_CUDA_CHECK(cudaStreamCreateWithFlags(&a.s[b], cudaStreamNonBlocking));
        VG_CUDA_CHECK(cudaEventCreateWithFlags(&a.join[b], cudaEventDisableTiming));
    }
    VG_CUDA_CHECK(cudaEventCreateWithFlags(&a.fork, cudaEventDisableTiming));
    g_aux[dev] = new AuxStreams(a);
    return VG_OK;
}

// The current device's streams, or nullptr before vg_batch_prepare ran on it.
AuxStreams *aux_of_current()
{
    int dev = 0;
    if (current_device(&dev)) return nullptr;
    std::lock_guard<std::mutex> lock(g_aux_mutex);
    return g_aux[dev];
}

}  // namespace

// Instrumentation: while set, vg_batch_prepare points integral j's job at
// stamps[3j .. 3j+2] (start and end of its iterations, globaltimer ns; SM).
static unsigned long long *g_batch_stamps = nullptr;

extern "C" int vg_batch_set_stamps(unsigned long long *stamps)
{
    g_batch_stamps = stamps;
    return VG_OK;
}

extern "C" int vg_batch_variants(void) { return NCONFIG; }

extern "C" size_t vg_batch_table_bytes(int njobs)
{
    return table_jobs_bytes(njobs) + (size_t)njobs * sizeof(VgParams);
}

extern "C" int vg_batch_prepare(const vg_integrator *its, int njobs, int kind, const double *params, int ldp,
                                const int *nparams, int nitn, double *out, double *res, unsigned int *sync,
                                const int *cfg, void *table, size_t table_bytes, size_t *smem_out, int *grid_out,
                                void *stream)
{
    VG_RANGE("vg_batch_prepare");
    vg_clear_error();
    if (njobs < 1) return vg_fail(VG_ERR_VALUE, "no integrals");
    if (kind != VG_F_LORENTZ && kind != VG_F_LATTICE)
        return vg_fail(VG_ERR_UNSUPPORTED, "batched launch: Lorentzian products and the lattice action only");
    for (int b = 0; b < NBUCKET; b++)
        if ((cfg[b] < 0 || cfg[b] >= NCONFIG) && cfg[b] != VG_BATCH_CFG_F64)
            return vg_fail(VG_ERR_VALUE, "bucket %d: configuration %d", b, cfg[b]);
    if (nitn < 1) return vg_fail(VG_ERR_VALUE, "nitn < 1");
    if (table_bytes < vg_batch_table_bytes(njobs)) return vg_fail(VG_ERR_VALUE, "job table too small");
    int rc = ensure_aux();
    if (rc) return rc;
    std::vector<BatchJob> jobs((size_t)njobs);
    std::vector<VgParams> prm((size_t)njobs);
    size_t smem_max[NBUCKET] = {0, 0, 0};
    int present[NBUCKET] = {0, 0, 0};
    for (int j = 0; j < njobs; j++) {
        const vg_integrator *it = &its[j];
        const int dim = it->dim;
        if (dim < 1 || dim > 16) return vg_fail(VG_ERR_UNSUPPORTED, "batched launch: dim %d outside 1..16", dim);
        const int b = bucket_of(dim);
        const int f64 = it->precision == VG_F64;
        if (f64 != (cfg[b] == VG_BATCH_CFG_F64))
            return vg_fail(VG_ERR_VALUE, "batched launch: FP64 integrals need configuration VG_BATCH_CFG_F64 "
                                         "and FP32 integrals one of the FP32 configurations");
        if (f64 && (kind != VG_F_LORENTZ || dim > F64_DIMB))
            return vg_fail(VG_ERR_UNSUPPORTED, "batched FP64 configuration: Lorentzian products of dim <= %d",
                           F64_DIMB);
        BatchJob &J = jobs[(size_t)j];
        memset(&J, 0, sizeof(J));
        if ((rc = vg::fill_iter_args(J.a, it, 0, nullptr))) return rc;
        int tab_len = 0;
        if ((rc = vg_build_params(kind, it->dim, params + (size_t)j * ldp, nparams[j], &prm[(size_t)j], &tab_len)))
            return rc;
        const BucketConfig C = f64 ? F64_CONFIG : BUCKET_CONFIGS[b][cfg[b]];
        J.bucket = b;
        present[b] = 1;
        IterArgs &a = J.a;
        const int TT = vg::NT * C.S;
        const size_t budget = smem_budget(C.minb);
        a.tab_len = tab_len;
        a.T = TT;
        a.ncta = 1;
        const int bins = a.train;
        // over budget: the grid table goes first (read through L1), then the
        // training histogram (global atomics)
        a.table_smem = 1;
        a.hist_smem = bins;
        auto plan = [&](int table, int hist) {
            return f64 ? vg::smem_plan<double>(dim, a.maxK, TT, table, hist, tab_len, bins, 1)
                       : vg::smem_plan<float>(dim, a.maxK, TT, table, hist, tab_len, bins, 1);
        };
        vg::SmemPlan p = plan(1, a.hist_smem);
        if (p.total > budget) {
            a.table_smem = 0;
            p = plan(0, a.hist_smem);
        }
        if (p.total > budget && a.hist_smem) {
            a.hist_smem = 0;
            p = plan(0, 0);
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
            ad.fast = f64 ? 0 : 1;
            const size_t an = sizeof(double) * (2 * (size_t)max_old + vg::NT);
            need = an > need ? an : need;
        }
        J.out = out + (size_t)j * 3 * nitn;
        J.res = res + (size_t)j * 4;
        J.sync = sync != nullptr ? sync + j : nullptr;
        J.stamp = g_batch_stamps != nullptr ? g_batch_stamps + 3 * (size_t)j : nullptr;
        smem_max[b] = need > smem_max[b] ? need : smem_max[b];
    }
    cudaStream_t st = (cudaStream_t)stream;
    char *tb = (char *)table;
    VG_CUDA_CHECK(cudaMemcpyAsync(tb, jobs.data(), sizeof(BatchJob) * (size_t)njobs, cudaMemcpyHostToDevice, st));
    VG_CUDA_CHECK(cudaMemcpyAsync(tb + table_jobs_bytes(njobs), prm.data(), sizeof(VgParams) * (size_t)njobs,
                                  cudaMemcpyHostToDevice, st));
    VG_CUDA_CHECK(cudaStreamSynchronize(st));   // the host staging buffers go out of scope
    for (int b = 0; b < NBUCKET; b++) {
        smem_out[b] = 0;
        grid_out[b] = 0;
        if (!present[b]) continue;
        int per_sm = 0;
        if ((rc = occupancy_dispatch(b, kind, cfg[b], smem_max[b], &per_sm))) return rc;
        if (per_sm < 1) return vg_fail(VG_ERR_UNSUPPORTED, "batched kernel (bucket %d) does not fit on an SM", b);
        smem_out[b] = smem_max[b];
        grid_out[b] = vg_num_sms() * per_sm;
    }
    return VG_OK;
}

// seg[2b], seg[2b+1]: first position and count of bucket b's integrals in
// `order`; queue[3]: one counter per bucket; group[b] > 1 (cooperative groups
// of CTAs per integral) only when a single bucket is present.
extern "C" int vg_batch_launch(const void *table, int njobs, int kind, int nitn, int nwarm, uint32_t itn0,
                               const int *order, const int *seg, unsigned int *queue, unsigned int *sync,
                               const int *group, int *status, const size_t *smem, const int *grid, const int *cfg,
                               void *stream)
{
    VG_RANGE("vg_batch_launch");
    vg_clear_error();
    if (nwarm < 0 || nwarm >= nitn) return vg_fail(VG_ERR_VALUE, "need 0 <= nwarm < nitn");
    AuxStreams *aux = aux_of_current();
    if (aux == nullptr) return vg_fail(VG_ERR_VALUE, "vg_batch_prepare was not called on this device");
    cudaStream_t st = (cudaStream_t)stream;
    const BatchJob *jobs = (const BatchJob *)table;
    const VgParams *prm = (const VgParams *)((const char *)table + table_jobs_bytes(njobs));
    int npresent = 0, anygroup = 0;
    for (int b = 0; b < NBUCKET; b++) {
        if (seg[2 * b + 1] <= 0) continue;
        npresent++;
        if ((cfg[b] < 0 || cfg[b] >= NCONFIG) && cfg[b] != VG_BATCH_CFG_F64)
            return vg_fail(VG_ERR_VALUE, "bucket %d: configuration %d", b, cfg[b]);
        if (seg[2 * b] < 0 || seg[2 * b] + seg[2 * b + 1] > njobs) return vg_fail(VG_ERR_VALUE, "bucket segment");
        if (grid[b] < 1) return vg_fail(VG_ERR_VALUE, "bucket %d was not prepared", b);
        if (group[b] > 1) {
            anygroup = 1;
            if ((int64_t)seg[2 * b + 1] * group[b] > grid[b])
                return vg_fail(VG_ERR_VALUE, "group launch needs integrals*group <= %d co-resident CTAs", grid[b]);
        }
    }
    if (npresent == 0) return vg_fail(VG_ERR_VALUE, "no integrals in the buckets");
    if (anygroup && npresent > 1)
        return vg_fail(VG_ERR_VALUE, "groups of CTAs per integral need integrals of one dimension bucket");
    if (anygroup) {
        if (sync == nullptr) return vg_fail(VG_ERR_VALUE, "group launch needs the sync counters");
        VG_CUDA_CHECK(cudaMemsetAsync(sync, 0, sizeof(unsigned int) * (size_t)njobs, st));
    }
    VG_CUDA_CHECK(cudaMemsetAsync(queue, 0, sizeof(unsigned int) * NBUCKET, st));
    // fork: the first bucket (largest dimension first) runs on the caller's
    // stream, the others on their own streams after it was enqueued
    if (npresent > 1) VG_CUDA_CHECK(cudaEventRecord(aux->fork, st));
    int first = 1;
    int joined[NBUCKET] = {0, 0, 0};
    for (int b = NBUCKET - 1; b >= 0; b--) {
        const int n = seg[2 * b + 1];
        if (n <= 0) continue;
        cudaStream_t sb = st;
        if (!first) {
            sb = aux->s[b];
            VG_CUDA_CHECK(cudaStreamWaitEvent(sb, aux->fork, 0));
        }
        const int g = group[b] > 1 ? n * group[b] : (grid[b] < n ? grid[b] : n);
        int rc = launch_dispatch(b, kind, cfg[b], jobs, prm, order + seg[2 * b], n, nitn, nwarm, itn0, queue + b,
                                 smem[b], g, group[b] > 1 ? group[b] : 1, status, sb);
        if (rc) return rc;
        if (!first) {
            VG_CUDA_CHECK(cudaEventRecord(aux->join[b], sb));
            joined[b] = 1;
        }
        first = 0;
    }
    for (int b = 0; b < NBUCKET; b++)
        if (joined[b]) VG_CUDA_CHECK(cudaStreamWaitEvent(st, aux->join[b], 0));
    return VG_OK;
}
