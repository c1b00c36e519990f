/*
 * vegas_gb300.h -- C ABI of the GB300 vegas+ hot path (libvegas_gb300.so).
 *
 * Conventions
 *   - Every entry point returns an int status (VG_OK = 0).  On failure a
 *     message is available from vg_last_error() (thread-local).
 *   - Pointers documented "device" point to GPU memory owned by the caller;
 *     the library never allocates device memory.  Scratch space is passed in
 *     as a workspace whose size comes from vg_workspace_bytes().
 *   - `stream` is a cudaStream_t passed as void*.  All device work is
 *     enqueued on it; nothing synchronises except where stated.
 *   - No torch types appear here: the Python package binds these symbols
 *     with ctypes; other hosts (C, C++, Fortran via ISO_C_BINDING) can bind
 *     them the same way.
 *
 * Each entry point names the reference code it replaces: src/vegas/_vegas.pyx
 * of gplepage/vegas 6.4.1 ("pyx:line").
 */
#ifndef VEGAS_GB300_H
#define VEGAS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VG_MAX_DIM 64

/* status codes; the Python layer maps them onto the reference's exceptions */
#define VG_OK 0
#define VG_ERR_VALUE 1       /* ValueError       (e.g. pyx:1319-1345)             */
#define VG_ERR_MEMORY 2      /* MemoryError      (pyx:1355-1356, 1440-1441)       */
#define VG_ERR_CUDA 3        /* CUDA runtime failure                                */
#define VG_ERR_NAN 4         /* "integrand evaluates to nan" ValueError, pyx:2133  */
#define VG_ERR_UNSUPPORTED 5 /* configuration outside what the kernels handle     */
#define VG_ERR_TIMEOUT 6     /* a bounded device-side wait gave up                 */

/* arithmetic of sampling / map / evaluation; sums are always FP64 */
#define VG_F32 0
#define VG_F64 1

/* built-in integrands evaluated inside the fused kernel */
#define VG_F_GAUSS 0   /* params {a, c, norm}: norm*exp(-a*sum_d (x_d-c)^2)                 */
#define VG_F_RIDGE 1   /* params {M, s}: (1/M) sum_j N_dim(x; c_j(1..1), s), c_j=(j+.5)/M     */
#define VG_F_LORENTZ 2 /* params {c[dim], w[dim]}: prod_d (w_d/pi)/((x_d-c_d)^2 + w_d^2)     */
#define VG_F_MIXTURE 3 /* params {K, sigma, c[K*dim]}: (1/K) sum_k N_dim(x; c_k, sigma)      */
#define VG_F_LATTICE 4 /* params {a, lambda}: exp(-sum_i (x_{i+1}-x_i)^2/2a + a(x_i^2/2+l x_i^4)) */
#define VG_F_CONST 5   /* params {value}                                                     */

/*
 * Device-resident per-iteration scalars.  `sum_sigf` carries the vegas+
 * stratification normaliser between iterations (Integrator.sum_sigf,
 * pyx:2209-2215); the rest is written by each iteration.
 */
typedef struct vg_stats {
    double sum_sigf;       /* in: used by the allocation; out: new value        */
    double mean;           /* iteration estimate (component 0)                  */
    double var;            /* its variance                                      */
    double neval_sigf;     /* neval_frac*neval/sum_sigf used by the allocation  */
    int64_t neval;         /* evaluations in the iteration (last_neval)         */
    int64_t range_lo;      /* neval_hcube_range                                 */
    int64_t range_hi;
    int64_t ntiles;        /* tiles of the iteration                            */
    int32_t nan_seen;      /* integrand returned NaN                            */
    int32_t sigf_reset;    /* sum_sigf was 0: sigf set to 1 (pyx:2210-2215)     */
    int32_t status;        /* device-side status (VG_ERR_*)                     */
    int32_t pad;
} vg_stats;

/*
 * One integrator (or one of many in a batch): geometry, adaptive map, vegas+
 * stratification state, training histogram and scratch.  All pointers are
 * device pointers except where noted.  Mirrors the state the reference keeps
 * in Integrator/AdaptiveMap (pyx:834-1446, _vegas.pxd:21-70).
 */
typedef struct vg_integrator {
    int32_t dim;
    int32_t precision;             /* VG_F32 or VG_F64                          */
    int64_t nhcube;                /* prod(nstrat)                              */
    int64_t nstrat[VG_MAX_DIM];    /* host values                               */
    int64_t ninc[VG_MAX_DIM];      /* host values                               */
    double *grid;                  /* [dim, ldg] x-space nodes                  */
    double *inc;                   /* [dim, ldi] increments                     */
    int64_t ldg, ldi;
    double *sigf;                  /* [nhcube] damped per-hypercube sdev        */
    double *sum_f;                 /* [dim, ldi] training sums (fdv2)           */
    uint64_t *n_f;                 /* [dim, ldi] training counts                */
    vg_stats *stats;               /* device scalars                            */
    void *work;                    /* workspace, vg_workspace_bytes() bytes     */
    size_t work_bytes;
    int64_t neval;
    double neval_frac;
    int64_t min_neval_hcube;
    int64_t max_neval_hcube;
    double alpha;
    double beta;
    int32_t adapt;                 /* Integrator.adapt                          */
    int32_t adapt_to_errors;       /* must be 0 for now                         */
    uint64_t seed;                 /* Philox key                                */
    uint32_t stream_id;            /* Philox counter word: integral id          */
    int32_t tile;                  /* samples per tile (0 = default)            */
} vg_integrator;

/* ---------------------------------------------------------------- library */
const char *vg_last_error(void);
int vg_version(void);
/* sizeof(vg_integrator) for which=0, sizeof(vg_stats) for which=1 (binding check) */
size_t vg_struct_size(int which);

/* --------------------------------------------------------------- host-side */
/*
 * Stratification and grid sizes, Integrator.set pyx:1335-1407.
 * mode 0: strata from neval (pyx:1346-1366); mode 1: explicit nstrat (sets
 * *neval when neval_given==0, pyx:1335-1345); mode 2: keep nstrat_in.
 * Returns VG_ERR_VALUE / VG_ERR_MEMORY as the reference raises.
 */
int vg_set_strata(int dim, int mode, int64_t *neval, int neval_given, const int64_t *nstrat_in,
                  double neval_frac, double beta, int adapt_to_errors, int uniform_nstrat,
                  double max_mem, int minimize_mem, int64_t maxinc_axis, int64_t *nstrat_out,
                  int64_t *ninc_out, int64_t *min_neval_hcube_out);

/* Set a device record to zero but for sum_sigf, the vegas+ normaliser the
 * next allocation uses (the value Integrator carries between iterations,
 * pyx:2209-2215); enqueued on `stream`. */
int vg_stats_reset(vg_stats *stats, double sum_sigf, void *stream);

/* Upper bound on the evaluations of one iteration (capacity of x / f buffers). */
int64_t vg_neval_cap(const vg_integrator *it);

/* Workspace for an iteration of at most neval_cap evaluations (bytes);
 * neval_cap <= 0 uses vg_neval_cap(it).  Zero it before its first use (and
 * after a change of the strata): the single-pass allocation keeps its block
 * ticket and epoch words in it. */
size_t vg_workspace_bytes(const vg_integrator *it, int64_t neval_cap);

/* -------------------------------------------------------- AdaptiveMap ops */
/* AdaptiveMap.make_uniform, pyx:205-241. xl/xu/ninc are host arrays. */
int vg_make_uniform(int dim, const int64_t *ninc, const double *xl, const double *xu,
                    double *grid, int64_t ldg, double *inc, int64_t ldi, void *stream);

/*
 * AdaptiveMap.adapt, pyx:467-594 (smoothing, damping, regrid to new_ninc).
 * old_ninc/new_ninc are host arrays; sum_f/n_f may be NULL (no training
 * data).  The new grid must not alias the old one.
 */
int vg_adapt(int dim, const int64_t *old_ninc, const int64_t *new_ninc, const double *grid,
             const double *inc, int64_t ldg, int64_t ldi, const double *sum_f,
             const uint64_t *n_f, double alpha, double *new_grid, double *new_inc,
             int64_t ldg_new, int64_t ldi_new, void *stream);

/* AdaptiveMap.map, pyx:310-360: y[n,dim] -> x[n,dim], jac[n] (dtype VG_F32/VG_F64). */
int vg_map(int dim, const int64_t *ninc, const double *grid, const double *inc, int64_t ldg,
           int64_t ldi, int64_t n, const void *y, void *x, void *jac, int dtype, void *stream);
/* AdaptiveMap.invmap (_vegas.pyx:362-413): y[n, dim] and jac[n] for x[n, dim]
 * (searchsorted per axis; y = 0 / 1 outside the grid), FP64 arithmetic,
 * dtype VG_F32 / VG_F64 for x, y and jac. */
int vg_invmap(int dim, const int64_t *ninc, const double *grid, const double *inc, int64_t ldg,
              int64_t ldi, int64_t n, const void *x, void *y, void *jac, int dtype, void *stream);
/* AdaptiveMap.jac1d (_vegas.pyx:265-295): out[n, dim] = dx[d]/dy[d] at y[n, dim]
 * (dtype VG_F32 / VG_F64 for y and out). */
int vg_jac1d(int dim, const int64_t *ninc, const double *inc, int64_t ldi, int64_t n, const void *y,
             void *out, int dtype, void *stream);

/* AdaptiveMap.add_training_data, pyx:421-464 (accumulates into sum_f / n_f). */
int vg_add_training_data(int dim, const int64_t *ninc, int64_t ldi, int64_t n, const void *y,
                         const void *f, int dtype, double *sum_f, uint64_t *n_f, void *stream);

/* ------------------------------------------------------ Integrator ops */
/*
 * Allocation of evaluations to hypercubes, Integrator._random_batch
 * pyx:1692-1710 (whole iteration at once): per-hypercube counts from sigf,
 * offsets, neval_hcube_range and the tile schedule.  Writes it->stats.
 */
int vg_allocate(const vg_integrator *it, void *stream);

/*
 * Integration points of the current allocation, pyx:1731-1752: x[n,dim]
 * (precision dtype), optional y[n,dim], wgt[n] (FP64) and hcube[n].  u is an
 * optional injected [n,dim] FP64 array of uniforms (ran_array_generator,
 * pyx:1676-1680); NULL draws Philox4x32-10 keyed by (seed, itn, sample).
 * n_cap is the capacity of the output arrays (>= stats->neval).
 */
int vg_sample(const vg_integrator *it, uint32_t itn, const double *u, void *x, void *y,
              double *wgt, int64_t *hcube, int64_t n_cap, void *stream);

/*
 * Per-hypercube two-pass reduction of the integrand values f[n] (dtype),
 * pyx:2136-2193, with the training histogram (pyx:2173, 2196-2197), the new
 * sigf and the iteration mean/var/sum_sigf (written to it->stats).
 */
int vg_reduce(const vg_integrator *it, uint32_t itn, const double *u, const void *f, int f_dtype,
              void *stream);

/*
 * The same pair with the samples kept between them, so that the reduction
 * streams what the sampler stored instead of regenerating every sample
 * (Philox draws, hypercube walk, map): vg_sample_keep writes what vg_sample
 * writes and, into `keep` (device, vg_keep_bytes(it, n_cap) bytes), each
 * sample's Jacobian (FP32 / FP64 by precision) and its training bins (16-bit
 * per axis); vg_reduce_kept then reads f, the Jacobians and the bins and
 * gives the same results as vg_reduce, bit for bit (itn and u as given to
 * the sampler).  Together they replace
 * the batch loop of Integrator.__call__ for a user integrand (pyx:2096-2197).
 */
size_t vg_keep_bytes(const vg_integrator *it, int64_t n_cap);
int vg_sample_keep(const vg_integrator *it, uint32_t itn, const double *u, void *x, void *y,
                   double *wgt, int64_t *hcube, int64_t n_cap, void *keep, size_t keep_bytes,
                   void *stream);
int vg_reduce_kept(const vg_integrator *it, uint32_t itn, const double *u, const void *f, int f_dtype,
                   const void *keep, size_t keep_bytes, void *stream);

/*
 * Fused iteration for a built-in integrand: sampling, map, evaluation,
 * reduction and training histogram in one persistent kernel (the whole
 * body of Integrator.__call__'s batch loop, pyx:2096-2197).  params are host
 * doubles.  Call vg_allocate first.
 */
int vg_fused_iteration(const vg_integrator *it, uint32_t itn, const double *u, int kind,
                       const double *params, int nparams, void *stream);

/*
 * End of iteration, pyx:2209-2217: adapt the map from the training
 * histogram (when alpha > 0 and adapt) and clear the histogram.  Uses the
 * workspace for the new grid.
 */
int vg_end_iteration(const vg_integrator *it, void *stream);

/*
 * One full iteration for a built-in integrand (pyx:2086-2217: allocation,
 * the fused batch loop, the iteration sums, the map adapt) in one call:
 * vg_allocate + vg_fused_iteration + vg_end_iteration, with the adapt on a
 * forked stream concurrently with the finalize when adapt_to_errors is off
 * (the adapt needs only the tile kernel's training histogram); joined back
 * into `stream` before returning.  Call it once outside any stream capture
 * before capturing it (the first call on a device creates the forked stream).
 */
int vg_iterate(const vg_integrator *it, uint32_t itn, int kind, const double *params, int nparams,
               void *stream);

/*
 * One vegas+ iteration (allocation, fused evaluation + reduction, adapt) for
 * a built-in integrand that allocates no device memory.  No counterpart in
 * the reference: it exists for callers that cannot allocate device memory --
 * plug-ins whose host application owns all device memory through its own
 * pool, services under a hard device-memory budget, callers that must not
 * allocate on their iteration path.  The caller still provides the
 * integrator's inputs and outputs (grid, inc, sigf, training histogram,
 * stats); it->work / it->work_bytes are ignored.  Scratch is a static device
 * array of VG_NOALLOC_SCRATCH_BYTES held by every GPU that loads the library
 * until the process exits; an iteration whose vg_workspace_bytes() exceeds it
 * fails with VG_ERR_MEMORY.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) and caches it per device; make that
 * first call before any stream capture.  The cache assumes the device's
 * primary context stays alive (after a cudaDeviceReset the address may
 * change).  All calls share the one array: calls that overlap on the
 * GPU (other streams, other threads) race and must be serialised by the
 * caller.  Every scratch region is rewritten before it is read; the tile
 * counter is zeroed on every call.
 */
#define VG_NOALLOC_SCRATCH_BYTES (16 * 1024 * 1024)
int vg_iteration_noalloc(const vg_integrator *it, uint32_t itn, const double *u, int kind,
                         const double *params, int nparams, void *stream);

/*
 * Array-valued integrands (reference Integrator.__call__ with fcn_size s > 1,
 * _vegas.pyx:2136-2197): after vg_reduce has run on component 0 (sigf and
 * the training histogram use it only), the iteration's mean[s] and
 * (co)variance var[s*s] of all components: f[n, s] (FP32 or FP64, row-major),
 * wgt[n] the sampler's weights (vg_sample).  correlate != 0: full covariance
 * with the reference's EPSILON rule (s <= 6); else the diagonal (s <= 16).
 * work: vg_reduce_array_work_bytes(s, correlate) device bytes.
 */
int vg_reduce_array(const vg_integrator *it, const void *f, int f_dtype, int s, int correlate,
                    const double *wgt, double *mean, double *var, void *work, size_t work_bytes,
                    void *stream);
size_t vg_reduce_array_work_bytes(int s, int correlate);

/* ------------------------------------------------------ learned proposal */
/*
 * Coupling-layer normalising flow with piecewise-quadratic transforms on the
 * unit cube (no counterpart in the reference: vegas has no learned
 * proposal).  It is composed after the AdaptiveMap: vegas samples zhat in the
 * unit cube, the flow maps it to z, the integration box maps z to x.
 * Parameters theta follow the layout of the FP64 checker
 * (oracle/flow_oracle.py); `mirror` holds BF16 copies of the dense layers for
 * the tensor cores (vg_flow_mirror_elems() 16-bit elements, rebuilt by
 * vg_flow_refresh after any change of theta).
 */
typedef struct vg_flow {
    int32_t dim, nlayers, K, hidden;   /* dim <= 16, nlayers <= 8, K <= 48, hidden == 128 */
    float *theta;                      /* [nparams] FP32 parameters                       */
    void *mirror;                      /* BF16 dense-layer copies                          */
    float *grad;                       /* [nparams] gradient accumulator (caller zeroes)   */
    float *adam_m, *adam_v;            /* [nparams] Adam moments                           */
    double *loss;                      /* [1] accumulated -sum w logdet                    */
} vg_flow;

int64_t vg_flow_nparams(int dim, int nlayers, int K, int hidden);
int64_t vg_flow_mirror_elems(int dim, int nlayers, int K, int hidden);
/* Workspace of vg_flow_grad for n rows (bytes). */
int64_t vg_flow_train_bytes(const vg_flow *fl, int64_t n);
int vg_flow_refresh(const vg_flow *fl, void *stream);
/* Sampling direction: zhat[n,dim] -> z[n,dim]; logdet[n] = sum log pdf, so
 * log|dz/dzhat| = -logdet. */
int vg_flow_sample(const vg_flow *fl, int64_t n, const float *zhat, float *z, float *logdet,
                   void *stream);
/* Density direction: z -> zhat, logdet = log q_flow(z). */
int vg_flow_density(const vg_flow *fl, int64_t n, const float *z, float *zhat, float *logdet,
                    void *stream);
/* Gradient of loss = -sum_i w_i logdet(z_i) w.r.t. theta, accumulated into fl->grad
 * (and the loss into fl->loss): forward and backward kernels, BF16 MMAs. */
int vg_flow_grad(const vg_flow *fl, int64_t n, const float *z, const float *w, void *work,
                 size_t work_bytes, void *stream);
/*
 * Training batch for the flow from one iteration's samples: m samples drawn
 * uniformly (Philox keyed by seed, step) from the n samples of the
 * iteration; zs[m,dim] = z of the drawn samples, ws[m] = their weights
 * normalised to mean 1: (|f_i| wgt_i)^2 neval_h[hc_i] (chi2 != 0: variance
 * loss) or |f_i| wgt_i (KL), where f is the integrand seen by the
 * stratification, wgt the sampler's weight and hc the hypercube.  scratch:
 * device doubles [m + 1].  Two kernels, no host synchronisation.
 */
int vg_flow_train_batch(int64_t n, int64_t m, uint64_t seed, uint32_t step, int dim, const float *z,
                        const float *f, const double *wgt, const int64_t *hc, const int32_t *neval_h,
                        int chi2, float *zs, float *ws, double *scratch, void *stream);
/* grad = 0, loss = 0 (before accumulating a new gradient). */
int vg_flow_zero_grad(const vg_flow *fl, void *stream);
/* Adam step on theta with gradient grad*scale (clipped at +-clip), then refresh. */
int vg_flow_adam(const vg_flow *fl, float scale, float lr, float beta1, float beta2, float eps,
                 int step, float clip, void *stream);
/* Device status of the flow kernels: VG_ERR_TIMEOUT when a bounded wait of
 * the tensor-core pass gave up (the pass then stopped early); reset clears it.
 * Synchronises with the device. */
int vg_flow_status(int *status, int reset);
/* 1: run inference on the mma.sync kernels even where the tcgen05 pass
 * applies (for comparisons); 0: default. */
int vg_flow_set_path(int legacy);

/*
 * Built-in integrand at given points (FP32): f[i] = vol * f(lo + width * z_i)
 * * jac[i] * exp(-logdet[i]) with z[n,dim], vol = prod(width), jac and
 * logdet optional (NULL).  The evaluation step of the flow path, where the
 * points come from the sampler, the flow and the map instead of the fused
 * kernel.  Replaces the integrand call of Integrator.__call__
 * (_vegas.pyx:2126-2129) for the built-in integrands.  lo, width: host
 * arrays [dim].
 */
int vg_eval_points(int kind, const double *params, int nparams, int dim, int64_t n,
                   const float *z, const double *lo, const double *width, const float *logdet,
                   const float *jac, float *f, void *stream);
/* out[i] = f[i] * jac[i] * exp(-logdet[i]) for integrand values computed by
 * the caller (jac, logdet optional). */
int vg_weight_points(int64_t n, const float *f, const float *jac, const float *logdet, float *out,
                     void *stream);

/* ----------------------------------------------- many integrals, one launch */
/*
 * Batched vegas+ (no counterpart in the reference, which integrates one
 * integrand per Integrator call): njobs independent integrals -- each
 * described by its own vg_integrator (dimension <= 16, FP32, its own device
 * grid, inc, sigf, training histogram, stats and workspace) and built-in
 * integrand parameters (kind VG_F_LORENTZ or VG_F_LATTICE; params + j*ldp,
 * nparams[j] values) -- run nitn iterations each in one persistent kernel
 * per dimension bucket (bucket 0: dim <= 4, 1: dim <= 8, 2: dim <= 16),
 * the buckets' kernels on forked streams joined back into `stream`.
 * cfg[3] picks each bucket's tile configuration (0 .. vg_batch_variants()-1:
 * samples per thread and CTAs per SM); vg_batch_prepare copies the job table
 * (vg_batch_table_bytes) to the device and returns each bucket's dynamic
 * shared memory smem[3] and co-resident grid grid[3] (0 for a bucket
 * without integrals).  Queue mode (group[b] <= 1): one CTA per integral at a
 * time, bucket b's integrals taken from a queue (queue: device uint[3]) in
 * the order order[seg[2b] .. seg[2b] + seg[2b+1]) (device int[njobs],
 * e.g. largest first).  Group mode (group[b] = G >= 2, one bucket only,
 * its integrals * G <= grid[b]): a cooperative launch in which G CTAs share
 * each integral's tiles (sync: device uint[njobs] barrier counters).  Each
 * iteration is the same allocation / fused evaluation + reduction / adapt
 * as vg_fused_iteration; out (device double[njobs][nitn][3]) receives every
 * iteration's mean, variance and number of evaluations, res (device double[njobs][4]) the weighted
 * average over the iterations after the first nwarm (mean, sdev, chi2, dof).
 * stats->sum_sigf of each integral must hold its starting value (nhcube for
 * a fresh one).  cfg[b] = VG_BATCH_CFG_F64 selects the FP64 parity
 * configuration instead: integrals with precision VG_F64 (Lorentzian
 * products of dim <= 8), sampling, map, evaluation and every sum in FP64, the
 * arithmetic of vg_fused_iteration's FP64 mode, for checks against the CPU
 * oracle; FP32 integrals need one of the FP32 configurations.  status (device int) becomes VG_ERR_TIMEOUT if a bounded
 * group barrier gave up.  vg_batch_launch neither allocates nor
 * synchronises, so it can be captured in a CUDA graph (after a
 * vg_batch_prepare on the same device, which creates the forked streams).
 */
#define VG_BATCH_CFG_F64 16
int vg_batch_variants(void);
size_t vg_batch_table_bytes(int njobs);
int vg_batch_prepare(const vg_integrator *its, int njobs, int kind, const double *params, int ldp,
                     const int *nparams, int nitn, double *out, double *res, unsigned int *sync, const int *cfg,
                     void *table, size_t table_bytes, size_t *smem, int *grid, void *stream);
int vg_batch_launch(const void *table, int njobs, int kind, int nitn, int nwarm, uint32_t itn0, const int *order,
                    const int *seg, unsigned int *queue, unsigned int *sync, const int *group, int *status,
                    const size_t *smem, const int *grid, const int *cfg, void *stream);

/* Instrumentation of the batched launch: while set (device
 * uint64[3 * njobs], NULL = off), vg_batch_prepare makes each integral j
 * record the start and end of its iterations (globaltimer, ns) and its SM in
 * stamps[3j .. 3j+2]. */
int vg_batch_set_stamps(unsigned long long *stamps);

/* Instrumentation: while set (device counter, NULL = off), the FP32 ridge
 * adds the number of Gaussian terms it evaluates -- the ones that can be
 * nonzero in FP32; the rest are exactly zero and skipped. */
int vg_set_term_counter(unsigned long long *count);

/* Bounded device-side waits (the allocation's look-back over its
 * predecessors' published totals; the batched launch's group barriers, four
 * times as many polls): how many polls a wait makes before it gives up and
 * the iteration reports VG_ERR_TIMEOUT in its vg_stats.status (the batched
 * launch in its status word) with no tiles scheduled.  Negative: the default
 * (2^24).  Read when an iteration's arguments are filled (vg_allocate,
 * vg_iterate, vg_iteration_noalloc, vg_batch_prepare).  No counterpart in the
 * reference, which has no device waits; its errors surface as exceptions
 * (pyx:2133-2134, 1355-1356), which the Python layer raises for a status. */
int vg_set_wait_budget(int64_t iters);

/* Tuning: how FP32 iterations of the many-term ridge run -- 0 automatic
 * (currently the fused kernel), 1 the single fused evaluate+reduce kernel,
 * 2 split into an evaluation kernel that writes f and a reduction kernel
 * that reads it back. */
int vg_set_eval_split(int policy);

/* Tuning of the tile kernels: samples per thread of the fused FP32 ridge for
 * dim <= 4 (0 automatic = 2, four CTAs per SM; or 4); grid table and
 * training histogram in shared memory (-1 automatic, 0 off, 1 on where it
 * fits). */
int vg_set_tile_tuning(int s_dim4, int table_smem, int hist_smem);

/* Tuning of the drop-in path's FP32 kernels at dim <= 4: samples per thread
 * of vg_sample / vg_sample_keep (0 automatic, or 2, 4, 8) and of
 * vg_reduce_kept (0 automatic, or 2, 4). */
int vg_set_dropin_tuning(int s_points, int s_reduce);

/* ------------------------------------------------------------- probes */
/* Throughput probes used for roofline denominators (see bench.py). */
int vg_probe_mufu_ex2(float *out, int64_t nthreads, int iters, void *stream);
int vg_probe_fp64_fma(double *out, int64_t nthreads, int iters, void *stream);
int vg_probe_fp32_fma(float *out, int64_t nthreads, int iters, void *stream);
/* tcgen05 check: D[128 x N] = A[128 x K] B[N x K]^T, bf16 inputs, FP32
 * output.  A is [128][K] (K-major) or, with a_mn, [K][128] (MN-major); B is
 * [N][K] or, with b_mn, [K][N].  status[0] = 1 if the bounded wait gave up. */
int vg_probe_umma_gemm(const void *A, const void *B, float *D, int N, int K, int a_mn, int b_mn, int *status,
                       void *stream);

#ifdef __cplusplus
}
#endif
#endif /* VEGAS_GB300_H */
