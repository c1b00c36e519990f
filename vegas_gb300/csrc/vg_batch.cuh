// vg_batch.cuh -- many independent vegas+ integrals in one persistent launch.
//
// One CTA runs one integral at a time, all of its iterations back to back:
// allocation of evaluations to hypercubes (pyx:1692-1706), the fused tile
// body of the single-integral kernel over all of the integral's tiles
// (sampling, map, integrand, two-pass per-hypercube reduction, training
// histogram), the merge of hypercubes cut by tile boundaries and the
// iteration sums (finalize), AdaptiveMap.adapt (pyx:467-594), and at the end
// the weighted average over the iterations after the warm-up ones
// (RAvg.add, pyx:2392-2410) -- all in FP64 where the single-integral path
// is.  CTAs take integrals from an atomic queue in an order given by the
// host (largest first), so nothing crosses CTAs and the launch needs no
// grid-wide synchronisation.
#pragma once
#include "vg_adapt.cuh"
#include "vg_tile.cuh"

namespace vgbatch {
using namespace vg;

struct BatchJob {
    IterArgs a;                  // per-integral arguments (its own workspace)
    vgadapt::AdaptArgs ad;       // adapt: grid -> scratch grid of the workspace
    double *out;                 // [nitn][3] iteration mean, variance, evaluations
    double *res;                 // [4] weighted mean, sdev, chi2, dof
    unsigned int *sync;          // group barrier counter (group mode)
    int bucket;                  // dimension bucket: 0 (dim <= 4), 1 (<= 8), 2 (<= 16)
    int adapt;                   // adapt the map after each iteration
    unsigned long long *stamp;   // instrumentation (or nullptr): [0] start, [1] end (globaltimer ns), [2] SM
};

__device__ __forceinline__ unsigned long long vg_globaltimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned int vg_smid()
{
    unsigned int r;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
    return r;
}

// Barrier of the G CTAs working on one integral (group mode; the launch is
// cooperative, so they are co-resident).  Thread 0 releases this CTA's
// writes, arrives, and waits (at most 4 wait_iters polls) until all G
// arrived `round` times.
// Returns false when the wait gave up.
__device__ __forceinline__ bool group_barrier(unsigned int *ctr, unsigned int target, uint32_t wait_iters)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(ctr, 1u);
        int ok = 0;
        const uint64_t budget = 4ull * wait_iters;
        for (uint64_t i = 0; i < budget; i++) {
            unsigned int v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
            if (v >= target) {
                ok = 1;
                break;
            }
            __nanosleep(256);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

constexpr int APER = 4;          // hypercubes per thread and pass of the allocation

// Allocation of one iteration by one CTA: neval_h, offsets, tile heads,
// totals in the integral's stats (the three allocation kernels' work).
static __device__ __noinline__ void cta_alloc(const IterArgs &a, int64_t *scan)
{
    const int tid = threadIdx.x;
    build_tablef(a, tid, NT);   // the FP32 grid table of this iteration
    vg_stats *st = a.stats;
    const double sum_sigf = st->sum_sigf;
    const double nsf = (a.beta > 0 && sum_sigf > 0)
                           ? __ddiv_rn(__dmul_rn(a.neval_frac, (double)a.neval), sum_sigf)
                           : 0.0;
    const int64_t mx = a.max_neval_hcube > a.min_neval_hcube ? a.max_neval_hcube : a.min_neval_hcube;
    const int64_t avg = (int64_t)((double)a.neval / (double)a.H);
    int64_t run = 0, mxn = 0;
    for (int64_t base = 0; base < a.H; base += (int64_t)NT * APER) {
        int64_t loc[APER];
        int64_t s = 0;
#pragma unroll
        for (int k = 0; k < APER; k++) {
            const int64_t h = base + (int64_t)tid * APER + k;
            int64_t n = 0;
            if (h < a.H) {
                if (a.adaptive_alloc) {
                    n = (int64_t)__dmul_rn(a.sigf[h], nsf) + a.min_neval_hcube;
                    if (n > mx) n = mx;
                } else {
                    n = avg;
                }
                mxn = n > mxn ? n : mxn;
            }
            loc[k] = n;
            s += n;
        }
        scan[tid] = s;
        __syncthreads();
        for (int off = 1; off < NT; off <<= 1) {
            const int64_t add = tid >= off ? scan[tid - off] : 0;
            __syncthreads();
            scan[tid] += add;
            __syncthreads();
        }
        int64_t off = run + scan[tid] - s;
        const int64_t total = scan[NT - 1];
#pragma unroll
        for (int k = 0; k < APER; k++) {
            const int64_t h = base + (int64_t)tid * APER + k;
            if (h >= a.H) break;
            const int64_t n = loc[k];
            a.neval_h[h] = (int32_t)n;
            a.offsets[h] = off;
            for (int64_t tt = (off + BASE_TILE - 1) / BASE_TILE; tt * BASE_TILE < off + n; tt++)
                if (tt < a.ntiles_cap) a.tile_h0[tt] = h;
            off += n;
        }
        run += total;
        __syncthreads();
    }
    // block maximum of the counts
    scan[tid] = mxn;
    __syncthreads();
    for (int o = NT / 2; o > 0; o >>= 1) {
        if (tid < o) scan[tid] = scan[tid + o] > scan[tid] ? scan[tid + o] : scan[tid];
        __syncthreads();
    }
    if (tid == 0) {
        const int64_t N = run;
        int64_t ntiles = (N + BASE_TILE - 1) / BASE_TILE;
        a.offsets[a.H] = N;
        st->neval = N;
        st->neval_sigf = nsf;
        st->range_lo = a.min_neval_hcube;
        st->range_hi = a.adaptive_alloc ? (scan[0] > a.min_neval_hcube ? scan[0] : a.min_neval_hcube)
                                        : a.min_neval_hcube;
        if (N > a.ncap || ntiles + 1 > a.ntiles_cap) {
            st->status = VG_ERR_MEMORY;
            ntiles = 0;
        } else {
            st->status = VG_OK;
            a.tile_h0[ntiles] = a.H;
        }
        st->ntiles = ntiles;
        st->nan_seen = 0;
        *a.counter = 0ull;
    }
    __syncthreads();
}

// Iteration sums of one integral by one CTA: the tile body's partial sums
// (parts[0]) plus the Chan et al. merge of every hypercube cut by tile
// boundaries (the finalize kernels' work); sum_sigf and the constant-integrand
// reset (pyx:2209-2215).
static __device__ __noinline__ void cta_finalize(const IterArgs &a, int ngroup, VgKSum *red, int *flag)
{
    // the group CTAs' float-float partials and the cut hypercubes, merged
    // and summed in float-float, converted to FP64 once (FP32 mode)
    const int tid = threadIdx.x;
    vg_stats *st = a.stats;
    const int64_t N = st->neval;
    const int64_t ntiles = st->ntiles ? (N + a.T - 1) / a.T : 0;
    float r6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (tid < ngroup && ntiles > 0) {   // the partial sums of each CTA of the group
        const TilePart p = a.parts[tid];
        ff_unpack(p.mean.s, r6[0], r6[1]);
        ff_unpack(p.var.s, r6[2], r6[3]);
        ff_unpack(p.sigf.s, r6[4], r6[5]);
    }
    for (int64_t t = tid; t < ntiles; t += NT) merge_cut_ff(a, t, ntiles, r6[0], r6[1], r6[2], r6[3], r6[4], r6[5]);
    ff_block_reduce6<NT>(r6, reinterpret_cast<float *>(red));
    if (tid == 0) {
        st->mean = vg_ff_value(r6[0], r6[1]);
        st->var = vg_ff_value(r6[2], r6[3]);
        st->sigf_reset = 0;
        *flag = 0;
        if (a.adaptive) {
            const double ss = vg_ff_value(r6[4], r6[5]);
            if (ss > 0) {
                st->sum_sigf = ss;
            } else {
                st->sum_sigf = (double)a.H;
                st->sigf_reset = 1;
                *flag = 1;
            }
        }
    }
    __syncthreads();
    if (*flag)
        for (int64_t h = tid; h < a.H; h += NT) a.sigf[h] = 1.0;
    __syncthreads();
}

// FP64 mode: the hypercube whose first piece is the tail record of tile t,
// merged in FP64 with its pieces in the following tiles (Chan et al.'s
// parallel-variance update, the FP64 finalize's formulas); adds its mean,
// variance and sigf to the compensated sums and stores its sigf.
static __device__ __noinline__ void merge_cut_f64(const IterArgs &a, int64_t t, int64_t ntiles, VgKSum &cm,
                                                  VgKSum &cv, VgKSum &cs)
{
    const TileRec r = a.recs[2 * t + 1];
    if (r.h < 0) return;
    double n = r.n, Sx = r.S, Q = r.Q, D = r.D;
    for (int64_t t2 = t + 1; t2 < ntiles; t2++) {
        const TileRec q = a.recs[2 * t2];
        if (q.h != r.h) break;
        const double n2 = n + q.n;
        const double delta = q.S / q.n - Sx / n;
        Q = Q + q.Q + delta * delta * (n * q.n / n2);
        Sx += q.S;
        D += q.D;
        n = n2;
        if (!q.spans) break;
    }
    const double num = __dsub_rn(__dmul_rn(n, Q), __dmul_rn(D, D));
    const double vh = __ddiv_rn(num, __dsub_rn(n, 1.));
    cm.add(__dadd_rn(Sx, D));
    cv.add(vh);
    if (a.adaptive) {
        const double sg = pow(fabs(vh), a.beta_half);
        a.sigf[r.h] = sg;
        cs.add(sg);
    }
}

// FP64 mode (the parity configuration of the batched launch): the group
// CTAs' FP64 partials plus the merged cut hypercubes, compensated FP64 sums
// in a fixed order; sum_sigf and the constant-integrand reset as
// cta_finalize.
static __device__ __noinline__ void cta_finalize_f64(const IterArgs &a, int ngroup, VgKSum *red, int *flag)
{
    const int tid = threadIdx.x;
    vg_stats *st = a.stats;
    const int64_t N = st->neval;
    const int64_t ntiles = st->ntiles ? (N + a.T - 1) / a.T : 0;
    VgKSum cm = {0.0, 0.0}, cv = {0.0, 0.0}, cs = {0.0, 0.0};
    if (tid < ngroup && ntiles > 0) {
        const TilePart p = a.parts[tid];
        cm = p.mean;
        cv = p.var;
        cs = p.sigf;
    }
    for (int64_t t = tid; t < ntiles; t += NT) merge_cut_f64(a, t, ntiles, cm, cv, cs);
    const VgKSum M = vg_block_ksum<NT>(cm, red);
    const VgKSum V = vg_block_ksum<NT>(cv, red);
    const VgKSum Sg = vg_block_ksum<NT>(cs, red);
    if (tid == 0) {
        st->mean = M.value();
        st->var = V.value();
        st->sigf_reset = 0;
        *flag = 0;
        if (a.adaptive) {
            const double ss = Sg.value();
            if (ss > 0) {
                st->sum_sigf = ss;
            } else {
                st->sum_sigf = (double)a.H;
                st->sigf_reset = 1;
                *flag = 1;
            }
        }
    }
    __syncthreads();
    if (*flag)
        for (int64_t h = tid; h < a.H; h += NT) a.sigf[h] = 1.0;
    __syncthreads();
}

// End of iteration: adapt the map (one axis after another), copy the new
// grid back, clear the training histogram (vg_end_iteration's work).
static __device__ __noinline__ void cta_adapt(const BatchJob &J, const IterArgs &a, unsigned char *smem)
{
    const int tid = threadIdx.x;
    const vgadapt::AdaptArgs &ad = J.ad;
    double *avg = (double *)smem;
    double *tmp = avg + ad.max_old;
    double *part = tmp + ad.max_old;
    for (int i = tid; i < ad.max_old; i += NT) avg[i] = 1.0;
    __syncthreads();
    for (int d = 0; d < ad.dim; d++) vgadapt::adapt_axis<NT>(ad, d, avg, tmp, part);
    __syncthreads();
    for (int d = 0; d < ad.dim; d++) {
        const int K = ad.old_ninc[d];
        double *g = const_cast<double *>(ad.grid) + d * ad.ldg;
        double *inc = const_cast<double *>(ad.inc) + d * ad.ldi;
        for (int i = tid; i <= K; i += NT) g[i] = ad.new_grid[d * ad.ldg_new + i];
        for (int i = tid; i < K; i += NT) {
            inc[i] = ad.new_inc[d * ad.ldi_new + i];
            a.sum_f[d * a.ldi + i] = 0.0;
            a.n_f[d * a.ldi + i] = 0ull;
        }
    }
    __syncthreads();
}

// Weighted average of iterations [nwarm, nitn) (RAvg, pyx:2392-2410):
// mean = sum(m/v)/sum(1/v), sdev = sum(1/v)^-1/2, chi2 = sum((m-mean)^2/v).
static __device__ __noinline__ void cta_ravg(const BatchJob &J, int nitn, int nwarm)
{
    if (threadIdx.x != 0) return;
    double sw = 0.0, swm = 0.0;
    int cnt = 0;
    for (int i = nwarm; i < nitn; i++) {
        const double m = J.out[3 * i], v = J.out[3 * i + 1];
        if (v > 0) {
            sw += 1.0 / v;
            swm += m / v;
        }
        cnt++;
    }
    const double mean = sw > 0 ? swm / sw : 0.0;
    double chi2 = 0.0;
    for (int i = nwarm; i < nitn; i++) {
        const double m = J.out[3 * i], v = J.out[3 * i + 1];
        if (v > 0) chi2 += (m - mean) * (m - mean) / v;
    }
    J.res[0] = mean;
    J.res[1] = sw > 0 ? 1.0 / sqrt(sw) : 0.0;
    J.res[2] = chi2;
    J.res[3] = (double)(cnt > 0 ? cnt - 1 : 0);
}

// The persistent kernel of one dimension bucket (every integral it takes has
// dim <= DIMB): sampling, map and evaluation in T (float; double in the
// FP64 parity configuration), S samples per thread and MINB CTAs per SM it is compiled for
// (the tile shape and occupancy the autotuner picks per bucket; one kernel
// per bucket lets the small-dimension integrals run at the occupancy their
// registers and shared memory allow).
//
// Queue mode (group <= 1): each CTA takes whole integrals from the queue.
// Group mode (group = G >= 2, cooperative launch): CTA c works on integral
// order[c / G] as rank c % G; rank 0 allocates, finalizes and adapts, all G
// ranks share the tiles (rank r takes tiles r, r + G, ...), with two group
// barriers per iteration.
template <typename T, int KIND, int DIMB, int S, int MINB>
__global__ void __launch_bounds__(NT, MINB) batch_kernel(const BatchJob *__restrict__ jobs,
                                                   const VgParams *__restrict__ params,
                                                   const int *__restrict__ order, int njobs, int nitn,
                                                   int nwarm, uint32_t itn0, unsigned int *queue,
                                                   int group, int *status)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ IterArgs sa;
    __shared__ int64_t scan[NT];
    __shared__ VgKSum red[NT / 32 + 4];   // also 6 floats per warp for float-float reductions
    __shared__ int s_q, s_flag;
    const int tid = threadIdx.x;
    const int G = group > 1 ? group : 1;
    const int rank = G > 1 ? (int)(blockIdx.x % G) : 0;
    bool first = true;
    for (;;) {
        int q;
        if (G > 1) {
            if (!first) break;
            q = (int)(blockIdx.x / G);
        } else {
            if (tid == 0) s_q = (int)atomicAdd(queue, 1u);
            __syncthreads();
            q = s_q;
            __syncthreads();
        }
        first = false;
        if (q >= njobs) break;
        const int j = order[q];
        const BatchJob &J = jobs[j];
        if (J.stamp != nullptr && tid == 0 && rank == 0) {
            J.stamp[0] = vg_globaltimer();
            J.stamp[2] = vg_smid();
        }
        {
            const int nw = (int)(sizeof(IterArgs) / 4);
            const uint32_t *src = reinterpret_cast<const uint32_t *>(&J.a);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&sa);
            for (int i = tid; i < nw; i += NT) dst[i] = src[i];
        }
        __syncthreads();
        unsigned int rounds = 0;
        bool ok = true;
        for (int it = 0; it < nitn && ok; it++) {
            if (tid == 0) sa.itn = itn0 + (uint32_t)it;
            __syncthreads();
            if (rank == 0) cta_alloc(sa, scan);
            if (G > 1 && !(ok = group_barrier(J.sync, (unsigned)G * ++rounds, sa.wait_iters))) break;
            if (sa.stats->ntiles > 0) tile_body<T, MODE_FUSED, KIND, DIMB, S>(sa, params[j], smem, rank, G, rank);
            __syncthreads();
            if (G > 1 && !(ok = group_barrier(J.sync, (unsigned)G * ++rounds, sa.wait_iters))) break;
            if (rank == 0) {
                if constexpr (sizeof(T) == 8) cta_finalize_f64(sa, G, red, &s_flag);
                else cta_finalize(sa, G, red, &s_flag);
                if (tid == 0) {
                    J.out[3 * it] = sa.stats->mean;
                    J.out[3 * it + 1] = sa.stats->var;
                    J.out[3 * it + 2] = (double)sa.stats->neval;
                }
                if (J.adapt) cta_adapt(J, sa, smem);
            }
            __syncthreads();
        }
        if (!ok) {
            if (tid == 0) atomicExch(status, VG_ERR_TIMEOUT);
            break;
        }
        if (rank == 0) cta_ravg(J, nitn, nwarm);
        __syncthreads();
        if (J.stamp != nullptr && tid == 0 && rank == 0) J.stamp[1] = vg_globaltimer();
    }
}

// Launch (queue mode, or cooperative for co-resident groups) and occupancy
// of one instantiation; the bucket files dispatch to these.
template <typename T, int KIND, int DIMB, int S, int MINB>
int launch_one(const BatchJob *jobs, const VgParams *prm, const int *order, int njobs, int nitn, int nwarm,
               uint32_t itn0, unsigned int *queue, size_t smem, int grid, int group, int *status, cudaStream_t st)
{
    auto k = batch_kernel<T, KIND, DIMB, S, MINB>;
    if (group > 1) {
        void *args[] = {(void *)&jobs, (void *)&prm, (void *)&order, (void *)&njobs, (void *)&nitn, (void *)&nwarm,
                        (void *)&itn0, (void *)&queue, (void *)&group, (void *)&status};
        VG_CUDA_CHECK(cudaLaunchCooperativeKernel((const void *)k, dim3((unsigned)grid), dim3(NT), args, smem, st));
        return VG_OK;
    }
    k<<<grid, NT, smem, st>>>(jobs, prm, order, njobs, nitn, nwarm, itn0, queue, group, status);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

// sets the kernel's shared-memory attribute (outside any stream capture)
template <typename T, int KIND, int DIMB, int S, int MINB>
int occupancy_one(size_t smem, int *per_sm)
{
    auto k = batch_kernel<T, KIND, DIMB, S, MINB>;
    VG_CUDA_CHECK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    VG_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k, NT, smem));
    return VG_OK;
}

// Tile configurations of each bucket: samples per thread and CTAs per SM.
struct BucketConfig {
    int S, minb;
};
constexpr int NCONFIG = 3;
constexpr int NBUCKET = 3;
constexpr int BUCKET_DIM[NBUCKET] = {4, 8, 16};
// FP64 parity configuration (cfg VG_BATCH_CFG_F64): Lorentzian products of
// dim <= 8 (buckets 0 and 1 share the one instantiation), 2 samples per
// thread, one CTA per SM -- the single-integral FP64 kernel's tile shape.
constexpr BucketConfig F64_CONFIG = {2, 1};
constexpr int F64_DIMB = 8;
constexpr BucketConfig BUCKET_CONFIGS[NBUCKET][NCONFIG] = {
    {{2, 4}, {4, 2}, {2, 2}},   // dim <= 4
    {{2, 2}, {4, 1}, {2, 3}},   // dim <= 8
    {{2, 1}, {1, 2}, {2, 2}},   // dim <= 16
};

// One bucket's launch and occupancy for configuration cfg (instantiated by
// the bucket's own translation unit, vg_batch_b<DIMB>.cu).
template <int KIND, int DIMB>
int bucket_launch(int cfg, const BatchJob *jobs, const VgParams *prm, const int *order, int njobs, int nitn,
                  int nwarm, uint32_t itn0, unsigned int *queue, size_t smem, int grid, int group, int *status,
                  cudaStream_t st)
{
    constexpr int b = DIMB == 4 ? 0 : (DIMB == 8 ? 1 : 2);
    constexpr BucketConfig c0 = BUCKET_CONFIGS[b][0], c1 = BUCKET_CONFIGS[b][1], c2 = BUCKET_CONFIGS[b][2];
    switch (cfg) {
    case 0:
        return launch_one<float, KIND, DIMB, c0.S, c0.minb>(jobs, prm, order, njobs, nitn, nwarm, itn0, queue, smem, grid,
                                                     group, status, st);
    case 1:
        return launch_one<float, KIND, DIMB, c1.S, c1.minb>(jobs, prm, order, njobs, nitn, nwarm, itn0, queue, smem, grid,
                                                     group, status, st);
    default:
        return launch_one<float, KIND, DIMB, c2.S, c2.minb>(jobs, prm, order, njobs, nitn, nwarm, itn0, queue, smem, grid,
                                                     group, status, st);
    }
}

template <int KIND, int DIMB>
int bucket_occupancy(int cfg, size_t smem, int *per_sm)
{
    constexpr int b = DIMB == 4 ? 0 : (DIMB == 8 ? 1 : 2);
    constexpr BucketConfig c0 = BUCKET_CONFIGS[b][0], c1 = BUCKET_CONFIGS[b][1], c2 = BUCKET_CONFIGS[b][2];
    switch (cfg) {
    case 0: return occupancy_one<float, KIND, DIMB, c0.S, c0.minb>(smem, per_sm);
    case 1: return occupancy_one<float, KIND, DIMB, c1.S, c1.minb>(smem, per_sm);
    default: return occupancy_one<float, KIND, DIMB, c2.S, c2.minb>(smem, per_sm);
    }
}

// The entry points of each bucket's translation unit.
#define VG_BATCH_BUCKET_ENTRY(DIMB)                                                                             \
    int launch_b##DIMB(int kind, int cfg, const BatchJob *jobs, const VgParams *prm, const int *order,          \
                       int njobs, int nitn, int nwarm, uint32_t itn0, unsigned int *queue, size_t smem,         \
                       int grid, int group, int *status, cudaStream_t st)                                       \
    {                                                                                                           \
        if (kind == VG_F_LATTICE)                                                                               \
            return bucket_launch<VG_F_LATTICE, DIMB>(cfg, jobs, prm, order, njobs, nitn, nwarm, itn0, queue,    \
                                                     smem, grid, group, status, st);                            \
        return bucket_launch<VG_F_LORENTZ, DIMB>(cfg, jobs, prm, order, njobs, nitn, nwarm, itn0, queue, smem,  \
                                                 grid, group, status, st);                                      \
    }                                                                                                           \
    int occupancy_b##DIMB(int kind, int cfg, size_t smem, int *per_sm)                                          \
    {                                                                                                           \
        if (kind == VG_F_LATTICE) return bucket_occupancy<VG_F_LATTICE, DIMB>(cfg, smem, per_sm);               \
        return bucket_occupancy<VG_F_LORENTZ, DIMB>(cfg, smem, per_sm);                                         \
    }

}  // namespace vgbatch
