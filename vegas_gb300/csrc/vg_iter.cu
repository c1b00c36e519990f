// vg_iter.cu -- one vegas+ iteration on the GPU.
//
// Reference: src/vegas/_vegas.pyx (vegas 6.4.1), Integrator._random_batch
// (pyx:1636-1765) and the batch loop of Integrator.__call__ (pyx:2096-2197).
//
// Layout of an iteration (all device-resident, no host round trip):
//   1. allocation (one single-pass kernel): neval_h[h] from sigf
//      (pyx:1692-1706), exclusive scan -> offsets[h], neval_hcube_range, the
//      tile schedule tile_h0[t] (first hypercube of each tile of TILE
//      samples).
//   2. a persistent tile kernel: each CTA walks tiles t = blockIdx.x,
//      += gridDim.x.  A tile is TILE consecutive samples (samples are ordered
//      by hypercube, as in the reference).  Per sample: Philox uniforms (or
//      injected ones), y = (y0 + u)/nstrat, the map y -> x, J from a grid
//      table staged in shared memory, the integrand (fused built-in or read
//      from an array), wf = wgt*f and the training histogram of
//      fdv2 = (wf*n_h)^2 in shared memory.  Then the reference's two-pass
//      per-hypercube mean/variance (with its EPSILON round-off guard) by a
//      segmented scan over the tile.  Hypercubes cut by tile boundaries
//      leave partial records (count, sum, sum of squared deviations).
//   3. finalize (one CTA): merges the partial records with Chan's parallel
//      variance formula, then sums the per-tile partials in tile order
//      (compensated FP64) into the iteration mean / var / sum_sigf.
// The tile kernel itself lives in vg_tile.cuh; its instantiations per
// integrand are spread over vg_fused_*.cu and vg_dropin.cu.
#include <math.h>
#include <string.h>

#include <mutex>

#include "vg_adapt.cuh"
#include "vg_tile.cuh"

namespace {
using namespace vg;

// ======================================================== allocation
// Block-wide exclusive prefix sum of one int64 per thread (warp shuffles,
// then a scan of the warp totals); *total = the block's sum.
template <int NTB>
__device__ __forceinline__ int64_t block_excl_scan(int64_t v, int64_t *wtot /* NTB/32 */, int64_t *total)
{
    constexpr int NW = NTB / 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) wtot[w] = x;
    __syncthreads();
    if (w == 0) {
        int64_t z = lane < NW ? wtot[lane] : 0;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, z, off);
            if (lane >= off) z += y;
        }
        if (lane < NW) wtot[lane] = z;
    }
    __syncthreads();
    *total = wtot[NW - 1];
    const int64_t r = (w > 0 ? wtot[w - 1] : 0) + x - v;
    __syncthreads();
    return r;
}

template <int NTB>
__device__ __forceinline__ int64_t block_max(int64_t v, int64_t *wtot /* NTB/32 */)
{
    constexpr int NW = NTB / 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const int64_t o = __shfl_xor_sync(0xffffffffu, v, off);
        v = o > v ? o : v;
    }
    if (lane == 0) wtot[w] = v;
    __syncthreads();
    int64_t m = wtot[0];
    for (int i = 1; i < NW; i++) m = wtot[i] > m ? wtot[i] : m;
    __syncthreads();
    return m;
}

// Allocation, pyx:1692-1706, in one pass over the hypercubes: block b
// (numbered by the order in which blocks start, so it only waits on blocks
// already running) counts neval_h for its ALLOC_NT * ALLOC_PER hypercubes,
// publishes its total, looks back over its predecessors' published totals
// for its offset (decoupled look-back: a predecessor that already knows its
// inclusive prefix ends the walk), publishes its inclusive prefix, and writes
// offsets[h] and the tile schedule.  The last block writes the iteration's
// totals and resets the pass for the next iteration.  Published words hold
// (epoch, state, value) so nothing has to be cleared between iterations;
// every wait is bounded and a timeout is reported as VG_ERR_TIMEOUT with no
// tiles scheduled.  With build_table the grid also builds the FP32 grid table.
struct AllocSync {
    unsigned int ticket, epoch, err, pad;
    unsigned long long maxacc;
};

constexpr int FLAG_AGG = 1, FLAG_INC = 2;

__device__ __forceinline__ unsigned long long flag_word(unsigned int epoch, int state, int64_t v)
{
    return ((unsigned long long)(epoch & 0x3fffffu) << 42) | ((unsigned long long)state << 40) |
           ((unsigned long long)v & ((1ull << 40) - 1));
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u64(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__global__ void __launch_bounds__(ALLOC_NT) alloc_kernel(IterArgs a, int64_t nblk, int build_table)
{
    __shared__ int64_t wtot[ALLOC_NT / 32];
    __shared__ double s_nsf;
    __shared__ int64_t s_avg, s_prefix;
    __shared__ unsigned int s_b, s_epoch;
    AllocSync *sy = reinterpret_cast<AllocSync *>(a.alloc_sync);
    unsigned long long *flags = reinterpret_cast<unsigned long long *>(a.bsum);
    const int t = threadIdx.x;
    if (t == 0) {
        s_b = atomicAdd(&sy->ticket, 1u);
        s_epoch = *(volatile unsigned int *)&sy->epoch;
        const double sum_sigf = a.stats->sum_sigf;
        s_nsf = (a.adaptive_alloc && sum_sigf > 0) ? __ddiv_rn(__dmul_rn(a.neval_frac, (double)a.neval), sum_sigf)
                                                 : 0.0;
        s_avg = (int64_t)((double)a.neval / (double)a.H);
        if (s_b == 0) a.stats->neval_sigf = s_nsf;
    }
    if (build_table)
        build_tablef(a, (int64_t)blockIdx.x * ALLOC_NT + t, (int64_t)gridDim.x * ALLOC_NT);
    __syncthreads();
    const int64_t b = (int64_t)(s_b % (unsigned int)nblk);
    const unsigned int epoch = s_epoch;
    const double nsf = s_nsf;
    const int64_t avg = s_avg;
    const int64_t mx = a.max_neval_hcube > a.min_neval_hcube ? a.max_neval_hcube : a.min_neval_hcube;
    // counts of this thread's ALLOC_PER consecutive hypercubes
    const int64_t h0 = (b * ALLOC_NT + t) * ALLOC_PER;
    int64_t loc[ALLOC_PER];
    int64_t sum = 0, m = 0;
#pragma unroll
    for (int k = 0; k < ALLOC_PER; k++) {
        const int64_t h = h0 + k;
        int64_t n = 0;
        if (h < a.H) {
            if (a.adaptive_alloc) {
                n = (int64_t)__dmul_rn(a.sigf[h], nsf) + a.min_neval_hcube;
                if (n > mx) n = mx;
            } else {
                n = avg;
            }
        }
        loc[k] = n;
        sum += n;
        m = n > m ? n : m;
    }
    if (h0 + ALLOC_PER <= a.H) {   // 16-byte aligned: h0 is a multiple of 4
        *reinterpret_cast<int4 *>(a.neval_h + h0) = make_int4((int)loc[0], (int)loc[1], (int)loc[2], (int)loc[3]);
    } else {
#pragma unroll
        for (int k = 0; k < ALLOC_PER; k++)
            if (h0 + k < a.H) a.neval_h[h0 + k] = (int32_t)loc[k];
    }
    int64_t tot;
    int64_t run = block_excl_scan<ALLOC_NT>(sum, wtot, &tot);
    const int64_t bm = block_max<ALLOC_NT>(m, wtot);
    // warp 0: publish the block total, then look back 32 predecessors at a
    // time (each lane waits for one published word; the nearest inclusive
    // prefix ends the walk)
    if (t < 32) {
        const int lane = t;
        if (lane == 0) {
            atomicMax(&sy->maxacc, (unsigned long long)bm);
            __threadfence();
            st_release_u64(&flags[b], flag_word(epoch, b == 0 ? FLAG_INC : FLAG_AGG, tot));
        }
        __syncwarp();
        int64_t prefix = 0;
        int ok = 1;
        for (int64_t hi = b - 1; hi >= 0; hi -= 32) {
            const int64_t p = hi - lane;
            int64_t v = 0;
            int inc = 1;   // before block 0: an inclusive prefix of 0
            if (p >= 0) {
                unsigned long long w = 0;
                uint32_t i = 0;
                const uint32_t budget = a.wait_iters;
                for (; i < budget; i++) {
                    w = ld_acquire_u64(&flags[p]);
                    if ((unsigned int)(w >> 42) == (epoch & 0x3fffffu) && ((w >> 40) & 3u) != 0) break;
                    if (i >= 64) __nanosleep(64);
                }
                if (i == budget) ok = 0;   // gave up: reported below, the walk goes on
                v = (int64_t)(w & ((1ull << 40) - 1));
                inc = ((w >> 40) & 3u) == (unsigned)FLAG_INC;
            }
            const unsigned int incm = __ballot_sync(0xffffffffu, inc);
            const int first = incm ? __ffs(incm) - 1 : 32;
            int64_t c = lane <= first ? v : 0;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) c += __shfl_xor_sync(0xffffffffu, c, off);
            prefix += c;
            if (incm) break;
        }
        ok = __all_sync(0xffffffffu, ok);
        if (lane == 0) {
            if (b > 0) {
                if (!ok) atomicOr(&sy->err, 1u);
                __threadfence();
                st_release_u64(&flags[b], flag_word(epoch, FLAG_INC, prefix + tot));
            }
            s_prefix = prefix;
        }
    }
    __syncthreads();
    run += s_prefix;
#pragma unroll
    for (int k = 0; k < ALLOC_PER; k++) {
        const int64_t h = h0 + k;
        if (h >= a.H) break;
        a.offsets[h] = run;
        // tiles whose first sample falls in [run, run + n)
        const int64_t n = loc[k];
        for (int64_t tt = (run + BASE_TILE - 1) / BASE_TILE; tt * BASE_TILE < run + n && tt < a.ntiles_cap; tt++)
            a.tile_h0[tt] = h;
        run += n;
    }
    if (b == nblk - 1 && t == 0) {   // every other block has published: totals, reset
        __threadfence();
        const int64_t N = s_prefix + tot;
        const int64_t mxn = (int64_t)*(volatile unsigned long long *)&sy->maxacc;
        const unsigned int err = *(volatile unsigned int *)&sy->err;
        vg_stats *st = a.stats;
        st->neval = N;
        // neval_hcube_range starts at [mnh, mnh] and every count is >= mnh
        // (pyx:1681, 1701-1704)
        st->range_lo = a.min_neval_hcube;
        st->range_hi = a.adaptive_alloc ? (mxn > a.min_neval_hcube ? mxn : a.min_neval_hcube) : a.min_neval_hcube;
        int64_t ntiles = (N + BASE_TILE - 1) / BASE_TILE;
        if (err) {
            st->status = VG_ERR_TIMEOUT;
            ntiles = 0;
        } else if (N > a.ncap || ntiles + 1 > a.ntiles_cap) {
            st->status = VG_ERR_MEMORY;
            ntiles = 0;
        } else {
            st->status = VG_OK;
            a.tile_h0[ntiles] = a.H;   // sentinel
        }
        a.offsets[a.H] = N;
        st->ntiles = ntiles;
        st->nan_seen = 0;
        *a.counter = 0ull;
        *a.fin_counter = 0u;
        sy->maxacc = 0ull;
        sy->err = 0u;
        sy->epoch = epoch + 1u;
        sy->ticket = 0u;
    }
}

// FP32 mode: the grid as an FP32 (x_node, inc) table for the tile CTAs.
__global__ void tablef_kernel(IterArgs a)
{
    build_tablef(a, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

// ========================================================== finalize
// Stage 1 (one thread per tile, FIN_TILES tiles per block): the tile's
// partial sums plus, for a tile whose last hypercube continues into later
// tiles, the Chan et al. merge of that hypercube's partial records; a
// fixed-order block reduction gives one partial per block.
// Stage 2 (one block): those partials in block order -> iteration mean, var,
// sum_sigf (compensated FP64), and the constant-integrand reset.
constexpr int FIN_TILES = 32;   // one warp per finalize block: few FP64 lanes per value

// Stage 2 body (one block): the stage-1 partials in block order -> the
// iteration's mean, var, sum_sigf and the constant-integrand reset.
__device__ __forceinline__ void finalize_totals(const IterArgs &a, int64_t nblk, VgKSum *red, int *reset)
{
    VgKSum cm = {0.0, 0.0}, cv = {0.0, 0.0}, cs = {0.0, 0.0};
    for (int64_t b = threadIdx.x; b < nblk; b += FIN_TILES) {
        const TilePart p = a.part2[b];
        cm.merge(p.mean);
        cv.merge(p.var);
        cs.merge(p.sigf);
    }
    const VgKSum M = vg_block_ksum<FIN_TILES>(cm, red);
    const VgKSum V = vg_block_ksum<FIN_TILES>(cv, red);
    const VgKSum Sg = vg_block_ksum<FIN_TILES>(cs, red);
    if (threadIdx.x == 0) {
        vg_stats *s = a.stats;
        s->mean = M.value();
        s->var = V.value();
        *reset = 0;
        s->sigf_reset = 0;
        if (a.adaptive) {
            const double ss = Sg.value();
            if (ss > 0) {
                s->sum_sigf = ss;
            } else {   // integrand looks constant: even distribution (pyx:2212-2215)
                s->sum_sigf = (double)a.H;
                s->sigf_reset = 1;
                *reset = 1;
            }
        }
    }
    __syncthreads();
    if (*reset)
        for (int64_t h = threadIdx.x; h < a.H; h += FIN_TILES) a.sigf[h] = 1.0;
}

// The iteration's results from the stats fields (mean, var, sum_sigf) and
// the constant-integrand reset (pyx:2209-2215); thread 0 has the sums.
__device__ __forceinline__ void finalize_store(const IterArgs &a, double mean, double var, double ss, int *reset)
{
    if (threadIdx.x == 0) {
        vg_stats *st = a.stats;
        st->mean = mean;
        st->var = var;
        *reset = 0;
        st->sigf_reset = 0;
        if (a.adaptive) {
            if (ss > 0) {
                st->sum_sigf = ss;
            } else {   // integrand looks constant: even distribution
                st->sum_sigf = (double)a.H;
                st->sigf_reset = 1;
                *reset = 1;
            }
        }
    }
    __syncthreads();
    if (*reset)
        for (int64_t h = threadIdx.x; h < a.H; h += blockDim.x) a.sigf[h] = 1.0;
}

// FP32 mode, stage 2: the blocks' float-float partials summed in float-float
// in block order (lane-strided, then a fixed tree), converted to FP64 once.
__device__ __forceinline__ void finalize_totals_ff(const IterArgs &a, int64_t nblk, int *reset)
{
    float r6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int64_t b = threadIdx.x; b < nblk; b += FIN_TILES) {
        const TilePart p = a.part2[b];
        float h, l;
        ff_unpack(p.mean.s, h, l);
        ff_add_pair(r6[0], r6[1], h, l);
        ff_unpack(p.var.s, h, l);
        ff_add_pair(r6[2], r6[3], h, l);
        ff_unpack(p.sigf.s, h, l);
        ff_add_pair(r6[4], r6[5], h, l);
    }
    ff_block_reduce6<FIN_TILES>(r6, nullptr);
    finalize_store(a, vg_ff_value(r6[0], r6[1]), vg_ff_value(r6[2], r6[3]), vg_ff_value(r6[4], r6[5]), reset);
}

// Stage 1, and stage 2 in the block that finishes last (a counter the
// allocation resets; the partials are read back in block order, so the
// result does not depend on which block that is).
template <int FAST>
__global__ void __launch_bounds__(FIN_TILES) finalize1_kernel(IterArgs a)
{
    __shared__ VgKSum red[1];
    __shared__ int s_last, s_reset;
    const vg_stats *st = a.stats;
    const int64_t N = st->neval;
    const int64_t ntiles = st->ntiles ? (N + a.T - 1) / a.T : 0;
    const int64_t nwork = ntiles > a.ncta ? ntiles : a.ncta;
    const int64_t nblk = (nwork + FIN_TILES - 1) / FIN_TILES;
    if (FAST && (int64_t)blockIdx.x < nblk) {
        // FP32 mode: the tile partials and the cut hypercubes' records hold
        // packed float-float values; merged and summed in float-float
        // (FP32 pipe, no FP64 instruction on the path)
        float r6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const int64_t t = (int64_t)blockIdx.x * FIN_TILES + threadIdx.x;
        if (t < a.ncta && ntiles > 0) {   // partial sums of the reduction CTA t
            const TilePart p = a.parts[t];
            ff_unpack(p.mean.s, r6[0], r6[1]);
            ff_unpack(p.var.s, r6[2], r6[3]);
            ff_unpack(p.sigf.s, r6[4], r6[5]);
        }
        if (t < ntiles) merge_cut_ff(a, t, ntiles, r6[0], r6[1], r6[2], r6[3], r6[4], r6[5]);
        ff_block_reduce6<FIN_TILES>(r6, nullptr);
        if (threadIdx.x == 0) {
            TilePart p;
            p.mean = VgKSum{ff_pack(r6[0], r6[1]), 0.0};
            p.var = VgKSum{ff_pack(r6[2], r6[3]), 0.0};
            p.sigf = VgKSum{ff_pack(r6[4], r6[5]), 0.0};
            a.part2[blockIdx.x] = p;
        }
    } else if ((int64_t)blockIdx.x < nblk) {
        const double beta_half = a.beta_half;
        VgKSum cm = {0.0, 0.0}, cv = {0.0, 0.0}, cs = {0.0, 0.0};
        const int64_t t = (int64_t)blockIdx.x * FIN_TILES + threadIdx.x;
        if (t < a.ncta && ntiles > 0) {   // partial sums of the reduction CTA t
            const TilePart p = a.parts[t];
            cm = p.mean;
            cv = p.var;
            cs = p.sigf;
        }
        if (t < ntiles) {   // a hypercube starting in tile t and cut by its end
            const TileRec r = a.recs[2 * t + 1];
            if (r.h >= 0) {
                double n = r.n, Sx = r.S, Q = r.Q, D = r.D;
                for (int64_t t2 = t + 1; t2 < ntiles; t2++) {
                    const TileRec q = a.recs[2 * t2];
                    if (q.h != r.h) break;
                    const double n2 = n + q.n;
                    // Chan et al. merge; FP32 mode: reciprocal-multiply divisions
                    const double delta = FAST ? vgadapt::div_fast(q.S, q.n) - vgadapt::div_fast(Sx, n)
                                              : q.S / q.n - Sx / n;
                    Q = Q + q.Q + delta * delta * (FAST ? vgadapt::div_fast(n * q.n, n2) : n * q.n / n2);
                    Sx += q.S;
                    D += q.D;
                    n = n2;
                    if (!q.spans) break;
                }
                const double num = __dsub_rn(__dmul_rn(n, Q), __dmul_rn(D, D));
                const double vh = FAST ? vgadapt::div_fast(num, __dsub_rn(n, 1.))
                                       : __ddiv_rn(num, __dsub_rn(n, 1.));
                if (a.train_hc) {   // adapt_to_errors: train at the hypercube's last sample
                    unsigned short b[VG_MAX_DIM];
                    last_sample_bins<double>(a, r.h, b);
                    train_hcube(a, b, fabs(vh));
                }
                cm.add(__dadd_rn(Sx, D));
                cv.add(vh);
                if (a.adaptive) {
                    const double sg = FAST ? vg_pow_fast(fabs(vh), beta_half) : pow(fabs(vh), beta_half);
                    a.sigf[r.h] = sg;
                    cs.add(sg);
                }
            }
        }
        const VgKSum M = vg_block_ksum<FIN_TILES>(cm, red);
        const VgKSum V = vg_block_ksum<FIN_TILES>(cv, red);
        const VgKSum Sg = vg_block_ksum<FIN_TILES>(cs, red);
        if (threadIdx.x == 0) {
            TilePart p;
            p.mean = M;
            p.var = V;
            p.sigf = Sg;
            a.part2[blockIdx.x] = p;
        }
    }
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = (atomicAdd(a.fin_counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    if (threadIdx.x == 0) *a.fin_counter = 0u;
    if (FAST) finalize_totals_ff(a, nblk, &s_reset);
    else finalize_totals(a, nblk, red, &s_reset);
}

// ================================================================ host
struct WorkLayout {
    size_t neval_h, offsets, bsum, tile_h0, counter, recs, parts, part2, feval, newgrid,
        newinc, tablef, total;
    int64_t nblk, ntiles_cap, ncap;
};

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

inline int64_t neval_cap(const vg_integrator *it)
{
    // sum_h min(max, int(sigf_h*nsf) + mnh) <= neval_frac*neval + H*mnh (+ rounding)
    const int64_t H = it->nhcube;
    const int64_t avg = (int64_t)((double)it->neval / (double)H);
    const int64_t mnh = it->min_neval_hcube > avg ? it->min_neval_hcube : avg;
    const double adaptive = it->neval_frac * (double)it->neval;
    return (int64_t)(adaptive * (1.0 + 1e-9)) + 64 + H * mnh;
}

WorkLayout layout(const vg_integrator *it, int64_t ncap)
{
    WorkLayout L;
    const int64_t H = it->nhcube;
    L.nblk = (H + ALLOC_NT * ALLOC_PER - 1) / (ALLOC_NT * ALLOC_PER);
    L.ntiles_cap = (ncap + BASE_TILE - 1) / BASE_TILE + 1;
    size_t o = 0;
    L.neval_h = o; o = align256(o + sizeof(int32_t) * H);
    L.offsets = o; o = align256(o + sizeof(int64_t) * (H + 1));
    L.bsum = o;    o = align256(o + sizeof(int64_t) * L.nblk);
    L.tile_h0 = o; o = align256(o + sizeof(int64_t) * (L.ntiles_cap + 1));
    L.counter = o; o = align256(o + 16 + sizeof(AllocSync));
    L.recs = o;    o = align256(o + sizeof(TileRec) * 2 * L.ntiles_cap);
    L.parts = o;   o = align256(o + sizeof(TilePart) * L.ntiles_cap);
    L.part2 = o;   o = align256(o + sizeof(TilePart) * (L.ntiles_cap / FIN_TILES + 4096 / FIN_TILES + 2));
    L.feval = o;   o = align256(o + sizeof(float) * ncap);
    L.ncap = ncap;
    L.newgrid = o; o = align256(o + sizeof(double) * it->dim * it->ldg);
    L.newinc = o;  o = align256(o + sizeof(double) * it->dim * it->ldi);
    int64_t maxK = 1;
    for (int d = 0; d < it->dim; d++) maxK = it->ninc[d] > maxK ? it->ninc[d] : maxK;
    L.tablef = o;  o = align256(o + sizeof(float2) * it->dim * (maxK + 1));
    L.total = o;
    return L;
}

int fill_args(IterArgs &a, const vg_integrator *it, uint32_t itn, const double *u)
{
    memset(&a, 0, sizeof(a));
    if (it->dim < 1 || it->dim > VG_MAX_DIM) return vg_fail(VG_ERR_UNSUPPORTED, "dim");
    if (!it->work || !it->stats) return vg_fail(VG_ERR_VALUE, "missing workspace/stats");
    a.dim = it->dim;
    int maxK = 1;
    for (int d = 0; d < it->dim; d++) {
        if (it->nstrat[d] < 1 || it->ninc[d] < 1 || it->ninc[d] > 65534)
            return vg_fail(VG_ERR_VALUE, "bad geometry (ninc must be in 1..65534)");
        a.nstrat[d] = (int)it->nstrat[d];
        a.ninc[d] = (int)it->ninc[d];
        maxK = a.ninc[d] > maxK ? a.ninc[d] : maxK;
        if (it->ninc[d] + 1 > it->ldg || it->ninc[d] > it->ldi)
            return vg_fail(VG_ERR_VALUE, "grid arrays too small");
    }
    a.maxK = maxK;
    a.grid = it->grid;
    a.inc = it->inc;
    a.ldg = it->ldg;
    a.ldi = it->ldi;
    a.H = it->nhcube;
    a.ncap = neval_cap(it);
    WorkLayout L = layout(it, a.ncap);
    if (it->work_bytes < L.total)
        return vg_fail(VG_ERR_VALUE, "workspace too small: %zu < %zu", it->work_bytes, L.total);
    char *w = (char *)it->work;
    a.sigf = it->sigf;
    a.beta = it->beta;
    // adapt_to_errors: uniform allocation, no sigf, the map trained on each
    // hypercube's variance (pyx:1659, 1675, 2187-2196, 2209)
    const int ate = it->adapt_to_errors ? 1 : 0;
    a.adaptive_alloc = (it->beta > 0 && it->nhcube > 1 && !ate) ? 1 : 0;
    a.adaptive = (a.adaptive_alloc && it->adapt) ? 1 : 0;
    a.train = (it->adapt && it->alpha > 0 && !ate) ? 1 : 0;
    a.train_hc = (ate && it->adapt) ? 1 : 0;
    a.sum_f = it->sum_f;
    a.n_f = (unsigned long long *)it->n_f;
    a.stats = it->stats;
    a.neval_h = (int32_t *)(w + L.neval_h);
    a.offsets = (int64_t *)(w + L.offsets);
    a.bsum = (int64_t *)(w + L.bsum);
    a.tile_h0 = (int64_t *)(w + L.tile_h0);
    a.counter = (unsigned long long *)(w + L.counter);
    a.fin_counter = (unsigned int *)(w + L.counter + sizeof(unsigned long long));
    a.alloc_sync = (unsigned int *)(w + L.counter + 16);
    a.recs = (TileRec *)(w + L.recs);
    a.parts = (TilePart *)(w + L.parts);
    a.part2 = (TilePart *)(w + L.part2);
    a.f_eval = (float *)(w + L.feval);
    a.tablef = (float2 *)(w + L.tablef);
    a.ntiles_cap = L.ntiles_cap;
    a.neval = it->neval;
    a.neval_frac = it->neval_frac;
    a.min_neval_hcube = it->min_neval_hcube;
    a.max_neval_hcube = it->max_neval_hcube;
    a.seed = it->seed;
    a.stream = it->stream_id;
    a.itn = itn;
    a.u = u;
    a.dv_y = 1.0 / (double)it->nhcube;
    a.beta_half = it->beta / 2.0;
    a.wait_iters = g_wait_iters;
    return VG_OK;
}

}  // namespace

namespace vg {
int finalize_launch(IterArgs &a, cudaStream_t st, int fast)
{
    // tiles of the launched kernel, bounded by the capacity
    const int64_t tcap = (a.ntiles_cap * BASE_TILE + a.T - 1) / a.T;
    const int64_t nwork = tcap > a.ncta ? tcap : a.ncta;
    const int64_t nblk = (nwork + FIN_TILES - 1) / FIN_TILES;
    if (fast) finalize1_kernel<1><<<(unsigned)nblk, FIN_TILES, 0, st>>>(a);
    else finalize1_kernel<0><<<(unsigned)nblk, FIN_TILES, 0, st>>>(a);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

int launch_points(IterArgs &a, int f64, cudaStream_t st);
int launch_reduce(IterArgs &a, int f64, cudaStream_t st);
int launch_fused(IterArgs &a, int kind, const VgParams &P, int tab_len, int f64, cudaStream_t st);

int fill_iter_args(IterArgs &a, const vg_integrator *it, uint32_t itn, const double *u)
{
    return fill_args(a, it, itn, u);
}

void scratch_grid(const vg_integrator *it, double **new_grid, double **new_inc)
{
    WorkLayout L = layout(it, neval_cap(it));
    char *w = (char *)it->work;
    *new_grid = (double *)(w + L.newgrid);
    *new_inc = (double *)(w + L.newinc);
}
}  // namespace vg

// ====================================================================== ABI
extern "C" int64_t vg_neval_cap(const vg_integrator *it) { return neval_cap(it); }

extern "C" size_t vg_workspace_bytes(const vg_integrator *it, int64_t ncap)
{
    if (it == nullptr || it->dim < 1 || it->dim > VG_MAX_DIM) {   // layout() reads ninc[0 .. dim)
        vg_fail(VG_ERR_VALUE, "vg_workspace_bytes: dim outside 1..%d", VG_MAX_DIM);
        return 0;
    }
    if (ncap <= 0) ncap = neval_cap(it);
    return layout(it, ncap).total;
}

extern "C" int vg_allocate(const vg_integrator *it, void *stream)
{
    VG_RANGE("vg_allocate");
    vg_clear_error();
    IterArgs a;
    int rc = fill_args(a, it, 0, nullptr);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    WorkLayout L = layout(it, a.ncap);
    // the FP32 grid table is built by the counting grid, or alone when that
    // grid has too few threads for it
    const int64_t ntab = (int64_t)a.dim * (a.maxK + 1);
    const int table_in_count = (it->precision == VG_F32) && ntab <= L.nblk * ALLOC_NT;
    alloc_kernel<<<(unsigned)L.nblk, ALLOC_NT, 0, st>>>(a, L.nblk, table_in_count);
    VG_LAUNCH_CHECK();
    if (it->precision == VG_F32 && !table_in_count) {
        tablef_kernel<<<(unsigned)((ntab + 255) / 256), 256, 0, st>>>(a);
        VG_LAUNCH_CHECK();
    }
    return VG_OK;
}

// Clears the single-pass allocation's published block words and its
// ticket / epoch for a workspace that other geometries have used (the
// static scratch of vg_iteration_noalloc).
int vg_alloc_sync_reset(const vg_integrator *it, void *stream)
{
    WorkLayout L = layout(it, neval_cap(it));
    char *w = (char *)it->work;
    cudaStream_t st = (cudaStream_t)stream;
    VG_CUDA_CHECK(cudaMemsetAsync(w + L.bsum, 0, sizeof(int64_t) * (size_t)L.nblk, st));
    VG_CUDA_CHECK(cudaMemsetAsync(w + L.counter, 0, 16 + sizeof(AllocSync), st));
    return VG_OK;
}

static int reset_counter(IterArgs &a, cudaStream_t st)
{
    VG_CUDA_CHECK(cudaMemsetAsync(a.counter, 0, sizeof(unsigned long long), st));
    return VG_OK;
}

extern "C" int vg_sample(const vg_integrator *it, uint32_t itn, const double *u, void *x, void *y,
                         double *wgt, int64_t *hcube, int64_t n_cap, void *stream)
{
    VG_RANGE("vg_sample");
    vg_clear_error();
    IterArgs a;
    int rc = fill_args(a, it, itn, u);
    if (rc) return rc;
    if (n_cap < a.ncap) return vg_fail(VG_ERR_VALUE, "output capacity %lld < %lld",
                                       (long long)n_cap, (long long)a.ncap);
    a.x_out = x;
    a.y_out = y;
    a.wgt_out = wgt;
    a.hc_out = hcube;
    a.train = 0;
    a.train_hc = 0;
    a.adaptive = 0;
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = reset_counter(a, st))) return rc;
    return vg::launch_points(a, it->precision == VG_F64, st);
}

extern "C" int vg_reduce(const vg_integrator *it, uint32_t itn, const double *u, const void *f,
                         int f_dtype, void *stream)
{
    VG_RANGE("vg_reduce");
    vg_clear_error();
    IterArgs a;
    int rc = fill_args(a, it, itn, u);
    if (rc) return rc;
    a.f_in = f;
    a.f_f64 = (f_dtype == VG_F64);
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = vg::launch_reduce(a, it->precision == VG_F64, st))) return rc;   // static tiles
    return vg::finalize_launch(a, st, it->precision == VG_F32);
}

// An iteration record set to zero but for the carried sum_sigf.
__global__ void stats_reset_kernel(vg_stats *st, double sum_sigf)
{
    if (threadIdx.x == 0) {
        vg_stats z;
        memset(&z, 0, sizeof(z));
        z.sum_sigf = sum_sigf;
        *st = z;
    }
}

extern "C" int vg_stats_reset(vg_stats *stats, double sum_sigf, void *stream)
{
    vg_clear_error();
    if (stats == nullptr) return vg_fail(VG_ERR_VALUE, "vg_stats_reset: no record");
    stats_reset_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(stats, sum_sigf);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

// The kept-sample buffer of vg_sample_keep / vg_reduce_kept: per sample its
// Jacobian (the precision's float type), then its training bins (16-bit per
// axis, rows padded to a multiple of 4 axes so that each 4 bins move as one
// 8-byte word).
static int keep_bstride(const vg_integrator *it) { return (it->dim + 3) & ~3; }

static size_t keep_jac_bytes(const vg_integrator *it, int64_t ncap)
{
    const size_t t = it->precision == VG_F64 ? sizeof(double) : sizeof(float);
    return (t * (size_t)ncap + 255) & ~(size_t)255;
}

extern "C" size_t vg_keep_bytes(const vg_integrator *it, int64_t n_cap)
{
    if (it == nullptr || it->dim < 1 || it->dim > VG_MAX_DIM) {
        vg_fail(VG_ERR_VALUE, "vg_keep_bytes: dim outside 1..%d", VG_MAX_DIM);
        return 0;
    }
    if (n_cap <= 0) n_cap = neval_cap(it);
    return keep_jac_bytes(it, n_cap) + sizeof(unsigned short) * (size_t)keep_bstride(it) * (size_t)n_cap;
}

static int keep_args(IterArgs &a, const vg_integrator *it, void *keep, size_t keep_bytes)
{
    if (keep == nullptr) return vg_fail(VG_ERR_VALUE, "kept-sample buffer missing");
    if (keep_bytes < vg_keep_bytes(it, a.ncap))
        return vg_fail(VG_ERR_VALUE, "kept-sample buffer too small: %zu < %zu", keep_bytes,
                       vg_keep_bytes(it, a.ncap));
    a.keep_jac = keep;
    a.keep_bins = (unsigned short *)((char *)keep + keep_jac_bytes(it, a.ncap));
    a.keep_bstride = keep_bstride(it);
    return VG_OK;
}

extern "C" int vg_sample_keep(const vg_integrator *it, uint32_t itn, const double *u, void *x, void *y,
                              double *wgt, int64_t *hcube, int64_t n_cap, void *keep, size_t keep_bytes,
                              void *stream)
{
    VG_RANGE("vg_sample_keep");
    vg_clear_error();
    IterArgs a;
    int rc = fill_args(a, it, itn, u);
    if (rc) return rc;
    if (n_cap < a.ncap) return vg_fail(VG_ERR_VALUE, "output capacity %lld < %lld",
                                       (long long)n_cap, (long long)a.ncap);
    if ((rc = keep_args(a, it, keep, keep_bytes))) return rc;
    a.x_out = x;
    a.y_out = y;
    a.wgt_out = wgt;
    a.hc_out = hcube;
    a.train = 0;
    a.train_hc = 0;
    a.adaptive = 0;
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = reset_counter(a, st))) return rc;
    return vg::launch_points(a, it->precision == VG_F64, st);
}

extern "C" int vg_reduce_kept(const vg_integrator *it, uint32_t itn, const double *u, const void *f, int f_dtype,
                              const void *keep, size_t keep_bytes, void *stream)
{
    VG_RANGE("vg_reduce_kept");
    vg_clear_error();
    IterArgs a;
    int rc = fill_args(a, it, itn, u);   // itn, u: the finalize regenerates a cut hypercube's last sample
                                         // under adapt_to_errors
    if (rc) return rc;
    if ((rc = keep_args(a, it, const_cast<void *>(keep), keep_bytes))) return rc;
    a.f_in = f;
    a.f_f64 = (f_dtype == VG_F64);
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = vg::launch_reduce_kept(a, it->precision == VG_F64, st))) return rc;   // static tiles
    return vg::finalize_launch(a, st, it->precision == VG_F32);
}

static unsigned long long *g_term_count = nullptr;
namespace vg {
uint32_t g_wait_iters = VG_WAIT_ITERS_DEFAULT;
int g_eval_split = 0;
int g_tile_s4 = 0, g_tile_table = -1, g_tile_hist = -1;
}

// Tuning of the tile kernels: samples per thread of the fused FP32 ridge for
// dim <= 4 (0 automatic = 2, with 4 CTAs per SM; or 4), grid table and
// training histogram in shared memory (-1 automatic, 0 off, 1 on where it
// fits).
extern "C" int vg_set_tile_tuning(int s_dim4, int table_smem, int hist_smem)
{
    if (s_dim4 != 0 && s_dim4 != 2 && s_dim4 != 4) return vg_fail(VG_ERR_VALUE, "s_dim4 %d", s_dim4);
    if (table_smem < -1 || table_smem > 1 || hist_smem < -1 || hist_smem > 1)
        return vg_fail(VG_ERR_VALUE, "shared-memory policy");
    vg::g_tile_s4 = s_dim4;
    vg::g_tile_table = table_smem;
    vg::g_tile_hist = hist_smem;
    return VG_OK;
}

// Polls of the bounded device-side waits (allocation look-back; four times
// as many for the batched launch's group barriers) before they give up and
// report VG_ERR_TIMEOUT; a negative value restores the default.  Read when
// an iteration's arguments are filled (vg_allocate, vg_iterate, ...,
// vg_batch_prepare).
extern "C" int vg_set_wait_budget(int64_t iters)
{
    vg::g_wait_iters = iters < 0 ? VG_WAIT_ITERS_DEFAULT
                                 : (iters > 0xffffffffll ? 0xffffffffu : (uint32_t)iters);
    return VG_OK;
}

// Tuning: how FP32 iterations of the ridge run -- 0 automatic, 1 the single
// fused kernel, 2 split into EVAL (writes f) + REDUCE.
extern "C" int vg_set_eval_split(int policy)
{
    if (policy < 0 || policy > 2) return vg_fail(VG_ERR_VALUE, "split policy %d", policy);
    vg::g_eval_split = policy;
    return VG_OK;
}

// Instrumentation: while set, the FP32 ridge adds the number of Gaussian
// terms it evaluates to *count (device); NULL turns it off.
extern "C" int vg_set_term_counter(unsigned long long *count)
{
    g_term_count = count;
    return VG_OK;
}

// Validate the parameters of a built-in integrand and fill P (including its
// host-precomputed FP32 constants); tab_len = length of its per-CTA table.
int vg_build_params(int kind, int dim, const double *params, int nparams, VgParams *Pp, int *tab_len_out)
{
    if (nparams < 0 || nparams > VG_MAX_PARAMS) return vg_fail(VG_ERR_VALUE, "too many params");
    VgParams &P = *Pp;
    memset(&P, 0, sizeof(P));
    P.n = nparams;
    for (int i = 0; i < nparams; i++) P.p[i] = params[i];
    int need = 0, tab_len = 0;
    switch (kind) {
    case VG_F_GAUSS: need = 3; break;
    case VG_F_RIDGE:
        need = 2;
        if (nparams >= 2 && (params[0] < 1 || params[0] > 16384))
            return vg_fail(VG_ERR_VALUE, "ridge M out of range 1..16384");
        tab_len = nparams >= 1 ? (int)params[0] : 0;
        break;
    case VG_F_LORENTZ: need = 2 * dim; tab_len = 4 * dim; break;
    case VG_F_MIXTURE:
        need = nparams >= 1 ? 2 + (int)params[0] * dim : 1;
        if (nparams >= 1 && (params[0] < 1 || params[0] * dim > VG_MAX_PARAMS - 2))
            return vg_fail(VG_ERR_VALUE, "mixture size out of range");
        tab_len = nparams >= 1 ? (int)params[0] * dim : 0;
        break;
    case VG_F_LATTICE: need = 2; break;
    case VG_F_CONST: need = 1; break;
    default: return vg_fail(VG_ERR_VALUE, "unknown integrand kind %d", kind);
    }
    if (nparams < need) return vg_fail(VG_ERR_VALUE, "integrand needs %d parameters", need);
    vg_prepare_f32_host(P, kind, dim);
    P.term_count = (kind == VG_F_RIDGE) ? g_term_count : nullptr;
    *tab_len_out = tab_len;
    return VG_OK;
}

extern "C" int vg_fused_iteration(const vg_integrator *it, uint32_t itn, const double *u, int kind,
                                  const double *params, int nparams, void *stream)
{
    VG_RANGE("vg_fused_iteration");
    vg_clear_error();
    IterArgs a;
    int rc = fill_args(a, it, itn, u);
    if (rc) return rc;
    VgParams P;   // copied into the kernel arguments at launch
    int tab_len = 0;
    if ((rc = vg_build_params(kind, it->dim, params, nparams, &P, &tab_len))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = vg::launch_fused(a, kind, P, tab_len, it->precision == VG_F64, st))) return rc;
    return vg::finalize_launch(a, st, it->precision == VG_F32);
}

// forward declaration: one full iteration (below)
extern "C" int vg_end_iteration(const vg_integrator *it, void *stream);

int vg_adapt_launch(int dim, const int64_t *old_ninc, const int64_t *new_ninc, const double *grid,
                    const double *inc, int64_t ldg, int64_t ldi, const double *sum_f,
                    const uint64_t *n_f, double alpha, double *new_grid, double *new_inc,
                    int64_t ldg_new, int64_t ldi_new, cudaStream_t st, int fast, int zero_hist);
int vg_adapt_in_place_ok(int max_old);

extern "C" int vg_end_iteration(const vg_integrator *it, void *stream)
{
    VG_RANGE("vg_end_iteration");
    vg_clear_error();
    cudaStream_t st = (cudaStream_t)stream;
    if (!(it->adapt && it->alpha > 0)) return VG_OK;
    int64_t kmin = it->ninc[0], kmax = it->ninc[0];
    for (int d = 1; d < it->dim; d++) {
        kmin = it->ninc[d] < kmin ? it->ninc[d] : kmin;
        kmax = it->ninc[d] > kmax ? it->ninc[d] : kmax;
    }
    if (kmin > 1 && vg_adapt_in_place_ok((int)kmax))   // one kernel: adapt in place, clear the histogram
        return vg_adapt_launch(it->dim, it->ninc, it->ninc, it->grid, it->inc, it->ldg, it->ldi, it->sum_f,
                               it->n_f, it->alpha, it->grid, it->inc, it->ldg, it->ldi, st,
                               it->precision == VG_F32, 1);
    WorkLayout L = layout(it, neval_cap(it));
    if (it->work_bytes < L.total) return vg_fail(VG_ERR_VALUE, "workspace too small");
    char *w = (char *)it->work;
    double *ng = (double *)(w + L.newgrid);
    double *ni = (double *)(w + L.newinc);
    int rc = vg_adapt_launch(it->dim, it->ninc, it->ninc, it->grid, it->inc, it->ldg, it->ldi,
                             it->sum_f, it->n_f, it->alpha, ng, ni, it->ldg, it->ldi, st,
                             it->precision == VG_F32, 0);
    if (rc) return rc;
    VG_CUDA_CHECK(cudaMemcpyAsync(it->grid, ng, sizeof(double) * it->dim * it->ldg,
                                  cudaMemcpyDeviceToDevice, st));
    VG_CUDA_CHECK(cudaMemcpyAsync(it->inc, ni, sizeof(double) * it->dim * it->ldi,
                                  cudaMemcpyDeviceToDevice, st));
    VG_CUDA_CHECK(cudaMemsetAsync(it->sum_f, 0, sizeof(double) * it->dim * it->ldi, st));
    VG_CUDA_CHECK(cudaMemsetAsync(it->n_f, 0, sizeof(uint64_t) * it->dim * it->ldi, st));
    return VG_OK;
}

// One full vegas+ iteration = vg_allocate + vg_fused_iteration +
// vg_end_iteration, enqueued by one call.  The map adapt needs only the
// training histogram the tile kernel completed, so (unless adapt_to_errors,
// whose finalize adds to that histogram) it runs on a forked stream while the
// finalize merges the hypercubes cut by tile boundaries; both join back into
// `stream` before the call returns.  The forked stream and events are created
// on the first call on a device (outside any stream capture).
namespace {
struct IterAux {
    cudaStream_t s;
    cudaEvent_t fork, join;
};
std::mutex g_iter_aux_mutex;
IterAux *g_iter_aux[VG_MAX_DEVICES];   // per device ordinal; created once, never replaced

// The forked stream and events of the current device, created on the first
// call on that device.
int iter_aux(IterAux **out)
{
    int dev = 0;
    VG_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= VG_MAX_DEVICES) return vg_fail(VG_ERR_UNSUPPORTED, "device ordinal %d", dev);
    std::lock_guard<std::mutex> lock(g_iter_aux_mutex);
    if (g_iter_aux[dev] == nullptr) {
        IterAux a;
        VG_CUDA_CHECK(cudaStreamCreateWithFlags(&a.s, cudaStreamNonBlocking));
        VG_CUDA_CHECK(cudaEventCreateWithFlags(&a.fork, cudaEventDisableTiming));
        VG_CUDA_CHECK(cudaEventCreateWithFlags(&a.join, cudaEventDisableTiming));
        g_iter_aux[dev] = new IterAux(a);
    }
    *out = g_iter_aux[dev];
    return VG_OK;
}
}  // namespace

extern "C" int vg_iterate(const vg_integrator *it, uint32_t itn, int kind, const double *params, int nparams,
                          void *stream)
{
    VG_RANGE("vg_iterate");
    int rc = vg_allocate(it, stream);
    if (rc) return rc;
    vg_clear_error();
    IterArgs a;
    if ((rc = fill_args(a, it, itn, nullptr))) return rc;
    VgParams P;   // copied into the kernel arguments at launch
    int tab_len = 0;
    if ((rc = vg_build_params(kind, it->dim, params, nparams, &P, &tab_len))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = vg::launch_fused(a, kind, P, tab_len, it->precision == VG_F64, st))) return rc;
    int64_t kmax = 0;
    for (int d = 0; d < it->dim; d++) kmax = it->ninc[d] > kmax ? it->ninc[d] : kmax;
    const int overlap = it->adapt && it->alpha > 0 && !it->adapt_to_errors && vg_adapt_in_place_ok((int)kmax);
    if (!overlap) {
        if ((rc = vg::finalize_launch(a, st, it->precision == VG_F32))) return rc;
        return vg_end_iteration(it, stream);
    }
    IterAux *aux = nullptr;
    if ((rc = iter_aux(&aux))) return rc;
    VG_CUDA_CHECK(cudaEventRecord(aux->fork, st));
    VG_CUDA_CHECK(cudaStreamWaitEvent(aux->s, aux->fork, 0));
    rc = vg_end_iteration(it, aux->s);
    VG_CUDA_CHECK(cudaEventRecord(aux->join, aux->s));
    if (rc == VG_OK) rc = vg::finalize_launch(a, st, it->precision == VG_F32);
    VG_CUDA_CHECK(cudaStreamWaitEvent(st, aux->join, 0));
    return rc;
}
