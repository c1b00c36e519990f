// vg_iter.cu -- one vegas+ iteration on the GPU.
//
// Reference: src/vegas/_vegas.pyx (vegas 6.4.1), Integrator._random_batch
// (pyx:1636-1765) and the batch loop of Integrator.__call__ (pyx:2096-2197).
//
// Layout of an iteration (all device-resident, no host round trip):
//   1. allocation (3 small kernels): neval_h[h] from sigf (pyx:1692-1706),
//      exclusive scan -> offsets[h], neval_hcube_range, the tile schedule
//      tile_h0[t] (first hypercube of each tile of TILE samples).
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
//      variance formula, then sums the per-CTA partials in a fixed order
//      (compensated FP64) into the iteration mean / var / sum_sigf.
#include <math.h>
#include <string.h>

#include "vg_common.cuh"
#include "vg_integrands.cuh"

namespace {

constexpr int NT = 256;          // threads per tile CTA
constexpr int ALLOC_NT = 1024;   // allocation kernels
constexpr int ALLOC_PER = 4;     // hypercubes per thread in the allocation
constexpr int FIN_NT = 1024;     // finalize CTA

enum { MODE_POINTS = 0, MODE_REDUCE = 1, MODE_FUSED = 2 };

// Partial statistics of a hypercube cut by a tile boundary.
struct TileRec {
    int64_t h;       // hypercube, -1 if the slot is empty
    double n;        // samples of h inside the tile
    double S;        // sum of wf
    double Q;        // sum of squared deviations about S/n (EPSILON-guarded)
    double D;        // sum of deviations (round-off residue, Neely correction)
    int32_t spans;   // head slot only: h also continues past the tile
    int32_t pad;
};

struct ChainRes {
    double mean, var, sigf;
};

struct CtaPart {
    VgKSum mean, var, sigf;
};

// Workspace carve-up (bytes, 256-aligned sections).
struct WorkLayout {
    size_t neval_h, offsets, bsum, bmax, tile_h0, recs, chain, parts, newgrid, newinc, total;
    int64_t nblk, ntiles_cap, nparts;
};

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

inline int tile_size(const vg_integrator *it)
{
    if (it->tile > 0) return it->tile;
    return it->precision == VG_F64 ? NT * 2 : NT * 4;
}

inline int samples_per_thread(const vg_integrator *it) { return tile_size(it) / NT; }

inline int64_t neval_cap(const vg_integrator *it)
{
    // sum_h min(max, int(sigf_h*nsf) + mnh) <= neval_frac*neval + H*mnh (+ rounding)
    int64_t H = it->nhcube;
    int64_t avg = (int64_t)((double)it->neval / (double)H);
    int64_t mnh = it->min_neval_hcube > avg ? it->min_neval_hcube : avg;
    double adaptive = it->neval_frac * (double)it->neval;
    return (int64_t)(adaptive * (1.0 + 1e-9)) + 64 + H * mnh;
}

WorkLayout layout(const vg_integrator *it, int64_t ncap)
{
    WorkLayout L;
    int64_t H = it->nhcube;
    int T = tile_size(it);
    L.nblk = (H + ALLOC_NT * ALLOC_PER - 1) / (ALLOC_NT * ALLOC_PER);
    L.ntiles_cap = (ncap + T - 1) / T + 1;
    L.nparts = 4096;
    size_t o = 0;
    L.neval_h = o; o = align256(o + sizeof(int32_t) * H);
    L.offsets = o; o = align256(o + sizeof(int64_t) * (H + 1));
    L.bsum = o;    o = align256(o + sizeof(int64_t) * L.nblk);
    L.bmax = o;    o = align256(o + sizeof(int64_t) * L.nblk);
    L.tile_h0 = o; o = align256(o + sizeof(int64_t) * (L.ntiles_cap + 1));
    L.recs = o;    o = align256(o + sizeof(TileRec) * 2 * L.ntiles_cap);
    L.chain = o;   o = align256(o + sizeof(ChainRes) * L.ntiles_cap);
    L.parts = o;   o = align256(o + sizeof(CtaPart) * L.nparts);
    int64_t maxK = 1;
    for (int d = 0; d < it->dim; d++) maxK = it->ninc[d] > maxK ? it->ninc[d] : maxK;
    L.newgrid = o; o = align256(o + sizeof(double) * it->dim * it->ldg);
    L.newinc = o;  o = align256(o + sizeof(double) * it->dim * it->ldi);
    (void)maxK;
    L.total = o;
    return L;
}

// ------------------------------------------------------------ arguments
struct IterArgs {
    int dim;
    int S;                    // samples per thread
    int T;                    // tile size
    int nstrat[VG_MAX_DIM];
    int ninc[VG_MAX_DIM];
    const double *grid, *inc;
    int64_t ldg, ldi;
    int64_t H;
    int64_t ncap;
    double *sigf;
    double beta;
    int adaptive;             // update sigf (pyx:2083, 2183-2186)
    int adaptive_alloc;       // allocate from sigf (pyx:1668)
    int train;                // accumulate training histogram (pyx:2196)
    double *sum_f;
    unsigned long long *n_f;
    vg_stats *stats;
    int32_t *neval_h;
    int64_t *offsets;
    int64_t *bsum, *bmax;
    int64_t *tile_h0;
    TileRec *recs;
    ChainRes *chain;
    CtaPart *parts;
    int nparts;
    int64_t ntiles_cap;
    int64_t neval;
    double neval_frac;
    int64_t min_neval_hcube, max_neval_hcube;
    uint64_t seed;
    uint32_t stream;
    uint32_t itn;
    const double *u;          // injected uniforms [n, dim] or nullptr
    // MODE_REDUCE
    const void *f_in;
    int f_f64;
    // MODE_POINTS
    void *x_out, *y_out;
    double *wgt_out;
    int64_t *hc_out;
    // shared-memory plan
    int table_smem;           // grid table staged in shared memory
    int hist_smem;            // training histogram in shared memory
    int maxK;
    int tab_len;              // integrand table length (floats)
};

// ======================================================== allocation
// pyx:1692-1706 for hypercubes of this thread; block totals for the scan.
__global__ void __launch_bounds__(ALLOC_NT) alloc_count_kernel(IterArgs a)
{
    __shared__ int64_t ssum[ALLOC_NT / 32], smax[ALLOC_NT / 32];
    const vg_stats *st = a.stats;
    double sum_sigf = st->sum_sigf;
    double nsf = (a.beta > 0 && sum_sigf > 0)
                     ? __ddiv_rn(__dmul_rn(a.neval_frac, (double)a.neval), sum_sigf)
                     : 0.0;
    int64_t mx = a.max_neval_hcube > a.min_neval_hcube ? a.max_neval_hcube : a.min_neval_hcube;
    int64_t avg = (int64_t)((double)a.neval / (double)a.H);
    int64_t h0 = ((int64_t)blockIdx.x * ALLOC_NT + threadIdx.x) * ALLOC_PER;
    int64_t s = 0, m = 0;
    for (int k = 0; k < ALLOC_PER; k++) {
        int64_t h = h0 + k;
        if (h >= a.H) break;
        int64_t n;
        if (a.adaptive_alloc) {
            n = (int64_t)__dmul_rn(a.sigf[h], nsf) + a.min_neval_hcube;
            if (n > mx) n = mx;
        } else {
            n = avg;
        }
        a.neval_h[h] = (int32_t)n;
        s += n;
        m = n > m ? n : m;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, off);
        int64_t o = __shfl_down_sync(0xffffffffu, m, off);
        m = o > m ? o : m;
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { ssum[w] = s; smax[w] = m; }
    __syncthreads();
    if (w == 0) {
        s = ssum[lane];
        m = smax[lane];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            s += __shfl_down_sync(0xffffffffu, s, off);
            int64_t o = __shfl_down_sync(0xffffffffu, m, off);
            m = o > m ? o : m;
        }
        if (lane == 0) {
            a.bsum[blockIdx.x] = s;
            a.bmax[blockIdx.x] = m;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) a.stats->neval_sigf = nsf;
}

// Exclusive scan of block totals (one CTA), totals, range, tile count.
__global__ void __launch_bounds__(ALLOC_NT) alloc_scan_kernel(IterArgs a, int64_t nblk)
{
    __shared__ int64_t part[ALLOC_NT];
    __shared__ int64_t pmax[ALLOC_NT];
    int t = threadIdx.x;
    int64_t per = (nblk + ALLOC_NT - 1) / ALLOC_NT;
    int64_t b = t * per, e = b + per < nblk ? b + per : nblk;
    int64_t s = 0, m = 0;
    for (int64_t i = b; i < e; i++) {
        s += a.bsum[i];
        m = a.bmax[i] > m ? a.bmax[i] : m;
    }
    part[t] = s;
    pmax[t] = m;
    __syncthreads();
    for (int off = 1; off < ALLOC_NT; off <<= 1) {
        int64_t add = t >= off ? part[t - off] : 0;
        int64_t mm = t >= off ? pmax[t - off] : 0;
        __syncthreads();
        part[t] += add;
        pmax[t] = mm > pmax[t] ? mm : pmax[t];
        __syncthreads();
    }
    int64_t run = t > 0 ? part[t - 1] : 0;
    for (int64_t i = b; i < e; i++) {
        int64_t v = a.bsum[i];
        a.bsum[i] = run;   // becomes the block offset
        run += v;
    }
    if (t == ALLOC_NT - 1) {
        int64_t N = part[ALLOC_NT - 1];
        int64_t mx = pmax[ALLOC_NT - 1];
        vg_stats *st = a.stats;
        st->neval = N;
        // neval_hcube_range starts at [mnh, mnh] and every count is >= mnh
        // (pyx:1681, 1701-1704)
        st->range_lo = a.min_neval_hcube;
        st->range_hi = a.adaptive_alloc ? (mx > a.min_neval_hcube ? mx : a.min_neval_hcube)
                                        : a.min_neval_hcube;
        int64_t ntiles = (N + a.T - 1) / a.T;
        if (N > a.ncap || ntiles + 1 > a.ntiles_cap) {
            st->status = VG_ERR_MEMORY;
            ntiles = 0;
        } else {
            st->status = VG_OK;
        }
        st->ntiles = ntiles;
        st->nan_seen = 0;
    }
}

// Offsets (exclusive scan within the block + block offset) and tile heads.
__global__ void __launch_bounds__(ALLOC_NT) alloc_offsets_kernel(IterArgs a)
{
    __shared__ int64_t part[ALLOC_NT];
    int t = threadIdx.x;
    int64_t h0 = ((int64_t)blockIdx.x * ALLOC_NT + t) * ALLOC_PER;
    int64_t loc[ALLOC_PER];
    int64_t s = 0;
    for (int k = 0; k < ALLOC_PER; k++) {
        int64_t h = h0 + k;
        loc[k] = (h < a.H) ? (int64_t)a.neval_h[h] : 0;
        s += loc[k];
    }
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < ALLOC_NT; off <<= 1) {
        int64_t add = t >= off ? part[t - off] : 0;
        __syncthreads();
        part[t] += add;
        __syncthreads();
    }
    int64_t run = a.bsum[blockIdx.x] + (t > 0 ? part[t - 1] : 0);
    const vg_stats *st = a.stats;
    int64_t N = st->neval;
    int64_t ntiles = st->ntiles;
    for (int k = 0; k < ALLOC_PER; k++) {
        int64_t h = h0 + k;
        if (h >= a.H) break;
        a.offsets[h] = run;
        // tiles whose first sample falls in [run, run + n)
        int64_t n = loc[k];
        int64_t tfirst = (run + a.T - 1) / a.T;
        for (int64_t tt = tfirst; tt * a.T < run + n && tt < ntiles; tt++) a.tile_h0[tt] = h;
        run += n;
        if (h == a.H - 1) {
            a.offsets[a.H] = N;
            a.tile_h0[ntiles] = a.H;   // sentinel
        }
    }
}

// ==================================================== tile kernel
template <typename T>
struct GridEntry;
template <>
struct GridEntry<float> {
    typedef float2 type;
};
template <>
struct GridEntry<double> {
    typedef double2 type;
};

// Shared-memory plan of the tile kernel (offsets in bytes).
struct SmemPlan {
    size_t table, hsum, hcnt, win_off, win_n, seg_S, keyF, keyL, P, red, itab, total;
};

template <typename T>
__host__ __device__ inline SmemPlan smem_plan(int dim, int maxK, int Ttile, int table_smem,
                                              int hist_smem, int tab_len)
{
    SmemPlan p;
    size_t o = 0;
    auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
    p.table = o;
    if (table_smem) o = al(o + sizeof(typename GridEntry<T>::type) * (size_t)dim * (maxK + 1));
    p.hsum = o;
    if (hist_smem) o = al(o + sizeof(T) * (size_t)dim * maxK);
    p.hcnt = o;
    if (hist_smem) o = al(o + sizeof(unsigned int) * (size_t)dim * maxK);
    p.win_off = o; o = al(o + sizeof(int) * (Ttile + 2));
    p.win_n = o;   o = al(o + sizeof(int) * (Ttile + 2));
    p.seg_S = o;   o = al(o + sizeof(double) * (Ttile + 2));
    p.keyF = o;    o = al(o + sizeof(int) * NT);
    p.keyL = o;    o = al(o + sizeof(int) * NT);
    p.P = o;       o = al(o + sizeof(double2) * NT);
    p.red = o;     o = al(o + sizeof(VgKSum) * (NT / 32) * 3 + 64);
    p.itab = o;    o = al(o + sizeof(float) * (tab_len + 4));
    p.total = o;
    return p;
}

// Inclusive segmented scan over the NT threads of (flag, value2).
// Returns the inclusive value for this thread; writes it to P[t].
__device__ __forceinline__ double2 seg_scan(int flag, double2 v, double2 *P, double2 *wsum,
                                            int *wflag)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int f = flag;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        double ux = __shfl_up_sync(0xffffffffu, v.x, off);
        double uy = __shfl_up_sync(0xffffffffu, v.y, off);
        int uf = __shfl_up_sync(0xffffffffu, f, off);
        if (lane >= off) {
            if (!f) {
                v.x = ux + v.x;
                v.y = uy + v.y;
            }
            f |= uf;
        }
    }
    if (lane == 31) {
        wsum[w] = v;
        wflag[w] = f;
    }
    __syncthreads();
    if (w == 0) {
        const int NW = NT / 32;
        double2 x = lane < NW ? wsum[lane] : make_double2(0.0, 0.0);
        int g = lane < NW ? wflag[lane] : 1;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            double ux = __shfl_up_sync(0xffffffffu, x.x, off);
            double uy = __shfl_up_sync(0xffffffffu, x.y, off);
            int ug = __shfl_up_sync(0xffffffffu, g, off);
            if (lane >= off) {
                if (!g) {
                    x.x = ux + x.x;
                    x.y = uy + x.y;
                }
                g |= ug;
            }
        }
        // exclusive carry for warp lane+1
        if (lane < NW) wsum[lane] = x;
    }
    __syncthreads();
    if (w > 0 && !f) {
        double2 c = wsum[w - 1];
        v.x = c.x + v.x;
        v.y = c.y + v.y;
    }
    P[threadIdx.x] = v;
    __syncthreads();
    return v;
}

template <typename T, int MODE, int KIND>
__global__ void __launch_bounds__(NT) tile_kernel(IterArgs a, VgParams prm)
{
    extern __shared__ __align__(16) unsigned char smem[];
    typedef typename GridEntry<T>::type GE;
    const int dim = a.dim;
    const int S = a.S;
    const int Tt = a.T;
    const int tid = threadIdx.x;
    const SmemPlan sp = smem_plan<T>(dim, a.maxK, Tt, a.table_smem, a.hist_smem, a.tab_len);
    GE *table = (GE *)(smem + sp.table);
    T *hsum = (T *)(smem + sp.hsum);
    unsigned int *hcnt = (unsigned int *)(smem + sp.hcnt);
    int *win_off = (int *)(smem + sp.win_off);
    int *win_n = (int *)(smem + sp.win_n);
    double *seg_S = (double *)(smem + sp.seg_S);
    int *keyF = (int *)(smem + sp.keyF);
    int *keyL = (int *)(smem + sp.keyL);
    double2 *Pv = (double2 *)(smem + sp.P);
    VgKSum *red = (VgKSum *)(smem + sp.red);
    float *itab = (float *)(smem + sp.itab);
    double2 *wsum = (double2 *)red;          // scan scratch (aliases red, used apart)
    int *wflag = (int *)(red + NT / 32 + 1);

    const int64_t ntiles = a.stats->ntiles;
    if ((int64_t)blockIdx.x >= ntiles) {   // uniform per CTA: nothing to do
        if (MODE != MODE_POINTS && tid == 0 && blockIdx.x < (unsigned)a.nparts) {
            CtaPart z;
            memset(&z, 0, sizeof(z));
            a.parts[blockIdx.x] = z;
        }
        return;
    }

    // ---- per-CTA setup: grid table, histogram, integrand constants
    if (a.table_smem) {
        for (int d = 0; d < dim; d++) {
            const int K = a.ninc[d];
            for (int i = tid; i <= K; i += NT) {
                GE e;
                if (i < K) {
                    e.x = (T)a.grid[d * a.ldg + i];
                    e.y = (T)a.inc[d * a.ldi + i];
                } else {
                    e.x = (T)a.grid[d * a.ldg + K];
                    e.y = (T)a.inc[d * a.ldi + K - 1];
                }
                table[(size_t)d * (a.maxK + 1) + i] = e;
            }
        }
    }
    if (MODE != MODE_POINTS && a.train && a.hist_smem) {
        for (int i = tid; i < dim * a.maxK; i += NT) {
            hsum[i] = (T)0;
            hcnt[i] = 0u;
        }
    }
    VgF32Consts kc;
    if (MODE == MODE_FUSED && sizeof(T) == 4) {
        kc = vg_prepare_f32<KIND>(prm, dim);
        vg_fill_table_f32<KIND>(prm, dim, itab, kc);
    }
    __syncthreads();

    VgKSum acc_mean = {0.0, 0.0}, acc_var = {0.0, 0.0}, acc_sigf = {0.0, 0.0};
    const double dv_y = __ddiv_rn(1.0, (double)a.H);
    const int64_t N = a.stats->neval;
    int nan_local = 0;
    const double beta_half = __ddiv_rn(a.beta, 2.0);

    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t tile_start = tile * (int64_t)Tt;
        const int tile_len = (int)min((int64_t)Tt, N - tile_start);
        const int64_t h0 = a.tile_h0[tile];
        const int64_t hnext = a.tile_h0[tile + 1];   // hypercube holding the next tile's first sample
        int64_t hlast = (hnext < a.H) ? hnext : a.H - 1;
        const int nwin = (int)(hlast - h0 + 1);
        if (nwin < 1 || nwin > Tt) {   // cannot happen when every count is >= 2
            if (tid == 0) a.stats->status = VG_ERR_UNSUPPORTED;
            break;
        }
        // window of relative offsets, clamped to [0, tile_len]
        for (int k = tid; k <= nwin; k += NT) {
            int64_t h = h0 + k;
            int64_t o = (h <= a.H) ? a.offsets[h] : N;
            int64_t r = o - tile_start;
            win_off[k] = (int)(r < 0 ? 0 : (r > tile_len ? tile_len : r));
            if (k < nwin) win_n[k] = a.neval_h[h];
        }
        __syncthreads();

        // ---- pass 0: samples of this thread: [li0, li0 + S)
        const int li0 = tid * S;
        int nmine = tile_len - li0;
        nmine = nmine < 0 ? 0 : (nmine > S ? S : nmine);
        double wf[8];
        int lhs[8];
        int lh = 0;
        if (nmine > 0) {
            int lo = 0, hi = nwin - 1;   // last k with win_off[k] <= li0
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (win_off[mid] <= li0) lo = mid;
                else hi = mid - 1;
            }
            lh = lo;
            while (lh + 1 < nwin && win_off[lh + 1] <= li0) lh++;
        }
        // mixed-radix decode of the first hypercube (axis 0 fastest, pyx:1736-1738)
        int y0[VG_MAX_DIM];
        {
            int64_t hh = h0 + lh;
            for (int d = 0; d < dim; d++) {
                int64_t q = hh / a.nstrat[d];
                y0[d] = (int)(hh - q * a.nstrat[d]);
                hh = q;
            }
        }
        int cur = lh;
        for (int k = 0; k < S; k++) {
            if (k >= nmine) break;
            const int li = li0 + k;
            while (li >= win_off[cur + 1]) {   // next hypercube: increment mixed radix
                cur++;
                for (int d = 0; d < dim; d++) {
                    if (++y0[d] < a.nstrat[d]) break;
                    y0[d] = 0;
                }
            }
            lhs[k] = cur;
            const int64_t ig = tile_start + li;
            const int nh = win_n[cur];
            T u[VG_MAX_DIM];
            if (a.u != nullptr) {
                for (int d = 0; d < dim; d++) u[d] = (T)a.u[ig * dim + d];
            } else {
                VgUniform<T>::draw(a.seed, a.stream, a.itn, (uint64_t)ig, dim, u);
            }
            T x[VG_MAX_DIM];
            T y[VG_MAX_DIM];
            int bins[VG_MAX_DIM];
            T jac = (T)1;
            for (int d = 0; d < dim; d++) {
                const int K = a.ninc[d];
                T yd;
                if (sizeof(T) == 8) {
                    yd = (T)__ddiv_rn(__dadd_rn((double)y0[d], (double)u[d]), (double)a.nstrat[d]);
                } else {
                    yd = __fdiv_rn((float)y0[d] + (float)u[d], (float)a.nstrat[d]);
                }
                y[d] = yd;
                T yn;
                if (sizeof(T) == 8) yn = (T)__dmul_rn((double)yd, (double)K);
                else yn = yd * (T)K;
                int iy = (sizeof(T) == 8) ? (int)floor((double)yn) : (int)floorf((float)yn);
                T dy = yn - (T)iy;
                GE e;
                int clamp = iy >= K;
                int ie = clamp ? K : iy;
                if (a.table_smem) {
                    e = table[(size_t)d * (a.maxK + 1) + ie];
                } else if (!clamp) {
                    e.x = (T)a.grid[d * a.ldg + ie];
                    e.y = (T)a.inc[d * a.ldi + ie];
                } else {
                    e.x = (T)a.grid[d * a.ldg + K];
                    e.y = (T)a.inc[d * a.ldi + K - 1];
                }
                if (sizeof(T) == 8) {
                    x[d] = clamp ? e.x : (T)__dadd_rn((double)e.x, __dmul_rn((double)e.y, (double)dy));
                    jac = (T)__dmul_rn((double)jac, __dmul_rn((double)e.y, (double)K));
                } else {
                    x[d] = clamp ? e.x : fmaf((float)e.y, (float)dy, (float)e.x);
                    jac = jac * (e.y * (T)K);
                }
                bins[d] = (yd > (T)0 && yd < (T)1 && iy < K) ? iy : -1;
            }
            // weight, pyx:1748-1749: jac *= dv_y / neval_hcube
            double wgt;
            if (sizeof(T) == 8) wgt = __dmul_rn((double)jac, __ddiv_rn(dv_y, (double)nh));
            else wgt = (double)((float)jac * ((float)dv_y / (float)nh));
            if (MODE == MODE_POINTS) {
                T *xo = (T *)a.x_out;
                for (int d = 0; d < dim; d++) xo[ig * dim + d] = x[d];
                if (a.y_out) {
                    T *yo = (T *)a.y_out;
                    for (int d = 0; d < dim; d++) yo[ig * dim + d] = y[d];
                }
                if (a.wgt_out) a.wgt_out[ig] = wgt;
                if (a.hc_out) a.hc_out[ig] = h0 + cur;
                continue;
            }
            double f;
            if (MODE == MODE_REDUCE) {
                f = a.f_f64 ? ((const double *)a.f_in)[ig] : (double)((const float *)a.f_in)[ig];
            } else {
                if (sizeof(T) == 8) f = vg_eval_f64<KIND>(prm, dim, (const double *)x);
                else f = (double)vg_eval_f32<KIND>(kc, itab, a.tab_len, dim, (const float *)x);
            }
            if (f != f) nan_local = 1;
            const double w1 = __dmul_rn(wgt, f);
            wf[k] = w1;
            if (a.train) {
                // fdv2 = (wgt*f*neval)^2, pyx:2173; |fdv2| into the bins, pyx:460-463
                double t1 = __dmul_rn(w1, (double)nh);
                double fd = __dmul_rn(t1, t1);
                for (int d = 0; d < dim; d++) {
                    if (bins[d] < 0) continue;
                    if (a.hist_smem) {
                        atomicAdd(&hsum[d * a.maxK + bins[d]], (T)fd);
                        atomicAdd(&hcnt[d * a.maxK + bins[d]], 1u);
                    } else {
                        atomicAdd(&a.sum_f[d * a.ldi + bins[d]], fd);
                        atomicAdd(&a.n_f[d * a.ldi + bins[d]], 1ull);
                    }
                }
            }
        }
        if (MODE == MODE_POINTS) {
            __syncthreads();
            continue;
        }

        // ---- pass 1: per-run sums of wf
        const int has = nmine > 0;
        const int fk = has ? lhs[0] : 0x7fffffff;
        const int lk = has ? lhs[nmine - 1] : 0x7fffffff;
        double fv = 0.0, lv = 0.0;
        {
            int k = 0;
            while (k < nmine && lhs[k] == fk) fv += wf[k++];
            if (lk != fk) {
                int kb = nmine - 1;
                while (kb > 0 && lhs[kb - 1] == lk) kb--;
                for (int q = kb; q < nmine; q++) lv += wf[q];
            } else {
                lv = fv;
            }
        }
        keyF[tid] = fk;
        keyL[tid] = lk;
        __syncthreads();
        const int prevL = tid > 0 ? keyL[tid - 1] : -1;
        const int nextF = tid < NT - 1 ? keyF[tid + 1] : -2;
        const int flag = (tid == 0) || (lk != prevL);
        double2 Pi = seg_scan(flag, make_double2(lv, 0.0), Pv, wsum, wflag);
        const double carry1 = (tid > 0 && prevL == fk && has) ? Pv[tid - 1].x : 0.0;
        const int ends_last = has && (lk != nextF);
        // segment totals of the first / last run
        double S_first = (lk != fk) ? fv + carry1 : (ends_last ? Pi.x : 0.0);
        double S_last = Pi.x;
        if (has && lk != fk) seg_S[fk] = S_first;
        if (ends_last) seg_S[lk] = S_last;
        __syncthreads();

        // ---- pass 2: deviations about the segment mean (pyx:2154-2171)
        double2 dq_first = make_double2(0.0, 0.0), dq_last = make_double2(0.0, 0.0);
        {
            int k = 0;
            while (k < nmine) {
                const int key = lhs[k];
                int k1 = k;
                double Sloc = 0.0;
                while (k1 < nmine && lhs[k1] == key) Sloc += wf[k1++];
                const int nin = win_off[key + 1] - win_off[key];
                const bool is_first = (key == fk), is_last = (key == lk);
                const double Sseg = (is_first || is_last) ? seg_S[key] : Sloc;
                const double m = __ddiv_rn(Sseg, (double)nin);
                const double thr = __dmul_rn(VG_EPSILON, fabs(m));
                double Dr = 0.0, Qr = 0.0;
                for (int q = k; q < k1; q++) {
                    double dwf = __dsub_rn(wf[q], m);
                    if (fabs(dwf) < thr) {
                        Qr = __dadd_rn(Qr, __dmul_rn(thr, thr));
                    } else {
                        Qr = __dadd_rn(Qr, __dmul_rn(dwf, dwf));
                        Dr = __dadd_rn(Dr, dwf);
                    }
                }
                if (is_first) dq_first = make_double2(Dr, Qr);
                if (is_last) dq_last = make_double2(Dr, Qr);
                if (!is_first && !is_last) {
                    // run wholly inside this thread: finalise now
                    const int64_t h = h0 + key;
                    const int nh = win_n[key];
                    const double nd = (double)nin;
                    double vh = __ddiv_rn(__dsub_rn(__dmul_rn(nd, Qr), __dmul_rn(Dr, Dr)),
                                          __dsub_rn(nd, 1.));
                    (void)nh;
                    acc_mean.add(__dadd_rn(Sseg, Dr));
                    acc_var.add(vh);
                    if (a.adaptive) {
                        double sg = pow(fabs(vh), beta_half);
                        a.sigf[h] = sg;
                        acc_sigf.add(sg);
                    }
                }
                k = k1;
            }
        }
        // cross-thread totals of (D, Q) for first/last runs
        __syncthreads();
        double2 Pq = seg_scan(flag, dq_last, Pv, wsum, wflag);
        double2 carry2 = (tid > 0 && prevL == fk && has) ? Pv[tid - 1] : make_double2(0.0, 0.0);
        // finalise segments ending in this thread: first run (if multi-run) and last run
        for (int which = 0; which < 2; which++) {
            int key;
            double2 dq;
            if (which == 0) {
                if (!(has && lk != fk)) continue;
                key = fk;
                dq = make_double2(dq_first.x + carry2.x, dq_first.y + carry2.y);
            } else {
                if (!ends_last) continue;
                key = lk;
                dq = Pq;
            }
            const int64_t h = h0 + key;
            const int nin = win_off[key + 1] - win_off[key];
            const int nh = win_n[key];
            const double Sseg = seg_S[key];
            const int64_t ostart = a.offsets[h];
            const bool starts_before = ostart < tile_start;
            const bool ends_after = ostart + nh > tile_start + tile_len;
            if (!starts_before && !ends_after) {
                const double nd = (double)nin;
                double vh = __ddiv_rn(__dsub_rn(__dmul_rn(nd, dq.y), __dmul_rn(dq.x, dq.x)),
                                      __dsub_rn(nd, 1.));
                acc_mean.add(__dadd_rn(Sseg, dq.x));
                acc_var.add(vh);
                if (a.adaptive) {
                    double sg = pow(fabs(vh), beta_half);
                    a.sigf[h] = sg;
                    acc_sigf.add(sg);
                }
            } else {
                TileRec r;
                r.h = h;
                r.n = (double)nin;
                r.S = Sseg;
                r.Q = dq.y;
                r.D = dq.x;
                r.spans = (starts_before && ends_after) ? 1 : 0;
                r.pad = 0;
                a.recs[2 * tile + (starts_before ? 0 : 1)] = r;
            }
        }
        // empty record slots: written by thread 0 when the tile has none
        if (tid == 0) {
            int64_t o0 = a.offsets[h0];
            if (!(o0 < tile_start)) a.recs[2 * tile].h = -1;
            int64_t hl = h0 + (nwin - 1);
            // the last hypercube touching the tile: does it continue past it?
            int lastkey = nwin - 1;
            while (lastkey > 0 && win_off[lastkey] >= tile_len) lastkey--;
            int64_t hL = h0 + lastkey;
            (void)hl;
            bool tail = (a.offsets[hL] + a.neval_h[hL] > tile_start + tile_len) &&
                        !(hL == h0 && o0 < tile_start);
            if (!tail) a.recs[2 * tile + 1].h = -1;
        }
        __syncthreads();
    }

    // ---- CTA epilogue: histogram flush, partial sums
    if (MODE != MODE_POINTS) {
        if (nan_local) atomicExch((int *)&a.stats->nan_seen, 1);
        if (a.train && a.hist_smem) {
            __syncthreads();
            for (int d = 0; d < dim; d++) {
                const int K = a.ninc[d];
                for (int i = tid; i < K; i += NT) {
                    unsigned int c = hcnt[d * a.maxK + i];
                    if (c) {
                        atomicAdd(&a.sum_f[d * a.ldi + i], (double)hsum[d * a.maxK + i]);
                        atomicAdd(&a.n_f[d * a.ldi + i], (unsigned long long)c);
                    }
                }
            }
        }
        VgKSum m = vg_block_ksum<NT>(acc_mean, red);
        VgKSum v = vg_block_ksum<NT>(acc_var, red);
        VgKSum s = vg_block_ksum<NT>(acc_sigf, red);
        if (tid == 0 && blockIdx.x < (unsigned)a.nparts) {
            CtaPart p;
            p.mean = m;
            p.var = v;
            p.sigf = s;
            a.parts[blockIdx.x] = p;
        }
    }
}

// ========================================================== finalize
// Chan et al. merge of partial (n, S, Q, D) for hypercubes cut by tiles,
// then the fixed-order compensated sums of all CTA partials.
__global__ void __launch_bounds__(FIN_NT) finalize_kernel(IterArgs a, int nctas)
{
    __shared__ VgKSum red[FIN_NT / 32];
    const vg_stats *st = a.stats;
    const int64_t ntiles = st->ntiles;
    const double beta_half = __ddiv_rn(a.beta, 2.0);
    VgKSum cm = {0.0, 0.0}, cv = {0.0, 0.0}, cs = {0.0, 0.0};
    for (int64_t t = threadIdx.x; t < ntiles; t += FIN_NT) {
        TileRec r = a.recs[2 * t + 1];
        if (r.h < 0) continue;
        double n = r.n, Sx = r.S, Q = r.Q, D = r.D;
        for (int64_t t2 = t + 1; t2 < ntiles; t2++) {
            TileRec q = a.recs[2 * t2];
            if (q.h != r.h) break;
            double n2 = n + q.n;
            double delta = q.S / q.n - Sx / n;
            Q = Q + q.Q + delta * delta * (n * q.n / n2);
            Sx += q.S;
            D += q.D;
            n = n2;
            if (!q.spans) break;
        }
        double vh = __ddiv_rn(__dsub_rn(__dmul_rn(n, Q), __dmul_rn(D, D)), __dsub_rn(n, 1.));
        cm.add(__dadd_rn(Sx, D));
        cv.add(vh);
        if (a.adaptive) {
            double sg = pow(fabs(vh), beta_half);
            a.sigf[r.h] = sg;
            cs.add(sg);
        }
    }
    // fixed order: every thread folds in its share of CTA partials
    for (int c = threadIdx.x; c < nctas; c += FIN_NT) {
        CtaPart p = a.parts[c];
        cm.merge(p.mean);
        cv.merge(p.var);
        cs.merge(p.sigf);
    }
    VgKSum M = vg_block_ksum<FIN_NT>(cm, red);
    VgKSum V = vg_block_ksum<FIN_NT>(cv, red);
    VgKSum Sg = vg_block_ksum<FIN_NT>(cs, red);
    __shared__ int reset;
    if (threadIdx.x == 0) {
        vg_stats *s = a.stats;
        s->mean = M.value();
        s->var = V.value();
        reset = 0;
        s->sigf_reset = 0;
        if (a.adaptive) {
            double ss = Sg.value();
            if (ss > 0) {
                s->sum_sigf = ss;
            } else {   // constant integrand: even distribution (pyx:2212-2215)
                s->sum_sigf = (double)a.H;
                s->sigf_reset = 1;
                reset = 1;
            }
        }
    }
    __syncthreads();
    if (reset)
        for (int64_t h = threadIdx.x; h < a.H; h += FIN_NT) a.sigf[h] = 1.0;
}

// ================================================================ host
int fill_args(IterArgs &a, const vg_integrator *it, uint32_t itn, const double *u)
{
    memset(&a, 0, sizeof(a));
    if (it->dim < 1 || it->dim > VG_MAX_DIM) return vg_fail(VG_ERR_UNSUPPORTED, "dim");
    if (it->adapt_to_errors) return vg_fail(VG_ERR_UNSUPPORTED, "adapt_to_errors");
    if (!it->work || !it->stats) return vg_fail(VG_ERR_VALUE, "missing workspace/stats");
    a.dim = it->dim;
    a.T = tile_size(it);
    a.S = samples_per_thread(it);
    if (a.S < 1 || a.S > 8 || a.S * NT != a.T) return vg_fail(VG_ERR_VALUE, "bad tile size");
    int maxK = 1;
    for (int d = 0; d < it->dim; d++) {
        if (it->nstrat[d] < 1 || it->ninc[d] < 1) return vg_fail(VG_ERR_VALUE, "bad geometry");
        a.nstrat[d] = (int)it->nstrat[d];
        a.ninc[d] = (int)it->ninc[d];
        maxK = a.ninc[d] > maxK ? a.ninc[d] : maxK;
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
    a.adaptive_alloc = (it->beta > 0 && it->nhcube > 1) ? 1 : 0;
    a.adaptive = (a.adaptive_alloc && it->adapt) ? 1 : 0;
    a.train = (it->adapt && it->alpha > 0) ? 1 : 0;
    a.sum_f = it->sum_f;
    a.n_f = (unsigned long long *)it->n_f;
    a.stats = it->stats;
    a.neval_h = (int32_t *)(w + L.neval_h);
    a.offsets = (int64_t *)(w + L.offsets);
    a.bsum = (int64_t *)(w + L.bsum);
    a.bmax = (int64_t *)(w + L.bmax);
    a.tile_h0 = (int64_t *)(w + L.tile_h0);
    a.recs = (TileRec *)(w + L.recs);
    a.chain = (ChainRes *)(w + L.chain);
    a.parts = (CtaPart *)(w + L.parts);
    a.nparts = (int)L.nparts;
    a.ntiles_cap = L.ntiles_cap;
    a.neval = it->neval;
    a.neval_frac = it->neval_frac;
    a.min_neval_hcube = it->min_neval_hcube;
    a.max_neval_hcube = it->max_neval_hcube;
    a.seed = it->seed;
    a.stream = it->stream_id;
    a.itn = itn;
    a.u = u;
    return VG_OK;
}

template <typename T, int MODE, int KIND>
int launch_tile(IterArgs &a, const VgParams *prm, int tab_len, cudaStream_t st)
{
    const int dim = a.dim;
    a.tab_len = tab_len;
    // shared-memory plan: table and histogram in shared memory when they fit
    const size_t budget = 200 * 1024;
    a.table_smem = 1;
    a.hist_smem = (MODE != MODE_POINTS && a.train) ? 1 : 0;
    SmemPlan p = smem_plan<T>(dim, a.maxK, a.T, a.table_smem, a.hist_smem, tab_len);
    if (p.total > budget && a.hist_smem) {
        a.hist_smem = 0;
        p = smem_plan<T>(dim, a.maxK, a.T, a.table_smem, a.hist_smem, tab_len);
    }
    if (p.total > budget) {
        a.table_smem = 0;
        p = smem_plan<T>(dim, a.maxK, a.T, a.table_smem, a.hist_smem, tab_len);
    }
    if (p.total > 227 * 1024) return vg_fail(VG_ERR_UNSUPPORTED, "shared memory plan too large");
    auto kern = tile_kernel<T, MODE, KIND>;
    static bool attr_set = false;
    if (!attr_set) {
        VG_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           227 * 1024));
        attr_set = true;
    }
    int per_sm = 0;
    VG_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, p.total));
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)vg_num_sms() * per_sm;
    if (grid > a.ntiles_cap) grid = a.ntiles_cap;
    if (grid > a.nparts) grid = a.nparts;
    if (grid < 1) grid = 1;
    static VgParams empty;
    kern<<<(unsigned)grid, NT, p.total, st>>>(a, prm ? *prm : empty);
    VG_LAUNCH_CHECK();
    if (MODE != MODE_POINTS) {
        finalize_kernel<<<1, FIN_NT, 0, st>>>(a, (int)grid);
        VG_LAUNCH_CHECK();
    }
    return VG_OK;
}

}  // namespace

// ====================================================================== ABI
extern "C" int64_t vg_neval_cap(const vg_integrator *it) { return neval_cap(it); }

extern "C" size_t vg_workspace_bytes(const vg_integrator *it, int64_t ncap)
{
    if (ncap <= 0) ncap = neval_cap(it);
    return layout(it, ncap).total;
}

extern "C" int vg_allocate(const vg_integrator *it, void *stream)
{
    vg_clear_error();
    IterArgs a;
    int rc = fill_args(a, it, 0, nullptr);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    WorkLayout L = layout(it, a.ncap);
    alloc_count_kernel<<<(unsigned)L.nblk, ALLOC_NT, 0, st>>>(a);
    VG_LAUNCH_CHECK();
    alloc_scan_kernel<<<1, ALLOC_NT, 0, st>>>(a, L.nblk);
    VG_LAUNCH_CHECK();
    alloc_offsets_kernel<<<(unsigned)L.nblk, ALLOC_NT, 0, st>>>(a);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

extern "C" int vg_sample(const vg_integrator *it, uint32_t itn, const double *u, void *x, void *y,
                         double *wgt, int64_t *hcube, int64_t n_cap, void *stream)
{
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
    if (it->precision == VG_F64)
        return launch_tile<double, MODE_POINTS, 0>(a, nullptr, 0, (cudaStream_t)stream);
    return launch_tile<float, MODE_POINTS, 0>(a, nullptr, 0, (cudaStream_t)stream);
}

extern "C" int vg_reduce(const vg_integrator *it, uint32_t itn, const double *u, const void *f,
                         int f_dtype, void *stream)
{
    vg_clear_error();
    IterArgs a;
    int rc = fill_args(a, it, itn, u);
    if (rc) return rc;
    a.f_in = f;
    a.f_f64 = (f_dtype == VG_F64);
    if (it->precision == VG_F64)
        return launch_tile<double, MODE_REDUCE, 0>(a, nullptr, 0, (cudaStream_t)stream);
    return launch_tile<float, MODE_REDUCE, 0>(a, nullptr, 0, (cudaStream_t)stream);
}

template <int KIND>
static int fused_dispatch(IterArgs &a, const vg_integrator *it, const VgParams &P, cudaStream_t st)
{
    int tab_len = 0;
    if (KIND == VG_F_RIDGE) tab_len = (int)P.p[0];
    else if (KIND == VG_F_MIXTURE) tab_len = (int)P.p[0] * it->dim;
    else if (KIND == VG_F_LORENTZ) tab_len = 4 * it->dim;
    if (it->precision == VG_F64) return launch_tile<double, MODE_FUSED, KIND>(a, &P, tab_len, st);
    return launch_tile<float, MODE_FUSED, KIND>(a, &P, tab_len, st);
}

extern "C" int vg_fused_iteration(const vg_integrator *it, uint32_t itn, const double *u, int kind,
                                  const double *params, int nparams, void *stream)
{
    vg_clear_error();
    IterArgs a;
    int rc = fill_args(a, it, itn, u);
    if (rc) return rc;
    if (nparams < 0 || nparams > VG_MAX_PARAMS) return vg_fail(VG_ERR_VALUE, "too many params");
    static VgParams P;
    memset(&P, 0, sizeof(P));
    P.n = nparams;
    for (int i = 0; i < nparams; i++) P.p[i] = params[i];
    // validate parameter counts per integrand
    int need = 0;
    switch (kind) {
    case VG_F_GAUSS: need = 3; break;
    case VG_F_RIDGE: need = 2; break;
    case VG_F_LORENTZ: need = 2 * it->dim; break;
    case VG_F_MIXTURE: need = nparams >= 1 ? 2 + (int)params[0] * it->dim : 1; break;
    case VG_F_LATTICE: need = 2; break;
    case VG_F_CONST: need = 1; break;
    default: return vg_fail(VG_ERR_VALUE, "unknown integrand kind %d", kind);
    }
    if (nparams < need) return vg_fail(VG_ERR_VALUE, "integrand needs %d parameters", need);
    if (kind == VG_F_RIDGE && (params[0] < 1 || params[0] > 65536))
        return vg_fail(VG_ERR_VALUE, "ridge M out of range");
    cudaStream_t st = (cudaStream_t)stream;
    switch (kind) {
    case VG_F_GAUSS: return fused_dispatch<VG_F_GAUSS>(a, it, P, st);
    case VG_F_RIDGE: return fused_dispatch<VG_F_RIDGE>(a, it, P, st);
    case VG_F_LORENTZ: return fused_dispatch<VG_F_LORENTZ>(a, it, P, st);
    case VG_F_MIXTURE: return fused_dispatch<VG_F_MIXTURE>(a, it, P, st);
    case VG_F_LATTICE: return fused_dispatch<VG_F_LATTICE>(a, it, P, st);
    default: return fused_dispatch<VG_F_CONST>(a, it, P, st);
    }
}

int vg_adapt_launch(int dim, const int64_t *old_ninc, const int64_t *new_ninc, const double *grid,
                    const double *inc, int64_t ldg, int64_t ldi, const double *sum_f,
                    const uint64_t *n_f, double alpha, double *new_grid, double *new_inc,
                    int64_t ldg_new, int64_t ldi_new, cudaStream_t st);

extern "C" int vg_end_iteration(const vg_integrator *it, void *stream)
{
    vg_clear_error();
    cudaStream_t st = (cudaStream_t)stream;
    if (!(it->adapt && it->alpha > 0)) return VG_OK;
    WorkLayout L = layout(it, neval_cap(it));
    if (it->work_bytes < L.total) return vg_fail(VG_ERR_VALUE, "workspace too small");
    char *w = (char *)it->work;
    double *ng = (double *)(w + L.newgrid);
    double *ni = (double *)(w + L.newinc);
    int rc = vg_adapt_launch(it->dim, it->ninc, it->ninc, it->grid, it->inc, it->ldg, it->ldi,
                             it->sum_f, it->n_f, it->alpha, ng, ni, it->ldg, it->ldi, st);
    if (rc) return rc;
    VG_CUDA_CHECK(cudaMemcpyAsync(it->grid, ng, sizeof(double) * it->dim * it->ldg,
                                  cudaMemcpyDeviceToDevice, st));
    VG_CUDA_CHECK(cudaMemcpyAsync(it->inc, ni, sizeof(double) * it->dim * it->ldi,
                                  cudaMemcpyDeviceToDevice, st));
    VG_CUDA_CHECK(cudaMemsetAsync(it->sum_f, 0, sizeof(double) * it->dim * it->ldi, st));
    VG_CUDA_CHECK(cudaMemsetAsync(it->n_f, 0, sizeof(uint64_t) * it->dim * it->ldi, st));
    return VG_OK;
}
