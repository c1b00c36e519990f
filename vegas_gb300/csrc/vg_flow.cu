// vg_flow.cu -- learned proposal: a coupling-layer normalising flow with
// piecewise-quadratic transforms (Mueller et al., "Neural Importance
// Sampling", ACM TOG 2019), composed after the AdaptiveMap.  No reference
// counterpart: the reference vegas has no learned proposal.
//
// The flow lives on the unit cube.  Density direction (training): z (sample)
// -> layer 0 CDF -> ... -> layer L-1 CDF -> zhat, logdet = sum log pdf.
// Sampling direction: zhat -> inverse CDFs L-1..0 -> z, log|dz/dzhat| =
// -logdet.  Conditioner of layer l: out = W3 relu(W2 relu(W1 z_A + b1) + b2)
// + b3; per transformed coordinate j, out[j(2K+1) + k] are K width logits and
// out[j(2K+1) + K + k] K+1 vertex logits.  Parameter layout, masks and spline
// match oracle/flow_oracle.py (the FP64 checker).
//
// Kernels on the 5th-generation tensor cores (CTA = 512 threads = 16 warps,
// one per SM, TMEM accumulators; K in {16, 32}):
//   flow_pass_umma_kernel   inference (sampling / density) and the training
//                           forward (storing each layer's input)
//   flow_bwd_umma_kernel    training backward of one layer: forward
//                           recomputation, spline backward in registers,
//                           dH2, dH1 and dW1 with TMEM accumulators
//   flow_wgrad_img_kernel   dW2, dW3 (and db2, db3) over the backward's
//                           tile images + flow_wgrad_img_reduce_kernel
// Kernels on mma.sync.m16n8k16 (BF16, FP32 accumulation; CTA = 256 threads,
// 128 rows per tile), for K outside {16, 32} and as the tests' comparison
// path:
//   flow_pass_kernel        inference and training forward
//   flow_bwd_kernel         training backward of one layer: recompute
//                           activations, spline backward, dOUT/dH2/dH1
//                           through the MLP, the transposed activations and
//                           gradients for flow_wgrad_umma_kernel (split-K
//                           weight gradients on tcgen05) + flow_wgrad_reduce_kernel
// Shared by both: flow_adam_kernel (Adam on the FP32 parameters),
// flow_mirror_kernel (BF16 copies and tcgen05 operand images of W2, W3),
// train_gather_kernel / train_norm_kernel (the training batch).
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include "vg_common.cuh"
#include "vg_umma.cuh"

namespace {

constexpr int FH = 128;           // hidden width (fixed)
constexpr int FROWS = 128;        // rows per tile
constexpr int FNT = 256;          // threads per CTA
constexpr int FMAXD = 16;         // maximum dimension
constexpr int FMAXL = 8;          // maximum layers
constexpr int FMAXK = 48;         // maximum bins (shared-memory bound of the backward)
constexpr int HSTR = FH + 8;      // padded row stride (bf16) of hidden activations
constexpr float EPS_W = 1e-3f;    // minimum bin width fraction (oracle EPS_W)
constexpr size_t VG_FLOW_SMEM_MAX = 227 * 1024;   // dynamic shared memory per CTA

struct FlowLayer {
    int dA, dB, P;                 // conditioning / transformed dims, outputs
    int A[FMAXD], B[FMAXD];
    int64_t oW1, ob1, oW2, ob2, oW3, ob3;   // offsets into theta
    int64_t mW2, mW2t, mW3, mW3t;           // offsets (elements) into the bf16 mirror
    int64_t mU2, mU3;              // tcgen05 operand images of W2 [128 x 128] and W3 [NP x 128]
    int NP;                        // W3 image rows: dB*CH padded to 16
    int realA;                     // 0 when the layer conditions on nothing
};

struct FlowGeom {
    int dim, L, K, CH;             // CH = per-coordinate output chunk rows (2K+1 padded to 8)
    int CHK;                       // CH padded to a multiple of 16 (K dim of dOUT . W3)
    FlowLayer ly[FMAXL];
    int64_t nparams, nmirror;
    int NPmax, dAmax, dBmax;
};

// masks: bit b = (l/2) % nbits of the coordinate index; B = bit == l % 2
int make_geom(FlowGeom &g, int dim, int L, int K, int hidden)
{
    memset(&g, 0, sizeof(g));
    if (dim < 1 || dim > FMAXD) return vg_fail(VG_ERR_UNSUPPORTED, "flow dim %d (1..%d)", dim, FMAXD);
    if (L < 1 || L > FMAXL) return vg_fail(VG_ERR_UNSUPPORTED, "flow layers %d (1..%d)", L, FMAXL);
    if (K < 2 || K > FMAXK) return vg_fail(VG_ERR_UNSUPPORTED, "flow bins %d (2..%d)", K, FMAXK);
    if (hidden != FH) return vg_fail(VG_ERR_UNSUPPORTED, "flow hidden width must be %d", FH);
    g.dim = dim;
    g.L = L;
    g.K = K;
    g.CH = ((2 * K + 1) + 7) / 8 * 8;
    g.CHK = (g.CH + 15) / 16 * 16;
    int nbits = 1;
    while ((1 << nbits) < dim) nbits++;
    int64_t o = 0, m = 0;
    for (int l = 0; l < L; l++) {
        FlowLayer &y = g.ly[l];
        int b = (l / 2) % nbits;
        y.dA = y.dB = 0;
        for (int i = 0; i < dim; i++) {
            if (((i >> b) & 1) == (l % 2)) y.B[y.dB++] = i;
            else y.A[y.dA++] = i;
        }
        y.realA = 1;
        if (y.dA == 0 || y.dB == 0) {   // dim 1: condition on nothing
            y.dA = 0;
            y.dB = dim;
            for (int i = 0; i < dim; i++) y.B[i] = i;
            y.realA = 0;
        }
        const int dA = y.dA > 0 ? y.dA : 1;
        y.P = y.dB * (2 * K + 1);
        y.oW1 = o; o += (int64_t)FH * dA;
        y.ob1 = o; o += FH;
        y.oW2 = o; o += (int64_t)FH * FH;
        y.ob2 = o; o += FH;
        y.oW3 = o; o += (int64_t)y.P * FH;
        y.ob3 = o; o += y.P;
        y.mW2 = m;  m += (int64_t)FH * HSTR;              // [n][k]
        y.mW2t = m; m += (int64_t)FH * HSTR;              // [k][n]
        y.mW3 = m;  m += (int64_t)y.dB * g.CH * HSTR;     // [j][o][k]
        y.mW3t = m; m += (int64_t)y.dB * FH * (g.CHK + 8);   // [j][k][o]
        y.NP = (y.dB * g.CH + 15) / 16 * 16;
        y.mU2 = m; m += (int64_t)FH * FH;
        y.mU3 = m; m += (int64_t)y.NP * FH;
        if (y.NP > g.NPmax) g.NPmax = y.NP;
        if (dA > g.dAmax) g.dAmax = dA;
        if (y.dB > g.dBmax) g.dBmax = y.dB;
    }
    g.nparams = o;
    g.nmirror = m;
    return VG_OK;
}

// ------------------------------------------------------------ MMA helpers
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Warp GEMM block: acc[MT][NT8] (+)= A[m0.., k] * B[k, n0..], K a multiple of
// 16.  A is row-major bf16 with K contiguous (lda elements per row); B is
// given as Bt[n][k] row-major (K contiguous, ldb).  Fragment layouts of
// mma.m16n8k16 (PTX ISA): g = lane/4, t = lane%4.
template <int MT, int NT8>
__device__ __forceinline__ void warp_gemm(float (&acc)[MT][NT8][4], const __nv_bfloat16 *A, int lda,
                                          int m0, const __nv_bfloat16 *Bt, int ldb, int n0, int K)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    for (int k0 = 0; k0 < K; k0 += 16) {
        uint32_t af[MT][4];
#pragma unroll
        for (int mt = 0; mt < MT; mt++) {
            const __nv_bfloat16 *r0 = A + (size_t)(m0 + 16 * mt + g) * lda + k0 + 2 * t;
            const __nv_bfloat16 *r1 = r0 + (size_t)8 * lda;
            af[mt][0] = *reinterpret_cast<const uint32_t *>(r0);
            af[mt][1] = *reinterpret_cast<const uint32_t *>(r1);
            af[mt][2] = *reinterpret_cast<const uint32_t *>(r0 + 8);
            af[mt][3] = *reinterpret_cast<const uint32_t *>(r1 + 8);
        }
#pragma unroll
        for (int nt = 0; nt < NT8; nt++) {
            const __nv_bfloat16 *c0 = Bt + (size_t)(n0 + 8 * nt + g) * ldb + k0 + 2 * t;
            uint32_t bf[2];
            bf[0] = *reinterpret_cast<const uint32_t *>(c0);
            bf[1] = *reinterpret_cast<const uint32_t *>(c0 + 8);
#pragma unroll
            for (int mt = 0; mt < MT; mt++) mma_bf16(acc[mt][nt], af[mt], bf);
        }
    }
}

template <int MT, int NT8>
__device__ __forceinline__ void zero_acc(float (&acc)[MT][NT8][4])
{
#pragma unroll
    for (int i = 0; i < MT; i++)
#pragma unroll
        for (int j = 0; j < NT8; j++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[i][j][q] = 0.f;
}

// ----------------------------------------------------------- spline math
// Row of 2K+1 logits o[]; forward and inverse of the piecewise-quadratic
// CDF.  On exit o[k] holds the softmax probability s_k (k < K) and o[K+k] the
// unnormalised vertex height u_k (k <= K), which the backward reuses.
struct SplineState {
    float Z, P, E, W, ub, ub1, alpha, num, pdfu;
    int b;
};

__device__ __forceinline__ void spline_prepare(float *o, int K, float &Zout)
{
    float mx = -3.0e38f, mv = -3.0e38f;
    for (int k = 0; k < K; k++) mx = fmaxf(mx, o[k]);
    for (int k = 0; k <= K; k++) mv = fmaxf(mv, o[K + k]);
    float se = 0.f;
    for (int k = 0; k < K; k++) {
        const float e = __expf(o[k] - mx);
        o[k] = e;
        se += e;
    }
    const float rse = 1.f / se;
    for (int k = 0; k < K; k++) o[k] *= rse;
    for (int k = 0; k <= K; k++) o[K + k] = __expf(o[K + k] - mv);
    const float c1 = 1.f - K * EPS_W;
    float Z = 0.f;
    for (int k = 0; k < K; k++) Z += 0.5f * (o[K + k] + o[K + k + 1]) * (EPS_W + c1 * o[k]);
    Zout = Z;
}

// CDF at x (density direction).
__device__ __forceinline__ float spline_cdf(const float *o, int K, float Z, float x,
                                            SplineState &s)
{
    const float c1 = 1.f - K * EPS_W;
    float E = 0.f, P = 0.f;
    int b = K - 1;
    for (int k = 0; k < K; k++) {
        const float W = EPS_W + c1 * o[k];
        if (x < E + W || k == K - 1) {
            b = k;
            break;
        }
        E += W;
        P += 0.5f * (o[K + k] + o[K + k + 1]) * W;
    }
    const float W = EPS_W + c1 * o[b];
    const float ub = o[K + b], ub1 = o[K + b + 1];
    float al = (x - E) / W;
    al = fminf(fmaxf(al, 0.f), 1.f);
    const float num = P + W * (al * ub + 0.5f * al * al * (ub1 - ub));
    s.Z = Z; s.P = P; s.E = E; s.W = W; s.ub = ub; s.ub1 = ub1; s.alpha = al; s.b = b;
    s.num = num;
    s.pdfu = (1.f - al) * ub + al * ub1;
    return num / Z;
}

// Inverse CDF at c (sampling direction): returns x, fills the state at x.
__device__ __forceinline__ float spline_inv(const float *o, int K, float Z, float c,
                                            SplineState &s)
{
    const float c1 = 1.f - K * EPS_W;
    const float cz = c * Z;
    float E = 0.f, P = 0.f;
    int b = K - 1;
    for (int k = 0; k < K; k++) {
        const float W = EPS_W + c1 * o[k];
        const float seg = 0.5f * (o[K + k] + o[K + k + 1]) * W;
        if (cz < P + seg || k == K - 1) {
            b = k;
            break;
        }
        E += W;
        P += seg;
    }
    const float W = EPS_W + c1 * o[b];
    const float ub = o[K + b], ub1 = o[K + b + 1];
    const float qa = 0.5f * W * (ub1 - ub), qb = W * ub;
    const float r = fmaxf(cz - P, 0.f);
    float al = 2.f * r / fmaxf(qb + sqrtf(fmaxf(qb * qb + 4.f * qa * r, 0.f)), 1e-30f);
    al = fminf(fmaxf(al, 0.f), 1.f);
    s.Z = Z; s.P = P; s.E = E; s.W = W; s.ub = ub; s.ub1 = ub1; s.alpha = al; s.b = b;
    s.num = P + W * (al * ub + 0.5f * al * al * (ub1 - ub));
    s.pdfu = (1.f - al) * ub + al * ub1;
    return E + al * W;
}

// Backward of (C, logpdf) at the state s w.r.t. x and the logits: on entry
// o[] holds the softmax probabilities and vertex heights left by
// spline_prepare; on exit o[0..2K] holds dL/dlogits.  Returns dL/dx.
//   C = (P_b + W_b (a u_b + a^2/2 (u_{b+1}-u_b))) / Z,
//   log pdf = log((1-a) u_b + a u_{b+1}) - log Z,   a = (x - E_b) / W_b,
//   W_k = EPS_W + (1 - K EPS_W) softmax(w)_k,  u_k = exp(v_k - max v).
__device__ __forceinline__ float spline_backward(float *o, int K, const SplineState &s, float gC,
                                                 float gL)
{
    const float c1 = 1.f - K * EPS_W;
    const float Z = s.Z, al = s.alpha, W = s.W, ub = s.ub, ub1 = s.ub1;
    const int b = s.b;
    const float g_num = gC / Z;
    const float g_Z = -gC * s.num / (Z * Z) - gL / Z;
    const float g_pdfu = gL / s.pdfu;
    const float g_al = g_pdfu * (ub1 - ub) + g_num * W * (ub + al * (ub1 - ub));
    const float g_ub = g_pdfu * (1.f - al) + g_num * W * (al - 0.5f * al * al);
    const float g_ub1 = g_pdfu * al + g_num * W * 0.5f * al * al;
    const float g_Wb = g_num * (al * ub + 0.5f * al * al * (ub1 - ub)) - g_al * al / W;
    const float g_x = g_al / W;
    const float g_E = -g_al / W;
    // pass A: dot = sum_k s_k c1 dL/dW_k (softmax Jacobian)
    float dot = 0.f;
    for (int k = 0; k < K; k++) {
        const float us = o[K + k] + o[K + k + 1];
        float gW = 0.5f * g_Z * us;
        if (k < b) gW += g_E + 0.5f * g_num * us;
        if (k == b) gW += g_Wb;
        dot += o[k] * c1 * gW;
    }
    // pass B: write the logit gradients in place (W_{k-1} carried in Wprev)
    float Wprev = 0.f;
    for (int k = 0; k <= K; k++) {
        const float Wk = (k < K) ? EPS_W + c1 * o[k] : 0.f;
        float gu = 0.5f * g_Z * (Wprev + Wk);
        if (k >= 1 && k <= b) gu += 0.5f * g_num * Wprev;
        if (k < b) gu += 0.5f * g_num * Wk;
        if (k == b) gu += g_ub;
        if (k == b + 1) gu += g_ub1;
        if (k < K) {
            const float us = o[K + k] + o[K + k + 1];
            float gW = 0.5f * g_Z * us;
            if (k < b) gW += g_E + 0.5f * g_num * us;
            if (k == b) gW += g_Wb;
            o[k] = o[k] * (c1 * gW - dot);
        }
        o[K + k] = gu * o[K + k];
        Wprev = Wk;
    }
    return g_x;
}

// ------------------------------------------------------------ shared tiles
struct FlowSmem {
    float *Z;             // [FROWS][FMAXD] state
    float *G;             // [FROWS][FMAXD] gradient w.r.t. the layer output
    __nv_bfloat16 *H1;    // [FROWS][HSTR]
    __nv_bfloat16 *H2;    // [FROWS][HSTR]
    float *OUT;           // [FROWS][ostr] f32 conditioner outputs (2 chunks)
    __nv_bfloat16 *DOB;   // [FROWS][dstr] bf16 dL/dout of one chunk (backward)
    float *LD;            // [FROWS]
    float *RED;           // [8 * FROWS] scratch (column sums, partial row sums)
    int ostr, dstr;
};

__host__ __device__ inline size_t flow_smem_bytes(int CH, int CHK, int backward)
{
    size_t o = 0;
    o += sizeof(float) * FROWS * FMAXD;                 // Z
    o += sizeof(float) * FROWS * FMAXD;                 // G
    o += sizeof(__nv_bfloat16) * FROWS * HSTR * 2;      // H1, H2
    o += sizeof(float) * FROWS * (2 * CH + 4);          // OUT
    if (backward) o += sizeof(__nv_bfloat16) * FROWS * (CHK + 8);   // DOB
    o += sizeof(float) * FROWS;                         // LD
    o += sizeof(float) * 8 * FROWS;                     // RED
    return o;
}

__device__ inline FlowSmem flow_smem(unsigned char *base, int CH, int CHK, int backward)
{
    FlowSmem s;
    size_t o = 0;
    s.Z = (float *)(base + o);           o += sizeof(float) * FROWS * FMAXD;
    s.G = (float *)(base + o);           o += sizeof(float) * FROWS * FMAXD;
    s.H1 = (__nv_bfloat16 *)(base + o);  o += sizeof(__nv_bfloat16) * FROWS * HSTR;
    s.H2 = (__nv_bfloat16 *)(base + o);  o += sizeof(__nv_bfloat16) * FROWS * HSTR;
    s.OUT = (float *)(base + o);         o += sizeof(float) * FROWS * (2 * CH + 4);
    s.DOB = (__nv_bfloat16 *)(base + o); if (backward) o += sizeof(__nv_bfloat16) * FROWS * (CHK + 8);
    s.LD = (float *)(base + o);          o += sizeof(float) * FROWS;
    s.RED = (float *)(base + o);
    s.ostr = 2 * CH + 4;
    s.dstr = CHK + 8;
    return s;
}

// H1 = relu(W1 z_A + b1) (FP32 FMA, K = dA is tiny), H2 = relu(H1 W2^T + b2)
// on the tensor cores.
__device__ void flow_hidden(const FlowGeom &g, const FlowLayer &y, const float *theta,
                            const __nv_bfloat16 *mirror, FlowSmem &sm)
{
    const int tid = threadIdx.x;
    {
        const int r = tid & (FROWS - 1), half = tid >> 7;
        const float *W1 = theta + y.oW1;
        const float *b1 = theta + y.ob1;
        const int dA = y.realA ? y.dA : 1;
        float xa[FMAXD];
        for (int a2 = 0; a2 < dA; a2++) xa[a2] = y.realA ? sm.Z[r * FMAXD + y.A[a2]] : 0.f;
        for (int c = 64 * half; c < 64 * half + 64; c += 2) {
            float v0 = b1[c], v1 = b1[c + 1];
            for (int a2 = 0; a2 < dA; a2++) {
                v0 = fmaf(W1[c * dA + a2], xa[a2], v0);
                v1 = fmaf(W1[(c + 1) * dA + a2], xa[a2], v1);
            }
            *reinterpret_cast<uint32_t *>(&sm.H1[r * HSTR + c]) = pack_bf16(fmaxf(v0, 0.f), fmaxf(v1, 0.f));
        }
    }
    __syncthreads();
    {
        const int w = tid >> 5, lane = tid & 31, gq = lane >> 2, t = lane & 3;
        const int m0 = 32 * (w & 3), n0 = 64 * (w >> 2);
        float acc[2][8][4];
        zero_acc(acc);
        warp_gemm<2, 8>(acc, sm.H1, HSTR, m0, mirror + y.mW2, HSTR, n0, FH);
        const float *b2 = theta + y.ob2;
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                const int r = m0 + 16 * mt + gq, c = n0 + 8 * nt + 2 * t;
                const float bb0 = b2[c], bb1 = b2[c + 1];
                *reinterpret_cast<uint32_t *>(&sm.H2[r * HSTR + c]) =
                    pack_bf16(fmaxf(acc[mt][nt][0] + bb0, 0.f), fmaxf(acc[mt][nt][1] + bb1, 0.f));
                *reinterpret_cast<uint32_t *>(&sm.H2[(r + 8) * HSTR + c]) =
                    pack_bf16(fmaxf(acc[mt][nt][2] + bb0, 0.f), fmaxf(acc[mt][nt][3] + bb1, 0.f));
            }
    }
    __syncthreads();
}

// OUT chunk(s) for transformed coordinates j0 (and j0+1): OUT[r][jj*CH + o]
__device__ void flow_out(const FlowGeom &g, const FlowLayer &y, const float *theta,
                         const __nv_bfloat16 *mirror, FlowSmem &sm, int j0, int nj)
{
    const int tid = threadIdx.x;
    const int w = tid >> 5, lane = tid & 31, gq = lane >> 2, t = lane & 3;
    const int jj = w >> 2;
    if (jj < nj) {
        const int j = j0 + jj;
        const int m0 = 32 * (w & 3);
        const __nv_bfloat16 *Bt = mirror + y.mW3 + (int64_t)j * g.CH * HSTR;
        const float *b3 = theta + y.ob3 + (int64_t)j * (2 * g.K + 1);
        const int nreal = 2 * g.K + 1;
        // CH/8 n-tiles, processed in groups of 3 to bound registers
        for (int nb = 0; nb < g.CH / 8; nb += 3) {
            float acc[2][3][4];
            zero_acc(acc);
            const int ntile = min(3, g.CH / 8 - nb);
            if (ntile == 3) warp_gemm<2, 3>(acc, sm.H2, HSTR, m0, Bt, HSTR, 8 * nb, FH);
            else if (ntile == 2) {
                float a2[2][2][4];
                zero_acc(a2);
                warp_gemm<2, 2>(a2, sm.H2, HSTR, m0, Bt, HSTR, 8 * nb, FH);
                for (int i = 0; i < 2; i++) for (int q = 0; q < 2; q++) for (int e = 0; e < 4; e++) acc[i][q][e] = a2[i][q][e];
            } else {
                float a1[2][1][4];
                zero_acc(a1);
                warp_gemm<2, 1>(a1, sm.H2, HSTR, m0, Bt, HSTR, 8 * nb, FH);
                for (int i = 0; i < 2; i++) for (int e = 0; e < 4; e++) acc[i][0][e] = a1[i][0][e];
            }
            for (int mt = 0; mt < 2; mt++)
                for (int nt = 0; nt < ntile; nt++) {
                    const int r = m0 + 16 * mt + gq, c = 8 * (nb + nt) + 2 * t;
                    const float bb0 = c < nreal ? b3[c] : 0.f, bb1 = c + 1 < nreal ? b3[c + 1] : 0.f;
                    float *o0 = sm.OUT + r * sm.ostr + jj * g.CH + c;
                    float *o1 = sm.OUT + (r + 8) * sm.ostr + jj * g.CH + c;
                    o0[0] = acc[mt][nt][0] + bb0;
                    o0[1] = acc[mt][nt][1] + bb1;
                    o1[0] = acc[mt][nt][2] + bb0;
                    o1[1] = acc[mt][nt][3] + bb1;
                }
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------- kernels
__global__ void flow_mirror_kernel(FlowGeom g, const float *__restrict__ theta,
                                   __nv_bfloat16 *__restrict__ mirror)
{
    const int l = blockIdx.y;
    const FlowLayer &y = g.ly[l];
    const int nreal = 2 * g.K + 1;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const float *W2 = theta + y.oW2;
    const float *W3 = theta + y.oW3;
    for (int64_t i = i0; i < (int64_t)FH * HSTR; i += stride) {
        const int r = (int)(i / HSTR), c = (int)(i % HSTR);
        mirror[y.mW2 + i] = __float2bfloat16(c < FH ? W2[r * FH + c] : 0.f);      // [n][k]
        mirror[y.mW2t + i] = __float2bfloat16(c < FH ? W2[c * FH + r] : 0.f);     // [k][n]
    }
    const int64_t n3 = (int64_t)y.dB * g.CH * HSTR;
    for (int64_t i = i0; i < n3; i += stride) {
        const int j = (int)(i / ((int64_t)g.CH * HSTR));
        const int rem = (int)(i % ((int64_t)g.CH * HSTR));
        const int o = rem / HSTR, k = rem % HSTR;
        const float v = (o < nreal && k < FH) ? W3[((int64_t)j * nreal + o) * FH + k] : 0.f;
        mirror[y.mW3 + i] = __float2bfloat16(v);
    }
    const int ls = g.CHK + 8;
    const int64_t n3t = (int64_t)y.dB * FH * ls;
    for (int64_t i = i0; i < n3t; i += stride) {
        const int j = (int)(i / ((int64_t)FH * ls));
        const int rem = (int)(i % ((int64_t)FH * ls));
        const int k = rem / ls, o = rem % ls;
        const float v = (o < nreal) ? W3[((int64_t)j * nreal + o) * FH + k] : 0.f;
        mirror[y.mW3t + i] = __float2bfloat16(v);
    }
    // tcgen05 operand images (K-major, 128-byte swizzle), byte-identical to
    // the shared-memory tiles the MMA reads
    for (int64_t i = i0; i < (int64_t)FH * FH; i += stride) {
        const int r = (int)(i / FH), k = (int)(i % FH);
        mirror[y.mU2 + umma::sw128_offset(FH, r, k) / 2] = __float2bfloat16(W2[r * FH + k]);
    }
    for (int64_t i = i0; i < (int64_t)y.NP * FH; i += stride) {
        const int row = (int)(i / FH), k = (int)(i % FH);
        const int j = row / g.CH, o = row % g.CH;
        const float v = (j < y.dB && o < nreal) ? W3[((int64_t)j * nreal + o) * FH + k] : 0.f;
        mirror[y.mU3 + umma::sw128_offset(y.NP, row, k) / 2] = __float2bfloat16(v);
    }
}

// Inference through all layers: DIR 0 = density (CDF, layers 0..L-1),
// DIR 1 = sampling (inverse CDF, layers L-1..0).  logdet = sum log pdf.
// When zl != nullptr (training forward) the input of every layer is stored
// to zl[l][row][dim].
template <int DIR>
__global__ void __launch_bounds__(FNT) flow_pass_kernel(FlowGeom g, const float *__restrict__ theta,
                                                       const __nv_bfloat16 *__restrict__ mirror,
                                                       int64_t n, const float *__restrict__ zin,
                                                       float *__restrict__ zout,
                                                       float *__restrict__ logdet,
                                                       float *__restrict__ zl)
{
    extern __shared__ __align__(16) unsigned char smem[];
    FlowSmem sm = flow_smem(smem, g.CH, g.CHK, 0);
    const int tid = threadIdx.x;
    const int dim = g.dim;
    const int64_t ntiles = (n + FROWS - 1) / FROWS;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t r0 = tile * FROWS;
        for (int i = tid; i < FROWS * dim; i += FNT) {
            const int r = i / dim, d = i % dim;
            sm.Z[r * FMAXD + d] = (r0 + r < n) ? zin[(r0 + r) * dim + d] : 0.5f;
        }
        if (tid < FROWS) sm.LD[tid] = 0.f;
        __syncthreads();
        for (int step = 0; step < g.L; step++) {
            const int l = DIR == 0 ? step : g.L - 1 - step;
            const FlowLayer &y = g.ly[l];
            if (zl != nullptr) {
                for (int i = tid; i < FROWS * dim; i += FNT) {
                    const int r = i / dim, d = i % dim;
                    if (r0 + r < n) zl[((int64_t)l * n + r0 + r) * dim + d] = sm.Z[r * FMAXD + d];
                }
            }
            flow_hidden(g, y, theta, mirror, sm);
            for (int j0 = 0; j0 < y.dB; j0 += 2) {
                const int nj = min(2, y.dB - j0);
                flow_out(g, y, theta, mirror, sm, j0, nj);
                const int r = tid & (FROWS - 1), jj = tid >> 7;
                if (jj < nj) {
                    float *o = sm.OUT + r * sm.ostr + jj * g.CH;
                    float Z;
                    spline_prepare(o, g.K, Z);
                    SplineState st;
                    const int col = y.B[j0 + jj];
                    const float xin = sm.Z[r * FMAXD + col];
                    float xo;
                    if (DIR == 0) xo = spline_cdf(o, g.K, Z, xin, st);
                    else xo = spline_inv(o, g.K, Z, xin, st);
                    sm.Z[r * FMAXD + col] = fminf(fmaxf(xo, 0.f), 1.f);
                    const float lp = __logf(st.pdfu) - __logf(st.Z);
                    if (jj == 0) sm.LD[r] += lp;
                    else sm.RED[r] = lp;
                }
                __syncthreads();
                if (nj == 2 && tid < FROWS) sm.LD[tid] += sm.RED[tid];
                __syncthreads();
            }
        }
        for (int i = tid; i < FROWS * dim; i += FNT) {
            const int r = i / dim, d = i % dim;
            if (r0 + r < n) zout[(r0 + r) * dim + d] = sm.Z[r * FMAXD + d];
        }
        if (tid < FROWS && r0 + tid < n) logdet[r0 + tid] = sm.LD[tid];
        __syncthreads();
    }
}

// Training backward of layer l for one tile of rows.  Inputs: zl (layer
// input), gout (dL/d layer output, rows x dim), w (loss weights).  Outputs:
// gin (dL/d layer input), the transposed bf16 activations H1^T, H2^T and
// gradients dOUT^T, dH2'^T, dH1'^T (column = row of the batch) for the
// weight-gradient GEMMs, and atomically accumulated dW1, db1, db2, db3.
__global__ void __launch_bounds__(FNT) flow_bwd_kernel(
    FlowGeom g, int l, const float *__restrict__ theta, const __nv_bfloat16 *__restrict__ mirror,
    int64_t n, int64_t ldn, const float *__restrict__ zl, const float *__restrict__ gout,
    const float *__restrict__ w, float *__restrict__ gin, __nv_bfloat16 *__restrict__ h1t,
    __nv_bfloat16 *__restrict__ h2t, __nv_bfloat16 *__restrict__ dot_, __nv_bfloat16 *__restrict__ dh2t,
    __nv_bfloat16 *__restrict__ dh1t, float *__restrict__ grad, double *__restrict__ loss)
{
    extern __shared__ __align__(16) unsigned char smem[];
    FlowSmem sm = flow_smem(smem, g.CH, g.CHK, 1);
    const FlowLayer &y = g.ly[l];
    const int tid = threadIdx.x, dim = g.dim, K = g.K;
    const int nreal = 2 * K + 1;
    const int w8 = tid >> 5, lane = tid & 31, gq = lane >> 2, t = lane & 3;
    const int64_t ntiles = ldn / FROWS;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t r0 = tile * FROWS;
        for (int i = tid; i < FROWS * dim; i += FNT) {
            const int r = i / dim, d = i % dim;
            const bool ok = r0 + r < n;
            sm.Z[r * FMAXD + d] = ok ? zl[((int64_t)l * n + r0 + r) * dim + d] : 0.5f;
            sm.G[r * FMAXD + d] = ok ? gout[(r0 + r) * dim + d] : 0.f;
        }
        if (tid < FROWS) sm.LD[tid] = (r0 + tid < n) ? -w[r0 + tid] : 0.f;   // dL/dlogpdf
        __syncthreads();
        flow_hidden(g, y, theta, mirror, sm);
        // transposed activations for dW2 = dH2'^T H1 and dW3 = dOUT^T H2
        {
            const int r = tid & (FROWS - 1), half = tid >> 7;
            for (int c = 64 * half; c < 64 * half + 64; c++) {
                h1t[(int64_t)c * ldn + r0 + r] = sm.H1[r * HSTR + c];
                h2t[(int64_t)c * ldn + r0 + r] = sm.H2[r * HSTR + c];
            }
        }
        // dH2 accumulated over the transformed coordinates: warp block 32x64
        const int m0 = 32 * (w8 & 3), n0 = 64 * (w8 >> 2);
        float dh2[2][8][4];
        zero_acc(dh2);
        // coordinates in pairs: the output GEMM of two coordinates on all 8
        // warps, their splines' backward on all 256 threads (thread = row,
        // coordinate), dL/dout left in OUT; then per coordinate dOUT (bf16)
        // -> global, db3, dH2 += dOUT_j W3_j
        for (int j0 = 0; j0 < y.dB; j0 += 2) {
            const int nj = y.dB - j0 < 2 ? y.dB - j0 : 2;
            flow_out(g, y, theta, mirror, sm, j0, nj);
            {
                const int r = tid & (FROWS - 1), half = tid >> 7;
                float lterm = 0.f;
                if (half < nj) {
                    const int j = j0 + half;
                    float *o = sm.OUT + r * sm.ostr + half * g.CH;
                    float Z;
                    spline_prepare(o, K, Z);
                    SplineState st;
                    const int col = y.B[j];
                    const float xin = sm.Z[r * FMAXD + col];
                    spline_cdf(o, K, Z, xin, st);
                    const float gC = sm.G[r * FMAXD + col];
                    const float gL = sm.LD[r];
                    lterm = (r0 + r < n) ? gL * (__logf(st.pdfu) - __logf(Z)) : 0.f;
                    const float gx = spline_backward(o, K, st, gC, gL);
                    sm.G[r * FMAXD + col] = gx;   // becomes dL/d(layer input) for B coordinates
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) lterm += __shfl_xor_sync(0xffffffffu, lterm, off);
                if ((tid & 31) == 0 && lterm != 0.f) atomicAdd(loss, (double)lterm);
            }
            __syncthreads();
            for (int jj = 0; jj < nj; jj++) {
                const int j = j0 + jj;
                // dL/dout of coordinate j as bf16
                for (int i = tid; i < FROWS * (sm.dstr / 2); i += FNT) {
                    const int r = i / (sm.dstr / 2), q = 2 * (i % (sm.dstr / 2));
                    const float *o = sm.OUT + r * sm.ostr + jj * g.CH;
                    const float v0 = q < nreal ? o[q] : 0.f, v1 = q + 1 < nreal ? o[q + 1] : 0.f;
                    *reinterpret_cast<uint32_t *>(&sm.DOB[r * sm.dstr + q]) = pack_bf16(v0, v1);
                }
                __syncthreads();
                // dOUT^T to global (rows of the transposed matrix = outputs of coordinate j)
                {
                    const int r = tid & (FROWS - 1), half = tid >> 7;
                    for (int q = half; q < nreal; q += 2)
                        dot_[((int64_t)j * nreal + q) * ldn + r0 + r] = sm.DOB[r * sm.dstr + q];
                }
                // db3 for coordinate j: column sums of dOUT, four row quarters
                // per column on all threads
                for (int i = tid; i < 4 * nreal; i += FNT) {
                    const int q = i % nreal, r0q = (i / nreal) * (FROWS / 4);
                    float sacc = 0.f;
                    for (int r = r0q; r < r0q + FROWS / 4; r++) sacc += __bfloat162float(sm.DOB[r * sm.dstr + q]);
                    atomicAdd(&grad[y.ob3 + (int64_t)j * nreal + q], sacc);
                }
                // dH2 += dOUT_j W3_j  (K = CHK outputs)
                warp_gemm<2, 8>(dh2, sm.DOB, sm.dstr, m0, mirror + y.mW3t + (int64_t)j * FH * (g.CHK + 8),
                                g.CHK + 8, n0, g.CHK);
                __syncthreads();
            }
        }
        // dH2' = dH2 * relu'(H2) -> H2 buffer (bf16) and dH2'^T to global; db2
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                const int r = m0 + 16 * mt + gq, c = n0 + 8 * nt + 2 * t;
                __nv_bfloat16 *p0 = &sm.H2[r * HSTR + c];
                __nv_bfloat16 *p1 = &sm.H2[(r + 8) * HSTR + c];
                const float a0 = __bfloat162float(p0[0]) > 0.f ? dh2[mt][nt][0] : 0.f;
                const float a1 = __bfloat162float(p0[1]) > 0.f ? dh2[mt][nt][1] : 0.f;
                const float a2 = __bfloat162float(p1[0]) > 0.f ? dh2[mt][nt][2] : 0.f;
                const float a3 = __bfloat162float(p1[1]) > 0.f ? dh2[mt][nt][3] : 0.f;
                *reinterpret_cast<uint32_t *>(p0) = pack_bf16(a0, a1);
                *reinterpret_cast<uint32_t *>(p1) = pack_bf16(a2, a3);
            }
        __syncthreads();
        {
            const int r = tid & (FROWS - 1), half = tid >> 7;
            for (int c = 64 * half; c < 64 * half + 64; c++)
                dh2t[(int64_t)c * ldn + r0 + r] = sm.H2[r * HSTR + c];
        }
        {   // db2: column sums of dH2', two row halves per column
            const int c = tid & (FH - 1), rh = (tid >> 7) * (FROWS / 2);
            float sacc = 0.f;
            for (int r = rh; r < rh + FROWS / 2; r++) sacc += __bfloat162float(sm.H2[r * HSTR + c]);
            atomicAdd(&grad[y.ob2 + c], sacc);
        }
        // dH1 = dH2' W2 ; dH1' = dH1 * relu'(H1) -> H1 buffer
        {
            float dh1[2][8][4];
            zero_acc(dh1);
            warp_gemm<2, 8>(dh1, sm.H2, HSTR, m0, mirror + y.mW2t, HSTR, n0, FH);
            __syncthreads();
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
#pragma unroll
                for (int nt = 0; nt < 8; nt++) {
                    const int r = m0 + 16 * mt + gq, c = n0 + 8 * nt + 2 * t;
                    __nv_bfloat16 *p0 = &sm.H1[r * HSTR + c];
                    __nv_bfloat16 *p1 = &sm.H1[(r + 8) * HSTR + c];
                    const float a0 = __bfloat162float(p0[0]) > 0.f ? dh1[mt][nt][0] : 0.f;
                    const float a1 = __bfloat162float(p0[1]) > 0.f ? dh1[mt][nt][1] : 0.f;
                    const float a2 = __bfloat162float(p1[0]) > 0.f ? dh1[mt][nt][2] : 0.f;
                    const float a3 = __bfloat162float(p1[1]) > 0.f ? dh1[mt][nt][3] : 0.f;
                    *reinterpret_cast<uint32_t *>(p0) = pack_bf16(a0, a1);
                    *reinterpret_cast<uint32_t *>(p1) = pack_bf16(a2, a3);
                }
        }
        __syncthreads();
        {
            const int r = tid & (FROWS - 1), half = tid >> 7;
            for (int c = 64 * half; c < 64 * half + 64; c++)
                dh1t[(int64_t)c * ldn + r0 + r] = sm.H1[r * HSTR + c];
        }
        // db1, dW1 (K = rows of the tile, FP32)
        const int dA = y.realA ? y.dA : 1;
        for (int idx = tid; idx < 2 * FH * (dA + 1); idx += FNT) {
            const int c = idx % FH, a2 = (idx / FH) % (dA + 1);   // a2 == dA -> bias
            const int rh = (idx / (FH * (dA + 1))) * (FROWS / 2);   // row half
            float sacc = 0.f;
            for (int r = rh; r < rh + FROWS / 2; r++) {
                const float d1 = __bfloat162float(sm.H1[r * HSTR + c]);
                const float xv = (a2 == dA) ? 1.f : (y.realA ? sm.Z[r * FMAXD + y.A[a2]] : 0.f);
                sacc = fmaf(d1, xv, sacc);
            }
            if (a2 == dA) atomicAdd(&grad[y.ob1 + c], sacc);
            else atomicAdd(&grad[y.oW1 + (int64_t)c * dA + a2], sacc);
        }
        // dL/dz_A += dH1' W1 (conditioning coordinates)
        if (y.realA) {   // thread (row, half): half of the hidden units, halves added in order
            const int r = tid & (FROWS - 1), hf = tid >> 7;
            const float *W1 = theta + y.oW1;
            for (int a0 = 0; a0 < y.dA; a0 += 8) {   // conditioning coordinates in chunks of 8
                const int na = y.dA - a0 < 8 ? y.dA - a0 : 8;
                float part[8];
                for (int q = 0; q < na; q++) {
                    float sacc = 0.f;
                    for (int c = 64 * hf; c < 64 * hf + 64; c++)
                        sacc = fmaf(__bfloat162float(sm.H1[r * HSTR + c]), W1[c * dA + a0 + q], sacc);
                    part[q] = sacc;
                }
                if (hf == 1)
                    for (int q = 0; q < na; q++) sm.RED[q * FROWS + r] = part[q];
                __syncthreads();
                if (hf == 0)
                    for (int q = 0; q < na; q++) sm.G[r * FMAXD + y.A[a0 + q]] += part[q] + sm.RED[q * FROWS + r];
                __syncthreads();
            }
        }
        __syncthreads();
        for (int i = tid; i < FROWS * dim; i += FNT) {
            const int r = i / dim, d = i % dim;
            if (r0 + r < n) gin[(r0 + r) * dim + d] = sm.G[r * FMAXD + d];
        }
        __syncthreads();
    }
}

// Weight gradients on the 5th-generation tensor cores: part[split][m][n] =
// sum over this CTA's K-split of A[m][k] B[n][k], A: M x ldn, B: 128 x ldn
// (bf16, K contiguous = K-major operands), one 128-row m-tile per CTA
// (blockIdx.x) and split (blockIdx.z).  Stages of 64 k are copied by the 128
// threads into the SW128 layout, double-buffered; thread 0 issues the MMAs
// (D in TMEM, 128 columns) and commits each stage to its buffer's mbarrier,
// which is waited on before the buffer is refilled.  Every wait is bounded:
// one that gives up sets g_flow_status, the MMAs are drained, TMEM is freed.
__device__ int g_flow_status;   // set to VG_ERR_TIMEOUT when a bounded wait gave up

constexpr int WGU_NT = 128;      // threads of the tcgen05 weight-gradient kernel
constexpr int WGU_KS = 64;       // k per stage (one SW128 block)

__global__ void __launch_bounds__(WGU_NT) flow_wgrad_umma_kernel(const __nv_bfloat16 *__restrict__ A,
                                                                 const __nv_bfloat16 *__restrict__ B, int M,
                                                                 int64_t ldn, int64_t kchunk,
                                                                 float *__restrict__ part)
{
    extern __shared__ uint8_t dsm[];
    __shared__ uint64_t bars[3];   // buffer 0, buffer 1, drain
    __shared__ uint32_t slot;
    __shared__ int s_ok;
    uint8_t *base = umma::align1024(dsm);
    constexpr uint32_t TILE = 128 * 128;   // bytes of a 128 x 64 bf16 tile
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.x * 128;
    const int64_t k0 = (int64_t)blockIdx.z * kchunk;
    const int64_t k1 = k0 + kchunk < ldn ? k0 + kchunk : ldn;
    const int nstage = k1 > k0 ? (int)((k1 - k0) / WGU_KS) : 0;
    if (warp == 0) umma::tmem_alloc(umma::smem_u32(&slot), 128);
    if (tid == 0) {
        for (int i = 0; i < 3; i++) umma::mbar_init(umma::smem_u32(&bars[i]), 1);
        s_ok = 1;
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = slot;
    uint32_t ph[2] = {0u, 0u};
    for (int st = 0; st < nstage; st++) {
        const int b = st & 1;
        uint8_t *sA = base + (uint32_t)b * 2u * TILE, *sB = sA + TILE;
        if (st >= 2) {   // the MMAs of stage st - 2 read this buffer
            if (tid == 0 && !umma::mbar_wait(umma::smem_u32(&bars[b]), ph[b])) s_ok = 0;
            ph[b] ^= 1u;
            __syncthreads();
            if (!s_ok) break;
        }
        const int64_t kk = k0 + (int64_t)st * WGU_KS;
        for (int i = tid; i < 128 * 8; i += WGU_NT) {
            const int r = i >> 3, c = (i & 7) * 8;
            uint4 va = make_uint4(0u, 0u, 0u, 0u);
            if (m0 + r < M) va = *reinterpret_cast<const uint4 *>(A + (int64_t)(m0 + r) * ldn + kk + c);
            *reinterpret_cast<uint4 *>(sA + umma::sw128_offset(128, r, c)) = va;
            *reinterpret_cast<uint4 *>(sB + umma::sw128_offset(128, r, c)) =
                *reinterpret_cast<const uint4 *>(B + (int64_t)r * ldn + kk + c);
        }
        umma::fence_async_smem();
        umma::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            umma::fence_after_sync();
            umma::gemm_128xN(tmem, umma::smem_u32(sA), umma::smem_u32(sB), 128, WGU_KS, 128, st > 0 ? 1u : 0u);
            umma::mma_commit(umma::smem_u32(&bars[b]));
        }
    }
    // drain: every MMA issued has completed before TMEM is read or freed
    if (tid == 0) {
        umma::mma_commit(umma::smem_u32(&bars[2]));
        if (!umma::mbar_wait(umma::smem_u32(&bars[2]), 0)) s_ok = 0;
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const bool ok = s_ok != 0;
    if (!ok && tid == 0) atomicExch(&g_flow_status, VG_ERR_TIMEOUT);
    const int m = m0 + 32 * warp + (tid & 31);
    float *P = part + (int64_t)blockIdx.z * M * 128;
    for (int c = 0; c < 128; c += 16) {
        float v[16];
        umma::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
        if (m < M) {
#pragma unroll
            for (int i = 0; i < 16; i++) P[(int64_t)m * 128 + c + i] = (ok && nstage > 0) ? v[i] : 0.f;
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (warp == 0) umma::tmem_dealloc(tmem, 128);
}

__global__ void flow_wgrad_reduce_kernel(const float *__restrict__ part, int nsplit, int64_t MN,
                                         float *__restrict__ out)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < MN;
         i += (int64_t)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int q = 0; q < nsplit; q++) s += part[(int64_t)q * MN + i];
        out[i] += s;
    }
}

__global__ void flow_adam_kernel(int64_t np, float *__restrict__ theta, const float *__restrict__ grad,
                                 float *__restrict__ m, float *__restrict__ v, float scale, float lr,
                                 float b1, float b2, float eps, float bc1, float bc2, float clip)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        float gi = grad[i] * scale;
        gi = fminf(fmaxf(gi, -clip), clip);
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        theta[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

// ------------------------------------------------- tcgen05 inference pass
// Spline of one coordinate with its 2K+1 logits in registers (compile-time
// K, fully unrolled).  DIR 0: CDF at x; DIR 1: inverse CDF at x.  Returns
// the transformed coordinate and lp = log pdf at the (input | output) point.
template <int K, int DIR>
__device__ __forceinline__ float spline_reg(float (&o)[2 * K + 1], float x, float &lp)
{
    // Written for instruction-level parallelism: every reduction runs as 4
    // independent chains; the bin search finds the block of 8 bins first,
    // then scans only that block.
    static_assert(K % 8 == 0, "K must be a multiple of 8");
    constexpr int NB = K / 8;
    constexpr float c1 = 1.f - K * EPS_W;
    float m4[4], v4[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        m4[q] = o[q];
        v4[q] = o[K + q];
    }
#pragma unroll
    for (int k = 4; k < K; k++) m4[k & 3] = fmaxf(m4[k & 3], o[k]);
#pragma unroll
    for (int k = 4; k <= K; k++) v4[k & 3] = fmaxf(v4[k & 3], o[K + k]);
    const float mx = fmaxf(fmaxf(m4[0], m4[1]), fmaxf(m4[2], m4[3]));
    const float mv = fmaxf(fmaxf(v4[0], v4[1]), fmaxf(v4[2], v4[3]));
    // exponentials as 2^(v log2 e - max log2 e): one FMA and the MUFU each;
    // the vertex heights are stored halved (exponent - 1), which absorbs the
    // trapezoid's 1/2 in the segment areas (the partial-bin formulas at the
    // end restore the factor 2)
    constexpr float L2E = 1.4426950408889634f;
    const float mxl = mx * L2E, mvl = fmaf(mv, L2E, 1.f);
    // width exponentials, summed per block of 8 bins (NB independent chains)
    float sB[NB];
#pragma unroll
    for (int b = 0; b < NB; b++) sB[b] = 0.f;
#pragma unroll
    for (int k = 0; k < K; k++) {
        o[k] = vg_ex2_approx(fmaf(o[k], L2E, -mxl));
        sB[k >> 3] += o[k];
    }
    float stot = 0.f;
#pragma unroll
    for (int b = 0; b < NB; b++) stot += sB[b];
    const float cw = __fdividef(c1, stot);
#pragma unroll
    for (int k = 0; k < K; k++) o[k] = fmaf(cw, o[k], EPS_W);   // bin widths
#pragma unroll
    for (int k = 0; k <= K; k++) o[K + k] = vg_ex2_approx(fmaf(o[K + k], L2E, -mvl));   // vertex heights / 2
    // per block: width EB = cw sum(exp) + 8 EPS_W, area PB = sum (u_k + u_k+1) W_k
    float EB[NB], PB[NB];
#pragma unroll
    for (int b = 0; b < NB; b++) {
        EB[b] = fmaf(cw, sB[b], 8.f * EPS_W);
        PB[b] = 0.f;
    }
#pragma unroll
    for (int k = 0; k < K; k++) PB[k >> 3] = fmaf(o[K + k] + o[K + k + 1], o[k], PB[k >> 3]);
    float Es[NB], Ps[NB];
    Es[0] = 0.f;
    Ps[0] = 0.f;
#pragma unroll
    for (int b = 1; b < NB; b++) {
        Es[b] = Es[b - 1] + EB[b - 1];
        Ps[b] = Ps[b - 1] + PB[b - 1];
    }
    const float Z = Ps[NB - 1] + PB[NB - 1];
    const float t = DIR == 0 ? x : x * Z;
    // two-level search: the block of 8 bins that holds t (compares of the
    // block prefixes), then a scan of that block's 8 bins, whose widths and
    // heights are selected from the NB blocks' registers once (no dynamic
    // register indexing) and whose areas are recomputed from them
    int bsel = 0;
#pragma unroll
    for (int b = 1; b < NB; b++) bsel += (DIR == 0 ? (t >= Es[b]) : (t >= Ps[b])) ? 1 : 0;
    float E = Es[0], P = Ps[0];
#pragma unroll
    for (int b = 1; b < NB; b++) {
        E = bsel == b ? Es[b] : E;
        P = bsel == b ? Ps[b] : P;
    }
    float wsel[8], usel[9];
#pragma unroll
    for (int q = 0; q < 8; q++) {
        wsel[q] = o[q];
#pragma unroll
        for (int b = 1; b < NB; b++) wsel[q] = bsel == b ? o[8 * b + q] : wsel[q];
    }
#pragma unroll
    for (int q = 0; q <= 8; q++) {
        usel[q] = o[K + q];
#pragma unroll
        for (int b = 1; b < NB; b++) usel[q] = bsel == b ? o[K + 8 * b + q] : usel[q];
    }
    float Wb = 0.f, ub = 0.f, ub1 = 0.f, Eb = 0.f, Pb = 0.f;
    bool f = false;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const float wq = wsel[q], sq = (usel[q] + usel[q + 1]) * wq;
        // the last bin of the block takes t when no earlier bin did
        const bool here = !f && (q == 7 || (DIR == 0 ? (t < E + wq) : (t < P + sq)));
        Wb = here ? wq : Wb;
        ub = here ? usel[q] : ub;
        ub1 = here ? usel[q + 1] : ub1;
        Eb = here ? E : Eb;
        Pb = here ? P : Pb;
        f = f || here;
        E += wq;
        P += sq;
    }
    // ub, ub1 are half the vertex heights: the area of the first al of the
    // bin is Wb (al 2 ub + al^2 (ub1 - ub)), the pdf 2 ((1 - al) ub + al ub1) / Z
    float al, xo;
    if (DIR == 0) {
        al = fminf(fmaxf(__fdividef(x - Eb, Wb), 0.f), 1.f);
        xo = __fdividef(Pb + Wb * al * (2.f * ub + al * (ub1 - ub)), Z);
    } else {
        const float qa = Wb * (ub1 - ub), qb = 2.f * Wb * ub;
        const float r = fmaxf(t - Pb, 0.f);
        al = __fdividef(2.f * r, fmaxf(qb + sqrtf(fmaxf(qb * qb + 4.f * qa * r, 0.f)), 1e-30f));
        al = fminf(fmaxf(al, 0.f), 1.f);
        xo = Eb + al * Wb;
    }
    const float pdfu = 2.f * ((1.f - al) * ub + al * ub1);
    lp = __logf(pdfu) - __logf(Z);
    return xo;
}


// Output biases staged in shared memory: coordinate j's 2K+1 values at
// j * bias_stride(K) floats (padded to a multiple of 4), added to the
// logits with 16-byte loads.
__host__ __device__ constexpr int bias_stride(int K) { return (2 * K + 1 + 3) / 4 * 4; }

template <int K>
__device__ __forceinline__ void add_bias(float (&o)[2 * K + 1], const float *bb)
{
    constexpr int NR = 2 * K + 1;
#pragma unroll
    for (int q = 0; q < NR; q += 4) {
        const float4 b = *reinterpret_cast<const float4 *>(bb + q);
        o[q] += b.x;
        if (q + 1 < NR) o[q + 1] += b.y;
        if (q + 2 < NR) o[q + 2] += b.z;
        if (q + 3 < NR) o[q + 3] += b.w;
    }
}

constexpr int UST_MAX = 16;      // 128-row sub-tiles per super-tile
constexpr int WG_SPLIT = 64;     // split-K chunks of the weight-gradient GEMMs
constexpr int UNT = 512;         // threads of the tcgen05 pass: 16 warps
constexpr int UNH = UNT / FROWS; // column groups of threads (4): H columns and coordinates per group
constexpr int UCOL = FH / UNH;   // H columns per thread in the epilogues (32)

struct UmmaPlan {
    int ST;                      // sub-tiles per super-tile
    int zst;                     // row stride of the state in shared memory (odd)
    size_t oW2, oW3, oA, oA2, oW1, ob1, ob2, ob3, oZ, oLD, total;
};

__host__ __device__ inline UmmaPlan umma_plan(const FlowGeom &g, int ST)
{
    UmmaPlan p;
    p.ST = ST;
    p.zst = g.dim | 1;
    size_t o = 0;
    p.oW2 = o; o += (size_t)FH * FH * 2;
    p.oW3 = o; o += (size_t)g.NPmax * FH * 2;
    p.oA = o;  o += (size_t)FH * FH * 2;
    p.oA2 = 0;   // second A buffer of the sub-tile pipeline (layers of at most UNH transformed coordinates)
    if (g.dBmax <= UNH) {
        p.oA2 = o;
        o += (size_t)FH * FH * 2;
    }
    p.oW1 = o; o += sizeof(float) * FH * 8;
    p.ob1 = o; o += sizeof(float) * FH;
    p.ob2 = o; o += sizeof(float) * FH;
    p.ob3 = o; o += sizeof(float) * 8 * bias_stride(g.K);   // dB <= 8 coordinates of 2K + 1 outputs (padded)
    p.oZ = o;  o += sizeof(float) * (size_t)ST * FROWS * p.zst;
    p.oLD = o; o += sizeof(float) * UNH * (size_t)ST * FROWS;
    p.total = o + 1024;          // + alignment slack of the dynamic base
    return p;
}

// Inference through all layers on the 5th-generation tensor cores.  One CTA
// (16 warps) per SM; a super-tile of ST x 128 rows stays in shared memory
// while the layers go by, so each layer's weights are fetched (bulk copy)
// once per super-tile.  Per 128-row sub-tile and layer:
//   H1 = relu(W1 z_A + b1)           FP32 FMA, written as the bf16 A operand
//   TMEM[0:128)   = H1 W2^T           tcgen05.mma, M=128 N=128 K=128
//   H2 = relu(TMEM + b2)              tcgen05.ld epilogue -> bf16 A operand
//   TMEM[128:...) = H2 W3[g]^T        four transformed coordinates per group
//                                     (two MMAs of two coordinates)
//   spline of each (row, coordinate)  registers; thread = (row, column
//                                     group), one spline per thread and group
// The splines (65 exponentials and a bin search each) dominate and are
// latency-bound: 16 warps, one (row, coordinate) each, hide twice the
// latency of the former 8 warps doing two each.
template <int K, int DIR>
__global__ void __launch_bounds__(UNT, 1) flow_pass_umma_kernel(FlowGeom g, const float *__restrict__ theta,
                                                               const __nv_bfloat16 *__restrict__ mirror,
                                                               int64_t n, const float *__restrict__ zin,
                                                               float *__restrict__ zout,
                                                               float *__restrict__ logdet,
                                                               float *__restrict__ zl, int ST)
{
    constexpr int NR = 2 * K + 1;
    extern __shared__ uint8_t dsm[];
    __shared__ uint64_t bars[5];   // 0 weights, 1 GEMM1, 2-3 GEMM2 buffers, 4 drain
    __shared__ uint32_t tslot;
    __shared__ int abort_flag;
    uint8_t *base = umma::align1024(dsm);
    const UmmaPlan pl = umma_plan(g, ST);
    uint8_t *sW2 = base + pl.oW2, *sW3 = base + pl.oW3, *sA = base + pl.oA;
    float *sW1 = (float *)(base + pl.oW1), *sb1 = (float *)(base + pl.ob1);
    float *sb2 = (float *)(base + pl.ob2), *sb3 = (float *)(base + pl.ob3);
    float *sZ = (float *)(base + pl.oZ), *sLD = (float *)(base + pl.oLD);
    uint8_t *sA2 = pl.oA2 ? base + pl.oA2 : nullptr;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int r = tid & (FROWS - 1), h = tid >> 7;
    const int dim = g.dim, zst = pl.zst, CH = g.CH;
    const uint32_t bar_w = umma::smem_u32(&bars[0]), bar_h = umma::smem_u32(&bars[1]);
    const uint32_t bar_o0 = umma::smem_u32(&bars[2]), bar_d = umma::smem_u32(&bars[4]);
    if (warp == 0) umma::tmem_alloc(umma::smem_u32(&tslot), 512);
    if (tid == 0) {
        for (int i = 0; i < 5; i++) umma::mbar_init(umma::smem_u32(&bars[i]), 1);
        abort_flag = 0;
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tslot;
    const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
    uint32_t ph_w = 0, ph_h = 0, ph_o0 = 0, ph_d = 0;
    const int64_t rows_per = (int64_t)ST * FROWS;
    const int64_t nsuper = (n + rows_per - 1) / rows_per;
    bool aborted = false;
    for (int64_t sup = blockIdx.x; sup < nsuper && !aborted; sup += gridDim.x) {
        const int64_t r0 = sup * rows_per;
        const int nrows = (int)((n - r0) < rows_per ? (n - r0) : rows_per);
        const int nsub = (nrows + FROWS - 1) / FROWS;
        for (int i = tid; i < nsub * FROWS * dim; i += UNT) {
            const int rr = i / dim, d = i % dim;
            sZ[rr * zst + d] = rr < nrows ? zin[(r0 + rr) * dim + d] : 0.5f;
        }
        for (int i = tid; i < nsub * FROWS; i += UNT)
#pragma unroll
            for (int q = 0; q < UNH; q++) sLD[(size_t)q * ST * FROWS + i] = 0.f;   // log-det partial of column group q
        __syncthreads();
        for (int step = 0; step < g.L && !aborted; step++) {
            const int l = DIR == 0 ? step : g.L - 1 - step;
            const FlowLayer &y = g.ly[l];
            const int dA = y.realA ? y.dA : 1;
            // weights of this layer: bf16 operand images by bulk copy, FP32 vectors by threads
            if (tid == 0) {
                const uint32_t b2 = (uint32_t)FH * FH * 2, b3 = (uint32_t)y.NP * FH * 2;
                umma::mbar_expect_tx(bar_w, b2 + b3);
                umma::bulk_g2s(umma::smem_u32(sW2), mirror + y.mU2, b2, bar_w);
                for (uint32_t off = 0; off < b3; off += 32768u) {
                    const uint32_t sz = (b3 - off) < 32768u ? (b3 - off) : 32768u;
                    umma::bulk_g2s(umma::smem_u32(sW3) + off, (const uint8_t *)(mirror + y.mU3) + off, sz, bar_w);
                }
            }
            for (int i = tid; i < FH * 8; i += UNT) {   // W1 padded to 8 columns: [128][8]
                const int c = i >> 3, a = i & 7;
                sW1[i] = a < dA ? theta[y.oW1 + c * dA + a] : 0.f;
            }
            for (int i = tid; i < FH; i += UNT) {
                sb1[i] = theta[y.ob1 + i];
                sb2[i] = theta[y.ob2 + i];
            }
            for (int i = tid; i < y.dB * NR; i += UNT) sb3[(i / NR) * bias_stride(K) + i % NR] = theta[y.ob3 + i];
            // one thread waits on the mbarrier; the others park at the CTA barrier
            if (tid == 0 && !umma::mbar_wait(bar_w, ph_w)) abort_flag = 1;
            ph_w ^= 1;
            __syncthreads();
            if (abort_flag) { aborted = true; break; }
            // ---- phases of one 128-row sub-tile (thread work; thread 0 issues the MMAs)
            auto store_zl = [&](int s) {
                if (zl == nullptr) return;
                const float *Zs = sZ + (size_t)s * FROWS * zst;
                for (int i = tid; i < FROWS * dim; i += UNT) {
                    const int rr = i / dim, d = i % dim;
                    const int64_t grow = r0 + (int64_t)s * FROWS + rr;
                    if (grow < n) zl[((int64_t)l * n + grow) * dim + d] = Zs[rr * zst + d];
                }
            };
            // H1 = relu(W1 z_A + b1) in FP32 -> A operand
            auto h1_phase = [&](int s, uint8_t *A) {
                const float *Zs = sZ + (size_t)s * FROWS * zst;
                float xa[8];
#pragma unroll
                for (int a = 0; a < 8; a++) xa[a] = (a < dA && y.realA) ? Zs[r * zst + y.A[a]] : 0.f;
                const bool wide = dA > 4;
#pragma unroll 2
                for (int c0 = UCOL * h; c0 < UCOL * h + UCOL; c0 += 8) {
                    float v[8];
                    const float4 bl = *reinterpret_cast<const float4 *>(sb1 + c0);
                    const float4 bh = *reinterpret_cast<const float4 *>(sb1 + c0 + 4);
                    v[0] = bl.x; v[1] = bl.y; v[2] = bl.z; v[3] = bl.w;
                    v[4] = bh.x; v[5] = bh.y; v[6] = bh.z; v[7] = bh.w;
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        const float4 w0 = *reinterpret_cast<const float4 *>(sW1 + (c0 + q) * 8);
                        float acc = v[q];
                        acc = fmaf(w0.x, xa[0], acc);
                        acc = fmaf(w0.y, xa[1], acc);
                        acc = fmaf(w0.z, xa[2], acc);
                        acc = fmaf(w0.w, xa[3], acc);
                        if (wide) {
                            const float4 w1 = *reinterpret_cast<const float4 *>(sW1 + (c0 + q) * 8 + 4);
                            acc = fmaf(w1.x, xa[4], acc);
                            acc = fmaf(w1.y, xa[5], acc);
                            acc = fmaf(w1.z, xa[6], acc);
                            acc = fmaf(w1.w, xa[7], acc);
                        }
                        v[q] = fmaxf(acc, 0.f);
                    }
                    uint4 pk;
                    pk.x = pack_bf16(v[0], v[1]);
                    pk.y = pack_bf16(v[2], v[3]);
                    pk.z = pack_bf16(v[4], v[5]);
                    pk.w = pack_bf16(v[6], v[7]);
                    *reinterpret_cast<uint4 *>(A + umma::sw128_offset(FH, r, c0)) = pk;
                }
            };
            // H2 epilogue: TMEM[0,128) + b2, relu -> A operand (in place of H1)
            auto h2_phase = [&](uint8_t *A) {
                for (int c0 = UCOL * h; c0 < UCOL * h + UCOL; c0 += 32) {
                    float v[32];
                    umma::tmem_ld32(tmem + lane_base + (uint32_t)c0, v);
#pragma unroll
                    for (int q8 = 0; q8 < 32; q8 += 8) {
                        uint4 pk;
                        const int c = c0 + q8;
                        const float4 bl = *reinterpret_cast<const float4 *>(sb2 + c);
                        const float4 bh = *reinterpret_cast<const float4 *>(sb2 + c + 4);
                        pk.x = pack_bf16(fmaxf(v[q8 + 0] + bl.x, 0.f), fmaxf(v[q8 + 1] + bl.y, 0.f));
                        pk.y = pack_bf16(fmaxf(v[q8 + 2] + bl.z, 0.f), fmaxf(v[q8 + 3] + bl.w, 0.f));
                        pk.z = pack_bf16(fmaxf(v[q8 + 4] + bh.x, 0.f), fmaxf(v[q8 + 5] + bh.y, 0.f));
                        pk.w = pack_bf16(fmaxf(v[q8 + 6] + bh.z, 0.f), fmaxf(v[q8 + 7] + bh.w, 0.f));
                        *reinterpret_cast<uint4 *>(A + umma::sw128_offset(FH, r, c)) = pk;
                    }
                }
            };
            // output layer of coordinate group gi (UNH coordinates, one per
            // column group of threads): two MMAs of up to two coordinates each
            // into TMEM[128, 128 + 4 CH); thread 0 only
            auto issue_out = [&](int gi, const uint8_t *A) {
#pragma unroll
                for (int p = 0; p < UNH / 2; p++) {
                    const int first = UNH * gi + 2 * p;
                    if (first >= y.dB) break;
                    const int ncoord = (first + 1 < y.dB) ? 2 : 1;
                    const int N = ncoord == 2 ? 2 * CH : (CH + 15) / 16 * 16;
                    umma::gemm_128xN(tmem + (uint32_t)(FH + 2 * p * CH), umma::smem_u32(A),
                                     umma::smem_u32(sW3) + (uint32_t)(first * CH) * 128u, N, FH, y.NP, 0);
                }
            };
            // spline of (row r, coordinate UNH gi + h) from the group's logits in TMEM
            auto spline_phase = [&](int s, int gi) {
                const int j = UNH * gi + h;
                if (j >= y.dB) return;
                float *Zs = sZ + (size_t)s * FROWS * zst;
                const uint32_t col = (uint32_t)(FH + h * CH);
                float o[NR];
                {
                    float v[32];
                    umma::tmem_ld32(tmem + lane_base + col, v);
#pragma unroll
                    for (int q = 0; q < 32; q++) o[q] = v[q];
                    if (NR > 32) {
                        umma::tmem_ld32(tmem + lane_base + col + 32u, v);
#pragma unroll
                        for (int q = 0; q < 32; q++)
                            if (32 + q < NR) o[32 + q] = v[q];
                    }
                    if (NR > 64) o[64] = umma::tmem_ld1(tmem + lane_base + col + 64u);
                }
                add_bias<K>(o, sb3 + j * bias_stride(K));
                const int cz = y.B[j];
                const float xin = Zs[r * zst + cz];
                float lp;
                const float xo = spline_reg<K, DIR>(o, xin, lp);
                Zs[r * zst + cz] = fminf(fmaxf(xo, 0.f), 1.f);
                sLD[(size_t)h * ST * FROWS + s * FROWS + r] += lp;
            };
            const int ngroups = (y.dB + UNH - 1) / UNH;
            if (sA2 != nullptr && ngroups == 1) {
                // Software pipeline over the sub-tiles (one coordinate group):
                // the tensor core runs sub-tile s+1's hidden-layer MMA during
                // sub-tile s's splines, and sub-tile s's output MMAs during
                // sub-tile s+1's H1; the two A buffers alternate.
                uint8_t *Ab[2] = {sA, sA2};
                do {
                    store_zl(0);
                    h1_phase(0, Ab[0]);
                    umma::fence_async_smem();
                    umma::fence_before_sync();
                    __syncthreads();
                    if (tid == 0) {
                        umma::fence_after_sync();
                        umma::gemm_128xN(tmem, umma::smem_u32(Ab[0]), umma::smem_u32(sW2), FH, FH, FH, 0);
                        umma::mma_commit(bar_h);
                        if (!umma::mbar_wait(bar_h, ph_h)) abort_flag = 1;
                    }
                    ph_h ^= 1;
                    __syncthreads();
                    umma::fence_after_sync();
                    if (abort_flag) { aborted = true; break; }
                    h2_phase(Ab[0]);
                    umma::fence_async_smem();
                    umma::fence_before_sync();
                    __syncthreads();
                    if (tid == 0) {
                        umma::fence_after_sync();
                        issue_out(0, Ab[0]);
                        umma::mma_commit(bar_o0);
                    }
                    for (int s = 0; s < nsub; s++) {
                        uint8_t *nxt = Ab[(s + 1) & 1];
                        const bool more = s + 1 < nsub;
                        if (more) {   // overlaps sub-tile s's output MMAs
                            store_zl(s + 1);
                            h1_phase(s + 1, nxt);
                        }
                        umma::fence_async_smem();
                        umma::fence_before_sync();
                        __syncthreads();
                        if (tid == 0) {
                            umma::fence_after_sync();
                            if (more) {
                                umma::gemm_128xN(tmem, umma::smem_u32(nxt), umma::smem_u32(sW2), FH, FH, FH, 0);
                                umma::mma_commit(bar_h);
                            }
                            if (!umma::mbar_wait(bar_o0, ph_o0)) abort_flag = 1;
                        }
                        ph_o0 ^= 1;
                        __syncthreads();
                        umma::fence_after_sync();
                        if (abort_flag) { aborted = true; break; }
                        spline_phase(s, 0);   // overlaps sub-tile s+1's hidden-layer MMA
                        umma::fence_before_sync();
                        __syncthreads();
                        if (more) {
                            if (tid == 0 && !umma::mbar_wait(bar_h, ph_h)) abort_flag = 1;
                            ph_h ^= 1;
                            __syncthreads();
                            umma::fence_after_sync();
                            if (abort_flag) { aborted = true; break; }
                            h2_phase(nxt);
                            umma::fence_async_smem();
                            umma::fence_before_sync();
                            __syncthreads();
                            if (tid == 0) {
                                umma::fence_after_sync();
                                issue_out(0, nxt);
                                umma::mma_commit(bar_o0);
                            }
                        }
                    }
                } while (0);
                if (aborted) break;
            } else {
                for (int s = 0; s < nsub; s++) {
                    store_zl(s);
                    h1_phase(s, sA);
                    umma::fence_async_smem();
                    umma::fence_before_sync();
                    __syncthreads();
                    if (tid == 0) {
                        umma::fence_after_sync();
                        umma::gemm_128xN(tmem, umma::smem_u32(sA), umma::smem_u32(sW2), FH, FH, FH, 0);
                        umma::mma_commit(bar_h);
                        if (!umma::mbar_wait(bar_h, ph_h)) abort_flag = 1;
                    }
                    ph_h ^= 1;
                    __syncthreads();
                    umma::fence_after_sync();
                    h2_phase(sA);
                    umma::fence_async_smem();
                    umma::fence_before_sync();
                    __syncthreads();
                    if (abort_flag) { aborted = true; break; }
                    for (int gi = 0; gi < ngroups; gi++) {
                        if (tid == 0) {
                            umma::fence_after_sync();
                            issue_out(gi, sA);
                            umma::mma_commit(bar_o0);
                            if (!umma::mbar_wait(bar_o0, ph_o0)) abort_flag = 1;
                        }
                        ph_o0 ^= 1;
                        __syncthreads();
                        const bool ok = abort_flag == 0;
                        umma::fence_after_sync();
                        if (ok) spline_phase(s, gi);
                        umma::fence_before_sync();
                        __syncthreads();
                        if (!ok) break;
                    }
                    if (abort_flag) { aborted = true; break; }
                }
                if (aborted) break;
            }
            __syncthreads();
        }
        if (aborted) break;
        for (int i = tid; i < nrows * dim; i += UNT) {
            const int rr = i / dim, d = i % dim;
            zout[(r0 + rr) * dim + d] = sZ[rr * zst + d];
        }
        for (int rr = tid; rr < nrows; rr += UNT) {
            float ld = 0.f;
#pragma unroll
            for (int q = 0; q < UNH; q++) ld += sLD[(size_t)q * ST * FROWS + rr];
            logdet[r0 + rr] = ld;
        }
        __syncthreads();
    }
    // drain: every MMA issued by thread 0 has completed before TMEM is freed
    if (tid == 0) {
        umma::mma_commit(bar_d);
        if (!umma::mbar_wait(bar_d, ph_d)) abort_flag = 1;
        if (aborted || abort_flag) atomicExch(&g_flow_status, VG_ERR_TIMEOUT);
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (warp == 0) umma::tmem_dealloc(tmem, 512);
}

// ------------------------------------------------ tcgen05 training backward
// Makes the compiler treat the values of o[] as redefined here (no
// instruction is emitted), so that sums of them are recomputed in the next
// pass instead of being kept live from the previous one: fewer values live
// across the backward's passes, fewer spills in a 512-thread CTA (128
// registers per thread).
template <int NRV>
__device__ __forceinline__ void regs_opaque(float (&o)[NRV])
{
#pragma unroll
    for (int q = 0; q < NRV; q++) asm volatile("" : "+f"(o[q]));
}

// Spline of one coordinate in registers (compile-time K): CDF at x (density
// direction), lp = its log pdf, and the backward of (C, log pdf) with the
// upstream gradients gC = dL/dC and gL = dL/dlp.  On exit o[] holds
// dL/dlogits; returns dL/dx.  The formulas are those of spline_prepare,
// spline_cdf and spline_backward above.
template <int K>
__device__ __forceinline__ float spline_grad_reg(float (&o)[2 * K + 1], float x, float gC, float gL, float &lp)
{
    constexpr float c1 = 1.f - K * EPS_W;
    float m4[4], v4[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        m4[q] = o[q];
        v4[q] = o[K + q];
    }
#pragma unroll
    for (int k = 4; k < K; k++) m4[k & 3] = fmaxf(m4[k & 3], o[k]);
#pragma unroll
    for (int k = 4; k <= K; k++) v4[k & 3] = fmaxf(v4[k & 3], o[K + k]);
    const float mx = fmaxf(fmaxf(m4[0], m4[1]), fmaxf(m4[2], m4[3]));
    const float mv = fmaxf(fmaxf(v4[0], v4[1]), fmaxf(v4[2], v4[3]));
    constexpr float L2E = 1.4426950408889634f;   // exponentials as 2^(v log2 e - max log2 e)
    const float mxl = mx * L2E, mvl = mv * L2E;
    float s4[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < K; k++) {
        o[k] = vg_ex2_approx(fmaf(o[k], L2E, -mxl));
        s4[k & 3] += o[k];
    }
    const float rse = 1.f / ((s4[0] + s4[1]) + (s4[2] + s4[3]));
#pragma unroll
    for (int k = 0; k < K; k++) o[k] *= rse;                               // softmax s_k
#pragma unroll
    for (int k = 0; k <= K; k++) o[K + k] = vg_ex2_approx(fmaf(o[K + k], L2E, -mvl));   // vertex heights u_k
    // bin of x with the prefix sums at it, in the CDF's sequential order
    float E = 0.f, P = 0.f, Eb = 0.f, Pb = 0.f, Wb = 1.f, ub = 0.f, ub1 = 0.f;
    int b = K - 1;
    bool f = false;
#pragma unroll
    for (int k = 0; k < K; k++) {
        const float W = EPS_W + c1 * o[k];
        const bool here = !f && (k == K - 1 || x < E + W);
        b = here ? k : b;
        Eb = here ? E : Eb;
        Pb = here ? P : Pb;
        Wb = here ? W : Wb;
        ub = here ? o[K + k] : ub;
        ub1 = here ? o[K + k + 1] : ub1;
        f = f || here;
        E += W;
        P += 0.5f * (o[K + k] + o[K + k + 1]) * W;
    }
    const float Z = P;
    regs_opaque(o);
    float al = (x - Eb) / Wb;
    al = fminf(fmaxf(al, 0.f), 1.f);
    const float du = ub1 - ub;
    const float num = Pb + Wb * (al * ub + 0.5f * al * al * du);
    const float pdfu = (1.f - al) * ub + al * ub1;
    lp = __logf(pdfu) - __logf(Z);
    const float g_num = gC / Z;
    const float g_Z = -gC * num / (Z * Z) - gL / Z;
    const float g_pdfu = gL / pdfu;
    const float g_al = g_pdfu * du + g_num * Wb * (ub + al * du);
    const float g_ub = g_pdfu * (1.f - al) + g_num * Wb * (al - 0.5f * al * al);
    const float g_ub1 = g_pdfu * al + g_num * Wb * 0.5f * al * al;
    const float g_Wb = g_num * (al * ub + 0.5f * al * al * du) - g_al * al / Wb;
    const float g_x = g_al / Wb;
    const float g_E = -g_al / Wb;
    const float hz = 0.5f * g_Z, hn = 0.5f * g_num;
    // dot = sum_k s_k c1 dL/dW_k (the softmax Jacobian)
    float d4[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < K; k++) {
        const float us = o[K + k] + o[K + k + 1];
        float gW = hz * us;
        gW += k < b ? g_E + hn * us : 0.f;
        gW += k == b ? g_Wb : 0.f;
        d4[k & 3] += o[k] * c1 * gW;
    }
    const float dot = (d4[0] + d4[1]) + (d4[2] + d4[3]);
    regs_opaque(o);
    float Wprev = 0.f;
#pragma unroll
    for (int k = 0; k <= K; k++) {
        const float Wk = k < K ? EPS_W + c1 * o[k] : 0.f;
        float gu = hz * (Wprev + Wk);
        gu += (k >= 1 && k <= b) ? hn * Wprev : 0.f;
        gu += k < b ? hn * Wk : 0.f;
        gu += k == b ? g_ub : 0.f;
        gu += k == b + 1 ? g_ub1 : 0.f;
        if (k < K) {
            const float us = o[K + k] + o[K + k + 1];
            float gW = hz * us;
            gW += k < b ? g_E + hn * us : 0.f;
            gW += k == b ? g_Wb : 0.f;
            o[k] = o[k] * (c1 * gW - dot);
        }
        o[K + k] = gu * o[K + k];
        Wprev = Wk;
    }
    return g_x;
}

// One (row, coordinate) of the backward's spline phase: logits from TMEM
// (taddr: this warp's lanes, the coordinate's first column) plus the bias
// bb, spline forward and backward, dL/dout as bf16 into row r, columns
// [c0, c0 + CH) of the K-major A-operand tile sD.  Returns (dL/dx, log pdf).
// Out of line so that its ~90 live values get the register budget of the
// 512-thread kernel to themselves: at K = 32 the function spills about 460
// bytes per thread and the kernel around it 170 (20 and 90 at K = 16),
// against 740 for the kernel with the function inlined.
template <int K>
__device__ __noinline__ float2 spline_grad_row(uint32_t taddr, const float *bb, float x, float gC, float gL,
                                               uint8_t *sD, int r, int c0)
{
    constexpr int NR = 2 * K + 1;
    constexpr int CHT = (NR + 7) / 8 * 8;
    float o[NR];
    {
        float v[32];
        umma::tmem_ld32(taddr, v);
#pragma unroll
        for (int q = 0; q < 32; q++) o[q] = v[q];
        if (NR > 32) {
            umma::tmem_ld32(taddr + 32u, v);
#pragma unroll
            for (int q = 0; q < 32; q++)
                if (32 + q < NR) o[32 + q] = v[q];
        }
        if (NR > 64) o[64] = umma::tmem_ld1(taddr + 64u);
    }
    add_bias<K>(o, bb);
    float lp;
    const float gx = spline_grad_reg<K>(o, x, gC, gL, lp);
#pragma unroll
    for (int c8 = 0; c8 < CHT; c8 += 8) {
        float a[8];
#pragma unroll
        for (int i = 0; i < 8; i++) a[i] = (c8 + i < NR) ? o[c8 + i] : 0.f;
        uint4 pk;
        pk.x = pack_bf16(a[0], a[1]);
        pk.y = pack_bf16(a[2], a[3]);
        pk.z = pack_bf16(a[4], a[5]);
        pk.w = pack_bf16(a[6], a[7]);
        *reinterpret_cast<uint4 *>(sD + umma::sw128_offset(FROWS, r, c0 + c8)) = pk;
    }
    return make_float2(gx, lp);
}

constexpr int BNT = 512;                 // threads of the tcgen05 backward: 16 warps
constexpr uint32_t BLK = FROWS * 128;    // bytes of one 64-column block of a 128-row tile (16 KB)
constexpr uint32_t TW1_COL = 448;        // TMEM columns [448, 480): dW1 | db1 accumulator

// Shared-memory plan of the tcgen05 backward (offsets from the 1024-aligned
// dynamic base).  The transformed coordinates of a layer go in groups of up
// to four (TMEM columns [128, 128 + 4 CH) hold one group's logits); W3 holds
// one group's rows of the W3 image (all of it when a layer has one group).
// RA holds, in turn: H1 | H2 (A operands of the forward recomputation),
// dL/dout of a group (A operand of dH2, NB3G blocks), dH2' | dH1' and the
// partial sums of dL/dz_A at 4 blocks.
struct BwdPlan {
    int NPG;                             // W3 rows of a group of four coordinates (4 CH, padded to 16)
    int NB3G;                            // 64-column blocks of a group's dL/dout tile
    size_t oW2, oW3, oRA, oRED, oBz, oW1, ob1, ob2, ob3, oZ, oG, oLW, total;
};

__host__ __device__ inline BwdPlan bwd_plan(const FlowGeom &g)
{
    BwdPlan p;
    const int ncg = g.dBmax < 4 ? g.dBmax : 4;
    p.NPG = (ncg * g.CH + 15) / 16 * 16;
    p.NB3G = (p.NPG + 63) / 64;
    const int zst = g.dim | 1;
    size_t o = 0;
    p.oW2 = o; o += (size_t)FH * FH * 2;
    p.oW3 = o; o += ((size_t)p.NPG * FH * 2 + 1023) / 1024 * 1024;
    p.oRA = o;
    p.oRED = o + (size_t)4 * BLK;              // dL/dz_A partials of column groups 1..3: [3][128][8] floats
    {
        const size_t a = (size_t)4 * BLK + sizeof(float) * 3 * FROWS * 8, d = (size_t)p.NB3G * BLK;
        o += ((a > d ? a : d) + 1023) / 1024 * 1024;
    }
    p.oBz = o; o += (size_t)32 * FROWS * 2;    // [z_A hi (8) | z_A lo (8) | 1 | 0...] x 128 rows, K-major
    p.oW1 = o; o += sizeof(float) * FH * 8;
    p.ob1 = o; o += sizeof(float) * FH;
    p.ob2 = o; o += sizeof(float) * FH;
    p.ob3 = o; o += sizeof(float) * g.dBmax * bias_stride(g.K);
    p.oZ = o;  o += sizeof(float) * FROWS * zst;
    p.oG = o;  o += sizeof(float) * FROWS * zst;
    p.oLW = o; o += sizeof(float) * FROWS;
    p.total = o + 1024;
    return p;
}

// Training backward of layer l on the 5th-generation tensor cores (layers
// with at most 8 transformed and 8 conditioning coordinates).  One CTA (16
// warps) per SM, persistent over 128-row tiles; the layer's W2 image is
// fetched once per CTA, its W3 image once per CTA when the layer has one
// group of (up to four) transformed coordinates, else one group's rows at a
// time (the next group's copy overlaps the recomputation of H1 and H2).
// Per tile and group g:
//   H1 = relu(W1 z_A + b1)                    FP32 FMA -> bf16 A operand
//   TMEM[T1, T1+128) = H1 W2^T                tcgen05, K-major A and B
//                                             (T1 = 0 for the first group,
//                                             128 after: [0,128) then holds
//                                             the dH2 sum)
//   H2 = relu(. + b2)                         epilogue -> bf16 A operand
//   TMEM[128,..)  = H2 W3_g^T                 the group's logits
//   spline forward + backward                 registers, thread = (row,
//                                             coordinate); dL/dout -> bf16
//   TMEM[0,128)  += dL/dout_g W3_g            B = the W3 rows read MN-major
// then, per tile:
//   dH2' = . relu'(H2)                        epilogue -> bf16 A operand
//   TMEM[128,256) = dH2' W2                   B = the W2 image read MN-major
//   dH1' = . relu'(H1)                        epilogue -> bf16; dL/dz_A
//   TMEM[448,480) += dH1'^T [z_A hi|lo|1]     dW1, db1 over the CTA's tiles
// The bf16 tiles H1, H2, dL/dout (per group) and dH2' go out by bulk copy as
// images (byte-identical to the shared-memory tiles) for
// flow_wgrad_img_kernel.  The relu masks of H1 and H2 stay in registers
// (thread = row, 32 columns).  Every wait is bounded; one that gives up
// sets g_flow_status.
template <int K>
__global__ void __launch_bounds__(BNT, 1) flow_bwd_umma_kernel(
    FlowGeom g, int l, const float *__restrict__ theta, const __nv_bfloat16 *__restrict__ mirror, int64_t n,
    int64_t ntiles, const float *__restrict__ zl, const float *__restrict__ gout, const float *__restrict__ w,
    float *__restrict__ gin, uint8_t *__restrict__ imgH1, uint8_t *__restrict__ imgH2, uint8_t *__restrict__ imgD,
    uint8_t *__restrict__ imgG2, float *__restrict__ grad, double *__restrict__ loss)
{
    constexpr int NR = 2 * K + 1;
    constexpr int CHT = (NR + 7) / 8 * 8;   // output rows per coordinate in the images (g.CH)
    extern __shared__ uint8_t dsm[];
    __shared__ uint64_t bars[2];            // 0 weights, 1 MMA completion
    __shared__ uint32_t tslot;
    __shared__ int abort_flag;
    uint8_t *base = umma::align1024(dsm);
    const BwdPlan pl = bwd_plan(g);
    const FlowLayer &y = g.ly[l];
    uint8_t *sW2 = base + pl.oW2, *sW3 = base + pl.oW3, *sRA = base + pl.oRA, *sBz = base + pl.oBz;
    uint8_t *sH1 = sRA, *sH2 = sRA + 2 * BLK, *sD = sRA, *sG2 = sRA, *sG1 = sRA + 2 * BLK;
    float *sW1 = (float *)(base + pl.oW1), *sb1 = (float *)(base + pl.ob1);
    float *sb2 = (float *)(base + pl.ob2), *sb3 = (float *)(base + pl.ob3);
    float *sZ = (float *)(base + pl.oZ), *sG = (float *)(base + pl.oG);
    float *sLW = (float *)(base + pl.oLW), *sRED = (float *)(base + pl.oRED);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int r = tid & (FROWS - 1), h = tid >> 7;
    const int dim = g.dim, zst = dim | 1;
    const int dA = y.realA ? y.dA : 1, dB = y.dB, NPl = y.NP;
    const int ngr = (dB + 3) / 4;                 // groups of transformed coordinates
    const int R3 = ngr == 1 ? NPl : pl.NPG;       // rows of the W3 tile in shared memory
    const uint32_t bar_w = umma::smem_u32(&bars[0]), bar_m = umma::smem_u32(&bars[1]);
    if (warp == 0) umma::tmem_alloc(umma::smem_u32(&tslot), 512);
    if (tid == 0) {
        umma::mbar_init(bar_w, 1);
        umma::mbar_init(bar_m, 1);
        abort_flag = 0;
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tslot;
    const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
    uint32_t ph_m = 0, ph_w = 0;
    // rows [g NPG, ...) of the W3 image (R = NPl rows, two 64-column blocks)
    // into the R3-row tile of shared memory; thread 0, completes on bar_w
    auto load_w3 = [&](int gi, uint32_t extra) {
        const int row0 = gi * pl.NPG;
        const int rows = ngr == 1 ? NPl : (NPl - row0 < pl.NPG ? NPl - row0 : pl.NPG);
        const uint32_t bytes = (uint32_t)rows * 128u;
        umma::mbar_expect_tx(bar_w, extra + 2u * bytes);
        for (int b = 0; b < 2; b++)
            for (uint32_t off = 0; off < bytes; off += 32768u)   // copies of at most 32 KB
                umma::bulk_g2s(umma::smem_u32(sW3) + (uint32_t)(b * R3) * 128u + off,
                               (const uint8_t *)(mirror + y.mU3) + ((size_t)b * NPl + row0) * 128 + off,
                               bytes - off < 32768u ? bytes - off : 32768u, bar_w);
    };
    // the layer's weights: W2 and the first group's W3 rows
    if (tid == 0) {
        const uint32_t b2 = (uint32_t)FH * FH * 2;
        load_w3(0, b2);
        umma::bulk_g2s(umma::smem_u32(sW2), mirror + y.mU2, b2, bar_w);
    }
    for (int i = tid; i < FH * 8; i += BNT) {
        const int c = i >> 3, a = i & 7;
        sW1[i] = a < dA ? theta[y.oW1 + c * dA + a] : 0.f;
    }
    for (int i = tid; i < FH; i += BNT) {
        sb1[i] = theta[y.ob1 + i];
        sb2[i] = theta[y.ob2 + i];
    }
    for (int i = tid; i < dB * NR; i += BNT) sb3[(i / NR) * bias_stride(K) + i % NR] = theta[y.ob3 + i];
    if (tid == 0 && !umma::mbar_wait(bar_w, ph_w)) abort_flag = 1;
    ph_w ^= 1;
    __syncthreads();
    int ndone = 0;
    bool w3_pending = false;   // a W3 copy in flight (thread 0's view; all threads track it alike)
    for (int64_t tile = blockIdx.x; tile < ntiles && !abort_flag; tile += gridDim.x) {
        const int64_t r0 = tile * FROWS;
        for (int i = tid; i < FROWS * dim; i += BNT) {
            const int rr = i / dim, d = i % dim;
            const bool ok = r0 + rr < n;
            sZ[rr * zst + d] = ok ? zl[((int64_t)l * n + r0 + rr) * dim + d] : 0.5f;
            sG[rr * zst + d] = ok ? gout[(r0 + rr) * dim + d] : 0.f;
        }
        if (tid < FROWS) sLW[tid] = (r0 + tid < n) ? -w[r0 + tid] : 0.f;   // dL/dlogpdf
        __syncthreads();
        uint32_t m1 = 0, m2 = 0;
        for (int gi = 0; gi < ngr; gi++) {
            const uint32_t T1 = gi == 0 ? 0u : (uint32_t)FH;   // TMEM columns of H1 W2^T
            const int nc = dB - 4 * gi < 4 ? dB - 4 * gi : 4;   // coordinates of this group
            const int Kg = (nc * CHT + 15) / 16 * 16;             // their dL/dout columns (MMA K)
            const int nbg = (Kg + 63) / 64;
            // ---- H1 (FP32) -> A operand, its relu mask; the [z_A hi | lo | 1] operand (first group)
            m1 = 0;
            m2 = 0;
            {
                float xa[8];
#pragma unroll
                for (int a = 0; a < 8; a++) xa[a] = (a < dA && y.realA) ? sZ[r * zst + y.A[a]] : 0.f;
                const bool wide = dA > 4;
#pragma unroll 2
                for (int c0 = UCOL * h; c0 < UCOL * h + UCOL; c0 += 8) {
                    float v[8];
                    const float4 bl = *reinterpret_cast<const float4 *>(sb1 + c0);
                    const float4 bh = *reinterpret_cast<const float4 *>(sb1 + c0 + 4);
                    v[0] = bl.x; v[1] = bl.y; v[2] = bl.z; v[3] = bl.w;
                    v[4] = bh.x; v[5] = bh.y; v[6] = bh.z; v[7] = bh.w;
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        const float4 w0 = *reinterpret_cast<const float4 *>(sW1 + (c0 + q) * 8);
                        float acc = v[q];
                        acc = fmaf(w0.x, xa[0], acc);
                        acc = fmaf(w0.y, xa[1], acc);
                        acc = fmaf(w0.z, xa[2], acc);
                        acc = fmaf(w0.w, xa[3], acc);
                        if (wide) {
                            const float4 w1 = *reinterpret_cast<const float4 *>(sW1 + (c0 + q) * 8 + 4);
                            acc = fmaf(w1.x, xa[4], acc);
                            acc = fmaf(w1.y, xa[5], acc);
                            acc = fmaf(w1.z, xa[6], acc);
                            acc = fmaf(w1.w, xa[7], acc);
                        }
                        m1 |= (acc > 0.f ? 1u : 0u) << (c0 - UCOL * h + q);
                        v[q] = fmaxf(acc, 0.f);
                    }
                    uint4 pk;
                    pk.x = pack_bf16(v[0], v[1]);
                    pk.y = pack_bf16(v[2], v[3]);
                    pk.z = pack_bf16(v[4], v[5]);
                    pk.w = pack_bf16(v[6], v[7]);
                    *reinterpret_cast<uint4 *>(sH1 + umma::sw128_offset(FROWS, r, c0)) = pk;
                }
                if (gi == 0) {
                    // rows 8h..8h+7 of the 32 x 128 operand: z_A hi (h = 0), z_A lo (h = 1), ones (row 16), zeros
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        const __nv_bfloat16 hi = __float2bfloat16(xa[q]);
                        const __nv_bfloat16 lo = __float2bfloat16(xa[q] - __bfloat162float(hi));
                        const __nv_bfloat16 v =
                            h == 0 ? hi : h == 1 ? lo : __float2bfloat16((h == 2 && q == 0) ? 1.f : 0.f);
                        *reinterpret_cast<__nv_bfloat16 *>(sBz + umma::sw128_offset(32, 8 * h + q, r)) = v;
                    }
                }
            }
            umma::fence_async_smem();
            umma::fence_before_sync();
            __syncthreads();
            if (tid == 0) {   // TMEM[T1, T1+128) = H1 W2^T; the H1 image out (first group)
                umma::fence_after_sync();
                umma::gemm_128xN(tmem + T1, umma::smem_u32(sH1), umma::smem_u32(sW2), FH, FH, FH, 0);
                umma::mma_commit(bar_m);
                if (gi == 0) {
                    umma::bulk_s2g(imgH1 + tile * 2 * BLK, umma::smem_u32(sH1), BLK);
                    umma::bulk_s2g(imgH1 + tile * 2 * BLK + BLK, umma::smem_u32(sH1) + BLK, BLK);
                    umma::bulk_commit();
                }
                if (!umma::mbar_wait(bar_m, ph_m)) abort_flag = 1;
            }
            ph_m ^= 1;
            __syncthreads();
            umma::fence_after_sync();
            if (abort_flag) break;
            // ---- H2 = relu(TMEM + b2) -> A operand, its relu mask
            {
                const int c0 = UCOL * h;
                float v[32];
                umma::tmem_ld32(tmem + lane_base + T1 + (uint32_t)c0, v);
#pragma unroll
                for (int q8 = 0; q8 < 32; q8 += 8) {
                    float a[8];
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        a[i] = v[q8 + i] + sb2[c0 + q8 + i];
                        m2 |= (a[i] > 0.f ? 1u : 0u) << (q8 + i);
                        a[i] = fmaxf(a[i], 0.f);
                    }
                    uint4 pk;
                    pk.x = pack_bf16(a[0], a[1]);
                    pk.y = pack_bf16(a[2], a[3]);
                    pk.z = pack_bf16(a[4], a[5]);
                    pk.w = pack_bf16(a[6], a[7]);
                    *reinterpret_cast<uint4 *>(sH2 + umma::sw128_offset(FROWS, r, c0 + q8)) = pk;
                }
            }
            umma::fence_async_smem();
            umma::fence_before_sync();
            __syncthreads();
            if (tid == 0) {   // logits of the group's coordinates (pairs); the H2 image out (first group)
                if (w3_pending && !umma::mbar_wait(bar_w, ph_w)) abort_flag = 1;
                umma::fence_after_sync();
#pragma unroll
                for (int p = 0; p < 2; p++) {
                    const int first = 2 * p;   // within the group
                    if (first >= nc) break;
                    const int N = (first + 1 < nc) ? 2 * CHT : (CHT + 15) / 16 * 16;
                    umma::gemm_128xN(tmem + (uint32_t)(FH + first * CHT), umma::smem_u32(sH2),
                                     umma::smem_u32(sW3) + (uint32_t)(first * CHT) * 128u, N, FH, R3, 0);
                }
                umma::mma_commit(bar_m);
                if (gi == 0) {
                    umma::bulk_s2g(imgH2 + tile * 2 * BLK, umma::smem_u32(sH2), BLK);
                    umma::bulk_s2g(imgH2 + tile * 2 * BLK + BLK, umma::smem_u32(sH2) + BLK, BLK);
                    umma::bulk_commit();
                }
                if (!umma::mbar_wait(bar_m, ph_m)) abort_flag = 1;
                umma::bulk_wait_read();   // H1 and H2 images read out: RA may be overwritten
            }
            if (w3_pending) ph_w ^= 1;
            w3_pending = false;
            ph_m ^= 1;
            __syncthreads();
            umma::fence_after_sync();
            if (abort_flag) break;
            // ---- spline forward + backward of (row r, coordinate 4 gi + h); dL/dout -> A operand
            {
                float lterm = 0.f;
                if (h < nc) {
                    const int j = 4 * gi + h;
                    const int cz = y.B[j];
                    const float gL = sLW[r];
                    const float2 gl = spline_grad_row<K>(tmem + lane_base + (uint32_t)(FH + h * CHT), sb3 + j * bias_stride(K),
                                                         sZ[r * zst + cz], sG[r * zst + cz], gL, sD, r, h * CHT);
                    sG[r * zst + cz] = gl.x;   // dL/d(layer input) of a transformed coordinate
                    lterm = (r0 + r < n) ? gL * gl.y : 0.f;
                } else if (h == 3) {   // fewer than 4 coordinates: zero the padding columns [nc CH, Kg)
                    for (int c8 = nc * CHT; c8 < Kg; c8 += 8)
                        *reinterpret_cast<uint4 *>(sD + umma::sw128_offset(FROWS, r, c8)) = make_uint4(0u, 0u, 0u, 0u);
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) lterm += __shfl_xor_sync(0xffffffffu, lterm, off);
                if ((tid & 31) == 0 && lterm != 0.f) atomicAdd(loss, (double)lterm);
            }
            umma::fence_async_smem();
            umma::fence_before_sync();
            __syncthreads();
            // next W3 rows: the following group of this tile, or the first group of the CTA's next tile
            const bool more = gi + 1 < ngr || (ngr > 1 && tile + gridDim.x < ntiles);
            if (tid == 0) {   // TMEM[0,128) (+)= dL/dout W3_g; the group's dL/dout image out
                umma::fence_after_sync();
                umma::gemm_128xN_ex(tmem, umma::smem_u32(sD), 0, FROWS, umma::smem_u32(sW3), 1, R3, FH, Kg,
                                    gi > 0 ? 1u : 0u);
                umma::mma_commit(bar_m);
                for (int q = 0; q < nbg; q++)
                    umma::bulk_s2g(imgD + ((tile * ngr + gi) * pl.NB3G + q) * (int64_t)BLK,
                                   umma::smem_u32(sD) + (uint32_t)q * BLK, BLK);
                umma::bulk_commit();
                if (!umma::mbar_wait(bar_m, ph_m)) abort_flag = 1;
                umma::bulk_wait_read();
                if (ngr > 1 && more && !abort_flag) load_w3(gi + 1 < ngr ? gi + 1 : 0, 0u);
            }
            if (ngr > 1 && more) w3_pending = true;
            ph_m ^= 1;
            __syncthreads();
            umma::fence_after_sync();
            if (abort_flag) break;
        }
        if (abort_flag) break;
        // ---- dH2' = dH2 relu'(H2) -> A operand
        {
            const int c0 = UCOL * h;
            float v[32];
            umma::tmem_ld32(tmem + lane_base + (uint32_t)c0, v);
#pragma unroll
            for (int q8 = 0; q8 < 32; q8 += 8) {
                float a[8];
#pragma unroll
                for (int i = 0; i < 8; i++) a[i] = ((m2 >> (q8 + i)) & 1u) ? v[q8 + i] : 0.f;
                uint4 pk;
                pk.x = pack_bf16(a[0], a[1]);
                pk.y = pack_bf16(a[2], a[3]);
                pk.z = pack_bf16(a[4], a[5]);
                pk.w = pack_bf16(a[6], a[7]);
                *reinterpret_cast<uint4 *>(sG2 + umma::sw128_offset(FROWS, r, c0 + q8)) = pk;
            }
        }
        umma::fence_async_smem();
        umma::fence_before_sync();
        __syncthreads();
        if (tid == 0) {   // TMEM[128,256) = dH2' W2; the dH2' image out
            umma::fence_after_sync();
            umma::gemm_128xN_ex(tmem + FH, umma::smem_u32(sG2), 0, FROWS, umma::smem_u32(sW2), 1, FH, FH, FH, 0);
            umma::mma_commit(bar_m);
            umma::bulk_s2g(imgG2 + tile * 2 * BLK, umma::smem_u32(sG2), BLK);
            umma::bulk_s2g(imgG2 + tile * 2 * BLK + BLK, umma::smem_u32(sG2) + BLK, BLK);
            umma::bulk_commit();
            if (!umma::mbar_wait(bar_m, ph_m)) abort_flag = 1;
        }
        ph_m ^= 1;
        __syncthreads();
        umma::fence_after_sync();
        if (abort_flag) break;
        // ---- dH1' = dH1 relu'(H1) (bf16) -> operand of dW1; dL/dz_A over this thread's 32 units
        float part[8];
#pragma unroll
        for (int a = 0; a < 8; a++) part[a] = 0.f;
        {
            const int c0 = UCOL * h;
            float v[32];
            umma::tmem_ld32(tmem + lane_base + (uint32_t)(FH + c0), v);
#pragma unroll
            for (int q = 0; q < 32; q++)
                v[q] = ((m1 >> q) & 1u) ? __bfloat162float(__float2bfloat16(v[q])) : 0.f;
#pragma unroll
            for (int q8 = 0; q8 < 32; q8 += 8) {
                uint4 pk;
                pk.x = pack_bf16(v[q8 + 0], v[q8 + 1]);
                pk.y = pack_bf16(v[q8 + 2], v[q8 + 3]);
                pk.z = pack_bf16(v[q8 + 4], v[q8 + 5]);
                pk.w = pack_bf16(v[q8 + 6], v[q8 + 7]);
                *reinterpret_cast<uint4 *>(sG1 + umma::sw128_offset(FROWS, r, c0 + q8)) = pk;
            }
            if (y.realA) {
#pragma unroll 4
                for (int q = 0; q < 32; q++) {
                    const float4 w0 = *reinterpret_cast<const float4 *>(sW1 + (c0 + q) * 8);
                    const float4 w1 = *reinterpret_cast<const float4 *>(sW1 + (c0 + q) * 8 + 4);
                    part[0] = fmaf(v[q], w0.x, part[0]);
                    part[1] = fmaf(v[q], w0.y, part[1]);
                    part[2] = fmaf(v[q], w0.z, part[2]);
                    part[3] = fmaf(v[q], w0.w, part[3]);
                    part[4] = fmaf(v[q], w1.x, part[4]);
                    part[5] = fmaf(v[q], w1.y, part[5]);
                    part[6] = fmaf(v[q], w1.z, part[6]);
                    part[7] = fmaf(v[q], w1.w, part[7]);
                }
            }
        }
        umma::fence_async_smem();
        umma::fence_before_sync();
        if (h > 0) {
            float4 *dst = reinterpret_cast<float4 *>(sRED + ((size_t)(h - 1) * FROWS + r) * 8);
            dst[0] = make_float4(part[0], part[1], part[2], part[3]);
            dst[1] = make_float4(part[4], part[5], part[6], part[7]);
        }
        __syncthreads();
        if (tid == 0) {   // TMEM[448,480) += dH1'^T [z_A hi | lo | 1] (A read MN-major)
            umma::fence_after_sync();
            umma::gemm_128xN_ex(tmem + TW1_COL, umma::smem_u32(sG1), 1, 0, umma::smem_u32(sBz), 0, 32, 32, FROWS,
                                ndone > 0 ? 1u : 0u);
            umma::mma_commit(bar_m);
        }
        if (h == 0 && y.realA) {   // dL/dz_A: the four column groups added in order
            for (int a = 0; a < dA; a++)
                sG[r * zst + y.A[a]] += ((part[a] + sRED[(0 * FROWS + r) * 8 + a]) + sRED[(1 * FROWS + r) * 8 + a]) +
                                        sRED[(2 * FROWS + r) * 8 + a];
        }
        __syncthreads();
        for (int i = tid; i < FROWS * dim; i += BNT) {
            const int rr = i / dim, d = i % dim;
            if (r0 + rr < n) gin[(r0 + rr) * dim + d] = sG[rr * zst + d];
        }
        if (tid == 0) {   // dW1 MMA done (its operands are rewritten by the next tile), dH2' image read out
            if (!umma::mbar_wait(bar_m, ph_m)) abort_flag = 1;
            umma::bulk_wait_read();
        }
        ph_m ^= 1;
        ndone++;
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
    }
    // drain every MMA and bulk copy (a W3 copy is in flight only after a
    // wait gave up), then flush the dW1 | db1 accumulator
    if (tid == 0) {
        umma::mma_commit(bar_m);
        if (!umma::mbar_wait(bar_m, ph_m)) abort_flag = 1;
        if (w3_pending && !umma::mbar_wait(bar_w, ph_w)) abort_flag = 1;
        umma::bulk_wait_all();
        if (abort_flag) atomicExch(&g_flow_status, VG_ERR_TIMEOUT);
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (!abort_flag && ndone > 0 && h == 0) {
        float v[32];
        umma::tmem_ld32(tmem + lane_base + TW1_COL, v);
        const int c = r;   // TMEM lane = hidden unit
        if (y.realA) {
#pragma unroll
            for (int a = 0; a < 8; a++)
                if (a < dA) atomicAdd(&grad[y.oW1 + (int64_t)c * dA + a], v[a] + v[8 + a]);
        }
        atomicAdd(&grad[y.ob1 + c], v[16]);
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (warp == 0) umma::tmem_dealloc(tmem, 512);
}

constexpr int WGI_NT = 128;   // threads of the image weight-gradient kernel
// floats between two splits' partials: 128 x Mtot plus 64, so that the
// reduction's loads of one element's splits are not a power of two apart
#define WGI_SPLIT_STRIDE(Mtot) ((int64_t)FH * (Mtot) + 64)

// Weight gradients from the backward's tile images.  blockIdx.y = job: 0 is
// dW2 = dH2'^T H1; c >= 1 is chunk (c-1) % NCg (rows [128 chunk, +128)) of
// coordinate group (c-1) / NCg of dW3 = dL/dout^T H2; blockIdx.x = split
// over the 128-row tiles.  A K-major
// image of a 128-row tile is the MN-major tile of its transpose with K =
// 128 rows, so both operands are read as they are: two stages by bulk copy,
// thread 0 issues the MMAs (D in TMEM[0,128)) and the row sums against a
// ones operand (the bias gradients, TMEM[128,144)).  part[split][col][Mtot],
// partb[split][Mtot] (column-major, so that the epilogue's stores coalesce;
// splits WGI_SPLIT_STRIDE floats apart).
__global__ void __launch_bounds__(WGI_NT) flow_wgrad_img_kernel(
    const uint8_t *__restrict__ imgH1, const uint8_t *__restrict__ imgH2, const uint8_t *__restrict__ imgD,
    const uint8_t *__restrict__ imgG2, int NB3G, int ngr, int NCg, int dB, int CH, int64_t ntiles, int tps,
    int Mtot, float *__restrict__ part, float *__restrict__ partb)
{
    extern __shared__ uint8_t dsm[];
    __shared__ uint64_t bars[5];   // full 0/1, empty 0/1, drain
    __shared__ uint32_t slot;
    __shared__ int s_ok;
    uint8_t *base = umma::align1024(dsm);
    uint8_t *sOnes = base;                    // 16 x 128 K-major ones (4 KB)
    uint8_t *stg = base + 4096;               // 2 stages x (A 2 blocks + B 2 blocks)
    const int tid = threadIdx.x, warp = tid >> 5;
    const int job = blockIdx.y;
    const int64_t t0 = (int64_t)blockIdx.x * tps;
    const int64_t t1 = t0 + tps < ntiles ? t0 + tps : ntiles;
    const int nst = t1 > t0 ? (int)(t1 - t0) : 0;
    // job c >= 1: the group's dL/dout tile has nbg 64-column blocks; this chunk reads two of them
    const int gq = job == 0 ? 0 : (job - 1) / NCg, cc = job == 0 ? 0 : (job - 1) % NCg;
    const int ncg = dB - 4 * gq < 4 ? dB - 4 * gq : 4;
    const int nbg = ((ncg * CH + 15) / 16 * 16 + 63) / 64;
    const int ablk0 = job == 0 ? 0 : gq * NB3G + 2 * cc;
    const int anb = job == 0 ? 2 : (nbg - 2 * cc < 2 ? nbg - 2 * cc : 2);
    const uint8_t *Asrc = job == 0 ? imgG2 : imgD;
    const int64_t astride = job == 0 ? 2 * (int64_t)BLK : (int64_t)ngr * NB3G * BLK;
    const uint8_t *Bsrc = job == 0 ? imgH1 : imgH2;
    for (int i = tid; i < 16 * FROWS; i += WGI_NT)
        *reinterpret_cast<__nv_bfloat16 *>(sOnes + umma::sw128_offset(16, i >> 7, i & 127)) = __float2bfloat16(1.f);
    umma::fence_async_smem();
    if (warp == 0) umma::tmem_alloc(umma::smem_u32(&slot), 256);
    if (tid == 0) {
        for (int i = 0; i < 5; i++) umma::mbar_init(umma::smem_u32(&bars[i]), 1);
        s_ok = 1;
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = slot;
    if (tid == 0 && anb > 0) {
        uint32_t pf[2] = {0u, 0u}, pe[2] = {0u, 0u};
        int issued = 0, used = 0;
        bool ok = true;
        auto issue = [&](int st) {
            const int b = st & 1;
            uint8_t *sA = stg + (uint32_t)b * 4u * BLK, *sB = sA + 2 * BLK;
            const int64_t t = t0 + st;
            const uint32_t fb = umma::smem_u32(&bars[b]);
            umma::mbar_expect_tx(fb, (uint32_t)(anb + 2) * BLK);
            umma::bulk_g2s(umma::smem_u32(sA), Asrc + t * astride + (int64_t)ablk0 * BLK, (uint32_t)anb * BLK, fb);
            umma::bulk_g2s(umma::smem_u32(sB), Bsrc + t * 2 * (int64_t)BLK, 2 * BLK, fb);
            issued++;
        };
        if (nst > 0) issue(0);
        if (nst > 1) issue(1);
        for (int st = 0; st < nst; st++) {
            const int b = st & 1;
            if (!umma::mbar_wait(umma::smem_u32(&bars[b]), pf[b])) { ok = false; break; }
            pf[b] ^= 1u;
            used++;
            const uint32_t sA = umma::smem_u32(stg + (uint32_t)b * 4u * BLK), sB = sA + 2 * BLK;
            umma::gemm_128xN_ex(tmem, sA, 1, 0, sB, 1, 0, FH, FROWS, st > 0 ? 1u : 0u);
            umma::gemm_128xN_ex(tmem + FH, sA, 1, 0, umma::smem_u32(sOnes), 0, 16, 16, FROWS, st > 0 ? 1u : 0u);
            umma::mma_commit(umma::smem_u32(&bars[2 + b]));
            if (st + 2 < nst) {
                if (!umma::mbar_wait(umma::smem_u32(&bars[2 + b]), pe[b])) { ok = false; break; }
                pe[b] ^= 1u;
                issue(st + 2);
            }
        }
        // loads still in flight (after a wait gave up) land before the CTA exits
        for (int s = used; s < issued; s++) {
            const int b = s & 1;
            if (!umma::mbar_wait(umma::smem_u32(&bars[b]), pf[b])) ok = false;
            pf[b] ^= 1u;
        }
        umma::mma_commit(umma::smem_u32(&bars[4]));
        if (!umma::mbar_wait(umma::smem_u32(&bars[4]), 0)) ok = false;
        if (!ok) s_ok = 0;
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const bool ok = s_ok != 0 && nst > 0 && anb > 0;
    if (s_ok == 0 && tid == 0) atomicExch(&g_flow_status, VG_ERR_TIMEOUT);
    const int m = 32 * warp + (tid & 31);
    const int mrow = job * FH + m;
    float *P = part + (int64_t)blockIdx.x * WGI_SPLIT_STRIDE(Mtot);
    for (int c = 0; c < FH; c += 32) {
        float v[32];
        umma::tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
#pragma unroll
        for (int i = 0; i < 32; i++) P[(int64_t)(c + i) * Mtot + mrow] = ok ? v[i] : 0.f;
    }
    {
        float v[16];
        umma::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)FH, v);
        partb[(int64_t)blockIdx.x * Mtot + mrow] = ok ? v[0] : 0.f;
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (warp == 0) umma::tmem_dealloc(tmem, 256);
}

// grad += the splits' sums: rows m < 128 of part are dW2 (db2), rows 128 + q
// of coordinate group q / (128 NCg) row ql = q % (128 NCg) = jl CH + o of
// the group (coordinate j = 4 group + jl: dW3 row j NR + o, db3); padding
// rows are skipped.  Four lanes per element, lane p adding splits p, p + 4, ...
// in order, the four partial sums combined in a fixed tree (deterministic).
__global__ void flow_wgrad_img_reduce_kernel(const float *__restrict__ part, const float *__restrict__ partb,
                                             int nsplit, int Mtot, int Mrows, int NCg, int64_t oW2, int64_t ob2,
                                             int64_t oW3, int64_t ob3, int dB, int CH, int NR,
                                             float *__restrict__ grad)
{
    const int64_t nw = (int64_t)FH * Mrows, ne = nw + Mrows;
    const int sub = threadIdx.x & 3;
    const int64_t e0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2;
    const int64_t estride = ((int64_t)gridDim.x * blockDim.x) >> 2;
    for (int64_t e = e0; (e & ~7LL) < ne; e += estride) {   // a warp's 8 elements (a multiple-of-8 base) move together
        const bool live = e < ne;
        const bool bias = e >= nw;
        const int m = live ? (bias ? (int)(e - nw) : (int)(e % Mrows)) : 0;
        const int c = (live && !bias) ? (int)(e / Mrows) : 0;
        const float *src = bias ? partb + m : part + (int64_t)c * Mtot + m;
        const int64_t step = bias ? (int64_t)Mtot : WGI_SPLIT_STRIDE(Mtot);
        float v[16];
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int sp = sub + 4 * q;
            v[q] = (live && sp < nsplit) ? src[(int64_t)sp * step] : 0.f;
        }
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < 16; q++) s += v[q];
        for (int sp = sub + 64; live && sp < nsplit; sp += 4) s += src[(int64_t)sp * step];
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if (!live || sub != 0) continue;
        int64_t dst;
        if (m < FH) {
            dst = bias ? ob2 + m : oW2 + (int64_t)m * FH + c;
        } else {
            const int q = m - FH, ql = q % (FH * NCg), jl = ql / CH, o = ql % CH;
            const int j = 4 * (q / (FH * NCg)) + jl;
            if (jl >= 4 || j >= dB || o >= NR) continue;
            dst = bias ? ob3 + (int64_t)j * NR + o : oW3 + ((int64_t)j * NR + o) * FH + c;
        }
        grad[dst] += s;
    }
}

// ------------------------------------------------------- training batch
// Draw m of the iteration's n samples (Philox: counter (i, step, 0, 0x7f00),
// key = seed; index = high 32 bits of word x times n), gather their z and
// form the raw weights in FP64; the block sums accumulate into scratch[m].
__global__ void train_gather_kernel(int64_t n, int64_t m, uint64_t seed, uint32_t step, int dim,
                                    const float *__restrict__ z, const float *__restrict__ f,
                                    const double *__restrict__ wgt, const int64_t *__restrict__ hc,
                                    const int32_t *__restrict__ nh, int chi2, float *__restrict__ zs,
                                    double *__restrict__ wraw)
{
    __shared__ double red[32];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double w = 0.0;
    if (i < m) {
        const VgU4 r = vg_philox((uint32_t)i, (uint32_t)(i >> 32), step, 0x7f00u, (uint32_t)seed,
                                 (uint32_t)(seed >> 32));
        const int64_t idx = (int64_t)(((uint64_t)r.x * (uint64_t)n) >> 32);
        for (int d = 0; d < dim; d++) zs[i * dim + d] = z[idx * dim + d];
        const double fw = fabs((double)f[idx]) * wgt[idx];
        w = chi2 ? fw * fw * (double)nh[hc[idx]] : fw;
        wraw[i] = w;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) w += __shfl_down_sync(0xffffffffu, w, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = w;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (threadIdx.x == 0) atomicAdd(wraw + m, v);
    }
}

// Weights normalised to mean 1 (FP32 for the backward).
__global__ void train_norm_kernel(int64_t m, const double *__restrict__ wraw, float *__restrict__ ws)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const double s = wraw[m];
    if (i < m) ws[i] = s > 0 ? (float)(wraw[i] * ((double)m / s)) : 1.f;
}

int geom_of(FlowGeom &g, const vg_flow *fl) { return make_geom(g, fl->dim, fl->nlayers, fl->K, fl->hidden); }

int set_smem(const void *kern, size_t bytes)
{
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return vg_fail(VG_ERR_CUDA, "flow smem attribute: %s", cudaGetErrorString(e));
    return VG_OK;
}

// Images and split-K partials of the tcgen05 backward for n rows: 128-row
// tiles, dL/dout blocks per tile, 128-row chunks of the W3 image, the
// weight-gradient grid (about one CTA per SM over all jobs).
struct BwdSizes {
    int64_t ntiles;
    int NB3G, NCg, ngr, Mtot, nsplit, tps;   // per coordinate group: image blocks, 128-row chunks
};

BwdSizes bwd_sizes(const FlowGeom &g, int64_t n)
{
    BwdSizes s;
    const BwdPlan pl = bwd_plan(g);
    s.ntiles = (n + FROWS - 1) / FROWS;
    s.NB3G = pl.NB3G;
    s.NCg = (pl.NPG + 127) / 128;
    s.ngr = (g.dBmax + 3) / 4;
    s.Mtot = FH * (1 + s.ngr * s.NCg);
    int64_t target = vg_num_sms() / (1 + s.ngr * s.NCg);
    if (target < 1) target = 1;
    s.tps = (int)((s.ntiles + target - 1) / target);
    if (s.tps < 1) s.tps = 1;
    s.nsplit = (int)((s.ntiles + s.tps - 1) / s.tps);
    return s;
}

// Workspace carve of the tcgen05 backward (the same order in both uses).
struct BwdWork {
    float *zl, *ga, *gb, *part, *partb, *ld, *zh;
    uint8_t *imgH1, *imgH2, *imgG2, *imgD;
    int64_t bytes;
};

BwdWork bwd_work(const FlowGeom &g, int64_t n, void *work)
{
    const BwdSizes s = bwd_sizes(g, n);
    BwdWork b;
    char *p = (char *)work;   // nullptr: sizes only
    int64_t o = 0;
    auto take = [&](int64_t bytes) {
        char *q = p != nullptr ? p + o : nullptr;
        o += (bytes + 255) & ~255LL;
        return q;
    };
    b.zl = (float *)take((int64_t)g.L * n * g.dim * 4);
    b.ga = (float *)take(n * g.dim * 4);
    b.gb = (float *)take(n * g.dim * 4);
    b.imgH1 = (uint8_t *)take(s.ntiles * 2 * (int64_t)BLK);
    b.imgH2 = (uint8_t *)take(s.ntiles * 2 * (int64_t)BLK);
    b.imgG2 = (uint8_t *)take(s.ntiles * 2 * (int64_t)BLK);
    b.imgD = (uint8_t *)take(s.ntiles * s.ngr * s.NB3G * (int64_t)BLK);
    b.part = (float *)take((int64_t)s.nsplit * WGI_SPLIT_STRIDE(s.Mtot) * 4);
    b.partb = (float *)take((int64_t)s.nsplit * s.Mtot * 4);
    b.ld = (float *)take(n * 4);
    b.zh = (float *)take(n * g.dim * 4);
    b.bytes = o;
    return b;
}

}  // namespace

// ====================================================================== ABI
extern "C" int64_t vg_flow_nparams(int dim, int nlayers, int K, int hidden)
{
    FlowGeom g;
    if (make_geom(g, dim, nlayers, K, hidden)) return -1;
    return g.nparams;
}

extern "C" int64_t vg_flow_mirror_elems(int dim, int nlayers, int K, int hidden)
{
    FlowGeom g;
    if (make_geom(g, dim, nlayers, K, hidden)) return -1;
    return g.nmirror;
}

extern "C" int64_t vg_flow_train_bytes(const vg_flow *fl, int64_t nrows)
{
    FlowGeom g;
    if (geom_of(g, fl)) return -1;
    const int64_t ldn = (nrows + FROWS - 1) / FROWS * FROWS;
    int maxP = 0;
    for (int l = 0; l < g.L; l++) maxP = g.ly[l].P > maxP ? g.ly[l].P : maxP;
    int64_t b = 0;
    b += (int64_t)g.L * nrows * g.dim * 4;        // layer inputs
    b += 2 * nrows * g.dim * 4;                   // gradient ping-pong
    b += (int64_t)FH * ldn * 2 * 4;               // h1t, h2t, dh2t, dh1t
    b += (int64_t)maxP * ldn * 2;                 // dout^T
    b += WG_SPLIT * (int64_t)(maxP > FH ? maxP : FH) * FH * 4;   // split-K partials (dW3, dW2)
    b += nrows * 4 + nrows * g.dim * 4;           // logdet + zhat scratch
    const int64_t bu = bwd_work(g, nrows, nullptr).bytes;   // the tcgen05 backward's carve
    return (bu > b ? bu : b) + 4096;
}

extern "C" int vg_flow_refresh(const vg_flow *fl, void *stream)
{
    VG_RANGE("vg_flow_refresh");
    vg_clear_error();
    FlowGeom g;
    int rc = geom_of(g, fl);
    if (rc) return rc;
    dim3 grid(64, g.L);
    flow_mirror_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(g, fl->theta, (__nv_bfloat16 *)fl->mirror);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

// tcgen05 inference pass when the configuration fits it (K in {16, 32},
// at most 8 conditioning coordinates per layer, shared memory); returns 1
// when it launched, 0 when the caller should use the mma.sync pass.
template <int K>
static int flow_pass_umma_k(const FlowGeom &g, const vg_flow *fl, int dir, int64_t n, const float *zin,
                            float *zout, float *logdet, float *zl, cudaStream_t st, int *rc)
{
    const void *k = dir == 0 ? (const void *)flow_pass_umma_kernel<K, 0> : (const void *)flow_pass_umma_kernel<K, 1>;
    // the dynamic shared memory left beside the kernel's static shared memory
    size_t stat = 0;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, k) == cudaSuccess) stat = fa.sharedSizeBytes;
    else (void)cudaGetLastError();
    const size_t limit = VG_FLOW_SMEM_MAX > stat ? VG_FLOW_SMEM_MAX - stat : 0;
    int STmax = UST_MAX;
    while (STmax > 1 && umma_plan(g, STmax).total > limit) STmax--;
    if (umma_plan(g, STmax).total > limit) return 0;   // the mma.sync pass instead
    // super-tile size: as large as shared memory allows (weights are fetched
    // once per layer and super-tile), but small enough that the static
    // round-robin over CTAs ends within one super-tile of balance
    const int64_t nsub_total = (n + FROWS - 1) / FROWS;
    const int64_t G = vg_num_sms();
    const int64_t rounds = (nsub_total + G * STmax - 1) / (G * STmax);
    int ST = (int)((nsub_total + G * rounds - 1) / (G * rounds));
    if (ST < 1) ST = 1;
    if (ST > STmax) ST = STmax;
    const UmmaPlan pl = umma_plan(g, ST);
    size_t smem = pl.total < 120 * 1024 ? 120 * 1024 : pl.total;   // one CTA per SM (TMEM: 512 columns)
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        (void)cudaGetLastError();   // not enough shared memory on this part: the mma.sync pass instead
        return 0;
    }
    const int64_t rows_per = (int64_t)ST * FROWS;
    const int64_t nsuper = (n + rows_per - 1) / rows_per;
    int64_t grid = (int64_t)vg_num_sms();
    if (grid > nsuper) grid = nsuper;
    if (dir == 0)
        flow_pass_umma_kernel<K, 0><<<(unsigned)grid, UNT, smem, st>>>(g, fl->theta, (const __nv_bfloat16 *)fl->mirror,
                                                                       n, zin, zout, logdet, zl, ST);
    else
        flow_pass_umma_kernel<K, 1><<<(unsigned)grid, UNT, smem, st>>>(g, fl->theta, (const __nv_bfloat16 *)fl->mirror,
                                                                       n, zin, zout, logdet, zl, ST);
    cudaError_t e = cudaGetLastError();
    *rc = e == cudaSuccess ? VG_OK : vg_fail(VG_ERR_CUDA, "flow umma launch: %s", cudaGetErrorString(e));
    return 1;
}

static int g_flow_force_legacy = 0;   // vg_flow_set_path(1): always use the mma.sync pass

static int flow_pass(const vg_flow *fl, int dir, int64_t n, const float *zin, float *zout,
                     float *logdet, float *zl, cudaStream_t st)
{
    FlowGeom g;
    int rc = geom_of(g, fl);
    if (rc) return rc;
    if (n <= 0) return VG_OK;
    if (!g_flow_force_legacy && g.dAmax <= 8 && g.dBmax <= 8) {
        int used = 0;
        if (g.K == 32) used = flow_pass_umma_k<32>(g, fl, dir, n, zin, zout, logdet, zl, st, &rc);
        else if (g.K == 16) used = flow_pass_umma_k<16>(g, fl, dir, n, zin, zout, logdet, zl, st, &rc);
        if (used) return rc;
    }
    const size_t sm = flow_smem_bytes(g.CH, g.CHK, 0);
    if (sm > VG_FLOW_SMEM_MAX) return vg_fail(VG_ERR_UNSUPPORTED, "flow bins %d: shared memory", g.K);
    const void *k = dir == 0 ? (const void *)flow_pass_kernel<0> : (const void *)flow_pass_kernel<1>;
    if ((rc = set_smem(k, sm))) return rc;
    const int64_t ntiles = (n + FROWS - 1) / FROWS;
    int64_t grid = (int64_t)vg_num_sms();
    if (grid > ntiles) grid = ntiles;
    if (dir == 0)
        flow_pass_kernel<0><<<(unsigned)grid, FNT, sm, st>>>(g, fl->theta, (const __nv_bfloat16 *)fl->mirror,
                                                             n, zin, zout, logdet, zl);
    else
        flow_pass_kernel<1><<<(unsigned)grid, FNT, sm, st>>>(g, fl->theta, (const __nv_bfloat16 *)fl->mirror,
                                                             n, zin, zout, logdet, zl);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

// Gradient through the tcgen05 backward when the configuration fits it (K in
// {16, 32}, at most 4 transformed and 8 conditioning coordinates per layer,
// shared memory): the training forward, then per layer (last first) the
// backward, the weight-gradient GEMMs over its images and their reduction.
// *used = 0 when the caller should use the mma.sync backward.
static int flow_grad_umma(const FlowGeom &g, const vg_flow *fl, int64_t n, const float *z, const float *w,
                          void *work, size_t work_bytes, cudaStream_t st, int *used)
{
    *used = 0;
    if (g_flow_force_legacy || (g.K != 32 && g.K != 16) || g.dBmax > 8 || g.dAmax > 8) return VG_OK;
    const void *kb = g.K == 32 ? (const void *)flow_bwd_umma_kernel<32> : (const void *)flow_bwd_umma_kernel<16>;
    size_t stat = 0;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, kb) == cudaSuccess) stat = fa.sharedSizeBytes;
    else (void)cudaGetLastError();
    const BwdPlan pl = bwd_plan(g);
    if (pl.total + stat > VG_FLOW_SMEM_MAX) return VG_OK;
    const size_t wsm = 4096 + 8 * (size_t)BLK + 1024;
    if (cudaFuncSetAttribute(kb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.total) != cudaSuccess ||
        cudaFuncSetAttribute((const void *)flow_wgrad_img_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)wsm) != cudaSuccess) {
        (void)cudaGetLastError();   // not enough shared memory on this part: the mma.sync backward instead
        return VG_OK;
    }
    *used = 1;
    const BwdSizes s = bwd_sizes(g, n);
    const BwdWork b = bwd_work(g, n, work);
    if ((int64_t)work_bytes < b.bytes) return vg_fail(VG_ERR_VALUE, "flow workspace too small");
    int rc;
    if ((rc = flow_pass(fl, 0, n, z, b.zh, b.ld, b.zl, st))) return rc;
    VG_CUDA_CHECK(cudaMemsetAsync(b.ga, 0, n * g.dim * 4, st));
    const int64_t grid = s.ntiles < vg_num_sms() ? s.ntiles : vg_num_sms();
    float *gcur = b.ga, *gnext = b.gb;
    for (int l = g.L - 1; l >= 0; l--) {
        const FlowLayer &y = g.ly[l];
        if (g.K == 32)
            flow_bwd_umma_kernel<32><<<(unsigned)grid, BNT, pl.total, st>>>(
                g, l, fl->theta, (const __nv_bfloat16 *)fl->mirror, n, s.ntiles, b.zl, gcur, w, gnext, b.imgH1,
                b.imgH2, b.imgD, b.imgG2, fl->grad, fl->loss);
        else
            flow_bwd_umma_kernel<16><<<(unsigned)grid, BNT, pl.total, st>>>(
                g, l, fl->theta, (const __nv_bfloat16 *)fl->mirror, n, s.ntiles, b.zl, gcur, w, gnext, b.imgH1,
                b.imgH2, b.imgD, b.imgG2, fl->grad, fl->loss);
        VG_LAUNCH_CHECK();
        const int ngl = (y.dB + 3) / 4, njobs = 1 + ngl * s.NCg;
        flow_wgrad_img_kernel<<<dim3((unsigned)s.nsplit, (unsigned)njobs), WGI_NT, wsm, st>>>(
            b.imgH1, b.imgH2, b.imgD, b.imgG2, s.NB3G, ngl, s.NCg, y.dB, g.CH, s.ntiles, s.tps, s.Mtot, b.part,
            b.partb);
        VG_LAUNCH_CHECK();
        flow_wgrad_img_reduce_kernel<<<1024, 256, 0, st>>>(b.part, b.partb, s.nsplit, s.Mtot, FH * njobs, s.NCg,
                                                          y.oW2, y.ob2, y.oW3, y.ob3, y.dB, g.CH, 2 * g.K + 1,
                                                          fl->grad);
        VG_LAUNCH_CHECK();
        float *tmp = gcur;
        gcur = gnext;
        gnext = tmp;
    }
    return VG_OK;
}

extern "C" int vg_flow_sample(const vg_flow *fl, int64_t n, const float *zhat, float *z,
                              float *logdet, void *stream)
{
    VG_RANGE("vg_flow_sample");
    vg_clear_error();
    return flow_pass(fl, 1, n, zhat, z, logdet, nullptr, (cudaStream_t)stream);
}

extern "C" int vg_flow_density(const vg_flow *fl, int64_t n, const float *z, float *zhat,
                               float *logdet, void *stream)
{
    VG_RANGE("vg_flow_density");
    vg_clear_error();
    return flow_pass(fl, 0, n, z, zhat, logdet, nullptr, (cudaStream_t)stream);
}

extern "C" int vg_flow_grad(const vg_flow *fl, int64_t n, const float *z, const float *w,
                            void *work, size_t work_bytes, void *stream)
{
    VG_RANGE("vg_flow_grad");
    vg_clear_error();
    FlowGeom g;
    int rc = geom_of(g, fl);
    if (rc) return rc;
    if (n <= 0) return VG_OK;
    const int64_t need = vg_flow_train_bytes(fl, n);
    if ((int64_t)work_bytes < need) return vg_fail(VG_ERR_VALUE, "flow workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    int used = 0;
    rc = flow_grad_umma(g, fl, n, z, w, work, work_bytes, st, &used);
    if (used) return rc;
    const int64_t ldn = (n + FROWS - 1) / FROWS * FROWS;
    int maxP = 0;
    for (int l = 0; l < g.L; l++) maxP = g.ly[l].P > maxP ? g.ly[l].P : maxP;
    char *p = (char *)work;
    auto take = [&](int64_t bytes) { char *q = p; p += (bytes + 255) & ~255LL; return q; };
    float *zl = (float *)take((int64_t)g.L * n * g.dim * 4);
    float *ga = (float *)take(n * g.dim * 4);
    float *gb = (float *)take(n * g.dim * 4);
    __nv_bfloat16 *h1t = (__nv_bfloat16 *)take((int64_t)FH * ldn * 2);
    __nv_bfloat16 *h2t = (__nv_bfloat16 *)take((int64_t)FH * ldn * 2);
    __nv_bfloat16 *dh2t = (__nv_bfloat16 *)take((int64_t)FH * ldn * 2);
    __nv_bfloat16 *dh1t = (__nv_bfloat16 *)take((int64_t)FH * ldn * 2);
    __nv_bfloat16 *dott = (__nv_bfloat16 *)take((int64_t)maxP * ldn * 2);
    float *part = (float *)take(WG_SPLIT * (int64_t)(maxP > FH ? maxP : FH) * FH * 4);
    float *ld = (float *)take(n * 4);
    float *zh = (float *)take(n * g.dim * 4);
    if (p > (char *)work + work_bytes) return vg_fail(VG_ERR_VALUE, "flow workspace layout");
    // forward (density direction) storing every layer's input
    if ((rc = flow_pass(fl, 0, n, z, zh, ld, zl, st))) return rc;
    VG_CUDA_CHECK(cudaMemsetAsync(ga, 0, n * g.dim * 4, st));
    const size_t smb = flow_smem_bytes(g.CH, g.CHK, 1);
    if (smb > VG_FLOW_SMEM_MAX) return vg_fail(VG_ERR_UNSUPPORTED, "flow bins %d: shared memory", g.K);
    if ((rc = set_smem((const void *)flow_bwd_kernel, smb))) return rc;
    int64_t grid = (int64_t)vg_num_sms();
    if (grid > ldn / FROWS) grid = ldn / FROWS;
    // split-K over the batch rows: at most WG_SPLIT chunks of a multiple of 64
    // rows (one tcgen05 stage), enough CTAs in flight
    const int64_t kchunk = ((ldn / WG_SPLIT) + WGU_KS - 1) / WGU_KS * WGU_KS;
    const size_t wgu_smem = 4 * 128 * 128 + 1024;   // two stages of A and B tiles + alignment
    if ((rc = set_smem((const void *)flow_wgrad_umma_kernel, wgu_smem))) return rc;
    float *gcur = ga, *gnext = gb;
    for (int l = g.L - 1; l >= 0; l--) {
        const FlowLayer &y = g.ly[l];
        flow_bwd_kernel<<<(unsigned)grid, FNT, smb, st>>>(g, l, fl->theta, (const __nv_bfloat16 *)fl->mirror,
                                                          n, ldn, zl, gcur, w, gnext, h1t, h2t, dott,
                                                          dh2t, dh1t, fl->grad, fl->loss);
        VG_LAUNCH_CHECK();
        // dW3 = dOUT^T H2  (M = P, N = hidden), dW2 = dH2'^T H1 (M = N = hidden)
        const int64_t ks = kchunk;
        const int ns = (int)((ldn + ks - 1) / ks);
        // dW3 = dOUT^T H2 and dW2 = dH2'^T H1 over the rows (split-K), on tcgen05
        flow_wgrad_umma_kernel<<<dim3((y.P + 127) / 128, 1, ns), WGU_NT, wgu_smem, st>>>(
            dott, h2t, y.P, ldn, ks, part);
        VG_LAUNCH_CHECK();
        flow_wgrad_reduce_kernel<<<256, 256, 0, st>>>(part, ns, (int64_t)y.P * FH, fl->grad + y.oW3);
        VG_LAUNCH_CHECK();
        flow_wgrad_umma_kernel<<<dim3(1, 1, ns), WGU_NT, wgu_smem, st>>>(dh2t, h1t, FH, ldn, ks, part);
        VG_LAUNCH_CHECK();
        flow_wgrad_reduce_kernel<<<256, 256, 0, st>>>(part, ns, (int64_t)FH * FH, fl->grad + y.oW2);
        VG_LAUNCH_CHECK();
        float *tmp = gcur;
        gcur = gnext;
        gnext = tmp;
    }
    return VG_OK;
}

extern "C" int vg_flow_adam(const vg_flow *fl, float scale, float lr, float beta1, float beta2,
                            float eps, int step, float clip, void *stream)
{
    VG_RANGE("vg_flow_adam");
    vg_clear_error();
    FlowGeom g;
    int rc = geom_of(g, fl);
    if (rc) return rc;
    const float bc1 = 1.f - powf(beta1, (float)step), bc2 = 1.f - powf(beta2, (float)step);
    flow_adam_kernel<<<512, 256, 0, (cudaStream_t)stream>>>(g.nparams, fl->theta, fl->grad, fl->adam_m,
                                                            fl->adam_v, scale, lr, beta1, beta2, eps,
                                                            bc1, bc2, clip);
    VG_LAUNCH_CHECK();
    return vg_flow_refresh(fl, stream);
}

extern "C" int vg_flow_set_path(int legacy)
{
    g_flow_force_legacy = legacy ? 1 : 0;
    return VG_OK;
}

extern "C" int vg_flow_status(int *status, int reset)
{
    vg_clear_error();
    int v = 0;
    VG_CUDA_CHECK(cudaMemcpyFromSymbol(&v, g_flow_status, sizeof(int)));
    if (reset) {
        const int z = 0;
        VG_CUDA_CHECK(cudaMemcpyToSymbol(g_flow_status, &z, sizeof(int)));
    }
    *status = v;
    return VG_OK;
}

extern "C" int vg_flow_train_batch(int64_t n, int64_t m, uint64_t seed, uint32_t step, int dim, const float *z,
                                   const float *f, const double *wgt, const int64_t *hc, const int32_t *neval_h,
                                   int chi2, float *zs, float *ws, double *scratch, void *stream)
{
    VG_RANGE("vg_flow_train_batch");
    vg_clear_error();
    if (n < 1 || m < 1 || n >= ((int64_t)1 << 32)) return vg_fail(VG_ERR_VALUE, "training batch sizes");
    if (dim < 1 || dim > FMAXD) return vg_fail(VG_ERR_UNSUPPORTED, "flow dim %d", dim);
    if (chi2 && (hc == nullptr || neval_h == nullptr)) return vg_fail(VG_ERR_VALUE, "chi2 weights need hc, neval_h");
    cudaStream_t st = (cudaStream_t)stream;
    VG_CUDA_CHECK(cudaMemsetAsync(scratch + m, 0, sizeof(double), st));
    const unsigned nb = (unsigned)((m + 255) / 256);
    train_gather_kernel<<<nb, 256, 0, st>>>(n, m, seed, step, dim, z, f, wgt, hc, neval_h, chi2, zs, scratch);
    VG_LAUNCH_CHECK();
    train_norm_kernel<<<nb, 256, 0, st>>>(m, scratch, ws);
    VG_LAUNCH_CHECK();
    return VG_OK;
}

extern "C" int vg_flow_zero_grad(const vg_flow *fl, void *stream)
{
    vg_clear_error();
    FlowGeom g;
    int rc = geom_of(g, fl);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    VG_CUDA_CHECK(cudaMemsetAsync(fl->grad, 0, sizeof(float) * (size_t)g.nparams, st));
    VG_CUDA_CHECK(cudaMemsetAsync(fl->loss, 0, sizeof(double), st));
    return VG_OK;
}
