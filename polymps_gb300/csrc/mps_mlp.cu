// mps_mlp.cu — learned PPE warm start on sm_103a (no reference counterpart): features of the
// new system, training, and the warm-start pipeline around the network.
//
// Per-particle MLP 16 -> 64 -> 64 -> 64 -> 1 with GELU, BF16 weights and FP32
// accumulation.  Inference runs on the fifth-generation tensor cores (tcgen05, mps_mlp_tc.cu).
// The network predicts the correction c of the temporal extrapolation
// x_e = 3 p_n - 3 p_{n-1} + p_{n-2} of the unclamped pressure on equation rows (in target
// units, de-normalised on output); the warm start is x0 = x_e + theta c with the
// residual-minimising step theta, and x0 = 0 on the identity rows of surface/dummy particles
// (their exact solution).
//
// Training uses mma.sync m16n8k16 tiles: a fused forward/backward kernel over blocks of 64
// recorded samples (one warp evaluates 16 samples; the FP32 accumulator fragment of one
// layer is re-packed in registers as the BF16 A fragment of the next; activation gradients
// on the tensor cores, weight gradients dW = dZ^T H from transposed BF16 tiles staged in
// shared memory), then an Adam kernel on the FP32 master weights that refreshes the BF16 copy.
#include <cstdio>
#include <cstring>
#include <vector>
#include <cmath>
#include "mps_common.cuh"
#include "mps_internal.h"
#include "mps_mlp.h"

#define H 64
#define NF 16
#define NNORM (2 * NF + 2)   // feature means, feature inverse spreads, target mean, target inverse spread
// parameter offsets in the packed FP32 master vector
#define OW1 0
#define OB1 (OW1 + H * NF)
#define OW2 (OB1 + H)
#define OB2 (OW2 + H * H)
#define OW3 (OB2 + H)
#define OB3 (OW3 + H * H)
#define OW4 (OB3 + H)
#define OB4 (OW4 + H)
#define NPARAM (OB4 + 1)
static_assert(NPARAM == MPSGPU_MLP_NPARAM, "parameter packing");
// BF16 weight copy offsets
#define BW1 0
#define BW2 (BW1 + H * NF)
#define BW3 (BW2 + H * H)
#define BW4 (BW3 + H * H)
#define NBF (BW4 + H)
// padded shared-memory row strides (bank-conflict-free fragment loads)
#define S1 24
#define S2 72

#include "mps_gelu.cuh"
#include "mps_mlp_feat.cuh"

// d gelu / dx = (1 + t)/2 + x/2 (1 - t^2) (k0 + 3 k0 k1 x^2), t = tanh(u) as gelu forms it
__device__ __forceinline__ float gelud(float x) {
    const float x2 = x * x;
    const float t = tanhHw(x * fmaf(GELU_K01, x2, GELU_K0));
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * fmaf(3.0f * GELU_K01, x2, GELU_K0);
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *(uint32_t*)&v;
}

__device__ __forceinline__ void mma16816(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

struct SmemW {
    __nv_bfloat16 w1[H * S1];
    __nv_bfloat16 w2[H * S2];
    __nv_bfloat16 w3[H * S2];
    float w4[H];
    float b1[H], b2[H], b3[H];
    float b4;
    float mean[NF], istd[NF];
};

__device__ void loadWeights(SmemW& s, const __nv_bfloat16* wbf, const float* master, const float* norm) {
    for (int k = threadIdx.x; k < H * NF; k += blockDim.x) s.w1[(k / NF) * S1 + (k % NF)] = wbf[BW1 + k];
    for (int k = threadIdx.x; k < H * H; k += blockDim.x) {
        s.w2[(k / H) * S2 + (k % H)] = wbf[BW2 + k];
        s.w3[(k / H) * S2 + (k % H)] = wbf[BW3 + k];
    }
    for (int k = threadIdx.x; k < H; k += blockDim.x) {
        s.w4[k] = __bfloat162float(wbf[BW4 + k]);
        s.b1[k] = master[OB1 + k]; s.b2[k] = master[OB2 + k]; s.b3[k] = master[OB3 + k];
    }
    for (int k = threadIdx.x; k < NF; k += blockDim.x) { s.mean[k] = norm[k]; s.istd[k] = norm[NF + k]; }
    if (threadIdx.x == 0) s.b4 = master[OB4];
}

// A fragment of 16 samples x 16 normalised features (rows g and g+8 of the tile); q scales
// the pressure-difference features 1, 5, 7 and 14 (1/sigma for raw features, 1 otherwise)
__device__ __forceinline__ float fin(const SmemW& s, const float* f, int c, float q) {
    float v = f[c];
    if (c == 1 || c == 5 || c == 7 || c == 14) v *= q;
    return (v - s.mean[c]) * s.istd[c];
}
__device__ __forceinline__ void loadInput(const SmemW& s, const float* f0, const float* f1, uint32_t* a, float q = 1.f) {
    int t = threadIdx.x & 3;
    int c0 = 2 * t, c1 = 2 * t + 8;
    a[0] = pack2(fin(s, f0, c0, q), fin(s, f0, c0 + 1, q));
    a[1] = pack2(fin(s, f1, c0, q), fin(s, f1, c0 + 1, q));
    a[2] = pack2(fin(s, f0, c1, q), fin(s, f0, c1 + 1, q));
    a[3] = pack2(fin(s, f1, c1, q), fin(s, f1, c1 + 1, q));
}

// z[8][4] = A(16 x K) W^T + b, W row-major [64][K] in smem with stride S
template <int KCH, int S>
__device__ __forceinline__ void layer(const uint32_t (*a)[4], const __nv_bfloat16* w, const float* b, float (*z)[4]) {
    int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        float b0 = b[8 * j + 2 * t], b1 = b[8 * j + 2 * t + 1];
        z[j][0] = b0; z[j][1] = b1; z[j][2] = b0; z[j][3] = b1;
#pragma unroll
        for (int kc = 0; kc < KCH; kc++) {
            const __nv_bfloat16* row = w + (8 * j + g) * S + 16 * kc + 2 * t;
            mma16816(z[j], a[kc], *(const uint32_t*)row, *(const uint32_t*)(row + 8));
        }
    }
}
// h = gelu(z), re-packed as 4 BF16 A fragments
__device__ __forceinline__ void activate(const float (*z)[4], uint32_t (*a)[4]) {
#pragma unroll
    for (int kc = 0; kc < 4; kc++) {
        a[kc][0] = pack2(gelu(z[2 * kc][0]), gelu(z[2 * kc][1]));
        a[kc][1] = pack2(gelu(z[2 * kc][2]), gelu(z[2 * kc][3]));
        a[kc][2] = pack2(gelu(z[2 * kc + 1][0]), gelu(z[2 * kc + 1][1]));
        a[kc][3] = pack2(gelu(z[2 * kc + 1][2]), gelu(z[2 * kc + 1][3]));
    }
}
// last layer: rows g and g+8 -> out (quad reduction)
__device__ __forceinline__ void headOut(const SmemW& s, const float (*z)[4], float& o0, float& o1) {
    int t = threadIdx.x & 3;
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        int c = 8 * j + 2 * t;
        s0 += gelu(z[j][0]) * s.w4[c] + gelu(z[j][1]) * s.w4[c + 1];
        s1 += gelu(z[j][2]) * s.w4[c] + gelu(z[j][3]) * s.w4[c + 1];
    }
    s0 += __shfl_xor_sync(0xffffffffu, s0, 1); s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 1); s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
    o0 = s0 + s.b4; o1 = s1 + s.b4;
}

// ------------------------------------------------------------------ features
// The network corrects the temporal extrapolation of the unclamped solutions,
// x_e = 3 p_n - 3 p_{n-1} + p_{n-2}: x0 = x_e + correction on the rows that carry an equation.
// Raw features of row i of the new system (normalised inside the network); pressures in
// Pa (1, 5, 7 and 14 then in units of the system scale sigma below), lengths in m,
// velocities in m/s:
//  0 (n_i - n0)/n0          1 b_i / A_ii              2 numNeigh / N0
//  3 row without pressure last solve (p_n == 0)       4 wall distance / reL (<= 1.5)
//  5 p_n - p_{n-1}          6 x_e                     7 (b - A x_e)_i / A_ii (Jacobi step)
//  8 p_n                    9 |v|                    10 v along -g
// 11 A_ii / (coeffPPE n0)  12 wall PND               13 height along -g
// 14 (b_i - b_i of the last solve) / A_ii            15 (pndi - pndki)/n0
__device__ __forceinline__ double extrapBase(const Dev& d, int j) {
    return 3.0 * (d.pressPPE[j] - d.pressPPEprev[j]) + d.pressPPEprev2[j];
}
// Block sums of two FP64 values per thread into part[block] and part[gridDim + block].
__device__ __forceinline__ void blockPartials2(double s0, double s1, double* part) {
    __shared__ double sm[2][32];
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    if ((threadIdx.x & 31) == 0) { sm[0][threadIdx.x >> 5] = s0; sm[1][threadIdx.x >> 5] = s1; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) { a += sm[0][k]; b += sm[1][k]; }
        part[blockIdx.x] = a;
        part[gridDim.x + blockIdx.x] = b;
    }
}
// Totals of nblk block partials (fixed order for a fixed block size), in every thread.
__device__ __forceinline__ void sumPartials2(const double* part, int nblk, double& a, double& b) {
    __shared__ double sm[2][32];
    double s0 = 0.0, s1 = 0.0;
    for (int k = threadIdx.x; k < nblk; k += blockDim.x) { s0 += part[k]; s1 += part[nblk + k]; }
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    if ((threadIdx.x & 31) == 0) { sm[0][threadIdx.x >> 5] = s0; sm[1][threadIdx.x >> 5] = s1; }
    __syncthreads();
    a = 0.0; b = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) { a += sm[0][k]; b += sm[1][k]; }
    __syncthreads();
}

// Features 1, 5, 7 and 14 (pressure differences, Pa) and the target are taken in units of
// the system scale sigma = RMS of feature 7 over the equation rows: their spread shrinks
// with the particle spacing, in units of sigma it does not, so a network trained at one
// spacing applies at another.  The features kernel leaves block partials of sum f7^2 and
// of the row count; sigma is formed once from them, and the network input, the recorded
// samples and the correction apply it.
#define FSIG 7
// x_e in FP32 for the neighbour gathers of the features (the features are FP32 numbers;
// GB300 runs FP64 at 1/64 of the FP32 rate, so the per-entry work stays in FP32)
__global__ void k_mlp_xe32(Dev d, float* xe32) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N0) return;
    xe32[i] = (i < liveN(d) && d.bc[i] == d.P.inner) ? (float)extrapBase(d, i) : 0.f;
}
// The FP64 start x = x_e on equation rows (0 on identity rows) written for the solver
__global__ void k_mlp_xe_start(Dev d, PpeBuffers B) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N0) return;
    const bool eq = i < liveN(d) && d.bc[i] == d.P.inner;
    B.x[i] = eq ? extrapBase(d, i) : 0.0;
}
// FP64 residual r_e = b - A x_e of that start into the solver's residual vector, one row per
// thread at full occupancy (the same row product, in the same order, as the solver's own
// residual passes): the features read it, and the solver's set-up takes it as its first
// residual instead of forming it again
__global__ void __launch_bounds__(256) k_mlp_resid64(Dev d, PpeBuffers B) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    B.r[i] = B.b[i] - ellRow<double, true>(B.diag, B.val, B.col, B.x, i, __ldg(B.rowLen + i), ellBase(B, i), B.ellStride);
}
// r_e = b - A x_e (FP32 copy of the matrix) for the features and the step: one row per
// thread, eight entries in flight with the next chunk's lines prefetched (ellRow)
__global__ void __launch_bounds__(256) k_mlp_resid(Dev d, PpeBuffers B, const float* xe32, float* re) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    re[i] = (float)B.b[i] - ellRow<float, true>(B.diagf, B.valf, B.col, xe32, i, __ldg(B.rowLen + i), ellBase(B, i), B.ellStride);
}
static_assert(NF == MLP_NF && FSIG == MLP_FSIG, "feature layout");
static FeatConst featConst(const MpsParams& P) {
    double gx = P.gravity[0], gy = P.gravity[1], gz = P.gravity[2];
    const double gn = std::sqrt(gx * gx + gy * gy + gz * gz);
    if (gn > 0) { gx /= gn; gy /= gn; gz /= gn; }
    FeatConst k;
    k.ggx = (float)gx; k.ggy = (float)gy; k.ggz = (float)gz;
    k.in0 = (float)(1.0 / P.pndSmallZero);
    k.iN0 = (float)(1.0 / P.numNeighZero);
    k.iRe = (float)(1.0 / P.reL);
    k.iA = (float)(1.0 / (P.coeffPPE * P.pndSmallZero));
    return k;
}
// The 16 raw features of the row from the FP64 start and its residual (k_mlp_xe_start,
// k_mlp_resid64; featRow64) and the block partials of the system scale (sum over equation
// rows of feature 7 squared, and their count): one memory-bound pass over the rows' fields,
// so the tensor-core forward only streams the feature rows.
__global__ void __launch_bounds__(256) k_mlp_feat64(Dev d, PpeBuffers B, float* feat, double* part, FeatConst K) {
    const int n = liveN(d);
    double q0 = 0.0, q1 = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float f[NF];
        featRow64(d, B, i, K, f);
        float4* o = (float4*)(feat + (size_t)i * NF);
        o[0] = make_float4(f[0], f[1], f[2], f[3]);
        o[1] = make_float4(f[4], f[5], f[6], f[7]);
        o[2] = make_float4(f[8], f[9], f[10], f[11]);
        o[3] = make_float4(f[12], f[13], f[14], f[15]);
        if (d.bc[i] == d.P.inner) { q0 += f2dExact(f[FSIG] * f[FSIG]); q1 += 1.0; }
    }
    blockPartials2(q0, q1, part);
}
__global__ void __launch_bounds__(256) k_mlp_features(Dev d, PpeBuffers B, const float* xe32, const float* re,
                                                      float* feat, double* part, FeatConst K) {
    const MpsParams& P = d.P;
    const float ggx = K.ggx, ggy = K.ggy, ggz = K.ggz, in0 = K.in0, iN0 = K.iN0, iRe = K.iRe, iA = K.iA;
    const int n = liveN(d);
    double q0 = 0.0, q1 = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const dvec4 x = d.pos[i], v = d.vel[i];
        const float diag = (float)B.diag[i], idg = 1.f / diag;
        const float pn = (float)d.pressPPE[i], pp = (float)d.pressPPEprev[i];
        const bool eq = d.bc[i] == P.inner;
        const float xe = xe32[i];
        const float bi = (float)B.b[i];
        const float rei = re[i];   // b_i - (A x_e)_i
        const float vx = (float)v.x, vy = (float)v.y, vz = (float)v.z;
        float f[NF];
        f[0] = ((float)d.pndSmall[i] - (float)P.pndSmallZero) * in0;
        f[1] = bi * idg;
        f[2] = (float)d.numNeigh[i] * iN0;
        f[3] = (d.pressPPE[i] == 0.0) ? 1.f : 0.f;
        f[4] = fminf(sqrtf((float)d.riw2[i]) * iRe, 1.5f);
        f[5] = pn - pp;
        f[6] = xe;
        f[7] = rei * idg;
        f[8] = pn;
        f[9] = sqrtf(vx * vx + vy * vy + vz * vz);
        f[10] = -(vx * ggx + vy * ggy + vz * ggz);
        f[11] = diag * iA;
        f[12] = (float)d.pndWall[i];
        f[13] = -((float)x.x * ggx + (float)x.y * ggy + (float)x.z * ggz);
        f[14] = (bi - (float)d.source[i]) * idg;
        f[15] = ((float)d.pndi[i] - (float)d.pndki[i]) * in0;
        float4* o = (float4*)(feat + (size_t)i * NF);
        o[0] = make_float4(f[0], f[1], f[2], f[3]);
        o[1] = make_float4(f[4], f[5], f[6], f[7]);
        o[2] = make_float4(f[8], f[9], f[10], f[11]);
        o[3] = make_float4(f[12], f[13], f[14], f[15]);
        if (eq) { q0 += (double)(f[FSIG] * f[FSIG]); q1 += 1.0; }
    }
    blockPartials2(q0, q1, part);
}
__global__ void __launch_bounds__(256) k_mlp_sig(const double* part, int nblk, double* sig) {
    double a, b;
    sumPartials2(part, nblk, a, b);
    if (threadIdx.x == 0) sig[0] = (b > 0.0 && a > 0.0) ? sqrt(a / b) : 1.0;
}
static void mlpFeatureLaunch(MlpState& m, const Dev& d, const PpeBuffers& B, cudaStream_t s) {
    k_mlp_xe32<<<gridFor(d.N0, 256), 256, 0, s>>>(d, m.xe32);
    k_mlp_resid<<<gridFor(d.N0, 256), 256, 0, s>>>(d, B, m.xe32, m.re);
    k_mlp_features<<<m.nblk, 256, 0, s>>>(d, B, m.xe32, m.re, m.feat, m.part, featConst(d.P));
    k_mlp_sig<<<1, 256, 0, s>>>(m.part, m.nblk, m.sig);
}

// The network's correction c = out / target_inv_std + target_mean of the extrapolation
// x_e on equation rows (identity rows: x = 0).  The start is x0 = x_e + theta c with the
// step theta = (r_e . A c) / (A c . A c) that minimises ||b - A x0||: a pointwise
// prediction error is rough, and A amplifies rough errors, so the full step can leave a
// larger residual than x_e even when it lowers the error; with the minimising step the
// start is never worse than the extrapolation (theta = 0) in the residual norm.
__global__ void k_mlp_combine(Dev d, PpeBuffers B, const float* out, const float* norm, const double* sig,
                              float* cdir) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N0) return;
    const bool eq = i < liveN(d) && d.bc[i] == d.P.inner;
    B.x[i] = eq ? extrapBase(d, i) : 0.0;
    cdir[i] = eq ? (out[i] / norm[2 * NF + 1] + norm[2 * NF]) * (float)sig[0] : 0.f;
}
__global__ void __launch_bounds__(256) k_mlp_step_dots(Dev d, PpeBuffers B, const float* cdir, const float* re,
                                                       double* part) {
    double s0 = 0.0, s1 = 0.0;
    const int n = liveN(d);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float ac = ellRow<float, true>(B.diagf, B.valf, B.col, cdir, i, __ldg(B.rowLen + i), ellBase(B, i), B.ellStride);
        s0 += (double)(re[i] * ac);
        s1 += (double)(ac * ac);
    }
    blockPartials2(s0, s1, part);
}
// theta from the block partials (one block, fixed order), then x0 += theta c
__global__ void __launch_bounds__(256) k_mlp_theta(const double* part, int nblk, double* theta) {
    double a, b;
    sumPartials2(part, nblk, a, b);
    // a non-finite correction (or product) keeps the extrapolated start: theta = 0
    if (threadIdx.x == 0) theta[0] = (b > 0.0 && b < 1.0 / 0.0 && a == a && fabs(a) < 1.0 / 0.0) ? a / b : 0.0;
}
__global__ void k_mlp_step_apply(Dev d, PpeBuffers B, const float* cdir, const double* theta) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.N0 && theta[0] != 0.0) B.x[i] += theta[0] * (double)cdir[i];   // (0 * NaN would poison x)
}

// ------------------------------------------------------------------ learned start
// q = A c (FP32 copy of the matrix) for the residual-minimising step the solver takes
__global__ void __launch_bounds__(256) k_mlp_ac(Dev d, PpeBuffers B, const float* cdir, float* q) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    q[i] = ellRow<float, true>(B.diagf, B.valf, B.col, cdir, i, __ldg(B.rowLen + i), ellBase(B, i), B.ellStride);
}

// sig: system scale of the raw features (nullptr: the features are network inputs as given)
static int mlpForwardLaunch(MlpState& m, const float* feat, int n, const double* sig, float* out, cudaStream_t s) {
    return mlpForwardTc(m, feat, n, nullptr, nullptr, 0, sig, out, s);
}

int mlpWarmStart(MlpState& m, const Dev& d, const PpeBuffers& B, cudaStream_t s, bool stepInSolver) {
    if (!m.ready) return MPSGPU_ERR_ARG;
    if (stepInSolver) {
        // x = x_e, its FP64 residual r_e (left in the solver's residual vector), the features
        // and the scale's partials, the scale, the network's correction c, and q = A c; the
        // residual-minimising step x_e + theta c is taken by the solver's set-up pass, which
        // starts from r_e (q in m.re)
        k_mlp_xe_start<<<gridFor(d.N0, 256), 256, 0, s>>>(d, B);
        k_mlp_resid64<<<gridFor(d.N0, 256), 256, 0, s>>>(d, B);
        k_mlp_feat64<<<m.nblkFeat, 256, 0, s>>>(d, B, m.feat, m.part, featConst(d.P));
        k_mlp_sig<<<1, 256, 0, s>>>(m.part, m.nblkFeat, m.sig);
        if (int e = mlpForwardTc(m, m.feat, d.N0, d.nLive, d.bc, d.P.inner, m.sig, m.cdir, s)) return e;
        k_mlp_ac<<<gridFor(d.N0, 256), 256, 0, s>>>(d, B, m.cdir, m.re);
        return cudaGetLastError() == cudaSuccess ? 0 : MPSGPU_ERR_CUDA;
    }
    mlpFeatureLaunch(m, d, B, s);
    int e = mlpForwardLaunch(m, m.feat, d.N0, m.sig, m.out, s);
    if (e) return e;
    k_mlp_combine<<<gridFor(d.N0, 256), 256, 0, s>>>(d, B, m.out, m.norm, m.sig, m.cdir);
    k_mlp_step_dots<<<m.nblk, 256, 0, s>>>(d, B, m.cdir, m.re, m.part);
    k_mlp_theta<<<1, 256, 0, s>>>(m.part, m.nblk, m.sig + 1);
    k_mlp_step_apply<<<gridFor(d.N0, 256), 256, 0, s>>>(d, B, m.cdir, m.sig + 1);
    return cudaGetLastError() == cudaSuccess ? 0 : MPSGPU_ERR_CUDA;
}

int mlpFeatures(MlpState& m, const Dev& d, const PpeBuffers& B, float* hostFeat, int n, cudaStream_t s) {
    mlpFeatureLaunch(m, d, B, s);
    if (cudaMemcpyAsync(hostFeat, m.feat, sizeof(float) * NF * n, cudaMemcpyDeviceToHost, s) != cudaSuccess) return MPSGPU_ERR_CUDA;
    return cudaStreamSynchronize(s) == cudaSuccess ? 0 : MPSGPU_ERR_CUDA;
}

// ------------------------------------------------------------------ weights
__global__ void k_to_bf16(const float* master, __nv_bfloat16* wbf) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < H * NF) wbf[BW1 + k] = __float2bfloat16(master[OW1 + k]);
    if (k < H * H) { wbf[BW2 + k] = __float2bfloat16(master[OW2 + k]); wbf[BW3 + k] = __float2bfloat16(master[OW3 + k]); }
    if (k < H) wbf[BW4 + k] = __float2bfloat16(master[OW4 + k]);
}

int mlpInit(MlpState& m, int n0, cudaStream_t s) {
    m.N0 = n0;
    size_t bytes = 0;
    auto al = [&](void** p, size_t b) { bytes += b; return cudaMalloc(p, b) == cudaSuccess; };
    bool ok = al((void**)&m.master, sizeof(float) * NPARAM) && al((void**)&m.adam_m, sizeof(float) * NPARAM) &&
              al((void**)&m.adam_v, sizeof(float) * NPARAM) && al((void**)&m.grad, sizeof(float) * NPARAM) &&
              al((void**)&m.wbf, sizeof(__nv_bfloat16) * NBF) && al((void**)&m.norm, sizeof(float) * NNORM) &&
              al((void**)&m.feat, sizeof(float) * NF * (size_t)n0) && al((void**)&m.out, sizeof(float) * (size_t)n0) &&
              al((void**)&m.lossAcc, sizeof(float) * 4);
    if (!ok) return MPSGPU_ERR_NOMEM;
    {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        m.nblk = std::max(1, sms) * 8;
        int per = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mlp_feat64, 256, 0) != cudaSuccess || per <= 0) per = 1;
        m.nblkFeat = std::min(m.nblk, std::max(1, sms) * per);
    }
    ok = al((void**)&m.re, sizeof(float) * (size_t)n0) && al((void**)&m.cdir, sizeof(float) * (size_t)n0) &&
         al((void**)&m.xe32, sizeof(float) * (size_t)n0) &&
         al((void**)&m.part, sizeof(double) * 2 * (size_t)m.nblk) && al((void**)&m.sig, 2 * sizeof(double)) &&
         al((void**)&m.tcErr, sizeof(int));
    if (!ok) return MPSGPU_ERR_NOMEM;
    cudaMemsetAsync(m.master, 0, sizeof(float) * NPARAM, s);
    cudaMemsetAsync(m.adam_m, 0, sizeof(float) * NPARAM, s);
    cudaMemsetAsync(m.adam_v, 0, sizeof(float) * NPARAM, s);
    cudaMemsetAsync(m.grad, 0, sizeof(float) * NPARAM, s);
    cudaMemsetAsync(m.tcErr, 0, sizeof(int), s);
    (void)bytes;
    return 0;
}

void mlpFree(MlpState& m) {
    for (void* p : {(void*)m.master, (void*)m.adam_m, (void*)m.adam_v, (void*)m.grad, (void*)m.wbf, (void*)m.norm,
                    (void*)m.feat, (void*)m.out, (void*)m.recFeat, (void*)m.recTarget, (void*)m.lossAcc,
                    (void*)m.re, (void*)m.cdir, (void*)m.part, (void*)m.sig, (void*)m.xe32, (void*)m.tcErr})
        if (p) cudaFree(p);
    m = MlpState();
}

int mlpSetWeights(MlpState& m, const float* params, const float* norm32, cudaStream_t s) {
    if (cudaMemcpyAsync(m.master, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice, s) != cudaSuccess) return MPSGPU_ERR_CUDA;
    if (cudaMemcpyAsync(m.norm, norm32, sizeof(float) * NNORM, cudaMemcpyHostToDevice, s) != cudaSuccess) return MPSGPU_ERR_CUDA;
    k_to_bf16<<<gridFor(H * H, 256), 256, 0, s>>>(m.master, m.wbf);
    cudaMemsetAsync(m.adam_m, 0, sizeof(float) * NPARAM, s);
    cudaMemsetAsync(m.adam_v, 0, sizeof(float) * NPARAM, s);
    m.adamStep = 0;
    if (cudaStreamSynchronize(s) != cudaSuccess) return MPSGPU_ERR_CUDA;
    m.ready = true;
    return 0;
}

int mlpGetWeights(MlpState& m, float* params, float* norm32, cudaStream_t s) {
    if (cudaMemcpyAsync(params, m.master, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, s) != cudaSuccess) return MPSGPU_ERR_CUDA;
    if (cudaMemcpyAsync(norm32, m.norm, sizeof(float) * NNORM, cudaMemcpyDeviceToHost, s) != cudaSuccess) return MPSGPU_ERR_CUDA;
    return cudaStreamSynchronize(s) == cudaSuccess ? 0 : MPSGPU_ERR_CUDA;
}

// ------------------------------------------------------------------ recording
int mlpRecordFeatures(MlpState& m, const Dev& d, const PpeBuffers& B, cudaStream_t s) {
    mlpFeatureLaunch(m, d, B, s);
    return cudaGetLastError() == cudaSuccess ? 0 : MPSGPU_ERR_CUDA;
}
__global__ void k_mlp_record(Dev d, PpeBuffers B, const float* feat, const double* sig, float* recFeat,
                             float* recTarget, unsigned long long* count, long long cap) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    if (d.bc[i] != d.P.inner) return;
    unsigned long long slot = atomicAdd(count, 1ull);
    if ((long long)slot >= cap) return;
    const float4* src = (const float4*)(feat + (size_t)i * NF);
    float4* dst = (float4*)(recFeat + slot * NF);
    const double sg = sig[0];
    const float q = (float)(1.0 / sg);
    float4 a = src[0], b = src[1], c = src[2], e = src[3];
    a.y *= q; b.y *= q; b.w *= q; e.z *= q;   // features 1, 5, 7, 14 in units of sigma
    dst[0] = a; dst[1] = b; dst[2] = c; dst[3] = e;
    recTarget[slot] = (float)((B.x[i] - extrapBase(d, i)) / sg);
}
int mlpRecordTargets(MlpState& m, const Dev& d, const PpeBuffers& B, cudaStream_t s) {
    if (!m.recFeat) {
        m.recCap = std::max<long long>(1 << 20, std::min<long long>(24ll << 20, 200ll * d.N0));
        if (cudaMalloc(&m.recFeat, sizeof(float) * NF * m.recCap) != cudaSuccess) return MPSGPU_ERR_NOMEM;
        if (cudaMalloc(&m.recTarget, sizeof(float) * m.recCap + 16) != cudaSuccess) return MPSGPU_ERR_NOMEM;
        cudaMemsetAsync((char*)m.recTarget + sizeof(float) * m.recCap, 0, 16, s);
    }
    unsigned long long* cnt = (unsigned long long*)((char*)m.recTarget + sizeof(float) * m.recCap);
    cudaMemcpyAsync(cnt, &m.recCount, sizeof(unsigned long long), cudaMemcpyHostToDevice, s);
    k_mlp_record<<<gridFor(d.N0, 256), 256, 0, s>>>(d, B, m.feat, m.sig, m.recFeat, m.recTarget, cnt, m.recCap);
    unsigned long long c = 0;
    cudaMemcpyAsync(&c, cnt, sizeof(c), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return MPSGPU_ERR_CUDA;
    m.recCount = std::min<long long>((long long)c, m.recCap);
    return 0;
}

// mean / inverse std of each recorded feature (FP64 partial sums), and of the target
__global__ void k_mlp_moments(const float* recFeat, const float* recTarget, long long n, double* acc) {
    __shared__ double sm[2 * (NF + 1)];
    for (int k = threadIdx.x; k < 2 * (NF + 1); k += blockDim.x) sm[k] = 0.0;
    __syncthreads();
    double s1[NF + 1], s2[NF + 1];
    for (int k = 0; k <= NF; k++) { s1[k] = 0; s2[k] = 0; }
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
        for (int k = 0; k < NF; k++) { double v = recFeat[r * NF + k]; s1[k] += v; s2[k] += v * v; }
        double y = recTarget[r];
        s1[NF] += y; s2[NF] += y * y;
    }
    for (int k = 0; k <= NF; k++) { atomicAdd(&sm[k], s1[k]); atomicAdd(&sm[NF + 1 + k], s2[k]); }
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * (NF + 1); k += blockDim.x) atomicAdd(&acc[k], sm[k]);
}
int mlpFitNormalization(MlpState& m, cudaStream_t s) {
    if (m.recCount <= 1) return MPSGPU_ERR_ARG;
    double* acc = nullptr;
    if (cudaMalloc(&acc, sizeof(double) * 2 * (NF + 1)) != cudaSuccess) return MPSGPU_ERR_NOMEM;
    cudaMemsetAsync(acc, 0, sizeof(double) * 2 * (NF + 1), s);
    k_mlp_moments<<<512, 256, 0, s>>>(m.recFeat, m.recTarget, m.recCount, acc);
    double h[2 * (NF + 1)];
    cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    cudaFree(acc);
    float norm[NNORM];
    double nn = (double)m.recCount;
    for (int k = 0; k < NF; k++) {
        double mu = h[k] / nn, var = h[NF + 1 + k] / nn - mu * mu;
        norm[k] = (float)mu;
        norm[NF + k] = (float)(var > 1e-20 ? 1.0 / sqrt(var) : 1.0);
    }
    // the network output is the correction in units of the target spread about its mean
    double my = h[NF] / nn, vy = h[2 * NF + 1] / nn - my * my;
    norm[2 * NF] = (float)my;
    norm[2 * NF + 1] = (float)(vy > 1e-20 ? 1.0 / sqrt(vy) : 1.0);
    if (cudaMemcpyAsync(m.norm, norm, sizeof(norm), cudaMemcpyHostToDevice, s) != cudaSuccess) return MPSGPU_ERR_CUDA;
    return cudaStreamSynchronize(s) == cudaSuccess ? 0 : MPSGPU_ERR_CUDA;
}

// ------------------------------------------------------------------ training
// Transposed BF16 tiles for dW = dZ^T H: [unit][sample], 64 samples per block iteration.
struct SmemT {
    __nv_bfloat16 w2t[H * S2];   // W2^T [in][out]
    __nv_bfloat16 w3t[H * S2];   // W3^T
    __nv_bfloat16 xT[NF * S2];   // inputs [feature][sample]
    __nv_bfloat16 h1T[H * S2], h2T[H * S2];
    __nv_bfloat16 d1T[H * S2], d2T[H * S2], d3T[H * S2];
    float w4g[H];
    float bg[3][H];
    float zero[H];
    float b4g;
    float loss;
};

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

// store a 16 x 64 C-layout tile (rows = samples rowBase.., cols = units) transposed into T[unit][sample]
__device__ __forceinline__ void storeT(__nv_bfloat16* T, const float (*z)[4], int rowBase, bool applyGelu) {
    int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        int c = 8 * j + 2 * t;
        float v0 = z[j][0], v1 = z[j][1], v2 = z[j][2], v3 = z[j][3];
        if (applyGelu) { v0 = gelu(v0); v1 = gelu(v1); v2 = gelu(v2); v3 = gelu(v3); }
        T[c * S2 + rowBase + g] = __float2bfloat16(v0);
        T[(c + 1) * S2 + rowBase + g] = __float2bfloat16(v1);
        T[c * S2 + rowBase + g + 8] = __float2bfloat16(v2);
        T[(c + 1) * S2 + rowBase + g + 8] = __float2bfloat16(v3);
    }
}
// acc[nt][4] += A^T-tile(m-tile mt of AT[unit][sample]) x B (BT[unit][sample]) over 64 samples
template <int NT>
__device__ __forceinline__ void wgrad(const __nv_bfloat16* AT, const __nv_bfloat16* BT, int mt, float (*acc)[4]) {
    int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
#pragma unroll
    for (int ks = 0; ks < 4; ks++) {
        uint32_t a[4];
        const __nv_bfloat16* r0 = AT + (16 * mt + g) * S2 + 16 * ks + 2 * t;
        const __nv_bfloat16* r1 = r0 + 8 * S2;
        a[0] = *(const uint32_t*)r0; a[1] = *(const uint32_t*)r1;
        a[2] = *(const uint32_t*)(r0 + 8); a[3] = *(const uint32_t*)(r1 + 8);
#pragma unroll
        for (int j = 0; j < NT; j++) {
            const __nv_bfloat16* b = BT + (8 * j + g) * S2 + 16 * ks + 2 * t;
            mma16816(acc[j], a, *(const uint32_t*)b, *(const uint32_t*)(b + 8));
        }
    }
}

__global__ void __launch_bounds__(128) k_mlp_train(const float* recFeat, const float* recTarget, long long nrec,
                                                  int batch, uint32_t seed, const __nv_bfloat16* wbf,
                                                  const float* master, const float* norm, float* grad, float* lossAcc) {
    extern __shared__ __align__(16) unsigned char smraw[];
    SmemW& s = *(SmemW*)smraw;
    SmemT& T = *(SmemT*)(smraw + ((sizeof(SmemW) + 15) / 16) * 16);
    loadWeights(s, wbf, master, norm);
    for (int k = threadIdx.x; k < H * H; k += blockDim.x) {
        int o = k / H, in = k % H;
        T.w2t[in * S2 + o] = wbf[BW2 + k];
        T.w3t[in * S2 + o] = wbf[BW3 + k];
    }
    for (int k = threadIdx.x; k < H; k += blockDim.x) {
        T.w4g[k] = 0.f; T.bg[0][k] = T.bg[1][k] = T.bg[2][k] = 0.f; T.zero[k] = 0.f;
    }
    if (threadIdx.x == 0) { T.b4g = 0.f; T.loss = 0.f; }
    __syncthreads();
    int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, w = threadIdx.x >> 5;
    float ysc = norm[2 * NF + 1], ymu = norm[2 * NF];
    float inv_b = 1.0f / (float)batch;
    float acc3[8][4], acc2[8][4], acc1[2][4];
#pragma unroll
    for (int j = 0; j < 8; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) { acc3[j][q] = 0.f; acc2[j][q] = 0.f; }
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc1[j][q] = 0.f;
    int iters = batch / 64;
    for (int it = blockIdx.x; it < iters; it += gridDim.x) {
        // sample rows for this warp's 16-sample tile
        int base = it * 64 + w * 16;
        // seed 0: samples in order (gradient checks); otherwise uniform with replacement
        long long r0 = seed ? hash32(seed * 2654435761u + (uint32_t)(base + g)) % (uint32_t)nrec : (base + g) % nrec;
        long long r1 = seed ? hash32(seed * 2654435761u + (uint32_t)(base + g + 8)) % (uint32_t)nrec : (base + g + 8) % nrec;
        const float* f0 = recFeat + r0 * NF;
        const float* f1 = recFeat + r1 * NF;
        float y0 = (recTarget[r0] - ymu) * ysc, y1 = (recTarget[r1] - ymu) * ysc;
        uint32_t ax[1][4], a1[4][4], a2[4][4];
        float z1[8][4], z2[8][4], z3[8][4];
        loadInput(s, f0, f1, ax[0]);
        layer<1, S1>(ax, s.w1, s.b1, z1);
        activate(z1, a1);
        layer<4, S2>(a1, s.w2, s.b2, z2);
        activate(z2, a2);
        layer<4, S2>(a2, s.w3, s.b3, z3);
        float o0, o1;
        headOut(s, z3, o0, o1);
        float e0 = o0 - y0, e1 = o1 - y1;
        float dout0 = 2.f * e0 * inv_b, dout1 = 2.f * e1 * inv_b;
        if (t == 0) atomicAdd(&T.loss, (e0 * e0 + e1 * e1) * inv_b);
        // stage inputs and activations transposed: rows of this warp's tile are w*16 + (g, g+8)
        {
            int c0 = 2 * t, c1 = 2 * t + 8;
            float in0[4] = {(f0[c0] - s.mean[c0]) * s.istd[c0], (f0[c0 + 1] - s.mean[c0 + 1]) * s.istd[c0 + 1],
                            (f0[c1] - s.mean[c1]) * s.istd[c1], (f0[c1 + 1] - s.mean[c1 + 1]) * s.istd[c1 + 1]};
            float in1[4] = {(f1[c0] - s.mean[c0]) * s.istd[c0], (f1[c0 + 1] - s.mean[c0 + 1]) * s.istd[c0 + 1],
                            (f1[c1] - s.mean[c1]) * s.istd[c1], (f1[c1 + 1] - s.mean[c1 + 1]) * s.istd[c1 + 1]};
            int cs[4] = {c0, c0 + 1, c1, c1 + 1};
#pragma unroll
            for (int q = 0; q < 4; q++) {
                T.xT[cs[q] * S2 + w * 16 + g] = __float2bfloat16(in0[q]);
                T.xT[cs[q] * S2 + w * 16 + g + 8] = __float2bfloat16(in1[q]);
            }
        }
        storeT(T.h1T, z1, w * 16, true);
        storeT(T.h2T, z2, w * 16, true);
        // head: dW4, db4, dz3 = dout * w4 * gelu'(z3)
        float d3[8][4];
        float gw[16];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            int c = 8 * j + 2 * t;
            gw[2 * j] = dout0 * gelu(z3[j][0]) + dout1 * gelu(z3[j][2]);
            gw[2 * j + 1] = dout0 * gelu(z3[j][1]) + dout1 * gelu(z3[j][3]);
            d3[j][0] = dout0 * s.w4[c] * gelud(z3[j][0]);
            d3[j][1] = dout0 * s.w4[c + 1] * gelud(z3[j][1]);
            d3[j][2] = dout1 * s.w4[c] * gelud(z3[j][2]);
            d3[j][3] = dout1 * s.w4[c + 1] * gelud(z3[j][3]);
        }
#pragma unroll
        for (int q = 0; q < 16; q++) {
            float v = gw[q];
            v += __shfl_xor_sync(0xffffffffu, v, 4); v += __shfl_xor_sync(0xffffffffu, v, 8);
            v += __shfl_xor_sync(0xffffffffu, v, 16);
            gw[q] = v;
        }
        if (g == 0) {
#pragma unroll
            for (int j = 0; j < 8; j++) { atomicAdd(&T.w4g[8 * j + 2 * t], gw[2 * j]); atomicAdd(&T.w4g[8 * j + 2 * t + 1], gw[2 * j + 1]); }
        }
        if (t == 0) {
            float db = dout0 + dout1;
            db += __shfl_xor_sync(0x11111111u, db, 4); db += __shfl_xor_sync(0x11111111u, db, 8);
            db += __shfl_xor_sync(0x11111111u, db, 16);
            if (g == 0) atomicAdd(&T.b4g, db);
        }
        storeT(T.d3T, d3, w * 16, false);
        // dh2 = dz3 W3 ; dz2 = dh2 * gelu'(z2)
        uint32_t ad[4][4];
#pragma unroll
        for (int kc = 0; kc < 4; kc++) {
            ad[kc][0] = pack2(d3[2 * kc][0], d3[2 * kc][1]);
            ad[kc][1] = pack2(d3[2 * kc][2], d3[2 * kc][3]);
            ad[kc][2] = pack2(d3[2 * kc + 1][0], d3[2 * kc + 1][1]);
            ad[kc][3] = pack2(d3[2 * kc + 1][2], d3[2 * kc + 1][3]);
        }
        float dh[8][4];
        layer<4, S2>(ad, T.w3t, T.zero, dh);
#pragma unroll
        for (int j = 0; j < 8; j++)
#pragma unroll
            for (int q = 0; q < 4; q++) dh[j][q] *= gelud(z2[j][q]);
        storeT(T.d2T, dh, w * 16, false);
#pragma unroll
        for (int kc = 0; kc < 4; kc++) {
            ad[kc][0] = pack2(dh[2 * kc][0], dh[2 * kc][1]);
            ad[kc][1] = pack2(dh[2 * kc][2], dh[2 * kc][3]);
            ad[kc][2] = pack2(dh[2 * kc + 1][0], dh[2 * kc + 1][1]);
            ad[kc][3] = pack2(dh[2 * kc + 1][2], dh[2 * kc + 1][3]);
        }
        layer<4, S2>(ad, T.w2t, T.zero, dh);
#pragma unroll
        for (int j = 0; j < 8; j++)
#pragma unroll
            for (int q = 0; q < 4; q++) dh[j][q] *= gelud(z1[j][q]);
        storeT(T.d1T, dh, w * 16, false);
        __syncthreads();
        // weight gradients: warp w owns output units 16w..16w+15 of every layer
        wgrad<8>(T.d3T, T.h2T, w, acc3);
        wgrad<8>(T.d2T, T.h1T, w, acc2);
        wgrad<2>(T.d1T, T.xT, w, acc1);
        // bias gradients: column sums of dZ over the 64 samples
        for (int u = threadIdx.x; u < 3 * H; u += blockDim.x) {
            int l = u / H, unit = u % H;
            const __nv_bfloat16* src = (l == 0 ? T.d1T : (l == 1 ? T.d2T : T.d3T)) + unit * S2;
            float sacc = 0.f;
            for (int q = 0; q < 64; q++) sacc += __bfloat162float(src[q]);
            T.bg[l][unit] += sacc;
        }
        __syncthreads();
    }
    // flush: acc[j] holds rows (units) 16w+g, 16w+g+8 and cols 8j+2t, +1
#pragma unroll
    for (int j = 0; j < 8; j++) {
        int r0 = 16 * w + g, c = 8 * j + 2 * t;
        atomicAdd(&grad[OW3 + r0 * H + c], acc3[j][0]); atomicAdd(&grad[OW3 + r0 * H + c + 1], acc3[j][1]);
        atomicAdd(&grad[OW3 + (r0 + 8) * H + c], acc3[j][2]); atomicAdd(&grad[OW3 + (r0 + 8) * H + c + 1], acc3[j][3]);
        atomicAdd(&grad[OW2 + r0 * H + c], acc2[j][0]); atomicAdd(&grad[OW2 + r0 * H + c + 1], acc2[j][1]);
        atomicAdd(&grad[OW2 + (r0 + 8) * H + c], acc2[j][2]); atomicAdd(&grad[OW2 + (r0 + 8) * H + c + 1], acc2[j][3]);
    }
#pragma unroll
    for (int j = 0; j < 2; j++) {
        int r0 = 16 * w + g, c = 8 * j + 2 * t;
        atomicAdd(&grad[OW1 + r0 * NF + c], acc1[j][0]); atomicAdd(&grad[OW1 + r0 * NF + c + 1], acc1[j][1]);
        atomicAdd(&grad[OW1 + (r0 + 8) * NF + c], acc1[j][2]); atomicAdd(&grad[OW1 + (r0 + 8) * NF + c + 1], acc1[j][3]);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < H; k += blockDim.x) {
        atomicAdd(&grad[OW4 + k], T.w4g[k]);
        atomicAdd(&grad[OB1 + k], T.bg[0][k]);
        atomicAdd(&grad[OB2 + k], T.bg[1][k]);
        atomicAdd(&grad[OB3 + k], T.bg[2][k]);
    }
    if (threadIdx.x == 0) { atomicAdd(&grad[OB4], T.b4g); atomicAdd(lossAcc, T.loss); }
}

// Adam (Kingma & Ba 2015) on the FP32 master weights, then the BF16 refresh; zeroes grad.
__global__ void k_adam(float* master, float* mo, float* ve, float* grad, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= NPARAM) return;
    float gk = grad[k];
    float m = b1 * mo[k] + (1.f - b1) * gk;
    float v = b2 * ve[k] + (1.f - b2) * gk * gk;
    mo[k] = m; ve[k] = v;
    master[k] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
    grad[k] = 0.f;
}

int mlpTrain(MlpState& m, int iters, int batch, float lr, unsigned long long seed, float* lossHist, cudaStream_t s) {
    if (m.recCount < 64 || batch < 64 || (batch % 64)) return MPSGPU_ERR_ARG;
    size_t smem = ((sizeof(SmemW) + 15) / 16) * 16 + sizeof(SmemT);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    int blocks = std::min(batch / 64, 1024);
    std::vector<float> lh(iters, 0.f);
    for (int it = 0; it < iters; it++) {
        cudaMemsetAsync(m.lossAcc, 0, sizeof(float), s);
        k_mlp_train<<<blocks, 128, smem, s>>>(m.recFeat, m.recTarget, m.recCount, batch,
                                              (uint32_t)(seed * 1000003ull + it), m.wbf, m.master, m.norm, m.grad, m.lossAcc);
        m.adamStep++;
        float c1 = 1.f - powf(0.9f, (float)m.adamStep), c2 = 1.f - powf(0.999f, (float)m.adamStep);
        k_adam<<<gridFor(NPARAM, 256), 256, 0, s>>>(m.master, m.adam_m, m.adam_v, m.grad, lr, 0.9f, 0.999f, 1e-8f, c1, c2);
        k_to_bf16<<<gridFor(H * H, 256), 256, 0, s>>>(m.master, m.wbf);
        if (lossHist) cudaMemcpyAsync(&lh[it], m.lossAcc, sizeof(float), cudaMemcpyDeviceToHost, s);
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) return MPSGPU_ERR_CUDA;
    if (cudaGetLastError() != cudaSuccess) return MPSGPU_ERR_CUDA;
    if (lossHist) std::memcpy(lossHist, lh.data(), sizeof(float) * iters);
    m.ready = true;
    return 0;
}

// ------------------------------------------------------------------ checks
// Network outputs for host-supplied raw features (inference check against a CPU model).
int mlpTcStatus(MlpState& m, cudaStream_t s) {
    int h = 0;
    if (cudaMemcpyAsync(&h, m.tcErr, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemsetAsync(m.tcErr, 0, sizeof(int), s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
        return MPSGPU_ERR_CUDA;
    return h ? MPSGPU_ERR_CUDA : 0;
}

int mlpForwardHost(MlpState& m, const float* hfeat, int n, float* hout, cudaStream_t s) {
    float *df = nullptr, *dout = nullptr;
    if (cudaMalloc(&df, sizeof(float) * NF * n) != cudaSuccess) return MPSGPU_ERR_NOMEM;
    if (cudaMalloc(&dout, sizeof(float) * n) != cudaSuccess) { cudaFree(df); return MPSGPU_ERR_NOMEM; }
    cudaMemcpyAsync(df, hfeat, sizeof(float) * NF * n, cudaMemcpyHostToDevice, s);
    int e = mlpForwardTc(m, df, n, nullptr, nullptr, 0, nullptr, dout, s);
    if (!e) cudaMemcpyAsync(hout, dout, sizeof(float) * n, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) e = MPSGPU_ERR_CUDA;
    if (!e) e = mlpTcStatus(m, s);
    cudaFree(df); cudaFree(dout);
    return e;
}

// Gradient of the mean squared error over n host samples (n a multiple of 64, in order),
// without an optimiser step (gradient check against a CPU model).
int mlpGradient(MlpState& m, const float* hfeat, const float* htarget, int n, float* hgrad, float* hloss,
                cudaStream_t s) {
    if (n < 64 || (n % 64)) return MPSGPU_ERR_ARG;
    float *df = nullptr, *dt = nullptr;
    if (cudaMalloc(&df, sizeof(float) * NF * n) != cudaSuccess) return MPSGPU_ERR_NOMEM;
    if (cudaMalloc(&dt, sizeof(float) * n) != cudaSuccess) { cudaFree(df); return MPSGPU_ERR_NOMEM; }
    cudaMemcpyAsync(df, hfeat, sizeof(float) * NF * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dt, htarget, sizeof(float) * n, cudaMemcpyHostToDevice, s);
    size_t smem = ((sizeof(SmemW) + 15) / 16) * 16 + sizeof(SmemT);
    cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaMemsetAsync(m.grad, 0, sizeof(float) * NPARAM, s);
    cudaMemsetAsync(m.lossAcc, 0, sizeof(float), s);
    k_mlp_train<<<std::min(n / 64, 1024), 128, smem, s>>>(df, dt, n, n, 0u, m.wbf, m.master, m.norm, m.grad, m.lossAcc);
    cudaMemcpyAsync(hgrad, m.grad, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(hloss, m.lossAcc, sizeof(float), cudaMemcpyDeviceToHost, s);
    cudaMemsetAsync(m.grad, 0, sizeof(float) * NPARAM, s);
    int e = (cudaStreamSynchronize(s) == cudaSuccess && cudaGetLastError() == cudaSuccess) ? 0 : MPSGPU_ERR_CUDA;
    cudaFree(df); cudaFree(dt);
    return e;
}
