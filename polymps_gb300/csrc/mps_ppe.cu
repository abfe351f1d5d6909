// mps_ppe.cu — pressure Poisson equation on sm_103a: assembly and solvers.
//
// Assembly replaces the serial Eigen triplet loop of MpsPressure::solvePressurePoissonPnd
// (src/MpsPressure.cpp:169-286): one thread per row walks its ELL neighbour row and writes
// the off-diagonal entries (j inner, not dummy) straight into an ELL matrix
// (val/col at ellBase(i) + k ellStride, coalesced across a warp), the diagonal and the right-hand side.
//
// The plain solver replaces Eigen's ConjugateGradient<..., Lower|Upper> with its default
// diagonal preconditioner (src/MpsPressure.cpp:424-445): Jacobi-PCG in FP64 warm-started
// from the previous unclamped solution, stopping when ||r||^2 < tol^2 ||b||^2.  Per
// iteration three grid-stride kernels (SpMV + p.Ap, x/r/z update + r.z and r.r,
// p update); the scalar reductions are deterministic (per-block partials, the last block
// to finish sums them in block order) and the solver state stays on the device: the host
// only polls the "done" word every few iterations.
//
// The mixed solver keeps FP64 for the iterative-refinement residual r = b - Ax, its norm
// and all dot products, and runs the inner CG on FP32 matrix values and vectors.
#include "mps_df.cuh"
#include "mps_internal.h"
#include "mps_bulk.cuh"

#define PBLK 256

// solver scalars in B.scal[]
enum { S_RZ = 0, S_RR, S_BB, S_ALPHA, S_BETA, S_PAP, S_THR, S_RZNEW, S_SCALE, S_INV, S_SQRT, S_ETA2, S_RR0,
       S_RHO, S_RHOOLD, S_OMEGA, S_R0N2, S_COUNT };

// ------------------------------------------------------------------ assembly
__global__ void __launch_bounds__(128) k_ppe_assemble(Dev d, PpeBuffers B) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    int bci = d.bc[i];
    if (bci == P.other || bci == P.surface) {
        B.diag[i] = 1.0; B.rowLen[i] = 0; B.b[i] = 0.0; B.mfMask[i] = maskNone();
        warpCount(d.counters + 1, 0u);
        return;
    }
    dvec4 pi = d.pos[i];
    double sum = 0.0, src = 0.0;
    int len = 0;
    Mask mm = maskNone();
    const double* wLc = d.cwL ? d.cwL : d.cw;
    forMaskK(d, i, d.maskL[i], [&](int j, size_t e, int ke) {
        double wL = wLc[e];
        double mij = wL * P.coeffPPE;
        if (d.type[j] == P.dummyWall) {
            dvec4 pj = d.pos[j];
            double v0 = pj.x - pi.x, v1 = pj.y - pi.y, v2 = pj.z - pi.z;
            double pgh = P.DNS_FL1 * (v0 * P.gravity[0] + v1 * P.gravity[1] + v2 * P.gravity[2]) * wL;
            src -= P.coeffPPE * pgh;
        } else {
            sum -= mij;
            if (d.bc[j] == P.inner) {
                size_t k = ellBase(B, i) + (size_t)len * B.ellStride;
                B.val[k] = mij;
                B.col[k] = j;
                len++;
                maskSet(mm, ke);
            }
        }
    });
    double rho = P.DNS_FL1;
    sum -= P.alphaCompressibility * rho / (P.timeStep * P.timeStep);
    B.diag[i] = sum;
    B.rowLen[i] = len;
    B.mfMask[i] = mm;
    B.b[i] = src + ppeSource(d, i, rho);
    warpCount(d.counters + 1, (unsigned)len);
}
void launchPpeAssemble(const Dev& d, const PpeBuffers& B, cudaStream_t s) {
    cudaMemsetAsync(d.counters + 1, 0, sizeof(unsigned long long), s);
    k_ppe_assemble<<<gridFor(d.N0, 128), 128, 0, s>>>(d, B);
}

// press = max(x, 0) (setZeroOnNegativePressure, src/MpsPressure.cpp:471-476); x is kept
// unclamped in pressPPE as the next warm start.
__global__ void k_ppe_copy_back(Dev d, PpeBuffers B) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    double x = B.x[i];
    d.pressPPEprev2[i] = d.pressPPEprev[i];
    d.pressPPEprev[i] = d.pressPPE[i];
    d.pressPPE[i] = x;
    d.source[i] = B.b[i];
    d.press[i] = x < 0.0 ? 0.0 : x;
}
// Warm start by extrapolation in time of the unclamped solutions on the rows of the new
// system that carry an equation (zero on the identity rows): linear x0 = 2 p_n - p_{n-1}
// or quadratic x0 = 3 p_n - 3 p_{n-1} + p_{n-2}.
__global__ void k_warm_extrap(Dev d, PpeBuffers B, int quad) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    double p = d.pressPPE[i], q = d.pressPPEprev[i];
    double x = quad ? 3.0 * (p - q) + d.pressPPEprev2[i] : (p + p) - q;
    B.x[i] = (d.bc[i] == d.P.inner) ? x : 0.0;
}
void launchWarmExtrapolate(const Dev& d, const PpeBuffers& B, cudaStream_t s, bool quadratic) {
    k_warm_extrap<<<gridFor(d.N0, 256), 256, 0, s>>>(d, B, quadratic ? 1 : 0);
}
void launchPpeCopyBack(const Dev& d, const PpeBuffers& B, cudaStream_t s) {
    k_ppe_copy_back<<<gridFor(d.N0, 256), 256, 0, s>>>(d, B);
}

// ------------------------------------------------------------------ reductions
// Block-wide sum of NV doubles; the last block to arrive sums the per-block partials in
// block order (deterministic) and calls fin(tot) with thread 0.
template <int NV>
__device__ __forceinline__ void blockSum(double (&v)[NV], double* sm) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; q++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    }
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; q++) sm[q * 32 + w] = v[q];
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) {
            double x = (lane < nw) ? sm[q * 32 + lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            v[q] = x;
        }
    }
    __syncthreads();
}

template <int NV, class Fin>
__device__ __forceinline__ void gridSum(double (&v)[NV], const PpeBuffers& B, Fin fin) {
    __shared__ double sm[NV * 32];
    __shared__ bool last;
    blockSum<NV>(v, sm);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) B.partials[q * gridDim.x + blockIdx.x] = v[q];
        __threadfence();
        unsigned int t = atomicInc(B.counter, gridDim.x - 1);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) {
        double s = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
            s += ((volatile double*)B.partials)[q * gridDim.x + b];
        acc[q] = s;
    }
    blockSum<NV>(acc, sm);
    if (threadIdx.x == 0) fin(acc);
}

// ------------------------------------------------------------------ ELL rows (ellRow: mps_common.cuh)
__device__ __forceinline__ double spmvRow(const PpeBuffers& B, const double* x, int i) {
    return ellRow<double, true>(B.diag, B.val, B.col, x, i, __ldg(B.rowLen + i), ellBase(B, i), B.ellStride);
}

// r = b - A x, z = r / diag, p = z; sums r.z, r.r, b.b
__global__ void __launch_bounds__(PBLK) k_cg_init(Dev d, PpeBuffers B, double tol) {
    int n = liveN(d);
    double v[3] = {0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double r = B.b[i] - spmvRow(B, B.x, i);
        double z = r / B.diag[i];
        B.r[i] = r; B.z[i] = z; B.p[i] = z;
        v[0] += r * z; v[1] += r * r; v[2] += B.b[i] * B.b[i];
    }
    gridSum<3>(v, B, [&](double* t) {
        B.scal[S_RZ] = t[0]; B.scal[S_RR] = t[1]; B.scal[S_BB] = t[2];
        double thr = tol * tol * t[2];
        if (thr < 2.2250738585072014e-308) thr = 2.2250738585072014e-308;
        B.scal[S_THR] = thr;
        B.scal[S_SCALE] = sqrt(t[1] / (t[2] > 0 ? t[2] : 1.0));   // initial relative residual
        B.flag[0] = (t[2] == 0.0 || t[1] < thr) ? 1 : 0;
        B.flag[1] = 0;
        if (!(t[0] == t[0]) || !(t[1] == t[1])) { B.flag[0] = 1; B.flag[2] = 1; }
    });
}
// Ap = A p; sum p.Ap -> alpha
__global__ void __launch_bounds__(PBLK) k_cg_spmv(Dev d, PpeBuffers B) {
    if (*(volatile int*)B.flag) return;
    int n = liveN(d);
    double v[1] = {0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double ap = spmvRow(B, B.p, i);
        B.Ap[i] = ap;
        v[0] += B.p[i] * ap;
    }
    gridSum<1>(v, B, [&](double* t) { B.scal[S_PAP] = t[0]; B.scal[S_ALPHA] = B.scal[S_RZ] / t[0]; });
}
// x += alpha p; r -= alpha Ap; z = r/diag; sums r.z, r.r -> beta, convergence
__global__ void __launch_bounds__(PBLK) k_cg_update(Dev d, PpeBuffers B) {
    if (*(volatile int*)B.flag) return;
    int n = liveN(d);
    double alpha = B.scal[S_ALPHA];
    double v[2] = {0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double p = B.p[i];
        B.x[i] += alpha * p;
        double r = B.r[i] - alpha * B.Ap[i];
        double z = r / B.diag[i];
        B.r[i] = r; B.z[i] = z;
        v[0] += r * z; v[1] += r * r;
    }
    gridSum<2>(v, B, [&](double* t) {
        B.flag[1] += 1;
        B.scal[S_RR] = t[1];
        B.scal[S_BETA] = t[0] / B.scal[S_RZ];
        B.scal[S_RZ] = t[0];
        if (t[1] < B.scal[S_THR]) B.flag[0] = 1;
        if (!(t[1] == t[1])) { B.flag[0] = 1; B.flag[2] = 1; }
    });
}
// p = z + beta p
__global__ void __launch_bounds__(PBLK) k_cg_p(Dev d, PpeBuffers B) {
    if (*(volatile int*)B.flag) return;
    int n = liveN(d);
    double beta = B.scal[S_BETA];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        B.p[i] = B.z[i] + beta * B.p[i];
}
// true residual ||b - A x||^2 (FP64) into scal[S_RR]
__global__ void __launch_bounds__(PBLK) k_true_residual(Dev d, PpeBuffers B) {
    int n = liveN(d);
    double v[1] = {0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double r = B.b[i] - spmvRow(B, B.x, i);
        B.r[i] = r;
        v[0] += r * r;
    }
    gridSum<1>(v, B, [&](double* t) { B.scal[S_RR] = t[0]; });
}

static int pollFlags(const PpeBuffers& B, cudaStream_t s, int* hostFlags) {
    if (cudaMemcpyAsync(hostFlags, B.flag, 3 * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1;
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    return 0;
}

int ppeSolvePlain(const Dev& d, const PpeBuffers& B, double tol, int maxIter, cudaStream_t s,
                  int* iters, double* relres, double* relres0, Prof* prof) {
    int nb = B.nblocks;
    static thread_local int hf[4];
    bool pr = prof && prof->on;
    cudaMemsetAsync(B.flag, 0, 4 * sizeof(int), s);
    if (pr) prof->begin(PROF_PPE_OTHER, s);
    k_cg_init<<<nb, PBLK, 0, s>>>(d, B, tol);
    if (pr) prof->end(s);
    countLaunch(1);
    const int batch = 8;
    int launched = 0;
    while (true) {
        for (int k = 0; k < batch; k++) {
            if (pr) prof->begin(PROF_PPE_SPMV, s);
            k_cg_spmv<<<nb, PBLK, 0, s>>>(d, B);
            if (pr) { prof->end(s); prof->begin(PROF_PPE_VECTOR, s); }
            k_cg_update<<<nb, PBLK, 0, s>>>(d, B);
            k_cg_p<<<nb, PBLK, 0, s>>>(d, B);
            if (pr) prof->end(s);
        }
        countLaunch(3 * batch);
        launched += batch;
        if (pollFlags(B, s, hf)) return MPSGPU_ERR_CUDA;
        if (hf[0] || launched >= maxIter) break;
    }
    double sc[S_COUNT];
    countLaunch(1);
    k_true_residual<<<nb, PBLK, 0, s>>>(d, B);
    cudaMemcpyAsync(sc, B.scal, sizeof(sc), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return MPSGPU_ERR_CUDA;
    *iters = hf[1];
    double bb = sc[S_BB] > 0 ? sc[S_BB] : 1.0;
    *relres = (sc[S_BB] > 0) ? sqrt(sc[S_RR] / bb) : 0.0;
    *relres0 = sc[S_SCALE];
    if (hf[2]) return MPSGPU_ERR_NOT_CONVERGED;
    if (!hf[0]) return MPSGPU_ERR_NOT_CONVERGED;
    return 0;
}

// ------------------------------------------------------------------ mixed FP32/FP64
// FP32 copies of the matrix values and the Jacobi inverse diagonal
__global__ void k_mixed_prepare(Dev d, PpeBuffers B) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    int len = B.rowLen[i];
    const size_t base = ellBase(B, i);
    for (int k = 0; k < len; k++) {
        size_t e = base + (size_t)k * B.ellStride;
        B.valf[e] = (float)B.val[e];
    }
    B.diagf[i] = (float)B.diag[i];
    B.diagInvf[i] = (float)(1.0 / B.diag[i]);
}
void launchMixedPrepare(const Dev& d, const PpeBuffers& B, cudaStream_t s) {
    k_mixed_prepare<<<gridFor(d.N0, 256), 256, 0, s>>>(d, B);
}
// FP64 residual r = b - A x (FP64 values), sums r.r (and b.b on the first call)
__global__ void __launch_bounds__(PBLK) k_mx_residual(Dev d, PpeBuffers B, int first, double tol) {
    int n = liveN(d);
    double v[2] = {0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double r = B.b[i] - spmvRow(B, B.x, i);
        B.r[i] = r;
        v[0] += r * r;
        if (first) v[1] += B.b[i] * B.b[i];
    }
    gridSum<2>(v, B, [&](double* t) {
        B.scal[S_RR] = t[0];
        if (first) {
            B.scal[S_BB] = t[1];
            double thr = tol * tol * t[1];
            if (thr < 2.2250738585072014e-308) thr = 2.2250738585072014e-308;
            B.scal[S_THR] = thr;
            B.scal[S_SCALE] = sqrt(t[0] / (t[1] > 0 ? t[1] : 1.0));
        }
        B.flag[0] = (B.scal[S_BB] == 0.0 || t[0] < B.scal[S_THR]) ? 1 : 0;
        if (!(t[0] == t[0])) { B.flag[0] = 1; B.flag[2] = 1; }
    });
}
// inner start: rf = r / ||r||, d = 0, z = M rf, p = z; r.z (FP64 accumulate)
__global__ void __launch_bounds__(PBLK) k_mx_inner_init(Dev d, PpeBuffers B) {
    int n = liveN(d);
    double inv = 1.0 / sqrt(B.scal[S_RR]);
    double v[1] = {0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float r = (float)(B.r[i] * inv);
        float z = r * B.diagInvf[i];
        B.rf[i] = r; B.zf[i] = z; B.pf[i] = z; B.xf[i] = 0.f;
        v[0] += (double)r * (double)z;
    }
    gridSum<1>(v, B, [&](double* t) { B.scal[S_RZ] = t[0]; B.flag[3] = 0; });
}
__device__ __forceinline__ float spmvRowF(const PpeBuffers& B, const float* x, int i) {
    return ellRow<float, true>(B.diagf, B.valf, B.col, x, i, __ldg(B.rowLen + i), ellBase(B, i), B.ellStride);
}
__global__ void __launch_bounds__(PBLK) k_mx_spmv(Dev d, PpeBuffers B) {
    if (*(volatile int*)(B.flag + 3)) return;
    int n = liveN(d);
    double v[1] = {0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float ap = spmvRowF(B, B.pf, i);
        B.Apf[i] = ap;
        v[0] += (double)B.pf[i] * (double)ap;
    }
    gridSum<1>(v, B, [&](double* t) { B.scal[S_ALPHA] = B.scal[S_RZ] / t[0]; });
}
// inner tolerance eta on the normalised residual (||rf_0|| = 1)
__global__ void __launch_bounds__(PBLK) k_mx_update(Dev d, PpeBuffers B, double eta2) {
    if (*(volatile int*)(B.flag + 3)) return;
    int n = liveN(d);
    float alpha = (float)B.scal[S_ALPHA];
    double v[2] = {0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float p = B.pf[i];
        B.xf[i] += alpha * p;
        float r = B.rf[i] - alpha * B.Apf[i];
        float z = r * B.diagInvf[i];
        B.rf[i] = r; B.zf[i] = z;
        v[0] += (double)r * (double)z; v[1] += (double)r * (double)r;
    }
    gridSum<2>(v, B, [&](double* t) {
        B.flag[1] += 1;
        B.scal[S_BETA] = t[0] / B.scal[S_RZ];
        B.scal[S_RZ] = t[0];
        if (t[1] < eta2 || !(t[1] == t[1])) B.flag[3] = 1;
    });
}
__global__ void __launch_bounds__(PBLK) k_mx_p(Dev d, PpeBuffers B) {
    if (*(volatile int*)(B.flag + 3)) return;
    int n = liveN(d);
    float beta = (float)B.scal[S_BETA];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        B.pf[i] = B.zf[i] + beta * B.pf[i];
}
// x += ||r|| * d  (FP64)
__global__ void k_mx_correct(Dev d, PpeBuffers B) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    double sc = sqrt(B.scal[S_RR]);
    B.x[i] += sc * (double)B.xf[i];
}

int ppeSolveMixed(const Dev& d, const PpeBuffers& B, double tol, int maxIter, cudaStream_t s,
                  int* iters, int* refinements, double* relres, double* relres0, Prof* prof) {
    int nb = B.nblocks;
    static thread_local int hf[4];
    bool pr = prof && prof->on;
    cudaMemsetAsync(B.flag, 0, 4 * sizeof(int), s);
    if (pr) prof->begin(PROF_PPE_OTHER, s);
    k_mixed_prepare<<<gridFor(d.N0, 256), 256, 0, s>>>(d, B);
    k_mx_residual<<<nb, PBLK, 0, s>>>(d, B, 1, tol);
    if (pr) prof->end(s);
    countLaunch(2);
    int refine = 0, total = 0;
    const double eta = 2e-4;   // inner relative tolerance (FP32 CG stagnates near 1e-6)
    const int batch = 8;
    while (true) {
        if (pollFlags(B, s, hf)) return MPSGPU_ERR_CUDA;
        if (hf[0] || total >= maxIter) break;
        k_mx_inner_init<<<nb, PBLK, 0, s>>>(d, B);
        countLaunch(1);
        int inner = 0;
        while (true) {
            for (int k = 0; k < batch; k++) {
                if (pr) prof->begin(PROF_PPE_SPMV, s);
                k_mx_spmv<<<nb, PBLK, 0, s>>>(d, B);
                if (pr) { prof->end(s); prof->begin(PROF_PPE_VECTOR, s); }
                k_mx_update<<<nb, PBLK, 0, s>>>(d, B, eta * eta);
                k_mx_p<<<nb, PBLK, 0, s>>>(d, B);
                if (pr) prof->end(s);
            }
            countLaunch(3 * batch);
            inner += batch;
            int f4[4];
            if (cudaMemcpyAsync(f4, B.flag, 4 * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return MPSGPU_ERR_CUDA;
            if (cudaStreamSynchronize(s) != cudaSuccess) return MPSGPU_ERR_CUDA;
            if (f4[3] || total + inner >= maxIter || inner >= 400) break;
        }
        total += inner;
        if (pr) prof->begin(PROF_PPE_OTHER, s);
        k_mx_correct<<<gridFor(d.N0, 256), 256, 0, s>>>(d, B);
        k_mx_residual<<<nb, PBLK, 0, s>>>(d, B, 0, tol);
        if (pr) prof->end(s);
        countLaunch(2);
        refine++;
        if (refine > 20) break;
    }
    double sc[S_COUNT];
    cudaMemcpyAsync(sc, B.scal, sizeof(sc), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return MPSGPU_ERR_CUDA;
    *iters = hf[1];
    *refinements = refine;
    double bb = sc[S_BB] > 0 ? sc[S_BB] : 1.0;
    *relres = (sc[S_BB] > 0) ? sqrt(sc[S_RR] / bb) : 0.0;
    *relres0 = sc[S_SCALE];
    if (hf[2] || !hf[0]) return MPSGPU_ERR_NOT_CONVERGED;
    return 0;
}

// ------------------------------------------------------------------ persistent solvers
// The whole solve in one cooperative launch (every block co-resident): no host polling,
// no per-iteration launches.  Each CG iteration is two grid-wide reductions in the form
//   Ap = A z + beta Ap,  p = z + beta p            (one SpMV, on z: A p follows by linearity)
//   x += alpha p, r -= alpha Ap, z = M^-1 r
// so the only vector every block gathers (z) is complete at the reduction before it.
// A reduction is one barrier: every block stores its partial sums, adds one to the
// arrival counter (release) and waits until the counter reaches the generation's target
// (acquire); then every block sums all partials in block order and derives the solver's
// scalars itself.  Identical inputs in identical order give every block identical
// scalars, so no block has to publish them and release the others.  The scalars and flags
// live in shared memory per block; block 0 stores its copy for the host at the end.  Waits are
// bounded: a block that waits longer than QSPIN polls sets the abort word and every
// block returns.
// Block sizes: one block per SM (1024 threads for the mixed solvers at <= 64 registers,
// 768 for the FP64 solvers at <= 80), so a reduction reads 152 partials per value
// instead of 608 (every block reads them all: measured 12 -> 7 us per reduction); the
// staged-tile operator keeps 256-thread blocks (its tiles are one row per thread).
#define QB 256
#define QBX 1024
#define QBC 768
#define QSPIN (1 << 21)
// barrier words, each on its own 128-byte line (the arrival counter is 64-bit and only
// grows within a launch; it is zeroed before each launch): arrivals, unused, abort
#define QB_ARR 0
#define QB_ABT 64
#define QB_WORDS 96

__device__ __forceinline__ double vd(const double* p) { return *(volatile const double*)p; }
__device__ __forceinline__ int vi(const int* p) { return *(volatile const int*)p; }

struct QCtl {
    unsigned int gen;
};
// block-local solver scalars and flags
struct QLocal {
    double scal[32];
    int flag[8];
    float scalf[4];   // FP32 copies of the inner-CG step scalars (SF_*), formed once by thread 0
};
#define SF_ALPHA 0
#define SF_BETA 1
__device__ __forceinline__ void qInit(QLocal& L) {
    for (int t = threadIdx.x; t < 32; t += blockDim.x) L.scal[t] = 0.0;
    for (int t = threadIdx.x; t < 8; t += blockDim.x) L.flag[t] = 0;
    for (int t = threadIdx.x; t < 4; t += blockDim.x) L.scalf[t] = 0.f;
    __syncthreads();
}
__device__ __forceinline__ float vf(const float* p) { return *(volatile const float*)p; }
// block 0's scalars and flags to the global words the host reads
__device__ __forceinline__ void qStore(const PpeBuffers& B, const QLocal& L) {
    __syncthreads();
    if (blockIdx.x == 0) {
        for (int t = threadIdx.x; t < 32; t += blockDim.x) B.scal[t] = L.scal[t];
        for (int t = threadIdx.x; t < 8; t += blockDim.x) B.flag[t] = L.flag[t];
    }
}

// Grid barrier: all writes of the block before it are visible to every block after it.
__device__ __forceinline__ bool qBarrier(const PpeBuffers& B, QCtl& c) {
    __shared__ int sOk;
    __syncthreads();
    c.gen++;
    if (threadIdx.x == 0) {
        unsigned long long* cnt = reinterpret_cast<unsigned long long*>(B.bar + QB_ARR);
        const unsigned long long target = (unsigned long long)c.gen * gridDim.x;
        asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(cnt) : "memory");
        int ok = 1;
        long long spins = 0;
        while (true) {
            unsigned long long v;
            asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(cnt) : "memory");
            if (v >= target) break;
            if (++spins > QSPIN) { atomicExch(B.bar + QB_ABT, 1u); ok = 0; break; }
            if ((spins & 15) == 0 && *(volatile unsigned int*)(B.bar + QB_ABT)) { ok = 0; break; }
            if (spins > 4) __nanosleep(32);
        }
        __threadfence();
        if (ok && *(volatile unsigned int*)(B.bar + QB_ABT)) ok = 0;
        sOk = ok;
    }
    __syncthreads();
    return sOk;
}
// Grid sum of NV (<= 4) FP64 values per thread; fin(tot) runs on thread 0 of every block
// with the same totals, and its writes to the block-local scalars are visible to the
// block's threads on return.  The partials of consecutive reductions alternate between
// two buffers: a block can be at most one reduction ahead of the slowest block's reads.
template <int NV, class Fin>
__device__ __forceinline__ bool qSum(double (&v)[NV], const PpeBuffers& B, QCtl& c, Fin fin) {
    __shared__ double sm[NV * 32];
    blockSum<NV>(v, sm);
    double* part = B.partials + (size_t)(c.gen & 1u) * 4u * gridDim.x;
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < NV; q++) part[q * gridDim.x + blockIdx.x] = v[q];
    if (!qBarrier(B, c)) return false;
    if (threadIdx.x < 32) {   // warp 0: lane-strided partial sums, then a fixed shuffle tree
        double acc[NV];
#pragma unroll
        for (int q = 0; q < NV; q++) {
            double s = 0.0;
            for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) s += ((volatile double*)part)[q * gridDim.x + b];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            acc[q] = s;
        }
        if (threadIdx.x == 0) fin(acc);
    }
    __syncthreads();
    return true;
}
// The same with float-float per-thread partials (FP32 vectors), reduced in float-float all
// the way: the warps' shuffle trees, the block's sum of its warps, the block partials (two
// floats in the same partial slots) and the final sum over the blocks, converted to FP64
// once for fin.  In FP64 the shuffle trees of every warp and the final sum ran on the FP64
// pipe (1/64 of the FP32 rate) between the last arrival and the release of every barrier.
__device__ __forceinline__ df shflXorDF(df a, int o) {
    return {__shfl_xor_sync(0xffffffffu, a.h, o), __shfl_xor_sync(0xffffffffu, a.l, o)};
}
template <int NV, class Fin>
__device__ __forceinline__ bool qSumDF(df (&a)[NV], const PpeBuffers& B, QCtl& c, Fin fin) {
    __shared__ float2 sm[NV * 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; q++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a[q] += shflXorDF(a[q], o);
        if (lane == 0) sm[q * 32 + w] = make_float2(a[q].h, a[q].l);
    }
    __syncthreads();
    float2* part = reinterpret_cast<float2*>(B.partials + (size_t)(c.gen & 1u) * 4u * gridDim.x);
    if (w == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) {
            const float2 x = (lane < nw) ? sm[q * 32 + lane] : make_float2(0.f, 0.f);
            df s = {x.x, x.y};
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += shflXorDF(s, o);
            if (lane == 0) part[q * gridDim.x + blockIdx.x] = make_float2(s.h, s.l);
        }
    }
    if (!qBarrier(B, c)) return false;
    if (threadIdx.x < 32) {   // warp 0: lane-strided partial sums, then a fixed shuffle tree
        double tot[NV];
#pragma unroll
        for (int q = 0; q < NV; q++) {
            df s = dfF(0.f);
            for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) {
                // both floats in one volatile 8-byte load (x at the lower address)
                const unsigned long long u = ((volatile unsigned long long*)part)[q * gridDim.x + b];
                s += df{__uint_as_float((unsigned)u), __uint_as_float((unsigned)(u >> 32))};
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += shflXorDF(s, o);
            tot[q] = dD(s);
        }
        if (threadIdx.x == 0) fin(tot);
    }
    __syncthreads();
    return true;
}

// FP64 per-thread partials summed as float-float from the warp level on (each partial split
// exactly into hi + lo to 48 bits): the per-iteration sums of the plain FP64 CG keep their
// trees off the FP64 pipe.  A tree of float-float sums over the 864k row terms rounds less
// than the sequential FP64 dot product of the reference's solver.
template <int NV, class Fin>
__device__ __forceinline__ bool qSumD(double (&v)[NV], const PpeBuffers& B, QCtl& c, Fin fin) {
    df a[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) a[q] = dfD(v[q]);
    return qSumDF<NV>(a, B, c, fin);
}

// Rows inside the persistent kernels: matrix arrays are read-only for the launch, the
// gathered vector is written by other blocks during it (plain loads, made visible by the
// barrier's fences).  forRows walks a thread's rows with the next row's length prefetched.
template <class F>
__device__ __forceinline__ void forRows(const PpeBuffers& B, int n, int t0, int T, F&& f) {
    int i = t0;
    int len = i < n ? __ldg(B.rowLen + i) : 0;
    while (i < n) {
        int in = i + T;
        int ln = in < n ? __ldg(B.rowLen + in) : 0;
        f(i, len);
        i = in;
        len = ln;
    }
}
// Balanced rows of one thread in the persistent kernels: full rounds of the grid (row =
// m T + b BS + t, T = G BS), then the remainder n - full T split evenly over the blocks, so
// every block gets the same number of rows (+-1 per thread).  A plain grid stride gives
// the first blocks one round more: at 864k rows and 152 x 1024 threads, 84 blocks did 6
// rounds and 68 did 5, and every grid sum waited for the 6-round blocks.
struct RowSet {
    int first, T, full, last;   // rows first + m T (m < full), then last (-1: none)
};
__device__ __forceinline__ RowSet rowSet(int n, int BS) {
    RowSet s;
    const int G = gridDim.x;
    s.T = G * BS;
    s.full = n / s.T;
    s.first = blockIdx.x * BS + threadIdx.x;
    const int rem = n - s.full * s.T;
    const int share = (rem + G - 1) / G;
    const int j = s.full * s.T + blockIdx.x * share + (int)threadIdx.x;
    s.last = ((int)threadIdx.x < share && j < n) ? j : -1;
    return s;
}
__device__ __forceinline__ int rowCount(const RowSet& s) { return s.full + (s.last >= 0 ? 1 : 0); }
__device__ __forceinline__ int rowAt(const RowSet& s, int m) { return m < s.full ? s.first + m * s.T : s.last; }
template <class F>
__device__ __forceinline__ void forOwn(const RowSet& s, F&& f) {
    int i = s.first;
    for (int m = 0; m < s.full; m++, i += s.T) f(i);
    if (s.last >= 0) f(s.last);
}
// The thread's rows in groups of RB: ld(i) for every row of a group (all loads in flight),
// then st(i, v) for each (a load cannot move above a store that may alias it, so a plain
// loop waits one memory latency per row)
template <int RB, class St, class LoadF, class StoreF>
__device__ __forceinline__ void forOwnGroup(const RowSet& s, LoadF&& ld, StoreF&& st) {
    const int cnt = rowCount(s);
    for (int m0 = 0; m0 < cnt; m0 += RB) {
        St v[RB];
        int ii[RB];
#pragma unroll
        for (int u = 0; u < RB; u++) {
            ii[u] = (m0 + u < cnt) ? rowAt(s, m0 + u) : -1;
            v[u] = ld(ii[u] >= 0 ? ii[u] : rowAt(s, m0));   // a valid row either way
        }
#pragma unroll
        for (int u = 0; u < RB; u++)
            if (ii[u] >= 0) st(ii[u], v[u]);
    }
}
// ELL rows with the next row's length prefetched
template <class F>
__device__ __forceinline__ void forRows(const PpeBuffers& B, const RowSet& s, F&& f) {
    const int cnt = rowCount(s);
    int i = cnt > 0 ? rowAt(s, 0) : 0;
    int len = cnt > 0 ? __ldg(B.rowLen + i) : 0;
    for (int m = 0; m < cnt; m++) {
        const int in = (m + 1 < cnt) ? rowAt(s, m + 1) : -1;
        const int ln = in >= 0 ? __ldg(B.rowLen + in) : 0;
        f(i, len);
        i = in;
        len = ln;
    }
}
__device__ __forceinline__ double qRow(const PpeBuffers& B, const double* x, int i, int len) {
    return ellRow<double, false>(B.diag, B.val, B.col, x, i, len, ellBase(B, i), B.ellStride);
}
__device__ __forceinline__ float qRowF(const PpeBuffers& B, const float* x, int i, int len) {
    return ellRow<float, false>(B.diagf, B.valf, B.col, x, i, len, ellBase(B, i), B.ellStride);
}

// Matrix-free FP32 row of the mixed solver's inner operator: the off-diagonal entries
// a_ij = coeffPPE w(r_ij; reL) are recomputed from the hi/lo position copies for the list
// entries that the assembly marked as matrix entries (mfMask), eight neighbours in flight;
// the diagonal is the assembled one.  Only the 4-byte neighbour indices are streamed.
__device__ __forceinline__ float mfWeight(float r2, float re, float invRe, int t) {
    float rinv = rsqrtf(r2);
    switch (t) {
        case 1: { float r = r2 * rinv; return re * rinv + r * invRe - 2.0f; }
        case 2: { float r = r2 * rinv; return re * rinv - r * invRe; }
        case 3: { float a = 1.0f - r2 * rinv * invRe; return a * a * a; }
        case 4: { float a = 1.0f - r2 * rinv * invRe; return a * a; }
        default: return re * rinv - 1.0f;
    }
}
__device__ __forceinline__ float mfRowF(const Dev& d, const PpeBuffers& B, const float* z, int i, float cP, float re,
                                       float invRe, int wt) {
    Mask m = B.mfMask[i];
    const float4 hi = __ldg(d.posf + i), li = __ldg(d.posLo + i);
    const int* row = d.nbr + i;
    const size_t N0 = d.N0;
    float acc[8];
#pragma unroll
    for (int u = 0; u < 8; u++) acc[u] = 0.f;
    while (m.lo | m.hi) {
        int jj[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int k = maskPop(m);
            jj[u] = (k >= 0) ? ldStream(row + (size_t)k * N0) : -1;
        }
#pragma unroll
        for (int u = 0; u < 8; u++) {
            if (jj[u] < 0) continue;
            const int j = jj[u];
            const float4 hj = __ldg(d.posf + j), lj = __ldg(d.posLo + j);
            float dx = (hj.x - hi.x) + (lj.x - li.x);
            float dy = (hj.y - hi.y) + (lj.y - li.y);
            float dz = (hj.z - hi.z) + (lj.z - li.z);
            float w = mfWeight(dx * dx + dy * dy + dz * dz, re, invRe, wt);
            acc[u] += (cP * w) * z[j];
        }
    }
    return __ldg(B.diagf + i) * z[i] + (((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7])));
}

// Compact inner operator: with s_i = 1/sqrt|A_ii| and sigma_i = sign(A_ii), the system
// A d = r is M y = c with M = diag(sigma s) A diag(s), c_i = sigma_i s_i r_i, d = s y.  M is
// symmetric (coupled rows are all equation rows, sigma = -1), has a unit diagonal and
// off-diagonals in (-1, 0): they are stored in FP16 (FP32 arithmetic), the columns as
// 16-bit offsets j - i (rows with a farther neighbour keep the 32-bit columns), 4 bytes
// per entry instead of 8, and CG on M needs no preconditioner.
__device__ __forceinline__ float h16Row(const PpeBuffers& B, const float* y, int i, int len) {
    const size_t N0 = B.ellStride, base = ellBase(B, i);
    const __half* v = B.valh + base;
    float acc[ELL_U];
#pragma unroll
    for (int u = 0; u < ELL_U; u++) acc[u] = 0.f;
    if (!__ldg(B.wideRow + i)) {
        const short* c = B.col16 + base;
        for (int k = 0; k < len; k += ELL_U) {
            if (k + ELL_U < len) {
#pragma unroll
                for (int u = 0; u < ELL_U; u += 2) {
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(c + (size_t)(k + ELL_U + u) * N0));
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(v + (size_t)(k + ELL_U + u) * N0));
                }
            }
            int cc[ELL_U];
            float vv[ELL_U];
#pragma unroll
            for (int u = 0; u < ELL_U; u++) {
                bool ok = k + u < len;
                cc[u] = ok ? i + (int)__ldg(c + (size_t)(k + u) * N0) : i;
                vv[u] = ok ? __half2float(__ldg(v + (size_t)(k + u) * N0)) : 0.f;
            }
#pragma unroll
            for (int u = 0; u < ELL_U; u++) acc[u] += vv[u] * y[cc[u]];
        }
    } else {
        const int* c = B.col + base;
        for (int k = 0; k < len; k += ELL_U) {
            int cc[ELL_U];
            float vv[ELL_U];
#pragma unroll
            for (int u = 0; u < ELL_U; u++) {
                bool ok = k + u < len;
                cc[u] = ok ? ldStream(c + (size_t)(k + u) * N0) : i;
                vv[u] = ok ? __half2float(__ldg(v + (size_t)(k + u) * N0)) : 0.f;
            }
#pragma unroll
            for (int u = 0; u < ELL_U; u++) acc[u] += vv[u] * y[cc[u]];
        }
    }
    return y[i] + (((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7])));
}

// ------------------------------------------------------------------ staged ELL tiles
// The FP32 inner SpMV with the matrix streamed through shared memory: a block owns the
// 256-row tiles t = blockIdx.x + m gridDim.x (the rows its threads own in every other
// phase); each tile's column and value slices (1 KB each, column-major ELL) are copied by
// the bulk-copy engine (cp.async.bulk, completion counted on an mbarrier) in chunks of
// TS_CH slices into a TS_NS-stage ring, up to TS_NS - 1 chunks ahead of the threads, which
// read their row's entries from shared memory and gather z.  The engine keeps the HBM
// stream in flight independently of the threads' gather latencies.  Every mbarrier wait
// is bounded; a wait that runs out sets the abort word (see qBarrier) and the block stops
// consuming, drains the copies it issued (again bounded) and returns at the next barrier.
#define TS_CH 8
#define TS_NS 3
#define TS_SPIN (1 << 20)
struct TsStage {
    int col[TS_CH][QB];
    float val[TS_CH][QB];
};
#define TS_MAXT 128   // tiles per block held in shared memory
struct TsSmem {
    TsStage st[TS_NS];
    unsigned long long full[TS_NS], empty[TS_NS];
    int tlen[TS_MAXT];
};
// bounded wait; false when it ran out
__device__ __forceinline__ bool mbarWait(unsigned long long* b, unsigned parity) { return mbarWaitN(b, parity, TS_SPIN); }
// Chunk walk of a block: its tiles in order (m-th tile = blockIdx.x + m gridDim.x, length
// tlen[m] = longest row), ceil(len / TS_CH) chunks each.
struct TsWalk {
    int m, chunk;
};
__device__ __forceinline__ bool tsNext(const TsSmem& sm, int mt, TsWalk& w) {
    while (w.m < mt) {
        if (w.chunk * TS_CH < sm.tlen[w.m]) return true;
        w.m++;
        w.chunk = 0;
    }
    return false;
}
// issue one chunk (thread 0): slices [c TS_CH, min(L, (c+1) TS_CH)) of the walk's tile
__device__ __forceinline__ void tsIssue(TsSmem& sm, const PpeBuffers& B, const TsWalk& w, unsigned q, bool& ok) {
    const int s = q % TS_NS;
    const unsigned use = q / TS_NS;
    if (use > 0 && !mbarWait(&sm.empty[s], (use - 1) & 1)) { ok = false; return; }
    const int L = sm.tlen[w.m];
    const int k0 = w.chunk * TS_CH, nsl = min(TS_CH, L - k0);
    const size_t r0 = (size_t)(blockIdx.x + w.m * gridDim.x) * QB;
    mbarExpectTx(&sm.full[s], (unsigned)(nsl * QB * (sizeof(int) + sizeof(float))));
    for (int u = 0; u < nsl; u++) {   // a tile's QB rows lie in one slice (the slice height is a multiple of QB)
        size_t e = ellBase(B, (int)r0) + (size_t)(k0 + u) * B.ellStride;
        bulkG2S(sm.st[s].col[u], B.col + e, QB * sizeof(int), &sm.full[s]);
        bulkG2S(sm.st[s].val[u], B.valf + e, QB * sizeof(float), &sm.full[s]);
    }
}

// One staged SpMV pass over the block's tiles: y_i = A_ii z_i + sum_k valf z[col] for the
// thread's row of every tile, then rowDone(i, y_i) (rows below the live count only).
// gq counts the chunks consumed, the same in every thread; returns false when a wait ran
// out (the abort word is then set; the copies issued are drained, bounded, before return).
template <class F>
__device__ __forceinline__ bool tsSpmv(TsSmem& sm, const PpeBuffers& B, const float* z, int n, int mt, unsigned& gq,
                                       F&& rowDone) {
    bool ok = true;
    TsWalk prod = {0, 0};
    unsigned qp = gq, q = gq;
    if (threadIdx.x == 0)
        for (int k = 0; k < TS_NS - 1 && ok && tsNext(sm, mt, prod); k++) { tsIssue(sm, B, prod, qp, ok); qp++; prod.chunk++; }
    for (int m = 0; m < mt; m++) {
        const int row = (blockIdx.x + m * gridDim.x) * QB + threadIdx.x;
        const int len = (row < n) ? __ldg(B.rowLen + row) : 0;
        const int L = sm.tlen[m];
        float acc[TS_CH];
#pragma unroll
        for (int u = 0; u < TS_CH; u++) acc[u] = 0.f;
        for (int c = 0; c * TS_CH < L; c++) {
            if (threadIdx.x == 0 && ok && tsNext(sm, mt, prod)) { tsIssue(sm, B, prod, qp, ok); qp++; prod.chunk++; }
            const int st = q % TS_NS;
            bool got = ok && mbarWait(&sm.full[st], (q / TS_NS) & 1);
            got = __all_sync(0xffffffffu, got);
            if (got) {
                const int k0 = c * TS_CH;
#pragma unroll
                for (int u = 0; u < TS_CH; u++)
                    if (k0 + u < len) acc[u] += sm.st[st].val[u][threadIdx.x] * z[sm.st[st].col[u][threadIdx.x]];
            } else {
                ok = false;
            }
            __syncwarp();
            if ((threadIdx.x & 31) == 0) mbarArrive(&sm.empty[st]);
            q++;
        }
        if (row < n)
            rowDone(row, __ldg(B.diagf + row) * z[row] +
                             (((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]))));
    }
    // a wait that ran out: stop, and let the copies this block issued land before leaving
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) {
            atomicExch(B.bar + QB_ABT, 1u);
            for (unsigned k = q; k < qp; k++) mbarWait(&sm.full[k % TS_NS], (k / TS_NS) & 1);
        }
        __syncthreads();
        return false;
    }
    gq = q;
    return true;
}

// Mixed solver: FP64 residual r = b - A x and its norm, FP32 inner CG on r / ||r|| to
// the relative tolerance eta_k, x += ||r|| d in FP64, repeated until ||r|| < tol ||b||.
// eta_k = max(eta, tol ||b|| / (2 ||r_k||)): an inner solve stops once its correction
// brings the outer residual to half the tolerance, so the last one does not over-solve;
// eta = 1e-6 is near the FP32 recurrence's attainable accuracy.
// Inner operator of k_mx_solve: the assembled FP32 ELL matrix with Jacobi preconditioning,
// the matrix-free FP32 operator with Jacobi preconditioning, or the compact scaled operator.
enum { OP_ELL32 = 0, OP_MATFREE = 1, OP_H16 = 2, OP_TILED = 3 };
template <int OP>
__global__ void __launch_bounds__(OP == 3 ? QB : QBX, OP == 3 ? 4 : 1) k_mx_solve(Dev d, PpeBuffers B, double tol, int maxIter, double eta2) {
    __shared__ QLocal qL;   // this block's copy of the solver scalars and flags
    qInit(qL);
    double* const qS = qL.scal;
    int* const qF = qL.flag;
    extern __shared__ __align__(128) unsigned char dynSmem[];
    const int n = liveN(d);
    const float cP = (float)d.P.coeffPPE, re = (float)d.P.reL, invRe = (float)(1.0 / d.P.reL);
    const int wt = d.P.weightType;
    // grid-stride rounds (at any moment the blocks work on one contiguous window of rows,
    // so the column slices of the ELL arrays stream through DRAM pages in order), the
    // remainder split evenly over the blocks
    constexpr int BS = (OP == OP_TILED) ? QB : QBX;
    const RowSet rs = rowSet(n, BS);   // this thread's rows
    QCtl c = {0u};
    // staged tiles: the block's tile lengths and the mbarriers of the ring
    TsSmem& sm = *reinterpret_cast<TsSmem*>(dynSmem);
    const int ntiles = (n + QB - 1) / QB;
    const int mt = (ntiles > (int)blockIdx.x) ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    unsigned gq = 0u;   // chunks consumed so far (the same count in every thread of the block)
    if (OP == OP_TILED) {
        if (threadIdx.x == 0) {
            for (int st = 0; st < TS_NS; st++) {
                mbarInit(&sm.full[st], 1u);
                mbarInit(&sm.empty[st], QB / 32);
            }
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        for (int m = threadIdx.x; m < TS_MAXT; m += QB) sm.tlen[m] = 0;
        __syncthreads();
        for (int m = 0; m < mt; m++) {
            const int row = (blockIdx.x + m * gridDim.x) * QB + threadIdx.x;
            int len = (row < n) ? __ldg(B.rowLen + row) : 0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) len = max(len, __shfl_xor_sync(0xffffffffu, len, o));
            if ((threadIdx.x & 31) == 0) atomicMax(&sm.tlen[m], len);
        }
        __syncthreads();
    }
    if (OP == OP_H16) {
        // scaling, then the compact copy of the FP32 matrix
        forOwn(rs, [&](int i) {
            double dd = __ldg(B.diag + i);
            double sc = 1.0 / sqrt(fabs(dd));
            B.sclf[i] = (float)sc;
            B.sgs[i] = (float)(dd < 0.0 ? -sc : sc);
        });
        if (!qBarrier(B, c)) return;
        forRows(B, rs, [&](int i, int len) {
            const float si = B.sgs[i];
            unsigned char wide = 0;
            const size_t base = ellBase(B, i);
            for (int k = 0; k < len; k++) {
                size_t e = base + (size_t)k * B.ellStride;
                int j = __ldg(B.col + e);
                B.valh[e] = __float2half_rn(si * __ldg(B.valf + e) * B.sclf[j]);
                int off = j - i;
                if (off < -32768 || off > 32767) wide = 1;
                B.col16[e] = (short)off;
            }
            B.wideRow[i] = wide;
        });
        if (!qBarrier(B, c)) return;
    }
    {
        double v[2] = {0.0, 0.0};
        forRows(B, rs, [&](int i, int len) {
            double r = B.b[i] - qRow(B, B.x, i, len);
            B.r[i] = r;
            v[0] += r * r;
            v[1] += B.b[i] * B.b[i];
        });
        if (!qSum<2>(v, B, c, [&](const double* t) {
                qS[S_RR] = t[0];
                qS[S_BB] = t[1];
                double thr = tol * tol * t[1];
                if (thr < 2.2250738585072014e-308) thr = 2.2250738585072014e-308;
                qS[S_THR] = thr;
                qS[S_SCALE] = sqrt(t[0] / (t[1] > 0 ? t[1] : 1.0));
                qS[S_SQRT] = sqrt(t[0]);
                qS[S_INV] = 1.0 / sqrt(t[0]);
                qS[S_ETA2] = fmax(eta2, 0.25 * thr / t[0]);
                qF[0] = (t[1] == 0.0 || t[0] < thr) ? 1 : 0;
                qF[1] = 0;
                qF[3] = 0;
                if (!(t[0] == t[0])) { qF[0] = 1; qF[2] = 1; }
            }))
            return;
    }
    int total = 0, refine = 0;
    while (!vi(qF) && total < maxIter && refine <= 20) {
        // inner start: rf = r / ||r|| (compact operator: sigma s r / ||r||), z = M^-1 rf, x_f = 0
        {
            const double inv = vd(qS + S_INV);
            df a[2] = {dfF(0.f), dfF(0.f)};
            forOwn(rs, [&](int i) {
                float r = (float)(B.r[i] * inv);
                if (OP == OP_H16) r *= B.sgs[i];
                float z = (OP == OP_H16) ? r : r * __ldg(B.diagInvf + i);
                B.rf[i] = r; B.zf[i] = z; B.xf[i] = 0.f;
                a[0] += prod2(r, z);
                a[1] += prod2(r, r);
            });
            if (!qSumDF<2>(a, B, c, [&](const double* t) { qS[S_RZ] = t[0]; qS[S_RR0] = t[1]; qF[3] = 0; }))
                return;
        }
        int inner = 0;
        while (true) {
            {
                const float beta = inner ? (float)vd(qS + S_BETA) : 0.f;
                df a[1] = {dfF(0.f)};
                if (OP == OP_TILED) {
                    bool okp = tsSpmv(sm, B, B.zf, n, mt, gq, [&](int i, float q) {
                        float z = B.zf[i];
                        float ap = inner ? q + beta * B.Apf[i] : q;
                        float p = inner ? z + beta * B.pf[i] : z;
                        B.Apf[i] = ap; B.pf[i] = p;
                        a[0] += prod2(p, ap);
                    });
                    (void)okp;   // an ran-out wait sets the abort word: the reduction below returns false
                } else forRows(B, rs, [&](int i, int len) {
                    float q = (OP == OP_MATFREE) ? mfRowF(d, B, B.zf, i, cP, re, invRe, wt)
                            : (OP == OP_H16)   ? h16Row(B, B.zf, i, len)
                                               : qRowF(B, B.zf, i, len);
                    float z = B.zf[i];
                    float ap = inner ? q + beta * B.Apf[i] : q;
                    float p = inner ? z + beta * B.pf[i] : z;
                    B.Apf[i] = ap; B.pf[i] = p;
                    a[0] += prod2(p, ap);
                });
                if (!qSumDF<1>(a, B, c, [&](const double* t) { qS[S_PAP] = t[0]; qS[S_ALPHA] = qS[S_RZ] / t[0]; }))
                    return;
            }
            {
                const float alpha = (float)vd(qS + S_ALPHA);
                df a[2] = {dfF(0.f), dfF(0.f)};
                struct VR { float x, p, r, q, m; };
                forOwnGroup<3, VR>(rs, [&](int i) {
                    VR v;
                    v.x = B.xf[i]; v.p = B.pf[i]; v.r = B.rf[i]; v.q = B.Apf[i];
                    v.m = (OP == OP_H16) ? 1.f : __ldg(B.diagInvf + i);
                    return v;
                }, [&](int i, const VR& v) {
                    const float r = v.r - alpha * v.q;
                    const float z = (OP == OP_H16) ? r : r * v.m;
                    B.xf[i] = v.x + alpha * v.p; B.rf[i] = r; B.zf[i] = z;
                    a[0] += prod2(r, z);
                    a[1] += prod2(r, r);
                });
                if (!qSumDF<2>(a, B, c, [&](const double* t) {
                        qF[1] += 1;
                        qS[S_BETA] = t[0] / qS[S_RZ];
                        qS[S_RZ] = t[0];
                        if (t[1] < qS[S_ETA2] * qS[S_RR0] || !(t[1] == t[1])) qF[3] = 1;
                    }))
                    return;
            }
            inner++;
            if (vi(qF + 3) || total + inner >= maxIter || inner >= 400) break;
        }
        total += inner;
        {
            const double sc = vd(qS + S_SQRT);
            forOwn(rs, [&](int i) {
                B.x[i] += sc * (double)((OP == OP_H16) ? B.xf[i] * B.sclf[i] : B.xf[i]);
            });
            if (!qBarrier(B, c)) return;
        }
        {
            double v[1] = {0.0};
            forRows(B, rs, [&](int i, int len) {
                double r = B.b[i] - qRow(B, B.x, i, len);
                B.r[i] = r;
                v[0] += r * r;
            });
            if (!qSum<1>(v, B, c, [&](const double* t) {
                    qS[S_RR] = t[0];
                    qS[S_SQRT] = sqrt(t[0]);
                    qS[S_INV] = 1.0 / sqrt(t[0]);
                    qS[S_ETA2] = fmax(eta2, 0.25 * qS[S_THR] / t[0]);
                    if (t[0] < qS[S_THR]) qF[0] = 1;
                    if (!(t[0] == t[0])) { qF[0] = 1; qF[2] = 1; }
                    qF[4] += 1;
                }))
                return;
        }
        refine++;
    }
    qStore(B, qL);
}

// ------------------------------------------------------------------ shared-memory vectors
// The mixed solver with the FP32 inner-CG vectors of each block's rows (x, r, p, Ap: 16
// bytes per row) in shared memory from the first inner iteration to the last; only z, the
// vector every block gathers through the matrix columns, goes through global memory.  A
// block's rows are those of the grid-stride rounds (RowSet: at any moment all blocks
// stream adjacent slices of the column-major ELL arrays, which measured 28% faster than one
// contiguous range per block), and the m-th row of thread t sits at slot m BS + t of the
// block's vectors.  The vector pass of an iteration is then shared-memory work plus one
// coalesced store of z.
#define OWN_CAPMAX OWN_CAP_ROWS   // slots per block: 4 x 13312 x 4 B = 208 KB of shared memory

// The thread's rows of a RowSet with their shared-memory slot l = m BS + t (m-th row of the
// thread), f(l, i, len) with the next row's length prefetched; forOwnL without the length.
template <class F>
__device__ __forceinline__ void forRowsL(const PpeBuffers& B, const RowSet& s, F&& f) {
    const int cnt = rowCount(s);
    int i = cnt > 0 ? rowAt(s, 0) : 0;
    int len = cnt > 0 ? __ldg(B.rowLen + i) : 0;
    for (int m = 0; m < cnt; m++) {
        const int in = (m + 1 < cnt) ? rowAt(s, m + 1) : -1;
        const int ln = in >= 0 ? __ldg(B.rowLen + in) : 0;
        f(m * (int)blockDim.x + (int)threadIdx.x, i, len);
        i = in;
        len = ln;
    }
}
template <class F>
__device__ __forceinline__ void forOwnL(const RowSet& s, F&& f) {
    const int cnt = rowCount(s);
    for (int m = 0; m < cnt; m++) f(m * (int)blockDim.x + (int)threadIdx.x, rowAt(s, m));
}

// Set-up of the shared-memory mixed solve: FP64 residual of the warm start, ||r||^2 and
// ||b||^2 and the solver scalars; with a learned correction c (B.cdir, with q = A c in
// B.cq) the residual r_e of the start x_e is already in B.r (the learned start's features
// read it), and the pass forms the dot products r.q and q.q, the residual-minimising step
// theta = r.q / q.q (the start x + theta c is never worse than x in the residual norm; its
// residual norm follows algebraically) and the update of x and r.  Returns false when a
// barrier wait ran out.
template <bool LEARNED>
__device__ __forceinline__ bool mxSetup(const PpeBuffers& B, const RowSet& rs, QCtl& c, QLocal& qL, double tol,
                                        double eta2) {
    double* const qS = qL.scal;
    int* const qF = qL.flag;
    double v[LEARNED ? 4 : 2] = {};
    if (LEARNED) {
        forOwn(rs, [&](int i) {
            const double bi = B.b[i], r = B.r[i];
            const double q = (double)__ldg(B.cq + i);
            v[0] += r * r;
            v[1] += bi * bi;
            v[LEARNED ? 2 : 0] += r * q;
            v[LEARNED ? 3 : 0] += q * q;
        });
    } else {
        forRows(B, rs, [&](int i, int len) {
            const double bi = B.b[i];
            const double r = bi - qRow(B, B.x, i, len);
            B.r[i] = r;
            v[0] += r * r;
            v[1] += bi * bi;
        });
    }
    if (!qSum<LEARNED ? 4 : 2>(v, B, c, [&](const double* t) {
            double th = 0.0, rr = t[0];
            if (LEARNED) {
                // a non-finite correction keeps the start x (theta = 0, its residual as is)
                const double rq = t[LEARNED ? 2 : 0], qq = t[LEARNED ? 3 : 0];
                if (qq > 0.0 && qq < 1.0 / 0.0 && rq == rq && fabs(rq) < 1.0 / 0.0) {
                    th = rq / qq;
                    rr = fmax(t[0] - th * rq, 0.0);
                }
            }
            qS[S_OMEGA] = th;
            qS[S_RR] = rr;
            qS[S_BB] = t[1];
            double thr = tol * tol * t[1];
            if (thr < 2.2250738585072014e-308) thr = 2.2250738585072014e-308;
            qS[S_THR] = thr;
            qS[S_SCALE] = sqrt(rr / (t[1] > 0 ? t[1] : 1.0));
            qS[S_SQRT] = sqrt(rr);
            qS[S_INV] = 1.0 / sqrt(rr);
            qS[S_ETA2] = fmax(eta2, 0.25 * thr / rr);
            qF[0] = (t[1] == 0.0 || rr < thr) ? 1 : 0;
            qF[1] = 0;
            qF[3] = 0;
            if (!(rr == rr)) { qF[0] = 1; qF[2] = 1; }
        }))
        return false;
    if (LEARNED && vd(qS + S_OMEGA) != 0.0) {   // x += theta c, r -= theta q on the thread's own rows
        const double th = vd(qS + S_OMEGA);
        forOwn(rs, [&](int i) {
            B.x[i] += th * (double)__ldg(B.cdir + i);
            B.r[i] -= th * (double)__ldg(B.cq + i);
        });
    }
    return true;
}

template <bool LEARNED>
__global__ void __launch_bounds__(QBX, 1) k_mx_own(Dev d, PpeBuffers B, double tol, int maxIter, double eta2, int cap) {
    __shared__ QLocal qL;   // this block's copy of the solver scalars and flags
    qInit(qL);
    double* const qS = qL.scal;
    int* const qF = qL.flag;
    extern __shared__ __align__(128) unsigned char dynSmem[];
    float* const sx = reinterpret_cast<float*>(dynSmem);   // inner correction x_f
    float* const sr = sx + cap;                             // inner residual
    float* const sp = sr + cap;                             // search direction
    float* const sap = sp + cap;                            // A p
    const int n = liveN(d);
    const RowSet rs = rowSet(n, QBX);   // this thread's rows (rowCount(rs) * QBX <= cap)
    QCtl c = {0u};
    if (!mxSetup<LEARNED>(B, rs, c, qL, tol, eta2)) return;
    int total = 0, refine = 0;
    while (!vi(qF) && total < maxIter && refine <= 20) {
        {   // inner start: r_f = r / ||r||, z = M^-1 r_f, x_f = 0
            const double inv = vd(qS + S_INV);
            df a[2] = {dfF(0.f), dfF(0.f)};
            forOwnL(rs, [&](int l, int i) {
                const float r = (float)(B.r[i] * inv);
                const float z = r * __ldg(B.diagInvf + i);
                sr[l] = r; sx[l] = 0.f;
                B.zf[i] = z;
                a[0] += prod2(r, z);
                a[1] += prod2(r, r);
            });
            if (!qSumDF<2>(a, B, c, [&](const double* t) { qS[S_RZ] = t[0]; qS[S_RR0] = t[1]; qF[3] = 0; }))
                return;
        }
        int inner = 0;
        while (true) {
            {   // Ap = A z + beta Ap, p = z + beta p, p.Ap
                const float beta = inner ? vf(qL.scalf + SF_BETA) : 0.f;
                df a[1] = {dfF(0.f)};
                forRowsL(B, rs, [&](int l, int i, int len) {
                    const float q = qRowF(B, B.zf, i, len);
                    const float z = B.zf[i];
                    const float ap = inner ? q + beta * sap[l] : q;
                    const float p = inner ? z + beta * sp[l] : z;
                    sap[l] = ap; sp[l] = p;
                    a[0] += prod2(p, ap);
                });
                if (!qSumDF<1>(a, B, c, [&](const double* t) {
                        qS[S_PAP] = t[0];
                        qS[S_ALPHA] = qS[S_RZ] / t[0];
                        qL.scalf[SF_ALPHA] = d2fRN(qS[S_ALPHA]);
                    }))
                    return;
            }
            {   // x_f += alpha p, r -= alpha Ap, z = M^-1 r; r.z, r.r
                const float alpha = vf(qL.scalf + SF_ALPHA);
                df a[2] = {dfF(0.f), dfF(0.f)};
                const int cnt = rowCount(rs);
                for (int m0 = 0; m0 < cnt; m0 += 4) {
                    float mi[4];
                    int ii[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        ii[u] = (m0 + u < cnt) ? rowAt(rs, m0 + u) : -1;
                        mi[u] = (ii[u] >= 0) ? __ldg(B.diagInvf + ii[u]) : 0.f;
                    }
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        if (ii[u] < 0) continue;
                        const int l = (m0 + u) * (int)blockDim.x + (int)threadIdx.x;
                        const float r = sr[l] - alpha * sap[l];
                        const float z = r * mi[u];
                        sx[l] += alpha * sp[l];
                        sr[l] = r;
                        B.zf[ii[u]] = z;
                        a[0] += prod2(r, z);
                        a[1] += prod2(r, r);
                    }
                }
                if (!qSumDF<2>(a, B, c, [&](const double* t) {
                        qF[1] += 1;
                        qS[S_BETA] = t[0] / qS[S_RZ];
                        qL.scalf[SF_BETA] = d2fRN(qS[S_BETA]);
                        qS[S_RZ] = t[0];
                        if (t[1] < qS[S_ETA2] * qS[S_RR0] || !(t[1] == t[1])) qF[3] = 1;
                    }))
                    return;
            }
            inner++;
            if (vi(qF + 3) || total + inner >= maxIter || inner >= 400) break;
        }
        total += inner;
        {   // x += ||r|| x_f (FP64)
            const double sc = vd(qS + S_SQRT);
            forOwnL(rs, [&](int l, int i) { B.x[i] += sc * (double)sx[l]; });
            if (!qBarrier(B, c)) return;
        }
        {   // FP64 residual r = b - A x
            double v[1] = {0.0};
            forRows(B, rs, [&](int i, int len) {
                const double r = B.b[i] - qRow(B, B.x, i, len);
                B.r[i] = r;
                v[0] += r * r;
            });
            if (!qSum<1>(v, B, c, [&](const double* t) {
                    qS[S_RR] = t[0];
                    qS[S_SQRT] = sqrt(t[0]);
                    qS[S_INV] = 1.0 / sqrt(t[0]);
                    qS[S_ETA2] = fmax(eta2, 0.25 * qS[S_THR] / t[0]);
                    if (t[0] < qS[S_THR]) qF[0] = 1;
                    if (!(t[0] == t[0])) { qF[0] = 1; qF[2] = 1; }
                    qF[4] += 1;
                }))
                return;
        }
        refine++;
    }
    qStore(B, qL);
}

// FP64 residual row of the refinement without a pass in between: x_j + d_j is formed from
// the FP64 iterate and the FP32 correction of the inner solve as the owner of j forms it.
__device__ __forceinline__ double qRowPlus(const PpeBuffers& B, const double* x, const float* dx, int i, int len) {
    double acc[ELL_U];
#pragma unroll
    for (int u = 0; u < ELL_U; u++) acc[u] = 0.0;
    const size_t base = ellBase(B, i), N0 = B.ellStride;
    const double* v = B.val + base;
    const int* c = B.col + base;
    for (int k = 0; k < len; k += ELL_U) {
        int cc[ELL_U];
        double vv[ELL_U];
#pragma unroll
        for (int u = 0; u < ELL_U; u++) {
            bool ok = k + u < len;
            cc[u] = ok ? ldStream(c + (size_t)(k + u) * N0) : i;
            vv[u] = ok ? ldStream(v + (size_t)(k + u) * N0) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < ELL_U; u++) acc[u] += vv[u] * (x[cc[u]] + (double)dx[cc[u]]);
    }
    return __ldg(B.diag + i) * (x[i] + (double)dx[i]) +
           (((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7])));
}

// Mixed solver with the pipelined inner CG (Ghysels & Vanroose, "Hiding global
// synchronization latency in the preconditioned Conjugate Gradient algorithm", Parallel
// Computing 40, 2014, Alg. 3), Jacobi M = diag^-1 applied on the fly: with u = M r,
// q = M s and m = M w recomputed from r, s and w, the recurrences kept are
//   z = A m + beta z,  s = w + beta s,  p = M r + beta p,  x += alpha p,
//   r -= alpha s,      w -= alpha z,    m' = M w
// and the three dot products (r.u, w.u, r.r) of the next iteration are summed in the same
// pass: one grid barrier per inner iteration (the standard form needs two).  m is double
// buffered (its owner writes m' while neighbours gather m).  The FP64 refinement forms
// r = b - A (x + d) in the pass that stores x + d into the other FP64 buffer, and starts
// the next inner solve there (u0 = M r), so a refinement costs two barriers.
__global__ void __launch_bounds__(QBX, 1) k_mx_pipe(Dev d, PpeBuffers B, double tol, int maxIter, double eta2) {
    __shared__ QLocal qL;   // this block's copy of the solver scalars and flags
    qInit(qL);
    double* const qS = qL.scal;
    int* const qF = qL.flag;
    const int n = liveN(d);
    const RowSet rs = rowSet(n, QBX);   // this thread's rows
    QCtl c = {0u};
    double* xa = B.x;      // current FP64 iterate
    double* xb = B.xalt;   // the next one
    float* mA = B.zf;      // u0, then m of odd iterations
    float* mB = B.mf2;     // m of even iterations
    {
        double v[2] = {0.0, 0.0};
        forRows(B, rs, [&](int i, int len) {
            double r = B.b[i] - qRow(B, xa, i, len);
            B.r[i] = r;
            float rf = (float)r;
            B.rf[i] = rf;
            mA[i] = rf * __ldg(B.diagInvf + i);
            v[0] += r * r;
            v[1] += B.b[i] * B.b[i];
        });
        if (!qSum<2>(v, B, c, [&](const double* t) {
                qS[S_RR] = t[0];
                qS[S_BB] = t[1];
                double thr = tol * tol * t[1];
                if (thr < 2.2250738585072014e-308) thr = 2.2250738585072014e-308;
                qS[S_THR] = thr;
                qS[S_SCALE] = sqrt(t[0] / (t[1] > 0 ? t[1] : 1.0));
                qS[S_ETA2] = fmax(eta2, 0.25 * thr / t[0]);
                qF[0] = (t[1] == 0.0 || t[0] < thr) ? 1 : 0;
                qF[1] = 0;
                if (!(t[0] == t[0])) { qF[0] = 1; qF[2] = 1; }
            }))
            return;
    }
    int total = 0, refine = 0;
    while (!vi(qF) && total < maxIter && refine <= 20) {
        // inner start: w0 = A u0, m0 = M w0; gamma0 = r.u, delta0 = w.u, rho0 = r.r
        {
            df a[3] = {dfF(0.f), dfF(0.f), dfF(0.f)};
            forRows(B, rs, [&](int i, int len) {
                const float w = qRowF(B, mA, i, len);
                const float u = mA[i], r = B.rf[i];
                B.wf[i] = w;
                mB[i] = w * __ldg(B.diagInvf + i);
                a[0] += prod2(r, u);
                a[1] += prod2(w, u);
                a[2] += prod2(r, r);
            });
            if (!qSumDF<3>(a, B, c, [&](const double* t) {
                    qF[3] = 0;
                    qS[S_RZ] = t[0];
                    qS[S_RR0] = t[2];
                    qS[S_BETA] = 0.0;
                    // the PPE matrix and its Jacobi preconditioner are negative definite:
                    // r.u and w.u share their sign and alpha > 0
                    const double al = t[0] / t[1];
                    if (al > 0.0 && al < 1e300) qS[S_ALPHA] = al;
                    else qF[3] = 1;   // zero residual or breakdown: nothing to solve
                }))
                return;
        }
        int inner = 0;
        while (!vi(qF + 3) && total + inner < maxIter && inner < 400) {
            const float alpha = (float)vd(qS + S_ALPHA), beta = (float)vd(qS + S_BETA);
            const float* mc = (inner & 1) ? mA : mB;
            float* mn = (inner & 1) ? mB : mA;
            const bool first = inner == 0;
            df a[3] = {dfF(0.f), dfF(0.f), dfF(0.f)};
            forRows(B, rs, [&](int i, int len) {
                const float an = qRowF(B, mc, i, len);   // A m
                const float di = __ldg(B.diagInvf + i);
                float w = B.wf[i], r = B.rf[i];
                float z = first ? an : an + beta * B.qzf[i];
                float sv = first ? w : w + beta * B.Apf[i];
                float p = first ? r * di : r * di + beta * B.pf[i];
                float x = first ? alpha * p : B.xf[i] + alpha * p;
                r -= alpha * sv;
                w -= alpha * z;
                B.qzf[i] = z; B.Apf[i] = sv; B.pf[i] = p; B.xf[i] = x;
                B.rf[i] = r; B.wf[i] = w;
                const float u = r * di;
                mn[i] = w * di;
                a[0] += prod2(r, u);
                a[1] += prod2(w, u);
                a[2] += prod2(r, r);
            });
            if (!qSumDF<3>(a, B, c, [&](const double* t) {
                    qF[1] += 1;
                    if (t[2] < qS[S_ETA2] * qS[S_RR0] || !(t[2] == t[2])) { qF[3] = 1; return; }
                    const double g0 = qS[S_RZ], al = qS[S_ALPHA];
                    const double bt = t[0] / g0;
                    const double aln = t[0] / (t[1] - bt * t[0] / al);
                    if (!(aln > 0.0 && aln < 1e300 && bt >= 0.0)) { qF[3] = 1; return; }
                    qS[S_BETA] = bt;
                    qS[S_ALPHA] = aln;
                    qS[S_RZ] = t[0];
                }))
                return;
            inner++;
        }
        total += inner;
        // refinement: x' = x + d into the other buffer, r = b - A x', next inner start u0
        {
            const bool any = inner > 0;
            double v[1] = {0.0};
            forRows(B, rs, [&](int i, int len) {
                double r;
                if (any) {
                    xb[i] = xa[i] + (double)B.xf[i];
                    r = B.b[i] - qRowPlus(B, xa, B.xf, i, len);
                } else {
                    xb[i] = xa[i];
                    r = B.r[i];
                }
                B.r[i] = r;
                float rf = (float)r;
                B.rf[i] = rf;
                mA[i] = rf * __ldg(B.diagInvf + i);
                v[0] += r * r;
            });
            if (!qSum<1>(v, B, c, [&](const double* t) {
                    qS[S_RR] = t[0];
                    qS[S_ETA2] = fmax(eta2, 0.25 * qS[S_THR] / t[0]);
                    if (t[0] < qS[S_THR]) qF[0] = 1;
                    if (!(t[0] == t[0])) { qF[0] = 1; qF[2] = 1; }
                    qF[4] += 1;
                }))
                return;
            double* tx = xa; xa = xb; xb = tx;
        }
        refine++;
    }
    if (xa != B.x)
        forOwn(rs, [&](int i) { B.x[i] = xa[i]; });
    qStore(B, qL);
}

// Plain FP64 Jacobi-PCG (Eigen's ConjugateGradient with its diagonal preconditioner,
// src/MpsPressure.cpp:424-445): z = invdiag * r, stop when ||r||^2 < tol^2 ||b||^2.
__global__ void __launch_bounds__(QBC, 1) k_cg_solve(Dev d, PpeBuffers B, double tol, int maxIter) {
    __shared__ QLocal qL;   // this block's copy of the solver scalars and flags
    qInit(qL);
    double* const qS = qL.scal;
    int* const qF = qL.flag;
    const int n = liveN(d);
    // grid-stride rounds (at any moment the blocks work on one contiguous window of rows,
    // so the column slices of the ELL arrays stream through DRAM pages in order), the
    // remainder split evenly over the blocks
    const RowSet rs = rowSet(n, QBC);   // this thread's rows
    QCtl c = {0u};
    {
        double v[3] = {0.0, 0.0, 0.0};
        forRows(B, rs, [&](int i, int len) {
            double di = 1.0 / __ldg(B.diag + i);
            double r = B.b[i] - qRow(B, B.x, i, len);
            double z = r * di;
            B.dinv[i] = di; B.r[i] = r; B.z[i] = z;
            v[0] += r * z; v[1] += r * r; v[2] += B.b[i] * B.b[i];
        });
        if (!qSum<3>(v, B, c, [&](const double* t) {
                qS[S_RZ] = t[0]; qS[S_RR] = t[1]; qS[S_BB] = t[2];
                double thr = tol * tol * t[2];
                if (thr < 2.2250738585072014e-308) thr = 2.2250738585072014e-308;
                qS[S_THR] = thr;
                qS[S_SCALE] = sqrt(t[1] / (t[2] > 0 ? t[2] : 1.0));
                qF[0] = (t[2] == 0.0 || t[1] < thr) ? 1 : 0;
                qF[1] = 0;
                if (!(t[0] == t[0]) || !(t[1] == t[1])) { qF[0] = 1; qF[2] = 1; }
            }))
            return;
    }
    int it = 0;
    while (!vi(qF) && it < maxIter) {
        {
            const double beta = it ? vd(qS + S_BETA) : 0.0;
            double v[1] = {0.0};
            forRows(B, rs, [&](int i, int len) {
                double q = qRow(B, B.z, i, len);
                double z = B.z[i];
                double ap = it ? q + beta * B.Ap[i] : q;
                double p = it ? z + beta * B.p[i] : z;
                B.Ap[i] = ap; B.p[i] = p;
                v[0] += p * ap;
            });
            if (!qSum<1>(v, B, c, [&](const double* t) { qS[S_PAP] = t[0]; qS[S_ALPHA] = qS[S_RZ] / t[0]; }))
                return;
        }
        {
            const double alpha = vd(qS + S_ALPHA);
            double v[2] = {0.0, 0.0};
            struct VR { double x, p, r, q, m; };
            forOwnGroup<4, VR>(rs, [&](int i) {
                VR w;
                w.x = B.x[i]; w.p = B.p[i]; w.r = B.r[i]; w.q = B.Ap[i]; w.m = B.dinv[i];
                return w;
            }, [&](int i, const VR& w) {
                const double r = w.r - alpha * w.q;
                const double z = r * w.m;
                B.x[i] = w.x + alpha * w.p; B.r[i] = r; B.z[i] = z;
                v[0] += r * z; v[1] += r * r;
            });
            if (!qSum<2>(v, B, c, [&](const double* t) {
                    qF[1] += 1;
                    qS[S_RR] = t[1];
                    qS[S_BETA] = t[0] / qS[S_RZ];
                    qS[S_RZ] = t[0];
                    if (t[1] < qS[S_THR]) qF[0] = 1;
                    if (!(t[1] == t[1])) { qF[0] = 1; qF[2] = 1; }
                }))
                return;
        }
        it++;
    }
    if (!qBarrier(B, c)) return;
    {
        double v[1] = {0.0};
        forRows(B, rs, [&](int i, int len) {
            double r = B.b[i] - qRow(B, B.x, i, len);
            v[0] += r * r;
        });
        qSum<1>(v, B, c, [&](const double* t) { qS[S_RR] = t[0]; });
    }
    qStore(B, qL);
}

// Plain FP64 Jacobi-PCG with shared-memory vectors: the same method, rows and stopping
// rule as k_cg_solve, with r, p and Ap of each block's rows (24 bytes per row) in shared
// memory (slot m BS + t for the m-th row of thread t); x, the inverse diagonal and z (gathered
// through the matrix columns) stay in global memory.
#define OWN64_CAPMAX OWN64_CAP_ROWS   // slots per block: 3 x 8448 x 8 B = 198 KB of shared memory
__global__ void __launch_bounds__(QBC, 1) k_cg_own(Dev d, PpeBuffers B, double tol, int maxIter, int cap) {
    __shared__ QLocal qL;   // this block's copy of the solver scalars and flags
    qInit(qL);
    double* const qS = qL.scal;
    int* const qF = qL.flag;
    extern __shared__ __align__(128) unsigned char dynSmem[];
    double* const sr = reinterpret_cast<double*>(dynSmem);
    double* const sp = sr + cap;
    double* const sap = sp + cap;
    const int n = liveN(d);
    const RowSet rs = rowSet(n, QBC);   // this thread's rows (rowCount(rs) * QBC <= cap)
    QCtl c = {0u};
    {
        double v[3] = {0.0, 0.0, 0.0};
        forRowsL(B, rs, [&](int l, int i, int len) {
            const double di = 1.0 / __ldg(B.diag + i);
            const double bi = B.b[i];
            const double r = bi - qRow(B, B.x, i, len);
            const double z = r * di;
            B.dinv[i] = di; sr[l] = r; B.z[i] = z;
            v[0] += r * z; v[1] += r * r; v[2] += bi * bi;
        });
        if (!qSum<3>(v, B, c, [&](const double* t) {
                qS[S_RZ] = t[0]; qS[S_RR] = t[1]; qS[S_BB] = t[2];
                double thr = tol * tol * t[2];
                if (thr < 2.2250738585072014e-308) thr = 2.2250738585072014e-308;
                qS[S_THR] = thr;
                qS[S_SCALE] = sqrt(t[1] / (t[2] > 0 ? t[2] : 1.0));
                qF[0] = (t[2] == 0.0 || t[1] < thr) ? 1 : 0;
                qF[1] = 0;
                if (!(t[0] == t[0]) || !(t[1] == t[1])) { qF[0] = 1; qF[2] = 1; }
            }))
            return;
    }
    int it = 0;
    while (!vi(qF) && it < maxIter) {
        {   // Ap = A z + beta Ap, p = z + beta p, p.Ap
            const double beta = it ? vd(qS + S_BETA) : 0.0;
            double v[1] = {0.0};
            forRowsL(B, rs, [&](int l, int i, int len) {
                const double q = qRow(B, B.z, i, len);
                const double z = B.z[i];
                const double ap = it ? q + beta * sap[l] : q;
                const double p = it ? z + beta * sp[l] : z;
                sap[l] = ap; sp[l] = p;
                v[0] += p * ap;
            });
            if (!qSumD<1>(v, B, c, [&](const double* t) { qS[S_PAP] = t[0]; qS[S_ALPHA] = qS[S_RZ] / t[0]; }))
                return;
        }
        {   // x += alpha p, r -= alpha Ap, z = M^-1 r; r.z, r.r
            const double alpha = vd(qS + S_ALPHA);
            double v[2] = {0.0, 0.0};
            const int cnt = rowCount(rs);
            for (int m0 = 0; m0 < cnt; m0 += 4) {
                double mi[4], xo[4];
                int ii[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    ii[u] = (m0 + u < cnt) ? rowAt(rs, m0 + u) : -1;
                    mi[u] = (ii[u] >= 0) ? B.dinv[ii[u]] : 0.0;
                    xo[u] = (ii[u] >= 0) ? B.x[ii[u]] : 0.0;
                }
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    if (ii[u] < 0) continue;
                    const int l = (m0 + u) * (int)blockDim.x + (int)threadIdx.x;
                    const double r = sr[l] - alpha * sap[l];
                    const double z = r * mi[u];
                    B.x[ii[u]] = xo[u] + alpha * sp[l];
                    sr[l] = r;
                    B.z[ii[u]] = z;
                    v[0] += r * z; v[1] += r * r;
                }
            }
            if (!qSumD<2>(v, B, c, [&](const double* t) {
                    qF[1] += 1;
                    qS[S_RR] = t[1];
                    qS[S_BETA] = t[0] / qS[S_RZ];
                    qS[S_RZ] = t[0];
                    if (t[1] < qS[S_THR]) qF[0] = 1;
                    if (!(t[1] == t[1])) { qF[0] = 1; qF[2] = 1; }
                }))
                return;
        }
        it++;
    }
    if (!qBarrier(B, c)) return;
    {   // FP64 residual of the result
        double v[1] = {0.0};
        forRows(B, rs, [&](int i, int len) {
            const double r = B.b[i] - qRow(B, B.x, i, len);
            v[0] += r * r;
        });
        qSum<1>(v, B, c, [&](const double* t) { qS[S_RR] = t[0]; });
    }
    qStore(B, qL);
}

// Jacobi-preconditioned BiCGSTAB (solver_type 1: Eigen::BiCGSTAB, src/MpsPressure.cpp:448-468;
// van der Vorst 1992 with the preconditioner on the right), in one cooperative launch: per
// iteration two SpMVs and five grid synchronisations (y and z must be complete before their
// SpMVs; (r0, v), (t, t) and (t, s), (r, r) and (r0, r) are grid sums).  The shadow residual
// is restarted when (r0, r) vanishes relative to its start, the stopping rule is
// ||r||^2 < tol^2 ||b||^2 on the recurrence residual, and the FP64 residual of the result is
// reported.
__global__ void __launch_bounds__(QBC, 1) k_bicgstab(Dev d, PpeBuffers B, double tol, int maxIter) {
    __shared__ QLocal qL;   // this block's copy of the solver scalars and flags
    qInit(qL);
    double* const qS = qL.scal;
    int* const qF = qL.flag;
    const int n = liveN(d);
    const RowSet rs = rowSet(n, QBC);   // this thread's rows
    QCtl c = {0u};
    double *r0 = B.bs[0], *sv = B.bs[1], *zz = B.bs[2], *tv = B.bs[3], *y = B.z, *v = B.Ap;
    auto restart = [&](bool first) -> bool {
        double a[2] = {0.0, 0.0};
        forRows(B, rs, [&](int i, int len) {
            if (first) B.dinv[i] = 1.0 / __ldg(B.diag + i);
            double r = B.b[i] - qRow(B, B.x, i, len);
            B.r[i] = r; r0[i] = r; B.p[i] = 0.0; v[i] = 0.0;
            a[0] += r * r;
            if (first) a[1] += B.b[i] * B.b[i];
        });
        return qSum<2>(a, B, c, [&](const double* t) {
            if (first) {
                qS[S_BB] = t[1];
                double thr = tol * tol * t[1];
                if (thr < 2.2250738585072014e-308) thr = 2.2250738585072014e-308;
                qS[S_THR] = thr;
                qS[S_SCALE] = sqrt(t[0] / (t[1] > 0 ? t[1] : 1.0));
                qF[1] = 0;
                if (t[1] == 0.0) qF[0] = 1;
            }
            qS[S_RR] = qS[S_RHO] = qS[S_R0N2] = t[0];
            qS[S_RHOOLD] = qS[S_ALPHA] = qS[S_OMEGA] = 1.0;
            qF[5] = 0;
            if (t[0] < qS[S_THR]) qF[0] = 1;
            if (!(t[0] == t[0])) { qF[0] = 1; qF[2] = 1; }
        });
    };
    if (!restart(true)) return;
    int it = 0;
    while (!vi(qF) && it < maxIter) {
        {   // p = r + beta (p - w v), y = M^-1 p
            const double rho = vd(qS + S_RHO), w = vd(qS + S_OMEGA);
            const double beta = (rho / vd(qS + S_RHOOLD)) * (vd(qS + S_ALPHA) / w);
            forOwn(rs, [&](int i) {
                double p = B.r[i] + beta * (B.p[i] - w * v[i]);
                B.p[i] = p;
                y[i] = p * B.dinv[i];
            });
            if (!qBarrier(B, c)) return;
        }
        {   // v = A y, alpha = rho / (r0, v)
            double a[1] = {0.0};
            forRows(B, rs, [&](int i, int len) {
                double q = qRow(B, y, i, len);
                v[i] = q;
                a[0] += r0[i] * q;
            });
            if (!qSum<1>(a, B, c, [&](const double* t) {
                    double al = qS[S_RHO] / t[0];
                    qS[S_ALPHA] = al;
                    if (!(al == al) || t[0] == 0.0) { qF[0] = 1; qF[2] = 1; }
                }))
                return;
        }
        if (vi(qF)) break;
        {   // s = r - alpha v, z = M^-1 s
            const double alpha = vd(qS + S_ALPHA);
            forOwn(rs, [&](int i) {
                double s = B.r[i] - alpha * v[i];
                sv[i] = s;
                zz[i] = s * B.dinv[i];
            });
            if (!qBarrier(B, c)) return;
        }
        {   // t = A z, w = (t, s) / (t, t)
            double a[2] = {0.0, 0.0};
            forRows(B, rs, [&](int i, int len) {
                double q = qRow(B, zz, i, len);
                tv[i] = q;
                a[0] += q * q;
                a[1] += q * sv[i];
            });
            if (!qSum<2>(a, B, c, [&](const double* t) { qS[S_OMEGA] = (t[0] > 0.0) ? t[1] / t[0] : 0.0; }))
                return;
        }
        {   // x += alpha y + w z, r = s - w t; (r, r) and the next rho = (r0, r)
            const double alpha = vd(qS + S_ALPHA), w = vd(qS + S_OMEGA);
            double a[2] = {0.0, 0.0};
            forOwn(rs, [&](int i) {
                B.x[i] += alpha * y[i] + w * zz[i];
                double r = sv[i] - w * tv[i];
                B.r[i] = r;
                a[0] += r * r;
                a[1] += r0[i] * r;
            });
            if (!qSum<2>(a, B, c, [&](const double* t) {
                    qF[1] += 1;
                    qS[S_RR] = t[0];
                    qS[S_RHOOLD] = qS[S_RHO];
                    qS[S_RHO] = t[1];
                    if (t[0] < qS[S_THR]) qF[0] = 1;
                    else if (fabs(t[1]) < 4.930380657631324e-32 * qS[S_R0N2]) qF[5] = 1;   // eps^2
                    if (!(t[0] == t[0]) || qS[S_OMEGA] == 0.0) { qF[0] = 1; qF[2] = 1; }
                }))
                return;
        }
        it++;
        if (vi(qF + 5) && !vi(qF))
            if (!restart(false)) return;
    }
    if (!qBarrier(B, c)) return;
    {
        double a[1] = {0.0};
        forRows(B, rs, [&](int i, int len) {
            double r = B.b[i] - qRow(B, B.x, i, len);
            a[0] += r * r;
        });
        qSum<1>(a, B, c, [&](const double* t) { qS[S_RR] = t[0]; });
    }
    qStore(B, qL);
}

// kind: 0 plain FP64, 1 mixed, 2 mixed with the matrix-free inner operator, 3 mixed with
// the compact scaled inner operator, 4 mixed with the staged tiles, 5 mixed with the
// pipelined inner CG, 6 BiCGSTAB, 7 mixed with block-owned rows (one block per SM), 8 plain
// FP64 with block-owned rows (one block per SM)
int ppePersistentGrid(int kind) {
    int dev = 0, sms = 0, coop = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) return 0;
    if (kind == 7) {
        const int dyn = OWN_CAPMAX * 16;
        if (cudaFuncSetAttribute(k_mx_own<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess ||
            cudaFuncSetAttribute(k_mx_own<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess)
            return 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mx_own<true>, QBX, dyn) != cudaSuccess || per <= 0) return 0;
        return sms;   // one block per SM: the ranges are sized for it
    }
    if (kind == 8) {
        const int dyn = OWN64_CAPMAX * 24;
        if (cudaFuncSetAttribute(k_cg_own, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess) return 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_cg_own, QBC, dyn) != cudaSuccess || per <= 0) return 0;
        return sms;
    }
    if (kind == 4) {
        if (cudaFuncSetAttribute(k_mx_solve<OP_TILED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(TsSmem)) != cudaSuccess)
            return 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mx_solve<OP_TILED>, QB, sizeof(TsSmem)) != cudaSuccess ||
            per <= 0)
            return 0;
        return per * sms;
    }
    cudaError_t e = kind == 6   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_bicgstab, QBC, 0)
                    : kind == 5 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mx_pipe, QBX, 0)
                    : kind == 3 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mx_solve<OP_H16>, QBX, 0)
                    : kind == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mx_solve<OP_MATFREE>, QBX, 0)
                    : kind == 1 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mx_solve<OP_ELL32>, QBX, 0)
                                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_cg_solve, QBC, 0);
    if (e != cudaSuccess || per <= 0) return 0;
    return per * sms;
}

static int finishPersistent(const PpeBuffers& B, cudaStream_t s, int* iters, int* refinements, double* relres,
                            double* relres0) {
    int f[5];
    unsigned int abortWord = 0;
    double sc[S_COUNT];
    if (cudaMemcpyAsync(f, B.flag, sizeof(f), cudaMemcpyDeviceToHost, s) != cudaSuccess) return MPSGPU_ERR_CUDA;
    if (cudaMemcpyAsync(&abortWord, B.bar + QB_ABT, sizeof(unsigned int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return MPSGPU_ERR_CUDA;
    if (cudaMemcpyAsync(sc, B.scal, sizeof(sc), cudaMemcpyDeviceToHost, s) != cudaSuccess) return MPSGPU_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return MPSGPU_ERR_CUDA;
    if (abortWord) return MPSGPU_ERR_CUDA;   // a grid-barrier wait ran out (reported by the caller)
    *iters = f[1];
    if (refinements) *refinements = f[4];
    double bb = sc[S_BB] > 0 ? sc[S_BB] : 1.0;
    *relres = (sc[S_BB] > 0) ? sqrt(sc[S_RR] / bb) : 0.0;
    *relres0 = sc[S_SCALE];
    if (f[2] || !f[0]) return MPSGPU_ERR_NOT_CONVERGED;
    return 0;
}

int ppeSolveBicgstab(const Dev& d, const PpeBuffers& B, double tol, int maxIter, cudaStream_t s, int* iters,
                     double* relres, double* relres0, Prof* prof) {
    if (B.pgridBi <= 0) return MPSGPU_ERR_UNSUPPORTED;
    bool pr = prof && prof->on;
    cudaMemsetAsync(B.flag, 0, 8 * sizeof(int), s);
    cudaMemsetAsync(B.bar, 0, QB_WORDS * sizeof(unsigned int), s);
    Dev dd = d;
    PpeBuffers bb = B;
    double t = tol;
    int mi = maxIter;
    void* args[4] = {&dd, &bb, &t, &mi};
    if (pr) prof->begin(PROF_PPE_SOLVE, s);
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_bicgstab, B.pgridBi, QBC, args, 0, s);
    if (pr) prof->end(s);
    if (e != cudaSuccess) return MPSGPU_ERR_CUDA;
    countLaunch(1);
    return finishPersistent(B, s, iters, nullptr, relres, relres0);
}

int ppeSolvePersistent(const Dev& d, const PpeBuffers& B, int mixed, double tol, int maxIter, cudaStream_t s,
                       int* iters, int* refinements, double* relres, double* relres0, Prof* prof) {
    int grid = !mixed ? B.pgridCg
                      : (B.matfree == 4 ? B.pgridPipe
                                        : (B.matfree == 3 ? B.pgridTs
                                                          : (B.matfree == 2 ? B.pgridH16 : (B.matfree ? B.pgridMf : B.pgridMx))));
    if (grid <= 0) return MPSGPU_ERR_UNSUPPORTED;
    bool pr = prof && prof->on;
    cudaMemsetAsync(B.flag, 0, 5 * sizeof(int), s);
    cudaMemsetAsync(B.bar, 0, QB_WORDS * sizeof(unsigned int), s);
    if (mixed && !B.prepared) {
        if (pr) prof->begin(PROF_PPE_OTHER, s);
        k_mixed_prepare<<<gridFor(d.N0, 256), 256, 0, s>>>(d, B);
        if (pr) prof->end(s);
        countLaunch(1);
    }
    Dev dd = d;
    PpeBuffers bb = B;
    // inner floor 1e-6: from a good warm start one FP32 inner solve reaches the whole
    // reduction and a single FP64 refinement confirms it (measured at 864k rows: one
    // refinement instead of two, 1.86 -> 1.74 ms); a coarser floor forces extra refinements
    double t = tol, eta2 = 1e-6 * 1e-6;
    int mi = maxIter;
    void* args[6] = {&dd, &bb, &t, &mi, &eta2, nullptr};
    if (!mixed && !B.ownOff && B.pgridOwn64 > 0 && B.ownCap64 > 0) {
        // block-owned rows: r, p, Ap of each block in its shared memory
        int cap = B.ownCap64;
        void* a4[5] = {&dd, &bb, &t, &mi, &cap};
        if (pr) prof->begin(PROF_PPE_SOLVE, s);
        cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_cg_own, B.pgridOwn64, QBC, a4, (size_t)cap * 24, s);
        if (pr) prof->end(s);
        if (e != cudaSuccess) return MPSGPU_ERR_CUDA;
        countLaunch(1);
        return finishPersistent(B, s, iters, refinements, relres, relres0);
    }
    if (mixed && B.matfree == 0 && !B.ownOff && B.pgridOwn > 0 && B.ownCap > 0) {
        // block-owned rows: the FP32 inner-CG vectors of each block in its shared memory
        int cap = B.ownCap;
        args[5] = &cap;
        if (pr) prof->begin(PROF_PPE_SOLVE, s);
        const void* fn = B.cdir ? (const void*)k_mx_own<true> : (const void*)k_mx_own<false>;
        cudaError_t e = cudaLaunchCooperativeKernel(fn, B.pgridOwn, QBX, args, (size_t)cap * 16, s);
        if (pr) prof->end(s);
        if (e != cudaSuccess) return MPSGPU_ERR_CUDA;
        countLaunch(1);
        return finishPersistent(B, s, iters, refinements, relres, relres0);
    }
    if (pr) prof->begin(PROF_PPE_SOLVE, s);
    const void* fn = !mixed              ? (const void*)k_cg_solve
                     : B.matfree == 4    ? (const void*)k_mx_pipe
                     : B.matfree == 3    ? (const void*)k_mx_solve<OP_TILED>
                     : B.matfree == 2    ? (const void*)k_mx_solve<OP_H16>
                     : B.matfree == 1    ? (const void*)k_mx_solve<OP_MATFREE>
                                         : (const void*)k_mx_solve<OP_ELL32>;
    size_t dyn = (mixed && B.matfree == 3) ? sizeof(TsSmem) : 0;
    const int bs = !mixed ? QBC : (B.matfree == 3 ? QB : QBX);
    cudaError_t e = cudaLaunchCooperativeKernel(fn, grid, bs, args, dyn, s);
    if (pr) prof->end(s);
    if (e != cudaSuccess) return MPSGPU_ERR_CUDA;
    countLaunch(1);
    return finishPersistent(B, s, iters, refinements, relres, relres0);
}
