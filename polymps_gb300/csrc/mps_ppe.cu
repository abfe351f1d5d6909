// mps_ppe.cu — pressure Poisson equation on sm_103a: assembly and solvers.
//
// Assembly replaces the serial Eigen triplet loop of MpsPressure::solvePressurePoissonPnd
// (src/MpsPressure.cpp:169-286): one thread per row walks its ELL neighbour row and writes
// the off-diagonal entries (j inner, not dummy) straight into an ELL matrix
// (val/col[k * N0 + i], coalesced across a warp), the diagonal and the right-hand side.
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
#include "mps_common.cuh"
#include "mps_internal.h"

#define PBLK 256

// solver scalars in B.scal[]
enum { S_RZ = 0, S_RR, S_BB, S_ALPHA, S_BETA, S_PAP, S_THR, S_RZNEW, S_SCALE, S_COUNT };

// ------------------------------------------------------------------ assembly
__global__ void __launch_bounds__(128) k_ppe_assemble(Dev d, PpeBuffers B) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    int bci = d.bc[i];
    if (bci == P.other || bci == P.surface) {
        B.diag[i] = 1.0; B.rowLen[i] = 0; B.b[i] = 0.0;
        warpCount(d.counters + 1, 0u);
        return;
    }
    dvec4 pi = d.pos[i];
    double sum = 0.0, src = 0.0;
    int len = 0;
    const double* wLc = d.cwL ? d.cwL : d.cw;
    forMask(d, i, d.maskL[i], [&](int j, size_t e) {
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
                size_t k = (size_t)len * B.N0 + i;
                B.val[k] = mij;
                B.col[k] = j;
                len++;
            }
        }
    });
    double rho = P.DNS_FL1;
    sum -= P.alphaCompressibility * rho / (P.timeStep * P.timeStep);
    B.diag[i] = sum;
    B.rowLen[i] = len;
    B.b[i] = src + (-P.coeffPPESource * rho * (d.pndSmall[i] - P.pndSmallZero));
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
    d.pressPPE[i] = x;
    d.source[i] = B.b[i];
    d.press[i] = x < 0.0 ? 0.0 : x;
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

// ------------------------------------------------------------------ plain FP64 PCG
// One ELL row, four entries in flight (independent value/column/gather loads).
__device__ __forceinline__ double spmvRow(const PpeBuffers& B, const double* x, int i) {
    double s = B.diag[i] * x[i];
    int len = B.rowLen[i];
    const size_t N0 = B.N0;
    const double* v = B.val + i;
    const int* c = B.col + i;
    int k = 0;
    double s1 = 0.0, s2 = 0.0, s3 = 0.0;
    for (; k + 4 <= len; k += 4) {
        int c0 = __ldg(c + k * N0), c1 = __ldg(c + (k + 1) * N0), c2 = __ldg(c + (k + 2) * N0), c3 = __ldg(c + (k + 3) * N0);
        double v0 = __ldg(v + k * N0), v1 = __ldg(v + (k + 1) * N0), v2 = __ldg(v + (k + 2) * N0), v3 = __ldg(v + (k + 3) * N0);
        s += v0 * __ldg(x + c0);
        s1 += v1 * __ldg(x + c1);
        s2 += v2 * __ldg(x + c2);
        s3 += v3 * __ldg(x + c3);
    }
    for (; k < len; k++) s += __ldg(v + k * N0) * __ldg(x + __ldg(c + k * N0));
    return s + ((s1 + s2) + s3);
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
    for (int k = 0; k < len; k++) {
        size_t e = (size_t)k * B.N0 + i;
        B.valf[e] = (float)B.val[e];
    }
    B.diagf[i] = (float)B.diag[i];
    B.diagInvf[i] = (float)(1.0 / B.diag[i]);
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
    float s = B.diagf[i] * x[i];
    int len = B.rowLen[i];
    const size_t N0 = B.N0;
    const float* v = B.valf + i;
    const int* c = B.col + i;
    int k = 0;
    float s1 = 0.f, s2 = 0.f, s3 = 0.f;
    for (; k + 4 <= len; k += 4) {
        int c0 = __ldg(c + k * N0), c1 = __ldg(c + (k + 1) * N0), c2 = __ldg(c + (k + 2) * N0), c3 = __ldg(c + (k + 3) * N0);
        float v0 = __ldg(v + k * N0), v1 = __ldg(v + (k + 1) * N0), v2 = __ldg(v + (k + 2) * N0), v3 = __ldg(v + (k + 3) * N0);
        s += v0 * __ldg(x + c0);
        s1 += v1 * __ldg(x + c1);
        s2 += v2 * __ldg(x + c2);
        s3 += v3 * __ldg(x + c3);
    }
    for (; k < len; k++) s += __ldg(v + k * N0) * __ldg(x + __ldg(c + k * N0));
    return s + ((s1 + s2) + s3);
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
