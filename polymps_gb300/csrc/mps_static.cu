// mps_static.cu — allocation-free Jacobi-preconditioned CG on a caller-supplied CSR system.
//
// Some callers cannot allocate device memory at the moment they need a pressure solve:
// a host application that runs inside a memory budget owned by another framework (its
// caching allocator must see every byte, and a raw cudaMalloc would bypass or fragment
// it), a real-time stepping loop that forbids allocation latency once running, or a plugin
// called back from a library that hands it only the arrays it owns.  For them this entry
// point keeps all of its working vectors in one file-scope device array reserved when the
// library is loaded: it calls no cudaMalloc/cudaFree and no allocating library routine.
//
// Limits and rules (the same as in the declaration in mpsgpu.h):
//  * at most MPSGPU_STATIC_MAX_ROWS rows; larger systems are rejected with an error;
//  * the array is shared by every call on a device and keeps the last call's contents:
//    each call clears the counters it relies on, and two calls that overlap on the GPU
//    (different streams, or different host threads) race on the same scratch;
//  * the first call on a device looks the array's device address up (with that device
//    current); make that first call before any stream capture begins.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <cuda_runtime.h>
#include "../../include/mpsgpu.h"

#define SBLOCKS 256
#define SBLK 256
#define SMAX MPSGPU_STATIC_MAX_ROWS

// layout in doubles: r, z, p, Ap, inverse diagonal (SMAX each), block partials (3 per block),
// scalars (16), control words (counter, flags; 8 unsigned ints) in the last 4 doubles
#define OFF_R 0
#define OFF_Z (1ull * SMAX)
#define OFF_P (2ull * SMAX)
#define OFF_AP (3ull * SMAX)
#define OFF_DINV (4ull * SMAX)
#define OFF_PART (5ull * SMAX)
#define OFF_SCAL (OFF_PART + 3ull * SBLOCKS)
#define OFF_CTRL (OFF_SCAL + 16ull)
#define SCRATCH_DOUBLES (OFF_CTRL + 4ull)

// The scratch every call uses (about 5.3 MB per GPU, held from library load until exit).
static __device__ __align__(256) double g_pcgScratch[SCRATCH_DOUBLES];

enum { SC_RZ = 0, SC_RR, SC_BB, SC_ALPHA, SC_BETA, SC_THR, SC_RR0 };

namespace {

struct View {
    double *r, *z, *p, *Ap, *dinv, *part, *scal;
    unsigned int* ctrl;   // [0] block counter, [1] done, [2] iterations, [3] breakdown,
                          // [4] UINT_MAX - (lowest row without a usable diagonal), 0 if none
};
__host__ __device__ inline View viewOf(double* S) {
    View v;
    v.r = S + OFF_R; v.z = S + OFF_Z; v.p = S + OFF_P; v.Ap = S + OFF_AP; v.dinv = S + OFF_DINV;
    v.part = S + OFF_PART; v.scal = S + OFF_SCAL;
    v.ctrl = (unsigned int*)(S + OFF_CTRL);
    return v;
}

// Sum of NV per-thread values over the grid: per-block partials, then the last block to
// arrive adds them in block order and calls fin(totals) on thread 0.
template <int NV, class Fin>
__device__ void gridTotal(double (&v)[NV], const View& w, Fin fin) {
    __shared__ double sm[NV][SBLK / 32];
    __shared__ bool last;
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int q = 0; q < NV; q++) {
        double x = v[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) sm[q][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 0; q < NV; q++) {
            double s = 0.0;
            for (int k = 0; k < SBLK / 32; k++) s += sm[q][k];
            w.part[q * SBLOCKS + blockIdx.x] = s;
        }
        __threadfence();
        last = (atomicInc(&w.ctrl[0], gridDim.x - 1) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double t[NV];
    for (int q = 0; q < NV; q++) {
        double s = 0.0;
        for (int b = 0; b < (int)gridDim.x; b++) s += ((volatile double*)w.part)[q * SBLOCKS + b];
        t[q] = s;
    }
    fin(t);
}

__device__ __forceinline__ double rowDot(const int* rowptr, const int* col, const double* val, const double* x, int i) {
    double s = 0.0;
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++) s += val[k] * x[col[k]];
    return s;
}

__global__ void __launch_bounds__(SBLK) k_s_init(int n, const int* rowptr, const int* col, const double* val,
                                                 const double* b, const double* x, double* S, double tol) {
    View w = viewOf(S);
    double v[3] = {0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double diag = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; k++)
            if (col[k] == i) diag = val[k];
        // a row without a stored non-zero diagonal cannot be Jacobi-scaled: record the
        // lowest such row (as UINT_MAX - row, so atomicMax keeps the lowest) and leave the
        // solve to the host, which rejects the system before any iteration runs
        double di = 0.0;
        if (diag != 0.0 && diag == diag) di = 1.0 / diag;
        else atomicMax(&w.ctrl[4], 0xFFFFFFFFu - (unsigned int)i);
        double r = b[i] - rowDot(rowptr, col, val, x, i);
        double z = r * di;
        w.dinv[i] = di; w.r[i] = r; w.z[i] = z; w.p[i] = z;
        v[0] += r * z; v[1] += r * r; v[2] += b[i] * b[i];
    }
    gridTotal<3>(v, w, [&](double* t) {
        w.scal[SC_RZ] = t[0]; w.scal[SC_RR] = t[1]; w.scal[SC_BB] = t[2];
        double thr = tol * tol * t[2];
        if (thr < 2.2250738585072014e-308) thr = 2.2250738585072014e-308;
        w.scal[SC_THR] = thr;
        w.ctrl[1] = (t[2] == 0.0 || t[1] < thr) ? 1u : 0u;
        w.ctrl[2] = 0u;
        if (!(t[0] == t[0]) || !(t[1] == t[1])) { w.ctrl[1] = 1u; w.ctrl[3] = 1u; }
        if (*(volatile unsigned int*)&w.ctrl[4]) w.ctrl[1] = 1u;   // malformed system: no iteration
    });
}
__global__ void __launch_bounds__(SBLK) k_s_spmv(int n, const int* rowptr, const int* col, const double* val, double* S) {
    View w = viewOf(S);
    if (*(volatile unsigned int*)&w.ctrl[1]) return;
    double v[1] = {0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double ap = rowDot(rowptr, col, val, w.p, i);
        w.Ap[i] = ap;
        v[0] += w.p[i] * ap;
    }
    gridTotal<1>(v, w, [&](double* t) { w.scal[SC_ALPHA] = w.scal[SC_RZ] / t[0]; });
}
__global__ void __launch_bounds__(SBLK) k_s_update(int n, double* x, double* S, unsigned int maxIter) {
    View w = viewOf(S);
    if (*(volatile unsigned int*)&w.ctrl[1]) return;
    double alpha = w.scal[SC_ALPHA];
    double v[2] = {0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += alpha * w.p[i];
        double r = w.r[i] - alpha * w.Ap[i];
        double z = r * w.dinv[i];
        w.r[i] = r; w.z[i] = z;
        v[0] += r * z; v[1] += r * r;
    }
    gridTotal<2>(v, w, [&](double* t) {
        w.ctrl[2] += 1u;
        w.scal[SC_RR] = t[1];
        w.scal[SC_BETA] = t[0] / w.scal[SC_RZ];
        w.scal[SC_RZ] = t[0];
        if (t[1] < w.scal[SC_THR]) w.ctrl[1] = 1u;
        else if (w.ctrl[2] >= maxIter) w.ctrl[1] = 2u;   // stopped at the iteration cap
        if (!(t[1] == t[1])) { w.ctrl[1] = 1u; w.ctrl[3] = 1u; }
    });
}
__global__ void __launch_bounds__(SBLK) k_s_p(int n, double* S) {
    View w = viewOf(S);
    if (*(volatile unsigned int*)&w.ctrl[1]) return;
    double beta = w.scal[SC_BETA];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        w.p[i] = w.z[i] + beta * w.p[i];
}
__global__ void __launch_bounds__(SBLK) k_s_residual(int n, const int* rowptr, const int* col, const double* val,
                                                     const double* b, const double* x, double* S) {
    View w = viewOf(S);
    double v[1] = {0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double r = b[i] - rowDot(rowptr, col, val, x, i);
        v[0] += r * r;
    }
    gridTotal<1>(v, w, [&](double* t) { w.scal[SC_RR0] = t[0]; });
}

std::mutex g_mu;
double* g_addr[256] = {nullptr};
std::string g_msg;

// Device address of the scratch array for the current device (looked up once per device).
int scratchFor(double** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) { g_msg = "no current CUDA device"; return MPSGPU_ERR_NOGPU; }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        double* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void**)&p, g_pcgScratch);
        if (e != cudaSuccess || !p) {
            g_msg = std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e);
            return MPSGPU_ERR_CUDA;
        }
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return 0;
}

}  // namespace

extern "C" int mpsgpu_pcg_solve_static(int n, const int* rowptr, const int* col, const double* val,
                                       const double* b, double* x, double tol, int max_iter, void* stream,
                                       int* iters, double* relres) {
    if (n <= 0 || n > SMAX) {
        g_msg = "mpsgpu_pcg_solve_static: " + std::to_string(n) + " rows outside 1.." + std::to_string(SMAX) +
                " (the static scratch holds MPSGPU_STATIC_MAX_ROWS rows)";
        return MPSGPU_ERR_ARG;
    }
    if (!rowptr || !col || !val || !b || !x || !(tol > 0) || max_iter <= 0) {
        g_msg = "mpsgpu_pcg_solve_static: bad argument";
        return MPSGPU_ERR_ARG;
    }
    double* S = nullptr;
    int e = scratchFor(&S);
    if (e) return e;
    cudaStream_t s = (cudaStream_t)stream;
    View w = viewOf(S);
    auto fail = [](const char* what, cudaError_t err) {
        g_msg = std::string("mpsgpu_pcg_solve_static: ") + what + ": " + cudaGetErrorString(err);
        return MPSGPU_ERR_CUDA;
    };
    // the array keeps the previous call's contents: reset the block counter and flags
    cudaError_t ce = cudaMemsetAsync(w.ctrl, 0, 8 * sizeof(unsigned int), s);
    if (ce != cudaSuccess) return fail("clearing the control words", ce);
    int nb = (n + SBLK - 1) / SBLK;
    if (nb > SBLOCKS) nb = SBLOCKS;
    k_s_init<<<nb, SBLK, 0, s>>>(n, rowptr, col, val, b, x, S, tol);
    if ((ce = cudaGetLastError()) != cudaSuccess) return fail("launch", ce);
    unsigned int ctrl[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    double scal[16];
    // the set-up's verdict before any iteration: a malformed system is rejected with x
    // untouched; a zero right-hand side has the solution x = 0 (as Eigen's CG returns)
    if ((ce = cudaMemcpyAsync(ctrl, w.ctrl, sizeof(ctrl), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(scal, w.scal, sizeof(scal), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail("set-up", ce);
    if (ctrl[4]) {
        g_msg = "mpsgpu_pcg_solve_static: row " + std::to_string(0xFFFFFFFFu - ctrl[4]) +
                " has no stored non-zero diagonal entry (Jacobi preconditioning needs one in every row)";
        return MPSGPU_ERR_ARG;
    }
    if (scal[SC_BB] == 0.0) {
        if ((ce = cudaMemsetAsync(x, 0, sizeof(double) * (size_t)n, s)) != cudaSuccess ||
            (ce = cudaStreamSynchronize(s)) != cudaSuccess)
            return fail("zeroing x", ce);
        if (iters) *iters = 0;
        if (relres) *relres = 0.0;
        return 0;
    }
    int launched = 0;
    const int batch = 8;
    while (!ctrl[1]) {
        for (int k = 0; k < batch; k++) {
            k_s_spmv<<<nb, SBLK, 0, s>>>(n, rowptr, col, val, S);
            k_s_update<<<nb, SBLK, 0, s>>>(n, x, S, (unsigned int)max_iter);
            k_s_p<<<nb, SBLK, 0, s>>>(n, S);
        }
        launched += batch;
        if ((ce = cudaGetLastError()) != cudaSuccess) return fail("launch", ce);
        if ((ce = cudaMemcpyAsync(ctrl, w.ctrl, sizeof(ctrl), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (ce = cudaStreamSynchronize(s)) != cudaSuccess)
            return fail("polling", ce);
        if (launched >= max_iter) break;
    }
    k_s_residual<<<nb, SBLK, 0, s>>>(n, rowptr, col, val, b, x, S);
    if ((ce = cudaGetLastError()) != cudaSuccess) return fail("launch", ce);
    if ((ce = cudaMemcpyAsync(scal, w.scal, sizeof(scal), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail("residual read-back", ce);
    if (iters) *iters = (int)ctrl[2];
    if (relres) *relres = std::sqrt(scal[SC_RR0] / scal[SC_BB]);
    if (ctrl[3] || ctrl[1] != 1u) { g_msg = "mpsgpu_pcg_solve_static: did not reach the tolerance"; return MPSGPU_ERR_NOT_CONVERGED; }
    return 0;
}

extern "C" const char* mpsgpu_pcg_static_error(void) { return g_msg.c_str(); }
