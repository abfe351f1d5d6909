// mps_mlp_tc.cu — inference of the learned warm-start network on the fifth-generation tensor
// cores (tcgen05, sm_103a): the MLP 16 -> 64 -> 64 -> 64 -> 1 with GELU, BF16 weights and
// activations, FP32 accumulation in tensor memory.
//
// A block of 128 threads takes tiles of 128 rows.  The weights (row-major [out][in] BF16
// copies) and the activations of the tile sit in shared memory in the canonical K-major
// layout without swizzle: 8 x 8 core matrices (8 rows of 16 bytes, stored contiguously), the
// k-blocks of a row block adjacent (leading byte offset 128) and the row blocks K * 16 bytes
// apart (stride byte offset).  Per layer one thread issues the tcgen05.mma instructions
// (M = 128, N = 64, K = 16 each; D in 64 columns of tensor memory, one lane per row) and
// commits them to an mbarrier; every thread then reads its row's 64 accumulators with
// tcgen05.ld (warp w owns lanes 32w..32w+31), adds the bias, applies the GELU and writes
// the BF16 activations of its row back as the next layer's A operand.  The last layer
// (64 -> 1) is a dot product in registers.  The contraction leaves the issue slots to the
// GELUs, which bound the kernel.
//
// Every mbarrier wait is bounded: a wait that runs out sets the error word, waits once more
// (bounded) for the tensor core to finish, and the block frees its tensor memory and returns.
#include <cstdint>
#include <cuda_bf16.h>
#include "mps_common.cuh"
#include "mps_internal.h"
#include "mps_mlp.h"
#include "mps_gelu.cuh"

namespace {

constexpr int H = 64, NF = 16, TM = 128;
// parameter offsets of the packed FP32 master vector and of the BF16 copy (mpsgpu.h order)
constexpr int OB1 = H * NF, OB2 = OB1 + H + H * H, OB3 = OB2 + H + H * H, OB4 = OB3 + H + H;
constexpr int BW1 = 0, BW2 = BW1 + H * NF, BW3 = BW2 + H * H, BW4 = BW3 + H * H;
constexpr int TMEM_COLS = 64;
constexpr long long TC_SPIN = 1ll << 24;

// instruction descriptor of tcgen05.mma kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at
// bits 24-28
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(H >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);

struct __align__(128) TcSmem {
    __nv_bfloat16 a[TM * H];    // activations of the tile (layer 1: the first TM * NF)
    __nv_bfloat16 w1[H * NF];
    __nv_bfloat16 w2[H * H];
    __nv_bfloat16 w3[H * H];
    float b1[H], b2[H], b3[H], w4[H], mean[NF], istd[NF];
    float b4;
    unsigned long long bar;
    uint32_t tmem;
    int ok;   // the issuing thread's verdict on the last commit wait
};

// element offset of (r, k) in a K-major tile with kdim columns of 8 x 8 core matrices
__device__ __forceinline__ int coreOff(int r, int k, int kdim) {
    return (r >> 3) * (kdim * 8) + (k >> 3) * 64 + (r & 7) * 8 + (k & 7);
}
__device__ __forceinline__ uint32_t sAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
// shared-memory matrix descriptor: start address, leading and stride byte offsets (>> 4),
// the fixed 0b001 at bits 46-48, no base offset, no swizzle
__device__ __forceinline__ uint64_t smemDesc(const void* p, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((sAddr(p) & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= 1ull << 46;
    return d;
}
__device__ __forceinline__ void mmaBf16(uint32_t tmem, uint64_t a, uint64_t b, int accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(tmem), "l"(a), "l"(b), "r"(IDESC), "r"(accumulate) : "memory");
}
__device__ __forceinline__ void fenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fenceProxy() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ bool barTry(unsigned long long* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok) : "r"(sAddr(b)), "r"(parity) : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool barWait(unsigned long long* b, uint32_t parity) {
    for (long long k = 0; k < TC_SPIN; k++)
        if (barTry(b, parity)) return true;
    return false;
}
// the issuing thread: K / 16 MMAs of one layer on the tile, then their commit to the barrier
__device__ __forceinline__ void layerMma(TcSmem& s, const __nv_bfloat16* w, int kdim) {
    fenceAfter();
    const uint32_t sbo = (uint32_t)kdim * 16u;
    // a K = 16 step spans two core matrices along K: the next step starts 2 * 128 bytes on
    for (int ks = 0; ks < kdim / 16; ks++)
        mmaBf16(s.tmem, smemDesc(s.a + ks * 128, 128u, sbo), smemDesc(w + ks * 128, 128u, sbo), ks > 0);
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(sAddr(&s.bar))
                 : "memory");
}
// the row's 64 accumulators of this thread (lane 32 w + l of the warp's lanes): four loads
// of 16 columns, then the wait, which takes the destination registers as operands so that
// nothing reads them before the loads completed
__device__ __forceinline__ void tmemRow(uint32_t taddr, float* v) {
    uint32_t r[64];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];" : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]) : "r"(taddr + 0u));
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];" : "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]) : "r"(taddr + 16u));
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];" : "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]) : "r"(taddr + 32u));
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];" : "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63]) : "r"(taddr + 48u));
    asm volatile("tcgen05.wait::ld.sync.aligned;" : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]), "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]), "+r"(r[29]), "+r"(r[30]), "+r"(r[31]), "+r"(r[32]), "+r"(r[33]), "+r"(r[34]), "+r"(r[35]), "+r"(r[36]), "+r"(r[37]), "+r"(r[38]), "+r"(r[39]), "+r"(r[40]), "+r"(r[41]), "+r"(r[42]), "+r"(r[43]), "+r"(r[44]), "+r"(r[45]), "+r"(r[46]), "+r"(r[47]), "+r"(r[48]), "+r"(r[49]), "+r"(r[50]), "+r"(r[51]), "+r"(r[52]), "+r"(r[53]), "+r"(r[54]), "+r"(r[55]), "+r"(r[56]), "+r"(r[57]), "+r"(r[58]), "+r"(r[59]), "+r"(r[60]), "+r"(r[61]), "+r"(r[62]), "+r"(r[63]) :: "memory");
#pragma unroll
    for (int k = 0; k < 64; k++) v[k] = __uint_as_float(r[k]);
}
// bias + GELU of the row, stored as BF16 in the next layer's A operand
__device__ __forceinline__ void storeHidden(TcSmem& s, int row, const float* v, const float* bias) {
#pragma unroll
    for (int kb = 0; kb < H / 8; kb++) {
        uint32_t pk[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            __nv_bfloat162 h = __floats2bfloat162_rn(gelu(v[8 * kb + 2 * q] + bias[8 * kb + 2 * q]),
                                                     gelu(v[8 * kb + 2 * q + 1] + bias[8 * kb + 2 * q + 1]));
            pk[q] = *reinterpret_cast<uint32_t*>(&h);
        }
        *reinterpret_cast<uint4*>(s.a + coreOff(row, 8 * kb, H)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
}

}  // namespace

// rows: the live count (nLive != nullptr) or n; out: the network output (bc == nullptr) or
// the correction c (Pa) of the learned start on equation rows (bc[i] == inner) and 0 elsewhere
__global__ void __launch_bounds__(TM, 4) k_mlp_forward_tc(const float* feat, int n, const int* nLive, const int* bc,
                                                          int inner, const __nv_bfloat16* wbf, const float* master,
                                                          const float* norm, const double* sig, float* out,
                                                          int* err) {
    __shared__ TcSmem s;
    const int t = threadIdx.x, warp = t >> 5;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sAddr(&s.tmem)),
                     "r"(TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sAddr(&s.bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int k = t; k < H * NF; k += TM) s.w1[coreOff(k / NF, k % NF, NF)] = wbf[BW1 + k];
    for (int k = t; k < H * H; k += TM) {
        s.w2[coreOff(k / H, k % H, H)] = wbf[BW2 + k];
        s.w3[coreOff(k / H, k % H, H)] = wbf[BW3 + k];
    }
    for (int k = t; k < H; k += TM) {
        s.w4[k] = __bfloat162float(wbf[BW4 + k]);
        s.b1[k] = master[OB1 + k]; s.b2[k] = master[OB2 + k]; s.b3[k] = master[OB3 + k];
    }
    for (int k = t; k < NF; k += TM) { s.mean[k] = norm[k]; s.istd[k] = norm[NF + k]; }
    if (t == 0) s.b4 = master[OB4];
    fenceProxy();
    fenceBefore();
    __syncthreads();
    fenceAfter();
    const uint32_t tmemRowAddr = s.tmem + ((uint32_t)(32 * warp) << 16);
    const int rows = nLive ? *nLive : n;
    const float q = sig ? (float)(1.0 / sig[0]) : 1.f;
    const float csc = sig ? (float)sig[0] / norm[2 * NF + 1] : 0.f, cmean = sig ? norm[2 * NF] * (float)sig[0] : 0.f;
    const int tiles = (rows + TM - 1) / TM;
    uint32_t phase = 0;
    bool ok = true;
    // the raw features of this thread's row in the block's next tile: loaded one tile ahead,
    // so that their latency runs under the current tile's layers
    float4 fq[4];
    auto loadFeat = [&](int tl) {
        const int r = tl * TM + t;
        if (tl < tiles && r < rows) {
            const float4* fp = reinterpret_cast<const float4*>(feat + (size_t)r * NF);
#pragma unroll
            for (int c = 0; c < 4; c++) fq[c] = __ldg(fp + c);
        }
    };
    loadFeat(blockIdx.x);
    for (int tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const int row = tile * TM + t;
        {   // layer 1 input: the row's 16 normalised features (pressure differences 1, 5, 7, 14
            // in units of sigma) as BF16
            float f[NF];
            if (row < rows) {
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    f[4 * c] = fq[c].x; f[4 * c + 1] = fq[c].y; f[4 * c + 2] = fq[c].z; f[4 * c + 3] = fq[c].w;
                }
                f[1] *= q; f[5] *= q; f[7] *= q; f[14] *= q;
#pragma unroll
                for (int k = 0; k < NF; k++) f[k] = (f[k] - s.mean[k]) * s.istd[k];
            } else {
#pragma unroll
                for (int k = 0; k < NF; k++) f[k] = 0.f;
            }
#pragma unroll
            for (int kb = 0; kb < NF / 8; kb++) {
                uint32_t pk[4];
#pragma unroll
                for (int p = 0; p < 4; p++) {
                    __nv_bfloat162 h = __floats2bfloat162_rn(f[8 * kb + 2 * p], f[8 * kb + 2 * p + 1]);
                    pk[p] = *reinterpret_cast<uint32_t*>(&h);
                }
                *reinterpret_cast<uint4*>(s.a + coreOff(t, 8 * kb, NF)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            }
        }
        loadFeat(tile + gridDim.x);
        float v[H];
        float o = 0.f;
#pragma unroll 1
        for (int layer = 0; layer < 3; layer++) {
            fenceProxy();   // the activations written by the threads, before the tensor core reads them
            fenceBefore();  // and every thread's tcgen05.ld of the previous layer, before D is rewritten
            __syncthreads();
            if (t == 0) {   // the issuing thread also waits for the commit (bounded) and tells the others
                layerMma(s, layer == 0 ? s.w1 : (layer == 1 ? s.w2 : s.w3), layer == 0 ? NF : H);
                s.ok = barWait(&s.bar, phase) ? 1 : 0;
            }
            fenceBefore();
            __syncthreads();
            fenceAfter();
            if (!s.ok) { ok = false; break; }
            phase ^= 1u;
            tmemRow(tmemRowAddr, v);
            if (layer < 2) {
                storeHidden(s, t, v, layer == 0 ? s.b1 : s.b2);
            } else {
#pragma unroll
                for (int k = 0; k < H; k++) o += gelu(v[k] + s.b3[k]) * s.w4[k];
                o += s.b4;
            }
        }
        if (!ok) break;
        if (row < rows) out[row] = bc ? ((bc[row] == inner) ? o * csc + cmean : 0.f) : o;
    }
    if (!ok && t == 0) {
        // a wait ran out: report it, let the tensor core finish (bounded), then free
        atomicExch(err, 1);
        barWait(&s.bar, phase);
    }
    fenceBefore();
    __syncthreads();
    if (warp == 0) {
        fenceAfter();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(s.tmem), "r"(TMEM_COLS) : "memory");
    }
}

int mlpForwardTc(const MlpState& m, const float* feat, int n, const int* nLive, const int* bc, int inner,
                 const double* sig, float* out, cudaStream_t st) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int tiles = (n + TM - 1) / TM;
    const int blocks = tiles < 4 * sms ? (tiles > 0 ? tiles : 1) : 4 * sms;
    k_mlp_forward_tc<<<blocks, TM, 0, st>>>(feat, n, nLive, bc, inner, m.wbf, m.master, m.norm, sig, out, m.tcErr);
    return cudaGetLastError() == cudaSuccess ? 0 : MPSGPU_ERR_CUDA;
}
