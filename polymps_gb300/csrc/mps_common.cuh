// mps_common.cuh — device state and helpers shared by the sm_103a kernels of the
// PolyMPS per-step particle path.
//
// Layout in HBM (all arrays sized for the initial particle count N0; the live count
// lives in device memory at *nLive so removals never need a host round trip):
//   * particle vectors as dvec4 (x, y, z, pad): one 32-byte sector per neighbour gather;
//   * particle scalars as double / int arrays;
//   * the stale bucket list of the step (MpsBucket::updateParticlesID) as a counting sort:
//     cellStart[nB+1] offsets into cellSorted[], particles ascending within a bucket,
//     so a scan of cellSorted visits them in the reference's linked-list order;
//   * the neighbour list of the current positions in ELL form, column-major
//     nbr[k * N0 + i] (coalesced across a warp), nbrCount[i] <= K.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/mpsgpu.h"

// 32-byte aligned FP64 vector (x, y, z, pad): one sector, one wide load per gather.
typedef double4_32a dvec4;
__host__ __device__ __forceinline__ dvec4 make_dvec4(double x, double y, double z, double w) {
    return make_double4_32a(x, y, z, w);
}

#define MPS_MAX_TRI 64
#define MPS_TAB 50

// Error bits OR-ed into Dev::err by kernels (read back by the host after each call).
#define MPSE_CAPACITY   1u   // a neighbour row exceeded K
#define MPSE_DOMAIN     2u   // a particle fell outside the bucket grid
#define MPSE_NOTCONV    4u   // PPE iteration cap reached
#define MPSE_NAN        8u   // non-finite value in a reduction

// Entry masks of a neighbour row (bit k: entry k of the row; rows hold up to 128 entries).
struct Mask {
    unsigned long long lo, hi;
};
__host__ __device__ __forceinline__ Mask operator&(const Mask& a, const Mask& b) { return {a.lo & b.lo, a.hi & b.hi}; }
#ifdef __CUDACC__
__device__ __forceinline__ Mask maskNone() { return {0ull, 0ull}; }
__device__ __forceinline__ Mask maskFirst(int c) {   // entries 0 .. c - 1
    Mask m;
    m.lo = c >= 64 ? ~0ull : ((1ull << c) - 1ull);
    m.hi = c >= 128 ? ~0ull : (c > 64 ? ((1ull << (c - 64)) - 1ull) : 0ull);
    return m;
}
__device__ __forceinline__ void maskSet(Mask& m, int k) {
    if (k < 64) m.lo |= 1ull << k;
    else m.hi |= 1ull << (k - 64);
}
__device__ __forceinline__ bool maskHas(const Mask& m, int k) {
    return k < 64 ? ((m.lo >> k) & 1ull) != 0ull : ((m.hi >> (k - 64)) & 1ull) != 0ull;
}
__device__ __forceinline__ int maskCount(const Mask& m) { return __popcll(m.lo) + __popcll(m.hi); }
// removes and returns the lowest entry (-1: none left)
__device__ __forceinline__ int maskPop(Mask& m) {
    if (m.lo) { const int k = __ffsll((long long)m.lo) - 1; m.lo &= m.lo - 1ull; return k; }
    if (m.hi) { const int k = __ffsll((long long)m.hi) - 1; m.hi &= m.hi - 1ull; return k + 64; }
    return -1;
}
#endif

struct Dev {
    MpsParams P;
    int N0;            // capacity
    int* nLive;        // current numParticles (device)
    int K;             // ELL row capacity
    int nB;            // numBucketsXYZ
    // particle vectors
    dvec4 *pos, *vel, *acc, *accStar, *mirror, *wallPos, *polyNormal, *npcd, *gradC, *forceWall;
    dvec4 *c1, *c2, *c3, *dvel, *shift;
    // particle scalars
    double *press, *pressPPE, *pndi, *pndki, *pndski, *pndSmall, *npcd2, *conc, *velDiv, *diffTerm;
    double *pndWall, *riw2, *devDot, *source, *aux1, *aux2;
    int *type, *bc, *numNeigh, *nNeighWall, *nearWall;
    float4* posf;      // FP32 copy of pos - domainMin (neighbour prefilter, FP32 sums)
    double* pressPPEprev;   // unclamped PPE solution of the solve before the last (warm start)
    double* pressPPEprev2;  // and the one before it
    // Storage numbering: particles are stored in bucket order (renumbered when the buckets
    // are rebuilt every few steps) and identified by their reference index at the API:
    // orig[s] = reference index of the particle stored in slot s, slotOf[r] = its slot.
    // Inside a bucket the stored particles are ordered by reference index, so every scan
    // visits them in the reference's order.
    int *orig, *slotOf;
    // buckets (stale list of the step): cellOf[i] = bucket, nB for a live particle in no
    // bucket (ghost type), -1 beyond the live count; cellStart has nB + 2 entries, the
    // range [cellStart[nB], cellStart[nB+1]) lists the live particles in no bucket
    int *cellOf, *cellStart, *cellCount, *cellSorted, *cellCursor;
    int* cellPos;      // inverse of cellSorted over the list (-1: slot not listed)
    // FP32 positions in bucket order (posfCell[s] = posf[cellSorted[s]]): the prefilter of
    // the 27-bucket scans reads contiguous 16-byte records and fetches the particle index
    // only for candidates that pass it
    float4* posfCell;
    // DF32 tier (float-float pair arithmetic): lo parts of the positions (posf holds the
    // hi parts) in particle and bucket order, velocity hi/lo parts, pressure as a
    // float-float pair, and the half-widths (m^2) of the decision margins of float-float
    // squared distances for the reS, reL, list and collision radii
    int prec;                       // MPSGPU_PRECISION_*
    // 1 inside a step between the prediction and the wall distance: every mirror is still the
    // far point the prediction wrote, so the collision's mirror-side test passes for every
    // pair and the collision does not read the mirror (the wall distance may be writing it)
    int mirrorFar;
    float4 *posLo, *posLoCell, *velHi, *velLo;
    dvec4 *c1n, *c2n, *c3n;         // correction matrix formed by the PND sweep, published by the
    float2* corrDFn;                // correction-matrix operator (pointer swap)
    float2* pressDF;
    float2* concDF;                 // shifting concentration as a float-float pair
    dvec4* normal;                  // fluid normal of the ARC free-surface test
    // start-of-step neighbour list with a skin (DF32 tier): candidates within reL + skin of
    // the start positions, in scan order; the viscosity sweep reads it, and the list of the
    // predicted positions is filtered from it while every particle stays within half the
    // skin of its start, no particle was removed and its bucket is unchanged
    float4* posSkin;                // start positions (hi parts)
    long long* skinCell;            // bucket coordinates of the start position (scan window)
    int* skinFlag;                  // [0] set: the skin list no longer covers the list
    float skinR2;                   // FP32 squared radius of the skin list (with the band)
    float skinMove2;                // FP32 squared displacement bound (half the skin, less the band)
    float invSidef, epsf;           // FP32 copies of invBucketSide and epsilonZero (bucket fast path)
    int dz3;                        // (int)(dim - 2): 1 in 3D (27 buckets), 0 in 2D (9)
    // out-of-domain bounds [min + bucket, max - bucket] (FP64, formed once as the reference does)
    double oodLo[3], oodHi[3];
    float mgS, mgL, mgMax, mgColl, mgSide;
    // float-float (hi, lo) constants of the DF32 sweeps, converted once on the host
    struct DfK {
        float2 reS, reL, invReS, invReL, reS2, reL2, reMax2, coll2;
        float2 neuW, neuF;          // viscosity: 2 mu / rho (wall neighbour), harmonic mean / rho
        float2 neuWall;             // wall viscosity coefficient
        float2 cPPE, cPPEg;         // coeffPPE, coeffPPE * DNS_FL1
        float2 g[3];
        float2 collF, collW;        // restitution * m_j / (m_i + m_j), fluid / wall neighbour
        float2 negCPG;              // -coeffPressGrad
    } k;
    float2* corrDF;                 // DF32 correction matrices: 9 values per particle, [c * N0 + i]
    // neighbour list (ELL) and its per-entry cache for the epoch: w(r; reS), w/r^2,
    // w(r; reL) (only when reL != reS)
    int *nbrCount, *nbr;
    int *skinCnt, *skinNbr;         // the start-of-step skin list (its own arrays once built)
    double *cw, *cwd, *cwL;
    // per-particle entry masks after the wall pass: bit k set when entry k is inside the
    // reS (maskS) / reL (maskL) ball and not on the mirror side
    Mask *maskS, *maskL;
    int *nearList, *nearCount;      // fluid particles near the polygon wall (compacted)
    double reMax2;                  // list radius^2 = max(reS^2, reL^2)
    float bandHiS, bandHiL;         // FP32 prefilter upper bounds for the reS / reL balls
    float bandHiColl;               // ... and for the collision distance
    // polygon mesh and wall tables
    int ntri;
    const double* tri;          // ntri * 9
    const double* triNormal;    // ntri * 3
    const double* triPlane;     // ntri * 16: unit normal and offset, three inward edge normals and offsets
    double wallReS, wallReL;    // sqrt(reS^2), sqrt(reL^2): the radii of the wall tables' interpolation
    const double* tab;          // xPND[50], Z[50], xNeigh[50], nNeigh[50] (as double)
    // meshes above MPS_MAX_TRI triangles: BVH nodes (FP32 boxes relative to domainMin, the
    // .w words hold child indices or leaf ranges), leaf order, FP32 triangle copies
    const float4 *bvhLo, *bvhHi;
    const int* bvhOrder;
    const float* triF;          // ntri * 9, relative to domainMin
    // prefilter band for the FP32 distance test (|d2f - reL2| <= band -> exact FP64)
    float reL2f, bandLo, bandHi;
    // scalars
    double* velMax;    // device scalar (written by the corrector)
    unsigned int* err; // error word
    double* redScratch;
    unsigned int* redCounter;
    unsigned long long* counters;   // [0] neighbour entries, [1] PPE off-diagonal non-zeros
};

// Warp-aggregated add of v into *ctr (one atomic per warp).
__device__ __forceinline__ void warpCount(unsigned long long* ctr, unsigned int v) {
    unsigned int m = __activemask();
    unsigned int s = __reduce_add_sync(m, v);   // valid for partial masks
    int lane = threadIdx.x & 31;
    if (lane == __ffs(m) - 1 && s) atomicAdd(ctr, (unsigned long long)s);
}

// ------------------------------------------------------------------ exact FP64
// Products and sums that decide a discrete outcome (bucket index, neighbour membership,
// mirror side, closest point) are evaluated with explicit round-to-nearest intrinsics
// so that no FMA contraction changes their rounding relative to the CPU reference.
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double xdot3(double ax, double ay, double az, double bx, double by, double bz) {
    return xadd(xadd(xmul(ax, bx), xmul(ay, by)), xmul(az, bz));
}
__device__ __forceinline__ double xnorm2(double x, double y, double z) { return xdot3(x, y, z, x, y, z); }

// ------------------------------------------------------------------ FP32 <-> FP64 conversions
// The conversion instructions run on the FP64 pipe, at 1/64 of the FP32 rate on GB300 like
// FP64 arithmetic; these build the same bits with integer operations.
// float -> double (exact: every float is a double; NaN payloads are kept).
__device__ __forceinline__ double f2dExact(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
    const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    unsigned long long b;
    if (e == 0xffu) b = s | 0x7ff0000000000000ull | ((unsigned long long)m << 29);   // inf, NaN
    else if (e != 0u) b = s | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
    else if (m == 0u) b = s;                                                           // +-0
    else {   // subnormal float m 2^-149: the leading one at bit p, exponent p - 149
        const int p = 31 - __clz((int)m);
        b = s | ((unsigned long long)(p + 874) << 52) | (((unsigned long long)m << (52 - p)) & 0xfffffffffffffull);
    }
    return __longlong_as_double((long long)b);
}
// double -> float rounded to nearest, ties to even (as __double2float_rn): the 52-bit
// significand rounded to 23 bits, a carry moving into the exponent (up to infinity);
// float-subnormal results shifted and rounded the same way; NaN gives the canonical NaN.
__device__ __forceinline__ float d2fRN(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned s = (unsigned)(b >> 32) & 0x80000000u;
    const unsigned E = (unsigned)(b >> 52) & 0x7ffu;
    const unsigned long long M = b & 0xfffffffffffffull;
    if (E == 0x7ffu) return __uint_as_float(M ? 0x7fffffffu : (s | 0x7f800000u));
    if (E >= 1151u) return __uint_as_float(s | 0x7f800000u);   // at least 2^128: infinity
    if (E < 897u) {                                            // below 2^-126: subnormal or zero
        if (E < 873u) return __uint_as_float(s);
        const unsigned long long m53 = M | (1ull << 52);
        const unsigned sh = 926u - E;                           // 30 .. 53
        unsigned long long q = m53 >> sh;
        const unsigned long long rem = m53 & ((1ull << sh) - 1ull), half = 1ull << (sh - 1u);
        q += (rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull;
        return __uint_as_float(s | (unsigned)q);
    }
    unsigned mh = (unsigned)(M >> 29);
    const unsigned rem = (unsigned)(M & 0x1fffffffu);
    mh += (rem > 0x10000000u || (rem == 0x10000000u && (mh & 1u))) ? 1u : 0u;
    return __uint_as_float(s | (((E - 896u) << 23) + mh));
}

// MpsBucket::bucketCoordinates, src/MpsBucket.cpp:420-425: (int)((x - min) * inv + eps)
__device__ __forceinline__ void bucketCoords(const MpsParams& P, double x, double y, double z,
                                             int& bx, int& by, int& bz) {
    bx = (int)xadd(xmul(xsub(x, P.domainMin[0]), P.invBucketSide), P.epsilonZero);
    by = (int)xadd(xmul(xsub(y, P.domainMin[1]), P.invBucketSide), P.epsilonZero);
    bz = (int)xadd(xmul(xsub(z, P.domainMin[2]), P.invBucketSide), P.epsilonZero);
}

// The same coordinates from hi = fl32(x - min) (the particle's current FP32 copy): the FP32
// quotient is within 4 * 2^-24 relative of the FP64 one, so its truncation is exact unless
// it lies within a margin of an integer (or below it), where the FP64 expression decides.
// The FP64 expressions sit out of line, for all three coordinates at once: inlined, the
// compiler predicates them into every call and their twelve FP64-pipe instructions then run
// for every particle.
static __device__ __noinline__ int3 bucketCoordsExact(const MpsParams& P, double x, double y, double z) {
    int3 b;
    bucketCoords(P, x, y, z, b.x, b.y, b.z);
    return b;
}
__device__ __forceinline__ bool bucketCoord1(float h, float inv, float eps, int& b) {
    const float q = fmaf(h, inv, eps);
    const float m = 5e-7f * fabsf(q) + 1e-6f;
    const float f = q - floorf(q);
    b = (int)q;
    return q > m && f > m && f < 1.0f - m;
}
__device__ __forceinline__ void bucketCoordsHi(const Dev& d, dvec4 p, float4 hi, int& bx, int& by, int& bz) {
    const bool ok = bucketCoord1(hi.x, d.invSidef, d.epsf, bx) & bucketCoord1(hi.y, d.invSidef, d.epsf, by) &
                    bucketCoord1(hi.z, d.invSidef, d.epsf, bz);
    if (!ok) {
        const int3 b = bucketCoordsExact(d.P, p.x, p.y, p.z);
        bx = b.x; by = b.y; bz = b.z;
    }
}

// PPE source of an equation row: PND deviation (src/MpsPressure.cpp:256), or with the
// velocity divergence and the previous PND for the PND + div u formulation (:388)
__device__ __forceinline__ double ppeSource(const Dev& d, int i, double rho) {
    const MpsParams& P = d.P;
    if (P.mpsType == 3)
        return -P.coeffPPESource * rho * (d.pndki[i] - P.pndSmallZero) +
               (1.0 - P.relaxPND) * rho * d.velDiv[i] / P.timeStep;
    return -P.coeffPPESource * rho * (d.pndSmall[i] - P.pndSmallZero);
}

// ------------------------------------------------------------------ weights
// MpsParticle::weight / delWeight, src/MpsParticle.cpp:57-108
__device__ __forceinline__ double wfun(double dst, double re, int t) {
    switch (t) {
        case 1: return re / dst + dst / re - 2.0;
        case 2: return re / dst - dst / re;
        case 3: { double a = 1.0 - dst / re; return a * a * a; }
        case 4: { double a = 1.0 - dst / re; return a * a; }
        default: return re / dst - 1.0;
    }
}
__device__ __forceinline__ double dwfun(double dst, double re, int t) {
    switch (t) {
        case 1: return -re / (dst * dst) + 1.0 / re;
        case 2: return -re / (dst * dst) - 1.0 / re;
        case 3: { double a = 1.0 - dst / re; return -3.0 / re * a * a; }
        case 4: return -2.0 / re * (1.0 - dst / re);
        default: return -re / (dst * dst);
    }
}

// ------------------------------------------------------------------ pairs
struct PairG {
    double v0, v1, v2, d2;   // r_ij = x_j - x_i and |r_ij|^2 (exact)
};
__device__ __forceinline__ PairG pairOf(dvec4 pj, dvec4 pi) {
    PairG q;
    q.v0 = xsub(pj.x, pi.x); q.v1 = xsub(pj.y, pi.y); q.v2 = xsub(pj.z, pi.z);
    q.d2 = xnorm2(q.v0, q.v1, q.v2);
    return q;
}
struct PairM {
    double m0, m1, m2, dm2;  // x_j - x_mirror(i) and its squared norm (exact)
};
__device__ __forceinline__ PairM pairMirror(dvec4 pj, dvec4 mi) {
    PairM q;
    q.m0 = xsub(pj.x, mi.x); q.m1 = xsub(pj.y, mi.y); q.m2 = xsub(pj.z, mi.z);
    q.dm2 = xnorm2(q.m0, q.m1, q.m2);
    return q;
}

// Per-particle context for the "j is not on the mirror side" test of every sweep
// (dstij2 < dstimj2 || wallType == PARTICLE, e.g. src/MpsPndNeigh.cpp:249).  When the
// mirror of i lies farther than 2.2 reL from i, every j within reL of i satisfies
// |x_j - m_i| >= |x_i - m_i| - r_ij > r_ij + 0.2 reL, so the test is skipped exactly.
struct SideCtx {
    dvec4 mi;
    bool check;
};
__device__ __forceinline__ SideCtx sideCtx(const Dev& d, int i, dvec4 pi) {
    SideCtx s;
    s.mi = d.mirror[i];
    if (d.P.wallType == 0) { s.check = false; return s; }
    double a = pi.x - s.mi.x, b = pi.y - s.mi.y, c = pi.z - s.mi.z;
    double lim = 2.2 * d.P.reL;
    s.check = (a * a + b * b + c * c) <= lim * lim;
    return s;
}
__device__ __forceinline__ bool sideOK(const SideCtx& s, dvec4 pj, double d2) {
    if (!s.check) return true;
    PairM m = pairMirror(pj, s.mi);
    return d2 < m.dm2;
}

__device__ __forceinline__ int liveN(const Dev& d) { return *d.nLive; }

// Iterate the ELL neighbour row of i (scan order of the reference).
// Streams read once per sweep (neighbour-list columns, matrix columns): loaded without L1
// allocation, so L1 keeps the lines of the gathered per-particle records.
__device__ __forceinline__ int ldStream(const int* p) {
    int v;
    asm("ld.global.nc.L1::no_allocate.s32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ float ldStream(const float* p) {
    float v;
    asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ double ldStream(const double* p) {
    double v;
    asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
}

template <class F>
__device__ __forceinline__ void forNbrs(const Dev& d, int i, F&& f) {
    int c = d.nbrCount[i];
    const int* row = d.nbr + i;
    for (int k = 0; k < c; k++) f(ldStream(row + (size_t)k * d.N0));
}
// The same with each entry's FP32 position copy, f(j, posf[j]): four entries' indices and
// gathers are issued before their bodies run (a body's stores would otherwise order the
// next gather after them).
template <class F>
__device__ __forceinline__ void forNbrsPosf(const Dev& d, int i, F&& f) {
    const int c = d.nbrCount[i];
    const int* row = d.nbr + i;
    int k = 0;
    for (; k + 4 <= c; k += 4) {
        int jj[4];
        float4 hh[4];
#pragma unroll
        for (int u = 0; u < 4; u++) jj[u] = ldStream(row + (size_t)(k + u) * d.N0);
#pragma unroll
        for (int u = 0; u < 4; u++) hh[u] = __ldg(&d.posf[jj[u]]);
#pragma unroll
        for (int u = 0; u < 4; u++) f(jj[u], hh[u]);
    }
    for (; k < c; k++) {
        const int j = ldStream(row + (size_t)k * d.N0);
        f(j, __ldg(&d.posf[j]));
    }
}

// Iterate the set bits of an entry mask in ascending entry order (the scan order).
// ELL matrix rows (PPE solvers, learned warm start)
// One ELL row, eight entries in flight: the column and value loads of a chunk are issued
// together, then the eight gathers; the last chunk is masked (predicated loads, the row's
// own index as a harmless column) instead of a serial remainder loop.  RO: the gathered
// vector is read-only for the launch (non-coherent cache path); otherwise plain loads.
// Entry k of row i sits at base + k * stride in val and col (base, stride: the layout's).
#define ELL_U 8
template <class T, bool RO>
__device__ __forceinline__ T ellRow(const T* diag, const T* val, const int* col, const T* x, int i, int len, size_t base,
                                    size_t stride) {
    T acc[ELL_U];
#pragma unroll
    for (int u = 0; u < ELL_U; u++) acc[u] = T(0);
    const T* v = val + base;
    const int* c = col + base;
    for (int k = 0; k < len; k += ELL_U) {
        // ask L2 for the next chunk's column and value lines while this chunk's gathers run
        if (k + ELL_U < len) {
#pragma unroll
            for (int u = 0; u < ELL_U; u++) {
                asm volatile("prefetch.global.L2 [%0];" ::"l"(c + (size_t)(k + ELL_U + u) * stride));
                asm volatile("prefetch.global.L2 [%0];" ::"l"(v + (size_t)(k + ELL_U + u) * stride));
            }
        }
        int cc[ELL_U];
        T vv[ELL_U];
#pragma unroll
        for (int u = 0; u < ELL_U; u++) {
            bool ok = k + u < len;
            cc[u] = ok ? ldStream(c + (size_t)(k + u) * stride) : i;
            vv[u] = ok ? ldStream(v + (size_t)(k + u) * stride) : T(0);
        }
#pragma unroll
        for (int u = 0; u < ELL_U; u++) acc[u] += vv[u] * (RO ? __ldg(x + cc[u]) : x[cc[u]]);
    }
    T xi = RO ? __ldg(x + i) : x[i];
    return __ldg(diag + i) * xi + (((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7])));
}

// f(j, e, k) for the entries k of the mask (e = k N0 + i, the entry's ELL index).
template <class F>
__device__ __forceinline__ void forMaskK(const Dev& d, int i, Mask m, F&& f) {
    const int* row = d.nbr + i;
    unsigned long long w = m.lo;   // entries 0..63, then 64..127 (rarely any)
    while (w) {
        const int k = __ffsll((long long)w) - 1;
        w &= w - 1ull;
        const size_t e = (size_t)k * d.N0 + i;
        f(ldStream(row + e - i), e, k);
    }
    w = m.hi;
    while (w) {
        const int k = __ffsll((long long)w) + 63;
        w &= w - 1ull;
        const size_t e = (size_t)k * d.N0 + i;
        f(ldStream(row + e - i), e, k);
    }
}
template <class F>
__device__ __forceinline__ void forMask(const Dev& d, int i, Mask m, F&& f) {
    forMaskK(d, i, m, [&](int j, size_t e, int) { f(j, e); });
}

// Weight for a squared distance through 1/r (rsqrt): w and w/r^2 (MpsParticle::weight,
// src/MpsParticle.cpp:57-72, evaluated as re*rinv - 1 for type 0).
__device__ __forceinline__ void weightR(double d2, double re, int t, double& w, double& wd) {
    double rinv = rsqrt(d2);
    double r = d2 * rinv;
    switch (t) {
        case 1: w = re * rinv + r / re - 2.0; break;
        case 2: w = re * rinv - r / re; break;
        case 3: { double a = 1.0 - r / re; w = a * a * a; } break;
        case 4: { double a = 1.0 - r / re; w = a * a; } break;
        default: w = re * rinv - 1.0; break;
    }
    wd = w * (rinv * rinv);
}

// Iterate the 27 (9 in 2D) buckets around x (bucketCoordinates of x) in the reference
// order, over the stale bucket list; out-of-grid bucket indices are skipped.
template <class F>
__device__ __forceinline__ void forCells(const Dev& d, dvec4 x, F&& f) {
    const MpsParams& P = d.P;
    int ix, iy, iz;
    bucketCoords(P, x.x, x.y, x.z, ix, iy, iz);
    int dz = (int)(P.dim - 2.0);
    int minZ = (iz - 1) * dz, maxZ = (iz + 1) * dz;
#pragma unroll 1
    for (int jz = minZ; jz <= maxZ; jz++)
#pragma unroll 1
        for (int jy = iy - 1; jy <= iy + 1; jy++)
#pragma unroll 1
            for (int jx = ix - 1; jx <= ix + 1; jx++) {
                long long jb = (long long)jz * P.numBucketsXY + (long long)jy * P.numBucketsX + jx;
                if (jb < 0 || jb >= d.nB) continue;
                int s0 = d.cellStart[jb], s1 = d.cellStart[jb + 1];
                for (int s = s0; s < s1; s++) f(__ldg(d.cellSorted + s));
            }
}

// 27-bucket scan with an FP32 prefilter: candidates whose FP32 squared distance (from the
// posf copy of the current positions) exceeds hi cannot be inside the ball; the others
// reach f(j, pj, q) with the exact FP64 pair, and f applies the reference's exact test.
template <class F>
__device__ __forceinline__ void forCellsNear(const Dev& d, dvec4 pi, float4 fi, float hi, F&& f) {
    const MpsParams& P = d.P;
    int ix, iy, iz;
    bucketCoords(P, pi.x, pi.y, pi.z, ix, iy, iz);
    int dz = (int)(P.dim - 2.0);
    int minZ = (iz - 1) * dz, maxZ = (iz + 1) * dz;
#pragma unroll 1
    for (int jz = minZ; jz <= maxZ; jz++)
#pragma unroll 1
        for (int jy = iy - 1; jy <= iy + 1; jy++)
#pragma unroll 1
            for (int jx = ix - 1; jx <= ix + 1; jx++) {
                long long jb = (long long)jz * P.numBucketsXY + (long long)jy * P.numBucketsX + jx;
                if (jb < 0 || jb >= d.nB) continue;
                int s0 = d.cellStart[jb], s1 = d.cellStart[jb + 1];
                for (int s = s0; s < s1; s++) {
                    float4 fj = __ldg(&d.posfCell[s]);
                    float ex = fj.x - fi.x, ey = fj.y - fi.y, ez = fj.z - fi.z;
                    if (ex * ex + ey * ey + ez * ez > hi) continue;
                    int j = __ldg(d.cellSorted + s);
                    dvec4 pj = d.pos[j];
                    f(j, pj, pairOf(pj, pi));
                }
            }
}

// Per-thread 27-bucket sweep driver: Op::begin/visit/end, Op::hi (prefilter bound) and
// Op::active (skip the scan for particles the sweep does not update).  visit receives
// the candidates that pass the FP32 prefilter, with the exact FP64 pair, j != i.
template <class Op>
__global__ void __launch_bounds__(128) k_scan(Dev d, Op op) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *d.nLive) return;
    typename Op::State st;
    op.begin(d, i, st);
    if (op.active(d, st))
        forCellsNear(d, d.pos[i], d.posf[i], op.hi(d), [&](int j, dvec4 pj, PairG q) {
            if (j != i) op.visit(d, i, st, j, pj, q);
        });
    op.end(d, i, st);
}
template <class Op>
void launchScan(const Dev& d, const Op& op, cudaStream_t s) {
    k_scan<Op><<<(d.N0 + 127) / 128, 128, 0, s>>>(d, op);
}

__device__ __forceinline__ void setErr(const Dev& d, unsigned int bit) { atomicOr(d.err, bit); }

// Reflection about the wall plane of i: n = (x_i - m_i)/2 normalised, R = I - 2 n n^T.
// useSqrt selects the normaliwSqrt > eps variant (src/MpsPndNeigh.cpp:118-131) or the
// normalMod2 > eps variant (src/MpsViscosity.cpp:1544-1556).
struct ReflG {
    double n[3], nsqrt, R[9];
};
__device__ __forceinline__ ReflG makeRefl(dvec4 xi, dvec4 mi, double eps, bool useSqrt) {
    ReflG r;
    r.n[0] = 0.5 * (xi.x - mi.x); r.n[1] = 0.5 * (xi.y - mi.y); r.n[2] = 0.5 * (xi.z - mi.z);
    double m2 = r.n[0] * r.n[0] + r.n[1] * r.n[1] + r.n[2] * r.n[2];
    double m = sqrt(m2);
    bool ok = useSqrt ? (m > eps) : (m2 > eps);
    r.nsqrt = useSqrt ? m : (ok ? m : 0.0);
    if (ok) { r.n[0] /= m; r.n[1] /= m; r.n[2] /= m; }
    else { r.n[0] = r.n[1] = r.n[2] = 0.0; }
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) r.R[a * 3 + b] = (a == b ? 1.0 : 0.0) - 2.0 * r.n[a] * r.n[b];
    return r;
}

// Repulsive wall force of MpsPressure::calcWallPressGradient (src/MpsPressure.cpp:1341-1611):
// f = -w n for a particle whose wall distance |x - m|/2 is below reRepulsiveForce.
__device__ __forceinline__ void wallRepulsion(const MpsParams& P, const ReflG& r, double vMax2, double f[3]) {
    f[0] = f[1] = f[2] = 0.0;
    double ns = r.nsqrt;
    if (ns < P.reRepulsiveForce && ns > P.epsilonZero) {
        double w;
        double rho = P.DNS_FL1;
        if (P.repulsiveForceType == 0) w = rho / (P.timeStep * P.timeStep) * (P.reRepulsiveForce - ns);
        else if (P.repulsiveForceType == 1) w = P.repForceCoefMitsume * wfun(ns, P.reRepulsiveForce, P.weightType);
        else if (P.repulsiveForceType == 2) {
            double R1 = (P.reRepulsiveForce / ns) * (P.reRepulsiveForce / ns);
            double R2 = R1 * R1;
            w = (P.repForceCoefLennardJones * vMax2 / ns) * (R2 - R1) * rho;
        } else {
            double a = 1.0 - ns / P.reRepulsiveForce;
            double W1 = (1.0 + 3.0 * 0.5 * ns / P.reRepulsiveForce), W2 = a * a * a;
            w = (P.repForceCoefMonaghanKajtar * vMax2 / (ns - 0.0 * P.partDist)) * (1.0 / 8.0) * W1 * W2 * rho;
        }
        f[0] = -w * r.n[0]; f[1] = -w * r.n[1]; f[2] = -w * r.n[2];
    }
}

// MpsVectorMatrix::correctionMatrix + inverseMatrix (Gauss-Jordan without pivoting,
// identity when det <= eps), src/MpsVectorMatrix.cpp:20-166
__device__ __forceinline__ void invert3(double* m, int dim, double eps) {
    double A[9], M[9];
#pragma unroll
    for (int k = 0; k < 9; k++) { A[k] = m[k]; M[k] = (k % 4 == 0) ? 1.0 : 0.0; }
    if (dim == 2) { A[2] = A[5] = A[6] = A[7] = 0.0; A[8] = 1.0; }
    double det = (A[0] * A[4] * A[8] + A[1] * A[5] * A[6] + A[2] * A[3] * A[7]) -
                 (A[2] * A[4] * A[6] + A[1] * A[3] * A[8] + A[0] * A[5] * A[7]);
    if (det <= eps) {
#pragma unroll
        for (int k = 0; k < 9; k++) m[k] = (k % 4 == 0) ? 1.0 : 0.0;
        return;
    }
    for (int k = 0; k < dim; k++)
        for (int r = 0; r < dim; r++) {
            if (r == k) continue;
            double f = A[r * 3 + k] / A[k * 3 + k];
            for (int c = 0; c < dim; c++) { A[r * 3 + c] -= f * A[k * 3 + c]; M[r * 3 + c] -= f * M[k * 3 + c]; }
        }
    for (int r = 0; r < dim; r++)
        for (int c = 0; c < dim; c++) M[r * 3 + c] /= A[r * 3 + r];
#pragma unroll
    for (int k = 0; k < 9; k++) m[k] = M[k];
}
static inline int gridFor(int n, int block) { return (n + block - 1) / block; }
