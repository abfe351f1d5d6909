// mps_ops_df.cu — the DF32 precision tier of the neighbour sweeps on sm_103a.
//
// Same operators, same reference order and same discrete decisions as mps_ops.cu, with
// the per-pair arithmetic in float-float (mps_df.cuh) instead of FP64: pair vectors come
// from the hi/lo position copies, weights are recomputed per entry from the float-float
// squared distance (no per-entry weight cache: FP32 work is cheaper than its HBM traffic),
// sums are float-float and each particle's result is assembled in FP64 once.  Radius and
// mirror-side decisions whose float-float value lies within the error margin fall back to
// the reference's FP64 expression, so entry sets, masks and flags equal the FP64 tier's.
#include "mps_df.cuh"
#include "mps_internal.h"

#define BLK 128

// ------------------------------------------------------------------ copies
__global__ void k_df_vel(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N0) return;
    dvec4 v = d.vel[i];
    float4 h = make_float4(d2fRN(v.x), d2fRN(v.y), d2fRN(v.z), 0.f);
    d.velHi[i] = h;
    d.velLo[i] = make_float4(d2fRN(v.x - f2dExact(h.x)), d2fRN(v.y - f2dExact(h.y)), d2fRN(v.z - f2dExact(h.z)), 0.f);
}
__global__ void k_df_press(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N0) return;
    df p = dfD(d.press[i]);
    d.pressDF[i] = make_float2(p.h, p.l);
}
static void launchVelDF(const Dev& d, cudaStream_t s) { k_df_vel<<<gridFor(d.N0, 256), 256, 0, s>>>(d); }
static void launchPressDF(const Dev& d, cudaStream_t s) { k_df_press<<<gridFor(d.N0, 256), 256, 0, s>>>(d); }

__device__ __forceinline__ df K(float2 v) { return {v.x, v.y}; }
__device__ __forceinline__ df loadDF(const float2* p, int j) {
    float2 v = __ldg(p + j);
    return {v.x, v.y};
}

// ------------------------------------------------------------------ neighbour list
// The list of the current positions through the stale buckets: candidates whose FP32
// squared distance is below the band are members, those above it were never seen by the
// prefilter, and only the band's few candidates are decided in float-float (and, inside
// the float-float margin, in FP64).  No per-entry weights: the DF32 sweeps recompute them.
template <bool STRAY>
__global__ void __launch_bounds__(128) k_build_nbr_df(Dev d) {
    const int i = scanParticle<STRAY>(d);
    if (i < 0) return;
    dvec4 pi = d.pos[i];
    float4 hi = d.posf[i], li = d.posLo[i];
    const df R2 = K(d.k.reMax2);
    int cnt = 0;
    const size_t N0 = d.N0;
    forCellsDF(d, pi, hi, d.bandHi, [&](int j, int s, float4 hj) {
        if (j == i) return;
        float ex = hj.x - hi.x, ey = hj.y - hi.y, ez = hj.z - hi.z;
        if (!(ex * ex + ey * ey + ez * ez < d.bandLo)) {
            PairF q = pairDF(hj, __ldg(&d.posLoCell[s]), hi, li);
            if (!inBallDF(d, q.d2, R2, d.mgMax, d.reMax2, i, j)) return;
        }
        if (cnt < d.K) d.nbr[(size_t)cnt * N0 + i] = j;
        cnt++;
    });
    if (cnt > d.K) { setErr(d, MPSE_CAPACITY); cnt = d.K; }
    d.nbrCount[i] = cnt;
    warpCount(d.counters, (unsigned)cnt);
}
void launchNeighborListDF(const Dev& d, cudaStream_t s) {
    cudaMemsetAsync(d.counters, 0, sizeof(unsigned long long), s);
    launchPosf(d, s);
    k_build_nbr_df<false><<<gridFor(d.N0, 128), 128, 0, s>>>(d);
    k_build_nbr_df<true><<<gridFor(d.N0, 128), 128, 0, s>>>(d);
}

// ------------------------------------------------------------------ entry masks
__global__ void __launch_bounds__(128, 10) k_side_masks_df(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    int c = d.nbrCount[i];
    const Mask all = maskFirst(c);
    dvec4 pi = d.pos[i];
    SideDF sc = sideDF(d, i, pi);
    bool fullS = P.reS2 >= d.reMax2, fullL = P.reL2 >= d.reMax2;
    Mask mS = all, mL = all;
    if (sc.check || !fullS || !fullL) {
        mS = maskNone(); mL = maskNone();
        float4 hi = d.posf[i], li = d.posLo[i];
        const df RS = K(d.k.reS2), RL = K(d.k.reL2);
        const int* row = d.nbr + i;
        for (int k = 0; k < c; k++) {
            int j = ldStream(row + (size_t)k * d.N0);
            float4 hj = d.posf[j], lj = d.posLo[j];
            df d2 = norm2(diff3(hj, lj, hi, li));
            if (!sideOkDF(d, sc, hj, lj, d2, i, j)) continue;
            if (fullS || inBallDF(d, d2, RS, d.mgS, P.reS2, i, j)) maskSet(mS, k);
            if (fullL || inBallDF(d, d2, RL, d.mgL, P.reL2, i, j)) maskSet(mL, k);
        }
    }
    d.maskS[i] = mS;
    d.maskL[i] = mL;
    if (P.wallType == 1 && d.type[i] == P.fluid && d.nearWall[i]) {
        int slot = atomicAdd(d.nearCount, 1);
        d.nearList[slot] = i;
    }
}
void launchSideMasksDF(const Dev& d, cudaStream_t s) {
    cudaMemsetAsync(d.nearCount, 0, sizeof(int), s);
    k_side_masks_df<<<gridFor(d.N0, 128), 128, 0, s>>>(d);
}

// ------------------------------------------------------------------ viscosity
// MpsViscosity::calcViscosity, src/MpsViscosity.cpp:20-100, at the start-of-step
// positions through the 27 buckets (Newtonian: uniform MEU and RHO).  Two phases per
// batch: the FP32 prefilter compacts the surviving slots of the thread's candidates into
// its shared-memory column (bucket order kept), then the float-float pair work runs over
// the compacted slots, so the lanes of a warp stay converged through the expensive part.
#define VCAP 48
#define VBLK 128
template <bool STRAY>
__global__ void __launch_bounds__(VBLK) k_visc_df(Dev d) {
    __shared__ int slots[VCAP * VBLK];
    const int t = threadIdx.x;
    const int i = scanParticle<STRAY>(d);
    if (i < 0) return;
    const MpsParams& P = d.P;
    const dvec4 pi = d.pos[i];
    const float4 hi = d.posf[i], li = d.posLo[i];
    const float4 vh = d.velHi[i], vl = d.velLo[i];
    const SideDF sc = sideDF(d, i, pi);
    const df R2 = K(d.k.reL2), neuW = K(d.k.neuW), neuF = K(d.k.neuF);
    const RadiusDF RL = {K(d.k.reL), K(d.k.invReL)};
    const float band = d.bandHiL;
    df ax = dfF(0.f), ay = dfF(0.f), az = dfF(0.f);
    int ix, iy, iz;
    bucketCoordsHi(d, pi, hi, ix, iy, iz);
    const int dz = (int)(P.dim - 2.0);
    const int nbk = dz ? 27 : 9;
    int bk = 0, s = 0, s1 = 0;
    bool more = true;
    while (more) {
        int n = 0;
        while (n < VCAP) {
            if (s >= s1) {
                if (bk >= nbk) { more = false; break; }
                int kz = bk / 9, ky = (bk / 3) % 3, kx = bk % 3;
                bk++;
                long long jb = (long long)((iz - 1) * dz + kz) * P.numBucketsXY +
                               (long long)(iy - 1 + ky) * P.numBucketsX + (ix - 1 + kx);
                if (jb < 0 || jb >= d.nB) continue;
                s = d.cellStart[jb];
                s1 = d.cellStart[jb + 1];
                continue;
            }
            float4 fj = __ldg(&d.posfCell[s]);
            float ex = fj.x - hi.x, ey = fj.y - hi.y, ez = fj.z - hi.z;
            if (ex * ex + ey * ey + ez * ez <= band) slots[n++ * VBLK + t] = s;
            s++;
        }
        for (int k = 0; k < n; k++) {
            const int sk = slots[k * VBLK + t];
            const int j = __ldg(d.cellSorted + sk);
            if (j == i) continue;
            const float4 hj = __ldg(&d.posfCell[sk]), lj = __ldg(&d.posLoCell[sk]);
            PairF q = pairDF(hj, lj, hi, li);
            if (!inBallDF(d, q.d2, R2, d.mgL, P.reL2, i, j)) continue;
            if (!sideOkDF(d, sc, hj, lj, q.d2, i, j)) continue;
            WeightDF w = weightDF(q.d2, RL, P.weightType);
            df c = w.w * ((d.type[j] == P.wall) ? neuW : neuF);
            float4 vhj = d.velHi[j], vlj = d.velLo[j];
            ax += diffDF(vhj.x, vlj.x, vh.x, vl.x) * c;
            ay += diffDF(vhj.y, vlj.y, vh.y, vl.y) * c;
            az += diffDF(vhj.z, vlj.z, vh.z, vl.z) * c;
        }
    }
    double cv = P.coeffViscMultiphase;
    d.acc[i] = make_dvec4(cv * dD(ax), cv * dD(ay), cv * dD(az), 0.0);
}
void launchViscosityDF(const Dev& d, cudaStream_t s) {
    launchVelDF(d, s);
    k_visc_df<false><<<gridFor(d.N0, VBLK), VBLK, 0, s>>>(d);
    k_visc_df<true><<<gridFor(d.N0, VBLK), VBLK, 0, s>>>(d);
}

// ------------------------------------------------------------------ collision
// MpsParticleCollision::checkParticleCollisions, src/MpsParticleCollision.cpp:22-119.
// The sign test fDT > 0 is decided in float-float outside a margin that bounds the
// difference from the FP64 value, and in FP64 inside it.
__global__ void __launch_bounds__(BLK) k_collision_df(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    df dvx = dfF(0.f), dvy = dfF(0.f), dvz = dfF(0.f);
    bool any = false;
    if (d.type[i] == P.fluid) {
        dvec4 pi = d.pos[i];
        float4 hi = d.posf[i], li = d.posLo[i];
        float4 vh = d.velHi[i], vl = d.velLo[i];
        float vin = fabsf(vh.x) + fabsf(vh.y) + fabsf(vh.z);
        const SideDF sc = d.mirrorFar ? SideDF{} : sideDF(d, i, pi);   // {}: no side test
        const df R2 = K(d.k.coll2), cF = K(d.k.collF), cW = K(d.k.collW);
        forNbrsPosf(d, i, [&](int j, float4 hj) {
            // FP32 prefilter: most list entries lie beyond the collision distance
            const float ex = hj.x - hi.x, ey = hj.y - hi.y, ez = hj.z - hi.z;
            if (ex * ex + ey * ey + ez * ez > d.bandHiColl) return;
            const float4 lj = __ldg(&d.posLo[j]);
            PairF q = pairDF(hj, lj, hi, li);
            if (!inBallDF(d, q.d2, R2, d.mgColl, P.distCollisionLimit2, i, j)) return;
            if (!sideOkDF(d, sc, hj, lj, q.d2, i, j)) return;
            float4 vhj = d.velHi[j], vlj = d.velLo[j];
            V3 dv = {diffDF(vh.x, vl.x, vhj.x, vlj.x), diffDF(vh.y, vl.y, vhj.y, vlj.y),
                     diffDF(vh.z, vl.z, vhj.z, vlj.z)};
            df fDT = dot3(dv, q.v);
            float rn = fabsf(q.v.x.h) + fabsf(q.v.y.h) + fabsf(q.v.z.h);
            float dn = fabsf(dv.x.h) + fabsf(dv.y.h) + fabsf(dv.z.h);
            float vjn = fabsf(vhj.x) + fabsf(vhj.y) + fabsf(vhj.z);
            float mg = 1e-9f * dn * rn + 1e-11f * (vin + vjn) * rn;
            bool pos;
            if (fDT.h > mg) pos = true;
            else if (fDT.h < -mg) pos = false;
            else {
                dvec4 pj = d.pos[j], vj = d.vel[j], vi = d.vel[i];
                PairG g = pairOf(pj, pi);
                pos = (vi.x - vj.x) * g.v0 + (vi.y - vj.y) * g.v1 + (vi.z - vj.z) * g.v2 > 0.0;
            }
            if (!pos) return;
            bool jf = d.type[j] == P.fluid;
            df rinv = rsqrtDF(q.d2);
            df k = fDT * (jf ? cF : cW) * (rinv * rinv);
            if (!jf) k = k * 2.0f;
            dvx -= q.v.x * k; dvy -= q.v.y * k; dvz -= q.v.z * k;
            any = true;
        });
    }
    d.dvel[i] = any ? make_dvec4(dD(dvx), dD(dvy), dD(dvz), 0.0) : make_dvec4(0, 0, 0, 0);
}
void launchCollisionDF(const Dev& d, cudaStream_t s) {
    launchVelDF(d, s);
    k_collision_df<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
    launchCollisionApply(d, s);
}

// ------------------------------------------------------------------ wall sweeps
__device__ __forceinline__ int nearIndexDF(const Dev& d) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    return (t < *d.nearCount) ? d.nearList[t] : -1;
}
struct MirrorDF {
    float4 mh, ml;
};
__device__ __forceinline__ MirrorDF mirrorDF(const Dev& d, dvec4 m) {
    MirrorDF o;
    const MpsParams& P = d.P;
    o.mh = make_float4(d2fRN(m.x - P.domainMin[0]), d2fRN(m.y - P.domainMin[1]), d2fRN(m.z - P.domainMin[2]), 0.f);
    o.ml = posLoOf(m, o.mh, P);
    return o;
}
// One wall-sweep entry: j within R of i, its mirror image within R of the mirror of i
// and j not on the mirror side (e.g. src/MpsPndNeigh.cpp:140-160).  Returns the mirror
// pair (x_j - m_i, |x_j - m_i|^2) through m.
// hj: the entry's FP32 copy (posf[j]); band: the FP32 upper bound of the radius R (an
// entry above it is outside the ball, and its lo part is never read)
__device__ __forceinline__ bool wallEntryDF(const Dev& d, int i, int j, float4 hj, float4 hi, float4 li,
                                            const MirrorDF& M, df R2f, float mg, double R2, float band, PairF& m) {
    const float ex = hj.x - hi.x, ey = hj.y - hi.y, ez = hj.z - hi.z;
    if (ex * ex + ey * ey + ez * ez > band) return false;
    const float4 lj = __ldg(&d.posLo[j]);
    PairF q = pairDF(hj, lj, hi, li);
    if (!inBallDF(d, q.d2, R2f, mg, R2, i, j)) return false;
    m = pairDF(hj, lj, M.mh, M.ml);
    if (!lessDF(m.d2, R2f, mg, [&] { return pairMirror(d.pos[j], d.mirror[i]).dm2 < R2; })) return false;
    return lessDF(q.d2, m.d2, d.mgSide, [&] {
        dvec4 pj = d.pos[j];
        return pairOf(pj, d.pos[i]).d2 < pairMirror(pj, d.mirror[i]).dm2;
    });
}

// MpsPndNeigh::calcWallNPCD, src/MpsPndNeigh.cpp:105-195
__global__ void __launch_bounds__(BLK) k_wall_npcd_df(Dev d) {
    int i = nearIndexDF(d);
    if (i < 0) return;
    const MpsParams& P = d.P;
    dvec4 pi = d.pos[i], mi = d.mirror[i];
    ReflG r = makeRefl(pi, mi, P.epsilonZero, true);
    float4 hi = d.posf[i], li = d.posLo[i];
    MirrorDF M = mirrorDF(d, mi);
    const df R2 = K(d.k.reS2);
    const RadiusDF RS = {K(d.k.reS), K(d.k.invReS)};
    df sx = dfF(0.f), sy = dfF(0.f), sz = dfF(0.f);
    forNbrsPosf(d, i, [&](int j, float4 hj) {
        PairF m;
        if (!wallEntryDF(d, i, j, hj, hi, li, M, R2, d.mgS, P.reS2, d.bandHiS, m)) return;
        df wS = weightDF(m.d2, RS, P.weightType).w;
        sx += m.v.x * wS; sy += m.v.y * wS; sz += m.v.z * wS;
    });
    double dx = dD(sx), dy = dD(sy), dz = dD(sz);
    PairM s = pairMirror(pi, mi);
    if (s.dm2 < P.reS2) {
        double wS = wfun(sqrt(s.dm2), P.reS, P.weightType);
        dx += s.m0 * wS; dy += s.m1 * wS; dz += s.m2 * wS;
    }
    dvec4 n = d.npcd[i];
    n.x += r.R[0] * dx + r.R[1] * dy + r.R[2] * dz;
    n.y += r.R[3] * dx + r.R[4] * dy + r.R[5] * dz;
    n.z += r.R[6] * dx + r.R[7] * dy + r.R[8] * dz;
    d.npcd[i] = n;
}
void launchWallNpcdDF(const Dev& d, cudaStream_t s) {
    if (d.P.wallType != 1) return;
    k_wall_npcd_df<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
}

// ------------------------------------------------------------------ correction matrix
// MpsVectorMatrix::correctionMatrix + inverseMatrix, src/MpsVectorMatrix.cpp:20-166: the
// moment matrix sum w/r^2 r r^T is accumulated in float-float and inverted through its
// adjugate in float-float (the reference eliminates without pivoting; both give the
// inverse to rounding), identity when det <= eps or numNeigh < 4.  The FP64 copy is the
// operator's output; the float-float copy feeds the DF32 pressure gradient.
__device__ __forceinline__ df recipDF(df a) {
    float y = 1.0f / a.h;
    df t = a * y;                              // ~1
    float e = fS(fS(1.0f, t.h), t.l);          // 1 - a y
    return quick2(y, fM(y, e));
}
__device__ __forceinline__ void corrFinish(const Dev& d, int i, int numNeigh, df m00, df m01, df m02, df m11,
                                           df m12, df m22, dvec4* c1, dvec4* c2, dvec4* c3, float2* cdf);
__global__ void __launch_bounds__(BLK) k_corr_matrix_df(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    float4 hi = d.posf[i], li = d.posLo[i];
    const RadiusDF RS = {K(d.k.reS), K(d.k.invReS)};
    df m00 = dfF(0.f), m01 = m00, m02 = m00, m11 = m00, m12 = m00, m22 = m00;
    forMask(d, i, d.maskS[i], [&](int j, size_t) {
        PairF q = pairDF(d.posf[j], d.posLo[j], hi, li);
        df wd = weightDF(q.d2, RS, P.weightType).wr2;
        df t0 = q.v.x * wd, t1 = q.v.y * wd, t2 = q.v.z * wd;
        m00 += t0 * q.v.x; m01 += t0 * q.v.y; m02 += t0 * q.v.z;
        m11 += t1 * q.v.y; m12 += t1 * q.v.z; m22 += t2 * q.v.z;
    });
    corrFinish(d, i, d.numNeigh[i], m00, m01, m02, m11, m12, m22, d.c1, d.c2, d.c3, d.corrDF);
}
// inverse of -coeffPressGrad * the moment matrix (identity when det <= eps or fewer than
// four neighbours), written as the FP64 rows and the float-float copy
__device__ __forceinline__ void corrFinish(const Dev& d, int i, int numNeigh, df m00, df m01, df m02, df m11,
                                           df m12, df m22, dvec4* c1, dvec4* c2, dvec4* c3, float2* cdf) {
    const MpsParams& P = d.P;
    const df c = K(d.k.negCPG);
    df A[9];
    A[0] = m00 * c; A[1] = m01 * c; A[2] = m02 * c;
    A[4] = m11 * c; A[5] = m12 * c; A[8] = m22 * c;
    A[3] = A[1]; A[6] = A[2]; A[7] = A[5];
    if (P.dim == 2) { A[2] = A[5] = A[6] = A[7] = dfF(0.f); A[8] = dfF(1.f); }
    df det = (A[0] * A[4] * A[8] + A[1] * A[5] * A[6] + A[2] * A[3] * A[7]) -
             (A[2] * A[4] * A[6] + A[1] * A[3] * A[8] + A[0] * A[5] * A[7]);
    df M[9];
    bool ident = numNeigh < 4 || !(det.h > (float)P.epsilonZero);
    if (ident) {
#pragma unroll
        for (int k = 0; k < 9; k++) M[k] = dfF((k % 4 == 0) ? 1.f : 0.f);
    } else {
        df r = recipDF(det);
        M[0] = (A[4] * A[8] - A[5] * A[7]) * r; M[1] = (A[2] * A[7] - A[1] * A[8]) * r;
        M[2] = (A[1] * A[5] - A[2] * A[4]) * r; M[3] = (A[5] * A[6] - A[3] * A[8]) * r;
        M[4] = (A[0] * A[8] - A[2] * A[6]) * r; M[5] = (A[2] * A[3] - A[0] * A[5]) * r;
        M[6] = (A[3] * A[7] - A[4] * A[6]) * r; M[7] = (A[1] * A[6] - A[0] * A[7]) * r;
        M[8] = (A[0] * A[4] - A[1] * A[3]) * r;
    }
#pragma unroll
    for (int k = 0; k < 9; k++) cdf[(size_t)k * d.N0 + i] = make_float2(M[k].h, M[k].l);
    c1[i] = make_dvec4(dD(M[0]), dD(M[1]), dD(M[2]), 0.0);
    c2[i] = make_dvec4(dD(M[3]), dD(M[4]), dD(M[5]), 0.0);
    c3[i] = make_dvec4(dD(M[6]), dD(M[7]), dD(M[8]), 0.0);
}
// float-float copy of matrices written through the field interface
__global__ void k_df_corr(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N0) return;
    dvec4 r[3] = {d.c1[i], d.c2[i], d.c3[i]};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        df x = dfD(r[a].x), y = dfD(r[a].y), z = dfD(r[a].z);
        d.corrDF[(size_t)(3 * a) * d.N0 + i] = make_float2(x.h, x.l);
        d.corrDF[(size_t)(3 * a + 1) * d.N0 + i] = make_float2(y.h, y.l);
        d.corrDF[(size_t)(3 * a + 2) * d.N0 + i] = make_float2(z.h, z.l);
    }
}
void launchCorrDF(const Dev& d, cudaStream_t s) { k_df_corr<<<gridFor(d.N0, 256), 256, 0, s>>>(d); }
void launchCorrectionMatrixDF(const Dev& d, cudaStream_t s) { k_corr_matrix_df<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d); }

// ------------------------------------------------------------------ PND / NPCD
// MpsPndNeigh::calcPndnNeighNPCD, src/MpsPndNeigh.cpp:199-331
// CORR: the correction matrix's moment sums over the reS entries in the same pass (one
// pair evaluation serves both; the PND sums take the entries also inside reL, in the same
// ascending order as the plain sweep, so both results equal the separate kernels').
template <bool CORR>
__global__ void __launch_bounds__(BLK, 9) k_pnd_npcd_df(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    float4 hi = d.posf[i], li = d.posLo[i];
    const RadiusDF RS = {K(d.k.reS), K(d.k.invReS)};
    const Mask mL = d.maskL[i];
    int nn = d.nNeighWall[i] + maskCount(mL);
    df ni = dfF(0.f), nx = ni, ny = ni, nz = ni;
    df m00 = dfF(0.f), m01 = m00, m02 = m00, m11 = m00, m12 = m00, m22 = m00;
    if (CORR) {
        Mask m = d.maskS[i];
        const int* row = d.nbr + i;
        int k;
        while ((k = maskPop(m)) >= 0) {
            const int j = ldStream(row + (size_t)k * d.N0);
            PairF q = pairDF(d.posf[j], d.posLo[j], hi, li);
            WeightDF w = weightDF(q.d2, RS, P.weightType);
            df t0 = q.v.x * w.wr2, t1 = q.v.y * w.wr2, t2 = q.v.z * w.wr2;
            m00 += t0 * q.v.x; m01 += t0 * q.v.y; m02 += t0 * q.v.z;
            m11 += t1 * q.v.y; m12 += t1 * q.v.z; m22 += t2 * q.v.z;
            if (maskHas(mL, k)) {
                ni += w.w;
                nx += q.v.x * w.w; ny += q.v.y * w.w; nz += q.v.z * w.w;
            }
        }
    } else {
        forMask(d, i, mL & d.maskS[i], [&](int j, size_t) {
            PairF q = pairDF(d.posf[j], d.posLo[j], hi, li);
            df wS = weightDF(q.d2, RS, P.weightType).w;
            ni += wS;
            nx += q.v.x * wS; ny += q.v.y * wS; nz += q.v.z * wS;
        });
    }
    double nd = dD(ni);
    dvec4 np = d.npcd[i];
    np.x += dD(nx); np.y += dD(ny); np.z += dD(nz);
    if (P.pndType == 0 || P.pndType == 1) {
        d.pndki[i] = d.pndi[i];
        d.pndi[i] = nd + d.pndWall[i];
    }
    double pndSmall = nd + d.pndWall[i];
    d.pndSmall[i] = pndSmall;
    d.numNeigh[i] = nn;
    if (nd > P.epsilonZero) { np.x /= pndSmall; np.y /= pndSmall; np.z /= pndSmall; }
    d.npcd[i] = np;
    d.npcd2[i] = np.x * np.x + np.y * np.y + np.z * np.z;
    dvec4 nw = d.polyNormal[i];
    d.devDot[i] = (np.x * nw.x + np.y * nw.y + np.z * nw.z < 0.0) ? 1.0 : -1.0;
    // into the staging arrays: the correction-matrix operator publishes them (the reference
    // writes the matrix there, not in this sweep)
    if (CORR) corrFinish(d, i, nn, m00, m01, m02, m11, m12, m22, d.c1n, d.c2n, d.c3n, d.corrDFn);
}
void launchPndNeighNpcdDF(const Dev& d, cudaStream_t s, bool withCorrection) {
    if (withCorrection) k_pnd_npcd_df<true><<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
    else k_pnd_npcd_df<false><<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
}

// ------------------------------------------------------------------ PPE assembly
// MpsPressure::solvePressurePoissonPnd, src/MpsPressure.cpp:169-286 (matrix values are
// assembled in float-float and stored in FP64)
__global__ void __launch_bounds__(128, 12) k_ppe_assemble_df(Dev d, PpeBuffers B) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    int bci = d.bc[i];
    if (bci == P.other || bci == P.surface) {
        B.diag[i] = 1.0; B.diagf[i] = 1.0f; B.diagInvf[i] = 1.0f; B.rowLen[i] = 0; B.b[i] = 0.0; B.mfMask[i] = maskNone();
        warpCount(d.counters + 1, 0u);
        return;
    }
    float4 hi = d.posf[i], li = d.posLo[i];
    const RadiusDF RL = {K(d.k.reL), K(d.k.invReL)};
    const df cP = K(d.k.cPPE), cG = K(d.k.cPPEg);
    const df gx = K(d.k.g[0]), gy = K(d.k.g[1]), gz = K(d.k.g[2]);
    df sum = dfF(0.f), src = dfF(0.f);
    int len = 0;
    Mask mm = maskNone();
    forMaskK(d, i, d.maskL[i], [&](int j, size_t, int ke) {
        PairF q = pairDF(d.posf[j], d.posLo[j], hi, li);
        df wL = weightDF(q.d2, RL, P.weightType).w;
        if (d.type[j] == P.dummyWall) {
            src -= (q.v.x * gx + q.v.y * gy + q.v.z * gz) * wL * cG;
        } else {
            df mij = wL * cP;
            sum -= mij;
            if (d.bc[j] == P.inner) {
                size_t k = ellBase(B, i) + (size_t)len * B.ellStride;
                B.val[k] = dD(mij);
                B.valf[k] = mij.h;   // the FP32 copy of the mixed solver (hi part = fl32)
                B.col[k] = j;
                len++;
                maskSet(mm, ke);
            }
        }
    });
    B.mfMask[i] = mm;
    double rho = P.DNS_FL1;
    double dg = dD(sum) - P.alphaCompressibility * rho / (P.timeStep * P.timeStep);
    B.diag[i] = dg;
    B.diagf[i] = (float)dg;
    B.diagInvf[i] = 1.0f / (float)dg;
    B.rowLen[i] = len;
    B.b[i] = dD(src) + ppeSource(d, i, rho);
    warpCount(d.counters + 1, (unsigned)len);
}
void launchPpeAssembleDF(const Dev& d, const PpeBuffers& B, cudaStream_t s) {
    cudaMemsetAsync(d.counters + 1, 0, sizeof(unsigned long long), s);
    k_ppe_assemble_df<<<gridFor(d.N0, 128), 128, 0, s>>>(d, B);
}

// ------------------------------------------------------------------ pressure gradient
// MpsPressure::calcPressGradient, src/MpsPressure.cpp:1217-1338
__global__ void __launch_bounds__(BLK, 9) k_press_grad_df(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    float4 hi = d.posf[i], li = d.posLo[i];
    const RadiusDF RS = {K(d.k.reS), K(d.k.invReS)};
    df Pi = loadDF(d.pressDF, i), pmin = Pi;
    double ni = d.pndi[i];
    int gt = P.gradientType;
    const Mask mS = d.maskS[i];
    if (gt == 0 || gt == 2) {
        forMask(d, i, mS, [&](int j, size_t) {
            df pj = loadDF(d.pressDF, j);
            if (pmin > pj) pmin = pj;
        });
    }
    df base = (gt == 0) ? -pmin : (gt == 1 ? Pi : Pi - pmin - pmin);
    // sum of r_ij f_ij; with gradient correction C (constant per particle) is applied to
    // the sum once: sum (C r) f = C (sum r f)
    df ax = dfF(0.f), ay = ax, az = ax;
    forMask(d, i, mS, [&](int j, size_t) {
        PairF q = pairDF(d.posf[j], d.posLo[j], hi, li);
        WeightDF w = weightDF(q.d2, RS, P.weightType);
        df f;
        if (gt <= 2) f = (loadDF(d.pressDF, j) + base) * w.wr2;
        else {
            double nj = d.pndi[j], Pj = d.press[j], Pid = d.press[i];
            f = (ni > P.epsilonZero && nj > P.epsilonZero) ? dfD(ni * Pj / nj + nj * Pid / ni) * w.wr2 : w.w;
        }
        ax += q.v.x * f; ay += q.v.y * f; az += q.v.z * f;
    });
    if (P.gradientCorrection) {
        df C[9];
#pragma unroll
        for (int k = 0; k < 9; k++) C[k] = loadDF(d.corrDF + (size_t)k * d.N0, i);
        df bx = C[0] * ax + C[1] * ay + C[2] * az;
        df by = C[3] * ax + C[4] * ay + C[5] * az;
        df bz = C[6] * ax + C[7] * ay + C[8] * az;
        ax = bx; ay = by; az = bz;
    }
    double c = P.relaxPress * P.coeffPressGrad / P.DNS_FL1;
    d.acc[i] = make_dvec4(dD(ax) * c, dD(ay) * c, dD(az) * c, 0.0);
}
void launchPressGradientDF(const Dev& d, cudaStream_t s) {
    launchPressDF(d, s);
    k_press_grad_df<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
}

// MpsPressure::calcWallPressGradient + repulsive forces, src/MpsPressure.cpp:1341-1611
__global__ void __launch_bounds__(BLK) k_wall_press_grad_df(Dev d) {
    int i = nearIndexDF(d);
    if (i < 0) return;
    const MpsParams& P = d.P;
    double vm = fmin(*d.velMax, P.expectMaxVelocity);
    double vMax2 = vm * vm;
    dvec4 pi = d.pos[i], mi = d.mirror[i];
    float4 hi = d.posf[i], li = d.posLo[i];
    MirrorDF M = mirrorDF(d, mi);
    const df R2 = K(d.k.reS2);
    const RadiusDF RS = {K(d.k.reS), K(d.k.invReS)};
    double Pid = d.press[i], ni = d.pndi[i];
    df Pi = loadDF(d.pressDF, i), pmin = Pi;
    int gt = P.gradientType;
    ReflG r = makeRefl(pi, mi, P.epsilonZero, true);
    if (gt == 0 || gt == 2) {
        forNbrs(d, i, [&](int j) {
            float4 hj = d.posf[j], lj = d.posLo[j];
            PairF q = pairDF(hj, lj, hi, li);
            if (!inBallDF(d, q.d2, R2, d.mgS, P.reS2, i, j)) return;
            df dm2 = norm2(diff3(hj, lj, M.mh, M.ml));
            bool side = lessDF(q.d2, dm2, d.mgSide, [&] {
                dvec4 pj = d.pos[j];
                return pairOf(pj, pi).d2 < pairMirror(pj, mi).dm2;
            });
            if (side) { df pj = loadDF(d.pressDF, j); if (pmin > pj) pmin = pj; }
        });
    }
    df base = (gt == 0) ? -pmin : (gt == 1 ? Pi : Pi - pmin - pmin);
    df sx = dfF(0.f), sy = sx, sz = sx;
    forNbrs(d, i, [&](int j) {
        PairF m;
        if (!wallEntryDF(d, i, j, d.posf[j], hi, li, M, R2, d.mgS, P.reS2, d.bandHiS, m)) return;
        WeightDF w = weightDF(m.d2, RS, P.weightType);
        df f;
        if (gt <= 2) f = (loadDF(d.pressDF, j) + base) * w.wr2;
        else {
            double nj = d.pndi[j], Pj = d.press[j];
            f = (ni > P.epsilonZero && nj > P.epsilonZero) ? dfD(ni * Pj / nj + nj * Pid / ni) * w.wr2 : w.w;
        }
        sx += m.v.x * f; sy += m.v.y * f; sz += m.v.z * f;
    });
    double ax = dD(sx), ay = dD(sy), az = dD(sz);
    double pmind = dD(pmin);
    auto phi = [&](double Pj, double nj, double dm2, double wS) {
        if (gt == 0) return wS * ((Pj - pmind) / dm2);
        if (gt == 1) return wS * ((Pj + Pid) / dm2);
        if (gt == 2) return wS * ((Pj + Pid - 2.0 * pmind) / dm2);
        if (gt == 3 && ni > P.epsilonZero && nj > P.epsilonZero) return wS * ((ni * Pj / nj + nj * Pid / ni) / dm2);
        return wS;
    };
    PairM s = pairMirror(pi, mi);
    if (s.dm2 < P.reS2) {
        double wS = wfun(sqrt(s.dm2), P.reS, P.weightType);
        wS = phi(Pid, ni, s.dm2, wS);
        ax += s.m0 * wS; ay += s.m1 * wS; az += s.m2 * wS;
    }
    double f[3];
    wallRepulsion(P, r, vMax2, f);
    double g0 = P.relaxPress * (r.R[0] * ax + r.R[1] * ay + r.R[2] * az) * P.coeffPressGrad - f[0];
    double g1 = P.relaxPress * (r.R[3] * ax + r.R[4] * ay + r.R[5] * az) * P.coeffPressGrad - f[1];
    double g2 = P.relaxPress * (r.R[6] * ax + r.R[7] * ay + r.R[8] * az) * P.coeffPressGrad - f[2];
    dvec4 a = d.acc[i];
    a.x += g0 / P.DNS_FL1; a.y += g1 / P.DNS_FL1; a.z += g2 / P.DNS_FL1;
    d.acc[i] = a;
    double vf = (P.dim == 3) ? P.partDist * P.partDist * P.partDist : P.partDist * P.partDist;
    dvec4 fw = d.forceWall[i];
    fw.x += -g0 * vf; fw.y += -g1 * vf; fw.z += -g2 * vf;
    d.forceWall[i] = fw;
}
void launchWallPressGradientDF(const Dev& d, cudaStream_t s) {
    if (d.P.wallType != 1) return;
    launchPressDF(d, s);
    k_wall_press_grad_df<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
}

// ------------------------------------------------------------------ wall viscosity
// MpsViscosity::calcWallNoSlipViscosity / calcWallSlipViscosity, src/MpsViscosity.cpp:1527-1910
__global__ void __launch_bounds__(BLK) k_wall_visc_df(Dev d) {
    int i = nearIndexDF(d);
    if (i < 0) return;
    const MpsParams& P = d.P;
    bool noslip = P.slipCondition == 0;
    dvec4 pi = d.pos[i], vi = d.vel[i], mi = d.mirror[i];
    ReflG r = makeRefl(pi, mi, P.epsilonZero, false);
    double M[9];
    if (noslip) {
#pragma unroll
        for (int k = 0; k < 9; k++) M[k] = (k % 4 == 0) ? -1.0 : 0.0;
    } else {
#pragma unroll
        for (int k = 0; k < 9; k++) M[k] = r.R[k];
    }
    double vm0 = M[0] * vi.x + M[1] * vi.y + M[2] * vi.z;
    double vm1 = M[3] * vi.x + M[4] * vi.y + M[5] * vi.z;
    double vm2 = M[6] * vi.x + M[7] * vi.y + M[8] * vi.z;
    df vmx = dfD(vm0), vmy = dfD(vm1), vmz = dfD(vm2);
    double mu = P.KNM_VS1 * P.DNS_FL1;
    const df neuF = K(d.k.neuWall);
    float4 hi = d.posf[i], li = d.posLo[i];
    MirrorDF Mi = mirrorDF(d, mi);
    const df R2 = K(d.k.reL2);
    const RadiusDF RL = {K(d.k.reL), K(d.k.invReL)};
    df sx = dfF(0.f), sy = sx, sz = sx;
    forNbrsPosf(d, i, [&](int j, float4 hj) {
        PairF m;
        if (!wallEntryDF(d, i, j, hj, hi, li, Mi, R2, d.mgL, P.reL2, d.bandHiL, m)) return;
        df c = weightDF(m.d2, RL, P.weightType).w * neuF;
        float4 vhj = d.velHi[j], vlj = d.velLo[j];
        sx += (dfOf(vhj.x, vlj.x) - vmx) * c;
        sy += (dfOf(vhj.y, vlj.y) - vmy) * c;
        sz += (dfOf(vhj.z, vlj.z) - vmz) * c;
    });
    double ax = dD(sx), ay = dD(sy), az = dD(sz);
    PairM s = pairMirror(pi, mi);
    if (s.dm2 < P.reL2) {
        double wL = wfun(sqrt(s.dm2), P.reL, P.weightType);
        double neuS = (mu > P.epsilonZero ? 2.0 * mu * mu / (mu + mu) : 0.0) / P.DNS_FL1;
        ax += (vi.x - vm0) * wL * neuS;
        ay += (vi.y - vm1) * wL * neuS;
        az += (vi.z - vm2) * wL * neuS;
    }
    double f0 = (M[0] * ax + M[1] * ay + M[2] * az) * P.coeffViscMultiphase;
    double f1 = (M[3] * ax + M[4] * ay + M[5] * az) * P.coeffViscMultiphase;
    double f2 = (M[6] * ax + M[7] * ay + M[8] * az) * P.coeffViscMultiphase;
    dvec4 a = d.acc[i];
    a.x += f0; a.y += f1; a.z += f2;
    d.acc[i] = a;
    double vf = (P.dim == 3) ? P.partDist * P.partDist * P.partDist : P.partDist * P.partDist;
    dvec4 fw = d.forceWall[i];
    fw.x += -f0 * vf * P.DNS_FL1; fw.y += -f1 * vf * P.DNS_FL1; fw.z += -f2 * vf * P.DNS_FL1;
    d.forceWall[i] = fw;
}
void launchWallViscosityDF(const Dev& d, cudaStream_t s) {
    if (d.P.wallType != 1) return;
    launchVelDF(d, s);
    k_wall_visc_df<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
}

// ------------------------------------------------------------------ shifting
// MpsShifting (src/MpsShifting.cpp:23-101 type 1, :432-691 type 2) at the post-corrector
// positions through the 27 buckets.  Each sweep runs in bucket order over the listed
// particles and once more over the unlisted ones; entries are the reS ball minus the
// mirror side, decided exactly as in the FP64 tier.
template <class Op, bool STRAY>
__global__ void __launch_bounds__(BLK) k_shift_scan_df(Dev d, Op op) {
    const int i = scanParticle<STRAY>(d);
    if (i < 0) return;
    typename Op::State st;
    const bool on = op.begin(d, i, st);
    if (on) {
        const MpsParams& P = d.P;
        const dvec4 pi = d.pos[i];
        const float4 hi = d.posf[i], li = d.posLo[i];
        const SideDF sc = sideDF(d, i, pi);
        const df R2 = K(d.k.reS2);
        forCellsDF(d, pi, hi, d.bandHiS, [&](int j, int s, float4 hj) {
            if (j == i) return;
            const float4 lj = __ldg(&d.posLoCell[s]);
            PairF q = pairDF(hj, lj, hi, li);
            if (!inBallDF(d, q.d2, R2, d.mgS, P.reS2, i, j)) return;
            if (!sideOkDF(d, sc, hj, lj, q.d2, i, j)) return;
            op.visit(d, st, j, q);
        });
    }
    op.end(d, i, st, on);
}
template <class Op>
static void launchShiftScanDF(const Dev& d, const Op& op, cudaStream_t s) {
    k_shift_scan_df<Op, false><<<gridFor(d.N0, BLK), BLK, 0, s>>>(d, op);
    k_shift_scan_df<Op, true><<<gridFor(d.N0, BLK), BLK, 0, s>>>(d, op);
}

// dw/dr of MpsParticle::delWeight (src/MpsParticle.cpp) from r^2, float-float
__device__ __forceinline__ df dweightDF(df d2, const RadiusDF& R, int t) {
    df rinv = rsqrtDF(d2);
    switch (t) {
        case 1: return -(R.re * (rinv * rinv)) + R.invRe;
        case 2: return -(R.re * (rinv * rinv)) - R.invRe;
        case 3: { df a = -(d2 * rinv * R.invRe) + 1.0f; return (a * a) * (R.invRe * -3.0f); }
        case 4: { df a = -(d2 * rinv * R.invRe) + 1.0f; return a * (R.invRe * -2.0f); }
        default: return -(R.re * (rinv * rinv));
    }
}

// type 1: dv_i = sum dw(r_ij) (v_j - v_i) over fluid particles, applied to inner ones
struct ShiftVelDF {
    struct State { float4 vh, vl; df ux, uy, uz; };
    __device__ bool begin(const Dev& d, int i, State& st) const {
        st.vh = d.velHi[i]; st.vl = d.velLo[i];
        st.ux = st.uy = st.uz = dfF(0.f);
        return d.type[i] == d.P.fluid;
    }
    __device__ void visit(const Dev& d, State& st, int j, const PairF& q) const {
        const RadiusDF RS = {K(d.k.reS), K(d.k.invReS)};
        df dw = dweightDF(q.d2, RS, d.P.weightType);
        float4 vhj = d.velHi[j], vlj = d.velLo[j];
        st.ux += diffDF(vhj.x, vlj.x, st.vh.x, st.vl.x) * dw;
        st.uy += diffDF(vhj.y, vlj.y, st.vh.y, st.vl.y) * dw;
        st.uz += diffDF(vhj.z, vlj.z, st.vh.z, st.vl.z) * dw;
    }
    __device__ void end(const Dev& d, int i, State& st, bool on) const {
        bool apply = on && d.bc[i] == d.P.inner;
        d.shift[i] = apply ? make_dvec4(dD(st.ux), dD(st.uy), dD(st.uz), 0.0) : make_dvec4(0, 0, 0, 0);
    }
};
// type 2, concentration: C_i = (sum w(r_ij) + wall PND) / pndSmallZero, every particle
struct ConcDF {
    struct State { df sum; };
    __device__ bool begin(const Dev&, int, State& st) const { st.sum = dfF(0.f); return true; }
    __device__ void visit(const Dev& d, State& st, int, const PairF& q) const {
        const RadiusDF RS = {K(d.k.reS), K(d.k.invReS)};
        st.sum += weightDF(q.d2, RS, d.P.weightType).w;
    }
    __device__ void end(const Dev& d, int i, State& st, bool) const {
        d.conc[i] = (dD(st.sum) + d.pndWall[i]) / d.P.pndSmallZero;
    }
};
__global__ void k_df_conc(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N0) return;
    df c = dfD(d.conc[i]);
    d.concDF[i] = make_float2(c.h, c.l);
}
// type 2, gradient: grad C_i = -coeffPressGrad sum (C_i + C_j) w/r^2 r_ij over fluid
// particles; the shift of inner particles is -coeffShifting2 grad C_i
struct GradConcDF {
    struct State { df ci, gx, gy, gz; };
    __device__ bool begin(const Dev& d, int i, State& st) const {
        st.ci = loadDF(d.concDF, i);
        st.gx = st.gy = st.gz = dfF(0.f);
        return d.type[i] == d.P.fluid;
    }
    __device__ void visit(const Dev& d, State& st, int j, const PairF& q) const {
        const RadiusDF RS = {K(d.k.reS), K(d.k.invReS)};
        df cc = (st.ci + loadDF(d.concDF, j)) * weightDF(q.d2, RS, d.P.weightType).wr2;
        st.gx += q.v.x * cc; st.gy += q.v.y * cc; st.gz += q.v.z * cc;
    }
    __device__ void end(const Dev& d, int i, State& st, bool on) const {
        const MpsParams& P = d.P;
        dvec4 sh = make_dvec4(0, 0, 0, 0);
        if (on) {
            double gx = dD(st.gx) * -P.coeffPressGrad, gy = dD(st.gy) * -P.coeffPressGrad,
                   gz = dD(st.gz) * -P.coeffPressGrad;
            d.gradC[i] = make_dvec4(gx, gy, gz, 0.0);
            if (d.bc[i] == P.inner)
                sh = make_dvec4(-P.coeffShifting2 * gx, -P.coeffShifting2 * gy, -P.coeffShifting2 * gz, 0.0);
        }
        d.shift[i] = sh;
    }
};
// type 2, wall contribution (src/MpsShifting.cpp:578-691) at the shifted positions:
// mirror entries of near-wall fluid particles, reflected by the wall plane of i.
__global__ void __launch_bounds__(BLK) k_wall_grad_conc_df(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    dvec4 sh = make_dvec4(0, 0, 0, 0);
    if (d.type[i] == P.fluid && d.nearWall[i]) {
        dvec4 pi = d.pos[i], mi = d.mirror[i];
        ReflG r = makeRefl(pi, mi, P.epsilonZero, true);
        const float4 hi = d.posf[i], li = d.posLo[i];
        const MirrorDF M = mirrorDF(d, mi);
        const df R2 = K(d.k.reS2);
        const RadiusDF RS = {K(d.k.reS), K(d.k.invReS)};
        const df ci = loadDF(d.concDF, i);
        df sx = dfF(0.f), sy = dfF(0.f), sz = dfF(0.f);
        forCellsDF(d, pi, hi, d.bandHiS, [&](int j, int s, float4 hj) {
            if (j == i) return;
            const float4 lj = __ldg(&d.posLoCell[s]);
            PairF q = pairDF(hj, lj, hi, li);
            if (!inBallDF(d, q.d2, R2, d.mgS, P.reS2, i, j)) return;
            PairF m = pairDF(hj, lj, M.mh, M.ml);
            if (!lessDF(m.d2, R2, d.mgS, [&] { return pairMirror(d.pos[j], mi).dm2 < P.reS2; })) return;
            if (!lessDF(q.d2, m.d2, d.mgSide, [&] {
                    dvec4 pj = d.pos[j];
                    return pairOf(pj, pi).d2 < pairMirror(pj, mi).dm2;
                }))
                return;
            df cc = (ci + loadDF(d.concDF, j)) * weightDF(m.d2, RS, P.weightType).wr2;
            sx += m.v.x * cc; sy += m.v.y * cc; sz += m.v.z * cc;
        });
        double dx = dD(sx), dy = dD(sy), dz = dD(sz);
        double cI = d.conc[i];
        PairM s = pairMirror(pi, mi);
        if (s.dm2 < P.reS2) {
            double wS = wfun(sqrt(s.dm2), P.reS, P.weightType);
            dx += (cI + cI) * s.m0 * wS / s.dm2; dy += (cI + cI) * s.m1 * wS / s.dm2; dz += (cI + cI) * s.m2 * wS / s.dm2;
        }
        double g0 = -(r.R[0] * dx + r.R[1] * dy + r.R[2] * dz) * P.coeffPressGrad;
        double g1 = -(r.R[3] * dx + r.R[4] * dy + r.R[5] * dz) * P.coeffPressGrad;
        double g2 = -(r.R[6] * dx + r.R[7] * dy + r.R[8] * dz) * P.coeffPressGrad;
        dvec4 g = d.gradC[i];
        g.x += g0; g.y += g1; g.z += g2;
        d.gradC[i] = g;
        if (d.bc[i] == P.inner)
            sh = make_dvec4(-P.coeffShifting2 * g0, -P.coeffShifting2 * g1, -P.coeffShifting2 * g2, 0.0);
    }
    d.shift[i] = sh;
}
// The shifting sums over the list of the post-corrector positions (filtered from the skin
// list) instead of the 27-bucket scan: the reS-ball entries off the mirror side are the
// maskS entries of that list, in scan order, so the sums are those of k_shift_scan_df.
template <class Op>
__global__ void __launch_bounds__(BLK) k_shift_list_df(Dev d, Op op) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    typename Op::State st;
    const bool on = op.begin(d, i, st);
    if (on) {
        const float4 hi = d.posf[i], li = d.posLo[i];
        forMask(d, i, d.maskS[i], [&](int j, size_t) {
            const PairF q = pairDF(__ldg(d.posf + j), __ldg(d.posLo + j), hi, li);
            op.visit(d, st, j, q);
        });
    }
    op.end(d, i, st, on);
}
// Shifting from the list of the current positions (built by the caller: filter + masks).
void launchShiftingListDF(const Dev& d, cudaStream_t s) {
    const MpsParams& P = d.P;
    if (P.shiftingType == 1) {
        launchVelDF(d, s);
        k_shift_list_df<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d, ShiftVelDF());
        launchShiftVelApply(d, s);
        return;
    }
    k_shift_list_df<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d, ConcDF());
    k_df_conc<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
    k_shift_list_df<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d, GradConcDF());
    launchApplyShift(d, s);
    if (P.wallType == 1) {
        launchPosfCell(d, s);
        k_wall_grad_conc_df<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
        launchApplyShift(d, s);
    }
}
void launchShiftingDF(const Dev& d, cudaStream_t s) {
    const MpsParams& P = d.P;
    if (P.shiftingType != 1 && P.shiftingType != 2) return;
    launchPosf(d, s);   // post-corrector positions (hi/lo, particle and bucket order)
    if (P.shiftingType == 1) {
        launchVelDF(d, s);
        launchShiftScanDF(d, ShiftVelDF(), s);
        launchShiftVelApply(d, s);
        return;
    }
    launchShiftScanDF(d, ConcDF(), s);
    k_df_conc<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
    launchShiftScanDF(d, GradConcDF(), s);
    launchApplyShift(d, s);
    if (P.wallType == 1) {
        launchPosfCell(d, s);   // the wall sweep sees the shifted positions
        k_wall_grad_conc_df<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
        launchApplyShift(d, s);
    }
}

// ------------------------------------------------------------------ start-of-step list
// Candidates of the 27-bucket scan within reMax + skin of the start positions (FP32 test
// against a radius that includes the rounding band: a superset of every list the step's
// sweeps can need while the particles stay within half the skin), in scan order.
template <bool STRAY>
__global__ void __launch_bounds__(128) k_build_skin_df(Dev d) {
    const int i = scanParticle<STRAY>(d);
    if (i < 0) return;
    const dvec4 pi = d.pos[i];
    const float4 hi = d.posf[i];
    int cnt = 0;
    const size_t N0 = d.N0;
    forCellsDF(d, pi, hi, d.skinR2, [&](int j, int, float4) {
        if (j == i) return;
        if (cnt < d.K) d.nbr[(size_t)cnt * N0 + i] = j;
        cnt++;
    });
    d.nbrCount[i] = cnt > d.K ? d.K + 1 : cnt;   // K + 1: the row overflowed, rescanned where read
    d.posSkin[i] = hi;
    d.skinCell[i] = cellKeyOf(d, pi, hi);
}
void launchSkinListDF(const Dev& d, cudaStream_t s) {
    cudaMemsetAsync(d.skinFlag, 0, sizeof(int), s);
    k_build_skin_df<false><<<gridFor(d.N0, 128), 128, 0, s>>>(d);
    k_build_skin_df<true><<<gridFor(d.N0, 128), 128, 0, s>>>(d);
}

// Viscosity (the sweep of k_visc_df: same entries in the same scan order, same float-float
// arithmetic, so the same sums) over the start-of-step list instead of the 27 buckets.
__global__ void __launch_bounds__(128) k_visc_list_df(Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    const dvec4 pi = d.pos[i];
    const float4 hi = d.posf[i], li = d.posLo[i];
    const float4 vh = d.velHi[i], vl = d.velLo[i];
    const SideDF sc = sideDF(d, i, pi);
    const df R2 = K(d.k.reL2), neuW = K(d.k.neuW), neuF = K(d.k.neuF);
    const RadiusDF RL = {K(d.k.reL), K(d.k.invReL)};
    df ax = dfF(0.f), ay = dfF(0.f), az = dfF(0.f);
    auto pair = [&](int j, float4 hj, float4 lj) {
        PairF q = pairDF(hj, lj, hi, li);
        if (!inBallDF(d, q.d2, R2, d.mgL, P.reL2, i, j)) return;
        if (!sideOkDF(d, sc, hj, lj, q.d2, i, j)) return;
        WeightDF w = weightDF(q.d2, RL, P.weightType);
        df c = w.w * ((d.type[j] == P.wall) ? neuW : neuF);
        float4 vhj = d.velHi[j], vlj = d.velLo[j];
        ax += diffDF(vhj.x, vlj.x, vh.x, vl.x) * c;
        ay += diffDF(vhj.y, vlj.y, vh.y, vl.y) * c;
        az += diffDF(vhj.z, vlj.z, vh.z, vl.z) * c;
    };
    const int c = d.nbrCount[i];
    if (c <= d.K) {
        // four entries' indices and FP32 copies ahead of their tests (forNbrsPosf's order)
        auto entry = [&](int j, float4 hj) {
            float ex = hj.x - hi.x, ey = hj.y - hi.y, ez = hj.z - hi.z;
            if (ex * ex + ey * ey + ez * ez > d.bandHiL) return;   // outside the reL band
            pair(j, hj, __ldg(&d.posLo[j]));
        };
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
            for (int u = 0; u < 4; u++) entry(jj[u], hh[u]);
        }
        for (; k < c; k++) {
            const int j = ldStream(row + (size_t)k * d.N0);
            entry(j, __ldg(&d.posf[j]));
        }
    } else {
        forCellsDF(d, pi, hi, d.bandHiL, [&](int j, int s, float4 hj) {
            if (j != i) pair(j, hj, __ldg(&d.posLoCell[s]));
        });
    }
    double cv = P.coeffViscMultiphase;
    d.acc[i] = make_dvec4(cv * dD(ax), cv * dD(ay), cv * dD(az), 0.0);
}
void launchViscosityListDF(const Dev& d, cudaStream_t s) {
    launchVelDF(d, s);
    k_visc_list_df<<<gridFor(d.N0, 128), 128, 0, s>>>(d);
}

// The skin list covers the list of the current positions while every particle is within
// half the skin of its start position (FP32 test with margin).
__global__ void k_skin_check(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    float4 a = d.posf[i], b = d.posSkin[i];
    float ex = a.x - b.x, ey = a.y - b.y, ez = a.z - b.z;
    if (!(ex * ex + ey * ey + ez * ez <= d.skinMove2)) d.skinFlag[0] = 1;
}
// List of the current positions (the set and order of k_build_nbr_df) filtered from the
// skin list; a particle whose scan window changed, whose skin row overflowed, or any
// particle after the skin list went stale, scans the 27 buckets as k_build_nbr_df does.
template <bool STRAY>
__global__ void __launch_bounds__(128) k_filter_nbr_df(Dev d) {
    const int i = scanParticle<STRAY>(d);
    if (i < 0) return;
    const dvec4 pi = d.pos[i];
    const float4 hi = d.posf[i], li = d.posLo[i];
    const df R2 = K(d.k.reMax2);
    const size_t N0 = d.N0;
    int cnt = 0;
    // the lo part (lo: where it sits) is read only for pairs in the uncertain band
    auto keep = [&](int j, float4 hj, const float4* lo) {
        float ex = hj.x - hi.x, ey = hj.y - hi.y, ez = hj.z - hi.z;
        float d2f = ex * ex + ey * ey + ez * ez;
        if (d2f > d.bandHi) return;
        if (!(d2f < d.bandLo)) {
            PairF q = pairDF(hj, __ldg(lo), hi, li);
            if (!inBallDF(d, q.d2, R2, d.mgMax, d.reMax2, i, j)) return;
        }
        if (cnt < d.K) d.nbr[(size_t)cnt * N0 + i] = j;
        cnt++;
    };
    const int c = d.skinCnt[i];
    if (!*(volatile int*)d.skinFlag && c <= d.K && d.skinCell[i] == cellKeyOf(d, pi, hi)) {
        // the skin list stays intact (a later sweep filters it again); four entries' loads
        // are issued before their tests (the list stores would otherwise order each gather
        // after the previous entry's store)
        const int* row = d.skinNbr + i;
        int k = 0;
        for (; k + 4 <= c; k += 4) {
            int jj[4];
            float4 hh[4];
#pragma unroll
            for (int u = 0; u < 4; u++) jj[u] = ldStream(row + (size_t)(k + u) * N0);
#pragma unroll
            for (int u = 0; u < 4; u++) hh[u] = __ldg(&d.posf[jj[u]]);
#pragma unroll
            for (int u = 0; u < 4; u++) keep(jj[u], hh[u], d.posLo + jj[u]);
        }
        for (; k < c; k++) {
            const int j = ldStream(row + (size_t)k * N0);
            keep(j, __ldg(&d.posf[j]), d.posLo + j);
        }
    } else {
        forCellsDF(d, pi, hi, d.bandHi, [&](int j, int s, float4 hj) {
            if (j != i) keep(j, hj, d.posLoCell + s);
        });
    }
    if (cnt > d.K) { setErr(d, MPSE_CAPACITY); cnt = d.K; }
    d.nbrCount[i] = cnt;
    warpCount(d.counters, (unsigned)cnt);
}
void launchSkinCheck(const Dev& d, cudaStream_t s) {
    k_skin_check<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
}
void launchNeighborFilterDF(const Dev& d, cudaStream_t s) {
    cudaMemsetAsync(d.counters, 0, sizeof(unsigned long long), s);
    launchPosf(d, s);
    k_skin_check<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
    k_filter_nbr_df<false><<<gridFor(d.N0, 128), 128, 0, s>>>(d);
    k_filter_nbr_df<true><<<gridFor(d.N0, 128), 128, 0, s>>>(d);
}
