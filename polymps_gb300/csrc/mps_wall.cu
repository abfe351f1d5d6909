// mps_wall.cu — polygon wall distance and mirror particles on sm_103a.
//
// Replaces PolygonMesh::closestPointPNDBoundaryAABB (src/PolygonMesh.cpp:585-715), which
// queries libigl's AABB tree, and updateParticlesNearPolygonMesh (src/PolygonMesh.cpp:718-795).
// The meshes of this path are small (12-24 triangles for the tank and obstacle boxes),
// so each block stages the whole triangle soup in shared memory and every thread walks
// it: exact point-triangle closest point (Ericson, Real-Time Collision Detection, 5.1.5),
// evaluated with explicit round-to-nearest FP64 so the mirror positions, which decide
// neighbour membership in every later sweep, match the FP64 CPU restatement bit for bit.
// Ties between triangles go to the lowest index.  A mirror enters a decision only within
// 1.1 reL of the wall (the side test of the sweeps, the wall sweeps, the near-wall flag);
// a particle farther than 2 reL whose nearest triangle is the only one within the FP32
// band and whose projection lies inside it takes that projection in FP64 (the same point
// up to rounding, a quarter of the FP64 operations).
#include "mps_common.cuh"
#include "mps_internal.h"

__device__ void closestPtTriX(double px, double py, double pz, const double* t, double& qx, double& qy, double& qz) {
    double ax = t[0], ay = t[1], az = t[2], bx = t[3], by = t[4], bz = t[5], cx = t[6], cy = t[7], cz = t[8];
    double abx = xsub(bx, ax), aby = xsub(by, ay), abz = xsub(bz, az);
    double acx = xsub(cx, ax), acy = xsub(cy, ay), acz = xsub(cz, az);
    double apx = xsub(px, ax), apy = xsub(py, ay), apz = xsub(pz, az);
    double d1 = xdot3(abx, aby, abz, apx, apy, apz);
    double d2 = xdot3(acx, acy, acz, apx, apy, apz);
    if (d1 <= 0.0 && d2 <= 0.0) { qx = ax; qy = ay; qz = az; return; }
    double bpx = xsub(px, bx), bpy = xsub(py, by), bpz = xsub(pz, bz);
    double d3 = xdot3(abx, aby, abz, bpx, bpy, bpz);
    double d4 = xdot3(acx, acy, acz, bpx, bpy, bpz);
    if (d3 >= 0.0 && d4 <= d3) { qx = bx; qy = by; qz = bz; return; }
    double vc = xsub(xmul(d1, d4), xmul(d3, d2));
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        double v = d1 / xsub(d1, d3);
        qx = xadd(ax, xmul(v, abx)); qy = xadd(ay, xmul(v, aby)); qz = xadd(az, xmul(v, abz));
        return;
    }
    double cpx = xsub(px, cx), cpy = xsub(py, cy), cpz = xsub(pz, cz);
    double d5 = xdot3(abx, aby, abz, cpx, cpy, cpz);
    double d6 = xdot3(acx, acy, acz, cpx, cpy, cpz);
    if (d6 >= 0.0 && d5 <= d6) { qx = cx; qy = cy; qz = cz; return; }
    double vb = xsub(xmul(d5, d2), xmul(d1, d6));
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        double w = d2 / xsub(d2, d6);
        qx = xadd(ax, xmul(w, acx)); qy = xadd(ay, xmul(w, acy)); qz = xadd(az, xmul(w, acz));
        return;
    }
    double va = xsub(xmul(d3, d6), xmul(d5, d4));
    double e43 = xsub(d4, d3), e56 = xsub(d5, d6);
    if (va <= 0.0 && e43 >= 0.0 && e56 >= 0.0) {
        double w = e43 / xadd(e43, e56);
        qx = xadd(bx, xmul(w, xsub(cx, bx))); qy = xadd(by, xmul(w, xsub(cy, by))); qz = xadd(bz, xmul(w, xsub(cz, bz)));
        return;
    }
    double denom = 1.0 / xadd(xadd(va, vb), vc);
    double v = xmul(vb, denom), w = xmul(vc, denom);
    qx = xadd(xadd(ax, xmul(abx, v)), xmul(acx, w));
    qy = xadd(xadd(ay, xmul(aby, v)), xmul(acy, w));
    qz = xadd(xadd(az, xmul(abz, v)), xmul(acz, w));
}

// FP32 version of the same walk: only used to pick the triangles that need the exact one.
__device__ float sqDistTriF(float px, float py, float pz, const float* t) {
    float ax = t[0], ay = t[1], az = t[2], bx = t[3], by = t[4], bz = t[5], cx = t[6], cy = t[7], cz = t[8];
    float abx = bx - ax, aby = by - ay, abz = bz - az, acx = cx - ax, acy = cy - ay, acz = cz - az;
    float apx = px - ax, apy = py - ay, apz = pz - az;
    float d1 = abx * apx + aby * apy + abz * apz, d2 = acx * apx + acy * apy + acz * apz;
    float qx, qy, qz;
    float bpx = px - bx, bpy = py - by, bpz = pz - bz;
    float d3 = abx * bpx + aby * bpy + abz * bpz, d4 = acx * bpx + acy * bpy + acz * bpz;
    float cpx = px - cx, cpy = py - cy, cpz = pz - cz;
    float d5 = abx * cpx + aby * cpy + abz * cpz, d6 = acx * cpx + acy * cpy + acz * cpz;
    float vc = d1 * d4 - d3 * d2, vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
    if (d1 <= 0.f && d2 <= 0.f) { qx = ax; qy = ay; qz = az; }
    else if (d3 >= 0.f && d4 <= d3) { qx = bx; qy = by; qz = bz; }
    else if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
        float v = d1 / (d1 - d3); qx = ax + v * abx; qy = ay + v * aby; qz = az + v * abz;
    } else if (d6 >= 0.f && d5 <= d6) { qx = cx; qy = cy; qz = cz; }
    else if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
        float w = d2 / (d2 - d6); qx = ax + w * acx; qy = ay + w * acy; qz = az + w * acz;
    } else if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
        float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        qx = bx + w * (cx - bx); qy = by + w * (cy - by); qz = bz + w * (cz - bz);
    } else {
        float den = 1.f / (va + vb + vc), v = vb * den, w = vc * den;
        qx = ax + abx * v + acx * w; qy = ay + aby * v + acy * w; qz = az + abz * v + acz * w;
    }
    float dx = px - qx, dy = py - qy, dz = pz - qz;
    return dx * dx + dy * dy + dz * dz;
}

// The projection of p on the triangle's plane when it lies at least 1e-9 m inside every
// edge (then Ericson's walk ends in its interior case, whose point is this projection).
// pl: the triangle's plane data (unit normal n and n.a, then per edge (a,b), (b,c), (c,a)
// the unit in-plane normal pointing into the triangle and its offset; hostTrianglePlanes).
__device__ __forceinline__ bool projectInside(const double* pl, double px, double py, double pz, double& qx,
                                              double& qy, double& qz) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const double* e = pl + 4 + 4 * k;
        if (!(e[0] * px + e[1] * py + e[2] * pz - e[3] >= 1e-9)) return false;
    }
    const double sd = pl[0] * px + pl[1] * py + pl[2] * pz - pl[3];
    qx = px - sd * pl[0]; qy = py - sd * pl[1]; qz = pz - sd * pl[2];
    return true;
}

// PolygonMesh::interpolateWij / interpolateNumNeighWall (src/PolygonMesh.cpp:533-581),
// linear interpolation with extrapolation over the 50-sample tables
// (the reference's left-to-right search for the interval, as a binary search with the
// same comparisons: i = the number of k >= 1 with xs[k] < r)
__device__ double interpTab(const double* xs, const double* ys, double re, double x) {
    double r = x / re;
    int i;
    if (r >= xs[MPS_TAB - 2]) i = MPS_TAB - 2;
    else {
        int lo = 1, hi = MPS_TAB - 2;   // first k in [1, MPS_TAB - 2] with !(xs[k] < r): xs[MPS_TAB - 2] > r
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (xs[mid] < r) lo = mid + 1;
            else hi = mid;
        }
        i = lo - 1;
    }
    double xL = xs[i], yL = ys[i], xR = xs[i + 1], yR = ys[i + 1];
    double dydx = (yR - yL) / xsub(xR, xL);
    return xadd(yL, xmul(dydx, xsub(r, xL)));
}

__device__ __forceinline__ void wallDistanceAt(const Dev& d, int i, const double* sTri, const float* sTriF,
                                               const double* sTab, const double* sPl) {
    const MpsParams& P = d.P;
    dvec4 p = d.pos[i];
    // FP32 pass over all triangles (coordinates relative to the domain corner)
    float pxf = d2fRN(p.x - P.domainMin[0]), pyf = d2fRN(p.y - P.domainMin[1]), pzf = d2fRN(p.z - P.domainMin[2]);
    float df[MPS_MAX_TRI];
    float bestf = 3.0e38f;
    for (int t = 0; t < d.ntri; t++) {
        df[t] = sqDistTriF(pxf, pyf, pzf, sTriF + t * 9);
        bestf = fminf(bestf, df[t]);
    }
    // exact FP64 walk for every triangle that can hold (or tie) the minimum: the FP32
    // squared distances are within ~1e-5 m^2 of the exact ones for domains of a few metres
    float lim = bestf + 1e-4f + 1e-5f * bestf;
    double best = 1.0 / 0.0;
    int bt = -1;
    double bx = 0, by = 0, bz = 0;
    int inBand = 0, only = -1;
    for (int t = 0; t < d.ntri; t++)
        if (df[t] <= lim) { inBand++; only = t; }
    // far from the wall (beyond 2 reL with the FP32 band to spare), one candidate: the
    // FP64 projection when it lies inside the triangle
    double qx, qy, qz;
    if (inBand == 1 && bestf > (float)(4.0 * P.reL2) + 1e-4f && projectInside(sPl + only * 16, p.x, p.y, p.z, qx, qy, qz)) {
        double dx = xsub(p.x, qx), dy = xsub(p.y, qy), dz = xsub(p.z, qz);
        best = xnorm2(dx, dy, dz);
        bt = only; bx = qx; by = qy; bz = qz;
    } else {
        for (int t = 0; t < d.ntri; t++) {
            if (df[t] > lim) continue;
            closestPtTriX(p.x, p.y, p.z, sTri + t * 9, qx, qy, qz);
            double dx = xsub(p.x, qx), dy = xsub(p.y, qy), dz = xsub(p.z, qz);
            double d2 = xnorm2(dx, dy, dz);
            if (d2 < best) { best = d2; bt = t; bx = qx; by = qy; bz = qz; }
        }
    }
    double riw2 = d.riw2[i];
    if (bt >= 0 && best < riw2) {
        riw2 = best;
        d.riw2[i] = best;
        d.wallPos[i] = make_dvec4(bx, by, bz, 0.0);
        d.mirror[i] = make_dvec4(xadd(p.x, xmul(2.0, xsub(bx, p.x))), xadd(p.y, xmul(2.0, xsub(by, p.y))),
                                   xadd(p.z, xmul(2.0, xsub(bz, p.z))), 0.0);
        d.polyNormal[i] = make_dvec4(d.triNormal[bt * 3], d.triNormal[bt * 3 + 1], d.triNormal[bt * 3 + 2], 0.0);
    }
    // updateParticlesNearPolygonMesh
    double pw = 0.0;
    int nw = 0;
    if (riw2 < P.reL2) {
        d.nearWall[i] = 1;
        double x = sqrt(riw2);
        pw = interpTab(sTab, sTab + MPS_TAB, d.wallReS, x);
        nw = (int)interpTab(sTab + 2 * MPS_TAB, sTab + 3 * MPS_TAB, d.wallReL, x);
    }
    d.pndWall[i] = pw;
    d.nNeighWall[i] = nw;
}

// Each block stages the triangles, their FP32 copies, plane data and the wall tables in
// shared memory; one particle per thread (a grid-stride loop over fewer resident blocks
// measured slower: 0.263 vs 0.225 ms at 864k).
__global__ void __launch_bounds__(128) k_wall_distance(Dev d) {
    __shared__ double sTri[MPS_MAX_TRI * 9];
    __shared__ float sTriF[MPS_MAX_TRI * 9];
    __shared__ double sTab[4 * MPS_TAB];
    __shared__ double sPl[MPS_MAX_TRI * 16];
    for (int k = threadIdx.x; k < d.ntri * 9; k += blockDim.x) {
        sTri[k] = d.tri[k];
        sTriF[k] = d2fRN(d.tri[k] - d.P.domainMin[k % 3]);
    }
    for (int k = threadIdx.x; k < 4 * MPS_TAB; k += blockDim.x) sTab[k] = d.tab[k];
    for (int k = threadIdx.x; k < d.ntri * 16; k += blockDim.x) sPl[k] = d.triPlane[k];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < liveN(d)) wallDistanceAt(d, i, sTri, sTriF, sTab, sPl);
}

// Meshes above MPS_MAX_TRI triangles (libigl's AABB query for large meshes): depth-first
// walk of the triangle BVH in FP32, nearer child first, pruning boxes whose FP32 distance
// exceeds the band of the best FP32 triangle distance so far; the triangles inside the band
// of the final best are then decided exactly as by the brute-force kernel (FP64 Ericson,
// smallest squared distance, ties to the lowest triangle index).
#define BVH_STACK 64
#define BVH_CAND 32
__device__ __forceinline__ float boxDist2(float4 lo, float4 hi, float px, float py, float pz) {
    float dx = fmaxf(fmaxf(lo.x - px, px - hi.x), 0.f);
    float dy = fmaxf(fmaxf(lo.y - py, py - hi.y), 0.f);
    float dz = fmaxf(fmaxf(lo.z - pz, pz - hi.z), 0.f);
    return dx * dx + dy * dy + dz * dz;
}
__device__ __forceinline__ float bandOf(float bestf) { return bestf + 1e-4f + 1e-5f * bestf; }
__global__ void __launch_bounds__(128) k_wall_distance_bvh(Dev d) {
    __shared__ double sTab[4 * MPS_TAB];
    for (int k = threadIdx.x; k < 4 * MPS_TAB; k += blockDim.x) sTab[k] = d.tab[k];
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    dvec4 p = d.pos[i];
    const float px = d2fRN(p.x - P.domainMin[0]), py = d2fRN(p.y - P.domainMin[1]), pz = d2fRN(p.z - P.domainMin[2]);
    int stack[BVH_STACK];
    int cand[BVH_CAND];
    float candD[BVH_CAND];
    int nc = 0;
    bool overflow = false;
    float bestf = 3.0e38f;
    // pass 1: best FP32 distance, keeping the triangles within the band of the best so far
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int nd = stack[--sp];
        const float4 lo = __ldg(d.bvhLo + nd), hi = __ldg(d.bvhHi + nd);
        if (boxDist2(lo, hi, px, py, pz) > bandOf(bestf)) continue;
        const int a = __float_as_int(lo.w), b = __float_as_int(hi.w);
        if (a < 0) {
            for (int q = -a - 1; q < -a - 1 + b; q++) {
                const int t = __ldg(d.bvhOrder + q);
                const float df = sqDistTriF(px, py, pz, d.triF + 9 * t);
                bestf = fminf(bestf, df);
                if (df <= bandOf(bestf)) {
                    if (nc < BVH_CAND) { cand[nc] = t; candD[nc] = df; nc++; }
                    else overflow = true;
                }
            }
        } else if (sp + 2 <= BVH_STACK) {
            const float da = boxDist2(__ldg(d.bvhLo + a), __ldg(d.bvhHi + a), px, py, pz);
            const float db = boxDist2(__ldg(d.bvhLo + b), __ldg(d.bvhHi + b), px, py, pz);
            if (da <= db) { stack[sp++] = b; stack[sp++] = a; }
            else { stack[sp++] = a; stack[sp++] = b; }
        } else {
            overflow = true;   // deeper than the stack: never for a median-split tree of < 2^60 leaves
        }
    }
    const float lim = bandOf(bestf);
    double best = 1.0 / 0.0;
    int bt = -1;
    double bx = 0, by = 0, bz = 0;
    auto exact = [&](int t) {
        double qx, qy, qz;
        closestPtTriX(p.x, p.y, p.z, d.tri + 9 * t, qx, qy, qz);
        double dx = xsub(p.x, qx), dy = xsub(p.y, qy), dz = xsub(p.z, qz);
        double d2 = xnorm2(dx, dy, dz);
        if (d2 < best || (d2 == best && t < bt)) { best = d2; bt = t; bx = qx; by = qy; bz = qz; }
    };
    if (!overflow) {
        for (int c = 0; c < nc; c++)
            if (candD[c] <= lim) exact(cand[c]);
    } else {
        // pass 2 (many near-ties): every triangle within the final band, by a second walk
        sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const int nd = stack[--sp];
            const float4 lo = __ldg(d.bvhLo + nd), hi = __ldg(d.bvhHi + nd);
            if (boxDist2(lo, hi, px, py, pz) > lim) continue;
            const int a = __float_as_int(lo.w), b = __float_as_int(hi.w);
            if (a < 0) {
                for (int q = -a - 1; q < -a - 1 + b; q++) {
                    const int t = __ldg(d.bvhOrder + q);
                    if (sqDistTriF(px, py, pz, d.triF + 9 * t) <= lim) exact(t);
                }
            } else if (sp + 2 <= BVH_STACK) {
                stack[sp++] = a;
                stack[sp++] = b;
            }
        }
    }
    double riw2 = d.riw2[i];
    if (bt >= 0 && best < riw2) {
        riw2 = best;
        d.riw2[i] = best;
        d.wallPos[i] = make_dvec4(bx, by, bz, 0.0);
        d.mirror[i] = make_dvec4(xadd(p.x, xmul(2.0, xsub(bx, p.x))), xadd(p.y, xmul(2.0, xsub(by, p.y))),
                                   xadd(p.z, xmul(2.0, xsub(bz, p.z))), 0.0);
        d.polyNormal[i] = make_dvec4(d.triNormal[bt * 3], d.triNormal[bt * 3 + 1], d.triNormal[bt * 3 + 2], 0.0);
    }
    double pw = 0.0;
    int nw = 0;
    if (riw2 < P.reL2) {
        d.nearWall[i] = 1;
        double x = sqrt(riw2);
        pw = interpTab(sTab, sTab + MPS_TAB, d.wallReS, x);
        nw = (int)interpTab(sTab + 2 * MPS_TAB, sTab + 3 * MPS_TAB, d.wallReL, x);
    }
    d.pndWall[i] = pw;
    d.nNeighWall[i] = nw;
}

void launchWallDistance(const Dev& d, cudaStream_t s) {
    if (d.P.wallType != 1 || d.ntri <= 0) return;
    if (d.ntri > MPS_MAX_TRI) k_wall_distance_bvh<<<gridFor(d.N0, 128), 128, 0, s>>>(d);
    else k_wall_distance<<<gridFor(d.N0, 128), 128, 0, s>>>(d);
}
