// mps_oracle.cpp — TEST INFRASTRUCTURE ONLY: the CPU oracle for the PolyMPS per-step
// particle path.  It restates, in FP64 C++ with OpenMP and no FMA contraction
// (-ffp-contract=off), the reference functions named in each comment (paths relative to
// the rubensamarojr/polymps source tree).  The reference cannot be compiled here (its
// Eigen/libigl/json submodules are empty), so this is a restatement, not a build:
//   * Eigen's ConjugateGradient is restated from its documented behaviour
//     (Jacobi preconditioner, stop when ||b-Ax||^2 < tol^2 ||b||^2, warm start).
//   * libigl's AABB point-mesh squared distance is restated as a brute-force exact
//     point-triangle closest point (Ericson, Real-Time Collision Detection, 5.1.5),
//     ties broken by the lowest triangle index.
// Parity of those two third-party pieces against the reference's own builds is
// UNPINNED (no reference test or golden vector covers them).
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this
// library; the product path (libmpsgpu.so) never does.

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cfloat>
#include <vector>
#include <algorithm>
#include <limits>
#include <chrono>
#include <omp.h>
#include "../include/mpsgpu.h"

namespace {

struct Orc {
    MpsParams P;
    int N = 0, N0 = 0;
    // scalars (include/MpsParticle.h:150-241)
    std::vector<int> type, bc, numNeigh, nNeighWall, nearMeshType, PTYPE;
    std::vector<char> nearWall;
    std::vector<double> press, pndi, pndki, pndski, pndSmall, npcd2, conc, velDiv, diffTerm,
        aux1, aux2, pndWall, devDot, riw2, RHO, MEU;
    // vectors, interleaved xyz
    std::vector<double> pos, vel, acc, accStar, npcd, gradC, c1, c2, c3, dvel, wallPos, mirror,
        polyNormal, forceWall, normal;
    std::vector<double> pressurePPE, sourceTerm;
    // buckets (include/MpsParticle.h:138-141)
    std::vector<int> first, last, next;
    // mesh
    int ntri = 0;
    std::vector<double> tri, triNormal;
    std::vector<double> xDataPND, Zij, xDataNeigh;
    std::vector<int> nNeighTab;
    // solver
    double tol = 1e-8;
    int maxIter = -1;
    int solverIter = 0;
    double solverError = 0.0, initialError = 0.0;
    double Dns[3] = {0, 0, 0};
    double velMax = 0.0, CFLcurrent = 0.0, timeCurrent = 0.0;
    int numOfIterations = 0;
    int outRemoved = 0;
    int sizeMismatch = 0;
    // PPE (CSR of the last assembly)
    std::vector<long long> Arow;
    std::vector<int> Acol;
    std::vector<double> Aval;
};

inline double sq(double a) { return a * a; }

// ------------------------------------------------------------------ weights
// MpsParticle::weight / weightGradient / delWeight, src/MpsParticle.cpp:57-108
double weight(double dst, double re, int t) {
    switch (t) {
        case 0: return re / dst - 1.0;
        case 1: return re / dst + dst / re - 2.0;
        case 2: return re / dst - dst / re;
        case 3: return (1.0 - dst / re) * (1.0 - dst / re) * (1.0 - dst / re);
        case 4: return (1.0 - dst / re) * (1.0 - dst / re);
        default: return re / dst - 1.0;
    }
}
double delWeight(double dst, double re, int t) {
    switch (t) {
        case 0: return -re / (dst * dst);
        case 1: return -re / (dst * dst) + 1.0 / re;
        case 2: return -re / (dst * dst) - 1.0 / re;
        case 3: return -3.0 / re * (1.0 - dst / re) * (1.0 - dst / re);
        case 4: return -2.0 / re * (1.0 - dst / re);
        default: return -re / (dst * dst);
    }
}

// ------------------------------------------------------------------ parameters
// MpsBucket::calcDomainLimits, non-periodic branch (src/MpsBucket.cpp:71-143, 289-294)
int domainLimits(MpsParams* P, int n, const double* pos) {
    double lim[3][2];
    if (P->limitTypeBC == 0) {
        for (int k = 0; k < 3; k++) lim[k][0] = lim[k][1] = pos[k];
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) {
                lim[k][0] = std::min(lim[k][0], pos[i * 3 + k]);
                lim[k][1] = std::max(lim[k][1], pos[i * 3 + k]);
            }
        int testdim = 0;
        for (int k = 0; k < 3; k++) if (lim[k][0] != lim[k][1]) testdim++;
        if (testdim != (int)P->dim) return MPSGPU_ERR_ARG;  // reference exits with code 10
    } else {
        for (int k = 0; k < 3; k++) { lim[k][0] = P->domainMin[k]; lim[k][1] = P->domainMax[k]; }
    }
    if (P->domainTypeBC == 0 && P->wallType == 0) {
        lim[0][0] -= 0.5 * P->partDist; lim[0][1] += 0.5 * P->partDist;
        lim[1][0] -= 0.5 * P->partDist; lim[1][1] += 0.5 * P->partDist;
        if (P->dim == 3) { lim[2][0] -= 0.5 * P->partDist; lim[2][1] += 0.5 * P->partDist; }
        int* nb[3] = {&P->numBucketsX, &P->numBucketsY, &P->numBucketsZ};
        for (int k = 0; k < (int)P->dim; k++) {
            lim[k][0] -= P->bucketSide;
            lim[k][1] += P->bucketSide;
            *nb[k] = (int)(long)((lim[k][1] - lim[k][0]) / P->bucketSide + 1);
            lim[k][1] = lim[k][0] + (*nb[k]) * P->bucketSide;
        }
    }
    for (int k = 0; k < 3; k++) { P->domainMin[k] = lim[k][0]; P->domainMax[k] = lim[k][1]; }
    return 0;
}

// MpsParticle::setParameters (src/MpsParticle.cpp:136-227) + MpsBucket::allocateMemory
// (src/MpsBucket.cpp:20-67)
int deriveParams(MpsParams* P, int n, const double* pos) {
    if (P->derived) return 0;
    P->epsilonZero = 10.0 * std::numeric_limits<double>::epsilon();
    for (int k = 0; k < 3; k++) { P->domainMin[k] -= P->partDist * 3.0; P->domainMax[k] += P->partDist * 3.0; }
    if ((int)P->dim == 2) { P->domainMin[2] = 0.0; P->domainMax[2] = 0.0; }
    P->reS = P->partDist * P->reS;
    P->reL = P->partDist * P->reL;
    P->reRepulsiveForce = P->partDist * P->reRepulsiveForce;
    P->reS2 = P->reS * P->reS;
    P->reL2 = P->reL * P->reL;
    P->EPS_RE = P->EPS_RE * P->reS2 / 4.0;
    P->pndSmallZero = P->pndLargeZero = P->pndGradientZero = P->lambdaZero = P->numNeighZero = 0.0;
    int lmin = (int)std::ceil(P->reL / P->partDist) + 1;
    int lmax = (int)std::ceil(P->reL / P->partDist) + 2;
    int f2 = 0, f3 = 1;
    if ((int)P->dim == 2) { f2 = 1; f3 = 0; }
    for (int ix = -lmin; ix < lmax; ix++)
        for (int iy = -lmin; iy < lmax; iy++)
            for (int iz = -lmin * f3; iz < lmax * f3 + f2; iz++) {
                double x = P->partDist * (double)ix, y = P->partDist * (double)iy, z = P->partDist * (double)iz;
                double d2 = x * x + y * y + z * z;
                if (d2 <= P->reL2) {
                    if (d2 <= P->epsilonZero) continue;
                    double d = std::sqrt(d2);
                    P->pndLargeZero += weight(d, P->reL, P->weightType);
                    P->lambdaZero += d2 * weight(d, P->reL, P->weightType);
                    P->numNeighZero += 1;
                    if (d2 <= P->reS2) {
                        P->pndSmallZero += weight(d, P->reS, P->weightType);
                        P->pndGradientZero += weight(d, P->reS, P->weightType);
                    }
                }
            }
    P->lambdaZero = P->lambdaZero / P->pndLargeZero;
    P->coeffViscosity = 2.0 * P->KNM_VS1 * P->dim / (P->pndLargeZero * P->lambdaZero);
    P->coeffViscMultiphase = 2.0 * P->dim / (P->pndLargeZero * P->lambdaZero);
    P->coeffPressEMPS = P->soundSpeed * P->soundSpeed / P->pndSmallZero;
    P->coeffPressGrad = -P->dim / P->pndGradientZero;
    P->coeffPressWCMPS = P->soundSpeed * P->soundSpeed;
    P->coeffShifting1 = P->dri * P->partDist / P->pndSmallZero;
    P->coeffShifting2 = P->coefA * P->partDist * P->partDist * P->cflNumber * P->machNumber;
    P->coeffPPE = 2.0 * P->dim / (P->pndLargeZero * P->lambdaZero);
    P->coeffPPESource = P->relaxPND / (P->timeStep * P->timeStep * P->pndSmallZero);
    P->invPartDist = 1.0 / P->partDist;
    P->distCollisionLimit = P->partDist * P->distLimitRatio;
    P->distCollisionLimit2 = P->distCollisionLimit * P->distCollisionLimit;
    P->restitutionCollision = 1.0 + P->collisionRatio;
    P->betaPnd = P->pndThreshold * P->pndSmallZero;
    P->betaNeigh = P->neighThreshold * P->numNeighZero;
    P->delta2 = P->npcdThreshold * P->npcdThreshold * P->partDist * P->partDist;
    P->thetaArc = P->thetaThreshold / 180.0 * 3.14159265;
    P->hThreshold2 = 1.33 * 1.33 * P->partDist * P->partDist;
    P->dstThreshold2 = 2.0 * P->hThreshold2;
    P->normThreshold2 = P->normThreshold * P->normThreshold;
    // MpsBucket::allocateMemory
    P->bucketSide = P->reL * (1.0 + P->cflNumber);
    P->invBucketSide = 1.0 / P->bucketSide;
    P->numBucketsX = (int)((P->domainMax[0] - P->domainMin[0]) * P->invBucketSide) + 3;
    P->numBucketsY = (int)((P->domainMax[1] - P->domainMin[1]) * P->invBucketSide) + 3;
    P->numBucketsZ = (int)((P->domainMax[2] - P->domainMin[2]) * P->invBucketSide) + 3;
    if ((int)P->dim == 2) P->numBucketsZ = 1;
    if (P->wallType == 0 || P->domainTypeBC == 1) {
        int e = domainLimits(P, n, pos);
        if (e) return e;
        P->invBucketSide = 1.0 / P->bucketSide;
    }
    P->numBucketsXY = P->numBucketsX * P->numBucketsY;
    P->numBucketsXYZ = P->numBucketsX * P->numBucketsY * P->numBucketsZ;
    P->derived = 1;
    return 0;
}

// ------------------------------------------------------------------ buckets
// MpsBucket::bucketCoordinates, src/MpsBucket.cpp:420-425 (always adds epsilonZero)
inline void bucketCoordinates(const MpsParams& P, double x, double y, double z, int& bx, int& by, int& bz) {
    bx = (int)((x - P.domainMin[0]) * P.invBucketSide + P.epsilonZero);
    by = (int)((y - P.domainMin[1]) * P.invBucketSide + P.epsilonZero);
    bz = (int)((z - P.domainMin[2]) * P.invBucketSide + P.epsilonZero);
}

// The 27-bucket (9 in 2D) linked-list scan used by every operator, in the reference's
// order (z, y, x, then insertion order), e.g. src/MpsPndNeigh.cpp:209-258.  Bucket
// indices outside the grid are skipped (the reference reads out of bounds there).
template <class F>
inline void forCandidates(const Orc& o, double xi, double yi, double zi, F&& f) {
    const MpsParams& P = o.P;
    int ix, iy, iz;
    bucketCoordinates(P, xi, yi, zi, ix, iy, iz);
    int minZ = (iz - 1) * ((int)(P.dim - 2.0));
    int maxZ = (iz + 1) * ((int)(P.dim - 2.0));
    for (int jz = minZ; jz <= maxZ; jz++)
        for (int jy = iy - 1; jy <= iy + 1; jy++)
            for (int jx = ix - 1; jx <= ix + 1; jx++) {
                long long jb = (long long)jz * P.numBucketsXY + (long long)jy * P.numBucketsX + jx;
                if (jb < 0 || jb >= P.numBucketsXYZ) continue;
                int j = o.first[jb];
                if (j == -1) continue;
                while (true) {
                    f(j);
                    j = o.next[j];
                    if (j == -1) break;
                }
            }
}

// MpsBucket::updateParticlesID, src/MpsBucket.cpp:299-353 (2D adds epsilonZero, 3D not)
int updateParticlesID(Orc& o) {
    const MpsParams& P = o.P;
    std::fill(o.first.begin(), o.first.end(), -1);
    std::fill(o.last.begin(), o.last.end(), -1);
    std::fill(o.next.begin(), o.next.end(), -1);
    int err = 0;
    for (int i = 0; i < o.N; i++) {
        if (o.type[i] == P.ghost) continue;
        int ix, iy, iz = 0;
        if ((int)P.dim == 2) {
            ix = (int)((o.pos[i * 3] - P.domainMin[0]) * P.invBucketSide + P.epsilonZero);
            iy = (int)((o.pos[i * 3 + 1] - P.domainMin[1]) * P.invBucketSide + P.epsilonZero);
        } else {
            ix = (int)((o.pos[i * 3] - P.domainMin[0]) * P.invBucketSide);
            iy = (int)((o.pos[i * 3 + 1] - P.domainMin[1]) * P.invBucketSide);
            iz = (int)((o.pos[i * 3 + 2] - P.domainMin[2]) * P.invBucketSide);
        }
        long long ib = (long long)iz * P.numBucketsXY + (long long)iy * P.numBucketsX + ix;
        if (ib < 0 || ib >= P.numBucketsXYZ) { err = MPSGPU_ERR_DOMAIN; continue; }
        int j = o.last[ib];
        o.last[ib] = i;
        if (j == -1) o.first[ib] = i;
        else o.next[j] = i;
    }
    return err;
}

// MpsParticle::checkParticleOutDomain, non-periodic part, src/MpsParticle.cpp:270-396
void checkParticleOutDomain(Orc& o) {
    const MpsParams& P = o.P;
    int newN = o.N;
    double mnx = P.domainMin[0] + P.bucketSide, mxx = P.domainMax[0] - P.bucketSide;
    double mny = P.domainMin[1] + P.bucketSide, mxy = P.domainMax[1] - P.bucketSide;
    double mnz = P.domainMin[2] + P.bucketSide, mxz = P.domainMax[2] - P.bucketSide;
    for (int i = 0; i < o.N; i++) {
        const double* p = &o.pos[i * 3];
        if (o.type[i] == P.fluid && i < newN &&
            (p[0] > mxx || p[0] < mnx || p[1] > mxy || p[1] < mny ||
             (P.dim == 3 && (p[2] > mxz || p[2] < mnz)))) {
            int L = newN - 1;
            o.type[i] = o.type[L]; o.bc[i] = o.bc[L]; o.numNeigh[i] = o.numNeigh[L];
            o.press[i] = o.press[L]; o.pndi[i] = o.pndi[L]; o.pndki[i] = o.pndki[L];
            o.pndski[i] = o.pndski[L]; o.pndSmall[i] = o.pndSmall[L]; o.npcd2[i] = o.npcd2[L];
            o.conc[i] = o.conc[L]; o.velDiv[i] = o.velDiv[L]; o.diffTerm[i] = o.diffTerm[L];
            o.nearMeshType[i] = o.nearMeshType[L]; o.nearWall[i] = o.nearWall[L];
            o.nNeighWall[i] = o.nNeighWall[L]; o.pndWall[i] = o.pndWall[L]; o.devDot[i] = o.devDot[L];
            o.riw2[i] = o.riw2[L]; o.PTYPE[i] = o.PTYPE[L]; o.RHO[i] = o.RHO[L]; o.MEU[i] = o.MEU[L];
            if (P.mpsType == 2 || P.mpsType == 3) {
                o.pressurePPE[i] = o.pressurePPE[L];
                o.sourceTerm[i] = o.sourceTerm[L];
            }
            for (int k = 0; k < 3; k++) {
                o.acc[i * 3 + k] = o.acc[L * 3 + k]; o.accStar[i * 3 + k] = o.accStar[L * 3 + k];
                o.pos[i * 3 + k] = o.pos[L * 3 + k]; o.vel[i * 3 + k] = o.vel[L * 3 + k];
                o.npcd[i * 3 + k] = o.npcd[L * 3 + k]; o.gradC[i * 3 + k] = o.gradC[L * 3 + k];
                o.c1[i * 3 + k] = o.c1[L * 3 + k]; o.c2[i * 3 + k] = o.c2[L * 3 + k];
                o.c3[i * 3 + k] = o.c3[L * 3 + k]; o.dvel[i * 3 + k] = o.dvel[L * 3 + k];
                o.wallPos[i * 3 + k] = o.wallPos[L * 3 + k]; o.mirror[i * 3 + k] = o.mirror[L * 3 + k];
                o.polyNormal[i * 3 + k] = o.polyNormal[L * 3 + k];
                o.forceWall[i * 3 + k] = o.forceWall[L * 3 + k];
            }
            o.type[L] = P.ghost; o.bc[L] = P.other; o.nearWall[L] = 0; o.nearMeshType[L] = 0;
            o.riw2[L] = 10e8 * P.partDist;
            for (int k = 0; k < 3; k++) o.vel[L * 3 + k] = 0.0;
            o.press[L] = 0.0;
            o.pos[L * 3] = P.domainMax[0] - P.partDist;
            o.pos[L * 3 + 1] = P.domainMax[1] - P.partDist;
            o.pos[L * 3 + 2] = (P.dim == 2) ? 0.0 : P.domainMax[2] - P.partDist;
            newN--;
            o.outRemoved++;
        }
        o.N = newN;  // the loop bound shrinks as particles are removed (as in the reference)
    }
}

// ------------------------------------------------------------------ polygon wall
// Exact closest point of p on triangle (a,b,c): Ericson, Real-Time Collision Detection
// (2005) 5.1.5, Voronoi-region walk.  Stands in for libigl AABB::squared_distance
// (src/PolygonMesh.cpp:611).  All products/sums are evaluated left to right without FMA;
// the CUDA kernel evaluates the same sequence so the two agree bit for bit.
inline double dot3(double ax, double ay, double az, double bx, double by, double bz) {
    return ax * bx + ay * by + az * bz;
}
void closestPtTri(const double* p, const double* t, double* q) {
    const double *a = t, *b = t + 3, *c = t + 6;
    double abx = b[0] - a[0], aby = b[1] - a[1], abz = b[2] - a[2];
    double acx = c[0] - a[0], acy = c[1] - a[1], acz = c[2] - a[2];
    double apx = p[0] - a[0], apy = p[1] - a[1], apz = p[2] - a[2];
    double d1 = dot3(abx, aby, abz, apx, apy, apz);
    double d2 = dot3(acx, acy, acz, apx, apy, apz);
    if (d1 <= 0.0 && d2 <= 0.0) { q[0] = a[0]; q[1] = a[1]; q[2] = a[2]; return; }
    double bpx = p[0] - b[0], bpy = p[1] - b[1], bpz = p[2] - b[2];
    double d3 = dot3(abx, aby, abz, bpx, bpy, bpz);
    double d4 = dot3(acx, acy, acz, bpx, bpy, bpz);
    if (d3 >= 0.0 && d4 <= d3) { q[0] = b[0]; q[1] = b[1]; q[2] = b[2]; return; }
    double vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        double v = d1 / (d1 - d3);
        q[0] = a[0] + v * abx; q[1] = a[1] + v * aby; q[2] = a[2] + v * abz; return;
    }
    double cpx = p[0] - c[0], cpy = p[1] - c[1], cpz = p[2] - c[2];
    double d5 = dot3(abx, aby, abz, cpx, cpy, cpz);
    double d6 = dot3(acx, acy, acz, cpx, cpy, cpz);
    if (d6 >= 0.0 && d5 <= d6) { q[0] = c[0]; q[1] = c[1]; q[2] = c[2]; return; }
    double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        double w = d2 / (d2 - d6);
        q[0] = a[0] + w * acx; q[1] = a[1] + w * acy; q[2] = a[2] + w * acz; return;
    }
    double va = d3 * d6 - d5 * d4;
    double e43 = d4 - d3, e56 = d5 - d6;
    if (va <= 0.0 && e43 >= 0.0 && e56 >= 0.0) {
        double w = e43 / (e43 + e56);
        q[0] = b[0] + w * (c[0] - b[0]); q[1] = b[1] + w * (c[1] - b[1]); q[2] = b[2] + w * (c[2] - b[2]);
        return;
    }
    double denom = 1.0 / (va + vb + vc);
    double v = vb * denom, w = vc * denom;
    q[0] = a[0] + abx * v + acx * w;
    q[1] = a[1] + aby * v + acy * w;
    q[2] = a[2] + abz * v + acz * w;
}

// PolygonMesh::initWijnNeigh, src/PolygonMesh.cpp:377-527 (wall PND Z(r) and wall
// neighbour-count tables, 50 samples over a half-space lattice offset by l0/2)
void initWijnNeigh(Orc& o) {
    const MpsParams& P = o.P;
    int dim = (int)P.dim, wt = P.weightType;
    double lo = P.partDist, reS = P.reS, reL = P.reL, reS2 = reS * reS, reL2 = reL * reL;
    int n = 50;
    int limS = (int)std::ceil(reS / lo), limL = (int)std::ceil(reL / lo);
    o.xDataPND.clear(); o.Zij.clear(); o.xDataNeigh.clear(); o.nNeighTab.clear();
    for (int i = 1; i <= n; i++) {
        double xi = 0.0, yi = i * reS / n, zi = 0.0;
        double riw = std::sqrt((0.0 - xi) * (0.0 - xi) + (0.0 - yi) * (0.0 - yi) + (0.0 - zi) * (0.0 - zi));
        if (dim == 2) riw = std::sqrt((0.0 - xi) * (0.0 - xi) + (0.0 - yi) * (0.0 - yi));
        o.xDataPND.push_back(riw / reS);
        o.xDataNeigh.push_back(riw / reL);
        double n0 = 0.0;
        int zlo = (dim == 3) ? -limS : 0, zhi = (dim == 3) ? limS : 0;
        for (int ix = -limS; ix <= limS; ix++)
            for (int iy = -limS; iy <= 0; iy++)
                for (int iz = zlo; iz <= zhi; iz++) {
                    double xj = lo * (double)ix, yj = lo * (double)(iy - 0.5), zj = lo * (double)iz;
                    double r2 = (dim == 3) ? (xj - xi) * (xj - xi) + (yj - yi) * (yj - yi) + (zj - zi) * (zj - zi)
                                           : (xj - xi) * (xj - xi) + (yj - yi) * (yj - yi);
                    if (r2 < reS2) {
                        if (r2 == 0.0) continue;
                        double r = std::sqrt(r2);
                        if (wt == 0) n0 += reS / r - 1.0;
                        else if (wt == 1) n0 += reS / r + r / reS - 2.0;
                        else if (wt == 2) n0 += reS / r - r / reS;
                        else if (wt == 3) n0 += std::pow(1.0 - r / reS, 3.0);
                        else if (wt == 4) n0 += std::pow(1.0 - r / reS, 2.0);
                        else n0 += reS / r - 1.0;
                    }
                }
        o.Zij.push_back(n0);
        int nn = 0;
        zlo = (dim == 3) ? -limL : 0; zhi = (dim == 3) ? limL : 0;
        for (int ix = -limL; ix <= limL; ix++)
            for (int iy = -limL; iy <= 0; iy++)
                for (int iz = zlo; iz <= zhi; iz++) {
                    double xj = lo * (double)ix, yj = lo * (double)(iy - 0.5), zj = lo * (double)iz;
                    double r2 = (dim == 3) ? (xj - xi) * (xj - xi) + (yj - yi) * (yj - yi) + (zj - zi) * (zj - zi)
                                           : (xj - xi) * (xj - xi) + (yj - yi) * (yj - yi);
                    if (r2 < reL2) {
                        if (r2 == 0.0) continue;
                        nn += 1;
                    }
                }
        o.nNeighTab.push_back(nn);
    }
}

// PolygonMesh::interpolateWij / interpolateNumNeighWall, src/PolygonMesh.cpp:533-581
double interpolateWij(const Orc& o, double re, double x) {
    int sz = (int)o.xDataPND.size();
    double r = x / re;
    int i = 0;
    if (r >= o.xDataPND[sz - 2]) i = sz - 2;
    else while (r > o.xDataPND[i + 1]) i++;
    double xL = o.xDataPND[i], yL = o.Zij[i], xR = o.xDataPND[i + 1], yR = o.Zij[i + 1];
    double dydx = (yR - yL) / (xR - xL);
    return yL + dydx * (r - xL);
}
int interpolateNumNeighWall(const Orc& o, double re, double x) {
    int sz = (int)o.xDataNeigh.size();
    double r = x / re;
    int i = 0;
    if (r >= o.xDataNeigh[sz - 2]) i = sz - 2;
    else while (r > o.xDataNeigh[i + 1]) i++;
    double xL = o.xDataNeigh[i], yL = (double)o.nNeighTab[i], xR = o.xDataNeigh[i + 1], yR = (double)o.nNeighTab[i + 1];
    double dydx = (yR - yL) / (xR - xL);
    return (int)(yL + dydx * (r - xL));
}

// PolygonMesh::closestPointPNDBoundaryAABB (src/PolygonMesh.cpp:585-715, rigid mesh)
// followed by updateParticlesNearPolygonMesh (src/PolygonMesh.cpp:718-795)
void wallDistance(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o.N; i++) {
        const double* p = &o.pos[i * 3];
        double best = std::numeric_limits<double>::infinity();
        int bt = -1;
        double bq[3] = {0, 0, 0};
        for (int t = 0; t < o.ntri; t++) {
            double q[3];
            closestPtTri(p, &o.tri[t * 9], q);
            double dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
            double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 < best) { best = d2; bt = t; bq[0] = q[0]; bq[1] = q[1]; bq[2] = q[2]; }
        }
        if (bt >= 0 && best < o.riw2[i]) {
            o.riw2[i] = best;
            for (int k = 0; k < 3; k++) {
                o.wallPos[i * 3 + k] = bq[k];
                o.mirror[i * 3 + k] = p[k] + 2.0 * (bq[k] - p[k]);
                o.polyNormal[i * 3 + k] = o.triNormal[bt * 3 + k];
            }
            o.nearMeshType[i] = 0;
        }
    }
    double reS = std::sqrt(P.reS2), reL = std::sqrt(P.reL2);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o.N; i++) {
        o.pndWall[i] = 0.0;
        o.nNeighWall[i] = 0;
        double x2 = o.riw2[i];
        if (x2 < P.reL2) {
            o.nearWall[i] = 1;
            double x = std::sqrt(x2);
            o.pndWall[i] = interpolateWij(o, reS, x);
            o.nNeighWall[i] = interpolateNumNeighWall(o, reL, x);
        }
    }
}

// ------------------------------------------------------------------ PND / neighbours
// Reflection R = I - 2 n n^T about the wall plane of i, n = (x_i - x_mirror)/|.|, as
// built in e.g. src/MpsPndNeigh.cpp:118-141 (normaliwSqrt variant) and :530-549.
struct Refl {
    double n[3], nsqrt, R[9];
};
Refl reflSqrt(const double* xi, const double* mi, double eps) {
    Refl r;
    r.n[0] = 0.5 * (xi[0] - mi[0]); r.n[1] = 0.5 * (xi[1] - mi[1]); r.n[2] = 0.5 * (xi[2] - mi[2]);
    r.nsqrt = std::sqrt(r.n[0] * r.n[0] + r.n[1] * r.n[1] + r.n[2] * r.n[2]);
    if (r.nsqrt > eps) { for (int k = 0; k < 3; k++) r.n[k] = r.n[k] / r.nsqrt; }
    else { r.n[0] = r.n[1] = r.n[2] = 0; }
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) r.R[a * 3 + b] = (a == b ? 1.0 : 0.0) - 2.0 * r.n[a] * r.n[b];
    return r;
}
// normalMod2 variant (src/MpsViscosity.cpp:1544-1560): threshold on the squared norm
Refl reflMod2(const double* xi, const double* mi, double eps) {
    Refl r;
    r.n[0] = 0.5 * (xi[0] - mi[0]); r.n[1] = 0.5 * (xi[1] - mi[1]); r.n[2] = 0.5 * (xi[2] - mi[2]);
    double m2 = r.n[0] * r.n[0] + r.n[1] * r.n[1] + r.n[2] * r.n[2];
    r.nsqrt = 0.0;
    if (m2 > eps) { double m = std::sqrt(m2); r.nsqrt = m; for (int k = 0; k < 3; k++) r.n[k] = r.n[k] / m; }
    else { r.n[0] = r.n[1] = r.n[2] = 0; }
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) r.R[a * 3 + b] = (a == b ? 1.0 : 0.0) - 2.0 * r.n[a] * r.n[b];
    return r;
}

struct Pair {
    double v0, v1, v2, d2, m0, m1, m2, dm2;
};
inline Pair pairOf(const Orc& o, int j, const double* xi, const double* mi) {
    Pair q;
    const double* pj = &o.pos[j * 3];
    q.v0 = (pj[0] + 0.0) - xi[0]; q.v1 = (pj[1] + 0.0) - xi[1]; q.v2 = (pj[2] + 0.0) - xi[2];
    q.d2 = q.v0 * q.v0 + q.v1 * q.v1 + q.v2 * q.v2;
    q.m0 = (pj[0] + 0.0) - mi[0]; q.m1 = (pj[1] + 0.0) - mi[1]; q.m2 = (pj[2] + 0.0) - mi[2];
    q.dm2 = q.m0 * q.m0 + q.m1 * q.m1 + q.m2 * q.m2;
    return q;
}
inline bool sideOK(const Orc& o, const Pair& q) { return q.d2 < q.dm2 || o.P.wallType == 0; }

// MpsPndNeigh::setInitialPndNumberOfNeighNPCD, src/MpsPndNeigh.cpp:21-101
void setInitialPnd(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        double wSum = 0.0;
        o.numNeigh[i] = 0;
        o.npcd[i * 3] = o.npcd[i * 3 + 1] = o.npcd[i * 3 + 2] = 0.0;
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reL2 && sideOK(o, q) && j != i) {
                o.numNeigh[i] += 1;
                if (q.d2 < P.reS2) {
                    double wS = weight(std::sqrt(q.d2), P.reS, P.weightType);
                    o.pndi[i] += wS;
                    o.npcd[i * 3] += q.v0 * wS; o.npcd[i * 3 + 1] += q.v1 * wS; o.npcd[i * 3 + 2] += q.v2 * wS;
                    wSum += wS;
                }
            }
        });
        o.pndi[i] += o.pndWall[i];
        if (o.type[i] == P.wall) o.pndi[i] = P.pndSmallZero;
        o.pndSmall[i] = o.pndi[i];
        o.pndki[i] = o.pndi[i];
        o.numNeigh[i] += o.nNeighWall[i];
        if (wSum > P.epsilonZero)
            for (int k = 0; k < 3; k++) o.npcd[i * 3 + k] /= o.pndSmall[i];
        double* d = &o.npcd[i * 3];
        o.npcd2[i] = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const double* nw = &o.polyNormal[i * 3];
        o.devDot[i] = (d[0] * nw[0] + d[1] * nw[1] + d[2] * nw[2] < 0.0) ? 1 : -1;
    }
}

// MpsPndNeigh::calcWallNPCD, src/MpsPndNeigh.cpp:105-195
void calcWallNPCD(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        if (!(o.type[i] == P.fluid && o.nearWall[i])) continue;
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        double dx = 0, dy = 0, dz = 0;
        Refl r = reflSqrt(xi, mi, P.epsilonZero);
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && q.dm2 < P.reS2 && q.d2 < q.dm2 && j != i) {
                double wS = weight(std::sqrt(q.dm2), P.reS, P.weightType);
                dx += q.m0 * wS; dy += q.m1 * wS; dz += q.m2 * wS;
            }
        });
        double a0 = xi[0] - mi[0], a1 = xi[1] - mi[1], a2 = xi[2] - mi[2];
        double dii = a0 * a0 + a1 * a1 + a2 * a2;
        if (dii < P.reS2) {
            double wS = weight(std::sqrt(dii), P.reS, P.weightType);
            dx += a0 * wS; dy += a1 * wS; dz += a2 * wS;
        }
        o.npcd[i * 3] += r.R[0] * dx + r.R[1] * dy + r.R[2] * dz;
        o.npcd[i * 3 + 1] += r.R[3] * dx + r.R[4] * dy + r.R[5] * dz;
        o.npcd[i * 3 + 2] += r.R[6] * dx + r.R[7] * dy + r.R[8] * dz;
    }
}

// MpsPndNeigh::calcPndnNeighNPCD, src/MpsPndNeigh.cpp:199-331
void calcPndnNeighNPCD(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        double ni = 0.0, wSum = 0.0;
        o.numNeigh[i] = 0;
        o.numNeigh[i] += o.nNeighWall[i];
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reL2 && sideOK(o, q) && j != i) {
                o.numNeigh[i] += 1;
                if (q.d2 < P.reS2) {
                    double wS = weight(std::sqrt(q.d2), P.reS, P.weightType);
                    ni += wS;
                    o.npcd[i * 3] += q.v0 * wS; o.npcd[i * 3 + 1] += q.v1 * wS; o.npcd[i * 3 + 2] += q.v2 * wS;
                    wSum += wS;
                }
            }
        });
        if (P.pndType == 0 || P.pndType == 1) {
            o.pndki[i] = o.pndi[i];
            o.pndi[i] = ni + o.pndWall[i];
        }
        o.pndSmall[i] = ni + o.pndWall[i];
        if (wSum > P.epsilonZero)
            for (int k = 0; k < 3; k++) o.npcd[i * 3 + k] /= o.pndSmall[i];
        double* d = &o.npcd[i * 3];
        o.npcd2[i] = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const double* nw = &o.polyNormal[i * 3];
        o.devDot[i] = (d[0] * nw[0] + d[1] * nw[1] + d[2] * nw[2] < 0.0) ? 1 : -1;
    }
}

// MpsPndNeigh::calcPndDiffusiveTerm, src/MpsPndNeigh.cpp:334-489
void calcPndDiffusiveTerm(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        double Di = 0.0, DivV = 0.0, flagDi = 1.0;
        const double* xi = &o.pos[i * 3];
        const double* vi = &o.vel[i * 3];
        const double* mi = &o.mirror[i * 3];
        double MC[9] = {o.c1[i * 3], o.c1[i * 3 + 1], o.c1[i * 3 + 2], o.c2[i * 3], o.c2[i * 3 + 1],
                        o.c2[i * 3 + 2], o.c3[i * 3], o.c3[i * 3 + 1], o.c3[i * 3 + 2]};
        double ni = o.pndi[i];
        if (ni < P.epsilonZero) continue;
        double Pi = o.press[i];
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reL2 && sideOK(o, q) && j != i) {
                double dst = std::sqrt(q.d2);
                double wL = weight(dst, P.reL, P.weightType);
                if (o.type[i] == P.fluid && o.type[j] == P.fluid) {
                    double pgh = -2.0 * (o.RHO[i] * o.RHO[j] / (o.RHO[i] + o.RHO[j])) *
                                 (P.gravity[0] * q.v0 + P.gravity[1] * q.v1 + P.gravity[2] * q.v2);
                    double Pj = o.press[j];
                    Di += P.timeStep / o.RHO[i] * P.coeffViscMultiphase * (Pj - Pi - pgh) * wL;
                }
                if (q.d2 < P.reS2) {
                    double vx = o.vel[j * 3] - vi[0], vy = o.vel[j * 3 + 1] - vi[1], vz = o.vel[j * 3 + 2] - vi[2];
                    double wS = weight(dst, P.reS, P.weightType);
                    if (!P.gradientCorrection) {
                        if (ni > P.epsilonZero)
                            DivV += (P.dim / P.pndSmallZero) * (o.pndi[j] / ni) * (vx * q.v0 + vy * q.v1 + vz * q.v2) * wS / q.d2;
                    } else {
                        double c0 = (q.v0 * MC[0] + q.v1 * MC[1] + q.v2 * MC[2]);
                        double c1 = (q.v0 * MC[3] + q.v1 * MC[4] + q.v2 * MC[5]);
                        double c2 = (q.v0 * MC[6] + q.v1 * MC[7] + q.v2 * MC[8]);
                        DivV += (P.dim / P.pndSmallZero) * (vx * c0 + vy * c1 + vz * c2) * wS / q.d2;
                    }
                }
            }
        });
        o.aux1[i] = o.pndi[i] * (1.0 + P.timeStep * (-DivV + Di * flagDi));
        o.velDiv[i] = DivV;
        o.diffTerm[i] = Di;
    }
}

// MpsPndNeigh::calcWallSlipPndDiffusiveTerm / calcWallNoSlipPndDiffusiveTerm,
// src/MpsPndNeigh.cpp:492-602 and :605-744
void calcWallPndDiffusiveTerm(Orc& o) {
    const MpsParams& P = o.P;
    bool noslip = (P.slipCondition == 0);
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        double ni = o.pndi[i];
        if (!(o.type[i] == P.fluid && o.nearWall[i] && ni > P.epsilonZero)) continue;
        double DivV = 0.0;
        const double* xi = &o.pos[i * 3];
        const double* vi = &o.vel[i * 3];
        const double* mi = &o.mirror[i * 3];
        Refl r = reflMod2(xi, mi, P.epsilonZero);
        double vm[3];
        if (noslip) {
            // wall velocity is zero (fixed mesh): vtil = v_i, mirror velocity = -vtil
            double vw[3] = {0, 0, 0};
            double dn = r.n[0] * vw[0] + r.n[1] * vw[1] + r.n[2] * vw[2];
            double vt[3];
            for (int k = 0; k < 3; k++) vt[k] = vi[k] - 2.0 * (vw[k] - dn * r.n[k]);
            // Rinv = -I (src/MpsPndNeigh.cpp:636-638)
            vm[0] = (-1.0 * vt[0] + 0.0 * vt[1] + 0.0 * vt[2]);
            vm[1] = (0.0 * vt[0] + -1.0 * vt[1] + 0.0 * vt[2]);
            vm[2] = (0.0 * vt[0] + 0.0 * vt[1] + -1.0 * vt[2]);
        } else {
            vm[0] = r.R[0] * vi[0] + r.R[1] * vi[1] + r.R[2] * vi[2];
            vm[1] = r.R[3] * vi[0] + r.R[4] * vi[1] + r.R[5] * vi[2];
            vm[2] = r.R[6] * vi[0] + r.R[7] * vi[1] + r.R[8] * vi[2];
        }
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && q.dm2 < P.reS2 && q.d2 < q.dm2 && j != i) {
                double wS = weight(std::sqrt(q.dm2), P.reS, P.weightType);
                double vx = o.vel[j * 3] - vm[0], vy = o.vel[j * 3 + 1] - vm[1], vz = o.vel[j * 3 + 2] - vm[2];
                if (noslip) {
                    vx = -vx; vy = -vy; vz = -vz;
                    double a0 = r.R[0] * q.m0 + r.R[1] * q.m1 + r.R[2] * q.m2;
                    double a1 = r.R[3] * q.m0 + r.R[4] * q.m1 + r.R[5] * q.m2;
                    double a2 = r.R[6] * q.m0 + r.R[7] * q.m1 + r.R[8] * q.m2;
                    DivV += (P.dim / P.pndSmallZero) * (o.pndi[j] / ni) * (vx * a0 + vy * a1 + vz * a2) * wS / q.dm2;
                } else {
                    DivV += (P.dim / P.pndSmallZero) * (o.pndi[j] / ni) * (vx * q.m0 + vy * q.m1 + vz * q.m2) * wS / q.dm2;
                }
            }
        });
        double a0 = xi[0] - mi[0], a1 = xi[1] - mi[1], a2 = xi[2] - mi[2];
        double dii = a0 * a0 + a1 * a1 + a2 * a2;
        if (dii < P.reS2) {
            double wS = weight(std::sqrt(dii), P.reS, P.weightType);
            double vx = vi[0] - vm[0], vy = vi[1] - vm[1], vz = vi[2] - vm[2];
            if (noslip) {
                vx = -vx; vy = -vy; vz = -vz;
                double b0 = r.R[0] * a0 + r.R[1] * a1 + r.R[2] * a2;
                double b1 = r.R[3] * a0 + r.R[4] * a1 + r.R[5] * a2;
                double b2 = r.R[6] * a0 + r.R[7] * a1 + r.R[8] * a2;
                DivV += (P.dim / P.pndSmallZero) * (o.pndi[i] / ni) * (vx * b0 + vy * b1 + vz * b2) * wS / dii;
            } else {
                DivV += (P.dim / P.pndSmallZero) * (o.pndi[i] / ni) * (vx * a0 + vy * a1 + vz * a2) * wS / dii;
            }
        }
        o.aux1[i] += -o.pndi[i] * P.timeStep * DivV;
    }
}

// MpsPndNeigh::updatePnd, src/MpsPndNeigh.cpp:747-774
void updatePnd(Orc& o) {
    for (int i = 0; i < o.N; i++) { o.pndi[i] = o.aux1[i]; o.aux1[i] = 0.0; }
}

// MpsPndNeigh::meanPndParticlesWallDummySurface, src/MpsPndNeigh.cpp:777-852
void meanPndParticlesWallDummySurface(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        o.aux1[i] = 0.0; o.aux2[i] = 0.0;
        if (!(o.type[i] == P.wall || o.bc[i] == P.surface)) continue;
        double up = 0.0, dn = 0.0;
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && sideOK(o, q) && j != i) {
                double wS = weight(std::sqrt(q.d2), P.reS, P.weightType);
                up += o.pndi[j] * wS; dn += wS;
            }
        });
        o.aux1[i] = up; o.aux2[i] = dn;
    }
    for (int i = 0; i < o.N; i++) {
        if (o.type[i] == P.wall || o.bc[i] == P.surface) {
            if (o.aux2[i] < P.epsilonZero) o.pndi[i] = o.aux1[i];
            else o.pndi[i] = o.aux1[i] / o.aux2[i];
        }
        o.aux1[i] = 0.0; o.aux2[i] = 0.0;
    }
}

// MpsPndNeigh::meanWallPnd, src/MpsPndNeigh.cpp:923-994
void meanWallPnd(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        o.aux1[i] = 0.0; o.aux2[i] = 0.0;
        if (!o.nearWall[i]) continue;
        double up = 0.0, dn = 0.0;
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && q.dm2 < P.reS2 && q.d2 < q.dm2 && j != i) {
                double wS = weight(std::sqrt(q.dm2), P.reS, P.weightType);
                up += o.pndi[j] * wS; dn += wS;
            }
        });
        double a0 = xi[0] - mi[0], a1 = xi[1] - mi[1], a2 = xi[2] - mi[2];
        double dii = a0 * a0 + a1 * a1 + a2 * a2;
        if (dii < P.reS2) {
            double wS = weight(std::sqrt(dii), P.reS, P.weightType);
            up += o.pndi[i] * wS; dn += wS;
        }
        o.aux1[i] = up; o.aux2[i] = dn;
    }
}

// MpsPndNeigh::meanPnd, src/MpsPndNeigh.cpp:855-920
void meanPnd(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        double up = 0.0, dn = 0.0;
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && sideOK(o, q) && j != i) {
                double wS = weight(std::sqrt(q.d2), P.reS, P.weightType);
                up += o.pndi[j] * wS; dn += wS;
            }
        });
        o.aux1[i] += up; o.aux2[i] += dn;
    }
    for (int i = 0; i < o.N; i++) {
        if (o.numNeigh[i] < 1) o.pndi[i] = o.aux1[i];
        else o.pndi[i] = o.aux1[i] / o.aux2[i];
        o.aux1[i] = 0.0; o.aux2[i] = 0.0;
    }
}

// MpsPndNeigh::meanNeighFluidPnd, src/MpsPndNeigh.cpp:997-1050
void meanNeighFluidPnd(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        double up = 0.0, dn = 0.0;
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && sideOK(o, q) && j != i && o.type[j] == P.fluid) {
                double wS = weight(std::sqrt(q.d2), P.reS, P.weightType);
                up += o.pndki[j] * wS; dn += wS;
            }
        });
        o.pndski[i] = (dn > P.epsilonZero) ? up / dn : up;
    }
}

// ------------------------------------------------------------------ viscosity
// MpsViscosity::calcViscosity, src/MpsViscosity.cpp:20-100
void calcViscosity(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        double meu_i = o.MEU[i];
        double ax = 0, ay = 0, az = 0;
        const double* xi = &o.pos[i * 3];
        const double* vi = &o.vel[i * 3];
        const double* mi = &o.mirror[i * 3];
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reL2 && sideOK(o, q) && j != i) {
                double wL = weight(std::sqrt(q.d2), P.reL, P.weightType);
                double neu;
                if ((meu_i + o.MEU[j]) > P.epsilonZero) neu = 2.0 * meu_i * o.MEU[j] / (meu_i + o.MEU[j]);
                else neu = 0.0;
                if (o.type[j] == P.wall) neu = 2.0 * meu_i;
                neu = neu / o.RHO[i];
                ax += (o.vel[j * 3] - vi[0]) * wL * neu;
                ay += (o.vel[j * 3 + 1] - vi[1]) * wL * neu;
                az += (o.vel[j * 3 + 2] - vi[2]) * wL * neu;
            }
        });
        o.acc[i * 3] = P.coeffViscMultiphase * ax;
        o.acc[i * 3 + 1] = P.coeffViscMultiphase * ay;
        o.acc[i * 3 + 2] = P.coeffViscMultiphase * az;
    }
}

// MpsViscosity::calcWallSlipViscosity / calcWallNoSlipViscosity (Newtonian),
// src/MpsViscosity.cpp:1527-1684 and :1687-1910
void calcWallViscosity(Orc& o) {
    const MpsParams& P = o.P;
    double VolumeForce = std::pow(P.partDist, P.dim);
    bool noslip = (P.slipCondition == 0);
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        if (!(o.type[i] == P.fluid && o.nearWall[i])) continue;
        double meu_i = o.MEU[i];
        double ax = 0, ay = 0, az = 0;
        const double* xi = &o.pos[i * 3];
        const double* vi = &o.vel[i * 3];
        const double* mi = &o.mirror[i * 3];
        Refl r = reflMod2(xi, mi, P.epsilonZero);
        double M[9];
        double vm[3];
        if (noslip) {
            for (int k = 0; k < 9; k++) M[k] = (k % 4 == 0) ? -1.0 : 0.0;
            double vw[3] = {0, 0, 0};
            double dn = r.n[0] * vw[0] + r.n[1] * vw[1] + r.n[2] * vw[2];
            double vt[3];
            for (int k = 0; k < 3; k++) vt[k] = vi[k] - 2.0 * (vw[k] - dn * r.n[k]);
            vm[0] = (M[0] * vt[0] + M[1] * vt[1] + M[2] * vt[2]);
            vm[1] = (M[3] * vt[0] + M[4] * vt[1] + M[5] * vt[2]);
            vm[2] = (M[6] * vt[0] + M[7] * vt[1] + M[8] * vt[2]);
        } else {
            for (int k = 0; k < 9; k++) M[k] = r.R[k];
            vm[0] = (M[0] * vi[0] + M[1] * vi[1] + M[2] * vi[2]);
            vm[1] = (M[3] * vi[0] + M[4] * vi[1] + M[5] * vi[2]);
            vm[2] = (M[6] * vi[0] + M[7] * vi[1] + M[8] * vi[2]);
        }
        double dens = (o.PTYPE[i] == 1) ? P.DNS_FL1 : P.DNS_FL2;
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reL2 && q.dm2 < P.reL2 && q.d2 < q.dm2 && j != i) {
                double wL = weight(std::sqrt(q.dm2), P.reL, P.weightType);
                double neu;
                if ((meu_i + o.MEU[j]) > P.epsilonZero) neu = 2.0 * meu_i * o.MEU[j] / (meu_i + o.MEU[j]);
                else neu = 0.0;
                neu = neu / dens;
                ax += (o.vel[j * 3] - vm[0]) * wL * neu;
                ay += (o.vel[j * 3 + 1] - vm[1]) * wL * neu;
                az += (o.vel[j * 3 + 2] - vm[2]) * wL * neu;
            }
        });
        double a0 = xi[0] - mi[0], a1 = xi[1] - mi[1], a2 = xi[2] - mi[2];
        double dii = a0 * a0 + a1 * a1 + a2 * a2;
        if (dii < P.reL2) {
            double wL = weight(std::sqrt(dii), P.reL, P.weightType);
            double neu = (meu_i > P.epsilonZero) ? 2.0 * meu_i * meu_i / (meu_i + meu_i) : 0.0;
            neu = neu / dens;
            ax += (vi[0] - vm[0]) * wL * neu;
            ay += (vi[1] - vm[1]) * wL * neu;
            az += (vi[2] - vm[2]) * wL * neu;
        }
        double f0 = (M[0] * ax + M[1] * ay + M[2] * az) * P.coeffViscMultiphase;
        double f1 = (M[3] * ax + M[4] * ay + M[5] * az) * P.coeffViscMultiphase;
        double f2 = (M[6] * ax + M[7] * ay + M[8] * az) * P.coeffViscMultiphase;
        o.acc[i * 3] += f0; o.acc[i * 3 + 1] += f1; o.acc[i * 3 + 2] += f2;
        o.forceWall[i * 3] += -f0 * VolumeForce * o.RHO[i];
        o.forceWall[i * 3 + 1] += -f1 * VolumeForce * o.RHO[i];
        o.forceWall[i * 3 + 2] += -f2 * VolumeForce * o.RHO[i];
    }
}

// ------------------------------------------------------------------ velocity / position
// MpsParticle::addGravity, src/MpsParticle.cpp:111-130
void addGravity(Orc& o) {
    for (int i = 0; i < o.N; i++)
        for (int k = 0; k < 3; k++) {
            o.acc[i * 3 + k] += o.P.gravity[k];
            o.accStar[i * 3 + k] = o.acc[i * 3 + k];
        }
}

// MpsParticleVelPos::predictionVelocityPosition, src/MpsParticleVelPos.cpp:20-50
void predict(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for
    for (int i = 0; i < o.N; i++) {
        if (o.type[i] == P.fluid) {
            for (int k = 0; k < 3; k++) o.vel[i * 3 + k] += o.acc[i * 3 + k] * P.timeStep;
            for (int k = 0; k < 3; k++) o.pos[i * 3 + k] += o.vel[i * 3 + k] * P.timeStep;
        }
        for (int k = 0; k < 3; k++) { o.acc[i * 3 + k] = 0.0; o.dvel[i * 3 + k] = 0.0; o.npcd[i * 3 + k] = 0.0; }
        o.nNeighWall[i] = 0;
        o.nearWall[i] = 0;
        o.riw2[i] = 10e8 * P.partDist;
        if (P.wallType == 1)
            for (int k = 0; k < 3; k++) o.mirror[i * 3 + k] = 10e8 * P.partDist;
    }
}

// MpsParticleVelPos::correctionVelocityPosition, src/MpsParticleVelPos.cpp:53-97
void correct(Orc& o) {
    const MpsParams& P = o.P;
    double vmax = 0.0;
#pragma omp parallel for reduction(max : vmax)
    for (int i = 0; i < o.N; i++) {
        if (o.type[i] != P.fluid) continue;
        for (int k = 0; k < 3; k++) o.vel[i * 3 + k] += o.acc[i * 3 + k] * P.timeStep;
        for (int k = 0; k < 3; k++) o.pos[i * 3 + k] += o.acc[i * 3 + k] * P.timeStep * P.timeStep;
        for (int k = 0; k < 3; k++) o.acc[i * 3 + k] = 0.0;
        double v2 = sq(o.vel[i * 3]) + sq(o.vel[i * 3 + 1]) + sq(o.vel[i * 3 + 2]);
        double v = std::sqrt(v2);
        if (v > vmax) vmax = v;
    }
    o.velMax = vmax;
    o.CFLcurrent = P.timeStep * o.velMax / P.partDist;
}

// MpsParticleVelPos::updateVelocityParticlesWallDummy, src/MpsParticleVelPos.cpp:100-158
void dummyVelocity(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        if (o.type[i] != P.dummyWall) continue;
        const double* xi = &o.pos[i * 3];
        double du[3] = {0, 0, 0}, ni = 0.0;
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            double v0 = o.pos[j * 3] - xi[0], v1 = o.pos[j * 3 + 1] - xi[1], v2 = o.pos[j * 3 + 2] - xi[2];
            double d2 = v0 * v0 + v1 * v1 + v2 * v2;
            if (d2 < P.reL2 && j != i && o.type[j] == P.fluid) {
                double wL = weight(std::sqrt(d2), P.reL, P.weightType);
                ni += wL;
                for (int k = 0; k < 3; k++) du[k] += o.vel[j * 3 + k] * wL;
            }
        });
        for (int k = 0; k < 3; k++)
            o.vel[i * 3 + k] = (ni > P.epsilonZero) ? 2.0 * 0.0 - du[k] / ni : 2.0 * 0.0 - du[k];
    }
}

// ------------------------------------------------------------------ collision
// MpsParticleCollision::checkParticleCollisions, src/MpsParticleCollision.cpp:22-119
void collision(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        if (o.type[i] != P.fluid) continue;
        double mi = (o.PTYPE[i] == 1) ? P.DNS_FL1 : P.DNS_FL2;
        const double* xi = &o.pos[i * 3];
        const double* vi = &o.vel[i * 3];
        const double* mr = &o.mirror[i * 3];
        double dv[3] = {0, 0, 0};
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mr);
            if (q.d2 < P.distCollisionLimit2 && sideOK(o, q) && j != i) {
                double fDT = (vi[0] - o.vel[j * 3]) * q.v0 + (vi[1] - o.vel[j * 3 + 1]) * q.v1 + (vi[2] - o.vel[j * 3 + 2]) * q.v2;
                if (fDT > 0.0) {
                    double mj;
                    if (o.type[j] == P.fluid) mj = (o.PTYPE[j] == 1) ? P.DNS_FL1 : P.DNS_FL2;
                    else mj = o.Dns[1];
                    fDT *= P.restitutionCollision * mj / (mi + mj) / q.d2;
                    if (o.type[j] == P.fluid) { dv[0] -= q.v0 * fDT; dv[1] -= q.v1 * fDT; dv[2] -= q.v2 * fDT; }
                    else { dv[0] -= 2.0 * q.v0 * fDT; dv[1] -= 2.0 * q.v1 * fDT; dv[2] -= 2.0 * q.v2 * fDT; }
                }
            }
        });
        for (int k = 0; k < 3; k++) o.dvel[i * 3 + k] = dv[k];
    }
    for (int i = 0; i < o.N; i++) {
        if (o.type[i] == P.fluid)
            for (int k = 0; k < 3; k++) o.vel[i * 3 + k] += o.dvel[i * 3 + k];
        for (int k = 0; k < 3; k++) o.dvel[i * 3 + k] = 0.0;
    }
}

// MpsParticleCollision::checkDynamicParticleCollisions (DPC), src/MpsParticleCollision.cpp:
// 120-292: pairs closer than l0 off the mirror side; approaching pairs exchange momentum
// with coefficient kappa (1 below l0/2, else chi = sqrt(W_ij / W(l0/2)) of the Wendland-type
// kernel (1 - r/l0)^4 (4 r/l0 + 1)), separating pairs get a dynamic background-pressure
// repulsion; then v += dv and x += dv dt for fluid particles.  (The wall pressure maximum
// the reference computes first is not used.)
void collisionDPC(Orc& o) {
    const MpsParams& P = o.P;
    const double Wij5 = 0.5 * 0.5 * 0.5 * 0.5 * 3.0;
    const double gMod = std::sqrt(P.gravity[0] * P.gravity[0] + P.gravity[1] * P.gravity[1] + P.gravity[2] * P.gravity[2]);
    const double l02 = P.partDist * P.partDist;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        if (o.type[i] != P.fluid) continue;
        double mi = (o.PTYPE[i] == 1) ? P.DNS_FL1 : P.DNS_FL2;
        const double* xi = &o.pos[i * 3];
        const double* vi = &o.vel[i * 3];
        const double* mr = &o.mirror[i * 3];
        double dv[3] = {0, 0, 0};
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mr);
            if (q.d2 < l02 && sideOK(o, q) && j != i) {
                double mj;
                if (o.type[j] == P.fluid) mj = (o.PTYPE[j] == 1) ? P.DNS_FL1 : P.DNS_FL2;
                else mj = o.Dns[1];
                double dst = std::sqrt(q.d2);
                double Wij = 0.0;
                if (dst > P.epsilonZero) {
                    double w1 = 1.0 - dst * P.invPartDist;
                    double w2 = 4.0 * dst * P.invPartDist + 1.0;
                    Wij = w1 * w1 * w1 * w1 * w2;
                }
                double chi = std::sqrt(Wij / Wij5);
                double kappa = (dst < 0.5 * P.partDist) ? 1.0 : chi;
                double fDT = (vi[0] - o.vel[j * 3]) * q.v0 + (vi[1] - o.vel[j * 3 + 1]) * q.v1 + (vi[2] - o.vel[j * 3 + 2]) * q.v2;
                double f2 = (o.type[j] == P.fluid) ? 1.0 : 2.0;
                if (fDT > 0.0) {
                    fDT *= kappa * 2.0 * mj / (mi + mj) / q.d2;
                    dv[0] -= f2 * q.v0 * fDT; dv[1] -= f2 * q.v1 * fDT; dv[2] -= f2 * q.v2 * fDT;
                } else {
                    double pmax = 2.0 / 3.0 * o.RHO[i] * gMod * 0.2;
                    double pmin = o.RHO[i] * gMod * P.partDist;
                    double ptil = std::max(std::min(P.lambdaCollision * std::fabs(o.press[i] + o.press[j]),
                                                    P.lambdaCollision * pmax), pmin);
                    double pb = ptil * chi;
                    double rep = P.timeStep / mi * chi * pb / q.d2;
                    dv[0] -= f2 * q.v0 * rep; dv[1] -= f2 * q.v1 * rep; dv[2] -= f2 * q.v2 * rep;
                }
            }
        });
        for (int k = 0; k < 3; k++) o.dvel[i * 3 + k] = dv[k];
    }
    for (int i = 0; i < o.N; i++) {
        if (o.type[i] == P.fluid)
            for (int k = 0; k < 3; k++) {
                o.vel[i * 3 + k] += o.dvel[i * 3 + k];
                o.pos[i * 3 + k] += o.dvel[i * 3 + k] * P.timeStep;
            }
        for (int k = 0; k < 3; k++) o.dvel[i * 3 + k] = 0.0;
    }
}

// ------------------------------------------------------------------ correction matrix
// MpsVectorMatrix::detMatrix / inverseMatrix, src/MpsVectorMatrix.cpp:96-166
double detMatrix(double a, double b, double c, double d, double e, double f, double g, double h, double k) {
    return (a * e * k + b * f * g + c * d * h) - (c * e * g + b * d * k + a * f * h);
}
void inverseMatrix(double* m, int dimension, double eps) {
    double M[3][3], A[3][3];
    for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) A[r][c] = m[r * 3 + c];
    if (dimension == 2) { A[0][2] = A[1][2] = A[2][0] = A[2][1] = 0.0; A[2][2] = 1.0; }
    for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) M[r][c] = (r == c) ? 1.0 : 0.0;
    double det = detMatrix(A[0][0], A[0][1], A[0][2], A[1][0], A[1][1], A[1][2], A[2][0], A[2][1], A[2][2]);
    if (det <= eps) {
        for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) m[r * 3 + c] = (r == c) ? 1.0 : 0.0;
        return;
    }
    for (int k = 0; k < dimension; k++)
        for (int r = 0; r < dimension; r++) {
            if (r == k) continue;
            double f = A[r][k] / A[k][k];
            for (int c = 0; c < dimension; c++) { A[r][c] -= f * A[k][c]; M[r][c] -= f * M[k][c]; }
        }
    for (int r = 0; r < dimension; r++) for (int c = 0; c < dimension; c++) M[r][c] /= A[r][r];
    for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) m[r * 3 + c] = M[r][c];
}

// MpsVectorMatrix::correctionMatrix, src/MpsVectorMatrix.cpp:20-93
void correctionMatrix(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        double m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && sideOK(o, q) && j != i) {
                double wS = weight(std::sqrt(q.d2), P.reS, P.weightType);
                double inv = 1.0 / q.d2;
                double v[3] = {q.v0, q.v1, q.v2};
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) m[a * 3 + b] += wS * v[a] * v[b] * inv;
            }
        });
        for (int k = 0; k < 9; k++) m[k] *= -P.coeffPressGrad;
        inverseMatrix(m, (int)P.dim, P.epsilonZero);
        if (o.numNeigh[i] < 4) for (int k = 0; k < 9; k++) m[k] = (k % 4 == 0) ? 1.0 : 0.0;
        for (int k = 0; k < 3; k++) { o.c1[i * 3 + k] = m[k]; o.c2[i * 3 + k] = m[3 + k]; o.c3[i * 3 + k] = m[6 + k]; }
    }
}

// ------------------------------------------------------------------ boundary condition
// MpsBoundaryCondition::updateParticleBC (types 0 and 1), src/MpsBoundaryCondition.cpp:173-204
// MpsShifting::calcNormalParticles, src/MpsShifting.cpp:106-166: n_i = -sum r_ij w / |r_ij| / n0
// over the reS ball off the mirror side (every particle)
void calcNormalParticles(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        double d[3] = {0, 0, 0};
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && sideOK(o, q) && j != i) {
                double dst = std::sqrt(q.d2);
                double wS = weight(dst, P.reS, P.weightType);
                d[0] += q.v0 * wS / dst; d[1] += q.v1 * wS / dst; d[2] += q.v2 * wS / dst;
            }
        });
        for (int k = 0; k < 3; k++) o.normal[i * 3 + k] = -d[k] / P.pndSmallZero;
    }
}
// MpsShifting::calcWallNormalParticles, src/MpsShifting.cpp:319-420: mirror entries of the
// fluid near the wall and i itself as a neighbour of its mirror, reflected by R
void calcWallNormalParticles(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        if (!(o.type[i] == P.fluid && o.nearWall[i])) continue;
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        Refl r = reflSqrt(xi, mi, P.epsilonZero);
        double d[3] = {0, 0, 0};
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && q.dm2 < P.reS2 && q.d2 < q.dm2 && j != i) {
                double dst = std::sqrt(q.dm2);
                double wS = weight(dst, P.reS, P.weightType);
                d[0] += q.m0 * wS / dst; d[1] += q.m1 * wS / dst; d[2] += q.m2 * wS / dst;
            }
        });
        double a0 = xi[0] - mi[0], a1 = xi[1] - mi[1], a2 = xi[2] - mi[2];
        double dii = a0 * a0 + a1 * a1 + a2 * a2;
        if (dii < P.reS2) {
            double dst = std::sqrt(dii);
            double wS = weight(dst, P.reS, P.weightType);
            d[0] += a0 * wS / dst; d[1] += a1 * wS / dst; d[2] += a2 * wS / dst;
        }
        for (int k = 0; k < 3; k++)
            o.normal[i * 3 + k] += -(r.R[k * 3] * d[0] + r.R[k * 3 + 1] * d[1] + r.R[k * 3 + 2] * d[2]) / P.pndSmallZero;
    }
}
// the normals the ARC test reads, computed right before it (src/main.cpp:169-175, :351-357)
void normalsForBC(Orc& o) {
    if (o.P.freeSurfType != 2) return;
    calcNormalParticles(o);
    if (o.P.wallType == 1) calcWallNormalParticles(o);
}
// MpsBoundaryCondition::updateParticleBC, src/MpsBoundaryCondition.cpp:66-400: types 0
// (PND + neighbours), 1 (NPCD) and 2 (ARC: inner when PND, neighbour count and normal allow
// it, else by the first neighbour in scan order, real or (polygon) mirrored, whose position
// relative to the normal satisfies the distance / angle tests; surface when some neighbour
// was tested and none passed)
void updateParticleBC(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        if (o.type[i] == P.dummyWall) { o.bc[i] = P.other; continue; }
        o.bc[i] = (o.pndSmall[i] < P.betaPnd) ? P.surface : P.inner;
        if (P.freeSurfType == 0) {
            if (o.pndSmall[i] < P.betaPnd && o.numNeigh[i] < P.betaNeigh) o.bc[i] = P.surface;
            else o.bc[i] = P.inner;
        } else if (P.freeSurfType == 1) {
            if (o.bc[i] == P.surface && o.numNeigh[i] > 4 && o.npcd2[i] < P.delta2) o.bc[i] = P.inner;
        } else if (P.freeSurfType == 2) {
            double n[3] = {o.normal[i * 3], o.normal[i * 3 + 1], o.normal[i * 3 + 2]};
            double norm2 = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
            if (o.pndi[i] >= P.betaPnd && o.numNeigh[i] >= P.betaNeigh && norm2 <= P.normThreshold2) {
                o.bc[i] = P.inner;
                continue;
            }
            const double* xi = &o.pos[i * 3];
            const double* mi = &o.mirror[i * 3];
            if (norm2 > P.epsilonZero) { double nn = std::sqrt(norm2); n[0] /= nn; n[1] /= nn; n[2] /= nn; }
            else n[0] = n[1] = n[2] = 0.0;
            Refl r = reflMod2(xi, mi, P.epsilonZero);
            double nm[3];
            for (int a = 0; a < 3; a++) nm[a] = r.R[a * 3] * n[0] + r.R[a * 3 + 1] * n[1] + r.R[a * 3 + 2] * n[2];
            double nm2 = nm[0] * nm[0] + nm[1] * nm[1] + nm[2] * nm[2];
            if (nm2 > P.epsilonZero) { double q = std::sqrt(nm2); nm[0] /= q; nm[1] /= q; nm[2] /= q; }
            else nm[0] = nm[1] = nm[2] = 0.0;
            bool done = false;
            int bcv = o.bc[i];
            forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
                if (done) return;
                Pair q = pairOf(o, j, xi, mi);
                if (q.d2 < P.reS2 && sideOK(o, q) && j != i) {
                    const double* pj = &o.pos[j * 3];
                    double c0 = pj[0] - (xi[0] + P.partDist * n[0]);
                    double c1 = pj[1] - (xi[1] + P.partDist * n[1]);
                    double c2 = pj[2] - (xi[2] + P.partDist * n[2]);
                    double dinj2 = c0 * c0 + c1 * c1 + c2 * c2;
                    double rijn = q.v0 * n[0] + q.v1 * n[1] + q.v2 * n[2];
                    double ang = std::acos(rijn / std::sqrt(q.d2));
                    if ((q.d2 >= P.dstThreshold2 && dinj2 < P.hThreshold2) || (q.d2 < P.dstThreshold2 && ang < P.thetaArc)) {
                        bcv = P.inner; done = true; return;
                    }
                    bcv = P.surface;
                }
                if (P.wallType == 1 && q.d2 < P.reS2 && q.dm2 < P.reS2 && q.d2 < q.dm2 && j != i) {
                    const double* pj = &o.pos[j * 3];
                    double c0 = pj[0] - (mi[0] + P.partDist * nm[0]);
                    double c1 = pj[1] - (mi[1] + P.partDist * nm[1]);
                    double c2 = pj[2] - (mi[2] + P.partDist * nm[2]);
                    double dimnj2 = c0 * c0 + c1 * c1 + c2 * c2;
                    double rimjn = q.m0 * nm[0] + q.m1 * nm[1] + q.m2 * nm[2];
                    double angm = std::acos(rimjn / std::sqrt(q.dm2));
                    if ((q.dm2 >= P.dstThreshold2 && dimnj2 < P.hThreshold2) || (q.dm2 < P.dstThreshold2 && angm < P.thetaArc)) {
                        bcv = P.inner; done = true; return;
                    }
                    bcv = P.surface;
                }
            });
            o.bc[i] = bcv;
        }
    }
}

// ------------------------------------------------------------------ pressure
// MpsPressure::calcPressEMPS / calcPressWCMPS, src/MpsPressure.cpp:62-163
void pressExplicit(Orc& o) {
    const MpsParams& P = o.P;
    for (int i = 0; i < o.N; i++) {
        double mi = (o.PTYPE[i] == 1) ? P.DNS_FL1 : P.DNS_FL2;
        double p = 0.0;
        if (o.bc[i] == P.inner) {
            if (P.mpsType == 0) p = (o.pndi[i] - P.pndSmallZero) * P.coeffPressEMPS * mi;
            else p = (mi * P.coeffPressWCMPS / P.gamma) * (std::pow(o.pndi[i] / P.pndSmallZero, P.gamma) - 1);
        }
        if (p < 0.0) p = 0.0;
        o.press[i] = p;
    }
}

// Jacobi-preconditioned CG with Eigen's documented stopping rule (||r||^2 < tol^2 ||b||^2,
// checked after each update; warm start x; maxIter default 2N), standing in for
// Eigen::ConjugateGradient<SparseMatrix,Lower|Upper> (src/MpsPressure.cpp:424-445).
// Single-threaded, as the reference's column-major Eigen CG is.
void pcg(Orc& o) {
    int n = o.N;
    const std::vector<long long>& R = o.Arow;
    std::vector<double> diag(n, 1.0), r(n), z(n), p(n), Ap(n);
    auto spmv = [&](const std::vector<double>& x, std::vector<double>& y) {
        for (int i = 0; i < n; i++) {
            double s = 0.0;
            for (long long k = R[i]; k < R[i + 1]; k++) s += o.Aval[k] * x[o.Acol[k]];
            y[i] = s;
        }
    };
    for (int i = 0; i < n; i++)
        for (long long k = R[i]; k < R[i + 1]; k++)
            if (o.Acol[k] == i) diag[i] = o.Aval[k];
    std::vector<double>& x = o.pressurePPE;
    const std::vector<double>& b = o.sourceTerm;
    double bn2 = 0.0;
    for (int i = 0; i < n; i++) bn2 += b[i] * b[i];
    o.solverIter = 0;
    if (bn2 == 0.0) {
        for (int i = 0; i < n; i++) x[i] = 0.0;
        o.solverError = 0.0; o.initialError = 0.0;
        return;
    }
    spmv(x, Ap);
    double rn2 = 0.0;
    for (int i = 0; i < n; i++) { r[i] = b[i] - Ap[i]; rn2 += r[i] * r[i]; }
    o.initialError = std::sqrt(rn2 / bn2);
    double thr = std::max(o.tol * o.tol * bn2, (double)std::numeric_limits<double>::min());
    if (rn2 < thr) { o.solverError = std::sqrt(rn2 / bn2); return; }
    int maxIt = (o.maxIter > 0) ? o.maxIter : 2 * n;
    double absNew = 0.0;
    for (int i = 0; i < n; i++) { z[i] = r[i] / diag[i]; p[i] = z[i]; absNew += r[i] * z[i]; }
    int it = 0;
    while (it < maxIt) {
        spmv(p, Ap);
        double pAp = 0.0;
        for (int i = 0; i < n; i++) pAp += p[i] * Ap[i];
        double alpha = absNew / pAp;
        rn2 = 0.0;
        for (int i = 0; i < n; i++) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; rn2 += r[i] * r[i]; }
        it++;
        if (rn2 < thr) break;
        double absOld = absNew;
        absNew = 0.0;
        for (int i = 0; i < n; i++) { z[i] = r[i] / diag[i]; absNew += r[i] * z[i]; }
        double beta = absNew / absOld;
        for (int i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
    }
    o.solverIter = it;
    o.solverError = std::sqrt(rn2 / bn2);
}

// Jacobi-preconditioned BiCGSTAB (van der Vorst 1992, preconditioner applied on the right)
// with Eigen's documented stopping rule ||r||^2 < tol^2 ||b||^2 and restart of the shadow
// residual when rho vanishes, standing in for Eigen::BiCGSTAB<SparseMatrix>
// (src/MpsPressure.cpp:448-468).  Single-threaded.
void bicgstab(Orc& o) {
    int n = o.N;
    const std::vector<long long>& R = o.Arow;
    std::vector<double> diag(n, 1.0), r(n), r0(n), p(n, 0.0), v(n, 0.0), y(n), s(n), zz(n), t(n);
    auto spmv = [&](const std::vector<double>& x, std::vector<double>& yv) {
        for (int i = 0; i < n; i++) {
            double acc = 0.0;
            for (long long k = R[i]; k < R[i + 1]; k++) acc += o.Aval[k] * x[o.Acol[k]];
            yv[i] = acc;
        }
    };
    auto dot = [&](const std::vector<double>& a, const std::vector<double>& b) {
        double acc = 0.0;
        for (int i = 0; i < n; i++) acc += a[i] * b[i];
        return acc;
    };
    for (int i = 0; i < n; i++)
        for (long long k = R[i]; k < R[i + 1]; k++)
            if (o.Acol[k] == i) diag[i] = o.Aval[k];
    std::vector<double>& x = o.pressurePPE;
    const std::vector<double>& b = o.sourceTerm;
    double bn2 = dot(b, b);
    o.solverIter = 0;
    if (bn2 == 0.0) {
        for (int i = 0; i < n; i++) x[i] = 0.0;
        o.solverError = 0.0; o.initialError = 0.0;
        return;
    }
    spmv(x, t);
    for (int i = 0; i < n; i++) { r[i] = b[i] - t[i]; r0[i] = r[i]; }
    double rn2 = dot(r, r);
    o.initialError = std::sqrt(rn2 / bn2);
    double thr = std::max(o.tol * o.tol * bn2, (double)std::numeric_limits<double>::min());
    double rho = 1.0, alpha = 1.0, w = 1.0;
    double r0n2 = rn2;
    int maxIt = (o.maxIter > 0) ? o.maxIter : 2 * n;
    int it = 0;
    const double eps = std::numeric_limits<double>::epsilon();
    while (rn2 > thr && it < maxIt) {
        double rhoOld = rho;
        rho = dot(r0, r);
        if (std::abs(rho) < eps * eps * r0n2) {   // the shadow residual went orthogonal: restart
            spmv(x, t);
            for (int i = 0; i < n; i++) { r[i] = b[i] - t[i]; r0[i] = r[i]; }
            rho = r0n2 = rn2 = dot(r, r);
            if (rn2 <= thr) break;
            for (int i = 0; i < n; i++) { p[i] = 0.0; v[i] = 0.0; }
            rhoOld = alpha = w = 1.0;
        }
        double beta = (rho / rhoOld) * (alpha / w);
        for (int i = 0; i < n; i++) p[i] = r[i] + beta * (p[i] - w * v[i]);
        for (int i = 0; i < n; i++) y[i] = p[i] / diag[i];
        spmv(y, v);
        alpha = rho / dot(r0, v);
        for (int i = 0; i < n; i++) s[i] = r[i] - alpha * v[i];
        for (int i = 0; i < n; i++) zz[i] = s[i] / diag[i];
        spmv(zz, t);
        double tt = dot(t, t);
        w = (tt > 0.0) ? dot(t, s) / tt : 0.0;
        for (int i = 0; i < n; i++) { x[i] += alpha * y[i] + w * zz[i]; r[i] = s[i] - w * t[i]; }
        rn2 = dot(r, r);
        it++;
    }
    o.solverIter = it;
    o.solverError = std::sqrt(rn2 / bn2);
}

// MpsPressure::calcVelDivergence, src/MpsPressure.cpp:479-557 (fluid particles; reS ball off
// the mirror side; with the correction matrix when gradient correction is on)
void calcVelDivergence(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        o.velDiv[i] = 0.0;
        if (o.type[i] != P.fluid) continue;
        double DivV = 0.0;
        double ni = o.pndi[i];
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        const double* vi = &o.vel[i * 3];
        const double MC[9] = {o.c1[i * 3], o.c1[i * 3 + 1], o.c1[i * 3 + 2], o.c2[i * 3], o.c2[i * 3 + 1],
                              o.c2[i * 3 + 2], o.c3[i * 3], o.c3[i * 3 + 1], o.c3[i * 3 + 2]};
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && sideOK(o, q) && j != i) {
                double vx = o.vel[j * 3] - vi[0], vy = o.vel[j * 3 + 1] - vi[1], vz = o.vel[j * 3 + 2] - vi[2];
                double wS = weight(std::sqrt(q.d2), P.reS, P.weightType);
                if (!P.gradientCorrection) {
                    if (ni > P.epsilonZero)
                        DivV += (P.dim / P.pndSmallZero) * (o.pndi[j] / ni) * (vx * q.v0 + vy * q.v1 + vz * q.v2) * wS / q.d2;
                } else {
                    double c0 = q.v0 * MC[0] + q.v1 * MC[1] + q.v2 * MC[2];
                    double c1 = q.v0 * MC[3] + q.v1 * MC[4] + q.v2 * MC[5];
                    double c2 = q.v0 * MC[6] + q.v1 * MC[7] + q.v2 * MC[8];
                    DivV += (P.dim / P.pndSmallZero) * (vx * c0 + vy * c1 + vz * c2) * wS / q.d2;
                }
            }
        });
        o.velDiv[i] = DivV;
    }
}

// MpsPressure::calcWallSlipVelDivergence / calcWallNoSlipVelDivergence,
// src/MpsPressure.cpp:560-645 / :648-790 (rigid mesh: wall velocity 0): mirror particles of the
// fluid near the wall, velocities mirrored (slip: R v_i; no-slip: -v_i), the no-slip pair
// vectors reflected by R.
void calcWallVelDivergence(Orc& o) {
    const MpsParams& P = o.P;
    const bool noslip = (P.slipCondition == 0);
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        double ni = o.pndi[i];
        if (!(o.type[i] == P.fluid && o.nearWall[i] && ni > P.epsilonZero)) continue;
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        const double* vi = &o.vel[i * 3];
        // both variants normalise with the normalMod2 > eps test (src/MpsPressure.cpp:575-588)
        Refl r = reflMod2(xi, mi, P.epsilonZero);
        double vm[3];
        if (noslip) { vm[0] = -vi[0]; vm[1] = -vi[1]; vm[2] = -vi[2]; }
        else
            for (int a = 0; a < 3; a++) vm[a] = r.R[a * 3] * vi[0] + r.R[a * 3 + 1] * vi[1] + r.R[a * 3 + 2] * vi[2];
        double DivV = 0.0;
        auto term = [&](double vx, double vy, double vz, double m0, double m1, double m2, double dm2, double pj) {
            double wS = weight(std::sqrt(dm2), P.reS, P.weightType);
            if (noslip) {
                vx = -vx; vy = -vy; vz = -vz;
                double a0 = r.R[0] * m0 + r.R[1] * m1 + r.R[2] * m2;
                double a1 = r.R[3] * m0 + r.R[4] * m1 + r.R[5] * m2;
                double a2 = r.R[6] * m0 + r.R[7] * m1 + r.R[8] * m2;
                m0 = a0; m1 = a1; m2 = a2;
            }
            DivV += (P.dim / P.pndSmallZero) * (pj / ni) * (vx * m0 + vy * m1 + vz * m2) * wS / dm2;
        };
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && q.dm2 < P.reS2 && q.d2 < q.dm2 && j != i)
                term(o.vel[j * 3] - vm[0], o.vel[j * 3 + 1] - vm[1], o.vel[j * 3 + 2] - vm[2], q.m0, q.m1, q.m2, q.dm2,
                     o.pndi[j]);
        });
        double a0 = xi[0] - mi[0], a1 = xi[1] - mi[1], a2 = xi[2] - mi[2];
        double dii = a0 * a0 + a1 * a1 + a2 * a2;
        if (dii < P.reS2) term(vi[0] - vm[0], vi[1] - vm[1], vi[2] - vm[2], a0, a1, a2, dii, o.pndi[i]);
        o.velDiv[i] += DivV;
    }
}

// MpsPressure::solvePressurePoissonPnd (src/MpsPressure.cpp:169-286): serial row assembly;
// the N*n_size zero padding triplets at (0,0) add nothing and are not materialised.
void assemblePPE(Orc& o) {
    const MpsParams& P = o.P;
    int n = o.N;
    o.sourceTerm.assign(n, 0.0);
    o.Arow.assign(n + 1, 0);
    o.Acol.clear(); o.Aval.clear();
    for (int i = 0; i < n; i++) {
        if (o.bc[i] == P.other || o.bc[i] == P.surface) {
            o.Acol.push_back(i); o.Aval.push_back(1.0);
            o.Arow[i + 1] = (long long)o.Acol.size();
            continue;
        }
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        double ni = o.pndSmall[i];
        double sum = 0.0;
        std::vector<int> cols; std::vector<double> vals;
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reL2 && sideOK(o, q) && j != i) {
                double wL = weight(std::sqrt(q.d2), P.reL, P.weightType);
                double mij = wL * P.coeffPPE;
                if (o.type[j] == P.dummyWall) {
                    double pgh = o.RHO[j] * (q.v0 * P.gravity[0] + q.v1 * P.gravity[1] + q.v2 * P.gravity[2]) * wL;
                    o.sourceTerm[i] -= P.coeffPPE * pgh;
                } else {
                    sum -= mij;
                    if (o.bc[j] == P.inner) { cols.push_back(j); vals.push_back(mij); }
                }
            }
        });
        double density = (o.PTYPE[i] == 1) ? P.DNS_FL1 : P.DNS_FL2;
        sum -= P.alphaCompressibility * density / (P.timeStep * P.timeStep);
        // CSR row in column order (setFromTriplets sorts); the diagonal merges into place
        cols.push_back(i); vals.push_back(sum);
        std::vector<int> idx(cols.size());
        for (size_t k = 0; k < idx.size(); k++) idx[k] = (int)k;
        std::sort(idx.begin(), idx.end(), [&](int a, int b) { return cols[a] < cols[b]; });
        for (int k : idx) { o.Acol.push_back(cols[k]); o.Aval.push_back(vals[k]); }
        o.Arow[i + 1] = (long long)o.Acol.size();
        if (P.mpsType == 3)   // PND + div u source (src/MpsPressure.cpp:388): the previous PND
            o.sourceTerm[i] += -P.coeffPPESource * density * (o.pndki[i] - P.pndSmallZero) +
                               (1.0 - P.relaxPND) * density * o.velDiv[i] / P.timeStep;
        else
            o.sourceTerm[i] += -P.coeffPPESource * density * (ni - P.pndSmallZero);
    }
}

// MpsPressure::calcPress dispatch (src/MpsPressure.cpp:32-58) with the PND-source PPE,
// CG solve and setZeroOnNegativePressure (src/MpsPressure.cpp:169-286, 424-476)
void calcPress(Orc& o) {
    const MpsParams& P = o.P;
    if (P.mpsType == 0 || P.mpsType == 1) { pressExplicit(o); return; }
    if ((int)o.pressurePPE.size() != o.N) o.sizeMismatch = 1;
    o.pressurePPE.resize(o.N, 0.0);
    if (P.mpsType == 3) {   // src/MpsPressure.cpp:44-56
        calcVelDivergence(o);
        if (P.wallType == 1) calcWallVelDivergence(o);
    }
    assemblePPE(o);
    if (P.solverType == 1) bicgstab(o);
    else pcg(o);
    for (int i = 0; i < o.N; i++) o.press[i] = o.pressurePPE[i];
    for (int i = 0; i < o.N; i++) if (o.press[i] < 0) o.press[i] = 0.0;
}

// MpsPressure::extrapolatePressParticlesWallDummy, src/MpsPressure.cpp:792-846
void extrapolatePress(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        if (!(o.type[i] == P.dummyWall || (P.mpsType == 1 && o.type[i] == P.wall))) continue;
        const double* xi = &o.pos[i * 3];
        double ni = 0.0, pr = 0.0;
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            double v0 = o.pos[j * 3] - xi[0], v1 = o.pos[j * 3 + 1] - xi[1], v2 = o.pos[j * 3 + 2] - xi[2];
            double d2 = v0 * v0 + v1 * v1 + v2 * v2;
            if (d2 < P.reS2 && j != i && o.type[j] == P.fluid) {
                double wS = weight(std::sqrt(d2), P.reS, P.weightType);
                ni += wS;
                pr += (o.press[j] - o.RHO[j] * (P.gravity[0] * v0 + P.gravity[1] * v1 + P.gravity[2] * v2)) * wS;
            }
        });
        if (pr < 0.0) continue;
        o.press[i] = (ni > 0) ? pr / ni : pr;
    }
}

// MpsPressure::calcPressGradient, src/MpsPressure.cpp:1217-1338
void pressGradient(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        double ax = 0, ay = 0, az = 0;
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        double pmin = o.press[i], Pi = o.press[i], ni = o.pndi[i];
        double MC[9] = {o.c1[i * 3], o.c1[i * 3 + 1], o.c1[i * 3 + 2], o.c2[i * 3], o.c2[i * 3 + 1],
                        o.c2[i * 3 + 2], o.c3[i * 3], o.c3[i * 3 + 1], o.c3[i * 3 + 2]};
        if (P.gradientType == 0 || P.gradientType == 2)
            forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
                Pair q = pairOf(o, j, xi, mi);
                if (q.d2 < P.reS2 && sideOK(o, q) && j != i)
                    if (pmin > o.press[j]) pmin = o.press[j];
            });
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && sideOK(o, q) && j != i) {
                double wS = weight(std::sqrt(q.d2), P.reS, P.weightType);
                if (P.gradientType == 0) wS *= (o.press[j] - pmin) / q.d2;
                else if (P.gradientType == 1) wS *= (o.press[j] + Pi) / q.d2;
                else if (P.gradientType == 2) wS *= (o.press[j] + Pi - 2.0 * pmin) / q.d2;
                else if (P.gradientType == 3) {
                    double nj = o.pndi[j];
                    if (ni > P.epsilonZero && nj > P.epsilonZero) wS *= (ni * o.press[j] / nj + nj * Pi / ni) / q.d2;
                }
                if (!P.gradientCorrection) { ax += q.v0 * wS; ay += q.v1 * wS; az += q.v2 * wS; }
                else {
                    ax += (q.v0 * MC[0] + q.v1 * MC[1] + q.v2 * MC[2]) * wS;
                    ay += (q.v0 * MC[3] + q.v1 * MC[4] + q.v2 * MC[5]) * wS;
                    az += (q.v0 * MC[6] + q.v1 * MC[7] + q.v2 * MC[8]) * wS;
                }
            }
        });
        o.acc[i * 3] = P.relaxPress * ax * P.coeffPressGrad / o.RHO[i];
        o.acc[i * 3 + 1] = P.relaxPress * ay * P.coeffPressGrad / o.RHO[i];
        o.acc[i * 3 + 2] = P.relaxPress * az * P.coeffPressGrad / o.RHO[i];
    }
}

// MpsPressure::repulsiveForce{Harada,Mitsume,LennardJones,MonaghanKajtar},
// src/MpsPressure.cpp:1554-1611
void repulsive(const Orc& o, int i, const double* n, double ns, double vMax2, double* f) {
    const MpsParams& P = o.P;
    double w = 0.0;
    if (P.repulsiveForceType == 0) w = o.RHO[i] / (P.timeStep * P.timeStep) * (P.reRepulsiveForce - ns);
    else if (P.repulsiveForceType == 1) w = P.repForceCoefMitsume * weight(ns, P.reRepulsiveForce, P.weightType);
    else if (P.repulsiveForceType == 2) {
        double R1 = (P.reRepulsiveForce / ns) * (P.reRepulsiveForce / ns);
        double R2 = R1 * R1;
        w = (P.repForceCoefLennardJones * vMax2 / ns) * (R2 - R1) * o.RHO[i];
    } else {
        double W1 = (1.0 + 3.0 * 0.5 * ns / (P.reRepulsiveForce));
        double W2 = (1.0 - ns / P.reRepulsiveForce) * (1.0 - ns / P.reRepulsiveForce) * (1.0 - ns / P.reRepulsiveForce);
        w = (P.repForceCoefMonaghanKajtar * vMax2 / (ns - 0.0 * P.partDist)) * (1.0 / 8.0) * W1 * W2 * o.RHO[i];
    }
    f[0] = -w * n[0]; f[1] = -w * n[1]; f[2] = -w * n[2];
}

// MpsPressure::predictionPressGradient, src/MpsPressure.cpp:932-1028 (relax_fact < 1,
// src/main.cpp:271-276): the previous pressure's gradient at the start-of-step positions,
// every particle, no correction matrix, (1 - relax_fact) of it added to the acceleration.
void predictPressGradient(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        double ax = 0, ay = 0, az = 0;
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        double Pi = o.press[i], ni = o.pndi[i], pmin = Pi;
        if (P.gradientType == 0 || P.gradientType == 2)
            forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
                Pair q = pairOf(o, j, xi, mi);
                if (q.d2 < P.reS2 && sideOK(o, q) && j != i)
                    if (pmin > o.press[j]) pmin = o.press[j];
            });
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && sideOK(o, q) && j != i) {
                double wS = weight(std::sqrt(q.d2), P.reS, P.weightType);
                if (P.gradientType == 0) wS *= (o.press[j] - pmin) / q.d2;
                else if (P.gradientType == 1) wS *= (o.press[j] + Pi) / q.d2;
                else if (P.gradientType == 2) wS *= (o.press[j] + Pi - 2.0 * pmin) / q.d2;
                else if (P.gradientType == 3) {
                    double nj = o.pndi[j];
                    if (ni > P.epsilonZero && nj > P.epsilonZero) wS *= (ni * o.press[j] / nj + nj * Pi / ni) / q.d2;
                }
                ax += q.v0 * wS; ay += q.v1 * wS; az += q.v2 * wS;
            }
        });
        o.acc[i * 3] += (1.0 - P.relaxPress) * ax * P.coeffPressGrad / o.RHO[i];
        o.acc[i * 3 + 1] += (1.0 - P.relaxPress) * ay * P.coeffPressGrad / o.RHO[i];
        o.acc[i * 3 + 2] += (1.0 - P.relaxPress) * az * P.coeffPressGrad / o.RHO[i];
    }
}

// MpsPressure::calcWallPressGradient, src/MpsPressure.cpp:1341-1550, and (predict)
// MpsPressure::predictionWallPressGradient, src/MpsPressure.cpp:1031-1214: the same sums
// with (1 - relax_fact) for relax_fact and no force on the wall.
void wallPressGradient(Orc& o, bool predict = false) {
    const MpsParams& P = o.P;
    const double fac = predict ? 1.0 - P.relaxPress : P.relaxPress;
    double VolumeForce = std::pow(P.partDist, P.dim);
    double maxVel = std::min(o.velMax, P.expectMaxVelocity);
    double vMax2 = maxVel * maxVel;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        if (!(o.type[i] == P.fluid && o.nearWall[i])) continue;
        double ax = 0, ay = 0, az = 0;
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        double pmin = o.press[i], Pi = o.press[i], ni = o.pndi[i];
        Refl r = reflSqrt(xi, mi, P.epsilonZero);
        if (P.gradientType == 0 || P.gradientType == 2)
            forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
                Pair q = pairOf(o, j, xi, mi);
                if (q.d2 < P.reS2 && q.d2 < q.dm2 && j != i)
                    if (pmin > o.press[j]) pmin = o.press[j];
            });
        auto phi = [&](double Pj, double nj, double d2, double wS) {
            if (P.gradientType == 0) return wS * ((Pj - pmin) / d2);
            if (P.gradientType == 1) return wS * ((Pj + Pi) / d2);
            if (P.gradientType == 2) return wS * ((Pj + Pi - 2.0 * pmin) / d2);
            if (P.gradientType == 3 && ni > P.epsilonZero && nj > P.epsilonZero) return wS * ((ni * Pj / nj + nj * Pi / ni) / d2);
            return wS;
        };
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && q.dm2 < P.reS2 && q.d2 < q.dm2 && j != i) {
                double wS = weight(std::sqrt(q.dm2), P.reS, P.weightType);
                wS = phi(o.press[j], o.pndi[j], q.dm2, wS);
                ax += q.m0 * wS; ay += q.m1 * wS; az += q.m2 * wS;
            }
        });
        double a0 = xi[0] - mi[0], a1 = xi[1] - mi[1], a2 = xi[2] - mi[2];
        double dii = a0 * a0 + a1 * a1 + a2 * a2;
        if (dii < P.reS2) {
            double wS = weight(std::sqrt(dii), P.reS, P.weightType);
            wS = phi(Pi, o.pndi[i], dii, wS);
            ax += a0 * wS; ay += a1 * wS; az += a2 * wS;
        }
        double f[3] = {0, 0, 0};
        if (r.nsqrt < P.reRepulsiveForce && r.nsqrt > P.epsilonZero) repulsive(o, i, r.n, r.nsqrt, vMax2, f);
        double g0 = fac * (r.R[0] * ax + r.R[1] * ay + r.R[2] * az) * P.coeffPressGrad - f[0];
        double g1 = fac * (r.R[3] * ax + r.R[4] * ay + r.R[5] * az) * P.coeffPressGrad - f[1];
        double g2 = fac * (r.R[6] * ax + r.R[7] * ay + r.R[8] * az) * P.coeffPressGrad - f[2];
        o.acc[i * 3] += g0 / o.RHO[i]; o.acc[i * 3 + 1] += g1 / o.RHO[i]; o.acc[i * 3 + 2] += g2 / o.RHO[i];
        if (predict) continue;
        o.forceWall[i * 3] += -g0 * VolumeForce;
        o.forceWall[i * 3 + 1] += -g1 * VolumeForce;
        o.forceWall[i * 3 + 2] += -g2 * VolumeForce;
    }
}

// ------------------------------------------------------------------ shifting
// MpsShifting::calcShifting (type 1), src/MpsShifting.cpp:23-101.  Velocities of
// neighbours are read before any update (race-free form of the OpenMP sweep).
void shiftVelocity(Orc& o) {
    const MpsParams& P = o.P;
    std::vector<double> v0 = o.vel;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        if (o.type[i] != P.fluid) continue;
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        double du[3] = {0, 0, 0};
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && sideOK(o, q) && j != i) {
                double dw = delWeight(std::sqrt(q.d2), P.reS, P.weightType);
                for (int k = 0; k < 3; k++) du[k] += dw * (v0[j * 3 + k] - v0[i * 3 + k]);
            }
        });
        if (o.bc[i] == P.inner)
            for (int k = 0; k < 3; k++) o.vel[i * 3 + k] -= P.coeffShifting1 * du[k];
    }
}

// MpsShifting::calcConcAndConcGradient + calcWallConcAndConcGradient (type 2),
// src/MpsShifting.cpp:432-575 and :578-691.  The reference moves positions inside the
// OpenMP sweep that reads them (an order-dependent race); here each sweep reads the
// positions as they were when it started, then applies its shifts.
void shiftPosition(Orc& o) {
    const MpsParams& P = o.P;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        double c = 0.0;
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && sideOK(o, q) && j != i) c += weight(std::sqrt(q.d2), P.reS, P.weightType);
        });
        c += o.pndWall[i];
        o.conc[i] = c / P.pndSmallZero;
    }
    std::vector<double> shift(o.N * 3, 0.0);
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        if (o.type[i] != P.fluid) continue;
        double g[3] = {0, 0, 0};
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        double ci = o.conc[i];
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && sideOK(o, q) && j != i) {
                double wS = weight(std::sqrt(q.d2), P.reS, P.weightType);
                g[0] += (ci + o.conc[j]) * q.v0 * wS / q.d2;
                g[1] += (ci + o.conc[j]) * q.v1 * wS / q.d2;
                g[2] += (ci + o.conc[j]) * q.v2 * wS / q.d2;
            }
        });
        for (int k = 0; k < 3; k++) { g[k] *= -P.coeffPressGrad; o.gradC[i * 3 + k] = g[k]; }
        if (o.bc[i] == P.inner)
            for (int k = 0; k < 3; k++) shift[i * 3 + k] = -P.coeffShifting2 * g[k];
    }
    for (int i = 0; i < o.N * 3; i++) o.pos[i] += shift[i];
    if (P.wallType != 1) return;
    std::fill(shift.begin(), shift.end(), 0.0);
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.N; i++) {
        if (!(o.type[i] == P.fluid && o.nearWall[i])) continue;
        const double* xi = &o.pos[i * 3];
        const double* mi = &o.mirror[i * 3];
        double dr[3] = {0, 0, 0};
        double ci = o.conc[i];
        Refl r = reflSqrt(xi, mi, P.epsilonZero);
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            Pair q = pairOf(o, j, xi, mi);
            if (q.d2 < P.reS2 && q.dm2 < P.reS2 && q.d2 < q.dm2 && j != i) {
                double wS = weight(std::sqrt(q.dm2), P.reS, P.weightType);
                dr[0] += (ci + o.conc[j]) * q.m0 * wS / q.dm2;
                dr[1] += (ci + o.conc[j]) * q.m1 * wS / q.dm2;
                dr[2] += (ci + o.conc[j]) * q.m2 * wS / q.dm2;
            }
        });
        double a0 = xi[0] - mi[0], a1 = xi[1] - mi[1], a2 = xi[2] - mi[2];
        double dii = a0 * a0 + a1 * a1 + a2 * a2;
        if (dii < P.reS2) {
            double wS = weight(std::sqrt(dii), P.reS, P.weightType);
            dr[0] += (ci + ci) * a0 * wS / dii; dr[1] += (ci + ci) * a1 * wS / dii; dr[2] += (ci + ci) * a2 * wS / dii;
        }
        double gw[3];
        gw[0] = -(r.R[0] * dr[0] + r.R[1] * dr[1] + r.R[2] * dr[2]) * P.coeffPressGrad;
        gw[1] = -(r.R[3] * dr[0] + r.R[4] * dr[1] + r.R[5] * dr[2]) * P.coeffPressGrad;
        gw[2] = -(r.R[6] * dr[0] + r.R[7] * dr[1] + r.R[8] * dr[2]) * P.coeffPressGrad;
        for (int k = 0; k < 3; k++) o.gradC[i * 3 + k] += gw[k];
        if (o.bc[i] == P.inner)
            for (int k = 0; k < 3; k++) shift[i * 3 + k] = -P.coeffShifting2 * gw[k];
    }
    for (int i = 0; i < o.N * 3; i++) o.pos[i] += shift[i];
}

// ------------------------------------------------------------------ sequences
int runOp(Orc& o, int op) {
    const MpsParams& P = o.P;
    switch (op) {
        case MPS_OP_UPDATE_BUCKETS: return updateParticlesID(o);
        case MPS_OP_VISCOSITY: calcViscosity(o); return 0;
        case MPS_OP_ADD_GRAVITY: addGravity(o); return 0;
        case MPS_OP_PREDICT: predict(o); return 0;
        case MPS_OP_OUT_OF_DOMAIN: checkParticleOutDomain(o); return 0;
        case MPS_OP_COLLISION: if (P.collisionType == 1) collisionDPC(o); else collision(o); return 0;
        case MPS_OP_WALL_DISTANCE: if (P.wallType == 1) wallDistance(o); return 0;
        case MPS_OP_WALL_NPCD: if (P.wallType == 1) calcWallNPCD(o); return 0;
        case MPS_OP_CORRECTION_MATRIX: correctionMatrix(o); return 0;
        case MPS_OP_PND_NEIGH_NPCD: calcPndnNeighNPCD(o); return 0;
        case MPS_OP_PND_DIFFUSIVE:
            calcPndDiffusiveTerm(o);
            if (P.wallType == 1) calcWallPndDiffusiveTerm(o);
            updatePnd(o);
            meanPndParticlesWallDummySurface(o);
            return 0;
        case MPS_OP_PND_MEAN:
            if (P.wallType == 1) meanWallPnd(o);
            meanPnd(o);
            return 0;
        case MPS_OP_UPDATE_BC: normalsForBC(o); updateParticleBC(o); return 0;
        case MPS_OP_CALC_PRESS: calcPress(o); return o.sizeMismatch ? MPSGPU_ERR_SIZE_MISMATCH : 0;
        case MPS_OP_EXTRAPOLATE_PRESS: extrapolatePress(o); return 0;
        case MPS_OP_PRESS_GRADIENT: pressGradient(o); return 0;
        case MPS_OP_WALL_PRESS_GRADIENT: if (P.wallType == 1) wallPressGradient(o); return 0;
        case MPS_OP_WALL_VISCOSITY: if (P.wallType == 1) calcWallViscosity(o); return 0;
        case MPS_OP_CORRECT: correct(o); return 0;
        case MPS_OP_SHIFTING:
            if (P.shiftingType == 1) shiftVelocity(o);
            else if (P.shiftingType == 2) shiftPosition(o);
            return 0;
        case MPS_OP_DUMMY_VELOCITY: dummyVelocity(o); return 0;
        case MPS_OP_PREDICT_PRESS_GRADIENT:
            if (P.relaxPress < 1.0) {
                predictPressGradient(o);
                if (P.wallType == 1) wallPressGradient(o, true);
            }
            return 0;
        case MPS_OP_INIT_PND:
            setInitialPnd(o);
            if (P.wallType == 1) meanWallPnd(o);
            meanPnd(o);
            meanNeighFluidPnd(o);
            return 0;
        default: return MPSGPU_ERR_ARG;
    }
}

// main(): src/main.cpp:116-180 (with initMesh, src/main.cpp:471-556)
int initialize(Orc& o) {
    const MpsParams& P = o.P;
    int e = updateParticlesID(o);
    if (e) return e;
    checkParticleOutDomain(o);
    if (P.wallType == 1) { wallDistance(o); calcWallNPCD(o); }
    if (P.mpsType == 2 || P.mpsType == 3) o.pressurePPE.assign(o.N, 0.0);
    runOp(o, MPS_OP_INIT_PND);
    normalsForBC(o);
    updateParticleBC(o);
    calcPress(o);
    return 0;
}

// mainLoopOfSimulation body, src/main.cpp:256-467
int step(Orc& o) {
    const MpsParams& P = o.P;
    o.outRemoved = 0;
    int e = updateParticlesID(o);
    if (e) return e;
    calcViscosity(o);
    addGravity(o);
    runOp(o, MPS_OP_PREDICT_PRESS_GRADIENT);
    predict(o);
    checkParticleOutDomain(o);
    if (P.collisionType == 1) collisionDPC(o);
    else collision(o);
    if (P.wallType == 1) { wallDistance(o); calcWallNPCD(o); }
    if (P.gradientCorrection) correctionMatrix(o);
    calcPndnNeighNPCD(o);
    if (P.pndType == 2) runOp(o, MPS_OP_PND_DIFFUSIVE);
    else if (P.pndType == 1) runOp(o, MPS_OP_PND_MEAN);
    normalsForBC(o);
    updateParticleBC(o);
    calcPress(o);
    if (P.wallType == 0) extrapolatePress(o);
    if (P.gradientCorrection) correctionMatrix(o);
    pressGradient(o);
    if (P.wallType == 1) { wallPressGradient(o); calcWallViscosity(o); }
    correct(o);
    checkParticleOutDomain(o);
    if (P.shiftingType == 1) shiftVelocity(o);
    else if (P.shiftingType == 2) shiftPosition(o);
    if (P.wallType == 0) dummyVelocity(o);
    checkParticleOutDomain(o);
    o.numOfIterations++;
    o.timeCurrent += P.timeStep;
    return o.sizeMismatch ? MPSGPU_ERR_SIZE_MISMATCH : 0;
}

enum Kind { KV, KS, KI, KB };
struct FieldRef { Kind kind; void* ptr; };
FieldRef fieldRef(Orc& o, int f) {
    switch (f) {
        case MPS_F_POS: return {KV, o.pos.data()};
        case MPS_F_VEL: return {KV, o.vel.data()};
        case MPS_F_ACC: return {KV, o.acc.data()};
        case MPS_F_ACCSTAR: return {KV, o.accStar.data()};
        case MPS_F_NPCD: return {KV, o.npcd.data()};
        case MPS_F_GRADC: return {KV, o.gradC.data()};
        case MPS_F_CORR1: return {KV, o.c1.data()};
        case MPS_F_CORR2: return {KV, o.c2.data()};
        case MPS_F_CORR3: return {KV, o.c3.data()};
        case MPS_F_MIRROR: return {KV, o.mirror.data()};
        case MPS_F_WALLPOS: return {KV, o.wallPos.data()};
        case MPS_F_POLYNORMAL: return {KV, o.polyNormal.data()};
        case MPS_F_FORCEWALL: return {KV, o.forceWall.data()};
        case MPS_F_NORMAL: return {KV, o.normal.data()};
        case MPS_F_PRESS: return {KS, o.press.data()};
        case MPS_F_PRESSPPE: return {KS, o.pressurePPE.data()};
        case MPS_F_PNDI: return {KS, o.pndi.data()};
        case MPS_F_PNDKI: return {KS, o.pndki.data()};
        case MPS_F_PNDSKI: return {KS, o.pndski.data()};
        case MPS_F_PNDSMALL: return {KS, o.pndSmall.data()};
        case MPS_F_NPCD2: return {KS, o.npcd2.data()};
        case MPS_F_CONC: return {KS, o.conc.data()};
        case MPS_F_VELDIV: return {KS, o.velDiv.data()};
        case MPS_F_DIFFTERM: return {KS, o.diffTerm.data()};
        case MPS_F_PNDWALL: return {KS, o.pndWall.data()};
        case MPS_F_RIW2: return {KS, o.riw2.data()};
        case MPS_F_DEVDOT: return {KS, o.devDot.data()};
        case MPS_F_SOURCE: return {KS, o.sourceTerm.data()};
        case MPS_F_TYPE: return {KI, o.type.data()};
        case MPS_F_BC: return {KI, o.bc.data()};
        case MPS_F_NUMNEIGH: return {KI, o.numNeigh.data()};
        case MPS_F_NNEIGHWALL: return {KI, o.nNeighWall.data()};
        case MPS_F_NEARWALL: return {KB, o.nearWall.data()};
        default: return {KS, nullptr};
    }
}

}  // namespace

extern "C" {

int orc_params_derive(MpsParams* p, int n, const double* pos3) { return deriveParams(p, n, pos3); }

int orc_create(const MpsParams* p, int n, const int* type, const double* pos3, const double* vel3,
               const double* press, const MpsMesh* mesh, void** out) {
    if (!p || !p->derived || n <= 0 || !type || !pos3 || !out) return MPSGPU_ERR_ARG;
    Orc* o = new Orc();
    o->P = *p;
    o->N = o->N0 = n;
    auto I = [&](std::vector<int>& v, int x) { v.assign(n, x); };
    auto S = [&](std::vector<double>& v, double x) { v.assign(n, x); };
    auto V = [&](std::vector<double>& v) { v.assign((size_t)n * 3, 0.0); };
    o->type.assign(type, type + n);
    I(o->bc, 0); I(o->numNeigh, 0); I(o->nNeighWall, 0); I(o->nearMeshType, 0); I(o->PTYPE, 1);
    o->nearWall.assign(n, 0);
    S(o->press, 0); S(o->pndi, 0); S(o->pndki, 0); S(o->pndski, 0); S(o->pndSmall, 0); S(o->npcd2, 0);
    S(o->conc, 0); S(o->velDiv, 0); S(o->diffTerm, 0); S(o->aux1, 0); S(o->aux2, 0); S(o->pndWall, 0);
    S(o->devDot, 0); S(o->riw2, 10e8 * p->partDist);
    // Newtonian: RHO = DNS_FL1, PTYPE = 1, MEU = KNM_VS1*DNS_FL1 (src/MpsInputOutput.cpp:833-838)
    S(o->RHO, p->DNS_FL1); S(o->MEU, p->KNM_VS1 * p->DNS_FL1);
    V(o->pos); V(o->vel); V(o->acc); V(o->accStar); V(o->npcd); V(o->gradC); V(o->c1); V(o->c2); V(o->c3);
    V(o->dvel); V(o->wallPos); V(o->mirror); V(o->polyNormal); V(o->forceWall); V(o->normal);
    std::memcpy(o->pos.data(), pos3, sizeof(double) * n * 3);
    if (vel3) std::memcpy(o->vel.data(), vel3, sizeof(double) * n * 3);
    if (press) std::memcpy(o->press.data(), press, sizeof(double) * n);
    o->pressurePPE.assign(n, 0.0);
    o->sourceTerm.assign(n, 0.0);
    o->first.assign(p->numBucketsXYZ, -1);
    o->last.assign(p->numBucketsXYZ, -1);
    o->next.assign(n, -1);
    o->Dns[0] = p->densityFluid; o->Dns[1] = p->densityWall;
    o->CFLcurrent = p->cflNumber;
    if (p->wallType == 1) {
        if (!mesh || mesh->ntri <= 0 || !mesh->tri_xyz) { delete o; return MPSGPU_ERR_ARG; }
        o->ntri = mesh->ntri;
        o->tri.assign(mesh->tri_xyz, mesh->tri_xyz + 9 * mesh->ntri);
        o->triNormal.assign(3 * mesh->ntri, 0.0);
        for (int t = 0; t < o->ntri; t++) {
            const double* v = &o->tri[t * 9];
            double e1[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]}, e2[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
            double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            double l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
            for (int k = 0; k < 3; k++) o->triNormal[t * 3 + k] = (l > 0) ? c[k] / l : 0.0;
        }
        initWijnNeigh(*o);
    }
    *out = o;
    return 0;
}

int orc_destroy(void* h) { delete (Orc*)h; return 0; }
int orc_initialize(void* h) { return initialize(*(Orc*)h); }
int orc_step(void* h, MpsStepStats* st) {
    Orc& o = *(Orc*)h;
    auto t0 = std::chrono::steady_clock::now();
    int e = step(o);
    auto t1 = std::chrono::steady_clock::now();
    if (st) {
        std::memset(st, 0, sizeof(*st));
        st->numParticles = o.N; st->ppeIterations = o.solverIter; st->outOfDomain = o.outRemoved;
        st->velMax = o.velMax; st->CFLcurrent = o.CFLcurrent; st->ppeRelResidual = o.solverError;
        st->ppeInitialRelResidual = o.initialError;
        st->stepMs = std::chrono::duration<double, std::milli>(t1 - t0).count();
    }
    return e;
}
int orc_run_op(void* h, int op) { return runOp(*(Orc*)h, op); }
int orc_set_solver(void* h, double tol, int max_iter) {
    Orc& o = *(Orc*)h; o.tol = tol; o.maxIter = max_iter; return 0;
}
int orc_num_particles(void* h, int* n) { *n = ((Orc*)h)->N; return 0; }
int orc_state(void* h, double* t, int* it, double* velMax, int* solverIter, double* solverErr) {
    Orc& o = *(Orc*)h;
    if (t) *t = o.timeCurrent;
    if (it) *it = o.numOfIterations;
    if (velMax) *velMax = o.velMax;
    if (solverIter) *solverIter = o.solverIter;
    if (solverErr) *solverErr = o.solverError;
    return 0;
}
int orc_set_velmax(void* h, double v) { ((Orc*)h)->velMax = v; return 0; }

int orc_get_field(void* h, int f, void* out) {
    Orc& o = *(Orc*)h;
    FieldRef r = fieldRef(o, f);
    if (!r.ptr) return MPSGPU_ERR_ARG;
    size_t n = o.N;
    if (r.kind == KV) std::memcpy(out, r.ptr, n * 3 * sizeof(double));
    else if (r.kind == KS) std::memcpy(out, r.ptr, n * sizeof(double));
    else if (r.kind == KI) std::memcpy(out, r.ptr, n * sizeof(int));
    else { int* d = (int*)out; const char* s = (const char*)r.ptr; for (size_t i = 0; i < n; i++) d[i] = s[i]; }
    return 0;
}
int orc_set_field(void* h, int f, const void* in) {
    Orc& o = *(Orc*)h;
    FieldRef r = fieldRef(o, f);
    if (!r.ptr) return MPSGPU_ERR_ARG;
    size_t n = o.N;
    if (r.kind == KV) std::memcpy(r.ptr, in, n * 3 * sizeof(double));
    else if (r.kind == KS) std::memcpy(r.ptr, in, n * sizeof(double));
    else if (r.kind == KI) std::memcpy(r.ptr, in, n * sizeof(int));
    else { const int* s = (const int*)in; char* d = (char*)r.ptr; for (size_t i = 0; i < n; i++) d[i] = (char)(s[i] != 0); }
    return 0;
}

// Neighbour sets as every sweep sees them: 27-bucket scan, dst^2 < reL^2, j != i.
int orc_get_neighbors(void* h, int* counts, int* nbr, long long cap) {
    Orc& o = *(Orc*)h;
    long long k = 0;
    for (int i = 0; i < o.N; i++) {
        const double* xi = &o.pos[i * 3];
        int c = 0;
        forCandidates(o, xi[0], xi[1], xi[2], [&](int j) {
            double v0 = o.pos[j * 3] - xi[0], v1 = o.pos[j * 3 + 1] - xi[1], v2 = o.pos[j * 3 + 2] - xi[2];
            double d2 = v0 * v0 + v1 * v1 + v2 * v2;
            if (d2 < o.P.reL2 && j != i) {
                if (nbr) { if (k >= cap) return; nbr[k] = j; }
                k++; c++;
            }
        });
        counts[i] = c;
    }
    return (nbr && k > cap) ? MPSGPU_ERR_CAPACITY : 0;
}

int orc_get_ppe(void* h, long long* nnz, long long* rowptr, int* col, double* val, double* rhs) {
    Orc& o = *(Orc*)h;
    if (nnz) *nnz = o.Arow.empty() ? 0 : o.Arow.back();
    if (!col) return 0;
    std::memcpy(rowptr, o.Arow.data(), sizeof(long long) * o.Arow.size());
    std::memcpy(col, o.Acol.data(), sizeof(int) * o.Acol.size());
    std::memcpy(val, o.Aval.data(), sizeof(double) * o.Aval.size());
    if (rhs) std::memcpy(rhs, o.sourceTerm.data(), sizeof(double) * o.sourceTerm.size());
    return 0;
}

// Wall tables (for the known-answer tests of initWijnNeigh)
int orc_wall_tables(void* h, double* xpnd, double* zij, double* xneigh, int* nneigh) {
    Orc& o = *(Orc*)h;
    if (o.xDataPND.size() != 50) return MPSGPU_ERR_ARG;
    for (int i = 0; i < 50; i++) { xpnd[i] = o.xDataPND[i]; zij[i] = o.Zij[i]; xneigh[i] = o.xDataNeigh[i]; nneigh[i] = o.nNeighTab[i]; }
    return 0;
}

// Standalone PCG on a caller-supplied CSR (used to cross-check the CG against scipy).
int orc_pcg_csr(int n, const long long* rowptr, const int* col, const double* val, const double* b,
                double* x, double tol, int max_iter, int* iters, double* err) {
    Orc o;
    o.N = n;
    o.Arow.assign(rowptr, rowptr + n + 1);
    o.Acol.assign(col, col + rowptr[n]);
    o.Aval.assign(val, val + rowptr[n]);
    o.sourceTerm.assign(b, b + n);
    o.pressurePPE.assign(x, x + n);
    o.tol = tol; o.maxIter = max_iter;
    pcg(o);
    std::memcpy(x, o.pressurePPE.data(), sizeof(double) * n);
    if (iters) *iters = o.solverIter;
    if (err) *err = o.solverError;
    return 0;
}

int orc_set_threads(int t) { omp_set_num_threads(t); return 0; }

}  // extern "C"
