// mps_host.cpp — host-side set-up of libmpsgpu (no CUDA): derived constants and wall
// tables.  Compiled with -ffp-contract=off so the derived constants are the IEEE results
// of the reference's own expressions on every host architecture.
#include <cmath>
#include <cstring>
#include <limits>
#include <algorithm>
#include "mps_host.h"

namespace {

// MpsParticle::weight, src/MpsParticle.cpp:57-72
double weightH(double dst, double re, int t) {
    switch (t) {
        case 1: return re / dst + dst / re - 2.0;
        case 2: return re / dst - dst / re;
        case 3: return (1.0 - dst / re) * (1.0 - dst / re) * (1.0 - dst / re);
        case 4: return (1.0 - dst / re) * (1.0 - dst / re);
        default: return re / dst - 1.0;
    }
}

// MpsBucket::calcDomainLimits, non-periodic branch (src/MpsBucket.cpp:71-143, 289-294):
// limits from the particle extents (limitTypeBC 0) or the JSON box, widened by half a
// particle spacing and one bucket, bucket counts rounded up to whole buckets.
int limitsFromParticles(MpsParams* P, int n, const double* pos) {
    double lo[3], hi[3];
    if (P->limitTypeBC == 0) {
        if (n <= 0 || !pos) return MPSGPU_ERR_ARG;
        for (int k = 0; k < 3; k++) lo[k] = hi[k] = pos[k];
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) {
                lo[k] = std::min(lo[k], pos[3 * i + k]);
                hi[k] = std::max(hi[k], pos[3 * i + k]);
            }
        int used = 0;
        for (int k = 0; k < 3; k++) used += (lo[k] != hi[k]) ? 1 : 0;
        if (used != (int)P->dim) return MPSGPU_ERR_ARG;   // the reference exits with code 10
    } else {
        for (int k = 0; k < 3; k++) { lo[k] = P->domainMin[k]; hi[k] = P->domainMax[k]; }
    }
    if (P->domainTypeBC == 0 && P->wallType == 0) {
        int dims = (P->dim == 3) ? 3 : 2;
        for (int k = 0; k < dims; k++) { lo[k] -= 0.5 * P->partDist; hi[k] += 0.5 * P->partDist; }
        int* counts[3] = {&P->numBucketsX, &P->numBucketsY, &P->numBucketsZ};
        for (int k = 0; k < (int)P->dim; k++) {
            lo[k] -= P->bucketSide;
            hi[k] += P->bucketSide;
            *counts[k] = (int)(long)((hi[k] - lo[k]) / P->bucketSide + 1);
            hi[k] = lo[k] + (*counts[k]) * P->bucketSide;
        }
    }
    for (int k = 0; k < 3; k++) { P->domainMin[k] = lo[k]; P->domainMax[k] = hi[k]; }
    return 0;
}

}  // namespace

// MpsParticle::setParameters (src/MpsParticle.cpp:136-227) and MpsBucket::allocateMemory
// (src/MpsBucket.cpp:20-67)
int hostDeriveParams(MpsParams* P, int n, const double* pos) {
    if (!P) return MPSGPU_ERR_ARG;
    if (P->derived) return 0;
    if (P->partDist <= 0 || (P->dim != 2 && P->dim != 3)) return MPSGPU_ERR_ARG;
    P->epsilonZero = 10.0 * std::numeric_limits<double>::epsilon();
    if (P->partDist * P->partDist <= P->epsilonZero) return MPSGPU_ERR_ARG;  // src/MpsInputOutput.cpp:531-536
    for (int k = 0; k < 3; k++) {
        P->domainMin[k] -= P->partDist * 3.0;
        P->domainMax[k] += P->partDist * 3.0;
    }
    if ((int)P->dim == 2) { P->domainMin[2] = 0.0; P->domainMax[2] = 0.0; }
    P->reS = P->partDist * P->reS;
    P->reL = P->partDist * P->reL;
    P->reRepulsiveForce = P->partDist * P->reRepulsiveForce;
    P->reS2 = P->reS * P->reS;
    P->reL2 = P->reL * P->reL;
    P->EPS_RE = P->EPS_RE * P->reS2 / 4.0;
    // lattice sums over a fully filled support
    double nS = 0, nL = 0, nG = 0, lam = 0, nn = 0;
    int lmin = (int)std::ceil(P->reL / P->partDist) + 1;
    int lmax = (int)std::ceil(P->reL / P->partDist) + 2;
    bool two = (int)P->dim == 2;
    int zlo = two ? 0 : -lmin, zhi = two ? 1 : lmax;
    for (int ix = -lmin; ix < lmax; ix++)
        for (int iy = -lmin; iy < lmax; iy++)
            for (int iz = zlo; iz < zhi; iz++) {
                double x = P->partDist * (double)ix, y = P->partDist * (double)iy, z = P->partDist * (double)iz;
                double r2 = x * x + y * y + z * z;
                if (r2 > P->reL2 || r2 <= P->epsilonZero) continue;
                double r = std::sqrt(r2);
                nL += weightH(r, P->reL, P->weightType);
                lam += r2 * weightH(r, P->reL, P->weightType);
                nn += 1;
                if (r2 <= P->reS2) {
                    nS += weightH(r, P->reS, P->weightType);
                    nG += weightH(r, P->reS, P->weightType);
                }
            }
    P->pndSmallZero = nS; P->pndLargeZero = nL; P->pndGradientZero = nG; P->numNeighZero = nn;
    P->lambdaZero = lam / nL;
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
    // bucket grid: side reL (1 + CFL), three spare buckets
    P->bucketSide = P->reL * (1.0 + P->cflNumber);
    P->invBucketSide = 1.0 / P->bucketSide;
    P->numBucketsX = (int)((P->domainMax[0] - P->domainMin[0]) * P->invBucketSide) + 3;
    P->numBucketsY = (int)((P->domainMax[1] - P->domainMin[1]) * P->invBucketSide) + 3;
    P->numBucketsZ = (int)((P->domainMax[2] - P->domainMin[2]) * P->invBucketSide) + 3;
    if (two) P->numBucketsZ = 1;
    if (P->wallType == 0 || P->domainTypeBC == 1) {
        int e = limitsFromParticles(P, n, pos);
        if (e) return e;
        P->invBucketSide = 1.0 / P->bucketSide;
    }
    P->numBucketsXY = P->numBucketsX * P->numBucketsY;
    P->numBucketsXYZ = P->numBucketsX * P->numBucketsY * P->numBucketsZ;
    P->derived = 1;
    return 0;
}

// PolygonMesh::initWijnNeigh (src/PolygonMesh.cpp:377-527): wall PND Z(r) and wall
// neighbour counts for a particle at distance r = k reS / 50 (k = 1..50) above a
// half-space lattice whose first layer sits l0/2 below the wall.
void hostWallTables(const MpsParams& P, double* tab) {
    const int n = 50;
    int dim = (int)P.dim, wt = P.weightType;
    double lo = P.partDist, reS = P.reS, reL = P.reL, reS2 = reS * reS, reL2 = reL * reL;
    int limS = (int)std::ceil(reS / lo), limL = (int)std::ceil(reL / lo);
    double* xPND = tab;
    double* Z = tab + n;
    double* xN = tab + 2 * n;
    double* cnt = tab + 3 * n;
    for (int s = 1; s <= n; s++) {
        double xi = 0.0, yi = s * reS / n, zi = 0.0;
        double riw = (dim == 3) ? std::sqrt((0.0 - xi) * (0.0 - xi) + (0.0 - yi) * (0.0 - yi) + (0.0 - zi) * (0.0 - zi))
                                : std::sqrt((0.0 - xi) * (0.0 - xi) + (0.0 - yi) * (0.0 - yi));
        xPND[s - 1] = riw / reS;
        xN[s - 1] = riw / reL;
        double sum = 0.0;
        int zl = (dim == 3) ? -limS : 0, zh = (dim == 3) ? limS : 0;
        for (int ix = -limS; ix <= limS; ix++)
            for (int iy = -limS; iy <= 0; iy++)
                for (int iz = zl; iz <= zh; iz++) {
                    double xj = lo * (double)ix, yj = lo * (double)(iy - 0.5), zj = lo * (double)iz;
                    double r2 = (dim == 3) ? (xj - xi) * (xj - xi) + (yj - yi) * (yj - yi) + (zj - zi) * (zj - zi)
                                           : (xj - xi) * (xj - xi) + (yj - yi) * (yj - yi);
                    if (!(r2 < reS2) || r2 == 0.0) continue;
                    double r = std::sqrt(r2);
                    if (wt == 1) sum += reS / r + r / reS - 2.0;
                    else if (wt == 2) sum += reS / r - r / reS;
                    else if (wt == 3) sum += std::pow(1.0 - r / reS, 3.0);
                    else if (wt == 4) sum += std::pow(1.0 - r / reS, 2.0);
                    else sum += reS / r - 1.0;
                }
        Z[s - 1] = sum;
        int c = 0;
        zl = (dim == 3) ? -limL : 0; zh = (dim == 3) ? limL : 0;
        for (int ix = -limL; ix <= limL; ix++)
            for (int iy = -limL; iy <= 0; iy++)
                for (int iz = zl; iz <= zh; iz++) {
                    double xj = lo * (double)ix, yj = lo * (double)(iy - 0.5), zj = lo * (double)iz;
                    double r2 = (dim == 3) ? (xj - xi) * (xj - xi) + (yj - yi) * (yj - yi) + (zj - zi) * (zj - zi)
                                           : (xj - xi) * (xj - xi) + (yj - yi) * (yj - yi);
                    if (r2 < reL2 && r2 != 0.0) c++;
                }
        cnt[s - 1] = (double)c;
    }
}

// Plane data of each triangle for the wall-distance kernel's projection path (16 doubles
// per triangle): unit normal n and n.a, then for each edge (a,b), (b,c), (c,a) its unit
// in-plane normal e pointing into the triangle and e.v0.  A degenerate triangle or edge
// gets zero normals and offsets 1, so no point is ever inside it.
void hostTrianglePlanes(int ntri, const double* tri, double* planes) {
    for (int t = 0; t < ntri; t++) {
        const double* v = tri + 9 * t;
        double* pl = planes + 16 * t;
        const double u[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};
        const double w[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
        double n[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
        const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int k = 0; k < 16; k++) pl[k] = (k % 4 == 3) ? 1.0 : 0.0;
        if (!(nn > 0.0)) continue;
        for (int k = 0; k < 3; k++) n[k] /= nn;
        pl[0] = n[0]; pl[1] = n[1]; pl[2] = n[2];
        pl[3] = n[0] * v[0] + n[1] * v[1] + n[2] * v[2];
        for (int k = 0; k < 3; k++) {
            const double* p0 = v + 3 * k;
            const double* p1 = v + 3 * ((k + 1) % 3);
            const double g[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
            double e[3] = {n[1] * g[2] - n[2] * g[1], n[2] * g[0] - n[0] * g[2], n[0] * g[1] - n[1] * g[0]};
            const double ee = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
            if (!(ee > 0.0)) continue;
            double* q = pl + 4 + 4 * k;
            for (int c = 0; c < 3; c++) q[c] = e[c] / ee;
            q[3] = q[0] * p0[0] + q[1] * p0[1] + q[2] * p0[2];
        }
    }
}

// Face normals of the triangle soup (igl::per_face_normals, src/PolygonMesh.cpp:98):
// normalised (v1 - v0) x (v2 - v0).
void hostTriNormals(int ntri, const double* tri, double* nrm) {
    for (int t = 0; t < ntri; t++) {
        const double* v = tri + 9 * t;
        double e1[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};
        double e2[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
        double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        double l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        for (int k = 0; k < 3; k++) nrm[3 * t + k] = (l > 0) ? c[k] / l : 0.0;
    }
}

// ------------------------------------------------------------------ triangle BVH
namespace {
struct BvhBuild {
    const double* tri;
    const double* origin;
    std::vector<float> cen;   // centroid (FP32, relative), 3 per triangle
    std::vector<float>& lo4;
    std::vector<float>& hi4;
    std::vector<int>& order;
    float vlo(int t, int k) const {   // smallest FP32 vertex coordinate, widened down
        double m = std::min(tri[9 * t + k], std::min(tri[9 * t + 3 + k], tri[9 * t + 6 + k])) - origin[k];
        return std::nextafter((float)m, -3.0e38f);
    }
    float vhi(int t, int k) const {
        double m = std::max(tri[9 * t + k], std::max(tri[9 * t + 3 + k], tri[9 * t + 6 + k])) - origin[k];
        return std::nextafter((float)m, 3.0e38f);
    }
    int build(int first, int count) {
        int node = (int)(lo4.size() / 4);
        lo4.resize(lo4.size() + 4);
        hi4.resize(hi4.size() + 4);
        float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        float clo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, chi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        for (int q = first; q < first + count; q++) {
            int t = order[q];
            for (int k = 0; k < 3; k++) {
                lo[k] = std::min(lo[k], vlo(t, k));
                hi[k] = std::max(hi[k], vhi(t, k));
                clo[k] = std::min(clo[k], cen[3 * t + k]);
                chi[k] = std::max(chi[k], cen[3 * t + k]);
            }
        }
        for (int k = 0; k < 3; k++) { lo4[4 * node + k] = lo[k]; hi4[4 * node + k] = hi[k]; }
        if (count <= 4) {
            int leaf[2] = {-(first + 1), count};
            std::memcpy(&lo4[4 * node + 3], &leaf[0], 4);
            std::memcpy(&hi4[4 * node + 3], &leaf[1], 4);
            return node;
        }
        int ax = 0;
        for (int k = 1; k < 3; k++)
            if (chi[k] - clo[k] > chi[ax] - clo[ax]) ax = k;
        int half = count / 2;
        std::nth_element(order.begin() + first, order.begin() + first + half, order.begin() + first + count,
                         [&](int a, int b) {
                             float ca = cen[3 * a + ax], cb = cen[3 * b + ax];
                             return ca < cb || (ca == cb && a < b);
                         });
        int l = build(first, half);
        int r = build(first + half, count - half);
        std::memcpy(&lo4[4 * node + 3], &l, 4);
        std::memcpy(&hi4[4 * node + 3], &r, 4);
        return node;
    }
};
}  // namespace

void hostBuildBvh(int ntri, const double* tri, const double* origin, std::vector<float>& lo4,
                  std::vector<float>& hi4, std::vector<int>& order) {
    lo4.clear(); hi4.clear();
    order.resize(ntri);
    for (int t = 0; t < ntri; t++) order[t] = t;
    BvhBuild b{tri, origin, std::vector<float>(3 * (size_t)ntri), lo4, hi4, order};
    for (int t = 0; t < ntri; t++)
        for (int k = 0; k < 3; k++)
            b.cen[3 * t + k] = (float)((tri[9 * t + k] + tri[9 * t + 3 + k] + tri[9 * t + 6 + k]) / 3.0 - origin[k]);
    if (ntri > 0) b.build(0, ntri);
}
