// mps_ops.cu — the per-particle operators of the PolyMPS step on sm_103a.
//
// One thread per particle i.  Sweeps at the post-prediction positions walk the ELL
// neighbour row of i (built once per position epoch through the stale bucket list, in
// the reference's scan order); the start-of-step viscosity and the post-correction
// shifting/dummy sweeps, which see their positions once, walk the 27 buckets directly.
// Every sweep applies the reference's own radius and mirror-side tests to each entry,
// with the distance comparisons evaluated in exact FP64 (see mps_common.cuh).
#include "mps_df.cuh"
#include "mps_internal.h"

#define BLK 128

// ------------------------------------------------------------------ viscosity
// MpsViscosity::calcViscosity, src/MpsViscosity.cpp:20-100 (Newtonian: MEU and RHO are
// uniform, src/MpsInputOutput.cpp:833-838, so the harmonic mean is hoisted).  Staged scan
// at the start-of-step positions; FP32 prefilter, exact FP64 radius/side tests.
struct OpViscosity {
    // the kinematic factors of a wall and of a fluid neighbour, (2 mu)/rho and
    // (2 mu mu / (mu + mu))/rho (src/MpsViscosity.cpp:55-62), are the same for every pair of
    // the run: formed once per particle with the reference's operations (same bits)
    struct State { dvec4 vi; SideCtx sc; double ax, ay, az, neuWall, neuFluid; };
    __device__ float hi(const Dev& d) const { return d.bandHiL; }
    __device__ bool active(const Dev&, const State&) const { return true; }
    __device__ void begin(const Dev& d, int i, State& st) const {
        st.vi = d.vel[i];
        st.sc = sideCtx(d, i, d.pos[i]);
        st.ax = st.ay = st.az = 0.0;
        const double mu = d.P.KNM_VS1 * d.P.DNS_FL1, rho = d.P.DNS_FL1;
        st.neuWall = (2.0 * mu) / rho;
        st.neuFluid = (2.0 * mu * mu / (mu + mu)) / rho;
    }
    __device__ void visit(const Dev& d, int i, State& st, int j, dvec4 pj, PairG q) const {
        const MpsParams& P = d.P;
        if (!(q.d2 < P.reL2) || !sideOK(st.sc, pj, q.d2)) return;
        const double neu = (d.type[j] == P.wall) ? st.neuWall : st.neuFluid;
        double wL, wd;
        weightR(q.d2, P.reL, P.weightType, wL, wd);
        dvec4 vj = d.vel[j];
        st.ax += (vj.x - st.vi.x) * wL * neu;
        st.ay += (vj.y - st.vi.y) * wL * neu;
        st.az += (vj.z - st.vi.z) * wL * neu;
    }
    __device__ void end(const Dev& d, int i, State& st) const {
        double c = d.P.coeffViscMultiphase;
        d.acc[i] = make_dvec4(c * st.ax, c * st.ay, c * st.az, 0.0);
    }
};
void launchViscosity(const Dev& d, cudaStream_t s) {
    launchScan(d, OpViscosity(), s);
}
// The same sweep over the start-of-step skin list (built just before from the same FP32
// copies): its entries within the reL band, in scan order, are exactly the candidates the
// 27-bucket scan passes to the exact FP64 test, so the sums are the scan's bit for bit.
// A row that overflowed the list capacity (count K + 1) scans the buckets.
__global__ void __launch_bounds__(128) k_visc_list(Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const OpViscosity op;
    OpViscosity::State st;
    op.begin(d, i, st);
    const dvec4 pi = d.pos[i];
    const float4 fi = d.posf[i];
    const float hi = op.hi(d);
    const int c = d.nbrCount[i];
    if (c <= d.K) {
        const int* row = d.nbr + i;
        for (int k = 0; k < c; k++) {
            const int j = ldStream(row + (size_t)k * d.N0);
            const float4 fj = d.posf[j];
            const float ex = fj.x - fi.x, ey = fj.y - fi.y, ez = fj.z - fi.z;
            if (ex * ex + ey * ey + ez * ez > hi) continue;
            const dvec4 pj = d.pos[j];
            op.visit(d, i, st, j, pj, pairOf(pj, pi));
        }
    } else {
        forCellsNear(d, pi, fi, hi, [&](int j, dvec4 pj, PairG q) {
            if (j != i) op.visit(d, i, st, j, pj, q);
        });
    }
    op.end(d, i, st);
}
void launchViscosityList(const Dev& d, cudaStream_t s) {
    k_visc_list<<<gridFor(d.N0, 128), 128, 0, s>>>(d);
}

// FP64 list of the current positions filtered from the skin list: the set, order and
// (WEIGHTS) per-entry weights of k_build_nbr (candidates within the FP32 band, exact FP64
// test d^2 < reMax^2).  A particle whose scan window changed or whose skin row overflowed,
// or every particle once the skin list went stale, scans the 27 buckets as k_build_nbr does.
template <bool WEIGHTS>
__global__ void __launch_bounds__(128) k_filter_nbr(Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    const dvec4 pi = d.pos[i];
    const float4 fi = d.posf[i];
    const size_t N0 = d.N0;
    int cnt = 0;
    auto keep = [&](int j, PairG q) {
        if (!(q.d2 < d.reMax2)) return;
        if (cnt < d.K) {
            const size_t e = (size_t)cnt * N0 + i;
            d.nbr[e] = j;
            if (WEIGHTS) {
                double w, wd;
                weightR(q.d2, P.reS, P.weightType, w, wd);
                d.cw[e] = w;
                d.cwd[e] = wd;
                if (d.cwL) { double wl, wdl; weightR(q.d2, P.reL, P.weightType, wl, wdl); d.cwL[e] = wl; }
            }
        }
        cnt++;
    };
    const int c = d.skinCnt[i];
    if (!*(volatile int*)d.skinFlag && c <= d.K && d.skinCell[i] == cellKeyOf(d, pi, fi)) {
        for (int k = 0; k < c; k++) {
            const int j = ldStream(d.skinNbr + (size_t)k * N0 + i);
            const float4 fj = d.posf[j];
            const float ex = fj.x - fi.x, ey = fj.y - fi.y, ez = fj.z - fi.z;
            if (ex * ex + ey * ey + ez * ez > d.bandHi) continue;
            const dvec4 pj = d.pos[j];
            keep(j, pairOf(pj, pi));
        }
    } else {
        forCellsNear(d, pi, fi, d.bandHi, [&](int j, dvec4, PairG q) {
            if (j != i) keep(j, q);
        });
    }
    if (cnt > d.K) { setErr(d, MPSE_CAPACITY); cnt = d.K; }
    d.nbrCount[i] = cnt;
    warpCount(d.counters, (unsigned)cnt);
}
void launchNeighborFilter(const Dev& d, cudaStream_t s, bool weights) {
    cudaMemsetAsync(d.counters, 0, sizeof(unsigned long long), s);
    launchPosf(d, s);
    launchSkinCheck(d, s);
    if (weights) k_filter_nbr<true><<<gridFor(d.N0, 128), 128, 0, s>>>(d);
    else k_filter_nbr<false><<<gridFor(d.N0, 128), 128, 0, s>>>(d);
}

// MpsParticle::addGravity, src/MpsParticle.cpp:111-130
__global__ void k_add_gravity(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    dvec4 a = d.acc[i];
    a.x += d.P.gravity[0]; a.y += d.P.gravity[1]; a.z += d.P.gravity[2];
    d.acc[i] = a;
    d.accStar[i] = a;
}
void launchAddGravity(const Dev& d, cudaStream_t s) { k_add_gravity<<<gridFor(d.N0, 256), 256, 0, s>>>(d); }

// MpsParticleVelPos::predictionVelocityPosition, src/MpsParticleVelPos.cpp:20-50
__global__ void k_predict(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    if (d.type[i] == P.fluid) {
        dvec4 v = d.vel[i], a = d.acc[i], x = d.pos[i];
        v.x += a.x * P.timeStep; v.y += a.y * P.timeStep; v.z += a.z * P.timeStep;
        x.x += v.x * P.timeStep; x.y += v.y * P.timeStep; x.z += v.z * P.timeStep;
        d.vel[i] = v; d.pos[i] = x;
    }
    dvec4 z = make_dvec4(0, 0, 0, 0);
    d.acc[i] = z; d.dvel[i] = z; d.npcd[i] = z;
    d.nNeighWall[i] = 0;
    d.nearWall[i] = 0;
    double big = 10e8 * P.partDist;
    d.riw2[i] = big;
    if (P.wallType == 1) d.mirror[i] = make_dvec4(big, big, big, 0.0);
}
void launchPredict(const Dev& d, cudaStream_t s) { k_predict<<<gridFor(d.N0, 256), 256, 0, s>>>(d); }

// ------------------------------------------------------------------ out of domain
// MpsParticle::checkParticleOutDomain, src/MpsParticle.cpp:270-396.  A parallel pass flags
// fluid particles outside [min + bucket, max - bucket] by reference index; when any is
// flagged, a single thread replays the reference's serial swap-with-last loop on reference
// indices: the data of the last live index is copied onto the removed one (the arrays the
// reference copies) and the last index becomes a ghost, exactly as in the reference, on
// the storage slots of those indices.  Live storage is then kept contiguous: the ghost's
// slot trades places with the last live slot (all arrays, the index maps and the two
// entries of the step's bucket list, so the list keeps pointing at the same data).
__device__ __forceinline__ bool outside(const Dev& d, dvec4 p) {
    return p.x > d.oodHi[0] || p.x < d.oodLo[0] || p.y > d.oodHi[1] || p.y < d.oodLo[1] ||
           (d.dz3 && (p.z > d.oodHi[2] || p.z < d.oodLo[2]));
}
// flags (by reference index) are zero between calls: only flagged particles write theirs,
// and the serial pass clears what it read
__global__ void k_out_flag(Dev d, int* flags, int* counter) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    int n = liveN(d);
    if (s >= n) return;
    if (d.type[s] == d.P.fluid && outside(d, d.pos[s])) {
        flags[d.orig[s]] = 1;
        atomicAdd(counter, 1);
    }
}
template <class T> __device__ __forceinline__ void mv(T* a, int i, int L) { a[i] = a[L]; }
template <class T> __device__ __forceinline__ void sw(T* a, int i, int j) { T t = a[i]; a[i] = a[j]; a[j] = t; }
// every per-particle array that lives across operators: a pure relocation of two slots
__device__ void swapSlots(const Dev& d, int a, int b) {
    for (dvec4* v : {d.pos, d.vel, d.acc, d.accStar, d.mirror, d.wallPos, d.polyNormal, d.normal, d.npcd, d.gradC,
                     d.forceWall, d.c1, d.c2, d.c3, d.dvel, d.shift})
        sw(v, a, b);
    for (double* v : {d.press, d.pressPPE, d.pressPPEprev, d.pressPPEprev2, d.pndi, d.pndki, d.pndski, d.pndSmall, d.npcd2, d.conc,
                      d.velDiv, d.diffTerm, d.pndWall, d.riw2, d.devDot, d.source, d.aux1, d.aux2})
        sw(v, a, b);
    for (int* v : {d.type, d.bc, d.numNeigh, d.nNeighWall, d.nearWall, d.cellOf}) sw(v, a, b);
    sw(d.posf, a, b);
    sw(d.posLo, a, b);
    int ra = d.orig[a], rb = d.orig[b];
    d.orig[a] = rb; d.orig[b] = ra;
    d.slotOf[ra] = b; d.slotOf[rb] = a;
    int pa = d.cellPos[a], pb = d.cellPos[b];
    if (pa >= 0) d.cellSorted[pa] = b;
    if (pb >= 0) d.cellSorted[pb] = a;
    d.cellPos[a] = pb; d.cellPos[b] = pa;
}
__global__ void k_out_serial(Dev d, int* flags, int* counter) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (*counter == 0) return;
    const MpsParams& P = d.P;
    const int oldN = *d.nLive;
    int newN = oldN;
    int removed = 0;
    for (int r = 0; r < newN; r++) {
        if (!flags[r]) continue;
        const int L = newN - 1;
        const int i = d.slotOf[r], l = d.slotOf[L];
        if (i != l) {
            mv(d.type, i, l); mv(d.bc, i, l); mv(d.numNeigh, i, l); mv(d.press, i, l); mv(d.pndi, i, l);
            mv(d.pndki, i, l); mv(d.pndski, i, l); mv(d.pndSmall, i, l); mv(d.npcd2, i, l); mv(d.conc, i, l);
            mv(d.velDiv, i, l); mv(d.diffTerm, i, l); mv(d.nearWall, i, l); mv(d.nNeighWall, i, l);
            mv(d.pndWall, i, l); mv(d.devDot, i, l); mv(d.riw2, i, l);
            if (P.mpsType == 2 || P.mpsType == 3) { mv(d.pressPPE, i, l); mv(d.source, i, l); mv(d.pressPPEprev, i, l); mv(d.pressPPEprev2, i, l); }
            mv(d.acc, i, l); mv(d.accStar, i, l); mv(d.pos, i, l); mv(d.vel, i, l); mv(d.npcd, i, l);
            mv(d.gradC, i, l); mv(d.c1, i, l); mv(d.c2, i, l); mv(d.c3, i, l); mv(d.dvel, i, l);
            mv(d.wallPos, i, l); mv(d.mirror, i, l); mv(d.polyNormal, i, l); mv(d.forceWall, i, l);
        }
        d.type[l] = P.ghost; d.bc[l] = P.other; d.nearWall[l] = 0; d.riw2[l] = 10e8 * P.partDist;
        d.vel[l] = make_dvec4(0, 0, 0, 0);
        d.press[l] = 0.0;
        d.pos[l] = make_dvec4(P.domainMax[0] - P.partDist, P.domainMax[1] - P.partDist,
                              (P.dim == 2) ? 0.0 : P.domainMax[2] - P.partDist, 0.0);
        if (l != newN - 1) swapSlots(d, l, newN - 1);
        newN--;
        removed++;
    }
    *d.nLive = newN;
    *counter = removed;
    if (removed) d.skinFlag[0] = 1;   // indices moved: the start-of-step list is stale
    for (int r = 0; r < oldN; r++) flags[r] = 0;
}
void launchOutOfDomain(const Dev& d, int* flags, int* counter, cudaStream_t s) {
    cudaMemsetAsync(counter, 0, sizeof(int), s);
    k_out_flag<<<gridFor(d.N0, 256), 256, 0, s>>>(d, flags, counter);
    k_out_serial<<<1, 32, 0, s>>>(d, flags, counter);
}

// ------------------------------------------------------------------ collision
// MpsParticleCollision::checkParticleCollisions (PC), src/MpsParticleCollision.cpp:22-119:
// velocity corrections computed from the pre-collision velocities, then applied.
__global__ void __launch_bounds__(BLK) k_collision(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    dvec4 dv = make_dvec4(0, 0, 0, 0);
    if (d.type[i] == P.fluid) {
        double mi = P.DNS_FL1;  // PTYPE == 1 for every Newtonian particle
        dvec4 pi = d.pos[i], vi = d.vel[i];
        const float4 fi = d.posf[i];
        const SideCtx sc = d.mirrorFar ? SideCtx{} : sideCtx(d, i, pi);   // {}: no side test
        forNbrsPosf(d, i, [&](int j, float4 fj) {
            // FP32 prefilter (the list's FP32 copies): most entries lie beyond the collision
            // distance; the exact FP64 test decides the others
            const float ex = fj.x - fi.x, ey = fj.y - fi.y, ez = fj.z - fi.z;
            if (ex * ex + ey * ey + ez * ez > d.bandHiColl) return;
            dvec4 pj = d.pos[j];
            PairG q = pairOf(pj, pi);
            if (q.d2 < P.distCollisionLimit2 && sideOK(sc, pj, q.d2)) {
                dvec4 vj = d.vel[j];
                double fDT = (vi.x - vj.x) * q.v0 + (vi.y - vj.y) * q.v1 + (vi.z - vj.z) * q.v2;
                if (fDT > 0.0) {
                    bool jf = d.type[j] == P.fluid;
                    double mj = jf ? P.DNS_FL1 : P.densityWall;
                    fDT *= P.restitutionCollision * mj / (mi + mj) / q.d2;
                    double f = jf ? 1.0 : 2.0;
                    dv.x -= f * q.v0 * fDT; dv.y -= f * q.v1 * fDT; dv.z -= f * q.v2 * fDT;
                }
            }
        });
    }
    d.dvel[i] = dv;
}
__global__ void k_collision_apply(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    if (d.type[i] == d.P.fluid) {
        dvec4 v = d.vel[i], dv = d.dvel[i];
        v.x += dv.x; v.y += dv.y; v.z += dv.z;
        d.vel[i] = v;
    }
    d.dvel[i] = make_dvec4(0, 0, 0, 0);
}
void launchCollisionApply(const Dev& d, cudaStream_t s) {
    k_collision_apply<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
}
void launchCollision(const Dev& d, cudaStream_t s) {
    k_collision<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
    launchCollisionApply(d, s);
}

// MpsParticleCollision::checkDynamicParticleCollisions (DPC, collision type 1),
// src/MpsParticleCollision.cpp:120-292: list entries closer than l0 off the mirror side;
// approaching pairs exchange momentum with kappa (1 below l0/2, else chi =
// sqrt(W_ij / W(l0/2)), W = (1 - r/l0)^4 (4 r/l0 + 1)), separating pairs get the dynamic
// background-pressure repulsion; then v += dv, x += dv dt for fluid particles.
__global__ void __launch_bounds__(BLK) k_collision_dpc(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    dvec4 dv = make_dvec4(0, 0, 0, 0);
    const MpsParams& P = d.P;
    if (d.type[i] == P.fluid) {
        const double mi = P.DNS_FL1;   // PTYPE == 1 for every Newtonian particle
        const double Wij5 = 0.5 * 0.5 * 0.5 * 0.5 * 3.0;
        const double gMod = sqrt(P.gravity[0] * P.gravity[0] + P.gravity[1] * P.gravity[1] + P.gravity[2] * P.gravity[2]);
        const double l02 = P.partDist * P.partDist;
        const double pmax = 2.0 / 3.0 * P.DNS_FL1 * gMod * 0.2, pmin = P.DNS_FL1 * gMod * P.partDist;
        const dvec4 pi = d.pos[i], vi = d.vel[i];
        const double pri = d.press[i];
        SideCtx sc = sideCtx(d, i, pi);
        forNbrs(d, i, [&](int j) {
            dvec4 pj = d.pos[j];
            PairG q = pairOf(pj, pi);
            if (!(q.d2 < l02 && sideOK(sc, pj, q.d2))) return;
            const bool jf = d.type[j] == P.fluid;
            const double mj = jf ? P.DNS_FL1 : P.densityWall;
            const double dst = sqrt(q.d2);
            double Wij = 0.0;
            if (dst > P.epsilonZero) {
                double w1 = 1.0 - dst * P.invPartDist;
                double w2 = 4.0 * dst * P.invPartDist + 1.0;
                Wij = w1 * w1 * w1 * w1 * w2;
            }
            const double chi = sqrt(Wij / Wij5);
            const double kappa = (dst < 0.5 * P.partDist) ? 1.0 : chi;
            const dvec4 vj = d.vel[j];
            double fDT = (vi.x - vj.x) * q.v0 + (vi.y - vj.y) * q.v1 + (vi.z - vj.z) * q.v2;
            const double f2 = jf ? 1.0 : 2.0;
            double k;
            if (fDT > 0.0) {
                k = fDT * kappa * 2.0 * mj / (mi + mj) / q.d2;
            } else {
                double ptil = fmax(fmin(P.lambdaCollision * fabs(pri + d.press[j]), P.lambdaCollision * pmax), pmin);
                double pb = ptil * chi;
                k = P.timeStep / mi * chi * pb / q.d2;
            }
            dv.x -= f2 * q.v0 * k; dv.y -= f2 * q.v1 * k; dv.z -= f2 * q.v2 * k;
        });
    }
    d.dvel[i] = dv;
}
__global__ void k_collision_dpc_apply(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    if (d.type[i] == d.P.fluid) {
        dvec4 v = d.vel[i], x = d.pos[i], dv = d.dvel[i];
        const double dt = d.P.timeStep;
        v.x += dv.x; v.y += dv.y; v.z += dv.z;
        x.x += dv.x * dt; x.y += dv.y * dt; x.z += dv.z * dt;
        d.vel[i] = v;
        d.pos[i] = x;
    }
    d.dvel[i] = make_dvec4(0, 0, 0, 0);
}
void launchCollisionDPC(const Dev& d, cudaStream_t s) {
    k_collision_dpc<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
    k_collision_dpc_apply<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
}

// ------------------------------------------------------------------ wall NPCD
// Wall-only sweeps run over the compacted list of fluid particles near the wall.
__device__ __forceinline__ int nearIndex(const Dev& d) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    return (t < *d.nearCount) ? d.nearList[t] : -1;
}
// MpsPndNeigh::calcWallNPCD, src/MpsPndNeigh.cpp:105-195
__global__ void __launch_bounds__(BLK) k_wall_npcd(Dev d) {
    int i = nearIndex(d);
    if (i < 0) return;
    const MpsParams& P = d.P;
    dvec4 pi = d.pos[i], mi = d.mirror[i];
    ReflG r = makeRefl(pi, mi, P.epsilonZero, true);
    double dx = 0, dy = 0, dz = 0;
    forNbrs(d, i, [&](int j) {
        dvec4 pj = d.pos[j];
        PairG q = pairOf(pj, pi);
        if (q.d2 < P.reS2) {
            PairM m = pairMirror(pj, mi);
            if (m.dm2 < P.reS2 && q.d2 < m.dm2) {
                double wS = wfun(sqrt(m.dm2), P.reS, P.weightType);
                dx += m.m0 * wS; dy += m.m1 * wS; dz += m.m2 * wS;
            }
        }
    });
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
void launchWallNpcd(const Dev& d, cudaStream_t s) {
    if (d.P.wallType != 1) return;
    k_wall_npcd<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
}

// ------------------------------------------------------------------ velocity divergence
// MpsPressure::calcVelDivergence, src/MpsPressure.cpp:479-557: fluid particles over the reS
// entries off the mirror side; PND-weighted, or through the correction matrix.
__global__ void __launch_bounds__(BLK) k_vel_div(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    double div = 0.0;
    if (d.type[i] == P.fluid) {
        const double ni = d.pndi[i];
        const dvec4 pi = d.pos[i], vi = d.vel[i];
        const dvec4 c1 = d.c1[i], c2 = d.c2[i], c3 = d.c3[i];
        const double f = P.dim / P.pndSmallZero;
        forMask(d, i, d.maskS[i], [&](int j, size_t) {
            dvec4 pj = d.pos[j], vj = d.vel[j];
            PairG q = pairOf(pj, pi);
            double vx = vj.x - vi.x, vy = vj.y - vi.y, vz = vj.z - vi.z;
            double wS = wfun(sqrt(q.d2), P.reS, P.weightType);
            if (!P.gradientCorrection) {
                if (ni > P.epsilonZero) div += f * (d.pndi[j] / ni) * (vx * q.v0 + vy * q.v1 + vz * q.v2) * wS / q.d2;
            } else {
                double a0 = q.v0 * c1.x + q.v1 * c1.y + q.v2 * c1.z;
                double a1 = q.v0 * c2.x + q.v1 * c2.y + q.v2 * c2.z;
                double a2 = q.v0 * c3.x + q.v1 * c3.y + q.v2 * c3.z;
                div += f * (vx * a0 + vy * a1 + vz * a2) * wS / q.d2;
            }
        });
    }
    d.velDiv[i] = div;
}
// calcWallSlipVelDivergence / calcWallNoSlipVelDivergence, src/MpsPressure.cpp:560-790
// (rigid mesh: wall velocity 0): mirror velocity R v_i (slip) or -v_i (no-slip), the no-slip
// pair vectors reflected by R, over the near-wall fluid with n_i > eps.
__global__ void __launch_bounds__(BLK) k_wall_vel_div(Dev d) {
    int i = nearIndex(d);
    if (i < 0) return;
    const MpsParams& P = d.P;
    const double ni = d.pndi[i];
    if (!(ni > P.epsilonZero)) return;
    const bool noslip = P.slipCondition == 0;
    const dvec4 pi = d.pos[i], mi = d.mirror[i], vi = d.vel[i];
    ReflG r = makeRefl(pi, mi, P.epsilonZero, false);
    double vm[3];
    if (noslip) { vm[0] = -vi.x; vm[1] = -vi.y; vm[2] = -vi.z; }
    else {
        vm[0] = r.R[0] * vi.x + r.R[1] * vi.y + r.R[2] * vi.z;
        vm[1] = r.R[3] * vi.x + r.R[4] * vi.y + r.R[5] * vi.z;
        vm[2] = r.R[6] * vi.x + r.R[7] * vi.y + r.R[8] * vi.z;
    }
    const double f = P.dim / P.pndSmallZero;
    double div = 0.0;
    auto term = [&](double vx, double vy, double vz, double m0, double m1, double m2, double dm2, double pj) {
        double wS = wfun(sqrt(dm2), P.reS, P.weightType);
        if (noslip) {
            vx = -vx; vy = -vy; vz = -vz;
            double a0 = r.R[0] * m0 + r.R[1] * m1 + r.R[2] * m2;
            double a1 = r.R[3] * m0 + r.R[4] * m1 + r.R[5] * m2;
            double a2 = r.R[6] * m0 + r.R[7] * m1 + r.R[8] * m2;
            m0 = a0; m1 = a1; m2 = a2;
        }
        div += f * (pj / ni) * (vx * m0 + vy * m1 + vz * m2) * wS / dm2;
    };
    forNbrs(d, i, [&](int j) {
        dvec4 pj = d.pos[j];
        PairG q = pairOf(pj, pi);
        if (q.d2 < P.reS2) {
            PairM m = pairMirror(pj, mi);
            if (m.dm2 < P.reS2 && q.d2 < m.dm2) {
                dvec4 vj = d.vel[j];
                term(vj.x - vm[0], vj.y - vm[1], vj.z - vm[2], m.m0, m.m1, m.m2, m.dm2, d.pndi[j]);
            }
        }
    });
    PairM s = pairMirror(pi, mi);
    if (s.dm2 < P.reS2) term(vi.x - vm[0], vi.y - vm[1], vi.z - vm[2], s.m0, s.m1, s.m2, s.dm2, ni);
    d.velDiv[i] += div;
}
void launchVelDivergence(const Dev& d, cudaStream_t s) {
    k_vel_div<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
    if (d.P.wallType == 1) k_wall_vel_div<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
}

// ------------------------------------------------------------------ correction matrix
// MpsVectorMatrix::correctionMatrix + inverseMatrix (Gauss-Jordan without pivoting,
// identity when det <= eps or numNeigh < 4), src/MpsVectorMatrix.cpp:20-166
__global__ void __launch_bounds__(BLK) k_corr_matrix(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    dvec4 pi = d.pos[i];
    double m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    forMask(d, i, d.maskS[i], [&](int j, size_t e) {
        dvec4 pj = d.pos[j];
        double v[3] = {pj.x - pi.x, pj.y - pi.y, pj.z - pi.z};
        double wd = d.cwd[e];   // w / r^2
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) m[a * 3 + b] += wd * v[a] * v[b];
    });
#pragma unroll
    for (int k = 0; k < 9; k++) m[k] *= -P.coeffPressGrad;
    invert3(m, (int)P.dim, P.epsilonZero);
    if (d.numNeigh[i] < 4) {
#pragma unroll
        for (int k = 0; k < 9; k++) m[k] = (k % 4 == 0) ? 1.0 : 0.0;
    }
    d.c1[i] = make_dvec4(m[0], m[1], m[2], 0.0);
    d.c2[i] = make_dvec4(m[3], m[4], m[5], 0.0);
    d.c3[i] = make_dvec4(m[6], m[7], m[8], 0.0);
}
void launchCorrectionMatrix(const Dev& d, cudaStream_t s) { k_corr_matrix<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d); }

// ------------------------------------------------------------------ PND / NPCD
// MpsPndNeigh::calcPndnNeighNPCD, src/MpsPndNeigh.cpp:199-331 (init == 0), and
// setInitialPndNumberOfNeighNPCD, src/MpsPndNeigh.cpp:21-101 (init == 1)
template <int INIT>
__global__ void __launch_bounds__(BLK) k_pnd_npcd(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    dvec4 pi = d.pos[i];
    double ni = 0.0, wSum = 0.0;
    const Mask mL = d.maskL[i];
    int nn = (INIT ? 0 : d.nNeighWall[i]) + maskCount(mL);
    dvec4 np = INIT ? make_dvec4(0, 0, 0, 0) : d.npcd[i];
    forMask(d, i, mL & d.maskS[i], [&](int j, size_t e) {
        dvec4 pj = d.pos[j];
        double wS = d.cw[e];
        ni += wS;
        np.x += (pj.x - pi.x) * wS; np.y += (pj.y - pi.y) * wS; np.z += (pj.z - pi.z) * wS;
        wSum += wS;
    });
    double pndSmall;
    if (INIT) {
        double pn = d.pndi[i] + ni;     // pndi accumulates onto its initial value
        pn += d.pndWall[i];
        if (d.type[i] == P.wall) pn = P.pndSmallZero;
        d.pndi[i] = pn;
        d.pndki[i] = pn;
        pndSmall = pn;
        nn += d.nNeighWall[i];
    } else {
        if (P.pndType == 0 || P.pndType == 1) {
            d.pndki[i] = d.pndi[i];
            d.pndi[i] = ni + d.pndWall[i];
        }
        pndSmall = ni + d.pndWall[i];
    }
    d.pndSmall[i] = pndSmall;
    d.numNeigh[i] = nn;
    if (wSum > P.epsilonZero) { np.x /= pndSmall; np.y /= pndSmall; np.z /= pndSmall; }
    d.npcd[i] = np;
    d.npcd2[i] = np.x * np.x + np.y * np.y + np.z * np.z;
    dvec4 nw = d.polyNormal[i];
    d.devDot[i] = (np.x * nw.x + np.y * nw.y + np.z * nw.z < 0.0) ? 1.0 : -1.0;
}
void launchPndNeighNpcd(const Dev& d, cudaStream_t s) { k_pnd_npcd<0><<<gridFor(d.N0, BLK), BLK, 0, s>>>(d); }

// ------------------------------------------------------------------ diffusive PND (pnd type 2)
// MpsPndNeigh::calcPndDiffusiveTerm, src/MpsPndNeigh.cpp:334-489
__global__ void __launch_bounds__(BLK) k_pnd_diffusive(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    double ni = d.pndi[i];
    if (ni < P.epsilonZero) return;
    dvec4 pi = d.pos[i], vi = d.vel[i];
    dvec4 C1 = d.c1[i], C2 = d.c2[i], C3 = d.c3[i];
    double Pi = d.press[i];
    double rho = P.DNS_FL1;
    bool fi = d.type[i] == P.fluid;
    double Di = 0.0, DivV = 0.0;
    double cdiv = P.dim / P.pndSmallZero;
    double invNi = 1.0 / ni;
    const Mask mL = d.maskL[i], mS = d.maskS[i] & mL;
    const double* wLc = d.cwL ? d.cwL : d.cw;
    forMaskK(d, i, mL, [&](int j, size_t e, int k) {
        dvec4 pj = d.pos[j];
        double v0 = pj.x - pi.x, v1 = pj.y - pi.y, v2 = pj.z - pi.z;
        double wL = wLc[e];
        if (fi && d.type[j] == P.fluid) {
            double pgh = -2.0 * (rho * rho / (rho + rho)) * (P.gravity[0] * v0 + P.gravity[1] * v1 + P.gravity[2] * v2);
            Di += P.timeStep / rho * P.coeffViscMultiphase * (d.press[j] - Pi - pgh) * wL;
        }
        if (maskHas(mS, k)) {
            dvec4 vj = d.vel[j];
            double vx = vj.x - vi.x, vy = vj.y - vi.y, vz = vj.z - vi.z;
            double wd = d.cwd[e];   // wS / r^2
            if (!P.gradientCorrection) {
                DivV += cdiv * (d.pndi[j] * invNi) * (vx * v0 + vy * v1 + vz * v2) * wd;
            } else {
                double a0 = v0 * C1.x + v1 * C1.y + v2 * C1.z;
                double a1 = v0 * C2.x + v1 * C2.y + v2 * C2.z;
                double a2 = v0 * C3.x + v1 * C3.y + v2 * C3.z;
                DivV += cdiv * (vx * a0 + vy * a1 + vz * a2) * wd;
            }
        }
    });
    d.aux1[i] = d.pndi[i] * (1.0 + P.timeStep * (-DivV + Di * 1.0));
    d.velDiv[i] = DivV;
    d.diffTerm[i] = Di;
}

// MpsPndNeigh::calcWallSlipPndDiffusiveTerm / calcWallNoSlipPndDiffusiveTerm,
// src/MpsPndNeigh.cpp:492-744 (fixed wall: wall velocity zero)
__global__ void __launch_bounds__(BLK) k_wall_pnd_diffusive(Dev d) {
    int i = nearIndex(d);
    if (i < 0) return;
    const MpsParams& P = d.P;
    double ni = d.pndi[i];
    if (!(ni > P.epsilonZero)) return;
    bool noslip = P.slipCondition == 0;
    dvec4 pi = d.pos[i], vi = d.vel[i], mi = d.mirror[i];
    ReflG r = makeRefl(pi, mi, P.epsilonZero, false);
    double vm[3];
    if (noslip) { vm[0] = -vi.x; vm[1] = -vi.y; vm[2] = -vi.z; }
    else {
        vm[0] = r.R[0] * vi.x + r.R[1] * vi.y + r.R[2] * vi.z;
        vm[1] = r.R[3] * vi.x + r.R[4] * vi.y + r.R[5] * vi.z;
        vm[2] = r.R[6] * vi.x + r.R[7] * vi.y + r.R[8] * vi.z;
    }
    double cdiv = P.dim / P.pndSmallZero;
    double DivV = 0.0;
    auto term = [&](double vx, double vy, double vz, double m0, double m1, double m2, double dm2, double pj) {
        double wS = wfun(sqrt(dm2), P.reS, P.weightType);
        if (noslip) {
            vx = -vx; vy = -vy; vz = -vz;
            double a0 = r.R[0] * m0 + r.R[1] * m1 + r.R[2] * m2;
            double a1 = r.R[3] * m0 + r.R[4] * m1 + r.R[5] * m2;
            double a2 = r.R[6] * m0 + r.R[7] * m1 + r.R[8] * m2;
            return cdiv * (pj / ni) * (vx * a0 + vy * a1 + vz * a2) * wS / dm2;
        }
        return cdiv * (pj / ni) * (vx * m0 + vy * m1 + vz * m2) * wS / dm2;
    };
    forNbrs(d, i, [&](int j) {
        dvec4 pj = d.pos[j];
        PairG q = pairOf(pj, pi);
        if (q.d2 < P.reS2) {
            PairM m = pairMirror(pj, mi);
            if (m.dm2 < P.reS2 && q.d2 < m.dm2) {
                dvec4 vj = d.vel[j];
                DivV += term(vj.x - vm[0], vj.y - vm[1], vj.z - vm[2], m.m0, m.m1, m.m2, m.dm2, d.pndi[j]);
            }
        }
    });
    PairM s = pairMirror(pi, mi);
    if (s.dm2 < P.reS2) DivV += term(vi.x - vm[0], vi.y - vm[1], vi.z - vm[2], s.m0, s.m1, s.m2, s.dm2, ni);
    d.aux1[i] += -ni * P.timeStep * DivV;
}

// MpsPndNeigh::updatePnd, src/MpsPndNeigh.cpp:747-774
__global__ void k_update_pnd(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    d.pndi[i] = d.aux1[i];
    d.aux1[i] = 0.0;
}

// MpsPndNeigh::meanPndParticlesWallDummySurface, src/MpsPndNeigh.cpp:777-852
__global__ void __launch_bounds__(BLK) k_mean_pnd_wds(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    double up = 0.0, dn = 0.0;
    if (d.type[i] == P.wall || d.bc[i] == P.surface) {
        forMask(d, i, d.maskS[i], [&](int j, size_t e) {
            double wS = d.cw[e];
            up += d.pndi[j] * wS; dn += wS;
        });
    }
    d.aux1[i] = up; d.aux2[i] = dn;
}
__global__ void k_mean_pnd_wds_apply(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    if (d.type[i] == P.wall || d.bc[i] == P.surface) {
        double a1 = d.aux1[i], a2 = d.aux2[i];
        d.pndi[i] = (a2 < P.epsilonZero) ? a1 : a1 / a2;
    }
    d.aux1[i] = 0.0; d.aux2[i] = 0.0;
}

void launchPndDiffusive(const Dev& d, cudaStream_t s) {
    k_pnd_diffusive<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
    if (d.P.wallType == 1) k_wall_pnd_diffusive<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
    k_update_pnd<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
    k_mean_pnd_wds<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
    k_mean_pnd_wds_apply<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
}

// ------------------------------------------------------------------ mean PND (pnd type 1 and init)
// MpsPndNeigh::meanWallPnd, src/MpsPndNeigh.cpp:923-994 (sets aux1/aux2)
__global__ void __launch_bounds__(BLK) k_mean_wall_pnd(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    double up = 0.0, dn = 0.0;
    if (d.nearWall[i]) {
        dvec4 pi = d.pos[i], mi = d.mirror[i];
        forNbrs(d, i, [&](int j) {
            dvec4 pj = d.pos[j];
            PairG q = pairOf(pj, pi);
            if (q.d2 < P.reS2) {
                PairM m = pairMirror(pj, mi);
                if (m.dm2 < P.reS2 && q.d2 < m.dm2) {
                    double wS = wfun(sqrt(m.dm2), P.reS, P.weightType);
                    up += d.pndi[j] * wS; dn += wS;
                }
            }
        });
        PairM s = pairMirror(pi, mi);
        if (s.dm2 < P.reS2) {
            double wS = wfun(sqrt(s.dm2), P.reS, P.weightType);
            up += d.pndi[i] * wS; dn += wS;
        }
    }
    d.aux1[i] = up; d.aux2[i] = dn;
}
// MpsPndNeigh::meanPnd, src/MpsPndNeigh.cpp:855-920 (adds onto aux1/aux2, then divides)
__global__ void __launch_bounds__(BLK) k_mean_pnd(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    double up = 0.0, dn = 0.0;
    forMask(d, i, d.maskS[i], [&](int j, size_t e) {
        double wS = d.cw[e];
        up += d.pndi[j] * wS; dn += wS;
    });
    d.aux1[i] += up; d.aux2[i] += dn;
}
__global__ void k_mean_pnd_apply(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    double a1 = d.aux1[i], a2 = d.aux2[i];
    d.pndi[i] = (d.numNeigh[i] < 1) ? a1 : a1 / a2;
    d.aux1[i] = 0.0; d.aux2[i] = 0.0;
}
// MpsPndNeigh::meanNeighFluidPnd, src/MpsPndNeigh.cpp:997-1050
__global__ void __launch_bounds__(BLK) k_mean_neigh_fluid_pnd(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    double up = 0.0, dn = 0.0;
    forMask(d, i, d.maskS[i], [&](int j, size_t e) {
        if (d.type[j] != P.fluid) return;
        double wS = d.cw[e];
        up += d.pndki[j] * wS; dn += wS;
    });
    d.pndski[i] = (dn > P.epsilonZero) ? up / dn : up;
}
void launchPndMean(const Dev& d, cudaStream_t s) {
    if (d.P.wallType == 1) k_mean_wall_pnd<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
    k_mean_pnd<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
    k_mean_pnd_apply<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
}
// step-0 sequence, src/main.cpp:158-166
void launchInitPnd(const Dev& d, cudaStream_t s) {
    k_pnd_npcd<1><<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
    launchPndMean(d, s);
    k_mean_neigh_fluid_pnd<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
}

// ------------------------------------------------------------------ boundary condition
// MpsBoundaryCondition::updateParticleBC, types 0 and 1, src/MpsBoundaryCondition.cpp:173-204
__global__ void k_update_bc(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    int bc;
    if (d.type[i] == P.dummyWall) bc = P.other;
    else {
        double ps = d.pndSmall[i];
        bc = (ps < P.betaPnd) ? P.surface : P.inner;
        if (P.freeSurfType == 0) {
            bc = (ps < P.betaPnd && d.numNeigh[i] < P.betaNeigh) ? P.surface : P.inner;
        } else if (P.freeSurfType == 1) {
            if (bc == P.surface && d.numNeigh[i] > 4 && d.npcd2[i] < P.delta2) bc = P.inner;
        }
    }
    d.bc[i] = bc;
}
void launchUpdateBC(const Dev& d, cudaStream_t s) { k_update_bc<<<gridFor(d.N0, 256), 256, 0, s>>>(d); }

// ------------------------------------------------------------------ ARC free surface
// MpsShifting::calcNormalParticles, src/MpsShifting.cpp:106-166: n_i = -sum r_ij w / |r_ij| / n0
// over the reS entries off the mirror side
__global__ void __launch_bounds__(BLK) k_normal(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    const dvec4 pi = d.pos[i];
    double nx = 0, ny = 0, nz = 0;
    forMask(d, i, d.maskS[i], [&](int j, size_t) {
        PairG q = pairOf(d.pos[j], pi);
        double dst = sqrt(q.d2);
        double wS = wfun(dst, P.reS, P.weightType);
        nx += q.v0 * wS / dst; ny += q.v1 * wS / dst; nz += q.v2 * wS / dst;
    });
    d.normal[i] = make_dvec4(-nx / P.pndSmallZero, -ny / P.pndSmallZero, -nz / P.pndSmallZero, 0.0);
}
// calcWallNormalParticles, src/MpsShifting.cpp:319-420: mirror entries of the near-wall fluid
// and i as a neighbour of its mirror, reflected by R
__global__ void __launch_bounds__(BLK) k_wall_normal(Dev d) {
    int i = nearIndex(d);
    if (i < 0) return;
    const MpsParams& P = d.P;
    const dvec4 pi = d.pos[i], mi = d.mirror[i];
    ReflG r = makeRefl(pi, mi, P.epsilonZero, true);
    double dx = 0, dy = 0, dz = 0;
    forNbrs(d, i, [&](int j) {
        dvec4 pj = d.pos[j];
        PairG q = pairOf(pj, pi);
        if (q.d2 < P.reS2) {
            PairM m = pairMirror(pj, mi);
            if (m.dm2 < P.reS2 && q.d2 < m.dm2) {
                double dst = sqrt(m.dm2);
                double wS = wfun(dst, P.reS, P.weightType);
                dx += m.m0 * wS / dst; dy += m.m1 * wS / dst; dz += m.m2 * wS / dst;
            }
        }
    });
    PairM s = pairMirror(pi, mi);
    if (s.dm2 < P.reS2) {
        double dst = sqrt(s.dm2);
        double wS = wfun(dst, P.reS, P.weightType);
        dx += s.m0 * wS / dst; dy += s.m1 * wS / dst; dz += s.m2 * wS / dst;
    }
    dvec4 n = d.normal[i];
    n.x += -(r.R[0] * dx + r.R[1] * dy + r.R[2] * dz) / P.pndSmallZero;
    n.y += -(r.R[3] * dx + r.R[4] * dy + r.R[5] * dz) / P.pndSmallZero;
    n.z += -(r.R[6] * dx + r.R[7] * dy + r.R[8] * dz) / P.pndSmallZero;
    d.normal[i] = n;
}
// MpsBoundaryCondition::updateParticleBC type 2 (ARC), src/MpsBoundaryCondition.cpp:205-395:
// inner when PND, neighbour count and normal allow it; otherwise the list entries in scan
// order (the reference's bucket scan order) decide: the first real or (polygon) mirrored
// neighbour that passes the distance / angle test makes the particle inner, a tested one
// that fails makes it surface (until a later one passes); untested: the PND flag stays.
__global__ void __launch_bounds__(BLK) k_update_bc_arc(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    if (d.type[i] == P.dummyWall) { d.bc[i] = P.other; return; }
    int bc = (d.pndSmall[i] < P.betaPnd) ? P.surface : P.inner;
    dvec4 nv = d.normal[i];
    double n[3] = {nv.x, nv.y, nv.z};
    double norm2 = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
    if (d.pndi[i] >= P.betaPnd && d.numNeigh[i] >= P.betaNeigh && norm2 <= P.normThreshold2) {
        d.bc[i] = P.inner;
        return;
    }
    const dvec4 pi = d.pos[i], mi = d.mirror[i];
    if (norm2 > P.epsilonZero) { double q = sqrt(norm2); n[0] /= q; n[1] /= q; n[2] /= q; }
    else n[0] = n[1] = n[2] = 0.0;
    ReflG r = makeRefl(pi, mi, P.epsilonZero, false);
    double nm[3];
    for (int a = 0; a < 3; a++) nm[a] = r.R[a * 3] * n[0] + r.R[a * 3 + 1] * n[1] + r.R[a * 3 + 2] * n[2];
    double nm2 = nm[0] * nm[0] + nm[1] * nm[1] + nm[2] * nm[2];
    if (nm2 > P.epsilonZero) { double q = sqrt(nm2); nm[0] /= q; nm[1] /= q; nm[2] /= q; }
    else nm[0] = nm[1] = nm[2] = 0.0;
    const double ax = pi.x + P.partDist * n[0], ay = pi.y + P.partDist * n[1], az = pi.z + P.partDist * n[2];
    const double bx = mi.x + P.partDist * nm[0], by = mi.y + P.partDist * nm[1], bz = mi.z + P.partDist * nm[2];
    SideCtx sc = sideCtx(d, i, pi);
    const int c = d.nbrCount[i];
    const int* row = d.nbr + i;
    for (int k = 0; k < c; k++) {
        const int j = ldStream(row + (size_t)k * d.N0);
        const dvec4 pj = d.pos[j];
        PairG q = pairOf(pj, pi);
        if (!(q.d2 < P.reS2)) continue;
        if (sideOK(sc, pj, q.d2)) {
            double c0 = pj.x - ax, c1 = pj.y - ay, c2 = pj.z - az;
            double dinj2 = c0 * c0 + c1 * c1 + c2 * c2;
            double ang = acos((q.v0 * n[0] + q.v1 * n[1] + q.v2 * n[2]) / sqrt(q.d2));
            if ((q.d2 >= P.dstThreshold2 && dinj2 < P.hThreshold2) || (q.d2 < P.dstThreshold2 && ang < P.thetaArc)) {
                bc = P.inner;
                break;
            }
            bc = P.surface;
        }
        if (P.wallType == 1) {
            PairM m = pairMirror(pj, mi);
            if (m.dm2 < P.reS2 && q.d2 < m.dm2) {
                double c0 = pj.x - bx, c1 = pj.y - by, c2 = pj.z - bz;
                double dimnj2 = c0 * c0 + c1 * c1 + c2 * c2;
                double angm = acos((m.m0 * nm[0] + m.m1 * nm[1] + m.m2 * nm[2]) / sqrt(m.dm2));
                if ((m.dm2 >= P.dstThreshold2 && dimnj2 < P.hThreshold2) || (m.dm2 < P.dstThreshold2 && angm < P.thetaArc)) {
                    bc = P.inner;
                    break;
                }
                bc = P.surface;
            }
        }
    }
    d.bc[i] = bc;
}
void launchUpdateBCArc(const Dev& d, cudaStream_t s) {
    k_normal<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
    if (d.P.wallType == 1) k_wall_normal<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
    k_update_bc_arc<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
}

// ------------------------------------------------------------------ EOS
// MpsPressure::calcPressEMPS / calcPressWCMPS, src/MpsPressure.cpp:62-163
__global__ void k_eos(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    double mi = P.DNS_FL1;
    double p = 0.0;
    if (d.bc[i] == P.inner) {
        if (P.mpsType == 0) p = (d.pndi[i] - P.pndSmallZero) * P.coeffPressEMPS * mi;
        else p = (mi * P.coeffPressWCMPS / P.gamma) * (pow(d.pndi[i] / P.pndSmallZero, P.gamma) - 1);
    }
    if (p < 0.0) p = 0.0;
    d.press[i] = p;
}
void launchEOS(const Dev& d, cudaStream_t s) { k_eos<<<gridFor(d.N0, 256), 256, 0, s>>>(d); }

// MpsPressure::extrapolatePressParticlesWallDummy, src/MpsPressure.cpp:792-846
__global__ void __launch_bounds__(BLK) k_extrapolate(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    if (!(d.type[i] == P.dummyWall || (P.mpsType == 1 && d.type[i] == P.wall))) return;
    dvec4 pi = d.pos[i];
    double ni = 0.0, pr = 0.0;
    // particle walls: maskS is exactly dst^2 < reS^2 (no mirror side test)
    forMask(d, i, d.maskS[i], [&](int j, size_t e) {
        if (d.type[j] != P.fluid) return;
        dvec4 pj = d.pos[j];
        double v0 = pj.x - pi.x, v1 = pj.y - pi.y, v2 = pj.z - pi.z;
        double wS = d.cw[e];
        ni += wS;
        pr += (d.press[j] - P.DNS_FL1 * (P.gravity[0] * v0 + P.gravity[1] * v1 + P.gravity[2] * v2)) * wS;
    });
    if (pr < 0.0) return;
    d.press[i] = (ni > 0) ? pr / ni : pr;
}
void launchExtrapolatePress(const Dev& d, cudaStream_t s) { k_extrapolate<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d); }

// ------------------------------------------------------------------ pressure gradient
// MpsPressure::calcPressGradient, src/MpsPressure.cpp:1217-1338 (p_min sweep, then sum)
__global__ void __launch_bounds__(BLK) k_press_grad(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    dvec4 pi = d.pos[i];
    double Pi = d.press[i], pmin = Pi, ni = d.pndi[i];
    int gt = P.gradientType;
    const Mask mS = d.maskS[i];
    if (gt == 0 || gt == 2) {
        forMask(d, i, mS, [&](int j, size_t e) {
            double pj_ = d.press[j];
            if (pmin > pj_) pmin = pj_;
        });
    }
    dvec4 C1 = d.c1[i], C2 = d.c2[i], C3 = d.c3[i];
    double ax = 0, ay = 0, az = 0;
    forMask(d, i, mS, [&](int j, size_t e) {
        dvec4 pj = d.pos[j];
        double v0 = pj.x - pi.x, v1 = pj.y - pi.y, v2 = pj.z - pi.z;
        double Pj = d.press[j];
        double wd = d.cwd[e];   // wS / r^2
        double f;
        if (gt == 0) f = (Pj - pmin) * wd;
        else if (gt == 1) f = (Pj + Pi) * wd;
        else if (gt == 2) f = (Pj + Pi - 2.0 * pmin) * wd;
        else {
            double nj = d.pndi[j];
            f = (ni > P.epsilonZero && nj > P.epsilonZero) ? (ni * Pj / nj + nj * Pi / ni) * wd : d.cw[e];
        }
        if (!P.gradientCorrection) { ax += v0 * f; ay += v1 * f; az += v2 * f; }
        else {
            ax += (v0 * C1.x + v1 * C1.y + v2 * C1.z) * f;
            ay += (v0 * C2.x + v1 * C2.y + v2 * C2.z) * f;
            az += (v0 * C3.x + v1 * C3.y + v2 * C3.z) * f;
        }
    });
    d.acc[i] = make_dvec4(P.relaxPress * ax * P.coeffPressGrad / P.DNS_FL1,
                          P.relaxPress * ay * P.coeffPressGrad / P.DNS_FL1,
                          P.relaxPress * az * P.coeffPressGrad / P.DNS_FL1, 0.0);
}
void launchPressGradient(const Dev& d, cudaStream_t s) { k_press_grad<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d); }

// Wall term of the pressure gradient at a fluid particle near the polygon wall (Mitsume's
// mirror model and the repulsive force), src/MpsPressure.cpp:1341-1611: the sums over the
// candidates that forCand passes as f(j, pj, q), j != i, returned as
// fac * R a * coeffPressGrad - f_rep (fac = relax_fact after the solve, 1 - relax_fact in
// the prediction, src/MpsPressure.cpp:1031-1214).
template <class C>
__device__ __forceinline__ void wallGradTerm(const Dev& d, int i, dvec4 pi, double fac, C&& forCand, double g[3]) {
    const MpsParams& P = d.P;
    // min(velMax of the last corrector, expected maximum velocity)^2 (src/MpsPressure.cpp:1342-1344)
    double vm = fmin(*d.velMax, P.expectMaxVelocity);
    double vMax2 = vm * vm;
    dvec4 mi = d.mirror[i];
    double Pi = d.press[i], pmin = Pi, ni = d.pndi[i];
    int gt = P.gradientType;
    ReflG r = makeRefl(pi, mi, P.epsilonZero, true);
    if (gt == 0 || gt == 2) {
        forCand([&](int j, dvec4 pj, PairG q) {
            if (q.d2 < P.reS2) {
                PairM m = pairMirror(pj, mi);
                if (q.d2 < m.dm2) { double pj_ = d.press[j]; if (pmin > pj_) pmin = pj_; }
            }
        });
    }
    auto phi = [&](double Pj, double nj, double dm2, double wS) {
        if (gt == 0) return wS * ((Pj - pmin) / dm2);
        if (gt == 1) return wS * ((Pj + Pi) / dm2);
        if (gt == 2) return wS * ((Pj + Pi - 2.0 * pmin) / dm2);
        if (gt == 3 && ni > P.epsilonZero && nj > P.epsilonZero) return wS * ((ni * Pj / nj + nj * Pi / ni) / dm2);
        return wS;
    };
    double ax = 0, ay = 0, az = 0;
    forCand([&](int j, dvec4 pj, PairG q) {
        if (q.d2 < P.reS2) {
            PairM m = pairMirror(pj, mi);
            if (m.dm2 < P.reS2 && q.d2 < m.dm2) {
                double wS = wfun(sqrt(m.dm2), P.reS, P.weightType);
                wS = phi(d.press[j], d.pndi[j], m.dm2, wS);
                ax += m.m0 * wS; ay += m.m1 * wS; az += m.m2 * wS;
            }
        }
    });
    PairM s = pairMirror(pi, mi);
    if (s.dm2 < P.reS2) {
        double wS = wfun(sqrt(s.dm2), P.reS, P.weightType);
        wS = phi(Pi, ni, s.dm2, wS);
        ax += s.m0 * wS; ay += s.m1 * wS; az += s.m2 * wS;
    }
    double f[3];
    wallRepulsion(P, r, vMax2, f);
    g[0] = fac * (r.R[0] * ax + r.R[1] * ay + r.R[2] * az) * P.coeffPressGrad - f[0];
    g[1] = fac * (r.R[3] * ax + r.R[4] * ay + r.R[5] * az) * P.coeffPressGrad - f[1];
    g[2] = fac * (r.R[6] * ax + r.R[7] * ay + r.R[8] * az) * P.coeffPressGrad - f[2];
}

// MpsPressure::calcWallPressGradient + repulsive forces, src/MpsPressure.cpp:1341-1611,
// over the post-prediction neighbour list.
__global__ void __launch_bounds__(BLK) k_wall_press_grad(Dev d) {
    int i = nearIndex(d);
    if (i < 0) return;
    const MpsParams& P = d.P;
    dvec4 pi = d.pos[i];
    double g[3];
    wallGradTerm(d, i, pi, P.relaxPress, [&](auto&& f) {
        forNbrs(d, i, [&](int j) { dvec4 pj = d.pos[j]; f(j, pj, pairOf(pj, pi)); });
    }, g);
    dvec4 a = d.acc[i];
    a.x += g[0] / P.DNS_FL1; a.y += g[1] / P.DNS_FL1; a.z += g[2] / P.DNS_FL1;
    d.acc[i] = a;
    double vf = (P.dim == 3) ? P.partDist * P.partDist * P.partDist : P.partDist * P.partDist;
    dvec4 fw = d.forceWall[i];
    fw.x += -g[0] * vf; fw.y += -g[1] * vf; fw.z += -g[2] * vf;
    d.forceWall[i] = fw;
}
void launchWallPressGradient(const Dev& d, cudaStream_t s) {
    if (d.P.wallType != 1) return;
    k_wall_press_grad<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
}

// ------------------------------------------------------------------ prediction-step pressure gradient
// relax_fact < 1 (src/main.cpp:271-276): before the prediction, (1 - relax_fact) of the
// previous pressure's gradient at the start-of-step positions is added to the
// acceleration.  The candidates of i in scan order: the start-of-step skin list when it
// is built for these positions (its entries within the FP32 band of the ball are the
// candidates the 27-bucket scan passes to the exact FP64 test), else the scan itself.
template <class F>
__device__ __forceinline__ void forStartCandidates(const Dev& d, int i, dvec4 pi, float hi, bool skin, F&& f) {
    const float4 fi = d.posf[i];
    const int c = skin ? d.skinCnt[i] : d.K + 1;
    if (c <= d.K) {
        const int* row = d.skinNbr + i;
        for (int k = 0; k < c; k++) {
            const int j = ldStream(row + (size_t)k * d.N0);
            const float4 fj = d.posf[j];
            const float ex = fj.x - fi.x, ey = fj.y - fi.y, ez = fj.z - fi.z;
            if (ex * ex + ey * ey + ez * ez > hi) continue;
            const dvec4 pj = d.pos[j];
            f(j, pj, pairOf(pj, pi));
        }
    } else {
        forCellsNear(d, pi, fi, hi, [&](int j, dvec4 pj, PairG q) {
            if (j != i) f(j, pj, q);
        });
    }
}

// MpsPressure::predictionPressGradient, src/MpsPressure.cpp:932-1028: every particle, the
// gradient type's pair term without the correction matrix, in the reference's operation
// order (w(r) from |r|, then times (...)/r^2).
__global__ void __launch_bounds__(BLK) k_pred_press_grad(Dev d, bool skin) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    const dvec4 pi = d.pos[i];
    const SideCtx sc = sideCtx(d, i, pi);
    const double Pi = d.press[i], ni = d.pndi[i];
    double pmin = Pi;
    const int gt = P.gradientType;
    if (gt == 0 || gt == 2) {
        forStartCandidates(d, i, pi, d.bandHiS, skin, [&](int j, dvec4 pj, PairG q) {
            if (q.d2 < P.reS2 && sideOK(sc, pj, q.d2)) { double pj_ = d.press[j]; if (pmin > pj_) pmin = pj_; }
        });
    }
    double ax = 0, ay = 0, az = 0;
    forStartCandidates(d, i, pi, d.bandHiS, skin, [&](int j, dvec4 pj, PairG q) {
        if (!(q.d2 < P.reS2) || !sideOK(sc, pj, q.d2)) return;
        double wS = wfun(sqrt(q.d2), P.reS, P.weightType);
        const double Pj = d.press[j];
        if (gt == 0) wS *= (Pj - pmin) / q.d2;
        else if (gt == 1) wS *= (Pj + Pi) / q.d2;
        else if (gt == 2) wS *= (Pj + Pi - 2.0 * pmin) / q.d2;
        else if (gt == 3) {
            const double nj = d.pndi[j];
            if (ni > P.epsilonZero && nj > P.epsilonZero) wS *= (ni * Pj / nj + nj * Pi / ni) / q.d2;
        }
        ax += q.v0 * wS; ay += q.v1 * wS; az += q.v2 * wS;
    });
    const double fac = 1.0 - P.relaxPress;
    dvec4 a = d.acc[i];
    a.x += fac * ax * P.coeffPressGrad / P.DNS_FL1;
    a.y += fac * ay * P.coeffPressGrad / P.DNS_FL1;
    a.z += fac * az * P.coeffPressGrad / P.DNS_FL1;
    d.acc[i] = a;
}

// MpsPressure::predictionWallPressGradient, src/MpsPressure.cpp:1031-1214: fluid particles
// flagged near the wall by the last wall pass (its flags and mirror positions are still
// held: the prediction resets them after this sweep), no force on the wall.
__global__ void __launch_bounds__(BLK) k_pred_wall_press_grad(Dev d, bool skin) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    if (d.type[i] != P.fluid || !d.nearWall[i]) return;
    const dvec4 pi = d.pos[i];
    double g[3];
    wallGradTerm(d, i, pi, 1.0 - P.relaxPress, [&](auto&& f) {
        forStartCandidates(d, i, pi, d.bandHiS, skin, f);
    }, g);
    dvec4 a = d.acc[i];
    a.x += g[0] / P.DNS_FL1; a.y += g[1] / P.DNS_FL1; a.z += g[2] / P.DNS_FL1;
    d.acc[i] = a;
}

void launchPredictPressGradient(const Dev& d, bool skin, cudaStream_t s) {
    k_pred_press_grad<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d, skin);
    // the wall sweep reads the accelerations the particle sweep has completed
    if (d.P.wallType == 1) k_pred_wall_press_grad<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d, skin);
}

// ------------------------------------------------------------------ wall viscosity
// MpsViscosity::calcWallNoSlipViscosity / calcWallSlipViscosity (Newtonian, fixed wall),
// src/MpsViscosity.cpp:1527-1910
__global__ void __launch_bounds__(BLK) k_wall_visc(Dev d) {
    int i = nearIndex(d);
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
    double mu = P.KNM_VS1 * P.DNS_FL1;
    double neu = ((mu + mu) > P.epsilonZero ? 2.0 * mu * mu / (mu + mu) : 0.0) / P.DNS_FL1;
    double ax = 0, ay = 0, az = 0;
    forNbrs(d, i, [&](int j) {
        dvec4 pj = d.pos[j];
        PairG q = pairOf(pj, pi);
        if (q.d2 < P.reL2) {
            PairM m = pairMirror(pj, mi);
            if (m.dm2 < P.reL2 && q.d2 < m.dm2) {
                double wL = wfun(sqrt(m.dm2), P.reL, P.weightType);
                dvec4 vj = d.vel[j];
                ax += (vj.x - vm0) * wL * neu;
                ay += (vj.y - vm1) * wL * neu;
                az += (vj.z - vm2) * wL * neu;
            }
        }
    });
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
void launchWallViscosity(const Dev& d, cudaStream_t s) {
    if (d.P.wallType != 1) return;
    k_wall_visc<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
}

// ------------------------------------------------------------------ corrector
// MpsParticleVelPos::correctionVelocityPosition, src/MpsParticleVelPos.cpp:53-97, with the
// maximum fluid speed reduced on the device (max is order independent).
__global__ void k_correct(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const MpsParams& P = d.P;
    double v = 0.0;
    if (i < liveN(d) && d.type[i] == P.fluid) {
        dvec4 u = d.vel[i], a = d.acc[i], x = d.pos[i];
        double dt = P.timeStep, dt2 = P.timeStep * P.timeStep;
        u.x += a.x * dt; u.y += a.y * dt; u.z += a.z * dt;
        x.x += a.x * dt2; x.y += a.y * dt2; x.z += a.z * dt2;
        d.vel[i] = u; d.pos[i] = x;
        d.acc[i] = make_dvec4(0, 0, 0, 0);
        v = sqrt(u.x * u.x + u.y * u.y + u.z * u.z);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __shared__ double sm[32];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sm[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (lane < (int)(blockDim.x >> 5)) ? sm[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0 && v > 0.0)
            atomicMax((unsigned long long*)d.velMax, (unsigned long long)__double_as_longlong(v));
    }
}
void launchCorrect(const Dev& d, cudaStream_t s) {
    cudaMemsetAsync(d.velMax, 0, sizeof(double), s);
    k_correct<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
}

// ------------------------------------------------------------------ shifting
// MpsShifting::calcShifting (type 1), src/MpsShifting.cpp:23-101: dv from the
// pre-shift velocities, then applied.
// Common head of the post-corrector scans: prefilter band of the reS ball, exact FP64
// radius and mirror-side tests; particles the sweep does not update skip the scan.
struct E2Base {
    struct Core { SideCtx sc; bool on; };
    __device__ static void start(const Dev& d, int i, Core& c, bool on) {
        c.on = on;
        if (on) c.sc = sideCtx(d, i, d.pos[i]);
    }
    __device__ static bool accept(const Dev& d, const Core& c, dvec4 pj, PairG q) {
        return q.d2 < d.P.reS2 && sideOK(c.sc, pj, q.d2);
    }
};
#define E2_COMMON \
    __device__ float hi(const Dev& d) const { return d.bandHiS; } \
    __device__ bool active(const Dev&, const State& st) const { return st.c.on; }
struct OpShiftVel {
    struct State { E2Base::Core c; dvec4 vi; double ux, uy, uz; };
    E2_COMMON
    __device__ void begin(const Dev& d, int i, State& st) const {
        E2Base::start(d, i, st.c, d.type[i] == d.P.fluid);
        st.vi = d.vel[i]; st.ux = st.uy = st.uz = 0.0;
    }
    __device__ void visit(const Dev& d, int i, State& st, int j, dvec4 pj, PairG q) const {
        if (!E2Base::accept(d, st.c, pj, q)) return;
        double dw = dwfun(sqrt(q.d2), d.P.reS, d.P.weightType);
        dvec4 vj = d.vel[j];
        st.ux += dw * (vj.x - st.vi.x); st.uy += dw * (vj.y - st.vi.y); st.uz += dw * (vj.z - st.vi.z);
    }
    __device__ void end(const Dev& d, int i, State& st) const {
        bool apply = st.c.on && d.bc[i] == d.P.inner;
        d.shift[i] = apply ? make_dvec4(st.ux, st.uy, st.uz, 0.0) : make_dvec4(0, 0, 0, 0);
    }
};
__global__ void k_shift_vel_apply(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    dvec4 v = d.vel[i], du = d.shift[i];
    double c = d.P.coeffShifting1;
    v.x -= c * du.x; v.y -= c * du.y; v.z -= c * du.z;
    d.vel[i] = v;
}
// MpsShifting::calcConcAndConcGradient, src/MpsShifting.cpp:432-575: concentration, then
// gradient and position shift (each sweep reads the positions it started with).
struct OpConc {
    struct State { E2Base::Core c; double sum; };
    E2_COMMON
    __device__ void begin(const Dev& d, int i, State& st) const { E2Base::start(d, i, st.c, true); st.sum = 0.0; }
    __device__ void visit(const Dev& d, int i, State& st, int j, dvec4 pj, PairG q) const {
        if (!E2Base::accept(d, st.c, pj, q)) return;
        double w, wd;
        weightR(q.d2, d.P.reS, d.P.weightType, w, wd);
        st.sum += w;
    }
    __device__ void end(const Dev& d, int i, State& st) const {
        d.conc[i] = (st.sum + d.pndWall[i]) / d.P.pndSmallZero;
    }
};
struct OpGradConc {
    struct State { E2Base::Core c; double ci, gx, gy, gz; };
    E2_COMMON
    __device__ void begin(const Dev& d, int i, State& st) const {
        E2Base::start(d, i, st.c, d.type[i] == d.P.fluid);
        st.ci = d.conc[i]; st.gx = st.gy = st.gz = 0.0;
    }
    __device__ void visit(const Dev& d, int i, State& st, int j, dvec4 pj, PairG q) const {
        if (!E2Base::accept(d, st.c, pj, q)) return;
        double wS, wd;
        weightR(q.d2, d.P.reS, d.P.weightType, wS, wd);
        double cc = (st.ci + d.conc[j]) * wd;
        st.gx += cc * q.v0; st.gy += cc * q.v1; st.gz += cc * q.v2;
    }
    __device__ void end(const Dev& d, int i, State& st) const {
        const MpsParams& P = d.P;
        dvec4 sh = make_dvec4(0, 0, 0, 0);
        if (st.c.on) {
            double gx = st.gx * -P.coeffPressGrad, gy = st.gy * -P.coeffPressGrad, gz = st.gz * -P.coeffPressGrad;
            d.gradC[i] = make_dvec4(gx, gy, gz, 0.0);
            if (d.bc[i] == P.inner)
                sh = make_dvec4(-P.coeffShifting2 * gx, -P.coeffShifting2 * gy, -P.coeffShifting2 * gz, 0.0);
        }
        d.shift[i] = sh;
    }
};
// MpsShifting::calcWallConcAndConcGradient, src/MpsShifting.cpp:578-691
__global__ void __launch_bounds__(BLK) k_wall_grad_conc(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    dvec4 sh = make_dvec4(0, 0, 0, 0);
    if (d.type[i] == P.fluid && d.nearWall[i]) {
        dvec4 pi = d.pos[i], mi = d.mirror[i];
        double ci = d.conc[i];
        ReflG r = makeRefl(pi, mi, P.epsilonZero, true);
        double dx = 0, dy = 0, dz = 0;
        forCellsNear(d, pi, d.posf[i], d.bandHiS, [&](int j, dvec4 pj, PairG q) {
            if (q.d2 < P.reS2 && j != i) {
                PairM m = pairMirror(pj, mi);
                if (m.dm2 < P.reS2 && q.d2 < m.dm2) {
                    double wS = wfun(sqrt(m.dm2), P.reS, P.weightType);
                    double cc = ci + d.conc[j];
                    dx += cc * m.m0 * wS / m.dm2; dy += cc * m.m1 * wS / m.dm2; dz += cc * m.m2 * wS / m.dm2;
                }
            }
        });
        PairM s = pairMirror(pi, mi);
        if (s.dm2 < P.reS2) {
            double wS = wfun(sqrt(s.dm2), P.reS, P.weightType);
            dx += (ci + ci) * s.m0 * wS / s.dm2; dy += (ci + ci) * s.m1 * wS / s.dm2; dz += (ci + ci) * s.m2 * wS / s.dm2;
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
// x += shift; the FP32 copy follows the new positions (next prefiltered scan)
__global__ void k_apply_shift(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    dvec4 x = d.pos[i], s = d.shift[i];
    x.x += s.x; x.y += s.y; x.z += s.z;
    d.pos[i] = x;
    float4 hi = make_float4(d2fRN(x.x - d.P.domainMin[0]), d2fRN(x.y - d.P.domainMin[1]),
                            d2fRN(x.z - d.P.domainMin[2]), 0.f);
    d.posf[i] = hi;
    d.posLo[i] = posLoOf(x, hi, d.P);
}
void launchShiftVelApply(const Dev& d, cudaStream_t s) { k_shift_vel_apply<<<gridFor(d.N0, 256), 256, 0, s>>>(d); }
void launchApplyShift(const Dev& d, cudaStream_t s) { k_apply_shift<<<gridFor(d.N0, 256), 256, 0, s>>>(d); }
// A 27-bucket sweep over the list of the current positions instead of the buckets: the
// list holds every candidate within reMax of the scan, in the scan's order, and each
// operator applies its own exact radius and side tests, so it sees the same neighbours in
// the same order (the same sums).
template <class Op>
__global__ void __launch_bounds__(128) k_list_scan(Dev d, Op op) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    typename Op::State st;
    op.begin(d, i, st);
    if (op.active(d, st)) {
        const dvec4 pi = d.pos[i];
        const int c = d.nbrCount[i];
        const int* row = d.nbr + i;
        for (int k = 0; k < c; k++) {
            const int j = ldStream(row + (size_t)k * d.N0);
            const dvec4 pj = d.pos[j];
            op.visit(d, i, st, j, pj, pairOf(pj, pi));
        }
    }
    op.end(d, i, st);
}
template <class Op>
static void launchSweep(const Dev& d, const Op& op, bool list, cudaStream_t s) {
    if (list) k_list_scan<Op><<<gridFor(d.N0, 128), 128, 0, s>>>(d, op);
    else launchScan(d, op, s);
}

// list: the sweeps read the list of the post-corrector positions, filtered from the kept
// start-of-step skin list (launchNeighborFilter without the weight cache, which also
// refreshes the FP32 copies) just before; else they scan the buckets
void launchShifting(const Dev& d, cudaStream_t s, bool list) {
    const MpsParams& P = d.P;
    if (P.shiftingType != 1 && P.shiftingType != 2) return;
    if (!list) launchPosf(d, s);   // post-corrector positions
    if (P.shiftingType == 1) {
        launchSweep(d, OpShiftVel(), list, s);
        k_shift_vel_apply<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
    } else {
        launchSweep(d, OpConc(), list, s);
        launchSweep(d, OpGradConc(), list, s);
        k_apply_shift<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
        if (P.wallType == 1) {
            launchPosfCell(d, s);   // the wall sweep sees the shifted positions
            k_wall_grad_conc<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
            k_apply_shift<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
        }
    }
}

// ------------------------------------------------------------------ dummy velocity
// MpsParticleVelPos::updateVelocityParticlesWallDummy, src/MpsParticleVelPos.cpp:100-158
// (dummy particles read fluid velocities only, so the update is race free in place)
__global__ void __launch_bounds__(BLK) k_dummy_vel(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    if (d.type[i] != P.dummyWall) return;
    dvec4 pi = d.pos[i];
    double ni = 0.0, ux = 0, uy = 0, uz = 0;
    forCellsNear(d, pi, d.posf[i], d.bandHiL, [&](int j, dvec4 pj, PairG q) {
        if (q.d2 < P.reL2 && j != i && d.type[j] == P.fluid) {
            double wL, wd;
            weightR(q.d2, P.reL, P.weightType, wL, wd);
            dvec4 vj = d.vel[j];
            ni += wL;
            ux += vj.x * wL; uy += vj.y * wL; uz += vj.z * wL;
        }
    });
    dvec4 v;
    if (ni > P.epsilonZero) v = make_dvec4(2.0 * 0.0 - ux / ni, 2.0 * 0.0 - uy / ni, 2.0 * 0.0 - uz / ni, 0.0);
    else v = make_dvec4(2.0 * 0.0 - ux, 2.0 * 0.0 - uy, 2.0 * 0.0 - uz, 0.0);
    d.vel[i] = v;
}
void launchDummyVelocity(const Dev& d, cudaStream_t s) {
    if (d.P.wallType != 0) return;
    launchPosf(d, s);
    k_dummy_vel<<<gridFor(d.N0, BLK), BLK, 0, s>>>(d);
}
