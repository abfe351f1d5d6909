// mps_api.cu — the C ABI of libmpsgpu (include/mpsgpu.h): handle, device memory,
// field transfer in the reference's host layout, and the step in the reference order
// (mainLoopOfSimulation, src/main.cpp:256-467).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include <utility>
#include <algorithm>
#include "mps_common.cuh"
#include "mps_internal.h"
#include "mps_host.h"
#include "mps_mlp.h"

namespace {
thread_local std::string g_lastError;
}

struct mpsgpu_s {
    Dev d;
    PpeBuffers B;
    cudaStream_t s = nullptr;
    int N0 = 0;
    std::vector<void*> allocs;
    int* scanScratch = nullptr;
    int* outFlags = nullptr;
    int* outCounter = nullptr;
    int* perm = nullptr;          // storage renumbering: permutation and gather scratch
    void* permScratch = nullptr;
    int renumberEvery = 20;       // bucket rebuilds between storage renumberings (0: never)
    int renumberCountdown = 0;    // 0: renumber at the next bucket rebuild
    // solver controls
    int solver = MPSGPU_SOLVER_PLAIN_FP64, warm = MPSGPU_WARM_PREVIOUS;
    double tol = 1e-8;
    int maxIter = 0;
    // host mirrors of a few scalars
    bool listValid = false;
    bool masksValid = false;
    bool skinValid = false;    // the skin list of this bucket list is built and not yet filtered
    bool skinShift = false;    // ... and still intact for the shifting sweeps of the step
    int nHost = -1;            // live count known on the host (-1: read it from the device)
    int *nbrAlt = nullptr, *cntAlt = nullptr;   // second list arrays (the skin list keeps its own)
    int skinOn = 1;            // viscosity and the post-prediction list from the start-of-step skin list
    bool corrFresh = false;    // the correction matrix of the current positions and masks is written
    bool opSkipped = false;    // the last operator had nothing left to launch
    void* vtuDev = nullptr;    // staging of the binary .vtu block (device, page-locked host)
    void* vtuHost = nullptr;
    size_t vtuCap = 0;
    bool cacheValid = false;   // per-entry FP64 weights of the current list
    int persistent = 1;        // PPE launch: 0 per kernel, 1 single cooperative launch, 2 + staged ELL tiles
    double timeCurrent = 0.0;
    int numIter = 0;
    int lastOut = 0;
    MpsStepStats last{};
    cudaEvent_t e0 = nullptr, e1 = nullptr, ea0 = nullptr, ea1 = nullptr, es0 = nullptr, es1 = nullptr;
    // second stream of the step (the wall distance beside the list filter and the collision)
    // and its fork and join events
    cudaStream_t s2 = nullptr;
    cudaEvent_t evFork = nullptr, evJoin = nullptr;
    std::string err;
    MlpState mlp;
    Prof prof;
};

// ------------------------------------------------------------------ profiler
void Prof::begin(int c, cudaStream_t s, bool count) {
    if (2 * used + 2 > ev.size()) {
        for (int k = 0; k < 64; k++) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            ev.push_back(e);
        }
        cls.resize(ev.size() / 2);
    }
    cls[used] = count ? c : (c | 0x10000);   // 0x10000: time only, no call counted
    cudaEventRecord(ev[2 * used], s);
    open.push_back(used);
    used++;
}
void Prof::end(cudaStream_t s) {
    if (open.empty()) return;
    size_t slot = open.back();
    open.pop_back();
    cudaEventRecord(ev[2 * slot + 1], s);
}
int Prof::flush() {
    if (!used || !open.empty()) return 0;
    if (cudaEventSynchronize(ev[2 * used - 1]) != cudaSuccess) return MPSGPU_ERR_CUDA;
    for (size_t k = 0; k < used; k++)
        if (cudaEventSynchronize(ev[2 * k + 1]) != cudaSuccess) return MPSGPU_ERR_CUDA;
    for (size_t k = 0; k < used; k++) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ev[2 * k], ev[2 * k + 1]);
        const int c = cls[k] & 0xffff;
        this->ms[c] += ms;
        if (!(cls[k] & 0x10000)) calls[c]++;
    }
    used = 0;
    return 0;
}
void Prof::reset() {
    used = 0;
    for (int k = 0; k < PROF_NCLASS; k++) { ms[k] = 0; calls[k] = 0; }
}
void Prof::destroy() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    ev.clear(); cls.clear(); used = 0;
}

// Kernels launched by one operator (fixed by the configuration; the solvers count theirs).
static int opLaunches(int op, const MpsParams& P, bool x) {
    switch (op) {
        case MPS_OP_UPDATE_BUCKETS: return 8;   // key, 3 scan, scatter, sort, list positions, bucket-ordered copy
        case MPS_OP_VISCOSITY: return x ? 3 : 1;   // (DF32: velocity copy) + sweep (+ unlisted particles)
        case MPS_OP_OUT_OF_DOMAIN: return 2;
        case MPS_OP_COLLISION: return P.collisionType == 1 ? 2 : (x ? 3 : 2);
        case MPS_OP_WALL_DISTANCE: case MPS_OP_WALL_NPCD: return P.wallType == 1 ? 1 : 0;
        case MPS_OP_WALL_PRESS_GRADIENT: case MPS_OP_WALL_VISCOSITY: return P.wallType == 1 ? (x ? 2 : 1) : 0;
        case MPS_OP_PRESS_GRADIENT: return x ? 2 : 1;
        case MPS_OP_PREDICT_PRESS_GRADIENT: return P.relaxPress < 1.0 ? (P.wallType == 1 ? 2 : 1) : 0;
        case MPS_OP_PND_DIFFUSIVE: return P.wallType == 1 ? 5 : 4;
        case MPS_OP_PND_MEAN: return P.wallType == 1 ? 3 : 2;
        case MPS_OP_INIT_PND: return 2 + (P.wallType == 1 ? 3 : 2);
        case MPS_OP_CALC_PRESS:   // (velocity divergence) + assemble + copy back | EOS
            return (P.mpsType == 2) ? 2 : (P.mpsType == 3 ? (P.wallType == 1 ? 4 : 3) : 1);
        case MPS_OP_SHIFTING:   // FP32 copies (2) + scans + apply kernels (DF32: two scans per sweep + copies)
            if (x) return P.shiftingType == 1 ? 6 : (P.shiftingType == 2 ? (P.wallType == 1 ? 11 : 8) : 0);
            return P.shiftingType == 1 ? 4 : (P.shiftingType == 2 ? (P.wallType == 1 ? 8 : 5) : 0);
        case MPS_OP_DUMMY_VELOCITY: return P.wallType == 0 ? 3 : 0;
        case MPS_OP_UPDATE_BC: return P.freeSurfType == 2 ? (P.wallType == 1 ? 3 : 2) : 1;   // (normals) + flags
        default: return 1;
    }
}

#define CK(x)                                                                    \
    do {                                                                         \
        cudaError_t _e = (x);                                                    \
        if (_e != cudaSuccess) {                                                 \
            g_lastError = std::string(#x) + ": " + cudaGetErrorString(_e);       \
            return MPSGPU_ERR_CUDA;                                              \
        }                                                                        \
    } while (0)

template <class T>
static int dalloc(mpsgpu_t h, T** p, size_t count) {
    void* q = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T));
    if (e != cudaSuccess) { g_lastError = std::string("cudaMalloc: ") + cudaGetErrorString(e); return MPSGPU_ERR_NOMEM; }
    cudaMemsetAsync(q, 0, count * sizeof(T), h->s);
    h->allocs.push_back(q);
    *p = (T*)q;
    return 0;
}

static int checkDeviceErrors(mpsgpu_t h) {
    unsigned int e = 0;
    CK(cudaMemcpyAsync(&e, h->d.err, sizeof(e), cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    if (e) {
        CK(cudaMemsetAsync(h->d.err, 0, sizeof(unsigned int), h->s));
        if (e & MPSE_CAPACITY) { g_lastError = "neighbour row capacity exceeded"; return MPSGPU_ERR_CAPACITY; }
        if (e & MPSE_DOMAIN) { g_lastError = "particle outside the bucket grid"; return MPSGPU_ERR_DOMAIN; }
        if (e & MPSE_NAN) { g_lastError = "non-finite value"; return MPSGPU_ERR_NOT_CONVERGED; }
    }
    return 0;
}

static int launchStatus() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { g_lastError = std::string("kernel launch: ") + cudaGetErrorString(e); return MPSGPU_ERR_CUDA; }
    return 0;
}

static bool df32(mpsgpu_t h) { return h->d.prec == MPSGPU_PRECISION_DF32; }
static void ensureList(mpsgpu_t h) {
    if (h->listValid) return;
    if (h->prof.on) h->prof.begin(PROF_NEIGHBOR_LIST, h->s);
    if (h->skinValid) {
        if (df32(h)) launchNeighborFilterDF(h->d, h->s);
        else launchNeighborFilter(h->d, h->s);
        countLaunch(df32(h) ? 5 : 4);   // FP32 copies (2), skin check, filter (DF32: listed + unlisted particles)
    } else {
        if (df32(h)) launchNeighborListDF(h->d, h->s);
        else launchNeighborList(h->d, h->s);
        countLaunch(df32(h) ? 4 : 3);   // FP32 copies (2), list build (DF32: + unlisted particles)
    }
    h->skinValid = false;
    if (h->prof.on) h->prof.end(h->s);
    h->listValid = true;
    h->masksValid = false;
    h->cacheValid = !df32(h);   // the FP64 list build stores the per-entry weights
}
// Per-entry FP64 weights for the FP64 sweeps that read them (in the DF32 tier only the
// operators without a DF32 kernel need them).
static void ensureCache(mpsgpu_t h) {
    ensureList(h);
    if (h->cacheValid) return;
    if (h->prof.on) h->prof.begin(PROF_NEIGHBOR_LIST, h->s);
    launchFillCache(h->d, h->s);
    if (h->prof.on) h->prof.end(h->s);
    countLaunch(1);
    h->cacheValid = true;
}
// Entry masks depend on the list and on the mirror positions of the wall pass.
static void ensureMasks(mpsgpu_t h) {
    ensureList(h);
    if (h->masksValid) return;
    if (h->prof.on) h->prof.begin(PROF_NEIGHBOR_LIST, h->s);
    if (df32(h)) launchSideMasksDF(h->d, h->s);
    else launchSideMasks(h->d, h->s);
    if (h->prof.on) h->prof.end(h->s);
    countLaunch(1);
    h->masksValid = true;
}

// Switches of the reference outside the implemented path, each with the reason.
static const char* unsupportedReason(const MpsParams& P) {
    if (P.femOn || P.forcedOn) return "fem_MESH / forced_MESH: deformable and forced meshes are not supported";
    if (P.domainTypeBC != 0) return "domain.boundary.type != 0: periodic domains are not supported";
    if (P.fluidType != 0) return "physical.fluid_type != 0: non-Newtonian rheology is not supported";
    if (P.collisionType != 0 && P.collisionType != 1)
        return "particle_collision.type: only 0 (PC) and 1 (DPC) are supported";
    if (P.solverType != 0 && P.solverType != 1)
        return "semi_implicit_mps.solver_type: only 0 (CG) and 1 (BiCGSTAB) are supported";
    if (P.wallType != 0 && P.wallType != 1) return "wall_type: only 0 (particles) and 1 (polygon) are supported";
    if (P.mpsType < 0 || P.mpsType > 3) return "mps_type: only 0 to 3 are supported";
    return nullptr;
}

int mpsgpu_check_params(const MpsParams* p) {
    if (!p) { g_lastError = "bad argument"; return MPSGPU_ERR_ARG; }
    if (const char* why = unsupportedReason(*p)) {
        g_lastError = std::string("configuration outside the implemented path: ") + why;
        return MPSGPU_ERR_UNSUPPORTED;
    }
    return 0;
}

// ------------------------------------------------------------------ pressure
static int calcPress(mpsgpu_t h) {
    const MpsParams& P = h->d.P;
    if (P.mpsType == 0 || P.mpsType == 1) {
        launchEOS(h->d, h->s);
        return launchStatus();
    }
    ensureMasks(h);
    cudaEventRecord(h->ea0, h->s);
    if (h->prof.on) h->prof.begin(PROF_PPE_ASSEMBLE, h->s);
    // PND + div u source: velocity divergence of the predicted velocities (src/MpsPressure.cpp:44-56)
    if (P.mpsType == 3) launchVelDivergence(h->d, h->s);
    if (df32(h)) launchPpeAssembleDF(h->d, h->B, h->s);
    else launchPpeAssemble(h->d, h->B, h->s);
    if (h->prof.on) h->prof.end(h->s);
    cudaEventRecord(h->ea1, h->s);
    // the solve's time includes its warm start's generation, whichever it is
    cudaEventRecord(h->es0, h->s);
    // warm start: previous unclamped solution (reference), zero, extrapolated, or the
    // learned predictor
    if (h->warm == MPSGPU_WARM_ZERO) cudaMemsetAsync(h->B.x, 0, sizeof(double) * h->N0, h->s);
    if (h->warm == MPSGPU_WARM_EXTRAPOLATE || h->warm == MPSGPU_WARM_EXTRAPOLATE2) {
        launchWarmExtrapolate(h->d, h->B, h->s, h->warm == MPSGPU_WARM_EXTRAPOLATE2);
        countLaunch(1);
    }
    h->B.prepared = df32(h) ? 1 : 0;   // the DF32 assembly writes the FP32 copies itself
    // the block-owned mixed solve takes the learned start's residual-minimising step itself
    const bool ownSolve = h->solver == MPSGPU_SOLVER_MIXED && h->persistent == 1 && !h->B.ownOff &&
                          h->B.pgridOwn > 0 && h->B.ownCap > 0 && P.solverType != 1;
    h->B.cdir = nullptr;
    if (h->warm == MPSGPU_WARM_MLP) {
        if (h->prof.on) h->prof.begin(PROF_PPE_OTHER, h->s);
        // the learned start reads the FP32 copy of the matrix
        if (!h->B.prepared) { launchMixedPrepare(h->d, h->B, h->s); h->B.prepared = 1; countLaunch(1); }
        int e = mlpWarmStart(h->mlp, h->d, h->B, h->s, ownSolve);
        if (h->prof.on) h->prof.end(h->s);
        // x_e, its FP64 residual, features, scale, forward, A c; or x_e copy, residual,
        // features, scale, forward, correction, step dot products, step, apply
        countLaunch(ownSolve ? 6 : 9);
        if (e) return e;
        if (ownSolve) { h->B.cdir = h->mlp.cdir; h->B.cq = h->mlp.re; }
    } else if (h->warm == MPSGPU_WARM_PREVIOUS) {
        cudaMemcpyAsync(h->B.x, h->d.pressPPE, sizeof(double) * h->N0, cudaMemcpyDeviceToDevice, h->s);
    }
    int iters = 0, refine = 0;
    double rr = 0, rr0 = 0;
    int maxIt = h->maxIter > 0 ? h->maxIter : 2 * h->N0;
    int e;
    const bool mixed = h->solver != MPSGPU_SOLVER_PLAIN_FP64;
    h->B.matfree = h->solver == MPSGPU_SOLVER_MIXED_MATFREE ? 1 : (h->solver == MPSGPU_SOLVER_MIXED_COMPACT ? 2 : 0);
    if (h->solver == MPSGPU_SOLVER_MIXED && h->persistent == 2 && h->B.pgridTs > 0) h->B.matfree = 3;
    if (h->solver == MPSGPU_SOLVER_MIXED && h->persistent == 3 && h->B.pgridPipe > 0) h->B.matfree = 4;
    int pgrid = !mixed ? h->B.pgridCg
                       : (h->B.matfree == 4 ? h->B.pgridPipe
                          : h->B.matfree == 3 ? h->B.pgridTs
                                              : (h->B.matfree == 2 ? h->B.pgridH16 : (h->B.matfree ? h->B.pgridMf : h->B.pgridMx)));
    if (h->B.matfree && (!h->persistent || pgrid <= 0)) {
        g_lastError = "this mixed inner operator needs the single-launch (cooperative) PPE solve";
        return MPSGPU_ERR_UNSUPPORTED;
    }
    if (P.solverType == 1) {   // BiCGSTAB (the reference's solver_type 1), FP64
        e = ppeSolveBicgstab(h->d, h->B, h->tol, maxIt, h->s, &iters, &rr, &rr0, &h->prof);
        if (e == MPSGPU_ERR_CUDA) g_lastError = "BiCGSTAB: launch failed or a grid-barrier wait ran out";
        if (e == MPSGPU_ERR_UNSUPPORTED) g_lastError = "BiCGSTAB needs cooperative launches";
    } else if (h->persistent && pgrid > 0) {
        e = ppeSolvePersistent(h->d, h->B, mixed ? 1 : 0, h->tol, maxIt, h->s, &iters, &refine, &rr, &rr0, &h->prof);
        if (e == MPSGPU_ERR_CUDA) g_lastError = "persistent PPE solve: launch failed or a grid-barrier wait ran out";
    } else if (mixed) {
        e = ppeSolveMixed(h->d, h->B, h->tol, maxIt, h->s, &iters, &refine, &rr, &rr0, &h->prof);
    } else {
        e = ppeSolvePlain(h->d, h->B, h->tol, maxIt, h->s, &iters, &rr, &rr0, &h->prof);
    }
    if (h->warm == MPSGPU_WARM_MLP && !e && (e = mlpTcStatus(h->mlp, h->s)))
        g_lastError = "learned warm start: a tensor-core completion wait ran out";
    // the final FP64 residual judges the fast solvers: a mixed solve that missed the
    // tolerance is redone by the plain FP64 CG from the previous unclamped solution
    h->last.ppeFallback = 0;
    if (mixed && e == MPSGPU_ERR_NOT_CONVERGED) {
        cudaMemcpyAsync(h->B.x, h->d.pressPPE, sizeof(double) * h->N0, cudaMemcpyDeviceToDevice, h->s);
        int fi = 0, fr = 0;
        if (h->persistent && h->B.pgridCg > 0)
            e = ppeSolvePersistent(h->d, h->B, 0, h->tol, maxIt, h->s, &fi, &fr, &rr, &rr0, &h->prof);
        else
            e = ppeSolvePlain(h->d, h->B, h->tol, maxIt, h->s, &fi, &rr, &rr0, &h->prof);
        if (e == MPSGPU_ERR_CUDA) g_lastError = "PPE fallback solve: launch failed or a grid-barrier wait ran out";
        iters += fi;
        h->last.ppeFallback = 1;
        h->last.runPpeFallbacks += 1;
    }
    cudaEventRecord(h->es1, h->s);
    if (h->mlp.recording && !e) {
        // features of this system with the previous solution, target = converged - previous
        if (!h->B.prepared) { launchMixedPrepare(h->d, h->B, h->s); h->B.prepared = 1; }   // features read valf
        int er = mlpRecordFeatures(h->mlp, h->d, h->B, h->s);
        if (!er) er = mlpRecordTargets(h->mlp, h->d, h->B, h->s);
        if (er) return er;
    }
    launchPpeCopyBack(h->d, h->B, h->s);
    h->last.ppeIterations = iters;
    h->last.ppeRefinements = refine;
    h->last.runPpeSolves += 1;
    h->last.runPpeIterations += iters;
    h->last.runPpeRefinements += refine;
    h->last.ppeRelResidual = rr;
    h->last.ppeInitialRelResidual = rr0;
    CK(cudaEventSynchronize(h->es1));
    float ms = 0;
    cudaEventElapsedTime(&ms, h->es0, h->es1);
    h->last.ppeSolveMs = ms;
    cudaEventElapsedTime(&ms, h->ea0, h->ea1);
    h->last.ppeAssembleMs = ms;
    if (e == MPSGPU_ERR_NOT_CONVERGED) g_lastError = "PPE solver did not reach the tolerance";
    int ls = launchStatus();
    return e ? e : ls;
}

static int runOpBody(mpsgpu_t h, int op);
static int runOpImpl(mpsgpu_t h, int op) {
    if (op < 0 || op >= MPS_OP_COUNT) { g_lastError = "unknown operator"; return MPSGPU_ERR_ARG; }
    bool pr = h->prof.on && op != MPS_OP_INIT_PND;
    if (pr) h->prof.begin(op, h->s);
    int e = runOpBody(h, op);
    if (pr) h->prof.end(h->s);
    if (!h->opSkipped) countLaunch(opLaunches(op, h->d.P, h->d.prec == MPSGPU_PRECISION_DF32));
    h->opSkipped = false;
    return e;
}
static int runOpBody(mpsgpu_t h, int op) {
    Dev& d = h->d;
    const MpsParams& P = d.P;
    cudaStream_t s = h->s;
    auto invalidate = [&]() {
        h->listValid = false; h->masksValid = false; h->cacheValid = false; h->corrFresh = false;
    };
    const bool x = df32(h);
    switch (op) {
        case MPS_OP_UPDATE_BUCKETS: {
            bool rn = h->renumberEvery > 0 && h->renumberCountdown <= 0;
            launchBuckets(d, h->scanScratch, s, rn ? h->perm : nullptr, h->permScratch);
            if (rn) { h->renumberCountdown = h->renumberEvery; countLaunch(renumberLaunches()); }
            h->renumberCountdown--;
            invalidate();
            h->skinValid = false;
            h->skinShift = false;
            break;
        }
        case MPS_OP_VISCOSITY:
            if (h->skinOn) {
                // start-of-step list with a skin: the viscosity sweep reads it, and the list of
                // the predicted positions is filtered from it (ensureList); in the FP64 tier
                // the sweep and the filter keep the bucket scan's FP64 arithmetic and order
                if (h->prof.on) { h->prof.end(s); h->prof.begin(PROF_NEIGHBOR_LIST, s, false); }
                launchSkinListDF(d, s);
                if (h->prof.on) { h->prof.end(s); h->prof.begin(MPS_OP_VISCOSITY, s, false); }
                if (x) launchViscosityListDF(d, s);
                else launchViscosityList(d, s);
                invalidate();
                // the skin list keeps its arrays; the lists filtered from it go to the others
                d.skinNbr = d.nbr;
                d.skinCnt = d.nbrCount;
                std::swap(d.nbr, h->nbrAlt);
                std::swap(d.nbrCount, h->cntAlt);
                h->skinValid = true;
                h->skinShift = true;   // the shifting sweeps filter the kept skin list again
                countLaunch(2);   // skin list (listed + unlisted particles); the sweep is counted below
            } else if (x) launchViscosityDF(d, s);
            else launchViscosity(d, s);
            break;
        case MPS_OP_ADD_GRAVITY: launchAddGravity(d, s); break;
        case MPS_OP_PREDICT_PRESS_GRADIENT:
            // FP64 in both tiers, over the start-of-step skin list while it is built for
            // these positions (else the bucket scan)
            if (P.relaxPress < 1.0) launchPredictPressGradient(d, h->skinValid, s);
            break;
        case MPS_OP_PREDICT: launchPredict(d, s); invalidate(); break;
        case MPS_OP_OUT_OF_DOMAIN:
            launchOutOfDomain(d, h->outFlags, h->outCounter, s);
            invalidate();
            h->nHost = -1;   // removals change the live count on the device
            break;
        case MPS_OP_COLLISION:
            ensureList(h);
            if (P.collisionType == 1) {   // DPC moves the positions: every list is stale
                launchCollisionDPC(d, s);
                invalidate();
            } else if (x) launchCollisionDF(d, s);
            else launchCollision(d, s);
            break;
        case MPS_OP_WALL_DISTANCE: launchWallDistance(d, s); h->masksValid = false; h->corrFresh = false; break;
        case MPS_OP_WALL_NPCD: ensureMasks(h); if (x) launchWallNpcdDF(d, s); else launchWallNpcd(d, s); break;
        case MPS_OP_CORRECTION_MATRIX:
            ensureMasks(h);
            if (x && h->corrFresh && h->masksValid) {   // formed by the PND sweep: publish it
                std::swap(d.c1, d.c1n); std::swap(d.c2, d.c2n); std::swap(d.c3, d.c3n);
                std::swap(d.corrDF, d.corrDFn);
                h->corrFresh = false;
                h->opSkipped = true;
                break;
            }
            if (x) launchCorrectionMatrixDF(d, s); else launchCorrectionMatrix(d, s);
            break;
        case MPS_OP_PND_NEIGH_NPCD: {
            ensureMasks(h);
            // the correction matrix of the step (read after the pressure solve, positions and
            // masks unchanged in between) is formed in the same pass
            bool corr = x && P.gradientCorrection && P.pndType != 2;
            if (x) launchPndNeighNpcdDF(d, s, corr); else launchPndNeighNpcd(d, s);
            h->corrFresh = corr;
            break;
        }
        case MPS_OP_PND_DIFFUSIVE: ensureMasks(h); ensureCache(h); launchPndDiffusive(d, s); break;
        case MPS_OP_PND_MEAN: ensureMasks(h); ensureCache(h); launchPndMean(d, s); break;
        case MPS_OP_UPDATE_BC:
            if (P.freeSurfType == 2) { ensureMasks(h); launchUpdateBCArc(d, s); }
            else launchUpdateBC(d, s);
            break;
        case MPS_OP_CALC_PRESS: { int e = calcPress(h); if (e) return e; break; }
        case MPS_OP_EXTRAPOLATE_PRESS: ensureMasks(h); ensureCache(h); launchExtrapolatePress(d, s); break;
        case MPS_OP_PRESS_GRADIENT: ensureMasks(h); if (x) launchPressGradientDF(d, s); else launchPressGradient(d, s); break;
        case MPS_OP_WALL_PRESS_GRADIENT:
            ensureMasks(h);
            if (x) launchWallPressGradientDF(d, s); else launchWallPressGradient(d, s);
            break;
        case MPS_OP_WALL_VISCOSITY: ensureMasks(h); if (x) launchWallViscosityDF(d, s); else launchWallViscosity(d, s); break;
        case MPS_OP_CORRECT: launchCorrect(d, s); invalidate(); break;
        case MPS_OP_SHIFTING:
            if (x && h->skinShift && (P.shiftingType == 1 || P.shiftingType == 2)) {
                // the list of the post-corrector positions filtered from the skin list (a
                // particle that moved out of its skin or scan window, or any particle after a
                // removal, scans the buckets), its masks, then list sweeps
                if (h->prof.on) { h->prof.end(s); h->prof.begin(PROF_NEIGHBOR_LIST, s, false); }
                launchNeighborFilterDF(d, s);
                launchSideMasksDF(d, s);
                if (h->prof.on) { h->prof.end(s); h->prof.begin(MPS_OP_SHIFTING, s, false); }
                launchShiftingListDF(d, s);
                invalidate();
                // posf + cell copy, skin check, filter (2), masks; then the sweeps and applies
                countLaunch(6 + (P.shiftingType == 1 ? 3 : (P.wallType == 1 ? 7 : 4)));
                h->opSkipped = true;
            } else if (!x && h->skinShift && (P.shiftingType == 1 || P.shiftingType == 2)) {
                // FP64: the same list (no weight cache), then the operators' sweeps over it
                if (h->prof.on) { h->prof.end(s); h->prof.begin(PROF_NEIGHBOR_LIST, s, false); }
                launchNeighborFilter(d, s, false);
                if (h->prof.on) { h->prof.end(s); h->prof.begin(MPS_OP_SHIFTING, s, false); }
                launchShifting(d, s, true);
                invalidate();
                // posf + cell copy, skin check, filter; then the sweeps and applies
                countLaunch(4 + (P.shiftingType == 1 ? 2 : (P.wallType == 1 ? 6 : 3)));
                h->opSkipped = true;
            } else {
                if (x) launchShiftingDF(d, s); else launchShifting(d, s, false);
                if (P.shiftingType == 2) invalidate();
            }
            break;
        case MPS_OP_DUMMY_VELOCITY: launchDummyVelocity(d, s); break;
        case MPS_OP_INIT_PND: ensureMasks(h); ensureCache(h); launchInitPnd(d, s); break;
        default: g_lastError = "unknown operator"; return MPSGPU_ERR_ARG;
    }
    return launchStatus();
}

static int stepImpl(mpsgpu_t h) {
    const MpsParams& P = h->d.P;
    int e;
#define RUN(op) do { if ((e = runOpImpl(h, op))) return e; } while (0)
    RUN(MPS_OP_UPDATE_BUCKETS);
    RUN(MPS_OP_VISCOSITY);
    RUN(MPS_OP_ADD_GRAVITY);
    if (P.relaxPress < 1.0) RUN(MPS_OP_PREDICT_PRESS_GRADIENT);
    RUN(MPS_OP_PREDICT);
    RUN(MPS_OP_OUT_OF_DOMAIN);
    // The wall distance reads the positions left by the out-of-domain removal and writes only
    // the wall fields (squared distance, wall point, mirror, normal, near-wall flag, wall PND
    // and neighbour count).  The list filter reads none of them; the collision reads only the
    // mirror, in its mirror-side test, and every mirror is still the far point the prediction
    // wrote, for which the test passes for every pair.  So the collision skips the test
    // (mirrorFar) and the wall distance runs on the second stream beside the filter and the
    // collision, joined before the wall PND.  DPC moves the positions: it keeps the order.
    const bool side = P.wallType == 1 && P.collisionType != 1 && h->d.ntri > 0;
    if (side) {
        cudaEventRecord(h->evFork, h->s);
        cudaStreamWaitEvent(h->s2, h->evFork, 0);
        if (h->prof.on) h->prof.begin(MPS_OP_WALL_DISTANCE, h->s2);
        launchWallDistance(h->d, h->s2);
        if (h->prof.on) h->prof.end(h->s2);
        cudaEventRecord(h->evJoin, h->s2);
        countLaunch(opLaunches(MPS_OP_WALL_DISTANCE, P, df32(h)));
        if ((e = launchStatus())) { cudaStreamWaitEvent(h->s, h->evJoin, 0); return e; }
    }
    ensureList(h);                       // post-prediction neighbour list
    h->d.mirrorFar = side ? 1 : 0;
    e = runOpImpl(h, MPS_OP_COLLISION);
    h->d.mirrorFar = 0;
    if (side) {
        cudaStreamWaitEvent(h->s, h->evJoin, 0);
        h->masksValid = false;   // as the wall-distance operator leaves them
        h->corrFresh = false;
    }
    if (e) return e;
    if (P.wallType == 1) {
        if (!side) RUN(MPS_OP_WALL_DISTANCE);
        RUN(MPS_OP_WALL_NPCD);
    }
    // The first correctionMatrix call (src/main.cpp:317-319) is read only by the diffusive
    // PND and the velocity divergence of the PND + div u source; otherwise the second call
    // (src/main.cpp:375-377, same positions) overwrites it.
    if (P.gradientCorrection && (P.pndType == 2 || P.mpsType == 3)) RUN(MPS_OP_CORRECTION_MATRIX);
    RUN(MPS_OP_PND_NEIGH_NPCD);
    if (P.pndType == 2) RUN(MPS_OP_PND_DIFFUSIVE);
    else if (P.pndType == 1) RUN(MPS_OP_PND_MEAN);
    RUN(MPS_OP_UPDATE_BC);
    RUN(MPS_OP_CALC_PRESS);
    if (P.wallType == 0) RUN(MPS_OP_EXTRAPOLATE_PRESS);
    if (P.gradientCorrection) RUN(MPS_OP_CORRECTION_MATRIX);
    RUN(MPS_OP_PRESS_GRADIENT);
    if (P.wallType == 1) { RUN(MPS_OP_WALL_PRESS_GRADIENT); RUN(MPS_OP_WALL_VISCOSITY); }
    RUN(MPS_OP_CORRECT);
    RUN(MPS_OP_OUT_OF_DOMAIN);
    if (P.shiftingType != 0) RUN(MPS_OP_SHIFTING);
    if (P.wallType == 0) RUN(MPS_OP_DUMMY_VELOCITY);
    RUN(MPS_OP_OUT_OF_DOMAIN);
#undef RUN
    if (h->prof.on && (e = h->prof.flush())) return e;
    h->numIter++;
    h->timeCurrent += P.timeStep;
    return 0;
}

static int finishStats(mpsgpu_t h, MpsStepStats* st, float stepMs) {
    double vmax = 0;
    int n = 0;
    unsigned long long cnt[2] = {0, 0};
    CK(cudaMemcpyAsync(&vmax, h->d.velMax, sizeof(double), cudaMemcpyDeviceToHost, h->s));
    CK(cudaMemcpyAsync(&n, h->d.nLive, sizeof(int), cudaMemcpyDeviceToHost, h->s));
    CK(cudaMemcpyAsync(cnt, h->d.counters, sizeof(cnt), cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    h->last.nbrEntries = (long long)cnt[0];
    h->last.ppeNnz = (h->d.P.mpsType == 2 || h->d.P.mpsType == 3) ? (long long)cnt[1] + n : 0;
    h->last.velMax = vmax;
    h->last.CFLcurrent = h->d.P.timeStep * vmax / h->d.P.partDist;
    h->last.numParticles = n;
    h->nHost = n;
    h->last.stepMs = stepMs;
    if (st) *st = h->last;
    return 0;
}

// Field transfers are in reference order; storage is in bucket order (mps_common.cuh).
template <class T>
__global__ void k_to_ref(const T* src, T* dst, const int* slotOf, int n) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) dst[r] = src[slotOf[r]];
}
template <class T>
__global__ void k_from_ref(const T* src, T* dst, const int* slotOf, int n) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) dst[slotOf[r]] = src[r];
}
// vector fields: storage dvec4 <-> the reference's interleaved N x 3 doubles, in one pass
__global__ void k_vec_to_ref(const dvec4* src, double* dst, const int* slotOf, int n) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    dvec4 v = src[slotOf[r]];
    dst[3 * r] = v.x; dst[3 * r + 1] = v.y; dst[3 * r + 2] = v.z;
}
__global__ void k_vec_from_ref(const double* src, dvec4* dst, const int* slotOf, int n) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    dst[slotOf[r]] = make_dvec4(src[3 * r], src[3 * r + 1], src[3 * r + 2], 0.0);
}
static void toRef(mpsgpu_t h, int kind, const void* p, int n) {
    void* sc = h->permScratch;
    if (kind == 0) k_vec_to_ref<<<gridFor(n, 256), 256, 0, h->s>>>((const dvec4*)p, (double*)sc, h->d.slotOf, n);
    else if (kind == 1) k_to_ref<double><<<gridFor(n, 256), 256, 0, h->s>>>((const double*)p, (double*)sc, h->d.slotOf, n);
    else k_to_ref<int><<<gridFor(n, 256), 256, 0, h->s>>>((const int*)p, (int*)sc, h->d.slotOf, n);
    countLaunch(1);
}
static void fromRef(mpsgpu_t h, int kind, void* p, int n) {
    const void* sc = h->permScratch;
    if (kind == 0) k_vec_from_ref<<<gridFor(n, 256), 256, 0, h->s>>>((const double*)sc, (dvec4*)p, h->d.slotOf, n);
    else if (kind == 1) k_from_ref<double><<<gridFor(n, 256), 256, 0, h->s>>>((const double*)sc, (double*)p, h->d.slotOf, n);
    else k_from_ref<int><<<gridFor(n, 256), 256, 0, h->s>>>((const int*)sc, (int*)p, h->d.slotOf, n);
    countLaunch(1);
}

// ------------------------------------------------------------------ binary .vtu output
// Arrays of the appended block in the reference's particle order (slotOf maps a reference
// index to its storage slot), converted as the ASCII writer converts them ((float) casts).
__global__ void k_vtu_vec(const dvec4* src, const int* slotOf, int n, float* dst) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    dvec4 v = src[slotOf[r]];
    dst[3 * r] = (float)v.x; dst[3 * r + 1] = (float)v.y; dst[3 * r + 2] = (float)v.z;
}
__global__ void k_vtu_sca(const double* src, const int* slotOf, int n, float* dst) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) dst[r] = (float)src[slotOf[r]];
}
__global__ void k_vtu_int(const int* src, const int* slotOf, int n, int* dst, int add) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) dst[r] = src ? src[slotOf[r]] : r + add;   // src == NULL: r + add (connectivity, offsets)
}
__global__ void k_vtu_u8(int n, unsigned char* dst, unsigned char v) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) dst[r] = v;
}

extern "C" {

int mpsgpu_params_derive(MpsParams* p, int n, const double* pos3) {
    int e = hostDeriveParams(p, n, pos3);
    if (e) g_lastError = "parameter derivation failed (dimension/limits)";
    return e;
}

const char* mpsgpu_last_error(mpsgpu_t h) {
    (void)h;
    return g_lastError.c_str();
}

int mpsgpu_profile(mpsgpu_t h, int enable) {
    if (!h) return MPSGPU_ERR_ARG;
    int e = h->prof.flush();
    h->prof.reset();
    h->prof.on = enable != 0;
    return e;
}

int mpsgpu_profile_get(mpsgpu_t h, int cls, double* ms, long long* calls) {
    if (!h || cls < 0 || cls >= PROF_NCLASS) return MPSGPU_ERR_ARG;
    int e = h->prof.flush();
    if (ms) *ms = h->prof.ms[cls];
    if (calls) *calls = h->prof.calls[cls];
    return e;
}

const char* mpsgpu_profile_name(int cls) {
    static const char* ops[] = {"UPDATE_BUCKETS", "VISCOSITY", "ADD_GRAVITY", "PREDICT", "OUT_OF_DOMAIN",
                                "COLLISION", "WALL_DISTANCE", "WALL_NPCD", "CORRECTION_MATRIX", "PND_NEIGH_NPCD",
                                "PND_DIFFUSIVE", "PND_MEAN", "UPDATE_BC", "CALC_PRESS", "EXTRAPOLATE_PRESS",
                                "PRESS_GRADIENT", "WALL_PRESS_GRADIENT", "WALL_VISCOSITY", "CORRECT", "SHIFTING",
                                "DUMMY_VELOCITY", "INIT_PND", "PREDICT_PRESS_GRADIENT"};
    static const char* extra[] = {"NEIGHBOR_LIST", "PPE_ASSEMBLE", "PPE_SPMV", "PPE_VECTOR", "PPE_OTHER", "PPE_SOLVE"};
    static_assert(sizeof(ops) / sizeof(ops[0]) == MPS_OP_COUNT, "operator names");
    if (cls >= 0 && cls < MPS_OP_COUNT) return ops[cls];
    if (cls >= MPS_OP_COUNT && cls < PROF_NCLASS) return extra[cls - MPS_OP_COUNT];
    return "";
}

int mpsgpu_launch_count(long long* n) {
    if (!n) return MPSGPU_ERR_ARG;
    *n = launchCount();
    return 0;
}

int mpsgpu_abi_sizes(int* params, int* stats, int* mesh) {
    if (params) *params = (int)sizeof(MpsParams);
    if (stats) *stats = (int)sizeof(MpsStepStats);
    if (mesh) *mesh = (int)sizeof(MpsMesh);
    return 0;
}

int mpsgpu_create(const MpsParams* p, int n, const int* type, const double* pos3, const double* vel3,
                  const double* press, const MpsMesh* mesh, mpsgpu_t* out) {
    if (!p || !p->derived || n <= 0 || !type || !pos3 || !out) { g_lastError = "bad argument"; return MPSGPU_ERR_ARG; }
    if (int e = mpsgpu_check_params(p)) return e;
    if (p->wallType == 1 && (!mesh || mesh->ntri <= 0 || !mesh->tri_xyz)) { g_lastError = "polygon walls need a mesh"; return MPSGPU_ERR_ARG; }
    if (mesh && mesh->ntri > (1 << 26)) { g_lastError = "mesh too large"; return MPSGPU_ERR_UNSUPPORTED; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { g_lastError = "no CUDA device"; return MPSGPU_ERR_NOGPU; }
    mpsgpu_t h = new mpsgpu_s();
    h->N0 = n;
    cudaError_t ce = cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking);
    if (ce != cudaSuccess) { g_lastError = cudaGetErrorString(ce); delete h; return MPSGPU_ERR_CUDA; }
    for (cudaEvent_t* ev : {&h->e0, &h->e1, &h->ea0, &h->ea1, &h->es0, &h->es1}) cudaEventCreate(ev);
    if (cudaStreamCreateWithFlags(&h->s2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->evFork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->evJoin, cudaEventDisableTiming) != cudaSuccess) {
        g_lastError = "second stream of the step";
        mpsgpu_destroy(h);
        return MPSGPU_ERR_CUDA;
    }
    Dev& d = h->d;
    std::memset(&d, 0, sizeof(d));
    d.P = *p;
    d.N0 = n;
    d.invSidef = (float)p->invBucketSide;
    d.epsf = (float)p->epsilonZero;
    d.dz3 = (int)(p->dim - 2.0);
    for (int k = 0; k < 3; k++) {
        d.oodLo[k] = p->domainMin[k] + p->bucketSide;
        d.oodHi[k] = p->domainMax[k] - p->bucketSide;
    }
    d.nB = p->numBucketsXYZ;
    d.K = ((int)p->dim == 3) ? 128 : 64;   // entries per neighbour row (compressed flows reach ~2x the rest count)
    int e = 0;
#define A(ptr, cnt) do { if ((e = dalloc(h, &(ptr), (cnt)))) { mpsgpu_destroy(h); return e; } } while (0)
    A(d.nLive, 1);
    for (dvec4** v : {&d.pos, &d.vel, &d.acc, &d.accStar, &d.mirror, &d.wallPos, &d.polyNormal, &d.npcd, &d.gradC,
                        &d.forceWall, &d.c1, &d.c2, &d.c3, &d.dvel, &d.shift})
        A(*v, n);
    for (double** v : {&d.press, &d.pressPPE, &d.pndi, &d.pndki, &d.pndski, &d.pndSmall, &d.npcd2, &d.conc, &d.velDiv,
                       &d.diffTerm, &d.pndWall, &d.riw2, &d.devDot, &d.source, &d.aux1, &d.aux2})
        A(*v, n);
    for (int** v : {&d.type, &d.bc, &d.numNeigh, &d.nNeighWall, &d.nearWall}) A(*v, n);
    A(d.posf, n);
    A(d.pressPPEprev, n);
    A(d.pressPPEprev2, n);
    A(d.cellOf, n);
    A(d.cellStart, d.nB + 2);
    A(d.cellCount, d.nB + 2);
    A(d.cellCursor, d.nB + 2);
    A(d.orig, n);
    A(d.slotOf, n);
    A(d.cellPos, n);
    A(h->perm, n);
    {
        double* sc = nullptr;   // 32 bytes per particle: the widest per-particle element
        A(sc, (size_t)4 * n);
        h->permScratch = sc;
    }
    A(d.cellSorted, n);
    A(d.posfCell, n);
    A(d.posLo, n);
    A(d.posLoCell, n);
    A(d.velHi, n);
    A(d.velLo, n);
    A(d.pressDF, n);
    A(d.concDF, n);
    A(d.normal, n);
    A(d.posSkin, n);
    A(d.skinCell, n);
    A(d.skinFlag, 2);
    A(d.corrDF, (size_t)9 * n);
    A(d.corrDFn, (size_t)9 * n);
    A(d.c1n, n);
    A(d.c2n, n);
    A(d.c3n, n);
    A(d.nbrCount, n);
    A(d.nbr, (size_t)d.K * n);
    A(h->cntAlt, n);
    A(h->nbrAlt, (size_t)d.K * n);
    d.skinCnt = d.nbrCount;
    d.skinNbr = d.nbr;
    A(d.cw, (size_t)d.K * n);
    A(d.cwd, (size_t)d.K * n);
    if (p->reS2 != p->reL2) A(d.cwL, (size_t)d.K * n);
    A(d.maskS, n);
    A(d.maskL, n);
    A(d.nearList, n);
    A(d.nearCount, 1);
    A(d.velMax, 1);
    A(d.err, 1);
    A(d.counters, 4);
    A(h->scanScratch, scanScratchInts(std::max(d.nB + 1, n)));
    A(h->outFlags, n);
    cudaMemsetAsync(h->outFlags, 0, sizeof(int) * n, h->s);
    A(h->outCounter, 1);
    // FP32 prefilter band (see k_build_nbr): |d2f - d2| <= 3.47 delta re + 3 delta^2 + 3.1 u re^2
    {
        double X = 0;
        for (int k = 0; k < 3; k++) X = std::max(X, p->domainMax[k] - p->domainMin[k]);
        X += 4.0 * p->bucketSide;
        double u = std::ldexp(1.0, -24);
        auto band = [&](double re2) {
            double re = std::sqrt(re2);
            double delta = u * (2.0 * X + 2.0 * re);
            return 2.0 * (3.47 * delta * re + 3.0 * delta * delta + 3.1 * u * re2);
        };
        d.reMax2 = std::max(p->reS2, p->reL2);
        d.reL2f = (float)d.reMax2;
        d.bandLo = (float)(d.reMax2 - band(d.reMax2));
        d.bandHi = (float)(d.reMax2 + band(d.reMax2));
        d.bandHiS = (float)(p->reS2 + band(p->reS2));
        d.bandHiL = (float)(p->reL2 + band(p->reL2));
        d.bandHiColl = (float)(p->distCollisionLimit2 + band(p->distCollisionLimit2));
        // start-of-step skin list: reMax + 0.15 l0 (covers steps that move no particle by
        // more than 0.075 l0 from its start position; otherwise the list is rebuilt)
        {
            double skin = 0.15 * p->partDist;
            double rs = std::sqrt(d.reMax2) + skin;
            d.skinR2 = (float)(rs * rs + band(rs * rs));
            double mv = 0.5 * skin - 8.0 * std::ldexp(1.0, -24) * X;   // FP32 hi-part error of both copies
            d.skinMove2 = (float)(mv > 0.0 ? mv * mv : 0.0);
        }
        // float-float squared distances: each coordinate difference is within
        // 4 * 2^-48 * X of the FP64 one (storage of both lo parts, the rounded lo difference
        // and the reference's own rounding), the float-float products and sums add about
        // 2^-44 relative; the margin is 8x that bound.
        auto margin = [&](double re2) {
            double re = std::sqrt(re2);
            double ddx = 4.0 * std::ldexp(1.0, -48) * X;
            return (float)(8.0 * (2.0 * std::sqrt(3.0) * re * ddx + std::ldexp(1.0, -40) * re2));
        };
        d.mgS = margin(p->reS2);
        d.mgL = margin(p->reL2);
        d.mgMax = margin(d.reMax2);
        d.mgColl = margin(std::max(p->distCollisionLimit2, 1e-300));
        d.mgSide = margin(3.3 * 3.3 * d.reMax2);
        d.prec = MPSGPU_PRECISION_FP64;
        // float-float constants: hi = fl32(x), lo = fl32(x - hi) (as the device converts)
        auto hd = [](double x) { float h = (float)x; return make_float2(h, (float)(x - (double)h)); };
        Dev::DfK& k = d.k;
        k.reS = hd(p->reS); k.reL = hd(p->reL);
        k.invReS = hd(1.0 / p->reS); k.invReL = hd(1.0 / p->reL);
        k.reS2 = hd(p->reS2); k.reL2 = hd(p->reL2); k.reMax2 = hd(d.reMax2);
        k.coll2 = hd(p->distCollisionLimit2);
        double mu = p->KNM_VS1 * p->DNS_FL1, rho = p->DNS_FL1;
        k.neuW = hd((2.0 * mu) / rho);
        k.neuF = hd((2.0 * mu * mu / (mu + mu)) / rho);
        k.neuWall = hd(((mu + mu) > p->epsilonZero ? 2.0 * mu * mu / (mu + mu) : 0.0) / p->DNS_FL1);
        k.cPPE = hd(p->coeffPPE);
        k.cPPEg = hd(p->coeffPPE * p->DNS_FL1);
        for (int c = 0; c < 3; c++) k.g[c] = hd(p->gravity[c]);
        k.collF = hd(p->restitutionCollision * p->DNS_FL1 / (p->DNS_FL1 + p->DNS_FL1));
        k.collW = hd(p->restitutionCollision * p->densityWall / (p->DNS_FL1 + p->densityWall));
        k.negCPG = hd(-p->coeffPressGrad);
    }
    if (d.K > 128) { g_lastError = "neighbour row capacity above the 128-entry masks"; mpsgpu_destroy(h); return MPSGPU_ERR_UNSUPPORTED; }
    // mesh and wall tables
    if (p->wallType == 1) {
        std::vector<double> nrm(3 * mesh->ntri), pln(16 * mesh->ntri), tab(4 * MPS_TAB);
        hostTriNormals(mesh->ntri, mesh->tri_xyz, nrm.data());
        hostTrianglePlanes(mesh->ntri, mesh->tri_xyz, pln.data());
        hostWallTables(*p, tab.data());
        double *dt = nullptr, *dn = nullptr, *dp = nullptr, *dtab = nullptr;
        A(dt, 9 * mesh->ntri);
        A(dn, 3 * mesh->ntri);
        A(dp, 16 * mesh->ntri);
        A(dtab, 4 * MPS_TAB);
        cudaMemcpyAsync(dt, mesh->tri_xyz, sizeof(double) * 9 * mesh->ntri, cudaMemcpyHostToDevice, h->s);
        cudaMemcpyAsync(dn, nrm.data(), sizeof(double) * nrm.size(), cudaMemcpyHostToDevice, h->s);
        cudaMemcpyAsync(dp, pln.data(), sizeof(double) * pln.size(), cudaMemcpyHostToDevice, h->s);
        cudaMemcpyAsync(dtab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, h->s);
        d.tri = dt; d.triNormal = dn; d.triPlane = dp; d.tab = dtab; d.ntri = mesh->ntri;
        // the reference interpolates at sqrt(reS2) and sqrt(reL2) (src/PolygonMesh.cpp:694-701);
        // both square roots are correctly rounded, so these are the device's values
        d.wallReS = std::sqrt(p->reS2);
        d.wallReL = std::sqrt(p->reL2);
        if (mesh->ntri > MPS_MAX_TRI) {
            // large mesh: triangle BVH (host build, FP32 boxes) and FP32 triangle copies
            std::vector<float> lo4, hi4, tf(9 * (size_t)mesh->ntri);
            std::vector<int> order;
            hostBuildBvh(mesh->ntri, mesh->tri_xyz, p->domainMin, lo4, hi4, order);
            for (size_t k = 0; k < tf.size(); k++) tf[k] = (float)(mesh->tri_xyz[k] - p->domainMin[k % 3]);
            float *blo = nullptr, *bhi = nullptr, *btf = nullptr;
            int* bord = nullptr;
            A(blo, lo4.size());
            A(bhi, hi4.size());
            A(bord, order.size());
            A(btf, tf.size());
            cudaMemcpyAsync(blo, lo4.data(), sizeof(float) * lo4.size(), cudaMemcpyHostToDevice, h->s);
            cudaMemcpyAsync(bhi, hi4.data(), sizeof(float) * hi4.size(), cudaMemcpyHostToDevice, h->s);
            cudaMemcpyAsync(bord, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice, h->s);
            cudaMemcpyAsync(btf, tf.data(), sizeof(float) * tf.size(), cudaMemcpyHostToDevice, h->s);
            d.bvhLo = (const float4*)blo; d.bvhHi = (const float4*)bhi; d.bvhOrder = bord; d.triF = btf;
        }
        cudaStreamSynchronize(h->s);
    }
    // PPE buffers
    PpeBuffers& B = h->B;
    std::memset(&B, 0, sizeof(B));
    // ELL rows padded to whole 256-row tiles: every slice of a tile is a 16-byte aligned,
    // in-bounds range for the bulk copies of the staged SpMV.  Layout: slices of 1024 rows,
    // each slice's entries column-major inside it, so the entries of a row lie 4 KB apart
    // (column-major over all rows they lie N0 x 4 B apart: 37 MB at 9.4M rows, where the
    // sliced layout measured 16.6 against 22.1 ms per solve; equal at 864k).
    // MPSGPU_ELL_SLICE = s selects 2^s rows per slice (8 <= s <= 20), 0 the column-major layout.
    B.K = d.K;
    B.sliceShift = 10; B.sliceMask = (1 << 10) - 1;
    if (const char* env = std::getenv("MPSGPU_ELL_SLICE")) {
        const int sh = std::atoi(env);
        if (sh == 0) { B.sliceShift = 31; B.sliceMask = 0x7fffffff; }
        else if (sh >= 8 && sh <= 20) { B.sliceShift = sh; B.sliceMask = (1 << sh) - 1; }
    }
    const int pad = B.sliceShift < 31 ? (1 << B.sliceShift) : 256;
    B.N0 = (n + pad - 1) / pad * pad;
    B.ellStride = B.sliceShift < 31 ? (size_t)1 << B.sliceShift : (size_t)B.N0;
    const size_t ell = (size_t)d.K * B.N0;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    B.nblocks = std::max(1, sms) * 8;
    if (p->mpsType == 2 || p->mpsType == 3) {
        for (double** v : {&B.diag, &B.x, &B.b, &B.r, &B.z, &B.p, &B.Ap, &B.bs[0], &B.bs[1], &B.bs[2], &B.bs[3]})
            A(*v, n);
        A(B.val, ell);
        A(B.col, ell);
        A(B.rowLen, n);
        A(B.valf, ell);
        for (float** v : {&B.diagf, &B.diagInvf, &B.rf, &B.zf, &B.pf, &B.Apf, &B.xf, &B.wf, &B.qzf, &B.mf2}) A(*v, n);
        A(B.xalt, n);
        B.pgridCg = ppePersistentGrid(0);
        B.pgridMx = ppePersistentGrid(1);
        A(B.scal, 32);
            A(B.partials, 8 * std::max(std::max(std::max(B.nblocks, ppePersistentGrid(4)), ppePersistentGrid(3)),
                                   std::max(std::max(B.pgridCg, std::max(ppePersistentGrid(5), ppePersistentGrid(6))),
                                            std::max(B.pgridMx, ppePersistentGrid(2)))));
        A(B.counter, 1);
        A(B.flag, 8);
        A(B.dinv, n);
        A(B.mfMask, n);
        B.pgridMf = ppePersistentGrid(2);
        B.pgridH16 = ppePersistentGrid(3);
        B.pgridTs = ppePersistentGrid(4);
        B.pgridPipe = ppePersistentGrid(5);
        B.pgridBi = ppePersistentGrid(6);
        // the staged tiles keep up to 128 tile lengths per block in shared memory
        if (B.pgridTs > 0 && (n + 255) / 256 > 128 * B.pgridTs) B.pgridTs = 0;
        A(B.valh, ell);
        A(B.col16, ell);
        A(B.sclf, n);
        A(B.sgs, n);
        A(B.wideRow, n);
        A(B.bar, 96);   // three 128-byte lines of barrier words
        // solver vectors in shared memory: a block's rows are its grid-stride rounds, at
        // most n / (G BS) + 1 of them per thread (the remainder is split over the blocks)
        B.pgridOwn = ppePersistentGrid(7);
        if (B.pgridOwn > 0) {
            const long long slots = ((long long)n / ((long long)B.pgridOwn * 1024) + 1) * 1024;
            if (slots <= OWN_CAP_ROWS) B.ownCap = (int)slots;
            else B.pgridOwn = 0;
        }
        B.pgridOwn64 = ppePersistentGrid(8);
        if (B.pgridOwn64 > 0) {
            const long long slots = ((long long)n / ((long long)B.pgridOwn64 * 768) + 1) * 768;
            if (slots <= OWN64_CAP_ROWS) B.ownCap64 = (int)slots;
            else B.pgridOwn64 = 0;
        }
    }
#undef A
    // upload the particle state (src/MpsInputOutput.cpp:759-856 initial values)
    std::vector<dvec4> v4(n);
    auto up4 = [&](dvec4* dst, const double* src3, double fill) {
        for (int i = 0; i < n; i++)
            v4[i] = src3 ? make_dvec4(src3[3 * i], src3[3 * i + 1], src3[3 * i + 2], 0.0)
                         : make_dvec4(fill, fill, fill, 0.0);
        cudaMemcpy(dst, v4.data(), sizeof(dvec4) * n, cudaMemcpyHostToDevice);
    };
    up4(d.pos, pos3, 0.0);
    up4(d.vel, vel3, 0.0);
    cudaMemcpy(d.type, type, sizeof(int) * n, cudaMemcpyHostToDevice);
    if (press) cudaMemcpy(d.press, press, sizeof(double) * n, cudaMemcpyHostToDevice);
    std::vector<double> big(n, 10e8 * p->partDist);
    cudaMemcpy(d.riw2, big.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(d.nLive, &n, sizeof(int), cudaMemcpyHostToDevice);
    {
        std::vector<int> id(n);
        for (int i = 0; i < n; i++) id[i] = i;   // storage starts in reference order
        cudaMemcpy(d.orig, id.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
        cudaMemcpy(d.slotOf, id.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
    }
    if (cudaDeviceSynchronize() != cudaSuccess || launchStatus()) { mpsgpu_destroy(h); return MPSGPU_ERR_CUDA; }
    h->maxIter = 0;
    if ((e = mlpInit(h->mlp, n, h->s))) { mpsgpu_destroy(h); return e; }
    *out = h;
    return 0;
}

int mpsgpu_destroy(mpsgpu_t h) {
    if (!h) return MPSGPU_ERR_ARG;
    if (h->s) cudaStreamSynchronize(h->s);
    if (h->s2) cudaStreamSynchronize(h->s2);
    mlpFree(h->mlp);
    h->prof.destroy();
    for (void* p : h->allocs) cudaFree(p);
    if (h->vtuDev) cudaFree(h->vtuDev);
    if (h->vtuHost) cudaFreeHost(h->vtuHost);
    for (cudaEvent_t ev : {h->e0, h->e1, h->ea0, h->ea1, h->es0, h->es1, h->evFork, h->evJoin}) if (ev) cudaEventDestroy(ev);
    if (h->s2) cudaStreamDestroy(h->s2);
    if (h->s) cudaStreamDestroy(h->s);
    delete h;
    return 0;
}

int mpsgpu_initialize(mpsgpu_t h) {
    if (!h) return MPSGPU_ERR_ARG;
    const MpsParams& P = h->d.P;
    int e;
    if ((e = runOpImpl(h, MPS_OP_UPDATE_BUCKETS))) return e;
    if ((e = runOpImpl(h, MPS_OP_OUT_OF_DOMAIN))) return e;
    if (P.wallType == 1) {      // initMesh, src/main.cpp:527-554
        if ((e = runOpImpl(h, MPS_OP_WALL_DISTANCE))) return e;
        if ((e = runOpImpl(h, MPS_OP_WALL_NPCD))) return e;
    }
    if ((e = runOpImpl(h, MPS_OP_INIT_PND))) return e;
    if ((e = runOpImpl(h, MPS_OP_UPDATE_BC))) return e;
    if ((e = runOpImpl(h, MPS_OP_CALC_PRESS))) return e;
    return checkDeviceErrors(h);
}

int mpsgpu_step(mpsgpu_t h, MpsStepStats* stats) {
    if (!h) return MPSGPU_ERR_ARG;
    std::memset(&h->last, 0, sizeof(h->last));
    h->last.runSteps = 1;
    cudaEventRecord(h->e0, h->s);
    int e = stepImpl(h);
    cudaEventRecord(h->e1, h->s);
    if (e) return e;
    if ((e = checkDeviceErrors(h))) return e;
    float ms = 0;
    cudaEventElapsedTime(&ms, h->e0, h->e1);
    return finishStats(h, stats, ms);
}

int mpsgpu_run(mpsgpu_t h, int nsteps, MpsStepStats* stats) {
    if (!h || nsteps < 0) return MPSGPU_ERR_ARG;
    cudaEventRecord(h->e0, h->s);
    h->last.runSteps = nsteps;
    h->last.runPpeSolves = 0;
    h->last.runPpeIterations = 0;
    h->last.runPpeRefinements = 0;
    h->last.runPpeFallbacks = 0;
    for (int k = 0; k < nsteps; k++) {
        int e = stepImpl(h);
        if (e) return e;
    }
    cudaEventRecord(h->e1, h->s);
    int e = checkDeviceErrors(h);
    if (e) return e;
    float ms = 0;
    cudaEventElapsedTime(&ms, h->e0, h->e1);
    return finishStats(h, stats, ms);
}

int mpsgpu_run_op(mpsgpu_t h, int op) {
    if (!h) return MPSGPU_ERR_ARG;
    int e = runOpImpl(h, op);
    if (e) return e;
    return checkDeviceErrors(h);
}

int mpsgpu_set_precision(mpsgpu_t h, int precision) {
    if (!h || (precision != MPSGPU_PRECISION_FP64 && precision != MPSGPU_PRECISION_DF32)) return MPSGPU_ERR_ARG;
    if (precision != h->d.prec) {
        h->d.prec = precision;
        h->listValid = false;
        h->skinValid = false;
        h->corrFresh = false;
        h->masksValid = false;
        h->cacheValid = false;
    }
    return 0;
}

int mpsgpu_set_ppe_launch(mpsgpu_t h, int mode) {
    if (!h || mode < 0 || mode > 4) return MPSGPU_ERR_ARG;
    h->persistent = mode == 4 ? 1 : mode;
    h->B.ownOff = mode == 4 ? 1 : 0;
    return 0;
}

int mpsgpu_set_solver(mpsgpu_t h, int solver, int warm, double tol, int max_iter) {
    if (!h || (solver != MPSGPU_SOLVER_PLAIN_FP64 && solver != MPSGPU_SOLVER_MIXED && solver != MPSGPU_SOLVER_MIXED_MATFREE &&
               solver != MPSGPU_SOLVER_MIXED_COMPACT) || warm < 0 || warm > 4 || !(tol > 0))
        return MPSGPU_ERR_ARG;
    if (warm == MPSGPU_WARM_MLP && !h->mlp.ready) { g_lastError = "MLP weights not set"; return MPSGPU_ERR_ARG; }
    h->solver = solver; h->warm = warm; h->tol = tol; h->maxIter = max_iter;
    return 0;
}

int mpsgpu_num_particles(mpsgpu_t h, int* n) {
    if (!h || !n) return MPSGPU_ERR_ARG;
    if (h->nHost >= 0) {   // unchanged since the last read (only removals change it)
        *n = h->nHost;
        return 0;
    }
    CK(cudaMemcpyAsync(n, h->d.nLive, sizeof(int), cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    h->nHost = *n;
    return 0;
}

int mpsgpu_time(mpsgpu_t h, double* t, int* it) {
    if (!h) return MPSGPU_ERR_ARG;
    if (t) *t = h->timeCurrent;
    if (it) *it = h->numIter;
    return 0;
}

int mpsgpu_stream(mpsgpu_t h, void** stream) {
    if (!h || !stream) return MPSGPU_ERR_ARG;
    *stream = (void*)h->s;
    return 0;
}

static void* fieldPtr(mpsgpu_t h, int f, int* kind) {
    Dev& d = h->d;
    *kind = 0;
    switch (f) {
        case MPS_F_POS: return d.pos;
        case MPS_F_VEL: return d.vel;
        case MPS_F_ACC: return d.acc;
        case MPS_F_ACCSTAR: return d.accStar;
        case MPS_F_NPCD: return d.npcd;
        case MPS_F_GRADC: return d.gradC;
        case MPS_F_CORR1: return d.c1;
        case MPS_F_CORR2: return d.c2;
        case MPS_F_CORR3: return d.c3;
        case MPS_F_MIRROR: return d.mirror;
        case MPS_F_WALLPOS: return d.wallPos;
        case MPS_F_POLYNORMAL: return d.polyNormal;
        case MPS_F_FORCEWALL: return d.forceWall;
        case MPS_F_NORMAL: return d.normal;
        default: break;
    }
    *kind = 1;
    switch (f) {
        case MPS_F_PRESS: return d.press;
        case MPS_F_PRESSPPE: return d.pressPPE;
        case MPS_F_PNDI: return d.pndi;
        case MPS_F_PNDKI: return d.pndki;
        case MPS_F_PNDSKI: return d.pndski;
        case MPS_F_PNDSMALL: return d.pndSmall;
        case MPS_F_NPCD2: return d.npcd2;
        case MPS_F_CONC: return d.conc;
        case MPS_F_VELDIV: return d.velDiv;
        case MPS_F_DIFFTERM: return d.diffTerm;
        case MPS_F_PNDWALL: return d.pndWall;
        case MPS_F_RIW2: return d.riw2;
        case MPS_F_DEVDOT: return d.devDot;
        case MPS_F_SOURCE: return d.source;
        case MPS_F_PRESSPPE_PREV: return d.pressPPEprev;
        case MPS_F_PRESSPPE_PREV2: return d.pressPPEprev2;
        default: break;
    }
    *kind = 2;
    switch (f) {
        case MPS_F_TYPE: return d.type;
        case MPS_F_BC: return d.bc;
        case MPS_F_NUMNEIGH: return d.numNeigh;
        case MPS_F_NNEIGHWALL: return d.nNeighWall;
        case MPS_F_NEARWALL: return d.nearWall;
        default: break;
    }
    return nullptr;
}

int mpsgpu_get_field(mpsgpu_t h, int f, void* host) {
    if (!h || !host) return MPSGPU_ERR_ARG;
    int kind;
    void* p = fieldPtr(h, f, &kind);
    if (!p) { g_lastError = "unknown field"; return MPSGPU_ERR_ARG; }
    int n = 0;
    int e = mpsgpu_num_particles(h, &n);
    if (e) return e;
    // reorder (and de-pad vectors) on the device, then one copy into the caller's array (for
    // page-locked arrays this beat the reorder kernel writing the host array directly over
    // the host link: 0.78 vs 0.97 ms per set + get of four fields at 864k particles)
    toRef(h, kind, p, n);
    size_t bytes = (kind == 0) ? 3 * sizeof(double) * n : ((kind == 1) ? sizeof(double) : sizeof(int)) * n;
    CK(cudaMemcpyAsync(host, h->permScratch, bytes, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    return 0;
}

int mpsgpu_write_vtu(mpsgpu_t h, const char* path, unsigned int groups) {
    if (!h || !path) return MPSGPU_ERR_ARG;
    int n = 0;
    int e = mpsgpu_num_particles(h, &n);
    if (e) return e;
    Dev& d = h->d;
    // the arrays of writeVtuAscii, in its order: 0 FP64 vector, 1 FP64 scalar, 2 int,
    // 3 generated int (r + add), 4 UInt8 constant, 5 Int32 zeros
    struct Arr { const char* name; int kind; const void* src; int add; };
    std::vector<Arr> pts = {{"Position", 0, d.pos, 0}};
    std::vector<Arr> pd = {{"Velocity", 0, d.vel, 0}, {"pressure", 1, d.press, 0}, {"BC", 2, d.bc, 0}};
    if (groups & MPSGPU_VTU_PND) { pd.push_back({"pnd", 1, d.pndi, 0}); pd.push_back({"pndSmall", 1, d.pndSmall, 0}); }
    if (groups & MPSGPU_VTU_NEIGH) pd.push_back({"nNeigh", 2, d.numNeigh, 0});
    if (groups & MPSGPU_VTU_DEVIATION) { pd.push_back({"npcdDeviation", 0, d.npcd, 0}); pd.push_back({"polygonNormal", 0, d.polyNormal, 0}); }
    if (groups & MPSGPU_VTU_CONCENTRATION) { pd.push_back({"concentration", 1, d.conc, 0}); pd.push_back({"GradCi", 0, d.gradC, 0}); }
    if (groups & MPSGPU_VTU_AUXILIAR) {
        pd.push_back({"ParticleType", 2, d.type, 0});
        if (d.P.wallType == 1) pd.push_back({"nearMeshType", 5, nullptr, 0});
    }
    std::vector<Arr> cells = {{"connectivity", 3, nullptr, 0}, {"offsets", 3, nullptr, 1}, {"types", 4, nullptr, 1}};
    auto bytesOf = [&](const Arr& a) -> size_t { return a.kind == 0 ? 12ull * n : (a.kind == 4 ? (size_t)n : 4ull * n); };
    size_t total = 0;
    for (auto* g : {&pts, &pd, &cells})
        for (auto& a : *g) total += 4 + bytesOf(a);
    if (total > h->vtuCap) {
        if (h->vtuDev) cudaFree(h->vtuDev);
        if (h->vtuHost) cudaFreeHost(h->vtuHost);
        h->vtuDev = h->vtuHost = nullptr;
        h->vtuCap = 0;
        CK(cudaMalloc(&h->vtuDev, total));
        CK(cudaMallocHost(&h->vtuHost, total));
        h->vtuCap = total;
    }
    // pack: each array is a UInt32 byte count followed by its data (4-byte aligned: the one
    // UInt8 array is the last)
    char* base = (char*)h->vtuDev;
    size_t off = 0;
    std::vector<size_t> offs;
    std::vector<unsigned int> heads;
    for (auto* g : {&pts, &pd, &cells})
        for (auto& a : *g) {
            offs.push_back(off);
            heads.push_back((unsigned int)bytesOf(a));
            char* dst = base + off + 4;
            int gr = gridFor(n, 256);
            if (n > 0) {
                if (a.kind == 0) k_vtu_vec<<<gr, 256, 0, h->s>>>((const dvec4*)a.src, d.slotOf, n, (float*)dst);
                else if (a.kind == 1) k_vtu_sca<<<gr, 256, 0, h->s>>>((const double*)a.src, d.slotOf, n, (float*)dst);
                else if (a.kind == 2) k_vtu_int<<<gr, 256, 0, h->s>>>((const int*)a.src, d.slotOf, n, (int*)dst, 0);
                else if (a.kind == 3) k_vtu_int<<<gr, 256, 0, h->s>>>(nullptr, d.slotOf, n, (int*)dst, a.add);
                else if (a.kind == 4) k_vtu_u8<<<gr, 256, 0, h->s>>>(n, (unsigned char*)dst, (unsigned char)a.add);
                else CK(cudaMemsetAsync(dst, 0, 4ull * n, h->s));
                countLaunch(a.kind == 5 ? 0 : 1);
            }
            off += 4 + bytesOf(a);
        }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h->vtuHost, h->vtuDev, total, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    char* hb = (char*)h->vtuHost;
    for (size_t k = 0; k < offs.size(); k++) std::memcpy(hb + offs[k], &heads[k], 4);
    FILE* fp = std::fopen(path, "wb");
    if (!fp) { g_lastError = std::string("cannot open ") + path; return MPSGPU_ERR_ARG; }
    size_t k = 0;
    auto arr = [&](const Arr& a, const char* indent) {
        const char* ty = a.kind == 4 ? "UInt8" : (a.kind >= 2 ? "Int32" : "Float32");
        if (a.kind == 0)
            std::fprintf(fp, "%s<DataArray type='%s' Name='%s' NumberOfComponents='3' format='appended' offset='%zu'/>\n",
                         indent, ty, a.name, offs[k]);
        else
            std::fprintf(fp, "%s<DataArray type='%s' Name='%s' format='appended' offset='%zu'/>\n", indent, ty, a.name,
                         offs[k]);
        k++;
    };
    std::fprintf(fp, "<?xml version='1.0' encoding='UTF-8'?>\n");
    std::fprintf(fp, "<VTKFile xmlns='VTK' byte_order='LittleEndian' version='0.1' type='UnstructuredGrid' "
                     "header_type='UInt32'>\n");
    std::fprintf(fp, "  <UnstructuredGrid>\n");
    std::fprintf(fp, "    <Piece NumberOfCells='%d' NumberOfPoints='%d'>\n", n, n);
    std::fprintf(fp, "      <Points>\n");
    for (auto& a : pts) arr(a, "        ");
    std::fprintf(fp, "      </Points>\n      <PointData>\n");
    for (auto& a : pd) arr(a, "        ");
    std::fprintf(fp, "      </PointData>\n      <Cells>\n");
    for (auto& a : cells) arr(a, "        ");
    std::fprintf(fp, "      </Cells>\n    </Piece>\n  </UnstructuredGrid>\n");
    std::fprintf(fp, "  <AppendedData encoding='raw'>\n_");
    size_t wr = std::fwrite(hb, 1, total, fp);
    std::fprintf(fp, "\n  </AppendedData>\n</VTKFile>\n");
    std::fclose(fp);
    if (wr != total) { g_lastError = std::string("short write to ") + path; return MPSGPU_ERR_ARG; }
    return 0;
}

int mpsgpu_last_stats(mpsgpu_t h, MpsStepStats* out) {
    if (!h || !out) return MPSGPU_ERR_ARG;
    *out = h->last;
    return 0;
}

int mpsgpu_set_field(mpsgpu_t h, int f, const void* host) {
    if (!h || !host) return MPSGPU_ERR_ARG;
    int kind;
    void* p = fieldPtr(h, f, &kind);
    if (!p) { g_lastError = "unknown field"; return MPSGPU_ERR_ARG; }
    int n = 0;
    int e = mpsgpu_num_particles(h, &n);
    if (e) return e;
    // one copy of the caller's array, then reorder (and pad vectors) on the device
    size_t bytes = (kind == 0) ? 3 * sizeof(double) * n : ((kind == 1) ? sizeof(double) : sizeof(int)) * n;
    CK(cudaMemcpyAsync(h->permScratch, host, bytes, cudaMemcpyHostToDevice, h->s));
    fromRef(h, kind, p, n);
    // any state change can alter list membership, masks or the near-wall set (the shifting
    // filter keeps the skin list: it re-checks every position against its start position and
    // scan window, so set positions fall back to the bucket scan where they must)
    h->listValid = false;
    h->skinValid = false;
    h->corrFresh = false;
    h->masksValid = false;
    h->cacheValid = false;
    if (f == MPS_F_POS) launchPosf(h->d, h->s);
    if (f == MPS_F_CORR1 || f == MPS_F_CORR2 || f == MPS_F_CORR3) launchCorrDF(h->d, h->s);
    CK(cudaStreamSynchronize(h->s));
    return 0;
}

int mpsgpu_get_neighbors(mpsgpu_t h, int* counts, int* nbr, long long cap) {
    if (!h || !counts) return MPSGPU_ERR_ARG;
    ensureList(h);
    int e = checkDeviceErrors(h);
    if (e) return e;
    int n = 0;
    if ((e = mpsgpu_num_particles(h, &n))) return e;
    // rows and entries in reference indices (storage is in bucket order)
    std::vector<int> cnt(n), orig(h->N0), slot(h->N0);
    CK(cudaMemcpyAsync(cnt.data(), h->d.nbrCount, sizeof(int) * n, cudaMemcpyDeviceToHost, h->s));
    CK(cudaMemcpyAsync(orig.data(), h->d.orig, sizeof(int) * h->N0, cudaMemcpyDeviceToHost, h->s));
    CK(cudaMemcpyAsync(slot.data(), h->d.slotOf, sizeof(int) * h->N0, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    for (int r = 0; r < n; r++) counts[r] = cnt[slot[r]];
    if (!nbr) return 0;
    std::vector<int> ell((size_t)h->d.K * h->N0);
    CK(cudaMemcpyAsync(ell.data(), h->d.nbr, sizeof(int) * ell.size(), cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    long long k = 0;
    for (int r = 0; r < n; r++) {
        int i = slot[r];
        for (int c = 0; c < counts[r]; c++) {
            if (k >= cap) return MPSGPU_ERR_CAPACITY;
            nbr[k++] = orig[ell[(size_t)c * h->N0 + i]];
        }
    }
    return 0;
}

int mpsgpu_get_ppe(mpsgpu_t h, long long* nnz_out, long long* rowptr, int* col, double* val, double* rhs) {
    if (!h || !nnz_out) return MPSGPU_ERR_ARG;
    if (h->d.P.mpsType != 2 && h->d.P.mpsType != 3) return MPSGPU_ERR_UNSUPPORTED;
    int n = 0;
    int e = mpsgpu_num_particles(h, &n);
    if (e) return e;
    std::vector<int> len(n), orig(h->N0), slot(h->N0);
    std::vector<double> diag(n), bst(n);
    CK(cudaMemcpyAsync(len.data(), h->B.rowLen, sizeof(int) * n, cudaMemcpyDeviceToHost, h->s));
    CK(cudaMemcpyAsync(diag.data(), h->B.diag, sizeof(double) * n, cudaMemcpyDeviceToHost, h->s));
    CK(cudaMemcpyAsync(orig.data(), h->d.orig, sizeof(int) * h->N0, cudaMemcpyDeviceToHost, h->s));
    CK(cudaMemcpyAsync(slot.data(), h->d.slotOf, sizeof(int) * h->N0, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    long long nnz = n;
    for (int i = 0; i < n; i++) nnz += len[i];
    *nnz_out = nnz;
    if (!col) return 0;
    size_t ellN = (size_t)h->d.K * h->B.N0;
    std::vector<int> ec(ellN);
    std::vector<double> ev(ellN);
    CK(cudaMemcpyAsync(ec.data(), h->B.col, sizeof(int) * ellN, cudaMemcpyDeviceToHost, h->s));
    CK(cudaMemcpyAsync(ev.data(), h->B.val, sizeof(double) * ellN, cudaMemcpyDeviceToHost, h->s));
    CK(cudaMemcpyAsync(bst.data(), h->B.b, sizeof(double) * n, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    long long k = 0;
    rowptr[0] = 0;
    std::vector<std::pair<int, double>> row;
    for (int r = 0; r < n; r++) {   // reference rows and columns
        int i = slot[r];
        if (rhs) rhs[r] = bst[i];
        row.clear();
        row.push_back({r, diag[i]});
        const size_t base = ellBase(h->B, i);
        for (int c = 0; c < len[i]; c++) {
            const size_t e = base + (size_t)c * h->B.ellStride;
            row.push_back({orig[ec[e]], ev[e]});
        }
        std::sort(row.begin(), row.end(), [](const std::pair<int, double>& a, const std::pair<int, double>& b) { return a.first < b.first; });
        for (auto& pr : row) { col[k] = pr.first; val[k] = pr.second; k++; }
        rowptr[r + 1] = k;
    }
    return 0;
}

int mpsgpu_mlp_set_weights(mpsgpu_t h, const float* params, const float* norm32) {
    if (!h || !params || !norm32) return MPSGPU_ERR_ARG;
    return mlpSetWeights(h->mlp, params, norm32, h->s);
}
int mpsgpu_mlp_get_weights(mpsgpu_t h, float* params, float* norm32) {
    if (!h || !params || !norm32) return MPSGPU_ERR_ARG;
    return mlpGetWeights(h->mlp, params, norm32, h->s);
}
int mpsgpu_ppe_features(mpsgpu_t h, float* feat) {
    if (!h || !feat) return MPSGPU_ERR_ARG;
    if (h->d.P.mpsType != 2 && h->d.P.mpsType != 3) return MPSGPU_ERR_UNSUPPORTED;
    int n = 0;
    int e = mpsgpu_num_particles(h, &n);
    if (e) return e;
    std::vector<float> st((size_t)MPSGPU_MLP_NFEAT * n);
    if (!h->B.prepared) { launchMixedPrepare(h->d, h->B, h->s); h->B.prepared = 1; }   // features read valf
    if ((e = mlpFeatures(h->mlp, h->d, h->B, st.data(), n, h->s))) return e;
    std::vector<int> slot(n);
    CK(cudaMemcpyAsync(slot.data(), h->d.slotOf, sizeof(int) * n, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    for (int r = 0; r < n; r++)   // rows in reference order
        std::memcpy(feat + (size_t)r * MPSGPU_MLP_NFEAT, st.data() + (size_t)slot[r] * MPSGPU_MLP_NFEAT,
                    sizeof(float) * MPSGPU_MLP_NFEAT);
    return 0;
}

int mpsgpu_mlp_record(mpsgpu_t h, int enable) {
    if (!h) return MPSGPU_ERR_ARG;
    if (h->d.P.mpsType != 2 && h->d.P.mpsType != 3) return MPSGPU_ERR_UNSUPPORTED;
    h->mlp.recording = enable != 0;
    return 0;
}
int mpsgpu_mlp_num_records(mpsgpu_t h, long long* n) {
    if (!h || !n) return MPSGPU_ERR_ARG;
    *n = h->mlp.recCount;
    return 0;
}
int mpsgpu_mlp_fit_normalization(mpsgpu_t h) {
    if (!h) return MPSGPU_ERR_ARG;
    return mlpFitNormalization(h->mlp, h->s);
}
int mpsgpu_mlp_train(mpsgpu_t h, int iters, int batch, float lr, unsigned long long seed, float* loss_hist) {
    if (!h || iters <= 0) return MPSGPU_ERR_ARG;
    return mlpTrain(h->mlp, iters, batch, lr, seed, loss_hist, h->s);
}
int mpsgpu_mlp_forward(mpsgpu_t h, const float* feat, int n, float* out) {
    if (!h || !feat || !out || n <= 0) return MPSGPU_ERR_ARG;
    return mlpForwardHost(h->mlp, feat, n, out, h->s);
}
int mpsgpu_mlp_gradient(mpsgpu_t h, const float* feat, const float* target, int n, float* grad, float* loss) {
    if (!h || !feat || !target || !grad || !loss) return MPSGPU_ERR_ARG;
    return mlpGradient(h->mlp, feat, target, n, grad, loss, h->s);
}

}  // extern "C"
