// mps_internal.h — launch wrappers shared between the translation units of libmpsgpu.
#pragma once
#include <cuda_runtime.h>
#include <vector>
#include <cuda_fp16.h>
#include "mps_common.cuh"

// Kernel-launch counter (all launches of this library, process-wide).
void countLaunch(int n);
long long launchCount();

// Per-class device timing with CUDA events on the handle's stream.  Classes 0..MPS_OP_COUNT-1
// are the operators; the extra classes split the pressure solve.
enum {
    PROF_NEIGHBOR_LIST = MPS_OP_COUNT, PROF_PPE_ASSEMBLE, PROF_PPE_SPMV, PROF_PPE_VECTOR,
    PROF_PPE_OTHER, PROF_PPE_SOLVE, PROF_NCLASS
};
struct Prof {
    bool on = false;
    std::vector<cudaEvent_t> ev;      // pairs
    std::vector<int> cls;
    std::vector<size_t> open;         // slots begun and not yet ended
    size_t used = 0;
    double ms[PROF_NCLASS] = {0};
    long long calls[PROF_NCLASS] = {0};
    void begin(int c, cudaStream_t s, bool count = true);
    void end(cudaStream_t s);
    int flush();                      // synchronises on the last event, accumulates
    void reset();
    void destroy();
};

// mps_cells.cu
void scanExclusive(const int* in, int* out, int n, int* scratch, cudaStream_t s);
int scanScratchInts(int n);
// perm != NULL: renumber the storage into bucket order (perm: N0 ints, permScratch: 32 N0 bytes)
void launchBuckets(const Dev& d, int* scanScratch, cudaStream_t s, int* perm, void* permScratch);
int renumberLaunches();
void launchNeighborList(const Dev& d, cudaStream_t s);
void launchPosf(const Dev& d, cudaStream_t s);       // FP32 copy, then its bucket-ordered copy
void launchPosfCell(const Dev& d, cudaStream_t s);   // bucket-ordered copy only
void launchSideMasks(const Dev& d, cudaStream_t s);
void launchFillCache(const Dev& d, cudaStream_t s);

// mps_ops.cu
void launchViscosity(const Dev& d, cudaStream_t s);
// FP64 tier over the start-of-step skin list (built by launchSkinListDF): the viscosity
// sweep, and the list of the current positions with its weights filtered from it
void launchViscosityList(const Dev& d, cudaStream_t s);
void launchNeighborFilter(const Dev& d, cudaStream_t s, bool weights = true);   // the FP64 list from the skin list
void launchAddGravity(const Dev& d, cudaStream_t s);
void launchPredict(const Dev& d, cudaStream_t s);
void launchOutOfDomain(const Dev& d, int* flags, int* counter, cudaStream_t s);
void launchCollision(const Dev& d, cudaStream_t s);
void launchCollisionApply(const Dev& d, cudaStream_t s);
void launchWallNpcd(const Dev& d, cudaStream_t s);
void launchCorrectionMatrix(const Dev& d, cudaStream_t s);
void launchPndNeighNpcd(const Dev& d, cudaStream_t s);
void launchPndDiffusive(const Dev& d, cudaStream_t s);
void launchPndMean(const Dev& d, cudaStream_t s);
void launchInitPnd(const Dev& d, cudaStream_t s);
void launchUpdateBC(const Dev& d, cudaStream_t s);
void launchEOS(const Dev& d, cudaStream_t s);
void launchExtrapolatePress(const Dev& d, cudaStream_t s);
void launchPressGradient(const Dev& d, cudaStream_t s);
void launchWallPressGradient(const Dev& d, cudaStream_t s);
void launchPredictPressGradient(const Dev& d, bool skin, cudaStream_t s);   // relax_fact < 1, before PREDICT
void launchWallViscosity(const Dev& d, cudaStream_t s);
void launchCorrect(const Dev& d, cudaStream_t s);
void launchShifting(const Dev& d, cudaStream_t s, bool list);   // list: filter the kept skin list first
void launchDummyVelocity(const Dev& d, cudaStream_t s);

// mps_ops_df.cu (DF32 tier)
void launchNeighborListDF(const Dev& d, cudaStream_t s);
void launchSideMasksDF(const Dev& d, cudaStream_t s);
void launchViscosityDF(const Dev& d, cudaStream_t s);
void launchCollisionDF(const Dev& d, cudaStream_t s);
void launchWallNpcdDF(const Dev& d, cudaStream_t s);
void launchCorrectionMatrixDF(const Dev& d, cudaStream_t s);
void launchCorrDF(const Dev& d, cudaStream_t s);
// withCorrection: also the correction matrix of the same positions and masks
void launchPndNeighNpcdDF(const Dev& d, cudaStream_t s, bool withCorrection = false);
void launchPressGradientDF(const Dev& d, cudaStream_t s);
void launchWallPressGradientDF(const Dev& d, cudaStream_t s);
void launchWallViscosityDF(const Dev& d, cudaStream_t s);
void launchShiftingDF(const Dev& d, cudaStream_t s);
// the same from the list of the current positions (filtered from the skin list, masks built)
void launchShiftingListDF(const Dev& d, cudaStream_t s);
// ARC free surface (free-surface type 2): fluid normals (+ wall term), then the BC test
void launchUpdateBCArc(const Dev& d, cudaStream_t s);
// dynamic particle collision (collision type 1, FP64, list based; moves positions)
void launchCollisionDPC(const Dev& d, cudaStream_t s);
// velocity divergence of the PND + div u source (list based, FP64; + the polygon-wall term)
void launchVelDivergence(const Dev& d, cudaStream_t s);
// start-of-step list with a skin: build, viscosity over it, and the list of the current
// positions filtered from it
void launchSkinListDF(const Dev& d, cudaStream_t s);
void launchViscosityListDF(const Dev& d, cudaStream_t s);
void launchNeighborFilterDF(const Dev& d, cudaStream_t s);
// the skin list's validity flag for the current positions (moved more than half the skin)
void launchSkinCheck(const Dev& d, cudaStream_t s);
void launchShiftVelApply(const Dev& d, cudaStream_t s);
void launchApplyShift(const Dev& d, cudaStream_t s);

// mps_wall.cu
void launchWallDistance(const Dev& d, cudaStream_t s);

// mps_ppe.cu
struct PpeBuffers {
    int N0, K;       // N0: rows padded to a multiple of 256 (and of the slice height)
    // ELL layout: entry k of row i at ellBase(i) + k * ellStride.  Column-major (sliceShift 31,
    // ellStride N0) or sliced: slices of 2^sliceShift consecutive rows, each slice's K entries
    // column-major inside it (ellStride = 2^sliceShift)
    int sliceShift, sliceMask;
    size_t ellStride;
    double *diag, *val, *x, *b, *r, *z, *p, *Ap, *scal;  // scal: solver scalars (device)
    int* col;
    int* rowLen;
    float *valf, *diagf, *diagInvf, *rf, *zf, *pf, *Apf, *xf;  // mixed-precision copies
    double* partials;
    unsigned int* counter;
    int* flag;       // [0] done, [1] iterations, [2] breakdown, [3] inner done, [4] refinements
    int nblocks;
    double* dinv;            // FP64 inverse diagonal (persistent plain solver)
    unsigned int* bar;       // grid barrier of the persistent solvers: arrivals, generation, abort
    int pgridCg, pgridMx;    // co-resident grid sizes of the persistent solvers (0: unavailable)
    int prepared;            // FP32 copies (valf, diagf, diagInvf) already written by the assembly
    Mask* mfMask;            // per row: neighbour-list entries that are matrix entries
    int matfree;             // mixed inner operator: 0 assembled FP32, 1 matrix-free, 2 compact scaled,
                             // 3 staged tiles, 4 assembled FP32 with the pipelined inner CG
    int pgridMf;             // co-resident grid of the matrix-free mixed solver
    __half* valh;            // compact scaled operator: FP16 off-diagonals of diag(sigma s) A diag(s)
    short* col16;            // and their column offsets j - i
    float *sclf, *sgs;       // s_i = 1/sqrt|A_ii| and sigma_i s_i
    unsigned char* wideRow;  // rows with an offset outside 16 bits (read the 32-bit columns)
    int pgridH16;
    int pgridTs;             // co-resident grid of the mixed solver with the staged ELL tiles (0: none)
    // pipelined inner CG: w = A u and z = A q recurrences, second buffer of m = M w, and the
    // second FP64 iterate of the refinement
    float *wf, *qzf, *mf2;
    double* xalt;
    int pgridPipe;
    double* bs[4];           // BiCGSTAB: shadow residual r0, s, M^-1 s, A M^-1 s
    int pgridBi;             // co-resident grid of the BiCGSTAB solver
    // solver vectors in shared memory (mixed: x_f, r_f, p, Ap; plain FP64: r, p, Ap): the
    // grid (one block per SM; 0: unavailable), the row slots per block, and 1 to keep every
    // vector in global memory instead
    int pgridOwn, ownCap, ownOff;
    int pgridOwn64, ownCap64;
    // learned warm start: the network's correction c of the start x (nullptr: none); the
    // shared-memory mixed solver takes the residual-minimising step x + theta c in its set-up
    const float* cdir;
    const float* cq;   // q = A c (FP32) of the learned correction
};
// Element offset of entry 0 of row i in the ELL arrays.
__host__ __device__ __forceinline__ size_t ellBase(const PpeBuffers& B, int i) {
    return (((size_t)(i >> B.sliceShift) * (size_t)B.K) << B.sliceShift) + (size_t)(i & B.sliceMask);
}
void launchPpeAssemble(const Dev& d, const PpeBuffers& B, cudaStream_t s);
void launchPpeCopyBack(const Dev& d, const PpeBuffers& B, cudaStream_t s);
void launchPpeAssembleDF(const Dev& d, const PpeBuffers& B, cudaStream_t s);
void launchWarmExtrapolate(const Dev& d, const PpeBuffers& B, cudaStream_t s, bool quadratic = false);
// FP32 copies of the assembled matrix (valf, diagf, diagInvf) for the FP64 assembly
void launchMixedPrepare(const Dev& d, const PpeBuffers& B, cudaStream_t s);
// Returns iterations and final relative residual through host pointers (synchronises).
int ppeSolvePlain(const Dev& d, const PpeBuffers& B, double tol, int maxIter, cudaStream_t s,
                  int* iters, double* relres, double* relres0, Prof* prof);
int ppeSolveMixed(const Dev& d, const PpeBuffers& B, double tol, int maxIter, cudaStream_t s,
                  int* iters, int* refinements, double* relres, double* relres0, Prof* prof);
// Whole solve in one cooperative launch (mixed = 1: FP32 inner CG under FP64 refinement).
int ppeSolvePersistent(const Dev& d, const PpeBuffers& B, int mixed, double tol, int maxIter, cudaStream_t s,
                       int* iters, int* refinements, double* relres, double* relres0, Prof* prof);
int ppePersistentGrid(int mixed);
// row slots per block of the shared-memory solvers at most (a multiple of their block sizes,
// 1024 mixed, 768 plain FP64)
#define OWN_CAP_ROWS 13312
#define OWN64_CAP_ROWS 8448
// BiCGSTAB (solver_type 1) in one cooperative launch
int ppeSolveBicgstab(const Dev& d, const PpeBuffers& B, double tol, int maxIter, cudaStream_t s, int* iters,
                     double* relres, double* relres0, Prof* prof);
