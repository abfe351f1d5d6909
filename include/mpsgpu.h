/*
 * mpsgpu.h — C ABI of the GB300 (sm_103a) implementation of the PolyMPS per-step
 * particle path (bucket cell list, PND/neighbour sums, EOS, PPE assembly + CG,
 * viscosity Laplacian, polygon wall distance/mirror, collision, shifting).
 *
 * The reference (rubensamarojr/polymps) has no FFI: its boundary is the class-method
 * stepping interface driven by mainLoopOfSimulation (src/main.cpp:221-469), where every
 * operator is `void Class::method(MpsParticleSystem*, MpsParticle*, MpsBucket*)`
 * (include/MpsPndNeigh.h:57, include/MpsPressure.h:49, include/MpsViscosity.h:43).
 * Each entry point below replaces one of those calls (cited per function) or a group of
 * them; plain pointers and sizes only, no C++ or torch types, and every call returns an
 * int status (0 = success, see MPSGPU_ERR_*) instead of printing and continuing.
 *
 * Ownership: the library owns all device memory behind the opaque handle; host arrays
 * passed in are only read (or written for downloads) during the call.  A handle is not
 * thread-safe and orders all its work on one CUDA stream (mpsgpu_stream): the one kernel a
 * step runs on a second internal stream (the wall distance, beside the list filter and the
 * collision) is forked from that stream and joined back into it within the step.
 */
#ifndef MPSGPU_H_
#define MPSGPU_H_

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status codes */
#define MPSGPU_OK                 0
#define MPSGPU_ERR_ARG            1   /* bad argument / NULL pointer / size          */
#define MPSGPU_ERR_CUDA           2   /* a CUDA runtime call failed                   */
#define MPSGPU_ERR_NOMEM          3   /* device allocation failed                     */
#define MPSGPU_ERR_UNSUPPORTED    4   /* configuration outside the implemented path   */
#define MPSGPU_ERR_NOT_CONVERGED  5   /* PPE solver hit its iteration cap             */
#define MPSGPU_ERR_CAPACITY       6   /* neighbour/PPE row capacity exceeded          */
#define MPSGPU_ERR_DOMAIN         7   /* particle outside the bucket grid             */
#define MPSGPU_ERR_NOGPU          8   /* no CUDA device visible                       */
#define MPSGPU_ERR_SIZE_MISMATCH  9   /* implicit run lost particles (pressurePPE size) */

/* ------------------------------------------------------------------ parameters
 * Mirrors the JSON inputs of MpsParticleSystem (include/MpsParticleSystem.h:133-221),
 * read by MpsInputOutput::readInputFile (src/MpsInputOutput.cpp:58-641), followed by the
 * derived constants computed in MpsParticle::setParameters (src/MpsParticle.cpp:136-227)
 * and MpsBucket::allocateMemory / calcDomainLimits (src/MpsBucket.cpp:20-295).
 * Fill the input block, then call mpsgpu_params_derive() to fill the derived block
 * (the radii reS/reL/reRepulsiveForce are given in units of partDist, as in the JSON;
 * derive() scales them, exactly as setParameters does). */
typedef struct MpsParams {
    /* --- inputs (JSON) --- */
    int    wallType;            /* 0 particle walls, 1 polygon                         */
    int    femOn, forcedOn;     /* must be 0 (deformable/forced meshes not supported)  */
    double domainMin[3], domainMax[3];
    int    domainTypeBC;        /* 0 none (1 periodic: not supported)                  */
    int    limitTypeBC;         /* 0 border particle positions, 1 JSON limits          */
    double densityFluid, densityWall, KNM_VS1;
    int    fluidType;           /* 0 Newtonian (1 non-Newtonian: not supported)        */
    double gravity[3];
    double KNM_VS2, DNS_FL1, DNS_FL2;
    double dim, partDist, timeStep, timeSimulation;
    int    iterOutput;
    double cflNumber;
    int    weightType, slipCondition;
    double reS, reL;            /* input: multiples of partDist; derived: metres       */
    int    gradientType, gradientCorrection;
    double relaxPress;
    int    mpsType;             /* 0 explicit, 1 weakly compressible, 2 implicit PND  */
    double soundSpeed, gamma;
    int    solverType;          /* 0 CG                                                */
    double alphaCompressibility, relaxPND;
    int    shiftingType;        /* 0 off, 1 velocity (DW*Uij), 2 position (GradC)      */
    double dri, coefA, machNumber;
    int    pndType;             /* 0 sum w, 1 mean, 2 diffusive                        */
    double diffusiveCoef;
    int    repulsiveForceType;  /* 0 Harada, 1 Mitsume, 2 Lennard-Jones, 3 Monaghan-K. */
    double reRepulsiveForce, expectMaxVelocity;
    double repForceCoefMitsume, repForceCoefLennardJones, repForceCoefMonaghanKajtar;
    double EPS_RE;
    int    freeSurfType;        /* 0 PND+neigh, 1 PND+NPCD, 2 ARC (normals + arc test) */
    double pndThreshold, neighThreshold, npcdThreshold, thetaThreshold, normThreshold;
    int    collisionType;       /* 0 PC, 1 DPC (src/main.cpp:285-290); others rejected */
    double collisionRatio, distLimitRatio, lambdaCollision;
    int    ghost, fluid, wall, dummyWall;   /* particle type IDs                        */
    int    surface, inner, other;           /* boundary type IDs                        */
    /* --- derived (mpsgpu_params_derive) --- */
    double epsilonZero;         /* 10*DBL_EPSILON, include/MpsParticleSystem.h:241     */
    double reS2, reL2;
    double pndSmallZero, pndLargeZero, pndGradientZero, lambdaZero, numNeighZero;
    double coeffViscosity, coeffViscMultiphase, coeffPressEMPS, coeffPressGrad;
    double coeffPressWCMPS, coeffShifting1, coeffShifting2, coeffPPE, coeffPPESource;
    double invPartDist, distCollisionLimit, distCollisionLimit2, restitutionCollision;
    double betaPnd, betaNeigh, delta2, thetaArc, hThreshold2, dstThreshold2, normThreshold2;
    double bucketSide, invBucketSide;
    int    numBucketsX, numBucketsY, numBucketsZ, numBucketsXY, numBucketsXYZ;
    int    derived;             /* set to 1 by mpsgpu_params_derive                    */
} MpsParams;

/* Triangle soup of the rigid polygon wall (what igl::readSTL yields,
 * src/PolygonMesh.cpp:51): tri_xyz holds ntri*9 doubles (v0,v1,v2 per triangle). */
typedef struct MpsMesh {
    int           ntri;
    const double* tri_xyz;
} MpsMesh;

/* Per-step statistics (what displayInfo prints, src/MpsInputOutput.cpp:37-55,
 * plus the PPE solve figures and device timings). */
typedef struct MpsStepStats {
    int    numParticles;
    int    ppeIterations;       /* SpMVs performed by the PPE solve                    */
    int    ppeRefinements;      /* FP64 residual refinements (mixed solver)            */
    int    outOfDomain;         /* particles removed this step                         */
    double velMax, CFLcurrent;
    double ppeRelResidual;      /* final FP64 ||b-Ax||/||b||                          */
    double ppeInitialRelResidual;/* ||b-Ax0||/||b|| of the warm start                  */
    double ppeSolveMs;          /* device time of the PPE solve (warm start+iterations)*/
    double ppeAssembleMs;       /* device time of the PPE assembly                     */
    double stepMs;              /* device time of the whole step                       */
    long long nbrEntries;       /* neighbour-list entries of the last list build       */
    long long ppeNnz;           /* non-zeros of the last PPE matrix (with diagonal)    */
    int    runSteps;            /* steps of the last mpsgpu_run / mpsgpu_step call     */
    int    runPpeSolves;        /* PPE solves in that call                             */
    long long runPpeIterations; /* their SpMV iterations, summed                       */
    long long runPpeRefinements;/* their FP64 refinements, summed                      */
    int    ppeFallback;         /* 1: the last solve was a mixed solve that missed the
                                   tolerance, redone by the plain FP64 CG from the
                                   previous solution (the reference's solver)          */
    int    runPpeFallbacks;     /* such solves in the last run call                    */
} MpsStepStats;

/* Field identifiers for get/set.  Vector fields use the reference's interleaved host
 * layout (N x 3 doubles, include/MpsParticle.h:155-165); scalars N doubles; integer
 * fields N int32 (nearWall: 0/1). */
enum MpsField {
    MPS_F_POS = 0, MPS_F_VEL, MPS_F_ACC, MPS_F_ACCSTAR, MPS_F_NPCD, MPS_F_GRADC,
    MPS_F_CORR1, MPS_F_CORR2, MPS_F_CORR3, MPS_F_MIRROR, MPS_F_WALLPOS, MPS_F_POLYNORMAL,
    MPS_F_FORCEWALL,
    MPS_F_NORMAL,                 /* fluid normal of the ARC free-surface test (MpsParticle::normal) */
    MPS_F_PRESS = 32, MPS_F_PRESSPPE, MPS_F_PNDI, MPS_F_PNDKI, MPS_F_PNDSKI, MPS_F_PNDSMALL,
    MPS_F_NPCD2, MPS_F_CONC, MPS_F_VELDIV, MPS_F_DIFFTERM, MPS_F_PNDWALL, MPS_F_RIW2,
    MPS_F_DEVDOT, MPS_F_SOURCE,
    MPS_F_PRESSPPE_PREV,          /* solution of the solve before the last (no reference
                                     array: the warm-start state of the extrapolation) */
    MPS_F_PRESSPPE_PREV2,         /* and the one before it (quadratic extrapolation) */
    MPS_F_TYPE = 64, MPS_F_BC, MPS_F_NUMNEIGH, MPS_F_NNEIGHWALL, MPS_F_NEARWALL
};

/* Operators, for the per-operator entry point mpsgpu_run_op (parity tests and the
 * thin C++ shim that re-presents the library as the reference's class methods). */
enum MpsOp {
    MPS_OP_UPDATE_BUCKETS = 0,   /* MpsBucket::updateParticlesID  src/MpsBucket.cpp:299-353          */
    MPS_OP_VISCOSITY,            /* MpsViscosity::calcViscosity  src/MpsViscosity.cpp:20-100          */
    MPS_OP_ADD_GRAVITY,          /* MpsParticle::addGravity  src/MpsParticle.cpp:111-130              */
    MPS_OP_PREDICT,              /* predictionVelocityPosition  src/MpsParticleVelPos.cpp:20-50       */
    MPS_OP_OUT_OF_DOMAIN,        /* checkParticleOutDomain  src/MpsParticle.cpp:234-402              */
    MPS_OP_COLLISION,            /* checkParticleCollisions  src/MpsParticleCollision.cpp:22-119     */
    MPS_OP_WALL_DISTANCE,        /* closestPointPNDBoundaryAABB + updateParticlesNearPolygonMesh
                                    src/PolygonMesh.cpp:585-795                                      */
    MPS_OP_WALL_NPCD,            /* calcWallNPCD  src/MpsPndNeigh.cpp:105-195                        */
    MPS_OP_CORRECTION_MATRIX,    /* correctionMatrix  src/MpsVectorMatrix.cpp:20-93                  */
    MPS_OP_PND_NEIGH_NPCD,       /* calcPndnNeighNPCD  src/MpsPndNeigh.cpp:199-331                   */
    MPS_OP_PND_DIFFUSIVE,        /* calcPndDiffusiveTerm (+wall), updatePnd,
                                    meanPndParticlesWallDummySurface  src/MpsPndNeigh.cpp:334-852   */
    MPS_OP_PND_MEAN,             /* meanWallPnd + meanPnd  src/MpsPndNeigh.cpp:855-994              */
    MPS_OP_UPDATE_BC,            /* updateParticleBC  src/MpsBoundaryCondition.cpp:66-400            */
    MPS_OP_CALC_PRESS,           /* calcPress (EOS or PPE+CG+clamp)  src/MpsPressure.cpp:32-476     */
    MPS_OP_EXTRAPOLATE_PRESS,    /* extrapolatePressParticlesWallDummy  src/MpsPressure.cpp:792-846 */
    MPS_OP_PRESS_GRADIENT,       /* calcPressGradient  src/MpsPressure.cpp:1217-1338                 */
    MPS_OP_WALL_PRESS_GRADIENT,  /* calcWallPressGradient  src/MpsPressure.cpp:1341-1550             */
    MPS_OP_WALL_VISCOSITY,       /* calcWall{NoSlip,Slip}Viscosity  src/MpsViscosity.cpp:1527-1910  */
    MPS_OP_CORRECT,              /* correctionVelocityPosition  src/MpsParticleVelPos.cpp:53-97      */
    MPS_OP_SHIFTING,             /* calcShifting / calcConcAndConcGradient (+wall)
                                    src/MpsShifting.cpp:23-101, 432-691                             */
    MPS_OP_DUMMY_VELOCITY,       /* updateVelocityParticlesWallDummy  src/MpsParticleVelPos.cpp:100-158 */
    MPS_OP_INIT_PND,             /* step-0 sequence src/main.cpp:158-166: setInitialPnd..., meanWallPnd,
                                    meanPnd, meanNeighFluidPnd                                       */
    MPS_OP_PREDICT_PRESS_GRADIENT, /* relax_fact < 1 only (src/main.cpp:271-276), before PREDICT:
                                    predictionPressGradient  src/MpsPressure.cpp:932-1028,
                                    predictionWallPressGradient  src/MpsPressure.cpp:1031-1214      */
    MPS_OP_COUNT
};

/* PPE solver selection (mpsgpu_set_solver).  PLAIN_FP64 is the drop-in for Eigen's
 * ConjugateGradient (src/MpsPressure.cpp:424-445): Jacobi-preconditioned CG in FP64,
 * warm-started from the previous unclamped solution.  MIXED runs FP32 SpMV/CG inner
 * solves under FP64 iterative refinement (FP64 residual r=b-Ax, FP64 dots).  The final
 * FP64 relative residual judges every solver: a MIXED solve (any warm start, the learned
 * one included) that misses the tolerance within max_iter is redone by PLAIN_FP64 from
 * the previous unclamped solution with its own max_iter (MpsStepStats.ppeFallback). */
#define MPSGPU_SOLVER_PLAIN_FP64   0
#define MPSGPU_SOLVER_MIXED        1
/* MIXED with a matrix-free inner operator: the FP32 off-diagonals are recomputed from the
 * particle positions in every inner SpMV (coeffPPE w(r_ij), entries marked at assembly)
 * instead of streamed from the assembled matrix; FP64 residuals use the assembled matrix.
 * Needs the single-launch PPE solve (mpsgpu_set_ppe_launch). */
#define MPSGPU_SOLVER_MIXED_MATFREE 2
/* MIXED with a compact inner operator: the FP32 inner CG runs on the symmetrically scaled
 * matrix diag(sign(A_ii)/sqrt|A_ii|) A diag(1/sqrt|A_ii|) (unit diagonal, no
 * preconditioner), stored as FP16 values with 16-bit column offsets (4 bytes per entry);
 * FP64 residuals use the assembled FP64 matrix.  Needs the single-launch PPE solve. */
#define MPSGPU_SOLVER_MIXED_COMPACT 3
#define MPSGPU_WARM_PREVIOUS       0   /* previous-step unclamped pressure (reference)  */
#define MPSGPU_WARM_MLP            1   /* learned per-particle MLP correction           */
#define MPSGPU_WARM_ZERO           2
#define MPSGPU_WARM_EXTRAPOLATE    3   /* 2 p_n - p_{n-1} of the unclamped solutions       */
#define MPSGPU_WARM_EXTRAPOLATE2   4   /* 3 p_n - 3 p_{n-1} + p_{n-2} (quadratic)         */

typedef struct mpsgpu_s* mpsgpu_t;

/* Derive the constants of MpsParticle::setParameters (src/MpsParticle.cpp:136-227) and
 * the bucket grid of MpsBucket::allocateMemory/calcDomainLimits (src/MpsBucket.cpp:20-295).
 * Host only (no GPU needed).  pos3 (N x 3) is only read for particle walls
 * (calcDomainLimits with limitTypeBC 0). */
int mpsgpu_params_derive(MpsParams* p, int n, const double* pos3);

/* Host-only check (no GPU needed) of the input switches against the implemented path:
 * 0, or MPSGPU_ERR_UNSUPPORTED with mpsgpu_last_error(NULL) naming the JSON switch and
 * the reason (deformable/forced meshes, periodic domains, non-Newtonian rheology,
 * unknown solver/collision/wall types).  mpsgpu_create makes the same
 * check.  Replaces the reference's silent acceptance of switches it marks "NOT WORKING"
 * (input/InputDamINC.json flags). */
int mpsgpu_check_params(const MpsParams* p);

/* Upload a particle system: replaces MpsInputOutput::readMpsParticleFile's arrays
 * (src/MpsInputOutput.cpp:645-857) plus PolygonMesh::initPolygonMesh/readPolygonMeshFile
 * (src/PolygonMesh.cpp:18-108) and initWijnNeigh (src/PolygonMesh.cpp:377-527).
 * p must have been derived.  mesh may be NULL for particle walls. */
int mpsgpu_create(const MpsParams* p, int n, const int* type, const double* pos3,
                  const double* vel3, const double* press, const MpsMesh* mesh,
                  mpsgpu_t* out);
int mpsgpu_destroy(mpsgpu_t h);

/* The step-0 sequence of main() (src/main.cpp:116-180): bucket update, out-of-domain,
 * initMesh wall distance, initial PND, mean PND smoothing, BC and the step-0 pressure. */
int mpsgpu_initialize(mpsgpu_t h);

/* One iteration of mainLoopOfSimulation (src/main.cpp:256-467), in the reference order. */
int mpsgpu_step(mpsgpu_t h, MpsStepStats* stats);
/* nsteps iterations back to back; stats (may be NULL) receives the last step's figures. */
int mpsgpu_run(mpsgpu_t h, int nsteps, MpsStepStats* stats);

/* One operator (see MpsOp) on the current device state. */
int mpsgpu_run_op(mpsgpu_t h, int op);
/* Figures of the last step or operator (PPE iterations/residual/timings after CALC_PRESS);
 * what PolyMPS reads through MpsPressure::getSolverIter/getSolverError
 * (include/MpsPressure.h:242-253). */
int mpsgpu_last_stats(mpsgpu_t h, MpsStepStats* out);

/* Solver controls, replacing the fixed Eigen CG of src/MpsPressure.cpp:424-445. */
int mpsgpu_set_solver(mpsgpu_t h, int solver, int warm_start, double tol, int max_iter);

/* Arithmetic of the neighbour sweeps (no reference counterpart: the reference is FP64
 * throughout).  FP64 (default) evaluates every pair in FP64 like the reference.  DF32
 * evaluates pair vectors, weights and sums in float-float (two FP32 numbers, ~48 bits)
 * and keeps every discrete decision (neighbour radius, mirror side, collision sign) equal
 * to the reference's by deciding in FP64 whenever the float-float value lies within its
 * error margin; per-particle results differ from FP64 by ~1e-11 relative.  Operators
 * without a DF32 kernel (diffusive/mean PND, extrapolation, dummy velocity, step-0 PND)
 * run their FP64 kernels in either mode. */
/* How the PPE solve is launched: 0 one launch per kernel with the host polling
 * convergence every few iterations; 1 (default) the whole solve in one cooperative launch
 * with device-side grid barriers (the mixed solver with every block owning one contiguous,
 * work-balanced range of rows and keeping its FP32 inner-CG vectors in shared memory, where
 * the rows fit: up to 13,824 rows per SM); 2 as 1, with the mixed solver's FP32 matrix
 * streamed through shared memory by bulk copies (measured slower than 1 at 864k rows: the
 * SpMV is bound by the neighbour gathers of z, not by the matrix stream); 3 as 1, with the
 * mixed solver's inner CG in the pipelined form (one grid reduction per iteration instead
 * of two, Ghysels & Vanroose 2014) and the refinement residual formed in the same pass as
 * the iterate update; 4 as 1 with grid-stride rows and every solver vector in global
 * memory.  Same method and results to the solver tolerance.
 * Modes 1 to 4 fall back to the previous modes where the device does not support them. */
int mpsgpu_set_ppe_launch(mpsgpu_t h, int mode);

#define MPSGPU_PRECISION_FP64  0
#define MPSGPU_PRECISION_DF32  1
int mpsgpu_set_precision(mpsgpu_t h, int precision);

/* Field transfer in the reference's host layout (see MpsField).  get writes
 * numParticles entries; set reads numParticles entries. */
int mpsgpu_get_field(mpsgpu_t h, int field, void* host);
int mpsgpu_set_field(mpsgpu_t h, int field, const void* host);
int mpsgpu_num_particles(mpsgpu_t h, int* n);
int mpsgpu_time(mpsgpu_t h, double* t, int* iterations);

/* Neighbour lists of the current positions through the current (stale) bucket list,
 * as every reference sweep sees them (the 27-bucket scan of e.g. src/MpsPndNeigh.cpp:209-258
 * with dst^2 < reL^2, j != i): counts[N] and, if nbr != NULL, the entries of particle i
 * at nbr[offsets(i) ...] in scan order, offsets being the exclusive prefix sum of counts.
 * nbr must hold sum(counts) ints.  Used by the bit-exact neighbour-set tests. */
int mpsgpu_get_neighbors(mpsgpu_t h, int* counts, int* nbr, long long nbr_capacity);

/* Last PPE system (ELL rows as CSR on the host): rowptr[N+1], col/val[nnz], rhs[N].
 * nnz_out receives the count; pass col == NULL to query it. */
int mpsgpu_get_ppe(mpsgpu_t h, long long* nnz_out, long long* rowptr, int* col,
                   double* val, double* rhs);

/* Learned warm start (N2): MLP 16->64->64->64->1, GELU (tanh form), BF16 weights, FP32 accumulate.
 * Weights are the FP32 master copy in this packed order:
 * W1[64x16] b1[64] W2[64x64] b2[64] W3[64x64] b3[64] W4[1x64] b4[1]  (row-major [out][in]),
 * The normalisation vector holds MPSGPU_MLP_NNORM floats: feature means[16], feature
 * inverse spreads[16], then the target's mean and inverse spread.  The network predicts
 * the correction c of the quadratic extrapolation x_e = 3 p_n - 3 p_{n-1} + p_{n-2}; features 1, 5, 7,
 * 14 (pressure differences) and the target are in units of the system scale sigma (RMS
 * over the equation rows of feature 7, the Jacobi step of the extrapolation residual).
 * The warm start is x_e + theta c with theta = argmin ||b - A (x_e + theta c)||, so the
 * start is never worse than the extrapolation in the residual norm. */
#define MPSGPU_MLP_NPARAM (64*16 + 64 + 64*64 + 64 + 64*64 + 64 + 64 + 1)
#define MPSGPU_MLP_NFEAT  16
#define MPSGPU_MLP_NNORM  34
int mpsgpu_mlp_set_weights(mpsgpu_t h, const float* params, const float* norm32);
int mpsgpu_mlp_get_weights(mpsgpu_t h, float* params, float* norm32);
/* Raw features of the current PPE system, N x 16 FP32 (host; before the sigma scaling). */
int mpsgpu_ppe_features(mpsgpu_t h, float* feat);
/* Training on the GPU with the library's own forward/backward/Adam kernels.  While
 * recording is enabled, every PPE solve appends (features, converged pressure minus
 * x_e, both scaled by sigma) of its equation rows to a device-resident training set. */
int mpsgpu_mlp_record(mpsgpu_t h, int enable);
int mpsgpu_mlp_num_records(mpsgpu_t h, long long* n);
int mpsgpu_mlp_fit_normalization(mpsgpu_t h);
/* iters Adam steps on mini-batches of `batch` recorded samples (multiple of 64);
 * loss_hist (may be NULL) receives iters mean-squared losses. */
int mpsgpu_mlp_train(mpsgpu_t h, int iters, int batch, float lr, unsigned long long seed,
                     float* loss_hist);
/* Network outputs for n host rows of raw features (N x 16 FP32). */
int mpsgpu_mlp_forward(mpsgpu_t h, const float* feat, int n, float* out);
/* Gradient (MPSGPU_MLP_NPARAM floats) and loss of the mean squared error of n host
 * samples (n a multiple of 64), no optimiser step. target is in normalised units. */
int mpsgpu_mlp_gradient(mpsgpu_t h, const float* feat, const float* target, int n,
                        float* grad, float* loss);

/* Device stream used by the handle (cudaStream_t as void*), for callers that
 * interleave their own work. */
int mpsgpu_stream(mpsgpu_t h, void** stream);

/* Human-readable text for the last error of this handle (or of the library if h==NULL). */
const char* mpsgpu_last_error(mpsgpu_t h);

/* ABI check for bindings: sizeof(MpsParams), sizeof(MpsStepStats), sizeof(MpsMesh). */
int mpsgpu_abi_sizes(int* params, int* stats, int* mesh);

/* Binary .vtu output written from device buffers (replaces MpsInputOutput::writeVtuAscii,
 * src/MpsInputOutput.cpp:1313-1580, and its non-working binary variant :921-1310): the same
 * arrays, names and types as the ASCII writer (Float32 values, Int32 flags, UInt8 cell
 * types), converted and reordered into the reference's particle order on the device and
 * copied to the host as one block, written as raw appended data with UInt32 headers.
 * groups: the optional arrays of the JSON's output_VTU section. */
#define MPSGPU_VTU_PND            1u   /* pnd, pndSmall */
#define MPSGPU_VTU_NEIGH          2u   /* nNeigh */
#define MPSGPU_VTU_DEVIATION      4u   /* npcdDeviation, polygonNormal */
#define MPSGPU_VTU_CONCENTRATION  8u   /* concentration, GradCi */
#define MPSGPU_VTU_AUXILIAR      16u   /* ParticleType (+ nearMeshType with polygon walls) */
int mpsgpu_write_vtu(mpsgpu_t h, const char* path, unsigned int groups);

/* Device timing per operator with CUDA events on the handle's stream (the per-kernel
 * timer the reference lacks; it only prints wall time, src/MpsInputOutput.cpp:31-55).
 * Classes 0..MPS_OP_COUNT-1 are the MpsOp operators, followed by NEIGHBOR_LIST,
 * PPE_ASSEMBLE, PPE_SPMV, PPE_VECTOR, PPE_OTHER, PPE_SOLVE (a whole solve in one launch).
 * Enabling resets the totals. */
#define MPSGPU_PROF_NCLASS (MPS_OP_COUNT + 6)
int mpsgpu_profile(mpsgpu_t h, int enable);
int mpsgpu_profile_get(mpsgpu_t h, int cls, double* ms, long long* calls);
const char* mpsgpu_profile_name(int cls);
/* Kernels launched by this library in this process so far. */
int mpsgpu_launch_count(long long* n);

/* Allocation-free pressure solve (no counterpart in the reference, whose Eigen
 * ConjugateGradient allocates its own work vectors on every solve).  For callers that
 * cannot allocate device memory when they solve: an application whose device memory is
 * owned by another framework's pool, or a stepping loop that forbids allocation once it
 * runs.  Jacobi-preconditioned CG with Eigen's stopping rule (|r| < tol |b|) on a CSR
 * system whose arrays (rowptr[n+1], col/val[nnz], b[n], x[n]) are DEVICE pointers; x holds
 * the initial guess on entry and the solution on return.  All work vectors live in one
 * file-scope device array of MPSGPU_STATIC_MAX_ROWS rows (about 5.3 MB per device),
 * reserved when the library's device code is loaded on a device (at the latest by the
 * first call there): the call itself makes no device allocation.  Rules:
 *  - n must be 1..MPSGPU_STATIC_MAX_ROWS, otherwise MPSGPU_ERR_ARG;
 *  - every row needs a stored non-zero diagonal entry (Jacobi scaling); otherwise the
 *    call returns MPSGPU_ERR_ARG naming the first such row, with x untouched;
 *  - b = 0 gives x = 0, 0 iterations and relres 0 (Eigen's CG returns the same);
 *  - each call clears the array's control words itself; nothing needs zeroing first;
 *  - the array is shared by every call on a device: calls that overlap on the GPU
 *    (two streams, two host threads) race and corrupt each other;
 *  - the first call on a device looks the array's address up with that device
 *    current; make it before any stream capture begins.
 * The call synchronises `stream` (cudaStream_t as void*, may be NULL) to poll
 * convergence.  iters / relres (may be NULL) receive the iteration count and the true
 * relative residual |b - Ax| / |b|.  mpsgpu_pcg_static_error() gives the last message. */
#define MPSGPU_STATIC_MAX_ROWS (1 << 17)
int mpsgpu_pcg_solve_static(int n, const int* rowptr, const int* col, const double* val,
                            const double* b, double* x, double tol, int max_iter, void* stream,
                            int* iters, double* relres);
const char* mpsgpu_pcg_static_error(void);

#ifdef __cplusplus
}
#endif
#endif /* MPSGPU_H_ */
