// mps_mlp.h — learned PPE warm start (per-particle MLP 16 -> 64 -> 64 -> 64 -> 1, GELU).
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include "mps_common.cuh"

struct PpeBuffers;

struct MlpState {
    bool ready = false;
    int N0 = 0;
    float* master = nullptr;       // FP32 master parameters (MPSGPU_MLP_NPARAM)
    float* adam_m = nullptr;       // Adam first moments
    float* adam_v = nullptr;       // Adam second moments
    float* grad = nullptr;         // gradient accumulator
    __nv_bfloat16* wbf = nullptr;  // BF16 weights W1|W2|W3|W4 (row-major [out][in])
    float* norm = nullptr;         // mean[16], inv_std[16]
    float* feat = nullptr;         // N0 x 16 raw features of the current system
    float* out = nullptr;          // N0 outputs
    // step along the network's correction: residual of the extrapolation, the correction
    // (Pa), block partials of the two dot products and the step length
    float* re = nullptr;
    float* cdir = nullptr;
    float* xe32 = nullptr;         // x_e in FP32 (gathered by the features)
    double* part = nullptr;
    int nblk = 0;
    int nblkFeat = 0;              // blocks of the FP64-start features pass (one wave, <= nblk)
    // system scale: RMS over equation rows of the Jacobi step of the extrapolation residual
    // (pressure-difference features and the target are in its units)
    double* sig = nullptr;         // [0] sigma, [1] step theta
    // training record: features and targets of recorded steps
    float* recFeat = nullptr;
    float* recTarget = nullptr;
    long long recCap = 0, recCount = 0;
    float* lossAcc = nullptr;      // device loss accumulator
    int adamStep = 0;
    bool recording = false;
    int* tcErr = nullptr;          // set by the tensor-core forward when a completion wait ran out
};

int mlpInit(MlpState& m, int n0, cudaStream_t s);
// Network outputs on the tensor cores (tcgen05): rows = *nLive if nLive else n; out = the
// raw output (bc == nullptr) or the learned correction c on rows with bc == inner, 0 on the
// others (sig: the system scale of the raw features, nullptr for normalised inputs as given).
int mlpForwardTc(const MlpState& m, const float* feat, int n, const int* nLive, const int* bc, int inner,
                 const double* sig, float* out, cudaStream_t s);
// 0, or MPSGPU_ERR_CUDA when a tensor-core forward since the last call reported a
// completion wait that ran out (clears the word; synchronises the stream)
int mlpTcStatus(MlpState& m, cudaStream_t s);
void mlpFree(MlpState& m);
int mlpSetWeights(MlpState& m, const float* params, const float* norm32, cudaStream_t s);
int mlpGetWeights(MlpState& m, float* params, float* norm32, cudaStream_t s);
int mlpFeatures(MlpState& m, const Dev& d, const PpeBuffers& B, float* hostFeat, int n, cudaStream_t s);
// Writes the warm start into B.x (assembled system, previous solution in d.pressPPE).
// stepInSolver: B.x = x_e, m.cdir = the network's correction c and m.re = A c only; the
// solver takes the residual-minimising step x_e + theta c in its set-up pass.
int mlpWarmStart(MlpState& m, const Dev& d, const PpeBuffers& B, cudaStream_t s, bool stepInSolver = false);
// Recording / training (device-resident data, own kernels).
int mlpRecordFeatures(MlpState& m, const Dev& d, const PpeBuffers& B, cudaStream_t s);
int mlpRecordTargets(MlpState& m, const Dev& d, const PpeBuffers& B, cudaStream_t s);
int mlpFitNormalization(MlpState& m, cudaStream_t s);
int mlpTrain(MlpState& m, int iters, int batch, float lr, unsigned long long seed, float* lossHist, cudaStream_t s);
int mlpForwardHost(MlpState& m, const float* hfeat, int n, float* hout, cudaStream_t s);
int mlpGradient(MlpState& m, const float* hfeat, const float* htarget, int n, float* hgrad, float* hloss,
                cudaStream_t s);
