// mps_mlp_feat.cuh — the 16 raw features of one row of the learned warm start, formed from
// the FP64 start x_e and its FP64 residual r_e = b - A x_e (the solver's x and r vectors);
// the recorded-feature pass (k_mlp_features) forms the same quantities from FP32 copies.
#pragma once
#include "mps_common.cuh"
#include "mps_internal.h"

#define MLP_NF 16
#define MLP_FSIG 7   // the feature whose RMS over the equation rows is the system scale

// Per-system constants of the features (FP64 divisions and a square root, formed once on
// the host instead of in every thread): the unit vector along g, 1/n0, 1/N0, 1/reL and
// 1/(coeffPPE n0).
struct FeatConst {
    float ggx, ggy, ggz, in0, iN0, iRe, iA;
};

// the row's features (raw: pressure differences 1, 5, 7, 14 in Pa); every FP64 field is
// rounded to FP32 by integer operations (d2fRN), not on the FP64 pipe
__device__ __forceinline__ void featRow64(const Dev& d, const PpeBuffers& B, int i, const FeatConst& K, float* f) {
    const MpsParams& P = d.P;
    const dvec4 x = d.pos[i], v = d.vel[i];
    const float diag = __ldg(B.diagf + i), idg = __ldg(B.diagInvf + i);
    const double pn = d.pressPPE[i];
    const float bi = d2fRN(B.b[i]);
    const float vx = d2fRN(v.x), vy = d2fRN(v.y), vz = d2fRN(v.z);
    f[0] = (d2fRN(d.pndSmall[i]) - d2fRN(P.pndSmallZero)) * K.in0;
    f[1] = bi * idg;
    f[2] = (float)d.numNeigh[i] * K.iN0;
    f[3] = ((__double_as_longlong(pn) << 1) == 0) ? 1.f : 0.f;   // pn == +-0
    f[4] = fminf(sqrtf(d2fRN(d.riw2[i])) * K.iRe, 1.5f);
    f[5] = d2fRN(pn) - d2fRN(d.pressPPEprev[i]);
    f[6] = d2fRN(B.x[i]);
    f[7] = d2fRN(B.r[i]) * idg;
    f[8] = d2fRN(pn);
    f[9] = sqrtf(vx * vx + vy * vy + vz * vz);
    f[10] = -(vx * K.ggx + vy * K.ggy + vz * K.ggz);
    f[11] = diag * K.iA;
    f[12] = d2fRN(d.pndWall[i]);
    f[13] = -(d2fRN(x.x) * K.ggx + d2fRN(x.y) * K.ggy + d2fRN(x.z) * K.ggz);
    f[14] = (bi - d2fRN(d.source[i])) * idg;
    f[15] = (d2fRN(d.pndi[i]) - d2fRN(d.pndki[i])) * K.in0;
}
