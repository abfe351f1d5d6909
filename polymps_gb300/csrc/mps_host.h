// mps_host.h — host-only helpers of libmpsgpu (no CUDA types).
#pragma once
#include "../../include/mpsgpu.h"

int hostDeriveParams(MpsParams* P, int n, const double* pos);
void hostWallTables(const MpsParams& P, double* tab);     // 4 x 50 doubles
void hostTriNormals(int ntri, const double* tri, double* nrm);
