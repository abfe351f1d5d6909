// mps_host.h — host-only helpers of libmpsgpu (no CUDA types).
#pragma once
#include <vector>
#include "../../include/mpsgpu.h"

int hostDeriveParams(MpsParams* P, int n, const double* pos);
void hostWallTables(const MpsParams& P, double* tab);     // 4 x 50 doubles
void hostTriNormals(int ntri, const double* tri, double* nrm);
void hostTrianglePlanes(int ntri, const double* tri, double* planes);   // 16 doubles per triangle
// Bounding-volume hierarchy over the triangles for the wall distance of large meshes:
// nodes as (lo, hi) boxes in FP32 relative to `origin`, widened outward by one FP32 ulp of
// every bound so they contain the FP32 copies of the vertices; lo[3]/hi[3] of an internal
// node hold the child indices, of a leaf -(first + 1) and the count into `order` (at most 4
// triangles).  Median split along the widest axis of the centroids.
void hostBuildBvh(int ntri, const double* tri, const double* origin, std::vector<float>& lo4,
                  std::vector<float>& hi4, std::vector<int>& order);
