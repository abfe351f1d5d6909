// mps_cellscan.cuh — warp-per-bucket staged neighbour scan.
//
// The reference's sweeps scan, for every particle i, the 27 (9 in 2D) buckets around the
// bucket of its current position (bucketCoordinates, src/MpsBucket.cpp:420-425) through
// the stale bucket lists.  All particles whose current position falls in the same bucket
// share that candidate set, so particles are grouped by this "query bucket" and one warp
// takes one query bucket: the warp stages the candidates (indices and FP32 positions) of
// the 27 buckets into shared memory once, in the reference order (z, y, x, ascending
// index), and every lane — one particle of the query bucket — walks them from shared
// memory (broadcast reads).  This replaces per-thread dependent global gathers and
// divergent trip counts with one cooperative load per bucket neighbourhood.
//
// Op provides: struct State; begin(d, i, st); visit(d, i, st, j, fj); end(d, i, st).
// Particles whose bucket coordinates fall outside the grid are handled by the per-thread
// fallback k_cellscan_stray (the reference reads out of bounds there).
#pragma once
#include "mps_common.cuh"

#define CS_WARPS 4
#define CS_CAP 448

template <class Op>
__global__ void __launch_bounds__(32 * CS_WARPS) k_cellscan(Dev d, Op op) {
    __shared__ int sIdx[CS_WARPS][CS_CAP];
    __shared__ float4 sPos[CS_WARPS][CS_CAP];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const MpsParams& P = d.P;
    const int ncells = *d.qNum;
    const int dz = (int)(P.dim - 2.0);
    const int nbk = 9 * (2 * dz + 1);
    for (int slot = blockIdx.x * CS_WARPS + w; slot < ncells; slot += gridDim.x * CS_WARPS) {
        const int c = d.qList[slot];
        const int iz = c / P.numBucketsXY;
        const int rem = c - iz * P.numBucketsXY;
        const int iy = rem / P.numBucketsX;
        const int ix = rem - iy * P.numBucketsX;
        const int minZ = (iz - 1) * dz;
        const int p0 = d.qStart[c], p1 = d.qStart[c + 1];
        for (int pb = p0; pb < p1; pb += 32) {
            const bool act = pb + lane < p1;
            const int i = act ? d.qSorted[pb + lane] : -1;
            typename Op::State st;
            if (act) op.begin(d, i, st);
            int b = 0, off = 0;
            while (b < nbk) {
                int n = 0;
                while (b < nbk && n < CS_CAP) {
                    int kz = b / 9, ky = (b / 3) % 3, kx = b % 3;
                    long long jb = (long long)(minZ + kz) * P.numBucketsXY + (long long)(iy - 1 + ky) * P.numBucketsX + (ix - 1 + kx);
                    if (jb < 0 || jb >= d.nB) { b++; off = 0; continue; }
                    int s0 = d.cellStart[jb], s1 = d.cellStart[jb + 1];
                    int len = s1 - s0 - off;
                    int take = min(len, CS_CAP - n);
                    for (int t = lane; t < take; t += 32) {
                        int j = d.cellSorted[s0 + off + t];
                        sIdx[w][n + t] = j;
                        sPos[w][n + t] = d.posf[j];
                    }
                    n += take;
                    off += take;
                    if (off >= s1 - s0) { b++; off = 0; }
                }
                __syncwarp();
                if (act)
                    for (int k = 0; k < n; k++) op.visit(d, i, st, sIdx[w][k], sPos[w][k]);
                __syncwarp();
            }
            if (act) op.end(d, i, st);
        }
    }
}

template <class Op>
__global__ void __launch_bounds__(128) k_cellscan_stray(Dev d, Op op) {
    int ns = *d.strayNum;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ns; t += gridDim.x * blockDim.x) {
        int i = d.strayList[t];
        typename Op::State st;
        op.begin(d, i, st);
        forCells(d, d.pos[i], [&](int j) { op.visit(d, i, st, j, d.posf[j]); });
        op.end(d, i, st);
    }
}

// Grid size for the staged scan: enough warps to cover the occupied buckets, capped.
static inline int cellscanBlocks(int nB) {
    int b = (nB + CS_WARPS - 1) / CS_WARPS;
    return b < 152 * 16 ? (b > 0 ? b : 1) : 152 * 16;
}

template <class Op>
void launchCellScan(const Dev& d, const Op& op, cudaStream_t s) {
    k_cellscan<Op><<<cellscanBlocks(d.nB), 32 * CS_WARPS, 0, s>>>(d, op);
    k_cellscan_stray<Op><<<8, 128, 0, s>>>(d, op);
}
