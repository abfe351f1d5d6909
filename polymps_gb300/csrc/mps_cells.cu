// mps_cells.cu — bucket list (MpsBucket::updateParticlesID, src/MpsBucket.cpp:299-353) as
// a counting sort, and the ELL neighbour list of the current positions through that
// stale list (the 27-bucket scan shared by every operator, e.g. src/MpsPndNeigh.cpp:209-258).
//
// Both are HBM/L2-latency bound integer work: one coalesced pass over the particles for
// the bucket keys, atomics into the per-bucket counters, a device-wide scan, a scatter
// and a per-bucket insertion sort that restores ascending particle order (the
// reference's linked lists are filled in ascending index order).
#include <atomic>
#include "mps_df.cuh"
#include "mps_internal.h"

__global__ void k_posf_cell(Dev d);

static std::atomic<long long> g_launches{0};
void countLaunch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launchCount() { return g_launches.load(std::memory_order_relaxed); }

// ------------------------------------------------------------------ bucket keys
// Warp-level counting: the lanes of a warp that share a bucket key (most of them, since the
// storage is kept in bucket order) form one group; its lowest lane adds the group's size to
// the bucket's counter (or cursor) and every lane's place is the group's base plus its rank
// among the group's lanes (lane order = particle order).  Returns that place.
__device__ __forceinline__ int warpGroupAdd(int* counters, int key, bool active) {
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!active) return -1;
    const unsigned grp = __match_any_sync(act, key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(grp) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counters + key, __popc(grp));
    base = __shfl_sync(grp, base, leader);
    return base + __popc(grp & ((1u << lane) - 1u));
}

// One bucket coordinate of updateParticlesID: (int)((x - min) * inv) in 3D,
// (int)((x - min) * inv + eps) in 2D, with dx = x - min (exact FP64 subtraction, the
// reference's first operation).  The FP32 product of the particle's FP32 copy h = fl32(dx)
// and fl32(inv) lies within 3 * 2^-24 relative of the FP64 one, so its truncation is exact
// unless it is within a margin of an integer (or below it); those rare cases evaluate the
// FP64 expression out of line (inlined, the compiler would predicate it into every thread).
static __device__ __noinline__ int bucketKeyCoordExact(double dx, double inv, double eps, bool withEps) {
    const double q = xmul(dx, inv);
    return (int)(withEps ? xadd(q, eps) : q);
}
__device__ __forceinline__ int bucketKeyCoord(float h, double dx, float invf, float epsf, double inv, double eps,
                                              bool withEps) {
    const float q = withEps ? fmaf(h, invf, epsf) : h * invf;
    const float m = 5e-7f * fabsf(q) + 1e-6f;
    const float f = q - floorf(q);
    if (q > m && f > m && f < 1.0f - m) return (int)q;
    return bucketKeyCoordExact(dx, inv, eps, withEps);
}

// 2D adds epsilonZero, 3D does not (src/MpsBucket.cpp:312-313 vs :333-335); ghosts skipped.
// Every lane of a warp reaches the warp-level count (lanes past N0 take part without a key).
__global__ void k_cell_key(Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = liveN(d);
    int key = -1;
    if (i < n && d.type[i] == d.P.ghost) {
        key = d.nB;   // live, in no bucket: listed after the buckets, never scanned
    } else if (i < n) {
        const MpsParams& P = d.P;
        dvec4 p = d.pos[i];
        // x - min once: the key's first operation and the FP32 copies' argument
        const double dx = xsub(p.x, P.domainMin[0]), dy = xsub(p.y, P.domainMin[1]), dzz = xsub(p.z, P.domainMin[2]);
        const float4 hi = make_float4(d2fRN(dx), d2fRN(dy), d2fRN(dzz), 0.f);
        const bool two = (int)P.dim == 2;
        int ix = bucketKeyCoord(hi.x, dx, d.invSidef, d.epsf, P.invBucketSide, P.epsilonZero, two);
        int iy = bucketKeyCoord(hi.y, dy, d.invSidef, d.epsf, P.invBucketSide, P.epsilonZero, two);
        int iz = two ? 0 : bucketKeyCoord(hi.z, dzz, d.invSidef, d.epsf, P.invBucketSide, P.epsilonZero, false);
        long long ib = (long long)iz * P.numBucketsXY + (long long)iy * P.numBucketsX + ix;
        if (ib < 0 || ib >= d.nB) {
            setErr(d, MPSE_DOMAIN);
            key = d.nB;
        } else {
            key = (int)ib;
        }
        // FP32 copy of the start-of-step positions for the prefiltered scans (hi, lo parts)
        d.posf[i] = hi;
        d.posLo[i] = make_float4(d2fRN(dx - f2dExact(hi.x)), d2fRN(dy - f2dExact(hi.y)), d2fRN(dzz - f2dExact(hi.z)), 0.f);
    }
    warpGroupAdd(d.cellCount, key, key >= 0);
    if (i < d.N0) d.cellOf[i] = key;
}

__global__ void k_cell_scatter(Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = (i < d.N0) ? d.cellOf[i] : -1;
    const int r = warpGroupAdd(d.cellCursor, c, c >= 0);
    if (c >= 0) d.cellSorted[d.cellStart[c] + r] = i;
}

// Order each bucket by reference index (the reference's linked-list order; buckets hold
// ~16 particles).  The range after the last bucket is ordered the same way.
__global__ void k_cell_sort(Dev d) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c > d.nB) return;
    int s0 = d.cellStart[c], s1 = d.cellStart[c + 1];
    for (int a = s0 + 1; a < s1; a++) {
        int v = d.cellSorted[a];
        int ov = d.orig[v];
        int b = a - 1;
        while (b >= s0 && d.orig[d.cellSorted[b]] > ov) { d.cellSorted[b + 1] = d.cellSorted[b]; b--; }
        d.cellSorted[b + 1] = v;
    }
}

// ------------------------------------------------------------------ exclusive scan
// Three-phase block scan for int arrays (n <= 4096 * 4096).
#define SCAN_BLOCK 1024
#define SCAN_PER_THREAD 4
#define SCAN_TILE (SCAN_BLOCK * SCAN_PER_THREAD)

__device__ __forceinline__ int blockExclusiveScan(int v, int* smem, int& total) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = (lane < (int)(blockDim.x >> 5)) ? smem[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        smem[lane] = w;
    }
    __syncthreads();
    int warpPrefix = (warp > 0) ? smem[warp - 1] : 0;
    total = smem[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warpPrefix + x - v;
}

__global__ void k_scan_tiles(const int* in, int* out, int* tileSums, int n) {
    __shared__ int smem[32];
    int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
    int v[SCAN_PER_THREAD];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_PER_THREAD; k++) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        s += v[k];
    }
    int total;
    int pre = blockExclusiveScan(s, smem, total);
#pragma unroll
    for (int k = 0; k < SCAN_PER_THREAD; k++) {
        if (base + k < n) out[base + k] = pre;
        pre += v[k];
    }
    if (threadIdx.x == 0 && tileSums) tileSums[blockIdx.x] = total;
}

__global__ void k_scan_add(int* out, const int* tileOffsets, int n, int* totalOut) {
    int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
    int add = tileOffsets[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_PER_THREAD; k++)
        if (base + k < n) out[base + k] += add;
    (void)totalOut;
}

// out[0..n) = exclusive scan of in; out[n] = total.  scratch holds >= 2*tiles+2 ints.
void scanExclusive(const int* in, int* out, int n, int* scratch, cudaStream_t s) {
    int tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    int* tileSums = scratch;
    int* tileOffsets = scratch + tiles + 1;
    k_scan_tiles<<<tiles, SCAN_BLOCK, 0, s>>>(in, out, tileSums, n);
    // second level: one tile covers up to 4096 tiles
    k_scan_tiles<<<1, SCAN_BLOCK, 0, s>>>(tileSums, tileOffsets, tileOffsets + tiles, tiles);
    k_scan_add<<<tiles, SCAN_BLOCK, 0, s>>>(out, tileOffsets, n, nullptr);
    // total = offset of last tile + its sum
    cudaMemcpyAsync(out + n, tileOffsets + tiles, sizeof(int), cudaMemcpyDeviceToDevice, s);
}
int scanScratchInts(int n) { return 2 * ((n + SCAN_TILE - 1) / SCAN_TILE) + 4; }

// ------------------------------------------------------------------ renumbering
// Storage renumbering into the order of the bucket list just built: slot s receives the
// particle listed at s (live particles; slots beyond the live count keep theirs), every
// per-particle array is gathered through a scratch buffer, the reference-index maps follow,
// and the list becomes the identity.  Neighbours are then stored next to each other, which
// is what the gathers of every sweep and the coalescing of the bucket-order scans want.
__global__ void k_perm_build(Dev d, int* perm) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.N0) return;
    perm[s] = (s < *d.nLive) ? d.cellSorted[s] : s;
}
template <class T>
__global__ void k_gather(const T* src, T* dst, const int* perm, int n) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) dst[s] = src[perm[s]];
}
__global__ void k_perm_maps(Dev d, const int* perm, const int* origOld) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.N0) return;
    int r = origOld[perm[s]];
    d.orig[s] = r;
    d.slotOf[r] = s;
    if (s < *d.nLive) d.cellSorted[s] = s;
}
template <class T>
static void permute(T* a, const int* perm, void* scratch, int n, cudaStream_t s) {
    if (!a) return;
    k_gather<T><<<gridFor(n, 256), 256, 0, s>>>(a, (T*)scratch, perm, n);
    cudaMemcpyAsync(a, scratch, sizeof(T) * n, cudaMemcpyDeviceToDevice, s);
}
int renumberLaunches() { return 1 + (15 + 17 + 5 + 3) + 1; }
static void launchRenumber(const Dev& d, int* perm, void* scratch, cudaStream_t s) {
    const int n = d.N0;
    k_perm_build<<<gridFor(n, 256), 256, 0, s>>>(d, perm);
    for (dvec4* v : {d.pos, d.vel, d.acc, d.accStar, d.mirror, d.wallPos, d.polyNormal, d.normal, d.npcd, d.gradC,
                     d.forceWall, d.c1, d.c2, d.c3, d.dvel, d.shift})
        permute(v, perm, scratch, n, s);
    for (double* v : {d.press, d.pressPPE, d.pressPPEprev, d.pressPPEprev2, d.pndi, d.pndki, d.pndski, d.pndSmall, d.npcd2, d.conc,
                      d.velDiv, d.diffTerm, d.pndWall, d.riw2, d.devDot, d.source, d.aux1, d.aux2})
        permute(v, perm, scratch, n, s);
    for (int* v : {d.type, d.bc, d.numNeigh, d.nNeighWall, d.nearWall}) permute(v, perm, scratch, n, s);
    permute(d.posf, perm, scratch, n, s);
    permute(d.posLo, perm, scratch, n, s);
    permute(d.cellOf, perm, scratch, n, s);
    // maps: the old orig goes through the scratch (the gather reads it while writing orig)
    cudaMemcpyAsync(scratch, d.orig, sizeof(int) * n, cudaMemcpyDeviceToDevice, s);
    k_perm_maps<<<gridFor(n, 256), 256, 0, s>>>(d, perm, (const int*)scratch);
}

__global__ void k_cell_pos(Dev d) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < d.cellStart[d.nB + 1]) d.cellPos[d.cellSorted[p]] = p;
}

void launchBuckets(const Dev& d, int* scanScratch, cudaStream_t s, int* perm, void* permScratch) {
    cudaMemsetAsync(d.cellCount, 0, sizeof(int) * (d.nB + 2), s);
    cudaMemsetAsync(d.cellCursor, 0, sizeof(int) * (d.nB + 2), s);
    k_cell_key<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
    scanExclusive(d.cellCount, d.cellStart, d.nB + 1, scanScratch, s);
    k_cell_scatter<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
    k_cell_sort<<<gridFor(d.nB + 1, 256), 256, 0, s>>>(d);
    if (perm) launchRenumber(d, perm, permScratch, s);
    cudaMemsetAsync(d.cellPos, 0xff, sizeof(int) * d.N0, s);
    k_cell_pos<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
    k_posf_cell<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
}

// ------------------------------------------------------------------ FP32 copy
__global__ void k_posf(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N0) return;   // every slot: stale bucket entries may name removed particles
    dvec4 p = d.pos[i];
    float4 hi = make_float4(d2fRN(p.x - d.P.domainMin[0]), d2fRN(p.y - d.P.domainMin[1]),
                            d2fRN(p.z - d.P.domainMin[2]), 0.f);
    d.posf[i] = hi;
    d.posLo[i] = posLoOf(p, hi, d.P);
}

// ------------------------------------------------------------------ neighbour list
// FP32 copy of the positions in bucket order, refreshed whenever positions change.
__global__ void k_posf_cell(Dev d) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.cellStart[d.nB]) return;
    int j = d.cellSorted[s];
    d.posfCell[s] = d.posf[j];
    d.posLoCell[s] = d.posLo[j];
}
void launchPosfCell(const Dev& d, cudaStream_t s) {
    k_posf_cell<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
}
void launchPosf(const Dev& d, cudaStream_t s) {
    k_posf<<<gridFor(d.N0, 256), 256, 0, s>>>(d);
    launchPosfCell(d, s);
}

// Candidates are tested in FP32 first; only those whose FP32 squared distance falls in
// the rounding band around the list radius^2 are re-tested in exact FP64, so membership
// equals the reference's FP64 test dst^2 < re^2 bit for bit while almost all candidate
// work is FP32 on contiguous bucket-ordered records.  Every accepted entry also gets its
// weights for the epoch: w(r; reS), w/r^2 and, when the radii differ, w(r; reL) — the
// FP64 divisions and square roots of all later sweeps happen here once.
__global__ void __launch_bounds__(128) k_build_nbr(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    dvec4 pi = d.pos[i];
    float4 fi = d.posf[i];
    int cnt = 0;
    const size_t N0 = d.N0;
    forCellsNear(d, pi, fi, d.bandHi, [&](int j, dvec4 pj, PairG q) {
        if (j == i || !(q.d2 < d.reMax2)) return;
        if (cnt < d.K) {
            size_t e = (size_t)cnt * N0 + i;
            d.nbr[e] = j;
            double w, wd;
            weightR(q.d2, P.reS, P.weightType, w, wd);
            d.cw[e] = w;
            d.cwd[e] = wd;
            if (d.cwL) { double wl, wdl; weightR(q.d2, P.reL, P.weightType, wl, wdl); d.cwL[e] = wl; }
        }
        cnt++;
    });
    if (cnt > d.K) { setErr(d, MPSE_CAPACITY); cnt = d.K; }
    d.nbrCount[i] = cnt;
    warpCount(d.counters, (unsigned)cnt);
}

// Per-entry weights of the current list for the FP64 sweeps, when the list was built by
// the DF32 tier (which stores none); the same expressions as k_build_nbr.
__global__ void __launch_bounds__(128) k_fill_cache(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    dvec4 pi = d.pos[i];
    int c = d.nbrCount[i];
    for (int k = 0; k < c; k++) {
        size_t e = (size_t)k * d.N0 + i;
        PairG q = pairOf(d.pos[d.nbr[e]], pi);
        double w, wd;
        weightR(q.d2, P.reS, P.weightType, w, wd);
        d.cw[e] = w;
        d.cwd[e] = wd;
        if (d.cwL) { double wl, wdl; weightR(q.d2, P.reL, P.weightType, wl, wdl); d.cwL[e] = wl; }
    }
}
void launchFillCache(const Dev& d, cudaStream_t s) {
    k_fill_cache<<<gridFor(d.N0, 128), 128, 0, s>>>(d);
}

void launchNeighborList(const Dev& d, cudaStream_t s) {
    cudaMemsetAsync(d.counters, 0, sizeof(unsigned long long), s);
    launchPosf(d, s);
    k_build_nbr<<<gridFor(d.N0, 128), 128, 0, s>>>(d);
}

// ------------------------------------------------------------------ entry masks
// After the wall pass: for each particle, which entries are inside the reS / reL ball and
// not on the mirror side (dstij2 < dstimj2, e.g. src/MpsPndNeigh.cpp:249), all in exact
// FP64.  Particles whose mirror is far (see SideCtx) and whose list radius equals the
// ball radius take every entry without per-entry work.  Fluid particles near the wall
// are appended to nearList for the wall-only sweeps.
__global__ void __launch_bounds__(128) k_side_masks(Dev d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= liveN(d)) return;
    const MpsParams& P = d.P;
    int c = d.nbrCount[i];
    const Mask all = maskFirst(c);
    dvec4 pi = d.pos[i];
    SideCtx sc = sideCtx(d, i, pi);
    bool fullS = P.reS2 >= d.reMax2, fullL = P.reL2 >= d.reMax2;
    Mask mS = all, mL = all;
    if (sc.check || !fullS || !fullL) {
        mS = maskNone(); mL = maskNone();
        const int* row = d.nbr + i;
        for (int k = 0; k < c; k++) {
            dvec4 pj = d.pos[__ldg(row + (size_t)k * d.N0)];
            PairG q = pairOf(pj, pi);
            bool side = sideOK(sc, pj, q.d2);
            if (side && q.d2 < P.reS2) maskSet(mS, k);
            if (side && q.d2 < P.reL2) maskSet(mL, k);
        }
    }
    d.maskS[i] = mS;
    d.maskL[i] = mL;
    if (P.wallType == 1 && d.type[i] == P.fluid && d.nearWall[i]) {
        int slot = atomicAdd(d.nearCount, 1);
        d.nearList[slot] = i;
    }
}

void launchSideMasks(const Dev& d, cudaStream_t s) {
    cudaMemsetAsync(d.nearCount, 0, sizeof(int), s);
    k_side_masks<<<gridFor(d.N0, 128), 128, 0, s>>>(d);
}
