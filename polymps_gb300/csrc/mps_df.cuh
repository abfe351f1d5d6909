// mps_df.cuh — float-float ("df") arithmetic for the DF32 precision tier.
//
// GB300 issues 304 FP64 FMA thread-instructions per cycle chip-wide against 19,456 FP32
// FMAs (1/64), so the exact-FP64 neighbour sweeps are bound by the FP64 pipe.  In the DF32
// tier a pair quantity is an unevaluated sum hi + lo of two FP32 numbers (about 48
// significant bits) built only from error-free FP32 transformations: Knuth's TwoSum,
// Dekker's Fast2Sum and the FMA-based TwoProd (as in Dekker 1971; Hida, Li & Bailey's
// double-double library).  Every primitive uses the explicitly rounded intrinsics so the
// compiler cannot contract a product into a later addition (that would break the
// error-free property).  FP64 remains for per-particle conversions, for the final
// per-particle results, and for the rare pairs whose discrete decision (radius, mirror
// side) lies inside the error margin of the float-float value, where the reference's own
// FP64 expression is evaluated instead — so every decision equals the reference's.
#pragma once
#include "mps_common.cuh"

struct df {
    float h, l;
};

__device__ __forceinline__ float fA(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fS(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fM(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fF(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// Fast2Sum (|a| >= |b| or a == 0): s + e == a + b exactly
__device__ __forceinline__ df quick2(float a, float b) {
    float s = fA(a, b);
    return {s, fS(b, fS(s, a))};
}
// TwoSum (any a, b): s + e == a + b exactly
__device__ __forceinline__ df two2(float a, float b) {
    float s = fA(a, b);
    float bb = fS(s, a);
    return {s, fA(fS(a, fS(s, bb)), fS(b, bb))};
}
// TwoProd: p + e == a * b exactly
__device__ __forceinline__ df prod2(float a, float b) {
    float p = fM(a, b);
    return {p, fF(a, b, -p)};
}

__device__ __forceinline__ df dfF(float a) { return {a, 0.f}; }
__device__ __forceinline__ df operator-(df a) { return {-a.h, -a.l}; }
__device__ __forceinline__ df operator+(df a, df b) {
    df s = two2(a.h, b.h);
    return quick2(s.h, fA(s.l, fA(a.l, b.l)));
}
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__device__ __forceinline__ df operator+(df a, float b) {
    df s = two2(a.h, b);
    return quick2(s.h, fA(s.l, a.l));
}
__device__ __forceinline__ df operator-(df a, float b) { return a + (-b); }
__device__ __forceinline__ df operator*(df a, df b) {
    df p = prod2(a.h, b.h);
    return quick2(p.h, fF(a.h, b.l, fF(a.l, b.h, p.l)));
}
__device__ __forceinline__ df operator*(df a, float b) {
    df p = prod2(a.h, b);
    return quick2(p.h, fF(a.l, b, p.l));
}
__device__ __forceinline__ df& operator+=(df& a, df b) { a = a + b; return a; }
__device__ __forceinline__ df& operator-=(df& a, df b) { a = a - b; return a; }
// ordering of normalised values (|l| <= ulp(h)/2)
__device__ __forceinline__ bool operator<(df a, df b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
__device__ __forceinline__ bool operator>(df a, df b) { return b < a; }

// conversions (per particle and per stored value; one FP64 addition each, the FP32 <-> FP64
// conversions in integer operations)
__device__ __forceinline__ df dfD(double x) {
    float h = d2fRN(x);
    return {h, d2fRN(x - f2dExact(h))};
}
__device__ __forceinline__ double dD(df a) { return f2dExact(a.h) + f2dExact(a.l); }

// 1/sqrt(a) for a > 0: FP32 estimate refined by one Newton step in float-float
// (y1 = y + y (1 - a y^2) / 2; the estimate's relative error ~2^-22 becomes ~2^-44).
__device__ __forceinline__ df rsqrtDF(df a) {
    float y = rsqrtf(a.h);
    df y2 = prod2(y, y);
    df t = a * y2;                       // ~1
    float r = fS(fS(1.0f, t.h), t.l);    // 1 - a y^2, exact leading difference
    return quick2(y, fM(fM(y, r), 0.5f));
}

// ------------------------------------------------------------------ particle copies
// Positions are held relative to domainMin as hi = fl32(x - min) (the posf copy the
// prefilters already read) and lo = fl32((x - min) - hi): |x - min - hi - lo| <= 2^-48 |x - min|.
__device__ __forceinline__ float4 posLoOf(dvec4 p, float4 hi, const MpsParams& P) {
    return make_float4(d2fRN((p.x - P.domainMin[0]) - f2dExact(hi.x)), d2fRN((p.y - P.domainMin[1]) - f2dExact(hi.y)),
                       d2fRN((p.z - P.domainMin[2]) - f2dExact(hi.z)), 0.f);
}

struct V3 {
    df x, y, z;
};
// x_j - x_i from the hi/lo copies: the hi difference is split exactly by TwoSum and the
// lo difference added, then renormalised.
__device__ __forceinline__ df diffDF(float hj, float lj, float hi, float li) {
    df s = two2(hj, -hi);
    return quick2(s.h, fA(s.l, fS(lj, li)));
}
__device__ __forceinline__ V3 diff3(float4 hj, float4 lj, float4 hi, float4 li) {
    return {diffDF(hj.x, lj.x, hi.x, li.x), diffDF(hj.y, lj.y, hi.y, li.y), diffDF(hj.z, lj.z, hi.z, li.z)};
}
__device__ __forceinline__ df norm2(const V3& v) { return v.x * v.x + v.y * v.y + v.z * v.z; }
__device__ __forceinline__ df dot3(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

struct PairF {
    V3 v;    // x_j - x_i
    df d2;   // |x_j - x_i|^2
};
__device__ __forceinline__ PairF pairDF(float4 hj, float4 lj, float4 hi, float4 li) {
    PairF q;
    q.v = diff3(hj, lj, hi, li);
    q.d2 = norm2(q.v);
    return q;
}

// Weight and weight / r^2 of MpsParticle::weight (src/MpsParticle.cpp:57-72) from r^2.
struct WeightDF {
    df w, wr2;
};
struct RadiusDF {
    df re, invRe;
};
__device__ __forceinline__ WeightDF weightDF(df d2, const RadiusDF& R, int t) {
    df rinv = rsqrtDF(d2);
    WeightDF o;
    switch (t) {
        case 1: { df r = d2 * rinv; o.w = R.re * rinv + r * R.invRe - 2.0f; } break;
        case 2: { df r = d2 * rinv; o.w = R.re * rinv - r * R.invRe; } break;
        case 3: { df a = -(d2 * rinv * R.invRe) + 1.0f; o.w = a * a * a; } break;
        case 4: { df a = -(d2 * rinv * R.invRe) + 1.0f; o.w = a * a; } break;
        default: o.w = R.re * rinv - 1.0f; break;
    }
    o.wr2 = o.w * (rinv * rinv);
    return o;
}

// ------------------------------------------------------------------ decisions
// a < b for two float-float values each within `mg` of the reference's FP64 value; inside
// the margin the reference's FP64 expression decides (exact()).
template <class F>
__device__ __forceinline__ bool lessDF(df a, df b, float mg, F&& exact) {
    df t = a - b;
    if (t.h < -mg) return true;
    if (t.h > mg) return false;
    return exact();
}
// dst_ij^2 < R2 (R2 the FP64 radius^2 of the reference's test)
__device__ __forceinline__ bool inBallDF(const Dev& d, df d2, df R2f, float mg, double R2, int i, int j) {
    return lessDF(d2, R2f, mg, [&] { return pairOf(d.pos[j], d.pos[i]).d2 < R2; });
}

// Mirror-side context of particle i (the SideCtx test in float-float): the mirror position
// split into hi/lo parts relative to domainMin.
struct SideDF {
    float4 mh, ml;
    bool check;
};
__device__ __forceinline__ SideDF sideDF(const Dev& d, int i, dvec4 pi) {
    SideDF s;
    s.check = false;
    if (d.P.wallType == 0) return s;
    dvec4 m = d.mirror[i];
    double a = pi.x - m.x, b = pi.y - m.y, c = pi.z - m.z;
    double lim = 2.2 * d.P.reL;
    s.check = (a * a + b * b + c * c) <= lim * lim;
    if (s.check) {
        const MpsParams& P = d.P;
        s.mh = make_float4(d2fRN(m.x - P.domainMin[0]), d2fRN(m.y - P.domainMin[1]), d2fRN(m.z - P.domainMin[2]), 0.f);
        s.ml = posLoOf(m, s.mh, P);
    }
    return s;
}
// dst_ij^2 < dst_imj^2 (j not on the mirror side of i), given the float-float d2
__device__ __forceinline__ bool sideOkDF(const Dev& d, const SideDF& s, float4 hj, float4 lj, df d2, int i, int j) {
    if (!s.check) return true;
    df dm2 = norm2(diff3(hj, lj, s.mh, s.ml));
    return lessDF(d2, dm2, d.mgSide, [&] {
        dvec4 pj = d.pos[j];
        return pairOf(pj, d.pos[i]).d2 < pairMirror(pj, d.mirror[i]).dm2;
    });
}

// Particle of thread t for the 27-bucket scans.  Threads walk the stale bucket list in
// bucket order (STRAY = false), so the lanes of a warp share most of their candidate
// buckets and their candidate loads coalesce; a live particle appears there once (an
// out-of-domain removal moves the last particle into the freed index, which the list
// still holds, and leaves the old last index beyond the live count).  STRAY = true
// covers, in index order, the live particles the list does not hold (cellOf == nB).
template <bool STRAY>
__device__ __forceinline__ int scanParticle(const Dev& d) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int n = *d.nLive;
    if (STRAY) return (t < n && d.cellOf[t] >= d.nB) ? t : -1;
    if (t >= d.cellStart[d.nB]) return -1;
    int i = d.cellSorted[t];
    return i < n ? i : -1;
}

// 27-bucket scan (reference order) over the stale bucket list with the FP32 prefilter on
// the hi parts; f(j, s, hj) receives every candidate with FP32 squared distance <= hi
// (s = its slot in bucket order, so posLoCell[s] is its lo part).  fi is the particle's
// current FP32 copy (the window comes from it, exactly, with the FP64 fallback).
template <class F>
__device__ __forceinline__ void forCellsDF(const Dev& d, dvec4 pi, float4 fi, float hi, F&& f) {
    const MpsParams& P = d.P;
    int ix, iy, iz;
    bucketCoordsHi(d, pi, fi, ix, iy, iz);
    int dz = d.dz3;
    int minZ = (iz - 1) * dz, maxZ = (iz + 1) * dz;
#pragma unroll 1
    for (int jz = minZ; jz <= maxZ; jz++)
#pragma unroll 1
        for (int jy = iy - 1; jy <= iy + 1; jy++)
#pragma unroll 1
            for (int jx = ix - 1; jx <= ix + 1; jx++) {
                long long jb = (long long)jz * P.numBucketsXY + (long long)jy * P.numBucketsX + jx;
                if (jb < 0 || jb >= d.nB) continue;
                int s0 = d.cellStart[jb], s1 = d.cellStart[jb + 1];
                for (int s = s0; s < s1; s++) {
                    float4 fj = __ldg(&d.posfCell[s]);
                    float ex = fj.x - fi.x, ey = fj.y - fi.y, ez = fj.z - fi.z;
                    if (ex * ex + ey * ey + ez * ez > hi) continue;
                    f(__ldg(d.cellSorted + s), s, fj);
                }
            }
}

__device__ __forceinline__ df dfOf(float h, float l) { return quick2(h, l); }

// Scan window key of a position: its three bucket coordinates (out-of-grid included).
__device__ __forceinline__ long long cellKeyOf(const Dev& d, dvec4 p, float4 hi) {
    int ix, iy, iz;
    bucketCoordsHi(d, p, hi, ix, iy, iz);
    return ((long long)(iz & 0x1fffff) << 42) | ((long long)(iy & 0x1fffff) << 21) | (long long)(ix & 0x1fffff);
}
