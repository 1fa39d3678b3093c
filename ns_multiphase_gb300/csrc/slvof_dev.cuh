/*
 * slvof_dev.cuh — device-side building blocks shared by the SL-VOF kernels.
 *
 * Index convention: the reference's Julia cell indices, interior 1..N, ghosts 1-g..0 and
 * N+1..N+g; VF carries three more layers (src/Tools.jl:144).  Arrays are OffsetArray
 * parents, i fastest.
 */
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "detmath.h"
#include "mesh_view.h"

namespace slvof {

constexpr double EPS64 = 2.220446049250313e-16; /* Julia eps() */
constexpr int CLIP_STACK = 12;                   /* max cutTet nesting held per thread */
constexpr int CLIP_MAX_LEAVES = 4096;            /* leaf budget of one top-level tet clip */
constexpr int CLIP_STACK32 = 8;                  /* FP32 clip nesting (pruned subtrees are shallow) */

/* Error bits, same values as SLVOF_DEV_* in include/slvof.h. */
enum : int { ERR_INDEX = 1, ERR_DEPTH = 2, ERR_NAN = 4, ERR_VOLUME = 8, ERR_WAIT = 16 };

__device__ __forceinline__ long cidx(const DevMesh& m, int i, int j, int k)
{
    return (long)(i - m.lo) + (long)(j - m.lo) * m.cs1 + (long)(k - m.lo) * m.cs2;
}
__device__ __forceinline__ long vidx(const DevMesh& m, int i, int j, int k)
{
    return (long)(i - m.vlo) + (long)(j - m.vlo) * m.vs1 + (long)(k - m.vlo) * m.vs2;
}
__device__ __forceinline__ double fco(const DevMesh& m, int q, int i) { return __ldg(m.f[q] + (i - m.lo)); }
__device__ __forceinline__ double cco(const DevMesh& m, int q, int i) { return __ldg(m.c[q] + (i - m.lo)); }

/* Julia max/min on Float64 (NaN-propagating, max(-0.0, 0.0) == 0.0). */
template <class R>
__device__ __forceinline__ R jmax(R a, R b)
{
    if (a != a || b != b) return a + b;
    return a > b ? a : (b > a ? b : (signbit(a) ? b : a));
}
template <class R>
__device__ __forceinline__ R jmin(R a, R b)
{
    if (a != a || b != b) return a + b;
    return a < b ? a : (b < a ? b : (signbit(a) ? a : b));
}

/* safe divide, src/Tools.jl:375-377 */
__device__ __forceinline__ double sdiv(double a, double b) { return fabs(b) <= EPS64 ? (double)INFINITY : a / b; }
/* mu = min(1, max(0, -d1 /^ (d2-d1))), src/VFgeom.jl:787 */
__device__ __forceinline__ double clamp_mu(double q) { return jmin(1.0, jmax(0.0, q)); }

/* cut tables (src/VFgeom.jl:55-165) in constant memory */
#define X_ -1
static __constant__ CutCase c_cut[16] = SLVOF_CUT_TABLE;
#undef X_


/* tet_vol, src/VFgeom.jl:669-681: -1/6 * det(v1-v4, v2-v4, v3-v4) in the reference's
 * expansion order. */
template <class R>
__device__ __forceinline__ R tet_vol(R x0, R y0, R z0, R x1, R y1, R z1, R x2, R y2, R z2, R x3, R y3, R z3)
{
    const R a1 = x0 - x3, a2 = y0 - y3, a3 = z0 - z3;
    const R b1 = x1 - x3, b2 = y1 - y3, b3 = z1 - z3;
    const R c1 = x2 - x3, c2 = y2 - y3, c3 = z2 - z3;
    return R(-1.0 / 6.0) * ((a1 * (b2 * c3 - c2 * b3) - a2 * (b1 * c3 - c1 * b3)) + a3 * (b1 * c2 - c1 * b2));
}

/* d2case, src/VFgeom.jl:693-708, on d[0..3] in place; returns the 0-based case.  eps is
 * the reference's absolute eps() for FP64 and a caller-chosen length for FP32 geometry. */
template <class R>
__device__ __forceinline__ int d2case(R& d0, R& d1, R& d2, R& d3, R eps, int& err)
{
    const int npos = (d0 > R(0)) + (d1 > R(0)) + (d2 > R(0)) + (d3 > R(0));
    const int nneg = (d0 < R(0)) + (d1 < R(0)) + (d2 < R(0)) + (d3 < R(0));
    const R fix = npos > nneg ? eps : -eps;
    if (fabs(d0) < eps) d0 = fix;
    if (fabs(d1) < eps) d1 = fix;
    if (fabs(d2) < eps) d2 = fix;
    if (fabs(d3) < eps) d3 = fix;
    if (d0 != d0 || d1 != d1 || d2 != d2 || d3 != d3) err |= ERR_NAN;
    return (d0 > R(0) ? 1 : 0) + (d1 > R(0) ? 2 : 0) + (d2 > R(0) ? 4 : 0) + (d3 > R(0) ? 8 : 0);
}

/* 3-element ascending sort (values only; ties are interchangeable). */
__device__ __forceinline__ void sort3(double& a, double& b, double& c)
{
    double t;
    if (a > b) { t = a; a = b; b = t; }
    if (b > c) { t = b; b = c; c = t; }
    if (a > b) { t = a; a = b; b = t; }
}

/* computeAlpha, src/VF.jl:164-214 (Scardovelli & Zaleski inverse), FP64 with the
 * deterministic cbrt/acos/sin/cos. */
__device__ __forceinline__ double compute_alpha64(double m1, double m2, double m3, double VF)
{
    sort3(m1, m2, m3);
    const double m12 = m1 + m2;
    const double V1 = m1 * m1 / jmax(6.0 * m2 * m3, EPS64);
    const double V2 = V1 + sdiv(0.5 * (m2 - m1), m3);
    double V3;
    if (m12 <= m3) V3 = sdiv(0.5 * m12, m3);
    else V3 = sdiv((m3 * m3 * (3.0 * m12 - m3) + m1 * m1 * (m1 - 3.0 * m3)) + m2 * m2 * (m2 - 3.0 * m3), 6.0 * m1 * m2 * m3);
    double alpha;
    if (0.0 <= VF && VF < V1) {
        alpha = detm_cbrt(6.0 * m1 * m2 * m3 * VF);
    } else if (V1 <= VF && VF < V2) {
        alpha = 0.5 * (m1 + sqrt(m1 * m1 + 8.0 * m2 * m3 * (VF - V1)));
    } else if (V2 <= VF && VF < V3) {
        double a0 = (m1 * m1 * m1 + m2 * m2 * m2) - 6.0 * m1 * m2 * m3 * VF;
        double a1 = -3.0 * (m1 * m1 + m2 * m2);
        double a2 = 3.0 * m12;
        const double a3 = -1.0;
        a0 = a0 / a3; a1 = a1 / a3; a2 = a2 / a3;
        const double p0 = a1 / 3.0 - a2 * a2 / 9.0;
        const double q0 = (a1 * a2 - 3.0 * a0) / 6.0 - a2 * a2 * a2 / 27.0;
        const double theta = detm_acos(jmin(1.0, jmax(-1.0, q0 / sqrt(-1.0 * (p0 * p0 * p0))))) / 3.0;
        alpha = sqrt(-p0) * (sqrt(3.0) * detm_sin(theta) - detm_cos(theta)) - a2 / 3.0;
    } else if (m12 <= m3) {
        alpha = m3 * VF + 0.5 * m12;
    } else {
        double a0 = ((m1 * m1 * m1 + m2 * m2 * m2) + m3 * m3 * m3) - 6.0 * m1 * m2 * m3 * VF;
        double a1 = -3.0 * ((m1 * m1 + m2 * m2) + m3 * m3);
        double a2 = 3.0;
        const double a3 = -2.0;
        a0 = a0 / a3; a1 = a1 / a3; a2 = a2 / a3;
        const double p0 = a1 / 3.0 - a2 * a2 / 9.0;
        const double q0 = (a1 * a2 - 3.0 * a0) / 6.0 - a2 * a2 * a2 / 27.0;
        const double theta = detm_acos(jmin(1.0, jmax(-1.0, q0 / sqrt(-(p0 * p0 * p0))))) / 3.0;
        alpha = sqrt(-p0) * (sqrt(3.0) * detm_sin(theta) - detm_cos(theta)) - a2 / 3.0;
    }
    return alpha;
}

/* computeDist, src/VF.jl:109-156 (cell centre from the mesh arrays). */
__device__ __forceinline__ double compute_dist64(const DevMesh& m, int i, int j, int k, double nx, double ny, double nz,
                                                 double VF)
{
    if (VF < m.VFlo) return -m.Lsum;
    if (VF > m.VFhi) return +m.Lsum;
    double m0 = nx * m.d[0], m1 = ny * m.d[1], m2 = nz * m.d[2];
    const double norm = ((fabs(m0) + fabs(m1)) + fabs(m2)) + EPS64;
    m0 = m0 / norm; m1 = m1 / norm; m2 = m2 / norm;
    double factor = 0.0;
    if (m0 < 0.0) factor += m0;
    if (m1 < 0.0) factor += m1;
    if (m2 < 0.0) factor += m2;
    const double VFo = VF > 0.5 ? 1.0 - VF : VF;
    double alpha = compute_alpha64(fabs(m0), fabs(m1), fabs(m2), VFo);
    alpha = VF > 0.5 ? 1.0 - alpha : alpha;
    alpha += factor;
    alpha -= 0.5 * ((m0 + m1) + m2);
    double dist = alpha * norm;
    dist += (nx * cco(m, 0, i) + ny * cco(m, 1, j)) + nz * cco(m, 2, k);
    return dist;
}

/* Block-aggregated append of K items per thread: one atomic on the list counter per block
 * instead of one per warp and item (band cells are a few percent of the grid, so with warp
 * atomics thousands of warps queue on the one counter).  Every thread of the block calls it
 * (it holds two __syncthreads); s holds NW * K + 1 ints of shared memory, NW the block's
 * warps.  Items land in (warp, k) order within the block's run. */
template <int K, int NW>
__device__ __forceinline__ void block_append(const bool (&flag)[K], const int (&item)[K], int* list, int* count, int* s)
{
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = tid & 31, w = tid >> 5;
    unsigned bal[K];
#pragma unroll
    for (int q = 0; q < K; ++q) {
        bal[q] = __ballot_sync(0xffffffffu, flag[q]);
        if (lane == 0) s[w * K + q] = __popc(bal[q]);
    }
    __syncthreads();
    if (tid == 0) {
        int run = 0;
        for (int e = 0; e < NW * K; ++e) {
            const int c = s[e];
            s[e] = run;
            run += c;
        }
        s[NW * K] = run > 0 ? atomicAdd(count, run) : 0;
    }
    __syncthreads();
    const int base = s[NW * K];
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int q = 0; q < K; ++q)
        if (flag[q]) list[base + s[w * K + q] + __popc(bal[q] & lt)] = item[q];
}

/* Warp-aggregated append of flagged items to a list. */
__device__ __forceinline__ void warp_append(bool flag, int item, int* list, int* count)
{
    const unsigned act = __activemask();
    const unsigned ballot = __ballot_sync(act, flag);
    if (!ballot) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(ballot) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(ballot));
    base = __shfl_sync(act, base, leader);
    if (flag) list[base + __popc(ballot & ((1u << lane) - 1))] = item;
}

/* ---- VF thresholds and sums on the integer pipe ------------------------------------------
 * GB300 issues double compares and adds on its narrow FP64 pipe.  For a positive threshold t
 * and any double x, x < t exactly when the bit pattern of x, read as a signed 64-bit integer,
 * is below that of t (negative x have the sign bit set); NaN is neither below nor above, as
 * in the floating-point compare. */
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ bool bits_nan(long long b) { return (b & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL; }
__device__ __forceinline__ bool bits_below(long long b, long long t) { return b < t && !bits_nan(b); }
__device__ __forceinline__ bool bits_above(long long b, long long t) { return b > t && !bits_nan(b); }

/* round(x * 2^62) for |x| < 2, from the bit pattern (zero for subnormals, saturated for
 * |x| >= 2 and non-finite values).  Volume fractions summed in this fixed point with 128-bit
 * integers give an exact, order-independent sum. */
__device__ __forceinline__ long long fx62(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF);
    if (e == 0) return 0;
    const unsigned long long mant = (b & ((1ull << 52) - 1)) | (1ull << 52);
    const int sh = e - 1023 + 10; /* x * 2^62 = mant * 2^(e - 1023 - 52 + 62) */
    long long r;
    if (sh >= 11) r = 0x7FFFFFFFFFFFFFFFLL;
    else if (sh >= 0) r = (long long)(mant << sh);
    else if (sh > -60) r = (long long)((mant + (1ull << (-sh - 1))) >> (-sh));
    else r = 0;
    return (b >> 63) ? -r : r;
}

/* 128-bit integer in two 64-bit words, for warp shuffles and storage */
__device__ __forceinline__ __int128 i128_from(long long hi, unsigned long long lo)
{
    return (__int128)(((unsigned __int128)(unsigned long long)hi << 64) | lo);
}
__device__ __forceinline__ __int128 i128_shfl_down(__int128 x, int off)
{
    const long long hi = (long long)(x >> 64);
    const unsigned long long lo = (unsigned long long)x;
    return i128_from(__shfl_down_sync(0xffffffffu, hi, off), __shfl_down_sync(0xffffffffu, lo, off));
}
__device__ __forceinline__ double i128_to_double(__int128 x)
{
    const bool neg = x < 0;
    const unsigned __int128 u = neg ? (unsigned __int128)(-x) : (unsigned __int128)x;
    const double r = (double)(unsigned long long)(u >> 64) * 18446744073709551616.0 + (double)(unsigned long long)u;
    return neg ? -r : r;
}

/* Neumaier-compensated pair (sum, correction). */
struct Comp {
    double s, c;
};
__device__ __forceinline__ void comp_add(Comp& a, double x)
{
    const double t = a.s + x;
    a.c += fabs(a.s) >= fabs(x) ? (a.s - t) + x : (x - t) + a.s;
    a.s = t;
}
__device__ __forceinline__ void comp_merge(Comp& a, const Comp& b)
{
    comp_add(a, b.s);
    a.c += b.c;
}

} // namespace slvof
