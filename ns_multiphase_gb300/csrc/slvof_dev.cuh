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

namespace slvof {

constexpr double EPS64 = 2.220446049250313e-16; /* Julia eps() */
constexpr int CLIP_STACK = 12;                   /* max cutTet nesting held per thread */
constexpr int CLIP_MAX_LEAVES = 4096;            /* leaf budget of one top-level tet clip */
constexpr int CLIP_STACK32 = 8;                  /* FP32 clip nesting (pruned subtrees are shallow) */

/* Error bits, same values as SLVOF_DEV_* in include/slvof.h. */
enum : int { ERR_INDEX = 1, ERR_DEPTH = 2, ERR_NAN = 4, ERR_VOLUME = 8 };

struct DevMesh {
    int N[3];
    int g;
    int nband;
    int projection;
    int per[3];
    int lo;  /* 1 - g, first cell index in every direction */
    int vlo; /* lo - 3, first VF index */
    int hi[3];
    int fast_pure; /* pure-donor shortcut valid (|coordinates| < Lx+Ly+Lz everywhere) */
    double d[3];
    double VFlo, VFhi;
    double Lsum;    /* (Lx+Ly)+Lz, |D| of pure cells (src/VF.jl:116-120) */
    double cellvol; /* (dx*dy)*dz */
    const double* f[3]; /* face coordinates, f[q][i - lo] */
    const double* c[3]; /* centre coordinates */
    long cs1, cs2;      /* cell-array strides (j, k) */
    long vs1, vs2;      /* VF strides */
};

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

/* Single-rank ghost fill as a source map.  Neumann! (x-,x+,y-,y+,z-,z+) followed by
 * update_borders! (x, y, z; two self-Sendrecv! copies per periodic direction) is a sequence
 * of slab copies, each reading the state before it.  Walking the copies backwards gives, for
 * every cell, the cell whose pre-fill value it ends with.  The copies of one direction only
 * move that direction's index, so the map is separable. */
__host__ __device__ __forceinline__ int ghost_src_1d(int p, int N, int g, bool periodic, bool neumann)
{
    if (periodic) {
        if (p >= 1 - g && p <= 0) p += N;     /* A[mino_:min_-1] <- A[max_-g+1:max_] (second copy) */
        if (p >= N + 1 && p <= N + g) p -= N; /* A[max_+1:maxo_] <- A[min_:min_+g-1] (first copy) */
    }
    if (neumann) {
        if (p == N + 1) p = N; /* A[max_+1] <- A[max_] */
        if (p == 0) p = 1;     /* A[min_-1] <- A[min_] */
    }
    return p;
}

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

/* ---- cut tables, src/VFgeom.jl:55-165, 0-based ---------------------------------------
 * For each cut case (0..15, = reference case - 1): number of new vertices on the plane, the
 * edges they lie on (v1, v2), number of tets, first liquid (negative-side) tet, the tets'
 * vertices (0..3 original, 4..7 new) and the side (0 negative, 1 positive) of each tet. */
struct CutCase {
    int8_t nvert, ntets, nntet, pad;
    int8_t v1[4], v2[4];
    int8_t vtet[6][4];
    int8_t side[6];
    int8_t pad2[2];
};

#define X_ -1
static __constant__ CutCase c_cut[16] = {
    {0, 1, 1, 0, {X_, X_, X_, X_}, {X_, X_, X_, X_},
     {{0, 1, 2, 3}, {X_, X_, X_, X_}, {X_, X_, X_, X_}, {X_, X_, X_, X_}, {X_, X_, X_, X_}, {X_, X_, X_, X_}},
     {0, X_, X_, X_, X_, X_}, {0, 0}},
    {3, 4, 2, 0, {0, 0, 0, X_}, {1, 2, 3, X_},
     {{4, 6, 5, 0}, {5, 1, 2, 3}, {3, 1, 4, 5}, {4, 5, 6, 3}, {X_, X_, X_, X_}, {X_, X_, X_, X_}},
     {1, 0, 0, 0, X_, X_}, {0, 0}},
    {3, 4, 2, 0, {1, 1, 1, X_}, {2, 3, 0, X_},
     {{6, 4, 5, 1}, {0, 2, 3, 5}, {0, 4, 2, 5}, {4, 6, 5, 0}, {X_, X_, X_, X_}, {X_, X_, X_, X_}},
     {1, 0, 0, 0, X_, X_}, {0, 0}},
    {4, 6, 4, 0, {0, 1, 0, 1}, {3, 3, 2, 2},
     {{4, 7, 5, 1}, {4, 6, 7, 0}, {4, 0, 7, 1}, {4, 5, 7, 3}, {4, 7, 6, 2}, {4, 7, 2, 3}},
     {1, 1, 1, 0, 0, 0}, {0, 0}},
    {3, 4, 2, 0, {2, 2, 2, X_}, {3, 0, 1, X_},
     {{5, 4, 6, 2}, {1, 0, 3, 5}, {5, 4, 3, 1}, {5, 6, 4, 1}, {X_, X_, X_, X_}, {X_, X_, X_, X_}},
     {1, 0, 0, 0, X_, X_}, {0, 0}},
    {4, 6, 4, 0, {0, 2, 0, 2}, {3, 3, 1, 1},
     {{4, 5, 7, 2}, {4, 7, 6, 0}, {4, 7, 0, 2}, {4, 7, 5, 3}, {4, 6, 7, 1}, {4, 7, 3, 1}},
     {1, 1, 1, 0, 0, 0}, {0, 0}},
    {4, 6, 4, 0, {1, 2, 1, 2}, {3, 3, 0, 0},
     {{7, 5, 4, 2}, {4, 6, 7, 1}, {7, 4, 1, 2}, {7, 4, 5, 3}, {4, 7, 6, 0}, {4, 7, 0, 3}},
     {1, 1, 1, 0, 0, 0}, {0, 0}},
    {3, 4, 4, 0, {3, 3, 3, X_}, {0, 1, 2, X_},
     {{0, 1, 2, 6}, {0, 1, 6, 5}, {4, 6, 5, 0}, {4, 5, 6, 3}, {X_, X_, X_, X_}, {X_, X_, X_, X_}},
     {1, 1, 1, 0, X_, X_}, {0, 0}},
    {3, 4, 2, 0, {3, 3, 3, X_}, {0, 1, 2, X_},
     {{4, 5, 6, 3}, {0, 1, 2, 5}, {4, 0, 2, 5}, {4, 6, 5, 2}, {X_, X_, X_, X_}, {X_, X_, X_, X_}},
     {1, 0, 0, 0, X_, X_}, {0, 0}},
    {4, 6, 4, 0, {0, 3, 0, 3}, {2, 2, 1, 1},
     {{4, 7, 5, 3}, {4, 6, 7, 0}, {4, 7, 3, 0}, {4, 5, 7, 2}, {4, 7, 6, 1}, {4, 7, 1, 2}},
     {1, 1, 1, 0, 0, 0}, {0, 0}},
    {4, 6, 4, 0, {1, 3, 1, 3}, {2, 2, 0, 0},
     {{7, 4, 5, 3}, {4, 7, 6, 1}, {7, 1, 4, 3}, {7, 5, 4, 2}, {4, 6, 7, 0}, {4, 7, 2, 0}},
     {1, 1, 1, 0, 0, 0}, {0, 0}},
    {3, 4, 4, 0, {2, 2, 2, X_}, {3, 0, 1, X_},
     {{0, 3, 1, 6}, {3, 0, 5, 6}, {5, 6, 4, 3}, {5, 4, 6, 2}, {X_, X_, X_, X_}, {X_, X_, X_, X_}},
     {1, 1, 1, 0, X_, X_}, {0, 0}},
    {4, 6, 4, 0, {2, 3, 2, 3}, {1, 1, 0, 0},
     {{7, 5, 4, 3}, {4, 6, 7, 2}, {7, 3, 4, 2}, {7, 4, 5, 1}, {4, 7, 6, 0}, {4, 7, 0, 1}},
     {1, 1, 1, 0, 0, 0}, {0, 0}},
    {3, 4, 4, 0, {1, 1, 1, X_}, {2, 3, 0, X_},
     {{2, 3, 0, 6}, {6, 5, 2, 3}, {6, 5, 4, 2}, {6, 4, 5, 1}, {X_, X_, X_, X_}, {X_, X_, X_, X_}},
     {1, 1, 1, 0, X_, X_}, {0, 0}},
    {3, 4, 4, 0, {0, 0, 0, X_}, {1, 2, 3, X_},
     {{6, 3, 1, 2}, {1, 2, 5, 6}, {4, 5, 6, 1}, {4, 6, 5, 0}, {X_, X_, X_, X_}, {X_, X_, X_, X_}},
     {1, 1, 1, 0, X_, X_}, {0, 0}},
    {0, 1, 2, 0, {X_, X_, X_, X_}, {X_, X_, X_, X_},
     {{0, 1, 2, 3}, {X_, X_, X_, X_}, {X_, X_, X_, X_}, {X_, X_, X_, X_}, {X_, X_, X_, X_}, {X_, X_, X_, X_}},
     {1, X_, X_, X_, X_, X_}, {0, 0}},
};
#undef X_

/* 5-tet split of the 8 cell vertices (src/VFgeom.jl:235-256), 0-based. */
__host__ __device__ constexpr int tet5(int t, int n)
{
    return (t == 0) ? (n == 0 ? 0 : n == 1 ? 1 : n == 2 ? 3 : 5)
         : (t == 1) ? (n == 0 ? 0 : n == 1 ? 3 : n == 2 ? 2 : 6)
         : (t == 2) ? (n == 0 ? 0 : n == 1 ? 4 : n == 2 ? 5 : 6)
         : (t == 3) ? (n == 0 ? 3 : n == 1 ? 6 : n == 2 ? 5 : 7)
                    : (n == 0 ? 0 : n == 1 ? 3 : n == 2 ? 6 : 5);
}

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
