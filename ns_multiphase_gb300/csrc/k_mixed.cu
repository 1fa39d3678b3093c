/*
 * k_mixed.cu — mixed-precision kernels of the SL-VOF path (FMA on).
 *
 * Geometry runs in FP32 in cell-normalised local coordinates: a point is u = (x - o)/d with o
 * the corner of the cell being updated, so mesh faces are small integers (exact in FP32)
 * and the cell volume is 1.  This needs a uniform mesh, which create_mesh builds
 * (src/Mesh.jl:83-100); slvof_create rejects the mixed mode otherwise.
 *
 *   k_elvira_iface32 : ELVIRA candidates (src/ELVIRA.jl:62-137) with FP32 candidate errors.
 *                      The liquid fraction of each 3x3x3 neighbour under a candidate plane is
 *                      the exact plane/cube volume in closed form (the quantity
 *                      computePLIC2VF evaluates with five tet clips), and the plane constant
 *                      is the inverse of the same function (computeAlpha's role).  The chosen
 *                      candidate is re-formed and normalised in FP64.
 *   k_sl32           : SL update (src/Transport.jl:111-148): FP32 RK trajectories through
 *                      FP32 face velocities, FP32 recursive clip (same cut tables and
 *                      recursion as cutTet), FP64 accumulation of the clipped volumes.
 */
#include "slvof_kernels.h"
#include "slvof_dev.cuh"

namespace slvof {

/* ======================================================================================
 * Plane/unit-cube volume.  For m1 <= m2 <= m3, m1+m2+m3 = 1 and 0 <= a <= 1/2, the volume
 * of {s in [0,1]^3 : m.s < a} is the inclusion-exclusion sum
 *   [a^3 - (a-m1)_+^3 - (a-m2)_+^3 - (a-m3)_+^3 + ...] / (6 m1 m2 m3),
 * rewritten per interval so that no term divides a cancellation by a small m_i:
 *   a < m1            : a^3 / (6 m1 m2 m3)
 *   m1 <= a < m2      : (3a^2 - 3a m1 + m1^2) / (6 m2 m3)
 *   m2 <= a < m12,m3  : same - (b/m1) b^2 / (6 m2 m3),  b = a - m2 < m1
 *   m3 <= a (m3<m12)  : same - [(b/m1) b^2 + (c/m1) c^2] / (6 m2 m3),  c = a - m3
 *   m12 <= a < m3     : (2a - m12) / (2 m3)
 * and V(a) = 1 - V(1-a) above 1/2.
 * ==================================================================================== */
struct Cube {
    float m1, m2, m3, m12, i6m23, i2m3, im1;
};

__device__ __forceinline__ Cube make_cube(float a, float b, float c)
{
    float t;
    if (a > b) { t = a; a = b; b = t; }
    if (b > c) { t = b; b = c; c = t; }
    if (a > b) { t = a; a = b; b = t; }
    Cube q;
    q.m1 = a; q.m2 = b; q.m3 = c; q.m12 = a + b;
    q.i6m23 = (b > 0.f) ? 1.f / (6.f * b * c) : 0.f;
    q.i2m3 = 0.5f / c;
    q.im1 = (a > 0.f) ? 1.f / a : 0.f;
    return q;
}

__device__ __forceinline__ float cube_lower(const Cube& q, float a)
{
    if (a < q.m1) return a * a * a * q.im1 * q.i6m23;
    const float base = (3.f * a * a - 3.f * a * q.m1 + q.m1 * q.m1) * q.i6m23;
    if (a < q.m2) return base;
    if (a < q.m12 && a < q.m3) {
        const float b = a - q.m2;
        return base - (b * q.im1) * b * b * q.i6m23;
    }
    if (q.m3 < q.m12) {
        const float b = a - q.m2, c = a - q.m3;
        return base - ((b * q.im1) * b * b + (c * q.im1) * c * c) * q.i6m23;
    }
    return (2.f * a - q.m12) * q.i2m3;
}

__device__ __forceinline__ float cube_frac(const Cube& q, float a)
{
    if (a <= 0.f) return 0.f;
    if (a >= 1.f) return 1.f;
    return a <= 0.5f ? cube_lower(q, a) : 1.f - cube_lower(q, 1.f - a);
}

/* d/da of cube_lower (cut area), for the Newton inverse. */
__device__ __forceinline__ float cube_area(const Cube& q, float a)
{
    if (a < q.m1) return 3.f * a * a * q.im1 * q.i6m23;
    const float base = (6.f * a - 3.f * q.m1) * q.i6m23;
    if (a < q.m2) return base;
    if (a < q.m12 && a < q.m3) {
        const float b = a - q.m2;
        return base - 3.f * (b * q.im1) * b * q.i6m23;
    }
    if (q.m3 < q.m12) {
        const float b = a - q.m2, c = a - q.m3;
        return base - 3.f * ((b * q.im1) * b + (c * q.im1) * c) * q.i6m23;
    }
    return 2.f * q.i2m3;
}

/* alpha with cube_frac(alpha) = V for V in [0, 1/2] (computeAlpha, src/VF.jl:164-214):
 * closed-form start on the first two intervals, then bracketed Newton. */
__device__ __forceinline__ float cube_alpha(const Cube& q, float V)
{
    if (V <= 0.f) return 0.f;
    if (q.m2 <= 0.f) return V; /* plane parallel to a face */
    const float V1 = q.m1 * q.m1 * q.i6m23;
    float a;
    if (V < V1) a = cbrtf(V * 6.f * q.m1 * q.m2 * q.m3);
    else a = 0.5f * (q.m1 + sqrtf(fmaxf(q.m1 * q.m1 + 8.f * q.m2 * q.m3 * (V - V1), 0.f)));
    float lo = 0.f, hi = 0.5f;
    a = fminf(fmaxf(a, lo), hi);
#pragma unroll 1
    for (int it = 0; it < 6; ++it) {
        const float f = cube_lower(q, a) - V;
        if (f > 0.f) hi = a;
        else lo = a;
        const float s = cube_area(q, a);
        float an = s > 0.f ? a - f / s : 0.5f * (lo + hi);
        if (!(an > lo && an < hi)) an = 0.5f * (lo + hi);
        a = an;
    }
    return a;
}

/* ======================================================================================
 * ELVIRA candidates in FP32.
 * ==================================================================================== */
constexpr int EL32_WARPS = 8;

/* Candidate normal of lane (family f, outer a, inner b) from a 3x3x3 VF block; R = float
 * for the error pass, double to re-form the chosen candidate exactly as the FP64 path. */
template <class R>
__device__ __forceinline__ void candidate(const R* sv, int f, int a, int b, R dx, R dy, R dz, const R* hx, const R* hy,
                                          const R* hz, R& cx, R& cy, R& cz)
{
    /* h[0] = xm[i]-xm[i-1], h[1] = xm[i+1]-xm[i-1], h[2] = xm[i+1]-xm[i]: the reference's
     * pairs {i-1,i}, {i-1,i+1}, {i,i+1} (src/ELVIRA.jl:72,82,92) */
#define V3(p, q, r) sv[((r) + 1) * 9 + ((q) + 1) * 3 + ((p) + 1)]
    const int o1 = a == 2 ? 0 : -1, o2 = a == 0 ? 0 : 1;
    const int i1 = b == 2 ? 0 : -1, i2 = b == 0 ? 0 : 1;
    if (f == 0) {
        const R s2x = (V3(i2, 0, -1) * dz + V3(i2, 0, 0) * dz) + V3(i2, 0, 1) * dz;
        const R s1x = (V3(i1, 0, -1) * dz + V3(i1, 0, 0) * dz) + V3(i1, 0, 1) * dz;
        cx = -(s2x - s1x) / hx[b];
        const R s2y = (V3(0, o2, -1) * dz + V3(0, o2, 0) * dz) + V3(0, o2, 1) * dz;
        const R s1y = (V3(0, o1, -1) * dz + V3(0, o1, 0) * dz) + V3(0, o1, 1) * dz;
        cy = -(s2y - s1y) / hy[a];
        cz = V3(0, 0, 1) > V3(0, 0, -1) ? R(-1) : R(1);
    } else if (f == 1) {
        const R s2x = (V3(i2, -1, 0) * dy + V3(i2, 0, 0) * dy) + V3(i2, 1, 0) * dy;
        const R s1x = (V3(i1, -1, 0) * dy + V3(i1, 0, 0) * dy) + V3(i1, 1, 0) * dy;
        cx = -(s2x - s1x) / hx[b];
        cy = V3(0, 1, 0) > V3(0, -1, 0) ? R(-1) : R(1);
        const R s2z = (V3(0, -1, o2) * dy + V3(0, 0, o2) * dy) + V3(0, 1, o2) * dy;
        const R s1z = (V3(0, -1, o1) * dy + V3(0, 0, o1) * dy) + V3(0, 1, o1) * dy;
        cz = -(s2z - s1z) / hz[a];
    } else {
        cx = V3(1, 0, 0) > V3(-1, 0, 0) ? R(-1) : R(1);
        const R s2y = (V3(-1, i2, 0) * dx + V3(0, i2, 0) * dx) + V3(1, i2, 0) * dx;
        const R s1y = (V3(-1, i1, 0) * dx + V3(0, i1, 0) * dx) + V3(1, i1, 0) * dx;
        cy = -(s2y - s1y) / hy[b];
        const R s2z = (V3(-1, 0, o2) * dx + V3(0, 0, o2) * dx) + V3(1, 0, o2) * dx;
        const R s1z = (V3(-1, 0, o1) * dx + V3(0, 0, o1) * dx) + V3(1, 0, o1) * dx;
        cz = -(s2z - s1z) / hz[a];
    }
#undef V3
}

__global__ void __launch_bounds__(EL32_WARPS * 32) k_elvira_iface32(DevMesh m, const double* __restrict__ VF,
                                                                    double* __restrict__ nx, double* __restrict__ ny,
                                                                    double* __restrict__ nz,
                                                                    const int* __restrict__ list,
                                                                    const int* __restrict__ count, int* work)
{
    __shared__ double s_vd[EL32_WARPS][27];
    __shared__ float s_vf[EL32_WARPS][27];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_items = *count;
    const int fam_on[3] = {m.N[2] > 1, m.N[1] > 1, m.N[0] > 1};
    const int ncand = 9 * (fam_on[0] + fam_on[1] + fam_on[2]);
    const float dx = (float)m.d[0], dy = (float)m.d[1], dz = (float)m.d[2];
    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(work, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= n_items) break;
        const int L = list[item];
        const int i = 1 + L % m.N[0];
        const int j = 1 + (L / m.N[0]) % m.N[1];
        const int k = 1 + L / (m.N[0] * m.N[1]);
        if (lane < 27) {
            const double v = VF[vidx(m, i - 1 + lane % 3, j - 1 + (lane / 3) % 3, k - 1 + lane / 9)];
            s_vd[w][lane] = v;
            s_vf[w][lane] = (float)v;
        }
        __syncwarp();
        const float* sv = s_vf[w];
        float err_ = INFINITY;
        int f = 0, a = 0, b = 0;
        if (lane < ncand) {
            const int fam = lane / 9;
            a = (lane % 9) / 3;
            b = lane % 3;
            for (int q = 0, seen = 0; q < 3; ++q)
                if (fam_on[q]) { if (seen == fam) { f = q; break; } ++seen; }
            float cx, cy, cz;
            const float hx[3] = {dx, 2.f * dx, dx}, hy[3] = {dy, 2.f * dy, dy}, hz[3] = {dz, 2.f * dz, dz};
            candidate<float>(sv, f, a, b, dx, dy, dz, hx, hy, hz, cx, cy, cz);
            const float nrm = sqrtf(cx * cx + cy * cy + cz * cz);
            cx /= nrm; cy /= nrm; cz /= nrm;
            /* computeDist in cell units: mm = n*d/|n*d|_1, plane mm.u = alpha' + sum(mm<0) */
            float m0 = cx * dx, m1 = cy * dy, m2 = cz * dz;
            const float n1 = fabsf(m0) + fabsf(m1) + fabsf(m2);
            m0 /= n1; m1 /= n1; m2 /= n1;
            const Cube q = make_cube(fabsf(m0), fabsf(m1), fabsf(m2));
            const float vc = sv[13];
            const float vo = vc > 0.5f ? 1.f - vc : vc;
            float al = cube_alpha(q, vo);
            al = vc > 0.5f ? 1.f - al : al;
            /* neighbour (p,r,s) takes the cube fraction at al - mm.(p,r,s) (sign-folded) */
            float e2 = 0.f;
#pragma unroll
            for (int c = 0; c < 27; ++c) {
                const float p = (float)(c % 3 - 1), r = (float)((c / 3) % 3 - 1), s = (float)(c / 9 - 1);
                const float ae = al - (m0 * p + m1 * r + m2 * s);
                const float d = sv[c] - cube_frac(q, ae);
                e2 += d * d;
            }
            err_ = e2;
        }
        float be = err_ < INFINITY ? err_ : INFINITY;
        int bl = err_ < INFINITY ? lane : 32;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, be, off);
            const int ol = __shfl_xor_sync(0xffffffffu, bl, off);
            if (ob < be || (ob == be && ol < bl)) { be = ob; bl = ol; }
        }
        if (bl < 32 && lane == bl) {
            /* re-form the chosen candidate in FP64 as check_normal! does */
            double cx, cy, cz;
            const double hx[3] = {cco(m, 0, i) - cco(m, 0, i - 1), cco(m, 0, i + 1) - cco(m, 0, i - 1),
                                  cco(m, 0, i + 1) - cco(m, 0, i)};
            const double hy[3] = {cco(m, 1, j) - cco(m, 1, j - 1), cco(m, 1, j + 1) - cco(m, 1, j - 1),
                                  cco(m, 1, j + 1) - cco(m, 1, j)};
            const double hz[3] = {cco(m, 2, k) - cco(m, 2, k - 1), cco(m, 2, k + 1) - cco(m, 2, k - 1),
                                  cco(m, 2, k + 1) - cco(m, 2, k)};
            candidate<double>(s_vd[w], f, a, b, m.d[0], m.d[1], m.d[2], hx, hy, hz, cx, cy, cz);
            const double norm = sqrt((cx * cx + cy * cy) + cz * cz);
            const long o = cidx(m, i, j, k);
            nx[o] = cx / norm; ny[o] = cy / norm; nz[o] = cz / norm;
        }
        __syncwarp();
    }
}

/* ======================================================================================
 * SL update in FP32 local coordinates.
 * ==================================================================================== */
struct Vel32 {
    const float *uf, *vf, *wf; /* face velocities in cells per unit time (u/dx, v/dy, w/dz) */
};

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ __forceinline__ float tri32(const DevMesh& m, const float* __restrict__ f, int I, int J, int K, float wx,
                                       float wy, float wz)
{
    const long b = cidx(m, I, J, K);
    const long sj = m.cs1, sk = m.cs2;
    const float f000 = __ldg(f + b), f100 = __ldg(f + b + 1), f010 = __ldg(f + b + sj), f110 = __ldg(f + b + 1 + sj);
    const float f001 = __ldg(f + b + sk), f101 = __ldg(f + b + 1 + sk), f011 = __ldg(f + b + sj + sk),
                f111 = __ldg(f + b + 1 + sj + sk);
    const float x00 = f000 + wx * (f100 - f000), x10 = f010 + wx * (f110 - f010);
    const float x01 = f001 + wx * (f101 - f001), x11 = f011 + wx * (f111 - f011);
    const float y0 = x00 + wy * (x10 - x00), y1 = x01 + wy * (x11 - x01);
    return y0 + wz * (y1 - y0);
}

/* get_velocity_{u,v,w}face (src/Tools.jl:516-641) on the uniform mesh: the interval search
 * becomes floor() clamped to [imino_, imaxo_-1]. */
__device__ __forceinline__ void vel32(const DevMesh& m, const Vel32& V, int i0, int j0, int k0, float x, float y,
                                      float z, float& u, float& v, float& w)
{
    /* keep the float->int conversions in range for any input (a NaN lands on the clamp) */
    const float B = 1.0e6f;
    const float fx = fminf(fmaxf(floorf(x), -B), B), fy = fminf(fmaxf(floorf(y), -B), B), fz = fminf(fmaxf(floorf(z), -B), B);
    const float gx = fminf(fmaxf(floorf(x - 0.5f), -B), B), gy = fminf(fmaxf(floorf(y - 0.5f), -B), B),
                gz = fminf(fmaxf(floorf(z - 0.5f), -B), B);
    const int Fx = clampi(i0 + (int)fx, m.lo, m.hi[0] - 1), Cx = clampi(i0 + (int)gx, m.lo, m.hi[0] - 1);
    const int Fy = clampi(j0 + (int)fy, m.lo, m.hi[1] - 1), Cy = clampi(j0 + (int)gy, m.lo, m.hi[1] - 1);
    const int Fz = clampi(k0 + (int)fz, m.lo, m.hi[2] - 1), Cz = clampi(k0 + (int)gz, m.lo, m.hi[2] - 1);
    const float wfx = x - (float)(Fx - i0), wcx = x - ((float)(Cx - i0) + 0.5f);
    const float wfy = y - (float)(Fy - j0), wcy = y - ((float)(Cy - j0) + 0.5f);
    const float wfz = z - (float)(Fz - k0), wcz = z - ((float)(Cz - k0) + 0.5f);
    u = tri32(m, V.uf, Fx, Cy, Cz, wfx, wcy, wcz);
    v = tri32(m, V.vf, Cx, Fy, Cz, wcx, wfy, wcz);
    w = tri32(m, V.wf, Cx, Cy, Fz, wcx, wcy, wfz);
}

__device__ __forceinline__ void project32(const DevMesh& m, const Vel32& V, int i0, int j0, int k0, float dt,
                                          float& x, float& y, float& z)
{
    float u1, v1, w1;
    vel32(m, V, i0, j0, k0, x, y, z, u1, v1, w1);
    if (m.projection == 2) {
        const float h = 0.5f * dt;
        float u2, v2, w2, u3, v3, w3, u4, v4, w4;
        vel32(m, V, i0, j0, k0, x - h * u1, y - h * v1, z - h * w1, u2, v2, w2);
        vel32(m, V, i0, j0, k0, x - h * u2, y - h * v2, z - h * w2, u3, v3, w3);
        vel32(m, V, i0, j0, k0, x - dt * u3, y - dt * v3, z - dt * w3, u4, v4, w4);
        const float s = -dt / 6.f;
        x += s * (u1 + 2.f * u2 + 2.f * u3 + u4);
        y += s * (v1 + 2.f * v2 + 2.f * v3 + v4);
        z += s * (w1 + 2.f * w2 + 2.f * w3 + w4);
    } else if (m.projection == 0) {
        x -= dt * u1; y -= dt * v1; z -= dt * w1;
    } else {
        const float h = 0.5f * dt;
        float u2, v2, w2;
        vel32(m, V, i0, j0, k0, x - h * u1, y - h * v1, z - h * w1, u2, v2, w2);
        x -= dt * u2; y -= dt * v2; z -= dt * w2;
    }
}

/* pt2index! (src/Tools.jl:424-434) in local units, seed s: faces sit at integers. */
constexpr int REL = 6; /* relative index range kept in the clip (|index - cell| <= REL) */

__device__ __forceinline__ int idx32(float u, int s, int lo, int hi, int& err)
{
    int I;
    if (u > (float)(s + 1)) I = (int)fminf(ceilf(u), 1.0e6f) - 1;
    else if (u < (float)s) I = (int)fmaxf(floorf(u), -1.0e6f);
    else I = s;
    if (I < lo) { I = lo; err |= ERR_INDEX; }
    if (I > hi) { I = hi; err |= ERR_INDEX; }
    return I;
}

struct Frame32 {
    float x[8], y[8], z[8];
    double acc_v, acc_l;
    signed char ind[8][3];
    signed char cs, next, dir, flags, cut;
};

struct Plane32 {
    const float4* P; /* (mx, my, mz, Dl): n*d and D - n.o in the donor's own cell frame */
};

__device__ __forceinline__ float tet_vol32(const float* vx, const float* vy, const float* vz, int p, int q, int r, int s)
{
    return tet_vol<float>(vx[p], vy[p], vz[p], vx[q], vy[q], vz[q], vx[r], vy[r], vz[r], vx[s], vy[s], vz[s]);
}

__device__ __forceinline__ void leaf32(const DevMesh& m, const CutCase* tab, const Plane32& PL, int i0, int j0, int k0,
                                       const float* cx, const float* cy, const float* cz, int di, int dj, int dk,
                                       double& rv, double& rl, int& err)
{
    const float4 pl = __ldg(PL.P + cidx(m, i0 + di, j0 + dj, k0 + dk));
    const float Dt = pl.w + pl.x * (float)di + pl.y * (float)dj + pl.z * (float)dk;
    float d[4], vx[8], vy[8], vz[8];
#pragma unroll
    for (int n = 0; n < 4; ++n) {
        d[n] = pl.x * cx[n] + pl.y * cy[n] + pl.z * cz[n] - Dt;
        vx[n] = cx[n]; vy[n] = cy[n]; vz[n] = cz[n];
    }
    float c0 = d[0], c1 = d[1], c2 = d[2], c3 = d[3];
    const int cs = d2case(c0, c1, c2, c3, 1e-30f, err);
    const CutCase& C = tab[cs];
    for (int n = 0; n < C.nvert; ++n) {
        const int v1 = C.v1[n], v2 = C.v2[n];
        const float den = d[v2] - d[v1];
        const float mu = fminf(1.f, fmaxf(0.f, den != 0.f ? -d[v1] / den : 1.f));
        vx[4 + n] = vx[v1] + mu * (vx[v2] - vx[v1]);
        vy[4 + n] = vy[v1] + mu * (vy[v2] - vy[v1]);
        vz[4 + n] = vz[v1] + mu * (vz[v2] - vz[v1]);
    }
    double vol = 0.0, liq = 0.0;
    for (int n = C.ntets - 1; n >= C.nntet - 1; --n) {
        const double tv = tet_vol32(vx, vy, vz, C.vtet[n][0], C.vtet[n][1], C.vtet[n][2], C.vtet[n][3]);
        vol += tv;
        liq += tv;
    }
    for (int n = 0; n < C.nntet - 1; ++n) vol += tet_vol32(vx, vy, vz, C.vtet[n][0], C.vtet[n][1], C.vtet[n][2], C.vtet[n][3]);
    rv = vol;
    rl = liq;
}

__device__ __forceinline__ void form_child32(const Frame32& F, const CutCase* tab, int n, float* cx, float* cy,
                                             float* cz, int (*ci)[3])
{
    const CutCase& C = tab[F.cs];
    const int side = C.side[n];
    for (int nn = 0; nn < 4; ++nn) {
        const int v = C.vtet[n][nn];
        cx[nn] = F.x[v]; cy[nn] = F.y[v]; cz[nn] = F.z[v];
        ci[nn][0] = F.ind[v][0]; ci[nn][1] = F.ind[v][1]; ci[nn][2] = F.ind[v][2];
        if (side == 1) ci[nn][(int)F.dir] = F.cut;
    }
}

/* cutTet (src/VFgeom.jl:713-900) with an explicit stack; indices relative to the cell. */
__device__ void clip32(const DevMesh& m, const CutCase* tab, const Plane32& PL, int i0, int j0, int k0,
                       const int* rlo, const int* rhi, float* cx, float* cy, float* cz, int (*ci)[3], double& out_v,
                       double& out_l, int& err)
{
    Frame32 st[CLIP_STACK];
    int depth = 0, flags = 0, leaves = 0;
    for (;;) {
        int dir = -1, cut = 0;
        for (int q = 0; q < 3; ++q) {
            if (flags & (1 << q)) continue;
            const int mx = max(max(ci[0][q], ci[1][q]), max(ci[2][q], ci[3][q]));
            const int mn = min(min(ci[0][q], ci[1][q]), min(ci[2][q], ci[3][q]));
            if (mx > mn) { dir = q; cut = mx; break; }
            flags |= 1 << q;
        }
        double rv, rl;
        if (dir >= 0 && depth == CLIP_STACK) { err |= ERR_DEPTH; dir = -1; }
        if (dir < 0) {
            if (++leaves > CLIP_MAX_LEAVES) {
                err |= ERR_DEPTH;
                out_v = 0.0; out_l = 0.0;
                return;
            }
            leaf32(m, tab, PL, i0, j0, k0, cx, cy, cz, ci[0][0], ci[0][1], ci[0][2], rv, rl, err);
        } else {
            Frame32& F = st[depth];
            const float pl = (float)cut;
            const float* cd = dir == 0 ? cx : (dir == 1 ? cy : cz);
            float d[4];
            for (int n = 0; n < 4; ++n) d[n] = cd[n] - pl;
            float c0 = d[0], c1 = d[1], c2 = d[2], c3 = d[3];
            const int cs = d2case(c0, c1, c2, c3, 1e-30f, err);
            for (int n = 0; n < 4; ++n) {
                F.x[n] = cx[n]; F.y[n] = cy[n]; F.z[n] = cz[n];
                F.ind[n][0] = (signed char)ci[n][0]; F.ind[n][1] = (signed char)ci[n][1];
                F.ind[n][2] = (signed char)ci[n][2];
                F.ind[n][dir] = (signed char)min(ci[n][dir], cut - 1);
            }
            const CutCase& C = tab[cs];
            for (int n = 0; n < C.nvert; ++n) {
                const int v1 = C.v1[n], v2 = C.v2[n];
                const float den = d[v2] - d[v1];
                const float mu = fminf(1.f, fmaxf(0.f, den != 0.f ? -d[v1] / den : 1.f));
                const float x = F.x[v1] + mu * (F.x[v2] - F.x[v1]);
                const float y = F.y[v1] + mu * (F.y[v2] - F.y[v1]);
                const float z = F.z[v1] + mu * (F.z[v2] - F.z[v1]);
                F.x[4 + n] = x; F.y[4 + n] = y; F.z[4 + n] = z;
                const int Iv[3] = {idx32(x, F.ind[n][0], rlo[0], rhi[0], err), idx32(y, F.ind[n][1], rlo[1], rhi[1], err),
                                   idx32(z, F.ind[n][2], rlo[2], rhi[2], err)};
                for (int q = 0; q < 3; ++q) {
                    int val = max(Iv[q], min((int)F.ind[v1][q], (int)F.ind[v2][q]));
                    val = min(val, max((int)F.ind[v1][q], (int)F.ind[v2][q]));
                    F.ind[4 + n][q] = (signed char)val;
                }
                F.ind[4 + n][dir] = (signed char)(cut - 1);
            }
            F.cs = (signed char)cs; F.dir = (signed char)dir; F.cut = (signed char)cut; F.flags = (signed char)flags;
            F.acc_v = 0.0; F.acc_l = 0.0; F.next = 1;
            ++depth;
            form_child32(F, tab, 0, cx, cy, cz, ci);
            continue;
        }
        for (;;) {
            if (depth == 0) { out_v = rv; out_l = rl; return; }
            Frame32& F = st[depth - 1];
            F.acc_v += rv;
            F.acc_l += rl;
            if (F.next < tab[F.cs].ntets) {
                form_child32(F, tab, F.next, cx, cy, cz, ci);
                F.next += 1;
                flags = F.flags;
                break;
            }
            rv = F.acc_v; rl = F.acc_l;
            --depth;
        }
    }
}

constexpr int SL32_THREADS = 128;

__device__ __forceinline__ void sl_cell32(const DevMesh& m, const CutCase* tab, float dt, double* __restrict__ VFout,
                                          const Vel32& V, const Plane32& PL, const signed char* __restrict__ phase,
                                          int L, int& err)
{
    const int i = 1 + L % m.N[0];
    const int j = 1 + (L / m.N[0]) % m.N[1];
    const int k = 1 + L / (m.N[0] * m.N[1]);
    const bool even = ((i + j + k) % 2) == 0;
    const double tetsign = even ? 1.0 : -1.0;
    /* relative index bounds: inside the arrays and within REL of the cell */
    const int rlo[3] = {max(m.lo - i, -REL), max(m.lo - j, -REL), max(m.lo - k, -REL)};
    const int rhi[3] = {min(m.hi[0] - i, REL), min(m.hi[1] - j, REL), min(m.hi[2] - k, REL)};
    float px[8], py[8], pz[8];
    int vi[8][3];
#pragma unroll 1
    for (int v = 0; v < 8; ++v) {
        const int a = v & 1;
        float x = (float)(even ? a : 1 - a), y = (float)((v >> 1) & 1), z = (float)(v >> 2);
        project32(m, V, i, j, k, dt, x, y, z);
        px[v] = x; py[v] = y; pz[v] = z;
        vi[v][0] = idx32(x, 0, rlo[0], rhi[0], err);
        vi[v][1] = idx32(y, 0, rlo[1], rhi[1], err);
        vi[v][2] = idx32(z, 0, rlo[2], rhi[2], err);
    }
    const long out = vidx(m, i, j, k);
    /* pure-donor shortcut (see k_fp64.cu) on the phase codes of the PLIC pass */
    if (m.fast_pure) {
        int lo0 = vi[0][0], hi0 = vi[0][0], lo1 = vi[0][1], hi1 = vi[0][1], lo2 = vi[0][2], hi2 = vi[0][2];
        for (int v = 1; v < 8; ++v) {
            lo0 = min(lo0, vi[v][0]); hi0 = max(hi0, vi[v][0]);
            lo1 = min(lo1, vi[v][1]); hi1 = max(hi1, vi[v][1]);
            lo2 = min(lo2, vi[v][2]); hi2 = max(hi2, vi[v][2]);
        }
        int ph = 2;
        if (hi0 - lo0 <= 3 && hi1 - lo1 <= 3 && hi2 - lo2 <= 3) {
            for (int c = lo2; c <= hi2 && ph != 0; ++c)
                for (int b = lo1; b <= hi1 && ph != 0; ++b)
                    for (int a = lo0; a <= hi0; ++a) {
                        const int p = __ldg(phase + cidx(m, i + a, j + b, k + c));
                        if (p == 0 || (ph != 2 && p != ph)) { ph = 0; break; }
                        ph = p;
                    }
        } else {
            ph = 0;
        }
        if (ph == 1 || ph == -1) {
            float vol = 0.f;
            for (int t = 0; t < 5; ++t)
                vol += tet_vol32(px, py, pz, tet5(t, 0), tet5(t, 1), tet5(t, 2), tet5(t, 3));
            vol *= (float)tetsign;
            if (vol > 0.25f && vol < 4.f) {
                VFout[out] = ph > 0 ? 1.0 : 0.0;
                return;
            }
        }
    }
    double vol = 0.0, liq = 0.0;
#pragma unroll 1
    for (int t = 0; t < 5; ++t) {
        float cx[4], cy[4], cz[4];
        int ci[4][3];
        for (int n = 0; n < 4; ++n) {
            const int v = tet5(t, n);
            cx[n] = px[v]; cy[n] = py[v]; cz[n] = pz[v];
            ci[n][0] = vi[v][0]; ci[n][1] = vi[v][1]; ci[n][2] = vi[v][2];
        }
        double tv, tl;
        clip32(m, tab, PL, i, j, k, rlo, rhi, cx, cy, cz, ci, tv, tl, err);
        vol += tetsign * tv;
        liq += tetsign * tl;
    }
    if (!(vol > 0.0) || !isfinite(vol)) err |= ERR_VOLUME;
    VFout[out] = liq / vol;
}

__global__ void __launch_bounds__(SL32_THREADS) k_sl32(DevMesh m, float dt, double* __restrict__ VFout, Vel32 V,
                                                       Plane32 PL, const signed char* __restrict__ phase,
                                                       const int* __restrict__ list, const int* __restrict__ count,
                                                       int* work, int* errw)
{
    __shared__ CutCase s_tab[16];
    for (int t = threadIdx.x; t < 16 * (int)sizeof(CutCase); t += blockDim.x)
        reinterpret_cast<char*>(s_tab)[t] = reinterpret_cast<const char*>(c_cut)[t];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int n_items = *count;
    int err = 0;
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(work, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n_items) break;
        const int item = base + lane;
        if (item < n_items) sl_cell32(m, s_tab, dt, VFout, V, PL, phase, list[item], err);
        __syncwarp();
    }
    if (err) atomicOr(errw, err);
}

/* ---- launchers ------------------------------------------------------------------------ */
void launch_elvira_iface32(const DevMesh& m, const double* VF, double* nx, double* ny, double* nz, const int* list,
                           const int* count, int* work, int nsm, cudaStream_t s)
{
    k_elvira_iface32<<<nsm * 8, EL32_WARPS * 32, 0, s>>>(m, VF, nx, ny, nz, list, count, work);
}

void launch_sl32(const DevMesh& m, double dt, double* VFout, const float* uf, const float* vf, const float* wf,
                 const float4* planes, const signed char* phase, const int* list, const int* count, int* work,
                 int* errw, int nsm, cudaStream_t s)
{
    Vel32 V{uf, vf, wf};
    Plane32 PL{planes};
    k_sl32<<<nsm * 8, SL32_THREADS, 0, s>>>(m, (float)dt, VFout, V, PL, phase, list, count, work, errw);
}

} // namespace slvof
