/*
 * k_elvira_mixed.cu — ELVIRA for interface cells in the mixed-precision path.  Built with
 * -fmad=false so that its FP64 part rounds exactly like the FP64 path; the FP32 hot loop uses
 * explicit fmaf.
 *
 * Candidate errors (check_normal!, src/ELVIRA.jl:106-137) are evaluated in FP32: the liquid
 * fraction of each 3x3x3 neighbour under a candidate plane is the exact plane/cube volume in
 * closed form (the quantity computePLIC2VF evaluates with five tet clips, src/VF.jl:219-278)
 * and the plane constant is the inverse of the same function (computeAlpha's role,
 * src/VF.jl:164-214).  Candidates whose FP32 error lies within its rounding bound of the best
 * are then re-scored in FP64 exactly as the FP64 path scores them (5-tet clips, lanes =
 * neighbours, errors summed in neighbour order), and the first strict minimum wins; the chosen
 * candidate is re-formed and normalised in FP64.
 */
#include "slvof_kernels.h"
#include "slvof_dev.cuh"
#include "plic64.cuh"

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

/* The volume below a in [0, 1/2], every interval's expression evaluated and the right one
 * selected, so a warp whose lanes score different candidate planes (in different intervals)
 * does not diverge; where b = a - m2 <= 0 or c = a - m3 <= 0 that cubic correction vanishes. */
__device__ __forceinline__ float cube_lower_sel(const Cube& q, float a)
{
    const float t1 = a * a * a * q.im1 * q.i6m23;
    const float base = fmaf(3.f * a, a - q.m1, q.m1 * q.m1) * q.i6m23;
    const float b = fmaxf(a - q.m2, 0.f), c = fmaxf(a - q.m3, 0.f);
    const float corr = fmaf((b * q.im1) * b, b, (c * q.im1) * c * c);
    const float cub = fmaf(-corr, q.i6m23, base);
    const float lin = fmaf(2.f, a, -q.m12) * q.i2m3;
    const float r = (q.m3 >= q.m12 && a >= q.m12) ? lin : cub;
    return a < q.m1 ? t1 : r;
}

/* d/da of cube_lower_sel (the cut area), for the Newton inverse, the same way. */
__device__ __forceinline__ float cube_area_sel(const Cube& q, float a)
{
    const float t1 = 3.f * a * a * q.im1 * q.i6m23;
    const float base = (6.f * a - 3.f * q.m1) * q.i6m23;
    const float b = fmaxf(a - q.m2, 0.f), c = fmaxf(a - q.m3, 0.f);
    const float cub = base - 3.f * ((b * q.im1) * b + (c * q.im1) * c) * q.i6m23;
    const float r = (q.m3 >= q.m12 && a >= q.m12) ? 2.f * q.i2m3 : cub;
    return a < q.m1 ? t1 : r;
}

/* The fraction for any a: 0 below the cube, 1 above, V(a) = 1 - V(1 - a) above 1/2. */
__device__ __forceinline__ float cube_frac(const Cube& q, float a)
{
    const bool upper = a > 0.5f;
    const float aa = fminf(fmaxf(upper ? 1.f - a : a, 0.f), 0.5f);
    const float r = cube_lower_sel(q, aa);
    return upper ? 1.f - r : r;
}

/* alpha with cube_lower_sel(alpha) = V for V in [0, 1/2] (computeAlpha's role, src/VF.jl:164-214).
 * The first two intervals and the linear one are inverted in closed form (cbrt, the
 * quadratic root, a line); on the cubic interval the bracket end points are known, so a
 * linear start and bracketed Newton converge to FP32 rounding in a few steps. */
__device__ __forceinline__ float cube_alpha(const Cube& q, float V)
{
    if (V <= 0.f) return 0.f;
    if (q.m2 <= 0.f) return V; /* plane parallel to a face: V(a) = a */
    const float V1 = q.m1 * q.m1 * q.i6m23;
    if (V < V1) return cbrtf(V * 6.f * q.m1 * q.m2 * q.m3);
    const float V2 = fmaf(3.f * q.m2, q.m2 - q.m1, q.m1 * q.m1) * q.i6m23;
    if (V < V2) return fmaf(0.5f, q.m1, sqrtf(fmaxf(fmaf(2.f * q.m2 * q.m3, V, -q.m1 * q.m1 * (1.f / 12.f)), 0.f)));
    float lo, hi;
    if (q.m3 >= q.m12) {
        if (V >= q.m12 * q.i2m3) return fmaf(V, q.m3, 0.5f * q.m12);
        lo = q.m2; hi = q.m12;
    } else {
        if (V < cube_lower_sel(q, q.m3)) { lo = q.m2; hi = q.m3; }
        else { lo = q.m3; hi = 0.5f; }
    }
    const float vl = cube_lower_sel(q, lo), vh = cube_lower_sel(q, hi);
    float a = vh > vl ? fmaf((V - vl) / (vh - vl), hi - lo, lo) : 0.5f * (lo + hi);
#pragma unroll 1
    for (int it = 0; it < 5; ++it) {
        const float f = cube_lower_sel(q, a) - V;
        if (f > 0.f) hi = a;
        else lo = a;
        const float s = cube_area_sel(q, a);
        float an = s > 0.f ? a - f / s : 0.5f * (lo + hi);
        if (!(an >= lo && an <= hi)) an = 0.5f * (lo + hi);
        a = an;
    }
    return a;
}

/* The same plane/cube volume and its derivative in FP64, for the plane-constant root of the
 * mixed path: the FP32 inverse above starts FP64 Newton steps on this function. */
struct Cube64 {
    double m1, m2, m3, m12, i6m23, i2m3, im1;
};

__device__ __forceinline__ Cube64 make_cube64(double a, double b, double c)
{
    double t;
    if (a > b) { t = a; a = b; b = t; }
    if (b > c) { t = b; b = c; c = t; }
    if (a > b) { t = a; a = b; b = t; }
    Cube64 q;
    q.m1 = a; q.m2 = b; q.m3 = c; q.m12 = a + b;
    q.i6m23 = (b > 0.0) ? 1.0 / (6.0 * b * c) : 0.0;
    q.i2m3 = c > 0.0 ? 0.5 / c : 0.0;
    q.im1 = (a > 0.0) ? 1.0 / a : 0.0;
    return q;
}

__device__ __forceinline__ void cube_lower64(const Cube64& q, double a, double& V, double& dV)
{
    if (a < q.m1) {
        V = a * a * a * q.im1 * q.i6m23;
        dV = 3.0 * a * a * q.im1 * q.i6m23;
        return;
    }
    V = (3.0 * a * (a - q.m1) + q.m1 * q.m1) * q.i6m23;
    dV = (6.0 * a - 3.0 * q.m1) * q.i6m23;
    if (a < q.m2) return;
    if (a < q.m12 && a < q.m3) {
        const double b = a - q.m2;
        V -= (b * q.im1) * b * b * q.i6m23;
        dV -= 3.0 * (b * q.im1) * b * q.i6m23;
        return;
    }
    if (q.m3 < q.m12) {
        const double b = a - q.m2, c = a - q.m3;
        V -= ((b * q.im1) * b * b + (c * q.im1) * c * c) * q.i6m23;
        dV -= 3.0 * ((b * q.im1) * b + (c * q.im1) * c) * q.i6m23;
        return;
    }
    V = (2.0 * a - q.m12) * q.i2m3;
    dV = 2.0 * q.i2m3;
}

/* computeDist (src/VF.jl:109-156) with computeAlpha's inverse (src/VF.jl:164-214) taken as the
 * FP32 closed-form inverse plus FP64 Newton steps on the exact volume: the same plane
 * constant to within a few units of FP64 rounding, without the trigonometric branch. */
__device__ __forceinline__ double compute_dist_newton(const DevMesh& m, int i, int j, int k, double nx, double ny,
                                                      double nz, double VF)
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
    const Cube64 q = make_cube64(fabs(m0), fabs(m1), fabs(m2));
    double alpha;
    if (q.m3 <= 0.0) {
        alpha = 0.0; /* n = 0: computeAlpha's quadratic branch gives 0 */
    } else if (q.m2 <= 0.0) {
        alpha = VFo; /* plane parallel to a face: V(a) = a */
    } else {
        alpha = (double)cube_alpha(make_cube((float)q.m1, (float)q.m2, (float)q.m3), (float)VFo);
        for (int it = 0; it < 3; ++it) {
            double V, dV;
            cube_lower64(q, alpha, V, dV);
            if (!(dV > 0.0)) break;
            const double step = (V - VFo) / dV;
            alpha -= step;
            if (fabs(step) <= 1e-17) break;
        }
        alpha = fmin(fmax(alpha, 0.0), 0.5);
    }
    alpha = VF > 0.5 ? 1.0 - alpha : alpha;
    alpha += factor;
    alpha -= 0.5 * ((m0 + m1) + m2);
    double dist = alpha * norm;
    dist += (nx * cco(m, 0, i) + ny * cco(m, 1, j)) + nz * cco(m, 2, k);
    return dist;
}

__global__ void k_plic_iface_newton(DevMesh m, const double* __restrict__ VF, const double* __restrict__ nx,
                                    const double* __restrict__ ny, const double* __restrict__ nz,
                                    double* __restrict__ D, float4* __restrict__ planes,
                                    signed char* __restrict__ phase, const int* __restrict__ list,
                                    const int* __restrict__ count)
{
    const long n0 = m.N[0] + 2 * m.g, n1 = m.N[1] + 2 * m.g;
    const int n = *count;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int t = list[q];
        const int ip = (int)(t % n0) + m.lo, jp = (int)((t / n0) % n1) + m.lo, kp = (int)(t / (n0 * n1)) + m.lo;
        const int i = ghost_src_1d(ip, m.N[0], m.g, m.per[0], false);
        const int j = ghost_src_1d(jp, m.N[1], m.g, m.per[1], false);
        const int k = ghost_src_1d(kp, m.N[2], m.g, m.per[2], false);
        const long c = cidx(m, i, j, k);
        const double dist = compute_dist_newton(m, i, j, k, nx[c], ny[c], nz[c], VF[vidx(m, i, j, k)]);
        plic_outputs(m, t, ip, jp, kp, dist, nx, ny, nz, D, planes, phase);
    }
}

void launch_plic_iface_newton(const DevMesh& m, const double* VF, const double* nx, const double* ny, const double* nz,
                              double* D, float4* planes, signed char* phase, const int* list, const int* count,
                              int nsm, cudaStream_t s)
{
    k_plic_iface_newton<<<nsm * 4, 128, 0, s>>>(m, VF, nx, ny, nz, D, planes, phase, list, count);
}

/* Candidate normal of lane (family f, outer a, inner b) from a 3x3x3 VF block; R = float
 * for the error pass, double to form candidates exactly as the FP64 path does. */
/* sg[0..2]: the family's third component, -1 where the +1 neighbour along that axis holds
 * more liquid than the -1 neighbour, else +1 (VF[+1] > VF[-1] ? -1 : 1), decided on the FP64
 * VF in both precisions: two values that differ in FP64 can round to the same float. */
template <class R>
__device__ __forceinline__ void candidate(const R* sv, int f, int a, int b, R dx, R dy, R dz, const R* hx, const R* hy,
                                          const R* hz, const R* sg, R& cx, R& cy, R& cz)
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
        cz = sg[2];
    } else if (f == 1) {
        const R s2x = (V3(i2, -1, 0) * dy + V3(i2, 0, 0) * dy) + V3(i2, 1, 0) * dy;
        const R s1x = (V3(i1, -1, 0) * dy + V3(i1, 0, 0) * dy) + V3(i1, 1, 0) * dy;
        cx = -(s2x - s1x) / hx[b];
        cy = sg[1];
        const R s2z = (V3(0, -1, o2) * dy + V3(0, 0, o2) * dy) + V3(0, 1, o2) * dy;
        const R s1z = (V3(0, -1, o1) * dy + V3(0, 0, o1) * dy) + V3(0, 1, o1) * dy;
        cz = -(s2z - s1z) / hz[a];
    } else {
        cx = sg[0];
        const R s2y = (V3(-1, i2, 0) * dx + V3(0, i2, 0) * dx) + V3(1, i2, 0) * dx;
        const R s1y = (V3(-1, i1, 0) * dx + V3(0, i1, 0) * dx) + V3(1, i1, 0) * dx;
        cy = -(s2y - s1y) / hy[b];
        const R s2z = (V3(-1, 0, o2) * dx + V3(0, 0, o2) * dx) + V3(1, 0, o2) * dx;
        const R s1z = (V3(-1, 0, o1) * dx + V3(0, 0, o1) * dx) + V3(1, 0, o1) * dx;
        cz = -(s2z - s1z) / hz[a];
    }
#undef V3
}


constexpr int EL32_WARPS = 8;

__device__ __forceinline__ int lane_family(const int* fam_on, int lane)
{
    const int fam = lane / 9;
    for (int q = 0, seen = 0; q < 3; ++q)
        if (fam_on[q]) { if (seen == fam) return q; ++seen; }
    return 0;
}

/* Candidate of lane c in FP64, L2-normalised (src/ELVIRA.jl:72-98,112-115). */
__device__ __forceinline__ void candidate64(const DevMesh& m, const double* sv, const int* fam_on, int c, int i, int j,
                                            int k, double& cx, double& cy, double& cz)
{
    const double hx[3] = {cco(m, 0, i) - cco(m, 0, i - 1), cco(m, 0, i + 1) - cco(m, 0, i - 1),
                          cco(m, 0, i + 1) - cco(m, 0, i)};
    const double hy[3] = {cco(m, 1, j) - cco(m, 1, j - 1), cco(m, 1, j + 1) - cco(m, 1, j - 1),
                          cco(m, 1, j + 1) - cco(m, 1, j)};
    const double hz[3] = {cco(m, 2, k) - cco(m, 2, k - 1), cco(m, 2, k + 1) - cco(m, 2, k - 1),
                          cco(m, 2, k + 1) - cco(m, 2, k)};
    /* VF[+1] > VF[-1] ? -1 : 1 along x, y, z (src/ELVIRA.jl:72-98) */
    const double sg[3] = {sv[14] > sv[12] ? -1.0 : 1.0, sv[16] > sv[10] ? -1.0 : 1.0, sv[22] > sv[4] ? -1.0 : 1.0};
    candidate<double>(sv, lane_family(fam_on, c), (c % 9) / 3, c % 3, m.d[0], m.d[1], m.d[2], hx, hy, hz, sg, cx, cy,
                      cz);
    const double norm = sqrt((cx * cx + cy * cy) + cz * cz);
    cx = cx / norm; cy = cy / norm; cz = cz / norm;
}

__global__ void __launch_bounds__(EL32_WARPS * 32) k_elvira_iface32(DevMesh m, const double* __restrict__ VF,
                                                                    const int* __restrict__ list,
                                                                    const int* __restrict__ count, int* work,
                                                                    int* n_arb, int2* __restrict__ arb,
                                                                    signed char* __restrict__ cand)
{
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
        double v64 = 0.0;
        if (lane < 27) {
            v64 = VF[vidx(m, i - 1 + lane % 3, j - 1 + (lane / 3) % 3, k - 1 + lane / 9)];
            s_vf[w][lane] = (float)v64;
        }
        /* the candidates' third components from the FP64 VF of the face neighbours */
        const double vxp = __shfl_sync(0xffffffffu, v64, 14), vxm = __shfl_sync(0xffffffffu, v64, 12);
        const double vyp = __shfl_sync(0xffffffffu, v64, 16), vym = __shfl_sync(0xffffffffu, v64, 10);
        const double vzp = __shfl_sync(0xffffffffu, v64, 22), vzm = __shfl_sync(0xffffffffu, v64, 4);
        const float sg[3] = {vxp > vxm ? -1.f : 1.f, vyp > vym ? -1.f : 1.f, vzp > vzm ? -1.f : 1.f};
        const double vc64 = __shfl_sync(0xffffffffu, v64, 13);
        const bool upper_c = vc64 > 0.5;
        const float vo_c = (float)(upper_c ? 1.0 - vc64 : vc64);
        __syncwarp();
        const float* sv = s_vf[w];
        float err_ = INFINITY, tol = 0.f;
        if (lane < ncand) {
            const int f = lane_family(fam_on, lane);
            const int a = (lane % 9) / 3, b = lane % 3;
            float cx, cy, cz;
            const float hx[3] = {dx, 2.f * dx, dx}, hy[3] = {dy, 2.f * dy, dy}, hz[3] = {dz, 2.f * dz, dz};
            candidate<float>(sv, f, a, b, dx, dy, dz, hx, hy, hz, sg, cx, cy, cz);
            const float nrm = sqrtf(fmaf(cx, cx, fmaf(cy, cy, cz * cz)));
            cx /= nrm; cy /= nrm; cz /= nrm;
            /* computeDist in cell units: mm = n*d/|n*d|_1; neighbour (p,r,s) holds the cube
             * fraction at al - mm.(p,r,s) (sign folding absorbed in al) */
            float m0 = cx * dx, m1 = cy * dy, m2 = cz * dz;
            const float n1 = fabsf(m0) + fabsf(m1) + fabsf(m2);
            m0 /= n1; m1 /= n1; m2 /= n1;
            const Cube q = make_cube(fabsf(m0), fabsf(m1), fabsf(m2));
            /* min(VF, 1 - VF) of the cell itself from its FP64 value: a VF within 3e-8 of 1
             * rounds to 1 in FP32, and the plane constant of a nearly full (or empty) cell
             * goes with the cube root of that small volume */
            float al = cube_alpha(q, vo_c);
            al = upper_c ? 1.f - al : al;
            float e2 = 0.f, sa = 0.f;
#pragma unroll
            for (int c = 0; c < 27; ++c) {
                const float p = (float)(c % 3 - 1), r = (float)((c / 3) % 3 - 1), s = (float)(c / 9 - 1);
                const float ae = al - fmaf(m0, p, fmaf(m1, r, m2 * s));
                const float d = sv[c] - cube_frac(q, ae);
                e2 = fmaf(d, d, e2);
                sa += fabsf(d);
            }
            err_ = e2;
            /* bound on the FP32 error of e2: each fraction is good to a few 1e-7 */
            tol = 4e-6f * sa + 1e-5f * e2 + 1e-12f;
        }
        /* FP32 winner and the set of candidates that could beat it in exact arithmetic */
        const bool fin = err_ < INFINITY;
        float hi = fin ? err_ + tol : INFINITY;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) hi = fminf(hi, __shfl_xor_sync(0xffffffffu, hi, off));
        const unsigned contend = __ballot_sync(0xffffffffu, fin && err_ - tol <= hi);
        if (lane == 0) {
            if (__popc(contend) <= 1) {
                cand[cidx(m, i, j, k)] = (signed char)(contend ? __ffs(contend) - 1 : -1);
            } else {
                /* near-tie: the FP64 scoring pass decides */
                const int slot = atomicAdd(n_arb, 1);
                arb[slot] = make_int2(L, (int)contend);
            }
        }
        __syncwarp();
    }
}

/* FP64 arbitration of the near-ties: the contending candidates scored exactly as
 * check_normal! scores them in the FP64 path (computeDist, 5-tet clips of the 27 neighbours,
 * squared errors summed in neighbour order), the first strict minimum wins.  A block per cell,
 * a thread per (candidate, neighbour) pair: the scoring's long FP64 chains run side by side
 * instead of one contender after another in one warp.  A separate pass keeps this FP64 code and
 * its registers out of the FP32 scoring kernel. */
constexpr int ARB_THREADS = 256;

__global__ void __launch_bounds__(ARB_THREADS) k_elvira_arb64(DevMesh m, const double* __restrict__ VF,
                                                              const int* __restrict__ n_arb,
                                                              const int2* __restrict__ arb,
                                                              signed char* __restrict__ cand, int* errw)
{
    __shared__ CutCase s_tab[16];
    __shared__ double s_vd[27], s_full[27], s_term[27][5];
    __shared__ double s_n[27][3], s_dist[27];
    __shared__ double s_r2[27][27];
    __shared__ int s_c[27];
    load_table(s_tab);
    const int tid = threadIdx.x;
    const int fam_on[3] = {m.N[2] > 1, m.N[1] > 1, m.N[0] > 1};
    const int n = *n_arb;
    int err = 0;
    for (int item = blockIdx.x; item < n; item += gridDim.x) {
        const int2 e = arb[item];
        const int L = e.x;
        const unsigned contend = (unsigned)e.y;
        const int nc = __popc(contend);
        const int i = 1 + L % m.N[0];
        const int j = 1 + (L / m.N[0]) % m.N[1];
        const int k = 1 + L / (m.N[0] * m.N[1]);
        if (tid < 27) {
            s_vd[tid] = VF[vidx(m, i - 1 + tid % 3, j - 1 + (tid / 3) % 3, k - 1 + tid / 9)];
            NbrGeom G;
            nbr_geom(m, i - 1 + tid % 3, j - 1 + (tid / 3) % 3, k - 1 + tid / 9, G);
            double full = 0.0;
#pragma unroll
            for (int t = 0; t < 5; ++t) {
                const int a = tet5(t, 0), b = tet5(t, 1), c = tet5(t, 2), ee = tet5(t, 3);
                const double tv = tet_vol(G.X[a & 1], G.Y[(a >> 1) & 1], G.Z[a >> 2], G.X[b & 1], G.Y[(b >> 1) & 1],
                                          G.Z[b >> 2], G.X[c & 1], G.Y[(c >> 1) & 1], G.Z[c >> 2], G.X[ee & 1],
                                          G.Y[(ee >> 1) & 1], G.Z[ee >> 2]);
                const double term = G.tetsign * tv / m.cellvol;
                s_term[tid][t] = term;
                full += term;
            }
            s_full[tid] = full;
            /* the q-th contending lane, in lane order */
            unsigned mask = contend;
            for (int q = 0; q < tid && mask; ++q) mask &= mask - 1;
            s_c[tid] = mask ? __ffs(mask) - 1 : -1;
        }
        __syncthreads();
        if (tid < nc) {
            double cx, cy, cz;
            candidate64(m, s_vd, fam_on, s_c[tid], i, j, k, cx, cy, cz);
            s_n[tid][0] = cx; s_n[tid][1] = cy; s_n[tid][2] = cz;
            s_dist[tid] = compute_dist64(m, i, j, k, cx, cy, cz, s_vd[13]);
        }
        __syncthreads();
        for (int pq = tid; pq < nc * 27; pq += ARB_THREADS) {
            const int c = pq / 27, q = pq - 27 * c;
            const int ii = i - 1 + q % 3, jj = j - 1 + (q / 3) % 3, kk = k - 1 + q / 9;
            double v_;
            if (m.tess == 5) {
                NbrGeom G;
                nbr_geom(m, ii, jj, kk, G);
                v_ = plic2vf64(s_tab, G, s_term[q], s_full[q], s_n[c][0], s_n[c][1], s_n[c][2], s_dist[c], m.cellvol,
                               err);
            } else {
                v_ = plic2vf64_gen(s_tab, m, ii, jj, kk, s_n[c][0], s_n[c][1], s_n[c][2], s_dist[c], err);
            }
            const double r = s_vd[q] - v_;
            s_r2[c][q] = r * r;
        }
        __syncthreads();
        if (tid == 0) {
            double bestE = INFINITY;
            int winner = -1;
            for (int c = 0; c < nc; ++c) {
                double e2 = 0.0;
                for (int q = 0; q < 27; ++q) e2 += s_r2[c][q];
                if (e2 < bestE) { bestE = e2; winner = s_c[c]; }
            }
            cand[cidx(m, i, j, k)] = (signed char)winner;
        }
        __syncthreads();
    }
    if (err) atomicOr(errw, err);
}

/* The chosen candidate of every interface cell re-formed from its VF block and normalised
 * in FP64 exactly as the FP64 path forms it (src/ELVIRA.jl:72-98,112-115), one thread per
 * cell: on GB300 the FP64 pipe is charged per warp instruction, so this runs 32 cells per
 * instruction instead of one lane of a per-cell warp. */
__global__ void k_elvira_winner64(DevMesh m, const double* __restrict__ VF, double* __restrict__ nx,
                                  double* __restrict__ ny, double* __restrict__ nz, const int* __restrict__ list,
                                  const int* __restrict__ count, const signed char* __restrict__ cand)
{
    const int fam_on[3] = {m.N[2] > 1, m.N[1] > 1, m.N[0] > 1};
    const int n = *count;
    for (int item = blockIdx.x * blockDim.x + threadIdx.x; item < n; item += gridDim.x * blockDim.x) {
        const int L = list[item];
        const int i = 1 + L % m.N[0];
        const int j = 1 + (L / m.N[0]) % m.N[1];
        const int k = 1 + L / (m.N[0] * m.N[1]);
        const long o = cidx(m, i, j, k);
        const int c = cand[o];
        if (c < 0) continue;
        double sv[27];
#pragma unroll
        for (int q = 0; q < 27; ++q) sv[q] = __ldg(VF + vidx(m, i - 1 + q % 3, j - 1 + (q / 3) % 3, k - 1 + q / 9));
        double cx, cy, cz;
        candidate64(m, sv, fam_on, c, i, j, k, cx, cy, cz);
        nx[o] = cx; ny[o] = cy; nz[o] = cz;
    }
}

void launch_elvira_iface32(const DevMesh& m, const double* VF, double* nx, double* ny, double* nz, const int* list,
                           const int* count, int* work, int* n_arb, int2* arb, signed char* cand, int* errw, int nsm,
                           cudaStream_t s)
{
    k_elvira_iface32<<<nsm * 4, EL32_WARPS * 32, 0, s>>>(m, VF, list, count, work, n_arb, arb, cand);
    k_elvira_arb64<<<nsm * 8, ARB_THREADS, 0, s>>>(m, VF, n_arb, arb, cand, errw);
    k_elvira_winner64<<<nsm * 8, 128, 0, s>>>(m, VF, nx, ny, nz, list, count, cand);
}

} // namespace slvof
