/*
 * k_fp64.cu — FP64 kernels of the SL-VOF path.  Built with -fmad=false: every expression
 * keeps the reference's operation order and IEEE rounding, so results match the CPU
 * restatement bit for bit (the elementary functions come from detmath.h).
 *
 *   k_elvira_iface64 : ELVIRA_calc!/check_normal! (src/ELVIRA.jl:62-137) for interface cells,
 *                      one warp per cell, lane = candidate normal, warp argmin.
 *   k_plic64         : computePLIC! (src/VF.jl:94-103) on every cell incl. ghosts, with the
 *                      single-rank border copy folded in through the ghost source map.
 *   k_sl64           : the SL cell update of transport! (src/Transport.jl:111-148): RK
 *                      pre-image (project!, src/Tools.jl:392-641), pt2index!, cutTet
 *                      (src/VFgeom.jl:713-900) with an explicit stack.
 */
#include "slvof_kernels.h"
#include "slvof_dev.cuh"
#include "plic64.cuh"

namespace slvof {

/* ======================================================================================
 * ELVIRA for interface cells: one warp per cell, lane = candidate (family XY, XZ, YZ in the
 * reference's order, outer list first), warp argmin keeping the first strict minimum.
 * ==================================================================================== */
constexpr int EL_WARPS = 4;

__global__ void __launch_bounds__(EL_WARPS * 32) k_elvira_iface64(DevMesh m, const double* __restrict__ VF,
                                                                  double* __restrict__ nx, double* __restrict__ ny,
                                                                  double* __restrict__ nz, const int* __restrict__ list,
                                                                  const int* __restrict__ count, int* work,
                                                                  signed char* __restrict__ cand, int* errw)
{
    __shared__ CutCase s_tab[16];
    __shared__ double s_term[EL_WARPS][27][5];
    __shared__ double s_full[EL_WARPS][27];
    __shared__ double s_vf[EL_WARPS][27];
    load_table(s_tab);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_items = *count;
    const int fam_on[3] = {m.N[2] > 1, m.N[1] > 1, m.N[0] > 1};
    const int ncand = 9 * (fam_on[0] + fam_on[1] + fam_on[2]);
    int err = 0;
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
            NbrGeom G;
            nbr_geom(m, i - 1 + lane % 3, j - 1 + (lane / 3) % 3, k - 1 + lane / 9, G);
            double full = 0.0;
#pragma unroll
            for (int t = 0; t < 5; ++t) {
                const int a = tet5(t, 0), b = tet5(t, 1), c = tet5(t, 2), e = tet5(t, 3);
                const double tv = tet_vol(G.X[a & 1], G.Y[(a >> 1) & 1], G.Z[a >> 2], G.X[b & 1], G.Y[(b >> 1) & 1],
                                          G.Z[b >> 2], G.X[c & 1], G.Y[(c >> 1) & 1], G.Z[c >> 2], G.X[e & 1],
                                          G.Y[(e >> 1) & 1], G.Z[e >> 2]);
                const double term = G.tetsign * tv / m.cellvol;
                s_term[w][lane][t] = term;
                full += term;
            }
            s_full[w][lane] = full;
            s_vf[w][lane] = VF[vidx(m, i - 1 + lane % 3, j - 1 + (lane / 3) % 3, k - 1 + lane / 9)];
        }
        __syncwarp();
        const double* sv = s_vf[w];
#define V3(a, b, c) sv[((c) + 1) * 9 + ((b) + 1) * 3 + ((a) + 1)]
        double err_ = INFINITY, cx = 0.0, cy = 0.0, cz = 0.0;
        if (lane < ncand) {
            const int fam = lane / 9, a = (lane % 9) / 3, b = lane % 3;
            int f = 0;
            for (int q = 0, seen = 0; q < 3; ++q)
                if (fam_on[q]) { if (seen == fam) { f = q; break; } ++seen; }
            const int o1 = a == 2 ? 0 : -1, o2 = a == 0 ? 0 : 1; /* {-1,0},{-1,1},{0,1} */
            const int i1 = b == 2 ? 0 : -1, i2 = b == 0 ? 0 : 1;
            if (f == 0) { /* X-Y stencils: jj outer, ii inner (src/ELVIRA.jl:71-78) */
                const double s2x = (V3(i2, 0, -1) * m.d[2] + V3(i2, 0, 0) * m.d[2]) + V3(i2, 0, 1) * m.d[2];
                const double s1x = (V3(i1, 0, -1) * m.d[2] + V3(i1, 0, 0) * m.d[2]) + V3(i1, 0, 1) * m.d[2];
                cx = -(s2x - s1x) / (cco(m, 0, i + i2) - cco(m, 0, i + i1));
                const double s2y = (V3(0, o2, -1) * m.d[2] + V3(0, o2, 0) * m.d[2]) + V3(0, o2, 1) * m.d[2];
                const double s1y = (V3(0, o1, -1) * m.d[2] + V3(0, o1, 0) * m.d[2]) + V3(0, o1, 1) * m.d[2];
                cy = -(s2y - s1y) / (cco(m, 1, j + o2) - cco(m, 1, j + o1));
                cz = V3(0, 0, 1) > V3(0, 0, -1) ? -1.0 : 1.0;
            } else if (f == 1) { /* X-Z stencils: kk outer, ii inner (src/ELVIRA.jl:81-88) */
                const double s2x = (V3(i2, -1, 0) * m.d[1] + V3(i2, 0, 0) * m.d[1]) + V3(i2, 1, 0) * m.d[1];
                const double s1x = (V3(i1, -1, 0) * m.d[1] + V3(i1, 0, 0) * m.d[1]) + V3(i1, 1, 0) * m.d[1];
                cx = -(s2x - s1x) / (cco(m, 0, i + i2) - cco(m, 0, i + i1));
                cy = V3(0, 1, 0) > V3(0, -1, 0) ? -1.0 : 1.0;
                const double s2z = (V3(0, -1, o2) * m.d[1] + V3(0, 0, o2) * m.d[1]) + V3(0, 1, o2) * m.d[1];
                const double s1z = (V3(0, -1, o1) * m.d[1] + V3(0, 0, o1) * m.d[1]) + V3(0, 1, o1) * m.d[1];
                cz = -(s2z - s1z) / (cco(m, 2, k + o2) - cco(m, 2, k + o1));
            } else { /* Y-Z stencils: kk outer, jj inner (src/ELVIRA.jl:91-98) */
                cx = V3(1, 0, 0) > V3(-1, 0, 0) ? -1.0 : 1.0;
                const double s2y = (V3(-1, i2, 0) * m.d[0] + V3(0, i2, 0) * m.d[0]) + V3(1, i2, 0) * m.d[0];
                const double s1y = (V3(-1, i1, 0) * m.d[0] + V3(0, i1, 0) * m.d[0]) + V3(1, i1, 0) * m.d[0];
                cy = -(s2y - s1y) / (cco(m, 1, j + i2) - cco(m, 1, j + i1));
                const double s2z = (V3(-1, 0, o2) * m.d[0] + V3(0, 0, o2) * m.d[0]) + V3(1, 0, o2) * m.d[0];
                const double s1z = (V3(-1, 0, o1) * m.d[0] + V3(0, 0, o1) * m.d[0]) + V3(1, 0, o1) * m.d[0];
                cz = -(s2z - s1z) / (cco(m, 2, k + o2) - cco(m, 2, k + o1));
            }
            /* check_normal! (src/ELVIRA.jl:106-137) */
            const double norm = sqrt((cx * cx + cy * cy) + cz * cz);
            cx = cx / norm; cy = cy / norm; cz = cz / norm;
            const double dist = compute_dist64(m, i, j, k, cx, cy, cz, V3(0, 0, 0));
            double e2 = 0.0;
            for (int c = 0; c < 27; ++c) {
                double v_;
                if (m.tess == 5) {
                    NbrGeom G;
                    nbr_geom(m, i - 1 + c % 3, j - 1 + (c / 3) % 3, k - 1 + c / 9, G);
                    v_ = plic2vf64(s_tab, G, s_term[w][c], s_full[w][c], cx, cy, cz, dist, m.cellvol, err);
                } else {
                    v_ = plic2vf64_gen(s_tab, m, i - 1 + c % 3, j - 1 + (c / 3) % 3, k - 1 + c / 9, cx, cy, cz, dist,
                                       err);
                }
                const double r = sv[c] - v_;
                e2 += r * r;
            }
            err_ = e2;
        }
#undef V3
        /* First strict minimum in candidate order: err < running best starting at Inf, so
         * NaN and Inf never win and ties go to the lower lane. */
        double be = err_ < INFINITY ? err_ : INFINITY;
        int bl = err_ < INFINITY ? lane : 32;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, be, off);
            const int ol = __shfl_xor_sync(0xffffffffu, bl, off);
            if (ob < be || (ob == be && ol < bl)) { be = ob; bl = ol; }
        }
        if (bl < 32 && lane == bl) {
            const long c = cidx(m, i, j, k);
            nx[c] = cx; ny[c] = cy; nz[c] = cz;
        }
        if (cand && lane == 0) cand[cidx(m, i, j, k)] = (signed char)(bl < 32 ? bl : -1);
        __syncwarp();
    }
    if (err) atomicOr(errw, err);
}

/* ======================================================================================
 * computePLIC! on every cell; D(p) = computeDist at the border-copy source of p.
 * ==================================================================================== */
/* Pure cells get D = -/+(Lx+Ly+Lz) directly; cells whose border source holds an interface
 * VF go to a list so that the FP64 plane-constant solve runs in full warps.  A pure cell's
 * normal is an axis normal or zero (ELVIRA!, src/ELVIRA.jl:19-46; zero in non-periodic ghost
 * layers), so its phase code is +-1, and the plane (0, 0, 0, D) in its cell frame puts every
 * point of the domain on the same side as its own plane does: no normals are read and no FP64
 * arithmetic is done for the 97% of cells that are pure.  Threads map to (i, j) of a plane
 * and blocks to PLIC_PK planes in k, so no index divides. */
constexpr int PLIC_PK = 4; /* planes per thread */

__global__ void __launch_bounds__(256) k_plic_pure(DevMesh m, const double* __restrict__ VF, double* __restrict__ D,
                                                   float4* __restrict__ planes, signed char* __restrict__ phase,
                                                   int* list, int* count, float Lsum_f)
{
    /* the thresholds are tested on the bit patterns (integer pipe), the outputs are copies */
    const long long lob = dbits(m.VFlo), hib = dbits(m.VFhi);
    const int n0 = m.N[0] + 2 * m.g, n1 = m.N[1] + 2 * m.g, n2 = m.N[2] + 2 * m.g;
    const int a = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y * blockDim.y + threadIdx.y;
    const int c0 = blockIdx.z * PLIC_PK;
    const bool col = a < n0 && b < n1;
    const int ip = a + m.lo, jp = b + m.lo;
    const int i = ghost_src_1d(ip, m.N[0], m.g, m.per[0], false);
    const int j = ghost_src_1d(jp, m.N[1], m.g, m.per[1], false);
    /* every load of the thread's column first (VF of the border source and the stored code),
     * so they overlap */
    long long v[PLIC_PK];
    signed char old[PLIC_PK];
    long t[PLIC_PK];
#pragma unroll
    for (int q = 0; q < PLIC_PK; ++q) {
        const bool in = col && c0 + q < n2;
        t[q] = (long)a + (long)b * n0 + (long)(c0 + q) * n0 * n1;
        const int k = ghost_src_1d(c0 + q + m.lo, m.N[2], m.g, m.per[2], false);
        v[q] = in ? dbits(VF[vidx(m, i, j, k)]) : 0;
        old[q] = in ? phase[t[q]] : (signed char)0;
    }
    bool defer[PLIC_PK];
    int item[PLIC_PK];
#pragma unroll
    for (int q = 0; q < PLIC_PK; ++q) {
        const bool in = col && c0 + q < n2;
        const bool gas = bits_below(v[q], lob);
        const bool pure = in && (gas || bits_above(v[q], hib));
        defer[q] = in && !pure; /* interface (or NaN) source */
        item[q] = (int)t[q];
        /* a stored code of -1 or +1 comes with D = -/+Lsum and a plane with every point of
         * the domain on that side (written here or by plic_outputs; the buffers start at
         * code 0), so only cells whose code changes are written */
        const signed char want = gas ? -1 : 1;
        if (pure && old[q] != want) {
            D[t[q]] = gas ? -m.Lsum : m.Lsum;
            phase[t[q]] = want;
            if (planes) planes[t[q]] = make_float4(0.f, 0.f, 0.f, gas ? -Lsum_f : Lsum_f);
        }
    }
    __shared__ int s_app[8 * PLIC_PK + 1];
    block_append<PLIC_PK, 8>(defer, item, list, count, s_app); /* blocks of 32 x 8 */
}

/* computeDist (src/VF.jl:109-156) for the deferred cells: D(p) = computeDist at the border
 * source of p (computePLIC! then update_borders!, src/VF.jl:94-103). */
__global__ void k_plic_iface(DevMesh m, const double* __restrict__ VF, const double* __restrict__ nx,
                             const double* __restrict__ ny, const double* __restrict__ nz, double* __restrict__ D,
                             float4* __restrict__ planes, signed char* __restrict__ phase, const int* __restrict__ list,
                             const int* __restrict__ count)
{
    const long n0 = m.N[0] + 2 * m.g, n1 = m.N[1] + 2 * m.g;
    const int n = *count;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const long t = list[q];
        const int ip = (int)(t % n0) + m.lo, jp = (int)((t / n0) % n1) + m.lo, kp = (int)(t / (n0 * n1)) + m.lo;
        const int i = ghost_src_1d(ip, m.N[0], m.g, m.per[0], false);
        const int j = ghost_src_1d(jp, m.N[1], m.g, m.per[1], false);
        const int k = ghost_src_1d(kp, m.N[2], m.g, m.per[2], false);
        const long c = cidx(m, i, j, k);
        const double dist = compute_dist64(m, i, j, k, nx[c], ny[c], nz[c], VF[vidx(m, i, j, k)]);
        plic_outputs(m, t, ip, jp, kp, dist, nx, ny, nz, D, planes, phase);
    }
}

/* ======================================================================================
 * Pre-image tracing.  Face-velocity interpolation (get_velocity_{u,v,w}face,
 * src/Tools.jl:516-641): the interval search and weight of one coordinate against face or
 * centre positions are shared between the three components that use them.
 * ==================================================================================== */
struct Axis64 {
    int I;
    double w1;
};

__device__ __forceinline__ Axis64 search64(const DevMesh& m, int q, bool face, double p, int seed)
{
    const double* a = face ? m.f[q] : m.c[q];
    int i = seed;
    while (p - __ldg(a + (i - m.lo)) < 0.0 && i > m.lo) i = i - 1;
    while (p - __ldg(a + (i + 1 - m.lo)) >= 0.0 && i + 1 < m.hi[q]) i = i + 1;
    const double lo = __ldg(a + (i - m.lo)), hi = __ldg(a + (i + 1 - m.lo));
    return {i, sdiv(p - lo, hi - lo)};
}

__device__ __forceinline__ double trilinear64(const DevMesh& m, const double* __restrict__ f, Axis64 X, Axis64 Y,
                                              Axis64 Z)
{
    const double wx1 = X.w1, wx2 = 1.0 - X.w1, wy1 = Y.w1, wy2 = 1.0 - Y.w1, wz1 = Z.w1, wz2 = 1.0 - Z.w1;
    const long b = cidx(m, X.I, Y.I, Z.I);
    const long sj = m.cs1, sk = m.cs2;
    const double f000 = __ldg(f + b), f100 = __ldg(f + b + 1), f010 = __ldg(f + b + sj), f110 = __ldg(f + b + 1 + sj);
    const double f001 = __ldg(f + b + sk), f101 = __ldg(f + b + 1 + sk), f011 = __ldg(f + b + sj + sk),
                 f111 = __ldg(f + b + 1 + sj + sk);
    return wz1 * (wy1 * (wx1 * f111 + wx2 * f011) + wy2 * (wx1 * f101 + wx2 * f001)) +
           wz2 * (wy1 * (wx1 * f110 + wx2 * f010) + wy2 * (wx1 * f100 + wx2 * f000));
}

struct Vel64 {
    const double *uf, *vf, *wf;
};

__device__ __forceinline__ void velocity64(const DevMesh& m, const Vel64& V, double px, double py, double pz, int i,
                                           int j, int k, double& u, double& v, double& w)
{
    const Axis64 fx = search64(m, 0, true, px, i), cx = search64(m, 0, false, px, i);
    const Axis64 fy = search64(m, 1, true, py, j), cy = search64(m, 1, false, py, j);
    const Axis64 fz = search64(m, 2, true, pz, k), cz = search64(m, 2, false, pz, k);
    u = trilinear64(m, V.uf, fx, cy, cz);
    v = trilinear64(m, V.vf, cx, fy, cz);
    w = trilinear64(m, V.wf, cx, cy, fz);
}

/* project!, src/Tools.jl:392-418 */
__device__ __forceinline__ void project64(const DevMesh& m, const Vel64& V, double& px, double& py, double& pz, int i,
                                          int j, int k, double dt)
{
    if (m.projection == 3) {
        /* test_case == "Zalesak": exact rotation about (0.5, 0.5), src/Tools.jl:396-399 */
        const double a = 6.283185307179586 * dt;
        const double c = detm_cos(a), s = detm_sin(a);
        const double x0 = px, y0 = py;
        px = (0.5 + c * (x0 - 0.5)) + s * (y0 - 0.5);
        py = (0.5 - s * (x0 - 0.5)) + c * (y0 - 0.5);
        return;
    }
    double u1, v1, w1;
    velocity64(m, V, px, py, pz, i, j, k, u1, v1, w1);
    if (m.projection == 2) {
        double u2, v2, w2, u3, v3, w3, u4, v4, w4;
        velocity64(m, V, px - 0.5 * dt * u1, py - 0.5 * dt * v1, pz - 0.5 * dt * w1, i, j, k, u2, v2, w2);
        velocity64(m, V, px - 0.5 * dt * u2, py - 0.5 * dt * v2, pz - 0.5 * dt * w2, i, j, k, u3, v3, w3);
        velocity64(m, V, px - dt * u3, py - dt * v3, pz - dt * w3, i, j, k, u4, v4, w4);
        px = px + (-dt) / 6.0 * (((u1 + 2.0 * u2) + 2.0 * u3) + u4);
        py = py + (-dt) / 6.0 * (((v1 + 2.0 * v2) + 2.0 * v3) + v4);
        pz = pz + (-dt) / 6.0 * (((w1 + 2.0 * w2) + 2.0 * w3) + w4);
    } else if (m.projection == 0) {
        px = px + (-dt) * u1;
        py = py + (-dt) * v1;
        pz = pz + (-dt) * w1;
    } else {
        double u2, v2, w2;
        velocity64(m, V, px - 0.5 * dt * u1, py - 0.5 * dt * v1, pz - 0.5 * dt * w1, i, j, k, u2, v2, w2);
        px = px + (-dt) * u2;
        py = py + (-dt) * v2;
        pz = pz + (-dt) * w2;
    }
}

/* pt2index!, src/Tools.jl:424-434, with the index kept inside the coordinate arrays. */
__device__ __forceinline__ int pt2index1(const DevMesh& m, int q, double p, int I, int& err)
{
    while (p > fco(m, q, I + 1) + EPS64) {
        if (I >= m.hi[q]) { err |= ERR_INDEX; break; }
        I += 1;
    }
    while (p < fco(m, q, I) - EPS64) {
        if (I <= m.lo) { err |= ERR_INDEX; break; }
        I -= 1;
    }
    return I;
}

/* ======================================================================================
 * cutTet with an explicit stack.  Each frame is one recursion level of the reference: the
 * parent tet, the new vertices on the cutting mesh plane, their side-1 indices, the cut
 * case and the running (vol, vLiq) of its children, so partial sums are added in exactly
 * the reference's tree order.
 * ==================================================================================== */
/* One cutTet level: parent vertices 0-3, new vertices 4-7, their cells, the children's running
 * sums (vol, vLiq, and with MOM vrhoU, vrhoV, vrhoW, vrho) and the level's case, next child,
 * cut direction and index. */
template <bool MOM>
struct Frame64 {
    double x[8], y[8], z[8];
    double acc[MOM ? 6 : 2];
    short ind[8][3]; /* side-1 indices; side 2 differs only in the cut direction (= cut) */
    signed char cs, next, dir, flags;
    int cut;
};

struct Plic64 {
    const double *nx, *ny, *nz, *D;
    const double *u, *v, *w; /* cell-centred velocities for the momentum sums (MOM only) */
    double rho_liq, rho_gas;
};

/* Leaf: clip by the donor cell's PLIC plane (src/VFgeom.jl:757-830): r = (vol, vLiq) and with
 * MOM (vrhoU, vrhoV, vrhoW, vrho) with the donor's velocity and each side's density. */
template <bool MOM>
__device__ __forceinline__ void leaf64(const DevMesh& m, const CutCase* tab, const Plic64& P, const double* cx,
                                       const double* cy, const double* cz, int di, int dj, int dk, double* r, int& err)
{
    const long c = cidx(m, di, dj, dk);
    const double a = __ldg(P.nx + c), b = __ldg(P.ny + c), e = __ldg(P.nz + c), Dd = __ldg(P.D + c);
    double d[4], vx[8], vy[8], vz[8];
    for (int n = 0; n < 4; ++n) {
        d[n] = ((a * cx[n] + b * cy[n]) + e * cz[n]) - Dd;
        vx[n] = cx[n]; vy[n] = cy[n]; vz[n] = cz[n];
    }
    double c0 = d[0], c1 = d[1], c2 = d[2], c3 = d[3]; /* d2case works on a copy here */
    const int cs = d2case(c0, c1, c2, c3, EPS64, err);
    const CutCase& C = tab[cs];
    for (int n = 0; n < C.nvert; ++n) {
        const int v1 = C.v1[n], v2 = C.v2[n];
        const double mu = clamp_mu(sdiv(-d[v1], d[v2] - d[v1]));
        vx[4 + n] = (1.0 - mu) * vx[v1] + mu * vx[v2];
        vy[4 + n] = (1.0 - mu) * vy[v1] + mu * vy[v2];
        vz[4 + n] = (1.0 - mu) * vz[v1] + mu * vz[v2];
    }
    double vol = 0.0, liq = 0.0, ru = 0.0, rv = 0.0, rw = 0.0, rho = 0.0;
    double uc = 0.0, vc = 0.0, wc = 0.0;
    if (MOM) { uc = __ldg(P.u + c); vc = __ldg(P.v + c); wc = __ldg(P.w + c); }
    for (int n = C.ntets - 1; n >= C.nntet - 1; --n) {
        const int p = C.vtet[n][0], q = C.vtet[n][1], t = C.vtet[n][2], s = C.vtet[n][3];
        const double tv = tet_vol(vx[p], vy[p], vz[p], vx[q], vy[q], vz[q], vx[t], vy[t], vz[t], vx[s], vy[s], vz[s]);
        vol += tv;
        liq += tv;
        if (MOM) {
            ru += tv * uc * P.rho_liq;
            rv += tv * vc * P.rho_liq;
            rw += tv * wc * P.rho_liq;
            rho += tv * P.rho_liq;
        }
    }
    for (int n = 0; n < C.nntet - 1; ++n) {
        const int p = C.vtet[n][0], q = C.vtet[n][1], t = C.vtet[n][2], s = C.vtet[n][3];
        const double tv = tet_vol(vx[p], vy[p], vz[p], vx[q], vy[q], vz[q], vx[t], vy[t], vz[t], vx[s], vy[s], vz[s]);
        vol += tv;
        if (MOM) {
            ru += tv * uc * P.rho_gas;
            rv += tv * vc * P.rho_gas;
            rw += tv * wc * P.rho_gas;
            rho += tv * P.rho_gas;
        }
    }
    r[0] = vol;
    r[1] = liq;
    if (MOM) { r[2] = ru; r[3] = rv; r[4] = rw; r[5] = rho; }
}

template <bool MOM>
__device__ __forceinline__ void form_child64(const Frame64<MOM>& F, const CutCase* tab, int n, double* cx, double* cy,
                                             double* cz, int (*ci)[3])
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

/* cutTet (src/VFgeom.jl:713-900) with an explicit stack; the children's sums are added in the
 * reference's order.  out = (vol, vLiq[, vrhoU, vrhoV, vrhoW, vrho]).  The first SL64_SMEM_FRAMES
 * levels live in the calling thread's slot of shared memory (sm), which holds every tree at
 * CFL <= 1 (one cut per direction); deeper levels of larger CFL numbers use a local array. */
constexpr int SL64_SMEM_FRAMES = 3;

template <bool MOM>
__device__ void clip_tet64(const DevMesh& m, const CutCase* tab, const Plic64& P, double* cx, double* cy, double* cz,
                           int (*ci)[3], double* out, int& err, Frame64<MOM>* sm)
{
    constexpr int NA = MOM ? 6 : 2;
    Frame64<MOM> st_deep[CLIP_STACK - SL64_SMEM_FRAMES];
    auto frame = [&](int d) -> Frame64<MOM>& { return d < SL64_SMEM_FRAMES ? sm[d] : st_deep[d - SL64_SMEM_FRAMES]; };
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
        double r[NA];
        if (dir >= 0 && depth == CLIP_STACK) { err |= ERR_DEPTH; dir = -1; }
        if (dir < 0) {
            if (++leaves > CLIP_MAX_LEAVES) { /* bounded work even for clamped, far-away pre-images */
                err |= ERR_DEPTH;
                for (int q = 0; q < NA; ++q) out[q] = 0.0;
                return;
            }
            leaf64<MOM>(m, tab, P, cx, cy, cz, ci[0][0], ci[0][1], ci[0][2], r, err);
        } else {
            Frame64<MOM>& F = frame(depth);
            const double pl = fco(m, dir, cut);
            const double* cd = dir == 0 ? cx : (dir == 1 ? cy : cz);
            double d[4];
            for (int n = 0; n < 4; ++n) d[n] = cd[n] - pl;
            double c0 = d[0], c1 = d[1], c2 = d[2], c3 = d[3];
            const int cs = d2case(c0, c1, c2, c3, EPS64, err);
            for (int n = 0; n < 4; ++n) {
                F.x[n] = cx[n]; F.y[n] = cy[n]; F.z[n] = cz[n];
                F.ind[n][0] = (short)ci[n][0]; F.ind[n][1] = (short)ci[n][1]; F.ind[n][2] = (short)ci[n][2];
                F.ind[n][dir] = (short)min(ci[n][dir], cut - 1);
            }
            const CutCase& C = tab[cs];
            for (int n = 0; n < C.nvert; ++n) {
                const int v1 = C.v1[n], v2 = C.v2[n];
                const double mu = clamp_mu(sdiv(-d[v1], d[v2] - d[v1]));
                const double x = (1.0 - mu) * F.x[v1] + mu * F.x[v2];
                const double y = (1.0 - mu) * F.y[v1] + mu * F.y[v2];
                const double z = (1.0 - mu) * F.z[v1] + mu * F.z[v2];
                F.x[4 + n] = x; F.y[4 + n] = y; F.z[4 + n] = z;
                /* pt2index! seeded with vertex n's side-1 index (src/VFgeom.jl:854-857), then
                 * bounded by the edge end points (src/VFgeom.jl:859-862) */
                const int I0 = pt2index1(m, 0, x, F.ind[n][0], err);
                const int I1 = pt2index1(m, 1, y, F.ind[n][1], err);
                const int I2 = pt2index1(m, 2, z, F.ind[n][2], err);
                const int Iv[3] = {I0, I1, I2};
                for (int q = 0; q < 3; ++q) {
                    int val = max(Iv[q], min((int)F.ind[v1][q], (int)F.ind[v2][q]));
                    val = min(val, max((int)F.ind[v1][q], (int)F.ind[v2][q]));
                    F.ind[4 + n][q] = (short)val;
                }
                F.ind[4 + n][dir] = (short)(cut - 1);
            }
            F.cs = (signed char)cs; F.dir = (signed char)dir; F.cut = cut; F.flags = (signed char)flags;
            for (int q = 0; q < NA; ++q) F.acc[q] = 0.0;
            F.next = 1;
            ++depth;
            form_child64<MOM>(F, tab, 0, cx, cy, cz, ci);
            continue;
        }
        for (;;) {
            if (depth == 0) {
                for (int q = 0; q < NA; ++q) out[q] = r[q];
                return;
            }
            Frame64<MOM>& F = frame(depth - 1);
            for (int q = 0; q < NA; ++q) F.acc[q] += r[q];
            if (F.next < tab[F.cs].ntets) {
                form_child64<MOM>(F, tab, F.next, cx, cy, cz, ci);
                F.next += 1;
                flags = F.flags;
                break;
            }
            for (int q = 0; q < NA; ++q) r[q] = F.acc[q];
            --depth;
        }
    }
}

/* Pure-donor shortcut.  If every donor cell the pre-image can reach has phase code +1 (or
 * every one -1), every leaf of the clip is d2case case 1 (or 16), vLiq and vol are the same
 * sums (or vLiq is zero), and vLiq/vol is exactly 1 (or 0) whenever vol is positive. */
__device__ __forceinline__ int pure_phase(const DevMesh& m, const signed char* __restrict__ phase, int lo0, int hi0,
                                          int lo1, int hi1, int lo2, int hi2)
{
    if (hi0 - lo0 > 3 || hi1 - lo1 > 3 || hi2 - lo2 > 3) return 0;
    int ph = 2;
    for (int k = lo2; k <= hi2; ++k)
        for (int j = lo1; j <= hi1; ++j)
            for (int i = lo0; i <= hi0; ++i) {
                const int p = __ldg(phase + cidx(m, i, j, k));
                if (p == 0 || (ph != 2 && p != ph)) return 0;
                ph = p;
            }
    return ph;
}

constexpr int SL_THREADS = 128;

/* SL update of one band cell: cell2tets!(project_verts=true, compute_indices=true)
 * (src/VFgeom.jl:345-420), then cutTet on the cell's tets and VFnew = vLiq/vol
 * (src/Transport.jl:116-145).  For 24_tets the mean points come from the projected vertices
 * and their cells from pt2index! seeded at the cell, as verts2tets! does.  With MOM also
 * us, vs, ws = vrhoU/vrho, ... (src/Transport.jl:146-148). */
/* vertices of the flux volume of face `dir`: index offsets and projection flag, even and odd */
__constant__ signed char c_fluxv[3][2][8][4] = {
    {{{0, 0, 0, 1}, {0, 0, 0, 0}, {0, 1, 0, 1}, {0, 1, 0, 0}, {0, 0, 1, 1}, {0, 0, 1, 0}, {0, 1, 1, 1}, {0, 1, 1, 0}},
     {{0, 0, 0, 0}, {0, 0, 0, 1}, {0, 1, 0, 0}, {0, 1, 0, 1}, {0, 0, 1, 0}, {0, 0, 1, 1}, {0, 1, 1, 0}, {0, 1, 1, 1}}},
    {{{0, 0, 0, 1}, {1, 0, 0, 1}, {0, 0, 0, 0}, {1, 0, 0, 0}, {0, 0, 1, 1}, {1, 0, 1, 1}, {0, 0, 1, 0}, {1, 0, 1, 0}},
     {{1, 0, 0, 1}, {0, 0, 0, 1}, {1, 0, 0, 0}, {0, 0, 0, 0}, {1, 0, 1, 1}, {0, 0, 1, 1}, {1, 0, 1, 0}, {0, 0, 1, 0}}},
    {{{0, 0, 0, 1}, {1, 0, 0, 1}, {0, 1, 0, 1}, {1, 1, 0, 1}, {0, 0, 0, 0}, {1, 0, 0, 0}, {0, 1, 0, 0}, {1, 1, 0, 0}},
     {{1, 0, 0, 1}, {0, 0, 0, 1}, {1, 1, 0, 1}, {0, 1, 0, 1}, {1, 0, 0, 0}, {0, 0, 0, 0}, {1, 1, 0, 0}, {0, 1, 0, 0}}}};

/* SLfluxVol (src/VFgeom.jl:428-509): the flux volume's vertices (tessellation order, mean
 * points for 24_tets) and its signed volume. */
__device__ double flux_verts64(const DevMesh& m, const Vel64& V, int dir, int i, int j, int k, double dt,
                               double (*p)[3])
{
    const bool even = tess_even(m.tess, i, j, k);
    const double tetsign = even ? 1.0 : -1.0;
    for (int n = 0; n < 8; ++n) {
        const signed char* f = c_fluxv[dir][even ? 0 : 1][n];
        double x = fco(m, 0, i + f[0]), y = fco(m, 1, j + f[1]), z = fco(m, 2, k + f[2]);
        if (f[3]) project64(m, V, x, y, z, i, j, k, dt);
        p[n][0] = x; p[n][1] = y; p[n][2] = z;
    }
    tess_means<double>(m.tess, p);
    double vol = 0.0; /* tets_vol, src/VFgeom.jl:683-689 */
    for (int t = 0; t < tess_ntets(m.tess); ++t) {
        const int a = tess_tet(m.tess, t, 0), b = tess_tet(m.tess, t, 1), c = tess_tet(m.tess, t, 2),
                  e = tess_tet(m.tess, t, 3);
        vol += tet_vol(p[a][0], p[a][1], p[a][2], p[b][0], p[b][1], p[b][2], p[c][0], p[c][1], p[c][2], p[e][0],
                       p[e][1], p[e][2]);
    }
    return vol * tetsign;
}

__device__ double sl_flux_vol64(const DevMesh& m, const Vel64& V, int dir, int i, int j, int k, double dt)
{
    double p[15][3];
    return flux_verts64(m, V, dir, i, j, k, dt, p);
}

/* add_correction_tets (src/VFgeom.jl:514-664), pressure_scheme "finite-difference", 5_tets:
 * two tets (a,b,d,e), (b,c,d,e) on each face (x-, x+, y-, y+, z-, z+) over the quad a,b,c,d of
 * the face's SLfluxVol vertices, with the apex e at the quad's mean except for the face-normal
 * coordinate, which makes their volume the difference between the finite-difference flux
 * volume dt * area * face velocity and the SL one.  Both volumes are affine in e with gradient
 * (a x b + d x a + b x c + c x d)/6, so that coordinate moves by 6 (vol - V(mean)) / its
 * component. */
__device__ void correction_tet64(const DevMesh& m, const Vel64& V, int i, int j, int k, double dt, int f,
                                 double (*tet)[3])
{
    const int dir = f >> 2, up = (f >> 1) & 1, second = f & 1; /* f = 4 dir + 2 up + second tet */
    const int fi = i + (dir == 0 ? up : 0), fj = j + (dir == 1 ? up : 0), fk = k + (dir == 2 ? up : 0);
    double fv[15][3];
    const double flux_vol = flux_verts64(m, V, dir, fi, fj, fk, dt, fv);
    const long t = cidx(m, fi, fj, fk);
    const double divg_vol = dir == 0 ? ((dt * m.d[1]) * m.d[2]) * V.uf[t]
                                     : (dir == 1 ? ((dt * m.d[0]) * m.d[2]) * V.vf[t] : ((dt * m.d[0]) * m.d[1]) * V.wf[t]);
    const bool even = tess_even(m.tess, fi, fj, fk);
    const double vol = even ? (divg_vol - flux_vol) : -(divg_vol - flux_vol);
    int q[4];
    if (dir == 0) {
        if (even) { q[0] = 4; q[1] = 6; q[2] = 2; q[3] = 0; }
        else { q[0] = 7; q[1] = 5; q[2] = 1; q[3] = 3; }
    } else if (dir == 1) { q[0] = 1; q[1] = 5; q[2] = 4; q[3] = 0; }
    else { q[0] = 1; q[1] = 0; q[2] = 2; q[3] = 3; }
    const double *a = fv[q[0]], *b = fv[q[1]], *c = fv[q[2]], *d = fv[q[3]];
    double e[3];
    for (int p = 0; p < 3; ++p) e[p] = 0.25 * (((a[p] + b[p]) + c[p]) + d[p]);
    const double v0 = tet_vol(a[0], a[1], a[2], b[0], b[1], b[2], d[0], d[1], d[2], e[0], e[1], e[2]) +
                      tet_vol(b[0], b[1], b[2], c[0], c[1], c[2], d[0], d[1], d[2], e[0], e[1], e[2]);
    const int p1 = (dir + 1) % 3, p2 = (dir + 2) % 3;
    auto cr = [&](const double* u, const double* w) { return u[p1] * w[p2] - u[p2] * w[p1]; };
    const double N = ((cr(a, b) + cr(d, a)) + cr(b, c)) + cr(c, d);
    e[dir] += 6.0 * (vol - v0) / N;
    const double* v4[4] = {second ? b : a, second ? c : b, d, e};
    for (int n = 0; n < 4; ++n)
        for (int p = 0; p < 3; ++p) tet[n][p] = v4[n][p];
}

template <bool MOM>
__device__ __forceinline__ void sl_cell64(const DevMesh& m, const CutCase* tab, double dt,
                                          const signed char* __restrict__ phase, double* __restrict__ VFout,
                                          const Vel64& V, const Plic64& P, int L, double* us, double* vs, double* ws,
                                          int& err, Frame64<MOM>* sm)
{
    const int i = 1 + L % m.N[0];
    const int j = 1 + (L / m.N[0]) % m.N[1];
    const int k = 1 + L / (m.N[0] * m.N[1]);
    const int tess = m.tess;
    const bool even = tess_even(tess, i, j, k);
    const double tetsign = even ? 1.0 : -1.0;
    const double X[2] = {fco(m, 0, even ? i : i + 1), fco(m, 0, even ? i + 1 : i)};
    const double Y[2] = {fco(m, 1, j), fco(m, 1, j + 1)};
    const double Z[2] = {fco(m, 2, k), fco(m, 2, k + 1)};
    double p[15][3];
    int vi[15][3];
#pragma unroll 1
    for (int v = 0; v < 8; ++v) {
        double x = X[v & 1], y = Y[(v >> 1) & 1], z = Z[v >> 2];
        project64(m, V, x, y, z, i, j, k, dt);
        p[v][0] = x; p[v][1] = y; p[v][2] = z;
    }
    tess_means<double>(tess, p);
    const int np = tess_npoints(tess), nt = tess_ntets(tess);
#pragma unroll 1
    for (int v = 0; v < np; ++v) {
        vi[v][0] = pt2index1(m, 0, p[v][0], i, err);
        vi[v][1] = pt2index1(m, 1, p[v][1], j, err);
        vi[v][2] = pt2index1(m, 2, p[v][2], k, err);
    }
    const long out = vidx(m, i, j, k);
    /* pure-donor shortcut (VF only: the momentum sums depend on each donor's share) */
    if (!MOM && m.fast_pure && !m.fd) {
        int lo0 = vi[0][0], hi0 = vi[0][0], lo1 = vi[0][1], hi1 = vi[0][1], lo2 = vi[0][2], hi2 = vi[0][2];
        for (int v = 1; v < np; ++v) {
            lo0 = min(lo0, vi[v][0]); hi0 = max(hi0, vi[v][0]);
            lo1 = min(lo1, vi[v][1]); hi1 = max(hi1, vi[v][1]);
            lo2 = min(lo2, vi[v][2]); hi2 = max(hi2, vi[v][2]);
        }
        const int ph = pure_phase(m, phase, lo0, hi0, lo1, hi1, lo2, hi2);
        if (ph != 0) {
            double vol = 0.0;
            for (int t = 0; t < nt; ++t) {
                const int a = tess_tet(tess, t, 0), b = tess_tet(tess, t, 1), c = tess_tet(tess, t, 2),
                          e = tess_tet(tess, t, 3);
                vol += tetsign * tet_vol(p[a][0], p[a][1], p[a][2], p[b][0], p[b][1], p[b][2], p[c][0], p[c][1],
                                         p[c][2], p[e][0], p[e][1], p[e][2]);
            }
            if (vol > 0.25 * m.cellvol && vol < 4.0 * m.cellvol) {
                VFout[out] = ph > 0 ? 1.0 : 0.0;
                return;
            }
        }
    }
    constexpr int NA = MOM ? 6 : 2;
    double sum[NA];
    for (int q = 0; q < NA; ++q) sum[q] = 0.0;
#pragma unroll 1
    for (int t = 0; t < nt; ++t) {
        double cx[4], cy[4], cz[4];
        int ci[4][3];
        for (int n = 0; n < 4; ++n) {
            const int v = tess_tet(tess, t, n);
            cx[n] = p[v][0]; cy[n] = p[v][1]; cz[n] = p[v][2];
            ci[n][0] = vi[v][0]; ci[n][1] = vi[v][1]; ci[n][2] = vi[v][2];
        }
        double r[NA];
        clip_tet64<MOM>(m, tab, P, cx, cy, cz, ci, r, err, sm);
        for (int q = 0; q < NA; ++q) sum[q] += tetsign * r[q];
    }
    if (m.fd) {
        /* pressure_scheme "finite-difference": the flux-correction tets, their vertices' cells
         * by pt2index! seeded at the cell (src/Transport.jl:121-124, src/VFgeom.jl:654-661) */
#pragma unroll 1
        for (int f = 0; f < 12; ++f) {
            double tet[4][3], cx[4], cy[4], cz[4];
            int ci[4][3];
            correction_tet64(m, V, i, j, k, dt, f, tet);
            for (int n = 0; n < 4; ++n) {
                cx[n] = tet[n][0]; cy[n] = tet[n][1]; cz[n] = tet[n][2];
                ci[n][0] = pt2index1(m, 0, cx[n], i, err);
                ci[n][1] = pt2index1(m, 1, cy[n], j, err);
                ci[n][2] = pt2index1(m, 2, cz[n], k, err);
            }
            double r[NA];
            clip_tet64<MOM>(m, tab, P, cx, cy, cz, ci, r, err, sm);
            for (int q = 0; q < NA; ++q) sum[q] += tetsign * r[q];
        }
    }
    if (!(sum[0] > 0.0) || !isfinite(sum[0])) err |= ERR_VOLUME;
    VFout[out] = sum[1] / sum[0];
    if (MOM) {
        const long c = cidx(m, i, j, k);
        us[c] = sum[2] / sum[5];
        vs[c] = sum[3] / sum[5];
        ws[c] = sum[4] / sum[5];
    }
}

template <bool MOM>
__global__ void __launch_bounds__(SL_THREADS) k_sl64(DevMesh m, double dt, const signed char* __restrict__ phase,
                                                     double* __restrict__ VFout, Vel64 V, Plic64 P,
                                                     const int* __restrict__ list, const int* __restrict__ count,
                                                     int* work, double* us, double* vs, double* ws, int* errw)
{
    __shared__ CutCase s_tab[16];
    extern __shared__ __align__(16) unsigned char sl64_smem[];
    Frame64<MOM>* sm = reinterpret_cast<Frame64<MOM>*>(sl64_smem) + threadIdx.x * SL64_SMEM_FRAMES;
    load_table(s_tab);
    const int lane = threadIdx.x & 31;
    const int n_items = *count;
    int err = 0;
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(work, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n_items) break;
        const int item = base + lane;
        if (item < n_items) sl_cell64<MOM>(m, s_tab, dt, phase, VFout, V, P, list[item], us, vs, ws, err, sm);
        __syncwarp();
    }
    if (err) atomicOr(errw, err);
}

/* ======================================================================================
 * Momentum of the cells outside the band (src/Transport.jl:34-104,150-166, pressure_scheme
 * "semi-lagrangian"): us = u + dt/(dx dy dz) * sum of face-flux differences.  A face between
 * two band cells carries no flux, a face with one band cell the semi-Lagrangian flux volume
 * (SLfluxVol, src/VFgeom.jl:428-509), every other face the finite-difference flux.
 * ==================================================================================== */
__device__ void face_flux64(const DevMesh& m, const Vel64& V, const Plic64& P, const short* __restrict__ band, int dir,
                            int i, int j, int k, double dt, double* F)
{
    const int li = i - (dir == 0), lj = j - (dir == 1), lk = k - (dir == 2);
    const long c = cidx(m, i, j, k), l = cidx(m, li, lj, lk);
    const double uface = 0.5 * (__ldg(P.u + l) + __ldg(P.u + c));
    const double vface = 0.5 * (__ldg(P.v + l) + __ldg(P.v + c));
    const double wface = 0.5 * (__ldg(P.w + l) + __ldg(P.w + c));
    const bool bl = abs((int)band[l]) <= m.nband, bc = abs((int)band[c]) <= m.nband;
    if (bl && bc) {
        F[0] = 0.0; F[1] = 0.0; F[2] = 0.0;
    } else if ((bl || bc) && !m.fd) {
        const double vol = sl_flux_vol64(m, V, dir, i, j, k, dt) / dt;
        F[0] = -uface * vol; F[1] = -vface * vol; F[2] = -wface * vol;
    } else {
        const double a = dir == 0 ? m.d[1] : m.d[0], b = dir == 2 ? m.d[1] : m.d[2];
        const double q = __ldg((dir == 0 ? V.uf : (dir == 1 ? V.vf : V.wf)) + c);
        F[0] = -uface * a * b * q; F[1] = -vface * a * b * q; F[2] = -wface * a * b * q;
    }
}

__global__ void k_mom_flux64(DevMesh m, double dt, Vel64 V, Plic64 P, const short* __restrict__ band,
                             double* __restrict__ us, double* __restrict__ vs, double* __restrict__ ws)
{
    const long total = (long)m.N[0] * m.N[1] * m.N[2];
    const double f = dt / m.cellvol;
    for (long L = (long)blockIdx.x * blockDim.x + threadIdx.x; L < total; L += (long)gridDim.x * blockDim.x) {
        const int i = 1 + (int)(L % m.N[0]), j = 1 + (int)((L / m.N[0]) % m.N[1]), k = 1 + (int)(L / ((long)m.N[0] * m.N[1]));
        const long c = cidx(m, i, j, k);
        if (abs((int)band[c]) <= m.nband) continue; /* band cell: written by the SL update */
        double Fx0[3], Fx1[3], Fy0[3], Fy1[3], Fz0[3], Fz1[3];
        face_flux64(m, V, P, band, 0, i, j, k, dt, Fx0);
        face_flux64(m, V, P, band, 0, i + 1, j, k, dt, Fx1);
        face_flux64(m, V, P, band, 1, i, j, k, dt, Fy0);
        face_flux64(m, V, P, band, 1, i, j + 1, k, dt, Fy1);
        face_flux64(m, V, P, band, 2, i, j, k, dt, Fz0);
        face_flux64(m, V, P, band, 2, i, j, k + 1, dt, Fz1);
        us[c] = __ldg(P.u + c) + f * (((((Fx1[0] - Fx0[0]) + Fy1[0]) - Fy0[0]) + Fz1[0]) - Fz0[0]);
        vs[c] = __ldg(P.v + c) + f * (((((Fx1[1] - Fx0[1]) + Fy1[1]) - Fy0[1]) + Fz1[1]) - Fz0[1]);
        ws[c] = __ldg(P.w + c) + f * (((((Fx1[2] - Fx0[2]) + Fy1[2]) - Fy0[2]) + Fz1[2]) - Fz0[2]);
    }
}

/* ======================================================================================
 * divg_cell / divergence! (src/Velocity.jl:59-122) and A! (src/Pressure.jl:83-115), FP64 in
 * the reference's operation order.  sl: pressure_scheme == "semi-lagrangian".  A band cell's
 * divergence is (v2 - v1)/v2/dt with v1 the volume of its projected cell; any other cell sums
 * face fluxes: SLfluxVol/dt through a face whose neighbour is a band cell, the
 * finite-difference flux otherwise.
 * ==================================================================================== */
__device__ double divg_cell64(const DevMesh& m, const Vel64& V, const short* __restrict__ band, bool sl, int i, int j,
                              int k, double dt)
{
    auto inband = [&](int a, int b, int c) { return sl && abs((int)__ldg(band + cidx(m, a, b, c))) <= m.nband; };
    if (inband(i, j, k)) {
        const int tess = m.tess;
        const bool even = tess_even(tess, i, j, k);
        const double tetsign = even ? 1.0 : -1.0;
        const double X[2] = {fco(m, 0, even ? i : i + 1), fco(m, 0, even ? i + 1 : i)};
        const double Y[2] = {fco(m, 1, j), fco(m, 1, j + 1)};
        const double Z[2] = {fco(m, 2, k), fco(m, 2, k + 1)};
        double p[15][3];
#pragma unroll 1
        for (int v = 0; v < 8; ++v) {
            double x = X[v & 1], y = Y[(v >> 1) & 1], z = Z[v >> 2];
            project64(m, V, x, y, z, i, j, k, dt);
            p[v][0] = x; p[v][1] = y; p[v][2] = z;
        }
        tess_means<double>(tess, p);
        double vol = 0.0; /* tets_vol, src/VFgeom.jl:683-689 */
        for (int t = 0; t < tess_ntets(tess); ++t) {
            const int a = tess_tet(tess, t, 0), b = tess_tet(tess, t, 1), c = tess_tet(tess, t, 2),
                      e = tess_tet(tess, t, 3);
            vol += tet_vol(p[a][0], p[a][1], p[a][2], p[b][0], p[b][1], p[b][2], p[c][0], p[c][1], p[c][2], p[e][0],
                           p[e][1], p[e][2]);
        }
        const double v2 = m.cellvol, v1 = tetsign * vol;
        return (v2 - v1) / v2 / dt;
    }
    auto flux = [&](int dir, int a, int b, int c, int na, int nb, int nc) {
        if (inband(na, nb, nc)) return sl_flux_vol64(m, V, dir, a, b, c, dt) / dt;
        const long t = cidx(m, a, b, c);
        if (dir == 0) return (m.d[1] * m.d[2]) * __ldg(V.uf + t);
        if (dir == 1) return (m.d[0] * m.d[2]) * __ldg(V.vf + t);
        return (m.d[0] * m.d[1]) * __ldg(V.wf + t);
    };
    const double Fxm = flux(0, i, j, k, i - 1, j, k), Fxp = flux(0, i + 1, j, k, i + 1, j, k);
    const double Fym = flux(1, i, j, k, i, j - 1, k), Fyp = flux(1, i, j + 1, k, i, j + 1, k);
    const double Fzm = flux(2, i, j, k, i, j, k - 1), Fzp = flux(2, i, j, k + 1, i, j, k + 1);
    return (((((Fxp - Fxm) + Fyp) - Fym) + Fzp) - Fzm) / m.cellvol;
}

__global__ void k_divg64(DevMesh m, double dt, Vel64 V, const short* __restrict__ band, int sl,
                         double* __restrict__ divg)
{
    const long total = (long)m.N[0] * m.N[1] * m.N[2];
    for (long L = (long)blockIdx.x * blockDim.x + threadIdx.x; L < total; L += (long)gridDim.x * blockDim.x) {
        const int i = 1 + (int)(L % m.N[0]), j = 1 + (int)((L / m.N[0]) % m.N[1]), k = 1 + (int)(L / ((long)m.N[0] * m.N[1]));
        divg[cidx(m, i, j, k)] = divg_cell64(m, V, band, sl != 0, i, j, k, dt);
    }
}

/* Neumann! + update_borders! of a cell array in place: every ghost takes its separable source
 * (sources are fixed points of the map, so no copy reads a written cell). */
__global__ void k_cell_ghost64(DevMesh m, double* A)
{
    const int n0 = m.N[0] + 2 * m.g, n1 = m.N[1] + 2 * m.g, n2 = m.N[2] + 2 * m.g;
    const long total = (long)n0 * n1 * n2;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int ip = (int)(t % n0) + m.lo, jp = (int)((t / n0) % n1) + m.lo, kp = (int)(t / ((long)n0 * n1)) + m.lo;
        const int si = ghost_src_1d(ip, m.N[0], m.g, m.per[0], true);
        const int sj = ghost_src_1d(jp, m.N[1], m.g, m.per[1], true);
        const int sk = ghost_src_1d(kp, m.N[2], m.g, m.per[2], true);
        if (si != ip || sj != jp || sk != kp) A[t] = A[cidx(m, si, sj, sk)];
    }
}

/* A!'s pressure-corrected face velocities over the reference's ranges (src/Pressure.jl:
 * 92-105), 0 elsewhere: gradx with plain divides, grady and gradz with the safe divide. */
__global__ void k_pgrad64(DevMesh m, double dt, const double* __restrict__ P, const double* __restrict__ uf,
                          const double* __restrict__ vf, const double* __restrict__ wf,
                          const double* __restrict__ denx, const double* __restrict__ deny,
                          const double* __restrict__ denz, double* __restrict__ gx, double* __restrict__ gy,
                          double* __restrict__ gz)
{
    const int n0 = m.N[0] + 2 * m.g, n1 = m.N[1] + 2 * m.g, n2 = m.N[2] + 2 * m.g;
    const long total = (long)n0 * n1 * n2;
    const long sj = m.cs1, sk = m.cs2;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int ii = (int)(t % n0) + m.lo, jj = (int)((t / n0) % n1) + m.lo, kk = (int)(t / ((long)n0 * n1)) + m.lo;
        const bool in0 = ii >= 0 && ii <= m.N[0] + 1, in1 = jj >= 0 && jj <= m.N[1] + 1, in2 = kk >= 0 && kk <= m.N[2] + 1;
        const bool x0 = ii >= 0 && ii <= m.N[0] + 2, y0 = jj >= 0 && jj <= m.N[1] + 2, z0 = kk >= 0 && kk <= m.N[2] + 2;
        gx[t] = (x0 && in1 && in2) ? uf[t] - dt / denx[t] * (P[t] - P[t - 1]) / m.d[0] : 0.0;
        gy[t] = (in0 && y0 && in2) ? vf[t] - sdiv(sdiv(dt, deny[t]) * (P[t] - P[t - sj]), m.d[1]) : 0.0;
        gz[t] = (in0 && in1 && z0) ? wf[t] - sdiv(sdiv(dt, denz[t]) * (P[t] - P[t - sk]), m.d[2]) : 0.0;
    }
}

void launch_divergence64(const DevMesh& m, double dt, int sl, const double* uf, const double* vf, const double* wf,
                         const short* band, double* divg, int nsm, cudaStream_t s)
{
    const long nc = (long)(m.N[0] + 2 * m.g) * (m.N[1] + 2 * m.g) * (m.N[2] + 2 * m.g);
    cudaMemsetAsync(divg, 0, nc * sizeof(double), s);
    Vel64 V{uf, vf, wf};
    k_divg64<<<nsm * 8, 128, 0, s>>>(m, dt, V, band, sl, divg);
}

void launch_pressure_A64(const DevMesh& m, double dt, int sl, double* LHS, double* P, const double* uf,
                         const double* vf, const double* wf, const double* denx, const double* deny,
                         const double* denz, const short* band, double* gx, double* gy, double* gz, int nsm,
                         cudaStream_t s)
{
    k_cell_ghost64<<<nsm * 8, 256, 0, s>>>(m, P);
    k_pgrad64<<<nsm * 8, 256, 0, s>>>(m, dt, P, uf, vf, wf, denx, deny, denz, gx, gy, gz);
    launch_divergence64(m, dt, sl, gx, gy, gz, band, LHS, nsm, s);
}

/* Phase codes (and mixed-path planes) of planes that were uploaded rather than computed:
 * the same outputs as the PLIC pass derives from its own D. */
__global__ void k_plic_phase(DevMesh m, const double* __restrict__ nx, const double* __restrict__ ny,
                             const double* __restrict__ nz, double* D, float4* __restrict__ planes,
                             signed char* __restrict__ phase)
{
    const int n0 = m.N[0] + 2 * m.g, n1 = m.N[1] + 2 * m.g, n2 = m.N[2] + 2 * m.g;
    const long total = (long)n0 * n1 * n2;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int ip = (int)(t % n0) + m.lo, jp = (int)((t / n0) % n1) + m.lo, kp = (int)(t / ((long)n0 * n1)) + m.lo;
        plic_outputs(m, t, ip, jp, kp, D[t], nx, ny, nz, D, planes, phase);
    }
}

void launch_plic_phase(const DevMesh& m, const double* nx, const double* ny, const double* nz, double* D,
                       float4* planes, signed char* phase, int nsm, cudaStream_t s)
{
    k_plic_phase<<<nsm * 8, 256, 0, s>>>(m, nx, ny, nz, D, planes, phase);
}

/* ---- launchers ------------------------------------------------------------------------ */
void launch_elvira_iface64(const DevMesh& m, const double* VF, double* nx, double* ny, double* nz, const int* list,
                           const int* count, int* work, signed char* cand, int* errw, int nsm, cudaStream_t s)
{
    k_elvira_iface64<<<nsm * 8, EL_WARPS * 32, 0, s>>>(m, VF, nx, ny, nz, list, count, work, cand, errw);
}

void launch_plic64(const DevMesh& m, const double* VF, const double* nx, const double* ny, const double* nz, double* D,
                   float4* planes, signed char* phase, int* list, int* count, bool newton_root, int nsm, cudaStream_t s)
{
    const dim3 grid((m.N[0] + 2 * m.g + 31) / 32, (m.N[1] + 2 * m.g + 7) / 8,
                    (m.N[2] + 2 * m.g + PLIC_PK - 1) / PLIC_PK);
    k_plic_pure<<<grid, dim3(32, 8), 0, s>>>(m, VF, D, planes, phase, list, count, (float)m.Lsum);
    if (newton_root)
        launch_plic_iface_newton(m, VF, nx, ny, nz, D, planes, phase, list, count, nsm, s);
    else
        k_plic_iface<<<nsm * 4, 128, 0, s>>>(m, VF, nx, ny, nz, D, planes, phase, list, count);
}

void launch_sl64(const DevMesh& m, double dt, const double* VFin, double* VFout, const double* uf, const double* vf,
                 const double* wf, const double* nx, const double* ny, const double* nz, const double* D,
                 const signed char* phase, const int* list, const int* count, int* work, int* errw, int nsm,
                 cudaStream_t s)
{
    (void)VFin;
    Vel64 V{uf, vf, wf};
    Plic64 P{nx, ny, nz, D, nullptr, nullptr, nullptr, 0.0, 0.0};
    /* the clip frames' shared-memory share: 3 frames x 128 threads (101 KB, two blocks per SM);
     * the grid holds as many blocks as fit at once, which fetch their cells from the list */
    const int smem = SL_THREADS * SL64_SMEM_FRAMES * (int)sizeof(Frame64<false>);
    cudaFuncSetAttribute(k_sl64<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sl64<false>, SL_THREADS, smem);
    k_sl64<false><<<nsm * max(per_sm, 1), SL_THREADS, smem, s>>>(m, dt, phase, VFout, V, P, list, count, work,
                                                                 nullptr, nullptr, nullptr, errw);
}

void launch_sl64_momentum(const DevMesh& m, double dt, double* VFout, const double* uf, const double* vf,
                          const double* wf, const double* nx, const double* ny, const double* nz, const double* D,
                          const signed char* phase, const short* band, const double* u, const double* v,
                          const double* w, double rho_liq, double rho_gas, double* us, double* vs, double* ws,
                          const int* list, const int* count, int* work, int* errw, int nsm, cudaStream_t s)
{
    Vel64 V{uf, vf, wf};
    Plic64 P{nx, ny, nz, D, u, v, w, rho_liq, rho_gas};
    const int smem = SL_THREADS * SL64_SMEM_FRAMES * (int)sizeof(Frame64<true>);
    cudaFuncSetAttribute(k_sl64<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sl64<true>, SL_THREADS, smem);
    k_sl64<true><<<nsm * max(per_sm, 1), SL_THREADS, smem, s>>>(m, dt, phase, VFout, V, P, list, count, work, us, vs,
                                                                ws, errw);
    k_mom_flux64<<<nsm * 8, 128, 0, s>>>(m, dt, V, P, band, us, vs, ws);
}

} // namespace slvof
