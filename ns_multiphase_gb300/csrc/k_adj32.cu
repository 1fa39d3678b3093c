/*
 * k_adj32.cu — reverse pass of one mixed-precision SL-VOF step: FP32 geometry in the mixed
 * path's cell frame, FP64 accumulation (atomics) of every derivative that leaves a cell.
 *
 * The derivatives of the clipped volumes come from the pre-image's boundary (adj32.cuh): the
 * liquid moments of its boundary triangles for the vertices, the PLIC polygons inside each tet
 * and donor cell for the planes, the plane polygon inside the cell for computeDist.  Nothing
 * walks the clip tree backwards, so there is no stack and no recursion here.  The kernels, in
 * the order the reverse runs (after the VF fold and the pass-through of cells outside the
 * band, k_adj64.cu):
 *
 *   k_adj32_cell    thread per clipped band cell (the forward's clip list): pre-image volume,
 *                   the cell's seed g * tetsign / vol and VFnew;
 *   k_adj32_faces   thread per (cell, boundary triangle): d(VFnew)/d(vertices), added to the
 *                   grid vertex each pre-image vertex was traced from (corners shared by up to
 *                   eight cells are traced once in the reverse);
 *   k_adj32_planes  thread per (cell, tet): d(VFnew)/d(n, D) of every donor whose plane cuts
 *                   the tet inside the donor cell;
 *   k_adj32_vert    thread per grid vertex: the RK trajectory again and its reverse to the
 *                   face velocities (project!, src/Tools.jl:392-418; get_velocity_*face,
 *                   src/Tools.jl:500-641);
 *   k_adj32_dist    thread per cell (ghosts included): computeDist backwards to VF and n.
 *
 * Cells that k_sl32_pre finishes (pre-image strictly on one side of every donor plane, VF = 1
 * or 0) have zero derivative and are not in the clip list.
 */
#include "slvof_kernels.h"
#include "slvof_dev.cuh"
#include "mixed32.cuh"
#include "adj32.cuh"

namespace slvof {

namespace {

constexpr int ADJ32_THREADS = 128;

__device__ __forceinline__ float tet_vol4(const float (&tv)[4][3])
{
    return tet_vol<float>(tv[0][0], tv[0][1], tv[0][2], tv[1][0], tv[1][1], tv[1][2], tv[2][0], tv[2][1], tv[2][2],
                          tv[3][0], tv[3][1], tv[3][2]);
}

/* tet t of clip cell s: vertices (cell units) and donor indices relative to the cell */
__device__ __forceinline__ void load_tet(const DevMesh& m, const float4* __restrict__ verts, long s, int t,
                                         float (&tv)[4][3], int (&ind)[4][3], int (&ids)[4])
{
    const int stride = m.tess == 24 ? 16 : 8;
#pragma unroll
    for (int n = 0; n < 4; ++n) {
        ids[n] = tess_tet(m.tess, t, n);
        const float4 p = __ldg(verts + s * stride + ids[n]);
        tv[n][0] = p.x; tv[n][1] = p.y; tv[n][2] = p.z;
        const unsigned pk = (unsigned)__float_as_int(p.w);
        ind[n][0] = unpack(pk, 0); ind[n][1] = unpack(pk, 1); ind[n][2] = unpack(pk, 2);
    }
}

__global__ void __launch_bounds__(ADJ32_THREADS) k_adj32_cell(DevMesh m, const int* __restrict__ cells,
                                                              const float4* __restrict__ verts,
                                                              const int* __restrict__ count,
                                                              const double* __restrict__ gfold,
                                                              const double* __restrict__ VFnext, float2* cinfo,
                                                              int* errw)
{
    const int n = *count, nt = tess_ntets(m.tess);
    int err = 0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        int i, j, k;
        cell_of(m, cells[s], i, j, k);
        const long v = vidx(m, i, j, k);
        const double g = gfold[v];
        const float tetsign = tess_even(m.tess, i, j, k) ? 1.f : -1.f;
        float vol = 0.f;
        for (int t = 0; t < nt; ++t) {
            float tv[4][3];
            int ind[4][3], ids[4];
            load_tet(m, verts, s, t, tv, ind, ids);
            vol += tetsign * tet_vol4(tv);
        }
        float coef = 0.f;
        if (!(vol > 0.f) || !isfinite(vol)) err |= ERR_VOLUME;
        else if (g != 0.0) coef = (float)g * tetsign / vol;
        cinfo[s] = make_float2(coef, (float)VFnext[v]);
    }
    if (err) atomicOr(errw, err);
}

/* add val to the derivative of pre-image point id of cell (i, j, k): a corner goes to the grid
 * vertex it was traced from, a mean point (24_tets) to the corners it averages */
__device__ __forceinline__ void scatter_point(const DevMesh& m, int i, int j, int k, bool even, int id,
                                              const float (&val)[3], double* gx, double* gy, double* gz)
{
    auto corner = [&](int v, float w) {
        const int xo = even ? (v & 1) : 1 - (v & 1);
        const long t = cidx(m, i + xo, j + ((v >> 1) & 1), k + (v >> 2));
        atomicAdd(gx + t, (double)(w * val[0]));
        atomicAdd(gy + t, (double)(w * val[1]));
        atomicAdd(gz + t, (double)(w * val[2]));
    };
    if (id < 8) {
        corner(id, 1.f);
    } else if (id == 8) {
        for (int v = 0; v < 8; ++v) corner(v, 0.125f);
    } else {
        for (int n = 0; n < 4; ++n) corner(face24(id - 9, n), 0.25f);
    }
}

constexpr int FACES_THREADS = 64; /* 7 polygons of workspace per thread in shared memory: 37.6 KB a block */
constexpr int PLANES_THREADS = 128; /* 2 polygons per thread: 31.7 KB a block */

__global__ void __launch_bounds__(FACES_THREADS) k_adj32_faces(DevMesh m, const float4* __restrict__ planes,
                                                               const signed char* __restrict__ phase,
                                                               const int* __restrict__ cells,
                                                               const float4* __restrict__ verts,
                                                               const float2* __restrict__ cinfo,
                                                               const int* __restrict__ count, sd::BFaces F,
                                                               double* gx, double* gy, double* gz)
{
    /* the polygon workspace lives in shared memory: in local memory it spilled to DRAM */
    __shared__ sd::Poly2<float> s_ws[FACES_THREADS * 7];
    sd::Poly2<float>* ws = s_ws + threadIdx.x * 7;
    const long n = (long)F.n * *count;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const long s = q / F.n;
        const int f = (int)(q % F.n);
        const float2 ci = cinfo[s];
        if (ci.x == 0.f) continue;
        int i, j, k;
        cell_of(m, cells[s], i, j, k);
        const int t = F.t[f], b = F.b[f];
        float tv[4][3], S[3];
        int ind[4][3], ids[4];
        load_tet(m, verts, s, t, tv, ind, ids);
        sd::face_area(tv, b, S);
        float p3[3][3], mm[3];
        int i3[3][3], fid[3], nf = 0;
#pragma unroll
        for (int sl = 0; sl < 4; ++sl) {
            if (sl == b) continue;
            fid[nf] = ids[sl];
            for (int p = 0; p < 3; ++p) { p3[nf][p] = tv[sl][p]; i3[nf][p] = ind[sl][p]; }
            ++nf;
        }
        auto donor = [&](int a, int bb, int c, int& ph, float& px, float& py, float& pz, float& Dt) {
            const long d = cidx(m, i + a, j + bb, k + c);
            ph = __ldg(phase + d);
            px = py = pz = Dt = 0.f;
            if (ph != 0) return;
            const float4 pl = __ldg(planes + d);
            px = pl.x; py = pl.y; pz = pl.z;
            Dt = pl.w + pl.x * (float)a + pl.y * (float)bb + pl.z * (float)c;
        };
        sd::face_moments(p3, i3, donor, mm, ws);
        const bool even = tess_even(m.tess, i, j, k);
        const float third = ci.y * (1.f / 3.f);
        for (int sl = 0; sl < 3; ++sl) {
            const float w = ci.x * (mm[sl] - third);
            if (w == 0.f) continue;
            const float val[3] = {w * S[0], w * S[1], w * S[2]};
            scatter_point(m, i, j, k, even, fid[sl], val, gx, gy, gz);
        }
    }
}

__global__ void __launch_bounds__(PLANES_THREADS) k_adj32_planes(DevMesh m, const float4* __restrict__ planes,
                                                                const signed char* __restrict__ phase,
                                                                const int* __restrict__ cells,
                                                                const float4* __restrict__ verts,
                                                                const float2* __restrict__ cinfo,
                                                                const int* __restrict__ count, double* gnx,
                                                                double* gny, double* gnz, double* gD)
{
    __shared__ sd::Poly3<float> s_ws[PLANES_THREADS * 2];
    sd::Poly3<float>* ws = s_ws + threadIdx.x * 2;
    const int nt = tess_ntets(m.tess);
    const long n = (long)nt * *count;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const long s = q / nt;
        const int t = (int)(q % nt);
        const float2 ci = cinfo[s];
        if (ci.x == 0.f) continue;
        int i, j, k;
        cell_of(m, cells[s], i, j, k);
        float tv[4][3];
        int ind[4][3], ids[4];
        load_tet(m, verts, s, t, tv, ind, ids);
        const float V = tet_vol4(tv);
        if (V == 0.f) continue;
        const float cs = V > 0.f ? ci.x : -ci.x;
        int lo[3], hi[3];
        for (int p = 0; p < 3; ++p) {
            lo[p] = min(min(ind[0][p], ind[1][p]), min(ind[2][p], ind[3][p]));
            hi[p] = max(max(ind[0][p], ind[1][p]), max(ind[2][p], ind[3][p]));
        }
        const double o[3] = {fco(m, 0, i), fco(m, 1, j), fco(m, 2, k)};
        for (int c = lo[2]; c <= hi[2]; ++c)
            for (int b = lo[1]; b <= hi[1]; ++b)
                for (int a = lo[0]; a <= hi[0]; ++a) {
                    const long d = cidx(m, i + a, j + b, k + c);
                    if (__ldg(phase + d) != 0) continue;
                    const float4 pl = __ldg(planes + d);
                    const float Dt = pl.w + pl.x * (float)a + pl.y * (float)b + pl.z * (float)c;
                    float A, C[3];
                    if (!sd::plane_piece(tv, lo, hi, a, b, c, pl.x, pl.y, pl.z, Dt, A, C, ws)) continue;
                    const float len = sqrtf(pl.x * pl.x + pl.y * pl.y + pl.z * pl.z);
                    const double c2 = (double)(cs * A / len);
                    atomicAdd(gD + d, c2);
                    atomicAdd(gnx + d, -c2 * (o[0] + m.d[0] * (double)C[0]));
                    atomicAdd(gny + d, -c2 * (o[1] + m.d[1] * (double)C[1]));
                    atomicAdd(gnz + d, -c2 * (o[2] + m.d[2] * (double)C[2]));
                }
    }
}

/* ---- RK reverse ------------------------------------------------------------------------ */
/* Reverse of tri32: adds gval * d(value)/d(node) to the eight nodes of gf (FP32, one step's
 * sums; the step's totals go to the FP64 velocity derivatives afterwards) and returns
 * gval * d(value)/d(wx, wy, wz). */
__device__ __forceinline__ void tri32_rev(const DevMesh& m, const float* __restrict__ f, float* gf, int I, int J,
                                          int K, float wx, float wy, float wz, float gval, float& dx, float& dy,
                                          float& dz)
{
    dx = dy = dz = 0.f;
    if (gval == 0.f) return;
    const long b = cidx(m, I, J, K);
    const long sj = m.cs1, sk = m.cs2;
    const float f000 = __ldg(f + b), f100 = __ldg(f + b + 1), f010 = __ldg(f + b + sj), f110 = __ldg(f + b + 1 + sj);
    const float f001 = __ldg(f + b + sk), f101 = __ldg(f + b + 1 + sk), f011 = __ldg(f + b + sj + sk),
                f111 = __ldg(f + b + 1 + sj + sk);
    const float ux = 1.f - wx, uy = 1.f - wy, uz = 1.f - wz;
    const float x00 = f000 + wx * (f100 - f000), x10 = f010 + wx * (f110 - f010);
    const float x01 = f001 + wx * (f101 - f001), x11 = f011 + wx * (f111 - f011);
    const float y0 = x00 + wy * (x10 - x00), y1 = x01 + wy * (x11 - x01);
    dz = gval * (y1 - y0);
    dy = gval * (uz * (x10 - x00) + wz * (x11 - x01));
    dx = gval * (uz * (uy * (f100 - f000) + wy * (f110 - f010)) + wz * (uy * (f101 - f001) + wy * (f111 - f011)));
    const float a0 = gval * uz, a1 = gval * wz;
    atomicAdd(gf + b, a0 * (ux * uy));
    atomicAdd(gf + b + 1, a0 * (wx * uy));
    atomicAdd(gf + b + sj, a0 * (ux * wy));
    atomicAdd(gf + b + 1 + sj, a0 * (wx * wy));
    atomicAdd(gf + b + sk, a1 * (ux * uy));
    atomicAdd(gf + b + 1 + sk, a1 * (wx * uy));
    atomicAdd(gf + b + sj + sk, a1 * (ux * wy));
    atomicAdd(gf + b + 1 + sj + sk, a1 * (wx * wy));
}

struct VelGrad32 {
    float *gu, *gv, *gw; /* one step's dL/d(face velocity in cells per unit time) */
};

/* Reverse of vel32 at (x, y, z): face-velocity derivatives of the cotangent (cu, cv, cw) of
 * the interpolated velocity (cells per unit time), and its pull-back to the point in g. */
__device__ __forceinline__ void vel32_rev(const DevMesh& m, const Vel32& V, const VelGrad32& G, int i0, int j0,
                                          int k0, float x, float y, float z, float cu, float cv, float cw, float (&g)[3])
{
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
    float a, b, c;
    g[0] = g[1] = g[2] = 0.f;
    tri32_rev(m, V.uf, G.gu, Fx, Cy, Cz, wfx, wcy, wcz, cu, a, b, c);
    g[0] += a; g[1] += b; g[2] += c;
    tri32_rev(m, V.vf, G.gv, Cx, Fy, Cz, wcx, wfy, wcz, cv, a, b, c);
    g[0] += a; g[1] += b; g[2] += c;
    tri32_rev(m, V.wf, G.gw, Cx, Cy, Fz, wcx, wcy, wfz, cw, a, b, c);
    g[0] += a; g[1] += b; g[2] += c;
}

/* Reverse of project32 for the trajectory of the grid vertex (I, J, K) (the origin of its
 * cell frame): g = dL/d(end point) in cell units. */
__device__ void project32_rev(const DevMesh& m, const Vel32& V, const VelGrad32& G, int I, int J, int K, float dt,
                              const float (&g)[3])
{
    if (m.projection == 3) return; /* Zalesak rotation: no velocity */
    float u1, v1, w1;
    vel32(m, V, I, J, K, 0.f, 0.f, 0.f, u1, v1, w1);
    float c1[3] = {0.f, 0.f, 0.f}, t[3];
    if (m.projection == 0) {
        for (int p = 0; p < 3; ++p) c1[p] = -dt * g[p];
    } else if (m.projection == 1) {
        const float h = 0.5f * dt;
        const float x2 = -h * u1, y2 = -h * v1, z2 = -h * w1;
        vel32_rev(m, V, G, I, J, K, x2, y2, z2, -dt * g[0], -dt * g[1], -dt * g[2], t);
        for (int p = 0; p < 3; ++p) c1[p] = -h * t[p];
    } else {
        const float h = 0.5f * dt;
        float u2, v2, w2, u3, v3, w3;
        const float x2 = -h * u1, y2 = -h * v1, z2 = -h * w1;
        vel32(m, V, I, J, K, x2, y2, z2, u2, v2, w2);
        const float x3 = -h * u2, y3 = -h * v2, z3 = -h * w2;
        vel32(m, V, I, J, K, x3, y3, z3, u3, v3, w3);
        const float x4 = -dt * u3, y4 = -dt * v3, z4 = -dt * w3;
        const float s = -dt / 6.f;
        float c2[3], c3[3], c4[3];
        for (int p = 0; p < 3; ++p) {
            c1[p] = s * g[p];
            c2[p] = 2.f * s * g[p];
            c3[p] = 2.f * s * g[p];
            c4[p] = s * g[p];
        }
        vel32_rev(m, V, G, I, J, K, x4, y4, z4, c4[0], c4[1], c4[2], t);
        for (int p = 0; p < 3; ++p) c3[p] += -dt * t[p];
        vel32_rev(m, V, G, I, J, K, x3, y3, z3, c3[0], c3[1], c3[2], t);
        for (int p = 0; p < 3; ++p) c2[p] += -h * t[p];
        vel32_rev(m, V, G, I, J, K, x2, y2, z2, c2[0], c2[1], c2[2], t);
        for (int p = 0; p < 3; ++p) c1[p] += -h * t[p];
    }
    vel32_rev(m, V, G, I, J, K, 0.f, 0.f, 0.f, c1[0], c1[1], c1[2], t);
}

__global__ void __launch_bounds__(ADJ32_THREADS) k_adj32_vert(DevMesh m, float dt, Vel32 V, VelGrad32 G, double* gx,
                                                              double* gy, double* gz)
{
    const long n0 = m.N[0] + 1, n1 = m.N[1] + 1, n2 = m.N[2] + 1;
    const long total = n0 * n1 * n2;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (long)gridDim.x * blockDim.x) {
        const int I = 1 + (int)(q % n0), J = 1 + (int)((q / n0) % n1), K = 1 + (int)(q / (n0 * n1));
        const long t = cidx(m, I, J, K);
        const double a = gx[t], b = gy[t], c = gz[t];
        if (a == 0.0 && b == 0.0 && c == 0.0) continue;
        gx[t] = 0.0; gy[t] = 0.0; gz[t] = 0.0;
        const float g[3] = {(float)a, (float)b, (float)c};
        project32_rev(m, V, G, I, J, K, dt, g);
    }
}

/* The step's face-velocity derivatives (cells per unit time, FP32) into the FP64 totals of
 * dL/d(face velocity): divided by the spacing, since the mixed path's velocities are u / d.
 * The FP32 sums are cleared for the next step. */
__global__ void k_adj32_vel_flush(long n, float* __restrict__ su, float* __restrict__ sv, float* __restrict__ sw,
                                  double* gu, double* gv, double* gw, double rx, double ry, double rz)
{
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const float a = su[t], b = sv[t], c = sw[t];
        if (a != 0.f) { gu[t] += rx * (double)a; su[t] = 0.f; }
        if (b != 0.f) { gv[t] += ry * (double)b; sv[t] = 0.f; }
        if (c != 0.f) { gw[t] += rz * (double)c; sw[t] = 0.f; }
    }
}

/* ELVIRA backwards at interior interface cells with a chosen candidate, in FP32 (the normal
 * is c/|c| with c linear in the 3x3x3 VF block, check_normal! and ELVIRA_calc!,
 * src/ELVIRA.jl:62-115; the same algebra as the FP64 reverse). */
__device__ void elvira_reverse32(const DevMesh& m, const double* __restrict__ VF, double* gVF, int i, int j, int k,
                                 int lane, const float (&gn)[3])
{
    const int fam_on[3] = {m.N[2] > 1, m.N[1] > 1, m.N[0] > 1};
    const int fam = lane / 9, oa = (lane % 9) / 3, ob = lane % 3;
    int f = 0;
    for (int q = 0, seen = 0; q < 3; ++q)
        if (fam_on[q]) {
            if (seen == fam) { f = q; break; }
            ++seen;
        }
    const int lo_b = oa == 2 ? 0 : -1, hi_b = oa == 0 ? 0 : 1;
    const int lo_a = ob == 2 ? 0 : -1, hi_a = ob == 0 ? 0 : 1;
    const int ta = f == 2 ? 1 : 0, tb = f == 0 ? 1 : 2, tn = f == 0 ? 2 : (f == 1 ? 1 : 0);
    const float hs = (float)m.d[tn];
    const int base[3] = {i, j, k};
    auto V_ = [&](const int* e) { return (float)__ldg(VF + vidx(m, i + e[0], j + e[1], k + e[2])); };
    int e[3];
    float c[3], s2 = 0.f, s1 = 0.f;
    for (int r = -1; r <= 1; ++r) {
        e[ta] = hi_a; e[tb] = 0; e[tn] = r;
        s2 += V_(e) * hs;
        e[ta] = lo_a;
        s1 += V_(e) * hs;
    }
    const float dca = (float)(cco(m, ta, base[ta] + hi_a) - cco(m, ta, base[ta] + lo_a));
    c[ta] = -(s2 - s1) / dca;
    s2 = 0.f;
    s1 = 0.f;
    for (int r = -1; r <= 1; ++r) {
        e[tb] = hi_b; e[ta] = 0; e[tn] = r;
        s2 += V_(e) * hs;
        e[tb] = lo_b;
        s1 += V_(e) * hs;
    }
    const float dcb = (float)(cco(m, tb, base[tb] + hi_b) - cco(m, tb, base[tb] + lo_b));
    c[tb] = -(s2 - s1) / dcb;
    int up[3] = {0, 0, 0}, dn[3] = {0, 0, 0};
    up[tn] = 1;
    dn[tn] = -1;
    c[tn] = V_(up) > V_(dn) ? -1.f : 1.f;
    const float norm = sqrtf(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    const float n[3] = {c[0] / norm, c[1] / norm, c[2] / norm};
    const float dot = n[0] * gn[0] + n[1] * gn[1] + n[2] * gn[2];
    const double wa = (double)((gn[ta] - n[ta] * dot) / norm * hs / dca);
    const double wb = (double)((gn[tb] - n[tb] * dot) / norm * hs / dcb);
    for (int r = -1; r <= 1; ++r) {
        e[ta] = hi_a; e[tb] = 0; e[tn] = r;
        atomicAdd(gVF + vidx(m, i + e[0], j + e[1], k + e[2]), -wa);
        e[ta] = lo_a;
        atomicAdd(gVF + vidx(m, i + e[0], j + e[1], k + e[2]), wa);
        e[tb] = hi_b; e[ta] = 0; e[tn] = r;
        atomicAdd(gVF + vidx(m, i + e[0], j + e[1], k + e[2]), -wb);
        e[tb] = lo_b;
        atomicAdd(gVF + vidx(m, i + e[0], j + e[1], k + e[2]), wb);
    }
}

__global__ void __launch_bounds__(256) k_adj32_elvira(DevMesh m, const double* __restrict__ VF,
                                                      const signed char* __restrict__ cand,
                                                      const double* __restrict__ gnx, const double* __restrict__ gny,
                                                      const double* __restrict__ gnz, double* gout)
{
    const long total = (long)m.N[0] * m.N[1] * m.N[2];
    for (long L = (long)blockIdx.x * blockDim.x + threadIdx.x; L < total; L += (long)gridDim.x * blockDim.x) {
        const int i = 1 + (int)(L % m.N[0]), j = 1 + (int)((L / m.N[0]) % m.N[1]), k = 1 + (int)(L / ((long)m.N[0] * m.N[1]));
        const long c = cidx(m, i, j, k);
        const double a = gnx[c], b = gny[c], d = gnz[c];
        if (a == 0.0 && b == 0.0 && d == 0.0) continue;
        const double vf = VF[vidx(m, i, j, k)];
        if (!(vf >= m.VFlo && vf <= m.VFhi)) continue; /* pure cells carry fixed axis normals */
        const int lane = cand[c];
        if (lane < 0) continue;
        const float gn[3] = {(float)a, (float)b, (float)d};
        elvira_reverse32(m, VF, gout, i, j, k, lane, gn);
    }
}

/* computeDist backwards at every cell (ghosts included) from the plane polygon in the cell:
 * dD/dVF = |∇d| / A, dD/dn = its centroid (physical units). */
__global__ void __launch_bounds__(ADJ32_THREADS) k_adj32_dist(DevMesh m, const double* __restrict__ VF,
                                                              const float4* __restrict__ planes,
                                                              const double* __restrict__ gDf, double* gnx, double* gny,
                                                              double* gnz, double* gout)
{
    const long n0 = m.hi[0] - m.lo + 1, n1 = m.hi[1] - m.lo + 1, n2 = m.hi[2] - m.lo + 1;
    const long total = n0 * n1 * n2;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const double g = gDf[t];
        if (g == 0.0) continue;
        const int i = m.lo + (int)(t % n0), j = m.lo + (int)((t / n0) % n1), k = m.lo + (int)(t / (n0 * n1));
        const long v = vidx(m, i, j, k);
        const double vf = VF[v];
        if (!(vf >= m.VFlo && vf <= m.VFhi)) continue; /* pure: D = +-(Lx+Ly+Lz) */
        const float4 pl = planes[t];
        float A, M[3];
        sd::plane_cube(pl.x, pl.y, pl.z, pl.w, A, M);
        if (!(A > 0.f)) continue;
        const float len = sqrtf(pl.x * pl.x + pl.y * pl.y + pl.z * pl.z);
        gout[v] += g * (double)(len / A);
        gnx[t] += g * (fco(m, 0, i) + m.d[0] * (double)(M[0] / A));
        gny[t] += g * (fco(m, 1, j) + m.d[1] * (double)(M[1] / A));
        gnz[t] += g * (fco(m, 2, k) + m.d[2] * (double)(M[2] / A));
    }
}

} // namespace

void launch_adjoint32_sl(const DevMesh& m, double dt, const double* VFnext, const float* uf32, const float* vf32,
                         const float* wf32, const float4* planes, const signed char* phase, const int* cells,
                         const float4* verts, const int* count, float2* cinfo, double* gvx, double* gvy, double* gvz,
                         float* const* gvel32, const AdjBuffers& b, int* errw, int nsm, cudaStream_t s)
{
    const sd::BFaces F = sd::boundary_faces(m.tess);
    k_adj32_cell<<<nsm * 8, ADJ32_THREADS, 0, s>>>(m, cells, verts, count, b.gfold, VFnext, cinfo, errw);
    k_adj32_faces<<<nsm * 24, FACES_THREADS, 0, s>>>(m, planes, phase, cells, verts, cinfo, count, F, gvx, gvy, gvz);
    k_adj32_planes<<<nsm * 12, PLANES_THREADS, 0, s>>>(m, planes, phase, cells, verts, cinfo, count, b.gn[0],
                                                       b.gn[1], b.gn[2], b.gD);
    Vel32 V{uf32, vf32, wf32};
    VelGrad32 G{gvel32[0], gvel32[1], gvel32[2]};
    k_adj32_vert<<<nsm * 8, ADJ32_THREADS, 0, s>>>(m, (float)dt, V, G, gvx, gvy, gvz);
    const long n = (long)(m.N[0] + 2 * m.g) * (m.N[1] + 2 * m.g) * (m.N[2] + 2 * m.g);
    k_adj32_vel_flush<<<nsm * 8, 256, 0, s>>>(n, gvel32[0], gvel32[1], gvel32[2], b.guf, b.gvf, b.gwf, 1.0 / m.d[0],
                                              1.0 / m.d[1], 1.0 / m.d[2]);
}

void launch_adjoint32_elvira(const DevMesh& m, const double* VF, const signed char* cand, const AdjBuffers& b,
                             int nsm, cudaStream_t s)
{
    k_adj32_elvira<<<nsm * 8, 256, 0, s>>>(m, VF, cand, b.gnf[0], b.gnf[1], b.gnf[2], b.gout);
}

void launch_adjoint32_dist(const DevMesh& m, const double* VF, const float4* planes, const AdjBuffers& b, int nsm,
                           cudaStream_t s)
{
    k_adj32_dist<<<nsm * 8, ADJ32_THREADS, 0, s>>>(m, VF, planes, b.gDf, b.gn[0], b.gn[1], b.gn[2], b.gout);
}

} // namespace slvof
