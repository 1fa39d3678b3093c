/*
 * plic64.cuh — FP64 liquid fraction of a cell under a plane (computePLIC2VF, src/VF.jl:219-278),
 * shared by the FP64 ELVIRA kernel and the FP64 arbitration of the mixed ELVIRA kernel.  Units
 * including it are built with -fmad=false so both round identically to the CPU restatement.
 */
#pragma once

#include "slvof_dev.cuh"

namespace slvof {

__device__ __forceinline__ void load_table(CutCase* s_tab)
{
    for (int t = threadIdx.x; t < 16 * (int)sizeof(CutCase); t += blockDim.x)
        reinterpret_cast<char*>(s_tab)[t] = reinterpret_cast<const char*>(c_cut)[t];
    __syncthreads();
}

/* ======================================================================================
 * computePLIC2VF (src/VF.jl:219-278) of one cell for one plane.  The five "uncut" terms
 * tetsign*tet_vol/(dx*dy*dz) of the cell are precomputed; a tet whose four distances are all
 * negative is d2case case 1 and contributes exactly that term, so the running sum
 * VF += ... is bit-identical to the reference's.
 * ==================================================================================== */
struct NbrGeom {
    double X[2], Y[2], Z[2]; /* cell2verts corners (odd cells mirrored in x, src/VFgeom.jl:190-216) */
    double tetsign;
};

__device__ __forceinline__ void nbr_geom(const DevMesh& m, int ii, int jj, int kk, NbrGeom& G)
{
    const bool even = ((ii + jj + kk) % 2) == 0;
    G.X[0] = fco(m, 0, even ? ii : ii + 1);
    G.X[1] = fco(m, 0, even ? ii + 1 : ii);
    G.Y[0] = fco(m, 1, jj); G.Y[1] = fco(m, 1, jj + 1);
    G.Z[0] = fco(m, 2, kk); G.Z[1] = fco(m, 2, kk + 1);
    G.tetsign = even ? 1.0 : -1.0;
}

static __device__ __noinline__ void cut_tet_accum64(const CutCase* tab, const NbrGeom& G, int t, double d0, double d1,
                                             double d2, double d3, double cellvol, double& VF, int& err)
{
    double vx[8], vy[8], vz[8], d[4];
    for (int n = 0; n < 4; ++n) {
        const int v = tet5(t, n);
        vx[n] = G.X[v & 1]; vy[n] = G.Y[(v >> 1) & 1]; vz[n] = G.Z[v >> 2];
    }
    const int cs = d2case(d0, d1, d2, d3, EPS64, err); /* in place, as computePLIC2VF does */
    d[0] = d0; d[1] = d1; d[2] = d2; d[3] = d3;
    const CutCase& C = tab[cs];
    for (int n = 0; n < C.nvert; ++n) {
        const int v1 = C.v1[n], v2 = C.v2[n];
        const double mu = clamp_mu(sdiv(-d[v1], d[v2] - d[v1]));
        vx[4 + n] = (1.0 - mu) * vx[v1] + mu * vx[v2];
        vy[4 + n] = (1.0 - mu) * vy[v1] + mu * vy[v2];
        vz[4 + n] = (1.0 - mu) * vz[v1] + mu * vz[v2];
    }
    for (int n = C.ntets - 1; n >= C.nntet - 1; --n) {
        const int a = C.vtet[n][0], b = C.vtet[n][1], c = C.vtet[n][2], e = C.vtet[n][3];
        const double tv = tet_vol(vx[a], vy[a], vz[a], vx[b], vy[b], vz[b], vx[c], vy[c], vz[c], vx[e], vy[e], vz[e]);
        VF += G.tetsign * tv / cellvol;
    }
}

__device__ __forceinline__ double plic2vf64(const CutCase* tab, const NbrGeom& G, const double* term, double full,
                                            double a, double b, double e, double dist, double cellvol, int& err)
{
    const double px0 = a * G.X[0], px1 = a * G.X[1];
    const double py0 = b * G.Y[0], py1 = b * G.Y[1];
    const double pz0 = e * G.Z[0], pz1 = e * G.Z[1];
    const double s00 = px0 + py0, s10 = px1 + py0, s01 = px0 + py1, s11 = px1 + py1;
    double dv[8];
    dv[0] = (s00 + pz0) - dist; dv[1] = (s10 + pz0) - dist; dv[2] = (s01 + pz0) - dist; dv[3] = (s11 + pz0) - dist;
    dv[4] = (s00 + pz1) - dist; dv[5] = (s10 + pz1) - dist; dv[6] = (s01 + pz1) - dist; dv[7] = (s11 + pz1) - dist;
    bool allneg = true, allpos = true;
#pragma unroll
    for (int v = 0; v < 8; ++v) { allneg = allneg && dv[v] < 0.0; allpos = allpos && dv[v] > 0.0; }
    if (allneg) return full;
    if (allpos) return 0.0;
    double VF = 0.0;
#pragma unroll
    for (int t = 0; t < 5; ++t) {
        const double d0 = dv[tet5(t, 0)], d1 = dv[tet5(t, 1)], d2 = dv[tet5(t, 2)], d3 = dv[tet5(t, 3)];
        if (d0 < 0.0 && d1 < 0.0 && d2 < 0.0 && d3 < 0.0) { VF += term[t]; continue; }
        if (d0 > 0.0 && d1 > 0.0 && d2 > 0.0 && d3 > 0.0) continue;
        cut_tet_accum64(tab, G, t, d0, d1, d2, d3, cellvol, VF, err);
    }
    return VF;
}

/* computePLIC2VF (src/VF.jl:219-278) for any tessellation, as the reference loops: the
 * cell's tets (cell2tets!, means for 24_tets), d2case in place, interpolated vertices from
 * the fixed-up distances, liquid tets from the last one down, VF += tetsign*tet_vol/cellvol.
 * The 5_tets case has the cached form plic2vf64 above. */
static __device__ __noinline__ double plic2vf64_gen(const CutCase* tab, const DevMesh& m, int i, int j, int k,
                                                    double nx, double ny, double nz, double dist, int& err)
{
    const int tess = m.tess;
    const bool even = tess_even(tess, i, j, k);
    const double tetsign = even ? 1.0 : -1.0;
    const double X[2] = {fco(m, 0, even ? i : i + 1), fco(m, 0, even ? i + 1 : i)};
    const double Y[2] = {fco(m, 1, j), fco(m, 1, j + 1)};
    const double Z[2] = {fco(m, 2, k), fco(m, 2, k + 1)};
    double p[15][3];
    for (int v = 0; v < 8; ++v) { p[v][0] = X[v & 1]; p[v][1] = Y[(v >> 1) & 1]; p[v][2] = Z[v >> 2]; }
    tess_means<double>(tess, p);
    double VF = 0.0;
    for (int t = 0; t < tess_ntets(tess); ++t) {
        double vx[8], vy[8], vz[8], d[4];
        for (int n = 0; n < 4; ++n) {
            const int v = tess_tet(tess, t, n);
            vx[n] = p[v][0]; vy[n] = p[v][1]; vz[n] = p[v][2];
            d[n] = ((nx * vx[n] + ny * vy[n]) + nz * vz[n]) - dist;
        }
        const int cs = d2case(d[0], d[1], d[2], d[3], EPS64, err);
        const CutCase& C = tab[cs];
        for (int n = 0; n < C.nvert; ++n) {
            const int v1 = C.v1[n], v2 = C.v2[n];
            const double mu = clamp_mu(sdiv(-d[v1], d[v2] - d[v1]));
            vx[4 + n] = (1.0 - mu) * vx[v1] + mu * vx[v2];
            vy[4 + n] = (1.0 - mu) * vy[v1] + mu * vy[v2];
            vz[4 + n] = (1.0 - mu) * vz[v1] + mu * vz[v2];
        }
        for (int n = C.ntets - 1; n >= C.nntet - 1; --n) {
            const int a = C.vtet[n][0], b = C.vtet[n][1], c = C.vtet[n][2], e = C.vtet[n][3];
            const double tv = tet_vol(vx[a], vy[a], vz[a], vx[b], vy[b], vz[b], vx[c], vy[c], vz[c], vx[e], vy[e], vz[e]);
            VF += tetsign * tv / m.cellvol;
        }
    }
    return VF;
}

/* The plane each cell donates with: its own border-updated normal and D.  Phase +1/-1 marks
 * |D| = Lx+Ly+Lz with a zero or axis normal: every point of the domain and its ghosts is then
 * strictly on one side, so a clip against the plane is all liquid (+1) or all gas (-1). */
static __device__ __forceinline__ void plic_outputs(const DevMesh& m, long t, int ip, int jp, int kp, double dist,
                                             const double* __restrict__ nx, const double* __restrict__ ny,
                                             const double* __restrict__ nz, double* __restrict__ D,
                                             float4* __restrict__ planes, signed char* __restrict__ phase)
{
    D[t] = dist;
    const double a = nx[t], b = ny[t], e = nz[t];
    const double l1 = fabs(a) + fabs(b) + fabs(e);
    phase[t] = (l1 <= 1.0 && dist == m.Lsum) ? 1 : ((l1 <= 1.0 && dist == -m.Lsum) ? -1 : 0);
    if (planes) {
        const double Dl = dist - ((a * fco(m, 0, ip) + b * fco(m, 1, jp)) + e * fco(m, 2, kp));
        planes[t] = make_float4((float)(a * m.d[0]), (float)(b * m.d[1]), (float)(e * m.d[2]), (float)Dl);
    }
}

} // namespace slvof
