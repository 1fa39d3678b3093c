/*
 * mesh_view.h — plain C++ view of the mesh and the constant tables of the SL-VOF path,
 * shared by the CUDA kernels and by host code (context setup, host-side test harnesses).
 * Nothing here depends on the CUDA runtime.
 *
 * Index convention: the reference's Julia cell indices, interior 1..N, ghosts 1-g..0 and
 * N+1..N+g; VF carries three more layers (src/Tools.jl:144).  Arrays are OffsetArray
 * parents, i fastest.
 */
#pragma once

#include <cmath>
#include <cstdint>

#include "../../include/slvof.h"

#if defined(__CUDACC__)
#define SLVOF_HD __host__ __device__ __forceinline__
#else
#define SLVOF_HD inline
#endif

namespace slvof {

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
    int tess;      /* tets per cell: 5, 6 or 24 (src/VFgeom.jl:229-332) */
    int fd;        /* pressure_scheme "finite-difference": band cells add the flux-correction tets */
    double d[3];
    double VFlo, VFhi;
    double Lsum;    /* (Lx+Ly)+Lz, |D| of pure cells (src/VF.jl:116-120) */
    double cellvol; /* (dx*dy)*dz */
    const double* f[3]; /* face coordinates, f[q][i - lo] */
    const double* c[3]; /* centre coordinates */
    long cs1, cs2;      /* cell-array strides (j, k) */
    long vs1, vs2;      /* VF strides */
};

/* Coordinate block of a mesh: x, y, z faces (N+2g+1 each) then xm, ym, zm centres (N+2g
 * each).  Returns the number of doubles; fills out[] when it is not null. */
inline long mesh_coords(const slvof_mesh* mesh, double* out)
{
    const long g = mesh->nghost;
    const long nn[3] = {mesh->Nx + 2 * g, mesh->Ny + 2 * g, mesh->Nz + 2 * g};
    const double* fsrc[3] = {mesh->x, mesh->y, mesh->z};
    const double* csrc[3] = {mesh->xm, mesh->ym, mesh->zm};
    long o = 0;
    for (int q = 0; q < 3; ++q)
        for (long t = 0; t <= nn[q]; ++t) {
            if (out) out[o] = fsrc[q][t];
            ++o;
        }
    for (int q = 0; q < 3; ++q)
        for (long t = 0; t < nn[q]; ++t) {
            if (out) out[o] = csrc[q][t];
            ++o;
        }
    return o;
}

/* DevMesh of a mesh whose coordinate block (mesh_coords layout) sits at coords, which may be
 * a device or a host pointer. */
inline void mesh_fill(const slvof_mesh* mesh, const double* coords, DevMesh& m)
{
    const long g = mesh->nghost;
    const long N[3] = {mesh->Nx, mesh->Ny, mesh->Nz};
    const long nn[3] = {N[0] + 2 * g, N[1] + 2 * g, N[2] + 2 * g};
    long o = 0;
    double maxabs = 0.0;
    const double* fsrc[3] = {mesh->x, mesh->y, mesh->z};
    for (int q = 0; q < 3; ++q) {
        m.N[q] = (int)N[q];
        m.hi[q] = (int)(N[q] + g);
        m.f[q] = coords + o;
        for (long t = 0; t <= nn[q]; ++t) maxabs = std::fmax(maxabs, std::fabs(fsrc[q][t]));
        o += nn[q] + 1;
    }
    for (int q = 0; q < 3; ++q) {
        m.c[q] = coords + o;
        o += nn[q];
    }
    m.g = (int)g;
    m.nband = mesh->nband;
    m.projection = mesh->projection;
    m.per[0] = mesh->xper != 0; m.per[1] = mesh->yper != 0; m.per[2] = mesh->zper != 0;
    m.lo = 1 - (int)g;
    m.vlo = m.lo - 3;
    m.d[0] = mesh->dx; m.d[1] = mesh->dy; m.d[2] = mesh->dz;
    m.VFlo = mesh->VFlo;
    m.VFhi = mesh->VFhi;
    m.Lsum = (mesh->Lx + mesh->Ly) + mesh->Lz;
    m.cellvol = (mesh->dx * mesh->dy) * mesh->dz;
    m.fast_pure = maxabs < m.Lsum * (1.0 - 1e-9);
    m.tess = mesh->tesselation == 0 ? 5 : mesh->tesselation;
    m.fd = mesh->pressure_scheme == 1;
    m.cs1 = nn[0]; m.cs2 = nn[0] * nn[1];
    m.vs1 = nn[0] + 6; m.vs2 = (nn[0] + 6) * (nn[1] + 6);
}

/* Single-rank ghost fill as a source map.  Neumann! (x-,x+,y-,y+,z-,z+) followed by
 * update_borders! (x, y, z; two self-Sendrecv! copies per periodic direction) is a sequence
 * of slab copies, each reading the state before it.  Walking the copies backwards gives, for
 * every cell, the cell whose pre-fill value it ends with.  The copies of one direction only
 * move that direction's index, so the map is separable. */
SLVOF_HD int ghost_src_1d(int p, int N, int g, bool periodic, bool neumann)
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

/* Initialiser of a CutCase[16] (0-based transcription of the reference tables); X_ marks
 * unused entries and must be defined as -1 where the table is instantiated. */
#define SLVOF_CUT_TABLE \
{ \
    {0, 1, 1, 0, {X_, X_, X_, X_}, {X_, X_, X_, X_}, \
     {{0, 1, 2, 3}, {X_, X_, X_, X_}, {X_, X_, X_, X_}, {X_, X_, X_, X_}, {X_, X_, X_, X_}, {X_, X_, X_, X_}}, \
     {0, X_, X_, X_, X_, X_}, {0, 0}}, \
    {3, 4, 2, 0, {0, 0, 0, X_}, {1, 2, 3, X_}, \
     {{4, 6, 5, 0}, {5, 1, 2, 3}, {3, 1, 4, 5}, {4, 5, 6, 3}, {X_, X_, X_, X_}, {X_, X_, X_, X_}}, \
     {1, 0, 0, 0, X_, X_}, {0, 0}}, \
    {3, 4, 2, 0, {1, 1, 1, X_}, {2, 3, 0, X_}, \
     {{6, 4, 5, 1}, {0, 2, 3, 5}, {0, 4, 2, 5}, {4, 6, 5, 0}, {X_, X_, X_, X_}, {X_, X_, X_, X_}}, \
     {1, 0, 0, 0, X_, X_}, {0, 0}}, \
    {4, 6, 4, 0, {0, 1, 0, 1}, {3, 3, 2, 2}, \
     {{4, 7, 5, 1}, {4, 6, 7, 0}, {4, 0, 7, 1}, {4, 5, 7, 3}, {4, 7, 6, 2}, {4, 7, 2, 3}}, \
     {1, 1, 1, 0, 0, 0}, {0, 0}}, \
    {3, 4, 2, 0, {2, 2, 2, X_}, {3, 0, 1, X_}, \
     {{5, 4, 6, 2}, {1, 0, 3, 5}, {5, 4, 3, 1}, {5, 6, 4, 1}, {X_, X_, X_, X_}, {X_, X_, X_, X_}}, \
     {1, 0, 0, 0, X_, X_}, {0, 0}}, \
    {4, 6, 4, 0, {0, 2, 0, 2}, {3, 3, 1, 1}, \
     {{4, 5, 7, 2}, {4, 7, 6, 0}, {4, 7, 0, 2}, {4, 7, 5, 3}, {4, 6, 7, 1}, {4, 7, 3, 1}}, \
     {1, 1, 1, 0, 0, 0}, {0, 0}}, \
    {4, 6, 4, 0, {1, 2, 1, 2}, {3, 3, 0, 0}, \
     {{7, 5, 4, 2}, {4, 6, 7, 1}, {7, 4, 1, 2}, {7, 4, 5, 3}, {4, 7, 6, 0}, {4, 7, 0, 3}}, \
     {1, 1, 1, 0, 0, 0}, {0, 0}}, \
    {3, 4, 4, 0, {3, 3, 3, X_}, {0, 1, 2, X_}, \
     {{0, 1, 2, 6}, {0, 1, 6, 5}, {4, 6, 5, 0}, {4, 5, 6, 3}, {X_, X_, X_, X_}, {X_, X_, X_, X_}}, \
     {1, 1, 1, 0, X_, X_}, {0, 0}}, \
    {3, 4, 2, 0, {3, 3, 3, X_}, {0, 1, 2, X_}, \
     {{4, 5, 6, 3}, {0, 1, 2, 5}, {4, 0, 2, 5}, {4, 6, 5, 2}, {X_, X_, X_, X_}, {X_, X_, X_, X_}}, \
     {1, 0, 0, 0, X_, X_}, {0, 0}}, \
    {4, 6, 4, 0, {0, 3, 0, 3}, {2, 2, 1, 1}, \
     {{4, 7, 5, 3}, {4, 6, 7, 0}, {4, 7, 3, 0}, {4, 5, 7, 2}, {4, 7, 6, 1}, {4, 7, 1, 2}}, \
     {1, 1, 1, 0, 0, 0}, {0, 0}}, \
    {4, 6, 4, 0, {1, 3, 1, 3}, {2, 2, 0, 0}, \
     {{7, 4, 5, 3}, {4, 7, 6, 1}, {7, 1, 4, 3}, {7, 5, 4, 2}, {4, 6, 7, 0}, {4, 7, 2, 0}}, \
     {1, 1, 1, 0, 0, 0}, {0, 0}}, \
    {3, 4, 4, 0, {2, 2, 2, X_}, {3, 0, 1, X_}, \
     {{0, 3, 1, 6}, {3, 0, 5, 6}, {5, 6, 4, 3}, {5, 4, 6, 2}, {X_, X_, X_, X_}, {X_, X_, X_, X_}}, \
     {1, 1, 1, 0, X_, X_}, {0, 0}}, \
    {4, 6, 4, 0, {2, 3, 2, 3}, {1, 1, 0, 0}, \
     {{7, 5, 4, 3}, {4, 6, 7, 2}, {7, 3, 4, 2}, {7, 4, 5, 1}, {4, 7, 6, 0}, {4, 7, 0, 1}}, \
     {1, 1, 1, 0, 0, 0}, {0, 0}}, \
    {3, 4, 4, 0, {1, 1, 1, X_}, {2, 3, 0, X_}, \
     {{2, 3, 0, 6}, {6, 5, 2, 3}, {6, 5, 4, 2}, {6, 4, 5, 1}, {X_, X_, X_, X_}, {X_, X_, X_, X_}}, \
     {1, 1, 1, 0, X_, X_}, {0, 0}}, \
    {3, 4, 4, 0, {0, 0, 0, X_}, {1, 2, 3, X_}, \
     {{6, 3, 1, 2}, {1, 2, 5, 6}, {4, 5, 6, 1}, {4, 6, 5, 0}, {X_, X_, X_, X_}, {X_, X_, X_, X_}}, \
     {1, 1, 1, 0, X_, X_}, {0, 0}}, \
    {0, 1, 2, 0, {X_, X_, X_, X_}, {X_, X_, X_, X_}, \
     {{0, 1, 2, 3}, {X_, X_, X_, X_}, {X_, X_, X_, X_}, {X_, X_, X_, X_}, {X_, X_, X_, X_}, {X_, X_, X_, X_}}, \
     {1, X_, X_, X_, X_, X_}, {0, 0}}, \
}

/* 5-tet split of the 8 cell vertices (src/VFgeom.jl:235-256), 0-based. */
SLVOF_HD constexpr int tet5(int t, int n)
{
    return (t == 0) ? (n == 0 ? 0 : n == 1 ? 1 : n == 2 ? 3 : 5)
         : (t == 1) ? (n == 0 ? 0 : n == 1 ? 3 : n == 2 ? 2 : 6)
         : (t == 2) ? (n == 0 ? 0 : n == 1 ? 4 : n == 2 ? 5 : 6)
         : (t == 3) ? (n == 0 ? 3 : n == 1 ? 6 : n == 2 ? 5 : 7)
                    : (n == 0 ? 0 : n == 1 ? 3 : n == 2 ? 6 : 5);
}


/* ---- tessellations (src/VFgeom.jl:171-184,229-332) --------------------------------------
 * A cell's points, 0-based: 0..7 its vertices in cell2verts! order, 8 the mean of the
 * vertices and 9..14 the means of its six faces (24_tets only).  Only 5_tets mirrors odd
 * cells (oddEvenCell); 6_tets and 24_tets use the even order and tet sign +1 everywhere. */
SLVOF_HD constexpr int tess_ntets(int tess) { return tess == 6 ? 6 : (tess == 24 ? 24 : 5); }
SLVOF_HD constexpr int tess_npoints(int tess) { return tess == 24 ? 15 : 8; }
SLVOF_HD constexpr bool tess_even(int tess, int i, int j, int k) { return tess != 5 || ((i + j + k) % 2) == 0; }

/* face f of 24_tets as vertex ids in the order of `vts` (src/VFgeom.jl:297-302), 0-based */
SLVOF_HD constexpr int face24(int f, int n)
{
    return f == 0 ? (n == 0 ? 0 : n == 1 ? 2 : n == 2 ? 6 : 4)
         : f == 1 ? (n == 0 ? 1 : n == 1 ? 5 : n == 2 ? 7 : 3)
         : f == 2 ? (n == 0 ? 0 : n == 1 ? 4 : n == 2 ? 5 : 1)
         : f == 3 ? (n == 0 ? 2 : n == 1 ? 3 : n == 2 ? 7 : 6)
         : f == 4 ? (n == 0 ? 0 : n == 1 ? 1 : n == 2 ? 3 : 2)
                  : (n == 0 ? 4 : n == 1 ? 6 : n == 2 ? 7 : 5);
}

/* point id of vertex n of tet t */
SLVOF_HD constexpr int tess_tet(int tess, int t, int n)
{
    return tess == 5 ? tet5(t, n)
         : tess == 6 ? ((t == 0) ? (n == 0 ? 4 : n == 1 ? 5 : n == 2 ? 3 : 7)
                      : (t == 1) ? (n == 0 ? 4 : n == 1 ? 5 : n == 2 ? 1 : 3)
                      : (t == 2) ? (n == 0 ? 4 : n == 1 ? 1 : n == 2 ? 0 : 3)
                      : (t == 3) ? (n == 0 ? 6 : n == 1 ? 7 : n == 2 ? 4 : 3)
                      : (t == 4) ? (n == 0 ? 2 : n == 1 ? 3 : n == 2 ? 6 : 4)
                                 : (n == 0 ? 0 : n == 1 ? 3 : n == 2 ? 2 : 4))
         /* 24_tets: face f = t/4, tets (v4,v1,f,m), (v1,v2,f,m), (v2,v3,f,m), (v3,v4,f,m) */
         : (n == 0 ? face24(t / 4, (t % 4 + 3) % 4)
            : n == 1 ? face24(t / 4, t % 4)
            : n == 2 ? 9 + t / 4 : 8);
}

/* Mean points of 24_tets from the vertices p[0..7], as Julia's Statistics.mean(eachcol(...))
 * computes them: the vectors summed in order, then divided by their count. */
template <class R>
SLVOF_HD void tess_means(int tess, R (*p)[3])
{
    if (tess != 24) return;
    for (int q = 0; q < 3; ++q) {
        R s = p[0][q];
        for (int n = 1; n < 8; ++n) s = s + p[n][q];
        p[8][q] = s / R(8);
    }
    for (int f = 0; f < 6; ++f)
        for (int q = 0; q < 3; ++q) {
            R s = p[face24(f, 0)][q];
            for (int n = 1; n < 4; ++n) s = s + p[face24(f, n)][q];
            p[9 + f][q] = s / R(4);
        }
}

/* Node n of the flux volume of face `dir` at the low side of cell (fi, fj, fk) (SLfluxVol,
 * src/VFgeom.jl:428-509): its grid node's offsets from that cell, and whether it is projected.
 * Along the face normal each node pair holds the projected node first in even cells and
 * second in odd ones (oddEvenCell mirrors x). */
SLVOF_HD bool flux_node(int dir, bool even, int n, int off[3])
{
    const int b0 = n & 1, b1 = (n >> 1) & 1, b2 = (n >> 2) & 1;
    if (dir == 0) {
        off[0] = 0; off[1] = b1; off[2] = b2;
        return even ? b0 == 0 : b0 == 1;
    }
    off[0] = even ? b0 : 1 - b0;
    if (dir == 1) {
        off[1] = 0; off[2] = b2;
        return b1 == 0;
    }
    off[1] = b1; off[2] = 0;
    return b2 == 0;
}

/* Corner q of the face quad a, b, c, d (the projected nodes, src/VFgeom.jl:590-646). */
SLVOF_HD int flux_quad(int dir, bool even, int q)
{
    if (dir == 0) return even ? (q == 0 ? 4 : (q == 1 ? 6 : (q == 2 ? 2 : 0))) : (q == 0 ? 7 : (q == 1 ? 5 : (q == 2 ? 1 : 3)));
    if (dir == 1) return q == 0 ? 1 : (q == 1 ? 5 : (q == 2 ? 4 : 0));
    return q == 0 ? 1 : (q == 1 ? 0 : (q == 2 ? 2 : 3));
}

} // namespace slvof
