/*
 * flux.cuh — the SL update of the mixed path in flux form: geometry of the swept face prisms.
 *
 * The reference's SL update (src/Transport.jl:111-148) clips each band cell's pre-image P_c,
 * the cell with its vertices traced back by project!, and sets VFnew = vLiq(P_c) / vol(P_c).
 * The pre-image's boundary is the cell's boundary triangulation (the face diagonals of the
 * tessellation, src/VFgeom.jl:229-332) with moved vertices.  For every boundary triangle t of
 * the cell C_c, the region between t and its moved copy t' is a prism S_t; with signs from
 * the outward orientation, the indicator functions satisfy
 *
 *     chi(P_c) = chi(C_c) + sum_t sigma_t chi(S_t)      (almost everywhere),
 *
 * provided every side quad (edge p-q swept to p'-q') is split into triangles the same way in
 * both prisms that share it.  Both liquid and total volume are linear in the indicator, so
 *
 *     vLiq(P_c) = VF_c |C_c| + sum_t sigma_t vLiq(S_t),   vol(P_c) = |C_c| + sum_t sigma_t |S_t|,
 *
 * where VF_c |C_c| is the liquid of the cell's own plane inside the cell, which is VF_c by the
 * definition of the PLIC constant (0 or 1 for cells below VFlo or above VFhi).  The
 * tessellations the reference uses give neighbouring cells the same diagonal on their shared
 * face (5_tets by mirroring odd cells, 6_tets by translation, 24_tets through the face's mean
 * point), so each face's prisms are the same set of points for both of its cells, with
 * opposite signs: a face's swept liquid and volume are computed once and shared.  In exact
 * arithmetic this is the reference's VFnew; in rounded arithmetic the sum over cells of the
 * liquid moved between cells cancels exactly, which is what keeps the mixed path's total mass
 * next to the FP64 path's.
 *
 * A face is named by its direction dir and the cell h on its high side (the face lies on the
 * mesh plane x_dir = x_dir[h_dir], the low face of h; the low-side cell is l = h - e_dir).
 * In the tangential axes (s, t), the two axes other than dir in increasing order, its corners
 * are A = (0,0), B = (1,0), D = (0,1), C = (1,1) from h's low corner; their grid-node
 * linear indices order them A < B < D < C.  The face's mean point M (24_tets) ranks after
 * them.  Points are numbered 0..4 = A, B, D, C, M and 5..9 = their moved copies.
 *
 * Prism of a triangle a < b < c (this order): tets (a,b,c,c'), (a,b,c',b'), (a,a',b',c').
 * The side quad of edge p < q is then split along p-q' in every prism that holds the edge, so
 * neighbouring prisms agree.  With tet_vol(p,q,r,s) = det(q-p, r-p, s-p)/6 (the reference's
 * tet_vol, src/VFgeom.jl:669-676), the three volumes sum to the prism volume, positive when
 * the triangle moves along (b-a) x (c-a).  sigma makes it the low cell's share: +1 when that
 * normal points along +e_dir, the low cell's outward normal on this face.
 */
#pragma once

#include "mesh_view.h"

namespace slvof {
namespace flux {

enum : int { PA = 0, PB = 1, PD = 2, PC = 3, PM = 4, MOVED = 5 };

/* tangential axes of a face direction */
SLVOF_HD void face_axes(int dir, int& s, int& t)
{
    s = dir == 0 ? 1 : 0;
    t = dir == 2 ? 1 : 2;
}

/* (ds, dt) offset of corner p (PA, PB, PD, PC) */
SLVOF_HD int corner_s(int p) { return p == PB || p == PC ? 1 : 0; }
SLVOF_HD int corner_t(int p) { return p == PD || p == PC ? 1 : 0; }

/* The diagonal of the face: true for A-C ("main"), false for B-D.  5_tets: main on the low
 * faces of even cells (i+j+k even) and on the high faces of odd ones, so on the face of high
 * cell h exactly when h is even; 6_tets: B-D on x and y faces, A-C on z faces. */
SLVOF_HD bool face_main_diagonal(int tess, int dir, int i, int j, int k)
{
    if (tess == 6) return dir == 2;
    return ((i + j + k) & 1) == 0;
}

/* Triangles of the face, each as points a < b < c in the ranking above, with sigma.
 * Returns the number of triangles (2, or 4 for 24_tets). */
SLVOF_HD int face_triangles(int tess, int dir, bool main_diag, int (*tri)[3], int* sigma)
{
    /* the 2D orientation (b-a) x (c-a) in (s, t) of each sorted triangle; e_dir = e_s x e_t
     * for dir 0 and 2, -(e_s x e_t) for dir 1 */
    const int ds = dir == 1 ? -1 : 1;
    if (tess == 24) {
        const int T[4][3] = {{PA, PB, PM}, {PB, PC, PM}, {PD, PC, PM}, {PA, PD, PM}};
        const int o[4] = {1, 1, -1, -1};
        for (int n = 0; n < 4; ++n) {
            tri[n][0] = T[n][0]; tri[n][1] = T[n][1]; tri[n][2] = T[n][2];
            sigma[n] = o[n] * ds;
        }
        return 4;
    }
    if (main_diag) {
        tri[0][0] = PA; tri[0][1] = PB; tri[0][2] = PC; sigma[0] = ds;
        tri[1][0] = PA; tri[1][1] = PD; tri[1][2] = PC; sigma[1] = -ds;
    } else {
        tri[0][0] = PA; tri[0][1] = PB; tri[0][2] = PD; sigma[0] = ds;
        tri[1][0] = PB; tri[1][1] = PD; tri[1][2] = PC; sigma[1] = -ds;
    }
    return 2;
}

/* Point ids of tet n (0..2) of the prism of sorted triangle (a, b, c). */
SLVOF_HD void prism_tet(const int* tr, int n, int* q)
{
    const int a = tr[0], b = tr[1], c = tr[2];
    if (n == 0) { q[0] = a; q[1] = b; q[2] = c; q[3] = c + MOVED; }
    else if (n == 1) { q[0] = a; q[1] = b; q[2] = c + MOVED; q[3] = b + MOVED; }
    else { q[0] = a; q[1] = a + MOVED; q[2] = b + MOVED; q[3] = c + MOVED; }
}

/* Grid node (i, j, k) of corner p of the face (dir, h). */
SLVOF_HD void corner_node(int dir, int hi, int hj, int hk, int p, int& i, int& j, int& k)
{
    int s, t;
    face_axes(dir, s, t);
    int n[3] = {hi, hj, hk};
    n[s] += corner_s(p);
    n[t] += corner_t(p);
    i = n[0]; j = n[1]; k = n[2];
}

} // namespace flux
} // namespace slvof
