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

/* add_correction_tets (src/VFgeom.jl:514-664; pressure_scheme "finite-difference", 5_tets) of one
 * face, on the flux form's traced nodes, in cell units and the low cell's frame.  The face's
 * flux volume (SLfluxVol, src/VFgeom.jl:428-509: the hexahedron between the face and its
 * projection, split by the five-tet pattern of the face's cell) and the finite-difference
 * volume dt * u_face / d give the volume that the tets (a, b, d, e) and (b, c, d, e) over the
 * projected quad must add; the apex e moves from the quad's mean along the face normal until
 * they do (the two volumes are affine in e).  A band cell adds these tets with its own parity
 * sign, and the two cells of a face have opposite parities, so like the swept prism they are a
 * face quantity: the result is the tets' FP64 volume signed for the low cell, and e. */
SLVOF_HD double face_correction(int dir, int hi, int hj, int hk, double dtu, const double (*P)[3], const double (*Q)[3],
                                double* e)
{
    int s, t;
    face_axes(dir, s, t);
    const bool ev = tess_even(5, hi, hj, hk);
    double fv[8][3];
    for (int n = 0; n < 8; ++n) {
        int off[3];
        const bool proj = flux_node(dir, ev, n, off);
        const int p = off[s] + 2 * off[t]; /* the corner at (s, t) offsets: PA, PB, PD, PC */
        for (int q = 0; q < 3; ++q) fv[n][q] = proj ? Q[p][q] : P[p][q];
    }
    auto tv = [](const double* a, const double* b, const double* c, const double* d) {
        /* tet_vol, src/VFgeom.jl:669-681, in the reference's expansion order */
        const double a1 = a[0] - d[0], a2 = a[1] - d[1], a3 = a[2] - d[2];
        const double b1 = b[0] - d[0], b2 = b[1] - d[1], b3 = b[2] - d[2];
        const double c1 = c[0] - d[0], c2 = c[1] - d[1], c3 = c[2] - d[2];
        return (-1.0 / 6.0) * ((a1 * (b2 * c3 - c2 * b3) - a2 * (b1 * c3 - c1 * b3)) + a3 * (b1 * c2 - c1 * b2));
    };
    double flux = 0.0;
    for (int q = 0; q < 5; ++q) flux += tv(fv[tet5(q, 0)], fv[tet5(q, 1)], fv[tet5(q, 2)], fv[tet5(q, 3)]);
    if (!ev) flux = -flux;
    const double vol = ev ? (dtu - flux) : -(dtu - flux);
    const double *a = fv[flux_quad(dir, ev, 0)], *b = fv[flux_quad(dir, ev, 1)], *c = fv[flux_quad(dir, ev, 2)],
                 *d = fv[flux_quad(dir, ev, 3)];
    for (int q = 0; q < 3; ++q) e[q] = 0.25 * (((a[q] + b[q]) + c[q]) + d[q]);
    const double v0 = tv(a, b, d, e) + tv(b, c, d, e);
    const int p1 = (dir + 1) % 3, p2 = (dir + 2) % 3;
    const double N = (((a[p1] * b[p2] - a[p2] * b[p1]) + (d[p1] * a[p2] - d[p2] * a[p1])) +
                      (b[p1] * c[p2] - b[p2] * c[p1])) +
                     (c[p1] * d[p2] - c[p2] * d[p1]);
    e[dir] += 6.0 * (vol - v0) / N;
    const double vt = tv(a, b, d, e) + tv(b, c, d, e);
    return ev ? -vt : vt; /* the low cell's parity is the opposite of the face's cell's */
}

} // namespace flux
} // namespace slvof
