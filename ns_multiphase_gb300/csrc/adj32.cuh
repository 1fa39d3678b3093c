/*
 * adj32.cuh — derivatives of a cell's SL update by the boundary of its pre-image, for the
 * reverse pass of mixed-precision contexts.  Host and device code, templated on the scalar
 * (float on the GPU; the CPU tests also build it with double).
 *
 * The SL update of a band cell (src/Transport.jl:111-148) is VFnew = vLiq / vol, with
 *   vol  = sum_t tetsign * V(T_t),   vLiq = sum_t tetsign * V(T_t ∩ L),
 * T_t the pre-image tets of the cell's tessellation and L the liquid region of the donor cells
 * (cell C_d below its PLIC plane n_d.x < D_d).  cutTet (src/VFgeom.jl:713-900) computes
 * V(T ∩ L) exactly, up to rounding, so the derivatives of the step are those of the exact
 * clipped volume.  These come from the boundary of the region instead of a reverse walk of the
 * clip tree:
 *
 *   vertices  moving vertex a of tet T by dv changes V(T ∩ L) by the flux of the moving faces,
 *             sum over the faces F of T holding a of  dv . S_F * m_{F,a},  where S_F is the
 *             face's oriented area vector (S_F = -3 dV/dv_b for b the vertex opposite F, which
 *             carries the sign of a negatively oriented tet) and m_{F,a} the liquid moment
 *             int_{F ∩ L} lambda_a dA / |F| of the barycentric coordinate of a.  Faces shared
 *             by two tets of the cell cancel, so only the pre-image's boundary faces are
 *             integrated.  For the whole volume m = 1/3, which gives d(vol).
 *   planes    moving the plane of donor d: dV(T ∩ L)/dD_d = sign(V(T)) A / |∇d| and
 *             dV/dn_d = -sign(V(T)) xbar A / |∇d|, with A and xbar the area and centroid of
 *             the plane's polygon inside T ∩ C_d (∇d the gradient of n.x - D in cell units).
 *   computeDist  D = computeDist(n, VF) inverts the cut-cell fraction F(n, D) (src/VF.jl:109-156),
 *             the exact plane/cube volume for every tessellation: dD/dVF = 1 / F_D and
 *             dD/dn = -F_n / F_D = xbar, the centroid of the plane's polygon in the cell.
 *
 * Geometry is in the updated cell's local frame in cell units (the mixed path's frame): mesh
 * planes are integers, a point's donor cell is the integer triple packed with it.  A face is
 * cut into donor pieces by the mesh planes between the smallest and largest donor index of its
 * vertices, so every piece goes to the donor cutTet gives it, also where pt2index! clamps an
 * index at the end of the grid.  Each piece is clipped by its donor's plane in the face's
 * barycentric coordinates (lambda_1, lambda_2), where the face is the unit right triangle.
 */
#pragma once

#include <cmath>

#include "mesh_view.h"

namespace slvof {
namespace sd {

SLVOF_HD int imin(int a, int b) { return a < b ? a : b; }
SLVOF_HD int imax(int a, int b) { return a > b ? a : b; }
SLVOF_HD float sqrt_of(float x) { return sqrtf(x); }
SLVOF_HD double sqrt_of(double x) { return sqrt(x); }

constexpr int MAXP = 10; /* a triangle cut by 6 box planes and a plane keeps at most 10 vertices */

template <class R>
struct Poly2 {
    int n;
    R a[MAXP], b[MAXP]; /* barycentric (lambda_1, lambda_2) of each vertex, in order */
};

template <class R>
struct Poly3 {
    int n;
    R x[MAXP], y[MAXP], z[MAXP];
};

/* Sutherland-Hodgman split of a convex polygon by f = f0 + f1*a + f2*b: the part with f <= 0
 * into lo, f >= 0 into up (either may be null).  Vertex order is kept. */
template <class R>
SLVOF_HD void split2(const Poly2<R>& P, R f0, R f1, R f2, Poly2<R>* lo, Poly2<R>* up)
{
    if (lo) lo->n = 0;
    if (up) up->n = 0;
    if (P.n < 3) return;
    int ip = P.n - 1;
    R fp = f0 + f1 * P.a[ip] + f2 * P.b[ip];
    for (int q = 0; q < P.n; ++q) {
        const R fq = f0 + f1 * P.a[q] + f2 * P.b[q];
        if ((fp < R(0) && fq > R(0)) || (fp > R(0) && fq < R(0))) {
            const R t = fp / (fp - fq);
            const R a = P.a[ip] + t * (P.a[q] - P.a[ip]), b = P.b[ip] + t * (P.b[q] - P.b[ip]);
            if (lo && lo->n < MAXP) { lo->a[lo->n] = a; lo->b[lo->n] = b; ++lo->n; }
            if (up && up->n < MAXP) { up->a[up->n] = a; up->b[up->n] = b; ++up->n; }
        }
        if (fq <= R(0) && lo && lo->n < MAXP) { lo->a[lo->n] = P.a[q]; lo->b[lo->n] = P.b[q]; ++lo->n; }
        if (fq >= R(0) && up && up->n < MAXP) { up->a[up->n] = P.a[q]; up->b[up->n] = P.b[q]; ++up->n; }
        fp = fq;
        ip = q;
    }
}

/* Twice the area and six times the first moments of a polygon in (a, b), added to A, M1, M2. */
template <class R>
SLVOF_HD void moments2(const Poly2<R>& P, R& A, R& M1, R& M2)
{
    if (P.n < 3) return;
    for (int q = 0; q < P.n; ++q) {
        const int r = q + 1 == P.n ? 0 : q + 1;
        const R c = P.a[q] * P.b[r] - P.a[r] * P.b[q];
        A += c;
        M1 += (P.a[q] + P.a[r]) * c;
        M2 += (P.b[q] + P.b[r]) * c;
    }
}

/* Liquid moments m[s] = int_{F ∩ L} lambda_s dA / |F| of the triangle F = (p[0], p[1], p[2])
 * (cell units) whose vertices lie in donor cells ind[s] (relative to the cell).  donor(a, b, c,
 * ph, px, py, pz, Dt) gives the phase code of donor (a, b, c) and, for ph == 0, its plane
 * px*x + py*y + pz*z - Dt in this frame (liquid below). */
template <class R, class Donor>
SLVOF_HD void face_moments(const R (&p)[3][3], const int (&ind)[3][3], const Donor& donor, R (&m)[3],
                           Poly2<R>* buf /* 7 polygons of workspace */)
{
    int lo[3], hi[3];
    R e1[3], e2[3];
    for (int q = 0; q < 3; ++q) {
        lo[q] = imin(ind[0][q], imin(ind[1][q], ind[2][q]));
        hi[q] = imax(ind[0][q], imax(ind[1][q], ind[2][q]));
        e1[q] = p[1][q] - p[0][q];
        e2[q] = p[2][q] - p[0][q];
    }
    Poly2<R>& X = buf[0]; /* remaining part below the current x plane */
    X.n = 3;
    X.a[0] = R(0); X.b[0] = R(0);
    X.a[1] = R(1); X.b[1] = R(0);
    X.a[2] = R(0); X.b[2] = R(1);
    R A = R(0), M1 = R(0), M2 = R(0);
    for (int a = hi[0]; a >= lo[0]; --a) {
        Poly2<R>* Px = &X;
        if (a > lo[0]) {
            split2(X, p[0][0] - R(a), e1[0], e2[0], &buf[6], &buf[1]);
            X = buf[6];
            Px = &buf[1];
        }
        if (Px->n < 3) continue;
        Poly2<R>& Y = buf[2];
        Y = *Px;
        for (int b = hi[1]; b >= lo[1]; --b) {
            Poly2<R>* Py = &Y;
            if (b > lo[1]) {
                split2(Y, p[0][1] - R(b), e1[1], e2[1], &buf[6], &buf[3]);
                Y = buf[6];
                Py = &buf[3];
            }
            if (Py->n < 3) continue;
            Poly2<R>& Z = buf[4];
            Z = *Py;
            for (int c = hi[2]; c >= lo[2]; --c) {
                Poly2<R>* Pz = &Z;
                if (c > lo[2]) {
                    split2(Z, p[0][2] - R(c), e1[2], e2[2], &buf[6], &buf[5]);
                    Z = buf[6];
                    Pz = &buf[5];
                }
                if (Pz->n < 3) continue;
                int ph;
                R px, py, pz, Dt;
                donor(a, b, c, ph, px, py, pz, Dt);
                if (ph > 0) {
                    moments2(*Pz, A, M1, M2);
                } else if (ph == 0) {
                    const R g0 = px * p[0][0] + py * p[0][1] + pz * p[0][2] - Dt;
                    const R g1 = px * e1[0] + py * e1[1] + pz * e1[2];
                    const R g2 = px * e2[0] + py * e2[1] + pz * e2[2];
                    split2(*Pz, g0, g1, g2, &buf[6], (Poly2<R>*)nullptr);
                    moments2(buf[6], A, M1, M2);
                }
            }
        }
    }
    m[1] = M1 / R(3);
    m[2] = M2 / R(3);
    m[0] = A - (M1 + M2) / R(3);
}

template <class R, class Donor>
SLVOF_HD void face_moments(const R (&p)[3][3], const int (&ind)[3][3], const Donor& donor, R (&m)[3])
{
    Poly2<R> buf[7];
    face_moments(p, ind, donor, m, buf);
}

/* Oriented area vector S_b = -3 dV/dv_b of the face opposite slot b of tet t (V the
 * reference's tet_vol, src/VFgeom.jl:669-681: -1/6 (v0-v3).((v1-v3)x(v2-v3))). */
template <class R>
SLVOF_HD void face_area(const R (&t)[4][3], int b, R (&S)[3])
{
    auto cr = [](const R* u, const R* w, R* o) {
        o[0] = u[1] * w[2] - u[2] * w[1];
        o[1] = u[2] * w[0] - u[0] * w[2];
        o[2] = u[0] * w[1] - u[1] * w[0];
    };
    R u[3], w[3], o[3];
    if (b == 3) {
        for (int q = 0; q < 3; ++q) { u[q] = t[1][q] - t[0][q]; w[q] = t[2][q] - t[0][q]; }
        cr(u, w, o);
        for (int q = 0; q < 3; ++q) S[q] = R(-0.5) * o[q];
        return;
    }
    const int i1 = b == 0 ? 1 : (b == 1 ? 2 : 0), i2 = b == 0 ? 2 : (b == 1 ? 0 : 1);
    for (int q = 0; q < 3; ++q) { u[q] = t[i1][q] - t[3][q]; w[q] = t[i2][q] - t[3][q]; }
    cr(u, w, o);
    for (int q = 0; q < 3; ++q) S[q] = R(0.5) * o[q];
}

/* Faces of a tessellation that belong to one tet only (the pre-image's boundary), as (tet,
 * opposite slot).  5_tets and 6_tets have 12, 24_tets 24. */
struct BFaces {
    int n;
    signed char t[24], b[24];
};

SLVOF_HD void face_ids(int tess, int t, int b, int (&id)[3])
{
    int n = 0;
    for (int s = 0; s < 4; ++s)
        if (s != b) id[n++] = tess_tet(tess, t, s);
    /* sorted, for comparison */
    if (id[0] > id[1]) { const int x = id[0]; id[0] = id[1]; id[1] = x; }
    if (id[1] > id[2]) { const int x = id[1]; id[1] = id[2]; id[2] = x; }
    if (id[0] > id[1]) { const int x = id[0]; id[0] = id[1]; id[1] = x; }
}

SLVOF_HD BFaces boundary_faces(int tess)
{
    BFaces F;
    F.n = 0;
    const int nt = tess_ntets(tess);
    for (int t = 0; t < nt; ++t)
        for (int b = 0; b < 4; ++b) {
            int id[3], cnt = 0;
            face_ids(tess, t, b, id);
            for (int t2 = 0; t2 < nt; ++t2)
                for (int b2 = 0; b2 < 4; ++b2) {
                    int i2[3];
                    face_ids(tess, t2, b2, i2);
                    cnt += (i2[0] == id[0] && i2[1] == id[1] && i2[2] == id[2]) ? 1 : 0;
                }
            if (cnt == 1 && F.n < 24) {
                F.t[F.n] = (signed char)t;
                F.b[F.n] = (signed char)b;
                ++F.n;
            }
        }
    return F;
}

/* Polygon of the plane px*x + py*y + pz*z = Dt inside tet t (vertex order around it); false
 * when the plane does not pass between the vertices. */
template <class R>
SLVOF_HD bool plane_tet(const R (&t)[4][3], R px, R py, R pz, R Dt, Poly3<R>& P)
{
    R d[4];
    int neg = 0;
    for (int n = 0; n < 4; ++n) {
        d[n] = px * t[n][0] + py * t[n][1] + pz * t[n][2] - Dt;
        neg += d[n] < R(0) ? 1 : 0;
    }
    P.n = 0;
    if (neg == 0 || neg == 4) return false;
    auto edge = [&](int u, int w) {
        const R s = d[u] / (d[u] - d[w]);
        P.x[P.n] = t[u][0] + s * (t[w][0] - t[u][0]);
        P.y[P.n] = t[u][1] + s * (t[w][1] - t[u][1]);
        P.z[P.n] = t[u][2] + s * (t[w][2] - t[u][2]);
        ++P.n;
    };
    if (neg == 1 || neg == 3) {
        const bool lone_neg = neg == 1;
        int l = 0;
        for (int n = 0; n < 4; ++n)
            if ((d[n] < R(0)) == lone_neg) l = n;
        for (int n = 0; n < 4; ++n)
            if (n != l) edge(l, n);
    } else {
        int a = -1, b = -1, c = -1, e = -1;
        for (int n = 0; n < 4; ++n) {
            if (d[n] < R(0)) { if (a < 0) a = n; else b = n; }
            else { if (c < 0) c = n; else e = n; }
        }
        edge(a, c); edge(a, e); edge(b, e); edge(b, c);
    }
    return true;
}

/* The part of a convex 3D polygon P with g = nx*x + ny*y + nz*z - off <= 0, into Q. */
template <class R>
SLVOF_HD void clip3(const Poly3<R>& P, Poly3<R>& Q, R nx, R ny, R nz, R off)
{
    Q.n = 0;
    if (P.n < 3) return;
    int ip = P.n - 1;
    R gp = nx * P.x[ip] + ny * P.y[ip] + nz * P.z[ip] - off;
    for (int q = 0; q < P.n; ++q) {
        const R gq = nx * P.x[q] + ny * P.y[q] + nz * P.z[q] - off;
        if (((gp < R(0) && gq > R(0)) || (gp > R(0) && gq < R(0))) && Q.n < MAXP) {
            const R s = gp / (gp - gq);
            Q.x[Q.n] = P.x[ip] + s * (P.x[q] - P.x[ip]);
            Q.y[Q.n] = P.y[ip] + s * (P.y[q] - P.y[ip]);
            Q.z[Q.n] = P.z[ip] + s * (P.z[q] - P.z[ip]);
            ++Q.n;
        }
        if (gq <= R(0) && Q.n < MAXP) { Q.x[Q.n] = P.x[q]; Q.y[Q.n] = P.y[q]; Q.z[Q.n] = P.z[q]; ++Q.n; }
        gp = gq;
        ip = q;
    }
}

/* Area (along the unit normal u) and first moment of a planar polygon, by a fan from its
 * first vertex; both change sign with the vertex order, their ratio is the centroid. */
template <class R>
SLVOF_HD void poly_area(const Poly3<R>& P, R ux, R uy, R uz, R& A, R (&M)[3])
{
    A = R(0);
    M[0] = M[1] = M[2] = R(0);
    for (int q = 1; q + 1 < P.n; ++q) {
        const R ax = P.x[q] - P.x[0], ay = P.y[q] - P.y[0], az = P.z[q] - P.z[0];
        const R bx = P.x[q + 1] - P.x[0], by = P.y[q + 1] - P.y[0], bz = P.z[q + 1] - P.z[0];
        const R a = R(0.5) * (ux * (ay * bz - az * by) + uy * (az * bx - ax * bz) + uz * (ax * by - ay * bx));
        A += a;
        M[0] += a * (P.x[0] + P.x[q] + P.x[q + 1]) / R(3);
        M[1] += a * (P.y[0] + P.y[q] + P.y[q + 1]) / R(3);
        M[2] += a * (P.z[0] + P.z[q] + P.z[q + 1]) / R(3);
    }
}

/* Area |A| and centroid C of the plane's polygon inside tet t and inside donor cell (a, b, c) of
 * the tet's donor index box lo..hi (cell units).  Only box faces between two indices of the box
 * cut: beyond the box's ends the donor extends, as cutTet assigns it. */
template <class R>
SLVOF_HD bool plane_piece(const R (&t)[4][3], const int (&lo)[3], const int (&hi)[3], int a, int b, int c, R px,
                          R py, R pz, R Dt, R& A, R (&C)[3], Poly3<R>* ws /* 2 polygons of workspace */)
{
    Poly3<R>* P = &ws[0];
    Poly3<R>* Q = &ws[1];
    if (!plane_tet(t, px, py, pz, Dt, *P)) return false;
    const int off[3] = {a, b, c};
    for (int q = 0; q < 3; ++q) {
        const R e0 = q == 0 ? R(1) : R(0), e1 = q == 1 ? R(1) : R(0), e2 = q == 2 ? R(1) : R(0);
        if (off[q] > lo[q]) {
            clip3(*P, *Q, -e0, -e1, -e2, -R(off[q]));
            Poly3<R>* x = P; P = Q; Q = x;
        }
        if (off[q] < hi[q]) {
            clip3(*P, *Q, e0, e1, e2, R(off[q] + 1));
            Poly3<R>* x = P; P = Q; Q = x;
        }
    }
    if (P->n < 3) return false;
    const R len = sqrt_of(px * px + py * py + pz * pz);
    if (!(len > R(0))) return false;
    R M[3];
    poly_area(*P, px / len, py / len, pz / len, A, M);
    if (A == R(0)) return false;
    for (int q = 0; q < 3; ++q) C[q] = M[q] / A;
    A = A < R(0) ? -A : A;
    return true;
}

/* Area and first moment (cell units, positive orientation) of the plane's polygon inside the
 * unit cube, from its pieces in the cube's five tets (tet5 on the unmirrored corners). */
template <class R>
SLVOF_HD void plane_cube(R px, R py, R pz, R Dt, R& A, R (&M)[3])
{
    A = R(0);
    M[0] = M[1] = M[2] = R(0);
    const R len = sqrt_of(px * px + py * py + pz * pz);
    if (!(len > R(0))) return;
    const R ux = px / len, uy = py / len, uz = pz / len;
    for (int t = 0; t < 5; ++t) {
        R tv[4][3];
        for (int n = 0; n < 4; ++n) {
            const int v = tet5(t, n);
            tv[n][0] = R(v & 1); tv[n][1] = R((v >> 1) & 1); tv[n][2] = R(v >> 2);
        }
        Poly3<R> P;
        if (!plane_tet(tv, px, py, pz, Dt, P)) continue;
        R a, mm[3];
        poly_area(P, ux, uy, uz, a, mm);
        const R s = a < R(0) ? R(-1) : R(1);
        A += s * a;
        for (int q = 0; q < 3; ++q) M[q] += s * mm[q];
    }
}

} // namespace sd
} // namespace slvof
