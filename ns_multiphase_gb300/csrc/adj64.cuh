/*
 * adj64.cuh — reverse-mode derivative of the FP64 SL-VOF step, one cell at a time.
 *
 * The forward step (src/Transport.jl:108-181, src/VF.jl:94-156, src/ELVIRA.jl:62-137) maps
 * (VF^n, face velocities) to VF^{n+1}.  Away from switches of discrete choices — the ELVIRA
 * candidate, the band, the cutTet case of each sub-tet, the donor cell of each vertex — it is
 * a smooth function, and these routines give its exact derivative in reverse mode:
 *
 *   SL update   VFnew = vLiq/vol over the clipped pre-image.  The clip tree of cutTet
 *               (src/VFgeom.jl:713-900) is walked once more, depth first, with an explicit
 *               stack; every leaf returns the derivative of its liquid volume with respect to
 *               its four vertices and its donor's plane (n, D), and every cut folds the
 *               derivatives of its new vertices (points on the cut edges, parameter mu) back
 *               onto the parent's vertices.  d(vol)/d(vertices) comes from the five uncut tets,
 *               whose volumes the pieces add up to.  The pre-image vertices go back through
 *               the RK stages of project! (src/Tools.jl:392-418) and the staggered trilinear
 *               interpolation (src/Tools.jl:500-641) to the face velocities.
 *   PLIC        D = computeDist(n, VF) is the inverse of the cut-cell volume fraction F(n, D)
 *               (computePLIC2VF, src/VF.jl:219-278), so dD = (dVF - dF/dn . dn) / (dF/dD);
 *               dF/d(n, D) is the same leaf derivative applied to the cell's own five tets.
 *   ELVIRA      the chosen candidate is c/|c| with c linear in the 3x3x3 VF block
 *               (src/ELVIRA.jl:62-115), a fixed linear map followed by the normalisation.
 *   ghost fills Neumann!/update_borders! copy cells (a source map); their reverse adds each
 *               copy's derivative to its source.
 *
 * Everything here is host/device code: the kernels in k_adj64.cu run it on the GPU, and a
 * host build checks it against finite differences of the CPU restatement.  The forward
 * recomputation inside (interpolation, project!, pt2index!, cutTet) keeps the operation
 * order of the FP64 forward path, so it sees the same pre-image and the same clip tree.
 */
#pragma once

#include <cmath>

#include "detmath.h"
#include "mesh_view.h"

namespace slvof {
namespace adj {

constexpr double EPS = 2.220446049250313e-16; /* Julia eps() */
constexpr int STACK = 12;                     /* cutTet nesting held per thread */
constexpr int MAX_LEAVES = 4096;              /* leaf budget of one top-level tet */
enum : int { E_INDEX = 1, E_DEPTH = 2, E_NAN = 4, E_VOLUME = 8 };

/* ---- memory access: read-only cache loads and atomic adds on the device ---------------- */
SLVOF_HD double ld(const double* p)
{
#if defined(__CUDA_ARCH__)
    return __ldg(p);
#else
    return *p;
#endif
}
SLVOF_HD void acc(double* p, double v)
{
#if defined(__CUDA_ARCH__)
    atomicAdd(p, v);
#else
    *p += v;
#endif
}

SLVOF_HD long ci(const DevMesh& m, int i, int j, int k)
{
    return (long)(i - m.lo) + (long)(j - m.lo) * m.cs1 + (long)(k - m.lo) * m.cs2;
}
SLVOF_HD long vi(const DevMesh& m, int i, int j, int k)
{
    return (long)(i - m.vlo) + (long)(j - m.vlo) * m.vs1 + (long)(k - m.vlo) * m.vs2;
}
SLVOF_HD double fc(const DevMesh& m, int q, int i) { return ld(m.f[q] + (i - m.lo)); }
SLVOF_HD double cc(const DevMesh& m, int q, int i) { return ld(m.c[q] + (i - m.lo)); }

/* Julia max/min on Float64 and the safe divide /^ (src/Tools.jl:375-377). */
SLVOF_HD double jmax(double a, double b)
{
    if (a != a || b != b) return a + b;
    return a > b ? a : (b > a ? b : (std::signbit(a) ? b : a));
}
SLVOF_HD double jmin(double a, double b)
{
    if (a != a || b != b) return a + b;
    return a < b ? a : (b < a ? b : (std::signbit(a) ? a : b));
}
SLVOF_HD double sdiv(double a, double b) { return fabs(b) <= EPS ? (double)INFINITY : a / b; }

/* d2case (src/VFgeom.jl:693-708) on a copy of d; 0-based case. */
SLVOF_HD int d2case(const double* d, int& err)
{
    double c[4] = {d[0], d[1], d[2], d[3]};
    int npos = 0, nneg = 0;
    for (int n = 0; n < 4; ++n) { npos += c[n] > 0.0; nneg += c[n] < 0.0; }
    int cs = 0;
    for (int n = 0; n < 4; ++n) {
        if (fabs(c[n]) < EPS) c[n] = npos > nneg ? EPS : -EPS;
        if (c[n] != c[n]) err |= E_NAN;
        cs += c[n] > 0.0 ? (1 << n) : 0;
    }
    return cs;
}

/* Edge parameter mu = min(1, max(0, -d1 /^ (d2 - d1))) (src/VFgeom.jl:787) and whether its
 * derivative is taken.  New vertices only sit on edges whose ends d2case puts on opposite
 * sides, so the clamp acts only when an end lies within eps of the plane (mu within about
 * eps of 0 or 1); there the clipped volume is still continuously differentiable (a vertex
 * crossing a plane changes it to third order) and its derivative is the one with mu free.
 * Only an edge lying in the plane (|d2 - d1| <= eps, mu = 1) has none. */
SLVOF_HD double edge_mu(double d1, double d2, bool& live)
{
    const double den = d2 - d1;
    const double q = sdiv(-d1, den);
    live = fabs(den) > EPS;
    return jmin(1.0, jmax(0.0, q));
}

/* tet_vol (src/VFgeom.jl:669-681) and w * its gradient added to g[4][3]. */
SLVOF_HD double tet_vol(const double* p0, const double* p1, const double* p2, const double* p3)
{
    const double a1 = p0[0] - p3[0], a2 = p0[1] - p3[1], a3 = p0[2] - p3[2];
    const double b1 = p1[0] - p3[0], b2 = p1[1] - p3[1], b3 = p1[2] - p3[2];
    const double c1 = p2[0] - p3[0], c2 = p2[1] - p3[1], c3 = p2[2] - p3[2];
    return -1.0 / 6.0 * ((a1 * (b2 * c3 - c2 * b3) - a2 * (b1 * c3 - c1 * b3)) + a3 * (b1 * c2 - c1 * b2));
}
SLVOF_HD void tet_vol_grad(const double* p0, const double* p1, const double* p2, const double* p3, double w,
                           double* g0, double* g1, double* g2, double* g3)
{
    const double a[3] = {p0[0] - p3[0], p0[1] - p3[1], p0[2] - p3[2]};
    const double b[3] = {p1[0] - p3[0], p1[1] - p3[1], p1[2] - p3[2]};
    const double c[3] = {p2[0] - p3[0], p2[1] - p3[1], p2[2] - p3[2]};
    const double s = -w / 6.0;
    const double bc[3] = {b[1] * c[2] - b[2] * c[1], b[2] * c[0] - b[0] * c[2], b[0] * c[1] - b[1] * c[0]};
    const double ca[3] = {c[1] * a[2] - c[2] * a[1], c[2] * a[0] - c[0] * a[2], c[0] * a[1] - c[1] * a[0]};
    const double ab[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    for (int q = 0; q < 3; ++q) {
        g0[q] += s * bc[q];
        g1[q] += s * ca[q];
        g2[q] += s * ab[q];
        g3[q] -= s * ((bc[q] + ca[q]) + ab[q]);
    }
}

/* oddEvenCell + cell2verts! (src/VFgeom.jl:171-216); returns tetsign (odd cells are
 * mirrored only by 5_tets). */
SLVOF_HD double cell_verts(const DevMesh& m, int i, int j, int k, double (*v)[3])
{
    const bool even = tess_even(m.tess, i, j, k);
    const int ia = even ? i : i + 1, ib = even ? i + 1 : i;
    const double xs[2] = {fc(m, 0, ia), fc(m, 0, ib)};
    const double ys[2] = {fc(m, 1, j), fc(m, 1, j + 1)};
    const double zs[2] = {fc(m, 2, k), fc(m, 2, k + 1)};
    for (int c = 0; c < 2; ++c)
        for (int b = 0; b < 2; ++b)
            for (int a = 0; a < 2; ++a) {
                double* p = v[a + 2 * b + 4 * c];
                p[0] = xs[a]; p[1] = ys[b]; p[2] = zs[c];
            }
    return even ? 1.0 : -1.0;
}

/* ---- staggered trilinear interpolation (get_velocity_{u,v,w}face, src/Tools.jl:500-641) -- */
struct Vel {
    const double *uf, *vf, *wf;
};
struct VelGrad {
    double *guf, *gvf, *gwf;
};

/* Coordinate q of the grid that is staggered (faces) in direction stag. */
SLVOF_HD double sco(const DevMesh& m, int stag, int d, int q) { return d == stag ? fc(m, d, q) : cc(m, d, q); }

struct Tri {
    int I[3];
    double w1[3], w2[3], ih[3]; /* weights and d(w1)/d(pt) */
};

SLVOF_HD void tri_locate(const DevMesh& m, int stag, const double* pt, int i, int j, int k, Tri& t)
{
    t.I[0] = i; t.I[1] = j; t.I[2] = k;
    for (int d = 0; d < 3; ++d) {
        while (pt[d] - sco(m, stag, d, t.I[d]) < 0.0 && t.I[d] > m.lo) t.I[d] -= 1;
        while (pt[d] - sco(m, stag, d, t.I[d] + 1) >= 0.0 && t.I[d] + 1 < m.hi[d]) t.I[d] += 1;
    }
    for (int d = 0; d < 3; ++d) {
        const double lo = sco(m, stag, d, t.I[d]), h = sco(m, stag, d, t.I[d] + 1) - lo;
        t.w1[d] = sdiv(pt[d] - lo, h);
        t.w2[d] = 1.0 - t.w1[d];
        t.ih[d] = fabs(h) <= EPS ? 0.0 : 1.0 / h;
    }
}

SLVOF_HD double tri_value(const DevMesh& m, const double* f, const Tri& t)
{
    const int a = t.I[0], b = t.I[1], c = t.I[2];
    const double* w1 = t.w1;
    const double* w2 = t.w2;
#define F_(ii, jj, kk) ld(f + ci(m, ii, jj, kk))
    return w1[2] * (w1[1] * (w1[0] * F_(a + 1, b + 1, c + 1) + w2[0] * F_(a, b + 1, c + 1)) +
                    w2[1] * (w1[0] * F_(a + 1, b, c + 1) + w2[0] * F_(a, b, c + 1))) +
           w2[2] * (w1[1] * (w1[0] * F_(a + 1, b + 1, c) + w2[0] * F_(a, b + 1, c)) +
                    w2[1] * (w1[0] * F_(a + 1, b, c) + w2[0] * F_(a, b, c)));
}

/* Reverse of one interpolation: gv times its derivative, to the eight face values (gf) and
 * to the point (gpt, may be null). */
SLVOF_HD void tri_reverse(const DevMesh& m, const double* f, double* gf, const Tri& t, double gv, double* gpt)
{
    if (gv == 0.0) return;
    const int a = t.I[0], b = t.I[1], c = t.I[2];
    double F[2][2][2];
    for (int z = 0; z < 2; ++z)
        for (int y = 0; y < 2; ++y)
            for (int x = 0; x < 2; ++x) F[z][y][x] = F_(a + x, b + y, c + z);
#undef F_
    const double wx[2] = {t.w2[0], t.w1[0]}, wy[2] = {t.w2[1], t.w1[1]}, wz[2] = {t.w2[2], t.w1[2]};
    for (int z = 0; z < 2; ++z)
        for (int y = 0; y < 2; ++y)
            for (int x = 0; x < 2; ++x) {
                const double w = (wx[x] * wy[y]) * wz[z];
                if (w != 0.0) acc(gf + ci(m, a + x, b + y, c + z), gv * w);
            }
    if (!gpt) return;
    double dx = 0.0, dy = 0.0, dz = 0.0;
    for (int z = 0; z < 2; ++z)
        for (int y = 0; y < 2; ++y) {
            dx += (wy[y] * wz[z]) * (F[z][y][1] - F[z][y][0]);
        }
    for (int z = 0; z < 2; ++z)
        for (int x = 0; x < 2; ++x) dy += (wx[x] * wz[z]) * (F[z][1][x] - F[z][0][x]);
    for (int y = 0; y < 2; ++y)
        for (int x = 0; x < 2; ++x) dz += (wx[x] * wy[y]) * (F[1][y][x] - F[0][y][x]);
    gpt[0] += gv * dx * t.ih[0];
    gpt[1] += gv * dy * t.ih[1];
    gpt[2] += gv * dz * t.ih[2];
}

/* velocity at pt (three staggered components), seeded at cell (i, j, k) */
SLVOF_HD void velocity(const DevMesh& m, const Vel& V, const double* pt, int i, int j, int k, double* out)
{
    Tri t;
    tri_locate(m, 0, pt, i, j, k, t);
    out[0] = tri_value(m, V.uf, t);
    tri_locate(m, 1, pt, i, j, k, t);
    out[1] = tri_value(m, V.vf, t);
    tri_locate(m, 2, pt, i, j, k, t);
    out[2] = tri_value(m, V.wf, t);
}

SLVOF_HD void velocity_reverse(const DevMesh& m, const Vel& V, const VelGrad& G, const double* pt, int i, int j, int k,
                               const double* gv, double* gpt)
{
    Tri t;
    tri_locate(m, 0, pt, i, j, k, t);
    tri_reverse(m, V.uf, G.guf, t, gv[0], gpt);
    tri_locate(m, 1, pt, i, j, k, t);
    tri_reverse(m, V.vf, G.gvf, t, gv[1], gpt);
    tri_locate(m, 2, pt, i, j, k, t);
    tri_reverse(m, V.wf, G.gwf, t, gv[2], gpt);
}

/* project! (src/Tools.jl:392-418): Euler (0), Midpoint (1), RK4 (2); velocity frozen in the
 * step.  Stage points x2..x4 are returned for the reverse pass. */
SLVOF_HD void project(const DevMesh& m, const Vel& V, double* pt, int i, int j, int k, double dt, double x[3][3])
{
    double v1[3], v2[3], v3[3], v4[3];
    if (m.projection == 3) {
        /* test_case == "Zalesak": exact rotation about (0.5, 0.5), src/Tools.jl:396-399 */
        const double a = 6.283185307179586 * dt;
        const double c = detm_cos(a), s = detm_sin(a);
        const double x0 = pt[0], y0 = pt[1];
        pt[0] = (0.5 + c * (x0 - 0.5)) + s * (y0 - 0.5);
        pt[1] = (0.5 - s * (x0 - 0.5)) + c * (y0 - 0.5);
        return;
    }
    if (m.projection == 2) {
        velocity(m, V, pt, i, j, k, v1);
        for (int d = 0; d < 3; ++d) x[0][d] = pt[d] - 0.5 * dt * v1[d];
        velocity(m, V, x[0], i, j, k, v2);
        for (int d = 0; d < 3; ++d) x[1][d] = pt[d] - 0.5 * dt * v2[d];
        velocity(m, V, x[1], i, j, k, v3);
        for (int d = 0; d < 3; ++d) x[2][d] = pt[d] - dt * v3[d];
        velocity(m, V, x[2], i, j, k, v4);
        for (int d = 0; d < 3; ++d) pt[d] = pt[d] + (-dt) / 6.0 * (((v1[d] + 2.0 * v2[d]) + 2.0 * v3[d]) + v4[d]);
    } else if (m.projection == 0) {
        velocity(m, V, pt, i, j, k, v1);
        for (int d = 0; d < 3; ++d) pt[d] = pt[d] + (-dt) * v1[d];
    } else {
        velocity(m, V, pt, i, j, k, v1);
        for (int d = 0; d < 3; ++d) x[0][d] = pt[d] - 0.5 * dt * v1[d];
        velocity(m, V, x[0], i, j, k, v2);
        for (int d = 0; d < 3; ++d) pt[d] = pt[d] + (-dt) * v2[d];
    }
}

/* Reverse of project!: gp = dL/d(projected point of the grid node p0) to the face velocities. */
SLVOF_HD void project_reverse(const DevMesh& m, const Vel& V, const VelGrad& G, const double* p0, int i, int j, int k,
                              double dt, const double* gp)
{
    if (m.projection == 3) return; /* the rotation does not depend on the velocities */
    double pt[3] = {p0[0], p0[1], p0[2]};
    double x[3][3];
    project(m, V, pt, i, j, k, dt, x);
    if (m.projection == 2) {
        const double s = (-dt) / 6.0;
        double g1[3], g2[3], g3[3], g4[3], gx[3];
        for (int d = 0; d < 3; ++d) { g1[d] = s * gp[d]; g2[d] = 2.0 * s * gp[d]; g3[d] = 2.0 * s * gp[d]; g4[d] = s * gp[d]; }
        gx[0] = gx[1] = gx[2] = 0.0;
        velocity_reverse(m, V, G, x[2], i, j, k, g4, gx); /* x4 = p0 - dt v3 */
        for (int d = 0; d < 3; ++d) { g3[d] += -dt * gx[d]; gx[d] = 0.0; }
        velocity_reverse(m, V, G, x[1], i, j, k, g3, gx); /* x3 = p0 - dt/2 v2 */
        for (int d = 0; d < 3; ++d) { g2[d] += -0.5 * dt * gx[d]; gx[d] = 0.0; }
        velocity_reverse(m, V, G, x[0], i, j, k, g2, gx); /* x2 = p0 - dt/2 v1 */
        for (int d = 0; d < 3; ++d) g1[d] += -0.5 * dt * gx[d];
        velocity_reverse(m, V, G, p0, i, j, k, g1, nullptr);
    } else if (m.projection == 0) {
        const double g1[3] = {-dt * gp[0], -dt * gp[1], -dt * gp[2]};
        velocity_reverse(m, V, G, p0, i, j, k, g1, nullptr);
    } else {
        const double g2[3] = {-dt * gp[0], -dt * gp[1], -dt * gp[2]};
        double gx[3] = {0.0, 0.0, 0.0};
        velocity_reverse(m, V, G, x[0], i, j, k, g2, gx);
        double g1[3];
        for (int d = 0; d < 3; ++d) g1[d] = -0.5 * dt * gx[d];
        velocity_reverse(m, V, G, p0, i, j, k, g1, nullptr);
    }
}

/* pt2index! (src/Tools.jl:424-434), bounded by the cell-array range. */
SLVOF_HD void pt2index(const DevMesh& m, int* I, const double* pt, int i, int j, int k, int& err)
{
    I[0] = i; I[1] = j; I[2] = k;
    for (int d = 0; d < 3; ++d) {
        while (pt[d] > fc(m, d, I[d] + 1) + EPS) {
            if (I[d] >= m.hi[d]) { err |= E_INDEX; break; }
            I[d] += 1;
        }
        while (pt[d] < fc(m, d, I[d]) - EPS) {
            if (I[d] <= m.lo) { err |= E_INDEX; break; }
            I[d] -= 1;
        }
    }
}

/* ---- PLIC leaf -------------------------------------------------------------------------
 * Leaf of cutTet (src/VFgeom.jl:757-830): the tet v[0..3] cut by the plane n.x = D, liquid on
 * the negative side.  Returns vol and vLiq; adds s * d(vLiq)/d(v) to gv and
 * s * d(vLiq)/d(nx, ny, nz, D) to gpl. */
SLVOF_HD void leaf(const CutCase* tab, const double v[4][3], double nx, double ny, double nz, double D, double s,
                   double& vol, double& vLiq, double gv[4][3], double* gpl, int& err)
{
    double vert[8][3], g8[8][3];
    double d[4];
    for (int n = 0; n < 4; ++n) {
        for (int p = 0; p < 3; ++p) vert[n][p] = v[n][p];
        d[n] = ((nx * vert[n][0] + ny * vert[n][1]) + nz * vert[n][2]) - D;
    }
    const int cs = d2case(d, err);
    const CutCase& C = tab[cs];
    double mu[4];
    bool live[4];
    for (int n = 0; n < C.nvert; ++n) {
        const int a = C.v1[n], b = C.v2[n];
        mu[n] = edge_mu(d[a], d[b], live[n]);
        for (int p = 0; p < 3; ++p) vert[4 + n][p] = (1.0 - mu[n]) * vert[a][p] + mu[n] * vert[b][p];
    }
    for (int n = 0; n < 8; ++n) g8[n][0] = g8[n][1] = g8[n][2] = 0.0;
    vol = 0.0;
    vLiq = 0.0;
    for (int t = C.ntets - 1; t >= C.nntet - 1; --t) {
        const int a = C.vtet[t][0], b = C.vtet[t][1], c = C.vtet[t][2], e = C.vtet[t][3];
        const double tv = tet_vol(vert[a], vert[b], vert[c], vert[e]);
        vol += tv;
        vLiq += tv;
        if (s != 0.0) tet_vol_grad(vert[a], vert[b], vert[c], vert[e], s, g8[a], g8[b], g8[c], g8[e]);
    }
    for (int t = 0; t < C.nntet - 1; ++t)
        vol += tet_vol(vert[C.vtet[t][0]], vert[C.vtet[t][1]], vert[C.vtet[t][2]], vert[C.vtet[t][3]]);
    if (s == 0.0) return;
    double gd[4] = {0.0, 0.0, 0.0, 0.0};
    for (int n = C.nvert - 1; n >= 0; --n) {
        const int a = C.v1[n], b = C.v2[n];
        double gmu = 0.0;
        for (int p = 0; p < 3; ++p) {
            g8[a][p] += (1.0 - mu[n]) * g8[4 + n][p];
            g8[b][p] += mu[n] * g8[4 + n][p];
            gmu += g8[4 + n][p] * (vert[b][p] - vert[a][p]);
        }
        if (live[n]) {
            const double e = d[b] - d[a], e2 = e * e;
            gd[a] += gmu * (-d[b] / e2);
            gd[b] += gmu * (d[a] / e2);
        }
    }
    for (int n = 0; n < 4; ++n) {
        gv[n][0] += g8[n][0] + gd[n] * nx;
        gv[n][1] += g8[n][1] + gd[n] * ny;
        gv[n][2] += g8[n][2] + gd[n] * nz;
        gpl[0] += gd[n] * vert[n][0];
        gpl[1] += gd[n] * vert[n][1];
        gpl[2] += gd[n] * vert[n][2];
        gpl[3] -= gd[n];
    }
}

/* ---- cutTet with its reverse pass -------------------------------------------------------- */
struct Plic {
    const double *nx, *ny, *nz, *D;  /* donor planes (border-updated, every cell) */
    double *gnx, *gny, *gnz, *gD;    /* their derivatives, accumulated */
    const signed char* phase;        /* +1/-1: the plane puts the whole domain on one side; may be null */
};

/* One cut level: parent vertices 0-3 and the new vertices 4-7 on the mesh plane, the
 * derivatives gathered from the children, the parent's plane distances, the side-0 cell
 * indices of all eight vertices, and the children's running sums. */
struct Frame {
    double v[8][3];
    double g[8][3];
    double d[4];
    double vol, vLiq;
    int ind[8][3];
    int cs, next, dir, cut, flags;
};

SLVOF_HD void form_child(const CutCase* tab, const Frame& F, int c, double cv[4][3], int cind[4][3])
{
    const CutCase& C = tab[F.cs];
    const int side = C.side[c];
    for (int nn = 0; nn < 4; ++nn) {
        const int vt = C.vtet[c][nn];
        for (int p = 0; p < 3; ++p) {
            cv[nn][p] = F.v[vt][p];
            cind[nn][p] = F.ind[vt][p];
        }
        if (side == 1) cind[nn][F.dir] = F.cut;
    }
}

/* +1 when every one of the np points is strictly on the liquid side of the PLIC plane of
 * every donor cell of the index box [lo, hi] (at most 2x2x2 cells), -1 when strictly on the gas
 * side of every one, 0 otherwise.  Every cutTet leaf of a (sub-)tet with such points is then
 * the one-tet case 1 (or 16), whatever the mesh cuts: its liquid volume is its own volume (or
 * 0) for every nearby position of the points. */
SLVOF_HD int points_side(const DevMesh& m, const Plic& P, const double (*v)[3], int np, const int* lo, const int* hi)
{
    for (int q = 0; q < 3; ++q)
        if (hi[q] - lo[q] > 1) return 0;
    int side = 2;
    for (int c = lo[2]; c <= hi[2]; ++c)
        for (int b = lo[1]; b <= hi[1]; ++b)
            for (int a = lo[0]; a <= hi[0]; ++a) {
                const long o = ci(m, a, b, c);
                const double nx = ld(P.nx + o), ny = ld(P.ny + o), nz = ld(P.nz + o), D = ld(P.D + o);
                bool neg = true, pos = true;
                for (int n = 0; n < np; ++n) {
                    const double d = ((nx * v[n][0] + ny * v[n][1]) + nz * v[n][2]) - D;
                    neg = neg && d < 0.0;
                    pos = pos && d > 0.0;
                }
                const int sd = neg ? 1 : (pos ? -1 : 0);
                if (sd == 0 || (side != 2 && sd != side)) return 0;
                side = sd;
            }
    return side;
}

/* The same decision from the donors' phase codes alone (pure donors whose plane puts every
 * point of the domain on one side): +1 / -1 when every donor of the node's index box (at most
 * 2x2x2) is pure of that phase, 0 otherwise.  Cheap (byte loads), so it is tried at every
 * node of the clip tree. */
SLVOF_HD int node_phase(const DevMesh& m, const Plic& P, const int ind[4][3])
{
    if (!P.phase || !m.fast_pure) return 0;
    int lo[3], hi[3];
    for (int q = 0; q < 3; ++q) {
        lo[q] = hi[q] = ind[0][q];
        for (int n = 1; n < 4; ++n) {
            lo[q] = ind[n][q] < lo[q] ? ind[n][q] : lo[q];
            hi[q] = ind[n][q] > hi[q] ? ind[n][q] : hi[q];
        }
        if (hi[q] - lo[q] > 1) return 0;
    }
    int ph = 2;
    for (int c = lo[2]; c <= hi[2]; ++c)
        for (int b = lo[1]; b <= hi[1]; ++b)
            for (int a = lo[0]; a <= hi[0]; ++a) {
                const int p = P.phase[ci(m, a, b, c)];
                if (p == 0 || (ph != 2 && p != ph)) return 0;
                ph = p;
            }
    return ph;
}

/* Whole pre-image (8 vertices, their cells) one-sided: VF is 1 (or 0) for every nearby input
 * and the derivative of the cell's update is zero. */
SLVOF_HD bool preimage_one_sided(const DevMesh& m, const Plic& P, const double vt[8][3], const int vind[8][3])
{
    if (!m.fast_pure) return false;
    int lo[3], hi[3];
    for (int q = 0; q < 3; ++q) {
        lo[q] = hi[q] = vind[0][q];
        for (int n = 1; n < 8; ++n) {
            lo[q] = vind[n][q] < lo[q] ? vind[n][q] : lo[q];
            hi[q] = vind[n][q] > hi[q] ? vind[n][q] : hi[q];
        }
    }
    return points_side(m, P, vt, 8, lo, hi) != 0;
}

/* Leaf kinds seen by a clip, OR-ed into `kinds`: liquid and gas one-sided nodes, and PLIC
 * leaves.  A pre-image whose leaves are all one-sided of one phase has VF = 1 (or 0) for every
 * nearby input: its derivative is zero. */
enum : int { LEAF_LIQ = 1, LEAF_GAS = 2, LEAF_CUT = 4 };

/* cutTet (src/VFgeom.jl:713-900) of one top-level tet of a pre-image, then its reverse:
 * returns the tet's vol and vLiq, adds s * d(vLiq)/d(tet vertices) to gtet and
 * s * d(vLiq)/d(donor planes) to the plane derivatives.  Nodes whose donors are all pure of
 * one phase (node_phase) are single leaves; the summation tree therefore differs from the
 * forward's, the value only by rounding and the derivative not at all. */
SLVOF_HD void clip(const DevMesh& m, const CutCase* tab, const Plic& P, const double tet[4][3], const int ind[4][3],
                   double s, Frame* st, double& vol_out, double& liq_out, double gtet[4][3], int& kinds, int& err)
{
    double cv[4][3];
    int cind[4][3];
    for (int n = 0; n < 4; ++n)
        for (int p = 0; p < 3; ++p) { cv[n][p] = tet[n][p]; cind[n][p] = ind[n][p]; }
    int flags = 0, depth = 0, leaves = 0;
    double rvol = 0.0, rliq = 0.0, rg[4][3];
    for (;;) {
        const int side = node_phase(m, P, cind);
        if (side != 0) {
            if (++leaves > MAX_LEAVES) {
                err |= E_DEPTH;
                vol_out = liq_out = 0.0;
                for (int n = 0; n < 4; ++n) gtet[n][0] = gtet[n][1] = gtet[n][2] = 0.0;
                return;
            }
            for (int n = 0; n < 4; ++n) rg[n][0] = rg[n][1] = rg[n][2] = 0.0;
            rvol = tet_vol(cv[0], cv[1], cv[2], cv[3]);
            rliq = side > 0 ? rvol : 0.0;
            if (side > 0 && s != 0.0) tet_vol_grad(cv[0], cv[1], cv[2], cv[3], s, rg[0], rg[1], rg[2], rg[3]);
            kinds |= side > 0 ? LEAF_LIQ : LEAF_GAS;
        }
        int dir = -1, cut = 0;
        if (side == 0) {
            for (int q = 0; q < 3; ++q) {
                if (flags & (1 << q)) continue;
                int mx = cind[0][q], mn = cind[0][q];
                for (int n = 1; n < 4; ++n) {
                    mx = cind[n][q] > mx ? cind[n][q] : mx;
                    mn = cind[n][q] < mn ? cind[n][q] : mn;
                }
                if (mx > mn) { dir = q; cut = mx; break; }
                flags |= 1 << q;
            }
            if (dir >= 0 && depth == STACK) { err |= E_DEPTH; dir = -1; }
        }
        if (side != 0) {
            /* one-sided node: finished above */
        } else if (dir < 0) {
            for (int n = 0; n < 4; ++n) rg[n][0] = rg[n][1] = rg[n][2] = 0.0;
            if (++leaves > MAX_LEAVES) {
                err |= E_DEPTH;
                vol_out = liq_out = 0.0;
                for (int n = 0; n < 4; ++n) gtet[n][0] = gtet[n][1] = gtet[n][2] = 0.0;
                return;
            }
            const long c = ci(m, cind[0][0], cind[0][1], cind[0][2]);
            double gpl[4] = {0.0, 0.0, 0.0, 0.0};
            leaf(tab, cv, ld(P.nx + c), ld(P.ny + c), ld(P.nz + c), ld(P.D + c), s, rvol, rliq, rg, gpl, err);
            kinds |= LEAF_CUT;
            if (gpl[0] != 0.0) acc(P.gnx + c, gpl[0]);
            if (gpl[1] != 0.0) acc(P.gny + c, gpl[1]);
            if (gpl[2] != 0.0) acc(P.gnz + c, gpl[2]);
            if (gpl[3] != 0.0) acc(P.gD + c, gpl[3]);
        } else {
            /* cut by the mesh plane x_dir = face(cut) (src/VFgeom.jl:832-899) */
            Frame& F = st[depth];
            const double pl = fc(m, dir, cut);
            for (int n = 0; n < 4; ++n) {
                for (int p = 0; p < 3; ++p) {
                    F.v[n][p] = cv[n][p];
                    F.ind[n][p] = cind[n][p];
                }
                F.ind[n][dir] = cind[n][dir] < cut - 1 ? cind[n][dir] : cut - 1;
                F.d[n] = cv[n][dir] - pl;
            }
            const int cs = d2case(F.d, err);
            const CutCase& C = tab[cs];
            for (int n = 0; n < C.nvert; ++n) {
                const int a = C.v1[n], b = C.v2[n];
                bool live;
                const double mu = edge_mu(F.d[a], F.d[b], live);
                for (int p = 0; p < 3; ++p) F.v[4 + n][p] = (1.0 - mu) * F.v[a][p] + mu * F.v[b][p];
                int I[3];
                pt2index(m, I, F.v[4 + n], F.ind[n][0], F.ind[n][1], F.ind[n][2], err);
                for (int p = 0; p < 3; ++p) {
                    const int lo = F.ind[a][p] < F.ind[b][p] ? F.ind[a][p] : F.ind[b][p];
                    const int hi = F.ind[a][p] > F.ind[b][p] ? F.ind[a][p] : F.ind[b][p];
                    int val = I[p] > lo ? I[p] : lo;
                    val = val < hi ? val : hi;
                    F.ind[4 + n][p] = val;
                }
                F.ind[4 + n][dir] = cut - 1;
            }
            for (int n = 0; n < 8; ++n) F.g[n][0] = F.g[n][1] = F.g[n][2] = 0.0;
            F.vol = 0.0;
            F.vLiq = 0.0;
            F.cs = cs;
            F.dir = dir;
            F.cut = cut;
            F.flags = flags;
            F.next = 1;
            ++depth;
            form_child(tab, F, 0, cv, cind);
            continue;
        }
        /* return the finished node to its parent; finish parents whose children are done */
        for (;;) {
            if (depth == 0) {
                vol_out = rvol;
                liq_out = rliq;
                for (int n = 0; n < 4; ++n)
                    for (int p = 0; p < 3; ++p) gtet[n][p] = rg[n][p];
                return;
            }
            Frame& F = st[depth - 1];
            const CutCase& C = tab[F.cs];
            const int child = F.next - 1;
            F.vol += rvol;
            F.vLiq += rliq;
            for (int nn = 0; nn < 4; ++nn) {
                const int vt = C.vtet[child][nn];
                for (int p = 0; p < 3; ++p) F.g[vt][p] += rg[nn][p];
            }
            if (F.next < C.ntets) {
                form_child(tab, F, F.next, cv, cind);
                F.next += 1;
                flags = F.flags;
                break;
            }
            /* new vertices back onto the parent's vertices; the mesh plane is fixed */
            for (int n = C.nvert - 1; n >= 0; --n) {
                const int a = C.v1[n], b = C.v2[n];
                bool live;
                const double mu = edge_mu(F.d[a], F.d[b], live);
                double gmu = 0.0;
                for (int p = 0; p < 3; ++p) {
                    F.g[a][p] += (1.0 - mu) * F.g[4 + n][p];
                    F.g[b][p] += mu * F.g[4 + n][p];
                    gmu += F.g[4 + n][p] * (F.v[b][p] - F.v[a][p]);
                }
                if (live) {
                    const double e = F.d[b] - F.d[a], e2 = e * e;
                    F.g[a][F.dir] += gmu * (-F.d[b] / e2);
                    F.g[b][F.dir] += gmu * (F.d[a] / e2);
                }
            }
            rvol = F.vol;
            rliq = F.vLiq;
            for (int n = 0; n < 4; ++n)
                for (int p = 0; p < 3; ++p) rg[n][p] = F.g[n][p];
            --depth;
        }
    }
}

/* ---- one SL cell ----------------------------------------------------------------------- */
/* Weight of point `id` of a cell's tessellation in vertex v (0..7): 1 for the vertex itself,
 * 1/8 for the cell's mean point, 1/4 for the mean point of a face that holds v (24_tets). */
SLVOF_HD double point_weight(int id, int v)
{
    if (id == v) return 1.0;
    if (id == 8) return 0.125;
    if (id >= 9) {
        const int f = id - 9;
        for (int n = 0; n < 4; ++n)
            if (face24(f, n) == v) return 0.25;
    }
    return 0.0;
}

/* VFnew of a cell from its pre-image points p (tessellation order: vertices, then for 24_tets
 * the mean points computed from them) and their cells, and g * d(VFnew)/d(vertices) added to
 * gvt[8] (the mean points' derivatives distributed to the vertices they average), plus
 * g * d(VFnew)/d(donor planes). */
SLVOF_HD double sl_vertices(const DevMesh& m, const CutCase* tab, const Plic& P, double tetsign, const double (*p)[3],
                            const int (*pind)[3], double g, Frame* st, double gvt[8][3], int& err)
{
    const int tess = m.tess, nt = tess_ntets(tess);
    /* pre-image volume from the uncut tets (the pieces add up to it) */
    double volu = 0.0;
    for (int t = 0; t < nt; ++t)
        volu += tetsign * tet_vol(p[tess_tet(tess, t, 0)], p[tess_tet(tess, t, 1)], p[tess_tet(tess, t, 2)],
                                  p[tess_tet(tess, t, 3)]);
    const double s = (g != 0.0 && volu != 0.0) ? tetsign * g / volu : 0.0;
    double vol = 0.0, vLiq = 0.0;
    double gsum[15][3];
    for (int n = 0; n < 15; ++n) gsum[n][0] = gsum[n][1] = gsum[n][2] = 0.0;
    int kinds = 0;
    for (int t = 0; t < nt; ++t) {
        double tet[4][3], gtet[4][3];
        int ind[4][3];
        for (int n = 0; n < 4; ++n)
            for (int q = 0; q < 3; ++q) {
                tet[n][q] = p[tess_tet(tess, t, n)][q];
                ind[n][q] = pind[tess_tet(tess, t, n)][q];
            }
        double rv, rl;
        clip(m, tab, P, tet, ind, s, st, rv, rl, gtet, kinds, err);
        vol += tetsign * rv;
        vLiq += tetsign * rl;
        for (int n = 0; n < 4; ++n)
            for (int q = 0; q < 3; ++q) gsum[tess_tet(tess, t, n)][q] += gtet[n][q];
    }
    if (!(vol > 0.0) || !std::isfinite(vol)) err |= E_VOLUME;
    const double VF = vLiq / vol;
    /* all leaves one-sided of one phase: VF is 1 (or 0) around this input, derivative zero */
    if (s == 0.0 || kinds == LEAF_LIQ || kinds == LEAF_GAS) return VF;
    /* d(VF)/d(vol) part: -g VF / vol times d(vol)/d(points) */
    const double w = -g * VF / vol;
    for (int t = 0; t < nt; ++t) {
        const int a = tess_tet(tess, t, 0), b = tess_tet(tess, t, 1), c = tess_tet(tess, t, 2), e = tess_tet(tess, t, 3);
        tet_vol_grad(p[a], p[b], p[c], p[e], w * tetsign, gsum[a], gsum[b], gsum[c], gsum[e]);
    }
    for (int id = 0; id < tess_npoints(tess); ++id)
        for (int v = 0; v < 8; ++v) {
            const double wgt = point_weight(id, v);
            if (wgt != 0.0)
                for (int q = 0; q < 3; ++q) gvt[v][q] += wgt * gsum[id][q];
        }
    return VF;
}

/* Reverse of the SL update of cell (i, j, k) (src/Transport.jl:111-148, cell2tets! with
 * projected vertices, src/VFgeom.jl:345-420): g = dL/dVFnew.  Adds dL/d(face velocities)
 * and dL/d(donor planes); returns VFnew.  st holds STACK frames. */
SLVOF_HD double sl_cell(const DevMesh& m, const CutCase* tab, const Vel& V, const VelGrad& GV, const Plic& P, double dt,
                        int i, int j, int k, double g, Frame* st, int& err)
{
    double p0[8][3], p[15][3], gvt[8][3];
    const double tetsign = cell_verts(m, i, j, k, p0);
    int pind[15][3];
    for (int n = 0; n < 8; ++n) {
        double x[3][3];
        for (int q = 0; q < 3; ++q) { p[n][q] = p0[n][q]; gvt[n][q] = 0.0; }
        project(m, V, p[n], i, j, k, dt, x);
    }
    tess_means<double>(m.tess, p);
    for (int n = 0; n < tess_npoints(m.tess); ++n) pt2index(m, pind[n], p[n], i, j, k, err);
    const double VF = sl_vertices(m, tab, P, tetsign, p, pind, g, st, gvt, err);
    if (g == 0.0) return VF;
    for (int n = 0; n < 8; ++n)
        if (gvt[n][0] != 0.0 || gvt[n][1] != 0.0 || gvt[n][2] != 0.0)
            project_reverse(m, V, GV, p0[n], i, j, k, dt, gvt[n]);
    return VF;
}

/* ---- the finite-difference scheme's flux-correction tets ------------------------------------
 * add_correction_tets (src/VFgeom.jl:514-664, 5_tets): on each face of a band cell two tets
 * (a,b,d,e), (b,c,d,e) over the quad a,b,c,d of the face's projected flux-volume nodes, whose
 * apex e is the quad's mean moved along the face normal by 6 (vol - V(mean)) / N, with
 * vol = +-(dt * area * face velocity - SLfluxVol) and N the normal component of
 * a x b + d x a + b x c + c x d.  Their clipped volumes join the cell's sums. */

/* The finite-difference path calls the clip, project! and their reverses from several places
 * per cell; these are compiled once as calls instead of being inlined at every site. */
#if defined(__CUDACC__)
/* static: each translation unit that includes this header keeps its own copy */
#define SLVOF_HD_CALL static __host__ __device__ __noinline__
#else
#define SLVOF_HD_CALL inline
#endif
SLVOF_HD_CALL void clip_call(const DevMesh& m, const CutCase* tab, const Plic& P, const double tet[4][3],
                             const int ind[4][3], double s, Frame* st, double& vol_out, double& liq_out,
                             double gtet[4][3], int& kinds, int& err)
{
    clip(m, tab, P, tet, ind, s, st, vol_out, liq_out, gtet, kinds, err);
}
SLVOF_HD_CALL void project_call(const DevMesh& m, const Vel& V, double* pt, int i, int j, int k, double dt)
{
    double x[3][3];
    project(m, V, pt, i, j, k, dt, x);
}
SLVOF_HD_CALL void project_reverse_call(const DevMesh& m, const Vel& V, const VelGrad& G, const double* p0, int i,
                                        int j, int k, double dt, const double* gp)
{
    project_reverse(m, V, G, p0, i, j, k, dt, gp);
}

/* One face's flux volume, target volume and apex, as the forward builds them. */
struct CorrFace {
    double fv[8][3]; /* flux-volume nodes */
    double mean[3], e[3];
    double A, sgn, vol, v0, N; /* dt * face area, +-1 (oddEvenCell of the face's cell) */
    int dir, fi, fj, fk;
    bool even;
};

/* Face f (x-, x+, y-, y+, z-, z+) of cell (i, j, k). */
SLVOF_HD_CALL void corr_face(const DevMesh& m, const Vel& V, int i, int j, int k, double dt, int f, CorrFace& C)
{
    const int dir = f >> 1, up = f & 1;
    C.dir = dir;
    C.fi = i + (dir == 0 ? up : 0);
    C.fj = j + (dir == 1 ? up : 0);
    C.fk = k + (dir == 2 ? up : 0);
    C.even = tess_even(m.tess, C.fi, C.fj, C.fk);
    C.sgn = C.even ? 1.0 : -1.0;
    for (int n = 0; n < 8; ++n) {
        int off[3];
        const bool proj = flux_node(dir, C.even, n, off);
        C.fv[n][0] = fc(m, 0, C.fi + off[0]);
        C.fv[n][1] = fc(m, 1, C.fj + off[1]);
        C.fv[n][2] = fc(m, 2, C.fk + off[2]);
        if (proj) project_call(m, V, C.fv[n], C.fi, C.fj, C.fk, dt);
    }
    double flux = 0.0; /* tets_vol, src/VFgeom.jl:683-689 */
    for (int t = 0; t < tess_ntets(m.tess); ++t)
        flux += tet_vol(C.fv[tess_tet(m.tess, t, 0)], C.fv[tess_tet(m.tess, t, 1)], C.fv[tess_tet(m.tess, t, 2)],
                        C.fv[tess_tet(m.tess, t, 3)]);
    flux = flux * C.sgn;
    const long t = ci(m, C.fi, C.fj, C.fk);
    C.A = dir == 0 ? (dt * m.d[1]) * m.d[2] : (dir == 1 ? (dt * m.d[0]) * m.d[2] : (dt * m.d[0]) * m.d[1]);
    const double divg = C.A * ld((dir == 0 ? V.uf : (dir == 1 ? V.vf : V.wf)) + t);
    C.vol = C.even ? (divg - flux) : -(divg - flux);
    const double *a = C.fv[flux_quad(dir, C.even, 0)], *b = C.fv[flux_quad(dir, C.even, 1)],
                 *c = C.fv[flux_quad(dir, C.even, 2)], *d = C.fv[flux_quad(dir, C.even, 3)];
    for (int p = 0; p < 3; ++p) {
        C.mean[p] = 0.25 * (((a[p] + b[p]) + c[p]) + d[p]);
        C.e[p] = C.mean[p];
    }
    C.v0 = tet_vol(a, b, d, C.e) + tet_vol(b, c, d, C.e);
    const int p1 = (dir + 1) % 3, p2 = (dir + 2) % 3;
    C.N = (((a[p1] * b[p2] - a[p2] * b[p1]) + (d[p1] * a[p2] - d[p2] * a[p1])) + (b[p1] * c[p2] - b[p2] * c[p1])) +
          (c[p1] * d[p2] - c[p2] * d[p1]);
    C.e[dir] += 6.0 * (C.vol - C.v0) / C.N;
}

/* Tet h (0: a,b,d,e; 1: b,c,d,e) of a face. */
SLVOF_HD void corr_tet(const CorrFace& C, int h, double tet[4][3])
{
    const int q0 = flux_quad(C.dir, C.even, h), q1 = flux_quad(C.dir, C.even, h + 1),
              q3 = flux_quad(C.dir, C.even, 3);
    for (int p = 0; p < 3; ++p) {
        tet[0][p] = C.fv[q0][p];
        tet[1][p] = C.fv[q1][p];
        tet[2][p] = C.fv[q3][p];
        tet[3][p] = C.e[p];
    }
}

/* Reverse of a face: gT[h][n] = dL/d(vertex n of tet h) to the face velocity of the target
 * volume and, through the quad, the apex and the flux volume, to the projected nodes. */
SLVOF_HD_CALL void corr_face_reverse(const DevMesh& m, const Vel& V, const VelGrad& G, double dt, const CorrFace& C,
                                const double (*gT)[4][3])
{
    const int dir = C.dir, p1 = (dir + 1) % 3, p2 = (dir + 2) % 3;
    const int qa = flux_quad(dir, C.even, 0), qb = flux_quad(dir, C.even, 1), qc = flux_quad(dir, C.even, 2),
              qd = flux_quad(dir, C.even, 3);
    const double *a = C.fv[qa], *b = C.fv[qb], *c = C.fv[qc], *d = C.fv[qd];
    double ga[3], gb[3], gc[3], gd[3], gm[3];
    for (int p = 0; p < 3; ++p) {
        ga[p] = gT[0][0][p];
        gb[p] = gT[0][1][p] + gT[1][0][p];
        gc[p] = gT[1][1][p];
        gd[p] = gT[0][2][p] + gT[1][2][p];
        gm[p] = gT[0][3][p] + gT[1][3][p]; /* e = mean + (shift along dir) */
    }
    const double se = gm[dir];
    const double gvol = 6.0 * se / C.N, gv0 = -gvol, gN = -6.0 * se * (C.vol - C.v0) / (C.N * C.N);
    /* v0 = V(a, b, d, mean) + V(b, c, d, mean) */
    tet_vol_grad(a, b, d, C.mean, gv0, ga, gb, gd, gm);
    tet_vol_grad(b, c, d, C.mean, gv0, gb, gc, gd, gm);
    /* N = cr(a, b) + cr(d, a) + cr(b, c) + cr(c, d), cr(u, w) = u[p1] w[p2] - u[p2] w[p1] */
    auto crg = [&](const double* u, const double* w, double* gu, double* gw) {
        gu[p1] += gN * w[p2];
        gu[p2] -= gN * w[p1];
        gw[p2] += gN * u[p1];
        gw[p1] -= gN * u[p2];
    };
    crg(a, b, ga, gb);
    crg(d, a, gd, ga);
    crg(b, c, gb, gc);
    crg(c, d, gc, gd);
    double gfv[8][3];
    for (int n = 0; n < 8; ++n) gfv[n][0] = gfv[n][1] = gfv[n][2] = 0.0;
    for (int p = 0; p < 3; ++p) {
        gfv[qa][p] += ga[p] + 0.25 * gm[p];
        gfv[qb][p] += gb[p] + 0.25 * gm[p];
        gfv[qc][p] += gc[p] + 0.25 * gm[p];
        gfv[qd][p] += gd[p] + 0.25 * gm[p];
    }
    /* vol = sgn (A U - flux), flux = sgn * sum of the flux volume's tet volumes */
    const long t = ci(m, C.fi, C.fj, C.fk);
    acc((dir == 0 ? G.guf : (dir == 1 ? G.gvf : G.gwf)) + t, gvol * C.sgn * C.A);
    const double gsum = -gvol * C.sgn * C.sgn;
    for (int q = 0; q < tess_ntets(m.tess); ++q) {
        const int n0 = tess_tet(m.tess, q, 0), n1 = tess_tet(m.tess, q, 1), n2 = tess_tet(m.tess, q, 2),
                  n3 = tess_tet(m.tess, q, 3);
        tet_vol_grad(C.fv[n0], C.fv[n1], C.fv[n2], C.fv[n3], gsum, gfv[n0], gfv[n1], gfv[n2], gfv[n3]);
    }
    for (int n = 0; n < 8; ++n) {
        int off[3];
        if (!flux_node(dir, C.even, n, off)) continue;
        if (gfv[n][0] == 0.0 && gfv[n][1] == 0.0 && gfv[n][2] == 0.0) continue;
        const double p0[3] = {fc(m, 0, C.fi + off[0]), fc(m, 1, C.fj + off[1]), fc(m, 2, C.fk + off[2])};
        project_reverse_call(m, V, G, p0, C.fi, C.fj, C.fk, dt, gfv[n]);
    }
}

/* Reverse of the SL update of band cell (i, j, k) under pressure_scheme "finite-difference"
 * (src/Transport.jl:111-148 with add_correction_tets, src/Transport.jl:121-124): the cell's
 * five tets and the twelve correction tets (vertex cells by pt2index! seeded at the cell), all
 * clipped and their sums divided; g = dL/dVFnew.  Adds dL/d(face velocities) and
 * dL/d(donor planes); returns VFnew. */
SLVOF_HD double sl_cell_fd(const DevMesh& m, const CutCase* tab, const Vel& V, const VelGrad& GV, const Plic& P,
                           double dt, int i, int j, int k, double g, Frame* st, int& err)
{
    double p0[8][3], p[8][3], gvt[8][3];
    const double tetsign = cell_verts(m, i, j, k, p0);
    int pind[8][3];
    for (int n = 0; n < 8; ++n) {
        for (int q = 0; q < 3; ++q) { p[n][q] = p0[n][q]; gvt[n][q] = 0.0; }
        project_call(m, V, p[n], i, j, k, dt);
        pt2index(m, pind[n], p[n], i, j, k, err);
    }
    const int nt = tess_ntets(m.tess);
    /* the six faces' flux volumes and apexes, formed once (each traces its face's four
     * corners) and used by the volume, the clips and the reverse below */
    CorrFace CF[6];
    for (int f = 0; f < 6; ++f) corr_face(m, V, i, j, k, dt, f, CF[f]);
    /* the uncut volume, which the clipped pieces add up to */
    double volu = 0.0;
    for (int t = 0; t < nt; ++t)
        volu += tetsign * tet_vol(p[tess_tet(m.tess, t, 0)], p[tess_tet(m.tess, t, 1)], p[tess_tet(m.tess, t, 2)],
                                  p[tess_tet(m.tess, t, 3)]);
    for (int f = 0; f < 6; ++f) {
        const CorrFace& C = CF[f];
        for (int h = 0; h < 2; ++h) {
            double tet[4][3];
            corr_tet(C, h, tet);
            volu += tetsign * tet_vol(tet[0], tet[1], tet[2], tet[3]);
        }
    }
    const double s = (g != 0.0 && volu != 0.0) ? tetsign * g / volu : 0.0;
    double vol = 0.0, vLiq = 0.0;
    int kinds = 0;
    for (int t = 0; t < nt; ++t) {
        double tet[4][3], gtet[4][3];
        int ind[4][3];
        for (int n = 0; n < 4; ++n)
            for (int q = 0; q < 3; ++q) {
                tet[n][q] = p[tess_tet(m.tess, t, n)][q];
                ind[n][q] = pind[tess_tet(m.tess, t, n)][q];
            }
        double rv, rl;
        clip_call(m, tab, P, tet, ind, s, st, rv, rl, gtet, kinds, err);
        vol += tetsign * rv;
        vLiq += tetsign * rl;
        for (int n = 0; n < 4; ++n)
            for (int q = 0; q < 3; ++q) gvt[tess_tet(m.tess, t, n)][q] += gtet[n][q];
    }
    double gct[12][4][3];
    for (int f = 0; f < 6; ++f) {
        const CorrFace& C = CF[f];
        for (int h = 0; h < 2; ++h) {
            double tet[4][3];
            int ind[4][3];
            corr_tet(C, h, tet);
            for (int n = 0; n < 4; ++n) pt2index(m, ind[n], tet[n], i, j, k, err);
            double rv, rl;
            clip_call(m, tab, P, tet, ind, s, st, rv, rl, gct[2 * f + h], kinds, err);
            vol += tetsign * rv;
            vLiq += tetsign * rl;
        }
    }
    if (!(vol > 0.0) || !std::isfinite(vol)) err |= E_VOLUME;
    const double VF = vLiq / vol;
    if (s == 0.0 || kinds == LEAF_LIQ || kinds == LEAF_GAS) return VF;
    /* d(VF)/d(vol) part: -g VF / vol times d(vol)/d(vertices) of every tet */
    const double w = -g * VF / vol;
    for (int t = 0; t < nt; ++t) {
        const int a = tess_tet(m.tess, t, 0), b = tess_tet(m.tess, t, 1), c = tess_tet(m.tess, t, 2),
                  e = tess_tet(m.tess, t, 3);
        tet_vol_grad(p[a], p[b], p[c], p[e], w * tetsign, gvt[a], gvt[b], gvt[c], gvt[e]);
    }
    for (int n = 0; n < 8; ++n)
        if (gvt[n][0] != 0.0 || gvt[n][1] != 0.0 || gvt[n][2] != 0.0)
            project_reverse_call(m, V, GV, p0[n], i, j, k, dt, gvt[n]);
    for (int f = 0; f < 6; ++f) {
        const CorrFace& C = CF[f];
        for (int h = 0; h < 2; ++h) {
            double tet[4][3];
            corr_tet(C, h, tet);
            double(*gt)[3] = gct[2 * f + h];
            tet_vol_grad(tet[0], tet[1], tet[2], tet[3], w * tetsign, gt[0], gt[1], gt[2], gt[3]);
        }
        corr_face_reverse(m, V, GV, dt, C, gct + 2 * f);
    }
    return VF;
}

/* ---- computeDist ----------------------------------------------------------------------- */
/* dD/d(nx, ny, nz) and dD/dVF of computeDist (src/VF.jl:109-156) at cell (i, j, k) with plane
 * (n, D): from F(n, D) = VF, F the liquid fraction of the cell under n.x < D (the five-tet
 * sum of computePLIC2VF).  Returns false when dF/dD vanishes (the plane misses the cell or
 * n = 0), where D does not move with n or VF. */
SLVOF_HD bool dist_partials(const DevMesh& m, const CutCase* tab, int i, int j, int k, double nx, double ny, double nz,
                            double D, double* dDdn, double& dDdVF, int& err)
{
    /* the cut-cell fraction is the exact plane/box volume whatever the tessellation: take
     * the five tets of the cell in its 5_tets vertex order */
    double v[8][3];
    const bool even = ((i + j + k) % 2) == 0;
    {
        const int ia = even ? i : i + 1, ib = even ? i + 1 : i;
        for (int c = 0; c < 2; ++c)
            for (int b = 0; b < 2; ++b)
                for (int a = 0; a < 2; ++a) {
                    double* q = v[a + 2 * b + 4 * c];
                    q[0] = fc(m, 0, a ? ib : ia); q[1] = fc(m, 1, j + b); q[2] = fc(m, 2, k + c);
                }
    }
    const double tetsign = even ? 1.0 : -1.0;
    const double w = tetsign / m.cellvol;
    double gpl[4] = {0.0, 0.0, 0.0, 0.0};
    for (int t = 0; t < 5; ++t) {
        double tet[4][3], gv[4][3];
        for (int n = 0; n < 4; ++n)
            for (int p = 0; p < 3; ++p) { tet[n][p] = v[tet5(t, n)][p]; gv[n][p] = 0.0; }
        double vol, liq;
        leaf(tab, tet, nx, ny, nz, D, w, vol, liq, gv, gpl, err);
    }
    if (!(fabs(gpl[3]) > 0.0) || !std::isfinite(gpl[3])) return false;
    dDdVF = 1.0 / gpl[3];
    dDdn[0] = -gpl[0] / gpl[3];
    dDdn[1] = -gpl[1] / gpl[3];
    dDdn[2] = -gpl[2] / gpl[3];
    return true;
}

/* ---- ELVIRA candidate ------------------------------------------------------------------ */
/* Candidate `lane` of cell (i, j, k) (ELVIRA_calc!, src/ELVIRA.jl:62-100; lane = 9 * family
 * + 3 * outer + inner over the families X-Y, X-Z, Y-Z that the grid has).  Two tangential
 * components c_t = -(sum2 - sum1) / (centre2 - centre1), the sums running over the family's
 * normal direction weighted by its spacing; the normal component is +-1. */
struct Cand {
    int ta, tb, tn;          /* tangential directions (inner pair, outer pair) and the normal one */
    int lo_a, hi_a, lo_b, hi_b;
    double hs, dca, dcb;     /* spacing of the summed direction, centre differences */
    double c[3];
};

SLVOF_HD void cand_eval(const DevMesh& m, const double* VF, int i, int j, int k, int lane, Cand& C)
{
    const int fam_on[3] = {m.N[2] > 1, m.N[1] > 1, m.N[0] > 1};
    const int fam = lane / 9, a = (lane % 9) / 3, b = lane % 3;
    int f = 0;
    for (int q = 0, seen = 0; q < 3; ++q)
        if (fam_on[q]) {
            if (seen == fam) { f = q; break; }
            ++seen;
        }
    C.lo_b = a == 2 ? 0 : -1; C.hi_b = a == 0 ? 0 : 1; /* outer pair {-1,0},{-1,1},{0,1} */
    C.lo_a = b == 2 ? 0 : -1; C.hi_a = b == 0 ? 0 : 1; /* inner pair */
    if (f == 0) { C.ta = 0; C.tb = 1; C.tn = 2; }
    else if (f == 1) { C.ta = 0; C.tb = 2; C.tn = 1; }
    else { C.ta = 1; C.tb = 2; C.tn = 0; }
    C.hs = m.d[C.tn];
    const int base[3] = {i, j, k};
    int e[3];
#define V_(p, q, r) ld(VF + vi(m, i + (p), j + (q), k + (r)))
    double s2 = 0.0, s1 = 0.0;
    for (int r = -1; r <= 1; ++r) {
        e[C.ta] = C.hi_a; e[C.tb] = 0; e[C.tn] = r;
        s2 += V_(e[0], e[1], e[2]) * C.hs;
        e[C.ta] = C.lo_a;
        s1 += V_(e[0], e[1], e[2]) * C.hs;
    }
    C.dca = cc(m, C.ta, base[C.ta] + C.hi_a) - cc(m, C.ta, base[C.ta] + C.lo_a);
    C.c[C.ta] = -(s2 - s1) / C.dca;
    s2 = 0.0;
    s1 = 0.0;
    for (int r = -1; r <= 1; ++r) {
        e[C.tb] = C.hi_b; e[C.ta] = 0; e[C.tn] = r;
        s2 += V_(e[0], e[1], e[2]) * C.hs;
        e[C.tb] = C.lo_b;
        s1 += V_(e[0], e[1], e[2]) * C.hs;
    }
    C.dcb = cc(m, C.tb, base[C.tb] + C.hi_b) - cc(m, C.tb, base[C.tb] + C.lo_b);
    C.c[C.tb] = -(s2 - s1) / C.dcb;
    int up[3] = {0, 0, 0}, dn[3] = {0, 0, 0};
    up[C.tn] = 1;
    dn[C.tn] = -1;
    C.c[C.tn] = V_(up[0], up[1], up[2]) > V_(dn[0], dn[1], dn[2]) ? -1.0 : 1.0;
#undef V_
}

/* Reverse of the chosen candidate and its normalisation (check_normal!, src/ELVIRA.jl:
 * 106-115): gn = dL/d(normal) of cell (i, j, k) to dL/dVF over the VF array. */
SLVOF_HD void elvira_reverse(const DevMesh& m, const double* VF, double* gVF, int i, int j, int k, int lane,
                             const double* gn)
{
    Cand C;
    cand_eval(m, VF, i, j, k, lane, C);
    const double norm = sqrt((C.c[0] * C.c[0] + C.c[1] * C.c[1]) + C.c[2] * C.c[2]);
    const double n[3] = {C.c[0] / norm, C.c[1] / norm, C.c[2] / norm};
    const double dot = (n[0] * gn[0] + n[1] * gn[1]) + n[2] * gn[2];
    double gc[3];
    for (int q = 0; q < 3; ++q) gc[q] = (gn[q] - n[q] * dot) / norm;
    const double wa = gc[C.ta] * C.hs / C.dca, wb = gc[C.tb] * C.hs / C.dcb;
    int e[3];
    for (int r = -1; r <= 1; ++r) {
        e[C.ta] = C.hi_a; e[C.tb] = 0; e[C.tn] = r;
        acc(gVF + vi(m, i + e[0], j + e[1], k + e[2]), -wa);
        e[C.ta] = C.lo_a;
        acc(gVF + vi(m, i + e[0], j + e[1], k + e[2]), wa);
        e[C.tb] = C.hi_b; e[C.ta] = 0; e[C.tn] = r;
        acc(gVF + vi(m, i + e[0], j + e[1], k + e[2]), -wb);
        e[C.tb] = C.lo_b;
        acc(gVF + vi(m, i + e[0], j + e[1], k + e[2]), wb);
    }
}

/* ---- ghost fills ----------------------------------------------------------------------- */
constexpr int MAXPRE = 16;
/* Indices p of [lo, hi] (one direction) whose ghost-fill source is q; at most MAXPRE. */
SLVOF_HD int preimage_1d(int q, int N, int g, bool per, bool neu, int lo, int hi, int* out)
{
    int n = 0;
    if (ghost_src_1d(q, N, g, per, neu) == q) out[n++] = q;
    for (int p = lo; p <= hi; ++p) {
        if (p >= 1 && p <= N) { p = N; continue; } /* interior indices map to themselves */
        if (p != q && n < MAXPRE && ghost_src_1d(p, N, g, per, neu) == q) out[n++] = p;
    }
    return n;
}

} // namespace adj
} // namespace slvof
