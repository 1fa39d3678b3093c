/*
 * Host build of the flux form of the SL update (ns_multiphase_gb300/csrc/flux.cuh) in FP64,
 * for the CPU tests: each band cell's VFnew from its six faces' swept prisms, clipped with the
 * FP64 cutTet of adj64.cuh, so that the flux form can be checked against the CPU restatement's
 * cell form.  Test infrastructure only; the library never loads it.
 */
#include <vector>

#include "../ns_multiphase_gb300/csrc/adj64.cuh"
#include "../ns_multiphase_gb300/csrc/flux.cuh"

using namespace slvof;

#define X_ -1
static const CutCase TAB[16] = SLVOF_CUT_TABLE;
#undef X_

namespace {
struct HostMesh {
    DevMesh m{};
    std::vector<double> coords;
    explicit HostMesh(const slvof_mesh* M)
    {
        coords.resize(mesh_coords(M, nullptr));
        mesh_coords(M, coords.data());
        mesh_fill(M, coords.data(), m);
    }
};

/* Swept volume and liquid of the face (dir, h) for its low cell: sum over the face's prisms of
 * sigma times the signed clipped volumes of the prism tets. */
void face_flux(const DevMesh& m, const adj::Vel& V, const adj::Plic& P, double dt, int dir, int hi, int hj, int hk,
               double& vol, double& liq, int& err)
{
    double p[10][3];
    for (int c = 0; c < 4; ++c) {
        int i, j, k;
        flux::corner_node(dir, hi, hj, hk, c, i, j, k);
        p[c][0] = adj::fc(m, 0, i);
        p[c][1] = adj::fc(m, 1, j);
        p[c][2] = adj::fc(m, 2, k);
        for (int q = 0; q < 3; ++q) p[c + flux::MOVED][q] = p[c][q];
        double x[3][3];
        adj::project(m, V, p[c + flux::MOVED], hi, hj, hk, dt, x);
    }
    for (int q = 0; q < 3; ++q) {
        p[flux::PM][q] = 0.25 * (((p[0][q] + p[1][q]) + p[3][q]) + p[2][q]);
        p[flux::PM + flux::MOVED][q] =
            0.25 * (((p[5][q] + p[6][q]) + p[8][q]) + p[7][q]);
    }
    int ind[10][3];
    for (int n = 0; n < 10; ++n) adj::pt2index(m, ind[n], p[n], hi, hj, hk, err);
    int tri[4][3], sigma[4];
    const int nt = flux::face_triangles(m.tess, dir, flux::face_main_diagonal(m.tess, dir, hi, hj, hk), tri, sigma);
    std::vector<adj::Frame> st(adj::STACK);
    vol = 0.0;
    liq = 0.0;
    for (int t = 0; t < nt; ++t)
        for (int n = 0; n < 3; ++n) {
            int q[4];
            flux::prism_tet(tri[t], n, q);
            double tet[4][3], gtet[4][3];
            int tind[4][3];
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 3; ++b) { tet[a][b] = p[q[a]][b]; tind[a][b] = ind[q[a]][b]; }
            double rv = 0.0, rl = 0.0;
            int kinds = 0;
            adj::clip(m, TAB, P, tet, tind, 0.0, st.data(), rv, rl, gtet, kinds, err);
            vol += sigma[t] * rv;
            liq += sigma[t] * rl;
        }
    if (m.fd) {
        /* pressure_scheme "finite-difference": the face's two correction tets (the low face of
         * h), with the low cell's parity sign, the opposite of h's */
        adj::CorrFace C;
        adj::corr_face(m, V, hi, hj, hk, dt, 2 * dir, C);
        for (int hh = 0; hh < 2; ++hh) {
            double tet[4][3], gtet[4][3];
            adj::corr_tet(C, hh, tet);
            int tind[4][3];
            for (int a = 0; a < 4; ++a) adj::pt2index(m, tind[a], tet[a], hi, hj, hk, err);
            double rv = 0.0, rl = 0.0;
            int kinds = 0;
            adj::clip(m, TAB, P, tet, tind, 0.0, st.data(), rv, rl, gtet, kinds, err);
            vol -= C.sgn * rv;
            liq -= C.sgn * rl;
        }
    }
}
} // namespace

extern "C" {

/* VFnew of cell (i, j, k) in flux form: (L |C| + sum +-F) / (|C| + sum +-V) over its six faces,
 * L = VF (0 below VFlo, 1 above VFhi). */
double fluxh_sl_cell(const slvof_mesh* M, double dt, int i, int j, int k, const double* VF, const double* uf,
                     const double* vf, const double* wf, const double* nx, const double* ny, const double* nz,
                     const double* D, int* err)
{
    HostMesh H(M);
    const DevMesh& m = H.m;
    adj::Vel V{uf, vf, wf};
    const long nc = m.cs2 * (m.N[2] + 2 * m.g);
    std::vector<signed char> phase(nc);
    for (long t = 0; t < nc; ++t) {
        const double l1 = std::fabs(nx[t]) + std::fabs(ny[t]) + std::fabs(nz[t]);
        phase[t] = (l1 <= 1.0 && D[t] == m.Lsum) ? 1 : ((l1 <= 1.0 && D[t] == -m.Lsum) ? -1 : 0);
    }
    adj::Plic P{nx, ny, nz, D, nullptr, nullptr, nullptr, nullptr, phase.data()};
    const double cv = m.cellvol;
    const double vfc = VF[adj::vi(m, i, j, k)];
    const double L = vfc < m.VFlo ? 0.0 : (vfc > m.VFhi ? 1.0 : vfc);
    double vol = cv, liq = L * cv;
    int e = 0;
    const int c0[3] = {i, j, k};
    for (int dir = 0; dir < 3; ++dir)
        for (int side = 0; side < 2; ++side) {
            /* side 0: the cell's low face (the cell is the face's high cell, sign -1);
             * side 1: its high face (the cell is the low cell, sign +1) */
            int h[3] = {c0[0], c0[1], c0[2]};
            if (side == 1) h[dir] += 1;
            double fv, fl;
            face_flux(m, V, P, dt, dir, h[0], h[1], h[2], fv, fl, e);
            const double s = side == 1 ? 1.0 : -1.0;
            vol += s * fv;
            liq += s * fl;
        }
    if (err) *err = e;
    return liq / vol;
}

} // extern "C"

extern "C" {
/* VFnew in flux form for a list of cells (i, j, k triples) of one state. */
int fluxh_sl_cells(const slvof_mesh* M, double dt, int n, const int* cells, const double* VF, const double* uf,
                   const double* vf, const double* wf, const double* nx, const double* ny, const double* nz,
                   const double* D, double* out)
{
    HostMesh H(M);
    const DevMesh& m = H.m;
    adj::Vel V{uf, vf, wf};
    const long nc = m.cs2 * (m.N[2] + 2 * m.g);
    std::vector<signed char> phase(nc);
    for (long t = 0; t < nc; ++t) {
        const double l1 = std::fabs(nx[t]) + std::fabs(ny[t]) + std::fabs(nz[t]);
        phase[t] = (l1 <= 1.0 && D[t] == m.Lsum) ? 1 : ((l1 <= 1.0 && D[t] == -m.Lsum) ? -1 : 0);
    }
    adj::Plic P{nx, ny, nz, D, nullptr, nullptr, nullptr, nullptr, phase.data()};
    int e = 0;
    for (int q = 0; q < n; ++q) {
        const int c0[3] = {cells[3 * q], cells[3 * q + 1], cells[3 * q + 2]};
        const double vfc = VF[adj::vi(m, c0[0], c0[1], c0[2])];
        double vol = 1.0 * m.cellvol, liq = (vfc < m.VFlo ? 0.0 : (vfc > m.VFhi ? 1.0 : vfc)) * m.cellvol;
        for (int dir = 0; dir < 3; ++dir)
            for (int side = 0; side < 2; ++side) {
                int h[3] = {c0[0], c0[1], c0[2]};
                if (side == 1) h[dir] += 1;
                double fv, fl;
                face_flux(m, V, P, dt, dir, h[0], h[1], h[2], fv, fl, e);
                const double s = side == 1 ? 1.0 : -1.0;
                vol += s * fv;
                liq += s * fl;
            }
        out[q] = liq / vol;
    }
    return e;
}
}

extern "C" {
/* Swept volume and liquid (for the low cell) of face (dir, h) in FP64, in cell units. */
int fluxh_face(const slvof_mesh* M, double dt, int dir, int hi, int hj, int hk, const double* uf, const double* vf,
               const double* wf, const double* nx, const double* ny, const double* nz, const double* D, double* out)
{
    HostMesh H(M);
    const DevMesh& m = H.m;
    adj::Vel V{uf, vf, wf};
    const long nc = m.cs2 * (m.N[2] + 2 * m.g);
    std::vector<signed char> phase(nc);
    for (long t = 0; t < nc; ++t) {
        const double l1 = std::fabs(nx[t]) + std::fabs(ny[t]) + std::fabs(nz[t]);
        phase[t] = (l1 <= 1.0 && D[t] == m.Lsum) ? 1 : ((l1 <= 1.0 && D[t] == -m.Lsum) ? -1 : 0);
    }
    adj::Plic P{nx, ny, nz, D, nullptr, nullptr, nullptr, nullptr, phase.data()};
    int e = 0;
    double fv, fl;
    face_flux(m, V, P, dt, dir, hi, hj, hk, fv, fl, e);
    out[0] = fv / m.cellvol;
    out[1] = fl / m.cellvol;
    return e;
}
}

extern "C" {

/* The correction tets of face (dir, h) two ways: out[0..3] = the FP64 reverse's corr_face in
 * physical units (apex, and the tets' volume signed for the low cell); out[4..7] = the mixed
 * path's flux::face_correction in cell units on the same traced corners, mapped back
 * (apex * d + the low cell's corner, volume * |cell|). */
int fluxh_face_correction(const slvof_mesh* M, double dt, int dir, int hi, int hj, int hk, const double* uf,
                          const double* vf, const double* wf, double* out)
{
    HostMesh H(M);
    const DevMesh& m = H.m;
    adj::Vel V{uf, vf, wf};
    adj::CorrFace C;
    adj::corr_face(m, V, hi, hj, hk, dt, 2 * dir, C);
    double tet[4][3];
    double vt = 0.0;
    for (int hh = 0; hh < 2; ++hh) {
        adj::corr_tet(C, hh, tet);
        vt += adj::tet_vol(tet[0], tet[1], tet[2], tet[3]);
    }
    for (int q = 0; q < 3; ++q) out[q] = C.e[q];
    out[3] = -C.sgn * vt;
    /* cell units, the low cell's frame */
    const int l[3] = {hi - (dir == 0), hj - (dir == 1), hk - (dir == 2)};
    const double o[3] = {adj::fc(m, 0, l[0]), adj::fc(m, 1, l[1]), adj::fc(m, 2, l[2])};
    const double d[3] = {m.d[0], m.d[1], m.d[2]};
    int s_, t_;
    flux::face_axes(dir, s_, t_);
    double P[5][3], Q[5][3];
    for (int c = 0; c < 4; ++c) {
        int i, j, k;
        flux::corner_node(dir, hi, hj, hk, c, i, j, k);
        double x[3] = {adj::fc(m, 0, i), adj::fc(m, 1, j), adj::fc(m, 2, k)};
        double w[3][3];
        adj::project(m, V, x, hi, hj, hk, dt, w);
        P[c][dir] = 1.0;
        P[c][s_] = flux::corner_s(c);
        P[c][t_] = flux::corner_t(c);
        for (int q = 0; q < 3; ++q) Q[c][q] = (x[q] - o[q]) / d[q];
    }
    const double* u = dir == 0 ? uf : (dir == 1 ? vf : wf);
    const double dtu = dt * u[adj::ci(m, hi, hj, hk)] / d[dir];
    double e[3];
    const double vc = flux::face_correction(dir, hi, hj, hk, dtu, P, Q, e);
    for (int q = 0; q < 3; ++q) out[4 + q] = e[q] * d[q] + o[q];
    out[7] = vc * (d[0] * d[1] * d[2]);
    return 0;
}

} // extern "C"
