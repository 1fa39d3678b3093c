/*
 * Host build of the adjoint routines (ns_multiphase_gb300/csrc/adj64.cuh) for the CPU tests:
 * the same source the GPU kernels run, compiled with g++ without FMA contraction, so that
 * its derivatives can be checked against finite differences of the CPU restatement.  Test
 * infrastructure only; the library never loads it.
 */
#include <vector>

#include "../ns_multiphase_gb300/csrc/adj64.cuh"
#include "../ns_multiphase_gb300/csrc/adj32.cuh"

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
} // namespace

extern "C" {

/* Reverse of the SL update of one cell: returns VFnew, adds g * dVFnew/d(...) to the
 * gradient arrays (cell-array shaped). */
double adjh_sl_cell(const slvof_mesh* M, double dt, int i, int j, int k, const double* uf, const double* vf,
                    const double* wf, const double* nx, const double* ny, const double* nz, const double* D, double g,
                    double* guf, double* gvf, double* gwf, double* gnx, double* gny, double* gnz, double* gD, int* err)
{
    HostMesh H(M);
    adj::Vel V{uf, vf, wf};
    adj::VelGrad G{guf, gvf, gwf};
    /* phase codes as the PLIC pass writes them: +-1 where |n|_1 <= 1 and D = +-(Lx+Ly+Lz) */
    const long nc = H.m.cs2 * (H.m.N[2] + 2 * H.m.g);
    std::vector<signed char> phase(nc);
    for (long t = 0; t < nc; ++t) {
        const double l1 = std::fabs(nx[t]) + std::fabs(ny[t]) + std::fabs(nz[t]);
        phase[t] = (l1 <= 1.0 && D[t] == H.m.Lsum) ? 1 : ((l1 <= 1.0 && D[t] == -H.m.Lsum) ? -1 : 0);
    }
    adj::Plic P{nx, ny, nz, D, gnx, gny, gnz, gD, phase.data()};
    std::vector<adj::Frame> st(adj::STACK);
    int e = 0;
    const double r = H.m.fd ? adj::sl_cell_fd(H.m, TAB, V, G, P, dt, i, j, k, g, st.data(), e)
                            : adj::sl_cell(H.m, TAB, V, G, P, dt, i, j, k, g, st.data(), e);
    if (err) *err = e;
    return r;
}

/* VFnew from given pre-image vertices (cell (i, j, k) fixes the tet sign; vertex cells from
 * pt2index! seeded at the cell) and g * d(VFnew)/d(vertices) in gvt[8][3]. */
double adjh_sl_vertices(const slvof_mesh* M, int i, int j, int k, const double* vt, const double* nx, const double* ny,
                        const double* nz, const double* D, double g, double* gvt, int* err)
{
    HostMesh H(M);
    double p0[8][3], v[15][3], gv[8][3];
    const double tetsign = adj::cell_verts(H.m, i, j, k, p0);
    int vind[15][3];
    int e = 0;
    for (int n = 0; n < 8; ++n)
        for (int p = 0; p < 3; ++p) { v[n][p] = vt[3 * n + p]; gv[n][p] = 0.0; }
    tess_means<double>(H.m.tess, v);
    for (int n = 0; n < tess_npoints(H.m.tess); ++n) adj::pt2index(H.m, vind[n], v[n], i, j, k, e);
    adj::Plic P{nx, ny, nz, D, nullptr, nullptr, nullptr, nullptr};
    std::vector<adj::Frame> st(adj::STACK);
    std::vector<double> sink(4 * H.m.cs2 * (H.m.N[2] + 2 * H.m.g), 0.0);
    double* s0 = sink.data();
    const long nc = H.m.cs2 * (H.m.N[2] + 2 * H.m.g);
    P.gnx = s0; P.gny = s0 + nc; P.gnz = s0 + 2 * nc; P.gD = s0 + 3 * nc;
    const double r = adj::sl_vertices(H.m, TAB, P, tetsign, v, vind, g, st.data(), gv, e);
    for (int n = 0; n < 8; ++n)
        for (int p = 0; p < 3; ++p) gvt[3 * n + p] = gv[n][p];
    if (err) *err = e;
    return r;
}

/* cutTet of one tet with its reverse: vLiq, and s * d(vLiq)/d(tet) in gtet[4][3]. */
double adjh_clip(const slvof_mesh* M, const double* tet, const int* ind, const double* nx, const double* ny,
                 const double* nz, const double* D, double s, double* gtet, double* vol, int* err)
{
    HostMesh H(M);
    double t[4][3], g[4][3];
    int I[4][3];
    for (int n = 0; n < 4; ++n)
        for (int p = 0; p < 3; ++p) { t[n][p] = tet[3 * n + p]; I[n][p] = ind[3 * n + p]; }
    const long nc = H.m.cs2 * (H.m.N[2] + 2 * H.m.g);
    std::vector<double> sink(4 * nc, 0.0);
    adj::Plic P{nx, ny, nz, D, sink.data(), sink.data() + nc, sink.data() + 2 * nc, sink.data() + 3 * nc};
    std::vector<adj::Frame> st(adj::STACK);
    int e = 0, kinds = 0;
    double rv, rl;
    adj::clip(H.m, TAB, P, t, I, s, st.data(), rv, rl, g, kinds, e);
    for (int n = 0; n < 4; ++n)
        for (int p = 0; p < 3; ++p) gtet[3 * n + p] = g[n][p];
    if (vol) *vol = rv;
    if (err) *err = e;
    return rl;
}

/* Projected pre-image vertices of cell (i, j, k), as sl_cell computes them. */
void adjh_preimage_vertices(const slvof_mesh* M, double dt, int i, int j, int k, const double* uf, const double* vf,
                            const double* wf, double* vt)
{
    HostMesh H(M);
    double p0[8][3];
    adj::cell_verts(H.m, i, j, k, p0);
    adj::Vel V{uf, vf, wf};
    for (int n = 0; n < 8; ++n) {
        double x[3][3];
        adj::project(H.m, V, p0[n], i, j, k, dt, x);
        for (int p = 0; p < 3; ++p) vt[3 * n + p] = p0[n][p];
    }
}

/* dD/d(nx, ny, nz) and dD/dVF of computeDist at cell (i, j, k); returns 1 if defined. */
int adjh_dist_partials(const slvof_mesh* M, int i, int j, int k, double nx, double ny, double nz, double D, double* out)
{
    HostMesh H(M);
    int e = 0;
    double dn[3], dv = 0.0;
    const bool ok = adj::dist_partials(H.m, TAB, i, j, k, nx, ny, nz, D, dn, dv, e);
    out[0] = dn[0]; out[1] = dn[1]; out[2] = dn[2]; out[3] = dv;
    return ok ? 1 : 0;
}

/* Raw ELVIRA candidate `lane` of cell (i, j, k) (before normalisation). */
void adjh_candidate(const slvof_mesh* M, const double* VF, int i, int j, int k, int lane, double* c)
{
    HostMesh H(M);
    adj::Cand C;
    adj::cand_eval(H.m, VF, i, j, k, lane, C);
    c[0] = C.c[0]; c[1] = C.c[1]; c[2] = C.c[2];
}

void adjh_elvira_reverse(const slvof_mesh* M, const double* VF, double* gVF, int i, int j, int k, int lane,
                         const double* gn)
{
    HostMesh H(M);
    adj::elvira_reverse(H.m, VF, gVF, i, j, k, lane, gn);
}

int adjh_preimage(int q, int N, int g, int per, int neu, int lo, int hi, int* out)
{
    return adj::preimage_1d(q, N, g, per != 0, neu != 0, lo, hi, out);
}


/* FP64 reverse of the clipped volume from given vertices, with the donor-plane derivatives:
 * g * dVFnew/d(vertices) in gvt[8][3], g * dVFnew/d(n, D) added to gpl (4 cell arrays). */
double adjh_sl_vertices_pl(const slvof_mesh* M, int i, int j, int k, const double* vt, const double* nx,
                           const double* ny, const double* nz, const double* D, double g, double* gvt, double* gpl,
                           int* err)
{
    HostMesh H(M);
    double p0[8][3], v[15][3], gv[8][3];
    const double tetsign = adj::cell_verts(H.m, i, j, k, p0);
    int vind[15][3];
    int e = 0;
    for (int n = 0; n < 8; ++n)
        for (int p = 0; p < 3; ++p) { v[n][p] = vt[3 * n + p]; gv[n][p] = 0.0; }
    tess_means<double>(H.m.tess, v);
    for (int n = 0; n < tess_npoints(H.m.tess); ++n) adj::pt2index(H.m, vind[n], v[n], i, j, k, e);
    const long nc = H.m.cs2 * (H.m.N[2] + 2 * H.m.g);
    adj::Plic P{nx, ny, nz, D, gpl, gpl + nc, gpl + 2 * nc, gpl + 3 * nc};
    std::vector<adj::Frame> st(adj::STACK);
    const double r = adj::sl_vertices(H.m, TAB, P, tetsign, v, vind, g, st.data(), gv, e);
    for (int n = 0; n < 8; ++n)
        for (int p = 0; p < 3; ++p) gvt[3 * n + p] = gv[n][p];
    if (err) *err = e;
    return r;
}
} // extern "C"

namespace {
/* The boundary form of the same derivatives (adj32.cuh) in scalar R, in the mixed path's
 * cell frame: vertices in cell units, donor planes as px*x + py*y + pz*z - Dt. */
template <class R>
void sd_cell(const DevMesh& m, int i, int j, int k, const double* vt, const double* nx, const double* ny,
             const double* nz, const double* D, const signed char* phase, double VF, double g, double* gvt, double* gpl)
{
    const long nc = m.cs2 * (m.N[2] + 2 * m.g);
    const double o[3] = {adj::fc(m, 0, i), adj::fc(m, 1, j), adj::fc(m, 2, k)};
    double v[15][3];
    R q[15][3];
    int ind[15][3];
    int e = 0;
    for (int n = 0; n < 8; ++n)
        for (int p = 0; p < 3; ++p) {
            v[n][p] = vt[3 * n + p];
            q[n][p] = (R)((vt[3 * n + p] - o[p]) / m.d[p]);
        }
    tess_means<double>(m.tess, v);
    tess_means<R>(m.tess, q);
    const int np = tess_npoints(m.tess), nt = tess_ntets(m.tess);
    for (int n = 0; n < np; ++n) {
        adj::pt2index(m, ind[n], v[n], i, j, k, e);
        ind[n][0] -= i; ind[n][1] -= j; ind[n][2] -= k;
    }
    const R tetsign = tess_even(m.tess, i, j, k) ? R(1) : R(-1);
    auto tetq = [&](int t, R (&tv)[4][3]) {
        for (int s = 0; s < 4; ++s)
            for (int p = 0; p < 3; ++p) tv[s][p] = q[tess_tet(m.tess, t, s)][p];
    };
    auto tvol = [](const R (&tv)[4][3]) {
        const R a[3] = {tv[0][0] - tv[3][0], tv[0][1] - tv[3][1], tv[0][2] - tv[3][2]};
        const R b[3] = {tv[1][0] - tv[3][0], tv[1][1] - tv[3][1], tv[1][2] - tv[3][2]};
        const R c[3] = {tv[2][0] - tv[3][0], tv[2][1] - tv[3][1], tv[2][2] - tv[3][2]};
        return R(-1) / R(6) * (a[0] * (b[1] * c[2] - c[1] * b[2]) - a[1] * (b[0] * c[2] - c[0] * b[2]) +
                               a[2] * (b[0] * c[1] - c[0] * b[1]));
    };
    R vol = R(0);
    for (int t = 0; t < nt; ++t) {
        R tv[4][3];
        tetq(t, tv);
        vol += tetsign * tvol(tv);
    }
    const R coef = (R)g * tetsign / vol;
    const R VFr = (R)VF;
    auto donor = [&](int a, int b, int c, int& ph, R& px, R& py, R& pz, R& Dt) {
        const long t = adj::ci(m, i + a, j + b, k + c);
        ph = phase[t];
        px = (R)(nx[t] * m.d[0]); py = (R)(ny[t] * m.d[1]); pz = (R)(nz[t] * m.d[2]);
        Dt = (R)(D[t] - ((nx[t] * o[0] + ny[t] * o[1]) + nz[t] * o[2]));
    };
    const sd::BFaces F = sd::boundary_faces(m.tess);
    R gq[15][3] = {};
    for (int f = 0; f < F.n; ++f) {
        const int t = F.t[f], b = F.b[f];
        R tv[4][3], S[3];
        tetq(t, tv);
        sd::face_area(tv, b, S);
        R p3[3][3], mm[3];
        int i3[3][3], ids[3], n = 0;
        for (int s = 0; s < 4; ++s) {
            if (s == b) continue;
            ids[n] = tess_tet(m.tess, t, s);
            for (int p = 0; p < 3; ++p) { p3[n][p] = tv[s][p]; i3[n][p] = ind[ids[n]][p]; }
            ++n;
        }
        sd::face_moments(p3, i3, donor, mm);
        for (int s = 0; s < 3; ++s)
            for (int p = 0; p < 3; ++p) gq[ids[s]][p] += coef * S[p] * (mm[s] - VFr / R(3));
    }
    for (int vtx = 0; vtx < 8; ++vtx)
        for (int p = 0; p < 3; ++p) {
            double s = 0.0;
            for (int id = 0; id < np; ++id) s += adj::point_weight(id, vtx) * (double)gq[id][p];
            gvt[3 * vtx + p] = s / m.d[p];
        }
    for (int t = 0; t < nt; ++t) {
        R tv[4][3];
        tetq(t, tv);
        const R V = tvol(tv);
        if (V == R(0)) continue;
        const R sgn = V > R(0) ? R(1) : R(-1);
        int lo[3], hi[3];
        for (int p = 0; p < 3; ++p) {
            lo[p] = hi[p] = ind[tess_tet(m.tess, t, 0)][p];
            for (int s = 1; s < 4; ++s) {
                lo[p] = std::min(lo[p], ind[tess_tet(m.tess, t, s)][p]);
                hi[p] = std::max(hi[p], ind[tess_tet(m.tess, t, s)][p]);
            }
        }
        for (int c = lo[2]; c <= hi[2]; ++c)
            for (int b = lo[1]; b <= hi[1]; ++b)
                for (int a = lo[0]; a <= hi[0]; ++a) {
                    int ph;
                    R px, py, pz, Dt, A, C[3];
                    donor(a, b, c, ph, px, py, pz, Dt);
                    if (ph != 0) continue;
                    sd::Poly3<R> ws[2];
                    if (!sd::plane_piece(tv, lo, hi, a, b, c, px, py, pz, Dt, A, C, ws)) continue;
                    const double len = std::sqrt((double)px * px + (double)py * py + (double)pz * pz);
                    const double c2 = (double)(coef * sgn) * (double)A / len;
                    const long td = adj::ci(m, i + a, j + b, k + c);
                    gpl[3 * nc + td] += c2;
                    for (int p = 0; p < 3; ++p) gpl[p * nc + td] -= c2 * (o[p] + m.d[p] * (double)C[p]);
                }
    }
}
} // namespace

extern "C" {
/* The boundary form in double (prec 0) or float (prec 1); phase codes from (n, D). */
void adjh_sd_vertices(const slvof_mesh* M, int prec, int i, int j, int k, const double* vt, const double* nx,
                      const double* ny, const double* nz, const double* D, double VF, double g, double* gvt,
                      double* gpl)
{
    HostMesh H(M);
    const long nc = H.m.cs2 * (H.m.N[2] + 2 * H.m.g);
    std::vector<signed char> phase(nc);
    for (long t = 0; t < nc; ++t) {
        const double l1 = std::fabs(nx[t]) + std::fabs(ny[t]) + std::fabs(nz[t]);
        phase[t] = (l1 <= 1.0 && D[t] == H.m.Lsum) ? 1 : ((l1 <= 1.0 && D[t] == -H.m.Lsum) ? -1 : 0);
    }
    if (prec == 0) sd_cell<double>(H.m, i, j, k, vt, nx, ny, nz, D, phase.data(), VF, g, gvt, gpl);
    else sd_cell<float>(H.m, i, j, k, vt, nx, ny, nz, D, phase.data(), VF, g, gvt, gpl);
}

/* computeDist's derivatives by the plane polygon (double or float): dD/dn in out[0..2],
 * dD/dVF in out[3]; 0 when the polygon is empty. */
int adjh_sd_dist(const slvof_mesh* M, int prec, int i, int j, int k, double nx, double ny, double nz, double D,
                 double* out)
{
    HostMesh H(M);
    const double o[3] = {adj::fc(H.m, 0, i), adj::fc(H.m, 1, j), adj::fc(H.m, 2, k)};
    const double px = nx * H.m.d[0], py = ny * H.m.d[1], pz = nz * H.m.d[2];
    const double Dt = D - ((nx * o[0] + ny * o[1]) + nz * o[2]);
    double A, Mm[3];
    if (prec == 0) {
        sd::plane_cube<double>(px, py, pz, Dt, A, Mm);
    } else {
        float Af, Mf[3];
        sd::plane_cube<float>((float)px, (float)py, (float)pz, (float)Dt, Af, Mf);
        A = Af; Mm[0] = Mf[0]; Mm[1] = Mf[1]; Mm[2] = Mf[2];
    }
    if (!(A > 0.0)) return 0;
    const double len = std::sqrt(px * px + py * py + pz * pz);
    for (int p = 0; p < 3; ++p) out[p] = o[p] + H.m.d[p] * (Mm[p] / A);
    out[3] = len / A;
    return 1;
}
} // extern "C"
