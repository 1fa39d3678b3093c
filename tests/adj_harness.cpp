/*
 * Host build of the adjoint routines (ns_multiphase_gb300/csrc/adj64.cuh) for the CPU tests:
 * the same source the GPU kernels run, compiled with g++ without FMA contraction, so that
 * its derivatives can be checked against finite differences of the CPU restatement.  Test
 * infrastructure only; the library never loads it.
 */
#include <vector>

#include "../ns_multiphase_gb300/csrc/adj64.cuh"

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
    const double r = adj::sl_cell(H.m, TAB, V, G, P, dt, i, j, k, g, st.data(), e);
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

} // extern "C"
