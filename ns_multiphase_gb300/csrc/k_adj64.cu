/*
 * k_adj64.cu — reverse pass of one FP64 SL-VOF step on the GPU.  Built with -fmad=false: the
 * forward recomputation inside (pre-image, clip tree) rounds as the FP64 forward path does,
 * so it walks the same tree.  The per-cell mathematics is adj64.cuh; the kernels here order
 * the reverse of the step (src/Transport.jl:108-184, src/VF.jl:94-103):
 *
 *   fold VF    the step ends with Neumann!/update_VF_borders! (src/Transport.jl:180-181):
 *              derivatives of ghost copies go to their sources;
 *   SL         cells outside the band copy VF (derivative passes through); band cells run
 *              the clip tree backwards, thread per cell, to the face velocities and to the
 *              donor planes (n, D);
 *   fold D     computePLIC!'s update_borders!(D) (src/VF.jl:102);
 *   PLIC       computeDist's derivative at every cell (ghosts included) to n and VF;
 *   fold n     ELVIRA!'s update_borders! of the normals (src/ELVIRA.jl:49-51);
 *   ELVIRA     interface cells: the chosen candidate's derivative to the VF block.
 */
#include "slvof_kernels.h"
#include "slvof_dev.cuh"
#include "adj64.cuh"

namespace slvof {

namespace {

constexpr int ADJ_SL_THREADS = 64;

__device__ __forceinline__ void load_cut_table(CutCase* s_tab)
{
    for (int t = threadIdx.x; t < 16 * (int)sizeof(CutCase); t += blockDim.x)
        reinterpret_cast<char*>(s_tab)[t] = reinterpret_cast<const char*>(c_cut)[t];
    __syncthreads();
}

/* out[q] = sum of in[p] over the cells p whose ghost-fill source is q (separable map), over
 * the VF array (vf = 1, Neumann + borders) or a cell array (vf = 0, borders only). */
constexpr int FOLD_BX = 32, FOLD_BY = 8; /* fold tile: 32 x 8 entries of one k plane */

__global__ void __launch_bounds__(FOLD_BX * FOLD_BY) k_adj_fold(DevMesh m, const double* __restrict__ in,
                                                                double* __restrict__ out, int vf, int neumann)
{
    const int lo = vf ? m.vlo : m.lo;
    const int ext = vf ? 3 : 0;
    const int hi[3] = {m.hi[0] + ext, m.hi[1] + ext, m.hi[2] + ext};
    const long n0 = hi[0] - lo + 1, n1 = hi[1] - lo + 1;
    const int x = blockIdx.x * FOLD_BX + threadIdx.x, y = blockIdx.y * FOLD_BY + threadIdx.y, z = blockIdx.z;
    if (x >= n0 || y >= n1) return;
    const int i = lo + x, j = lo + y, k = lo + z;
    const long t = x + n0 * (y + n1 * z);
    /* farther than g from every end no ghost copies the cell: it is its own only preimage */
    if (i > m.g && i <= m.N[0] - m.g && j > m.g && j <= m.N[1] - m.g && k > m.g && k <= m.N[2] - m.g) {
        out[t] = in[t];
        return;
    }
    int pa[adj::MAXPRE], pb[adj::MAXPRE], pc[adj::MAXPRE];
    const int na = adj::preimage_1d(i, m.N[0], m.g, m.per[0], neumann, lo, hi[0], pa);
    const int nb = adj::preimage_1d(j, m.N[1], m.g, m.per[1], neumann, lo, hi[1], pb);
    const int nc = adj::preimage_1d(k, m.N[2], m.g, m.per[2], neumann, lo, hi[2], pc);
    double s = 0.0;
    for (int c = 0; c < nc; ++c)
        for (int b = 0; b < nb; ++b)
            for (int a = 0; a < na; ++a)
                s += in[(long)(pa[a] - lo) + (long)(pb[b] - lo) * n0 + (long)(pc[c] - lo) * n0 * n1];
    out[t] = s;
}

/* One thread per entry of a cell array (vf = 0) or of VF (vf = 1), (x, y) from the tile and the
 * plane from the grid: no index divides. */
void fold(const DevMesh& m, const double* in, double* out, int vf, int neumann, cudaStream_t s)
{
    const int ext = vf ? 3 : 0, lo = vf ? m.vlo : m.lo;
    const int n0 = m.hi[0] + ext - lo + 1, n1 = m.hi[1] + ext - lo + 1, n2 = m.hi[2] + ext - lo + 1;
    const dim3 grid((n0 + FOLD_BX - 1) / FOLD_BX, (n1 + FOLD_BY - 1) / FOLD_BY, n2);
    k_adj_fold<<<grid, dim3(FOLD_BX, FOLD_BY), 0, s>>>(m, in, out, vf, neumann);
}

/* Cells outside the band: VFnew = VF, the derivative passes through.  Band cells with a
 * nonzero incoming derivative go to the list. */
__global__ void __launch_bounds__(FOLD_BX * FOLD_BY) k_adj_split(DevMesh m, const short* __restrict__ band,
                                                                 const double* __restrict__ gfold,
                                                                 double* __restrict__ gout, int* list, int* count)
{
    const int i = 1 + blockIdx.x * FOLD_BX + threadIdx.x, j = 1 + blockIdx.y * FOLD_BY + threadIdx.y;
    const int k = 1 + blockIdx.z;
    bool take = false;
    int L = 0;
    if (i <= m.N[0] && j <= m.N[1]) {
        L = (i - 1) + (j - 1) * m.N[0] + (k - 1) * m.N[0] * m.N[1];
        const long v = vidx(m, i, j, k);
        const double g = gfold[v];
        const int b = band[cidx(m, i, j, k)];
        const bool sl = (b < 0 ? -b : b) <= m.nband;
        if (!sl) gout[v] = g;
        take = sl && g != 0.0;
    }
    warp_append(take, L, list, count);
}

/* ---- SL reverse in three kernels ------------------------------------------------------
 * A cell's reverse is 8 RK reverses and 5 independent tet clips; one thread per cell runs
 * them in series and a warp waits for its slowest cell.  Instead:
 *   k_adj_pre   thread per band cell: FP64 pre-image (as the forward computes it) and the
 *               uncut pre-image volume; cells whose whole pre-image is strictly on one side of
 *               every donor plane it reaches (VF = 1 or 0 around this input, zero derivative)
 *               are dropped, the others are compacted with their vertices;
 *   k_adj_tet   thread per (cell, tet): the tet's clip and its reverse (adj::clip), seeded with
 *               tetsign * g / vol; results per (cell, tet);
 *   k_adj_vert  thread per (cell, vertex): the vertex's derivative gathered from its tets in
 *               a fixed order, the d(vol) term, and the RK reverse to the face velocities.
 * The buffers are sized from the list counts by the host. */
__global__ void k_adj_pre(DevMesh m, double dt, adj::Vel V, adj::Plic P, const int* __restrict__ list,
                          const int* __restrict__ count, const double* __restrict__ gfold, AdjCell* cells,
                          int* count2, int* errw)
{
    const int n = *count;
    int err = 0;
    for (int item = blockIdx.x * blockDim.x + threadIdx.x; item - (int)(threadIdx.x & 31) < n;
         item += gridDim.x * blockDim.x) {
        bool keep = false;
        AdjCell r;
        if (item < n) {
            r.L = list[item];
            const int i = 1 + r.L % m.N[0], j = 1 + (r.L / m.N[0]) % m.N[1], k = 1 + r.L / (m.N[0] * m.N[1]);
            r.tetsign = adj::cell_verts(m, i, j, k, r.vt);
            for (int v = 0; v < 8; ++v) {
                double x[3][3];
                adj::project(m, V, r.vt[v], i, j, k, dt, x);
            }
            tess_means<double>(m.tess, r.vt);
            for (int v = 0; v < tess_npoints(m.tess); ++v) adj::pt2index(m, r.vind[v], r.vt[v], i, j, k, err);
            r.volu = 0.0;
            for (int t = 0; t < tess_ntets(m.tess); ++t)
                r.volu += r.tetsign * adj::tet_vol(r.vt[tess_tet(m.tess, t, 0)], r.vt[tess_tet(m.tess, t, 1)],
                                                   r.vt[tess_tet(m.tess, t, 2)], r.vt[tess_tet(m.tess, t, 3)]);
            r.g = gfold[vidx(m, i, j, k)];
            keep = r.volu != 0.0 && !adj::preimage_one_sided(m, P, r.vt, r.vind);
        }
        /* warp-aggregated slot in the compacted list */
        const unsigned ballot = __ballot_sync(0xffffffffu, keep);
        const int lane = threadIdx.x & 31;
        int base = 0;
        if (lane == 0 && ballot) base = atomicAdd(count2, __popc(ballot));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (keep) cells[base + __popc(ballot & ((1u << lane) - 1u))] = r;
    }
    if (err) atomicOr(errw, err);
}

__global__ void __launch_bounds__(ADJ_SL_THREADS) k_adj_tet(DevMesh m, adj::Plic P, const AdjCell* __restrict__ cells,
                                                            const int* __restrict__ count2, AdjTet* tets, int* errw)
{
    __shared__ CutCase s_tab[16];
    load_cut_table(s_tab);
    adj::Frame st[adj::STACK];
    const int nt = tess_ntets(m.tess);
    const long n = (long)nt * *count2;
    int err = 0;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const AdjCell& r = cells[q / nt];
        const int t = (int)(q % nt);
        double tet[4][3];
        int ind[4][3];
        for (int v = 0; v < 4; ++v)
            for (int p = 0; p < 3; ++p) {
                tet[v][p] = r.vt[tess_tet(m.tess, t, v)][p];
                ind[v][p] = r.vind[tess_tet(m.tess, t, v)][p];
            }
        const double s = r.tetsign * r.g / r.volu;
        AdjTet o;
        o.kinds = 0;
        adj::clip(m, s_tab, P, tet, ind, s, st, o.rv, o.rl, o.g, o.kinds, err);
        tets[q] = o;
    }
    if (err) atomicOr(errw, err);
}

__global__ void k_adj_vert(DevMesh m, double dt, adj::Vel V, adj::VelGrad GV, const AdjCell* __restrict__ cells,
                           const AdjTet* __restrict__ tets, const int* __restrict__ count2, int* errw)
{
    const long n = 8L * *count2;
    int err = 0;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const long c = q / 8;
        const int vtx = (int)(q % 8);
        const AdjCell& r = cells[c];
        const int nt = tess_ntets(m.tess);
        const AdjTet* T = tets + (long)nt * c;
        double vol = 0.0, vLiq = 0.0;
        int kinds = 0;
        for (int t = 0; t < nt; ++t) {
            vol += r.tetsign * T[t].rv;
            vLiq += r.tetsign * T[t].rl;
            kinds |= T[t].kinds;
        }
        if (!(vol > 0.0) || !isfinite(vol)) err |= adj::E_VOLUME;
        /* all leaves one-sided of one phase: VF is 1 (or 0) around this input */
        if (kinds == adj::LEAF_LIQ || kinds == adj::LEAF_GAS) continue;
        const double VF = vLiq / vol;
        const double w = -r.g * VF / vol;
        /* this vertex's derivative: from the tets that hold it, and (24_tets) a share of the
         * derivatives of the mean points that average it */
        double gp[3] = {0.0, 0.0, 0.0};
        for (int t = 0; t < nt; ++t)
            for (int v = 0; v < 4; ++v) {
                const int id = tess_tet(m.tess, t, v);
                const double wgt = adj::point_weight(id, vtx);
                if (wgt == 0.0) continue;
                double g4[4][3] = {};
                adj::tet_vol_grad(r.vt[tess_tet(m.tess, t, 0)], r.vt[tess_tet(m.tess, t, 1)],
                                  r.vt[tess_tet(m.tess, t, 2)], r.vt[tess_tet(m.tess, t, 3)], w * r.tetsign, g4[0],
                                  g4[1], g4[2], g4[3]);
                for (int p = 0; p < 3; ++p) gp[p] += wgt * (T[t].g[v][p] + g4[v][p]);
            }
        if (gp[0] == 0.0 && gp[1] == 0.0 && gp[2] == 0.0) continue;
        const int L = r.L;
        const int i = 1 + L % m.N[0], j = 1 + (L / m.N[0]) % m.N[1], k = 1 + L / (m.N[0] * m.N[1]);
        double p0[8][3];
        adj::cell_verts(m, i, j, k, p0);
        adj::project_reverse(m, V, GV, p0[vtx], i, j, k, dt, gp);
    }
    if (err) atomicOr(errw, err);
}

/* pressure_scheme "finite-difference": thread per band cell, the whole reverse of its SL update
 * with the twelve flux-correction tets (adj::sl_cell_fd), seeded with the folded dL/dVFnew.
 * The correction tets of a cell reach the flux volumes of all six faces, so this path keeps
 * the cell in one thread instead of splitting it into tets and vertices. */
__global__ void __launch_bounds__(ADJ_SL_THREADS) k_adj_sl_fd(DevMesh m, double dt, adj::Vel V, adj::VelGrad GV,
                                                              adj::Plic P, const int* __restrict__ list,
                                                              const int* __restrict__ count,
                                                              const double* __restrict__ gfold, int* errw)
{
    __shared__ CutCase s_tab[16];
    load_cut_table(s_tab);
    adj::Frame st[adj::STACK];
    const int n = *count;
    int err = 0;
    for (int item = blockIdx.x * blockDim.x + threadIdx.x; item < n; item += gridDim.x * blockDim.x) {
        const int L = list[item];
        const int i = 1 + L % m.N[0], j = 1 + (L / m.N[0]) % m.N[1], k = 1 + L / (m.N[0] * m.N[1]);
        const double g = gfold[vidx(m, i, j, k)];
        if (g != 0.0) adj::sl_cell_fd(m, s_tab, V, GV, P, dt, i, j, k, g, st, err);
    }
    if (err) atomicOr(errw, err);
}

/* computeDist backwards at every cell (ghosts included): gDf -> gn (+=) and gout. */
__global__ void k_adj_dist(DevMesh m, const double* __restrict__ VF, const double* __restrict__ nx,
                           const double* __restrict__ ny, const double* __restrict__ nz, const double* __restrict__ D,
                           const double* __restrict__ gDf, double* gnx, double* gny, double* gnz, double* gout,
                           int* errw)
{
    __shared__ CutCase s_tab[16];
    load_cut_table(s_tab);
    const long n0 = m.hi[0] - m.lo + 1, n1 = m.hi[1] - m.lo + 1, n2 = m.hi[2] - m.lo + 1;
    const long total = n0 * n1 * n2;
    int err = 0;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const double g = gDf[t];
        if (g == 0.0) continue;
        const int i = m.lo + (int)(t % n0), j = m.lo + (int)((t / n0) % n1), k = m.lo + (int)(t / (n0 * n1));
        const long v = vidx(m, i, j, k);
        const double vf = VF[v];
        if (!(vf >= m.VFlo && vf <= m.VFhi)) continue; /* pure: D = +-(Lx+Ly+Lz) */
        double dn[3], dv;
        if (!adj::dist_partials(m, s_tab, i, j, k, nx[t], ny[t], nz[t], D[t], dn, dv, err)) continue;
        gnx[t] += dn[0] * g;
        gny[t] += dn[1] * g;
        gnz[t] += dn[2] * g;
        gout[v] += dv * g;
    }
    if (err) atomicOr(errw, err);
}

/* ELVIRA backwards at interior interface cells with a chosen candidate. */
__global__ void k_adj_elvira(DevMesh m, const double* __restrict__ VF, const signed char* __restrict__ cand,
                             const double* __restrict__ gnx, const double* __restrict__ gny,
                             const double* __restrict__ gnz, double* gout)
{
    const long total = (long)m.N[0] * m.N[1] * m.N[2];
    for (long L = (long)blockIdx.x * blockDim.x + threadIdx.x; L < total; L += (long)gridDim.x * blockDim.x) {
        const int i = 1 + (int)(L % m.N[0]), j = 1 + (int)((L / m.N[0]) % m.N[1]), k = 1 + (int)(L / ((long)m.N[0] * m.N[1]));
        const long c = cidx(m, i, j, k);
        const double gn[3] = {gnx[c], gny[c], gnz[c]};
        if (gn[0] == 0.0 && gn[1] == 0.0 && gn[2] == 0.0) continue;
        const double vf = VF[vidx(m, i, j, k)];
        if (!(vf >= m.VFlo && vf <= m.VFhi)) continue; /* pure cells carry fixed axis normals */
        const int lane = cand[c];
        if (lane < 0) continue;
        adj::elvira_reverse(m, VF, gout, i, j, k, lane, gn);
    }
}

} // namespace

void launch_adjoint_fold_vf(const DevMesh& m, const double* gin, double* gout, int nsm, cudaStream_t s)
{
    (void)nsm;
    fold(m, gin, gout, 1, 1, s);
}

void launch_adjoint_fold_cell(const DevMesh& m, const double* gin, double* gout, int nsm, cudaStream_t s)
{
    (void)nsm;
    fold(m, gin, gout, 0, 0, s);
}

void launch_adjoint_elvira(const DevMesh& m, const double* VF, const signed char* cand, const AdjBuffers& b, int nsm,
                           cudaStream_t s)
{
    k_adj_elvira<<<nsm * 8, 256, 0, s>>>(m, VF, cand, b.gnf[0], b.gnf[1], b.gnf[2], b.gout);
}

void launch_adjoint_head(const DevMesh& m, const short* band, const AdjBuffers& b, int* list, int* count, int* count2,
                         int nsm, cudaStream_t s)
{
    const long vbytes = (long)(m.N[0] + 2 * m.g + 6) * (m.N[1] + 2 * m.g + 6) * (m.N[2] + 2 * m.g + 6) * sizeof(double);
    const long cbytes = (long)(m.N[0] + 2 * m.g) * (m.N[1] + 2 * m.g) * (m.N[2] + 2 * m.g) * sizeof(double);
    cudaMemsetAsync(b.gout, 0, vbytes, s);
    for (int q = 0; q < 3; ++q) cudaMemsetAsync(b.gn[q], 0, cbytes, s);
    cudaMemsetAsync(b.gD, 0, cbytes, s);
    cudaMemsetAsync(count, 0, sizeof(int), s);
    cudaMemsetAsync(count2, 0, sizeof(int), s);
    fold(m, b.gin, b.gfold, 1, 1, s);
    const dim3 grid((m.N[0] + FOLD_BX - 1) / FOLD_BX, (m.N[1] + FOLD_BY - 1) / FOLD_BY, m.N[2]);
    k_adj_split<<<grid, dim3(FOLD_BX, FOLD_BY), 0, s>>>(m, band, b.gfold, b.gout, list, count);
}

void launch_adjoint_pre(const DevMesh& m, double dt, const double* uf, const double* vf, const double* wf,
                        const double* nx, const double* ny, const double* nz, const double* D, const signed char* phase,
                        const AdjBuffers& b, const int* list, const int* count, int* count2, int* errw, int nsm,
                        cudaStream_t s)
{
    adj::Vel V{uf, vf, wf};
    adj::Plic P{nx, ny, nz, D, b.gn[0], b.gn[1], b.gn[2], b.gD, phase};
    k_adj_pre<<<nsm * 8, 128, 0, s>>>(m, dt, V, P, list, count, b.gfold, b.cells, count2, errw);
}

/* computeDist and ELVIRA backwards, after the SL update's reverse has filled gD and gn. */
static void adjoint_geometry(const DevMesh& m, const double* VF, const double* nx, const double* ny,
                             const double* nz, const double* D, const signed char* cand, const AdjBuffers& b,
                             int* errw, int nsm, cudaStream_t s)
{
    fold(m, b.gD, b.gDf, 0, 0, s);
    k_adj_dist<<<nsm * 8, 128, 0, s>>>(m, VF, nx, ny, nz, D, b.gDf, b.gn[0], b.gn[1], b.gn[2], b.gout, errw);
    for (int q = 0; q < 3; ++q) fold(m, b.gn[q], b.gnf[q], 0, 0, s);
    k_adj_elvira<<<nsm * 8, 256, 0, s>>>(m, VF, cand, b.gnf[0], b.gnf[1], b.gnf[2], b.gout);
}

void launch_adjoint_tail(const DevMesh& m, double dt, const double* VF, const double* uf, const double* vf,
                         const double* wf, const double* nx, const double* ny, const double* nz, const double* D,
                         const signed char* cand, const signed char* phase, const AdjBuffers& b, const int* count2,
                         int* errw, int nsm, cudaStream_t s)
{
    adj::Vel V{uf, vf, wf};
    adj::VelGrad GV{b.guf, b.gvf, b.gwf};
    adj::Plic P{nx, ny, nz, D, b.gn[0], b.gn[1], b.gn[2], b.gD, phase};
    k_adj_tet<<<nsm * 16, ADJ_SL_THREADS, 0, s>>>(m, P, b.cells, count2, b.tets, errw);
    k_adj_vert<<<nsm * 8, 128, 0, s>>>(m, dt, V, GV, b.cells, b.tets, count2, errw);
    adjoint_geometry(m, VF, nx, ny, nz, D, cand, b, errw, nsm, s);
}

void launch_adjoint_fd(const DevMesh& m, double dt, const double* VF, const double* uf, const double* vf,
                       const double* wf, const double* nx, const double* ny, const double* nz, const double* D,
                       const signed char* cand, const signed char* phase, const AdjBuffers& b, const int* list,
                       const int* count, int* errw, int nsm, cudaStream_t s)
{
    adj::Vel V{uf, vf, wf};
    adj::VelGrad GV{b.guf, b.gvf, b.gwf};
    adj::Plic P{nx, ny, nz, D, b.gn[0], b.gn[1], b.gn[2], b.gD, phase};
    k_adj_sl_fd<<<nsm * 16, ADJ_SL_THREADS, 0, s>>>(m, dt, V, GV, P, list, count, b.gfold, errw);
    adjoint_geometry(m, VF, nx, ny, nz, D, cand, b, errw, nsm, s);
}

} // namespace slvof
