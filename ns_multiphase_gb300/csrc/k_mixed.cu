/*
 * k_mixed.cu — mixed-precision kernels of the SL-VOF path (FMA on).
 *
 * Geometry runs in FP32 in cell-normalised local coordinates: a point is u = (x - o)/d with o
 * the corner of the cell being updated, so mesh faces are small integers (exact in FP32)
 * and the cell volume is 1.  This needs a uniform mesh, which create_mesh builds
 * (src/Mesh.jl:83-100); slvof_create rejects the mixed mode otherwise.
 *
 * The step's SL update is the flux form: VFnew = (L + sum +-F_f) / (1 + sum +-V_f) over each band
 * cell's six faces, with F_f the liquid and V_f the volume swept through face f (the prism
 * between the face and its traced pre-image, split as the cell pre-images of the reference are,
 * src/VFgeom.jl:229-332), so each face is computed once and shared by the two cells beside it.
 *
 *   k_flux_lists     : band-cell nodes and faces, each listed by the band cell that owns it.
 *   k_flux_nodes     : the RK trace of every listed grid node (FP64, from the FP64 face
 *                      velocities), stored once and read by every prism that uses the node.
 *   k_flux_faces     : each face's swept volume V_f in FP64 (closed form); faces whose prism
 *                      lies in cells of one phase take F_f = V_f or 0, the others are listed.
 *   k_flux_clip      : warp-cooperative FP32 clip of the listed faces' prism tets (cutTet's cut
 *                      tables and cuts, src/VFgeom.jl:713-900), pending sub-tets of a batch of
 *                      faces in a shared-memory stack, liquid and volume summed in float-float;
 *                      the liquid is then rescaled to the FP64 volume.
 *   k_flux_cells     : VFnew per band cell; cells with an all-liquid or all-gas pre-image give
 *                      exactly 1 or 0, cells within 1e-6 of 0 or 1 are listed for the cell form.
 *   k_sl32_pre       : the cell form's eight FP32 pre-image vertices per band cell (the
 *                      reverse pass's input).
 *   k_sl32_clipw     : the cell form's warp-cooperative clip of listed cells' tets (the flux
 *                      form's near-pure cells).
 */
#include "slvof_kernels.h"
#include "slvof_dev.cuh"
#include "mixed32.cuh"
#include "flux.cuh"

namespace slvof {

/* ======================================================================================
 * SL update in FP32 local coordinates.
 * ==================================================================================== */
/* One cutTet recursion level: parent tet (vertices 0-3), new vertices on the cutting mesh
 * plane (4-7), their side-1 cell indices packed as bytes, the children's running sums, and
 * case / next child / direction / done flags / cut index packed in meta. */
struct Frame32 {
    float x[8], y[8], z[8];
    unsigned ind[8];
    FF vol, liq;
    int meta;
};
__device__ __forceinline__ int meta_pack(int cs, int next, int dir, int flags, int cut)
{
    return cs | (next << 4) | (dir << 8) | (flags << 10) | ((cut + 128) << 16);
}

__device__ __forceinline__ float tet_vol32(const float* vx, const float* vy, const float* vz, int p, int q, int r, int s)
{
    return tet_vol<float>(vx[p], vy[p], vz[p], vx[q], vy[q], vz[q], vx[r], vy[r], vz[r], vx[s], vy[s], vz[s]);
}

__device__ __forceinline__ void leaf32(const DevMesh& m, const CutCase* tab, const Plane32& PL, int i0, int j0, int k0,
                                       const float* cx, const float* cy, const float* cz, int di, int dj, int dk,
                                       FF& rv, FF& rl, int& err)
{
    const float4 pl = __ldg(PL.P + cidx(m, i0 + di, j0 + dj, k0 + dk));
    const float Dt = pl.w + pl.x * (float)di + pl.y * (float)dj + pl.z * (float)dk;
    float d[4], vx[8], vy[8], vz[8];
#pragma unroll
    for (int n = 0; n < 4; ++n) {
        d[n] = pl.x * cx[n] + pl.y * cy[n] + pl.z * cz[n] - Dt;
        vx[n] = cx[n]; vy[n] = cy[n]; vz[n] = cz[n];
    }
    float c0 = d[0], c1 = d[1], c2 = d[2], c3 = d[3];
    const int cs = d2case(c0, c1, c2, c3, 1e-30f, err);
    const CutCase& C = tab[cs];
    for (int n = 0; n < C.nvert; ++n) {
        const int v1 = C.v1[n], v2 = C.v2[n];
        const float den = d[v2] - d[v1];
        const float mu = fminf(1.f, fmaxf(0.f, den != 0.f ? -d[v1] / den : 1.f));
        vx[4 + n] = vx[v1] + mu * (vx[v2] - vx[v1]);
        vy[4 + n] = vy[v1] + mu * (vy[v2] - vy[v1]);
        vz[4 + n] = vz[v1] + mu * (vz[v2] - vz[v1]);
    }
    FF vol{0.f, 0.f}, liq{0.f, 0.f};
    for (int n = C.ntets - 1; n >= C.nntet - 1; --n) {
        const float tv = tet_vol32(vx, vy, vz, C.vtet[n][0], C.vtet[n][1], C.vtet[n][2], C.vtet[n][3]);
        ff_add(vol, tv);
        ff_add(liq, tv);
    }
    for (int n = 0; n < C.nntet - 1; ++n) ff_add(vol, tet_vol32(vx, vy, vz, C.vtet[n][0], C.vtet[n][1], C.vtet[n][2], C.vtet[n][3]));
    rv = vol;
    rl = liq;
}

__device__ __forceinline__ void form_child32(const Frame32& F, const CutCase* tab, int n, float* cx, float* cy,
                                             float* cz, int (*ci)[3])
{
    const int cs = F.meta & 15, dir = (F.meta >> 8) & 3, cut = ((F.meta >> 16) & 255) - 128;
    const CutCase& C = tab[cs];
    const int side = C.side[n];
    for (int nn = 0; nn < 4; ++nn) {
        const int v = C.vtet[n][nn];
        cx[nn] = F.x[v]; cy[nn] = F.y[v]; cz[nn] = F.z[v];
        const unsigned p = F.ind[v];
        ci[nn][0] = unpack(p, 0); ci[nn][1] = unpack(p, 1); ci[nn][2] = unpack(p, 2);
        if (side == 1) ci[nn][dir] = cut;
    }
}

/* Side of a point set against every donor PLIC plane of an index box (at most 2x2x2 cells):
 * +1 when every point is strictly on the liquid side of every donor's plane, -1 when strictly
 * on the gas side of every one, 0 otherwise.  Every PLIC leaf under a (sub-)tet with +1 is
 * then d2case case 1 (all liquid) and with -1 case 16 (all gas), whatever the mesh cuts, so
 * the clipped volume needs no cuts.  Pure donors have planes at |D| = Lx+Ly+Lz, which put
 * everything on one side, so this covers the pure-donor case. */
template <int NP>
__device__ __forceinline__ int box_plane_side(const DevMesh& m, const Plane32& PL, int i0, int j0, int k0, int lo0,
                                              int hi0, int lo1, int hi1, int lo2, int hi2, const float* cx,
                                              const float* cy, const float* cz)
{
    if (hi0 - lo0 > 1 || hi1 - lo1 > 1 || hi2 - lo2 > 1) return 0;
    int side = 2;
    for (int c = lo2; c <= hi2; ++c)
        for (int b = lo1; b <= hi1; ++b)
            for (int a = lo0; a <= hi0; ++a) {
                const float4 p = __ldg(PL.P + cidx(m, i0 + a, j0 + b, k0 + c));
                const float Dt = p.w + p.x * (float)a + p.y * (float)b + p.z * (float)c;
                bool neg = true, pos = true;
#pragma unroll
                for (int n = 0; n < NP; ++n) {
                    const float d = fmaf(p.x, cx[n], fmaf(p.y, cy[n], fmaf(p.z, cz[n], -Dt)));
                    neg = neg && d < 0.f;
                    pos = pos && d > 0.f;
                }
                const int sd = neg ? 1 : (pos ? -1 : 0);
                if (sd == 0 || (side != 2 && sd != side)) return 0;
                side = sd;
            }
    return side;
}

/* cutTet (src/VFgeom.jl:713-900) with an explicit stack; indices relative to the cell.
 * A (sub-)tet whose donor box is uniformly pure is one leaf: every PLIC leaf below it would
 * be d2case case 1 (or 16), so its clipped volume is the tet's own volume, all liquid (or
 * all gas); the mesh-plane cuts under it are skipped. */
__device__ __noinline__ void clip32(const DevMesh& m, const CutCase* tab, const Plane32& PL,
                                    const signed char* __restrict__ phase,
                       int i0, int j0, int k0, const int* rlo, const int* rhi, float* cx, float* cy, float* cz,
                       int (*ci)[3], FF& out_v, FF& out_l, int& err)
{
    Frame32 st[CLIP_STACK32];
    int depth = 0, flags = 0, leaves = 0;
    for (;;) {
        int dir = -1, cut = 0;
        int lo[3], hi[3];
        for (int q = 0; q < 3; ++q) {
            lo[q] = min(min(ci[0][q], ci[1][q]), min(ci[2][q], ci[3][q]));
            hi[q] = max(max(ci[0][q], ci[1][q]), max(ci[2][q], ci[3][q]));
        }
        FF rv, rl;
        const int bp = m.fast_pure ? box_plane_side<4>(m, PL, i0, j0, k0, lo[0], hi[0], lo[1], hi[1], lo[2], hi[2], cx, cy, cz) : 0;
        if (bp != 0) {
            const float tv = tet_vol<float>(cx[0], cy[0], cz[0], cx[1], cy[1], cz[1], cx[2], cy[2], cz[2], cx[3], cy[3], cz[3]);
            rv = FF{tv, 0.f};
            rl = FF{bp > 0 ? tv : 0.f, 0.f};
            if (++leaves > CLIP_MAX_LEAVES) { err |= ERR_DEPTH; out_v = FF{0.f, 0.f}; out_l = FF{0.f, 0.f}; return; }
        } else {
            for (int q = 0; q < 3; ++q) {
                if (flags & (1 << q)) continue;
                if (hi[q] > lo[q]) { dir = q; cut = hi[q]; break; }
                flags |= 1 << q;
            }
            if (dir >= 0 && depth == CLIP_STACK32) { err |= ERR_DEPTH; dir = -1; }
            if (dir < 0) {
                if (++leaves > CLIP_MAX_LEAVES) { err |= ERR_DEPTH; out_v = FF{0.f, 0.f}; out_l = FF{0.f, 0.f}; return; }
                leaf32(m, tab, PL, i0, j0, k0, cx, cy, cz, ci[0][0], ci[0][1], ci[0][2], rv, rl, err);
            } else {
                Frame32& F = st[depth];
                const float pl = (float)cut;
                const float* cd = dir == 0 ? cx : (dir == 1 ? cy : cz);
                float d[4];
                for (int n = 0; n < 4; ++n) d[n] = cd[n] - pl;
                float c0 = d[0], c1 = d[1], c2 = d[2], c3 = d[3];
                const int cs = d2case(c0, c1, c2, c3, 1e-30f, err);
                int s1[8][3];
                for (int n = 0; n < 4; ++n) {
                    F.x[n] = cx[n]; F.y[n] = cy[n]; F.z[n] = cz[n];
                    s1[n][0] = ci[n][0]; s1[n][1] = ci[n][1]; s1[n][2] = ci[n][2];
                    s1[n][dir] = min(ci[n][dir], cut - 1);
                    F.ind[n] = pack3(s1[n][0], s1[n][1], s1[n][2]);
                }
                const CutCase& C = tab[cs];
                for (int n = 0; n < C.nvert; ++n) {
                    const int v1 = C.v1[n], v2 = C.v2[n];
                    const float den = d[v2] - d[v1];
                    const float mu = fminf(1.f, fmaxf(0.f, den != 0.f ? -d[v1] / den : 1.f));
                    const float x = fmaf(mu, F.x[v2] - F.x[v1], F.x[v1]);
                    const float y = fmaf(mu, F.y[v2] - F.y[v1], F.y[v1]);
                    const float z = fmaf(mu, F.z[v2] - F.z[v1], F.z[v1]);
                    F.x[4 + n] = x; F.y[4 + n] = y; F.z[4 + n] = z;
                    const int Iv[3] = {idx32(x, s1[n][0], rlo[0], rhi[0], err), idx32(y, s1[n][1], rlo[1], rhi[1], err),
                                       idx32(z, s1[n][2], rlo[2], rhi[2], err)};
                    int nv[3];
                    for (int q = 0; q < 3; ++q) {
                        const int a1 = unpack(F.ind[v1], q), a2 = unpack(F.ind[v2], q);
                        int val = max(Iv[q], min(a1, a2));
                        nv[q] = min(val, max(a1, a2));
                    }
                    nv[dir] = cut - 1;
                    F.ind[4 + n] = pack3(nv[0], nv[1], nv[2]);
                }
                F.vol = FF{0.f, 0.f};
                F.liq = FF{0.f, 0.f};
                F.meta = meta_pack(cs, 1, dir, flags, cut);
                ++depth;
                form_child32(F, tab, 0, cx, cy, cz, ci);
                continue;
            }
        }
        for (;;) {
            if (depth == 0) { out_v = rv; out_l = rl; return; }
            Frame32& F = st[depth - 1];
            ff_add(F.vol, rv);
            ff_add(F.liq, rl);
            const int cs = F.meta & 15, next = (F.meta >> 4) & 15;
            if (next < tab[cs].ntets) {
                form_child32(F, tab, next, cx, cy, cz, ci);
                F.meta += 1 << 4;
                flags = (F.meta >> 10) & 7;
                break;
            }
            rv = F.vol; rl = F.liq;
            --depth;
        }
    }
}

constexpr int SL32_THREADS = 128;

/* Stage 1 of the SL update, uniform work per band cell: the eight RK pre-image vertices
 * (cell2tets! with project_verts, src/VFgeom.jl:345-420) and their cells (pt2index!).  A cell
 * whose pre-image lies strictly on one side of every donor plane it reaches is finished here
 * (VF = 1 or 0); the others are compacted, with their vertices, for the clip stage. */
__global__ void __launch_bounds__(SL32_THREADS) k_sl32_pre(DevMesh m, float dt, double* __restrict__ VFout, Vel32 V,
                                                           Plane32 PL, const signed char* __restrict__ phase,
                                                           const int* __restrict__ list, const int* __restrict__ count,
                                                           int* work, int* slow_cells, float4* slow_verts,
                                                           int* slow_count, int* errw)
{
    const int lane = threadIdx.x & 31;
    const int n_items = *count;
    int err = 0;
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(work, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n_items) break;
        const int item = base + lane;
        bool slow = false;
        int L = 0;
        float px[8], py[8], pz[8];
        int vi[8][3];
        if (item < n_items) {
            L = list[item];
            int i, j, k;
            cell_of(m, L, i, j, k);
            const bool even = tess_even(m.tess, i, j, k);
            int rlo[3], rhi[3];
            rel_bounds(m, i, j, k, rlo, rhi);
#pragma unroll 1
            for (int v = 0; v < 8; ++v) {
                const int a = v & 1;
                float x = (float)(even ? a : 1 - a), y = (float)((v >> 1) & 1), z = (float)(v >> 2);
                project32(m, V, i, j, k, dt, x, y, z);
                px[v] = x; py[v] = y; pz[v] = z;
                vi[v][0] = idx32(x, 0, rlo[0], rhi[0], err);
                vi[v][1] = idx32(y, 0, rlo[1], rhi[1], err);
                vi[v][2] = idx32(z, 0, rlo[2], rhi[2], err);
            }
            slow = true;
            if (m.fast_pure) {
                int lo0 = vi[0][0], hi0 = vi[0][0], lo1 = vi[0][1], hi1 = vi[0][1], lo2 = vi[0][2], hi2 = vi[0][2];
                for (int v = 1; v < 8; ++v) {
                    lo0 = min(lo0, vi[v][0]); hi0 = max(hi0, vi[v][0]);
                    lo1 = min(lo1, vi[v][1]); hi1 = max(hi1, vi[v][1]);
                    lo2 = min(lo2, vi[v][2]); hi2 = max(hi2, vi[v][2]);
                }
                const int ph = box_plane_side<8>(m, PL, i, j, k, lo0, hi0, lo1, hi1, lo2, hi2, px, py, pz);
                if (ph != 0) {
                    float vol = 0.f;
                    for (int t = 0; t < 5; ++t)
                        vol += tet_vol32(px, py, pz, tet5(t, 0), tet5(t, 1), tet5(t, 2), tet5(t, 3));
                    vol *= even ? 1.f : -1.f;
                    if (vol > 0.25f && vol < 4.f) {
                        if (VFout) VFout[vidx(m, i, j, k)] = ph > 0 ? 1.0 : 0.0;
                        slow = false;
                    }
                }
            }
        }
        const int slot = warp_slot(slow, slow_count);
        if (slot >= 0) {
            slow_cells[slot] = L;
            const int stride = m.tess == 24 ? 16 : 8;
            for (int v = 0; v < 8; ++v) {
                const unsigned pk = pack3(vi[v][0], vi[v][1], vi[v][2]);
                slow_verts[(long)slot * stride + v] = make_float4(px[v], py[v], pz[v], __int_as_float((int)pk));
            }
            if (m.tess == 24) {
                /* mean points of the projected vertices (verts2tets!, src/VFgeom.jl:283-330),
                 * their cells seeded at the cell */
                int i, j, k, rlo[3], rhi[3];
                cell_of(m, L, i, j, k);
                rel_bounds(m, i, j, k, rlo, rhi);
                for (int f = -1; f < 6; ++f) {
                    const int nv = f < 0 ? 8 : 4;
                    float x = 0.f, y = 0.f, z = 0.f;
                    for (int n = 0; n < nv; ++n) {
                        const int v = f < 0 ? n : face24(f, n);
                        x = n == 0 ? px[v] : x + px[v];
                        y = n == 0 ? py[v] : y + py[v];
                        z = n == 0 ? pz[v] : z + pz[v];
                    }
                    x /= (float)nv; y /= (float)nv; z /= (float)nv;
                    const unsigned pk = pack3(idx32(x, 0, rlo[0], rhi[0], err), idx32(y, 0, rlo[1], rhi[1], err),
                                              idx32(z, 0, rlo[2], rhi[2], err));
                    slow_verts[(long)slot * 16 + 9 + f] = make_float4(x, y, z, __int_as_float((int)pk));
                }
            }
        }
    }
    if (err) atomicOr(errw, err);
}

/* ======================================================================================
 * Stage 2: warp-cooperative clip.  The clip of one tet is a tree (cutTet's recursion); run
 * thread per cell its depth varies so much that a warp idles most lanes.  Here a warp takes a
 * batch of cells and keeps their pending sub-tets in a LIFO stack in shared memory: each round
 * every lane pops one node and classifies it —
 *   pruned: strictly on one side of every donor plane of its index box (one leaf, no cuts),
 *   leaf:   one donor cell left, cut by that donor's PLIC plane,
 *   cut:    split by the next mesh plane, children pushed (warp prefix sum) —
 * and all three then run one code path: distances to a plane, d2case, new vertices on the
 * cut edges, then per child tet either its volume (leaf; liquid when on the plane's negative
 * side) or a push.  A pruned node is the one-tet case 1 (all liquid) or 16 (all gas).
 * Cutters whose children do not fit put their node back; if no cutter fits, the first one
 * finishes its node with the private-stack clip.  Lanes' partial sums are combined per cell
 * by a fixed shuffle tree; which lane takes which piece depends on the batch, so the last
 * bits of VF depend on how cells are batched.  vol and vLiq are sums over the same
 * pieces, so a pre-image that is all liquid gives VF = 1 exactly, as in the reference.
 *
 * Shared memory per warp: the node stack as four arrays of float4 (x, y, z, packed donor
 * indices), one per vertex, so a warp's pops and pushes hit consecutive 16-byte words; the
 * eight vertices of each lane's current cut (vertex-major, lane fastest); and the donor
 * planes of the 3x3x3 neighbourhood of each batch cell, which covers every donor a pre-image
 * reaches at CFL <= 0.5 (farther donors are read from global memory), with their constants
 * moved to the batch cell's frame and two 27-bit masks of its pure liquid and pure gas donors,
 * so that the pruning test evaluates planes only for the interface donors of a node's box.
 * ==================================================================================== */
constexpr int CLIPW_WARPS = 4;
/* Sizes: 2 cells per batch (10 seed tets for 5_tets) and 140 stack nodes per warp take
 * 55.2 KB of shared memory per block, the most that keeps four blocks (16 warps) on an SM.
 * Measured at 256^3: 4 cells and 112 nodes took 9.5 ms; a deeper stack puts fewer cutters
 * back (112 nodes: 11 of 31 cuts per step went back) and a smaller batch frees the plane
 * cache's share and halves the accumulator selects; 8.7 ms here.  Past 4 blocks per SM
 * (3 blocks, 12 warps) the clip is slower at any depth. */
constexpr int CLIPW_CAP = 140;  /* stack nodes per warp */
constexpr int CLIPW_BATCH = 2;  /* cells per warp batch */
constexpr int CLIPW_NBR = 27;   /* cached donor planes per batch cell */

/* acc[b] += x with a compile-time index (keeps the accumulators in registers) */
__device__ __forceinline__ void acc_add(FF* acc, int b, float x)
{
#pragma unroll
    for (int q = 0; q < CLIPW_BATCH; ++q)
        if (q == b) ff_add(acc[q], x);
}
__device__ __forceinline__ void acc_add(FF* acc, int b, const FF& x)
{
#pragma unroll
    for (int q = 0; q < CLIPW_BATCH; ++q)
        if (q == b) ff_add(acc[q], x);
}

struct ClipShared {
    CutCase tab[16];
    float4 stk[CLIPW_WARPS][4][CLIPW_CAP];
    float4 scr[8][CLIPW_WARPS * 32];
    float4 pl[CLIPW_WARPS][CLIPW_BATCH][CLIPW_NBR];
    uint2 msk[CLIPW_WARPS][CLIPW_BATCH];
};

/* Donor plane at index offset (a, b, c) from the batch cell (i0, j0, k0), in the batch cell's
 * frame: the cache holds the 3x3x3 neighbourhood already moved. */
__device__ __forceinline__ float4 nbr_plane(const DevMesh& m, const Plane32& PL, const float4* cache, int i0, int j0,
                                            int k0, int a, int b, int c)
{
    if ((unsigned)(a + 1) <= 2u && (unsigned)(b + 1) <= 2u && (unsigned)(c + 1) <= 2u)
        return cache[(c + 1) * 9 + (b + 1) * 3 + (a + 1)];
    float4 p = __ldg(PL.P + cidx(m, i0 + a, j0 + b, k0 + c));
    p.w = rel_dt(p, a, b, c);
    return p;
}

/* box_plane_side for a node: the common side of its four vertices against every donor plane
 * of its index box (at most 2x2x2), 0 when there is none.  LM and GM mark the pure liquid and
 * pure gas donors of the cached neighbourhood (bit (c+1)*9 + (b+1)*3 + (a+1)). */
__device__ __forceinline__ int node_side(const DevMesh& m, const Plane32& PL, const float4* cache, unsigned LM,
                                         unsigned GM, int i0, int j0, int k0, const int* lo, const int* hi,
                                         const float4* v)
{
    if (hi[0] - lo[0] > 1 || hi[1] - lo[1] > 1 || hi[2] - lo[2] > 1) return 0;
    if (lo[0] >= -1 && lo[1] >= -1 && lo[2] >= -1 && hi[0] <= 1 && hi[1] <= 1 && hi[2] <= 1) {
        /* box inside the cached neighbourhood: pure donors from the phase masks, planes only
         * for the interface donors */
        const unsigned row = (hi[0] > lo[0] ? 3u : 1u) << (lo[0] + 1);
        unsigned pln = row << (3 * (lo[1] + 1));
        if (hi[1] > lo[1]) pln |= row << (3 * (hi[1] + 1));
        unsigned box = pln << (9 * (lo[2] + 1));
        if (hi[2] > lo[2]) box |= pln << (9 * (hi[2] + 1));
        const bool liq = (box & LM) != 0u, gas = (box & GM) != 0u;
        if (liq && gas) return 0;
        int sd_all = liq ? 1 : (gas ? -1 : 2);
        for (unsigned im = box & ~(LM | GM); im != 0u; im &= im - 1u) {
            const int sd = plane_side4(cache[__ffs((int)im) - 1], v);
            if (sd == 0 || (sd_all != 2 && sd != sd_all)) return 0;
            sd_all = sd;
        }
        return sd_all == 2 ? 0 : sd_all;
    }
    int side = 2;
    for (int c = lo[2]; c <= hi[2]; ++c)
        for (int b = lo[1]; b <= hi[1]; ++b)
            for (int a = lo[0]; a <= hi[0]; ++a) {
                const int sd = plane_side4(nbr_plane(m, PL, cache, i0, j0, k0, a, b, c), v);
                if (sd == 0 || (side != 2 && sd != side)) return 0;
                side = sd;
            }
    return side;
}

__global__ void __launch_bounds__(CLIPW_WARPS * 32) k_sl32_clipw(DevMesh m, double* __restrict__ VFout, Plane32 PL,
                                                                  const int* __restrict__ slow_cells,
                                                                  const float4* __restrict__ slow_verts,
                                                                  const int* __restrict__ slow_count, int* work,
                                                                  int* errw)
{
    extern __shared__ __align__(16) unsigned char clip_smem[];
    ClipShared& S = *reinterpret_cast<ClipShared*>(clip_smem);
    for (int t = threadIdx.x; t < 16 * (int)sizeof(CutCase); t += blockDim.x)
        reinterpret_cast<char*>(S.tab)[t] = reinterpret_cast<const char*>(c_cut)[t];
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, tid = threadIdx.x;
    const unsigned lanemask_lt = (1u << lane) - 1u;
    const int n_cells = *slow_count;
    int err = 0;
    for (;;) {
        int base = 0;
        /* cells per batch: every tet of the batch is seeded in one round (<= 32 lanes) */
        const int B = (m.tess == 24 || m.fd) ? 1 : CLIPW_BATCH;
        if (lane == 0) base = atomicAdd(work, B);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n_cells) break;
        const int nb = min(B, n_cells - base);
        /* cell geometry of the batch (lane b holds cell b) */
        int ci_ = 0, cj_ = 0, ck_ = 0;
        if (lane < nb) cell_of(m, slow_cells[base + lane], ci_, cj_, ck_);
        /* donor planes of each batch cell's 3x3x3 neighbourhood */
        for (int t0 = 0; t0 < CLIPW_BATCH * CLIPW_NBR; t0 += 32) {
            const int t = t0 + lane;
            const int b = min(t / CLIPW_NBR, CLIPW_BATCH - 1);
            const int ii = __shfl_sync(0xffffffffu, ci_, b), jj = __shfl_sync(0xffffffffu, cj_, b),
                      kk = __shfl_sync(0xffffffffu, ck_, b);
            if (t < nb * CLIPW_NBR) {
                const int r = t - b * CLIPW_NBR;
                const int a = r % 3 - 1, bq = (r / 3) % 3 - 1, c = r / 9 - 1;
                float4 p = __ldg(PL.P + cidx(m, ii + a, jj + bq, kk + c));
                p.w = rel_dt(p, a, bq, c);
                S.pl[w][b][r] = p;
            }
        }
        __syncwarp();
        /* phase masks of the cached neighbourhoods: bit r set for a pure liquid (lm) or pure
         * gas (gm) donor; a pure cell's plane is (0, 0, 0, +-Lsum) */
#pragma unroll
        for (int bb = 0; bb < CLIPW_BATCH; ++bb) {
            float4 p = make_float4(1.f, 0.f, 0.f, 0.f);
            if (bb < nb && lane < CLIPW_NBR) p = S.pl[w][bb][lane];
            const bool pure = p.x == 0.f && p.y == 0.f && p.z == 0.f;
            const unsigned l_ = __ballot_sync(0xffffffffu, pure && p.w > 0.f);
            const unsigned g_ = __ballot_sync(0xffffffffu, pure && p.w < 0.f);
            if (lane == 0) S.msk[w][bb] = make_uint2(l_, g_);
        }
        __syncwarp();
        /* seed: lane q < 5*nb pushes tet q%5 of cell q/5, its tag (cell in batch) in vertex 0 */
        FF acc[CLIPW_BATCH], avol[CLIPW_BATCH];
#pragma unroll
        for (int b = 0; b < CLIPW_BATCH; ++b) { acc[b] = FF{0.f, 0.f}; avol[b] = FF{0.f, 0.f}; }
        /* under pressure_scheme "finite-difference" (5_tets, one cell a batch) lanes 5..16 seed
         * the twelve correction tets: (a, b, d, e) and (b, c, d, e) of each face, a..d its
         * projected corners (four of the cell's eight) and e its apex; a cell's liquid and volume
         * both carry its parity sign, which cancels in their ratio, as the cell tets' mirrored
         * corners do */
        const int ntet = tess_ntets(m.tess) + (m.fd ? 12 : 0), stride = (m.tess == 24 || m.fd) ? 16 : 8;
        const int ci0 = __shfl_sync(0xffffffffu, ci_, 0), cj0 = __shfl_sync(0xffffffffu, cj_, 0),
                  ck0 = __shfl_sync(0xffffffffu, ck_, 0); /* the batch's cell when it holds one */
        if (lane < ntet * nb) {
            const int b = lane / ntet, t = lane - ntet * b;
            int vid[4];
            if (t < 5 || m.tess != 5 || !m.fd) {
                for (int n = 0; n < 4; ++n) vid[n] = tess_tet(m.tess, t, n);
            } else {
                const int f = (t - 5) >> 1, hh = (t - 5) & 1, dir = f >> 1, up = f & 1;
                const bool ev_c = tess_even(5, ci0, cj0, ck0);
                const bool ev_h = up ? !ev_c : ev_c; /* the face's cell h = c + up e_dir */
                const int qn[3] = {flux_quad(dir, ev_h, hh), flux_quad(dir, ev_h, hh + 1), flux_quad(dir, ev_h, 3)};
                for (int r = 0; r < 3; ++r) {
                    int off[3];
                    flux_node(dir, ev_h, qn[r], off);
                    off[dir] += up; /* from h to the cell */
                    vid[r] = (ev_c ? off[0] : 1 - off[0]) + 2 * off[1] + 4 * off[2];
                }
                vid[3] = 8 + f;
            }
#pragma unroll
            for (int n = 0; n < 4; ++n) {
                float4 q = __ldg(slow_verts + (long)(base + b) * stride + vid[n]);
                if (n == 0) q.w = __int_as_float((int)(wbits(q) | ((unsigned)b << 24)));
                S.stk[w][n][lane] = q;
            }
        }
        int size = ntet * nb;
        __syncwarp();
        int guard = 0;
        while (size > 0) {
            if (++guard > 1 << 20) { err |= ERR_DEPTH; break; }
            /* phase 1: pop up to 32 nodes and classify them */
            const int n = min(32, size);
            const int top = size - n;
            const bool act = lane < n;
            float4 v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = act ? S.stk[w][q][top + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
            __syncwarp();
            size = top;
            const unsigned tag = wbits(v[0]) >> 24;
            const int b = (int)(tag & 3u);
            int flags = (int)((tag >> 2) & 7u);
            const int i0 = __shfl_sync(0xffffffffu, ci_, b), j0 = __shfl_sync(0xffffffffu, cj_, b),
                      k0 = __shfl_sync(0xffffffffu, ck_, b);
            const float4* cache = S.pl[w][b];
            int mode = 0; /* 0 idle, 1 leaf (pruned or PLIC), 2 cut */
            int cs = 0, dir = -1, cut = 0, nchild = 0;
            int rlo[3], rhi[3];
            int cind[4][3];
            float d0 = 0.f, d1 = 0.f, d2 = 0.f, d3 = 0.f;
            if (act) {
                rlo[0] = max(m.lo - i0, -REL); rlo[1] = max(m.lo - j0, -REL); rlo[2] = max(m.lo - k0, -REL);
                rhi[0] = min(m.hi[0] - i0, REL); rhi[1] = min(m.hi[1] - j0, REL); rhi[2] = min(m.hi[2] - k0, REL);
#pragma unroll
                for (int nn = 0; nn < 4; ++nn)
#pragma unroll
                    for (int q = 0; q < 3; ++q) cind[nn][q] = unpack(wbits(v[nn]), q);
                int lo[3], hi[3];
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    lo[q] = min(min(cind[0][q], cind[1][q]), min(cind[2][q], cind[3][q]));
                    hi[q] = max(max(cind[0][q], cind[1][q]), max(cind[2][q], cind[3][q]));
                }
                const uint2 mk = S.msk[w][b];
                const unsigned LM = mk.x, GM = mk.y;
                const int bp = m.fast_pure ? node_side(m, PL, cache, LM, GM, i0, j0, k0, lo, hi, v) : 0;
                if (bp != 0) {
                    mode = 1;
                    cs = bp > 0 ? 0 : 15;
                } else {
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        if (dir >= 0 || (flags & (1 << q))) continue;
                        if (hi[q] > lo[q]) { dir = q; cut = hi[q]; }
                        else flags |= 1 << q;
                    }
                    if (dir < 0) {
                        /* PLIC leaf (src/VFgeom.jl:760-830): the donor is the cell of vertex 0 */
                        mode = 1;
                        const int di = cind[0][0], dj = cind[0][1], dk = cind[0][2];
                        const float4 p = nbr_plane(m, PL, cache, i0, j0, k0, di, dj, dk);
                        const float Dt = p.w;
                        d0 = p.x * v[0].x + p.y * v[0].y + p.z * v[0].z - Dt;
                        d1 = p.x * v[1].x + p.y * v[1].y + p.z * v[1].z - Dt;
                        d2 = p.x * v[2].x + p.y * v[2].y + p.z * v[2].z - Dt;
                        d3 = p.x * v[3].x + p.y * v[3].y + p.z * v[3].z - Dt;
                    } else {
                        /* mesh-plane cut (src/VFgeom.jl:832-899) */
                        mode = 2;
                        const float pl = (float)cut;
                        d0 = (dir == 0 ? v[0].x : (dir == 1 ? v[0].y : v[0].z)) - pl;
                        d1 = (dir == 0 ? v[1].x : (dir == 1 ? v[1].y : v[1].z)) - pl;
                        d2 = (dir == 0 ? v[2].x : (dir == 1 ? v[2].y : v[2].z)) - pl;
                        d3 = (dir == 0 ? v[3].x : (dir == 1 ? v[3].y : v[3].z)) - pl;
                    }
                    cs = d2case(d0, d1, d2, d3, 1e-30f, err);
                    if (mode == 2) nchild = S.tab[cs].ntets;
                }
            }
            /* children placement: cutters in lane order while they fit.  Cutter q fits when the
             * children of the cutters up to q, plus one slot for each later cutter (which may
             * have to go back), fit above the remaining stack; the fitting cutters are a prefix
             * (each cutter adds nchild - 1 >= 0 to the need), so all placements fit.  If none
             * fits, the first cutter finishes its node privately. */
            int incl = nchild;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= off) incl += y;
            }
            const unsigned cutmask = __ballot_sync(0xffffffffu, mode == 2);
            const int later_cuts = __popc(cutmask) - __popc(cutmask & (lanemask_lt | (1u << lane)));
            const bool fits = mode == 2 && size + incl + later_cuts <= CLIPW_CAP;
            const unsigned fitmask = __ballot_sync(0xffffffffu, fits);
            bool back = mode == 2 && !fits;
            bool priv = false;
            if (!fitmask && cutmask && lane == __ffs(cutmask) - 1) { back = false; priv = true; }
            const int pushed = fits ? nchild : 0;
            int ipush = pushed;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, ipush, off);
                if (lane >= off) ipush += y;
            }
            const int tot_push = __shfl_sync(0xffffffffu, ipush, 31);
            const unsigned backmask = __ballot_sync(0xffffffffu, back);
            /* phase 2: leaves and fitting cuts share the plane-cut code */
            if (mode == 1 || fits) {
                const CutCase& C = S.tab[cs];
                unsigned s1p[4];
#pragma unroll
                for (int nn = 0; nn < 4; ++nn) {
                    int a0 = cind[nn][0], a1 = cind[nn][1], a2 = cind[nn][2];
                    if (mode == 2) {
                        if (dir == 0) a0 = min(a0, cut - 1);
                        else if (dir == 1) a1 = min(a1, cut - 1);
                        else a2 = min(a2, cut - 1);
                    }
                    s1p[nn] = pack3(a0, a1, a2);
                    S.scr[nn][tid] = make_float4(v[nn].x, v[nn].y, v[nn].z, __int_as_float((int)s1p[nn]));
                }
                const int nvert = C.nvert;
#pragma unroll
                for (int nn = 0; nn < 4; ++nn) {
                    if (nn >= nvert) break;
                    const int e1 = C.v1[nn], e2 = C.v2[nn];
                    const float4 A = S.scr[e1][tid], B = S.scr[e2][tid];
                    const float da = sel4(d0, d1, d2, d3, e1), db = sel4(d0, d1, d2, d3, e2);
                    const float den = db - da;
                    const float mu = fminf(1.f, fmaxf(0.f, den != 0.f ? -da / den : 1.f));
                    const float x = fmaf(mu, B.x - A.x, A.x);
                    const float y = fmaf(mu, B.y - A.y, A.y);
                    const float z = fmaf(mu, B.z - A.z, A.z);
                    unsigned pk = 0u;
                    if (mode == 2) {
                        /* pt2index! seeded with vertex nn's indices, bracketed by the edge's ends */
                        const unsigned pa = wbits(A), pb = wbits(B);
                        int nv[3];
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            const float u = q == 0 ? x : (q == 1 ? y : z);
                            const int Iv = idx32(u, unpack(s1p[nn], q), rlo[q], rhi[q], err);
                            const int a1 = unpack(pa, q), a2 = unpack(pb, q);
                            nv[q] = min(max(Iv, min(a1, a2)), max(a1, a2));
                        }
                        if (dir == 0) nv[0] = cut - 1;
                        else if (dir == 1) nv[1] = cut - 1;
                        else nv[2] = cut - 1;
                        pk = pack3(nv[0], nv[1], nv[2]);
                    }
                    S.scr[4 + nn][tid] = make_float4(x, y, z, __int_as_float((int)pk));
                }
                const int nt = C.ntets;
                if (mode == 1) {
                    for (int c = 0; c < nt; ++c) {
                        const float4 P0 = S.scr[C.vtet[c][0]][tid], P1 = S.scr[C.vtet[c][1]][tid];
                        const float4 P2 = S.scr[C.vtet[c][2]][tid], P3 = S.scr[C.vtet[c][3]][tid];
                        const float tv = tet_vol<float>(P0.x, P0.y, P0.z, P1.x, P1.y, P1.z, P2.x, P2.y, P2.z, P3.x,
                                                        P3.y, P3.z);
                        acc_add(avol, b, tv);
                        if (C.side[c] == 0) acc_add(acc, b, tv);
                    }
                } else {
                    const int pos = size + ipush - pushed;
                    const unsigned tagc = ((unsigned)b | ((unsigned)flags << 2)) << 24;
                    const int sh = 8 * dir;
                    for (int c = 0; c < nt; ++c) {
                        const bool up = C.side[c] == 1;
#pragma unroll
                        for (int nn = 0; nn < 4; ++nn) {
                            float4 q = S.scr[C.vtet[c][nn]][tid];
                            unsigned pk = wbits(q);
                            if (up) pk = (pk & ~(255u << sh)) | ((unsigned)(cut + 128) << sh);
                            if (nn == 0) pk |= tagc;
                            q.w = __int_as_float((int)pk);
                            S.stk[w][nn][pos + c] = q;
                        }
                    }
                }
            } else if (priv) {
                FF rv, rl;
                float cx[4], cy[4], cz[4];
#pragma unroll
                for (int nn = 0; nn < 4; ++nn) { cx[nn] = v[nn].x; cy[nn] = v[nn].y; cz[nn] = v[nn].z; }
                clip32(m, S.tab, PL, nullptr, i0, j0, k0, rlo, rhi, cx, cy, cz, cind, rv, rl, err);
                acc_add(avol, b, rv);
                acc_add(acc, b, rl);
            }
            /* nodes that did not fit go back above the children, in lane order */
            if (back) {
                const int p = size + tot_push + __popc(backmask & lanemask_lt);
#pragma unroll
                for (int q = 0; q < 4; ++q) S.stk[w][q][p] = v[q];
            }
            size += tot_push + __popc(backmask);
            __syncwarp();
        }
        /* per-cell liquid volume: fixed-order shuffle tree over lanes */
#pragma unroll
        for (int b = 0; b < CLIPW_BATCH; ++b) {
            if (b >= nb) break;
            double vl = (double)acc[b].hi + (double)acc[b].lo;
            double u = (double)avol[b].hi + (double)avol[b].lo;
            for (int off = 16; off > 0; off >>= 1) {
                vl += __shfl_xor_sync(0xffffffffu, vl, off);
                u += __shfl_xor_sync(0xffffffffu, u, off);
            }
            if (lane == b) {
                const double tetsign = tess_even(m.tess, ci_, cj_, ck_) ? 1.0 : -1.0;
                const double vol = tetsign * u, liq = tetsign * vl;
                if (!(vol > 0.0) || !isfinite(vol)) err |= ERR_VOLUME;
                VFout[vidx(m, ci_, cj_, ck_)] = liq / vol;
            }
        }
        __syncwarp();
    }
    if (err) atomicOr(errw, err);
}

/* ======================================================================================
 * SL update in flux form (flux.cuh): each face of the band region is swept once and its
 * volume and liquid are shared by the two cells beside it.
 *
 *   k_flux_lists : per band cell, the grid nodes it owns (the first band cell among the
 *                  node's eight, in offset order) and the faces it owns (its three low
 *                  faces, and a high face when the cell across it is not a band cell).
 *   k_flux_nodes : per owned node, its RK pre-image (project!, src/Tools.jl:392-418) as a
 *                  displacement in cell units; every face that holds the node reads this one
 *                  value, so neighbouring prisms share their vertices exactly.
 *   k_flux_faces : per face, the swept volume V of its prisms in FP64 from the node
 *                  displacements; a face whose points lie strictly on one side of every donor
 *                  plane of their index box gets its liquid F = V (or 0) here, the others are
 *                  listed for the clip.
 *   k_flux_clip  : warp-cooperative FP32 clip of the listed faces' prism tets (cutTet's cuts
 *                  and cut tables, src/VFgeom.jl:713-900), five faces per warp batch; each
 *                  face's liquid and volume are summed in float-float and its liquid F is
 *                  rescaled to the FP64 volume (below).
 *   k_flux_cells : per band cell, VFnew = (L + sum +-F) / (1 + sum +-V) in cell units.
 *
 * The FP32 clip's liquid F32 and volume V32 of a face are sums over the same pieces.  The
 * face's volume enters every cell in FP64 (V), and its liquid as F = F32 + (V - V32) w with
 * w = 1 when the face met no gas piece, 0 when it met no liquid piece, else F32/V32 clamped to
 * [0, 1]: a prism entirely in liquid then carries exactly its volume, so a cell whose
 * neighbourhood is all liquid keeps VF = 1 exactly (as the reference's vLiq/vol of equal
 * sums), and one in gas keeps 0.
 * ==================================================================================== */
struct FluxBufs {
    double* nd[3];    /* node displacement (cell units), indexed by the node's cell index */
    double2* fvf[3];  /* per face direction, by the high cell's index: (V, F) for the low cell */
    unsigned* nodes;  /* owned nodes: cell index of the node */
    unsigned* faces;  /* owned faces: (cell index of h) << 2 | dir */
    unsigned* clip;   /* faces for the clip */
    float4* fapex[3]; /* pressure_scheme "finite-difference": each face's correction apex (the low
                       * cell's frame), by direction and the high cell's index */
    int* n_nodes;
    int* n_faces;
    int* n_clip;
    int* work;        /* clip work counter */
};

__device__ __forceinline__ bool in_band(const DevMesh& m, const short* __restrict__ band, int i, int j, int k)
{
    if (i < 1 || j < 1 || k < 1 || i > m.N[0] || j > m.N[1] || k > m.N[2]) return false;
    return abs((int)band[cidx(m, i, j, k)]) <= m.nband;
}

__device__ __forceinline__ void cell_of_index(const DevMesh& m, long c, int& i, int& j, int& k)
{
    i = m.lo + (int)(c % m.cs1);
    j = m.lo + (int)((c / m.cs1) % (m.cs2 / m.cs1));
    k = m.lo + (int)(c / m.cs2);
}

constexpr int FLUX_THREADS = 128;

__global__ void __launch_bounds__(FLUX_THREADS) k_flux_lists(DevMesh m, const short* __restrict__ band,
                                                             const int* __restrict__ list, const int* __restrict__ count,
                                                             FluxBufs F)
{
    const int n = *count;
    for (int base = blockIdx.x * FLUX_THREADS; base < n; base += gridDim.x * FLUX_THREADS) {
        const int t = base + threadIdx.x;
        const bool act = t < n;
        int i = 0, j = 0, k = 0;
        if (act) cell_of(m, list[t], i, j, k);
        for (int o = 0; o < 8; ++o) {
            const int a = o & 1, b = (o >> 1) & 1, c = o >> 2;
            bool own = act;
            for (int o2 = 0; o2 < o; ++o2)
                own = own && !in_band(m, band, i + a - (o2 & 1), j + b - ((o2 >> 1) & 1), k + c - (o2 >> 2));
            const int slot = warp_slot(own, F.n_nodes);
            if (slot >= 0) F.nodes[slot] = (unsigned)cidx(m, i + a, j + b, k + c);
        }
        for (int f = 0; f < 6; ++f) {
            const int dir = f >> 1;
            int h[3] = {i, j, k};
            const bool high = f & 1;
            if (high) h[dir] += 1;
            const bool own = act && (!high || !in_band(m, band, h[0], h[1], h[2]));
            const int slot = warp_slot(own, F.n_faces);
            if (slot >= 0) F.faces[slot] = ((unsigned)cidx(m, h[0], h[1], h[2]) << 2) | (unsigned)dir;
        }
    }
}

/* Staggered trilinear interpolation of an FP64 face-velocity array (physical units), in
 * the reference's lerp order along x, then y, then z. */
__device__ __forceinline__ double tri64(const DevMesh& m, const double* __restrict__ f, int I, int J, int K, double wx,
                                       double wy, double wz)
{
    const long b = cidx(m, I, J, K);
    const long sj = m.cs1, sk = m.cs2;
    const double f000 = __ldg(f + b), f100 = __ldg(f + b + 1), f010 = __ldg(f + b + sj), f110 = __ldg(f + b + 1 + sj);
    const double f001 = __ldg(f + b + sk), f101 = __ldg(f + b + 1 + sk), f011 = __ldg(f + b + sj + sk),
                 f111 = __ldg(f + b + 1 + sj + sk);
    const double x00 = f000 + wx * (f100 - f000), x10 = f010 + wx * (f110 - f010);
    const double x01 = f001 + wx * (f101 - f001), x11 = f011 + wx * (f111 - f011);
    const double y0 = x00 + wy * (x10 - x00), y1 = x01 + wy * (x11 - x01);
    return y0 + wz * (y1 - y0);
}

struct Vel64c {
    const double *uf, *vf, *wf; /* face velocities, physical units */
    double id[3];               /* 1/dx, 1/dy, 1/dz: to cells per unit time */
};

/* get_velocity_{u,v,w}face (src/Tools.jl:516-641) on the uniform mesh, at a point given in
 * cell units relative to cell (i0, j0, k0): floor() for the interval search, clamped to
 * [imino_, imaxo_-1]; the result in cells per unit time. */
__device__ __forceinline__ void vel64c(const DevMesh& m, const Vel64c& V, int i0, int j0, int k0, double x, double y,
                                       double z, double* u)
{
    const double B = 1.0e6;
    const double fx = fmin(fmax(floor(x), -B), B), fy = fmin(fmax(floor(y), -B), B), fz = fmin(fmax(floor(z), -B), B);
    const double gx = fmin(fmax(floor(x - 0.5), -B), B), gy = fmin(fmax(floor(y - 0.5), -B), B),
                 gz = fmin(fmax(floor(z - 0.5), -B), B);
    const int Fx = clampi(i0 + (int)fx, m.lo, m.hi[0] - 1), Cx = clampi(i0 + (int)gx, m.lo, m.hi[0] - 1);
    const int Fy = clampi(j0 + (int)fy, m.lo, m.hi[1] - 1), Cy = clampi(j0 + (int)gy, m.lo, m.hi[1] - 1);
    const int Fz = clampi(k0 + (int)fz, m.lo, m.hi[2] - 1), Cz = clampi(k0 + (int)gz, m.lo, m.hi[2] - 1);
    const double wfx = x - (double)(Fx - i0), wcx = x - ((double)(Cx - i0) + 0.5);
    const double wfy = y - (double)(Fy - j0), wcy = y - ((double)(Cy - j0) + 0.5);
    const double wfz = z - (double)(Fz - k0), wcz = z - ((double)(Cz - k0) + 0.5);
    u[0] = tri64(m, V.uf, Fx, Cy, Cz, wfx, wcy, wcz) * V.id[0];
    u[1] = tri64(m, V.vf, Cx, Fy, Cz, wcx, wfy, wcz) * V.id[1];
    u[2] = tri64(m, V.wf, Cx, Cy, Fz, wcx, wcy, wfz) * V.id[2];
}

/* A grid node's pre-image (project!, src/Tools.jl:392-418) as a displacement in cell units, in
 * FP64: the face volumes that enter the mass are only as good as the nodes they are built on
 * (the Zalesak rotation uses the FP32 form of the other kernels). */
__device__ __forceinline__ void node_disp64(const DevMesh& m, const Vel64c& V, const Vel32& V32, int i, int j, int k,
                                            double dt, double* disp)
{
    if (m.projection == 3) {
        float x = 0.f, y = 0.f, z = 0.f;
        project32(m, V32, i, j, k, (float)dt, x, y, z);
        disp[0] = x; disp[1] = y; disp[2] = z;
        return;
    }
    double u1[3];
    vel64c(m, V, i, j, k, 0.0, 0.0, 0.0, u1);
    if (m.projection == 0) {
        for (int q = 0; q < 3; ++q) disp[q] = -dt * u1[q];
        return;
    }
    const double h = 0.5 * dt;
    double u2[3];
    vel64c(m, V, i, j, k, -h * u1[0], -h * u1[1], -h * u1[2], u2);
    if (m.projection == 1) {
        for (int q = 0; q < 3; ++q) disp[q] = -dt * u2[q];
        return;
    }
    double u3[3], u4[3];
    vel64c(m, V, i, j, k, -h * u2[0], -h * u2[1], -h * u2[2], u3);
    vel64c(m, V, i, j, k, -dt * u3[0], -dt * u3[1], -dt * u3[2], u4);
    const double c = -dt / 6.0;
#pragma unroll
    for (int q = 0; q < 3; ++q) disp[q] = c * (((u1[q] + 2.0 * u2[q]) + 2.0 * u3[q]) + u4[q]);
}

__global__ void __launch_bounds__(FLUX_THREADS) k_flux_nodes(DevMesh m, double dt, Vel64c V, Vel32 V32, FluxBufs F)
{
    const int n = *F.n_nodes;
    for (int t = blockIdx.x * FLUX_THREADS + threadIdx.x; t < n; t += gridDim.x * FLUX_THREADS) {
        const unsigned c = F.nodes[t];
        int i, j, k;
        cell_of_index(m, c, i, j, k);
        double d[3];
        node_disp64(m, V, V32, i, j, k, dt, d);
        F.nd[0][c] = d[0];
        F.nd[1][c] = d[1];
        F.nd[2][c] = d[2];
    }
}

/* The face's points in the low cell's frame (cell units): corners P[0..3] and, for 24_tets,
 * the face centre P[4]; their moved copies Q. */
__device__ __forceinline__ void face_points(const DevMesh& m, const FluxBufs& F, int dir, int hi, int hj, int hk,
                                            double (*P)[3], double (*Q)[3])
{
    int s, t;
    flux::face_axes(dir, s, t);
    for (int p = 0; p < 4; ++p) {
        int i, j, k;
        flux::corner_node(dir, hi, hj, hk, p, i, j, k);
        const long c = cidx(m, i, j, k);
        P[p][dir] = 1.0;
        P[p][s] = (double)flux::corner_s(p);
        P[p][t] = (double)flux::corner_t(p);
        for (int q = 0; q < 3; ++q) Q[p][q] = P[p][q] + F.nd[q][c];
    }
    if (m.tess != 24) return; /* the face centre is a point of 24_tets only */
    P[4][dir] = 1.0;
    P[4][s] = 0.5;
    P[4][t] = 0.5;
    for (int q = 0; q < 3; ++q) Q[4][q] = 0.25 * (((Q[0][q] + Q[1][q]) + Q[3][q]) + Q[2][q]);
}

__device__ __forceinline__ void face_decode(const DevMesh& m, unsigned code, int& dir, int& hi, int& hj, int& hk)
{
    dir = (int)(code & 3u);
    cell_of_index(m, (long)(code >> 2), hi, hj, hk);
}

/* Point id (0..3 corners, 5..8 their moved copies) of a 5_tets or 6_tets face, as face_points
 * forms it (the same FP64 sum for a moved corner, so the same bits), rounded to FP32: a seed
 * lane forms only the four points of its own tet. */
__device__ __forceinline__ float4 seed_point(const DevMesh& m, const FluxBufs& F, int dir, int hi, int hj, int hk,
                                             int id)
{
    int s, t;
    flux::face_axes(dir, s, t);
    const int p = id < 5 ? id : id - 5;
    const float cs = (float)flux::corner_s(p), ct = (float)flux::corner_t(p);
    const float b0 = dir == 0 ? 1.f : (s == 0 ? cs : ct);
    const float b1 = dir == 1 ? 1.f : (s == 1 ? cs : ct);
    const float b2 = dir == 2 ? 1.f : (s == 2 ? cs : ct);
    if (id < 5) return make_float4(b0, b1, b2, 0.f);
    int i, j, k;
    flux::corner_node(dir, hi, hj, hk, p, i, j, k);
    const long c = cidx(m, i, j, k);
    return make_float4((float)((double)b0 + F.nd[0][c]), (float)((double)b1 + F.nd[1][c]),
                       (float)((double)b2 + F.nd[2][c]), 0.f);
}

__global__ void __launch_bounds__(FLUX_THREADS) k_flux_faces(DevMesh m, Plane32 PL, FluxBufs F, double dt, Vel64c U,
                                                             int* errw)
{
    const int n = *F.n_faces;
    int err = 0;
    for (int base = blockIdx.x * FLUX_THREADS; base < n; base += gridDim.x * FLUX_THREADS) {
        const int t = base + threadIdx.x;
        bool clip = false;
        unsigned code = 0;
        float4 cap = make_float4(0.f, 0.f, 0.f, 0.f);
        if (t < n) {
            code = F.faces[t];
            int dir, hi, hj, hk;
            face_decode(m, code, dir, hi, hj, hk);
            double P[5][3], Q[5][3];
            face_points(m, F, dir, hi, hj, hk, P, Q);
            const int npt = m.tess == 24 ? 5 : 4;
            const long hc = (long)(code >> 2);
            bool flat = !m.fd; /* with the correction tets every face carries volume */
            for (int p = 0; p < npt; ++p) flat = flat && Q[p][dir] == 1.0;
            if (flat) {
                F.fvf[dir][hc] = make_double2(0.0, 0.0); /* no motion across the face: a flat prism */
            } else {
                int tri[4][3], sg[4];
                const int nt = flux::face_triangles(m.tess, dir, flux::face_main_diagonal(m.tess, dir, hi, hj, hk),
                                                    tri, sg);
                /* the prism's three tet volumes in closed form: with e1 = b - a, e2 = c - a in
                 * the face plane and displacements da, db, dc (a' = a + da, ...),
                 *   6 V = (e1 x e2).(da + db + dc) + e1.(dc x db) + da.(e1 x dc) + da.(db x e2)
                 *         + da.(db x dc),
                 * the sum of tet_vol over (a,b,c,c'), (a,b,c',b'), (a,a',b',c') */
                /* with the two terms in e1 merged (e1.(dc x db) + da.(e1 x dc) = e1.(dc x (da + db)))
                 * and da.(db x e2) = e2.(da x db):
                 *   6 V = N.(da + db + dc) + e1.(dc x (da + db)) + e2.(da x db) + da.(db x dc)
                 * (two triple products fewer on the FP64 pipe, the kernel's bound) */
                double V6 = 0.0; /* 6 V, divided once */
                auto cross = [](const double* u, const double* w, double* r) {
                    r[0] = u[1] * w[2] - u[2] * w[1];
                    r[1] = u[2] * w[0] - u[0] * w[2];
                    r[2] = u[0] * w[1] - u[1] * w[0];
                };
                auto dot = [](const double* u, const double* w) { return (u[0] * w[0] + u[1] * w[1]) + u[2] * w[2]; };
                for (int tr = 0; tr < nt; ++tr) {
                    const int ia = tri[tr][0], ib = tri[tr][1], ic = tri[tr][2];
                    double e1[3], e2[3], da[3], db[3], dc[3], sd[3], ab[3], N[3], t[3];
                    for (int q = 0; q < 3; ++q) {
                        e1[q] = P[ib][q] - P[ia][q];
                        e2[q] = P[ic][q] - P[ia][q];
                        da[q] = Q[ia][q] - P[ia][q];
                        db[q] = Q[ib][q] - P[ib][q];
                        dc[q] = Q[ic][q] - P[ic][q];
                        ab[q] = da[q] + db[q];
                        sd[q] = ab[q] + dc[q];
                    }
                    cross(e1, e2, N);
                    double six = dot(N, sd);
                    cross(dc, ab, t);
                    six += dot(e1, t);
                    cross(da, db, t);
                    six += dot(e2, t);
                    cross(db, dc, t);
                    six += dot(da, t);
                    V6 += sg[tr] > 0 ? six : -six;
                }
                double V = V6 / 6.0;
                double ape[3] = {0.0, 0.0, 0.0};
                if (m.fd) {
                    const double* u = dir == 0 ? U.uf : (dir == 1 ? U.vf : U.wf);
                    V += flux::face_correction(dir, hi, hj, hk, dt * (u[hc] * U.id[dir]), P, Q, ape);
                }
                /* index box of the prism points, relative to the low cell l = h - e_dir */
                int li = hi, lj = hj, lk = hk;
                if (dir == 0) --li; else if (dir == 1) --lj; else --lk;
                int rlo[3], rhi[3];
                rel_bounds(m, li, lj, lk, rlo, rhi);
                float px[10], py[10], pz[10];
                int lo[3] = {0, 0, 0}, hiB[3] = {0, 0, 0};
                lo[dir] = 1 << 20; hiB[dir] = -(1 << 20);
                for (int p = 0; p < npt; ++p) {
                    px[p] = (float)P[p][0]; py[p] = (float)P[p][1]; pz[p] = (float)P[p][2];
                    px[npt + p] = (float)Q[p][0]; py[npt + p] = (float)Q[p][1]; pz[npt + p] = (float)Q[p][2];
                    const float u[3] = {px[npt + p], py[npt + p], pz[npt + p]};
                    for (int q = 0; q < 3; ++q) {
                        const int I = idx32(u[q], 0, rlo[q], rhi[q], err);
                        lo[q] = min(lo[q], I);
                        hiB[q] = max(hiB[q], I);
                    }
                }
                /* along dir the prism also spans the layers between the face (between
                 * layers 0 and 1) and its moved points */
                lo[dir] = min(lo[dir], 1);
                hiB[dir] = max(hiB[dir], 0);
                if (m.fd) {
                    /* the correction tets span the moved corners and the apex */
                    px[8] = (float)ape[0]; py[8] = (float)ape[1]; pz[8] = (float)ape[2];
                    cap = make_float4(px[8], py[8], pz[8], 0.f);
                    const float u[3] = {px[8], py[8], pz[8]};
                    for (int q = 0; q < 3; ++q) {
                        const int I = idx32(u[q], 0, rlo[q], rhi[q], err);
                        lo[q] = min(lo[q], I);
                        hiB[q] = max(hiB[q], I);
                    }
                }
                int side = 0;
                if (m.fast_pure) {
                    side = npt == 5 ? box_plane_side<10>(m, PL, li, lj, lk, lo[0], hiB[0], lo[1], hiB[1], lo[2], hiB[2],
                                                         px, py, pz)
                         : m.fd     ? box_plane_side<9>(m, PL, li, lj, lk, lo[0], hiB[0], lo[1], hiB[1], lo[2], hiB[2],
                                                        px, py, pz)
                                    : box_plane_side<8>(m, PL, li, lj, lk, lo[0], hiB[0], lo[1], hiB[1], lo[2], hiB[2],
                                                        px, py, pz);
                }
                F.fvf[dir][hc] = make_double2(V, side > 0 ? V : 0.0);
                if (m.fd) F.fapex[dir][hc] = cap;
                clip = side == 0;
            }
        }
        const int slot = warp_slot(clip, F.n_clip);
        if (slot >= 0) F.clip[slot] = code;
    }
    if (err) atomicOr(errw, err);
}

constexpr int FCLIP_BATCH = 5; /* faces per warp batch: 30 seed tets for 5_tets and 6_tets */
constexpr int CAPEX = 10;      /* seed point id of a face's correction apex */
constexpr int FCLIP_CAP = 120; /* stack nodes per warp: keeps the block at 55.3 KB, four per SM */

/* acc[b] += x for a lane-varying b over register-held accumulators: the accumulator is
 * selected, added to once and written back (one float-float add in the code instead of one
 * per face of the batch) */
__device__ __forceinline__ void facc_add(FF* acc, int b, const FF& x)
{
    FF s = acc[0];
#pragma unroll
    for (int q = 1; q < FCLIP_BATCH; ++q)
        if (q == b) s = acc[q];
    ff_add(s, x);
#pragma unroll
    for (int q = 0; q < FCLIP_BATCH; ++q)
        if (q == b) acc[q] = s;
}
__device__ __forceinline__ void fflag_or(int* f, int b, int x)
{
#pragma unroll
    for (int q = 0; q < FCLIP_BATCH; ++q)
        if (q == b) f[q] |= x;
}

struct FluxShared {
    CutCase tab[16];
    float4 stk[CLIPW_WARPS][4][FCLIP_CAP];
    float4 scr[8][CLIPW_WARPS * 32];
    float4 pl[CLIPW_WARPS][FCLIP_BATCH][CLIPW_NBR];
    uint2 msk[CLIPW_WARPS][FCLIP_BATCH];
};

enum : int { PIECE_LIQ = 1, PIECE_GAS = 2 };

/* The clip's seeding by tessellation and pressure scheme, fixed per instantiation: the
 * kernel is bound by instruction fetch, and each instantiation carries only its own seeding
 * code. */
enum : int { SEED_PRISM = 0, SEED_FD = 1, SEED_24 = 2 };

template <int SEED>
__global__ void __launch_bounds__(CLIPW_WARPS * 32, 4) k_flux_clip(DevMesh m, Plane32 PL, FluxBufs F, int* errw)
{
    extern __shared__ __align__(16) unsigned char flux_smem[];
    FluxShared& S = *reinterpret_cast<FluxShared*>(flux_smem);
    for (int t = threadIdx.x; t < 16 * (int)sizeof(CutCase); t += blockDim.x)
        reinterpret_cast<char*>(S.tab)[t] = reinterpret_cast<const char*>(c_cut)[t];
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, tid = threadIdx.x;
    const unsigned lanemask_lt = (1u << lane) - 1u;
    const int n_faces = *F.n_clip;
    /* seed tets per face: the prism's, and under pressure_scheme "finite-difference" (5_tets)
     * the two correction tets */
    constexpr bool T24 = SEED == SEED_24, FD = SEED == SEED_FD;
    const int ntet = T24 ? 12 : (FD ? 8 : 6);
    const int B = T24 ? 2 : (FD ? 4 : FCLIP_BATCH);
    int err = 0;
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(F.work, B);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n_faces) break;
        const int nb = min(B, n_faces - base);
        /* lane b < nb holds face b: its code and low cell */
        unsigned code_ = 0;
        int fd_ = 0, li_ = 0, lj_ = 0, lk_ = 0;
        if (lane < nb) {
            code_ = F.clip[base + lane];
            int hi, hj, hk;
            face_decode(m, code_, fd_, hi, hj, hk);
            li_ = hi - (fd_ == 0); lj_ = hj - (fd_ == 1); lk_ = hk - (fd_ == 2);
        }
        /* donor planes of each face's low cell's 3x3x3 neighbourhood, in that cell's frame */
        for (int t0 = 0; t0 < FCLIP_BATCH * CLIPW_NBR; t0 += 32) {
            const int t = t0 + lane;
            const int b = min(t / CLIPW_NBR, FCLIP_BATCH - 1);
            const int ii = __shfl_sync(0xffffffffu, li_, b), jj = __shfl_sync(0xffffffffu, lj_, b),
                      kk = __shfl_sync(0xffffffffu, lk_, b);
            if (t < nb * CLIPW_NBR) {
                const int r = t - b * CLIPW_NBR;
                const int a = r % 3 - 1, bq = (r / 3) % 3 - 1, c = r / 9 - 1;
                float4 p = __ldg(PL.P + cidx(m, ii + a, jj + bq, kk + c));
                p.w = rel_dt(p, a, bq, c);
                S.pl[w][b][r] = p;
            }
        }
        __syncwarp();
#pragma unroll
        for (int bb = 0; bb < FCLIP_BATCH; ++bb) {
            float4 p = make_float4(1.f, 0.f, 0.f, 0.f);
            if (bb < nb && lane < CLIPW_NBR) p = S.pl[w][bb][lane];
            const bool pure = p.x == 0.f && p.y == 0.f && p.z == 0.f;
            const unsigned l_ = __ballot_sync(0xffffffffu, pure && p.w > 0.f);
            const unsigned g_ = __ballot_sync(0xffffffffu, pure && p.w < 0.f);
            if (lane == 0) S.msk[w][bb] = make_uint2(l_, g_);
        }
        __syncwarp();
        /* seed: lane q < ntet*nb takes prism tet q % ntet of face q / ntet, oriented for the
         * low cell (two vertices swapped where sigma is -1); its tag (face in batch) in
         * vertex 0 */
        FF acc[FCLIP_BATCH], avol[FCLIP_BATCH];
        int flg[FCLIP_BATCH];
#pragma unroll
        for (int b = 0; b < FCLIP_BATCH; ++b) { acc[b] = FF{0.f, 0.f}; avol[b] = FF{0.f, 0.f}; flg[b] = 0; }
        const unsigned code = __shfl_sync(0xffffffffu, code_, min(lane / ntet, FCLIP_BATCH - 1));
        if (lane < ntet * nb) {
            const int b = lane / ntet, n = lane - ntet * b;
            int dir, hi, hj, hk;
            face_decode(m, code, dir, hi, hj, hk);
            int q[4];
            if (!FD || n < 6) {
                int tri[4][3], sg[4];
                flux::face_triangles(m.tess, dir, flux::face_main_diagonal(m.tess, dir, hi, hj, hk), tri, sg);
                flux::prism_tet(tri[n / 3], n % 3, q);
                if (sg[n / 3] < 0) { const int x = q[0]; q[0] = q[1]; q[1] = x; }
            } else {
                /* correction tet n - 6: (a, b, d, e) or (b, c, d, e) over the projected quad
                 * (moved corners), e the apex (id CAPEX); with the low cell's parity sign, so
                 * swapped where the face's cell is even */
                int s_, t_;
                flux::face_axes(dir, s_, t_);
                const bool ev = tess_even(5, hi, hj, hk);
                const int h = n - 6;
                const int qn[3] = {flux_quad(dir, ev, h), flux_quad(dir, ev, h + 1), flux_quad(dir, ev, 3)};
                for (int r = 0; r < 3; ++r) {
                    int off[3];
                    flux_node(dir, ev, qn[r], off);
                    q[r] = off[s_] + 2 * off[t_] + flux::MOVED;
                }
                q[3] = CAPEX;
                if (ev) { const int x = q[0]; q[0] = q[1]; q[1] = x; }
            }
            const int li = hi - (dir == 0), lj = hj - (dir == 1), lk = hk - (dir == 2);
            int rlo[3], rhi[3];
            rel_bounds(m, li, lj, lk, rlo, rhi);
            float4 v[4];
            int I[4][3];
            int mlo = 1 << 20;
            if (T24) {
                double P[5][3], Q[5][3];
                face_points(m, F, dir, hi, hj, hk, P, Q);
                for (int nn = 0; nn < 4; ++nn) {
                    const double* x = q[nn] < 5 ? P[q[nn]] : Q[q[nn] - 5];
                    v[nn] = make_float4((float)x[0], (float)x[1], (float)x[2], 0.f);
                }
            } else {
                for (int nn = 0; nn < 4; ++nn) {
                    if (FD && q[nn] == CAPEX) {
                        const float4 e = F.fapex[dir][(long)(code >> 2)];
                        v[nn] = make_float4(e.x, e.y, e.z, 0.f);
                    } else {
                        v[nn] = seed_point(m, F, dir, hi, hj, hk, q[nn]);
                    }
                }
            }
            for (int nn = 0; nn < 4; ++nn) {
                if (q[nn] >= 5) {
                    I[nn][0] = idx32(v[nn].x, 0, rlo[0], rhi[0], err);
                    I[nn][1] = idx32(v[nn].y, 0, rlo[1], rhi[1], err);
                    I[nn][2] = idx32(v[nn].z, 0, rlo[2], rhi[2], err);
                    mlo = min(mlo, I[nn][dir]);
                }
            }
            /* the face's own points lie on the plane between l (0) and h (1) and inside the
             * tangential range of l's column: index 0 across, and along dir the side of this
             * tet's moved points (either index contains them) */
            for (int nn = 0; nn < 4; ++nn)
                if (q[nn] < 5) {
                    I[nn][0] = I[nn][1] = I[nn][2] = 0;
                    I[nn][dir] = mlo >= 1 ? 1 : 0;
                }
            for (int nn = 0; nn < 4; ++nn) {
                unsigned pk = pack3(I[nn][0], I[nn][1], I[nn][2]);
                if (nn == 0) pk |= (unsigned)b << 24;
                v[nn].w = __int_as_float((int)pk);
                S.stk[w][nn][lane] = v[nn];
            }
        }
        int size = ntet * nb;
        __syncwarp();
        int guard = 0;
        while (size > 0) {
            if (++guard > 1 << 20) { err |= ERR_DEPTH; break; }
            const int n = min(32, size);
            const int top = size - n;
            const bool act = lane < n;
            float4 v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = act ? S.stk[w][q][top + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
            __syncwarp();
            size = top;
            const unsigned tag = wbits(v[0]) >> 24;
            const int b = (int)(tag & 7u);
            int flags = (int)((tag >> 3) & 7u);
            const int i0 = __shfl_sync(0xffffffffu, li_, b), j0 = __shfl_sync(0xffffffffu, lj_, b),
                      k0 = __shfl_sync(0xffffffffu, lk_, b);
            const float4* cache = S.pl[w][b];
            int mode = 0; /* 0 idle, 1 leaf (pruned or PLIC), 2 cut */
            int cs = 0, dir = -1, cut = 0, nchild = 0;
            int rlo[3], rhi[3];
            int cind[4][3];
            float d0 = 0.f, d1 = 0.f, d2 = 0.f, d3 = 0.f;
            if (act) {
                rel_bounds(m, i0, j0, k0, rlo, rhi);
#pragma unroll
                for (int nn = 0; nn < 4; ++nn)
#pragma unroll
                    for (int q = 0; q < 3; ++q) cind[nn][q] = unpack(wbits(v[nn]), q);
                int lo[3], hi[3];
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    lo[q] = min(min(cind[0][q], cind[1][q]), min(cind[2][q], cind[3][q]));
                    hi[q] = max(max(cind[0][q], cind[1][q]), max(cind[2][q], cind[3][q]));
                }
                const uint2 mk = S.msk[w][b];
                const int bp = m.fast_pure ? node_side(m, PL, cache, mk.x, mk.y, i0, j0, k0, lo, hi, v) : 0;
                if (bp != 0) {
                    mode = 1;
                    cs = bp > 0 ? 0 : 15;
                } else {
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        if (dir >= 0 || (flags & (1 << q))) continue;
                        if (hi[q] > lo[q]) { dir = q; cut = hi[q]; }
                        else flags |= 1 << q;
                    }
                    if (dir < 0) {
                        mode = 1;
                        const float4 p = nbr_plane(m, PL, cache, i0, j0, k0, cind[0][0], cind[0][1], cind[0][2]);
                        const float Dt = p.w;
                        d0 = p.x * v[0].x + p.y * v[0].y + p.z * v[0].z - Dt;
                        d1 = p.x * v[1].x + p.y * v[1].y + p.z * v[1].z - Dt;
                        d2 = p.x * v[2].x + p.y * v[2].y + p.z * v[2].z - Dt;
                        d3 = p.x * v[3].x + p.y * v[3].y + p.z * v[3].z - Dt;
                    } else {
                        mode = 2;
                        const float pl = (float)cut;
                        d0 = (dir == 0 ? v[0].x : (dir == 1 ? v[0].y : v[0].z)) - pl;
                        d1 = (dir == 0 ? v[1].x : (dir == 1 ? v[1].y : v[1].z)) - pl;
                        d2 = (dir == 0 ? v[2].x : (dir == 1 ? v[2].y : v[2].z)) - pl;
                        d3 = (dir == 0 ? v[3].x : (dir == 1 ? v[3].y : v[3].z)) - pl;
                    }
                    cs = d2case(d0, d1, d2, d3, 1e-30f, err);
                    if (mode == 2) nchild = S.tab[cs].ntets;
                }
            }
            int incl = nchild;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= off) incl += y;
            }
            const unsigned cutmask = __ballot_sync(0xffffffffu, mode == 2);
            const int later_cuts = __popc(cutmask) - __popc(cutmask & (lanemask_lt | (1u << lane)));
            const bool fits = mode == 2 && size + incl + later_cuts <= FCLIP_CAP;
            const unsigned fitmask = __ballot_sync(0xffffffffu, fits);
            bool back = mode == 2 && !fits;
            bool priv = false;
            if (!fitmask && cutmask && lane == __ffs(cutmask) - 1) { back = false; priv = true; }
            const int pushed = fits ? nchild : 0;
            int ipush = pushed;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, ipush, off);
                if (lane >= off) ipush += y;
            }
            const int tot_push = __shfl_sync(0xffffffffu, ipush, 31);
            const unsigned backmask = __ballot_sync(0xffffffffu, back);
            if (mode == 1 || fits) {
                const CutCase& C = S.tab[cs];
                unsigned s1p[4];
#pragma unroll
                for (int nn = 0; nn < 4; ++nn) {
                    int a0 = cind[nn][0], a1 = cind[nn][1], a2 = cind[nn][2];
                    if (mode == 2) {
                        if (dir == 0) a0 = min(a0, cut - 1);
                        else if (dir == 1) a1 = min(a1, cut - 1);
                        else a2 = min(a2, cut - 1);
                    }
                    s1p[nn] = pack3(a0, a1, a2);
                    S.scr[nn][tid] = make_float4(v[nn].x, v[nn].y, v[nn].z, __int_as_float((int)s1p[nn]));
                }
                const int nvert = C.nvert;
#pragma unroll 1 /* rolled: a smaller loop body (the kernel is instruction-fetch bound) */
                for (int nn = 0; nn < nvert; ++nn) {
                    const int e1 = C.v1[nn], e2 = C.v2[nn];
                    const float4 A = S.scr[e1][tid], Bv = S.scr[e2][tid];
                    const float da = sel4(d0, d1, d2, d3, e1), db = sel4(d0, d1, d2, d3, e2);
                    const float den = db - da;
                    const float mu = fminf(1.f, fmaxf(0.f, den != 0.f ? -da / den : 1.f));
                    const float x = fmaf(mu, Bv.x - A.x, A.x);
                    const float y = fmaf(mu, Bv.y - A.y, A.y);
                    const float z = fmaf(mu, Bv.z - A.z, A.z);
                    unsigned pk = 0u;
                    if (mode == 2) {
                        const unsigned pa = wbits(A), pb = wbits(Bv);
                        int nv[3];
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            const float u = q == 0 ? x : (q == 1 ? y : z);
                            const int Iv = idx32(u, unpack(wbits(S.scr[nn][tid]), q), rlo[q], rhi[q], err);
                            const int a1 = unpack(pa, q), a2 = unpack(pb, q);
                            nv[q] = min(max(Iv, min(a1, a2)), max(a1, a2));
                        }
                        if (dir == 0) nv[0] = cut - 1;
                        else if (dir == 1) nv[1] = cut - 1;
                        else nv[2] = cut - 1;
                        pk = pack3(nv[0], nv[1], nv[2]);
                    }
                    S.scr[4 + nn][tid] = make_float4(x, y, z, __int_as_float((int)pk));
                }
                const int nt = C.ntets;
                if (mode == 1) {
                    /* the node's pieces summed here, then added to its face's sums once */
                    int fl = 0;
                    FF nv{0.f, 0.f}, nl{0.f, 0.f};
#pragma unroll 1 /* rolled, as the loops below: less code (the kernel is instruction-fetch bound) */
                    for (int c = 0; c < nt; ++c) {
                        const float4 P0 = S.scr[C.vtet[c][0]][tid], P1 = S.scr[C.vtet[c][1]][tid];
                        const float4 P2 = S.scr[C.vtet[c][2]][tid], P3 = S.scr[C.vtet[c][3]][tid];
                        const float tv = tet_vol<float>(P0.x, P0.y, P0.z, P1.x, P1.y, P1.z, P2.x, P2.y, P2.z, P3.x,
                                                        P3.y, P3.z);
                        ff_add(nv, tv);
                        if (C.side[c] == 0) { ff_add(nl, tv); fl |= PIECE_LIQ; }
                        else fl |= PIECE_GAS;
                    }
                    facc_add(avol, b, nv);
                    facc_add(acc, b, nl);
                    fflag_or(flg, b, fl);
                } else {
                    const int pos = size + ipush - pushed;
                    const unsigned tagc = ((unsigned)b | ((unsigned)flags << 3)) << 24;
                    const int sh = 8 * dir;
#pragma unroll 1
                    for (int c = 0; c < nt; ++c) {
                        const bool up = C.side[c] == 1;
#pragma unroll
                        for (int nn = 0; nn < 4; ++nn) {
                            float4 qv = S.scr[C.vtet[c][nn]][tid];
                            unsigned pk = wbits(qv);
                            if (up) pk = (pk & ~(255u << sh)) | ((unsigned)(cut + 128) << sh);
                            if (nn == 0) pk |= tagc;
                            qv.w = __int_as_float((int)pk);
                            S.stk[w][nn][pos + c] = qv;
                        }
                    }
                }
            } else if (priv) {
                FF rv, rl;
                float cx[4], cy[4], cz[4];
#pragma unroll
                for (int nn = 0; nn < 4; ++nn) { cx[nn] = v[nn].x; cy[nn] = v[nn].y; cz[nn] = v[nn].z; }
                clip32(m, S.tab, PL, nullptr, i0, j0, k0, rlo, rhi, cx, cy, cz, cind, rv, rl, err);
                facc_add(avol, b, rv);
                facc_add(acc, b, rl);
                fflag_or(flg, b, PIECE_LIQ | PIECE_GAS);
            }
            if (back) {
                const int p = size + tot_push + __popc(backmask & lanemask_lt);
#pragma unroll
                for (int q = 0; q < 4; ++q) S.stk[w][q][p] = v[q];
            }
            size += tot_push + __popc(backmask);
            __syncwarp();
        }
        /* per face: fixed-order float-float shuffle tree (no FP64 on the warp), then on the
         * face's lane the liquid rescaled to the FP64 volume */
#pragma unroll
        for (int b = 0; b < FCLIP_BATCH; ++b) {
            if (b >= nb) break;
            FF a = acc[b], vv = avol[b];
            int fg = flg[b];
#pragma unroll 1
            for (int off = 16; off > 0; off >>= 1) {
                const FF oa{__shfl_xor_sync(0xffffffffu, a.hi, off), __shfl_xor_sync(0xffffffffu, a.lo, off)};
                const FF ov{__shfl_xor_sync(0xffffffffu, vv.hi, off), __shfl_xor_sync(0xffffffffu, vv.lo, off)};
                ff_add(a, oa);
                ff_add(vv, ov);
                fg |= __shfl_xor_sync(0xffffffffu, fg, off);
            }
            if (lane == b) {
                const double fl = (double)a.hi + (double)a.lo, u = (double)vv.hi + (double)vv.lo;
                double2* out = F.fvf[fd_] + (code_ >> 2);
                const double V = out->x;
                double wgt;
                if (!(fg & PIECE_GAS)) wgt = 1.0;
                else if (!(fg & PIECE_LIQ)) wgt = 0.0;
                else wgt = u != 0.0 ? fmin(1.0, fmax(0.0, fl / u)) : 0.5;
                out->y = fl + (V - u) * wgt;
            }
        }
        __syncwarp();
    }
    if (err) atomicOr(errw, err);
}

/* VFnew = (L + sum +-F) / (1 + sum +-V) over the cell's six faces, in cell units; L is the
 * cell's own liquid, VF (0 below VFlo, 1 above VFhi).  A cell whose eight traced corners lie
 * strictly on one side of every donor plane of their index box has a pre-image entirely in
 * liquid (or gas): VFnew is 1 (or 0) exactly, as the reference's vLiq/vol of equal sums gives,
 * instead of the faces' rounded sum.
 *
 * The faces' FP32 liquid carries rounding of order 1e-7 of a face's flux, which cancels
 * between the two cells of a face but not within one cell: a cell whose pre-image holds no
 * liquid (or only liquid), where the reference gives exactly 0 (or 1), would come out at
 * +-1e-7 and turn into an interface cell of its own.  Cells whose flux-form value lies within
 * NEAR_PURE of 0 or 1 are therefore listed, with their pre-image vertices (the same traced
 * nodes), for the cell-form clip (k_sl32_clipw), whose liquid and volume are sums over the same
 * pieces: exactly 0 or 1 when every piece is gas or liquid, and otherwise a liquid volume with
 * rounding proportional to itself. */
constexpr double NEAR_PURE = 1e-6;

__global__ void __launch_bounds__(FLUX_THREADS) k_flux_cells(DevMesh m, const double* __restrict__ VFin,
                                                             double* __restrict__ VFout, Plane32 PL,
                                                             const int* __restrict__ list,
                                                             const int* __restrict__ count, FluxBufs F,
                                                             int* slow_cells, float4* slow_verts, int* slow_count,
                                                             int* errw)
{
    const int n = *count;
    int err = 0;
    for (int t = blockIdx.x * FLUX_THREADS + threadIdx.x; t < n; t += gridDim.x * FLUX_THREADS) {
        int i, j, k;
        cell_of(m, list[t], i, j, k);
        const long v = vidx(m, i, j, k);
        const double vf = VFin[v];
        double vol = 1.0, liq = vf < m.VFlo ? 0.0 : (vf > m.VFhi ? 1.0 : vf);
        const long c = cidx(m, i, j, k);
        const long st[3] = {1, m.cs1, m.cs2};
#pragma unroll
        for (int dir = 0; dir < 3; ++dir) {
            const double2 lo = F.fvf[dir][c], hi = F.fvf[dir][c + st[dir]];
            vol -= lo.x;
            liq -= lo.y;
            vol += hi.x;
            liq += hi.y;
        }
        if (!(vol > 0.0) || !isfinite(vol)) err |= ERR_VOLUME;
        double r = liq / vol;
        int rlo[3], rhi[3];
        rel_bounds(m, i, j, k, rlo, rhi);
        /* with correction tets (pressure_scheme "finite-difference") the pre-image also reaches
         * the six faces' apexes (stored in each face's low cell's frame) */
        if (m.fast_pure && vol > 0.25 && vol < 4.0) {
            float px[14], py[14], pz[14];
            int lo[3] = {1 << 20, 1 << 20, 1 << 20}, hi[3] = {-(1 << 20), -(1 << 20), -(1 << 20)};
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int a = q & 1, b = (q >> 1) & 1, e = q >> 2;
                const long nc = c + a + b * m.cs1 + e * m.cs2;
                px[q] = (float)((double)a + F.nd[0][nc]);
                py[q] = (float)((double)b + F.nd[1][nc]);
                pz[q] = (float)((double)e + F.nd[2][nc]);
                const int I[3] = {idx32(px[q], 0, rlo[0], rhi[0], err), idx32(py[q], 0, rlo[1], rhi[1], err),
                                  idx32(pz[q], 0, rlo[2], rhi[2], err)};
                for (int d = 0; d < 3; ++d) { lo[d] = min(lo[d], I[d]); hi[d] = max(hi[d], I[d]); }
            }
            int side;
            if (m.fd) {
#pragma unroll
                for (int f = 0; f < 6; ++f) {
                    const int dir = f >> 1, up = f & 1;
                    const float4 e = F.fapex[dir][c + (up ? st[dir] : 0)];
                    /* a low face's apex is in the lower neighbour's frame: one cell back */
                    px[8 + f] = e.x - (!up && dir == 0 ? 1.f : 0.f);
                    py[8 + f] = e.y - (!up && dir == 1 ? 1.f : 0.f);
                    pz[8 + f] = e.z - (!up && dir == 2 ? 1.f : 0.f);
                    const int I[3] = {idx32(px[8 + f], 0, rlo[0], rhi[0], err), idx32(py[8 + f], 0, rlo[1], rhi[1], err),
                                      idx32(pz[8 + f], 0, rlo[2], rhi[2], err)};
                    for (int d = 0; d < 3; ++d) { lo[d] = min(lo[d], I[d]); hi[d] = max(hi[d], I[d]); }
                }
                side = box_plane_side<14>(m, PL, i, j, k, lo[0], hi[0], lo[1], hi[1], lo[2], hi[2], px, py, pz);
            } else {
                side = box_plane_side<8>(m, PL, i, j, k, lo[0], hi[0], lo[1], hi[1], lo[2], hi[2], px, py, pz);
            }
            if (side != 0) r = side > 0 ? 1.0 : 0.0;
        }
        VFout[v] = r;
        const bool near = r != 0.0 && r != 1.0 && (fabs(r) < NEAR_PURE || fabs(1.0 - r) < NEAR_PURE);
        const int slot = warp_slot(near, slow_count);
        if (slot >= 0) {
            /* the cell's pre-image vertices in cell2verts! order (x mirrored on odd cells under
             * 5_tets), as k_sl32_pre stores them, from the traced nodes; under pressure_scheme
             * "finite-difference" then its six faces' correction apexes (x-, x+, y-, ... in
             * the cell's frame) */
            const bool even = tess_even(m.tess, i, j, k);
            const int stride = (m.tess == 24 || m.fd) ? 16 : 8;
            float px[8], py[8], pz[8];
            for (int q = 0; q < 8; ++q) {
                const int a = even ? (q & 1) : 1 - (q & 1), b = (q >> 1) & 1, e = q >> 2;
                const long nc = c + a + b * m.cs1 + e * m.cs2;
                px[q] = (float)((double)a + F.nd[0][nc]);
                py[q] = (float)((double)b + F.nd[1][nc]);
                pz[q] = (float)((double)e + F.nd[2][nc]);
                const unsigned pk = pack3(idx32(px[q], 0, rlo[0], rhi[0], err), idx32(py[q], 0, rlo[1], rhi[1], err),
                                          idx32(pz[q], 0, rlo[2], rhi[2], err));
                slow_verts[(long)slot * stride + q] = make_float4(px[q], py[q], pz[q], __int_as_float((int)pk));
            }
            if (m.fd) {
                for (int f = 0; f < 6; ++f) {
                    const int dir = f >> 1, up = f & 1;
                    const float4 e = F.fapex[dir][c + (up ? st[dir] : 0)];
                    const float x = e.x - (!up && dir == 0 ? 1.f : 0.f);
                    const float y = e.y - (!up && dir == 1 ? 1.f : 0.f);
                    const float z = e.z - (!up && dir == 2 ? 1.f : 0.f);
                    const unsigned pk = pack3(idx32(x, 0, rlo[0], rhi[0], err), idx32(y, 0, rlo[1], rhi[1], err),
                                              idx32(z, 0, rlo[2], rhi[2], err));
                    slow_verts[(long)slot * 16 + 8 + f] = make_float4(x, y, z, __int_as_float((int)pk));
                }
            }
            if (m.tess == 24) {
                for (int f = -1; f < 6; ++f) {
                    const int nv = f < 0 ? 8 : 4;
                    float x = 0.f, y = 0.f, z = 0.f;
                    for (int q = 0; q < nv; ++q) {
                        const int w = f < 0 ? q : face24(f, q);
                        x = q == 0 ? px[w] : x + px[w];
                        y = q == 0 ? py[w] : y + py[w];
                        z = q == 0 ? pz[w] : z + pz[w];
                    }
                    x /= (float)nv; y /= (float)nv; z /= (float)nv;
                    const unsigned pk = pack3(idx32(x, 0, rlo[0], rhi[0], err), idx32(y, 0, rlo[1], rhi[1], err),
                                              idx32(z, 0, rlo[2], rhi[2], err));
                    slow_verts[(long)slot * 16 + 9 + f] = make_float4(x, y, z, __int_as_float((int)pk));
                }
            }
            slow_cells[slot] = list[t];
        }
    }
    if (err) atomicOr(errw, err);
}

/* ---- launchers ------------------------------------------------------------------------ */
void launch_sl32_pre(const DevMesh& m, double dt, double* VFout, const float* uf, const float* vf, const float* wf,
                     const float4* planes, const signed char* phase, const int* list, const int* count, int* work,
                     int* slow_cells, float4* slow_verts, int* slow_count, int* errw, int nsm, cudaStream_t s)
{
    Vel32 V{uf, vf, wf};
    Plane32 PL{planes};
    k_sl32_pre<<<nsm * 8, SL32_THREADS, 0, s>>>(m, (float)dt, VFout, V, PL, phase, list, count, work, slow_cells,
                                                slow_verts, slow_count, errw);
}

void launch_sl32_clip(const DevMesh& m, double* VFout, const float4* planes, int* work2, const int* slow_cells,
                      const float4* slow_verts, const int* slow_count, int* errw, int nsm, cudaStream_t s)
{
    Plane32 PL{planes};
    /* 55.2 KB of dynamic shared memory per block: above the 48 KB default, four blocks per SM */
    const int smem = (int)sizeof(ClipShared);
    cudaFuncSetAttribute(k_sl32_clipw, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k_sl32_clipw<<<nsm * 4, CLIPW_WARPS * 32, smem, s>>>(m, VFout, PL, slow_cells, slow_verts, slow_count, work2,
                                                          errw);
}

void launch_sl32_flux(const DevMesh& m, double dt, const double* VFin, double* VFout, const float* uf32,
                      const float* vf32, const float* wf32, const double* uf, const double* vf, const double* wf,
                      const float4* planes, const short* band, const int* list, const int* count,
                      const FluxLaunch& L, int* slow_cells, float4* slow_verts, int* slow_count, int* work2,
                      int* errw, int nsm, cudaStream_t s)
{
    FluxBufs F{{L.nd[0], L.nd[1], L.nd[2]}, {L.fvf[0], L.fvf[1], L.fvf[2]}, L.nodes, L.faces, L.clip,
               {L.fapex[0], L.fapex[1], L.fapex[2]}, L.ctr, L.ctr + 1, L.ctr + 2, L.ctr + 3};
    const Vel64c V64{uf, vf, wf, {1.0 / m.d[0], 1.0 / m.d[1], 1.0 / m.d[2]}};
    Plane32 PL{planes};
    cudaMemsetAsync(L.ctr, 0, 4 * sizeof(int), s);
    k_flux_lists<<<nsm * 8, FLUX_THREADS, 0, s>>>(m, band, list, count, F);
    k_flux_nodes<<<nsm * 8, FLUX_THREADS, 0, s>>>(m, dt, V64, Vel32{uf32, vf32, wf32}, F);
    k_flux_faces<<<nsm * 8, FLUX_THREADS, 0, s>>>(m, PL, F, dt, V64, errw);
    const int smem = (int)sizeof(FluxShared);
    auto clip = m.tess == 24 ? k_flux_clip<SEED_24> : (m.fd ? k_flux_clip<SEED_FD> : k_flux_clip<SEED_PRISM>);
    cudaFuncSetAttribute(clip, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    clip<<<nsm * 4, CLIPW_WARPS * 32, smem, s>>>(m, PL, F, errw);
    k_flux_cells<<<nsm * 8, FLUX_THREADS, 0, s>>>(m, VFin, VFout, PL, list, count, F, slow_cells, slow_verts,
                                                   slow_count, errw);
    /* near-pure cells: the cell form's FP32 clip (with the correction tets under
     * pressure_scheme "finite-difference") */
    launch_sl32_clip(m, VFout, planes, work2, slow_cells, slow_verts, slow_count, errw, nsm, s);
}

} // namespace slvof
