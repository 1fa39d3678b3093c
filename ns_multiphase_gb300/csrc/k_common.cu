/*
 * k_common.cu — kernels shared by the FP64 and mixed paths (exact integer/copy work and the
 * pure-cell part of ELVIRA).  Built with -fmad=false.
 */
#include "slvof_kernels.h"
#include "slvof_dev.cuh"
#include "tma.cuh"

namespace slvof {

__device__ __forceinline__ bool interior(const DevMesh& m, int i, int j, int k)
{
    return i >= 1 && i <= m.N[0] && j >= 1 && j <= m.N[1] && k >= 1 && k <= m.N[2];
}

/* Neumann!(VF) + update_VF_borders!(VF) after the interior was overwritten
 * (src/Transport.jl:179-181): ghost p takes the pre-fill value at its source cell, which is
 * the new interior value or an old ghost value.  update_VF_borders! moves nghost layers, not
 * six (src/Parallel.jl:71-83 compares nghost == VFghost without assigning), so the three
 * extra layers keep their values. */
__global__ void k_vf_ghost(DevMesh m, const double* __restrict__ VFin, double* __restrict__ VFout)
{
    const long n0 = m.N[0] + 2 * m.g + 6, n1 = m.N[1] + 2 * m.g + 6, n2 = m.N[2] + 2 * m.g + 6;
    const long total = n0 * n1 * n2;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t % n0) + m.vlo, j = (int)((t / n0) % n1) + m.vlo, k = (int)(t / (n0 * n1)) + m.vlo;
        if (interior(m, i, j, k)) continue;
        const int si = ghost_src_1d(i, m.N[0], m.g, m.per[0], true);
        const int sj = ghost_src_1d(j, m.N[1], m.g, m.per[1], true);
        const int sk = ghost_src_1d(k, m.N[2], m.g, m.per[2], true);
        const long s = vidx(m, si, sj, sk);
        VFout[t] = interior(m, si, sj, sk) ? VFout[s] : VFin[s];
    }
}

constexpr int PURE_BX = 32, PURE_BY = 8; /* pure-cell tile: 32 i x 8 j of one k plane */

/* ELVIRA! for pure cells (src/ELVIRA.jl:19-46): the axis normal from the first face
 * neighbour of the opposite phase (x-, x+, y-, y+, z-, z+), zero otherwise; interface cells
 * go to the candidate list.  The interior VF is also summed for the mass, exactly: each value
 * in 62-bit fixed point, 128-bit integer sums, one partial per block.  A thread per cell,
 * (i, j) from the block's tile and k from the grid, and threshold tests on the bit patterns,
 * so the pass runs on the integer pipes. */
__global__ void __launch_bounds__(PURE_BX * PURE_BY) k_elvira_pure(DevMesh m, const double* __restrict__ VF,
                                                                   double* __restrict__ nx, double* __restrict__ ny,
                                                                   double* __restrict__ nz, int* list, int* count,
                                                                   long long* partials)
{
    const int i = 1 + blockIdx.x * PURE_BX + threadIdx.x, j = 1 + blockIdx.y * PURE_BY + threadIdx.y;
    const int k = 1 + blockIdx.z;
    const long long lo = dbits(m.VFlo), hi = dbits(m.VFhi);
    const long sj = m.vs1, sk = m.vs2;
    __int128 acc = 0;
    bool iface = false;
    int L = 0;
    if (i <= m.N[0] && j <= m.N[1]) {
        L = (i - 1) + (j - 1) * m.N[0] + (k - 1) * m.N[0] * m.N[1];
        const long v = vidx(m, i, j, k);
        const double c = VF[v];
        const long long cb = dbits(c);
        acc = fx62(c);
        /* the six face neighbours are loaded together (one latency, not six in a chain) and
         * tested in the reference's order */
        const long long xm = dbits(VF[v - 1]), xp = dbits(VF[v + 1]);
        const long long ym = dbits(VF[v - sj]), yp = dbits(VF[v + sj]);
        const long long zm = dbits(VF[v - sk]), zp = dbits(VF[v + sk]);
        double ax = 0.0, ay = 0.0, az = 0.0;
        if (bits_below(cb, lo)) {
            if (bits_above(xm, hi)) ax = 1.0;
            else if (bits_above(xp, hi)) ax = -1.0;
            else if (bits_above(ym, hi)) ay = 1.0;
            else if (bits_above(yp, hi)) ay = -1.0;
            else if (bits_above(zm, hi)) az = 1.0;
            else if (bits_above(zp, hi)) az = -1.0;
        } else if (bits_above(cb, hi)) {
            if (bits_below(xm, lo)) ax = -1.0;
            else if (bits_below(xp, lo)) ax = 1.0;
            else if (bits_below(ym, lo)) ay = -1.0;
            else if (bits_below(yp, lo)) ay = 1.0;
            else if (bits_below(zm, lo)) az = -1.0;
            else if (bits_below(zp, lo)) az = 1.0;
        } else {
            iface = true; /* VFlo <= VF <= VFhi (or NaN, as the reference's compares) */
        }
        if (nx) {
            const long o = cidx(m, i, j, k);
            nx[o] = ax; ny[o] = ay; nz[o] = az;
        }
    }
    if (list) {
        __shared__ int s_app[PURE_BX * PURE_BY / 32 + 1];
        const bool f[1] = {iface};
        const int it[1] = {L};
        block_append<1, PURE_BX * PURE_BY / 32>(f, it, list, count, s_app);
    }
    /* block sum: exact, so its order does not matter */
    for (int off = 16; off > 0; off >>= 1) acc += i128_shfl_down(acc, off);
    __shared__ long long sh_hi[PURE_BX * PURE_BY / 32];
    __shared__ unsigned long long sh_lo[PURE_BX * PURE_BY / 32];
    const int t = threadIdx.y * PURE_BX + threadIdx.x, w = t >> 5;
    if ((t & 31) == 0) { sh_hi[w] = (long long)(acc >> 64); sh_lo[w] = (unsigned long long)acc; }
    __syncthreads();
    if (t == 0) {
        __int128 b = 0;
        for (int q = 0; q < PURE_BX * PURE_BY / 32; ++q) b += i128_from(sh_hi[q], sh_lo[q]);
        const long blk = blockIdx.x + (long)gridDim.x * (blockIdx.y + (long)gridDim.y * blockIdx.z);
        partials[2 * blk] = (long long)(b >> 64);
        partials[2 * blk + 1] = (long long)(unsigned long long)b;
    }
}

/* Sum of the exact partials, scaled: mass = sum(VF) * dx*dy*dz (src/WriteData.jl:33).  One
 * block of MASS_THREADS; integer sums, so the order is free. */
constexpr int MASS_THREADS = 1024;
__global__ void __launch_bounds__(MASS_THREADS) k_mass_final(const long long* __restrict__ partials, long nblocks,
                                                             double cellvol, double* out)
{
    __int128 a = 0;
    for (long b = threadIdx.x; b < nblocks; b += MASS_THREADS)
        a += i128_from(partials[2 * b], (unsigned long long)partials[2 * b + 1]);
    for (int off = 16; off > 0; off >>= 1) a += i128_shfl_down(a, off);
    __shared__ long long sh_hi[MASS_THREADS / 32];
    __shared__ unsigned long long sh_lo[MASS_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sh_hi[w] = (long long)(a >> 64); sh_lo[w] = (unsigned long long)a; }
    __syncthreads();
    if (w == 0) {
        a = i128_from(sh_hi[lane], sh_lo[lane]);
        for (int off = 16; off > 0; off >>= 1) a += i128_shfl_down(a, off);
        if (lane == 0) out[0] = ldexp(i128_to_double(a), -62) * cellvol;
    }
}

/* update_borders!(nx/ny/nz) after ELVIRA! zeroed the whole arrays (src/ELVIRA.jl:11-13,50-52):
 * periodic ghosts copy the interior, all other ghosts stay zero. */
__global__ void k_normal_ghost(DevMesh m, double* nx, double* ny, double* nz)
{
    const long n0 = m.N[0] + 2 * m.g, n1 = m.N[1] + 2 * m.g, n2 = m.N[2] + 2 * m.g;
    const long total = n0 * n1 * n2;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t % n0) + m.lo, j = (int)((t / n0) % n1) + m.lo, k = (int)(t / (n0 * n1)) + m.lo;
        if (interior(m, i, j, k)) continue;
        const int si = ghost_src_1d(i, m.N[0], m.g, m.per[0], false);
        const int sj = ghost_src_1d(j, m.N[1], m.g, m.per[1], false);
        const int sk = ghost_src_1d(k, m.N[2], m.g, m.per[2], false);
        double a = 0.0, b = 0.0, c = 0.0;
        if (interior(m, si, sj, sk)) {
            const long s = cidx(m, si, sj, sk);
            a = nx[s]; b = ny[s]; c = nz[s];
        }
        nx[t] = a; ny[t] = b; nz[t] = c;
    }
}

/* computeBand! (src/VF.jl:16-74).  The first pass marks pure cells touching the opposite
 * pure phase (Julia's combined for-loop break leaves all three loops: band 0 if any of the
 * 27 cells qualifies). */
/* Band kernels as a 3D stencil: a block owns a BX x BY tile of an x-y plane and marches up a
 * chunk of BZ planes.  Each plane of the tile plus a one-cell halo is classified once into
 * bits (bit 0: VF >= VFhi, bit 1: VF <= VFlo for the first pass; bit 0: |band| == n-1 for a
 * sweep), OR-ed over its 3x3 x-y neighbourhood in shared memory, and kept for three planes;
 * a cell's 3x3x3 test is then the OR of the three dilated planes.  Every cell value is read
 * once per plane (plus the halo), coalesced along x. */
constexpr int BX = 32, BY = 8, BZ = 16;

/* bits of one (tile + halo) plane k into shared memory, then its x-y dilation */
template <class Classify>
__device__ __forceinline__ void band_plane(int i0, int j0, int k, unsigned char (*raw)[BX + 2],
                                          unsigned char (*dil)[BX], Classify cls)
{
    for (int t = threadIdx.y * BX + threadIdx.x; t < (BX + 2) * (BY + 2); t += BX * BY) {
        const int a = t % (BX + 2), b = t / (BX + 2);
        raw[b][a] = cls(i0 - 1 + a, j0 - 1 + b, k);
    }
    __syncthreads();
    const int x = threadIdx.x + 1, y = threadIdx.y + 1;
    unsigned char d = 0;
#pragma unroll
    for (int b = -1; b <= 1; ++b)
#pragma unroll
        for (int a = -1; a <= 1; ++a) d |= raw[y + b][x + a];
    dil[threadIdx.y][threadIdx.x] = d;
}

template <class Classify, class Finish>
__device__ __forceinline__ void band_march(const DevMesh& m, Classify cls, Finish fin)
{
    __shared__ unsigned char raw[BY + 2][BX + 2];
    __shared__ unsigned char dil[3][BY][BX];
    const int i0 = 1 + blockIdx.x * BX, j0 = 1 + blockIdx.y * BY;
    const int kbeg = 1 + blockIdx.z * BZ, kend = min(kbeg + BZ - 1, m.N[2]);
    const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
    /* planes kbeg-1 and kbeg */
    band_plane(i0, j0, kbeg - 1, raw, dil[0], cls);
    __syncthreads();
    band_plane(i0, j0, kbeg, raw, dil[1], cls);
    __syncthreads();
    for (int k = kbeg; k <= kend; ++k) {
        const int s0 = (k - kbeg) % 3, s1 = (k - kbeg + 1) % 3, s2 = (k - kbeg + 2) % 3;
        band_plane(i0, j0, k + 1, raw, dil[s2], cls);
        __syncthreads();
        const unsigned char any = dil[s0][threadIdx.y][threadIdx.x] | dil[s1][threadIdx.y][threadIdx.x] |
                                  dil[s2][threadIdx.y][threadIdx.x];
        if (i <= m.N[0] && j <= m.N[1]) fin(i, j, k, any);
        __syncthreads();
    }
}

/* computeBand! first pass (src/VF.jl:16-45): pure cells next to the opposite phase (3x3x3
 * block, the cell itself included) get 0, other pure cells +-(nband+1), interface cells 0. */
__global__ void __launch_bounds__(BX * BY) k_band_first(DevMesh m, const double* __restrict__ VF,
                                                       short* __restrict__ bout)
{
    const short nb1 = (short)(m.nband + 1);
    const long long lob = dbits(m.VFlo), hib = dbits(m.VFhi);
    auto cls = [&](int a, int b, int c) -> unsigned char {
        /* the halo reaches index 0 and N+1 (ghost cells); beyond the tile's cells of a partial
         * tile it stays inside the ghost layers (g >= 3) */
        const int aa = min(a, m.N[0] + 1), bb = min(b, m.N[1] + 1);
        const long long v = dbits(__ldg(VF + vidx(m, aa, bb, c)));
        return (unsigned char)((!bits_below(v, hib) ? 1 : 0) | (!bits_above(v, lob) ? 2 : 0));
    };
    auto fin = [&](int i, int j, int k, unsigned char any) {
        const long long c = dbits(__ldg(VF + vidx(m, i, j, k)));
        short b = 0;
        if (bits_below(c, lob)) b = (any & 1) ? (short)0 : (short)-nb1;
        else if (bits_above(c, hib)) b = (any & 2) ? (short)0 : nb1;
        bout[cidx(m, i, j, k)] = b;
    };
    band_march(m, cls, fin);
}

/* The first pass with each (tile + halo) plane of VF brought into shared memory by the TMA
 * unit: a ring of TB_STAGES planes, the load of plane p + TB_STAGES issued as soon as plane p
 * is classified, so the loads run ahead of the march instead of every thread issuing its
 * own.  The tile's first halo element sits at an odd VF element on grids with g = 3 (VF
 * starts 3 + g cells before cell 1) and a bulk tensor copy must start on a 16-byte boundary,
 * so the box starts one element lower where needed and is TB_W = BX + 4 elements wide.  A
 * wait that runs out sets ERR_WAIT and the block stops (after waiting, bounded again, for its
 * copies in flight). */
constexpr int TB_STAGES = 4;
constexpr int TB_W = BX + 4, TB_H = BY + 2;
constexpr int TB_BYTES = TB_W * TB_H * (int)sizeof(double);
constexpr int TB_STRIDE = (TB_BYTES + 127) / 128 * 128;

__global__ void __launch_bounds__(BX * BY) k_band_first_tma(DevMesh m, const __grid_constant__ CUtensorMap map,
                                                           short* __restrict__ bout, int* errw)
{
    __shared__ __align__(128) unsigned char stage[TB_STAGES * TB_STRIDE];
    __shared__ __align__(8) unsigned long long bar[TB_STAGES];
    __shared__ unsigned char raw[BY + 2][BX + 2];
    __shared__ unsigned char dil[3][BY][BX];
    __shared__ int stop;
    const short nb1 = (short)(m.nband + 1);
    const long long lob = dbits(m.VFlo), hib = dbits(m.VFhi);
    const int tid = threadIdx.y * BX + threadIdx.x;
    const int i0 = 1 + blockIdx.x * BX, j0 = 1 + blockIdx.y * BY;
    const int kbeg = 1 + blockIdx.z * BZ, kend = min(kbeg + BZ - 1, m.N[2]);
    const int nplanes = kend - kbeg + 3; /* planes kbeg-1 .. kend+1 */
    const int x0 = i0 - 1 - m.vlo, xa = x0 & ~1, xoff = x0 - xa;
    const int y0 = j0 - 1 - m.vlo, z0 = kbeg - 1 - m.vlo;
    if (tid == 0) {
        for (int r = 0; r < TB_STAGES; ++r) tma::bar_init(&bar[r], 1);
        tma::fence_bar_init();
        stop = 0;
        for (int p = 0; p < min(TB_STAGES, nplanes); ++p) {
            tma::bar_arrive_expect(&bar[p], TB_BYTES);
            tma::load_3d(stage + p * TB_STRIDE, &map, xa, y0, z0 + p, &bar[p]);
        }
    }
    __syncthreads();
    const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
    long long cprev = 0;
    int p = 0;
    for (; p < nplanes; ++p) {
        const int r = p % TB_STAGES;
        if (!tma::bar_wait(&bar[r], (unsigned)(p / TB_STAGES) & 1u)) stop = 1;
        __syncthreads();
        if (stop) break;
        const double* V = reinterpret_cast<const double*>(stage + r * TB_STRIDE);
        for (int t = tid; t < (BX + 2) * (BY + 2); t += BX * BY) {
            const int a = t % (BX + 2), b = t / (BX + 2);
            const long long v = dbits(V[b * TB_W + a + xoff]);
            raw[b][a] = (unsigned char)((!bits_below(v, hib) ? 1 : 0) | (!bits_above(v, lob) ? 2 : 0));
        }
        const long long ccur = dbits(V[(threadIdx.y + 1) * TB_W + threadIdx.x + 1 + xoff]);
        __syncthreads(); /* raw complete; every thread is done with stage r */
        if (tid == 0 && p + TB_STAGES < nplanes) {
            tma::fence_proxy_async();
            tma::bar_arrive_expect(&bar[r], TB_BYTES);
            tma::load_3d(stage + r * TB_STRIDE, &map, xa, y0, z0 + p + TB_STAGES, &bar[r]);
        }
        unsigned char d = 0;
#pragma unroll
        for (int b = 0; b <= 2; ++b)
#pragma unroll
            for (int a = 0; a <= 2; ++a) d |= raw[threadIdx.y + b][threadIdx.x + a];
        dil[p % 3][threadIdx.y][threadIdx.x] = d;
        __syncthreads();
        if (p >= 2 && i <= m.N[0] && j <= m.N[1]) {
            /* cell (i, j, k) of plane p - 1, its 3x3x3 block in the three dilated planes */
            const int k = kbeg - 2 + p;
            const unsigned char any = dil[0][threadIdx.y][threadIdx.x] | dil[1][threadIdx.y][threadIdx.x] |
                                      dil[2][threadIdx.y][threadIdx.x];
            short bv = 0;
            if (bits_below(cprev, lob)) bv = (any & 1) ? (short)0 : (short)-nb1;
            else if (bits_above(cprev, hib)) bv = (any & 2) ? (short)0 : nb1;
            bout[cidx(m, i, j, k)] = bv;
        }
        cprev = ccur;
    }
    if (stop && tid == 0) {
        atomicOr(errw, ERR_WAIT);
        for (int q = p; q < min(p + TB_STAGES, nplanes); ++q) tma::bar_wait(&bar[q % TB_STAGES], (unsigned)(q / TB_STAGES) & 1u);
    }
}

/* Neumann!(band) + update_borders!(band) (neumann=true) or update_borders!(band) alone. */
__global__ void k_band_ghost(DevMesh m, const short* __restrict__ bin, short* __restrict__ bout, bool neumann)
{
    const long n0 = m.N[0] + 2 * m.g, n1 = m.N[1] + 2 * m.g, n2 = m.N[2] + 2 * m.g;
    const long total = n0 * n1 * n2;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t % n0) + m.lo, j = (int)((t / n0) % n1) + m.lo, k = (int)(t / (n0 * n1)) + m.lo;
        if (interior(m, i, j, k)) continue;
        const int si = ghost_src_1d(i, m.N[0], m.g, m.per[0], neumann);
        const int sj = ghost_src_1d(j, m.N[1], m.g, m.per[1], neumann);
        const int sk = ghost_src_1d(k, m.N[2], m.g, m.per[2], neumann);
        const long s = cidx(m, si, sj, sk);
        bout[t] = interior(m, si, sj, sk) ? bout[s] : bin[s];
    }
}

/* One band sweep: |band| > n next to |band| == n-1 becomes n*sign(band).  The result does
 * not depend on the update order, so the sweep reads one buffer and writes the other. */
__global__ void __launch_bounds__(BX * BY) k_band_sweep(DevMesh m, const short* __restrict__ bin,
                                                       short* __restrict__ bout, int n)
{
    auto cls = [&](int a, int b, int c) -> unsigned char {
        const int aa = min(a, m.N[0] + 1), bb = min(b, m.N[1] + 1);
        return (unsigned char)(abs((int)bin[cidx(m, aa, bb, c)]) == n - 1 ? 1 : 0);
    };
    auto fin = [&](int i, int j, int k, unsigned char any) {
        const long o = cidx(m, i, j, k);
        short b = bin[o];
        if (abs((int)b) > n && (any & 1)) b = (short)(b > 0 ? n : -n);
        bout[o] = b;
    };
    band_march(m, cls, fin);
}

/* transport! band gate (src/Transport.jl:111,153): band cells go to the SL list, the rest
 * keep VF.  Thread per (i, j) column of CLS_K cells in k on the pure-cell tiles, so no index
 * divides: a warp reads rows of 32 band entries and copies rows of VF.  Every band entry and
 * VF value of the column is loaded before any is used (the VF of band cells too, which are
 * about a tenth), so the loads of a thread overlap instead of waiting on each other; the band
 * cells of a block join the list with one atomic. */
constexpr int CLS_K = 4;

__global__ void __launch_bounds__(PURE_BX * PURE_BY) k_sl_classify(DevMesh m, const short* __restrict__ band,
                                                                   const double* __restrict__ VFin,
                                                                   double* __restrict__ VFout, int* list,
                                                                   int* count)
{
    const int i = 1 + blockIdx.x * PURE_BX + threadIdx.x, j = 1 + blockIdx.y * PURE_BY + threadIdx.y;
    const int k0 = 1 + blockIdx.z * CLS_K;
    const bool col = i <= m.N[0] && j <= m.N[1];
    short b[CLS_K];
    double v[CLS_K];
#pragma unroll
    for (int q = 0; q < CLS_K; ++q) {
        const bool in = col && k0 + q <= m.N[2];
        b[q] = in ? __ldg(band + cidx(m, i, j, k0 + q)) : (short)0;
        v[q] = in ? __ldg(VFin + vidx(m, i, j, k0 + q)) : 0.0;
    }
    bool sl[CLS_K];
    int item[CLS_K];
#pragma unroll
    for (int q = 0; q < CLS_K; ++q) {
        const int k = k0 + q;
        const bool in = col && k <= m.N[2];
        sl[q] = in && abs((int)b[q]) <= m.nband;
        item[q] = (i - 1) + (j - 1) * m.N[0] + (k - 1) * m.N[0] * m.N[1];
        if (in && !sl[q]) VFout[vidx(m, i, j, k)] = v[q];
    }
    __shared__ int s_app[PURE_BX * PURE_BY / 32 * CLS_K + 1];
    block_append<CLS_K, PURE_BX * PURE_BY / 32>(sl, item, list, count, s_app);
}

/* FP64 array to FP32 times a scale (face velocities to cells per unit time): the conversion
 * first and the scale in FP32, so that only the conversion issues on GB300's narrow FP64 pipe
 * (with the double multiply as well the kernel was FP64-bound at 2.7 TB/s).  For a power-of-two
 * scale, 1/dx on a 2^k grid of a unit box, the result equals the rounded double product. */
__global__ void k_to_float(const double* __restrict__ a, float* __restrict__ b, long n, double scale)
{
    const float s = (float)scale;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
        b[t] = __double2float_rn(a[t]) * s;
}

/* ---- synthetic inputs ------------------------------------------------------------------
 * VFsphere's rule (src/Tools.jl:907-922) for a union of spheres: nF points per direction at
 * xmin + i/(nF+1)*(xmax-xmin); a point is liquid when rad^2 - ((xh-xo)^2 + (yh-yo)^2 +
 * (zh-zo)^2) > 0 for some sphere; VF is the sequential sum of count copies of 1/nF^dims. */
constexpr int CASE_MAXS = 32;

__global__ void k_case_spheres(DevMesh m, const double* __restrict__ cen, const double* __restrict__ rad, int ns,
                               int nF, int dims, const double* __restrict__ table, double* __restrict__ VF)
{
    const long n0 = m.N[0] + 2 * m.g, n1 = m.N[1] + 2 * m.g, n2 = m.N[2] + 2 * m.g;
    const long total = n0 * n1 * n2;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t % n0) + m.lo, j = (int)((t / n0) % n1) + m.lo, k = (int)(t / (n0 * n1)) + m.lo;
        const double x0 = fco(m, 0, i), x1 = fco(m, 0, i + 1);
        const double y0 = fco(m, 1, j), y1 = fco(m, 1, j + 1);
        const double z0 = fco(m, 2, k), z1 = fco(m, 2, k + 1);
        int cand[CASE_MAXS];
        int nc = 0;
        bool overflow = false, full = false;
        for (int s = 0; s < ns; ++s) {
            const double cx = cen[3 * s], cy = cen[3 * s + 1], cz = cen[3 * s + 2], r = rad[s];
            /* conservative box-box reject */
            if (x1 < cx - r || x0 > cx + r || y1 < cy - r || y0 > cy + r) continue;
            if (dims == 3 && (z1 < cz - r || z0 > cz + r)) continue;
            const double fx = fmax(fabs(x0 - cx), fabs(x1 - cx)), fy = fmax(fabs(y0 - cy), fabs(y1 - cy));
            const double fz = dims == 3 ? fmax(fabs(z0 - cz), fabs(z1 - cz)) : 0.0;
            if (fx * fx + fy * fy + fz * fz < r * r * (1.0 - 1e-12)) { full = true; break; }
            if (nc < CASE_MAXS) cand[nc++] = s;
            else overflow = true;
        }
        const int npts = dims == 3 ? nF * nF * nF : nF * nF;
        int cnt = 0;
        if (full) {
            cnt = npts;
        } else if (nc > 0) {
            const int nzp = dims == 3 ? nF : 1;
            for (int c = 1; c <= nzp; ++c) {
                const double zh = z0 + (double)c / (double)(nF + 1) * (z1 - z0);
                for (int b = 1; b <= nF; ++b) {
                    const double yh = y0 + (double)b / (double)(nF + 1) * (y1 - y0);
                    for (int a = 1; a <= nF; ++a) {
                        const double xh = x0 + (double)a / (double)(nF + 1) * (x1 - x0);
                        bool hit = false;
                        const int nloop = overflow ? ns : nc;
                        for (int q = 0; q < nloop && !hit; ++q) {
                            const int s = overflow ? q : cand[q];
                            const double r = rad[s];
                            const double ex = xh - cen[3 * s], ey = yh - cen[3 * s + 1];
                            double G;
                            if (dims == 3) {
                                const double ez = zh - cen[3 * s + 2];
                                G = r * r - ((ex * ex + ey * ey) + ez * ez);
                            } else {
                                G = r * r - (ex * ex + ey * ey);
                            }
                            hit = G > 0.0;
                        }
                        cnt += hit;
                    }
                }
            }
        }
        VF[vidx(m, i, j, k)] = table[cnt];
    }
}

/* Deformation3D (src/Tools.jl:660-662) with period T, sampled at face centres incl. ghosts. */
__global__ void k_case_deformation3d(DevMesh m, double t, double T, double* uf, double* vf, double* wf)
{
    const long n0 = m.N[0] + 2 * m.g, n1 = m.N[1] + 2 * m.g, n2 = m.N[2] + 2 * m.g;
    const long total = n0 * n1 * n2;
    const double pi = 3.141592653589793;
    const double ct = cos(pi * t / T);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < total; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % n0) + m.lo, j = (int)((q / n0) % n1) + m.lo, k = (int)(q / (n0 * n1)) + m.lo;
        const double x = fco(m, 0, i), y = fco(m, 1, j), z = fco(m, 2, k);
        const double xm = cco(m, 0, i), ym = cco(m, 1, j), zm = cco(m, 2, k);
        const double sx = sin(pi * x), sy = sin(pi * y), sz = sin(pi * z);
        uf[q] = ((2.0 * (sx * sx)) * sin(2.0 * pi * ym)) * sin(2.0 * pi * zm) * ct;
        vf[q] = ((-(sy * sy)) * sin(2.0 * pi * xm)) * sin(2.0 * pi * zm) * ct;
        wf[q] = ((-(sz * sz)) * sin(2.0 * pi * xm)) * sin(2.0 * pi * ym) * ct;
    }
}

/* ---- height-function curvature and face properties --------------------------------------
 * compute_curvature! (src/ELVIRA.jl:141-184) on the interior, in the reference's operation
 * order: 7-cell heights along the normal's strictly dominant axis in the 3x3 columns, times the
 * spacing; central differences; the height function's curvature.  x^(3/2) is x*sqrt(x) (IEEE
 * sqrt, one rounded product).  No strictly dominant component: Curve = 0. */
__device__ __forceinline__ double pow32(double x) { return x * sqrt(x); }

__global__ void k_curvature64(DevMesh m, const double* __restrict__ VF, const double* __restrict__ nx,
                              const double* __restrict__ ny, const double* __restrict__ nz, double* __restrict__ Curve)
{
    const long total = (long)m.N[0] * m.N[1] * m.N[2];
    for (long L = (long)blockIdx.x * blockDim.x + threadIdx.x; L < total; L += (long)gridDim.x * blockDim.x) {
        const int i = 1 + (int)(L % m.N[0]), j = 1 + (int)((L / m.N[0]) % m.N[1]), k = 1 + (int)(L / ((long)m.N[0] * m.N[1]));
        const long c = cidx(m, i, j, k);
        const double ax = fabs(nx[c]), ay = fabs(ny[c]), az = fabs(nz[c]);
        /* dominant axis q, tangential axes (a, b) in the reference's hf index order */
        int q, a, b;
        if (ax > ay && ax > az) { q = 0; a = 1; b = 2; }
        else if (ay > ax && ay > az) { q = 1; a = 2; b = 0; }
        else if (az > ay && az > ax) { q = 2; a = 0; b = 1; }
        else { Curve[c] = 0.0; continue; }
        const long st[3] = {1, m.vs1, m.vs2};
        const long v0 = vidx(m, i, j, k);
        double h[3][3];
        for (int ob = -1; ob <= 1; ++ob)
            for (int oa = -1; oa <= 1; ++oa) {
                const long base = v0 + oa * st[a] + ob * st[b];
                double s = 0.0;
                for (int r = -3; r <= 3; ++r) s += __ldg(VF + base + r * st[q]);
                h[oa + 1][ob + 1] = s * m.d[q];
            }
        const double da = m.d[a], db = m.d[b];
        const double ha = (h[2][1] - h[0][1]) / (2 * da), hb = (h[1][2] - h[1][0]) / (2 * db);
        const double haa = ((h[2][1] - 2 * h[1][1]) + h[0][1]) / (da * da);
        const double hbb = ((h[1][2] - 2 * h[1][1]) + h[1][0]) / (db * db);
        double hab;
        if (q == 0) hab = (((h[2][2] - h[0][2]) - h[2][0]) + h[0][0]) / ((4 * da) * db);
        else hab = (((h[2][2] - h[2][0]) - h[0][2]) + h[0][0]) / (q == 1 ? (4 * da) * db : (4 * db) * da);
        Curve[c] = ((((haa + hbb) + haa * (hb * hb)) + hbb * (ha * ha)) - ((2 * hab) * ha) * hb) /
                   pow32((1 + ha * ha) + hb * hb);
    }
}

/* compute_props! (src/Tools.jl:1186-1210) on every cell: face VF clamp((VF + VF[-1])/2, 0, 1),
 * density and (when visc[0] is not null) viscosity; compute_dens! without viscosities. */
__global__ void k_props64(DevMesh m, const double* __restrict__ VF, double rho_liq, double rho_gas, double mu_liq,
                          double mu_gas, double* denx, double* deny, double* denz, double* viscx, double* viscy,
                          double* viscz)
{
    const int n0 = m.N[0] + 2 * m.g, n1 = m.N[1] + 2 * m.g, n2 = m.N[2] + 2 * m.g;
    const long total = (long)n0 * n1 * n2;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t % n0) + m.lo, j = (int)((t / n0) % n1) + m.lo, k = (int)(t / ((long)n0 * n1)) + m.lo;
        const long v = vidx(m, i, j, k);
        const double c = VF[v];
        const double f[3] = {jmin(1.0, jmax(0.0, (c + VF[v - 1]) / 2)), jmin(1.0, jmax(0.0, (c + VF[v - m.vs1]) / 2)),
                             jmin(1.0, jmax(0.0, (c + VF[v - m.vs2]) / 2))};
        double* den[3] = {denx, deny, denz};
        double* visc[3] = {viscx, viscy, viscz};
        for (int d = 0; d < 3; ++d) {
            den[d][t] = rho_liq * f[d] + rho_gas * (1 - f[d]);
            if (visc[0]) visc[d][t] = f[d] * mu_liq + (1 - f[d]) * mu_gas;
        }
    }
}

/* ---- launchers ------------------------------------------------------------------------ */
void launch_curvature64(const DevMesh& m, const double* VF, const double* nx, const double* ny, const double* nz,
                        double* Curve, int nsm, cudaStream_t s)
{
    const long nc = (long)(m.N[0] + 2 * m.g) * (m.N[1] + 2 * m.g) * (m.N[2] + 2 * m.g);
    cudaMemsetAsync(Curve, 0, nc * sizeof(double), s);
    k_curvature64<<<nsm * 8, 256, 0, s>>>(m, VF, nx, ny, nz, Curve);
}
void launch_props64(const DevMesh& m, const double* VF, double rho_liq, double rho_gas, double mu_liq, double mu_gas,
                    double* denx, double* deny, double* denz, double* viscx, double* viscy, double* viscz, int nsm,
                    cudaStream_t s)
{
    k_props64<<<nsm * 8, 256, 0, s>>>(m, VF, rho_liq, rho_gas, mu_liq, mu_gas, denx, deny, denz, viscx, viscy, viscz);
}
void launch_vf_ghost(const DevMesh& m, const double* VFin, double* VFout, int nsm, cudaStream_t s)
{
    k_vf_ghost<<<nsm * 8, 256, 0, s>>>(m, VFin, VFout);
}
long pure_blocks(long nx, long ny, long nz)
{
    return ((nx + PURE_BX - 1) / PURE_BX) * ((ny + PURE_BY - 1) / PURE_BY) * nz;
}
void launch_elvira_pure(const DevMesh& m, const double* VF, double* nx, double* ny, double* nz, int* list, int* count,
                        long long* partials, cudaStream_t s)
{
    const dim3 grid((m.N[0] + PURE_BX - 1) / PURE_BX, (m.N[1] + PURE_BY - 1) / PURE_BY, m.N[2]);
    k_elvira_pure<<<grid, dim3(PURE_BX, PURE_BY), 0, s>>>(m, VF, nx, ny, nz, list, count, partials);
}
void launch_normal_ghost(const DevMesh& m, double* nx, double* ny, double* nz, int nsm, cudaStream_t s)
{
    k_normal_ghost<<<nsm * 8, 256, 0, s>>>(m, nx, ny, nz);
}
void launch_mass_final(const long long* partials, long nblocks, double cellvol, double* out, cudaStream_t s)
{
    k_mass_final<<<1, MASS_THREADS, 0, s>>>(partials, nblocks, cellvol, out);
}
/* cuTensorMapEncodeTiled, from the driver through the runtime (no link against libcuda) */
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled()
{
    static const EncodeTiledFn fn = []() -> EncodeTiledFn {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return reinterpret_cast<EncodeTiledFn>(f);
    }();
    return fn;
}

/* The TMA map of a VF array for k_band_first_tma: 3D, FP64, box TB_W x TB_H x 1, zero fill
 * outside the array (only cells past N + 1 of a partial tile read there, and no output
 * depends on them).  False where the row or plane stride is not a multiple of 16 bytes (an
 * odd Nx) or the base is not 16-byte aligned: the plain kernel runs then. */
static bool band_tma_map(const DevMesh& m, const double* VF, CUtensorMap* map)
{
    const EncodeTiledFn enc = encode_tiled();
    if (!enc || (m.vs1 * sizeof(double)) % 16 != 0 || (m.vs2 * sizeof(double)) % 16 != 0 ||
        reinterpret_cast<uintptr_t>(VF) % 16 != 0)
        return false;
    const cuuint64_t dims[3] = {(cuuint64_t)m.vs1, (cuuint64_t)(m.vs2 / m.vs1),
                                (cuuint64_t)(m.N[2] + 2 * m.g + 6)};
    const cuuint64_t strides[2] = {(cuuint64_t)m.vs1 * sizeof(double), (cuuint64_t)m.vs2 * sizeof(double)};
    const cuuint32_t box[3] = {TB_W, TB_H, 1}, estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double*>(VF), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

void launch_band_first(const DevMesh& m, const double* VF, short* bout, int* errw, int nsm, cudaStream_t s)
{
    (void)nsm;
    const dim3 grid((m.N[0] + BX - 1) / BX, (m.N[1] + BY - 1) / BY, (m.N[2] + BZ - 1) / BZ);
    CUtensorMap map;
    if (band_tma_map(m, VF, &map))
        k_band_first_tma<<<grid, dim3(BX, BY), 0, s>>>(m, map, bout, errw);
    else
        k_band_first<<<grid, dim3(BX, BY), 0, s>>>(m, VF, bout);
}
void launch_band_ghost(const DevMesh& m, const short* bin, short* bout, bool neumann, int nsm, cudaStream_t s)
{
    k_band_ghost<<<nsm * 8, 256, 0, s>>>(m, bin, bout, neumann);
}
void launch_band_sweep(const DevMesh& m, const short* bin, short* bout, int n, int nsm, cudaStream_t s)
{
    const dim3 grid((m.N[0] + BX - 1) / BX, (m.N[1] + BY - 1) / BY, (m.N[2] + BZ - 1) / BZ);
    k_band_sweep<<<grid, dim3(BX, BY), 0, s>>>(m, bin, bout, n);
}
void launch_sl_classify(const DevMesh& m, const short* band, const double* VFin, double* VFout, int* list, int* count,
                        int nsm, cudaStream_t s)
{
    (void)nsm;
    const dim3 grid((m.N[0] + PURE_BX - 1) / PURE_BX, (m.N[1] + PURE_BY - 1) / PURE_BY, (m.N[2] + CLS_K - 1) / CLS_K);
    k_sl_classify<<<grid, dim3(PURE_BX, PURE_BY), 0, s>>>(m, band, VFin, VFout, list, count);
}
void launch_to_float(const double* a, float* b, long n, double scale, int nsm, cudaStream_t s)
{
    k_to_float<<<nsm * 8, 256, 0, s>>>(a, b, n, scale);
}
void launch_case_spheres(const DevMesh& m, const double* cen, const double* rad, int n, int nF, int dims,
                         const double* table, double* VF, int nsm, cudaStream_t s)
{
    k_case_spheres<<<nsm * 8, 128, 0, s>>>(m, cen, rad, n, nF, dims, table, VF);
}
void launch_case_deformation3d(const DevMesh& m, double t, double T, double* uf, double* vf, double* wf, int nsm,
                               cudaStream_t s)
{
    k_case_deformation3d<<<nsm * 8, 256, 0, s>>>(m, t, T, uf, vf, wf);
}

} // namespace slvof
