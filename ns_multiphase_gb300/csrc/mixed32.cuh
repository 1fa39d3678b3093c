/*
 * mixed32.cuh — FP32 pieces of the mixed-precision SL path shared by the forward kernels
 * (k_mixed.cu) and the reverse pass (k_adj32.cu): face velocities in cell units, their
 * trilinear interpolation, the RK pre-image projection, pt2index! in local units, the packed
 * donor indices and the donor planes.  Both units build with the same flags, so a trajectory
 * recomputed in the reverse pass rounds as the forward's.
 */
#pragma once

#include "slvof_dev.cuh"

namespace slvof {

struct Vel32 {
    const float *uf, *vf, *wf; /* face velocities in cells per unit time (u/dx, v/dy, w/dz) */
};

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ __forceinline__ float tri32(const DevMesh& m, const float* __restrict__ f, int I, int J, int K, float wx,
                                       float wy, float wz)
{
    const long b = cidx(m, I, J, K);
    const long sj = m.cs1, sk = m.cs2;
    const float f000 = __ldg(f + b), f100 = __ldg(f + b + 1), f010 = __ldg(f + b + sj), f110 = __ldg(f + b + 1 + sj);
    const float f001 = __ldg(f + b + sk), f101 = __ldg(f + b + 1 + sk), f011 = __ldg(f + b + sj + sk),
                f111 = __ldg(f + b + 1 + sj + sk);
    const float x00 = f000 + wx * (f100 - f000), x10 = f010 + wx * (f110 - f010);
    const float x01 = f001 + wx * (f101 - f001), x11 = f011 + wx * (f111 - f011);
    const float y0 = x00 + wy * (x10 - x00), y1 = x01 + wy * (x11 - x01);
    return y0 + wz * (y1 - y0);
}

/* get_velocity_{u,v,w}face (src/Tools.jl:516-641) on the uniform mesh: the interval search
 * becomes floor() clamped to [imino_, imaxo_-1]. */
__device__ __forceinline__ void vel32(const DevMesh& m, const Vel32& V, int i0, int j0, int k0, float x, float y,
                                      float z, float& u, float& v, float& w)
{
    /* keep the float->int conversions in range for any input (a NaN lands on the clamp) */
    const float B = 1.0e6f;
    const float fx = fminf(fmaxf(floorf(x), -B), B), fy = fminf(fmaxf(floorf(y), -B), B), fz = fminf(fmaxf(floorf(z), -B), B);
    const float gx = fminf(fmaxf(floorf(x - 0.5f), -B), B), gy = fminf(fmaxf(floorf(y - 0.5f), -B), B),
                gz = fminf(fmaxf(floorf(z - 0.5f), -B), B);
    const int Fx = clampi(i0 + (int)fx, m.lo, m.hi[0] - 1), Cx = clampi(i0 + (int)gx, m.lo, m.hi[0] - 1);
    const int Fy = clampi(j0 + (int)fy, m.lo, m.hi[1] - 1), Cy = clampi(j0 + (int)gy, m.lo, m.hi[1] - 1);
    const int Fz = clampi(k0 + (int)fz, m.lo, m.hi[2] - 1), Cz = clampi(k0 + (int)gz, m.lo, m.hi[2] - 1);
    const float wfx = x - (float)(Fx - i0), wcx = x - ((float)(Cx - i0) + 0.5f);
    const float wfy = y - (float)(Fy - j0), wcy = y - ((float)(Cy - j0) + 0.5f);
    const float wfz = z - (float)(Fz - k0), wcz = z - ((float)(Cz - k0) + 0.5f);
    u = tri32(m, V.uf, Fx, Cy, Cz, wfx, wcy, wcz);
    v = tri32(m, V.vf, Cx, Fy, Cz, wcx, wfy, wcz);
    w = tri32(m, V.wf, Cx, Cy, Fz, wcx, wcy, wfz);
}

__device__ __forceinline__ void project32(const DevMesh& m, const Vel32& V, int i0, int j0, int k0, float dt,
                                          float& x, float& y, float& z)
{
    if (m.projection == 3) {
        /* test_case == "Zalesak": rotation about (0.5, 0.5) (src/Tools.jl:396-399).  In cell
         * units only the displacement is formed, with cos(a) - 1 = -2 sin^2(a/2), so the
         * absolute error stays near 1e-6 of a cell. */
        const float a = 6.2831853f * dt;
        const float s = sinf(a), h = sinf(0.5f * a), cm1 = -2.f * h * h;
        const float X = (float)(fco(m, 0, i0) - 0.5) + x * (float)m.d[0];
        const float Y = (float)(fco(m, 1, j0) - 0.5) + y * (float)m.d[1];
        const float dX = cm1 * X + s * Y, dY = -s * X + cm1 * Y;
        x += dX / (float)m.d[0];
        y += dY / (float)m.d[1];
        return;
    }
    float u1, v1, w1;
    vel32(m, V, i0, j0, k0, x, y, z, u1, v1, w1);
    if (m.projection == 2) {
        const float h = 0.5f * dt;
        float u2, v2, w2, u3, v3, w3, u4, v4, w4;
        vel32(m, V, i0, j0, k0, x - h * u1, y - h * v1, z - h * w1, u2, v2, w2);
        vel32(m, V, i0, j0, k0, x - h * u2, y - h * v2, z - h * w2, u3, v3, w3);
        vel32(m, V, i0, j0, k0, x - dt * u3, y - dt * v3, z - dt * w3, u4, v4, w4);
        const float s = -dt / 6.f;
        x += s * (u1 + 2.f * u2 + 2.f * u3 + u4);
        y += s * (v1 + 2.f * v2 + 2.f * v3 + v4);
        z += s * (w1 + 2.f * w2 + 2.f * w3 + w4);
    } else if (m.projection == 0) {
        x -= dt * u1; y -= dt * v1; z -= dt * w1;
    } else {
        const float h = 0.5f * dt;
        float u2, v2, w2;
        vel32(m, V, i0, j0, k0, x - h * u1, y - h * v1, z - h * w1, u2, v2, w2);
        x -= dt * u2; y -= dt * v2; z -= dt * w2;
    }
}

/* pt2index! (src/Tools.jl:424-434) in local units, seed s: faces sit at integers. */
constexpr int REL = 6; /* relative index range kept in the clip (|index - cell| <= REL) */

__device__ __forceinline__ int idx32(float u, int s, int lo, int hi, int& err)
{
    int I;
    if (u > (float)(s + 1)) I = (int)fminf(ceilf(u), 1.0e6f) - 1;
    else if (u < (float)s) I = (int)fmaxf(floorf(u), -1.0e6f);
    else I = s;
    if (I < lo) { I = lo; err |= ERR_INDEX; }
    if (I > hi) { I = hi; err |= ERR_INDEX; }
    return I;
}

__device__ __forceinline__ unsigned pack3(int a, int b, int c)
{
    return (unsigned)(a + 128) | ((unsigned)(b + 128) << 8) | ((unsigned)(c + 128) << 16);
}
__device__ __forceinline__ int unpack(unsigned p, int q) { return (int)((p >> (8 * q)) & 255u) - 128; }
struct Plane32 {
    const float4* P; /* (mx, my, mz, Dl): n*d and D - n.o in the donor's own cell frame */
};

__device__ __forceinline__ void cell_of(const DevMesh& m, int L, int& i, int& j, int& k)
{
    i = 1 + L % m.N[0];
    j = 1 + (L / m.N[0]) % m.N[1];
    k = 1 + L / (m.N[0] * m.N[1]);
}

__device__ __forceinline__ void rel_bounds(const DevMesh& m, int i, int j, int k, int* rlo, int* rhi)
{
    rlo[0] = max(m.lo - i, -REL); rlo[1] = max(m.lo - j, -REL); rlo[2] = max(m.lo - k, -REL);
    rhi[0] = min(m.hi[0] - i, REL); rhi[1] = min(m.hi[1] - j, REL); rhi[2] = min(m.hi[2] - k, REL);
}

/* ---- pieces of the warp-cooperative clips (k_sl32_clipw, k_flux_clip) ----------------- */
/* float-float running sum (TwoSum error-free transformation): ~48-bit accumulation of the
 * FP32 sub-tet volumes without using the FP64 pipe. */
struct FF {
    float hi, lo;
};
__device__ __forceinline__ void ff_add(FF& a, float x)
{
    const float s = a.hi + x;
    const float bb = s - a.hi;
    const float e = (a.hi - (s - bb)) + (x - bb);
    a.hi = s;
    a.lo += e;
}
__device__ __forceinline__ void ff_add(FF& a, const FF& b)
{
    ff_add(a, b.hi);
    a.lo += b.lo;
}

/* Warp-aggregated slot reservation: returns this lane's slot (or -1 if !flag). */
__device__ __forceinline__ int warp_slot(bool flag, int* count)
{
    const unsigned act = __activemask();
    const unsigned ballot = __ballot_sync(act, flag);
    if (!ballot) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(ballot) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(ballot));
    base = __shfl_sync(act, base, leader);
    return flag ? base + __popc(ballot & ((1u << lane) - 1)) : -1;
}

__device__ __forceinline__ unsigned wbits(const float4& v) { return (unsigned)__float_as_int(v.w); }
__device__ __forceinline__ float sel4(float a, float b, float c, float d, int i)
{
    return i == 0 ? a : (i == 1 ? b : (i == 2 ? c : d));
}

/* A donor plane's constant moved from the donor's frame to the frame of the cell at index
 * offset -(a, b, c) from it: w + n.(a, b, c). */
__device__ __forceinline__ float rel_dt(const float4& p, int a, int b, int c)
{
    return p.w + p.x * (float)a + p.y * (float)b + p.z * (float)c;
}

/* Side of a node's four vertices against one donor plane (in the batch cell's frame): 1 all
 * strictly liquid, -1 all strictly gas, 0 otherwise. */
__device__ __forceinline__ int plane_side4(const float4& p, const float4* v)
{
    bool neg = true, pos = true;
#pragma unroll
    for (int n = 0; n < 4; ++n) {
        const float d = fmaf(p.x, v[n].x, fmaf(p.y, v[n].y, fmaf(p.z, v[n].z, -p.w)));
        neg = neg && d < 0.f;
        pos = pos && d > 0.f;
    }
    return neg ? 1 : (pos ? -1 : 0);
}

} // namespace slvof
