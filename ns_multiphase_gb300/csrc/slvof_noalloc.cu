/*
 * slvof_noalloc.cu — total liquid volume of a device-resident VF array without allocating.
 *
 * slvof_mass needs a context, and creating a context allocates device memory.  Some callers
 * cannot allocate: a host framework that owns every device allocation through its own pool
 * (a Julia CUDA.jl program that hands in CuArray pointers, for example), or a monitoring hook
 * that runs between steps of a solver that has reserved all device memory.  This entry point
 * takes the caller's VF and result pointers and keeps its only scratch — one compensated
 * partial sum per z-plane — in a fixed array in the library's static device memory, so it
 * calls no cudaMalloc, cudaFree or allocating library routine.
 *
 * The scratch array lives on every device that loads the library, until the process exits.
 * Its size fixes the largest grid: Nz <= SLVOF_NOALLOC_MAX_PLANES.  Every call uses the same
 * array, so calls that overlap on the GPU (different streams, or several host threads) race;
 * the caller must order them.  Every plane's slot is written before it is read, so nothing
 * has to be cleared between calls.
 */
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/slvof.h"
#include "slvof_dev.cuh"

namespace {

using slvof::Comp;
using slvof::comp_add;
using slvof::comp_merge;

/* (sum, correction) per z-plane.  In host code this name is only a stand-in for the device
 * symbol; kernels receive the device address obtained with cudaGetSymbolAddress. */
static __device__ __align__(256) double g_noalloc_planes[2 * SLVOF_NOALLOC_MAX_PLANES];

constexpr int MASS_THREADS = 256;

/* Block per z-plane (grid-stride over planes): compensated sum of the plane's interior VF. */
__global__ void __launch_bounds__(MASS_THREADS) k_mass_planes(const double* __restrict__ VF, int Nx, int Ny, int Nz,
                                                              long s1, long s2, int off, double* __restrict__ part)
{
    __shared__ double ss[MASS_THREADS / 32], sc[MASS_THREADS / 32];
    const long plane = (long)Nx * Ny;
    for (int k = blockIdx.x; k < Nz; k += gridDim.x) {
        Comp acc{0.0, 0.0};
        for (long t = threadIdx.x; t < plane; t += blockDim.x) {
            const long i = t % Nx, j = t / Nx;
            comp_add(acc, VF[(i + off) + (j + off) * s1 + (k + off) * s2]);
        }
        for (int o = 16; o > 0; o >>= 1) {
            Comp other{__shfl_down_sync(0xffffffffu, acc.s, o), __shfl_down_sync(0xffffffffu, acc.c, o)};
            comp_merge(acc, other);
        }
        const int w = threadIdx.x >> 5;
        if ((threadIdx.x & 31) == 0) { ss[w] = acc.s; sc[w] = acc.c; }
        __syncthreads();
        if (threadIdx.x == 0) {
            Comp b{ss[0], sc[0]};
            for (int q = 1; q < MASS_THREADS / 32; ++q) comp_merge(b, Comp{ss[q], sc[q]});
            part[2 * k] = b.s;
            part[2 * k + 1] = b.c;
        }
        __syncthreads();
    }
}

/* Planes merged in order, times the cell volume (src/WriteData.jl:33). */
__global__ void k_mass_planes_final(const double* __restrict__ part, int Nz, double cellvol, double* out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    Comp a{0.0, 0.0};
    for (int k = 0; k < Nz; ++k) comp_merge(a, Comp{part[2 * k], part[2 * k + 1]});
    out[0] = (a.s + a.c) * cellvol;
}

/* Device address of the scratch array, looked up once per device with that device current. */
constexpr int MAX_DEVICES = 64;
struct ScratchSlot {
    std::once_flag once;
    double* ptr = nullptr;
    cudaError_t status = cudaSuccess;
};
ScratchSlot g_slots[MAX_DEVICES];

} // namespace

extern "C" int slvof_mass_noalloc(const slvof_mesh* mesh, const double* d_VF, double* d_mass, void* stream)
{
    if (!mesh || !d_VF || !d_mass) return SLVOF_E_ARG;
    if (mesh->Nx < 1 || mesh->Ny < 1 || mesh->Nz < 1 || mesh->nghost < 1) return SLVOF_E_ARG;
    if (mesh->Nz > SLVOF_NOALLOC_MAX_PLANES) return SLVOF_E_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SLVOF_E_CUDA;
    if (dev < 0 || dev >= MAX_DEVICES) return SLVOF_E_UNSUPPORTED;
    ScratchSlot& slot = g_slots[dev];
    std::call_once(slot.once, [&] { slot.status = cudaGetSymbolAddress((void**)&slot.ptr, g_noalloc_planes); });
    if (slot.status != cudaSuccess || !slot.ptr) return SLVOF_E_CUDA;
    const long g = mesh->nghost;
    const long n0 = mesh->Nx + 2 * g + 6, n1 = mesh->Ny + 2 * g + 6;
    const int off = (int)(g + 3); /* parent index of interior cell 1 in the VF array */
    const double cellvol = (mesh->dx * mesh->dy) * mesh->dz;
    cudaStream_t s = (cudaStream_t)stream;
    const int blocks = mesh->Nz < 4096 ? mesh->Nz : 4096;
    k_mass_planes<<<blocks, MASS_THREADS, 0, s>>>(d_VF, mesh->Nx, mesh->Ny, mesh->Nz, n0, n0 * n1, off, slot.ptr);
    k_mass_planes_final<<<1, 32, 0, s>>>(slot.ptr, mesh->Nz, cellvol, d_mass);
    return cudaGetLastError() == cudaSuccess ? SLVOF_OK : SLVOF_E_CUDA;
}
