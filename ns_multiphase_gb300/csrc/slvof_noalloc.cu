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
 *
 * The array's device address belongs to the CUDA context the module is loaded in.  It is
 * looked up (cudaGetSymbolAddress, which allocates nothing) on the first call in a context and
 * kept together with that context's unique id; a call in another context — a non-primary
 * context made current by the caller, or the primary context created again after a device
 * reset — looks it up again.  A failed lookup is not kept.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

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
constexpr int MASS_WARPS = MASS_THREADS / 32;

/* Block per z-plane (grid-stride over planes), warp per row j, lanes over i: compensated sum
 * of the plane's interior VF. */
__global__ void __launch_bounds__(MASS_THREADS) k_mass_planes(const double* __restrict__ VF, int Nx, int Ny, int Nz,
                                                              long s1, long s2, int off, double* __restrict__ part)
{
    __shared__ double ss[MASS_WARPS], sc[MASS_WARPS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = blockIdx.x; k < Nz; k += gridDim.x) {
        Comp acc{0.0, 0.0};
        const double* pk = VF + off + (long)(k + off) * s2;
        for (int j = w; j < Ny; j += MASS_WARPS) {
            const double* row = pk + (long)(j + off) * s1;
            for (int i = lane; i < Nx; i += 32) comp_add(acc, row[i]);
        }
        for (int o = 16; o > 0; o >>= 1) {
            Comp other{__shfl_down_sync(0xffffffffu, acc.s, o), __shfl_down_sync(0xffffffffu, acc.c, o)};
            comp_merge(acc, other);
        }
        if (lane == 0) { ss[w] = acc.s; sc[w] = acc.c; }
        __syncthreads();
        if (threadIdx.x == 0) {
            Comp b{ss[0], sc[0]};
            for (int q = 1; q < MASS_WARPS; ++q) comp_merge(b, Comp{ss[q], sc[q]});
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

/* Unique id of the calling thread's current context (0 if none is current or the driver
 * entry points are unavailable), through the runtime's driver entry-point query, so the
 * library needs no link against the driver library. */
PFN_cuCtxGetCurrent_v4000 p_ctx_current = nullptr;
PFN_cuCtxGetId_v12000 p_ctx_id = nullptr;
std::once_flag g_entry_once;

unsigned long long current_ctx_id()
{
    std::call_once(g_entry_once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            p_ctx_current = (PFN_cuCtxGetCurrent_v4000)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            p_ctx_id = (PFN_cuCtxGetId_v12000)f;
    });
    if (!p_ctx_current || !p_ctx_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (p_ctx_current(&ctx) != CUDA_SUCCESS || !ctx || p_ctx_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

/* Device address of the scratch array per device, with the id of the context it was looked
 * up in. */
constexpr int MAX_DEVICES = 64;
struct ScratchSlot {
    std::mutex mu;
    unsigned long long ctx = 0;
    double* ptr = nullptr;
};
ScratchSlot g_slots[MAX_DEVICES];

cudaError_t scratch_address(int dev, double** out)
{
    ScratchSlot& slot = g_slots[dev];
    std::lock_guard<std::mutex> lock(slot.mu);
    unsigned long long id = current_ctx_id();
    if (id != 0 && slot.ptr && slot.ctx == id) {
        *out = slot.ptr;
        return cudaSuccess;
    }
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_planes);
    if (e != cudaSuccess || !p) {
        slot.ptr = nullptr;
        slot.ctx = 0;
        return e != cudaSuccess ? e : cudaErrorInvalidSymbol;
    }
    /* the lookup makes the device's context current if none was */
    id = current_ctx_id();
    slot.ptr = (double*)p;
    slot.ctx = id; /* 0: no id available, so the next call looks the address up again */
    *out = slot.ptr;
    return cudaSuccess;
}

} // namespace

extern "C" int slvof_mass_noalloc(const slvof_mesh* mesh, const double* d_VF, double* d_mass, void* stream)
{
    if (!mesh || !d_VF || !d_mass) return SLVOF_E_ARG;
    if (mesh->Nx < 1 || mesh->Ny < 1 || mesh->Nz < 1 || mesh->nghost < 1) return SLVOF_E_ARG;
    if (mesh->Nz > SLVOF_NOALLOC_MAX_PLANES) return SLVOF_E_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SLVOF_E_CUDA;
    if (dev < 0 || dev >= MAX_DEVICES) return SLVOF_E_UNSUPPORTED;
    double* part = nullptr;
    if (scratch_address(dev, &part) != cudaSuccess) return SLVOF_E_CUDA;
    const long g = mesh->nghost;
    const long n0 = mesh->Nx + 2 * g + 6, n1 = mesh->Ny + 2 * g + 6;
    int off = (int)(g + 3); /* parent index of interior cell 1 in the VF array */
    int Nx = mesh->Nx, Ny = mesh->Ny, Nz = mesh->Nz;
    long s1 = n0, s2 = n0 * n1;
    double cellvol = (mesh->dx * mesh->dy) * mesh->dz;
    const double* vf = d_VF;
    cudaStream_t s = (cudaStream_t)stream;
    /* launched through cudaLaunchKernel so that the status is this launch's own, not an error
     * left pending by earlier unrelated work */
    const unsigned blocks = (unsigned)(Nz < 4096 ? Nz : 4096);
    void* a1[] = {(void*)&vf, (void*)&Nx, (void*)&Ny, (void*)&Nz, (void*)&s1, (void*)&s2, (void*)&off, (void*)&part};
    if (cudaLaunchKernel((const void*)k_mass_planes, dim3(blocks), dim3(MASS_THREADS), a1, 0, s) != cudaSuccess)
        return SLVOF_E_CUDA;
    const double* cpart = part;
    void* a2[] = {(void*)&cpart, (void*)&Nz, (void*)&cellvol, (void*)&d_mass};
    if (cudaLaunchKernel((const void*)k_mass_planes_final, dim3(1), dim3(32), a2, 0, s) != cudaSuccess)
        return SLVOF_E_CUDA;
    return SLVOF_OK;
}
