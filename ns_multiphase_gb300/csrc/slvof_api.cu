/*
 * slvof_api.cu — C ABI of the SL-VOF library (declared in include/slvof.h).
 *
 * A context owns every device buffer of one mesh and a private stream.  The resident step
 * runs, without host round trips between kernels:
 *   classify band cells + copy the rest  ->  SL update (FP64 or mixed)  ->  VF ghost fill
 *   ->  ELVIRA pure cells + interface list + mass partials  ->  ELVIRA candidates
 *   ->  normal borders  ->  PLIC distances  ->  [band]  ->  [mass]
 * and reads back the device error word once at the end.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/slvof.h"
#include "slvof_kernels.h"

using namespace slvof;

struct slvof_ctx {
    int precision = SLVOF_FP64;
    int device = 0;
    int nsm = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    DevMesh m{};
    double* coords = nullptr;
    long ncell = 0, nvf = 0;
    double* VF[2] = {nullptr, nullptr};
    int vcur = 0;
    double *uf = nullptr, *vf = nullptr, *wf = nullptr;
    float *uf32 = nullptr, *vf32 = nullptr, *wf32 = nullptr;
    double *nx = nullptr, *ny = nullptr, *nz = nullptr, *D = nullptr;
    float4* planes = nullptr;     /* mixed: donor planes in cell units */
    int2* arb = nullptr;          /* mixed ELVIRA: near-tie cells (cell, contending lanes) for FP64 scoring */
    int* slow_cells = nullptr;    /* mixed SL: cells that need the clip */
    float4* slow_verts = nullptr; /* mixed SL: their pre-image vertices (cell units) + packed indices */
    FluxLaunch flux{};            /* mixed SL in flux form: node displacements, face sums, lists */
    signed char* phase = nullptr; /* pure-donor codes of the PLIC pass */
    signed char* cand = nullptr;  /* ELVIRA: chosen candidate lane of each interface cell */
    /* reverse pass (allocated on first use) */
    double* gvf[2] = {nullptr, nullptr}; /* dL/dVF (current, scratch) */
    double* gfold = nullptr;
    double *gn[3] = {nullptr, nullptr, nullptr}, *gD = nullptr;
    double *gnf[3] = {nullptr, nullptr, nullptr}, *gDf = nullptr;
    double *guf = nullptr, *gvf_ = nullptr, *gwf = nullptr;
    int* list_adj = nullptr;
    double* gvtx[3] = {nullptr, nullptr, nullptr}; /* mixed: dL/d(traced grid vertices), cell units */
    float2* cinfo = nullptr;                       /* mixed: per clip cell g * tetsign / vol and VFnew */
    float* gvel32[3] = {nullptr, nullptr, nullptr}; /* mixed: one step's face-velocity derivatives */
    /* momentum of transport! (allocated on first use): cell-centred velocities in, us/vs/ws out */
    double *cu = nullptr, *cv = nullptr, *cw = nullptr, *us = nullptr, *vs = nullptr, *ws = nullptr;
    /* divergence and A! with host arrays (allocated on first use): face velocities, P,
     * densities, corrected velocities, the result, and the band */
    double* pr[11] = {};
    short* pr_band = nullptr;
    AdjCell* adj_cells = nullptr;
    AdjTet* adj_tets = nullptr;
    long adj_cells_cap = 0, adj_tets_cap = 0;
    short* band[2] = {nullptr, nullptr};
    int bcur = 0;
    int* list_sl = nullptr;
    int* list_if = nullptr;
    int* list_plic = nullptr; /* cells whose PLIC solve is deferred to full warps */
    int* ctr = nullptr; /* 0 sl count, 1 if count, 2 sl work, 3 if work, 4 error bits */
    long long* partials = nullptr; /* exact mass partials, (high, low) words of a 128-bit sum per block */
    long npure = 0;
    double* mass_d = nullptr;
    double* table = nullptr; /* case generator scratch */
    int table_n = 0;
    double* spheres = nullptr;
    int spheres_n = 0;
    bool normals_valid = false;
    /* slvof_step_host with SLVOF_STEP_DEFER left the new state's normals and PLIC (and its band
     * when deferred_band) to the next call; deferred_err holds device error bits of deferred
     * stages that another entry point ran, until its status reports them */
    bool deferred = false, deferred_band = false;
    int deferred_err = 0;
    double rho_liq = 1.0, rho_gas = 1.0;
    double last_ms = 0.0;
    cudaStream_t own_stream = nullptr;
    /* slvof_step_host copies VF out on copy_stream while the next state's geometry is built;
     * the steps build the band on band_stream beside the normals and PLIC */
    cudaStream_t copy_stream = nullptr, band_stream = nullptr;
    cudaEvent_t ev_state = nullptr, ev_copied = nullptr, ev_band = nullptr, ev_up = nullptr;
    cudaEvent_t sev[SLVOF_NSTAGES][2] = {};
    bool sran[SLVOF_NSTAGES] = {};
    std::string err;
};

namespace {

enum { C_SL = 0, C_IF = 1, C_SLW = 2, C_IFW = 3, C_ERR = 4, C_PL = 5, C_SLOW = 6, C_SLW2 = 7, C_ARB = 8, C_ADJ = 9,
       C_ADJW = 10, C_ADJ2 = 11, C_N = 16 };

int fail(slvof_ctx* c, int code, const std::string& msg)
{
    if (c) c->err = msg;
    return code;
}

#define CK(call)                                                                                             \
    do {                                                                                                     \
        cudaError_t e_ = (call);                                                                             \
        if (e_ != cudaSuccess) return fail(c, SLVOF_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define TRY(x)                \
    do {                      \
        int r_ = (x);         \
        if (r_ < 0) return r_; \
    } while (0)

enum { S_CLASSIFY, S_SL, S_VFGHOST, S_PURE, S_IFACE, S_NGHOST, S_PLIC, S_BAND, S_MASS };

int flush_deferred(slvof_ctx* c);

/* Every entry point starts here; all but a deferring slvof_step_host first build the state a
 * deferring call left (flush). */
int begin(slvof_ctx* c, bool flush = true)
{
    if (!c) return SLVOF_E_ARG;
    CK(cudaSetDevice(c->device));
    if (flush && c->deferred) {
        const int r = flush_deferred(c);
        if (r < 0) return r;
    }
    CK(cudaEventRecord(c->ev0, c->stream));
    for (bool& r : c->sran) r = false;
    return 0;
}

/* stage markers: events around each launch group (on the stream the group runs on) */
void s_beg(slvof_ctx* c, int s, cudaStream_t st = nullptr)
{
    cudaEventRecord(c->sev[s][0], st ? st : c->stream);
    c->sran[s] = true;
}
void s_end(slvof_ctx* c, int s, cudaStream_t st = nullptr) { cudaEventRecord(c->sev[s][1], st ? st : c->stream); }

/* Synchronise, time the call and fold the device error word into the status. */
int finish(slvof_ctx* c, bool read_err = true)
{
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    c->last_ms = ms;
    if (!read_err) return SLVOF_OK;
    int e = 0;
    CK(cudaMemcpy(&e, c->ctr + C_ERR, sizeof(int), cudaMemcpyDeviceToHost));
    e |= c->deferred_err;
    c->deferred_err = 0;
    if (e) {
        char buf[160];
        snprintf(buf, sizeof buf, "device error bits 0x%x (1 index range, 2 clip depth, 4 NaN distance, 8 volume)", e);
        c->err = buf;
    }
    return e;
}

int clear_err(slvof_ctx* c)
{
    CK(cudaMemsetAsync(c->ctr + C_ERR, 0, sizeof(int), c->stream));
    return 0;
}

/* ---- stages (enqueue only) -------------------------------------------------------------- */
int st_vf_ghost_inplace(slvof_ctx* c)
{
    const int o = 1 - c->vcur;
    CK(cudaMemcpyAsync(c->VF[o], c->VF[c->vcur], c->nvf * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    launch_vf_ghost(c->m, c->VF[c->vcur], c->VF[o], c->nsm, c->stream);
    c->vcur = o;
    return 0;
}

int st_normals(slvof_ctx* c)
{
    CK(cudaMemsetAsync(c->ctr + C_IF, 0, sizeof(int), c->stream));
    CK(cudaMemsetAsync(c->ctr + C_IFW, 0, sizeof(int), c->stream));
    CK(cudaMemsetAsync(c->ctr + C_ARB, 0, sizeof(int), c->stream));
    s_beg(c, S_PURE);
    launch_elvira_pure(c->m, c->VF[c->vcur], c->nx, c->ny, c->nz, c->list_if, c->ctr + C_IF, c->partials, c->stream);
    s_end(c, S_PURE);
    s_beg(c, S_IFACE);
    if (c->precision == SLVOF_FP64)
        launch_elvira_iface64(c->m, c->VF[c->vcur], c->nx, c->ny, c->nz, c->list_if, c->ctr + C_IF, c->ctr + C_IFW,
                              c->cand, c->ctr + C_ERR, c->nsm, c->stream);
    else
        launch_elvira_iface32(c->m, c->VF[c->vcur], c->nx, c->ny, c->nz, c->list_if, c->ctr + C_IF, c->ctr + C_IFW,
                              c->ctr + C_ARB, c->arb, c->cand, c->ctr + C_ERR, c->nsm, c->stream);
    s_end(c, S_IFACE);
    s_beg(c, S_NGHOST);
    launch_normal_ghost(c->m, c->nx, c->ny, c->nz, c->nsm, c->stream);
    s_end(c, S_NGHOST);
    c->normals_valid = true;
    return 0;
}

int st_plic(slvof_ctx* c)
{
    s_beg(c, S_PLIC);
    CK(cudaMemsetAsync(c->ctr + C_PL, 0, sizeof(int), c->stream));
    launch_plic64(c->m, c->VF[c->vcur], c->nx, c->ny, c->nz, c->D, c->planes, c->phase, c->list_plic, c->ctr + C_PL,
                  c->precision == SLVOF_MIXED, c->nsm, c->stream);
    s_end(c, S_PLIC);
    return 0;
}

int st_band(slvof_ctx* c, cudaStream_t st = nullptr)
{
    cudaStream_t s = st ? st : c->stream;
    int b = c->bcur;
    s_beg(c, S_BAND, s);
    launch_band_first(c->m, c->VF[c->vcur], c->band[1 - b], c->ctr + C_ERR, c->nsm, s);
    launch_band_ghost(c->m, c->band[b], c->band[1 - b], true, c->nsm, s);
    b = 1 - b;
    for (int n = 1; n <= c->m.nband; ++n) {
        launch_band_sweep(c->m, c->band[b], c->band[1 - b], n, c->nsm, s);
        launch_band_ghost(c->m, c->band[b], c->band[1 - b], false, c->nsm, s);
        b = 1 - b;
    }
    c->bcur = b;
    s_end(c, S_BAND, s);
    return 0;
}

/* The band of the new state reads only VF, which the normals, PLIC and mass only read, and
 * they do not touch the band: after the transport it is built on band_stream beside them, and
 * the call's stream waits for ev_band before the call ends (join_band). */
int st_band_side(slvof_ctx* c)
{
    CK(cudaEventRecord(c->ev_state, c->stream));
    CK(cudaStreamWaitEvent(c->band_stream, c->ev_state, 0));
    st_band(c, c->band_stream);
    CK(cudaEventRecord(c->ev_band, c->band_stream));
    return 0;
}

/* The call's stream waits for the side band; after an error the band stream is drained so
 * that no band kernel outlives the call. */
int join_band(slvof_ctx* c, int r)
{
    const cudaError_t e = cudaStreamWaitEvent(c->stream, c->ev_band, 0);
    if (r < 0 || e != cudaSuccess) {
        cudaStreamSynchronize(c->band_stream);
        return r < 0 ? r : fail(c, SLVOF_E_CUDA, std::string("band join: ") + cudaGetErrorString(e));
    }
    return 0;
}

/* Mixed SL update of the band cells into VF[o]: the flux form (each face swept once, its
 * volume in FP64 and its liquid from the FP32 clip, shared by the two cells beside it). */
void st_sl32(slvof_ctx* c, double dt, int o)
{
    cudaMemsetAsync(c->ctr + C_SLOW, 0, 2 * sizeof(int), c->stream); /* near-pure cells, their clip work */
    launch_sl32_flux(c->m, dt, c->VF[c->vcur], c->VF[o], c->uf32, c->vf32, c->wf32, c->uf, c->vf, c->wf, c->planes,
                     c->band[c->bcur], c->list_sl, c->ctr + C_SL, c->flux, c->slow_cells, c->slow_verts,
                     c->ctr + C_SLOW, c->ctr + C_SLW2, c->ctr + C_ERR, c->nsm, c->stream);
}

int st_transport(slvof_ctx* c, double dt)
{
    const int o = 1 - c->vcur;
    CK(cudaMemsetAsync(c->ctr + C_SL, 0, sizeof(int), c->stream));
    CK(cudaMemsetAsync(c->ctr + C_SLW, 0, sizeof(int), c->stream));
    CK(cudaMemsetAsync(c->ctr + C_SLOW, 0, 2 * sizeof(int), c->stream)); /* slow count, clip work */
    s_beg(c, S_CLASSIFY);
    launch_sl_classify(c->m, c->band[c->bcur], c->VF[c->vcur], c->VF[o], c->list_sl, c->ctr + C_SL, c->nsm, c->stream);
    s_end(c, S_CLASSIFY);
    s_beg(c, S_SL);
    if (c->precision == SLVOF_FP64)
        launch_sl64(c->m, dt, c->VF[c->vcur], c->VF[o], c->uf, c->vf, c->wf, c->nx, c->ny, c->nz, c->D, c->phase,
                    c->list_sl, c->ctr + C_SL, c->ctr + C_SLW, c->ctr + C_ERR, c->nsm, c->stream);
    else
        st_sl32(c, dt, o);
    s_end(c, S_SL);
    s_beg(c, S_VFGHOST);
    launch_vf_ghost(c->m, c->VF[c->vcur], c->VF[o], c->nsm, c->stream);
    s_end(c, S_VFGHOST);
    c->vcur = o;
    c->normals_valid = false;
    return 0;
}

int mom_alloc(slvof_ctx* c)
{
    if (c->cu) return 0;
    double** bufs[6] = {&c->cu, &c->cv, &c->cw, &c->us, &c->vs, &c->ws};
    for (double** b : bufs) {
        if (cudaMalloc((void**)b, c->ncell * sizeof(double)) != cudaSuccess ||
            cudaMemset(*b, 0, c->ncell * sizeof(double)) != cudaSuccess)
            return fail(c, SLVOF_E_NOMEM, "momentum buffers");
    }
    return 0;
}

/* transport!'s SL section with its momentum (src/Transport.jl:34-181, pressure_scheme
 * "semi-lagrangian"), FP64. */
int st_transport_mom(slvof_ctx* c, double dt)
{
    const int o = 1 - c->vcur;
    CK(cudaMemsetAsync(c->ctr + C_SL, 0, sizeof(int), c->stream));
    CK(cudaMemsetAsync(c->ctr + C_SLW, 0, sizeof(int), c->stream));
    s_beg(c, S_CLASSIFY);
    launch_sl_classify(c->m, c->band[c->bcur], c->VF[c->vcur], c->VF[o], c->list_sl, c->ctr + C_SL, c->nsm, c->stream);
    s_end(c, S_CLASSIFY);
    s_beg(c, S_SL);
    launch_sl64_momentum(c->m, dt, c->VF[o], c->uf, c->vf, c->wf, c->nx, c->ny, c->nz, c->D, c->phase,
                         c->band[c->bcur], c->cu, c->cv, c->cw, c->rho_liq, c->rho_gas, c->us, c->vs, c->ws,
                         c->list_sl, c->ctr + C_SL, c->ctr + C_SLW, c->ctr + C_ERR, c->nsm, c->stream);
    s_end(c, S_SL);
    s_beg(c, S_VFGHOST);
    launch_vf_ghost(c->m, c->VF[c->vcur], c->VF[o], c->nsm, c->stream);
    s_end(c, S_VFGHOST);
    c->vcur = o;
    c->normals_valid = false;
    return 0;
}

int st_mass(slvof_ctx* c, double* mass, bool partials_ready)
{
    s_beg(c, S_MASS);
    if (!partials_ready)
        launch_elvira_pure(c->m, c->VF[c->vcur], nullptr, nullptr, nullptr, nullptr, nullptr, c->partials, c->stream);
    launch_mass_final(c->partials, c->npure, c->m.cellvol, c->mass_d, c->stream);
    s_end(c, S_MASS);
    CK(cudaMemcpyAsync(mass, c->mass_d, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    return 0;
}

int h2d(slvof_ctx* c, void* dst, const void* src, size_t bytes)
{
    if (!src) return fail(c, SLVOF_E_ARG, "null host pointer");
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream));
    return 0;
}
int d2h(slvof_ctx* c, void* dst, const void* src, size_t bytes)
{
    if (!dst) return fail(c, SLVOF_E_ARG, "null host pointer");
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
    return 0;
}

/* Mixed mode keeps FP32 face velocities in cells per unit time (u/dx, v/dy, w/dz). */
void to_float_velocity(slvof_ctx* c)
{
    if (c->precision != SLVOF_MIXED) return;
    launch_to_float(c->uf, c->uf32, c->ncell, 1.0 / c->m.d[0], c->nsm, c->stream);
    launch_to_float(c->vf, c->vf32, c->ncell, 1.0 / c->m.d[1], c->nsm, c->stream);
    launch_to_float(c->wf, c->wf32, c->ncell, 1.0 / c->m.d[2], c->nsm, c->stream);
}

int up_velocity(slvof_ctx* c, const double* uf, const double* vf, const double* wf)
{
    int r;
    const size_t b = c->ncell * sizeof(double);
    if ((r = h2d(c, c->uf, uf, b)) || (r = h2d(c, c->vf, vf, b)) || (r = h2d(c, c->wf, wf, b))) return r;
    to_float_velocity(c);
    return 0;
}

/* The state a deferring slvof_step_host left (normals, PLIC and, when asked, the band of its
 * VF), built on the call's stream while this call's face velocities upload on copy_stream.
 * The stages read VF, the normals and the band, never the face velocities, so nothing orders
 * them against the upload; the upload waits only for the caller's earlier work on the stream.
 * The kernels are enqueued before the copies, since a copy from pageable memory returns only
 * once its data is staged. */
int up_velocity_beside(slvof_ctx* c, const double* uf, const double* vf, const double* wf)
{
    if (!uf || !vf || !wf) return fail(c, SLVOF_E_ARG, "null host pointer");
    CK(cudaEventRecord(c->ev_state, c->stream));
    CK(cudaStreamWaitEvent(c->copy_stream, c->ev_state, 0));
    if (!c->normals_valid) {
        const bool band = c->deferred && c->deferred_band;
        int r = band ? st_band_side(c) : 0;
        if (r >= 0) r = st_normals(c);
        if (r >= 0) r = st_plic(c);
        if (band) r = join_band(c, r);
        if (r < 0) return r;
    }
    c->deferred = c->deferred_band = false;
    const size_t b = c->ncell * sizeof(double);
    cudaError_t e = cudaMemcpyAsync(c->uf, uf, b, cudaMemcpyHostToDevice, c->copy_stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->vf, vf, b, cudaMemcpyHostToDevice, c->copy_stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->wf, wf, b, cudaMemcpyHostToDevice, c->copy_stream);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev_up, c->copy_stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->ev_up, 0);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(c->copy_stream);
        return fail(c, SLVOF_E_CUDA, std::string("velocity upload: ") + cudaGetErrorString(e));
    }
    to_float_velocity(c);
    return 0;
}

/* Builds the state a deferring slvof_step_host left, before another entry point reads or
 * replaces it; the device error bits of these stages join that entry point's status. */
int flush_deferred(slvof_ctx* c)
{
    const bool band = c->deferred_band;
    c->deferred = c->deferred_band = false;
    TRY(clear_err(c));
    if (band) TRY(st_band(c));
    if (!c->normals_valid) {
        TRY(st_normals(c));
        TRY(st_plic(c));
    }
    CK(cudaStreamSynchronize(c->stream));
    int e = 0;
    CK(cudaMemcpy(&e, c->ctr + C_ERR, sizeof(int), cudaMemcpyDeviceToHost));
    c->deferred_err |= e;
    return 0;
}

} // namespace

extern "C" {

int slvof_create(const slvof_mesh* mesh, int precision, slvof_ctx** out)
{
    if (!mesh || !out) return SLVOF_E_ARG;
    *out = nullptr;
    if (precision != SLVOF_FP64 && precision != SLVOF_MIXED) return SLVOF_E_ARG;
    if (mesh->Nx < 1 || mesh->Ny < 1 || mesh->Nz < 1 || mesh->nghost < 3) return SLVOF_E_ARG;
    if (mesh->projection < 0 || mesh->projection > 3 || mesh->nband < 0) return SLVOF_E_ARG;
    if (mesh->tesselation != 0 && mesh->tesselation != 5 && mesh->tesselation != 6 && mesh->tesselation != 24)
        return SLVOF_E_ARG;
    if (!mesh->x || !mesh->y || !mesh->z || !mesh->xm || !mesh->ym || !mesh->zm) return SLVOF_E_ARG;
    if (mesh->pressure_scheme != SLVOF_PRESSURE_SEMI_LAGRANGIAN && mesh->pressure_scheme != SLVOF_PRESSURE_FINITE_DIFFERENCE)
        return SLVOF_E_ARG;
    /* the flux-correction tets of the finite-difference scheme exist for 5_tets in the
     * reference (add_correction_tets keeps the first five tets), and run in FP64 here */
    if (mesh->pressure_scheme == SLVOF_PRESSURE_FINITE_DIFFERENCE && mesh->tesselation != 0 && mesh->tesselation != 5)
        return SLVOF_E_UNSUPPORTED;
    /* the pure/interface thresholds are compared as bit patterns, which orders doubles like the
     * floating-point compare only against positive finite thresholds */
    if (!(mesh->VFlo > 0.0 && mesh->VFhi > 0.0 && mesh->VFlo < 1e300 && mesh->VFhi < 1e300)) return SLVOF_E_UNSUPPORTED;
    const long g = mesh->nghost;
    const long N[3] = {mesh->Nx, mesh->Ny, mesh->Nz};
    const long n0 = N[0] + 2 * g, n1 = N[1] + 2 * g, n2 = N[2] + 2 * g;
    if (n0 * n1 * n2 > (1L << 31) - 1 || N[0] > 30000 || N[1] > 30000 || N[2] > 30000) return SLVOF_E_UNSUPPORTED;
    /* the mixed path's face lists hold (cell index << 2 | direction) in 32 bits */
    if (precision == SLVOF_MIXED && n0 * n1 * n2 >= (1L << 30)) return SLVOF_E_UNSUPPORTED;
    slvof_ctx* c = new slvof_ctx();
    c->precision = precision;
    auto bail = [&](int code) {
        slvof_destroy(c);
        return code;
    };
    if (cudaGetDevice(&c->device) != cudaSuccess) return bail(SLVOF_E_CUDA);
    if (cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess) return bail(SLVOF_E_CUDA);
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) return bail(SLVOF_E_CUDA);
    c->stream = c->own_stream;
    if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) return bail(SLVOF_E_CUDA);
    if (cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->band_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_state, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_copied, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_band, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_up, cudaEventDisableTiming) != cudaSuccess)
        return bail(SLVOF_E_CUDA);
    for (int q = 0; q < SLVOF_NSTAGES; ++q)
        if (cudaEventCreate(&c->sev[q][0]) != cudaSuccess || cudaEventCreate(&c->sev[q][1]) != cudaSuccess)
            return bail(SLVOF_E_CUDA);
    c->ncell = n0 * n1 * n2;
    c->nvf = (n0 + 6) * (n1 + 6) * (n2 + 6);
    const long interior = N[0] * N[1] * N[2];
    c->npure = pure_blocks(N[0], N[1], N[2]);
    auto alloc = [&](void** p, size_t bytes) { return cudaMalloc(p, bytes) == cudaSuccess && cudaMemset(*p, 0, bytes) == cudaSuccess; };
    const long ncoord = mesh_coords(mesh, nullptr);
    bool ok = alloc((void**)&c->coords, ncoord * sizeof(double)) && alloc((void**)&c->VF[0], c->nvf * sizeof(double)) &&
              alloc((void**)&c->VF[1], c->nvf * sizeof(double)) && alloc((void**)&c->uf, c->ncell * sizeof(double)) &&
              alloc((void**)&c->vf, c->ncell * sizeof(double)) && alloc((void**)&c->wf, c->ncell * sizeof(double)) &&
              alloc((void**)&c->nx, c->ncell * sizeof(double)) && alloc((void**)&c->ny, c->ncell * sizeof(double)) &&
              alloc((void**)&c->nz, c->ncell * sizeof(double)) && alloc((void**)&c->D, c->ncell * sizeof(double)) &&
              alloc((void**)&c->phase, c->ncell * sizeof(signed char)) &&
              alloc((void**)&c->cand, c->ncell * sizeof(signed char)) &&
              alloc((void**)&c->band[0], c->ncell * sizeof(short)) && alloc((void**)&c->band[1], c->ncell * sizeof(short)) &&
              alloc((void**)&c->list_sl, interior * sizeof(int)) && alloc((void**)&c->list_if, interior * sizeof(int)) &&
              alloc((void**)&c->list_plic, c->ncell * sizeof(int)) &&
              alloc((void**)&c->ctr, C_N * sizeof(int)) && alloc((void**)&c->partials, 2 * c->npure * sizeof(long long)) &&
              alloc((void**)&c->mass_d, sizeof(double));
    if (ok && precision == SLVOF_MIXED)
        ok = alloc((void**)&c->uf32, c->ncell * sizeof(float)) && alloc((void**)&c->vf32, c->ncell * sizeof(float)) &&
             alloc((void**)&c->wf32, c->ncell * sizeof(float)) && alloc((void**)&c->planes, c->ncell * sizeof(float4)) &&
             alloc((void**)&c->slow_cells, interior * sizeof(int)) &&
             alloc((void**)&c->slow_verts, interior *
                                               ((mesh->tesselation == 24 ||
                                                 mesh->pressure_scheme == SLVOF_PRESSURE_FINITE_DIFFERENCE) ? 16 : 8) *
                                               sizeof(float4)) &&
             alloc((void**)&c->arb, interior * sizeof(int2));
    if (ok && precision == SLVOF_MIXED) {
        for (int q = 0; q < 3 && ok; ++q)
            ok = alloc((void**)&c->flux.nd[q], c->ncell * sizeof(double)) &&
                 alloc((void**)&c->flux.fvf[q], c->ncell * sizeof(double2));
        ok = ok && alloc((void**)&c->flux.nodes, c->ncell * sizeof(unsigned)) &&
             alloc((void**)&c->flux.faces, 3 * c->ncell * sizeof(unsigned)) &&
             alloc((void**)&c->flux.clip, 3 * c->ncell * sizeof(unsigned)) &&
             alloc((void**)&c->flux.ctr, 4 * sizeof(int));
        for (int q = 0; q < 3 && ok && mesh->pressure_scheme == SLVOF_PRESSURE_FINITE_DIFFERENCE; ++q)
            ok = alloc((void**)&c->flux.fapex[q], c->ncell * sizeof(float4));
    }
    if (!ok) return bail(SLVOF_E_NOMEM);
    /* coordinates: x, y, z (faces) then xm, ym, zm (centres) */
    std::vector<double> h(ncoord);
    mesh_coords(mesh, h.data());
    const double* fsrc[3] = {mesh->x, mesh->y, mesh->z};
    const long nn[3] = {n0, n1, n2};
    if (precision == SLVOF_MIXED) {
        /* the FP32 geometry works in cell units and needs a uniform mesh (src/Mesh.jl:83-100) */
        const double dd[3] = {mesh->dx, mesh->dy, mesh->dz};
        for (int q = 0; q < 3; ++q)
            for (long t = 0; t <= nn[q]; ++t)
                if (std::fabs(fsrc[q][t] - (fsrc[q][0] + (double)t * dd[q])) > 1e-9 * dd[q]) return bail(SLVOF_E_UNSUPPORTED);
    }
    if (cudaMemcpy(c->coords, h.data(), ncoord * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(SLVOF_E_CUDA);
    mesh_fill(mesh, c->coords, c->m);
    c->rho_liq = mesh->rho_liq;
    c->rho_gas = mesh->rho_gas;
    *out = c;
    return SLVOF_OK;
}

int slvof_destroy(slvof_ctx* c)
{
    if (!c) return SLVOF_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    void* bufs[] = {c->coords, c->VF[0], c->VF[1], c->uf, c->vf, c->wf, c->uf32, c->vf32, c->wf32, c->nx, c->ny,
                    c->nz, c->D, c->planes, c->phase, c->cand, c->band[0], c->band[1], c->list_sl, c->list_if,
                    c->list_plic, c->slow_cells, c->slow_verts, c->arb, c->ctr, c->partials, c->mass_d, c->table,
                    c->spheres, c->gvf[0], c->gvf[1], c->gfold, c->gn[0], c->gn[1], c->gn[2], c->gD, c->gnf[0],
                    c->gnf[1], c->gnf[2], c->gDf, c->guf, c->gvf_, c->gwf, c->list_adj, c->adj_cells, c->adj_tets,
                    c->gvtx[0], c->gvtx[1], c->gvtx[2], c->cinfo, c->gvel32[0], c->gvel32[1], c->gvel32[2],
                    c->flux.nd[0], c->flux.nd[1], c->flux.nd[2], c->flux.fvf[0], c->flux.fvf[1], c->flux.fvf[2],
                    c->flux.nodes, c->flux.faces, c->flux.clip, c->flux.fapex[0], c->flux.fapex[1], c->flux.fapex[2],
                    c->flux.ctr,
                    c->cu, c->cv, c->cw, c->us, c->vs, c->ws, c->pr[0], c->pr[1], c->pr[2], c->pr[3],
                    c->pr[4], c->pr[5], c->pr[6], c->pr[7], c->pr[8], c->pr[9], c->pr[10], c->pr_band};
    for (void* b : bufs)
        if (b) cudaFree(b);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (int q = 0; q < SLVOF_NSTAGES; ++q)
        for (int e = 0; e < 2; ++e)
            if (c->sev[q][e]) cudaEventDestroy(c->sev[q][e]);
    if (c->ev_state) cudaEventDestroy(c->ev_state);
    if (c->ev_copied) cudaEventDestroy(c->ev_copied);
    if (c->ev_band) cudaEventDestroy(c->ev_band);
    if (c->ev_up) cudaEventDestroy(c->ev_up);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->band_stream) cudaStreamDestroy(c->band_stream);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
    return SLVOF_OK;
}

int slvof_last_error(const slvof_ctx* c, char* buf, size_t n)
{
    if (!c || !buf || n == 0) return SLVOF_E_ARG;
    snprintf(buf, n, "%s", c->err.c_str());
    return SLVOF_OK;
}

int slvof_last_kernel_ms(const slvof_ctx* c, double* ms)
{
    if (!c || !ms) return SLVOF_E_ARG;
    *ms = c->last_ms;
    return SLVOF_OK;
}

int slvof_stage_ms(const slvof_ctx* c, double* ms, int n)
{
    if (!c || !ms || n < 0) return SLVOF_E_ARG;
    for (int q = 0; q < n && q < SLVOF_NSTAGES; ++q) {
        float t = 0.f;
        ms[q] = (c->sran[q] && cudaEventElapsedTime(&t, c->sev[q][0], c->sev[q][1]) == cudaSuccess) ? t : 0.0;
    }
    return SLVOF_OK;
}

int slvof_counters(const slvof_ctx* c, int* out, int n)
{
    if (!c || !out || n < 0) return SLVOF_E_ARG;
    int h[C_N] = {0};
    if (cudaMemcpy(h, c->ctr, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess) return SLVOF_E_CUDA;
    int f[4] = {0, 0, 0, 0};
    if (c->flux.ctr && cudaMemcpy(f, c->flux.ctr, sizeof f, cudaMemcpyDeviceToHost) != cudaSuccess)
        return SLVOF_E_CUDA;
    const int v[SLVOF_NCOUNTERS] = {h[C_SL], h[C_IF], h[C_SLOW], h[C_PL], h[C_ARB], f[0], f[1], f[2]};
    for (int q = 0; q < n && q < SLVOF_NCOUNTERS; ++q) out[q] = v[q];
    return SLVOF_OK;
}

int slvof_set_stream(slvof_ctx* c, void* stream)
{
    if (!c) return SLVOF_E_ARG;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return SLVOF_OK;
}

int slvof_upload_vf(slvof_ctx* c, const double* VF)
{
    TRY(begin(c));
    TRY(h2d(c, c->VF[c->vcur], VF, c->nvf * sizeof(double)));
    c->normals_valid = false;
    return finish(c, false);
}

int slvof_upload_velocity(slvof_ctx* c, const double* uf, const double* vf, const double* wf)
{
    TRY(begin(c));
    TRY(up_velocity(c, uf, vf, wf));
    return finish(c, false);
}

int slvof_upload_band(slvof_ctx* c, const int16_t* band)
{
    TRY(begin(c));
    TRY(h2d(c, c->band[c->bcur], band, c->ncell * sizeof(short)));
    return finish(c, false);
}

int slvof_upload_plic(slvof_ctx* c, const double* nx, const double* ny, const double* nz, const double* D)
{
    TRY(begin(c));
    const size_t b = c->ncell * sizeof(double);
    TRY(h2d(c, c->nx, nx, b));
    TRY(h2d(c, c->ny, ny, b));
    TRY(h2d(c, c->nz, nz, b));
    TRY(h2d(c, c->D, D, b));
    launch_plic_phase(c->m, c->nx, c->ny, c->nz, c->D, c->planes, c->phase, c->nsm, c->stream);
    c->normals_valid = true;
    return finish(c, false);
}

int slvof_download_vf(slvof_ctx* c, double* VF)
{
    TRY(begin(c));
    TRY(d2h(c, VF, c->VF[c->vcur], c->nvf * sizeof(double)));
    return finish(c, false);
}

int slvof_download_normals(slvof_ctx* c, double* nx, double* ny, double* nz)
{
    TRY(begin(c));
    const size_t b = c->ncell * sizeof(double);
    TRY(d2h(c, nx, c->nx, b));
    TRY(d2h(c, ny, c->ny, b));
    TRY(d2h(c, nz, c->nz, b));
    return finish(c, false);
}

int slvof_download_plic(slvof_ctx* c, double* D)
{
    TRY(begin(c));
    TRY(d2h(c, D, c->D, c->ncell * sizeof(double)));
    return finish(c, false);
}

int slvof_download_band(slvof_ctx* c, int16_t* band)
{
    TRY(begin(c));
    TRY(d2h(c, band, c->band[c->bcur], c->ncell * sizeof(short)));
    return finish(c, false);
}

int slvof_vf_ghost_fill(slvof_ctx* c)
{
    TRY(begin(c));
    TRY(st_vf_ghost_inplace(c));
    c->normals_valid = false;
    return finish(c, false);
}

int slvof_compute_normal(slvof_ctx* c)
{
    TRY(begin(c));
    TRY(clear_err(c));
    TRY(st_normals(c));
    return finish(c);
}

int slvof_compute_plic(slvof_ctx* c)
{
    TRY(begin(c));
    TRY(st_plic(c));
    return finish(c, false);
}

int slvof_compute_band(slvof_ctx* c)
{
    TRY(begin(c));
    TRY(st_band(c));
    return finish(c, false);
}

int slvof_transport(slvof_ctx* c, double dt)
{
    TRY(begin(c));
    TRY(clear_err(c));
    TRY(st_transport(c, dt));
    return finish(c);
}

int slvof_step(slvof_ctx* c, double dt, int flags, double* mass)
{
    TRY(begin(c));
    if ((flags & SLVOF_STEP_MASS) && !mass) return fail(c, SLVOF_E_ARG, "mass requested with a null pointer");
    TRY(clear_err(c));
    if (!c->normals_valid) {
        TRY(st_normals(c));
        TRY(st_plic(c));
    }
    TRY(st_transport(c, dt));
    const bool band = (flags & SLVOF_STEP_BAND) != 0;
    int r = band ? st_band_side(c) : 0;
    if (r >= 0) r = st_normals(c);
    if (r >= 0) r = st_plic(c);
    if (r >= 0 && (flags & SLVOF_STEP_MASS)) r = st_mass(c, mass, true);
    if (band) r = join_band(c, r);
    if (r < 0) return r;
    return finish(c);
}

int slvof_mass(slvof_ctx* c, double* mass)
{
    TRY(begin(c));
    if (!mass) return fail(c, SLVOF_E_ARG, "null mass pointer");
    TRY(st_mass(c, mass, false));
    return finish(c, false);
}

int slvof_computeNormal(slvof_ctx* c, double* nx, double* ny, double* nz, const double* VF)
{
    TRY(begin(c));
    TRY(clear_err(c));
    TRY(h2d(c, c->VF[c->vcur], VF, c->nvf * sizeof(double)));
    TRY(st_normals(c));
    const size_t b = c->ncell * sizeof(double);
    TRY(d2h(c, nx, c->nx, b));
    TRY(d2h(c, ny, c->ny, b));
    TRY(d2h(c, nz, c->nz, b));
    return finish(c);
}

int slvof_computePLIC(slvof_ctx* c, double* D, const double* nx, const double* ny, const double* nz, const double* VF)
{
    TRY(begin(c));
    const size_t b = c->ncell * sizeof(double);
    TRY(h2d(c, c->VF[c->vcur], VF, c->nvf * sizeof(double)));
    TRY(h2d(c, c->nx, nx, b));
    TRY(h2d(c, c->ny, ny, b));
    TRY(h2d(c, c->nz, nz, b));
    TRY(st_plic(c));
    TRY(d2h(c, D, c->D, b));
    c->normals_valid = true;
    return finish(c, false);
}

int slvof_computeBand(slvof_ctx* c, int16_t* band, const double* VF)
{
    TRY(begin(c));
    TRY(h2d(c, c->VF[c->vcur], VF, c->nvf * sizeof(double)));
    TRY(h2d(c, c->band[c->bcur], band, c->ncell * sizeof(short)));
    TRY(st_band(c));
    TRY(d2h(c, band, c->band[c->bcur], c->ncell * sizeof(short)));
    c->normals_valid = false;
    return finish(c, false);
}

int slvof_transportSL(slvof_ctx* c, double dt, double* VF, const double* uf, const double* vf, const double* wf,
                      const double* nx, const double* ny, const double* nz, const double* D, const int16_t* band)
{
    TRY(begin(c));
    TRY(clear_err(c));
    const size_t b = c->ncell * sizeof(double);
    TRY(h2d(c, c->VF[c->vcur], VF, c->nvf * sizeof(double)));
    TRY(up_velocity(c, uf, vf, wf));
    TRY(h2d(c, c->nx, nx, b));
    TRY(h2d(c, c->ny, ny, b));
    TRY(h2d(c, c->nz, nz, b));
    TRY(h2d(c, c->D, D, b));
    TRY(h2d(c, c->band[c->bcur], band, c->ncell * sizeof(short)));
    launch_plic_phase(c->m, c->nx, c->ny, c->nz, c->D, c->planes, c->phase, c->nsm, c->stream);
    TRY(st_transport(c, dt));
    TRY(d2h(c, VF, c->VF[c->vcur], c->nvf * sizeof(double)));
    return finish(c);
}

int slvof_step_host(slvof_ctx* c, double dt, int flags, const double* uf, const double* vf, const double* wf,
                    double* VF, double* mass)
{
    const bool defer = (flags & SLVOF_STEP_DEFER) != 0;
    TRY(begin(c, !defer));
    if ((flags & SLVOF_STEP_MASS) && !mass) return fail(c, SLVOF_E_ARG, "mass requested with a null pointer");
    if (!VF) return fail(c, SLVOF_E_ARG, "null host pointer");
    TRY(clear_err(c));
    if (defer) {
        TRY(up_velocity_beside(c, uf, vf, wf));
    } else {
        TRY(up_velocity(c, uf, vf, wf));
        if (!c->normals_valid) {
            TRY(st_normals(c));
            TRY(st_plic(c));
        }
    }
    TRY(st_transport(c, dt));
    /* the new VF is final here (normals, PLIC, band and mass only read it): it goes to the host
     * on the copy stream while they run */
    CK(cudaEventRecord(c->ev_state, c->stream));
    CK(cudaStreamWaitEvent(c->copy_stream, c->ev_state, 0));
    cudaError_t ce = cudaMemcpyAsync(VF, c->VF[c->vcur], c->nvf * sizeof(double), cudaMemcpyDeviceToHost,
                                     c->copy_stream);
    if (ce == cudaSuccess) ce = cudaEventRecord(c->ev_copied, c->copy_stream);
    int r = 0;
    const bool band = (flags & SLVOF_STEP_BAND) != 0;
    if (ce == cudaSuccess && defer) {
        /* the next call builds this state's normals, PLIC and band beside its upload */
        if (flags & SLVOF_STEP_MASS) r = st_mass(c, mass, false);
        c->deferred = true;
        c->deferred_band = band;
        ce = cudaStreamWaitEvent(c->stream, c->ev_copied, 0);
    } else if (ce == cudaSuccess) {
        r = band ? st_band_side(c) : 0;
        if (r >= 0) r = st_normals(c);
        if (r >= 0) r = st_plic(c);
        if (r >= 0 && (flags & SLVOF_STEP_MASS)) r = st_mass(c, mass, true);
        if (band) r = join_band(c, r);
        ce = cudaStreamWaitEvent(c->stream, c->ev_copied, 0);
    }
    if (r < 0 || ce != cudaSuccess) {
        cudaStreamSynchronize(c->copy_stream); /* the host buffer is the caller's again on return */
        return r < 0 ? r : fail(c, SLVOF_E_CUDA, std::string("VF download: ") + cudaGetErrorString(ce));
    }
    return finish(c);
}

int slvof_case_vf_spheres(slvof_ctx* c, const double* centres, const double* radii, int n, int nF, int dims)
{
    if (!c || !centres || !radii || n < 1 || nF < 1 || nF > 64 || (dims != 2 && dims != 3)) return SLVOF_E_ARG;
    TRY(begin(c));
    const int npts = dims == 3 ? nF * nF * nF : nF * nF;
    if (c->table_n < npts + 1) {
        if (c->table) cudaFree(c->table);
        c->table = nullptr;
        CK(cudaMalloc(&c->table, (npts + 1) * sizeof(double)));
        c->table_n = npts + 1;
    }
    if (c->spheres_n < n) {
        if (c->spheres) cudaFree(c->spheres);
        c->spheres = nullptr;
        CK(cudaMalloc(&c->spheres, 4 * n * sizeof(double)));
        c->spheres_n = n;
    }
    /* running sum VF += 1/nF^dims, as the reference accumulates it */
    std::vector<double> tab(npts + 1);
    const double sub = 1.0 / (double)npts;
    double s = 0.0;
    tab[0] = 0.0;
    for (int q = 1; q <= npts; ++q) { s = s + sub; tab[q] = s; }
    CK(cudaMemcpyAsync(c->table, tab.data(), (npts + 1) * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->spheres, centres, 3 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->spheres + 3 * n, radii, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemsetAsync(c->VF[c->vcur], 0, c->nvf * sizeof(double), c->stream));
    launch_case_spheres(c->m, c->spheres, c->spheres + 3 * n, n, nF, dims, c->table, c->VF[c->vcur], c->nsm, c->stream);
    CK(cudaStreamSynchronize(c->stream)); /* host vectors go out of scope */
    TRY(st_vf_ghost_inplace(c));
    c->normals_valid = false;
    return finish(c, false);
}

int slvof_case_deformation3d(slvof_ctx* c, double t, double T)
{
    TRY(begin(c));
    launch_case_deformation3d(c->m, t, T, c->uf, c->vf, c->wf, c->nsm, c->stream);
    to_float_velocity(c);
    return finish(c, false);
}

/* ---- momentum ---------------------------------------------------------------------------- */
int slvof_upload_cell_velocity(slvof_ctx* c, const double* u, const double* v, const double* w)
{
    TRY(begin(c));
    TRY(mom_alloc(c));
    const size_t b = c->ncell * sizeof(double);
    TRY(h2d(c, c->cu, u, b));
    TRY(h2d(c, c->cv, v, b));
    TRY(h2d(c, c->cw, w, b));
    return finish(c, false);
}

int slvof_download_momentum(slvof_ctx* c, double* us, double* vs, double* ws)
{
    TRY(begin(c));
    TRY(mom_alloc(c));
    const size_t b = c->ncell * sizeof(double);
    TRY(d2h(c, us, c->us, b));
    TRY(d2h(c, vs, c->vs, b));
    TRY(d2h(c, ws, c->ws, b));
    return finish(c, false);
}

int slvof_transport_momentum(slvof_ctx* c, double dt)
{
    TRY(begin(c));
    TRY(mom_alloc(c));
    TRY(clear_err(c));
    TRY(st_transport_mom(c, dt));
    return finish(c);
}

int slvof_transportSL_momentum(slvof_ctx* c, double dt, double* VF, const double* uf, const double* vf,
                               const double* wf, const double* nx, const double* ny, const double* nz, const double* D,
                               const int16_t* band, const double* u, const double* v, const double* w, double* us,
                               double* vs, double* ws)
{
    TRY(begin(c));
    TRY(mom_alloc(c));
    TRY(clear_err(c));
    const size_t b = c->ncell * sizeof(double);
    TRY(h2d(c, c->VF[c->vcur], VF, c->nvf * sizeof(double)));
    TRY(h2d(c, c->uf, uf, b));
    TRY(h2d(c, c->vf, vf, b));
    TRY(h2d(c, c->wf, wf, b));
    TRY(h2d(c, c->nx, nx, b));
    TRY(h2d(c, c->ny, ny, b));
    TRY(h2d(c, c->nz, nz, b));
    TRY(h2d(c, c->D, D, b));
    TRY(h2d(c, c->band[c->bcur], band, c->ncell * sizeof(short)));
    TRY(h2d(c, c->cu, u, b));
    TRY(h2d(c, c->cv, v, b));
    TRY(h2d(c, c->cw, w, b));
    /* phase codes of the uploaded planes */
    launch_plic_phase(c->m, c->nx, c->ny, c->nz, c->D, c->planes, c->phase, c->nsm, c->stream);
    TRY(st_transport_mom(c, dt));
    TRY(d2h(c, VF, c->VF[c->vcur], c->nvf * sizeof(double)));
    TRY(d2h(c, us, c->us, b));
    TRY(d2h(c, vs, c->vs, b));
    TRY(d2h(c, ws, c->ws, b));
    return finish(c);
}

/* ---- divergence and the pressure operator ----------------------------------------------- */
namespace {
enum { PR_U = 0, PR_V, PR_W, PR_P, PR_DX, PR_DY, PR_DZ, PR_GX, PR_GY, PR_GZ, PR_OUT };

int pr_alloc(slvof_ctx* c)
{
    if (c->pr_band) return 0;
    for (double*& b : c->pr)
        if (cudaMalloc((void**)&b, c->ncell * sizeof(double)) != cudaSuccess ||
            cudaMemset(b, 0, c->ncell * sizeof(double)) != cudaSuccess)
            return fail(c, SLVOF_E_NOMEM, "divergence buffers");
    if (cudaMalloc((void**)&c->pr_band, c->ncell * sizeof(short)) != cudaSuccess)
        return fail(c, SLVOF_E_NOMEM, "divergence buffers");
    return 0;
}

int scheme_ok(slvof_ctx* c, int scheme)
{
    return (scheme == SLVOF_PRESSURE_SEMI_LAGRANGIAN || scheme == SLVOF_PRESSURE_FINITE_DIFFERENCE)
               ? 0
               : fail(c, SLVOF_E_ARG, "scheme: SLVOF_PRESSURE_SEMI_LAGRANGIAN or SLVOF_PRESSURE_FINITE_DIFFERENCE");
}
} // namespace

int slvof_divergence(slvof_ctx* c, double dt, int scheme, double* divg, const double* uf, const double* vf,
                     const double* wf, const int16_t* band)
{
    TRY(begin(c));
    TRY(scheme_ok(c, scheme));
    TRY(pr_alloc(c));
    const size_t b = c->ncell * sizeof(double);
    TRY(h2d(c, c->pr[PR_U], uf, b));
    TRY(h2d(c, c->pr[PR_V], vf, b));
    TRY(h2d(c, c->pr[PR_W], wf, b));
    TRY(h2d(c, c->pr_band, band, c->ncell * sizeof(short)));
    launch_divergence64(c->m, dt, scheme == SLVOF_PRESSURE_SEMI_LAGRANGIAN, c->pr[PR_U], c->pr[PR_V], c->pr[PR_W], c->pr_band, c->pr[PR_OUT], c->nsm,
                        c->stream);
    TRY(d2h(c, divg, c->pr[PR_OUT], b));
    return finish(c, false);
}

int slvof_divergence_device(slvof_ctx* c, double dt, int scheme, double* d_divg, const double* d_uf,
                            const double* d_vf, const double* d_wf, const int16_t* d_band)
{
    TRY(begin(c));
    TRY(scheme_ok(c, scheme));
    if (!d_divg || !d_uf || !d_vf || !d_wf || !d_band) return fail(c, SLVOF_E_ARG, "null device pointer");
    launch_divergence64(c->m, dt, scheme == SLVOF_PRESSURE_SEMI_LAGRANGIAN, d_uf, d_vf, d_wf, (const short*)d_band, d_divg, c->nsm, c->stream);
    return finish(c, false);
}

int slvof_A(slvof_ctx* c, double dt, int scheme, double* LHS, double* P, const double* uf, const double* vf,
            const double* wf, const double* denx, const double* deny, const double* denz, const int16_t* band)
{
    TRY(begin(c));
    TRY(scheme_ok(c, scheme));
    TRY(pr_alloc(c));
    const size_t b = c->ncell * sizeof(double);
    const double* in[7] = {uf, vf, wf, P, denx, deny, denz};
    for (int q = 0; q < 7; ++q) TRY(h2d(c, c->pr[q], in[q], b));
    TRY(h2d(c, c->pr_band, band, c->ncell * sizeof(short)));
    launch_pressure_A64(c->m, dt, scheme == SLVOF_PRESSURE_SEMI_LAGRANGIAN, c->pr[PR_OUT], c->pr[PR_P], c->pr[PR_U], c->pr[PR_V], c->pr[PR_W],
                        c->pr[PR_DX], c->pr[PR_DY], c->pr[PR_DZ], c->pr_band, c->pr[PR_GX], c->pr[PR_GY],
                        c->pr[PR_GZ], c->nsm, c->stream);
    TRY(d2h(c, LHS, c->pr[PR_OUT], b));
    TRY(d2h(c, P, c->pr[PR_P], b));
    return finish(c, false);
}

int slvof_A_device(slvof_ctx* c, double dt, int scheme, double* d_LHS, double* d_P, const double* d_uf,
                   const double* d_vf, const double* d_wf, const double* d_denx, const double* d_deny,
                   const double* d_denz, const int16_t* d_band)
{
    TRY(begin(c));
    TRY(scheme_ok(c, scheme));
    if (!d_LHS || !d_P || !d_uf || !d_vf || !d_wf || !d_denx || !d_deny || !d_denz || !d_band)
        return fail(c, SLVOF_E_ARG, "null device pointer");
    TRY(pr_alloc(c));
    launch_pressure_A64(c->m, dt, scheme == SLVOF_PRESSURE_SEMI_LAGRANGIAN, d_LHS, d_P, d_uf, d_vf, d_wf, d_denx, d_deny, d_denz,
                        (const short*)d_band, c->pr[PR_GX], c->pr[PR_GY], c->pr[PR_GZ], c->nsm, c->stream);
    return finish(c, false);
}

/* ---- curvature and face properties ------------------------------------------------------- */
int slvof_computeCurvature(slvof_ctx* c, double* Curve, const double* VF, const double* nx, const double* ny,
                           const double* nz)
{
    TRY(begin(c));
    TRY(pr_alloc(c));
    const size_t b = c->ncell * sizeof(double);
    double* vf = c->VF[1 - c->vcur]; /* the step's scratch copy */
    TRY(h2d(c, vf, VF, c->nvf * sizeof(double)));
    TRY(h2d(c, c->pr[0], nx, b));
    TRY(h2d(c, c->pr[1], ny, b));
    TRY(h2d(c, c->pr[2], nz, b));
    launch_curvature64(c->m, vf, c->pr[0], c->pr[1], c->pr[2], c->pr[PR_OUT], c->nsm, c->stream);
    TRY(d2h(c, Curve, c->pr[PR_OUT], b));
    return finish(c, false);
}

int slvof_compute_curvature_device(slvof_ctx* c, double* d_Curve)
{
    TRY(begin(c));
    if (!d_Curve) return fail(c, SLVOF_E_ARG, "null device pointer");
    if (!c->normals_valid) return fail(c, SLVOF_E_ARG, "normals of the current VF are not computed (slvof_prepare)");
    launch_curvature64(c->m, c->VF[c->vcur], c->nx, c->ny, c->nz, d_Curve, c->nsm, c->stream);
    return finish(c, false);
}

int slvof_computeProps(slvof_ctx* c, double rho_liq, double rho_gas, double mu_liq, double mu_gas, double* denx,
                       double* deny, double* denz, double* viscx, double* viscy, double* viscz, const double* VF)
{
    TRY(begin(c));
    const bool visc = viscx != nullptr;
    if (!denx || !deny || !denz || (visc && (!viscy || !viscz)) || (!visc && (viscy || viscz)))
        return fail(c, SLVOF_E_ARG, "density arrays, and all three or none of the viscosity arrays");
    TRY(pr_alloc(c));
    const size_t b = c->ncell * sizeof(double);
    double* vf = c->VF[1 - c->vcur];
    TRY(h2d(c, vf, VF, c->nvf * sizeof(double)));
    launch_props64(c->m, vf, rho_liq, rho_gas, mu_liq, mu_gas, c->pr[0], c->pr[1], c->pr[2], visc ? c->pr[3] : nullptr,
                   visc ? c->pr[4] : nullptr, visc ? c->pr[5] : nullptr, c->nsm, c->stream);
    double* out[6] = {denx, deny, denz, viscx, viscy, viscz};
    for (int q = 0; q < (visc ? 6 : 3); ++q) TRY(d2h(c, out[q], c->pr[q], b));
    return finish(c, false);
}

/* ---- reverse pass ----------------------------------------------------------------------- */
namespace {
int adj_alloc(slvof_ctx* c)
{
    if (c->gvf[0]) return 0;
    auto alloc = [&](double** p, long n) {
        return cudaMalloc((void**)p, n * sizeof(double)) == cudaSuccess &&
               cudaMemset(*p, 0, n * sizeof(double)) == cudaSuccess;
    };
    const long interior = (long)c->m.N[0] * c->m.N[1] * c->m.N[2];
    bool ok = alloc(&c->gvf[0], c->nvf) && alloc(&c->gvf[1], c->nvf) && alloc(&c->gfold, c->nvf) &&
              alloc(&c->gD, c->ncell) && alloc(&c->gDf, c->ncell) && alloc(&c->guf, c->ncell) &&
              alloc(&c->gvf_, c->ncell) && alloc(&c->gwf, c->ncell);
    for (int q = 0; q < 3 && ok; ++q) ok = alloc(&c->gn[q], c->ncell) && alloc(&c->gnf[q], c->ncell);
    ok = ok && cudaMalloc((void**)&c->list_adj, interior * sizeof(int)) == cudaSuccess;
    if (c->precision == SLVOF_MIXED) {
        for (int q = 0; q < 3 && ok; ++q) ok = alloc(&c->gvtx[q], c->ncell);
        ok = ok && cudaMalloc((void**)&c->cinfo, interior * sizeof(float2)) == cudaSuccess;
        for (int q = 0; q < 3 && ok; ++q)
            ok = cudaMalloc((void**)&c->gvel32[q], c->ncell * sizeof(float)) == cudaSuccess &&
                 cudaMemset(c->gvel32[q], 0, c->ncell * sizeof(float)) == cudaSuccess;
    }
    if (!ok) return fail(c, SLVOF_E_NOMEM, "reverse-pass buffers");
    return 0;
}
} // namespace

int slvof_prepare(slvof_ctx* c)
{
    TRY(begin(c));
    TRY(clear_err(c));
    TRY(st_vf_ghost_inplace(c));
    TRY(st_normals(c));
    TRY(st_plic(c));
    TRY(st_band(c));
    return finish(c);
}

int slvof_copy_vf_device(slvof_ctx* c, double* d_dst)
{
    TRY(begin(c));
    if (!d_dst) return fail(c, SLVOF_E_ARG, "null device pointer");
    CK(cudaMemcpyAsync(d_dst, c->VF[c->vcur], c->nvf * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    return finish(c, false);
}

int slvof_load_vf_device(slvof_ctx* c, const double* d_src)
{
    TRY(begin(c));
    if (!d_src) return fail(c, SLVOF_E_ARG, "null device pointer");
    CK(cudaMemcpyAsync(c->VF[c->vcur], d_src, c->nvf * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    c->normals_valid = false;
    return finish(c, false);
}

int slvof_adjoint_set_vf(slvof_ctx* c, const double* gVF)
{
    TRY(begin(c));
    TRY(adj_alloc(c));
    if (gVF) TRY(h2d(c, c->gvf[0], gVF, c->nvf * sizeof(double)));
    else CK(cudaMemsetAsync(c->gvf[0], 0, c->nvf * sizeof(double), c->stream));
    return finish(c, false);
}

int slvof_adjoint_get(slvof_ctx* c, double* gVF, double* guf, double* gvf, double* gwf)
{
    TRY(begin(c));
    TRY(adj_alloc(c));
    const size_t b = c->ncell * sizeof(double);
    if (gVF) TRY(d2h(c, gVF, c->gvf[0], c->nvf * sizeof(double)));
    if (guf) TRY(d2h(c, guf, c->guf, b));
    if (gvf) TRY(d2h(c, gvf, c->gvf_, b));
    if (gwf) TRY(d2h(c, gwf, c->gwf, b));
    return finish(c, false);
}

int slvof_adjoint_zero_velocity(slvof_ctx* c)
{
    TRY(begin(c));
    TRY(adj_alloc(c));
    const size_t b = c->ncell * sizeof(double);
    CK(cudaMemsetAsync(c->guf, 0, b, c->stream));
    CK(cudaMemsetAsync(c->gvf_, 0, b, c->stream));
    CK(cudaMemsetAsync(c->gwf, 0, b, c->stream));
    return finish(c, false);
}

int slvof_adjoint_fold(slvof_ctx* c)
{
    TRY(begin(c));
    TRY(adj_alloc(c));
    launch_adjoint_fold_vf(c->m, c->gvf[0], c->gvf[1], c->nsm, c->stream);
    std::swap(c->gvf[0], c->gvf[1]);
    return finish(c, false);
}

namespace {
/* Reverse of the mixed-precision step: pre-images of the band cells again (k_sl32_pre, which
 * also lists the cells the clip needs), VFnew given or recomputed by the clip, then the
 * boundary-form SL reverse, computeDist's reverse from the plane polygons, and the FP64 folds
 * and ELVIRA reverse shared with the FP64 path. */
int adjoint_step32(slvof_ctx* c, double dt, const double* d_next, AdjBuffers& b)
{
    const int o = 1 - c->vcur;
    CK(cudaMemsetAsync(c->ctr + C_SL, 0, sizeof(int), c->stream));
    CK(cudaMemsetAsync(c->ctr + C_SLW, 0, sizeof(int), c->stream));
    launch_sl_classify(c->m, c->band[c->bcur], c->VF[c->vcur], c->VF[o], c->list_sl, c->ctr + C_SL, c->nsm, c->stream);
    if (!d_next) {
        /* the step's result as the forward computes it */
        st_sl32(c, dt, o);
        d_next = c->VF[o];
    }
    /* the band cells' FP32 pre-images and the list of those the reverse clips (VF untouched) */
    CK(cudaMemsetAsync(c->ctr + C_SLW, 0, sizeof(int), c->stream));
    CK(cudaMemsetAsync(c->ctr + C_SLOW, 0, 2 * sizeof(int), c->stream)); /* clip count, clip work */
    launch_sl32_pre(c->m, dt, nullptr, c->uf32, c->vf32, c->wf32, c->planes, c->phase, c->list_sl, c->ctr + C_SL,
                    c->ctr + C_SLW, c->slow_cells, c->slow_verts, c->ctr + C_SLOW, c->ctr + C_ERR, c->nsm, c->stream);
    launch_adjoint32_sl(c->m, dt, d_next, c->uf32, c->vf32, c->wf32, c->planes, c->phase, c->slow_cells,
                        c->slow_verts, c->ctr + C_SLOW, c->cinfo, c->gvtx[0], c->gvtx[1], c->gvtx[2], c->gvel32, b,
                        c->ctr + C_ERR, c->nsm, c->stream);
    launch_adjoint_fold_cell(c->m, b.gD, b.gDf, c->nsm, c->stream);
    launch_adjoint32_dist(c->m, c->VF[c->vcur], c->planes, b, c->nsm, c->stream);
    for (int q = 0; q < 3; ++q) launch_adjoint_fold_cell(c->m, b.gn[q], b.gnf[q], c->nsm, c->stream);
    launch_adjoint32_elvira(c->m, c->VF[c->vcur], c->cand, b, c->nsm, c->stream);
    return 0;
}

int adjoint_step(slvof_ctx* c, double dt, const double* d_next)
{
    TRY(begin(c));
    TRY(adj_alloc(c));
    if (!c->normals_valid) return fail(c, SLVOF_E_ARG, "normals/PLIC/band of the current VF are not computed (slvof_prepare)");
    TRY(clear_err(c));
    AdjBuffers b{};
    b.gin = c->gvf[0];
    b.gfold = c->gfold;
    b.gout = c->gvf[1];
    for (int q = 0; q < 3; ++q) { b.gn[q] = c->gn[q]; b.gnf[q] = c->gnf[q]; }
    b.gD = c->gD;
    b.gDf = c->gDf;
    b.guf = c->guf;
    b.gvf = c->gvf_;
    b.gwf = c->gwf;
    /* head: fold, pass-through of cells outside the band, band list; its count sizes the
     * pre-image records, the pre-pass's count the per-tet records */
    launch_adjoint_head(c->m, c->band[c->bcur], b, c->list_adj, c->ctr + C_ADJ, c->ctr + C_ADJ2, c->nsm, c->stream);
    /* the finite-difference scheme's update runs the FP64 clip in either precision (on the
     * mixed context's FP64 winner normals and plane constants), and so does its reverse */
    if (c->m.fd) {
        launch_adjoint_fd(c->m, dt, c->VF[c->vcur], c->uf, c->vf, c->wf, c->nx, c->ny, c->nz, c->D, c->cand, c->phase,
                          b, c->list_adj, c->ctr + C_ADJ, c->ctr + C_ERR, c->nsm, c->stream);
        std::swap(c->gvf[0], c->gvf[1]);
        return finish(c);
    }
    if (c->precision == SLVOF_MIXED) {
        TRY(adjoint_step32(c, dt, d_next, b));
        std::swap(c->gvf[0], c->gvf[1]);
        return finish(c);
    }
    int n1 = 0, n2 = 0;
    CK(cudaMemcpyAsync(&n1, c->ctr + C_ADJ, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (n1 > c->adj_cells_cap) {
        if (c->adj_cells) cudaFree(c->adj_cells);
        c->adj_cells = nullptr;
        c->adj_cells_cap = 0;
        const long cap = n1 + n1 / 4 + 1024;
        CK(cudaMalloc((void**)&c->adj_cells, cap * sizeof(AdjCell)));
        c->adj_cells_cap = cap;
    }
    b.cells = c->adj_cells;
    launch_adjoint_pre(c->m, dt, c->uf, c->vf, c->wf, c->nx, c->ny, c->nz, c->D, c->phase, b, c->list_adj,
                       c->ctr + C_ADJ, c->ctr + C_ADJ2, c->ctr + C_ERR, c->nsm, c->stream);
    CK(cudaMemcpyAsync(&n2, c->ctr + C_ADJ2, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    const long ntet = tess_ntets(c->m.tess);
    if (ntet * n2 > c->adj_tets_cap) {
        if (c->adj_tets) cudaFree(c->adj_tets);
        c->adj_tets = nullptr;
        c->adj_tets_cap = 0;
        const long cap = ntet * (n2 + n2 / 4 + 1024);
        CK(cudaMalloc((void**)&c->adj_tets, cap * sizeof(AdjTet)));
        c->adj_tets_cap = cap;
    }
    b.tets = c->adj_tets;
    launch_adjoint_tail(c->m, dt, c->VF[c->vcur], c->uf, c->vf, c->wf, c->nx, c->ny, c->nz, c->D, c->cand, c->phase, b,
                        c->ctr + C_ADJ2, c->ctr + C_ERR, c->nsm, c->stream);
    std::swap(c->gvf[0], c->gvf[1]);
    return finish(c);
}
} // namespace

int slvof_adjoint_step(slvof_ctx* c, double dt) { return adjoint_step(c, dt, nullptr); }

int slvof_adjoint_step_next(slvof_ctx* c, double dt, const double* d_VFnext) { return adjoint_step(c, dt, d_VFnext); }

} // extern "C"
