/* slvof_kernels.h — host-side launchers of the SL-VOF kernels (internal to the library). */
#pragma once

#include <cuda_runtime.h>

#include "slvof_dev.cuh"

namespace slvof {

/* k_common.cu */
void launch_vf_ghost(const DevMesh& m, const double* VFin, double* VFout, int nsm, cudaStream_t s);
/* pure-cell normals, interface list and exact mass partials: pure_blocks(m) pairs of int64 */
long pure_blocks(long nx, long ny, long nz);
void launch_elvira_pure(const DevMesh& m, const double* VF, double* nx, double* ny, double* nz, int* list, int* count,
                        long long* partials, cudaStream_t s);
void launch_normal_ghost(const DevMesh& m, double* nx, double* ny, double* nz, int nsm, cudaStream_t s);
void launch_mass_final(const long long* partials, long nblocks, double cellvol, double* out, cudaStream_t s);
void launch_band_first(const DevMesh& m, const double* VF, short* bout, int* errw, int nsm, cudaStream_t s);
void launch_band_ghost(const DevMesh& m, const short* bin, short* bout, bool neumann, int nsm, cudaStream_t s);
void launch_band_sweep(const DevMesh& m, const short* bin, short* bout, int n, int nsm, cudaStream_t s);
void launch_sl_classify(const DevMesh& m, const short* band, const double* VFin, double* VFout, int* list, int* count,
                        int nsm, cudaStream_t s);
void launch_to_float(const double* a, float* b, long n, double scale, int nsm, cudaStream_t s);
void launch_case_spheres(const DevMesh& m, const double* cen, const double* rad, int n, int nF, int dims,
                         const double* table, double* VF, int nsm, cudaStream_t s);
void launch_case_deformation3d(const DevMesh& m, double t, double T, double* uf, double* vf, double* wf, int nsm,
                               cudaStream_t s);

/* k_fp64.cu */
void launch_elvira_iface64(const DevMesh& m, const double* VF, double* nx, double* ny, double* nz, const int* list,
                           const int* count, int* work, signed char* cand, int* errw, int nsm, cudaStream_t s);
/* newton_root: the mixed path's plane constants (FP32 inverse + FP64 Newton, k_elvira_mixed.cu);
 * otherwise computeAlpha's closed form, bit-identical to the CPU restatement */
void launch_plic64(const DevMesh& m, const double* VF, const double* nx, const double* ny, const double* nz, double* D,
                   float4* planes, signed char* phase, int* list, int* count, bool newton_root, int nsm, cudaStream_t s);
void launch_plic_iface_newton(const DevMesh& m, const double* VF, const double* nx, const double* ny, const double* nz,
                              double* D, float4* planes, signed char* phase, const int* list, const int* count,
                              int nsm, cudaStream_t s);
void launch_sl64(const DevMesh& m, double dt, const double* VFin, double* VFout, const double* uf, const double* vf,
                 const double* wf, const double* nx, const double* ny, const double* nz, const double* D,
                 const signed char* phase, const int* list, const int* count, int* work, int* errw, int nsm,
                 cudaStream_t s);

/* phase codes and mixed-path planes of uploaded normals and D */
void launch_plic_phase(const DevMesh& m, const double* nx, const double* ny, const double* nz, double* D,
                       float4* planes, signed char* phase, int nsm, cudaStream_t s);
/* SL update with the momentum of transport! (us, vs, ws of every interior cell) */
void launch_sl64_momentum(const DevMesh& m, double dt, double* VFout, const double* uf, const double* vf,
                          const double* wf, const double* nx, const double* ny, const double* nz, const double* D,
                          const signed char* phase, const short* band, const double* u, const double* v,
                          const double* w, double rho_liq, double rho_gas, double* us, double* vs, double* ws,
                          const int* list, const int* count, int* work, int* errw, int nsm, cudaStream_t s);

/* k_mixed.cu, k_elvira_mixed.cu */
/* the mixed path's SL update in flux form: node displacements and per-direction face
 * (volume, liquid) arrays indexed like the cell arrays, the node / face / clip-face lists
 * (capacity: cells, 3 x cells, 3 x cells) and four counters */
struct FluxLaunch {
    double* nd[3];
    double2* fvf[3];
    unsigned* nodes;
    unsigned* faces;
    unsigned* clip;
    float4* fapex[3]; /* pressure_scheme "finite-difference": each face's correction apex */
    int* ctr;
};
void launch_sl32_flux(const DevMesh& m, double dt, const double* VFin, double* VFout, const float* uf32,
                      const float* vf32, const float* wf32, const double* uf, const double* vf, const double* wf,
                      const float4* planes, const short* band, const int* list, const int* count,
                      const FluxLaunch& L, int* slow_cells, float4* slow_verts, int* slow_count, int* work2,
                      int* errw, int nsm, cudaStream_t s);
/* mixed ELVIRA: FP32 scoring (warp per cell), FP64 arbitration of the near-ties listed in arb
 * (n_arb zeroed by the caller; capacity: the interface count), FP64 winner normals */
void launch_elvira_iface32(const DevMesh& m, const double* VF, double* nx, double* ny, double* nz, const int* list,
                           const int* count, int* work, int* n_arb, int2* arb, signed char* cand, int* errw, int nsm,
                           cudaStream_t s);

/* k_adj64.cu: reverse pass of one FP64 step (see adj64.cuh) */
struct AdjCell {  /* a band cell whose pre-image clips: pre-image points and seed */
    double vt[15][3]; /* vertices, then the mean points of 24_tets */
    int vind[15][3];
    double tetsign, volu, g;
    int L;
};
struct AdjTet {   /* one tet's clip: vol, vLiq, s * d(vLiq)/d(vertices), leaf kinds */
    double rv, rl;
    double g[4][3];
    int kinds;
};
struct AdjBuffers {
    const double* gin;  /* dL/dVF^{n+1}, VF array */
    double* gfold;      /* gin with ghost copies folded onto their sources */
    double* gout;       /* dL/dVF^n, VF array */
    double *gn[3], *gD; /* dL/d(border-updated normal, D) */
    double *gnf[3], *gDf; /* the same folded onto the border copies' sources */
    double *guf, *gvf, *gwf; /* dL/d(face velocities), accumulated */
    AdjCell* cells;          /* capacity: the band count of the step (head's count) */
    AdjTet* tets;            /* capacity: tets per cell x the clip count (pre's count2) */
};
/* The reverse of one step in three launches; the host reads `count` after the head and
 * `count2` after the pre-pass to size cells and tets. */
void launch_adjoint_head(const DevMesh& m, const short* band, const AdjBuffers& b, int* list, int* count, int* count2,
                         int nsm, cudaStream_t s);
void launch_adjoint_pre(const DevMesh& m, double dt, const double* uf, const double* vf, const double* wf,
                        const double* nx, const double* ny, const double* nz, const double* D, const signed char* phase,
                        const AdjBuffers& b, const int* list, const int* count, int* count2, int* errw, int nsm,
                        cudaStream_t s);
void launch_adjoint_tail(const DevMesh& m, double dt, const double* VF, const double* uf, const double* vf,
                         const double* wf, const double* nx, const double* ny, const double* nz, const double* D,
                         const signed char* cand, const signed char* phase, const AdjBuffers& b, const int* count2,
                         int* errw, int nsm, cudaStream_t s);
/* pressure_scheme "finite-difference" (FP64): the band cells' reverse with the flux-correction
 * tets, one thread per cell of the head's list, then the same computeDist and ELVIRA reverse. */
void launch_adjoint_fd(const DevMesh& m, double dt, const double* VF, const double* uf, const double* vf,
                       const double* wf, const double* nx, const double* ny, const double* nz, const double* D,
                       const signed char* cand, const signed char* phase, const AdjBuffers& b, const int* list,
                       const int* count, int* errw, int nsm, cudaStream_t s);
void launch_adjoint_fold_vf(const DevMesh& m, const double* gin, double* gout, int nsm, cudaStream_t s);
void launch_adjoint_fold_cell(const DevMesh& m, const double* gin, double* gout, int nsm, cudaStream_t s);
void launch_adjoint_elvira(const DevMesh& m, const double* VF, const signed char* cand, const AdjBuffers& b, int nsm,
                           cudaStream_t s);
/* Reverse of the mixed-precision SL update (k_adj32.cu): the clip list and pre-image vertices
 * of k_sl32_pre, VFnew of the step, dL/d(grid vertices) and per-step face-velocity sums (FP32)
 * as scratch (zero on entry, left zero). */
void launch_adjoint32_sl(const DevMesh& m, double dt, const double* VFnext, const float* uf32, const float* vf32,
                         const float* wf32, const float4* planes, const signed char* phase, const int* cells,
                         const float4* verts, const int* count, float2* cinfo, double* gvx, double* gvy, double* gvz,
                         float* const* gvel32, const AdjBuffers& b, int* errw, int nsm, cudaStream_t s);
void launch_adjoint32_elvira(const DevMesh& m, const double* VF, const signed char* cand, const AdjBuffers& b,
                             int nsm, cudaStream_t s);
void launch_adjoint32_dist(const DevMesh& m, const double* VF, const float4* planes, const AdjBuffers& b, int nsm,
                           cudaStream_t s);
/* compute_curvature! on the interior (Curve zeroed first) and compute_props! / compute_dens!
 * (visc* null) on every cell (k_common.cu). */
void launch_curvature64(const DevMesh& m, const double* VF, const double* nx, const double* ny, const double* nz,
                        double* Curve, int nsm, cudaStream_t s);
void launch_props64(const DevMesh& m, const double* VF, double rho_liq, double rho_gas, double mu_liq, double mu_gas,
                    double* denx, double* deny, double* denz, double* viscx, double* viscy, double* viscz, int nsm,
                    cudaStream_t s);
/* divergence! / divg_cell and A! (k_fp64.cu); sl: pressure_scheme "semi-lagrangian".  A!
 * fills P's ghosts in place and uses gx, gy, gz as its corrected face velocities. */
void launch_divergence64(const DevMesh& m, double dt, int sl, const double* uf, const double* vf, const double* wf,
                         const short* band, double* divg, int nsm, cudaStream_t s);
void launch_pressure_A64(const DevMesh& m, double dt, int sl, double* LHS, double* P, const double* uf,
                         const double* vf, const double* wf, const double* denx, const double* deny,
                         const double* denz, const short* band, double* gx, double* gy, double* gz, int nsm,
                         cudaStream_t s);
void launch_sl32_pre(const DevMesh& m, double dt, double* VFout, const float* uf, const float* vf, const float* wf,
                     const float4* planes, const signed char* phase, const int* list, const int* count, int* work,
                     int* slow_cells, float4* slow_verts, int* slow_count, int* errw, int nsm, cudaStream_t s);
void launch_sl32_clip(const DevMesh& m, double* VFout, const float4* planes, int* work2, const int* slow_cells,
                      const float4* slow_verts, const int* slow_count, int* errw, int nsm, cudaStream_t s);

} // namespace slvof
