/*
 * slvof.h — C ABI of the GB300 (sm_103a) SL-VOF transport library.
 *
 * Drop-in for Mist.jl's semi-Lagrangian geometric VOF transport path: the Julia host keeps
 * its OffsetArrays and calls these entry points through ccall with pointers to the arrays'
 * parents (column-major, i fastest).  Extents follow src/Tools.jl:136-191:
 *   cell arrays (uf, vf, wf, nx, ny, nz, D, band): (Nx+2g) x (Ny+2g) x (Nz+2g), g = nghost;
 *   VF: (Nx+2g+6) x (Ny+2g+6) x (Nz+2g+6)  (three extra ghost layers, src/Tools.jl:144).
 * Reals are IEEE double, band is int16.  One MPI rank: the library fills ghost cells itself
 * with the reference's single-rank semantics (Neumann! src/Tools.jl:4-18, update_borders!
 * src/Parallel.jl:63-143, periodic directions wrapping onto the same rank).
 *
 * Return codes: SLVOF_OK, a positive OR of SLVOF_DEV_* bits raised by a kernel (the result
 * of that call is still written), or a negative SLVOF_E_* host error.  No call aborts or
 * throws across the ABI; slvof_last_error() gives a message for the last nonzero status.
 * Calls on one context are serialised by the caller; distinct contexts are independent.
 */
#ifndef SLVOF_H
#define SLVOF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SLVOF_OK 0
/* device-side error bits (kernels record them instead of trapping) */
#define SLVOF_DEV_INDEX 1  /* a pre-image vertex left the ghost region (pt2index!, src/Tools.jl:424-434) */
#define SLVOF_DEV_DEPTH 2  /* cutTet recursion deeper than the clip stack (src/VFgeom.jl:713-900) */
#define SLVOF_DEV_NAN 4    /* NaN signed distance in a cut (reference: InexactError in d2case) */
#define SLVOF_DEV_VOLUME 8 /* non-positive or non-finite pre-image volume (src/Transport.jl:145) */
#define SLVOF_DEV_WAIT 16  /* a kernel's bounded wait on its own bulk copies ran out (its output is incomplete) */
/* host errors */
#define SLVOF_E_ARG (-1)
#define SLVOF_E_CUDA (-2)
#define SLVOF_E_UNSUPPORTED (-3)
#define SLVOF_E_NOMEM (-4)
#define SLVOF_E_TOO_LARGE (-5) /* grid larger than a fixed scratch maximum (slvof_mass_noalloc) */

#define SLVOF_FP64 0  /* every stage in FP64, rounding identical to the CPU restatement */
#define SLVOF_MIXED 1 /* the SL update in flux form (FP64 node traces and swept-face volumes, FP32 clip
                         geometry), FP32 ELVIRA candidate errors with FP64 arbitration; FP64 PLIC
                         root, volume accumulation and mass sums */

#define SLVOF_STEP_BAND 1 /* recompute the band after the step (run_solver, src/NavierStokes_Parallel.jl:143) */
#define SLVOF_STEP_MASS 2 /* return sum(VF)*dx*dy*dz over the interior (src/WriteData.jl:33) */
#define SLVOF_STEP_DEFER 4 /* slvof_step_host only: leave the new state's normals, PLIC (and band) to
                              the next call, which builds them while its velocities upload */

/* Mesh and parameters.  Mirrors mesh_struct (src/Mesh.jl:1-53) and the parameters knobs the
 * path reads (src/Parameters.jl:68-77).  Coordinate arrays are the parents of mesh.x/y/z
 * (length N+2g+1, starting at imino_) and mesh.xm/ym/zm (length N+2g); they are copied at
 * slvof_create and not retained. */
typedef struct slvof_mesh {
    int32_t Nx, Ny, Nz;
    int32_t nghost;     /* 3 + max(0, ceil(CFL)-2), src/Mesh.jl:66 */
    int32_t nband;      /* ceil(CFL), src/Parameters.jl:70 */
    int32_t projection; /* 0 Euler, 1 Midpoint, 2 RK4 (src/Tools.jl:392-418); 3 the exact rotation of
                           test_case "Zalesak" (src/Tools.jl:396-399) */
    int32_t xper, yper, zper;
    double Lx, Ly, Lz, dx, dy, dz;
    double VFlo, VFhi, rho_liq, rho_gas; /* VFlo, VFhi > 0 and finite (src/Parameters.jl:68-69 default
                                            1e-10 and 1 - VFlo); others give SLVOF_E_UNSUPPORTED */
    const double *x, *y, *z;
    const double *xm, *ym, *zm;
    int32_t tesselation; /* param.tesselation (src/Parameters.jl:77): 5 "5_tets" (also 0), 6 "6_tets",
                            24 "24_tets" (src/VFgeom.jl:229-332) */
    int32_t pressure_scheme; /* param.pressure_scheme (src/Parameters.jl:60): SLVOF_PRESSURE_SEMI_LAGRANGIAN
                                (0, the default) or SLVOF_PRESSURE_FINITE_DIFFERENCE (1), whose band cells
                                add the flux-correction tets (src/Transport.jl:121-124; 5_tets; a mixed
                                context adds them to its flux form, clipped in FP32) and whose
                                band-edge momentum fluxes are finite differences */
} slvof_mesh;

#define SLVOF_PRESSURE_SEMI_LAGRANGIAN 0
#define SLVOF_PRESSURE_FINITE_DIFFERENCE 1

typedef struct slvof_ctx slvof_ctx;

/* ---- context ----------------------------------------------------------------------------
 * Device-resident state for one mesh: VF (double-buffered), face velocities, normals, PLIC
 * distances, band, cell lists and the error word, on a private CUDA stream of the current
 * device.  Replaces the per-call scratch of transport! (src/Transport.jl:23-27). */
int slvof_create(const slvof_mesh* mesh, int precision, slvof_ctx** out);
int slvof_destroy(slvof_ctx* ctx);
int slvof_last_error(const slvof_ctx* ctx, char* buf, size_t n);
/* Kernel-side time of the last call, milliseconds (CUDA events on the context's stream). */
int slvof_last_kernel_ms(const slvof_ctx* ctx, double* ms);
/* Device time of each stage of the last call, milliseconds; stages that did not run give 0.
 * Order: SL classify, SL update, VF ghost fill, ELVIRA pure cells, ELVIRA candidates,
 * normal borders, PLIC, band, mass (SLVOF_NSTAGES entries).  No counterpart in the reference
 * (its only instrumentation is @time around run_solver). */
#define SLVOF_NSTAGES 9
int slvof_stage_ms(const slvof_ctx* ctx, double* ms, int n);
/* Run the context's work on a caller-owned cudaStream_t (NULL: back to the private stream),
 * e.g. the stream of a Julia CUDA.jl task.  slvof_step and slvof_step_host also use two
 * streams of their own (the band and the VF download), ordered after the caller's stream by
 * events; the caller's stream waits for both before the call returns.  No counterpart in the
 * reference (CPU only). */
int slvof_set_stream(slvof_ctx* ctx, void* stream);
/* Work-list sizes of the last step: [0] band cells updated by the SL clip pipeline,
 * [1] interface cells given ELVIRA candidates, [2] band cells clipped whole in FP32 (in a mixed
 * step the flux form's near-pure cells; in the mixed reverse pass the cells whose pre-image is
 * not all liquid or all gas), [3] cells whose PLIC
 * plane constant was solved, [4] interface cells whose ELVIRA choice was arbitrated in FP64
 * (mixed mode), and for the mixed mode's flux-form SL update [5] grid nodes traced, [6] faces
 * swept, [7] faces that needed the clip.  No counterpart in the reference. */
#define SLVOF_NCOUNTERS 8
int slvof_counters(const slvof_ctx* ctx, int* out, int n);

/* ---- host <-> device ---------------------------------------------------------------------- */
int slvof_upload_vf(slvof_ctx* ctx, const double* VF);
int slvof_upload_velocity(slvof_ctx* ctx, const double* uf, const double* vf, const double* wf);
int slvof_upload_band(slvof_ctx* ctx, const int16_t* band);
int slvof_upload_plic(slvof_ctx* ctx, const double* nx, const double* ny, const double* nz, const double* D);
int slvof_download_vf(slvof_ctx* ctx, double* VF);
int slvof_download_normals(slvof_ctx* ctx, double* nx, double* ny, double* nz);
int slvof_download_plic(slvof_ctx* ctx, double* D);
int slvof_download_band(slvof_ctx* ctx, int16_t* band);

/* ---- resident operations (device state in, device state out) ---------------------------- */
/* Neumann!(VF) + update_VF_borders!(VF): src/Tools.jl:4-18, src/Parallel.jl:71-77. */
int slvof_vf_ghost_fill(slvof_ctx* ctx);
/* computeNormal! -> ELVIRA!: src/VF.jl:79-89, src/ELVIRA.jl:6-137. */
int slvof_compute_normal(slvof_ctx* ctx);
/* computePLIC!: src/VF.jl:94-156 (computeDist, computeAlpha). */
int slvof_compute_plic(slvof_ctx* ctx);
/* computeBand!: src/VF.jl:16-74. */
int slvof_compute_band(slvof_ctx* ctx);
/* The SL cell loop of transport! with the VF copy and ghost fill that follow it:
 * src/Transport.jl:108-151,179-181 (cell2tets!, project!, pt2index!, cutTet, d2case). */
int slvof_transport(slvof_ctx* ctx, double dt);
/* One resident step as transport! leaves the SL state: SL update + VF ghosts, ELVIRA
 * (src/Transport.jl:184), computePLIC! (src/Transport.jl:260); optionally computeBand!
 * (SLVOF_STEP_BAND) and the mass sum (SLVOF_STEP_MASS, written to *mass).  The normals used
 * by the SL update are the ones already in the context (the reference's first ELVIRA call at
 * src/Transport.jl:17 recomputes exactly those from the unchanged VF). */
int slvof_step(slvof_ctx* ctx, double dt, int flags, double* mass);
/* sum(VF[interior])*dx*dy*dz, compensated FP64 (src/WriteData.jl:33). */
int slvof_mass(slvof_ctx* ctx, double* mass);

/* ---- momentum of transport! (FP64 in either precision) ---------------------------------------
 * With the cell-centred velocities u, v, w (cell arrays), the SL update also gives us, vs, ws
 * of every interior cell (src/Transport.jl:34-166 with pressure_scheme "semi-lagrangian"):
 * band cells from the clipped pre-image (vrhoU/vrho with rho_liq/rho_gas on each side of the
 * donors' planes), the others from the face fluxes (finite-difference flux, no flux between
 * two band cells, the semi-Lagrangian flux volume SLfluxVol at band edges).  The clipped
 * momentum sums need each donor's share of a pre-image, so these calls run the FP64 clip in a
 * mixed-precision context too (its VF update is then the FP64 one). */
int slvof_upload_cell_velocity(slvof_ctx* ctx, const double* u, const double* v, const double* w);
int slvof_download_momentum(slvof_ctx* ctx, double* us, double* vs, double* ws);
/* the SL section of transport! with its momentum, on the resident state */
int slvof_transport_momentum(slvof_ctx* ctx, double dt);

/* ---- host-buffer drop-ins: one call per reference function, arrays in host memory --------
 * Each copies its inputs to the device, runs the operation and copies the outputs back.  */
/* computeNormal!(nx,ny,nz,VF,param,mesh,par_env), src/VF.jl:79 */
int slvof_computeNormal(slvof_ctx* ctx, double* nx, double* ny, double* nz, const double* VF);
/* computePLIC!(D,nx,ny,nz,VF,param,mesh,par_env), src/VF.jl:94 */
int slvof_computePLIC(slvof_ctx* ctx, double* D, const double* nx, const double* ny, const double* nz,
                      const double* VF);
/* computeBand!(band,VF,param,mesh,par_env), src/VF.jl:16 */
int slvof_computeBand(slvof_ctx* ctx, int16_t* band, const double* VF);
/* SL section of transport!(...): src/Transport.jl:108-151,179-181.  VF is updated in place. */
int slvof_transportSL(slvof_ctx* ctx, double dt, double* VF, const double* uf, const double* vf, const double* wf,
                      const double* nx, const double* ny, const double* nz, const double* D, const int16_t* band);
/* SL and momentum sections of transport! (src/Transport.jl:34-181): VF updated in place,
 * us, vs, ws written (cell arrays; interior cells). */
int slvof_transportSL_momentum(slvof_ctx* ctx, double dt, double* VF, const double* uf, const double* vf,
                               const double* wf, const double* nx, const double* ny, const double* nz, const double* D,
                               const int16_t* band, const double* u, const double* v, const double* w, double* us,
                               double* vs, double* ws);
/* Per-step drop-in for run_solver's loop with the state resident between calls: uploads
 * this step's face velocities, runs slvof_step and downloads VF (and the mass).  VF is
 * downloaded on a second stream while the new state's normals, PLIC, band and mass are built;
 * the call returns when both are done.  VF must not be null.
 * With SLVOF_STEP_DEFER the new state's normals, PLIC and (with SLVOF_STEP_BAND) band are built
 * at the start of the next slvof_step_host call with that flag, beside its velocity upload, and
 * the mass is summed from VF directly; the results are the same as without the flag.  Any other
 * entry point builds the deferred state first; device errors of those stages are reported by
 * the first status after them that reports device errors.  No counterpart in the reference (its loop is on the CPU). */
int slvof_step_host(slvof_ctx* ctx, double dt, int flags, const double* uf, const double* vf, const double* wf,
                    double* VF, double* mass);

/* ---- divergence and the pressure operator ---------------------------------------------------
 * FP64 in the reference's operation order, in either context precision (they are the pressure
 * solver's operators, not part of the interface step).  scheme: SLVOF_PRESSURE_SEMI_LAGRANGIAN or
 * SLVOF_PRESSURE_FINITE_DIFFERENCE (param.pressure_scheme).  Cell arrays (N+2g)^3; band Int16.  Each call stands
 * alone: the context's transport state is not read or changed.  For a multigrid level, use a
 * context created on that level's mesh. */
/* divergence! (src/Velocity.jl:59-68) with divg_cell (src/Velocity.jl:71-122): divg = 0 on every
 * cell, the divergence of (uf, vf, wf) over dt on the interior.  A band cell's is
 * (dx*dy*dz - v1)/(dx*dy*dz)/dt with v1 the volume of the cell projected back through the face
 * velocities; any other cell's comes from face fluxes (SLfluxVol/dt through a face next to a
 * band cell).  Host arrays. */
int slvof_divergence(slvof_ctx* ctx, double dt, int scheme, double* divg, const double* uf, const double* vf,
                     const double* wf, const int16_t* band);
/* The same on device arrays of the caller, on the context's stream. */
int slvof_divergence_device(slvof_ctx* ctx, double dt, int scheme, double* d_divg, const double* d_uf,
                            const double* d_vf, const double* d_wf, const int16_t* d_band);
/* A! (src/Pressure.jl:83-115), the left-hand side of the pressure equation: Neumann! +
 * update_borders! of P in place, the corrected face velocities uf - dt/denx * dP/dx (and y, z)
 * over the reference's index ranges, and LHS = 0 on every cell, divg_cell of the corrected
 * velocities on the interior.  Host arrays (P is read and its ghosts written back). */
int slvof_A(slvof_ctx* ctx, double dt, int scheme, double* LHS, double* P, const double* uf, const double* vf,
            const double* wf, const double* denx, const double* deny, const double* denz, const int16_t* band);
/* The same on device arrays of the caller (the corrected velocities are context scratch). */
int slvof_A_device(slvof_ctx* ctx, double dt, int scheme, double* d_LHS, double* d_P, const double* d_uf,
                   const double* d_vf, const double* d_wf, const double* d_denx, const double* d_deny,
                   const double* d_denz, const int16_t* d_band);

/* ---- curvature and face properties (FP64 in either precision) ------------------------------
 * The curvature section of transport! (src/Transport.jl:187-191): Curve = 0 on every cell, then
 * compute_curvature! (src/ELVIRA.jl:141-184) on the interior: heights of 7 cells along the
 * normal's strictly dominant axis over the 3x3 columns, central differences, the height
 * function's curvature; no strictly dominant component leaves 0.  x^(3/2) is x*sqrt(x).  Host
 * arrays: VF (N+2g+6)^3, normals and Curve (N+2g)^3. */
int slvof_computeCurvature(slvof_ctx* ctx, double* Curve, const double* VF, const double* nx, const double* ny,
                           const double* nz);
/* The same from the context's current VF and normals (after slvof_step or slvof_prepare), into a
 * device array of the caller. */
int slvof_compute_curvature_device(slvof_ctx* ctx, double* d_Curve);
/* compute_props! (src/Tools.jl:1186-1210) on every cell: face VF clamp((VF + VF[-1])/2, 0, 1),
 * density rho_liq*vf + rho_gas*(1 - vf) and viscosity vf*mu_liq + (1 - vf)*mu_gas per face
 * direction.  Null viscosity arrays give compute_dens! (src/Tools.jl:1212-1231). */
int slvof_computeProps(slvof_ctx* ctx, double rho_liq, double rho_gas, double mu_liq, double mu_gas, double* denx,
                       double* deny, double* denz, double* viscx, double* viscy, double* viscz, const double* VF);

/* ---- state save/restore and the reverse pass ------------------------------------------------
 * Reverse-mode derivative of the FP64 step (the hand-written adjoint; the reference has no
 * counterpart, its Julia callers would wrap it as a ChainRules rrule).  It treats the step as
 * the smooth function it is between switches of its discrete choices (ELVIRA candidate, band,
 * cut cases, donor cells) and is exact there.  An FP64 context runs the clip trees backwards
 * in FP64 geometry; a mixed-precision context takes the clipped volumes' derivatives from the
 * pre-images' boundaries (liquid moments of their faces, PLIC polygons) in FP32 cell-local
 * geometry, accumulated in FP64. */
/* Neumann! + VF borders, computeNormal!, computePLIC!, computeBand! on the current VF: the
 * state a step starts from (run_solver, src/NavierStokes_Parallel.jl:73-98). */
int slvof_prepare(slvof_ctx* ctx);
/* Copy the current VF (VF-array shaped) to / from a device buffer of the caller, for
 * checkpoints that stay on the device.  After loading, call slvof_prepare before stepping. */
int slvof_copy_vf_device(slvof_ctx* ctx, double* d_dst);
int slvof_load_vf_device(slvof_ctx* ctx, const double* d_src);
/* The context's VF-derivative buffer (VF-array shaped, ghosts included; NULL sets zero) and
 * its face-velocity derivative buffers (cell-array shaped).  Any NULL output is skipped. */
int slvof_adjoint_set_vf(slvof_ctx* ctx, const double* gVF);
int slvof_adjoint_get(slvof_ctx* ctx, double* gVF, double* guf, double* gvf, double* gwf);
int slvof_adjoint_zero_velocity(slvof_ctx* ctx);
/* Reverse of one slvof_step(ctx, dt, SLVOF_STEP_BAND, .) from the current state.  Before the
 * call the context holds the VF the step started from with its normals, PLIC planes and band
 * (as slvof_step or slvof_prepare leave them), the step's face velocities, and dL/dVF of the
 * step's result in the VF-derivative buffer.  After it the buffer holds dL/dVF of the
 * starting VF (ghost entries: derivatives with respect to the ghost values) and dL/d(face
 * velocities) of the step has been added to the velocity buffers.  The state is unchanged.
 * With SLVOF_PRESSURE_FINITE_DIFFERENCE the reverse includes the flux-correction tets; it runs
 * in FP64 in either precision, as that scheme's update does. */
int slvof_adjoint_step(slvof_ctx* ctx, double dt);
/* The same with the step's result given: d_VFnext is the VF (VF-array shaped, device) that
 * slvof_step(ctx, dt, SLVOF_STEP_BAND, .) produces from the current state, e.g. the next
 * checkpoint of a rollout.  A mixed-precision context then skips recomputing the clipped
 * volumes; an FP64 context ignores it.  NULL recomputes, as slvof_adjoint_step. */
int slvof_adjoint_step_next(slvof_ctx* ctx, double dt, const double* d_VFnext);
/* Fold the VF-derivative buffer's ghost entries onto the interior cells they are copies of
 * (the reverse of Neumann! + VF borders): the derivative with respect to the interior of a
 * VF whose ghosts were filled from it, e.g. the initial condition after IC!. */
int slvof_adjoint_fold(slvof_ctx* ctx);

/* ---- synthetic inputs (not part of the reference path) -----------------------------------
 * VF of a union of spheres by VFsphere's sub-sampling rule (src/Tools.jl:907-922), nF points
 * per direction, written to every cell of imino_:imaxo_ (extra VF layers zero); dims=2 uses
 * circles in x-y.  Then Neumann! + VF borders as run_solver does after IC!. */
int slvof_case_vf_spheres(slvof_ctx* ctx, const double* centres, const double* radii, int n, int nF, int dims);
/* Deformation3D face velocities at time t with period T (src/Tools.jl:660-662). */
int slvof_case_deformation3d(slvof_ctx* ctx, double t, double T);

/* ---- no-allocation variant ----------------------------------------------------------------
 * sum(VF[interior])*dx*dy*dz of a VF array that is already on the device, written to the
 * device double *d_mass, on the given cudaStream_t (NULL: the default stream).  No counterpart
 * in the reference: it serves callers that cannot allocate device memory (a host framework
 * that owns every device allocation through its own pool, or code that runs after the solver
 * has reserved all device memory), so it needs no context and calls no cudaMalloc, cudaFree or
 * allocating library routine.  Its scratch, one compensated partial sum per z-plane, is a
 * fixed static device array of the library, held on every device that loads the library
 * until the process exits; grids with Nz > SLVOF_NOALLOC_MAX_PLANES return SLVOF_E_TOO_LARGE.
 * The first call on a device looks up that array's device address in the current CUDA
 * context, so make it before any stream capture; a call in a different context (one the
 * caller made current, or the primary context created again after a device reset) looks it
 * up again.  All calls share the array: calls that overlap on the GPU race, so order them.  Only Nx, Ny, Nz, nghost, dx, dy, dz of *mesh are read.  The result is written in
 * stream order; synchronise the stream before reading it. */
#define SLVOF_NOALLOC_MAX_PLANES 8192
int slvof_mass_noalloc(const slvof_mesh* mesh, const double* d_VF, double* d_mass, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SLVOF_H */
