/* tenjin_gpu.h -- C ABI of the GB300 implementation of Tenjin's per-timestep
 * update (libtenjin_gpu.so).
 *
 * The reference has no plugin or FFI layer: its operator surface is a set of
 * C++ free functions and class methods called from the time loop
 * (main.cpp:121-191). Each entry point below replaces one of them, working on
 * state held in device memory by a context. The host exchanges state in the
 * reference's own layout: one AMReX FArrayBox per box, components in
 * AccessPattern order (accesspattern.cpp:44-79), component-major SoA with i
 * fastest (Array4(i,j,k,n)), over the box grown by ngrow cells.
 *
 * Conventions
 *   - Every call returns TJ_OK (0) or a negative TJ_ERR_* status; the
 *     reference prints and calls exit(1) instead (e.g. hllc.cpp:199,
 *     boxaccesscellarray.cpp:561,587). tj_last_error() gives the message.
 *   - A context owns its device memory. Host buffers are read or written only
 *     during the call. Work is ordered on the context's CUDA stream; calls
 *     that return data to the host synchronise it. A context is not thread
 *     safe: use one per host thread.
 *   - All arithmetic of TJ_PRECISION_FP64 is IEEE binary64 in the
 *     reference's evaluation order.
 */
#ifndef TENJIN_GPU_H
#define TENJIN_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define TJ_MAX_MATERIALS 4
#define TJ_MAX_EOS_PARAMS 16

/* status codes */
#define TJ_OK 0
#define TJ_ERR_ARG -1        /* invalid argument or unsupported parameter combination */
#define TJ_ERR_CUDA -2       /* a CUDA call failed */
#define TJ_ERR_NAN -3        /* NaN in the state (main.cpp:183-187) */
#define TJ_ERR_WAVESPEED -4  /* NaN wave speed in the 5-wave solver (hllc.cpp:169-200,367-373) */
#define TJ_ERR_ALPHA -5      /* volume-fraction scaling error (boxaccesscellarray.cpp:553-588) */
#define TJ_ERR_PLASTIC -6    /* plastic divide by zero (plastic.cpp:189-193) */
#define TJ_ERR_STATE -7      /* call out of order (no domain, no state) */
#define TJ_ERR_ROOT -8       /* no sign change in the mixture root bisection (equationofstate.cpp:327-335) */

/* equation-of-state kinds; parameter vectors as getMaterialParameters builds
 * them (initialise.cpp:125-235) */
#define TJ_EOS_MIEGRUNEISEN 0 /* [gamma, pref, eref, CV]                         equationofstate.cpp:5-115 */
#define TJ_EOS_ROMENSKII 1    /* [gamma, pref, eref, CV, rho0, K0, a, b, G0]     equationofstate.cpp:403-495 */
#define TJ_EOS_WILKINS 2      /* [gamma, pref, eref, CV, rho0, e1..e5, G0]       equationofstate.cpp:502-596 */
#define TJ_EOS_HUGONIOT 3     /* [gamma, pref, eref, CV, rho0, c0, s, G0]: linear us-up Hugoniot reference
                                 curve with constant Gruneisen gamma; no reference counterpart */
#define TJ_EOS_MIXTURE 4      /* [gamma, pref, eref, CV] of the reactant, then of the products:
                                 MixtureEOS (equationofstate.cpp:117-396), a "mixture" fluid; material
                                 0 only, with n_mixtures = 1 */

#define TJ_PHASE_SOLID 0 /* Material_type (structdefinitions.h:36-40) */
#define TJ_PHASE_FLUID 1

#define TJ_BC_TRANSMISSIVE 0 /* Boundary_type (structdefinitions.h:51-55): foextrap */
#define TJ_BC_REFLECTIVE 1   /* reflect_even, reflect_odd for the normal velocity and momentum */

#define TJ_PRECISION_FP64 0  /* every operation in binary64, reference order */
#define TJ_PRECISION_MIXED 1 /* fused kernels in binary32 (2-D; 3-D fluids without THINC over
                                any number of domains); total energy and the pressure-closure
                                numerator as compensated pairs */
#define TJ_PRECISION_FUSED64 2 /* the fused 2-D kernels in binary64: agrees with
                                  TJ_PRECISION_FP64 to round-off, not bit for bit */

typedef struct tj_material {
    int phase;        /* TJ_PHASE_* */
    int eos;          /* TJ_EOS_* */
    int nparams;
    double params[TJ_MAX_EOS_PARAMS];
    double yield_stress; /* PlasticEOS::yieldStress (plastic.h:21), solids only */
} tj_material;

/* Mirrors ParameterStruct (structdefinitions.h:105-144) plus the boundary
 * types of InitialStruct (structdefinitions.h:165-166). */
typedef struct tj_params {
    int dim;          /* AMREX_SPACEDIM: 1, 2 or 3 */
    int n_materials;  /* numberOfMaterials */
    int n_mixtures;   /* numberOfMixtures: 0, or 1 with material 0 a TJ_EOS_MIXTURE fluid */
    int SOLID, THINC, RADIAL, PLASTIC, REACTIVE, MUSCL; /* RADIAL: not with elastic solids (SOLID
                                                          without PLASTIC); mixtures: SOLID = 0 */
    int nghost;       /* Nghost: must be >= 2 */
    int lo_bc[3], hi_bc[3];
    double CFL, THINCbeta;
    int precision;    /* TJ_PRECISION_* */
    tj_material materials[TJ_MAX_MATERIALS];
} tj_params;

typedef struct tj_ctx tj_ctx;

/* Context lifetime. */
int tj_create(const tj_params* params, tj_ctx** out);
int tj_destroy(tj_ctx* ctx);
int tj_last_error(const tj_ctx* ctx, char* buf, unsigned long len);
/* AccessPattern size Ncomp (main.cpp:55). */
int tj_ncomp(const tj_ctx* ctx);

/* Geometry. A context holds one or more independent domains (each its own
 * Geometry with its own physical boundaries); they share one dt. Domain d
 * covers cells [0, n_cells[3d+k]) along axis k with physical length
 * dim_l[3d+k]. Replaces the BoxArray / Geometry set-up of main.cpp:34-46.
 * Reallocates the device state (zeroed). */
int tj_set_domains(tj_ctx* ctx, int ndomains, const int* n_cells, const double* dim_l);
/* Box list of one domain in MFIter order, lo/hi inclusive (6 ints per box).
 * Defaults to one box per domain. The box list must tile the domain. It
 * matters for BVD-THINC only (thinc.cpp:57-63 reads box ghost cells). */
int tj_set_boxes(tj_ctx* ctx, int domain, int nbox, const int* lohi);
/* max_grid_size chopping of a domain (BoxArray::maxSize, main.cpp:36). */
int tj_set_max_grid_size(tj_ctx* ctx, int domain, int max_grid_size);
int tj_num_boxes(const tj_ctx* ctx, int domain);
int tj_get_box(const tj_ctx* ctx, int domain, int box, int* lohi);
int tj_num_cells(const tj_ctx* ctx, long long* ncells);

/* State exchange in the reference's FArrayBox layout (box grown by ngrow,
 * ncomp must equal tj_ncomp). Upload reads the valid cells of the components
 * the update carries from step to step (alpha, alphaRho, rho_k, rho, rhoU, u,
 * E, p, and rhomix, lambda, alphaRhoLambda, V, HenckyJ2, epsilon,
 * alphaRhoEpsilon where present); the derived ones (a, uStar, sigma, VStar,
 * devH) are recomputed on the device and not read. Download writes every
 * component of the valid cells (ghosts untouched). When the device accesses
 * host memory coherently (Grace + NVLink-C2C), the conversion kernels read a
 * page-locked upload buffer (cudaHostAlloc or cudaHostRegister, a pinned
 * torch tensor) in place, and write a download buffer from cudaHostAlloc in
 * place; other buffers are staged through device memory. Both give the same
 * bytes; every call returns with the transfer complete. */
int tj_upload_state(tj_ctx* ctx, int domain, int box, const double* fab, int ncomp, int ngrow);
int tj_download_state(tj_ctx* ctx, int domain, int box, double* fab, int ncomp, int ngrow);
/* Whole-domain exchange: ncomp blocks of nx*ny*nz doubles (valid cells, i
 * fastest), AccessPattern order. */
int tj_upload_domain(tj_ctx* ctx, int domain, const double* data);
int tj_download_domain(tj_ctx* ctx, int domain, double* data);
/* Initial condition from primitive fields (alpha[M], rho_k[M], u[3], p,
 * V[9] if SOLID, epsilon[M] if PLASTIC, lambda if n_mixtures; each nx*ny*nz
 * doubles), then primitiveToConservative: the last step of
 * setInitialConditions (initialise.cpp:111-123). The mixture densities start
 * at rho_k (initialise.cpp:66-71). */
int tj_set_primitive(tj_ctx* ctx, int domain, const double* prim);

/* Operators of the time loop. */
/* TimeStep::getTimeStep (timestep.cpp:36-70): CFL * min over cells and
 * directions of dx/(a+|u|), after the halo fill of main.cpp:124-126. */
int tj_compute_dt(tj_ctx* ctx, double* dt);
/* advance (hllc.cpp:699-707): two HLLCadvance stages and U1 = (U + U2)/2. */
int tj_advance(tj_ctx* ctx, double dt);
/* One RK stage of advance, for testing (FP64 precision only). stage 0: the
 * state becomes U1 = HLLCadvance(U^n) (hllc.cpp:701), U^n is kept; stage 1:
 * the state becomes U^n/2 + HLLCadvance(U1)/2 (703-705). Stage 0 then stage
 * 1 with the same dt equals tj_advance. */
int tj_advance_stage(tj_ctx* ctx, int stage, double dt);
/* PlasticEOS::plasticUpdate (plastic.cpp:227-244), radial return. */
int tj_plastic_update(tj_ctx* ctx, double dt);
/* geometricSourceTerm (radial.cpp:37-54): the radial source of a spherical
 * (1-D) or cylindrical (2-D, 3-D) problem with x the radius, then
 * conservativeToPrimitive. The stress it reads is the state's as its last
 * conservativeToPrimitive left it. tj_step applies it after plasticUpdate
 * when RADIAL is set (main.cpp:159-161). */
int tj_geometric_source(tj_ctx* ctx, double dt);
/* reactiveUpdate (reactive.cpp:60-103): the pressure-based burn of the
 * mixture's mass fraction by two Euler steps averaged with the start value,
 * then conservativeToPrimitive. A no-op without mixtures. tj_step applies it
 * after advance when REACTIVE is set (main.cpp:149-152). */
int tj_reactive_update(tj_ctx* ctx, double dt);
/* CellArray::cleanUpV (boxaccesscellarray.cpp:476-528). */
int tj_cleanup_v(tj_ctx* ctx);
/* CellArray::cleanUpAlpha (boxaccesscellarray.cpp:530-599). */
int tj_cleanup_alpha(tj_ctx* ctx);
/* CellArray::conservativeToPrimitive / primitiveToConservative
 * (boxaccesscellarray.cpp:67-174), on every valid cell. */
int tj_cons_to_prim(tj_ctx* ctx);
int tj_prim_to_cons(tj_ctx* ctx);
/* CellArray::contains_nan (cellarray.cpp:101-116): *flag = 1 if NaN. */
int tj_contains_nan(tj_ctx* ctx, int* flag);

/* Global conservation sums of the current state in binary64: sums[k] for
 * k < n_materials is the sum over the valid cells of every domain of
 * alphaRho_k * cell volume, sums[n_materials + r] (r = 0, 1, 2) that of rhoU_r,
 * sums[n_materials + 3] that of E. The reduction order is fixed, so the same
 * state gives the same bits on any GPU. HOST array of n_materials + 4 doubles.
 * No reference counterpart (the reference checks only for NaN,
 * cellarray.cpp:101-116). */
int tj_conservation_sums(tj_ctx* ctx, double* sums);
/* One AccessPattern component (accesspattern.cpp:44-79) of one domain's valid
 * cells, nx*ny*nz doubles, i fastest: the plane tj_download_domain writes at
 * that component, without moving the others. */
int tj_download_component(tj_ctx* ctx, int domain, int comp, double* data);

/* One iteration of the time loop of main.cpp:121-191 with dt and t kept on
 * the device: dt = getTimeStep, clamped to t_end, times 0.2 for the first
 * five steps; advance; reactiveUpdate (REACTIVE); plasticUpdate (PLASTIC);
 * geometricSourceTerm (RADIAL); cleanUpV (SOLID);
 * cleanUpAlpha; NaN check. Does not synchronise. */
int tj_step(tj_ctx* ctx, double t_end);
/* Run up to nsteps iterations or until t >= t_end. Steps are issued in
 * groups captured as CUDA graphs; the host polls t between groups. */
int tj_run(tj_ctx* ctx, int nsteps, double t_end, int* steps_done, double* t_out);
/* Simulated time, step count and last dt (synchronises). */
int tj_get_time(tj_ctx* ctx, double* t, int* nsteps, double* last_dt);
int tj_set_time(tj_ctx* ctx, double t, int nsteps);
/* Device-side status word of the last steps (sticky; TJ_OK if clean). */
int tj_status(tj_ctx* ctx);
int tj_synchronize(tj_ctx* ctx);
/* Number of this library's kernel launches issued by the context so far. */
int tj_launch_count(const tj_ctx* ctx, long long* count);
/* The cudaStream_t that orders all work of the context. */
int tj_get_stream(tj_ctx* ctx, void** stream);
/* Per-kernel timing: when on, CUDA events are recorded around every launch of
 * this library's kernels (also inside captured graphs); tj_kernel_time
 * returns the summed duration and launch count of one kernel name since
 * profiling was switched on. */
int tj_set_profiling(tj_ctx* ctx, int on);
int tj_kernel_time(tj_ctx* ctx, const char* kernel, double* ms_total, long long* launches);

/* The launch configuration the fused kernels use (for 3-D: the tile shape
 * the autotuner chose, the number of tiles and the persistent grid). No
 * reference counterpart. */
int tj_kernel_config(const tj_ctx* ctx, char* buf, unsigned long len);

/* Adjoint pair (the forward / backward of a torch.autograd.Function). The
 * reference has no adjoint; the pair differentiates its per-timestep update
 * (main.cpp:145-187 with the loop of main.cpp:121-191), TJ_PRECISION_FP64,
 * one domain, dt frozen. 2-D fluids with the stiffened-gas EOS (BVD-THINC
 * included) take the dedicated reverse sweep; every other configuration
 * without BVD-THINC and mixtures (1-, 2- and 3-D, solids with the 5-wave
 * solver, the plastic radial return, cleanUpV, the radial source, every EOS)
 * takes the general reverse mode, built from local Jacobians of the FP64
 * path's own device functions (forward-mode passes, one per input of each
 * cell's update and each face's Riemann problem): exact, deterministic, a
 * backward 50-110 times the forward's time.
 * tj_forward: initial state from the primitives prim0 (the tj_set_primitive
 * layout without mixture words) with the EOS parameters eos
 * ([n_materials][TJ_MAX_EOS_PARAMS] in the getMaterialParameters order,
 * initialise.cpp:125-235; NULL keeps the current ones), THINC scratch zeroed,
 * then nsteps steps of advance and the post-advance operators with dt[n]
 * (HOST array); the state (and the THINC scratch) are saved every `stride`
 * steps. The final state is the context's state.
 * tj_backward: from grad_state, the gradient of a scalar objective with
 * respect to the final state (tj_download_domain layout; components derived
 * from others - sound speed, sigma, USTAR, VSTAR, devH - are ignored), to the
 * gradient with respect to prim0 (grad_prim0, same layout as prim0) and to
 * the EOS parameters (grad_eos, HOST, [n_materials][TJ_MAX_EOS_PARAMS]). Each
 * interval of `stride` steps is recomputed from its checkpoint and reversed;
 * limiter, THINC, Riemann-solver and yield branches are differentiated at
 * their forward choice. prim0, grad_state and grad_prim0 may be host or
 * device pointers. */
int tj_forward(tj_ctx* ctx, int domain, const double* prim0, const double* eos, int nsteps, const double* dt,
               int stride);
int tj_backward(tj_ctx* ctx, int domain, const double* grad_state, double* grad_prim0, double* grad_eos);

/* Tangent-linear (forward-mode) run of the update: one directional
 * derivative of the final state. The reference has no derivative; the run is
 * the FP64 path (its per-direction kernels instantiated with values that
 * carry a direction) from the initial state of the primitives prim0 (the
 * tj_set_primitive layout, without mixture words) along dprim0 (same layout,
 * NULL: zero) and the EOS parameters along deos (HOST,
 * [n_materials][TJ_MAX_EOS_PARAMS], NULL: zero; eos as in tj_forward), over
 * nsteps steps of advance with the post-advance operators (main.cpp:145-187)
 * with dt[n] (HOST). Every configuration of a TJ_PRECISION_FP64 context with
 * one domain and no mixtures: fluids and solids, the 5-wave solver, the
 * plastic radial return, cleanUpV, the radial source, BVD-THINC. Branches
 * are differentiated at the side the FP64 run takes, whose values the run
 * reproduces bit for bit. state (may be NULL) receives the final values and
 * dstate their directions, in the tj_download_domain layout (components
 * derived from the carried ones -- sound speed, USTAR, sigma, VSTAR, devH --
 * are zero); prim0, dprim0, state and dstate may be host or device pointers.
 * The context's own state is not changed. With tj_forward / tj_backward on
 * the same run, <grad_state, dstate> = <grad_prim0, dprim0> + <grad_eos,
 * deos> to rounding. */
int tj_tangent(tj_ctx* ctx, int domain, const double* prim0, const double* dprim0, const double* eos,
               const double* deos, int nsteps, const double* dt, double* state, double* dstate);

/* Time step without any device allocation. No counterpart in the reference:
 * it exists for callers that cannot allocate device memory themselves (a
 * host whose framework owns the GPU's memory pool, a plugin restricted to the
 * buffers its host hands it, a running loop that must not allocate). Needs no
 * context. state: DEVICE pointer to one domain's state in the AccessPattern
 * layout (tj_ncomp blocks of nx*ny*nz doubles, i fastest); dt: HOST pointer
 * receiving CFL * min(dx/(a+|u|)) computed in binary64, as tj_compute_dt
 * computes it for a TJ_PRECISION_FP64 context (params->precision is not
 * read); stream: the cudaStream_t to order the work on (NULL: the default
 * stream). Working memory is a fixed array inside the library
 * (TJ_NOALLOC_MAX_CELLS bounds the domain; larger domains return
 * TJ_ERR_ARG). The first call on a device looks up that array's address.
 * Every call copies dt to the host and synchronises the stream, so no call
 * may be made while that stream is being captured. Calls that overlap on the
 * GPU share the array and race: serialise them. */
#define TJ_NOALLOC_MAX_CELLS (1 << 24)
int tj_compute_dt_noalloc(const tj_params* params, const int* n_cells, const double* dim_l, const double* state,
                          double* dt, void* stream);

#ifdef __cplusplus
}
#endif
#endif
