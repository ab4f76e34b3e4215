/* CPU restatement ("port") of the Tenjin per-timestep update, FP64.
 *
 * TEST INFRASTRUCTURE ONLY: it is the parity oracle that travels to machines
 * where the reference tree is absent, and the timed CPU baseline. It is never
 * linked into the product. Every function restates the reference's arithmetic
 * in the reference's operation order; citations are file:line in the
 * reference tree.
 *
 * State layout: for each domain, all Ncomp components of the reference's
 * CellArray in AccessPattern order (accesspattern.cpp:44-79), each a block of
 * nx*ny*nz doubles over the valid cells, i fastest. Ghost cells are not
 * stored: they are the images of valid cells given by the boundary
 * conditions (foextrap or reflect, boundary.cpp:3-42).
 */
#ifndef TENJIN_PORT_H
#define TENJIN_PORT_H

#ifdef __cplusplus
extern "C" {
#endif

#define TJP_MAX_MAT 4
#define TJP_MAX_PARAMS 16

typedef struct {
    int dim, M, solid, thinc, plastic, muscl;
    int lo_bc[3], hi_bc[3]; /* 0 transmissive, 1 reflective */
    double cfl, thinc_beta;
    int phase[TJP_MAX_MAT]; /* 0 solid, 1 fluid */
    int eos[TJP_MAX_MAT];   /* 0 MieGruneisen, 1 Romenskii, 2 Wilkins, 3 Hugoniot, 4 MixtureEOS */
    double eos_params[TJP_MAX_MAT][TJP_MAX_PARAMS];
    double yield_stress[TJP_MAX_MAT];
    int radial; /* RADIAL: geometric source term (radial.cpp) after plasticUpdate */
    int nmix;     /* numberOfMixtures: 0, or 1 with material 0 the MixtureEOS (eos 4) */
    int reactive; /* REACTIVE: reactiveUpdate (reactive.cpp) after advance */
} tjp_params;

typedef struct tjp_sim tjp_sim;

/* Number of components for the given parameters (AccessPattern size). */
int tjp_ncomp(const tjp_params* p);

tjp_sim* tjp_create(const tjp_params* p, int ndomains, const int* n_cells /* 3 per domain */,
                    const double* dim_l /* 3 per domain */, const int* nbox /* per domain */,
                    const int* boxes /* 6 per box, all domains concatenated */);
void tjp_destroy(tjp_sim* s);

/* Set the initial primitive state of a domain (alpha[M], rho_k[M], u[3], p,
 * V[9] if solid, epsilon[M] if plastic, lambda if nmix; each a block over
 * valid cells) and run primitiveToConservative (initialise.cpp:111-123); the
 * mixture densities start at rho_k (initialise.cpp:66-71). */
int tjp_set_primitive(tjp_sim* s, int domain, const double* prim);

/* Copy a domain's full state (Ncomp blocks) in / out. */
int tjp_get_state(tjp_sim* s, int domain, double* out);
int tjp_set_state(tjp_sim* s, int domain, const double* in);

/* Run the time loop of main.cpp:121-191 until t >= final_t or max_steps.
 * Writes each step's dt into dts (capacity max_steps). Returns the number of
 * steps taken, or a negative error code (-1 NaN in the state, -2 NaN wave
 * speed, -3 volume-fraction scaling error, -4 plastic divide by zero, -5 no
 * sign change for the mixture root bisection). */
int tjp_run(tjp_sim* s, double final_t, int max_steps, double* dts, double* t_out);

/* Number of OpenMP threads the port uses (1 when built without OpenMP). */
int tjp_threads(void);

#ifdef __cplusplus
}
#endif
#endif
