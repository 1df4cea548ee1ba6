/*
 * libnsem_gpu -- GB300 (sm_103a) explicit dGSEM Euler right-hand side and
 * SSP-RK stage update behind a C ABI.
 *
 * This library replaces the hot path of NebulaSEM's euler solver: the three
 * operator chains of apps/euler/euler.cpp:181-258 -- divf with Rusanov face
 * flux (src/field/field.h:3417-3478, 2928-2943), the weak surface lift
 * (field.h:3086-3117), the hydrostatic-perturbation gravity source
 * (euler.cpp:218-225, src field.h:3712-3723), the equation of state
 * (euler.cpp:211-213), the ghost-node boundary conditions
 * (applyExplicitBCs, field.h:2586-2727) -- and the explicit time update that
 * addTemporal/ddt/SolveTexplicit perform (field.h:3741-3920,
 * src/solvers/solve.cpp:563-564), here as a coupled Shu-Osher SSP-RK3.
 *
 * The reference has no plugin or FFI layer: its operator API is the set of
 * header templates in src/field/field.h over MeshField arrays and the Mesh::
 * and DG:: globals.  A C++ caller of the reference binds this ABI by passing
 * those globals and arrays directly: nsem_mesh_desc below names, field by
 * field, the global each member takes.
 *
 * Conventions
 *  - node index n = e*NP + i*NPY*NPZ + j*NPZ + k (src/field/dg.h:43-44);
 *    interior nodes [0, n_int) come first, ghost ("boundary cell") nodes
 *    [n_int, n_all) after them, n_all is the unused-slot sentinel
 *    (Mesh::gBCSfield / Mesh::gALLfield);
 *  - tensors in XX,YY,ZZ,XY,YZ,XZ,YX,ZY,ZX order (src/tensor/tensor.h:450);
 *  - state = conserved (rho, rho*u, rho*theta) on interior nodes, theta the
 *    full potential temperature (the euler app's T + T0);
 *  - every call returns nsem_status; nsem_last_error() describes the last
 *    failure on a context.  Nothing exits, traps or prints.
 *  - One context per host thread.  All device memory belongs to the context;
 *    host pointers are never kept after a call returns.
 */
#ifndef NSEM_H
#define NSEM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NSEM_ABI_VERSION 5

typedef enum {
    NSEM_OK = 0,
    NSEM_BAD_ARG = 1,     /* invalid argument or mesh description          */
    NSEM_CUDA_ERROR = 2,  /* CUDA runtime error (message in last_error)    */
    NSEM_NONFINITE = 3,   /* a NaN/Inf appeared in the state               */
    NSEM_TIMEOUT = 4,     /* a bounded device wait ran out                 */
    NSEM_UNSUPPORTED = 5, /* configuration not implemented                 */
    NSEM_NO_MEMORY = 6,   /* device or host allocation failed              */
    NSEM_TOO_LARGE = 7    /* request exceeds a fixed-size working array    */
} nsem_status;

typedef enum {
    NSEM_FP64 = 0,  /* plain form: FP64 throughout, reference operation order */
    NSEM_MIXED = 1  /* precision form: FP32 bulk, FP64 background/RK/sums;
                       hex meshes with N+1 = 4, 5, 8 (2D: 4, 5) and SYMMETRY
                       walls, any metric (axis-aligned, inclined, curved),
                       2:1 mortar faces on straight or curved elements */
} nsem_precision;

typedef enum {
    NSEM_SSPRK3 = 0,         /* coupled Shu-Osher SSP-RK3                              */
    NSEM_REF_SEGREGATED = 1  /* the reference's own update: segregated forward Euler
                              * (rho, then U, then T; euler.cpp:179-287, BDF1) on the
                              * primitive fields, FP64 only */
} nsem_scheme;

/* Mesh in the reference's own layout (Mesh:: and DG:: globals after
 * Mesh::LoadMesh / DG::init_geom, src/field/field.cpp:95-384,
 * src/field/dg.cpp:167-477).  All arrays are host memory; they are copied. */
typedef struct nsem_mesh_desc {
    int32_t npx, npy, npz;      /* DG::NPX, NPY, NPZ (LGL nodes per direction) */
    int32_t npf;                /* DG::NPF (slots per facet)                    */
    int32_t n_elem;             /* Mesh::gBCS   interior cells                  */
    int32_t n_cells;            /* Mesh::gNCells interior + boundary cells      */
    int32_t n_face;             /* Mesh::gNFacets                               */
    const double* cC;           /* [n_all*3] Mesh::cC node coordinates          */
    const double* cV;           /* [n_all]   Mesh::cV node mass weights         */
    const double* Jinv;         /* [n_all*9] DG::Jinv (inverse-transposed J)    */
    const uint32_t* FO;         /* [n_face*npf] Mesh::FO owner node per slot    */
    const uint32_t* FN;         /* [n_face*npf] Mesh::FN neighbour node         */
    const double* fN;           /* [n_face*npf*3] Mesh::fN weighted normal      */
    const double* fI;           /* [n_face*npf] Mesh::fI owner weight           */
    const uint32_t* all_faces;  /* Mesh::allFaces (cell face lists)             */
    const uint32_t* face_idx0;  /* [n_cells] Mesh::faceIndices[0]              */
    const uint32_t* face_idx1;  /* [n_cells] Mesh::faceIndices[1]              */
    const double* psi[3];       /* DG::psi[d]  [npd*npd]                         */
    const double* dpsi[3];      /* DG::dpsi[d] [npd*npd]                         */
    const uint32_t* bc_U;       /* [n_face*npf] velocity BC per slot:
                                   0 none, 1 NEUMANN, 2 SYMMETRY; scalars
                                   (rho, T, p) are NEUMANN wherever bc_U != 0 */
    /* Non-conforming (2:1) faces left by the adaptive refinement
     * (Mesh::gFMC >= 1; scatter_non_conforming / gather_non_conforming,
     * field.h:2019-2248).  n_mortar = 0 (and NULL pointers) on a conforming
     * mesh.  The FP64 forms (NSEM_REF_SEGREGATED; NSEM_SSPRK3 and
     * nsem_tendency with NSEM_FP64), nsem_convection_*, the precision form's
     * steps (NSEM_MIXED) and the FP64 tangent-linear and adjoint calls take a
     * mesh with n_mortar > 0, with or without the artificial viscosity, and
     * so does the precision form's adjoint.
     * mortar[4*q .. 4*q+3]: the facet, gFMC (1: the neighbour side FN is the
     * coarse cell, 2: the owner side FO), the coarse cell's face id
     * (gFaceID, 0..5), and the halves of that face the facet covers (bit 0
     * along the face's first in-plane axis x|x|y for ids 0-1|2-3|4-5, bit 1
     * along the second y|z|z), as scatter_non_conforming finds them. */
    int32_t n_mortar;
    const uint32_t* mortar;
    const double* psi_ref[6];   /* DG::psiRef[d*2+half] [npd*npd] */
    const double* psi_cor[6];   /* DG::psiCor[d*2+half] [npd*npd] */
} nsem_mesh_desc;

typedef struct nsem_params {
    double P0, T0, cp, cv;      /* Fluid:: properties (R = cp - cv, gamma = cp/cv) */
    double gravity[3];          /* Controls::gravity                               */
    double dt;                  /* Controls::dt                                    */
    const double* p_ref;        /* [n_all] hydrostatic p (euler.cpp:122), or NULL  */
    const double* rho_ref;      /* [n_all] hydrostatic rho (euler.cpp:123), or NULL*/
    int32_t device;             /* CUDA device ordinal                             */
    double viscosity;           /* Fluid::viscosity when the euler app runs with
                                   diffusion YES (mu = rho viscosity), else 0;
                                   used by NSEM_REF_SEGREGATED                     */
    double Pr;                  /* Fluid::Pr (> 0 when viscosity > 0)              */
} nsem_params;

typedef struct nsem_ctx nsem_ctx;

/* Replaces the setup of euler.cpp:104-131 plus the mesh upload.  If p_ref or
 * rho_ref is NULL they are computed on the host from gh = g . cC exactly as
 * euler.cpp:114-123 does (C library pow). */
nsem_status nsem_create(const nsem_mesh_desc* mesh, const nsem_params* params,
                        nsem_ctx** out);
void nsem_destroy(nsem_ctx* ctx);
const char* nsem_last_error(const nsem_ctx* ctx);
int nsem_abi_version(void);

/* Interior node count (Mesh::gBCSfield) and the context's CUDA stream. */
int64_t nsem_num_nodes(const nsem_ctx* ctx);
void* nsem_stream(const nsem_ctx* ctx);

/* Conserved state on interior nodes: rho[n], rhoU[3n] (AoS, as a
 * VectorCellField), rhoTheta[n].  Host buffers. */
nsem_status nsem_set_state(nsem_ctx* ctx, const double* rho, const double* rhoU,
                           const double* rhoTheta);
nsem_status nsem_get_state(nsem_ctx* ctx, double* rho, double* rhoU, double* rhoTheta);

/* Same in the solver's own field layout (euler.cpp:58-61): rho, U (AoS
 * velocity), T (theta' = theta - T0).  Conversion as euler.cpp:181,
 * 200, 233, 251 (rho*U, rho*(T+T0)). */
nsem_status nsem_set_fields(nsem_ctx* ctx, const double* rho, const double* U,
                            const double* T);
nsem_status nsem_get_fields(nsem_ctx* ctx, double* rho, double* U, double* T);

/* The euler app's pressure field p (= p - p_ref, euler.cpp:211-213) on
 * interior nodes, as the solver holds it when it writes its fields: after a
 * segregated step the p' of that step (from rho^{n+1} and theta^n,
 * euler.cpp:210-213); otherwise p' of the current state (euler.cpp:155-160),
 * with the correctly rounded pow.  Host buffer. */
nsem_status nsem_get_pressure(nsem_ctx* ctx, double* p_prime);

/* Tendencies L = -Su/cV of (rho, rho u, rho v, rho w, rho theta) for the
 * current state, the divf + src chains of euler.cpp:193-258 evaluated on one
 * state.  L is five host arrays of n_int doubles; p_prime (optional, may be
 * NULL) receives p - p_ref on interior nodes. */
nsem_status nsem_tendency(nsem_ctx* ctx, nsem_precision prec, double* const L[5],
                          double* p_prime);

/* Advance the state by nsteps SSP-RK3 steps of size params.dt.  Launches are
 * captured once per (precision, nsteps) into a CUDA graph and replayed. */
nsem_status nsem_step(nsem_ctx* ctx, int nsteps, nsem_scheme scheme, nsem_precision prec);

/* Mass, energy and volume sums over interior nodes (euler.cpp:165-176,
 * 263-274) with compensated summation; gh = g . cC. */
nsem_status nsem_diagnostics(nsem_ctx* ctx, double* mass, double* energy, double* volume);

/* Discrete adjoint of the plain (FP64) form.  No reference counterpart: the
 * reference has no adjoint or tangent-linear model.
 *
 * nsem_vjp: g = J_L(u)^T w for the current state u (w, g: five host arrays
 * of n_int doubles, SoA rho, rho u, rho v, rho w, rho theta).
 *
 * nsem_forward_checkpointed: advance the state by nsteps SSP-RK3 steps (FP64)
 * keeping device checkpoints of the state every ckpt_every steps.
 * nsem_adjoint: given lam_final = dJ/du at the final state of the last
 * nsem_forward_checkpointed call, return lam0 = dJ/du at its initial state
 * (reverse Shu-Osher sweep, each segment recomputed from its checkpoint with
 * its stage states kept).  The context's state is left at the final state.
 * ms_fwd / ms_adj (optional) receive the device time of the forward pass and
 * of the reverse sweep. */
nsem_status nsem_vjp(nsem_ctx* ctx, const double* const w[5], double* const g[5]);
/* Tangent-linear counterparts (no reference counterpart either).
 * nsem_jvp: Ld = J_L(u) dv for the current state u (dv, Ld: five host arrays
 * of n_int doubles, SoA).
 * nsem_tlm: advance the state by nsteps FP64 SSP-RK3 steps and propagate the
 * perturbation du0 through the linearised steps; du_final receives it at the
 * final state.  ms_tlm (optional) receives the device time. */
nsem_status nsem_jvp(nsem_ctx* ctx, const double* const dv[5], double* const Ld[5]);
nsem_status nsem_tlm(nsem_ctx* ctx, int nsteps, const double* const du0[5], double* const du_final[5],
                     double* ms_tlm);
nsem_status nsem_forward_checkpointed(nsem_ctx* ctx, int nsteps, int ckpt_every, double* ms_fwd);
nsem_status nsem_adjoint(nsem_ctx* ctx, const double* const lam_final[5], double* const lam0[5],
                         double* ms_adj);

/* The same pair in either form (no reference counterpart).
 * nsem_forward_checkpointed_prec: as nsem_forward_checkpointed, in the plain
 * (NSEM_FP64) or the precision form (NSEM_MIXED: checkpoints of the FP64
 * perturbation state; each segment's recomputation keeps the FP32 stage
 * states).  nsem_adjoint then differentiates that run in its own form: the
 * precision form's reverse sweep evaluates the transposed stage in FP32 at
 * the forward's own FP32 stage states and accumulates the adjoint state in
 * FP64.  nsem_vjp_prec: g = J_L(u)^T w in the given form (the precision form
 * at the FP32 shadow of the current state).  The precision form's adjoint
 * takes any element metric and 2:1 mortar faces, with or without the
 * artificial viscosity. */
nsem_status nsem_forward_checkpointed_prec(nsem_ctx* ctx, int nsteps, int ckpt_every,
                                           nsem_precision prec, double* ms_fwd);
nsem_status nsem_vjp_prec(nsem_ctx* ctx, nsem_precision prec, const double* const w[5],
                          double* const g[5]);

/* Scalar DG convection: the reference's convection app (apps/convection/
 * convection.cpp with problem_init NONE and time_scheme BDF1), a scalar T
 * carried by a fixed wind U with the same weak divergence, Rusanov speed
 * cds(|U|)/2 and explicit update; FP64, bit-identical to the reference where
 * no pow is involved (none is).  U: [n_int*3] AoS, T: [n_int], host arrays;
 * the wind's ghost values follow bc_U, T is NEUMANN on every wall.  Runs on
 * the context's mesh and dt, independent of the Euler state. */
nsem_status nsem_convection_set(nsem_ctx* ctx, const double* U, const double* T);
nsem_status nsem_convection_step(nsem_ctx* ctx, int nsteps);
nsem_status nsem_convection_get(nsem_ctx* ctx, double* T);

/* The convection app's analytic winds and its AB2 scheme
 * (apps/convection/convection.cpp:45-93, 103-123 with problem_init LEVEQUE;
 * src/field/field.h:3787-3804, 3885-3906 with time_scheme AB2).  Call after
 * nsem_convection_set, which resets both.
 * nsem_convection_wind: U_all [n_all*3] AoS is the wind's spatial part on
 * every node, ghost nodes included (the app fills the whole cell field from
 * the node coordinates, e.g. (sin^2(pi x) sin(2 pi y), -sin^2(pi y) sin(2 pi x),
 * 0) for LEVEQUE), or NULL to keep nsem_convection_set's wind and its wall
 * ghosts; time_scheme 1 = BDF1/AB1, 2 = AB2 (the first step AB1, as the app's
 * history starts with one stored right-hand side).
 * nsem_convection_step_scaled: nsteps steps, the wind of step s being the
 * spatial part times scale[s] in its first two components (the app's
 * u, v times cos(pi t / T); w as given); scale NULL means 1.  The AB2
 * history carries over from one call to the next. */
nsem_status nsem_convection_wind(nsem_ctx* ctx, const double* U_all, int time_scheme);
nsem_status nsem_convection_step_scaled(nsem_ctx* ctx, int nsteps, const double* scale);

/* Measurement helper: run nsteps SSP-RK3 steps launch by launch (no graph)
 * with CUDA events on the context's stream around every kernel, and report
 * per kernel class the summed device time in ms, the launch count and the
 * class name (names: 8 slots of 32 chars).  Advances the state like
 * nsem_step.  No reference counterpart (the reference has no GPU path). */
nsem_status nsem_profile(nsem_ctx* ctx, int nsteps, nsem_precision prec, double ms[8],
                         int launches[8], char names[8 * 32]);

/* Wait for all work on the context's stream. */
nsem_status nsem_sync(nsem_ctx* ctx);

/* Allocation-free mass / energy / volume sums (no counterpart in the
 * reference; it is the nsem_diagnostics computation for callers that may not
 * allocate).  For host codes that own every byte of device memory -- a solver
 * embedded in an application with its own pre-reserved pool, or a time loop
 * that must not call cudaMalloc once running (cudaMalloc can synchronise the
 * device and escapes the caller's memory accounting).
 *
 * All pointers are DEVICE memory of the current device, n_nodes entries each
 * (state SoA: rho, rho u, rho v, rho w, rho theta; node weights cV; gh = g.x;
 * hydrostatic p_ref); out3 receives mass, energy, volume in device memory,
 * enqueued on `stream` (a cudaStream_t, NULL for the default stream).
 * Nothing is allocated: the working memory is one fixed file-scope device
 * array of 3 MiB, resident on every GPU that loads the library until the
 * process exits.  n_nodes above NSEM_NOALLOC_MAX_NODES returns
 * NSEM_TOO_LARGE; NULL pointers or bad constants return NSEM_BAD_ARG.
 * The first call on a device resolves the array's device address for that
 * device (set-up once per device); make that first call before any stream
 * capture.  The address is kept for the life of the process: after
 * cudaDeviceReset on that device, or when the caller runs in a context other
 * than the device's primary context, it no longer names the array, so such
 * callers must not use this entry point.  Every call shares the one array and
 * fully rewrites the part it uses, so calls that overlap on the GPU
 * (different streams or host threads without ordering) race with each other.
 * A launch error left pending by the caller's own earlier work is returned
 * (and cleared) as NSEM_CUDA_ERROR. */
#define NSEM_NOALLOC_MAX_NODES ((int64_t)4096 * 65536)
nsem_status nsem_conservation_sums_noalloc(const double* rho, const double* rhou,
                                           const double* rhov, const double* rhow,
                                           const double* rhoTheta, const double* cV,
                                           const double* gh, const double* p_ref,
                                           int64_t n_nodes, double P0, double cp, double cv,
                                           double* out3, void* stream);

#ifdef __cplusplus
}
#endif
#endif
