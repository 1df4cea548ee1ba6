/*
 * CPU restatement of NebulaSEM's explicit dGSEM Euler operator chain.
 *
 * TEST INFRASTRUCTURE ONLY: this is the oracle the CUDA library is checked
 * against (tests, smoke check, and the timed CPU baseline).  Nothing in the
 * shipped library links or calls it.
 *
 * Pinned against the reference itself: the golden fixtures under
 * tests/golden/ were produced by oracle/ref_harness.cpp linked with the
 * reference's own library, and tests/test_oracle_golden.py requires this
 * restatement to reproduce them bit for bit.
 *
 * Layout follows the reference's MeshField storage (src/field/field.h:810-853):
 * nodes of element e are e*NP + INDEX3(i,j,k) (src/field/dg.h:43-47), interior
 * nodes first, then the ghost "boundary cell" nodes, then NP padding nodes
 * whose first index (n_all) is the unused-slot sentinel.  Face slots are
 * face*NPF + n with owner/neighbour node ids FO/FN (src/field/dg.cpp:323-410).
 */
#ifndef NSEM_ORACLE_H
#define NSEM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int32_t npx, npy, npz, np, npf;
    int32_t n_elem;     /* interior elements (gBCS)                 */
    int32_t n_cells;    /* interior + ghost cells (gNCells)         */
    int32_t n_int;      /* interior nodes (gBCSfield)               */
    int32_t n_all;      /* all nodes incl. ghosts (gALLfield)       */
    int32_t n_face;     /* facets (gNFacets)                        */
    const double* cC;       /* [n_all*3] node coordinates           */
    const double* cV;       /* [n_all]   node mass weights          */
    const double* Jinv;     /* [n_all*9] XX,YY,ZZ,XY,YZ,XZ,YX,ZY,ZX */
    const uint32_t* FO;     /* [n_face*npf]                          */
    const uint32_t* FN;     /* [n_face*npf]                          */
    const double* fN;       /* [n_face*npf*3] weighted area normal   */
    const double* fI;       /* [n_face*npf] owner interpolation      */
    const uint32_t* all_faces;  /* concatenated cell face lists     */
    const uint32_t* face_idx0;  /* [n_cells] start in all_faces     */
    const uint32_t* face_idx1;  /* [n_cells] end in all_faces       */
    const double* psi[3];   /* [npd*npd] basis values at LGL points   */
    const double* dpsi[3];  /* [npd*npd] basis derivatives            */
    const uint32_t* bcU;    /* [n_face*npf] 0 none, 1 NEUMANN, 2 SYMMETRY */
    const double* p_ref;    /* [n_all] hydrostatic pressure           */
    const double* rho_ref;  /* [n_all] hydrostatic density            */
    double gravity[3];
    double P0, R, gamma;
    double T0;              /* background potential temperature (segregated scheme) */
    double nu, Pr;          /* artificial viscosity (mu = rho nu) and Prandtl number;
                             * nu = 0: diffusion NO (segregated scheme) */
    /* non-conforming (2:1) faces of an adaptively refined mesh (segregated
     * scheme): per face {face id, gFMC (1 coarse side FN, 2 coarse side FO),
     * the coarse cell's face id, halves (bit 0 first in-plane axis, bit 1
     * second)}; the 2:1 tables psiRef / psiCor per direction d and half h at
     * [d * 2 + h] (npd * npd each).  n_mortar = 0: conforming mesh. */
    int32_t n_mortar;
    const uint32_t* mortar;
    const double* psi_ref[6];
    const double* psi_cor[6];
} nsem_oracle_mesh;

/* pow used for the equation of state: 0 = C library pow (as the reference),
 * 1 = double-double correctly rounded restatement (see oracle_pow_dd). */
void nsem_oracle_set_pow(int which);
int nsem_oracle_get_pow(void);

/* Tendencies L = -Su/cV of (rho, rho u, rho v, rho w, rho theta) on interior
 * nodes for the conserved state u (SoA, 5 arrays of n_int).  p_out, if not
 * NULL, receives p' = p - p_ref on all n_all nodes. */
void nsem_oracle_tendency(const nsem_oracle_mesh* m, const double* const u[5],
                          double* const L[5], double* p_out);

/* nsteps of the coupled Shu-Osher SSP-RK3 in place on u (SoA, n_int each). */
void nsem_oracle_ssprk3(const nsem_oracle_mesh* m, double* const u[5], double dt,
                        int nsteps);

/* Conservation sums over interior nodes (euler.cpp:165-176 with full theta):
 * mass = sum rho cV, energy = sum rho cV (gh + |u|^2/2 + cv theta (p/P0)^(R/cp)),
 * volume = sum cV.  gh is g.x per node. */
void nsem_oracle_diagnostics(const nsem_oracle_mesh* m, const double* const u[5],
                             const double* gh, double cv_heat, double out[3]);

double nsem_oracle_pow_dd(double x, double y);

/* Tangent-linear model (nsem_tlm.cpp, dual numbers): Ld = J_L(u) du; and
 * (u, du) advanced through nsteps SSP-RK3 steps. */
void nsem_oracle_jvp(const nsem_oracle_mesh* m, const double* const u[5], const double* const du[5],
                     double* const L[5], double* const Ld[5]);
void nsem_oracle_tlm_ssprk3(const nsem_oracle_mesh* m, double* const u[5], double* const du[5],
                            double dt, int nsteps);
/* nd <= 8 tangent directions in one pass: du[5*d + c] is direction d,
 * variable c.  Returns 0, or -1 if nd is out of range. */
int nsem_oracle_tlm_ssprk3_multi(const nsem_oracle_mesh* m, double* const u[5], double* const* du,
                                 int nd, double dt, int nsteps);

/* The reference's own segregated forward-Euler update (euler.cpp:179-287,
 * BDF1, no diffusion) on the primitive fields: rho[n_int], U[n_int*3] (AoS),
 * T[n_int] = theta' (perturbation), advanced in place by nsteps steps. */
void nsem_oracle_segregated(const nsem_oracle_mesh* m, double* rho, double* U, double* T,
                            double dt, int nsteps);

/* The reference's scalar DG convection (apps/convection/convection.cpp,
 * problem_init NONE, BDF1): T[n_int] advected by the fixed wind U[n_int*3]
 * (AoS) for nsteps steps, in place. */
void nsem_oracle_convection(const nsem_oracle_mesh* m, const double* U, double* T, double dt,
                            int nsteps);
void nsem_oracle_convection_wind(const nsem_oracle_mesh* m, const double* U_all, const double* scale,
                                 int order, double* T, double dt, int nsteps);

int nsem_oracle_threads(void);

#ifdef __cplusplus
}
#endif
#endif
