/*
 * Discrete adjoint of the plain form (nsem_adjoint.cu).
 */
#ifndef NSEM_ADJOINT_H
#define NSEM_ADJOINT_H

#include <stdint.h>

#include "nsem_internal.h"

struct NsemAdjBuf {
    double* adjO[6] = {};   /* per slot: owner-side primitive adjoints   */
    double* adjN[6] = {};   /* per slot: neighbour-side primitive adjoints */
    double* lam[5] = {};    /* adjoint of the current step state          */
    double* a3[5] = {};
    double* lu2[5] = {};
    double* lu1[5] = {};
    double* g[5] = {};      /* VJP output                                 */
    double* fin[5] = {};    /* final forward state (restored afterwards)  */
    double* ckpt = nullptr; /* [n_ckpt][5][n_int] states every k steps     */
    double* seg = nullptr;  /* [k][3][5][n_int] u^n, u1, u2 of a segment   */
    int64_t seg_slots = 0;  /* state slots allocated in seg                 */
    /* artificial viscosity (nu != 0): per node U, theta of the state and their
     * tangents / adjoints, gradients (9 + 3) and their tangents / adjoints;
     * per slot cds(U, theta) and its tangent, face adjoints */
    bool visc = false;
    double* pU[4] = {};
    double* dpU[4] = {};
    double* Gv[12] = {};
    double* dGv[12] = {};
    double* fF[4] = {};
    double* dfF[4] = {};
    double* dbv[4] = {};    /* per slot: momentum and theta flux adjoints        */
    double* Gbs[12] = {};   /* per node: gradient adjoints divided by cV         */
    double* mub = nullptr;  /* per node: adjoint of mu = rho nu                   */
    double* agO[4] = {};    /* per slot: gradient face-term adjoints, owner side  */
    double* agN[4] = {};    /* per slot: neighbour side                           */
    /* non-conforming (2:1) faces: per mortar slot the coarse
     * side's 19 interpolated face quantities and their tangents, the tangent
     * flux vectors (15) and the projected, lifted tangents (5), the adjoints of
     * the interpolated quantities; per node the transposed interpolation */
    double* mq[19] = {};
    double* dmq[19] = {};
    double* dmf[15] = {};
    double* ddC[5] = {};
    double* mqb[19] = {};
    double* qb[19] = {};
    /* non-conforming faces with the artificial viscosity: the gradients'
     * projected coarse-side face values and their tangents (4 per mortar
     * slot), the fine side's viscous quantity adjoints (12 per mortar slot),
     * the gradient face values' adjoints from the fine side and the coarse
     * side (4 each per mortar slot), and per node the mortars' (U, theta)
     * adjoints of the gradient face terms */
    double* gC[4] = {};
    double* dgC[4] = {};
    double* mqv[12] = {};
    double* fFb[4] = {};
    double* gCb[4] = {};
    double* pbM[4] = {};
    int nsteps = 0, every = 0, n_ckpt = 0;
    bool ready = false;
};

/* g = J_L(S)^T W (all device pointers, 5 SoA arrays each) */
int nsem_adj_vjp(const NsemDev* m, const NsemTables* t, const double* const* S,
                 const double* const* W, double* const* G, NsemAdjBuf* ab, void* stream);
/* out = J_L(S) dS (tangent-linear product; uses ab->adjO[0..4] as slot scratch) */
int nsem_adj_jvp(const NsemDev* m, const NsemTables* t, const double* const* S,
                 const double* const* dS, double* const* out, NsemAdjBuf* ab, void* stream);
/* out = cx x + cy y + cz z (y, z may be null) */
int nsem_adj_lin3(double* const* out, const double* const* x, double cx, const double* const* y,
                  double cy, const double* const* z, double cz, int64_t n, void* stream);
int nsem_adj_prepare(const NsemDev* m);

#endif
