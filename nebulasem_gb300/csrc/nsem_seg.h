/*
 * The reference's segregated forward-Euler update (nsem_seg.cu): device
 * buffers of the primitive fields and launchers.
 */
#ifndef NSEM_SEG_H
#define NSEM_SEG_H

#include "nsem_internal.h"

struct NsemSegBuf {
    bool ready = false;
    int cur = 0;                  /* rho[cur] holds rho^n                   */
    double* rho[2] = {};          /* density, ping-pong                     */
    double* U[3] = {};            /* velocity (SoA)                         */
    double* Tp = nullptr;         /* theta' (the euler app's T field)       */
    double* Tf = nullptr;         /* theta of the step                      */
    double* Fc[3] = {};           /* rho^n U^n                              */
    double* mu = nullptr;         /* |U^n|                                  */
    double* cs = nullptr;         /* sqrt(gamma R theta^n)                  */
    double* pp = nullptr;         /* p' from rho^{n+1}, theta^n             */
    double* lam = nullptr;        /* per slot: Rusanov speed of the step    */
    double* d[5] = {};            /* per slot: lifted fluxes                */
    /* artificial viscosity (diffusion YES) */
    double* G[12] = {};           /* per node: grad U (XX..ZX), grad theta  */
    double* fF[4] = {};           /* per slot: cds(U), cds(theta)           */
    /* non-conforming faces, per mortar slot */
    double* mq[19] = {};          /* coarse side's interpolated quantities  */
    double* mf[15] = {};          /* face flux vectors / tensors            */
    double* dC[5] = {};           /* projected, lifted coarse-side fluxes   */
    double* gC[4] = {};           /* projected cds(U), cds(theta)           */
};

/* scalar DG convection (the reference's convection app): T in a fixed wind */
struct NsemConvBuf {
    bool ready = false;
    int cur = 0;                  /* T[cur] holds T^n                       */
    double* T[2] = {};
    double* U[3] = {};
    double* lam = nullptr;        /* per slot: cds(|U|) / 2                 */
    double* d = nullptr;          /* per slot: lifted flux                  */
    /* non-conforming faces, per mortar slot (the segregated scheme's buffers) */
    double* mq[4] = {};           /* coarse side: |U| (lambda), then U T, T */
    double* mf[3] = {};           /* face flux vectors                      */
    double* dC = nullptr;         /* projected, lifted coarse-side flux     */
    /* analytic winds (the app's problem_init LEVEQUE) and the AB2 scheme */
    bool analytic = false;        /* wind = A(x) scaled per step            */
    double* A[3] = {};            /* spatial part on interior nodes         */
    double* Ag[3] = {};           /* spatial part at each used slot's ghost */
    double* Ug[3] = {};           /* the step's wind at each slot's ghost   */
    double* R[2] = {};            /* right-hand sides of the last two steps */
    int order = 1;                /* 1: BDF1 / AB1, 2: AB2                  */
    int hist = 0;                 /* right-hand sides stored (AB2)          */
};

int nsem_seg_prepare(const NsemDev* m);
/* convection steps with the analytic wind scaled by scale[s] (NULL: 1) and
 * the buffer's time scheme; advances b->cur and the AB2 history */
int nsem_conv_steps_wind(const NsemDev* m, const NsemTables* t, NsemConvBuf* b, int nsteps,
                         double dt, const double* scale, void* stream);
/* strong-form gradients of U (3 arrays) and the full theta T into G (12 per
 * node) with the per-slot scratch fF (4), for the viscous fluxes */
/* the volume part of the gradients only, from given per-slot face values fF
 * (cds of U and theta) and, on a mesh with non-conforming faces, the
 * projected coarse-side values gC (4 arrays per mortar slot; else null);
 * linear in (U, T, fF, gC) */
int nsem_grad_vol(const NsemDev* m, const NsemTables* t, const double* const* U, const double* T,
                  double* const* G, const double* const* fF, const double* const* gC, void* stream);
/* the mortar slots' face values of the gradients alone: cds(U, theta) with
 * the coarse side interpolated into fF, and its projection onto the coarse
 * side into gC; linear in (U, T) */
int nsem_grad_mortar_faces(const NsemDev* m, const double* const* U, const double* T,
                           double* const* fF, double* const* gC, void* stream);
int nsem_grad_ut(const NsemDev* m, const NsemTables* t, const double* const* U, const double* T,
                 double* const* G, double* const* fF, void* stream);
/* the same on a mesh with non-conforming faces: gC (4 arrays per mortar
 * slot) receives the projected face values */
int nsem_grad_ut_mortar(const NsemDev* m, const NsemTables* t, const double* const* U,
                        const double* T, double* const* G, double* const* fF, double* const* gC,
                        void* stream);
/* lambda of the fixed wind (once, after U is set) */
int nsem_conv_lambda(const NsemDev* m, NsemConvBuf* b, void* stream);
int nsem_conv_steps(const NsemDev* m, const NsemTables* t, NsemConvBuf* b, int nsteps, double dt,
                    void* stream);
int nsem_seg_steps(const NsemDev* m, const NsemTables* t, NsemSegBuf* b, int nsteps, double dt,
                   void* stream);
/* u = conserved state of the primitive fields rho[cur], U, T' */
int nsem_seg_to_cons(const NsemDev* m, const NsemSegBuf* b, double* const* u, void* stream);
/* primitive fields from the conserved state u */
int nsem_cons_to_seg(const NsemDev* m, NsemSegBuf* b, double* const* u, void* stream);

#endif
