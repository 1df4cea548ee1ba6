/*
 * CPU restatement of the reference's explicit dGSEM Euler right-hand side and
 * of the coupled SSP-RK3 driver used as the parity oracle.
 *
 * TEST INFRASTRUCTURE ONLY (see nsem_oracle.h).  Every operation is written
 * in the order the reference evaluates it, so that with -ffp-contract=off the
 * result is bit-identical to the reference library's on the same inputs:
 *
 *   tensor helpers       src/tensor/tensor.h:116-118 (right-nested Vector dot),
 *                        src/tensor/tensor.cpp:15-27 (outer product), 72-78
 *                        (Tensor.Vector), tensor.h:486-494 (sym)
 *   boundary ghosts      src/field/field.h:2670-2685 (NEUMANN, SYMMETRY)
 *   equation of state    apps/euler/euler.cpp:211-213
 *   wave speed           apps/euler/euler.cpp:186, cds field.h:2881-2893
 *   Rusanov flux         src/field/field.h:2928-2943
 *   surface lift         src/field/field.h:3086-3117 (weak form)
 *   volume term          src/field/field.h:3440-3464 with DPSI dg.h:67-75
 *   gravity source       apps/euler/euler.cpp:224-234, src field.h:3712-3723
 *   tendency             L = -Su/cV (forward-Euler update of solve.cpp:563-564
 *                        written per unit time)
 */
#include "nsem_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { XX, YY, ZZ, XY, YZ, XZ, YX, ZY, ZX };

static int g_pow_mode = 0;

void nsem_oracle_set_pow(int which) { g_pow_mode = which; }
int nsem_oracle_get_pow(void) { return g_pow_mode; }

int nsem_oracle_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static inline double eos_pow(double x, double y) {
    return g_pow_mode ? nsem_oracle_pow_dd(x, y) : pow(x, y);
}

/* Vector dot, nested from the right as the reference's unrolled loop. */
static inline double vdot(const double* a, const double* b) {
    return a[0] * b[0] + (a[1] * b[1] + (a[2] * b[2] + 0.0));
}
static inline double vmag(const double* a) { return sqrt(vdot(a, a)); }

/* Tensor . Vector, row by row, summed left to right. */
static inline void tdot(const double* q, const double* p, double* r) {
    r[0] = q[XX] * p[0] + q[XY] * p[1] + q[XZ] * p[2];
    r[1] = q[YX] * p[0] + q[YY] * p[1] + q[YZ] * p[2];
    r[2] = q[ZX] * p[0] + q[ZY] * p[1] + q[ZZ] * p[2];
}

/* Outer product p (x) q in XX,YY,ZZ,XY,YZ,XZ,YX,ZY,ZX order. */
static inline void outer(const double* p, const double* q, double* r) {
    r[XX] = p[0] * q[0];
    r[YY] = p[1] * q[1];
    r[ZZ] = p[2] * q[2];
    r[XY] = p[0] * q[1];
    r[YZ] = p[1] * q[2];
    r[XZ] = p[0] * q[2];
    r[YX] = p[1] * q[0];
    r[ZY] = p[2] * q[1];
    r[ZX] = p[2] * q[0];
}

/* Symmetry ghost velocity: tangential projection rescaled to |p|. */
static inline void sym_vec(const double* p, const double* n, double* out) {
    double mg = vmag(n);
    double en[3] = {n[0] / mg, n[1] / mg, n[2] / mg};
    /* A = I - en en^T (symmetric storage XX,YY,ZZ,XY,YZ,XZ) */
    double A[6];
    A[0] = 1.0 - en[0] * en[0];
    A[1] = 1.0 - en[1] * en[1];
    A[2] = 1.0 - en[2] * en[2];
    A[3] = 0.0 - en[0] * en[1];
    A[4] = 0.0 - en[1] * en[2];
    A[5] = 0.0 - en[0] * en[2];
    double r[3];
    r[0] = A[0] * p[0] + A[3] * p[1] + A[5] * p[2];
    r[1] = A[3] * p[0] + A[1] * p[1] + A[4] * p[2];
    r[2] = A[5] * p[0] + A[4] * p[1] + A[2] * p[2];
    double magR = vmag(r);
    if (fabs(magR - 0.0) <= 1e-7) {
        out[0] = r[0]; out[1] = r[1]; out[2] = r[2];
        return;
    }
    double s = vmag(p) / magR;
    out[0] = r[0] * s; out[1] = r[1] * s; out[2] = r[2] * s;
}

typedef struct {
    double *rho, *U, *T, *p;    /* primitive fields on n_all (+pad) nodes */
    double *d_rho, *d_mom, *d_th; /* per-slot lifted fluxes                */
    double *r_rho, *r_mom, *r_th; /* residuals on n_all nodes              */
    double *mu, *GU, *GT;         /* artificial viscosity: rho nu, grad U, grad theta */
    /* non-conforming faces: coarse-side slot values, node quantities, face
     * flux vectors, their projection, projected lifted values, gradient cds */
    int8_t* side;
    double *mq, *nq, *mF, *mP, *dC, *gS, *gC, *gT;
} work_t;

static void work_alloc(const nsem_oracle_mesh* m, work_t* w) {
    size_t na = (size_t)m->n_all + (size_t)m->np;
    size_t ns = (size_t)m->n_face * (size_t)m->npf;
    w->rho = calloc(na, sizeof(double));
    w->U = calloc(na * 3, sizeof(double));
    w->T = calloc(na, sizeof(double));
    w->p = calloc(na, sizeof(double));
    w->d_rho = calloc(ns, sizeof(double));
    w->d_mom = calloc(ns * 3, sizeof(double));
    w->d_th = calloc(ns, sizeof(double));
    w->r_rho = calloc(na, sizeof(double));
    w->r_mom = calloc(na * 3, sizeof(double));
    w->r_th = calloc(na, sizeof(double));
    w->mu = w->GU = w->GT = NULL;
    if (m->nu != 0.0) {
        w->mu = calloc(na, sizeof(double));
        w->GU = calloc(na * 9, sizeof(double));
        w->GT = calloc(na * 3, sizeof(double));
    }
    w->side = NULL;
    w->mq = w->nq = w->mF = w->mP = w->dC = w->gS = w->gC = w->gT = NULL;
}

static void work_free(work_t* w) {
    free(w->rho); free(w->U); free(w->T); free(w->p);
    free(w->d_rho); free(w->d_mom); free(w->d_th);
    free(w->r_rho); free(w->r_mom); free(w->r_th);
    free(w->mu); free(w->GU); free(w->GT);
    free(w->side); free(w->mq); free(w->nq); free(w->mF); free(w->mP); free(w->dC);
    free(w->gS); free(w->gC); free(w->gT);
}

/* NEUMANN (value 0) ghost: interior value + 0*|dv| (field.h:2674-2676). */
static inline double neumann(const nsem_oracle_mesh* m, const double* f, uint32_t c1,
                             uint32_t c2) {
    const double* a = m->cC + 3 * (size_t)c1;
    const double* b = m->cC + 3 * (size_t)c2;
    double dv[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    return f[c1] + 0.0 * vmag(dv);
}

static void grad_strong(const nsem_oracle_mesh* m, int ncomp, const double* p, double* G,
                        const int8_t* side, const double* fS, const double* fC);
static int8_t* mortar_sides(const nsem_oracle_mesh* m);
static void mortar_scatter(const nsem_oracle_mesh* m, int ncomp, const double* Q, double* out);
static void mortar_gather(const nsem_oracle_mesh* m, int ncomp, const double* F, double* out);
static void mortar_cds(const nsem_oracle_mesh* m, int ncomp, const double* p, const int8_t* side,
                       double* tmp, double* fS, double* fC);

/* the coupled residual's node quantities a mortar's coarse side interpolates:
 * |U|, c, U rho (3), rho, the momentum flux tensor (9), the theta flux (3),
 * rho theta */
#define NQ_COUPLED 19

static void residual(const nsem_oracle_mesh* m, const double* const u[5], work_t* w,
                     double* p_out) {
    const int32_t NPX = m->npx, NPY = m->npy, NPZ = m->npz, NP = m->np, NPF = m->npf;
    const int64_t n_int = m->n_int, n_all = m->n_all;
    const int64_t n_slot = (int64_t)m->n_face * NPF;
    const double P0 = m->P0, R = m->R, gam = m->gamma;

    /* primitive variables on interior nodes */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n_int; i++) {
        double r = u[0][i];
        w->rho[i] = r;
        w->U[3 * i + 0] = u[1][i] / r;
        w->U[3 * i + 1] = u[2][i] / r;
        w->U[3 * i + 2] = u[3][i] / r;
        w->T[i] = u[4][i] / r;
    }
    /* ghost values: rho, T Neumann; U symmetry */
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n_slot; k++) {
        if (!m->bcU[k]) continue;
        uint32_t c1 = m->FO[k], c2 = m->FN[k];
        if (c2 >= (uint32_t)n_all) continue;
        w->rho[c2] = neumann(m, w->rho, c1, c2);
        w->T[c2] = neumann(m, w->T, c1, c2);
        if (m->bcU[k] == 2) {
            sym_vec(w->U + 3 * (size_t)c1, m->fN + 3 * k, w->U + 3 * (size_t)c2);
        } else {
            for (int c = 0; c < 3; c++) {
                const double* a = m->cC + 3 * (size_t)c1;
                const double* b = m->cC + 3 * (size_t)c2;
                double dv[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
                w->U[3 * (size_t)c2 + c] = w->U[3 * (size_t)c1 + c] + 0.0 * vmag(dv);
            }
        }
    }
    /* equation of state on every node, then Neumann ghosts, then p' */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n_all; i++)
        w->p[i] = P0 * eos_pow(((w->rho[i] * w->T[i]) * R) / P0, gam);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n_slot; k++) {
        if (!m->bcU[k]) continue;
        uint32_t c1 = m->FO[k], c2 = m->FN[k];
        if (c2 >= (uint32_t)n_all) continue;
        w->p[c2] = neumann(m, w->p, c1, c2);
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n_all; i++) w->p[i] -= m->p_ref[i];
    if (p_out) memcpy(p_out, w->p, (size_t)n_all * sizeof(double));

    /* artificial viscosity (diffusion YES, euler.cpp:189-190, 232, 250):
     * mu = rho nu; strong-form gradients of U and theta, zero on wall ghosts */
    const int visc = m->nu != 0.0;
    const double iPr = visc ? 1 / m->Pr : 0.0;
    /* non-conforming faces (scatter_non_conforming / gather_non_conforming) */
    const int mort = m->n_mortar > 0;
    if (mort && !w->side) {
        const size_t na = (size_t)n_all + (size_t)NP;
        w->side = mortar_sides(m);
        w->mq = calloc((size_t)NQ_COUPLED * n_slot, sizeof(double));
        w->nq = calloc((size_t)NQ_COUPLED * na, sizeof(double));
        w->mF = calloc(15 * (size_t)n_slot, sizeof(double));
        w->mP = calloc(15 * (size_t)n_slot, sizeof(double));
        w->dC = calloc(5 * (size_t)n_slot, sizeof(double));
        w->gS = calloc(3 * (size_t)n_slot, sizeof(double));
        w->gC = calloc(3 * (size_t)n_slot, sizeof(double));
        w->gT = calloc(9 * (size_t)n_slot, sizeof(double));
    }
    const int8_t* side = w->side;
    if (visc) {
        for (int64_t i = 0; i < n_all; i++) w->mu[i] = w->rho[i] * m->nu;
        if (mort) mortar_cds(m, 3, w->U, side, w->gT, w->gS, w->gC);
        grad_strong(m, 3, w->U, w->GU, side, w->gS, w->gC);
        if (mort) mortar_cds(m, 1, w->T, side, w->gT, w->gS, w->gC);
        grad_strong(m, 1, w->T, w->GT, side, w->gS, w->gC);
    }

    const double gR = gam * R;
    if (mort) {
        /* the coarse sides' node quantities, interpolated onto every mortar slot */
        for (int64_t i = 0; i < n_int; i++) {
            double* q = w->nq + (size_t)NQ_COUPLED * i;
            const double* U = w->U + 3 * i;
            const double r = w->rho[i], T = w->T[i];
            q[0] = vmag(U);
            q[1] = sqrt(gR * T);
            for (int c = 0; c < 3; c++) q[2 + c] = U[c] * r;
            q[5] = r;
            double Fc[3] = {U[0] * r, U[1] * r, U[2] * r}, A[9];
            outer(Fc, U, A);
            for (int c = 0; c < 9; c++) {
                A[c] = A[c] + ((c < 3) ? 1.0 : 0.0) * w->p[i];
                if (visc) A[c] = A[c] - w->mu[i] * w->GU[9 * i + c];
                q[6 + c] = A[c];
            }
            for (int c = 0; c < 3; c++) {
                double a = (U[c] * r) * T;
                if (visc) a = a - (w->mu[i] * iPr) * w->GT[3 * i + c];
                q[15 + c] = a;
            }
            q[18] = r * T;
        }
        mortar_scatter(m, NQ_COUPLED, w->nq, w->mq);
    }
    /* face slots: Rusanov fluxes of the three equations dotted with fN */
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n_slot; k++) {
        uint32_t c1 = m->FO[k], c2 = m->FN[k];
        if (c1 >= (uint32_t)n_all || c2 >= (uint32_t)n_all) continue;
        const double fi = m->fI[k], fo = 1 - fi;
        const double* n = m->fN + 3 * k;
        const double mgn = vmag(n);
        const double en[3] = {n[0] / mgn, n[1] / mgn, n[2] / mgn};
        const double *U1 = w->U + 3 * (size_t)c1, *U2 = w->U + 3 * (size_t)c2;
        const double T1 = w->T[c1], T2 = w->T[c2];
        const double p1 = w->p[c1], p2 = w->p[c2];
        /* a mortar's coarse side (1: owner, 2: neighbour) takes interpolated values */
        const int ms = mort ? side[k] : 0;
        const double* mq = mort ? w->mq + (size_t)NQ_COUPLED * k : NULL;
        double r1 = w->rho[c1], r2 = w->rho[c2];
        double u1 = vmag(U1), u2 = vmag(U2), s1 = sqrt(gR * T1), s2 = sqrt(gR * T2);
        if (ms == 1) { u1 = mq[0]; s1 = mq[1]; r1 = mq[5]; }
        if (ms == 2) { u2 = mq[0]; s2 = mq[1]; r2 = mq[5]; }
        double lam = ((u1 * fi + u2 * fo) + (s1 * fi + s2 * fo)) / 2;
        /* rho: flux U*rho, state rho */
        {
            double F[3], jump = lam * (r2 - r1);
            for (int c = 0; c < 3; c++) {
                double a = U1[c] * w->rho[c1], b = U2[c] * w->rho[c2];
                if (ms == 1) a = mq[2 + c];
                if (ms == 2) b = mq[2 + c];
                F[c] = (a * fi + b * fo) - en[c] * jump;
            }
            w->d_rho[k] = vdot(F, n);
            if (ms)
                for (int c = 0; c < 3; c++) w->mF[15 * k + c] = F[c];
        }
        /* momentum: flux (rho U) (x) U + p' I, state rho U */
        {
            const double ra = w->rho[c1], rb = w->rho[c2];
            double Fc1[3] = {U1[0] * ra, U1[1] * ra, U1[2] * ra};
            double Fc2[3] = {U2[0] * rb, U2[1] * rb, U2[2] * rb};
            double T1t[9], T2t[9], F[9], O[9];
            outer(Fc1, U1, T1t);
            outer(Fc2, U2, T2t);
            for (int c = 0; c < 9; c++) {
                double i1 = (c < 3) ? 1.0 : 0.0;
                T1t[c] = T1t[c] + i1 * p1;
                T2t[c] = T2t[c] + i1 * p2;
            }
            if (visc) {
                const int g1 = c1 < (uint32_t)n_int, g2 = c2 < (uint32_t)n_int;
                for (int c = 0; c < 9; c++) {
                    T1t[c] = T1t[c] - w->mu[c1] * (g1 ? w->GU[9 * (size_t)c1 + c] : 0.0);
                    T2t[c] = T2t[c] - w->mu[c2] * (g2 ? w->GU[9 * (size_t)c2 + c] : 0.0);
                }
            }
            if (ms) {
                double* Tm = ms == 1 ? T1t : T2t;
                double* Fm = ms == 1 ? Fc1 : Fc2;
                for (int c = 0; c < 9; c++) Tm[c] = mq[6 + c];
                for (int c = 0; c < 3; c++) Fm[c] = mq[2 + c];
            }
            double dq[3];
            for (int c = 0; c < 3; c++) dq[c] = (Fc2[c] - Fc1[c]) * lam;
            outer(en, dq, O);
            for (int c = 0; c < 9; c++) F[c] = (T1t[c] * fi + T2t[c] * fo) - O[c];
            tdot(F, n, w->d_mom + 3 * k);
            if (ms)
                for (int c = 0; c < 9; c++) w->mF[15 * k + 3 + c] = F[c];
        }
        /* rho theta: flux (rho U) theta, state rho theta */
        {
            const double ra = w->rho[c1], rb = w->rho[c2];
            double q1 = ra * T1, q2 = rb * T2;
            if (ms == 1) q1 = mq[18];
            if (ms == 2) q2 = mq[18];
            double F[3], jump = lam * (q2 - q1);
            for (int c = 0; c < 3; c++) {
                double a = (U1[c] * ra) * T1, b = (U2[c] * rb) * T2;
                if (visc) {
                    a = a - (w->mu[c1] * iPr) * (c1 < (uint32_t)n_int ? w->GT[3 * (size_t)c1 + c] : 0.0);
                    b = b - (w->mu[c2] * iPr) * (c2 < (uint32_t)n_int ? w->GT[3 * (size_t)c2 + c] : 0.0);
                }
                if (ms == 1) a = mq[15 + c];
                if (ms == 2) b = mq[15 + c];
                F[c] = (a * fi + b * fo) - en[c] * jump;
            }
            w->d_th[k] = vdot(F, n);
            if (ms)
                for (int c = 0; c < 3; c++) w->mF[15 * k + 12 + c] = F[c];
        }
    }
    if (mort) {
        /* the coarse sides' lifted values: projected flux vectors dotted with
         * the slot's own weighted normal */
        mortar_gather(m, 15, w->mF, w->mP);
        for (int64_t k = 0; k < n_slot; k++) {
            if (!side[k]) continue;
            const double* P = w->mP + 15 * k;
            const double* n = m->fN + 3 * k;
            w->dC[5 * k] = vdot(P, n);
            tdot(P + 3, n, w->dC + 5 * k + 1);
            w->dC[5 * k + 4] = vdot(P + 12, n);
        }
    }

    /* surface lift (div_flux, weak form) then volume term, per element */
    const int64_t n_elem = m->n_elem;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < n_elem; e++) {
        const int64_t base = e * NP;
        for (int32_t a = 0; a < NP; a++) {
            w->r_rho[base + a] = 0.0;
            w->r_th[base + a] = 0.0;
            w->r_mom[3 * (base + a) + 0] = 0.0;
            w->r_mom[3 * (base + a) + 1] = 0.0;
            w->r_mom[3 * (base + a) + 2] = 0.0;
        }
        for (uint32_t f = m->face_idx0[e]; f < m->face_idx1[e]; f++) {
            for (int32_t nn = 0; nn < NPF; nn++) {
                int64_t k = (int64_t)m->all_faces[f] * NPF + nn;
                uint32_t c1 = m->FO[k], c2 = m->FN[k];
                if (c1 >= base && c1 < base + NP) {
                    if (side && side[k] == 1) {
                        const double* v = w->dC + 5 * k;
                        w->r_rho[c1] += v[0];
                        for (int c = 0; c < 3; c++) w->r_mom[3 * (size_t)c1 + c] += v[1 + c];
                        w->r_th[c1] += v[4];
                    } else {
                        w->r_rho[c1] += w->d_rho[k];
                        for (int c = 0; c < 3; c++) w->r_mom[3 * (size_t)c1 + c] += w->d_mom[3 * k + c];
                        w->r_th[c1] += w->d_th[k];
                    }
                } else if (c2 < (uint32_t)n_all) {
                    if (side && side[k] == 2) {
                        const double* v = w->dC + 5 * k;
                        w->r_rho[c2] -= v[0];
                        for (int c = 0; c < 3; c++) w->r_mom[3 * (size_t)c2 + c] -= v[1 + c];
                        w->r_th[c2] -= v[4];
                    } else {
                        w->r_rho[c2] -= w->d_rho[k];
                        for (int c = 0; c < 3; c++) w->r_mom[3 * (size_t)c2 + c] -= w->d_mom[3 * k + c];
                        w->r_th[c2] -= w->d_th[k];
                    }
                }
            }
        }
        /* volume term, scattered from node b to the nodes of its 3 lines */
        for (int32_t ii = 0; ii < NPX; ii++)
        for (int32_t jj = 0; jj < NPY; jj++)
        for (int32_t kk = 0; kk < NPZ; kk++) {
            const int64_t b = base + (int64_t)ii * NPY * NPZ + jj * NPZ + kk;
            double Jin[9];
            for (int c = 0; c < 9; c++) Jin[c] = m->Jinv[9 * b + c] * m->cV[b];
            const double rb = w->rho[b], Tb = w->T[b], pb = w->p[b];
            const double* Ub = w->U + 3 * b;
            double fr[3] = {Ub[0] * rb, Ub[1] * rb, Ub[2] * rb};    /* U*rho */
            double Fc[3] = {Ub[0] * rb, Ub[1] * rb, Ub[2] * rb};    /* rho*U */
            double fm[9];
            outer(Fc, Ub, fm);
            for (int c = 0; c < 9; c++) fm[c] = fm[c] + ((c < 3) ? 1.0 : 0.0) * pb;
            double ft[3] = {Fc[0] * Tb, Fc[1] * Tb, Fc[2] * Tb};
            if (visc) {
                for (int c = 0; c < 9; c++) fm[c] = fm[c] - w->mu[b] * w->GU[9 * b + c];
                for (int c = 0; c < 3; c++) ft[c] = ft[c] - (w->mu[b] * iPr) * w->GT[3 * b + c];
            }
            for (int pass = 0; pass < 3; pass++) {
                const int32_t lim = pass == 0 ? NPX : pass == 1 ? NPY : NPZ;
                for (int32_t q = 0; q < lim; q++) {
                    int32_t im = ii, jm = jj, km = kk;
                    if (pass == 0) im = q;
                    else if (pass == 1) { if (q == jj) continue; jm = q; }
                    else { if (q == kk) continue; km = q; }
                    const int64_t a = base + (int64_t)im * NPY * NPZ + jm * NPZ + km;
                    double dv[3], dj[3], t[3];
                    dv[0] = m->dpsi[0][ii * NPX + im] * m->psi[1][jj * NPY + jm] * m->psi[2][kk * NPZ + km];
                    dv[1] = m->psi[0][ii * NPX + im] * m->dpsi[1][jj * NPY + jm] * m->psi[2][kk * NPZ + km];
                    dv[2] = m->psi[0][ii * NPX + im] * m->psi[1][jj * NPY + jm] * m->dpsi[2][kk * NPZ + km];
                    tdot(Jin, dv, dj);
                    w->r_rho[a] -= vdot(fr, dj);
                    tdot(fm, dj, t);
                    w->r_mom[3 * a + 0] -= t[0];
                    w->r_mom[3 * a + 1] -= t[1];
                    w->r_mom[3 * a + 2] -= t[2];
                    w->r_th[a] -= vdot(ft, dj);
                }
            }
        }
    }
    /* momentum source: Su -= ((rho - rho_ref) g) cV */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n_int; i++) {
        double s = w->rho[i] - m->rho_ref[i];
        for (int c = 0; c < 3; c++) {
            double sc = 0.0 + m->gravity[c] * s;
            w->r_mom[3 * i + c] = w->r_mom[3 * i + c] - sc * m->cV[i];
        }
    }
}

static void tendency_w(const nsem_oracle_mesh* m, const double* const u[5],
                       double* const L[5], work_t* w, double* p_out) {
    residual(m, u, w, p_out);
    const int64_t n_int = m->n_int;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n_int; i++) {
        double cv = m->cV[i];
        L[0][i] = -(w->r_rho[i] / cv);
        L[1][i] = -(w->r_mom[3 * i + 0] / cv);
        L[2][i] = -(w->r_mom[3 * i + 1] / cv);
        L[3][i] = -(w->r_mom[3 * i + 2] / cv);
        L[4][i] = -(w->r_th[i] / cv);
    }
}

void nsem_oracle_tendency(const nsem_oracle_mesh* m, const double* const u[5],
                          double* const L[5], double* p_out) {
    work_t w;
    work_alloc(m, &w);
    tendency_w(m, u, L, &w, p_out);
    work_free(&w);
}

void nsem_oracle_ssprk3(const nsem_oracle_mesh* m, double* const u[5], double dt,
                        int nsteps) {
    const int64_t n = m->n_int;
    work_t w;
    work_alloc(m, &w);
    double *L[5], *s[5];
    for (int c = 0; c < 5; c++) {
        L[c] = malloc((size_t)n * sizeof(double));
        s[c] = malloc((size_t)n * sizeof(double));
    }
    const double a2 = 0.75, b2 = 0.25, a3 = 1.0 / 3.0, b3 = 2.0 / 3.0;
    for (int step = 0; step < nsteps; step++) {
        tendency_w(m, (const double* const*)u, L, &w, NULL);
        for (int c = 0; c < 5; c++) {
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) s[c][i] = u[c][i] + dt * L[c][i];
        }
        tendency_w(m, (const double* const*)s, L, &w, NULL);
        for (int c = 0; c < 5; c++) {
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) {
                double t = s[c][i] + dt * L[c][i];
                s[c][i] = a2 * u[c][i] + b2 * t;
            }
        }
        tendency_w(m, (const double* const*)s, L, &w, NULL);
        for (int c = 0; c < 5; c++) {
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) {
                double t = s[c][i] + dt * L[c][i];
                u[c][i] = a3 * u[c][i] + b3 * t;
            }
        }
    }
    for (int c = 0; c < 5; c++) { free(L[c]); free(s[c]); }
    work_free(&w);
}

void nsem_oracle_diagnostics(const nsem_oracle_mesh* m, const double* const u[5],
                             const double* gh, double cv_heat, double out[3]) {
    const double P0 = m->P0, R = m->R, cp = m->R + cv_heat;
    double mass = 0, energy = 0, vol = 0;
    work_t w;
    work_alloc(m, &w);
    residual(m, u, &w, NULL);
    for (int64_t i = 0; i < m->n_int; i++) {
        double rho = w.rho[i], cvn = m->cV[i];
        const double* U = w.U + 3 * i;
        mass += rho * cvn;
        double sf = gh[i] + 0.5 * vdot(U, U) +
                    pow((w.p[i] + m->p_ref[i]) / P0, R / cp) * w.T[i] * cv_heat;
        energy += rho * cvn * sf;
        vol += cvn;
    }
    work_free(&w);
    out[0] = mass; out[1] = energy; out[2] = vol;
}

/* ------------------------------------------------------------------------
 * The reference's own time update (apps/euler/euler.cpp:179-287 with
 * time_scheme BDF1, diffusion NO): segregated forward Euler over the
 * primitive fields.  Per step, on every node including the ghosts:
 *   T += T0; lambda from U^n, T^n; rho-eq with flux U rho^n, state rho^n;
 *   rho^{n+1} = Su/ap (ddt, field.h:3741-3841 BDF1: ap = (-1/dt) cV,
 *   Su += rho^n ap; SolveTexplicit, solve.cpp:563-564) and Neumann ghosts;
 *   p' from rho^{n+1}, T^n; U-eq with flux (rho^n U^n) (x) U^n + p' I, state
 *   rho^{n+1} U^n, source (rho^{n+1} - rho_ref) g; U^{n+1} = Su/ap with
 *   ap = (-1/dt) cV rho^{n+1}, Su += (U^n rho^n)(-1/dt) cV; symmetry ghosts;
 *   T-eq with flux (rho^n U^n) T^n, state rho^{n+1} T^n, the same update;
 *   T -= T0.
 * With diffusion YES the fluxes also carry the artificial viscosity
 * mu = rho^n nu: - mu grad U^n in the U equation and - (mu / Pr) grad theta^n in
 * the T equation, strong-form DG gradients (euler.cpp:189-190, 232, 250).
 * ------------------------------------------------------------------------ */

/* Non-conforming (2:1) faces of an adaptively refined mesh
 * (scatter_non_conforming / gather_non_conforming, field.h:2019-2248).  On a
 * mortar face the coarse cell's side of every face slot is the interpolation
 * of the coarse face's node values onto the (finer) mortar nodes with psiRef,
 * and the face values go back to the coarse face's nodes projected with
 * psiCor; the fine side is conforming. */
typedef struct {
    int64_t fi;          /* the face */
    int fm;              /* 1: the neighbour (FN) side is coarse, 2: the owner (FO) */
    int a, b, oa, ob;    /* in-plane axes of the coarse face (a < b) and halves */
    int fix_axis, fix;   /* its normal axis and node index along it */
    int64_t cbase;       /* first node of the coarse cell */
} mortar_geo;

static mortar_geo mortar_get(const nsem_oracle_mesh* m, int q) {
    mortar_geo g;
    const uint32_t* r = m->mortar + 4 * (size_t)q;
    const int npd[3] = {m->npx, m->npy, m->npz};
    const int fid = (int)r[2];
    g.fi = r[0];
    g.fm = (int)r[1];
    g.oa = (int)(r[3] & 1);
    g.ob = (int)((r[3] >> 1) & 1);
    if (fid <= 1) { g.a = 0; g.b = 1; g.fix_axis = 2; }
    else if (fid <= 3) { g.a = 0; g.b = 2; g.fix_axis = 1; }
    else { g.a = 1; g.b = 2; g.fix_axis = 0; }
    g.fix = (fid & 1) ? npd[g.fix_axis] - 1 : 0;
    const int64_t k0 = g.fi * m->npf;
    const uint32_t cnode = g.fm == 1 ? m->FN[k0] : m->FO[k0];
    g.cbase = (int64_t)(cnode / (uint32_t)m->np) * m->np;
    return g;
}

static int64_t mortar_node(const nsem_oracle_mesh* m, const mortar_geo* g, int na, int nb) {
    int idx[3];
    idx[g->a] = na;
    idx[g->b] = nb;
    idx[g->fix_axis] = g->fix;
    return g->cbase + ((int64_t)idx[0] * m->npy + idx[1]) * m->npz + idx[2];
}

/* per slot: 0 conforming, 1 the owner (FO) side is a mortar's coarse side,
 * 2 the neighbour (FN) side is */
static int8_t* mortar_sides(const nsem_oracle_mesh* m) {
    const int64_t n_slot = (int64_t)m->n_face * m->npf;
    int8_t* side = calloc((size_t)n_slot, 1);
    for (int q = 0; q < m->n_mortar; q++) {
        const mortar_geo g = mortar_get(m, q);
        for (int32_t n = 0; n < m->npf; n++) side[g.fi * m->npf + n] = (int8_t)(g.fm == 2 ? 1 : 2);
    }
    return side;
}

/* coarse-side value of the node quantity Q (ncomp per node) at every slot of
 * every mortar face: sum over the coarse face nodes of Q psiRef_a psiRef_b */
static void mortar_scatter(const nsem_oracle_mesh* m, int ncomp, const double* Q, double* out) {
    const int npd[3] = {m->npx, m->npy, m->npz};
    if (ncomp > 32) abort();
    for (int q = 0; q < m->n_mortar; q++) {
        const mortar_geo g = mortar_get(m, q);
        const int Na = npd[g.a], Nb = npd[g.b];
        const double* Pa = m->psi_ref[g.a * 2 + g.oa];
        const double* Pb = m->psi_ref[g.b * 2 + g.ob];
        for (int ia = 0; ia < Na; ia++)
            for (int ib = 0; ib < Nb; ib++) {
                double sum[32] = {0};
                for (int na = 0; na < Na; na++)
                    for (int nb = 0; nb < Nb; nb++) {
                        const double* v = Q + (size_t)ncomp * mortar_node(m, &g, na, nb);
                        const double fa = Pa[na * Na + ia], fb = Pb[nb * Nb + ib];
                        for (int c = 0; c < ncomp; c++) sum[c] += v[c] * fa * fb;
                    }
                const int64_t k = g.fi * m->npf + (int64_t)ia * Nb + ib;
                for (int c = 0; c < ncomp; c++) out[(size_t)ncomp * k + c] = sum[c];
            }
    }
}

/* face values F (ncomp per slot) of every mortar face projected onto the
 * coarse face's nodes: out at slot (na, nb) = sum over the mortar slots of
 * F psiCor_a psiCor_b */
static void mortar_gather(const nsem_oracle_mesh* m, int ncomp, const double* F, double* out) {
    const int npd[3] = {m->npx, m->npy, m->npz};
    if (ncomp > 32) abort();
    for (int q = 0; q < m->n_mortar; q++) {
        const mortar_geo g = mortar_get(m, q);
        const int Na = npd[g.a], Nb = npd[g.b];
        const double* Pa = m->psi_cor[g.a * 2 + g.oa];
        const double* Pb = m->psi_cor[g.b * 2 + g.ob];
        const int64_t k0 = g.fi * m->npf;
        for (int na = 0; na < Na; na++)
            for (int nb = 0; nb < Nb; nb++) {
                double sum[32] = {0};
                for (int ia = 0; ia < Na; ia++)
                    for (int ib = 0; ib < Nb; ib++) {
                        const double* v = F + (size_t)ncomp * (k0 + (int64_t)ia * Nb + ib);
                        const double fa = Pa[ia * Na + na], fb = Pb[ib * Nb + nb];
                        for (int c = 0; c < ncomp; c++) sum[c] += v[c] * fa * fb;
                    }
                const int64_t k = k0 + (int64_t)na * Nb + nb;
                for (int c = 0; c < ncomp; c++) out[(size_t)ncomp * k + c] = sum[c];
            }
    }
}

/* ghosts of a scalar (Neumann) and of the velocity (per slot BC) */
static void ghosts_scalar(const nsem_oracle_mesh* m, double* f) {
    const int64_t n_slot = (int64_t)m->n_face * m->npf;
    for (int64_t k = 0; k < n_slot; k++) {
        if (!m->bcU[k]) continue;
        uint32_t c1 = m->FO[k], c2 = m->FN[k];
        if (c2 >= (uint32_t)m->n_all) continue;
        f[c2] = neumann(m, f, c1, c2);
    }
}

static void ghosts_velocity(const nsem_oracle_mesh* m, double* U) {
    const int64_t n_slot = (int64_t)m->n_face * m->npf;
    for (int64_t k = 0; k < n_slot; k++) {
        if (!m->bcU[k]) continue;
        uint32_t c1 = m->FO[k], c2 = m->FN[k];
        if (c2 >= (uint32_t)m->n_all) continue;
        if (m->bcU[k] == 2) {
            sym_vec(U + 3 * (size_t)c1, m->fN + 3 * k, U + 3 * (size_t)c2);
        } else {
            const double* a = m->cC + 3 * (size_t)c1;
            const double* b = m->cC + 3 * (size_t)c2;
            double dv[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
            for (int c = 0; c < 3; c++)
                U[3 * (size_t)c2 + c] = U[3 * (size_t)c1 + c] + 0.0 * vmag(dv);
        }
    }
}

/* weak divergence Su of one equation (field.h:3417-3478): lift of the per-slot
 * fluxes d (ncomp per slot) in the cell's face order, then the volume term of
 * the nodal flux F (ncomp x 3 per node: Vector flux for ncomp 1, Tensor for 3) */
static void seg_divf(const nsem_oracle_mesh* m, int ncomp, const double* F, const double* d,
                     const int8_t* side, const double* dC, double* r) {
    const int32_t NPX = m->npx, NPY = m->npy, NPZ = m->npz, NP = m->np, NPF = m->npf;
    const int64_t n_all = m->n_all;
    const int w = ncomp == 1 ? 3 : 9;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m->n_elem; e++) {
        const int64_t base = e * NP;
        for (int32_t a = 0; a < NP; a++)
            for (int c = 0; c < ncomp; c++) r[ncomp * (base + a) + c] = 0.0;
        for (uint32_t f = m->face_idx0[e]; f < m->face_idx1[e]; f++) {
            for (int32_t nn = 0; nn < NPF; nn++) {
                int64_t k = (int64_t)m->all_faces[f] * NPF + nn;
                uint32_t c1 = m->FO[k], c2 = m->FN[k];
                /* a mortar's coarse side takes the projected face value */
                if (c1 >= base && c1 < base + NP) {
                    const double* v = (side && side[k] == 1) ? dC : d;
                    for (int c = 0; c < ncomp; c++) r[ncomp * (size_t)c1 + c] += v[ncomp * k + c];
                } else if (c2 < (uint32_t)n_all) {
                    const double* v = (side && side[k] == 2) ? dC : d;
                    for (int c = 0; c < ncomp; c++) r[ncomp * (size_t)c2 + c] -= v[ncomp * k + c];
                }
            }
        }
        for (int32_t ii = 0; ii < NPX; ii++)
        for (int32_t jj = 0; jj < NPY; jj++)
        for (int32_t kk = 0; kk < NPZ; kk++) {
            const int64_t b = base + (int64_t)ii * NPY * NPZ + jj * NPZ + kk;
            double Jin[9];
            for (int c = 0; c < 9; c++) Jin[c] = m->Jinv[9 * b + c] * m->cV[b];
            const double* Fb = F + (size_t)w * b;
            for (int pass = 0; pass < 3; pass++) {
                const int32_t lim = pass == 0 ? NPX : pass == 1 ? NPY : NPZ;
                for (int32_t q = 0; q < lim; q++) {
                    int32_t im = ii, jm = jj, km = kk;
                    if (pass == 0) im = q;
                    else if (pass == 1) { if (q == jj) continue; jm = q; }
                    else { if (q == kk) continue; km = q; }
                    const int64_t a = base + (int64_t)im * NPY * NPZ + jm * NPZ + km;
                    double dv[3], dj[3];
                    dv[0] = m->dpsi[0][ii * NPX + im] * m->psi[1][jj * NPY + jm] * m->psi[2][kk * NPZ + km];
                    dv[1] = m->psi[0][ii * NPX + im] * m->dpsi[1][jj * NPY + jm] * m->psi[2][kk * NPZ + km];
                    dv[2] = m->psi[0][ii * NPX + im] * m->psi[1][jj * NPY + jm] * m->dpsi[2][kk * NPZ + km];
                    tdot(Jin, dv, dj);
                    if (ncomp == 1) {
                        r[a] -= vdot(Fb, dj);
                    } else {
                        double t[3];
                        tdot(Fb, dj, t);
                        r[3 * a + 0] -= t[0];
                        r[3 * a + 1] -= t[1];
                        r[3 * a + 2] -= t[2];
                    }
                }
            }
        }
    }
}

/* strong-form DG gradient per unit volume (gradf<true>, field.h:3327-3360 with
 * grad_flux<true>, field.h:3050-3083): face terms fN (x) (cds(p) - p) in the
 * cell's face order, then the volume derivative at the node from its three
 * lines, divided by cV; ncomp 1 (Scalar -> Vector) or 3 (Vector -> Tensor in
 * XX..ZX order, G[r][c] = d_r p_c).  Interior nodes only: the ghosts' gradient
 * is set to zero on every wall (fillBCs, field.h:2731-2769). */
static void grad_strong(const nsem_oracle_mesh* m, int ncomp, const double* p, double* G,
                        const int8_t* side, const double* fS, const double* fC) {
    const int32_t NPX = m->npx, NPY = m->npy, NPZ = m->npz, NP = m->np, NPF = m->npf;
    const int64_t n_all = m->n_all;
    const int w = ncomp == 1 ? 3 : 9;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m->n_elem; e++) {
        const int64_t base = e * NP;
        for (int32_t a = 0; a < NP; a++)
            for (int c = 0; c < w; c++) G[(size_t)w * (base + a) + c] = 0.0;
        for (uint32_t f = m->face_idx0[e]; f < m->face_idx1[e]; f++) {
            for (int32_t nn = 0; nn < NPF; nn++) {
                const int64_t k = (int64_t)m->all_faces[f] * NPF + nn;
                const uint32_t c1 = m->FO[k], c2 = m->FN[k];
                if (c1 >= (uint32_t)n_all || c2 >= (uint32_t)n_all) continue;
                const double fi = m->fI[k], fo = 1 - fi;
                const double* n = m->fN + 3 * k;
                uint32_t own;
                double sg;
                if (c1 >= base && c1 < base + NP) { own = c1; sg = 1.0; }
                else { own = c2; sg = -1.0; }
                double fF[3];
                if (side && side[k]) {
                    /* mortar: cds with the coarse side interpolated, projected
                     * back onto the coarse side's nodes */
                    const int coarse = (side[k] == 1) == (sg > 0);
                    for (int c = 0; c < ncomp; c++) fF[c] = (coarse ? fC : fS)[(size_t)ncomp * k + c];
                } else {
                    for (int c = 0; c < ncomp; c++)
                        fF[c] = (p[(size_t)ncomp * c1 + c] * fi) + (p[(size_t)ncomp * c2 + c] * fo);
                }
                double d[3], t[9];
                for (int c = 0; c < ncomp; c++) d[c] = fF[c] - p[(size_t)ncomp * own + c];
                if (ncomp == 1) {
                    for (int r = 0; r < 3; r++) t[r] = n[r] * d[0];
                } else {
                    outer(n, d, t);
                }
                double* g = G + (size_t)w * own;
                if (sg > 0) for (int c = 0; c < w; c++) g[c] += t[c];
                else for (int c = 0; c < w; c++) g[c] -= t[c];
            }
        }
        for (int32_t ii = 0; ii < NPX; ii++)
        for (int32_t jj = 0; jj < NPY; jj++)
        for (int32_t kk = 0; kk < NPZ; kk++) {
            const int64_t a = base + (int64_t)ii * NPY * NPZ + jj * NPZ + kk;
            double Jin[9];
            for (int c = 0; c < 9; c++) Jin[c] = m->Jinv[9 * a + c] * m->cV[a];
            double* g = G + (size_t)w * a;
            for (int pass = 0; pass < 3; pass++) {
                const int32_t lim = pass == 0 ? NPX : pass == 1 ? NPY : NPZ;
                for (int32_t q = 0; q < lim; q++) {
                    int32_t im = ii, jm = jj, km = kk;
                    if (pass == 0) im = q;
                    else if (pass == 1) { if (q == jj) continue; jm = q; }
                    else { if (q == kk) continue; km = q; }
                    const int64_t b = base + (int64_t)im * NPY * NPZ + jm * NPZ + km;
                    double dv[3], dj[3], t[9];
                    dv[0] = m->dpsi[0][ii * NPX + im] * m->psi[1][jj * NPY + jm] * m->psi[2][kk * NPZ + km];
                    dv[1] = m->psi[0][ii * NPX + im] * m->dpsi[1][jj * NPY + jm] * m->psi[2][kk * NPZ + km];
                    dv[2] = m->psi[0][ii * NPX + im] * m->psi[1][jj * NPY + jm] * m->dpsi[2][kk * NPZ + km];
                    tdot(Jin, dv, dj);
                    if (ncomp == 1) {
                        for (int r = 0; r < 3; r++) t[r] = dj[r] * p[b];
                    } else {
                        outer(dj, p + 3 * (size_t)b, t);
                    }
                    for (int c = 0; c < w; c++) g[c] += t[c];
                }
            }
            for (int c = 0; c < w; c++) g[c] = g[c] / m->cV[a];
        }
    }
}

/* cds of a node quantity p (ncomp per node) on every mortar slot with the
 * coarse side interpolated (fS), and fS projected back onto the coarse side
 * (fC): the face values the strong-form gradient lifts on mortar faces */
static void mortar_cds(const nsem_oracle_mesh* m, int ncomp, const double* p, const int8_t* side,
                       double* tmp, double* fS, double* fC) {
    const int64_t n_slot = (int64_t)m->n_face * m->npf;
    mortar_scatter(m, ncomp, p, tmp);
    for (int64_t k = 0; k < n_slot; k++) {
        if (!side[k]) continue;
        const uint32_t c1 = m->FO[k], c2 = m->FN[k];
        if (c1 >= (uint32_t)m->n_all || c2 >= (uint32_t)m->n_all) continue;
        const double fi = m->fI[k], fo = 1 - fi;
        for (int c = 0; c < ncomp; c++) {
            const double a = side[k] == 1 ? tmp[(size_t)ncomp * k + c] : p[(size_t)ncomp * c1 + c];
            const double b = side[k] == 2 ? tmp[(size_t)ncomp * k + c] : p[(size_t)ncomp * c2 + c];
            fS[(size_t)ncomp * k + c] = (a * fi) + (b * fo);
        }
    }
    mortar_gather(m, ncomp, fS, fC);
}

void nsem_oracle_segregated(const nsem_oracle_mesh* m, double* rho_in, double* U_in, double* T_in,
                            double dt, int nsteps) {
    const int64_t n_int = m->n_int, n_all = m->n_all;
    const int64_t n_slot = (int64_t)m->n_face * m->npf;
    const size_t na = (size_t)n_all + (size_t)m->np;
    const double P0 = m->P0, R = m->R, gam = m->gamma, T0 = m->T0;
    double* rho = calloc(na, sizeof(double));
    double* rhof = calloc(na, sizeof(double));
    double* U = calloc(3 * na, sizeof(double));
    double* T = calloc(na, sizeof(double));
    double* p = calloc(na, sizeof(double));
    double* lam = calloc((size_t)n_slot, sizeof(double));
    double* Fv = calloc(9 * na, sizeof(double));
    double* q = calloc(3 * na, sizeof(double));
    double* d = calloc(3 * (size_t)n_slot, sizeof(double));
    double* r = calloc(3 * na, sizeof(double));
    double* Fc = calloc(3 * na, sizeof(double));
    const int visc = m->nu != 0.0;
    double* mu = visc ? calloc(na, sizeof(double)) : NULL;
    double* G = visc ? calloc(9 * na, sizeof(double)) : NULL;
    const double iPr = visc ? 1 / m->Pr : 0.0;
    /* non-conforming faces: coarse-side values per slot (ms*), face flux
     * vectors on mortar slots (mF), their projection (mP), lifted values (dC) */
    const int mort = m->n_mortar > 0;
    int8_t* side = mort ? mortar_sides(m) : NULL;
    double* nq = mort ? calloc(2 * na, sizeof(double)) : NULL;   /* per node |U|, c; rho theta */
    double* ms = mort ? calloc(9 * (size_t)n_slot, sizeof(double)) : NULL;
    double* ms2 = mort ? calloc(3 * (size_t)n_slot, sizeof(double)) : NULL;
    double* mF = mort ? calloc(9 * (size_t)n_slot, sizeof(double)) : NULL;
    double* mP = mort ? calloc(9 * (size_t)n_slot, sizeof(double)) : NULL;
    double* dC = mort ? calloc(3 * (size_t)n_slot, sizeof(double)) : NULL;
    double* gS = (mort && visc) ? calloc(3 * (size_t)n_slot, sizeof(double)) : NULL;
    double* gC = (mort && visc) ? calloc(3 * (size_t)n_slot, sizeof(double)) : NULL;
    /* the coarse side of a mortar slot: 1 = FO, 2 = FN */
#define SIDE(k) (mort ? side[k] : 0)
    memcpy(rho, rho_in, (size_t)n_int * sizeof(double));
    memcpy(U, U_in, 3 * (size_t)n_int * sizeof(double));
    memcpy(T, T_in, (size_t)n_int * sizeof(double));
    ghosts_scalar(m, rho);
    ghosts_velocity(m, U);
    ghosts_scalar(m, T);
    const double c_dt = -1.0 / dt;
    for (int step = 0; step < nsteps; step++) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n_all; i++) T[i] += T0;
        memcpy(rhof, rho, (size_t)n_all * sizeof(double));
        /* artificial viscosity mu = rho nu (euler.cpp:189-190) */
        if (visc)
            for (int64_t i = 0; i < n_all; i++) mu[i] = rho[i] * m->nu;
        /* Fc = flxc(rho U), lambda = (cds|U| + cds sqrt(gamma R T)) / 2 */
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n_all; i++)
            for (int c = 0; c < 3; c++) Fc[3 * i + c] = rho[i] * U[3 * i + c];
        const double gR = gam * R;
        if (mort) {
            for (int64_t i = 0; i < n_all; i++) {
                nq[2 * i] = vmag(U + 3 * i);
                nq[2 * i + 1] = sqrt(gR * T[i]);
            }
            mortar_scatter(m, 2, nq, ms);
        }
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < n_slot; k++) {
            uint32_t c1 = m->FO[k], c2 = m->FN[k];
            if (c1 >= (uint32_t)n_all || c2 >= (uint32_t)n_all) continue;
            const double fi = m->fI[k], fo = 1 - fi;
            double u1 = vmag(U + 3 * (size_t)c1), u2 = vmag(U + 3 * (size_t)c2);
            double s1 = sqrt(gR * T[c1]), s2 = sqrt(gR * T[c2]);
            if (SIDE(k) == 1) { u1 = ms[2 * k]; s1 = ms[2 * k + 1]; }
            if (SIDE(k) == 2) { u2 = ms[2 * k]; s2 = ms[2 * k + 1]; }
            lam[k] = ((u1 * fi + u2 * fo) + (s1 * fi + s2 * fo)) / 2;
        }
        /* rho equation: flux U rho, state rho */
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n_all; i++)
            for (int c = 0; c < 3; c++) Fv[3 * i + c] = U[3 * i + c] * rho[i];
        if (mort) {
            mortar_scatter(m, 3, Fv, ms);
            mortar_scatter(m, 1, rho, ms2);
        }
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < n_slot; k++) {
            uint32_t c1 = m->FO[k], c2 = m->FN[k];
            if (c1 >= (uint32_t)n_all || c2 >= (uint32_t)n_all) continue;
            const double fi = m->fI[k], fo = 1 - fi;
            const double* n = m->fN + 3 * k;
            const double mgn = vmag(n);
            const double en[3] = {n[0] / mgn, n[1] / mgn, n[2] / mgn};
            const double* F1 = Fv + 3 * (size_t)c1;
            const double* F2 = Fv + 3 * (size_t)c2;
            double r1 = rho[c1], r2 = rho[c2];
            if (SIDE(k) == 1) { F1 = ms + 3 * k; r1 = ms2[k]; }
            if (SIDE(k) == 2) { F2 = ms + 3 * k; r2 = ms2[k]; }
            double F[3], jump = lam[k] * (r2 - r1);
            for (int c = 0; c < 3; c++) F[c] = (F1[c] * fi + F2[c] * fo) - en[c] * jump;
            d[k] = vdot(F, n);
            if (SIDE(k))
                for (int c = 0; c < 3; c++) mF[3 * k + c] = F[c];
        }
        if (mort) {
            mortar_gather(m, 3, mF, mP);
            for (int64_t k = 0; k < n_slot; k++)
                if (side[k]) dC[k] = vdot(mP + 3 * k, m->fN + 3 * k);
        }
        seg_divf(m, 1, Fv, d, side, dC, r);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n_int; i++) {
            const double ap = c_dt * m->cV[i];
            rho[i] = (r[i] + rho[i] * ap) / (0.0 + ap);
        }
        ghosts_scalar(m, rho);
        /* p' from the new rho and the old theta */
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n_all; i++) p[i] = P0 * eos_pow(((rho[i] * T[i]) * R) / P0, gam);
        ghosts_scalar(m, p);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n_all; i++) p[i] -= m->p_ref[i];
        /* U equation: flux Fc (x) U + p' I - mu grad U, state rho U */
        if (visc) {
            if (mort) mortar_cds(m, 3, U, side, mP, gS, gC);
            grad_strong(m, 3, U, G, side, gS, gC);
        }
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n_all; i++) {
            double* Ft = Fv + 9 * i;
            outer(Fc + 3 * i, U + 3 * i, Ft);
            for (int c = 0; c < 9; c++) Ft[c] = Ft[c] + ((c < 3) ? 1.0 : 0.0) * p[i];
            if (visc) {
                /* the ghosts' gradient is zero on the walls */
                const double* g = G + 9 * i;
                for (int c = 0; c < 9; c++) Ft[c] = Ft[c] - mu[i] * (i < n_int ? g[c] : 0.0);
            }
            for (int c = 0; c < 3; c++) q[3 * i + c] = rho[i] * U[3 * i + c];
        }
        if (mort) {
            mortar_scatter(m, 9, Fv, ms);
            mortar_scatter(m, 3, q, ms2);
        }
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < n_slot; k++) {
            uint32_t c1 = m->FO[k], c2 = m->FN[k];
            if (c1 >= (uint32_t)n_all || c2 >= (uint32_t)n_all) continue;
            const double fi = m->fI[k], fo = 1 - fi;
            const double* n = m->fN + 3 * k;
            const double mgn = vmag(n);
            const double en[3] = {n[0] / mgn, n[1] / mgn, n[2] / mgn};
            const double* A1 = Fv + 9 * (size_t)c1;
            const double* A2 = Fv + 9 * (size_t)c2;
            const double* q1 = q + 3 * (size_t)c1;
            const double* q2 = q + 3 * (size_t)c2;
            if (SIDE(k) == 1) { A1 = ms + 9 * k; q1 = ms2 + 3 * k; }
            if (SIDE(k) == 2) { A2 = ms + 9 * k; q2 = ms2 + 3 * k; }
            double dq[3], O[9], F[9];
            for (int c = 0; c < 3; c++) dq[c] = (q2[c] - q1[c]) * lam[k];
            outer(en, dq, O);
            for (int c = 0; c < 9; c++) F[c] = (A1[c] * fi + A2[c] * fo) - O[c];
            tdot(F, n, d + 3 * k);
            if (SIDE(k))
                for (int c = 0; c < 9; c++) mF[9 * k + c] = F[c];
        }
        if (mort) {
            mortar_gather(m, 9, mF, mP);
            for (int64_t k = 0; k < n_slot; k++)
                if (side[k]) tdot(mP + 9 * k, m->fN + 3 * k, dC + 3 * k);
        }
        seg_divf(m, 3, Fv, d, side, dC, r);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n_int; i++) {
            const double s = rho[i] - m->rho_ref[i];
            const double ap0 = c_dt * m->cV[i];
            const double ap = ap0 * rho[i];
            for (int c = 0; c < 3; c++) {
                const double sc = 0.0 + m->gravity[c] * s;
                const double su = r[3 * i + c] - sc * m->cV[i];
                U[3 * i + c] = (su + (U[3 * i + c] * rhof[i]) * ap0) / (0.0 + ap);
            }
        }
        ghosts_velocity(m, U);
        /* T equation: flux Fc T - (mu / Pr) grad T, state rho T (U no longer enters) */
        if (visc) {
            if (mort) mortar_cds(m, 1, T, side, mP, gS, gC);
            grad_strong(m, 1, T, G, side, gS, gC);
        }
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n_all; i++)
            for (int c = 0; c < 3; c++) {
                Fv[3 * i + c] = Fc[3 * i + c] * T[i];
                if (visc)
                    Fv[3 * i + c] = Fv[3 * i + c] - (mu[i] * iPr) * (i < n_int ? G[3 * i + c] : 0.0);
            }
        if (mort) {
            for (int64_t i = 0; i < n_all; i++) nq[i] = rho[i] * T[i];
            mortar_scatter(m, 3, Fv, ms);
            mortar_scatter(m, 1, nq, ms2);
        }
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < n_slot; k++) {
            uint32_t c1 = m->FO[k], c2 = m->FN[k];
            if (c1 >= (uint32_t)n_all || c2 >= (uint32_t)n_all) continue;
            const double fi = m->fI[k], fo = 1 - fi;
            const double* n = m->fN + 3 * k;
            const double mgn = vmag(n);
            const double en[3] = {n[0] / mgn, n[1] / mgn, n[2] / mgn};
            const double* F1 = Fv + 3 * (size_t)c1;
            const double* F2 = Fv + 3 * (size_t)c2;
            double s1 = rho[c1] * T[c1], s2 = rho[c2] * T[c2];
            if (SIDE(k) == 1) { F1 = ms + 3 * k; s1 = ms2[k]; }
            if (SIDE(k) == 2) { F2 = ms + 3 * k; s2 = ms2[k]; }
            double F[3], jump = lam[k] * (s2 - s1);
            for (int c = 0; c < 3; c++) F[c] = (F1[c] * fi + F2[c] * fo) - en[c] * jump;
            d[k] = vdot(F, n);
            if (SIDE(k))
                for (int c = 0; c < 3; c++) mF[3 * k + c] = F[c];
        }
        if (mort) {
            mortar_gather(m, 3, mF, mP);
            for (int64_t k = 0; k < n_slot; k++)
                if (side[k]) dC[k] = vdot(mP + 3 * k, m->fN + 3 * k);
        }
        seg_divf(m, 1, Fv, d, side, dC, r);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n_int; i++) {
            const double ap0 = c_dt * m->cV[i];
            const double ap = ap0 * rho[i];
            T[i] = (r[i] + (T[i] * rhof[i]) * ap0) / (0.0 + ap);
        }
        ghosts_scalar(m, T);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n_all; i++) T[i] -= T0;
    }
#undef SIDE
    memcpy(rho_in, rho, (size_t)n_int * sizeof(double));
    memcpy(U_in, U, 3 * (size_t)n_int * sizeof(double));
    memcpy(T_in, T, (size_t)n_int * sizeof(double));
    free(rho); free(rhof); free(U); free(T); free(p); free(lam); free(Fv); free(q); free(d);
    free(r); free(Fc);
    free(mu); free(G);
    free(side); free(nq); free(ms); free(ms2); free(mF); free(mP); free(dC); free(gS); free(gC);
}

/* The reference's scalar DG convection (apps/convection/convection.cpp with
 * problem_init NONE and BDF1): a fixed wind U, Fc = flxc(U) = U,
 * lambda = cds(|U|)/2 (convection.cpp:106-108); per step the flux Fc T with the
 * Rusanov state T, T^{n+1} = Su/ap with ap = (-1/dt) cV and Su += T^n ap
 * (addTemporal<1> without density), Neumann ghosts of T. */
static void convection_core(const nsem_oracle_mesh* m, const double* U_in, const double* U_all,
                            const double* scale, int order, double* T_in, double dt, int nsteps) {
    const int64_t n_int = m->n_int, n_all = m->n_all;
    const int64_t n_slot = (int64_t)m->n_face * m->npf;
    const size_t na = (size_t)n_all + (size_t)m->np;
    double* U = calloc(3 * na, sizeof(double));
    double* T = calloc(na, sizeof(double));
    double* Fv = calloc(3 * na, sizeof(double));
    double* lam = calloc((size_t)n_slot, sizeof(double));
    double* d = calloc((size_t)n_slot, sizeof(double));
    double* r = calloc(na, sizeof(double));
    double* r0 = order == 2 ? calloc(na, sizeof(double)) : NULL;  /* previous rhs (AB2) */
    if (U_all) {
        /* the app's analytic wind: every cell node, ghosts included, from
         * the node coordinates (convection.cpp:64-93 loops over the whole
         * cell field) */
        memcpy(U, U_all, 3 * (size_t)n_all * sizeof(double));
    } else {
        memcpy(U, U_in, 3 * (size_t)n_int * sizeof(double));
        ghosts_velocity(m, U);
    }
    memcpy(T, T_in, (size_t)n_int * sizeof(double));
    ghosts_scalar(m, T);
    /* non-conforming faces: coarse side interpolated, fluxes projected back */
    const int mort = m->n_mortar > 0;
    int8_t* side = mort ? mortar_sides(m) : NULL;
    double* nq = mort ? calloc(4 * na, sizeof(double)) : NULL;
    double* ms = mort ? calloc(4 * (size_t)n_slot, sizeof(double)) : NULL;
    double* mF = mort ? calloc(3 * (size_t)n_slot, sizeof(double)) : NULL;
    double* mP = mort ? calloc(3 * (size_t)n_slot, sizeof(double)) : NULL;
    double* dC = mort ? calloc((size_t)n_slot, sizeof(double)) : NULL;
    const double c_dt = -1.0 / dt;
    for (int step = 0; step < nsteps; step++) {
        if (U_all || step == 0) {
            /* the wind of this step (U = U(x) cos(pi t / T) for the app's
             * analytic winds: the product with the step's factor in the
             * horizontal components, in the app's operation order; w = 0 as
             * the app sets it) and its Rusanov speed cds(|U|)/2 */
            if (U_all && scale) {
#pragma omp parallel for schedule(static)
                for (int64_t i = 0; i < n_all; i++) {
                    U[3 * i] = U_all[3 * i] * scale[step];
                    U[3 * i + 1] = U_all[3 * i + 1] * scale[step];
                    U[3 * i + 2] = U_all[3 * i + 2];
                }
            }
            if (mort) {
                for (int64_t i = 0; i < n_int; i++) nq[i] = vmag(U + 3 * i);
                mortar_scatter(m, 1, nq, ms);
            }
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < n_slot; k++) {
                uint32_t c1 = m->FO[k], c2 = m->FN[k];
                if (c1 >= (uint32_t)n_all || c2 >= (uint32_t)n_all) continue;
                const double fi = m->fI[k], fo = 1 - fi;
                double u1 = vmag(U + 3 * (size_t)c1), u2 = vmag(U + 3 * (size_t)c2);
                if (mort && side[k] == 1) u1 = ms[k];
                if (mort && side[k] == 2) u2 = ms[k];
                lam[k] = (u1 * fi + u2 * fo) / 2;
            }
        }
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n_all; i++)
            for (int c = 0; c < 3; c++) Fv[3 * i + c] = U[3 * i + c] * T[i];
        if (mort) {
            for (int64_t i = 0; i < n_int; i++) {
                for (int c = 0; c < 3; c++) nq[4 * i + c] = Fv[3 * i + c];
                nq[4 * i + 3] = T[i];
            }
            mortar_scatter(m, 4, nq, ms);
        }
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < n_slot; k++) {
            uint32_t c1 = m->FO[k], c2 = m->FN[k];
            if (c1 >= (uint32_t)n_all || c2 >= (uint32_t)n_all) continue;
            const double fi = m->fI[k], fo = 1 - fi;
            const double* n = m->fN + 3 * k;
            const double mgn = vmag(n);
            const double en[3] = {n[0] / mgn, n[1] / mgn, n[2] / mgn};
            const double* F1 = Fv + 3 * (size_t)c1;
            const double* F2 = Fv + 3 * (size_t)c2;
            double T1 = T[c1], T2 = T[c2];
            const int sd = mort ? side[k] : 0;
            if (sd == 1) { F1 = ms + 4 * k; T1 = ms[4 * k + 3]; }
            if (sd == 2) { F2 = ms + 4 * k; T2 = ms[4 * k + 3]; }
            double F[3], jump = lam[k] * (T2 - T1);
            for (int c = 0; c < 3; c++) F[c] = (F1[c] * fi + F2[c] * fo) - en[c] * jump;
            d[k] = vdot(F, n);
            if (sd)
                for (int c = 0; c < 3; c++) mF[3 * k + c] = F[c];
        }
        if (mort) {
            mortar_gather(m, 3, mF, mP);
            for (int64_t k = 0; k < n_slot; k++)
                if (side[k]) dC[k] = vdot(mP + 3 * k, m->fN + 3 * k);
        }
        seg_divf(m, 1, Fv, d, side, dC, r);
        if (order == 2 && step > 0) {
            /* AB2 (field.h:3796-3798): Su = T ap + (3 R^n - R^{n-1}) / 2, T = Su / ap */
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n_int; i++) {
                const double ap = c_dt * m->cV[i];
                const double rn = r[i];
                T[i] = (T[i] * ap + (3.0 * rn - r0[i]) / 2.0) / ap;
                r0[i] = rn;
            }
        } else {
            /* BDF1 / AB1 (the first AB2 step): T = (R + T ap) / ap */
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n_int; i++) {
                const double ap = c_dt * m->cV[i];
                if (r0) r0[i] = r[i];
                T[i] = (r[i] + T[i] * ap) / (0.0 + ap);
            }
        }
        ghosts_scalar(m, T);
    }
    memcpy(T_in, T, (size_t)n_int * sizeof(double));
    free(U); free(T); free(Fv); free(lam); free(d); free(r);
    free(side); free(nq); free(ms); free(mF); free(mP); free(dC); free(r0);
}

void nsem_oracle_convection(const nsem_oracle_mesh* m, const double* U_in, double* T_in, double dt,
                            int nsteps) {
    convection_core(m, U_in, NULL, NULL, 1, T_in, dt, nsteps);
}

/* The convection app with an analytic wind (problem_init LEVEQUE,
 * convection.cpp:45-93, 103-123): U_all [n_all*3] is the wind's spatial part
 * on every node (ghosts included) and scale[step] its time factor
 * cos(pi t / T), multiplied into the first two components in the app's
 * order; order 1 = BDF1/AB1, 2 = AB2 (the first step AB1). */
void nsem_oracle_convection_wind(const nsem_oracle_mesh* m, const double* U_all, const double* scale,
                                 int order, double* T_in, double dt, int nsteps) {
    convection_core(m, NULL, U_all, scale, order, T_in, dt, nsteps);
}
