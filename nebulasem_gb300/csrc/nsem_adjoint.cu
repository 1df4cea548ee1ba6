/*
 * Discrete adjoint of the FP64 dGSEM Euler tendency and of the SSP-RK3 step.
 *
 * Vector-Jacobian product g = J_L(v)^T w of the operator chain of the plain
 * form (nsem_fp64.cu; reference: euler.cpp:181-258, field.h:2881-2943,
 * 3086-3117, 3417-3478), hand-derived in reverse mode:
 *   r = -cV L                     ->  rbar = -w / cV
 *   source  r_m -= g (rho - rho_ref) cV
 *   volume  r[a] -= F_b . (Jin_b dpsi(b->a))  -> Fbar_b = -sum_a rbar[a] (x) dj(b->a)
 *           (the transposed line contraction, gathered per source node b)
 *   lift    r[c1] += d_k, r[c2] -= d_k         -> dbar_k = rbar[c1] - rbar[c2]
 *   Rusanov d = (cds F - n^ (x) lambda dq) . fN, lambda = (cds|U| + cds c) / 2
 *   ghosts  NEUMANN copies, SYMMETRY velocity (tangential projection
 *           rescaled to |U|, tensor.h:486-494), adjoint folded into the owner
 *   EOS     p = P0 (rho theta R / P0)^gamma -> dp/drho = gamma p / rho,
 *                                              dp/dtheta = gamma p / theta
 * Non-smooth points take the one-sided choice of the value's branch
 * (d|U| = U/|U|, 0 at U = 0; the SYMMETRY threshold |r| <= 1e-7 as forward).
 *
 * Kernels: k_adj_face (per used slot: adjoint of the face flux for both
 * sides, in primitive variables), k_adj_volume (per element, thread per node:
 * transposed volume gather, source, face contributions gathered through the
 * lift lists, primitive -> conserved chain rule).  The tangent-linear product
 * (k_tan_face, k_tan_volume) linearises the same chain in forward mode.
 * FP64 throughout; this file
 * may use FMA contraction (the adjoint is checked to 1e-6, not bitwise).
 */
#include <cuda_runtime.h>

#include "nsem_adjoint.h"
#include "nsem_seg.h"
#include "nsem_gather.cuh"
#include "nsem_mortar.cuh"

namespace {

enum { XX, YY, ZZ, XY, YZ, XZ, YX, ZY, ZX };
constexpr int NPA = 6;   /* primitive adjoints per side: rho, U0, U1, U2, theta, p' */

__device__ __forceinline__ double vdot3(const double* a, const double* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

/* tensor index of d_r U_c (XX,YY,ZZ,XY,YZ,XZ,YX,ZY,ZX) */
__device__ __forceinline__ constexpr int tix(int r, int c) {
    return r == c ? r : (r == 0 ? (c == 1 ? XY : XZ) : r == 1 ? (c == 2 ? YZ : YX) : (c == 0 ? ZX : ZY));
}

struct NodePrim {
    double r, U[3], T, p, pp, mu, c;   /* p: full pressure, pp = p - p_ref */
};

__device__ __forceinline__ NodePrim node_prim(const NsemDev& m, const double* const* S, int64_t i) {
    NodePrim q;
    q.r = S[0][i];
    q.U[0] = S[1][i] / q.r;
    q.U[1] = S[2][i] / q.r;
    q.U[2] = S[3][i] / q.r;
    q.T = S[4][i] / q.r;
    q.p = m.P0 * pow(((q.r * q.T) * m.R) / m.P0, m.gamma);
    q.pp = q.p - m.p_ref[i];
    q.mu = sqrt(vdot3(q.U, q.U));
    q.c = sqrt(m.gR * q.T);
    return q;
}

/* ghost velocity of the SYMMETRY condition and the transpose of its
 * Jacobian applied to gbar (adds into ubar) */
__device__ __forceinline__ void sym_fwd(const double* p, const double* en, double* out, double* r,
                                        double& magR, double& magP, bool& scaled) {
    const double dn = vdot3(p, en);
    r[0] = p[0] - en[0] * dn;
    r[1] = p[1] - en[1] * dn;
    r[2] = p[2] - en[2] * dn;
    magR = sqrt(vdot3(r, r));
    magP = sqrt(vdot3(p, p));
    scaled = !(fabs(magR) <= 1e-7);
    const double s = scaled ? magP / magR : 1.0;
    out[0] = r[0] * s; out[1] = r[1] * s; out[2] = r[2] * s;
}

__device__ __forceinline__ void sym_vjp(const double* p, const double* en, const double* r,
                                        double magR, double magP, bool scaled, const double* gbar,
                                        double* ubar) {
    /* out = A p s, A = I - en en^T (symmetric), s = |p| / |A p| */
    double Ag[3];
    const double gn = vdot3(gbar, en);
    Ag[0] = gbar[0] - en[0] * gn;
    Ag[1] = gbar[1] - en[1] * gn;
    Ag[2] = gbar[2] - en[2] * gn;
    if (!scaled) {
        ubar[0] += Ag[0]; ubar[1] += Ag[1]; ubar[2] += Ag[2];
        return;
    }
    const double s = magP / magR;
    const double rg = vdot3(r, gbar);        /* d out = A dp s + r ds */
    /* ds = (p . dp) / (|p| |r|) - |p| (r . A dp) / |r|^3 ; A r = r */
    const double c1 = (magP > 0) ? rg / (magP * magR) : 0.0;
    const double c2 = rg * magP / (magR * magR * magR);
    for (int k = 0; k < 3; k++) ubar[k] += s * Ag[k] + c1 * p[k] - c2 * r[k];
}

struct FaceAdjArgs {
    const double* S[5];      /* state v */
    const double* W[5];      /* w = adjoint of L */
    double* adjO[NPA];       /* per slot, owner side primitive adjoints */
    double* adjN[NPA];       /* per slot, neighbour side (0 for ghosts) */
    double* dbv[4];          /* viscous runs: momentum and theta flux adjoints (else null) */
};

__global__ void __launch_bounds__(128) k_adj_face(const NsemDev m, FaceAdjArgs a) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.n_slot) return;
    if (m.n_ms && m.ms_of[k] >= 0) return;   /* non-conforming: k_adj_face_mortar */
    const int32_t c1 = m.c1[k], c2 = m.c2[k];
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    const double en[3] = {m.en[k], m.en[m.n_slot + k], m.en[2 * m.n_slot + k]};
    const double nmag = sqrt(vdot3(n, n));
    const double fi = m.fi[k], fo = 1 - fi;

    const NodePrim P1 = node_prim(m, a.S, c1);
    NodePrim P2;
    double rsym[3] = {0, 0, 0}, magR = 0, magP = 0;
    bool scaled = false;
    if (c2 >= 0) {
        P2 = node_prim(m, a.S, c2);
    } else {
        P2 = P1;
        if (m.bc[k] == 2) sym_fwd(P1.U, en, P2.U, rsym, magR, magP, scaled);
        P2.mu = sqrt(vdot3(P2.U, P2.U));
    }
    /* dbar from rbar = -w / cV */
    double db[5];
    for (int v = 0; v < 5; v++) {
        double x = -a.W[v][c1] / m.cv[c1];
        if (c2 >= 0) x -= -a.W[v][c2] / m.cv[c2];
        db[v] = x;
    }
    if (a.dbv[0]) {
        for (int c = 0; c < 3; c++) a.dbv[c][k] = db[1 + c];
        a.dbv[3][k] = db[4];
    }
    const double lam = ((P1.mu * fi + P2.mu * fo) + (P1.c * fi + P2.c * fo)) / 2;
    /* primitive adjoints of both sides */
    double rb1 = 0, rb2 = 0, Ub1[3] = {0, 0, 0}, Ub2[3] = {0, 0, 0}, Tb1 = 0, Tb2 = 0, pb1 = 0,
           pb2 = 0, lamb = 0;
    /* continuity */
    {
        const double A0 = db[0] * nmag;     /* sum_c Fbar_c en_c */
        for (int c = 0; c < 3; c++) {
            const double Fb = db[0] * n[c];
            Ub1[c] += Fb * P1.r * fi; rb1 += Fb * P1.U[c] * fi;
            Ub2[c] += Fb * P2.r * fo; rb2 += Fb * P2.U[c] * fo;
        }
        lamb += -A0 * (P2.r - P1.r);
        rb2 += -A0 * lam;
        rb1 += A0 * lam;
    }
    /* momentum */
    {
        const double Fc1[3] = {P1.U[0] * P1.r, P1.U[1] * P1.r, P1.U[2] * P1.r};
        const double Fc2[3] = {P2.U[0] * P2.r, P2.U[1] * P2.r, P2.U[2] * P2.r};
        double Fcb1[3] = {0, 0, 0}, Fcb2[3] = {0, 0, 0};
        const double dmen = db[1] * en[0] + db[2] * en[1] + db[3] * en[2];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                const double Fb = db[1 + r] * n[c];      /* Fbar[r][c] */
                const double Ab = fi * Fb, Bb = fo * Fb;
                Fcb1[r] += Ab * P1.U[c]; Ub1[c] += Ab * Fc1[r];
                Fcb2[r] += Bb * P2.U[c]; Ub2[c] += Bb * Fc2[r];
                if (r == c) { pb1 += Ab; pb2 += Bb; }
            }
        for (int c = 0; c < 3; c++) {
            const double dqb = -dmen * n[c];
            Fcb2[c] += dqb * lam;
            Fcb1[c] -= dqb * lam;
            lamb += dqb * (Fc2[c] - Fc1[c]);
        }
        for (int c = 0; c < 3; c++) {
            Ub1[c] += Fcb1[c] * P1.r; rb1 += Fcb1[c] * P1.U[c];
            Ub2[c] += Fcb2[c] * P2.r; rb2 += Fcb2[c] * P2.U[c];
        }
    }
    /* potential temperature */
    {
        const double B4 = db[4] * nmag;
        for (int c = 0; c < 3; c++) {
            const double Fb = db[4] * n[c];
            Ub1[c] += Fb * P1.r * P1.T * fi; rb1 += Fb * P1.U[c] * P1.T * fi; Tb1 += Fb * P1.U[c] * P1.r * fi;
            Ub2[c] += Fb * P2.r * P2.T * fo; rb2 += Fb * P2.U[c] * P2.T * fo; Tb2 += Fb * P2.U[c] * P2.r * fo;
        }
        lamb += -B4 * (P2.r * P2.T - P1.r * P1.T);
        rb2 += -B4 * lam * P2.T; Tb2 += -B4 * lam * P2.r;
        rb1 += B4 * lam * P1.T;  Tb1 += B4 * lam * P1.r;
    }
    /* lambda -> |U|, c */
    {
        const double mub1 = lamb * fi / 2, mub2 = lamb * fo / 2;
        const double cb1 = lamb * fi / 2, cb2 = lamb * fo / 2;
        if (P1.mu > 0) for (int c = 0; c < 3; c++) Ub1[c] += mub1 * P1.U[c] / P1.mu;
        if (P2.mu > 0) for (int c = 0; c < 3; c++) Ub2[c] += mub2 * P2.U[c] / P2.mu;
        if (P1.c > 0) Tb1 += cb1 * m.gR / (2 * P1.c);
        if (P2.c > 0) Tb2 += cb2 * m.gR / (2 * P2.c);
    }
    if (c2 < 0) {
        /* ghost: fold into the owner */
        rb1 += rb2; Tb1 += Tb2; pb1 += pb2;
        if (m.bc[k] == 2) sym_vjp(P1.U, en, rsym, magR, magP, scaled, Ub2, Ub1);
        else for (int c = 0; c < 3; c++) Ub1[c] += Ub2[c];
        rb2 = 0; Tb2 = 0; pb2 = 0; Ub2[0] = Ub2[1] = Ub2[2] = 0;
    }
    a.adjO[0][k] = rb1; a.adjO[1][k] = Ub1[0]; a.adjO[2][k] = Ub1[1]; a.adjO[3][k] = Ub1[2];
    a.adjO[4][k] = Tb1; a.adjO[5][k] = pb1;
    a.adjN[0][k] = rb2; a.adjN[1][k] = Ub2[0]; a.adjN[2][k] = Ub2[1]; a.adjN[3][k] = Ub2[2];
    a.adjN[4][k] = Tb2; a.adjN[5][k] = pb2;
}

/* ------------------------------------------------------------------------
 * Non-conforming (2:1) faces.  The forward face flux of a mortar
 * slot (nsem_fp64.cu, k_face) reads the coarse side through 19 quantities
 * interpolated from the coarse face's nodes: |U|, c, U rho (3), rho, the
 * momentum flux tensor (rho U) (x) U + p' I (9, tensor order), the theta flux
 * (rho U) theta (3), rho theta.  The flux is a function of the two sides'
 * quantity sets alone, so its tangent and transpose are written on quantity
 * sets: the fine side's from its node, the coarse side's interpolated
 * (tangents: interpolated tangents; adjoints: scattered back through the
 * transposed interpolation, then through the quantities' chain at each
 * coarse node).  The coarse side lifts the projection of the slot fluxes
 * (psiCor) dotted with each slot's normal: its transpose gathers over the
 * facet's slots.  With the artificial viscosity the momentum and theta flux
 * quantities carry - mu grad U and - (mu / Pr) grad theta of their node, so
 * the quantity sets' adjoints also give the nodes' gradient and mu adjoints;
 * the gradients' own mortar face terms (the coarse side interpolated into
 * cds, the projection onto the coarse side) are transposed by
 * k_adj_grad_mortar_a / _b.
 * ------------------------------------------------------------------------ */
__device__ __forceinline__ void tens_rc(int t, int& ra, int& rb) {
    ra = t < 3 ? t : (t == XY || t == XZ) ? 0 : (t == YZ || t == YX) ? 1 : 2;
    rb = t < 3 ? t : (t == YX || t == ZX) ? 0 : (t == XY || t == ZY) ? 1 : 2;
}

/* adjoints qb of the 19 face quantities of a node -> its primitive adjoints */
__device__ __forceinline__ void face_q_vjp(const NsemDev& m, const NodePrim& P, const double* qb,
                                           double& rbar, double* Ub, double& Tb, double& pb) {
    const double Fc[3] = {P.U[0] * P.r, P.U[1] * P.r, P.U[2] * P.r};
    if (P.mu > 0)
        for (int c = 0; c < 3; c++) Ub[c] += qb[0] * P.U[c] / P.mu;
    if (P.c > 0) Tb += qb[1] * m.gR / (2 * P.c);
    double Fcb[3] = {qb[2], qb[3], qb[4]};
    rbar += qb[5];
    for (int t = 0; t < 9; t++) {
        int ra, rb;
        tens_rc(t, ra, rb);
        Fcb[ra] += qb[6 + t] * P.U[rb];
        Ub[rb] += qb[6 + t] * Fc[ra];
        if (t < 3) pb += qb[6 + t];
    }
    for (int c = 0; c < 3; c++) {
        Fcb[c] += qb[15 + c] * P.T;
        Tb += qb[15 + c] * Fc[c];
    }
    rbar += qb[18] * P.T;
    Tb += qb[18] * P.r;
    for (int c = 0; c < 3; c++) {
        Ub[c] += Fcb[c] * P.r;
        rbar += Fcb[c] * P.U[c];
    }
}

struct VolAdjArgs {
    const double* S[5];
    const double* W[5];
    const double* adjO[NPA];
    const double* adjN[NPA];
    double* G[5];            /* output: J_L(v)^T w */
    /* viscous runs (else null): gradients of the state, slot flux adjoints;
     * out: gradient adjoints / cV and the adjoint of mu per node */
    const double* Gv[12];
    const double* dbv[4];
    double* Gbs[12];
    double* mub;
    /* non-conforming faces: per node the adjoints of the 19 face quantities
     * interpolated from it onto mortar slots (else null); viscous runs: per
     * mortar slot the fine side's viscous quantity adjoints */
    const double* qb[19];
    const double* mqv[12];
};

/* registers capped for the largest element: 736 threads (N+1 = 9) inviscid,
 * 512 (N+1 = 8) with the viscous terms */
template <bool VISC>
__global__ void __maxnreg__(VISC ? 128 : 88) k_adj_volume(const NsemDev m, const NsemTables tab,
                                                          VolAdjArgs a) {
    extern __shared__ double sm[];
    const int NPX = m.npx, NPY = m.npy, NPZ = m.npz, NP = m.np;
    double* rb = sm;                                 /* [5][NP] rbar of the element */
    double* dps = sm + 5 * NP;                       /* dpsi tables */
    const int t = threadIdx.x;
    for (int q = t; q < 3 * NSEM_MAX_NPD * NSEM_MAX_NPD; q += blockDim.x)
        dps[q] = (&tab.dpsi[0][0])[q];
    const int64_t e = blockIdx.x;
    const int64_t node = e * NP + t;
    const bool active = t < NP;
    if (active) {
        const double cv = m.cv[node];
        for (int v = 0; v < 5; v++) rb[v * NP + t] = -a.W[v][node] / cv;
    }
    __syncthreads();
    if (!active) return;
    const int ia = t / (NPY * NPZ), ja = (t / NPZ) % NPY, ka = t % NPZ;
    const NodePrim P = node_prim(m, a.S, node);
    double Jin[9];
    for (int c = 0; c < 9; c++) Jin[c] = m.jin[(int64_t)c * m.n_int + node];

    /* transposed volume gather: G_c, H_rc, K_c over the targets a of node b */
    double Gv[3] = {0, 0, 0}, H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, K[3] = {0, 0, 0};
    const double* Dx = dps;
    const double* Dy = dps + NSEM_MAX_NPD * NSEM_MAX_NPD;
    const double* Dz = dps + 2 * NSEM_MAX_NPD * NSEM_MAX_NPD;
    auto acc = [&](int la, const double* dj) {
        const double r0 = rb[la], r4 = rb[4 * NP + la];
        const double rm[3] = {rb[NP + la], rb[2 * NP + la], rb[3 * NP + la]};
        for (int c = 0; c < 3; c++) {
            Gv[c] += r0 * dj[c];
            K[c] += r4 * dj[c];
            for (int r = 0; r < 3; r++) H[r][c] += rm[r] * dj[c];
        }
    };
    /* targets on the x line (including self), then y and z lines */
    for (int im = 0; im < NPX; im++) {
        double dv[3];
        dv[0] = Dx[ia * NPX + im];
        dv[1] = (im == ia) ? Dy[ja * NPY + ja] : 0.0;
        dv[2] = (im == ia) ? Dz[ka * NPZ + ka] : 0.0;
        double dj[3];
        dj[0] = Jin[XX] * dv[0] + Jin[XY] * dv[1] + Jin[XZ] * dv[2];
        dj[1] = Jin[YX] * dv[0] + Jin[YY] * dv[1] + Jin[YZ] * dv[2];
        dj[2] = Jin[ZX] * dv[0] + Jin[ZY] * dv[1] + Jin[ZZ] * dv[2];
        acc(t + (im - ia) * NPY * NPZ, dj);
    }
    /* the y and z lines without the node itself: the same trip count on
     * every thread, the node's own index skipped by the mapping */
    for (int q = 0; q + 1 < NPY; q++) {
        const int jm = q < ja ? q : q + 1;
        const double D = Dy[ja * NPY + jm];
        const double dj[3] = {Jin[XY] * D, Jin[YY] * D, Jin[ZY] * D};
        acc(t + (jm - ja) * NPZ, dj);
    }
    for (int q = 0; q + 1 < NPZ; q++) {
        const int km = q < ka ? q : q + 1;
        const double D = Dz[ka * NPZ + km];
        const double dj[3] = {Jin[XZ] * D, Jin[YZ] * D, Jin[ZZ] * D};
        acc(t + (km - ka), dj);
    }
    /* viscous fluxes fm -= mu grad U, ft -= (mu / Pr) grad theta (volume) and the
     * node's side of its face fluxes: adjoints of the node's gradients and of mu */
    if constexpr (VISC) {
        const double mu = P.r * m.nu, mt = mu * m.iPr;
        double Gn[12], Gb[12], mb = 0;
        for (int c = 0; c < 12; c++) Gn[c] = a.Gv[c][node];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                const int q = tix(r, c);
                Gb[q] = mu * H[r][c];
                mb += Gn[q] * H[r][c];
            }
        for (int c = 0; c < 3; c++) {
            Gb[9 + c] = mt * K[c];
            mb += m.iPr * Gn[9 + c] * K[c];
        }
        for (int j = 0; j < m.n_lift; j++) {
            const int32_t code = m.lift[(int64_t)j * m.n_int + node];
            if (code < 0) break;
            if (code & 2) continue;                 /* a mortar's coarse side: through qb */
            const int64_t k = code >> 2;
            const int32_t ms = m.n_ms ? m.ms_of[k] : -1;
            if (ms >= 0) {
                /* the fine side of a mortar slot */
                for (int q = 0; q < 9; q++) {
                    const double b = a.mqv[q][ms];
                    Gb[q] -= mu * b;
                    mb -= b * Gn[q];
                }
                for (int c = 0; c < 3; c++) {
                    const double b = a.mqv[9 + c][ms];
                    Gb[9 + c] -= mt * b;
                    mb -= m.iPr * b * Gn[9 + c];
                }
                continue;
            }
            const double f = (code & 1) ? 1.0 - m.fi[k] : m.fi[k];
            const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
            const double dm[3] = {a.dbv[0][k], a.dbv[1][k], a.dbv[2][k]}, dt = a.dbv[3][k];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                    const int q = tix(r, c);
                    Gb[q] -= f * mu * dm[r] * n[c];
                    mb -= f * dm[r] * n[c] * Gn[q];
                }
            for (int c = 0; c < 3; c++) {
                Gb[9 + c] -= f * mt * dt * n[c];
                mb -= f * m.iPr * dt * n[c] * Gn[9 + c];
            }
        }
        if (a.qb[0]) {
            /* a coarse side of mortar slots: the viscous parts of the node's
             * interpolated quantities */
            for (int q = 0; q < 9; q++) {
                const double b = a.qb[6 + q][node];
                Gb[q] -= mu * b;
                mb -= b * Gn[q];
            }
            for (int c = 0; c < 3; c++) {
                const double b = a.qb[15 + c][node];
                Gb[9 + c] -= mt * b;
                mb -= m.iPr * b * Gn[9 + c];
            }
        }
        const double icv = 1.0 / m.cv[node];
        for (int c = 0; c < 12; c++) a.Gbs[c][node] = Gb[c] * icv;
        a.mub[node] = mb;
    }
    /* flux adjoints -> primitive adjoints (fr = U rho, fm = (rho U) (x) U + p' I,
     * ft = (rho U) theta; Fbar = -(G, H, K)) */
    double rbar = 0, Ub[3] = {0, 0, 0}, Tb = 0, pb = 0;
    const double Fc[3] = {P.U[0] * P.r, P.U[1] * P.r, P.U[2] * P.r};
    double Fcb[3] = {0, 0, 0};
    for (int c = 0; c < 3; c++) {
        const double frb = -Gv[c];
        Ub[c] += frb * P.r;
        rbar += frb * P.U[c];
        const double ftb = -K[c];
        Fcb[c] += ftb * P.T;
        Tb += ftb * Fc[c];
    }
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            const double fmb = -H[r][c];
            Fcb[r] += fmb * P.U[c];
            Ub[c] += fmb * Fc[r];
            if (r == c) pb += fmb;
        }
    for (int c = 0; c < 3; c++) {
        Ub[c] += Fcb[c] * P.r;
        rbar += Fcb[c] * P.U[c];
    }
    /* gravity source: r_m -= g (rho - rho_ref) cV */
    const double cv = m.cv[node];
    rbar += -(rb[NP + t] * m.g[0] + rb[2 * NP + t] * m.g[1] + rb[3 * NP + t] * m.g[2]) * cv;
    /* face contributions gathered through the lift lists (a coarse side of a
     * non-conforming face contributes through its interpolated quantities) */
    for (int j = 0; j < m.n_lift; j++) {
        const int32_t code = m.lift[(int64_t)j * m.n_int + node];
        if (code < 0) break;
        if (code & 2) continue;
        const int64_t k = code >> 2;
        const double* const* src = (code & 1) ? a.adjN : a.adjO;
        rbar += src[0][k]; Ub[0] += src[1][k]; Ub[1] += src[2][k]; Ub[2] += src[3][k];
        Tb += src[4][k]; pb += src[5][k];
    }
    if (a.qb[0]) {
        double q[19];
        for (int c = 0; c < 19; c++) q[c] = a.qb[c][node];
        face_q_vjp(m, P, q, rbar, Ub, Tb, pb);
    }
    /* EOS: p = P0 (rho theta R / P0)^gamma */
    rbar += pb * m.gamma * P.p / P.r;
    Tb += pb * m.gamma * P.p / P.T;
    /* U = m / rho, theta = E / rho */
    const double inv = 1.0 / P.r;
    double g0 = rbar - inv * vdot3(Ub, P.U) - inv * Tb * P.T;
    a.G[0][node] = g0;
    a.G[1][node] = Ub[0] * inv;
    a.G[2][node] = Ub[1] * inv;
    a.G[3][node] = Ub[2] * inv;
    a.G[4][node] = Tb * inv;
}

/* ------------------------------------------------------------------------
 * Tangent-linear (forward-mode) product Ld = J_L(v) dv of the same operator
 * chain: the linearisation of every step of the forward kernels, taken at v
 * along dv, with the same one-sided choices at non-smooth points.
 * ------------------------------------------------------------------------ */
struct NodeTan {
    double r, U[3], T, p, mu, c;
};

__device__ __forceinline__ NodeTan node_tan(const NsemDev& m, const NodePrim& P,
                                            const double* const* dS, int64_t i) {
    NodeTan d;
    d.r = dS[0][i];
    const double inv = 1.0 / P.r;
    for (int c = 0; c < 3; c++) d.U[c] = (dS[1 + c][i] - P.U[c] * d.r) * inv;
    d.T = (dS[4][i] - P.T * d.r) * inv;
    /* p = P0 (rho theta R / P0)^gamma: dp / p = gamma (drho / rho + dtheta / theta) */
    d.p = m.gamma * P.p * (d.r / P.r + d.T / P.T);
    d.mu = P.mu > 0 ? vdot3(P.U, d.U) / P.mu : 0.0;
    d.c = P.c > 0 ? m.gR * d.T / (2 * P.c) : 0.0;
    return d;
}

/* tangent of the SYMMETRY ghost velocity out = A p s (A = I - en en^T,
 * s = |p| / |A p| when scaled) along dp */
__device__ __forceinline__ void sym_jvp(const double* p, const double* en, const double* r,
                                        double magR, double magP, bool scaled, const double* dp,
                                        double* dout) {
    const double dn = vdot3(dp, en);
    const double Ad[3] = {dp[0] - en[0] * dn, dp[1] - en[1] * dn, dp[2] - en[2] * dn};
    if (!scaled) {
        dout[0] = Ad[0]; dout[1] = Ad[1]; dout[2] = Ad[2];
        return;
    }
    const double s = magP / magR;
    const double ds = (magP > 0 ? vdot3(p, dp) / (magP * magR) : 0.0) -
                      magP * vdot3(r, dp) / (magR * magR * magR);
    for (int k = 0; k < 3; k++) dout[k] = Ad[k] * s + r[k] * ds;
}

/* the 19 face quantities of a node, and their tangents along d (d may be
 * null); viscous runs (Gn: the node's 12 gradients, dGn their tangents) take
 * the momentum and theta fluxes with - mu grad U and - (mu / Pr) grad theta,
 * mu = rho nu, as the forward's mortar quantities (nsem_fp64.cu) */
__device__ __forceinline__ void face_q(const NodePrim& P, const NodeTan* d, double* q, double* dq,
                                       const double* Gn = nullptr, const double* dGn = nullptr,
                                       double nu = 0.0, double iPr = 0.0) {
    const double Fc[3] = {P.U[0] * P.r, P.U[1] * P.r, P.U[2] * P.r};
    q[0] = P.mu;
    q[1] = P.c;
    for (int c = 0; c < 3; c++) q[2 + c] = Fc[c];
    q[5] = P.r;
    for (int t = 0; t < 9; t++) {
        int ra, rb;
        tens_rc(t, ra, rb);
        q[6 + t] = Fc[ra] * P.U[rb] + (t < 3 ? P.pp : 0.0);
    }
    for (int c = 0; c < 3; c++) q[15 + c] = Fc[c] * P.T;
    q[18] = P.r * P.T;
    const double mu = P.r * nu, mt = mu * iPr;
    if (Gn) {
        for (int t = 0; t < 9; t++) q[6 + t] -= mu * Gn[t];
        for (int c = 0; c < 3; c++) q[15 + c] -= mt * Gn[9 + c];
    }
    if (!d) return;
    double dFc[3];
    for (int c = 0; c < 3; c++) dFc[c] = d->U[c] * P.r + P.U[c] * d->r;
    dq[0] = d->mu;
    dq[1] = d->c;
    for (int c = 0; c < 3; c++) dq[2 + c] = dFc[c];
    dq[5] = d->r;
    for (int t = 0; t < 9; t++) {
        int ra, rb;
        tens_rc(t, ra, rb);
        dq[6 + t] = dFc[ra] * P.U[rb] + Fc[ra] * d->U[rb] + (t < 3 ? d->p : 0.0);
    }
    for (int c = 0; c < 3; c++) dq[15 + c] = dFc[c] * P.T + Fc[c] * d->T;
    dq[18] = d->r * P.T + P.r * d->T;
    if (Gn) {
        const double dmu = nu * d->r, dmt = dmu * iPr;
        for (int t = 0; t < 9; t++) dq[6 + t] -= dmu * Gn[t] + mu * dGn[t];
        for (int c = 0; c < 3; c++) dq[15 + c] -= dmt * Gn[9 + c] + mt * dGn[9 + c];
    }
}

struct MortarArgs {
    const double* S[5];
    const double* dS[5];     /* tangent runs (else null) */
    const double* W[5];      /* adjoint runs: w */
    double* mq[19];
    double* dmq[19];
    double* dmf[15];
    double* ddC[5];
    double* dd[5];           /* tangent runs: per slot lifted tangent (fine side) */
    double* mqb[19];
    double* qb[19];
    double* adjO[NPA];
    double* adjN[NPA];
    /* viscous runs (else null): the state's gradients and their tangents per
     * node; out: the fine side's viscous quantity adjoints per mortar slot */
    const double* G[12];
    const double* dG[12];
    double* mqv[12];
};

/* the 12 gradients (and tangents) of a node for face_q, or null */
__device__ __forceinline__ const double* node_grads(const double* const* G, int64_t i, double* buf) {
    if (!G[0]) return nullptr;
    for (int c = 0; c < 12; c++) buf[c] = G[c][i];
    return buf;
}

/* per mortar slot: the coarse side's quantities (and tangents) interpolated */
__global__ void __launch_bounds__(128) k_mortar_q(const NsemDev m, MortarArgs a) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    const bool tan = a.dS[0] != nullptr;
    double out[38];
    mortar_interp<38>(m, ms, [&](int64_t node, double* v) {
        const NodePrim P = node_prim(m, a.S, node);
        double gb[12], dgb[12];
        const double* Gn = node_grads(a.G, node, gb);
        if (tan) {
            const NodeTan d = node_tan(m, P, a.dS, node);
            face_q(P, &d, v, v + 19, Gn, Gn ? node_grads(a.dG, node, dgb) : nullptr, m.nu, m.iPr);
        } else {
            face_q(P, nullptr, v, nullptr, Gn, nullptr, m.nu, m.iPr);
            for (int c = 19; c < 38; c++) v[c] = 0.0;
        }
    }, out);
    for (int c = 0; c < 19; c++) {
        a.mq[c][ms] = out[c];
        if (tan) a.dmq[c][ms] = out[19 + c];
    }
}

/* the two sides' quantity sets of a mortar slot: the fine node's own, the
 * coarse side's interpolated */
__device__ __forceinline__ void mortar_sides(const NsemDev& m, const MortarArgs& a, int64_t ms,
                                             int64_t k, int side, bool tan, double* q1, double* dq1,
                                             double* q2, double* dq2, NodePrim& Pf) {
    const int64_t fine = side == 1 ? m.c2[k] : m.c1[k];
    Pf = node_prim(m, a.S, fine);
    double* qf = side == 1 ? q2 : q1;
    double* dqf = side == 1 ? dq2 : dq1;
    double* qc = side == 1 ? q1 : q2;
    double* dqc = side == 1 ? dq1 : dq2;
    double gb[12], dgb[12];
    const double* Gn = node_grads(a.G, fine, gb);
    if (tan) {
        const NodeTan d = node_tan(m, Pf, a.dS, fine);
        face_q(Pf, &d, qf, dqf, Gn, Gn ? node_grads(a.dG, fine, dgb) : nullptr, m.nu, m.iPr);
    } else {
        face_q(Pf, nullptr, qf, nullptr, Gn, nullptr, m.nu, m.iPr);
    }
    for (int c = 0; c < 19; c++) {
        qc[c] = a.mq[c][ms];
        if (tan) dqc[c] = a.dmq[c][ms];
    }
}

/* tangent of a mortar slot's flux: the fine side's lifted value and the flux
 * vectors for the coarse side's projection */
__global__ void __launch_bounds__(128) k_tan_face_mortar(const NsemDev m, MortarArgs a) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    const int64_t k = ms_field(m, NSEM_MS_K, ms);
    const int side = ms_field(m, NSEM_MS_SIDE, ms);
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    const double en[3] = {m.en[k], m.en[m.n_slot + k], m.en[2 * m.n_slot + k]};
    const double fi = m.fi[k], fo = 1 - fi;
    double q1[19], dq1[19], q2[19], dq2[19];
    NodePrim Pf;
    mortar_sides(m, a, ms, k, side, true, q1, dq1, q2, dq2, Pf);
    const double lam = ((q1[0] * fi + q2[0] * fo) + (q1[1] * fi + q2[1] * fo)) / 2;
    const double dlam = ((dq1[0] * fi + dq2[0] * fo) + (dq1[1] * fi + dq2[1] * fo)) / 2;
    double dF[15];
    for (int c = 0; c < 3; c++)
        dF[c] = dq1[2 + c] * fi + dq2[2 + c] * fo -
                en[c] * (dlam * (q2[5] - q1[5]) + lam * (dq2[5] - dq1[5]));
    double ddq[3];
    for (int c = 0; c < 3; c++)
        ddq[c] = (dq2[2 + c] - dq1[2 + c]) * lam + (q2[2 + c] - q1[2 + c]) * dlam;
    for (int t = 0; t < 9; t++) {
        int r, c;
        tens_rc(t, r, c);
        dF[3 + t] = dq1[6 + t] * fi + dq2[6 + t] * fo - en[r] * ddq[c];
    }
    for (int c = 0; c < 3; c++)
        dF[12 + c] = dq1[15 + c] * fi + dq2[15 + c] * fo -
                     en[c] * (dlam * (q2[18] - q1[18]) + lam * (dq2[18] - dq1[18]));
    for (int c = 0; c < 15; c++) a.dmf[c][ms] = dF[c];
    a.dd[0][k] = vdot3(dF, n);
    a.dd[1][k] = dF[3 + XX] * n[0] + dF[3 + XY] * n[1] + dF[3 + XZ] * n[2];
    a.dd[2][k] = dF[3 + YX] * n[0] + dF[3 + YY] * n[1] + dF[3 + YZ] * n[2];
    a.dd[3][k] = dF[3 + ZX] * n[0] + dF[3 + ZY] * n[1] + dF[3 + ZZ] * n[2];
    a.dd[4][k] = vdot3(dF + 12, n);
}

/* the coarse side's lifted tangents: projected flux tangents . the slot's normal */
__global__ void __launch_bounds__(128) k_tan_mortar_gather(const NsemDev m, MortarArgs a) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= 5 * m.n_ms) return;
    const int64_t ms = id / 5;
    const int r = (int)(id % 5);
    const int64_t k = ms_field(m, NSEM_MS_K, ms);
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    double P[3];
    if (r == 0 || r == 4) {
        double* src[3] = {a.dmf[r == 0 ? 0 : 12], a.dmf[r == 0 ? 1 : 13], a.dmf[r == 0 ? 2 : 14]};
        mortar_project<3>(m, ms, src, P);
    } else {
        const int q = r - 1;
        double* src[3] = {a.dmf[3 + (q == 0 ? XX : q == 1 ? YX : ZX)],
                          a.dmf[3 + (q == 0 ? XY : q == 1 ? YY : ZY)],
                          a.dmf[3 + (q == 0 ? XZ : q == 1 ? YZ : ZZ)]};
        mortar_project<3>(m, ms, src, P);
    }
    a.ddC[r][ms] = vdot3(P, n);
}

/* adjoint of a mortar slot's flux: the flux-vector adjoints from the fine
 * side's lift of this slot and from the coarse side's lifts of the facet's
 * projections, then the two quantity sets' adjoints: the fine side's to its
 * primitive adjoints (gathered by the volume kernel), the coarse side's kept
 * per slot for the transposed interpolation */
__global__ void __launch_bounds__(128) k_adj_face_mortar(const NsemDev m, MortarArgs a) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    const int64_t k = ms_field(m, NSEM_MS_K, ms);
    const int side = ms_field(m, NSEM_MS_SIDE, ms);
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    const double en[3] = {m.en[k], m.en[m.n_slot + k], m.en[2 * m.n_slot + k]};
    const double fi = m.fi[k], fo = 1 - fi;
    double q1[19], q2[19];
    NodePrim Pf;
    mortar_sides(m, a, ms, k, side, false, q1, nullptr, q2, nullptr, Pf);
    const double lam = ((q1[0] * fi + q2[0] * fo) + (q1[1] * fi + q2[1] * fo)) / 2;
    /* flux-vector adjoints: rbar = -w / cV; the owner lifts +, the neighbour - */
    double Fb[15] = {0};
    {
        const int64_t fine = side == 1 ? m.c2[k] : m.c1[k];
        const double sg = side == 1 ? -1.0 : 1.0;
        double db[5];
        for (int v = 0; v < 5; v++) db[v] = sg * (-a.W[v][fine] / m.cv[fine]);
        for (int c = 0; c < 3; c++) {
            Fb[c] += db[0] * n[c];
            Fb[12 + c] += db[4] * n[c];
        }
        for (int t = 0; t < 9; t++) {
            int r, c;
            tens_rc(t, r, c);
            Fb[3 + t] += db[1 + r] * n[c];
        }
    }
    {
        /* the coarse side: dC[s'] = (sum_j Pcor(j -> s') F_j) . n_s' over the
         * facet's slots s' */
        const int Na = ms_field(m, NSEM_MS_NA, ms), Nb = ms_field(m, NSEM_MS_NB, ms);
        const int64_t first = ms_field(m, NSEM_MS_FIRST, ms);
        const int ja = (int)((ms - first) / Nb), jb = (int)((ms - first) % Nb);
        for (int sa = 0; sa < Na; sa++)
            for (int sb = 0; sb < Nb; sb++) {
                const int64_t s2 = first + sa * Nb + sb;
                const int64_t k2 = ms_field(m, NSEM_MS_K, s2);
                const int side2 = ms_field(m, NSEM_MS_SIDE, s2);
                const int64_t coarse = side2 == 1 ? m.c1[k2] : m.c2[k2];
                const double sg = side2 == 1 ? 1.0 : -1.0;
                const double* Pa = m.psic + ms_field(m, NSEM_MS_TA, s2) * NSEM_MAX_NPD * NSEM_MAX_NPD;
                const double* Pb = m.psic + ms_field(m, NSEM_MS_TB, s2) * NSEM_MAX_NPD * NSEM_MAX_NPD;
                const int na = ms_field(m, NSEM_MS_IA, s2), nb = ms_field(m, NSEM_MS_IB, s2);
                const double w = Pa[ja * Na + na] * Pb[jb * Nb + nb];
                const double n2[3] = {m.fn[k2], m.fn[m.n_slot + k2], m.fn[2 * m.n_slot + k2]};
                double db[5];
                for (int v = 0; v < 5; v++) db[v] = w * sg * (-a.W[v][coarse] / m.cv[coarse]);
                for (int c = 0; c < 3; c++) {
                    Fb[c] += db[0] * n2[c];
                    Fb[12 + c] += db[4] * n2[c];
                }
                for (int t = 0; t < 9; t++) {
                    int r, c;
                    tens_rc(t, r, c);
                    Fb[3 + t] += db[1 + r] * n2[c];
                }
            }
    }
    /* the quantity sets' adjoints */
    const double A0 = vdot3(Fb, en), B4 = vdot3(Fb + 12, en);
    double dqb[3] = {0, 0, 0};
    for (int t = 0; t < 9; t++) {
        int r, c;
        tens_rc(t, r, c);
        dqb[c] -= Fb[3 + t] * en[r];
    }
    double lamb = -A0 * (q2[5] - q1[5]) - B4 * (q2[18] - q1[18]);
    for (int c = 0; c < 3; c++) lamb += dqb[c] * (q2[2 + c] - q1[2 + c]);
    double qb1[19], qb2[19];
    qb1[0] = lamb * fi / 2; qb2[0] = lamb * fo / 2;
    qb1[1] = lamb * fi / 2; qb2[1] = lamb * fo / 2;
    for (int c = 0; c < 3; c++) {
        qb1[2 + c] = Fb[c] * fi - dqb[c] * lam;
        qb2[2 + c] = Fb[c] * fo + dqb[c] * lam;
    }
    qb1[5] = A0 * lam; qb2[5] = -A0 * lam;
    for (int t = 0; t < 9; t++) { qb1[6 + t] = Fb[3 + t] * fi; qb2[6 + t] = Fb[3 + t] * fo; }
    for (int c = 0; c < 3; c++) { qb1[15 + c] = Fb[12 + c] * fi; qb2[15 + c] = Fb[12 + c] * fo; }
    qb1[18] = B4 * lam; qb2[18] = -B4 * lam;
    const double* qbf = side == 1 ? qb2 : qb1;
    const double* qbc = side == 1 ? qb1 : qb2;
    double rbar = 0, Ub[3] = {0, 0, 0}, Tb = 0, pb = 0;
    face_q_vjp(m, Pf, qbf, rbar, Ub, Tb, pb);
    double* const* fine_out = side == 1 ? a.adjN : a.adjO;
    double* const* coarse_out = side == 1 ? a.adjO : a.adjN;
    fine_out[0][k] = rbar; fine_out[1][k] = Ub[0]; fine_out[2][k] = Ub[1]; fine_out[3][k] = Ub[2];
    fine_out[4][k] = Tb; fine_out[5][k] = pb;
    for (int v = 0; v < NPA; v++) coarse_out[v][k] = 0.0;
    for (int c = 0; c < 19; c++) a.mqb[c][ms] = qbc[c];
    if (a.mqv[0]) {
        /* the fine node's - mu grad U, - (mu / Pr) grad theta parts: taken
         * by the volume kernel into the node's gradient and mu adjoints */
        for (int t = 0; t < 9; t++) a.mqv[t][ms] = qbf[6 + t];
        for (int c = 0; c < 3; c++) a.mqv[9 + c][ms] = qbf[15 + c];
    }
}

/* the transposed interpolation: each mortar slot's coarse-side adjoints back
 * onto the coarse face's nodes (atomic: a node takes several slots) */
__global__ void __launch_bounds__(128) k_adj_mortar_scatter(const NsemDev m, MortarArgs a) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    const int base = ms_field(m, NSEM_MS_BASE, ms), sa = ms_field(m, NSEM_MS_SA, ms),
              sb = ms_field(m, NSEM_MS_SB, ms), Na = ms_field(m, NSEM_MS_NA, ms),
              Nb = ms_field(m, NSEM_MS_NB, ms), ia = ms_field(m, NSEM_MS_IA, ms),
              ib = ms_field(m, NSEM_MS_IB, ms);
    const double* Pa = m.psir + ms_field(m, NSEM_MS_TA, ms) * NSEM_MAX_NPD * NSEM_MAX_NPD;
    const double* Pb = m.psir + ms_field(m, NSEM_MS_TB, ms) * NSEM_MAX_NPD * NSEM_MAX_NPD;
    double qb[19];
    for (int c = 0; c < 19; c++) qb[c] = a.mqb[c][ms];
    for (int na = 0; na < Na; na++)
        for (int nb = 0; nb < Nb; nb++) {
            const int64_t node = (int64_t)base + na * sa + nb * sb;
            const double w = Pa[na * Na + ia] * Pb[nb * Nb + ib];
            for (int c = 0; c < 19; c++) atomicAdd(a.qb[c] + node, w * qb[c]);
        }
}

struct FaceTanArgs {
    const double* S[5];
    const double* dS[5];
    double* dd[5];           /* per slot: tangent of the lifted face flux */
    const double* G[12];     /* viscous runs: grad U, grad theta of the state (else null) */
    const double* dG[12];    /* and their tangents */
};

/* U and theta of the state and their tangents, per node (gradient inputs) */
struct PrimTanArgs {
    const double* S[5];
    const double* dS[5];
    double* pU[4];
    double* dpU[4];
};

__global__ void __launch_bounds__(256) k_tan_prims(const NsemDev m, PrimTanArgs a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n_int) return;
    const double r = a.S[0][i];
    const double U[3] = {a.S[1][i] / r, a.S[2][i] / r, a.S[3][i] / r};
    const double T = a.S[4][i] / r;
    const double dr = a.dS[0][i], inv = 1.0 / r;
    for (int c = 0; c < 3; c++) {
        a.pU[c][i] = U[c];
        a.dpU[c][i] = (a.dS[1 + c][i] - U[c] * dr) * inv;
    }
    a.pU[3][i] = T;
    a.dpU[3][i] = (a.dS[4][i] - T * dr) * inv;
}

/* tangent of the gradients' face values: d cds(U, theta) per slot, the wall
 * ghost linearised as the forward ghost (SYMMETRY projection, NEUMANN copy) */
struct GradFaceTanArgs {
    const double* pU[4];
    const double* dpU[4];
    double* dfF[4];
};

__global__ void __launch_bounds__(256) k_tan_grad_face(const NsemDev m, GradFaceTanArgs a) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.n_slot) return;
    const int32_t c1 = m.c1[k], c2 = m.c2[k];
    const double fi = m.fi[k], fo = 1 - fi;
    const double dU1[3] = {a.dpU[0][c1], a.dpU[1][c1], a.dpU[2][c1]};
    double dU2[3], dT2;
    if (c2 >= 0) {
        for (int c = 0; c < 3; c++) dU2[c] = a.dpU[c][c2];
        dT2 = a.dpU[3][c2];
    } else {
        dT2 = a.dpU[3][c1];
        if (m.bc[k] == 2) {
            const double en[3] = {m.en[k], m.en[m.n_slot + k], m.en[2 * m.n_slot + k]};
            const double U1[3] = {a.pU[0][c1], a.pU[1][c1], a.pU[2][c1]};
            double U2[3], rsym[3], magR, magP;
            bool scaled;
            sym_fwd(U1, en, U2, rsym, magR, magP, scaled);
            sym_jvp(U1, en, rsym, magR, magP, scaled, dU1, dU2);
        } else {
            for (int c = 0; c < 3; c++) dU2[c] = dU1[c];
        }
    }
    for (int c = 0; c < 3; c++) a.dfF[c][k] = dU1[c] * fi + dU2[c] * fo;
    a.dfF[3][k] = a.dpU[3][c1] * fi + dT2 * fo;
}

__global__ void __launch_bounds__(128) k_tan_face(const NsemDev m, FaceTanArgs a) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.n_slot) return;
    if (m.n_ms && m.ms_of[k] >= 0) return;   /* non-conforming: k_tan_face_mortar */
    const int32_t c1 = m.c1[k], c2 = m.c2[k];
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    const double en[3] = {m.en[k], m.en[m.n_slot + k], m.en[2 * m.n_slot + k]};
    const double fi = m.fi[k], fo = 1 - fi;

    const NodePrim P1 = node_prim(m, a.S, c1);
    const NodeTan d1 = node_tan(m, P1, a.dS, c1);
    NodePrim P2;
    NodeTan d2;
    if (c2 >= 0) {
        P2 = node_prim(m, a.S, c2);
        d2 = node_tan(m, P2, a.dS, c2);
    } else {
        /* ghost: NEUMANN copies rho, theta, p; the velocity is copied or
         * takes the SYMMETRY projection */
        P2 = P1;
        d2 = d1;
        if (m.bc[k] == 2) {
            double rsym[3], magR, magP;
            bool scaled;
            sym_fwd(P1.U, en, P2.U, rsym, magR, magP, scaled);
            sym_jvp(P1.U, en, rsym, magR, magP, scaled, d1.U, d2.U);
        }
        P2.mu = sqrt(vdot3(P2.U, P2.U));
        d2.mu = P2.mu > 0 ? vdot3(P2.U, d2.U) / P2.mu : 0.0;
    }
    const double lam = ((P1.mu * fi + P2.mu * fo) + (P1.c * fi + P2.c * fo)) / 2;
    const double dlam = ((d1.mu * fi + d2.mu * fo) + (d1.c * fi + d2.c * fo)) / 2;
    const double Fc1[3] = {P1.U[0] * P1.r, P1.U[1] * P1.r, P1.U[2] * P1.r};
    const double Fc2[3] = {P2.U[0] * P2.r, P2.U[1] * P2.r, P2.U[2] * P2.r};
    double dFc1[3], dFc2[3];
    for (int c = 0; c < 3; c++) {
        dFc1[c] = d1.U[c] * P1.r + P1.U[c] * d1.r;
        dFc2[c] = d2.U[c] * P2.r + P2.U[c] * d2.r;
    }
    /* continuity: F = (U rho)_avg - lam (rho_N - rho_O) en */
    double dd0 = 0;
    {
        const double jump = P2.r - P1.r, djump = d2.r - d1.r;
        for (int c = 0; c < 3; c++)
            dd0 += (dFc1[c] * fi + dFc2[c] * fo - (dlam * jump + lam * djump) * en[c]) * n[c];
    }
    /* viscous flux tangents: - d(mu grad U) = - (dmu G + mu dG), mu = rho nu,
     * zero gradient on a wall ghost */
    const bool visc = a.G[0] != nullptr;
    const bool g2 = c2 >= 0;
    const double mu1 = P1.r * m.nu, mu2 = P2.r * m.nu, dmu1 = d1.r * m.nu, dmu2 = d2.r * m.nu;
    /* momentum: F[r][c] = (Fc U + p' I)_avg[r][c] - lam (Fc_N - Fc_O)[c] en[r] */
    double ddm[3];
    for (int r = 0; r < 3; r++) {
        double acc = 0;
        for (int c = 0; c < 3; c++) {
            double dA = dFc1[r] * P1.U[c] + Fc1[r] * d1.U[c] + (r == c ? d1.p : 0.0);
            double dB = dFc2[r] * P2.U[c] + Fc2[r] * d2.U[c] + (r == c ? d2.p : 0.0);
            if (visc) {
                const int q = tix(r, c);
                dA -= dmu1 * a.G[q][c1] + mu1 * a.dG[q][c1];
                if (g2) dB -= dmu2 * a.G[q][c2] + mu2 * a.dG[q][c2];
            }
            const double ddq = (dFc2[c] - dFc1[c]) * lam + (Fc2[c] - Fc1[c]) * dlam;
            acc += (dA * fi + dB * fo - ddq * en[r]) * n[c];
        }
        ddm[r] = acc;
    }
    /* potential temperature: F = (U rho theta)_avg - lam (rho theta_N - rho theta_O) en */
    double dd4 = 0;
    {
        const double e1 = P1.r * P1.T, e2 = P2.r * P2.T;
        const double de1 = d1.r * P1.T + P1.r * d1.T, de2 = d2.r * P2.T + P2.r * d2.T;
        for (int c = 0; c < 3; c++) {
            double f1 = dFc1[c] * P1.T + Fc1[c] * d1.T;
            double f2 = dFc2[c] * P2.T + Fc2[c] * d2.T;
            if (visc) {
                f1 -= m.iPr * (dmu1 * a.G[9 + c][c1] + mu1 * a.dG[9 + c][c1]);
                if (g2) f2 -= m.iPr * (dmu2 * a.G[9 + c][c2] + mu2 * a.dG[9 + c][c2]);
            }
            dd4 += (f1 * fi + f2 * fo - (dlam * (e2 - e1) + lam * (de2 - de1)) * en[c]) * n[c];
        }
    }
    a.dd[0][k] = dd0; a.dd[1][k] = ddm[0]; a.dd[2][k] = ddm[1]; a.dd[3][k] = ddm[2];
    a.dd[4][k] = dd4;
}

struct VolTanArgs {
    const double* S[5];
    const double* dS[5];
    const double* dd[5];
    const double* ddC[5];    /* non-conforming faces: projected, lifted tangents */
    double* out[5];          /* J_L(v) dv */
    const double* G[12];     /* viscous runs (else null) */
    const double* dG[12];
};

/* shared layout per node: dfr[3] dfm[9] dft[3] jin[9] */
constexpr int TAN_W = 24;

__global__ void k_tan_volume(const NsemDev m, const NsemTables tab, VolTanArgs a) {
    extern __shared__ double sm[];
    const int NPX = m.npx, NPY = m.npy, NPZ = m.npz, NP = m.np;
    double* dps = sm + (size_t)NP * TAN_W;
    const int t = threadIdx.x;
    for (int q = t; q < 3 * NSEM_MAX_NPD * NSEM_MAX_NPD; q += blockDim.x)
        dps[q] = (&tab.dpsi[0][0])[q];
    const int64_t e = blockIdx.x;
    const bool active = t < NP;
    const int64_t node = e * NP + t;
    double drho = 0;
    if (active) {
        const NodePrim P = node_prim(m, a.S, node);
        const NodeTan d = node_tan(m, P, a.dS, node);
        drho = d.r;
        double* my = sm + (size_t)t * TAN_W;
        const double Fc[3] = {P.U[0] * P.r, P.U[1] * P.r, P.U[2] * P.r};
        double dFc[3];
        for (int c = 0; c < 3; c++) dFc[c] = d.U[c] * P.r + P.U[c] * d.r;
        for (int c = 0; c < 3; c++) my[c] = dFc[c];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                const int idx = (r == c) ? r : (r == 0 && c == 1) ? XY : (r == 1 && c == 2) ? YZ
                              : (r == 0 && c == 2) ? XZ : (r == 1 && c == 0) ? YX
                              : (r == 2 && c == 1) ? ZY : ZX;
                my[3 + idx] = dFc[r] * P.U[c] + Fc[r] * d.U[c] + (r == c ? d.p : 0.0);
            }
        for (int c = 0; c < 3; c++) my[12 + c] = dFc[c] * P.T + Fc[c] * d.T;
        if (a.G[0]) {
            const double mu = P.r * m.nu, dmu = d.r * m.nu;
            for (int c = 0; c < 9; c++) my[3 + c] -= dmu * a.G[c][node] + mu * a.dG[c][node];
            for (int c = 0; c < 3; c++)
                my[12 + c] -= m.iPr * (dmu * a.G[9 + c][node] + mu * a.dG[9 + c][node]);
        }
        for (int c = 0; c < 9; c++) my[15 + c] = m.jin[(int64_t)c * m.n_int + node];
    }
    __syncthreads();
    if (!active) return;
    double r[5] = {0, 0, 0, 0, 0};
    /* surface lift (a coarse side of a non-conforming face lifts the
     * projected tangent) */
    for (int j = 0; j < m.n_lift; j++) {
        const int32_t code = m.lift[(int64_t)j * m.n_int + node];
        if (code < 0) break;
        const int64_t k = code >> 2;
        const double sg = (code & 1) ? -1.0 : 1.0;
        if (code & 2) {
            for (int v = 0; v < 5; v++) r[v] += sg * a.ddC[v][k];
        } else {
            for (int v = 0; v < 5; v++) r[v] += sg * a.dd[v][k];
        }
    }
    /* volume term: r[a] -= dF_b . (Jin_b dpsi(b -> a)) over the lines through a */
    nsem_volume_gather<TAN_W, 15>(NPX, NPY, NPZ, sm, dps, t, [&](int lb, const double* dj) {
        const double* sb = sm + (size_t)lb * TAN_W;
        r[0] -= vdot3(sb, dj);
        const double* F = sb + 3;
        r[1] -= F[XX] * dj[0] + F[XY] * dj[1] + F[XZ] * dj[2];
        r[2] -= F[YX] * dj[0] + F[YY] * dj[1] + F[YZ] * dj[2];
        r[3] -= F[ZX] * dj[0] + F[ZY] * dj[1] + F[ZZ] * dj[2];
        r[4] -= vdot3(sb + 12, dj);
    });
    /* gravity source: r_m -= g (rho - rho_ref) cV */
    const double cv = m.cv[node];
    for (int c = 0; c < 3; c++) r[1 + c] -= m.g[c] * drho * cv;
    for (int v = 0; v < 5; v++) a.out[v][node] = -(r[v] / cv);
}

/* Transpose of the strong-form gradient (gradf<true>) for the viscous
 * adjoint.  Forward, per node a: G_a = (1/cV_a) [sum_slots s fN (x) (cds - p_a)
 * + sum_b (jin_a dpsi(b at a)) (x) p_b], cds = fi p_c1 + fo p_c2 (the wall ghost
 * p_c2 = SYMMETRY projection / NEUMANN copy of p_c1).  Given Gbs = Gbar / cV:
 *   face (per slot): v_c1 = fN . Gbs_c1, v_c2 = -fN . Gbs_c2; cdsbar = v_c1 + v_c2;
 *     pbar_c1 += fi cdsbar - v_c1, pbar_c2 += fo cdsbar - v_c2 (the ghost's
 *     share folded into c1 through the ghost's transpose);
 *   volume (per node b): pbar_b += sum over the nodes a on b's lines of
 *     (jin_a dpsi(b at a))^T Gbs_a. */
struct GradAdjArgs {
    const double* S[5];
    const double* pU[4];      /* U, theta of the state (the ghost's linearisation point) */
    const double* Gbs[12];
    double* agO[4];
    double* agN[4];
    double* G[5];             /* conserved-state adjoint, added to */
    const double* mub;
    /* non-conforming faces (else null): per node the (U, theta) adjoints of
     * the mortar slots' gradient face terms; per mortar slot the adjoints of
     * the fine side's face value and of the coarse side's projected value */
    double* pbM[4];
    double* fFb[4];
    double* gCb[4];
};

__global__ void __launch_bounds__(256) k_adj_grad_face(const NsemDev m, GradAdjArgs a) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.n_slot) return;
    if (m.n_ms && m.ms_of[k] >= 0) {
        /* a mortar slot: k_adj_grad_mortar_* */
        for (int c = 0; c < 4; c++) a.agO[c][k] = a.agN[c][k] = 0.0;
        return;
    }
    const int32_t c1 = m.c1[k], c2 = m.c2[k];
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    const double fi = m.fi[k], fo = 1 - fi;
    double v1[4], v2[4] = {0, 0, 0, 0};
    for (int c = 0; c < 3; c++) {
        v1[c] = n[0] * a.Gbs[tix(0, c)][c1] + n[1] * a.Gbs[tix(1, c)][c1] + n[2] * a.Gbs[tix(2, c)][c1];
        if (c2 >= 0)
            v2[c] = -(n[0] * a.Gbs[tix(0, c)][c2] + n[1] * a.Gbs[tix(1, c)][c2] +
                      n[2] * a.Gbs[tix(2, c)][c2]);
    }
    v1[3] = n[0] * a.Gbs[9][c1] + n[1] * a.Gbs[10][c1] + n[2] * a.Gbs[11][c1];
    if (c2 >= 0) v2[3] = -(n[0] * a.Gbs[9][c2] + n[1] * a.Gbs[10][c2] + n[2] * a.Gbs[11][c2]);
    double cb[4], p1[4], p2[4];
    for (int c = 0; c < 4; c++) {
        cb[c] = v1[c] + v2[c];
        p1[c] = fi * cb[c] - v1[c];
        p2[c] = fo * cb[c] - v2[c];
    }
    if (c2 < 0) {
        /* ghost: theta copies theta_c1; U is the SYMMETRY projection or a copy */
        const double gU[3] = {fo * cb[0], fo * cb[1], fo * cb[2]};
        p1[3] += fo * cb[3];
        if (m.bc[k] == 2) {
            const double en[3] = {m.en[k], m.en[m.n_slot + k], m.en[2 * m.n_slot + k]};
            const double U1[3] = {a.pU[0][c1], a.pU[1][c1], a.pU[2][c1]};
            double U2[3], rsym[3], magR, magP;
            bool scaled;
            sym_fwd(U1, en, U2, rsym, magR, magP, scaled);
            sym_vjp(U1, en, rsym, magR, magP, scaled, gU, p1);
        } else {
            for (int c = 0; c < 3; c++) p1[c] += gU[c];
        }
        for (int c = 0; c < 4; c++) p2[c] = 0;
    }
    for (int c = 0; c < 4; c++) {
        a.agO[c][k] = p1[c];
        a.agN[c][k] = p2[c];
    }
}

/* Gradient face terms on mortar slots (forward: k_seg_mortar_gcds,
 * k_seg_mortar_ggather, k_seg_grad_vol).  Forward, per mortar slot ms with
 * fine node f and coarse node c (the slot's c1 / c2 by its side), the
 * gradients take s_f n (x) (fF[ms] - p_f) at f and s_c n (x) (gC[ms] - p_c)
 * at c (s = +1 on the owner side, -1 on the neighbour side), with
 * fF = cds of p_f and the coarse side interpolated onto the slot, gC the
 * facet's fF projected onto c's position.  Adjoint, first pass (per slot):
 * v = s n . Gbar/cV at f and at c, taken off the nodes' (U, theta) adjoints
 * and kept as the adjoints of fF (fine) and gC (coarse). */
__global__ void __launch_bounds__(128) k_adj_grad_mortar_a(const NsemDev m, GradAdjArgs a) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    const int64_t k = ms_field(m, NSEM_MS_K, ms);
    const int side = ms_field(m, NSEM_MS_SIDE, ms);
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    /* side 1: the coarse node is the owner c1; side 2: the neighbour c2 */
    const int64_t fine = side == 1 ? m.c2[k] : m.c1[k];
    const int64_t coarse = side == 1 ? m.c1[k] : m.c2[k];
    const double sf = side == 1 ? -1.0 : 1.0, sc = -sf;
    double vf[4], vc[4];
    for (int c = 0; c < 3; c++) {
        vf[c] = sf * (n[0] * a.Gbs[tix(0, c)][fine] + n[1] * a.Gbs[tix(1, c)][fine] +
                      n[2] * a.Gbs[tix(2, c)][fine]);
        vc[c] = sc * (n[0] * a.Gbs[tix(0, c)][coarse] + n[1] * a.Gbs[tix(1, c)][coarse] +
                      n[2] * a.Gbs[tix(2, c)][coarse]);
    }
    vf[3] = sf * (n[0] * a.Gbs[9][fine] + n[1] * a.Gbs[10][fine] + n[2] * a.Gbs[11][fine]);
    vc[3] = sc * (n[0] * a.Gbs[9][coarse] + n[1] * a.Gbs[10][coarse] + n[2] * a.Gbs[11][coarse]);
    for (int c = 0; c < 4; c++) {
        atomicAdd(a.pbM[c] + fine, -vf[c]);
        atomicAdd(a.pbM[c] + coarse, -vc[c]);
        a.fFb[c][ms] = vf[c];
        a.gCb[c][ms] = vc[c];
    }
}

/* second pass (per slot): the adjoint of fF[ms] -- its own part plus the
 * transposed projection of the facet's gC adjoints -- split by the cds
 * weights onto the fine node and onto the interpolated coarse value, which
 * the transposed interpolation returns to the coarse face's nodes */
__global__ void __launch_bounds__(128) k_adj_grad_mortar_b(const NsemDev m, GradAdjArgs a) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    const int64_t k = ms_field(m, NSEM_MS_K, ms);
    const int side = ms_field(m, NSEM_MS_SIDE, ms);
    const int Na = ms_field(m, NSEM_MS_NA, ms), Nb = ms_field(m, NSEM_MS_NB, ms);
    const int64_t first = ms_field(m, NSEM_MS_FIRST, ms);
    const int ja = (int)((ms - first) / Nb), jb = (int)((ms - first) % Nb);
    double fb[4];
    for (int c = 0; c < 4; c++) fb[c] = a.fFb[c][ms];
    for (int sa = 0; sa < Na; sa++)
        for (int sb = 0; sb < Nb; sb++) {
            const int64_t s2 = first + sa * Nb + sb;
            const double* Pa = m.psic + ms_field(m, NSEM_MS_TA, s2) * NSEM_MAX_NPD * NSEM_MAX_NPD;
            const double* Pb = m.psic + ms_field(m, NSEM_MS_TB, s2) * NSEM_MAX_NPD * NSEM_MAX_NPD;
            const int na = ms_field(m, NSEM_MS_IA, s2), nb = ms_field(m, NSEM_MS_IB, s2);
            const double w = Pa[ja * Na + na] * Pb[jb * Nb + nb];
            for (int c = 0; c < 4; c++) fb[c] += w * a.gCb[c][s2];
        }
    /* fF = p1 fi + p2 fo, the coarse (interpolated) value on side `side` */
    const double fi = m.fi[k], fo = 1 - fi;
    const double wf = side == 1 ? fo : fi, wc = side == 1 ? fi : fo;
    const int64_t fine = side == 1 ? m.c2[k] : m.c1[k];
    for (int c = 0; c < 4; c++) atomicAdd(a.pbM[c] + fine, wf * fb[c]);
    const int base = ms_field(m, NSEM_MS_BASE, ms), sa = ms_field(m, NSEM_MS_SA, ms),
              sb = ms_field(m, NSEM_MS_SB, ms), ia = ms_field(m, NSEM_MS_IA, ms),
              ib = ms_field(m, NSEM_MS_IB, ms);
    const double* Ra = m.psir + ms_field(m, NSEM_MS_TA, ms) * NSEM_MAX_NPD * NSEM_MAX_NPD;
    const double* Rb = m.psir + ms_field(m, NSEM_MS_TB, ms) * NSEM_MAX_NPD * NSEM_MAX_NPD;
    for (int na = 0; na < Na; na++)
        for (int nb = 0; nb < Nb; nb++) {
            const int64_t node = (int64_t)base + na * sa + nb * sb;
            const double w = wc * Ra[na * Na + ia] * Rb[nb * Nb + ib];
            for (int c = 0; c < 4; c++) atomicAdd(a.pbM[c] + node, w * fb[c]);
        }
}

/* shared layout per node: Gbs[12] jin[9] */
constexpr int GADJ_W = 21;

__global__ void k_adj_grad_vol(const NsemDev m, const NsemTables tab, GradAdjArgs a) {
    extern __shared__ double sm[];
    const int NPX = m.npx, NPY = m.npy, NPZ = m.npz, NP = m.np;
    double* dps = sm + (size_t)NP * GADJ_W;
    const int t = threadIdx.x;
    for (int q = t; q < 3 * NSEM_MAX_NPD * NSEM_MAX_NPD; q += blockDim.x)
        dps[q] = (&tab.dpsi[0][0])[q];
    const int64_t e = blockIdx.x;
    const bool active = t < NP;
    const int64_t node = e * NP + t;
    if (active) {
        double* my = sm + (size_t)t * GADJ_W;
        for (int c = 0; c < 12; c++) my[c] = a.Gbs[c][node];
        for (int c = 0; c < 9; c++) my[12 + c] = m.jin[(int64_t)c * m.n_int + node];
    }
    __syncthreads();
    if (!active) return;
    const int ib = t / (NPY * NPZ), jb = (t / NPZ) % NPY, kb = t % NPZ;
    const double* Dx = dps;
    const double* Dy = dps + NSEM_MAX_NPD * NSEM_MAX_NPD;
    const double* Dz = dps + 2 * NSEM_MAX_NPD * NSEM_MAX_NPD;
    double pb[4] = {0, 0, 0, 0};
    auto add = [&](int la, const double* dj) {
        const double* sa = sm + (size_t)la * GADJ_W;
        for (int c = 0; c < 3; c++)
            pb[c] += dj[0] * sa[tix(0, c)] + dj[1] * sa[tix(1, c)] + dj[2] * sa[tix(2, c)];
        pb[3] += dj[0] * sa[9] + dj[1] * sa[10] + dj[2] * sa[11];
    };
    /* the nodes a whose gradient used p_b: b's x line (a = b: the full
     * jin_b . (Dx_bb, Dy_bb, Dz_bb)), its y and z lines without b */
    for (int ia = 0; ia < NPX; ia++) {
        const int la = t + (ia - ib) * NPY * NPZ;
        const double* J = sm + (size_t)la * GADJ_W + 12;
        double dj[3];
        if (ia == ib) {
            const double dv[3] = {Dx[ib * NPX + ib], Dy[jb * NPY + jb], Dz[kb * NPZ + kb]};
            dj[0] = J[XX] * dv[0] + J[XY] * dv[1] + J[XZ] * dv[2];
            dj[1] = J[YX] * dv[0] + J[YY] * dv[1] + J[YZ] * dv[2];
            dj[2] = J[ZX] * dv[0] + J[ZY] * dv[1] + J[ZZ] * dv[2];
        } else {
            const double D = Dx[ia * NPX + ib];
            dj[0] = J[XX] * D; dj[1] = J[YX] * D; dj[2] = J[ZX] * D;
        }
        add(la, dj);
    }
    for (int q = 0; q + 1 < NPY; q++) {
        const int ja = q < jb ? q : q + 1;
        const int la = t + (ja - jb) * NPZ;
        const double* J = sm + (size_t)la * GADJ_W + 12;
        const double D = Dy[ja * NPY + jb];
        const double dj[3] = {J[XY] * D, J[YY] * D, J[ZY] * D};
        add(la, dj);
    }
    for (int q = 0; q + 1 < NPZ; q++) {
        const int ka = q < kb ? q : q + 1;
        const int la = t + (ka - kb);
        const double* J = sm + (size_t)la * GADJ_W + 12;
        const double D = Dz[ka * NPZ + kb];
        const double dj[3] = {J[XZ] * D, J[YZ] * D, J[ZZ] * D};
        add(la, dj);
    }
    /* face terms gathered through the lift lists (mortar slots: pbM) */
    for (int j = 0; j < m.n_lift; j++) {
        const int32_t code = m.lift[(int64_t)j * m.n_int + node];
        if (code < 0) break;
        if (code & 2) continue;
        const int64_t k = code >> 2;
        const double* const* src = (code & 1) ? a.agN : a.agO;
        for (int c = 0; c < 4; c++) pb[c] += src[c][k];
    }
    if (a.pbM[0])
        for (int c = 0; c < 4; c++) pb[c] += a.pbM[c][node];
    /* (rho, U, theta) adjoints -> conserved: U = m / rho, theta = E / rho; mu = rho nu */
    const double r = a.S[0][node], inv = 1.0 / r;
    const double U[3] = {a.S[1][node] * inv, a.S[2][node] * inv, a.S[3][node] * inv};
    const double T = a.S[4][node] / r;
    const double rbar = m.nu * a.mub[node];
    a.G[0][node] += rbar - inv * (pb[0] * U[0] + pb[1] * U[1] + pb[2] * U[2]) - inv * pb[3] * T;
    for (int c = 0; c < 3; c++) a.G[1 + c][node] += pb[c] * inv;
    a.G[4][node] += pb[3] * inv;
}

/* lam = c0 * lam + c1 * x + c2 * y (elementwise over 5 arrays) */
struct Lin3Args {
    double* out[5];
    const double* x[5];
    const double* y[5];
    const double* z[5];
    double cx, cy, cz;
    int64_t n;
};

__global__ void k_lin3(Lin3Args a) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
         i += (int64_t)gridDim.x * blockDim.x)
        for (int v = 0; v < 5; v++) {
            double s = a.cx * a.x[v][i];
            if (a.y[0]) s += a.cy * a.y[v][i];
            if (a.z[0]) s += a.cz * a.z[v][i];
            a.out[v][i] = s;
        }
}

int grid_for(int64_t n) {
    int64_t g = (n + 255) / 256;
    if (g > 152 * 8) g = 152 * 8;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

int nsem_adj_vjp(const NsemDev* m, const NsemTables* t, const double* const* S,
                 const double* const* W, double* const* G, NsemAdjBuf* ab, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    FaceAdjArgs fa{};
    VolAdjArgs va{};
    if (ab->visc) {
        /* U, theta and the gradients of the state */
        PrimTanArgs pa;
        for (int v = 0; v < 5; v++) { pa.S[v] = S[v]; pa.dS[v] = S[v]; }
        for (int c = 0; c < 4; c++) { pa.pU[c] = ab->pU[c]; pa.dpU[c] = ab->dpU[c]; }
        k_tan_prims<<<(unsigned)((m->n_int + 255) / 256), 256, 0, st>>>(*m, pa);
        const int e = nsem_grad_ut_mortar(m, t, ab->pU, ab->pU[3], ab->Gv, ab->fF,
                                          m->n_ms > 0 ? ab->gC : nullptr, stream);
        if (e) return e;
        for (int c = 0; c < 4; c++) fa.dbv[c] = ab->dbv[c];
        for (int c = 0; c < 12; c++) { va.Gv[c] = ab->Gv[c]; va.Gbs[c] = ab->Gbs[c]; }
        for (int c = 0; c < 4; c++) va.dbv[c] = ab->dbv[c];
        va.mub = ab->mub;
    }
    for (int v = 0; v < 5; v++) { fa.S[v] = S[v]; fa.W[v] = W[v]; }
    for (int v = 0; v < NPA; v++) { fa.adjO[v] = ab->adjO[v]; fa.adjN[v] = ab->adjN[v]; }
    const int64_t fb = (m->n_slot + 127) / 128;
    k_adj_face<<<(unsigned)fb, 128, 0, st>>>(*m, fa);
    for (int c = 0; c < 19; c++) va.qb[c] = nullptr;
    if (m->n_ms > 0) {
        MortarArgs ma{};
        for (int v = 0; v < 5; v++) { ma.S[v] = S[v]; ma.W[v] = W[v]; }
        if (ab->visc)
            for (int c = 0; c < 12; c++) { ma.G[c] = ab->Gv[c]; ma.mqv[c] = ab->mqv[c]; va.mqv[c] = ab->mqv[c]; }
        for (int c = 0; c < 19; c++) { ma.mq[c] = ab->mq[c]; ma.mqb[c] = ab->mqb[c]; ma.qb[c] = ab->qb[c]; }
        for (int v = 0; v < NPA; v++) { ma.adjO[v] = ab->adjO[v]; ma.adjN[v] = ab->adjN[v]; }
        for (int c = 0; c < 19; c++) {
            const cudaError_t ce = cudaMemsetAsync(ab->qb[c], 0, (size_t)m->n_int * sizeof(double), st);
            if (ce != cudaSuccess) return (int)ce;
        }
        const unsigned mb = (unsigned)((m->n_ms + 127) / 128);
        k_mortar_q<<<mb, 128, 0, st>>>(*m, ma);
        k_adj_face_mortar<<<mb, 128, 0, st>>>(*m, ma);
        k_adj_mortar_scatter<<<mb, 128, 0, st>>>(*m, ma);
        for (int c = 0; c < 19; c++) va.qb[c] = ab->qb[c];
    }
    for (int v = 0; v < 5; v++) { va.S[v] = S[v]; va.W[v] = W[v]; va.G[v] = G[v]; }
    for (int v = 0; v < NPA; v++) { va.adjO[v] = ab->adjO[v]; va.adjN[v] = ab->adjN[v]; }
    const int threads = ((m->np + 31) / 32) * 32;
    const size_t smem = (5 * (size_t)m->np + 3 * NSEM_MAX_NPD * NSEM_MAX_NPD) * sizeof(double);
    if (ab->visc) k_adj_volume<true><<<(unsigned)m->n_elem, threads, smem, st>>>(*m, *t, va);
    else k_adj_volume<false><<<(unsigned)m->n_elem, threads, smem, st>>>(*m, *t, va);
    if (ab->visc) {
        /* the gradients' transpose, added to the conserved adjoint */
        GradAdjArgs ga{};
        for (int v = 0; v < 5; v++) { ga.S[v] = S[v]; ga.G[v] = G[v]; }
        for (int c = 0; c < 4; c++) { ga.pU[c] = ab->pU[c]; ga.agO[c] = ab->agO[c]; ga.agN[c] = ab->agN[c]; }
        for (int c = 0; c < 12; c++) ga.Gbs[c] = ab->Gbs[c];
        ga.mub = ab->mub;
        k_adj_grad_face<<<(unsigned)((m->n_slot + 255) / 256), 256, 0, st>>>(*m, ga);
        if (m->n_ms > 0) {
            for (int c = 0; c < 4; c++) {
                ga.pbM[c] = ab->pbM[c]; ga.fFb[c] = ab->fFb[c]; ga.gCb[c] = ab->gCb[c];
                const cudaError_t ce = cudaMemsetAsync(ab->pbM[c], 0, (size_t)m->n_int * sizeof(double), st);
                if (ce != cudaSuccess) return (int)ce;
            }
            const unsigned mb = (unsigned)((m->n_ms + 127) / 128);
            k_adj_grad_mortar_a<<<mb, 128, 0, st>>>(*m, ga);
            k_adj_grad_mortar_b<<<mb, 128, 0, st>>>(*m, ga);
        }
        const size_t gsm = ((size_t)m->np * GADJ_W + 3 * NSEM_MAX_NPD * NSEM_MAX_NPD) * sizeof(double);
        k_adj_grad_vol<<<(unsigned)m->n_elem, threads, gsm, st>>>(*m, *t, ga);
    }
    return (int)cudaGetLastError();
}

int nsem_adj_jvp(const NsemDev* m, const NsemTables* t, const double* const* S,
                 const double* const* dS, double* const* out, NsemAdjBuf* ab, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    FaceTanArgs fa{};
    VolTanArgs va{};
    if (ab->visc) {
        /* gradients of the state and their tangents (the gradient is linear
         * in its node and face values) */
        PrimTanArgs pa;
        for (int v = 0; v < 5; v++) { pa.S[v] = S[v]; pa.dS[v] = dS[v]; }
        for (int c = 0; c < 4; c++) { pa.pU[c] = ab->pU[c]; pa.dpU[c] = ab->dpU[c]; }
        k_tan_prims<<<(unsigned)((m->n_int + 255) / 256), 256, 0, st>>>(*m, pa);
        const bool mort = m->n_ms > 0;
        int e = nsem_grad_ut_mortar(m, t, ab->pU, ab->pU[3], ab->Gv, ab->fF, mort ? ab->gC : nullptr, stream);
        if (e) return e;
        GradFaceTanArgs ga;
        for (int c = 0; c < 4; c++) { ga.pU[c] = ab->pU[c]; ga.dpU[c] = ab->dpU[c]; ga.dfF[c] = ab->dfF[c]; }
        k_tan_grad_face<<<(unsigned)((m->n_slot + 255) / 256), 256, 0, st>>>(*m, ga);
        /* mortar slots: the face values' tangents are the (linear) mortar
         * face values of the tangents */
        if (mort && (e = nsem_grad_mortar_faces(m, ab->dpU, ab->dpU[3], ab->dfF, ab->dgC, stream)))
            return e;
        e = nsem_grad_vol(m, t, ab->dpU, ab->dpU[3], ab->dGv, ab->dfF, mort ? ab->dgC : nullptr, stream);
        if (e) return e;
        for (int c = 0; c < 12; c++) {
            fa.G[c] = va.G[c] = ab->Gv[c];
            fa.dG[c] = va.dG[c] = ab->dGv[c];
        }
    }
    for (int v = 0; v < 5; v++) { fa.S[v] = S[v]; fa.dS[v] = dS[v]; fa.dd[v] = ab->adjO[v]; }
    const int64_t fb = (m->n_slot + 127) / 128;
    k_tan_face<<<(unsigned)fb, 128, 0, st>>>(*m, fa);
    for (int v = 0; v < 5; v++) va.ddC[v] = nullptr;
    if (m->n_ms > 0) {
        MortarArgs ma{};
        for (int v = 0; v < 5; v++) { ma.S[v] = S[v]; ma.dS[v] = dS[v]; ma.dd[v] = ab->adjO[v]; }
        if (ab->visc)
            for (int c = 0; c < 12; c++) { ma.G[c] = ab->Gv[c]; ma.dG[c] = ab->dGv[c]; }
        for (int c = 0; c < 19; c++) { ma.mq[c] = ab->mq[c]; ma.dmq[c] = ab->dmq[c]; }
        for (int c = 0; c < 15; c++) ma.dmf[c] = ab->dmf[c];
        for (int v = 0; v < 5; v++) ma.ddC[v] = ab->ddC[v];
        const unsigned mb = (unsigned)((m->n_ms + 127) / 128);
        k_mortar_q<<<mb, 128, 0, st>>>(*m, ma);
        k_tan_face_mortar<<<mb, 128, 0, st>>>(*m, ma);
        k_tan_mortar_gather<<<(unsigned)((5 * m->n_ms + 127) / 128), 128, 0, st>>>(*m, ma);
        for (int v = 0; v < 5; v++) va.ddC[v] = ab->ddC[v];
    }
    for (int v = 0; v < 5; v++) { va.S[v] = S[v]; va.dS[v] = dS[v]; va.dd[v] = ab->adjO[v]; va.out[v] = out[v]; }
    const int threads = ((m->np + 31) / 32) * 32;
    const size_t smem = ((size_t)m->np * TAN_W + 3 * NSEM_MAX_NPD * NSEM_MAX_NPD) * sizeof(double);
    k_tan_volume<<<(unsigned)m->n_elem, threads, smem, st>>>(*m, *t, va);
    return (int)cudaGetLastError();
}

int nsem_adj_lin3(double* const* out, const double* const* x, double cx, const double* const* y,
                  double cy, const double* const* z, double cz, int64_t n, void* stream) {
    Lin3Args a;
    for (int v = 0; v < 5; v++) {
        a.out[v] = out[v];
        a.x[v] = x[v];
        a.y[v] = y ? y[v] : nullptr;
        a.z[v] = z ? z[v] : nullptr;
    }
    a.cx = cx; a.cy = cy; a.cz = cz; a.n = n;
    k_lin3<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(a);
    return (int)cudaGetLastError();
}

int nsem_adj_prepare(const NsemDev* m) {
    const size_t smem = (5 * (size_t)m->np + 3 * NSEM_MAX_NPD * NSEM_MAX_NPD) * sizeof(double);
    if (smem > 48 * 1024) {
        int e = (int)cudaFuncSetAttribute(k_adj_volume<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem);
        if (!e) e = (int)cudaFuncSetAttribute(k_adj_volume<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem);
        if (e) return e;
    }
    const size_t tsm = ((size_t)m->np * TAN_W + 3 * NSEM_MAX_NPD * NSEM_MAX_NPD) * sizeof(double);
    if (tsm > 48 * 1024) {
        const int e = (int)cudaFuncSetAttribute(k_tan_volume, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)tsm);
        if (e) return e;
    }
    const size_t gsm = ((size_t)m->np * GADJ_W + 3 * NSEM_MAX_NPD * NSEM_MAX_NPD) * sizeof(double);
    if (gsm > 48 * 1024)
        return (int)cudaFuncSetAttribute(k_adj_grad_vol, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)gsm);
    return 0;
}
