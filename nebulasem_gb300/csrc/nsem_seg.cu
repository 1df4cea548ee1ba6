/*
 * The reference's own time update on the GPU: segregated forward Euler over
 * the primitive fields (apps/euler/euler.cpp:179-287 with time_scheme BDF1,
 * with or without diffusion), the drop-in counterpart of the shipped euler
 * solver.
 *
 * Compiled with --fmad=false; every operation in the order the reference
 * evaluates it (the same restatement as the oracle's nsem_oracle_segregated),
 * so the result is bit-identical to the reference wherever its C library pow
 * is correctly rounded (the equation of state uses nsem_ddpow.h).
 *
 * One step, five kernels:
 *   prep      per node: theta = theta' + T0 (T += T0, euler.cpp:181),
 *             Fc = rho U (flxc, field.h:3392-3395), |U|, sqrt(gamma R theta);
 *   face_rho  per used slot: lambda = (cds|U| + cds c)/2 (euler.cpp:186),
 *             Rusanov flux of the rho equation (flux U rho, state rho);
 *   vol_rho   per element: lift + weak volume term of the rho equation, then
 *             rho^{n+1} = Su/ap with ap = (-1/dt) cV, Su += rho^n ap
 *             (addTemporal<1> / ddt BDF1, field.h:3741-3841, 3875-3920;
 *             SolveTexplicit, solve.cpp:563-564), and p' = P0 (rho^{n+1}
 *             theta R / P0)^gamma - p_ref (euler.cpp:211-213);
 *   face_ut   per used slot: Rusanov fluxes of the U equation (flux
 *             Fc (x) U + p' I, state rho^{n+1} U) and the T equation (flux
 *             Fc theta, state rho^{n+1} theta), lambda of the step;
 *   vol_ut    per element: lift + volume terms, gravity source (rho^{n+1} -
 *             rho_ref) g, U^{n+1} = Su/ap with ap = (-1/dt) cV rho^{n+1} and
 *             Su += (U^n rho^n)(-1/dt) cV, likewise theta, then T -= T0.
 * Ghost values follow applyExplicitBCs (field.h:2586-2727) on the fly:
 * NEUMANN owner + 0, SYMMETRY velocity the rescaled tangential projection.
 * With diffusion YES (viscosity nu > 0) two more kernels per step form the
 * strong-form DG gradients of U^n and theta^n (gradf<true>, field.h:3327-3360:
 * face terms fN (x) (cds(p) - p) in the cell's face order, then the volume
 * derivative along the three lines, divided by cV; zero on the wall ghosts,
 * fillBCs field.h:2731-2769), and the fluxes carry - mu grad U and
 * - (mu / Pr) grad theta with mu = rho^n nu (euler.cpp:189-190, 232, 250).
 *
 * Also here: the reference's scalar DG convection (apps/convection/
 * convection.cpp, problem_init NONE, BDF1) -- a scalar T in a fixed wind U,
 * Fc = U, lambda = cds(|U|)/2, the same weak divergence and BDF1 update.
 */
#include <cuda_runtime.h>

#include "nsem_ddpow.h"
#include "nsem_gather.cuh"
#include "nsem_mortar.cuh"
#include "nsem_seg.h"

namespace {

enum { XX, YY, ZZ, XY, YZ, XZ, YX, ZY, ZX };

__device__ __forceinline__ double vdot3(const double* a, const double* b) {
    return a[0] * b[0] + (a[1] * b[1] + (a[2] * b[2] + 0.0));
}

__device__ __forceinline__ void tdot(const double* q, const double* p, double* r) {
    r[0] = q[XX] * p[0] + q[XY] * p[1] + q[XZ] * p[2];
    r[1] = q[YX] * p[0] + q[YY] * p[1] + q[YZ] * p[2];
    r[2] = q[ZX] * p[0] + q[ZY] * p[1] + q[ZZ] * p[2];
}

__device__ __forceinline__ void outer(const double* p, const double* q, double* r) {
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

/* SYMMETRY ghost velocity (src/tensor/tensor.h:486-494) */
__device__ __forceinline__ void sym_vec(const double* p, const double* n, double* out) {
    const double mg = sqrt(vdot3(n, n));
    const double en[3] = {n[0] / mg, n[1] / mg, n[2] / mg};
    const double A0 = 1.0 - en[0] * en[0];
    const double A1 = 1.0 - en[1] * en[1];
    const double A2 = 1.0 - en[2] * en[2];
    const double A3 = 0.0 - en[0] * en[1];
    const double A4 = 0.0 - en[1] * en[2];
    const double A5 = 0.0 - en[0] * en[2];
    double r[3];
    r[0] = A0 * p[0] + A3 * p[1] + A5 * p[2];
    r[1] = A3 * p[0] + A1 * p[1] + A4 * p[2];
    r[2] = A5 * p[0] + A4 * p[1] + A2 * p[2];
    const double magR = sqrt(vdot3(r, r));
    if (fabs(magR - 0.0) <= 1e-7) {
        out[0] = r[0]; out[1] = r[1]; out[2] = r[2];
        return;
    }
    const double s = sqrt(vdot3(p, p)) / magR;
    out[0] = r[0] * s; out[1] = r[1] * s; out[2] = r[2] * s;
}

/* ghost velocity of slot k from the owner's */
__device__ __forceinline__ void ghost_U(const NsemDev& m, int64_t k, const double* n,
                                        const double* U1, double* U2) {
    if (m.bc[k] == 2) {
        sym_vec(U1, n, U2);
    } else {
        U2[0] = U1[0] + 0.0; U2[1] = U1[1] + 0.0; U2[2] = U1[2] + 0.0;
    }
}

struct SegArgs {
    const double* rho_o;     /* rho^n            */
    double* rho_n;           /* rho^{n+1}        */
    double* U[3];            /* U^n -> U^{n+1}   */
    double* Tp;              /* theta' in/out    */
    double* Tf;              /* theta = theta' + T0 of the step */
    double* Fc[3];
    double* mu;
    double* cs;
    double* pp;
    double* lam;             /* per slot */
    double* d[5];            /* per slot */
    double* G[12];           /* per node: grad U, grad theta (viscous runs) */
    double* fF[4];           /* per slot: cds(U), cds(theta) (viscous runs) */
    /* non-conforming faces, per mortar slot */
    double* mq[16];          /* the coarse side's interpolated quantities */
    double* mf[12];          /* face flux vectors / tensors */
    double* dC[5];           /* projected, lifted coarse-side fluxes */
    double* gC[4];           /* projected cds(U), cds(theta) */
    double c_dt;             /* -1 / dt */
    int visc;
};

/* One thread per (mortar slot, quantity): each sum is a short dependent
 * chain over the coarse face's nodes, so the slots' quantities run side by
 * side. */

/* rho equation and lambda: |U|, c, U rho, rho of the coarse side */
__global__ void __launch_bounds__(128) k_seg_mortar_rho(const NsemDev m, SegArgs a) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= 6 * m.n_ms) return;
    const int64_t ms = id / 6;
    const int c = (int)(id % 6);
    double out[1];
    mortar_interp<1>(m, ms, [&](int64_t node, double* v) {
        if (c == 0) v[0] = a.mu[node];
        else if (c == 1) v[0] = a.cs[node];
        else if (c == 5) v[0] = a.rho_o[node];
        else v[0] = a.U[c - 2][node] * a.rho_o[node];
    }, out);
    a.mq[c][ms] = out[0];
}

/* U and theta equations: the flux tensor Fc (x) U + p' I - mu grad U, the
 * state rho U, the flux Fc theta - (mu / Pr) grad theta, the state rho theta
 * of the coarse side (component c of 16) */
__global__ void __launch_bounds__(128) k_seg_mortar_ut(const NsemDev m, SegArgs a) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= 16 * m.n_ms) return;
    const int64_t ms = id / 16;
    const int c = (int)(id % 16);
    /* outer(Fc, U) components XX YY ZZ XY YZ XZ YX ZY ZX */
    const int ra = c < 9 ? (c < 3 ? c : (c == 3 || c == 5) ? 0 : (c == 4 || c == 6) ? 1 : 2) : 0;
    const int rb = c < 9 ? (c < 3 ? c : (c == 6 || c == 8) ? 0 : (c == 3 || c == 7) ? 1 : 2) : 0;
    double out[1];
    mortar_interp<1>(m, ms, [&](int64_t node, double* v) {
        const double mu = a.visc ? a.rho_o[node] * m.nu : 0.0;
        if (c < 9) {
            double x = a.Fc[ra][node] * a.U[rb][node];
            x = x + ((c < 3) ? 1.0 : 0.0) * a.pp[node];
            if (a.visc) x = x - mu * a.G[c][node];
            v[0] = x;
        } else if (c < 12) {
            v[0] = a.rho_n[node] * a.U[c - 9][node];
        } else if (c < 15) {
            double x = a.Fc[c - 12][node] * a.Tf[node];
            if (a.visc) x = x - (mu * m.iPr) * a.G[9 + c - 12][node];
            v[0] = x;
        } else {
            v[0] = a.rho_n[node] * a.Tf[node];
        }
    }, out);
    a.mq[c][ms] = out[0];
}

/* the coarse side's lifted values: the projected flux vectors dotted with the
 * slot's own weighted normal (div_flux, field.h:3086-3117); for the U and
 * theta equations one thread per (mortar slot, output row) */
template <int EQ>
__global__ void __launch_bounds__(128) k_seg_mortar_gather(const NsemDev m, SegArgs a) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int rows = EQ == 0 ? 1 : 4;
    if (id >= rows * m.n_ms) return;
    const int64_t ms = id / rows;
    const int r = (int)(id % rows);
    const int64_t k = ms_field(m, NSEM_MS_K, ms);
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    if (EQ == 0) {
        double F[3];
        mortar_project<3>(m, ms, a.mf, F);
        a.dC[0][ms] = vdot3(F, n);
    } else if (r < 3) {
        /* row r of the tensor-vector product: components (r,x) (r,y) (r,z) */
        const int cx = r == 0 ? XX : r == 1 ? YX : ZX;
        const int cy = r == 0 ? XY : r == 1 ? YY : ZY;
        const int cz = r == 0 ? XZ : r == 1 ? YZ : ZZ;
        double* src[3] = {a.mf[cx], a.mf[cy], a.mf[cz]};
        double P[3];
        mortar_project<3>(m, ms, src, P);
        a.dC[1 + r][ms] = P[0] * n[0] + P[1] * n[1] + P[2] * n[2];
    } else {
        double FT[3];
        mortar_project<3>(m, ms, a.mf + 9, FT);
        a.dC[4][ms] = vdot3(FT, n);
    }
}

__global__ void __launch_bounds__(256) k_seg_prep(const NsemDev m, SegArgs a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n_int) return;
    const double r = a.rho_o[i];
    const double U[3] = {a.U[0][i], a.U[1][i], a.U[2][i]};
    const double Tf = a.Tp[i] + m.T0;
    a.Tf[i] = Tf;
    for (int c = 0; c < 3; c++) a.Fc[c][i] = r * U[c];
    a.mu[i] = sqrt(vdot3(U, U));
    a.cs[i] = sqrt(m.gR * Tf);
}

__global__ void __launch_bounds__(256) k_seg_face_rho(const NsemDev m, SegArgs a) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.n_slot) return;
    const int32_t c1 = m.c1[k], c2 = m.c2[k];
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    const double en[3] = {m.en[k], m.en[m.n_slot + k], m.en[2 * m.n_slot + k]};
    const double fi = m.fi[k], fo = 1 - fi;
    const double r1 = a.rho_o[c1];
    const double U1[3] = {a.U[0][c1], a.U[1][c1], a.U[2][c1]};
    const double mu1 = a.mu[c1], cs1 = a.cs[c1];
    double r2, U2[3], mu2, cs2;
    if (c2 >= 0) {
        r2 = a.rho_o[c2];
        U2[0] = a.U[0][c2]; U2[1] = a.U[1][c2]; U2[2] = a.U[2][c2];
        mu2 = a.mu[c2]; cs2 = a.cs[c2];
    } else {
        r2 = r1 + 0.0;
        ghost_U(m, k, n, U1, U2);
        mu2 = sqrt(vdot3(U2, U2));
        cs2 = sqrt(m.gR * (a.Tf[c1] + 0.0));
    }
    double X1[3], X2[3];
    for (int c = 0; c < 3; c++) {
        X1[c] = U1[c] * r1;
        X2[c] = U2[c] * r2;
    }
    /* a mortar's coarse side: interpolated from the coarse face's nodes */
    const int32_t ms = m.n_ms ? m.ms_of[k] : -1;
    double mu1v = mu1, cs1v = cs1, r1v = r1;
    if (ms >= 0) {
        if (ms_field(m, NSEM_MS_SIDE, ms) == 1) {
            mu1v = a.mq[0][ms];
            cs1v = a.mq[1][ms];
            for (int c = 0; c < 3; c++) X1[c] = a.mq[2 + c][ms];
            r1v = a.mq[5][ms];
        } else {
            mu2 = a.mq[0][ms];
            cs2 = a.mq[1][ms];
            for (int c = 0; c < 3; c++) X2[c] = a.mq[2 + c][ms];
            r2 = a.mq[5][ms];
        }
    }
    const double lam = ((mu1v * fi + mu2 * fo) + (cs1v * fi + cs2 * fo)) / 2;
    a.lam[k] = lam;
    double F[3];
    const double jump = lam * (r2 - r1v);
    for (int c = 0; c < 3; c++) F[c] = (X1[c] * fi + X2[c] * fo) - en[c] * jump;
    a.d[0][k] = vdot3(F, n);
    if (ms >= 0)
        for (int c = 0; c < 3; c++) a.mf[c][ms] = F[c];
}

/* weak volume term of one node, sources in the reference's scatter order */
template <int W, int JOFF, typename Apply>
__device__ __forceinline__ void volume_gather(const NsemDev& m, const double* sm, const double* dps,
                                              int t, Apply apply) {
    nsem_volume_gather<W, JOFF>(m.npx, m.npy, m.npz, sm, dps, t, apply);
}

/* inputs and outputs of the strong-form gradients of U and theta */
struct GradArgs {
    const double* U[3];
    const double* Tf;        /* full potential temperature */
    double* G[12];           /* per node: grad U (XX..ZX), grad theta */
    double* fF[4];           /* per slot: cds(U), cds(theta) */
    double* gC[4];           /* per mortar slot: the projection onto the coarse side */
};

/* mortar faces: cds(U), cds(theta) with the coarse side interpolated (over
 * the conforming values of k_seg_grad_face), then projected back */
__global__ void __launch_bounds__(128) k_seg_mortar_gcds(const NsemDev m, GradArgs a) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    double I[4];
    mortar_interp<4>(m, ms, [&](int64_t node, double* v) {
        for (int c = 0; c < 3; c++) v[c] = a.U[c][node];
        v[3] = a.Tf[node];
    }, I);
    const int64_t k = ms_field(m, NSEM_MS_K, ms);
    const bool own = ms_field(m, NSEM_MS_SIDE, ms) == 1;
    const double fi = m.fi[k], fo = 1 - fi;
    const int64_t fine = own ? m.c2[k] : m.c1[k];
    for (int c = 0; c < 4; c++) {
        const double pf = c < 3 ? a.U[c][fine] : a.Tf[fine];
        const double p1 = own ? I[c] : pf, p2 = own ? pf : I[c];
        a.fF[c][k] = (p1 * fi) + (p2 * fo);
    }
}

__global__ void __launch_bounds__(128) k_seg_mortar_ggather(const NsemDev m, GradArgs a) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    const int Na = ms_field(m, NSEM_MS_NA, ms), Nb = ms_field(m, NSEM_MS_NB, ms),
              na = ms_field(m, NSEM_MS_IA, ms), nb = ms_field(m, NSEM_MS_IB, ms),
              first = ms_field(m, NSEM_MS_FIRST, ms);
    const double* Pa = m.psic + ms_field(m, NSEM_MS_TA, ms) * NSEM_MAX_NPD * NSEM_MAX_NPD;
    const double* Pb = m.psic + ms_field(m, NSEM_MS_TB, ms) * NSEM_MAX_NPD * NSEM_MAX_NPD;
    double out[4] = {0.0, 0.0, 0.0, 0.0};
    for (int ja = 0; ja < Na; ja++)
        for (int jb = 0; jb < Nb; jb++) {
            const int64_t k2 = ms_field(m, NSEM_MS_K, first + ja * Nb + jb);
            const double fa = Pa[ja * Na + na], fb = Pb[jb * Nb + nb];
            for (int c = 0; c < 4; c++) out[c] += a.fF[c][k2] * fa * fb;
        }
    for (int c = 0; c < 4; c++) a.gC[c][ms] = out[c];
}

/* cds(U), cds(theta) per slot for the gradients */
__global__ void __launch_bounds__(256) k_seg_grad_face(const NsemDev m, GradArgs a) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.n_slot) return;
    const int32_t c1 = m.c1[k], c2 = m.c2[k];
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    const double fi = m.fi[k], fo = 1 - fi;
    const double U1[3] = {a.U[0][c1], a.U[1][c1], a.U[2][c1]};
    const double T1 = a.Tf[c1];
    double U2[3], T2;
    if (c2 >= 0) {
        U2[0] = a.U[0][c2]; U2[1] = a.U[1][c2]; U2[2] = a.U[2][c2];
        T2 = a.Tf[c2];
    } else {
        ghost_U(m, k, n, U1, U2);
        T2 = T1 + 0.0;
    }
    for (int c = 0; c < 3; c++) a.fF[c][k] = (U1[c] * fi) + (U2[c] * fo);
    a.fF[3][k] = (T1 * fi) + (T2 * fo);
}

constexpr int W_GRAD = 13;   /* U[3] theta jin[9] */

__global__ void k_seg_grad_vol(const NsemDev m, const NsemTables tab, GradArgs a) {
    extern __shared__ double sm[];
    const int NP = m.np, NPX = m.npx, NPY = m.npy, NPZ = m.npz;
    double* dps = sm + (size_t)NP * W_GRAD;
    const int t = threadIdx.x;
    for (int q = t; q < 3 * NSEM_MAX_NPD * NSEM_MAX_NPD; q += blockDim.x)
        dps[q] = (&tab.dpsi[0][0])[q];
    const int64_t e = blockIdx.x;
    const bool active = t < NP;
    const int64_t node = e * NP + t;
    if (active) {
        double* my = sm + (size_t)t * W_GRAD;
        for (int c = 0; c < 3; c++) my[c] = a.U[c][node];
        my[3] = a.Tf[node];
        for (int c = 0; c < 9; c++) my[4 + c] = m.jin[(int64_t)c * m.n_int + node];
    }
    __syncthreads();
    if (!active) return;
    const double* me = sm + (size_t)t * W_GRAD;
    double gU[9], gT[3];
    for (int c = 0; c < 9; c++) gU[c] = 0.0;
    for (int c = 0; c < 3; c++) gT[c] = 0.0;
    /* face terms, in the cell's face order; a mortar's coarse side takes the
     * projected face values */
    for (int j = 0; j < m.n_lift; j++) {
        const int32_t code = m.lift[(int64_t)j * m.n_int + node];
        if (code < 0) break;
        const int64_t idx = code >> 2;
        const bool coarse = code & 2;
        const int64_t k = coarse ? ms_field(m, NSEM_MS_K, idx) : idx;
        double f4[4];
        for (int c = 0; c < 4; c++) f4[c] = coarse ? a.gC[c][idx] : a.fF[c][k];
        const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
        const double dU[3] = {f4[0] - me[0], f4[1] - me[1], f4[2] - me[2]};
        const double dT = f4[3] - me[3];
        double tU[9];
        outer(n, dU, tU);
        if (code & 1) {
            for (int c = 0; c < 9; c++) gU[c] -= tU[c];
            for (int c = 0; c < 3; c++) gT[c] -= n[c] * dT;
        } else {
            for (int c = 0; c < 9; c++) gU[c] += tU[c];
            for (int c = 0; c < 3; c++) gT[c] += n[c] * dT;
        }
    }
    /* volume derivative at the node: sources on the x line (self included),
     * then the y and z lines (field.h:3338-3356) */
    const int ia = t / (NPY * NPZ), ja = (t / NPZ) % NPY, ka = t % NPZ;
    const double* J = me + 4;
    const double* Dx = dps;
    const double* Dy = dps + NSEM_MAX_NPD * NSEM_MAX_NPD;
    const double* Dz = dps + 2 * NSEM_MAX_NPD * NSEM_MAX_NPD;
    auto add = [&](int lb, const double* dj) {
        const double* sb = sm + (size_t)lb * W_GRAD;
        double tU[9];
        outer(dj, sb, tU);
        for (int c = 0; c < 9; c++) gU[c] += tU[c];
        for (int c = 0; c < 3; c++) gT[c] += dj[c] * sb[3];
    };
    const int sx = NPY * NPZ, sy = NPZ;
    /* every thread runs the same trip counts: the node's own term is selected
     * on the x line, and the y and z loops map past the node's index */
    double dj_self[3];
    {
        const double dv[3] = {Dx[ia * NPX + ia], Dy[ja * NPY + ja], Dz[ka * NPZ + ka]};
        tdot(J, dv, dj_self);
    }
    for (int ii = 0; ii < NPX; ii++) {
        const double D = Dx[ia * NPX + ii];
        const bool self = ii == ia;
        const double dj[3] = {self ? dj_self[0] : J[XX] * D, self ? dj_self[1] : J[YX] * D,
                              self ? dj_self[2] : J[ZX] * D};
        add(t + (ii - ia) * sx, dj);
    }
    for (int q = 0; q + 1 < NPY; q++) {
        const int jj = q < ja ? q : q + 1;
        const double D = Dy[ja * NPY + jj];
        const double dj[3] = {J[XY] * D, J[YY] * D, J[ZY] * D};
        add(t + (jj - ja) * sy, dj);
    }
    for (int q = 0; q + 1 < NPZ; q++) {
        const int kk = q < ka ? q : q + 1;
        const double D = Dz[ka * NPZ + kk];
        const double dj[3] = {J[XZ] * D, J[YZ] * D, J[ZZ] * D};
        add(t + (kk - ka), dj);
    }
    const double cv = m.cv[node];
    for (int c = 0; c < 9; c++) a.G[c][node] = gU[c] / cv;
    for (int c = 0; c < 3; c++) a.G[9 + c][node] = gT[c] / cv;
}

constexpr int W_RHO = 12;   /* fr[3] jin[9] */
constexpr int W_UT = 21;    /* fm[9] ft[3] jin[9] */

__global__ void k_seg_vol_rho(const NsemDev m, const NsemTables tab, SegArgs a) {
    extern __shared__ double sm[];
    const int NP = m.np;
    double* dps = sm + (size_t)NP * W_RHO;
    const int t = threadIdx.x;
    for (int q = t; q < 3 * NSEM_MAX_NPD * NSEM_MAX_NPD; q += blockDim.x)
        dps[q] = (&tab.dpsi[0][0])[q];
    const int64_t e = blockIdx.x;
    const bool active = t < NP;
    const int64_t node = e * NP + t;
    double rho = 0;
    if (active) {
        rho = a.rho_o[node];
        double* my = sm + (size_t)t * W_RHO;
        for (int c = 0; c < 3; c++) my[c] = a.U[c][node] * rho;     /* U * rho */
        for (int c = 0; c < 9; c++) my[3 + c] = m.jin[(int64_t)c * m.n_int + node];
    }
    __syncthreads();
    if (!active) return;
    double r = 0.0;
    for (int j = 0; j < m.n_lift; j++) {
        const int32_t code = m.lift[(int64_t)j * m.n_int + node];
        if (code < 0) break;
        const int64_t idx = code >> 2;
        const double v = (code & 2) ? a.dC[0][idx] : a.d[0][idx];
        if (code & 1) r -= v;
        else r += v;
    }
    volume_gather<W_RHO, 3>(m, sm, dps, t, [&](int lb, const double* dj) {
        r -= vdot3(sm + (size_t)lb * W_RHO, dj);
    });
    const double cv = m.cv[node];
    const double ap = a.c_dt * cv;
    const double rn = (r + rho * ap) / (0.0 + ap);
    a.rho_n[node] = rn;
    const double p = m.P0 * nsem_pow(((rn * a.Tf[node]) * m.R) / m.P0, m.gamma);
    a.pp[node] = p - m.p_ref[node];
}

__global__ void __launch_bounds__(256) k_seg_face_ut(const NsemDev m, SegArgs a) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.n_slot) return;
    const int32_t c1 = m.c1[k], c2 = m.c2[k];
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    const double en[3] = {m.en[k], m.en[m.n_slot + k], m.en[2 * m.n_slot + k]};
    const double fi = m.fi[k], fo = 1 - fi;
    const double lam = a.lam[k];
    const double r1 = a.rho_n[c1];
    const double U1[3] = {a.U[0][c1], a.U[1][c1], a.U[2][c1]};
    const double Fc1[3] = {a.Fc[0][c1], a.Fc[1][c1], a.Fc[2][c1]};
    const double T1 = a.Tf[c1], p1 = a.pp[c1];
    double r2, U2[3], Fc2[3], T2, p2;
    if (c2 >= 0) {
        r2 = a.rho_n[c2];
        for (int c = 0; c < 3; c++) { U2[c] = a.U[c][c2]; Fc2[c] = a.Fc[c][c2]; }
        T2 = a.Tf[c2];
        p2 = a.pp[c2];
    } else {
        r2 = r1 + 0.0;
        ghost_U(m, k, n, U1, U2);
        const double ro2 = a.rho_o[c1] + 0.0;
        for (int c = 0; c < 3; c++) Fc2[c] = ro2 * U2[c];
        T2 = T1 + 0.0;
        p2 = p1;
    }
    /* artificial viscosity mu = rho^n nu; the wall ghosts' gradient is zero */
    const double mu1 = a.visc ? a.rho_o[c1] * m.nu : 0.0;
    const double mu2 = a.visc ? (c2 >= 0 ? a.rho_o[c2] : a.rho_o[c1] + 0.0) * m.nu : 0.0;
    /* a mortar's coarse side: interpolated from the coarse face's nodes */
    const int32_t ms = m.n_ms ? m.ms_of[k] : -1;
    const int mside = ms >= 0 ? ms_field(m, NSEM_MS_SIDE, ms) : 0;
    /* U equation: flux Fc (x) U + p' I - mu grad U, state rho U */
    {
        double A[9], B[9], O[9], F[9], dq[3], out[3], q1[3], q2[3];
        outer(Fc1, U1, A);
        outer(Fc2, U2, B);
        for (int c = 0; c < 9; c++) {
            const double i1 = (c < 3) ? 1.0 : 0.0;
            A[c] = A[c] + i1 * p1;
            B[c] = B[c] + i1 * p2;
        }
        if (a.visc)
            for (int c = 0; c < 9; c++) {
                A[c] = A[c] - mu1 * a.G[c][c1];
                B[c] = B[c] - mu2 * (c2 >= 0 ? a.G[c][c2] : 0.0);
            }
        for (int c = 0; c < 3; c++) {
            q1[c] = r1 * U1[c];
            q2[c] = r2 * U2[c];
        }
        if (mside == 1) {
            for (int c = 0; c < 9; c++) A[c] = a.mq[c][ms];
            for (int c = 0; c < 3; c++) q1[c] = a.mq[9 + c][ms];
        } else if (mside == 2) {
            for (int c = 0; c < 9; c++) B[c] = a.mq[c][ms];
            for (int c = 0; c < 3; c++) q2[c] = a.mq[9 + c][ms];
        }
        for (int c = 0; c < 3; c++) dq[c] = (q2[c] - q1[c]) * lam;
        outer(en, dq, O);
        for (int c = 0; c < 9; c++) F[c] = (A[c] * fi + B[c] * fo) - O[c];
        tdot(F, n, out);
        a.d[1][k] = out[0];
        a.d[2][k] = out[1];
        a.d[3][k] = out[2];
        if (mside)
            for (int c = 0; c < 9; c++) a.mf[c][ms] = F[c];
    }
    /* T equation: flux Fc theta - (mu / Pr) grad theta, state rho theta */
    {
        double F[3], x[3], y[3];
        double s1 = r1 * T1, s2 = r2 * T2;
        for (int c = 0; c < 3; c++) {
            x[c] = Fc1[c] * T1;
            y[c] = Fc2[c] * T2;
            if (a.visc) {
                x[c] = x[c] - (mu1 * m.iPr) * a.G[9 + c][c1];
                y[c] = y[c] - (mu2 * m.iPr) * (c2 >= 0 ? a.G[9 + c][c2] : 0.0);
            }
        }
        if (mside == 1) {
            for (int c = 0; c < 3; c++) x[c] = a.mq[12 + c][ms];
            s1 = a.mq[15][ms];
        } else if (mside == 2) {
            for (int c = 0; c < 3; c++) y[c] = a.mq[12 + c][ms];
            s2 = a.mq[15][ms];
        }
        const double jump = lam * (s2 - s1);
        for (int c = 0; c < 3; c++) F[c] = (x[c] * fi + y[c] * fo) - en[c] * jump;
        a.d[4][k] = vdot3(F, n);
        if (mside)
            for (int c = 0; c < 3; c++) a.mf[9 + c][ms] = F[c];
    }
}

__global__ void k_seg_vol_ut(const NsemDev m, const NsemTables tab, SegArgs a) {
    extern __shared__ double sm[];
    const int NP = m.np;
    double* dps = sm + (size_t)NP * W_UT;
    const int t = threadIdx.x;
    for (int q = t; q < 3 * NSEM_MAX_NPD * NSEM_MAX_NPD; q += blockDim.x)
        dps[q] = (&tab.dpsi[0][0])[q];
    const int64_t e = blockIdx.x;
    const bool active = t < NP;
    const int64_t node = e * NP + t;
    double U[3] = {0, 0, 0}, Tf = 0;
    if (active) {
        double* my = sm + (size_t)t * W_UT;
        double Fc[3];
        for (int c = 0; c < 3; c++) { U[c] = a.U[c][node]; Fc[c] = a.Fc[c][node]; }
        Tf = a.Tf[node];
        const double p = a.pp[node];
        outer(Fc, U, my);
        for (int c = 0; c < 9; c++) my[c] = my[c] + ((c < 3) ? 1.0 : 0.0) * p;
        for (int c = 0; c < 3; c++) my[9 + c] = Fc[c] * Tf;
        if (a.visc) {
            const double mu = a.rho_o[node] * m.nu;
            for (int c = 0; c < 9; c++) my[c] = my[c] - mu * a.G[c][node];
            for (int c = 0; c < 3; c++) my[9 + c] = my[9 + c] - (mu * m.iPr) * a.G[9 + c][node];
        }
        for (int c = 0; c < 9; c++) my[12 + c] = m.jin[(int64_t)c * m.n_int + node];
    }
    __syncthreads();
    if (!active) return;
    double r1 = 0.0, r2 = 0.0, r3 = 0.0, r4 = 0.0;
    for (int j = 0; j < m.n_lift; j++) {
        const int32_t code = m.lift[(int64_t)j * m.n_int + node];
        if (code < 0) break;
        const int64_t idx = code >> 2;
        double v1, v2, v3, v4;
        if (code & 2) {
            v1 = a.dC[1][idx]; v2 = a.dC[2][idx]; v3 = a.dC[3][idx]; v4 = a.dC[4][idx];
        } else {
            v1 = a.d[1][idx]; v2 = a.d[2][idx]; v3 = a.d[3][idx]; v4 = a.d[4][idx];
        }
        if (code & 1) {
            r1 -= v1; r2 -= v2; r3 -= v3; r4 -= v4;
        } else {
            r1 += v1; r2 += v2; r3 += v3; r4 += v4;
        }
    }
    volume_gather<W_UT, 12>(m, sm, dps, t, [&](int lb, const double* dj) {
        const double* sb = sm + (size_t)lb * W_UT;
        double tv[3];
        tdot(sb, dj, tv);
        r1 -= tv[0]; r2 -= tv[1]; r3 -= tv[2];
        r4 -= vdot3(sb + 9, dj);
    });
    const double cv = m.cv[node];
    const double rn = a.rho_n[node];
    const double ro = a.rho_o[node];
    const double s = rn - m.rho_ref[node];
    const double ap0 = a.c_dt * cv;
    const double ap = ap0 * rn;
    const double r[3] = {r1, r2, r3};
    bool finite = isfinite(rn);
    for (int c = 0; c < 3; c++) {
        const double sc = 0.0 + m.g[c] * s;
        const double su = r[c] - sc * cv;
        const double un = (su + (U[c] * ro) * ap0) / (0.0 + ap);
        a.U[c][node] = un;
        finite = finite && isfinite(un);
    }
    const double Tn = (r4 + (Tf * ro) * ap0) / (0.0 + ap);
    a.Tp[node] = Tn - m.T0;
    finite = finite && isfinite(Tn);
    if (!finite) atomicOr(m.status, NSEM_STATUS_NONFINITE);
}

/* conversions between the primitive fields and the conserved state */
struct ConvArgs {
    const double* rho;
    double* rho_w;
    double* U[3];
    double* Tp;
    double* u[5];
};

__global__ void __launch_bounds__(256) k_seg_to_cons(const NsemDev m, ConvArgs a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n_int) return;
    const double r = a.rho[i];
    a.u[0][i] = r;
    for (int c = 0; c < 3; c++) a.u[1 + c][i] = r * a.U[c][i];
    a.u[4][i] = r * (a.Tp[i] + m.T0);
}

__global__ void __launch_bounds__(256) k_cons_to_seg(const NsemDev m, ConvArgs a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n_int) return;
    const double r = a.u[0][i];
    a.rho_w[i] = r;
    for (int c = 0; c < 3; c++) a.U[c][i] = a.u[1 + c][i] / r;
    a.Tp[i] = a.u[4][i] / r - m.T0;
}

SegArgs seg_args(const NsemDev* m, NsemSegBuf* b, int cur, double dt) {
    SegArgs a;
    a.rho_o = b->rho[cur];
    a.rho_n = b->rho[cur ^ 1];
    for (int c = 0; c < 3; c++) { a.U[c] = b->U[c]; a.Fc[c] = b->Fc[c]; }
    a.Tp = b->Tp;
    a.Tf = b->Tf;
    a.mu = b->mu;
    a.cs = b->cs;
    a.pp = b->pp;
    a.lam = b->lam;
    for (int c = 0; c < 5; c++) a.d[c] = b->d[c];
    for (int c = 0; c < 12; c++) a.G[c] = b->G[c];
    for (int c = 0; c < 4; c++) a.fF[c] = b->fF[c];
    for (int c = 0; c < 16; c++) a.mq[c] = b->mq[c];
    for (int c = 0; c < 12; c++) a.mf[c] = b->mf[c];
    for (int c = 0; c < 5; c++) a.dC[c] = b->dC[c];
    for (int c = 0; c < 4; c++) a.gC[c] = b->gC[c];
    a.c_dt = -1.0 / dt;
    a.visc = m->nu != 0.0;
    return a;
}

size_t smem_rho(const NsemDev* m) {
    return ((size_t)m->np * W_RHO + 3 * NSEM_MAX_NPD * NSEM_MAX_NPD) * sizeof(double);
}
size_t smem_grad(const NsemDev* m) {
    return ((size_t)m->np * W_GRAD + 3 * NSEM_MAX_NPD * NSEM_MAX_NPD) * sizeof(double);
}
size_t smem_ut(const NsemDev* m) {
    return ((size_t)m->np * W_UT + 3 * NSEM_MAX_NPD * NSEM_MAX_NPD) * sizeof(double);
}


/* ------------------------------------------------------------ convection */

struct AdvArgs {
    const double* T_o;
    double* T_n;
    const double* U[3];
    const double* Ug[3];   /* analytic wind at each slot's ghost (or null: bc_U) */
    double* lam;
    double* d;
    double* mq[4];
    double* mf[3];
    double* dC;
    double* R_n;           /* AB2: this step's right-hand side (or null)        */
    const double* R_o;     /* AB2: the previous step's                          */
    int ab2;               /* AB2 update (field.h:3796-3798)                    */
    double c_dt;
};

/* the step's analytic wind: U = A s for the horizontal components (the app
 * forms u, v as the spatial part times cos(pi t / T) and sets w = 0,
 * convection.cpp:86-91), on interior nodes and at each used slot's ghost */
__global__ void k_conv_wind(const NsemDev m, NsemConvBuf b, double s) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m.n_int)
        for (int c = 0; c < 3; c++) b.U[c][i] = c < 2 ? b.A[c][i] * s : b.A[c][i];
    if (i < m.n_slot)
        for (int c = 0; c < 3; c++) b.Ug[c][i] = c < 2 ? b.Ag[c][i] * s : b.Ag[c][i];
}

/* non-conforming faces: the coarse side's |U| (stage 0) or U T, T (stage 1)
 * interpolated onto each mortar slot, one thread per (slot, quantity) */
template <int STAGE>
__global__ void __launch_bounds__(128) k_conv_mortar(const NsemDev m, AdvArgs a) {
    const int nq = STAGE == 0 ? 1 : 4;
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nq * m.n_ms) return;
    const int64_t ms = id / nq;
    const int c = (int)(id % nq);
    double out[1];
    mortar_interp<1>(m, ms, [&](int64_t node, double* v) {
        if (STAGE == 0) {
            const double U[3] = {a.U[0][node], a.U[1][node], a.U[2][node]};
            v[0] = sqrt(vdot3(U, U));
        } else {
            v[0] = c < 3 ? a.U[c][node] * a.T_o[node] : a.T_o[node];
        }
    }, out);
    a.mq[c][ms] = out[0];
}

__global__ void __launch_bounds__(128) k_conv_mortar_gather(const NsemDev m, AdvArgs a) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    const int64_t k = ms_field(m, NSEM_MS_K, ms);
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    double F[3];
    mortar_project<3>(m, ms, a.mf, F);
    a.dC[ms] = vdot3(F, n);
}

__global__ void __launch_bounds__(256) k_conv_lambda(const NsemDev m, AdvArgs a) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.n_slot) return;
    const int32_t c1 = m.c1[k], c2 = m.c2[k];
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    const double fi = m.fi[k], fo = 1 - fi;
    const double U1[3] = {a.U[0][c1], a.U[1][c1], a.U[2][c1]};
    double U2[3];
    if (c2 >= 0) {
        U2[0] = a.U[0][c2]; U2[1] = a.U[1][c2]; U2[2] = a.U[2][c2];
    } else if (a.Ug[0]) {
        U2[0] = a.Ug[0][k]; U2[1] = a.Ug[1][k]; U2[2] = a.Ug[2][k];
    } else {
        ghost_U(m, k, n, U1, U2);
    }
    double u1 = sqrt(vdot3(U1, U1)), u2 = sqrt(vdot3(U2, U2));
    const int32_t ms = m.n_ms ? m.ms_of[k] : -1;
    if (ms >= 0) {
        if (ms_field(m, NSEM_MS_SIDE, ms) == 1) u1 = a.mq[0][ms];
        else u2 = a.mq[0][ms];
    }
    a.lam[k] = (u1 * fi + u2 * fo) / 2;
}

__global__ void __launch_bounds__(256) k_conv_face(const NsemDev m, AdvArgs a) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.n_slot) return;
    const int32_t c1 = m.c1[k], c2 = m.c2[k];
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    const double en[3] = {m.en[k], m.en[m.n_slot + k], m.en[2 * m.n_slot + k]};
    const double fi = m.fi[k], fo = 1 - fi;
    const double U1[3] = {a.U[0][c1], a.U[1][c1], a.U[2][c1]};
    const double T1 = a.T_o[c1];
    double U2[3], T2;
    if (c2 >= 0) {
        U2[0] = a.U[0][c2]; U2[1] = a.U[1][c2]; U2[2] = a.U[2][c2];
        T2 = a.T_o[c2];
    } else {
        if (a.Ug[0]) {
            U2[0] = a.Ug[0][k]; U2[1] = a.Ug[1][k]; U2[2] = a.Ug[2][k];
        } else {
            ghost_U(m, k, n, U1, U2);
        }
        T2 = T1 + 0.0;
    }
    double X1[3], X2[3];
    for (int c = 0; c < 3; c++) {
        X1[c] = U1[c] * T1;
        X2[c] = U2[c] * T2;
    }
    const int32_t ms = m.n_ms ? m.ms_of[k] : -1;
    const int side = ms >= 0 ? ms_field(m, NSEM_MS_SIDE, ms) : 0;
    double T1v = T1, T2v = T2;
    if (side == 1) {
        for (int c = 0; c < 3; c++) X1[c] = a.mq[c][ms];
        T1v = a.mq[3][ms];
    } else if (side == 2) {
        for (int c = 0; c < 3; c++) X2[c] = a.mq[c][ms];
        T2v = a.mq[3][ms];
    }
    double F[3];
    const double jump = a.lam[k] * (T2v - T1v);
    for (int c = 0; c < 3; c++) F[c] = (X1[c] * fi + X2[c] * fo) - en[c] * jump;
    a.d[k] = vdot3(F, n);
    if (side)
        for (int c = 0; c < 3; c++) a.mf[c][ms] = F[c];
}

constexpr int W_CONV = 12;   /* fv[3] jin[9] */

__global__ void k_conv_vol(const NsemDev m, const NsemTables tab, AdvArgs a) {
    extern __shared__ double sm[];
    const int NP = m.np;
    double* dps = sm + (size_t)NP * W_CONV;
    const int t = threadIdx.x;
    for (int q = t; q < 3 * NSEM_MAX_NPD * NSEM_MAX_NPD; q += blockDim.x)
        dps[q] = (&tab.dpsi[0][0])[q];
    const int64_t e = blockIdx.x;
    const bool active = t < NP;
    const int64_t node = e * NP + t;
    double T = 0;
    if (active) {
        T = a.T_o[node];
        double* my = sm + (size_t)t * W_CONV;
        for (int c = 0; c < 3; c++) my[c] = a.U[c][node] * T;
        for (int c = 0; c < 9; c++) my[3 + c] = m.jin[(int64_t)c * m.n_int + node];
    }
    __syncthreads();
    if (!active) return;
    double r = 0.0;
    for (int j = 0; j < m.n_lift; j++) {
        const int32_t code = m.lift[(int64_t)j * m.n_int + node];
        if (code < 0) break;
        const int64_t k = code >> 2;
        const double v = (code & 2) ? a.dC[k] : a.d[k];
        if (code & 1) r -= v;
        else r += v;
    }
    volume_gather<W_CONV, 3>(m, sm, dps, t, [&](int lb, const double* dj) {
        r -= vdot3(sm + (size_t)lb * W_CONV, dj);
    });
    const double ap = a.c_dt * m.cv[node];
    double Tn;
    if (a.ab2) {
        /* AB2: Su = T ap + (3 R^n - R^{n-1}) / 2, T = Su / ap */
        Tn = (T * ap + (3.0 * r - a.R_o[node]) / 2.0) / ap;
    } else {
        /* BDF1 / AB1 (the same sum in either order): T = (R + T ap) / ap */
        Tn = (r + T * ap) / (0.0 + ap);
    }
    if (a.R_n) a.R_n[node] = r;
    a.T_n[node] = Tn;
    if (!isfinite(Tn)) atomicOr(m.status, NSEM_STATUS_NONFINITE);
}

size_t smem_conv(const NsemDev* m) {
    return ((size_t)m->np * W_CONV + 3 * NSEM_MAX_NPD * NSEM_MAX_NPD) * sizeof(double);
}

AdvArgs adv_args(NsemConvBuf* b, int cur, double dt) {
    AdvArgs a;
    a.T_o = b->T[cur];
    a.T_n = b->T[cur ^ 1];
    for (int c = 0; c < 3; c++) a.U[c] = b->U[c];
    for (int c = 0; c < 3; c++) a.Ug[c] = b->analytic ? b->Ug[c] : nullptr;
    a.R_n = nullptr;
    a.R_o = nullptr;
    a.ab2 = 0;
    a.lam = b->lam;
    a.d = b->d;
    for (int c = 0; c < 4; c++) a.mq[c] = b->mq[c];
    for (int c = 0; c < 3; c++) a.mf[c] = b->mf[c];
    a.dC = b->dC;
    a.c_dt = -1.0 / dt;
    return a;
}

}  // namespace

int nsem_grad_ut_mortar(const NsemDev* m, const NsemTables* t, const double* const* U,
                        const double* T, double* const* G, double* const* fF, double* const* gC,
                        void* stream) {
    GradArgs ga;
    for (int c = 0; c < 3; c++) ga.U[c] = U[c];
    ga.Tf = T;
    for (int c = 0; c < 12; c++) ga.G[c] = G[c];
    for (int c = 0; c < 4; c++) ga.fF[c] = fF[c];
    for (int c = 0; c < 4; c++) ga.gC[c] = gC ? gC[c] : nullptr;
    cudaStream_t st = (cudaStream_t)stream;
    const int threads = ((m->np + 31) / 32) * 32;
    k_seg_grad_face<<<(unsigned)((m->n_slot + 255) / 256), 256, 0, st>>>(*m, ga);
    if (m->n_ms > 0 && gC) {
        const unsigned mb = (unsigned)((m->n_ms + 127) / 128);
        k_seg_mortar_gcds<<<mb, 128, 0, st>>>(*m, ga);
        k_seg_mortar_ggather<<<mb, 128, 0, st>>>(*m, ga);
    }
    k_seg_grad_vol<<<(unsigned)m->n_elem, threads, smem_grad(m), st>>>(*m, *t, ga);
    return (int)cudaGetLastError();
}

int nsem_grad_ut(const NsemDev* m, const NsemTables* t, const double* const* U, const double* T,
                 double* const* G, double* const* fF, void* stream) {
    return nsem_grad_ut_mortar(m, t, U, T, G, fF, nullptr, stream);
}

int nsem_grad_mortar_faces(const NsemDev* m, const double* const* U, const double* T,
                           double* const* fF, double* const* gC, void* stream) {
    if (m->n_ms == 0) return 0;
    GradArgs ga{};
    for (int c = 0; c < 3; c++) ga.U[c] = U[c];
    ga.Tf = T;
    for (int c = 0; c < 4; c++) { ga.fF[c] = fF[c]; ga.gC[c] = gC[c]; }
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned mb = (unsigned)((m->n_ms + 127) / 128);
    k_seg_mortar_gcds<<<mb, 128, 0, st>>>(*m, ga);
    k_seg_mortar_ggather<<<mb, 128, 0, st>>>(*m, ga);
    return (int)cudaGetLastError();
}

int nsem_grad_vol(const NsemDev* m, const NsemTables* t, const double* const* U, const double* T,
                  double* const* G, const double* const* fF, const double* const* gC, void* stream) {
    GradArgs ga;
    for (int c = 0; c < 3; c++) ga.U[c] = U[c];
    ga.Tf = T;
    for (int c = 0; c < 12; c++) ga.G[c] = G[c];
    for (int c = 0; c < 4; c++) ga.fF[c] = const_cast<double*>(fF[c]);
    for (int c = 0; c < 4; c++) ga.gC[c] = gC ? const_cast<double*>(gC[c]) : nullptr;
    const int threads = ((m->np + 31) / 32) * 32;
    k_seg_grad_vol<<<(unsigned)m->n_elem, threads, smem_grad(m), (cudaStream_t)stream>>>(*m, *t, ga);
    return (int)cudaGetLastError();
}

int nsem_conv_lambda(const NsemDev* m, NsemConvBuf* b, void* stream) {
    const AdvArgs a = adv_args(b, b->cur, 1.0);
    if (m->n_ms > 0)
        k_conv_mortar<0><<<(unsigned)((m->n_ms + 127) / 128), 128, 0, (cudaStream_t)stream>>>(*m, a);
    k_conv_lambda<<<(unsigned)((m->n_slot + 255) / 256), 256, 0, (cudaStream_t)stream>>>(*m, a);
    return (int)cudaGetLastError();
}

int nsem_conv_steps(const NsemDev* m, const NsemTables* t, NsemConvBuf* b, int nsteps, double dt,
                    void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned sb = (unsigned)((m->n_slot + 255) / 256);
    const int threads = ((m->np + 31) / 32) * 32;
    int cur = b->cur;
    for (int s = 0; s < nsteps; s++) {
        const AdvArgs a = adv_args(b, cur, dt);
        const unsigned mb = (unsigned)((m->n_ms + 127) / 128);
        if (m->n_ms > 0) k_conv_mortar<1><<<4 * mb, 128, 0, st>>>(*m, a);
        k_conv_face<<<sb, 256, 0, st>>>(*m, a);
        if (m->n_ms > 0) k_conv_mortar_gather<<<mb, 128, 0, st>>>(*m, a);
        k_conv_vol<<<(unsigned)m->n_elem, threads, smem_conv(m), st>>>(*m, *t, a);
        const int e = (int)cudaGetLastError();
        if (e) return e;
        cur ^= 1;
    }
    return 0;
}

int nsem_conv_steps_wind(const NsemDev* m, const NsemTables* t, NsemConvBuf* b, int nsteps,
                         double dt, const double* scale, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned sb = (unsigned)((m->n_slot + 255) / 256);
    const int threads = ((m->np + 31) / 32) * 32;
    const int64_t nw = m->n_int > m->n_slot ? m->n_int : m->n_slot;
    for (int s = 0; s < nsteps; s++) {
        if (b->analytic) {
            k_conv_wind<<<(unsigned)((nw + 255) / 256), 256, 0, st>>>(*m, *b, scale ? scale[s] : 1.0);
            int e = (int)cudaGetLastError();
            if (!e) e = nsem_conv_lambda(m, b, stream);
            if (e) return e;
        }
        AdvArgs a = adv_args(b, b->cur, dt);
        if (b->order == 2) {
            /* the first step of a run is AB1 (one right-hand side stored) */
            a.R_n = b->R[b->hist & 1];
            a.R_o = b->R[(b->hist + 1) & 1];
            a.ab2 = b->hist >= 1;
        }
        const unsigned mb = (unsigned)((m->n_ms + 127) / 128);
        if (m->n_ms > 0) k_conv_mortar<1><<<4 * mb, 128, 0, st>>>(*m, a);
        k_conv_face<<<sb, 256, 0, st>>>(*m, a);
        if (m->n_ms > 0) k_conv_mortar_gather<<<mb, 128, 0, st>>>(*m, a);
        k_conv_vol<<<(unsigned)m->n_elem, threads, smem_conv(m), st>>>(*m, *t, a);
        const int e = (int)cudaGetLastError();
        if (e) return e;
        b->cur ^= 1;
        if (b->order == 2) b->hist++;
    }
    return 0;
}

int nsem_seg_prepare(const NsemDev* m) {
    if (smem_conv(m) > 48 * 1024) {
        const int e = (int)cudaFuncSetAttribute(k_conv_vol, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)smem_conv(m));
        if (e) return e;
    }
    if (smem_rho(m) > 48 * 1024) {
        const int e = (int)cudaFuncSetAttribute(k_seg_vol_rho, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)smem_rho(m));
        if (e) return e;
    }
    if (smem_grad(m) > 48 * 1024) {
        const int e = (int)cudaFuncSetAttribute(k_seg_grad_vol, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)smem_grad(m));
        if (e) return e;
    }
    if (smem_ut(m) > 48 * 1024)
        return (int)cudaFuncSetAttribute(k_seg_vol_ut, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem_ut(m));
    return 0;
}

int nsem_seg_steps(const NsemDev* m, const NsemTables* t, NsemSegBuf* b, int nsteps, double dt,
                   void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned nb = (unsigned)((m->n_int + 255) / 256);
    const unsigned sb = (unsigned)((m->n_slot + 255) / 256);
    const int threads = ((m->np + 31) / 32) * 32;
    const bool mort = m->n_ms > 0;
    const unsigned mb = (unsigned)((m->n_ms + 127) / 128);
    int cur = b->cur;
    for (int s = 0; s < nsteps; s++) {
        const SegArgs a = seg_args(m, b, cur, dt);
        k_seg_prep<<<nb, 256, 0, st>>>(*m, a);
        if (a.visc) {
            GradArgs ga;
            for (int c = 0; c < 3; c++) ga.U[c] = a.U[c];
            ga.Tf = a.Tf;
            for (int c = 0; c < 12; c++) ga.G[c] = a.G[c];
            for (int c = 0; c < 4; c++) ga.fF[c] = a.fF[c];
            for (int c = 0; c < 4; c++) ga.gC[c] = a.gC[c];
            k_seg_grad_face<<<sb, 256, 0, st>>>(*m, ga);
            if (mort) {
                k_seg_mortar_gcds<<<mb, 128, 0, st>>>(*m, ga);
                k_seg_mortar_ggather<<<mb, 128, 0, st>>>(*m, ga);
            }
            k_seg_grad_vol<<<(unsigned)m->n_elem, threads, smem_grad(m), st>>>(*m, *t, ga);
        }
        if (mort) k_seg_mortar_rho<<<6 * mb, 128, 0, st>>>(*m, a);
        k_seg_face_rho<<<sb, 256, 0, st>>>(*m, a);
        if (mort) k_seg_mortar_gather<0><<<mb, 128, 0, st>>>(*m, a);
        k_seg_vol_rho<<<(unsigned)m->n_elem, threads, smem_rho(m), st>>>(*m, *t, a);
        if (mort) k_seg_mortar_ut<<<16 * mb, 128, 0, st>>>(*m, a);
        k_seg_face_ut<<<sb, 256, 0, st>>>(*m, a);
        if (mort) k_seg_mortar_gather<1><<<4 * mb, 128, 0, st>>>(*m, a);
        k_seg_vol_ut<<<(unsigned)m->n_elem, threads, smem_ut(m), st>>>(*m, *t, a);
        const int e = (int)cudaGetLastError();
        if (e) return e;
        cur ^= 1;
    }
    return 0;
}

int nsem_seg_to_cons(const NsemDev* m, const NsemSegBuf* b, double* const* u, void* stream) {
    ConvArgs a{};
    a.rho = b->rho[b->cur];
    for (int c = 0; c < 3; c++) a.U[c] = b->U[c];
    a.Tp = b->Tp;
    for (int v = 0; v < 5; v++) a.u[v] = u[v];
    k_seg_to_cons<<<(unsigned)((m->n_int + 255) / 256), 256, 0, (cudaStream_t)stream>>>(*m, a);
    return (int)cudaGetLastError();
}

int nsem_cons_to_seg(const NsemDev* m, NsemSegBuf* b, double* const* u, void* stream) {
    ConvArgs a{};
    a.rho_w = b->rho[b->cur];
    for (int c = 0; c < 3; c++) a.U[c] = b->U[c];
    a.Tp = b->Tp;
    for (int v = 0; v < 5; v++) a.u[v] = u[v];
    k_cons_to_seg<<<(unsigned)((m->n_int + 255) / 256), 256, 0, (cudaStream_t)stream>>>(*m, a);
    return (int)cudaGetLastError();
}
