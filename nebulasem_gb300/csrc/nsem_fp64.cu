/*
 * Plain (FP64) form of the dGSEM Euler right-hand side and SSP-RK3 stage.
 *
 * Compiled with --fmad=false: every product and sum is rounded on its own, in
 * the order the reference evaluates it, so the GPU reproduces the reference's
 * CPU result bit for bit wherever the C library's pow is correctly rounded
 * (the equation of state uses the double-double pow of nsem_ddpow.h).
 *
 * Three kernels per stage:
 *   prim    per node: U = rho U / rho, theta = rho theta / rho,
 *           p' = P0 ((rho theta) R / P0)^gamma - p_ref, |U|, c = sqrt(gamma R theta)
 *           (apps/euler/euler.cpp:181-186, 211-213); run once per step, later
 *           stages get it from the volume kernel's epilogue;
 *   face    per used face slot: Rusanov fluxes of the three equations dotted
 *           with the weighted normal (src/field/field.h:2881-2943, 3086-3117),
 *           ghost states from applyExplicitBCs (field.h:2670-2685);
 *   volume  per element (one thread per node): surface lift in div_flux
 *           order, weak volume term gathered in the order the reference's
 *           scatter loop (field.h:3440-3464) adds it, gravity source,
 *           L = -Su/cV, Shu-Osher combination, primitives of the new state.
 * Roofline: FP64-pipe bound (about 1e3 FP64 instructions per node-stage
 * against 40-80 bytes of traffic).
 */
#include <cuda_runtime.h>

#include "nsem_ddpow.h"
#include "nsem_gather.cuh"
#include "nsem_internal.h"
#include "nsem_mortar.cuh"

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

/* ghost velocity of the SYMMETRY condition (src/tensor/tensor.h:486-494) */
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

struct PrimArgs {
    const double* S[5];
    double* prim[NSEM_NPRIM];
};

__device__ __forceinline__ void prim_at(const NsemDev& m, const double* const* S,
                                        double* const* prim, int64_t i) {
    const double r = S[0][i];
    double U[3];
    U[0] = S[1][i] / r;
    U[1] = S[2][i] / r;
    U[2] = S[3][i] / r;
    const double T = S[4][i] / r;
    const double p = m.P0 * nsem_pow(((r * T) * m.R) / m.P0, m.gamma);
    prim[0][i] = U[0];
    prim[1][i] = U[1];
    prim[2][i] = U[2];
    prim[3][i] = T;
    prim[4][i] = p - m.p_ref[i];
    prim[5][i] = sqrt(vdot3(U, U));
    prim[6][i] = sqrt(m.gR * T);
}

__global__ void __launch_bounds__(256) k_prim(const NsemDev m, PrimArgs a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n_int) return;
    prim_at(m, a.S, a.prim, i);
}

struct FaceArgs {
    const double* S0;            /* rho of the stage state */
    const double* prim[NSEM_NPRIM];
    double* d[5];
    const double* G[12];         /* viscous runs: grad U, grad theta (else null) */
    /* non-conforming faces, per mortar slot */
    double* mq[19];              /* the coarse side's interpolated quantities */
    double* mf[15];              /* face flux vectors (rho 3, momentum 9, theta 3) */
    double* dC[5];               /* projected, lifted coarse-side fluxes */
};

/* Non-conforming faces: the coarse side's node quantities of the stage
 * state interpolated onto each mortar slot, one thread per (slot, quantity):
 * |U|, c, U rho (3), rho, the momentum flux tensor (rho U) (x) U + p' I
 * - mu grad U (9), the theta flux (rho U) theta - (mu / Pr) grad theta (3),
 * rho theta; each exactly as the face kernel forms it at a node. */
__global__ void __launch_bounds__(128) k_mortar_coupled(const NsemDev m, FaceArgs a) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= 19 * m.n_ms) return;
    const int64_t ms = id / 19;
    const int c = (int)(id % 19);
    const int t = c - 6;   /* tensor component of the momentum flux */
    const int ra = (t >= 0 && t < 9) ? (t < 3 ? t : (t == 3 || t == 5) ? 0 : (t == 4 || t == 6) ? 1 : 2) : 0;
    const int rb = (t >= 0 && t < 9) ? (t < 3 ? t : (t == 6 || t == 8) ? 0 : (t == 3 || t == 7) ? 1 : 2) : 0;
    double out[1];
    mortar_interp<1>(m, ms, [&](int64_t node, double* v) {
        const double r = a.S0[node];
        if (c == 0) v[0] = a.prim[5][node];
        else if (c == 1) v[0] = a.prim[6][node];
        else if (c < 5) v[0] = a.prim[c - 2][node] * r;
        else if (c == 5) v[0] = r;
        else if (c < 15) {
            double x = (a.prim[ra][node] * r) * a.prim[rb][node];
            x = x + ((t < 3) ? 1.0 : 0.0) * a.prim[4][node];
            if (a.G[0]) x = x - (r * m.nu) * a.G[t][node];
            v[0] = x;
        } else if (c < 18) {
            double x = (a.prim[c - 15][node] * r) * a.prim[3][node];
            if (a.G[0]) x = x - ((r * m.nu) * m.iPr) * a.G[9 + c - 15][node];
            v[0] = x;
        } else {
            v[0] = r * a.prim[3][node];
        }
    }, out);
    a.mq[c][ms] = out[0];
}

/* the coarse side's lifted values: the projected flux vectors dotted with the
 * slot's own weighted normal; one thread per (mortar slot, output row) */
__global__ void __launch_bounds__(128) k_mortar_coupled_gather(const NsemDev m, FaceArgs a) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= 5 * m.n_ms) return;
    const int64_t ms = id / 5;
    const int r = (int)(id % 5);
    const int64_t k = ms_field(m, NSEM_MS_K, ms);
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    double P[3];
    if (r == 0 || r == 4) {
        double* src[3] = {a.mf[r == 0 ? 0 : 12], a.mf[r == 0 ? 1 : 13], a.mf[r == 0 ? 2 : 14]};
        mortar_project<3>(m, ms, src, P);
        a.dC[r][ms] = vdot3(P, n);
    } else {
        const int q = r - 1;
        const int cx = q == 0 ? XX : q == 1 ? YX : ZX;
        const int cy = q == 0 ? XY : q == 1 ? YY : ZY;
        const int cz = q == 0 ? XZ : q == 1 ? YZ : ZZ;
        double* src[3] = {a.mf[3 + cx], a.mf[3 + cy], a.mf[3 + cz]};
        mortar_project<3>(m, ms, src, P);
        a.dC[r][ms] = P[0] * n[0] + P[1] * n[1] + P[2] * n[2];
    }
}

__global__ void __launch_bounds__(256) k_face(const NsemDev m, FaceArgs a) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.n_slot) return;
    const int32_t c1 = m.c1[k], c2 = m.c2[k];
    const double n[3] = {m.fn[k], m.fn[m.n_slot + k], m.fn[2 * m.n_slot + k]};
    const double en[3] = {m.en[k], m.en[m.n_slot + k], m.en[2 * m.n_slot + k]};
    const double fi = m.fi[k], fo = 1 - fi;

    const double r1 = a.S0[c1];
    const double U1[3] = {a.prim[0][c1], a.prim[1][c1], a.prim[2][c1]};
    const double T1 = a.prim[3][c1], p1 = a.prim[4][c1];
    const double mu1 = a.prim[5][c1], cs1 = a.prim[6][c1];
    double r2, U2[3], T2, p2, mu2, cs2;
    if (c2 >= 0) {
        r2 = a.S0[c2];
        U2[0] = a.prim[0][c2]; U2[1] = a.prim[1][c2]; U2[2] = a.prim[2][c2];
        T2 = a.prim[3][c2]; p2 = a.prim[4][c2];
        mu2 = a.prim[5][c2]; cs2 = a.prim[6][c2];
    } else {
        /* ghost node: NEUMANN (value 0) for rho, theta, p; velocity per bc */
        r2 = r1 + 0.0;
        T2 = T1 + 0.0;
        p2 = p1;
        if (m.bc[k] == 2) {
            sym_vec(U1, n, U2);
        } else {
            U2[0] = U1[0] + 0.0; U2[1] = U1[1] + 0.0; U2[2] = U1[2] + 0.0;
        }
        mu2 = sqrt(vdot3(U2, U2));
        cs2 = sqrt(m.gR * T2);
    }
    /* a mortar's coarse side (1: c1, 2: c2) takes interpolated quantities */
    const int32_t ms = m.n_ms ? m.ms_of[k] : -1;
    const int side = ms >= 0 ? ms_field(m, NSEM_MS_SIDE, ms) : 0;
    double mu1v = mu1, cs1v = cs1, r1v = r1, r2v = r2;
    if (side == 1) { mu1v = a.mq[0][ms]; cs1v = a.mq[1][ms]; r1v = a.mq[5][ms]; }
    if (side == 2) { mu2 = a.mq[0][ms]; cs2 = a.mq[1][ms]; r2v = a.mq[5][ms]; }
    const double lam = ((mu1v * fi + mu2 * fo) + (cs1v * fi + cs2 * fo)) / 2;

    /* continuity: flux U rho, state rho */
    {
        double F[3];
        const double jump = lam * (r2v - r1v);
        for (int c = 0; c < 3; c++) {
            double x = U1[c] * r1, y = U2[c] * r2;
            if (side == 1) x = a.mq[2 + c][ms];
            if (side == 2) y = a.mq[2 + c][ms];
            F[c] = (x * fi + y * fo) - en[c] * jump;
        }
        a.d[0][k] = vdot3(F, n);
        if (side)
            for (int c = 0; c < 3; c++) a.mf[c][ms] = F[c];
    }
    /* momentum: flux (rho U)(x)U + p' I, state rho U */
    {
        double Fc1[3] = {U1[0] * r1, U1[1] * r1, U1[2] * r1};
        double Fc2[3] = {U2[0] * r2, U2[1] * r2, U2[2] * r2};
        double A[9], B[9], O[9], F[9], dq[3], out[3];
        outer(Fc1, U1, A);
        outer(Fc2, U2, B);
        for (int c = 0; c < 9; c++) {
            const double i1 = (c < 3) ? 1.0 : 0.0;
            A[c] = A[c] + i1 * p1;
            B[c] = B[c] + i1 * p2;
        }
        if (a.G[0]) {
            /* artificial viscosity: - mu grad U, mu = rho nu; zero gradient
             * on the wall ghosts (euler.cpp:189-190, 232) */
            const double mu1 = r1 * m.nu, mu2 = r2 * m.nu;
            for (int c = 0; c < 9; c++) {
                A[c] = A[c] - mu1 * a.G[c][c1];
                B[c] = B[c] - mu2 * (c2 >= 0 ? a.G[c][c2] : 0.0);
            }
        }
        if (side == 1) {
            for (int c = 0; c < 9; c++) A[c] = a.mq[6 + c][ms];
            for (int c = 0; c < 3; c++) Fc1[c] = a.mq[2 + c][ms];
        } else if (side == 2) {
            for (int c = 0; c < 9; c++) B[c] = a.mq[6 + c][ms];
            for (int c = 0; c < 3; c++) Fc2[c] = a.mq[2 + c][ms];
        }
        for (int c = 0; c < 3; c++) dq[c] = (Fc2[c] - Fc1[c]) * lam;
        outer(en, dq, O);
        for (int c = 0; c < 9; c++) F[c] = (A[c] * fi + B[c] * fo) - O[c];
        tdot(F, n, out);
        a.d[1][k] = out[0];
        a.d[2][k] = out[1];
        a.d[3][k] = out[2];
        if (side)
            for (int c = 0; c < 9; c++) a.mf[3 + c][ms] = F[c];
    }
    /* potential temperature: flux (rho U) theta, state rho theta */
    {
        double F[3];
        double s1 = r1 * T1, s2 = r2 * T2;
        if (side == 1) s1 = a.mq[18][ms];
        if (side == 2) s2 = a.mq[18][ms];
        const double jump = lam * (s2 - s1);
        for (int c = 0; c < 3; c++) {
            double x = (U1[c] * r1) * T1, y = (U2[c] * r2) * T2;
            if (a.G[0]) {
                /* - (mu / Pr) grad theta (euler.cpp:250) */
                x = x - ((r1 * m.nu) * m.iPr) * a.G[9 + c][c1];
                y = y - ((r2 * m.nu) * m.iPr) * (c2 >= 0 ? a.G[9 + c][c2] : 0.0);
            }
            if (side == 1) x = a.mq[15 + c][ms];
            if (side == 2) y = a.mq[15 + c][ms];
            F[c] = (x * fi + y * fo) - en[c] * jump;
        }
        a.d[4][k] = vdot3(F, n);
        if (side)
            for (int c = 0; c < 3; c++) a.mf[12 + c][ms] = F[c];
    }
}

struct VolArgs {
    const double* S[5];     /* stage state (input)               */
    const double* U0[5];    /* u^n (stages 2, 3)                 */
    double* out[5];         /* new stage state, or L (stage 0)   */
    double* prim[NSEM_NPRIM];
    const double* d[5];
    int stage;
    double dt;
    const double* G[12];    /* viscous runs: grad U, grad theta (else null) */
    const double* dC[5];    /* non-conforming faces: the coarse side's lifted values */
};

/* shared layout per node: fr[3] fm[9] ft[3] jin[9] = 24 doubles */
constexpr int SM_W = 24;

__global__ void k_volume(const NsemDev m, const NsemTables tab, VolArgs a) {
    extern __shared__ double sm[];
    const int NPX = m.npx, NPY = m.npy, NPZ = m.npz, NP = m.np;
    double* dps = sm + (size_t)NP * SM_W;           /* 3 * npd^2 tables */
    const int t = threadIdx.x;
    for (int q = t; q < 3 * NSEM_MAX_NPD * NSEM_MAX_NPD; q += blockDim.x)
        dps[q] = (&tab.dpsi[0][0])[q];

    const int64_t e = blockIdx.x;
    const bool active = t < NP;
    const int64_t node = e * NP + t;
    double rho = 0, U[3] = {0, 0, 0}, T = 0, pp = 0;
    if (active) {
        rho = a.S[0][node];
        U[0] = a.prim[0][node]; U[1] = a.prim[1][node]; U[2] = a.prim[2][node];
        T = a.prim[3][node];
        pp = a.prim[4][node];
        double* my = sm + (size_t)t * SM_W;
        const double Fc[3] = {U[0] * rho, U[1] * rho, U[2] * rho};
        my[0] = Fc[0]; my[1] = Fc[1]; my[2] = Fc[2];          /* U*rho == rho*U */
        double fm[9];
        outer(Fc, U, fm);
        for (int c = 0; c < 9; c++) fm[c] = fm[c] + ((c < 3) ? 1.0 : 0.0) * pp;
        double ft[3] = {Fc[0] * T, Fc[1] * T, Fc[2] * T};
        if (a.G[0]) {
            const double mu = rho * m.nu;
            for (int c = 0; c < 9; c++) fm[c] = fm[c] - mu * a.G[c][node];
            for (int c = 0; c < 3; c++) ft[c] = ft[c] - (mu * m.iPr) * a.G[9 + c][node];
        }
        for (int c = 0; c < 9; c++) my[3 + c] = fm[c];
        my[12] = ft[0]; my[13] = ft[1]; my[14] = ft[2];
        for (int c = 0; c < 9; c++) my[15 + c] = m.jin[(int64_t)c * m.n_int + node];
    }
    __syncthreads();
    if (!active) return;

    /* surface lift, in the order div_flux visits the element's faces */
    double r0 = 0.0, r1 = 0.0, r2 = 0.0, r3 = 0.0, r4 = 0.0;
    for (int j = 0; j < m.n_lift; j++) {
        const int32_t code = m.lift[(int64_t)j * m.n_int + node];
        if (code < 0) break;
        const int64_t k = code >> 2;
        double v0, v1, v2, v3, v4;
        if (code & 2) {
            v0 = a.dC[0][k]; v1 = a.dC[1][k]; v2 = a.dC[2][k]; v3 = a.dC[3][k]; v4 = a.dC[4][k];
        } else {
            v0 = a.d[0][k]; v1 = a.d[1][k]; v2 = a.d[2][k]; v3 = a.d[3][k]; v4 = a.d[4][k];
        }
        if (code & 1) {
            r0 -= v0; r1 -= v1; r2 -= v2; r3 -= v3; r4 -= v4;
        } else {
            r0 += v0; r1 += v1; r2 += v2; r3 += v3; r4 += v4;
        }
    }

    /* weak volume term.  Source b adds -F_b . (Jin_b . dpsi(b->a)); sources
     * arrive in lexicographic order of b: X-line below, Y-line below, Z-line
     * below, self, Z above, Y above, X above. */
    nsem_volume_gather<SM_W, 15>(NPX, NPY, NPZ, sm, dps, t, [&](int lb, const double* dj) {
        const double* sb = sm + (size_t)lb * SM_W;
        double tv[3];
        r0 -= vdot3(sb, dj);
        tdot(sb + 3, dj, tv);
        r1 -= tv[0]; r2 -= tv[1]; r3 -= tv[2];
        r4 -= vdot3(sb + 12, dj);
    });

    /* gravity source: Su -= ((rho - rho_ref) g) cV */
    const double cv = m.cv[node];
    {
        const double s = rho - m.rho_ref[node];
        const double sc0 = 0.0 + m.g[0] * s, sc1 = 0.0 + m.g[1] * s, sc2 = 0.0 + m.g[2] * s;
        r1 = r1 - sc0 * cv;
        r2 = r2 - sc1 * cv;
        r3 = r3 - sc2 * cv;
    }
    const double L[5] = {-(r0 / cv), -(r1 / cv), -(r2 / cv), -(r3 / cv), -(r4 / cv)};

    if (a.stage == 0) {
        for (int c = 0; c < 5; c++) a.out[c][node] = L[c];
        return;
    }
    double nu[5];
    const double dt = a.dt;
    if (a.stage == 1) {
        for (int c = 0; c < 5; c++) nu[c] = a.S[c][node] + dt * L[c];
    } else if (a.stage == 2) {
        for (int c = 0; c < 5; c++) {
            const double s = a.S[c][node] + dt * L[c];
            nu[c] = 0.75 * a.U0[c][node] + 0.25 * s;
        }
    } else {
        const double a3 = 1.0 / 3.0, b3 = 2.0 / 3.0;
        for (int c = 0; c < 5; c++) {
            const double s = a.S[c][node] + dt * L[c];
            nu[c] = a3 * a.U0[c][node] + b3 * s;
        }
    }
    bool finite = true;
    for (int c = 0; c < 5; c++) {
        a.out[c][node] = nu[c];
        finite = finite && isfinite(nu[c]);
    }
    if (!finite) atomicOr(m.status, NSEM_STATUS_NONFINITE);
    /* primitives of the new stage state for the next face kernel */
    const double* const outc[5] = {a.out[0], a.out[1], a.out[2], a.out[3], a.out[4]};
    prim_at(m, outc, a.prim, node);
}

inline int launch_err() { return (int)cudaGetLastError(); }

}  // namespace

extern "C" int nsem_fp64_prim(const NsemDev* m, NsemBuf* b, int from_state, void* stream) {
    PrimArgs a;
    for (int c = 0; c < 5; c++) a.S[c] = from_state ? b->u[c] : b->s[c];
    for (int c = 0; c < NSEM_NPRIM; c++) a.prim[c] = b->prim[c];
    const int64_t blocks = (m->n_int + 255) / 256;
    k_prim<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(*m, a);
    return launch_err();
}

extern "C" int nsem_fp64_face(const NsemDev* m, NsemBuf* b, int from_state, void* stream) {
    FaceArgs a;
    a.S0 = from_state ? b->u[0] : b->s[0];
    for (int c = 0; c < NSEM_NPRIM; c++) a.prim[c] = b->prim[c];
    for (int c = 0; c < 5; c++) a.d[c] = b->d[c];
    for (int c = 0; c < 12; c++) a.G[c] = b->G[c];
    for (int c = 0; c < 19; c++) a.mq[c] = b->mq[c];
    for (int c = 0; c < 15; c++) a.mf[c] = b->mf[c];
    for (int c = 0; c < 5; c++) a.dC[c] = b->dC[c];
    const int64_t blocks = (m->n_slot + 255) / 256;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned mb = (unsigned)((m->n_ms + 127) / 128);
    if (m->n_ms > 0) k_mortar_coupled<<<19 * mb, 128, 0, st>>>(*m, a);
    k_face<<<(unsigned)blocks, 256, 0, st>>>(*m, a);
    if (m->n_ms > 0) k_mortar_coupled_gather<<<5 * mb, 128, 0, st>>>(*m, a);
    return launch_err();
}

static size_t vol_smem(const NsemDev* m) {
    return ((size_t)m->np * SM_W + 3 * NSEM_MAX_NPD * NSEM_MAX_NPD) * sizeof(double);
}

extern "C" int nsem_fp64_check_smem(const NsemDev* m) {
    const size_t smem = vol_smem(m);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_volume, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return (int)e;
    }
    return 0;
}

extern "C" int nsem_fp64_volume(const NsemDev* m, const NsemTables* t, NsemBuf* b, int stage,
                                double dt, void* stream) {
    VolArgs a;
    a.stage = stage;
    a.dt = dt;
    for (int c = 0; c < 5; c++) {
        a.d[c] = b->d[c];
        a.U0[c] = b->u[c];
        if (stage == 0) { a.S[c] = b->u[c]; a.out[c] = b->L[c]; }
        else if (stage == 1) { a.S[c] = b->u[c]; a.out[c] = b->s[c]; }
        else if (stage == 2) { a.S[c] = b->s[c]; a.out[c] = b->s[c]; }
        else { a.S[c] = b->s[c]; a.out[c] = b->u[c]; }
    }
    for (int c = 0; c < NSEM_NPRIM; c++) a.prim[c] = b->prim[c];
    for (int c = 0; c < 12; c++) a.G[c] = b->G[c];
    for (int c = 0; c < 5; c++) a.dC[c] = b->dC[c];
    const int threads = ((m->np + 31) / 32) * 32;
    k_volume<<<(unsigned)m->n_elem, threads, vol_smem(m), (cudaStream_t)stream>>>(*m, *t, a);
    return launch_err();
}
