/*
 * Discrete adjoint of the precision form (FP32 bulk, FP64 adjoint state).
 * No reference counterpart: the reference has no adjoint.  This is the
 * transpose of the precision form's stage (nsem_mixed.cu), i.e. of the
 * operator chain of field.h:2928-2943 (Rusanov flux), 3086-3117 (weak lift)
 * and 3440-3464 (volume term), evaluated at the precision form's own FP32
 * stage states.
 *
 * Tendency of node a (element e, stage state x, FP32):
 *   L_a = sum_d J_d sum_m Q_d[a_d][m] F_d(x_m)                (volume)
 *       - sum_{faces f through a} C_f Phi_f(x_a, x_o)           (lift, C_f = J_d / w_end)
 *       + (0, rho'_a g, 0)                                      (buoyancy)
 * with Phi_f = s (F_n(x_a) + F_n(x_o)) / 2 - lam (q_o - q_a) (mass, normal
 * momentum, Theta' components), lam = (|u|_a + |u|_o + c_a + c_o) / 4, or on a
 * wall Phi = e_n (s p'_a + lam_w m_n,a), lam_w = (|u_ghost| + c_a) / 2.  The
 * neighbour's element sees -Phi.  Given gbar per node, the transpose is
 *   xbar_b = sum_d JF_d(x_b)^T Fbar_d(b) + face terms + buoyancy, with
 *   Fbar_d(b) = J_d sum_a Q_d[a_d][b_d] gbar_a       (transposed line sums),
 * and on each face node of the element Phibar = C'_f gbar_o - C_f gbar_a
 * (both elements' lifts of the shared flux): JF_n(x_a)^T (s Phibar / 2) is
 * merged into Fbar_n, and the terms of lam and of the jump are added directly.
 *
 * Reverse of one SSP-RK3 step in increment form (x1 = S, x2 = S + d1,
 * x3 = S + d2 the FP32 stage states of the forward step, S = fp32(u'^n)):
 *   R3: gbar = 2/3 lam;   xbar3 = dt J(x3)^T gbar;  A = xbar3;  B = 2/3 lam + xbar3
 *   R2: gbar = B / 4;     xbar2 = dt J(x2)^T gbar;  A += xbar2; C = B / 4 + xbar2
 *   R1: gbar = C;         xbar1 = dt J(x1)^T gbar;  lam <- lam + A + xbar1 (FP64)
 * One fused kernel per reverse stage, one element per CTA, structured like the
 * forward stage kernel: phase 1 (node) primitives and derivative data, phase 2
 * (face node) face adjoints, phase 3 (node) transposed line sums, pointwise
 * transposes and the stage combination.
 */
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "nsem_mixed_adj.cuh"

using namespace nsem_mx;
using namespace nsem_mxa;

namespace {

/* phase 2: adjoint of the flux through face node t (the face's axis a
 * run-time value: selects, no divergent branches between axes) */
template <int NX, int NY, int NZ>
__device__ __forceinline__ void face_adj(const FaceSlot& fs, int32_t nb, const float* xo,
                                         const float* bgo, const float* go, float cn,
                                         const float* sGb, const float4* sP,
                                         const float* sT, float cs, const AdjArgs& a, float4& fa4,
                                         float& fa1, float4& xd4, float& xd1) {
    constexpr int NP = Geo<NX, NY, NZ>::NP;
    const int DIR = fs.dir;
    const bool d0 = DIR == 0, d1 = DIR == 1;
    const float sg = fs.side ? 1.0f : -1.0f;
    const float4 P0 = sP[fs.la], P1 = sP[NP + fs.la], P2 = sP[2 * NP + fs.la];
    const float tp_s = sT[fs.la];
    /* own values: P0 = (rho', m0, m1, m2), P1 = (rho, |u|, c, 1/Theta),
     * P2 = (u0, u1, u2, dp'/dTheta') */
    const float rho = P1.x, um = P1.y, c = P1.z, iTh = P1.w;
    const float inv = rcp_nr(rho);
    const float4 ga4 = make_float4(sGb[fs.la], sGb[NP + fs.la], sGb[2 * NP + fs.la], sGb[3 * NP + fs.la]);
    const float ga1 = sGb[4 * NP + fs.la];
    const float md = d0 ? P0.y : d1 ? P0.z : P0.w;
    const float uvec[3] = {P2.x, P2.y, P2.z};
    if (nb >= 0) {
        const Pt q = pointwise(xo, bgo, a.eos, a.gamma, a.gR);
        const float lam = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(um, q.umag), __fadd_rn(c, q.c)));
        /* Phibar = C' gbar_o - C gbar_a */
        const float pb0 = fmaf(cn, go[0], -cs * ga4.x);
        const float pb1 = fmaf(cn, go[1], -cs * ga4.y);
        const float pb2 = fmaf(cn, go[2], -cs * ga4.z);
        const float pb3 = fmaf(cn, go[3], -cs * ga4.w);
        const float pb4 = fmaf(cn, go[4], -cs * ga1);
        const float h = 0.5f * sg;
        fa4 = make_float4(h * pb0, h * pb1, h * pb2, h * pb3);
        fa1 = h * pb4;
        const float pbm = d0 ? pb1 : d1 ? pb2 : pb3;
        /* jump terms: d(-lam (q_o - q_a))/dx_a = lam on the masked components,
         * minus (jump . Phibar) dlam/dx_a */
        const float xmo = d0 ? xo[1] : d1 ? xo[2] : xo[3];
        const float jr = xo[0] - P0.x, jm = xmo - md, jt = xo[4] - tp_s;
        const float s = fmaf(jr, pb0, fmaf(jm, pbm, jt * pb4));
        /* dlam/dx_a = (d|u| + dc) / 4: d|u|/drho' = -|u|/rho, d|u|/dm_k = u_k/(rho |u|),
         * dc/drho' = -c/(2 rho), dc/dTheta' = c/(2 Theta) */
        const float ku = um > 0.0f ? inv * rcp_nr(um) : 0.0f;
        const float q4 = -0.25f * s;
        float x0 = fmaf(q4, -fmaf(0.5f, c, um) * inv, lam * pb0);
        float xm[3];
#pragma unroll
        for (int k = 0; k < 3; k++) xm[k] = q4 * (uvec[k] * ku);
#pragma unroll
        for (int k = 0; k < 3; k++) xm[k] = k == DIR ? fmaf(lam, pbm, xm[k]) : xm[k];
        const float x4 = fmaf(q4, 0.5f * c * iTh, lam * pb4);
        xd4 = make_float4(x0, xm[0], xm[1], xm[2]);
        xd1 = x4;
    } else {
        /* wall: Phi_n = s p' + lam_w m_n; Phibar = -C gbar_a (normal momentum) */
        const float pbm = -cs * (d0 ? ga4.y : d1 ? ga4.z : ga4.w);
        const float r0 = d0 ? 0.0f : uvec[0];
        const float r1 = d1 ? 0.0f : uvec[1];
        const float r2 = DIR == 2 ? 0.0f : uvec[2];
        const float mr = safe_sqrt(__fmaf_rn(r0, r0, __fmaf_rn(r1, r1, __fmul_rn(r2, r2))));
        const bool full = mr > 1e-7f;
        const float um_g = full ? um : mr;
        const float lam = __fmul_rn(0.5f, __fadd_rn(um_g, c));
        /* d|u_ghost|: of |u| (rescaled tangential velocity) or of |r| */
        const float nrm = full ? um : mr;
        const float ku = nrm > 0.0f ? inv * rcp_nr(nrm) : 0.0f;
        const float q2 = 0.5f * md * pbm;
        const float vr[3] = {full ? uvec[0] : r0, full ? uvec[1] : r1, full ? uvec[2] : r2};
        float x0 = q2 * -fmaf(0.5f, c, um_g) * inv;
        float xm[3];
#pragma unroll
        for (int k = 0; k < 3; k++) xm[k] = q2 * (vr[k] * ku);
#pragma unroll
        for (int k = 0; k < 3; k++) xm[k] = k == DIR ? fmaf(lam, pbm, xm[k]) : xm[k];
        const float x4 = fmaf(q2, 0.5f * c * iTh, sg * P2.w * pbm);
        fa4 = make_float4(0, 0, 0, 0);
        fa1 = 0.0f;
        xd4 = make_float4(x0, xm[0], xm[1], xm[2]);
        xd1 = x4;
    }
}

template <int NX, int NY, int NZ, int RS, bool VISC>
__global__ void __launch_bounds__(Geo<NX, NY, NZ>::BLOCK, (adj_min_blocks<NX, NY, NZ>()))
k_mixed_adj(AdjArgs a) {
    using G = Geo<NX, NY, NZ>;
    using SM = AdjSmem<NX, NY, NZ>;
    constexpr int NP = G::NP;
    constexpr int NFS = G::NFS;
    extern __shared__ float4 asm4[];
    float* smem = reinterpret_cast<float*>(asm4);
    float* sGb = smem;                                          /* [5][NP] */
    float* sR = smem + SM::OFF_R;
    float4* sP = reinterpret_cast<float4*>(smem + SM::OFF_P);
    float* sT = smem + SM::OFF_T;
    float4* sFa4 = reinterpret_cast<float4*>(smem + SM::OFF_FA4);
    float* sFa1 = smem + SM::OFF_FA1;
    float4* sXd4 = reinterpret_cast<float4*>(smem + SM::OFF_XD4);
    float* sXd1 = smem + SM::OFF_XD1;
    float* sMeta = smem + SM::OFF_META;

    const int t = threadIdx.x;
    const int64_t e = blockIdx.x;
    constexpr bool has_din = RS == 3 || RS == 2;

    float x[5], gb[5], bgs[4] = {0, 0, 0, 0};
    if (t < NP) {
        const int64_t o = e * 5 * NP + t;
#pragma unroll
        for (int v = 0; v < 5; v++) x[v] = __ldg(a.S + o + v * NP);
        if constexpr (has_din) {
#pragma unroll
            for (int v = 0; v < 5; v++) x[v] = __fadd_rn(x[v], __ldg(a.Din + o + v * NP));
        }
        load_gbar<RS>(a, o, NP, gb);
        const float* bg = a.bg + (int64_t)__ldg(a.layer + e) * 4 * NP + t;
#pragma unroll
        for (int c = 0; c < 4; c++) bgs[c] = __ldg(bg + c * NP);
    }
    float gv[12];
    if constexpr (VISC) {
        if (t < NP) {
            const float* gr = a.Gv + e * 12 * NP + t;
#pragma unroll
            for (int c = 0; c < 12; c++) gv[c] = __ldg(gr + c * NP);
        }
    }
    FaceSlot fs{};
    int32_t nb = -1;
    float xo[5], bgo[4], go[5], cn = 0.0f;
    if (t < NFS) {
        fs = face_slot<NX, NY, NZ>(t);
        nb = __ldg(a.nbr + (int64_t)fs.face * a.n_elem + e);
        if (nb >= 0) {
            const int64_t o = (int64_t)nb * 5 * NP + fs.lo;
#pragma unroll
            for (int v = 0; v < 5; v++) xo[v] = __ldg(a.S + o + v * NP);
            if constexpr (has_din) {
#pragma unroll
                for (int v = 0; v < 5; v++) xo[v] = __fadd_rn(xo[v], __ldg(a.Din + o + v * NP));
            }
            load_gbar<RS>(a, o, NP, go);
            const float* bg = a.bg + (int64_t)__ldg(a.layer + nb) * 4 * NP + fs.lo;
#pragma unroll
            for (int c = 0; c < 4; c++) bgo[c] = __ldg(bg + c * NP);
            cn = __ldg(a.J + (int64_t)fs.dir * a.n_elem + nb) * a.lift[fs.dir];
        }
    }
    if (t < 3) sMeta[t] = __ldg(a.J + (int64_t)t * a.n_elem + e);

    /* phase 1: gbar and the node's values for the face and pointwise transposes */
    float uu[3], th = 0.0f, pth = 0.0f, rho = 0.0f;
    if (t < NP) {
        const Pt p = pointwise(x, bgs, a.eos, a.gamma, a.gR);
        rho = p.rho;
        const float Th = __fadd_rn(bgs[1], x[4]);
        const float iTh = rcp_nr(Th);
        pth = a.gamma * (bgs[3] + p.pp) * iTh;      /* dp'/dTheta' = gamma p / Theta */
        uu[0] = p.u[0]; uu[1] = p.u[1]; uu[2] = p.u[2];
        th = p.th;
#pragma unroll
        for (int v = 0; v < 5; v++) sGb[v * NP + t] = gb[v];
        sP[t] = make_float4(x[0], x[1], x[2], x[3]);
        sP[NP + t] = make_float4(p.rho, p.umag, p.c, iTh);
        sP[2 * NP + t] = make_float4(p.u[0], p.u[1], p.u[2], pth);
        sT[t] = x[4];
    }
    __syncthreads();

    /* phase 2: face adjoints */
    if (t < NFS) {
        /* a face on a 2:1 mortar (nb <= -2) lifts the mortar's outward value,
         * not a flux of its own: a zero coefficient zeroes its face terms
         * (the mortar transposes add the node's state adjoint afterwards) */
        const float cs = nb <= -2 ? 0.0f : sMeta[fs.dir] * a.lift[fs.dir];
        float4 fa4, xd4;
        float fa1, xd1;
        face_adj<NX, NY, NZ>(fs, nb, xo, bgo, go, cn, sGb, sP, sT, cs, a, fa4, fa1, xd4, xd1);
        sFa4[t] = fa4;
        sFa1[t] = fa1;
        sXd4[t] = xd4;
        sXd1[t] = xd1;
    }
    /* the transposed line sums of the three directions */
    line_transform_t<NX, NY, NZ, 0>(sGb, sR, a, t);
    if constexpr (G::HAS_Y) line_transform_t<NX, NY, NZ, 1>(sGb, sR, a, t);
    line_transform_t<NX, NY, NZ, 2>(sGb, sR, a, t);
    __syncthreads();

    /* phase 3: transposed line sums, pointwise transposes, face and source terms */
    if (t >= NP) return;
    const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
    float xb[5] = {0, 0, 0, 0, 0};
    /* viscous runs: gradient adjoints and the mu sums of the flux adjoints */
    float gbv[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    float smv = 0.0f, stv = 0.0f;
    const float mu = rho * a.nu, mt = rho * a.nu_pr;
    {
        /* x: Fbar_x(b) = J_x sum_a Q_x[a][i] gbar(a, j, k) */
        const float* rr = sR + LineLay<NX, NY, NZ, 0>::at(i, j, k);
        constexpr int NL = LineLay<NX, NY, NZ, 0>::NL;
        float4 acc = make_float4(rr[0], rr[NL], rr[2 * NL], rr[3 * NL]);
        float acc1 = rr[4 * NL];
        const float Jx = sMeta[0];
        acc.x *= Jx; acc.y *= Jx; acc.z *= Jx; acc.w *= Jx; acc1 *= Jx;
        const int sx = face_of_node<NX, NY, NZ, 0>(i, j, k);
        if (sx >= 0) {
            const float4 f = sFa4[sx];
            acc.x += f.x; acc.y += f.y; acc.z += f.z; acc.w += f.w; acc1 += sFa1[sx];
        }
        jft<0>(uu, th, pth, acc.x, acc.y, acc.z, acc.w, acc1, xb);
        if constexpr (VISC) visc_t<0>(acc, acc1, gv, mu, mt, gbv, smv, stv);
    }
    if constexpr (G::HAS_Y) {
        const float* rr = sR + LineLay<NX, NY, NZ, 1>::at(i, j, k);
        constexpr int NL = LineLay<NX, NY, NZ, 1>::NL;
        float4 acc = make_float4(rr[0], rr[NL], rr[2 * NL], rr[3 * NL]);
        float acc1 = rr[4 * NL];
        const float Jy = sMeta[1];
        acc.x *= Jy; acc.y *= Jy; acc.z *= Jy; acc.w *= Jy; acc1 *= Jy;
        const int sy = face_of_node<NX, NY, NZ, 1>(i, j, k);
        if (sy >= 0) {
            const float4 f = sFa4[sy];
            acc.x += f.x; acc.y += f.y; acc.z += f.z; acc.w += f.w; acc1 += sFa1[sy];
        }
        jft<1>(uu, th, pth, acc.x, acc.y, acc.z, acc.w, acc1, xb);
        if constexpr (VISC) visc_t<1>(acc, acc1, gv, mu, mt, gbv, smv, stv);
    }
    {
        const float* rr = sR + LineLay<NX, NY, NZ, 2>::at(i, j, k);
        constexpr int NL = LineLay<NX, NY, NZ, 2>::NL;
        float4 acc = make_float4(rr[0], rr[NL], rr[2 * NL], rr[3 * NL]);
        float acc1 = rr[4 * NL];
        const float Jz = sMeta[2];
        acc.x *= Jz; acc.y *= Jz; acc.z *= Jz; acc.w *= Jz; acc1 *= Jz;
        const int sz = face_of_node<NX, NY, NZ, 2>(i, j, k);
        if (sz >= 0) {
            const float4 f = sFa4[sz];
            acc.x += f.x; acc.y += f.y; acc.z += f.z; acc.w += f.w; acc1 += sFa1[sz];
        }
        jft<2>(uu, th, pth, acc.x, acc.y, acc.z, acc.w, acc1, xb);
        if constexpr (VISC) visc_t<2>(acc, acc1, gv, mu, mt, gbv, smv, stv);
    }
    /* direct face terms of the faces through the node */
    auto direct = [&](int slot) {
        const float4 f = sXd4[slot];
        xb[0] += f.x; xb[1] += f.y; xb[2] += f.z; xb[3] += f.w; xb[4] += sXd1[slot];
    };
    {
        const int sx = face_of_node<NX, NY, NZ, 0>(i, j, k);
        if (sx >= 0) direct(sx);
        if constexpr (G::HAS_Y) {
            const int sy = face_of_node<NX, NY, NZ, 1>(i, j, k);
            if (sy >= 0) direct(sy);
        }
        const int sz = face_of_node<NX, NY, NZ, 2>(i, j, k);
        if (sz >= 0) direct(sz);
    }
    /* buoyancy: L_m += rho' g */
    xb[0] = fmaf(a.g[0], gb[1], fmaf(a.g[1], gb[2], fmaf(a.g[2], gb[3], xb[0])));

    const int64_t o = e * 5 * NP + t;
    if constexpr (VISC) {
        /* mu = (rho_ref + rho') nu: the density adjoint of the viscous
         * fluxes; the first pass ends here, the gradients' transpose and the
         * stage combination follow in k_mixed_adj_grad */
        xb[0] = fmaf(-a.nu, smv, fmaf(-a.nu_pr, stv, xb[0]));
#pragma unroll
        for (int v = 0; v < 5; v++) a.XB[o + v * NP] = xb[v];
        float* gbo = a.GB + e * 12 * NP + t;
#pragma unroll
        for (int c = 0; c < 12; c++) gbo[c * NP] = gbv[c];
        return;
    }
    if constexpr (RS == 0) {
#pragma unroll
        for (int v = 0; v < 5; v++) a.Bout[o + v * NP] = xb[v];
        return;
    }
    const float dt = a.dt;
    if constexpr (RS == 3) {
        /* A = xbar3; B = 2/3 lam + xbar3 (gb = 2/3 lam) */
#pragma unroll
        for (int v = 0; v < 5; v++) {
            const float x3 = dt * xb[v];
            a.A[o + v * NP] = x3;
            a.Bout[o + v * NP] = gb[v] + x3;
        }
    } else if constexpr (RS == 2) {
        /* A += xbar2; C = B/4 + xbar2 (gb = B/4) */
#pragma unroll
        for (int v = 0; v < 5; v++) {
            const float x2 = dt * xb[v];
            a.A[o + v * NP] = __ldg(a.A + o + v * NP) + x2;
            a.Bout[o + v * NP] = gb[v] + x2;
        }
    } else {
        /* lam <- lam + A + xbar1 (FP64) */
#pragma unroll
        for (int v = 0; v < 5; v++) {
            const float x1 = dt * xb[v];
            const double l = __ldg(a.lam + o + v * NP);
            a.lam_out[o + v * NP] = l + (f2d(__ldg(a.A + o + v * NP)) + f2d(x1));
        }
    }
}

template <int NX, int NY, int NZ, int RS>
__global__ void __launch_bounds__(Geo<NX, NY, NZ>::BLOCK)
k_mixed_adj_grad(AdjArgs a) {
    using G = Geo<NX, NY, NZ>;
    using SM = AdjGradSmem<NX, NY, NZ>;
    constexpr int NP = G::NP;
    constexpr int NFS = G::NFS;
    extern __shared__ float4 agm4[];
    float* smem = reinterpret_cast<float*>(agm4);
    float* sR = smem;
    float4* sV = reinterpret_cast<float4*>(smem + SM::OFF_V);
    float4* sF = reinterpret_cast<float4*>(smem + SM::OFF_F);
    float* sMeta = smem + SM::OFF_META;
    const int t = threadIdx.x;
    const int64_t e = blockIdx.x;
    constexpr bool has_din = RS == 3 || RS == 2;

    float x[5], rref = 0.0f, gbv[12], xbp[5], gb[5];
    if (t < NP) {
        const int64_t o = e * 5 * NP + t;
#pragma unroll
        for (int v = 0; v < 5; v++) x[v] = __ldg(a.S + o + v * NP);
        if constexpr (has_din) {
#pragma unroll
            for (int v = 0; v < 5; v++) x[v] = __fadd_rn(x[v], __ldg(a.Din + o + v * NP));
        }
        rref = __ldg(a.bg + (int64_t)__ldg(a.layer + e) * 4 * NP + t);
        const float* gr = a.GB + e * 12 * NP + t;
#pragma unroll
        for (int c = 0; c < 12; c++) gbv[c] = gr[c * NP];
#pragma unroll
        for (int v = 0; v < 5; v++) xbp[v] = a.XB[o + v * NP];
        load_gbar<RS>(a, o, NP, gb);
    }
    FaceSlot fs{};
    int32_t nb = -1;
    float4 gbn = make_float4(0, 0, 0, 0);
    float Jn = 0.0f;
    if (t < NFS) {
        fs = face_slot<NX, NY, NZ>(t);
        nb = __ldg(a.nbr + (int64_t)fs.face * a.n_elem + e);
        if (nb >= 0) {
            /* the neighbour's gradient adjoints along this face's axis at its node */
            const float* gr = a.GB + (int64_t)nb * 12 * NP + fs.lo;
            const int d = fs.dir;
            gbn = make_float4(gr[tidx(d, 0) * NP], gr[tidx(d, 1) * NP], gr[tidx(d, 2) * NP],
                              gr[(9 + d) * NP]);
            Jn = __ldg(a.J + (int64_t)d * a.n_elem + nb);
        }
    }
    if (t < 3) sMeta[t] = __ldg(a.J + (int64_t)t * a.n_elem + e);

    /* phase 1: V of the node, the gradient adjoints into their rows */
    float inv = 0.0f;
    if (t < NP) {
        inv = rcp_nr(__fadd_rn(rref, x[0]));
        sV[t] = make_float4(__fmul_rn(x[1], inv), __fmul_rn(x[2], inv), __fmul_rn(x[3], inv),
                            __fmul_rn(__fmaf_rn(-a.T0, x[0], x[4]), inv));
        const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
        auto put = [&](float* f, int nl, int r) {
            f[0] = gbv[tidx(r, 0)]; f[nl] = gbv[tidx(r, 1)]; f[2 * nl] = gbv[tidx(r, 2)];
            f[3 * nl] = gbv[9 + r];
        };
        put(sR + LineLay<NX, NY, NZ, 0>::at(i, j, k), LineLay<NX, NY, NZ, 0>::NL, 0);
        if constexpr (G::HAS_Y) put(sR + LineLay<NX, NY, NZ, 1>::at(i, j, k), LineLay<NX, NY, NZ, 1>::NL, 1);
        put(sR + LineLay<NX, NY, NZ, 2>::at(i, j, k), LineLay<NX, NY, NZ, 2>::NL, 2);
    }
    __syncthreads();

    /* phase 2: per face node the face terms' adjoints for the node */
    if (t < NFS) {
        const int r = fs.dir;
        const int la = fs.la;
        const int i = la / (NY * NZ), j = (la / NZ) % NY, k = la % NZ;
        using L0 = LineLay<NX, NY, NZ, 0>;
        using L1 = LineLay<NX, NY, NZ, 1>;
        using L2 = LineLay<NX, NY, NZ, 2>;
        const float* f = sR + (r == 0 ? L0::at(i, j, k) : r == 1 ? L1::at(i, j, k) : L2::at(i, j, k));
        const int nl = r == 0 ? L0::NL : r == 1 ? L1::NL : L2::NL;
        const float sg = fs.side ? 1.0f : -1.0f;
        /* a face on a 2:1 mortar: a zero coefficient zeroes the face terms
         * here; the mortar gradient transposes take them */
        const float co = nb <= -2 ? 0.0f : sg * sMeta[r] * a.lift[r];
        const float4 sd = make_float4(co * f[0], co * f[nl], co * f[2 * nl], co * f[3 * nl]);
        float4 out;
        if (nb >= 0) {
            /* own: cds - V_a -> -1/2; the neighbour's face term has V_a in its
             * cds with weight 1/2 and its own sign (the opposite side) */
            const float cn = -sg * Jn * a.lift[r];
            out = make_float4(0.5f * fmaf(cn, gbn.x, -sd.x), 0.5f * fmaf(cn, gbn.y, -sd.y),
                              0.5f * fmaf(cn, gbn.z, -sd.z), 0.5f * fmaf(cn, gbn.w, -sd.w));
        } else {
            /* wall: sD = ghost(V) - V; the ghost's theta is V's (no term), its
             * velocity the SYMMETRY projection rescaled to |U| (as the forward) */
            const float4 V = sV[la];
            const float p[3] = {V.x, V.y, V.z};
            float rv[3] = {r == 0 ? 0.0f : V.x, r == 1 ? 0.0f : V.y, r == 2 ? 0.0f : V.z};
            const float gs[3] = {sd.x, sd.y, sd.z};
            const float Ag[3] = {r == 0 ? 0.0f : gs[0], r == 1 ? 0.0f : gs[1], r == 2 ? 0.0f : gs[2]};
            const float mr = safe_sqrt(__fmaf_rn(rv[0], rv[0], __fmaf_rn(rv[1], rv[1], __fmul_rn(rv[2], rv[2]))));
            float ub[3];
            if (mr > 1e-7f) {
                const float mp = safe_sqrt(__fmaf_rn(p[0], p[0], __fmaf_rn(p[1], p[1], __fmul_rn(p[2], p[2]))));
                const float sc = mp / mr;
                const float rg = rv[0] * gs[0] + rv[1] * gs[1] + rv[2] * gs[2];
                const float c1 = mp > 0.0f ? rg / (mp * mr) : 0.0f;
                const float c2 = rg * mp / (mr * mr * mr);
#pragma unroll
                for (int c = 0; c < 3; c++) ub[c] = sc * Ag[c] + c1 * p[c] - c2 * rv[c];
            } else {
#pragma unroll
                for (int c = 0; c < 3; c++) ub[c] = Ag[c];
            }
            out = make_float4(ub[0] - sd.x, ub[1] - sd.y, ub[2] - sd.z, 0.0f);
        }
        sF[t] = out;
    }
    __syncthreads();

    /* phase 3: transposed line sums */
    grad_transform_t<NX, NY, NZ, 0>(sR, a, t);
    if constexpr (G::HAS_Y) grad_transform_t<NX, NY, NZ, 1>(sR, a, t);
    grad_transform_t<NX, NY, NZ, 2>(sR, a, t);
    __syncthreads();
    if (t >= NP) return;
    const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
    float vb[4] = {0, 0, 0, 0};
    auto lines = [&](const float* f, int nl, float J) {
#pragma unroll
        for (int c = 0; c < 4; c++) vb[c] = fmaf(J, f[c * nl], vb[c]);
    };
    lines(sR + LineLay<NX, NY, NZ, 0>::at(i, j, k), LineLay<NX, NY, NZ, 0>::NL, sMeta[0]);
    if constexpr (G::HAS_Y) lines(sR + LineLay<NX, NY, NZ, 1>::at(i, j, k), LineLay<NX, NY, NZ, 1>::NL, sMeta[1]);
    lines(sR + LineLay<NX, NY, NZ, 2>::at(i, j, k), LineLay<NX, NY, NZ, 2>::NL, sMeta[2]);
    auto face = [&](int slot) {
        const float4 f = sF[slot];
        vb[0] += f.x; vb[1] += f.y; vb[2] += f.z; vb[3] += f.w;
    };
    {
        const int sx = face_of_node<NX, NY, NZ, 0>(i, j, k);
        if (sx >= 0) face(sx);
        if constexpr (G::HAS_Y) {
            const int sy = face_of_node<NX, NY, NZ, 1>(i, j, k);
            if (sy >= 0) face(sy);
        }
        const int sz = face_of_node<NX, NY, NZ, 2>(i, j, k);
        if (sz >= 0) face(sz);
    }
    /* V = (m / rho, (Theta' - T0 rho') / rho), rho = rho_ref + rho' */
    const float4 V = sV[t];
    float xb[5];
    xb[0] = xbp[0] - inv * (vb[0] * V.x + vb[1] * V.y + vb[2] * V.z + vb[3] * (a.T0 + V.w));
    xb[1] = xbp[1] + vb[0] * inv;
    xb[2] = xbp[2] + vb[1] * inv;
    xb[3] = xbp[3] + vb[2] * inv;
    xb[4] = xbp[4] + vb[3] * inv;

    const int64_t o = e * 5 * NP + t;
    if constexpr (RS == 0) {
#pragma unroll
        for (int v = 0; v < 5; v++) a.Bout[o + v * NP] = xb[v];
        return;
    }
    const float dt = a.dt;
    if constexpr (RS == 3) {
#pragma unroll
        for (int v = 0; v < 5; v++) {
            const float x3 = dt * xb[v];
            a.A[o + v * NP] = x3;
            a.Bout[o + v * NP] = gb[v] + x3;
        }
    } else if constexpr (RS == 2) {
#pragma unroll
        for (int v = 0; v < 5; v++) {
            const float x2 = dt * xb[v];
            a.A[o + v * NP] = __ldg(a.A + o + v * NP) + x2;
            a.Bout[o + v * NP] = gb[v] + x2;
        }
    } else {
#pragma unroll
        for (int v = 0; v < 5; v++) {
            const float x1 = dt * xb[v];
            const double l = __ldg(a.lam + o + v * NP);
            a.lam_out[o + v * NP] = l + (f2d(__ldg(a.A + o + v * NP)) + f2d(x1));
        }
    }
}

template <int NX, int NY, int NZ>
int launch_adj(const AdjArgs& a, int rs, cudaStream_t st, int passes) {
    using G = Geo<NX, NY, NZ>;
    constexpr int SMEM = (int)AdjSmem<NX, NY, NZ>::BYTES;
    const unsigned grid = (unsigned)a.n_elem;
    if (a.GB) {
        /* viscous: pass 1 the flux transposes, pass 2 the gradients'
         * transpose and the stage combination */
        constexpr int GS = (int)AdjGradSmem<NX, NY, NZ>::BYTES;
        if (passes & 1) {
            switch (rs) {
                case 0: k_mixed_adj<NX, NY, NZ, 0, true><<<grid, G::BLOCK, SMEM, st>>>(a); break;
                case 1: k_mixed_adj<NX, NY, NZ, 1, true><<<grid, G::BLOCK, SMEM, st>>>(a); break;
                case 2: k_mixed_adj<NX, NY, NZ, 2, true><<<grid, G::BLOCK, SMEM, st>>>(a); break;
                default: k_mixed_adj<NX, NY, NZ, 3, true><<<grid, G::BLOCK, SMEM, st>>>(a); break;
            }
        }
        if (passes & 2) {
            switch (rs) {
                case 0: k_mixed_adj_grad<NX, NY, NZ, 0><<<grid, G::BLOCK, GS, st>>>(a); break;
                case 1: k_mixed_adj_grad<NX, NY, NZ, 1><<<grid, G::BLOCK, GS, st>>>(a); break;
                case 2: k_mixed_adj_grad<NX, NY, NZ, 2><<<grid, G::BLOCK, GS, st>>>(a); break;
                default: k_mixed_adj_grad<NX, NY, NZ, 3><<<grid, G::BLOCK, GS, st>>>(a); break;
            }
        }
        return (int)cudaGetLastError();
    }
    switch (rs) {
        case 0: k_mixed_adj<NX, NY, NZ, 0, false><<<grid, G::BLOCK, SMEM, st>>>(a); break;
        case 1: k_mixed_adj<NX, NY, NZ, 1, false><<<grid, G::BLOCK, SMEM, st>>>(a); break;
        case 2: k_mixed_adj<NX, NY, NZ, 2, false><<<grid, G::BLOCK, SMEM, st>>>(a); break;
        default: k_mixed_adj<NX, NY, NZ, 3, false><<<grid, G::BLOCK, SMEM, st>>>(a); break;
    }
    return (int)cudaGetLastError();
}

template <int NX, int NY, int NZ>
int prepare_adj() {
    constexpr int SMEM = (int)AdjSmem<NX, NY, NZ>::BYTES;
    constexpr int GS = (int)AdjGradSmem<NX, NY, NZ>::BYTES;
    const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
    int e = 0;
    if (SMEM > 48 * 1024) {
        e = (int)cudaFuncSetAttribute(k_mixed_adj<NX, NY, NZ, 0, false>, at, SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj<NX, NY, NZ, 1, false>, at, SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj<NX, NY, NZ, 2, false>, at, SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj<NX, NY, NZ, 3, false>, at, SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj<NX, NY, NZ, 0, true>, at, SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj<NX, NY, NZ, 1, true>, at, SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj<NX, NY, NZ, 2, true>, at, SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj<NX, NY, NZ, 3, true>, at, SMEM);
    }
    if (!e && GS > 48 * 1024) {
        e = (int)cudaFuncSetAttribute(k_mixed_adj_grad<NX, NY, NZ, 0>, at, GS);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj_grad<NX, NY, NZ, 1>, at, GS);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj_grad<NX, NY, NZ, 2>, at, GS);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj_grad<NX, NY, NZ, 3>, at, GS);
    }
    return e;
}

/* ------------------------------------------------------------------------
 * Transposes of the mortar kernels.  On a face on a 2:1 mortar the stage
 * kernel lifts MF = sum over the face node's entries of coef d, with
 * d = F.n at the fine node's slot and dC its projection onto a coarse node
 * (psiCor); F, the Rusanov flux of the slot, is formed from the fine node's
 * 19 face quantities and the coarse face's, interpolated with psiRef (|u|,
 * c, m, rho', the momentum flux tensor, the theta flux, Theta'; viscous runs
 * carry -mu grad U and -(mu/Pr) grad theta in the flux tensors).  Per
 * reverse stage, after the transposed stage kernel (whose face terms are
 * zero on mortar faces; in viscous runs after its first pass):
 *   k_mxa_fill_t  per mortar face node: MFbar = -C gbar (C the node's lift
 *                 coefficient), handed to its entries' dbar and dCbar (each
 *                 slot has one fine and one coarse entry);
 *   k_mxa_flux_t  per slot: Fbar = n dbar + the psiCor-weighted n dCbar of
 *                 the sub-face's slots; the Rusanov transpose gives both
 *                 sides' face-quantity adjoints; the fine side's go through
 *                 the fine node's quantity Jacobian into its state adjoint,
 *                 the coarse side's are kept per slot;
 *   k_mxa_gather  per mortar face node: the fine node takes its slot's state
 *                 adjoint; a coarse node sums, per sub-face, the psiRef-
 *                 weighted coarse-side adjoints of the slots interpolating
 *                 from it and applies its own quantity Jacobian; the result
 *                 enters the stage combination like the kernel's xbar
 *                 (atomic adds: an edge node lies on two faces), or in
 *                 viscous runs the first pass's state and gradient adjoints.
 * ------------------------------------------------------------------------ */
struct MxaArgs {
    const int32_t* mi;     /* [MX_FIELDS][n_ms] */
    const float* mf;       /* [8][n_ms] */
    const float* psiR;     /* [6][MAXN^2] */
    const float* psiC;     /* [6][MAXN^2] */
    const int32_t* ent;    /* [n_mf][nfmax][4] */
    const float* acoef;    /* [n_mf][nfmax][4] */
    const float* gs;       /* [n_mf][nfmax][4] gradient weights */
    const int32_t* node;   /* [n_mf][nfmax] */
    const int32_t* face;   /* [n_mf] */
    float* db;             /* [5][n_ms] */
    float* dCb;            /* [5][n_ms] */
    float* qb;             /* [19][n_ms] */
    float* xf;             /* [5][n_ms] */
    float* gf;             /* viscous: [12][n_ms] */
    float* gFb;            /* viscous: [4][n_ms] */
    float* gCb;            /* viscous: [4][n_ms] */
    float* vh;             /* viscous: [4][n_ms] */
    float* vown;           /* viscous: [4][n_mf nfmax] */
    int64_t n_ms, n_mf;
    int nfmax, np;
};

/* stage state, background and primitives of one node */
template <bool HAS_DIN>
__device__ __forceinline__ Pt mxa_node(const AdjArgs& a, int np, int64_t node, float* x, float* b) {
    const int64_t e = node / np;
    const int l = (int)(node - e * np);
    const int64_t o = e * 5 * np + l;
#pragma unroll
    for (int v = 0; v < 5; v++) x[v] = __ldg(a.S + o + v * np);
    if constexpr (HAS_DIN) {
#pragma unroll
        for (int v = 0; v < 5; v++) x[v] = __fadd_rn(x[v], __ldg(a.Din + o + v * np));
    }
    const float* bg = a.bg + (int64_t)__ldg(a.layer + e) * 4 * np + l;
#pragma unroll
    for (int c = 0; c < 4; c++) b[c] = __ldg(bg + c * np);
    return pointwise(x, b, a.eos, a.gamma, a.gR);
}

/* the node's gradients (viscous runs) */
__device__ __forceinline__ void mxa_grad(const AdjArgs& a, int np, int64_t node, float* g) {
    const int64_t e = node / np;
    const float* gr = a.Gv + e * 12 * np + (node - e * np);
#pragma unroll
    for (int c = 0; c < 12; c++) g[c] = __ldg(gr + c * np);
}

/* the 19 face quantities of a node, in the mortar flux kernel's layout;
 * viscous runs carry -mu grad U and -(mu/Pr) grad theta, mu = rho nu */
template <bool VISC>
__device__ __forceinline__ void face_q19(const float* x, const Pt& p, const float* g, const AdjArgs& a,
                                         float* f) {
    f[0] = p.umag;
    f[1] = p.c;
#pragma unroll
    for (int c = 0; c < 3; c++) f[2 + c] = x[1 + c];
    f[5] = x[0];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) f[6 + tidx(r, c)] = fmaf(x[1 + r], p.u[c], r == c ? p.pp : 0.0f);
#pragma unroll
    for (int c = 0; c < 3; c++) f[15 + c] = x[1 + c] * p.th;
    f[18] = x[4];
    if constexpr (VISC) {
        const float mu = p.rho * a.nu, mt = p.rho * a.nu_pr;
#pragma unroll
        for (int c = 0; c < 9; c++) f[6 + c] = fmaf(-mu, g[c], f[6 + c]);
#pragma unroll
        for (int c = 0; c < 3; c++) f[15 + c] = fmaf(-mt, g[9 + c], f[15 + c]);
    }
}

/* xb += (d q19 / dx)^T qb: |u| and c (d|u|/drho' = -|u|/rho, d|u|/dm_k =
 * u_k / (rho |u|), dc/drho' = -c / (2 rho), dc/dTheta' = c / (2 Theta)),
 * rho' and Theta' directly, and per direction c the flux vector
 * (m_c, m_r u_c + p' delta_rc, m_c theta) through the flux Jacobian;
 * viscous runs: the density adjoint of mu and the gradient adjoints gb */
template <bool VISC>
__device__ __forceinline__ void face_q19_t(const float* x, const float* b, const Pt& p,
                                           const float* g, const float* qb, const AdjArgs& a,
                                           float* xb, float* gb) {
    const float Th = __fadd_rn(b[1], x[4]);
    const float iTh = rcp_nr(Th);
    const float ku = p.umag > 0.0f ? p.inv * rcp_nr(p.umag) : 0.0f;
    xb[0] += fmaf(qb[0], -p.umag * p.inv, fmaf(qb[1], -0.5f * p.c * p.inv, qb[5]));
#pragma unroll
    for (int k = 0; k < 3; k++) xb[1 + k] = fmaf(qb[0], p.u[k] * ku, xb[1 + k]);
    xb[4] += fmaf(qb[1], 0.5f * p.c * iTh, qb[18]);
    const float pth = a.gamma * (b[3] + p.pp) * iTh;
    jft<0>(p.u, p.th, pth, qb[2], qb[6 + tidx(0, 0)], qb[6 + tidx(1, 0)], qb[6 + tidx(2, 0)], qb[15], xb);
    jft<1>(p.u, p.th, pth, qb[3], qb[6 + tidx(0, 1)], qb[6 + tidx(1, 1)], qb[6 + tidx(2, 1)], qb[16], xb);
    jft<2>(p.u, p.th, pth, qb[4], qb[6 + tidx(0, 2)], qb[6 + tidx(1, 2)], qb[6 + tidx(2, 2)], qb[17], xb);
    if constexpr (VISC) {
        const float mu = p.rho * a.nu, mt = p.rho * a.nu_pr;
        float sm = 0.0f, st = 0.0f;
#pragma unroll
        for (int c = 0; c < 9; c++) {
            sm = fmaf(g[c], qb[6 + c], sm);
            gb[c] = -mu * qb[6 + c];
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            st = fmaf(g[9 + c], qb[15 + c], st);
            gb[9 + c] = -mt * qb[15 + c];
        }
        xb[0] = fmaf(-a.nu, sm, fmaf(-a.nu_pr, st, xb[0]));
    }
}

/* a mortar term of the state adjoint into the stage combination (after the
 * transposed stage kernel): R3, R2 add dt xbar to A and to the stage output,
 * R1 to lam (FP64), R0 returns xbar; atomic adds, an edge node lies on two
 * element faces */
template <int RS>
__device__ __forceinline__ void add_to_stage(const AdjArgs& a, int64_t o, int np, const float* xb) {
#pragma unroll
    for (int v = 0; v < 5; v++) {
        if constexpr (RS == 0) {
            atomicAdd(a.Bout + o + v * np, xb[v]);
        } else if constexpr (RS == 1) {
            atomicAdd(a.lam_out + o + v * np, (double)(a.dt * xb[v]));
        } else {
            const float xv = a.dt * xb[v];
            atomicAdd(a.A + o + v * np, xv);
            atomicAdd(a.Bout + o + v * np, xv);
        }
    }
}

template <int RS>
__global__ void __launch_bounds__(128) k_mxa_fill_t(AdjArgs a, MxaArgs m) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= m.n_mf * m.nfmax) return;
    const int32_t node = __ldg(m.node + id);
    if (node < 0) return;
    const int64_t e = node / m.np;
    float gb[5];
    load_gbar<RS>(a, e * 5 * m.np + (node - e * m.np), m.np, gb);
    for (int q = 0; q < 4; q++) {
        const int32_t en = __ldg(m.ent + id * 4 + q);
        if (en < 0) break;
        const float c = __ldg(m.acoef + id * 4 + q);
        float* dst = (en & MX_COARSE) ? m.dCb : m.db;
        const int64_t ms = en & (MX_COARSE - 1);
#pragma unroll
        for (int v = 0; v < 5; v++) dst[v * m.n_ms + ms] = c * gb[v];
    }
}

template <bool HAS_DIN, bool VISC>
__global__ void __launch_bounds__(128) k_mxa_flux_t(AdjArgs a, MxaArgs m) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    auto fld = [&](int f) { return __ldg(m.mi + (int64_t)f * m.n_ms + ms); };
    /* the forward's face quantities: the fine node's, and the coarse face's
     * interpolated onto the slot */
    float xf[5], bf[4], gfn[12], f[19], q[19];
    const int64_t fnode = fld(MX_FINE);
    const Pt pf = mxa_node<HAS_DIN>(a, m.np, fnode, xf, bf);
    if constexpr (VISC) mxa_grad(a, m.np, fnode, gfn);
    face_q19<VISC>(xf, pf, gfn, a, f);
#pragma unroll
    for (int c = 0; c < 19; c++) q[c] = 0.0f;
    const int base = fld(MX_BASE), sa = fld(MX_SA), sb = fld(MX_SB), Na = fld(MX_NA),
              Nb = fld(MX_NB), ia = fld(MX_IA), ib = fld(MX_IB), first = fld(MX_FIRST),
              ta = fld(MX_TA), tb = fld(MX_TB);
    {
        const float* Pa = m.psiR + ta * MAXN * MAXN;
        const float* Pb = m.psiR + tb * MAXN * MAXN;
        for (int na = 0; na < Na; na++)
            for (int nb = 0; nb < Nb; nb++) {
                float x[5], b[4], g[12], qn[19];
                const int64_t cn = (int64_t)base + na * sa + nb * sb;
                const Pt p = mxa_node<HAS_DIN>(a, m.np, cn, x, b);
                if constexpr (VISC) mxa_grad(a, m.np, cn, g);
                face_q19<VISC>(x, p, g, a, qn);
                const float w = __ldg(Pa + na * Na + ia) * __ldg(Pb + nb * Nb + ib);
#pragma unroll
                for (int c = 0; c < 19; c++) q[c] = fmaf(w, qn[c], q[c]);
            }
    }
    const float* g = m.mf + ms;
    q[5] += __ldg(g + 6 * m.n_ms);
    q[18] += __ldg(g + 7 * m.n_ms);
    const float en[3] = {__ldg(g + 3 * m.n_ms), __ldg(g + 4 * m.n_ms), __ldg(g + 5 * m.n_ms)};
    /* Fbar: the fine side's d = F.n and the projections of the sub-face's
     * slots onto their coarse nodes, P(slot k) = sum_j psiCor(j -> k) F_j */
    float nd[5][3];
    {
        const float n[3] = {__ldg(g), __ldg(g + m.n_ms), __ldg(g + 2 * m.n_ms)};
#pragma unroll
        for (int v = 0; v < 5; v++) {
            const float d = __ldg(m.db + v * m.n_ms + ms);
#pragma unroll
            for (int c = 0; c < 3; c++) nd[v][c] = d * n[c];
        }
        const float* Pa = m.psiC + ta * MAXN * MAXN;
        const float* Pb = m.psiC + tb * MAXN * MAXN;
        for (int ka = 0; ka < Na; ka++)
            for (int kb = 0; kb < Nb; kb++) {
                const int64_t k = first + ka * Nb + kb;
                const float w = __ldg(Pa + ia * Na + ka) * __ldg(Pb + ib * Nb + kb);
                const float* gk = m.mf + k;
                const float nk[3] = {w * __ldg(gk), w * __ldg(gk + m.n_ms), w * __ldg(gk + 2 * m.n_ms)};
#pragma unroll
                for (int v = 0; v < 5; v++) {
                    const float d = __ldg(m.dCb + v * m.n_ms + k);
#pragma unroll
                    for (int c = 0; c < 3; c++) nd[v][c] = fmaf(d, nk[c], nd[v][c]);
                }
            }
    }
    /* Rusanov transpose: F_mass = (A_m + B_m)/2 - en lam (B_rho' - A_rho'),
     * F_mom[r][c] = (A + B)/2 - en_r lam (B_m - A_m)_c, F_theta likewise with
     * Theta', lam = ((|u|_A + |u|_B) + (c_A + c_B)) / 4; side 1 is the fine
     * side when MX_FINE_C1 is set */
    const bool fine1 = fld(MX_FINE_C1) != 0;
    float A[19], B[19];
#pragma unroll
    for (int c = 0; c < 19; c++) {
        A[c] = fine1 ? f[c] : q[c];
        B[c] = fine1 ? q[c] : f[c];
    }
    const float lam = 0.25f * ((A[0] + B[0]) + (A[1] + B[1]));
    float Ab[19], Bb[19];
#pragma unroll
    for (int c = 0; c < 19; c++) { Ab[c] = 0.0f; Bb[c] = 0.0f; }
    float lb = 0.0f;
    {
        const float jrb = -(en[0] * nd[0][0] + en[1] * nd[0][1] + en[2] * nd[0][2]);
        const float jtb = -(en[0] * nd[4][0] + en[1] * nd[4][1] + en[2] * nd[4][2]);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            Ab[2 + c] = 0.5f * nd[0][c];
            Ab[15 + c] = 0.5f * nd[4][c];
        }
        lb = fmaf(jrb, B[5] - A[5], jtb * (B[18] - A[18]));
        Ab[5] = -lam * jrb;
        Bb[5] = lam * jrb;
        Ab[18] = -lam * jtb;
        Bb[18] = lam * jtb;
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int c = 0; c < 3; c++) Ab[6 + tidx(r, c)] = 0.5f * nd[1 + r][c];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float dqb = -(en[0] * nd[1][c] + en[1] * nd[2][c] + en[2] * nd[3][c]);
            lb = fmaf(dqb, B[2 + c] - A[2 + c], lb);
            Bb[2 + c] = fmaf(lam, dqb, Ab[2 + c]);
            Ab[2 + c] = fmaf(-lam, dqb, Ab[2 + c]);
        }
#pragma unroll
        for (int c = 6; c < 18; c++) Bb[c] = Ab[c];
        Ab[0] = Ab[1] = Bb[0] = Bb[1] = 0.25f * lb;
    }
    /* the fine side through its node's Jacobian; the coarse side kept */
    float fb[19];
#pragma unroll
    for (int c = 0; c < 19; c++) {
        fb[c] = fine1 ? Ab[c] : Bb[c];
        m.qb[c * m.n_ms + ms] = fine1 ? Bb[c] : Ab[c];
    }
    float xb[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f}, gb[12];
    face_q19_t<VISC>(xf, bf, pf, gfn, fb, a, xb, gb);
#pragma unroll
    for (int v = 0; v < 5; v++) m.xf[v * m.n_ms + ms] = xb[v];
    if constexpr (VISC) {
#pragma unroll
        for (int c = 0; c < 12; c++) m.gf[c * m.n_ms + ms] = gb[c];
    }
}

/* per mortar face node: the fine node takes its slot's adjoints; a coarse
 * node (node (IA, IB) of the coarse face) sums, per sub-face, the psiRef-
 * weighted coarse-side adjoints of the slots interpolating from it and
 * applies its own quantity Jacobian.  Inviscid runs add the result to the
 * stage combination; viscous runs add it to the first pass's state adjoint
 * and gradient adjoints, before the gradients' transpose. */
template <int RS, bool VISC>
__global__ void __launch_bounds__(128) k_mxa_gather(AdjArgs a, MxaArgs m) {
    constexpr bool HAS_DIN = RS == 3 || RS == 2;
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= m.n_mf * m.nfmax) return;
    const int32_t node = __ldg(m.node + id);
    if (node < 0) return;
    float acc[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f}, gacc[12];
#pragma unroll
    for (int c = 0; c < 12; c++) gacc[c] = 0.0f;
    float qs[19];
#pragma unroll
    for (int c = 0; c < 19; c++) qs[c] = 0.0f;
    bool coarse = false;
    for (int q = 0; q < 4; q++) {
        const int32_t en = __ldg(m.ent + id * 4 + q);
        if (en < 0) break;
        const int64_t ms = en & (MX_COARSE - 1);
        if (!(en & MX_COARSE)) {
#pragma unroll
            for (int v = 0; v < 5; v++) acc[v] += __ldg(m.xf + v * m.n_ms + ms);
            if constexpr (VISC) {
#pragma unroll
                for (int c = 0; c < 12; c++) gacc[c] += __ldg(m.gf + c * m.n_ms + ms);
            }
            continue;
        }
        coarse = true;
        auto fld = [&](int f) { return __ldg(m.mi + (int64_t)f * m.n_ms + ms); };
        const int Na = fld(MX_NA), Nb = fld(MX_NB), na = fld(MX_IA), nb = fld(MX_IB),
                  first = fld(MX_FIRST);
        const float* Pa = m.psiR + fld(MX_TA) * MAXN * MAXN;
        const float* Pb = m.psiR + fld(MX_TB) * MAXN * MAXN;
        for (int ia = 0; ia < Na; ia++)
            for (int ib = 0; ib < Nb; ib++) {
                const int64_t k = first + ia * Nb + ib;
                const float w = __ldg(Pa + na * Na + ia) * __ldg(Pb + nb * Nb + ib);
#pragma unroll
                for (int c = 0; c < 19; c++) qs[c] = fmaf(w, __ldg(m.qb + c * m.n_ms + k), qs[c]);
            }
    }
    if (coarse) {
        float x[5], b[4], g[12], gb[12];
        const Pt p = mxa_node<HAS_DIN>(a, m.np, node, x, b);
        if constexpr (VISC) mxa_grad(a, m.np, node, g);
        face_q19_t<VISC>(x, b, p, g, qs, a, acc, gb);
        if constexpr (VISC) {
#pragma unroll
            for (int c = 0; c < 12; c++) gacc[c] += gb[c];
        }
    }
    const int64_t e = node / m.np;
    const int l = (int)(node - e * m.np);
    if constexpr (VISC) {
        const int64_t o = e * 5 * m.np + l;
#pragma unroll
        for (int v = 0; v < 5; v++) atomicAdd(a.XB + o + v * m.np, acc[v]);
        float* gr = a.GB + e * 12 * m.np + l;
#pragma unroll
        for (int c = 0; c < 12; c++) atomicAdd(gr + c * m.np, gacc[c]);
    } else {
        add_to_stage<RS>(a, e * 5 * m.np + l, m.np, acc);
    }
}

/* Viscous runs: the transposes of the gradients' mortar face values (after
 * the gradients' transpose, whose face terms are zero on mortar faces).  The
 * forward lifts on a mortar face node MF = sum_entries s (cds - V_own), s the
 * entry's weight (axis-aligned: gs; general geometry: the outward sign times
 * the slot's weighted normal per row), cds = (V_fine + psiRef-interpolated
 * V_coarse) / 2 at a slot, projected onto the coarse nodes with psiCor.
 *   k_mxa_gfill_t  per mortar face node: MFbar from the node's gradient
 *                  adjoints (the lift coefficient of the face, or 1/cV),
 *                  handed to the entries' cds adjoints, minus their sum to
 *                  the node's own V;
 *   k_mxa_ggather_t per slot: its cds adjoint plus the psiCor-weighted coarse
 *                  entries of the sub-face, halved;
 *   k_mxa_gcds_t   per mortar face node: own, fine-slot and psiRef-weighted
 *                  coarse-slot V adjoints, through V = (m / rho, (Theta' -
 *                  T0 rho') / rho) into the stage combination. */
template <bool GEN>
__global__ void __launch_bounds__(128) k_mxa_gfill_t(AdjArgs a, MxaArgs m) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nid = m.n_mf * m.nfmax;
    if (id >= nid) return;
    const int32_t node = __ldg(m.node + id);
    if (node < 0) return;
    const int64_t e = node / m.np;
    const int l = (int)(node - e * m.np);
    const float* gr = a.GB + e * 12 * m.np + l;
    constexpr int ND = GEN ? 12 : 4;
    float D[ND];
    if constexpr (GEN) {
        const float icv = __ldg(a.Jg + (e * 10 + 9) * m.np + l);
#pragma unroll
        for (int r = 0; r < 3; r++) {
            D[4 * r] = icv * gr[tidx(r, 0) * m.np];
            D[4 * r + 1] = icv * gr[tidx(r, 1) * m.np];
            D[4 * r + 2] = icv * gr[tidx(r, 2) * m.np];
            D[4 * r + 3] = icv * gr[(9 + r) * m.np];
        }
    } else {
        const int face = __ldg(m.face + id / m.nfmax), r = face >> 1;
        const float co = ((face & 1) ? 1.0f : -1.0f) * __ldg(a.J + (int64_t)r * a.n_elem + e) * a.lift[r];
        D[0] = co * gr[tidx(r, 0) * m.np];
        D[1] = co * gr[tidx(r, 1) * m.np];
        D[2] = co * gr[tidx(r, 2) * m.np];
        D[3] = co * gr[(9 + r) * m.np];
    }
    float own[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int q = 0; q < 4; q++) {
        const int32_t en = __ldg(m.ent + id * 4 + q);
        if (en < 0) break;
        const float w = __ldg(m.gs + id * 4 + q);
        const int64_t ms = en & (MX_COARSE - 1);
        float sv[4];
        if constexpr (GEN) {
            const float n0 = w * __ldg(m.mf + ms), n1 = w * __ldg(m.mf + m.n_ms + ms),
                        n2 = w * __ldg(m.mf + 2 * m.n_ms + ms);
#pragma unroll
            for (int c = 0; c < 4; c++) sv[c] = fmaf(n0, D[c], fmaf(n1, D[4 + c], n2 * D[8 + c]));
        } else {
#pragma unroll
            for (int c = 0; c < 4; c++) sv[c] = w * D[c];
        }
        float* dst = (en & MX_COARSE) ? m.gCb : m.gFb;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            dst[c * m.n_ms + ms] = sv[c];
            own[c] -= sv[c];
        }
    }
#pragma unroll
    for (int c = 0; c < 4; c++) m.vown[c * nid + id] = own[c];
}

__global__ void __launch_bounds__(128) k_mxa_ggather_t(MxaArgs m) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    auto fld = [&](int f) { return __ldg(m.mi + (int64_t)f * m.n_ms + ms); };
    const int Na = fld(MX_NA), Nb = fld(MX_NB), ia = fld(MX_IA), ib = fld(MX_IB),
              first = fld(MX_FIRST);
    const float* Pa = m.psiC + fld(MX_TA) * MAXN * MAXN;
    const float* Pb = m.psiC + fld(MX_TB) * MAXN * MAXN;
    float g[4];
#pragma unroll
    for (int c = 0; c < 4; c++) g[c] = __ldg(m.gFb + c * m.n_ms + ms);
    for (int ka = 0; ka < Na; ka++)
        for (int kb = 0; kb < Nb; kb++) {
            const int64_t k = first + ka * Nb + kb;
            const float w = __ldg(Pa + ia * Na + ka) * __ldg(Pb + ib * Nb + kb);
#pragma unroll
            for (int c = 0; c < 4; c++) g[c] = fmaf(w, __ldg(m.gCb + c * m.n_ms + k), g[c]);
        }
#pragma unroll
    for (int c = 0; c < 4; c++) m.vh[c * m.n_ms + ms] = 0.5f * g[c];
}

template <int RS>
__global__ void __launch_bounds__(128) k_mxa_gcds_t(AdjArgs a, MxaArgs m) {
    constexpr bool HAS_DIN = RS == 3 || RS == 2;
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nid = m.n_mf * m.nfmax;
    if (id >= nid) return;
    const int32_t node = __ldg(m.node + id);
    if (node < 0) return;
    float vb[4];
#pragma unroll
    for (int c = 0; c < 4; c++) vb[c] = __ldg(m.vown + c * nid + id);
    for (int q = 0; q < 4; q++) {
        const int32_t en = __ldg(m.ent + id * 4 + q);
        if (en < 0) break;
        const int64_t ms = en & (MX_COARSE - 1);
        if (!(en & MX_COARSE)) {
#pragma unroll
            for (int c = 0; c < 4; c++) vb[c] += __ldg(m.vh + c * m.n_ms + ms);
            continue;
        }
        auto fld = [&](int f) { return __ldg(m.mi + (int64_t)f * m.n_ms + ms); };
        const int Na = fld(MX_NA), Nb = fld(MX_NB), na = fld(MX_IA), nb = fld(MX_IB),
                  first = fld(MX_FIRST);
        const float* Pa = m.psiR + fld(MX_TA) * MAXN * MAXN;
        const float* Pb = m.psiR + fld(MX_TB) * MAXN * MAXN;
        for (int ia = 0; ia < Na; ia++)
            for (int ib = 0; ib < Nb; ib++) {
                const int64_t k = first + ia * Nb + ib;
                const float w = __ldg(Pa + na * Na + ia) * __ldg(Pb + nb * Nb + ib);
#pragma unroll
                for (int c = 0; c < 4; c++) vb[c] = fmaf(w, __ldg(m.vh + c * m.n_ms + k), vb[c]);
            }
    }
    /* V = (m / rho, (Theta' - T0 rho') / rho), rho = rho_ref + rho' */
    float x[5], b[4];
    mxa_node<HAS_DIN>(a, m.np, node, x, b);
    const float inv = rcp_nr(__fadd_rn(b[0], x[0]));
    const float V[4] = {__fmul_rn(x[1], inv), __fmul_rn(x[2], inv), __fmul_rn(x[3], inv),
                        __fmul_rn(__fmaf_rn(-a.T0, x[0], x[4]), inv)};
    float xb[5];
    xb[0] = -inv * (vb[0] * V[0] + vb[1] * V[1] + vb[2] * V[2] + vb[3] * (a.T0 + V[3]));
    xb[1] = vb[0] * inv;
    xb[2] = vb[1] * inv;
    xb[3] = vb[2] * inv;
    xb[4] = vb[3] * inv;
    const int64_t e = node / m.np;
    add_to_stage<RS>(a, e * 5 * m.np + (node - e * m.np), m.np, xb);
}

MxaArgs mxa_args(const NsemMixedBuf* mb) {
    MxaArgs m{};
    m.mi = mb->mx_i;
    m.mf = mb->mx_f;
    m.psiR = mb->mx_psi;
    m.psiC = mb->mx_psi + 6 * MAXN * MAXN;
    m.ent = mb->mf_ent;
    m.acoef = mb->mf_acoef;
    m.gs = mb->mf_gs;
    m.node = mb->mf_node;
    m.face = mb->mf_face;
    m.db = mb->mxa_db;
    m.dCb = mb->mxa_dCb;
    m.qb = mb->mxa_qb;
    m.xf = mb->mxa_xf;
    m.gf = mb->mxa_gf;
    m.gFb = mb->mxa_gFb;
    m.gCb = mb->mxa_gCb;
    m.vh = mb->mxa_vh;
    m.vown = mb->mxa_vown;
    m.n_ms = mb->n_ms;
    m.n_mf = mb->n_mf;
    m.nfmax = mb->nfmax;
    m.np = mb->npd[0] * mb->npd[1] * mb->npd[2];
    return m;
}

template <int RS>
void launch_mxa_flux(const MxaArgs& m, const AdjArgs& a, bool visc, cudaStream_t st) {
    constexpr bool HD = RS == 3 || RS == 2;
    const unsigned gn = (unsigned)((m.n_mf * m.nfmax + 127) / 128);
    const unsigned gs = (unsigned)((m.n_ms + 127) / 128);
    k_mxa_fill_t<RS><<<gn, 128, 0, st>>>(a, m);
    if (visc) {
        k_mxa_flux_t<HD, true><<<gs, 128, 0, st>>>(a, m);
        k_mxa_gather<RS, true><<<gn, 128, 0, st>>>(a, m);
    } else {
        k_mxa_flux_t<HD, false><<<gs, 128, 0, st>>>(a, m);
        k_mxa_gather<RS, false><<<gn, 128, 0, st>>>(a, m);
    }
}

template <int RS>
void launch_mxa_grad(const MxaArgs& m, const AdjArgs& a, bool gen, cudaStream_t st) {
    const unsigned gn = (unsigned)((m.n_mf * m.nfmax + 127) / 128);
    const unsigned gs = (unsigned)((m.n_ms + 127) / 128);
    if (gen) k_mxa_gfill_t<true><<<gn, 128, 0, st>>>(a, m);
    else k_mxa_gfill_t<false><<<gn, 128, 0, st>>>(a, m);
    k_mxa_ggather_t<<<gs, 128, 0, st>>>(m);
    k_mxa_gcds_t<RS><<<gn, 128, 0, st>>>(a, m);
}

/* part 1: the mortar flux transposes; part 2 (viscous runs): the
 * transposes of the gradients' mortar face values */
int launch_mortar_adj(const NsemMixedBuf* mb, const AdjArgs& a, int rs, cudaStream_t st, int part) {
    const MxaArgs m = mxa_args(mb);
    if (part == 1) {
        switch (rs) {
            case 3: launch_mxa_flux<3>(m, a, mb->visc, st); break;
            case 2: launch_mxa_flux<2>(m, a, mb->visc, st); break;
            case 1: launch_mxa_flux<1>(m, a, mb->visc, st); break;
            default: launch_mxa_flux<0>(m, a, mb->visc, st); break;
        }
    } else {
        switch (rs) {
            case 3: launch_mxa_grad<3>(m, a, mb->gen, st); break;
            case 2: launch_mxa_grad<2>(m, a, mb->gen, st); break;
            case 1: launch_mxa_grad<1>(m, a, mb->gen, st); break;
            default: launch_mxa_grad<0>(m, a, mb->gen, st); break;
        }
    }
    return (int)cudaGetLastError();
}

/* the transposed stage kernels: passes as launch_adj_general */
int launch_stage_adj(const NsemMixedBuf* mb, const AdjArgs& a, int rs, cudaStream_t st, int passes) {
    const int nx = mb->npd[0], ny = mb->npd[1], nz = mb->npd[2];
    if (mb->gen) return launch_adj_general(nx, ny, nz, a, rs, st, passes);
#define NSEM_ADJ(A, B, C) \
    if (nx == A && ny == B && nz == C) return launch_adj<A, B, C>(a, rs, st, passes);
    NSEM_MIXED_DIMS(NSEM_ADJ)
#undef NSEM_ADJ
    return (int)cudaErrorNotSupported;
}

int dispatch_adj(const NsemMixedBuf* mb, const AdjArgs& a, int rs, cudaStream_t st) {
    if (mb->n_ms == 0) return launch_stage_adj(mb, a, rs, st, 3);
    int e;
    if (!mb->visc) {
        /* the stage kernel, then the mortar transposes into its combination */
        if ((e = launch_stage_adj(mb, a, rs, st, 3))) return e;
        return launch_mortar_adj(mb, a, rs, st, 1);
    }
    /* viscous: the flux transposes (stage kernel, then mortar), the
     * gradients' transpose with the combination, then the mortar terms of
     * the gradients */
    if ((e = launch_stage_adj(mb, a, rs, st, 1))) return e;
    if ((e = launch_mortar_adj(mb, a, rs, st, 1))) return e;
    if ((e = launch_stage_adj(mb, a, rs, st, 2))) return e;
    return launch_mortar_adj(mb, a, rs, st, 2);
}

AdjArgs adj_args(const NsemDev* dev, const NsemMixedBuf* mb, double dt) {
    AdjArgs a{};
    a.nbr = mb->nbr;
    a.J = mb->J;
    a.layer = mb->layer;
    a.Qg = mb->Qg;
    a.bg = mb->bg;
    a.n_elem = mb->n_elem;
    if (mb->visc) {
        a.Gv = mb->G;
        a.GB = mb->GB;
        a.XB = mb->XB;
    }
    a.nu = mb->nu;
    a.nu_pr = mb->nu_pr;
    a.T0 = (float)dev->T0;
    std::memcpy(a.dc, mb->dc, sizeof(a.dc));
    a.Jg = mb->Jg;
    a.Fn = mb->Fn;
    a.dt = (float)dt;
    a.gamma = (float)dev->gamma;
    a.gR = (float)dev->gR;
    for (int c = 0; c < 3; c++) {
        a.g[c] = (float)dev->g[c];
        a.lift[c] = mb->lift[c];
    }
    std::memcpy(a.qc, mb->qc, sizeof(a.qc));
    double ck = 1.0;
    for (int k = 1; k <= 6; k++) {
        ck *= (dev->gamma - (k - 1)) / k;
        a.eos[k - 1] = (float)ck;
    }
    return a;
}

/* node-order SoA (5 arrays) <-> element-blocked, FP64 or FP32 */
struct CPtr5 {
    const double* p[5];
};
struct DPtr5 {
    double* p[5];
};

template <int NP>
__global__ void k_soa_to_blk(CPtr5 src, double* dst, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i / NP, o = e * 5 * NP + (i - e * NP);
#pragma unroll
        for (int v = 0; v < 5; v++) dst[o + v * NP] = src.p[v][i];
    }
}

template <int NP>
__global__ void k_soa_to_blk32(CPtr5 src, float* dst, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i / NP, o = e * 5 * NP + (i - e * NP);
#pragma unroll
        for (int v = 0; v < 5; v++) dst[o + v * NP] = (float)src.p[v][i];
    }
}

template <int NP>
__global__ void k_blk_to_soa(const double* src, DPtr5 dst, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i / NP, o = e * 5 * NP + (i - e * NP);
#pragma unroll
        for (int v = 0; v < 5; v++) dst.p[v][i] = src[o + v * NP];
    }
}

template <int NP>
__global__ void k_blk32_to_soa(const float* src, DPtr5 dst, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i / NP, o = e * 5 * NP + (i - e * NP);
#pragma unroll
        for (int v = 0; v < 5; v++) dst.p[v][i] = (double)src[o + v * NP];
    }
}

__global__ void k_shadow(const double* U, float* S, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        S[i] = d2f_rn(U[i]);
}

int grid_for(int64_t n) {
    int64_t g = (n + 255) / 256;
    if (g > 152 * 8) g = 152 * 8;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

int nsem_mixed_adj_prepare(const NsemMixedBuf* mb) {
    const int nx = mb->npd[0], ny = mb->npd[1], nz = mb->npd[2];
#define NSEM_PREP(A, B, C)                                                  \
    if (nx == A && ny == B && nz == C) {                                    \
        const int e = prepare_adj<A, B, C>();                              \
        return e ? e : prepare_adj_general(nx, ny, nz);                     \
    }
    NSEM_MIXED_DIMS(NSEM_PREP)
#undef NSEM_PREP
    return (int)cudaErrorNotSupported;
}

int nsem_mixed_layout(const NsemMixedBuf* mb, int dir, const double* const soa[5], double* blk,
                      double* const soa_out[5], void* stream) {
    const int NP = mb->npd[0] * mb->npd[1] * mb->npd[2];
    const int64_t n = mb->n_int;
    cudaStream_t st = (cudaStream_t)stream;
#define NSEM_LAY(A, B, C)                                                               \
    if (NP == A * B * C) {                                                              \
        if (dir == 0) {                                                                 \
            CPtr5 s;                                                                    \
            for (int v = 0; v < 5; v++) s.p[v] = soa[v];                                \
            k_soa_to_blk<A * B * C><<<grid_for(n), 256, 0, st>>>(s, blk, n);            \
        } else {                                                                        \
            DPtr5 d;                                                                    \
            for (int v = 0; v < 5; v++) d.p[v] = soa_out[v];                            \
            k_blk_to_soa<A * B * C><<<grid_for(n), 256, 0, st>>>(blk, d, n);            \
        }                                                                               \
        return (int)cudaGetLastError();                                                 \
    }
    NSEM_MIXED_DIMS(NSEM_LAY)
#undef NSEM_LAY
    return (int)cudaErrorNotSupported;
}

/* g = J_L(u)^T w for the current precision-form state (tendency VJP, FP32
 * bulk): w in five node-order FP64 arrays, g out likewise */
int nsem_mixed_vjp(const NsemDev* dev, NsemMixedBuf* mb, const double* const w[5],
                   double* const g[5], float* scratch_in, float* scratch_out, void* stream) {
    const int NP = mb->npd[0] * mb->npd[1] * mb->npd[2];
    const int64_t n = mb->n_int;
    cudaStream_t st = (cudaStream_t)stream;
    int e = 0;
#define NSEM_W(A, B, C)                                                                 \
    if (NP == A * B * C) {                                                              \
        CPtr5 s;                                                                        \
        for (int v = 0; v < 5; v++) s.p[v] = w[v];                                      \
        k_soa_to_blk32<A * B * C><<<grid_for(n), 256, 0, st>>>(s, scratch_in, n);       \
        e = (int)cudaGetLastError();                                                    \
    }
    NSEM_MIXED_DIMS(NSEM_W)
#undef NSEM_W
    if (e) return e;
    AdjArgs a = adj_args(dev, mb, 0.0);
    a.S = mb->S[mb->cur];
    a.Gin = scratch_in;
    a.Bout = scratch_out;
    if (mb->visc && (e = nsem_mixed_grad_at(dev, mb, a.S, nullptr, stream))) return e;
    if ((e = dispatch_adj(mb, a, 0, st))) return e;
#define NSEM_G(A, B, C)                                                                 \
    if (NP == A * B * C) {                                                              \
        DPtr5 d;                                                                        \
        for (int v = 0; v < 5; v++) d.p[v] = g[v];                                      \
        k_blk32_to_soa<A * B * C><<<grid_for(n), 256, 0, st>>>(scratch_out, d, n);      \
        return (int)cudaGetLastError();                                                 \
    }
    NSEM_MIXED_DIMS(NSEM_G)
#undef NSEM_G
    return (int)cudaErrorNotSupported;
}

/* adjoint arrays (lam, fin, abar), allocated on first use */
int nsem_mixed_adj_alloc(NsemMixedBuf* mb) {
    if (mb->lam) return 0;
    const int64_t n5 = 5 * mb->n_int;
    cudaError_t ce = cudaMalloc((void**)&mb->lam, (size_t)n5 * sizeof(double));
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&mb->fin, (size_t)n5 * sizeof(double));
    for (int q = 0; q < 3 && ce == cudaSuccess; q++)
        ce = cudaMalloc((void**)&mb->abar[q], (size_t)n5 * sizeof(float));
    if (ce == cudaSuccess && mb->visc) {
        ce = cudaMalloc((void**)&mb->GB, (size_t)12 * mb->n_int * sizeof(float));
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&mb->XB, (size_t)n5 * sizeof(float));
    }
    if (ce == cudaSuccess && mb->n_ms > 0) {
        ce = cudaMalloc((void**)&mb->mxa_db, (size_t)5 * mb->n_ms * sizeof(float));
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&mb->mxa_dCb, (size_t)5 * mb->n_ms * sizeof(float));
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&mb->mxa_qb, (size_t)19 * mb->n_ms * sizeof(float));
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&mb->mxa_xf, (size_t)5 * mb->n_ms * sizeof(float));
        if (ce == cudaSuccess && mb->visc) {
            const size_t nid = (size_t)mb->n_mf * mb->nfmax;
            ce = cudaMalloc((void**)&mb->mxa_gf, (size_t)12 * mb->n_ms * sizeof(float));
            if (ce == cudaSuccess) ce = cudaMalloc((void**)&mb->mxa_gFb, (size_t)4 * mb->n_ms * sizeof(float));
            if (ce == cudaSuccess) ce = cudaMalloc((void**)&mb->mxa_gCb, (size_t)4 * mb->n_ms * sizeof(float));
            if (ce == cudaSuccess) ce = cudaMalloc((void**)&mb->mxa_vh, (size_t)4 * mb->n_ms * sizeof(float));
            if (ce == cudaSuccess) ce = cudaMalloc((void**)&mb->mxa_vown, 4 * nid * sizeof(float));
        }
    }
    if (ce != cudaSuccess) return (int)ce;
    return nsem_mixed_adj_prepare(mb);
}

/* Checkpointed forward run of the precision form from u'^n = U[cur]:
 * checkpoints of u' (FP64) every `every` steps.  Storage (checkpoints, one
 * segment of stage states, adjoint arrays) is allocated here, outside any
 * stream capture. */
int nsem_mixed_fwd_ckpt(const NsemDev* dev, NsemMixedBuf* mb, int nsteps, int every, double dt,
                        void* stream) {
    const int64_t n5 = 5 * mb->n_int;
    const int n_ckpt = (nsteps + every - 1) / every;
    cudaStream_t st = (cudaStream_t)stream;
    if (mb->ckpt_slots < n_ckpt) {
        if (mb->ckpt) cudaFree(mb->ckpt);
        mb->ckpt = nullptr;
        mb->ckpt_slots = 0;
        cudaError_t ce = cudaMalloc((void**)&mb->ckpt, (size_t)n_ckpt * n5 * sizeof(double));
        if (ce != cudaSuccess) return (int)ce;
        mb->ckpt_slots = n_ckpt;
    }
    if (mb->seg_steps < every) {
        if (mb->seg) cudaFree(mb->seg);
        mb->seg = nullptr;
        mb->seg_steps = 0;
        cudaError_t ce = cudaMalloc((void**)&mb->seg, (size_t)every * 3 * n5 * sizeof(float));
        if (ce != cudaSuccess) return (int)ce;
        mb->seg_steps = every;
    }
    int e = nsem_mixed_adj_alloc(mb);
    if (e) return e;
    int cur = mb->cur;
    for (int s = 0; s < nsteps; s++) {
        if (s % every == 0) {
            cudaError_t ce = cudaMemcpyAsync(mb->ckpt + (int64_t)(s / every) * n5, mb->U[cur],
                                             (size_t)n5 * sizeof(double), cudaMemcpyDeviceToDevice, st);
            if (ce != cudaSuccess) return (int)ce;
        }
        if ((e = nsem_mixed_step_bufs(dev, mb, mb->U[cur], mb->S[cur], mb->D[0], mb->D[1],
                                      mb->U[cur ^ 1], mb->S[cur ^ 1], dt, stream)))
            return e;
        cur ^= 1;
    }
    mb->cur = cur;
    mb->nsteps = nsteps;
    mb->every = every;
    mb->n_ckpt = n_ckpt;
    return 0;
}

/* Reverse sweep: lam (element-blocked FP64, mb->lam) holds dJ/du' at the
 * final state; on return it holds dJ/du' at the initial state.  Each segment
 * is recomputed from its checkpoint keeping S, d1, d2 of every step, then
 * swept backwards.  The forward's final state is restored afterwards. */
int nsem_mixed_adjoint_run(const NsemDev* dev, NsemMixedBuf* mb, double dt, void* stream) {
    const int64_t n5 = 5 * mb->n_int;
    cudaStream_t st = (cudaStream_t)stream;
    const int cur = mb->cur;
    /* keep the final state (the recomputation uses the ping-pong buffers) */
    cudaError_t ce = cudaMemcpyAsync(mb->fin, mb->U[cur], (size_t)n5 * sizeof(double),
                                     cudaMemcpyDeviceToDevice, st);
    if (ce != cudaSuccess) return (int)ce;
    int e = 0;
    AdjArgs a = adj_args(dev, mb, dt);
    for (int sg = mb->n_ckpt - 1; sg >= 0; sg--) {
        const int start = sg * mb->every;
        const int cnt = (mb->nsteps - start < mb->every) ? mb->nsteps - start : mb->every;
        /* recompute the segment: step j reads U (FP64) and its shadow seg_S[j],
         * writes d1, d2 into the segment and the next shadow into seg_S[j+1] */
        const double* Uin = mb->ckpt + (int64_t)sg * n5;
        float* S0 = mb->seg;
        k_shadow<<<grid_for(n5), 256, 0, st>>>(Uin, S0, n5);
        if ((e = (int)cudaGetLastError())) return e;
        int pp = 0;
        for (int j = 0; j < cnt; j++) {
            float* Sj = mb->seg + (int64_t)j * 3 * n5;
            float* d1 = Sj + n5;
            float* d2 = Sj + 2 * n5;
            /* the last step's next shadow is not needed: write it to the
             * ping-pong shadow instead of past the segment */
            float* Snext = (j + 1 < cnt) ? mb->seg + (int64_t)(j + 1) * 3 * n5 : mb->S[pp];
            double* Unext = mb->U[pp];
            if ((e = nsem_mixed_step_bufs(dev, mb, Uin, Sj, d1, d2, Unext, Snext, dt, stream)))
                return e;
            Uin = Unext;
            pp ^= 1;
        }
        for (int j = cnt - 1; j >= 0; j--) {
            const float* Sj = mb->seg + (int64_t)j * 3 * n5;
            const float* d1 = Sj + n5;
            const float* d2 = Sj + 2 * n5;
            /* R3 at x3 = S + d2 (viscous runs: the stage state's gradients first) */
            a.S = Sj; a.Din = d2; a.lam = mb->lam; a.A = mb->abar[0]; a.Bout = mb->abar[1];
            if (mb->visc && (e = nsem_mixed_grad_at(dev, mb, Sj, d2, stream))) return e;
            if ((e = dispatch_adj(mb, a, 3, st))) return e;
            /* R2 at x2 = S + d1 */
            a.S = Sj; a.Din = d1; a.Gin = mb->abar[1]; a.A = mb->abar[0]; a.Bout = mb->abar[2];
            if (mb->visc && (e = nsem_mixed_grad_at(dev, mb, Sj, d1, stream))) return e;
            if ((e = dispatch_adj(mb, a, 2, st))) return e;
            /* R1 at x1 = S */
            a.S = Sj; a.Din = nullptr; a.Gin = mb->abar[2]; a.A = mb->abar[0];
            a.lam = mb->lam; a.lam_out = mb->lam;
            if (mb->visc && (e = nsem_mixed_grad_at(dev, mb, Sj, nullptr, stream))) return e;
            if ((e = dispatch_adj(mb, a, 1, st))) return e;
        }
    }
    /* restore the final state and its shadow */
    ce = cudaMemcpyAsync(mb->U[cur], mb->fin, (size_t)n5 * sizeof(double), cudaMemcpyDeviceToDevice, st);
    if (ce != cudaSuccess) return (int)ce;
    k_shadow<<<grid_for(n5), 256, 0, st>>>(mb->U[cur], mb->S[cur], n5);
    return (int)cudaGetLastError();
}
