/*
 * Discrete adjoint of the precision form on inclined and curved elements:
 * the transposed stage (k_mixed_adj_gen) and, for viscous runs, the
 * transpose of the full-metric gradients (k_mixed_adj_grad_gen), with their
 * launches.  The algorithm is described in nsem_mixed_adj.cu.
 */
#include <cuda_runtime.h>

#include "nsem_mixed_adj.cuh"

using namespace nsem_mx;
using namespace nsem_mxa;

namespace {

/* ------------------------------------------------------------------------
 * Inclined and curved elements (the transpose of k_mixed_stage_gen).  With
 * L_a = (1/cV_a) [sum_d sum_m T_d[a_d][m] G_d(m) - sum_faces F_out] + rho'_a g,
 * G_d = sum_c F_c (Jinv cV)[c][d] and F_out = (F_a + F_o).fN / 2
 * - lam (|fN| drho', en (dm.fN), |fN| dTheta'), given gbar per node:
 *   vbar = gbar / cV;  Gbar_d(m) = sum_a T_d[a_d][m] vbar_a (transposed line
 *   sums);  Fbar_c = sum_d (Jinv cV)[c][d] Gbar_d + sum_faces fN_c Phibar / 2;
 *   xbar = sum_c JF_c^T Fbar_c + the jump and lam terms + rho' g,
 * with Phibar = -vbar_a + vbar_o on a face node (the neighbour lifts -F_out
 * with its own 1/cV).  The Cartesian flux transposes are the axis-aligned
 * kernel's (jft, visc_t).
 * ------------------------------------------------------------------------ */
template <int NX, int NY, int NZ>
struct AdjGenSmem {
    using G = Geo<NX, NY, NZ>;
    static constexpr int NP = G::NP, NFS = G::NFS;
    /* floats: vbar [5][NP]; the transposed line sums (line-major); own values
     * P[3][NP] (x4) and Theta'; per face node Phibar / 2 (x4 + 1) and the
     * direct terms (x4 + 1) */
    static constexpr int OFF_R = (5 * NP + 3) / 4 * 4;
    static constexpr int OFF_P = (OFF_R + line_floats<NX, NY, NZ>() + 3) / 4 * 4;
    static constexpr int OFF_T = OFF_P + 12 * NP;
    static constexpr int OFF_FA4 = (OFF_T + NP + 3) / 4 * 4;
    static constexpr int OFF_FA1 = OFF_FA4 + 4 * NFS;
    static constexpr int OFF_XD4 = (OFF_FA1 + NFS + 3) / 4 * 4;
    static constexpr int OFF_XD1 = OFF_XD4 + 4 * NFS;
    static constexpr size_t BYTES = sizeof(float) * (OFF_XD1 + NFS);
};

template <int NX, int NY, int NZ, int RS, bool VISC>
__global__ void __launch_bounds__(Geo<NX, NY, NZ>::BLOCK, (adj_min_blocks<NX, NY, NZ>()))
k_mixed_adj_gen(AdjArgs a) {
    using G = Geo<NX, NY, NZ>;
    using SM = AdjGenSmem<NX, NY, NZ>;
    constexpr int NP = G::NP;
    constexpr int NFS = G::NFS;
    extern __shared__ float4 agen4[];
    float* smem = reinterpret_cast<float*>(agen4);
    float* sVb = smem;                                            /* [5][NP] */
    float* sR = smem + SM::OFF_R;
    float4* sP = reinterpret_cast<float4*>(smem + SM::OFF_P);
    float* sT = smem + SM::OFF_T;
    float4* sFa4 = reinterpret_cast<float4*>(smem + SM::OFF_FA4);
    float* sFa1 = smem + SM::OFF_FA1;
    float4* sXd4 = reinterpret_cast<float4*>(smem + SM::OFF_XD4);
    float* sXd1 = smem + SM::OFF_XD1;

    const int t = threadIdx.x;
    const int64_t e = blockIdx.x;
    constexpr bool has_din = RS == 3 || RS == 2;

    float x[5], gb[5], bgs[4] = {0, 0, 0, 0}, jin[9], icv = 0.0f;
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
        const float* jg = a.Jg + e * 10 * NP + t;
#pragma unroll
        for (int c = 0; c < 9; c++) jin[c] = __ldg(jg + c * NP);
        icv = __ldg(jg + 9 * NP);
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
    float xo[5], bgo[4], go[5], icvo = 0.0f, fno[3] = {0, 0, 0};
    if (t < NFS) {
        fs = face_slot<NX, NY, NZ>(t);
        nb = __ldg(a.nbr + (int64_t)fs.face * a.n_elem + e);
        /* a face on a 2:1 mortar (nb <= -2) lifts the mortar's outward value,
         * not a flux of its own: a zero normal zeroes its face terms (the
         * mortar transposes add the node's state adjoint afterwards) */
#pragma unroll
        for (int c = 0; c < 3; c++) fno[c] = nb <= -2 ? 0.0f : __ldg(a.Fn + (e * 3 + c) * NFS + t);
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
            icvo = __ldg(a.Jg + ((int64_t)nb * 10 + 9) * NP + fs.lo);
        }
    }

    /* phase 1: vbar = gbar / cV and the node's values */
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
        for (int v = 0; v < 5; v++) sVb[v * NP + t] = icv * gb[v];
        sP[t] = make_float4(x[0], x[1], x[2], x[3]);
        sP[NP + t] = make_float4(p.rho, p.umag, p.c, iTh);
        sP[2 * NP + t] = make_float4(p.u[0], p.u[1], p.u[2], pth);
        sT[t] = x[4];
    }
    __syncthreads();

    /* phase 2: face adjoints, per face node */
    if (t < NFS) {
        const int la = fs.la;
        const float4 P0 = sP[la], P1 = sP[NP + la], P2 = sP[2 * NP + la];
        const float tp_s = sT[la];
        const float rh = P1.x, um = P1.y, c = P1.z, iTh = P1.w;
        const float inv = rcp_nr(rh);
        const float nrm = safe_sqrt(fno[0] * fno[0] + fno[1] * fno[1] + fno[2] * fno[2]);
        const float inrm = nrm > 0.0f ? 1.0f / nrm : 0.0f;
        const float en[3] = {fno[0] * inrm, fno[1] * inrm, fno[2] * inrm};
        const float uv[3] = {P2.x, P2.y, P2.z};
        float pb[5];
#pragma unroll
        for (int v = 0; v < 5; v++) pb[v] = -sVb[v * NP + la];
        float4 fa4 = make_float4(0, 0, 0, 0), xd4;
        float fa1 = 0.0f, xd1;
        if (nb >= 0) {
            const Pt q = pointwise(xo, bgo, a.eos, a.gamma, a.gR);
            const float lam = 0.25f * ((um + q.umag) + (c + q.c));
#pragma unroll
            for (int v = 0; v < 5; v++) pb[v] = fmaf(icvo, go[v], pb[v]);
            fa4 = make_float4(0.5f * pb[0], 0.5f * pb[1], 0.5f * pb[2], 0.5f * pb[3]);
            fa1 = 0.5f * pb[4];
            const float jr = xo[0] - P0.x, jt = xo[4] - tp_s;
            const float dmn = (xo[1] - P0.y) * fno[0] + (xo[2] - P0.z) * fno[1] + (xo[3] - P0.w) * fno[2];
            const float epm = en[0] * pb[1] + en[1] * pb[2] + en[2] * pb[3];
            const float sj = fmaf(nrm, fmaf(jr, pb[0], jt * pb[4]), dmn * epm);
            const float q4 = -0.25f * sj;
            const float ku = um > 0.0f ? inv * rcp_nr(um) : 0.0f;
            xd4.x = fmaf(q4, -fmaf(0.5f, c, um) * inv, lam * nrm * pb[0]);
            xd4.y = fmaf(q4, uv[0] * ku, lam * fno[0] * epm);
            xd4.z = fmaf(q4, uv[1] * ku, lam * fno[1] * epm);
            xd4.w = fmaf(q4, uv[2] * ku, lam * fno[2] * epm);
            xd1 = fmaf(q4, 0.5f * c * iTh, lam * nrm * pb[4]);
        } else {
            /* wall: F_m = lam en (m.fN) + p' fN, lam = (|u_ghost| + c) / 2 */
            const float un = uv[0] * en[0] + uv[1] * en[1] + uv[2] * en[2];
            const float r3[3] = {uv[0] - un * en[0], uv[1] - un * en[1], uv[2] - un * en[2]};
            const float mr = safe_sqrt(r3[0] * r3[0] + r3[1] * r3[1] + r3[2] * r3[2]);
            const bool full = mr > 1e-7f;
            const float um_g = full ? um : mr;
            const float lam = 0.5f * (um_g + c);
            const float mn = P0.y * fno[0] + P0.z * fno[1] + P0.w * fno[2];
            const float epm = en[0] * pb[1] + en[1] * pb[2] + en[2] * pb[3];
            const float fpm = fno[0] * pb[1] + fno[1] * pb[2] + fno[2] * pb[3];
            const float q2 = 0.5f * mn * epm;
            const float nv = full ? um : mr;
            const float ku = nv > 0.0f ? inv * rcp_nr(nv) : 0.0f;
            const float vr[3] = {full ? uv[0] : r3[0], full ? uv[1] : r3[1], full ? uv[2] : r3[2]};
            xd4.x = q2 * -fmaf(0.5f, c, um_g) * inv;
            xd4.y = fmaf(q2, vr[0] * ku, lam * epm * fno[0]);
            xd4.z = fmaf(q2, vr[1] * ku, lam * epm * fno[1]);
            xd4.w = fmaf(q2, vr[2] * ku, lam * epm * fno[2]);
            xd1 = fmaf(q2, 0.5f * c * iTh, P2.w * fpm);
        }
        sFa4[t] = fa4;
        sFa1[t] = fa1;
        sXd4[t] = xd4;
        sXd1[t] = xd1;
    }
    /* the transposed line sums of the three reference directions */
    line_transform_t<NX, NY, NZ, 0>(sVb, sR, a, t);
    if constexpr (G::HAS_Y) line_transform_t<NX, NY, NZ, 1>(sVb, sR, a, t);
    line_transform_t<NX, NY, NZ, 2>(sVb, sR, a, t);
    __syncthreads();

    /* phase 3: Cartesian flux adjoints, transposes, face terms, update */
    if (t >= NP) return;
    const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
    float R[3][5];
    {
        const float* r0 = sR + LineLay<NX, NY, NZ, 0>::at(i, j, k);
        const float* r2 = sR + LineLay<NX, NY, NZ, 2>::at(i, j, k);
        constexpr int NL0 = LineLay<NX, NY, NZ, 0>::NL, NL2 = LineLay<NX, NY, NZ, 2>::NL;
#pragma unroll
        for (int v = 0; v < 5; v++) { R[0][v] = r0[v * NL0]; R[2][v] = r2[v * NL2]; R[1][v] = 0.0f; }
        if constexpr (G::HAS_Y) {
            const float* r1 = sR + LineLay<NX, NY, NZ, 1>::at(i, j, k);
            constexpr int NL1 = LineLay<NX, NY, NZ, 1>::NL;
#pragma unroll
            for (int v = 0; v < 5; v++) R[1][v] = r1[v * NL1];
        }
    }
    float F[3][5];
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int v = 0; v < 5; v++)
            F[c][v] = fmaf(jin[tidx(c, 0)], R[0][v], fmaf(jin[tidx(c, 1)], R[1][v], jin[tidx(c, 2)] * R[2][v]));
    float xb[5] = {0, 0, 0, 0, 0};
    auto face = [&](int slot) {
        const float4 f4 = sFa4[slot];
        const float f1 = sFa1[slot];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float n = __ldg(a.Fn + (e * 3 + c) * NFS + slot);
            F[c][0] = fmaf(n, f4.x, F[c][0]); F[c][1] = fmaf(n, f4.y, F[c][1]);
            F[c][2] = fmaf(n, f4.z, F[c][2]); F[c][3] = fmaf(n, f4.w, F[c][3]);
            F[c][4] = fmaf(n, f1, F[c][4]);
        }
        const float4 d4 = sXd4[slot];
        xb[0] += d4.x; xb[1] += d4.y; xb[2] += d4.z; xb[3] += d4.w; xb[4] += sXd1[slot];
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
    float gbv[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    float smv = 0.0f, stv = 0.0f;
    const float mu = rho * a.nu, mt = rho * a.nu_pr;
    {
        const float4 f0 = make_float4(F[0][0], F[0][1], F[0][2], F[0][3]);
        const float4 f1 = make_float4(F[1][0], F[1][1], F[1][2], F[1][3]);
        const float4 f2 = make_float4(F[2][0], F[2][1], F[2][2], F[2][3]);
        jft<0>(uu, th, pth, f0.x, f0.y, f0.z, f0.w, F[0][4], xb);
        jft<1>(uu, th, pth, f1.x, f1.y, f1.z, f1.w, F[1][4], xb);
        jft<2>(uu, th, pth, f2.x, f2.y, f2.z, f2.w, F[2][4], xb);
        if constexpr (VISC) {
            visc_t<0>(f0, F[0][4], gv, mu, mt, gbv, smv, stv);
            visc_t<1>(f1, F[1][4], gv, mu, mt, gbv, smv, stv);
            visc_t<2>(f2, F[2][4], gv, mu, mt, gbv, smv, stv);
        }
    }
    /* buoyancy: L_m += rho' g */
    xb[0] = fmaf(a.g[0], gb[1], fmaf(a.g[1], gb[2], fmaf(a.g[2], gb[3], xb[0])));

    const int64_t o = e * 5 * NP + t;
    if constexpr (VISC) {
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

/* Viscous runs on inclined and curved elements, second pass: the transpose
 * of k_mixed_grad_gen, G_r(a) = (1/cV_a) [sum_d (Jinv cV)[r][d](a)
 * sum_m D_d[a_d][m] V_m + sum_faces fN[r] (cds - V_a)]: per reference
 * direction the rows y_d = (1/cV) sum_r (Jinv cV)[r][d] Gbar_r go through
 * the transposed line sums, and per face node sDbar = (1/cV) sum_r fN[r]
 * Gbar_r: -1/2 to the node, +1/2 of the neighbour's (with its normal -fN and
 * its 1/cV) from the neighbour's side; on a wall the SYMMETRY ghost along the
 * unit normal is transposed. */
template <int NX, int NY, int NZ, int RS>
__global__ void __launch_bounds__(Geo<NX, NY, NZ>::BLOCK)
k_mixed_adj_grad_gen(AdjArgs a) {
    using G = Geo<NX, NY, NZ>;
    using SM = AdjGradSmem<NX, NY, NZ>;
    constexpr int NP = G::NP;
    constexpr int NFS = G::NFS;
    extern __shared__ float4 aggm4[];
    float* smem = reinterpret_cast<float*>(aggm4);
    float* sR = smem;
    float4* sV = reinterpret_cast<float4*>(smem + SM::OFF_V);
    float4* sF = reinterpret_cast<float4*>(smem + SM::OFF_F);
    const int t = threadIdx.x;
    const int64_t e = blockIdx.x;
    constexpr bool has_din = RS == 3 || RS == 2;

    float x[5], rref = 0.0f, gbv[12], xbp[5], gb[5], jin[9], icv = 0.0f;
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
        const float* jg = a.Jg + e * 10 * NP + t;
#pragma unroll
        for (int c = 0; c < 9; c++) jin[c] = __ldg(jg + c * NP);
        icv = __ldg(jg + 9 * NP);
    }
    FaceSlot fs{};
    int32_t nb = -1;
    float4 own_n = make_float4(0, 0, 0, 0), nb_n = make_float4(0, 0, 0, 0);
    float fno[3] = {0, 0, 0};
    if (t < NFS) {
        fs = face_slot<NX, NY, NZ>(t);
        nb = __ldg(a.nbr + (int64_t)fs.face * a.n_elem + e);
        /* a face on a 2:1 mortar: a zero normal zeroes the face terms here;
         * the mortar gradient transposes take them */
#pragma unroll
        for (int c = 0; c < 3; c++) fno[c] = nb <= -2 ? 0.0f : __ldg(a.Fn + (e * 3 + c) * NFS + t);
        /* sum_r fN[r] Gbar_r / cV at the own node and, with -fN, at the
         * neighbour's */
        auto dotn = [&](const float* gr, float ic, float sgn) {
            float4 r4 = make_float4(0, 0, 0, 0);
#pragma unroll
            for (int r = 0; r < 3; r++) {
                const float n = sgn * ic * fno[r];
                r4.x = fmaf(n, gr[tidx(r, 0) * NP], r4.x);
                r4.y = fmaf(n, gr[tidx(r, 1) * NP], r4.y);
                r4.z = fmaf(n, gr[tidx(r, 2) * NP], r4.z);
                r4.w = fmaf(n, gr[(9 + r) * NP], r4.w);
            }
            return r4;
        };
        own_n = dotn(a.GB + e * 12 * NP + fs.la, __ldg(a.Jg + (e * 10 + 9) * NP + fs.la), 1.0f);
        if (nb >= 0)
            nb_n = dotn(a.GB + (int64_t)nb * 12 * NP + fs.lo,
                        __ldg(a.Jg + ((int64_t)nb * 10 + 9) * NP + fs.lo), -1.0f);
    }

    /* phase 1: V and the rows y_d */
    float inv = 0.0f;
    if (t < NP) {
        inv = rcp_nr(__fadd_rn(rref, x[0]));
        sV[t] = make_float4(__fmul_rn(x[1], inv), __fmul_rn(x[2], inv), __fmul_rn(x[3], inv),
                            __fmul_rn(__fmaf_rn(-a.T0, x[0], x[4]), inv));
        const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
        auto put = [&](float* f, int nl, int d) {
            float y[4] = {0, 0, 0, 0};
#pragma unroll
            for (int r = 0; r < 3; r++) {
                const float w = icv * jin[tidx(r, d)];
                y[0] = fmaf(w, gbv[tidx(r, 0)], y[0]);
                y[1] = fmaf(w, gbv[tidx(r, 1)], y[1]);
                y[2] = fmaf(w, gbv[tidx(r, 2)], y[2]);
                y[3] = fmaf(w, gbv[9 + r], y[3]);
            }
            f[0] = y[0]; f[nl] = y[1]; f[2 * nl] = y[2]; f[3 * nl] = y[3];
        };
        put(sR + LineLay<NX, NY, NZ, 0>::at(i, j, k), LineLay<NX, NY, NZ, 0>::NL, 0);
        if constexpr (G::HAS_Y) put(sR + LineLay<NX, NY, NZ, 1>::at(i, j, k), LineLay<NX, NY, NZ, 1>::NL, 1);
        put(sR + LineLay<NX, NY, NZ, 2>::at(i, j, k), LineLay<NX, NY, NZ, 2>::NL, 2);
    }
    __syncthreads();

    /* phase 2: the face terms' adjoints for each face node */
    if (t < NFS) {
        const float4 sd = own_n;
        float4 out;
        if (nb >= 0) {
            out = make_float4(0.5f * (nb_n.x - sd.x), 0.5f * (nb_n.y - sd.y), 0.5f * (nb_n.z - sd.z),
                              0.5f * (nb_n.w - sd.w));
        } else {
            /* wall: the SYMMETRY ghost along the unit normal, theta copied */
            const float4 V = sV[fs.la];
            const float nrm = safe_sqrt(fno[0] * fno[0] + fno[1] * fno[1] + fno[2] * fno[2]);
            const float inrm = nrm > 0.0f ? 1.0f / nrm : 0.0f;
            const float en[3] = {fno[0] * inrm, fno[1] * inrm, fno[2] * inrm};
            const float p[3] = {V.x, V.y, V.z};
            const float un = p[0] * en[0] + p[1] * en[1] + p[2] * en[2];
            const float rv[3] = {p[0] - un * en[0], p[1] - un * en[1], p[2] - un * en[2]};
            const float gs[3] = {sd.x, sd.y, sd.z};
            const float gn = gs[0] * en[0] + gs[1] * en[1] + gs[2] * en[2];
            const float Ag[3] = {gs[0] - gn * en[0], gs[1] - gn * en[1], gs[2] - gn * en[2]};
            const float mr = safe_sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
            float ub[3];
            if (mr > 1e-7f) {
                const float mp = safe_sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
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

    /* phase 3: transposed line sums, face terms, back to the state, combination */
    grad_transform_t<NX, NY, NZ, 0>(sR, a, t);
    if constexpr (G::HAS_Y) grad_transform_t<NX, NY, NZ, 1>(sR, a, t);
    grad_transform_t<NX, NY, NZ, 2>(sR, a, t);
    __syncthreads();
    if (t >= NP) return;
    const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
    float vb[4] = {0, 0, 0, 0};
    auto lines = [&](const float* f, int nl) {
#pragma unroll
        for (int c = 0; c < 4; c++) vb[c] += f[c * nl];
    };
    lines(sR + LineLay<NX, NY, NZ, 0>::at(i, j, k), LineLay<NX, NY, NZ, 0>::NL);
    if constexpr (G::HAS_Y) lines(sR + LineLay<NX, NY, NZ, 1>::at(i, j, k), LineLay<NX, NY, NZ, 1>::NL);
    lines(sR + LineLay<NX, NY, NZ, 2>::at(i, j, k), LineLay<NX, NY, NZ, 2>::NL);
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
int launch_adj_gen(const AdjArgs& a, int rs, cudaStream_t st, int passes) {
    using G = Geo<NX, NY, NZ>;
    constexpr int SMEM = (int)AdjGenSmem<NX, NY, NZ>::BYTES;
    constexpr int GS = (int)AdjGradSmem<NX, NY, NZ>::BYTES;
    const unsigned grid = (unsigned)a.n_elem;
    if (a.GB) {
        /* viscous: pass 1 the flux transposes, pass 2 the gradients'
         * transpose and the stage combination */
        if (passes & 1) {
            switch (rs) {
                case 0: k_mixed_adj_gen<NX, NY, NZ, 0, true><<<grid, G::BLOCK, SMEM, st>>>(a); break;
                case 1: k_mixed_adj_gen<NX, NY, NZ, 1, true><<<grid, G::BLOCK, SMEM, st>>>(a); break;
                case 2: k_mixed_adj_gen<NX, NY, NZ, 2, true><<<grid, G::BLOCK, SMEM, st>>>(a); break;
                default: k_mixed_adj_gen<NX, NY, NZ, 3, true><<<grid, G::BLOCK, SMEM, st>>>(a); break;
            }
        }
        if (passes & 2) {
            switch (rs) {
                case 0: k_mixed_adj_grad_gen<NX, NY, NZ, 0><<<grid, G::BLOCK, GS, st>>>(a); break;
                case 1: k_mixed_adj_grad_gen<NX, NY, NZ, 1><<<grid, G::BLOCK, GS, st>>>(a); break;
                case 2: k_mixed_adj_grad_gen<NX, NY, NZ, 2><<<grid, G::BLOCK, GS, st>>>(a); break;
                default: k_mixed_adj_grad_gen<NX, NY, NZ, 3><<<grid, G::BLOCK, GS, st>>>(a); break;
            }
        }
        return (int)cudaGetLastError();
    }
    switch (rs) {
        case 0: k_mixed_adj_gen<NX, NY, NZ, 0, false><<<grid, G::BLOCK, SMEM, st>>>(a); break;
        case 1: k_mixed_adj_gen<NX, NY, NZ, 1, false><<<grid, G::BLOCK, SMEM, st>>>(a); break;
        case 2: k_mixed_adj_gen<NX, NY, NZ, 2, false><<<grid, G::BLOCK, SMEM, st>>>(a); break;
        default: k_mixed_adj_gen<NX, NY, NZ, 3, false><<<grid, G::BLOCK, SMEM, st>>>(a); break;
    }
    return (int)cudaGetLastError();
}

template <int NX, int NY, int NZ>
int prepare_adj_gen() {
    constexpr int SMEM = (int)AdjGenSmem<NX, NY, NZ>::BYTES;
    const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
    int e = 0;
    if (SMEM > 48 * 1024) {
        e = (int)cudaFuncSetAttribute(k_mixed_adj_gen<NX, NY, NZ, 0, false>, at, SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj_gen<NX, NY, NZ, 1, false>, at, SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj_gen<NX, NY, NZ, 2, false>, at, SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj_gen<NX, NY, NZ, 3, false>, at, SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj_gen<NX, NY, NZ, 0, true>, at, SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj_gen<NX, NY, NZ, 1, true>, at, SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj_gen<NX, NY, NZ, 2, true>, at, SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj_gen<NX, NY, NZ, 3, true>, at, SMEM);
    }
    constexpr int GS = (int)AdjGradSmem<NX, NY, NZ>::BYTES;
    if (!e && GS > 48 * 1024) {
        e = (int)cudaFuncSetAttribute(k_mixed_adj_grad_gen<NX, NY, NZ, 0>, at, GS);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj_grad_gen<NX, NY, NZ, 1>, at, GS);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj_grad_gen<NX, NY, NZ, 2>, at, GS);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_adj_grad_gen<NX, NY, NZ, 3>, at, GS);
    }
    return e;
}

}  // namespace

namespace nsem_mxa {

int launch_adj_general(int nx, int ny, int nz, const AdjArgs& a, int rs, cudaStream_t st, int passes) {
#define NSEM_ADJG(A, B, C) if (nx == A && ny == B && nz == C) return launch_adj_gen<A, B, C>(a, rs, st, passes);
    NSEM_MIXED_DIMS(NSEM_ADJG)
#undef NSEM_ADJG
    return (int)cudaErrorNotSupported;
}

int prepare_adj_general(int nx, int ny, int nz) {
#define NSEM_PREPG(A, B, C) if (nx == A && ny == B && nz == C) return prepare_adj_gen<A, B, C>();
    NSEM_MIXED_DIMS(NSEM_PREPG)
#undef NSEM_PREPG
    return (int)cudaErrorNotSupported;
}

}  // namespace nsem_mxa
