/*
 * Precision form on inclined and curved elements: the general-geometry stage
 * kernel k_mixed_stage_gen and the viscous runs' gradient kernel
 * k_mixed_grad_gen (full metric per node, face normals per face node), with
 * their launches.
 */
#include <cuda_runtime.h>

#include "nsem_mixed_kern.cuh"

using namespace nsem_mx;

namespace {

/* ------------------------------------------------------------------------
 * General geometry (inclined, curved elements): the metric is a
 * full 3x3 per node and the faces' normals are per face node.  The volume term
 * in the weak form of the plain form (field.h:3440-3464): per node the
 * contravariant fluxes G_d = sum_c F_c (Jinv cV)[c][d] -- mass M.Jcol_d,
 * momentum m_r (u.Jcol_d) + p' Jcol_d[r], theta (M.Jcol_d) theta -- and
 *   L_a = (1/cV_a) [sum_d sum_m l_a'(x_m) G_d(m) - sum_faces F_out] + rho' g,
 * F_out = (F_s + F_o).fN / 2 - lam (|fN| drho', en (dm.fN), |fN| dTheta'),
 * fN the face node's weighted normal pointing out of the element (the
 * reference's Rusanov flux, field.h:2928-2943, with the jump of the normal
 * momentum).  Both elements of a face evaluate it with fN and -fN: the
 * results are exact negatives, the face conserves exactly.
 * ------------------------------------------------------------------------ */
template <int NX, int NY, int NZ, bool VISC = false>
struct GenSmem {
    using G = Geo<NX, NY, NZ>;
    static constexpr int NP = G::NP, NFS = G::NFS;
    /* floats: contravariant fluxes, line-major per direction [3][n][5][NL];
     * own values P[4][NP] (x4); face fluxes FF4[NFS] (x4) + FF1[NFS];
     * viscous runs: the nodes' gradients GV[12][NP] */
    static constexpr int OFF_P = (line_floats<NX, NY, NZ>() + 3) / 4 * 4;
    static constexpr int OFF_FF4 = OFF_P + 16 * NP;
    static constexpr int OFF_FF1 = OFF_FF4 + 4 * NFS;
    static constexpr int OFF_GV = OFF_FF1 + NFS;
    static constexpr size_t BYTES = sizeof(float) * (OFF_GV + (VISC ? 12 * NP : 0));
};

/* normal flux F(x).fN of one side */
__device__ __forceinline__ void normal_flux(const float* m, const float* u, float pp, float th,
                                            const float* fN, float4& f4, float& f1) {
    const float mn = __fmaf_rn(m[0], fN[0], __fmaf_rn(m[1], fN[1], __fmul_rn(m[2], fN[2])));
    const float un = __fmaf_rn(u[0], fN[0], __fmaf_rn(u[1], fN[1], __fmul_rn(u[2], fN[2])));
    f4.x = mn;
    f4.y = __fmaf_rn(m[0], un, __fmul_rn(pp, fN[0]));
    f4.z = __fmaf_rn(m[1], un, __fmul_rn(pp, fN[1]));
    f4.w = __fmaf_rn(m[2], un, __fmul_rn(pp, fN[2]));
    f1 = __fmul_rn(mn, th);
}

/* resident CTAs per SM the registers are sized for (order 4 and below,
 * inviscid): stages 1-2, and stage 3, which loads the FP64 state only at the
 * update (measured on GB300, 32^3 box tilted by 30 degrees: 185 us at 8 CTAs,
 * 191 us at 6 or 7) */
#ifndef NSEM_GEN_MB12
#define NSEM_GEN_MB12 7
#endif
#ifndef NSEM_GEN_MB3
#define NSEM_GEN_MB3 8
#endif

template <int NX, int NY, int NZ, int STAGE, bool VISC>
__global__ void __launch_bounds__(Geo<NX, NY, NZ>::BLOCK,
                                  (min_blocks(NX == 8 ? 2 : (VISC ? 4 : (STAGE == 1 || STAGE == 2) ? NSEM_GEN_MB12 : NSEM_GEN_MB3), Geo<NX, NY, NZ>::BLOCK,
                                              GenSmem<NX, NY, NZ, VISC>::BYTES)))
k_mixed_stage_gen(StageArgs a) {
    using G = Geo<NX, NY, NZ>;
    using SM = GenSmem<NX, NY, NZ, VISC>;
    constexpr int NP = G::NP;
    constexpr int NFS = G::NFS;
    extern __shared__ float4 gen4[];
    float* smem = reinterpret_cast<float*>(gen4);
    float4* sP = reinterpret_cast<float4*>(smem + SM::OFF_P);
    float4* sFF4 = reinterpret_cast<float4*>(smem + SM::OFF_FF4);
    float* sFF1 = smem + SM::OFF_FF1;
    float* sGV = smem + SM::OFF_GV;     /* viscous runs: [12][NP] */
    const int t = threadIdx.x;
    const int64_t e = blockIdx.x;
    constexpr bool has_din = STAGE >= 2;

    float own[5], din[5] = {0, 0, 0, 0, 0}, bgs[4] = {0, 0, 0, 0}, jin[9], icv = 0.0f;
    float gown[12];
    if (t < NP) {
        const float* sp = a.S + e * 5 * NP + t;
#pragma unroll
        for (int v = 0; v < 5; v++) own[v] = __ldg(sp + v * NP);
        if constexpr (has_din) {
            const float* d = a.Din + e * 5 * NP + t;
#pragma unroll
            for (int v = 0; v < 5; v++) {
                din[v] = __ldg(d + v * NP);
                own[v] = __fadd_rn(own[v], din[v]);
            }
        }
        const float* bg = a.bg + (int64_t)__ldg(a.layer + e) * 4 * NP + t;
#pragma unroll
        for (int c = 0; c < 4; c++) bgs[c] = __ldg(bg + c * NP);
        const float* jg = a.Jg + e * 10 * NP + t;
#pragma unroll
        for (int c = 0; c < 9; c++) jin[c] = __ldg(jg + c * NP);
        icv = __ldg(jg + 9 * NP);
        if constexpr (STAGE == 3) {
            /* u'^n is needed only at the update: fetched into L2 here, loaded
             * there (with the increment reloaded), so that neither holds
             * registers through the element */
            const double* u = a.U + e * 5 * NP + t;
#pragma unroll
            for (int v = 0; v < 5; v++) asm volatile("prefetch.global.L2 [%0];" ::"l"(u + v * NP));
        }
        if constexpr (VISC) {
            const float* gr = a.G + e * 12 * NP + t;
#pragma unroll
            for (int c = 0; c < 12; c++) {
                gown[c] = __ldg(gr + c * NP);
                sGV[c * NP + t] = gown[c];
            }
        }
    }
    FaceSlot fs{};
    int32_t nb = -1;
    float oth[5], bgo[4], fno[3] = {0, 0, 0};
    if (t < NFS) {
        fs = face_slot<NX, NY, NZ, STAGE == 1 || STAGE == 2>(t);
        nb = __ldg(a.nbr + (int64_t)fs.face * a.n_elem + e);
#pragma unroll
        for (int c = 0; c < 3; c++) fno[c] = __ldg(a.Fn + (e * 3 + c) * NFS + t);
        if (nb <= -2) {
            /* a face on a 2:1 mortar: its outward values from the mortar kernels */
            const float* mf = a.MF + (int64_t)(-2 - nb) * MF_ROWS_GEN * a.nfmax + face_local<NX, NY, NZ>(t);
#pragma unroll
            for (int v = 0; v < 5; v++) oth[v] = __ldg(mf + v * a.nfmax);
        }
        if (nb >= 0) {
            const float* sp = a.S + (int64_t)nb * 5 * NP + fs.lo;
#pragma unroll
            for (int v = 0; v < 5; v++) oth[v] = __ldg(sp + v * NP);
            if constexpr (has_din) {
                const float* d = a.Din + (int64_t)nb * 5 * NP + fs.lo;
#pragma unroll
                for (int v = 0; v < 5; v++) oth[v] = __fadd_rn(oth[v], __ldg(d + v * NP));
            }
            const float* bg = a.bg + (int64_t)__ldg(a.layer + nb) * 4 * NP + fs.lo;
#pragma unroll
            for (int c = 0; c < 4; c++) bgo[c] = __ldg(bg + c * NP);
        }
    }
    /* viscous runs: the neighbour's gradients along the face node's normal,
     * sum_c d_r U_c n_c (r = 0..2) and sum_c d_c theta n_c */
    float gno[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if constexpr (VISC) {
        if (t < NFS && nb >= 0) {
            const float* gr = a.G + (int64_t)nb * 12 * NP + fs.lo;
            float g[12];
#pragma unroll
            for (int c = 0; c < 12; c++) g[c] = __ldg(gr + c * NP);
            /* the same association as the own side's (exact antisymmetry) */
#pragma unroll
            for (int r = 0; r < 3; r++)
                gno[r] = __fmaf_rn(g[tidx(r, 0)], fno[0],
                                   __fmaf_rn(g[tidx(r, 1)], fno[1], __fmul_rn(g[tidx(r, 2)], fno[2])));
            gno[3] = __fmaf_rn(g[9], fno[0], __fmaf_rn(g[10], fno[1], __fmul_rn(g[11], fno[2])));
        }
    }

    /* phase 1: primitives and contravariant fluxes */
    if (t < NP) {
        const Pt p = pointwise(own, bgs, a.eos, a.gamma, a.gR);
        sP[t] = make_float4(own[0], own[1], own[2], own[3]);
        sP[NP + t] = make_float4(own[4], p.rho, p.umag, p.c);
        sP[2 * NP + t] = make_float4(p.u[0], p.u[1], p.u[2], p.pp);
        sP[3 * NP + t] = make_float4(p.th, 0.0f, 0.0f, 0.0f);
        const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
        const int lpos[3] = {LineLay<NX, NY, NZ, 0>::at(i, j, k), LineLay<NX, NY, NZ, 1>::at(i, j, k),
                             LineLay<NX, NY, NZ, 2>::at(i, j, k)};
        const int lnl[3] = {LineLay<NX, NY, NZ, 0>::NL, LineLay<NX, NY, NZ, 1>::NL, LineLay<NX, NY, NZ, 2>::NL};
#pragma unroll
        for (int d = 0; d < 3; d++) {
            if (d == 1 && !G::HAS_Y) continue;
            const float j0 = jin[tidx(0, d)], j1 = jin[tidx(1, d)], j2 = jin[tidx(2, d)];
            const float Mt = fmaf(own[1], j0, fmaf(own[2], j1, own[3] * j2));
            const float ut = fmaf(p.u[0], j0, fmaf(p.u[1], j1, p.u[2] * j2));
            float4 g4 = make_float4(Mt, fmaf(own[1], ut, p.pp * j0), fmaf(own[2], ut, p.pp * j1),
                                    fmaf(own[3], ut, p.pp * j2));
            float g1 = Mt * p.th;
            if constexpr (VISC) {
                /* - mu d_r U_c (momentum r, direction c) and - (mu / Pr) d_c theta
                 * along the metric column, mu = rho nu */
                const float mu = p.rho * a.nu, mt = p.rho * a.nu_pr;
                g4.y = fmaf(-mu, fmaf(gown[tidx(0, 0)], j0, fmaf(gown[tidx(0, 1)], j1, gown[tidx(0, 2)] * j2)), g4.y);
                g4.z = fmaf(-mu, fmaf(gown[tidx(1, 0)], j0, fmaf(gown[tidx(1, 1)], j1, gown[tidx(1, 2)] * j2)), g4.z);
                g4.w = fmaf(-mu, fmaf(gown[tidx(2, 0)], j0, fmaf(gown[tidx(2, 1)], j1, gown[tidx(2, 2)] * j2)), g4.w);
                g1 = fmaf(-mt, fmaf(gown[9], j0, fmaf(gown[10], j1, gown[11] * j2)), g1);
            }
            float* f = smem + lpos[d];
            const int nl = lnl[d];
            f[0] = g4.x; f[nl] = g4.y; f[2 * nl] = g4.z; f[3 * nl] = g4.w; f[4 * nl] = g1;
        }
    }
    __syncthreads();

    /* phase 2: Rusanov flux through every face node, dotted with its normal */
    if (t < NFS) {
        const float4 P0 = sP[fs.la], P1 = sP[NP + fs.la], P2 = sP[2 * NP + fs.la];
        const float th_s = sP[3 * NP + fs.la].x;
        const float ms[3] = {P0.y, P0.z, P0.w}, us[3] = {P2.x, P2.y, P2.z};
        const float nrm = __fsqrt_rn(__fmaf_rn(fno[0], fno[0], __fmaf_rn(fno[1], fno[1], __fmul_rn(fno[2], fno[2]))));
        const float inrm = nrm > 0.0f ? 1.0f / nrm : 0.0f;
        const float en[3] = {__fmul_rn(fno[0], inrm), __fmul_rn(fno[1], inrm), __fmul_rn(fno[2], inrm)};
        float4 o4;
        float o1;
        if (nb <= -2) {
            o4 = make_float4(oth[0], oth[1], oth[2], oth[3]);
            o1 = oth[4];
        } else if (nb >= 0) {
            const Pt q = pointwise(oth, bgo, a.eos, a.gamma, a.gR);
            float4 A4, B4;
            float A1, B1;
            normal_flux(ms, us, P2.w, th_s, fno, A4, A1);
            normal_flux(oth + 1, q.u, q.pp, q.th, fno, B4, B1);
            const float lam = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(P1.z, q.umag), __fadd_rn(P1.w, q.c)));
            const float dm0 = __fsub_rn(oth[1], ms[0]), dm1 = __fsub_rn(oth[2], ms[1]),
                        dm2 = __fsub_rn(oth[3], ms[2]);
            const float dmn = __fmaf_rn(dm0, fno[0], __fmaf_rn(dm1, fno[1], __fmul_rn(dm2, fno[2])));
            const float jr = __fmul_rn(nrm, __fsub_rn(oth[0], P0.x));
            const float jt = __fmul_rn(nrm, __fsub_rn(oth[4], P1.x));
            if constexpr (VISC) {
                /* both sides' viscous normal fluxes, - mu (grad U) n and
                 * - (mu / Pr) (grad theta) . n, each side's from its own node */
                const float* gs = sGV + fs.la;
                float sn[4];
#pragma unroll
                for (int r = 0; r < 3; r++)
                    sn[r] = __fmaf_rn(gs[tidx(r, 0) * NP], fno[0],
                                      __fmaf_rn(gs[tidx(r, 1) * NP], fno[1], __fmul_rn(gs[tidx(r, 2) * NP], fno[2])));
                sn[3] = __fmaf_rn(gs[9 * NP], fno[0], __fmaf_rn(gs[10 * NP], fno[1], __fmul_rn(gs[11 * NP], fno[2])));
                const float mus = __fmul_rn(P1.y, a.nu), muo = __fmul_rn(q.rho, a.nu);
                const float mts = __fmul_rn(P1.y, a.nu_pr), mto = __fmul_rn(q.rho, a.nu_pr);
                A4.y = __fmaf_rn(-mus, sn[0], A4.y);
                A4.z = __fmaf_rn(-mus, sn[1], A4.z);
                A4.w = __fmaf_rn(-mus, sn[2], A4.w);
                A1 = __fmaf_rn(-mts, sn[3], A1);
                B4.y = __fmaf_rn(-muo, gno[0], B4.y);
                B4.z = __fmaf_rn(-muo, gno[1], B4.z);
                B4.w = __fmaf_rn(-muo, gno[2], B4.w);
                B1 = __fmaf_rn(-mto, gno[3], B1);
            }
            o4.x = __fmaf_rn(-lam, jr, __fmul_rn(0.5f, __fadd_rn(A4.x, B4.x)));
            o4.y = __fmaf_rn(-lam, __fmul_rn(en[0], dmn), __fmul_rn(0.5f, __fadd_rn(A4.y, B4.y)));
            o4.z = __fmaf_rn(-lam, __fmul_rn(en[1], dmn), __fmul_rn(0.5f, __fadd_rn(A4.z, B4.z)));
            o4.w = __fmaf_rn(-lam, __fmul_rn(en[2], dmn), __fmul_rn(0.5f, __fadd_rn(A4.w, B4.w)));
            o1 = __fmaf_rn(-lam, jt, __fmul_rn(0.5f, __fadd_rn(A1, B1)));
        } else {
            /* wall ghost (SYMMETRY velocity, NEUMANN rho, theta, p): the ghost's
             * normal flux is p' fN, the jump term lam en (m.fN) */
            const float un = __fmaf_rn(us[0], en[0], __fmaf_rn(us[1], en[1], __fmul_rn(us[2], en[2])));
            const float r0 = __fmaf_rn(-un, en[0], us[0]), r1 = __fmaf_rn(-un, en[1], us[1]),
                        r2 = __fmaf_rn(-un, en[2], us[2]);
            const float mr = safe_sqrt(__fmaf_rn(r0, r0, __fmaf_rn(r1, r1, __fmul_rn(r2, r2))));
            const float um_g = mr > 1e-7f ? P1.z : mr;
            const float lam = __fmul_rn(0.5f, __fadd_rn(um_g, P1.w));
            const float mn = __fmaf_rn(ms[0], fno[0], __fmaf_rn(ms[1], fno[1], __fmul_rn(ms[2], fno[2])));
            o4.x = 0.0f;
            o4.y = __fmaf_rn(lam, __fmul_rn(en[0], mn), __fmul_rn(P2.w, fno[0]));
            o4.z = __fmaf_rn(lam, __fmul_rn(en[1], mn), __fmul_rn(P2.w, fno[1]));
            o4.w = __fmaf_rn(lam, __fmul_rn(en[2], mn), __fmul_rn(P2.w, fno[2]));
            o1 = 0.0f;
        }
        sFF4[t] = o4;
        sFF1[t] = o1;
    }
    __syncthreads();

    /* phase 3: line sums l_a'(x_m) G_d(m) (in-place line transform), lift,
     * 1/cV, buoyancy, update */
    line_transform<NX, NY, NZ, 0>(smem, a, t);
    if constexpr (G::HAS_Y) line_transform<NX, NY, NZ, 1>(smem, a, t);
    line_transform<NX, NY, NZ, 2>(smem, a, t);
    __syncthreads();
    if (t >= NP) return;
    const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
    float4 acc;
    float acc1;
    {
        const float* rx = smem + LineLay<NX, NY, NZ, 0>::at(i, j, k);
        const float* rz = smem + LineLay<NX, NY, NZ, 2>::at(i, j, k);
        constexpr int NLX = LineLay<NX, NY, NZ, 0>::NL, NLZ = LineLay<NX, NY, NZ, 2>::NL;
        acc = make_float4(rx[0], rx[NLX], rx[2 * NLX], rx[3 * NLX]);
        acc1 = rx[4 * NLX];
        if constexpr (G::HAS_Y) {
            const float* ry = smem + LineLay<NX, NY, NZ, 1>::at(i, j, k);
            constexpr int NLY = LineLay<NX, NY, NZ, 1>::NL;
            acc.x += ry[0]; acc.y += ry[NLY]; acc.z += ry[2 * NLY]; acc.w += ry[3 * NLY];
            acc1 += ry[4 * NLY];
        }
        acc.x += rz[0]; acc.y += rz[NLZ]; acc.z += rz[2 * NLZ]; acc.w += rz[3 * NLZ];
        acc1 += rz[4 * NLZ];
    }
    auto lift = [&](int slot) {
        const float4 f = sFF4[slot];
        acc.x -= f.x; acc.y -= f.y; acc.z -= f.z; acc.w -= f.w; acc1 -= sFF1[slot];
    };
    {
        const int sx = face_of_node<NX, NY, NZ, 0>(i, j, k);
        if (sx >= 0) lift(sx);
        if constexpr (G::HAS_Y) {
            const int sy = face_of_node<NX, NY, NZ, 1>(i, j, k);
            if (sy >= 0) lift(sy);
        }
        const int sz = face_of_node<NX, NY, NZ, 2>(i, j, k);
        if (sz >= 0) lift(sz);
    }
    const float rp = own[0];
    const float Lv[5] = {icv * acc.x, fmaf(rp, a.g[0], icv * acc.y), fmaf(rp, a.g[1], icv * acc.z),
                         fmaf(rp, a.g[2], icv * acc.w), icv * acc1};
    if constexpr (STAGE == 0) {
        const int64_t n = e * NP + t;
#pragma unroll
        for (int v = 0; v < 5; v++) a.L[v][n] = f2d(Lv[v]);
        return;
    }
    const int64_t o = e * 5 * NP + t;
    const float dt = a.dt;
    if constexpr (STAGE == 1) {
#pragma unroll
        for (int v = 0; v < 5; v++) a.Dout[o + v * NP] = dt * Lv[v];
    } else if constexpr (STAGE == 2) {
#pragma unroll
        for (int v = 0; v < 5; v++) a.Dout[o + v * NP] = 0.25f * fmaf(dt, Lv[v], din[v]);
    } else {
        bool finite = true;
#pragma unroll
        for (int v = 0; v < 5; v++) {
            const float D = (2.0f / 3.0f) * fmaf(dt, Lv[v], __ldg(a.Din + o + v * NP));
            const double un = __ldg(a.U + o + v * NP) + f2d(D);
            a.Unew[o + v * NP] = un;
            a.Snew[o + v * NP] = d2f_rn(un);
            finite = finite && ((__double2hiint(un) & 0x7ff00000) != 0x7ff00000);
        }
        if (!finite) atomicOr(a.status, NSEM_STATUS_NONFINITE);
    }
}

/* General geometry (inclined, curved elements): the same gradients with the
 * node's full metric and the face nodes' normals (k_seg_grad_vol's strong
 * form, field.h:3327-3360):
 *   d_r q = (1/cV) [ sum_d (Jinv cV)[r][d] sum_m D_d[a_d][m] q_m
 *                    + sum_faces fN_out[r] (cds(q) - q) ],
 * the SYMMETRY ghost velocity along the face node's unit normal on walls. */
template <int NX, int NY, int NZ, int SIN>
__global__ void __launch_bounds__(Geo<NX, NY, NZ>::BLOCK)
k_mixed_grad_gen(StageArgs a) {
    using G = Geo<NX, NY, NZ>;
    constexpr int NP = G::NP;
    constexpr int NFS = G::NFS;
    constexpr bool has_din = SIN >= 2;
    extern __shared__ float4 ggsm4[];
    float4* sV = ggsm4;                                             /* [NP]  U, theta - T0 */
    float4* sD = ggsm4 + NP;                                        /* [NFS] cds - own */
    float* sDg = reinterpret_cast<float*>(ggsm4 + NP + NFS);       /* line tables */
    const int t = threadIdx.x;
    const int64_t e = blockIdx.x;

    float own[5], bgs0 = 0.0f, jin[9], icv = 0.0f;
    if (t < NP) {
        const float* s = a.S + e * 5 * NP + t;
#pragma unroll
        for (int v = 0; v < 5; v++) own[v] = __ldg(s + v * NP);
        if (has_din) {
            const float* d = a.Din + e * 5 * NP + t;
#pragma unroll
            for (int v = 0; v < 5; v++) own[v] = __fadd_rn(own[v], __ldg(d + v * NP));
        }
        bgs0 = __ldg(a.bg + (int64_t)__ldg(a.layer + e) * 4 * NP + t);
        const float* jg = a.Jg + e * 10 * NP + t;
#pragma unroll
        for (int c = 0; c < 9; c++) jin[c] = __ldg(jg + c * NP);
        icv = __ldg(jg + 9 * NP);
    }
    FaceSlot fs{};
    int32_t nb = -1;
    float oth[5], bgo0 = 0.0f, fno[3] = {0, 0, 0};
    if (t < NFS) {
        fs = face_slot<NX, NY, NZ>(t);
        nb = __ldg(a.nbr + (int64_t)fs.face * a.n_elem + e);
#pragma unroll
        for (int c = 0; c < 3; c++) fno[c] = __ldg(a.Fn + (e * 3 + c) * NFS + t);
        if (nb >= 0) {
            const float* s = a.S + (int64_t)nb * 5 * NP + fs.lo;
#pragma unroll
            for (int v = 0; v < 5; v++) oth[v] = __ldg(s + v * NP);
            if (has_din) {
                const float* d = a.Din + (int64_t)nb * 5 * NP + fs.lo;
#pragma unroll
                for (int v = 0; v < 5; v++) oth[v] = __fadd_rn(oth[v], __ldg(d + v * NP));
            }
            bgo0 = __ldg(a.bg + (int64_t)__ldg(a.layer + nb) * 4 * NP + fs.lo);
        }
    }
    for (int q = t; q < QTAB; q += G::BLOCK) sDg[q] = __ldg(a.Dg + q);

    const float T0 = a.T0;
    auto prim_ut = [T0](const float* s, float rref) {
        const float inv = rcp_nr(__fadd_rn(rref, s[0]));
        return make_float4(__fmul_rn(s[1], inv), __fmul_rn(s[2], inv), __fmul_rn(s[3], inv),
                           __fmul_rn(__fmaf_rn(-T0, s[0], s[4]), inv));
    };
    if (t < NP) sV[t] = prim_ut(own, bgs0);
    __syncthreads();

    if (t < NFS && nb > -2) {
        const float4 S = sV[fs.la];
        float4 c;
        if (nb >= 0) {
            const float4 O = prim_ut(oth, bgo0);
            c = make_float4(0.5f * S.x + 0.5f * O.x, 0.5f * S.y + 0.5f * O.y,
                            0.5f * S.z + 0.5f * O.z, 0.5f * S.w + 0.5f * O.w);
        } else {
            /* wall ghost: SYMMETRY velocity (tangential part rescaled to |U|),
             * NEUMANN theta */
            const float nrm = safe_sqrt(fno[0] * fno[0] + fno[1] * fno[1] + fno[2] * fno[2]);
            const float inrm = nrm > 0.0f ? 1.0f / nrm : 0.0f;
            const float en[3] = {fno[0] * inrm, fno[1] * inrm, fno[2] * inrm};
            const float un = S.x * en[0] + S.y * en[1] + S.z * en[2];
            float r0 = S.x - un * en[0], r1 = S.y - un * en[1], r2 = S.z - un * en[2];
            const float mr = safe_sqrt(r0 * r0 + r1 * r1 + r2 * r2);
            if (mr > 1e-7f) {
                const float sc = safe_sqrt(S.x * S.x + S.y * S.y + S.z * S.z) / mr;
                r0 *= sc; r1 *= sc; r2 *= sc;
            }
            c = make_float4(r0, r1, r2, S.w);
        }
        sD[t] = make_float4(c.x - S.x, c.y - S.y, c.z - S.z, c.w - S.w);
    }
    __syncthreads();

    if (t >= NP) return;
    const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
    /* derivatives along the reference directions */
    float4 d[3];
#pragma unroll
    for (int r = 0; r < 3; r++) d[r] = make_float4(0, 0, 0, 0);
    {
        const float* q = sDg + i * QS;
#pragma unroll
        for (int m = 0; m < NX; m++) {
            const float4 v = sV[(m * NY + j) * NZ + k];
            d[0].x = fmaf(q[m], v.x, d[0].x); d[0].y = fmaf(q[m], v.y, d[0].y);
            d[0].z = fmaf(q[m], v.z, d[0].z); d[0].w = fmaf(q[m], v.w, d[0].w);
        }
    }
    if constexpr (G::HAS_Y) {
        const float* q = sDg + MAXN * QS + j * QS;
#pragma unroll
        for (int m = 0; m < NY; m++) {
            const float4 v = sV[(i * NY + m) * NZ + k];
            d[1].x = fmaf(q[m], v.x, d[1].x); d[1].y = fmaf(q[m], v.y, d[1].y);
            d[1].z = fmaf(q[m], v.z, d[1].z); d[1].w = fmaf(q[m], v.w, d[1].w);
        }
    }
    {
        const float* q = sDg + 2 * MAXN * QS + k * QS;
#pragma unroll
        for (int m = 0; m < NZ; m++) {
            const float4 v = sV[(i * NY + j) * NZ + m];
            d[2].x = fmaf(q[m], v.x, d[2].x); d[2].y = fmaf(q[m], v.y, d[2].y);
            d[2].z = fmaf(q[m], v.z, d[2].z); d[2].w = fmaf(q[m], v.w, d[2].w);
        }
    }
    /* physical components: sum_d (Jinv cV)[r][d] d_d, then the face terms */
    float4 g[3];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        const float j0 = jin[tidx(r, 0)], j1 = jin[tidx(r, 1)], j2 = jin[tidx(r, 2)];
        g[r] = make_float4(fmaf(j0, d[0].x, fmaf(j1, d[1].x, j2 * d[2].x)),
                           fmaf(j0, d[0].y, fmaf(j1, d[1].y, j2 * d[2].y)),
                           fmaf(j0, d[0].z, fmaf(j1, d[1].z, j2 * d[2].z)),
                           fmaf(j0, d[0].w, fmaf(j1, d[1].w, j2 * d[2].w)));
    }
    auto lift = [&](int slot) {
        const FaceSlot f2 = face_slot<NX, NY, NZ>(slot);
        const int32_t nbf = __ldg(a.nbr + (int64_t)f2.face * a.n_elem + e);
        if (nbf <= -2) {
            /* a face on a 2:1 mortar: fN_out[r] (cds - own) summed by the mortar kernels */
            const float* gf = a.MF + ((int64_t)(-2 - nbf) * MF_ROWS_GEN + 5) * a.nfmax +
                              face_local<NX, NY, NZ>(slot);
#pragma unroll
            for (int r = 0; r < 3; r++) {
                g[r].x += __ldg(gf + (4 * r) * a.nfmax);
                g[r].y += __ldg(gf + (4 * r + 1) * a.nfmax);
                g[r].z += __ldg(gf + (4 * r + 2) * a.nfmax);
                g[r].w += __ldg(gf + (4 * r + 3) * a.nfmax);
            }
            return;
        }
        const float4 f = sD[slot];
#pragma unroll
        for (int r = 0; r < 3; r++) {
            const float n = __ldg(a.Fn + (e * 3 + r) * NFS + slot);
            g[r].x = fmaf(n, f.x, g[r].x); g[r].y = fmaf(n, f.y, g[r].y);
            g[r].z = fmaf(n, f.z, g[r].z); g[r].w = fmaf(n, f.w, g[r].w);
        }
    };
    {
        const int sx = face_of_node<NX, NY, NZ, 0>(i, j, k);
        if (sx >= 0) lift(sx);
        if constexpr (G::HAS_Y) {
            const int sy = face_of_node<NX, NY, NZ, 1>(i, j, k);
            if (sy >= 0) lift(sy);
        }
        const int sz = face_of_node<NX, NY, NZ, 2>(i, j, k);
        if (sz >= 0) lift(sz);
    }
    float* out = a.Gout + e * 12 * NP + t;
#pragma unroll
    for (int r = 0; r < 3; r++) {
        out[tidx(r, 0) * NP] = icv * g[r].x;
        out[tidx(r, 1) * NP] = icv * g[r].y;
        out[tidx(r, 2) * NP] = icv * g[r].z;
        out[(9 + r) * NP] = icv * g[r].w;
    }
}


template <int NX, int NY, int NZ>
int launch_gen(const StageArgs& a, int stage, cudaStream_t st, bool visc) {
    using G = Geo<NX, NY, NZ>;
    const unsigned grid = (unsigned)a.n_elem;
    if (visc) {
        constexpr size_t SMEM = GenSmem<NX, NY, NZ, true>::BYTES;
        switch (stage) {
            case 0: k_mixed_stage_gen<NX, NY, NZ, 0, true><<<grid, G::BLOCK, SMEM, st>>>(a); break;
            case 1: k_mixed_stage_gen<NX, NY, NZ, 1, true><<<grid, G::BLOCK, SMEM, st>>>(a); break;
            case 2: k_mixed_stage_gen<NX, NY, NZ, 2, true><<<grid, G::BLOCK, SMEM, st>>>(a); break;
            default: k_mixed_stage_gen<NX, NY, NZ, 3, true><<<grid, G::BLOCK, SMEM, st>>>(a); break;
        }
        return (int)cudaGetLastError();
    }
    constexpr size_t SMEM = GenSmem<NX, NY, NZ>::BYTES;
    switch (stage) {
        case 0: k_mixed_stage_gen<NX, NY, NZ, 0, false><<<grid, G::BLOCK, SMEM, st>>>(a); break;
        case 1: k_mixed_stage_gen<NX, NY, NZ, 1, false><<<grid, G::BLOCK, SMEM, st>>>(a); break;
        case 2: k_mixed_stage_gen<NX, NY, NZ, 2, false><<<grid, G::BLOCK, SMEM, st>>>(a); break;
        default: k_mixed_stage_gen<NX, NY, NZ, 3, false><<<grid, G::BLOCK, SMEM, st>>>(a); break;
    }
    return (int)cudaGetLastError();
}

template <int NX, int NY, int NZ>
int launch_grad_gen(const StageArgs& a, int stage, cudaStream_t st) {
    using G = Geo<NX, NY, NZ>;
    const unsigned grid = (unsigned)a.n_elem;
    constexpr size_t gs = grad_smem<NX, NY, NZ>();
    if (stage <= 1) k_mixed_grad_gen<NX, NY, NZ, 1><<<grid, G::BLOCK, gs, st>>>(a);
    else k_mixed_grad_gen<NX, NY, NZ, 2><<<grid, G::BLOCK, gs, st>>>(a);
    return (int)cudaGetLastError();
}

template <int NX, int NY, int NZ>
int prepare_gen() {
    int e = 0;
    constexpr int GS = (int)GenSmem<NX, NY, NZ>::BYTES;
    constexpr int GSV = (int)GenSmem<NX, NY, NZ, true>::BYTES;
    const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
    if (GS > 48 * 1024) {
        e = (int)cudaFuncSetAttribute(k_mixed_stage_gen<NX, NY, NZ, 0, false>, at, GS);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_stage_gen<NX, NY, NZ, 1, false>, at, GS);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_stage_gen<NX, NY, NZ, 2, false>, at, GS);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_stage_gen<NX, NY, NZ, 3, false>, at, GS);
    }
    if (!e && GSV > 48 * 1024) {
        e = (int)cudaFuncSetAttribute(k_mixed_stage_gen<NX, NY, NZ, 0, true>, at, GSV);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_stage_gen<NX, NY, NZ, 1, true>, at, GSV);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_stage_gen<NX, NY, NZ, 2, true>, at, GSV);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_stage_gen<NX, NY, NZ, 3, true>, at, GSV);
    }
    constexpr size_t gs = grad_smem<NX, NY, NZ>();
    if (!e && gs > 48 * 1024) {
        e = (int)cudaFuncSetAttribute(k_mixed_grad_gen<NX, NY, NZ, 1>, at, (int)gs);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_grad_gen<NX, NY, NZ, 2>, at, (int)gs);
    }
    return e;
}

}  // namespace

namespace nsem_mx {

int prepare_general(int nx, int ny, int nz) {
#define NSEM_PREPG(A, B, C) if (nx == A && ny == B && nz == C) return prepare_gen<A, B, C>();
    NSEM_MIXED_DIMS(NSEM_PREPG)
#undef NSEM_PREPG
    return (int)cudaErrorNotSupported;
}

int launch_stage_general(int nx, int ny, int nz, const StageArgs& a, int stage, cudaStream_t st,
                         bool visc) {
#define NSEM_DISP(A, B, C) \
    if (nx == A && ny == B && nz == C) return launch_gen<A, B, C>(a, stage, st, visc);
    NSEM_MIXED_DIMS(NSEM_DISP)
#undef NSEM_DISP
    return (int)cudaErrorNotSupported;
}

int launch_grad_general(int nx, int ny, int nz, const StageArgs& a, int stage, cudaStream_t st) {
#define NSEM_DISPG(A, B, C) \
    if (nx == A && ny == B && nz == C) return launch_grad_gen<A, B, C>(a, stage, st);
    NSEM_MIXED_DIMS(NSEM_DISPG)
#undef NSEM_DISPG
    return (int)cudaErrorNotSupported;
}

}  // namespace nsem_mx
