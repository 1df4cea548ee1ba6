/*
 * Precision form of the dGSEM Euler stage: FP32 bulk arithmetic with FP64
 * where stability needs it.
 *
 * State.  The FP64 state is kept as the perturbation from the hydrostatic
 * background, u' = (rho - rho_ref, rho u, rho v, rho w, rho theta - rho_ref T0):
 * the background is subtracted once, in FP64, when the state enters this
 * form, so no FP32 operation ever cancels two numbers of size 1e5 (p) or 1
 * (rho).  The equation of state is evaluated on the perturbation,
 *     p' = p_ref ((1 + d)^gamma - 1),  d = Theta'/Theta_ref,
 * which equals P0 (rho theta R / P0)^gamma - p_ref (apps/euler/euler.cpp:211-213)
 * because p_ref = P0 (rho_ref T0 R / P0)^gamma (euler.cpp:122-123).
 *
 * Shu-Osher SSP-RK3 in increment form: with d1 = dt L(u^n),
 * d2 = (d1 + dt L(u^n + d1)) / 4, D = 2/3 (d2 + dt L(u^n + d2)),
 * u^{n+1} = u^n + D -- algebraically the stages u1 = u^n + d1,
 * u2 = 3/4 u^n + 1/4 (u1 + dt L1), u^{n+1} = 1/3 u^n + 2/3 (u2 + dt L2).
 * The increments are FP32; the accumulation u'^{n+1} = u'^n + D is FP64.
 *
 * One fused kernel per stage, one element per CTA:
 *   phase 1 (thread per node): stage state -> primitives and volume fluxes
 *            in shared memory;
 *   phase 2 (thread per face node, all six faces): Rusanov flux seen from
 *            the element, F_out = s avg(F_n) - lam (q_other - q_own), s = +-1
 *            the sign of the outward normal along the face's axis; the own
 *            side's normal flux is the volume flux of phase 1, the other
 *            side's is formed by the same code from the neighbour's stage
 *            state.  Averages and lam are sums of the two sides' values
 *            (commutative, correctly rounded) and the jump changes sign
 *            exactly, so the two elements of a face compute F_out and
 *            -F_out bit for bit: the face conserves exactly;
 *   phase 3 (thread per node): weak volume term as tensor-product line sums
 *            with Q = W^-1 D^T W, surface lift, buoyancy, RK update.
 * Geometry: axis-aligned affine elements (the rising-bubble boxes); per
 * element the metric diagonal and the six neighbours, per z-layer the
 * background.  Discretisation identical to the plain form (same Rusanov
 * speed and jump -- normal momentum component only, field.h:2928-2943 --,
 * same symmetry ghost velocity, same weak form).  Inclined and curved
 * elements (inviscid runs) take k_mixed_stage_gen: the full metric Jinv cV
 * per node, contravariant volume fluxes and per-node face normals.
 *
 * Artificial viscosity (diffusion YES, euler.cpp:189-190, 232, 250): a
 * gradient kernel per stage forms the strong-form DG gradients of U and
 * theta of the stage state (gradf<true>, field.h:3327-3360: line derivatives
 * plus the face terms (cds - own) lifted by J/w_end; zero gradient on the
 * wall ghosts) into FP32 arrays, and the stage kernel subtracts mu grad U and
 * (mu / Pr) grad theta, mu = rho nu, from the volume and face fluxes.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "nsem_mixed_kern.cuh"

using namespace nsem_mx;

namespace {

/* ------------------------------------------------------------------------
 * Non-conforming (2:1) faces in the precision form (inviscid, axis-aligned
 * elements): the plain form's mortar treatment (field.h:2019-2248) in FP32 on
 * the perturbation state.  Per stage, before the stage kernel:
 *   k_mx_mortar_flux  per mortar slot: the fine node's stage state and the
 *       coarse side's face quantities interpolated from the coarse face's nodes
 *       with psiRef (|U|, c, rho U, rho', the momentum flux tensor, the theta
 *       flux, Theta'; rho' and Theta' corrected by the interpolated minus the
 *       fine node's background, so that their jumps are those of the full
 *       fields), the Rusanov flux vectors and the fine side's F.n;
 *   k_mx_mortar_proj  per mortar slot: the sub-face's flux vectors projected
 *       onto the slot's coarse node with psiCor, dotted with its normal;
 *   k_mx_mortar_fill  per node of an element face on a mortar: the sum of its
 *       entries (fine: one, coarse: one per sub-face), scaled by sign / (cV
 *       J_d / w_end) into the outward value the stage kernel lifts.
 * ------------------------------------------------------------------------ */
struct MortarMxArgs {
    const int32_t* mi;     /* [MX_FIELDS][n_ms] */
    const float* mf;       /* [8][n_ms] */
    const float* psiR;     /* [6][MAXN^2] */
    const float* psiC;     /* [6][MAXN^2] */
    float* F;              /* [15][n_ms] */
    float* d;              /* [5][n_ms] */
    float* dC;             /* [5][n_ms] */
    const int32_t* ent;    /* [n_mf][nfmax][4] */
    const float* coef;     /* [n_mf][nfmax][4] */
    float* MF;             /* [n_mf][9][nfmax]: outward values (0-4), gradient terms (5-8) */
    int rows;              /* MF_ROWS or MF_ROWS_GEN */
    float* gF;             /* viscous: [4][n_ms] */
    float* gC;             /* viscous: [4][n_ms] */
    const int32_t* node;   /* viscous: [n_mf][nfmax] */
    const float* gs;       /* viscous: [n_mf][nfmax][4] */
    int64_t n_ms, n_mf;
    int nfmax, np;
};

/* stage state and primitives of one node (element-blocked layout) */
template <bool HAS_DIN>
__device__ __forceinline__ Pt mx_node(const StageArgs& a, int np, int64_t node, float* x) {
    const int64_t e = node / np;
    const int l = (int)(node - e * np);
    const float* s = a.S + e * 5 * np + l;
#pragma unroll
    for (int v = 0; v < 5; v++) x[v] = __ldg(s + v * np);
    if constexpr (HAS_DIN) {
        const float* d = a.Din + e * 5 * np + l;
#pragma unroll
        for (int v = 0; v < 5; v++) x[v] = __fadd_rn(x[v], __ldg(d + v * np));
    }
    const float* bg = a.bg + (int64_t)__ldg(a.layer + e) * 4 * np + l;
    float b[4];
#pragma unroll
    for (int c = 0; c < 4; c++) b[c] = __ldg(bg + c * np);
    return pointwise(x, b, a.eos, a.gamma, a.gR);
}

/* the node's gradients (viscous runs) */
__device__ __forceinline__ void mx_grad(const StageArgs& a, int np, int64_t node, float* g) {
    const int64_t e = node / np;
    const float* gr = a.G + e * 12 * np + (node - e * np);
#pragma unroll
    for (int c = 0; c < 12; c++) g[c] = __ldg(gr + c * np);
}

template <bool HAS_DIN, bool VISC>
__global__ void __launch_bounds__(128) k_mx_mortar_flux(StageArgs a, MortarMxArgs m) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    auto fld = [&](int f) { return __ldg(m.mi + (int64_t)f * m.n_ms + ms); };
    /* the fine side: its own node */
    float xf[5];
    const Pt pf = mx_node<HAS_DIN>(a, m.np, fld(MX_FINE), xf);
    /* the coarse side: quantities interpolated over the coarse face's nodes
     * (coarse index along a outer, along b inner) */
    float q[19];
#pragma unroll
    for (int c = 0; c < 19; c++) q[c] = 0.0f;
    const int base = fld(MX_BASE), sa = fld(MX_SA), sb = fld(MX_SB), Na = fld(MX_NA),
              Nb = fld(MX_NB), ia = fld(MX_IA), ib = fld(MX_IB);
    const float* Pa = m.psiR + fld(MX_TA) * MAXN * MAXN;
    const float* Pb = m.psiR + fld(MX_TB) * MAXN * MAXN;
    for (int na = 0; na < Na; na++)
        for (int nb = 0; nb < Nb; nb++) {
            float x[5];
            const int64_t cn = (int64_t)base + na * sa + nb * sb;
            const Pt p = mx_node<HAS_DIN>(a, m.np, cn, x);
            const float w = __ldg(Pa + na * Na + ia) * __ldg(Pb + nb * Nb + ib);
            float g[12], mu = 0.0f, mt = 0.0f;
            if constexpr (VISC) {
                mx_grad(a, m.np, cn, g);
                mu = p.rho * a.nu;
                mt = p.rho * a.nu_pr;
            }
            q[0] = fmaf(w, p.umag, q[0]);
            q[1] = fmaf(w, p.c, q[1]);
#pragma unroll
            for (int c = 0; c < 3; c++) q[2 + c] = fmaf(w, x[1 + c], q[2 + c]);
            q[5] = fmaf(w, x[0], q[5]);
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    float fl = fmaf(x[1 + r], p.u[c], r == c ? p.pp : 0.0f);
                    if constexpr (VISC) fl = fmaf(-mu, g[tidx(r, c)], fl);
                    q[6 + tidx(r, c)] = fmaf(w, fl, q[6 + tidx(r, c)]);
                }
#pragma unroll
            for (int c = 0; c < 3; c++) {
                float fl = x[1 + c] * p.th;
                if constexpr (VISC) fl = fmaf(-mt, g[9 + c], fl);
                q[15 + c] = fmaf(w, fl, q[15 + c]);
            }
            q[18] = fmaf(w, x[4], q[18]);
        }
    const float* g = m.mf + ms;
    const float n[3] = {__ldg(g), __ldg(g + m.n_ms), __ldg(g + 2 * m.n_ms)};
    const float en[3] = {__ldg(g + 3 * m.n_ms), __ldg(g + 4 * m.n_ms), __ldg(g + 5 * m.n_ms)};
    q[5] += __ldg(g + 6 * m.n_ms);
    q[18] += __ldg(g + 7 * m.n_ms);
    /* the fine side's face quantities, in the same layout */
    float f[19];
    f[0] = pf.umag;
    f[1] = pf.c;
#pragma unroll
    for (int c = 0; c < 3; c++) f[2 + c] = xf[1 + c];
    f[5] = xf[0];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) f[6 + tidx(r, c)] = fmaf(xf[1 + r], pf.u[c], r == c ? pf.pp : 0.0f);
#pragma unroll
    for (int c = 0; c < 3; c++) f[15 + c] = xf[1 + c] * pf.th;
    f[18] = xf[4];
    if constexpr (VISC) {
        float g[12];
        mx_grad(a, m.np, fld(MX_FINE), g);
        const float mu = pf.rho * a.nu, mt = pf.rho * a.nu_pr;
#pragma unroll
        for (int c = 0; c < 9; c++) f[6 + c] = fmaf(-mu, g[c], f[6 + c]);
#pragma unroll
        for (int c = 0; c < 3; c++) f[15 + c] = fmaf(-mt, g[9 + c], f[15 + c]);
    }
    /* side 1 (FO) and side 2 (FN) of the slot; the normal points 1 -> 2 */
    const bool fine1 = fld(MX_FINE_C1) != 0;
    const float* A = fine1 ? f : q;
    const float* B = fine1 ? q : f;
    const float lam = 0.25f * ((A[0] + B[0]) + (A[1] + B[1]));
    float F[15];
    {
        const float jr = lam * (B[5] - A[5]);
#pragma unroll
        for (int c = 0; c < 3; c++) F[c] = fmaf(-en[c], jr, 0.5f * (A[2 + c] + B[2 + c]));
        const float jt = lam * (B[18] - A[18]);
#pragma unroll
        for (int c = 0; c < 3; c++) F[12 + c] = fmaf(-en[c], jt, 0.5f * (A[15 + c] + B[15 + c]));
        float dq[3];
#pragma unroll
        for (int c = 0; c < 3; c++) dq[c] = (B[2 + c] - A[2 + c]) * lam;
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int c = 0; c < 3; c++)
                F[3 + tidx(r, c)] = fmaf(-en[r], dq[c], 0.5f * (A[6 + tidx(r, c)] + B[6 + tidx(r, c)]));
    }
#pragma unroll
    for (int c = 0; c < 15; c++) m.F[c * m.n_ms + ms] = F[c];
    m.d[ms] = fmaf(F[0], n[0], fmaf(F[1], n[1], F[2] * n[2]));
#pragma unroll
    for (int r = 0; r < 3; r++)
        m.d[(1 + r) * m.n_ms + ms] =
            fmaf(F[3 + tidx(r, 0)], n[0], fmaf(F[3 + tidx(r, 1)], n[1], F[3 + tidx(r, 2)] * n[2]));
    m.d[4 * m.n_ms + ms] = fmaf(F[12], n[0], fmaf(F[13], n[1], F[14] * n[2]));
}

__global__ void __launch_bounds__(128) k_mx_mortar_proj(MortarMxArgs m) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    auto fld = [&](int f) { return __ldg(m.mi + (int64_t)f * m.n_ms + ms); };
    const int Na = fld(MX_NA), Nb = fld(MX_NB), na = fld(MX_IA), nb = fld(MX_IB),
              first = fld(MX_FIRST);
    const float* Pa = m.psiC + fld(MX_TA) * MAXN * MAXN;
    const float* Pb = m.psiC + fld(MX_TB) * MAXN * MAXN;
    float P[15];
#pragma unroll
    for (int c = 0; c < 15; c++) P[c] = 0.0f;
    for (int ja = 0; ja < Na; ja++)
        for (int jb = 0; jb < Nb; jb++) {
            const int64_t s2 = first + ja * Nb + jb;
            const float w = __ldg(Pa + ja * Na + na) * __ldg(Pb + jb * Nb + nb);
#pragma unroll
            for (int c = 0; c < 15; c++) P[c] = fmaf(w, __ldg(m.F + c * m.n_ms + s2), P[c]);
        }
    const float* g = m.mf + ms;
    const float n[3] = {__ldg(g), __ldg(g + m.n_ms), __ldg(g + 2 * m.n_ms)};
    m.dC[ms] = fmaf(P[0], n[0], fmaf(P[1], n[1], P[2] * n[2]));
#pragma unroll
    for (int r = 0; r < 3; r++)
        m.dC[(1 + r) * m.n_ms + ms] =
            fmaf(P[3 + tidx(r, 0)], n[0], fmaf(P[3 + tidx(r, 1)], n[1], P[3 + tidx(r, 2)] * n[2]));
    m.dC[4 * m.n_ms + ms] = fmaf(P[12], n[0], fmaf(P[13], n[1], P[14] * n[2]));
}

__global__ void __launch_bounds__(128) k_mx_mortar_fill(MortarMxArgs m) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= m.n_mf * m.nfmax) return;
    const int64_t f = id / m.nfmax;
    const int r = (int)(id - f * m.nfmax);
    float acc[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    for (int q = 0; q < 4; q++) {
        const int32_t en = __ldg(m.ent + id * 4 + q);
        if (en < 0) break;
        const float c = __ldg(m.coef + id * 4 + q);
        const float* src = (en & MX_COARSE) ? m.dC : m.d;
        const int64_t ms = en & (MX_COARSE - 1);
#pragma unroll
        for (int v = 0; v < 5; v++) acc[v] = fmaf(c, __ldg(src + v * m.n_ms + ms), acc[v]);
    }
#pragma unroll
    for (int v = 0; v < 5; v++) m.MF[(f * m.rows + v) * m.nfmax + r] = acc[v];
}

/* Viscous runs: the gradients' face values on mortars (the plain form's
 * k_seg_mortar_gcds / k_seg_mortar_ggather in FP32).  Per mortar slot
 * cds = (fine + interpolated coarse) / 2 of U and theta - T0; per slot its
 * sub-face's values projected onto the slot's coarse node; per node of an
 * element face on a mortar sum_entries gs (value - own), which the gradient
 * kernel lifts like a conforming face's cds - own. */
__device__ __forceinline__ float4 mx_ut(const StageArgs& a, const float* x, int np, int64_t node) {
    const int64_t e = node / np;
    const float rref = __ldg(a.bg + (int64_t)__ldg(a.layer + e) * 4 * np + (node - e * np));
    const float inv = rcp_nr(__fadd_rn(rref, x[0]));
    return make_float4(__fmul_rn(x[1], inv), __fmul_rn(x[2], inv), __fmul_rn(x[3], inv),
                       __fmul_rn(__fmaf_rn(-a.T0, x[0], x[4]), inv));
}

template <bool HAS_DIN>
__device__ __forceinline__ float4 mx_node_ut(const StageArgs& a, int np, int64_t node) {
    const int64_t e = node / np;
    const int l = (int)(node - e * np);
    float x[5];
    const float* s = a.S + e * 5 * np + l;
#pragma unroll
    for (int v = 0; v < 5; v++) x[v] = __ldg(s + v * np);
    if constexpr (HAS_DIN) {
        const float* d = a.Din + e * 5 * np + l;
#pragma unroll
        for (int v = 0; v < 5; v++) x[v] = __fadd_rn(x[v], __ldg(d + v * np));
    }
    return mx_ut(a, x, np, node);
}

template <bool HAS_DIN>
__global__ void __launch_bounds__(128) k_mx_mortar_gcds(StageArgs a, MortarMxArgs m) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    auto fld = [&](int f) { return __ldg(m.mi + (int64_t)f * m.n_ms + ms); };
    const int base = fld(MX_BASE), sa = fld(MX_SA), sb = fld(MX_SB), Na = fld(MX_NA),
              Nb = fld(MX_NB), ia = fld(MX_IA), ib = fld(MX_IB);
    const float* Pa = m.psiR + fld(MX_TA) * MAXN * MAXN;
    const float* Pb = m.psiR + fld(MX_TB) * MAXN * MAXN;
    float4 I = make_float4(0, 0, 0, 0);
    for (int na = 0; na < Na; na++)
        for (int nb = 0; nb < Nb; nb++) {
            const float4 v = mx_node_ut<HAS_DIN>(a, m.np, (int64_t)base + na * sa + nb * sb);
            const float w = __ldg(Pa + na * Na + ia) * __ldg(Pb + nb * Nb + ib);
            I.x = fmaf(w, v.x, I.x); I.y = fmaf(w, v.y, I.y);
            I.z = fmaf(w, v.z, I.z); I.w = fmaf(w, v.w, I.w);
        }
    const float4 f = mx_node_ut<HAS_DIN>(a, m.np, fld(MX_FINE));
    m.gF[ms] = 0.5f * f.x + 0.5f * I.x;
    m.gF[m.n_ms + ms] = 0.5f * f.y + 0.5f * I.y;
    m.gF[2 * m.n_ms + ms] = 0.5f * f.z + 0.5f * I.z;
    m.gF[3 * m.n_ms + ms] = 0.5f * f.w + 0.5f * I.w;
}

__global__ void __launch_bounds__(128) k_mx_mortar_ggather(MortarMxArgs m) {
    const int64_t ms = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ms >= m.n_ms) return;
    auto fld = [&](int f) { return __ldg(m.mi + (int64_t)f * m.n_ms + ms); };
    const int Na = fld(MX_NA), Nb = fld(MX_NB), na = fld(MX_IA), nb = fld(MX_IB),
              first = fld(MX_FIRST);
    const float* Pa = m.psiC + fld(MX_TA) * MAXN * MAXN;
    const float* Pb = m.psiC + fld(MX_TB) * MAXN * MAXN;
    float o[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int ja = 0; ja < Na; ja++)
        for (int jb = 0; jb < Nb; jb++) {
            const int64_t s2 = first + ja * Nb + jb;
            const float w = __ldg(Pa + ja * Na + na) * __ldg(Pb + jb * Nb + nb);
#pragma unroll
            for (int c = 0; c < 4; c++) o[c] = fmaf(w, __ldg(m.gF + c * m.n_ms + s2), o[c]);
        }
#pragma unroll
    for (int c = 0; c < 4; c++) m.gC[c * m.n_ms + ms] = o[c];
}

template <bool HAS_DIN, bool GEN>
__global__ void __launch_bounds__(128) k_mx_mortar_gfill(StageArgs a, MortarMxArgs m) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= m.n_mf * m.nfmax) return;
    const int64_t f = id / m.nfmax;
    const int r = (int)(id - f * m.nfmax);
    const int32_t node = __ldg(m.node + id);
    constexpr int NA = GEN ? 12 : 4;
    float acc[NA];
#pragma unroll
    for (int c = 0; c < NA; c++) acc[c] = 0.0f;
    if (node >= 0) {
        const float4 o = mx_node_ut<HAS_DIN>(a, m.np, node);
        const float own[4] = {o.x, o.y, o.z, o.w};
        for (int q = 0; q < 4; q++) {
            const int32_t en = __ldg(m.ent + id * 4 + q);
            if (en < 0) break;
            const float w = __ldg(m.gs + id * 4 + q);
            const float* src = (en & MX_COARSE) ? m.gC : m.gF;
            const int64_t ms = en & (MX_COARSE - 1);
            float dv[4];
#pragma unroll
            for (int c = 0; c < 4; c++) dv[c] = __ldg(src + c * m.n_ms + ms) - own[c];
            if constexpr (GEN) {
                /* w the outward sign; the slot's weighted normal per row */
#pragma unroll
                for (int rr = 0; rr < 3; rr++) {
                    const float n = w * __ldg(m.mf + rr * m.n_ms + ms);
#pragma unroll
                    for (int c = 0; c < 4; c++) acc[rr * 4 + c] = fmaf(n, dv[c], acc[rr * 4 + c]);
                }
            } else {
#pragma unroll
                for (int c = 0; c < 4; c++) acc[c] = fmaf(w, dv[c], acc[c]);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < NA; c++) m.MF[(f * m.rows + 5 + c) * m.nfmax + r] = acc[c];
}

/* full (FP64, node order, SoA) <-> perturbation state (element-blocked):
 * u' = u - (rho_ref, 0, 0, 0, rho_ref T0), FP32 shadow of u' */
struct Ptr5 {
    double* p[5];
};

template <int NP>
__global__ void k_to_pert(Ptr5 full, double* U, float* S, const double* rho_ref, double T0,
                          int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i / NP;
        const int64_t o = e * 5 * NP + (i - e * NP);
        /* explicitly rounded: rho_ref T0 must round as on the host (no FMA) */
        const double rr = rho_ref[i];
        const double tr = __dmul_rn(rr, T0);
        const double v[5] = {__dsub_rn(full.p[0][i], rr), full.p[1][i], full.p[2][i],
                             full.p[3][i], __dsub_rn(full.p[4][i], tr)};
#pragma unroll
        for (int c = 0; c < 5; c++) {
            U[o + c * NP] = v[c];
            S[o + c * NP] = d2f_rn(v[c]);
        }
    }
}

template <int NP>
__global__ void k_from_pert(const double* U, Ptr5 full, const double* rho_ref, double T0,
                            int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i / NP;
        const int64_t o = e * 5 * NP + (i - e * NP);
        const double rr = rho_ref[i];
        const double tr = __dmul_rn(rr, T0);
        full.p[0][i] = __dadd_rn(U[o], rr);
        full.p[1][i] = U[o + NP];
        full.p[2][i] = U[o + 2 * NP];
        full.p[3][i] = U[o + 3 * NP];
        full.p[4][i] = __dadd_rn(U[o + 4 * NP], tr);
    }
}

/* the host boundary's layout (rho, rho U as AoS xyz, rho theta; node order)
 * <-> perturbation state, in one pass each way (no conserved SoA copy) */
template <int NP>
__global__ void k_host_to_pert(const double* rho, const double* mom, const double* rt, double* U,
                               float* S, const double* rho_ref, double T0, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i / NP;
        const int64_t o = e * 5 * NP + (i - e * NP);
        const double rr = rho_ref[i];
        const double tr = __dmul_rn(rr, T0);
        const double v[5] = {__dsub_rn(rho[i], rr), mom[3 * i], mom[3 * i + 1], mom[3 * i + 2],
                             __dsub_rn(rt[i], tr)};
#pragma unroll
        for (int c = 0; c < 5; c++) {
            U[o + c * NP] = v[c];
            S[o + c * NP] = d2f_rn(v[c]);
        }
    }
}

template <int NP>
__global__ void k_pert_to_host(const double* U, double* rho, double* mom, double* rt,
                               const double* rho_ref, double T0, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i / NP;
        const int64_t o = e * 5 * NP + (i - e * NP);
        const double rr = rho_ref[i];
        const double tr = __dmul_rn(rr, T0);
        rho[i] = __dadd_rn(U[o], rr);
        mom[3 * i] = U[o + NP];
        mom[3 * i + 1] = U[o + 2 * NP];
        mom[3 * i + 2] = U[o + 3 * NP];
        rt[i] = __dadd_rn(U[o + 4 * NP], tr);
    }
}

/* launch configuration of the stage kernels: tensor-core line sums (order 7),
 * persistent CTAs and their grid per stage (resident CTAs x SMs) */

}  // namespace

bool nsem_mixed_supported(int nx, int ny, int nz) {
#define NSEM_SUP(A, B, C) if (nx == A && ny == B && nz == C) return true;
    NSEM_MIXED_DIMS(NSEM_SUP)
#undef NSEM_SUP
    return false;
}

namespace {

int prepare(int nx, int ny, int nz, LaunchCfg* c) {
    const int e = prepare_aligned(nx, ny, nz, c);
    return e ? e : prepare_general(nx, ny, nz);
}

int dispatch_stage(int nx, int ny, int nz, const StageArgs& a, int stage, cudaStream_t st,
                   const LaunchCfg& c) {
    if (c.gen) return launch_stage_general(nx, ny, nz, a, stage, st, c.visc);
    return launch_stage_aligned(nx, ny, nz, a, stage, st, c);
}

int dispatch_grad(int nx, int ny, int nz, const StageArgs& a, int stage, cudaStream_t st,
                  const LaunchCfg& c) {
    if (c.gen) return launch_grad_general(nx, ny, nz, a, stage, st);
    return launch_grad_aligned(nx, ny, nz, a, stage, st);
}

int grid_for(int64_t n) {
    int64_t g = (n + 255) / 256;
    if (g > 152 * 8) g = 152 * 8;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

/* ------------------------------------------------------------------ setup */

nsem_status nsem_mixed_setup(const NsemDev& dev, const nsem_mesh_desc* m, NsemMixedBuf* mb,
                             std::vector<void*>* allocs, std::string& err) {
    mb->ready = false;
    const int NX = m->npx, NY = m->npy, NZ = m->npz;
    if (!nsem_mixed_supported(NX, NY, NZ)) {
        err = "precision form built for N+1 = 4, 5, 8 per direction (and 2D N+1 = 4, 5)";
        return NSEM_UNSUPPORTED;
    }
    const int64_t NP = (int64_t)NX * NY * NZ;
    const int64_t ne = m->n_elem;
    const int64_t n_int = ne * NP;
    const int64_t n_all = (int64_t)m->n_cells * NP;
    const int npd[3] = {NX, NY, NZ};

    /* per-element diagonal metric of axis-aligned affine elements; any other
     * element (inclined, curved) selects the general-geometry kernels */
    std::vector<float> J(3 * ne);
    bool gen = false;
    for (int64_t e = 0; e < ne && !gen; e++) {
        const double* J0 = m->Jinv + 9 * (e * NP);
        const double diag0[3] = {J0[0], J0[1], J0[2]};
        const double scale = std::fabs(diag0[0]) + std::fabs(diag0[1]) + std::fabs(diag0[2]);
        for (int64_t a = 0; a < NP && !gen; a++) {
            const double* Ja = m->Jinv + 9 * (e * NP + a);
            for (int c = 0; c < 9; c++) {
                const double ref = (c < 3) ? diag0[c] : 0.0;
                if (std::fabs(Ja[c] - ref) > 1e-9 * scale) gen = true;
            }
        }
        for (int d = 0; d < 3; d++) J[d * ne + e] = (float)diag0[d];
    }
    /* non-conforming (2:1) faces: the fine sub-faces' ids */
    std::vector<int8_t> on_mortar(m->n_mortar > 0 ? m->n_face : 0, 0);
    if (m->n_mortar > 0) {
        for (int32_t q = 0; q < m->n_mortar; q++) on_mortar[m->mortar[4 * (size_t)q]] = 1;
    }
    /* general geometry: Jinv cV and 1/cV per node, outward weighted normals
     * per element face slot */
    const int nfx = NY * NZ, nfy = NX * NZ, nfz = NX * NY;
    const int off_y = 2 * nfx, off_z = 2 * nfx + (NY > 1 ? 2 * nfy : 0);
    const int nfs = off_z + 2 * nfz;
    std::vector<float> Jg, Fn;
    if (gen) {
        Jg.assign((size_t)ne * 10 * NP, 0.0f);
        Fn.assign((size_t)ne * 3 * nfs, 0.0f);
        for (int64_t e = 0; e < ne; e++)
            for (int64_t a = 0; a < NP; a++) {
                const int64_t i = e * NP + a;
                for (int c = 0; c < 9; c++)
                    Jg[(e * 10 + c) * NP + a] = (float)(m->Jinv[9 * i + c] * m->cV[i]);
                Jg[(e * 10 + 9) * NP + a] = (float)(1.0 / m->cV[i]);
            }
    }

    /* neighbours from the face slots: element face lists + FO/FN */
    std::vector<int32_t> nbr(6 * ne, -1);
    auto local = [&](int64_t node) { return node % NP; };
    for (int64_t e = 0; e < ne; e++) {
        for (uint32_t f = m->face_idx0[e]; f < m->face_idx1[e]; f++) {
            const int64_t fid = m->all_faces[f];
            if (m->n_mortar > 0 && on_mortar[fid]) continue;   /* below */
            /* find the first used slot of this face */
            int64_t k = -1;
            for (int q = 0; q < m->npf; q++) {
                const int64_t kk = fid * m->npf + q;
                if (m->FO[kk] < (uint64_t)n_all && m->FN[kk] < (uint64_t)n_all) { k = kk; break; }
            }
            if (k < 0) continue;
            const uint32_t o = m->FO[k], n = m->FN[k];
            const bool own = (o / NP) == (uint64_t)e;
            const int64_t mine = own ? o : n;
            const int64_t other = own ? n : o;
            (void)mine;
            /* which face of e: the local index direction held at one end by
             * every node of the face */
            int dir = -1, side = 0;
            for (int d = 0; d < 3 && dir < 0; d++) {
                if (npd[d] == 1) continue;
                for (int sd = 0; sd < 2 && dir < 0; sd++) {
                    const int want = sd ? npd[d] - 1 : 0;
                    bool all = true;
                    for (int q = 0; q < m->npf && all; q++) {
                        const int64_t kk = fid * m->npf + q;
                        if (m->FO[kk] >= (uint64_t)n_all || m->FN[kk] >= (uint64_t)n_all) continue;
                        const int l2 = (int)local(own ? m->FO[kk] : m->FN[kk]);
                        const int c2[3] = {l2 / (NY * NZ), (l2 / NZ) % NY, l2 % NZ};
                        all = c2[d] == want;
                    }
                    if (all) { dir = d; side = sd; }
                }
            }
            if (dir < 0) {
                err = "precision form needs faces on the element's local index planes";
                return NSEM_UNSUPPORTED;
            }
            const int32_t nb = (other < (int64_t)n_int) ? (int32_t)(other / NP) : -1;
            nbr[(2 * dir + side) * ne + e] = nb;
            /* verify the structured slot mapping on every used slot */
            for (int q = 0; q < m->npf; q++) {
                const int64_t kk = fid * m->npf + q;
                if (m->FO[kk] >= (uint64_t)n_all || m->FN[kk] >= (uint64_t)n_all) continue;
                const uint32_t o2 = m->FO[kk], n2 = m->FN[kk];
                const int64_t mine2 = own ? o2 : n2, other2 = own ? n2 : o2;
                if (mine2 / NP != e) { err = "face slot outside its element"; return NSEM_UNSUPPORTED; }
                const int l2 = (int)local(mine2);
                int c2[3] = {l2 / (NY * NZ), (l2 / NZ) % NY, l2 % NZ};
                if (c2[dir] != (side ? npd[dir] - 1 : 0)) {
                    err = "precision form needs faces on the element's local index planes";
                    return NSEM_UNSUPPORTED;
                }
                if (gen) {
                    const int t = dir == 0 ? side * nfx + c2[1] * NZ + c2[2]
                                : dir == 1 ? off_y + side * nfy + c2[0] * NZ + c2[2]
                                           : off_z + side * nfz + c2[0] * NY + c2[1];
                    const double sg = own ? 1.0 : -1.0;
                    for (int c = 0; c < 3; c++)
                        Fn[(e * 3 + c) * nfs + t] = (float)(sg * m->fN[3 * kk + c]);
                }
                if (nb >= 0) {
                    if (other2 / NP != nb) { err = "face with two neighbours"; return NSEM_UNSUPPORTED; }
                    int c3[3] = {c2[0], c2[1], c2[2]};
                    c3[dir] = side ? 0 : npd[dir] - 1;
                    const int lo = (c3[0] * NY + c3[1]) * NZ + c3[2];
                    if ((int)local(other2) != lo) {
                        err = "precision form needs conforming, aligned face nodes";
                        return NSEM_UNSUPPORTED;
                    }
                } else if (m->bc_U[kk] != 2) {
                    err = "precision form supports SYMMETRY walls only";
                    return NSEM_UNSUPPORTED;
                }
            }
        }
    }

    /* background per layer: elements with identical node backgrounds share one */
    std::vector<double> rref_h(n_int), pref_h(n_int);
    if (cudaMemcpy(rref_h.data(), dev.rho_ref, n_int * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(pref_h.data(), dev.p_ref, n_int * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
        err = "precision form: background copy failed";
        return NSEM_CUDA_ERROR;
    }
    std::vector<int32_t> layer(ne);
    std::vector<float> bg;
    std::map<std::vector<float>, int32_t> seen;
    for (int64_t e = 0; e < ne; e++) {
        std::vector<float> key(4 * NP);
        for (int64_t a = 0; a < NP; a++) {
            const double rr = rref_h[e * NP + a];
            const double tr = rr * dev.T0;
            key[a] = (float)rr;
            key[NP + a] = (float)tr;
            key[2 * NP + a] = (float)(1.0 / tr);
            key[3 * NP + a] = (float)pref_h[e * NP + a];
        }
        auto it = seen.find(key);
        if (it == seen.end()) {
            int32_t id = (int32_t)seen.size();
            seen.emplace(key, id);
            bg.insert(bg.end(), key.begin(), key.end());
            layer[e] = id;
        } else {
            layer[e] = it->second;
        }
    }

    /* quadrature weights per direction from the node mass weights of the
     * first element (cV = V w_i w_j w_k / 8, dg.cpp:315-318), normalised to
     * sum 2; tables Q_d[a][m] = D_d[m][a] w_m / w_a and lift 1/w_end */
    std::vector<double> wdir[3];
    for (int d = 0; d < 3; d++) {
        const int n = npd[d];
        double sum = 0;
        for (int q = 0; q < n; q++) {
            int c[3] = {0, 0, 0};
            c[d] = q;
            const double v = m->cV[(c[0] * NY + c[1]) * NZ + c[2]];
            wdir[d].push_back(v);
            sum += v;
        }
        for (int q = 0; q < n; q++) wdir[d][q] = 2.0 * wdir[d][q] / sum;
    }
    std::vector<float> qtab(QTAB, 0.0f), dtab(QTAB, 0.0f);
    for (int d = 0; d < 3; d++) {
        const int n = npd[d];
        const std::vector<double>& w = wdir[d];
        for (int aa = 0; aa < n; aa++)
            for (int mm = 0; mm < n; mm++) {
                /* general geometry: the plain weak-form table l_a'(x_m), the
                 * weights sit in Jinv cV and 1/cV */
                qtab[d * MAXN * QS + aa * QS + mm] =
                    gen ? (float)m->dpsi[d][mm * n + aa] : (float)(m->dpsi[d][mm * n + aa] * w[mm] / w[aa]);
                /* D_d[a][m] = l_m'(x_a) = dpsi[a * n + m] for the gradient kernel */
                dtab[d * MAXN * QS + aa * QS + mm] = (float)m->dpsi[d][aa * n + mm];
            }
        mb->lift[d] = (float)(1.0 / w[0]);
        for (int aa = 0; aa < n && aa < 8; aa++)
            for (int mm = 0; mm < n && mm < 8; mm++) {
                mb->qc[d][aa][mm] = qtab[d * MAXN * QS + aa * QS + mm];
                mb->dc[d][aa][mm] = dtab[d * MAXN * QS + aa * QS + mm];
            }
    }
    /* order 7: the tensor-core line sums' B fragments, Q_d^T split into TF32
     * high and low parts as cvt.rna.tf32 does (round to nearest, ties away
     * from zero, in the magnitude: + 2^12 and the low 13 bits cleared) */
    if (NX == 8 && NY == 8 && NZ == 8 && !gen) {
        auto rna = [](float x) {
            uint32_t b;
            std::memcpy(&b, &x, 4);
            b = (b + 0x1000u) & 0xffffe000u;
            float r;
            std::memcpy(&r, &b, 4);
            return r;
        };
        std::vector<float> tcb(TC_QTAB, 0.0f);
        for (int d = 0; d < 3; d++)
            for (int k = 0; k < 8; k++)
                for (int n = 0; n < 8; n++) {
                    const float q = qtab[d * MAXN * QS + n * QS + k];   /* B[k][n] = Q[n][k] */
                    const float hi = rna(q);
                    tcb[d * 128 + k * 8 + n] = hi;
                    tcb[d * 128 + 64 + k * 8 + n] = rna(q - hi);
                }
        qtab.insert(qtab.end(), tcb.begin(), tcb.end());
    }


    /* non-conforming faces: per mortar slot (entries in order, (ia, ib)
     * row-major, the numbering of the plain form) the fine node, the coarse
     * face and the interpolation indices, normals and background corrections;
     * per element face on a mortar its node entries */
    std::vector<int32_t> mxi[MX_FIELDS];
    std::vector<float> mxf[8];
    std::vector<int32_t> ment, mnode, mface;
    std::vector<float> mcoef, mgs, macoef;
    std::map<int64_t, int32_t> mf_of;
    const int nfmax = std::max(nfx, std::max(nfy, nfz));
    if (m->n_mortar > 0) {
        const int64_t stride[3] = {(int64_t)NY * NZ, NZ, 1};
        auto loc = [&](int64_t node, int c[3]) {
            const int l = (int)(node % NP);
            c[0] = l / (NY * NZ); c[1] = (l / NZ) % NY; c[2] = l % NZ;
        };
        auto in_face = [&](int dir, const int c[3]) {
            return dir == 0 ? c[1] * NZ + c[2] : dir == 1 ? c[0] * NZ + c[2] : c[0] * NY + c[1];
        };
        auto mf_index = [&](int64_t e, int face) {
            const int64_t key = e * 6 + face;
            auto it = mf_of.find(key);
            if (it != mf_of.end()) return it->second;
            const int32_t id = (int32_t)mf_of.size();
            mf_of.emplace(key, id);
            mface.push_back(face);
            nbr[(int64_t)face * ne + e] = -2 - id;
            ment.resize((size_t)(id + 1) * nfmax * 4, -1);
            mcoef.resize((size_t)(id + 1) * nfmax * 4, 0.0f);
            macoef.resize((size_t)(id + 1) * nfmax * 4, 0.0f);
            mgs.resize((size_t)(id + 1) * nfmax * 4, 0.0f);
            mnode.resize((size_t)(id + 1) * nfmax, -1);
            return id;
        };
        /* the lift coefficient of a face node of direction dir in the stage
         * kernel: J_d / w_end (axis-aligned elements, formed as the kernel
         * forms it) or 1 / cV (general geometry) */
        auto liftc = [&](int64_t node, int dir) {
            if (gen) return 1.0 / m->cV[node];
            return (double)(J[(int64_t)dir * ne + node / NP] * mb->lift[dir]);
        };
        /* an entry of a face node: the mortar slot, the flux coefficient, the
         * gradient weight and the adjoint weight (minus the lift coefficient
         * times the flux coefficient) */
        auto add = [&](int32_t mf, int r, int64_t node, int32_t code, double c, double g,
                       int dir) -> bool {
            mnode[(size_t)mf * nfmax + r] = (int32_t)node;
            for (int q = 0; q < 4; q++) {
                const size_t at = ((size_t)mf * nfmax + r) * 4 + q;
                if (ment[at] < 0) {
                    ment[at] = code; mcoef[at] = (float)c; mgs[at] = (float)g;
                    macoef[at] = (float)(-liftc(node, dir) * c);
                    return true;
                }
            }
            return false;
        };
        /* 1 / (cV J_d / w_end), with J_d / w_end as the stage kernel forms it */
        auto scale = [&](int64_t node, int dir) {
            const float coef = J[(int64_t)dir * ne + node / NP] * mb->lift[dir];
            return 1.0 / (m->cV[node] * (double)coef);
        };
        for (int32_t q = 0; q < m->n_mortar; q++) {
            const uint32_t* r = m->mortar + 4 * (size_t)q;
            const int64_t fi = r[0];
            const int fm = (int)r[1], fid = (int)r[2];
            int aa, bb, fix;
            if (fid <= 1) { aa = 0; bb = 1; fix = 2; }
            else if (fid <= 3) { aa = 0; bb = 2; fix = 1; }
            else { aa = 1; bb = 2; fix = 0; }
            const int Na = npd[aa], Nb = npd[bb];
            const int64_t k0 = fi * m->npf;
            const int64_t cnode0 = fm == 1 ? m->FN[k0] : m->FO[k0];
            const int64_t fnode0 = fm == 1 ? m->FO[k0] : m->FN[k0];
            if (cnode0 >= n_int || fnode0 >= n_int) {
                err = "precision form: mortar face on a boundary";
                return NSEM_UNSUPPORTED;
            }
            const int64_t cell_c = cnode0 / NP, cell_f = fnode0 / NP;
            const int64_t base = cell_c * NP + ((fid & 1) ? npd[fix] - 1 : 0) * stride[fix];
            /* the fine element's face: the index plane every fine node lies on */
            int dir_f = -1, side_f = 0;
            for (int d = 0; d < 3 && dir_f < 0; d++) {
                if (npd[d] == 1) continue;
                for (int sd = 0; sd < 2 && dir_f < 0; sd++) {
                    bool all = true;
                    for (int w = 0; w < Na * Nb && all; w++) {
                        const int64_t node = fm == 1 ? m->FO[k0 + w] : m->FN[k0 + w];
                        int c[3];
                        loc(node, c);
                        all = node / NP == cell_f && c[d] == (sd ? npd[d] - 1 : 0);
                    }
                    if (all) { dir_f = d; side_f = sd; }
                }
            }
            if (dir_f < 0) {
                err = "precision form: mortar face off the fine element's index planes";
                return NSEM_UNSUPPORTED;
            }
            const int32_t mf_f = mf_index(cell_f, 2 * dir_f + side_f);
            const int32_t mf_c = mf_index(cell_c, 2 * fix + (fid & 1));
            const int32_t first = (int32_t)mxi[0].size();
            const int ta = 2 * aa + (int)(r[3] & 1), tb = 2 * bb + (int)((r[3] >> 1) & 1);
            const double* Pa = m->psi_ref[ta];
            const double* Pb = m->psi_ref[tb];
            for (int ia = 0; ia < Na; ia++)
                for (int ib = 0; ib < Nb; ib++) {
                    const int64_t k = k0 + (int64_t)ia * Nb + ib;
                    const int64_t fnode = fm == 1 ? m->FO[k] : m->FN[k];
                    const int64_t cnode = fm == 1 ? m->FN[k] : m->FO[k];
                    /* the slot's coarse node is node (ia, ib) of the coarse
                     * face: the projection lands there and the adjoint's
                     * interpolation transpose starts from it */
                    if (fnode / NP != cell_f || cnode / NP != cell_c || m->fI[k] != 0.5 ||
                        cnode != base + ia * stride[aa] + ib * stride[bb]) {
                        err = "precision form: unexpected mortar slot layout";
                        return NSEM_UNSUPPORTED;
                    }
                    const int32_t ms = (int32_t)mxi[0].size();
                    const int32_t fld[MX_FIELDS] = {(int32_t)fnode, fm == 1 ? 1 : 0, (int32_t)base,
                                                    (int32_t)stride[aa], (int32_t)stride[bb], Na, Nb,
                                                    ia, ib, first, ta, tb};
                    for (int c = 0; c < MX_FIELDS; c++) mxi[c].push_back(fld[c]);
                    const double* v = m->fN + 3 * k;
                    const double mg = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                    for (int c = 0; c < 3; c++) {
                        mxf[c].push_back((float)v[c]);
                        mxf[3 + c].push_back((float)(v[c] / mg));
                    }
                    /* interpolated minus own background (rho_ref, Theta_ref) */
                    double ir = 0.0;
                    for (int na = 0; na < Na; na++)
                        for (int nb = 0; nb < Nb; nb++)
                            ir += rref_h[base + na * stride[aa] + nb * stride[bb]] * Pa[na * Na + ia] *
                                  Pb[nb * Nb + ib];
                    mxf[6].push_back((float)(ir - rref_h[fnode]));
                    mxf[7].push_back((float)((ir - rref_h[fnode]) * dev.T0));
                    int c[3];
                    loc(fnode, c);
                    /* general geometry: the stage kernel lifts F.n itself (1/cV
                     * in its update) and the gradient kernel the normal-weighted
                     * terms, so both weights are the outward sign only */
                    const double sf = gen ? 1.0 : scale(fnode, dir_f), sc = gen ? 1.0 : scale(cnode, fix);
                    const double gf = gen ? (fm == 1 ? 1.0 : -1.0) : mg * sf;
                    const double gc = gen ? (fm == 2 ? 1.0 : -1.0) : mg * sc;
                    bool ok = add(mf_f, in_face(dir_f, c), fnode, ms, (fm == 1 ? 1.0 : -1.0) * sf, gf,
                                  dir_f);
                    loc(cnode, c);
                    ok = ok && add(mf_c, in_face(fix, c), cnode, ms | MX_COARSE,
                                   (fm == 2 ? 1.0 : -1.0) * sc, gc, fix);
                    if (!ok) {
                        err = "precision form: more than four mortar entries on a face node";
                        return NSEM_UNSUPPORTED;
                    }
                }
        }
    }

    auto up = [&](auto** ptr, const auto& vec) -> bool {
        using T = typename std::remove_reference<decltype(vec[0])>::type;
        size_t bytes = vec.size() * sizeof(T);
        if (cudaMalloc((void**)ptr, bytes ? bytes : 1) != cudaSuccess) return false;
        allocs->push_back((void*)*ptr);
        return cudaMemcpy(*ptr, vec.data(), bytes, cudaMemcpyHostToDevice) == cudaSuccess;
    };
    if (!up(&mb->nbr, nbr) || !up(&mb->J, J) || !up(&mb->layer, layer) || !up(&mb->bg, bg) ||
        !up(&mb->Qg, qtab) || !up(&mb->Dg, dtab) || (gen && (!up(&mb->Jg, Jg) || !up(&mb->Fn, Fn)))) {
        err = "precision form: device allocation failed";
        return NSEM_NO_MEMORY;
    }
    mb->gen = gen;
    mb->n_ms = (int64_t)mxi[0].size();
    mb->n_mf = (int64_t)mf_of.size();
    mb->nfmax = nfmax;
    if (mb->n_ms > 0) {
        std::vector<int32_t> mi;
        for (int c = 0; c < MX_FIELDS; c++) mi.insert(mi.end(), mxi[c].begin(), mxi[c].end());
        std::vector<float> mf, psi(2 * 6 * MAXN * MAXN, 0.0f);
        for (int c = 0; c < 8; c++) mf.insert(mf.end(), mxf[c].begin(), mxf[c].end());
        for (int t = 0; t < 6; t++) {
            const int n = npd[t / 2];
            for (int q = 0; q < n * n; q++) {
                psi[t * MAXN * MAXN + q] = (float)m->psi_ref[t][q];
                psi[(6 + t) * MAXN * MAXN + q] = (float)m->psi_cor[t][q];
            }
        }
        const std::vector<float> scratch15(15 * mb->n_ms, 0.0f), scratch5(5 * mb->n_ms, 0.0f),
            scratch4(4 * mb->n_ms, 0.0f),
            mfv((size_t)(gen ? MF_ROWS_GEN : MF_ROWS) * mb->n_mf * nfmax, 0.0f);
        if (!up(&mb->mx_i, mi) || !up(&mb->mx_f, mf) || !up(&mb->mx_psi, psi) ||
            !up(&mb->mx_F, scratch15) || !up(&mb->mx_d, scratch5) || !up(&mb->mx_dC, scratch5) ||
            !up(&mb->mf_ent, ment) || !up(&mb->mf_coef, mcoef) || !up(&mb->MF, mfv) ||
            !up(&mb->mx_gF, scratch4) || !up(&mb->mx_gC, scratch4) || !up(&mb->mf_node, mnode) ||
            !up(&mb->mf_gs, mgs) || !up(&mb->mf_acoef, macoef) || !up(&mb->mf_face, mface)) {
            err = "precision form: device allocation failed";
            return NSEM_NO_MEMORY;
        }
    }
    auto dal = [&](auto** p, size_t bytes) -> bool {
        if (cudaMalloc((void**)p, bytes) != cudaSuccess) return false;
        allocs->push_back((void*)*p);
        return true;
    };
    for (int s = 0; s < 2; s++)
        if (!dal(&mb->U[s], 5 * n_int * sizeof(double)) || !dal(&mb->S[s], 5 * n_int * sizeof(float)) ||
            !dal(&mb->D[s], 5 * n_int * sizeof(float))) {
            err = "precision form: device allocation failed";
            return NSEM_NO_MEMORY;
        }
    mb->visc = dev.nu != 0.0;
    mb->nu = (float)dev.nu;
    mb->nu_pr = (float)(dev.nu * dev.iPr);
    if (mb->visc && !dal(&mb->G, 12 * n_int * sizeof(float))) {
        err = "precision form: device allocation failed";
        return NSEM_NO_MEMORY;
    }
    /* persistent stage kernels only with NSEM_MIXED_PERSIST=1: measured on
     * GB300 (32^3, N = 4) they are slower than one CTA per element -- the
     * register cap of 8 resident CTAs makes the element loop spill, and with
     * fewer CTAs the prefetch only breaks even */
    {
        const char* pers = std::getenv("NSEM_MIXED_PERSIST");
        LaunchCfg c{};
        c.persist = pers && std::string(pers) == "1";
        if (prepare(NX, NY, NZ, &c) != 0) {
            err = "precision form: cannot reserve the kernel's shared memory";
            return NSEM_CUDA_ERROR;
        }
        mb->persist = c.persist;
        for (int q = 0; q < 4; q++) mb->pgrid[q] = c.pgrid[q];
    }
    /* order 7: line sums on the FP32 pipes (measured faster than the
     * tensor-core variant on GB300); NSEM_MIXED_LINES=tensor selects the
     * tensor-core line sums */
    {
        const char* lines = std::getenv("NSEM_MIXED_LINES");
        mb->tc = NX == 8 && NY == 8 && NZ == 8 && lines && std::string(lines) == "tensor";
    }
    mb->n_elem = ne;
    mb->n_int = n_int;
    mb->npd[0] = NX; mb->npd[1] = NY; mb->npd[2] = NZ;
    mb->n_layers = (int)seen.size();
    mb->ready = true;
    return NSEM_OK;
}

/* ------------------------------------------------------------ launches */

namespace {

StageArgs base_args(const NsemDev* dev, const NsemMixedBuf* mb, double dt) {
    StageArgs a{};
    a.nbr = mb->nbr;
    a.J = mb->J;
    a.layer = mb->layer;
    a.Qg = mb->Qg;
    a.Dg = mb->Dg;
    a.G = mb->G;
    a.Gout = mb->G;
    a.nu = mb->nu;
    a.nu_pr = mb->nu_pr;
    a.T0 = (float)dev->T0;
    a.bg = mb->bg;
    a.Jg = mb->Jg;
    a.Fn = mb->Fn;
    a.MF = mb->MF;
    a.nfmax = mb->nfmax;
    a.n_elem = mb->n_elem;
    a.dt = (float)dt;
    a.gamma = (float)dev->gamma;
    a.gR = (float)dev->gR;
    for (int c = 0; c < 3; c++) {
        a.g[c] = (float)dev->g[c];
        a.lift[c] = mb->lift[c];
    }
    std::memcpy(a.qc, mb->qc, sizeof(a.qc));
    /* binomial coefficients C(gamma, k) of (1 + d)^gamma - 1 */
    double ck = 1.0;
    for (int k = 1; k <= 6; k++) {
        ck *= (dev->gamma - (k - 1)) / k;
        a.eos[k - 1] = (float)ck;
    }
    a.status = dev->status;
    return a;
}

MortarMxArgs mortar_args(const NsemMixedBuf* mb) {
    MortarMxArgs m{};
    m.mi = mb->mx_i;
    m.mf = mb->mx_f;
    m.psiR = mb->mx_psi;
    m.psiC = mb->mx_psi + 6 * MAXN * MAXN;
    m.F = mb->mx_F;
    m.d = mb->mx_d;
    m.dC = mb->mx_dC;
    m.ent = mb->mf_ent;
    m.coef = mb->mf_coef;
    m.MF = mb->MF;
    m.n_ms = mb->n_ms;
    m.n_mf = mb->n_mf;
    m.nfmax = mb->nfmax;
    m.np = mb->npd[0] * mb->npd[1] * mb->npd[2];
    m.gF = mb->mx_gF;
    m.gC = mb->mx_gC;
    m.node = mb->mf_node;
    m.gs = mb->mf_gs;
    m.rows = mb->gen ? MF_ROWS_GEN : MF_ROWS;
    return m;
}

/* the mortar kernels of the stage's fluxes */
int launch_mortars(const NsemMixedBuf* mb, const StageArgs& a, int stage, cudaStream_t st) {
    const MortarMxArgs m = mortar_args(mb);
    const unsigned gs = (unsigned)((mb->n_ms + 127) / 128);
    if (mb->visc) {
        if (stage >= 2) k_mx_mortar_flux<true, true><<<gs, 128, 0, st>>>(a, m);
        else k_mx_mortar_flux<false, true><<<gs, 128, 0, st>>>(a, m);
    } else {
        if (stage >= 2) k_mx_mortar_flux<true, false><<<gs, 128, 0, st>>>(a, m);
        else k_mx_mortar_flux<false, false><<<gs, 128, 0, st>>>(a, m);
    }
    k_mx_mortar_proj<<<gs, 128, 0, st>>>(m);
    k_mx_mortar_fill<<<(unsigned)((mb->n_mf * mb->nfmax + 127) / 128), 128, 0, st>>>(m);
    return (int)cudaGetLastError();
}

/* the mortar kernels of the gradients' face values (viscous runs) */
int launch_mortar_grads(const NsemMixedBuf* mb, const StageArgs& a, int stage, cudaStream_t st) {
    const MortarMxArgs m = mortar_args(mb);
    const unsigned gs = (unsigned)((mb->n_ms + 127) / 128);
    const unsigned gf = (unsigned)((mb->n_mf * mb->nfmax + 127) / 128);
    if (stage >= 2) k_mx_mortar_gcds<true><<<gs, 128, 0, st>>>(a, m);
    else k_mx_mortar_gcds<false><<<gs, 128, 0, st>>>(a, m);
    k_mx_mortar_ggather<<<gs, 128, 0, st>>>(m);
    if (mb->gen) {
        if (stage >= 2) k_mx_mortar_gfill<true, true><<<gf, 128, 0, st>>>(a, m);
        else k_mx_mortar_gfill<false, true><<<gf, 128, 0, st>>>(a, m);
    } else {
        if (stage >= 2) k_mx_mortar_gfill<true, false><<<gf, 128, 0, st>>>(a, m);
        else k_mx_mortar_gfill<false, false><<<gf, 128, 0, st>>>(a, m);
    }
    return (int)cudaGetLastError();
}

int launch_args(const NsemMixedBuf* mb, const StageArgs& a, int stage, cudaStream_t st) {
    LaunchCfg c{};
    c.visc = mb->visc;
    c.gen = mb->gen;
    if (mb->visc) {
        /* the stage state's gradients first (their mortar face values before them) */
        if (mb->n_ms > 0) {
            const int e = launch_mortar_grads(mb, a, stage, st);
            if (e) return e;
        }
        const int e = dispatch_grad(mb->npd[0], mb->npd[1], mb->npd[2], a, stage, st, c);
        if (e) return e;
    }
    if (mb->n_ms > 0) {
        const int e = launch_mortars(mb, a, stage, st);
        if (e) return e;
    }
    c.visc = mb->visc;
    c.tc = mb->tc;
    c.persist = mb->persist;
    c.gen = mb->gen;
    for (int q = 0; q < 4; q++) c.pgrid[q] = mb->pgrid[q];
    return dispatch_stage(mb->npd[0], mb->npd[1], mb->npd[2], a, stage, st, c);
}

}  // namespace

/* one SSP-RK3 step of the precision form with explicit buffers: shadow S of
 * u'^n (stage base), increments d1 and d2, FP64 state U -> Unew with shadow
 * Snew.  Used by the plain steps and by the checkpointed forward runs of the
 * adjoint, which keep S, d1, d2 of every step. */
int nsem_mixed_step_bufs(const NsemDev* dev, const NsemMixedBuf* mb, const double* U,
                         const float* S, float* d1, float* d2, double* Unew, float* Snew,
                         double dt, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    StageArgs a = base_args(dev, mb, dt);
    a.U = U;
    a.S = S;
    a.Din = nullptr;
    a.Dout = d1;
    int e = launch_args(mb, a, 1, st);
    if (e) return e;
    a.Din = d1;
    a.Dout = d2;
    if ((e = launch_args(mb, a, 2, st))) return e;
    a.Din = d2;
    a.Dout = nullptr;
    a.Unew = Unew;
    a.Snew = Snew;
    return launch_args(mb, a, 3, st);
}

int nsem_mixed_grad_at(const NsemDev* dev, const NsemMixedBuf* mb, const float* S,
                       const float* Din, void* stream) {
    StageArgs a = base_args(dev, mb, 0.0);
    a.S = S;
    a.Din = Din;
    LaunchCfg c{};
    c.visc = true;
    c.gen = mb->gen;
    /* the gradients' face values on mortars first */
    if (mb->n_ms > 0) {
        const int e = launch_mortar_grads(mb, a, Din ? 2 : 1, (cudaStream_t)stream);
        if (e) return e;
    }
    return dispatch_grad(mb->npd[0], mb->npd[1], mb->npd[2], a, Din ? 2 : 1, (cudaStream_t)stream, c);
}

int nsem_mixed_convert(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, int to_pert,
                       void* stream) {
    Ptr5 full;
    for (int v = 0; v < 5; v++) full.p[v] = b->u[v];
    const int NP = mb->npd[0] * mb->npd[1] * mb->npd[2];
    cudaStream_t st = (cudaStream_t)stream;
    const int grid = grid_for(dev->n_int);
    double* U = mb->U[mb->cur];
    float* S = mb->S[mb->cur];
#define NSEM_CONV(A, B, C)                                                                     \
    if (NP == A * B * C) {                                                                     \
        if (to_pert)                                                                           \
            k_to_pert<A * B * C><<<grid, 256, 0, st>>>(full, U, S, dev->rho_ref, dev->T0,      \
                                                       dev->n_int);                            \
        else                                                                                   \
            k_from_pert<A * B * C><<<grid, 256, 0, st>>>(U, full, dev->rho_ref, dev->T0,       \
                                                         dev->n_int);                          \
        return (int)cudaGetLastError();                                                        \
    }
    NSEM_MIXED_DIMS(NSEM_CONV)
#undef NSEM_CONV
    return (int)cudaErrorNotSupported;
}

int nsem_mixed_host_layout(const NsemDev* dev, NsemMixedBuf* mb, int to_pert, double* rho,
                           double* mom, double* rt, void* stream) {
    const int NP = mb->npd[0] * mb->npd[1] * mb->npd[2];
    cudaStream_t st = (cudaStream_t)stream;
    const int grid = grid_for(dev->n_int);
    double* U = mb->U[mb->cur];
    float* S = mb->S[mb->cur];
#define NSEM_HOSTL(A, B, C)                                                                    \
    if (NP == A * B * C) {                                                                     \
        if (to_pert)                                                                           \
            k_host_to_pert<A * B * C><<<grid, 256, 0, st>>>(rho, mom, rt, U, S, dev->rho_ref,  \
                                                            dev->T0, dev->n_int);              \
        else                                                                                   \
            k_pert_to_host<A * B * C><<<grid, 256, 0, st>>>(U, rho, mom, rt, dev->rho_ref,     \
                                                            dev->T0, dev->n_int);              \
        return (int)cudaGetLastError();                                                        \
    }
    NSEM_MIXED_DIMS(NSEM_HOSTL)
#undef NSEM_HOSTL
    return (int)cudaErrorNotSupported;
}

int nsem_mixed_steps(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf*, const NsemTables*,
                     int nsteps, double dt, void* stream) {
    int cur = mb->cur;
    for (int n = 0; n < nsteps; n++) {
        int e = nsem_mixed_step_bufs(dev, mb, mb->U[cur], mb->S[cur], mb->D[0], mb->D[1],
                                     mb->U[cur ^ 1], mb->S[cur ^ 1], dt, stream);
        if (e) return e;
        cur ^= 1;
    }
    return 0;
}

int nsem_mixed_tendency(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, const NsemTables*,
                        void* stream) {
    StageArgs a = base_args(dev, mb, 0.0);
    a.U = mb->U[mb->cur];
    a.S = mb->S[mb->cur];
    for (int v = 0; v < 5; v++) a.L[v] = b->L[v];
    return launch_args(mb, a, 0, (cudaStream_t)stream);
}

static const char* const k_names[] = {"mixed_stage1", "mixed_stage2", "mixed_stage3", nullptr};
const char* const* nsem_mixed_kernel_names() { return k_names; }
int nsem_mixed_launches_per_step() { return 3; }
int nsem_mixed_launch_class(int k) { return k; }

int nsem_mixed_launch(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf*, const NsemTables*, int k,
                      int, double dt, void* stream) {
    const int cur = mb->cur;
    StageArgs a = base_args(dev, mb, dt);
    a.U = mb->U[cur];
    a.S = mb->S[cur];
    a.Din = k == 1 ? mb->D[0] : k == 2 ? mb->D[1] : nullptr;
    a.Dout = k == 0 ? mb->D[0] : k == 1 ? mb->D[1] : nullptr;
    a.Unew = mb->U[cur ^ 1];
    a.Snew = mb->S[cur ^ 1];
    int e = launch_args(mb, a, k + 1, (cudaStream_t)stream);
    if (k == 2) mb->cur ^= 1;
    return e;
}
