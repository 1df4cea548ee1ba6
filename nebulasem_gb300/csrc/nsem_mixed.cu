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

#include "nsem_mixed.h"
#include "nsem_mixed_dev.cuh"

using namespace nsem_mx;

namespace {

struct StageArgs {
    const double* U;           /* u'^n (FP64), [e][5][NP]                  */
    const float* S;            /* stage base state: FP32 shadow of u'^n    */
    const float* Din;          /* previous stage increment (or null)      */
    float* Dout;               /* stage increment out (stages 1, 2)       */
    double* Unew;              /* u'^{n+1} (stage 3)                      */
    float* Snew;               /* its FP32 shadow (stage 3)               */
    double* L[5];              /* tendency out (stage 0), node order      */
    const int32_t* nbr;        /* [6][n_elem]                             */
    const float* J;            /* [3][n_elem]                             */
    const int32_t* layer;      /* [n_elem]                                */
    const float* Qg;           /* line-sum weights                        */
    const float* Dg;           /* derivative tables (gradient kernel)     */
    const float* G;            /* viscous runs: [e][12][NP] gradients      */
    float* Gout;               /* gradient kernel output                   */
    const float* bg;           /* [layers][4][NP]                          */
    const float* Jg;           /* general geometry: [e][10][NP] Jinv cV (9), 1/cV */
    const float* Fn;           /* general geometry: [e][3][NFS] outward weighted normals */
    const float* MF;           /* mortar faces: [n_mf][9][nfmax] outward face values (0-4),
                                  viscous runs' gradient face terms (5-8) */
    int nfmax;
    int64_t n_elem;
    float dt, gamma, gR, g[3];
    float nu, nu_pr, T0;
    float lift[3];             /* 1 / w_end per direction                  */
    float eos[6];              /* binomial coefficients C(gamma, k), k = 1..6 */
    uint32_t* status;
};

/* rows per element face of the mortar face buffer: the 5 outward values,
 * then the gradient face terms: 4 (cds - own, axis-aligned elements) or
 * 12 (fN_out[r] (cds - own)_c, general geometry) */
constexpr int MF_ROWS = 9, MF_ROWS_GEN = 17;

/* tensor-core flux layout (order 7): a variable's fluxes of one direction
 * F[a][m][b] -- m the node index along the direction, (a, b) the other two
 * (x: (j, k), y: (i, k), z: (i, j)) -- at a * TC_SA + p(m) * 8 + (b ^ s(m)),
 * p(m) = m ^ (m >> 2 & 1), s(m) = 4 (m >> 2 & 1).  TC_SA = 72 puts four
 * consecutive a in distinct groups of 8 banks; p keeps the rows m = 0-3,
 * 4-7, the even and the odd rows each in four distinct groups; s separates
 * the rows that share a group.  Every access is then conflict-free: the
 * node threads' stores and reads in all three directions (a warp holds one i,
 * four j and eight k), the face threads' reads, the A-fragment loads (rows
 * m = tg, tg + 4) and the in-place result stores (rows 2 tg, 2 tg + 1). */
constexpr int TC_SA = 72;
constexpr int TC_NP = 8 * TC_SA;
constexpr int TC_QTAB = 3 * 2 * 64;   /* B fragments per direction: high, low; [k][n] */

template <int NX, int NY, int NZ, bool TC = false>
struct StageSmem {
    using G = Geo<NX, NY, NZ>;
    static constexpr int NP = G::NP, NFS = G::NFS;
    /* floats: volume fluxes F4[3][NP] (x4) + F1[3][NP] (tensor-core line sums:
     * F[3][5][TC_NP]); own values P[3][NP] (x4); face fluxes FF4[NFS] (x4) +
     * FF1[NFS]; Q; metric */
    static constexpr int FLUX = TC ? 15 * TC_NP : 15 * NP;
    static constexpr int OFF_F1 = 12 * NP;
    static constexpr int OFF_P = (FLUX + 3) / 4 * 4;
    static constexpr int OFF_FF4 = OFF_P + 12 * NP;
    static constexpr int OFF_FF1 = OFF_FF4 + 4 * NFS;
    static constexpr int OFF_Q = OFF_FF1 + NFS;
    static constexpr int OFF_META = OFF_Q + QTAB;
    static_assert(OFF_P % 4 == 0 && OFF_FF4 % 4 == 0, "float4 regions must be 16-byte aligned");
    /* tensor-core line sums: the B fragments of Q_d^T pre-split into TF32
     * high and low parts, [3][2][8][8] words after the metric */
    static constexpr int OFF_QTC = OFF_META + 4;
    static constexpr size_t BYTES = sizeof(float) * (OFF_META + 4 + (TC ? TC_QTAB : 0));
    /* persistent kernels: the next element's stage base, increment and
     * background, staged by asynchronous copies while the current element
     * computes */
    static constexpr int OFF_STG = OFF_META + 4;
    static constexpr size_t BYTES_P = sizeof(float) * (OFF_STG + 14 * NP);
};

/* 4-byte asynchronous copies global -> shared (no registers held while in
 * flight) */
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

/* Tensor-core line sums (order 7, 8 nodes per direction).  The volume term
 * of direction d is, per conserved variable v and line l through the
 * element, r_l = Q_d f_l: as a matrix product R^T = F^T Q_d^T with the rows
 * (v, l) of F^T as M (5 x 64 = 320 rows: 20 tiles of 16), the 8 nodes along
 * the line as K and the 8 output nodes as N, one mma.sync m16n8k8 per tile
 * and TF32 pass.  FP32 accuracy from three TF32 products (a_lo b_hi +
 * a_hi b_lo + a_hi b_hi, Markidis' split; FP32 accumulation).  The fluxes
 * are kept per direction as F_d[v][a][m][b] in the swizzled layout tc_pos. */
__device__ __forceinline__ int tc_pos(int a, int m, int b) {
    const int hi = (m >> 2) & 1;
    return a * TC_SA + ((m ^ hi) << 3) + (b ^ (hi << 2));
}

template <int D>
__device__ __forceinline__ int tc_idx(int i, int j, int k) {
    return D == 0 ? tc_pos(j, i, k) : D == 1 ? tc_pos(i, j, k) : tc_pos(i, k, j);
}

/* index of face slot t within its face: x (j, k), y (i, k), z (i, j) */
template <int NX, int NY, int NZ>
__device__ __forceinline__ int face_local(int t) {
    using G = Geo<NX, NY, NZ>;
    if (t < G::OFF_Y) return t % G::NFX;
    if (t < G::OFF_Z) return (t - G::OFF_Y) % G::NFY;
    return (t - G::OFF_Z) % G::NFZ;
}

__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hi) : "f"(x));
    const float r = x - __uint_as_float(hi);
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lo) : "f"(r));
}

__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

/* registers sized for 8 resident CTAs per SM in stages 1-2 and 7 in the stage
 * that also carries the FP64 state (measured best on GB300), 6 when viscous */
#ifndef NSEM_MIXED_MB12
#define NSEM_MIXED_MB12 8
#endif
#ifndef NSEM_MIXED_MB3
#define NSEM_MIXED_MB3 7
#endif
template <int NX, int NY, int NZ, int STAGE, bool VISC, bool PERSIST = false>
constexpr int stage_min_blocks() {
    /* order 7 (512 threads, 64 KB of shared memory): three CTAs, two for the
     * stages that hold more live values (no spills) */
    if (Geo<NX, NY, NZ>::BLOCK >= 512)
        return min_blocks((VISC || STAGE == 3 || STAGE == 0) ? 2 : 3, Geo<NX, NY, NZ>::BLOCK,
                          StageSmem<NX, NY, NZ>::BYTES);
    return min_blocks(VISC ? 6 : (STAGE == 1 || STAGE == 2) ? NSEM_MIXED_MB12 : NSEM_MIXED_MB3,
                      Geo<NX, NY, NZ>::BLOCK,
                      PERSIST ? StageSmem<NX, NY, NZ>::BYTES_P : StageSmem<NX, NY, NZ>::BYTES);
}

/* phase 2: flux through face node t of direction DIR, seen from the element */
template <int NX, int NY, int NZ, int DIR, bool VISC, bool TC>
__device__ __forceinline__ void face_flux(const FaceSlot& fs, int32_t nb, const float* oth,
                                          const float* bgo, const float* gfo, const float4* sF4,
                                          const float* sF1, const float4* sP, const StageArgs& a,
                                          float4& o4, float& o1) {
    constexpr int NP = Geo<NX, NY, NZ>::NP;
    const float sg = fs.side ? 1.0f : -1.0f;   /* outward normal = sg e_DIR */
    const float4 P0 = sP[fs.la], P1 = sP[NP + fs.la];
    const float md_s = DIR == 0 ? P0.y : DIR == 1 ? P0.z : P0.w;
    const float um_s = P1.z, c_s = P1.w;
    if (nb >= 0) {
        float4 A4;
        float A1;
        if constexpr (TC) {
            const float* f = reinterpret_cast<const float*>(sF4) + DIR * 5 * TC_NP +
                             tc_idx<DIR>(fs.la >> 6, (fs.la >> 3) & 7, fs.la & 7);
            A4 = make_float4(f[0], f[TC_NP], f[2 * TC_NP], f[3 * TC_NP]);
            A1 = f[4 * TC_NP];
        } else {
            A4 = sF4[DIR * NP + fs.la];
            A1 = sF1[DIR * NP + fs.la];
        }
        const Pt q = pointwise(oth, bgo, a.eos, a.gamma, a.gR);
        float g12[12] = {};
        if constexpr (VISC) {
            g12[tidx(0, DIR)] = gfo[0];
            g12[tidx(1, DIR)] = gfo[1];
            g12[tidx(2, DIR)] = gfo[2];
            g12[9 + DIR] = gfo[3];
        }
        float4 B4;
        float B1;
        vol_flux<DIR, VISC>(oth, q, g12, a.nu, a.nu_pr, B4, B1);
        const float lam = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(um_s, q.umag), __fadd_rn(c_s, q.c)));
        const float av0 = __fmul_rn(0.5f, __fadd_rn(A4.x, B4.x));
        const float av1 = __fmul_rn(0.5f, __fadd_rn(A4.y, B4.y));
        const float av2 = __fmul_rn(0.5f, __fadd_rn(A4.z, B4.z));
        const float av3 = __fmul_rn(0.5f, __fadd_rn(A4.w, B4.w));
        const float av4 = __fmul_rn(0.5f, __fadd_rn(A1, B1));
        const float jr = __fsub_rn(oth[0], P0.x);
        const float jm = __fsub_rn(oth[1 + DIR], md_s);
        const float jt = __fsub_rn(oth[4], P1.x);
        o4.x = __fmaf_rn(-lam, jr, sg * av0);
        o4.y = DIR == 0 ? __fmaf_rn(-lam, jm, sg * av1) : sg * av1;
        o4.z = DIR == 1 ? __fmaf_rn(-lam, jm, sg * av2) : sg * av2;
        o4.w = DIR == 2 ? __fmaf_rn(-lam, jm, sg * av3) : sg * av3;
        o1 = __fmaf_rn(-lam, jt, sg * av4);
    } else {
        /* wall ghost: rho, theta, p NEUMANN; SYMMETRY velocity (tangential
         * projection rescaled to |U|, tensor.h:486-494), normal velocity 0.
         * The ghost value alone is the face average (fI = 0 on a wall,
         * field.cpp:257-266), so only the normal momentum flux remains:
         * s p' + lam m_n, lam = (|U_ghost| + c) / 2.  No viscous wall flux
         * (zero ghost gradient). */
        const float4 P2 = sP[2 * NP + fs.la];
        const float r0 = DIR == 0 ? 0.0f : P2.x;
        const float r1 = DIR == 1 ? 0.0f : P2.y;
        const float r2 = DIR == 2 ? 0.0f : P2.z;
        const float mr = safe_sqrt(__fmaf_rn(r0, r0, __fmaf_rn(r1, r1, __fmul_rn(r2, r2))));
        const float um_g = mr > 1e-7f ? um_s : mr;
        const float lam = __fmul_rn(0.5f, __fadd_rn(um_g, c_s));
        const float fn = __fmaf_rn(lam, md_s, sg * P2.w);
        o4 = make_float4(0.0f, DIR == 0 ? fn : 0.0f, DIR == 1 ? fn : 0.0f, DIR == 2 ? fn : 0.0f);
        o1 = 0.0f;
    }
}

/* one kernel per stage (0: tendency only): the stage's own loads and update */
/* PERSIST: a grid of resident CTAs walks the elements (e, e + grid, ...);
 * while one element computes, the next element's own stage base and
 * increment stream into shared memory, so their load latency is hidden; the
 * line-sum table is staged once per CTA. */
template <int NX, int NY, int NZ, int STAGE, bool VISC, bool TC, bool PERSIST>
__global__ void __launch_bounds__(Geo<NX, NY, NZ>::BLOCK,
                                  (stage_min_blocks<NX, NY, NZ, STAGE, VISC, PERSIST>()))
k_mixed_stage(StageArgs a) {
    static_assert(!TC || (NX == 8 && NY == 8 && NZ == 8), "tensor-core line sums: order 7");
    using G = Geo<NX, NY, NZ>;
    using SM = StageSmem<NX, NY, NZ, TC>;
    constexpr int NP = G::NP;
    constexpr int NFS = G::NFS;
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    float4* sF4 = smem4;                                          /* [3][NP] */
    float* sF1 = smem + SM::OFF_F1;                               /* [3][NP] */
    float4* sP = reinterpret_cast<float4*>(smem + SM::OFF_P);     /* [3][NP] */
    float4* sFF4 = reinterpret_cast<float4*>(smem + SM::OFF_FF4); /* [NFS] */
    float* sFF1 = smem + SM::OFF_FF1;                             /* [NFS] */
    float* sQ = smem + SM::OFF_Q;
    float* sMeta = smem + SM::OFF_META;

    const int t = threadIdx.x;
    constexpr bool has_din = STAGE >= 2;
    float* sStg = smem + SM::OFF_STG;                             /* [14][NP] (PERSIST) */
    for (int q = t; q < QTAB; q += G::BLOCK) sQ[q] = __ldg(a.Qg + q);
    if constexpr (TC) {
        float* sQtc = smem + SM::OFF_QTC;
        for (int q = t; q < TC_QTAB; q += G::BLOCK) sQtc[q] = __ldg(a.Qg + QTAB + q);
    }
    auto prefetch = [&](int64_t en, int32_t lay) {
        if (t < NP) {
            const float* s = a.S + en * 5 * NP + t;
#pragma unroll
            for (int v = 0; v < 5; v++) cp_async4(sStg + v * NP + t, s + v * NP);
            if constexpr (has_din) {
                const float* d = a.Din + en * 5 * NP + t;
#pragma unroll
                for (int v = 0; v < 5; v++) cp_async4(sStg + (5 + v) * NP + t, d + v * NP);
            }
            const float* bg = a.bg + (int64_t)lay * 4 * NP + t;
#pragma unroll
            for (int c = 0; c < 4; c++) cp_async4(sStg + (10 + c) * NP + t, bg + c * NP);
        }
        cp_async_commit();
    };
    const int64_t e_step = gridDim.x;
    auto element = [&](const int64_t e) {
    int32_t lay_next = 0;
    if constexpr (PERSIST) {
        cp_async_wait_all();
        __syncthreads();
        /* the next element's background layer, needed when its copies start */
        if (e + e_step < a.n_elem) lay_next = __ldg(a.layer + e + e_step);
    }

    /* issue every global load first: own node, face neighbour, stage-3 FP64 */
    float own[5], din[5] = {0, 0, 0, 0, 0}, bgs[4] = {0, 0, 0, 0};
    double u64[5];
    float gown[12];
    if (t < NP) {
        if constexpr (PERSIST) {
#pragma unroll
            for (int v = 0; v < 5; v++) own[v] = sStg[v * NP + t];
            if constexpr (has_din) {
#pragma unroll
                for (int v = 0; v < 5; v++) {
                    din[v] = sStg[(5 + v) * NP + t];
                    own[v] = __fadd_rn(own[v], din[v]);
                }
            }
        } else {
            const float* s = a.S + e * 5 * NP + t;
#pragma unroll
            for (int v = 0; v < 5; v++) own[v] = __ldg(s + v * NP);
            if constexpr (has_din) {
                const float* d = a.Din + e * 5 * NP + t;
#pragma unroll
                for (int v = 0; v < 5; v++) {
                    din[v] = __ldg(d + v * NP);
                    own[v] = __fadd_rn(own[v], din[v]);
                }
            }
        }
        if constexpr (PERSIST) {
#pragma unroll
            for (int c = 0; c < 4; c++) bgs[c] = sStg[(10 + c) * NP + t];
        } else {
            const float* bg = a.bg + (int64_t)__ldg(a.layer + e) * 4 * NP + t;
#pragma unroll
            for (int c = 0; c < 4; c++) bgs[c] = __ldg(bg + c * NP);
        }
        if constexpr (STAGE == 3) {
            const double* u = a.U + e * 5 * NP + t;
#pragma unroll
            for (int v = 0; v < 5; v++) u64[v] = __ldg(u + v * NP);
        }
        if constexpr (VISC) {
            const float* gr = a.G + e * 12 * NP + t;
#pragma unroll
            for (int c = 0; c < 12; c++) gown[c] = __ldg(gr + c * NP);
        }
    }
    FaceSlot fs{};
    int32_t nb = -1;
    float oth[5], bgo[4];
    float gfo[4] = {0, 0, 0, 0};
    if (t < NFS) {
        fs = face_slot<NX, NY, NZ>(t);
        nb = __ldg(a.nbr + (int64_t)fs.face * a.n_elem + e);
        if (nb <= -2) {
            /* a face on a 2:1 mortar: its outward values come from the
             * mortar kernels */
            const float* mf = a.MF + (int64_t)(-2 - nb) * MF_ROWS * a.nfmax + face_local<NX, NY, NZ>(t);
#pragma unroll
            for (int v = 0; v < 5; v++) oth[v] = __ldg(mf + v * a.nfmax);
        }
        if (nb >= 0) {
            const float* s = a.S + (int64_t)nb * 5 * NP + fs.lo;
#pragma unroll
            for (int v = 0; v < 5; v++) oth[v] = __ldg(s + v * NP);
            if constexpr (has_din) {
                const float* d = a.Din + (int64_t)nb * 5 * NP + fs.lo;
#pragma unroll
                for (int v = 0; v < 5; v++) oth[v] = __fadd_rn(oth[v], __ldg(d + v * NP));
            }
            const float* bg = a.bg + (int64_t)__ldg(a.layer + nb) * 4 * NP + fs.lo;
#pragma unroll
            for (int c = 0; c < 4; c++) bgo[c] = __ldg(bg + c * NP);
            if constexpr (VISC) {
                /* the neighbour's gradients along the face's axis only:
                 * d_c U_dir (c = 0..2) and d_dir theta */
                const float* gr = a.G + (int64_t)nb * 12 * NP + fs.lo;
                const int d = fs.dir;
                gfo[0] = __ldg(gr + tidx(0, d) * NP);
                gfo[1] = __ldg(gr + tidx(1, d) * NP);
                gfo[2] = __ldg(gr + tidx(2, d) * NP);
                gfo[3] = __ldg(gr + (9 + d) * NP);
            }
        }
    }
    if (t < 3) sMeta[t] = __ldg(a.J + (int64_t)t * a.n_elem + e);

    /* phase 1: own node primitives and volume fluxes */
    if (t < NP) {
        const Pt p = pointwise(own, bgs, a.eos, a.gamma, a.gR);
        sP[t] = make_float4(own[0], own[1], own[2], own[3]);
        sP[NP + t] = make_float4(own[4], p.rho, p.umag, p.c);
        sP[2 * NP + t] = make_float4(p.u[0], p.u[1], p.u[2], p.pp);
        float4 f4;
        float f1;
        if constexpr (TC) {
            const int i = t >> 6, j = (t >> 3) & 7, k = t & 7;
            auto put = [&](int d, int idx, const float4& v4, float v1) {
                float* f = smem + d * 5 * TC_NP + idx;
                f[0] = v4.x; f[TC_NP] = v4.y; f[2 * TC_NP] = v4.z; f[3 * TC_NP] = v4.w;
                f[4 * TC_NP] = v1;
            };
            vol_flux<0, VISC>(own, p, gown, a.nu, a.nu_pr, f4, f1);
            put(0, tc_idx<0>(i, j, k), f4, f1);
            vol_flux<1, VISC>(own, p, gown, a.nu, a.nu_pr, f4, f1);
            put(1, tc_idx<1>(i, j, k), f4, f1);
            vol_flux<2, VISC>(own, p, gown, a.nu, a.nu_pr, f4, f1);
            put(2, tc_idx<2>(i, j, k), f4, f1);
        } else {
            vol_flux<0, VISC>(own, p, gown, a.nu, a.nu_pr, f4, f1);
            sF4[t] = f4; sF1[t] = f1;
            if constexpr (G::HAS_Y) {
                vol_flux<1, VISC>(own, p, gown, a.nu, a.nu_pr, f4, f1);
                sF4[NP + t] = f4; sF1[NP + t] = f1;
            }
            vol_flux<2, VISC>(own, p, gown, a.nu, a.nu_pr, f4, f1);
            sF4[2 * NP + t] = f4; sF1[2 * NP + t] = f1;
        }
    }
    __syncthreads();
    if constexpr (PERSIST) {
        /* the staging area is free: stream in the next element */
        if (e + e_step < a.n_elem) prefetch(e + e_step, lay_next);
    }

    /* phase 2: Rusanov flux on every face node */
    if (t < NFS) {
        float4 o4;
        float o1;
        if (nb <= -2) {
            o4 = make_float4(oth[0], oth[1], oth[2], oth[3]);
            o1 = oth[4];
        } else if (fs.dir == 0)
            face_flux<NX, NY, NZ, 0, VISC, TC>(fs, nb, oth, bgo, gfo, sF4, sF1, sP, a, o4, o1);
        else if (G::HAS_Y && fs.dir == 1)
            face_flux<NX, NY, NZ, 1, VISC, TC>(fs, nb, oth, bgo, gfo, sF4, sF1, sP, a, o4, o1);
        else
            face_flux<NX, NY, NZ, 2, VISC, TC>(fs, nb, oth, bgo, gfo, sF4, sF1, sP, a, o4, o1);
        sFF4[t] = o4;
        sFF1[t] = o1;
    }
    __syncthreads();

    /* phase 3: weak volume term (line sums with Q), lift, buoyancy, update */
    if constexpr (TC) {
        /* tensor-core line sums, results in place of the fluxes */
        const int lane = t & 31, w = t >> 5, gq = lane >> 2, tg = lane & 3;
        /* lane offsets of the A fragment (rows m = tg, tg + 4) and of the C
         * fragment (rows 2 tg, 2 tg + 1), line b = gq, within a tile */
        const int oa0 = tc_pos(0, tg, gq), oa2 = tc_pos(0, tg + 4, gq);
        const int oc0 = tc_pos(0, 2 * tg, gq), oc1 = tc_pos(0, 2 * tg + 1, gq);
        for (int q = w; q < 60; q += G::BLOCK / 32) {
            const int d = q / 20, r = q % 20, v = r >> 2, a0 = (r & 3) * 2;
            float* base = smem + d * 5 * TC_NP + v * TC_NP + a0 * TC_SA;
            uint32_t ah[4], al[4], bh0, bl0, bh1, bl1;
            split_tf32(base[oa0], ah[0], al[0]);
            split_tf32(base[TC_SA + oa0], ah[1], al[1]);
            split_tf32(base[oa2], ah[2], al[2]);
            split_tf32(base[TC_SA + oa2], ah[3], al[3]);
            /* B = Q_d^T, pre-split on the host exactly as split_tf32 would:
             * rows k = tg, tg + 4 of the high and the low part, column n = gq */
            const float* qb = smem + SM::OFF_QTC + d * 128 + tg * 8 + gq;
            bh0 = __float_as_uint(qb[0]);
            bh1 = __float_as_uint(qb[32]);
            bl0 = __float_as_uint(qb[64]);
            bl1 = __float_as_uint(qb[96]);
            float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            mma_tf32(c, al, bh0, bh1);
            mma_tf32(c, ah, bl0, bl1);
            mma_tf32(c, ah, bh0, bh1);
            base[oc0] = c[0];
            base[oc1] = c[1];
            base[TC_SA + oc0] = c[2];
            base[TC_SA + oc1] = c[3];
        }
        __syncthreads();
    }
    if (t < NP) {
    const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
    float L0, L1, L2, L3, L4;
    if constexpr (TC) {
        const float Jx = sMeta[0], Jy = sMeta[1], Jz = sMeta[2];
        const float* rx = smem + tc_idx<0>(i, j, k);
        const float* ry = smem + 5 * TC_NP + tc_idx<1>(i, j, k);
        const float* rz = smem + 10 * TC_NP + tc_idx<2>(i, j, k);
        float Lt[5];
#pragma unroll
        for (int v = 0; v < 5; v++)
            Lt[v] = fmaf(Jz, rz[v * TC_NP], fmaf(Jy, ry[v * TC_NP], Jx * rx[v * TC_NP]));
        L0 = Lt[0]; L1 = Lt[1]; L2 = Lt[2]; L3 = Lt[3]; L4 = Lt[4];
    } else {
    {
        float4 acc = make_float4(0, 0, 0, 0);
        float acc1 = 0.0f;
        const float* q = sQ + i * QS;
#pragma unroll
        for (int m = 0; m < NX; m++) {
            const int b = (m * NY + j) * NZ + k;
            const float4 f = sF4[b];
            acc.x = fmaf(q[m], f.x, acc.x); acc.y = fmaf(q[m], f.y, acc.y);
            acc.z = fmaf(q[m], f.z, acc.z); acc.w = fmaf(q[m], f.w, acc.w);
            acc1 = fmaf(q[m], sF1[b], acc1);
        }
        const float Jx = sMeta[0];
        L0 = Jx * acc.x; L1 = Jx * acc.y; L2 = Jx * acc.z; L3 = Jx * acc.w; L4 = Jx * acc1;
    }
    if constexpr (G::HAS_Y) {
        float4 acc = make_float4(0, 0, 0, 0);
        float acc1 = 0.0f;
        const float* q = sQ + MAXN * QS + j * QS;
#pragma unroll
        for (int m = 0; m < NY; m++) {
            const int b = (i * NY + m) * NZ + k;
            const float4 f = sF4[NP + b];
            acc.x = fmaf(q[m], f.x, acc.x); acc.y = fmaf(q[m], f.y, acc.y);
            acc.z = fmaf(q[m], f.z, acc.z); acc.w = fmaf(q[m], f.w, acc.w);
            acc1 = fmaf(q[m], sF1[NP + b], acc1);
        }
        const float Jy = sMeta[1];
        L0 = fmaf(Jy, acc.x, L0); L1 = fmaf(Jy, acc.y, L1); L2 = fmaf(Jy, acc.z, L2);
        L3 = fmaf(Jy, acc.w, L3); L4 = fmaf(Jy, acc1, L4);
    }
    {
        float4 acc = make_float4(0, 0, 0, 0);
        float acc1 = 0.0f;
        const float* q = sQ + 2 * MAXN * QS + k * QS;
#pragma unroll
        for (int m = 0; m < NZ; m++) {
            const int b = (i * NY + j) * NZ + m;
            const float4 f = sF4[2 * NP + b];
            acc.x = fmaf(q[m], f.x, acc.x); acc.y = fmaf(q[m], f.y, acc.y);
            acc.z = fmaf(q[m], f.z, acc.z); acc.w = fmaf(q[m], f.w, acc.w);
            acc1 = fmaf(q[m], sF1[2 * NP + b], acc1);
        }
        const float Jz = sMeta[2];
        L0 = fmaf(Jz, acc.x, L0); L1 = fmaf(Jz, acc.y, L1); L2 = fmaf(Jz, acc.z, L2);
        L3 = fmaf(Jz, acc.w, L3); L4 = fmaf(Jz, acc1, L4);
    }
    }
    /* surface lift: -(J_d / w_end) F_out for the face of each axis through
     * the node (at most one per axis) */
    auto lift = [&](int slot, float coef) {
        const float4 f = sFF4[slot];
        L0 = fmaf(-coef, f.x, L0); L1 = fmaf(-coef, f.y, L1); L2 = fmaf(-coef, f.z, L2);
        L3 = fmaf(-coef, f.w, L3); L4 = fmaf(-coef, sFF1[slot], L4);
    };
    {
        const int sx = face_of_node<NX, NY, NZ, 0>(i, j, k);
        if (sx >= 0) lift(sx, sMeta[0] * a.lift[0]);
        if constexpr (G::HAS_Y) {
            const int sy = face_of_node<NX, NY, NZ, 1>(i, j, k);
            if (sy >= 0) lift(sy, sMeta[1] * a.lift[1]);
        }
        const int sz = face_of_node<NX, NY, NZ, 2>(i, j, k);
        if (sz >= 0) lift(sz, sMeta[2] * a.lift[2]);
    }
    /* buoyancy (rho - rho_ref) g */
    const float rp = own[0];
    L1 = fmaf(rp, a.g[0], L1);
    L2 = fmaf(rp, a.g[1], L2);
    L3 = fmaf(rp, a.g[2], L3);
    const float Lv[5] = {L0, L1, L2, L3, L4};

    if constexpr (STAGE == 0) {
        const int64_t n = e * NP + t;
#pragma unroll
        for (int v = 0; v < 5; v++) a.L[v][n] = f2d(Lv[v]);
    }
    const int64_t o = e * 5 * NP + t;
    const float dt = a.dt;
    if constexpr (STAGE == 1) {
#pragma unroll
        for (int v = 0; v < 5; v++) a.Dout[o + v * NP] = dt * Lv[v];
    } else if constexpr (STAGE == 2) {
#pragma unroll
        for (int v = 0; v < 5; v++) a.Dout[o + v * NP] = 0.25f * fmaf(dt, Lv[v], din[v]);
    } else if constexpr (STAGE == 3) {
        bool finite = true;
#pragma unroll
        for (int v = 0; v < 5; v++) {
            const float D = (2.0f / 3.0f) * fmaf(dt, Lv[v], din[v]);
            const double un = u64[v] + f2d(D);
            a.Unew[o + v * NP] = un;
            a.Snew[o + v * NP] = d2f_rn(un);
            /* exponent field all ones = inf or nan (integer test, no FP64 op) */
            finite = finite && ((__double2hiint(un) & 0x7ff00000) != 0x7ff00000);
        }
        if (!finite) atomicOr(a.status, NSEM_STATUS_NONFINITE);
    }
    }  /* t < NP */
    };  /* element */
    if constexpr (PERSIST) {
        prefetch(blockIdx.x, __ldg(a.layer + blockIdx.x));
        for (int64_t e = blockIdx.x; e < a.n_elem; e += e_step) element(e);
        cp_async_wait_all();
    } else {
        element(blockIdx.x);
    }
}


/* ------------------------------------------------------------------------
 * General geometry (inclined, curved elements; inviscid): the metric is a
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
    /* floats: contravariant fluxes G4[3][NP] (x4) + G1[3][NP]; own values
     * P[4][NP] (x4); face fluxes FF4[NFS] (x4) + FF1[NFS]; line table;
     * viscous runs: the nodes' gradients GV[12][NP] */
    static constexpr int OFF_G1 = 12 * NP;
    static constexpr int OFF_P = (15 * NP + 3) / 4 * 4;
    static constexpr int OFF_FF4 = OFF_P + 16 * NP;
    static constexpr int OFF_FF1 = OFF_FF4 + 4 * NFS;
    static constexpr int OFF_Q = OFF_FF1 + NFS;
    static constexpr int OFF_GV = OFF_Q + QTAB;
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

template <int NX, int NY, int NZ, int STAGE, bool VISC>
__global__ void __launch_bounds__(Geo<NX, NY, NZ>::BLOCK,
                                  (min_blocks(NX == 8 ? 2 : (VISC ? 4 : 6), Geo<NX, NY, NZ>::BLOCK,
                                              GenSmem<NX, NY, NZ, VISC>::BYTES)))
k_mixed_stage_gen(StageArgs a) {
    using G = Geo<NX, NY, NZ>;
    using SM = GenSmem<NX, NY, NZ, VISC>;
    constexpr int NP = G::NP;
    constexpr int NFS = G::NFS;
    extern __shared__ float4 gen4[];
    float* smem = reinterpret_cast<float*>(gen4);
    float4* sG4 = gen4;
    float* sG1 = smem + SM::OFF_G1;
    float4* sP = reinterpret_cast<float4*>(smem + SM::OFF_P);
    float4* sFF4 = reinterpret_cast<float4*>(smem + SM::OFF_FF4);
    float* sFF1 = smem + SM::OFF_FF1;
    float* sQ = smem + SM::OFF_Q;
    float* sGV = smem + SM::OFF_GV;     /* viscous runs: [12][NP] */
    const int t = threadIdx.x;
    const int64_t e = blockIdx.x;
    constexpr bool has_din = STAGE >= 2;
    for (int q = t; q < QTAB; q += G::BLOCK) sQ[q] = __ldg(a.Qg + q);

    float own[5], din[5] = {0, 0, 0, 0, 0}, bgs[4] = {0, 0, 0, 0}, jin[9], icv = 0.0f;
    float gown[12];
    double u64[5];
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
            const double* u = a.U + e * 5 * NP + t;
#pragma unroll
            for (int v = 0; v < 5; v++) u64[v] = __ldg(u + v * NP);
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
        fs = face_slot<NX, NY, NZ>(t);
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
            sG4[d * NP + t] = g4;
            sG1[d * NP + t] = g1;
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

    /* phase 3: line sums l_a'(x_m) G_d(m), lift, 1/cV, buoyancy, update */
    if (t >= NP) return;
    const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
    float4 acc = make_float4(0, 0, 0, 0);
    float acc1 = 0.0f;
    {
        const float* q = sQ + i * QS;
#pragma unroll
        for (int m = 0; m < NX; m++) {
            const int b = (m * NY + j) * NZ + k;
            const float4 f = sG4[b];
            acc.x = fmaf(q[m], f.x, acc.x); acc.y = fmaf(q[m], f.y, acc.y);
            acc.z = fmaf(q[m], f.z, acc.z); acc.w = fmaf(q[m], f.w, acc.w);
            acc1 = fmaf(q[m], sG1[b], acc1);
        }
    }
    if constexpr (G::HAS_Y) {
        const float* q = sQ + MAXN * QS + j * QS;
#pragma unroll
        for (int m = 0; m < NY; m++) {
            const int b = (i * NY + m) * NZ + k;
            const float4 f = sG4[NP + b];
            acc.x = fmaf(q[m], f.x, acc.x); acc.y = fmaf(q[m], f.y, acc.y);
            acc.z = fmaf(q[m], f.z, acc.z); acc.w = fmaf(q[m], f.w, acc.w);
            acc1 = fmaf(q[m], sG1[NP + b], acc1);
        }
    }
    {
        const float* q = sQ + 2 * MAXN * QS + k * QS;
#pragma unroll
        for (int m = 0; m < NZ; m++) {
            const int b = (i * NY + j) * NZ + m;
            const float4 f = sG4[2 * NP + b];
            acc.x = fmaf(q[m], f.x, acc.x); acc.y = fmaf(q[m], f.y, acc.y);
            acc.z = fmaf(q[m], f.z, acc.z); acc.w = fmaf(q[m], f.w, acc.w);
            acc1 = fmaf(q[m], sG1[2 * NP + b], acc1);
        }
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
            const float D = (2.0f / 3.0f) * fmaf(dt, Lv[v], din[v]);
            const double un = u64[v] + f2d(D);
            a.Unew[o + v * NP] = un;
            a.Snew[o + v * NP] = d2f_rn(un);
            finite = finite && ((__double2hiint(un) & 0x7ff00000) != 0x7ff00000);
        }
        if (!finite) atomicOr(a.status, NSEM_STATUS_NONFINITE);
    }
}

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
enum { MX_FINE, MX_FINE_C1, MX_BASE, MX_SA, MX_SB, MX_NA, MX_NB, MX_IA, MX_IB, MX_FIRST, MX_TA,
       MX_TB, MX_FIELDS };
constexpr int MX_COARSE = 1 << 30;

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

/* Strong-form DG gradients of U and theta of a stage state (gradf<true>,
 * field.h:3327-3360) for the viscous fluxes: per node
 *   d_r q = J_r sum_m D_r[a_r][m] q_m  +  (J_r / w_end) (cds(q) - q)  on the
 *   lower (-) / upper (+) face normal to r through the node,
 * cds = (own + neighbour) / 2 inside, the ghost value on a wall (SYMMETRY
 * velocity, NEUMANN theta: cds(theta) - theta = 0 there).  The state is the
 * stage kernel's (FP32 shadow plus the previous increment for SIN >= 2).
 * Output [e][12][NP]: tidx(r, c) = d_r U_c, 9 + r = d_r theta. */
template <int NX, int NY, int NZ>
constexpr size_t grad_smem() {
    using G = Geo<NX, NY, NZ>;
    return sizeof(float4) * (G::NP + G::NFS) + sizeof(float) * (QTAB + 4);
}

template <int NX, int NY, int NZ, int SIN>
__global__ void __launch_bounds__(Geo<NX, NY, NZ>::BLOCK)
k_mixed_grad(StageArgs a) {
    using G = Geo<NX, NY, NZ>;
    constexpr int NP = G::NP;
    constexpr int NFS = G::NFS;
    constexpr bool has_din = SIN >= 2;
    extern __shared__ float4 gsm4[];
    float4* sV = gsm4;                                              /* [NP]  U, theta */
    float4* sD = gsm4 + NP;                                         /* [NFS] cds - own */
    float* sDg = reinterpret_cast<float*>(gsm4 + NP + NFS);        /* line tables */
    float* sJ = sDg + QTAB;                                         /* [3] */
    const int t = threadIdx.x;
    const int64_t e = blockIdx.x;

    float own[5], bgs0 = 0.0f;
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
    }
    FaceSlot fs{};
    int32_t nb = -1;
    float oth[5], bgo0 = 0.0f;
    if (t < NFS) {
        fs = face_slot<NX, NY, NZ>(t);
        nb = __ldg(a.nbr + (int64_t)fs.face * a.n_elem + e);
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
    if (t < 3) sJ[t] = __ldg(a.J + (int64_t)t * a.n_elem + e);

    /* U = m / rho as the stage kernel forms it, and theta - T0 from the
     * perturbation: the background has theta = T0 (Theta_ref = rho_ref T0),
     * so theta - T0 = (Theta' - T0 rho') / rho -- the same gradient as theta
     * without FP32 cancellation against T0 */
    const float T0 = a.T0;
    auto prim_ut = [T0](const float* s, float rref) {
        const float inv = rcp_nr(__fadd_rn(rref, s[0]));
        return make_float4(__fmul_rn(s[1], inv), __fmul_rn(s[2], inv), __fmul_rn(s[3], inv),
                           __fmul_rn(__fmaf_rn(-T0, s[0], s[4]), inv));
    };
    if (t < NP) sV[t] = prim_ut(own, bgs0);
    __syncthreads();

    if (t < NFS && nb <= -2) {
        /* a face on a 2:1 mortar: the projected values from the mortar kernels */
        const float* gf = a.MF + ((int64_t)(-2 - nb) * MF_ROWS + 5) * a.nfmax + face_local<NX, NY, NZ>(t);
        sD[t] = make_float4(__ldg(gf), __ldg(gf + a.nfmax), __ldg(gf + 2 * a.nfmax),
                            __ldg(gf + 3 * a.nfmax));
    } else if (t < NFS) {
        const float4 S = sV[fs.la];
        float4 c;
        if (nb >= 0) {
            const float4 O = prim_ut(oth, bgo0);
            c = make_float4(0.5f * S.x + 0.5f * O.x, 0.5f * S.y + 0.5f * O.y,
                            0.5f * S.z + 0.5f * O.z, 0.5f * S.w + 0.5f * O.w);
        } else {
            /* wall ghost: SYMMETRY velocity, NEUMANN theta */
            const int dir = fs.dir;
            float r0 = dir == 0 ? 0.0f : S.x;
            float r1 = dir == 1 ? 0.0f : S.y;
            float r2 = dir == 2 ? 0.0f : S.z;
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
    float4 d[3];
    {
        float4 acc = make_float4(0, 0, 0, 0);
        const float* q = sDg + i * QS;
#pragma unroll
        for (int m = 0; m < NX; m++) {
            const float4 v = sV[(m * NY + j) * NZ + k];
            acc.x = fmaf(q[m], v.x, acc.x); acc.y = fmaf(q[m], v.y, acc.y);
            acc.z = fmaf(q[m], v.z, acc.z); acc.w = fmaf(q[m], v.w, acc.w);
        }
        d[0] = acc;
    }
    {
        float4 acc = make_float4(0, 0, 0, 0);
        if (NY > 1) {
            const float* q = sDg + MAXN * QS + j * QS;
#pragma unroll
            for (int m = 0; m < NY; m++) {
                const float4 v = sV[(i * NY + m) * NZ + k];
                acc.x = fmaf(q[m], v.x, acc.x); acc.y = fmaf(q[m], v.y, acc.y);
                acc.z = fmaf(q[m], v.z, acc.z); acc.w = fmaf(q[m], v.w, acc.w);
            }
        }
        d[1] = acc;
    }
    {
        float4 acc = make_float4(0, 0, 0, 0);
        const float* q = sDg + 2 * MAXN * QS + k * QS;
#pragma unroll
        for (int m = 0; m < NZ; m++) {
            const float4 v = sV[(i * NY + j) * NZ + m];
            acc.x = fmaf(q[m], v.x, acc.x); acc.y = fmaf(q[m], v.y, acc.y);
            acc.z = fmaf(q[m], v.z, acc.z); acc.w = fmaf(q[m], v.w, acc.w);
        }
        d[2] = acc;
    }
    const float Jd[3] = {sJ[0], sJ[1], sJ[2]};
#pragma unroll
    for (int r = 0; r < 3; r++) {
        d[r].x *= Jd[r]; d[r].y *= Jd[r]; d[r].z *= Jd[r]; d[r].w *= Jd[r];
    }
    /* face terms: + (J_r / w_end) (cds - own) on the upper face, - on the lower */
    auto lift = [&](int r, int slot, float coef) {
        const float4 f = sD[slot];
        d[r].x = fmaf(coef, f.x, d[r].x); d[r].y = fmaf(coef, f.y, d[r].y);
        d[r].z = fmaf(coef, f.z, d[r].z); d[r].w = fmaf(coef, f.w, d[r].w);
    };
    const float cx = Jd[0] * a.lift[0], cy = Jd[1] * a.lift[1], cz = Jd[2] * a.lift[2];
    if (i == 0) lift(0, G::OFF_X + j * NZ + k, -cx);
    if (i == NX - 1) lift(0, G::OFF_X + G::NFX + j * NZ + k, cx);
    if (NY > 1) {
        if (j == 0) lift(1, G::OFF_Y + i * NZ + k, -cy);
        if (j == NY - 1) lift(1, G::OFF_Y + G::NFY + i * NZ + k, cy);
    }
    if (k == 0) lift(2, G::OFF_Z + i * NY + j, -cz);
    if (k == NZ - 1) lift(2, G::OFF_Z + G::NFZ + i * NY + j, cz);
    float* out = a.Gout + e * 12 * NP + t;
#pragma unroll
    for (int r = 0; r < 3; r++) {
        out[tidx(r, 0) * NP] = d[r].x;
        out[tidx(r, 1) * NP] = d[r].y;
        out[tidx(r, 2) * NP] = d[r].z;
        out[(9 + r) * NP] = d[r].w;
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
struct LaunchCfg {
    bool visc, tc, persist, gen;
    int pgrid[4];
};

template <int NX, int NY, int NZ, bool VISC, bool TC, bool PERSIST>
void launch_stage_v(const StageArgs& a, int stage, cudaStream_t st, const LaunchCfg& c) {
    using G = Geo<NX, NY, NZ>;
    constexpr size_t SMEM = PERSIST ? StageSmem<NX, NY, NZ>::BYTES_P : StageSmem<NX, NY, NZ, TC>::BYTES;
    int64_t g = a.n_elem;
    if (PERSIST && c.pgrid[stage] > 0 && c.pgrid[stage] < g) g = c.pgrid[stage];
    const unsigned grid = (unsigned)g;
    switch (stage) {
        case 0: k_mixed_stage<NX, NY, NZ, 0, VISC, TC, PERSIST><<<grid, G::BLOCK, SMEM, st>>>(a); break;
        case 1: k_mixed_stage<NX, NY, NZ, 1, VISC, TC, PERSIST><<<grid, G::BLOCK, SMEM, st>>>(a); break;
        case 2: k_mixed_stage<NX, NY, NZ, 2, VISC, TC, PERSIST><<<grid, G::BLOCK, SMEM, st>>>(a); break;
        default: k_mixed_stage<NX, NY, NZ, 3, VISC, TC, PERSIST><<<grid, G::BLOCK, SMEM, st>>>(a); break;
    }
}

/* the tensor-core line sums exist for order 7 only; persistent CTAs for the
 * inviscid kernels of up to 256 threads (order 7's 64 KB of shared memory
 * leaves no room for the staging area) */
template <int NX, int NY, int NZ>
constexpr bool tc_dims() {
    return NX == 8 && NY == 8 && NZ == 8;
}
template <int NX, int NY, int NZ>
constexpr bool persist_dims() {
    return Geo<NX, NY, NZ>::BLOCK <= 256;
}

template <int NX, int NY, int NZ, bool VISC>
void launch_stage_tc(const StageArgs& a, int stage, cudaStream_t st, const LaunchCfg& c) {
    if constexpr (tc_dims<NX, NY, NZ>()) {
        if (c.tc) {
            launch_stage_v<NX, NY, NZ, VISC, true, false>(a, stage, st, c);
            return;
        }
    }
    if constexpr (!VISC && persist_dims<NX, NY, NZ>()) {
        if (c.persist) {
            launch_stage_v<NX, NY, NZ, false, false, true>(a, stage, st, c);
            return;
        }
    }
    launch_stage_v<NX, NY, NZ, VISC, false, false>(a, stage, st, c);
}

/* one stage; viscous runs first form the gradients of the stage state */
template <int NX, int NY, int NZ>
int launch_stage(const StageArgs& a, int stage, cudaStream_t st, const LaunchCfg& c) {
    using G = Geo<NX, NY, NZ>;
    if (c.gen) {
        /* general geometry */
        const unsigned grid = (unsigned)a.n_elem;
        if (c.visc) {
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
    if (!c.visc) {
        launch_stage_tc<NX, NY, NZ, false>(a, stage, st, c);
        return (int)cudaGetLastError();
    }
    launch_stage_tc<NX, NY, NZ, true>(a, stage, st, c);
    return (int)cudaGetLastError();
}

/* viscous runs: the gradients of the stage state, before the stage */
template <int NX, int NY, int NZ>
int launch_grad(const StageArgs& a, int stage, cudaStream_t st, const LaunchCfg& c) {
    using G = Geo<NX, NY, NZ>;
    const unsigned grid = (unsigned)a.n_elem;
    constexpr size_t gs = grad_smem<NX, NY, NZ>();
    if (c.gen) {
        if (stage <= 1) k_mixed_grad_gen<NX, NY, NZ, 1><<<grid, G::BLOCK, gs, st>>>(a);
        else k_mixed_grad_gen<NX, NY, NZ, 2><<<grid, G::BLOCK, gs, st>>>(a);
    } else {
        if (stage <= 1) k_mixed_grad<NX, NY, NZ, 1><<<grid, G::BLOCK, gs, st>>>(a);
        else k_mixed_grad<NX, NY, NZ, 2><<<grid, G::BLOCK, gs, st>>>(a);
    }
    return (int)cudaGetLastError();
}

template <int NX, int NY, int NZ, bool VISC, bool TC, bool PERSIST>
int set_smem(int stage) {
    constexpr int SMEM = (int)(PERSIST ? StageSmem<NX, NY, NZ>::BYTES_P : StageSmem<NX, NY, NZ, TC>::BYTES);
    if (SMEM <= 48 * 1024) return 0;
    const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
    switch (stage) {
        case 0: return (int)cudaFuncSetAttribute(k_mixed_stage<NX, NY, NZ, 0, VISC, TC, PERSIST>, at, SMEM);
        case 1: return (int)cudaFuncSetAttribute(k_mixed_stage<NX, NY, NZ, 1, VISC, TC, PERSIST>, at, SMEM);
        case 2: return (int)cudaFuncSetAttribute(k_mixed_stage<NX, NY, NZ, 2, VISC, TC, PERSIST>, at, SMEM);
        default: return (int)cudaFuncSetAttribute(k_mixed_stage<NX, NY, NZ, 3, VISC, TC, PERSIST>, at, SMEM);
    }
}

/* resident CTAs of a persistent stage kernel on the whole GPU */
template <int NX, int NY, int NZ, int STAGE>
int persist_grid() {
    int per_sm = 0, dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, k_mixed_stage<NX, NY, NZ, STAGE, false, false, true>, Geo<NX, NY, NZ>::BLOCK,
            StageSmem<NX, NY, NZ>::BYTES_P) != cudaSuccess)
        return 0;
    return per_sm * sms;
}

template <int NX, int NY, int NZ>
int prepare_stage(LaunchCfg* c) {
    int e = 0;
    for (int st = 0; st < 4 && !e; st++) {
        e = set_smem<NX, NY, NZ, false, false, false>(st);
        if (!e) e = set_smem<NX, NY, NZ, true, false, false>(st);
        if constexpr (tc_dims<NX, NY, NZ>()) {
            if (!e) e = set_smem<NX, NY, NZ, false, true, false>(st);
            if (!e) e = set_smem<NX, NY, NZ, true, true, false>(st);
        }
        if constexpr (persist_dims<NX, NY, NZ>()) {
            if (!e) e = set_smem<NX, NY, NZ, false, false, true>(st);
        }
    }
    if constexpr (persist_dims<NX, NY, NZ>()) {
        c->pgrid[0] = persist_grid<NX, NY, NZ, 0>();
        c->pgrid[1] = persist_grid<NX, NY, NZ, 1>();
        c->pgrid[2] = persist_grid<NX, NY, NZ, 2>();
        c->pgrid[3] = persist_grid<NX, NY, NZ, 3>();
        if (!c->pgrid[0] || !c->pgrid[1] || !c->pgrid[2] || !c->pgrid[3]) c->persist = false;
    } else {
        c->persist = false;
    }
    {
        constexpr int GS = (int)GenSmem<NX, NY, NZ>::BYTES;
        constexpr int GSV = (int)GenSmem<NX, NY, NZ, true>::BYTES;
        const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
        if (!e && GS > 48 * 1024) {
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
    }
    constexpr size_t gs = grad_smem<NX, NY, NZ>();
    const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
    if (!e && gs > 48 * 1024) {
        e = (int)cudaFuncSetAttribute(k_mixed_grad<NX, NY, NZ, 1>, at, (int)gs);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_grad<NX, NY, NZ, 2>, at, (int)gs);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_grad_gen<NX, NY, NZ, 1>, at, (int)gs);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_grad_gen<NX, NY, NZ, 2>, at, (int)gs);
    }
    return e;
}

}  // namespace

/* dispatch on the supported node counts per direction (also used by the
 * adjoint translation unit) */
#define NSEM_MIXED_DIMS(X)  X(5, 5, 5) X(8, 8, 8) X(4, 4, 4) X(5, 1, 5) X(4, 1, 4)

bool nsem_mixed_supported(int nx, int ny, int nz) {
#define NSEM_SUP(A, B, C) if (nx == A && ny == B && nz == C) return true;
    NSEM_MIXED_DIMS(NSEM_SUP)
#undef NSEM_SUP
    return false;
}

namespace {

int prepare(int nx, int ny, int nz, LaunchCfg* c) {
#define NSEM_PREP(A, B, C) if (nx == A && ny == B && nz == C) return prepare_stage<A, B, C>(c);
    NSEM_MIXED_DIMS(NSEM_PREP)
#undef NSEM_PREP
    return (int)cudaErrorNotSupported;
}

int dispatch_stage(int nx, int ny, int nz, const StageArgs& a, int stage, cudaStream_t st,
                   const LaunchCfg& c) {
#define NSEM_DISP(A, B, C) \
    if (nx == A && ny == B && nz == C) return launch_stage<A, B, C>(a, stage, st, c);
    NSEM_MIXED_DIMS(NSEM_DISP)
#undef NSEM_DISP
    return (int)cudaErrorNotSupported;
}

int dispatch_grad(int nx, int ny, int nz, const StageArgs& a, int stage, cudaStream_t st,
                  const LaunchCfg& c) {
#define NSEM_DISPG(A, B, C) \
    if (nx == A && ny == B && nz == C) return launch_grad<A, B, C>(a, stage, st, c);
    NSEM_MIXED_DIMS(NSEM_DISPG)
#undef NSEM_DISPG
    return (int)cudaErrorNotSupported;
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
    std::vector<int32_t> ment, mnode;
    std::vector<float> mcoef, mgs;
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
            nbr[(int64_t)face * ne + e] = -2 - id;
            ment.resize((size_t)(id + 1) * nfmax * 4, -1);
            mcoef.resize((size_t)(id + 1) * nfmax * 4, 0.0f);
            mgs.resize((size_t)(id + 1) * nfmax * 4, 0.0f);
            mnode.resize((size_t)(id + 1) * nfmax, -1);
            return id;
        };
        /* an entry of a face node: the mortar slot, the flux coefficient and
         * the gradient weight */
        auto add = [&](int32_t mf, int r, int64_t node, int32_t code, double c, double g) -> bool {
            mnode[(size_t)mf * nfmax + r] = (int32_t)node;
            for (int q = 0; q < 4; q++) {
                const size_t at = ((size_t)mf * nfmax + r) * 4 + q;
                if (ment[at] < 0) {
                    ment[at] = code; mcoef[at] = (float)c; mgs[at] = (float)g;
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
                    if (fnode / NP != cell_f || cnode / NP != cell_c || m->fI[k] != 0.5) {
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
                    bool ok = add(mf_f, in_face(dir_f, c), fnode, ms, (fm == 1 ? 1.0 : -1.0) * sf, gf);
                    loc(cnode, c);
                    ok = ok && add(mf_c, in_face(fix, c), cnode, ms | MX_COARSE,
                                   (fm == 2 ? 1.0 : -1.0) * sc, gc);
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
            !up(&mb->mf_gs, mgs)) {
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
