/*
 * Precision form on axis-aligned affine elements: the fused SSP-RK3 stage
 * kernel k_mixed_stage (FP32 line sums, or TF32 tensor-core line sums at
 * order 7; optional persistent CTAs) and the viscous runs' gradient kernel
 * k_mixed_grad, with their launches.  The algorithm is described in
 * nsem_mixed.cu.
 */
#include <cuda_runtime.h>

#include "nsem_mixed_kern.cuh"

using namespace nsem_mx;

namespace {

template <int NX, int NY, int NZ, bool TC = false>
struct StageSmem {
    using G = Geo<NX, NY, NZ>;
    static constexpr int NP = G::NP, NFS = G::NFS;
    /* floats: volume fluxes, line-major per direction [3][n][5][NL] (tensor-core
     * line sums: F[3][5][TC_NP]); own values P[3][NP] (x4); face fluxes
     * FF4[NFS] (x4) + FF1[NFS]; metric */
    static constexpr int FLUX = TC ? 15 * TC_NP : line_floats<NX, NY, NZ>();
    static constexpr int OFF_P = (FLUX + 3) / 4 * 4;
    static constexpr int OFF_FF4 = OFF_P + 12 * NP;
    static constexpr int OFF_FF1 = OFF_FF4 + 4 * NFS;
    static constexpr int OFF_META = OFF_FF1 + NFS;
    static_assert(OFF_P % 4 == 0 && OFF_FF4 % 4 == 0, "float4 regions must be 16-byte aligned");
    /* tensor-core line sums: the B fragments of Q_d^T pre-split into TF32
     * high and low parts, [3][2][8][8] words after the metric */
    static constexpr int OFF_QTC = OFF_META + 4;
    static constexpr size_t BYTES = sizeof(float) * (OFF_QTC + (TC ? TC_QTAB : 0));
    /* persistent kernels: the next element's stage base, increment and
     * background, staged by asynchronous copies while the current element
     * computes */
    static constexpr int OFF_STG = OFF_META + 4;
    static constexpr size_t BYTES_P = sizeof(float) * (OFF_STG + 14 * NP);
    static_assert(BYTES_P > BYTES || TC, "the persistent layout extends the plain one");
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

/* registers sized for 8 resident CTAs per SM in stages 1-2 and 9 in stage 3,
 * which loads the FP64 state only at the update (measured best on GB300:
 * 152 us at 32^3, against 172 us with the state held in registers at 7 CTAs
 * and 163 us at 8); viscous runs 6, and 5 in stage 3 (its gradients spill at
 * 6) */
#ifndef NSEM_MIXED_MB12
#define NSEM_MIXED_MB12 8
#endif
#ifndef NSEM_MIXED_MB3
#define NSEM_MIXED_MB3 9
#endif
template <int NX, int NY, int NZ, int STAGE, bool VISC, bool PERSIST = false>
constexpr int stage_min_blocks() {
    /* order 7 (512 threads, 64 KB of shared memory): three CTAs, two for the
     * stages that hold more live values (no spills) */
    if (Geo<NX, NY, NZ>::BLOCK >= 512)
        return min_blocks((VISC || STAGE == 0) ? 2 : 3, Geo<NX, NY, NZ>::BLOCK,
                          StageSmem<NX, NY, NZ>::BYTES);
    return min_blocks(VISC ? (STAGE == 3 ? 5 : 6) : (STAGE == 1 || STAGE == 2) ? NSEM_MIXED_MB12 : NSEM_MIXED_MB3,
                      Geo<NX, NY, NZ>::BLOCK,
                      PERSIST ? StageSmem<NX, NY, NZ>::BYTES_P : StageSmem<NX, NY, NZ>::BYTES);
}

/* Strong-form DG gradients of U and theta of a stage state (gradf<true>,
 * field.h:3327-3360) for the viscous fluxes: per node
 *   d_r q = J_r sum_m D_r[a_r][m] q_m  +  (J_r / w_end) (cds(q) - q)  on the
 *   lower (-) / upper (+) face normal to r through the node,
 * cds = (own + neighbour) / 2 inside, the ghost value on a wall (SYMMETRY
 * velocity, NEUMANN theta: cds(theta) - theta = 0 there).  The state is the
 * stage kernel's (FP32 shadow plus the previous increment for SIN >= 2).
 * Output [e][12][NP]: tidx(r, c) = d_r U_c, 9 + r = d_r theta.
 * Written with explicit rounding throughout (no contraction left to the
 * compiler), so any kernel using these helpers forms the same bits. */

/* U = m / rho as the stage kernel forms it, and theta - T0 from the
 * perturbation: the background has theta = T0 (Theta_ref = rho_ref T0), so
 * theta - T0 = (Theta' - T0 rho') / rho -- the same gradient as theta without
 * FP32 cancellation against T0 */
__device__ __forceinline__ float4 prim_ut(const float* s, float rref, float T0) {
    const float inv = rcp_nr(__fadd_rn(rref, s[0]));
    return make_float4(__fmul_rn(s[1], inv), __fmul_rn(s[2], inv), __fmul_rn(s[3], inv),
                       __fmul_rn(__fmaf_rn(-T0, s[0], s[4]), inv));
}

/* the face term cds - own of face node slot t: O the neighbour's values, or
 * (o == nullptr) the wall ghost of the face's axis */
__device__ __forceinline__ float4 cds_minus_own(const float4 S, const float4* O, int dir) {
    float4 c;
    if (O) {
        c = make_float4(__fadd_rn(__fmul_rn(0.5f, S.x), __fmul_rn(0.5f, O->x)),
                        __fadd_rn(__fmul_rn(0.5f, S.y), __fmul_rn(0.5f, O->y)),
                        __fadd_rn(__fmul_rn(0.5f, S.z), __fmul_rn(0.5f, O->z)),
                        __fadd_rn(__fmul_rn(0.5f, S.w), __fmul_rn(0.5f, O->w)));
    } else {
        /* wall ghost: SYMMETRY velocity, NEUMANN theta */
        float r0 = dir == 0 ? 0.0f : S.x;
        float r1 = dir == 1 ? 0.0f : S.y;
        float r2 = dir == 2 ? 0.0f : S.z;
        const float mr = safe_sqrt(__fmaf_rn(r0, r0, __fmaf_rn(r1, r1, __fmul_rn(r2, r2))));
        if (mr > 1e-7f) {
            const float sc =
                __fdiv_rn(safe_sqrt(__fmaf_rn(S.x, S.x, __fmaf_rn(S.y, S.y, __fmul_rn(S.z, S.z)))), mr);
            r0 = __fmul_rn(r0, sc); r1 = __fmul_rn(r1, sc); r2 = __fmul_rn(r2, sc);
        }
        c = make_float4(r0, r1, r2, S.w);
    }
    return make_float4(__fsub_rn(c.x, S.x), __fsub_rn(c.y, S.y), __fsub_rn(c.z, S.z),
                       __fsub_rn(c.w, S.w));
}

/* the gradients of node (i, j, k) from the element's values sV [NP], the
 * face terms sD [NFS] and the derivative tables sDg; out in the 12-entry
 * layout */
template <int NX, int NY, int NZ>
__device__ __forceinline__ void grad_node(int i, int j, int k, const float4* sV, const float4* sD,
                                          const float* sDg, const float* Jd, const float* lift,
                                          float* out) {
    using G = Geo<NX, NY, NZ>;
    float4 d[3];
    {
        float4 acc = make_float4(0, 0, 0, 0);
        const float* q = sDg + i * QS;
#pragma unroll
        for (int m = 0; m < NX; m++) {
            const float4 v = sV[(m * NY + j) * NZ + k];
            acc.x = __fmaf_rn(q[m], v.x, acc.x); acc.y = __fmaf_rn(q[m], v.y, acc.y);
            acc.z = __fmaf_rn(q[m], v.z, acc.z); acc.w = __fmaf_rn(q[m], v.w, acc.w);
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
                acc.x = __fmaf_rn(q[m], v.x, acc.x); acc.y = __fmaf_rn(q[m], v.y, acc.y);
                acc.z = __fmaf_rn(q[m], v.z, acc.z); acc.w = __fmaf_rn(q[m], v.w, acc.w);
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
            acc.x = __fmaf_rn(q[m], v.x, acc.x); acc.y = __fmaf_rn(q[m], v.y, acc.y);
            acc.z = __fmaf_rn(q[m], v.z, acc.z); acc.w = __fmaf_rn(q[m], v.w, acc.w);
        }
        d[2] = acc;
    }
#pragma unroll
    for (int r = 0; r < 3; r++) {
        d[r].x = __fmul_rn(d[r].x, Jd[r]); d[r].y = __fmul_rn(d[r].y, Jd[r]);
        d[r].z = __fmul_rn(d[r].z, Jd[r]); d[r].w = __fmul_rn(d[r].w, Jd[r]);
    }
    /* face terms: + (J_r / w_end) (cds - own) on the upper face, - on the lower */
    auto lf = [&](int r, int slot, float coef) {
        const float4 f = sD[slot];
        d[r].x = __fmaf_rn(coef, f.x, d[r].x); d[r].y = __fmaf_rn(coef, f.y, d[r].y);
        d[r].z = __fmaf_rn(coef, f.z, d[r].z); d[r].w = __fmaf_rn(coef, f.w, d[r].w);
    };
    const float cx = __fmul_rn(Jd[0], lift[0]), cy = __fmul_rn(Jd[1], lift[1]),
                cz = __fmul_rn(Jd[2], lift[2]);
    if (i == 0) lf(0, G::OFF_X + j * NZ + k, -cx);
    if (i == NX - 1) lf(0, G::OFF_X + G::NFX + j * NZ + k, cx);
    if (NY > 1) {
        if (j == 0) lf(1, G::OFF_Y + i * NZ + k, -cy);
        if (j == NY - 1) lf(1, G::OFF_Y + G::NFY + i * NZ + k, cy);
    }
    if (k == 0) lf(2, G::OFF_Z + i * NY + j, -cz);
    if (k == NZ - 1) lf(2, G::OFF_Z + G::NFZ + i * NY + j, cz);
#pragma unroll
    for (int r = 0; r < 3; r++) {
        out[tidx(r, 0)] = d[r].x;
        out[tidx(r, 1)] = d[r].y;
        out[tidx(r, 2)] = d[r].z;
        out[9 + r] = d[r].w;
    }
}

/* phase 2: flux through face node t, seen from the element.  The face's
 * axis is a run-time value (selects, no branches), so a warp whose face
 * nodes lie on faces of two axes runs one instruction stream; the operations
 * and their operands are those of the plain per-axis form, so the two
 * elements of a face still produce exact negatives. */
template <int NX, int NY, int NZ, bool VISC, bool TC>
__device__ __forceinline__ void face_flux(const FaceSlot& fs, int32_t nb, const float* oth,
                                          const float* bgo, const float* gfo, const float* sF,
                                          const float4* sP, const StageArgs& a,
                                          float4& o4, float& o1) {
    constexpr int NP = Geo<NX, NY, NZ>::NP;
    const int dir = fs.dir;
    const bool d0 = dir == 0, d1 = dir == 1, d2 = dir == 2;
    const float sg = fs.side ? 1.0f : -1.0f;   /* outward normal = sg e_dir */
    const float4 P0 = sP[fs.la], P1 = sP[NP + fs.la];
    const float md_s = d0 ? P0.y : d1 ? P0.z : P0.w;
    const float um_s = P1.z, c_s = P1.w;
    if (nb >= 0) {
        float4 A4;
        float A1;
        if constexpr (TC) {
            const int i = fs.la / (NY * NZ), j = (fs.la / NZ) % NY, k = fs.la % NZ;
            const float* f = sF + dir * 5 * TC_NP +
                             (d0 ? tc_idx<0>(i, j, k) : d1 ? tc_idx<1>(i, j, k) : tc_idx<2>(i, j, k));
            A4 = make_float4(f[0], f[TC_NP], f[2 * TC_NP], f[3 * TC_NP]);
            A1 = f[4 * TC_NP];
        } else {
            /* the node's flux row along the face's axis: the face plane's
             * row (first or last) at the node's in-plane index */
            using L0 = LineLay<NX, NY, NZ, 0>;
            using L1 = LineLay<NX, NY, NZ, 1>;
            using L2 = LineLay<NX, NY, NZ, 2>;
            const int row = d0 ? L0::BASE + (fs.side ? NX - 1 : 0) * L0::ROW
                          : d1 ? L1::BASE + (fs.side ? NY - 1 : 0) * L1::ROW
                               : L2::BASE + (fs.side ? NZ - 1 : 0) * L2::ROW;
            const float* f = sF + row + fs.r;
            const int nl = d0 ? L0::NL : d1 ? L1::NL : L2::NL;
            A4 = make_float4(f[0], f[nl], f[2 * nl], f[3 * nl]);
            A1 = f[4 * nl];
        }
        const Pt q = pointwise(oth, bgo, a.eos, a.gamma, a.gR);
        /* the neighbour's volume flux along the axis (vol_flux of its node) */
        const float ud = d0 ? q.u[0] : d1 ? q.u[1] : q.u[2];
        const float mdo = d0 ? oth[1] : d1 ? oth[2] : oth[3];
        float4 B4;
        float B1;
        B4.x = mdo;
        B4.y = __fmaf_rn(oth[1], ud, d0 ? q.pp : 0.0f);
        B4.z = __fmaf_rn(oth[2], ud, d1 ? q.pp : 0.0f);
        B4.w = __fmaf_rn(oth[3], ud, d2 ? q.pp : 0.0f);
        B1 = __fmul_rn(mdo, q.th);
        if constexpr (VISC) {
            /* gfo: the neighbour's d_c U_dir (c = 0..2) and d_dir theta */
            const float mu = __fmul_rn(q.rho, a.nu), mt = __fmul_rn(q.rho, a.nu_pr);
            B4.y = __fmaf_rn(-mu, gfo[0], B4.y);
            B4.z = __fmaf_rn(-mu, gfo[1], B4.z);
            B4.w = __fmaf_rn(-mu, gfo[2], B4.w);
            B1 = __fmaf_rn(-mt, gfo[3], B1);
        }
        const float lam = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(um_s, q.umag), __fadd_rn(c_s, q.c)));
        const float av0 = __fmul_rn(0.5f, __fadd_rn(A4.x, B4.x));
        const float av1 = __fmul_rn(0.5f, __fadd_rn(A4.y, B4.y));
        const float av2 = __fmul_rn(0.5f, __fadd_rn(A4.z, B4.z));
        const float av3 = __fmul_rn(0.5f, __fadd_rn(A4.w, B4.w));
        const float av4 = __fmul_rn(0.5f, __fadd_rn(A1, B1));
        const float jr = __fsub_rn(oth[0], P0.x);
        const float jm = __fsub_rn(mdo, md_s);
        const float jt = __fsub_rn(oth[4], P1.x);
        const float s1 = sg * av1, s2 = sg * av2, s3 = sg * av3;
        o4.x = __fmaf_rn(-lam, jr, sg * av0);
        o4.y = d0 ? __fmaf_rn(-lam, jm, s1) : s1;
        o4.z = d1 ? __fmaf_rn(-lam, jm, s2) : s2;
        o4.w = d2 ? __fmaf_rn(-lam, jm, s3) : s3;
        o1 = __fmaf_rn(-lam, jt, sg * av4);
    } else {
        /* wall ghost: rho, theta, p NEUMANN; SYMMETRY velocity (tangential
         * projection rescaled to |U|, tensor.h:486-494), normal velocity 0.
         * The ghost value alone is the face average (fI = 0 on a wall,
         * field.cpp:257-266), so only the normal momentum flux remains:
         * s p' + lam m_n, lam = (|U_ghost| + c) / 2.  No viscous wall flux
         * (zero ghost gradient). */
        const float4 P2 = sP[2 * NP + fs.la];
        const float r0 = d0 ? 0.0f : P2.x;
        const float r1 = d1 ? 0.0f : P2.y;
        const float r2 = d2 ? 0.0f : P2.z;
        const float mr = safe_sqrt(__fmaf_rn(r0, r0, __fmaf_rn(r1, r1, __fmul_rn(r2, r2))));
        const float um_g = mr > 1e-7f ? um_s : mr;
        const float lam = __fmul_rn(0.5f, __fadd_rn(um_g, c_s));
        const float fn = __fmaf_rn(lam, md_s, sg * P2.w);
        o4 = make_float4(0.0f, d0 ? fn : 0.0f, d1 ? fn : 0.0f, d2 ? fn : 0.0f);
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
    float4* sP = reinterpret_cast<float4*>(smem + SM::OFF_P);     /* [3][NP] */
    float4* sFF4 = reinterpret_cast<float4*>(smem + SM::OFF_FF4); /* [NFS] */
    float* sFF1 = smem + SM::OFF_FF1;                             /* [NFS] */
    float* sMeta = smem + SM::OFF_META;

    const int t = threadIdx.x;
    constexpr bool has_din = STAGE >= 2;
    float* sStg = smem + SM::OFF_STG;                             /* [14][NP] (PERSIST) */
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
            /* u'^n is needed only at the update: inviscid runs fetch it into L2
             * here and load it there (with the increment reloaded from L1/L2),
             * so that neither holds registers through the element and nine
             * CTAs fit per SM; viscous runs (five CTAs either way) hold it */
            const double* u = a.U + e * 5 * NP + t;
            if constexpr (VISC) {
#pragma unroll
                for (int v = 0; v < 5; v++) u64[v] = __ldg(u + v * NP);
            } else {
#pragma unroll
                for (int v = 0; v < 5; v++) asm volatile("prefetch.global.L2 [%0];" ::"l"(u + v * NP));
            }
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
        fs = face_slot<NX, NY, NZ, STAGE == 1 || STAGE == 2>(t);
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
            const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
            auto put = [&](float* f, int nl, const float4& v4, float v1) {
                f[0] = v4.x; f[nl] = v4.y; f[2 * nl] = v4.z; f[3 * nl] = v4.w; f[4 * nl] = v1;
            };
            vol_flux<0, VISC>(own, p, gown, a.nu, a.nu_pr, f4, f1);
            put(smem + LineLay<NX, NY, NZ, 0>::at(i, j, k), LineLay<NX, NY, NZ, 0>::NL, f4, f1);
            if constexpr (G::HAS_Y) {
                vol_flux<1, VISC>(own, p, gown, a.nu, a.nu_pr, f4, f1);
                put(smem + LineLay<NX, NY, NZ, 1>::at(i, j, k), LineLay<NX, NY, NZ, 1>::NL, f4, f1);
            }
            vol_flux<2, VISC>(own, p, gown, a.nu, a.nu_pr, f4, f1);
            put(smem + LineLay<NX, NY, NZ, 2>::at(i, j, k), LineLay<NX, NY, NZ, 2>::NL, f4, f1);
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
        } else {
            face_flux<NX, NY, NZ, VISC, TC>(fs, nb, oth, bgo, gfo, smem, sP, a, o4, o1);
        }
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
    } else {
        line_transform<NX, NY, NZ, 0>(smem, a, t);
        if constexpr (G::HAS_Y) line_transform<NX, NY, NZ, 1>(smem, a, t);
        line_transform<NX, NY, NZ, 2>(smem, a, t);
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
        /* the three directions' line sums at this node, scaled by J_d */
        const float* rx = smem + LineLay<NX, NY, NZ, 0>::at(i, j, k);
        const float* rz = smem + LineLay<NX, NY, NZ, 2>::at(i, j, k);
        constexpr int NLX = LineLay<NX, NY, NZ, 0>::NL, NLZ = LineLay<NX, NY, NZ, 2>::NL;
        const float Jx = sMeta[0], Jz = sMeta[2];
        float Lt[5];
#pragma unroll
        for (int v = 0; v < 5; v++) Lt[v] = Jx * rx[v * NLX];
        if constexpr (G::HAS_Y) {
            const float* ry = smem + LineLay<NX, NY, NZ, 1>::at(i, j, k);
            constexpr int NLY = LineLay<NX, NY, NZ, 1>::NL;
            const float Jy = sMeta[1];
#pragma unroll
            for (int v = 0; v < 5; v++) Lt[v] = fmaf(Jy, ry[v * NLY], Lt[v]);
        }
#pragma unroll
        for (int v = 0; v < 5; v++) Lt[v] = fmaf(Jz, rz[v * NLZ], Lt[v]);
        L0 = Lt[0]; L1 = Lt[1]; L2 = Lt[2]; L3 = Lt[3]; L4 = Lt[4];
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
            const float D = (2.0f / 3.0f) * fmaf(dt, Lv[v], VISC ? din[v] : __ldg(a.Din + o + v * NP));
            const double un = (VISC ? u64[v] : __ldg(a.U + o + v * NP)) + f2d(D);
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

    if (t < NP) sV[t] = prim_ut(own, bgs0, a.T0);
    __syncthreads();

    if (t < NFS && nb <= -2) {
        /* a face on a 2:1 mortar: the projected values from the mortar kernels */
        const float* gf = a.MF + ((int64_t)(-2 - nb) * MF_ROWS + 5) * a.nfmax + face_local<NX, NY, NZ>(t);
        sD[t] = make_float4(__ldg(gf), __ldg(gf + a.nfmax), __ldg(gf + 2 * a.nfmax),
                            __ldg(gf + 3 * a.nfmax));
    } else if (t < NFS) {
        const float4 O = nb >= 0 ? prim_ut(oth, bgo0, a.T0) : make_float4(0, 0, 0, 0);
        sD[t] = cds_minus_own(sV[fs.la], nb >= 0 ? &O : nullptr, fs.dir);
    }
    __syncthreads();

    if (t >= NP) return;
    const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
    float g12[12];
    grad_node<NX, NY, NZ>(i, j, k, sV, sD, sDg, sJ, a.lift, g12);
    float* out = a.Gout + e * 12 * NP + t;
#pragma unroll
    for (int c = 0; c < 12; c++) out[c * NP] = g12[c];
}

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

template <int NX, int NY, int NZ>
int launch_stage(const StageArgs& a, int stage, cudaStream_t st, const LaunchCfg& c) {
    if (c.visc) launch_stage_tc<NX, NY, NZ, true>(a, stage, st, c);
    else launch_stage_tc<NX, NY, NZ, false>(a, stage, st, c);
    return (int)cudaGetLastError();
}

/* viscous runs: the gradients of the stage state, before the stage */
template <int NX, int NY, int NZ>
int launch_grad(const StageArgs& a, int stage, cudaStream_t st) {
    using G = Geo<NX, NY, NZ>;
    const unsigned grid = (unsigned)a.n_elem;
    constexpr size_t gs = grad_smem<NX, NY, NZ>();
    if (stage <= 1) k_mixed_grad<NX, NY, NZ, 1><<<grid, G::BLOCK, gs, st>>>(a);
    else k_mixed_grad<NX, NY, NZ, 2><<<grid, G::BLOCK, gs, st>>>(a);
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
    constexpr size_t gs = grad_smem<NX, NY, NZ>();
    const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
    if (!e && gs > 48 * 1024) {
        e = (int)cudaFuncSetAttribute(k_mixed_grad<NX, NY, NZ, 1>, at, (int)gs);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_grad<NX, NY, NZ, 2>, at, (int)gs);
    }
    return e;
}

}  // namespace

namespace nsem_mx {

int prepare_aligned(int nx, int ny, int nz, LaunchCfg* c) {
#define NSEM_PREP(A, B, C) if (nx == A && ny == B && nz == C) return prepare_stage<A, B, C>(c);
    NSEM_MIXED_DIMS(NSEM_PREP)
#undef NSEM_PREP
    return (int)cudaErrorNotSupported;
}

int launch_stage_aligned(int nx, int ny, int nz, const StageArgs& a, int stage, cudaStream_t st,
                         const LaunchCfg& c) {
#define NSEM_DISP(A, B, C) \
    if (nx == A && ny == B && nz == C) return launch_stage<A, B, C>(a, stage, st, c);
    NSEM_MIXED_DIMS(NSEM_DISP)
#undef NSEM_DISP
    return (int)cudaErrorNotSupported;
}

int launch_grad_aligned(int nx, int ny, int nz, const StageArgs& a, int stage, cudaStream_t st) {
#define NSEM_DISPG(A, B, C) \
    if (nx == A && ny == B && nz == C) return launch_grad<A, B, C>(a, stage, st);
    NSEM_MIXED_DIMS(NSEM_DISPG)
#undef NSEM_DISPG
    return (int)cudaErrorNotSupported;
}

}  // namespace nsem_mx
