/*
 * Precision form's discrete adjoint: the kernels' arguments and the device
 * helpers shared by its translation units -- nsem_mixed_adj.cu (axis-aligned
 * elements, host side) and nsem_mixed_adj_gen.cu (inclined and curved elements).
 */
#ifndef NSEM_MIXED_ADJ_CUH
#define NSEM_MIXED_ADJ_CUH

#include <cuda_runtime.h>

#include "nsem_mixed.h"
#include "nsem_mixed_dev.cuh"

namespace nsem_mxa {

using namespace nsem_mx;

struct AdjArgs {
    const float* S;            /* stage base: FP32 shadow of u'^n, [e][5][NP] */
    const float* Din;          /* d2 (R3), d1 (R2), null (R1, R0)             */
    const double* lam;         /* FP64 adjoint state (R3 input, R1 in/out)    */
    double* lam_out;           /* R1                                          */
    const float* Gin;          /* B (R2), C (R1), w (R0)                      */
    float* A;                  /* sbar accumulator (R3 writes, R2 updates, R1 reads) */
    float* Bout;               /* R3: d2bar; R2: d1bar (C); R0: xbar          */
    const int32_t* nbr;
    const float* J;
    const int32_t* layer;
    const float* Qg;
    const float* bg;
    int64_t n_elem;
    float dt, gamma, gR, g[3];
    float lift[3];
    float eos[6];
    float qc[3][8][8];         /* line-sum weights Q_d[a][m] (constant-bank operands) */
    /* viscous runs: the stage state's gradients [e][12][NP] (forward), the
     * gradient adjoints [e][12][NP] and the first pass's state adjoint
     * [e][5][NP] (between the two passes), mu / rho, mu / (rho Pr), T0 and the
     * derivative tables D_d[a][m] = l_m'(x_a) */
    const float* Gv;
    float* GB;
    float* XB;
    float nu, nu_pr, T0;
    float dc[3][8][8];
    /* inclined and curved elements: per node Jinv cV (9) and 1/cV, per face
     * node the outward weighted normal */
    const float* Jg;
    const float* Fn;
};

template <int NX, int NY, int NZ>
struct AdjSmem {
    using G = Geo<NX, NY, NZ>;
    static constexpr int NP = G::NP, NFS = G::NFS;
    /* floats: gbar GB[5][NP]; the transposed line sums, line-major per
     * direction; own values P[3][NP] (x4) and Theta'; face results Fa4[NFS]
     * (x4) + Fa1[NFS] (merged into Fbar_n), Xd4[NFS] (x4) + Xd1[NFS] (added
     * to xbar); metric */
    static constexpr int OFF_R = (5 * NP + 3) / 4 * 4;
    static constexpr int OFF_P = (OFF_R + line_floats<NX, NY, NZ>() + 3) / 4 * 4;
    static constexpr int OFF_T = OFF_P + 12 * NP;
    static constexpr int OFF_FA4 = (OFF_T + NP + 3) / 4 * 4;
    static constexpr int OFF_FA1 = OFF_FA4 + 4 * NFS;
    static constexpr int OFF_XD4 = (OFF_FA1 + NFS + 3) / 4 * 4;
    static constexpr int OFF_XD1 = OFF_XD4 + 4 * NFS;
    static constexpr int OFF_META = OFF_XD1 + NFS;
    static constexpr size_t BYTES = sizeof(float) * (OFF_META + 4);
};

template <int NX, int NY, int NZ>
constexpr int adj_min_blocks() {
    /* order 7 (512 threads): two CTAs with 64 registers, no spills */
    return min_blocks(Geo<NX, NY, NZ>::BLOCK >= 512 ? 2 : 6, Geo<NX, NY, NZ>::BLOCK,
                      AdjSmem<NX, NY, NZ>::BYTES);
}

/* Transposed line sums as a line transform: for direction D, line l and
 * variable v (thread r = v NL + l), R(b) = sum_m Q_D[m][b] gbar(m) over the
 * line's nodes, written line-major (the forward's layout) for the node
 * threads to read.  gbar is read from its node-ordered rows. */
template <int NX, int NY, int NZ, int D>
__device__ __forceinline__ void line_transform_t(const float* gbn, float* R, const AdjArgs& a, int t) {
    using LL = LineLay<NX, NY, NZ, D>;
    constexpr int NP = LL::NP, NL = LL::NL, n = LL::n;
    constexpr int BLOCK = Geo<NX, NY, NZ>::BLOCK;
    float* f = R + LL::BASE;
#pragma unroll 1
    for (int r = t; r < 5 * NL; r += BLOCK) {
        const int v = r / NL, l = r - v * NL;
        /* node of position m on line l: x (m, l), y (l / NZ, m, l % NZ), z (l, m) */
        const int n0 = D == 0 ? l : D == 1 ? (l / NZ) * NY * NZ + (l % NZ) : l * NZ;
        constexpr int ms = D == 0 ? NY * NZ : D == 1 ? NZ : 1;
        float x[n];
#pragma unroll
        for (int m = 0; m < n; m++) x[m] = gbn[v * NP + n0 + m * ms];
#pragma unroll
        for (int b = 0; b < n; b++) {
            float acc = 0.0f;
#pragma unroll
            for (int m = 0; m < n; m++) acc = fmaf(a.qc[D][m][b], x[m], acc);
            f[b * LL::ROW + r] = acc;
        }
    }
}

/* gbar of a node from the stage's input: 2/3 lam (R3), B/4 (R2), C (R1), w (R0) */
template <int RS>
__device__ __forceinline__ void load_gbar(const AdjArgs& a, int64_t o, int np, float* gb) {
#pragma unroll
    for (int v = 0; v < 5; v++) {
        if constexpr (RS == 3) gb[v] = (2.0f / 3.0f) * d2f_rn(__ldg(a.lam + o + v * np));
        else if constexpr (RS == 2) gb[v] = 0.25f * __ldg(a.Gin + o + v * np);
        else gb[v] = __ldg(a.Gin + o + v * np);
    }
}

/* xbar += JF_d(x)^T fb for the volume flux along d:
 *   F_d = (m_d, m_c u_d + p' delta_cd, m_d theta) */
template <int D>
__device__ __forceinline__ void jft(const float* u, float th, float pth, float fa, float fb0,
                                    float fb1, float fb2, float ft, float* xb) {
    const float ud = u[D];
    const float bu = fmaf(fb0, u[0], fmaf(fb1, u[1], fb2 * u[2]));
    const float w = fmaf(ft, th, bu);                 /* b.u + t theta */
    xb[0] = fmaf(-ud, w, xb[0]);
    xb[1] = fmaf(fb0, ud, xb[1]);
    xb[2] = fmaf(fb1, ud, xb[2]);
    xb[3] = fmaf(fb2, ud, xb[3]);
    xb[1 + D] += fa + w;
    const float fbd = D == 0 ? fb0 : D == 1 ? fb1 : fb2;
    xb[4] = fmaf(fbd, pth, fmaf(ft, ud, xb[4]));
}

/* viscous runs, first pass: the volume flux of direction D carries
 * - mu d_r U_D (momentum r) and - (mu / Pr) d_D theta, mu = rho nu, so its
 * adjoint Fbar_D also gives the node's gradient adjoints and, through mu,
 * a density adjoint */
template <int D>
__device__ __forceinline__ void visc_t(const float4& fb, float fb1, const float* gv, float mu,
                                       float mt, float* gbv, float& sm, float& st) {
    gbv[tidx(0, D)] = -mu * fb.y;
    gbv[tidx(1, D)] = -mu * fb.z;
    gbv[tidx(2, D)] = -mu * fb.w;
    gbv[9 + D] = -mt * fb1;
    sm = fmaf(fb.y, gv[tidx(0, D)], fmaf(fb.z, gv[tidx(1, D)], fmaf(fb.w, gv[tidx(2, D)], sm)));
    st = fmaf(fb1, gv[9 + D], st);
}

/* Viscous runs, second pass: the transpose of the gradients of U and
 * theta - T0 (k_mixed_grad) applied to the first pass's gradient adjoints,
 * then the stage combination.  Forward, per node a and axis r:
 *   G_r(a) = J_r sum_m D_r[a_r][m] V_m + sum_faces s (J_r / w_end) (cds - V_a),
 * V = (U, theta - T0) = prim_ut(x), cds = (V_a + V_o) / 2 inside, the wall
 * ghost's value on a wall.  Transpose: the line sums with D_r^T (a line
 * transform, the weights constant operands), and per face node the face
 * term's adjoint sDbar = s (J_r / w_end) Gbar_r(a): -sDbar / 2 to the node and
 * +sDbar / 2 to the neighbour's node -- which this element takes from the
 * neighbour's side of the same face (its gradient adjoints at its face node,
 * its J_r), so no element writes another's adjoint.  On a wall the ghost's
 * transpose (the SYMMETRY rescaling) replaces the neighbour's half. */
template <int NX, int NY, int NZ>
struct AdjGradSmem {
    using G = Geo<NX, NY, NZ>;
    static constexpr int NP = G::NP, NFS = G::NFS;
    /* floats: gradient-adjoint rows, line-major per axis (4 of the 5 slots);
     * V [NP] (x4); face contributions [NFS] (x4); metric */
    static constexpr int OFF_V = (line_floats<NX, NY, NZ>() + 3) / 4 * 4;
    static constexpr int OFF_F = OFF_V + 4 * NP;
    static constexpr int OFF_META = OFF_F + 4 * NFS;
    static constexpr size_t BYTES = sizeof(float) * (OFF_META + 4);
};

/* the transposed line sums of the gradient rows of axis D (4 quantities) */
template <int NX, int NY, int NZ, int D>
__device__ __forceinline__ void grad_transform_t(float* R, const AdjArgs& a, int t) {
    using LL = LineLay<NX, NY, NZ, D>;
    constexpr int BLOCK = Geo<NX, NY, NZ>::BLOCK;
    float* f = R + LL::BASE;
#pragma unroll 1
    for (int r = t; r < 4 * LL::NL; r += BLOCK) {
        float in[LL::n];
#pragma unroll
        for (int m = 0; m < LL::n; m++) in[m] = f[m * LL::ROW + r];
#pragma unroll
        for (int b = 0; b < LL::n; b++) {
            float acc = 0.0f;
#pragma unroll
            for (int m = 0; m < LL::n; m++) acc = fmaf(a.dc[D][m][b], in[m], acc);
            f[b * LL::ROW + r] = acc;
        }
    }
}

/* general-geometry kernels (nsem_mixed_adj_gen.cu), dispatched on the node
 * counts per direction; passes (viscous runs): bit 0 the flux transposes,
 * bit 1 the gradients' transpose with the stage combination */
int launch_adj_general(int nx, int ny, int nz, const AdjArgs& a, int rs, cudaStream_t st,
                       int passes);
int prepare_adj_general(int nx, int ny, int nz);

}  // namespace nsem_mxa

#endif
