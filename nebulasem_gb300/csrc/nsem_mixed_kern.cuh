/*
 * Precision form: the stage kernels' arguments and the layouts and device
 * helpers shared by its translation units -- nsem_mixed.cu (setup, mortar and
 * layout kernels, launches), nsem_mixed_stage.cu (axis-aligned affine
 * elements) and nsem_mixed_gen.cu (inclined and curved elements).
 */
#ifndef NSEM_MIXED_KERN_CUH
#define NSEM_MIXED_KERN_CUH

#include <cuda_runtime.h>

#include <cstdint>

#include "nsem_mixed.h"
#include "nsem_mixed_dev.cuh"

namespace nsem_mx {

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
    /* line-sum weights Q_d[a][m] as kernel parameters: read with
     * compile-time indices they are constant-bank operands of the FMAs */
    float qc[3][8][8];
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

/* the in-place line transform of the stage kernels (layout: LineLay) */
template <int NX, int NY, int NZ, int D>
__device__ __forceinline__ void line_transform(float* F, const StageArgs& a, int t) {
    using LL = LineLay<NX, NY, NZ, D>;
    constexpr int BLOCK = Geo<NX, NY, NZ>::BLOCK;
    float* f = F + LL::BASE;
#pragma unroll 1
    for (int r = t; r < 5 * LL::NL; r += BLOCK) {
        float in[LL::n];
#pragma unroll
        for (int m = 0; m < LL::n; m++) in[m] = f[m * LL::ROW + r];
#pragma unroll
        for (int q = 0; q < LL::n; q++) {
            float acc = 0.0f;
#pragma unroll
            for (int m = 0; m < LL::n; m++) acc = fmaf(a.qc[D][q][m], in[m], acc);
            f[q * LL::ROW + r] = acc;
        }
    }
}

/* index of face slot t within its face: x (j, k), y (i, k), z (i, j) */
template <int NX, int NY, int NZ>
__device__ __forceinline__ int face_local(int t) {
    using G = Geo<NX, NY, NZ>;
    if (t < G::OFF_Y) return t % G::NFX;
    if (t < G::OFF_Z) return (t - G::OFF_Y) % G::NFY;
    return (t - G::OFF_Z) % G::NFZ;
}

/* dynamic shared memory of the gradient kernels: the nodes' U and theta,
 * the face values, the derivative tables */
template <int NX, int NY, int NZ>
constexpr size_t grad_smem() {
    using G = Geo<NX, NY, NZ>;
    return sizeof(float4) * (G::NP + G::NFS) + sizeof(float) * (QTAB + 4);
}

struct LaunchCfg {
    bool visc, tc, persist, gen;
    int pgrid[4];
};

/* per translation unit: the kernels' shared-memory attributes (and the
 * persistent kernels' grids), the stage launches and the gradient launches
 * of viscous runs, each dispatched on the node counts per direction */
int prepare_aligned(int nx, int ny, int nz, LaunchCfg* c);
int prepare_general(int nx, int ny, int nz);
int launch_stage_aligned(int nx, int ny, int nz, const StageArgs& a, int stage, cudaStream_t st,
                         const LaunchCfg& c);
int launch_stage_general(int nx, int ny, int nz, const StageArgs& a, int stage, cudaStream_t st,
                         bool visc);
int launch_grad_aligned(int nx, int ny, int nz, const StageArgs& a, int stage, cudaStream_t st);
int launch_grad_general(int nx, int ny, int nz, const StageArgs& a, int stage, cudaStream_t st);

}  // namespace nsem_mx

#endif
