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
 *   phase 1 (thread per node): stage state -> primitives, volume fluxes in smem;
 *   phase 2 (thread per face node, all six faces): Rusanov flux with the
 *            neighbour's trace read from its stage state (both elements of a
 *            face evaluate the same expression with sides swapped);
 *   phase 3 (thread per node): weak volume term as tensor-product line sums
 *            with Q = W^-1 D^T W, surface lift, buoyancy, RK update.
 * Geometry: axis-aligned affine elements (the rising-bubble boxes); per
 * element the metric diagonal and the six neighbours, per z-layer the
 * background.  Discretisation identical to the plain form (same Rusanov
 * speed and jump, same symmetry ghost velocity, same weak form).
 */
#include <cuda_runtime.h>

#include <cmath>
#include <map>
#include <vector>

#include "nsem_mixed.h"

namespace {

constexpr int MAXN = NSEM_MAX_NPD;

struct MixedTabs {
    float Q[3][MAXN * MAXN];   /* Q_d[a][m] = D_d[m][a] w_m / w_a */
    float lift[3];             /* 1 / w_end per direction          */
};

struct StageArgs {
    const double* U[5];        /* u'^n (FP64)                        */
    const float* Din[5];       /* previous stage increment (or null) */
    float* Dout[5];            /* stage increment out (stages 1, 2)  */
    double* Unew[5];           /* u'^{n+1} (stage 3)                 */
    double* L[5];              /* tendency out (stage 0)             */
    const int32_t* nbr;        /* [6][n_elem]                        */
    const float* J;            /* [3][n_elem]                        */
    const int32_t* layer;      /* [n_elem]                           */
    const float* bg;           /* [layers][3][NP]: rho_ref, Theta_ref, p_ref */
    int64_t n_elem;
    float dt, gamma, gR, g[3];
    int stage;
    uint32_t* status;
};

template <int NX, int NY, int NZ>
struct Geo {
    static constexpr int NP = NX * NY * NZ;
    static constexpr bool HAS_Y = NY > 1;
    static constexpr int NFX = NY * NZ, NFY = NX * NZ, NFZ = NX * NY;
    static constexpr int OFF_X = 0;
    static constexpr int OFF_Y = 2 * NFX;
    static constexpr int OFF_Z = 2 * NFX + (HAS_Y ? 2 * NFY : 0);
    static constexpr int NFS = OFF_Z + 2 * NFZ;
    static constexpr int BLOCK = ((NP > NFS ? NP : NFS) + 31) / 32 * 32;
    /* dynamic shared memory: F[3][5][NP], P[13][NP], FF[5][NFS], Q[3][MAXN^2], meta[4] */
    static constexpr size_t SMEM =
        sizeof(float) * (15 * NP + 13 * NP + 5 * NFS + 3 * NSEM_MAX_NPD * NSEM_MAX_NPD + 4);
};

/* (1 + d)^gamma - 1, accurate relative to d */
__device__ __forceinline__ float pow1m(float d, float gamma) {
    return expm1f(gamma * log1pf(d));
}

struct Prim {
    float rp, m0, m1, m2, tp;   /* perturbation conserved */
    float rho, u0, u1, u2, th, pp, c, umag;
};

__device__ __forceinline__ Prim make_prim(float rp, float m0, float m1, float m2, float tp,
                                          float rref, float tref, float pref, float gamma,
                                          float gR) {
    Prim p;
    p.rp = rp; p.m0 = m0; p.m1 = m1; p.m2 = m2; p.tp = tp;
    p.rho = rref + rp;
    const float inv = 1.0f / p.rho;
    p.u0 = m0 * inv; p.u1 = m1 * inv; p.u2 = m2 * inv;
    p.th = (tref + tp) * inv;
    p.pp = pref * pow1m(tp / tref, gamma);
    p.c = sqrtf(gR * p.th);
    p.umag = sqrtf(p.u0 * p.u0 + p.u1 * p.u1 + p.u2 * p.u2);
    return p;
}

template <int NX, int NY, int NZ>
__global__ void __launch_bounds__(Geo<NX, NY, NZ>::BLOCK)
k_mixed_stage(StageArgs a, MixedTabs tab) {
    using G = Geo<NX, NY, NZ>;
    constexpr int NP = G::NP;
    constexpr int NFS = G::NFS;
    /* shared: volume fluxes F[dir][var][node], primitives for the faces,
     * face fluxes, tables */
    extern __shared__ float smem[];
    float(*sF)[5][NP] = reinterpret_cast<float(*)[5][NP]>(smem);
    float(*sP)[NP] = reinterpret_cast<float(*)[NP]>(smem + 15 * NP);
    float(*sFF)[NFS] = reinterpret_cast<float(*)[NFS]>(smem + 28 * NP);
    float(*sQ)[MAXN * MAXN] = reinterpret_cast<float(*)[MAXN * MAXN]>(smem + 28 * NP + 5 * NFS);
    float* sMeta = smem + 28 * NP + 5 * NFS + 3 * MAXN * MAXN;

    const int t = threadIdx.x;
    const int64_t e = blockIdx.x;
    for (int q = t; q < 3 * MAXN * MAXN; q += blockDim.x) (&sQ[0][0])[q] = (&tab.Q[0][0])[q];
    if (t < 3) sMeta[t] = a.J[(int64_t)t * a.n_elem + e];

    const int lay = a.layer[e];
    const float* bg = a.bg + (int64_t)lay * 3 * NP;

    /* phase 1: own node */
    if (t < NP) {
        const int64_t n = e * NP + t;
        float s[5];
        for (int v = 0; v < 5; v++) {
            float x = (float)a.U[v][n];
            if (a.Din[0]) x += a.Din[v][n];
            s[v] = x;
        }
        const Prim p = make_prim(s[0], s[1], s[2], s[3], s[4], bg[t], bg[NP + t], bg[2 * NP + t],
                                 a.gamma, a.gR);
        sP[0][t] = p.rp; sP[1][t] = p.m0; sP[2][t] = p.m1; sP[3][t] = p.m2; sP[4][t] = p.tp;
        sP[5][t] = p.rho; sP[6][t] = p.u0; sP[7][t] = p.u1; sP[8][t] = p.u2;
        sP[9][t] = p.th; sP[10][t] = p.pp; sP[11][t] = p.c; sP[12][t] = p.umag;
        const float u[3] = {p.u0, p.u1, p.u2};
        const float m[3] = {p.m0, p.m1, p.m2};
        for (int d = 0; d < 3; d++) {
            sF[d][0][t] = m[d];
            sF[d][1][t] = m[0] * u[d] + (d == 0 ? p.pp : 0.0f);
            sF[d][2][t] = m[1] * u[d] + (d == 1 ? p.pp : 0.0f);
            sF[d][3][t] = m[2] * u[d] + (d == 2 ? p.pp : 0.0f);
            sF[d][4][t] = m[d] * p.th;
        }
    }
    __syncthreads();

    /* phase 2: face nodes */
    if (t < NFS) {
        int dir, side, s0, s1;  /* side: 0 low face, 1 high face; (s0,s1) in-face coords */
        if (t < G::OFF_Y) {
            dir = 0; side = t / G::NFX; const int r = t % G::NFX; s0 = r / NZ; s1 = r % NZ;
        } else if (t < G::OFF_Z) {
            dir = 1; const int q = t - G::OFF_Y; side = q / G::NFY; const int r = q % G::NFY;
            s0 = r / NZ; s1 = r % NZ;
        } else {
            dir = 2; const int q = t - G::OFF_Z; side = q / G::NFZ; const int r = q % G::NFZ;
            s0 = r / NY; s1 = r % NY;
        }
        int i, j, k, io, jo, ko;
        if (dir == 0) { i = side ? NX - 1 : 0; j = s0; k = s1; io = side ? 0 : NX - 1; jo = j; ko = k; }
        else if (dir == 1) { i = s0; j = side ? NY - 1 : 0; k = s1; io = i; jo = side ? 0 : NY - 1; ko = k; }
        else { i = s0; j = s1; k = side ? NZ - 1 : 0; io = i; jo = j; ko = side ? 0 : NZ - 1; }
        const int la = (i * NY + j) * NZ + k;
        const int face = 2 * dir + side;
        const int32_t nb = a.nbr[(int64_t)face * a.n_elem + e];
        const float sg = side ? 1.0f : -1.0f;   /* outward normal = sg e_dir */
        Prim S;
        S.rp = sP[0][la]; S.m0 = sP[1][la]; S.m1 = sP[2][la]; S.m2 = sP[3][la]; S.tp = sP[4][la];
        S.rho = sP[5][la]; S.u0 = sP[6][la]; S.u1 = sP[7][la]; S.u2 = sP[8][la];
        S.th = sP[9][la]; S.pp = sP[10][la]; S.c = sP[11][la]; S.umag = sP[12][la];
        Prim O;
        if (nb >= 0) {
            const int lo = (io * NY + jo) * NZ + ko;
            const int64_t n = (int64_t)nb * NP + lo;
            float s[5];
            for (int v = 0; v < 5; v++) {
                float x = (float)a.U[v][n];
                if (a.Din[0]) x += a.Din[v][n];
                s[v] = x;
            }
            const float* bgo = a.bg + (int64_t)a.layer[nb] * 3 * NP;
            O = make_prim(s[0], s[1], s[2], s[3], s[4], bgo[lo], bgo[NP + lo], bgo[2 * NP + lo],
                          a.gamma, a.gR);
        } else {
            /* wall ghost: NEUMANN for rho, theta, p; SYMMETRY velocity
             * (tangential projection rescaled to |U|, tensor.h:486-494) */
            O = S;
            float r[3] = {S.u0, S.u1, S.u2};
            r[dir] = 0.0f;
            const float mr = sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
            if (mr > 1e-7f) {
                const float sc = S.umag / mr;
                r[0] *= sc; r[1] *= sc; r[2] *= sc;
            }
            O.u0 = r[0]; O.u1 = r[1]; O.u2 = r[2];
            O.m0 = O.rho * r[0]; O.m1 = O.rho * r[1]; O.m2 = O.rho * r[2];
            O.umag = sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        }
        const float us[3] = {S.u0, S.u1, S.u2}, uo[3] = {O.u0, O.u1, O.u2};
        const float ms[3] = {S.m0, S.m1, S.m2}, mo[3] = {O.m0, O.m1, O.m2};
        const float uns = sg * us[dir], uno = sg * uo[dir];
        /* face average with the reference's weights (field.h:2888-2890, fI of
         * field.cpp:257-266): 1/2 inside, the ghost value alone on a wall */
        const float ws = (nb >= 0) ? 0.5f : 0.0f, wo = (nb >= 0) ? 0.5f : 1.0f;
        /* sums of two products are rounded explicitly (no contraction), so the
         * two elements of a face get exactly opposite fluxes */
        const float lam = 0.5f * __fadd_rn(__fadd_rn(__fmul_rn(ws, S.umag), __fmul_rn(wo, O.umag)),
                                           __fadd_rn(__fmul_rn(ws, S.c), __fmul_rn(wo, O.c)));
        /* F* . n_out = avg(F) . n_out - lam (q_other - q_self) (normal part only
         * for momentum), field.h:2928-2943 */
        const float fr = __fadd_rn(__fmul_rn(ws, S.rho * uns), __fmul_rn(wo, O.rho * uno)) -
                         lam * (O.rp - S.rp);
        float fm[3];
        for (int c = 0; c < 3; c++) {
            const float pn = (c == dir) ? sg : 0.0f;
            const float fs = __fadd_rn(__fmul_rn(ms[c], uns), __fmul_rn(S.pp, pn));
            const float fo = __fadd_rn(__fmul_rn(mo[c], uno), __fmul_rn(O.pp, pn));
            fm[c] = __fadd_rn(__fmul_rn(ws, fs), __fmul_rn(wo, fo));
        }
        fm[dir] -= lam * (mo[dir] - ms[dir]);
        const float ft = __fadd_rn(__fmul_rn(ws, S.rho * uns * S.th), __fmul_rn(wo, O.rho * uno * O.th)) -
                         lam * (O.tp - S.tp);
        sFF[0][t] = fr; sFF[1][t] = fm[0]; sFF[2][t] = fm[1]; sFF[3][t] = fm[2]; sFF[4][t] = ft;
    }
    __syncthreads();

    /* phase 3: own node residual and update */
    if (t >= NP) return;
    const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
    float Lv[5] = {0, 0, 0, 0, 0};
    {
        float acc[5] = {0, 0, 0, 0, 0};
#pragma unroll
        for (int m = 0; m < NX; m++) {
            const float q = sQ[0][i * MAXN + m];
            const int b = (m * NY + j) * NZ + k;
#pragma unroll
            for (int v = 0; v < 5; v++) acc[v] = fmaf(q, sF[0][v][b], acc[v]);
        }
        const float Jx = sMeta[0];
#pragma unroll
        for (int v = 0; v < 5; v++) Lv[v] = Jx * acc[v];
    }
    if (NY > 1) {
        float acc[5] = {0, 0, 0, 0, 0};
#pragma unroll
        for (int m = 0; m < NY; m++) {
            const float q = sQ[1][j * MAXN + m];
            const int b = (i * NY + m) * NZ + k;
#pragma unroll
            for (int v = 0; v < 5; v++) acc[v] = fmaf(q, sF[1][v][b], acc[v]);
        }
        const float Jy = sMeta[1];
#pragma unroll
        for (int v = 0; v < 5; v++) Lv[v] = fmaf(Jy, acc[v], Lv[v]);
    }
    {
        float acc[5] = {0, 0, 0, 0, 0};
#pragma unroll
        for (int m = 0; m < NZ; m++) {
            const float q = sQ[2][k * MAXN + m];
            const int b = (i * NY + j) * NZ + m;
#pragma unroll
            for (int v = 0; v < 5; v++) acc[v] = fmaf(q, sF[2][v][b], acc[v]);
        }
        const float Jz = sMeta[2];
#pragma unroll
        for (int v = 0; v < 5; v++) Lv[v] = fmaf(Jz, acc[v], Lv[v]);
    }
    /* surface lift: -(J_d / w_end) F*.n_out for each face through the node */
    auto lift = [&](int slot, float coef) {
#pragma unroll
        for (int v = 0; v < 5; v++) Lv[v] = fmaf(-coef, sFF[v][slot], Lv[v]);
    };
    const float cx = sMeta[0] * tab.lift[0], cy = sMeta[1] * tab.lift[1], cz = sMeta[2] * tab.lift[2];
    if (i == 0) lift(G::OFF_X + j * NZ + k, cx);
    if (i == NX - 1) lift(G::OFF_X + G::NFX + j * NZ + k, cx);
    if (NY > 1) {
        if (j == 0) lift(G::OFF_Y + i * NZ + k, cy);
        if (j == NY - 1) lift(G::OFF_Y + G::NFY + i * NZ + k, cy);
    }
    if (k == 0) lift(G::OFF_Z + i * NY + j, cz);
    if (k == NZ - 1) lift(G::OFF_Z + G::NFZ + i * NY + j, cz);
    /* buoyancy (rho - rho_ref) g */
    const float rp = sP[0][t];
    Lv[1] = fmaf(rp, a.g[0], Lv[1]);
    Lv[2] = fmaf(rp, a.g[1], Lv[2]);
    Lv[3] = fmaf(rp, a.g[2], Lv[3]);

    const int64_t n = e * NP + t;
    if (a.stage == 0) {
#pragma unroll
        for (int v = 0; v < 5; v++) a.L[v][n] = (double)Lv[v];
        return;
    }
    const float dt = a.dt;
    if (a.stage == 1) {
#pragma unroll
        for (int v = 0; v < 5; v++) a.Dout[v][n] = dt * Lv[v];
    } else if (a.stage == 2) {
#pragma unroll
        for (int v = 0; v < 5; v++) a.Dout[v][n] = 0.25f * fmaf(dt, Lv[v], a.Din[v][n]);
    } else {
        bool finite = true;
#pragma unroll
        for (int v = 0; v < 5; v++) {
            const float D = (2.0f / 3.0f) * fmaf(dt, Lv[v], a.Din[v][n]);
            const double un = a.U[v][n] + (double)D;
            a.Unew[v][n] = un;
            finite = finite && isfinite(un);
        }
        if (!finite) atomicOr(a.status, NSEM_STATUS_NONFINITE);
    }
}

/* full <-> perturbation state (FP64): u' = u - (rho_ref, 0, 0, 0, rho_ref T0) */
struct Ptr5 {
    double* p[5];
};

__global__ void k_convert(Ptr5 src, Ptr5 dst, const double* rho_ref, double T0, int64_t n,
                          int to_pert) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        /* explicitly rounded: rho_ref T0 must round as on the host (no FMA) */
        const double rr = rho_ref[i];
        const double tr = __dmul_rn(rr, T0);
        if (to_pert) {
            dst.p[0][i] = __dsub_rn(src.p[0][i], rr);
            dst.p[4][i] = __dsub_rn(src.p[4][i], tr);
        } else {
            dst.p[0][i] = __dadd_rn(src.p[0][i], rr);
            dst.p[4][i] = __dadd_rn(src.p[4][i], tr);
        }
        dst.p[1][i] = src.p[1][i];
        dst.p[2][i] = src.p[2][i];
        dst.p[3][i] = src.p[3][i];
    }
}

template <int NX, int NY, int NZ>
int launch_stage(const StageArgs& a, const MixedTabs& t, cudaStream_t st) {
    using G = Geo<NX, NY, NZ>;
    k_mixed_stage<NX, NY, NZ><<<(unsigned)a.n_elem, G::BLOCK, G::SMEM, st>>>(a, t);
    return (int)cudaGetLastError();
}

template <int NX, int NY, int NZ>
int prepare_stage() {
    using G = Geo<NX, NY, NZ>;
    if (G::SMEM <= 48 * 1024) return 0;
    return (int)cudaFuncSetAttribute(k_mixed_stage<NX, NY, NZ>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM);
}

int prepare(int nx, int ny, int nz) {
    if (nx == 5 && ny == 5 && nz == 5) return prepare_stage<5, 5, 5>();
    if (nx == 8 && ny == 8 && nz == 8) return prepare_stage<8, 8, 8>();
    if (nx == 4 && ny == 4 && nz == 4) return prepare_stage<4, 4, 4>();
    if (nx == 5 && ny == 1 && nz == 5) return prepare_stage<5, 1, 5>();
    if (nx == 4 && ny == 1 && nz == 4) return prepare_stage<4, 1, 4>();
    return (int)cudaErrorNotSupported;
}

int dispatch_stage(int nx, int ny, int nz, const StageArgs& a, const MixedTabs& t,
                   cudaStream_t st) {
    if (nx == 5 && ny == 5 && nz == 5) return launch_stage<5, 5, 5>(a, t, st);
    if (nx == 8 && ny == 8 && nz == 8) return launch_stage<8, 8, 8>(a, t, st);
    if (nx == 4 && ny == 4 && nz == 4) return launch_stage<4, 4, 4>(a, t, st);
    if (nx == 5 && ny == 1 && nz == 5) return launch_stage<5, 1, 5>(a, t, st);
    if (nx == 4 && ny == 1 && nz == 4) return launch_stage<4, 1, 4>(a, t, st);
    return (int)cudaErrorNotSupported;
}

bool supported(int nx, int ny, int nz) {
    return (nx == 5 && ny == 5 && nz == 5) || (nx == 8 && ny == 8 && nz == 8) ||
           (nx == 4 && ny == 4 && nz == 4) || (nx == 5 && ny == 1 && nz == 5) ||
           (nx == 4 && ny == 1 && nz == 4);
}

}  // namespace

/* ------------------------------------------------------------------ setup */

nsem_status nsem_mixed_setup(const NsemDev& dev, const nsem_mesh_desc* m, NsemMixedBuf* mb,
                             std::vector<void*>* allocs, std::string& err) {
    mb->ready = false;
    const int NX = m->npx, NY = m->npy, NZ = m->npz;
    if (!supported(NX, NY, NZ)) {
        err = "precision form built for N+1 = 4, 5, 8 per direction (and 2D N+1 = 4, 5)";
        return NSEM_UNSUPPORTED;
    }
    const int64_t NP = (int64_t)NX * NY * NZ;
    const int64_t ne = m->n_elem;
    const int64_t n_int = ne * NP;
    const int64_t n_all = (int64_t)m->n_cells * NP;
    const int npd[3] = {NX, NY, NZ};

    /* per-element diagonal metric; reject non-affine or rotated elements */
    std::vector<float> J(3 * ne);
    for (int64_t e = 0; e < ne; e++) {
        const double* J0 = m->Jinv + 9 * (e * NP);
        const double diag0[3] = {J0[0], J0[1], J0[2]};
        for (int64_t a = 0; a < NP; a++) {
            const double* Ja = m->Jinv + 9 * (e * NP + a);
            for (int c = 0; c < 9; c++) {
                const double ref = (c < 3) ? diag0[c] : 0.0;
                const double scale = std::fabs(diag0[0]) + std::fabs(diag0[1]) + std::fabs(diag0[2]);
                if (std::fabs(Ja[c] - ref) > 1e-9 * scale) {
                    err = "precision form needs axis-aligned affine elements";
                    return NSEM_UNSUPPORTED;
                }
            }
        }
        for (int d = 0; d < 3; d++) J[d * ne + e] = (float)diag0[d];
    }

    /* neighbours from the face slots: element face lists + FO/FN */
    std::vector<int32_t> nbr(6 * ne, -1);
    auto local = [&](int64_t node) { return node % NP; };
    for (int64_t e = 0; e < ne; e++) {
        for (uint32_t f = m->face_idx0[e]; f < m->face_idx1[e]; f++) {
            const int64_t fid = m->all_faces[f];
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
            const int la = (int)local(mine);
            const int ia = la / (NY * NZ), ja = (la / NZ) % NY, ka = la % NZ;
            /* which face of e: the coordinate that is at an end on this face */
            const double* nv = m->fN + 3 * k;
            int dir = 0;
            const double ax = std::fabs(nv[0]), ay = std::fabs(nv[1]), az = std::fabs(nv[2]);
            if (ay > ax && ay > az) dir = 1;
            else if (az > ax && az > ay) dir = 2;
            const int cidx[3] = {ia, ja, ka};
            const int side = (cidx[dir] == npd[dir] - 1 && npd[dir] > 1) ? 1 : 0;
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
                    err = "precision form needs axis-aligned faces";
                    return NSEM_UNSUPPORTED;
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
        std::vector<float> key(3 * NP);
        for (int64_t a = 0; a < NP; a++) {
            const double rr = rref_h[e * NP + a];
            key[a] = (float)rr;
            key[NP + a] = (float)(rr * dev.T0);
            key[2 * NP + a] = (float)pref_h[e * NP + a];
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
    MixedTabs* tabs = new MixedTabs();
    for (int d = 0; d < 3; d++) {
        const int n = npd[d];
        const std::vector<double>& w = wdir[d];
        for (int aa = 0; aa < n; aa++)
            for (int mm = 0; mm < n; mm++)
                tabs->Q[d][aa * MAXN + mm] =
                    (float)(m->dpsi[d][mm * n + aa] * w[mm] / w[aa]);
        tabs->lift[d] = (float)(1.0 / w[0]);
    }
    mb->tabs = tabs;
    mb->tabs_size = sizeof(MixedTabs);

    auto up = [&](auto** ptr, const auto& vec) -> bool {
        using T = typename std::remove_reference<decltype(vec[0])>::type;
        size_t bytes = vec.size() * sizeof(T);
        if (cudaMalloc((void**)ptr, bytes ? bytes : 1) != cudaSuccess) return false;
        allocs->push_back((void*)*ptr);
        return cudaMemcpy(*ptr, vec.data(), bytes, cudaMemcpyHostToDevice) == cudaSuccess;
    };
    if (!up(&mb->nbr, nbr) || !up(&mb->J, J) || !up(&mb->layer, layer) || !up(&mb->bg, bg)) {
        err = "precision form: device allocation failed";
        return NSEM_NO_MEMORY;
    }
    for (int s = 0; s < 2; s++)
        for (int v = 0; v < 5; v++) {
            if (cudaMalloc((void**)&mb->U[s][v], n_int * sizeof(double)) != cudaSuccess ||
                cudaMalloc((void**)&mb->D[s][v], n_int * sizeof(float)) != cudaSuccess) {
                err = "precision form: device allocation failed";
                return NSEM_NO_MEMORY;
            }
            allocs->push_back(mb->U[s][v]);
            allocs->push_back(mb->D[s][v]);
        }
    if (prepare(NX, NY, NZ) != 0) {
        err = "precision form: cannot reserve the kernel's shared memory";
        return NSEM_CUDA_ERROR;
    }
    mb->n_elem = ne;
    mb->npd[0] = NX; mb->npd[1] = NY; mb->npd[2] = NZ;
    mb->n_layers = (int)seen.size();
    mb->ready = true;
    return NSEM_OK;
}

/* ------------------------------------------------------------ launches */

namespace {

StageArgs stage_args(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, int stage, int cur,
                     double dt) {
    StageArgs a{};
    for (int v = 0; v < 5; v++) {
        a.U[v] = mb->U[cur][v];
        a.Din[v] = (stage == 2) ? mb->D[0][v] : (stage == 3) ? mb->D[1][v] : nullptr;
        a.Dout[v] = (stage == 1) ? mb->D[0][v] : (stage == 2) ? mb->D[1][v] : nullptr;
        a.Unew[v] = mb->U[cur ^ 1][v];
        a.L[v] = b->L[v];
    }
    a.nbr = mb->nbr;
    a.J = mb->J;
    a.layer = mb->layer;
    a.bg = mb->bg;
    a.n_elem = mb->n_elem;
    a.dt = (float)dt;
    a.gamma = (float)dev->gamma;
    a.gR = (float)dev->gR;
    for (int c = 0; c < 3; c++) a.g[c] = (float)dev->g[c];
    a.stage = stage;
    a.status = dev->status;
    return a;
}

int launch(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, int stage, int cur, double dt,
           cudaStream_t st) {
    StageArgs a = stage_args(dev, mb, b, stage, cur, dt);
    return dispatch_stage(mb->npd[0], mb->npd[1], mb->npd[2], a, *(const MixedTabs*)mb->tabs, st);
}

int grid_for(int64_t n) {
    int64_t g = (n + 255) / 256;
    if (g > 152 * 8) g = 152 * 8;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

int nsem_mixed_convert(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, int to_pert,
                       void* stream) {
    Ptr5 full, pert;
    for (int v = 0; v < 5; v++) {
        full.p[v] = b->u[v];
        pert.p[v] = mb->U[mb->cur][v];
    }
    if (to_pert)
        k_convert<<<grid_for(dev->n_int), 256, 0, (cudaStream_t)stream>>>(full, pert, dev->rho_ref,
                                                                          dev->T0, dev->n_int, 1);
    else
        k_convert<<<grid_for(dev->n_int), 256, 0, (cudaStream_t)stream>>>(pert, full, dev->rho_ref,
                                                                          dev->T0, dev->n_int, 0);
    return (int)cudaGetLastError();
}

int nsem_mixed_steps(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, const NsemTables*,
                     int nsteps, double dt, void* stream) {
    int cur = mb->cur;
    for (int n = 0; n < nsteps; n++) {
        for (int stage = 1; stage <= 3; stage++) {
            int e = launch(dev, mb, b, stage, cur, dt, (cudaStream_t)stream);
            if (e) return e;
        }
        cur ^= 1;
    }
    return 0;
}

int nsem_mixed_tendency(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, const NsemTables*,
                        void* stream) {
    return launch(dev, mb, b, 0, mb->cur, 0.0, (cudaStream_t)stream);
}

static const char* const k_names[] = {"mixed_stage1", "mixed_stage2", "mixed_stage3", nullptr};
const char* const* nsem_mixed_kernel_names() { return k_names; }
int nsem_mixed_launches_per_step() { return 3; }
int nsem_mixed_launch_class(int k) { return k; }

int nsem_mixed_launch(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, const NsemTables*, int k,
                      int, double dt, void* stream) {
    int e = launch(dev, mb, b, k + 1, mb->cur, dt, (cudaStream_t)stream);
    if (k == 2) mb->cur ^= 1;
    return e;
}
