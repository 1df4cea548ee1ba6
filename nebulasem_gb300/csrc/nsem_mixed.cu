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
 *
 * Artificial viscosity (diffusion YES, euler.cpp:189-190, 232, 250): a
 * gradient kernel per stage forms the strong-form DG gradients of U and
 * theta of the stage state (gradf<true>, field.h:3327-3360: line derivatives
 * plus the face terms (cds - own) lifted by J/w_end; zero gradient on the
 * wall ghosts) into FP32 arrays, and the stage kernel subtracts mu grad U and
 * (mu / Pr) grad theta, mu = rho nu, from the volume and face fluxes.
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
    const double* U[5];        /* u'^n (FP64)                             */
    const float* U32[5];       /* FP32 shadow of u'^n                     */
    const float* Din[5];       /* previous stage increment (or null)      */
    float* Dout[5];            /* stage increment out (stages 1, 2)       */
    double* Unew[5];           /* u'^{n+1} (stage 3)                      */
    float* U32new[5];          /* its FP32 shadow (stage 3)               */
    double* L[5];              /* tendency out (stage 0)                  */
    const int32_t* nbr;        /* [6][n_elem]                             */
    const float* J;            /* [3][n_elem]                             */
    const int32_t* layer;      /* [n_elem]                                */
    const float* Qg;           /* device copy of MixedTabs::Q (coalesced loads) */
    const float* Dg;           /* derivative tables (gradient kernel)     */
    const float* Gv[12];       /* viscous runs: grad U (XX..ZX), grad theta */
    float* Gout[12];           /* gradient kernel output                   */
    float nu, nu_pr;           /* viscous runs: nu, nu / Pr                */
    float T0;                  /* background potential temperature        */
    const float* bg;           /* [layers][3][NP]: rho_ref, Theta_ref, p_ref */
    int64_t n_elem;
    float dt, gamma, gR, g[3];
    float eos[6];              /* binomial coefficients C(gamma, k), k = 1..6 */
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
    /* dynamic shared memory (floats): flux F4[3][NP] (x4) + F1[3][NP],
     * primitives P[4][NP] (x4), face fluxes FF4[NFS] (x4) + FF1[NFS],
     * Q[3][MAXN^2], meta[4] */
    /* every float4 region starts on a 16-byte boundary (offsets in floats
     * rounded up to a multiple of 4) */
    static constexpr int OFF_F1 = 12 * NP;
    static constexpr int OFF_P = (15 * NP + 3) / 4 * 4;
    static constexpr int OFF_FF4 = OFF_P + 16 * NP;
    static constexpr int OFF_FF1 = OFF_FF4 + 4 * NFS;
    static constexpr int OFF_Q = OFF_FF1 + NFS;
    static constexpr int OFF_META = OFF_Q + 3 * NSEM_MAX_NPD * NSEM_MAX_NPD;
    static_assert(OFF_P % 4 == 0 && OFF_FF4 % 4 == 0, "float4 regions must be 16-byte aligned");
    static constexpr size_t SMEM = sizeof(float) * (OFF_META + 4);
};

/* Exact-rounding conversions on the integer pipes.  GB300 executes F2F
 * conversions on its (narrow) FP64 pipe; these use the ALU instead. */
__device__ __forceinline__ float d2f_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned long long sgn = b & 0x8000000000000000ull;
    const unsigned long long m = b ^ sgn;
    const unsigned long long r = m + 0x0fffffffull + ((m >> 29) & 1ull);  /* round to nearest even */
    unsigned int f = (unsigned int)(r >> 29) - (896u << 23);               /* rebias exponent */
    f = (m < 0x3810000000000000ull) ? 0u : f;                              /* below FLT_MIN: 0 */
    f = (m >= 0x47effffff0000000ull) ? 0x7f800000u : f;                    /* overflow: inf   */
    return __uint_as_float(f | (unsigned int)(sgn >> 32));
}

__device__ __forceinline__ double f2d(float f) {
    const unsigned int u = __float_as_uint(f);
    const unsigned int sgn = u & 0x80000000u;
    const unsigned int a = u ^ sgn;
    unsigned int hi = (a >> 3) + (896u << 20);
    unsigned int lo = a << 29;
    hi = (a < 0x00800000u) ? 0u : hi;                                      /* zero, subnormal */
    lo = (a < 0x00800000u) ? 0u : lo;
    hi = (a >= 0x7f800000u) ? (0x7ff00000u | ((a >> 3) & 0xfffffu)) : hi;   /* inf, nan */
    return __hiloint2double((int)(hi | sgn), (int)lo);
}

/* (1 + d)^gamma - 1, accurate relative to d: binomial series for |d| < 1/32
 * (truncation < 1e-9 relative), log1p/expm1 otherwise */
__device__ __forceinline__ float pow1m(float d, const float* c, float gamma) {
    if (fabsf(d) < 0.03125f) {
        float p = c[5];
        p = fmaf(p, d, c[4]);
        p = fmaf(p, d, c[3]);
        p = fmaf(p, d, c[2]);
        p = fmaf(p, d, c[1]);
        p = fmaf(p, d, c[0]);
        return p * d;
    }
    return expm1f(gamma * log1pf(d));
}

struct Prim {
    float rp, m0, m1, m2, tp;   /* perturbation conserved */
    float rho, u0, u1, u2, th, pp, c, umag;
};

__device__ __forceinline__ float safe_sqrt(float s) { return s > 0.0f ? s * rsqrtf(s) : 0.0f; }

/* reciprocal: hardware approximation refined by one Newton step (within an
 * ulp; both elements of a face evaluate it on the same bits) */
__device__ __forceinline__ float rcp_nr(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return __fmaf_rn(__fmaf_rn(-x, r, 1.0f), r, r);
}

__device__ __forceinline__ Prim make_prim(const float* s, float rref, float tref, float pref,
                                          const StageArgs& a) {
    Prim p;
    p.rp = s[0]; p.m0 = s[1]; p.m1 = s[2]; p.m2 = s[3]; p.tp = s[4];
    p.rho = rref + p.rp;
    const float inv = rcp_nr(p.rho);
    p.u0 = p.m0 * inv; p.u1 = p.m1 * inv; p.u2 = p.m2 * inv;
    p.th = (tref + p.tp) * inv;
    p.pp = pref * pow1m(p.tp * rcp_nr(tref), a.eos, a.gamma);
    p.c = safe_sqrt(a.gR * p.th);
    p.umag = safe_sqrt(p.u0 * p.u0 + p.u1 * p.u1 + p.u2 * p.u2);
    return p;
}

template <int NX, int NY, int NZ>
struct FaceSlot {
    int dir, side, la, lo, face;
};

template <int NX, int NY, int NZ>
__device__ __forceinline__ FaceSlot<NX, NY, NZ> face_slot(int t) {
    using G = Geo<NX, NY, NZ>;
    int dir, side, s0, s1;
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
    FaceSlot<NX, NY, NZ> f;
    f.dir = dir; f.side = side; f.face = 2 * dir + side;
    f.la = (i * NY + j) * NZ + k;
    f.lo = (io * NY + jo) * NZ + ko;
    return f;
}

/* one kernel per stage (0: tendency only): the stage's own loads and update
 * only; registers sized for 8 resident CTAs per SM in stages 1-2 and 7 in the
 * stage that also carries the FP64 state (measured best on GB300) */
/* tensor index of d_r U_c (XX,YY,ZZ,XY,YZ,XZ,YX,ZY,ZX) */
__device__ __forceinline__ constexpr int tidx(int r, int c) {
    return r == c ? r : (r == 0 ? (c == 1 ? 3 : 5) : r == 1 ? (c == 2 ? 4 : 6) : (c == 0 ? 8 : 7));
}

template <int NX, int NY, int NZ, int STAGE, bool VISC>
__global__ void __launch_bounds__(Geo<NX, NY, NZ>::BLOCK, VISC ? 6 : (STAGE == 1 || STAGE == 2) ? 8 : 7)
k_mixed_stage(StageArgs a, MixedTabs tab) {
    using G = Geo<NX, NY, NZ>;
    constexpr int NP = G::NP;
    constexpr int NFS = G::NFS;
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    float4* sF4 = smem4;                                   /* [3][NP] */
    float* sF1 = smem + G::OFF_F1;                         /* [3][NP] */
    float4* sP = reinterpret_cast<float4*>(smem + G::OFF_P);     /* [4][NP] */
    float4* sFF4 = reinterpret_cast<float4*>(smem + G::OFF_FF4); /* [NFS] */
    float* sFF1 = smem + G::OFF_FF1;                       /* [NFS] */
    float* sQ = smem + G::OFF_Q;
    float* sMeta = smem + G::OFF_META;

    const int t = threadIdx.x;
    const int64_t e = blockIdx.x;
    constexpr bool has_din = STAGE >= 2;

    /* issue every global load first: own node, face neighbour, stage-3 FP64 */
    float own[5], din[5] = {0, 0, 0, 0, 0}, bgs[3] = {0, 0, 0};
    double u64[5];
    if (t < NP) {
        const int64_t n = e * NP + t;
#pragma unroll
        for (int v = 0; v < 5; v++) own[v] = __ldg(a.U32[v] + n);
        if (has_din) {
#pragma unroll
            for (int v = 0; v < 5; v++) {
                din[v] = __ldg(a.Din[v] + n);
                own[v] += din[v];
            }
        }
        const float* bg = a.bg + (int64_t)__ldg(a.layer + e) * 3 * NP;
        bgs[0] = __ldg(bg + t); bgs[1] = __ldg(bg + NP + t); bgs[2] = __ldg(bg + 2 * NP + t);
        if constexpr (STAGE == 3) {
#pragma unroll
            for (int v = 0; v < 5; v++) u64[v] = __ldg(a.U[v] + n);
        }
    }
    float gown[12];
    if constexpr (VISC) {
        if (t < NP) {
            const int64_t n = e * NP + t;
#pragma unroll
            for (int c = 0; c < 12; c++) gown[c] = __ldg(a.Gv[c] + n);
        }
    }
    FaceSlot<NX, NY, NZ> fs;
    int32_t nb = -1;
    float oth[5], bgo[3];
    float gfs[4] = {0, 0, 0, 0}, gfo[4] = {0, 0, 0, 0};   /* d_c U_dir (c = 0..2), d_dir theta */
    if (t < NFS) {
        fs = face_slot<NX, NY, NZ>(t);
        nb = __ldg(a.nbr + (int64_t)fs.face * a.n_elem + e);
        if constexpr (VISC) {
            const int64_t ns = e * NP + fs.la;
#pragma unroll
            for (int c = 0; c < 3; c++) gfs[c] = __ldg(a.Gv[tidx(c, fs.dir)] + ns);
            gfs[3] = __ldg(a.Gv[9 + fs.dir] + ns);
            if (nb >= 0) {
                const int64_t no = (int64_t)nb * NP + fs.lo;
#pragma unroll
                for (int c = 0; c < 3; c++) gfo[c] = __ldg(a.Gv[tidx(c, fs.dir)] + no);
                gfo[3] = __ldg(a.Gv[9 + fs.dir] + no);
            }
        }
        if (nb >= 0) {
            const int64_t n = (int64_t)nb * NP + fs.lo;
#pragma unroll
            for (int v = 0; v < 5; v++) oth[v] = __ldg(a.U32[v] + n);
            if (has_din) {
#pragma unroll
                for (int v = 0; v < 5; v++) oth[v] += __ldg(a.Din[v] + n);
            }
            const float* bg = a.bg + (int64_t)__ldg(a.layer + nb) * 3 * NP;
            bgo[0] = __ldg(bg + fs.lo); bgo[1] = __ldg(bg + NP + fs.lo); bgo[2] = __ldg(bg + 2 * NP + fs.lo);
        }
    }
    for (int q = t; q < 3 * MAXN * MAXN; q += blockDim.x) sQ[q] = __ldg(a.Qg + q);
    if (t < 3) sMeta[t] = __ldg(a.J + (int64_t)t * a.n_elem + e);

    /* phase 1: own node primitives and volume fluxes */
    if (t < NP) {
        const Prim p = make_prim(own, bgs[0], bgs[1], bgs[2], a);
        sP[t] = make_float4(p.rp, p.m0, p.m1, p.m2);
        sP[NP + t] = make_float4(p.tp, p.rho, p.u0, p.u1);
        sP[2 * NP + t] = make_float4(p.u2, p.th, p.pp, p.c);
        sP[3 * NP + t] = make_float4(p.umag, 0.0f, 0.0f, 0.0f);
        const float u[3] = {p.u0, p.u1, p.u2};
        const float m[3] = {p.m0, p.m1, p.m2};
#pragma unroll
        for (int d = 0; d < 3; d++) {
            float4 f = make_float4(m[d], fmaf(m[0], u[d], d == 0 ? p.pp : 0.0f),
                                   fmaf(m[1], u[d], d == 1 ? p.pp : 0.0f),
                                   fmaf(m[2], u[d], d == 2 ? p.pp : 0.0f));
            float f1 = m[d] * p.th;
            if constexpr (VISC) {
                /* - mu grad U (momentum r along d: d_r U_d), - (mu / Pr) d_d theta */
                const float mu = p.rho * a.nu, mt = p.rho * a.nu_pr;
                f.y = fmaf(-mu, gown[tidx(0, d)], f.y);
                f.z = fmaf(-mu, gown[tidx(1, d)], f.z);
                f.w = fmaf(-mu, gown[tidx(2, d)], f.w);
                f1 = fmaf(-mt, gown[9 + d], f1);
            }
            sF4[d * NP + t] = f;
            sF1[d * NP + t] = f1;
        }
    }
    __syncthreads();

    /* phase 2: Rusanov flux on every face node */
    if (t < NFS) {
        const int dir = fs.dir;
        const float sg = fs.side ? 1.0f : -1.0f;   /* outward normal = sg e_dir */
        const float4 P0 = sP[fs.la], P1 = sP[NP + fs.la], P2 = sP[2 * NP + fs.la], P3 = sP[3 * NP + fs.la];
        Prim S;
        S.rp = P0.x; S.m0 = P0.y; S.m1 = P0.z; S.m2 = P0.w;
        S.tp = P1.x; S.rho = P1.y; S.u0 = P1.z; S.u1 = P1.w;
        S.u2 = P2.x; S.th = P2.y; S.pp = P2.z; S.c = P2.w; S.umag = P3.x;
        Prim O;
        if (nb >= 0) {
            O = make_prim(oth, bgo[0], bgo[1], bgo[2], a);
        } else {
            /* wall ghost: NEUMANN for rho, theta, p; SYMMETRY velocity
             * (tangential projection rescaled to |U|, tensor.h:486-494) */
            O = S;
            float r0 = dir == 0 ? 0.0f : S.u0;
            float r1 = dir == 1 ? 0.0f : S.u1;
            float r2 = dir == 2 ? 0.0f : S.u2;
            const float mr = safe_sqrt(r0 * r0 + r1 * r1 + r2 * r2);
            if (mr > 1e-7f) {
                const float sc = S.umag / mr;
                r0 *= sc; r1 *= sc; r2 *= sc;
            }
            O.u0 = r0; O.u1 = r1; O.u2 = r2;
            O.m0 = O.rho * r0; O.m1 = O.rho * r1; O.m2 = O.rho * r2;
            O.umag = safe_sqrt(r0 * r0 + r1 * r1 + r2 * r2);
        }
        /* Canonical orientation: L is the element below the face along +e_dir,
         * R the one above (the ghost on a wall).  Both elements of an interior
         * face evaluate the same expression on the same (L, R) data, so their
         * fluxes are bit-identical and the face conserves exactly. */
        const bool self_low = fs.side == 1;
        const Prim& Lp = self_low ? S : O;
        const Prim& Rp = self_low ? O : S;
        /* face average with the reference's weights (field.h:2888-2890, fI of
         * field.cpp:257-266): 1/2 inside, the ghost value alone on a wall */
        float wL = 0.5f, wR = 0.5f;
        if (nb < 0) { wL = self_low ? 0.0f : 1.0f; wR = 1.0f - wL; }
        const float uL = dir == 0 ? Lp.u0 : dir == 1 ? Lp.u1 : Lp.u2;
        const float uR = dir == 0 ? Rp.u0 : dir == 1 ? Rp.u1 : Rp.u2;
        const float lam = 0.5f * ((wL * Lp.umag + wR * Rp.umag) + (wL * Lp.c + wR * Rp.c));
        /* F* . e_dir = avg(F) . e_dir - lam (q_R - q_L) (normal component only for
         * momentum), field.h:2928-2943; the self element takes sg * F* */
        const float fr = (wL * (Lp.rho * uL) + wR * (Rp.rho * uR)) - lam * (Rp.rp - Lp.rp);
        const float mL[3] = {Lp.m0, Lp.m1, Lp.m2}, mR[3] = {Rp.m0, Rp.m1, Rp.m2};
        float fm[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float pL = (c == dir) ? Lp.pp : 0.0f, pR = (c == dir) ? Rp.pp : 0.0f;
            fm[c] = wL * fmaf(mL[c], uL, pL) + wR * fmaf(mR[c], uR, pR);
            if (c == dir) fm[c] -= lam * (mR[c] - mL[c]);
        }
        float ft = (wL * (Lp.rho * uL * Lp.th) + wR * (Rp.rho * uR * Rp.th)) - lam * (Rp.tp - Lp.tp);
        if constexpr (VISC) {
            /* average of the two sides' viscous fluxes; the wall ghost has zero
             * gradient (and weight 1 on a wall, so no viscous wall flux) */
            const float* gL = self_low ? gfs : gfo;
            const float* gR = self_low ? gfo : gfs;
            const float mL_ = Lp.rho * a.nu, mR_ = Rp.rho * a.nu;
            const float tL_ = Lp.rho * a.nu_pr, tR_ = Rp.rho * a.nu_pr;
#pragma unroll
            for (int c = 0; c < 3; c++) fm[c] -= wL * (mL_ * gL[c]) + wR * (mR_ * gR[c]);
            ft -= wL * (tL_ * gL[3]) + wR * (tR_ * gR[3]);
        }
        const float fr_o = sg * fr, ft_o = sg * ft;
        fm[0] *= sg; fm[1] *= sg; fm[2] *= sg;
        sFF4[t] = make_float4(fr_o, fm[0], fm[1], fm[2]);
        sFF1[t] = ft_o;
    }
    __syncthreads();

    /* phase 3: weak volume term (line sums with Q), lift, buoyancy, update */
    if (t >= NP) return;
    const int i = t / (NY * NZ), j = (t / NZ) % NY, k = t % NZ;
    float L0, L1, L2, L3, L4;
    {
        float4 acc = make_float4(0, 0, 0, 0);
        float acc1 = 0.0f;
#pragma unroll
        for (int m = 0; m < NX; m++) {
            const float q = sQ[i * MAXN + m];
            const int b = (m * NY + j) * NZ + k;
            const float4 f = sF4[b];
            acc.x = fmaf(q, f.x, acc.x); acc.y = fmaf(q, f.y, acc.y);
            acc.z = fmaf(q, f.z, acc.z); acc.w = fmaf(q, f.w, acc.w);
            acc1 = fmaf(q, sF1[b], acc1);
        }
        const float Jx = sMeta[0];
        L0 = Jx * acc.x; L1 = Jx * acc.y; L2 = Jx * acc.z; L3 = Jx * acc.w; L4 = Jx * acc1;
    }
    if (NY > 1) {
        float4 acc = make_float4(0, 0, 0, 0);
        float acc1 = 0.0f;
#pragma unroll
        for (int m = 0; m < NY; m++) {
            const float q = sQ[MAXN * MAXN + j * MAXN + m];
            const int b = (i * NY + m) * NZ + k;
            const float4 f = sF4[NP + b];
            acc.x = fmaf(q, f.x, acc.x); acc.y = fmaf(q, f.y, acc.y);
            acc.z = fmaf(q, f.z, acc.z); acc.w = fmaf(q, f.w, acc.w);
            acc1 = fmaf(q, sF1[NP + b], acc1);
        }
        const float Jy = sMeta[1];
        L0 = fmaf(Jy, acc.x, L0); L1 = fmaf(Jy, acc.y, L1); L2 = fmaf(Jy, acc.z, L2);
        L3 = fmaf(Jy, acc.w, L3); L4 = fmaf(Jy, acc1, L4);
    }
    {
        float4 acc = make_float4(0, 0, 0, 0);
        float acc1 = 0.0f;
#pragma unroll
        for (int m = 0; m < NZ; m++) {
            const float q = sQ[2 * MAXN * MAXN + k * MAXN + m];
            const int b = (i * NY + j) * NZ + m;
            const float4 f = sF4[2 * NP + b];
            acc.x = fmaf(q, f.x, acc.x); acc.y = fmaf(q, f.y, acc.y);
            acc.z = fmaf(q, f.z, acc.z); acc.w = fmaf(q, f.w, acc.w);
            acc1 = fmaf(q, sF1[2 * NP + b], acc1);
        }
        const float Jz = sMeta[2];
        L0 = fmaf(Jz, acc.x, L0); L1 = fmaf(Jz, acc.y, L1); L2 = fmaf(Jz, acc.z, L2);
        L3 = fmaf(Jz, acc.w, L3); L4 = fmaf(Jz, acc1, L4);
    }
    /* surface lift: -(J_d / w_end) F*.n_out for each face through the node */
    auto lift = [&](int slot, float coef) {
        const float4 f = sFF4[slot];
        L0 = fmaf(-coef, f.x, L0); L1 = fmaf(-coef, f.y, L1); L2 = fmaf(-coef, f.z, L2);
        L3 = fmaf(-coef, f.w, L3); L4 = fmaf(-coef, sFF1[slot], L4);
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
    const float rp = own[0];
    L1 = fmaf(rp, a.g[0], L1);
    L2 = fmaf(rp, a.g[1], L2);
    L3 = fmaf(rp, a.g[2], L3);
    const float Lv[5] = {L0, L1, L2, L3, L4};

    const int64_t n = e * NP + t;
    if constexpr (STAGE == 0) {
#pragma unroll
        for (int v = 0; v < 5; v++) a.L[v][n] = f2d(Lv[v]);
        return;
    }
    const float dt = a.dt;
    if constexpr (STAGE == 1) {
#pragma unroll
        for (int v = 0; v < 5; v++) a.Dout[v][n] = dt * Lv[v];
    } else if constexpr (STAGE == 2) {
#pragma unroll
        for (int v = 0; v < 5; v++) a.Dout[v][n] = 0.25f * fmaf(dt, Lv[v], din[v]);
    } else {
        bool finite = true;
#pragma unroll
        for (int v = 0; v < 5; v++) {
            const float D = (2.0f / 3.0f) * fmaf(dt, Lv[v], din[v]);
            const double un = u64[v] + f2d(D);
            a.Unew[v][n] = un;
            a.U32new[v][n] = d2f_rn(un);
            /* exponent field all ones = inf or nan (integer test, no FP64 op) */
            finite = finite && ((__double2hiint(un) & 0x7ff00000) != 0x7ff00000);
        }
        if (!finite) atomicOr(a.status, NSEM_STATUS_NONFINITE);
    }
}


/* Strong-form DG gradients of U and theta of a stage state (gradf<true>,
 * field.h:3327-3360) for the viscous fluxes: per node
 *   d_r q = J_r sum_m D_r[a_r][m] q_m  +  (J_r / w_end) (cds(q) - q)  on the
 *   lower (-) / upper (+) face normal to r through the node,
 * cds = (own + neighbour) / 2 inside, the ghost value on a wall (SYMMETRY
 * velocity, NEUMANN theta: cds(theta) - theta = 0 there).  The state is the
 * stage kernel's (FP32 shadow plus the previous increment for SIN >= 2).
 * Output Gout[tidx(r, c)] = d_r U_c, Gout[9 + r] = d_r theta. */
template <int NX, int NY, int NZ, int SIN>
__global__ void __launch_bounds__(Geo<NX, NY, NZ>::BLOCK)
k_mixed_grad(StageArgs a, MixedTabs tab) {
    using G = Geo<NX, NY, NZ>;
    constexpr int NP = G::NP;
    constexpr int NFS = G::NFS;
    constexpr bool has_din = SIN >= 2;
    extern __shared__ float4 gsm4[];
    float4* sV = gsm4;                                              /* [NP]  U, theta */
    float4* sD = gsm4 + NP;                                         /* [NFS] cds - own */
    float* sDg = reinterpret_cast<float*>(gsm4 + NP + NFS);        /* [3][MAXN^2] */
    float* sJ = sDg + 3 * MAXN * MAXN;                              /* [3] */
    const int t = threadIdx.x;
    const int64_t e = blockIdx.x;

    float own[5], bgs[1] = {0};
    if (t < NP) {
        const int64_t n = e * NP + t;
#pragma unroll
        for (int v = 0; v < 5; v++) own[v] = __ldg(a.U32[v] + n);
        if (has_din) {
#pragma unroll
            for (int v = 0; v < 5; v++) own[v] += __ldg(a.Din[v] + n);
        }
        const float* bg = a.bg + (int64_t)__ldg(a.layer + e) * 3 * NP;
        bgs[0] = __ldg(bg + t);
    }
    FaceSlot<NX, NY, NZ> fs;
    int32_t nb = -1;
    float oth[5], bgo[1];
    if (t < NFS) {
        fs = face_slot<NX, NY, NZ>(t);
        nb = __ldg(a.nbr + (int64_t)fs.face * a.n_elem + e);
        if (nb >= 0) {
            const int64_t n = (int64_t)nb * NP + fs.lo;
#pragma unroll
            for (int v = 0; v < 5; v++) oth[v] = __ldg(a.U32[v] + n);
            if (has_din) {
#pragma unroll
                for (int v = 0; v < 5; v++) oth[v] += __ldg(a.Din[v] + n);
            }
            const float* bg = a.bg + (int64_t)__ldg(a.layer + nb) * 3 * NP;
            bgo[0] = __ldg(bg + fs.lo);
        }
    }
    for (int q = t; q < 3 * MAXN * MAXN; q += blockDim.x) sDg[q] = __ldg(a.Dg + q);
    if (t < 3) sJ[t] = __ldg(a.J + (int64_t)t * a.n_elem + e);

    /* U = m / rho as make_prim forms it, and theta - T0 from the perturbation:
     * the background has theta = T0 (Theta_ref = rho_ref T0), so
     * theta - T0 = (Theta' - T0 rho') / rho -- the same gradient as theta
     * without FP32 cancellation against T0 */
    const float T0 = a.T0;
    auto prim_ut = [T0](const float* s, float rref) {
        const float inv = rcp_nr(rref + s[0]);
        return make_float4(s[1] * inv, s[2] * inv, s[3] * inv, fmaf(-T0, s[0], s[4]) * inv);
    };
    if (t < NP) sV[t] = prim_ut(own, bgs[0]);
    __syncthreads();

    if (t < NFS) {
        const float4 S = sV[fs.la];
        float4 c;
        if (nb >= 0) {
            const float4 O = prim_ut(oth, bgo[0]);
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
#pragma unroll
        for (int m = 0; m < NX; m++) {
            const float q = sDg[i * MAXN + m];
            const float4 v = sV[(m * NY + j) * NZ + k];
            acc.x = fmaf(q, v.x, acc.x); acc.y = fmaf(q, v.y, acc.y);
            acc.z = fmaf(q, v.z, acc.z); acc.w = fmaf(q, v.w, acc.w);
        }
        d[0] = acc;
    }
    {
        float4 acc = make_float4(0, 0, 0, 0);
        if (NY > 1) {
#pragma unroll
            for (int m = 0; m < NY; m++) {
                const float q = sDg[MAXN * MAXN + j * MAXN + m];
                const float4 v = sV[(i * NY + m) * NZ + k];
                acc.x = fmaf(q, v.x, acc.x); acc.y = fmaf(q, v.y, acc.y);
                acc.z = fmaf(q, v.z, acc.z); acc.w = fmaf(q, v.w, acc.w);
            }
        }
        d[1] = acc;
    }
    {
        float4 acc = make_float4(0, 0, 0, 0);
#pragma unroll
        for (int m = 0; m < NZ; m++) {
            const float q = sDg[2 * MAXN * MAXN + k * MAXN + m];
            const float4 v = sV[(i * NY + j) * NZ + m];
            acc.x = fmaf(q, v.x, acc.x); acc.y = fmaf(q, v.y, acc.y);
            acc.z = fmaf(q, v.z, acc.z); acc.w = fmaf(q, v.w, acc.w);
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
    const float cx = Jd[0] * tab.lift[0], cy = Jd[1] * tab.lift[1], cz = Jd[2] * tab.lift[2];
    if (i == 0) lift(0, G::OFF_X + j * NZ + k, -cx);
    if (i == NX - 1) lift(0, G::OFF_X + G::NFX + j * NZ + k, cx);
    if (NY > 1) {
        if (j == 0) lift(1, G::OFF_Y + i * NZ + k, -cy);
        if (j == NY - 1) lift(1, G::OFF_Y + G::NFY + i * NZ + k, cy);
    }
    if (k == 0) lift(2, G::OFF_Z + i * NY + j, -cz);
    if (k == NZ - 1) lift(2, G::OFF_Z + G::NFZ + i * NY + j, cz);
    const int64_t n = e * NP + t;
#pragma unroll
    for (int r = 0; r < 3; r++) {
        a.Gout[tidx(r, 0)][n] = d[r].x;
        a.Gout[tidx(r, 1)][n] = d[r].y;
        a.Gout[tidx(r, 2)][n] = d[r].z;
        a.Gout[9 + r][n] = d[r].w;
    }
}

template <int NX, int NY, int NZ>
constexpr size_t grad_smem() {
    using G = Geo<NX, NY, NZ>;
    return sizeof(float4) * (G::NP + G::NFS) + sizeof(float) * (3 * MAXN * MAXN + 4);
}

/* full <-> perturbation state (FP64): u' = u - (rho_ref, 0, 0, 0, rho_ref T0) */
struct Ptr5 {
    double* p[5];
};

struct FPtr5 {
    float* p[5];
};

__global__ void k_convert(Ptr5 src, Ptr5 dst, FPtr5 shadow, const double* rho_ref, double T0,
                          int64_t n, int to_pert) {
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
        if (to_pert)
            for (int v = 0; v < 5; v++) shadow.p[v][i] = d2f_rn(dst.p[v][i]);
    }
}

template <int NX, int NY, int NZ, bool VISC>
void launch_stage_v(const StageArgs& a, const MixedTabs& t, cudaStream_t st) {
    using G = Geo<NX, NY, NZ>;
    const unsigned grid = (unsigned)a.n_elem;
    switch (a.stage) {
        case 0: k_mixed_stage<NX, NY, NZ, 0, VISC><<<grid, G::BLOCK, G::SMEM, st>>>(a, t); break;
        case 1: k_mixed_stage<NX, NY, NZ, 1, VISC><<<grid, G::BLOCK, G::SMEM, st>>>(a, t); break;
        case 2: k_mixed_stage<NX, NY, NZ, 2, VISC><<<grid, G::BLOCK, G::SMEM, st>>>(a, t); break;
        default: k_mixed_stage<NX, NY, NZ, 3, VISC><<<grid, G::BLOCK, G::SMEM, st>>>(a, t); break;
    }
}

/* one stage; viscous runs first form the gradients of the stage state */
template <int NX, int NY, int NZ>
int launch_stage(const StageArgs& a, const MixedTabs& t, cudaStream_t st, bool visc) {
    using G = Geo<NX, NY, NZ>;
    if (!visc) {
        launch_stage_v<NX, NY, NZ, false>(a, t, st);
        return (int)cudaGetLastError();
    }
    const unsigned grid = (unsigned)a.n_elem;
    const size_t gs = grad_smem<NX, NY, NZ>();
    if (a.stage <= 1) k_mixed_grad<NX, NY, NZ, 1><<<grid, G::BLOCK, gs, st>>>(a, t);
    else k_mixed_grad<NX, NY, NZ, 2><<<grid, G::BLOCK, gs, st>>>(a, t);
    int e = (int)cudaGetLastError();
    if (e) return e;
    launch_stage_v<NX, NY, NZ, true>(a, t, st);
    return (int)cudaGetLastError();
}

template <int NX, int NY, int NZ>
int prepare_stage() {
    using G = Geo<NX, NY, NZ>;
    const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
    int e = 0;
    if (G::SMEM > 48 * 1024) {
        e = (int)cudaFuncSetAttribute(k_mixed_stage<NX, NY, NZ, 0, false>, at, (int)G::SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_stage<NX, NY, NZ, 1, false>, at, (int)G::SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_stage<NX, NY, NZ, 2, false>, at, (int)G::SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_stage<NX, NY, NZ, 3, false>, at, (int)G::SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_stage<NX, NY, NZ, 0, true>, at, (int)G::SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_stage<NX, NY, NZ, 1, true>, at, (int)G::SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_stage<NX, NY, NZ, 2, true>, at, (int)G::SMEM);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_stage<NX, NY, NZ, 3, true>, at, (int)G::SMEM);
    }
    constexpr size_t gs = grad_smem<NX, NY, NZ>();
    if (!e && gs > 48 * 1024) {
        e = (int)cudaFuncSetAttribute(k_mixed_grad<NX, NY, NZ, 1>, at, (int)gs);
        if (!e) e = (int)cudaFuncSetAttribute(k_mixed_grad<NX, NY, NZ, 2>, at, (int)gs);
    }
    return e;
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
                   cudaStream_t st, bool visc) {
    if (nx == 5 && ny == 5 && nz == 5) return launch_stage<5, 5, 5>(a, t, st, visc);
    if (nx == 8 && ny == 8 && nz == 8) return launch_stage<8, 8, 8>(a, t, st, visc);
    if (nx == 4 && ny == 4 && nz == 4) return launch_stage<4, 4, 4>(a, t, st, visc);
    if (nx == 5 && ny == 1 && nz == 5) return launch_stage<5, 1, 5>(a, t, st, visc);
    if (nx == 4 && ny == 1 && nz == 4) return launch_stage<4, 1, 4>(a, t, st, visc);
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
    const std::vector<float> qtab(&tabs->Q[0][0], &tabs->Q[0][0] + 3 * MAXN * MAXN);
    /* D_d[a][m] = l_m'(x_a) = dpsi[a * n + m] for the gradient kernel */
    std::vector<float> dtab(3 * MAXN * MAXN, 0.0f);
    for (int d = 0; d < 3; d++)
        for (int aa = 0; aa < npd[d]; aa++)
            for (int mm = 0; mm < npd[d]; mm++)
                dtab[d * MAXN * MAXN + aa * MAXN + mm] = (float)m->dpsi[d][aa * npd[d] + mm];
    if (!up(&mb->nbr, nbr) || !up(&mb->J, J) || !up(&mb->layer, layer) || !up(&mb->bg, bg) ||
        !up(&mb->Qg, qtab) || !up(&mb->Dg, dtab)) {
        err = "precision form: device allocation failed";
        return NSEM_NO_MEMORY;
    }
    for (int s = 0; s < 2; s++)
        for (int v = 0; v < 5; v++) {
            if (cudaMalloc((void**)&mb->U[s][v], n_int * sizeof(double)) != cudaSuccess ||
                cudaMalloc((void**)&mb->U32[s][v], n_int * sizeof(float)) != cudaSuccess ||
                cudaMalloc((void**)&mb->D[s][v], n_int * sizeof(float)) != cudaSuccess) {
                err = "precision form: device allocation failed";
                return NSEM_NO_MEMORY;
            }
            allocs->push_back(mb->U[s][v]);
            allocs->push_back(mb->U32[s][v]);
            allocs->push_back(mb->D[s][v]);
        }
    mb->visc = dev.nu != 0.0;
    mb->nu = (float)dev.nu;
    mb->nu_pr = (float)(dev.nu * dev.iPr);
    if (mb->visc)
        for (int c = 0; c < 12; c++) {
            if (cudaMalloc((void**)&mb->Gv[c], n_int * sizeof(float)) != cudaSuccess) {
                err = "precision form: device allocation failed";
                return NSEM_NO_MEMORY;
            }
            allocs->push_back(mb->Gv[c]);
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
        a.U32[v] = mb->U32[cur][v];
        a.U32new[v] = mb->U32[cur ^ 1][v];
        a.Din[v] = (stage == 2) ? mb->D[0][v] : (stage == 3) ? mb->D[1][v] : nullptr;
        a.Dout[v] = (stage == 1) ? mb->D[0][v] : (stage == 2) ? mb->D[1][v] : nullptr;
        a.Unew[v] = mb->U[cur ^ 1][v];
        a.L[v] = b->L[v];
    }
    a.nbr = mb->nbr;
    a.J = mb->J;
    a.layer = mb->layer;
    a.Qg = mb->Qg;
    a.Dg = mb->Dg;
    for (int c = 0; c < 12; c++) {
        a.Gv[c] = mb->Gv[c];
        a.Gout[c] = mb->Gv[c];
    }
    a.nu = mb->nu;
    a.nu_pr = mb->nu_pr;
    a.T0 = (float)dev->T0;
    a.bg = mb->bg;
    a.n_elem = mb->n_elem;
    a.dt = (float)dt;
    a.gamma = (float)dev->gamma;
    a.gR = (float)dev->gR;
    for (int c = 0; c < 3; c++) a.g[c] = (float)dev->g[c];
    /* binomial coefficients C(gamma, k) of (1 + d)^gamma - 1 */
    double ck = 1.0;
    for (int k = 1; k <= 6; k++) {
        ck *= (dev->gamma - (k - 1)) / k;
        a.eos[k - 1] = (float)ck;
    }
    a.stage = stage;
    a.status = dev->status;
    return a;
}

int launch(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, int stage, int cur, double dt,
           cudaStream_t st) {
    StageArgs a = stage_args(dev, mb, b, stage, cur, dt);
    return dispatch_stage(mb->npd[0], mb->npd[1], mb->npd[2], a, *(const MixedTabs*)mb->tabs, st,
                          mb->visc);
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
    FPtr5 shadow;
    for (int v = 0; v < 5; v++) {
        full.p[v] = b->u[v];
        pert.p[v] = mb->U[mb->cur][v];
        shadow.p[v] = mb->U32[mb->cur][v];
    }
    if (to_pert)
        k_convert<<<grid_for(dev->n_int), 256, 0, (cudaStream_t)stream>>>(
            full, pert, shadow, dev->rho_ref, dev->T0, dev->n_int, 1);
    else
        k_convert<<<grid_for(dev->n_int), 256, 0, (cudaStream_t)stream>>>(
            pert, full, shadow, dev->rho_ref, dev->T0, dev->n_int, 0);
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
