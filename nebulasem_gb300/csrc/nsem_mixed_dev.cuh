/*
 * Device helpers shared by the precision form's stage kernels (nsem_mixed.cu)
 * and their discrete adjoint (nsem_mixed_adj.cu): element geometry, the
 * element-blocked state layout, exact-rounding FP32 <-> FP64 conversions on
 * the integer pipes, and the pointwise physics (primitives of the
 * perturbation state, volume fluxes) written with explicit rounding
 * intrinsics so that every inlined copy produces the same bits.
 *
 * State layout (element-blocked structure of arrays): variable v of local
 * node t of element e lives at (e * 5 + v) * NP + t, so one 64-bit address
 * per (element, node) serves all five variables through immediate offsets.
 * Background per z-layer of elements: [layer][4][NP] = rho_ref, Theta_ref =
 * rho_ref T0, 1 / Theta_ref, p_ref.
 */
#ifndef NSEM_MIXED_DEV_CUH
#define NSEM_MIXED_DEV_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "nsem_internal.h"

/* the node counts per direction the precision form is built for (the
 * kernels' dispatch in every translation unit of the form) */
#define NSEM_MIXED_DIMS(X) X(5, 5, 5) X(8, 8, 8) X(4, 4, 4) X(5, 1, 5) X(4, 1, 4)

namespace nsem_mx {

constexpr int MAXN = NSEM_MAX_NPD;

/* fields of a mortar slot ([MX_FIELDS][n_ms]): the fine node, whether the
 * fine element is side 1, the coarse face's first node and strides, its node
 * counts, the slot's interpolation indices (ia, ib), the sub-face's first
 * slot and its psiRef / psiCor tables.  A face node's entry names a slot,
 * with MX_COARSE set for the coarse side's projected value. */
enum { MX_FINE, MX_FINE_C1, MX_BASE, MX_SA, MX_SB, MX_NA, MX_NB, MX_IA, MX_IB, MX_FIRST, MX_TA,
       MX_TB, MX_FIELDS };
constexpr int MX_COARSE = 1 << 30;
constexpr int QS = MAXN + 1;            /* row stride of the line tables (bank-conflict free) */
constexpr int QTAB = 3 * MAXN * QS;     /* floats per line table */

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
};

/* resident CTAs per SM asked of the register allocator: the wanted count,
 * capped by the threads and the shared memory an SM holds */
constexpr int min_blocks(int want, int block, size_t smem) {
    const int by_threads = 2048 / block;
    const int by_smem = (int)((227 * 1024) / (smem + 1024));
    int m = want < by_threads ? want : by_threads;
    m = m < by_smem ? m : by_smem;
    return m < 1 ? 1 : m;
}

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

/* reciprocal: hardware approximation refined by one Newton step (within an
 * ulp; deterministic, so every element evaluating it on the same bits gets
 * the same result) */
__device__ __forceinline__ float rcp_nr(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return __fmaf_rn(__fmaf_rn(-x, r, 1.0f), r, r);
}

__device__ __forceinline__ float safe_sqrt(float s) {
    return s > 0.0f ? __fmul_rn(s, rsqrtf(s)) : 0.0f;
}

/* (1 + d)^gamma - 1, accurate relative to d: binomial series for |d| < 1/32
 * (truncation < 1e-9 relative), log1p/expm1 otherwise; c[k-1] = C(gamma, k) */
__device__ __forceinline__ float pow1m(float d, const float* c, float gamma) {
    if (fabsf(d) < 0.03125f) {
        float p = c[5];
        p = __fmaf_rn(p, d, c[4]);
        p = __fmaf_rn(p, d, c[3]);
        p = __fmaf_rn(p, d, c[2]);
        p = __fmaf_rn(p, d, c[1]);
        p = __fmaf_rn(p, d, c[0]);
        return __fmul_rn(p, d);
    }
    return expm1f(__fmul_rn(gamma, log1pf(d)));
}

/* Primitives of a perturbation state x = (rho', rho u, rho v, rho w, Theta')
 * over the background (rho_ref, Theta_ref, 1/Theta_ref, p_ref):
 *   rho = rho_ref + rho',  u = m / rho,  theta = (Theta_ref + Theta') / rho,
 *   p' = p_ref ((1 + Theta'/Theta_ref)^gamma - 1)      (euler.cpp:211-213 on
 *   the perturbation), c = sqrt(gamma R theta) (euler.cpp:186), |u|. */
struct Pt {
    float rho, inv, u[3], th, pp, c, umag;
};

struct PhysConst {
    float gamma, gR;
    float eos[6];
};

__device__ __forceinline__ Pt pointwise(const float* x, const float* bgv, const float* eos,
                                        float gamma, float gR) {
    Pt p;
    p.rho = __fadd_rn(bgv[0], x[0]);
    p.inv = rcp_nr(p.rho);
    p.u[0] = __fmul_rn(x[1], p.inv);
    p.u[1] = __fmul_rn(x[2], p.inv);
    p.u[2] = __fmul_rn(x[3], p.inv);
    p.th = __fmul_rn(__fadd_rn(bgv[1], x[4]), p.inv);
    p.pp = __fmul_rn(bgv[3], pow1m(__fmul_rn(x[4], bgv[2]), eos, gamma));
    p.c = safe_sqrt(__fmul_rn(gR, p.th));
    p.umag = safe_sqrt(__fmaf_rn(p.u[0], p.u[0], __fmaf_rn(p.u[1], p.u[1], __fmul_rn(p.u[2], p.u[2]))));
    return p;
}

/* tensor index of d_r U_c (XX,YY,ZZ,XY,YZ,XZ,YX,ZY,ZX) */
__host__ __device__ __forceinline__ constexpr int tidx(int r, int c) {
    return r == c ? r : (r == 0 ? (c == 1 ? 3 : 5) : r == 1 ? (c == 2 ? 4 : 6) : (c == 0 ? 8 : 7));
}

/* Volume flux along direction D at one node: (m_D, m u_D + p' e_D, m_D theta)
 * minus, for viscous runs, (0, mu d_c U_D, (mu/Pr) d_D theta) with mu = rho nu
 * (g: the node's gradients in the 12-entry layout). */
template <int D, bool VISC>
__device__ __forceinline__ void vol_flux(const float* x, const Pt& p, const float* gr, float nu,
                                         float nu_pr, float4& f4, float& f1) {
    const float ud = p.u[D];
    f4.x = x[1 + D];
    f4.y = __fmaf_rn(x[1], ud, D == 0 ? p.pp : 0.0f);
    f4.z = __fmaf_rn(x[2], ud, D == 1 ? p.pp : 0.0f);
    f4.w = __fmaf_rn(x[3], ud, D == 2 ? p.pp : 0.0f);
    f1 = __fmul_rn(x[1 + D], p.th);
    if constexpr (VISC) {
        const float mu = __fmul_rn(p.rho, nu), mt = __fmul_rn(p.rho, nu_pr);
        f4.y = __fmaf_rn(-mu, gr[tidx(0, D)], f4.y);
        f4.z = __fmaf_rn(-mu, gr[tidx(1, D)], f4.z);
        f4.w = __fmaf_rn(-mu, gr[tidx(2, D)], f4.w);
        f1 = __fmaf_rn(-mt, gr[9 + D], f1);
    }
}

/* face node t of an element: direction, side (1 = the element's upper face
 * along +e_dir), own local node and the neighbour's local node, and the
 * in-plane index r of the node within its face (x: j NZ + k, y: i NZ + k,
 * z: i NY + j) */
struct FaceSlot {
    int dir, side, la, lo, face, r;
};

/* CUBE: on elements with NX = NY = NZ, slot t = face q * NF + r with
 * q = 2 dir + side and r the in-plane index (s0, s1) = (r / N, r % N); the
 * node index of each face plane follows from r without the general
 * decomposition (fewer instructions; measured faster in the precision form's
 * stages 1-2 and slower in stage 3, which therefore keeps the general form) */
template <int NX, int NY, int NZ, bool CUBE = false>
__device__ __forceinline__ FaceSlot face_slot(int t) {
    using G = Geo<NX, NY, NZ>;
    if constexpr (CUBE && NX == NY && NY == NZ) {
        constexpr int N = NX, NF = NX * NX;
        const int q = t / NF, r = t - q * NF;
        const int dir = q >> 1, side = q & 1;
        const int s0 = r / N, s1 = r - s0 * N;
        const int hi = side ? N - 1 : 0, ho = N - 1 - hi;
        FaceSlot f;
        f.dir = dir; f.side = side; f.face = q; f.r = r;
        f.la = dir == 0 ? hi * NF + r : dir == 1 ? (s0 * N + hi) * N + s1 : r * N + hi;
        f.lo = dir == 0 ? ho * NF + r : dir == 1 ? (s0 * N + ho) * N + s1 : r * N + ho;
        return f;
    }
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
    FaceSlot f;
    f.dir = dir; f.side = side; f.face = 2 * dir + side;
    f.r = dir == 2 ? s0 * NY + s1 : s0 * NZ + s1;
    f.la = (i * NY + j) * NZ + k;
    f.lo = (io * NY + jo) * NZ + ko;
    return f;
}

/* FP32 line sums as an in-place line transform (the stage kernels, and
 * transposed in the adjoint).  The fluxes of direction D are kept line-major:
 * variable v at node m along line l (x: l = j NZ + k, y: l = i NZ + k,
 * z: l = i NY + j) at BASE_D + m ROW + v NL + l, with NL lines and
 * ROW = 5 NL + padding.  After the face phase, thread r < 5 NL takes the
 * line and variable (v, l) = (r / NL, r % NL) of each direction: it reads
 * the n values m ROW + r (a warp reads consecutive words), forms
 * R_a = sum_m Q_D[a][m] F_m with the weights (the weak-form table of the
 * kernel's geometry) as constant-bank operands, and writes R_a over F_a.  A
 * node then reads its three R's.  Each flux value is read once from shared
 * memory instead of once per node of its line.
 *
 * Row padding (floats) per direction: puts the node threads' accesses
 * (stores in phase 1, reads of the results) and the face threads' reads in
 * distinct banks as far as possible -- chosen by counting the wavefronts of
 * every such warp access for each padding up to 31. */
template <int NX, int NY, int NZ>
constexpr int line_pad(int D) {
    return (NX == 5 && NY == 5) ? (D == 0 ? 28 : D == 1 ? 30 : 16)
         : (NX == 8 && NY == 8) ? (D == 0 ? 0 : D == 1 ? 8 : 4)
         : (NX == 4 && NY == 4) ? (D == 0 ? 0 : 8)
         : (NX == 5 && NY == 1) ? (D == 1 ? 0 : 1)
         : 0;
}

template <int NX, int NY, int NZ, int D>
struct LineLay {
    static constexpr int NP = NX * NY * NZ;
    static constexpr int n = D == 0 ? NX : D == 1 ? NY : NZ;
    static constexpr int NL = NP / n;
    static constexpr int ROW = 5 * NL + line_pad<NX, NY, NZ>(D);
    static constexpr int SIZE = n * ROW;
    static constexpr int BASE = D == 0 ? 0 : LineLay<NX, NY, NZ, D - 1>::BASE + LineLay<NX, NY, NZ, D - 1>::SIZE;
    /* position of variable 0 at node (i, j, k) */
    __device__ static __forceinline__ int at(int i, int j, int k) {
        return BASE + (D == 0 ? i : D == 1 ? j : k) * ROW +
               (D == 0 ? j * NZ + k : D == 1 ? i * NZ + k : i * NY + j);
    }
};
template <int NX, int NY, int NZ>
struct LineLay<NX, NY, NZ, -1> {
    static constexpr int BASE = 0, SIZE = 0;
};
/* floats of the three directions' flux rows */
template <int NX, int NY, int NZ>
constexpr int line_floats() {
    return LineLay<NX, NY, NZ, 2>::BASE + LineLay<NX, NY, NZ, 2>::SIZE;
}

/* slot of the face of direction D through local node (i, j, k), or -1 */
template <int NX, int NY, int NZ, int D>
__device__ __forceinline__ int face_of_node(int i, int j, int k) {
    using G = Geo<NX, NY, NZ>;
    if constexpr (D == 0) {
        return (i == 0) ? G::OFF_X + j * NZ + k : (i == NX - 1) ? G::OFF_X + G::NFX + j * NZ + k : -1;
    } else if constexpr (D == 1) {
        if constexpr (!G::HAS_Y) return -1;
        return (j == 0) ? G::OFF_Y + i * NZ + k : (j == NY - 1) ? G::OFF_Y + G::NFY + i * NZ + k : -1;
    } else {
        return (k == 0) ? G::OFF_Z + i * NY + j : (k == NZ - 1) ? G::OFF_Z + G::NFZ + i * NY + j : -1;
    }
}

}  // namespace nsem_mx

#endif
