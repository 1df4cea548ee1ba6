/*
 * Weak-form volume term gathered per target node in the order of the
 * reference's scatter loop (src/field/field.h:3440-3464): sources on the
 * X line below the node, Y below, Z below, the node itself, Z above, Y above,
 * X above.  Every node has the same number of sources, NPX + NPY + NPZ - 2, so
 * the loop runs over source positions p with one trip count for all threads
 * of the element; the (direction, source) of a position differs per thread and
 * is chosen by integer selects, and the floating-point work of the caller's
 * apply is issued once per position for the whole warp.  Per-line loops with
 * trip counts set by the node's own (i, j, k) leave about half of the lanes
 * idle in every FP64 instruction of the gather.
 *
 * sm: W doubles per node in shared memory with the metric Jinv cV of the node
 * at offset JOFF (components XX,YY,ZZ,XY,YZ,XZ,YX,ZY,ZX); dps: the three dpsi
 * tables (dpsi[d][s * npd + i], NSEM_MAX_NPD^2 apart).  A source on a line
 * contributes its own metric column times one derivative (J[col] D), the node
 * itself the product Jinv . (Dx_ii, Dy_jj, Dz_kk) -- the reference's products,
 * evaluated in its operand order.
 */
#ifndef NSEM_GATHER_CUH
#define NSEM_GATHER_CUH

#include "nsem_internal.h"

template <int W, int JOFF, typename Apply>
__device__ __forceinline__ void nsem_volume_gather(int npx, int npy, int npz, const double* sm,
                                                   const double* dps, int t, Apply apply) {
    constexpr int M2 = NSEM_MAX_NPD * NSEM_MAX_NPD;
    /* metric columns of the X, Y and Z derivatives: (XX,YX,ZX), (XY,YY,ZY),
     * (XZ,YZ,ZZ), four bits per component index */
    constexpr int COLS_X = 0 | (6 << 4) | (8 << 8);
    constexpr int COLS_Y = 3 | (1 << 4) | (7 << 8);
    constexpr int COLS_Z = 5 | (4 << 4) | (2 << 8);
    const int ia = t / (npy * npz), ja = (t / npz) % npy, ka = t % npz;
    const int sx = npy * npz, sy = npz;
    double dj_self[3];
    {
        const double* J = sm + (size_t)t * W + JOFF;
        const double d0 = dps[ia * npx + ia], d1 = dps[M2 + ja * npy + ja],
                     d2 = dps[2 * M2 + ka * npz + ka];
        dj_self[0] = J[0] * d0 + J[3] * d1 + J[5] * d2;
        dj_self[1] = J[6] * d0 + J[1] * d1 + J[4] * d2;
        dj_self[2] = J[8] * d0 + J[7] * d1 + J[2] * d2;
    }
    const int L = npx + npy + npz - 2;
    const int xb = ia, yb = ia + ja, zb = ia + ja + ka;   /* ends of X<, Y<, Z< */
    const int za = ia + ja + npz;                         /* end of Z> */
    const int ya = ia + npy + npz - 1;                    /* end of Y> */
#pragma unroll 1
    for (int p = 0; p < L; p++) {
        /* direction of position p and the source's index q along that line */
        const bool on_x = p < xb || p >= ya;
        const bool on_y = !on_x && (p < yb || p >= za);
        const int q = on_x ? (p < xb ? p : p - npy - npz + 2)
                    : on_y ? (p < yb ? p - ia : p - ia - npz + 1)
                           : p - ia - ja;               /* Z line; q == ka at the node itself */
        const int da = on_x ? ia : on_y ? ja : ka;
        const int dn = on_x ? npx : on_y ? npy : npz;
        const int st = on_x ? sx : on_y ? sy : 1;
        const int off = on_x ? 0 : on_y ? M2 : 2 * M2;
        const int cols = on_x ? COLS_X : on_y ? COLS_Y : COLS_Z;
        const int lb = t + (q - da) * st;
        const bool self = p == zb;
        const double* J = sm + (size_t)lb * W + JOFF;
        const double D = dps[off + q * dn + da];
        const double l0 = J[cols & 15] * D, l1 = J[(cols >> 4) & 15] * D, l2 = J[cols >> 8] * D;
        const double dj[3] = {self ? dj_self[0] : l0, self ? dj_self[1] : l1, self ? dj_self[2] : l2};
        apply(lb, dj);
    }
}

#endif
