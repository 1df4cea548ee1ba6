/*
 * Internal device data layout shared by the host side (nsem_api.cpp) and the
 * kernels (nsem_fp64.cu, nsem_mixed.cu).
 *
 * HBM layout, all structure-of-arrays so that consecutive threads touch
 * consecutive addresses:
 *   node arrays   [n_int]       state u[5], stage s[5], primitives prim[7]
 *                               (U0,U1,U2,theta,p',|U|,c), Jinv*cV jin[9],
 *                               cV, rho_ref, p_ref, gh, lift[3]
 *   slot arrays   [n_slot]      used face slots in the reference's slot order:
 *                               owner c1, neighbour c2 (-1: boundary ghost),
 *                               bc, fI, weighted normal fN[3], unit normal en[3],
 *                               lifted fluxes d[5]
 * lift[j][a] lists, in the order the reference's div_flux visits them
 * (field.h:3097-3113), the slots touching interior node a: value
 * (slot << 1) | (a is the neighbour side), or -1.
 */
#ifndef NSEM_INTERNAL_H
#define NSEM_INTERNAL_H

#include <stdint.h>

#define NSEM_MAX_NPD 10          /* up to order 9 per direction */
#define NSEM_NPRIM 7
#define NSEM_STATUS_NONFINITE 1u

struct NsemTables {
    double dpsi[3][NSEM_MAX_NPD * NSEM_MAX_NPD]; /* dpsi[d][s*npd + i] = l_i'(x_s) */
};

/* per mortar slot (ms_i rows): its used slot, the coarse side (1: c1, 2: c2),
 * the coarse face's node (0, 0), node strides and node counts along the face's
 * two in-plane axes, their 2:1 table ids (axis * 2 + half), the slot's position
 * on the face, and the face's first mortar slot */
enum { NSEM_MS_K, NSEM_MS_SIDE, NSEM_MS_BASE, NSEM_MS_SA, NSEM_MS_SB, NSEM_MS_NA, NSEM_MS_NB,
       NSEM_MS_TA, NSEM_MS_TB, NSEM_MS_IA, NSEM_MS_IB, NSEM_MS_FIRST, NSEM_MS_FIELDS };

struct NsemDev {
    int32_t npx, npy, npz, np;
    int64_t n_elem, n_int, n_slot;
    /* physical constants */
    double P0, R, gamma, gR, cv_heat, cp, T0;
    double nu, iPr;    /* artificial viscosity (segregated scheme), 1 / Pr */
    double g[3];
    /* node arrays */
    double* jin;       /* [9][n_int] */
    double* cv;
    double* rho_ref;
    double* p_ref;
    double* gh;
    int32_t* lift;     /* [n_lift][n_int]: (index << 2) | (mortar coarse side << 1) | subtract */
    int32_t n_lift;    /* entries per node: 3 on a conforming mesh */
    /* non-conforming (2:1) faces, segregated scheme only */
    int64_t n_ms;      /* mortar slots (0: conforming mesh) */
    int32_t* ms_of;    /* [n_slot] mortar slot of a used slot, -1 */
    int32_t* ms_i;     /* [NSEM_MS_FIELDS][n_ms], fields below */
    double* psir;      /* [6][NSEM_MAX_NPD^2] DG::psiRef, row stride npd */
    double* psic;      /* [6][NSEM_MAX_NPD^2] DG::psiCor */
    /* slot arrays */
    int32_t* c1;
    int32_t* c2;
    uint8_t* bc;
    double* fi;
    double* fn;        /* [3][n_slot] */
    double* en;        /* [3][n_slot] */
    /* element -> geometry for the mixed form (affine per element) */
    float* ejin;       /* [9][n_elem] Jinv*cV/w at element level (mixed form) */
    /* status word (bit flags) */
    uint32_t* status;
};

/* Buffers of one solver state. */
struct NsemBuf {
    double* u[5];      /* state u^n                    */
    double* s[5];      /* stage state                  */
    double* prim[NSEM_NPRIM];
    double* d[5];      /* face fluxes per used slot    */
    double* L[5];      /* tendency output (nsem_tendency) */
    double* G[12];     /* viscous runs: grad U, grad theta of the stage state */
    double* fF[4];     /* viscous runs: per-slot scratch of the gradients   */
    /* non-conforming faces, per mortar slot (shared with the segregated scheme) */
    double* mq[19];    /* the coarse side's interpolated quantities */
    double* mf[15];    /* face flux vectors / tensors */
    double* dC[5];     /* projected, lifted coarse-side fluxes */
    double* gC[4];     /* projected cds(U), cds(theta) */
};

#ifdef __cplusplus
extern "C" {
#endif
/* FP64 (plain) form launchers, nsem_fp64.cu.  stage: 0 = tendency only
 * (writes L), 1..3 = Shu-Osher stage. */
int nsem_fp64_prim(const NsemDev* m, NsemBuf* b, int from_state, void* stream);
int nsem_fp64_face(const NsemDev* m, NsemBuf* b, int from_state, void* stream);
int nsem_fp64_volume(const NsemDev* m, const NsemTables* t, NsemBuf* b, int stage,
                     double dt, void* stream);
int nsem_fp64_check_smem(const NsemDev* m);
#ifdef __cplusplus
}
#endif

#endif
