/*
 * Non-conforming (2:1) faces of adaptively refined meshes, shared by the FP64
 * kernels (scatter_non_conforming / gather_non_conforming,
 * src/field/field.h:2019-2248): on a mortar face the coarse cell's side of
 * each face quantity is interpolated from the coarse face's nodes onto the
 * finer mortar nodes (psiRef along the face's two axes), and the face values
 * are projected back onto the coarse face's nodes (psiCor) before the coarse
 * cell lifts them.  Compiled with --fmad=false like the kernels that use it.
 */
#ifndef NSEM_MORTAR_CUH
#define NSEM_MORTAR_CUH

#include "nsem_internal.h"

__device__ __forceinline__ int32_t ms_field(const NsemDev& m, int f, int64_t ms) {
    return m.ms_i[(int64_t)f * m.n_ms + ms];
}

/* sum over the coarse face's nodes of Q(node) psiRef_a psiRef_b, in the
 * reference's order (coarse index along a outer, along b inner) */
template <int NQ, typename Q>
__device__ __forceinline__ void mortar_interp(const NsemDev& m, int64_t ms, Q q, double* out) {
    const int base = ms_field(m, NSEM_MS_BASE, ms), sa = ms_field(m, NSEM_MS_SA, ms),
              sb = ms_field(m, NSEM_MS_SB, ms), Na = ms_field(m, NSEM_MS_NA, ms),
              Nb = ms_field(m, NSEM_MS_NB, ms), ia = ms_field(m, NSEM_MS_IA, ms),
              ib = ms_field(m, NSEM_MS_IB, ms);
    const double* Pa = m.psir + ms_field(m, NSEM_MS_TA, ms) * NSEM_MAX_NPD * NSEM_MAX_NPD;
    const double* Pb = m.psir + ms_field(m, NSEM_MS_TB, ms) * NSEM_MAX_NPD * NSEM_MAX_NPD;
    for (int c = 0; c < NQ; c++) out[c] = 0.0;
    for (int na = 0; na < Na; na++)
        for (int nb = 0; nb < Nb; nb++) {
            double v[NQ];
            q((int64_t)base + na * sa + nb * sb, v);
            const double fa = Pa[na * Na + ia], fb = Pb[nb * Nb + ib];
            for (int c = 0; c < NQ; c++) out[c] += v[c] * fa * fb;
        }
}

/* projection of the face's values src (NC arrays over its mortar slots) onto
 * this slot's coarse node: sum over the face's slots of src psiCor_a psiCor_b */
template <int NC>
__device__ __forceinline__ void mortar_project(const NsemDev& m, int64_t ms, double* const* src,
                                               double* out) {
    const int Na = ms_field(m, NSEM_MS_NA, ms), Nb = ms_field(m, NSEM_MS_NB, ms),
              na = ms_field(m, NSEM_MS_IA, ms), nb = ms_field(m, NSEM_MS_IB, ms),
              first = ms_field(m, NSEM_MS_FIRST, ms);
    const double* Pa = m.psic + ms_field(m, NSEM_MS_TA, ms) * NSEM_MAX_NPD * NSEM_MAX_NPD;
    const double* Pb = m.psic + ms_field(m, NSEM_MS_TB, ms) * NSEM_MAX_NPD * NSEM_MAX_NPD;
    for (int c = 0; c < NC; c++) out[c] = 0.0;
    for (int ja = 0; ja < Na; ja++)
        for (int jb = 0; jb < Nb; jb++) {
            const int64_t s2 = first + ja * Nb + jb;
            const double fa = Pa[ja * Na + na], fb = Pb[jb * Nb + nb];
            for (int c = 0; c < NC; c++) out[c] += src[c][s2] * fa * fb;
        }
}

#endif
