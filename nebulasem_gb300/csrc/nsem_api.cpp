/*
 * Host side of libnsem_gpu: the C ABI of include/nsem.h.
 *
 * Converts the reference's mesh layout (Mesh:: / DG:: globals) into the
 * device layout of nsem_internal.h, owns all device memory of a context,
 * captures the RK step launches into CUDA graphs and reports errors as
 * nsem_status codes.  Compiled with -ffp-contract=off: the host-side products
 * it precomputes (Jinv*cV, unit normals, hydrostatic background) must round
 * exactly like the reference's.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "nsem.h"
#include "nsem_internal.h"
#include "nsem_adjoint.h"
#include "nsem_mixed.h"
#include "nsem_seg.h"

struct nsem_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    NsemDev dev{};
    NsemTables tab{};
    NsemBuf buf{};
    NsemMixedBuf mbuf{};
    NsemAdjBuf abuf{};
    NsemSegBuf sbuf{};
    NsemConvBuf cbuf{};
    bool mixed_ready = false;
    /* where the state lives: 0 conserved in buf.u; 1 perturbation in
     * mbuf.U[cur]; 2 primitive fields in sbuf (segregated scheme); 3 as the
     * caller passed it to nsem_set_state: rho in buf.u[0], rho theta in
     * buf.u[4], rho U (AoS) in scratch_aos -- converted on first use, straight
     * into the form that steps it */
    int rep = 0;
    bool seg_pp_valid = false;   /* sbuf.pp holds the p' of the last segregated step */
    int adj_form = -1;           /* form of the last checkpointed forward run (-1: none) */
    double dt = 0, T0 = 0;
    int64_t n_all = 0;
    std::vector<void*> allocations;
    std::vector<int64_t> slot_ghost;  /* per used slot: its ghost node (-1: interior face) */
    double* scratch_aos = nullptr;   /* [3*n_int] AoS staging for rhoU */
    double* red = nullptr;           /* reduction partials */
    double* h_red = nullptr;         /* pinned host copy of the reduction result */
    uint32_t* h_status = nullptr;    /* pinned host copy of the status word */
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;  /* key: (form*2 + cur, nsteps) */
    std::string err;
};

namespace {

enum { XX, YY, ZZ, XY, YZ, XZ, YX, ZY, ZX };

nsem_status fail(nsem_ctx* c, nsem_status s, const std::string& msg) {
    if (c) c->err = msg;
    return s;
}

/* calls built for conforming faces only: the precision form's adjoint and the
 * per-launch profile of the FP64 forms */
nsem_status require_conforming(nsem_ctx* c) {
    if (c && c->dev.n_ms > 0)
        return fail(c, NSEM_UNSUPPORTED,
                    "non-conforming (2:1) faces: this call is built for conforming meshes "
                    "(the FP64 forms, the precision form's steps and the FP64 adjoint "
                    "take them)");
    return NSEM_OK;
}

nsem_status cuda_fail(nsem_ctx* c, cudaError_t e, const char* where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    return fail(c, NSEM_CUDA_ERROR, m);
}

#define NSEM_CUDA(call)                                               \
    do {                                                              \
        cudaError_t e_ = (call);                                      \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);      \
    } while (0)

template <typename T>
nsem_status dalloc(nsem_ctx* ctx, T** p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(ctx, NSEM_NO_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    ctx->allocations.push_back((void*)*p);
    return NSEM_OK;
}

template <typename T>
nsem_status upload(nsem_ctx* ctx, T** p, const std::vector<T>& h) {
    nsem_status s = dalloc(ctx, p, h.size());
    if (s != NSEM_OK) return s;
    NSEM_CUDA(cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return NSEM_OK;
}

inline double vdot3(const double* a, const double* b) {
    return a[0] * b[0] + (a[1] * b[1] + (a[2] * b[2] + 0.0));
}

nsem_status check_desc(nsem_ctx* ctx, const nsem_mesh_desc* m) {
    if (!m) return fail(ctx, NSEM_BAD_ARG, "mesh description is NULL");
    const int npd[3] = {m->npx, m->npy, m->npz};
    for (int d = 0; d < 3; d++) {
        if (npd[d] < 1 || npd[d] > NSEM_MAX_NPD)
            return fail(ctx, NSEM_UNSUPPORTED, "nodes per direction must be 1..10");
        if (!m->psi[d] || !m->dpsi[d]) return fail(ctx, NSEM_BAD_ARG, "psi/dpsi table is NULL");
    }
    if (m->n_elem <= 0 || m->n_cells < m->n_elem || m->n_face < 0 || m->npf <= 0)
        return fail(ctx, NSEM_BAD_ARG, "inconsistent element/cell/face counts");
    if (!m->cC || !m->cV || !m->Jinv || !m->FO || !m->FN || !m->fN || !m->fI ||
        !m->all_faces || !m->face_idx0 || !m->face_idx1 || !m->bc_U)
        return fail(ctx, NSEM_BAD_ARG, "a mesh array is NULL");
    const int64_t np = (int64_t)m->npx * m->npy * m->npz;
    if ((int64_t)m->n_cells * np >= (int64_t)0x7fffffff)
        return fail(ctx, NSEM_UNSUPPORTED, "more than 2^31 nodes");
    /* the volume gather assumes nodal (Kronecker) basis values at LGL points */
    for (int d = 0; d < 3; d++)
        for (int s = 0; s < npd[d]; s++)
            for (int i = 0; i < npd[d]; i++)
                if (m->psi[d][s * npd[d] + i] != (s == i ? 1.0 : 0.0))
                    return fail(ctx, NSEM_UNSUPPORTED, "psi is not the identity at LGL nodes");
    return NSEM_OK;
}

nsem_status build_device_mesh(nsem_ctx* ctx, const nsem_mesh_desc* m, const nsem_params* p) {
    NsemDev& D = ctx->dev;
    D.npx = m->npx; D.npy = m->npy; D.npz = m->npz;
    D.np = m->npx * m->npy * m->npz;
    const int64_t NP = D.np;
    D.n_elem = m->n_elem;
    D.n_int = (int64_t)m->n_elem * NP;
    const int64_t n_int = D.n_int;
    const int64_t n_all = (int64_t)m->n_cells * NP;
    ctx->n_all = n_all;
    const int64_t n_slot_all = (int64_t)m->n_face * m->npf;

    D.R = p->cp - p->cv;
    D.gamma = p->cp / p->cv;
    D.gR = D.gamma * D.R;
    D.P0 = p->P0;
    D.cp = p->cp;
    D.T0 = p->T0;
    D.nu = p->viscosity;
    D.iPr = p->viscosity != 0.0 ? 1 / p->Pr : 0.0;
    D.cv_heat = p->cv;
    for (int c = 0; c < 3; c++) D.g[c] = p->gravity[c];
    ctx->dt = p->dt;
    ctx->T0 = p->T0;

    /* tables: dpsi[d][s*npd + i] */
    const int npd[3] = {m->npx, m->npy, m->npz};
    std::memset(&ctx->tab, 0, sizeof(ctx->tab));
    for (int d = 0; d < 3; d++)
        for (int q = 0; q < npd[d] * npd[d]; q++) ctx->tab.dpsi[d][q] = m->dpsi[d][q];

    /* used slots in reference order */
    std::vector<int64_t> compact(n_slot_all, -1);
    std::vector<int32_t> c1, c2;
    std::vector<uint8_t> bc;
    std::vector<double> fi, fn[3], en[3];
    for (int64_t k = 0; k < n_slot_all; k++) {
        const uint32_t o = m->FO[k], n = m->FN[k];
        if (o >= (uint64_t)n_all || n >= (uint64_t)n_all) continue;
        if (o >= (uint64_t)n_int)
            return fail(ctx, NSEM_BAD_ARG, "face slot owner is not an interior node");
        compact[k] = (int64_t)c1.size();
        c1.push_back((int32_t)o);
        const bool ghost = n >= (uint64_t)n_int;
        c2.push_back(ghost ? -1 : (int32_t)n);
        ctx->slot_ghost.push_back(ghost ? (int64_t)n : -1);
        if (ghost && m->bc_U[k] == 0)
            return fail(ctx, NSEM_BAD_ARG, "boundary slot without a boundary condition");
        if (m->bc_U[k] > 2) return fail(ctx, NSEM_UNSUPPORTED, "velocity BC other than NEUMANN/SYMMETRY");
        bc.push_back(ghost ? (uint8_t)m->bc_U[k] : 0);
        fi.push_back(m->fI[k]);
        const double* v = m->fN + 3 * k;
        const double mg = std::sqrt(vdot3(v, v));
        for (int c = 0; c < 3; c++) {
            fn[c].push_back(v[c]);
            en[c].push_back(v[c] / mg);
        }
    }
    D.n_slot = (int64_t)c1.size();

    /* non-conforming faces: per used slot of a mortar face the coarse side
     * (1: FO, 2: FN) and its mortar slot; mortar slots numbered face by face,
     * (ia, ib) row-major over the face's in-plane node counts */
    std::vector<int8_t> mside(n_slot_all, 0);
    std::vector<int32_t> ms_full(n_slot_all, -1);
    std::vector<int32_t> msi[NSEM_MS_FIELDS];
    if (m->n_mortar < 0 || (m->n_mortar > 0 && !m->mortar))
        return fail(ctx, NSEM_BAD_ARG, "mortar faces: bad count or NULL list");
    if (m->n_mortar > 0) {
        for (int t = 0; t < 6; t++)
            if (!m->psi_ref[t] || !m->psi_cor[t])
                return fail(ctx, NSEM_BAD_ARG, "mortar faces need psi_ref / psi_cor");
        const int64_t stride[3] = {(int64_t)m->npy * m->npz, m->npz, 1};
        for (int32_t q = 0; q < m->n_mortar; q++) {
            const uint32_t* r = m->mortar + 4 * (size_t)q;
            const int64_t fi = r[0];
            const int fm = (int)r[1], fid = (int)r[2];
            if (fi >= m->n_face || (fm != 1 && fm != 2) || fid > 5 || r[3] > 3)
                return fail(ctx, NSEM_BAD_ARG, "mortar face entry out of range");
            int a, b, fix;
            if (fid <= 1) { a = 0; b = 1; fix = 2; }
            else if (fid <= 3) { a = 0; b = 2; fix = 1; }
            else { a = 1; b = 2; fix = 0; }
            const int Na = npd[a], Nb = npd[b];
            if ((int64_t)Na * Nb > m->npf) return fail(ctx, NSEM_BAD_ARG, "mortar face larger than npf");
            const uint32_t cnode = fm == 1 ? m->FN[fi * m->npf] : m->FO[fi * m->npf];
            if (cnode >= (uint64_t)n_int) return fail(ctx, NSEM_BAD_ARG, "mortar coarse cell is not interior");
            const int64_t cell = cnode / NP;
            const int64_t base = cell * NP + ((fid & 1) ? npd[fix] - 1 : 0) * stride[fix];
            const int32_t first = (int32_t)msi[0].size();
            for (int ia = 0; ia < Na; ia++)
                for (int ib = 0; ib < Nb; ib++) {
                    const int64_t k = fi * m->npf + (int64_t)ia * Nb + ib;
                    if (compact[k] < 0) return fail(ctx, NSEM_BAD_ARG, "mortar slot unused");
                    if (m->FN[k] >= (uint64_t)n_int) return fail(ctx, NSEM_BAD_ARG, "mortar face on a boundary");
                    if (ms_full[k] >= 0) return fail(ctx, NSEM_BAD_ARG, "mortar face listed twice");
                    ms_full[k] = (int32_t)msi[0].size();
                    mside[k] = (int8_t)(fm == 2 ? 1 : 2);
                    const int32_t f[NSEM_MS_FIELDS] = {
                        (int32_t)compact[k], fm == 2 ? 1 : 2, (int32_t)base,
                        (int32_t)stride[a], (int32_t)stride[b], Na, Nb,
                        2 * a + (int)(r[3] & 1), 2 * b + (int)((r[3] >> 1) & 1), ia, ib, first};
                    for (int c = 0; c < NSEM_MS_FIELDS; c++) msi[c].push_back(f[c]);
                }
        }
    }
    D.n_ms = (int64_t)msi[0].size();

    /* per-node lift lists in div_flux order (field.h:3097-3113): the used slot
     * (or, on a mortar's coarse side, the mortar slot) << 2, bit 1 the coarse
     * side, bit 0 subtract */
    std::vector<std::vector<int32_t>> lists(n_int);
    for (int64_t e = 0; e < m->n_elem; e++) {
        const int64_t lo = e * NP, hi = lo + NP;
        for (uint32_t f = m->face_idx0[e]; f < m->face_idx1[e]; f++) {
            for (int q = 0; q < m->npf; q++) {
                const int64_t k = (int64_t)m->all_faces[f] * m->npf + q;
                if (k >= n_slot_all) return fail(ctx, NSEM_BAD_ARG, "face id out of range");
                const uint32_t o = m->FO[k], n = m->FN[k];
                int64_t node;
                int neg;
                if (o >= lo && o < hi) { node = o; neg = 0; }
                else if (n < (uint64_t)n_all) { node = n; neg = 1; }
                else continue;
                if (node < lo || node >= hi)
                    return fail(ctx, NSEM_BAD_ARG, "face slot does not belong to its cell");
                if (compact[k] < 0) return fail(ctx, NSEM_BAD_ARG, "lift from an unused slot");
                const bool coarse = mside[k] == (neg ? 2 : 1);
                const int64_t idx = coarse ? ms_full[k] : compact[k];
                if (idx >= (int64_t)1 << 29) return fail(ctx, NSEM_UNSUPPORTED, "more than 2^29 face slots");
                lists[node].push_back((int32_t)((idx << 2) | (coarse ? 2 : 0) | neg));
            }
        }
    }
    size_t n_lift = 3;
    for (const auto& l : lists) n_lift = std::max(n_lift, l.size());
    if (m->n_mortar == 0 && n_lift > 3) return fail(ctx, NSEM_BAD_ARG, "node on more than 3 faces");
    D.n_lift = (int32_t)n_lift;
    std::vector<int32_t> lift(n_lift * n_int, -1);
    for (int64_t i = 0; i < n_int; i++)
        for (size_t j = 0; j < lists[i].size(); j++) lift[(int64_t)j * n_int + i] = lists[i][j];

    /* node arrays: Jinv*cV (field.h:3445), cV, background */
    std::vector<double> jin(9 * n_int), cv(n_int), pref(n_int), rref(n_int), gh(n_int);
    for (int64_t i = 0; i < n_int; i++) {
        cv[i] = m->cV[i];
        for (int c = 0; c < 9; c++) jin[(int64_t)c * n_int + i] = m->Jinv[9 * i + c] * m->cV[i];
        /* gh = g . cC (euler.cpp:114), right-nested like the reference's Vector dot */
        gh[i] = vdot3(p->gravity, m->cC + 3 * i);
    }
    const double R = D.R, gam = D.gamma, P0 = p->P0, cp = p->cp, T0 = p->T0;
    for (int64_t i = 0; i < n_int; i++) {
        /* euler.cpp:122-123 */
        pref[i] = p->p_ref ? p->p_ref[i] : P0 * std::pow(1.0 + gh[i] / (cp * T0), cp / R);
        rref[i] = p->rho_ref ? p->rho_ref[i] : (P0 / (R * T0)) * std::pow(pref[i] / P0, 1 / gam);
    }

    nsem_status s;
#define UP(ptr, vec) if ((s = upload(ctx, &(ptr), vec)) != NSEM_OK) return s
    UP(D.jin, jin);
    UP(D.cv, cv);
    UP(D.p_ref, pref);
    UP(D.rho_ref, rref);
    UP(D.gh, gh);
    UP(D.lift, lift);
    if (D.n_ms > 0) {
        std::vector<int32_t> ms_of(D.n_slot, -1), ms_i;
        for (int64_t k = 0; k < n_slot_all; k++)
            if (ms_full[k] >= 0) ms_of[compact[k]] = ms_full[k];
        for (int c = 0; c < NSEM_MS_FIELDS; c++) ms_i.insert(ms_i.end(), msi[c].begin(), msi[c].end());
        std::vector<double> pr(6 * NSEM_MAX_NPD * NSEM_MAX_NPD, 0.0), pc(pr.size(), 0.0);
        for (int t = 0; t < 6; t++) {
            const int n = npd[t / 2];
            for (int q = 0; q < n * n; q++) {
                pr[t * NSEM_MAX_NPD * NSEM_MAX_NPD + q] = m->psi_ref[t][q];
                pc[t * NSEM_MAX_NPD * NSEM_MAX_NPD + q] = m->psi_cor[t][q];
            }
        }
        UP(D.ms_of, ms_of);
        UP(D.ms_i, ms_i);
        UP(D.psir, pr);
        UP(D.psic, pc);
    }
    UP(D.c1, c1);
    UP(D.c2, c2);
    UP(D.bc, bc);
    UP(D.fi, fi);
    std::vector<double> fn3, en3;
    for (int c = 0; c < 3; c++) {
        fn3.insert(fn3.end(), fn[c].begin(), fn[c].end());
        en3.insert(en3.end(), en[c].begin(), en[c].end());
    }
    UP(D.fn, fn3);
    UP(D.en, en3);
#undef UP
    if ((s = dalloc(ctx, &D.status, 1)) != NSEM_OK) return s;
    NSEM_CUDA(cudaMemset(D.status, 0, sizeof(uint32_t)));

    /* state buffers */
    NsemBuf& b = ctx->buf;
    for (int c = 0; c < 5; c++) {
        if ((s = dalloc(ctx, &b.u[c], n_int)) != NSEM_OK) return s;
        if ((s = dalloc(ctx, &b.s[c], n_int)) != NSEM_OK) return s;
        if ((s = dalloc(ctx, &b.d[c], D.n_slot)) != NSEM_OK) return s;
        if ((s = dalloc(ctx, &b.L[c], n_int)) != NSEM_OK) return s;
    }
    for (int c = 0; c < NSEM_NPRIM; c++)
        if ((s = dalloc(ctx, &b.prim[c], n_int)) != NSEM_OK) return s;
    if ((s = dalloc(ctx, &ctx->scratch_aos, 3 * n_int)) != NSEM_OK) return s;
    if ((s = dalloc(ctx, &ctx->red, NSEM_RED_PARTIALS * 6 + 8)) != NSEM_OK) return s;
    NSEM_CUDA(cudaMallocHost((void**)&ctx->h_red, 8 * sizeof(double)));
    NSEM_CUDA(cudaMallocHost((void**)&ctx->h_status, sizeof(uint32_t)));
    *ctx->h_status = 0;

    /* mixed form: per-element affine data, FP32 */
    if ((s = nsem_mixed_setup(ctx->dev, m, &ctx->mbuf, &ctx->allocations, ctx->err)) != NSEM_OK) {
        ctx->mixed_ready = false;
        if (s != NSEM_UNSUPPORTED) return s;
    } else {
        ctx->mixed_ready = true;
    }
    return NSEM_OK;
}

nsem_status check_status(nsem_ctx* ctx) {
    NSEM_CUDA(cudaStreamSynchronize(ctx->stream));
    uint32_t st = *ctx->h_status;
    if (st & NSEM_STATUS_NONFINITE) {
        *ctx->h_status = 0;
        NSEM_CUDA(cudaMemset(ctx->dev.status, 0, sizeof(uint32_t)));
        return fail(ctx, NSEM_NONFINITE, "non-finite value in the state");
    }
    return NSEM_OK;
}

/* move the current state to the representation a form needs */
nsem_status seg_alloc(nsem_ctx* ctx) {
    NsemSegBuf& S = ctx->sbuf;
    if (S.ready) return NSEM_OK;
    const size_t n = (size_t)ctx->dev.n_int, ns = (size_t)ctx->dev.n_slot;
    nsem_status s;
    double** node_arrays[] = {&S.rho[0], &S.rho[1], &S.U[0], &S.U[1], &S.U[2], &S.Tp, &S.Tf,
                              &S.Fc[0], &S.Fc[1], &S.Fc[2], &S.mu, &S.cs, &S.pp};
    for (double** a : node_arrays)
        if ((s = dalloc(ctx, a, n)) != NSEM_OK) return s;
    if ((s = dalloc(ctx, &S.lam, ns)) != NSEM_OK) return s;
    for (int v = 0; v < 5; v++)
        if ((s = dalloc(ctx, &S.d[v], ns)) != NSEM_OK) return s;
    if (ctx->dev.nu != 0.0) {
        for (int c = 0; c < 12; c++)
            if ((s = dalloc(ctx, &S.G[c], n)) != NSEM_OK) return s;
        for (int c = 0; c < 4; c++)
            if ((s = dalloc(ctx, &S.fF[c], ns)) != NSEM_OK) return s;
    }
    if (ctx->dev.n_ms > 0) {
        const size_t nm = (size_t)ctx->dev.n_ms;
        for (int c = 0; c < 19; c++)
            if ((s = dalloc(ctx, &S.mq[c], nm)) != NSEM_OK) return s;
        for (int c = 0; c < 15; c++)
            if ((s = dalloc(ctx, &S.mf[c], nm)) != NSEM_OK) return s;
        for (int c = 0; c < 5; c++)
            if ((s = dalloc(ctx, &S.dC[c], nm)) != NSEM_OK) return s;
        for (int c = 0; c < 4; c++)
            if ((s = dalloc(ctx, &S.gC[c], nm)) != NSEM_OK) return s;
    }
    const int e = nsem_seg_prepare(&ctx->dev);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "segregated-scheme shared memory");
    S.cur = 0;
    S.ready = true;
    return NSEM_OK;
}

nsem_status ensure_rep(nsem_ctx* ctx, int want) {
    if (ctx->rep == want) return NSEM_OK;
    int e = 0;
    if (ctx->rep == 3) {
        if (want == 1 && ctx->mixed_ready) {
            /* one pass from the caller's layout to the precision form */
            if ((e = nsem_mixed_host_layout(&ctx->dev, &ctx->mbuf, 1, ctx->buf.u[0],
                                            ctx->scratch_aos, ctx->buf.u[4], ctx->stream)))
                return cuda_fail(ctx, (cudaError_t)e, "state conversion");
            ctx->rep = 1;
            return NSEM_OK;
        }
        if ((e = nsem_aos_to_soa(ctx->scratch_aos, ctx->buf.u[1], ctx->buf.u[2], ctx->buf.u[3],
                                 ctx->dev.n_int, ctx->stream)))
            return cuda_fail(ctx, (cudaError_t)e, "aos_to_soa");
        ctx->rep = 0;
        if (want == 0) return NSEM_OK;
    }
    if (ctx->rep == 2) {
        /* primitive fields -> conserved state */
        if ((e = nsem_seg_to_cons(&ctx->dev, &ctx->sbuf, ctx->buf.u, ctx->stream)))
            return cuda_fail(ctx, (cudaError_t)e, "state conversion");
        ctx->rep = 0;
        if (want == 0) return NSEM_OK;
    }
    if (want == 2) {
        if (ctx->rep == 1 &&
            (e = nsem_mixed_convert(&ctx->dev, &ctx->mbuf, &ctx->buf, 0, ctx->stream)))
            return cuda_fail(ctx, (cudaError_t)e, "state conversion");
        nsem_status s = seg_alloc(ctx);
        if (s != NSEM_OK) return s;
        if ((e = nsem_cons_to_seg(&ctx->dev, &ctx->sbuf, ctx->buf.u, ctx->stream)))
            return cuda_fail(ctx, (cudaError_t)e, "state conversion");
        ctx->rep = 2;
        return NSEM_OK;
    }
    e = nsem_mixed_convert(&ctx->dev, &ctx->mbuf, &ctx->buf, want == 1, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "state conversion");
    ctx->rep = want;
    return NSEM_OK;
}

/* the conserved state in buf.u for reading, without moving the state out of
 * the primitive fields (a segregated run stays bit-exact across reads) */
nsem_status materialise_conserved(nsem_ctx* ctx) {
    if (ctx->rep == 2) {
        const int e = nsem_seg_to_cons(&ctx->dev, &ctx->sbuf, ctx->buf.u, ctx->stream);
        return e ? cuda_fail(ctx, (cudaError_t)e, "state conversion") : NSEM_OK;
    }
    return ensure_rep(ctx, 0);
}

/* the FP64 face kernel of a stage, after the gradients of its state when the
 * run is viscous */
int fp64_face(nsem_ctx* ctx, int from_state) {
    NsemBuf* b = &ctx->buf;
    if (b->G[0]) {
        const double* U[3] = {b->prim[0], b->prim[1], b->prim[2]};
        const int e = nsem_grad_ut_mortar(&ctx->dev, &ctx->tab, U, b->prim[3], b->G, b->fF,
                                          ctx->dev.n_ms > 0 ? b->gC : nullptr, ctx->stream);
        if (e) return e;
    }
    return nsem_fp64_face(&ctx->dev, b, from_state, ctx->stream);
}

/* launches of one nsem_step call (captured into a graph) */
nsem_status enqueue_steps(nsem_ctx* ctx, int nsteps, nsem_precision prec) {
    NsemDev* D = &ctx->dev;
    NsemBuf* b = &ctx->buf;
    void* st = (void*)ctx->stream;
    int e;
    if (prec == NSEM_FP64) {
        if ((e = nsem_fp64_prim(D, b, 1, st))) return cuda_fail(ctx, (cudaError_t)e, "prim");
        for (int n = 0; n < nsteps; n++) {
            for (int stage = 1; stage <= 3; stage++) {
                if ((e = fp64_face(ctx, stage == 1)))
                    return cuda_fail(ctx, (cudaError_t)e, "face");
                if ((e = nsem_fp64_volume(D, &ctx->tab, b, stage, ctx->dt, st)))
                    return cuda_fail(ctx, (cudaError_t)e, "volume");
            }
        }
    } else {
        if (!ctx->mixed_ready) return fail(ctx, NSEM_UNSUPPORTED, ctx->err);
        if ((e = nsem_mixed_steps(D, &ctx->mbuf, b, &ctx->tab, nsteps, ctx->dt, st)))
            return cuda_fail(ctx, (cudaError_t)e, "mixed step");
    }
    return NSEM_OK;
}

}  // namespace

extern "C" {

int nsem_abi_version(void) { return NSEM_ABI_VERSION; }

const char* nsem_last_error(const nsem_ctx* ctx) {
    return ctx ? ctx->err.c_str() : "context is NULL";
}

int64_t nsem_num_nodes(const nsem_ctx* ctx) { return ctx ? ctx->dev.n_int : 0; }

void* nsem_stream(const nsem_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

nsem_status nsem_create(const nsem_mesh_desc* mesh, const nsem_params* params, nsem_ctx** out) {
    if (!out) return NSEM_BAD_ARG;
    *out = nullptr;
    nsem_ctx* ctx = new (std::nothrow) nsem_ctx();
    if (!ctx) return NSEM_NO_MEMORY;
    *out = ctx;
    if (!params) return fail(ctx, NSEM_BAD_ARG, "params is NULL");
    if (params->viscosity != 0.0 && !(params->viscosity > 0 && params->Pr > 0))
        return fail(ctx, NSEM_BAD_ARG, "viscosity must be >= 0, with Pr > 0 when it is not 0");
    if (!(params->cp > params->cv) || !(params->cv > 0) || !(params->P0 > 0) || !(params->T0 > 0))
        return fail(ctx, NSEM_BAD_ARG, "invalid fluid properties");
    nsem_status s = check_desc(ctx, mesh);
    if (s != NSEM_OK) return s;
    ctx->device = params->device;
    NSEM_CUDA(cudaSetDevice(ctx->device));
    NSEM_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    s = build_device_mesh(ctx, mesh, params);
    if (s != NSEM_OK) return s;
    int e = nsem_fp64_check_smem(&ctx->dev);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "volume kernel shared memory");
    if (ctx->dev.nu != 0.0) {
        /* viscous runs: gradient buffers shared by the coupled and the
         * segregated schemes (the precision form keeps its own FP32 ones) */
        if ((s = seg_alloc(ctx)) != NSEM_OK) return s;
        for (int c = 0; c < 12; c++) ctx->buf.G[c] = ctx->sbuf.G[c];
        for (int c = 0; c < 4; c++) ctx->buf.fF[c] = ctx->sbuf.fF[c];
    }
    if (ctx->dev.n_ms > 0) {
        /* non-conforming faces: mortar buffers shared by both FP64 schemes */
        if ((s = seg_alloc(ctx)) != NSEM_OK) return s;
        for (int c = 0; c < 19; c++) ctx->buf.mq[c] = ctx->sbuf.mq[c];
        for (int c = 0; c < 15; c++) ctx->buf.mf[c] = ctx->sbuf.mf[c];
        for (int c = 0; c < 5; c++) ctx->buf.dC[c] = ctx->sbuf.dC[c];
        for (int c = 0; c < 4; c++) ctx->buf.gC[c] = ctx->sbuf.gC[c];
    }
    return NSEM_OK;
}

void nsem_destroy(nsem_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
    for (void* p : ctx->allocations) cudaFree(p);
    if (ctx->abuf.ckpt) cudaFree(ctx->abuf.ckpt);
    if (ctx->abuf.seg) cudaFree(ctx->abuf.seg);
    {
        NsemMixedBuf& M = ctx->mbuf;
        void* mp[] = {M.ckpt, M.seg, M.lam, M.fin, M.abar[0], M.abar[1], M.abar[2], M.GB, M.XB,
                      M.mxa_db, M.mxa_dCb, M.mxa_qb, M.mxa_xf, M.mxa_gf, M.mxa_gFb, M.mxa_gCb,
                      M.mxa_vh, M.mxa_vown};
        for (void* p : mp)
            if (p) cudaFree(p);
    }
    if (ctx->h_red) cudaFreeHost(ctx->h_red);
    if (ctx->h_status) cudaFreeHost(ctx->h_status);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

nsem_status nsem_set_state(nsem_ctx* ctx, const double* rho, const double* rhoU,
                           const double* rhoTheta) {
    if (!ctx) return NSEM_BAD_ARG;
    if (!rho || !rhoU || !rhoTheta) return fail(ctx, NSEM_BAD_ARG, "state pointer is NULL");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    const size_t n = (size_t)ctx->dev.n_int;
    NSEM_CUDA(cudaMemcpyAsync(ctx->buf.u[0], rho, n * 8, cudaMemcpyHostToDevice, ctx->stream));
    NSEM_CUDA(cudaMemcpyAsync(ctx->buf.u[4], rhoTheta, n * 8, cudaMemcpyHostToDevice, ctx->stream));
    NSEM_CUDA(cudaMemcpyAsync(ctx->scratch_aos, rhoU, 3 * n * 8, cudaMemcpyHostToDevice, ctx->stream));
    /* converted when first used, into the form that uses it */
    ctx->rep = 3;
    return NSEM_OK;
}

nsem_status nsem_get_state(nsem_ctx* ctx, double* rho, double* rhoU, double* rhoTheta) {
    if (!ctx) return NSEM_BAD_ARG;
    if (!rho || !rhoU || !rhoTheta) return fail(ctx, NSEM_BAD_ARG, "state pointer is NULL");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    const size_t n = (size_t)ctx->dev.n_int;
    if (ctx->rep == 1) {
        /* precision form: one pass into the caller's layout; the state stays
         * where it is (a following precision-form step needs no conversion) */
        int e = nsem_mixed_host_layout(&ctx->dev, &ctx->mbuf, 0, ctx->buf.u[0], ctx->scratch_aos,
                                       ctx->buf.u[4], ctx->stream);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "state conversion");
        NSEM_CUDA(cudaMemcpyAsync(rho, ctx->buf.u[0], n * 8, cudaMemcpyDeviceToHost, ctx->stream));
        NSEM_CUDA(cudaMemcpyAsync(rhoTheta, ctx->buf.u[4], n * 8, cudaMemcpyDeviceToHost, ctx->stream));
        NSEM_CUDA(cudaMemcpyAsync(rhoU, ctx->scratch_aos, 3 * n * 8, cudaMemcpyDeviceToHost, ctx->stream));
        return check_status(ctx);
    }
    nsem_status rs = materialise_conserved(ctx);
    if (rs != NSEM_OK) return rs;
    int e = nsem_soa_to_aos(ctx->buf.u[1], ctx->buf.u[2], ctx->buf.u[3], ctx->scratch_aos,
                            ctx->dev.n_int, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "soa_to_aos");
    NSEM_CUDA(cudaMemcpyAsync(rho, ctx->buf.u[0], n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    NSEM_CUDA(cudaMemcpyAsync(rhoTheta, ctx->buf.u[4], n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    NSEM_CUDA(cudaMemcpyAsync(rhoU, ctx->scratch_aos, 3 * n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    return check_status(ctx);
}

nsem_status nsem_set_fields(nsem_ctx* ctx, const double* rho, const double* U, const double* T) {
    if (!ctx) return NSEM_BAD_ARG;
    if (!rho || !U || !T) return fail(ctx, NSEM_BAD_ARG, "field pointer is NULL");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    /* the fields are kept as given (the segregated scheme steps them
     * directly); other forms convert them on the device when they step */
    nsem_status s = seg_alloc(ctx);
    if (s != NSEM_OK) return s;
    NsemSegBuf& S = ctx->sbuf;
    const size_t n = (size_t)ctx->dev.n_int;
    NSEM_CUDA(cudaMemcpyAsync(S.rho[S.cur], rho, n * 8, cudaMemcpyHostToDevice, ctx->stream));
    NSEM_CUDA(cudaMemcpyAsync(S.Tp, T, n * 8, cudaMemcpyHostToDevice, ctx->stream));
    NSEM_CUDA(cudaMemcpyAsync(ctx->scratch_aos, U, 3 * n * 8, cudaMemcpyHostToDevice, ctx->stream));
    int e = nsem_aos_to_soa(ctx->scratch_aos, S.U[0], S.U[1], S.U[2], ctx->dev.n_int, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "aos_to_soa");
    ctx->rep = 2;
    ctx->seg_pp_valid = false;
    NSEM_CUDA(cudaStreamSynchronize(ctx->stream));
    return NSEM_OK;
}

nsem_status nsem_get_pressure(nsem_ctx* ctx, double* p_prime) {
    if (!ctx) return NSEM_BAD_ARG;
    if (!p_prime) return fail(ctx, NSEM_BAD_ARG, "p_prime is NULL");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    const size_t n = (size_t)ctx->dev.n_int;
    if (ctx->rep == 2 && ctx->seg_pp_valid) {
        NSEM_CUDA(cudaMemcpyAsync(p_prime, ctx->sbuf.pp, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
        return check_status(ctx);
    }
    nsem_status rs = materialise_conserved(ctx);
    if (rs != NSEM_OK) return rs;
    const int e = nsem_fp64_prim(&ctx->dev, &ctx->buf, 1, (void*)ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "prim");
    NSEM_CUDA(cudaMemcpyAsync(p_prime, ctx->buf.prim[4], n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    return check_status(ctx);
}

nsem_status nsem_get_fields(nsem_ctx* ctx, double* rho, double* U, double* T) {
    if (!ctx) return NSEM_BAD_ARG;
    if (!rho || !U || !T) return fail(ctx, NSEM_BAD_ARG, "field pointer is NULL");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    const int64_t n = ctx->dev.n_int;
    if (ctx->rep == 2) {
        NsemSegBuf& S = ctx->sbuf;
        int e = nsem_soa_to_aos(S.U[0], S.U[1], S.U[2], ctx->scratch_aos, n, ctx->stream);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "soa_to_aos");
        NSEM_CUDA(cudaMemcpyAsync(rho, S.rho[S.cur], n * 8, cudaMemcpyDeviceToHost, ctx->stream));
        NSEM_CUDA(cudaMemcpyAsync(T, S.Tp, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
        NSEM_CUDA(cudaMemcpyAsync(U, ctx->scratch_aos, 3 * n * 8, cudaMemcpyDeviceToHost, ctx->stream));
        return check_status(ctx);
    }
    std::vector<double> ru(3 * n), rt(n);
    nsem_status s = nsem_get_state(ctx, rho, ru.data(), rt.data());
    if (s != NSEM_OK) return s;
    for (int64_t i = 0; i < n; i++) {
        const double r = rho[i];
        for (int c = 0; c < 3; c++) U[3 * i + c] = ru[3 * i + c] / r;
        T[i] = rt[i] / r - ctx->T0;
    }
    return NSEM_OK;
}

nsem_status nsem_tendency(nsem_ctx* ctx, nsem_precision prec, double* const L[5],
                          double* p_prime) {
    if (!ctx) return NSEM_BAD_ARG;
    if (!L) return fail(ctx, NSEM_BAD_ARG, "L is NULL");
    for (int c = 0; c < 5; c++) if (!L[c]) return fail(ctx, NSEM_BAD_ARG, "L[c] is NULL");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    NsemDev* D = &ctx->dev;
    NsemBuf* b = &ctx->buf;
    void* st = (void*)ctx->stream;
    int e;
    if (prec == NSEM_MIXED && !ctx->mixed_ready) return fail(ctx, NSEM_UNSUPPORTED, ctx->err);
    nsem_status rs = (prec == NSEM_MIXED) ? ensure_rep(ctx, 1) : materialise_conserved(ctx);
    if (rs != NSEM_OK) return rs;
    if (prec == NSEM_FP64) {
        if ((e = nsem_fp64_prim(D, b, 1, st))) return cuda_fail(ctx, (cudaError_t)e, "prim");
        if ((e = fp64_face(ctx, 1))) return cuda_fail(ctx, (cudaError_t)e, "face");
        if ((e = nsem_fp64_volume(D, &ctx->tab, b, 0, ctx->dt, st)))
            return cuda_fail(ctx, (cudaError_t)e, "volume");
    } else if (prec == NSEM_MIXED) {
        if (!ctx->mixed_ready) return fail(ctx, NSEM_UNSUPPORTED, ctx->err);
        if ((e = nsem_mixed_tendency(D, &ctx->mbuf, b, &ctx->tab, st)))
            return cuda_fail(ctx, (cudaError_t)e, "mixed tendency");
    } else {
        return fail(ctx, NSEM_BAD_ARG, "unknown precision");
    }
    const size_t n = (size_t)D->n_int;
    for (int c = 0; c < 5; c++)
        NSEM_CUDA(cudaMemcpyAsync(L[c], b->L[c], n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (p_prime && prec == NSEM_FP64)
        NSEM_CUDA(cudaMemcpyAsync(p_prime, b->prim[4], n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    return check_status(ctx);
}

nsem_status nsem_step(nsem_ctx* ctx, int nsteps, nsem_scheme scheme, nsem_precision prec) {
    if (!ctx) return NSEM_BAD_ARG;
    if (nsteps < 0) return fail(ctx, NSEM_BAD_ARG, "nsteps < 0");
    if (scheme != NSEM_SSPRK3 && scheme != NSEM_REF_SEGREGATED)
        return fail(ctx, NSEM_BAD_ARG, "unknown scheme");
    if (prec != NSEM_FP64 && prec != NSEM_MIXED) return fail(ctx, NSEM_BAD_ARG, "unknown precision");
    if (scheme == NSEM_REF_SEGREGATED && prec != NSEM_FP64)
        return fail(ctx, NSEM_UNSUPPORTED, "the segregated scheme runs in FP64 only");
    if (nsteps == 0) return NSEM_OK;
    NSEM_CUDA(cudaSetDevice(ctx->device));
    if (prec == NSEM_MIXED && !ctx->mixed_ready) return fail(ctx, NSEM_UNSUPPORTED, ctx->err);
    const int form = (scheme == NSEM_REF_SEGREGATED) ? 2 : (prec == NSEM_MIXED ? 1 : 0);
    ctx->seg_pp_valid = false;
    nsem_status rs = ensure_rep(ctx, form);
    if (rs != NSEM_OK) return rs;
    const int cur = form == 1 ? ctx->mbuf.cur : form == 2 ? ctx->sbuf.cur : 0;
    auto key = std::make_pair(form * 2 + cur, nsteps);
    auto it = ctx->graphs.find(key);
    if (it == ctx->graphs.end()) {
        cudaGraph_t g;
        NSEM_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        nsem_status s;
        if (form == 2) {
            const int e = nsem_seg_steps(&ctx->dev, &ctx->tab, &ctx->sbuf, nsteps, ctx->dt, ctx->stream);
            s = e ? cuda_fail(ctx, (cudaError_t)e, "segregated step") : NSEM_OK;
        } else {
            s = enqueue_steps(ctx, nsteps, prec);
        }
        cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
        if (s != NSEM_OK) {
            if (ce == cudaSuccess) cudaGraphDestroy(g);
            return s;
        }
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaStreamEndCapture");
        cudaGraphExec_t ex;
        ce = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaGraphInstantiate");
        it = ctx->graphs.emplace(key, ex).first;
    }
    NSEM_CUDA(cudaGraphLaunch(it->second, ctx->stream));
    if (form == 1) ctx->mbuf.cur ^= (nsteps & 1);
    if (form == 2) {
        ctx->sbuf.cur ^= (nsteps & 1);
        ctx->seg_pp_valid = true;
    }
    NSEM_CUDA(cudaMemcpyAsync(ctx->h_status, ctx->dev.status, sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, ctx->stream));
    return NSEM_OK;
}

/* ---------------------------------------------------------------- adjoint */

static nsem_status adj_alloc(nsem_ctx* ctx) {
    NsemAdjBuf& A = ctx->abuf;
    if (A.ready) return NSEM_OK;
    nsem_status s;
    for (int v = 0; v < 6; v++) {
        if ((s = dalloc(ctx, &A.adjO[v], ctx->dev.n_slot)) != NSEM_OK) return s;
        if ((s = dalloc(ctx, &A.adjN[v], ctx->dev.n_slot)) != NSEM_OK) return s;
    }
    if (ctx->dev.n_ms > 0) {
        /* non-conforming faces: per mortar slot and per node */
        const size_t nm = (size_t)ctx->dev.n_ms, n = (size_t)ctx->dev.n_int;
        for (int c = 0; c < 19; c++) {
            if ((s = dalloc(ctx, &A.mq[c], nm)) != NSEM_OK) return s;
            if ((s = dalloc(ctx, &A.dmq[c], nm)) != NSEM_OK) return s;
            if ((s = dalloc(ctx, &A.mqb[c], nm)) != NSEM_OK) return s;
            if ((s = dalloc(ctx, &A.qb[c], n)) != NSEM_OK) return s;
        }
        for (int c = 0; c < 15; c++)
            if ((s = dalloc(ctx, &A.dmf[c], nm)) != NSEM_OK) return s;
        for (int c = 0; c < 5; c++)
            if ((s = dalloc(ctx, &A.ddC[c], nm)) != NSEM_OK) return s;
    }
    for (int v = 0; v < 5; v++) {
        const size_t n = (size_t)ctx->dev.n_int;
        if ((s = dalloc(ctx, &A.lam[v], n)) != NSEM_OK) return s;
        if ((s = dalloc(ctx, &A.a3[v], n)) != NSEM_OK) return s;
        if ((s = dalloc(ctx, &A.lu2[v], n)) != NSEM_OK) return s;
        if ((s = dalloc(ctx, &A.lu1[v], n)) != NSEM_OK) return s;
        if ((s = dalloc(ctx, &A.g[v], n)) != NSEM_OK) return s;
        if ((s = dalloc(ctx, &A.fin[v], n)) != NSEM_OK) return s;
    }
    if (ctx->dev.nu != 0.0) {
        const size_t n = (size_t)ctx->dev.n_int, ns = (size_t)ctx->dev.n_slot;
        for (int c = 0; c < 4; c++) {
            if ((s = dalloc(ctx, &A.pU[c], n)) != NSEM_OK) return s;
            if ((s = dalloc(ctx, &A.dpU[c], n)) != NSEM_OK) return s;
            if ((s = dalloc(ctx, &A.fF[c], ns)) != NSEM_OK) return s;
            if ((s = dalloc(ctx, &A.dfF[c], ns)) != NSEM_OK) return s;
        }
        for (int c = 0; c < 12; c++) {
            if ((s = dalloc(ctx, &A.Gv[c], n)) != NSEM_OK) return s;
            if ((s = dalloc(ctx, &A.dGv[c], n)) != NSEM_OK) return s;
            if ((s = dalloc(ctx, &A.Gbs[c], n)) != NSEM_OK) return s;
        }
        for (int c = 0; c < 4; c++) {
            if ((s = dalloc(ctx, &A.dbv[c], ns)) != NSEM_OK) return s;
            if ((s = dalloc(ctx, &A.agO[c], ns)) != NSEM_OK) return s;
            if ((s = dalloc(ctx, &A.agN[c], ns)) != NSEM_OK) return s;
        }
        if ((s = dalloc(ctx, &A.mub, n)) != NSEM_OK) return s;
        if (ctx->dev.n_ms > 0) {
            const size_t nm = (size_t)ctx->dev.n_ms;
            for (int c = 0; c < 4; c++) {
                if ((s = dalloc(ctx, &A.gC[c], nm)) != NSEM_OK) return s;
                if ((s = dalloc(ctx, &A.dgC[c], nm)) != NSEM_OK) return s;
                if ((s = dalloc(ctx, &A.fFb[c], nm)) != NSEM_OK) return s;
                if ((s = dalloc(ctx, &A.gCb[c], nm)) != NSEM_OK) return s;
                if ((s = dalloc(ctx, &A.pbM[c], n)) != NSEM_OK) return s;
            }
            for (int c = 0; c < 12; c++)
                if ((s = dalloc(ctx, &A.mqv[c], nm)) != NSEM_OK) return s;
        }
        A.visc = true;
    }
    int e = nsem_adj_prepare(&ctx->dev);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "adjoint shared memory");
    A.ready = true;
    return NSEM_OK;
}

static nsem_status copy_state(nsem_ctx* ctx, double* const* dst, const double* const* src) {
    const size_t bytes = (size_t)ctx->dev.n_int * sizeof(double);
    for (int v = 0; v < 5; v++)
        NSEM_CUDA(cudaMemcpyAsync(dst[v], src[v], bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    return NSEM_OK;
}

/* pointer set of state slot j of a [count][5][n_int] block */
static void slots(double* block, int64_t j, int64_t n, double* out[5]) {
    for (int v = 0; v < 5; v++) out[v] = block + (j * 5 + v) * n;
}

/* one FP64 step; optionally keeps the two stage states */
static nsem_status fp64_step(nsem_ctx* ctx, double* const* keep1, double* const* keep2) {
    NsemDev* D = &ctx->dev;
    NsemBuf* b = &ctx->buf;
    void* st = (void*)ctx->stream;
    int e;
    if ((e = nsem_fp64_prim(D, b, 1, st))) return cuda_fail(ctx, (cudaError_t)e, "prim");
    for (int stage = 1; stage <= 3; stage++) {
        if ((e = fp64_face(ctx, stage == 1))) return cuda_fail(ctx, (cudaError_t)e, "face");
        if ((e = nsem_fp64_volume(D, &ctx->tab, b, stage, ctx->dt, st)))
            return cuda_fail(ctx, (cudaError_t)e, "volume");
        nsem_status s = NSEM_OK;
        if (stage == 1 && keep1) s = copy_state(ctx, keep1, b->s);
        if (stage == 2 && keep2) s = copy_state(ctx, keep2, b->s);
        if (s != NSEM_OK) return s;
    }
    return NSEM_OK;
}

extern "C" nsem_status nsem_vjp(nsem_ctx* ctx, const double* const w[5], double* const g[5]) {
    if (!ctx) return NSEM_BAD_ARG;
    if (!w || !g) return fail(ctx, NSEM_BAD_ARG, "w or g is NULL");
    for (int v = 0; v < 5; v++)
        if (!w[v] || !g[v]) return fail(ctx, NSEM_BAD_ARG, "w[v] or g[v] is NULL");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    nsem_status s = materialise_conserved(ctx);
    if (s != NSEM_OK) return s;
    if ((s = adj_alloc(ctx)) != NSEM_OK) return s;
    NsemAdjBuf& A = ctx->abuf;
    const size_t bytes = (size_t)ctx->dev.n_int * sizeof(double);
    for (int v = 0; v < 5; v++)
        NSEM_CUDA(cudaMemcpyAsync(A.lam[v], w[v], bytes, cudaMemcpyHostToDevice, ctx->stream));
    int e = nsem_adj_vjp(&ctx->dev, &ctx->tab, ctx->buf.u, A.lam, A.g, &A, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "vjp");
    for (int v = 0; v < 5; v++)
        NSEM_CUDA(cudaMemcpyAsync(g[v], A.g[v], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return check_status(ctx);
}

extern "C" nsem_status nsem_jvp(nsem_ctx* ctx, const double* const dv[5], double* const Ld[5]) {
    if (!ctx) return NSEM_BAD_ARG;
    if (!dv || !Ld) return fail(ctx, NSEM_BAD_ARG, "dv or Ld is NULL");
    for (int v = 0; v < 5; v++)
        if (!dv[v] || !Ld[v]) return fail(ctx, NSEM_BAD_ARG, "dv[v] or Ld[v] is NULL");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    nsem_status s = materialise_conserved(ctx);
    if (s != NSEM_OK) return s;
    if ((s = adj_alloc(ctx)) != NSEM_OK) return s;
    NsemAdjBuf& A = ctx->abuf;
    const size_t bytes = (size_t)ctx->dev.n_int * sizeof(double);
    for (int v = 0; v < 5; v++)
        NSEM_CUDA(cudaMemcpyAsync(A.lam[v], dv[v], bytes, cudaMemcpyHostToDevice, ctx->stream));
    int e = nsem_adj_jvp(&ctx->dev, &ctx->tab, ctx->buf.u, A.lam, A.g, &A, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "jvp");
    for (int v = 0; v < 5; v++)
        NSEM_CUDA(cudaMemcpyAsync(Ld[v], A.g[v], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return check_status(ctx);
}

extern "C" nsem_status nsem_tlm(nsem_ctx* ctx, int nsteps, const double* const du0[5],
                                double* const du_final[5], double* ms_tlm) {
    if (!ctx) return NSEM_BAD_ARG;
    if (nsteps < 1) return fail(ctx, NSEM_BAD_ARG, "nsteps must be >= 1");
    if (!du0 || !du_final) return fail(ctx, NSEM_BAD_ARG, "du0 or du_final is NULL");
    for (int v = 0; v < 5; v++)
        if (!du0[v] || !du_final[v]) return fail(ctx, NSEM_BAD_ARG, "du array is NULL");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    nsem_status s = ensure_rep(ctx, 0);
    if (s != NSEM_OK) return s;
    if ((s = adj_alloc(ctx)) != NSEM_OK) return s;
    NsemAdjBuf& A = ctx->abuf;
    const int64_t n = ctx->dev.n_int;
    const size_t bytes = (size_t)n * sizeof(double);
    /* stage states of one step: u^n, u1, u2 */
    if (!A.seg || A.seg_slots < 3) {
        if (A.seg) { cudaFree(A.seg); A.seg = nullptr; }
        if (cudaMalloc((void**)&A.seg, (size_t)3 * 5 * n * sizeof(double)) != cudaSuccess)
            return fail(ctx, NSEM_NO_MEMORY, "stage-state allocation failed");
        A.seg_slots = 3;
    }
    for (int v = 0; v < 5; v++)
        NSEM_CUDA(cudaMemcpyAsync(A.lam[v], du0[v], bytes, cudaMemcpyHostToDevice, ctx->stream));
    const double dt = ctx->dt;
    void* st = (void*)ctx->stream;
    cudaEvent_t e0, e1;
    NSEM_CUDA(cudaEventCreate(&e0));
    NSEM_CUDA(cudaEventCreate(&e1));
    NSEM_CUDA(cudaEventRecord(e0, ctx->stream));
    int e = 0;
    double *u0[5], *u1[5], *u2[5];
    slots(A.seg, 0, n, u0);
    slots(A.seg, 1, n, u1);
    slots(A.seg, 2, n, u2);
    for (int step = 0; step < nsteps && s == NSEM_OK && !e; step++) {
        if ((s = copy_state(ctx, u0, ctx->buf.u)) != NSEM_OK) break;
        if ((s = fp64_step(ctx, u1, u2)) != NSEM_OK) break;
        /* du1 = du + dt J(u^n) du */
        if ((e = nsem_adj_jvp(&ctx->dev, &ctx->tab, u0, A.lam, A.g, &A, st))) break;
        if ((e = nsem_adj_lin3(A.lu1, A.lam, 1.0, A.g, dt, nullptr, 0, n, st))) break;
        /* du2 = 3/4 du + 1/4 (du1 + dt J(u1) du1) */
        if ((e = nsem_adj_jvp(&ctx->dev, &ctx->tab, u1, A.lu1, A.g, &A, st))) break;
        if ((e = nsem_adj_lin3(A.lu2, A.lam, 0.75, A.lu1, 0.25, A.g, 0.25 * dt, n, st))) break;
        /* du^{n+1} = 1/3 du + 2/3 (du2 + dt J(u2) du2) */
        if ((e = nsem_adj_jvp(&ctx->dev, &ctx->tab, u2, A.lu2, A.g, &A, st))) break;
        if ((e = nsem_adj_lin3(A.lam, A.lam, 1.0 / 3.0, A.lu2, 2.0 / 3.0, A.g, 2.0 / 3.0 * dt, n, st))) break;
    }
    if (e) s = cuda_fail(ctx, (cudaError_t)e, "tangent-linear sweep");
    if (s != NSEM_OK) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return s;
    }
    NSEM_CUDA(cudaEventRecord(e1, ctx->stream));
    for (int v = 0; v < 5; v++)
        NSEM_CUDA(cudaMemcpyAsync(du_final[v], A.lam[v], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    ctx->rep = 0;
    s = check_status(ctx);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != NSEM_OK) return s;
    if (ms_tlm) *ms_tlm = ms;
    return NSEM_OK;
}

extern "C" nsem_status nsem_forward_checkpointed(nsem_ctx* ctx, int nsteps, int ckpt_every,
                                                 double* ms_fwd) {
    if (!ctx) return NSEM_BAD_ARG;
    if (nsteps < 1 || ckpt_every < 1) return fail(ctx, NSEM_BAD_ARG, "nsteps and ckpt_every must be >= 1");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    nsem_status s = ensure_rep(ctx, 0);
    if (s != NSEM_OK) return s;
    if ((s = adj_alloc(ctx)) != NSEM_OK) return s;
    NsemAdjBuf& A = ctx->abuf;
    const int64_t n = ctx->dev.n_int;
    const int n_ckpt = (nsteps + ckpt_every - 1) / ckpt_every;
    if (A.ckpt) { cudaFree(A.ckpt); A.ckpt = nullptr; }
    if (A.seg) { cudaFree(A.seg); A.seg = nullptr; }
    cudaError_t ce = cudaMalloc((void**)&A.ckpt, (size_t)n_ckpt * 5 * n * sizeof(double));
    if (ce != cudaSuccess) return fail(ctx, NSEM_NO_MEMORY, "checkpoint allocation failed");
    ce = cudaMalloc((void**)&A.seg, (size_t)ckpt_every * 3 * 5 * n * sizeof(double));
    if (ce != cudaSuccess) return fail(ctx, NSEM_NO_MEMORY, "segment allocation failed");
    A.seg_slots = 3 * (int64_t)ckpt_every;
    cudaEvent_t e0, e1;
    NSEM_CUDA(cudaEventCreate(&e0));
    NSEM_CUDA(cudaEventCreate(&e1));
    NSEM_CUDA(cudaEventRecord(e0, ctx->stream));
    for (int st = 0; st < nsteps; st++) {
        if (st % ckpt_every == 0) {
            double* c[5];
            slots(A.ckpt, st / ckpt_every, n, c);
            if ((s = copy_state(ctx, c, ctx->buf.u)) != NSEM_OK) return s;
        }
        if ((s = fp64_step(ctx, nullptr, nullptr)) != NSEM_OK) return s;
    }
    NSEM_CUDA(cudaEventRecord(e1, ctx->stream));
    if ((s = copy_state(ctx, A.fin, ctx->buf.u)) != NSEM_OK) return s;
    NSEM_CUDA(cudaMemcpyAsync(ctx->h_status, ctx->dev.status, sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, ctx->stream));
    s = check_status(ctx);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != NSEM_OK) return s;
    if (ms_fwd) *ms_fwd = ms;
    A.nsteps = nsteps;
    A.every = ckpt_every;
    A.n_ckpt = n_ckpt;
    ctx->adj_form = 0;
    return NSEM_OK;
}

/* the precision form's checkpointed forward run */
static nsem_status mixed_forward_checkpointed(nsem_ctx* ctx, int nsteps, int ckpt_every,
                                              double* ms_fwd) {
    if (!ctx->mixed_ready) return fail(ctx, NSEM_UNSUPPORTED, ctx->err);
    nsem_status s = ensure_rep(ctx, 1);
    if (s != NSEM_OK) return s;
    ctx->adj_form = -1;
    cudaEvent_t e0, e1;
    NSEM_CUDA(cudaEventCreate(&e0));
    NSEM_CUDA(cudaEventCreate(&e1));
    NSEM_CUDA(cudaEventRecord(e0, ctx->stream));
    int e = nsem_mixed_fwd_ckpt(&ctx->dev, &ctx->mbuf, nsteps, ckpt_every, ctx->dt, ctx->stream);
    if (e) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return e == (int)cudaErrorMemoryAllocation
                   ? fail(ctx, NSEM_NO_MEMORY, "checkpoint allocation failed")
                   : cuda_fail(ctx, (cudaError_t)e, "checkpointed forward");
    }
    NSEM_CUDA(cudaEventRecord(e1, ctx->stream));
    NSEM_CUDA(cudaMemcpyAsync(ctx->h_status, ctx->dev.status, sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, ctx->stream));
    s = check_status(ctx);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != NSEM_OK) return s;
    if (ms_fwd) *ms_fwd = ms;
    ctx->adj_form = 1;
    return NSEM_OK;
}

extern "C" nsem_status nsem_forward_checkpointed_prec(nsem_ctx* ctx, int nsteps, int ckpt_every,
                                                      nsem_precision prec, double* ms_fwd) {
    if (!ctx) return NSEM_BAD_ARG;
    if (prec == NSEM_FP64) return nsem_forward_checkpointed(ctx, nsteps, ckpt_every, ms_fwd);
    if (prec != NSEM_MIXED) return fail(ctx, NSEM_BAD_ARG, "unknown precision");
    if (nsteps < 1 || ckpt_every < 1) return fail(ctx, NSEM_BAD_ARG, "nsteps and ckpt_every must be >= 1");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    return mixed_forward_checkpointed(ctx, nsteps, ckpt_every, ms_fwd);
}

extern "C" nsem_status nsem_vjp_prec(nsem_ctx* ctx, nsem_precision prec, const double* const w[5],
                                     double* const g[5]) {
    if (!ctx) return NSEM_BAD_ARG;
    if (prec == NSEM_FP64) return nsem_vjp(ctx, w, g);
    if (prec != NSEM_MIXED) return fail(ctx, NSEM_BAD_ARG, "unknown precision");
    if (!w || !g) return fail(ctx, NSEM_BAD_ARG, "w or g is NULL");
    for (int v = 0; v < 5; v++)
        if (!w[v] || !g[v]) return fail(ctx, NSEM_BAD_ARG, "w[v] or g[v] is NULL");
    if (!ctx->mixed_ready) return fail(ctx, NSEM_UNSUPPORTED, ctx->err);
    NSEM_CUDA(cudaSetDevice(ctx->device));
    nsem_status s = ensure_rep(ctx, 1);
    if (s != NSEM_OK) return s;
    int e = nsem_mixed_adj_alloc(&ctx->mbuf);
    if (e) return fail(ctx, NSEM_NO_MEMORY, "adjoint allocation failed");
    const size_t bytes = (size_t)ctx->dev.n_int * sizeof(double);
    NsemBuf* b = &ctx->buf;
    for (int v = 0; v < 5; v++)
        NSEM_CUDA(cudaMemcpyAsync(b->L[v], w[v], bytes, cudaMemcpyHostToDevice, ctx->stream));
    e = nsem_mixed_vjp(&ctx->dev, &ctx->mbuf, b->L, b->L, ctx->mbuf.abar[0], ctx->mbuf.abar[1],
                       ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "precision-form vjp");
    for (int v = 0; v < 5; v++)
        NSEM_CUDA(cudaMemcpyAsync(g[v], b->L[v], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return check_status(ctx);
}

/* the precision form's reverse sweep of the last checkpointed run */
static nsem_status mixed_adjoint(nsem_ctx* ctx, const double* const lam_final[5],
                                 double* const lam0[5], double* ms_adj) {
    NsemMixedBuf& M = ctx->mbuf;
    NsemBuf* b = &ctx->buf;
    const size_t bytes = (size_t)ctx->dev.n_int * sizeof(double);
    for (int v = 0; v < 5; v++) {
        if (!lam_final[v] || !lam0[v]) return fail(ctx, NSEM_BAD_ARG, "lam array is NULL");
        NSEM_CUDA(cudaMemcpyAsync(b->L[v], lam_final[v], bytes, cudaMemcpyHostToDevice, ctx->stream));
    }
    /* the state is read back through ensure_rep after the sweep: the sweep
     * needs the precision form's buffers, not the conserved copy */
    nsem_status s = ensure_rep(ctx, 1);
    if (s != NSEM_OK) return s;
    int e = nsem_mixed_layout(&M, 0, b->L, M.lam, nullptr, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "adjoint layout");
    cudaEvent_t e0, e1;
    NSEM_CUDA(cudaEventCreate(&e0));
    NSEM_CUDA(cudaEventCreate(&e1));
    NSEM_CUDA(cudaEventRecord(e0, ctx->stream));
    e = nsem_mixed_adjoint_run(&ctx->dev, &M, ctx->dt, ctx->stream);
    if (e) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return cuda_fail(ctx, (cudaError_t)e, "precision-form adjoint sweep");
    }
    NSEM_CUDA(cudaEventRecord(e1, ctx->stream));
    e = nsem_mixed_layout(&M, 1, nullptr, M.lam, b->L, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "adjoint layout");
    for (int v = 0; v < 5; v++)
        NSEM_CUDA(cudaMemcpyAsync(lam0[v], b->L[v], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    s = check_status(ctx);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != NSEM_OK) return s;
    if (ms_adj) *ms_adj = ms;
    return NSEM_OK;
}

extern "C" nsem_status nsem_adjoint(nsem_ctx* ctx, const double* const lam_final[5],
                                    double* const lam0[5], double* ms_adj) {
    if (!ctx) return NSEM_BAD_ARG;
    if (!lam_final || !lam0) return fail(ctx, NSEM_BAD_ARG, "lam_final or lam0 is NULL");
    if (ctx->adj_form == 1) {
        NSEM_CUDA(cudaSetDevice(ctx->device));
        return mixed_adjoint(ctx, lam_final, lam0, ms_adj);
    }
    NsemAdjBuf& A = ctx->abuf;
    if (!A.ready || !A.ckpt || A.nsteps < 1)
        return fail(ctx, NSEM_BAD_ARG, "no checkpointed forward run to differentiate");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    const int64_t n = ctx->dev.n_int;
    const size_t bytes = (size_t)n * sizeof(double);
    for (int v = 0; v < 5; v++) {
        if (!lam_final[v] || !lam0[v]) return fail(ctx, NSEM_BAD_ARG, "lam array is NULL");
        NSEM_CUDA(cudaMemcpyAsync(A.lam[v], lam_final[v], bytes, cudaMemcpyHostToDevice, ctx->stream));
    }
    const double dt = ctx->dt;
    void* st = (void*)ctx->stream;
    cudaEvent_t e0, e1;
    NSEM_CUDA(cudaEventCreate(&e0));
    NSEM_CUDA(cudaEventCreate(&e1));
    NSEM_CUDA(cudaEventRecord(e0, ctx->stream));
    nsem_status s = NSEM_OK;
    int e = 0;
    for (int sg = A.n_ckpt - 1; sg >= 0 && s == NSEM_OK; sg--) {
        const int start = sg * A.every;
        const int cnt = (A.nsteps - start < A.every) ? A.nsteps - start : A.every;
        double* c[5];
        slots(A.ckpt, sg, n, c);
        if ((s = copy_state(ctx, ctx->buf.u, c)) != NSEM_OK) break;
        for (int j = 0; j < cnt && s == NSEM_OK; j++) {
            double *u0[5], *u1[5], *u2[5];
            slots(A.seg, 3 * j, n, u0);
            slots(A.seg, 3 * j + 1, n, u1);
            slots(A.seg, 3 * j + 2, n, u2);
            if ((s = copy_state(ctx, u0, ctx->buf.u)) != NSEM_OK) break;
            s = fp64_step(ctx, u1, u2);
        }
        if (s != NSEM_OK) break;
        for (int j = cnt - 1; j >= 0; j--) {
            double *u0[5], *u1[5], *u2[5];
            slots(A.seg, 3 * j, n, u0);
            slots(A.seg, 3 * j + 1, n, u1);
            slots(A.seg, 3 * j + 2, n, u2);
            /* u3 = u/3 + 2/3 (u2 + dt L(u2)) */
            if ((s = copy_state(ctx, A.a3, A.lam)) != NSEM_OK) break;
            if ((e = nsem_adj_vjp(&ctx->dev, &ctx->tab, u2, A.a3, A.g, &A, st))) break;
            if ((e = nsem_adj_lin3(A.lu2, A.a3, 2.0 / 3.0, A.g, 2.0 / 3.0 * dt, nullptr, 0, n, st))) break;
            /* u2 = 3/4 u + 1/4 (u1 + dt L(u1)) */
            if ((e = nsem_adj_vjp(&ctx->dev, &ctx->tab, u1, A.lu2, A.g, &A, st))) break;
            if ((e = nsem_adj_lin3(A.lu1, A.lu2, 0.25, A.g, 0.25 * dt, nullptr, 0, n, st))) break;
            /* u1 = u + dt L(u) */
            if ((e = nsem_adj_vjp(&ctx->dev, &ctx->tab, u0, A.lu1, A.g, &A, st))) break;
            if ((e = nsem_adj_lin3(A.lam, A.a3, 1.0 / 3.0, A.lu2, 0.75, A.lu1, 1.0, n, st))) break;
            if ((e = nsem_adj_lin3(A.lam, A.lam, 1.0, A.g, dt, nullptr, 0, n, st))) break;
        }
    }
    if (e) s = cuda_fail(ctx, (cudaError_t)e, "adjoint sweep");
    if (s != NSEM_OK) return s;
    NSEM_CUDA(cudaEventRecord(e1, ctx->stream));
    for (int v = 0; v < 5; v++)
        NSEM_CUDA(cudaMemcpyAsync(lam0[v], A.lam[v], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    if ((s = copy_state(ctx, ctx->buf.u, A.fin)) != NSEM_OK) return s;
    ctx->rep = 0;
    s = check_status(ctx);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != NSEM_OK) return s;
    if (ms_adj) *ms_adj = ms;
    return NSEM_OK;
}

/* --------------------------------------------------- scalar convection */

extern "C" nsem_status nsem_convection_set(nsem_ctx* ctx, const double* U, const double* T) {
    if (!ctx) return NSEM_BAD_ARG;
    if (!U || !T) return fail(ctx, NSEM_BAD_ARG, "U or T is NULL");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    NsemConvBuf& C = ctx->cbuf;
    const size_t n = (size_t)ctx->dev.n_int, ns = (size_t)ctx->dev.n_slot;
    nsem_status s;
    /* the staging buffer below may still hold the Euler state as passed */
    if (ctx->rep == 3 && (s = ensure_rep(ctx, 0)) != NSEM_OK) return s;
    if (!C.ready) {
        double** arrays[] = {&C.T[0], &C.T[1], &C.U[0], &C.U[1], &C.U[2]};
        for (double** a : arrays)
            if ((s = dalloc(ctx, a, n)) != NSEM_OK) return s;
        if ((s = dalloc(ctx, &C.lam, ns)) != NSEM_OK) return s;
        if ((s = dalloc(ctx, &C.d, ns)) != NSEM_OK) return s;
        if ((s = seg_alloc(ctx)) != NSEM_OK) return s;   /* shared-memory attributes */
        /* non-conforming faces: the segregated scheme's mortar buffers */
        for (int c = 0; c < 4; c++) C.mq[c] = ctx->sbuf.mq[c];
        for (int c = 0; c < 3; c++) C.mf[c] = ctx->sbuf.mf[c];
        C.dC = ctx->sbuf.dC[0];
        C.ready = true;
    }
    C.cur = 0;
    C.analytic = false;
    C.order = 1;
    C.hist = 0;
    NSEM_CUDA(cudaMemcpyAsync(C.T[0], T, n * 8, cudaMemcpyHostToDevice, ctx->stream));
    NSEM_CUDA(cudaMemcpyAsync(ctx->scratch_aos, U, 3 * n * 8, cudaMemcpyHostToDevice, ctx->stream));
    int e = nsem_aos_to_soa(ctx->scratch_aos, C.U[0], C.U[1], C.U[2], (int64_t)n, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "aos_to_soa");
    if ((e = nsem_conv_lambda(&ctx->dev, &C, ctx->stream)))
        return cuda_fail(ctx, (cudaError_t)e, "convection speed");
    NSEM_CUDA(cudaStreamSynchronize(ctx->stream));
    return NSEM_OK;
}

extern "C" nsem_status nsem_convection_step(nsem_ctx* ctx, int nsteps) {
    
    if (!ctx) return NSEM_BAD_ARG;
    if (nsteps < 0) return fail(ctx, NSEM_BAD_ARG, "nsteps < 0");
    NsemConvBuf& C = ctx->cbuf;
    if (!C.ready) return fail(ctx, NSEM_BAD_ARG, "nsem_convection_set was not called");
    if (nsteps == 0) return NSEM_OK;
    if (C.analytic || C.order != 1) return nsem_convection_step_scaled(ctx, nsteps, nullptr);
    NSEM_CUDA(cudaSetDevice(ctx->device));
    auto key = std::make_pair(3 * 2 + C.cur, nsteps);
    auto it = ctx->graphs.find(key);
    if (it == ctx->graphs.end()) {
        cudaGraph_t g;
        NSEM_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        const int e = nsem_conv_steps(&ctx->dev, &ctx->tab, &C, nsteps, ctx->dt, ctx->stream);
        cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
        if (e) {
            if (ce == cudaSuccess) cudaGraphDestroy(g);
            return cuda_fail(ctx, (cudaError_t)e, "convection step");
        }
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaStreamEndCapture");
        cudaGraphExec_t ex;
        ce = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaGraphInstantiate");
        it = ctx->graphs.emplace(key, ex).first;
    }
    NSEM_CUDA(cudaGraphLaunch(it->second, ctx->stream));
    C.cur ^= (nsteps & 1);
    NSEM_CUDA(cudaMemcpyAsync(ctx->h_status, ctx->dev.status, sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, ctx->stream));
    return NSEM_OK;
}

extern "C" nsem_status nsem_convection_wind(nsem_ctx* ctx, const double* U_all, int time_scheme) {
    if (!ctx) return NSEM_BAD_ARG;
    if (time_scheme != 1 && time_scheme != 2)
        return fail(ctx, NSEM_UNSUPPORTED, "convection time schemes: 1 (BDF1/AB1) or 2 (AB2)");
    NsemConvBuf& C = ctx->cbuf;
    if (!C.ready) return fail(ctx, NSEM_BAD_ARG, "nsem_convection_set was not called");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    const int64_t n = ctx->dev.n_int, ns = ctx->dev.n_slot;
    nsem_status s;
    if (time_scheme == 2 && !C.R[0]) {
        if ((s = dalloc(ctx, &C.R[0], (size_t)n)) != NSEM_OK) return s;
        if ((s = dalloc(ctx, &C.R[1], (size_t)n)) != NSEM_OK) return s;
    }
    C.order = time_scheme;
    C.hist = 0;
    if (!U_all) return NSEM_OK;
    if (!C.A[0])
        for (int c = 0; c < 3; c++) {
            if ((s = dalloc(ctx, &C.A[c], (size_t)n)) != NSEM_OK) return s;
            if ((s = dalloc(ctx, &C.Ag[c], (size_t)ns)) != NSEM_OK) return s;
            if ((s = dalloc(ctx, &C.Ug[c], (size_t)ns)) != NSEM_OK) return s;
        }
    /* spatial part on interior nodes (SoA) and at each used slot's ghost */
    std::vector<double> a((size_t)n), g((size_t)ns, 0.0);
    for (int c = 0; c < 3; c++) {
        for (int64_t i = 0; i < n; i++) a[i] = U_all[3 * i + c];
        for (int64_t k = 0; k < ns; k++)
            g[k] = ctx->slot_ghost[k] >= 0 ? U_all[3 * ctx->slot_ghost[k] + c] : 0.0;
        NSEM_CUDA(cudaMemcpy(C.A[c], a.data(), (size_t)n * 8, cudaMemcpyHostToDevice));
        NSEM_CUDA(cudaMemcpy(C.Ag[c], g.data(), (size_t)ns * 8, cudaMemcpyHostToDevice));
    }
    C.analytic = true;
    return NSEM_OK;
}

extern "C" nsem_status nsem_convection_step_scaled(nsem_ctx* ctx, int nsteps, const double* scale) {
    if (!ctx) return NSEM_BAD_ARG;
    if (nsteps < 0) return fail(ctx, NSEM_BAD_ARG, "nsteps < 0");
    NsemConvBuf& C = ctx->cbuf;
    if (!C.ready) return fail(ctx, NSEM_BAD_ARG, "nsem_convection_set was not called");
    if (nsteps == 0) return NSEM_OK;
    NSEM_CUDA(cudaSetDevice(ctx->device));
    const int e = nsem_conv_steps_wind(&ctx->dev, &ctx->tab, &C, nsteps, ctx->dt, scale, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "convection step");
    NSEM_CUDA(cudaMemcpyAsync(ctx->h_status, ctx->dev.status, sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, ctx->stream));
    return NSEM_OK;
}

extern "C" nsem_status nsem_convection_get(nsem_ctx* ctx, double* T) {
    if (!ctx) return NSEM_BAD_ARG;
    if (!T) return fail(ctx, NSEM_BAD_ARG, "T is NULL");
    NsemConvBuf& C = ctx->cbuf;
    if (!C.ready) return fail(ctx, NSEM_BAD_ARG, "nsem_convection_set was not called");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    NSEM_CUDA(cudaMemcpyAsync(T, C.T[C.cur], (size_t)ctx->dev.n_int * 8, cudaMemcpyDeviceToHost,
                              ctx->stream));
    return check_status(ctx);
}

nsem_status nsem_profile(nsem_ctx* ctx, int nsteps, nsem_precision prec, double ms[8],
                         int launches[8], char names[8 * 32]) {
    if (ctx && ctx->dev.n_ms > 0 && prec != NSEM_MIXED) return require_conforming(ctx);
    if (!ctx) return NSEM_BAD_ARG;
    if (!ms || !launches || !names) return fail(ctx, NSEM_BAD_ARG, "output pointer is NULL");
    if (nsteps < 1) return fail(ctx, NSEM_BAD_ARG, "nsteps < 1");
    NSEM_CUDA(cudaSetDevice(ctx->device));
    if (prec == NSEM_MIXED && !ctx->mixed_ready) return fail(ctx, NSEM_UNSUPPORTED, ctx->err);
    {
        nsem_status rs = ensure_rep(ctx, prec == NSEM_MIXED ? 1 : 0);
        if (rs != NSEM_OK) return rs;
    }
    for (int i = 0; i < 8; i++) { ms[i] = 0; launches[i] = 0; }
    std::memset(names, 0, 8 * 32);
    NsemDev* D = &ctx->dev;
    NsemBuf* b = &ctx->buf;
    void* st = (void*)ctx->stream;
    /* one event pair per launch, timed after the whole run */
    struct Rec { int cls; cudaEvent_t a, z; };
    std::vector<Rec> recs;
    auto timed = [&](int cls, auto&& launch) -> nsem_status {
        Rec r;
        r.cls = cls;
        NSEM_CUDA(cudaEventCreate(&r.a));
        NSEM_CUDA(cudaEventCreate(&r.z));
        NSEM_CUDA(cudaEventRecord(r.a, ctx->stream));
        int e = launch();
        if (e) return cuda_fail(ctx, (cudaError_t)e, "profiled launch");
        NSEM_CUDA(cudaEventRecord(r.z, ctx->stream));
        recs.push_back(r);
        return NSEM_OK;
    };
    nsem_status s = NSEM_OK;
    if (prec == NSEM_FP64) {
        std::strncpy(names + 0 * 32, "fp64_prim", 31);
        std::strncpy(names + 1 * 32, "fp64_face", 31);
        std::strncpy(names + 2 * 32, "fp64_volume", 31);
        s = timed(0, [&] { return nsem_fp64_prim(D, b, 1, st); });
        for (int n = 0; n < nsteps && s == NSEM_OK; n++)
            for (int stage = 1; stage <= 3 && s == NSEM_OK; stage++) {
                s = timed(1, [&] { return fp64_face(ctx, stage == 1); });
                if (s == NSEM_OK)
                    s = timed(2, [&] { return nsem_fp64_volume(D, &ctx->tab, b, stage, ctx->dt, st); });
            }
    } else if (prec == NSEM_MIXED) {
        if (!ctx->mixed_ready) return fail(ctx, NSEM_UNSUPPORTED, ctx->err);
        const char* const* nm = nsem_mixed_kernel_names();
        for (int i = 0; i < 8 && nm[i]; i++) std::strncpy(names + i * 32, nm[i], 31);
        for (int n = 0; n < nsteps && s == NSEM_OK; n++) {
            for (int k = 0; k < nsem_mixed_launches_per_step() && s == NSEM_OK; k++) {
                int cls = nsem_mixed_launch_class(k);
                s = timed(cls, [&] {
                    return nsem_mixed_launch(D, &ctx->mbuf, b, &ctx->tab, k, n == 0, ctx->dt, st);
                });
            }
        }
    } else {
        return fail(ctx, NSEM_BAD_ARG, "unknown precision");
    }
    cudaError_t ce = cudaStreamSynchronize(ctx->stream);
    for (Rec& r : recs) {
        float t = 0;
        if (ce == cudaSuccess && s == NSEM_OK) {
            cudaEventElapsedTime(&t, r.a, r.z);
            ms[r.cls] += t;
            launches[r.cls] += 1;
        }
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.z);
    }
    if (s != NSEM_OK) return s;
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "profile sync");
    NSEM_CUDA(cudaMemcpyAsync(ctx->h_status, ctx->dev.status, sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, ctx->stream));
    return check_status(ctx);
}

nsem_status nsem_sync(nsem_ctx* ctx) {
    if (!ctx) return NSEM_BAD_ARG;
    NSEM_CUDA(cudaSetDevice(ctx->device));
    return check_status(ctx);
}

nsem_status nsem_diagnostics(nsem_ctx* ctx, double* mass, double* energy, double* volume) {
    if (!ctx) return NSEM_BAD_ARG;
    NSEM_CUDA(cudaSetDevice(ctx->device));
    nsem_status rs = materialise_conserved(ctx);
    if (rs != NSEM_OK) return rs;
    int e = nsem_reduce_diagnostics(&ctx->dev, &ctx->buf, ctx->red, ctx->h_red, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "diagnostics");
    nsem_status s = check_status(ctx);
    if (s != NSEM_OK) return s;
    if (mass) *mass = ctx->h_red[0];
    if (energy) *energy = ctx->h_red[1];
    if (volume) *volume = ctx->h_red[2];
    return NSEM_OK;
}

}  // extern "C"
