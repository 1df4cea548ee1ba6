/*
 * Precision form (FP32 bulk arithmetic, FP64 state, background subtraction,
 * RK accumulation and conservation sums), its discrete adjoint, and
 * auxiliary kernels.
 */
#ifndef NSEM_MIXED_H
#define NSEM_MIXED_H

#include <string>
#include <vector>

#include "nsem.h"
#include "nsem_internal.h"

#define NSEM_RED_PARTIALS 1024

/* State arrays are element-blocked: [n_elem][5][NP] (see nsem_mixed_dev.cuh). */
struct NsemMixedBuf {
    bool ready = false;
    int64_t n_elem = 0;
    int64_t n_int = 0;
    int npd[3] = {0, 0, 0};
    int n_layers = 0;
    int cur = 0;                  /* which of U[0], U[1] holds u'^n        */
    double* U[2] = {};            /* FP64 perturbation state, ping-pong     */
    float* S[2] = {};             /* FP32 shadow of U (read by the stages)  */
    float* D[2] = {};             /* FP32 stage increments                  */
    int32_t* nbr = nullptr;       /* [6][n_elem] neighbour element, -1 wall */
    float* J = nullptr;           /* [3][n_elem] metric diagonal 2/h        */
    int32_t* layer = nullptr;     /* [n_elem] background layer              */
    float qc[3][8][8] = {};       /* host copy of the line-sum weights      */
    float dc[3][8][8] = {};       /* host copy of the derivative tables D_d[a][m] */
    float* bg = nullptr;          /* [layers][4][NP] rho_ref, Theta_ref, 1/Theta_ref, p_ref */
    float* Qg = nullptr;          /* line-sum weights Q_d[a][m], row stride MAXN+1 */
    float* Dg = nullptr;          /* derivative tables D_d[a][m] = l_m'(x_a), same layout */
    float* G = nullptr;           /* viscous runs: [n_elem][12][NP] gradients of the stage state */
    bool visc = false;            /* artificial viscosity (diffusion YES)   */
    bool tc = false;              /* order-7 line sums on the tensor cores  */
    bool persist = false;         /* persistent stage kernels               */
    bool gen = false;             /* general geometry (inclined, curved)    */
    float* Jg = nullptr;          /* gen: [n_elem][10][NP] Jinv cV, 1/cV    */
    float* Fn = nullptr;          /* gen: [n_elem][3][NFS] outward fN       */
    int pgrid[4] = {0, 0, 0, 0};  /* their grids (resident CTAs), per stage */
    /* non-conforming (2:1) faces (inviscid runs on axis-aligned elements):
     * per mortar slot the fine node, the coarse face and the interpolation
     * indices; the flux vectors, the fine side's F.n and the coarse side's
     * projected F.n; per element face on a mortar the outward face values
     * that the stage kernels lift (nbr = -2 - index) */
    int64_t n_ms = 0;             /* mortar slots                           */
    int32_t* mx_i = nullptr;      /* [MX_FIELDS][n_ms]                      */
    float* mx_f = nullptr;        /* [8][n_ms]: fN (3), unit normal (3), interpolated minus own rho_ref, Theta_ref */
    float* mx_psi = nullptr;      /* [2][6][MAXN^2] psiRef, psiCor (FP32)   */
    float* mx_F = nullptr;        /* [15][n_ms] face flux vectors           */
    float* mx_d = nullptr;        /* [5][n_ms] fine side F.n                */
    float* mx_dC = nullptr;       /* [5][n_ms] coarse side projected F.n    */
    int64_t n_mf = 0;             /* element faces on mortars               */
    int nfmax = 0;                /* nodes per face (largest direction)     */
    int32_t* mf_ent = nullptr;    /* [n_mf][nfmax][4] mortar slot (| 1<<30: coarse value), -1 */
    float* mf_coef = nullptr;     /* [n_mf][nfmax][4] sign / (cV J_d / w_end) */
    float* MF = nullptr;          /* [n_mf][9][nfmax] outward face values (0-4) and,
                                     viscous runs, gradient face terms (5-8) */
    /* viscous runs: the gradients' face values on mortars */
    float* mx_gF = nullptr;       /* [4][n_ms] cds(U), cds(theta - T0) per slot */
    float* mx_gC = nullptr;       /* [4][n_ms] their projection onto the coarse node */
    int32_t* mf_node = nullptr;   /* [n_mf][nfmax] the element face's node  */
    float* mf_gs = nullptr;       /* [n_mf][nfmax][4] |fN| / (cV J_d / w_end) */
    float* mf_acoef = nullptr;    /* [n_mf][nfmax][4] the entry's weight in the adjoint: minus
                                     the lift coefficient of the face node times mf_coef */
    int32_t* mf_face = nullptr;   /* [n_mf] the element face (2 dir + side) */
    float nu = 0, nu_pr = 0;      /* nu and nu / Pr                         */
    float lift[3] = {0, 0, 0};    /* 1 / w_end per direction                */
    /* discrete adjoint (allocated on first use) */
    double* ckpt = nullptr;       /* [n_ckpt][5 n_int] FP64 checkpoints of u'      */
    float* seg = nullptr;         /* [seg_steps][3][5 n_int] per step: shadow, d1, d2 */
    int64_t seg_steps = 0, ckpt_slots = 0;
    double* lam = nullptr;        /* [5 n_int] FP64 adjoint state             */
    double* fin = nullptr;        /* [5 n_int] FP64 final state of the forward */
    float* abar[3] = {};          /* FP32 stage adjoints: sbar, d2bar, d1bar  */
    float* GB = nullptr;          /* viscous adjoint: gradient adjoints [e][12][NP] */
    float* XB = nullptr;          /* viscous adjoint: first-pass state adjoint [e][5][NP] */
    /* adjoint on mortar faces: the fine side's and the projected coarse
     * side's F.n adjoints, the coarse side's interpolated-quantity adjoints
     * and the fine node's state adjoint, per slot */
    float* mxa_db = nullptr;      /* [5][n_ms]  */
    float* mxa_dCb = nullptr;     /* [5][n_ms]  */
    float* mxa_qb = nullptr;      /* [19][n_ms] */
    float* mxa_xf = nullptr;      /* [5][n_ms]  */
    /* viscous runs: the fine node's gradient adjoints per slot, the
     * gradients' face values' adjoints (fine and coarse entries), their
     * half-weighted totals per slot, and per mortar face node the adjoint of
     * its own V through the face terms */
    float* mxa_gf = nullptr;      /* [12][n_ms] */
    float* mxa_gFb = nullptr;     /* [4][n_ms]  */
    float* mxa_gCb = nullptr;     /* [4][n_ms]  */
    float* mxa_vh = nullptr;      /* [4][n_ms]  */
    float* mxa_vown = nullptr;    /* [4][n_mf nfmax] */
    int nsteps = 0, every = 0, n_ckpt = 0;
    int fin_cur = 0;
};

/* u' <-> u conversion of the current state (to_pert: buf.u -> U[cur]) */
int nsem_mixed_convert(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, int to_pert,
                       void* stream);

/* the host boundary's layout (rho, rho U AoS, rho theta in node order) <->
 * the current perturbation state U[cur] (to_pert: host layout -> U, S) */
int nsem_mixed_host_layout(const NsemDev* dev, NsemMixedBuf* mb, int to_pert, double* rho,
                           double* mom, double* rt, void* stream);

nsem_status nsem_mixed_setup(const NsemDev& dev, const nsem_mesh_desc* m, NsemMixedBuf* mb,
                             std::vector<void*>* allocs, std::string& err);
int nsem_mixed_steps(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, const NsemTables* t,
                     int nsteps, double dt, void* stream);
int nsem_mixed_tendency(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, const NsemTables* t,
                        void* stream);

bool nsem_mixed_supported(int nx, int ny, int nz);
/* one SSP-RK3 step with explicit buffers (element-blocked): stage base S (the
 * FP32 shadow of u'^n), increments d1 and d2, FP64 u'^n -> Unew with its
 * shadow Snew */
int nsem_mixed_step_bufs(const NsemDev* dev, const NsemMixedBuf* mb, const double* U,
                         const float* S, float* d1, float* d2, double* Unew, float* Snew,
                         double dt, void* stream);
/* viscous runs: the gradients of the stage state S (+ Din) into mb->G */
int nsem_mixed_grad_at(const NsemDev* dev, const NsemMixedBuf* mb, const float* S,
                       const float* Din, void* stream);

/* discrete adjoint of the precision form (nsem_mixed_adj.cu) */
int nsem_mixed_adj_prepare(const NsemMixedBuf* mb);
int nsem_mixed_adj_alloc(NsemMixedBuf* mb);
/* dir 0: node-order SoA soa[5] -> element-blocked blk; dir 1: blk -> soa_out[5] */
int nsem_mixed_layout(const NsemMixedBuf* mb, int dir, const double* const soa[5], double* blk,
                      double* const soa_out[5], void* stream);
int nsem_mixed_vjp(const NsemDev* dev, NsemMixedBuf* mb, const double* const w[5],
                   double* const g[5], float* scratch_in, float* scratch_out, void* stream);
int nsem_mixed_fwd_ckpt(const NsemDev* dev, NsemMixedBuf* mb, int nsteps, int every, double dt,
                        void* stream);
int nsem_mixed_adjoint_run(const NsemDev* dev, NsemMixedBuf* mb, double dt, void* stream);

/* launch-by-launch interface for measurement (nsem_profile) */
const char* const* nsem_mixed_kernel_names();
int nsem_mixed_launches_per_step();
int nsem_mixed_launch_class(int k);
int nsem_mixed_launch(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, const NsemTables* t, int k,
                      int first_step, double dt, void* stream);

/* auxiliary kernels (nsem_aux.cu) */
int nsem_aos_to_soa(const double* aos, double* x, double* y, double* z, int64_t n, void* stream);
int nsem_soa_to_aos(const double* x, const double* y, const double* z, double* aos, int64_t n,
                    void* stream);
int nsem_reduce_diagnostics(const NsemDev* dev, const NsemBuf* b, double* partials,
                            double* h_out, void* stream);

#endif
