/*
 * Precision form (FP32 bulk arithmetic, FP64 state, background subtraction,
 * RK accumulation and conservation sums) and auxiliary kernels.
 */
#ifndef NSEM_MIXED_H
#define NSEM_MIXED_H

#include <string>
#include <vector>

#include "nsem.h"
#include "nsem_internal.h"

#define NSEM_RED_PARTIALS 1024

struct NsemMixedBuf {
    bool ready = false;
    int64_t n_elem = 0;
    int npd[3] = {0, 0, 0};
    int n_layers = 0;
    int cur = 0;                  /* which of U[0], U[1] holds u'^n      */
    double* U[2][5] = {};         /* FP64 perturbation state, ping-pong   */
    float* U32[2][5] = {};        /* FP32 shadow of U (read by the stages) */
    float* D[2][5] = {};          /* FP32 stage increments                */
    int32_t* nbr = nullptr;       /* [6][n_elem] neighbour element, -1 wall */
    float* J = nullptr;           /* [3][n_elem] metric diagonal 2/h       */
    int32_t* layer = nullptr;     /* [n_elem] background layer             */
    float* bg = nullptr;          /* [layers][3][NP] rho_ref, rho_ref T0, p_ref */
    float* Qg = nullptr;          /* device copy of the line-sum weights   */
    float* Dg = nullptr;          /* derivative tables D_d[a][m] = l_m'(x_a) */
    float* Gv[12] = {};           /* viscous runs: grad U, grad theta of the stage state (FP32) */
    bool visc = false;            /* artificial viscosity (diffusion YES) */
    float nu = 0, nu_pr = 0;      /* nu and nu / Pr */
    void* tabs = nullptr;         /* host copy of the kernel tables        */
    size_t tabs_size = 0;
};

/* u' <-> u conversion of the current state (to_pert: buf.u -> U[cur]) */
int nsem_mixed_convert(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, int to_pert,
                       void* stream);

nsem_status nsem_mixed_setup(const NsemDev& dev, const nsem_mesh_desc* m, NsemMixedBuf* mb,
                             std::vector<void*>* allocs, std::string& err);
int nsem_mixed_steps(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, const NsemTables* t,
                     int nsteps, double dt, void* stream);
int nsem_mixed_tendency(const NsemDev* dev, NsemMixedBuf* mb, NsemBuf* b, const NsemTables* t,
                        void* stream);

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
