/*
 * Auxiliary kernels: AoS <-> SoA conversion of the momentum field at the
 * host boundary, and the conservation sums of euler.cpp:165-176 / 263-274
 * (mass, energy, volume) with compensated (two-sum) accumulation.
 * Compiled with --fmad=false like the plain form.
 */
#include <cuda_runtime.h>

#include "nsem_ddpow.h"
#include "nsem_mixed.h"

namespace {

__global__ void k_aos_to_soa(const double* __restrict__ aos, double* __restrict__ x,
                             double* __restrict__ y, double* __restrict__ z, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = aos[3 * i + 0];
        y[i] = aos[3 * i + 1];
        z[i] = aos[3 * i + 2];
    }
}

__global__ void k_soa_to_aos(const double* __restrict__ x, const double* __restrict__ y,
                             const double* __restrict__ z, double* __restrict__ aos, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        aos[3 * i + 0] = x[i];
        aos[3 * i + 1] = y[i];
        aos[3 * i + 2] = z[i];
    }
}

struct CSum {
    double s, c;
};

__device__ __forceinline__ CSum cadd(CSum a, double x) {
    /* Neumaier step */
    const double t = a.s + x;
    if (fabs(a.s) >= fabs(x)) a.c += (a.s - t) + x;
    else a.c += (x - t) + a.s;
    a.s = t;
    return a;
}

__device__ __forceinline__ CSum cmerge(CSum a, CSum b) {
    const double t = a.s + b.s;
    const double bb = t - a.s;
    const double err = (a.s - (t - bb)) + (b.s - bb);
    CSum r;
    r.s = t;
    r.c = (a.c + b.c) + err;
    return r;
}

constexpr int RB = 256;

__device__ void block_reduce3(CSum v[3], CSum* sh) {
    const int t = threadIdx.x;
    for (int q = 0; q < 3; q++) sh[q * RB + t] = v[q];
    __syncthreads();
    for (int w = RB / 2; w > 0; w >>= 1) {
        if (t < w)
            for (int q = 0; q < 3; q++) sh[q * RB + t] = cmerge(sh[q * RB + t], sh[q * RB + t + w]);
        __syncthreads();
    }
    for (int q = 0; q < 3; q++) v[q] = sh[q * RB];
}

struct StatePtrs {
    const double* p[5];
};

__global__ void __launch_bounds__(RB) k_diag_partial(const NsemDev m, StatePtrs sp,
                                                     double* partials) {
    __shared__ CSum sh[3 * RB];
    const double* const* S = sp.p;
    CSum acc[3] = {{0, 0}, {0, 0}, {0, 0}};
    const double kappa = m.R / m.cp;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m.n_int;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double r = S[0][i];
        const double U[3] = {S[1][i] / r, S[2][i] / r, S[3][i] / r};
        const double T = S[4][i] / r;
        const double p = m.P0 * nsem_pow(((r * T) * m.R) / m.P0, m.gamma);
        const double pp = p - m.p_ref[i];
        const double cv = m.cv[i];
        const double ke = U[0] * U[0] + (U[1] * U[1] + (U[2] * U[2] + 0.0));
        const double sf = (m.gh[i] + 0.5 * ke) +
                          (nsem_pow((pp + m.p_ref[i]) / m.P0, kappa) * T) * m.cv_heat;
        acc[0] = cadd(acc[0], r * cv);
        acc[1] = cadd(acc[1], (r * cv) * sf);
        acc[2] = cadd(acc[2], cv);
    }
    block_reduce3(acc, sh);
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; q++) {
            partials[(int64_t)q * 2 * NSEM_RED_PARTIALS + blockIdx.x] = acc[q].s;
            partials[(int64_t)(q * 2 + 1) * NSEM_RED_PARTIALS + blockIdx.x] = acc[q].c;
        }
}

__global__ void __launch_bounds__(RB) k_diag_final(const double* partials, int nblk, double* out) {
    __shared__ CSum sh[3 * RB];
    CSum acc[3] = {{0, 0}, {0, 0}, {0, 0}};
    for (int b = threadIdx.x; b < nblk; b += RB)
        for (int q = 0; q < 3; q++) {
            CSum x;
            x.s = partials[(int64_t)q * 2 * NSEM_RED_PARTIALS + b];
            x.c = partials[(int64_t)(q * 2 + 1) * NSEM_RED_PARTIALS + b];
            acc[q] = cmerge(acc[q], x);
        }
    block_reduce3(acc, sh);
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; q++) out[q] = acc[q].s + acc[q].c;
}

int grid_for(int64_t n) {
    int64_t g = (n + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

int nsem_aos_to_soa(const double* aos, double* x, double* y, double* z, int64_t n, void* stream) {
    k_aos_to_soa<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(aos, x, y, z, n);
    return (int)cudaGetLastError();
}

int nsem_soa_to_aos(const double* x, const double* y, const double* z, double* aos, int64_t n,
                    void* stream) {
    k_soa_to_aos<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(x, y, z, aos, n);
    return (int)cudaGetLastError();
}

int nsem_reduce_diagnostics(const NsemDev* dev, const NsemBuf* b, double* partials,
                            double* h_out, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    int64_t nblk = (dev->n_int + RB - 1) / RB;
    if (nblk > NSEM_RED_PARTIALS) nblk = NSEM_RED_PARTIALS;
    StatePtrs sp;
    for (int c = 0; c < 5; c++) sp.p[c] = b->u[c];
    k_diag_partial<<<(unsigned)nblk, RB, 0, st>>>(*dev, sp, partials);
    /* partials holds 6 * NSEM_RED_PARTIALS values, the 3 results follow */
    double* dout = partials + 6 * NSEM_RED_PARTIALS;
    k_diag_final<<<1, RB, 0, st>>>(partials, (int)nblk, dout);
    cudaError_t e = cudaMemcpyAsync(h_out, dout, 3 * sizeof(double), cudaMemcpyDeviceToHost, st);
    return (int)(e != cudaSuccess ? e : cudaGetLastError());
}
