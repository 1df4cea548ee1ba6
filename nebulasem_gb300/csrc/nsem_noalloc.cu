/*
 * Allocation-free conservation sums.
 *
 * nsem_conservation_sums_noalloc() computes the same mass / energy / volume
 * sums as nsem_diagnostics(), but works entirely on buffers the caller
 * already owns and never allocates device or host memory.  It exists for
 * host codes that manage every byte of device memory themselves -- a solver
 * embedded in a larger application with its own pre-reserved memory pool, or
 * a time loop that must not call cudaMalloc once running, because cudaMalloc
 * can synchronise the whole device and its allocations escape the host
 * code's own memory accounting.  Such callers cannot use a context created
 * by nsem_create() in the middle of a run, so this entry point takes raw
 * device pointers.
 *
 * Its only working memory is the file-scope device array below: partial
 * sums of at most NSEM_NOALLOC_MAX_CHUNKS chunks of NSEM_NOALLOC_CHUNK nodes
 * (6 doubles per chunk, 3 MiB in total), which bounds the node count to
 * NSEM_NOALLOC_MAX_NODES.  Every process that loads the library holds this
 * array on every GPU it uses until the process exits.
 */
#include <cuda_runtime.h>

#include <mutex>

#include "nsem.h"
#include "nsem_ddpow.h"

#define NSEM_NOALLOC_CHUNK 4096                 /* nodes per partial sum        */
#define NSEM_NOALLOC_MAX_CHUNKS 65536           /* partial sums kept            */
static_assert(NSEM_NOALLOC_MAX_NODES == (int64_t)NSEM_NOALLOC_CHUNK * NSEM_NOALLOC_MAX_CHUNKS,
              "NSEM_NOALLOC_MAX_NODES in nsem.h must equal chunk size x chunk count");

/* partial sums: 3 quantities x (sum, compensation) x chunks, then 3 results */
static __device__ __align__(256) double nsem_noalloc_scratch[6 * NSEM_NOALLOC_MAX_CHUNKS + 8];

namespace {

constexpr int NT = 256;                                   /* threads per chunk */
constexpr int PER_THREAD = NSEM_NOALLOC_CHUNK / NT;       /* nodes per thread  */
constexpr int MAX_DEVICES = 64;

/* device address of the scratch array, resolved once per device */
double* g_scratch[MAX_DEVICES] = {nullptr};
std::mutex g_lock;

struct CSum {
    double s, c;
};

__device__ __forceinline__ CSum cadd(CSum a, double x) {
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

__device__ void block_reduce3(CSum v[3], CSum* sh) {
    const int t = threadIdx.x;
    for (int q = 0; q < 3; q++) sh[q * NT + t] = v[q];
    __syncthreads();
    for (int w = NT / 2; w > 0; w >>= 1) {
        if (t < w)
            for (int q = 0; q < 3; q++) sh[q * NT + t] = cmerge(sh[q * NT + t], sh[q * NT + t + w]);
        __syncthreads();
    }
    for (int q = 0; q < 3; q++) v[q] = sh[q * NT];
}

struct Inputs {
    const double* u[5];
    const double* cV;
    const double* gh;
    const double* p_ref;
    int64_t n;
    double P0, R, gamma, kappa, cv_heat;
};

/* one block per chunk of NSEM_NOALLOC_CHUNK nodes */
__global__ void __launch_bounds__(NT) k_chunk_sums(Inputs in, double* scratch, int nchunks) {
    __shared__ CSum sh[3 * NT];
    CSum acc[3] = {{0, 0}, {0, 0}, {0, 0}};
    const int64_t base = (int64_t)blockIdx.x * NSEM_NOALLOC_CHUNK;
    for (int q = 0; q < PER_THREAD; q++) {
        const int64_t i = base + (int64_t)q * NT + threadIdx.x;
        if (i >= in.n) break;
        const double r = in.u[0][i];
        const double U[3] = {in.u[1][i] / r, in.u[2][i] / r, in.u[3][i] / r};
        const double T = in.u[4][i] / r;
        const double p = in.P0 * nsem_pow(((r * T) * in.R) / in.P0, in.gamma);
        const double pp = p - in.p_ref[i];
        const double cv = in.cV[i];
        const double ke = U[0] * U[0] + (U[1] * U[1] + (U[2] * U[2] + 0.0));
        const double sf = (in.gh[i] + 0.5 * ke) +
                          (nsem_pow((pp + in.p_ref[i]) / in.P0, in.kappa) * T) * in.cv_heat;
        acc[0] = cadd(acc[0], r * cv);
        acc[1] = cadd(acc[1], (r * cv) * sf);
        acc[2] = cadd(acc[2], cv);
    }
    block_reduce3(acc, sh);
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; q++) {
            scratch[(int64_t)(2 * q) * NSEM_NOALLOC_MAX_CHUNKS + blockIdx.x] = acc[q].s;
            scratch[(int64_t)(2 * q + 1) * NSEM_NOALLOC_MAX_CHUNKS + blockIdx.x] = acc[q].c;
        }
}

__global__ void __launch_bounds__(NT) k_final(const double* scratch, int nchunks, double* out) {
    __shared__ CSum sh[3 * NT];
    CSum acc[3] = {{0, 0}, {0, 0}, {0, 0}};
    for (int b = threadIdx.x; b < nchunks; b += NT)
        for (int q = 0; q < 3; q++) {
            CSum x;
            x.s = scratch[(int64_t)(2 * q) * NSEM_NOALLOC_MAX_CHUNKS + b];
            x.c = scratch[(int64_t)(2 * q + 1) * NSEM_NOALLOC_MAX_CHUNKS + b];
            acc[q] = cmerge(acc[q], x);
        }
    block_reduce3(acc, sh);
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; q++) out[q] = acc[q].s + acc[q].c;
}

}  // namespace

extern "C" nsem_status nsem_conservation_sums_noalloc(
    const double* rho, const double* rhou, const double* rhov, const double* rhow,
    const double* rhoTheta, const double* cV, const double* gh, const double* p_ref,
    int64_t n_nodes, double P0, double cp, double cv, double* out3, void* stream) {
    if (!rho || !rhou || !rhov || !rhow || !rhoTheta || !cV || !gh || !p_ref || !out3)
        return NSEM_BAD_ARG;
    if (n_nodes < 1) return NSEM_BAD_ARG;
    if (n_nodes > NSEM_NOALLOC_MAX_NODES) return NSEM_TOO_LARGE;
    if (!(cp > cv) || !(cv > 0) || !(P0 > 0)) return NSEM_BAD_ARG;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES)
        return NSEM_CUDA_ERROR;
    double* scratch;
    {
        /* set-up on the first call on this device: resolve the array's
         * device address with the device current */
        std::lock_guard<std::mutex> lk(g_lock);
        if (!g_scratch[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, nsem_noalloc_scratch) != cudaSuccess || !p)
                return NSEM_CUDA_ERROR;
            g_scratch[dev] = (double*)p;
        }
        scratch = g_scratch[dev];
    }
    Inputs in;
    in.u[0] = rho; in.u[1] = rhou; in.u[2] = rhov; in.u[3] = rhow; in.u[4] = rhoTheta;
    in.cV = cV;
    in.gh = gh;
    in.p_ref = p_ref;
    in.n = n_nodes;
    in.P0 = P0;
    in.R = cp - cv;
    in.gamma = cp / cv;
    in.kappa = in.R / cp;
    in.cv_heat = cv;
    const int nchunks = (int)((n_nodes + NSEM_NOALLOC_CHUNK - 1) / NSEM_NOALLOC_CHUNK);
    cudaStream_t st = (cudaStream_t)stream;
    /* each launch is checked right after it; cudaGetLastError also returns
     * (and clears) an error left pending by the caller's earlier launches,
     * which is then reported as this call's NSEM_CUDA_ERROR */
    k_chunk_sums<<<nchunks, NT, 0, st>>>(in, scratch, nchunks);
    if (cudaGetLastError() != cudaSuccess) return NSEM_CUDA_ERROR;
    k_final<<<1, NT, 0, st>>>(scratch, nchunks, out3);
    return cudaGetLastError() == cudaSuccess ? NSEM_OK : NSEM_CUDA_ERROR;
}
