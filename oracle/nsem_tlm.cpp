/*
 * CPU FP64 tangent-linear model of the coupled SSP-RK3 dGSEM Euler step.
 *
 * TEST INFRASTRUCTURE ONLY: the reference for the GPU discrete adjoint.  The
 * operator chain of nsem_oracle.c (itself a bit-exact restatement of the
 * reference's divf / rusanov / applyExplicitBCs / src, see that file) is
 * written once as a template and evaluated on dual numbers (value,
 * derivative), which gives the exact directional derivative J_L(u) du of the
 * tendency and, through the Shu-Osher stages, of the step map.  Non-smooth
 * points take one-sided choices: d|x| = sign(x) dx with sign(0) = 0, and the
 * SYMMETRY ghost follows the same branch (|r| <= 1e-7) as the value.
 */
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "nsem_oracle.h"

namespace {

/* the equation-of-state pow follows the oracle's switch (C library or the
 * correctly rounded restatement), so values match nsem_oracle_tendency */
inline double eos_pow(double a, double e) {
    return nsem_oracle_get_pow() ? nsem_oracle_pow_dd(a, e) : std::pow(a, e);
}

/* value plus K directional derivatives (K directions share one pass) */
template <int K>
struct DualN {
    double v, d[K];
    DualN() : v(0) { for (int i = 0; i < K; i++) d[i] = 0; }
    DualN(double x) : v(x) { for (int i = 0; i < K; i++) d[i] = 0; }
};
template <int K>
inline DualN<K> operator+(const DualN<K>& a, const DualN<K>& b) {
    DualN<K> r(a.v + b.v);
    for (int i = 0; i < K; i++) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <int K>
inline DualN<K> operator-(const DualN<K>& a, const DualN<K>& b) {
    DualN<K> r(a.v - b.v);
    for (int i = 0; i < K; i++) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <int K>
inline DualN<K> operator-(const DualN<K>& a) {
    DualN<K> r(-a.v);
    for (int i = 0; i < K; i++) r.d[i] = -a.d[i];
    return r;
}
template <int K>
inline DualN<K> operator*(const DualN<K>& a, const DualN<K>& b) {
    DualN<K> r(a.v * b.v);
    for (int i = 0; i < K; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
template <int K>
inline DualN<K> operator*(const DualN<K>& a, double b) {
    DualN<K> r(a.v * b);
    for (int i = 0; i < K; i++) r.d[i] = a.d[i] * b;
    return r;
}
template <int K>
inline DualN<K> operator*(double a, const DualN<K>& b) {
    DualN<K> r(a * b.v);
    for (int i = 0; i < K; i++) r.d[i] = a * b.d[i];
    return r;
}
template <int K>
inline DualN<K> operator+(const DualN<K>& a, double b) {
    DualN<K> r(a.v + b);
    for (int i = 0; i < K; i++) r.d[i] = a.d[i];
    return r;
}
template <int K>
inline DualN<K> operator-(const DualN<K>& a, double b) {
    DualN<K> r(a.v - b);
    for (int i = 0; i < K; i++) r.d[i] = a.d[i];
    return r;
}
template <int K>
inline DualN<K> operator/(const DualN<K>& a, const DualN<K>& b) {
    const double q = a.v / b.v;
    DualN<K> r(q);
    for (int i = 0; i < K; i++) r.d[i] = (a.d[i] - q * b.d[i]) / b.v;
    return r;
}
template <int K>
inline DualN<K> operator/(const DualN<K>& a, double b) {
    DualN<K> r(a.v / b);
    for (int i = 0; i < K; i++) r.d[i] = a.d[i] / b;
    return r;
}
template <int K>
inline DualN<K> sqrt_(const DualN<K>& a) {
    const double s = std::sqrt(a.v);
    DualN<K> r(s);
    for (int i = 0; i < K; i++) r.d[i] = s > 0 ? a.d[i] / (2 * s) : 0.0;
    return r;
}
template <int K>
inline DualN<K> pow_(const DualN<K>& a, double e) {
    const double p = eos_pow(a.v, e);
    DualN<K> r(p);
    const double f = a.v != 0 ? e * p / a.v : 0.0;
    for (int i = 0; i < K; i++) r.d[i] = f * a.d[i];
    return r;
}
template <int K>
inline double val(const DualN<K>& a) { return a.v; }
using Dual = DualN<1>;
inline double val(double a) { return a; }
inline double sqrt_(double a) { return std::sqrt(a); }
inline double pow_(double a, double e) { return eos_pow(a, e); }

enum { XX, YY, ZZ, XY, YZ, XZ, YX, ZY, ZX };

template <typename T>
inline T vdot(const T* a, const T* b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }
template <typename T>
inline T vdotd(const T* a, const double* b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }

template <typename T>
inline void tdotd(const T* q, const double* p, T* r) {
    r[0] = q[XX] * p[0] + q[XY] * p[1] + q[XZ] * p[2];
    r[1] = q[YX] * p[0] + q[YY] * p[1] + q[YZ] * p[2];
    r[2] = q[ZX] * p[0] + q[ZY] * p[1] + q[ZZ] * p[2];
}
template <typename T>
inline void outer(const T* p, const T* q, T* r) {
    r[XX] = p[0] * q[0]; r[YY] = p[1] * q[1]; r[ZZ] = p[2] * q[2];
    r[XY] = p[0] * q[1]; r[YZ] = p[1] * q[2]; r[XZ] = p[0] * q[2];
    r[YX] = p[1] * q[0]; r[ZY] = p[2] * q[1]; r[ZX] = p[2] * q[0];
}

/* SYMMETRY ghost velocity (tangential projection rescaled to |p|) */
template <typename T>
inline void sym_vec(const T* p, const double* n, T* out) {
    const double mg = std::sqrt(n[0] * n[0] + (n[1] * n[1] + n[2] * n[2]));
    const double en[3] = {n[0] / mg, n[1] / mg, n[2] / mg};
    const double A[6] = {1.0 - en[0] * en[0], 1.0 - en[1] * en[1], 1.0 - en[2] * en[2],
                         -en[0] * en[1], -en[1] * en[2], -en[0] * en[2]};
    T r[3];
    r[0] = p[0] * A[0] + p[1] * A[3] + p[2] * A[5];
    r[1] = p[0] * A[3] + p[1] * A[1] + p[2] * A[4];
    r[2] = p[0] * A[5] + p[1] * A[4] + p[2] * A[2];
    const T magR = sqrt_(vdot(r, r));
    if (std::fabs(val(magR)) <= 1e-7) {
        out[0] = r[0]; out[1] = r[1]; out[2] = r[2];
        return;
    }
    const T s = sqrt_(vdot(p, p)) / magR;
    out[0] = r[0] * s; out[1] = r[1] * s; out[2] = r[2] * s;
}

/* strong-form DG gradient of ncomp (1 or 3) components per node, as
 * nsem_oracle.c grad_strong(): face terms fN (x) (cds(p) - p) in the cell's face
 * order, the volume derivative along the node's three lines, divided by cV;
 * G[r][c] = d_r p_c (XX..ZX) for vectors, interior nodes only */
template <typename T>
void grad_strong_t(const nsem_oracle_mesh* m, int ncomp, const std::vector<T>& p, std::vector<T>& G) {
    const int NPX = m->npx, NPY = m->npy, NPZ = m->npz, NP = m->np, NPF = m->npf;
    const int64_t n_all = m->n_all;
    const int w = ncomp == 1 ? 3 : 9;
    G.assign((size_t)w * n_all, T(0.0));
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m->n_elem; e++) {
        const int64_t base = e * NP;
        for (uint32_t f = m->face_idx0[e]; f < m->face_idx1[e]; f++)
            for (int nn = 0; nn < NPF; nn++) {
                const int64_t k = (int64_t)m->all_faces[f] * NPF + nn;
                const uint32_t c1 = m->FO[k], c2 = m->FN[k];
                if (c1 >= (uint32_t)n_all || c2 >= (uint32_t)n_all) continue;
                const double fi = m->fI[k], fo = 1 - fi;
                const double* n = m->fN + 3 * k;
                const bool mine = c1 >= base && c1 < base + NP;
                const uint32_t own = mine ? c1 : c2;
                T d[3];
                for (int c = 0; c < ncomp; c++)
                    d[c] = (p[(size_t)ncomp * c1 + c] * fi + p[(size_t)ncomp * c2 + c] * fo) -
                           p[(size_t)ncomp * own + c];
                T* g = &G[(size_t)w * own];
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < ncomp; c++) {
                        const int idx = ncomp == 1 ? r : (r == c) ? r : (r == 0 && c == 1) ? XY
                                      : (r == 1 && c == 2) ? YZ : (r == 0 && c == 2) ? XZ
                                      : (r == 1 && c == 0) ? YX : (r == 2 && c == 1) ? ZY : ZX;
                        const T t = n[r] * d[c];
                        g[idx] = mine ? g[idx] + t : g[idx] - t;
                    }
            }
        for (int ii = 0; ii < NPX; ii++)
        for (int jj = 0; jj < NPY; jj++)
        for (int kk = 0; kk < NPZ; kk++) {
            const int64_t a = base + (int64_t)ii * NPY * NPZ + jj * NPZ + kk;
            double Jin[9];
            for (int c = 0; c < 9; c++) Jin[c] = m->Jinv[9 * a + c] * m->cV[a];
            T* g = &G[(size_t)w * a];
            for (int pass = 0; pass < 3; pass++) {
                const int lim = pass == 0 ? NPX : pass == 1 ? NPY : NPZ;
                for (int q = 0; q < lim; q++) {
                    int im = ii, jm = jj, km = kk;
                    if (pass == 0) im = q;
                    else if (pass == 1) { if (q == jj) continue; jm = q; }
                    else { if (q == kk) continue; km = q; }
                    const int64_t b = base + (int64_t)im * NPY * NPZ + jm * NPZ + km;
                    double dv[3], dj[3];
                    dv[0] = m->dpsi[0][ii * NPX + im] * m->psi[1][jj * NPY + jm] * m->psi[2][kk * NPZ + km];
                    dv[1] = m->psi[0][ii * NPX + im] * m->dpsi[1][jj * NPY + jm] * m->psi[2][kk * NPZ + km];
                    dv[2] = m->psi[0][ii * NPX + im] * m->psi[1][jj * NPY + jm] * m->dpsi[2][kk * NPZ + km];
                    dj[0] = Jin[XX] * dv[0] + Jin[XY] * dv[1] + Jin[XZ] * dv[2];
                    dj[1] = Jin[YX] * dv[0] + Jin[YY] * dv[1] + Jin[YZ] * dv[2];
                    dj[2] = Jin[ZX] * dv[0] + Jin[ZY] * dv[1] + Jin[ZZ] * dv[2];
                    for (int r = 0; r < 3; r++)
                        for (int c = 0; c < ncomp; c++) {
                            const int idx = ncomp == 1 ? r : (r == c) ? r : (r == 0 && c == 1) ? XY
                                          : (r == 1 && c == 2) ? YZ : (r == 0 && c == 2) ? XZ
                                          : (r == 1 && c == 0) ? YX : (r == 2 && c == 1) ? ZY : ZX;
                            g[idx] = g[idx] + dj[r] * p[(size_t)ncomp * b + c];
                        }
                }
            }
            for (int c = 0; c < w; c++) g[c] = g[c] / m->cV[a];
        }
    }
}

/* tendency L = -Su/cV on interior nodes, same operator chain as
 * nsem_oracle.c residual() (with its artificial viscosity when nu != 0) */
template <typename T>
void tendency(const nsem_oracle_mesh* m, const std::vector<T>* u, std::vector<T>* L) {
    const int NPX = m->npx, NPY = m->npy, NPZ = m->npz, NP = m->np, NPF = m->npf;
    const int64_t n_int = m->n_int, n_all = m->n_all;
    const int64_t n_slot = (int64_t)m->n_face * NPF;
    const double P0 = m->P0, R = m->R, gam = m->gamma, gR = gam * R;
    std::vector<T> rho(n_all), U(3 * n_all), Th(n_all), p(n_all);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n_int; i++) {
        const T r = u[0][i];
        rho[i] = r;
        U[3 * i + 0] = u[1][i] / r;
        U[3 * i + 1] = u[2][i] / r;
        U[3 * i + 2] = u[3][i] / r;
        Th[i] = u[4][i] / r;
    }
    for (int64_t k = 0; k < n_slot; k++) {
        if (!m->bcU[k]) continue;
        const uint32_t c1 = m->FO[k], c2 = m->FN[k];
        if (c2 >= (uint32_t)n_all) continue;
        rho[c2] = rho[c1];
        Th[c2] = Th[c1];
        if (m->bcU[k] == 2) sym_vec(&U[3 * (size_t)c1], m->fN + 3 * k, &U[3 * (size_t)c2]);
        else for (int c = 0; c < 3; c++) U[3 * (size_t)c2 + c] = U[3 * (size_t)c1 + c];
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n_all; i++) p[i] = P0 * pow_(((rho[i] * Th[i]) * R) / P0, gam) - m->p_ref[i];

    /* artificial viscosity: mu = rho nu, gradients of U and theta (zero on ghosts) */
    const bool visc = m->nu != 0.0;
    const double iPr = visc ? 1 / m->Pr : 0.0;
    std::vector<T> mu, GU, GT;
    if (visc) {
        mu.resize(n_all);
        for (int64_t i = 0; i < n_all; i++) mu[i] = rho[i] * m->nu;
        grad_strong_t(m, 3, U, GU);
        grad_strong_t(m, 1, Th, GT);
    }

    std::vector<T> dr(n_slot), dm(3 * n_slot), dt_(n_slot);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n_slot; k++) {
        const uint32_t c1 = m->FO[k], c2 = m->FN[k];
        if (c1 >= (uint32_t)n_all || c2 >= (uint32_t)n_all) continue;
        const double fi = m->fI[k], fo = 1 - fi;
        const double* n = m->fN + 3 * k;
        const double mgn = std::sqrt(n[0] * n[0] + (n[1] * n[1] + n[2] * n[2]));
        const double en[3] = {n[0] / mgn, n[1] / mgn, n[2] / mgn};
        const T* U1 = &U[3 * (size_t)c1];
        const T* U2 = &U[3 * (size_t)c2];
        const T r1 = rho[c1], r2 = rho[c2], T1 = Th[c1], T2 = Th[c2], p1 = p[c1], p2 = p[c2];
        const T lam = ((sqrt_(vdot(U1, U1)) * fi + sqrt_(vdot(U2, U2)) * fo) +
                       (sqrt_(T1 * gR) * fi + sqrt_(T2 * gR) * fo)) * 0.5;
        {
            T F[3];
            const T jump = lam * (r2 - r1);
            for (int c = 0; c < 3; c++) F[c] = (U1[c] * r1 * fi + U2[c] * r2 * fo) - jump * en[c];
            dr[k] = vdotd(F, n);
        }
        {
            T Fc1[3], Fc2[3], A[9], B[9], F[9], out[3];
            for (int c = 0; c < 3; c++) { Fc1[c] = U1[c] * r1; Fc2[c] = U2[c] * r2; }
            outer(Fc1, U1, A);
            outer(Fc2, U2, B);
            for (int c = 0; c < 3; c++) { A[c] = A[c] + p1; B[c] = B[c] + p2; }
            if (visc) {
                const bool g1 = c1 < (uint32_t)n_int, g2 = c2 < (uint32_t)n_int;
                for (int c = 0; c < 9; c++) {
                    A[c] = A[c] - mu[c1] * (g1 ? GU[9 * (size_t)c1 + c] : T(0.0));
                    B[c] = B[c] - mu[c2] * (g2 ? GU[9 * (size_t)c2 + c] : T(0.0));
                }
            }
            T dq[3];
            for (int c = 0; c < 3; c++) dq[c] = (Fc2[c] - Fc1[c]) * lam;
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                    const int idx = (r == c) ? r : (r == 0 && c == 1) ? XY : (r == 1 && c == 2) ? YZ
                                  : (r == 0 && c == 2) ? XZ : (r == 1 && c == 0) ? YX
                                  : (r == 2 && c == 1) ? ZY : ZX;
                    F[idx] = (A[idx] * fi + B[idx] * fo) - dq[c] * en[r];
                }
            tdotd(F, n, out);
            for (int c = 0; c < 3; c++) dm[3 * k + c] = out[c];
        }
        {
            T F[3];
            const T jump = lam * (r2 * T2 - r1 * T1);
            for (int c = 0; c < 3; c++) {
                T a = U1[c] * r1 * T1, b = U2[c] * r2 * T2;
                if (visc) {
                    a = a - (mu[c1] * iPr) * (c1 < (uint32_t)n_int ? GT[3 * (size_t)c1 + c] : T(0.0));
                    b = b - (mu[c2] * iPr) * (c2 < (uint32_t)n_int ? GT[3 * (size_t)c2 + c] : T(0.0));
                }
                F[c] = (a * fi + b * fo) - jump * en[c];
            }
            dt_[k] = vdotd(F, n);
        }
    }

    std::vector<T> rr(n_int), rm(3 * n_int), rt(n_int);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m->n_elem; e++) {
        const int64_t base = e * NP;
        for (uint32_t f = m->face_idx0[e]; f < m->face_idx1[e]; f++)
            for (int nn = 0; nn < NPF; nn++) {
                const int64_t k = (int64_t)m->all_faces[f] * NPF + nn;
                const uint32_t c1 = m->FO[k], c2 = m->FN[k];
                if (c1 >= base && c1 < base + NP) {
                    rr[c1] = rr[c1] + dr[k];
                    for (int c = 0; c < 3; c++) rm[3 * (size_t)c1 + c] = rm[3 * (size_t)c1 + c] + dm[3 * k + c];
                    rt[c1] = rt[c1] + dt_[k];
                } else if (c2 < (uint32_t)n_all) {
                    rr[c2] = rr[c2] - dr[k];
                    for (int c = 0; c < 3; c++) rm[3 * (size_t)c2 + c] = rm[3 * (size_t)c2 + c] - dm[3 * k + c];
                    rt[c2] = rt[c2] - dt_[k];
                }
            }
        for (int ii = 0; ii < NPX; ii++)
        for (int jj = 0; jj < NPY; jj++)
        for (int kk = 0; kk < NPZ; kk++) {
            const int64_t b = base + (int64_t)ii * NPY * NPZ + jj * NPZ + kk;
            double Jin[9];
            for (int c = 0; c < 9; c++) Jin[c] = m->Jinv[9 * b + c] * m->cV[b];
            const T* Ub = &U[3 * b];
            T Fc[3] = {Ub[0] * rho[b], Ub[1] * rho[b], Ub[2] * rho[b]};
            T fm[9];
            outer(Fc, Ub, fm);
            for (int c = 0; c < 3; c++) fm[c] = fm[c] + p[b];
            T ft[3] = {Fc[0] * Th[b], Fc[1] * Th[b], Fc[2] * Th[b]};
            if (visc) {
                for (int c = 0; c < 9; c++) fm[c] = fm[c] - mu[b] * GU[9 * b + c];
                for (int c = 0; c < 3; c++) ft[c] = ft[c] - (mu[b] * iPr) * GT[3 * b + c];
            }
            for (int pass = 0; pass < 3; pass++) {
                const int lim = pass == 0 ? NPX : pass == 1 ? NPY : NPZ;
                for (int q = 0; q < lim; q++) {
                    int im = ii, jm = jj, km = kk;
                    if (pass == 0) im = q;
                    else if (pass == 1) { if (q == jj) continue; jm = q; }
                    else { if (q == kk) continue; km = q; }
                    const int64_t a = base + (int64_t)im * NPY * NPZ + jm * NPZ + km;
                    double dv[3], dj[3];
                    dv[0] = m->dpsi[0][ii * NPX + im] * m->psi[1][jj * NPY + jm] * m->psi[2][kk * NPZ + km];
                    dv[1] = m->psi[0][ii * NPX + im] * m->dpsi[1][jj * NPY + jm] * m->psi[2][kk * NPZ + km];
                    dv[2] = m->psi[0][ii * NPX + im] * m->psi[1][jj * NPY + jm] * m->dpsi[2][kk * NPZ + km];
                    dj[0] = Jin[XX] * dv[0] + Jin[XY] * dv[1] + Jin[XZ] * dv[2];
                    dj[1] = Jin[YX] * dv[0] + Jin[YY] * dv[1] + Jin[YZ] * dv[2];
                    dj[2] = Jin[ZX] * dv[0] + Jin[ZY] * dv[1] + Jin[ZZ] * dv[2];
                    rr[a] = rr[a] - vdotd(Fc, dj);
                    T t[3];
                    tdotd(fm, dj, t);
                    for (int c = 0; c < 3; c++) rm[3 * a + c] = rm[3 * a + c] - t[c];
                    rt[a] = rt[a] - vdotd(ft, dj);
                }
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n_int; i++) {
        const T s = rho[i] - m->rho_ref[i];
        for (int c = 0; c < 3; c++) rm[3 * i + c] = rm[3 * i + c] - s * m->gravity[c] * m->cV[i];
        const double cv = m->cV[i];
        L[0][i] = -(rr[i] / cv);
        L[1][i] = -(rm[3 * i + 0] / cv);
        L[2][i] = -(rm[3 * i + 1] / cv);
        L[3][i] = -(rm[3 * i + 2] / cv);
        L[4][i] = -(rt[i] / cv);
    }
}

/* Tangent-linear SSP-RK3 on K directions at once: u (values) and du[d][c]
 * advanced in place by nsteps steps; nd <= K directions are used. */
template <int K>
void tlm_ssprk3(const nsem_oracle_mesh* m, double* const u[5], double* const* du, int nd,
                double dt, int nsteps) {
    const int64_t n = m->n_int;
    std::vector<DualN<K>> u0[5], s[5], L[5];
    for (int c = 0; c < 5; c++) {
        u0[c].resize(n); s[c].resize(n); L[c].resize(n);
        for (int64_t i = 0; i < n; i++) {
            u0[c][i] = DualN<K>(u[c][i]);
            for (int d = 0; d < nd; d++) u0[c][i].d[d] = du[5 * d + c][i];
        }
    }
    const double a2 = 0.75, b2 = 0.25, a3 = 1.0 / 3.0, b3 = 2.0 / 3.0;
    for (int st = 0; st < nsteps; st++) {
        tendency<DualN<K>>(m, u0, L);
        for (int c = 0; c < 5; c++) {
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) s[c][i] = u0[c][i] + L[c][i] * dt;
        }
        tendency<DualN<K>>(m, s, L);
        for (int c = 0; c < 5; c++) {
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) s[c][i] = u0[c][i] * a2 + (s[c][i] + L[c][i] * dt) * b2;
        }
        tendency<DualN<K>>(m, s, L);
        for (int c = 0; c < 5; c++) {
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; i++) u0[c][i] = u0[c][i] * a3 + (s[c][i] + L[c][i] * dt) * b3;
        }
    }
    for (int c = 0; c < 5; c++)
        for (int64_t i = 0; i < n; i++) {
            u[c][i] = u0[c][i].v;
            for (int d = 0; d < nd; d++) du[5 * d + c][i] = u0[c][i].d[d];
        }
}

}  // namespace

extern "C" {

/* Directional derivative of the tendency: Ld = J_L(u) du (and L itself). */
void nsem_oracle_jvp(const nsem_oracle_mesh* m, const double* const u[5], const double* const du[5],
                     double* const L[5], double* const Ld[5]) {
    const int64_t n = m->n_int;
    std::vector<Dual> uu[5], LL[5];
    for (int c = 0; c < 5; c++) {
        uu[c].resize(n);
        LL[c].resize(n);
        for (int64_t i = 0; i < n; i++) {
            uu[c][i] = Dual(u[c][i]);
            uu[c][i].d[0] = du[c][i];
        }
    }
    tendency<Dual>(m, uu, LL);
    for (int c = 0; c < 5; c++)
        for (int64_t i = 0; i < n; i++) {
            if (L) L[c][i] = LL[c][i].v;
            Ld[c][i] = LL[c][i].d[0];
        }
}

/* Tangent-linear SSP-RK3: advances (u, du) in place by nsteps steps. */
void nsem_oracle_tlm_ssprk3(const nsem_oracle_mesh* m, double* const u[5], double* const du[5],
                            double dt, int nsteps) {
    tlm_ssprk3<1>(m, u, du, 1, dt, nsteps);
}

/* Same for nd <= 8 directions in one pass; du holds 5*nd arrays, direction
 * d's variable c at du[5*d + c].  Returns 0, or -1 if nd is out of range. */
int nsem_oracle_tlm_ssprk3_multi(const nsem_oracle_mesh* m, double* const u[5], double* const* du,
                                 int nd, double dt, int nsteps) {
    if (nd < 1 || nd > 8) return -1;
    if (nd == 1) tlm_ssprk3<1>(m, u, du, 1, dt, nsteps);
    else if (nd <= 4) tlm_ssprk3<4>(m, u, du, nd, dt, nsteps);
    else tlm_ssprk3<8>(m, u, du, nd, dt, nsteps);
    return 0;
}

}  // extern "C"
