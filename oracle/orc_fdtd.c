/* orc_fdtd.c — FP64 CPU restatement of the reference Yee FDTD time loop.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY (see ems_oracle.h).
 *
 * Restates fdtd/fdtd_simulation.cpp:
 *   - field layout with ghost padding            (57-68)
 *   - H update from curl E                       (119-169)
 *   - E update from curl H                       (170-220)
 *   - point sources E[src] -= s(t)*dt/eps        (222-239), s(t) at 24-36
 *   - run loop, receiver averaging, sampling     (242-306)
 * In the reference-only configuration (no material table, no CPML, kind-0
 * sources) every floating-point operation is performed in the reference's
 * order, so results are bit-identical to the reference built with
 * -ffp-contract=off.  Extensions (not in the reference):
 *   - per-cell eps/sigma through a material table, each E sample taking the
 *     material of one owning cell; E = ca*E + cb*curl, which for sigma = 0 is
 *     exactly the reference update (ca = 1, cb = dt/eps/h);
 *   - a convolutional PML (Roden & Gedney, 2000) on all faces, with
 *     polynomially graded sigma and kappa and linearly graded alpha.
 */
#include "ems_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define EX(i, j, k) ((size_t)(i) + (size_t)(j) * (nx + 1) + (size_t)(k) * (nx + 1) * (ny + 2))
#define EY(i, j, k) ((size_t)(i) + (size_t)(j) * (nx + 2) + (size_t)(k) * (nx + 2) * (ny + 1))
#define EZ(i, j, k) ((size_t)(i) + (size_t)(j) * (nx + 2) + (size_t)(k) * (nx + 2) * (ny + 2))
#define HX(i, j, k) ((size_t)(i) + (size_t)(j) * nx + (size_t)(k) * nx * (ny + 1))
#define HY(i, j, k) ((size_t)(i) + (size_t)(j) * (nx + 1) + (size_t)(k) * (nx + 1) * ny)
#define HZ(i, j, k) ((size_t)(i) + (size_t)(j) * (nx + 1) + (size_t)(k) * (nx + 1) * (ny + 1))

/* fdtd/fdtd_simulation.cpp:24-36 (kind 0: Gaussian derivative, f0 = 1 GHz in
 * the reference; kind 1: the Ricker wavelet the reference keeps commented
 * out at 28-32, centred at sqrt(2)/f0).  dl = 1 mm Hertz dipole over h^3. */
double orc_fdtd_source(int kind, double f0, double t, double h)
{
    if (kind == 0)
        return -4.0 * M_PI * M_PI * f0 * f0 * (t - 1.0 / f0) *
               exp(-2.0 * M_PI * M_PI * f0 * f0 * (t - 1.0 / f0) * (t - 1.0 / f0)) / h / h / h * 0.001;
    double tau = t - sqrt(2.0) / f0;
    return (1.0 - 2.0 * M_PI * M_PI * f0 * f0 * tau * tau) * exp(-M_PI * M_PI * f0 * f0 * tau * tau) / h / h / h * 0.001;
}

typedef struct { double *b, *a, *kinv; int *on; } pml_prof;

/* CPML coefficients at positions x = s + shift (units of h), s in [0, n]. */
static void make_prof(pml_prof *p, int n, int L, double shift, const orc_fdtd_case *c)
{
    p->b = calloc((size_t)n + 2, sizeof(double));
    p->a = calloc((size_t)n + 2, sizeof(double));
    p->kinv = calloc((size_t)n + 2, sizeof(double));
    p->on = calloc((size_t)n + 2, sizeof(int));
    double eta = sqrt(c->mu / c->eps);
    double smax = L > 0 ? -(c->pml_m + 1.0) * log(c->pml_R0) / (2.0 * eta * L * c->h) : 0.0;
    for (int s = 0; s <= n + 1; ++s) {
        double x = s + shift, d = 0.0;
        if (L > 0) {
            double lo = L - x, hi = x - (n - L);
            d = lo > hi ? lo : hi;
            d = d < 0.0 ? 0.0 : (d > L ? 1.0 : d / L);
        }
        p->kinv[s] = 1.0;
        if (d <= 0.0) continue;
        double g = pow(d, c->pml_m);
        double sig = smax * g, kap = 1.0 + (c->pml_kmax - 1.0) * g, alp = c->pml_amax * (1.0 - d);
        double b = exp(-(sig / kap + alp) * c->dt / c->eps);
        p->b[s] = b;
        p->a[s] = sig > 0.0 ? sig / (sig * kap + kap * kap * alp) * (b - 1.0) : 0.0;
        p->kinv[s] = 1.0 / kap;
        p->on[s] = 1;
    }
}

int orc_fdtd_run(const orc_fdtd_case *c, int nsteps, double *E[3], double *H[3], double *traces)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz, tf = c->time_frequency;
    const double dt = c->dt;
    double *Ex = E[0], *Ey = E[1], *Ez = E[2], *Hx = H[0], *Hy = H[1], *Hz = H[2];
    const double ch = dt / c->mu / c->h;    /* fdtd_simulation.cpp:128 operand order */
    const double ce = dt / c->eps / c->h;   /* fdtd_simulation.cpp:179 */
    const int L = c->pml;

    /* per-material update coefficients */
    int nmat = c->mat_id ? c->nmat : 0;
    double *ca = NULL, *cb = NULL, *cs = NULL;
    if (nmat) {
        ca = malloc(sizeof(double) * nmat); cb = malloc(sizeof(double) * nmat); cs = malloc(sizeof(double) * nmat);
        for (int m = 0; m < nmat; ++m) {
            double s = c->mat_sigma[m] * dt / (2.0 * c->mat_eps[m]);
            ca[m] = (1.0 - s) / (1.0 + s);
            cb[m] = dt / c->mat_eps[m] / c->h / (1.0 + s);
            cs[m] = 1.0 + s;
        }
    }
#define CELL(i, j, k) c->mat_id[(size_t)(i) + (size_t)(j) * nx + (size_t)(k) * nx * ny]

    /* CPML: E-type derivatives at s - 1/2, H-type at s, per direction */
    pml_prof pe[3], ph[3];
    double *psiE[3][2], *psiH[3][2];
    const int n3[3] = {nx, ny, nz};
    size_t nE[3] = {(size_t)(nx + 1) * (ny + 2) * (nz + 2), (size_t)(nx + 2) * (ny + 1) * (nz + 2), (size_t)(nx + 2) * (ny + 2) * (nz + 1)};
    size_t nH[3] = {(size_t)nx * (ny + 1) * (nz + 1), (size_t)(nx + 1) * ny * (nz + 1), (size_t)(nx + 1) * (ny + 1) * nz};
    if (L > 0) {
        for (int d = 0; d < 3; ++d) { make_prof(&pe[d], n3[d], L, -0.5, c); make_prof(&ph[d], n3[d], L, 0.0, c); }
        for (int q = 0; q < 3; ++q)
            for (int r = 0; r < 2; ++r) { psiE[q][r] = calloc(nE[q], sizeof(double)); psiH[q][r] = calloc(nH[q], sizeof(double)); }
    }

    int nsamp = nsteps / tf + 1;
    if (traces) memset(traces, 0, sizeof(double) * (size_t)c->nobs * nsamp * 3);
    double t = 0.0;

    for (int step = 1; step < nsteps + 1; ++step) {
        /* ---- H from curl E (fdtd_simulation.cpp:119-169) ---- */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < nz + 1; ++k)
            for (int j = 0; j < ny + 1; ++j)
                for (int i = 0; i < nx; ++i) {
                    size_t p = HX(i, j, k);
                    if (L > 0 && (ph[1].on[j] || ph[2].on[k])) {
                        double d1 = Ez[EZ(i + 1, j + 1, k)] - Ez[EZ(i + 1, j, k)];
                        double d2 = Ey[EY(i + 1, j, k + 1)] - Ey[EY(i + 1, j, k)];
                        double *p1 = &psiH[0][0][p], *p2 = &psiH[0][1][p];
                        *p1 = ph[1].b[j] * *p1 + ph[1].a[j] * d1;
                        *p2 = ph[2].b[k] * *p2 + ph[2].a[k] * d2;
                        Hx[p] -= ch * (ph[1].kinv[j] * d1 - ph[2].kinv[k] * d2 + *p1 - *p2);
                    } else {
                        Hx[p] -= ch * (Ez[EZ(i + 1, j + 1, k)] - Ez[EZ(i + 1, j, k)] - Ey[EY(i + 1, j, k + 1)] + Ey[EY(i + 1, j, k)]);
                    }
                }
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < nz + 1; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx + 1; ++i) {
                    size_t p = HY(i, j, k);
                    if (L > 0 && (ph[2].on[k] || ph[0].on[i])) {
                        double d1 = Ex[EX(i, j + 1, k + 1)] - Ex[EX(i, j + 1, k)];
                        double d2 = Ez[EZ(i + 1, j + 1, k)] - Ez[EZ(i, j + 1, k)];
                        double *p1 = &psiH[1][0][p], *p2 = &psiH[1][1][p];
                        *p1 = ph[2].b[k] * *p1 + ph[2].a[k] * d1;
                        *p2 = ph[0].b[i] * *p2 + ph[0].a[i] * d2;
                        Hy[p] -= ch * (ph[2].kinv[k] * d1 - ph[0].kinv[i] * d2 + *p1 - *p2);
                    } else {
                        Hy[p] -= ch * (Ex[EX(i, j + 1, k + 1)] - Ex[EX(i, j + 1, k)] - Ez[EZ(i + 1, j + 1, k)] + Ez[EZ(i, j + 1, k)]);
                    }
                }
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny + 1; ++j)
                for (int i = 0; i < nx + 1; ++i) {
                    size_t p = HZ(i, j, k);
                    if (L > 0 && (ph[0].on[i] || ph[1].on[j])) {
                        double d1 = Ey[EY(i + 1, j, k + 1)] - Ey[EY(i, j, k + 1)];
                        double d2 = Ex[EX(i, j + 1, k + 1)] - Ex[EX(i, j, k + 1)];
                        double *p1 = &psiH[2][0][p], *p2 = &psiH[2][1][p];
                        *p1 = ph[0].b[i] * *p1 + ph[0].a[i] * d1;
                        *p2 = ph[1].b[j] * *p2 + ph[1].a[j] * d2;
                        Hz[p] -= ch * (ph[0].kinv[i] * d1 - ph[1].kinv[j] * d2 + *p1 - *p2);
                    } else {
                        Hz[p] -= ch * (Ey[EY(i + 1, j, k + 1)] - Ey[EY(i, j, k + 1)] - Ex[EX(i, j + 1, k + 1)] + Ex[EX(i, j, k + 1)]);
                    }
                }
        /* ---- E from curl H (fdtd_simulation.cpp:170-220) ---- */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 1; k < nz + 1; ++k)
            for (int j = 1; j < ny + 1; ++j)
                for (int i = 0; i < nx + 1; ++i) {
                    size_t p = EX(i, j, k);
                    double a = 1.0, b = ce;
                    if (nmat) { int m = CELL(i < nx ? i : nx - 1, j - 1, k - 1); a = ca[m]; b = cb[m]; }
                    if (L > 0 && (pe[1].on[j] || pe[2].on[k])) {
                        double d1 = Hz[HZ(i, j, k - 1)] - Hz[HZ(i, j - 1, k - 1)];
                        double d2 = Hy[HY(i, j - 1, k)] - Hy[HY(i, j - 1, k - 1)];
                        double *p1 = &psiE[0][0][p], *p2 = &psiE[0][1][p];
                        *p1 = pe[1].b[j] * *p1 + pe[1].a[j] * d1;
                        *p2 = pe[2].b[k] * *p2 + pe[2].a[k] * d2;
                        Ex[p] = a * Ex[p] + b * (pe[1].kinv[j] * d1 - pe[2].kinv[k] * d2 + *p1 - *p2);
                    } else {
                        double curl = Hz[HZ(i, j, k - 1)] - Hz[HZ(i, j - 1, k - 1)] - Hy[HY(i, j - 1, k)] + Hy[HY(i, j - 1, k - 1)];
                        Ex[p] = nmat ? a * Ex[p] + b * curl : Ex[p] + ce * curl;
                    }
                }
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 1; k < nz + 1; ++k)
            for (int j = 0; j < ny + 1; ++j)
                for (int i = 1; i < nx + 1; ++i) {
                    size_t p = EY(i, j, k);
                    double a = 1.0, b = ce;
                    if (nmat) { int m = CELL(i - 1, j < ny ? j : ny - 1, k - 1); a = ca[m]; b = cb[m]; }
                    if (L > 0 && (pe[2].on[k] || pe[0].on[i])) {
                        double d1 = Hx[HX(i - 1, j, k)] - Hx[HX(i - 1, j, k - 1)];
                        double d2 = Hz[HZ(i, j, k - 1)] - Hz[HZ(i - 1, j, k - 1)];
                        double *p1 = &psiE[1][0][p], *p2 = &psiE[1][1][p];
                        *p1 = pe[2].b[k] * *p1 + pe[2].a[k] * d1;
                        *p2 = pe[0].b[i] * *p2 + pe[0].a[i] * d2;
                        Ey[p] = a * Ey[p] + b * (pe[2].kinv[k] * d1 - pe[0].kinv[i] * d2 + *p1 - *p2);
                    } else {
                        double curl = Hx[HX(i - 1, j, k)] - Hx[HX(i - 1, j, k - 1)] - Hz[HZ(i, j, k - 1)] + Hz[HZ(i - 1, j, k - 1)];
                        Ey[p] = nmat ? a * Ey[p] + b * curl : Ey[p] + ce * curl;
                    }
                }
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < nz + 1; ++k)
            for (int j = 1; j < ny + 1; ++j)
                for (int i = 1; i < nx + 1; ++i) {
                    size_t p = EZ(i, j, k);
                    double a = 1.0, b = ce;
                    if (nmat) { int m = CELL(i - 1, j - 1, k < nz ? k : nz - 1); a = ca[m]; b = cb[m]; }
                    if (L > 0 && (pe[0].on[i] || pe[1].on[j])) {
                        double d1 = Hy[HY(i, j - 1, k)] - Hy[HY(i - 1, j - 1, k)];
                        double d2 = Hx[HX(i - 1, j, k)] - Hx[HX(i - 1, j - 1, k)];
                        double *p1 = &psiE[2][0][p], *p2 = &psiE[2][1][p];
                        *p1 = pe[0].b[i] * *p1 + pe[0].a[i] * d1;
                        *p2 = pe[1].b[j] * *p2 + pe[1].a[j] * d2;
                        Ez[p] = a * Ez[p] + b * (pe[0].kinv[i] * d1 - pe[1].kinv[j] * d2 + *p1 - *p2);
                    } else {
                        double curl = Hy[HY(i, j - 1, k)] - Hy[HY(i - 1, j - 1, k)] - Hx[HX(i - 1, j, k)] + Hx[HX(i - 1, j - 1, k)];
                        Ez[p] = nmat ? a * Ez[p] + b * curl : Ez[p] + ce * curl;
                    }
                }
        /* ---- point sources (fdtd_simulation.cpp:222-239) ---- */
        for (int s = 0; s < c->nsrc; ++s) {
            const int *q = c->src_ijk + 3 * s;
            int kind = c->src_kind ? c->src_kind[s] : 0;
            double f0 = c->src_f0 ? c->src_f0[s] : 1.0e9;
            double amp = c->src_amp ? c->src_amp[s] : 1.0;
            double eps = c->eps, div = 1.0;
            int comp = c->src_comp[s];
            if (nmat) {
                int ci = q[0], cj = q[1], ck = q[2];
                if (comp == 0) { ci = ci < nx ? ci : nx - 1; cj -= 1; ck -= 1; }
                else if (comp == 1) { ci -= 1; cj = cj < ny ? cj : ny - 1; ck -= 1; }
                else { ci -= 1; cj -= 1; ck = ck < nz ? ck : nz - 1; }
                int m = CELL(ci, cj, ck);
                eps = c->mat_eps[m]; div = cs[m];
            }
            double v = orc_fdtd_source(kind, f0, t, c->h) * amp * dt / eps;
            if (div != 1.0) v /= div;
            if (comp == 0) Ex[EX(q[0], q[1], q[2])] -= v;
            else if (comp == 1) Ey[EY(q[0], q[1], q[2])] -= v;
            else Ez[EZ(q[0], q[1], q[2])] -= v;
        }
        /* ---- receivers (fdtd_simulation.cpp:261-303) ---- */
        if (traces && step % tf == 0) {
            const int *q = c->obs_ijk;
            for (int o = 0; o < c->nobs; ++o) {
                double *out = traces + ((size_t)o * nsamp + step / tf) * 3;
                for (int comp = 0; comp < 3; ++comp) {
                    int n = c->obs_n[3 * o + comp];
                    for (int r = 0; r < n; ++r, q += 3) {
                        if (comp == 0) out[0] += Ex[EX(q[0], q[1], q[2])];
                        else if (comp == 1) out[1] += Ey[EY(q[0], q[1], q[2])];
                        else out[2] += Ez[EZ(q[0], q[1], q[2])];
                    }
                    out[comp] /= (double)n;
                }
            }
        }
        t += dt;
    }
    if (L > 0) {
        for (int d = 0; d < 3; ++d) {
            free(pe[d].b); free(pe[d].a); free(pe[d].kinv); free(pe[d].on);
            free(ph[d].b); free(ph[d].a); free(ph[d].kinv); free(ph[d].on);
        }
        for (int q = 0; q < 3; ++q)
            for (int r = 0; r < 2; ++r) { free(psiE[q][r]); free(psiH[q][r]); }
    }
    free(ca); free(cb); free(cs);
    return 0;
}
