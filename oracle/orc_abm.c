/* orc_abm.c — FP64 CPU restatement of the reference Adams-Bashforth-Moulton
 * hexahedral edge-element solver (E and H both on primal edges, order 1).
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY (see ems_oracle.h).
 *
 * Restates fem_abm/fem_simulation.cpp:
 *   32-43     source function (Gaussian derivative, f0 = 1 GHz, dl = 1 mm)
 *   98-122    connectivity in the cyclic local order: x-edges (y,z), y-edges
 *             (z,x), z-edges (x,y), first coordinate fastest
 *   143-246   element matrix K = A + 0.05 Abar: A has, on the four rows of a
 *             component, one half of the element-averaged discrete curl of
 *             that component; Abar is the order-1 curl-curl matrix (the
 *             fem_v2 lamped1.csv data, permuted to the cyclic order)
 *   278-833   one step: AB2 predictors E* = E^n + K^T (3H^n - H^{n-1}) dt/(8 eps h)
 *             and H* = H^n - K (3E^n - E^{n-1}) dt/(8 mu h), AM3 correctors with
 *             (5X* + 8X^n - X^{n-1}) dt/48, point and Hertz-dipole sources
 *   835-943   PEC: tangential E and the edge-normal H next to each face
 *   945-1017  run loop: sample E^{n+1} every tf steps (step counted from 1)
 * Elements are visited in k-j-i order and every accumulation keeps the
 * reference's order, so results equal the serial reference bit for bit.
 */
#include "ems_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define SF 0.05   /* stabilisation factor, fem_abm/fem_simulation.cpp:29 */

static double abm_source(double t, double h)
{
    const double f0 = 1.0e9;
    return -4.0 * M_PI * M_PI * f0 * f0 * (t - 1.0 / f0) *
           exp(-2.0 * M_PI * M_PI * f0 * f0 * (t - 1.0 / f0) * (t - 1.0 / f0)) / h / h / h * 0.001;
}

/* Element matrix of the ABM solver from its definition.  lamped1 is the
 * order-1 curl-curl matrix in the x-fastest local order of kmat/lamped1.csv. */
void orc_abm_kmat(const double *lamped1, double *K)
{
    /* element-averaged curl (times 1/2) in the cyclic order */
    static const double curl_x[12] = {0, 0, 0, 0, 0.5, -0.5, 0.5, -0.5, -0.5, -0.5, 0.5, 0.5};
    static const double curl_y[12] = {-0.5, -0.5, 0.5, 0.5, 0, 0, 0, 0, 0.5, -0.5, 0.5, -0.5};
    static const double curl_z[12] = {0.5, -0.5, 0.5, -0.5, -0.5, -0.5, 0.5, 0.5, 0, 0, 0, 0};
    int perm[12];
    for (int q = 0; q < 4; ++q) { perm[q] = q; perm[8 + q] = 8 + q; perm[4 + q] = 4 + (q / 2) + 2 * (q % 2); }
    for (int r = 0; r < 12; ++r)
        for (int c = 0; c < 12; ++c) {
            const double *cr = r < 4 ? curl_x : r < 8 ? curl_y : curl_z;
            double a = cr[c];
            double abar = lamped1[perm[r] * 12 + perm[c]];
            K[r * 12 + c] = a + SF * abar;
        }
}

typedef struct {
    int gx, gy, gz;
    size_t n[3];
    int *conn[3];
} abm_mesh;

static void abm_build(abm_mesh *m, int gx, int gy, int gz)
{
    m->gx = gx; m->gy = gy; m->gz = gz;
    m->n[0] = (size_t)gx * (gy + 1) * (gz + 1);
    m->n[1] = (size_t)(gx + 1) * gy * (gz + 1);
    m->n[2] = (size_t)(gx + 1) * (gy + 1) * gz;
    size_t ne = (size_t)gx * gy * gz;
    for (int c = 0; c < 3; ++c) m->conn[c] = malloc(sizeof(int) * 4 * ne);
    for (int k = 0; k < gz; ++k)
        for (int j = 0; j < gy; ++j)
            for (int i = 0; i < gx; ++i) {
                size_t b = 4 * ((size_t)i + (size_t)j * gx + (size_t)k * gx * gy);
                for (int q = 0; q < 4; ++q) {
                    int a0 = q & 1, a1 = q >> 1;
                    /* x-edge (i, j+a0, k+a1); y-edge (i+a1, j, k+a0); z-edge (i+a0, j+a1, k) */
                    m->conn[0][b + q] = i + (j + a0) * gx + (k + a1) * gx * (gy + 1);
                    m->conn[1][b + q] = (i + a1) + j * (gx + 1) + (k + a0) * (gx + 1) * gy;
                    m->conn[2][b + q] = (i + a0) + (j + a1) * (gx + 1) + k * (gx + 1) * (gy + 1);
                }
            }
}

/* out += K^T in (transpose) or K in, per element (fem_abm 321-366, 510-555) */
static void abm_sweep(const abm_mesh *m, const double *K, double *in[3], double *out[3], int transpose)
{
    int gx = m->gx, gy = m->gy, gz = m->gz;
    for (int k = 0; k < gz; ++k)
        for (int j = 0; j < gy; ++j)
            for (int i = 0; i < gx; ++i) {
                size_t b = 4 * ((size_t)i + (size_t)j * gx + (size_t)k * gx * gy);
                double loc[12];
                for (int c = 0; c < 3; ++c)
                    for (int q = 0; q < 4; ++q) loc[4 * c + q] = in[c][m->conn[c][b + q]];
                for (int l = 0; l < 4; ++l) {
                    double t0 = 0, t1 = 0, t2 = 0;
                    for (int mm = 0; mm < 12; ++mm) {
                        if (transpose) {
                            t0 += K[mm * 12 + l] * loc[mm];
                            t1 += K[mm * 12 + l + 4] * loc[mm];
                            t2 += K[mm * 12 + l + 8] * loc[mm];
                        } else {
                            t0 += K[l * 12 + mm] * loc[mm];
                            t1 += K[(l + 4) * 12 + mm] * loc[mm];
                            t2 += K[(l + 8) * 12 + mm] * loc[mm];
                        }
                    }
                    out[0][m->conn[0][b + l]] += t0;
                    out[1][m->conn[1][b + l]] += t1;
                    out[2][m->conn[2][b + l]] += t2;
                }
            }
}

/* Hertz dipole along x over the 2x2 cells around (i,j,k)
 * (fem_abm/fem_simulation.cpp:407-481 and 758-833). */
static void abm_dipole(const abm_mesh *m, const int *p, double temp, double *E2[3])
{
    int gx = m->gx, gy = m->gy;
    size_t c0 = 4 * ((size_t)p[0] + (size_t)p[1] * gx + (size_t)p[2] * gx * gy);
    size_t c1 = 4 * ((size_t)p[0] + (size_t)(p[1] + 1) * gx + (size_t)p[2] * gx * gy);
    size_t c2 = 4 * ((size_t)p[0] + (size_t)p[1] * gx + (size_t)(p[2] + 1) * gx * gy);
    size_t c3 = 4 * ((size_t)p[0] + (size_t)(p[1] + 1) * gx + (size_t)(p[2] + 1) * gx * gy);
    int *X = m->conn[0], *Y = m->conn[1], *Z = m->conn[2];
    E2[0][X[c0]] += 1.0 / 8.0 * temp;
    E2[0][X[c0 + 1]] += 3.0 / 4.0 * temp;
    E2[0][X[c0 + 2]] += 3.0 / 4.0 * temp;
    E2[0][X[c0 + 3]] += 9.0 / 2.0 * temp;
    E2[0][X[c1 + 1]] += 1.0 / 8.0 * temp;
    E2[0][X[c1 + 3]] += 3.0 / 4.0 * temp;
    E2[0][X[c2 + 2]] += 1.0 / 8.0 * temp;
    E2[0][X[c2 + 3]] += 3.0 / 4.0 * temp;
    E2[0][X[c3 + 3]] += 1.0 / 8.0 * temp;
    E2[1][Y[c0]] += SF / 2.0 * temp;
    E2[1][Y[c0 + 2]] += SF / 2.0 * temp;
    E2[1][Y[c1]] += SF / 2.0 * temp;
    E2[1][Y[c1 + 2]] += SF / 2.0 * temp;
    E2[1][Y[c2 + 1]] -= SF / 2.0 * temp;
    E2[1][Y[c2 + 3]] -= SF / 2.0 * temp;
    E2[1][Y[c3 + 1]] -= SF / 2.0 * temp;
    E2[1][Y[c3 + 3]] -= SF / 2.0 * temp;
    E2[2][Z[c0]] -= SF / 2.0 * temp;
    E2[2][Z[c0 + 1]] -= SF / 2.0 * temp;
    E2[2][Z[c1 + 2]] += SF / 2.0 * temp;
    E2[2][Z[c1 + 3]] += SF / 2.0 * temp;
    E2[2][Z[c2]] -= SF / 2.0 * temp;
    E2[2][Z[c2 + 1]] -= SF / 2.0 * temp;
    E2[2][Z[c3 + 2]] += SF / 2.0 * temp;
    E2[2][Z[c3 + 3]] += SF / 2.0 * temp;
}

/* fem_abm/fem_simulation.cpp:835-943 */
static void abm_pec(const abm_mesh *m, double *E2[3], double *H2[3])
{
    int gx = m->gx, gy = m->gy, gz = m->gz;
    for (int k = 0; k <= gz; ++k)
        for (int j = 0; j <= gy; ++j)
            for (int i = 0; i < gx; ++i)
                if (j == 0 || j == gy || k == 0 || k == gz) E2[0][i + j * gx + (size_t)k * gx * (gy + 1)] = 0.0;
    for (int k = 0; k <= gz; ++k)
        for (int j = 0; j < gy; ++j)
            for (int i = 0; i <= gx; ++i)
                if (i == 0 || i == gx || k == 0 || k == gz) E2[1][i + j * (gx + 1) + (size_t)k * (gx + 1) * gy] = 0.0;
    for (int k = 0; k < gz; ++k)
        for (int j = 0; j <= gy; ++j)
            for (int i = 0; i <= gx; ++i)
                if (i == 0 || i == gx || j == 0 || j == gy) E2[2][i + j * (gx + 1) + (size_t)k * (gx + 1) * (gy + 1)] = 0.0;
    for (int k = 0; k <= gz; ++k)
        for (int j = 0; j <= gy; ++j) {
            H2[0][j * gx + (size_t)k * gx * (gy + 1)] = 0.0;
            H2[0][j * gx + (size_t)k * gx * (gy + 1) + gx - 1] = 0.0;
        }
    for (int k = 0; k <= gz; ++k)
        for (int i = 0; i <= gx; ++i) {
            H2[1][i + (size_t)k * (gx + 1) * gy] = 0.0;
            H2[1][i + (size_t)k * (gx + 1) * gy + (size_t)(gx + 1) * (gy - 1)] = 0.0;
        }
    for (int i = 0; i <= gx; ++i)
        for (int j = 0; j <= gy; ++j) {
            H2[2][i + j * (gx + 1)] = 0.0;
            H2[2][i + j * (gx + 1) + (size_t)(gx + 1) * (gy + 1) * (gz - 1)] = 0.0;
        }
}

int orc_abm_run(const orc_abm_case *c, int nsteps, double *E[3], double *H[3], double *traces)
{
    abm_mesh m;
    abm_build(&m, c->gx, c->gy, c->gz);
    double K[144];
    orc_abm_kmat(c->lamped1, K);
    const double dt = c->dt, h = c->h, eps = c->eps, mu = c->mu;
    const int tf = c->time_frequency;
    const int nsamp = nsteps / tf + 1;
    if (traces) memset(traces, 0, sizeof(double) * (size_t)c->nobs * nsamp * 3);
    int r0 = 0, r1 = 1, r2 = 2;
    double t = 0.0;
    for (int step = 1; step < nsteps + 1; ++step) {
        double *E0[3], *E1[3], *E2[3], *Es[3], *H0[3], *H1[3], *H2[3], *Hs[3];
        for (int q = 0; q < 3; ++q) {
            size_t n = m.n[q];
            E0[q] = E[q] + r0 * n; E1[q] = E[q] + r1 * n; E2[q] = E[q] + r2 * n; Es[q] = E[q] + 3 * n;
            H0[q] = H[q] + r0 * n; H1[q] = H[q] + r1 * n; H2[q] = H[q] + r2 * n; Hs[q] = H[q] + 3 * n;
        }
        /* AB2 predictor for E (fem_abm 295-405) */
        for (int q = 0; q < 3; ++q)
            for (size_t i = 0; i < m.n[q]; ++i) {
                Es[q][i] = (3.0 * H1[q][i] - H0[q][i]) * dt / 8.0 / eps / h;
                E2[q][i] = 0.0;
            }
        abm_sweep(&m, K, Es, E2, 1);
        for (int q = 0; q < 3; ++q)
            for (size_t i = 0; i < m.n[q]; ++i) E2[q][i] += E1[q][i];
        for (int s = 0; s < c->nsrc; ++s) {
            const int *p = c->src_ijk + 3 * s;
            int q = c->src_comp[s];
            size_t idx = q == 0 ? (size_t)p[0] + (size_t)p[1] * m.gx + (size_t)p[2] * m.gx * (m.gy + 1)
                       : q == 1 ? (size_t)p[0] + (size_t)p[1] * (m.gx + 1) + (size_t)p[2] * (m.gx + 1) * m.gy
                                : (size_t)p[0] + (size_t)p[1] * (m.gx + 1) + (size_t)p[2] * (m.gx + 1) * (m.gy + 1);
            E2[q][idx] -= (3.0 * abm_source(t, h) - abm_source(t - dt, h)) * dt / 2.0 / eps / h / h / h;
        }
        for (int s = 0; s < c->ndip; ++s) {
            double temp = -(3.0 * abm_source(t, h) - abm_source(t - dt, h)) * dt / 16.0 / eps;
            abm_dipole(&m, c->dip_ijk + 3 * s, temp, E2);
        }
        /* AB2 predictor for H (484-571) */
        for (int q = 0; q < 3; ++q)
            for (size_t i = 0; i < m.n[q]; ++i) {
                Hs[q][i] = -(3.0 * E1[q][i] - E0[q][i]) * dt / 8.0 / mu / h;
                H2[q][i] = 0.0;
            }
        abm_sweep(&m, K, Hs, H2, 0);
        for (int q = 0; q < 3; ++q)
            for (size_t i = 0; i < m.n[q]; ++i) H2[q][i] += H1[q][i];
        /* AM3 corrector (573-833) */
        for (int q = 0; q < 3; ++q)
            for (size_t i = 0; i < m.n[q]; ++i) {
                Es[q][i] = (5.0 * H2[q][i] + 8.0 * H1[q][i] - H0[q][i]) * dt / 48.0 / eps / h;
                Hs[q][i] = -(5.0 * E2[q][i] + 8.0 * E1[q][i] - E0[q][i]) * dt / 48.0 / mu / h;
                E2[q][i] = 0.0;
                H2[q][i] = 0.0;
            }
        abm_sweep(&m, K, Es, E2, 1);
        abm_sweep(&m, K, Hs, H2, 0);
        for (int q = 0; q < 3; ++q)
            for (size_t i = 0; i < m.n[q]; ++i) {
                E2[q][i] += E1[q][i];
                H2[q][i] += H1[q][i];
            }
        for (int s = 0; s < c->nsrc; ++s) {
            const int *p = c->src_ijk + 3 * s;
            int q = c->src_comp[s];
            size_t idx = q == 0 ? (size_t)p[0] + (size_t)p[1] * m.gx + (size_t)p[2] * m.gx * (m.gy + 1)
                       : q == 1 ? (size_t)p[0] + (size_t)p[1] * (m.gx + 1) + (size_t)p[2] * (m.gx + 1) * m.gy
                                : (size_t)p[0] + (size_t)p[1] * (m.gx + 1) + (size_t)p[2] * (m.gx + 1) * (m.gy + 1);
            E2[q][idx] -= (5.0 * abm_source(t + dt, h) + 8.0 * abm_source(t, h) - abm_source(t - dt, h)) * dt / 12.0 / eps / h / h / h;
        }
        for (int s = 0; s < c->ndip; ++s) {
            double temp = -(5.0 * abm_source(t + dt, h) + 8.0 * abm_source(t, h) - abm_source(t - dt, h)) * dt / 96.0 / eps;
            abm_dipole(&m, c->dip_ijk + 3 * s, temp, E2);
        }
        abm_pec(&m, E2, H2);
        /* receivers (945-1013): lists of edges per component, averaged */
        if (traces && step % tf == 0) {
            const int *q = c->obs_ijk;
            for (int o = 0; o < c->nobs; ++o) {
                double *out = traces + ((size_t)o * nsamp + step / tf) * 3;
                for (int comp = 0; comp < 3; ++comp) {
                    int n = c->obs_n[3 * o + comp];
                    for (int r = 0; r < n; ++r, q += 3) {
                        size_t idx = comp == 0 ? (size_t)q[0] + (size_t)q[1] * m.gx + (size_t)q[2] * m.gx * (m.gy + 1)
                                   : comp == 1 ? (size_t)q[0] + (size_t)q[1] * (m.gx + 1) + (size_t)q[2] * (m.gx + 1) * m.gy
                                               : (size_t)q[0] + (size_t)q[1] * (m.gx + 1) + (size_t)q[2] * (m.gx + 1) * (m.gy + 1);
                        out[comp] += E2[comp][idx];
                    }
                    out[comp] /= (double)n;
                }
            }
        }
        t += dt;
        r0 = (r0 + 1) % 3; r1 = (r1 + 1) % 3; r2 = (r2 + 1) % 3;
    }
    for (int q = 0; q < 3; ++q) free(m.conn[q]);
    return 0;
}
