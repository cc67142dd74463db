/* orc_hexfem.c — FP64 CPU restatement of the fem_v2-family hexahedral
 * edge-element time loops (leapfrog, 2nd- and 4th-order symplectic).
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY (see ems_oracle.h).
 *
 * Restates, for one subdomain holding the whole grid:
 *   fem_v2/fem_simulation.cpp
 *     369-423  element -> fine-grid edge connectivity (x-fastest local order)
 *     424-455  outer-element list (processed before the inner elements)
 *     458-490  element matrix scaling for leapfrog
 *     560-655  leapfrog step: F = -K E1, exchange, F += 2E1 - E0, source
 *     1007-1112 exchange unpack, which on one rank zeroes the tangential
 *              boundary entries of the accumulator level
 *     1115-1247 PEC: tangential E on the six faces set to zero
 *     1249-1317 run loop, receivers (4 x-edges, 4 y-edges, 1 z-edge), ring
 *   fem_v2/fem_kernels.hpp:13-175  per element: gather, dense row x vector,
 *              scatter (-= for leapfrog, += for the symplectic variants)
 *   symplectic_2/fem_simulation.cpp
 *     473      K = 4/((h o)^2 mu eps) Kcsv
 *     557-672  drift U += dt/2 P/m, F = K U + src(t+off+dt/2), kick P -= dt F,
 *              drift, PEC on U and P; m = 8/o^3
 *     1278-1350 run loop sampling U before each step
 *   symplectic_4/fem_simulation.cpp:1280-1281,1347-1350  triple jump.
 * Elements are visited in the reference's order (outer list, then inner
 * elements k-j-i), so the accumulation order per DOF matches the serial
 * reference and results are bit-identical to it.
 */
#include "ems_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

size_t orc_hexfem_ncomp(int gx, int gy, int gz, int comp)
{
    if (comp == 0) return (size_t)gx * (gy + 1) * (gz + 1);
    if (comp == 1) return (size_t)(gx + 1) * gy * (gz + 1);
    return (size_t)(gx + 1) * (gy + 1) * gz;
}

/* fem_v2/fem_simulation.cpp:77-87 — second derivative of a Gaussian, f = 1 GHz */
static double femv2_source(double t)
{
    const double freq = 1.0e9;
    const double chi = 1.0 / freq;
    double delay = t - chi;
    double zeta = 2.0 * M_PI * M_PI * freq * freq;
    return 2.0 * zeta * (2.0 * zeta * delay * delay - 1.0) * exp(0.0 - zeta * delay * delay) * 0.001;
}

typedef struct {
    int o, gx, gy, gz, ex, ey, ez, dof, total;
    int *cx, *cy, *cz;     /* connectivity, dof ints per element each */
    int *order;            /* element visiting order */
    int nelem, nouter;
    double *K;             /* scaled element matrix */
} hexmesh;

static void build_mesh(hexmesh *m, const orc_hexfem_case *c)
{
    int o = c->order, gx = c->gx, gy = c->gy, gz = c->gz;
    m->o = o; m->gx = gx; m->gy = gy; m->gz = gz;
    m->ex = gx / o; m->ey = gy / o; m->ez = gz / o;
    m->dof = o * (o + 1) * (o + 1);
    m->total = 3 * m->dof;
    size_t ne = (size_t)m->ex * m->ey * m->ez;
    m->cx = malloc(sizeof(int) * ne * m->dof);
    m->cy = malloc(sizeof(int) * ne * m->dof);
    m->cz = malloc(sizeof(int) * ne * m->dof);
    for (int k = 0; k < m->ez; ++k)
        for (int j = 0; j < m->ey; ++j)
            for (int i = 0; i < m->ex; ++i) {
                size_t base = ((size_t)i + (size_t)j * m->ex + (size_t)k * m->ex * m->ey) * m->dof;
                int fx = o * i, fy = o * j, fz = o * k;
                for (int n = 0; n < o + 1; ++n)
                    for (int mm = 0; mm < o + 1; ++mm)
                        for (int l = 0; l < o; ++l)
                            m->cx[base + l + mm * o + n * o * (o + 1)] =
                                (fx + l) + (fy + mm) * gx + (fz + n) * gx * (gy + 1);
                for (int n = 0; n < o + 1; ++n)
                    for (int mm = 0; mm < o; ++mm)
                        for (int l = 0; l < o + 1; ++l)
                            m->cy[base + l + mm * (o + 1) + n * o * (o + 1)] =
                                (fx + l) + (fy + mm) * (gx + 1) + (fz + n) * (gx + 1) * gy;
                for (int n = 0; n < o; ++n)
                    for (int mm = 0; mm < o + 1; ++mm)
                        for (int l = 0; l < o + 1; ++l)
                            m->cz[base + l + mm * (o + 1) + n * (o + 1) * (o + 1)] =
                                (fx + l) + (fy + mm) * (gx + 1) + (fz + n) * (gx + 1) * (gy + 1);
            }
    /* visiting order: outer list (fem_simulation.cpp:424-455) then inner */
    int EX = m->ex, EY = m->ey, EZ = m->ez;
    m->order = malloc(sizeof(int) * (ne + 8));
    int q = 0;
    for (int j = 0; j < EY; ++j)
        for (int i = 0; i < EX; ++i) m->order[q + i + j * EX] = i + j * EX;
    q += EX * EY;
    for (int j = 0; j < EY; ++j)
        for (int i = 0; i < EX; ++i) m->order[q + i + j * EX] = EX * EY * (EZ - 1) + i + j * EX;
    q += EX * EY;
    for (int k = 1; k < EZ - 1; ++k)
        for (int j = 0; j < EY; ++j) {
            m->order[q + j + (k - 1) * EY] = j * EX + k * EX * EY;
            m->order[q + EY * (EZ - 2) + j + (k - 1) * EY] = (EX - 1) + j * EX + k * EX * EY;
        }
    q += 2 * EY * (EZ - 2);
    for (int i = 1; i < EX - 1; ++i)
        for (int k = 1; k < EZ - 1; ++k) {
            m->order[q + k - 1 + (i - 1) * (EZ - 2)] = i + k * EX * EY;
            m->order[q + (EZ - 2) * (EX - 2) + k - 1 + (i - 1) * (EZ - 2)] = EX * (EY - 1) + i + k * EX * EY;
        }
    q += 2 * (EZ - 2) * (EX - 2);
    m->nouter = q;
    for (int k = 1; k < EZ - 1; ++k)
        for (int j = 1; j < EY - 1; ++j)
            for (int i = 1; i < EX - 1; ++i) m->order[q++] = i + j * EX + k * EX * EY;
    m->nelem = q;
}

/* fem_kernels.hpp:30-85: per element y_local = K x_local, scattered into F */
static void apply_K(const hexmesh *m, const double *in[3], double *out[3], double sign, int q0, int q1)
{
    int D = m->dof, T = m->total;
    double *loc = malloc(sizeof(double) * T);
    for (int q = q0; q < q1; ++q) {
        size_t base = (size_t)m->order[q] * D;
        for (int l = 0; l < D; ++l) {
            loc[l] = in[0][m->cx[base + l]];
            loc[l + D] = in[1][m->cy[base + l]];
            loc[l + 2 * D] = in[2][m->cz[base + l]];
        }
        for (int l = 0; l < T; ++l) {
            double temp = 0;
            const double *row = m->K + (size_t)l * T;
            for (int mm = 0; mm < T; ++mm) temp += row[mm] * loc[mm];
            int comp = l / D;
            const int *conn = comp == 0 ? m->cx : comp == 1 ? m->cy : m->cz;
            int n = conn[base + l - comp * D];
            if (sign < 0) out[comp][n] -= temp; else out[comp][n] += temp;
        }
    }
    free(loc);
}

/* Zero the tangential DOFs on the six faces of one level: the PEC of
 * fem_simulation.cpp:1115-1247; the single-rank exchange unpack zeroes the
 * same set. */
static void pec(const hexmesh *m, double *lv[3])
{
    int gx = m->gx, gy = m->gy, gz = m->gz;
    for (int k = 0; k < gz + 1; ++k)
        for (int j = 0; j < gy + 1; ++j)
            for (int i = 0; i < gx; ++i)
                if (j == 0 || j == gy || k == 0 || k == gz) lv[0][i + j * gx + (size_t)k * gx * (gy + 1)] = 0.0;
    for (int k = 0; k < gz + 1; ++k)
        for (int j = 0; j < gy; ++j)
            for (int i = 0; i < gx + 1; ++i)
                if (i == 0 || i == gx || k == 0 || k == gz) lv[1][i + j * (gx + 1) + (size_t)k * (gx + 1) * gy] = 0.0;
    for (int k = 0; k < gz; ++k)
        for (int j = 0; j < gy + 1; ++j)
            for (int i = 0; i < gx + 1; ++i)
                if (i == 0 || i == gx || j == 0 || j == gy) lv[2][i + j * (gx + 1) + (size_t)k * (gx + 1) * (gy + 1)] = 0.0;
}

static int src_index(const hexmesh *m, int comp, const int *p)
{
    int gx = m->gx, gy = m->gy;
    if (comp == 0) return p[0] + p[1] * gx + p[2] * gx * (gy + 1);
    if (comp == 1) return p[0] + p[1] * (gx + 1) + p[2] * (gx + 1) * gy;
    return p[0] + p[1] * (gx + 1) + p[2] * (gx + 1) * (gy + 1);
}

/* fem_simulation.cpp:1273-1312: Ex = mean of x-edges (i-1,j,k),(i,j,k),
 * (i-1,j,k+1),(i,j,k+1); Ey likewise in y; Ez = the z-edge (i,j,k). */
static void sample(const hexmesh *m, const orc_hexfem_case *c, double *lv[3], double t, double *traces, int nsamp, int s)
{
    int gx = m->gx, gy = m->gy;
    for (int o = 0; o < c->nobs; ++o) {
        const int *p = c->obs_ijk + 3 * o;
        int ox = p[0] + p[1] * gx + p[2] * gx * (gy + 1);
        int oy = p[0] + p[1] * (gx + 1) + p[2] * (gx + 1) * gy;
        int oz = p[0] + p[1] * (gx + 1) + p[2] * (gx + 1) * (gy + 1);
        double *out = traces + ((size_t)o * nsamp + s) * 4;
        out[0] = t;
        out[1] = (lv[0][ox - 1] + lv[0][ox] + lv[0][ox + gx * (gy + 1) - 1] + lv[0][ox + gx * (gy + 1)]) / 4.0;
        out[2] = (lv[1][oy - (gx + 1)] + lv[1][oy] + lv[1][oy + (gx + 1) * (gy - 1)] + lv[1][oy + (gx + 1) * gy]) / 4.0;
        out[3] = lv[2][oz];
    }
}

/* symplectic_2/fem_simulation.cpp:557-672 */
static void symp_substep(const hexmesh *m, const orc_hexfem_case *c, double *U[3], double *P[3], double *F[3],
                         size_t nc[3], double deltat, double t)
{
    int o = m->o;
    for (int q = 0; q < 3; ++q) memset(F[q], 0, sizeof(double) * nc[q]);
    for (int q = 0; q < 3; ++q)
        for (size_t i = 0; i < nc[q]; ++i) U[q][i] += 0.5 * deltat * P[q][i] / (8.0 / o / o / o);
    /* outer elements, source (symplectic_2 615-621), then inner elements */
    apply_K(m, (const double **)U, F, +1.0, 0, m->nouter);
    for (int s = 0; s < c->nsrc; ++s) {
        double temp = femv2_source(t + 0.5 * deltat) * 8.0 / c->eps / (c->h * o) / (c->h * o) / (c->h * o);
        F[c->src_comp[s]][src_index(m, c->src_comp[s], c->src_ijk + 3 * s)] += temp;
    }
    apply_K(m, (const double **)U, F, +1.0, m->nouter, m->nelem);
    pec(m, F);
    for (int q = 0; q < 3; ++q)
        for (size_t i = 0; i < nc[q]; ++i) {
            P[q][i] -= deltat * F[q][i];
            U[q][i] += 0.5 * deltat * P[q][i] / (8.0 / o / o / o);
        }
    pec(m, U);
    pec(m, P);
}

int orc_hexfem_run(const orc_hexfem_case *c, int nsteps, double *ef[3], double *traces)
{
    hexmesh m;
    build_mesh(&m, c);
    int o = c->order, T = m.total;
    size_t nc[3];
    for (int q = 0; q < 3; ++q) nc[q] = orc_hexfem_ncomp(c->gx, c->gy, c->gz, q);
    /* element matrix scaling (fem_v2 458-490 / symplectic_2 473) */
    double scale;
    if (c->integrator == ORC_LEAPFROG)
        scale = 4.0 * c->dt * c->dt / (c->h * o) / (c->h * o) / c->mu / c->eps / (8.0 / o / o / o);
    else
        scale = 4.0 / (c->h * o) / (c->h * o) / c->mu / c->eps;
    m.K = malloc(sizeof(double) * T * T);
    for (int i = 0; i < T * T; ++i) m.K[i] = scale * c->kmat[i];

    int tf = c->time_frequency;
    int nsamp = (nsteps - 1) / tf + 1;
    double t = 0.0;
    if (c->integrator == ORC_LEAPFROG) {
        int l0 = 0, l1 = 1, l2 = 2;
        for (int step = 0; step < nsteps; ++step) {
            double *E0[3], *E1[3], *E2[3];
            for (int q = 0; q < 3; ++q) {
                E0[q] = ef[q] + l0 * nc[q]; E1[q] = ef[q] + l1 * nc[q]; E2[q] = ef[q] + l2 * nc[q];
                memset(E2[q], 0, sizeof(double) * nc[q]);
            }
            apply_K(&m, (const double **)E1, E2, -1.0, 0, m.nelem);
            pec(&m, E2);
            for (int q = 0; q < 3; ++q)
                for (size_t i = 0; i < nc[q]; ++i) E2[q][i] += 2.0 * E1[q][i] - E0[q][i];
            for (int s = 0; s < c->nsrc; ++s) {
                double temp = femv2_source(t) * c->dt * c->dt / c->eps / c->h / c->h / c->h;
                E2[c->src_comp[s]][src_index(&m, c->src_comp[s], c->src_ijk + 3 * s)] -= temp;
            }
            pec(&m, E2);
            if (traces && step % tf == 0) sample(&m, c, E1, t, traces, nsamp, step / tf);
            t += c->dt;
            l0 = (l0 + 1) % 3; l1 = (l1 + 1) % 3; l2 = (l2 + 1) % 3;
        }
    } else {
        double *U[3], *P[3], *F[3];
        for (int q = 0; q < 3; ++q) { U[q] = ef[q]; P[q] = ef[q] + nc[q]; F[q] = ef[q] + 2 * nc[q]; }
        double x1 = 1.0 / (2.0 - pow(2.0, 1.0 / 3.0));
        double x2 = 1.0 - 2.0 * x1;
        for (int step = 0; step < nsteps; ++step) {
            if (traces && step % tf == 0) sample(&m, c, U, t, traces, nsamp, step / tf);
            if (c->integrator == ORC_SYMP2) {
                symp_substep(&m, c, U, P, F, nc, c->dt, t + 0.0);
            } else {
                symp_substep(&m, c, U, P, F, nc, x1 * c->dt, t + 0.0);
                symp_substep(&m, c, U, P, F, nc, x2 * c->dt, t + x1 * c->dt);
                symp_substep(&m, c, U, P, F, nc, x1 * c->dt, t + (x1 + x2) * c->dt);
            }
            t += c->dt;
        }
    }
    free(m.cx); free(m.cy); free(m.cz); free(m.order); free(m.K);
    return 0;
}
