/* orc_femstab.c — FP64 CPU restatement of the reference's stabilised
 * order-1 hexahedral edge-element solver (the fem/ directory).
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY (see ems_oracle.h).
 *
 * Restates fem/fem_simulation.cpp:
 *   28-38     source function (f0 = 1 GHz, times mu / h^3, dl = 1 mm)
 *   61-123    connectivity in the cyclic local order: x-edges (y,z), y-edges
 *             (z,x), z-edges (x,y), first coordinate fastest
 *   125-434   element matrix K = dt^2 / (2 mu eps h^2) Ct Bt^-1 At with
 *             At = A + s Abar, Bt = B + s Bbar, Ct = C + s Cbar, in the
 *             conventional basis or the orthogonal (OFEM) one
 *   466-634   update: E^{n+1} = -K E^n scattered per element in k-j-i order,
 *             then + (2 E^n - E^{n-1}), then point sources
 *   636-740   x-directed Hertz dipole (conventional: 9 x-edges and the
 *             stabilisation terms on 8 y- and 8 z-edges; OFEM: one x-edge)
 *   743-833   PEC: tangential E zeroed on the faces
 *   836-903   run loop: sample E^{n+1} every tf steps (step counted from 1)
 * Elements are visited in k-j-i order and every accumulation keeps the
 * reference's order, so the loop equals the serial reference bit for bit.
 *
 * The element matrices are formed from their structure, not typed in:
 *   A     rows of one component = one half of the element-averaged discrete
 *         curl of that component (the same rows as fem_abm's)
 *   B     per component the 4x4 tensor-product mass (8/9) 2^-d(a,b), d the
 *         number of transverse axes on which local edges a and b differ
 *   Bbar  = C = A^T
 *   Abar  = Cbar^T, the stabilisation: in the modal basis of each component
 *         (constant, linear along the first and the second transverse axis,
 *         bilinear; the 4x4 matrix H below) it couples every non-constant
 *         mode with the matching mode of the other components (rule R)
 *   OFEM  the same operators in the modal basis: A_o = T A, B_o = T B T^T,
 *         Bbar_o = T Bbar T^T, C_o = C T^T, Abar_o = R T, T = diag(H, H, H);
 *         the conventional Abar = T^T W R T / 16 with mode weights
 *         W = (0, 4, 4, 8/3)
 * Every entry is an integer or a correctly rounded k/3 or k/9, the values the
 * reference's literal tables hold.  B^-1 is formed by Gauss-Jordan
 * elimination with partial pivoting and the products by plain row-column
 * sums in index order (the arithmetic of the dense-matrix stand-in the
 * reference is compiled with here; the reference names Eigen, absent from
 * this machine).
 */
#include "ems_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

static const double kCurl[3][12] = {
    {0, 0, 0, 0, 0.5, -0.5, 0.5, -0.5, -0.5, -0.5, 0.5, 0.5},
    {-0.5, -0.5, 0.5, 0.5, 0, 0, 0, 0, 0.5, -0.5, 0.5, -0.5},
    {0.5, -0.5, 0.5, -0.5, -0.5, -0.5, 0.5, 0.5, 0, 0, 0, 0}};
/* modes of the four cyclic edges of a component: constant, sign by the first
 * transverse offset, sign by the second, their product */
static const double kModes[4][4] = {{1, 1, 1, 1}, {-1, 1, -1, 1}, {-1, -1, 1, 1}, {1, -1, -1, 1}};

static void mat_mul(const double *a, const double *b, double *c)   /* c = a b, 12 x 12 */
{
    double t[144];
    for (int i = 0; i < 12; ++i)
        for (int j = 0; j < 12; ++j) {
            double s = 0.0;
            for (int k = 0; k < 12; ++k) s += a[i * 12 + k] * b[k * 12 + j];
            t[i * 12 + j] = s;
        }
    memcpy(c, t, sizeof(t));
}

static void transpose(const double *a, double *b)
{
    double t[144];
    for (int i = 0; i < 12; ++i)
        for (int j = 0; j < 12; ++j) t[j * 12 + i] = a[i * 12 + j];
    memcpy(b, t, sizeof(t));
}

/* Gauss-Jordan inverse with partial pivoting (the first row of largest
 * magnitude), pivot row scaled, then eliminated from every other row. */
static int gauss_jordan(const double *m, double *inv)
{
    double a[144];
    memcpy(a, m, sizeof(a));
    for (int i = 0; i < 144; ++i) inv[i] = (i / 12 == i % 12) ? 1.0 : 0.0;
    for (int col = 0; col < 12; ++col) {
        int piv = col;
        for (int i = col + 1; i < 12; ++i)
            if (fabs(a[i * 12 + col]) > fabs(a[piv * 12 + col])) piv = i;
        if (a[piv * 12 + col] == 0.0) return -1;
        if (piv != col)
            for (int j = 0; j < 12; ++j) {
                double x = a[piv * 12 + j]; a[piv * 12 + j] = a[col * 12 + j]; a[col * 12 + j] = x;
                x = inv[piv * 12 + j]; inv[piv * 12 + j] = inv[col * 12 + j]; inv[col * 12 + j] = x;
            }
        const double d = a[col * 12 + col];
        for (int j = 0; j < 12; ++j) { a[col * 12 + j] /= d; inv[col * 12 + j] /= d; }
        for (int i = 0; i < 12; ++i) {
            if (i == col) continue;
            const double f = a[i * 12 + col];
            if (f == 0.0) continue;
            for (int j = 0; j < 12; ++j) { a[i * 12 + j] -= f * a[col * 12 + j]; inv[i * 12 + j] -= f * inv[col * 12 + j]; }
        }
    }
    return 0;
}

/* The six 12 x 12 matrices A, Abar, B, Bbar, C, Cbar of one basis. */
void orc_femstab_parts(int use_ofem, double *A, double *Abar, double *B, double *Bbar, double *C, double *Cbar)
{
    static const int ax[3][2] = {{1, 2}, {2, 0}, {0, 1}};   /* transverse axes, cyclic order */
    double T[144] = {0}, R[144] = {0}, Ac[144], B9[144] = {0};
    for (int c = 0; c < 3; ++c)
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) {
                T[(4 * c + a) * 12 + 4 * c + b] = kModes[a][b];
                int d = ((a ^ b) & 1) + ((a ^ b) >> 1);
                B9[(4 * c + a) * 12 + 4 * c + b] = (double)(8 >> d);   /* 9 x the mass */
            }
    for (int c = 0; c < 3; ++c) {
        for (int m = 1; m <= 2; ++m) {
            const int t = ax[c][m - 1];
            R[(4 * c + m) * 12 + 4 * c + m] = 2.0;
            R[(4 * c + m) * 12 + 4 * t + (ax[t][0] == c ? 1 : 2)] = -2.0;
        }
        R[(4 * c + 3) * 12 + 4 * c + 3] = 2.0;
        for (int t = 0; t < 3; ++t)
            if (t != c) R[(4 * c + 3) * 12 + 4 * t + 3] = -1.0;
    }
    for (int r = 0; r < 12; ++r)
        for (int m = 0; m < 12; ++m) Ac[r * 12 + m] = kCurl[r / 4][m];
    double Tt[144], tmp[144];
    transpose(T, Tt);
    if (!use_ofem) {
        memcpy(A, Ac, sizeof(Ac));
        /* 3 Abar = T^T (3 W R) T / 16, integers */
        static const double w3[4] = {0.0, 12.0, 12.0, 8.0};
        for (int r = 0; r < 144; ++r) tmp[r] = w3[(r / 12) % 4] * R[r];
        mat_mul(tmp, T, tmp);
        mat_mul(Tt, tmp, tmp);
        for (int r = 0; r < 144; ++r) Abar[r] = (tmp[r] / 16.0) / 3.0;
        for (int r = 0; r < 144; ++r) B[r] = B9[r] / 9.0;
        transpose(Ac, Bbar);
    } else {
        mat_mul(T, Ac, A);
        mat_mul(R, T, Abar);
        mat_mul(T, B9, tmp);
        mat_mul(tmp, Tt, tmp);
        for (int r = 0; r < 144; ++r) B[r] = tmp[r] / 9.0;
        transpose(Ac, tmp);
        mat_mul(T, tmp, tmp);
        mat_mul(tmp, Tt, Bbar);
    }
    transpose(A, C);
    transpose(Abar, Cbar);
}

int orc_femstab_kmat(double dt, double mu, double eps, double h, double sf, int use_ofem, double *K)
{
    double A[144], Ab[144], B[144], Bb[144], C[144], Cb[144], Bi[144];
    orc_femstab_parts(use_ofem, A, Ab, B, Bb, C, Cb);
    for (int r = 0; r < 144; ++r) {
        A[r] = A[r] + sf * Ab[r];
        B[r] = B[r] + sf * Bb[r];
        C[r] = C[r] + sf * Cb[r];
    }
    if (gauss_jordan(B, Bi) != 0) return -1;
    const double s0 = 0.5 * dt * dt / mu / eps / h / h;
    for (int r = 0; r < 144; ++r) C[r] = s0 * C[r];
    mat_mul(C, Bi, C);
    mat_mul(C, A, K);
    return 0;
}

static double fs_source(double t, double mu, double h)
{
    const double f0 = 1.0e9;
    return 4.0 * M_PI * M_PI * f0 * f0 * (1.0 - 4.0 * M_PI * M_PI * f0 * f0 * (t - 1.0 / f0) * (t - 1.0 / f0)) *
           exp(-2.0 * M_PI * M_PI * f0 * f0 * (t - 1.0 / f0) * (t - 1.0 / f0)) * mu / h / h / h * 0.001;
}

static size_t fs_edge(int gx, int gy, int c, int i, int j, int k)
{
    if (c == 0) return (size_t)i + (size_t)j * gx + (size_t)k * gx * (gy + 1);
    if (c == 1) return (size_t)i + (size_t)j * (gx + 1) + (size_t)k * (gx + 1) * gy;
    return (size_t)i + (size_t)j * (gx + 1) + (size_t)k * (gx + 1) * (gy + 1);
}

/* local edge q of component c of cell (i,j,k): x (i, j+q0, k+q1),
 * y (i+q1, j, k+q0), z (i+q0, j+q1, k), q = q0 + 2 q1 */
static size_t fs_local(int gx, int gy, int c, int i, int j, int k, int q)
{
    const int a0 = q & 1, a1 = q >> 1;
    if (c == 0) return fs_edge(gx, gy, 0, i, j + a0, k + a1);
    if (c == 1) return fs_edge(gx, gy, 1, i + a1, j, k + a0);
    return fs_edge(gx, gy, 2, i + a0, j + a1, k);
}

int orc_femstab_run(const orc_femstab_case *c, int nsteps, double *E[3], double *traces)
{
    const int gx = c->gx, gy = c->gy, gz = c->gz;
    const size_t n[3] = {(size_t)gx * (gy + 1) * (gz + 1), (size_t)(gx + 1) * gy * (gz + 1), (size_t)(gx + 1) * (gy + 1) * gz};
    double K[144];
    if (orc_femstab_kmat(c->dt, c->mu, c->eps, c->h, c->stabilization, c->use_ofem, K) != 0) return -1;
    const double dt = c->dt, h = c->h, eps = c->eps, mu = c->mu, sf = c->stabilization;
    const int tf = c->time_frequency;
    const int nsamp = nsteps / tf + 1;
    if (traces) memset(traces, 0, sizeof(double) * (size_t)c->nobs * nsamp * 3);
    int r0 = 0, r1 = 1, r2 = 2;
    double t = 0.0;
    for (int step = 1; step < nsteps + 1; ++step) {
        double *E0[3], *E1[3], *E2[3];
        for (int q = 0; q < 3; ++q) {
            E0[q] = E[q] + r0 * n[q]; E1[q] = E[q] + r1 * n[q]; E2[q] = E[q] + r2 * n[q];
            memset(E2[q], 0, sizeof(double) * n[q]);
        }
        for (int k = 0; k < gz; ++k)
            for (int j = 0; j < gy; ++j)
                for (int i = 0; i < gx; ++i) {
                    double loc[12];
                    for (int m = 0; m < 12; ++m) loc[m] = E1[m / 4][fs_local(gx, gy, m / 4, i, j, k, m % 4)];
                    for (int l = 0; l < 12; ++l) {
                        double temp = 0.0;
                        for (int m = 0; m < 12; ++m) temp += K[l * 12 + m] * loc[m];
                        E2[l / 4][fs_local(gx, gy, l / 4, i, j, k, l % 4)] -= temp;
                    }
                }
        for (int q = 0; q < 3; ++q)
            for (size_t e = 0; e < n[q]; ++e) E2[q][e] += 2.0 * E1[q][e] - E0[q][e];
        for (int q = 0; q < 3; ++q)
            for (int s = 0; s < c->nsrc; ++s)
                if (c->src_comp[s] == q) {
                    const int *p = c->src_ijk + 3 * s;
                    E2[q][fs_edge(gx, gy, q, p[0], p[1], p[2])] += fs_source(t, mu, h) * dt * dt / mu / eps / h / h / h;
                }
        for (int s = 0; s < c->ndip; ++s) {
            const int *p = c->dip_ijk + 3 * s;
            const double temp = fs_source(t, mu, h) * dt * dt / mu / eps / 8.0;
            const int i = p[0], j = p[1], k = p[2];
            /* cells c0 (i,j,k), c1 (i,j+1,k), c2 (i,j,k+1), c3 (i,j+1,k+1) */
            const int cj[4] = {j, j + 1, j, j + 1}, ck[4] = {k, k, k + 1, k + 1};
#define X(cell, q) E2[0][fs_local(gx, gy, 0, i, cj[cell], ck[cell], q)]
#define Y(cell, q) E2[1][fs_local(gx, gy, 1, i, cj[cell], ck[cell], q)]
#define Z(cell, q) E2[2][fs_local(gx, gy, 2, i, cj[cell], ck[cell], q)]
            if (!c->use_ofem) {
                X(0, 0) += 1.0 / 8.0 * temp; X(0, 1) += 3.0 / 4.0 * temp; X(0, 2) += 3.0 / 4.0 * temp;
                X(0, 3) += 9.0 / 2.0 * temp; X(1, 1) += 1.0 / 8.0 * temp; X(1, 3) += 3.0 / 4.0 * temp;
                X(2, 2) += 1.0 / 8.0 * temp; X(2, 3) += 3.0 / 4.0 * temp; X(3, 3) += 1.0 / 8.0 * temp;
                Y(0, 0) += sf / 2.0 * temp; Y(0, 2) += sf / 2.0 * temp; Y(1, 0) += sf / 2.0 * temp;
                Y(1, 2) += sf / 2.0 * temp; Y(2, 1) -= sf / 2.0 * temp; Y(2, 3) -= sf / 2.0 * temp;
                Y(3, 1) -= sf / 2.0 * temp; Y(3, 3) -= sf / 2.0 * temp;
                Z(0, 0) -= sf / 2.0 * temp; Z(0, 1) -= sf / 2.0 * temp; Z(1, 2) += sf / 2.0 * temp;
                Z(1, 3) += sf / 2.0 * temp; Z(2, 0) -= sf / 2.0 * temp; Z(2, 1) -= sf / 2.0 * temp;
                Z(3, 2) += sf / 2.0 * temp; Z(3, 3) += sf / 2.0 * temp;
            } else {
                X(0, 3) += 8.0 * temp;
            }
#undef X
#undef Y
#undef Z
        }
        /* PEC: tangential E on every face (fem/fem_simulation.cpp:743-833) */
        for (int k = 0; k <= gz; ++k)
            for (int j = 0; j <= gy; ++j)
                for (int i = 0; i < gx; ++i)
                    if (j == 0 || j == gy || k == 0 || k == gz) E2[0][fs_edge(gx, gy, 0, i, j, k)] = 0.0;
        for (int k = 0; k <= gz; ++k)
            for (int j = 0; j < gy; ++j)
                for (int i = 0; i <= gx; ++i)
                    if (i == 0 || i == gx || k == 0 || k == gz) E2[1][fs_edge(gx, gy, 1, i, j, k)] = 0.0;
        for (int k = 0; k < gz; ++k)
            for (int j = 0; j <= gy; ++j)
                for (int i = 0; i <= gx; ++i)
                    if (i == 0 || i == gx || j == 0 || j == gy) E2[2][fs_edge(gx, gy, 2, i, j, k)] = 0.0;
        if (traces && step % tf == 0) {
            const int *q = c->obs_ijk;
            for (int o = 0; o < c->nobs; ++o) {
                double *out = traces + ((size_t)o * nsamp + step / tf) * 3;
                for (int comp = 0; comp < 3; ++comp) {
                    const int cnt = c->obs_n[3 * o + comp];
                    for (int r = 0; r < cnt; ++r, q += 3) out[comp] += E2[comp][fs_edge(gx, gy, comp, q[0], q[1], q[2])];
                    out[comp] /= (double)cnt;
                }
            }
        }
        t += dt;
        r0 = (r0 + 1) % 3; r1 = (r1 + 1) % 3; r2 = (r2 + 1) % 3;
    }
    return 0;
}
