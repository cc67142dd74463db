/* orc_tetfem.c — FP64 CPU restatement of the tetrahedral edge-element
 * (Nedelec, lowest order / Whitney) time loop.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY (see ems_oracle.h).
 *
 * The reference has no tetrahedral solver; this file defines the discrete
 * scheme the GPU solver must reproduce.  It follows the structure of the
 * reference's symplectic hexahedral step (symplectic_2/fem_simulation.cpp:
 * 557-672: drift, force, kick, drift; symplectic_4/fem_simulation.cpp:
 * 1280-1281,1347-1350: triple jump; fem_v2/fem_simulation.cpp:627-654:
 * three-level leapfrog) with:
 *   - mesh: n_x x n_y x n_z cubes, each split into the 6 Kuhn tetrahedra
 *     v0=c, v1=v0+e_a, v2=v1+e_b, v3=v2+e_c for the permutations (a,b,c);
 *   - DOFs: edge slots 7*node + d, d over the 7 edge directions
 *     (1,0,0) (0,1,0) (0,0,1) (1,1,0) (1,0,1) (0,1,1) (1,1,1) leaving the node;
 *     slots leaving the grid are unused, slots in a boundary face are PEC;
 *   - stiffness K = C^T diag(|T|/mu_T) C with C the per-element curl of the
 *     Whitney functions (curl w_mn = 2 grad(l_m) x grad(l_n));
 *   - mass: per-node 7x7 blocks M_v = W S^+ W^T + alpha (I - D D^+), where
 *     W_i = sum_T eps_T int_T w_i, D_i the edge vector, S = sym(D^T W) and
 *     alpha the mean consistent diagonal; exact for constant fields, SPD, and
 *     block diagonal, so M^-1 is applied block by block;
 *   - source: point dipole, load f_i = w_i(x0).dir * g(t); receivers: Whitney
 *     interpolation of E at a point.
 * Units are normalised: cube edge 1, c0 = 1 (time unit h/c0), relative
 * eps and mu.
 */
#include "ems_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

static const int PERM[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
static const int LOC[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
static const int DIRV[7][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};

int orc_tet_dir_index(int dx, int dy, int dz)
{
    for (int d = 0; d < 7; ++d)
        if (DIRV[d][0] == dx && DIRV[d][1] == dy && DIRV[d][2] == dz) return d;
    return -1;
}

/* Geometry of Kuhn tetrahedron type p (unit cube): gradients of the
 * barycentric coordinates, vertex offsets, curls and integrals of the six
 * Whitney functions. */
void orc_tet_shape(int p, double grad[4][3], int vert[4][3], double curl[6][3], double wint[6][3], double wsq[6])
{
    int a = PERM[p][0], b = PERM[p][1], c = PERM[p][2];
    memset(grad, 0, sizeof(double) * 12);
    grad[0][a] = -1.0;
    grad[1][a] = 1.0; grad[1][b] = -1.0;
    grad[2][b] = 1.0; grad[2][c] = -1.0;
    grad[3][c] = 1.0;
    memset(vert, 0, sizeof(int) * 12);
    vert[1][a] = 1;
    vert[2][a] = 1; vert[2][b] = 1;
    vert[3][0] = vert[3][1] = vert[3][2] = 1;
    const double vol = 1.0 / 6.0;
    for (int l = 0; l < 6; ++l) {
        const double *gm = grad[LOC[l][0]], *gn = grad[LOC[l][1]];
        curl[l][0] = 2.0 * (gm[1] * gn[2] - gm[2] * gn[1]);
        curl[l][1] = 2.0 * (gm[2] * gn[0] - gm[0] * gn[2]);
        curl[l][2] = 2.0 * (gm[0] * gn[1] - gm[1] * gn[0]);
        for (int q = 0; q < 3; ++q) wint[l][q] = vol / 4.0 * (gn[q] - gm[q]);
        double nn = gn[0] * gn[0] + gn[1] * gn[1] + gn[2] * gn[2];
        double mm = gm[0] * gm[0] + gm[1] * gm[1] + gm[2] * gm[2];
        double mn = gm[0] * gn[0] + gm[1] * gn[1] + gm[2] * gn[2];
        wsq[l] = vol / 10.0 * (nn - mn + mm);
    }
}

typedef struct {
    int nx, ny, nz;
    size_t nnode, nslot, ntet;
    int *tet_edge;        /* ntet*6 edge slots */
    unsigned char *pec;   /* per slot: 1 = unused or PEC */
    int *inc_ptr, *inc;   /* slot -> (tet*8 + local) incidence, CSR */
    double shape_curl[6][6][3], shape_wint[6][6][3], shape_wsq[6][6], shape_grad[6][4][3];
    int shape_vert[6][4][3];
} tetmesh;

static size_t node_id(const tetmesh *m, int i, int j, int k)
{
    return (size_t)i + (size_t)(m->nx + 1) * ((size_t)j + (size_t)(m->ny + 1) * k);
}

static void build_tetmesh(tetmesh *m, int nx, int ny, int nz)
{
    m->nx = nx; m->ny = ny; m->nz = nz;
    m->nnode = (size_t)(nx + 1) * (ny + 1) * (nz + 1);
    m->nslot = 7 * m->nnode;
    m->ntet = 6 * (size_t)nx * ny * nz;
    for (int p = 0; p < 6; ++p)
        orc_tet_shape(p, m->shape_grad[p], m->shape_vert[p], m->shape_curl[p], m->shape_wint[p], m->shape_wsq[p]);
    m->tet_edge = malloc(sizeof(int) * 6 * m->ntet);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i)
                for (int p = 0; p < 6; ++p) {
                    size_t t = 6 * ((size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k)) + p;
                    for (int l = 0; l < 6; ++l) {
                        const int *vm = m->shape_vert[p][LOC[l][0]], *vn = m->shape_vert[p][LOC[l][1]];
                        int d = orc_tet_dir_index(vn[0] - vm[0], vn[1] - vm[1], vn[2] - vm[2]);
                        m->tet_edge[6 * t + l] = (int)(7 * node_id(m, i + vm[0], j + vm[1], k + vm[2]) + d);
                    }
                }
    m->pec = malloc(m->nslot);
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i)
                for (int d = 0; d < 7; ++d) {
                    int b[3] = {i + DIRV[d][0], j + DIRV[d][1], k + DIRV[d][2]};
                    int a[3] = {i, j, k}, lim[3] = {nx, ny, nz};
                    int bad = b[0] > nx || b[1] > ny || b[2] > nz;
                    for (int q = 0; q < 3 && !bad; ++q)
                        if (a[q] == b[q] && (a[q] == 0 || a[q] == lim[q])) bad = 1;
                    m->pec[7 * node_id(m, i, j, k) + d] = (unsigned char)bad;
                }
    /* incidence CSR, entries ordered by tet then local index */
    m->inc_ptr = calloc(m->nslot + 1, sizeof(int));
    for (size_t t = 0; t < m->ntet; ++t)
        for (int l = 0; l < 6; ++l) m->inc_ptr[m->tet_edge[6 * t + l] + 1]++;
    for (size_t s = 0; s < m->nslot; ++s) m->inc_ptr[s + 1] += m->inc_ptr[s];
    m->inc = malloc(sizeof(int) * 6 * m->ntet);
    int *fill = calloc(m->nslot, sizeof(int));
    for (size_t t = 0; t < m->ntet; ++t)
        for (int l = 0; l < 6; ++l) {
            int e = m->tet_edge[6 * t + l];
            m->inc[m->inc_ptr[e] + fill[e]++] = (int)(t * 8 + l);
        }
    free(fill);
}

static void free_tetmesh(tetmesh *m)
{
    free(m->tet_edge); free(m->pec); free(m->inc_ptr); free(m->inc);
}

/* symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations */
void orc_sym3_eig(const double A_in[3][3], double w[3], double V[3][3])
{
    double A[3][3];
    memcpy(A, A_in, sizeof(A));
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) V[i][j] = i == j ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
        /* converged: the off-diagonal sum at the rounding floor (exact zero
           is rarely reached, and each further sweep only rounds again) */
        if (off <= 1e-14 * (fabs(A[0][0]) + fabs(A[1][1]) + fabs(A[2][2]))) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                if (A[p][q] == 0.0) continue;
                double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; ++k) {
                    double akp = A[k][p], akq = A[k][q];
                    A[k][p] = c * akp - s * akq;
                    A[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = c * apk - s * aqk;
                    A[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - s * vkq;
                    V[k][q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < 3; ++i) w[i] = A[i][i];
}

/* pseudo-inverse of a symmetric 3x3 (eigenvalues <= tol * max dropped) */
void orc_sym3_pinv(const double A[3][3], double P[3][3])
{
    double w[3], V[3][3];
    orc_sym3_eig(A, w, V);
    double mx = fmax(fabs(w[0]), fmax(fabs(w[1]), fabs(w[2])));
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k)
                if (w[k] > 1e-10 * mx) s += V[i][k] * V[j][k] / w[k];
            P[i][j] = s;
        }
}

/* In-place inverse of an SPD k x k matrix (row-major, stride 7) by Cholesky.
 * Returns 0 on success, -1 if not positive definite. */
int orc_spd_inverse7(double *A, int k)
{
    double L[7][7] = {{0}}, Li[7][7] = {{0}};
    for (int i = 0; i < k; ++i)
        for (int j = 0; j <= i; ++j) {
            double s = A[i * 7 + j];
            for (int q = 0; q < j; ++q) s -= L[i][q] * L[j][q];
            if (i == j) {
                if (!(s > 0.0)) return -1;
                L[i][i] = sqrt(s);
            } else {
                L[i][j] = s / L[j][j];
            }
        }
    for (int i = 0; i < k; ++i) {
        Li[i][i] = 1.0 / L[i][i];
        for (int j = 0; j < i; ++j) {
            double s = 0.0;
            for (int q = j; q < i; ++q) s += L[i][q] * Li[q][j];
            Li[i][j] = -s / L[i][i];
        }
    }
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) {
            double s = 0.0;
            for (int q = (i > j ? i : j); q < k; ++q) s += Li[q][i] * Li[q][j];
            A[i * 7 + j] = s;
        }
    return 0;
}

/* Parts of the mass block of node v: live slots, W, D, diag, S = sym(D^T W)
 * with its pseudo-inverse, G = D^T D with its pseudo-inverse, alpha. */
typedef struct {
    int k, slot[7];
    double W[7][3], D[7][3], diag[7], S[3][3], Sp[3][3], G[3][3], Gp[3][3], alpha;
} massparts;

static void mass_parts(const tetmesh *m, const double *eps_r, size_t v, massparts *b)
{
    int k = 0;
    for (int d = 0; d < 7; ++d)
        if (!m->pec[7 * v + d]) b->slot[k++] = d;
    b->k = k;
    memset(b->W, 0, sizeof(b->W));
    memset(b->diag, 0, sizeof(b->diag));
    for (int r = 0; r < k; ++r) {
        int e = (int)(7 * v + b->slot[r]);
        for (int q = 0; q < 3; ++q) b->D[r][q] = DIRV[b->slot[r]][q];
        for (int s = m->inc_ptr[e]; s < m->inc_ptr[e + 1]; ++s) {
            int t = m->inc[s] >> 3, l = m->inc[s] & 7, p = t % 6;
            double ep = eps_r[t];
            for (int q = 0; q < 3; ++q) b->W[r][q] += ep * m->shape_wint[p][l][q];
            b->diag[r] += ep * m->shape_wsq[p][l];
        }
    }
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) {
            double s1 = 0.0, s2 = 0.0, g = 0.0;
            for (int r = 0; r < k; ++r) { s1 += b->D[r][a] * b->W[r][c]; s2 += b->W[r][a] * b->D[r][c]; g += b->D[r][a] * b->D[r][c]; }
            b->S[a][c] = 0.5 * (s1 + s2);
            b->G[a][c] = g;
        }
    orc_sym3_pinv(b->S, b->Sp);
    orc_sym3_pinv(b->G, b->Gp);
    double alpha = 0.0;
    for (int r = 0; r < k; ++r) alpha += b->diag[r];
    b->alpha = k ? alpha / k : 0.0;
}

/* The mass block M_v = W S^+ W^T + alpha (I - D G^+ D^T) over the live slots
 * (k x k, row stride 7). */
static void mass_block(const massparts *b, double *M)
{
    for (int r = 0; r < b->k; ++r)
        for (int c = 0; c < b->k; ++c) {
            double ws = 0.0, dq = 0.0;
            for (int a = 0; a < 3; ++a)
                for (int e = 0; e < 3; ++e) {
                    ws += b->W[r][a] * b->Sp[a][e] * b->W[c][e];
                    dq += b->D[r][a] * b->Gp[a][e] * b->D[c][e];
                }
            M[r * 7 + c] = ws + b->alpha * ((r == c ? 1.0 : 0.0) - dq);
        }
}

/* Per-node inverse mass blocks (7x7 each, zero rows/cols for PEC/unused slots). */
static int build_minv(const tetmesh *m, const double *eps_r, double *minv)
{
    for (size_t v = 0; v < m->nnode; ++v) {
        massparts b;
        mass_parts(m, eps_r, v, &b);
        double *B = minv + 49 * v;
        memset(B, 0, sizeof(double) * 49);
        if (b.k == 0) continue;
        double M[49] = {0};
        mass_block(&b, M);
        if (orc_spd_inverse7(M, b.k) != 0) return -1;
        for (int r = 0; r < b.k; ++r)
            for (int c = 0; c < b.k; ++c) B[b.slot[r] * 7 + b.slot[c]] = M[r * 7 + c];
    }
    return 0;
}

/* F = K U: curl per element, then curl-transpose gathered per edge slot. */
static void apply_K_tet(const tetmesh *m, const double *mu_inv, const double *U, double *F, double *curl_buf)
{
    const double vol = 1.0 / 6.0;
#pragma omp parallel for schedule(static)
    for (long t = 0; t < (long)m->ntet; ++t) {
        int p = (int)(t % 6);
        double c0 = 0, c1 = 0, c2 = 0;
        for (int l = 0; l < 6; ++l) {
            double u = U[m->tet_edge[6 * t + l]];
            c0 += u * m->shape_curl[p][l][0];
            c1 += u * m->shape_curl[p][l][1];
            c2 += u * m->shape_curl[p][l][2];
        }
        double s = vol * (mu_inv ? mu_inv[t] : 1.0);
        curl_buf[3 * t] = s * c0; curl_buf[3 * t + 1] = s * c1; curl_buf[3 * t + 2] = s * c2;
    }
#pragma omp parallel for schedule(static)
    for (long e = 0; e < (long)m->nslot; ++e) {
        double f = 0.0;
        if (!m->pec[e])
            for (int s = m->inc_ptr[e]; s < m->inc_ptr[e + 1]; ++s) {
                int t = m->inc[s] >> 3, l = m->inc[s] & 7, p = t % 6;
                f += curl_buf[3 * t] * m->shape_curl[p][l][0] + curl_buf[3 * t + 1] * m->shape_curl[p][l][1] +
                     curl_buf[3 * t + 2] * m->shape_curl[p][l][2];
            }
        F[e] = f;
    }
}

static void apply_minv(const tetmesh *m, const double *minv, const double *X, double *Y)
{
#pragma omp parallel for schedule(static)
    for (long v = 0; v < (long)m->nnode; ++v)
        for (int r = 0; r < 7; ++r) {
            double s = 0.0;
            for (int c = 0; c < 7; ++c) s += minv[49 * v + 7 * r + c] * X[7 * v + c];
            Y[7 * v + r] = s;
        }
}

/* Ricker wavelet (delay sqrt(2)/f0) or the reference's second derivative of
 * a Gaussian (fem_v2/fem_simulation.cpp:77-87 form, centre 1/f0). */
double orc_tet_wave(int kind, double f0, double t)
{
    if (kind == 1) {
        double tau = t - sqrt(2.0) / f0;
        return (1.0 - 2.0 * M_PI * M_PI * f0 * f0 * tau * tau) * exp(-M_PI * M_PI * f0 * f0 * tau * tau);
    }
    double delay = t - 1.0 / f0, zeta = 2.0 * M_PI * M_PI * f0 * f0;
    return 2.0 * zeta * (2.0 * zeta * delay * delay - 1.0) * exp(0.0 - zeta * delay * delay) / (2.0 * zeta);
}

/* Locates x (normalised coordinates) and returns the tet index and the six
 * Whitney vectors at x. */
long orc_tet_locate(int nx, int ny, int nz, const double x[3], double w[6][3], int edges[6])
{
    int cell[3], lim[3] = {nx, ny, nz};
    double s[3];
    for (int q = 0; q < 3; ++q) {
        int c = (int)floor(x[q]);
        if (c < 0) c = 0;
        if (c > lim[q] - 1) c = lim[q] - 1;
        cell[q] = c;
        s[q] = x[q] - c;
    }
    /* order axes by decreasing fractional coordinate (stable) */
    int ax[3] = {0, 1, 2};
    for (int a = 1; a < 3; ++a)
        for (int b = a; b > 0 && s[ax[b - 1]] < s[ax[b]]; --b) { int t = ax[b]; ax[b] = ax[b - 1]; ax[b - 1] = t; }
    int p = 0;
    for (; p < 6; ++p)
        if (PERM[p][0] == ax[0] && PERM[p][1] == ax[1] && PERM[p][2] == ax[2]) break;
    double lam[4] = {1.0 - s[ax[0]], s[ax[0]] - s[ax[1]], s[ax[1]] - s[ax[2]], s[ax[2]]};
    double grad[4][3], curl[6][3], wint[6][3], wsq[6];
    int vert[4][3];
    orc_tet_shape(p, grad, vert, curl, wint, wsq);
    for (int l = 0; l < 6; ++l) {
        int a = LOC[l][0], b = LOC[l][1];
        for (int q = 0; q < 3; ++q) w[l][q] = lam[a] * grad[b][q] - lam[b] * grad[a][q];
        const int *vm = vert[a], *vn = vert[b];
        int d = orc_tet_dir_index(vn[0] - vm[0], vn[1] - vm[1], vn[2] - vm[2]);
        size_t node = (size_t)(cell[0] + vm[0]) + (size_t)(nx + 1) * ((size_t)(cell[1] + vm[1]) + (size_t)(ny + 1) * (cell[2] + vm[2]));
        edges[l] = (int)(7 * node + d);
    }
    return 6 * ((long)cell[0] + (long)nx * ((long)cell[1] + (long)ny * cell[2])) + p;
}

int orc_tet_minv(int nx, int ny, int nz, const double *eps_r, double *minv)
{
    tetmesh m;
    build_tetmesh(&m, nx, ny, nz);
    int rc = build_minv(&m, eps_r, minv);
    free_tetmesh(&m);
    return rc;
}

/* Largest eigenvalue of M^-1 K by power iteration with the Rayleigh quotient
 * x.Kx / x.Mx (x.Mx evaluated as x.p with x = M^-1 p). */
double orc_tet_lambda_max(int nx, int ny, int nz, const double *eps_r, const double *mu_inv, int iters)
{
    tetmesh m;
    build_tetmesh(&m, nx, ny, nz);
    double *minv = malloc(sizeof(double) * 49 * m.nnode);
    if (build_minv(&m, eps_r, minv) != 0) { free(minv); free_tetmesh(&m); return -1.0; }
    double *x = malloc(sizeof(double) * m.nslot), *z = malloc(sizeof(double) * m.nslot);
    double *p = malloc(sizeof(double) * m.nslot), *cb = malloc(sizeof(double) * 3 * m.ntet);
    /* deterministic start vector */
    unsigned long long st = 0x9E3779B97F4A7C15ull;
    for (size_t e = 0; e < m.nslot; ++e) {
        st ^= st << 13; st ^= st >> 7; st ^= st << 17;
        x[e] = m.pec[e] ? 0.0 : ((double)(st >> 11) / 9007199254740992.0 - 0.5);
    }
    apply_K_tet(&m, mu_inv, x, p, cb);      /* p = K x0, x1 = M^-1 p */
    apply_minv(&m, minv, p, x);
    double lam = 0.0;
    for (int it = 0; it < iters; ++it) {
        apply_K_tet(&m, mu_inv, x, z, cb);
        double num = 0.0, den = 0.0, nrm = 0.0;
        for (size_t e = 0; e < m.nslot; ++e) { num += x[e] * z[e]; den += x[e] * p[e]; }
        lam = num / den;
        memcpy(p, z, sizeof(double) * m.nslot);
        apply_minv(&m, minv, p, x);
        for (size_t e = 0; e < m.nslot; ++e) nrm += x[e] * x[e];
        nrm = 1.0 / sqrt(nrm);
        for (size_t e = 0; e < m.nslot; ++e) { x[e] *= nrm; p[e] *= nrm; }
    }
    free(x); free(z); free(p); free(cb); free(minv);
    free_tetmesh(&m);
    return lam;
}

/* Stability limit of one step of the integrator for lambda_max of M^-1 K:
 * dt * sqrt(lambda_max) < c with c = 2 (leapfrog / Stormer-Verlet) or the
 * triple-jump value found by scanning its scalar transfer matrix. */
double orc_stability_constant(int integrator)
{
    if (integrator != ORC_SYMP4) return 2.0;
    double x1 = 1.0 / (2.0 - pow(2.0, 1.0 / 3.0)), x2 = 1.0 - 2.0 * x1;
    double sub[3] = {x1, x2, x1};
    double lo = 0.0, hi = 4.0;
    for (int it = 0; it < 200; ++it) {   /* bisection on the first loss of |trace| <= 2 */
        double mid = 0.5 * (lo + hi);
        int stable = 1;
        for (int s = 1; s <= 64 && stable; ++s) {
            double w = mid * s / 64.0;
            double A[2][2] = {{1, 0}, {0, 1}};
            for (int q = 0; q < 3; ++q) {
                double a = sub[q] * w;   /* drift a/2, kick a, drift a/2 on (u, p), omega = 1 */
                double D[2][2] = {{1, a / 2}, {0, 1}}, K[2][2] = {{1, 0}, {-a, 1}};
                double T1[2][2], T2[2][2];
                for (int i = 0; i < 2; ++i)
                    for (int j = 0; j < 2; ++j) T1[i][j] = K[i][0] * D[0][j] + K[i][1] * D[1][j];
                for (int i = 0; i < 2; ++i)
                    for (int j = 0; j < 2; ++j) T2[i][j] = D[i][0] * T1[0][j] + D[i][1] * T1[1][j];
                double R[2][2];
                for (int i = 0; i < 2; ++i)
                    for (int j = 0; j < 2; ++j) R[i][j] = T2[i][0] * A[0][j] + T2[i][1] * A[1][j];
                memcpy(A, R, sizeof(A));
            }
            if (fabs(A[0][0] + A[1][1]) > 2.0) stable = 0;
        }
        if (stable) lo = mid; else hi = mid;
    }
    return lo;
}

/* Conductivity as a per-node loss rate: rho_v = sum sigma_T w / sum eps_T w
 * over the incidences (T, l) of the node's live slots, w = |w_l|^2 integral
 * (the weights of the mass block's alpha term), so that M_sigma,v =
 * rho_v M_eps,v and the loss term M_sigma dU/dt of the momentum equation is
 * rho_v P.  The symplectic loop applies its flow dP/dt = -rho P exactly,
 * P *= exp(-rho dt/2), on each side of the middle kick of every step (a
 * time-symmetric composition, second order when sigma != 0); leapfrog uses
 * the centred difference of the loss term.  den (if given) gets the
 * denominators.  New: the reference has no conductivity in its FEM. */
static void loss_rate(const tetmesh *m, const double *eps_r, const double *sigma, double *rho, double *den)
{
    for (size_t v = 0; v < m->nnode; ++v) {
        double num = 0.0, dd = 0.0;
        for (int d = 0; d < 7; ++d) {
            size_t e = 7 * v + d;
            if (m->pec[e]) continue;
            for (int s = m->inc_ptr[e]; s < m->inc_ptr[e + 1]; ++s) {
                int t = m->inc[s] >> 3, l = m->inc[s] & 7, p = t % 6;
                num += sigma[t] * m->shape_wsq[p][l];
                dd += eps_r[t] * m->shape_wsq[p][l];
            }
        }
        rho[v] = dd > 0.0 ? num / dd : 0.0;
        if (den) den[v] = dd;
    }
}

int orc_tet_loss_rate(int nx, int ny, int nz, const double *eps_r, const double *sigma, double *rho)
{
    tetmesh m;
    build_tetmesh(&m, nx, ny, nz);
    loss_rate(&m, eps_r, sigma, rho, NULL);
    free_tetmesh(&m);
    return 0;
}

/* Time loop.  U, P: nslot values (in/out).  traces: nrec * nsamp * 4
 * (t, Ex, Ey, Ez), sampled before the step every tf steps (symplectic) or
 * E^n at step n (leapfrog, which uses U as E^n and P as E^{n-1}). */
int orc_tet_run(const orc_tet_case *c, int nsteps, double *U, double *P, double *traces)
{
    tetmesh m;
    build_tetmesh(&m, c->nx, c->ny, c->nz);
    double *minv = malloc(sizeof(double) * 49 * m.nnode);
    if (build_minv(&m, c->eps_r, minv) != 0) { free(minv); free_tetmesh(&m); return -1; }
    double *F = calloc(m.nslot, sizeof(double)), *Y = calloc(m.nslot, sizeof(double));
    double *cb = malloc(sizeof(double) * 3 * m.ntet);
    double *mu_inv = NULL;
    if (c->mu_r) {
        mu_inv = malloc(sizeof(double) * m.ntet);
        for (size_t t = 0; t < m.ntet; ++t) mu_inv[t] = 1.0 / c->mu_r[t];
    }
    /* sources and receivers */
    int nd = c->ndip;
    double (*dw)[6] = malloc(sizeof(double) * 6 * (nd > 0 ? nd : 1));
    int (*de)[6] = malloc(sizeof(int) * 6 * (nd > 0 ? nd : 1));
    for (int s = 0; s < nd; ++s) {
        double w[6][3];
        orc_tet_locate(c->nx, c->ny, c->nz, c->dip_pos + 3 * s, w, de[s]);
        const double *dir = c->dip_dir + 3 * s;
        for (int l = 0; l < 6; ++l) dw[s][l] = (w[l][0] * dir[0] + w[l][1] * dir[1] + w[l][2] * dir[2]) * c->dip_amp[s];
    }
    int nr = c->nrec;
    double (*rw)[6][3] = malloc(sizeof(double) * 18 * (nr > 0 ? nr : 1));
    int (*re)[6] = malloc(sizeof(int) * 6 * (nr > 0 ? nr : 1));
    for (int r = 0; r < nr; ++r) orc_tet_locate(c->nx, c->ny, c->nz, c->rec_pos + 3 * r, rw[r], re[r]);
    const int tf = c->time_frequency;
    const int nsamp = nsteps > 0 ? (nsteps - 1) / tf + 1 : 0;
    double t = 0.0, dt = c->dt;
    const double x1 = 1.0 / (2.0 - pow(2.0, 1.0 / 3.0)), x2 = 1.0 - 2.0 * x1;
    double *rho = NULL;
    if (c->sigma) {
        rho = malloc(sizeof(double) * m.nnode);
        loss_rate(&m, c->eps_r, c->sigma, rho, NULL);
    }

#define ADD_SOURCE(vec, time, sign)                                                             \
    for (int s = 0; s < nd; ++s) {                                                              \
        double g = orc_tet_wave(c->dip_kind[s], c->dip_f0[s], (time));                          \
        for (int l = 0; l < 6; ++l) (vec)[de[s][l]] += (sign) * dw[s][l] * g;                   \
    }
    for (int step = 0; step < nsteps; ++step) {
        if (traces && step % tf == 0)
            for (int r = 0; r < nr; ++r) {
                double *o = traces + ((size_t)r * nsamp + step / tf) * 4;
                o[0] = t; o[1] = o[2] = o[3] = 0.0;
                for (int l = 0; l < 6; ++l)
                    for (int q = 0; q < 3; ++q) o[1 + q] += U[re[r][l]] * rw[r][l][q];
            }
        if (c->integrator == ORC_LEAPFROG) {
            /* U = E^n, P = E^{n-1}: E^{n+1} = 2E^n - E^{n-1} - dt^2 M^-1 (K E^n - f(t_n)) */
            apply_K_tet(&m, mu_inv, U, F, cb);
            ADD_SOURCE(F, t, -1.0)
            for (size_t e = 0; e < m.nslot; ++e) if (m.pec[e]) F[e] = 0.0;
            apply_minv(&m, minv, F, Y);
            for (size_t e = 0; e < m.nslot; ++e) {
                double en = U[e];
                if (rho) {   /* (1 + r) E^{n+1} = 2 E^n - (1 - r) E^{n-1} - dt^2 Y,  r = rho dt / 2 */
                    double r = 0.5 * rho[e / 7] * dt;
                    U[e] = m.pec[e] ? 0.0 : (2.0 * en - (1.0 - r) * P[e] - dt * dt * Y[e]) / (1.0 + r);
                } else {
                    U[e] = m.pec[e] ? 0.0 : 2.0 * en - P[e] - dt * dt * Y[e];
                }
                P[e] = en;
            }
        } else {
            double sub[3] = {dt, 0, 0}, off[3] = {0, 0, 0};
            int nsub = 1;
            if (c->integrator == ORC_SYMP4) { nsub = 3; sub[0] = x1 * dt; sub[1] = x2 * dt; sub[2] = x1 * dt; off[1] = x1 * dt; off[2] = (x1 + x2) * dt; }
            for (int q = 0; q < nsub; ++q) {
                double a = sub[q];
                apply_minv(&m, minv, P, Y);
                for (size_t e = 0; e < m.nslot; ++e) U[e] += 0.5 * a * Y[e];
                apply_K_tet(&m, mu_inv, U, F, cb);
                ADD_SOURCE(F, t + off[q] + 0.5 * a, -1.0)
                const int damp = rho && q == nsub / 2;
                if (damp)
                    for (size_t e = 0; e < m.nslot; ++e) P[e] *= exp(-0.5 * dt * rho[e / 7]);
                for (size_t e = 0; e < m.nslot; ++e) {
                    if (m.pec[e]) F[e] = 0.0;
                    P[e] -= a * F[e];
                }
                if (damp)
                    for (size_t e = 0; e < m.nslot; ++e) P[e] *= exp(-0.5 * dt * rho[e / 7]);
                apply_minv(&m, minv, P, Y);
                for (size_t e = 0; e < m.nslot; ++e) U[e] += 0.5 * a * Y[e];
            }
        }
        t += dt;
    }
#undef ADD_SOURCE
    free(F); free(Y); free(cb); free(mu_inv); free(minv); free(rho);
    free(dw); free(de); free(rw); free(re);
    free_tetmesh(&m);
    return 0;
}

/* Discrete energy H = 1/2 P.M^-1 P + 1/2 U.K U (symplectic state). */
double orc_tet_energy(int nx, int ny, int nz, const double *eps_r, const double *U, const double *P)
{
    tetmesh m;
    build_tetmesh(&m, nx, ny, nz);
    double *minv = malloc(sizeof(double) * 49 * m.nnode);
    build_minv(&m, eps_r, minv);
    double *F = malloc(sizeof(double) * m.nslot), *Y = malloc(sizeof(double) * m.nslot);
    double *cb = malloc(sizeof(double) * 3 * m.ntet);
    apply_K_tet(&m, NULL, U, F, cb);
    apply_minv(&m, minv, P, Y);
    double e = 0.0;
    for (size_t q = 0; q < m.nslot; ++q) e += 0.5 * (P[q] * Y[q] + U[q] * F[q]);
    free(minv); free(F); free(Y); free(cb);
    free_tetmesh(&m);
    return e;
}

/* y = M^-1 K x (x, y: nslot values); the spatial operator of the scheme. */
int orc_tet_apply_op(int nx, int ny, int nz, const double *eps_r, const double *x, double *y)
{
    tetmesh m;
    build_tetmesh(&m, nx, ny, nz);
    double *minv = malloc(sizeof(double) * 49 * m.nnode);
    if (build_minv(&m, eps_r, minv) != 0) { free(minv); free_tetmesh(&m); return -1; }
    double *F = malloc(sizeof(double) * m.nslot), *cb = malloc(sizeof(double) * 3 * m.ntet);
    apply_K_tet(&m, NULL, x, F, cb);
    apply_minv(&m, minv, F, y);
    free(F); free(cb); free(minv);
    free_tetmesh(&m);
    return 0;
}

/* Marks unused/PEC slots (1) for tests. */
void orc_tet_pec_mask(int nx, int ny, int nz, unsigned char *mask)
{
    tetmesh m;
    build_tetmesh(&m, nx, ny, nz);
    memcpy(mask, m.pec, m.nslot);
    free_tetmesh(&m);
}

/* f = K x (the stiffness operator alone). */
int orc_tet_apply_K(int nx, int ny, int nz, const double *x, double *f)
{
    tetmesh m;
    build_tetmesh(&m, nx, ny, nz);
    double *cb = malloc(sizeof(double) * 3 * m.ntet);
    apply_K_tet(&m, NULL, x, f, cb);
    free(cb);
    free_tetmesh(&m);
    return 0;
}

/* ------------------------------------------------------------ adjoint ---
 * Gradient of a receiver-trace functional J with respect to the per-tet
 * permittivity, by the discrete adjoint of the symplectic loop of
 * orc_tet_run.  Only the mass blocks depend on eps, so every drift
 * U += c M^-1 P contributes -c (M^-1 Ubar)^T (dM/deps_t) (M^-1 P); these
 * outer products are summed per node (Q_v) over the whole run and
 * contracted with dM_v/deps_t at the end.  All forward P vectors are kept
 * (small cases only). */

/* dM_v/deps_t over the live slots of v (k x k, row stride 7):
 *   dM = dW S^+ W^T + W S^+ dW^T + W d(S^+) W^T + dalpha (I - D G^+ D^T).
 * S^+ keeps the eigenvalues above 1e-10 max|lambda| (orc_sym3_pinv), so at
 * edge and corner nodes, where S is indefinite, it is the spectral function
 * f(lambda) = 1/lambda on the kept eigenvalues and 0 elsewhere; its
 * derivative is V (F o (V^T dS V)) V^T with the divided differences
 * F_ij = (f(l_i) - f(l_j)) / (l_i - l_j), F_ii = f'(l_i) (Daleckii-Krein). */
static void sym3_pinv_deriv(const double S[3][3], const double dS[3][3], double dSp[3][3])
{
    double w[3], V[3][3];
    orc_sym3_eig(S, w, V);
    double mx = fmax(fabs(w[0]), fmax(fabs(w[1]), fabs(w[2])));
    int keep[3];
    for (int i = 0; i < 3; ++i) keep[i] = w[i] > 1e-10 * mx;
    double A[3][3], B[3][3];
    for (int i = 0; i < 3; ++i)          /* A = V^T dS V */
        for (int j = 0; j < 3; ++j) {
            double x = 0.0;
            for (int a = 0; a < 3; ++a)
                for (int c = 0; c < 3; ++c) x += V[a][i] * dS[a][c] * V[c][j];
            A[i][j] = x;
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double F;
            if (keep[i] && keep[j]) F = -1.0 / (w[i] * w[j]);
            else if (keep[i]) F = 1.0 / (w[i] * (w[i] - w[j]));
            else if (keep[j]) F = 1.0 / (w[j] * (w[j] - w[i]));
            else F = 0.0;
            B[i][j] = F * A[i][j];
        }
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) {
            double x = 0.0;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) x += V[a][i] * B[i][j] * V[c][j];
            dSp[a][c] = x;
        }
}

static void mass_block_deriv(const tetmesh *m, const massparts *b, size_t v, size_t t, double *dM)
{
    const int k = b->k, p = (int)(t % 6);
    double dW[7][3] = {{0}}, dd[7] = {0};
    for (int r = 0; r < k; ++r) {
        int e = (int)(7 * v + b->slot[r]);
        for (int s = m->inc_ptr[e]; s < m->inc_ptr[e + 1]; ++s)
            if ((size_t)(m->inc[s] >> 3) == t) {
                int l = m->inc[s] & 7;
                for (int q = 0; q < 3; ++q) dW[r][q] += m->shape_wint[p][l][q];
                dd[r] += m->shape_wsq[p][l];
            }
    }
    double dalpha = 0.0;
    for (int r = 0; r < k; ++r) dalpha += dd[r];
    dalpha = k ? dalpha / k : 0.0;
    double dS[3][3], dSp[3][3];
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) {
            double x = 0.0;
            for (int r = 0; r < k; ++r) x += b->D[r][a] * dW[r][c] + dW[r][a] * b->D[r][c];
            dS[a][c] = 0.5 * x;
        }
    sym3_pinv_deriv(b->S, dS, dSp);
    for (int r = 0; r < k; ++r)
        for (int c = 0; c < k; ++c) {
            double x = 0.0, dq = 0.0;
            for (int a = 0; a < 3; ++a)
                for (int e = 0; e < 3; ++e) {
                    x += dW[r][a] * b->Sp[a][e] * b->W[c][e] + b->W[r][a] * b->Sp[a][e] * dW[c][e] +
                         b->W[r][a] * dSp[a][e] * b->W[c][e];
                    dq += b->D[r][a] * b->Gp[a][e] * b->D[c][e];
                }
            dM[r * 7 + c] = x + dalpha * ((r == c ? 1.0 : 0.0) - dq);
        }
}

/* The mass block of node v (7 x 7 over all slots, zero rows/cols for dead
 * slots) and, when t >= 0, its derivative with respect to eps_t. */
int orc_tet_mass_block(int nx, int ny, int nz, const double *eps_r, long v, long t, double *M, double *dM)
{
    tetmesh m;
    build_tetmesh(&m, nx, ny, nz);
    if (v < 0 || (size_t)v >= m.nnode || t >= (long)m.ntet) { free_tetmesh(&m); return -1; }
    massparts b;
    mass_parts(&m, eps_r, (size_t)v, &b);
    double Mk[49] = {0}, dMk[49] = {0};
    mass_block(&b, Mk);
    if (t >= 0) mass_block_deriv(&m, &b, (size_t)v, (size_t)t, dMk);
    memset(M, 0, sizeof(double) * 49);
    if (dM) memset(dM, 0, sizeof(double) * 49);
    for (int r = 0; r < b.k; ++r)
        for (int c = 0; c < b.k; ++c) {
            M[b.slot[r] * 7 + b.slot[c]] = Mk[r * 7 + c];
            if (dM) dM[b.slot[r] * 7 + b.slot[c]] = dMk[r * 7 + c];
        }
    free_tetmesh(&m);
    return 0;
}

/* Q_v += c/2 (y z^T + z y^T) over every node (y, z: nslot vectors). */
static void accumulate_outer(const tetmesh *m, double c, const double *y, const double *z, double *Q)
{
#pragma omp parallel for schedule(static)
    for (long v = 0; v < (long)m->nnode; ++v)
        for (int r = 0; r < 7; ++r)
            for (int s = 0; s < 7; ++s)
                Q[49 * v + 7 * r + s] += 0.5 * c * (y[7 * v + r] * z[7 * v + s] + z[7 * v + r] * y[7 * v + s]);
}

/* dJ/deps (and dJ/dsigma when grad_sigma is given) for the symplectic
 * integrators.  trace_grad: dJ/dtraces in the layout of orc_tet_run's traces
 * (nrec * nsamp * 4, column 0 ignored).  The run starts from zero fields at
 * t = 0.  With conductivity, each loss factor g_v = exp(-rho_v dt/2) acts
 * twice per step (P_out = g P_in at the middle kick); the adjoint collects
 * zr_v = sum Pbar_out,v . P_in,v, so dJ/drho_v = -(dt/2) g_v zr_v, and rho_v
 * = sum sigma_T c_Tv / sum eps_T c_Tv (c_Tv the loss weights of T at v)
 * gives dJ/dsigma_T = sum_v dJ/drho_v c_Tv / den_v and the extra
 * dJ/deps_T = -sum_v dJ/drho_v rho_v c_Tv / den_v. */
int orc_tet_gradient(const orc_tet_case *c, int nsteps, const double *trace_grad, double *grad_eps, double *grad_sigma)
{
    if (c->integrator == ORC_LEAPFROG) return -2;
    tetmesh m;
    build_tetmesh(&m, c->nx, c->ny, c->nz);
    const size_t ns = m.nslot;
    double *minv = malloc(sizeof(double) * 49 * m.nnode);
    if (build_minv(&m, c->eps_r, minv) != 0) { free(minv); free_tetmesh(&m); return -1; }
    double *mu_inv = NULL;
    if (c->mu_r) {
        mu_inv = malloc(sizeof(double) * m.ntet);
        for (size_t t = 0; t < m.ntet; ++t) mu_inv[t] = 1.0 / c->mu_r[t];
    }
    int nd = c->ndip;
    double (*dw)[6] = malloc(sizeof(double) * 6 * (nd > 0 ? nd : 1));
    int (*de)[6] = malloc(sizeof(int) * 6 * (nd > 0 ? nd : 1));
    for (int s = 0; s < nd; ++s) {
        double w[6][3];
        orc_tet_locate(c->nx, c->ny, c->nz, c->dip_pos + 3 * s, w, de[s]);
        const double *dir = c->dip_dir + 3 * s;
        for (int l = 0; l < 6; ++l) dw[s][l] = (w[l][0] * dir[0] + w[l][1] * dir[1] + w[l][2] * dir[2]) * c->dip_amp[s];
    }
    int nr = c->nrec;
    double (*rw)[6][3] = malloc(sizeof(double) * 18 * (nr > 0 ? nr : 1));
    int (*re)[6] = malloc(sizeof(int) * 6 * (nr > 0 ? nr : 1));
    for (int r = 0; r < nr; ++r) orc_tet_locate(c->nx, c->ny, c->nz, c->rec_pos + 3 * r, rw[r], re[r]);
    const int tf = c->time_frequency;
    const int nsamp = nsteps > 0 ? (nsteps - 1) / tf + 1 : 0;
    const double dt = c->dt, x1 = 1.0 / (2.0 - pow(2.0, 1.0 / 3.0)), x2 = 1.0 - 2.0 * x1;
    double sub[3] = {dt, 0, 0}, off[3] = {0, 0, 0};
    int nsub = 1;
    if (c->integrator == ORC_SYMP4) { nsub = 3; sub[0] = x1 * dt; sub[1] = x2 * dt; sub[2] = x1 * dt; off[1] = x1 * dt; off[2] = (x1 + x2) * dt; }

    double *rho = NULL, *den = NULL, *gl = NULL;
    if (c->sigma) {
        rho = malloc(sizeof(double) * m.nnode);
        den = malloc(sizeof(double) * m.nnode);
        gl = malloc(sizeof(double) * m.nnode);
        loss_rate(&m, c->eps_r, c->sigma, rho, den);
        for (size_t v = 0; v < m.nnode; ++v) gl[v] = exp(-0.5 * dt * rho[v]);
    }
    const int qm = nsub / 2;

    /* forward: Pk[i] = P after kick i (i = 0 .. nsteps*nsub-1), Pk[-1] = 0;
     * Pmid[step] = P after the middle kick, before its second loss factor */
    const size_t nk = (size_t)nsteps * nsub;
    double *Pstore = calloc((nk + 1) * ns, sizeof(double));
    double *Pmid = rho ? calloc((size_t)(nsteps > 0 ? nsteps : 1) * ns, sizeof(double)) : NULL;
    double *U = calloc(ns, sizeof(double)), *P = calloc(ns, sizeof(double));
    double *F = calloc(ns, sizeof(double)), *Y = calloc(ns, sizeof(double)), *Z = calloc(ns, sizeof(double));
    double *cb = malloc(sizeof(double) * 3 * m.ntet);
    double t = 0.0;
    for (int step = 0; step < nsteps; ++step) {
        for (int q = 0; q < nsub; ++q) {
            double a = sub[q];
            apply_minv(&m, minv, P, Y);
            for (size_t e = 0; e < ns; ++e) U[e] += 0.5 * a * Y[e];
            apply_K_tet(&m, mu_inv, U, F, cb);
            for (int s = 0; s < nd; ++s) {
                double g = orc_tet_wave(c->dip_kind[s], c->dip_f0[s], t + off[q] + 0.5 * a);
                for (int l = 0; l < 6; ++l) F[de[s][l]] -= dw[s][l] * g;
            }
            const int damp = rho && q == qm;
            if (damp)
                for (size_t e = 0; e < ns; ++e) P[e] *= gl[e / 7];
            for (size_t e = 0; e < ns; ++e) {
                if (m.pec[e]) F[e] = 0.0;
                P[e] -= a * F[e];
            }
            if (damp) {
                memcpy(Pmid + (size_t)step * ns, P, sizeof(double) * ns);
                for (size_t e = 0; e < ns; ++e) P[e] *= gl[e / 7];
            }
            memcpy(Pstore + (1 + (size_t)step * nsub + q) * ns, P, sizeof(double) * ns);
            apply_minv(&m, minv, P, Y);
            for (size_t e = 0; e < ns; ++e) U[e] += 0.5 * a * Y[e];
        }
        t += dt;
    }
    /* reverse */
    double *Ub = calloc(ns, sizeof(double)), *Pb = calloc(ns, sizeof(double));
    double *Q = calloc(49 * m.nnode, sizeof(double));
    double *zr = calloc(m.nnode, sizeof(double));
    for (int step = nsteps - 1; step >= 0; --step) {
        for (int q = nsub - 1; q >= 0; --q) {
            double a = sub[q];
            size_t i = (size_t)step * nsub + q;
            /* second half drift, with P after kick i */
            apply_minv(&m, minv, Ub, Y);
            for (size_t e = 0; e < ns; ++e) Pb[e] += 0.5 * a * Y[e];
            apply_minv(&m, minv, Pstore + (1 + i) * ns, Z);
            accumulate_outer(&m, 0.5 * a, Y, Z, Q);
            const int damp = rho && q == qm;
            if (damp)   /* second loss factor: P = g Pmid */
                for (size_t e = 0; e < ns; ++e) {
                    zr[e / 7] += Pb[e] * Pmid[(size_t)step * ns + e];
                    Pb[e] *= gl[e / 7];
                }
            /* kick: P -= a Pi K U  =>  Ubar -= a K Pi Pbar */
            for (size_t e = 0; e < ns; ++e) Y[e] = m.pec[e] ? 0.0 : Pb[e];
            apply_K_tet(&m, mu_inv, Y, F, cb);
            for (size_t e = 0; e < ns; ++e) Ub[e] -= a * F[e];
            if (damp)   /* first loss factor: P = g P_before */
                for (size_t e = 0; e < ns; ++e) {
                    zr[e / 7] += Pb[e] * Pstore[i * ns + e];
                    Pb[e] *= gl[e / 7];
                }
            /* first half drift, with P before kick i */
            apply_minv(&m, minv, Ub, Y);
            for (size_t e = 0; e < ns; ++e) Pb[e] += 0.5 * a * Y[e];
            apply_minv(&m, minv, Pstore + i * ns, Z);
            accumulate_outer(&m, 0.5 * a, Y, Z, Q);
        }
        if (step % tf == 0)
            for (int r = 0; r < nr; ++r) {
                const double *g = trace_grad + ((size_t)r * nsamp + step / tf) * 4;
                for (int l = 0; l < 6; ++l)
                    Ub[re[r][l]] += rw[r][l][0] * g[1] + rw[r][l][1] * g[2] + rw[r][l][2] * g[3];
            }
    }
    /* contraction: grad_t = -sum_v <dM_v/deps_t, Q_v> over the nodes whose
     * blocks depend on eps_t (the tails of t's edges) */
    memset(grad_eps, 0, sizeof(double) * m.ntet);
    for (size_t v = 0; v < m.nnode; ++v) {
        massparts b;
        mass_parts(&m, c->eps_r, v, &b);
        if (b.k == 0) continue;
        long seen[64];
        int nseen = 0;
        for (int r = 0; r < b.k; ++r) {
            int e = (int)(7 * v + b.slot[r]);
            for (int s = m.inc_ptr[e]; s < m.inc_ptr[e + 1]; ++s) {
                long tt = m.inc[s] >> 3;
                int dup = 0;
                for (int u = 0; u < nseen; ++u) dup |= seen[u] == tt;
                if (dup || nseen == 64) continue;
                seen[nseen++] = tt;
                double dM[49];
                mass_block_deriv(&m, &b, v, (size_t)tt, dM);
                double acc = 0.0;
                for (int i = 0; i < b.k; ++i)
                    for (int j = 0; j < b.k; ++j) acc += dM[i * 7 + j] * Q[49 * v + 7 * b.slot[i] + b.slot[j]];
                grad_eps[tt] -= acc;
            }
        }
    }
    /* loss-rate terms */
    if (grad_sigma) memset(grad_sigma, 0, sizeof(double) * m.ntet);
    if (rho)
        for (size_t v = 0; v < m.nnode; ++v) {
            if (den[v] <= 0.0) continue;
            const double gr = -0.5 * dt * gl[v] * zr[v];   /* dJ/drho_v */
            for (int d = 0; d < 7; ++d) {
                size_t e = 7 * v + d;
                if (m.pec[e]) continue;
                for (int s = m.inc_ptr[e]; s < m.inc_ptr[e + 1]; ++s) {
                    int tt = m.inc[s] >> 3, l = m.inc[s] & 7, p = tt % 6;
                    const double w = m.shape_wsq[p][l] / den[v];
                    if (grad_sigma) grad_sigma[tt] += gr * w;
                    grad_eps[tt] -= gr * rho[v] * w;
                }
            }
        }
    free(Pstore); free(U); free(P); free(F); free(Y); free(Z); free(cb); free(Ub); free(Pb); free(Q);
    free(zr); free(Pmid); free(rho); free(den); free(gl);
    free(mu_inv); free(minv); free(dw); free(de); free(rw); free(re);
    free_tetmesh(&m);
    return 0;
}
