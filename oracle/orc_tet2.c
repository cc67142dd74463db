/* orc_tet2.c — FP64 CPU restatement of the second-order (20-DOF) Nedelec
 * tetrahedral time loop.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY (see ems_oracle.h).
 *
 * The reference has no tetrahedral solver; its edge-element family is the
 * hexahedral fem_v2 of orders 1-3 (fem_v2/fem_kernels.hpp:6-8,13-86: per
 * element, gather the element's DOFs, contract them with the reference
 * matrix of the order, scatter back).  This file defines the discrete
 * scheme of the second-order tetrahedra that the GPU solver reproduces, on
 * the same Kuhn-split cube mesh as orc_tetfem.c (order 1):
 *   - space: Nedelec first kind of degree 2 (complete curl space, 20 DOFs per
 *     tetrahedron).  With barycentrics l_0..l_3 and Whitney functions
 *     w_ij = l_i grad l_j - l_j grad l_i:
 *       edge (i,j), i < j, other vertices k, l:
 *         tail  (l_i - 5/8 (l_k + l_l)) w_ij,   head  (l_j - 5/8 (l_k + l_l)) w_ij
 *       face (i,j,k), i < j < k:   l_k w_ij,   l_i w_jk
 *     l_k + l_l = 1 - l_i - l_j, so the edge functions depend on the edge's
 *     own vertices only and are tangentially continuous; vertex order is the
 *     global node order (the Kuhn chain), so the face functions agree
 *     between the two tetrahedra of a face.  The -5/8 admixture of the face
 *     functions minimises the condition number of the pair-block
 *     preconditioned mass matrix (element bound 16.2) and keeps every curl
 *     coefficient dyadic;
 *   - DOF layout: 38 planes per node, DOF = plane * nnode + node, node = the
 *     entity's lowest vertex: planes 0..6 edge tails and 7..13 edge heads of
 *     the 7 edge directions of orc_tetfem.c, planes 14 + 2 f and 15 + 2 f the
 *     two functions of face type f (f over the 12 ordered pairs (S1, S2) of
 *     disjoint non-empty axis sets, vertices v, v + e_S1, v + e_S1 + e_S2);
 *   - stiffness K = sum_T (1/mu_T) int curl phi_a . curl phi_b and consistent
 *     mass M = sum_T eps_T int phi_a . phi_b, integrated exactly
 *     (int_T l^a = 6 |T| a! / (|a| + 3)!);
 *   - mass inverse: the drift applies Y = q(M) P, the degree-m Chebyshev
 *     polynomial of the pair-block (2 x 2 blocks of each edge and face)
 *     Jacobi-preconditioned mass on the element bounds [lo, hi] of the
 *     generalised eigenvalues of (M_T, blockdiag M_T) over the six
 *     tetrahedron types (independent of eps and of the mesh).  q(M) is
 *     symmetric positive definite and within 2 r^m (r = (sqrt(hi/lo) - 1) /
 *     (sqrt(hi/lo) + 1)) of M^-1 in the energy norm; the scheme is the
 *     symplectic scheme of the mass q(M)^-1, so its energy
 *     1/2 P.q(M)P + 1/2 U.KU is conserved exactly;
 *   - integrators, sources and receivers as orc_tet_run (symplectic_2/
 *     fem_simulation.cpp:557-672 drift-kick-drift, symplectic_4/
 *     fem_simulation.cpp:1280-1281,1347-1350 triple jump, fem_v2/
 *     fem_simulation.cpp:627-654 three-level leapfrog), the dipole load and
 *     the receiver interpolation with the 20 functions of the containing
 *     tetrahedron.
 * Units as orc_tetfem.c: cube edge 1, c0 = 1, relative eps and mu.
 */
#include "ems_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

static const int PERM2[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
static const int EDGE2[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
static const int FACE2[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};
#define ADMIX (-0.625)

/* ---------------------------------------------------------- polynomials ---
 * Polynomials in the four barycentrics (total degree <= 4) as term lists. */
typedef struct {
    int n;
    unsigned char e[70][4];
    double c[70];
} poly;

static void poly_zero(poly *p) { p->n = 0; }
static void poly_add_term(poly *p, const unsigned char *e, double c)
{
    for (int k = 0; k < p->n; ++k)
        if (!memcmp(p->e[k], e, 4)) { p->c[k] += c; return; }
    memcpy(p->e[p->n], e, 4);
    p->c[p->n++] = c;
}
static void poly_lam(poly *p, int i, double s)
{
    unsigned char e[4] = {0, 0, 0, 0};
    e[i] = 1;
    poly_add_term(p, e, s);
}
static void poly_mul(const poly *a, const poly *b, poly *r)
{
    poly_zero(r);
    for (int i = 0; i < a->n; ++i)
        for (int j = 0; j < b->n; ++j) {
            unsigned char e[4];
            for (int q = 0; q < 4; ++q) e[q] = (unsigned char)(a->e[i][q] + b->e[j][q]);
            poly_add_term(r, e, a->c[i] * b->c[j]);
        }
}
static double fact(int n) { double f = 1.0; for (int k = 2; k <= n; ++k) f *= k; return f; }
/* integral over a tetrahedron of volume 1/6 */
static double poly_int(const poly *a)
{
    double s = 0.0;
    for (int k = 0; k < a->n; ++k) {
        const unsigned char *e = a->e[k];
        s += a->c[k] * fact(e[0]) * fact(e[1]) * fact(e[2]) * fact(e[3]) / fact(e[0] + e[1] + e[2] + e[3] + 3);
    }
    return s;
}
static void poly_deriv(const poly *a, int n, poly *r)
{
    poly_zero(r);
    for (int k = 0; k < a->n; ++k) {
        if (a->e[k][n] == 0) continue;
        unsigned char e[4];
        memcpy(e, a->e[k], 4);
        double m = e[n];
        e[n] -= 1;
        poly_add_term(r, e, a->c[k] * m);
    }
}

/* Basis function a of the reference element as sum_m coef[m] grad l_m. */
typedef struct { poly coef[4]; } vfun;

static void basis_fun(int a, vfun *f)
{
    for (int m = 0; m < 4; ++m) poly_zero(&f->coef[m]);
    poly pre, li, lj, t;
    int i, j;
    poly_zero(&pre);
    if (a < 12) {
        int l = a % 6;
        i = EDGE2[l][0]; j = EDGE2[l][1];
        poly_lam(&pre, a < 6 ? i : j, 1.0);
        for (int k = 0; k < 4; ++k)
            if (k != i && k != j) poly_lam(&pre, k, ADMIX);
    } else {
        int fc = (a - 12) / 2, w = (a - 12) % 2;
        const int *v = FACE2[fc];
        if (w == 0) { poly_lam(&pre, v[2], 1.0); i = v[0]; j = v[1]; }
        else        { poly_lam(&pre, v[0], 1.0); i = v[1]; j = v[2]; }
    }
    /* pre * (l_i grad l_j - l_j grad l_i) */
    poly_zero(&li); poly_lam(&li, i, 1.0);
    poly_zero(&lj); poly_lam(&lj, j, -1.0);
    poly_mul(&pre, &li, &t); f->coef[j] = t;
    poly_mul(&pre, &lj, &t); f->coef[i] = t;
}

static void kuhn_geometry(int p, double g[4][3], int vert[4][3])
{
    int a = PERM2[p][0], b = PERM2[p][1], c = PERM2[p][2];
    memset(g, 0, sizeof(double) * 12);
    g[0][a] = -1.0; g[1][a] = 1.0; g[1][b] = -1.0; g[2][b] = 1.0; g[2][c] = -1.0; g[3][c] = 1.0;
    memset(vert, 0, sizeof(int) * 12);
    vert[1][a] = 1; vert[2][a] = 1; vert[2][b] = 1;
    vert[3][0] = vert[3][1] = vert[3][2] = 1;
}

static void cross3(const double *x, const double *y, double *r)
{
    r[0] = x[1] * y[2] - x[2] * y[1];
    r[1] = x[2] * y[0] - x[0] * y[2];
    r[2] = x[0] * y[1] - x[1] * y[0];
}

/* Element mass and stiffness (20 x 20, row-major) of Kuhn type p with
 * eps = mu = 1, by exact integration (computed once per process). */
static void element_exact(int p, double *M, double *K);
static double elem_cache_M[6][400], elem_cache_K[6][400];
static int elem_cached[6];

void orc_tet2_element(int p, double *M, double *K)
{
    if (!elem_cached[p]) {
        element_exact(p, elem_cache_M[p], elem_cache_K[p]);
        elem_cached[p] = 1;
    }
    memcpy(M, elem_cache_M[p], sizeof(elem_cache_M[p]));
    memcpy(K, elem_cache_K[p], sizeof(elem_cache_K[p]));
}

static void element_exact(int p, double *M, double *K)
{
    double g[4][3];
    int vert[4][3];
    kuhn_geometry(p, g, vert);
    static vfun F[20];
    for (int a = 0; a < 20; ++a) basis_fun(a, &F[a]);
    /* curl (c grad l_m) = sum_n dc/dl_n grad l_n x grad l_m */
    static poly D[20][4][4];
    for (int a = 0; a < 20; ++a)
        for (int n = 0; n < 4; ++n)
            for (int m = 0; m < 4; ++m) poly_deriv(&F[a].coef[m], n, &D[a][n][m]);
    double gg[4][4], cx[4][4][3];
    for (int n = 0; n < 4; ++n)
        for (int m = 0; m < 4; ++m) {
            gg[n][m] = g[n][0] * g[m][0] + g[n][1] * g[m][1] + g[n][2] * g[m][2];
            cross3(g[n], g[m], cx[n][m]);
        }
    poly t;
    for (int a = 0; a < 20; ++a)
        for (int b = 0; b < 20; ++b) {
            double s = 0.0;
            for (int m = 0; m < 4; ++m)
                for (int n = 0; n < 4; ++n) {
                    if (gg[m][n] == 0.0) continue;
                    poly_mul(&F[a].coef[m], &F[b].coef[n], &t);
                    s += gg[m][n] * poly_int(&t);
                }
            M[20 * a + b] = s;
            s = 0.0;
            for (int n = 0; n < 4; ++n) for (int m = 0; m < 4; ++m)
                for (int n2 = 0; n2 < 4; ++n2) for (int m2 = 0; m2 < 4; ++m2) {
                    double d = cx[n][m][0] * cx[n2][m2][0] + cx[n][m][1] * cx[n2][m2][1] + cx[n][m][2] * cx[n2][m2][2];
                    if (d == 0.0) continue;
                    poly_mul(&D[a][n][m], &D[b][n2][m2], &t);
                    s += d * poly_int(&t);
                }
            K[20 * a + b] = s;
        }
}

/* The 20 basis vectors of type p at barycentric point lam. */
static void basis_eval(int p, const double lam[4], double val[20][3])
{
    double g[4][3];
    int vert[4][3];
    kuhn_geometry(p, g, vert);
    for (int a = 0; a < 20; ++a) {
        double pre, li, lj;
        int i, j;
        if (a < 12) {
            int l = a % 6;
            i = EDGE2[l][0]; j = EDGE2[l][1];
            pre = lam[a < 6 ? i : j];
            for (int k = 0; k < 4; ++k)
                if (k != i && k != j) pre += ADMIX * lam[k];
        } else {
            int fc = (a - 12) / 2, w = (a - 12) % 2;
            const int *v = FACE2[fc];
            if (w == 0) { pre = lam[v[2]]; i = v[0]; j = v[1]; }
            else        { pre = lam[v[0]]; i = v[1]; j = v[2]; }
        }
        li = lam[i]; lj = lam[j];
        for (int q = 0; q < 3; ++q) val[a][q] = pre * (li * g[j][q] - lj * g[i][q]);
    }
}

/* ---------------------------------------------------------------- mesh --- */
static const int DIR2[7][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};

static int dir2_index(const int d[3])
{
    for (int k = 0; k < 7; ++k)
        if (DIR2[k][0] == d[0] && DIR2[k][1] == d[1] && DIR2[k][2] == d[2]) return k;
    return -1;
}
/* face type of (S1, S2) as bit masks (bit q = axis q): enumeration order of
 * s1 = 1..7, s2 = 1..7 with disjoint bits */
int orc_tet2_face_type(int s1, int s2)
{
    int t = 0;
    for (int a = 1; a < 8; ++a)
        for (int b = 1; b < 8; ++b) {
            if (a & b) continue;
            if (a == s1 && b == s2) return t;
            ++t;
        }
    return -1;
}
static void face_sets(int f, int *s1, int *s2)
{
    int t = 0;
    for (int a = 1; a < 8; ++a)
        for (int b = 1; b < 8; ++b) {
            if (a & b) continue;
            if (t == f) { *s1 = a; *s2 = b; return; }
            ++t;
        }
}
static int bits_of(const int d[3]) { return (d[0] ? 1 : 0) | (d[1] ? 2 : 0) | (d[2] ? 4 : 0); }

/* Plane and lowest-vertex (local vertex index) of local DOF a of type p. */
void orc_tet2_dof(int p, int a, int *plane, int *lowvert)
{
    double g[4][3];
    int vert[4][3];
    kuhn_geometry(p, g, vert);
    if (a < 12) {
        int l = a % 6, i = EDGE2[l][0], j = EDGE2[l][1];
        int d[3] = {vert[j][0] - vert[i][0], vert[j][1] - vert[i][1], vert[j][2] - vert[i][2]};
        *plane = dir2_index(d) + (a < 6 ? 0 : 7);
        *lowvert = i;
    } else {
        int fc = (a - 12) / 2, w = (a - 12) % 2;
        const int *v = FACE2[fc];
        int d1[3], d2[3];
        for (int q = 0; q < 3; ++q) { d1[q] = vert[v[1]][q] - vert[v[0]][q]; d2[q] = vert[v[2]][q] - vert[v[1]][q]; }
        *plane = 14 + 2 * orc_tet2_face_type(bits_of(d1), bits_of(d2)) + w;
        *lowvert = v[0];
    }
}

typedef struct {
    int nx, ny, nz;
    size_t nnode, ndof, ntet;
    long *tet_dof;          /* ntet * 20 */
    unsigned char *pec;     /* per DOF: unused or tangential on the boundary */
    long *inc_ptr, *inc;    /* DOF -> tet * 32 + local, CSR, ascending tetrahedron order */
    double Mref[6][400], Kref[6][400];
    long *pair;             /* ndof: partner DOF of the same entity */
} t2mesh;

static size_t nid2(const t2mesh *m, long i, long j, long k)
{
    return (size_t)i + (size_t)(m->nx + 1) * ((size_t)j + (size_t)(m->ny + 1) * (size_t)k);
}

void orc_tet2_pec_mask(int nx, int ny, int nz, unsigned char *mask)
{
    size_t nnode = (size_t)(nx + 1) * (ny + 1) * (nz + 1);
    int lim[3] = {nx, ny, nz};
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                size_t v = (size_t)i + (size_t)(nx + 1) * ((size_t)j + (size_t)(ny + 1) * k);
                int x[3] = {i, j, k};
                for (int d = 0; d < 7; ++d) {
                    int bad = 0;
                    for (int q = 0; q < 3; ++q) {
                        if (x[q] + DIR2[d][q] > lim[q]) bad = 1;
                        if (DIR2[d][q] == 0 && (x[q] == 0 || x[q] == lim[q])) bad = 1;
                    }
                    mask[(size_t)d * nnode + v] = mask[(size_t)(7 + d) * nnode + v] = (unsigned char)bad;
                }
                for (int f = 0; f < 12; ++f) {
                    int s1 = 0, s2 = 0, bad = 0;
                    face_sets(f, &s1, &s2);
                    for (int q = 0; q < 3; ++q) {
                        int in = ((s1 | s2) >> q) & 1;
                        if (x[q] + in > lim[q]) bad = 1;
                        if (!in && (x[q] == 0 || x[q] == lim[q])) bad = 1;
                    }
                    mask[(size_t)(14 + 2 * f) * nnode + v] = mask[(size_t)(15 + 2 * f) * nnode + v] = (unsigned char)bad;
                }
            }
}

static void build_t2mesh(t2mesh *m, int nx, int ny, int nz)
{
    m->nx = nx; m->ny = ny; m->nz = nz;
    m->nnode = (size_t)(nx + 1) * (ny + 1) * (nz + 1);
    m->ndof = 38 * m->nnode;
    m->ntet = 6 * (size_t)nx * ny * nz;
    for (int p = 0; p < 6; ++p) orc_tet2_element(p, m->Mref[p], m->Kref[p]);
    int plane[6][20], low[6][20], vert[6][4][3];
    for (int p = 0; p < 6; ++p) {
        double g[4][3];
        kuhn_geometry(p, g, vert[p]);
        for (int a = 0; a < 20; ++a) orc_tet2_dof(p, a, &plane[p][a], &low[p][a]);
    }
    m->tet_dof = malloc(sizeof(long) * 20 * m->ntet);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i)
                for (int p = 0; p < 6; ++p) {
                    size_t t = 6 * ((size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k)) + p;
                    for (int a = 0; a < 20; ++a) {
                        const int *v = vert[p][low[p][a]];
                        m->tet_dof[20 * t + a] = (long)((size_t)plane[p][a] * m->nnode + nid2(m, i + v[0], j + v[1], k + v[2]));
                    }
                }
    m->pec = malloc(m->ndof);
    orc_tet2_pec_mask(nx, ny, nz, m->pec);
    m->inc_ptr = calloc(m->ndof + 1, sizeof(long));
    for (size_t q = 0; q < 20 * m->ntet; ++q) m->inc_ptr[m->tet_dof[q] + 1]++;
    for (size_t s = 0; s < m->ndof; ++s) m->inc_ptr[s + 1] += m->inc_ptr[s];
    m->inc = malloc(sizeof(long) * 20 * m->ntet);
    long *fill = calloc(m->ndof, sizeof(long));
    for (size_t t = 0; t < m->ntet; ++t)
        for (int a = 0; a < 20; ++a) {
            long e = m->tet_dof[20 * t + a];
            m->inc[m->inc_ptr[e] + fill[e]++] = (long)(t * 32 + a);
        }
    free(fill);
    m->pair = malloc(sizeof(long) * m->ndof);
    for (size_t e = 0; e < m->ndof; ++e) {
        size_t pl = e / m->nnode, v = e % m->nnode;
        size_t pp = pl < 14 ? (pl < 7 ? pl + 7 : pl - 7) : (pl % 2 == 0 ? pl + 1 : pl - 1);
        m->pair[e] = (long)(pp * m->nnode + v);
    }
}

static void free_t2mesh(t2mesh *m)
{
    free(m->tet_dof); free(m->pec); free(m->inc_ptr); free(m->inc); free(m->pair);
}

/* y = sum_T s_T A_T x over the live DOFs (A = Mref or Kref, s = eps or
 * 1/mu), by a per-DOF gather of the element products in ascending
 * tetrahedron order. */
static void apply_elem(const t2mesh *m, int stiff, const double *s, const double *x, double *y)
{
#pragma omp parallel for schedule(static)
    for (long e = 0; e < (long)m->ndof; ++e) {
        double acc = 0.0;
        if (!m->pec[e])
            for (long q = m->inc_ptr[e]; q < m->inc_ptr[e + 1]; ++q) {
                long t = m->inc[q] >> 5;
                int a = (int)(m->inc[q] & 31), p = (int)(t % 6);
                const double *A = (stiff ? m->Kref[p] : m->Mref[p]) + 20 * a;
                const long *gd = m->tet_dof + 20 * t;
                double r = 0.0;
                for (int b = 0; b < 20; ++b) r += A[b] * x[gd[b]];
                acc += (s ? s[t] : 1.0) * r;
            }
        y[e] = acc;
    }
}

/* ------------------------------------------------------- mass inverse --- */
/* eigenvalues of a symmetric n x n matrix (cyclic Jacobi), ascending */
static void sym_eig(int n, double *A, double *w)
{
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = i + 1; j < n; ++j) off += A[i * n + j] * A[i * n + j];
        if (off < 1e-30) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                double apq = A[p * n + q];
                if (fabs(apq) < 1e-300) continue;
                double th = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
                double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {
                    double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
            }
    }
    for (int i = 0; i < n; ++i) w[i] = A[i * n + i];
    for (int i = 1; i < n; ++i)
        for (int j = i; j > 0 && w[j - 1] > w[j]; --j) { double t = w[j]; w[j] = w[j - 1]; w[j - 1] = t; }
}

/* Element bounds [lo, hi] of the generalised eigenvalues of (M_T, P_T), P_T
 * the 2 x 2 entity blocks of M_T, over the six types. */
void orc_tet2_cheb_bounds(double *lo, double *hi)
{
    double M[400], K[400];
    *lo = 1e300; *hi = 0.0;
    for (int p = 0; p < 6; ++p) {
        orc_tet2_element(p, M, K);
        /* L^-1 M L^-T with L the Cholesky factor of the block diagonal */
        double Li[400];
        memset(Li, 0, sizeof(Li));
        for (int e = 0; e < 10; ++e) {
            int i0 = e < 6 ? e : 12 + 2 * (e - 6), i1 = e < 6 ? e + 6 : 13 + 2 * (e - 6);
            double a = M[20 * i0 + i0], b = M[20 * i0 + i1], c = M[20 * i1 + i1];
            double l00 = sqrt(a), l10 = b / l00, l11 = sqrt(c - l10 * l10);
            /* inverse of [[l00,0],[l10,l11]] */
            Li[20 * i0 + i0] = 1.0 / l00;
            Li[20 * i1 + i1] = 1.0 / l11;
            Li[20 * i1 + i0] = -l10 / (l00 * l11);
        }
        double T[400], A[400], w[20];
        for (int i = 0; i < 20; ++i)
            for (int j = 0; j < 20; ++j) {
                double s = 0.0;
                for (int k = 0; k < 20; ++k) s += Li[20 * i + k] * M[20 * k + j];
                T[20 * i + j] = s;
            }
        for (int i = 0; i < 20; ++i)
            for (int j = 0; j < 20; ++j) {
                double s = 0.0;
                for (int k = 0; k < 20; ++k) s += T[20 * i + k] * Li[20 * j + k];
                A[20 * i + j] = s;
            }
        sym_eig(20, A, w);
        if (w[0] < *lo) *lo = w[0];
        if (w[19] > *hi) *hi = w[19];
    }
}

typedef struct {
    const t2mesh *m;
    const double *eps;
    double *pinv;     /* ndof: per DOF, the row of its entity block's inverse: (own, partner) pairs */
    double lo, hi;
    int iters;
    double *r, *d;
} t2mass;

static void mass_setup(t2mass *q, const t2mesh *m, const double *eps, int iters)
{
    q->m = m; q->eps = eps; q->iters = iters;
    orc_tet2_cheb_bounds(&q->lo, &q->hi);
    q->pinv = calloc(2 * m->ndof, sizeof(double));
    q->r = calloc(m->ndof, sizeof(double));
    q->d = calloc(m->ndof, sizeof(double));
    /* assembled entity blocks: M[e][e], M[e][partner] */
    for (size_t e = 0; e < m->ndof; ++e) {
        if (m->pec[e]) continue;
        long pe = m->pair[e];
        double a = 0.0, b = 0.0, c = 0.0;
        for (long s = m->inc_ptr[e]; s < m->inc_ptr[e + 1]; ++s) {
            long t = m->inc[s] >> 5;
            int la = (int)(m->inc[s] & 31), p = (int)(t % 6), lb = -1;
            for (int k = 0; k < 20; ++k)
                if (m->tet_dof[20 * t + k] == pe) lb = k;
            a += eps[t] * m->Mref[p][20 * la + la];
            b += eps[t] * m->Mref[p][20 * la + lb];
            c += eps[t] * m->Mref[p][20 * lb + lb];
        }
        double det = a * c - b * b;
        q->pinv[2 * e] = c / det;
        q->pinv[2 * e + 1] = -b / det;
    }
}

static void mass_free(t2mass *q) { free(q->pinv); free(q->r); free(q->d); }

static void precond(const t2mass *q, const double *r, double *z, double scale)
{
    const t2mesh *m = q->m;
#pragma omp parallel for schedule(static)
    for (long e = 0; e < (long)m->ndof; ++e)
        z[e] = m->pec[e] ? 0.0 : scale * (q->pinv[2 * e] * r[e] + q->pinv[2 * e + 1] * r[m->pair[e]]);
}

/* x = q(M) b: degree-m Chebyshev iteration from x = 0 (b, x distinct). */
static void mass_solve(t2mass *q, const double *b, double *x)
{
    const t2mesh *m = q->m;
    const size_t n = m->ndof;
    const double th = 0.5 * (q->hi + q->lo), de = 0.5 * (q->hi - q->lo), sg = th / de;
    double rho = 1.0 / sg;
    precond(q, b, q->d, 1.0 / th);
    memcpy(x, q->d, sizeof(double) * n);
    for (int k = 1; k < q->iters; ++k) {
        apply_elem(m, 0, q->eps, x, q->r);
        for (size_t e = 0; e < n; ++e) q->r[e] = b[e] - q->r[e];
        double rn = 1.0 / (2.0 * sg - rho);
        double c1 = rn * rho, c2 = 2.0 * rn / de;
        /* d = c1 d + c2 Pinv r, x += d */
        for (size_t e = 0; e < n; ++e) {
            if (m->pec[e]) { q->d[e] = 0.0; continue; }
            double z = q->pinv[2 * e] * q->r[e] + q->pinv[2 * e + 1] * q->r[m->pair[e]];
            q->d[e] = c1 * q->d[e] + c2 * z;
        }
        for (size_t e = 0; e < n; ++e) x[e] += q->d[e];
        rho = rn;
    }
}

/* ------------------------------------------------------ point location --- */
/* Containing tetrahedron of x (normalised coordinates; the order-1 rule of
 * orc_tet_locate), its 20 DOFs and the 20 basis vectors at x. */
long orc_tet2_locate(int nx, int ny, int nz, const double x[3], double val[20][3], long dofs[20])
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
    int ax[3] = {0, 1, 2};
    for (int a = 1; a < 3; ++a)
        for (int b = a; b > 0 && s[ax[b - 1]] < s[ax[b]]; --b) { int t = ax[b]; ax[b] = ax[b - 1]; ax[b - 1] = t; }
    int p = 0;
    for (; p < 6; ++p)
        if (PERM2[p][0] == ax[0] && PERM2[p][1] == ax[1] && PERM2[p][2] == ax[2]) break;
    double lam[4] = {1.0 - s[ax[0]], s[ax[0]] - s[ax[1]], s[ax[1]] - s[ax[2]], s[ax[2]]};
    basis_eval(p, lam, val);
    double g[4][3];
    int vert[4][3];
    kuhn_geometry(p, g, vert);
    size_t nnode = (size_t)(nx + 1) * (ny + 1) * (nz + 1);
    for (int a = 0; a < 20; ++a) {
        int pl, lv;
        orc_tet2_dof(p, a, &pl, &lv);
        size_t node = (size_t)(cell[0] + vert[lv][0]) +
                      (size_t)(nx + 1) * ((size_t)(cell[1] + vert[lv][1]) + (size_t)(ny + 1) * (cell[2] + vert[lv][2]));
        dofs[a] = (long)((size_t)pl * nnode + node);
    }
    return 6 * ((long)cell[0] + (long)nx * ((long)cell[1] + (long)ny * cell[2])) + p;
}

/* -------------------------------------------------------------- public --- */
static double *mu_inverse(const t2mesh *m, const double *mu_r)
{
    if (!mu_r) return NULL;
    double *r = malloc(sizeof(double) * m->ntet);
    for (size_t t = 0; t < m->ntet; ++t) r[t] = 1.0 / mu_r[t];
    return r;
}

int orc_tet2_apply(int nx, int ny, int nz, int stiff, const double *coef, const double *x, double *y)
{
    t2mesh m;
    build_t2mesh(&m, nx, ny, nz);
    apply_elem(&m, stiff, coef, x, y);
    free_t2mesh(&m);
    return 0;
}

int orc_tet2_mass_solve(int nx, int ny, int nz, const double *eps_r, int iters, const double *b, double *x)
{
    t2mesh m;
    t2mass q;
    build_t2mesh(&m, nx, ny, nz);
    mass_setup(&q, &m, eps_r, iters);
    mass_solve(&q, b, x);
    mass_free(&q);
    free_t2mesh(&m);
    return 0;
}

double orc_tet2_lambda_max(int nx, int ny, int nz, const double *eps_r, const double *mu_r, int mass_iters, int iters)
{
    t2mesh m;
    t2mass q;
    build_t2mesh(&m, nx, ny, nz);
    mass_setup(&q, &m, eps_r, mass_iters);
    double *mi = mu_inverse(&m, mu_r);
    size_t n = m.ndof;
    double *x = malloc(sizeof(double) * n), *z = malloc(sizeof(double) * n), *p = malloc(sizeof(double) * n);
    unsigned long long st = 0x9E3779B97F4A7C15ull;
    for (size_t e = 0; e < n; ++e) {
        st ^= st << 13; st ^= st >> 7; st ^= st << 17;
        x[e] = m.pec[e] ? 0.0 : ((double)(st >> 11) / 9007199254740992.0 - 0.5);
    }
    /* Rayleigh quotient x.Kx / x.q(M)^-1 x with x = q(M) p */
    apply_elem(&m, 1, mi, x, p);
    mass_solve(&q, p, x);
    double lam = 0.0;
    for (int it = 0; it < iters; ++it) {
        apply_elem(&m, 1, mi, x, z);
        double num = 0.0, den = 0.0, nrm = 0.0;
        for (size_t e = 0; e < n; ++e) { num += x[e] * z[e]; den += x[e] * p[e]; }
        lam = num / den;
        memcpy(p, z, sizeof(double) * n);
        mass_solve(&q, p, x);
        for (size_t e = 0; e < n; ++e) nrm += x[e] * x[e];
        nrm = 1.0 / sqrt(nrm);
        for (size_t e = 0; e < n; ++e) { x[e] *= nrm; p[e] *= nrm; }
    }
    free(x); free(z); free(p); free(mi);
    mass_free(&q);
    free_t2mesh(&m);
    return lam;
}

double orc_tet2_energy(int nx, int ny, int nz, const double *eps_r, int mass_iters, const double *U, const double *P)
{
    t2mesh m;
    t2mass q;
    build_t2mesh(&m, nx, ny, nz);
    mass_setup(&q, &m, eps_r, mass_iters);
    double *F = malloc(sizeof(double) * m.ndof), *Y = malloc(sizeof(double) * m.ndof);
    apply_elem(&m, 1, NULL, U, F);
    mass_solve(&q, P, Y);
    double e = 0.0;
    for (size_t k = 0; k < m.ndof; ++k) e += 0.5 * (P[k] * Y[k] + U[k] * F[k]);
    free(F); free(Y);
    mass_free(&q);
    free_t2mesh(&m);
    return e;
}

/* Time loop: as orc_tet_run with the 20-DOF element; U, P: 38 * nnode values
 * in the plane layout (in/out).  sigma must be NULL. */
int orc_tet2_run(const orc_tet_case *c, int mass_iters, int nsteps, double *U, double *P, double *traces)
{
    if (c->sigma) return -2;
    t2mesh m;
    t2mass q;
    build_t2mesh(&m, c->nx, c->ny, c->nz);
    mass_setup(&q, &m, c->eps_r, mass_iters);
    double *mi = mu_inverse(&m, c->mu_r);
    const size_t n = m.ndof;
    double *F = calloc(n, sizeof(double)), *Y = calloc(n, sizeof(double));
    int nd = c->ndip, nr = c->nrec;
    double (*dw)[20] = malloc(sizeof(double) * 20 * (nd > 0 ? nd : 1));
    long (*de)[20] = malloc(sizeof(long) * 20 * (nd > 0 ? nd : 1));
    for (int s = 0; s < nd; ++s) {
        double val[20][3];
        orc_tet2_locate(c->nx, c->ny, c->nz, c->dip_pos + 3 * s, val, de[s]);
        const double *dir = c->dip_dir + 3 * s;
        for (int a = 0; a < 20; ++a) dw[s][a] = (val[a][0] * dir[0] + val[a][1] * dir[1] + val[a][2] * dir[2]) * c->dip_amp[s];
    }
    double (*rw)[20][3] = malloc(sizeof(double) * 60 * (nr > 0 ? nr : 1));
    long (*re)[20] = malloc(sizeof(long) * 20 * (nr > 0 ? nr : 1));
    for (int r = 0; r < nr; ++r) orc_tet2_locate(c->nx, c->ny, c->nz, c->rec_pos + 3 * r, rw[r], re[r]);
    const int tf = c->time_frequency;
    const int nsamp = nsteps > 0 ? (nsteps - 1) / tf + 1 : 0;
    double t = 0.0, dt = c->dt;
    const double x1 = 1.0 / (2.0 - pow(2.0, 1.0 / 3.0)), x2 = 1.0 - 2.0 * x1;
    int have_y = 0;

#define ADD_SOURCE2(vec, time, sign)                                                            \
    for (int s = 0; s < nd; ++s) {                                                              \
        double g = orc_tet_wave(c->dip_kind[s], c->dip_f0[s], (time));                          \
        for (int a = 0; a < 20; ++a) (vec)[de[s][a]] += (sign) * dw[s][a] * g;                  \
    }
    for (int step = 0; step < nsteps; ++step) {
        if (traces && step % tf == 0)
            for (int r = 0; r < nr; ++r) {
                double *o = traces + ((size_t)r * nsamp + step / tf) * 4;
                o[0] = t; o[1] = o[2] = o[3] = 0.0;
                for (int a = 0; a < 20; ++a)
                    for (int qq = 0; qq < 3; ++qq) o[1 + qq] += U[re[r][a]] * rw[r][a][qq];
            }
        if (c->integrator == ORC_LEAPFROG) {
            apply_elem(&m, 1, mi, U, F);
            ADD_SOURCE2(F, t, -1.0)
            for (size_t e = 0; e < n; ++e) if (m.pec[e]) F[e] = 0.0;
            mass_solve(&q, F, Y);
            for (size_t e = 0; e < n; ++e) {
                double en = U[e];
                U[e] = m.pec[e] ? 0.0 : 2.0 * en - P[e] - dt * dt * Y[e];
                P[e] = en;
            }
        } else {
            double sub[3] = {dt, 0, 0}, off[3] = {0, 0, 0};
            int nsub = 1;
            if (c->integrator == ORC_SYMP4) { nsub = 3; sub[0] = x1 * dt; sub[1] = x2 * dt; sub[2] = x1 * dt; off[1] = x1 * dt; off[2] = (x1 + x2) * dt; }
            for (int qi = 0; qi < nsub; ++qi) {
                double a = sub[qi];
                /* P is unchanged since the last solve: Y = q(M) P is reused */
                if (!have_y) { mass_solve(&q, P, Y); have_y = 1; }
                for (size_t e = 0; e < n; ++e) U[e] += 0.5 * a * Y[e];
                apply_elem(&m, 1, mi, U, F);
                ADD_SOURCE2(F, t + off[qi] + 0.5 * a, -1.0)
                for (size_t e = 0; e < n; ++e) {
                    if (m.pec[e]) F[e] = 0.0;
                    P[e] -= a * F[e];
                }
                mass_solve(&q, P, Y);
                for (size_t e = 0; e < n; ++e) U[e] += 0.5 * a * Y[e];
            }
        }
        t += dt;
    }
#undef ADD_SOURCE2
    free(F); free(Y); free(mi); free(dw); free(de); free(rw); free(re);
    mass_free(&q);
    free_t2mesh(&m);
    return 0;
}

/* ------------------------------------------------------------ adjoint ---
 * Gradient of a receiver-trace functional with respect to the per-tet
 * permittivity by the discrete adjoint of the symplectic loop of
 * orc_tet2_run (drifts merged as the GPU merges them: U += a_0/2 Y at the
 * start of a step, U += (a_q + a_{q+1})/2 Y after kick q).  Only the mass
 * depends on eps; the derivative of the drift increment Y = q(M) P is taken
 * as that of M^-1 P, -q(M) M_T Y, which differs from the derivative of the
 * polynomial by the polynomial's own error (within 2 r^m, see the mass
 * inverse above).  All forward states are kept (small cases only). */
static void elem_contract(const t2mesh *m, const double *Z, const double *Y, double c, double *grad)
{
#pragma omp parallel for schedule(static)
    for (long t = 0; t < (long)m->ntet; ++t) {
        const long *gd = m->tet_dof + 20 * t;
        const double *A = m->Mref[t % 6];
        double s = 0.0;
        for (int a = 0; a < 20; ++a) {
            double r = 0.0;
            for (int b = 0; b < 20; ++b) r += A[20 * a + b] * Y[gd[b]];
            s += Z[gd[a]] * r;
        }
        grad[t] += c * s;
    }
}

int orc_tet2_gradient(const orc_tet_case *c, int mass_iters, int nsteps, const double *trace_grad, double *grad_eps)
{
    if (c->sigma || c->integrator == ORC_LEAPFROG) return -2;
    t2mesh m;
    t2mass q;
    build_t2mesh(&m, c->nx, c->ny, c->nz);
    mass_setup(&q, &m, c->eps_r, mass_iters);
    double *mi = mu_inverse(&m, c->mu_r);
    const size_t n = m.ndof;
    int nd = c->ndip, nr = c->nrec;
    double (*dw)[20] = malloc(sizeof(double) * 20 * (nd > 0 ? nd : 1));
    long (*de)[20] = malloc(sizeof(long) * 20 * (nd > 0 ? nd : 1));
    for (int s = 0; s < nd; ++s) {
        double val[20][3];
        orc_tet2_locate(c->nx, c->ny, c->nz, c->dip_pos + 3 * s, val, de[s]);
        const double *dir = c->dip_dir + 3 * s;
        for (int a = 0; a < 20; ++a) dw[s][a] = (val[a][0] * dir[0] + val[a][1] * dir[1] + val[a][2] * dir[2]) * c->dip_amp[s];
    }
    double (*rw)[20][3] = malloc(sizeof(double) * 60 * (nr > 0 ? nr : 1));
    long (*re)[20] = malloc(sizeof(long) * 20 * (nr > 0 ? nr : 1));
    for (int r = 0; r < nr; ++r) orc_tet2_locate(c->nx, c->ny, c->nz, c->rec_pos + 3 * r, rw[r], re[r]);
    const int tf = c->time_frequency;
    const int nsamp = nsteps > 0 ? (nsteps - 1) / tf + 1 : 0;
    const double dt = c->dt;
    const double x1 = 1.0 / (2.0 - pow(2.0, 1.0 / 3.0)), x2 = 1.0 - 2.0 * x1;
    double sub[3] = {dt, 0, 0}, off[3] = {0, 0, 0};
    int nsub = 1;
    if (c->integrator == ORC_SYMP4) { nsub = 3; sub[0] = x1 * dt; sub[1] = x2 * dt; sub[2] = x1 * dt; off[1] = x1 * dt; off[2] = (x1 + x2) * dt; }
    double hq[3];
    for (int k = 0; k < nsub; ++k) hq[k] = 0.5 * sub[k] + (k + 1 < nsub ? 0.5 * sub[k + 1] : 0.0);

    double *Us = calloc((size_t)(nsteps + 1) * n, sizeof(double)), *Ps = calloc((size_t)(nsteps + 1) * n, sizeof(double));
    double *U = calloc(n, sizeof(double)), *P = calloc(n, sizeof(double)), *F = calloc(n, sizeof(double));
    double *Y[4];
    for (int k = 0; k < 4; ++k) Y[k] = calloc(n, sizeof(double));
    double *Ub = calloc(n, sizeof(double)), *Pb = calloc(n, sizeof(double)), *Z = calloc(n, sizeof(double));
    memset(grad_eps, 0, sizeof(double) * m.ntet);

    /* one step from (U, P) at time t, keeping the drift increments Y[0..nsub] */
#define T2_STEP(time)                                                                                   \
    do {                                                                                                \
        mass_solve(&q, P, Y[0]);                                                                        \
        for (size_t e = 0; e < n; ++e) U[e] += 0.5 * sub[0] * Y[0][e];                                  \
        for (int k = 0; k < nsub; ++k) {                                                                \
            apply_elem(&m, 1, mi, U, F);                                                                \
            for (int s = 0; s < nd; ++s) {                                                              \
                double g = orc_tet_wave(c->dip_kind[s], c->dip_f0[s], (time) + off[k] + 0.5 * sub[k]);  \
                for (int a = 0; a < 20; ++a) F[de[s][a]] -= dw[s][a] * g;                               \
            }                                                                                           \
            for (size_t e = 0; e < n; ++e) P[e] -= m.pec[e] ? 0.0 : sub[k] * F[e];                      \
            mass_solve(&q, P, Y[k + 1]);                                                                \
            for (size_t e = 0; e < n; ++e) U[e] += hq[k] * Y[k + 1][e];                                 \
        }                                                                                               \
    } while (0)

    for (int st = 0; st < nsteps; ++st) {
        memcpy(Us + (size_t)st * n, U, sizeof(double) * n);
        memcpy(Ps + (size_t)st * n, P, sizeof(double) * n);
        T2_STEP(st * dt);
    }
    for (int st = nsteps - 1; st >= 0; --st) {
        memcpy(U, Us + (size_t)st * n, sizeof(double) * n);
        memcpy(P, Ps + (size_t)st * n, sizeof(double) * n);
        T2_STEP(st * dt);
        for (int k = nsub - 1; k >= 0; --k) {
            mass_solve(&q, Ub, Z);                      /* post-drift of substage k */
            for (size_t e = 0; e < n; ++e) Pb[e] += hq[k] * Z[e];
            elem_contract(&m, Z, Y[k + 1], -hq[k], grad_eps);
            apply_elem(&m, 1, mi, Pb, F);                /* kick k */
            for (size_t e = 0; e < n; ++e) Ub[e] -= m.pec[e] ? 0.0 : sub[k] * F[e];
        }
        mass_solve(&q, Ub, Z);                          /* start-of-step drift */
        for (size_t e = 0; e < n; ++e) Pb[e] += 0.5 * sub[0] * Z[e];
        elem_contract(&m, Z, Y[0], -0.5 * sub[0], grad_eps);
        if (st % tf == 0 && st / tf < nsamp)           /* the sample taken at the start of the step */
            for (int r = 0; r < nr; ++r) {
                const double *gr = trace_grad + ((size_t)r * nsamp + st / tf) * 4;
                for (int a = 0; a < 20; ++a)
                    Ub[re[r][a]] += rw[r][a][0] * gr[1] + rw[r][a][1] * gr[2] + rw[r][a][2] * gr[3];
            }
    }
#undef T2_STEP
    free(Us); free(Ps); free(U); free(P); free(F); free(Ub); free(Pb); free(Z);
    for (int k = 0; k < 4; ++k) free(Y[k]);
    free(mi); free(dw); free(de); free(rw); free(re);
    mass_free(&q);
    free_t2mesh(&m);
    return 0;
}
