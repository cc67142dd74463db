/* ems_oracle.h — FP64 CPU restatement of the EMSolvers time loops.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or
 * calls this code; only the tests, the smoke check and the CPU-baseline leg of
 * bench.py load it, as the checker.  Each function states the reference
 * file:line it restates (paths relative to the EMSolvers `src/` tree).
 *
 * Parity pinning: the FDTD and fem_v2-family functions are checked against
 * binaries built from the unmodified reference sources (oracle/build_ref.sh)
 * and against the golden fixtures in tests/golden/.  Extensions that the
 * reference does not have (per-cell materials, CPML, tetrahedral elements,
 * adjoints) reduce exactly to the reference where they overlap and are
 * otherwise pinned by physical invariants (reflection, cavity modes, energy,
 * finite differences) in the tests.
 */
#ifndef EMS_ORACLE_H
#define EMS_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- FDTD --- */
typedef struct {
    int nx, ny, nz;
    double h, dt, eps, mu;        /* uniform background (absolute eps, mu) */
    int time_frequency;
    /* optional per-cell material: mat_id[nx*ny*nz] indexes mat_eps/mat_sigma */
    const uint16_t *mat_id;
    const double *mat_eps;        /* absolute permittivity per material */
    const double *mat_sigma;      /* conductivity per material [S/m] */
    int nmat;
    /* optional CPML on all six faces, `pml` cells thick (0 = none) */
    int pml;
    double pml_m, pml_kmax, pml_amax, pml_R0;
    /* point sources: component 0/1/2 = Ex/Ey/Ez, stored (i,j,k) index */
    int nsrc;
    const int *src_comp;
    const int *src_ijk;
    const int *src_kind;          /* 0 = reference Gaussian derivative, 1 = Ricker */
    const double *src_f0;
    const double *src_amp;
    /* receivers: obs_n[3*o+c] samples of component c for receiver o */
    int nobs;
    const int *obs_n;
    const int *obs_ijk;           /* concatenated (i,j,k) triples */
} orc_fdtd_case;

/* Runs nsteps; E[3], H[3] hold the fields in the reference padded layout
 * (in/out).  traces: nobs*(nsteps/tf+1)*3 doubles. */
int orc_fdtd_run(const orc_fdtd_case *c, int nsteps, double *E[3], double *H[3], double *traces);
double orc_fdtd_source(int kind, double f0, double t, double h);

/* ------------------------------------------------------ hexahedral FEM --- */
enum { ORC_LEAPFROG = 0, ORC_SYMP2 = 1, ORC_SYMP4 = 2 };
typedef struct {
    int order, gx, gy, gz;
    double h, dt, eps, mu;
    int time_frequency;
    int integrator;               /* ORC_LEAPFROG / ORC_SYMP2 / ORC_SYMP4 */
    const double *kmat;           /* unscaled element matrix, TOTAL x TOTAL */
    int nsrc; const int *src_comp; const int *src_ijk;
    int nobs; const int *obs_ijk;
} orc_hexfem_case;

/* ef[c] holds all three levels of component c (reference layout). traces:
 * nobs * ((nsteps-1)/tf+1) * 4 doubles (t, Ex, Ey, Ez). */
int orc_hexfem_run(const orc_hexfem_case *c, int nsteps, double *ef[3], double *traces);
size_t orc_hexfem_ncomp(int gx, int gy, int gz, int comp);

/* ----------------------------------------------------- tetrahedral FEM --- */
typedef struct {
    int nx, ny, nz;               /* cubes; 6 Kuhn tetrahedra each */
    const double *eps_r;          /* per tetrahedron */
    const double *mu_r;           /* per tetrahedron or NULL (= 1) */
    int integrator;               /* ORC_LEAPFROG / ORC_SYMP2 / ORC_SYMP4 */
    double dt;                    /* normalised time step */
    int time_frequency;
    int ndip;
    const double *dip_pos, *dip_dir, *dip_f0, *dip_amp;   /* normalised units */
    const int *dip_kind;          /* 1 = Ricker, 0 = Gaussian second derivative */
    int nrec;
    const double *rec_pos;
    const double *sigma;          /* conductivity per tetrahedron or NULL (= 0) */
} orc_tet_case;

int orc_tet_run(const orc_tet_case *c, int nsteps, double *U, double *P, double *traces);
int orc_tet_minv(int nx, int ny, int nz, const double *eps_r, double *minv);
double orc_tet_lambda_max(int nx, int ny, int nz, const double *eps_r, const double *mu_inv, int iters);
double orc_stability_constant(int integrator);
double orc_tet_energy(int nx, int ny, int nz, const double *eps_r, const double *U, const double *P);
double orc_tet_wave(int kind, double f0, double t);
long orc_tet_locate(int nx, int ny, int nz, const double x[3], double w[6][3], int edges[6]);
void orc_tet_shape(int p, double grad[4][3], int vert[4][3], double curl[6][3], double wint[6][3], double wsq[6]);
int orc_tet_dir_index(int dx, int dy, int dz);
void orc_sym3_eig(const double A[3][3], double w[3], double V[3][3]);
void orc_sym3_pinv(const double A[3][3], double P[3][3]);
int orc_spd_inverse7(double *A, int k);
int orc_tet_apply_op(int nx, int ny, int nz, const double *eps_r, const double *x, double *y);
void orc_tet_pec_mask(int nx, int ny, int nz, unsigned char *mask);
int orc_tet_apply_K(int nx, int ny, int nz, const double *x, double *f);
int orc_tet_mass_block(int nx, int ny, int nz, const double *eps_r, long v, long t, double *M, double *dM);
int orc_tet_gradient(const orc_tet_case *c, int nsteps, const double *trace_grad, double *grad_eps, double *grad_sigma);
int orc_tet_loss_rate(int nx, int ny, int nz, const double *eps_r, const double *sigma, double *rho);

/* ------------------------------- second-order tetrahedral FEM (orc_tet2.c) --- */
/* Element mass and stiffness of Kuhn type p (20 x 20, eps = mu = 1). */
void orc_tet2_element(int p, double *M, double *K);
/* Plane (0..37) and lowest local vertex of local DOF a of type p. */
void orc_tet2_dof(int p, int a, int *plane, int *lowvert);
int orc_tet2_face_type(int s1, int s2);
/* Unused / tangential-boundary DOFs (38 * nnode, plane layout). */
void orc_tet2_pec_mask(int nx, int ny, int nz, unsigned char *mask);
/* Element bounds of the pair-block preconditioned mass. */
void orc_tet2_cheb_bounds(double *lo, double *hi);
/* y = sum_T coef_T A_T x with A = Kref (stiff) or Mref; coef NULL = 1. */
int orc_tet2_apply(int nx, int ny, int nz, int stiff, const double *coef, const double *x, double *y);
/* x = q(M) b, the degree-iters Chebyshev mass inverse. */
int orc_tet2_mass_solve(int nx, int ny, int nz, const double *eps_r, int iters, const double *b, double *x);
long orc_tet2_locate(int nx, int ny, int nz, const double x[3], double val[20][3], long dofs[20]);
double orc_tet2_lambda_max(int nx, int ny, int nz, const double *eps_r, const double *mu_r, int mass_iters, int iters);
double orc_tet2_energy(int nx, int ny, int nz, const double *eps_r, int mass_iters, const double *U, const double *P);
int orc_tet2_run(const orc_tet_case *c, int mass_iters, int nsteps, double *U, double *P, double *traces);
/* dJ/deps_r per tetrahedron (API order 6 * cell + p) of the symplectic loop
 * from zero fields, given dJ/dtraces (nrec x nsamp x 4, column 0 ignored). */
int orc_tet2_gradient(const orc_tet_case *c, int mass_iters, int nsteps, const double *trace_grad, double *grad_eps);

/* ----------------------------------------- Adams-Bashforth-Moulton (hex) --- */
typedef struct {
    int gx, gy, gz;
    double h, dt, eps, mu;
    int time_frequency;
    const double *lamped1;        /* kmat/lamped1.csv, 12 x 12 */
    int nsrc; const int *src_comp; const int *src_ijk;
    int ndip; const int *dip_ijk;   /* x-directed Hertz dipoles */
    int nobs; const int *obs_n; const int *obs_ijk;
} orc_abm_case;

/* E[c], H[c]: 4 levels each (ring of 3 + scratch).  traces: nobs*(nsteps/tf+1)*3. */
int orc_abm_run(const orc_abm_case *c, int nsteps, double *E[3], double *H[3], double *traces);
void orc_abm_kmat(const double *lamped1, double *K);

/* ------------------------------ stabilised order-1 hexahedral FEM (fem/) --- */
typedef struct {
    int gx, gy, gz;
    double h, dt, eps, mu;
    int time_frequency;
    double stabilization;
    int use_ofem;
    int nsrc; const int *src_comp; const int *src_ijk;
    int ndip; const int *dip_ijk;   /* x-directed Hertz dipoles */
    int nobs; const int *obs_n; const int *obs_ijk;
} orc_femstab_case;

/* E[c]: 3 levels per component (the reference's ring).  traces: nobs*(nsteps/tf+1)*3. */
int orc_femstab_run(const orc_femstab_case *c, int nsteps, double *E[3], double *traces);
/* K of the reference (12 x 12, row-major, the dt^2 / (2 mu eps h^2) factor included) */
int orc_femstab_kmat(double dt, double mu, double eps, double h, double stabilization, int use_ofem, double *K);
/* A, Abar, B, Bbar, C, Cbar of the conventional (0) or OFEM (1) basis */
void orc_femstab_parts(int use_ofem, double *A, double *Abar, double *B, double *Bbar, double *C, double *Cbar);

#ifdef __cplusplus
}
#endif
#endif
