/* ems.h — C ABI of libems, the GB300 (sm_103a) time-domain Maxwell engine.
 *
 * Drop-in for the time loops of EMSolvers (paths relative to its src/ tree):
 *   fdtd/          Yee FDTD                 -> ems_fdtd_*
 *   fem_v2/, symplectic_2/, symplectic_4/   -> ems_hexfem_* (leapfrog, symp2, symp4)
 *   fem_abm/       Adams-Bashforth-Moulton  -> ems_hexfem_* with EMS_ABM
 *   fem/           stabilised order 1       -> ems_femstab_*
 *   (new)          tetrahedral Nedelec FEM  -> ems_tetfem_*
 * The reference exposes C++ classes named FemSimulation; each entry point
 * below names the member it replaces.  Conventions:
 *   - every function returns an int status: EMS_OK (0) or a negative code;
 *     ems_last_error() gives a message for the handle;
 *   - handles are independent (the reference keeps file-scope globals, so
 *     only one instance per process works there); each handle owns its
 *     device memory and one CUDA stream;
 *   - the caller owns every host buffer passed in; plain pointers and sizes,
 *     no library types cross the boundary;
 *   - all sizes count elements, not bytes.
 */
#ifndef EMS_H
#define EMS_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define EMS_ABI_VERSION 1

typedef struct ems_sim ems_sim;

enum ems_status {
    EMS_OK = 0,
    EMS_ERR_INVALID_ARGUMENT = -1,  /* bad parameter, index out of domain, CFL violated */
    EMS_ERR_CUDA = -2,              /* a CUDA runtime call failed */
    EMS_ERR_OUT_OF_MEMORY = -3,     /* device or host allocation failed */
    EMS_ERR_IO = -4,                /* file missing / unreadable / malformed */
    EMS_ERR_STATE = -5,             /* call not valid in the handle's state */
    EMS_ERR_DEVICE_TIMEOUT = -6,    /* a bounded device-side wait gave up: a grid barrier of the persistent
                                       tetrahedral step (ems_run); the fields are invalid, reset the handle */
    EMS_ERR_NOT_FINITE = -7,        /* NaN/Inf in the fields after ems_run (the run's traces stay readable),
                                       or a tetrahedral mass block that is not positive definite */
    EMS_ERR_UNSUPPORTED = -8        /* combination not implemented */
};

enum ems_precision { EMS_FP64 = 0, EMS_FP32 = 1 };
enum ems_integrator { EMS_LEAPFROG = 0, EMS_SYMP2 = 1, EMS_SYMP4 = 2, EMS_ABM = 3 };
enum ems_waveform {
    EMS_WAVE_REFERENCE = 0,  /* the reference solver's own source function */
    EMS_WAVE_RICKER = 1      /* Ricker wavelet, centre frequency f0, delay sqrt(2)/f0 */
};

int ems_abi_version(void);
const char *ems_status_string(int status);
const char *ems_last_error(const ems_sim *sim);
/* Number of CUDA devices visible (0 when none); never fails. */
int ems_device_count(void);

/* ------------------------------------------------------------------ FDTD */
typedef struct {
    int grid[3];                /* cells nx, ny, nz */
    double h;                   /* cell size [m] (reference: domain_size) */
    double dt;                  /* time step [s] */
    double permittivity;        /* background eps [F/m] */
    double permeability;        /* mu [H/m] */
    int time_frequency;         /* sample receivers every this many steps */
    int precision;              /* EMS_FP64 (bit-identical to the reference) or EMS_FP32 */
    int pml_cells;              /* CPML thickness on every face (0 = PEC only, as the reference) */
    double pml_order;           /* polynomial grading m (default 3 if 0) */
    double pml_kappa_max;       /* kappa_max (default 1 if 0) */
    double pml_alpha_max;       /* alpha_max [S/m] */
    double pml_reflection;      /* target normal reflection R0 (default 1e-6 if 0) */
} ems_fdtd_params;

/* Replaces FemSimulation::FemSimulation (fdtd/fdtd_simulation.cpp:38-53,
 * layout 55-88).  Fields use the reference's padded layout: Ex (nx+1)(ny+2)(nz+2),
 * Ey (nx+2)(ny+1)(nz+2), Ez (nx+2)(ny+2)(nz+1), Hx nx(ny+1)(nz+1),
 * Hy (nx+1)ny(nz+1), Hz (nx+1)(ny+1)nz, x fastest. */
int ems_fdtd_create(const ems_fdtd_params *params, ems_sim **out);
/* Replaces setSource_x/_y/_z (fdtd/fdtd_simulation.cpp:90-106; injection
 * 222-239).  component 0/1/2 = Ex/Ey/Ez; ijk is the padded-array index. */
int ems_fdtd_set_source(ems_sim *sim, int component, const int ijk[3], int waveform, double f0, double amplitude);
/* Replaces setObservationPoint (fdtd/fdtd_simulation.cpp:108-113): one
 * receiver averaging n_x Ex samples, n_y Ey samples and n_z Ez samples
 * (triples of padded indices).  As in the reference, an empty list gives NaN. */
int ems_fdtd_add_observation(ems_sim *sim, const int *x_ijk, int n_x, const int *y_ijk, int n_y,
                             const int *z_ijk, int n_z);
/* New: per-cell absolute permittivity [F/m] and conductivity [S/m], arrays of
 * nx*ny*nz (x fastest).  Each E sample takes the material of one owning cell
 * (Ex(i,j,k) -> cell (min(i,nx-1), j-1, k-1), Ey -> (i-1, min(j,ny-1), k-1),
 * Ez -> (i-1, j-1, min(k,nz-1))).  At most 65535 distinct (eps, sigma) pairs. */
int ems_fdtd_set_material(ems_sim *sim, const double *eps, const double *sigma);

/* --------------------------------------------------------- hexahedral FEM */
typedef struct {
    int order;                  /* element order 1..3 */
    int grid[3];                /* fine grid (edges) per direction; elements = grid/order */
    double h;                   /* fine cell size [m] (reference: domain_size) */
    double dt;                  /* time step [s] */
    double permittivity, permeability;
    int time_frequency;
    int use_ofem;               /* 1: kmat/{o}.csv, 0: kmat/lamped{o}.csv */
    int integrator;             /* EMS_LEAPFROG (fem_v2), EMS_SYMP2, EMS_SYMP4, EMS_ABM */
    int precision;              /* EMS_FP64 or EMS_FP32 */
    const char *kmat_dir;       /* directory holding the element-matrix CSVs ("kmat" if NULL) */
} ems_hexfem_params;

/* Replaces FemSimulation::FemSimulation + calculateElementStiffnessMatrix of
 * fem_v2/fem_simulation.cpp:89-160,458-490 (symplectic_2 scaling at 473).
 * Field levels keep the reference layout: per component 3 levels of
 * gx(gy+1)(gz+1) / (gx+1)gy(gz+1) / (gx+1)(gy+1)gz values.
 * Leapfrog: levels rotate (E^{n-1}, E^n, E^{n+1}); symplectic: U, P, F. */
int ems_hexfem_create(const ems_hexfem_params *params, ems_sim **out);
/* Replaces setSource_x/_y/_z (fem_v2/fem_simulation.cpp:492-545): a point
 * source on the fine-grid edge (i,j,k) of the given component. */
int ems_hexfem_set_source(ems_sim *sim, int component, const int ijk[3]);
/* Replaces setObservationPoint (fem_v2/fem_simulation.cpp:547-563). */
int ems_hexfem_add_observation(ems_sim *sim, const int ijk[3]);
/* EMS_ABM handles (fem_abm): replaces setSourceDipole_x
 * (fem_abm/fem_simulation.cpp:266-269; injection 407-481, 758-833): an
 * x-directed Hertz dipole spread over the cells (i, j..j+1, k..k+1). */
int ems_hexfem_add_dipole(ems_sim *sim, const int ijk[3]);
/* EMS_ABM handles: replaces setObservationPoint with edge lists
 * (fem_abm/fem_simulation.cpp:271-276, sampling 972-1013): one receiver
 * averaging n_x x-edges, n_y y-edges and n_z z-edges of E. */
int ems_hexfem_add_observation_edges(ems_sim *sim, const int *x_ijk, int n_x, const int *y_ijk, int n_y, const int *z_ijk,
                                     int n_z);

/* ------------------------------- stabilised order-1 hexahedral FEM (fem/) */
typedef struct {
    int grid[3];                /* cells per direction (order 1: one edge per cell side) */
    double h;                   /* cell size [m] (reference: domain_size) */
    double dt;                  /* time step [s] */
    double permittivity, permeability;
    int time_frequency;
    double stabilization_factor;/* s of At = A + s Abar, Bt = B + s Bbar, Ct = C + s Cbar (reference default 0.3) */
    int use_ofem;               /* 0: conventional basis, 1: orthogonal (OFEM) basis */
    int precision;              /* EMS_FP64 (bit-identical to the reference) or EMS_FP32 */
} ems_femstab_params;

/* Replaces FemSimulation::FemSimulation + calculateElementStiffnessMatrix of
 * fem/fem_simulation.cpp:40-57,125-434: the three-level update
 * E^{n+1} = -K E^n + 2 E^n - E^{n-1} with K = dt^2 / (2 mu eps h^2) Ct Bt^-1 At.
 * The handle takes point sources (ems_hexfem_set_source, fem/:436-454),
 * x-directed Hertz dipoles (ems_hexfem_add_dipole, fem/:456-459, injection
 * 636-740) and edge-list receivers (ems_hexfem_add_observation_edges,
 * fem/:461-466, sampling 856-903).  Fields: which 0..2 = Ex, Ey, Ez, the
 * reference's three levels per component (fem/:67-72). */
int ems_femstab_create(const ems_femstab_params *params, ems_sim **out);
/* The handle's element matrix K (12 x 12 row-major, the dt^2 / (2 mu eps h^2)
 * factor included; the reference's element_stiffness_matrix_), n = 144. */
int ems_femstab_element_matrix(const ems_sim *sim, double *K, size_t n);

/* -------------------------------------------------------- tetrahedral FEM */
typedef struct {
    int cells[3];               /* structured cube of cells, each split into 6 tetrahedra */
    double h;                   /* cube edge [m] */
    int order;                  /* Nedelec order: 1 (Whitney, 6 DOFs per tetrahedron) or 2 (20 DOFs) */
    int integrator;             /* EMS_LEAPFROG, EMS_SYMP2, EMS_SYMP4 */
    int precision;              /* EMS_FP64 or EMS_FP32 */
    double dt;                  /* time step [s]; 0 = cfl_fraction x stability limit */
    double cfl_fraction;        /* used when dt == 0 (default 0.9) */
    int time_frequency;
} ems_tetfem_params;

/* Order 2: the complete second-order Nedelec space (2 DOFs per edge, 2 per
 * face), 38 DOFs per node: fields and DOF vectors are 38*(nx+1)(ny+1)(nz+1)
 * values per shot, DOF 38*node + plane (planes 0..6 the edge tails and 7..13
 * the edge heads of the 7 edge directions, 14+2f and 15+2f the two
 * functions of face type f), the consistent mass inverted by a fixed-degree
 * Chebyshev polynomial in every drift.  Order-2 handles have no
 * conductivity (sigma NULL or zero) and no adjoint (EMS_ERR_UNSUPPORTED). */
int ems_tetfem_create(const ems_tetfem_params *params, ems_sim **out);
/* The order-2 element's mass (eps = 1) and stiffness (mu = 1) matrices of
 * Kuhn tetrahedron type 0..5 as the solver computes them, 20 x 20
 * row-major each (n = 400); no handle needed.  New: the reference's element
 * matrices are the fem_v2 kmat CSV files (fem_v2/fem_simulation.cpp:1477-1524). */
int ems_tetfem_element_matrices(int order, int type, double *M, double *K, size_t n);
/* Relative permittivity and conductivity [S/m] per tetrahedron (6 per cell,
 * cells x fastest, tetrahedron index = 6*cell + permutation). sigma may be NULL. */
int ems_tetfem_set_material(ems_sim *sim, const double *eps_r, const double *sigma);
/* Point dipole at pos [m] with direction dir, Ricker (or reference) wavelet. */
int ems_tetfem_add_dipole(ems_sim *sim, const double pos[3], const double dir[3], int waveform, double f0,
                          double amplitude);
/* Receiver recording E (x,y,z) at pos [m] by Whitney interpolation. */
int ems_tetfem_add_receiver(ems_sim *sim, const double pos[3]);
/* Time step in use (after automatic selection) and the stability limit. */
int ems_tetfem_time_step(const ems_sim *sim, double *dt, double *dt_limit);
/* One application of the stiffness operator, f = K u, on edge-slot vectors of
 * 7*(nx+1)(ny+1)(nz+1) values (slot 7*node + d), in normalised units (cube
 * edge 1, K = C^T diag(|T|/mu) C): the element-by-element curl followed by
 * the curl-transpose gather of the time step (symplectic_2/fem_simulation.cpp
 * :603-639 applies the hexahedral counterpart).  Computed in the handle's
 * precision; PEC and unused slots of f are zero.  Does not touch the state. */
int ems_tetfem_apply_stiffness(ems_sim *sim, const double *u, double *f, size_t n);
/* The same f = K u for callers that cannot allocate device memory (their
 * device memory belongs to another allocator, or they run in loops where
 * cudaMalloc/cudaFree must not occur): FP32, on device arrays u and f of
 * 7*(nx+1)(ny+1)(nz+1) floats owned by the caller, enqueued on `stream`
 * (a cudaStream_t; NULL = the default stream).  This entry point has no
 * counterpart in the reference.  It allocates nothing: the per-tetrahedron
 * scratch is a fixed file-scope device array of 2^20 tetrahedra x 3 floats
 * (12 MiB, held on every device that loads the library until exit); larger
 * meshes are rejected with EMS_ERR_INVALID_ARGUMENT.  The first call on a
 * device looks up the scratch address for that device (make that first call
 * before any stream capture); the address is kept until the process exits,
 * so do not call this entry point on a device after a cudaDeviceReset of it.  Every call shares the one scratch array, so
 * calls that overlap on the GPU race; the scratch is fully overwritten before
 * it is read, so nothing needs clearing between calls.  Errors are reported
 * through ems_last_error(NULL). */
int ems_tet_stiffness_apply_static(const int cells[3], const float *u, float *f, void *stream);

/* Batch of independent shots (configurations that differ in mesh size,
 * material, source and receivers) advanced together: shot s is a cube of
 * cells[3s..3s+2] cells split into tetrahedra; all shots share the time step
 * (with dt == 0, cfl_fraction x the stability limit of the stiffest shot).
 * Fields, materials (ems_tetfem_set_material) and edge-slot vectors are the
 * shots' arrays concatenated in shot order.  New: the reference runs one
 * configuration per process. */
int ems_tetbatch_create(const ems_tetfem_params *params, int nshots, const int *cells, ems_sim **out);
int ems_tetbatch_add_dipole(ems_sim *sim, int shot, const double pos[3], const double dir[3], int waveform, double f0,
                            double amplitude);
int ems_tetbatch_add_receiver(ems_sim *sim, int shot, const double pos[3]);

/* ------------------------------------------------ misfit gradient (adjoint)
 * New: the reference has no adjoint.  The gradient of a receiver-trace
 * functional J with respect to the per-tetrahedron permittivity comes from
 * the discrete adjoint of the symplectic time loop (EMS_SYMP2, EMS_SYMP4):
 *   ems_tetfem_set_checkpoints(sim, nsnap); ems_reset(sim); ems_run(sim, n);
 *   ... dJ/dtraces from the traces (ems_trace_misfit or the caller) ...
 *   ems_tetfem_backward(sim, dJ_dtraces, len, grad_eps, ntet);
 * The recorded run keeps nsnap snapshots of the state on the device (one per
 * segment of ceil(n / nsnap) steps); the backward sweep recomputes each
 * segment from its snapshot and runs the reversed steps over it.  Fields are
 * in the handle's precision; the gradient is accumulated in FP64 (the
 * products of four time steps are summed in the field precision first).
 * Works on batch handles too (one gradient value per tetrahedron of every
 * shot). */
/* Discrete energy H = 1/2 P.Minv P + 1/2 U.K U of the current state of a
 * symplectic run (EMS_SYMP2, EMS_SYMP4), the quantity those integrators
 * keep bounded without drift; computed in FP64 on the GPU from the run's
 * fields and mass blocks.  One value per shot (nshots = 1 for
 * ems_create_tetfem handles).  New: the reference has no energy check.
 * EMS_ERR_UNSUPPORTED for EMS_LEAPFROG. */
int ems_tetfem_energy(ems_sim *sim, double *energy, int nshots);


/* Record the next ems_run that starts from the reset state (nsnap > 0), or
 * stop recording (nsnap = 0).  EMS_ERR_UNSUPPORTED for EMS_LEAPFROG. */
int ems_tetfem_set_checkpoints(ems_sim *sim, int nsnap);
/* dJ/deps_r and, when grad_sigma is not NULL, dJ/dsigma (per S/m) per
 * tetrahedron (ntet values each) of the recorded run, given dJ/dtraces in
 * the layout of ems_get_traces (nobs x nsamp x 4, column 0, the time,
 * ignored; n = nobs * nsamp * 4).  EMS_ERR_STATE when there is no recorded
 * run (or the material, dipoles or receivers changed since). */
int ems_tetfem_backward(ems_sim *sim, const double *trace_grad, size_t n, double *grad_eps, double *grad_sigma,
                        size_t ntet);

/* The whole gradient in one call (the pipeline above with ems_trace_misfit):
 * reset, record nsteps steps with nsnap snapshots, misfit of the traces
 * against `observed` (nobs x nsamp x 4), dJ/deps_r into grad_eps and, when
 * not NULL, dJ/dsigma into grad_sigma (ntet each).  The fields end in the
 * state after the forward run. */
int ems_tetfem_gradient(ems_sim *sim, int nsteps, int nsnap, int misfit_kind, const double *observed,
                        const double *tf_band, double *misfit, double *grad_eps, double *grad_sigma, size_t ntet);

enum {
    EMS_MISFIT_L2 = 0,          /* J = 1/2 sum (E - E_obs)^2 over receivers, samples, components */
    EMS_MISFIT_TF_ENVELOPE = 1, /* single-valued time-frequency envelope misfit EM (Kristekova et al. 2006) */
    EMS_MISFIT_TF_PHASE = 2     /* single-valued time-frequency phase misfit PM (same paper) */
};
/* Misfit of traces against observed traces (both nobs x nsamp x 4 in the
 * ems_get_traces layout; column 0 holds the sample times) and its gradient
 * with respect to the traces (same layout, column 0 zero; may be NULL).
 * EMS_MISFIT_TF_ENVELOPE / _PHASE: J = 1/2 sum of EM^2 / PM^2 over receivers
 * and components, EM / PM the single-valued envelope / phase misfit with the
 * observed trace as reference
 * (TF_MISFIT_GOF's IS_S2_REFERENCE = T, LOCAL_NORM = F, one component per
 * pair); tf_band = {fmin, fmax, nf} in the units of the time column (NULL:
 * 4/T .. 1/(4 dt), 32 log-spaced frequencies); ignored for EMS_MISFIT_L2. */
int ems_trace_misfit(int kind, int nobs, int nsamp, const double *traces, const double *observed, const double *tf_band,
                     double *misfit, double *trace_grad);

/* ------------------------------------------------------ common operations */
/* Replaces FemSimulation::run (fdtd :242-306, fem_v2 :1249-1320,
 * symplectic_2/4 :1278-1351): advance num_steps steps, recording receivers.
 * Blocks until the device work has finished. */
int ems_run(ems_sim *sim, int num_steps);
/* Trace table written by the last ems_run: nobs receivers x nsamp samples x
 * ncols columns (FDTD: Ex,Ey,Ez; FEM: t,Ex,Ey,Ez). */
int ems_trace_shape(const ems_sim *sim, int *nobs, int *nsamp, int *ncols);
int ems_get_traces(const ems_sim *sim, double *out, size_t n);
/* Replaces saveResults (fdtd :308-331 names results_<i>_<dt>_<h>_<N>.csv;
 * fem_v2 :1322-1344 writes the given file name, one file per receiver with
 * suffix _<i> when there is more than one). */
int ems_save_results(const ems_sim *sim, const char *path);
/* One component (0 = x, 1 = y, 2 = z) of one receiver of the last run as the
 * `t,u` CSV that TF_MISFIT_GOF_master/main.py:6-40 converts for the
 * third-party misfit program (header t,u; 15 significant digits). */
int ems_save_trace_component(const ems_sim *sim, int receiver, int component, const char *path);
/* Field access in the reference layout, converted to/from double.
 * FDTD: which 0..5 = Ex,Ey,Ez,Hx,Hy,Hz.  Hex FEM: which 0..2 = component
 * x,y,z (all levels).  Tet FEM: 0 = U (edge values), 1 = P. */
int ems_field_size(const ems_sim *sim, int which, size_t *n);
int ems_get_field(const ems_sim *sim, int which, double *out, size_t n);
int ems_set_field(ems_sim *sim, int which, const double *in, size_t n);
/* Device time of the last ems_run [ms] and the number of kernel launches it
 * made; the average device time of one launch of the dominant kernel, timed
 * by CUDA events on the handle's stream over `launches` repeated launches on
 * the current state (fields are restored afterwards). */
int ems_last_run_stats(const ems_sim *sim, double *device_ms, long long *launches);
int ems_time_dominant_kernel(ems_sim *sim, int launches, double *ms_per_launch, double *bytes_per_launch,
                             char *name, size_t name_cap);
/* Threads per block (x, y, z) of the main time-step kernels as the handle's
 * autotuner chose them by timing candidates on its own grid: tetrahedral
 * handles time the node kernel at 32, 64, 128, 256 threads, the slot-split
 * kernel (block 32 x 7: one warp per edge direction of 32 nodes) and the
 * persistent step (the same block; 12 steps per cooperative launch with grid
 * barriers between substeps, for symplectic lossless runs whose grid fits on
 * the device at once; ems_time_dominant_kernel names it) inside their first
 * unrecorded run of at least 156 steps (EMS_TET_STEP_BLOCK = 32, 64, 128,
 * 256, slot or persist forces one); FDTD handles time the shapes 32x8, 32x4,
 * 64x4, 128x2, 256x1, 64x2 on the first steps of their first run of at
 * least 40 steps (EMS_FDTD_BLOCK="XxY" forces one; 32x8 before tuning).
 * Launch shapes change no result.  Zeros for solvers with fixed shapes.
 * New: the reference has fixed OpenACC launch shapes. */
int ems_launch_shape(ems_sim *sim, int block[3]);
/* Zero every field level and rewind the simulation clock to t = 0, keeping
 * mesh, materials, sources and receivers: the state a freshly constructed
 * reference FemSimulation starts from. */
int ems_reset(ems_sim *sim);
int ems_destroy(ems_sim *sim);

#ifdef __cplusplus
}
#endif
#endif
