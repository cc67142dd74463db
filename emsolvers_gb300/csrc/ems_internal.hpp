// Internal declarations shared by the libems translation units.
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <cstdio>
#include <initializer_list>
#include <utility>
#include <type_traits>
#include <string>
#include <vector>

#include "../../include/ems.h"

namespace ems {

// Status carrier used inside the library; converted to int at the C ABI.
struct Error {
    int code;
    std::string msg;
};

#define EMS_CUDA(call)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) {                                                                    \
            if (e_ == cudaErrorMemoryAllocation)                                                    \
                throw ::ems::Error{EMS_ERR_OUT_OF_MEMORY, std::string(#call) + ": " + cudaGetErrorString(e_)}; \
            throw ::ems::Error{EMS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)};   \
        }                                                                                           \
    } while (0)

#define EMS_CHECK_ARG(cond, text)                                          \
    do {                                                                   \
        if (!(cond)) throw ::ems::Error{EMS_ERR_INVALID_ARGUMENT, (text)}; \
    } while (0)

// Device buffer owned by a simulation handle.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void alloc(size_t b);
    void ensure(size_t b);   // alloc(b) unless the buffer already holds exactly b bytes
    void zero(cudaStream_t s);
    void release();
    template <class T> T *as() const { return static_cast<T *>(p); }
};

enum class Kind { FDTD, HEXFEM, TETFEM };

// Base of every simulation handle (the opaque ems_sim of the C ABI).
struct Sim {
    Kind kind;
    std::string last_error;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0.0;
    long long last_launches = 0;
    int nobs = 0, nsamp = 0, ncols = 0;
    std::vector<double> traces;   // host copy of the last run's receiver table
    explicit Sim(Kind k) : kind(k) {}
    virtual ~Sim();
    void init_stream();
    virtual void run(int nsteps) = 0;
    virtual size_t field_size(int which) const = 0;
    virtual void get_field(int which, double *out) const = 0;
    virtual void set_field(int which, const double *in) = 0;
    virtual void save(const char *path) const = 0;
    virtual void time_dominant(int launches, double *ms, double *bytes, std::string *name) = 0;
    virtual void reset() = 0;
    // Threads per block (x, y, z) of the solver's main kernels as its
    // autotuner chose them; zeros where a solver has fixed shapes.
    virtual void launch_shape(int b[3]) { b[0] = b[1] = b[2] = 0; }
    // Time [s] of sample j of the last run (FEM tables carry it in column 0).
    virtual double sample_time(int j) const { return traces[(size_t)j * ncols]; }
    // One receiver component as the `t,u` CSV that
    // TF_MISFIT_GOF_master/main.py:6-40 reads.
    void save_component(int receiver, int component, const char *path) const;
    // Throws EMS_ERR_NOT_FINITE when one of the device arrays (pointer,
    // element count; FP64 or FP32) holds a NaN or an Inf.
    void check_finite(std::initializer_list<std::pair<const void *, size_t>> arrays, bool fp64);
    DevBuf d_finite;
};

// CSV element matrices in the reference format (fem_v2/fem_simulation.cpp:1477-1524).
double parse_value(const std::string &s);
std::vector<std::vector<double>> load_matrix_csv(const std::string &path);
// Reference file-name helper (fem_v2/fem_simulation.cpp:1446-1475).
std::string compress_number(double v);

Sim *make_fdtd(const ems_fdtd_params *p);
Sim *make_hexfem(const ems_hexfem_params *p);
Sim *make_tetfem(const ems_tetfem_params *p);
Sim *make_abm(const ems_hexfem_params *p);
Sim *make_tetbatch(const ems_tetfem_params *p, int nshots, const int *cells);
void tetbatch_add_dipole(Sim *s, int shot, const double pos[3], const double dir[3], int waveform, double f0, double amp);
void tetbatch_add_receiver(Sim *s, int shot, const double pos[3]);
bool is_abm(const Sim *s);
// second-order tetrahedra (tet2.cu)
Sim *make_tet2(const ems_tetfem_params *p, const std::vector<std::array<int, 3>> &cells);
bool is_tet2(const Sim *s);
void tet2_set_material(Sim *s, const double *eps_r, const double *sigma);
void tet2_add_dipole(Sim *s, int shot, const double pos[3], const double dir[3], int waveform, double f0, double amp);
void tet2_add_receiver(Sim *s, int shot, const double pos[3]);
void tet2_time_step(const Sim *s, double *dt, double *lim);
void tet2_apply_stiffness(Sim *s, const double *u, double *f, size_t n);
void tet2_energy(Sim *s, double *out, int n);
void tet2_set_checkpoints(Sim *s, int nsnap);
void tet2_backward(Sim *s, const double *trace_grad, size_t ntg, double *grad_eps, double *grad_sigma, size_t ngrad);
size_t tet2_ntet(const Sim *s);
void tet2_element_matrices(int type, double *M, double *K);
Sim *make_femstab(const ems_femstab_params *p);
bool is_femstab(const Sim *s);
void femstab_set_source(Sim *s, int comp, const int ijk[3]);
void femstab_add_dipole(Sim *s, const int ijk[3]);
void femstab_add_observation(Sim *s, const int *x, int nx, const int *y, int ny, const int *z, int nz);
void femstab_element_matrix(const Sim *s, double *K);
void abm_set_source(Sim *s, int comp, const int ijk[3]);
void abm_add_dipole(Sim *s, const int ijk[3]);
void abm_add_observation(Sim *s, const int *x, int nx, const int *y, int ny, const int *z, int nz);

// per-kind setters (throw Error on misuse)
void fdtd_set_source(Sim *s, int comp, const int ijk[3], int waveform, double f0, double amp);
void fdtd_add_observation(Sim *s, const int *x, int nx, const int *y, int ny, const int *z, int nz);
void fdtd_set_material(Sim *s, const double *eps, const double *sigma);
void hexfem_set_source(Sim *s, int comp, const int ijk[3]);
void hexfem_add_observation(Sim *s, const int ijk[3]);
void tetfem_set_material(Sim *s, const double *eps_r, const double *sigma);
void tetfem_add_dipole(Sim *s, const double pos[3], const double dir[3], int waveform, double f0, double amp);
void tetfem_add_receiver(Sim *s, const double pos[3]);
void tetfem_time_step(const Sim *s, double *dt, double *lim);
void tetfem_apply_stiffness(Sim *s, const double *u, double *f, size_t n);
void tetfem_set_checkpoints(Sim *s, int nsnap);
void tetfem_energy(Sim *s, double *out, int n);
void tetfem_backward(Sim *s, const double *trace_grad, size_t ntg, double *grad_eps, double *grad_sigma, size_t ngrad);
void tetfem_gradient(Sim *s, int nsteps, int nsnap, int kind, const double *observed, const double *tf_band, double *misfit,
                     double *grad_eps, double *grad_sigma, size_t ngrad);
void trace_misfit(int kind, int nobs, int nsamp, const double *traces, const double *observed, double *misfit,
                  double *trace_grad, const double *tf_band);

// Source waveforms evaluated on the host in FP64.
double fdtd_source_value(int kind, double f0, double t, double h);

}  // namespace ems

struct ems_sim {
    ems::Sim *impl;
};
