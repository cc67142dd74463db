// C ABI entry points of libems (declared in include/ems.h).  Every function
// converts internal exceptions into a status code and keeps the message on
// the handle (or in a thread-local slot for calls that have no handle yet).
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>

#include "ems_internal.hpp"

using ems::Error;
using ems::Sim;

static thread_local std::string g_create_error;

namespace ems {
// Message for calls that have no handle; read back with ems_last_error(NULL).
void record_error(const std::string &msg) { g_create_error = msg; }
}  // namespace ems

template <class F> static int guard(ems_sim *s, F &&f)
{
    try {
        f();
        if (s) s->impl->last_error.clear();
        return EMS_OK;
    } catch (const Error &e) {
        if (s) s->impl->last_error = e.msg; else g_create_error = e.msg;
        return e.code;
    } catch (const std::bad_alloc &) {
        if (s) s->impl->last_error = "host allocation failed"; else g_create_error = "host allocation failed";
        return EMS_ERR_OUT_OF_MEMORY;
    } catch (const std::exception &e) {
        if (s) s->impl->last_error = e.what(); else g_create_error = e.what();
        return EMS_ERR_INVALID_ARGUMENT;
    }
}

template <class Mk> static int create(ems_sim **out, Mk &&mk)
{
    if (!out) return EMS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(nullptr, [&] {
        Sim *impl = mk();
        ems_sim *h = new ems_sim{impl};
        *out = h;
    });
}

#define NEED(s, k)                                                                                 \
    do {                                                                                           \
        if (!(s)) return EMS_ERR_INVALID_ARGUMENT;                                                 \
        if ((s)->impl->kind != (k)) {                                                              \
            (s)->impl->last_error = "handle is of a different solver kind";                       \
            return EMS_ERR_STATE;                                                                  \
        }                                                                                          \
    } while (0)

extern "C" {

int ems_abi_version(void) { return EMS_ABI_VERSION; }

const char *ems_status_string(int st)
{
    switch (st) {
    case EMS_OK: return "ok";
    case EMS_ERR_INVALID_ARGUMENT: return "invalid argument";
    case EMS_ERR_CUDA: return "CUDA error";
    case EMS_ERR_OUT_OF_MEMORY: return "out of memory";
    case EMS_ERR_IO: return "I/O error";
    case EMS_ERR_STATE: return "invalid state";
    case EMS_ERR_DEVICE_TIMEOUT: return "device wait timed out";
    case EMS_ERR_NOT_FINITE: return "non-finite values";
    case EMS_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
    }
}

const char *ems_last_error(const ems_sim *s) { return s ? s->impl->last_error.c_str() : g_create_error.c_str(); }

int ems_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int ems_fdtd_create(const ems_fdtd_params *p, ems_sim **out)
{
    if (!p) return EMS_ERR_INVALID_ARGUMENT;
    return create(out, [&] { return ems::make_fdtd(p); });
}
int ems_fdtd_set_source(ems_sim *s, int comp, const int ijk[3], int wf, double f0, double amp)
{
    NEED(s, ems::Kind::FDTD);
    return guard(s, [&] { ems::fdtd_set_source(s->impl, comp, ijk, wf, f0, amp); });
}
int ems_fdtd_add_observation(ems_sim *s, const int *x, int nx, const int *y, int ny, const int *z, int nz)
{
    NEED(s, ems::Kind::FDTD);
    return guard(s, [&] { ems::fdtd_add_observation(s->impl, x, nx, y, ny, z, nz); });
}
int ems_fdtd_set_material(ems_sim *s, const double *eps, const double *sigma)
{
    NEED(s, ems::Kind::FDTD);
    return guard(s, [&] { ems::fdtd_set_material(s->impl, eps, sigma); });
}

int ems_hexfem_create(const ems_hexfem_params *p, ems_sim **out)
{
    if (!p) return EMS_ERR_INVALID_ARGUMENT;
    return create(out, [&] { return p->integrator == EMS_ABM ? ems::make_abm(p) : ems::make_hexfem(p); });
}
int ems_hexfem_set_source(ems_sim *s, int comp, const int ijk[3])
{
    NEED(s, ems::Kind::HEXFEM);
    return guard(s, [&] {
        if (comp < 0 || comp > 2 || !ijk) throw Error{EMS_ERR_INVALID_ARGUMENT, "component must be 0, 1 or 2"};
        if (ems::is_abm(s->impl)) ems::abm_set_source(s->impl, comp, ijk);
        else if (ems::is_femstab(s->impl)) ems::femstab_set_source(s->impl, comp, ijk);
        else ems::hexfem_set_source(s->impl, comp, ijk);
    });
}
int ems_hexfem_add_observation(ems_sim *s, const int ijk[3])
{
    NEED(s, ems::Kind::HEXFEM);
    return guard(s, [&] {
        if (ems::is_abm(s->impl) || ems::is_femstab(s->impl))
            throw Error{EMS_ERR_STATE, "this solver's receivers take edge lists (ems_hexfem_add_observation_edges)"};
        ems::hexfem_add_observation(s->impl, ijk);
    });
}
int ems_hexfem_add_dipole(ems_sim *s, const int ijk[3])
{
    NEED(s, ems::Kind::HEXFEM);
    return guard(s, [&] {
        if (ems::is_femstab(s->impl)) ems::femstab_add_dipole(s->impl, ijk);
        else if (ems::is_abm(s->impl)) ems::abm_add_dipole(s->impl, ijk);
        else throw Error{EMS_ERR_STATE, "Hertz dipoles belong to the Adams-Bashforth-Moulton and fem/ solvers"};
    });
}
int ems_hexfem_add_observation_edges(ems_sim *s, const int *x, int nx, const int *y, int ny, const int *z, int nz)
{
    NEED(s, ems::Kind::HEXFEM);
    return guard(s, [&] {
        if (ems::is_femstab(s->impl)) ems::femstab_add_observation(s->impl, x, nx, y, ny, z, nz);
        else if (ems::is_abm(s->impl)) ems::abm_add_observation(s->impl, x, nx, y, ny, z, nz);
        else throw Error{EMS_ERR_STATE, "edge-list receivers belong to the Adams-Bashforth-Moulton and fem/ solvers"};
    });
}

int ems_femstab_create(const ems_femstab_params *p, ems_sim **out)
{
    if (!p) return EMS_ERR_INVALID_ARGUMENT;
    return create(out, [&] { return ems::make_femstab(p); });
}
int ems_femstab_element_matrix(const ems_sim *s, double *K, size_t n)
{
    if (!s) return EMS_ERR_INVALID_ARGUMENT;
    auto *m = const_cast<ems_sim *>(s);
    return guard(m, [&] {
        if (!ems::is_femstab(s->impl)) throw Error{EMS_ERR_STATE, "handle is not a fem/ (ems_femstab_create) solver"};
        EMS_CHECK_ARG(K != nullptr && n == 144, "K must hold 144 values");
        ems::femstab_element_matrix(s->impl, K);
    });
}

int ems_tetfem_element_matrices(int order, int type, double *M, double *K, size_t n)
{
    return guard(nullptr, [&] {
        if (order != 2) throw Error{EMS_ERR_UNSUPPORTED, "element matrices are defined for order-2 tetrahedra"};
        EMS_CHECK_ARG(M != nullptr && K != nullptr && n == 400, "M and K must hold 400 values each");
        ems::tet2_element_matrices(type, M, K);
    });
}

int ems_tetfem_create(const ems_tetfem_params *p, ems_sim **out)
{
    if (!p) return EMS_ERR_INVALID_ARGUMENT;
    return create(out, [&] { return ems::make_tetfem(p); });
}
int ems_tetbatch_create(const ems_tetfem_params *p, int nshots, const int *cells, ems_sim **out)
{
    if (!p) return EMS_ERR_INVALID_ARGUMENT;
    return create(out, [&] { return ems::make_tetbatch(p, nshots, cells); });
}
int ems_tetbatch_add_dipole(ems_sim *s, int shot, const double pos[3], const double dir[3], int wf, double f0, double amp)
{
    NEED(s, ems::Kind::TETFEM);
    return guard(s, [&] { ems::tetbatch_add_dipole(s->impl, shot, pos, dir, wf, f0, amp); });
}
int ems_tetbatch_add_receiver(ems_sim *s, int shot, const double pos[3])
{
    NEED(s, ems::Kind::TETFEM);
    return guard(s, [&] { ems::tetbatch_add_receiver(s->impl, shot, pos); });
}
int ems_tetfem_set_material(ems_sim *s, const double *eps_r, const double *sigma)
{
    NEED(s, ems::Kind::TETFEM);
    return guard(s, [&] { ems::tetfem_set_material(s->impl, eps_r, sigma); });
}
int ems_tetfem_add_dipole(ems_sim *s, const double pos[3], const double dir[3], int wf, double f0, double amp)
{
    NEED(s, ems::Kind::TETFEM);
    return guard(s, [&] { ems::tetfem_add_dipole(s->impl, pos, dir, wf, f0, amp); });
}
int ems_tetfem_add_receiver(ems_sim *s, const double pos[3])
{
    NEED(s, ems::Kind::TETFEM);
    return guard(s, [&] { ems::tetfem_add_receiver(s->impl, pos); });
}
int ems_tetfem_time_step(const ems_sim *s, double *dt, double *lim)
{
    NEED(s, ems::Kind::TETFEM);
    return guard(const_cast<ems_sim *>(s), [&] { ems::tetfem_time_step(s->impl, dt, lim); });
}

int ems_tetfem_apply_stiffness(ems_sim *s, const double *u, double *f, size_t n)
{
    NEED(s, ems::Kind::TETFEM);
    return guard(s, [&] { ems::tetfem_apply_stiffness(s->impl, u, f, n); });
}

int ems_tetfem_set_checkpoints(ems_sim *s, int nsnap)
{
    NEED(s, ems::Kind::TETFEM);
    return guard(s, [&] { ems::tetfem_set_checkpoints(s->impl, nsnap); });
}
int ems_tetfem_energy(ems_sim *s, double *energy, int nshots)
{
    NEED(s, ems::Kind::TETFEM);
    return guard(s, [&] { ems::tetfem_energy(s->impl, energy, nshots); });
}
int ems_tetfem_backward(ems_sim *s, const double *tg, size_t n, double *grad, double *grad_sigma, size_t ntet)
{
    NEED(s, ems::Kind::TETFEM);
    return guard(s, [&] { ems::tetfem_backward(s->impl, tg, n, grad, grad_sigma, ntet); });
}
int ems_tetfem_gradient(ems_sim *s, int nsteps, int nsnap, int kind, const double *obs, const double *band, double *misfit,
                        double *grad, double *grad_sigma, size_t ntet)
{
    NEED(s, ems::Kind::TETFEM);
    return guard(s, [&] { ems::tetfem_gradient(s->impl, nsteps, nsnap, kind, obs, band, misfit, grad, grad_sigma, ntet); });
}
int ems_trace_misfit(int kind, int nobs, int nsamp, const double *tr, const double *obs, const double *band, double *misfit,
                     double *tg)
{
    return guard(nullptr, [&] { ems::trace_misfit(kind, nobs, nsamp, tr, obs, misfit, tg, band); });
}

int ems_run(ems_sim *s, int n)
{
    if (!s) return EMS_ERR_INVALID_ARGUMENT;
    return guard(s, [&] { s->impl->run(n); });
}
int ems_trace_shape(const ems_sim *s, int *nobs, int *nsamp, int *ncols)
{
    if (!s || !nobs || !nsamp || !ncols) return EMS_ERR_INVALID_ARGUMENT;
    *nobs = s->impl->nobs; *nsamp = s->impl->nsamp; *ncols = s->impl->ncols;
    return EMS_OK;
}
int ems_get_traces(const ems_sim *s, double *out, size_t n)
{
    if (!s || (!out && n)) return EMS_ERR_INVALID_ARGUMENT;
    const auto &t = s->impl->traces;
    if (n < t.size()) {
        s->impl->last_error = "output buffer too small for the trace table";
        return EMS_ERR_INVALID_ARGUMENT;
    }
    if (!t.empty()) std::memcpy(out, t.data(), t.size() * sizeof(double));
    return EMS_OK;
}
int ems_save_results(const ems_sim *s, const char *path)
{
    if (!s) return EMS_ERR_INVALID_ARGUMENT;
    return guard(const_cast<ems_sim *>(s), [&] { s->impl->save(path); });
}
int ems_save_trace_component(const ems_sim *s, int receiver, int component, const char *path)
{
    if (!s) return EMS_ERR_INVALID_ARGUMENT;
    return guard(const_cast<ems_sim *>(s), [&] { s->impl->save_component(receiver, component, path); });
}
int ems_field_size(const ems_sim *s, int which, size_t *n)
{
    if (!s || !n) return EMS_ERR_INVALID_ARGUMENT;
    return guard(const_cast<ems_sim *>(s), [&] { *n = s->impl->field_size(which); });
}
int ems_get_field(const ems_sim *s, int which, double *out, size_t n)
{
    if (!s || !out) return EMS_ERR_INVALID_ARGUMENT;
    return guard(const_cast<ems_sim *>(s), [&] {
        if (n < s->impl->field_size(which)) throw Error{EMS_ERR_INVALID_ARGUMENT, "output buffer too small"};
        s->impl->get_field(which, out);
    });
}
int ems_set_field(ems_sim *s, int which, const double *in, size_t n)
{
    if (!s || !in) return EMS_ERR_INVALID_ARGUMENT;
    return guard(s, [&] {
        if (n != s->impl->field_size(which)) throw Error{EMS_ERR_INVALID_ARGUMENT, "input size does not match the field"};
        s->impl->set_field(which, in);
    });
}
int ems_last_run_stats(const ems_sim *s, double *ms, long long *launches)
{
    if (!s || !ms || !launches) return EMS_ERR_INVALID_ARGUMENT;
    *ms = s->impl->last_ms;
    *launches = s->impl->last_launches;
    return EMS_OK;
}
int ems_time_dominant_kernel(ems_sim *s, int launches, double *ms, double *bytes, char *name, size_t cap)
{
    if (!s || !ms || !bytes || launches <= 0) return EMS_ERR_INVALID_ARGUMENT;
    return guard(s, [&] {
        std::string nm;
        s->impl->time_dominant(launches, ms, bytes, &nm);
        if (name && cap) {
            std::strncpy(name, nm.c_str(), cap - 1);
            name[cap - 1] = 0;
        }
    });
}
int ems_launch_shape(ems_sim *s, int block[3])
{
    if (!s || !block) return EMS_ERR_INVALID_ARGUMENT;
    return guard(s, [&] { s->impl->launch_shape(block); });
}
int ems_reset(ems_sim *s)
{
    if (!s) return EMS_ERR_INVALID_ARGUMENT;
    return guard(s, [&] { s->impl->reset(); });
}
int ems_destroy(ems_sim *s)
{
    if (!s) return EMS_OK;
    delete s->impl;
    delete s;
    return EMS_OK;
}

}  // extern "C"
