"""Python mirror of the reference solver classes, calling libems through its
C ABI.  Method names and argument meanings follow the reference's
``FemSimulation`` classes so scripts written against them read the same:

* :class:`FdtdSimulation`  — fdtd/fdtd_simulation.hpp:9-30
* :class:`HexFemSimulation` — fem_v2/fem_simulation.hpp:10-42 (with the
  integrator of symplectic_2 / symplectic_4 selectable)
* :class:`FemStabSimulation` — fem/fem_simulation.hpp:9-36 (stabilised
  order-1 hexahedra)
* :class:`TetFemSimulation` — tetrahedral Nedelec elements (new)
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import FP32, FP64, LEAPFROG, SYMP2, SYMP4, WAVE_REFERENCE, WAVE_RICKER, check, lib

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _dptr(a):
    return a.ctypes.data_as(_dp)


class _Sim:
    def __init__(self):
        self._h = C.c_void_p()

    def _check(self, st):
        check(st, self._h)

    def run(self, num_steps):
        """FemSimulation::run: advance num_steps steps, recording receivers."""
        self._check(lib().ems_run(self._h, int(num_steps)))

    def traces(self):
        """Receiver table of the last run: [nobs, nsamp, ncols]."""
        nobs, ns, nc = C.c_int(), C.c_int(), C.c_int()
        self._check(lib().ems_trace_shape(self._h, C.byref(nobs), C.byref(ns), C.byref(nc)))
        out = np.zeros(max(nobs.value * ns.value * nc.value, 1))
        self._check(lib().ems_get_traces(self._h, _dptr(out), out.size))
        return out[:nobs.value * ns.value * nc.value].reshape(nobs.value, ns.value, nc.value)

    def field_size(self, which):
        n = C.c_size_t()
        self._check(lib().ems_field_size(self._h, which, C.byref(n)))
        return n.value

    def get_field(self, which):
        out = np.zeros(self.field_size(which))
        self._check(lib().ems_get_field(self._h, which, _dptr(out), out.size))
        return out

    def set_field(self, which, values):
        a = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        self._check(lib().ems_set_field(self._h, which, _dptr(a), a.size))

    def save_component(self, receiver, component, path):
        """One receiver component as the `t,u` CSV read by the reference's
        TF_MISFIT_GOF_master/main.py."""
        self._check(lib().ems_save_trace_component(self._h, int(receiver), int(component), str(path).encode()))

    def launch_shape(self):
        """Threads per block (x, y, z) of the main kernels as the handle's
        autotuner chose them (zeros for fixed shapes)."""
        b = (C.c_int * 3)()
        self._check(lib().ems_launch_shape(self._h, b))
        return tuple(b)

    def run_stats(self):
        ms, n = C.c_double(), C.c_longlong()
        self._check(lib().ems_last_run_stats(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def time_dominant_kernel(self, launches=20):
        ms, b = C.c_double(), C.c_double()
        name = C.create_string_buffer(128)
        self._check(lib().ems_time_dominant_kernel(self._h, launches, C.byref(ms), C.byref(b), name, 128))
        return ms.value, b.value, name.value.decode()

    def reset(self):
        """Zero all fields and rewind time (a freshly constructed solver)."""
        self._check(lib().ems_reset(self._h))

    def close(self):
        if self._h:
            lib().ems_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class FdtdSimulation(_Sim):
    """fdtd/fdtd_simulation.hpp:13-14 constructor arguments; extra keywords
    select precision, a CPML and nothing else."""

    def __init__(self, grid_size, domain_size, time_step, permittivity, permeability, time_frequency,
                 precision=FP64, pml_cells=0, pml_order=3.0, pml_kappa_max=1.0, pml_alpha_max=0.0,
                 pml_reflection=1e-6):
        super().__init__()
        p = _lib.FdtdParams()
        p.grid[:] = list(grid_size)
        p.h, p.dt, p.permittivity, p.permeability = domain_size, time_step, permittivity, permeability
        p.time_frequency, p.precision = time_frequency, precision
        p.pml_cells, p.pml_order, p.pml_kappa_max = pml_cells, pml_order, pml_kappa_max
        p.pml_alpha_max, p.pml_reflection = pml_alpha_max, pml_reflection
        self.params = p
        check(lib().ems_fdtd_create(C.byref(p), C.byref(self._h)))

    def _src(self, comp, position, waveform, f0, amplitude):
        ijk = (C.c_int * 3)(*[int(v) for v in position])
        self._check(lib().ems_fdtd_set_source(self._h, comp, ijk, waveform, f0, amplitude))

    def setSource_x(self, position, waveform=WAVE_REFERENCE, f0=1.0e9, amplitude=1.0):
        self._src(0, position, waveform, f0, amplitude)

    def setSource_y(self, position, waveform=WAVE_REFERENCE, f0=1.0e9, amplitude=1.0):
        self._src(1, position, waveform, f0, amplitude)

    def setSource_z(self, position, waveform=WAVE_REFERENCE, f0=1.0e9, amplitude=1.0):
        self._src(2, position, waveform, f0, amplitude)

    def setObservationPoint(self, position):
        """position: three lists of (i,j,k) padded indices (Ex, Ey, Ez)."""
        arrs = [np.ascontiguousarray(np.array(l, np.int32).reshape(-1)) for l in position]
        ptrs = [a.ctypes.data_as(_ip) for a in arrs]
        self._check(lib().ems_fdtd_add_observation(self._h, ptrs[0], len(position[0]), ptrs[1], len(position[1]),
                                                   ptrs[2], len(position[2])))

    def set_material(self, eps, sigma=None):
        """Per-cell absolute permittivity and conductivity, arrays [nz,ny,nx]."""
        e = np.ascontiguousarray(eps, dtype=np.float64).reshape(-1)
        s = None if sigma is None else np.ascontiguousarray(sigma, dtype=np.float64).reshape(-1)
        self._check(lib().ems_fdtd_set_material(self._h, _dptr(e), _dptr(s) if s is not None else None))
        self._keep = (e, s)

    def fields(self):
        nx, ny, nz = self.params.grid
        shapes = [(nz + 2, ny + 2, nx + 1), (nz + 2, ny + 1, nx + 2), (nz + 1, ny + 2, nx + 2),
                  (nz + 1, ny + 1, nx), (nz + 1, ny, nx + 1), (nz, ny + 1, nx + 1)]
        return {n: self.get_field(q).reshape(s) for q, (n, s) in enumerate(zip(("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"), shapes))}

    def saveResults(self, num_steps=None, c=None, directory="."):
        """fdtd_simulation.cpp:308: results_<i>_<dt>_<h>_<N>.csv files."""
        self._check(lib().ems_save_results(self._h, directory.encode()))


class HexFemSimulation(_Sim):
    """fem_v2/fem_simulation.hpp:14-24 constructor (one subdomain: the MPI
    arguments are gone); ``integrator`` selects fem_v2 leapfrog or the
    symplectic_2 / symplectic_4 step."""

    def __init__(self, order, grid_size, domain_size, time_step, permittivity, permeability, time_frequency,
                 use_ofem, integrator=LEAPFROG, precision=FP64, kmat_dir="kmat"):
        super().__init__()
        p = _lib.HexFemParams()
        p.order = order
        p.grid[:] = list(grid_size)
        p.h, p.dt, p.permittivity, p.permeability = domain_size, time_step, permittivity, permeability
        p.time_frequency, p.use_ofem, p.integrator, p.precision = time_frequency, use_ofem, integrator, precision
        self._kdir = kmat_dir.encode()
        p.kmat_dir = self._kdir
        self.params = p
        check(lib().ems_hexfem_create(C.byref(p), C.byref(self._h)))

    def _src(self, comp, position):
        ijk = (C.c_int * 3)(*[int(v) for v in position])
        self._check(lib().ems_hexfem_set_source(self._h, comp, ijk))

    def setSource_x(self, position):
        self._src(0, position)

    def setSource_y(self, position):
        self._src(1, position)

    def setSource_z(self, position):
        self._src(2, position)

    def setObservationPoint(self, position):
        """fem_v2 family: a node (i, j, k).  Adams-Bashforth-Moulton
        (fem_abm): three lists of (i, j, k) edges of Ex, Ey and Ez."""
        if len(position) == 3 and all(np.isscalar(v) for v in position):
            ijk = (C.c_int * 3)(*[int(v) for v in position])
            self._check(lib().ems_hexfem_add_observation(self._h, ijk))
            return
        arrs = [np.ascontiguousarray(np.array(l, np.int32).reshape(-1)) for l in position]
        ptrs = [a.ctypes.data_as(_ip) for a in arrs]
        self._check(lib().ems_hexfem_add_observation_edges(self._h, ptrs[0], len(position[0]), ptrs[1], len(position[1]),
                                                           ptrs[2], len(position[2])))

    def setSourceDipole_x(self, position):
        """fem_abm setSourceDipole_x: Hertz dipole over cells (i, j..j+1, k..k+1)."""
        ijk = (C.c_int * 3)(*[int(v) for v in position])
        self._check(lib().ems_hexfem_add_dipole(self._h, ijk))

    def levels(self):
        return [self.get_field(q) for q in range(3)]

    def saveResults(self, num_steps, filename):
        self._check(lib().ems_save_results(self._h, filename.encode()))


class FemStabSimulation(_Sim):
    """fem/fem_simulation.hpp:12-14 constructor: the stabilised order-1
    hexahedral solver (conventional or OFEM basis, stabilisation factor s)."""

    def __init__(self, grid_size, domain_size, time_step, permittivity, permeability, time_frequency,
                 stabilization_factor, use_ofem, precision=FP64):
        super().__init__()
        p = _lib.FemStabParams()
        p.grid[:] = list(grid_size)
        p.h, p.dt, p.permittivity, p.permeability = domain_size, time_step, permittivity, permeability
        p.time_frequency, p.stabilization_factor = time_frequency, stabilization_factor
        p.use_ofem, p.precision = use_ofem, precision
        self.params = p
        check(lib().ems_femstab_create(C.byref(p), C.byref(self._h)))

    def _src(self, comp, position):
        ijk = (C.c_int * 3)(*[int(v) for v in position])
        self._check(lib().ems_hexfem_set_source(self._h, comp, ijk))

    def setSource_x(self, position):
        self._src(0, position)

    def setSource_y(self, position):
        self._src(1, position)

    def setSource_z(self, position):
        self._src(2, position)

    def setSourceDipole_x(self, position):
        """x-directed Hertz dipole over cells (i, j..j+1, k..k+1)."""
        ijk = (C.c_int * 3)(*[int(v) for v in position])
        self._check(lib().ems_hexfem_add_dipole(self._h, ijk))

    def setObservationPoint(self, position):
        """Three lists of (i, j, k) edges of Ex, Ey and Ez, averaged."""
        arrs = [np.ascontiguousarray(np.array(l, np.int32).reshape(-1)) for l in position]
        ptrs = [a.ctypes.data_as(_ip) for a in arrs]
        self._check(lib().ems_hexfem_add_observation_edges(self._h, ptrs[0], len(position[0]), ptrs[1], len(position[1]),
                                                           ptrs[2], len(position[2])))

    def element_matrix(self):
        """The element matrix K (12 x 12) of the handle."""
        K = np.zeros(144)
        self._check(lib().ems_femstab_element_matrix(self._h, _dptr(K), K.size))
        return K.reshape(12, 12)

    def saveResults(self, num_steps, filename):
        self._check(lib().ems_save_results(self._h, filename.encode()))


class TetFemSimulation(_Sim):
    """Structured cube of cells x 6 tetrahedra, Nedelec elements of order 1
    (Whitney, one DOF per edge, fields of 7*(n+1)^3 values in the order
    7*node + direction) or 2 (two DOFs per edge and per face, 38*(n+1)^3
    values in the order 38*node + plane; no conductivity)."""

    def __init__(self, cells, h, order=1, integrator=SYMP2, precision=FP32, dt=0.0, cfl_fraction=0.9,
                 time_frequency=1):
        super().__init__()
        p = _lib.TetFemParams()
        p.cells[:] = list(cells)
        p.h, p.order, p.integrator, p.precision = h, order, integrator, precision
        p.dt, p.cfl_fraction, p.time_frequency = dt, cfl_fraction, time_frequency
        self.params = p
        check(lib().ems_tetfem_create(C.byref(p), C.byref(self._h)))

    def set_material(self, eps_r, sigma=None):
        e = np.ascontiguousarray(eps_r, dtype=np.float64).reshape(-1)
        s = None if sigma is None else np.ascontiguousarray(sigma, dtype=np.float64).reshape(-1)
        self._check(lib().ems_tetfem_set_material(self._h, _dptr(e), _dptr(s) if s is not None else None))

    def add_dipole(self, pos, direction=(0.0, 0.0, 1.0), waveform=WAVE_RICKER, f0=1.0, amplitude=1.0):
        a = np.ascontiguousarray(pos, dtype=np.float64)
        d = np.ascontiguousarray(direction, dtype=np.float64)
        self._check(lib().ems_tetfem_add_dipole(self._h, _dptr(a), _dptr(d), waveform, f0, amplitude))

    def add_receiver(self, pos):
        a = np.ascontiguousarray(pos, dtype=np.float64)
        self._check(lib().ems_tetfem_add_receiver(self._h, _dptr(a)))

    def apply_stiffness(self, u):
        """f = K u on edge-slot vectors (normalised units)."""
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        f = np.zeros_like(u)
        self._check(lib().ems_tetfem_apply_stiffness(self._h, _dptr(u), _dptr(f), u.size))
        return f

    def time_step(self):
        dt, lim = C.c_double(), C.c_double()
        self._check(lib().ems_tetfem_time_step(self._h, C.byref(dt), C.byref(lim)))
        return dt.value, lim.value

    def set_checkpoints(self, nsnap):
        """Record the next run from the reset state for :meth:`backward`,
        keeping nsnap snapshots on the device (0 stops recording)."""
        self._check(lib().ems_tetfem_set_checkpoints(self._h, int(nsnap)))

    def energy(self):
        """Discrete energy 1/2 P.Minv P + 1/2 U.K U of the current symplectic
        state, per shot (FP64, computed on the GPU); a float for a single
        shot, an array for a batch."""
        n = len(self._cells())
        out = np.zeros(n)
        self._check(lib().ems_tetfem_energy(self._h, _dptr(out), n))
        return out if isinstance(self, TetFemBatch) else float(out[0])

    def backward(self, trace_grad, sigma=False):
        """dJ/deps_r per tetrahedron (FP64) of the recorded run, given
        dJ/dtraces shaped like :meth:`traces` (column 0 ignored); with
        sigma=True the pair (dJ/deps_r, dJ/dsigma per S/m)."""
        g = np.ascontiguousarray(trace_grad, dtype=np.float64).reshape(-1)
        out = np.zeros(self.ntet)
        gs = np.zeros(self.ntet) if sigma else None
        self._check(lib().ems_tetfem_backward(self._h, _dptr(g), g.size, _dptr(out),
                                              _dptr(gs) if sigma else None, out.size))
        return (out, gs) if sigma else out

    def gradient(self, nsteps, observed, kind=0, nsnap=64, tf_band=None, sigma=False):
        """Misfit J of an nsteps run from the reset state against `observed`
        traces and dJ/deps_r per tetrahedron (one call of ems_tetfem_gradient);
        with sigma=True, (J, dJ/deps_r, dJ/dsigma)."""
        ob = np.ascontiguousarray(observed, dtype=np.float64)
        band = None if tf_band is None else np.ascontiguousarray(tf_band, dtype=np.float64)
        J = C.c_double()
        out = np.zeros(self.ntet)
        gs = np.zeros(self.ntet) if sigma else None
        self._check(lib().ems_tetfem_gradient(self._h, int(nsteps), int(nsnap), int(kind), _dptr(ob),
                                              _dptr(band) if band is not None else None, C.byref(J), _dptr(out),
                                              _dptr(gs) if sigma else None, out.size))
        return (J.value, out, gs) if sigma else (J.value, out)

    @property
    def ntet(self):
        return sum(6 * c[0] * c[1] * c[2] for c in self._cells())

    def _cells(self):
        return [tuple(self.params.cells)]


class TetFemBatch(TetFemSimulation):
    """Independent shots (cubes of cells[s] cells) advanced together by the
    same kernels; materials and fields are the shots' arrays concatenated."""

    def __init__(self, cells, h, order=1, integrator=SYMP4, precision=FP32, dt=0.0, cfl_fraction=0.9,
                 time_frequency=1):
        _Sim.__init__(self)
        p = _lib.TetFemParams()
        p.cells[:] = list(cells[0])
        p.h, p.order, p.integrator, p.precision = h, order, integrator, precision
        p.dt, p.cfl_fraction, p.time_frequency = dt, cfl_fraction, time_frequency
        self.params = p
        flat = np.ascontiguousarray(np.array(cells, np.int32).reshape(-1))
        self.cells = [tuple(c) for c in cells]
        check(lib().ems_tetbatch_create(C.byref(p), len(cells), flat.ctypes.data_as(_ip), C.byref(self._h)))

    def add_dipole(self, shot, pos, direction=(0.0, 0.0, 1.0), waveform=WAVE_RICKER, f0=1.0, amplitude=1.0):
        a = np.ascontiguousarray(pos, dtype=np.float64)
        d = np.ascontiguousarray(direction, dtype=np.float64)
        self._check(lib().ems_tetbatch_add_dipole(self._h, shot, _dptr(a), _dptr(d), waveform, f0, amplitude))

    def add_receiver(self, shot, pos):
        a = np.ascontiguousarray(pos, dtype=np.float64)
        self._check(lib().ems_tetbatch_add_receiver(self._h, shot, _dptr(a)))

    def _cells(self):
        return self.cells


MISFIT_L2, MISFIT_TF_ENVELOPE, MISFIT_TF_PHASE = 0, 1, 2


def tet_element_matrices(order, ptype):
    """(M, K) of the second-order tetrahedron of Kuhn type ptype (20 x 20,
    eps = mu = 1) as the solver computes them."""
    M, K = np.zeros(400), np.zeros(400)
    check(lib().ems_tetfem_element_matrices(int(order), int(ptype), _dptr(M), _dptr(K), 400))
    return M.reshape(20, 20), K.reshape(20, 20)


def trace_misfit(traces, observed, kind=MISFIT_L2, tf_band=None):
    """Misfit J of traces against observed traces (both [nobs, nsamp, 4] as
    returned by ``traces()``) and dJ/dtraces (same shape, column 0 zero).
    kind: MISFIT_L2 (1/2 sum of squared differences), MISFIT_TF_ENVELOPE or
    MISFIT_TF_PHASE (1/2 sum of squared single-valued TF envelope / phase
    misfits, Kristekova et al. 2006); tf_band = (fmin, fmax, nf) in the units
    of the time column."""
    tr = np.ascontiguousarray(traces, dtype=np.float64)
    ob = np.ascontiguousarray(observed, dtype=np.float64)
    if tr.shape != ob.shape or tr.ndim != 3 or tr.shape[2] != 4:
        raise ValueError("traces and observed must both be [nobs, nsamp, 4]")
    g = np.zeros_like(tr)
    J = C.c_double()
    band = None if tf_band is None else np.ascontiguousarray(tf_band, dtype=np.float64)
    check(lib().ems_trace_misfit(kind, tr.shape[0], tr.shape[1], _dptr(tr), _dptr(ob),
                                 _dptr(band) if band is not None else None, C.byref(J), _dptr(g)))
    return J.value, g
