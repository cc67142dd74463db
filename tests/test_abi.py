"""C-ABI checks that need no GPU: the library loads, exports every function
declared in include/ems.h, and rejects bad arguments before touching a
device (the reference's check_params and CSV errors, as status codes)."""
import ctypes as C

import pytest

import emsolvers_gb300 as ems
from emsolvers_gb300 import _lib

EPS0, MU0 = 8.854187817e-12, 1.25663706212e-6


def test_library_exports_every_declared_function():
    L = ems.lib()
    names = ems.declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert missing == []
    assert L.ems_abi_version() == 1


def test_status_strings():
    L = ems.lib()
    for st in (0, -1, -2, -3, -4, -5, -6, -7, -8):
        assert L.ems_status_string(st)


def _fdtd_status(**kw):
    p = _lib.FdtdParams()
    p.grid[:] = kw.get("grid", (8, 8, 8))
    p.h, p.dt = kw.get("h", 1e-3), kw.get("dt", 1e-12)
    p.permittivity, p.permeability = kw.get("eps", EPS0), kw.get("mu", MU0)
    p.time_frequency, p.precision = kw.get("tf", 1), kw.get("precision", 0)
    p.pml_cells = kw.get("pml", 0)
    h = C.c_void_p()
    st = ems.lib().ems_fdtd_create(C.byref(p), C.byref(h))
    if h:
        ems.lib().ems_destroy(h)
    return st


@pytest.mark.parametrize("kw", [dict(grid=(0, 8, 8)), dict(h=-1.0), dict(dt=0.0), dict(tf=0), dict(precision=7),
                                dict(dt=1e-9), dict(pml=4)])
def test_fdtd_create_rejects_bad_parameters(kw):
    assert _fdtd_status(**kw) == -1


def test_cfl_check_is_the_reference_condition():
    # fdtd_simulation.cpp:358 rejects c*dt >= h; accepts anything below
    c = 1 / (EPS0 * MU0) ** 0.5
    assert _fdtd_status(dt=1.0001e-3 / c) == -1
    st = _fdtd_status(dt=0.999e-3 / c)
    assert st in (0, -2)  # -2 only when no GPU is present


def test_hexfem_missing_kmat_is_io_error(tmp_path):
    p = _lib.HexFemParams()
    p.order, p.grid[:] = 1, (6, 6, 6)
    p.h, p.dt, p.permittivity, p.permeability = 0.1, 1e-10, EPS0, MU0
    p.time_frequency, p.use_ofem, p.integrator, p.precision = 2, 1, 0, 0
    p.kmat_dir = str(tmp_path).encode()
    h = C.c_void_p()
    assert ems.lib().ems_hexfem_create(C.byref(p), C.byref(h)) == -4
    assert b"cannot open" in ems.lib().ems_last_error(None)


def test_hexfem_malformed_kmat_is_io_error(tmp_path):
    (tmp_path / "1.csv").write_text('"1/2","x/3"\n')
    p = _lib.HexFemParams()
    p.order, p.grid[:] = 1, (6, 6, 6)
    p.h, p.dt, p.permittivity, p.permeability = 0.1, 1e-10, EPS0, MU0
    p.time_frequency, p.use_ofem, p.integrator, p.precision = 2, 1, 0, 0
    p.kmat_dir = str(tmp_path).encode()
    h = C.c_void_p()
    assert ems.lib().ems_hexfem_create(C.byref(p), C.byref(h)) == -4


def test_hexfem_too_few_elements_rejected():
    p = _lib.HexFemParams()
    p.order, p.grid[:] = 2, (2, 8, 8)
    p.h, p.dt, p.permittivity, p.permeability = 0.1, 1e-10, EPS0, MU0
    p.time_frequency, p.use_ofem, p.integrator, p.precision = 2, 1, 0, 0
    h = C.c_void_p()
    assert ems.lib().ems_hexfem_create(C.byref(p), C.byref(h)) == -1


def test_null_handles_are_rejected():
    L = ems.lib()
    assert L.ems_run(None, 1) == -1
    assert L.ems_destroy(None) == 0
