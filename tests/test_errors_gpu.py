"""Error statuses produced by runs: EMS_ERR_NOT_FINITE when the fields hold
a NaN or an Inf after ems_run (an unstable or corrupted run), with the run's
traces still readable; finite runs return EMS_OK.  EMS_ERR_DEVICE_TIMEOUT
when a grid barrier of the persistent step gives up its bounded wait (made
to run out on purpose: the barrier expects one block more than the grid
holds, a count that nothing reaches)."""
import os
import subprocess
import sys

import numpy as np
import pytest

import golden_io
import oracle
import emsolvers_gb300 as ems

pytestmark = pytest.mark.gpu
NOT_FINITE = -7
DEVICE_TIMEOUT = -6


def test_tetrahedral_run_from_huge_fields_reports_not_finite():
    # FP32 fields near the top of the float range: the first kick overflows
    n = (6, 5, 4)
    _, nslot, ntet = oracle.tet_sizes(n)
    pec = oracle.tet_pec_mask(n)
    s = ems.TetFemSimulation(n, 1e-3, 1, ems.SYMP4, ems.FP32, dt=0.0, cfl_fraction=0.9)
    s.set_material(np.full(ntet, 2.0))
    s.add_receiver(np.array([3.1, 2.4, 2.2]) * 1e-3)
    s.set_field(0, np.where(pec, 0.0, 3e38))
    with pytest.raises(ems.EmsError) as e:
        s.run(5)
    assert e.value.status == NOT_FINITE
    assert s.traces().shape == (1, 5, 4)
    # a fresh state runs clean again
    s.reset()
    s.run(5)


def test_order2_tetrahedral_run_from_huge_fields_reports_not_finite():
    n = (4, 4, 3)
    _, ndof, ntet = oracle.tet2_sizes(n)
    pec = oracle.tet2_pec_mask(n)
    s = ems.TetFemSimulation(n, 1e-3, 2, ems.SYMP4, ems.FP32, dt=0.0, cfl_fraction=0.9)
    s.set_material(np.full(ntet, 2.0))
    s.add_receiver(np.array([2.1, 1.4, 1.2]) * 1e-3)
    nnode = ndof // 38
    U = np.where(pec, 0.0, 3e38).reshape(38, nnode).T.reshape(-1)   # API order: 38 * node + plane
    s.set_field(0, U)
    with pytest.raises(ems.EmsError) as e:
        s.run(5)
    assert e.value.status == NOT_FINITE
    assert s.traces().shape == (1, 5, 4)
    s.reset()
    s.run(5)


def test_fdtd_run_with_a_nan_field_reports_not_finite():
    s = ems.FdtdSimulation((8, 8, 8), 1e-3, 1e-12, 8.854187817e-12, 1.25663706212e-6, 1)
    ez = s.get_field(2)
    ez[ez.size // 2] = np.nan
    s.set_field(2, ez)
    with pytest.raises(ems.EmsError) as e:
        s.run(3)
    assert e.value.status == NOT_FINITE


@pytest.mark.parametrize("case", list(golden_io.femstab_cases())[:1], ids=lambda c: c[0]["name"])
def test_femstab_and_abm_runs_report_not_finite(case):
    m = case[0]
    s = ems.FemStabSimulation(m["grid"], m["h"], m["dt"], m["eps"], m["mu"], m["tf"], m["stabilization"], m["use_ofem"])
    e1 = s.get_field(1)
    e1[len(e1) // 2] = np.inf
    s.set_field(1, e1)
    with pytest.raises(ems.EmsError) as e:
        s.run(2)
    assert e.value.status == NOT_FINITE
    a = ems.HexFemSimulation(1, (6, 6, 6), 0.1, 1e-10, 8.854187817e-12, 1.25663706212e-6, 1, 0, integrator=ems.ABM,
                             kmat_dir=golden_io.KMAT_DIR)
    h = a.get_field(4)
    h[h.size // 3] = np.nan
    a.set_field(4, h)
    with pytest.raises(ems.EmsError) as e:
        a.run(2)
    assert e.value.status == NOT_FINITE


_BARRIER_PROBE = (
    "import os, time, numpy as np, emsolvers_gb300 as ems\n"
    "os.environ['EMS_TET_STEP_BLOCK'] = 'persist'\n"
    "os.environ['EMS_TET_BARRIER_PROBE'] = '1'\n"
    "s = ems.TetFemSimulation((8, 8, 8), 1e-3, 1, ems.SYMP4, ems.FP32, dt=0.0, cfl_fraction=0.9)\n"
    "s.set_material(np.full(6 * 512, 2.0))\n"
    "s.add_dipole(np.array([4.1, 3.3, 4.2]) * 1e-3, (0.2, 0.3, 1.0), ems.WAVE_RICKER, 4e10, 1.0)\n"
    "s.add_receiver(np.array([3.1, 2.4, 2.2]) * 1e-3)\n"
    "t0 = time.perf_counter()\n"
    "try:\n"
    "    s.run(30)\n"
    "    status = 0\n"
    "except ems.EmsError as e:\n"
    "    status = e.status\n"
    "waited = time.perf_counter() - t0\n"
    "del os.environ['EMS_TET_BARRIER_PROBE']\n"
    "s.reset()\n"
    "s.run(30)\n"
    "tr = s.traces()\n"
    "print(status, waited, int(np.isfinite(tr).all()), float(np.abs(tr[..., 1:]).max()))\n")


def test_persistent_step_barrier_timeout_reports_device_timeout():
    # every block's wait gives up after 20 ms, the run returns
    # EMS_ERR_DEVICE_TIMEOUT, and the same handle, reset, runs again (the
    # context stays usable); a child process keeps the variables out of
    # this one
    env = dict(os.environ)
    env.pop("EMS_TET_BARRIER_PROBE", None)
    r = subprocess.run([sys.executable, "-c", _BARRIER_PROBE], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    status, waited, finite, peak = r.stdout.split()[-4:]
    assert int(status) == DEVICE_TIMEOUT
    assert float(waited) < 20.0
    assert int(finite) == 1 and float(peak) > 0.0
