"""Error statuses produced by runs: EMS_ERR_NOT_FINITE when the fields hold
a NaN or an Inf after ems_run (an unstable or corrupted run), with the run's
traces still readable; finite runs return EMS_OK."""
import numpy as np
import pytest

import golden_io
import oracle
import emsolvers_gb300 as ems

pytestmark = pytest.mark.gpu
NOT_FINITE = -7


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
