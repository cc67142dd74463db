"""Adams-Bashforth-Moulton hexahedral solver (fem_abm) on the GPU through the
C ABI: FP64 bit-identical to the reference fixtures (traces, every E and H
level); FP32 within relative L2 1e-4 of them on traces and E."""
import numpy as np
import pytest

import golden_io
from gpu_util import rel_l2
import emsolvers_gb300 as ems

pytestmark = pytest.mark.gpu


def _run(m, precision):
    s = ems.HexFemSimulation(1, m["grid"], m["h"], m["dt"], m["eps"], m["mu"], m["tf"], 0, integrator=ems.ABM,
                             precision=precision, kmat_dir=golden_io.KMAT_DIR)
    for c, p in m["sources"]:
        [s.setSource_x, s.setSource_y, s.setSource_z][c](p)
    for d in m["dipoles"]:
        s.setSourceDipole_x(d)
    for o in m["observations"]:
        s.setObservationPoint(o)
    s.run(m["nsteps"])
    return s


@pytest.mark.parametrize("case", list(golden_io.abm_cases()), ids=lambda c: c[0]["name"])
def test_fp64_bitwise_equal_to_reference(case):
    m, tr, E, H = case
    s = _run(m, ems.FP64)
    np.testing.assert_array_equal(s.traces(), tr)
    for q in range(3):
        np.testing.assert_array_equal(s.get_field(q), E[q])
        np.testing.assert_array_equal(s.get_field(3 + q), H[q])


@pytest.mark.parametrize("case", list(golden_io.abm_cases()), ids=lambda c: c[0]["name"])
def test_fp32_within_tolerance(case):
    m, tr, E, H = case
    s = _run(m, ems.FP32)
    assert rel_l2(s.traces(), tr) < 1e-4
    num = sum(np.sum((s.get_field(q) - E[q]) ** 2) for q in range(3))
    den = sum(np.sum(E[q] ** 2) for q in range(3))
    assert np.sqrt(num / den) < 1e-4


def test_abm_rejects_fem_v2_receivers():
    m, _, _, _ = next(iter(golden_io.abm_cases()))
    s = ems.HexFemSimulation(1, m["grid"], m["h"], m["dt"], m["eps"], m["mu"], m["tf"], 0, integrator=ems.ABM,
                             kmat_dir=golden_io.KMAT_DIR)
    with pytest.raises(ems.EmsError) as e:
        s.setObservationPoint((3, 3, 3))
    assert e.value.status == -5
