"""Stabilised order-1 hexahedral solver (the reference's fem/) on the GPU
through the C ABI: the element matrix and the FP64 traces and E levels are
bit-identical to the reference fixtures (conventional and OFEM bases,
stabilisation factors 0, 0.1 and 0.3); FP32 within relative L2 1e-4 of
them on traces and fields."""
import ctypes as C
import os

import numpy as np
import pytest

import golden_io
from gpu_util import rel_l2
import emsolvers_gb300 as ems

pytestmark = pytest.mark.gpu


def _run(m, precision):
    s = ems.FemStabSimulation(m["grid"], m["h"], m["dt"], m["eps"], m["mu"], m["tf"], m["stabilization"], m["use_ofem"],
                              precision=precision)
    for c, p in m["sources"]:
        [s.setSource_x, s.setSource_y, s.setSource_z][c](p)
    for d in m["dipoles"]:
        s.setSourceDipole_x(d)
    for o in m["observations"]:
        s.setObservationPoint(o)
    s.run(m["nsteps"])
    return s


@pytest.mark.parametrize("case", list(golden_io.femstab_cases()), ids=lambda c: c[0]["name"])
def test_fp64_bitwise_equal_to_reference(case):
    m, tr, E, K = case
    s = _run(m, ems.FP64)
    np.testing.assert_array_equal(s.element_matrix(), K)
    np.testing.assert_array_equal(s.traces(), tr)
    for q in range(3):
        np.testing.assert_array_equal(s.get_field(q), E[q])


@pytest.mark.parametrize("case", list(golden_io.femstab_cases()), ids=lambda c: c[0]["name"])
def test_fp32_within_tolerance(case):
    m, tr, E, K = case
    s = _run(m, ems.FP32)
    assert rel_l2(s.traces(), tr) < 1e-4
    num = sum(np.sum((s.get_field(q) - E[q]) ** 2) for q in range(3))
    den = sum(np.sum(E[q] ** 2) for q in range(3))
    assert np.sqrt(num / den) < 1e-4


def test_continued_runs_and_reset_equal_one_run():
    m, tr, E, K = next(iter(golden_io.femstab_cases()))
    s = ems.FemStabSimulation(m["grid"], m["h"], m["dt"], m["eps"], m["mu"], m["tf"], m["stabilization"], m["use_ofem"])
    for c, p in m["sources"]:
        [s.setSource_x, s.setSource_y, s.setSource_z][c](p)
    for d in m["dipoles"]:
        s.setSourceDipole_x(d)
    s.run(7)
    s.reset()
    s.run(m["nsteps"] // 2)
    s.run(m["nsteps"] - m["nsteps"] // 2)
    for q in range(3):
        np.testing.assert_array_equal(s.get_field(q), E[q])


def test_save_results_writes_the_reference_csv(tmp_path):
    m, tr, E, K = next(iter(golden_io.femstab_cases()))
    s = _run(m, ems.FP64)
    path = os.path.join(tmp_path, "fem_0.3_1.csv")
    s.saveResults(m["nsteps"], path)
    rows = open(path).read().splitlines()
    assert rows[0] == "time,Ex,Ey,Ez"
    assert len(rows) == 1 + m["nsteps"] // m["tf"] + 1
    vals = np.array([[float(x) for x in r.split(",")] for r in rows[1:]])
    np.testing.assert_allclose(vals[:, 1:], tr[0], rtol=1e-5)      # default stream precision: 6 digits
    np.testing.assert_allclose(vals[:, 0], np.arange(len(rows) - 1) * m["tf"] * m["dt"], rtol=1e-5)


def test_rejects_fem_v2_receivers_and_bad_parameters():
    m, _, _, _ = next(iter(golden_io.femstab_cases()))
    s = ems.FemStabSimulation(m["grid"], m["h"], m["dt"], m["eps"], m["mu"], m["tf"], 0.3, 0)
    ijk = (C.c_int * 3)(3, 3, 3)
    assert ems.lib().ems_hexfem_add_observation(s._h, ijk) == -5   # node receivers belong to fem_v2
    with pytest.raises(ems.EmsError) as e:
        ems.FemStabSimulation(m["grid"], m["h"], m["h"] / 2.9e8, m["eps"], m["mu"], 1, 0.3, 0)   # c dt >= h
    assert e.value.status == -1
