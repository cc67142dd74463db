"""Hexahedral FEM (fem_v2 leapfrog, symplectic_2, symplectic_4; orders 1-3)
on the GPU through the C ABI.  FP64 must equal the reference bit for bit
(golden fixtures); FP32 is compared with the FP64 reference by relative L2
error, tolerance 1e-4 on traces and fields."""
import numpy as np
import pytest

import golden_io
import oracle
from gpu_util import rel_l2
import emsolvers_gb300 as ems

pytestmark = pytest.mark.gpu
INTEG = {"fem_v2": ems.LEAPFROG, "symplectic_2": ems.SYMP2, "symplectic_4": ems.SYMP4}
FP32_TOL = 1e-4


def _run(m, precision):
    s = ems.HexFemSimulation(m["order"], m["grid"], m["h"], m["dt"], m["eps"], m["mu"], m["tf"], m["use_ofem"],
                             integrator=INTEG[m["variant"]], precision=precision, kmat_dir=golden_io.KMAT_DIR)
    [s.setSource_x, s.setSource_y, s.setSource_z][m["source"][0]](m["source"][1])
    s.setObservationPoint(m["observation"])
    s.run(m["nsteps"])
    return s.traces()[0], s.levels()


@pytest.mark.parametrize("case", list(golden_io.femv2_cases()), ids=lambda c: c[0]["name"])
def test_fp64_bitwise_equal_to_reference(case):
    m, tr, ef = case
    t, lv = _run(m, ems.FP64)
    np.testing.assert_array_equal(t, tr)
    for q in range(3):
        np.testing.assert_array_equal(lv[q], ef[q])


@pytest.mark.parametrize("case", list(golden_io.femv2_cases()), ids=lambda c: c[0]["name"])
def test_fp32_within_tolerance_of_reference(case):
    m, tr, ef = case
    t, lv = _run(m, ems.FP32)
    assert rel_l2(t[:, 1:], tr[:, 1:]) < FP32_TOL
    assert np.array_equal(t[:, 0], tr[:, 0])
    # compare all stored levels, normalised by the norm of all components
    num = sum(np.sum((lv[q] - ef[q]) ** 2) for q in range(3))
    den = sum(np.sum(ef[q] ** 2) for q in range(3))
    assert np.sqrt(num / den) < FP32_TOL


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4, oracle.LEAPFROG])
def test_fp64_longer_run_matches_oracle(order, integ):
    g = (8 * order, 6 * order, 6 * order) if order == 1 else (8, 8, 10)
    h = 0.05
    c0 = 1 / np.sqrt(8.8541878128e-12 * 1.25663706212e-6)
    dt = h / (c0 * np.sqrt(3.0)) / 2.0
    km = oracle.load_kmat(golden_io.kmat_path(order, 1))
    src = (2, (g[0] // 2, g[1] // 2, g[2] // 2))
    obs = [(g[0] // 2 + 1, g[1] // 2, g[2] // 2), (2, 2, 2)]
    tr_o, ef_o = oracle.hexfem_run(order, g, h, dt, 8.8541878128e-12, 1.25663706212e-6, 3, integ, km, 120, [src], obs)
    s = ems.HexFemSimulation(order, g, h, dt, 8.8541878128e-12, 1.25663706212e-6, 3, 1, integrator=integ,
                             precision=ems.FP64, kmat_dir=golden_io.KMAT_DIR)
    s.setSource_z(src[1])
    for o in obs:
        s.setObservationPoint(o)
    s.run(120)
    np.testing.assert_array_equal(s.traces(), tr_o)
    for q, lv in enumerate(s.levels()):
        np.testing.assert_array_equal(lv, ef_o[q])


def test_save_results_format(tmp_path):
    m, tr, _ = next(iter(golden_io.femv2_cases()))
    s = ems.HexFemSimulation(m["order"], m["grid"], m["h"], m["dt"], m["eps"], m["mu"], m["tf"], m["use_ofem"],
                             kmat_dir=golden_io.KMAT_DIR)
    s.setSource_z(m["source"][1])
    s.setObservationPoint(m["observation"])
    s.run(m["nsteps"])
    fn = tmp_path / "out.csv"
    s.saveResults(m["nsteps"], str(fn))
    lines = fn.read_text().splitlines()
    assert lines[0] == "time,Ex,Ey,Ez"
    vals = np.array([[float(v) for v in l.split(",")] for l in lines[1:]])
    np.testing.assert_allclose(vals, tr, rtol=1e-14, atol=0)
    assert "e" in lines[2]  # scientific, 15 digits
