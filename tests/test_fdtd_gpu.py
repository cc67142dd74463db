"""FDTD on the GPU through the C ABI against the reference (golden fixtures
produced by the unmodified reference) and the FP64 oracle.

FP64 results must be bit-identical.  FP32 results are compared to the FP64
oracle by relative L2 error with tolerance 2e-5 on fields and traces (single
precision rounding over a few hundred steps)."""
import numpy as np
import pytest

import golden_io
import oracle
from gpu_util import rel_l2
import emsolvers_gb300 as ems

pytestmark = pytest.mark.gpu
EPS0, MU0 = 8.854187817e-12, 1.25663706212e-6
FP32_TOL = 2e-5


def field_errors(f, ref):
    """Relative L2 error of each component, normalised by the norm of all
    components of the same field (E or H): a component that is zero up to
    round-off in FP64 (e.g. Hx of an x-directed dipole) is judged against the
    field it belongs to."""
    out = {}
    for group in (("Ex", "Ey", "Ez"), ("Hx", "Hy", "Hz")):
        norm = np.sqrt(sum(np.sum(np.asarray(ref[k], np.float64) ** 2) for k in group))
        for k in group:
            out[k] = np.linalg.norm((np.asarray(f[k], np.float64) - ref[k]).ravel()) / norm
    return out


def _run(m, precision):
    nx, ny, nz = m["grid"]
    s = ems.FdtdSimulation((nx, ny, nz), m["h"], m["dt"], m["eps"], m["mu"], m["tf"], precision=precision)
    for c, p in m["sources"]:
        [s.setSource_x, s.setSource_y, s.setSource_z][c](p)
    for o in m["observations"]:
        s.setObservationPoint(o)
    s.run(m["nsteps"])
    return s.traces(), s.fields()


@pytest.mark.parametrize("case", list(golden_io.fdtd_cases()), ids=lambda c: c[0]["name"])
def test_fp64_bitwise_equal_to_reference(case):
    m, tr, fields = case
    t, f = _run(m, ems.FP64)
    assert np.array_equal(t, tr)
    for k in fields:
        assert np.array_equal(f[k], fields[k]), k


@pytest.mark.parametrize("case", list(golden_io.fdtd_cases()), ids=lambda c: c[0]["name"])
def test_fp32_within_tolerance_of_reference(case):
    m, tr, fields = case
    t, f = _run(m, ems.FP32)
    assert rel_l2(t, tr) < FP32_TOL
    for k, err in field_errors(f, fields).items():
        assert err < FP32_TOL, k


def _sphere_case(n=20, pml=0, sigma=0.0):
    h = 1e-3
    dt = 0.99 * h / (2.998e8 * np.sqrt(3))
    zz, yy, xx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    r = np.sqrt((xx + 0.5 - n / 2) ** 2 + (yy + 0.5 - n / 2) ** 2 + (zz + 0.5 - n / 2) ** 2)
    eps = np.where(r < n / 4, 4.0, 1.0) * EPS0
    sig = np.where(r < n / 4, sigma, 0.0)
    return h, dt, eps, sig


@pytest.mark.parametrize("pml,sigma", [(0, 0.0), (0, 0.02), (4, 0.0), (4, 0.01)])
def test_fp64_materials_and_cpml_bitwise_equal_to_oracle(pml, sigma):
    n = 20
    h, dt, eps, sig = _sphere_case(n, pml, sigma)
    c = n // 2
    src = [(2, (c, c, c), ems.WAVE_RICKER, 10e9, 1.0)]
    obs = [([(c + 3, c, c)], [(c, c + 3, c)], [(c + 4, c, c)]), ([], [], [(c, c + 5, c)])]
    pmld = dict(cells=pml, m=3.0, kmax=2.0, amax=0.02, R0=1e-6) if pml else None
    # oracle material table in the library's first-occurrence order
    keys = {}
    ids = np.zeros(eps.size, np.uint16)
    for q, (e, s) in enumerate(zip(eps.ravel(), sig.ravel())):
        ids[q] = keys.setdefault((e, s), len(keys))
    table = sorted(keys.items(), key=lambda kv: kv[1])
    mat = (ids.reshape(eps.shape), np.array([k[0] for k, _ in table]), np.array([k[1] for k, _ in table]))
    tr_o, f_o = oracle.fdtd_run(n, n, n, h, dt, EPS0, MU0, 1, 60, src, obs, material=mat, pml=pmld)
    s = ems.FdtdSimulation((n, n, n), h, dt, EPS0, MU0, 1, precision=ems.FP64, pml_cells=pml, pml_order=3.0,
                           pml_kappa_max=2.0, pml_alpha_max=0.02, pml_reflection=1e-6)
    s.set_material(eps, sig)
    s.setSource_z((c, c, c), waveform=ems.WAVE_RICKER, f0=10e9)
    for o in obs:
        s.setObservationPoint(o)
    s.run(60)
    t = s.traces()
    np.testing.assert_array_equal(t[0], tr_o[0])
    assert np.isnan(t[1, 1:, 0]).all() and np.isnan(tr_o[1, 1:, 0]).all()  # empty list: 0/0 as the reference
    np.testing.assert_array_equal(t[1, :, 2], tr_o[1, :, 2])
    f = s.fields()
    for k in f:
        np.testing.assert_array_equal(f[k], f_o[k], err_msg=k)
    # FP32 of the same case
    s32 = ems.FdtdSimulation((n, n, n), h, dt, EPS0, MU0, 1, precision=ems.FP32, pml_cells=pml, pml_order=3.0,
                             pml_kappa_max=2.0, pml_alpha_max=0.02, pml_reflection=1e-6)
    s32.set_material(eps, sig)
    s32.setSource_z((c, c, c), waveform=ems.WAVE_RICKER, f0=10e9)
    for o in obs:
        s32.setObservationPoint(o)
    s32.run(60)
    assert rel_l2(s32.traces()[0], tr_o[0]) < FP32_TOL
    for k, err in field_errors(s32.fields(), f_o).items():
        assert err < FP32_TOL, k


def test_save_results_matches_reference_format(tmp_path):
    m, tr, _ = next(iter(golden_io.fdtd_cases()))
    nx, ny, nz = m["grid"]
    s = ems.FdtdSimulation((nx, ny, nz), m["h"], m["dt"], m["eps"], m["mu"], m["tf"])
    s.setSource_x(m["sources"][0][1])
    s.setObservationPoint(m["observations"][0])
    s.run(m["nsteps"])
    s.saveResults(directory=str(tmp_path))
    files = list(tmp_path.glob("results_0_*.csv"))
    assert len(files) == 1
    lines = files[0].read_text().splitlines()
    assert lines[0] == "time,Ex,Ey,Ez"
    assert len(lines) == m["nsteps"] // m["tf"] + 2
    assert lines[1].startswith("0,0,0,0")
    s.save_component(0, 1, tmp_path / "ey.csv")
    rows = (tmp_path / "ey.csv").read_text().splitlines()
    tu = np.array([[float(x) for x in r.split(",")] for r in rows[1:]])
    assert rows[0] == "t,u"
    np.testing.assert_allclose(tu[:, 0], np.arange(len(tu)) * m["tf"] * m["dt"], rtol=1e-14)
    np.testing.assert_allclose(tu[:, 1], s.traces()[0, :, 1], rtol=1e-14)


def test_runs_are_deterministic():
    m, _, _ = next(iter(golden_io.fdtd_cases()))
    a, fa = _run(m, ems.FP32)
    b, fb = _run(m, ems.FP32)
    assert np.array_equal(a, b)
    for k in fa:
        assert np.array_equal(fa[k], fb[k])


def test_launch_shape_autotuner_picks_a_candidate_and_changes_no_result():
    # the first run of >= 24 steps times six launch shapes and keeps the
    # fastest; forced shapes (EMS_FDTD_BLOCK, child processes) must give the
    # same fields and traces bit for bit
    import os
    import subprocess
    import sys
    code = (
        "import numpy as np, emsolvers_gb300 as ems\n"
        "g = (37, 29, 23)\n"
        "rng = np.random.default_rng(5)\n"
        "s = ems.FdtdSimulation(g, 1e-3, 1.5e-12, 8.854187817e-12, 1.25663706212e-6, 2, precision=ems.FP32,\n"
        "                       pml_cells=4)\n"
        "s.set_material(rng.uniform(1, 4, g[::-1]) * 8.854187817e-12, rng.uniform(0, 0.05, g[::-1]))\n"
        "s.setSource_z((18, 14, 11))\n"
        "s.setObservationPoint(([(20, 15, 12)], [(20, 15, 12)], [(20, 15, 12)]))\n"
        "s.run(40)\n"
        "print('%%d %%d' %% s.launch_shape()[:2])\n"
        "f = s.fields()\n"
        "np.save('%s', np.concatenate([s.traces().ravel()] + [np.ravel(f[k]) for k in sorted(f)]))\n")
    # the two-kernel step (default) in its autotuned and forced launch shapes
    # and the opt-in fused H+E step give the same bits
    out = {}
    for shape in ("fused", "", "32x8", "256x1", "64x2"):
        env = dict(os.environ)
        env.pop("EMS_FDTD_BLOCK", None)
        env.pop("EMS_FDTD_FUSED", None)
        if shape == "fused":
            env["EMS_FDTD_FUSED"] = "1"
        if shape not in ("", "fused"):
            env["EMS_FDTD_BLOCK"] = shape
        path = f"/tmp/ems_fdtd_shape_{shape or 'auto'}_{os.getpid()}.npy"
        r = subprocess.run([sys.executable, "-c", code % path], env=env, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        x, y = map(int, r.stdout.strip().splitlines()[-1].split())
        assert (x, y) in [(32, 8), (32, 4), (64, 4), (128, 2), (256, 1), (64, 2)]
        if shape not in ("", "fused"):
            assert f"{x}x{y}" == shape
        out[shape] = np.load(path)
        os.remove(path)
    for shape in ("", "32x8", "256x1", "64x2"):
        assert np.array_equal(out["fused"], out[shape])


def _cpml_traces(n, src, recs, steps, precision, pml_cells, kmax=1.0, amax=0.0, f0=None):
    h, c0 = 1e-3, 299792458.0
    dt = 0.99 * h / (c0 * np.sqrt(3))
    s = ems.FdtdSimulation((n, n, n), h, dt, 8.854187817e-12, 1.25663706212e-6, 1, precision=precision,
                           pml_cells=pml_cells, pml_order=3.0, pml_kappa_max=kmax, pml_alpha_max=amax, pml_reflection=1e-6)
    s.setSource_z(src, waveform=ems.WAVE_RICKER, f0=f0 or c0 / (15 * h))
    for r in recs:
        s.setObservationPoint(([], [], [r]))
    s.run(steps)
    tr = s.traces()[:, :, 2]
    s.close()
    return tr


@pytest.mark.parametrize("precision", [ems.FP64, ems.FP32], ids=["fp64", "fp32"])
def test_cpml_reflection_on_the_gpu(precision):
    # the physical CPML pin of test_fdtd_cpml.py through the library: 8-cell
    # CPML against a box too large for echoes within 160 steps
    n, L, big = 40, 8, 104
    c, off = n // 2, (big - n) // 2
    recs = [(c, c, c + 9), (c + 8, c + 8, c), (c + 7, c + 7, c + 7)]
    small = _cpml_traces(n, (c, c, c), recs, 160, precision, L)
    ref = _cpml_traces(big, (c + off,) * 3, [tuple(v + off for v in r) for r in recs], 160, precision, 0)
    for q in range(3):
        assert np.linalg.norm(small[q] - ref[q]) / np.linalg.norm(ref[q]) < 1e-3


def test_cfs_cpml_stays_stable_over_10000_steps():
    # kappa_max > 1 and alpha_max > 0, FP32, 10,000 steps: the CPML absorbs
    # the pulse and nothing grows back (late-time fields far below the early
    # peak and still decaying)
    n, c = 32, 16
    recs = [(c, c, c + 5), (c + 5, c + 5, c), (c - 4, c + 3, c - 5)]
    tr = np.abs(_cpml_traces(n, (c, c, c), recs, 10000, ems.FP32, 10, kmax=5.0, amax=0.05))
    early = tr[:, :2000].max()
    assert early > 0
    assert tr[:, 6000:8000].max() < 1e-3 * early
    assert tr[:, 8000:].max() <= tr[:, 6000:8000].max() + 1e-6 * early


def test_sphere_workload_at_full_size_bitwise_equal_to_oracle():
    # the FP64 workload of the reference's FDTD family at its full size:
    # 64^3 cells of 1 mm, vacuum with a centred sphere of radius 16 cells,
    # eps_r 4, PEC walls, dt = 0.99 x CFL, a Jz Ricker point source (10 GHz)
    # at the centre, 1000 steps, Ez at 8 receivers on a 20-cell ring in the
    # source's z plane: traces and all six fields bit-identical to the oracle
    n, h = 64, 1e-3
    dt = 0.99 * h / (299792458.0 * np.sqrt(3))
    zz, yy, xx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    r = np.sqrt((xx + 0.5 - n / 2) ** 2 + (yy + 0.5 - n / 2) ** 2 + (zz + 0.5 - n / 2) ** 2)
    inside = r < 16
    eps = np.where(inside, 4.0, 1.0) * EPS0
    c = n // 2
    recs = [(c + int(round(20 * np.cos(a))), c + int(round(20 * np.sin(a))), c) for a in np.arange(8) * np.pi / 4]
    obs = [([], [], [q]) for q in recs]
    first = 0 if not inside.ravel()[0] else 1          # library table: materials in first-occurrence order
    ids = np.where(inside, 1 - first, first).astype(np.uint16)
    table = np.array([EPS0, 4.0 * EPS0]) if first == 0 else np.array([4.0 * EPS0, EPS0])
    tr_o, f_o = oracle.fdtd_run(n, n, n, h, dt, EPS0, MU0, 1, 1000, [(2, (c, c, c), ems.WAVE_RICKER, 10e9, 1.0)], obs,
                                material=(ids, table, np.zeros(2)))
    s = ems.FdtdSimulation((n, n, n), h, dt, EPS0, MU0, 1, precision=ems.FP64)
    s.set_material(eps, np.zeros_like(eps))
    s.setSource_z((c, c, c), waveform=ems.WAVE_RICKER, f0=10e9)
    for o in obs:
        s.setObservationPoint(o)
    s.run(1000)
    t = s.traces()
    assert np.abs(tr_o[:, :, 2]).max() > 0
    np.testing.assert_array_equal(t[:, :, 2], tr_o[:, :, 2])
    for k, v in s.fields().items():
        np.testing.assert_array_equal(v, f_o[k], err_msg=k)
