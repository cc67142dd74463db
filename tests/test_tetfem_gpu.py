"""Tetrahedral FEM on the GPU through the C ABI against the FP64 oracle.

Tolerances (relative L2): FP64 GPU vs FP64 oracle 1e-10 (the GPU merges the
drifts inside a 4th-order step and sums gathers in a different order);
FP32 GPU vs FP64 oracle 1e-4 on receiver traces, the bound the FP32 path
must meet."""
import numpy as np
import pytest

import oracle
from gpu_util import rel_l2
import emsolvers_gb300 as ems

pytestmark = pytest.mark.gpu
C0 = 299792458.0
H = 1e-3
TS = H / C0          # seconds per normalised time unit
FP64_TOL = 1e-10
FP32_TOL = 1e-4
INTEG = {oracle.SYMP2: ems.SYMP2, oracle.SYMP4: ems.SYMP4, oracle.LEAPFROG: ems.LEAPFROG}


def _case(n, seed):
    _, nslot, ntet = oracle.tet_sizes(n)
    rng = np.random.default_rng(seed)
    eps = rng.uniform(1.0, 4.0, ntet)
    dip = ((n[0] * 0.41, n[1] * 0.52, n[2] * 0.47), (0.2, 0.3, 1.0), 1, 0.08, 1.0)
    recs = [(n[0] * 0.7, n[1] * 0.5, n[2] * 0.5), (n[0] * 0.25, n[1] * 0.3, n[2] * 0.6)]
    return eps, dip, recs


def _gpu(n, eps, dip, recs, integ, dtn, nsteps, precision, tf=1):
    s = ems.TetFemSimulation(n, H, 1, INTEG[integ], precision, dt=dtn * TS, time_frequency=tf)
    s.set_material(eps)
    s.add_dipole(np.array(dip[0]) * H, dip[1], ems.WAVE_RICKER, dip[3] / TS, dip[4])
    for r in recs:
        s.add_receiver(np.array(r) * H)
    s.run(nsteps)
    return s


@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4, oracle.LEAPFROG])
def test_fp64_matches_oracle(integ):
    n = (6, 5, 4)
    eps, dip, recs = _case(n, 7)
    dtn = 0.8 * oracle.stability_constant(integ) / np.sqrt(oracle.tet_lambda_max(n, eps, 300))
    tr_o, U_o, P_o = oracle.tet_run(n, eps, integ, dtn, 150, 2, [dip], recs)
    s = _gpu(n, eps, dip, recs, integ, dtn, 150, ems.FP64, tf=2)
    t = s.traces()
    np.testing.assert_allclose(t[:, :, 0], tr_o[:, :, 0] * TS, rtol=1e-12)
    assert rel_l2(t[:, :, 1:], tr_o[:, :, 1:]) < FP64_TOL
    assert rel_l2(s.get_field(0), U_o) < FP64_TOL
    assert rel_l2(s.get_field(1), P_o) < FP64_TOL


@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4])
def test_fp32_traces_within_1e4_of_fp64_oracle(integ):
    n = (12, 12, 12)
    eps, dip, recs = _case(n, 11)
    dtn = 0.9 * oracle.stability_constant(integ) / np.sqrt(oracle.tet_lambda_max(n, eps, 300))
    tr_o, U_o, _ = oracle.tet_run(n, eps, integ, dtn, 400, 1, [dip], recs)
    s = _gpu(n, eps, dip, recs, integ, dtn, 400, ems.FP32)
    assert rel_l2(s.traces()[:, :, 1:], tr_o[:, :, 1:]) < FP32_TOL
    assert rel_l2(s.get_field(0), U_o) < FP32_TOL


@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4, oracle.LEAPFROG])
def test_automatic_time_step_matches_oracle_stability_limit(integ):
    n = (8, 7, 6)
    eps, _, _ = _case(n, 3)
    s = ems.TetFemSimulation(n, H, 1, INTEG[integ], ems.FP32, dt=0.0, cfl_fraction=0.9)
    s.set_material(eps)
    dt, lim = s.time_step()
    lim_o = oracle.stability_constant(integ) / np.sqrt(oracle.tet_lambda_max(n, eps, 600)) * TS
    assert abs(lim - lim_o) / lim_o < 1e-5
    assert abs(dt - 0.9 * lim) / dt < 1e-12


def test_fp32_runs_are_bitwise_deterministic():
    n = (10, 9, 8)
    eps, dip, recs = _case(n, 5)
    dtn = 0.8 * oracle.stability_constant(oracle.SYMP4) / np.sqrt(oracle.tet_lambda_max(n, eps, 200))
    a = _gpu(n, eps, dip, recs, oracle.SYMP4, dtn, 100, ems.FP32)
    b = _gpu(n, eps, dip, recs, oracle.SYMP4, dtn, 100, ems.FP32)
    assert np.array_equal(a.traces(), b.traces())
    assert np.array_equal(a.get_field(0), b.get_field(0))


def test_gpu_symplectic_state_conserves_discrete_energy():
    n = (6, 6, 6)
    _, nslot, ntet = oracle.tet_sizes(n)
    rng = np.random.default_rng(9)
    eps = rng.uniform(1, 4, ntet)
    pec = oracle.tet_pec_mask(n)
    U0 = np.where(pec, 0.0, rng.standard_normal(nslot))
    dtn = 0.4 * oracle.stability_constant(oracle.SYMP4) / np.sqrt(oracle.tet_lambda_max(n, eps, 300))
    s = ems.TetFemSimulation(n, H, 1, ems.SYMP4, ems.FP64, dt=dtn * TS)
    s.set_material(eps)
    s.set_field(0, U0)
    e0 = oracle.tet_energy(n, eps, U0, np.zeros(nslot))
    errs = []
    for _ in range(10):
        s.run(30)
        errs.append(abs(oracle.tet_energy(n, eps, s.get_field(0), s.get_field(1)) - e0) / e0)
    assert max(errs) < 5e-3
    assert max(errs[5:]) < 1.3 * max(errs[:5]) + 1e-12


@pytest.mark.parametrize("precision,tol", [(ems.FP64, 1e-12), (ems.FP32, 2e-6)], ids=["fp64", "fp32"])
def test_gpu_energy_matches_oracle_energy_of_the_same_state(precision, tol):
    # the GPU's FP64 energy of the run's state against the oracle's energy
    # of the same (widened) fields; FP32 runs keep FP32 mass blocks, which
    # differ from the oracle's by ~1e-7 relative
    n = (5, 6, 4)
    _, nslot, ntet = oracle.tet_sizes(n)
    rng = np.random.default_rng(21)
    eps = rng.uniform(1, 4, ntet)
    pec = oracle.tet_pec_mask(n)
    U0 = np.where(pec, 0.0, rng.standard_normal(nslot))
    dtn = 0.5 * oracle.stability_constant(oracle.SYMP4) / np.sqrt(oracle.tet_lambda_max(n, eps, 300))
    s = ems.TetFemSimulation(n, H, 1, ems.SYMP4, precision, dt=dtn * TS)
    s.set_material(eps)
    s.set_field(0, U0)
    s.run(40)
    e_gpu = s.energy()
    e_orc = oracle.tet_energy(n, eps, s.get_field(0), s.get_field(1))
    assert abs(e_gpu - e_orc) < tol * e_orc


@pytest.mark.parametrize("precision,bound", [(ems.FP64, 5e-3), (ems.FP32, 5e-3)], ids=["fp64", "fp32"])
def test_gpu_energy_stays_bounded_without_drift(precision, bound):
    # symplectic: the energy error oscillates at O(dt^4) and does not grow
    n = (6, 6, 6)
    _, nslot, ntet = oracle.tet_sizes(n)
    rng = np.random.default_rng(9)
    eps = rng.uniform(1, 4, ntet)
    pec = oracle.tet_pec_mask(n)
    U0 = np.where(pec, 0.0, rng.standard_normal(nslot))
    dtn = 0.4 * oracle.stability_constant(oracle.SYMP4) / np.sqrt(oracle.tet_lambda_max(n, eps, 300))
    s = ems.TetFemSimulation(n, H, 1, ems.SYMP4, precision, dt=dtn * TS)
    s.set_material(eps)
    s.set_field(0, U0)
    e0 = s.energy()
    errs = []
    for _ in range(10):
        s.run(30)
        errs.append(abs(s.energy() - e0) / e0)
    assert max(errs) < bound
    assert max(errs[5:]) < 1.3 * max(errs[:5]) + 1e-6


def test_gpu_energy_per_shot_of_a_batch_and_leapfrog_rejected():
    cells = [(4, 5, 3), (3, 3, 6)]
    rng = np.random.default_rng(13)
    eps = [rng.uniform(1, 4, 6 * c[0] * c[1] * c[2]) for c in cells]
    dt = 0.5 * 2.0 * TS / np.sqrt(max(oracle.tet_lambda_max(c, e, 100) for c, e in zip(cells, eps)))
    b = ems.TetFemBatch(cells, H, integrator=ems.SYMP4, precision=ems.FP64, dt=dt)
    b.set_material(np.concatenate(eps))
    U = []
    for c in cells:
        _, ns, _ = oracle.tet_sizes(c)
        U.append(np.where(oracle.tet_pec_mask(c), 0.0, rng.standard_normal(ns)))
    b.set_field(0, np.concatenate(U))
    b.run(25)
    e = b.energy()
    u, p = b.get_field(0), b.get_field(1)
    off = 0
    for k, c in enumerate(cells):
        _, ns, _ = oracle.tet_sizes(c)
        ref = oracle.tet_energy(c, eps[k], u[off:off + ns], p[off:off + ns])
        assert abs(e[k] - ref) < 1e-12 * ref
        off += ns
    lf = ems.TetFemSimulation((3, 3, 3), H, 1, ems.LEAPFROG, ems.FP64, dt=1e-13)
    lf.set_material(np.full(162, 2.0))
    with pytest.raises(ems.EmsError) as err:
        lf.energy()
    assert err.value.status == -8


def test_save_results_writes_reference_trace_format(tmp_path):
    n = (6, 5, 4)
    eps, dip, recs = _case(n, 7)
    dtn = 0.5 * 2.0 / np.sqrt(oracle.tet_lambda_max(n, eps, 200))
    s = _gpu(n, eps, dip, recs, oracle.SYMP2, dtn, 20, ems.FP32)
    fn = tmp_path / "tet.csv"
    s.saveResults = None
    assert ems.lib().ems_save_results(s._h, str(fn).encode()) == 0
    lines = fn.read_text().splitlines()
    assert lines[0] == "time,Ex,Ey,Ez" and len(lines) == 21
    assert (tmp_path / "tet_1.csv").exists()
    # per-component t,u file for the TF misfit pipeline
    tr = s.traces()
    s.save_component(1, 2, tmp_path / "u.csv")
    rows = (tmp_path / "u.csv").read_text().splitlines()
    assert rows[0] == "t,u" and len(rows) == tr.shape[1] + 1
    tu = np.array([[float(x) for x in r.split(",")] for r in rows[1:]])
    np.testing.assert_allclose(tu[:, 0], tr[1, :, 0], rtol=1e-14)
    np.testing.assert_allclose(tu[:, 1], tr[1, :, 3], rtol=1e-14)
    with pytest.raises(ems.EmsError):
        s.save_component(5, 0, tmp_path / "bad.csv")


@pytest.mark.parametrize("precision,tol", [(ems.FP64, 1e-13), (ems.FP32, 1e-6)])
def test_apply_stiffness_matches_oracle(precision, tol):
    n = (7, 6, 5)
    _, nslot, ntet = oracle.tet_sizes(n)
    rng = np.random.default_rng(13)
    u = rng.standard_normal(nslot)
    s = ems.TetFemSimulation(n, H, 1, ems.SYMP2, precision, dt=1e-13)
    f = s.apply_stiffness(u)
    f_o = oracle.tet_apply_K(n, u)
    assert rel_l2(f, f_o) < tol
    pec = oracle.tet_pec_mask(n)
    assert np.all(f[pec] == 0.0)
    # the solver state is untouched
    assert np.all(s.get_field(0) == 0.0)


_LAUNCH_SHAPE_CASE = (
    "import sys, numpy as np, emsolvers_gb300 as ems\n"
    "prec, lossy = {'fp32': ems.FP32, 'fp64': ems.FP64}[sys.argv[2]], sys.argv[3] == '1'\n"
    "n = (9, 7, 8)\n"
    "rng = np.random.default_rng(3)\n"
    "eps = rng.uniform(1, 4, 6 * 9 * 7 * 8)\n"
    "sig = rng.uniform(0.0, 0.3, eps.size) if lossy else None\n"
    "s = ems.TetFemSimulation(n, 1e-3, 1, ems.SYMP4, prec, dt=0.0, cfl_fraction=0.8)\n"
    "s.set_material(eps, sig)\n"
    "s.add_dipole(np.array([4.1, 3.3, 4.2]) * 1e-3, (0.2, 0.3, 1.0), ems.WAVE_RICKER, 4e10, 1.0)\n"
    "for p in ([6.2, 2.1, 3.3], [2.2, 5.1, 6.3], [4.4, 3.9, 1.1]):\n"
    "    s.add_receiver(np.array(p) * 1e-3)\n"
    "s.set_checkpoints(5)\n"
    "s.reset()\n"
    "s.run(80)\n"
    "tg = s.traces().copy(); tg[..., 0] = 0.0\n"
    "g = s.backward(tg)\n"
    "print(*s.launch_shape())\n"
    "np.save(sys.argv[1], np.concatenate([s.traces().ravel(), s.get_field(0), s.get_field(1), g]))\n")


@pytest.mark.parametrize("prec,lossy", [("fp32", "0"), ("fp64", "0"), ("fp32", "1")], ids=["fp32", "fp64", "fp32-lossy"])
def test_step_launch_shapes_change_no_result(prec, lossy):
    # forced launch shapes (EMS_TET_STEP_BLOCK) in child processes: the node
    # kernel at two block sizes, the slot-split kernel (seven warps per 32
    # nodes) and the persistent step (the slot-split step with grid barriers
    # between substeps; lossy runs fall back to the slot-split kernel) are
    # launch shapes of the same arithmetic, so traces, fields and the adjoint
    # gradient are bit-identical; the autotuner picks one of them
    import os
    import subprocess
    import sys
    out = {}
    for b in ("", "32", "256", "slot", "persist"):
        env = dict(os.environ)
        env.pop("EMS_TET_STEP_BLOCK", None)
        if b:
            env["EMS_TET_STEP_BLOCK"] = b
        path = f"/tmp/ems_step_block_{b or 'auto'}_{prec}_{lossy}_{os.getpid()}.npy"
        r = subprocess.run([sys.executable, "-c", _LAUNCH_SHAPE_CASE, path, prec, lossy], env=env, capture_output=True,
                           text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        shape = tuple(int(v) for v in r.stdout.strip().splitlines()[-1].split())
        assert shape in ((32, 1, 1), (64, 1, 1), (128, 1, 1), (256, 1, 1), (32, 7, 1))
        if b in ("slot", "persist"):
            assert shape == (32, 7, 1)
        elif b:
            assert shape == (int(b), 1, 1)
        out[b] = np.load(path)
        os.remove(path)
    for b in ("32", "256", "slot", "persist"):
        assert np.array_equal(out[""], out[b]), b


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("integ", [ems.SYMP2, ems.SYMP4], ids=["symp2", "symp4"])
def test_persistent_step_matches_the_slot_kernel(monkeypatch, integ, prec):
    # the persistent step (one cooperative launch per CUDA graph of 12 steps,
    # grid barriers between substeps, P and its compensation kept in shared
    # memory between them) gives the slot-split kernel's bits: 30 receivers
    # (two sampling blocks), samples every third step, a run continued
    # across calls (a graph of 12 steps and a shorter remainder launch)
    n = (10, 9, 8)
    rng = np.random.default_rng(11)
    eps = rng.uniform(1, 4, 6 * n[0] * n[1] * n[2])
    recs = rng.uniform(0.5, 1.0, (30, 3)) * (np.array(n) - 1.0)
    P = {"fp32": ems.FP32, "fp64": ems.FP64}[prec]
    out = {}
    for shape in ("slot", "persist"):
        monkeypatch.setenv("EMS_TET_STEP_BLOCK", shape)
        s = ems.TetFemSimulation(n, H, 1, integ, P, dt=0.0, cfl_fraction=0.85, time_frequency=3)
        s.set_material(eps)
        s.add_dipole(np.array([4.1, 3.3, 4.2]) * H, (0.2, 0.3, 1.0), ems.WAVE_RICKER, 4e10, 1.0)
        for r in recs:
            s.add_receiver(r * H)
        s.run(40)
        t1 = s.traces().copy()
        s.run(23)
        t2 = s.traces().copy()
        name = s.time_dominant_kernel(24)[2]
        out[shape] = (t1, t2, s.get_field(0), s.get_field(1), name)
        s.close()
    for i in range(4):
        assert np.array_equal(out["slot"][i], out["persist"][i]), i
    assert np.abs(out["slot"][1][..., 1:]).max() > 0
    assert out["slot"][4].startswith("tet_slot_kernel")
    assert out["persist"][4].startswith("tet_persist_kernel")


@pytest.mark.parametrize("integ", [oracle.SYMP4, oracle.LEAPFROG], ids=["symp4", "leapfrog"])
def test_dipoles_sharing_slots_match_oracle(integ):
    # three dipoles, two of them in the same tetrahedron (their six slots
    # coincide) and one in a neighbouring cell: the step kernels find a
    # slot's entries in the sorted source list and sum them in dipole order
    n = (6, 5, 5)
    eps, _, recs = _case(n, 17)
    p = (n[0] * 0.43, n[1] * 0.51, n[2] * 0.46)
    dips = [(p, (0.2, 0.3, 1.0), 1, 0.08, 1.0), (p, (1.0, -0.5, 0.2), 1, 0.11, 0.7),
            ((p[0] + 1.0, p[1], p[2]), (0.0, 1.0, 0.3), 1, 0.09, 1.3)]
    dtn = 0.8 * oracle.stability_constant(integ) / np.sqrt(oracle.tet_lambda_max(n, eps, 300))
    tr_o, U_o, _ = oracle.tet_run(n, eps, integ, dtn, 120, 1, dips, recs)
    s = ems.TetFemSimulation(n, H, 1, INTEG[integ], ems.FP64, dt=dtn * TS)
    s.set_material(eps)
    for d in dips:
        s.add_dipole(np.array(d[0]) * H, d[1], ems.WAVE_RICKER, d[3] / TS, d[4])
    for r in recs:
        s.add_receiver(np.array(r) * H)
    s.run(120)
    assert rel_l2(s.traces()[..., 1:], tr_o[..., 1:]) < FP64_TOL
    assert rel_l2(s.get_field(0), U_o) < FP64_TOL


@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4, oracle.LEAPFROG], ids=["symp2", "symp4", "leapfrog"])
def test_a_continued_run_matches_one_long_run(integ):
    # the second run restarts the step counter and the receivers' Minv P
    # buffer; its traces are the tail of one run over both intervals (FP64;
    # the symplectic runs close and reopen the merged half drift in between,
    # which changes the last bits only)
    n = (6, 5, 5)
    eps, dip, recs = _case(n, 21)
    dtn = 0.8 * oracle.stability_constant(integ) / np.sqrt(oracle.tet_lambda_max(n, eps, 300))
    one = _gpu(n, eps, dip, recs, integ, dtn, 75, ems.FP64)
    two = _gpu(n, eps, dip, recs, integ, dtn, 40, ems.FP64)
    first = two.traces()
    two.run(35)
    second = two.traces()
    full = one.traces()
    np.testing.assert_allclose(first[..., 0], full[:, :40, 0], rtol=1e-12)
    np.testing.assert_allclose(second[..., 0], full[:, 40:, 0], rtol=1e-12)
    assert rel_l2(first[..., 1:], full[:, :40, 1:]) < 1e-13
    assert rel_l2(second[..., 1:], full[:, 40:, 1:]) < 1e-11


@pytest.mark.parametrize("precision", [ems.FP32, ems.FP64], ids=["fp32", "fp64"])
def test_material_change_on_one_handle_equals_fresh_handles(precision):
    # the handle keeps its stability-limit workspace, the captured graph of
    # its iterations and its run tables between set_material calls: a second
    # material on the same handle must give what a fresh handle gives
    n = (9, 8, 7)
    _, _, ntet = oracle.tet_sizes(n)
    rng = np.random.default_rng(21)
    eps = [rng.uniform(1.0, 4.0, ntet), rng.uniform(2.0, 9.0, ntet)]
    _, dip, recs = _case(n, 21)

    def fresh(e):
        s = ems.TetFemSimulation(n, H, 1, ems.SYMP4, precision, dt=0.0, cfl_fraction=0.9)
        s.set_material(e)
        s.add_dipole(np.array(dip[0]) * H, dip[1], ems.WAVE_RICKER, dip[3] / TS, dip[4])
        for r in recs:
            s.add_receiver(np.array(r) * H)
        s.run(60)
        return s.time_step(), s.traces()

    s = ems.TetFemSimulation(n, H, 1, ems.SYMP4, precision, dt=0.0, cfl_fraction=0.9)
    s.add_dipole(np.array(dip[0]) * H, dip[1], ems.WAVE_RICKER, dip[3] / TS, dip[4])
    for r in recs:
        s.add_receiver(np.array(r) * H)
    for e in eps + eps[:1]:
        s.set_material(e)
        s.reset()
        s.run(60)
        ts, tr = fresh(e)
        assert s.time_step() == ts
        assert np.array_equal(s.traces(), tr)
        # the oracle's power iteration converges linearly: 600 iterations leave
        # about 3e-5 of lambda on this mesh, 4000 converge it
        lim_o = oracle.stability_constant(oracle.SYMP4) / np.sqrt(oracle.tet_lambda_max(n, e, 4000)) * TS
        assert abs(ts[1] - lim_o) / lim_o < 1e-5


def test_receivers_added_between_runs_equal_a_fresh_handle():
    # the receiver slot table is rebuilt only when the receiver set changes
    n = (8, 8, 8)
    eps, dip, recs = _case(n, 22)
    more = [(n[0] * 0.33, n[1] * 0.61, n[2] * 0.52), recs[0]]
    dtn = 0.8 * oracle.stability_constant(oracle.SYMP4) / np.sqrt(oracle.tet_lambda_max(n, eps, 300))
    s = _gpu(n, eps, dip, recs, oracle.SYMP4, dtn, 50, ems.FP32)
    s.run(50)   # unchanged receivers
    for r in more:
        s.add_receiver(np.array(r) * H)
    s.reset()
    s.run(70)
    f = _gpu(n, eps, dip, recs + more, oracle.SYMP4, dtn, 70, ems.FP32)
    assert np.array_equal(s.traces(), f.traces())
    assert np.array_equal(s.get_field(0), f.get_field(0))


def test_headline_workload_at_full_size_against_the_oracle():
    # the headline configuration at its full size: 32^3 cubes x 6 tets,
    # eps_r U[1,4], symp4, dt = 0.9 x the stability limit chosen by the GPU,
    # 2000 steps, one Ricker dipole (10 elements per wavelength), 8
    # receivers on a ring.  FP64 within 1e-9 of the FP64 oracle (rounding
    # differences over 2000 steps).  FP32 within the 1e-4 trace bound: its
    # U and P updates are compensated sums (without them the FP32 error
    # reached 1.08e-4 here and grew faster than linearly with the run length)
    n = (32, 32, 32)
    eps = np.random.default_rng(1234).uniform(1.0, 4.0, 6 * 32 ** 3)
    f0 = C0 / (10 * H * np.sqrt(2.0))
    src = (16.3, 15.7, 16.1)
    recs = [(16 + 10 * np.cos(k), 16 + 10 * np.sin(k), 16.2) for k in range(8)]
    out = {}
    for precision in (ems.FP32, ems.FP64):
        s = ems.TetFemSimulation(n, H, 1, ems.SYMP4, precision, dt=0.0, cfl_fraction=0.9)
        s.set_material(eps)
        s.add_dipole(np.array(src) * H, (0.0, 0.0, 1.0), ems.WAVE_RICKER, f0, 1.0)
        for r in recs:
            s.add_receiver(np.array(r) * H)
        s.run(2000)
        out[precision] = (s.time_step()[0], s.traces())
    dt = out[ems.FP32][0]
    assert out[ems.FP64][0] == dt
    tr_o, _, _ = oracle.tet_run(n, eps, oracle.SYMP4, dt / TS, 2000, 1, [(src, (0.0, 0.0, 1.0), 1, f0 * TS, 1.0)], recs)
    assert np.abs(tr_o[..., 1:]).max() > 0
    assert rel_l2(out[ems.FP64][1][..., 1:], tr_o[..., 1:]) < 1e-9
    assert rel_l2(out[ems.FP32][1][..., 1:], tr_o[..., 1:]) < FP32_TOL


def _blob_eps(n, seed):
    # background 2 plus three Gaussian blobs (amplitude U[1,3], width U[4,8]
    # cells) at the tetrahedron centroids
    rng = np.random.default_rng(seed)
    perm = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    off = np.zeros((6, 3))
    for p, (a, b, c) in enumerate(perm):
        off[p, a], off[p, b], off[p, c] = 0.75, 0.5, 0.25
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    corner = np.stack([i.ravel(), j.ravel(), k.ravel()], 1).astype(float)
    cen = (corner[:, None, :] + off[None, :, :]).reshape(-1, 3)
    eps = np.full(cen.shape[0], 2.0)
    for _ in range(3):
        c = rng.uniform(0.25, 0.75, 3) * n
        amp, width = rng.uniform(1.0, 3.0), rng.uniform(4.0, 8.0)
        eps += amp * np.exp(-np.sum((cen - c) ** 2, 1) / (2 * width ** 2))
    return eps


@pytest.mark.parametrize("side,steps,model", [(40, 3000, "uniform16"), (48, 4000, "blobs")],
                         ids=["n40_3000_steps", "n48_4000_steps"])
def test_fp32_long_runs_within_1e4_of_fp64(side, steps, model):
    # the run lengths of the batched (40^3 is the largest shot, 3000 steps,
    # eps_r U[1,6]) and inversion (48^3 blob model, 4000 steps) workloads:
    # FP32 traces against the FP64 GPU path of the same handle
    # configuration (the FP64 path is within 1e-9 of the oracle at 2000
    # steps, above), 1e-4 over the whole run
    n = (side, side, side)
    rng = np.random.default_rng(side)
    eps = rng.uniform(1.0, 6.0, 6 * side ** 3) if model == "uniform16" else _blob_eps(side, side)
    f0 = C0 / (10 * H * np.sqrt(np.mean(eps)))
    src = tuple(rng.uniform(0.3, 0.7, 3) * side)
    recs = [tuple(rng.uniform(0.2, 0.8, 3) * side) for _ in range(4)]
    out = {}
    dt = None
    for precision in (ems.FP64, ems.FP32):
        s = ems.TetFemSimulation(n, H, 1, ems.SYMP4, precision, dt=dt or 0.0, cfl_fraction=0.9)
        s.set_material(eps)
        s.add_dipole(np.array(src) * H, (0.0, 0.0, 1.0), ems.WAVE_RICKER, f0, 1.0)
        for r in recs:
            s.add_receiver(np.array(r) * H)
        dt = dt or s.time_step()[0]
        s.run(steps)
        out[precision] = s.traces()
        s.close()
    assert np.abs(out[ems.FP64][..., 1:]).max() > 0
    assert rel_l2(out[ems.FP32][..., 1:], out[ems.FP64][..., 1:]) < FP32_TOL


def test_fp32_field_access_carries_the_compensation():
    # an FP32 symplectic handle keeps P as hi + lo (FP32 value plus a
    # bfloat16 compensation); get_field returns the sum, set_field splits a
    # double again, so a round trip of P keeps about 24 + 8 significant bits
    # and one of U (plain FP32) 24
    n = (5, 4, 6)
    _, nslot, ntet = oracle.tet_sizes(n)
    rng = np.random.default_rng(31)
    eps = rng.uniform(1, 4, ntet)
    pec = oracle.tet_pec_mask(n)
    U0 = np.where(pec, 0.0, rng.standard_normal(nslot))
    P0 = np.where(pec, 0.0, rng.standard_normal(nslot))
    s = ems.TetFemSimulation(n, H, 1, ems.SYMP4, ems.FP32, dt=0.0, cfl_fraction=0.5)
    s.set_material(eps)
    s.set_field(0, U0)
    s.set_field(1, P0)
    rel = lambda a, b: np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-30))
    assert rel(s.get_field(1), P0) < 2.0 ** -30
    assert rel(s.get_field(0), U0) < 2.0 ** -23
    assert np.array_equal(s.get_field(1)[pec], np.zeros(pec.sum()))
    # a continued run equals one run of the same total length
    a = ems.TetFemSimulation(n, H, 1, ems.SYMP4, ems.FP32, dt=0.0, cfl_fraction=0.5)
    a.set_material(eps)
    a.set_field(0, U0)
    a.set_field(1, P0)
    a.run(40)
    s.run(25)
    s.run(15)
    assert rel_l2(s.get_field(0), a.get_field(0)) < 1e-6
    assert rel_l2(s.get_field(1), a.get_field(1)) < 1e-6


def _cavity_mode_U(L):
    """Edge integrals of the PEC cavity mode E = (0, 0, sin(pi x/L) sin(pi y/L))
    (omega = pi sqrt(2) / L, unit cells) on the slots of the L^3 mesh."""
    n = (L, L, L)
    nnode, nslot, _ = oracle.tet_sizes(n)
    g, w = np.polynomial.legendre.leggauss(8)
    s, w = 0.5 * (g + 1), 0.5 * w
    v = np.arange(nnode)
    i, j = v % (L + 1), (v // (L + 1)) % (L + 1)
    U = np.zeros(nslot)
    for d, dv in enumerate(oracle.TET_DIRS):
        if dv[2]:
            x, y = i[:, None] + s * dv[0], j[:, None] + s * dv[1]
            U[7 * v + d] = (np.sin(np.pi * x / L) * np.sin(np.pi * y / L)) @ w
    U[oracle.tet_pec_mask(n)] = 0.0
    return U


def _fit_omega(t, y, w0):
    """omega of the best fit a cos(omega t) to y (grid search, then refinement)."""
    def resid(om):
        c = np.cos(om * t)
        return np.sum((y - (c @ y) / (c @ c) * c) ** 2)
    om = min(np.linspace(0.97 * w0, 1.03 * w0, 601), key=resid)
    for h in (1e-4, 1e-5, 1e-6):
        om = min(om + w0 * h * np.arange(-60, 61), key=resid)
    return om


def test_analytic_cavity_mode_converges_on_the_gpu():
    """The Whitney interpolant of an analytic PEC cavity mode, released with
    P = 0, oscillates at the scheme's discrete frequency: FP32 and FP64 GPU
    traces at the centre over three periods on the 16^3 and 32^3 (headline
    resolution) meshes, symp4 at half the stability limit.  The fitted
    frequency approaches pi sqrt(2) / L (0.57% and 0.27% low: the block-
    lumped mass converges at first order here, the consistent mass at h^2);
    FP32 stays within 1e-4 of FP64, FP64 within 1e-9 of the oracle."""
    errs = []
    for L in (16, 32):
        n = (L, L, L)
        U0 = _cavity_mode_U(L)
        w0 = np.pi * np.sqrt(2) / L
        rec = (L / 2 + 0.31, L / 2 + 0.17, L / 2 + 0.23)   # inside a tetrahedron, near the centre
        tr = {}
        for prec in (ems.FP64, ems.FP32):
            s = ems.TetFemSimulation(n, H, 1, ems.SYMP4, prec, dt=0.0, cfl_fraction=0.5)
            s.set_material(np.ones(6 * L ** 3))
            s.add_receiver(np.array(rec) * H)
            dtn = s.time_step()[0] / TS
            nsteps = int(np.ceil(3 * 2 * np.pi / w0 / dtn))
            s.set_field(0, U0)
            s.run(nsteps)
            tr[prec] = s.traces()[0].copy()
            s.close()
        t = tr[ems.FP64][:, 0] / TS
        assert rel_l2(tr[ems.FP32][:, 1:], tr[ems.FP64][:, 1:]) < 1e-4
        if L == 16:
            tr_o, _, _ = oracle.tet_run(n, np.ones(6 * L ** 3), oracle.SYMP4, dtn, nsteps, 1, [], [rec], U=U0)
            assert rel_l2(tr[ems.FP64][:, 1:], tr_o[0][:, 1:]) < 1e-9
        errs.append(abs(_fit_omega(t, tr[ems.FP32][:, 3], w0) - w0) / w0)
    assert errs[1] < 0.004, errs
    assert errs[0] / errs[1] > 1.7, errs
