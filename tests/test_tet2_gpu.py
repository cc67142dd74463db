"""Second-order (20-DOF) tetrahedra on the GPU through the C ABI against the
FP64 oracle (orc_tet2.c).

Tolerances (relative L2): FP64 GPU vs FP64 oracle 1e-10 (sums in another
order, the same Chebyshev polynomial); FP32 GPU vs FP64 1e-4 on receiver
traces, the bound of the FP32 path.  The API orders DOFs node-major
(38 * node + plane); the oracle keeps planes (plane * nnode + node)."""
import numpy as np
import pytest

import oracle
from gpu_util import rel_l2
import emsolvers_gb300 as ems

pytestmark = pytest.mark.gpu
C0 = 299792458.0
H = 1e-3
TS = H / C0
FP64_TOL = 1e-10
FP32_TOL = 1e-4
INTEG = {oracle.SYMP2: ems.SYMP2, oracle.SYMP4: ems.SYMP4, oracle.LEAPFROG: ems.LEAPFROG}


def to_api(n, x):
    nnode, _, _ = oracle.tet2_sizes(n)
    return np.asarray(x).reshape(38, nnode).T.reshape(-1)


def from_api(n, x):
    nnode, _, _ = oracle.tet2_sizes(n)
    return np.asarray(x).reshape(nnode, 38).T.reshape(-1)


def _case(n, seed):
    _, _, ntet = oracle.tet2_sizes(n)
    rng = np.random.default_rng(seed)
    eps = rng.uniform(1.0, 4.0, ntet)
    dip = ((n[0] * 0.41, n[1] * 0.52, n[2] * 0.47), (0.2, 0.3, 1.0), 1, 0.08, 1.0)
    recs = [(n[0] * 0.7, n[1] * 0.5, n[2] * 0.5), (n[0] * 0.25, n[1] * 0.3, n[2] * 0.6)]
    return eps, dip, recs


def _gpu(n, eps, dip, recs, integ, dtn, nsteps, precision, tf=1):
    s = ems.TetFemSimulation(n, H, 2, INTEG[integ], precision, dt=dtn * TS, time_frequency=tf)
    s.set_material(eps)
    s.add_dipole(np.array(dip[0]) * H, dip[1], ems.WAVE_RICKER, dip[3] / TS, dip[4])
    for r in recs:
        s.add_receiver(np.array(r) * H)
    s.run(nsteps)
    return s


@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4, oracle.LEAPFROG])
def test_fp64_matches_oracle(integ):
    n = (5, 4, 4)
    eps, dip, recs = _case(n, 7)
    dtn = 0.8 * oracle.stability_constant(integ) / np.sqrt(oracle.tet2_lambda_max(n, eps, 200))
    tr_o, U_o, P_o = oracle.tet2_run(n, eps, integ, dtn, 120, 2, [dip], recs)
    s = _gpu(n, eps, dip, recs, integ, dtn, 120, ems.FP64, tf=2)
    t = s.traces()
    np.testing.assert_allclose(t[:, :, 0], tr_o[:, :, 0] * TS, rtol=1e-12)
    assert rel_l2(t[:, :, 1:], tr_o[:, :, 1:]) < FP64_TOL
    assert rel_l2(from_api(n, s.get_field(0)), U_o) < FP64_TOL
    assert rel_l2(from_api(n, s.get_field(1)), P_o) < FP64_TOL


def test_run_continues_across_calls():
    n = (4, 4, 5)
    eps, dip, recs = _case(n, 9)
    dtn = 0.8 * oracle.stability_constant(oracle.SYMP4) / np.sqrt(oracle.tet2_lambda_max(n, eps, 200))
    _, U_o, P_o = oracle.tet2_run(n, eps, oracle.SYMP4, dtn, 60, 1, [dip], recs)
    s = ems.TetFemSimulation(n, H, 2, ems.SYMP4, ems.FP64, dt=dtn * TS)
    s.set_material(eps)
    s.add_dipole(np.array(dip[0]) * H, dip[1], ems.WAVE_RICKER, dip[3] / TS, dip[4])
    s.run(25)
    s.run(35)
    assert rel_l2(from_api(n, s.get_field(0)), U_o) < FP64_TOL
    # a state set through the API is taken up by the next run
    U1, P1 = s.get_field(0), s.get_field(1)
    s.reset()
    s.set_field(0, U1)
    s.set_field(1, P1)
    s.run(20)
    _, U_o2, _ = oracle.tet2_run(n, eps, oracle.SYMP4, dtn, 20, 1, [], [], U=U_o, P=P_o)
    # the dipole keeps acting: compare against the oracle with the source at t = 0 instead
    s2 = ems.TetFemSimulation(n, H, 2, ems.SYMP4, ems.FP64, dt=dtn * TS)
    s2.set_material(eps)
    s2.set_field(0, U1)
    s2.set_field(1, P1)
    s2.run(20)
    assert rel_l2(from_api(n, s2.get_field(0)), U_o2) < FP64_TOL


@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4])
def test_fp32_traces_within_1e4_of_fp64(integ):
    n = (10, 10, 10)
    eps, dip, recs = _case(n, 11)
    dtn = 0.9 * oracle.stability_constant(integ) / np.sqrt(oracle.tet2_lambda_max(n, eps, 200))
    tr_o, U_o, _ = oracle.tet2_run(n, eps, integ, dtn, 300, 1, [dip], recs)
    s = _gpu(n, eps, dip, recs, integ, dtn, 300, ems.FP32)
    assert rel_l2(s.traces()[:, :, 1:], tr_o[:, :, 1:]) < FP32_TOL
    assert rel_l2(from_api(n, s.get_field(0)), U_o) < FP32_TOL


@pytest.mark.parametrize("steps", [2000, 4000])
def test_fp32_long_runs_within_1e4_of_the_fp64_gpu_path(steps):
    """Long runs where FP32 rounding in the kick would accumulate (the
    gradient null space of K): the FP32 path against the FP64 GPU path,
    which the test above pins to the oracle."""
    n = (14, 14, 14)
    eps, dip, recs = _case(n, 13)
    recs = recs + [(n[0] * 0.5, n[1] * 0.8, n[2] * 0.3)]
    dtn = 0.9 * oracle.stability_constant(oracle.SYMP4) / np.sqrt(oracle.tet2_lambda_max(n, eps, 200))
    dip = (dip[0], dip[1], dip[2], 1.0 / (10 * np.sqrt(2.5)), dip[4])   # 10 cells per wavelength
    t64 = _gpu(n, eps, dip, recs, oracle.SYMP4, dtn, steps, ems.FP64).traces()
    t32 = _gpu(n, eps, dip, recs, oracle.SYMP4, dtn, steps, ems.FP32).traces()
    assert rel_l2(t32[:, :, 1:], t64[:, :, 1:]) < FP32_TOL


@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4, oracle.LEAPFROG])
def test_automatic_time_step_matches_oracle_stability_limit(integ):
    n = (6, 5, 5)
    eps, _, _ = _case(n, 3)
    s = ems.TetFemSimulation(n, H, 2, INTEG[integ], ems.FP64, dt=0.0, cfl_fraction=0.9)
    s.set_material(eps)
    dt, lim = s.time_step()
    lim_o = oracle.stability_constant(integ) / np.sqrt(oracle.tet2_lambda_max(n, eps, 600)) * TS
    assert abs(lim - lim_o) / lim_o < 2e-3
    assert abs(dt - 0.9 * lim) / dt < 1e-12


def test_stiffness_and_energy_match_oracle():
    n = (4, 5, 4)
    _, ndof, ntet = oracle.tet2_sizes(n)
    rng = np.random.default_rng(4)
    eps = rng.uniform(1, 4, ntet)
    pec = oracle.tet2_pec_mask(n)
    U = np.where(pec, 0.0, rng.standard_normal(ndof))
    P = np.where(pec, 0.0, rng.standard_normal(ndof))
    s = ems.TetFemSimulation(n, H, 2, ems.SYMP4, ems.FP64, dt=0.1 * TS)
    s.set_material(eps)
    f = from_api(n, s.apply_stiffness(to_api(n, U)))
    assert rel_l2(f, oracle.tet2_apply(n, U, True)) < 1e-13
    s.set_field(0, to_api(n, U))
    s.set_field(1, to_api(n, P))
    e = float(np.ravel(s.energy())[0])
    assert abs(e - oracle.tet2_energy(n, eps, U, P)) / abs(e) < 1e-12


def test_batch_shots_equal_single_runs_bitwise():
    cells = [(4, 4, 4), (6, 5, 4), (5, 6, 7)]
    rng = np.random.default_rng(21)
    dtn = 0.05
    b = ems.TetFemBatch(cells, H, order=2, integrator=ems.SYMP4, precision=ems.FP32, dt=dtn * TS)
    epss, singles = [], []
    for k, c in enumerate(cells):
        eps = rng.uniform(1, 4, 6 * c[0] * c[1] * c[2])
        epss.append(eps)
        s = ems.TetFemSimulation(c, H, 2, ems.SYMP4, ems.FP32, dt=dtn * TS)
        s.set_material(eps)
        pos = (np.array(c) * 0.45) * H
        s.add_dipole(pos, (0, 0, 1), ems.WAVE_RICKER, 0.09 / TS, 1.0)
        s.add_receiver(np.array(c) * 0.6 * H)
        s.run(80)
        singles.append(s.traces())
        b.add_dipole(k, pos, (0, 0, 1), ems.WAVE_RICKER, 0.09 / TS, 1.0)
        b.add_receiver(k, np.array(c) * 0.6 * H)
    b.set_material(np.concatenate(epss))
    b.run(80)
    tb = b.traces()
    for k in range(len(cells)):
        assert np.array_equal(tb[k], singles[k][0])


def test_fp32_runs_are_bitwise_deterministic():
    n = (6, 6, 6)
    eps, dip, recs = _case(n, 5)
    a = _gpu(n, eps, dip, recs, oracle.SYMP4, 0.1, 60, ems.FP32)
    b = _gpu(n, eps, dip, recs, oracle.SYMP4, 0.1, 60, ems.FP32)
    assert np.array_equal(a.traces(), b.traces())
    assert np.array_equal(a.get_field(0), b.get_field(0))


def test_order2_rejects_conductivity_and_leapfrog_adjoint():
    n = (3, 3, 3)
    s = ems.TetFemSimulation(n, H, 2, ems.SYMP4, ems.FP32, dt=0.1 * TS)
    sigma = np.full(6 * 27, 0.01)
    with pytest.raises(ems.EmsError):
        s.set_material(np.ones(6 * 27), sigma)
    lf = ems.TetFemSimulation(n, H, 2, ems.LEAPFROG, ems.FP32, dt=0.1 * TS)
    with pytest.raises(ems.EmsError):
        lf.set_checkpoints(4)


def _adjoint(n, eps, dip, recs, integ, dtn, steps, precision, nsnap, g, batch=1, tf=1):
    if batch == 1:
        s = ems.TetFemSimulation(n, H, 2, INTEG[integ], precision, dt=dtn * TS, time_frequency=tf)
        s.set_material(eps)
        s.add_dipole(np.array(dip[0]) * H, dip[1], ems.WAVE_RICKER, dip[3] / TS, dip[4])
        for r in recs:
            s.add_receiver(np.array(r) * H)
    else:
        s = ems.TetFemBatch([n] * batch, H, order=2, integrator=INTEG[integ], precision=precision, dt=dtn * TS)
        s.set_material(np.tile(eps, batch))
        for k in range(batch):
            s.add_dipole(k, np.array(dip[0]) * H, dip[1], ems.WAVE_RICKER, dip[3] / TS, dip[4])
            for r in recs:
                s.add_receiver(k, np.array(r) * H)
    s.set_checkpoints(nsnap)
    s.reset()
    s.run(steps)
    tr = s.traces()
    gg = np.tile(g, (batch, 1, 1)) if batch > 1 else g
    return tr, s.backward(gg)


@pytest.mark.parametrize("integ,nsnap,tf", [(oracle.SYMP4, 4, 1), (oracle.SYMP2, 7, 1), (oracle.SYMP4, 5, 3)])
def test_fp64_adjoint_matches_oracle(integ, nsnap, tf):
    n = (3, 4, 3)
    _, _, ntet = oracle.tet2_sizes(n)
    rng = np.random.default_rng(31)
    eps = rng.uniform(1, 4, ntet)
    dip = ((1.4, 1.6, 1.5), (0.2, 0.3, 1.0), 1, 0.25, 1.0)
    recs = [(2.2, 1.3, 1.7), (0.8, 2.1, 1.2)]
    steps, dtn = 30, 0.1
    tr_o, _, _ = oracle.tet2_run(n, eps, integ, dtn, steps, tf, [dip], recs)
    g = rng.standard_normal(tr_o.shape)
    g[..., 0] = 0.0
    grad_o = oracle.tet2_gradient(n, eps, integ, dtn, steps, g, tf, [dip], recs)
    tr, grad = _adjoint(n, eps, dip, recs, integ, dtn, steps, ems.FP64, nsnap, g, tf=tf)
    assert rel_l2(tr[..., 1:], tr_o[..., 1:]) < FP64_TOL
    assert rel_l2(grad, grad_o) < 1e-9


def test_fp32_adjoint_close_to_fp64_and_batch_equals_single():
    n = (6, 6, 6)
    _, _, ntet = oracle.tet2_sizes(n)
    rng = np.random.default_rng(33)
    eps = rng.uniform(1, 4, ntet)
    dip = ((2.6, 3.1, 2.9), (0.0, 0.0, 1.0), 1, 0.12, 1.0)
    recs = [(4.2, 1.3, 3.7), (1.8, 4.1, 2.2), (3.3, 3.3, 4.6)]
    steps, dtn = 200, 0.12
    tr64, _ = _adjoint(n, eps, dip, recs, oracle.SYMP4, dtn, steps, ems.FP64, 8, np.zeros((3, steps, 4)))
    g = np.zeros_like(tr64)
    g[..., 1:] = tr64[..., 1:] * rng.uniform(0.5, 1.5, tr64[..., 1:].shape)
    _, g64 = _adjoint(n, eps, dip, recs, oracle.SYMP4, dtn, steps, ems.FP64, 8, g)
    _, g32 = _adjoint(n, eps, dip, recs, oracle.SYMP4, dtn, steps, ems.FP32, 8, g)
    assert rel_l2(g32, g64) < 1e-3
    _, gb = _adjoint(n, eps, dip, recs, oracle.SYMP4, dtn, steps, ems.FP32, 8, g, batch=2)
    assert np.array_equal(gb[:ntet], g32) and np.array_equal(gb[ntet:], g32)


def test_both_iteration_forms_match_the_oracle():
    """The fused and the two-pass Chebyshev iteration (chosen per handle by
    timing) give the same bits, so the choice never changes a result, and
    reproduce the oracle; each is forced here in a fresh process through
    EMS_TET2_ITERATION."""
    import os
    import subprocess
    import sys
    n = (4, 5, 4)
    eps, dip, recs = _case(n, 17)
    dtn = 0.8 * oracle.stability_constant(oracle.SYMP4) / np.sqrt(oracle.tet2_lambda_max(n, eps, 200))
    tr_o, _, _ = oracle.tet2_run(n, eps, oracle.SYMP4, dtn, 60, 1, [dip], recs)
    code = (
        "import sys, numpy as np, emsolvers_gb300 as ems\n"
        f"n = {n!r}; H = {H!r}; TS = {TS!r}\n"
        "eps = np.load(sys.argv[1])\n"
        f"s = ems.TetFemSimulation(n, H, 2, ems.SYMP4, ems.{{p}}, dt={dtn!r} * TS)\n"
        "s.set_material(eps)\n"
        f"s.add_dipole(np.array({dip[0]!r}) * H, {dip[1]!r}, ems.WAVE_RICKER, {dip[3]!r} / TS, {dip[4]!r})\n"
        f"for r in {recs!r}:\n"
        "    s.add_receiver(np.array(r) * H)\n"
        "s.run(60)\n"
        "np.save(sys.argv[2], s.traces())\n")
    path_e = f"/tmp/ems_t2_eps_{os.getpid()}.npy"
    np.save(path_e, eps)
    out = {}
    forms = ("fused", "twopass")
    for form in forms:
        for prec in ("FP64", "FP32"):
            env = dict(os.environ, EMS_TET2_ITERATION=form)
            path = f"/tmp/ems_t2_{form}_{prec}_{os.getpid()}.npy"
            r = subprocess.run([sys.executable, "-c", code.replace("{p}", prec), path_e, path], env=env,
                               capture_output=True, text=True, timeout=300)
            assert r.returncode == 0, r.stderr
            out[form, prec] = np.load(path)
            os.remove(path)
    os.remove(path_e)
    for prec in ("FP64", "FP32"):
        assert np.array_equal(out["fused", prec], out["twopass", prec])
    for form in forms:
        assert rel_l2(out[form, "FP64"][..., 1:], tr_o[..., 1:]) < FP64_TOL
        assert rel_l2(out[form, "FP32"][..., 1:], tr_o[..., 1:]) < FP32_TOL
