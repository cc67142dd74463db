"""Discrete adjoint of the tetrahedral solver on the GPU: the FP64 gradient
against the FP64 oracle adjoint (any snapshot count), the FP32 gradient
against FP64, gradients against central finite differences of GPU FP64
runs (L2 and TF envelope misfits), batches against single shots, the
torch.autograd bridge, and the error paths.

Tolerances (relative L2 over all tetrahedra): FP64 GPU vs FP64 oracle 1e-9
(the GPU runs the merged drifts and a different summation order); FP32 GPU
vs FP64 oracle 1e-3; central differences (h = 1e-4 on eps_r) 1e-6."""
import numpy as np
import pytest

import oracle
from gpu_util import rel_l2
import emsolvers_gb300 as ems

pytestmark = pytest.mark.gpu
C0 = 299792458.0
H = 1e-3
TS = H / C0
INTEG = {oracle.SYMP2: ems.SYMP2, oracle.SYMP4: ems.SYMP4}


def _case(n, seed, integ, cfl=0.8):
    _, _, ntet = oracle.tet_sizes(n)
    rng = np.random.default_rng(seed)
    eps = rng.uniform(1.0, 4.0, ntet)
    dips = [((n[0] * 0.41, n[1] * 0.52, n[2] * 0.47), (0.2, 0.3, 1.0), 1, 0.12, 1.0),
            ((n[0] * 0.63, n[1] * 0.35, n[2] * 0.55), (1.0, -0.4, 0.1), 1, 0.09, 0.7)]
    recs = [(n[0] * 0.7, n[1] * 0.5, n[2] * 0.5), (n[0] * 0.25, n[1] * 0.3, n[2] * 0.6),
            (n[0] * 0.52, n[1] * 0.77, n[2] * 0.31)]
    dtn = cfl * oracle.stability_constant(integ) / np.sqrt(oracle.tet_lambda_max(n, eps, 300))
    return eps, dips, recs, dtn


def _sim(n, eps, dips, recs, integ, dtn, precision, tf=1, nsnap=4):
    s = ems.TetFemSimulation(n, H, 1, INTEG[integ], precision, dt=dtn * TS, time_frequency=tf)
    s.set_material(eps)
    for d in dips:
        s.add_dipole(np.array(d[0]) * H, d[1], ems.WAVE_RICKER, d[3] / TS, d[4])
    for r in recs:
        s.add_receiver(np.array(r) * H)
    s.set_checkpoints(nsnap)
    return s


def _residual(traces, seed):
    rng = np.random.default_rng(seed)
    r = 0.3 * traces + 0.05 * rng.standard_normal(traces.shape) * np.abs(traces[..., 1:]).max()
    r[..., 0] = 0.0
    return r


@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4], ids=["symp2", "symp4"])
@pytest.mark.parametrize("nsnap", [1, 2, 5, 37],
                         ids=["one_segment", "odd_graph_remainder", "uneven_segments", "step_per_segment"])
def test_fp64_gradient_matches_oracle_adjoint(integ, nsnap):
    n, nsteps, tf = (4, 3, 5), 37, 2
    eps, dips, recs, dtn = _case(n, 5, integ)
    tr_o, _, _ = oracle.tet_run(n, eps, integ, dtn, nsteps, tf, dips, recs)
    resid = _residual(tr_o, 1)
    g_o = oracle.tet_gradient(n, eps, integ, dtn, nsteps, resid, tf, dips, recs)
    s = _sim(n, eps, dips, recs, integ, dtn, ems.FP64, tf, nsnap)
    s.reset()
    s.run(nsteps)
    assert rel_l2(s.traces()[..., 1:], tr_o[..., 1:]) < 1e-10
    g = s.backward(resid)
    assert rel_l2(g, g_o) < 1e-9


@pytest.mark.parametrize("nsnap", [3, 7, 40])
def test_recorded_forward_equals_plain_forward(nsnap):
    # a recorded run advances segment by segment (graph replays plus single
    # steps); it must give the same fields and traces bit for bit
    integ, n, nsteps = oracle.SYMP4, (9, 8, 7), 121
    eps, dips, recs, dtn = _case(n, 12, integ, cfl=0.9)
    plain = _sim(n, eps, dips, recs, integ, dtn, ems.FP32, 1, 0)
    plain.run(nsteps)
    rec = _sim(n, eps, dips, recs, integ, dtn, ems.FP32, 1, nsnap)
    rec.reset()
    rec.run(nsteps)
    assert np.array_equal(plain.traces(), rec.traces())
    assert np.array_equal(plain.get_field(0), rec.get_field(0))
    assert np.array_equal(plain.get_field(1), rec.get_field(1))


def test_fp32_gradient_within_1e3_of_fp64_oracle():
    integ, n, nsteps = oracle.SYMP4, (10, 9, 10), 300
    eps, dips, recs, dtn = _case(n, 9, integ, cfl=0.9)
    tr_o, _, _ = oracle.tet_run(n, eps, integ, dtn, nsteps, 1, dips, recs)
    resid = _residual(tr_o, 2)
    g_o = oracle.tet_gradient(n, eps, integ, dtn, nsteps, resid, 1, dips, recs)
    s = _sim(n, eps, dips, recs, integ, dtn, ems.FP32, 1, 16)
    s.reset()
    s.run(nsteps)
    g = s.backward(resid)
    assert rel_l2(g, g_o) < 1e-3


def _misfit_fd(integ, kind, band=None, seed=3):
    n, nsteps = (5, 4, 4), 60
    eps, dips, recs, dtn = _case(n, seed, integ)
    true = eps * np.random.default_rng(seed + 1).uniform(0.9, 1.1, eps.size)
    s = _sim(n, true, dips, recs, integ, dtn, ems.FP64, 1, 6)
    s.reset()
    s.run(nsteps)
    obs = s.traces()

    def J(e):
        s.set_material(e)
        s.reset()
        s.run(nsteps)
        return ems.trace_misfit(s.traces(), obs, kind, band)

    _, tg = J(eps)
    g = s.backward(tg)
    idx = np.argsort(-np.abs(g))[:3].tolist() + np.random.default_rng(seed).choice(eps.size, 3, replace=False).tolist()
    fd = []
    for t in idx:
        e1, e2 = eps.copy(), eps.copy()
        e1[t] += 1e-4
        e2[t] -= 1e-4
        fd.append((J(e1)[0] - J(e2)[0]) / 2e-4)
    return g[idx], np.array(fd)


@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4], ids=["symp2", "symp4"])
def test_l2_gradient_matches_central_differences(integ):
    g, fd = _misfit_fd(integ, ems.MISFIT_L2)
    assert np.abs(g - fd).max() < 1e-6 * np.abs(fd).max()


def test_tf_envelope_gradient_matches_central_differences():
    g, fd = _misfit_fd(oracle.SYMP4, ems.MISFIT_TF_ENVELOPE)
    assert np.abs(g - fd).max() < 1e-5 * np.abs(fd).max()


@pytest.mark.parametrize("precision", [ems.FP32, ems.FP64])
def test_batch_gradient_equals_single_shot_gradients(precision):
    cells = [(4, 5, 3), (5, 4, 4)]
    rng = np.random.default_rng(4)
    eps = [rng.uniform(1, 4, 6 * c[0] * c[1] * c[2]) for c in cells]
    dt = 0.7 * 2.0 * TS / np.sqrt(max(oracle.tet_lambda_max(c, e, 100) for c, e in zip(cells, eps)))
    src = [np.array(c) * 0.45 * H for c in cells]
    rec = [[np.array(c) * f * H for f in (0.3, 0.7)] for c in cells]
    b = ems.TetFemBatch(cells, H, integrator=ems.SYMP4, precision=precision, dt=dt)
    b.set_material(np.concatenate(eps))
    for s in range(2):
        b.add_dipole(s, src[s], (0.1, 0.2, 1.0), ems.WAVE_RICKER, 0.1 / TS)
        for r in rec[s]:
            b.add_receiver(s, r)
    b.set_checkpoints(3)
    b.reset()
    b.run(40)
    tb = b.traces()
    gb = b.backward(_residual(tb, 6))
    rb = _residual(tb, 6)
    off = 0
    for s, c in enumerate(cells):
        one = ems.TetFemSimulation(c, H, 1, ems.SYMP4, precision, dt=dt)
        one.set_material(eps[s])
        one.add_dipole(src[s], (0.1, 0.2, 1.0), ems.WAVE_RICKER, 0.1 / TS)
        for r in rec[s]:
            one.add_receiver(r)
        one.set_checkpoints(3)
        one.reset()
        one.run(40)
        g1 = one.backward(rb[2 * s:2 * s + 2])
        assert np.array_equal(g1, gb[off:off + g1.size])
        off += g1.size


def test_autograd_bridge_matches_oracle_adjoint():
    torch = pytest.importorskip("torch")
    from emsolvers_gb300.autograd import TetTraces
    integ, n, nsteps = oracle.SYMP4, (4, 4, 3), 30
    eps, dips, recs, dtn = _case(n, 8, integ)
    data = oracle.tet_run(n, eps * 1.05, integ, dtn, nsteps, 1, dips, recs)[0]
    s = _sim(n, eps, dips, recs, integ, dtn, ems.FP64, 1, 4)
    e = torch.tensor(eps, dtype=torch.float64, requires_grad=True)
    tr = TetTraces.apply(e, s, nsteps, 4)
    J = 0.5 * ((tr[..., 1:] - torch.from_numpy(data[..., 1:])) ** 2).sum()
    J.backward()
    resid = tr.detach().numpy() - data
    resid[..., 0] = 0.0
    g_o = oracle.tet_gradient(n, eps, integ, dtn, nsteps, resid, 1, dips, recs)
    assert rel_l2(e.grad.numpy(), g_o) < 1e-9


def test_backward_error_paths():
    n = (3, 3, 3)
    eps, dips, recs, dtn = _case(n, 2, oracle.SYMP2)
    s = _sim(n, eps, dips, recs, oracle.SYMP2, dtn, ems.FP64, 1, 0)
    s.run(10)
    with pytest.raises(ems.EmsError) as e:
        s.backward(np.zeros((3, 10, 4)))
    assert e.value.status == -5          # nothing recorded
    s.set_checkpoints(2)
    s.run(10)                            # not from the reset state: not recorded
    with pytest.raises(ems.EmsError):
        s.backward(np.zeros((3, 10, 4)))
    s.reset()
    s.run(10)
    with pytest.raises(ems.EmsError) as e:
        s.backward(np.zeros((3, 9, 4)))
    assert e.value.status == -1          # wrong trace-gradient length
    s.backward(np.zeros((3, 10, 4)))
    s.set_material(eps)                  # new mass blocks invalidate the recording
    with pytest.raises(ems.EmsError):
        s.backward(np.zeros((3, 10, 4)))
    lf = ems.TetFemSimulation(n, H, 1, ems.LEAPFROG, ems.FP64, dt=dtn * TS)
    with pytest.raises(ems.EmsError) as e:
        lf.set_checkpoints(2)
    assert e.value.status == -8


def test_one_call_gradient_equals_the_pipeline():
    integ, n, nsteps = oracle.SYMP4, (5, 4, 4), 50
    eps, dips, recs, dtn = _case(n, 14, integ)
    s = _sim(n, eps * 1.1, dips, recs, integ, dtn, ems.FP32, 1, 5)
    s.reset()
    s.run(nsteps)
    obs = s.traces()
    s.set_material(eps)
    J1, g1 = s.gradient(nsteps, obs, ems.MISFIT_TF_ENVELOPE, nsnap=5)
    s.set_checkpoints(5)
    s.reset()
    s.run(nsteps)
    J2, tg = ems.trace_misfit(s.traces(), obs, ems.MISFIT_TF_ENVELOPE)
    g2 = s.backward(tg)
    assert J1 == J2 and np.array_equal(g1, g2)
