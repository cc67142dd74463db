"""Conductivity on the tetrahedral GPU path against the FP64 oracle: traces
of lossy runs (leapfrog, symp2, symp4; FP64 within 1e-10, FP32 within
1e-4), the FP64 gradients with respect to eps and sigma within 1e-9 of the
oracle adjoint, sigma = 0 leaving runs unchanged bit for bit, and lossy
batches equal to their single shots.  The API takes sigma in S/m; the
oracle works in normalised units, sigma_n = sigma (h / c0) / eps0."""
import numpy as np
import pytest

import oracle
from gpu_util import rel_l2
import emsolvers_gb300 as ems

pytestmark = pytest.mark.gpu
C0 = 299792458.0
EPS0 = 8.8541878128e-12
H = 1e-3
TS = H / C0
SIG_UNIT = TS / EPS0          # sigma_n per S/m
INTEG = {oracle.LEAPFROG: ems.LEAPFROG, oracle.SYMP2: ems.SYMP2, oracle.SYMP4: ems.SYMP4}


def _case(n, seed, integ, cfl=0.8):
    _, _, ntet = oracle.tet_sizes(n)
    rng = np.random.default_rng(seed)
    eps = rng.uniform(1.0, 4.0, ntet)
    sig_n = rng.uniform(0.02, 0.3, ntet)
    dips = [((n[0] * 0.41, n[1] * 0.52, n[2] * 0.47), (0.2, 0.3, 1.0), 1, 0.12, 1.0)]
    recs = [(n[0] * 0.7, n[1] * 0.5, n[2] * 0.5), (n[0] * 0.25, n[1] * 0.3, n[2] * 0.6)]
    dtn = cfl * oracle.stability_constant(integ) / np.sqrt(oracle.tet_lambda_max(n, eps, 300))
    return eps, sig_n, dips, recs, dtn


def _sim(n, eps, sig_n, dips, recs, integ, dtn, precision, nsnap=0):
    s = ems.TetFemSimulation(n, H, 1, INTEG[integ], precision, dt=dtn * TS)
    s.set_material(eps, None if sig_n is None else sig_n / SIG_UNIT)
    for d in dips:
        s.add_dipole(np.array(d[0]) * H, d[1], ems.WAVE_RICKER, d[3] / TS, d[4])
    for r in recs:
        s.add_receiver(np.array(r) * H)
    if nsnap:
        s.set_checkpoints(nsnap)
    return s


@pytest.mark.parametrize("integ", [oracle.LEAPFROG, oracle.SYMP2, oracle.SYMP4], ids=["leapfrog", "symp2", "symp4"])
@pytest.mark.parametrize("precision,tol", [(ems.FP64, 1e-10), (ems.FP32, 1e-4)], ids=["fp64", "fp32"])
def test_lossy_traces_match_the_oracle(integ, precision, tol):
    n, nsteps = (6, 5, 5), 150
    eps, sig_n, dips, recs, dtn = _case(n, 3, integ)
    tr_o, _, _ = oracle.tet_run(n, eps, integ, dtn, nsteps, 1, dips, recs, sigma=sig_n)
    s = _sim(n, eps, sig_n, dips, recs, integ, dtn, precision)
    s.run(nsteps)
    assert rel_l2(s.traces()[..., 1:], tr_o[..., 1:]) < tol
    # the losses matter at this size: the lossless traces differ at the percent level
    tr_0, _, _ = oracle.tet_run(n, eps, integ, dtn, nsteps, 1, dips, recs)
    assert rel_l2(tr_0[..., 1:], tr_o[..., 1:]) > 1e-2


@pytest.mark.parametrize("integ", [oracle.LEAPFROG, oracle.SYMP4], ids=["leapfrog", "symp4"])
def test_zero_conductivity_runs_are_bitwise_the_lossless_runs(integ):
    n = (5, 4, 6)
    eps, _, dips, recs, dtn = _case(n, 4, integ)
    a = _sim(n, eps, None, dips, recs, integ, dtn, ems.FP32)
    b = _sim(n, eps, np.zeros_like(eps), dips, recs, integ, dtn, ems.FP32)
    a.run(60)
    b.run(60)
    assert np.array_equal(a.traces(), b.traces())
    assert np.array_equal(a.get_field(0), b.get_field(0))


@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4], ids=["symp2", "symp4"])
@pytest.mark.parametrize("nsnap", [1, 5, 37], ids=["one_segment", "uneven_segments", "step_per_segment"])
def test_fp64_eps_and_sigma_gradients_match_the_oracle_adjoint(integ, nsnap):
    n, nsteps = (4, 3, 5), 37
    eps, sig_n, dips, recs, dtn = _case(n, 5, integ)
    tr_o, _, _ = oracle.tet_run(n, eps, integ, dtn, nsteps, 1, dips, recs, sigma=sig_n)
    rng = np.random.default_rng(1)
    resid = 0.3 * tr_o + 0.05 * rng.standard_normal(tr_o.shape) * np.abs(tr_o[..., 1:]).max()
    resid[..., 0] = 0.0
    ge_o, gs_o = oracle.tet_gradient(n, eps, integ, dtn, nsteps, resid, 1, dips, recs, sigma=sig_n)
    s = _sim(n, eps, sig_n, dips, recs, integ, dtn, ems.FP64, nsnap)
    s.reset()
    s.run(nsteps)
    assert rel_l2(s.traces()[..., 1:], tr_o[..., 1:]) < 1e-10
    ge, gs = s.backward(resid, sigma=True)
    assert rel_l2(ge, ge_o) < 1e-9
    assert rel_l2(gs, gs_o * SIG_UNIT) < 1e-9


def test_fp32_lossy_gradient_within_1e3_of_the_oracle():
    integ, n, nsteps = oracle.SYMP4, (8, 7, 8), 200
    eps, sig_n, dips, recs, dtn = _case(n, 9, integ, cfl=0.9)
    tr_o, _, _ = oracle.tet_run(n, eps, integ, dtn, nsteps, 1, dips, recs, sigma=sig_n)
    resid = 0.3 * tr_o
    resid[..., 0] = 0.0
    ge_o, gs_o = oracle.tet_gradient(n, eps, integ, dtn, nsteps, resid, 1, dips, recs, sigma=sig_n)
    s = _sim(n, eps, sig_n, dips, recs, integ, dtn, ems.FP32, 12)
    s.reset()
    s.run(nsteps)
    ge, gs = s.backward(resid, sigma=True)
    assert rel_l2(ge, ge_o) < 1e-3
    assert rel_l2(gs, gs_o * SIG_UNIT) < 1e-3


def test_lossy_batch_gradient_equals_single_shot_gradients():
    cells = [(4, 5, 3), (5, 4, 4)]
    rng = np.random.default_rng(4)
    eps = [rng.uniform(1, 4, 6 * c[0] * c[1] * c[2]) for c in cells]
    sig = [rng.uniform(0.0, 0.3, e.size) / SIG_UNIT for e in eps]
    dt = 0.7 * 2.0 * TS / np.sqrt(max(oracle.tet_lambda_max(c, e, 100) for c, e in zip(cells, eps)))
    src = [np.array(c) * 0.45 * H for c in cells]
    rec = [[np.array(c) * f * H for f in (0.3, 0.7)] for c in cells]
    b = ems.TetFemBatch(cells, H, integrator=ems.SYMP4, precision=ems.FP32, dt=dt)
    b.set_material(np.concatenate(eps), np.concatenate(sig))
    for s in range(2):
        b.add_dipole(s, src[s], (0.1, 0.2, 1.0), ems.WAVE_RICKER, 0.1 / TS)
        for r in rec[s]:
            b.add_receiver(s, r)
    b.set_checkpoints(3)
    b.reset()
    b.run(40)
    rb = 0.5 * b.traces()
    rb[..., 0] = 0.0
    gbe, gbs = b.backward(rb, sigma=True)
    off = 0
    for s, c in enumerate(cells):
        one = ems.TetFemSimulation(c, H, 1, ems.SYMP4, ems.FP32, dt=dt)
        one.set_material(eps[s], sig[s])
        one.add_dipole(src[s], (0.1, 0.2, 1.0), ems.WAVE_RICKER, 0.1 / TS)
        for r in rec[s]:
            one.add_receiver(r)
        one.set_checkpoints(3)
        one.reset()
        one.run(40)
        ge, gs = one.backward(rb[2 * s:2 * s + 2], sigma=True)
        assert np.array_equal(ge, gbe[off:off + ge.size])
        assert np.array_equal(gs, gbs[off:off + gs.size])
        off += ge.size


def test_negative_conductivity_is_rejected():
    n = (3, 3, 3)
    _, _, ntet = oracle.tet_sizes(n)
    s = ems.TetFemSimulation(n, H, 1, ems.SYMP2, ems.FP32, dt=1e-13)
    with pytest.raises(ems.EmsError) as e:
        s.set_material(np.ones(ntet), np.full(ntet, -0.01))
    assert e.value.status == -1
