"""Batched tetrahedral shots: every shot of a batch reproduces its own
stand-alone run bit for bit (same time step, FP32 and FP64), and the
automatic time step of a batch is that of its stiffest shot."""
import numpy as np
import pytest

import oracle
import emsolvers_gb300 as ems

pytestmark = pytest.mark.gpu
H = 1e-3
TS = H / 299792458.0


def _shots(seed, n=4):
    rng = np.random.default_rng(seed)
    cells = [tuple(int(v) for v in rng.integers(5, 10, 3)) for _ in range(n)]
    eps = [rng.uniform(1, 6, 6 * c[0] * c[1] * c[2]) for c in cells]
    src = [(np.array(c) * rng.uniform(0.3, 0.7, 3)) * H for c in cells]
    rec = [(np.array(c) * rng.uniform(0.2, 0.8, 3)) * H for c in cells]
    return cells, eps, src, rec


@pytest.mark.parametrize("precision", [ems.FP32, ems.FP64])
@pytest.mark.parametrize("integ", [ems.SYMP4, ems.LEAPFROG])
def test_batch_equals_individual_runs(precision, integ):
    cells, eps, src, rec = _shots(3)
    dt = 0.3 * 2.0 * TS / np.sqrt(max(oracle.tet_lambda_max(c, e, 100) for c, e in zip(cells, eps)))
    b = ems.TetFemBatch(cells, H, integrator=integ, precision=precision, dt=dt)
    b.set_material(np.concatenate(eps))
    for s in range(len(cells)):
        b.add_dipole(s, src[s], (0.1, 0.2, 1.0), ems.WAVE_RICKER, 0.08 / TS)
        b.add_receiver(s, rec[s])
    b.run(60)
    tb = b.traces()
    ub = b.get_field(0)
    off = 0
    for s, c in enumerate(cells):
        one = ems.TetFemSimulation(c, H, 1, integ, precision, dt=dt)
        one.set_material(eps[s])
        one.add_dipole(src[s], (0.1, 0.2, 1.0), ems.WAVE_RICKER, 0.08 / TS)
        one.add_receiver(rec[s])
        one.run(60)
        assert np.array_equal(one.traces()[0], tb[s])
        u1 = one.get_field(0)
        assert np.array_equal(u1, ub[off:off + u1.size])
        off += u1.size


def test_batch_time_step_is_the_stiffest_shots():
    cells, eps, _, _ = _shots(4, 3)
    b = ems.TetFemBatch(cells, H, integrator=ems.SYMP2, dt=0.0, cfl_fraction=0.9)
    b.set_material(np.concatenate(eps))
    dt, lim = b.time_step()
    lims = [2.0 * TS / np.sqrt(oracle.tet_lambda_max(c, e, 600)) for c, e in zip(cells, eps)]
    assert abs(lim - min(lims)) / min(lims) < 1e-4
