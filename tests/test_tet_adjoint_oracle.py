"""Checks of the FP64 oracle of the tetrahedral discrete adjoint (no reference
counterpart): the analytic derivative of the per-node mass blocks against
central differences of the block construction at interior, face, edge and
corner nodes, and the adjoint gradient of an L2 trace misfit against central
finite differences of the forward run."""
import numpy as np
import pytest

import oracle

N = (3, 3, 3)
DIPOLES = [((1.4, 1.6, 1.5), (0.2, 0.3, 1.0), 1, 0.25, 1.0)]
RECEIVERS = [(2.2, 1.3, 1.7), (0.8, 2.1, 1.2)]


def _eps(seed=1):
    _, _, ntet = oracle.tet_sizes(N)
    return np.random.default_rng(seed).uniform(1.0, 4.0, ntet)


def _node(i, j, k):
    return i + (N[0] + 1) * (j + (N[1] + 1) * k)


@pytest.mark.parametrize("ijk", [(1, 1, 1), (0, 1, 1), (0, 0, 1), (0, 0, 0), (1, 0, 2), (2, 1, 0)],
                         ids=["interior", "face_x", "edge", "corner", "face_y", "face_z"])
def test_mass_block_derivative_matches_central_differences(ijk):
    eps = _eps()
    v = _node(*ijk)
    M, _ = oracle.tet_mass_block(N, eps, v)
    h, worst, touched = 1e-5, 0.0, 0
    for t in range(eps.size):
        _, dM = oracle.tet_mass_block(N, eps, v, t)
        e1, e2 = eps.copy(), eps.copy()
        e1[t] += h
        e2[t] -= h
        fd = (oracle.tet_mass_block(N, e1, v)[0] - oracle.tet_mass_block(N, e2, v)[0]) / (2 * h)
        touched += np.abs(fd).max() > 0
        worst = max(worst, np.abs(dM - fd).max() / np.abs(M).max())
    assert touched > 0
    assert worst < 1e-8


def _misfit_setup(integrator, steps=40, dt=0.3):
    eps = _eps()
    tr, _, _ = oracle.tet_run(N, eps, integrator, dt, steps, 1, DIPOLES, RECEIVERS)
    data = tr * 0.9

    def J(e):
        t = oracle.tet_run(N, e, integrator, dt, steps, 1, DIPOLES, RECEIVERS)[0]
        return 0.5 * np.sum((t[..., 1:] - data[..., 1:]) ** 2)

    resid = tr - data
    resid[..., 0] = 0.0
    return eps, J, resid, dt, steps


@pytest.mark.parametrize("integrator", [oracle.SYMP2, oracle.SYMP4], ids=["symp2", "symp4"])
def test_oracle_gradient_matches_finite_differences(integrator):
    eps, J, resid, dt, steps = _misfit_setup(integrator)
    g = oracle.tet_gradient(N, eps, integrator, dt, steps, resid, 1, DIPOLES, RECEIVERS)
    idx = np.random.default_rng(7).choice(eps.size, 10, replace=False)
    fd = []
    for t in idx:
        e1, e2 = eps.copy(), eps.copy()
        e1[t] += 1e-4
        e2[t] -= 1e-4
        fd.append((J(e1) - J(e2)) / 2e-4)
    fd = np.array(fd)
    assert np.abs(g[idx] - fd).max() < 1e-7 * np.abs(fd).max()


def test_oracle_gradient_is_linear_in_the_trace_weights():
    eps, _, resid, dt, steps = _misfit_setup(oracle.SYMP4, steps=25)
    rng = np.random.default_rng(3)
    r2 = rng.standard_normal(resid.shape)
    g1 = oracle.tet_gradient(N, eps, oracle.SYMP4, dt, steps, resid, 1, DIPOLES, RECEIVERS)
    g2 = oracle.tet_gradient(N, eps, oracle.SYMP4, dt, steps, r2, 1, DIPOLES, RECEIVERS)
    g12 = oracle.tet_gradient(N, eps, oracle.SYMP4, dt, steps, 2.0 * resid - 0.5 * r2, 1, DIPOLES, RECEIVERS)
    assert np.allclose(g12, 2.0 * g1 - 0.5 * g2, rtol=1e-10, atol=1e-14 * np.abs(g12).max())
