"""Checks of the second-order (20-DOF) tetrahedral scheme itself (the FP64
oracle, orc_tet2.c), which has no reference counterpart, and of the
solver's own element matrices against it (host code of libems, no GPU):

* the element space is the complete second-order Nedelec space: per
  element the curl has the 9-dimensional kernel of the P2 gradients; on a
  mesh the discrete kernel of K is exactly the gradient space (live nodes +
  live edges of the P2 scalar space), i.e. no spurious modes;
* cavity eigenvalues converge to the analytic PEC modes at the rate h^4;
* the Chebyshev mass inverse meets its a-priori energy-norm bound;
* the symplectic steps conserve the discrete energy (no drift) and the
  stability limit is sharp;
* the discrete adjoint gradient agrees with central differences.
"""
import numpy as np
import pytest

import oracle


def _dense(n, stiff, eps=None):
    _, ndof, ntet = oracle.tet2_sizes(n)
    live = np.where(~oracle.tet2_pec_mask(n))[0]
    A = np.zeros((len(live), len(live)))
    for c, e in enumerate(live):
        x = np.zeros(ndof)
        x[e] = 1.0
        A[:, c] = oracle.tet2_apply(n, x, stiff, None if stiff else eps)[live]
    return A, live


def _analytic(L, k):
    ex = []
    for a in range(6):
        for b in range(6):
            for c in range(6):
                if (a > 0) + (b > 0) + (c > 0) >= 2:
                    ex += [np.pi ** 2 * (a * a + b * b + c * c) / L ** 2] * (2 if min(a, b, c) > 0 else 1)
    return np.sort(ex)[:k]


def test_element_matrices_are_the_second_order_space():
    for p in range(6):
        M, K = oracle.tet2_element(p)
        np.testing.assert_allclose(M, M.T, atol=1e-15)
        np.testing.assert_allclose(K, K.T, atol=1e-14)
        assert np.linalg.eigvalsh(M)[0] > 1e-5
        ek = np.linalg.eigvalsh(K)
        assert np.sum(np.abs(ek) < 1e-12 * ek[-1]) == 9      # grad P2 (10 - constants)
        assert ek[0] > -1e-13


def test_solver_element_matrices_match_the_oracle():
    """libems computes M by collapsed Gauss-Legendre quadrature and K from the
    vertex values of the curls; the oracle integrates barycentric monomials
    exactly.  Independent routes, same matrices."""
    import emsolvers_gb300 as ems
    for p in range(6):
        M, K = ems.tet_element_matrices(2, p)
        Mo, Ko = oracle.tet2_element(p)
        assert np.abs(M - Mo).max() <= 1e-14 * np.abs(Mo).max()
        assert np.abs(K - Ko).max() <= 1e-14 * np.abs(Ko).max()


def test_kernel_of_K_is_the_discrete_gradient_space():
    n = (3, 3, 3)
    K, live = _dense(n, True)
    M, _ = _dense(n, False, np.ones(oracle.tet2_sizes(n)[2]))
    w = np.linalg.eigvalsh(np.linalg.solve(np.linalg.cholesky(M), np.linalg.solve(np.linalg.cholesky(M), K).T))
    nzero = int(np.sum(np.abs(w) < 1e-9 * w.max()))
    nnode, _, _ = oracle.tet2_sizes(n)
    interior_nodes = (n[0] - 1) * (n[1] - 1) * (n[2] - 1)
    mask = oracle.tet2_pec_mask(n)
    live_edges = int((~mask[:7 * nnode]).sum())               # edge tails: one per live edge
    assert nzero == interior_nodes + live_edges


def test_cavity_eigenvalues_converge_at_fourth_order():
    errs = []
    for L in (2, 3, 4):
        n = (L, L, L)
        K, _ = _dense(n, True)
        M, _ = _dense(n, False, np.ones(oracle.tet2_sizes(n)[2]))
        Li = np.linalg.inv(np.linalg.cholesky(M))
        w = np.sort(np.linalg.eigvalsh(Li @ K @ Li.T))
        w = w[w > 1e-8][:6]
        ex = _analytic(L, 6)
        errs.append(np.abs(w - ex).max() / ex.max())
    rate = np.log(errs[1] / errs[2]) / np.log(4 / 3)
    assert errs[2] < 2e-3
    assert rate > 3.3, (errs, rate)   # h^4 (order-1 elements: h^2)


def test_chebyshev_mass_inverse_meets_its_bound():
    n = (4, 3, 3)
    _, ndof, ntet = oracle.tet2_sizes(n)
    rng = np.random.default_rng(5)
    eps = rng.uniform(1, 6, ntet)
    M, live = _dense(n, False, eps)
    lo, hi = oracle.tet2_cheb_bounds()
    assert 0.18 < lo < 0.19 and 2.9 < hi < 3.0
    r = (np.sqrt(hi / lo) - 1) / (np.sqrt(hi / lo) + 1)
    for m in (8, 16, oracle.TET2_MASS_ITERS):
        b = np.zeros(ndof)
        b[live] = rng.standard_normal(len(live))
        x = oracle.tet2_mass_solve(n, eps, b, m)[live]
        xs = np.linalg.solve(M, b[live])
        err = np.sqrt((x - xs) @ M @ (x - xs)) / np.sqrt(xs @ M @ xs)
        assert err <= 2 * r ** m * 1.0001, (m, err)
    # the approximate inverse is symmetric positive definite
    Q = np.zeros((len(live), len(live)))
    for c, e in enumerate(live):
        b = np.zeros(ndof)
        b[e] = 1.0
        Q[:, c] = oracle.tet2_mass_solve(n, eps, b)[live]
    np.testing.assert_allclose(Q, Q.T, atol=1e-12 * np.abs(Q).max())
    assert np.linalg.eigvalsh(0.5 * (Q + Q.T))[0] > 0


@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4])
def test_energy_is_conserved(integ):
    n = (4, 4, 4)
    _, ndof, ntet = oracle.tet2_sizes(n)
    rng = np.random.default_rng(7)
    eps = rng.uniform(1, 4, ntet)
    pec = oracle.tet2_pec_mask(n)
    U0 = np.where(pec, 0.0, rng.standard_normal(ndof))
    lim = oracle.stability_constant(integ) / np.sqrt(oracle.tet2_lambda_max(n, eps, 150))
    U, P = U0.copy(), np.zeros(ndof)
    e0 = oracle.tet2_energy(n, eps, U, P)
    es = []
    for _ in range(8):
        _, U, P = oracle.tet2_run(n, eps, integ, 0.5 * lim, 25, U=U, P=P)
        es.append(abs(oracle.tet2_energy(n, eps, U, P) - e0) / e0)
    assert max(es[4:]) < 1.3 * max(es[:4]) + 1e-12
    assert max(es) < (0.1 if integ == oracle.SYMP2 else 0.01)


@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4, oracle.LEAPFROG])
def test_stability_limit_is_sharp(integ):
    n = (3, 3, 3)
    _, ndof, ntet = oracle.tet2_sizes(n)
    eps = np.ones(ntet)
    pec = oracle.tet2_pec_mask(n)
    rng = np.random.default_rng(3)
    U0 = np.where(pec, 0.0, rng.standard_normal(ndof))
    lim = oracle.stability_constant(integ) / np.sqrt(oracle.tet2_lambda_max(n, eps, 300))
    P0 = U0.copy() if integ == oracle.LEAPFROG else None
    stable = oracle.tet2_run(n, eps, integ, 0.97 * lim, 300, U=U0, P=P0)[1]
    unstable = oracle.tet2_run(n, eps, integ, 1.05 * lim, 300, U=U0, P=P0)[1]
    assert np.abs(stable).max() < 100 * np.abs(U0).max()
    assert not np.isfinite(unstable).all() or np.abs(unstable).max() > 1e3 * np.abs(U0).max()


@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4])
def test_adjoint_gradient_matches_central_differences(integ):
    """The adjoint differentiates the drift increment q(M) P as M^-1 P; the
    difference from the derivative of the degree-28 polynomial stays far
    below the 1e-3 bound on the gradient (3e-6 at degree 32, 1.5e-4 at 24)."""
    n = (3, 3, 3)
    _, _, ntet = oracle.tet2_sizes(n)
    rng = np.random.default_rng(1)
    eps = rng.uniform(1, 4, ntet)
    dip = ((1.4, 1.6, 1.5), (0.2, 0.3, 1.0), 1, 0.25, 1.0)
    recs = [(2.2, 1.3, 1.7), (0.8, 2.1, 1.2)]
    steps, dtn = 24, 0.1
    tr, _, _ = oracle.tet2_run(n, eps, integ, dtn, steps, 1, [dip], recs)
    g = rng.standard_normal(tr.shape)
    g[..., 0] = 0.0
    grad = oracle.tet2_gradient(n, eps, integ, dtn, steps, g, 1, [dip], recs)
    pick = rng.choice(ntet, 12, replace=False)
    fd = []
    for t in pick:
        h = 1e-5 * eps[t]
        ep, em = eps.copy(), eps.copy()
        ep[t] += h
        em[t] -= h
        Jp = np.sum(g * oracle.tet2_run(n, ep, integ, dtn, steps, 1, [dip], recs)[0])
        Jm = np.sum(g * oracle.tet2_run(n, em, integ, dtn, steps, 1, [dip], recs)[0])
        fd.append((Jp - Jm) / (2 * h))
    fd = np.array(fd)
    assert np.linalg.norm(grad[pick] - fd) / np.linalg.norm(fd) < 1e-4
