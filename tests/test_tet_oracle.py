"""Checks of the tetrahedral scheme itself (the FP64 oracle), which has no
reference counterpart: cavity eigenvalues converge to the analytic PEC modes,
the block-lumped mass is exact for constant fields, the symplectic steps
conserve the discrete energy, and the stability limit is sharp."""
import numpy as np
import pytest

import oracle


def _operator(n):
    _, nslot, ntet = oracle.tet_sizes(n)
    eps = np.ones(ntet)
    pec = oracle.tet_pec_mask(n)
    act = np.where(~pec)[0]
    A = np.zeros((len(act), len(act)))
    for c, i in enumerate(act):
        x = np.zeros(nslot)
        x[i] = 1.0
        A[:, c] = oracle.tet_apply_op(n, eps, x)[act]
    return A


def test_cavity_eigenvalues_converge_to_analytic_modes():
    # unit-edge cubes, cavity of side L: k^2 = (pi/L)^2 (l^2+m^2+n^2); lowest 2,2,2,3,3
    errs = []
    for L in (4, 6):
        w = np.sort(np.linalg.eigvals(_operator((L, L, L))).real)
        w = w[w > 1e-8] / (np.pi / L) ** 2
        errs.append(np.abs(w[:5] - np.array([2, 2, 2, 3, 3])).max())
    assert errs[1] < errs[0] * 0.75
    assert errs[1] < 0.3


def test_block_mass_is_exact_for_constant_fields():
    n = (5, 4, 6)
    _, nslot, ntet = oracle.tet_sizes(n)
    rng = np.random.default_rng(1)
    eps = np.ones(ntet)
    minv = oracle.tet_minv(n, eps)
    pec = oracle.tet_pec_mask(n)
    # interior node: M_v (D E0) = W E0 with W_i = int w_i  =>  Minv W E0 = D E0
    nx, ny, nz = n
    v = 2 + (nx + 1) * (2 + (ny + 1) * 3)
    assert not pec[7 * v:7 * v + 7].any()
    E0 = rng.standard_normal(3)
    u = oracle.TET_DIRS @ E0
    M = np.linalg.inv(minv[v])
    # W rows for a translation-invariant interior node satisfy D^T W = I (unit cube volume)
    W = M @ oracle.TET_DIRS
    np.testing.assert_allclose(oracle.TET_DIRS.T @ W, np.eye(3), atol=1e-12)
    assert np.all(np.linalg.eigvalsh(M) > 0)
    np.testing.assert_allclose(minv[v] @ (W @ E0), u, atol=1e-12)


@pytest.mark.parametrize("integ,order", [(oracle.SYMP2, 2), (oracle.SYMP4, 4)])
def test_symplectic_energy_error_is_bounded_and_of_the_right_order(integ, order):
    """No secular drift of H = P.M^-1 P/2 + U.K U/2, and the oscillation of H
    shrinks like dt^2 (symplectic_2) or dt^4 (symplectic_4)."""
    n = (5, 5, 5)
    _, nslot, ntet = oracle.tet_sizes(n)
    rng = np.random.default_rng(2)
    eps = rng.uniform(1, 4, ntet)
    pec = oracle.tet_pec_mask(n)
    U0 = np.where(pec, 0.0, rng.standard_normal(nslot))
    lim = oracle.stability_constant(integ) / np.sqrt(oracle.tet_lambda_max(n, eps, 300))
    amp = []
    for frac in (0.5, 0.25):
        U, P = U0.copy(), np.zeros(nslot)
        e0 = oracle.tet_energy(n, eps, U, P)
        es = []
        for _ in range(16):
            _, U, P = oracle.tet_run(n, eps, integ, frac * lim, 20, 1, U=U, P=P)
            es.append(abs(oracle.tet_energy(n, eps, U, P) - e0) / e0)
        assert max(es[8:]) < 1.3 * max(es[:8]) + 1e-12   # bounded, no growth
        amp.append(max(es))
    assert amp[0] < (0.1 if order == 2 else 0.01)
    assert amp[0] / amp[1] > 0.75 * 2 ** order


@pytest.mark.parametrize("integ", [oracle.SYMP2, oracle.SYMP4, oracle.LEAPFROG])
def test_stability_limit_is_sharp(integ):
    n = (4, 4, 4)
    _, nslot, ntet = oracle.tet_sizes(n)
    eps = np.ones(ntet)
    pec = oracle.tet_pec_mask(n)
    rng = np.random.default_rng(3)
    U0 = np.where(pec, 0.0, rng.standard_normal(nslot))
    lim = oracle.stability_constant(integ) / np.sqrt(oracle.tet_lambda_max(n, eps, 400))
    stable = oracle.tet_run(n, eps, integ, 0.97 * lim, 400, 1, U=U0, P=(U0.copy() if integ == oracle.LEAPFROG else None))[1]
    unstable = oracle.tet_run(n, eps, integ, 1.05 * lim, 400, 1, U=U0, P=(U0.copy() if integ == oracle.LEAPFROG else None))[1]
    assert np.abs(stable).max() < 100 * np.abs(U0).max()
    assert not np.isfinite(unstable).all() or np.abs(unstable).max() > 1e3 * np.abs(U0).max()


def test_symp4_stability_constant():
    assert abs(oracle.stability_constant(oracle.SYMP4) - 1.5734) < 1e-3
    assert oracle.stability_constant(oracle.SYMP2) == 2.0


_KUHN = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]


def _consistent_whitney_mass(L):
    """The consistent mass of the Whitney space on the Kuhn-split cube of
    side L (eps = 1), assembled here from int l_i l_j = |T| (1 + d_ij) / 20
    and the barycentric gradients, independently of the solver and the
    oracle (which use per-node mass blocks)."""
    n = (L, L, L)
    _, nslot, _ = oracle.tet_sizes(n)
    dirs = {tuple(int(c) for c in d): k for k, d in enumerate(oracle.TET_DIRS)}
    ll = (np.ones((4, 4)) + np.eye(4)) / 120.0
    edges = [(m, q) for m in range(4) for q in range(m + 1, 4)]
    M = np.zeros((nslot, nslot))
    for a, b, c in _KUHN:
        vert = np.zeros((4, 3), int)
        vert[1, a] = 1
        vert[2, a] = vert[2, b] = 1
        vert[3] = 1
        G = np.zeros((4, 3))
        G[0, a], G[1, a], G[1, b], G[2, b], G[2, c], G[3, c] = -1, 1, -1, 1, -1, 1
        Me = np.array([[ll[i1, i2] * G[j1] @ G[j2] - ll[i1, j2] * G[j1] @ G[i2] - ll[j1, i2] * G[i1] @ G[j2]
                        + ll[j1, j2] * G[i1] @ G[i2] for (i2, j2) in edges] for (i1, j1) in edges])
        ed = [dirs[tuple(vert[q] - vert[m])] for m, q in edges]
        for k in range(L):
            for j in range(L):
                for i in range(L):
                    sl = [7 * ((i + vert[m][0]) + (L + 1) * ((j + vert[m][1]) + (L + 1) * (k + vert[m][2]))) + ed[e]
                          for e, (m, _) in enumerate(edges)]
                    M[np.ix_(sl, sl)] += Me
    return M


def test_block_lumped_mass_against_the_consistent_mass():
    """The per-node mass blocks against the consistent Whitney mass on the
    same mesh and stiffness: lowest PEC cavity eigenvalues (the analytic
    triple k^2 = 2 (pi/L)^2).  The consistent mass converges at h^2; the
    block-lumped mass converges too but more slowly (order about 1.4 over
    L = 4..8, 2-3 times the consistent error), which bounds the dispersion
    error the lumping adds."""
    import scipy.linalg as la
    errs = {"consistent": [], "block": []}
    for L in (4, 6, 8):
        n = (L, L, L)
        _, nslot, ntet = oracle.tet_sizes(n)
        live = np.where(~oracle.tet_pec_mask(n))[0]
        eye = np.eye(nslot)
        K = np.stack([oracle.tet_apply_K(n, eye[e]) for e in live], axis=1)[live]
        Mb = np.zeros((nslot, nslot))
        eps = np.ones(ntet)
        for v in range(nslot // 7):
            Mb[7 * v:7 * v + 7, 7 * v:7 * v + 7] = oracle.tet_mass_block(n, eps, v)[0]
        Mc = _consistent_whitney_mass(L)
        s = (np.pi / L) ** 2
        for name, M in (("consistent", Mc), ("block", Mb)):
            w = la.eigh(K, M[np.ix_(live, live)], eigvals_only=True, subset_by_value=(1e-6 * s, 2.5 * s)) / s
            assert len(w) >= 3
            errs[name].append(np.abs(np.sort(w)[:3] - 2.0).max() / 2.0)
    c, b = np.array(errs["consistent"]), np.array(errs["block"])
    rate = lambda e: np.log(e[0] / e[2]) / np.log(8 / 4)
    assert rate(c) > 1.8, c                  # h^2
    assert 1.2 < rate(b) < 1.8, b            # between first and second order
    assert np.all(b < 3.5 * c), (b, c)
    assert b[2] < 0.035                      # 3.2% at L = 8
