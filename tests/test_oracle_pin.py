"""Pins the FP64 CPU oracle against the reference: bit-identical traces and
fields on the golden fixtures produced by the unmodified reference solvers,
and (where the reference tree is present) on live reference runs."""
import numpy as np
import pytest

import golden_io
import oracle
import refrun

INTEG = {"fem_v2": oracle.LEAPFROG, "symplectic_2": oracle.SYMP2, "symplectic_4": oracle.SYMP4}


@pytest.mark.parametrize("case", list(golden_io.fdtd_cases()), ids=lambda c: c[0]["name"])
def test_fdtd_oracle_matches_reference_bitwise(case):
    m, tr, fields = case
    nx, ny, nz = m["grid"]
    srcs = [(c, tuple(p), 0, 1e9, 1.0) for c, p in m["sources"]]
    obs = [tuple([tuple(q) for q in l] for l in o) for o in m["observations"]]
    tr_o, f_o = oracle.fdtd_run(nx, ny, nz, m["h"], m["dt"], m["eps"], m["mu"], m["tf"], m["nsteps"], srcs, obs)
    assert np.array_equal(tr_o, tr)
    for k in fields:
        assert np.array_equal(f_o[k], fields[k]), k


@pytest.mark.parametrize("case", list(golden_io.femv2_cases()), ids=lambda c: c[0]["name"])
def test_hexfem_oracle_matches_reference_bitwise(case):
    m, tr, ef = case
    km = oracle.load_kmat(golden_io.kmat_path(m["order"], m["use_ofem"]))
    src = (m["source"][0], tuple(m["source"][1]))
    tr_o, ef_o = oracle.hexfem_run(m["order"], tuple(m["grid"]), m["h"], m["dt"], m["eps"], m["mu"], m["tf"],
                                   INTEG[m["variant"]], km, m["nsteps"], [src], [tuple(m["observation"])])
    assert np.array_equal(tr_o[0], tr)
    for q in range(3):
        assert np.array_equal(ef_o[q], ef[q])


def test_kmat_parser_reads_rationals(golden_dir):
    k = oracle.load_kmat(golden_io.kmat_path(1, 1))
    assert k.shape == (12, 12)
    assert k[0, 0] == 7.0 / 4.0 and k[0, 4] == -7.0 / 8.0
    assert np.allclose(k, k.T)
    for o, n in ((2, 54), (3, 144)):
        assert oracle.load_kmat(golden_io.kmat_path(o, 1)).shape == (n, n)


@pytest.mark.skipif(not refrun.available(), reason="reference sources not present")
def test_fdtd_oracle_matches_live_reference_cubic_grid():
    n = 9
    h = 1e-3
    dt = 0.9 * h / (2.998e8 * np.sqrt(3))
    src = [(2, (4, 4, 4)), (1, (2, 6, 3))]
    obs = [([(4, 4, 5)], [(4, 4, 5)], [(4, 4, 5)])]
    tr_r, f_r = refrun.fdtd(n, n, n, h, dt, 8.854187817e-12, 1.25663706212e-6, 3, 45, src, obs)
    tr_o, f_o = oracle.fdtd_run(n, n, n, h, dt, 8.854187817e-12, 1.25663706212e-6, 3, 45,
                                [(c, p, 0, 1e9, 1.0) for c, p in src], obs)
    assert np.array_equal(tr_r, tr_o)
    for k in f_r:
        assert np.array_equal(f_r[k], f_o[k])


def test_fdtd_material_table_reduces_to_reference_update():
    """Uniform eps through the material table, sigma = 0: identical bits."""
    n = 7
    h, dt, eps, mu = 1e-3, 1.5e-12, 8.854187817e-12, 1.25663706212e-6
    src = [(0, (3, 3, 3), 0, 1e9, 1.0)]
    obs = [([(3, 3, 3)], [(3, 3, 3)], [(3, 3, 3)])]
    tr_a, f_a = oracle.fdtd_run(n, n, n, h, dt, eps, mu, 1, 20, src, obs)
    mat = (np.zeros((n, n, n), np.uint16), np.array([eps]), np.array([0.0]))
    tr_b, f_b = oracle.fdtd_run(n, n, n, h, dt, eps, mu, 1, 20, src, obs, material=mat)
    assert np.array_equal(tr_a, tr_b)
    for k in f_a:
        assert np.array_equal(f_a[k], f_b[k])


@pytest.mark.parametrize("case", list(golden_io.abm_cases()), ids=lambda c: c[0]["name"])
def test_abm_oracle_matches_reference_bitwise(case):
    m, tr, E, H = case
    lam = oracle.load_kmat(golden_io.kmat_path(1, 0))
    src = [(c, tuple(p)) for c, p in m["sources"]]
    dip = [tuple(p) for p in m["dipoles"]]
    obs = [tuple([tuple(q) for q in l] for l in o) for o in m["observations"]]
    tr_o, E_o, H_o = oracle.abm_run(tuple(m["grid"]), m["h"], m["dt"], m["eps"], m["mu"], m["tf"], m["nsteps"], lam,
                                     src, dip, obs)
    assert np.array_equal(tr_o, tr)
    for q in range(3):
        assert np.array_equal(E_o[q], E[q])
        assert np.array_equal(H_o[q], H[q])


def test_abm_element_matrix_is_curl_plus_stabilised_curl_curl():
    """K = A + 0.05 Abar: A holds half the element-averaged curl (rows of one
    component identical), Abar the order-1 curl-curl matrix."""
    lam = oracle.load_kmat(golden_io.kmat_path(1, 0))
    K = oracle.abm_kmat(lam)
    A = K - 0.05 * lam[np.ix_([0, 1, 2, 3, 4, 6, 5, 7, 8, 9, 10, 11], [0, 1, 2, 3, 4, 6, 5, 7, 8, 9, 10, 11])]
    for c in range(3):
        rows = A[4 * c:4 * c + 4]
        assert np.allclose(rows, rows[0])
        assert np.allclose(rows[:, 4 * c:4 * c + 4], 0.0)
    # the curl of a gradient field vanishes: A annihilates edge values of phi = x^2 + y z
    assert np.allclose(np.abs(A).sum(1), 4.0)


@pytest.mark.parametrize("case", list(golden_io.femstab_cases()), ids=lambda c: c[0]["name"])
def test_femstab_oracle_matches_reference_bitwise(case):
    """fem/ (stabilised order 1): the oracle's element matrix, traces and all
    three E levels equal the reference's bit for bit."""
    m, tr, E, K = case
    src = [(c, tuple(p)) for c, p in m["sources"]]
    dip = [tuple(p) for p in m["dipoles"]]
    obs = [tuple([tuple(q) for q in l] for l in o) for o in m["observations"]]
    assert np.array_equal(oracle.femstab_kmat(m["dt"], m["mu"], m["eps"], m["h"], m["stabilization"], m["use_ofem"]), K)
    tr_o, E_o = oracle.femstab_run(tuple(m["grid"]), m["h"], m["dt"], m["eps"], m["mu"], m["tf"], m["stabilization"],
                                   m["use_ofem"], m["nsteps"], src, dip, obs)
    assert np.array_equal(tr_o, tr)
    for q in range(3):
        assert np.array_equal(E_o[q], E[q])


def _cube_gradient(phi):
    """Edge values (cyclic local order) of the gradient of a nodal potential
    phi[x, y, z] on one cube: x-edges (y, z), y-edges (z, x), z-edges (x, y)."""
    e = []
    for q in range(4):
        e.append(phi[1, q & 1, q >> 1] - phi[0, q & 1, q >> 1])
    for q in range(4):
        e.append(phi[q >> 1, 1, q & 1] - phi[q >> 1, 0, q & 1])
    for q in range(4):
        e.append(phi[q & 1, q >> 1, 1] - phi[q & 1, q >> 1, 0])
    return np.array(e)


@pytest.mark.parametrize("ofem", [0, 1], ids=["conventional", "ofem"])
def test_femstab_element_matrices_structure(ofem):
    """The fem/ matrices as the oracle forms them: C = A^T, Cbar = Abar^T, B
    symmetric positive definite; conventional Bbar = A^T and B the 4x4
    tensor-product mass per component; OFEM the same operators in the modal
    basis of each component.  A and Abar annihilate discrete gradients, so
    K has the gradient null space of a curl-curl operator."""
    A, Ab, B, Bb, C, Cb = oracle.femstab_parts(ofem)
    assert np.array_equal(C, A.T) and np.array_equal(Cb, Ab.T)
    assert np.array_equal(B, B.T) and np.all(np.linalg.eigvalsh(B) > 0)
    rng = np.random.default_rng(3)
    for _ in range(4):
        g = _cube_gradient(rng.standard_normal((2, 2, 2)))
        assert np.abs(A @ g).max() < 1e-14 and np.abs(Ab @ g).max() < 1e-14
    K = oracle.femstab_kmat(2e-11, 1.25663706212e-6, 8.854187817e-12, 0.02, 0.3, ofem)
    g = _cube_gradient(rng.standard_normal((2, 2, 2)))
    assert np.abs(K @ g).max() < 1e-14 * np.abs(K).max()
    Ac, Abc, Bc, Bbc, Cc, Cbc = oracle.femstab_parts(0)
    H = np.array([[1, 1, 1, 1], [-1, 1, -1, 1], [-1, -1, 1, 1], [1, -1, -1, 1]], float)
    T = np.kron(np.eye(3), H)
    if ofem:
        assert np.array_equal(A, T @ Ac)
        assert np.allclose(B, T @ Bc @ T.T, rtol=1e-15, atol=1e-14)
        assert np.array_equal(Bb, T @ Bbc @ T.T)
        assert np.array_equal(C, Cc @ T.T)
    else:
        assert np.array_equal(Bb, A.T)
        mass = np.array([[8.0 / 9.0 / 2 ** bin(a ^ b).count("1") for b in range(4)] for a in range(4)])
        assert np.array_equal(B, np.kron(np.eye(3), mass))
        # Abar is the order-1 curl-curl matrix of kmat/lamped1.csv in the cyclic order
        lam = oracle.load_kmat(golden_io.kmat_path(1, 0))
        perm = [0, 1, 2, 3, 4, 6, 5, 7, 8, 9, 10, 11]
        assert np.array_equal(Ab, lam[np.ix_(perm, perm)])


@pytest.mark.skipif(not refrun.available(), reason="reference sources not present")
@pytest.mark.parametrize("ofem", [0, 1], ids=["conventional", "ofem"])
def test_femstab_oracle_matches_live_reference(ofem):
    g, h, dt = (7, 9, 6), 0.02, 1.5e-11
    src, dip = [(1, (3, 4, 3)), (0, (2, 5, 2))], [(2, 4, 2)]
    obs = [([(3, 4, 3)], [(3, 4, 3), (4, 4, 3)], [(3, 4, 3)])]
    tr_r, E_r, K_r = refrun.femstab(g, h, dt, 8.854187817e-12, 1.25663706212e-6, 3, 0.45, ofem, 45, src, dip, obs)
    tr_o, E_o = oracle.femstab_run(g, h, dt, 8.854187817e-12, 1.25663706212e-6, 3, 0.45, ofem, 45, src, dip, obs)
    assert np.array_equal(oracle.femstab_kmat(dt, 1.25663706212e-6, 8.854187817e-12, h, 0.45, ofem), K_r)
    assert np.array_equal(tr_r, tr_o)
    for q in range(3):
        assert np.array_equal(E_r[q], E_o[q])
