"""ctypes front end of the FP64 C oracle (oracle/*.c).

ORACLE / TEST INFRASTRUCTURE ONLY — see the package docstring.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(path)
        _lib.orc_fdtd_run.restype = C.c_int
        _lib.orc_fdtd_source.restype = C.c_double
        _lib.orc_fdtd_source.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double]
        _lib.orc_hexfem_run.restype = C.c_int
        if hasattr(_lib, "orc_tet_run"):
            _lib.orc_tet_run.restype = C.c_int
    return _lib


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t) if a is not None else None


class _FdtdCase(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("h", C.c_double), ("dt", C.c_double), ("eps", C.c_double), ("mu", C.c_double),
                ("time_frequency", C.c_int),
                ("mat_id", C.POINTER(C.c_uint16)), ("mat_eps", _dp), ("mat_sigma", _dp), ("nmat", C.c_int),
                ("pml", C.c_int), ("pml_m", C.c_double), ("pml_kmax", C.c_double), ("pml_amax", C.c_double),
                ("pml_R0", C.c_double),
                ("nsrc", C.c_int), ("src_comp", _ip), ("src_ijk", _ip), ("src_kind", _ip),
                ("src_f0", _dp), ("src_amp", _dp),
                ("nobs", C.c_int), ("obs_n", _ip), ("obs_ijk", _ip)]


def fdtd_shapes(nx, ny, nz):
    """Reference padded layout (fdtd/fdtd_simulation.cpp:57-68), x fastest."""
    return {"Ex": (nz + 2, ny + 2, nx + 1), "Ey": (nz + 2, ny + 1, nx + 2), "Ez": (nz + 1, ny + 2, nx + 2),
            "Hx": (nz + 1, ny + 1, nx), "Hy": (nz + 1, ny, nx + 1), "Hz": (nz, ny + 1, nx + 1)}


def fdtd_source(kind, f0, t, h):
    return lib().orc_fdtd_source(kind, f0, t, h)


def fdtd_run(nx, ny, nz, h, dt, eps, mu, tf, nsteps, sources=(), observations=(),
             material=None, pml=None, fields=None):
    """Runs the FP64 oracle FDTD.

    sources: [(comp, (i,j,k), kind, f0, amp)]; observations: [(xs, ys, zs)]
    lists of (i,j,k) per component; material: (mat_id[nz,ny,nx] uint16,
    eps_table, sigma_table); pml: dict(cells, m, kmax, amax, R0).
    Returns (traces[nobs, nsteps//tf+1, 3], fields dict)."""
    sh = fdtd_shapes(nx, ny, nz)
    if fields is None:
        fields = {k: np.zeros(v) for k, v in sh.items()}
    else:
        fields = {k: np.ascontiguousarray(fields[k], dtype=np.float64).copy() for k in sh}
    c = _FdtdCase()
    c.nx, c.ny, c.nz, c.h, c.dt, c.eps, c.mu, c.time_frequency = nx, ny, nz, h, dt, eps, mu, tf
    keep = []
    if material is not None:
        mid = np.ascontiguousarray(material[0], dtype=np.uint16)
        me = np.ascontiguousarray(material[1], dtype=np.float64)
        ms = np.ascontiguousarray(material[2], dtype=np.float64)
        keep += [mid, me, ms]
        c.mat_id = mid.ctypes.data_as(C.POINTER(C.c_uint16))
        c.mat_eps, c.mat_sigma, c.nmat = _ptr(me), _ptr(ms), len(me)
    if pml:
        c.pml = pml["cells"]
        c.pml_m, c.pml_kmax, c.pml_amax, c.pml_R0 = pml.get("m", 3.0), pml.get("kmax", 1.0), pml.get("amax", 0.0), pml.get("R0", 1e-6)
    c.nsrc = len(sources)
    if sources:
        comp = np.array([s[0] for s in sources], np.int32)
        ijk = np.array([s[1] for s in sources], np.int32).reshape(-1)
        kind = np.array([s[2] if len(s) > 2 else 0 for s in sources], np.int32)
        f0 = np.array([s[3] if len(s) > 3 else 1e9 for s in sources], np.float64)
        amp = np.array([s[4] if len(s) > 4 else 1.0 for s in sources], np.float64)
        keep += [comp, ijk, kind, f0, amp]
        c.src_comp, c.src_ijk, c.src_kind = _ptr(comp, _ip), _ptr(ijk, _ip), _ptr(kind, _ip)
        c.src_f0, c.src_amp = _ptr(f0), _ptr(amp)
    c.nobs = len(observations)
    if observations:
        on = np.array([len(l) for o in observations for l in o], np.int32)
        oi = np.array([p for o in observations for l in o for p in l], np.int32).reshape(-1)
        keep += [on, oi]
        c.obs_n, c.obs_ijk = _ptr(on, _ip), _ptr(oi, _ip)
    nsamp = nsteps // tf + 1
    traces = np.zeros((max(len(observations), 1), nsamp, 3))
    E = (_dp * 3)(*[_ptr(fields[k]) for k in ("Ex", "Ey", "Ez")])
    H = (_dp * 3)(*[_ptr(fields[k]) for k in ("Hx", "Hy", "Hz")])
    rc = lib().orc_fdtd_run(C.byref(c), C.c_int(nsteps), E, H, _ptr(traces))
    if rc != 0:
        raise RuntimeError(f"orc_fdtd_run failed: {rc}")
    return traces[:len(observations)], fields


# ------------------------------------------------------------ hexahedral FEM
LEAPFROG, SYMP2, SYMP4 = 0, 1, 2


class _HexCase(C.Structure):
    _fields_ = [("order", C.c_int), ("gx", C.c_int), ("gy", C.c_int), ("gz", C.c_int),
                ("h", C.c_double), ("dt", C.c_double), ("eps", C.c_double), ("mu", C.c_double),
                ("time_frequency", C.c_int), ("integrator", C.c_int), ("kmat", _dp),
                ("nsrc", C.c_int), ("src_comp", _ip), ("src_ijk", _ip),
                ("nobs", C.c_int), ("obs_ijk", _ip)]


def hexfem_sizes(gx, gy, gz):
    return (gx * (gy + 1) * (gz + 1), (gx + 1) * gy * (gz + 1), (gx + 1) * (gy + 1) * gz)


def parse_value(s):
    """Restates fem_v2/fem_simulation.cpp:1477-1493 (trim quotes/space, a/b)."""
    t = s.strip(" \t\r\n\"")
    if not t:
        return 0.0
    if "/" in t:
        a, b = t.split("/", 1)
        return float(a) / float(b)
    return float(t)


def load_kmat(path):
    """Restates fem_v2/fem_simulation.cpp:1495-1524 (rows of comma cells)."""
    rows = []
    with open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            if not line:
                continue
            rows.append([parse_value(c) for c in line.split(",")])
    return np.array(rows, dtype=np.float64)


def hexfem_run(order, grid, h, dt, eps, mu, tf, integrator, kmat, nsteps, sources=(), observations=(), ef=None):
    """FP64 oracle for the fem_v2 family.  sources: [(comp, (i,j,k))];
    observations: [(i,j,k)].  ef: optional [3] arrays of 3 levels each.
    Returns (traces[nobs, (nsteps-1)//tf+1, 4], ef)."""
    gx, gy, gz = grid
    sz = hexfem_sizes(gx, gy, gz)
    if ef is None:
        ef = [np.zeros(3 * n) for n in sz]
    else:
        ef = [np.ascontiguousarray(a, dtype=np.float64).copy() for a in ef]
    km = np.ascontiguousarray(kmat, dtype=np.float64)
    c = _HexCase()
    c.order, c.gx, c.gy, c.gz = order, gx, gy, gz
    c.h, c.dt, c.eps, c.mu, c.time_frequency, c.integrator = h, dt, eps, mu, tf, integrator
    c.kmat = _ptr(km)
    comp = np.array([s[0] for s in sources] or [0], np.int32)
    sijk = np.array([s[1] for s in sources] or [(0, 0, 0)], np.int32).reshape(-1)
    oijk = np.array(list(observations) or [(0, 0, 0)], np.int32).reshape(-1)
    c.nsrc, c.src_comp, c.src_ijk = len(sources), _ptr(comp, _ip), _ptr(sijk, _ip)
    c.nobs, c.obs_ijk = len(observations), _ptr(oijk, _ip)
    nsamp = (nsteps - 1) // tf + 1
    traces = np.zeros((max(len(observations), 1), nsamp, 4))
    arr = (_dp * 3)(*[_ptr(a) for a in ef])
    rc = lib().orc_hexfem_run(C.byref(c), C.c_int(nsteps), arr, _ptr(traces))
    if rc != 0:
        raise RuntimeError(f"orc_hexfem_run failed: {rc}")
    return traces[:len(observations)], ef


# ------------------------------------------------------------ tetrahedral FEM
class _TetCase(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("eps_r", _dp), ("mu_r", _dp),
                ("integrator", C.c_int), ("dt", C.c_double), ("time_frequency", C.c_int),
                ("ndip", C.c_int), ("dip_pos", _dp), ("dip_dir", _dp), ("dip_f0", _dp), ("dip_amp", _dp),
                ("dip_kind", _ip), ("nrec", C.c_int), ("rec_pos", _dp), ("sigma", _dp)]


def tet_sizes(n):
    nx, ny, nz = n
    nnode = (nx + 1) * (ny + 1) * (nz + 1)
    return nnode, 7 * nnode, 6 * nx * ny * nz


def _tlib():
    L = lib()
    L.orc_tet_lambda_max.restype = C.c_double
    L.orc_stability_constant.restype = C.c_double
    L.orc_tet_energy.restype = C.c_double
    L.orc_tet_wave.restype = C.c_double
    L.orc_tet_wave.argtypes = [C.c_int, C.c_double, C.c_double]
    L.orc_tet_locate.restype = C.c_long
    return L


def _tet_case(n, eps_r, integrator, dt, tf, dipoles, receivers, mu_r, sigma=None):
    """orc_tet_case for the arguments of tet_run; returns (case, arrays kept alive)."""
    _, _, ntet = tet_sizes(n)
    eps = np.ascontiguousarray(eps_r, dtype=np.float64).reshape(-1)
    assert eps.size == ntet
    mu = None if mu_r is None else np.ascontiguousarray(mu_r, dtype=np.float64).reshape(-1)
    sg = None if sigma is None else np.ascontiguousarray(sigma, dtype=np.float64).reshape(-1)
    assert sg is None or sg.size == ntet
    c = _TetCase()
    c.nx, c.ny, c.nz = n
    c.eps_r, c.mu_r = _ptr(eps), _ptr(mu) if mu is not None else None
    c.sigma = _ptr(sg) if sg is not None else None
    c.integrator, c.dt, c.time_frequency = integrator, dt, tf
    dp = np.array([d[0] for d in dipoles] or [(0, 0, 0)], np.float64).reshape(-1)
    dd = np.array([d[1] for d in dipoles] or [(0, 0, 1)], np.float64).reshape(-1)
    dk = np.array([d[2] for d in dipoles] or [1], np.int32)
    df = np.array([d[3] for d in dipoles] or [1.0], np.float64)
    da = np.array([d[4] for d in dipoles] or [1.0], np.float64)
    rp = np.array(list(receivers) or [(0, 0, 0)], np.float64).reshape(-1)
    c.ndip, c.dip_pos, c.dip_dir, c.dip_kind, c.dip_f0, c.dip_amp = len(dipoles), _ptr(dp), _ptr(dd), _ptr(dk, _ip), _ptr(df), _ptr(da)
    c.nrec, c.rec_pos = len(receivers), _ptr(rp)
    return c, (eps, mu, sg, dp, dd, dk, df, da, rp)


def tet_run(n, eps_r, integrator, dt, nsteps, tf=1, dipoles=(), receivers=(), mu_r=None, U=None, P=None, sigma=None):
    """FP64 oracle of the tetrahedral solver in normalised units (cube edge 1,
    c0 = 1).  dipoles: [(pos, dir, kind, f0, amp)]; receivers: [pos];
    sigma: conductivity per tetrahedron (normalised, a loss rate) or None.
    Returns (traces[nrec, nsamp, 4], U, P)."""
    _, nslot, _ = tet_sizes(n)
    U = np.zeros(nslot) if U is None else np.ascontiguousarray(U, dtype=np.float64).copy()
    P = np.zeros(nslot) if P is None else np.ascontiguousarray(P, dtype=np.float64).copy()
    c, keep = _tet_case(n, eps_r, integrator, dt, tf, dipoles, receivers, mu_r, sigma)
    nsamp = (nsteps - 1) // tf + 1 if nsteps > 0 else 0
    tr = np.zeros((max(len(receivers), 1), max(nsamp, 1), 4))
    rc = _tlib().orc_tet_run(C.byref(c), C.c_int(nsteps), _ptr(U), _ptr(P), _ptr(tr))
    if rc != 0:
        raise RuntimeError(f"orc_tet_run failed: {rc}")
    return tr[:len(receivers), :nsamp], U, P


def tet_gradient(n, eps_r, integrator, dt, nsteps, trace_grad, tf=1, dipoles=(), receivers=(), mu_r=None, sigma=None):
    """dJ/deps_r per tetrahedron by the FP64 discrete adjoint of tet_run
    (symplectic integrators, zero initial fields).  trace_grad: dJ/dtraces,
    shaped like tet_run's traces (column 0, the time, is ignored).  With
    sigma given, returns (dJ/deps_r, dJ/dsigma)."""
    _, _, ntet = tet_sizes(n)
    nsamp = (nsteps - 1) // tf + 1 if nsteps > 0 else 0
    g = np.zeros((max(len(receivers), 1), max(nsamp, 1), 4))
    tg = np.asarray(trace_grad, np.float64)
    if len(receivers):
        g[:len(receivers), :nsamp] = tg.reshape(len(receivers), nsamp, 4)
    c, keep = _tet_case(n, eps_r, integrator, dt, tf, dipoles, receivers, mu_r, sigma)
    out = np.zeros(ntet)
    gs = np.zeros(ntet)
    rc = _tlib().orc_tet_gradient(C.byref(c), C.c_int(nsteps), _ptr(g), _ptr(out), _ptr(gs))
    if rc != 0:
        raise RuntimeError(f"orc_tet_gradient failed: {rc}")
    return out if sigma is None else (out, gs)


def tet_loss_rate(n, eps_r, sigma):
    """Per-node loss rate rho_v of the conductivity model."""
    nnode, _, _ = tet_sizes(n)
    rho = np.zeros(nnode)
    _tlib().orc_tet_loss_rate(C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]), _ptr(np.ascontiguousarray(eps_r, np.float64)),
                              _ptr(np.ascontiguousarray(sigma, np.float64)), _ptr(rho))
    return rho


def tet_mass_block(n, eps_r, v, t=-1):
    """Mass block M_v (7x7 over the node's slots) and, for t >= 0, dM_v/deps_t."""
    eps = np.ascontiguousarray(eps_r, dtype=np.float64).reshape(-1)
    M, dM = np.zeros((7, 7)), np.zeros((7, 7))
    if _tlib().orc_tet_mass_block(C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]), _ptr(eps), C.c_long(v), C.c_long(t),
                                  _ptr(M), _ptr(dM)) != 0:
        raise ValueError("node or tetrahedron index out of range")
    return M, dM


def tet_minv(n, eps_r):
    nnode, _, _ = tet_sizes(n)
    out = np.zeros((nnode, 7, 7))
    eps = np.ascontiguousarray(eps_r, dtype=np.float64).reshape(-1)
    if _tlib().orc_tet_minv(C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]), _ptr(eps), _ptr(out)) != 0:
        raise RuntimeError("mass block not positive definite")
    return out


def tet_lambda_max(n, eps_r, iters=300, mu_r=None):
    eps = np.ascontiguousarray(eps_r, dtype=np.float64).reshape(-1)
    mui = None if mu_r is None else np.ascontiguousarray(1.0 / np.asarray(mu_r, np.float64).reshape(-1))
    return _tlib().orc_tet_lambda_max(C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]), _ptr(eps),
                                      _ptr(mui) if mui is not None else None, C.c_int(iters))


def stability_constant(integrator):
    return _tlib().orc_stability_constant(C.c_int(integrator))


def tet_energy(n, eps_r, U, P):
    eps = np.ascontiguousarray(eps_r, dtype=np.float64).reshape(-1)
    return _tlib().orc_tet_energy(C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]), _ptr(eps),
                                  _ptr(np.ascontiguousarray(U, np.float64)), _ptr(np.ascontiguousarray(P, np.float64)))


def tet_wave(kind, f0, t):
    return _tlib().orc_tet_wave(kind, f0, t)


def tet_apply_op(n, eps_r, x):
    """y = M^-1 K x of the tetrahedral scheme."""
    _, nslot, _ = tet_sizes(n)
    eps = np.ascontiguousarray(eps_r, dtype=np.float64).reshape(-1)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(nslot)
    if _tlib().orc_tet_apply_op(C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]), _ptr(eps), _ptr(x), _ptr(y)) != 0:
        raise RuntimeError("mass block not positive definite")
    return y


def tet_pec_mask(n):
    _, nslot, _ = tet_sizes(n)
    m = np.zeros(nslot, np.uint8)
    _tlib().orc_tet_pec_mask(C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]), m.ctypes.data_as(C.POINTER(C.c_uint8)))
    return m.astype(bool)


TET_DIRS = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [1, 0, 1], [0, 1, 1], [1, 1, 1]], np.float64)


def tet_apply_K(n, x):
    """f = K x of the tetrahedral scheme (normalised units, mu_r = 1)."""
    _, nslot, _ = tet_sizes(n)
    x = np.ascontiguousarray(x, dtype=np.float64)
    f = np.zeros(nslot)
    _tlib().orc_tet_apply_K(C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]), _ptr(x), _ptr(f))
    return f


# ------------------------------------------------- second-order tetrahedra
TET2_MASS_ITERS = 28


def tet2_sizes(n):
    nx, ny, nz = n
    nnode = (nx + 1) * (ny + 1) * (nz + 1)
    return nnode, 38 * nnode, 6 * nx * ny * nz


def _t2lib():
    L = _tlib()
    L.orc_tet2_lambda_max.restype = C.c_double
    L.orc_tet2_energy.restype = C.c_double
    L.orc_tet2_locate.restype = C.c_long
    return L


def tet2_element(p):
    """(M, K) 20 x 20 of Kuhn type p (eps = mu = 1), exact integration."""
    M, K = np.zeros((20, 20)), np.zeros((20, 20))
    _t2lib().orc_tet2_element(C.c_int(p), _ptr(M), _ptr(K))
    return M, K


def tet2_dof(p, a):
    pl, lv = C.c_int(), C.c_int()
    _t2lib().orc_tet2_dof(C.c_int(p), C.c_int(a), C.byref(pl), C.byref(lv))
    return pl.value, lv.value


def tet2_pec_mask(n):
    _, ndof, _ = tet2_sizes(n)
    m = np.zeros(ndof, np.uint8)
    _t2lib().orc_tet2_pec_mask(C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]), m.ctypes.data_as(C.POINTER(C.c_uint8)))
    return m.astype(bool)


def tet2_cheb_bounds():
    lo, hi = C.c_double(), C.c_double()
    _t2lib().orc_tet2_cheb_bounds(C.byref(lo), C.byref(hi))
    return lo.value, hi.value


def tet2_apply(n, x, stiff, coef=None):
    """y = sum_T coef_T A_T x (A = element stiffness if stiff else mass)."""
    _, ndof, _ = tet2_sizes(n)
    x = np.ascontiguousarray(x, dtype=np.float64)
    cf = None if coef is None else np.ascontiguousarray(coef, dtype=np.float64).reshape(-1)
    y = np.zeros(ndof)
    _t2lib().orc_tet2_apply(C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]), C.c_int(1 if stiff else 0),
                            _ptr(cf) if cf is not None else None, _ptr(x), _ptr(y))
    return y


def tet2_mass_solve(n, eps_r, b, iters=TET2_MASS_ITERS):
    _, ndof, _ = tet2_sizes(n)
    eps = np.ascontiguousarray(eps_r, dtype=np.float64).reshape(-1)
    x = np.zeros(ndof)
    _t2lib().orc_tet2_mass_solve(C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]), _ptr(eps), C.c_int(iters),
                                 _ptr(np.ascontiguousarray(b, np.float64)), _ptr(x))
    return x


def tet2_locate(n, x):
    """(tet, values[20, 3], dofs[20]) of the point x (normalised)."""
    val = np.zeros((20, 3))
    dofs = np.zeros(20, np.int64)
    t = _t2lib().orc_tet2_locate(C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]), _ptr(np.asarray(x, np.float64)),
                                 _ptr(val), dofs.ctypes.data_as(C.POINTER(C.c_long)))
    return t, val, dofs


def tet2_lambda_max(n, eps_r, iters=300, mu_r=None, mass_iters=TET2_MASS_ITERS):
    eps = np.ascontiguousarray(eps_r, dtype=np.float64).reshape(-1)
    mu = None if mu_r is None else np.ascontiguousarray(mu_r, np.float64).reshape(-1)
    return _t2lib().orc_tet2_lambda_max(C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]), _ptr(eps),
                                        _ptr(mu) if mu is not None else None, C.c_int(mass_iters), C.c_int(iters))


def tet2_energy(n, eps_r, U, P, mass_iters=TET2_MASS_ITERS):
    eps = np.ascontiguousarray(eps_r, dtype=np.float64).reshape(-1)
    return _t2lib().orc_tet2_energy(C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]), _ptr(eps), C.c_int(mass_iters),
                                    _ptr(np.ascontiguousarray(U, np.float64)), _ptr(np.ascontiguousarray(P, np.float64)))


def tet2_run(n, eps_r, integrator, dt, nsteps, tf=1, dipoles=(), receivers=(), mu_r=None, U=None, P=None,
             mass_iters=TET2_MASS_ITERS):
    """FP64 oracle of the second-order tetrahedral solver (normalised units).
    U, P: 38 * nnode values in the plane layout (plane * nnode + node).
    Returns (traces[nrec, nsamp, 4], U, P)."""
    _, ndof, _ = tet2_sizes(n)
    U = np.zeros(ndof) if U is None else np.ascontiguousarray(U, dtype=np.float64).copy()
    P = np.zeros(ndof) if P is None else np.ascontiguousarray(P, dtype=np.float64).copy()
    c, keep = _tet_case(n, eps_r, integrator, dt, tf, dipoles, receivers, mu_r, None)
    nsamp = (nsteps - 1) // tf + 1 if nsteps > 0 else 0
    tr = np.zeros((max(len(receivers), 1), max(nsamp, 1), 4))
    rc = _t2lib().orc_tet2_run(C.byref(c), C.c_int(mass_iters), C.c_int(nsteps), _ptr(U), _ptr(P), _ptr(tr))
    if rc != 0:
        raise RuntimeError(f"orc_tet2_run failed: {rc}")
    return tr[:len(receivers), :nsamp], U, P


def tet2_gradient(n, eps_r, integrator, dt, nsteps, trace_grad, tf=1, dipoles=(), receivers=(), mu_r=None,
                  mass_iters=TET2_MASS_ITERS):
    """dJ/deps_r per tetrahedron by the FP64 discrete adjoint of tet2_run
    (symplectic integrators, zero initial fields)."""
    _, _, ntet = tet2_sizes(n)
    nsamp = (nsteps - 1) // tf + 1 if nsteps > 0 else 0
    g = np.zeros((max(len(receivers), 1), max(nsamp, 1), 4))
    if len(receivers):
        g[:len(receivers), :nsamp] = np.asarray(trace_grad, np.float64).reshape(len(receivers), nsamp, 4)
    c, keep = _tet_case(n, eps_r, integrator, dt, tf, dipoles, receivers, mu_r, None)
    out = np.zeros(ntet)
    rc = _t2lib().orc_tet2_gradient(C.byref(c), C.c_int(mass_iters), C.c_int(nsteps), _ptr(g), _ptr(out))
    if rc != 0:
        raise RuntimeError(f"orc_tet2_gradient failed: {rc}")
    return out


# ------------------------------------------------- Adams-Bashforth-Moulton (hex)
class _AbmCase(C.Structure):
    _fields_ = [("gx", C.c_int), ("gy", C.c_int), ("gz", C.c_int),
                ("h", C.c_double), ("dt", C.c_double), ("eps", C.c_double), ("mu", C.c_double),
                ("time_frequency", C.c_int), ("lamped1", _dp),
                ("nsrc", C.c_int), ("src_comp", _ip), ("src_ijk", _ip),
                ("ndip", C.c_int), ("dip_ijk", _ip),
                ("nobs", C.c_int), ("obs_n", _ip), ("obs_ijk", _ip)]


def abm_run(grid, h, dt, eps, mu, tf, nsteps, lamped1, sources=(), dipoles=(), observations=(), E=None, H=None):
    """FP64 oracle of fem_abm.  sources: [(comp, (i,j,k))]; dipoles: [(i,j,k)]
    (x-directed); observations: [(xs, ys, zs)].  Returns (traces, E, H) with
    E, H lists of 4-level arrays per component."""
    gx, gy, gz = grid
    sz = hexfem_sizes(gx, gy, gz)
    E = [np.zeros(4 * n) for n in sz] if E is None else [np.ascontiguousarray(a, np.float64).copy() for a in E]
    H = [np.zeros(4 * n) for n in sz] if H is None else [np.ascontiguousarray(a, np.float64).copy() for a in H]
    km = np.ascontiguousarray(lamped1, np.float64)
    c = _AbmCase()
    c.gx, c.gy, c.gz, c.h, c.dt, c.eps, c.mu, c.time_frequency = gx, gy, gz, h, dt, eps, mu, tf
    c.lamped1 = _ptr(km)
    comp = np.array([s[0] for s in sources] or [0], np.int32)
    sijk = np.array([s[1] for s in sources] or [(0, 0, 0)], np.int32).reshape(-1)
    dijk = np.array(list(dipoles) or [(0, 0, 0)], np.int32).reshape(-1)
    on = np.array([len(l) for o in observations for l in o] or [0], np.int32)
    oi = np.array([p for o in observations for l in o for p in l] or [(0, 0, 0)], np.int32).reshape(-1)
    c.nsrc, c.src_comp, c.src_ijk = len(sources), _ptr(comp, _ip), _ptr(sijk, _ip)
    c.ndip, c.dip_ijk = len(dipoles), _ptr(dijk, _ip)
    c.nobs, c.obs_n, c.obs_ijk = len(observations), _ptr(on, _ip), _ptr(oi, _ip)
    nsamp = nsteps // tf + 1
    tr = np.zeros((max(len(observations), 1), nsamp, 3))
    Ea = (_dp * 3)(*[_ptr(a) for a in E])
    Ha = (_dp * 3)(*[_ptr(a) for a in H])
    if lib().orc_abm_run(C.byref(c), C.c_int(nsteps), Ea, Ha, _ptr(tr)) != 0:
        raise RuntimeError("orc_abm_run failed")
    return tr[:len(observations)], E, H


def abm_kmat(lamped1):
    K = np.zeros(144)
    lib().orc_abm_kmat(_ptr(np.ascontiguousarray(lamped1, np.float64)), _ptr(K))
    return K.reshape(12, 12)


# -------------------------------------------- stabilised hexahedral FEM (fem/)
class _FemStabCase(C.Structure):
    _fields_ = [("gx", C.c_int), ("gy", C.c_int), ("gz", C.c_int),
                ("h", C.c_double), ("dt", C.c_double), ("eps", C.c_double), ("mu", C.c_double),
                ("time_frequency", C.c_int), ("stabilization", C.c_double), ("use_ofem", C.c_int),
                ("nsrc", C.c_int), ("src_comp", _ip), ("src_ijk", _ip),
                ("ndip", C.c_int), ("dip_ijk", _ip),
                ("nobs", C.c_int), ("obs_n", _ip), ("obs_ijk", _ip)]


def femstab_run(grid, h, dt, eps, mu, tf, stabilization, use_ofem, nsteps, sources=(), dipoles=(), observations=(), E=None):
    """FP64 oracle of the reference's fem/ solver.  sources: [(comp, (i,j,k))];
    dipoles: [(i,j,k)] (x-directed Hertz); observations: [(xs, ys, zs)].
    Returns (traces, E) with E the 3-level array of each component."""
    gx, gy, gz = grid
    sz = hexfem_sizes(gx, gy, gz)
    E = [np.zeros(3 * n) for n in sz] if E is None else [np.ascontiguousarray(a, np.float64).copy() for a in E]
    c = _FemStabCase()
    c.gx, c.gy, c.gz, c.h, c.dt, c.eps, c.mu, c.time_frequency = gx, gy, gz, h, dt, eps, mu, tf
    c.stabilization, c.use_ofem = stabilization, use_ofem
    comp = np.array([s[0] for s in sources] or [0], np.int32)
    sijk = np.array([s[1] for s in sources] or [(0, 0, 0)], np.int32).reshape(-1)
    dijk = np.array(list(dipoles) or [(0, 0, 0)], np.int32).reshape(-1)
    on = np.array([len(l) for o in observations for l in o] or [0], np.int32)
    oi = np.array([p for o in observations for l in o for p in l] or [(0, 0, 0)], np.int32).reshape(-1)
    c.nsrc, c.src_comp, c.src_ijk = len(sources), _ptr(comp, _ip), _ptr(sijk, _ip)
    c.ndip, c.dip_ijk = len(dipoles), _ptr(dijk, _ip)
    c.nobs, c.obs_n, c.obs_ijk = len(observations), _ptr(on, _ip), _ptr(oi, _ip)
    nsamp = nsteps // tf + 1
    tr = np.zeros((max(len(observations), 1), nsamp, 3))
    Ea = (_dp * 3)(*[_ptr(a) for a in E])
    if lib().orc_femstab_run(C.byref(c), C.c_int(nsteps), Ea, _ptr(tr)) != 0:
        raise RuntimeError("orc_femstab_run failed")
    return tr[:len(observations)], E


def femstab_kmat(dt, mu, eps, h, stabilization, use_ofem):
    """The fem/ element matrix K (12 x 12)."""
    K = np.zeros(144)
    if lib().orc_femstab_kmat(C.c_double(dt), C.c_double(mu), C.c_double(eps), C.c_double(h),
                              C.c_double(stabilization), C.c_int(use_ofem), _ptr(K)) != 0:
        raise RuntimeError("element mass matrix is singular")
    return K.reshape(12, 12)


def femstab_parts(use_ofem):
    """(A, Abar, B, Bbar, C, Cbar) of the conventional (0) or OFEM (1) basis."""
    m = [np.zeros(144) for _ in range(6)]
    lib().orc_femstab_parts(C.c_int(use_ofem), *[_ptr(a) for a in m])
    return [a.reshape(12, 12) for a in m]
