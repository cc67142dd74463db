"""Runs the reference solvers built from the unmodified EMSolvers sources
(oracle/_ref, produced by oracle/build_ref.sh) and reads back their traces
and fields.  Only available where those binaries were built (a checkout
with the reference sources); tests that need them skip elsewhere, and the
committed fixtures in tests/golden/ carry their outputs to machines without
them."""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BIN = os.path.join(os.path.dirname(HERE), "oracle", "_ref")
GOLDEN = os.path.join(HERE, "golden")   # holds kmat/, the reference's element-matrix files


def available():
    return all(os.access(os.path.join(REF_BIN, b), os.X_OK) for b in ("fdtd_ref", "fem_v2_ref", "fem_abm_ref", "fem_ref"))


def fdtd(nx, ny, nz, h, dt, eps, mu, tf, nsteps, sources, observations):
    """sources: [(comp, (i,j,k))]; observations: [(xs, ys, zs)]."""
    lines = [f"{nx} {ny} {nz} {float(h)!r} {float(dt)!r} {float(eps)!r} {float(mu)!r} {tf} {nsteps}", str(len(sources))]
    lines += [f"{c} {i} {j} {k}" for c, (i, j, k) in sources]
    lines.append(str(len(observations)))
    for o in observations:
        toks = []
        for lst in o:
            toks.append(str(len(lst)))
            toks += [f"{i} {j} {k}" for (i, j, k) in lst]
        lines.append(" ".join(toks))
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "o.bin")
        subprocess.run([os.path.join(REF_BIN, "fdtd_ref"), out], input="\n".join(lines) + "\n",
                       text=True, check=True, stderr=subprocess.DEVNULL)
        if os.path.getsize(out) < 8:
            raise RuntimeError("reference FDTD driver wrote no output")
        raw = open(out, "rb").read()
    nobs, ns = np.frombuffer(raw[:8], np.int32)
    off = 8
    tr = np.frombuffer(raw[off:off + 8 * nobs * ns * 3]).reshape(nobs, ns, 3)
    off += 8 * nobs * ns * 3
    shapes = [(nz + 2, ny + 2, nx + 1), (nz + 2, ny + 1, nx + 2), (nz + 1, ny + 2, nx + 2),
              (nz + 1, ny + 1, nx), (nz + 1, ny, nx + 1), (nz, ny + 1, nx + 1)]
    f = {}
    for name, s in zip(("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"), shapes):
        n = int(np.prod(s))
        f[name] = np.frombuffer(raw[off:off + 8 * n]).reshape(s).copy()
        off += 8 * n
    return tr.copy(), f


def femv2(variant, order, use_ofem, grid, h, dt, eps, mu, tf, nsteps, src, obs):
    """variant: fem_v2 | symplectic_2 | symplectic_4; src: (comp, (i,j,k))."""
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "o.bin")
        args = [os.path.join(REF_BIN, f"{variant}_ref"), out, GOLDEN, str(order), str(use_ofem),
                *map(str, grid), repr(float(h)), repr(float(dt)), repr(float(eps)), repr(float(mu)), str(tf), str(nsteps),
                str(src[0]), *map(str, src[1]), *map(str, obs)]
        subprocess.run(args, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        raw = open(out, "rb").read()
    ns = int(np.frombuffer(raw[:4], np.int32)[0])
    off = 4
    tr = np.frombuffer(raw[off:off + 32 * ns]).reshape(ns, 4).copy()
    off += 32 * ns
    n3 = np.frombuffer(raw[off:off + 12], np.int32)
    off += 12
    ef = []
    for n in n3:
        ef.append(np.frombuffer(raw[off:off + 8 * int(n)]).copy())
        off += 8 * int(n)
    return tr, ef


def abm(grid, h, dt, eps, mu, tf, nsteps, sources, dipoles, observations):
    """Reference fem_abm run.  sources: [(comp, (i,j,k))]; dipoles: [(i,j,k)]."""
    gx, gy, gz = grid
    lines = [f"{gx} {gy} {gz} {float(h)!r} {float(dt)!r} {float(eps)!r} {float(mu)!r} {tf} {nsteps}", str(len(sources))]
    lines += [f"{c} {i} {j} {k}" for c, (i, j, k) in sources]
    lines.append(str(len(dipoles)))
    lines += [f"{i} {j} {k}" for (i, j, k) in dipoles]
    lines.append(str(len(observations)))
    for o in observations:
        toks = []
        for lst in o:
            toks.append(str(len(lst)))
            toks += [f"{i} {j} {k}" for (i, j, k) in lst]
        lines.append(" ".join(toks))
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "o.bin")
        subprocess.run([os.path.join(REF_BIN, "fem_abm_ref"), out], input="\n".join(lines) + "\n",
                       text=True, check=True, stderr=subprocess.DEVNULL, stdout=subprocess.DEVNULL)
        raw = open(out, "rb").read()
    nobs, ns = np.frombuffer(raw[:8], np.int32)
    off = 8
    tr = np.frombuffer(raw[off:off + 8 * nobs * ns * 3]).reshape(nobs, ns, 3).copy()
    off += 8 * nobs * ns * 3
    sz = [gx * (gy + 1) * (gz + 1), (gx + 1) * gy * (gz + 1), (gx + 1) * (gy + 1) * gz]
    fields = []
    for q in range(6):
        n = 4 * sz[q % 3]
        fields.append(np.frombuffer(raw[off:off + 8 * n]).copy())
        off += 8 * n
    return tr, fields[:3], fields[3:]


def femstab(grid, h, dt, eps, mu, tf, stabilization, use_ofem, nsteps, sources, dipoles, observations):
    """Reference fem/ run: (traces, E levels per component, element matrix K)."""
    gx, gy, gz = grid
    lines = [f"{gx} {gy} {gz} {float(h)!r} {float(dt)!r} {float(eps)!r} {float(mu)!r} {tf} "
             f"{float(stabilization)!r} {int(use_ofem)} {nsteps}", str(len(sources))]
    lines += [f"{c} {i} {j} {k}" for c, (i, j, k) in sources]
    lines.append(str(len(dipoles)))
    lines += [f"{i} {j} {k}" for (i, j, k) in dipoles]
    lines.append(str(len(observations)))
    for o in observations:
        toks = []
        for lst in o:
            toks.append(str(len(lst)))
            toks += [f"{i} {j} {k}" for (i, j, k) in lst]
        lines.append(" ".join(toks))
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "o.bin")
        subprocess.run([os.path.join(REF_BIN, "fem_ref"), out], input="\n".join(lines) + "\n",
                       text=True, check=True, stderr=subprocess.DEVNULL, stdout=subprocess.DEVNULL)
        raw = open(out, "rb").read()
    nobs, ns = np.frombuffer(raw[:8], np.int32)
    off = 8
    tr = np.frombuffer(raw[off:off + 8 * nobs * ns * 3]).reshape(nobs, ns, 3).copy()
    off += 8 * nobs * ns * 3
    sz = [gx * (gy + 1) * (gz + 1), (gx + 1) * gy * (gz + 1), (gx + 1) * (gy + 1) * gz]
    E = []
    for q in range(3):
        n = 3 * sz[q]
        E.append(np.frombuffer(raw[off:off + 8 * n]).copy())
        off += 8 * n
    K = np.frombuffer(raw[off:off + 8 * 144]).reshape(12, 12).copy()
    return tr, E, K


def reference_program(variant, argv, kmat_dir):
    """Runs the reference's own program of `variant` (its main.cpp) with argv
    in a scratch directory holding kmat/; returns (file name, file text)."""
    import shutil
    with tempfile.TemporaryDirectory() as td:
        shutil.copytree(kmat_dir, os.path.join(td, "kmat"))
        subprocess.run([os.path.join(REF_BIN, f"{variant}_main"), *argv], cwd=td, check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        out = [f for f in os.listdir(td) if f.endswith(".csv")]
        if len(out) != 1:
            raise RuntimeError(f"expected one result file, found {out}")
        return out[0], open(os.path.join(td, out[0])).read()
