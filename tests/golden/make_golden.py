"""Generates the golden fixtures in this folder from the reference solvers.

Run in a checkout that has the EMSolvers sources, with EMS_REFERENCE_DIR
naming their src/ directory:

    EMS_REFERENCE_DIR=<EMSolvers>/src python oracle/build.py          # builds oracle/_ref
    EMS_REFERENCE_DIR=<EMSolvers>/src python tests/golden/make_golden.py

Outputs (committed, small):
  kmat/{1,2,3,lamped1}.csv   the reference's element-matrix data files
                              (fem_v2/kmat), copied byte for byte: they are
                              solver input data that the engine reads at run
                              time in the reference's CSV format.
  fdtd_cases.npz             reference FDTD traces and final fields
  femv2_cases.npz            reference fem_v2 / symplectic_2 / symplectic_4
                              traces and final fields, orders 1-3
  abm_cases.npz              reference fem_abm traces and E, H levels
  femstab_cases.npz          reference fem/ (stabilised order 1, conventional
                              and OFEM bases) traces, E levels and the
                              element matrix
  cli_cases.json             argv of the reference's fem_v2 / symplectic_2 /
                              symplectic_4 programs, the file name each wrote
                              and its contents
Each case records its inputs beside the outputs so the tests can replay it.
"""
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import refrun  # noqa: E402

EPS0_FDTD, MU0 = 8.854187817e-12, 1.25663706212e-6
EPS0_FEM = 8.8541878128e-12
C0 = 1.0 / np.sqrt(EPS0_FEM * MU0)

FDTD_CASES = [
    # name, grid, h, dt, tf, nsteps, sources, observations
    ("cube8_jx", (8, 8, 8), 1e-3, 1.6e-12, 1, 30, [(0, (3, 4, 4))],
     [([(4, 4, 4)], [(3, 3, 4), (3, 4, 4), (4, 3, 4), (4, 4, 4)], [(3, 4, 3), (3, 4, 4), (4, 4, 3), (4, 4, 4)])]),
    ("box10x10x7_multi", (10, 10, 7), 1e-3, 0.5e-3 / (2.998e8 * np.sqrt(3)), 2, 60,
     [(0, (3, 4, 4)), (2, (5, 5, 3)), (1, (6, 2, 5))],
     [([(4, 4, 4)], [(3, 3, 4), (3, 4, 4), (4, 3, 4), (4, 4, 4)], [(3, 4, 3), (3, 4, 4), (4, 4, 3), (4, 4, 4)]),
      ([(5, 5, 5)], [(5, 5, 5)], [(5, 5, 5), (6, 6, 5)])]),
]

ABM_CASES = [
    ("box9x8x7_point_and_dipole", (9, 8, 7), 0.1, 0.4, 2, 40, [(0, (3, 4, 3)), (2, (5, 4, 4))], [(4, 3, 3)],
     [([(4, 4, 4)], [(3, 3, 4), (3, 4, 4), (4, 3, 4), (4, 4, 4)], [(3, 4, 3), (3, 4, 4), (4, 4, 3), (4, 4, 4)])]),
    ("cube8_dipole", (8, 8, 8), 0.05, 0.6, 1, 30, [], [(3, 3, 3)],
     [([(4, 4, 4), (3, 4, 4)], [(4, 4, 4)], [(4, 4, 4)])]),
]

# fem/ (stabilised order-1 hexahedra): h and dt of the reference driver
# (fem/main.cpp: h = 4 m / 200, dt = 0.8e-8 s / 400, c dt / h = 0.3)
FEMSTAB_CASES = [
    # name, grid, stabilization, use_ofem, tf, nsteps, sources, dipoles, observations
    ("conv_s0.3_point_dipole", (9, 8, 7), 0.3, 0, 2, 60, [(0, (4, 3, 3)), (2, (5, 4, 3))], [(3, 3, 2)],
     [([(5, 4, 4)], [(4, 3, 4), (4, 4, 4), (5, 3, 4), (5, 4, 4)], [(4, 4, 3), (4, 4, 4), (5, 4, 3), (5, 4, 4)])]),
    ("ofem_s0.3_point_dipole", (9, 8, 7), 0.3, 1, 2, 60, [(1, (4, 3, 3))], [(3, 3, 2)],
     [([(5, 4, 4)], [(4, 3, 4), (4, 4, 4), (5, 3, 4), (5, 4, 4)], [(4, 4, 3), (4, 4, 4), (5, 4, 3), (5, 4, 4)])]),
    ("conv_s0_dipole", (8, 8, 8), 0.0, 0, 1, 50, [], [(3, 3, 3)], [([(4, 4, 4), (3, 4, 4)], [(4, 4, 4)], [(4, 4, 4)])]),
    ("ofem_s0.1_dipole", (8, 8, 8), 0.1, 1, 1, 50, [], [(3, 3, 3)], [([(4, 4, 4), (3, 4, 4)], [(4, 4, 4)], [(4, 4, 4)])]),
]

# the reference's own programs (fem_v2, symplectic_2, symplectic_4 main.cpp):
# argv, the file name they write and its bytes
CLI_CASES = [
    ("fem_v2", ["1", "1", "2", "0.8", "0.8", "0.8", "8", "2e-9", "0.4", "0.4", "0.4", "0.5", "0.4", "0.3", "1", "1", "1"]),
    ("fem_v2", ["1", "0", "1", "0.6", "0.6", "0.6", "10", "1.5e-9", "0.3", "0.32", "0.28", "0.42", "0.3", "0.3", "1", "1", "1"]),
    ("symplectic_2", ["1", "1", "1", "0.6", "0.6", "0.6", "9", "1.5e-9", "0.3", "0.3", "0.3", "0.4", "0.3", "0.3", "1", "1", "1"]),
    ("symplectic_4", ["2", "1", "2", "0.8", "0.8", "0.8", "4", "1e-9", "0.4", "0.4", "0.4", "0.5", "0.4", "0.4", "1", "1", "1"]),
]

FEM_CASES = []
for variant in ("fem_v2", "symplectic_2", "symplectic_4"):
    for order, ofem in ((1, 1), (1, 0), (2, 1), (3, 1)):
        g = (6 * order, 5 * order, 4 * order) if order < 3 else (9, 9, 9)
        FEM_CASES.append((variant, order, ofem, g))


def main():
    src = os.environ.get("EMS_REFERENCE_DIR")
    if not src or not os.path.isdir(src):
        raise SystemExit("set EMS_REFERENCE_DIR to the EMSolvers src/ directory")
    if not refrun.available():
        raise SystemExit("reference binaries missing: run python oracle/build.py first")
    kdir = os.path.join(HERE, "kmat")
    os.makedirs(kdir, exist_ok=True)
    for f in ("1.csv", "2.csv", "3.csv", "lamped1.csv"):
        shutil.copyfile(os.path.join(src, "fem_v2", "kmat", f), os.path.join(kdir, f))

    out = {}
    meta = []
    for name, (nx, ny, nz), h, dt, tf, ns, src, obs in FDTD_CASES:
        tr, f = refrun.fdtd(nx, ny, nz, h, dt, EPS0_FDTD, MU0, tf, ns, src, obs)
        out[f"{name}/traces"] = tr
        for k, v in f.items():
            out[f"{name}/{k}"] = v
        meta.append(dict(name=name, grid=[nx, ny, nz], h=h, dt=float(dt), eps=EPS0_FDTD, mu=MU0, tf=tf,
                         nsteps=ns, sources=[[c, list(p)] for c, p in src],
                         observations=[[list(map(list, l)) for l in o] for o in obs]))
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "fdtd_cases.npz"), **out)

    out = {}
    meta = []
    for variant, order, ofem, g in FEM_CASES:
        h = 0.1
        dt = h / (C0 * np.sqrt(3.0)) / 2.0
        src = (2, (g[0] // 2, g[1] // 2, g[2] // 2))
        obs = (g[0] // 2 + 1, g[1] // 2, g[2] // 2)
        tr, ef = refrun.femv2(variant, order, ofem, g, h, dt, EPS0_FEM, MU0, 2, 40, src, obs)
        name = f"{variant}_o{order}_{'ofem' if ofem else 'lumped'}"
        out[f"{name}/traces"] = tr
        for q in range(3):
            out[f"{name}/ef{q}"] = ef[q]
        meta.append(dict(name=name, variant=variant, order=order, use_ofem=ofem, grid=list(g), h=h, dt=float(dt),
                         eps=EPS0_FEM, mu=MU0, tf=2, nsteps=40, source=[src[0], list(src[1])], observation=list(obs)))
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "femv2_cases.npz"), **out)
    out = {}
    meta = []
    for name, g, h, dtf, tf, ns, src, dip, obs in ABM_CASES:
        dt = dtf * h / (2.998e8 * np.sqrt(3))
        tr, E, Hh = refrun.abm(g, h, dt, EPS0_FDTD, MU0, tf, ns, src, dip, obs)
        out[f"{name}/traces"] = tr
        for q in range(3):
            out[f"{name}/E{q}"] = E[q]
            out[f"{name}/H{q}"] = Hh[q]
        meta.append(dict(name=name, grid=list(g), h=h, dt=float(dt), eps=EPS0_FDTD, mu=MU0, tf=tf, nsteps=ns,
                         sources=[[c, list(p)] for c, p in src], dipoles=[list(p) for p in dip],
                         observations=[[list(map(list, l)) for l in o] for o in obs]))
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "abm_cases.npz"), **out)
    out = {}
    meta = []
    for name, g, sf, ofem, tf, ns, src, dip, obs in FEMSTAB_CASES:
        h, dt = 4.0 / 200, 0.8e-8 / 400
        tr, E, K = refrun.femstab(g, h, dt, EPS0_FDTD, MU0, tf, sf, ofem, ns, src, dip, obs)
        out[f"{name}/traces"] = tr
        out[f"{name}/K"] = K
        for q in range(3):
            out[f"{name}/E{q}"] = E[q]
        meta.append(dict(name=name, grid=list(g), h=h, dt=dt, eps=EPS0_FDTD, mu=MU0, tf=tf, stabilization=sf,
                         use_ofem=ofem, nsteps=ns, sources=[[c, list(p)] for c, p in src], dipoles=[list(p) for p in dip],
                         observations=[[list(map(list, l)) for l in o] for o in obs]))
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "femstab_cases.npz"), **out)
    cli = []
    for variant, argv in CLI_CASES:
        name, content = refrun.reference_program(variant, argv, kdir)
        cli.append(dict(variant=variant, argv=argv, filename=name, content=content))
    with open(os.path.join(HERE, "cli_cases.json"), "w") as f:
        json.dump(cli, f, indent=1)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
