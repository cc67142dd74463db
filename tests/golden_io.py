"""Readers for the golden fixtures in tests/golden/ (see make_golden.py)."""
import json
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KMAT_DIR = os.path.join(HERE, "kmat")


def load(name):
    z = np.load(os.path.join(HERE, name))
    meta = json.loads(bytes(z["meta"]).decode())
    return z, meta


def fdtd_cases():
    z, meta = load("fdtd_cases.npz")
    for m in meta:
        fields = {k: z[f"{m['name']}/{k}"] for k in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")}
        yield m, z[f"{m['name']}/traces"], fields


def femv2_cases():
    z, meta = load("femv2_cases.npz")
    for m in meta:
        yield m, z[f"{m['name']}/traces"], [z[f"{m['name']}/ef{q}"] for q in range(3)]


def kmat_path(order, use_ofem):
    return os.path.join(KMAT_DIR, f"{order}.csv" if use_ofem else f"lamped{order}.csv")


def abm_cases():
    z, meta = load("abm_cases.npz")
    for m in meta:
        n = m["name"]
        yield m, z[f"{n}/traces"], [z[f"{n}/E{q}"] for q in range(3)], [z[f"{n}/H{q}"] for q in range(3)]


def femstab_cases():
    z, meta = load("femstab_cases.npz")
    for m in meta:
        n = m["name"]
        yield m, z[f"{n}/traces"], [z[f"{n}/E{q}"] for q in range(3)], z[f"{n}/K"]
