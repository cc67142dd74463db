"""Builds the C restatement in this folder into ``oracle/_build/liboracle.so``.

ORACLE / TEST INFRASTRUCTURE ONLY.  Plain gcc, -O2, OpenMP for the CPU
baseline, and -ffp-contract=off so FP64 results do not depend on whether the
host compiler fuses multiply-adds (x86 and Arm give identical bits).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["orc_fdtd.c", "orc_hexfem.c", "orc_tetfem.c", "orc_abm.c", "orc_femstab.c", "orc_tet2.c"]
LIB = os.path.join(HERE, "_build", "liboracle.so")


def build(force=False):
    os.makedirs(os.path.join(HERE, "_build"), exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    deps = srcs + [os.path.join(HERE, "ems_oracle.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp",
           "-Wall", "-Wno-unknown-pragmas", "-D_GNU_SOURCE", "-o", LIB + ".tmp"] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


# where the development container keeps the EMSolvers checkout; the
# environment variable EMS_REFERENCE_DIR overrides it
DEFAULT_REFERENCE_DIR = "/root/reference/src"


def build_reference():
    """Compiles the unmodified reference solvers into oracle/_ref when the
    reference tree is present (EMS_REFERENCE_DIR, else the development
    container's checkout); returns False where it is absent."""
    ref = os.environ.get("EMS_REFERENCE_DIR", DEFAULT_REFERENCE_DIR)
    if not os.path.isdir(ref):
        return False
    subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], check=True, env=dict(os.environ, EMS_REFERENCE_DIR=ref))
    return True


if __name__ == "__main__":
    print(build(force=True))
    print("reference built:", build_reference())
