"""The ems_fem program (argv of the reference's fem_v2 / symplectic_2 /
symplectic_4 programs, fem_v2/main.cpp:51-115) against the reference
programs themselves: for the same argv it writes a file of the same name
with the same bytes (FP64 traces bit-identical, the reference's CSV format
of fem_v2/fem_simulation.cpp:1322-1344).  The expected names and contents
were recorded from the reference programs (tests/golden/cli_cases.json)."""
import json
import os
import shutil
import subprocess

import pytest

import golden_io

pytestmark = pytest.mark.gpu
CLI = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "emsolvers_gb300", "_build", "ems_fem")
INTEG = {"fem_v2": "leapfrog", "symplectic_2": "symp2", "symplectic_4": "symp4"}
CASES = json.load(open(os.path.join(golden_io.HERE, "cli_cases.json")))


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["filename"][:40])
def test_ems_fem_writes_the_reference_programs_file(case, tmp_path):
    shutil.copytree(golden_io.KMAT_DIR, os.path.join(tmp_path, "kmat"))
    env = dict(os.environ, EMS_INTEGRATOR=INTEG[case["variant"]], EMS_PRECISION="fp64")
    r = subprocess.run([CLI, *case["argv"]], cwd=tmp_path, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    written = sorted(f for f in os.listdir(tmp_path) if f.endswith(".csv"))
    assert written == [case["filename"]]
    assert open(os.path.join(tmp_path, written[0])).read() == case["content"]


def test_ems_fem_rejects_a_wrong_argument_count(tmp_path):
    r = subprocess.run([CLI, "1", "1"], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Usage" in r.stdout
