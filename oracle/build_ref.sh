#!/bin/bash
# Builds the reference solvers from their unmodified sources into oracle/_ref/
# (git-ignored).  Oracle test infrastructure only: these binaries pin the CPU
# restatement in oracle/ and generate the golden fixtures in tests/golden/.
# The reference tree is read in place; nothing is copied into this repository.
# -ffp-contract=off keeps the reference's FP64 arithmetic free of fused
# multiply-adds on every host, so its results are reproducible across hosts.
set -euo pipefail
REF=${EMS_REFERENCE_DIR:?set EMS_REFERENCE_DIR to the EMSolvers src/ directory}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -d "$REF" ] || { echo "reference sources not found at $REF" >&2; exit 3; }
mkdir -p "$OUT"
CXX="g++ -std=c++17 -O2 -ffp-contract=off -w -I$HERE/shim"
pids=()
$CXX -I"$REF/fdtd" "$HERE/ref_drivers/fdtd_ref_main.cpp" "$REF/fdtd/fdtd_simulation.cpp" -o "$OUT/fdtd_ref" & pids+=($!)
for v in fem_v2 symplectic_2 symplectic_4; do
  $CXX -I"$REF/$v" "$HERE/ref_drivers/femv2_ref_main.cpp" "$REF/$v/fem_simulation.cpp" -o "$OUT/${v}_ref" & pids+=($!)
done
$CXX -I"$REF/fem_abm" "$HERE/ref_drivers/abm_ref_main.cpp" "$REF/fem_abm/fem_simulation.cpp" -o "$OUT/fem_abm_ref" & pids+=($!)
$CXX -I"$REF/fem" "$HERE/ref_drivers/femstab_ref_main.cpp" "$REF/fem/fem_simulation.cpp" -o "$OUT/fem_ref" & pids+=($!)
# the reference's own fem_v2 program (argv interface, output file name and format)
for v in fem_v2 symplectic_2 symplectic_4; do
  $CXX -fopenmp -I"$REF/$v" "$REF/$v/main.cpp" "$REF/$v/fem_simulation.cpp" -o "$OUT/${v}_main" & pids+=($!)
done
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
exit $rc
