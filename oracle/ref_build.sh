#!/usr/bin/env bash
# ref_build.sh — compile the reference's own RHS-path sources, unmodified,
# against the host-only Kokkos shim in oracle/refshim/, into
# oracle/_ref/libfiesta_ref.so.  TEST INFRASTRUCTURE ONLY: the library is the
# checker that pins the oracle restatement (oracle/fst_oracle.cpp) and makes
# the golden vectors in tests/golden/.  It is never shipped or committed.
#
# The reference tree is read where it lies (FST_REFERENCE, default
# /root/reference); nothing is copied out of it.  Reference files compiled:
#   src/cart3d.cpp src/cart2d.cpp src/rk.cpp src/rkfunction.cpp  (-DHAVE_MPI:
#       the single-rank MPI path, where fsMax returns an initialised maximum)
#   src/bc.cpp  (no HAVE_MPI: periodic ghosts by bc_xPer/yPer/zPer)
#   src/gen2d.cpp src/gen3d.cpp  (no HAVE_MPI: single-rank metric ghosts;
#       constructed only from refshim/ref_gen.cpp, built the same way;
#       -DNDEBUG as in the reference's default RelWithDebInfo build, whose
#       constructors would otherwise assert varNames.size() == nvt, which
#       fails with the C-equation on)
# plus the kernel headers they include (secondary, velocity, flux, advect,
# presgrad, viscosity, ceq3d, ceq, buoyancy, noise, kokkosTypes, debug,
# diagnostics, metric).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${FST_REFERENCE:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
  echo "ref_build: reference sources not found at $REF/src; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS=(-std=c++17 -O2 -ffp-contract=off -fPIC -fopenmp -w
       -I "$HERE/refshim" -I "$REF/src" -include "$HERE/refshim/prelude.hpp")
pids=()
"$CXX" "${FLAGS[@]}" -DHAVE_MPI -c "$REF/src/cart3d.cpp" -o "$OUT/cart3d.o" & pids+=($!)
"$CXX" "${FLAGS[@]}" -DHAVE_MPI -c "$REF/src/cart2d.cpp" -o "$OUT/cart2d.o" & pids+=($!)
"$CXX" "${FLAGS[@]}" -DHAVE_MPI -c "$REF/src/rk.cpp" -o "$OUT/rk.o" & pids+=($!)
"$CXX" "${FLAGS[@]}" -DHAVE_MPI -c "$REF/src/rkfunction.cpp" -o "$OUT/rkfunction.o" & pids+=($!)
"$CXX" "${FLAGS[@]}" -c "$REF/src/bc.cpp" -o "$OUT/bc.o" & pids+=($!)
"$CXX" "${FLAGS[@]}" -DNDEBUG -c "$REF/src/gen2d.cpp" -o "$OUT/gen2d.o" & pids+=($!)
"$CXX" "${FLAGS[@]}" -DNDEBUG -c "$REF/src/gen3d.cpp" -o "$OUT/gen3d.o" & pids+=($!)
"$CXX" "${FLAGS[@]}" -c "$HERE/refshim/ref_gen.cpp" -o "$OUT/ref_gen.o" & pids+=($!)
"$CXX" "${FLAGS[@]}" -DHAVE_MPI -c "$HERE/refshim/ref_harness.cpp" -o "$OUT/ref_harness.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
"$CXX" -shared -fopenmp -o "$OUT/libfiesta_ref.so" \
  "$OUT/cart3d.o" "$OUT/cart2d.o" "$OUT/rk.o" "$OUT/rkfunction.o" "$OUT/bc.o" \
  "$OUT/gen2d.o" "$OUT/gen3d.o" "$OUT/ref_gen.o" "$OUT/ref_harness.o"
echo "ref_build: $OUT/libfiesta_ref.so"
