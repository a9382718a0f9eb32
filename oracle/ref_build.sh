#!/usr/bin/env bash
# ref_build.sh — compile the reference's own RHS-path sources, unmodified,
# against the host-only Kokkos shim in oracle/refshim/, into
# oracle/_ref/libfiesta_ref.so.  TEST INFRASTRUCTURE ONLY: the library is the
# checker that pins the oracle restatement (oracle/fst_oracle.cpp) and makes
# the golden vectors in tests/golden/.  It is never shipped or committed.
#
# The reference tree is read where it lies (FST_REFERENCE, default
# /root/reference).  A machine without it (the GPU host) builds the same
# library from the bundle this recipe leaves in oracle/_ref/ where the tree
# is present: the reference files these units include, the sample decks and
# the vendored Lua 5.3 sources, copied into oracle/_ref/src, oracle/_ref/samples
# and oracle/_ref/lua.  oracle/_ref/ is
# git-ignored: the bundle travels with the working tree and is never
# committed.  Reference files compiled:
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
OUT="$HERE/_ref"
REF="${FST_REFERENCE:-/root/reference}"
STAGE=1
if [ ! -d "$REF/src" ]; then
  if [ -d "$OUT/src" ]; then
    REF="$OUT"  # the bundle left where the reference tree was present
    STAGE=0
  else
    echo "ref_build: reference sources not found at $REF/src and no bundle in $OUT; skipping" >&2
    exit 0
  fi
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS=(-std=c++17 -O2 -ffp-contract=off -fPIC -fopenmp -w
       -I "$HERE/refshim" -I "$REF/src" -include "$HERE/refshim/prelude.hpp")
UNITS=(cart3d cart2d rk rkfunction bc gen2d gen3d)
if [ "$STAGE" = 1 ]; then
  mkdir -p "$OUT/src" "$OUT/samples"
  deps=$(for u in "${UNITS[@]}"; do
           "$CXX" "${FLAGS[@]}" -DHAVE_MPI -MM "$REF/src/$u.cpp"
         done; "$CXX" "${FLAGS[@]}" -DHAVE_MPI -MM "$HERE/refshim/ref_harness.cpp" \
                 "$HERE/refshim/ref_gen.cpp")
  for f in $(echo "$deps" | tr ' \\' '\n\n' | grep "^$REF/src/" | sort -u); do
    cp "$f" "$OUT/src/"
  done
  # the Lua 5.3 sources the reference vendors, for the Lua deck reader's
  # tests on a host without the tree (fiesta_gb300/build.py build_deck)
  if [ -d "$REF/tpls/lua/src" ]; then
    mkdir -p "$OUT/lua"
    cp "$REF"/tpls/lua/src/*.c "$REF"/tpls/lua/src/*.h "$OUT/lua/"
  fi
  for d in "$REF"/samples/*/; do
    if [ -f "$d/fiesta.lua" ]; then
      mkdir -p "$OUT/samples/$(basename "$d")"
      cp "$d/fiesta.lua" "$OUT/samples/$(basename "$d")/"
    fi
  done
fi
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
