#!/usr/bin/env bash
# Builds the reference's own C++ sources, unmodified, into oracle/_ref/ref_harness
# (test infrastructure).  The sources are compiled where they lie under the
# reference checkout; only the Eigen-subset header (oracle/compat) and the
# harness (oracle/ref_harness.cpp) come from this repository.  Outputs go to
# oracle/_ref/ only (git-ignored).
# Usage: build_ref.sh <reference checkout>  (or SBR_REFERENCE_DIR=<checkout>)
# -ffp-contract=off keeps a*b+c as two rounded operations on every host
# (aarch64 g++ would otherwise fuse them), matching the GPU's __dmul_rn /
# __dadd_rn arithmetic.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
root="${1:-${SBR_REFERENCE_DIR:-}}"
if [ -z "$root" ]; then
  echo "usage: $0 <reference checkout> (or set SBR_REFERENCE_DIR)" >&2
  exit 2
fi
ref="$root/SBRSolver_rev2"
out="$here/_ref"
if [ ! -f "$ref/RTSolver.cpp" ]; then
  echo "reference sources not found at $ref" >&2
  exit 3
fi
mkdir -p "$out/alias" "$out/obj"
# Icosahedron.cpp includes "icosahedron.h" (lower case); alias it.
ln -sf "$ref/Icosahedron.h" "$out/alias/icosahedron.h"
flags=(-O2 -std=c++17 -ffp-contract=off -fno-fast-math -w -I"$here/compat" -I"$out/alias" -I"$ref")
srcs=(RTSolver FieldCompute Ray Triangle Icosahedron Preprocessor GlobalConfig timer/Timer)
pids=()
for s in "${srcs[@]}"; do
  o="$out/obj/$(basename "$s").o"
  g++ "${flags[@]}" -c "$ref/$s.cpp" -o "$o" & pids+=($!)
done
g++ "${flags[@]}" -c "$here/ref_harness.cpp" -o "$out/obj/ref_harness.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -o "$out/ref_harness" "$out"/obj/*.o -lpthread
echo "built $out/ref_harness"
