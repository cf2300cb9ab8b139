#!/usr/bin/env bash
# Build the reference library (DCM-UPB/MCIntegratorPlusPlus) from its own
# sources, where they lie, into oracle/_ref/, and link the golden-vector
# recorder (oracle/ref_recorder.cpp) against it.  Test infrastructure only.
#
# Usage: oracle/ref_build.sh REFERENCE_ROOT
#    or: MCIG_REFERENCE_ROOT=... oracle/ref_build.sh
#
# The reference's own build system (cmake) is not used: its few sources are
# compiled directly with g++.  Flags: baseline target (no -march=native, hence
# no FMA contraction, matching the oracle's -ffp-contract=off) and the standard
# headers the sources use without including them (src/AccumulatorInterface.cpp
# needs <stdexcept>, others <cmath>, <limits>, <fstream>, <cstdint>).
set -euo pipefail
REF="${1:-${MCIG_REFERENCE_ROOT:-}}"
if [ -z "$REF" ] || [ ! -d "$REF/src" ]; then
  echo "usage: $0 REFERENCE_ROOT (or set MCIG_REFERENCE_ROOT to the reference checkout)" >&2
  exit 2
fi
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
mkdir -p "$OUT"
CXXFLAGS="-O2 -std=c++14 -fPIC -ffp-contract=off -I$REF/include \
  -include stdexcept -include cmath -include limits -include fstream -include cstdint"
objs=()
for src in "$REF"/src/*.cpp; do
  o="$OUT/$(basename "${src%.cpp}").o"
  g++ $CXXFLAGS -c "$src" -o "$o" &
  objs+=("$o")
done
wait
ar rcs "$OUT/libmci_ref.a" "${objs[@]}"
gcc -O2 -std=c11 -fPIC -ffp-contract=off -c "$HERE/mci_oracle.c" -o "$OUT/mci_oracle_for_recorder.o"
g++ $CXXFLAGS -I"$REF/test" "$HERE/ref_recorder.cpp" "$OUT/mci_oracle_for_recorder.o" "$OUT/libmci_ref.a" \
  -o "$OUT/ref_recorder" -lpthread
echo "built $OUT/libmci_ref.a and $OUT/ref_recorder"
