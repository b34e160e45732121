#!/usr/bin/env bash
# Build the unmodified PT-ICM reference sources as a single-rank CPU checker.
#
#   oracle/_ref/pt_icm_ref    the reference CLI (src/main.cc + every src/*.cc)
#
# The sources are compiled where they lie; nothing is copied into this
# repository.  -DWHOLE drops the second main() in src/cae_estimator.cc:431-450,
# -DNDEBUG matches the reference's Release build (CMakeLists.txt:4-8), and the
# single-rank <mpi.h> stand-in lives in oracle/ref_stub/.  The output directory
# is git-ignored.
#
#   oracle/build_ref.sh [REFERENCE_DIR | --if-present]
#
# The reference directory is the argument, else $PTICM_REFERENCE_DIR, else
# the read-only checkout this recipe was written against.  With --if-present
# a missing checkout is not an error (machines without the reference, such as
# the GPU hosts, use the C oracle alone).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OPTIONAL=0
ARG="${1:-}"
if [ "$ARG" = "--if-present" ]; then OPTIONAL=1; ARG=""; fi
REF="${ARG:-${PTICM_REFERENCE_DIR:-/root/reference}}"
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
    if [ "$OPTIONAL" = 1 ]; then exit 0; fi
    echo "reference sources not found at $REF" >&2
    exit 2
fi
mkdir -p "$OUT"
CXXFLAGS="-std=c++17 -O3 -DNDEBUG -DWHOLE -w"
g++ $CXXFLAGS -I "$HERE/ref_stub" -I "$REF/include" "$REF"/src/*.cc -o "$OUT/pt_icm_ref.tmp"
mv "$OUT/pt_icm_ref.tmp" "$OUT/pt_icm_ref"
echo "built $OUT/pt_icm_ref"
