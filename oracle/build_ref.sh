#!/usr/bin/env bash
# build_ref.sh -- compile the reference's own, unmodified continuum-LDOS sources into
# oracle/_ref/ (test infrastructure only; oracle/_ref/ is git-ignored).
#
# The reference's build (src/Makefile + config/config.mk.*) links GSL and FFTW, which
# this image does not have, and generates src/gitversion.cc from git; so its build
# system is not used.  Instead the path's source files are compiled directly with g++
# against oracle/compat/ (a project-written subset of the GSL/FFTW C API) and a
# two-line gitversion stub.  Outputs:
#   oracle/_ref/calcqpi   the reference CLI (src/calcqpi.cc main)
#   oracle/_ref/refdump   oracle/refdump.cc driving the reference's classes, float64 dumps
#   oracle/_ref/mkwavefunctions   the reference's orbital-file tool (src/mkwavefunctions.cc main)
#   oracle/_ref/seam_check   oracle/seam_check.cc: the GB300QPI backend built against the
#                            reference's GPUQPI interface and linked with libcqpi.so
# Usage: oracle/build_ref.sh <reference-root>   (or the root in $CQPI_REFERENCE)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${CQPI_REFERENCE:-}}"
if [ -z "$REF" ]; then
  echo "no reference root given (argument or CQPI_REFERENCE); nothing to build" >&2
  exit 3
fi
OUT="$HERE/_ref"
if [ ! -f "$REF/src/qpi.cc" ]; then
  echo "reference sources not found under $REF; nothing to build" >&2
  exit 3
fi
mkdir -p "$OUT"
echo 'const char *gitversion = "reference-sources", *gitbranch = "unknown";' > "$OUT/gitversion.cc"
CXX="${CXX:-g++}"
FLAGS="-O2 -fopenmp -w -std=c++14 -I$HERE/compat -I$REF/include -I$REF/src"
SRCS="qpi tightbinding wannierfunctions idl loadxcf"
pids=()
for s in $SRCS calcqpi gethostdata mkwavefunctions; do
  $CXX $FLAGS -c "$REF/src/$s.cc" -o "$OUT/$s.o" &
  pids+=($!)
done
$CXX $FLAGS -c "$OUT/gitversion.cc" -o "$OUT/gitversion.o" &
pids+=($!)
$CXX $FLAGS -c "$HERE/refdump.cc" -o "$OUT/refdump.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
objs=""
for s in $SRCS; do objs="$objs $OUT/$s.o"; done
$CXX -fopenmp -o "$OUT/calcqpi" "$OUT/calcqpi.o" "$OUT/gethostdata.o" "$OUT/gitversion.o" $objs
$CXX -fopenmp -o "$OUT/refdump" "$OUT/refdump.o" $objs
$CXX -fopenmp -o "$OUT/mkwavefunctions" "$OUT/mkwavefunctions.o" "$OUT/gitversion.o" $objs
# the GB300QPI backend of the narrow seam, compiled against the reference's GPUQPI interface
# and linked with libcqpi.so (when the library has been built)
LIBDIR="$(cd "$HERE/.." && pwd)/calcqpi-release_gb300/_build"
if [ -f "$LIBDIR/libcqpi.so" ]; then
  $CXX $FLAGS -I"$HERE/../include" -I"$HERE/../calcqpi-release_gb300/seam" -c "$HERE/seam_check.cc" \
    -o "$OUT/seam_check.o"
  $CXX -fopenmp -o "$OUT/seam_check" "$OUT/seam_check.o" "$OUT/wannierfunctions.o" "$OUT/idl.o" \
    "$OUT/loadxcf.o" -L"$LIBDIR" -lcqpi -Wl,-rpath,"$LIBDIR"
fi
echo "built $OUT/calcqpi $OUT/refdump $OUT/mkwavefunctions"
