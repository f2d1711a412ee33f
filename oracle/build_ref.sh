#!/usr/bin/env bash
# Compile the reference's own operator sources (TMat/utility, tmat, tmatreduce,
# tmat3d, tmatphys) where they lie, against the project's minimal container
# header (oracle/refshim/Eigen/Core) and the extern "C" shim, into
# oracle/_ref/libtmat_ref.so.  Test infrastructure only.
#
# The reference's eigensolver driver (TMat/pfunc.*, main.cpp, tests.cpp) needs
# Spectra and Eigen, which are absent, so it is not built; the oracle's own
# Lanczos drives the compiled perform_op instead.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# (default: $TMAT_REFERENCE_ROOT, else /root/reference, where the reference is
# mounted in the build container; exits 3 when the sources are absent)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${TMAT_REFERENCE_ROOT:-/root/reference}}"
SRC="$REF/TMat"
if [ ! -f "$SRC/tmatreduce.cpp" ]; then
  echo "reference sources not found under $SRC; skipping oracle/_ref" >&2
  exit 3
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS=(-std=c++14 -O3 -fPIC -fopenmp -w -DNDEBUG -I"$HERE/refshim" -I"$SRC")
case "$(uname -m)" in
  x86_64) FLAGS+=(-mpopcnt) ;;
esac
OBJS=()
PIDS=()
for f in utility tmat tmatreduce tmat3d tmatphys; do
  "$CXX" "${FLAGS[@]}" -c "$SRC/$f.cpp" -o "$OUT/$f.o" &
  PIDS+=($!)
  OBJS+=("$OUT/$f.o")
done
"$CXX" "${FLAGS[@]}" -c "$HERE/refshim/ref_shim.cpp" -o "$OUT/ref_shim.o" &
PIDS+=($!)
# configuration planting (DumpConfig), for its golden fixtures
DSRC="$REF/DumpConfig"
for f in dumpconfig dumpreduce utilityb; do
  "$CXX" "${FLAGS[@]}" -I"$DSRC" -c "$DSRC/$f.cpp" -o "$OUT/dump_$f.o" &
  PIDS+=($!)
  OBJS+=("$OUT/dump_$f.o")
done
"$CXX" "${FLAGS[@]}" -I"$DSRC" -c "$HERE/refshim/dump_shim.cpp" -o "$OUT/dump_shim.o" &
PIDS+=($!)
OBJS+=("$OUT/dump_shim.o")
for p in "${PIDS[@]}"; do wait "$p"; done
"$CXX" -shared -fopenmp -o "$OUT/libtmat_ref.so" "${OBJS[@]}" "$OUT/ref_shim.o"
echo "built $OUT/libtmat_ref.so"
